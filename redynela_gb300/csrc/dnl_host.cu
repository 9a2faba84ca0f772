// Host side of libdnlgpu: the C ABI of include/dnl_gpu.h, the nodal kernels (assembly, Chung-Hulbert
// update, boundary conditions) and the device-side time-step logic.
//
// Kernels:
//   k_gather     Fint(n*dim+j) = sum of element forces in ascending element order, the order of
//                Domain::computeInternalForces strategy 0 on one thread (Domain.C:158-195);
//                a node-centric CSR gather, no atomics, identical from run to run.
//   k_node       k_gather + ExplicitSolverCH::computePredictions (ExplicitSolverCH.C:387-431),
//                explicitSolve (:490-545), updateGrid (:555-567) and the constant boundary
//                conditions (Boundary.C:478-525, 636-665) of one node, with the reference's
//                rounding (__dmul_rn/__dadd_rn in its operation order).
//   k_bc_current the boundary conditions' writes to the Current field that computeStress reads
//                (imposed speed: delta_disp = v * dt with this step's dt).
//   k_dt         Solver::computeTimeStep (Solver.C:220-267), ExplicitSolverCH::initStep (:434-447),
//                updateTime and Solver::betweenTimeBounds in one thread, so a run needs no
//                host round trip per step.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "dnl_common.cuh"
#include "dnl_node.cuh"

using namespace dnl;

#define RMUL __dmul_rn
#define RADD __dadd_rn
#define RSUB __dsub_rn

namespace {

// ----------------------------------------------------------------------------- gather
template <int DIM>
__global__ void __launch_bounds__(256) k_gather(GatherArgs g)
{
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= g.N) return;
  const int b = g.start[n], e = g.start[n + 1];
  double f[DIM];
#pragma unroll
  for (int c = 0; c < DIM; c++) f[c] = 0.0;
  for (int q = b; q < e; q++) {
    const int ent = __ldg(g.entry + q);
#pragma unroll
    for (int c = 0; c < DIM; c++) f[c] = RADD(f[c], __ldg(g.fe + (long)c * g.EN + ent));
  }
#pragma unroll
  for (int c = 0; c < DIM; c++) g.fint[(long)n * DIM + c] = f[c];
}

// scalar gather (mass): out[n] = sum of me entries in ascending element order
__global__ void __launch_bounds__(256) k_gather1(int N, const int *start, const int *entry,
                                                 const double *me, double *out)
{
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  double s = 0.;
  for (int q = start[n]; q < start[n + 1]; q++) s = RADD(s, me[entry[q]]);
  out[n] = s;
}

// nodal update (node_update, apply_bc) and time-step logic (dt_update): dnl_node.cuh

template <int DIM>
__global__ void __launch_bounds__(256) k_node(NodeArgs g)
{
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= g.N) return;
  DevTime *tm = g.tm;
  if (tm->done | tm->status) return;
  node_update<DIM>(g, n, tm->timeStep, g.alphaM, g.beta, g.gamma);
}

// batched: node n belongs to instance nodeInst[n] with its own time record and constants
template <int DIM>
__global__ void __launch_bounds__(256) k_node_batch(NodeArgs g, const int *nodeInst,
                                                    const InstParams *prm, DevTime *tms)
{
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= g.N) return;
  const int i = nodeInst[n];
  const DevTime *tm = tms + i;
  if (tm->done | tm->status) return;
  node_update<DIM>(g, n, tm->timeStep, prm[i].alphaM, prm[i].beta, prm[i].gamma);
}

// Current-field writes of the constant boundary conditions before the element pass; in a batch
// node n's time record is tm[nodeInst[n]], otherwise tm[0]
__global__ void k_bc_current(int nb, const int *nodes, const int *code, const double *speed,
                             NodeFields cur, DevTime *tmBase, const int *nodeInst)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nb) return;
  const DevTime *tm = tmBase + (nodeInst ? nodeInst[nodes[i]] : 0);
  if (tm->done | tm->status) return;
  const int n = nodes[i];
  const double dt = tm->timeStep;
  const int cd = code[i];
#pragma unroll
  for (int c = 0; c < 3; c++) {
    const int act = (cd >> (2 * c)) & 3;
    if (act == 1) {
      cur.du[c][n] = 0.;
      cur.v[c][n] = 0.;
      cur.a[c][n] = 0.;
    } else if (act == 2) {
      const double s = speed[3 * i + c];
      cur.a[c][n] = 0.;
      cur.v[c][n] = s;
      cur.du[c][n] = RMUL(s, dt);
    }
  }
}

// k_bc_current split in two for dnl_step_host, whose Current v and a arrive on a second stream
// beside the element pass: the delta_disp writes before the pass (recording whether they were
// made: the run neither done nor in error), then the v and a writes, made iff the first were, once
// those fields are on the device.  Together the same writes as k_bc_current.
__global__ void k_bc_current_du(int nb, const int *nodes, const int *code, const double *speed,
                                NodeFields cur, const DevTime *tm, int *applied)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool live = !(tm->done | tm->status);
  if (i == 0) *applied = live;
  if (i >= nb || !live) return;
  const int n = nodes[i];
  const double dt = tm->timeStep;
  const int cd = code[i];
#pragma unroll
  for (int c = 0; c < 3; c++) {
    const int act = (cd >> (2 * c)) & 3;
    if (act == 1)
      cur.du[c][n] = 0.;
    else if (act == 2)
      cur.du[c][n] = RMUL(speed[3 * i + c], dt);
  }
}

__global__ void k_bc_current_va(int nb, const int *nodes, const int *code, const double *speed,
                                NodeFields cur, const int *applied)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nb || !*applied) return;
  const int n = nodes[i];
  const int cd = code[i];
#pragma unroll
  for (int c = 0; c < 3; c++) {
    const int act = (cd >> (2 * c)) & 3;
    if (act == 1) {
      cur.v[c][n] = 0.;
      cur.a[c][n] = 0.;
    } else if (act == 2) {
      cur.a[c][n] = 0.;
      cur.v[c][n] = speed[3 * i + c];
    }
  }
}

// ----------------------------------------------------------------------------- time step
struct DtArgs {
  DevTime *tm;
  int mode, freq, method;
  double safetyOmega, Cs;
};

__global__ void k_dt(DtArgs a)
{
  dt_update(a.tm, a.mode, a.freq, a.method, a.safetyOmega, a.Cs);
}

__global__ void k_dt_batch(DevTime *tms, const InstParams *prm, int count, int mode)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  dt_update(tms + i, mode, prm[i].freq, prm[i].method, prm[i].safetyOmega, prm[i].Cs);
}

// node-major (x,y,z) host layout <-> component arrays on the device, several nodal fields in one
// launch: field blockIdx.y of the set, its node-major staging slot and its three component arrays
struct FieldSet {
  double *aos[5];
  double *c[5][3];
  int nf;
};
__global__ void k_aos_to_soa_set(int N, FieldSet s)
{
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  const int f = blockIdx.y;
  const double *a = s.aos[f];
#pragma unroll
  for (int k = 0; k < 3; k++) s.c[f][k][n] = a[3L * n + k];
}
__global__ void k_soa_to_aos_set(int N, FieldSet s)
{
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  const int f = blockIdx.y;
  double *a = s.aos[f];
#pragma unroll
  for (int k = 0; k < 3; k++) a[3L * n + k] = s.c[f][k][n];
}
// the handle's nodal field f (0 coords, 1 du, 2 v, 3 a, 4 disp of the Current bank) with staging
// slot f, appended to a set
void add_field(dnl_handle *h, FieldSet &s, int f)
{
  NodeFields &b = h->bank[h->cur];
  double *const *p = f == 0 ? h->x : f == 1 ? b.du : f == 2 ? b.v : f == 3 ? b.a : b.disp;
  s.aos[s.nf] = h->stage + (size_t)f * 3 * h->N;
  for (int k = 0; k < 3; k++) s.c[s.nf][k] = p[k];
  s.nf++;
}
int transpose_set(dnl_handle *h, const FieldSet &s, bool toDevice, cudaStream_t st);

// FP64 throughput probe: 8 independent DFMA chains per thread, ITER rounds
__global__ void k_fill(double *p, long n, double v)
{
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

// cached evp^n at evp = 1e-10 per element material (several materials)
__global__ void k_fill_evpn(long nIP, int nip, const int *elemMat, const double *evpn0, double *out)
{
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nIP) out[i] = evpn0[elemMat[i / nip]];
}

__global__ void k_fp64_peak(double *out, double a, double b, int iters)
{
  double x0 = threadIdx.x * 1e-9, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5,
         x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; i++) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  const double s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
  if (s == 12345.678) out[0] = s;  // keeps the chains live
}

// self-check of the reciprocal and quotient helpers against CUDA's IEEE division
__global__ void k_check_quotients(int n, const double *a, const double *b, double *out)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double r = nr_rcp(b[i]);
  out[i] = r;
  out[(long)n + i] = quot(a[i], b[i], r);
  out[2L * n + i] = __drcp_rn(b[i]);
  out[3L * n + i] = __ddiv_rn(a[i], b[i]);
}

// kinetic energy of the Current field (Domain::getTotalKineticEnergy), fixed-order block sums
__global__ void k_kinetic(int N, NodeFields f, const double *mass, double *partial)
{
  __shared__ double sh[256];
  double s = 0.;
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
    const double v0 = f.v[0][n], v1 = f.v[1][n], v2 = f.v[2][n];
    s += .5 * mass[n] * (v0 * v0 + v1 * v1 + v2 * v2);
  }
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

// ----------------------------------------------------------------------------- helpers
#define CK(call)                                                                              \
  do {                                                                                        \
    cudaError_t err_ = (call);                                                                \
    if (err_ != cudaSuccess) {                                                                \
      snprintf(g_lastError, sizeof g_lastError, "%s: %s", #call, cudaGetErrorString(err_));  \
      return DNL_ERR_CUDA;                                                                    \
    }                                                                                         \
  } while (0)

char g_lastError[256] = "";

int check_launch()
{
  cudaError_t e = cudaPeekAtLastError();
  if (e != cudaSuccess) {
    snprintf(g_lastError, sizeof g_lastError, "kernel launch: %s", cudaGetErrorString(e));
    return DNL_ERR_CUDA;
  }
  return 0;
}

// Material::getHookeMatrix (Material.C:270-331): the diagonal f = E (1 - nu) / ((1 + nu) (1 - 2 nu)),
// the off-diagonal nu / (1 - nu) f and the shear (1 - 2 nu) / (2 (1 - nu)) f, in the reference's
// expressions
void hooke_entries(double young, double nu, double c[3])
{
  const double f = (young * (1.0 - nu) / ((1.0 + nu) * (1.0 - 2.0 * nu)));
  c[0] = 1 * f;
  c[1] = (nu / (1. - nu)) * f;
  c[2] = ((1.0 - 2.0 * nu) / (2. * (1.0 - nu))) * f;
}

// node-major staging slots <-> component arrays for every field of the set, one launch
int transpose_set(dnl_handle *h, const FieldSet &s, bool toDevice, cudaStream_t st)
{
  if (!s.nf) return 0;
  const dim3 grid((h->N + 255) / 256, s.nf);
  if (toDevice)
    k_aos_to_soa_set<<<grid, 256, 0, st>>>(h->N, s);
  else
    k_soa_to_aos_set<<<grid, 256, 0, st>>>(h->N, s);
  launch_counter()++;
  return check_launch();
}

GatherArgs gather_args(dnl_handle *h)
{
  GatherArgs g;
  g.N = h->N;
  g.EN = (int)h->EN;
  g.start = h->n2eStart;
  g.entry = h->n2e;
  g.fe = h->fe;
  g.fint = h->fint;
  return g;
}

int launch_gather(dnl_handle *h)
{
  GatherArgs g = gather_args(h);
  const int grid = (h->N + 255) / 256;
  prof_begin(h, h->stream);
  if (h->dim == 2)
    k_gather<2><<<grid, 256, 0, h->stream>>>(g);
  else
    k_gather<3><<<grid, 256, 0, h->stream>>>(g);
  prof_end(h, DNL_PROF_NODE, h->stream);
  launch_counter()++;
  return check_launch();
}

int launch_node(dnl_handle *h, bool keepFint)
{
  NodeArgs g;
  g.N = h->N;
  g.EN = (int)h->EN;
  g.start = h->n2eStart;
  g.entry = h->n2e;
  g.fe = h->fe;
  g.mass = h->mass;
  g.cur = h->bank[h->cur];
  g.nxt = h->bank[1 - h->cur];
  for (int i = 0; i < 3; i++) g.x[i] = h->x[i];
  g.bcIdx = h->bcIdx;
  g.bcCode = h->bcCode;
  g.bcSpeed = h->bcSpeed;
  g.fint = keepFint ? h->fint : nullptr;
  g.tm = h->tm;
  g.alphaM = h->alphaM;
  g.beta = h->beta;
  g.gamma = h->gamma;
  const int grid = (h->N + 255) / 256;
  prof_begin(h, h->stream);
  if (h->dim == 2)
    k_node<2><<<grid, 256, 0, h->stream>>>(g);
  else
    k_node<3><<<grid, 256, 0, h->stream>>>(g);
  prof_end(h, DNL_PROF_NODE, h->stream);
  launch_counter()++;
  return check_launch();
}

int launch_dt(dnl_handle *h, int mode)
{
  DtArgs a;
  a.tm = h->tm;
  a.mode = mode;
  a.freq = h->freq;
  a.method = h->method;
  a.safetyOmega = h->safetyOmega;
  a.Cs = h->elemCs ? 1.0 : h->mat.Cs;  // several materials: k_courant reduced len / Cs per element
  prof_begin(h, h->stream);
  k_dt<<<1, 1, 0, h->stream>>>(a);
  prof_end(h, DNL_PROF_OTHER, h->stream);
  launch_counter()++;
  return check_launch();
}

int launch_bc_current(dnl_handle *h)
{
  if (!h->nbcNodes) return 0;
  prof_begin(h, h->stream);
  k_bc_current<<<(h->nbcNodes + 127) / 128, 128, 0, h->stream>>>(h->nbcNodes, h->bcNodeList, h->bcCode,
                                                                  h->bcSpeed, h->bank[h->cur], h->tm,
                                                                  nullptr);
  prof_end(h, DNL_PROF_OTHER, h->stream);
  launch_counter()++;
  return check_launch();
}

// critical-time-step computation that precedes a DT_FORCE or a due DT_POST
int launch_time_step_source(dnl_handle *h)
{
  if (h->method == DNL_COURANT) return launch_courant(h, h->stream);
  return launch_pulse(h, h->stream);
}

int read_time(dnl_handle *h, DevTime *out)
{
  CK(cudaMemcpyAsync(out, h->tm, sizeof(DevTime), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return 0;
}


// one explicit step's launches; post = complete this step's time update afterwards
int enqueue_step(dnl_handle *h, long long incAfter, bool last)
{
  int r;
  if (h->hasSpeedBC || h->nbcNodes) {
    if ((r = launch_bc_current(h))) return r;
  }
  if ((r = launch_elem(h, h->stream, 1))) return r;
  if ((r = launch_node(h, true))) return r;
  h->cur = 1 - h->cur;  // endStep: Node::transfertNodalField
  if (incAfter % h->freq == 0) {
    if ((r = launch_time_step_source(h))) return r;
  }
  return launch_dt(h, last ? DT_POST : (DT_POST | DT_PRE));
}

}  // namespace

namespace dnl {
int launch_node_batch(dnl_handle *h, const int *nodeInst, const InstParams *prm, DevTime *tms)
{
  NodeArgs g;
  g.N = h->N;
  g.EN = (int)h->EN;
  g.start = h->n2eStart;
  g.entry = h->n2e;
  g.fe = h->fe;
  g.mass = h->mass;
  g.cur = h->bank[h->cur];
  g.nxt = h->bank[1 - h->cur];
  for (int i = 0; i < 3; i++) g.x[i] = h->x[i];
  g.bcIdx = h->bcIdx;
  g.bcCode = h->bcCode;
  g.bcSpeed = h->bcSpeed;
  g.fint = h->fint;
  g.tm = nullptr;
  g.alphaM = g.beta = g.gamma = 0.;
  const int grid = (h->N + 255) / 256;
  prof_begin(h, h->stream);
  if (h->dim == 2)
    k_node_batch<2><<<grid, 256, 0, h->stream>>>(g, nodeInst, prm, tms);
  else
    k_node_batch<3><<<grid, 256, 0, h->stream>>>(g, nodeInst, prm, tms);
  prof_end(h, DNL_PROF_NODE, h->stream);
  launch_counter()++;
  return check_launch();
}

int launch_dt_batch(dnl_handle *h, DevTime *tms, const InstParams *prm, int count, int mode)
{
  prof_begin(h, h->stream);
  k_dt_batch<<<(count + 127) / 128, 128, 0, h->stream>>>(tms, prm, count, mode);
  prof_end(h, DNL_PROF_OTHER, h->stream);
  launch_counter()++;
  return check_launch();
}

int launch_bc_batch(dnl_handle *h, DevTime *tms, const int *nodeInst)
{
  if (!h->nbcNodes) return 0;
  prof_begin(h, h->stream);
  k_bc_current<<<(h->nbcNodes + 127) / 128, 128, 0, h->stream>>>(h->nbcNodes, h->bcNodeList, h->bcCode,
                                                                  h->bcSpeed, h->bank[h->cur], tms,
                                                                  nodeInst);
  prof_end(h, DNL_PROF_OTHER, h->stream);
  launch_counter()++;
  return check_launch();
}

int launch_gather_mass(dnl_handle *h, const double *me)
{
  k_gather1<<<(h->N + 255) / 256, 256, 0, h->stream>>>(h->N, h->n2eStart, h->n2e, me, h->mass);
  launch_counter()++;
  return check_launch();
}

__global__ void k_set_time(DevTime *tm, double t)
{
  tm->currentTime = t;
  tm->tsDate = tm->lastTsDate = t;
}

// restart at time t from the state already loaded: Solver::computeTimeStep(True) on it
int restart_time(dnl_handle *h, double t)
{
  k_set_time<<<1, 1, 0, h->stream>>>(h->tm, t);
  launch_counter()++;
  int r;
  if ((r = launch_time_step_source(h))) return r;
  if ((r = launch_dt(h, DT_FORCE))) return r;
  DevTime tt;
  if ((r = read_time(h, &tt))) return r;
  return tt.status;
}

// the primal per-step launches, for the sensitivity run (dnl_sens.cu)
int enqueue_bc_current(dnl_handle *h) { return (h->hasSpeedBC || h->nbcNodes) ? launch_bc_current(h) : 0; }
int enqueue_node(dnl_handle *h) { return launch_node(h, true); }
int read_time_state(dnl_handle *h, DevTime *t) { return read_time(h, t); }

int launch_gather_raw(int dim, const GatherArgs &g, cudaStream_t s)
{
  const int grid = (g.N + 255) / 256;
  if (dim == 2)
    k_gather<2><<<grid, 256, 0, s>>>(g);
  else
    k_gather<3><<<grid, 256, 0, s>>>(g);
  launch_counter()++;
  return cudaPeekAtLastError() == cudaSuccess ? 0 : DNL_ERR_CUDA;
}
}  // namespace dnl

// ------------------------------------------------------------------------------ profiling
namespace {
struct ProfRec {
  int kind;
  cudaEvent_t a, b;
};
struct Prof {
  std::vector<ProfRec> recs;
  std::vector<cudaEvent_t> pool;
  cudaEvent_t open;
};
cudaEvent_t prof_event(Prof *p)
{
  if (!p->pool.empty()) {
    cudaEvent_t e = p->pool.back();
    p->pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  cudaEventCreate(&e);
  return e;
}
}  // namespace

namespace dnl {
void prof_begin(dnl_handle *h, cudaStream_t s)
{
  if (!h->profiling) return;
  Prof *p = (Prof *)h->prof;
  p->open = prof_event(p);
  cudaEventRecord(p->open, s);
}
void prof_end(dnl_handle *h, int kind, cudaStream_t s)
{
  if (!h->profiling) return;
  Prof *p = (Prof *)h->prof;
  cudaEvent_t b = prof_event(p);
  cudaEventRecord(b, s);
  p->recs.push_back(ProfRec{kind, p->open, b});
}
}  // namespace dnl

// =============================================================================== C ABI
// ------------------------------------------------------------------------------ element groups
namespace {
bool solid_reference_element(int etype)
{
  return etype == DNL_ELHEX8N3D || etype == DNL_ELTET4N3D || etype == DNL_ELTET10N3D;
}

// every element group's connectivity, node-major per element, in element order
int all_connectivity(dnl_handle *h, std::vector<int> &conn, std::vector<int> &nenOf)
{
  conn.clear();
  nenOf.clear();
  for (int gi = -1; gi < h->nextra; gi++) {
    const int E = gi < 0 ? h->E : h->extra[gi].E, nen = gi < 0 ? h->nen : h->extra[gi].nen;
    const int *dc = gi < 0 ? h->conn : h->extra[gi].conn;
    std::vector<int> t((size_t)nen * E);
    CK(cudaMemcpy(t.data(), dc, sizeof(int) * t.size(), cudaMemcpyDeviceToHost));
    for (int e = 0; e < E; e++) {
      for (int k = 0; k < nen; k++) conn.push_back(t[(size_t)k * E + e]);
      nenOf.push_back(nen);
    }
  }
  return 0;
}
}  // namespace

extern "C" {

const char *dnl_error_string(int status)
{
  switch (status) {
    case DNL_OK: return "ok";
    case DNL_ERR_NEG_DETJ: return "negative Jacobian determinant";
    case DNL_ERR_RR_NOCONV: return "radial return did not converge in 2000 iterations";
    case DNL_ERR_JACOBI_NOCONV: return "polar decomposition did not converge in 29 Jacobi rotations";
    case DNL_ERR_PULSE_NOCONV: return "power iteration did not converge in 1000 iterations";
    case DNL_ERR_DT: return "time step not positive or not finite";
    case DNL_ERR_ARG: return "invalid argument";
    case DNL_ERR_CUDA: return g_lastError[0] ? g_lastError : "CUDA error";
    case DNL_ERR_SINGULAR: return "singular element Jacobian";
    case DNL_ERR_TIMEOUT: return "device-side wait ran out";
    default: return "unknown status";
  }
}

int dnl_device_count(int *count)
{
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) n = 0;
  if (count) *count = n;
  return 0;
}

long long dnl_kernel_launches(void) { return launch_counter(); }

int dnl_profile_begin(dnl_handle *h)
{
  if (!h) return DNL_ERR_ARG;
  if (!h->prof) h->prof = new Prof();
  ((Prof *)h->prof)->recs.clear();
  h->profiling = true;
  return 0;
}

int dnl_profile_end(dnl_handle *h, double *ms, long long *launches)
{
  if (!h || !h->prof) return DNL_ERR_ARG;
  h->profiling = false;
  CK(cudaStreamSynchronize(h->stream));
  Prof *p = (Prof *)h->prof;
  for (int k = 0; k < DNL_PROF_KINDS; k++) {
    if (ms) ms[k] = 0.;
    if (launches) launches[k] = 0;
  }
  for (auto &r : p->recs) {
    float t = 0.f;
    CK(cudaEventElapsedTime(&t, r.a, r.b));
    if (ms) ms[r.kind] += t;
    if (launches) launches[r.kind]++;
    p->pool.push_back(r.a);
    p->pool.push_back(r.b);
  }
  p->recs.clear();
  return 0;
}

int dnl_timer_mark(dnl_handle *h, int slot)
{
  if (!h || slot < 0 || slot >= 8) return DNL_ERR_ARG;
  if (!h->marks[slot]) CK(cudaEventCreate(&h->marks[slot]));
  CK(cudaEventRecord(h->marks[slot], h->stream));
  return 0;
}

int dnl_timer_elapsed(dnl_handle *h, int from, int to, double *ms)
{
  if (!h || !ms || from < 0 || from >= 8 || to < 0 || to >= 8 || !h->marks[from] || !h->marks[to])
    return DNL_ERR_ARG;
  CK(cudaEventSynchronize(h->marks[to]));
  float t = 0.f;
  CK(cudaEventElapsedTime(&t, h->marks[from], h->marks[to]));
  *ms = t;
  return 0;
}

int dnl_measure_fp64_peak(double *tflops)
{
  if (!tflops) return DNL_ERR_ARG;
  int dev = 0, sms = 0;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  double *out;
  CK(cudaMalloc(&out, sizeof(double)));
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  const int threads = 256, blocks = sms * 8, iters = 4096;
  k_fp64_peak<<<blocks, threads>>>(out, 0.999999, 1e-7, 64);  // warm-up
  CK(cudaEventRecord(e0));
  k_fp64_peak<<<blocks, threads>>>(out, 0.999999, 1e-7, iters);
  CK(cudaEventRecord(e1));
  CK(cudaEventSynchronize(e1));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, e0, e1));
  launch_counter() += 2;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  const double flops = 2.0 * 8.0 * iters * (double)threads * blocks;
  *tflops = flops / (ms * 1e-3) / 1e12;
  return 0;
}

int dnl_set_iteration_caps(int rotations, int newton, int power)
{
  if (rotations > kPolarMaxIt - 1 || newton > kRadialReturnMaxIt || power > kPulseMaxIt || power == 0)
    return DNL_ERR_ARG;
  const int rot = rotations < 0 ? kPolarMaxIt - 1 : rotations;
  const int nwt = newton < 0 ? kRadialReturnMaxIt : newton;
  if (int r = set_iteration_caps(rot, nwt)) {
    snprintf(g_lastError, sizeof g_lastError, "cudaMemcpyToSymbol of the iteration caps failed");
    return r;
  }
  pulse_cap() = power < 0 ? kPulseMaxIt : power;
  return 0;
}

int dnl_set_stop_tolerances(double polar, double radial)
{
  if (!(polar < 1.0) || !(radial < 1.0) || polar == 0.0 || radial == 0.0) return DNL_ERR_ARG;
  if (int r = set_stop_tolerances(polar < 0 ? kPolarPrecision : polar, radial < 0 ? kRadialReturnPrecision : radial)) {
    snprintf(g_lastError, sizeof g_lastError, "cudaMemcpyToSymbol of the stop tolerances failed");
    return r;
  }
  return 0;
}

int dnl_check_quotients(int n, const double *a, const double *b, double *out)
{
  if (n <= 0 || !a || !b || !out) return DNL_ERR_ARG;
  double *d;
  CK(cudaMalloc(&d, sizeof(double) * 6 * (size_t)n));
  int r = 0;
  auto run = [&]() -> int {
    CK(cudaMemcpy(d, a, sizeof(double) * n, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d + n, b, sizeof(double) * n, cudaMemcpyHostToDevice));
    k_check_quotients<<<(n + 255) / 256, 256>>>(n, d, d + n, d + 2 * (size_t)n);
    launch_counter()++;
    if (int c = check_launch()) return c;
    CK(cudaMemcpy(out, d + 2 * (size_t)n, sizeof(double) * 4 * (size_t)n, cudaMemcpyDeviceToHost));
    return 0;
  };
  r = run();
  cudaFree(d);
  return r;
}

int dnl_range_push(const char *name)
{
  nvtxRangePushA(name ? name : "dnl");
  return 0;
}

int dnl_range_pop(void)
{
  nvtxRangePop();
  return 0;
}

int dnl_set_device(int device)
{
  CK(cudaSetDevice(device));
  return 0;
}

int dnl_host_alloc(unsigned long long bytes, void **ptr)
{
  if (!ptr) return DNL_ERR_ARG;
  CK(cudaMallocHost(ptr, bytes));
  return 0;
}

int dnl_host_free(void *ptr)
{
  if (ptr) CK(cudaFreeHost(ptr));
  return 0;
}

int dnl_get_stream(dnl_handle *h, void **stream)
{
  if (!h || !stream) return DNL_ERR_ARG;
  *stream = (void *)h->stream;
  return 0;
}

int dnl_destroy(dnl_handle *h)
{
  if (!h) return DNL_ERR_ARG;
  dnl::sens_free(h);
  dnl::adj_free(h);
  for (int i = 0; i < h->ngraphs; i++) cudaGraphExecDestroy(h->graphs[i].exec);
  void *ptrs[] = {h->conn, h->x[0], h->n2eStart, h->n2e, h->mass, h->fieldMem, h->ip, h->detJ,
                  h->stepT, h->fe, h->fint, h->stage, h->bcIdx, h->bcCode, h->bcNodeList, h->bcSpeed,
                  h->pj, h->ev, h->kx, h->tm, h->x0, h->elemMat, h->dmats, h->elemCs,
                  h->matTab, h->evpn0, h->hooke};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  for (int gi = 0; gi < h->nextra; gi++) {
    // (the integration-point state is inside h->ip)
    void *gp[] = {h->extra[gi].conn, h->extra[gi].detJ, h->extra[gi].pj, h->extra[gi].Cs,
                  h->extra[gi].stepT};
    for (void *p : gp)
      if (p) cudaFree(p);
  }
  delete[] h->extra;
  for (int i = 0; i < 8; i++)
    if (h->marks[i]) cudaEventDestroy(h->marks[i]);
  for (int i = 0; i < 3; i++)
    if (h->ioEv[i]) cudaEventDestroy(h->ioEv[i]);
  if (h->ioStream) cudaStreamDestroy(h->ioStream);
  if (h->bcApplied) cudaFree(h->bcApplied);
  if (h->stream) cudaStreamDestroy(h->stream);
  if (h->prof) {
    Prof *p = (Prof *)h->prof;
    for (auto &r : p->recs) {
      cudaEventDestroy(r.a);
      cudaEventDestroy(r.b);
    }
    for (auto e : p->pool) cudaEventDestroy(e);
    delete p;
  }
  delete[] h->nodeRo;
  delete[] h->elemMatHost;
  delete[] h->matExpHost;
  delete h;
  return 0;
}

int dnl_set_materials(dnl_handle *h, int nmat, const dnl_material_law *mats, const int *elem_material)
{
  if (!h || nmat < 1 || !mats || h->prologueDone || h->batchUnion) return DNL_ERR_ARG;
  if (nmat > 1 && !elem_material) return DNL_ERR_ARG;
  const long N = h->N, E = h->E;
  long Eall = E;  // elements of every group, in element order
  for (int gi = 0; gi < h->nextra; gi++) Eall += h->extra[gi].E;
  if (elem_material)
    for (long e = 0; e < Eall; e++)
      if (elem_material[e] < 0 || elem_material[e] >= nmat) return DNL_ERR_ARG;
  long ntab = 0;
  for (int i = 0; i < nmat; i++) {
    const dnl_material_law &ml = mats[i];
    if (ml.law < DNL_HARD_POWER || ml.law > DNL_HARD_METAFOR) return DNL_ERR_ARG;
    if (!(ml.young > 0. && ml.density > 0.)) return DNL_ERR_ARG;
    if (ml.law == DNL_HARD_TABULAR) {
      if (ml.npoints < 1 || !ml.table_x || !ml.table_y) return DNL_ERR_ARG;
      for (int k = 1; k < ml.npoints; k++)
        if (!(ml.table_x[k] >= ml.table_x[k - 1])) return DNL_ERR_ARG;  // ascending (sorted DiscreteFunction)
      ntab += 2 * ml.npoints;
    }
  }
  // drop an earlier assignment
  void *old[] = {h->elemMat, h->dmats, h->elemCs, h->matTab, h->evpn0, h->hooke};
  for (void *p : old)
    if (p) cudaFree(p);
  h->elemMat = nullptr;
  h->dmats = nullptr;
  h->elemCs = nullptr;
  h->matTab = nullptr;
  h->evpn0 = nullptr;
  h->hooke = nullptr;
  delete[] h->nodeRo;
  h->nodeRo = nullptr;
  delete[] h->elemMatHost;
  h->elemMatHost = nullptr;
  delete[] h->matExpHost;
  h->matExpHost = nullptr;
  if (ntab) CK(cudaMalloc(&h->matTab, sizeof(double) * ntab));
  std::vector<Material> hm(nmat);
  std::vector<double> pn(nmat, 0.);
  long off = 0;
  for (int i = 0; i < nmat; i++) {
    const dnl_material_law &ml = mats[i];
    const double *tab = nullptr;
    if (ml.law == DNL_HARD_TABULAR) {
      CK(cudaMemcpy(h->matTab + off, ml.table_x, sizeof(double) * ml.npoints, cudaMemcpyHostToDevice));
      CK(cudaMemcpy(h->matTab + off + ml.npoints, ml.table_y, sizeof(double) * ml.npoints, cudaMemcpyHostToDevice));
      tab = h->matTab + off;
      off += 2 * ml.npoints;
    }
    hm[i] = make_material_law(ml, tab);
    if (ml.law == DNL_HARD_POWER) pn[i] = pow(1e-10, ml.params[2]);
  }
  h->nmat = nmat;
  h->mat = hm[0];
  {  // Material::getHookeMatrix of material 0 for the Pulse estimate, and of every material when
     // the Pulse products take each element's
    double c[3];
    hooke_entries(h->mat.young, h->mat.nu, c);
    h->C00 = c[0];
    h->C01 = c[1];
    h->C33 = c[2];
    if (nmat > 1 && h->method == DNL_PULSE) {
      std::vector<double> hk(3 * (size_t)nmat);
      for (int i = 0; i < nmat; i++) hooke_entries(hm[i].young, hm[i].nu, &hk[3 * (size_t)i]);
      CK(cudaMalloc(&h->hooke, sizeof(double) * hk.size()));
      CK(cudaMemcpy(h->hooke, hk.data(), sizeof(double) * hk.size(), cudaMemcpyHostToDevice));
    }
  }
  // nodal densities as Domain::initSolve assigns them: element order over every group, the last
  // element wins
  std::vector<int> conn, nenOf;  // every element's nodes, node-major per element, element order
  if (all_connectivity(h, conn, nenOf)) return DNL_ERR_CUDA;
  std::vector<size_t> first(Eall + 1, 0);
  for (long e = 0; e < Eall; e++) first[e + 1] = first[e] + nenOf[e];
  auto matOf = [&](long e) { return elem_material ? elem_material[e] : 0; };
  h->nodeRo = new double[N];
  for (long n = 0; n < N; n++) h->nodeRo[n] = hm[0].rho;
  for (long e = 0; e < Eall; e++)
    for (size_t k = first[e]; k < first[e + 1]; k++) h->nodeRo[conn[k]] = hm[matOf(e)].rho;
  // the cached evp^n of each group's points at rest, (1e-10)^n of its element's material
  const int ns = etype_ns(h->etype);  // the same for every group of a domain (one family)
  for (int gi = -1; gi < h->nextra; gi++) {
    const long gE = gi < 0 ? E : h->extra[gi].E, gOff = gi < 0 ? 0 : h->extra[gi].eOff;
    const int gnip = gi < 0 ? h->nip : h->extra[gi].nip;
    const long gIP = gE * gnip;
    double *gip = gi < 0 ? h->ip : h->extra[gi].ip;
    std::vector<double> pnIP(gIP);
    for (long e = 0; e < gE; e++)
      for (int q = 0; q < gnip; q++) pnIP[e * gnip + q] = pn[matOf(gOff + e)];
    CK(cudaMemcpy(gip + (size_t)(3 * ns + 2) * gIP, pnIP.data(), sizeof(double) * gIP, cudaMemcpyHostToDevice));
  }
  CK(cudaMalloc(&h->evpn0, sizeof(double) * nmat));
  CK(cudaMemcpy(h->evpn0, pn.data(), sizeof(double) * nmat, cudaMemcpyHostToDevice));
  // Element::getSoundSpeed: the element's E and nu, the mean of its nodes' densities; kept per
  // element with several materials, and on a domain of several element types (each group's
  // array, the first group's in h->elemCs) whatever the materials
  std::vector<double> cs(Eall);
  for (long e = 0; e < Eall; e++) {
    const Material &m = hm[matOf(e)];
    double ro = 0.;
    for (size_t k = first[e]; k < first[e + 1]; k++) ro += h->nodeRo[conn[k]];
    ro /= nenOf[e];
    const double Nu = m.nu;
    cs[e] = sqrt((m.young * (1 - Nu)) / (ro * (1 + Nu) * (1 - 2 * Nu)));
  }
  if (nmat > 1 || (h->nextra && h->method == DNL_COURANT)) {
    CK(cudaMalloc(&h->elemCs, sizeof(double) * E));
    CK(cudaMemcpy(h->elemCs, cs.data(), sizeof(double) * E, cudaMemcpyHostToDevice));
    for (int gi = 0; gi < h->nextra; gi++) {
      ElemGroup &g = h->extra[gi];
      if (!g.Cs) CK(cudaMalloc(&g.Cs, sizeof(double) * g.E));
      CK(cudaMemcpy(g.Cs, cs.data() + g.eOff, sizeof(double) * g.E, cudaMemcpyHostToDevice));
    }
  }
  if (nmat > 1) {
    h->elemMatHost = new int[Eall];
    std::copy(elem_material, elem_material + Eall, h->elemMatHost);
    h->matExpHost = new double[nmat];
    for (int i = 0; i < nmat; i++) h->matExpHost[i] = mats[i].law == DNL_HARD_POWER ? mats[i].params[2] : 0.;
    std::vector<int> em(elem_material, elem_material + Eall);
    CK(cudaMalloc(&h->elemMat, sizeof(int) * Eall));
    CK(cudaMemcpy(h->elemMat, em.data(), sizeof(int) * Eall, cudaMemcpyHostToDevice));
    CK(cudaMalloc(&h->dmats, sizeof(Material) * nmat));
    CK(cudaMemcpy(h->dmats, hm.data(), sizeof(Material) * nmat, cudaMemcpyHostToDevice));
  }
  for (int i = 0; i < h->ngraphs; i++) cudaGraphExecDestroy(h->graphs[i].exec);
  h->ngraphs = 0;
  return 0;
}

int dnl_set_hourglass(dnl_handle *h, double coefficient)
{
  if (!h || !(coefficient >= 0.) || coefficient > 1e3) return DNL_ERR_ARG;
  h->hourglass = coefficient;
  for (int i = 0; i < h->ngraphs; i++) cudaGraphExecDestroy(h->graphs[i].exec);
  h->ngraphs = 0;  // captured launches hold the coefficient by value
  return 0;
}

int dnl_reset(dnl_handle *h, const dnl_material *mat, const double *v0)
{
  if (!h) return DNL_ERR_ARG;
  if (mat && (h->nmat > 1 || h->mat.hard.law != DNL_HARD_POWER)) return DNL_ERR_ARG;
  cudaStream_t s = h->stream;
  CK(cudaStreamSynchronize(s));
  for (int i = 0; i < h->ngraphs; i++) cudaGraphExecDestroy(h->graphs[i].exec);
  h->ngraphs = 0;  // captured launches hold the old material and state by value
  if (mat) {
    h->mat = make_material(*mat, h->nen);
    double c[3];
    hooke_entries(h->mat.young, h->mat.nu, c);
    h->C00 = c[0];
    h->C01 = c[1];
    h->C33 = c[2];
    // a domain of several element types: each group's Courant sound speed with its own node count
    // (one material, so h->elemCs holds the first group's speed when it exists)
    if (h->nextra && h->elemCs) {
      k_fill<<<(unsigned)((h->E + 255) / 256), 256, 0, s>>>(h->elemCs, h->E, h->mat.Cs);
      launch_counter()++;
    }
    for (int gi = 0; gi < h->nextra; gi++)
      if (h->extra[gi].Cs) {
        const ElemGroup &g = h->extra[gi];
        k_fill<<<(unsigned)((g.E + 255) / 256), 256, 0, s>>>(g.Cs, g.E, make_material(*mat, g.nen).Cs);
        launch_counter()++;
      }
  }
  if (v0) {
    const double vn = sqrt(v0[0] * v0[0] + v0[1] * v0[1] + v0[2] * v0[2]);
    for (int c = 0; c < 3; c++) {
      h->v0[c] = v0[c];
      h->v0dir[c] = vn > 0 ? v0[c] / vn : 0.;
    }
  }
  const long N = h->N, nIP = h->nIP;
  CK(cudaMemcpyAsync(h->x[0], h->x0, sizeof(double) * 3 * N, cudaMemcpyDeviceToDevice, s));
  CK(cudaMemsetAsync(h->fieldMem, 0, sizeof(double) * 24 * N, s));
  for (int b = 0; b < 2; b++)
    for (int c = 0; c < 3; c++) {
      k_fill<<<(unsigned)((N + 255) / 256), 256, 0, s>>>(h->bank[b].v[c], N, h->v0[c]);
      launch_counter()++;
    }
  const int ncomp = 3 * etype_ns(h->etype) + 3;  // IpLayout::NCOMP
  const int ns = etype_ns(h->etype);
  CK(cudaMemsetAsync(h->ip, 0, sizeof(double) * ncomp * nIP, s));
  k_fill<<<(unsigned)((nIP + 255) / 256), 256, 0, s>>>(h->ip + (size_t)(3 * ns + 1) * nIP, nIP, 1e-10);
  if (h->elemMat)
    k_fill_evpn<<<(unsigned)((nIP + 255) / 256), 256, 0, s>>>(nIP, h->nip, h->elemMat, h->evpn0,
                                                              h->ip + (size_t)(3 * ns + 2) * nIP);
  else
    k_fill<<<(unsigned)((nIP + 255) / 256), 256, 0, s>>>(h->ip + (size_t)(3 * ns + 2) * nIP, nIP,
                                                         h->mat.hard.law == DNL_HARD_POWER ? pow(1e-10, h->mat.n) : 0.);
  launch_counter() += 2;
  for (int gi = 0; gi < h->nextra; gi++) {  // further element groups, as the first
    const ElemGroup &g = h->extra[gi];
    const int gns = etype_ns(g.etype), gnc = 3 * gns + 3;
    CK(cudaMemsetAsync(g.ip, 0, sizeof(double) * gnc * g.nIP, s));
    k_fill<<<(unsigned)((g.nIP + 255) / 256), 256, 0, s>>>(g.ip + (size_t)(3 * gns + 1) * g.nIP, g.nIP, 1e-10);
    if (h->elemMat)
      k_fill_evpn<<<(unsigned)((g.nIP + 255) / 256), 256, 0, s>>>(g.nIP, g.nip, h->elemMat + g.eOff, h->evpn0,
                                                                  g.ip + (size_t)(3 * gns + 2) * g.nIP);
    else
      k_fill<<<(unsigned)((g.nIP + 255) / 256), 256, 0, s>>>(g.ip + (size_t)(3 * gns + 2) * g.nIP, g.nIP,
                                                             h->mat.hard.law == DNL_HARD_POWER ? pow(1e-10, h->mat.n) : 0.);
    launch_counter() += 2;
    if (g.stepT) CK(cudaMemsetAsync(g.stepT, 0, sizeof(double) * 18 * g.nIP, s));
  }
  CK(cudaMemsetAsync(h->fint, 0, sizeof(double) * h->dim * N, s));
  if (h->stepT) CK(cudaMemsetAsync(h->stepT, 0, sizeof(double) * 18 * nIP, s));
  DevTime t;
  memset(&t, 0, sizeof t);
  t.upTime = h->endTime;
  t.endTime = h->endTime;
  t.startTime = 0.;
  t.lenMinBits = 0x7ff0000000000000ull;
  t.badElem = -1;
  CK(cudaMemcpyAsync(h->tm, &t, sizeof t, cudaMemcpyHostToDevice, s));
  CK(cudaStreamSynchronize(s));
  if (check_launch()) return DNL_ERR_CUDA;
  h->cur = 0;
  h->prologueDone = false;
  h->hostIncrement = 0;
  return 0;
}

int dnl_create(const dnl_mesh_desc *mesh, const dnl_material *mat, const dnl_solver_params *sp,
               dnl_handle **out)
{
  if (!mesh || !mat || !sp || !out) return DNL_ERR_ARG;
  *out = nullptr;
  if (!etype_valid(mesh->etype)) return DNL_ERR_ARG;
  if (mesh->num_nodes <= 0 || mesh->num_elements <= 0 || !mesh->coords || !mesh->conn) return DNL_ERR_ARG;
  if (sp->frequency < 1 || !(sp->end_time > 0) || !(sp->safety > 0)) return DNL_ERR_ARG;
  if (sp->method != DNL_COURANT && sp->method != DNL_PULSE) return DNL_ERR_ARG;
  if (sp->method == DNL_COURANT && mesh->etype == DNL_ELHEX8N3D) return DNL_ERR_ARG;  // ElHex8n3D.C:188-192
  // the one-point hexahedron's stiffness is singular in its hourglass modes: Courant only
  if (sp->method == DNL_PULSE && mesh->etype == DNL_ELHEX8N3D_1PT) return DNL_ERR_ARG;
  // Node::Current->ro is set only on one NodalField (Domain.C:1088) and the fields swap every step,
  // so a Courant recomputation at an odd increment reads a zero density; the reference would then
  // take a zero time step.  Only even frequencies are accepted with Courant.
  if (sp->method == DNL_COURANT && (sp->frequency % 2)) return DNL_ERR_ARG;
  if (mesh->num_bc < 0 || (mesh->num_bc > 0 && (!mesh->bc_kind || !mesh->bc_val || !mesh->bc_start || !mesh->bc_nodes)))
    return DNL_ERR_ARG;
  const int N = mesh->num_nodes, E = mesh->num_elements;
  const int nen = etype_nen(mesh->etype);
  for (long i = 0; i < (long)E * nen; i++)
    if (mesh->conn[i] < 0 || mesh->conn[i] >= N) return DNL_ERR_ARG;
  for (int g = 0; g < mesh->num_bc; g++)
    for (int q = mesh->bc_start[g]; q < mesh->bc_start[g + 1]; q++)
      if (mesh->bc_nodes[q] < 0 || mesh->bc_nodes[q] >= N) return DNL_ERR_ARG;

  static bool tablesSet = false;
  if (!tablesSet) {
    set_shape_tables();
    tablesSet = true;
  }

  dnl_handle *h = new dnl_handle();
  memset(h, 0, sizeof(dnl_handle));
  h->etype = mesh->etype;
  h->dim = etype_dim(mesh->etype);
  h->nen = nen;
  h->nip = etype_nip(mesh->etype);
  h->N = N;
  h->E = E;
  h->nIP = E * h->nip;
  h->EN = (long)E * nen;
  h->flags = sp->flags;
  h->freq = sp->frequency;
  h->method = sp->method;
  h->endTime = sp->end_time;
  h->rhoB = sp->rho_b;
  h->safety = sp->safety;
  h->cur = 0;
  *out = h;
  auto fail = [&](int code) {
    dnl_destroy(h);
    *out = nullptr;
    return code;
  };
#define CKF(call)                                                                             \
  do {                                                                                        \
    cudaError_t err_ = (call);                                                                \
    if (err_ != cudaSuccess) {                                                                \
      snprintf(g_lastError, sizeof g_lastError, "%s: %s", #call, cudaGetErrorString(err_));  \
      return fail(DNL_ERR_CUDA);                                                              \
    }                                                                                         \
  } while (0)
  CKF(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));

  // material constants, in the reference's expressions
  const Material m = make_material(*mat, nen);
  h->mat = m;
  // ExplicitSolverCH::computeIntegrationParameters (ExplicitSolverCH.C:336-343)
  const double rb = sp->rho_b;
  h->alphaM = (2.0 * rb - 1.0) / (1.0 + rb);
  h->beta = (5.0 - 3.0 * rb) / ((1.0 + rb) * (1.0 + rb) * (2.0 - rb));
  h->gamma = 1.5 - h->alphaM;
  h->omegaS = sqrt((12.0 * pow((1 + rb), 3) * (2.0 - rb)) / (10 + 15 * rb - rb * rb + pow(rb, 3) - pow(rb, 4)));
  h->safetyOmega = sp->safety * h->omegaS;
  h->hourglass = 0.05;

  // ---- mesh
  std::vector<int> connT((size_t)nen * E);
  for (int e = 0; e < E; e++)
    for (int k = 0; k < nen; k++) connT[(size_t)k * E + e] = mesh->conn[(size_t)e * nen + k];
  CKF(cudaMalloc(&h->conn, sizeof(int) * connT.size()));
  CKF(cudaMemcpy(h->conn, connT.data(), sizeof(int) * connT.size(), cudaMemcpyHostToDevice));
  {
    double *xm;
    CKF(cudaMalloc(&xm, sizeof(double) * 3 * (size_t)N));
    std::vector<double> xs(3 * (size_t)N);
    for (int n = 0; n < N; n++)
      for (int r = 0; r < 3; r++) xs[(size_t)r * N + n] = mesh->coords[3 * (size_t)n + r];
    CKF(cudaMemcpy(xm, xs.data(), sizeof(double) * xs.size(), cudaMemcpyHostToDevice));
    for (int r = 0; r < 3; r++) h->x[r] = xm + (size_t)r * N;
    CKF(cudaMalloc(&h->x0, sizeof(double) * 3 * (size_t)N));
    CKF(cudaMemcpy(h->x0, xm, sizeof(double) * 3 * (size_t)N, cudaMemcpyDeviceToDevice));
  }
  // node -> (element, local node) CSR, ascending element order
  {
    std::vector<int> start(N + 1, 0), entry((size_t)E * nen), fill(N, 0);
    for (long i = 0; i < (long)E * nen; i++) start[mesh->conn[i] + 1]++;
    for (int n = 0; n < N; n++) start[n + 1] += start[n];
    for (int e = 0; e < E; e++)
      for (int k = 0; k < nen; k++) {
        const int n = mesh->conn[(size_t)e * nen + k];
        entry[start[n] + fill[n]++] = e * nen + k;
      }
    CKF(cudaMalloc(&h->n2eStart, sizeof(int) * (N + 1)));
    CKF(cudaMalloc(&h->n2e, sizeof(int) * entry.size()));
    CKF(cudaMemcpy(h->n2eStart, start.data(), sizeof(int) * (N + 1), cudaMemcpyHostToDevice));
    CKF(cudaMemcpy(h->n2e, entry.data(), sizeof(int) * entry.size(), cudaMemcpyHostToDevice));
  }
  // ---- nodal fields: 2 banks x 4 fields x 3 components
  CKF(cudaMalloc(&h->fieldMem, sizeof(double) * 24 * (size_t)N));
  CKF(cudaMemset(h->fieldMem, 0, sizeof(double) * 24 * (size_t)N));
  for (int b = 0; b < 2; b++)
    for (int c = 0; c < 3; c++) {
      double *base = h->fieldMem + (size_t)b * 12 * N;
      h->bank[b].du[c] = base + (size_t)(0 + c) * N;
      h->bank[b].v[c] = base + (size_t)(3 + c) * N;
      h->bank[b].a[c] = base + (size_t)(6 + c) * N;
      h->bank[b].disp[c] = base + (size_t)(9 + c) * N;
    }
  {  // BoundarySpeed::applyInitial_V0 on both fields
    const double vn = sqrt(mesh->v0[0] * mesh->v0[0] + mesh->v0[1] * mesh->v0[1] + mesh->v0[2] * mesh->v0[2]);
    for (int c = 0; c < 3; c++) {
      h->v0[c] = mesh->v0[c];
      h->v0dir[c] = vn > 0 ? mesh->v0[c] / vn : 0.;
    }
    std::vector<double> v(N);
    for (int b = 0; b < 2; b++)
      for (int c = 0; c < 3; c++) {
        for (int n = 0; n < N; n++) v[n] = mesh->v0[c];
        CKF(cudaMemcpy(h->bank[b].v[c], v.data(), sizeof(double) * N, cudaMemcpyHostToDevice));
      }
  }
  CKF(cudaMalloc(&h->stage, sizeof(double) * 15 * (size_t)N));
  CKF(cudaMalloc(&h->mass, sizeof(double) * N));
  CKF(cudaMemset(h->mass, 0, sizeof(double) * N));
  // ---- integration points
  const int ncomp = 3 * etype_ns(h->etype) + 3;  // IpLayout::NCOMP
  const int ns = etype_ns(h->etype);
  CKF(cudaMalloc(&h->ip, sizeof(double) * (size_t)ncomp * h->nIP));
  CKF(cudaMemset(h->ip, 0, sizeof(double) * (size_t)ncomp * h->nIP));
  {  // evp = 1e-10 (IntegrationPoint::flush) and its cached power
    std::vector<double> v(h->nIP, 1e-10);
    CKF(cudaMemcpy(h->ip + (size_t)(3 * ns + 1) * h->nIP, v.data(), sizeof(double) * h->nIP, cudaMemcpyHostToDevice));
    const double pn = pow(1e-10, m.n);
    for (auto &x : v) x = pn;
    CKF(cudaMemcpy(h->ip + (size_t)(3 * ns + 2) * h->nIP, v.data(), sizeof(double) * h->nIP, cudaMemcpyHostToDevice));
  }
  CKF(cudaMalloc(&h->detJ, sizeof(double) * h->nIP));
  if (h->flags & DNL_FLAG_STEP_TENSORS) {
    CKF(cudaMalloc(&h->stepT, sizeof(double) * 18 * (size_t)h->nIP));
    CKF(cudaMemset(h->stepT, 0, sizeof(double) * 18 * (size_t)h->nIP));
  }
  CKF(cudaMalloc(&h->fe, sizeof(double) * (size_t)h->dim * E * nen));
  CKF(cudaMalloc(&h->fint, sizeof(double) * (size_t)h->dim * N));
  CKF(cudaMemset(h->fint, 0, sizeof(double) * (size_t)h->dim * N));
  // ---- boundary conditions: final action per node and component (the last group wins, as
  // each BoundaryCondition::applyConstant overwrites delta_disp, mat_speed and dmat_speed)
  {
    std::vector<int> codeN(N, 0);
    std::vector<double> spdN(3 * (size_t)N, 0.);
    std::vector<char> has(N, 0);
    for (int g = 0; g < mesh->num_bc; g++) {
      for (int q = mesh->bc_start[g]; q < mesh->bc_start[g + 1]; q++) {
        const int n = mesh->bc_nodes[q];
        has[n] = 1;
        for (int c = 0; c < 3; c++) {
          const double v = mesh->bc_val[3 * g + c];
          if (mesh->bc_kind[g] == DNL_BC_RESTRAIN) {
            if (v == 1.) codeN[n] = (codeN[n] & ~(3 << (2 * c))) | (1 << (2 * c));
          } else if (v != 0.) {
            codeN[n] = (codeN[n] & ~(3 << (2 * c))) | (2 << (2 * c));
            spdN[3 * (size_t)n + c] = v;
            h->hasSpeedBC = true;
          }
        }
      }
    }
    std::vector<int> idx(N, -1), nodes, codes;
    std::vector<double> spds;
    for (int n = 0; n < N; n++)
      if (has[n] && codeN[n]) {
        idx[n] = (int)nodes.size();
        nodes.push_back(n);
        codes.push_back(codeN[n]);
        for (int c = 0; c < 3; c++) spds.push_back(spdN[3 * (size_t)n + c]);
      }
    h->nbcNodes = (int)nodes.size();
    CKF(cudaMalloc(&h->bcIdx, sizeof(int) * N));
    CKF(cudaMemcpy(h->bcIdx, idx.data(), sizeof(int) * N, cudaMemcpyHostToDevice));
    const size_t nb = nodes.size() ? nodes.size() : 1;
    CKF(cudaMalloc(&h->bcNodeList, sizeof(int) * nb));
    CKF(cudaMalloc(&h->bcCode, sizeof(int) * nb));
    CKF(cudaMalloc(&h->bcSpeed, sizeof(double) * 3 * nb));
    if (nodes.size()) {
      CKF(cudaMemcpy(h->bcNodeList, nodes.data(), sizeof(int) * nodes.size(), cudaMemcpyHostToDevice));
      CKF(cudaMemcpy(h->bcCode, codes.data(), sizeof(int) * codes.size(), cudaMemcpyHostToDevice));
      CKF(cudaMemcpy(h->bcSpeed, spds.data(), sizeof(double) * spds.size(), cudaMemcpyHostToDevice));
    }
  }
  // ---- Pulse: per-Gauss-point kinematics, iterated vector, element products
  if (h->method == DNL_PULSE) {
    const int npj = h->dim * h->dim + 2;
    CKF(cudaMalloc(&h->pj, sizeof(double) * (size_t)npj * h->nIP));
    CKF(cudaMalloc(&h->ev, sizeof(double) * (size_t)h->dim * N));
    CKF(cudaMalloc(&h->kx, sizeof(double) * (size_t)h->dim * E * nen));
    double c[3];
    hooke_entries(m.young, m.nu, c);
    h->C00 = c[0];
    h->C01 = c[1];
    h->C33 = c[2];
  }
  // ---- time state
  CKF(cudaMalloc(&h->tm, sizeof(DevTime)));
  {
    DevTime t;
    memset(&t, 0, sizeof t);
    t.upTime = sp->end_time;
    t.endTime = sp->end_time;
    t.startTime = 0.;
    t.lenMinBits = 0x7ff0000000000000ull;
    t.badElem = -1;
    CKF(cudaMemcpy(h->tm, &t, sizeof t, cudaMemcpyHostToDevice));
  }
  CKF(cudaDeviceSynchronize());
#undef CKF
  return 0;
}


int dnl_add_elements(dnl_handle *h, int etype, int num_elements, const int *conn)
{
  if (!h || !conn || num_elements <= 0 || !etype_valid(etype)) return DNL_ERR_ARG;
  // before the run starts: the lumped mass, the first time step and the element numbering cover
  // every group
  if (h->prologueDone || h->hostIncrement || h->batchUnion) return DNL_ERR_ARG;
  // one family (Domain.C:1042-1060): the 3D reference elements; ElHex8n3D has no Courant length
  if (!solid_reference_element(h->etype) || !solid_reference_element(etype)) return DNL_ERR_ARG;
  if (h->method == DNL_COURANT && etype == DNL_ELHEX8N3D) return DNL_ERR_ARG;
  // one material; no sensitivity or adjoint state
  if (h->elemMat || h->nmat > 1 || h->mat.hard.law != DNL_HARD_POWER || h->sens || h->adj) return DNL_ERR_ARG;
  const int nen = etype_nen(etype), nip = etype_nip(etype), N = h->N, E = num_elements;
  // element-node slots are int32 indices in the node -> slot map
  if (h->EN + (long)E * nen > 2147483647L) return DNL_ERR_ARG;
  for (long i = 0; i < (long)E * nen; i++)
    if (conn[i] < 0 || conn[i] >= N) return DNL_ERR_ARG;
  CK(cudaStreamSynchronize(h->stream));
  for (int i = 0; i < h->ngraphs; i++) cudaGraphExecDestroy(h->graphs[i].exec);
  h->ngraphs = 0;

  ElemGroup g;
  memset(&g, 0, sizeof g);
  g.etype = etype;
  g.nen = nen;
  g.nip = nip;
  g.E = E;
  g.eOff = h->E;
  for (int gi = 0; gi < h->nextra; gi++) g.eOff += h->extra[gi].E;
  g.nIP = (long)E * nip;
  g.feOff = h->EN;
  g.ipOff = ip_total(h);
  double *ipAll = nullptr;  // every group's integration-point state, this group's block last
  auto fail = [&](int code) {
    void *gp[] = {g.conn, ipAll, g.detJ, g.pj, g.Cs, g.stepT};
    for (void *p : gp)
      if (p) cudaFree(p);
    return code;
  };
#define CKG(call)                                                                             \
  do {                                                                                        \
    cudaError_t err_ = (call);                                                                \
    if (err_ != cudaSuccess) {                                                                \
      snprintf(g_lastError, sizeof g_lastError, "%s: %s", #call, cudaGetErrorString(err_));  \
      return fail(DNL_ERR_CUDA);                                                              \
    }                                                                                         \
  } while (0)
  {
    std::vector<int> connT((size_t)nen * E);
    for (int e = 0; e < E; e++)
      for (int k = 0; k < nen; k++) connT[(size_t)k * E + e] = conn[(size_t)e * nen + k];
    CKG(cudaMalloc(&g.conn, sizeof(int) * connT.size()));
    CKG(cudaMemcpy(g.conn, connT.data(), sizeof(int) * connT.size(), cudaMemcpyHostToDevice));
  }
  // one allocation for every group's integration points, each group's [NCOMP][nIP] block after
  // the previous one (a state copy is then one copy); this group's at rest: zero stresses and
  // strains, evp = 1e-10 (IntegrationPoint.C:117)
  const int ns = etype_ns(etype), ncomp = 3 * ns + 3;  // IpLayout::NCOMP (ns = 6 for every solid)
  CKG(cudaMalloc(&ipAll, sizeof(double) * (size_t)ncomp * (g.ipOff + g.nIP)));
  CKG(cudaMemcpy(ipAll, h->ip, sizeof(double) * (size_t)ncomp * g.ipOff, cudaMemcpyDeviceToDevice));
  g.ip = ipAll + (size_t)ncomp * g.ipOff;
  CKG(cudaMemset(g.ip, 0, sizeof(double) * (size_t)ncomp * g.nIP));
  {
    std::vector<double> v(g.nIP, 1e-10);
    CKG(cudaMemcpy(g.ip + (size_t)(3 * ns + 1) * g.nIP, v.data(), sizeof(double) * g.nIP, cudaMemcpyHostToDevice));
    const double pn = pow(1e-10, h->mat.n);
    for (auto &x : v) x = pn;
    CKG(cudaMemcpy(g.ip + (size_t)(3 * ns + 2) * g.nIP, v.data(), sizeof(double) * g.nIP, cudaMemcpyHostToDevice));
  }
  CKG(cudaMalloc(&g.detJ, sizeof(double) * g.nIP));
  if (h->stepT) {  // the handle keeps each step's dEps and R (results files): for this group too
    CKG(cudaMalloc(&g.stepT, sizeof(double) * 18 * (size_t)g.nIP));
    CKG(cudaMemset(g.stepT, 0, sizeof(double) * 18 * (size_t)g.nIP));
  }
  if (h->method == DNL_PULSE) CKG(cudaMalloc(&g.pj, sizeof(double) * (size_t)(h->dim * h->dim + 2) * g.nIP));
  // Courant: Element::getSoundSpeed averages the element's nodal densities over its own node
  // count, which can round differently for another element type; then every element's length is
  // divided by its own group's speed before the minimum (Domain::computeCourantTimeStep)
  dnl_material dm;
  dm.young = h->mat.young;
  dm.poisson = h->mat.nu;
  dm.density = h->mat.rho;
  dm.A = h->mat.A;
  dm.B = h->mat.B;
  dm.n = h->mat.n;
  const double csG = make_material(dm, nen).Cs;
  // (kept per element whenever the step is Courant's: a later dnl_reset with another material can
  // make speeds differ that are equal now)
  const bool perElementCs = h->method == DNL_COURANT;

  // element-force and Pulse-product arrays over the slots of every group; the node -> slot map
  const long EN = h->EN + (long)E * nen;
  double *fe = nullptr, *kx = nullptr, *cs0 = nullptr;
  int *start = nullptr, *entry = nullptr;
  auto freeNew = [&]() {
    void *np[] = {fe, kx, cs0, start, entry};
    for (void *p : np)
      if (p) cudaFree(p);
  };
#define CKN(call)                                                                             \
  do {                                                                                        \
    cudaError_t err_ = (call);                                                                \
    if (err_ != cudaSuccess) {                                                                \
      snprintf(g_lastError, sizeof g_lastError, "%s: %s", #call, cudaGetErrorString(err_));  \
      freeNew();                                                                              \
      return fail(DNL_ERR_CUDA);                                                              \
    }                                                                                         \
  } while (0)
  CKN(cudaMalloc(&fe, sizeof(double) * (size_t)h->dim * EN));
  if (h->method == DNL_PULSE) CKN(cudaMalloc(&kx, sizeof(double) * (size_t)h->dim * EN));
  {
    std::vector<int> all, nenOf;
    if (all_connectivity(h, all, nenOf)) {
      freeNew();
      return fail(DNL_ERR_CUDA);
    }
    for (int e = 0; e < E; e++) {
      for (int k = 0; k < nen; k++) all.push_back(conn[(size_t)e * nen + k]);
      nenOf.push_back(nen);
    }
    // node -> element-node slot, ascending element order (the slots of element e are its first
    // slot + k, elements of every group one after another)
    std::vector<int> st(N + 1, 0), en(all.size()), fill(N, 0);
    for (size_t i = 0; i < all.size(); i++) st[all[i] + 1]++;
    for (int n = 0; n < N; n++) st[n + 1] += st[n];
    size_t slot = 0;
    for (size_t e = 0; e < nenOf.size(); e++)
      for (int k = 0; k < nenOf[e]; k++, slot++) {
        const int n = all[slot];
        en[st[n] + fill[n]++] = (int)slot;
      }
    CKN(cudaMalloc(&start, sizeof(int) * (N + 1)));
    CKN(cudaMalloc(&entry, sizeof(int) * en.size()));
    CKN(cudaMemcpy(start, st.data(), sizeof(int) * (N + 1), cudaMemcpyHostToDevice));
    CKN(cudaMemcpy(entry, en.data(), sizeof(int) * en.size(), cudaMemcpyHostToDevice));
  }
  if (perElementCs) {
    // the first group's and each group's own speed per element
    if (!h->elemCs) {
      std::vector<double> v(h->E, h->mat.Cs);
      CKN(cudaMalloc(&cs0, sizeof(double) * h->E));
      CKN(cudaMemcpy(cs0, v.data(), sizeof(double) * h->E, cudaMemcpyHostToDevice));
    }
    std::vector<double> v(E, csG);
    CKN(cudaMalloc(&g.Cs, sizeof(double) * E));
    CKN(cudaMemcpy(g.Cs, v.data(), sizeof(double) * E, cudaMemcpyHostToDevice));
  }
#undef CKN
#undef CKG
  // commit
  cudaFree(h->ip);
  h->ip = ipAll;
  for (int gi = 0; gi < h->nextra; gi++) h->extra[gi].ip = ipAll + (size_t)ncomp * h->extra[gi].ipOff;
  cudaFree(h->fe);
  h->fe = fe;
  if (kx) {
    cudaFree(h->kx);
    h->kx = kx;
  }
  if (cs0) h->elemCs = cs0;
  cudaFree(h->n2eStart);
  cudaFree(h->n2e);
  h->n2eStart = start;
  h->n2e = entry;
  ElemGroup *grown = new ElemGroup[h->nextra + 1];
  for (int gi = 0; gi < h->nextra; gi++) grown[gi] = h->extra[gi];
  grown[h->nextra] = g;
  delete[] h->extra;
  h->extra = grown;
  h->nextra++;
  h->EN = EN;
  return 0;
}

// ------------------------------------------------------------------------------ state access
namespace {
// the integration points of each element group: its device state (component-major over its own
// points) and its first point in the element order of the host arrays
struct IpSeg {
  double *ip, *stepT;
  size_t nIP, off;
  long eOff;  // the domain's number of the group's first element
  int nip;
};
std::vector<IpSeg> ip_segments(dnl_handle *h)
{
  std::vector<IpSeg> v{{h->ip, h->stepT, (size_t)h->nIP, 0, 0, h->nip}};
  size_t off = h->nIP;
  for (int gi = 0; gi < h->nextra; gi++) {
    const ElemGroup &g = h->extra[gi];
    v.push_back({g.ip, g.stepT, (size_t)g.nIP, off, g.eOff, g.nip});
    off += g.nIP;
  }
  return v;
}
}  // namespace

int dnl_set_state(dnl_handle *h, const dnl_state_view *s)
{
  if (!h || !s) return DNL_ERR_ARG;
  const int N = h->N;
  // the host arrays' copies first, back to back, each into its own staging slot; then the
  // transpositions to the component-major device arrays
  const double *src[5] = {s->coords, s->du, s->v, s->a, s->disp};
  FieldSet fs;
  fs.nf = 0;
  for (int f = 0; f < 5; f++)
    if (src[f]) {
      CK(cudaMemcpyAsync(h->stage + (size_t)f * 3 * N, src[f], sizeof(double) * 3 * (size_t)N,
                         cudaMemcpyHostToDevice, h->stream));
      add_field(h, fs, f);
    }
  int r;
  if ((r = transpose_set(h, fs, true, h->stream))) return r;
  const int ns = etype_ns(h->etype);  // the same for every group of a domain (one family)
  const int I0[6] = {0, 1, 2, 0, 0, 1}, I1[6] = {0, 1, 2, 1, 2, 2};
  CK(cudaStreamSynchronize(h->stream));
  if (!(s->S || s->Eps || s->EpsPlas || s->p || s->evp)) return 0;
  for (const IpSeg &g : ip_segments(h)) {
    const size_t nIP = g.nIP, o = g.off;
    std::vector<double> ib(nIP);
    auto putT = [&](const double *src, int base) -> int {
      for (int k = 0; k < ns; k++) {
        for (size_t i = 0; i < nIP; i++) ib[i] = src[9 * (o + i) + 3 * I0[k] + I1[k]];
        CK(cudaMemcpy(g.ip + (size_t)(base + k) * nIP, ib.data(), sizeof(double) * nIP, cudaMemcpyHostToDevice));
      }
      return 0;
    };
    if (s->S && (r = putT(s->S, 0))) return r;
    if (s->Eps && (r = putT(s->Eps, ns))) return r;
    if (s->EpsPlas && (r = putT(s->EpsPlas, 2 * ns))) return r;
    if (s->p) CK(cudaMemcpy(g.ip + (size_t)(3 * ns) * nIP, s->p + o, sizeof(double) * nIP, cudaMemcpyHostToDevice));
    if (s->evp) {
      CK(cudaMemcpy(g.ip + (size_t)(3 * ns + 1) * nIP, s->evp + o, sizeof(double) * nIP, cudaMemcpyHostToDevice));
      // the cached evp^n: the exponent of each point's element's material
      for (size_t i = 0; i < nIP; i++)
        ib[i] = pow(s->evp[o + i], h->elemMatHost ? h->matExpHost[h->elemMatHost[g.eOff + (long)(i / g.nip)]]
                                                   : h->mat.n);
      CK(cudaMemcpy(g.ip + (size_t)(3 * ns + 2) * nIP, ib.data(), sizeof(double) * nIP, cudaMemcpyHostToDevice));
    }
  }
  return 0;
}

int dnl_get_state(dnl_handle *h, dnl_state_view *s)
{
  if (!h || !s) return DNL_ERR_ARG;
  const int N = h->N;
  // all transpositions into the staging slots, then the copies back to back, one synchronisation
  double *out[5] = {s->coords, s->du, s->v, s->a, s->disp};
  FieldSet fs;
  fs.nf = 0;
  for (int f = 0; f < 5; f++)
    if (out[f]) add_field(h, fs, f);
  int r;
  if ((r = transpose_set(h, fs, false, h->stream))) return r;
  for (int f = 0; f < 5; f++)
    if (out[f])
      CK(cudaMemcpyAsync(out[f], h->stage + (size_t)f * 3 * N, sizeof(double) * 3 * (size_t)N,
                         cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  if (s->mass) CK(cudaMemcpy(s->mass, h->mass, sizeof(double) * N, cudaMemcpyDeviceToHost));
  if (!(s->S || s->Eps || s->EpsPlas || s->p || s->evp || s->Sig)) return 0;
  const int ns = etype_ns(h->etype);  // the same for every group of a domain (one family)
  const int I0[6] = {0, 1, 2, 0, 0, 1}, I1[6] = {0, 1, 2, 1, 2, 2};
  for (const IpSeg &g : ip_segments(h)) {
    const size_t nIP = g.nIP, o = g.off;
    std::vector<double> ib(nIP), pb(nIP);
    auto getT = [&](double *dst, int base, const double *addP) -> int {
      dst += 9 * o;
      for (size_t i = 0; i < 9 * nIP; i++) dst[i] = 0.;
      for (int k = 0; k < ns; k++) {
        CK(cudaMemcpy(ib.data(), g.ip + (size_t)(base + k) * nIP, sizeof(double) * nIP, cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < nIP; i++) {
          dst[9 * i + 3 * I0[k] + I1[k]] = ib[i];
          dst[9 * i + 3 * I1[k] + I0[k]] = ib[i];
        }
      }
      if (addP)
        for (size_t i = 0; i < nIP; i++)
          for (int d = 0; d < 3; d++) dst[9 * i + 4 * d] += addP[i];
      return 0;
    };
    if (s->S && (r = getT(s->S, 0, nullptr))) return r;
    if (s->Eps && (r = getT(s->Eps, ns, nullptr))) return r;
    if (s->EpsPlas && (r = getT(s->EpsPlas, 2 * ns, nullptr))) return r;
    if (s->p || s->Sig) CK(cudaMemcpy(pb.data(), g.ip + (size_t)(3 * ns) * nIP, sizeof(double) * nIP, cudaMemcpyDeviceToHost));
    if (s->p) memcpy(s->p + o, pb.data(), sizeof(double) * nIP);
    if (s->Sig && (r = getT(s->Sig, 0, pb.data()))) return r;
    if (s->evp) CK(cudaMemcpy(s->evp + o, g.ip + (size_t)(3 * ns + 1) * nIP, sizeof(double) * nIP, cudaMemcpyDeviceToHost));
  }
  return 0;
}

int dnl_get_step_tensors(dnl_handle *h, double *dEps, double *R)
{
  if (!h || !h->stepT) return DNL_ERR_ARG;
  CK(cudaStreamSynchronize(h->stream));
  for (const IpSeg &g : ip_segments(h)) {  // every group's points, in element order
    const size_t nIP = g.nIP, o = g.off;
    std::vector<double> ib(nIP);
    for (int k = 0; k < 18; k++) {
      double *dst = k < 9 ? dEps : R;
      if (!dst) continue;
      CK(cudaMemcpy(ib.data(), g.stepT + (size_t)k * nIP, sizeof(double) * nIP, cudaMemcpyDeviceToHost));
      for (size_t i = 0; i < nIP; i++) dst[9 * (o + i) + (k % 9)] = ib[i];
    }
  }
  return 0;
}

int dnl_get_fint(dnl_handle *h, double *fint)
{
  if (!h || !fint) return DNL_ERR_ARG;
  CK(cudaStreamSynchronize(h->stream));
  CK(cudaMemcpy(fint, h->fint, sizeof(double) * (size_t)h->dim * h->N, cudaMemcpyDeviceToHost));
  return 0;
}

// ------------------------------------------------------------------------------ the drop-in
int dnl_internal_forces(dnl_handle *h, const double *coords, const double *du, double dt, double *fint)
{
  (void)dt;  // read by Element::computeStress (Element.C:225) but unused by the J2 update
  if (!h) return DNL_ERR_ARG;
  if (coords || du) {
    dnl_state_view s;
    memset(&s, 0, sizeof s);
    s.coords = const_cast<double *>(coords);
    s.du = const_cast<double *>(du);
    int r = dnl_set_state(h, &s);
    if (r) return r;
  }
  const int zero = 0, minus1 = -1;
  CK(cudaMemcpyAsync(&h->tm->status, &zero, sizeof(int), cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(&h->tm->badElem, &minus1, sizeof(int), cudaMemcpyHostToDevice, h->stream));
  int r;
  if ((r = launch_elem(h, h->stream, 0))) return r;
  if ((r = launch_gather(h))) return r;
  DevTime t;
  if ((r = read_time(h, &t))) return r;
  if (t.status) return t.status;
  if (fint) CK(cudaMemcpy(fint, h->fint, sizeof(double) * (size_t)h->dim * h->N, cudaMemcpyDeviceToHost));
  return 0;
}

// ------------------------------------------------------------------------------ time loop
int dnl_prologue(dnl_handle *h)
{
  if (!h) return DNL_ERR_ARG;
  if (h->prologueDone) return 0;
  int r;
  // computeMassMatrix (ExplicitSolverCH.C:145): per-element lumped masses, gathered per node
  double *me;
  CK(cudaMalloc(&me, sizeof(double) * (size_t)h->EN));
  if ((r = launch_mass(h, h->stream, me))) {
    cudaFree(me);
    return r;
  }
  k_gather1<<<(h->N + 255) / 256, 256, 0, h->stream>>>(h->N, h->n2eStart, h->n2e, me, h->mass);
  launch_counter()++;
  if ((r = check_launch())) {
    cudaFree(me);
    return r;
  }
  CK(cudaStreamSynchronize(h->stream));
  cudaFree(me);
  // computeInternalForces with the initial Current field (:157), then computeTimeStep(True) (:172)
  if ((r = launch_elem(h, h->stream, 1))) return r;
  if ((r = launch_gather(h))) return r;
  if ((r = launch_time_step_source(h))) return r;
  if ((r = launch_dt(h, DT_FORCE))) return r;
  DevTime t;
  if ((r = read_time(h, &t))) return r;
  h->hostIncrement = t.increment;
  h->prologueDone = true;
  return t.status;
}

int dnl_step(dnl_handle *h, int nsteps, int *steps_done)
{
  if (steps_done) *steps_done = 0;
  if (!h || nsteps < 0) return DNL_ERR_ARG;
  int r;
  if (!h->prologueDone && (r = dnl_prologue(h))) return r;
  if (nsteps == 0) return 0;
  const long long inc0 = h->hostIncrement;
  if ((r = launch_dt(h, DT_PRE))) return r;
  for (int s = 0; s < nsteps; s++)
    if ((r = enqueue_step(h, inc0 + s + 1, s == nsteps - 1))) return r;
  DevTime t;
  if ((r = read_time(h, &t))) return r;
  if (steps_done) *steps_done = (int)(t.increment - inc0);
  h->hostIncrement = t.increment;
  // if the run ended early, the bank parity followed the launches, not the steps done
  if (t.increment - inc0 != nsteps) {
    const long long extra = nsteps - (t.increment - inc0);
    if (extra % 2) h->cur = 1 - h->cur;
  }
  return t.status;
}

// nsteps steps with the nodal state exchanged with host memory (dnl_set_state + dnl_step +
// dnl_get_state in one call, the same results).  Coordinates and delta_disp, which the element
// pass reads, are uploaded first on the handle's stream (and v for the one-point hexahedron, whose
// hourglass force reads it); v, a and disp on a second stream while the first element pass runs,
// the boundary conditions' v and a writes after them (k_bc_current_du / _va), and the first nodal
// update waits for that stream.  The download is queued on the second stream as soon as the last
// nodal update has run, beside the next time step's computation.
static int step_host(dnl_handle *h, const dnl_state_view *in, int nsteps, dnl_state_view *out, int *steps_done);

int dnl_step_host(dnl_handle *h, const dnl_state_view *in, int nsteps, dnl_state_view *out, int *steps_done)
{
  const int r = step_host(h, in, nsteps, out, steps_done);
  // a failed launch leaves no work of this call running on the second stream
  if (r == DNL_ERR_CUDA && h && h->ioStream) cudaStreamSynchronize(h->ioStream);
  return r;
}

static int step_host(dnl_handle *h, const dnl_state_view *in, int nsteps, dnl_state_view *out, int *steps_done)
{
  if (steps_done) *steps_done = 0;
  if (!h || nsteps < 1) return DNL_ERR_ARG;
  for (const dnl_state_view *sv : {in, (const dnl_state_view *)out})
    if (sv && (sv->S || sv->Eps || sv->EpsPlas || sv->p || sv->evp || sv->Sig || sv->mass)) return DNL_ERR_ARG;
  int r;
  if (!h->prologueDone && (r = dnl_prologue(h))) return r;
  cudaStream_t s = h->stream;
  if (!h->ioStream) {
    CK(cudaStreamCreateWithFlags(&h->ioStream, cudaStreamNonBlocking));
    for (int i = 0; i < 3; i++) CK(cudaEventCreateWithFlags(&h->ioEv[i], cudaEventDisableTiming));
    CK(cudaMalloc(&h->bcApplied, sizeof(int)));
  }
  cudaStream_t io = h->ioStream;
  const int N = h->N;
  const size_t n3 = 3 * (size_t)N;
  // fields: 0 coords, 1 du, 2 v, 3 a, 4 disp (staging slot f)
  const double *src[5] = {in ? in->coords : nullptr, in ? in->du : nullptr, in ? in->v : nullptr,
                          in ? in->a : nullptr, in ? in->disp : nullptr};
  // the fields of `in` that `pick` selects: copied into their staging slots, then one transposition
  auto upload = [&](bool (*pick)(int, bool), bool vFirstArg, cudaStream_t st) -> int {
    FieldSet fs;
    fs.nf = 0;
    for (int f = 0; f < 5; f++)
      if (src[f] && pick(f, vFirstArg)) {
        CK(cudaMemcpyAsync(h->stage + f * n3, src[f], sizeof(double) * n3, cudaMemcpyHostToDevice, st));
        add_field(h, fs, f);
      }
    return transpose_set(h, fs, true, st);
  };
  // before the element pass: coordinates and delta_disp (and v when the pass reads it); beside it
  // the rest
  auto early = [](int f, bool vf) { return f < 2 || (f == 2 && vf); };
  auto late = [](int f, bool vf) { return f >= 2 && !(f == 2 && vf); };
  const bool vFirst = h->etype == DNL_ELHEX8N3D_1PT;  // its element pass reads Current v
  const bool side = src[3] || src[4] || (src[2] && !vFirst);
  const bool bc = h->nbcNodes > 0;
  if ((r = upload(early, vFirst, s))) return r;
  CK(cudaEventRecord(h->ioEv[0], s));  // the handle's earlier work and these uploads
  const long long inc0 = h->hostIncrement;
  if ((r = launch_dt(h, DT_PRE))) return r;
  for (int k = 0; k < nsteps; k++) {
    const long long incAfter = inc0 + k + 1;
    const bool last = k == nsteps - 1;
    if (k == 0 && side) {
      if (bc) {
        k_bc_current_du<<<(h->nbcNodes + 127) / 128, 128, 0, s>>>(h->nbcNodes, h->bcNodeList, h->bcCode,
                                                                   h->bcSpeed, h->bank[h->cur], h->tm,
                                                                   h->bcApplied);
        launch_counter()++;
        if ((r = check_launch())) return r;
      }
      CK(cudaEventRecord(h->ioEv[1], s));
      if ((r = launch_elem(h, s, 1))) return r;
      // the second stream: v, a, disp beside the element pass, then the boundary conditions'
      // writes to v and a
      CK(cudaStreamWaitEvent(io, h->ioEv[0], 0));
      if ((r = upload(late, vFirst, io))) return r;
      if (bc) {
        CK(cudaStreamWaitEvent(io, h->ioEv[1], 0));
        k_bc_current_va<<<(h->nbcNodes + 127) / 128, 128, 0, io>>>(h->nbcNodes, h->bcNodeList, h->bcCode,
                                                                    h->bcSpeed, h->bank[h->cur], h->bcApplied);
        launch_counter()++;
        if ((r = check_launch())) return r;
      }
      CK(cudaEventRecord(h->ioEv[2], io));
      CK(cudaStreamWaitEvent(s, h->ioEv[2], 0));
    } else {
      if (bc && (r = launch_bc_current(h))) return r;
      if ((r = launch_elem(h, s, 1))) return r;
    }
    if ((r = launch_node(h, true))) return r;
    h->cur = 1 - h->cur;
    if (last && out) {  // the download, beside the time step's computation
      CK(cudaEventRecord(h->ioEv[1], s));
      CK(cudaStreamWaitEvent(io, h->ioEv[1], 0));
      double *dst[5] = {out->coords, out->du, out->v, out->a, out->disp};
      FieldSet fs;
      fs.nf = 0;
      for (int f = 0; f < 5; f++)
        if (dst[f]) add_field(h, fs, f);
      if ((r = transpose_set(h, fs, false, io))) return r;
      for (int f = 0; f < 5; f++)
        if (dst[f]) CK(cudaMemcpyAsync(dst[f], h->stage + f * n3, sizeof(double) * n3, cudaMemcpyDeviceToHost, io));
    }
    if (incAfter % h->freq == 0 && (r = launch_time_step_source(h))) return r;
    if ((r = launch_dt(h, last ? DT_POST : (DT_POST | DT_PRE)))) return r;
  }
  // the handle's later work waits for the second stream (its staging slots, the Current fields)
  CK(cudaEventRecord(h->ioEv[2], io));
  CK(cudaStreamWaitEvent(s, h->ioEv[2], 0));
  DevTime t;
  if ((r = read_time(h, &t))) return r;
  CK(cudaStreamSynchronize(io));
  if (steps_done) *steps_done = (int)(t.increment - inc0);
  h->hostIncrement = t.increment;
  if (t.increment - inc0 != nsteps) {
    // the run ended early: the bank parity follows the steps done, and the fields downloaded
    // above came from the other bank -- download again from the Current one
    if ((nsteps - (t.increment - inc0)) % 2) h->cur = 1 - h->cur;
    if (out) {
      dnl_state_view o = *out;
      if ((r = dnl_get_state(h, &o))) return r;
    }
  }
  return t.status;
}

int dnl_run(dnl_handle *h, int *steps_done)
{
  if (steps_done) *steps_done = 0;
  if (!h) return DNL_ERR_ARG;
  int total = 0, r = 0;
  for (;;) {
    int done = 0;
    r = dnl_step(h, 1000, &done);
    total += done;
    if (r) break;
    DevTime t;
    if ((r = read_time(h, &t))) break;
    if (t.done) break;
  }
  if (steps_done) *steps_done = total;
  return r;
}

int dnl_step_graph(dnl_handle *h, int nsteps, int *steps_done)
{
  if (steps_done) *steps_done = 0;
  if (!h || nsteps <= 0) return DNL_ERR_ARG;
  if (h->method == DNL_PULSE) return DNL_ERR_ARG;  // Pulse iterates to convergence with host checks
  int r;
  if (!h->prologueDone && (r = dnl_prologue(h))) return r;
  const long long inc0 = h->hostIncrement;
  const int parity = h->cur, phase = (int)(inc0 % h->freq);
  cudaGraphExec_t exec = nullptr;
  for (int i = 0; i < h->ngraphs; i++)
    if (h->graphs[i].nsteps == nsteps && h->graphs[i].parity == parity && h->graphs[i].phase == phase)
      exec = h->graphs[i].exec;
  const int curBefore = h->cur;
  if (!exec) {
    cudaGraph_t graph;
    CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    int rr = launch_dt(h, DT_PRE);
    for (int s = 0; s < nsteps && !rr; s++) rr = enqueue_step(h, inc0 + s + 1, s == nsteps - 1);
    cudaError_t ce = cudaStreamEndCapture(h->stream, &graph);
    if (rr) return rr;
    if (ce != cudaSuccess) {
      snprintf(g_lastError, sizeof g_lastError, "graph capture: %s", cudaGetErrorString(ce));
      return DNL_ERR_CUDA;
    }
    CK(cudaGraphInstantiate(&exec, graph, 0));
    cudaGraphDestroy(graph);
    if (h->ngraphs < 8) {
      h->graphs[h->ngraphs++] = GraphEntry{nsteps, parity, phase, exec};
    }
  } else {
    h->cur = (nsteps % 2) ? 1 - curBefore : curBefore;
  }
  CK(cudaGraphLaunch(exec, h->stream));
  launch_counter() += 0;  // kernel launches inside a graph are counted at capture
  DevTime t;
  if ((r = read_time(h, &t))) return r;
  if (steps_done) *steps_done = (int)(t.increment - inc0);
  h->hostIncrement = t.increment;
  if (t.increment - inc0 != nsteps) {
    const long long extra = nsteps - (t.increment - inc0);
    if (extra % 2) h->cur = 1 - h->cur;
  }
  if (h->ngraphs >= 8) {
    bool cached = false;
    for (int i = 0; i < h->ngraphs; i++) cached |= h->graphs[i].exec == exec;
    if (!cached) cudaGraphExecDestroy(exec);
  }
  return t.status;
}

int dnl_time_step(dnl_handle *h, double *dt)
{
  if (!h || !dt) return DNL_ERR_ARG;
  DevTime t;
  int r = read_time(h, &t);
  if (r) return r;
  *dt = t.timeStep;
  return 0;
}

int dnl_dt(dnl_handle *h, double *dt) { return dnl_time_step(h, dt); }

int dnl_get_time_info(dnl_handle *h, dnl_time_info *info)
{
  if (!h || !info) return DNL_ERR_ARG;
  DevTime t;
  int r = read_time(h, &t);
  if (r) return r;
  // kinetic energy of the Current field = the New field of the last step before the swap
  const int blocks = 64;
  double *part;
  CK(cudaMalloc(&part, sizeof(double) * blocks));
  k_kinetic<<<blocks, 256, 0, h->stream>>>(h->N, h->bank[h->cur], h->mass, part);
  launch_counter()++;
  double hp[blocks];
  CK(cudaMemcpyAsync(hp, part, sizeof hp, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  cudaFree(part);
  double ke = 0.;
  for (int b = 0; b < blocks; b++) ke += hp[b];
  info->time = t.currentTime;
  info->time_step = t.timeStep;
  info->computed_step = t.computedTimeStep;
  info->kinetic = ke;
  info->increment = t.increment;
  info->done = t.done;
  info->status = t.status;
  info->bad_element = t.badElem;
  return 0;
}

}  // extern "C"
