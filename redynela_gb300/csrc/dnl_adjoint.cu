// Reverse-mode gradients of an explicit run (dnl_adjoint), with checkpointing.
//
// The run is the scheduled explicit run of dnl_sens_run (ExplicitSolverCH.C:179-274 with the step
// sizes of dnl_set_dt_schedule).  dnl_adjoint returns grad = (dx_final/dp)^T dL/dx_final for the
// hardening parameters A, B, n and the initial-velocity magnitude |v0|, by one forward sweep and
// one reverse sweep:
//
//  * forward: the run from the handle's initial state, with the state (coordinates, the Current
//    nodal field, integration-point state, time record) copied aside before every `stride`-th step
//    -- ceil(n / stride) checkpoints (stride = ceil(sqrt(n)) by default);
//  * reverse: for each segment from the last, the state is restored from its checkpoint and the
//    segment's steps run again, each saving the coordinates, the Current delta_disp the element
//    pass reads and the integration-point state before it (stride records); then the segment's
//    steps are undone in reverse order, each by
//      - the element pass again from its saved state with its per-point record (k_elem<ET, true>),
//      - the adjoint of the nodal update (k_node_adj): Chung-Hulbert corrector and predictor and
//        the constant boundary conditions, whose formulas are linear in the state,
//      - the adjoint of the element pass (k_elem_adj), and
//      - the reverse gather (k_gather_adj): each node sums its element nodes' coordinate and
//        delta_disp adjoints in ascending element order, no atomics.
//    The hardening parameters' derivatives accumulate per integration point over the steps; the
//    initial velocity's is the adjoint of the first step's Current velocity along v0's direction.
//
// Memory: ceil(n / stride) checkpoints plus stride step records, each of the size of the nodal
// fields and integration-point state -- O(sqrt(n)) states instead of the n of a stored trajectory
// -- for one extra forward run of every segment (the recomputation).  The derivative is that of the
// run as computed at the converged return-mapping multipliers and computed eigenpairs, the same
// linearisation as the forward-mode tangent (dnl_sens_run), so the two agree to rounding.
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <vector>

#include "dnl_common.cuh"

namespace dnl {

namespace {

struct AdjState {
  int E = 0, N = 0, nsteps = 0, stride = 0, nseg = 0, etype = -1;
  long nIP = 0;                 // integration points of every element group
  // Per-point arrays below ([X][nIP]) hold one block per element group, [X][nIP_g] at X ipOff, as
  // the handle's integration-point state; gpar alone is [3][nIP] over all points (its sum runs in
  // element order); element-node arrays ([DIM][E NEN]) span every group's slots (EN).
  size_t ckptDoubles = 0, slotDoubles = 0;
  double *mem = nullptr;
  double *ckpt = nullptr;       // nseg x [x(3N) | Current du, v, a, disp (12N) | ip (NCOMP nIP)]
  DevTime *ckptTm = nullptr;    // nseg time records
  std::vector<int> ckptCur;     // Current bank index at each checkpoint
  double *slot = nullptr;       // stride x [x(3N) | Current du (3N) | ip (NCOMP nIP)]
  double *tape = nullptr;       // [NT][nIP]
  double *ipWork = nullptr;     // [NCOMP][nIP]: a step's state, the pass run on it in place
  double *feWork = nullptr;     // [DIM][E NEN]
  DevTime *tmWork = nullptr;
  double *lam[2] = {nullptr, nullptr};  // nodal adjoints [du, v, a, disp][3][N]
  double *xbar = nullptr, *fbar = nullptr;  // [3][N]
  double *ipAdj = nullptr;      // [TanLayout::NCOMP][nIP]
  double *xe = nullptr, *ue = nullptr;  // [DIM][E NEN]
  double *gpar = nullptr;       // [3][nIP]
  // each step's per-point record [NT][nIP] of the segment being undone, written by its
  // recomputation when stride x NT x nIP doubles fit kept_record_budget(); otherwise the reverse
  // step runs the element pass again from the step's stored state to regenerate it
  double *tapes = nullptr;
  size_t tapeDoubles = 0;
  double *dts = nullptr;        // the schedule on the device
  double *host = nullptr;       // page-locked staging, 3 max(N, nIP) doubles
  size_t bytes = 0;
  long long recomputed = 0;
  dnl_adjoint_info info;        // figures of the last dnl_adjoint
  bool hasInfo = false;
  double *runDts = nullptr;     // dnl_run_schedule's schedule on the device
  double *runOut = nullptr;     // and its staging for the coordinates (3N)
  int runCap = 0, runN = 0;
  std::vector<double> sched;    // the schedule of the last forward sweep (host)
  bool ready = false;           // a forward sweep's checkpoints await the reverse sweep
  // segments replayed from captured graphs: kind (0 forward, 1 recomputation with records,
  // 2 reverse), length, the handle's bank parity and the adjoint bank at the segment's start
  struct SegGraph {
    int kind, len, cur, nw;
    cudaGraphExec_t exec;
    long long kernels;
  };
  std::vector<SegGraph> graphs;
  Material graphMat;            // the material the graphs hold by value
};

void adj_drop_graphs(AdjState *A)
{
  for (auto &g : A->graphs) cudaGraphExecDestroy(g.exec);
  A->graphs.clear();
}

// the time record between scheduled steps: phase 0 initStep with the scheduled step, 1 updateTime,
// 2 both (updateTime of one step then initStep of the next: one launch between two steps)
__global__ void k_adj_dt(DevTime *tm, const double *dts, int phase)
{
  if (tm->status) return;
  if (phase != 0)  // updateTime
    tm->currentTime = __dadd_rn(tm->currentTime, tm->timeStep);
  if (phase != 1) {  // initStep with the scheduled step
    const double dt = dts[tm->increment];
    tm->timeStep = dt;
    tm->nextTime = __dadd_rn(tm->currentTime, dt);
    tm->increment++;
  }
}

// a step's record: the coordinates (3N), the Current delta_disp (3N) and the integration-point
// state (n doubles) copied into rec one after another, in one launch
__global__ void k_adj_record(long N, long nip, const double *x, const double *du, const double *ip,
                             double *rec)
{
  const long total = 6 * N + nip;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x)
    rec[i] = i < 3 * N ? x[i] : (i < 6 * N ? du[i - 3 * N] : ip[i - 6 * N]);
}

struct AdjNodeArgs {
  int N;
  const double *mass;
  const int *bcIdx, *bcCode;
  const double *ln;  // adjoints of the New field after the step, [du, v, a, disp][3][N]
  double *lc;        // adjoints of the Current field before it (v, a, disp written here)
  const double *xbar;
  double *fbar;
  const double *dts; // the schedule; the step undone is the time record's increment - 1
  const DevTime *tm;
  double alphaM, beta, gamma;
};

// Adjoint of node_update (dnl_host.cu) for one node.  Per free component, with
// u = adj(New du) + adj(New disp) + adj(x') (delta_disp feeds the New field, the displacement and
// the coordinates) and a' = adj(New a) + dt gamma adj(New v) + dt^2 beta u:
//   adj(F) = a' / (m (1 - alphaM)),
//   adj(Current a) = -alphaM / (1 - alphaM) a' + dt (1 - gamma) adj(New v) + dt^2 (1/2 - beta) u,
//   adj(Current v) = adj(New v) + dt u,  adj(Current disp) = adj(New disp).
// A restrained or imposed-speed component's New du, v, a are constants: no force or Current
// velocity / acceleration adjoint from it.
template <int DIM>
__global__ void __launch_bounds__(256) k_node_adj(AdjNodeArgs g)
{
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= g.N) return;
  const long N = g.N;
  const int bc = g.bcIdx[n];
  const int code = bc >= 0 ? g.bcCode[bc] : 0;
  const double dt = g.dts[g.tm->increment - 1];
  const double rm = 1.0 / g.mass[n], roma = 1.0 / (1.0 - g.alphaM);
  const double c1 = dt * (0.5 - g.beta), c2 = dt * (1.0 - g.gamma);
  const double cg = dt * g.gamma, cb = dt * dt * g.beta;
#pragma unroll
  for (int i = 0; i < DIM; i++) {
    const long o = (long)i * N + n;
    const double nu = g.ln[o], nv = g.ln[3 * N + o], na = g.ln[6 * N + o], nd = g.ln[9 * N + o];
    const double u = nu + nd + g.xbar[o];
    double fb = 0., cv = 0., ca = 0.;
    if (!((code >> (2 * i)) & 3)) {
      const double ab = fma(cb, u, fma(cg, nv, na));
      fb = ab * rm * roma;
      ca = fma(-g.alphaM * roma, ab, fma(c2, nv, dt * c1 * u));
      cv = fma(dt, u, nv);
    }
    g.fbar[o] = fb;
    g.lc[3 * N + o] = cv;
    g.lc[6 * N + o] = ca;
    g.lc[9 * N + o] = nd;
  }
}

// Reverse gather: adj(x) += sum of the element nodes' coordinate adjoints, adj(Current du) = sum of
// their delta_disp adjoints (ascending element order, as k_gather); then the constant boundary
// conditions, which overwrite the Current du, v, a of their components before the element pass
// reads them (k_bc_current), zero those components' adjoints.  The time record's increment steps
// back to the step undone next, whose size the next k_node_adj reads from the schedule.
template <int DIM>
__global__ void __launch_bounds__(256) k_gather_adj(int N, int EN, const int *start, const int *entry,
                                                    const double *xe, const double *ue, double *xbar,
                                                    double *lc, const int *bcIdx, const int *bcCode,
                                                    DevTime *tm)
{
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n == 0) tm->increment--;  // the step undone; nothing else in this kernel reads the record
  if (n >= N) return;
  double sx[DIM], su[DIM];
#pragma unroll
  for (int c = 0; c < DIM; c++) sx[c] = su[c] = 0.;
  for (int q = start[n]; q < start[n + 1]; q++) {
    const int ent = __ldg(entry + q);
#pragma unroll
    for (int c = 0; c < DIM; c++) {
      sx[c] += __ldg(xe + (long)c * EN + ent);
      su[c] += __ldg(ue + (long)c * EN + ent);
    }
  }
  const int bc = bcIdx[n];
  const int code = bc >= 0 ? bcCode[bc] : 0;
#pragma unroll
  for (int c = 0; c < DIM; c++) {
    const long o = (long)c * N + n;
    xbar[o] += sx[c];
    const bool fixed = (code >> (2 * c)) & 3;
    lc[o] = fixed ? 0. : su[c];
    if (fixed) {
      lc[3L * N + o] = 0.;
      lc[6L * N + o] = 0.;
    }
  }
}

// dL/d|v0| = sum over nodes of adj(Current v) at the first step . u (u = v0 / |v0|), and the
// per-point parameter sums, reduced in a fixed order by one block
__global__ void k_adj_reduce(int N, long nIP, const double *lcv, double u0, double u1, double u2,
                             const double *gpar, double *out)
{
  __shared__ double sh[4][256];
  double s[4] = {0., 0., 0., 0.};
  for (long i = threadIdx.x; i < nIP; i += blockDim.x)
    for (int p = 0; p < 3; p++) s[p] += gpar[p * nIP + i];
  for (int n = threadIdx.x; n < N; n += blockDim.x)
    s[3] += fma(lcv[n], u0, fma(lcv[(long)N + n], u1, lcv[2L * N + n] * u2));
  for (int p = 0; p < 4; p++) sh[p][threadIdx.x] = s[p];
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o)
      for (int p = 0; p < 4; p++) sh[p][threadIdx.x] += sh[p][threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x < 4) out[threadIdx.x] = sh[threadIdx.x][0];
}

__global__ void k_aos3(int N, const double *soa, double *aos)
{
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
#pragma unroll
  for (int c = 0; c < 3; c++) aos[3L * n + c] = soa[(long)c * N + n];
}

__global__ void k_soa3(int N, const double *aos, double *soa)
{
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
#pragma unroll
  for (int c = 0; c < 3; c++) soa[(long)c * N + n] = aos[3L * n + c];
}

#define CKA(x)                                      \
  do {                                              \
    if ((x) != cudaSuccess) return DNL_ERR_CUDA;    \
  } while (0)

int ip_ncomp(int etype) { return 3 * etype_ns(etype) + 3; }
int tan_ncomp_of(int etype) { return 3 * etype_ns(etype) + 2; }
int tape_nt_of(int etype)
{
  return etype_dim(etype) == 3 ? TapeLayout<DNL_ELHEX8N3D>::NT : TapeLayout<DNL_ELQUA4NAX>::NT;
}

void adj_release(AdjState *A)
{
  adj_drop_graphs(A);
  if (A->runDts) cudaFree(A->runDts);
  if (A->runOut) cudaFree(A->runOut);
  if (A->mem) cudaFree(A->mem);
  if (A->ckptTm) cudaFree(A->ckptTm);
  if (A->tmWork) cudaFree(A->tmWork);
  if (A->dts) cudaFree(A->dts);
  if (A->host) cudaFreeHost(A->host);
  *A = AdjState();
}

// device memory the reverse sweep may spend on keeping a segment's per-point records
// (dnl_set_adjoint_record_budget; 2 GiB by default)
size_t &kept_record_budget()
{
  static size_t bytes = size_t(2) << 30;
  return bytes;
}

int adj_alloc(dnl_handle *h, AdjState *A, int nsteps, int stride)
{
  const int nseg = (nsteps + stride - 1) / stride;
  const size_t nIP0 = ip_total(h);
  const bool keep = sizeof(double) * (size_t)stride * tape_nt_of(h->etype) * nIP0 <= kept_record_budget();
  if (A->mem && A->E == h->E && A->N == h->N && A->nIP == (long)nIP0 && A->etype == h->etype &&
      A->stride == stride && A->nsteps == nsteps && (A->tapes != nullptr) == keep)
    return 0;
  {
    double *rd = A->runDts, *ro = A->runOut;
    const int rc = A->runCap, rn = A->runN;
    A->runDts = A->runOut = nullptr;
    adj_release(A);
    A->runDts = rd;
    A->runOut = ro;
    A->runCap = rc;
    A->runN = rn;
  }
  // per-point arrays over every element group's points (each group's block at its ipOff; one
  // layout width per dimension), element-node arrays over every group's slots
  const size_t N = h->N, nIP = nIP0, EN = (size_t)h->EN;
  const int NC = ip_ncomp(h->etype), NT = tape_nt_of(h->etype), TC = tan_ncomp_of(h->etype);
  A->E = h->E;
  A->N = h->N;
  A->nIP = (long)nIP;
  A->etype = h->etype;
  A->nsteps = nsteps;
  A->stride = stride;
  A->nseg = nseg;
  A->ckptDoubles = 15 * N + NC * nIP;
  A->slotDoubles = 6 * N + NC * nIP;
  A->tapeDoubles = NT * nIP;
  const size_t total = nseg * A->ckptDoubles + stride * A->slotDoubles + NT * nIP + NC * nIP +
                       h->dim * EN + 2 * 12 * N + 6 * N + TC * nIP + 2 * h->dim * EN + 3 * nIP +
                       (keep ? stride * A->tapeDoubles : 0);
  CKA(cudaMalloc(&A->mem, sizeof(double) * total));
  CKA(cudaMalloc(&A->ckptTm, sizeof(DevTime) * nseg));
  CKA(cudaMalloc(&A->tmWork, sizeof(DevTime)));
  CKA(cudaMalloc(&A->dts, sizeof(double) * nsteps));
  const size_t hostN = 4 * (N > nIP ? N : nIP);
  CKA(cudaMallocHost(&A->host, sizeof(double) * hostN));
  double *p = A->mem;
  A->ckpt = p;
  p += nseg * A->ckptDoubles;
  A->slot = p;
  p += stride * A->slotDoubles;
  A->tape = p;
  p += NT * nIP;
  A->ipWork = p;
  p += NC * nIP;
  A->feWork = p;
  p += h->dim * EN;
  A->lam[0] = p;
  p += 12 * N;
  A->lam[1] = p;
  p += 12 * N;
  A->xbar = p;
  p += 3 * N;
  A->fbar = p;
  p += 3 * N;
  A->ipAdj = p;
  p += TC * nIP;
  A->xe = p;
  p += h->dim * EN;
  A->ue = p;
  p += h->dim * EN;
  A->gpar = p;
  p += 3 * nIP;
  A->tapes = keep ? p : nullptr;
  A->ckptCur.assign(nseg, 0);
  A->bytes = sizeof(double) * total + sizeof(DevTime) * (nseg + 1) + sizeof(double) * nsteps;
  return 0;
}

// one scheduled explicit step of the handle (the launches of dnl_sens_run's primal); with `rec`,
// the coordinates, the Current delta_disp and the integration-point state the element pass reads
// are copied there first
// `first`: the step opens with initStep; `last`: it ends with updateTime; between two steps of a
// sequence one launch does both (the same operations in the same order)
int adj_primal_step(dnl_handle *h, const double *dtsDev, double *rec, double *tapeOut = nullptr,
                    bool first = true, bool last = true)
{
  cudaStream_t s = h->stream;
  const size_t N = h->N, nIP = ip_total(h);  // one allocation holds every group's state
  if (first) {
    k_adj_dt<<<1, 1, 0, s>>>(h->tm, dtsDev, 0);
    launch_counter()++;
  }
  int r;
  if ((r = enqueue_bc_current(h))) return r;
  if (rec) {
    const long total = 6 * (long)N + (long)ip_ncomp(h->etype) * nIP;
    k_adj_record<<<(unsigned)((total + 255) / 256 < 4096 ? (total + 255) / 256 : 4096), 256, 0, s>>>(
        (long)N, (long)ip_ncomp(h->etype) * nIP, h->x[0], h->bank[h->cur].du[0], h->ip, rec);
    launch_counter()++;
  }
  // with tapeOut: the same pass (bit for bit) also writing its per-point record there
  if ((r = tapeOut ? launch_elem_tape(h, s, tapeOut) : launch_elem(h, s, 1))) return r;
  if ((r = enqueue_node(h))) return r;
  h->cur = 1 - h->cur;
  k_adj_dt<<<1, 1, 0, s>>>(h->tm, dtsDev, last ? 1 : 2);
  launch_counter()++;
  return cudaPeekAtLastError() == cudaSuccess ? 0 : DNL_ERR_CUDA;
}

int adj_save(dnl_handle *h, AdjState *A, int seg)
{
  cudaStream_t s = h->stream;
  const size_t N = h->N, nIP = A->nIP;
  double *c = A->ckpt + seg * A->ckptDoubles;
  CKA(cudaMemcpyAsync(c, h->x[0], sizeof(double) * 3 * N, cudaMemcpyDeviceToDevice, s));
  CKA(cudaMemcpyAsync(c + 3 * N, h->bank[h->cur].du[0], sizeof(double) * 12 * N, cudaMemcpyDeviceToDevice, s));
  CKA(cudaMemcpyAsync(c + 15 * N, h->ip, sizeof(double) * ip_ncomp(h->etype) * nIP, cudaMemcpyDeviceToDevice, s));
  CKA(cudaMemcpyAsync(A->ckptTm + seg, h->tm, sizeof(DevTime), cudaMemcpyDeviceToDevice, s));
  A->ckptCur[seg] = h->cur;
  return 0;
}

int adj_restore(dnl_handle *h, AdjState *A, int seg)
{
  cudaStream_t s = h->stream;
  const size_t N = h->N, nIP = A->nIP;
  h->cur = A->ckptCur[seg];
  const double *c = A->ckpt + seg * A->ckptDoubles;
  CKA(cudaMemcpyAsync(h->x[0], c, sizeof(double) * 3 * N, cudaMemcpyDeviceToDevice, s));
  CKA(cudaMemcpyAsync(h->bank[h->cur].du[0], c + 3 * N, sizeof(double) * 12 * N, cudaMemcpyDeviceToDevice, s));
  CKA(cudaMemcpyAsync(h->ip, c + 15 * N, sizeof(double) * ip_ncomp(h->etype) * nIP, cudaMemcpyDeviceToDevice, s));
  CKA(cudaMemcpyAsync(h->tm, A->ckptTm + seg, sizeof(DevTime), cudaMemcpyDeviceToDevice, s));
  return 0;
}

// undo one step from its record: its per-point record (kept from the recomputation in `tape`, or
// regenerated by running the pass again on the step's stored state), then the adjoints of the
// nodal update, the element pass and the gather; ln / lc: the New / Current nodal adjoints; ipOut:
// the integration-point state after the step (with a kept record)
int adj_reverse_step(dnl_handle *h, AdjState *A, const double *rec, const double *ln, double *lc,
                     const double *tape = nullptr, const double *ipOut = nullptr)
{
  cudaStream_t s = h->stream;
  const size_t N = h->N, nIP = A->nIP;
  const int NC = ip_ncomp(h->etype), NT = tape_nt_of(h->etype), TC = tan_ncomp_of(h->etype);
  int r = 0;
  if (!tape) {
    CKA(cudaMemcpyAsync(A->ipWork, rec + 6 * N, sizeof(double) * NC * nIP, cudaMemcpyDeviceToDevice, s));
    prof_begin(h, s);
    for (int gi = -1; gi < h->nextra && !r; gi++) {
      const long ipOff = gi < 0 ? 0 : h->extra[gi].ipOff, feOff = gi < 0 ? 0 : h->extra[gi].feOff;
      ElemArgs ea = group_args_of(h, gi);
      ea.gate = 0;
      for (int c = 0; c < 3; c++) {
        ea.x[c] = const_cast<double *>(rec) + c * N;
        ea.du[c] = rec + 3 * N + c * N;
      }
      ea.ip = A->ipWork + NC * ipOff;
      ea.fe = A->feWork + feOff;
      ea.detJ = nullptr;
      ea.stepT = nullptr;
      ea.tape = A->tape + NT * ipOff;
      ea.tm = A->tmWork;
      r = launch_elem_tape_raw(gi < 0 ? h->etype : h->extra[gi].etype, ea, s);
    }
    prof_end(h, DNL_PROF_ELEM, s);
    if (r) return r;
    tape = A->tape;
    ipOut = A->ipWork;
  }
  AdjNodeArgs g;
  g.N = h->N;
  g.mass = h->mass;
  g.bcIdx = h->bcIdx;
  g.bcCode = h->bcCode;
  g.ln = ln;
  g.lc = lc;
  g.xbar = A->xbar;
  g.fbar = A->fbar;
  g.dts = A->dts;
  g.tm = h->tm;
  g.alphaM = h->alphaM;
  g.beta = h->beta;
  g.gamma = h->gamma;
  const int gridN = (h->N + 255) / 256;
  prof_begin(h, s);
  if (h->dim == 2)
    k_node_adj<2><<<gridN, 256, 0, s>>>(g);
  else
    k_node_adj<3><<<gridN, 256, 0, s>>>(g);
  prof_end(h, DNL_PROF_NODE, s);
  launch_counter()++;
  AdjElemArgs aa;
  aa.N = h->N;
  for (int c = 0; c < 3; c++) aa.x[c] = rec + c * N;
  aa.fbar = A->fbar;
  aa.feStride = h->EN;
  aa.gStride = (long)nIP;
  aa.mat = h->mat;
  prof_begin(h, s);
  // each element group on its own blocks of the per-point arrays and its own element-node slots
  for (int gi = -1; gi < h->nextra && !r; gi++) {
    const long ipOff = gi < 0 ? 0 : h->extra[gi].ipOff, feOff = gi < 0 ? 0 : h->extra[gi].feOff;
    aa.E = gi < 0 ? h->E : h->extra[gi].E;
    aa.conn = gi < 0 ? h->conn : h->extra[gi].conn;
    aa.tape = tape + NT * ipOff;
    aa.ipOut = ipOut + NC * ipOff;
    aa.ipAdj = A->ipAdj + TC * ipOff;
    aa.xe = A->xe + feOff;
    aa.ue = A->ue + feOff;
    aa.gpar = A->gpar + ipOff;
    r = launch_elem_adj(gi < 0 ? h->etype : h->extra[gi].etype, aa, s);
  }
  prof_end(h, DNL_PROF_TANGENT, s);
  if (r) return r;
  prof_begin(h, s);
  if (h->dim == 2)
    k_gather_adj<2><<<gridN, 256, 0, s>>>(h->N, (int)h->EN, h->n2eStart, h->n2e, A->xe, A->ue,
                                          A->xbar, lc, h->bcIdx, h->bcCode, h->tm);
  else
    k_gather_adj<3><<<gridN, 256, 0, s>>>(h->N, (int)h->EN, h->n2eStart, h->n2e, A->xe, A->ue,
                                          A->xbar, lc, h->bcIdx, h->bcCode, h->tm);
  prof_end(h, DNL_PROF_NODE, s);
  launch_counter()++;
  return cudaPeekAtLastError() == cudaSuccess ? 0 : DNL_ERR_CUDA;
}

// `len` steps of one kind from the handle's bank parity h->cur and adjoint bank nw: 0 the forward
// steps, 1 the recomputation writing the step records, 2 the reverse steps (from the last record).
// Segments of two steps or more replay a graph captured on first use (one per kind, length, parity
// and adjoint bank: every full segment of a run shares them); profiled runs launch step by step.
int adj_segment(dnl_handle *h, AdjState *A, int kind, int len, int &nw)
{
  auto enqueue = [&]() -> int {
    int r;
    if (kind == 2) {
      for (int j = len - 1; j >= 0; j--) {
        // with kept records: step j's record, and the state after it -- the next step's stored
        // state, or the handle's own after the segment's last step
        const double *tape = A->tapes ? A->tapes + j * A->tapeDoubles : nullptr;
        const double *ipOut = j < len - 1 ? A->slot + (j + 1) * A->slotDoubles + 6 * (size_t)h->N : h->ip;
        if ((r = adj_reverse_step(h, A, A->slot + j * A->slotDoubles, A->lam[nw], A->lam[1 - nw], tape,
                                  tape ? ipOut : nullptr)))
          return r;
        nw = 1 - nw;
      }
      return 0;
    }
    for (int j = 0; j < len; j++)
      if ((r = adj_primal_step(h, A->dts, kind == 1 ? A->slot + j * A->slotDoubles : nullptr,
                               kind == 1 && A->tapes ? A->tapes + j * A->tapeDoubles : nullptr, j == 0,
                               j == len - 1)))
        return r;
    return 0;
  };
  if (h->profiling || len < 2) return enqueue();
  if (!A->graphs.empty() && memcmp(&A->graphMat, &h->mat, offsetof(Material, hard)) != 0) adj_drop_graphs(A);
  cudaStream_t s = h->stream;
  const int cur0 = h->cur, nw0 = nw;
  AdjState::SegGraph *g = nullptr;
  for (auto &x : A->graphs)
    if (x.kind == kind && x.len == len && x.cur == cur0 && x.nw == nw0) g = &x;
  if (!g) {
    const long long k0 = launch_counter();
    cudaGraph_t graph;
    CKA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    const int rr = enqueue();
    const cudaError_t ce = cudaStreamEndCapture(s, &graph);
    h->cur = cur0;  // captured, not run
    nw = nw0;
    if (rr) {
      if (ce == cudaSuccess) cudaGraphDestroy(graph);
      return rr;
    }
    if (ce != cudaSuccess) return DNL_ERR_CUDA;
    cudaGraphExec_t exec;
    const cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ie != cudaSuccess) return DNL_ERR_CUDA;
    A->graphs.push_back(AdjState::SegGraph{kind, len, cur0, nw0, exec, launch_counter() - k0});
    launch_counter() = k0;
    A->graphMat = h->mat;
    g = &A->graphs.back();
  }
  CKA(cudaGraphLaunch(g->exec, s));
  launch_counter() += g->kernels;
  if (kind == 2)
    nw = (len & 1) ? 1 - nw0 : nw0;
  else
    h->cur = (len & 1) ? 1 - cur0 : cur0;
  return 0;
}

}  // namespace

void adj_free(dnl_handle *h)
{
  AdjState *A = (AdjState *)h->adj;
  if (!A) return;
  adj_release(A);
  delete A;
  h->adj = nullptr;
}

// forward sweep: the scheduled run from the initial state with a checkpoint before every
// `stride`-th step; the final coordinates are left in the handle
int adjoint_forward(dnl_handle *h, const double *dts, int nsteps, int stride)
{
  if (!etype_has_sens(h->etype) || h->etype == DNL_ELHEX8N3D_1PT) return DNL_ERR_ARG;
  if (h->elemMat || h->mat.hard.law != DNL_HARD_POWER) return DNL_ERR_ARG;
  if (stride <= 0) {
    // ceil(sqrt(n)), made even so that every full segment starts on the same nodal-field bank and
    // replays the same graphs
    stride = (int)ceil(sqrt((double)nsteps));
    stride += stride & 1;
  }
  if (stride > nsteps) stride = nsteps;
  if (!h->adj) h->adj = new AdjState();
  AdjState *A = (AdjState *)h->adj;
  int r;
  A->ready = false;
  if ((r = adj_alloc(h, A, nsteps, stride))) return r;
  cudaStream_t s = h->stream;
  CKA(cudaMemcpyAsync(A->dts, dts, sizeof(double) * nsteps, cudaMemcpyHostToDevice, s));
  A->sched.assign(dts, dts + nsteps);
  A->recomputed = 0;
  int nw = 0;
  for (int seg = 0; seg < A->nseg; seg++) {
    if ((r = adj_save(h, A, seg))) return r;
    const int len = seg == A->nseg - 1 ? nsteps - seg * stride : stride;
    if ((r = adj_segment(h, A, 0, len, nw))) return r;
  }
  DevTime t;
  CKA(cudaMemcpyAsync(&t, h->tm, sizeof t, cudaMemcpyDeviceToHost, s));
  CKA(cudaStreamSynchronize(s));
  if (t.status) return t.status;
  A->ready = true;
  return 0;
}

// reverse sweep over the checkpoints of the last forward sweep, from dL/dx_final (3N node-major);
// the handle is back at its initial state afterwards
int adjoint_backward(dnl_handle *h, const double *dL_dx, double *grad, dnl_adjoint_info *info)
{
  AdjState *A = (AdjState *)h->adj;
  if (!A || !A->ready) return DNL_ERR_ARG;
  A->ready = false;
  int r;
  cudaStream_t s = h->stream;
  const size_t N = h->N, nIP = A->nIP;
  const int nsteps = A->nsteps, stride = A->stride;
  memcpy(A->host, dL_dx, sizeof(double) * 3 * N);
  CKA(cudaMemcpyAsync(A->fbar, A->host, sizeof(double) * 3 * N, cudaMemcpyHostToDevice, s));
  k_soa3<<<(unsigned)((N + 255) / 256), 256, 0, s>>>((int)N, A->fbar, A->xbar);
  launch_counter()++;
  CKA(cudaMemsetAsync(A->lam[0], 0, sizeof(double) * 24 * N, s));
  CKA(cudaMemsetAsync(A->ipAdj, 0, sizeof(double) * tan_ncomp_of(h->etype) * nIP, s));
  CKA(cudaMemsetAsync(A->gpar, 0, sizeof(double) * 3 * nIP, s));
  if (h->dim == 2) CKA(cudaMemsetAsync(A->xbar + 2 * N, 0, sizeof(double) * N, s));

  int nw = 0;  // lam[nw]: adjoints of the New field after the step being undone
  for (int seg = A->nseg - 1; seg >= 0; seg--) {
    if ((r = adj_restore(h, A, seg))) return r;
    const int len = seg == A->nseg - 1 ? nsteps - seg * stride : stride;
    if ((r = adj_segment(h, A, 1, len, nw))) return r;
    A->recomputed += len;
    if ((r = adj_segment(h, A, 2, len, nw))) return r;
  }
  // lam[nw] now holds the adjoints of the first step's Current field
  k_adj_reduce<<<1, 256, 0, s>>>((int)N, (long)nIP, A->lam[nw] + 3 * N, h->v0dir[0], h->v0dir[1],
                                 h->v0dir[2], A->gpar, A->fbar);
  launch_counter()++;
  double out[4];
  CKA(cudaMemcpyAsync(out, A->fbar, sizeof out, cudaMemcpyDeviceToHost, s));
  CKA(cudaStreamSynchronize(s));
  CKA(cudaGetLastError());
  for (int p = 0; p < 4; p++) grad[p] = out[p];
  // back to the initial state: the first checkpoint
  if ((r = adj_restore(h, A, 0))) return r;
  CKA(cudaStreamSynchronize(s));
  if (info) {
    info->checkpoints = A->nseg;
    info->stride = stride;
    info->nsteps = nsteps;
    info->recomputed_steps = A->recomputed;
    info->bytes = (long long)A->bytes;
    info->checkpoint_bytes = (long long)(sizeof(double) * A->nseg * A->ckptDoubles);
    info->record_bytes = (long long)(sizeof(double) * A->stride * A->slotDoubles);
    info->kept_record_bytes = A->tapes ? (long long)(sizeof(double) * A->stride * A->tapeDoubles) : 0;
  }
  return 0;
}

}  // namespace dnl

using namespace dnl;

extern "C" {

int dnl_adjoint_forward(dnl_handle *h, int ckpt_stride, double *coords)
{
  if (!h || ckpt_stride < 0) return DNL_ERR_ARG;
  const double *dts;
  int n;
  if (sens_schedule(h, &dts, &n)) return DNL_ERR_ARG;
  if (h->hostIncrement != 0) return DNL_ERR_ARG;  // starts from the initial state
  int r;
  if (!h->prologueDone && (r = dnl_prologue(h))) return r;
  if ((r = adjoint_forward(h, dts, n, ckpt_stride))) return r;
  AdjState *A = (AdjState *)h->adj;
  h->hostIncrement = n;
  if (coords) {
    cudaStream_t s = h->stream;
    k_aos3<<<(unsigned)((h->N + 255) / 256), 256, 0, s>>>(h->N, h->x[0], A->fbar);
    launch_counter()++;
    CKA(cudaMemcpyAsync(coords, A->fbar, sizeof(double) * 3 * (size_t)h->N, cudaMemcpyDeviceToHost, s));
    CKA(cudaStreamSynchronize(s));
  }
  return 0;
}

int dnl_adjoint_backward(dnl_handle *h, const double *dL_dx, double *grad)
{
  if (!h || !dL_dx || !grad || !h->adj || !((AdjState *)h->adj)->ready) return DNL_ERR_ARG;
  dnl_adjoint_info info;
  memset(&info, 0, sizeof info);
  int r = adjoint_backward(h, dL_dx, grad, &info);
  if (r) return r;
  AdjState *A = (AdjState *)h->adj;
  A->info = info;
  A->hasInfo = true;
  h->hostIncrement = 0;
  return 0;
}

int dnl_adjoint(dnl_handle *h, const double *dL_dx, double *grad, int ckpt_stride)
{
  if (!h || !dL_dx || !grad || ckpt_stride < 0) return DNL_ERR_ARG;
  int r;
  if ((r = dnl_adjoint_forward(h, ckpt_stride, nullptr))) return r;
  return dnl_adjoint_backward(h, dL_dx, grad);
}

int dnl_set_adjoint_record_budget(unsigned long long bytes)
{
  kept_record_budget() = (size_t)bytes;
  return 0;
}

int dnl_adjoint_stats(dnl_handle *h, dnl_adjoint_info *info)
{
  if (!h || !info || !h->adj || !((AdjState *)h->adj)->hasInfo) return DNL_ERR_ARG;
  *info = ((AdjState *)h->adj)->info;
  return 0;
}

int dnl_run_schedule(dnl_handle *h, int nsteps, const double *dts, double *coords)
{
  if (!h || nsteps <= 0 || !dts) return DNL_ERR_ARG;
  for (int k = 0; k < nsteps; k++)
    if (!(dts[k] > 0. && dts[k] < 1e300)) return DNL_ERR_ARG;
  if (h->hostIncrement != 0) return DNL_ERR_ARG;  // starts from the initial state
  int r;
  if (!h->prologueDone && (r = dnl_prologue(h))) return r;
  if (!h->adj) h->adj = new AdjState();
  AdjState *A = (AdjState *)h->adj;
  cudaStream_t s = h->stream;
  if (A->runCap < nsteps || A->runN != h->N) {
    if (A->runDts) cudaFree(A->runDts);
    if (A->runOut) cudaFree(A->runOut);
    A->runDts = A->runOut = nullptr;
    A->runCap = 0;
    CKA(cudaMalloc(&A->runDts, sizeof(double) * nsteps));
    CKA(cudaMalloc(&A->runOut, sizeof(double) * 3 * (size_t)h->N));
    A->runCap = nsteps;
    A->runN = h->N;
  }
  CKA(cudaMemcpyAsync(A->runDts, dts, sizeof(double) * nsteps, cudaMemcpyHostToDevice, s));
  for (int k = 0; k < nsteps; k++)
    if ((r = adj_primal_step(h, A->runDts, nullptr, nullptr, k == 0, k == nsteps - 1))) return r;
  DevTime t;
  CKA(cudaMemcpyAsync(&t, h->tm, sizeof t, cudaMemcpyDeviceToHost, s));
  if (coords) {
    k_aos3<<<(unsigned)((h->N + 255) / 256), 256, 0, s>>>(h->N, h->x[0], A->runOut);
    launch_counter()++;
    CKA(cudaMemcpyAsync(coords, A->runOut, sizeof(double) * 3 * (size_t)h->N, cudaMemcpyDeviceToHost, s));
  }
  CKA(cudaStreamSynchronize(s));
  h->hostIncrement = t.increment;
  return t.status;
}

}  // extern "C"
