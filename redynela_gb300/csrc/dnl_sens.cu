// Forward-mode sensitivities of an explicit run (dnl_sens_run, dnl_batch_sens_run).
//
// The run advances the primal state exactly as dnl_step does (boundary conditions, element pass,
// nodal Chung-Hulbert update of ExplicitSolverCH.C:387-567), except that the step sizes come from
// the caller's schedule instead of the Courant/Pulse estimate, and the element pass writes its
// per-integration-point record.  After each primal launch a tangent launch carries the derivative
// of the state with respect to the four parameters (A, B, n of IsoHardElastoplastic and the
// initial-velocity magnitude |v0|) -- four tangent copies of every nodal field and
// integration-point variable.  It stores no trajectory: the derivatives of every final coordinate
// come out of one run, where the reverse sweep of dnl_adjoint (dnl_adjoint.cu) gives one loss's
// gradient from checkpoints and recomputation.
#include <cstddef>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "dnl_common.cuh"

namespace dnl {

struct SensState {
  int E, N;
  double *mem = nullptr;
  double *tape = nullptr;  // [NT][nIP_g] per element group, at NT ipOff
  double *tx = nullptr;    // [dir][3][N]
  double *tb[2][4];        // [bank][du, v, a, disp] -> [dir][3][N]
  double *tip = nullptr;   // [dir][NCOMP][nIP_g] per element group, at 4 NCOMP ipOff
  double *tfe = nullptr;   // [dir][DIM][EN]: every group's element-node slots
  double *dts = nullptr;   // step sizes on the device
  double *out = nullptr;   // N*3 staging for node-major results
  int dtsCap = 0;
  std::vector<double> schedule;  // dnl_set_dt_schedule
  // single-mesh runs: two consecutive steps (bank parity 0 then 1, or 1 then 0) captured as a CUDA
  // graph and replayed; the element kernels take the material by value, so a graph is valid for
  // the material, hourglass coefficient and schedule buffer it was captured with
  cudaGraphExec_t pair[2] = {nullptr, nullptr};
  long long pairLaunches[2] = {0, 0};
  Material pairMat;
  double pairHourglass = 0.;
  const double *pairDts = nullptr;
};

static void drop_pairs(SensState *S)
{
  for (int p = 0; p < 2; p++)
    if (S->pair[p]) {
      cudaGraphExecDestroy(S->pair[p]);
      S->pair[p] = nullptr;
    }
}

namespace {

__global__ void k_sens_dt(DevTime *tms, int count, const double *dts, int phase)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  DevTime *tm = tms + i;
  if (tm->status) return;
  if (phase == 0) {  // initStep with the scheduled step
    const double dt = dts[tm->increment];
    tm->timeStep = dt;
    tm->nextTime = __dadd_rn(tm->currentTime, dt);
    tm->increment++;
  } else {  // updateTime
    tm->currentTime = __dadd_rn(tm->currentTime, tm->timeStep);
  }
}

// constant boundary conditions on the Current tangents: a restrained or imposed-speed component
// has a parameter-independent value, so its tangents are zero
__global__ void k_bc_tan(int nb, const int *nodes, const int *code, int N, double *du, double *v,
                         double *a)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nb) return;
  const int n = nodes[i], cd = code[i];
  for (int dir = 0; dir < kSensParams; dir++)
#pragma unroll
    for (int c = 0; c < 3; c++)
      if ((cd >> (2 * c)) & 3) {
        const long o = ((long)dir * 3 + c) * N + n;
        du[o] = 0.;
        v[o] = 0.;
        a[o] = 0.;
      }
}

struct SensNodeArgs {
  int N, EN;
  const int *start, *entry;
  const double *tfe, *mass;
  double *cur[4], *nxt[4];  // du, v, a, disp: [dir][3][N]
  double *tx;
  const int *bcIdx, *bcCode;
  const DevTime *tm;
  double alphaM, beta, gamma;
  const int *nodeInst;      // batched: instance of each node (its time record and constants)
  const InstParams *prm;
  const DevTime *tms;
};

// tangent of node_update (dnl_host.cu): the predictor, the assembled force, the corrector and the
// boundary conditions are linear in the state, so the tangents follow the same formulas
template <int DIM>
__global__ void __launch_bounds__(256) k_node_tan(SensNodeArgs g)
{
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  const int dir = blockIdx.y;
  if (n >= g.N) return;
  const int inst = g.nodeInst ? g.nodeInst[n] : 0;
  const DevTime *tm = g.nodeInst ? g.tms + inst : g.tm;
  if (tm->status) return;
  const double dt = tm->timeStep;
  const double alphaM = g.nodeInst ? g.prm[inst].alphaM : g.alphaM;
  const double beta = g.nodeInst ? g.prm[inst].beta : g.beta;
  const double gamma = g.nodeInst ? g.prm[inst].gamma : g.gamma;
  // 2D: the third components stay 0 and are neither read nor written
  const long N = g.N, base = (long)dir * 3 * N;
  double cdu[3] = {0., 0., 0.}, cv[3] = {0., 0., 0.}, ca[3] = {0., 0., 0.}, cd[3] = {0., 0., 0.};
  double ndu[3] = {0., 0., 0.}, nv[3] = {0., 0., 0.}, na[3] = {0., 0., 0.};
#pragma unroll
  for (int i = 0; i < DIM; i++) {
    cdu[i] = g.cur[0][base + i * N + n];
    cv[i] = g.cur[1][base + i * N + n];
    ca[i] = g.cur[2][base + i * N + n];
    cd[i] = g.cur[3][base + i * N + n];
  }
  (void)cdu;
  const double c1 = dt * (0.5 - beta), c2 = dt * (1. - gamma);
#pragma unroll
  for (int i = 0; i < DIM; i++) {
    ndu[i] = (ca[i] * c1 + cv[i]) * dt;
    nv[i] = ca[i] * c2 + cv[i];
    na[i] = 0.;
  }
  const int bc = g.bcIdx[n];
  const int code = bc >= 0 ? g.bcCode[bc] : 0;
#pragma unroll
  for (int i = 0; i < 3; i++)
    if ((code >> (2 * i)) & 3) ca[i] = cv[i] = ndu[i] = nv[i] = 0.;
  double f[DIM];
#pragma unroll
  for (int c = 0; c < DIM; c++) f[c] = 0.;
  const double *fe = g.tfe + (long)dir * DIM * g.EN;
  for (int q = g.start[n]; q < g.start[n + 1]; q++) {
    const int ent = __ldg(g.entry + q);
#pragma unroll
    for (int c = 0; c < DIM; c++) f[c] += __ldg(fe + (long)c * g.EN + ent);
  }
  // the tangents need no correctly rounded quotients: reciprocals (nr_rcp) times the numerators
  const double rm = nr_rcp(g.mass[n]);
#pragma unroll
  for (int c = 0; c < DIM; c++) na[c] = f[c] * rm;
  const double cg = dt * gamma, cb = dt * dt * beta, roma = nr_rcp(1. - alphaM);
#pragma unroll
  for (int i = 0; i < DIM; i++) {
    na[i] = (na[i] - alphaM * ca[i]) * roma;
    nv[i] = fma(cg, na[i], nv[i]);
    ndu[i] = fma(cb, na[i], ndu[i]);
    if ((code >> (2 * i)) & 3) na[i] = nv[i] = ndu[i] = 0.;
  }
#pragma unroll
  for (int i = 0; i < DIM; i++) {
    const long o = base + i * N + n;
    g.nxt[0][o] = ndu[i];
    g.nxt[1][o] = nv[i];
    g.nxt[2][o] = na[i];
    g.nxt[3][o] = cd[i] + ndu[i];
    g.tx[o] += ndu[i];
  }
}

// initial tangents: the initial velocity v0 = |v0| u on both fields, d v / d|v0| = u (per
// instance in a batch: u of the node's instance)
__global__ void k_sens_seed(int N, double *v0bank, double *v1bank, double u0, double u1, double u2,
                            const int *nodeInst, const double *v0dir)
{
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  const long base = 3L * 3 * N;  // direction 3
  double u[3] = {u0, u1, u2};
  if (nodeInst)
    for (int c = 0; c < 3; c++) u[c] = v0dir[3 * nodeInst[n] + c];
#pragma unroll
  for (int c = 0; c < 3; c++) {
    v0bank[base + c * (long)N + n] = u[c];
    v1bank[base + c * (long)N + n] = u[c];
  }
}

__global__ void k_to_nodes(int N, double *out, const double *c0, const double *c1, const double *c2)
{
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  out[3L * n] = c0[n];
  out[3L * n + 1] = c1[n];
  out[3L * n + 2] = c2[n];
}

#define CKS(x)                                \
  do {                                        \
    if ((x) != cudaSuccess) return DNL_ERR_CUDA; \
  } while (0)

// the record and tangent-state widths depend on the dimension only (TapeLayout, TanLayout)
static_assert(TapeLayout<DNL_ELTET4N3D>::NT == TapeLayout<DNL_ELHEX8N3D>::NT &&
                  TapeLayout<DNL_ELTET10N3D>::NT == TapeLayout<DNL_ELHEX8N3D>::NT &&
                  TapeLayout<DNL_ELHEX8N3D_1PT>::NT == TapeLayout<DNL_ELHEX8N3D>::NT &&
                  TapeLayout<DNL_ELQUA4N2D>::NT == TapeLayout<DNL_ELQUA4NAX>::NT,
              "tape width by dimension");
static_assert(TanLayout<DNL_ELTET4N3D>::NCOMP == TanLayout<DNL_ELHEX8N3D>::NCOMP &&
                  TanLayout<DNL_ELQUA4N2D>::NCOMP == TanLayout<DNL_ELQUA4NAX>::NCOMP,
              "tangent state width by dimension");
static int tape_nt(int etype)
{
  return etype_dim(etype) == 3 ? TapeLayout<DNL_ELHEX8N3D>::NT : TapeLayout<DNL_ELQUA4NAX>::NT;
}
static int tan_ncomp(int etype)
{
  return etype_dim(etype) == 3 ? TanLayout<DNL_ELHEX8N3D>::NCOMP : TanLayout<DNL_ELQUA4NAX>::NCOMP;
}

// per-point arrays cover every element group's points (each group's block at its ipOff), the
// element-node tangents every group's slots (component stride EN)
int sens_alloc(dnl_handle *h, SensState *S)
{
  const long nIP = ip_total(h), N = h->N;
  const int NT = tape_nt(h->etype), NC = tan_ncomp(h->etype);
  const long nodal = (long)kSensParams * 3 * N;
  const long total = NT * nIP + nodal * 9 + (long)kSensParams * NC * nIP +
                     (long)kSensParams * h->dim * h->EN + 3 * N;
  CKS(cudaMalloc(&S->mem, sizeof(double) * total));
  double *p = S->mem;
  S->tape = p;
  p += NT * nIP;
  S->tx = p;
  p += nodal;
  for (int b = 0; b < 2; b++)
    for (int f = 0; f < 4; f++) {
      S->tb[b][f] = p;
      p += nodal;
    }
  S->tip = p;
  p += (long)kSensParams * NC * nIP;
  S->tfe = p;
  p += (long)kSensParams * h->dim * h->EN;
  S->out = p;
  S->E = h->E;
  S->N = h->N;
  return 0;
}

}  // namespace

// The sensitivity run on a handle (bt == nullptr) or on a batch's union mesh: zero the tangents,
// seed d v / d|v0|, then per step the primal launches of the single-mesh or batched path with the
// scheduled step size, each followed by its tangent launch.
int sens_run(dnl_handle *h, int nsteps, const double *dts, const SensBatch *bt)
{
  // the tangent formulas are those of the power law and one material (per instance in a batch)
  if (!etype_has_sens(h->etype)) return DNL_ERR_ARG;
  if (!bt && (h->elemMat || h->mat.hard.law != DNL_HARD_POWER)) return DNL_ERR_ARG;
  for (int k = 0; k < nsteps; k++)
    if (!(dts[k] > 0. && dts[k] < 1e300)) return DNL_ERR_ARG;
  int r;
  if (!h->sens) h->sens = new SensState();
  SensState *S = (SensState *)h->sens;
  if (!S->mem && (r = sens_alloc(h, S))) return r;
  cudaStream_t s = h->stream;
  const long nIP = ip_total(h);
  {
    const int NT = tape_nt(h->etype);
    const size_t bytes = sizeof(double) * (size_t)((S->out - S->mem) - NT * nIP);
    CKS(cudaMemsetAsync(S->tx, 0, bytes, s));
  }
  k_sens_seed<<<(h->N + 255) / 256, 256, 0, s>>>(h->N, S->tb[0][1], S->tb[1][1], h->v0dir[0], h->v0dir[1],
                                                  h->v0dir[2], bt ? bt->nodeInst : nullptr,
                                                  bt ? bt->v0dir : nullptr);
  launch_counter()++;
  if (S->dtsCap < nsteps) {
    if (S->dts) cudaFree(S->dts);
    S->dts = nullptr;
    S->dtsCap = 0;
    CKS(cudaMalloc(&S->dts, sizeof(double) * nsteps));
    S->dtsCap = nsteps;
  }
  CKS(cudaMemcpyAsync(S->dts, dts, sizeof(double) * nsteps, cudaMemcpyHostToDevice, s));

  DevTime *tms = bt ? bt->tms : h->tm;
  const int ninst = bt ? bt->count : 1;
  SensElemArgs ea;
  memset(&ea, 0, sizeof ea);
  ea.E = h->E;
  ea.N = h->N;
  ea.conn = h->conn;
  for (int c = 0; c < 3; c++) ea.x[c] = h->x[c];
  ea.ip = h->ip;
  ea.tape = S->tape;
  ea.tx = S->tx;
  ea.tip = S->tip;
  ea.tfe = S->tfe;
  ea.feStride = h->EN;
  ea.tm = h->tm;
  ea.mat = h->mat;
  ea.hourglass = h->hourglass;
  ea.elemInst = bt ? bt->elemInst : nullptr;
  ea.mats = bt ? bt->mats : nullptr;
  SensNodeArgs na;
  memset(&na, 0, sizeof na);
  na.N = h->N;
  na.EN = (int)h->EN;
  na.start = h->n2eStart;
  na.entry = h->n2e;
  na.tfe = S->tfe;
  na.mass = h->mass;
  na.tx = S->tx;
  na.bcIdx = h->bcIdx;
  na.bcCode = h->bcCode;
  na.tm = h->tm;
  na.alphaM = h->alphaM;
  na.beta = h->beta;
  na.gamma = h->gamma;
  na.nodeInst = bt ? bt->nodeInst : nullptr;
  na.prm = bt ? bt->prm : nullptr;
  na.tms = bt ? bt->tms : nullptr;
  const dim3 ngrid((h->N + 255) / 256, kSensParams);
  const int tgrid = (ninst + 127) / 128;
  // one step: the primal launches with the scheduled step size, each followed by its tangent
  auto one_step = [&]() -> int {
    int r;
    k_sens_dt<<<tgrid, 128, 0, s>>>(tms, ninst, S->dts, 0);
    launch_counter()++;
    if (bt)
      r = launch_bc_batch(h, bt->tms, bt->nodeInst);
    else
      r = enqueue_bc_current(h);
    if (r) return r;
    if (h->nbcNodes) {
      double **tc = S->tb[h->cur];
      k_bc_tan<<<(h->nbcNodes + 127) / 128, 128, 0, s>>>(h->nbcNodes, h->bcNodeList, h->bcCode, h->N, tc[0],
                                                         tc[1], tc[2]);
      launch_counter()++;
    }
    if (bt) {
      ElemArgs a = elem_args_of(h);
      a.tape = S->tape;
      prof_begin(h, s);
      r = launch_elem_batch_tape(h->etype, a, bt->elemInst, bt->mats, bt->tms, s);
      prof_end(h, DNL_PROF_ELEM, s);
    } else {
      r = launch_elem_tape(h, s, S->tape);
    }
    if (r) return r;
    for (int c = 0; c < 3; c++) {
      ea.du[c] = h->bank[h->cur].du[c];
      ea.v[c] = h->bank[h->cur].v[c];
    }
    ea.tdu = S->tb[h->cur][0];
    ea.tv = S->tb[h->cur][1];
    prof_begin(h, s);
    r = launch_elem_tan(h->etype, ea, s);
    // further element groups: their own connectivity, state, records and element-node slots
    for (int gi = 0; gi < h->nextra && !r; gi++) {
      const ElemGroup &g = h->extra[gi];
      SensElemArgs eg = ea;
      eg.E = g.E;
      eg.conn = g.conn;
      eg.ip = g.ip;
      eg.tape = S->tape + (long)tape_nt(g.etype) * g.ipOff;
      eg.tip = S->tip + (long)kSensParams * tan_ncomp(g.etype) * g.ipOff;
      eg.tfe = S->tfe + g.feOff;
      r = launch_elem_tan(g.etype, eg, s);
    }
    prof_end(h, DNL_PROF_TANGENT, s);
    if (r) return r;
    if (bt)
      r = launch_node_batch(h, bt->nodeInst, bt->prm, bt->tms);
    else
      r = enqueue_node(h);
    if (r) return r;
    for (int f = 0; f < 4; f++) {
      na.cur[f] = S->tb[h->cur][f];
      na.nxt[f] = S->tb[1 - h->cur][f];
    }
    prof_begin(h, s);
    if (h->dim == 2)
      k_node_tan<2><<<ngrid, 256, 0, s>>>(na);
    else
      k_node_tan<3><<<ngrid, 256, 0, s>>>(na);
    prof_end(h, DNL_PROF_NODE, s);
    launch_counter()++;
    h->cur = 1 - h->cur;
    k_sens_dt<<<tgrid, 128, 0, s>>>(tms, ninst, S->dts, 1);
    launch_counter()++;
    return cudaPeekAtLastError() == cudaSuccess ? 0 : DNL_ERR_CUDA;
  };
  // single-mesh runs replay two-step graphs (launch-latency bound on small meshes); batches, odd
  // remainders and profiled runs launch step by step
  if (S->pairDts != S->dts || std::memcmp(&S->pairMat, &h->mat, offsetof(Material, hard)) != 0 ||
      S->pairHourglass != h->hourglass)
    drop_pairs(S);
  int k = 0;
  while (k < nsteps) {
    if (!bt && !h->profiling && nsteps - k >= 2) {
      const int par = h->cur;
      if (!S->pair[par]) {
        const long long c0 = launch_counter();
        cudaGraph_t g;
        if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return DNL_ERR_CUDA;
        int rr = one_step();
        if (!rr) rr = one_step();
        const cudaError_t ce = cudaStreamEndCapture(s, &g);
        h->cur = par;  // nothing ran: the host's bank parity stays with the device state
        if (rr) {
          if (ce == cudaSuccess) cudaGraphDestroy(g);
          return rr;
        }
        if (ce != cudaSuccess) return DNL_ERR_CUDA;
        const cudaError_t ie = cudaGraphInstantiate(&S->pair[par], g, 0);
        cudaGraphDestroy(g);
        if (ie != cudaSuccess) {
          S->pair[par] = nullptr;
          return DNL_ERR_CUDA;
        }
        S->pairLaunches[par] = launch_counter() - c0;
        launch_counter() = c0;
        S->pairMat = h->mat;
        S->pairHourglass = h->hourglass;
        S->pairDts = S->dts;
      }
      if (cudaGraphLaunch(S->pair[par], s) != cudaSuccess) return DNL_ERR_CUDA;
      launch_counter() += S->pairLaunches[par];
      k += 2;  // two bank swaps: the parity is unchanged
    } else {
      if ((r = one_step())) return r;
      k++;
    }
  }
  std::vector<DevTime> t(ninst);
  CKS(cudaMemcpyAsync(t.data(), tms, sizeof(DevTime) * ninst, cudaMemcpyDeviceToHost, s));
  CKS(cudaStreamSynchronize(s));
  h->hostIncrement = t[0].increment;
  for (const DevTime &ti : t)
    if (ti.status) return ti.status;
  return 0;
}

// final coordinates (3N, node-major) and their derivatives (4 x 3N) of the last sensitivity run
int sens_outputs(dnl_handle *h, double *coords, double *dcoords)
{
  SensState *S = (SensState *)h->sens;
  if (!S || !S->mem) return DNL_ERR_ARG;
  cudaStream_t s = h->stream;
  const long N = h->N;
  const int grid = (h->N + 255) / 256;
  if (coords) {
    k_to_nodes<<<grid, 256, 0, s>>>(h->N, S->out, h->x[0], h->x[1], h->x[2]);
    CKS(cudaMemcpyAsync(coords, S->out, sizeof(double) * 3 * N, cudaMemcpyDeviceToHost, s));
    CKS(cudaStreamSynchronize(s));
  }
  if (dcoords)
    for (int dir = 0; dir < kSensParams; dir++) {
      const double *b = S->tx + (long)dir * 3 * N;
      k_to_nodes<<<grid, 256, 0, s>>>(h->N, S->out, b, b + N, b + 2 * N);
      CKS(cudaMemcpyAsync(dcoords + (long)dir * 3 * N, S->out, sizeof(double) * 3 * N,
                          cudaMemcpyDeviceToHost, s));
      CKS(cudaStreamSynchronize(s));
    }
  return 0;
}

// the schedule dnl_set_dt_schedule stored (nullptr / 0 when none)
int sens_schedule(dnl_handle *h, const double **dts, int *n)
{
  SensState *S = (SensState *)h->sens;
  if (!S || S->schedule.empty()) {
    *dts = nullptr;
    *n = 0;
    return DNL_ERR_ARG;
  }
  *dts = S->schedule.data();
  *n = (int)S->schedule.size();
  return 0;
}

void sens_free(dnl_handle *h)
{
  SensState *S = (SensState *)h->sens;
  if (!S) return;
  drop_pairs(S);
  if (S->mem) cudaFree(S->mem);
  if (S->dts) cudaFree(S->dts);
  delete S;
  h->sens = nullptr;
}

}  // namespace dnl

using namespace dnl;

extern "C" {

int dnl_set_dt_schedule(dnl_handle *h, const double *dts, int nsteps)
{
  if (!h || !dts || nsteps <= 0) return DNL_ERR_ARG;
  for (int k = 0; k < nsteps; k++)
    if (!(dts[k] > 0. && dts[k] < 1e300)) return DNL_ERR_ARG;
  if (!h->sens) h->sens = new SensState();
  ((SensState *)h->sens)->schedule.assign(dts, dts + nsteps);
  return 0;
}

int dnl_sens_run(dnl_handle *h, int nsteps, const double *dts, double *coords, double *dcoords)
{
  if (!h || nsteps <= 0 || !dts) return DNL_ERR_ARG;
  if (h->hostIncrement != 0) return DNL_ERR_ARG;  // starts from the initial state
  int r;
  if (!h->prologueDone && (r = dnl_prologue(h))) return r;
  if ((r = sens_run(h, nsteps, dts, nullptr))) return r;
  return sens_outputs(h, coords, dcoords);
}

}  // extern "C"
