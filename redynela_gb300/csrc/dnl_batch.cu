// Batched explicit dynamics: many independent meshes (e.g. Taylor bars of different sizes and
// materials) advanced together.
//
// The meshes are concatenated into one union mesh (node and element indices offset per instance)
// stored in an ordinary handle, plus an instance index per element and per node, a material and
// integration constants per instance and one time record per instance (each instance has its own
// time step, increment counter and end).  A step is the same five kernels as the single-mesh path,
// each launched once for all instances: time logic (one thread per instance), boundary conditions,
// element pass, assembly + nodal update, and every `frequency` increments the Courant reduction
// into each instance's minimum.  Small meshes that could not fill the GPU alone share its SMs, and
// the per-step launch cost is paid once for the batch; `dnl_batch_step_graph` captures a run of
// steps into a CUDA graph and replays it.
//
// Autotuning: the element pass is launched with 64, 128 or 256 threads per block (16, 32 or 64
// axisymmetric elements per block), and a step is either the launch sequence or one persistent
// kernel; `dnl_batch_autotune` times live steps of the six candidates taken in turn and keeps the
// fastest.  Every element's arithmetic is independent of both choices, so they do not change
// results.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "dnl_common.cuh"

using namespace dnl;

struct dnl_batch {
  int count;
  dnl_handle *h;  // union mesh
  int *elemInst, *nodeInst;
  Material *mats;
  InstParams *prm;
  DevTime *tms;
  std::vector<int> nodeOff, elemOff;  // count+1 offsets
  std::vector<InstParams> hprm;
  int freq;
  int block;
  int mode;             // DNL_BATCH_LAUNCHES or DNL_BATCH_PERSISTENT
  unsigned *bar;        // persistent mode: grid barrier (arrival count, generation) and
  int *barErr;          // its time-out flag
  long long increment;  // host copy (all instances advance in lockstep until they finish)
  bool prologueDone;
  bool massDone;
  bool canStep;         // axisymmetric Courant instances: dnl_batch_step; any: dnl_batch_sens_run
  double *v0dir;        // [count][3] unit initial velocity per instance
  double *v0;           // [count][3] initial velocity per instance (dnl_batch_reset)
  double *evpn0;        // [count] (1e-10)^n per instance (dnl_batch_reset)
  std::vector<DevTime> t0;  // initial time records
  struct Graph {
    int nsteps, parity, phase;
    cudaGraphExec_t exec;
    long long kernels;
  } graphs[8];
  int ngraphs;
};

namespace {

char g_batchError[256] = "";

#define BK(call)                                                                                 \
  do {                                                                                           \
    cudaError_t err_ = (call);                                                                   \
    if (err_ != cudaSuccess) {                                                                   \
      snprintf(g_batchError, sizeof g_batchError, "%s: %s", #call, cudaGetErrorString(err_));   \
      return DNL_ERR_CUDA;                                                                       \
    }                                                                                            \
  } while (0)

enum { BT_FORCE = 1, BT_POST = 2, BT_PRE = 4 };  // same modes as the single-mesh time kernel

// initial nodal velocities and evp^n cache per instance (dnl_batch_reset)
__global__ void k_batch_init(int N, long nIP, int nip, const int *nodeInst, const int *elemInst,
                             const double *v0, const double *evpn0, NodeFields b0, NodeFields b1,
                             double *evp, double *evpn)
{
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) {
    const int inst = nodeInst[i];
#pragma unroll
    for (int c = 0; c < 3; c++) b0.v[c][i] = b1.v[c][i] = v0[3 * inst + c];
  }
  if (i < nIP) {
    evp[i] = 1e-10;
    evpn[i] = evpn0[elemInst[i / nip]];
  }
}

int read_tms(dnl_batch *b, std::vector<DevTime> &t)
{
  t.resize(b->count);
  BK(cudaMemcpyAsync(t.data(), b->tms, sizeof(DevTime) * b->count, cudaMemcpyDeviceToHost, b->h->stream));
  BK(cudaStreamSynchronize(b->h->stream));
  return 0;
}

int first_status(const std::vector<DevTime> &t, int *inst)
{
  for (size_t i = 0; i < t.size(); i++)
    if (t[i].status) {
      if (inst) *inst = (int)i;
      return t[i].status;
    }
  return 0;
}

// one step as a single persistent cooperative launch (the same phases as the launch sequence
// below, separated by grid barriers); first: the step opens with initStep
int enqueue_batch_step_persistent(dnl_batch *b, long long incAfter, bool first, bool last)
{
  dnl_handle *h = b->h;
  BatchStepArgs a;
  memset(&a, 0, sizeof a);
  a.ea = elem_args_of(h);
  NodeArgs &g = a.na;
  g.N = h->N;
  g.EN = h->E * h->nen;
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
  a.cur = h->bank[h->cur];
  a.elemInst = b->elemInst;
  a.nodeInst = b->nodeInst;
  a.mats = b->mats;
  a.prm = b->prm;
  a.tms = b->tms;
  a.count = b->count;
  a.nbc = h->nbcNodes;
  a.bcNodes = h->bcNodeList;
  a.preFirst = first ? 1 : 0;
  a.courant = incAfter % b->freq == 0 ? 1 : 0;
  a.postMode = last ? BT_POST : (BT_POST | BT_PRE);
  a.bar = b->bar;
  a.err = b->barErr;
  prof_begin(h, h->stream);
  const int r = launch_batch_persistent(h->etype, b->block, a, h->stream);
  prof_end(h, DNL_PROF_ELEM, h->stream);
  h->cur = 1 - h->cur;
  return r;
}

int enqueue_batch_step(dnl_batch *b, long long incAfter, bool last)
{
  dnl_handle *h = b->h;
  int r;
  if ((r = launch_bc_batch(h, b->tms, b->nodeInst))) return r;
  ElemArgs a = elem_args_of(h);
  prof_begin(h, h->stream);
  r = launch_elem_batch(h->etype, b->block, a, b->elemInst, b->mats, b->tms, h->stream);
  prof_end(h, DNL_PROF_ELEM, h->stream);
  if (r) return r;
  if ((r = launch_node_batch(h, b->nodeInst, b->prm, b->tms))) return r;
  h->cur = 1 - h->cur;
  if (incAfter % b->freq == 0) {
    ElemArgs c = elem_args_of(h);
    prof_begin(h, h->stream);
    r = launch_courant_batch(h->etype, c, b->elemInst, b->tms, h->stream);
    prof_end(h, DNL_PROF_COURANT, h->stream);
    if (r) return r;
  }
  return launch_dt_batch(h, b->tms, b->prm, b->count, last ? BT_POST : (BT_POST | BT_PRE));
}

// evp^n of every integration point with its instance's n (the cached yield term), after a state
// copy
__global__ void k_batch_evpn(long nIP, int nip, const int *elemInst, const Material *mats,
                             const double *evp, double *evpn)
{
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nIP) return;
  evpn[i] = pow(evp[i], mats[elemInst[i / nip]].n);
}

// the launches of nsteps steps from increment inc0 in the batch's mode
int enqueue_steps(dnl_batch *b, long long inc0, int nsteps)
{
  dnl_handle *h = b->h;
  int r;
  if (b->mode == DNL_BATCH_PERSISTENT) {
    for (int s = 0; s < nsteps; s++)
      if ((r = enqueue_batch_step_persistent(b, inc0 + s + 1, s == 0, s == nsteps - 1))) return r;
    return 0;
  }
  if ((r = launch_dt_batch(h, b->tms, b->prm, b->count, BT_PRE))) return r;
  for (int s = 0; s < nsteps; s++)
    if ((r = enqueue_batch_step(b, inc0 + s + 1, s == nsteps - 1))) return r;
  return 0;
}

// after a run of persistent steps: a barrier that ran out is reported (and its words cleared)
int barrier_status(dnl_batch *b)
{
  if (b->mode != DNL_BATCH_PERSISTENT) return 0;
  int err = 0;
  BK(cudaMemcpyAsync(&err, b->barErr, sizeof err, cudaMemcpyDeviceToHost, b->h->stream));
  BK(cudaStreamSynchronize(b->h->stream));
  if (!err) return 0;
  BK(cudaMemsetAsync(b->bar, 0, sizeof(unsigned) * 2, b->h->stream));
  BK(cudaMemsetAsync(b->barErr, 0, sizeof(int), b->h->stream));
  BK(cudaStreamSynchronize(b->h->stream));
  snprintf(g_batchError, sizeof g_batchError, "persistent batch step: a grid barrier wait ran out");
  return DNL_ERR_TIMEOUT;
}

}  // namespace

extern "C" {

int dnl_batch_destroy(dnl_batch *b)
{
  if (!b) return DNL_ERR_ARG;
  for (int i = 0; i < b->ngraphs; i++) cudaGraphExecDestroy(b->graphs[i].exec);
  void *ptrs[] = {b->elemInst, b->nodeInst, b->mats, b->prm, b->tms, b->v0dir, b->v0, b->evpn0,
                  b->bar, b->barErr};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  if (b->h) dnl_destroy(b->h);
  delete b;
  return 0;
}

int dnl_batch_create(int count, const dnl_mesh_desc *meshes, const dnl_material *mats,
                     const dnl_solver_params *sps, dnl_batch **out)
{
  if (!out || count <= 0 || !meshes || !mats || !sps) return DNL_ERR_ARG;
  *out = nullptr;
  const int etype = meshes[0].etype;
  if (!etype_valid(etype)) return DNL_ERR_ARG;
  const int nen = etype_nen(etype);
  // plain batched stepping needs the Courant step of every instance (ElHex8n3D has no Courant
  // length); sensitivity runs take a step schedule and accept any time-step method
  bool canStep = etype != DNL_ELHEX8N3D;
  for (int i = 0; i < count; i++) {
    if (meshes[i].etype != etype) return DNL_ERR_ARG;
    if (sps[i].method != sps[0].method || sps[i].frequency != sps[0].frequency) return DNL_ERR_ARG;
    if (sps[i].method != DNL_COURANT || (sps[i].frequency % 2)) canStep = false;
    if (meshes[i].num_nodes <= 0 || meshes[i].num_elements <= 0) return DNL_ERR_ARG;
  }
  // ---- the union mesh
  std::vector<int> nodeOff(count + 1, 0), elemOff(count + 1, 0);
  for (int i = 0; i < count; i++) {
    nodeOff[i + 1] = nodeOff[i] + meshes[i].num_nodes;
    elemOff[i + 1] = elemOff[i] + meshes[i].num_elements;
  }
  const int N = nodeOff[count], E = elemOff[count];
  std::vector<double> coords(3 * (size_t)N);
  std::vector<int> conn((size_t)nen * E), elemInst(E), nodeInst(N);
  std::vector<int> bcKind, bcStart(1, 0), bcNodes;
  std::vector<double> bcVal;
  for (int i = 0; i < count; i++) {
    const dnl_mesh_desc &m = meshes[i];
    memcpy(&coords[3 * (size_t)nodeOff[i]], m.coords, sizeof(double) * 3 * m.num_nodes);
    for (long q = 0; q < (long)m.num_elements * nen; q++) {
      if (m.conn[q] < 0 || m.conn[q] >= m.num_nodes) return DNL_ERR_ARG;
      conn[(size_t)elemOff[i] * nen + q] = m.conn[q] + nodeOff[i];
    }
    for (int e = 0; e < m.num_elements; e++) elemInst[elemOff[i] + e] = i;
    for (int n = 0; n < m.num_nodes; n++) nodeInst[nodeOff[i] + n] = i;
    for (int g = 0; g < m.num_bc; g++) {
      bcKind.push_back(m.bc_kind[g]);
      for (int c = 0; c < 3; c++) bcVal.push_back(m.bc_val[3 * g + c]);
      for (int q = m.bc_start[g]; q < m.bc_start[g + 1]; q++) {
        if (m.bc_nodes[q] < 0 || m.bc_nodes[q] >= m.num_nodes) return DNL_ERR_ARG;
        bcNodes.push_back(m.bc_nodes[q] + nodeOff[i]);
      }
      bcStart.push_back((int)bcNodes.size());
    }
  }
  dnl_mesh_desc u;
  memset(&u, 0, sizeof u);
  u.etype = etype;
  u.num_nodes = N;
  u.num_elements = E;
  u.coords = coords.data();
  u.conn = conn.data();
  for (int c = 0; c < 3; c++) u.v0[c] = meshes[0].v0[c];
  u.num_bc = (int)bcKind.size();
  u.bc_kind = bcKind.data();
  u.bc_val = bcVal.data();
  u.bc_start = bcStart.data();
  u.bc_nodes = bcNodes.data();
  dnl_solver_params sp0 = sps[0];
  dnl_handle *h = nullptr;
  int r = dnl_create(&u, &mats[0], &sp0, &h);
  if (r) return r;
  h->batchUnion = true;  // its kernels cover one element group: no dnl_add_elements
  dnl_batch *b = new dnl_batch();
  b->count = count;
  b->h = h;
  b->nodeOff = nodeOff;
  b->elemOff = elemOff;
  b->freq = sps[0].frequency;
  b->block = 128;
  b->mode = DNL_BATCH_LAUNCHES;
  b->bar = nullptr;
  b->barErr = nullptr;
  b->ngraphs = 0;
  b->increment = 0;
  b->prologueDone = false;
  b->massDone = false;
  b->canStep = canStep;
  b->v0dir = nullptr;
  b->v0 = nullptr;
  b->evpn0 = nullptr;
  *out = b;
  auto fail = [&](int code) {
    dnl_batch_destroy(b);
    *out = nullptr;
    return code;
  };
#define BKF(call)                                                                                \
  do {                                                                                           \
    cudaError_t err_ = (call);                                                                   \
    if (err_ != cudaSuccess) {                                                                   \
      snprintf(g_batchError, sizeof g_batchError, "%s: %s", #call, cudaGetErrorString(err_));   \
      return fail(DNL_ERR_CUDA);                                                                 \
    }                                                                                            \
  } while (0)
  // ---- per-instance constants, in the reference's expressions (as dnl_create)
  std::vector<Material> hm(count);
  b->hprm.resize(count);
  std::vector<DevTime> ht(count);
  for (int i = 0; i < count; i++) {
    hm[i] = make_material(mats[i], nen);
    const double rb = sps[i].rho_b;
    InstParams &p = b->hprm[i];
    p.alphaM = (2.0 * rb - 1.0) / (1.0 + rb);
    p.beta = (5.0 - 3.0 * rb) / ((1.0 + rb) * (1.0 + rb) * (2.0 - rb));
    p.gamma = 1.5 - p.alphaM;
    const double omegaS = sqrt((12.0 * pow((1 + rb), 3) * (2.0 - rb)) /
                               (10 + 15 * rb - rb * rb + pow(rb, 3) - pow(rb, 4)));
    p.safetyOmega = sps[i].safety * omegaS;
    p.Cs = hm[i].Cs;
    p.freq = sps[i].frequency;
    p.method = DNL_COURANT;
    DevTime &t = ht[i];
    memset(&t, 0, sizeof t);
    t.upTime = t.endTime = sps[i].end_time;
    t.lenMinBits = 0x7ff0000000000000ull;
    t.badElem = -1;
  }
  BKF(cudaMalloc(&b->elemInst, sizeof(int) * E));
  BKF(cudaMalloc(&b->nodeInst, sizeof(int) * N));
  BKF(cudaMalloc(&b->mats, sizeof(Material) * count));
  BKF(cudaMalloc(&b->prm, sizeof(InstParams) * count));
  BKF(cudaMalloc(&b->tms, sizeof(DevTime) * count));
  BKF(cudaMalloc(&b->bar, sizeof(unsigned) * 2));
  BKF(cudaMemset(b->bar, 0, sizeof(unsigned) * 2));
  BKF(cudaMalloc(&b->barErr, sizeof(int)));
  BKF(cudaMemset(b->barErr, 0, sizeof(int)));
  BKF(cudaMemcpy(b->elemInst, elemInst.data(), sizeof(int) * E, cudaMemcpyHostToDevice));
  BKF(cudaMemcpy(b->nodeInst, nodeInst.data(), sizeof(int) * N, cudaMemcpyHostToDevice));
  BKF(cudaMemcpy(b->mats, hm.data(), sizeof(Material) * count, cudaMemcpyHostToDevice));
  BKF(cudaMemcpy(b->prm, b->hprm.data(), sizeof(InstParams) * count, cudaMemcpyHostToDevice));
  BKF(cudaMemcpy(b->tms, ht.data(), sizeof(DevTime) * count, cudaMemcpyHostToDevice));
  {
    std::vector<double> dirs(3 * (size_t)count);
    for (int i = 0; i < count; i++) {
      const double *v = meshes[i].v0;
      const double vn = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
      for (int c = 0; c < 3; c++) dirs[3 * (size_t)i + c] = vn > 0 ? v[c] / vn : 0.;
    }
    BKF(cudaMalloc(&b->v0dir, sizeof(double) * 3 * count));
    BKF(cudaMemcpy(b->v0dir, dirs.data(), sizeof(double) * 3 * count, cudaMemcpyHostToDevice));
    std::vector<double> v0s(3 * (size_t)count), pn0(count);
    for (int i = 0; i < count; i++) {
      for (int c = 0; c < 3; c++) v0s[3 * (size_t)i + c] = meshes[i].v0[c];
      pn0[i] = pow(1e-10, mats[i].n);
    }
    BKF(cudaMalloc(&b->v0, sizeof(double) * 3 * count));
    BKF(cudaMemcpy(b->v0, v0s.data(), sizeof(double) * 3 * count, cudaMemcpyHostToDevice));
    BKF(cudaMalloc(&b->evpn0, sizeof(double) * count));
    BKF(cudaMemcpy(b->evpn0, pn0.data(), sizeof(double) * count, cudaMemcpyHostToDevice));
    b->t0 = ht;
  }
  // ---- per-instance initial speed (both fields) and cached evp^n at evp = 1e-10
  {
    std::vector<double> v(N);
    for (int c = 0; c < 3; c++) {
      for (int i = 0; i < count; i++)
        for (int n = nodeOff[i]; n < nodeOff[i + 1]; n++) v[n] = meshes[i].v0[c];
      for (int bk = 0; bk < 2; bk++)
        BKF(cudaMemcpy(h->bank[bk].v[c], v.data(), sizeof(double) * N, cudaMemcpyHostToDevice));
    }
    const size_t nIP = (size_t)E * h->nip;
    std::vector<double> pn(nIP);
    for (int i = 0; i < count; i++) {
      const double val = pow(1e-10, mats[i].n);
      for (size_t q = (size_t)elemOff[i] * h->nip; q < (size_t)elemOff[i + 1] * h->nip; q++) pn[q] = val;
    }
    const int ns = etype_ns(etype);
    BKF(cudaMemcpy(h->ip + (size_t)(3 * ns + 2) * nIP, pn.data(), sizeof(double) * nIP, cudaMemcpyHostToDevice));
  }
  BKF(cudaDeviceSynchronize());
#undef BKF
  return 0;
}

static int batch_mass(dnl_batch *b)
{
  if (b->massDone) return 0;
  dnl_handle *h = b->h;
  double *me;
  BK(cudaMalloc(&me, sizeof(double) * (size_t)h->E * h->nen));
  ElemArgs a = elem_args_of(h);
  int r = launch_mass_batch(h->etype, a, me, b->elemInst, b->mats, h->stream);
  if (!r) r = launch_gather_mass(h, me);
  if (r) {
    cudaFree(me);
    return r;
  }
  BK(cudaStreamSynchronize(h->stream));
  cudaFree(me);
  b->massDone = true;
  return 0;
}

int dnl_batch_prologue(dnl_batch *b)
{
  if (!b || !b->canStep) return DNL_ERR_ARG;
  if (b->prologueDone) return 0;
  dnl_handle *h = b->h;
  int r;
  if ((r = batch_mass(b))) return r;
  // computeInternalForces with the initial (zero) Current field, then computeTimeStep(True)
  ElemArgs a = elem_args_of(h);
  if ((r = launch_elem_batch(h->etype, b->block, a, b->elemInst, b->mats, b->tms, h->stream))) return r;
  if ((r = launch_courant_batch(h->etype, a, b->elemInst, b->tms, h->stream))) return r;
  if ((r = launch_dt_batch(h, b->tms, b->prm, b->count, BT_FORCE))) return r;
  std::vector<DevTime> t;
  if ((r = read_tms(b, t))) return r;
  b->prologueDone = true;
  return first_status(t, nullptr);
}

int dnl_batch_step(dnl_batch *b, int nsteps, int *active)
{
  if (active) *active = 0;
  if (!b || nsteps < 0) return DNL_ERR_ARG;
  int r;
  if (!b->prologueDone && (r = dnl_batch_prologue(b))) return r;
  dnl_handle *h = b->h;
  if (nsteps > 0) {
    const long long inc0 = b->increment;
    if ((r = enqueue_steps(b, inc0, nsteps))) return r;
    b->increment += nsteps;
  }
  if ((r = barrier_status(b))) return r;
  std::vector<DevTime> t;
  if ((r = read_tms(b, t))) return r;
  int n = 0;
  for (auto &x : t) n += !x.done;
  if (active) *active = n;
  return first_status(t, nullptr);
}

// The graph of nsteps batched steps from the current increment (keyed by nsteps, the nodal field
// parity and the phase in the time-step recomputation cycle): found among the captured ones or
// captured now.  On return h->cur is the parity after the nsteps steps.
static int batch_graph(dnl_batch *b, int nsteps, cudaGraphExec_t *out)
{
  dnl_handle *h = b->h;
  const long long inc0 = b->increment;
  const int parity = h->cur, phase = (int)(inc0 % b->freq);
  cudaGraphExec_t exec = nullptr;
  for (int i = 0; i < b->ngraphs; i++)
    if (b->graphs[i].nsteps == nsteps && b->graphs[i].parity == parity && b->graphs[i].phase == phase)
      exec = b->graphs[i].exec;
  if (!exec) {
    cudaGraph_t graph;
    const long long k0 = launch_counter();
    BK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    int rr = enqueue_steps(b, inc0, nsteps);
    cudaError_t ce = cudaStreamEndCapture(h->stream, &graph);
    if (rr) return rr;
    if (ce != cudaSuccess) {
      snprintf(g_batchError, sizeof g_batchError, "graph capture: %s", cudaGetErrorString(ce));
      return DNL_ERR_CUDA;
    }
    BK(cudaGraphInstantiate(&exec, graph, 0));
    cudaGraphDestroy(graph);
    const long long kernels = launch_counter() - k0;
    launch_counter() = k0;
    if (b->ngraphs < 8) b->graphs[b->ngraphs++] = dnl_batch::Graph{nsteps, parity, phase, exec, kernels};
  } else {
    h->cur = (nsteps % 2) ? 1 - parity : parity;
  }
  *out = exec;
  return 0;
}

int dnl_batch_graph_capture(dnl_batch *b, int nsteps)
{
  if (!b || nsteps <= 0) return DNL_ERR_ARG;
  int r;
  if (!b->prologueDone && (r = dnl_batch_prologue(b))) return r;
  dnl_handle *h = b->h;
  const int cur0 = h->cur;
  cudaGraphExec_t exec;
  r = batch_graph(b, nsteps, &exec);
  h->cur = cur0;  // captured, not run
  if (r) return r;
  bool cached = false;
  for (int i = 0; i < b->ngraphs; i++) cached |= b->graphs[i].exec == exec;
  if (!cached) {  // the cache is full: nothing to keep
    cudaGraphExecDestroy(exec);
    return DNL_ERR_ARG;
  }
  return 0;
}

int dnl_batch_step_graph(dnl_batch *b, int nsteps, int *active)
{
  if (active) *active = 0;
  if (!b || nsteps <= 0) return DNL_ERR_ARG;
  int r;
  if (!b->prologueDone && (r = dnl_batch_prologue(b))) return r;
  dnl_handle *h = b->h;
  cudaGraphExec_t exec;
  if ((r = batch_graph(b, nsteps, &exec))) return r;
  for (int i = 0; i < b->ngraphs; i++)
    if (b->graphs[i].exec == exec) launch_counter() += b->graphs[i].kernels;
  BK(cudaGraphLaunch(exec, h->stream));
  b->increment += nsteps;
  if ((r = barrier_status(b))) return r;
  std::vector<DevTime> t;
  if ((r = read_tms(b, t))) return r;
  int n = 0;
  for (auto &x : t) n += !x.done;
  if (active) *active = n;
  bool cached = false;
  for (int i = 0; i < b->ngraphs; i++) cached |= b->graphs[i].exec == exec;
  if (!cached) cudaGraphExecDestroy(exec);
  return first_status(t, nullptr);
}

int dnl_batch_autotune(dnl_batch *b, int steps_per_candidate, int *block)
{
  if (!b || steps_per_candidate <= 0) return DNL_ERR_ARG;
  int r;
  if (!b->prologueDone && (r = dnl_batch_prologue(b))) return r;
  // candidates (mode, block): each first runs one untimed step (the first launch of its kernels
  // loads them), then the candidates are timed one step each in turn, steps_per_candidate rounds:
  // a run's cost per step drifts as it proceeds (the wave spreads, points yield), and taking the
  // candidates in turn lets that drift fall on all of them alike
  const int cands[3] = {64, 128, 256};
  constexpr int NC = 2 * 3;
  double total[NC] = {};
  const int mode0 = b->mode, block0 = b->block;
  cudaEvent_t e0, e1;
  BK(cudaEventCreate(&e0));
  BK(cudaEventCreate(&e1));
  r = 0;
  for (int round = -1; round < steps_per_candidate && !r; round++)
    for (int c = 0; c < NC && !r; c++) {
      b->mode = c < 3 ? DNL_BATCH_LAUNCHES : DNL_BATCH_PERSISTENT;
      b->block = cands[c % 3];
      int active = 0;
      float ms = 0.f;
      if (cudaEventRecord(e0, b->h->stream) != cudaSuccess) r = DNL_ERR_CUDA;
      if (!r) r = dnl_batch_step(b, 1, &active);
      if (!r && cudaEventRecord(e1, b->h->stream) != cudaSuccess) r = DNL_ERR_CUDA;
      if (!r && cudaEventSynchronize(e1) != cudaSuccess) r = DNL_ERR_CUDA;
      if (!r && cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) r = DNL_ERR_CUDA;
      if (round >= 0) total[c] += ms;
    }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  int bestC = -1;
  for (int c = 0; c < NC && !r; c++)
    if (bestC < 0 || total[c] < total[bestC]) bestC = c;
  const int bestM = bestC < 0 ? mode0 : (bestC < 3 ? DNL_BATCH_LAUNCHES : DNL_BATCH_PERSISTENT);
  const int bestB = bestC < 0 ? block0 : cands[bestC % 3];
  b->block = bestB;
  b->mode = bestM;
  for (int i = 0; i < b->ngraphs; i++) cudaGraphExecDestroy(b->graphs[i].exec);
  b->ngraphs = 0;
  if (block) *block = bestB;
  return r;
}

int dnl_batch_set_mode(dnl_batch *b, int mode)
{
  if (!b || (mode != DNL_BATCH_LAUNCHES && mode != DNL_BATCH_PERSISTENT)) return DNL_ERR_ARG;
  if (mode == DNL_BATCH_PERSISTENT && b->h->etype != DNL_ELQUA4NAX) return DNL_ERR_ARG;
  b->mode = mode;
  for (int i = 0; i < b->ngraphs; i++) cudaGraphExecDestroy(b->graphs[i].exec);
  b->ngraphs = 0;
  return 0;
}

int dnl_batch_get_tuning(dnl_batch *b, int *mode, int *block)
{
  if (!b) return DNL_ERR_ARG;
  if (mode) *mode = b->mode;
  if (block) *block = b->block;
  return 0;
}

int dnl_batch_reset(dnl_batch *b)
{
  if (!b) return DNL_ERR_ARG;
  dnl_handle *h = b->h;
  cudaStream_t s = h->stream;
  BK(cudaStreamSynchronize(s));
  for (int i = 0; i < b->ngraphs; i++) cudaGraphExecDestroy(b->graphs[i].exec);
  b->ngraphs = 0;
  const long N = h->N, nIP = h->nIP;
  const int ns = etype_ns(h->etype), ncomp = 3 * ns + 3;  // IpLayout::NCOMP
  BK(cudaMemcpyAsync(h->x[0], h->x0, sizeof(double) * 3 * N, cudaMemcpyDeviceToDevice, s));
  BK(cudaMemsetAsync(h->fieldMem, 0, sizeof(double) * 24 * N, s));
  BK(cudaMemsetAsync(h->ip, 0, sizeof(double) * ncomp * nIP, s));
  BK(cudaMemsetAsync(h->fint, 0, sizeof(double) * h->dim * N, s));
  const long n = N > nIP ? N : nIP;
  k_batch_init<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(
      (int)N, nIP, h->nip, b->nodeInst, b->elemInst, b->v0, b->evpn0, h->bank[0], h->bank[1],
      h->ip + (size_t)(3 * ns + 1) * nIP, h->ip + (size_t)(3 * ns + 2) * nIP);
  launch_counter()++;
  BK(cudaMemcpyAsync(b->tms, b->t0.data(), sizeof(DevTime) * b->count, cudaMemcpyHostToDevice, s));
  BK(cudaStreamSynchronize(s));
  BK(cudaGetLastError());
  h->cur = 0;
  h->hostIncrement = 0;
  b->increment = 0;
  b->prologueDone = false;
  return 0;
}

int dnl_batch_sens_run(dnl_batch *b, int nsteps, const double *dts, double *coords, double *dcoords)
{
  if (!b || nsteps <= 0 || !dts || b->increment != 0) return DNL_ERR_ARG;
  int r;
  if ((r = batch_mass(b))) return r;
  SensBatch bt;
  bt.count = b->count;
  bt.elemInst = b->elemInst;
  bt.nodeInst = b->nodeInst;
  bt.mats = b->mats;
  bt.prm = b->prm;
  bt.tms = b->tms;
  bt.v0dir = b->v0dir;
  r = sens_run(b->h, nsteps, dts, &bt);
  b->increment = nsteps;
  if (r) return r;
  return sens_outputs(b->h, coords, dcoords);
}

int dnl_batch_broadcast_state(dnl_batch *b, dnl_handle *src)
{
  if (!b || !src) return DNL_ERR_ARG;
  dnl_handle *h = b->h;
  if (src->etype != h->etype || src->nextra) return DNL_ERR_ARG;
  for (int i = 0; i < b->count; i++)
    if (b->nodeOff[i + 1] - b->nodeOff[i] != src->N || b->elemOff[i + 1] - b->elemOff[i] != src->E)
      return DNL_ERR_ARG;
  // the lumped mass is that of the initial mesh (Domain::computeMassMatrix at t = 0): form it
  // before the coordinates are replaced
  int r;
  if ((r = batch_mass(b))) return r;
  cudaStream_t s = h->stream;
  BK(cudaStreamSynchronize(src->stream));
  const size_t N = src->N, nIP = src->nIP, uN = h->N, unIP = h->nIP;
  const int ncomp = 3 * etype_ns(h->etype) + 3;
  for (int i = 0; i < b->count; i++) {
    const size_t n0 = b->nodeOff[i], q0 = (size_t)b->elemOff[i] * h->nip;
    for (int c = 0; c < 3; c++) {
      BK(cudaMemcpyAsync(h->x[c] + n0, src->x[c], sizeof(double) * N, cudaMemcpyDeviceToDevice, s));
      const double *from[4] = {src->bank[src->cur].du[c], src->bank[src->cur].v[c],
                               src->bank[src->cur].a[c], src->bank[src->cur].disp[c]};
      double *to[4] = {h->bank[h->cur].du[c], h->bank[h->cur].v[c], h->bank[h->cur].a[c],
                       h->bank[h->cur].disp[c]};
      for (int f = 0; f < 4; f++)
        BK(cudaMemcpyAsync(to[f] + n0, from[f], sizeof(double) * N, cudaMemcpyDeviceToDevice, s));
    }
    for (int k = 0; k < ncomp - 1; k++)  // all but evp^n, formed below with each instance's n
      BK(cudaMemcpyAsync(h->ip + k * unIP + q0, src->ip + k * nIP, sizeof(double) * nIP,
                         cudaMemcpyDeviceToDevice, s));
  }
  k_batch_evpn<<<(unsigned)((unIP + 255) / 256), 256, 0, s>>>((long)unIP, h->nip, b->elemInst, b->mats,
                                                             h->ip + (size_t)(ncomp - 2) * unIP,
                                                             h->ip + (size_t)(ncomp - 1) * unIP);
  launch_counter()++;
  BK(cudaStreamSynchronize(s));
  BK(cudaGetLastError());
  (void)uN;
  return 0;
}

int dnl_batch_set_block(dnl_batch *b, int block)
{
  if (!b || (block != 64 && block != 128 && block != 256)) return DNL_ERR_ARG;
  b->block = block;
  for (int i = 0; i < b->ngraphs; i++) cudaGraphExecDestroy(b->graphs[i].exec);
  b->ngraphs = 0;
  return 0;
}

int dnl_batch_time_info(dnl_batch *b, int inst, dnl_time_info *info)
{
  if (!b || !info || inst < 0 || inst >= b->count) return DNL_ERR_ARG;
  std::vector<DevTime> t;
  int r = read_tms(b, t);
  if (r) return r;
  const DevTime &x = t[inst];
  info->time = x.currentTime;
  info->time_step = x.timeStep;
  info->computed_step = x.computedTimeStep;
  info->kinetic = 0.;
  info->increment = x.increment;
  info->done = x.done;
  info->status = x.status;
  info->bad_element = x.badElem >= 0 ? x.badElem - b->elemOff[inst] : -1;
  return 0;
}

int dnl_batch_get_coords(dnl_batch *b, int inst, double *coords)
{
  if (!b || !coords || inst < 0 || inst >= b->count) return DNL_ERR_ARG;
  dnl_handle *h = b->h;
  const int n0 = b->nodeOff[inst], n1 = b->nodeOff[inst + 1];
  std::vector<double> c(n1 - n0);
  BK(cudaStreamSynchronize(h->stream));
  for (int r = 0; r < 3; r++) {
    BK(cudaMemcpy(c.data(), h->x[r] + n0, sizeof(double) * (n1 - n0), cudaMemcpyDeviceToHost));
    for (int n = 0; n < n1 - n0; n++) coords[3 * (size_t)n + r] = c[n];
  }
  return 0;
}

int dnl_batch_get_fint(dnl_batch *b, int inst, double *fint)
{
  if (!b || !fint || inst < 0 || inst >= b->count) return DNL_ERR_ARG;
  dnl_handle *h = b->h;
  BK(cudaStreamSynchronize(h->stream));
  BK(cudaMemcpy(fint, h->fint + (size_t)h->dim * b->nodeOff[inst],
                sizeof(double) * h->dim * (b->nodeOff[inst + 1] - b->nodeOff[inst]),
                cudaMemcpyDeviceToHost));
  return 0;
}

int dnl_batch_sizes(dnl_batch *b, int *elements, int *nodes)
{
  if (!b) return DNL_ERR_ARG;
  if (elements) *elements = b->h->E;
  if (nodes) *nodes = b->h->N;
  return 0;
}

int dnl_batch_handle(dnl_batch *b, dnl_handle **h)
{
  if (!b || !h) return DNL_ERR_ARG;
  *h = b->h;
  return 0;
}

}  // extern "C"
