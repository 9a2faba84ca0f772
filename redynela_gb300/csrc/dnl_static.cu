// dnl_internal_forces_static: the internal-force pass for callers that cannot allocate device
// memory.
//
// Who needs it: a host application or framework whose memory manager owns every device byte and
// hands out buffers from its own pool, forbidding libraries their own cudaMalloc (a solver embedded
// in such a framework, or a process whose device-memory budget is fixed before the solver starts
// and must not grow).  Such a caller owns and passes every input and output buffer; the only other
// device memory this entry point uses is the fixed array below, which is part of the library image.
//
// Scratch: the per-element force vectors that the element pass writes and the node-centric
// assembly reads (E * nen * dim doubles) live in g_static_fe, a file-scope device array of
// DNL_STATIC_MAX_ELEMENT_DOFS doubles (8 MiB).  Every GPU that loads the library holds this array
// until the process exits.  Host code cannot use the array's name as a device address (on the host
// it names a host-side stand-in), so the first call on a device looks up the array's device address
// with cudaGetSymbolAddress while that device is current, checks the result and caches it, once per
// device under a lock; that first call should come before any stream capture.  All calls share the
// array and it keeps the last call's contents: every entry is written before it is read, and the
// error word, which must start clear, is reset at the start of each call.  Calls whose GPU work
// overlaps (two streams, or two host threads) race on the array and on the error word and must be
// serialised by the caller.
//
// No cudaMalloc, cudaFree or allocating library routine is called on this path.
#include <cmath>
#include <cstring>
#include <mutex>

#include "dnl_common.cuh"

namespace {

__device__ __align__(256) double g_static_fe[DNL_STATIC_MAX_ELEMENT_DOFS];
__device__ __align__(256) dnl::DevTime g_static_tm;

struct StaticPtrs {
  double *fe;
  dnl::DevTime *tm;
  bool ready;
};
constexpr int kMaxDevices = 64;
StaticPtrs g_ptrs[kMaxDevices];
std::mutex g_ptrs_lock;

// the device addresses of the two arrays on the current device, looked up once per device
int static_setup(StaticPtrs **out)
{
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return DNL_ERR_CUDA;
  std::lock_guard<std::mutex> guard(g_ptrs_lock);
  StaticPtrs &p = g_ptrs[dev];
  if (!p.ready) {
    double *fe = nullptr;
    dnl::DevTime *tm = nullptr;
    if (cudaGetSymbolAddress((void **)&fe, g_static_fe) != cudaSuccess) return DNL_ERR_CUDA;
    if (cudaGetSymbolAddress((void **)&tm, g_static_tm) != cudaSuccess) return DNL_ERR_CUDA;
    p.fe = fe;
    p.tm = tm;
    p.ready = true;
  }
  *out = &p;
  return 0;
}

}  // namespace

extern "C" int dnl_internal_forces_static(const dnl_static_args *a, void *stream, int *bad_element)
{
  using namespace dnl;
  if (bad_element) *bad_element = -1;
  if (!a) return DNL_ERR_ARG;
  // the one-point hexahedron's hourglass viscosity needs nodal velocities this entry does not take
  if (!etype_valid(a->etype) || a->etype == DNL_ELHEX8N3D_1PT) return DNL_ERR_ARG;
  const int nen = etype_nen(a->etype), dim = etype_dim(a->etype);
  if (a->num_nodes <= 0 || a->num_elements <= 0) return DNL_ERR_ARG;
  if ((long long)a->num_elements * nen * dim > DNL_STATIC_MAX_ELEMENT_DOFS) return DNL_ERR_ARG;
  if (!a->conn || !a->node_start || !a->node_entry || !a->coords || !a->du || !a->ip || !a->fint)
    return DNL_ERR_ARG;
  StaticPtrs *sp;
  if (int r = static_setup(&sp)) return r;
  cudaStream_t s = (cudaStream_t)stream;

  // the error word starts clear on every call (status 0, element -1); the force array needs no
  // clearing (the element pass writes every entry the assembly reads)
  if (cudaMemsetAsync(sp->tm, 0, sizeof(DevTime), s) != cudaSuccess) return DNL_ERR_CUDA;
  if (cudaMemsetAsync(&sp->tm->badElem, 0xff, sizeof(int), s) != cudaSuccess) return DNL_ERR_CUDA;

  const Material m = make_material(a->mat, nen);

  const int N = a->num_nodes, E = a->num_elements;
  ElemArgs ea;
  memset(&ea, 0, sizeof ea);
  ea.E = E;
  ea.N = N;
  ea.gate = 0;
  ea.conn = a->conn;
  for (int r = 0; r < 3; r++) {
    ea.x[r] = const_cast<double *>(a->coords) + (size_t)r * N;
    ea.du[r] = a->du + (size_t)r * N;
  }
  ea.ip = a->ip;
  ea.fe = sp->fe;
  ea.feStride = (long)E * nen;
  ea.detJ = nullptr;
  ea.stepT = nullptr;
  ea.tm = sp->tm;
  ea.mat = m;
  if (int r = launch_elem_raw(a->etype, ea, s)) return r;

  GatherArgs g;
  g.N = N;
  g.EN = E * nen;
  g.start = a->node_start;
  g.entry = a->node_entry;
  g.fe = sp->fe;
  g.fint = a->fint;
  if (int r = launch_gather_raw(dim, g, s)) return r;

  int word[2];
  if (cudaMemcpyAsync(word, &sp->tm->status, sizeof word, cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return DNL_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return DNL_ERR_CUDA;
  if (word[0] && bad_element) *bad_element = word[1];
  return word[0];
}
