// dnl_internal_forces_static: the internal-force pass for callers that cannot allocate device
// memory.
//
// Who needs it: code that runs where cudaMalloc is off limits -- inside a CUDA stream capture
// (allocation is not a capturable operation), under an external memory manager that owns every
// device byte (a host application or framework pool that hands out buffers but forbids the
// library from taking its own), or in a process whose device-memory budget is fixed before the
// solver starts.  Such a caller owns and passes every input and output buffer; the only other
// device memory this entry point uses is the fixed array below, which is part of the library image.
//
// Scratch: the per-element force vectors that the element pass writes and the node-centric
// assembly reads (E * nen * dim doubles) live in g_static_fe, a file-scope device array of
// DNL_STATIC_MAX_ELEMENT_DOFS doubles (8 MiB).  Every GPU that loads the library holds this array
// until the process exits.  The first call on a device looks up the array's device address with
// cudaGetSymbolAddress while that device is current and caches it; make that first call before
// any stream capture.  All calls share the array and it keeps the last call's contents; the error
// word is reset at the start of each call.  Calls whose GPU work overlaps (two streams, or two
// host threads) race on the array and must be serialised by the caller.
//
// No cudaMalloc, cudaFree or allocating library routine is called on this path.
#include <cmath>
#include <cstring>

#include "dnl_common.cuh"

namespace {

__device__ __align__(256) double g_static_fe[DNL_STATIC_MAX_ELEMENT_DOFS];
__device__ __align__(256) dnl::DevTime g_static_tm;

struct StaticPtrs {
  double *fe;
  dnl::DevTime *tm;
  bool ready;
};
StaticPtrs g_ptrs[64];

int static_setup(StaticPtrs **out)
{
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return DNL_ERR_CUDA;
  StaticPtrs &p = g_ptrs[dev];
  if (!p.ready) {
    if (cudaGetSymbolAddress((void **)&p.fe, g_static_fe) != cudaSuccess) return DNL_ERR_CUDA;
    if (cudaGetSymbolAddress((void **)&p.tm, g_static_tm) != cudaSuccess) return DNL_ERR_CUDA;
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

  // the error word starts at zero on every call; the array itself needs no clearing (fully written)
  if (cudaMemsetAsync(sp->tm, 0, sizeof(DevTime), s) != cudaSuccess) return DNL_ERR_CUDA;

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
