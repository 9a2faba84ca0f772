// Pulse critical time step: Domain::getMaximumFrequency (Domain.C:817-945), a power iteration on
// M^-1 K started from the ramp 1 .. -1 (or the previous call's vector) and stopped when the
// max-norm estimate changes by less than 1e-4 (DefaultValues.h:35-36).
//
// The reference assembles every element's elastic stiffness Ke (Element3D.C:242-333,
// Element2D.C:129-226) and multiplies Ke x_e in each iteration.  Here K x_e is applied without
// forming Ke: per Gauss point the strain of x_e through the shape-function gradients, the Hooke
// stress (Material::getHookeMatrix, Material.C:270-331) and B^T sigma W -- the same bilinear
// form, fewer FP64 operations than a 24x24 product and no 4.6 KB per element to stream.
//
// Kernels: k_pulse_setup (J^-1, W, R per Gauss point, once per call), then per iteration
// k_pulse_kx (element products of the stored, not yet normalised iterate; Gauss points summed in
// order in shared memory), k_pulse_gather (CSR sum in element order, / previous max, / mass,
// max |.| by an unsigned atomicMax on the bits)
// and k_pulse_check (convergence test, one thread).  The host runs iterations in batches and reads
// the convergence flag between batches.
#include <cstring>
#include <vector>

#include "dnl_common.cuh"

namespace dnl {

#define RMUL __dmul_rn
#define RADD __dadd_rn
#define RSUB __dsub_rn

// shape functions, same construction as dnl_elem.cu
struct PShape {
  double axN[3], axD[2], hxN[4], hxD[3];
  double t10N[4][10], t10D[4][10][3];
};
__constant__ PShape c_pshape;

__device__ __forceinline__ int psgx(int k) { return (k ^ (k >> 1)) & 1; }
__device__ __forceinline__ int psgy(int k) { return (k >> 1) & 1; }
__device__ __forceinline__ int psgz(int k) { return (k >> 2) & 1; }

template <int ET> __device__ __forceinline__ double pN(int pt, int k);
template <int ET> __device__ __forceinline__ double pdN(int pt, int k, int c);
template <> __device__ __forceinline__ double pN<DNL_ELQUA4NAX>(int pt, int k)
{
  const int d = (psgx(k) ^ psgx(pt)) + (psgy(k) ^ psgy(pt));
  return d == 0 ? c_pshape.axN[0] : (d == 1 ? c_pshape.axN[1] : c_pshape.axN[2]);
}
template <> __device__ __forceinline__ double pdN<DNL_ELQUA4NAX>(int pt, int k, int c)
{
  const int other = c == 0 ? (psgy(k) ^ psgy(pt)) : (psgx(k) ^ psgx(pt));
  const double v = other ? c_pshape.axD[1] : c_pshape.axD[0];
  return (c == 0 ? psgx(k) : psgy(k)) ? v : -v;
}
template <> __device__ __forceinline__ double pN<DNL_ELQUA4N2D>(int pt, int k)
{
  return pN<DNL_ELQUA4NAX>(pt, k);
}
template <> __device__ __forceinline__ double pdN<DNL_ELQUA4N2D>(int pt, int k, int c)
{
  return pdN<DNL_ELQUA4NAX>(pt, k, c);
}
template <> __device__ __forceinline__ double pN<DNL_ELTET4N3D>(int, int) { return 0.25; }
template <> __device__ __forceinline__ double pdN<DNL_ELTET4N3D>(int, int k, int c)
{
  return k == 0 ? -1.0 : (k - 1 == c ? 1.0 : 0.0);
}
template <> __device__ __forceinline__ double pN<DNL_ELTET10N3D>(int pt, int k) { return c_pshape.t10N[pt][k]; }
template <> __device__ __forceinline__ double pdN<DNL_ELTET10N3D>(int pt, int k, int c)
{
  return c_pshape.t10D[pt][k][c];
}
// the one-point hexahedron's centre (compiled for the dispatch; dnl_create refuses Pulse for it)
template <> __device__ __forceinline__ double pN<DNL_ELHEX8N3D_1PT>(int, int) { return 0.125; }
template <> __device__ __forceinline__ double pdN<DNL_ELHEX8N3D_1PT>(int, int k, int c)
{
  return (c == 0 ? psgx(k) : (c == 1 ? psgy(k) : psgz(k))) ? 0.125 : -0.125;
}
// integration weight (ElTet4n3D.C:33, ElTet10n3D.C:30; the quads and the hexahedron: 1)
template <int ET> constexpr double pweight()
{
  return ET == DNL_ELTET4N3D ? 1. / 6.
                             : (ET == DNL_ELTET10N3D ? 1.0 / 24.0 : (ET == DNL_ELHEX8N3D_1PT ? 8.0 : 1.0));
}
template <> __device__ __forceinline__ double pN<DNL_ELHEX8N3D>(int pt, int k)
{
  const int d = (psgx(k) ^ psgx(pt)) + (psgy(k) ^ psgy(pt)) + (psgz(k) ^ psgz(pt));
  return d == 0 ? c_pshape.hxN[0] : (d == 1 ? c_pshape.hxN[1] : (d == 2 ? c_pshape.hxN[2] : c_pshape.hxN[3]));
}
template <> __device__ __forceinline__ double pdN<DNL_ELHEX8N3D>(int pt, int k, int c)
{
  const int dx = psgx(k) ^ psgx(pt), dy = psgy(k) ^ psgy(pt), dz = psgz(k) ^ psgz(pt);
  const int d = c == 0 ? dy + dz : (c == 1 ? dx + dz : dx + dy);
  const double v = d == 0 ? c_pshape.hxD[0] : (d == 1 ? c_pshape.hxD[1] : c_pshape.hxD[2]);
  return (c == 0 ? psgx(k) : (c == 1 ? psgy(k) : psgz(k))) ? v : -v;
}

static void set_pulse_tables()
{
  PShape s;
  s.axN[0] = (2.0 + sqrt(3.0)) / 6.0;
  s.axN[1] = 1.0 / 6.0;
  s.axN[2] = (2.0 - sqrt(3.0)) / 6.0;
  s.axD[0] = (3.0 + sqrt(3.0)) / 12.0;
  s.axD[1] = (3.0 - sqrt(3.0)) / 12.0;
  s.hxN[0] = (9.0 + 5.0 * sqrt(3.0)) / 36.0;
  s.hxN[1] = (3.0 + sqrt(3.0)) / 36.0;
  s.hxN[2] = (3.0 - sqrt(3.0)) / 36.0;
  s.hxN[3] = (9.0 - 5.0 * sqrt(3.0)) / 36.0;
  s.hxD[0] = (2.0 + sqrt(3.0)) / 12.0;
  s.hxD[1] = 1.0 / 12.0;
  s.hxD[2] = (2.0 - sqrt(3.0)) / 12.0;
  tet10_tables(s.t10N, s.t10D);
  cudaMemcpyToSymbol(c_pshape, &s, sizeof s);
}

struct PulseArgs {
  int E, N;
  const int *conn;
  const double *x[3];
  double *pj;        // [DIM*DIM + 2][nIP]: J^-1 (row-major), W, R
  double *ev;        // raw iterate [N*DIM]; the normalised vector is ev / tm->pulseScale
  double *kx;        // element products: component i of element e's node k at kx[i kxStride + e NEN + k]
  long kxStride;     // element-node slots of the handle's element groups
  const int *start, *entry;
  const double *mass;
  DevTime *tm;
  double C00, C01, C33;
  // several materials: each element's material (elemMat) and the materials' Hooke entries
  // (hooke, 3 per material: C00, C01, C33), or nullptr (one material: C00, C01, C33 above)
  const int *elemMat;
  const double *hooke;
};

// ------------------------------------------------------------------ per-Gauss-point kinematics
template <int ET>
__global__ void __launch_bounds__(128) k_pulse_setup(PulseArgs a)
{
  using T = Elem<ET>;
  constexpr int NIP = T::NIP, NEN = T::NEN, DIM = T::DIM;
  constexpr bool AXI = ET == DNL_ELQUA4NAX, TWO_D = DIM == 2;
  constexpr bool EDGES = ET == DNL_ELHEX8N3D || ET == DNL_ELQUA4NAX || ET == DNL_ELQUA4N2D;
  __shared__ double ex[128 / 32][EDGES ? 32 / NIP : 1][EDGES ? Edges<ET>::NE * DIM : 1];
  if (a.tm->done | a.tm->status) return;
  const long gtid = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long nIP = (long)a.E * NIP;
  if ((gtid & ~31L) >= nIP) return;  // whole warps only: the element's lanes exchange through ex
  const bool valid = gtid < nIP;
  const long g = valid ? gtid : nIP - 1;
  const int e = (int)(g / NIP), pt = (int)(g % NIP);
  double J[DIM][DIM] = {};
  double Rad = 0.;
  if constexpr (EDGES) {
    // J from the element's edge differences, a few per lane, shared by its lanes (Edges)
    using EG = Edges<ET>;
    constexpr int NE = EG::NE, PER = NE / DIM;
    double *buf = ex[threadIdx.x >> 5][(threadIdx.x & 31) / NIP];
#pragma unroll
    for (int j = 0; j < (NE + NIP - 1) / NIP; j++) {
      const int eg = pt + j * NIP;
      if (eg < NE) {
        const int lo = __ldg(a.conn + (long)edge_node(EG::LO, eg) * a.E + e);
        const int hi = __ldg(a.conn + (long)edge_node(EG::HI, eg) * a.E + e);
#pragma unroll
        for (int r = 0; r < DIM; r++) buf[eg * DIM + r] = a.x[r][hi] - a.x[r][lo];
      }
    }
    __syncwarp();
#pragma unroll
    for (int c = 0; c < DIM; c++)
#pragma unroll
      for (int q = 0; q < PER; q++) {
        const int eg = c * PER + q;
        const double w = pdN<ET>(pt, edge_node(EG::HI, eg), c);
#pragma unroll
        for (int r = 0; r < DIM; r++) J[r][c] = fma(w, buf[eg * DIM + r], J[r][c]);
      }
    if (AXI) {
#pragma unroll
      for (int k = 0; k < NEN; k++) Rad = fma(pN<ET>(pt, k), a.x[0][__ldg(a.conn + (long)k * a.E + e)], Rad);
    }
  } else {
#pragma unroll
    for (int k = 0; k < NEN; k++) {
      const int nd = a.conn[(long)k * a.E + e];
#pragma unroll
      for (int r = 0; r < DIM; r++) {
        const double xr = a.x[r][nd];
#pragma unroll
        for (int c = 0; c < DIM; c++) J[r][c] = fma(pdN<ET>(pt, k, c), xr, J[r][c]);
      }
      if (AXI) Rad = fma(pN<ET>(pt, k), a.x[0][nd], Rad);
    }
  }
  if (!valid) return;
  double Ji[DIM][DIM], detJ;
  if (TWO_D) {
    detJ = J[0][0] * J[1][1] - J[0][1] * J[1][0];
    const double r = 1. / detJ;
    Ji[0][0] = J[1][1] * r;
    Ji[0][1] = -J[0][1] * r;
    Ji[1][0] = -J[1][0] * r;
    Ji[1][1] = J[0][0] * r;
  } else {
    const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
    const double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
    const double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
    detJ = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
    const double r = 1. / detJ;
    Ji[0][0] = c00 * r;
    Ji[1][0] = c01 * r;
    Ji[2][0] = c02 * r;
    Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * r;
    Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * r;
    Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * r;
    Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * r;
    Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * r;
    Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * r;
  }
  double W = pweight<ET>() == 1.0 ? detJ : pweight<ET>() * detJ;
  if (AXI) W *= 2 * kPi * Rad;
#pragma unroll
  for (int l = 0; l < DIM; l++)
#pragma unroll
    for (int c = 0; c < DIM; c++) a.pj[(l * DIM + c) * nIP + gtid] = Ji[l][c];
  a.pj[(DIM * DIM) * nIP + gtid] = W;
  a.pj[(DIM * DIM + 1) * nIP + gtid] = Rad;
}

// ------------------------------------------------------------------ element products K x_e
template <int ET>
__global__ void __launch_bounds__(128) k_pulse_kx(PulseArgs a)
{
  using T = Elem<ET>;
  constexpr int NIP = T::NIP, NEN = T::NEN, DIM = T::DIM;
  constexpr bool AXI = ET == DNL_ELQUA4NAX;
  constexpr int EPW = 32 / NIP;
  __shared__ double red[128 / 32][EPW][NIP][NEN * DIM];
  const DevTime *tm = a.tm;
  if (tm->done | tm->status | tm->pulseDone) return;
  const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
  if ((gtid & ~31) / NIP >= a.E) return;
  const int eRaw = gtid / NIP;
  const bool valid = eRaw < a.E;
  const int e = valid ? eRaw : a.E - 1;
  const int pt = gtid % NIP;
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, slot = lane / NIP;
  const long nIP = (long)a.E * NIP;
  const long ipx = (long)e * NIP + pt;
  double Ji[DIM][DIM];
#pragma unroll
  for (int l = 0; l < DIM; l++)
#pragma unroll
    for (int c = 0; c < DIM; c++) Ji[l][c] = a.pj[(l * DIM + c) * nIP + ipx];
  const double W = a.pj[(DIM * DIM) * nIP + ipx];
  const double Rad = a.pj[(DIM * DIM + 1) * nIP + ipx];
  // G(r, l) = sum_k x_k(r) dN/dxi_k(l); grad = G J^-1
  double G[DIM][DIM] = {};
  double ur = 0.;  // axi: sum N_k x_k(r)
  double *buf = &red[wib][slot][0][0];  // this element's shared memory, NIP x NEN*DIM doubles
  constexpr bool EDGES = ET == DNL_ELHEX8N3D || ET == DNL_ELQUA4NAX || ET == DNL_ELQUA4N2D;
  if constexpr (EDGES) {
    // from the element's edge differences (a few per lane, exchanged through its shared memory):
    // the dN/dxi_c of an edge's two nodes are opposite at every Gauss point (Edges)
    using EG = Edges<ET>;
    constexpr int NE = EG::NE, PER = NE / DIM;
#pragma unroll
    for (int j = 0; j < (NE + NIP - 1) / NIP; j++) {
      const int eg = pt + j * NIP;
      if (eg < NE) {
        const int lo = __ldg(a.conn + (long)edge_node(EG::LO, eg) * a.E + e);
        const int hi = __ldg(a.conn + (long)edge_node(EG::HI, eg) * a.E + e);
#pragma unroll
        for (int r = 0; r < DIM; r++) buf[eg * DIM + r] = a.ev[(long)hi * DIM + r] - a.ev[(long)lo * DIM + r];
      }
    }
    __syncwarp();
#pragma unroll
    for (int c = 0; c < DIM; c++)
#pragma unroll
      for (int q = 0; q < PER; q++) {
        const int eg = c * PER + q;
        const double w = pdN<ET>(pt, edge_node(EG::HI, eg), c);
#pragma unroll
        for (int r = 0; r < DIM; r++) G[r][c] = fma(w, buf[eg * DIM + r], G[r][c]);
      }
    __syncwarp();  // the force exchange reuses the buffer
    if (AXI) {
#pragma unroll
      for (int k = 0; k < NEN; k++) ur = fma(pN<ET>(pt, k), a.ev[(long)__ldg(a.conn + (long)k * a.E + e) * DIM], ur);
    }
  } else {
#pragma unroll
    for (int k = 0; k < NEN; k++) {
      const int nk = a.conn[(long)k * a.E + e];
      double xk[DIM];
#pragma unroll
      for (int r = 0; r < DIM; r++) xk[r] = a.ev[(long)nk * DIM + r];
#pragma unroll
      for (int r = 0; r < DIM; r++)
#pragma unroll
        for (int l = 0; l < DIM; l++) G[r][l] = fma(xk[r], pdN<ET>(pt, k, l), G[r][l]);
      if (AXI) ur = fma(pN<ET>(pt, k), xk[0], ur);
    }
  }
  double gr[DIM][DIM];
#pragma unroll
  for (int r = 0; r < DIM; r++)
#pragma unroll
    for (int c = 0; c < DIM; c++) {
      double s = 0.;
#pragma unroll
      for (int l = 0; l < DIM; l++) s = fma(G[r][l], Ji[l][c], s);
      gr[r][c] = s;
    }
  // Hooke stress S of the in-plane components and, axisymmetric, the hoop stress (plane strain:
  // the upper-left block of the axisymmetric matrix, no hoop strain); with several materials the
  // element's own matrix (Element2D/3D::computeElasticStiffnessMatrix reads the element's material)
  double C00 = a.C00, C01 = a.C01, C33 = a.C33;
  if (a.elemMat) {
    const double *c = a.hooke + 3 * __ldg(a.elemMat + e);
    C00 = c[0];
    C01 = c[1];
    C33 = c[2];
  }
  double S[DIM][DIM], hoop = 0.;
  if (DIM == 2) {
    const double e0 = gr[0][0], e1 = gr[1][1], e2 = gr[0][1] + gr[1][0], e3 = AXI ? ur / Rad : 0.;
    S[0][0] = C00 * e0 + C01 * (e1 + e3);
    S[1][1] = C00 * e1 + C01 * (e0 + e3);
    S[0][1] = S[1][0] = C33 * e2;
    hoop = C00 * e3 + C01 * (e0 + e1);
  } else {
    const double e0 = gr[0][0], e1 = gr[1][1], e2 = gr[2][2];
    S[0][0] = C00 * e0 + C01 * (e1 + e2);
    S[1][1] = C00 * e1 + C01 * (e0 + e2);
    S[2][2] = C00 * e2 + C01 * (e0 + e1);
    S[0][1] = S[1][0] = C33 * (gr[0][1] + gr[1][0]);
    S[1][2] = S[2][1] = C33 * (gr[1][2] + gr[2][1]);
    S[0][2] = S[2][0] = C33 * (gr[0][2] + gr[2][0]);
  }
  double M[DIM][DIM];
#pragma unroll
  for (int l = 0; l < DIM; l++)
#pragma unroll
    for (int i = 0; i < DIM; i++) {
      double s = 0.;
#pragma unroll
      for (int j = 0; j < DIM; j++) s = fma(Ji[l][j], S[j][i], s);
      M[l][i] = s * W;
    }
  const double hw = AXI ? hoop / Rad * W : 0.;
  if constexpr (NEN == NIP) {
    // the quads and the hexahedron: every point's J^-1 S W (and hoop term) through the element's
    // shared memory; lane k assembles node k from all of them
    constexpr int ST = DIM * DIM + (AXI ? 1 : 0);
    double *mine = buf + pt * ST;
#pragma unroll
    for (int l = 0; l < DIM; l++)
#pragma unroll
      for (int i = 0; i < DIM; i++) mine[l * DIM + i] = M[l][i];
    if (AXI) mine[DIM * DIM] = hw;
    __syncwarp();
    if (valid) {
      double f[DIM];
#pragma unroll
      for (int i = 0; i < DIM; i++) f[i] = 0.;
#pragma unroll
      for (int q = 0; q < NIP; q++) {
        const double *Mq = buf + q * ST;
#pragma unroll
        for (int l = 0; l < DIM; l++) {
          const double d = pdN<ET>(q, pt, l);
#pragma unroll
          for (int i = 0; i < DIM; i++) f[i] = fma(d, Mq[l * DIM + i], f[i]);
        }
        if (AXI) f[0] = fma(pN<ET>(q, pt), Mq[DIM * DIM], f[0]);
      }
#pragma unroll
      for (int i = 0; i < DIM; i++) a.kx[(long)i * a.kxStride + (long)e * NEN + pt] = f[i];
    }
    return;
  }
  double *row = red[wib][slot][pt];
#pragma unroll
  for (int k = 0; k < NEN; k++)
#pragma unroll
    for (int i = 0; i < DIM; i++) {
      double s = 0.;
#pragma unroll
      for (int l = 0; l < DIM; l++) s = fma(pdN<ET>(pt, k, l), M[l][i], s);
      if (AXI && i == 0) s = fma(pN<ET>(pt, k), hw, s);
      row[k * DIM + i] = s;
    }
  __syncwarp();
  if (valid) {
    // lane pt sums node pt (and pt + NIP, ... when the element has more nodes than points)
#pragma unroll
    for (int j = 0; j < (NEN + NIP - 1) / NIP; j++) {
      const int k = pt + j * NIP;
      if (k < NEN) {
#pragma unroll
        for (int i = 0; i < DIM; i++) {
          double s = 0.;
#pragma unroll
          for (int q = 0; q < NIP; q++) s += red[wib][slot][q][k * DIM + i];
          a.kx[(long)i * a.kxStride + (long)e * NEN + k] = s;
        }
      }
    }
  }
}

// ------------------------------------------------------------------ assembly, / mass, max |.|
template <int DIM>
__global__ void __launch_bounds__(256) k_pulse_gather(PulseArgs a, int EN)
{
  DevTime *tm = a.tm;
  if (tm->done | tm->status | tm->pulseDone) return;
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  double mx = 0.;
  if (n < a.N) {
    double f[DIM];
#pragma unroll
    for (int c = 0; c < DIM; c++) f[c] = 0.;
    for (int q = a.start[n]; q < a.start[n + 1]; q++) {
      const int ent = a.entry[q];
#pragma unroll
      for (int c = 0; c < DIM; c++) f[c] = RADD(f[c], a.kx[(long)c * EN + ent]);
    }
    // K (x_raw / scale) = (K x_raw) / scale: the normalisation of the previous iterate
    // (Domain.C:926 EV /= fmax) is applied here once per degree of freedom
    const double m = a.mass[n], scale = tm->pulseScale;
#pragma unroll
    for (int c = 0; c < DIM; c++) {
      const double val = f[c] / scale / m;
      mx = fmax(mx, fabs(val));
      a.ev[(long)n * DIM + c] = val;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  __shared__ double wm[8];
  if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x == 0) {
    double b = wm[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); w++) b = fmax(b, wm[w]);
    atomicMax(&tm->pulseMaxBits, (unsigned long long)__double_as_longlong(b));
  }
}

__global__ void k_pulse_check(DevTime *tm, int maxIt)
{
  if (tm->done | tm->status | tm->pulseDone) return;
  const double fmax = __longlong_as_double((long long)tm->pulseMaxBits);
  tm->pulseMaxBits = 0ull;
  tm->pulseIter++;
  tm->pulseTotal++;
  const double d = RSUB(fmax, tm->fmax0);
  const double convergence = (d < 0 ? -d : d) / fmax;
  if (convergence < kPulseConvergence) tm->pulseDone = 1;
  tm->fmax0 = fmax;
  tm->pulseScale = fmax;
  if (tm->pulseIter > maxIt) {
    tm->status = DNL_ERR_PULSE_NOCONV;
    tm->badElem = -1;
    return;
  }
  if (tm->pulseDone) tm->fmax = sqrt(fmax);
  if (!(fmax > 0.)) {
    tm->status = DNL_ERR_PULSE_NOCONV;
    tm->badElem = -1;
  }
}

// Limit of the power iteration (Domain.C:936-939, 1000 iterations); dnl_set_iteration_caps lowers
// it to exercise the non-convergence status.
int &pulse_cap()
{
  static int cap = kPulseMaxIt;
  return cap;
}

__global__ void k_pulse_begin(DevTime *tm)
{
  if (tm->done | tm->status) return;
  tm->pulseDone = 0;
  tm->pulseIter = 0;
  tm->pulseMaxBits = 0ull;
}

// ------------------------------------------------------------------ driver
int launch_pulse(dnl_handle *h, cudaStream_t s)
{
  static bool tables = false;
  if (!tables) {
    set_pulse_tables();
    tables = true;
  }
  if (!h->pj) return DNL_ERR_ARG;
  PulseArgs a;
  a.E = h->E;
  a.N = h->N;
  a.conn = h->conn;
  for (int r = 0; r < 3; r++) a.x[r] = h->x[r];
  a.pj = h->pj;
  a.ev = h->ev;
  a.kx = h->kx;
  a.kxStride = h->EN;
  a.start = h->n2eStart;
  a.entry = h->n2e;
  a.mass = h->mass;
  a.tm = h->tm;
  a.C00 = h->C00;
  a.C01 = h->C01;
  a.C33 = h->C33;
  a.elemMat = h->hooke ? h->elemMat : nullptr;
  a.hooke = h->hooke;
  // Domain::fmax0 == 0: the vector starts as the ramp EV(0) = 1, EV(i) = EV(i-1) - 2/(noddl-1)
  DevTime t;
  if (cudaMemcpyAsync(&t, h->tm, sizeof t, cudaMemcpyDeviceToHost, s) != cudaSuccess) return DNL_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return DNL_ERR_CUDA;
  if (t.done || t.status) return 0;
  if (t.fmax0 == 0) {
    const long noddl = (long)h->dim * h->N;
    std::vector<double> ev(noddl);
    ev[0] = 1.0;
    for (long i = 1; i < noddl; i++) ev[i] = ev[i - 1] - 2. / (noddl - 1);
    if (cudaMemcpyAsync(h->ev, ev.data(), sizeof(double) * noddl, cudaMemcpyHostToDevice, s) != cudaSuccess)
      return DNL_ERR_CUDA;
    const double one = 1.0;
    if (cudaMemcpyAsync(&h->tm->pulseScale, &one, sizeof one, cudaMemcpyHostToDevice, s) != cudaSuccess)
      return DNL_ERR_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return DNL_ERR_CUDA;
  }
  const long nthreads = (long)h->E * h->nip;
  const int gridIP = (int)((nthreads + 127) / 128);
  const int gridN = (h->N + 255) / 256;
  // further element groups: their own element type, connectivity, kinematics and product slots
  std::vector<PulseArgs> ga(h->nextra, a);
  for (int gi = 0; gi < h->nextra; gi++) {
    const ElemGroup &g = h->extra[gi];
    ga[gi].E = g.E;
    ga[gi].conn = g.conn;
    ga[gi].pj = g.pj;
    ga[gi].kx = h->kx + g.feOff;
    ga[gi].elemMat = h->hooke ? h->elemMat + g.eOff : nullptr;  // element materials over all groups
    if (!g.pj) return DNL_ERR_ARG;
  }
  auto gridOf = [](const ElemGroup &g) { return (int)(((long)g.E * g.nip + 127) / 128); };
  prof_begin(h, s);
  k_pulse_begin<<<1, 1, 0, s>>>(h->tm);
  DNL_BY_ETYPE(h->etype, (k_pulse_setup<ET><<<gridIP, 128, 0, s>>>(a)));
  for (int gi = 0; gi < h->nextra; gi++)
    DNL_BY_ETYPE(h->extra[gi].etype, (k_pulse_setup<ET><<<gridOf(h->extra[gi]), 128, 0, s>>>(ga[gi])));
  prof_end(h, DNL_PROF_PULSE, s);
  launch_counter() += 2 + h->nextra;
  const int batch = 4;
  for (int round = 0; round < (pulse_cap() + batch) / batch + 1; round++) {
    for (int b = 0; b < batch; b++) {
      prof_begin(h, s);
      DNL_BY_ETYPE(h->etype, (k_pulse_kx<ET><<<gridIP, 128, 0, s>>>(a)));
      for (int gi = 0; gi < h->nextra; gi++)
        DNL_BY_ETYPE(h->extra[gi].etype, (k_pulse_kx<ET><<<gridOf(h->extra[gi]), 128, 0, s>>>(ga[gi])));
      if (h->dim == 2) {
        k_pulse_gather<2><<<gridN, 256, 0, s>>>(a, (int)h->EN);
      } else {
        k_pulse_gather<3><<<gridN, 256, 0, s>>>(a, (int)h->EN);
      }
      k_pulse_check<<<1, 1, 0, s>>>(h->tm, pulse_cap());
      prof_end(h, DNL_PROF_PULSE, s);
      launch_counter() += 3 + h->nextra;
    }
    if (cudaPeekAtLastError() != cudaSuccess) return DNL_ERR_CUDA;
    if (cudaMemcpyAsync(&t, h->tm, sizeof t, cudaMemcpyDeviceToHost, s) != cudaSuccess) return DNL_ERR_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return DNL_ERR_CUDA;
    if (t.pulseDone || t.status || t.done) break;
  }
  return 0;
}

}  // namespace dnl
