// Element kernels of libdnlgpu (sm_103a, FP64).
//
// k_elem<ET>   one pass of Domain::computeInternalMatrices + Domain::computeInternalForces:
//              per integration point the shape-function gradients (Element2D.C:53-126,
//              Element3D.C:53-113), the incremental F of the Current delta_disp
//              (ElementAx.C:114-136, Element3D.C:182-205), the Jacobi polar decomposition
//              (Tensor2.C:1154-1259), the J2 radial return (Element.C:245-345), the element-mean
//              pressure and RFI rotation (Element.C:351-401) and B^T sigma (Element.C:164-214).
// k_mass<ET>   Element::computeMassMatrix (Element.C:411-454).
// k_courant    ElQua4nAx::getLength (ElQua4nAx.C:131-143) or the tetrahedra's shortest edge
//              (ElTet4n3D.C:151-166) over Element::getSoundSpeed, min-reduced (Domain.C:1613-1646).
//
// Threading: one thread per integration point; the NIP threads of an element are adjacent lanes
// of one warp (32 % NIP == 0), so the element-mean pressure and the force sum over integration
// points are warp-local (shuffles and a per-warp shared-memory transpose), and the
// integration-point state, stored component-major, is read and written with coalesced accesses.
// Where an element has more nodes than integration points (the tetrahedra), lane pt assembles
// nodes pt, pt + NIP, ...
//
// Rounding: GB300 executes FP64 at a small fraction of its other rates, so the kernels are written
// to minimise FP64 instructions with explicit fused multiply-adds (this file is compiled with
// -fmad=false: the compiler fuses nothing by itself, so every instantiation of the element code --
// single mesh, batch, tape, caller-allocated -- rounds identically) -- except in C = F^T F, which
// uses __dmul_rn/__dadd_rn in the reference's association order (F itself is formed as
// I + G_u J^-1, its diagonal sums added to 1 last); the Jacobi rotations then move the eigenvalues
// by a few ulps of 1 against the reference's (see jacobi_rotate).  Elsewhere results differ from
// the reference by a few units in the last place; the parity tests hold them to 1e-12 per pass.
#include <cstdio>
#include <cstring>

#include "dnl_common.cuh"
#include "dnl_node.cuh"

namespace dnl {

#define RMUL __dmul_rn
#define RADD __dadd_rn
#define RSUB __dsub_rn

// Shape-function values at the Gauss points, formed by the same constant expressions as
// ElQua4nAx.C:43-67 and ElHex8n3D.C:73-104 (e.g. (2.0 + sqrt(3.0)) / 6.0); the 10-node
// tetrahedron's full tables (tet10_tables).
struct ShapeConst {
  double axN[3], axD[2];  // axi: N by number of sign disagreements, dN/dxi by the other axis
  double hxN[4], hxD[3];  // hex: likewise over three axes
  double t10N[4][10], t10D[4][10][3];
};
__constant__ ShapeConst c_shape;

void set_shape_tables()
{
  ShapeConst s;
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
  cudaMemcpyToSymbol(c_shape, &s, sizeof s);
}

// Limits of the element pass's bounded loops: Jacobi passes of the polar decomposition (a
// convergence check and a rotation each; Tensor2.C:1169, 29) and Newton iterations of the radial
// return (Element.C:327-330, 2000).  The defaults are the reference's; dnl_set_iteration_caps lowers
// them to exercise the non-convergence statuses.
__constant__ int c_caps[2] = {kPolarMaxIt - 1, kRadialReturnMaxIt};

int set_iteration_caps(int rotations, int newton)
{
  const int caps[2] = {rotations, newton};
  return cudaMemcpyToSymbol(c_caps, caps, sizeof caps) == cudaSuccess ? 0 : DNL_ERR_CUDA;
}

// Stopping tests of the same two loops: the polar decomposition stops once every off-diagonal
// |C_pq| is below c_polarTol (Tensor2.C:1180, 1e-9), the radial return once |f / sigma_y| is at
// most c_returnTol (Element.C:315, 1e-8).  The defaults are the reference's; dnl_set_stop_tolerances
// tightens them for checks of derivatives against difference quotients, which these tests make
// non-smooth (a parameter change can add or remove an iteration).
__constant__ double c_polarTol = kPolarPrecision;
__constant__ double c_returnTol = kRadialReturnPrecision;

int set_stop_tolerances(double polar, double radial)
{
  return cudaMemcpyToSymbol(c_polarTol, &polar, sizeof polar) == cudaSuccess &&
                 cudaMemcpyToSymbol(c_returnTol, &radial, sizeof radial) == cudaSuccess
             ? 0
             : DNL_ERR_CUDA;
}

long long &launch_counter()
{
  static long long n = 0;
  return n;
}

// Node / Gauss-point signs: xi = bit0^bit1, eta = bit1, zeta = bit2 of the local index
// (ElQua4nAx and ElHex8n3D number nodes counter-clockwise per face, bottom face first, and list
// Gauss points in the same pattern).
__device__ __forceinline__ int sgx(int k) { return (k ^ (k >> 1)) & 1; }
__device__ __forceinline__ int sgy(int k) { return (k >> 1) & 1; }
__device__ __forceinline__ int sgz(int k) { return (k >> 2) & 1; }

// -x on the bit pattern (integer pipe, not FP64).
__device__ __forceinline__ double flip_sign(double a)
{
  return __longlong_as_double(__double_as_longlong(a) ^ (long long)0x8000000000000000ull);
}

template <int ET> struct Shape;
template <> struct Shape<DNL_ELQUA4NAX> {
  __device__ __forceinline__ static double N(int pt, int k)
  {
    const int d = (sgx(k) ^ sgx(pt)) + (sgy(k) ^ sgy(pt));
    return d == 0 ? c_shape.axN[0] : (d == 1 ? c_shape.axN[1] : c_shape.axN[2]);
  }
  __device__ __forceinline__ static double dN(int pt, int k, int c)
  {
    const int other = c == 0 ? (sgy(k) ^ sgy(pt)) : (sgx(k) ^ sgx(pt));
    const double v = other ? c_shape.axD[1] : c_shape.axD[0];
    const int s = c == 0 ? sgx(k) : sgy(k);
    return s ? v : flip_sign(v);
  }
};
template <> struct Shape<DNL_ELQUA4N2D> : Shape<DNL_ELQUA4NAX> {};  // same tables (ElQua4n2D.C:31-101)
template <> struct Shape<DNL_ELHEX8N3D> {
  __device__ __forceinline__ static double N(int pt, int k)
  {
    const int d = (sgx(k) ^ sgx(pt)) + (sgy(k) ^ sgy(pt)) + (sgz(k) ^ sgz(pt));
    return d == 0 ? c_shape.hxN[0] : (d == 1 ? c_shape.hxN[1] : (d == 2 ? c_shape.hxN[2] : c_shape.hxN[3]));
  }
  __device__ __forceinline__ static double dN(int pt, int k, int c)
  {
    const int dx = sgx(k) ^ sgx(pt), dy = sgy(k) ^ sgy(pt), dz = sgz(k) ^ sgz(pt);
    const int d = c == 0 ? dy + dz : (c == 1 ? dx + dz : dx + dy);
    const double v = d == 0 ? c_shape.hxD[0] : (d == 1 ? c_shape.hxD[1] : c_shape.hxD[2]);
    const int s = c == 0 ? sgx(k) : (c == 1 ? sgy(k) : sgz(k));
    return s ? v : flip_sign(v);
  }
};


// ElTet4n3D (ElTet4n3D.C:33-57): one point, N = 1/4, dN/dxi of the barycentric coordinates
template <> struct Shape<DNL_ELTET4N3D> {
  static constexpr double kWeight = 1. / 6.;
  __device__ __forceinline__ static double N(int, int) { return 0.25; }
  __device__ __forceinline__ static double dN(int, int k, int c)
  {
    return k == 0 ? -1.0 : (k - 1 == c ? 1.0 : 0.0);
  }
};
template <> struct Shape<DNL_ELTET10N3D> {
  static constexpr double kWeight = 1.0 / 24.0;
  __device__ __forceinline__ static double N(int pt, int k) { return c_shape.t10N[pt][k]; }
  __device__ __forceinline__ static double dN(int pt, int k, int c) { return c_shape.t10D[pt][k][c]; }
};
// The one-point hexahedron (not a reference element): the centre of ElHex8n3D's reference cube,
// N = 1/8, dN/dxi = (sign of the node's coordinate) / 8, weight 8
template <> struct Shape<DNL_ELHEX8N3D_1PT> {
  static constexpr double kWeight = 8.0;
  __device__ __forceinline__ static double N(int, int) { return 0.125; }
  __device__ __forceinline__ static double dN(int, int k, int c)
  {
    const int s = c == 0 ? sgx(k) : (c == 1 ? sgy(k) : sgz(k));
    return s ? 0.125 : -0.125;
  }
};
// integration weight x detJ (Element.C:183); the quads' and the hexahedron's weight is 1
template <int ET> __device__ __forceinline__ double weighted(double detJ)
{
  if constexpr (ET == DNL_ELTET4N3D || ET == DNL_ELTET10N3D || ET == DNL_ELHEX8N3D_1PT)
    return RMUL(Shape<ET>::kWeight, detJ);
  else
    return detJ;
}

__device__ __forceinline__ void record_error(DevTime *tm, int code, int e)
{
  if (atomicCAS(&tm->status, 0, code) == 0) tm->badElem = e;
}

// |a| > |b| and |a| < |b| on the bit patterns (finite doubles): integer compares keep them off the
// FP64 pipe, which on GB300 issues 2 thread-instructions per SM per cycle.
__device__ __forceinline__ unsigned long long abits(double a)
{
  return (unsigned long long)__double_as_longlong(a) & 0x7fffffffffffffffull;
}
__device__ __forceinline__ bool abs_gt(double a, double b) { return abits(a) > abits(b); }

constexpr int ilog2(int n) { return n <= 1 ? 0 : 1 + ilog2(n / 2); }

// x * 2^K by adding K to the exponent field (integer pipe): the product's exact value for +-0 and
// for normal x whose product is normal, which is every call site's case (eigenvalue logarithms,
// sums of strain traces, pivot entries and diagonal differences of C, all far from the ends of the
// range); infinite and NaN x are returned unchanged (as the product would be, NaN payload aside).
template <int K>
__device__ __forceinline__ double scale2(double x)
{
  const int hi = __double2hiint(x);
  const int ef = (hi >> 20) & 0x7ff;
  const double y = __hiloint2double(hi + K * (1 << 20), __double2loint(x));
  return ef == 0 || ef == 0x7ff ? x : y;
}

// ln(1 + x) for |x| <= 2^-6 by the Mercator series x - x^2/2 + x^3/3 - ... in Horner form, to
// x^9/9, to x^6/6 when |x| <= 2^-9, to x^4/4 when |x| <= 2^-14: the alternating series' truncation,
// at most the first omitted term, is below 2^-56 |x| in each case (2^-54 / 10, 2^-54 / 7,
// 2^-56 / 5), under a tenth of an ulp of the result, which is within about an ulp (9, 6 or 4 FP64
// instructions where the library logarithm takes 28).  The length depends on the point's own x
// only, so a point's result does not depend on the other points of its warp; a warp runs the
// longest form any of its points needs.
__device__ __forceinline__ double log1p_series(double x)
{
  double s = -1. / 4.;
  if (abits(x) > abits(0x1p-14)) {
    double u = -1. / 6.;
    if (abits(x) > abits(0x1p-9)) {
      double v = 1. / 9.;
      v = fma(x, v, -1. / 8.);
      v = fma(x, v, 1. / 7.);
      u = fma(x, v, -1. / 6.);
    }
    u = fma(x, u, 1. / 5.);
    s = fma(x, u, -1. / 4.);
  }
  s = fma(x, s, 1. / 3.);
  s = fma(x, s, -1. / 2.);
  s = fma(x, s, 1.);
  return x * s;
}
constexpr double kSeriesMax = 0.015625;  // 2^-6

// ln(l) of an eigenvalue of C = F^T F: l - 1 is exact for l in [1/2, 2], and within 2^-6 of 1
// (strain increments below ~0.8 % per step, nearly every point of every step) the series above
// applies; elsewhere the library logarithm.
__device__ __forceinline__ double ln_eig(double l)
{
  const double x = l - 1.0;
  return abits(x) <= abits(kSeriesMax) ? log1p_series(x) : log(l);
}

// e^t for |t| <= 2^-5 by its Taylor series in Horner form, to t^7/7!, to t^5/5! when |t| <= 2^-9,
// to t^3/3! when |t| <= 2^-14: the truncation is below 2^-55 (2^-40 / 8!, 2^-54 / 6!,
// 2^-56 / 4!), with e^t within 4 % of 1 a tenth of an ulp (7, 5 or 3 FP64 instructions where the
// library exponential takes 15); the length depends on t only (as log1p_series).
__device__ __forceinline__ double exp_series(double t)
{
  double s = 1. / 6.;
  if (abits(t) > abits(0x1p-14)) {
    double u = 1. / 120.;
    if (abits(t) > abits(0x1p-9)) u = fma(t, fma(t, 1. / 5040., 1. / 720.), 1. / 120.);
    s = fma(t, fma(t, u, 1. / 24.), 1. / 6.);
  }
  s = fma(t, s, 0.5);
  s = fma(t, s, 1.);
  return fma(t, s, 1.);
}

// Yield stress and hardening slope of the non-power laws at x = evp + sqrt(2/3) gamma:
// IsoHardElastoplasticTabular through DiscreteFunction::getValue / getSlope (the segment ending at
// the first abscissa >= x, that point's own ordinate when equal, 0 beyond the table; the table is
// ascending, so a binary search finds the same segment as the reference's linear one) and
// IsoHardMetafor (IsoHardMetafor.C:132-153, operations in the reference's order).
__device__ __noinline__ void hardening_law(const HardLaw m, double x, double &sig, double &h)
{
  if (m.law == DNL_HARD_TABULAR) {
    const double *X = m.tab, *Y = m.tab + m.tabN;
    int lo = 1, hi = m.tabN;  // first i in [1, N) with X[i] >= x, else N
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (X[mid] >= x)
        hi = mid;
      else
        lo = mid + 1;
    }
    if (lo >= m.tabN) {
      sig = 0.;
      h = 0.;
      return;
    }
    const double x0 = X[lo - 1], x1 = X[lo], y0 = Y[lo - 1], y1 = Y[lo];
    sig = x1 == x ? y1 : ((x - x0) / (x1 - x0)) * (y1 - y0) + y0;
    h = (y1 - y0) / (x1 - x0);
    return;
  }
  const double *P = m.P;  // P1..P8
  const double e3 = exp(-P[2] * (x)), w = 1 + P[5] * x;
  sig = (P[1] - P[0]) * (1 - e3) + P[3] * pow(x, P[4]) + P[0] * pow(w, P[6]) + P[7] * x;
  if (x > 0.)
    h = ((P[1] - P[0]) * P[2] * e3 + P[3] * P[4] * pow(x, (P[4] - 1.0)) +
         P[0] * P[5] * P[6] * pow((1.0 + P[5] * x), (P[6] - 1.0)) + P[7]);
  else
    h = ((P[1] - P[0]) * P[2] * e3 + P[0] * P[5] * P[6] * pow((1.0 + P[5] * x), (P[6] - 1.0)) + P[7]);
}

// |x| and -x on the bit pattern (integer pipe).
__device__ __forceinline__ double iabs(double a) { return __longlong_as_double((long long)abits(a)); }
__device__ __forceinline__ double ineg(double a) { return flip_sign(a); }

// ----------------------------------------------------------------------------- Jacobi rotation
// Rotation angle of Tensor2.C:1195-1208.  With d = C_qq - C_pp and e = 2 C_pq the reference's
// t = 1 / (alpha + sign(alpha) sqrt(alpha^2 + 1)), alpha = d / e, is tan(theta) with
// cos(2 theta) = |d| / sqrt(d^2 + e^2) >= 0 and sign(theta) = sign(d e) (theta = +pi/4 when
// d = 0).  Half-angle identities give c = sqrt((1 + cos 2theta) / 2) and
// s = sin(2 theta) / (2 c) = |C_pq| w / c with w = 1 / sqrt(d^2 + e^2), and t = s / c: two
// reciprocal square roots (1 / c is the second) and no division.  The angle agrees with the
// reference's to a few ulps; the rotated diagonal is stationary in the angle.
__device__ __forceinline__ void jacobi_angle(double fpp, double fqq, double fpq, double &c, double &s,
                                             double &t)
{
  const double d = fqq - fpp;
  const double w = rsqrt(fma(d, d, scale2<2>(fpq) * fpq));
  const double h = fma(scale2<-1>(iabs(d)), w, 0.5);  // cos^2(theta)
  const double r = rsqrt(h);                    // 1 / c
  c = h * r;
  const double sv = iabs(fpq) * w * r;
  const double tv = sv * r;
  const bool neg = abits(d) != 0 && ((__double_as_longlong(d) ^ __double_as_longlong(fpq)) < 0);
  s = neg ? ineg(sv) : sv;
  t = neg ? ineg(tv) : tv;
}

// One rotation of Tensor2::polarDecomposeLnU (Tensor2.C:1183-1240): C <- R^T C R with R the plane
// rotation (c, s) on pivot (P, Q), Rot <- Rot R.  The pivot is a run-time case k (0: (0,1),
// 1: (0,2), 2: (1,2); O is the third index) so that the lanes of a warp, which pick different
// pivots, execute one rotation instead of one per distinct pivot.  On a = C_PP, b = C_QQ,
// x = C_PQ, y = C_PO, z = C_QO the rotation that annihilates x gives, in closed form,
// a' = a - t x, b' = b + t x, x' = 0, y' = c y - s z, z' = s y + c z (Rutishauser's form of the
// Jacobi update): 6 FP64 operations instead of the 27 products and sums of R^T C R.  The
// reference forms R^T C R in full, so its diagonal carries several roundings at the scale of 1 and
// its x' a rounding residual; the closed form rounds once.  The two diagonals differ by a few ulps
// of 1 (at most 9 in 4e5 random 3x3 cases, the same order as the angle's own effect) and the
// pivot sequences are the same (x' is below the 1e-9 stop either way).
// TWO_D (axisymmetric and plane strain): C is block diagonal and the pivot is always (0, 1).
// FIRST: Rot is still the identity, so Rot R is R itself, whose entries are c, s, -s, 0 and 1:
// selected, not multiplied (the products by 0 and 1 that the general update forms are exact and
// give the same doubles, +0 included).
template <bool TWO_D, bool FIRST = false>
__device__ __forceinline__ void jacobi_rotate(int k, double &f00, double &f11, double &f22, double &f01,
                                              double &f02, double &f12, double rot[3][3], double x)
{
  const double a = k == 2 ? f11 : f00;
  const double b = k == 0 ? f11 : f22;
  double c, s, t;
  jacobi_angle(a, b, x, c, s, t);
  const double ms = ineg(s);
  const double a2 = fma(ineg(t), x, a);
  const double b2 = fma(t, x, b);
  const double x2 = 0.;
  if (TWO_D) {
    f00 = a2;
    f11 = b2;
    f01 = x2;
  } else {
    const double y = k == 0 ? f02 : f01, z = k == 2 ? f02 : f12;
    const double y2 = fma(c, y, ms * z);
    const double z2 = fma(s, y, c * z);
    f00 = k == 2 ? f00 : a2;
    f11 = k == 0 ? b2 : (k == 2 ? a2 : f11);
    f22 = k == 0 ? f22 : b2;
    f01 = k == 0 ? x2 : y2;
    f02 = k == 0 ? y2 : (k == 1 ? x2 : z2);
    f12 = k == 2 ? x2 : z2;
  }
  if (FIRST) {
    // pivot (p, q): R_pp = R_qq = c, R_pq = s, R_qp = -s, R_oo = 1, zero elsewhere
    const int p = k == 2 ? 1 : 0, q = k == 0 ? 1 : 2;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++)
        rot[i][j] = (i == p && j == p) || (i == q && j == q) ? c
                    : (i == p && j == q)                     ? s
                    : (i == q && j == p)                     ? ms
                    : (i != p && i != q && i == j)           ? 1.
                                                             : 0.;
    return;
  }
#pragma unroll
  for (int i = 0; i < (TWO_D ? 2 : 3); i++) {
    const double rp = k == 2 ? rot[i][1] : rot[i][0];
    const double rq = k == 0 ? rot[i][1] : rot[i][2];
    const double np = fma(rp, c, rq * ms), nq = fma(rp, s, rq * c);
    rot[i][0] = k == 2 ? rot[i][0] : np;
    rot[i][1] = k == 0 ? nq : (k == 2 ? np : rot[i][1]);
    rot[i][2] = k == 0 ? rot[i][2] : nq;
  }
}

// ----------------------------------------------------------------------------- element kernel
// One Gauss point of one element: lane `pt` of the NIP adjacent lanes that hold element e.  All
// lanes of a warp must call it (the pressure average and the force sum are warp-collective);
// lanes with valid == false compute on a clamped element and store nothing.  `red` is this
// element's NIP x NEN*DIM slice of shared memory; `m` and `tm` are the element's material and
// time/status record (one per mesh, or per instance in a batch).
// GENERAL: the material may carry any hardening law (otherwise the power law, compiled alone).
template <int ET, bool TAPE = false, bool GENERAL = false>
__device__ __forceinline__ void elem_ip(const ElemArgs &a, const Material &m, DevTime *tm, int e,
                                        int pt, bool valid, int lane, double *red)
{
  using T = Elem<ET>;
  using L = IpLayout<ET>;
  using SH = Shape<ET>;
  using TL = TapeLayout<ET>;
  constexpr int NIP = T::NIP, NEN = T::NEN, DIM = T::DIM, NS = T::NS;
  constexpr bool AXI = ET == DNL_ELQUA4NAX;  // radius, hoop strain and hoop force
  constexpr bool TWO_D = DIM == 2;           // the 2 + 1 block structure of F, C, R, S
  const long nIP = (long)a.E * NIP;
  const long ipx = (long)e * NIP + pt;
  auto tape = [&](int slot, double v) {
    if (TAPE && valid) a.tape[(long)slot * nIP + ipx] = v;
  };

  int node[NEN];
#pragma unroll
  for (int k = 0; k < NEN; k++) node[k] = __ldg(a.conn + (long)k * a.E + e);

  // ---- kinematics: J = sum_k dN/dxi (x) x_k and G_u = sum_k dN/dxi (x) du_k (Current field)
  double J[DIM][DIM], GU[DIM][DIM];
#pragma unroll
  for (int r = 0; r < DIM; r++)
#pragma unroll
    for (int c = 0; c < DIM; c++) J[r][c] = GU[r][c] = 0.;
  double Rad = 0.;  // axisymmetric radius at the Gauss point, sum N_k x_k
  double vR = 0.;   // axisymmetric sum N_k du_k,r
  constexpr bool EDGES = ET == DNL_ELHEX8N3D || ET == DNL_ELQUA4NAX || ET == DNL_ELQUA4N2D;
  if constexpr (EDGES) {
    // the element's edge differences of x and du, a few per lane, exchanged through its shared
    // memory (free until the force assembly): DIM^2 (NEN / 2) FMA each instead of DIM^2 NEN
    using EG = Edges<ET>;
    constexpr int NE = EG::NE, PER = NE / DIM;
    double *ex = red, *eu = red + NE * DIM;
#pragma unroll
    for (int j = 0; j < (NE + NIP - 1) / NIP; j++) {
      const int eg = pt + j * NIP;
      if (eg < NE) {
        const int lo = __ldg(a.conn + (long)edge_node(EG::LO, eg) * a.E + e);
        const int hi = __ldg(a.conn + (long)edge_node(EG::HI, eg) * a.E + e);
#pragma unroll
        for (int r = 0; r < DIM; r++) {
          ex[eg * DIM + r] = RSUB(a.x[r][hi], a.x[r][lo]);
          eu[eg * DIM + r] = RSUB(a.du[r][hi], a.du[r][lo]);
        }
      }
    }
    __syncwarp();
#pragma unroll
    for (int c = 0; c < DIM; c++)
#pragma unroll
      for (int q = 0; q < PER; q++) {
        const int eg = c * PER + q;
        const double w = SH::dN(pt, edge_node(EG::HI, eg), c);
#pragma unroll
        for (int r = 0; r < DIM; r++) {
          J[r][c] = fma(w, ex[eg * DIM + r], J[r][c]);
          GU[r][c] = fma(w, eu[eg * DIM + r], GU[r][c]);
        }
      }
    __syncwarp();  // the force assembly reuses the buffer
    if (AXI) {
#pragma unroll
      for (int k = 0; k < NEN; k++) {
        Rad = fma(SH::N(pt, k), a.x[0][node[k]], Rad);
        vR = fma(SH::N(pt, k), a.du[0][node[k]], vR);
      }
    }
  } else {
#pragma unroll
    for (int k = 0; k < NEN; k++) {
      double xk[DIM], uk[DIM];
#pragma unroll
      for (int r = 0; r < DIM; r++) {
        xk[r] = a.x[r][node[k]];
        uk[r] = a.du[r][node[k]];
      }
#pragma unroll
      for (int c = 0; c < DIM; c++) {
        const double d = SH::dN(pt, k, c);
#pragma unroll
        for (int r = 0; r < DIM; r++) {
          J[r][c] = fma(d, xk[r], J[r][c]);
          GU[r][c] = fma(d, uk[r], GU[r][c]);
        }
      }
    }
  }
  double detJ, Ji[DIM][DIM];
  if (TWO_D) {
    detJ = fma(J[0][0], J[1][1], -J[0][1] * J[1][0]);
    const double r = nr_rcp(detJ);  // the IEEE reciprocal but in rare hard cases (within an ulp)
    Ji[0][0] = J[1][1] * r;
    Ji[0][1] = -J[0][1] * r;
    Ji[1][0] = -J[1][0] * r;
    Ji[1][1] = J[0][0] * r;
    if (detJ < 0. && valid) record_error(tm, DNL_ERR_NEG_DETJ, a.eBase + e);
  } else {
    const double c00 = fma(J[1][1], J[2][2], -J[1][2] * J[2][1]);
    const double c01 = fma(J[1][2], J[2][0], -J[1][0] * J[2][2]);
    const double c02 = fma(J[1][0], J[2][1], -J[1][1] * J[2][0]);
    detJ = fma(J[0][0], c00, fma(J[0][1], c01, J[0][2] * c02));
    const double r = nr_rcp(detJ);  // the IEEE reciprocal but in rare hard cases (within an ulp)
    Ji[0][0] = c00 * r;
    Ji[1][0] = c01 * r;
    Ji[2][0] = c02 * r;
    Ji[0][1] = fma(J[0][2], J[2][1], -J[0][1] * J[2][2]) * r;
    Ji[1][1] = fma(J[0][0], J[2][2], -J[0][2] * J[2][0]) * r;
    Ji[2][1] = fma(J[0][1], J[2][0], -J[0][0] * J[2][1]) * r;
    Ji[0][2] = fma(J[0][1], J[1][2], -J[0][2] * J[1][1]) * r;
    Ji[1][2] = fma(J[0][2], J[1][0], -J[0][0] * J[1][2]) * r;
    Ji[2][2] = fma(J[0][0], J[1][1], -J[0][1] * J[1][0]) * r;
    if (detJ == 0. && valid) record_error(tm, DNL_ERR_SINGULAR, a.eBase + e);
  }
  if (TAPE) {
#pragma unroll
    for (int l = 0; l < DIM; l++)
#pragma unroll
      for (int c = 0; c < DIM; c++) tape(TL::JI + l * DIM + c, Ji[l][c]);
    tape(TL::DETJ, detJ);
    tape(TL::RAD, Rad);
  }

  // ---- F = I + sum_k du_k (x) dN_k = I + G_u J^-1 (no per-node physical gradients); the
  // diagonal's sums are added to 1 last
  double F[3][3] = {{1., 0., 0.}, {0., 1., 0.}, {0., 0., 1.}};
#pragma unroll
  for (int r = 0; r < DIM; r++)
#pragma unroll
    for (int c = 0; c < DIM; c++) {
      double s = 0.;
#pragma unroll
      for (int l = 0; l < DIM; l++) s = fma(GU[r][l], Ji[l][c], s);
      F[r][c] = r == c ? RADD(1.0, s) : s;
    }
  // hoop stretch u_r / R by a reciprocal and one residual correction (quot)
  double vRR = 0.;
  if (AXI) {
    vRR = quot(vR, Rad, nr_rcp(Rad));
    F[2][2] = RADD(F[2][2], vRR);
  }
  if (TAPE) {
#pragma unroll
    for (int k = 0; k < 9; k++) tape(TL::F + k, F[k / 3][k % 3]);
#pragma unroll
    for (int r = 0; r < DIM; r++)
#pragma unroll
      for (int l = 0; l < DIM; l++) tape(TL::GU + r * DIM + l, GU[r][l]);
    tape(TL::VRR, vRR);
  }

  // ---- C = F^T F (Tensor2::Transpose then operator*), exact reference rounding
  double f[3][3];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = i; j < 3; j++) {
      double s;
      if (TWO_D && (i == 2) != (j == 2)) {
        s = 0.;
      } else if (TWO_D && i == 2) {
        s = RMUL(F[2][2], F[2][2]);
      } else if (TWO_D) {
        s = RADD(RMUL(F[0][i], F[0][j]), RMUL(F[1][i], F[1][j]));
      } else {
        s = RADD(RADD(RMUL(F[0][i], F[0][j]), RMUL(F[1][i], F[1][j])), RMUL(F[2][i], F[2][j]));
      }
      f[i][j] = s;
      f[j][i] = s;
    }

  // ---- Jacobi eigen-iteration (at most 29 rotations, c_caps[0]; Tensor2.C:1169)
  double rot[3][3] = {{1., 0., 0.}, {0., 1., 0.}, {0., 0., 1.}};
  bool conv = false;
  {
    double f00 = f[0][0], f11 = f[1][1], f22 = f[2][2], f01 = f[0][1], f02 = f[0][2], f12 = f[1][2];
    for (int it = 1; it <= c_caps[0]; it++) {
      // pivot of Tensor2.C:1173-1178: q = |C01| > |C02| ? 1 : 2, p = |C0q| > |C12| ? 0 : 1
      int k = 0;
      double fpq = f01;
      if (!TWO_D) {
        const bool q1 = abs_gt(f01, f02);
        const double f0q = q1 ? f01 : f02;
        const bool p0 = abs_gt(f0q, f12);
        k = p0 ? (q1 ? 0 : 1) : 2;
        fpq = p0 ? f0q : f12;
      }
      if (abits(fpq) < abits(c_polarTol)) {
        conv = true;
        break;
      }
      // the lanes still in the loop are all at the same iteration: a uniform branch
      if (it == 1)
        jacobi_rotate<TWO_D, true>(k, f00, f11, f22, f01, f02, f12, rot, fpq);
      else
        jacobi_rotate<TWO_D>(k, f00, f11, f22, f01, f02, f12, rot, fpq);
    }
    f[0][0] = f00;
    f[1][1] = f11;
    f[2][2] = f22;
  }
  if (!conv && valid) record_error(tm, DNL_ERR_JACOBI_NOCONV, a.eBase + e);

  // ---- ln U = sum ln(l)/2 v v^T,  R = F sum l^-1/2 v v^T
  double dE[3][3], Rr[3][3];
  {
    double lg[3], il[3];
#pragma unroll
    for (int cc = 0; cc < 3; cc++) {
      lg[cc] = scale2<-1>(ln_eig(f[cc][cc]));
      il[cc] = rsqrt(f[cc][cc]);
    }
    if (TAPE) {
      // eigenvectors and the divided differences of ln(l)/2 and l^-1/2 (Daleckii-Krein factors)
#pragma unroll
      for (int k = 0; k < 9; k++) tape(TL::V + k, rot[k / 3][k % 3]);
      const int P0[6] = {0, 1, 2, 0, 0, 1}, P1[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
      for (int k = 0; k < 6; k++) {
        const int i = P0[k], j = P1[k];
        double g, hh;
        if (i == j) {
          g = 0.5 * il[i] * il[i];        // 1 / (2 l)
          hh = -0.5 * il[i] * il[i] * il[i];  // -l^-3/2 / 2
        } else {
          const double li = f[i][i], lj = f[j][j];
          const double mean = 0.5 * (li + lj), q = (li - lj) / mean;
          // 2 atanh(q/2) / (2 q mean) for near-equal eigenvalues (series to q^4)
          g = fabs(q) < 1e-3 ? 0.5 * fma(q * q, fma(q * q, 1. / 80., 1. / 12.), 1.) / mean
                             : (lg[i] - lg[j]) / (li - lj);
          hh = -il[i] * il[j] / fma(li, il[i], lj * il[j]);
        }
        tape(TL::GD + k, g);
        tape(TL::HD + k, hh);
      }
    }
    // 2 + 1 block: Rot is the identity or the one rotation's [[c, s], [-s, c]], so the products
    // Rot_ic Rot_jc of the block are c c, s s and +-c s (the same doubles, three multiplications)
    const double pcc = TWO_D ? rot[0][0] * rot[0][0] : 0., pss = TWO_D ? rot[0][1] * rot[0][1] : 0.;
    const double pcs = TWO_D ? rot[0][0] * rot[0][1] : 0.;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = i; j < 3; j++) {
        double su = 0., sr = 0.;
        if (TWO_D && (i == 2 || j == 2)) {
          if (i == 2 && j == 2) {
            su = lg[2];
            sr = il[2];
          }
        } else {
#pragma unroll
          for (int cc = 0; cc < (TWO_D ? 2 : 3); cc++) {
            const double ext = !TWO_D      ? rot[i][cc] * rot[j][cc]
                               : i != j    ? (cc == 0 ? ineg(pcs) : pcs)
                               : (i == cc) ? pcc
                                           : pss;
            su = fma(lg[cc], ext, su);
            sr = fma(il[cc], ext, sr);
          }
        }
        dE[i][j] = dE[j][i] = su;
        Rr[i][j] = Rr[j][i] = sr;
      }
    if (TAPE) {
      const int P0[6] = {0, 1, 2, 0, 0, 1}, P1[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
      for (int k = 0; k < 6; k++) tape(TL::UI + k, Rr[P0[k]][P1[k]]);
    }
  }
  double R[3][3];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      if (TWO_D && (i == 2) != (j == 2)) {
        R[i][j] = 0.;
      } else if (TWO_D && i == 2) {
        R[i][j] = F[2][2] * Rr[2][2];
      } else {
        double s = 0.;
#pragma unroll
        for (int k = 0; k < (TWO_D ? 2 : 3); k++) s = fma(F[i][k], Rr[k][j], s);
        R[i][j] = s;
      }
    }
  if (TAPE) {
#pragma unroll
    for (int k = 0; k < 9; k++) tape(TL::R + k, R[k / 3][k % 3]);
  }

  // ---- strain, trial stress, J2 radial return (Element.C:245-345)
  double S[3][3], Ep[3][3], Epl[3][3];
  {
    // symmetric component order: xx yy zz xy [xz yz]
    const int I0[6] = {0, 1, 2, 0, 0, 1}, I1[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
    for (int k = 0; k < NS; k++) {
      const double sv = a.ip[(L::S + k) * nIP + ipx];
      const double ev = a.ip[(L::EPS + k) * nIP + ipx];
      const double pv = a.ip[(L::EPSP + k) * nIP + ipx];
      S[I0[k]][I1[k]] = S[I1[k]][I0[k]] = sv;
      Ep[I0[k]][I1[k]] = Ep[I1[k]][I0[k]] = ev + dE[I0[k]][I1[k]];
      Epl[I0[k]][I1[k]] = Epl[I1[k]][I0[k]] = pv;
    }
    if (TWO_D) {
      S[0][2] = S[2][0] = S[1][2] = S[2][1] = 0.;
      Ep[0][2] = Ep[2][0] = Ep[1][2] = Ep[2][1] = 0.;
      Epl[0][2] = Epl[2][0] = Epl[1][2] = Epl[2][1] = 0.;
    }
  }
  const double trace = dE[0][0] + dE[1][1] + dE[2][2];
  {
    const double tr3 = trace * (1.0 / 3.0);
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = i; j < 3; j++) {
        if (TWO_D && (i == 2) != (j == 2)) continue;
        const double dv = i == j ? dE[i][j] - tr3 : dE[i][j];
        S[i][j] = fma(m.G2, dv, S[i][j]);
        S[j][i] = S[i][j];
      }
  }
  double evp = a.ip[L::EVP * nIP + ipx];
  double evpn = a.ip[L::EVPN * nIP + ipx];
  bool plastic = false;
  {
    double ss = fma(S[0][0], S[0][0], fma(S[1][1], S[1][1], S[2][2] * S[2][2]));
    double off = S[0][1] * S[0][1];
    if (!TWO_D) off = fma(S[0][2], S[0][2], fma(S[1][2], S[1][2], off));
    ss = fma(2., off, ss);
    const double normS = sqrt(ss);
    const double Strial = kSqrt32 * normS;
    const bool power = !GENERAL || m.hard.law == DNL_HARD_POWER;
    double Sigv0, h0 = 0.;
    if (power)
      Sigv0 = RADD(m.A, RMUL(m.B, evpn));
    else if (GENERAL)
      hardening_law(m.hard, evp, Sigv0, h0);
    if (TAPE) {
      const int I0[6] = {0, 1, 2, 0, 0, 1}, I1[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
      for (int k = 0; k < NS; k++) tape(TL::STR + k, S[I0[k]][I1[k]]);
      tape(TL::NORMS, normS);
      tape(TL::GAM, 0.);
      tape(TL::XV, evp);
      tape(TL::XN, evpn);
      tape(TL::LXV, 0.);
    }
    if (GENERAL && !power && m.hard.law != DNL_HARD_ELASTIC && Strial > Sigv0) {
      // any other hardening law: the return of Element.C:282-345 with the law's
      // getIsotropicYieldStress / getIsotropicYieldHardening at evp + sqrt(2/3) gamma
      plastic = true;
      double gamma = (normS - kSqrt23 * Sigv0) / (m.G2 * (1.0 + h0 / m.G3));
      int iteration = 0;
      for (;;) {
        double Sigv, h;
        hardening_law(m.hard, RADD(evp, RMUL(kSqrt23, gamma)), Sigv, h);
        const double dfun = kSqrt32 * m.G2 + kSqrt23 * h;
        const double fun = dfun * gamma - (Strial - Sigv + h * kSqrt23 * gamma);
        if (fabs(fun / Sigv) > c_returnTol) {
          double dgamma = -fun / dfun;
          if (dgamma < 0 && fabs(dgamma) > gamma) dgamma = -gamma * 0.9;
          gamma += dgamma;
        } else {
          break;
        }
        iteration++;
        if (iteration > c_caps[1]) {
          if (valid) record_error(tm, DNL_ERR_RR_NOCONV, a.eBase + e);
          break;
        }
      }
      const double inv = 1. / normS;
      evp = RADD(evp, RMUL(kSqrt23, gamma));
      const double c2 = m.G2 * gamma;
#pragma unroll
      for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = i; j < 3; j++) {
          if (TWO_D && (i == 2) != (j == 2)) continue;
          const double n1 = S[i][j] * inv;
          S[i][j] = fma(-c2, n1, S[i][j]);
          Epl[i][j] = fma(gamma, n1, Epl[i][j]);
          S[j][i] = S[i][j];
          Epl[j][i] = Epl[i][j];
        }
    } else if (power && __double_as_longlong(Strial) > __double_as_longlong(Sigv0)) {  // both >= 0
      plastic = true;
      const double revp = nr_rcp(evp);
      double h = m.nB * evpn * revp;
      double gamma = fma(-kSqrt23, Sigv0, normS) * nr_rcp(m.G2 * fma(h, m.rG3, 1.0));
      double xn = evpn;
      // xv^n = evp^n (1 + q)^n with q = (xv - evp) / evp: by the series above from the cached
      // evp^n when |q| <= 2^-6 and n <= 2 (|n ln(1 + q)| <= 2^-5), else exp(n ln xv)
      const bool series = m.n <= 2.0;
      int iteration = 0;
      for (;;) {
        const double xv = RADD(evp, RMUL(kSqrt23, gamma));
        const double q = (xv - evp) * revp;
        if (series && abits(q) <= abits(kSeriesMax))
          xn = evpn * exp_series(m.n * log1p_series(q));
        else
          xn = exp(m.n * log(xv));  // xv^n
        const double Sigv = RADD(m.A, RMUL(m.B, xn));
        h = m.nB * xn * nr_rcp(xv);  // n B xv^(n-1)
        const double dfun = fma(kSqrt23, h, m.dfun0);
        const double fun = fma(dfun, gamma, -fma(h * kSqrt23, gamma, Strial - Sigv));
        if (abs_gt(fun, c_returnTol * Sigv)) {  // |fun / Sigv| > 1e-8, Sigv > 0
          double dgamma = -fun * nr_rcp(dfun);
          // dgamma < 0 && |dgamma| > gamma, with gamma > 0
          if (__double_as_longlong(dgamma) < 0 && abs_gt(dgamma, gamma)) dgamma = -gamma * 0.9;
          gamma += dgamma;
        } else {
          break;
        }
        iteration++;
        if (iteration > c_caps[1]) {
          if (valid) record_error(tm, DNL_ERR_RR_NOCONV, a.eBase + e);
          break;
        }
      }
      const double inv = nr_rcp(normS);  // normS > 0: the trial stress is above A > 0
      tape(TL::GAM, gamma);
      tape(TL::XV, RADD(evp, RMUL(kSqrt23, gamma)));
      tape(TL::XN, xn);
      if (TAPE) tape(TL::LXV, log(RADD(evp, RMUL(kSqrt23, gamma))));
      evp = RADD(evp, RMUL(kSqrt23, gamma));
      evpn = xn;
      const double c2 = m.G2 * gamma;
#pragma unroll
      for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = i; j < 3; j++) {
          if (TWO_D && (i == 2) != (j == 2)) continue;
          const double n1 = S[i][j] * inv;
          S[i][j] = fma(-c2, n1, S[i][j]);
          Epl[i][j] = fma(gamma, n1, Epl[i][j]);
          S[j][i] = S[i][j];
          Epl[j][i] = Epl[i][j];
        }
    }
  }

  // ---- element-mean pressure: sum of the NIP traces in Gauss-point order (Element.C:254, 351)
  double pressure = 0.0;
  {
    const int base = lane - pt;
#pragma unroll
    for (int k = 0; k < NIP; k++) pressure += __shfl_sync(0xffffffffu, trace, base + k);
    pressure = scale2<-ilog2(NIP)>(pressure);  // exact: NIP is a power of two
  }
  const double p = fma(m.K, pressure, a.ip[L::P * nIP + ipx]);

  // ---- RFI: X <- R X R^T for S, Eps, EpsPlas (Element.C:386-388)
  auto rfi = [&](double X[3][3]) {
    if (TWO_D) {
      double Tm[2][2];
#pragma unroll
      for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 2; j++) Tm[i][j] = fma(X[i][0], R[j][0], X[i][1] * R[j][1]);
      const double y00 = fma(R[0][0], Tm[0][0], R[0][1] * Tm[1][0]);
      const double y01 = fma(R[0][0], Tm[0][1], R[0][1] * Tm[1][1]);
      const double y11 = fma(R[1][0], Tm[0][1], R[1][1] * Tm[1][1]);
      X[0][0] = y00;
      X[0][1] = X[1][0] = y01;
      X[1][1] = y11;
      X[2][2] = R[2][2] * (X[2][2] * R[2][2]);
    } else {
      double Tm[3][3];
#pragma unroll
      for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) Tm[i][j] = fma(X[i][0], R[j][0], fma(X[i][1], R[j][1], X[i][2] * R[j][2]));
      double Y[3][3];
#pragma unroll
      for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = i; j < 3; j++) Y[i][j] = fma(R[i][0], Tm[0][j], fma(R[i][1], Tm[1][j], R[i][2] * Tm[2][j]));
#pragma unroll
      for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = i; j < 3; j++) X[i][j] = X[j][i] = Y[i][j];
    }
  };
  rfi(S);
  rfi(Ep);
  {  // a point that never yielded has EpsPlas = 0 exactly, and R 0 R^T = 0
    unsigned long long nz = 0;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = i; j < 3; j++) nz |= abits(Epl[i][j]);
    if (nz) rfi(Epl);
  }

  if (valid) {
    const int I0[6] = {0, 1, 2, 0, 0, 1}, I1[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
    for (int k = 0; k < NS; k++) {
      a.ip[(L::S + k) * nIP + ipx] = S[I0[k]][I1[k]];
      a.ip[(L::EPS + k) * nIP + ipx] = Ep[I0[k]][I1[k]];
      a.ip[(L::EPSP + k) * nIP + ipx] = Epl[I0[k]][I1[k]];
    }
    a.ip[L::P * nIP + ipx] = p;
    if (plastic) {
      a.ip[L::EVP * nIP + ipx] = evp;
      a.ip[L::EVPN * nIP + ipx] = evpn;
    }
    if (a.stepT) {
#pragma unroll
      for (int k = 0; k < 9; k++) {
        a.stepT[k * nIP + ipx] = dE[k / 3][k % 3];
        a.stepT[(9 + k) * nIP + ipx] = R[k / 3][k % 3];
      }
      a.detJ[ipx] = detJ;
    }
  }

  // ---- forces: c_k = dN_k . Sig . W with dN = dN/dxi J^-1, i.e. M = J^-1 Sig W (Element.C:179-212)
  double W = weighted<ET>(detJ);
  double hoop = 0.;
  if (AXI) {
    W = W * (kDeuxPi * Rad);
    hoop = (S[2][2] + p) * (detJ * kDeuxPi);  // sigma_tt / R x W, W = detJ 2 pi R
  }
  double M[DIM][DIM];
#pragma unroll
  for (int l = 0; l < DIM; l++)
#pragma unroll
    for (int i = 0; i < DIM; i++) {
      double s = 0.;
#pragma unroll
      for (int j = 0; j < DIM; j++) {
        const double sig = i == j ? S[j][i] + p : S[j][i];
        s = fma(Ji[l][j], sig, s);
      }
      M[l][i] = s * W;
    }
  if constexpr (NEN == NIP) {
    // lane k assembles node k: Fe_k = -sum over Gauss points q of dN_k(q) . M(q) (+ the hoop
    // term), with every point's M (and hoop) exchanged through the element's shared memory
    constexpr int ST = DIM * DIM + (AXI ? 1 : 0);
    double *mine = red + pt * ST;
#pragma unroll
    for (int l = 0; l < DIM; l++)
#pragma unroll
      for (int i = 0; i < DIM; i++) mine[l * DIM + i] = M[l][i];
    if (AXI) mine[DIM * DIM] = hoop;
    __syncwarp();
    if (valid) {
      // each dN_k(q) (a lane-dependent table lookup) once, for all DIM components
      double s[DIM];
#pragma unroll
      for (int i = 0; i < DIM; i++) s[i] = 0.0;
#pragma unroll
      for (int q = 0; q < NIP; q++) {
        const double *Mq = red + q * ST;
#pragma unroll
        for (int l = 0; l < DIM; l++) {
          const double d = SH::dN(q, pt, l);
#pragma unroll
          for (int i = 0; i < DIM; i++) s[i] = fma(d, Mq[l * DIM + i], s[i]);
        }
        if (AXI) s[0] = fma(SH::N(q, pt), Mq[DIM * DIM], s[0]);
      }
#pragma unroll
      for (int i = 0; i < DIM; i++) a.fe[(long)i * a.feStride + (long)e * NEN + pt] = ineg(s[i]);
    }
  } else {
    double *row = red + pt * (NEN * DIM);
#pragma unroll
    for (int k = 0; k < NEN; k++)
#pragma unroll
      for (int i = 0; i < DIM; i++) {
        double s = 0.;
#pragma unroll
        for (int l = 0; l < DIM; l++) s = fma(SH::dN(pt, k, l), M[l][i], s);
        if (AXI && i == 0) s = fma(SH::N(pt, k), hoop, s);
        row[k * DIM + i] = s;
      }
    if constexpr (ET == DNL_ELHEX8N3D_1PT) {
      // Flanagan-Belytschko viscous hourglass control (Int. J. Numer. Meth. Eng. 17, 1981): the
      // hourglass vectors h_a of the node signs (xi eta, eta zeta, zeta xi, xi eta zeta), made
      // orthogonal to the linear fields, gamma_a = h_a - sum_i (h_a . x_i) b_i with b_i the
      // centre-point gradients; the resisting force f_k = -a_h sum_a gamma_ak (gamma_a . v) with
      // a_h = coefficient rho c V^(2/3) / 4 on the Current velocities, V = 8 detJ.
      double hx[4][3];
#pragma unroll
      for (int q = 0; q < 4; q++)
#pragma unroll
        for (int i = 0; i < 3; i++) hx[q][i] = 0.;
      auto hsign = [](int q, int k) {
        const int sx = sgx(k), sy = sgy(k), sz = sgz(k);
        const int par = q == 0 ? sx ^ sy : (q == 1 ? sy ^ sz : (q == 2 ? sz ^ sx : sx ^ sy ^ sz));
        return q == 3 ? par : !par;  // +1 where the product of the (+-1) signs is +1
      };
#pragma unroll
      for (int k = 0; k < NEN; k++)
#pragma unroll
        for (int i = 0; i < 3; i++) {
          const double xk = a.x[i][node[k]];
#pragma unroll
          for (int q = 0; q < 4; q++) hx[q][i] += hsign(q, k) ? xk : ineg(xk);
        }
      double g[4][NEN], qv[4][3];
#pragma unroll
      for (int q = 0; q < 4; q++)
#pragma unroll
        for (int i = 0; i < 3; i++) qv[q][i] = 0.;
#pragma unroll
      for (int k = 0; k < NEN; k++) {
        double b[3];
#pragma unroll
        for (int i = 0; i < 3; i++) {
          double s = 0.;
#pragma unroll
          for (int l = 0; l < 3; l++) s = fma(Ji[l][i], SH::dN(pt, k, l), s);
          b[i] = s;
        }
        double vk[3];
#pragma unroll
        for (int i = 0; i < 3; i++) vk[i] = a.v[i][node[k]];
#pragma unroll
        for (int q = 0; q < 4; q++) {
          const double gq = fma(-hx[q][2], b[2], fma(-hx[q][1], b[1], fma(-hx[q][0], b[0], hsign(q, k) ? 1. : -1.)));
          g[q][k] = gq;
#pragma unroll
          for (int i = 0; i < 3; i++) qv[q][i] = fma(gq, vk[i], qv[q][i]);
        }
      }
      const double V = weighted<ET>(detJ), cv = cbrt(V);
      const double ah = 0.25 * a.hourglass * m.rho * m.Cs * (cv * cv);
#pragma unroll
      for (int k = 0; k < NEN; k++)
#pragma unroll
        for (int i = 0; i < 3; i++) {
          double s = 0.;
#pragma unroll
          for (int q = 0; q < 4; q++) s = fma(g[q][k], qv[q][i], s);
          row[k * DIM + i] = fma(ah, s, row[k * DIM + i]);
        }
    }
    __syncwarp();
    if (valid) {
      // lane pt assembles nodes pt, pt + NIP, ...: Fe = - sum over Gauss points of the rows
#pragma unroll
      for (int j = 0; j < (NEN + NIP - 1) / NIP; j++) {
        const int k = pt + j * NIP;
        if (k < NEN) {
#pragma unroll
          for (int i = 0; i < DIM; i++) {
            double s = 0.0;
#pragma unroll
            for (int q = 0; q < NIP; q++) s -= red[q * (NEN * DIM) + k * DIM + i];
            a.fe[(long)i * a.feStride + (long)e * NEN + k] = s;
          }
        }
      }
    }
  }
}

template <int ET, bool TAPE = false, bool GENERAL = false>
__global__ void __launch_bounds__(128) k_elem(ElemArgs a)
{
  constexpr int NIP = Elem<ET>::NIP, NEN = Elem<ET>::NEN, DIM = Elem<ET>::DIM;
  constexpr int EPW = 32 / NIP;  // elements per warp
  __shared__ double red[128 / 32][EPW][NIP * NEN * DIM];
  if (a.gate && (a.tm->done | a.tm->status)) return;
  const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
  if ((gtid & ~31) / NIP >= a.E) return;
  const int eRaw = gtid / NIP;
  const bool valid = eRaw < a.E;
  const int lane = threadIdx.x & 31;
  const int e = valid ? eRaw : a.E - 1;
  if (GENERAL && a.elemMat)
    elem_ip<ET, TAPE, true>(a, a.mats[a.elemMat[e]], a.tm, e, gtid % NIP, valid, lane,
                            red[threadIdx.x >> 5][lane / NIP]);
  else
    elem_ip<ET, TAPE, GENERAL>(a, a.mat, a.tm, e, gtid % NIP, valid, lane,
                               red[threadIdx.x >> 5][lane / NIP]);
}

// Batched element pass over the union of many meshes: element e belongs to instance inst[e],
// whose material and time record are mats[inst] and tms[inst]; instances that have finished or
// failed keep their lanes in the warp but store nothing.
template <int ET, int BLOCK, bool TAPE = false>
__global__ void __launch_bounds__(BLOCK) k_elem_batch(ElemArgs a, const int *elemInst,
                                                      const Material *mats, DevTime *tms)
{
  constexpr int NIP = Elem<ET>::NIP, NEN = Elem<ET>::NEN, DIM = Elem<ET>::DIM;
  constexpr int EPW = 32 / NIP;
  __shared__ double red[BLOCK / 32][EPW][NIP * NEN * DIM];
  const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
  if ((gtid & ~31) / NIP >= a.E) return;
  const int eRaw = gtid / NIP;
  const int e = eRaw < a.E ? eRaw : a.E - 1;
  const int inst = elemInst[e];
  DevTime *tm = tms + inst;
  const bool valid = eRaw < a.E && !(tm->done | tm->status);
  const int lane = threadIdx.x & 31;
  elem_ip<ET, TAPE>(a, mats[inst], tm, e, gtid % NIP, valid, lane, red[threadIdx.x >> 5][lane / NIP]);
}

// ----------------------------------------------------------------------------- tangent pass
#include "dnl_sens_elem.cuh"

// ----------------------------------------------------------------------------- adjoint pass
#include "dnl_adj_elem.cuh"

// ----------------------------------------------------------------------------- mass kernel
// Element::computeMassMatrix with the reference's rounding: M_k = sum_pt (rho N_k) W,
// W = weight detJ (2 pi R).  Writes me[e*NEN + k]; Domain::computeMassMatrix's assembly is the
// gather.
template <int ET>
__global__ void __launch_bounds__(128) k_mass(ElemArgs a, double *me, const int *elemInst,
                                              const Material *mats)
{
  using T = Elem<ET>;
  using SH = Shape<ET>;
  constexpr int NIP = T::NIP, NEN = T::NEN, DIM = T::DIM;
  constexpr bool AXI = ET == DNL_ELQUA4NAX;
  constexpr bool TWO_D = DIM == 2;
  constexpr int EPW = 32 / NIP;
  __shared__ double red[128 / 32][EPW][NIP][NEN];
  const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
  if ((gtid & ~31) / NIP >= a.E) return;
  const int eRaw = gtid / NIP;
  const bool valid = eRaw < a.E;
  const int e = valid ? eRaw : a.E - 1;
  const int pt = gtid % NIP;
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, slot = lane / NIP;
  double J[DIM][DIM];
#pragma unroll
  for (int r = 0; r < DIM; r++)
#pragma unroll
    for (int c = 0; c < DIM; c++) J[r][c] = 0.;
  double Rad = 0.;
#pragma unroll
  for (int k = 0; k < NEN; k++) {
    const int nd = a.conn[(long)k * a.E + e];
#pragma unroll
    for (int r = 0; r < DIM; r++) {
      const double xr = a.x[r][nd];
#pragma unroll
      for (int c = 0; c < DIM; c++) J[r][c] = RADD(J[r][c], RMUL(SH::dN(pt, k, c), xr));
    }
    if (AXI) Rad = RADD(Rad, RMUL(SH::N(pt, k), a.x[0][nd]));
  }
  double detJ;
  if (TWO_D) {
    detJ = RSUB(RMUL(J[0][0], J[1][1]), RMUL(J[0][1], J[1][0]));
  } else {
    detJ = RADD(RADD(RMUL(RMUL(J[0][0], J[1][1]), J[2][2]), RMUL(RMUL(J[1][0], J[2][1]), J[0][2])),
                RMUL(RMUL(J[2][0], J[0][1]), J[1][2]));
    detJ = RSUB(detJ, RMUL(RMUL(J[2][0], J[1][1]), J[0][2]));
    detJ = RSUB(detJ, RMUL(RMUL(J[0][0], J[2][1]), J[1][2]));
    detJ = RSUB(detJ, RMUL(RMUL(J[1][0], J[0][1]), J[2][2]));
  }
  double W = weighted<ET>(detJ);
  if (AXI) W = RMUL(W, RMUL(RMUL(2., kPi), Rad));
  const double rho = elemInst ? mats[elemInst[e]].rho : a.mat.rho;
#pragma unroll
  for (int k = 0; k < NEN; k++) red[wib][slot][pt][k] = RMUL(RMUL(rho, SH::N(pt, k)), W);
  __syncwarp();
  if (valid) {
#pragma unroll
    for (int j = 0; j < (NEN + NIP - 1) / NIP; j++) {
      const int k = pt + j * NIP;
      if (k < NEN) {
        double s = 0.;
#pragma unroll
        for (int q = 0; q < NIP; q++) s = RADD(s, red[wib][slot][q][k]);
        me[(long)e * NEN + k] = s;
      }
    }
  }
  (void)lane;
}

// ----------------------------------------------------------------------------- Courant
// The element's characteristic length with the reference's rounding: ElQua4nAx::getLength /
// ElQua4n2D::getLength (ElQua4nAx.C:131-143, ElQua4n2D.C:130-143) for the quads (KIND 0), the
// tetrahedra's shortest corner edge (ElTet4n3D.C:151-166, ElTet10n3D.C:140-155; Vec3D::distance,
// Vec3D.h:380-430, and the Min chain of Math.h:62) (KIND 1); for the one-point hexahedron, which
// is not a reference element, its centre-point volume over its largest face area (KIND 2; each
// face's area half the norm of the cross product of its diagonals).
template <int KIND>
__device__ __forceinline__ double elem_length(const ElemArgs &a, int e)
{
  const int n0 = a.conn[e], n1 = a.conn[a.E + e], n2 = a.conn[2L * a.E + e], n3 = a.conn[3L * a.E + e];
  if constexpr (KIND == 2) {
    double X[8][3];
#pragma unroll
    for (int k = 0; k < 8; k++)
#pragma unroll
      for (int i = 0; i < 3; i++) X[k][i] = a.x[i][a.conn[(long)k * a.E + e]];
    double J[3][3];
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
      for (int c = 0; c < 3; c++) {
        double s = 0.;
#pragma unroll
        for (int k = 0; k < 8; k++) s = fma(Shape<DNL_ELHEX8N3D_1PT>::dN(0, k, c), X[k][r], s);
        J[r][c] = s;
      }
    const double V = 8. * fma(J[0][0], fma(J[1][1], J[2][2], -J[1][2] * J[2][1]),
                              fma(J[0][1], fma(J[1][2], J[2][0], -J[1][0] * J[2][2]),
                                  J[0][2] * fma(J[1][0], J[2][1], -J[1][1] * J[2][0])));
    const int F[6][4] = {{0, 1, 2, 3}, {4, 5, 6, 7}, {0, 1, 5, 4}, {1, 2, 6, 5}, {2, 3, 7, 6}, {3, 0, 4, 7}};
    double a2max = 0.;  // (2 area)^2
#pragma unroll
    for (int f = 0; f < 6; f++) {
      double d1[3], d2[3];
#pragma unroll
      for (int i = 0; i < 3; i++) {
        d1[i] = X[F[f][2]][i] - X[F[f][0]][i];
        d2[i] = X[F[f][3]][i] - X[F[f][1]][i];
      }
      const double c0 = fma(d1[1], d2[2], -d1[2] * d2[1]), c1 = fma(d1[2], d2[0], -d1[0] * d2[2]);
      const double c2 = fma(d1[0], d2[1], -d1[1] * d2[0]);
      a2max = fmax(a2max, fma(c0, c0, fma(c1, c1, c2 * c2)));
    }
    return V / (0.5 * sqrt(a2max));
  } else if constexpr (KIND == 0) {
    const double x31 = RSUB(a.x[0][n2], a.x[0][n0]), x24 = RSUB(a.x[0][n1], a.x[0][n3]);
    const double y42 = RSUB(a.x[1][n3], a.x[1][n1]), y31 = RSUB(a.x[1][n2], a.x[1][n0]);
    const double num = RADD(RMUL(x31, y42), RMUL(x24, y31));
    const double sq = RADD(RADD(RADD(RMUL(x24, x24), RMUL(y42, y42)), RMUL(x31, x31)), RMUL(y31, y31));
    return num / sqrt(RMUL(2., sq));
  } else {
    const int n[4] = {n0, n1, n2, n3};
    const int ea[6] = {0, 0, 1, 0, 1, 2}, eb[6] = {1, 2, 2, 3, 3, 3};
    double ll = 0.;
#pragma unroll
    for (int m = 0; m < 6; m++) {
      double q = 0.;
#pragma unroll
      for (int c = 0; c < 3; c++) {
        const double d = RSUB(a.x[c][n[eb[m]]], a.x[c][n[ea[m]]]);
        q = c == 0 ? RMUL(d, d) : RADD(q, RMUL(d, d));
      }
      const double l = sqrt(q);
      ll = m == 0 ? l : (ll < l ? ll : l);
    }
    return ll;
  }
}

// Min over elements via an unsigned atomicMin on the bit pattern (positive doubles order like
// their bits).  A non-positive or NaN length is an error: the reference would turn it into a
// negative or NaN time step.
template <int KIND>
__global__ void __launch_bounds__(256) k_courant(ElemArgs a)
{
  if (a.tm->done | a.tm->status) return;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  double len = 1e300;
  if (e < a.E) {
    len = elem_length<KIND>(a, e);
    if (!(len > 0.)) {
      record_error(a.tm, DNL_ERR_DT, a.eBase + e);
      len = 1e300;
    } else if (a.elemCs) {
      len = len / a.elemCs[e];  // several materials: the critical time of this element
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) len = fmin(len, __shfl_xor_sync(0xffffffffu, len, o));
  __shared__ double wmin[8];
  if ((threadIdx.x & 31) == 0) wmin[threadIdx.x >> 5] = len;
  __syncthreads();
  if (threadIdx.x == 0) {
    double b = wmin[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); w++) b = fmin(b, wmin[w]);
    atomicMin(&a.tm->lenMinBits, (unsigned long long)__double_as_longlong(b));
  }
}

// Batched Courant lengths: each element folds its length into its instance's minimum; a warp whose
// lanes all belong to one instance reduces first and issues one atomic.
template <int KIND>
__global__ void __launch_bounds__(256) k_courant_batch(ElemArgs a, const int *elemInst, DevTime *tms)
{
  const int eRaw = blockIdx.x * blockDim.x + threadIdx.x;
  if ((eRaw & ~31) >= a.E) return;
  const int e = eRaw < a.E ? eRaw : a.E - 1;
  const int inst = elemInst[e];
  DevTime *tm = tms + inst;
  double len = 1e300;
  if (eRaw < a.E && !(tm->done | tm->status)) {
    len = elem_length<KIND>(a, e);
    if (!(len > 0.)) {
      record_error(tm, DNL_ERR_DT, e);
      len = 1e300;
    }
  }
  const int first = __shfl_sync(0xffffffffu, inst, 0);
  if (__all_sync(0xffffffffu, inst == first)) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) len = fmin(len, __shfl_xor_sync(0xffffffffu, len, o));
    if ((threadIdx.x & 31) == 0 && len < 1e300)
      atomicMin(&tm->lenMinBits, (unsigned long long)__double_as_longlong(len));
  } else if (len < 1e300) {
    atomicMin(&tm->lenMinBits, (unsigned long long)__double_as_longlong(len));
  }
}

// ----------------------------------------------------------------------------- persistent batch step
// Grid-wide barrier of a cooperative launch (every block resident): thread 0 of each block arrives
// on a counter; the last arrival resets it and advances the generation the others wait on.  The
// wait is bounded: past kBarrierSpins polls it sets *err and gives up, and every block leaves the
// kernel at its next barrier.  Fences order each phase's global writes before the next phase.
constexpr long long kBarrierSpins = 1ll << 25;

__device__ __forceinline__ bool grid_barrier(unsigned *bar, int *err)
{
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned *gen = bar + 1;
    const unsigned g = *gen;
    __threadfence();
    if (atomicAdd(bar, 1u) + 1u == gridDim.x) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      long long spins = 0;
      while (*gen == g) {
        if (++spins > kBarrierSpins) {
          atomicExch(err, 1);
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return *(volatile int *)err == 0;
}

template <int ET, int BLOCK>
__global__ void __launch_bounds__(BLOCK) k_batch_persistent(BatchStepArgs a)
{
  constexpr int NIP = Elem<ET>::NIP, NEN = Elem<ET>::NEN, DIM = Elem<ET>::DIM;
  constexpr int EPW = 32 / NIP;
  __shared__ double red[BLOCK / 32][EPW][NIP * NEN * DIM];
  const int tid = blockIdx.x * BLOCK + threadIdx.x, nthreads = gridDim.x * BLOCK;
  // ---- time logic: initStep of every unfinished instance
  if (a.preFirst) {
    for (int i = tid; i < a.count; i += nthreads) {
      const InstParams &p = a.prm[i];
      dt_update(a.tms + i, DT_PRE, p.freq, p.method, p.safetyOmega, p.Cs);
    }
    if (!grid_barrier(a.bar, a.err)) return;
  }
  // ---- constant boundary conditions on the Current field (k_bc_current)
  for (int i = tid; i < a.nbc; i += nthreads) {
    const int n = a.bcNodes[i];
    const DevTime *tm = a.tms + a.nodeInst[n];
    if (tm->done | tm->status) continue;
    const double dt = tm->timeStep;
    const int cd = a.na.bcCode[i];
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const int act = (cd >> (2 * c)) & 3;
      if (act == 1) {
        a.cur.du[c][n] = 0.;
        a.cur.v[c][n] = 0.;
        a.cur.a[c][n] = 0.;
      } else if (act == 2) {
        const double sp = a.na.bcSpeed[3 * i + c];
        a.cur.a[c][n] = 0.;
        a.cur.v[c][n] = sp;
        a.cur.du[c][n] = __dmul_rn(sp, dt);
      }
    }
  }
  if (!grid_barrier(a.bar, a.err)) return;
  // ---- element pass: warp-aligned tiles of Gauss points, grid-stride (as k_elem_batch)
  {
    const long total = ((long)a.ea.E * NIP + 31) & ~31L;
    const int lane = threadIdx.x & 31;
    for (long base = (long)blockIdx.x * BLOCK; base < total; base += (long)gridDim.x * BLOCK) {
      const long gtid = base + threadIdx.x;
      if ((gtid & ~31L) / NIP >= a.ea.E) continue;  // the whole warp
      const int eRaw = (int)(gtid / NIP);
      const int e = eRaw < a.ea.E ? eRaw : a.ea.E - 1;
      const int inst = a.elemInst[e];
      DevTime *tm = a.tms + inst;
      const bool valid = eRaw < a.ea.E && !(tm->done | tm->status);
      elem_ip<ET>(a.ea, a.mats[inst], tm, e, (int)(gtid % NIP), valid, lane,
                  red[threadIdx.x >> 5][lane / NIP]);
      __syncwarp();
    }
  }
  if (!grid_barrier(a.bar, a.err)) return;
  // ---- assembly + nodal update (k_node_batch)
  for (int n = tid; n < a.na.N; n += nthreads) {
    const int i = a.nodeInst[n];
    const DevTime *tm = a.tms + i;
    if (tm->done | tm->status) continue;
    node_update<DIM>(a.na, n, tm->timeStep, a.prm[i].alphaM, a.prm[i].beta, a.prm[i].gamma);
  }
  if (!grid_barrier(a.bar, a.err)) return;
  // ---- Courant lengths of the updated mesh into each instance's minimum (k_courant_batch)
  if (a.courant) {
    for (int base = blockIdx.x * BLOCK; base < ((a.ea.E + 31) & ~31); base += gridDim.x * BLOCK) {
      const int eRaw = base + threadIdx.x;
      if ((eRaw & ~31) >= a.ea.E) continue;
      const int e = eRaw < a.ea.E ? eRaw : a.ea.E - 1;
      const int inst = a.elemInst[e];
      DevTime *tm = a.tms + inst;
      double len = 1e300;
      if (eRaw < a.ea.E && !(tm->done | tm->status)) {
        len = elem_length<etype_length_kind(ET)>(a.ea, e);
        if (!(len > 0.)) {
          record_error(tm, DNL_ERR_DT, e);
          len = 1e300;
        }
      }
      const int first = __shfl_sync(0xffffffffu, inst, 0);
      if (__all_sync(0xffffffffu, inst == first)) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) len = fmin(len, __shfl_xor_sync(0xffffffffu, len, o));
        if ((threadIdx.x & 31) == 0 && len < 1e300)
          atomicMin(&tm->lenMinBits, (unsigned long long)__double_as_longlong(len));
      } else if (len < 1e300) {
        atomicMin(&tm->lenMinBits, (unsigned long long)__double_as_longlong(len));
      }
    }
    if (!grid_barrier(a.bar, a.err)) return;
  }
  // ---- time logic: updateTime, the time step (recomputed when due), initStep of the next step
  for (int i = tid; i < a.count; i += nthreads) {
    const InstParams &p = a.prm[i];
    dt_update(a.tms + i, a.postMode, p.freq, p.method, p.safetyOmega, p.Cs);
  }
}

int launch_batch_persistent(int etype, int block, const BatchStepArgs &a, cudaStream_t s)
{
  if (etype != DNL_ELQUA4NAX) return DNL_ERR_ARG;  // the batched stepping's element type
  void *fn;
  if (block == 64)
    fn = (void *)k_batch_persistent<DNL_ELQUA4NAX, 64>;
  else if (block == 256)
    fn = (void *)k_batch_persistent<DNL_ELQUA4NAX, 256>;
  else {
    block = 128;
    fn = (void *)k_batch_persistent<DNL_ELQUA4NAX, 128>;
  }
  int dev = 0, sms = 0, per = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return DNL_ERR_CUDA;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return DNL_ERR_CUDA;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, block, 0) != cudaSuccess || per < 1)
    return DNL_ERR_CUDA;
  // no more blocks than the element pass has tiles
  const long tiles = ((long)a.ea.E * etype_nip(etype) + block - 1) / block;
  int grid = sms * per;
  if (grid > tiles) grid = (int)tiles;
  if (grid < 1) grid = 1;
  BatchStepArgs args = a;
  void *params[] = {&args};
  const cudaError_t e = cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(block), params, 0, s);
  launch_counter()++;
  return e == cudaSuccess ? 0 : DNL_ERR_CUDA;
}

// ----------------------------------------------------------------------------- launchers
static ElemArgs elem_args(dnl_handle *h)
{
  ElemArgs a;
  memset(&a, 0, sizeof a);
  a.E = h->E;
  a.N = h->N;
  a.conn = h->conn;
  for (int r = 0; r < 3; r++) {
    a.x[r] = h->x[r];
    a.du[r] = h->bank[h->cur].du[r];
  }
  for (int r = 0; r < 3; r++) a.v[r] = h->bank[h->cur].v[r];
  a.hourglass = h->hourglass;
  a.ip = h->ip;
  a.fe = h->fe;
  a.feStride = h->EN;
  a.detJ = h->detJ;
  a.stepT = h->stepT;
  a.tm = h->tm;
  a.mat = h->mat;
  a.elemMat = h->elemMat;
  a.mats = h->dmats;
  a.elemCs = h->elemCs;
  a.gate = 1;
  return a;
}

// the element arguments of a further element group g: its connectivity, integration points and
// slots of the handle's element-force array (one material; no step tensors)
static ElemArgs group_args(dnl_handle *h, const ElemGroup &g)
{
  ElemArgs a = elem_args(h);
  a.E = g.E;
  a.conn = g.conn;
  a.ip = g.ip;
  a.fe = h->fe + g.feOff;
  a.detJ = g.detJ;
  a.stepT = g.stepT;
  a.elemMat = h->elemMat ? h->elemMat + g.eOff : nullptr;  // several materials: over all groups
  a.mats = h->elemMat ? h->dmats : nullptr;
  a.elemCs = g.Cs;
  a.eBase = g.eOff;
  return a;
}

int launch_elem(dnl_handle *h, cudaStream_t s, int gate)
{
  ElemArgs a = elem_args(h);
  a.gate = gate;
  const long threads = (long)h->E * h->nip;
  const int grid = (int)((threads + 127) / 128);
  prof_begin(h, s);
  const bool general = h->elemMat || h->mat.hard.law != DNL_HARD_POWER;
  if (general)
    DNL_BY_ETYPE(h->etype, (k_elem<ET, false, true><<<grid, 128, 0, s>>>(a)));
  else
    DNL_BY_ETYPE(h->etype, (k_elem<ET><<<grid, 128, 0, s>>>(a)));
  launch_counter()++;
  // further element groups: same pass, their own element type (one material: the power law or
  // the general instance as above)
  for (int gi = 0; gi < h->nextra; gi++) {
    const ElemGroup &g = h->extra[gi];
    ElemArgs b = group_args(h, g);
    b.gate = gate;
    const int gg = (int)(((long)g.E * g.nip + 127) / 128);
    if (general)
      DNL_BY_ETYPE(g.etype, (k_elem<ET, false, true><<<gg, 128, 0, s>>>(b)));
    else
      DNL_BY_ETYPE(g.etype, (k_elem<ET><<<gg, 128, 0, s>>>(b)));
    launch_counter()++;
  }
  prof_end(h, DNL_PROF_ELEM, s);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : DNL_ERR_CUDA;
}

// the element pass with its per-integration-point record (forward-mode sensitivities, the
// adjoint's recomputation): each element group's record is the block at tape + NT ipOff of the
// [NT][points] record (one layout width NT per dimension)
int launch_elem_tape(dnl_handle *h, cudaStream_t s, double *tape)
{
  if (!etype_has_sens(h->etype)) return DNL_ERR_ARG;
  prof_begin(h, s);
  for (int gi = -1; gi < h->nextra; gi++) {
    ElemArgs a = gi < 0 ? elem_args(h) : group_args(h, h->extra[gi]);
    const int et = gi < 0 ? h->etype : h->extra[gi].etype;
    a.gate = 1;
    a.tape = tape + (gi < 0 ? 0 : (long)TapeLayout<DNL_ELHEX8N3D>::NT * h->extra[gi].ipOff);
    const long threads = (long)a.E * etype_nip(et);
    const int grid = (int)((threads + 127) / 128);
    DNL_BY_ETYPE(et, (k_elem<ET, true><<<grid, 128, 0, s>>>(a)));
    launch_counter()++;
  }
  prof_end(h, DNL_PROF_ELEM, s);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : DNL_ERR_CUDA;
}

int launch_elem_raw(int etype, const ElemArgs &a, cudaStream_t s)
{
  const long threads = (long)a.E * etype_nip(etype);
  const int grid = (int)((threads + 127) / 128);
  DNL_BY_ETYPE(etype, (k_elem<ET><<<grid, 128, 0, s>>>(a)));
  launch_counter()++;
  return cudaPeekAtLastError() == cudaSuccess ? 0 : DNL_ERR_CUDA;
}

int launch_mass(dnl_handle *h, cudaStream_t s, double *me)
{
  ElemArgs a = elem_args(h);
  const long threads = (long)h->E * h->nip;
  const int grid = (int)((threads + 127) / 128);
  DNL_BY_ETYPE(h->etype, (k_mass<ET><<<grid, 128, 0, s>>>(a, me, h->elemMat, h->dmats)));
  launch_counter()++;
  for (int gi = 0; gi < h->nextra; gi++) {
    const ElemGroup &g = h->extra[gi];
    ElemArgs b = group_args(h, g);
    const int gg = (int)(((long)g.E * g.nip + 127) / 128);
    DNL_BY_ETYPE(g.etype, (k_mass<ET><<<gg, 128, 0, s>>>(b, me + g.feOff, b.elemMat, b.mats)));
    launch_counter()++;
  }
  return cudaPeekAtLastError() == cudaSuccess ? 0 : DNL_ERR_CUDA;
}

int launch_elem_batch(int etype, int block, const ElemArgs &a, const int *elemInst,
                      const Material *mats, DevTime *tms, cudaStream_t s)
{
  // the hexahedra's and the 10-node tetrahedron's shared-memory transpose fits 128 threads at most
  if ((etype == DNL_ELHEX8N3D || etype == DNL_ELTET10N3D || etype == DNL_ELHEX8N3D_1PT) && block > 128)
    block = 128;
  const long threads = (long)a.E * etype_nip(etype);
  const int grid = (int)((threads + block - 1) / block);
#define DNL_EB(ET, B) k_elem_batch<ET, B><<<grid, B, 0, s>>>(a, elemInst, mats, tms)
  if (etype == DNL_ELHEX8N3D_1PT) {
    if (block == 64) DNL_EB(DNL_ELHEX8N3D_1PT, 64);
    else DNL_EB(DNL_ELHEX8N3D_1PT, 128);
  } else if (etype == DNL_ELTET4N3D) {
    if (block == 64) DNL_EB(DNL_ELTET4N3D, 64);
    else if (block == 256) DNL_EB(DNL_ELTET4N3D, 256);
    else DNL_EB(DNL_ELTET4N3D, 128);
  } else if (etype == DNL_ELTET10N3D) {
    if (block == 64) DNL_EB(DNL_ELTET10N3D, 64);
    else DNL_EB(DNL_ELTET10N3D, 128);
  } else if (etype != DNL_ELHEX8N3D) {
    if (etype == DNL_ELQUA4N2D) {
      if (block == 64) DNL_EB(DNL_ELQUA4N2D, 64);
      else if (block == 256) DNL_EB(DNL_ELQUA4N2D, 256);
      else DNL_EB(DNL_ELQUA4N2D, 128);
    } else if (block == 64) DNL_EB(DNL_ELQUA4NAX, 64);
    else if (block == 256) DNL_EB(DNL_ELQUA4NAX, 256);
    else DNL_EB(DNL_ELQUA4NAX, 128);
  } else {
    if (block == 64) DNL_EB(DNL_ELHEX8N3D, 64);
    else DNL_EB(DNL_ELHEX8N3D, 128);
  }
#undef DNL_EB
  launch_counter()++;
  return cudaPeekAtLastError() == cudaSuccess ? 0 : DNL_ERR_CUDA;
}

// batched element pass with its per-integration-point record (batched sensitivities)
int launch_elem_batch_tape(int etype, const ElemArgs &a, const int *elemInst, const Material *mats,
                           DevTime *tms, cudaStream_t s)
{
  if (!etype_has_sens(etype)) return DNL_ERR_ARG;
  const long threads = (long)a.E * etype_nip(etype);
  const int grid = (int)((threads + 127) / 128);
  DNL_BY_ETYPE(etype, (k_elem_batch<ET, 128, true><<<grid, 128, 0, s>>>(a, elemInst, mats, tms)));
  launch_counter()++;
  return cudaPeekAtLastError() == cudaSuccess ? 0 : DNL_ERR_CUDA;
}

int launch_mass_batch(int etype, const ElemArgs &a, double *me, const int *elemInst,
                      const Material *mats, cudaStream_t s)
{
  const long threads = (long)a.E * etype_nip(etype);
  const int grid = (int)((threads + 127) / 128);
  DNL_BY_ETYPE(etype, (k_mass<ET><<<grid, 128, 0, s>>>(a, me, elemInst, mats)));
  launch_counter()++;
  return cudaPeekAtLastError() == cudaSuccess ? 0 : DNL_ERR_CUDA;
}

int launch_courant_batch(int etype, const ElemArgs &a, const int *elemInst, DevTime *tms,
                         cudaStream_t s)
{
  const int kind = etype_length_kind(etype), grid = (a.E + 255) / 256;
  if (kind == 0)
    k_courant_batch<0><<<grid, 256, 0, s>>>(a, elemInst, tms);
  else if (kind == 1)
    k_courant_batch<1><<<grid, 256, 0, s>>>(a, elemInst, tms);
  else
    k_courant_batch<2><<<grid, 256, 0, s>>>(a, elemInst, tms);
  launch_counter()++;
  return cudaPeekAtLastError() == cudaSuccess ? 0 : DNL_ERR_CUDA;
}

ElemArgs elem_args_of(dnl_handle *h) { return elem_args(h); }
ElemArgs group_args_of(dnl_handle *h, int gi) { return gi < 0 ? elem_args(h) : group_args(h, h->extra[gi]); }

int launch_courant(dnl_handle *h, cudaStream_t s)
{
  prof_begin(h, s);
  // every element group's lengths into the one minimum (its kernels reduce into the time record)
  for (int gi = -1; gi < h->nextra; gi++) {
    const ElemArgs a = gi < 0 ? elem_args(h) : group_args(h, h->extra[gi]);
    const int et = gi < 0 ? h->etype : h->extra[gi].etype;
    const int kind = etype_length_kind(et), grid = (a.E + 255) / 256;
    if (kind == 0)
      k_courant<0><<<grid, 256, 0, s>>>(a);
    else if (kind == 1)
      k_courant<1><<<grid, 256, 0, s>>>(a);
    else
      k_courant<2><<<grid, 256, 0, s>>>(a);
    launch_counter()++;
  }
  prof_end(h, DNL_PROF_COURANT, s);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : DNL_ERR_CUDA;
}

}  // namespace dnl
