/* Forward-mode sensitivities of the explicit Chung-Hulbert run -- ORACLE (test infrastructure).
 *
 * Only tests and bench.py's CPU-baseline leg load this library, as the checker of the GPU
 * sensitivities (libdnlgpu.so's dnl_sens_* entry points) and as their timed CPU baseline.
 *
 * What it computes: the final nodal coordinates x(T) of a run with a prescribed step-size
 * schedule and their derivatives with respect to the four parameters (A, B, n) of the hardening
 * law sigma_y = A + B evp^n (IsoHardElastoplastic.C:171-184) and the magnitude s of the initial
 * velocity v0 = s u (BoundarySpeed::applyInitial_V0, Boundary.C:378-385).
 *
 * How: FP64 dual numbers (a value and four tangents) carried through the same restatement of the
 * step as dnl_oracle.c -- the Jacobian and its LAPACK-order inverse (Element2D.C:53-126,
 * Element3D.C:53-113, Matrix.C:1653-1700), F of the Current field (ElementAx.C:114-136,
 * Element3D.C:182-205), the stress update and the J2 radial return with its Newton iterations
 * (Element.C:217-403), RFI, B^T sigma (Element.C:164-214), the assembly, and the Chung-Hulbert
 * predictor/corrector with its boundary conditions (ExplicitSolverCH.C:387-567, Boundary.C) -- so
 * the value parts repeat dnl_oracle.c's arithmetic operation for operation.  One exception: the
 * Jacobi polar decomposition (Tensor2.C:1154-1259) stops at |C_pq| < 1e-9, and dual numbers pushed
 * through its rotations would drop the tangents of the off-diagonal terms left below that
 * threshold; there the tangents use the derivative of the exact spectral functions at the computed
 * eigenpairs, d f(C) = V (F o (V^T dC V)) V^T with F_ij the divided differences of
 * f = ln(sqrt(.)) and f = 1/sqrt(.) (Daleckii-Krein).  The time step is the caller's schedule (a
 * parameter-independent dt sequence), so no Courant or Pulse step enters the derivative. */
#include "tet10_tables.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

namespace {

constexpr int NP = 4;  // A, B, n, v0 magnitude

struct D {
  double v;
  double d[NP];
};

inline D cst(double v)
{
  D r;
  r.v = v;
  for (int k = 0; k < NP; k++) r.d[k] = 0.;
  return r;
}
inline D operator+(const D &a, const D &b)
{
  D r;
  r.v = a.v + b.v;
  for (int k = 0; k < NP; k++) r.d[k] = a.d[k] + b.d[k];
  return r;
}
inline D operator-(const D &a, const D &b)
{
  D r;
  r.v = a.v - b.v;
  for (int k = 0; k < NP; k++) r.d[k] = a.d[k] - b.d[k];
  return r;
}
inline D operator-(const D &a)
{
  D r;
  r.v = -a.v;
  for (int k = 0; k < NP; k++) r.d[k] = -a.d[k];
  return r;
}
inline D operator*(const D &a, const D &b)
{
  D r;
  r.v = a.v * b.v;
  for (int k = 0; k < NP; k++) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
  return r;
}
inline D operator/(const D &a, const D &b)
{
  D r;
  r.v = a.v / b.v;
  for (int k = 0; k < NP; k++) r.d[k] = (a.d[k] - r.v * b.d[k]) / b.v;
  return r;
}
inline D operator*(double a, const D &b)
{
  D r;
  r.v = a * b.v;
  for (int k = 0; k < NP; k++) r.d[k] = a * b.d[k];
  return r;
}
inline D operator*(const D &a, double b) { return b * a; }
inline D operator/(const D &a, double b)
{
  D r;
  r.v = a.v / b;
  for (int k = 0; k < NP; k++) r.d[k] = a.d[k] / b;
  return r;
}
inline D operator+(const D &a, double b)
{
  D r = a;
  r.v = a.v + b;
  return r;
}
inline D operator+(double a, const D &b) { return b + a; }
inline D operator-(const D &a, double b)
{
  D r = a;
  r.v = a.v - b;
  return r;
}
inline D operator-(double a, const D &b)
{
  D r = -b;
  r.v = a - b.v;
  return r;
}
inline D &operator+=(D &a, const D &b) { return a = a + b; }
inline D &operator-=(D &a, const D &b) { return a = a - b; }
inline D &operator*=(D &a, const D &b) { return a = a * b; }
inline D &operator/=(D &a, const D &b) { return a = a / b; }
inline D dsqrt(const D &a)
{
  D r;
  r.v = sqrt(a.v);
  for (int k = 0; k < NP; k++) r.d[k] = a.d[k] / (2. * r.v);
  return r;
}
inline D dcbrt(const D &a)
{
  D r;
  r.v = cbrt(a.v);
  const double s = 1.0 / (3.0 * r.v * r.v);
  for (int k = 0; k < NP; k++) r.d[k] = a.d[k] * s;
  return r;
}
// x^n for x > 0: value pow(x, n); d = n x^(n-1) dx + x^n ln(x) dn
inline D dpow(const D &x, const D &n)
{
  D r;
  r.v = pow(x.v, n.v);
  const double dx = n.v * pow(x.v, n.v - 1.), dn = r.v * log(x.v);
  for (int k = 0; k < NP; k++) r.d[k] = dx * x.d[k] + dn * n.d[k];
  return r;
}
inline double ABSV(const D &a) { return a.v < 0 ? -a.v : a.v; }

constexpr double SQRT23 = 0.8164965809277260327324280249019;
constexpr double SQRT32 = 1.2247448713915890490986420373529;
constexpr double DEUXPI = 6.283185307179586476925286766559;
constexpr double PRECISION_POLAR = 10.0E-10;
constexpr double RR_PRECISION = 1.0E-8;
constexpr int RR_MAXIT = 2000;

const int AX_XI[4] = {-1, 1, 1, -1}, AX_ETA[4] = {-1, -1, 1, 1};
const int HX_XI[8] = {-1, 1, 1, -1, -1, 1, 1, -1};
const int HX_ETA[8] = {-1, -1, 1, 1, -1, -1, 1, 1};
const int HX_ZETA[8] = {-1, -1, -1, -1, 1, 1, 1, 1};

}  // namespace

struct dnls {
  int etype, dim, nen, nip;
  long N, E;
  std::vector<long> conn;
  std::vector<D> coords;   // (N, 3)
  std::vector<D> fld[2][4];  // [NodalField][delta_disp, mat_speed, dmat_speed, disp], (N, 3)
  int cur;
  std::vector<double> mass;  // per node (constant in the parameters)
  std::vector<D> fint, fe;
  std::vector<D> S, Eps, EpsPlas, Sig, p, evp, detJ, dN;
  double young, nu;
  D A, B, n;
  std::vector<long> bcn_start, n2e_start, n2e;
  std::vector<int> bcn_kind;
  std::vector<double> bcn_val;
  double alphaM, beta, gamma, timeStep;
  double Nt[8][10], dNxi[8][10][3], weight[8];
  double rho, hourglass;  // the one-point hexahedron's hourglass force
  int err;
};

namespace {

#define IPX(h, e, pt) ((long)(e) * (h)->nip + (pt))
#define DNS(h, e, pt, k, c) (h)->dN[(IPX(h, e, pt) * (h)->nen + (k)) * 3 + (c)]

void build_tables(dnls *h)
{
  if (h->etype == 5) {  // the one-point hexahedron (not a reference element): the cube's centre
    h->weight[0] = 8.0;
    for (int k = 0; k < 8; k++) {
      h->Nt[0][k] = 0.125;
      h->dNxi[0][k][0] = HX_XI[k] * 0.125;
      h->dNxi[0][k][1] = HX_ETA[k] * 0.125;
      h->dNxi[0][k][2] = HX_ZETA[k] * 0.125;
    }
  } else if (h->etype == 3) {  // ElTet4n3D (ElTet4n3D.C:33-57): one point, weight 1/6
    h->weight[0] = 1. / 6.;
    for (int k = 0; k < 4; k++) {
      h->Nt[0][k] = 0.25;
      for (int c = 0; c < 3; c++) h->dNxi[0][k][c] = k == 0 ? -1.0 : (k - 1 == c ? 1.0 : 0.0);
    }
  } else if (h->etype == 4) {  // ElTet10n3D (ElTet10n3D.C:45-72), as the compiled reference holds it
    dnl_tet10_tables(h->Nt, h->dNxi, h->weight);
  } else if (h->etype != 1) {  // ElQua4nAx and ElQua4n2D share their tables
    const double cN[3] = {(2.0 + sqrt(3.0)) / 6.0, 1.0 / 6.0, (2.0 - sqrt(3.0)) / 6.0};
    const double cD[2] = {(3.0 + sqrt(3.0)) / 12.0, (3.0 - sqrt(3.0)) / 12.0};
    for (int pt = 0; pt < 4; pt++) {
      h->weight[pt] = 1;
      for (int k = 0; k < 4; k++) {
        int dx = AX_XI[k] != AX_XI[pt], dy = AX_ETA[k] != AX_ETA[pt];
        h->Nt[pt][k] = cN[dx + dy];
        h->dNxi[pt][k][0] = AX_XI[k] > 0 ? cD[dy] : -cD[dy];
        h->dNxi[pt][k][1] = AX_ETA[k] > 0 ? cD[dx] : -cD[dx];
        h->dNxi[pt][k][2] = 0;
      }
    }
  } else {
    const double cN[4] = {(9.0 + 5.0 * sqrt(3.0)) / 36.0, (3.0 + sqrt(3.0)) / 36.0,
                          (3.0 - sqrt(3.0)) / 36.0, (9.0 - 5.0 * sqrt(3.0)) / 36.0};
    const double cD[3] = {(2.0 + sqrt(3.0)) / 12.0, 1.0 / 12.0, (2.0 - sqrt(3.0)) / 12.0};
    for (int pt = 0; pt < 8; pt++) {
      h->weight[pt] = 1;
      for (int k = 0; k < 8; k++) {
        int dx = HX_XI[k] != HX_XI[pt], dy = HX_ETA[k] != HX_ETA[pt], dz = HX_ZETA[k] != HX_ZETA[pt];
        h->Nt[pt][k] = cN[dx + dy + dz];
        h->dNxi[pt][k][0] = HX_XI[k] > 0 ? cD[dy + dz] : -cD[dy + dz];
        h->dNxi[pt][k][1] = HX_ETA[k] > 0 ? cD[dx + dz] : -cD[dx + dz];
        h->dNxi[pt][k][2] = HX_ZETA[k] > 0 ? cD[dx + dy] : -cD[dx + dy];
      }
    }
  }
}

// Tensor2 arithmetic, row-major v[i*3+j]
void t2_mul(const D *a, const D *b, D *c)
{
  D t[9];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      D s = cst(0.);
      for (int k = 0; k < 3; k++) s += a[i * 3 + k] * b[k * 3 + j];
      t[i * 3 + j] = s;
    }
  for (int k = 0; k < 9; k++) c[k] = t[k];
}
void t2_transpose(const D *a, D *t)
{
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) t[j * 3 + i] = a[i * 3 + j];
}
void t2_identity(D *t)
{
  for (int k = 0; k < 9; k++) t[k] = cst(0.);
  t[0] = t[4] = t[8] = cst(1.);
}
void t2_rotate(const D *R, D *X)
{
  D Rt[9], tmp[9];
  t2_transpose(R, Rt);
  t2_mul(X, Rt, tmp);
  t2_mul(R, tmp, X);
}

/* Tensor2::polarDecomposeLnU (Tensor2.C:1154-1259) on the values, as in dnl_oracle.c; tangents
 * from the spectral derivative at the computed eigenpairs (C = V diag(l) V^T):
 *   d ln U  = V (G o (V^T dC V)) V^T,  G_ij = (ln l_i - ln l_j) / (2 (l_i - l_j)),  G_ii = 1/(2 l_i)
 *   d U^-1  = V (H o (V^T dC V)) V^T,  H_ij = -1 / (sqrt(l_i) sqrt(l_j) (sqrt(l_i) + sqrt(l_j)))
 *   dR      = dF U^-1 + F dU^-1. */
int polar_ln_u(const D *Fd, D *Ud, D *Rd)
{
  double F[9], FF[9], Rot[9], Rr[9], Ut[9], Ft[9];
  for (int k = 0; k < 9; k++) F[k] = Fd[k].v;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) Ft[j * 3 + i] = F[i * 3 + j];
  auto mul = [](const double *a, const double *b, double *c) {
    double t[9];
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) {
        double s = 0;
        for (int k = 0; k < 3; k++) s += a[i * 3 + k] * b[k * 3 + j];
        t[i * 3 + j] = s;
      }
    memcpy(c, t, sizeof t);
  };
  auto ident = [](double *t) {
    memset(t, 0, 9 * sizeof(double));
    t[0] = t[4] = t[8] = 1.;
  };
  mul(Ft, F, FF);
  ident(Rot);
  int it = 1;
  bool conv = false;
  while (it < 30) {
    int q = (fabs(FF[1]) > fabs(FF[2]) ? 1 : 2);
    int p = (fabs(FF[q]) > fabs(FF[5]) ? 0 : 1);
    if (p == 1) q = 2;
    if (fabs(FF[p * 3 + q]) < PRECISION_POLAR) {
      conv = true;
      break;
    }
    const double alpha = (FF[q * 3 + q] - FF[p * 3 + p]) / (2. * FF[p * 3 + q]);
    const double t = (alpha != 0. ? 1. / (alpha + sqrt(alpha * alpha + 1.) * (alpha > 0. ? 1. : -1.)) : 1.);
    const double Ct = 1. / (sqrt(1. + t * t));
    const double St = t * Ct;
    ident(Rr);
    Rr[p * 3 + q] = St;
    Rr[q * 3 + p] = -St;
    Rr[p * 3 + p] = Rr[q * 3 + q] = Ct;
    const double *r = Rr;
    Ut[0] = r[0] * (FF[0] * r[0] + FF[3] * r[3] + FF[6] * r[6]) +
            r[3] * (FF[1] * r[0] + FF[4] * r[3] + FF[7] * r[6]) +
            r[6] * (FF[2] * r[0] + FF[5] * r[3] + FF[8] * r[6]);
    Ut[1] = r[1] * (FF[0] * r[0] + FF[3] * r[3] + FF[6] * r[6]) +
            r[4] * (FF[1] * r[0] + FF[4] * r[3] + FF[7] * r[6]) +
            (FF[2] * r[0] + FF[5] * r[3] + FF[8] * r[6]) * r[7];
    Ut[2] = r[2] * (FF[0] * r[0] + FF[3] * r[3] + FF[6] * r[6]) +
            r[5] * (FF[1] * r[0] + FF[4] * r[3] + FF[7] * r[6]) +
            (FF[2] * r[0] + FF[5] * r[3] + FF[8] * r[6]) * r[8];
    Ut[4] = r[1] * (FF[0] * r[1] + FF[3] * r[4] + FF[6] * r[7]) +
            r[4] * (FF[1] * r[1] + FF[4] * r[4] + FF[7] * r[7]) +
            r[7] * (FF[2] * r[1] + FF[5] * r[4] + FF[8] * r[7]);
    Ut[5] = r[2] * (FF[0] * r[1] + FF[3] * r[4] + FF[6] * r[7]) +
            r[5] * (FF[1] * r[1] + FF[4] * r[4] + FF[7] * r[7]) +
            (FF[2] * r[1] + FF[5] * r[4] + FF[8] * r[7]) * r[8];
    Ut[8] = r[2] * (FF[0] * r[2] + FF[3] * r[5] + FF[6] * r[8]) +
            r[5] * (FF[1] * r[2] + FF[4] * r[5] + FF[7] * r[8]) +
            r[8] * (FF[2] * r[2] + FF[5] * r[5] + FF[8] * r[8]);
    FF[0] = Ut[0]; FF[1] = Ut[1]; FF[2] = Ut[2];
    FF[3] = Ut[1]; FF[4] = Ut[4]; FF[5] = Ut[5];
    FF[6] = Ut[2]; FF[7] = Ut[5]; FF[8] = Ut[8];
    mul(Rot, Rr, Rot);
    it++;
  }
  if (!conv) return 3;
  double lnl[3], il[3], sq[3], U[9] = {0}, Ui[9] = {0}, R[9];
  for (int c = 0; c < 3; c++) {
    lnl[c] = log(FF[c * 4]) / 2.;
    il[c] = 1. / sqrt(FF[c * 4]);
    sq[c] = sqrt(FF[c * 4]);
    double vec[3] = {Rot[c], Rot[3 + c], Rot[6 + c]}, ext[9];
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) ext[i * 3 + j] = vec[i] * vec[j];
    for (int k = 0; k < 9; k++) {
      if (c == 0) {
        U[k] = lnl[c] * ext[k];
        Ui[k] = il[c] * ext[k];
      } else {
        U[k] += lnl[c] * ext[k];
        Ui[k] += il[c] * ext[k];
      }
    }
  }
  mul(F, Ui, R);
  // divided differences
  double G[3][3], H[3][3];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      const double li = FF[i * 4], lj = FF[j * 4];
      const double m = 0.5 * (li + lj), q = (li - lj) / m;
      if (fabs(q) < 1e-3)  // 2 atanh(q/2) / (q m) = (1 + q^2/12 + q^4/80) / m
        G[i][j] = 0.5 * (1. + q * q / 12. + q * q * q * q / 80.) / m;
      else
        G[i][j] = (lnl[i] - lnl[j]) / (li - lj);
      H[i][j] = -il[i] * il[j] / (sq[i] + sq[j]);
    }
  for (int k = 0; k < 9; k++) {
    Ud[k] = cst(U[k]);
    Rd[k] = cst(R[k]);
  }
  for (int dir = 0; dir < NP; dir++) {
    double dF[9], dC[9], A[9], T[9], dL[9], dUi[9];
    for (int k = 0; k < 9; k++) dF[k] = Fd[k].d[dir];
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) {
        double s = 0;
        for (int k = 0; k < 3; k++) s += dF[k * 3 + i] * F[k * 3 + j] + F[k * 3 + i] * dF[k * 3 + j];
        dC[i * 3 + j] = s;
      }
    // A = V^T dC V
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) {
        double s = 0;
        for (int k = 0; k < 3; k++) s += dC[i * 3 + k] * Rot[k * 3 + j];
        T[i * 3 + j] = s;
      }
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) {
        double s = 0;
        for (int k = 0; k < 3; k++) s += Rot[k * 3 + i] * T[k * 3 + j];
        A[i * 3 + j] = s;
      }
    for (int pass = 0; pass < 2; pass++) {
      double B[9], *out = pass ? dUi : dL;
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) B[i * 3 + j] = (pass ? H[i][j] : G[i][j]) * A[i * 3 + j];
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
          double s = 0;
          for (int k = 0; k < 3; k++) s += B[i * 3 + k] * Rot[j * 3 + k];
          T[i * 3 + j] = s;
        }
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
          double s = 0;
          for (int k = 0; k < 3; k++) s += Rot[i * 3 + k] * T[k * 3 + j];
          out[i * 3 + j] = s;
        }
    }
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) {
        double s = 0;
        for (int k = 0; k < 3; k++) s += dF[i * 3 + k] * Ui[k * 3 + j] + F[i * 3 + k] * dUi[k * 3 + j];
        Rd[i * 3 + j].d[dir] = s;
        Ud[i * 3 + j].d[dir] = dL[i * 3 + j];
      }
  }
  return 0;
}

/* Matrix::inverse for n = 3 in the unblocked LAPACK order of dnl_oracle.c (dgetf2, dtrti2, dgetri);
 * pivots on the values; zero-skipping tests of the value-only routine are dropped (adding an
 * exact zero leaves the value unchanged and keeps its tangent). */
int inv3_lapack(D *a)
{
#define A_(r, c) a[(c) * 3 + (r)]
  int ipiv[3], info = 0;
  for (int j = 0; j < 3; j++) {
    int jp = j;
    double dmax = ABSV(A_(j, j));
    for (int i = j + 1; i < 3; i++)
      if (ABSV(A_(i, j)) > dmax) {
        dmax = ABSV(A_(i, j));
        jp = i;
      }
    ipiv[j] = jp;
    if (A_(jp, j).v != 0.) {
      if (jp != j)
        for (int c = 0; c < 3; c++) {
          D t = A_(j, c);
          A_(j, c) = A_(jp, c);
          A_(jp, c) = t;
        }
      if (j < 2) {
        D r = cst(1.) / A_(j, j);
        for (int i = j + 1; i < 3; i++) A_(i, j) = r * A_(i, j);
      }
    } else if (info == 0) {
      info = j + 1;
    }
    if (j < 2)
      for (int c = j + 1; c < 3; c++) {
        D temp = -1. * A_(j, c);
        for (int i = j + 1; i < 3; i++) A_(i, c) = A_(i, c) + A_(i, j) * temp;
      }
  }
  if (info) return info;
  for (int j = 0; j < 3; j++) {
    A_(j, j) = cst(1.) / A_(j, j);
    D ajj = -A_(j, j);
    for (int jj = 0; jj < j; jj++) {
      D temp = A_(jj, j);
      for (int i = 0; i < jj; i++) A_(i, j) += temp * A_(i, jj);
      A_(jj, j) *= A_(jj, jj);
    }
    for (int i = 0; i < j; i++) A_(i, j) = ajj * A_(i, j);
  }
  D work[3];
  for (int j = 2; j >= 0; j--) {
    for (int i = j + 1; i < 3; i++) {
      work[i] = A_(i, j);
      A_(i, j) = cst(0.);
    }
    for (int jc = j + 1; jc < 3; jc++) {
      D temp = -1. * work[jc];
      for (int i = 0; i < 3; i++) A_(i, j) += temp * A_(i, jc);
    }
  }
  for (int j = 1; j >= 0; j--) {
    int jp = ipiv[j];
    if (jp != j)
      for (int i = 0; i < 3; i++) {
        D t = A_(i, j);
        A_(i, j) = A_(i, jp);
        A_(i, jp) = t;
      }
  }
  return 0;
#undef A_
}

// Element2D/3D::computeInternalMatrices for one element (dnl_oracle.c elem_matrices)
int elem_matrices(dnls *h, long e)
{
  const long *cn = h->conn.data() + e * h->nen;
  int err = 0;
  for (int pt = 0; pt < h->nip; pt++) {
    const long ix = IPX(h, e, pt);
    if (h->dim == 2) {
      D J00 = cst(0.), J01 = cst(0.), J10 = cst(0.), J11 = cst(0.);
      for (int k = 0; k < 4; k++) {
        const D *x = h->coords.data() + cn[k] * 3;
        J00 += h->dNxi[pt][k][0] * x[0];
        J01 += h->dNxi[pt][k][1] * x[0];
        J10 += h->dNxi[pt][k][0] * x[1];
        J11 += h->dNxi[pt][k][1] * x[1];
      }
      const D detJ = (J00 * J11) - (J01 * J10);
      h->detJ[ix] = detJ;
      if (detJ.v < 0.) err = 1;
      D inv[4];
      inv[0] = J11 / detJ;
      inv[2] = -J01 / detJ;
      inv[1] = -J10 / detJ;
      inv[3] = J00 / detJ;
      for (int k = 0; k < 4; k++)
        for (int c = 0; c < 2; c++) {
          D acc = cst(0.);
          for (int l = 0; l < 2; l++) acc += inv[c * 2 + l] * h->dNxi[pt][k][l];
          DNS(h, e, pt, k, c) = acc;
        }
    } else {
      D J[3][3];
      for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) J[r][c] = cst(0.);
      for (int k = 0; k < h->nen; k++) {
        const D *x = h->coords.data() + cn[k] * 3;
        for (int r = 0; r < 3; r++)
          for (int c = 0; c < 3; c++) J[r][c] += h->dNxi[pt][k][c] * x[r];
      }
      const D detJ = (J[0][0] * J[1][1] * J[2][2]) + (J[1][0] * J[2][1] * J[0][2]) +
                     (J[2][0] * J[0][1] * J[1][2]) - (J[2][0] * J[1][1] * J[0][2]) -
                     (J[0][0] * J[2][1] * J[1][2]) - (J[1][0] * J[0][1] * J[2][2]);
      h->detJ[ix] = detJ;
      D a[9];
      for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) a[c * 3 + r] = J[r][c];
      if (inv3_lapack(a)) err = 7;
      for (int k = 0; k < h->nen; k++)
        for (int c = 0; c < 3; c++) {
          D acc = cst(0.);
          for (int l = 0; l < 3; l++) acc += a[c * 3 + l] * h->dNxi[pt][k][l];
          DNS(h, e, pt, k, c) = acc;
        }
    }
  }
  return err;
}

D elem_radius(const dnls *h, long e, int pt)
{
  const long *cn = h->conn.data() + e * h->nen;
  D R = cst(0.);
  for (int i = 0; i < h->nen; i++) R += h->Nt[pt][i] * h->coords[cn[i] * 3];
  return R;
}

void elem_F(const dnls *h, long e, int pt, D *F)
{
  const long *cn = h->conn.data() + e * h->nen;
  const D *du = h->fld[h->cur][0].data();
  t2_identity(F);
  if (h->dim == 2) {
    D v = cst(0.);
    for (int k = 0; k < 4; k++) {
      const D *d = du + cn[k] * 3;
      F[0] += DNS(h, e, pt, k, 0) * d[0];
      F[1] += DNS(h, e, pt, k, 1) * d[0];
      F[3] += DNS(h, e, pt, k, 0) * d[1];
      F[4] += DNS(h, e, pt, k, 1) * d[1];
      v += h->Nt[pt][k] * d[0];
    }
    if (h->etype == 0) {  // ElementPlane (etype 2) has no hoop stretch
      const D R = elem_radius(h, e, pt);
      F[8] += v / R;
    }
  } else {
    for (int k = 0; k < h->nen; k++) {
      const D *d = du + cn[k] * 3;
      for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) F[r * 3 + c] += DNS(h, e, pt, k, c) * d[r];
    }
  }
}

D yield_stress(const dnls *h, const D &evp, const D &shift)
{
  const D x = evp + SQRT23 * shift;
  return (h->A + h->B * dpow(x, h->n));
}
D yield_hardening(const dnls *h, const D &evp, const D &shift)
{
  const D x = evp + SQRT23 * shift;
  return (h->n * h->B * dpow(x, (h->n - 1.)));
}

// the one-point hexahedron's viscous hourglass force (dnl_oracle.c elem_hourglass; Flanagan and
// Belytschko, Int. J. Numer. Meth. Eng. 17, 1981) on the Current velocities
void elem_hourglass(const dnls *h, long e, D *fe)
{
  const long *cn = h->conn.data() + e * 8;
  const D *v = h->fld[h->cur][1].data();
  double hs[4][8];
  for (int k = 0; k < 8; k++) {
    const int sx = HX_XI[k], sy = HX_ETA[k], sz = HX_ZETA[k];
    hs[0][k] = sx * sy;
    hs[1][k] = sy * sz;
    hs[2][k] = sz * sx;
    hs[3][k] = sx * sy * sz;
  }
  D hx[4][3];
  for (int q = 0; q < 4; q++)
    for (int i = 0; i < 3; i++) {
      D s = cst(0.);
      for (int k = 0; k < 8; k++) s += hs[q][k] * h->coords[cn[k] * 3 + i];
      hx[q][i] = s;
    }
  D g[4][8], qv[4][3];
  for (int q = 0; q < 4; q++) {
    for (int i = 0; i < 3; i++) qv[q][i] = cst(0.);
    for (int k = 0; k < 8; k++) {
      D s = cst(hs[q][k]);
      for (int i = 0; i < 3; i++) s -= hx[q][i] * DNS(h, e, 0, k, i);
      g[q][k] = s;
      for (int i = 0; i < 3; i++) qv[q][i] += s * v[cn[k] * 3 + i];
    }
  }
  const double E = h->young, Nu = h->nu, rho = h->rho;
  const double c = sqrt((E * (1 - Nu)) / (rho * (1 + Nu) * (1 - 2 * Nu)));
  const D V = h->weight[0] * h->detJ[IPX(h, e, 0)], cv = dcbrt(V);
  const D ah = (0.25 * h->hourglass * rho * c) * (cv * cv);
  for (int k = 0; k < 8; k++)
    for (int i = 0; i < 3; i++) {
      D s = cst(0.);
      for (int q = 0; q < 4; q++) s += g[q][k] * qv[q][i];
      fe[k * 3 + i] -= ah * s;
    }
}

// Element::computeStress + Element::computeInternalForces (dnl_oracle.c elem_forces)
int elem_forces(dnls *h, long e, D *fe)
{
  const int nip = h->nip, nen = h->nen, dim = h->dim;
  const double K = h->young / (3. * (1. - 2. * h->nu));
  const double G = h->young / (2. * (1. + h->nu));
  D pressure = cst(0.0);
  int err = 0;
  D Rk[8][9];
  for (int pt = 0; pt < nip; pt++) {
    const long ix = IPX(h, e, pt);
    D F[9], dEps[9];
    D *R = Rk[pt];
    D *S = h->S.data() + ix * 9, *Eps = h->Eps.data() + ix * 9, *EpsPlas = h->EpsPlas.data() + ix * 9;
    elem_F(h, e, pt, F);
    int pe = polar_ln_u(F, dEps, R);
    if (pe) err = pe;
    for (int k = 0; k < 9; k++) Eps[k] += dEps[k];
    pressure += (dEps[0] + dEps[4] + dEps[8]);
    {
      const D tr = (dEps[0] + dEps[4] + dEps[8]) / 3.0;
      D dev[9];
      for (int k = 0; k < 9; k++) dev[k] = dEps[k];
      dev[0] = dEps[0] - tr;
      dev[4] = dEps[4] - tr;
      dev[8] = dEps[8] - tr;
      const double g2 = 2.0 * G;
      for (int k = 0; k < 9; k++) S[k] += g2 * dev[k];
    }
    D gamma = cst(0.0), h_ = cst(0.0);
    {
      const D Sigv0 = yield_stress(h, h->evp[ix], cst(0.0));
      D ss = cst(0.);
      for (int k = 0; k < 9; k++) ss += S[k] * S[k];
      const D Strial = SQRT32 * dsqrt(ss);
      if (Strial.v > Sigv0.v) {
        h_ = yield_hardening(h, h->evp[ix], cst(0.0));
        const D normS = dsqrt(ss);
        gamma = (normS - SQRT23 * Sigv0) / (2.0 * G * (1.0 + (h_) / (3.0 * G)));
        D dgamma = cst(0), Sigv, dfun, fun;
        int run = 1, iteration = 0;
        while (run) {
          Sigv = yield_stress(h, h->evp[ix], gamma);
          h_ = yield_hardening(h, h->evp[ix], gamma);
          dfun = SQRT32 * 2.0 * G + SQRT23 * h_;
          fun = dfun * gamma - (Strial - Sigv + h_ * SQRT23 * gamma);
          if (fabs(fun.v / Sigv.v) > RR_PRECISION) {
            dgamma = -fun / dfun;
            if (dgamma.v < 0 && ABSV(dgamma) > gamma.v) dgamma = -gamma * 0.9;
            gamma += dgamma;
          } else {
            run = 0;
          }
          iteration++;
          if (iteration > RR_MAXIT) {
            err = 2;
            run = 0;
          }
        }
        D n1[9];
        D ns = cst(0.);
        for (int k = 0; k < 9; k++) ns += S[k] * S[k];
        const D nrm = dsqrt(ns);
        for (int k = 0; k < 9; k++) n1[k] = S[k] / nrm;
        h->evp[ix] += SQRT23 * gamma;
        const D c = 2.0 * G * gamma;
        for (int k = 0; k < 9; k++) S[k] -= c * n1[k];
        for (int k = 0; k < 9; k++) EpsPlas[k] += gamma * n1[k];
      }
    }
  }
  pressure = pressure / (double)nip;
  for (int pt = 0; pt < nip; pt++) {
    const long ix = IPX(h, e, pt);
    D *S = h->S.data() + ix * 9, *Eps = h->Eps.data() + ix * 9, *EpsPlas = h->EpsPlas.data() + ix * 9;
    h->p[ix] += K * pressure;
    t2_rotate(Rk[pt], S);
    t2_rotate(Rk[pt], Eps);
    t2_rotate(Rk[pt], EpsPlas);
    D *Sig = h->Sig.data() + ix * 9;
    D pI[9];
    t2_identity(pI);
    for (int k = 0; k < 9; k++) pI[k] = h->p[ix] * pI[k];
    for (int k = 0; k < 9; k++) Sig[k] = S[k] + pI[k];
  }
  for (int k = 0; k < nen * dim; k++) fe[k] = cst(0.0);
  for (int pt = 0; pt < nip; pt++) {
    const long ix = IPX(h, e, pt);
    const D *Sig = h->Sig.data() + ix * 9;
    D WxdJ = h->weight[pt] * h->detJ[ix];
    D R = cst(0.);
    if (h->etype == 0) {
      R = elem_radius(h, e, pt);
      WxdJ *= DEUXPI * R;
    }
    for (int I = 0; I < nen; I++)
      for (int i = 0; i < dim; i++)
        for (int j = 0; j < dim; j++) fe[I * dim + i] -= DNS(h, e, pt, I, j) * Sig[j * 3 + i] * WxdJ;
    if (h->etype == 0)
      for (int I = 0; I < nen; I++) fe[I * dim] -= (h->Nt[pt][I] * Sig[8] / R) * WxdJ;
  }
  if (h->etype == 5) elem_hourglass(h, e, fe);
  return err;
}

int internal_forces(dnls *h)
{
  const int nd = h->nen * h->dim;
  int err = 0;
#pragma omp parallel for schedule(static) reduction(max : err)
  for (long e = 0; e < h->E; e++) {
    int r = elem_matrices(h, e);
    if (r > err) err = r;
    r = elem_forces(h, e, h->fe.data() + e * nd);
    if (r > err) err = r;
  }
#pragma omp parallel for schedule(static)
  for (long n = 0; n < h->N; n++)
    for (int j = 0; j < h->dim; j++) {
      D acc = cst(0.0);
      for (long q = h->n2e_start[n]; q < h->n2e_start[n + 1]; q++) {
        const long ent = h->n2e[q];
        acc += h->fe[(ent / h->nen) * nd + (ent % h->nen) * h->dim + j];
      }
      h->fint[n * h->dim + j] = acc;
    }
  return err;
}

void apply_bc(dnls *h, long n)
{
  D *cdu = h->fld[h->cur][0].data() + n * 3, *cv = h->fld[h->cur][1].data() + n * 3;
  D *ca = h->fld[h->cur][2].data() + n * 3;
  D *ndu = h->fld[1 - h->cur][0].data() + n * 3, *nv = h->fld[1 - h->cur][1].data() + n * 3;
  D *na = h->fld[1 - h->cur][2].data() + n * 3;
  for (long q = h->bcn_start[n]; q < h->bcn_start[n + 1]; q++) {
    const double *val = h->bcn_val.data() + q * 3;
    if (h->bcn_kind[q] == 0) {
      for (int i = 0; i < 3; i++)
        if (val[i] == 1.) cdu[i] = ndu[i] = cv[i] = nv[i] = ca[i] = na[i] = cst(0.);
    } else {
      for (int i = 0; i < 3; i++)
        if (val[i] != 0.) {
          ca[i] = na[i] = cst(0.);
          cv[i] = nv[i] = cst(val[i]);
          cdu[i] = cv[i] * h->timeStep;
          ndu[i] = nv[i] * h->timeStep;
        }
    }
  }
}

void predictions(dnls *h)
{
  const double dt = h->timeStep;
  const double c1 = dt * (0.5 - h->beta), c2 = dt * (1 - h->gamma);
#pragma omp parallel for schedule(static)
  for (long n = 0; n < h->N; n++) {
    D *cv = h->fld[h->cur][1].data() + n * 3, *ca = h->fld[h->cur][2].data() + n * 3;
    D *cd = h->fld[h->cur][3].data() + n * 3;
    D *ndu = h->fld[1 - h->cur][0].data() + n * 3, *nv = h->fld[1 - h->cur][1].data() + n * 3;
    D *na = h->fld[1 - h->cur][2].data() + n * 3, *nd = h->fld[1 - h->cur][3].data() + n * 3;
    for (int i = 0; i < 3; i++) {
      D du = ca[i];
      du = du * c1;
      du += cv[i];
      du = du * dt;
      ndu[i] = du;
      nd[i] = cd[i] + ndu[i];
      D v = ca[i];
      v = v * c2;
      v += cv[i];
      nv[i] = v;
      na[i] = cst(0.0);
    }
    apply_bc(h, n);
  }
}

void explicit_solve(dnls *h)
{
  const double dt = h->timeStep;
  const double cg = dt * h->gamma, cb = (dt * dt) * h->beta;
#pragma omp parallel for schedule(static)
  for (long n = 0; n < h->N; n++) {
    D *ca = h->fld[h->cur][2].data() + n * 3, *cd = h->fld[h->cur][3].data() + n * 3;
    D *ndu = h->fld[1 - h->cur][0].data() + n * 3, *nv = h->fld[1 - h->cur][1].data() + n * 3;
    D *na = h->fld[1 - h->cur][2].data() + n * 3, *nd = h->fld[1 - h->cur][3].data() + n * 3;
    for (int j = 0; j < h->dim; j++) na[j] = h->fint[n * h->dim + j] / h->mass[n];
    for (int i = 0; i < 3; i++) {
      na[i] -= h->alphaM * ca[i];
      na[i] = na[i] / (1.0 - h->alphaM);
      nv[i] += cg * na[i];
      ndu[i] += cb * na[i];
    }
    apply_bc(h, n);
    for (int i = 0; i < 3; i++) nd[i] = cd[i] + ndu[i];
    for (int i = 0; i < 3; i++) h->coords[n * 3 + i] += ndu[i];
  }
}

}  // namespace

extern "C" {

/* mat[6] = {E, nu, rho, A, B, n}; v0[3] the initial velocity (its magnitude is parameter 3);
 * mass[N] the lumped nodal masses; BC groups as in dnlo_create. */
dnls *dnls_create(int etype, long N, long E, const double *coords, const long *conn,
                  const double *mat, const double *v0, const double *mass, long nbc,
                  const long *bc_kind, const double *bc_val, const long *bc_start,
                  const long *bc_nodes, double rho_b)
{
  if (etype < 0 || etype > 5 || N <= 0 || E <= 0) return nullptr;
  dnls *h = new dnls();
  h->etype = etype;
  h->dim = (etype == 0 || etype == 2) ? 2 : 3;
  h->nen = (etype == 1 || etype == 5) ? 8 : (etype == 4 ? 10 : 4);
  h->nip = etype == 1 ? 8 : ((etype == 3 || etype == 5) ? 1 : 4);
  h->rho = mat[2];
  h->hourglass = 0.05;
  h->N = N;
  h->E = E;
  h->conn.assign(conn, conn + E * h->nen);
  for (long v : h->conn)
    if (v < 0 || v >= N) {
      delete h;
      return nullptr;
    }
  h->coords.resize(N * 3);
  for (long i = 0; i < N * 3; i++) h->coords[i] = cst(coords[i]);
  const double vn = sqrt(v0[0] * v0[0] + v0[1] * v0[1] + v0[2] * v0[2]);
  for (int b = 0; b < 2; b++)
    for (int f = 0; f < 4; f++) h->fld[b][f].assign(N * 3, cst(0.));
  for (long n = 0; n < N; n++)
    for (int i = 0; i < 3; i++) {
      D v = cst(v0[i]);
      v.d[3] = vn > 0 ? v0[i] / vn : 0.;
      h->fld[0][1][n * 3 + i] = v;
      h->fld[1][1][n * 3 + i] = v;
    }
  h->cur = 0;
  h->mass.assign(mass, mass + N);
  h->fint.assign(N * h->dim, cst(0.));
  h->fe.assign(E * h->nen * h->dim, cst(0.));
  const long nI = E * h->nip;
  for (auto *v : {&h->S, &h->Eps, &h->EpsPlas, &h->Sig}) v->assign(nI * 9, cst(0.));
  h->p.assign(nI, cst(0.));
  h->evp.assign(nI, cst(1e-10));
  h->detJ.assign(nI, cst(0.));
  h->dN.assign(nI * h->nen * 3, cst(0.));
  h->young = mat[0];
  h->nu = mat[1];
  h->A = cst(mat[3]);
  h->A.d[0] = 1.;
  h->B = cst(mat[4]);
  h->B.d[1] = 1.;
  h->n = cst(mat[5]);
  h->n.d[2] = 1.;
  h->bcn_start.assign(N + 1, 0);
  for (long g = 0; g < nbc; g++)
    for (long q = bc_start[g]; q < bc_start[g + 1]; q++) h->bcn_start[bc_nodes[q] + 1]++;
  for (long n = 0; n < N; n++) h->bcn_start[n + 1] += h->bcn_start[n];
  const long nb = h->bcn_start[N];
  h->bcn_kind.assign(nb > 0 ? nb : 1, 0);
  h->bcn_val.assign((nb > 0 ? nb : 1) * 3, 0.);
  std::vector<long> fill(N, 0);
  for (long g = 0; g < nbc; g++)
    for (long q = bc_start[g]; q < bc_start[g + 1]; q++) {
      const long n = bc_nodes[q];
      const long at = h->bcn_start[n] + fill[n]++;
      h->bcn_kind[at] = (int)bc_kind[g];
      for (int i = 0; i < 3; i++) h->bcn_val[at * 3 + i] = bc_val[g * 3 + i];
    }
  h->n2e_start.assign(N + 1, 0);
  for (long i = 0; i < E * h->nen; i++) h->n2e_start[h->conn[i] + 1]++;
  for (long n = 0; n < N; n++) h->n2e_start[n + 1] += h->n2e_start[n];
  h->n2e.assign(E * h->nen, 0);
  std::fill(fill.begin(), fill.end(), 0);
  for (long i = 0; i < E * h->nen; i++) {
    const long n = h->conn[i];
    h->n2e[h->n2e_start[n] + fill[n]++] = i;
  }
  const double rb = rho_b;
  h->alphaM = (2.0 * rb - 1.0) / (1.0 + rb);
  h->beta = (5.0 - 3.0 * rb) / ((1.0 + rb) * (1.0 + rb) * (2.0 - rb));
  h->gamma = 1.5 - h->alphaM;
  h->err = 0;
  build_tables(h);
  return h;
}

void dnls_destroy(dnls *h) { delete h; }

/* the one-point hexahedron's hourglass coefficient (dnlo_set_hourglass) */
int dnls_set_hourglass(dnls *h, double coefficient)
{
  if (!(coefficient >= 0.) || coefficient > 1e300) return 1;
  h->hourglass = coefficient;
  return 0;
}

/* nsteps explicit steps with the step sizes dts[0..nsteps): the ExplicitSolverCH::solve loop body
 * (predictions, internal forces on the current coordinates, explicit solve, swap). */
int dnls_run(dnls *h, long nsteps, const double *dts)
{
  for (long k = 0; k < nsteps; k++) {
    h->timeStep = dts[k];
    predictions(h);
    int r = internal_forces(h);
    if (r) return h->err = r;
    explicit_solve(h);
    h->cur = 1 - h->cur;
  }
  return 0;
}

/* coords (N*3) and their derivatives dx[p*N*3 + n*3 + i] for p = A, B, n, |v0| */
void dnls_coords(const dnls *h, double *x, double *dx)
{
  const long n3 = h->N * 3;
  for (long i = 0; i < n3; i++) {
    if (x) x[i] = h->coords[i].v;
    if (dx)
      for (int p = 0; p < NP; p++) dx[p * n3 + i] = h->coords[i].d[p];
  }
}

}  // extern "C"
