/* CPU restatement of DynELA's explicit-dynamics step -- the ORACLE (test infrastructure only).
 *
 * Only tests, __graft_entry__.smoke() and bench.py's CPU-baseline leg load this file's library,
 * as the checker or as the timed CPU baseline.  Nothing on the product path calls it.
 *
 * Every routine restates one reference routine, named with file:line (paths relative to
 * Sources/Libraries/ of pantale/ReDynELA), keeping its arithmetic in the same order so that,
 * compiled with -ffp-contract=off, results agree with the reference bit for bit where the
 * reference itself is deterministic.  Deliberate differences:
 *   - assembly sums element contributions to each node in ascending element order, which is
 *     what Domain::computeInternalForces strategy 0 (Domain.C:158-195) does on one thread;
 *     element loops run on OpenMP threads but the sums stay in that order;
 *   - the Pulse power iteration (Domain.C:817-945) accumulates K.x in ascending element order;
 *     the reference uses its Jobs order (elements sorted by centroid, Jobs.C:129-165) and one
 *     partial vector per thread, so the two differ in the last bits;
 *   - fatal errors (exit(-1) in the reference) become status codes.
 */
#include "dnl_oracle.h"
#include "tet10_tables.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* basicTools/Math.h:36-46 */
#define DNL_PI 3.1415926535897932384626433832795
#define DNL_DEUXPI 6.283185307179586476925286766559
#define DNL_SQRT23 0.8164965809277260327324280249019
#define DNL_SQRT32 1.2247448713915890490986420373529
/* linearAlgebra/Tensor2.C:34 */
#define DNL_PRECISION_POLAR 10.0E-10
/* finiteElement/DefaultValues.h:24-36 */
#define DNL_RR_PRECISION 1.0E-8
#define DNL_RR_MAXIT 2000
#define DNL_PULSE_MAXIT 1000
#define DNL_PULSE_CONV 1e-4

#define ABS(x) ((x) < 0 ? -(x) : (x))

struct dnlo {
  int etype, dim, nen, nip;
  long N, E;
  long *conn;
  double *coords, *coords0;
  double *fld[2][4]; /* [NodalField][delta_disp, mat_speed, dmat_speed, disp], N*3 each */
  double *ro[2];     /* NodalField::ro */
  int cur;           /* index of Node::Current */
  double *mass;      /* Node::mass */
  double *Mass;      /* Domain::Mass, dim*N */
  double *fint;      /* Domain::Fint, dim*N */
  double *fe;        /* per-element force vectors, E*nen*dim */
  double *S, *Eps, *EpsPlas, *Sig, *dEps, *R;
  double *p, *evp, *detJ, *detJ0;
  double *dN; /* (E, nip, nen, 3) */
  double young, nu, rho, A, B, n;
  double hourglass; /* etype 5: viscous hourglass coefficient */
  /* materials (Structure::attachMaterialToElements): per material E, nu, rho, hardening law and
   * its parameters / table; material 0 is the one of dnlo_create */
  int nmat;
  double *mE, *mNu, *mRho, *mP; /* mP: nmat x 8 (POWER: A B n; METAFOR: P1..P8) */
  int *mLaw;
  long *mTab;                   /* nmat + 1 offsets into tabX / tabY */
  double *tabX, *tabY;
  int *elemMat;                 /* E material indices, or NULL: material 0 */
  double v0[3];
  long *bcn_start; /* per node: its constant BCs, in attachment order */
  int *bcn_kind;
  double *bcn_val;
  double tend, rho_b, safety;
  long freq;
  int method;
  double alphaM, beta, gamma, omegaS;
  double timeStep, currentTime, nextTime, upTime, startTime;
  long increment;
  double computedTimeStep, lastTimeStep, tsDate, lastTsDate;
  double *EV, *Ke, *kx;
  double fmax0;
  long pulse_iter, pulse_total;
  long *n2e_start, *n2e;
  double Nt[8][10];
  double dNxi[8][10][3];
  double weight[8];
  int bad_elem;
  int mass_done;
};

/* ---------------------------------------------------------------------- element tables
 * finiteElement/ElQua4nAx.C:31-101 and ElHex8n3D.C:26-161 tabulate N and dN/dxi at the Gauss
 * points +-1/sqrt(3) with weight 1.  The tables are rebuilt here from the bilinear/trilinear shape
 * functions; each value is formed by the same constant expression the reference writes
 * (e.g. (2.0 + sqrt(3.0)) / 6.0), so the doubles are identical. */
static const int AX_XI[4] = {-1, 1, 1, -1}, AX_ETA[4] = {-1, -1, 1, 1};
static const int HX_XI[8] = {-1, 1, 1, -1, -1, 1, 1, -1};
static const int HX_ETA[8] = {-1, -1, 1, 1, -1, -1, 1, 1};
static const int HX_ZETA[8] = {-1, -1, -1, -1, 1, 1, 1, 1};

static void build_tables(dnlo *h)
{
  if (h->etype == 5) { /* the one-point hexahedron (not a reference element): the cube's centre */
    h->weight[0] = 8.0;
    for (int k = 0; k < 8; k++) {
      h->Nt[0][k] = 0.125;
      h->dNxi[0][k][0] = HX_XI[k] * 0.125;
      h->dNxi[0][k][1] = HX_ETA[k] * 0.125;
      h->dNxi[0][k][2] = HX_ZETA[k] * 0.125;
    }
  } else if (h->etype == 3) { /* ElTet4n3D (ElTet4n3D.C:33-57): one point, weight 1/6 */
    h->weight[0] = 1. / 6.;
    for (int k = 0; k < 4; k++) {
      h->Nt[0][k] = 0.25;
      for (int c = 0; c < 3; c++) h->dNxi[0][k][c] = k == 0 ? -1.0 : (k - 1 == c ? 1.0 : 0.0);
    }
  } else if (h->etype == 4) {
    dnl_tet10_tables(h->Nt, h->dNxi, h->weight); /* tet10_tables.h */
  } else if (h->etype != 1) { /* ElQua4nAx and ElQua4n2D share their tables (ElQua4n2D.C:26-70) */
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
        int dx = HX_XI[k] != HX_XI[pt], dy = HX_ETA[k] != HX_ETA[pt],
            dz = HX_ZETA[k] != HX_ZETA[pt];
        h->Nt[pt][k] = cN[dx + dy + dz];
        h->dNxi[pt][k][0] = HX_XI[k] > 0 ? cD[dy + dz] : -cD[dy + dz];
        h->dNxi[pt][k][1] = HX_ETA[k] > 0 ? cD[dx + dz] : -cD[dx + dz];
        h->dNxi[pt][k][2] = HX_ZETA[k] > 0 ? cD[dx + dy] : -cD[dx + dy];
      }
    }
  }
}

/* ---------------------------------------------------------------------- Tensor2 arithmetic */
/* linearAlgebra/Tensor2.C:360-381, row-major v[i*3+j] */
static void t2_mul(const double *a, const double *b, double *c)
{
  double t[9];
  t[0] = a[0] * b[0] + a[1] * b[3] + a[2] * b[6];
  t[1] = a[0] * b[1] + a[1] * b[4] + a[2] * b[7];
  t[2] = a[0] * b[2] + a[1] * b[5] + a[2] * b[8];
  t[3] = a[3] * b[0] + a[4] * b[3] + a[5] * b[6];
  t[4] = a[3] * b[1] + a[4] * b[4] + a[5] * b[7];
  t[5] = a[3] * b[2] + a[4] * b[5] + a[5] * b[8];
  t[6] = a[6] * b[0] + a[7] * b[3] + a[8] * b[6];
  t[7] = a[6] * b[1] + a[7] * b[4] + a[8] * b[7];
  t[8] = a[6] * b[2] + a[7] * b[5] + a[8] * b[8];
  memcpy(c, t, sizeof t);
}

static void t2_transpose(const double *a, double *t)
{
  t[0] = a[0]; t[1] = a[3]; t[2] = a[6];
  t[3] = a[1]; t[4] = a[4]; t[5] = a[7];
  t[6] = a[2]; t[7] = a[5]; t[8] = a[8];
}

static void t2_identity(double *t)
{
  for (int k = 0; k < 9; k++) t[k] = 0.;
  t[0] = t[4] = t[8] = 1.;
}

/* R X R^T as written in Element.C:386-388: R * (X * R.Transpose()) */
static void t2_rotate(const double *R, double *X)
{
  double Rt[9], tmp[9];
  t2_transpose(R, Rt);
  t2_mul(X, Rt, tmp);
  t2_mul(R, tmp, X);
}

/* Tensor2::polarDecomposeLnU, linearAlgebra/Tensor2.C:1154-1259: Jacobi eigen-iteration on F^T F,
 * U <- ln(U) = sum ln(lambda_i)/2 v_i (x) v_i, R <- F sum lambda_i^{-1/2} v_i (x) v_i. */
static int polar_ln_u(const double *F, double *U, double *R)
{
  double Ft[9], FF[9], Rot[9], Rr[9], Ut[9];
  t2_transpose(F, Ft);
  t2_mul(Ft, F, FF);
  t2_identity(Rot);
  int it = 1;
  while (it < 30) {
    int q = (ABS(FF[1]) > ABS(FF[2]) ? 1 : 2);
    int p = (ABS(FF[q]) > ABS(FF[5]) ? 0 : 1);
    if (p == 1) q = 2;
    if (ABS(FF[p * 3 + q]) < DNL_PRECISION_POLAR) {
      double ext[9], vec[3];
      for (int c = 0; c < 3; c++) {
        const double lnl = log(FF[c * 4]) / 2.;
        const double il = 1. / sqrt(FF[c * 4]);
        vec[0] = Rot[c]; vec[1] = Rot[3 + c]; vec[2] = Rot[6 + c];
        for (int i = 0; i < 3; i++)
          for (int j = 0; j < 3; j++) ext[i * 3 + j] = vec[i] * vec[j];
        for (int k = 0; k < 9; k++) {
          if (c == 0) {
            U[k] = lnl * ext[k];
            Rr[k] = il * ext[k];
          } else {
            U[k] += lnl * ext[k];
            Rr[k] += il * ext[k];
          }
        }
      }
      t2_mul(F, Rr, R);
      return 0;
    }
    const double alpha = (FF[q * 3 + q] - FF[p * 3 + p]) / (2. * FF[p * 3 + q]);
    const double t = (alpha != 0. ? 1. / (alpha + sqrt(alpha * alpha + 1.) * (alpha > 0. ? 1. : -1.)) : 1.);
    const double Ct = 1. / (sqrt(1. + t * t));
    const double St = t * Ct;
    t2_identity(Rr);
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
    t2_mul(Rot, Rr, Rot);
    it++;
  }
  return DNLO_ERR_JACOBI_NOCONV;
}

/* ---------------------------------------------------------------------- 3x3 inverse
 * Matrix::inverse (linearAlgebra/Matrix.C:1653-1700) calls LAPACK dgetrf + dgetri on the column
 * major copy.  For n = 3 the f2c LAPACK takes its unblocked paths: dgetf2 (partial pivoting with
 * idamax, reciprocal scaling by dscal, rank-1 update by dger), then dtrti2 (dtrmv + dscal) and the
 * unblocked back-substitution of dgetri (dgemv), then the column interchanges.  a[c*3 + r]. */
static int inv3_lapack(double *a)
{
#define A_(r, c) a[(c) * 3 + (r)]
  int ipiv[3], info = 0;
  for (int j = 0; j < 3; j++) {
    int jp = j;
    double dmax = ABS(A_(j, j));
    for (int i = j + 1; i < 3; i++)
      if (ABS(A_(i, j)) > dmax) {
        dmax = ABS(A_(i, j));
        jp = i;
      }
    ipiv[j] = jp;
    if (A_(jp, j) != 0.) {
      if (jp != j)
        for (int c = 0; c < 3; c++) {
          double t = A_(j, c);
          A_(j, c) = A_(jp, c);
          A_(jp, c) = t;
        }
      if (j < 2) {
        double r = 1. / A_(j, j);
        for (int i = j + 1; i < 3; i++) A_(i, j) = r * A_(i, j);
      }
    } else if (info == 0) {
      info = j + 1;
    }
    if (j < 2)
      for (int c = j + 1; c < 3; c++)
        if (A_(j, c) != 0.) {
          double temp = -1. * A_(j, c);
          for (int i = j + 1; i < 3; i++) A_(i, c) = A_(i, c) + A_(i, j) * temp;
        }
  }
  if (info) return info;
  for (int j = 0; j < 3; j++) { /* dtrti2, upper, non-unit */
    A_(j, j) = 1. / A_(j, j);
    double ajj = -A_(j, j);
    for (int jj = 0; jj < j; jj++)
      if (A_(jj, j) != 0.) {
        double temp = A_(jj, j);
        for (int i = 0; i < jj; i++) A_(i, j) += temp * A_(i, jj);
        A_(jj, j) *= A_(jj, jj);
      }
    for (int i = 0; i < j; i++) A_(i, j) = ajj * A_(i, j);
  }
  double work[3];
  for (int j = 2; j >= 0; j--) { /* dgetri, unblocked */
    for (int i = j + 1; i < 3; i++) {
      work[i] = A_(i, j);
      A_(i, j) = 0.;
    }
    for (int jc = j + 1; jc < 3; jc++)
      if (work[jc] != 0.) {
        double temp = -1. * work[jc];
        for (int i = 0; i < 3; i++) A_(i, j) += temp * A_(i, jc);
      }
  }
  for (int j = 1; j >= 0; j--) {
    int jp = ipiv[j];
    if (jp != j)
      for (int i = 0; i < 3; i++) {
        double t = A_(i, j);
        A_(i, j) = A_(i, jp);
        A_(i, jp) = t;
      }
  }
  return 0;
#undef A_
}

/* ---------------------------------------------------------------------- kinematics */
#define IPX(h, e, pt) ((long)(e) * (h)->nip + (pt))
#define DN(h, e, pt, k, c) (h)->dN[(IPX(h, e, pt) * (h)->nen + (k)) * 3 + (c)]

/* Element2D::computeInternalMatrices (Element2D.C:53-126) and Element3D::computeInternalMatrices
 * (Element3D.C:53-113) for one element. */
static int elem_matrices(dnlo *h, long e, int reference)
{
  const long *cn = h->conn + e * h->nen;
  int err = 0;
  for (int pt = 0; pt < h->nip; pt++) {
    const long ix = IPX(h, e, pt);
    if (h->dim == 2) {
      double J00 = 0., J01 = 0., J10 = 0., J11 = 0.;
      for (int k = 0; k < 4; k++) {
        const double *x = h->coords + cn[k] * 3;
        J00 += h->dNxi[pt][k][0] * x[0];
        J01 += h->dNxi[pt][k][1] * x[0];
        J10 += h->dNxi[pt][k][0] * x[1];
        J11 += h->dNxi[pt][k][1] * x[1];
      }
      const double detJ = (J00 * J11) - (J01 * J10);
      h->detJ[ix] = detJ;
      if (reference) h->detJ0[ix] = detJ;
      if (detJ < 0.) err = DNLO_ERR_NEG_DETJ;
      double inv[4]; /* column major: inv[c*2+r] */
      inv[0] = J11 / detJ;
      inv[2] = -J01 / detJ;
      inv[1] = -J10 / detJ;
      inv[3] = J00 / detJ;
      for (int k = 0; k < 4; k++)
        for (int c = 0; c < 2; c++) { /* dgemm: C(k,c) = sum_l Inv(l,c) dNxi(k,l) */
          double acc = 0.;
          for (int l = 0; l < 2; l++)
            if (inv[c * 2 + l] != 0.) acc += inv[c * 2 + l] * h->dNxi[pt][k][l];
          DN(h, e, pt, k, c) = acc;
        }
    } else {
      double J[3][3] = {{0., 0., 0.}, {0., 0., 0.}, {0., 0., 0.}};
      for (int k = 0; k < h->nen; k++) {
        const double *x = h->coords + cn[k] * 3;
        for (int r = 0; r < 3; r++)
          for (int c = 0; c < 3; c++) J[r][c] += h->dNxi[pt][k][c] * x[r];
      }
      const double detJ = (J[0][0] * J[1][1] * J[2][2]) + (J[1][0] * J[2][1] * J[0][2]) +
                          (J[2][0] * J[0][1] * J[1][2]) - (J[2][0] * J[1][1] * J[0][2]) -
                          (J[0][0] * J[2][1] * J[1][2]) - (J[1][0] * J[0][1] * J[2][2]);
      h->detJ[ix] = detJ;
      if (reference) h->detJ0[ix] = detJ;
      /* a negative 3D Jacobian is only reported by the reference (Element3D.C:98-105) */
      double a[9];
      for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) a[c * 3 + r] = J[r][c];
      if (inv3_lapack(a)) err = DNLO_ERR_SINGULAR;
      for (int k = 0; k < h->nen; k++)
        for (int c = 0; c < 3; c++) {
          double acc = 0.;
          for (int l = 0; l < 3; l++)
            if (a[c * 3 + l] != 0.) acc += a[c * 3 + l] * h->dNxi[pt][k][l];
          DN(h, e, pt, k, c) = acc;
        }
    }
  }
  return err;
}

/* Element2D::getRadius_atIntPoint (Element2D.C:233-246), current coordinates */
static double elem_radius(const dnlo *h, long e, int pt)
{
  const long *cn = h->conn + e * h->nen;
  double R = 0.;
  for (int i = 0; i < h->nen; i++) R += h->Nt[pt][i] * h->coords[cn[i] * 3];
  return R;
}

/* ElementAx::getF_atIntPoint (ElementAx.C:114-136) / ElementPlane::getF_atIntPoint
 * (ElementPlane.C:83-99, no hoop stretch) / Element3D::getF_atIntPoint (Element3D.C:182-205) with
 * the Current nodal field (Node::getFieldAtTime(0), Node.h:178-183) */
static void elem_F(const dnlo *h, long e, int pt, double *F)
{
  const long *cn = h->conn + e * h->nen;
  const double *du = h->fld[h->cur][0];
  t2_identity(F);
  if (h->dim == 2) {
    double v = 0.;
    for (int k = 0; k < 4; k++) {
      const double *d = du + cn[k] * 3;
      F[0] += DN(h, e, pt, k, 0) * d[0];
      F[1] += DN(h, e, pt, k, 1) * d[0];
      F[3] += DN(h, e, pt, k, 0) * d[1];
      F[4] += DN(h, e, pt, k, 1) * d[1];
      v += h->Nt[pt][k] * d[0];
    }
    if (h->etype == 0) {
      const double R = elem_radius(h, e, pt);
      F[8] += v / R;
    }
  } else {
    for (int k = 0; k < h->nen; k++) {
      const double *d = du + cn[k] * 3;
      for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) F[r * 3 + c] += DN(h, e, pt, k, c) * d[r];
    }
  }
}

#define MATOF(h, e) ((h)->elemMat ? (h)->elemMat[e] : 0)

/* DiscreteFunction::getValue / getSlope (linearAlgebra/DiscreteFunction.C:169-201, 274-297):
 * the segment ending at the first point with x >= a (the first segment below the table), the
 * point's own value when x == a, and 0 beyond the last point. */
static double tab_value(const double *x, const double *y, long n, double a)
{
  for (long i = 1; i < n; i++)
    if (x[i] >= a) {
      if (x[i] == a) return y[i];
      return ((a - x[i - 1]) / (x[i] - x[i - 1])) * (y[i] - y[i - 1]) + y[i - 1];
    }
  return 0;
}
static double tab_slope(const double *x, const double *y, long n, double a)
{
  for (long i = 1; i < n; i++)
    if (x[i] >= a) return (y[i] - y[i - 1]) / (x[i] - x[i - 1]);
  return 0;
}

/* getIsotropicYieldStress / getIsotropicYieldHardening of the material's hardening law at
 * evp + sqrt(2/3) shift: IsoHardElastoplastic (IsoHardElastoplastic.C:171-184),
 * IsoHardElastoplasticTabular (IsoHardElastoplasticTabular.C:103-116), IsoHardMetafor
 * (IsoHardMetafor.C:132-153). */
static double yield_stress(const dnlo *h, int mi, double evp, double shift)
{
  const double x = evp + DNL_SQRT23 * shift;
  const double *P = h->mP + 8 * mi;
  switch (h->mLaw[mi]) {
  case DNLO_HARD_TABULAR:
    return tab_value(h->tabX + h->mTab[mi], h->tabY + h->mTab[mi], h->mTab[mi + 1] - h->mTab[mi], x);
  case DNLO_HARD_METAFOR:
    return (P[1] - P[0]) * (1 - exp(-P[2] * (x))) + P[3] * pow(x, P[4]) + P[0] * pow((1 + P[5] * x), P[6]) + P[7] * x;
  default:
    return (P[0] + P[1] * pow(x, P[2]));
  }
}
static double yield_hardening(const dnlo *h, int mi, double evp, double shift)
{
  const double x = evp + DNL_SQRT23 * shift;
  const double *P = h->mP + 8 * mi;
  switch (h->mLaw[mi]) {
  case DNLO_HARD_TABULAR:
    return tab_slope(h->tabX + h->mTab[mi], h->tabY + h->mTab[mi], h->mTab[mi + 1] - h->mTab[mi], x);
  case DNLO_HARD_METAFOR:
    if (x > 0.)
      return ((P[1] - P[0]) * P[2] * exp(-P[2] * (x)) + P[3] * P[4] * pow(x, (P[4] - 1.0)) +
              P[0] * P[5] * P[6] * pow((1.0 + P[5] * x), (P[6] - 1.0)) + P[7]);
    return ((P[1] - P[0]) * P[2] * exp(-P[2] * (x)) + P[0] * P[5] * P[6] * pow((1.0 + P[5] * x), (P[6] - 1.0)) + P[7]);
  default:
    return (P[2] * P[1] * pow(x, (P[2] - 1.)));
  }
}

/* The one-point hexahedron's viscous hourglass forces, Flanagan & Belytschko (Int. J. Numer.
 * Meth. Eng. 17, 1981): hourglass vectors h_q of the node signs (xi eta, eta zeta, zeta xi,
 * xi eta zeta) made orthogonal to the linear fields, g_q = h_q - sum_i (h_q . x_i) b_i with b the
 * centre-point gradients; fe_k -= a_h sum_q g_qk (g_q . v) with a_h = coefficient rho c V^(2/3)/4
 * on the Current velocities, V = 8 detJ at the centre, c the material's sound speed.  Not a
 * reference element: this is the restatement of the GPU element's own formulation. */
static void elem_hourglass(const dnlo *h, long e, double *fe)
{
  const long *cn = h->conn + e * 8;
  const int mi = h->elemMat ? h->elemMat[e] : 0;
  const double *v = h->fld[h->cur][1];
  double hs[4][8];
  for (int k = 0; k < 8; k++) {
    const int sx = HX_XI[k], sy = HX_ETA[k], sz = HX_ZETA[k];
    hs[0][k] = sx * sy;
    hs[1][k] = sy * sz;
    hs[2][k] = sz * sx;
    hs[3][k] = sx * sy * sz;
  }
  double hx[4][3];
  for (int q = 0; q < 4; q++)
    for (int i = 0; i < 3; i++) {
      double s = 0.;
      for (int k = 0; k < 8; k++) s += hs[q][k] * h->coords[cn[k] * 3 + i];
      hx[q][i] = s;
    }
  double g[4][8], qv[4][3];
  for (int q = 0; q < 4; q++) {
    for (int i = 0; i < 3; i++) qv[q][i] = 0.;
    for (int k = 0; k < 8; k++) {
      double s = hs[q][k];
      for (int i = 0; i < 3; i++) s -= hx[q][i] * DN(h, e, 0, k, i);
      g[q][k] = s;
      for (int i = 0; i < 3; i++) qv[q][i] += s * v[cn[k] * 3 + i];
    }
  }
  const double E = h->mE[mi], Nu = h->mNu[mi], rho = h->mRho[mi];
  const double c = sqrt((E * (1 - Nu)) / (rho * (1 + Nu) * (1 - 2 * Nu)));
  const double V = h->weight[0] * h->detJ[IPX(h, e, 0)], cv = cbrt(V);
  const double ah = 0.25 * h->hourglass * rho * c * (cv * cv);
  for (int k = 0; k < 8; k++)
    for (int i = 0; i < 3; i++) {
      double s = 0.;
      for (int q = 0; q < 4; q++) s += g[q][k] * qv[q][i];
      fe[k * 3 + i] -= ah * s;
    }
}

/* Element::computeStress (Element.C:217-403) followed by Element::computeInternalForces
 * (Element.C:164-214) for one element; writes the element force vector to fe. */
static int elem_forces(dnlo *h, long e, double *fe)
{
  const int nip = h->nip, nen = h->nen, dim = h->dim;
  const int mi = MATOF(h, e);
  const double K = h->mE[mi] / (3. * (1. - 2. * h->mNu[mi]));
  const double G = h->mE[mi] / (2. * (1. + h->mNu[mi])); /* Material::mu(), Material.h:167-172 */
  const int yields = h->mLaw[mi] != DNLO_HARD_ELASTIC; /* Material::isYield (Material.C:366-371) */
  double pressure = 0.0;
  int err = 0;
  for (int pt = 0; pt < nip; pt++) {
    const long ix = IPX(h, e, pt);
    double F[9];
    double *dEps = h->dEps + ix * 9, *R = h->R + ix * 9;
    double *S = h->S + ix * 9, *Eps = h->Eps + ix * 9, *EpsPlas = h->EpsPlas + ix * 9;
    elem_F(h, e, pt, F);
    int pe = polar_ln_u(F, dEps, R);
    if (pe) err = pe;
    for (int k = 0; k < 9; k++) Eps[k] += dEps[k];
    pressure += (dEps[0] + dEps[4] + dEps[8]);
    {
      const double tr = (dEps[0] + dEps[4] + dEps[8]) / 3.0; /* Tensor2::deviator, :543-560 */
      double dev[9];
      for (int k = 0; k < 9; k++) dev[k] = dEps[k];
      dev[0] = dEps[0] - tr;
      dev[4] = dEps[4] - tr;
      dev[8] = dEps[8] - tr;
      const double g2 = 2.0 * G;
      for (int k = 0; k < 9; k++) S[k] += g2 * dev[k];
    }
    double gamma = 0.0, h_ = 0.0;
    if (yields) {
      const double Sigv0 = yield_stress(h, mi, h->evp[ix], 0.0);
      double ss = 0.;
      for (int k = 0; k < 9; k++) ss += S[k] * S[k];
      const double Strial = DNL_SQRT32 * sqrt(ss); /* Tensor2::J2, :505-510 */
      if (Strial > Sigv0) {
        h_ = yield_hardening(h, mi, h->evp[ix], 0.0);
        const double normS = sqrt(ss); /* Tensor2::norme, :484-489 */
        gamma = (normS - DNL_SQRT23 * Sigv0) / (2.0 * G * (1.0 + (h_) / (3.0 * G)));
        double dgamma = 0, Sigv, dfun, fun;
        int run = 1, iteration = 0;
        while (run) {
          Sigv = yield_stress(h, mi, h->evp[ix], gamma);
          h_ = yield_hardening(h, mi, h->evp[ix], gamma);
          dfun = DNL_SQRT32 * 2.0 * G + DNL_SQRT23 * h_;
          fun = dfun * gamma - (Strial - Sigv + h_ * DNL_SQRT23 * gamma);
          if (ABS(fun / Sigv) > DNL_RR_PRECISION) {
            dgamma = -fun / dfun;
            if (dgamma < 0 && ABS(dgamma) > gamma) dgamma = -gamma * 0.9;
            gamma += dgamma;
          } else {
            run = 0;
          }
          iteration++;
          if (iteration > DNL_RR_MAXIT) {
            err = DNLO_ERR_RR_NOCONV;
            run = 0;
          }
        }
        double n1[9];
        double ns = 0.;
        for (int k = 0; k < 9; k++) ns += S[k] * S[k];
        const double nrm = sqrt(ns);
        for (int k = 0; k < 9; k++) n1[k] = S[k] / nrm;
        h->evp[ix] += DNL_SQRT23 * gamma;
        const double c = 2.0 * G * gamma;
        for (int k = 0; k < 9; k++) S[k] -= c * n1[k];
        for (int k = 0; k < 9; k++) EpsPlas[k] += gamma * n1[k];
      }
    }
  }
  pressure /= nip;
  for (int pt = 0; pt < nip; pt++) {
    const long ix = IPX(h, e, pt);
    double *R = h->R + ix * 9;
    double *S = h->S + ix * 9, *Eps = h->Eps + ix * 9, *EpsPlas = h->EpsPlas + ix * 9;
    h->p[ix] += K * pressure; /* under-integrated pressure (Solver.C:75, G2TR_STUDY) */
    t2_rotate(R, S);          /* RFI (Element.C:386-388) */
    t2_rotate(R, Eps);
    t2_rotate(R, EpsPlas);
    double *Sig = h->Sig + ix * 9;
    double pI[9];
    t2_identity(pI);
    for (int k = 0; k < 9; k++) pI[k] = h->p[ix] * pI[k];
    for (int k = 0; k < 9; k++) Sig[k] = S[k] + pI[k];
  }
  /* Element::computeInternalForces body */
  for (int k = 0; k < nen * dim; k++) fe[k] = 0.0;
  for (int pt = 0; pt < nip; pt++) {
    const long ix = IPX(h, e, pt);
    const double *Sig = h->Sig + ix * 9;
    double WxdJ = h->weight[pt] * h->detJ[ix];
    double R = 0.;
    if (h->etype == 0) {
      R = elem_radius(h, e, pt);
      WxdJ *= DNL_DEUXPI * R;
    }
    for (int I = 0; I < nen; I++)
      for (int i = 0; i < dim; i++)
        for (int j = 0; j < dim; j++) fe[I * dim + i] -= DN(h, e, pt, I, j) * Sig[j * 3 + i] * WxdJ;
    if (h->etype == 0)
      for (int I = 0; I < nen; I++) fe[I * dim] -= (h->Nt[pt][I] * Sig[8] / R) * WxdJ;
  }
  if (h->etype == 5) elem_hourglass(h, e, fe);
  return err;
}

/* ---------------------------------------------------------------------- domain level */
int dnlo_internal_matrices(dnlo *h, int reference)
{
  int err = 0;
  long bad = -1;
#pragma omp parallel for schedule(static) reduction(max : err)
  for (long e = 0; e < h->E; e++) {
    int r = elem_matrices(h, e, reference);
    if (r > err) err = r;
    if (r) {
#pragma omp critical
      if (bad < 0 || e < bad) bad = e;
    }
  }
  if (err) h->bad_elem = (int)bad;
  return err;
}

/* Domain::computeInternalForces (Domain.C:130-738), strategy 0 order: Fint(Id*dim+j) accumulates
 * the element vectors in ascending element order.  Fint starts at 0 (Domain.C:145-146). */
int dnlo_internal_forces(dnlo *h)
{
  const int nd = h->nen * h->dim;
  int err = 0;
  long bad = -1;
#pragma omp parallel for schedule(static) reduction(max : err)
  for (long e = 0; e < h->E; e++) {
    int r = elem_forces(h, e, h->fe + e * nd);
    if (r > err) err = r;
    if (r) {
#pragma omp critical
      if (bad < 0 || e < bad) bad = e;
    }
  }
#pragma omp parallel for schedule(static)
  for (long n = 0; n < h->N; n++)
    for (int j = 0; j < h->dim; j++) {
      double acc = 0.0;
      for (long q = h->n2e_start[n]; q < h->n2e_start[n + 1]; q++) {
        const long ent = h->n2e[q]; /* e*nen + local node */
        acc += h->fe[(ent / h->nen) * nd + (ent % h->nen) * h->dim + j];
      }
      h->fint[n * h->dim + j] = acc;
    }
  if (err) h->bad_elem = (int)bad;
  return err;
}

/* Domain::computeMassMatrix (Domain.C:948-1005) + Element::computeMassMatrix (Element.C:411-454) */
int dnlo_mass(dnlo *h)
{
  if (h->mass_done) return 0;
  const long nd = (long)h->dim * h->N;
  for (long i = 0; i < nd; i++) h->Mass[i] = 0.;
  for (long e = 0; e < h->E; e++) {
    double Me[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int pt = 0; pt < h->nip; pt++) {
      double WxdJ = h->weight[pt] * h->detJ[IPX(h, e, pt)];
      if (h->etype == 0) {
        double R = elem_radius(h, e, pt);
        WxdJ *= 2. * DNL_PI * R;
      }
      for (int i = 0; i < h->nen; i++) Me[i] += h->mRho[MATOF(h, e)] * (h->Nt[pt][i]) * WxdJ;
    }
    for (int i = 0; i < h->nen; i++) {
      long glob = h->conn[e * h->nen + i];
      for (int j = 0; j < h->dim; j++) h->Mass[glob * h->dim + j] += Me[i];
    }
  }
  h->mass_done = 1;
  for (long n = 0; n < h->N; n++) h->mass[n] = h->Mass[n * h->dim];
  return 0;
}

/* Vec3D::distance (Vec3D.h:380-430): the norm of (b - a) */
static double dist3(const double *a, const double *b)
{
  const double x = b[0] - a[0], y = b[1] - a[1], z = b[2] - a[2];
  return sqrt(x * x + y * y + z * z);
}
#define MIN2(i, j) ((i) < (j) ? (i) : (j)) /* Math.h:62 */

/* Domain::computeCourantTimeStep (Domain.C:1613-1646) with ElQua4nAx::getLength
 * (ElQua4nAx.C:131-143, also ElQua4n2D's), ElTet4n3D::getLength (ElTet4n3D.C:151-166, also
 * ElTet10n3D's) and Element::getSoundSpeed (Element.C:607-621). */
static double elem_courant(const dnlo *h, long e)
{
  const long *cn = h->conn + e * h->nen;
  const double *x0 = h->coords + cn[0] * 3, *x1 = h->coords + cn[1] * 3;
  const double *x2 = h->coords + cn[2] * 3, *x3 = h->coords + cn[3] * 3;
  double len;
  if (h->dim == 2) {
    const double x31 = x2[0] - x0[0], x24 = x1[0] - x3[0];
    const double y42 = x3[1] - x1[1], y31 = x2[1] - x0[1];
    len = ((x31 * y42 + x24 * y31) / sqrt(2. * ((x24) * (x24) + (y42) * (y42) + (x31) * (x31) + (y31) * (y31))));
  } else if (h->etype == 5) { /* centre-point volume / largest face area (half |d1 x d2|) */
    double J[3][3] = {{0., 0., 0.}, {0., 0., 0.}, {0., 0., 0.}};
    for (int k = 0; k < 8; k++)
      for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) J[r][c] += h->dNxi[0][k][c] * h->coords[cn[k] * 3 + r];
    const double V = 8. * (J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) +
                           J[0][1] * (J[1][2] * J[2][0] - J[1][0] * J[2][2]) +
                           J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]));
    static const int F[6][4] = {{0, 1, 2, 3}, {4, 5, 6, 7}, {0, 1, 5, 4}, {1, 2, 6, 5}, {2, 3, 7, 6}, {3, 0, 4, 7}};
    double a2max = 0.;
    for (int f = 0; f < 6; f++) {
      double d1[3], d2[3];
      for (int i = 0; i < 3; i++) {
        d1[i] = h->coords[cn[F[f][2]] * 3 + i] - h->coords[cn[F[f][0]] * 3 + i];
        d2[i] = h->coords[cn[F[f][3]] * 3 + i] - h->coords[cn[F[f][1]] * 3 + i];
      }
      const double c0 = d1[1] * d2[2] - d1[2] * d2[1], c1 = d1[2] * d2[0] - d1[0] * d2[2];
      const double c2 = d1[0] * d2[1] - d1[1] * d2[0];
      const double a2 = c0 * c0 + c1 * c1 + c2 * c2;
      if (a2 > a2max) a2max = a2;
    }
    len = V / (0.5 * sqrt(a2max));
  } else {
    const double l1 = dist3(x0, x1), l2 = dist3(x0, x2), l3 = dist3(x1, x2);
    const double l4 = dist3(x0, x3), l5 = dist3(x1, x3), l6 = dist3(x2, x3);
    len = MIN2(l1, l2);
    len = MIN2(len, l3);
    len = MIN2(len, l4);
    len = MIN2(len, l5);
    len = MIN2(len, l6);
  }
  const double *ro = h->ro[h->cur];
  double r = 0.;
  for (int i = 0; i < h->nen; i++) r += ro[cn[i]];
  r /= h->nen;
  const double E = h->mE[MATOF(h, e)], Nu = h->mNu[MATOF(h, e)];
  const double Cs = sqrt((E * (1 - Nu)) / (r * (1 + Nu) * (1 - 2 * Nu)));
  return len / (Cs);
}

double dnlo_courant(dnlo *h)
{
  double crit = elem_courant(h, 0);
#pragma omp parallel for schedule(static) reduction(min : crit)
  for (long e = 1; e < h->E; e++) {
    double t = elem_courant(h, e);
    if (t < crit) crit = t;
  }
  return crit;
}

/* Element2D::computeElasticStiffnessMatrix (Element2D.C:129-226) and Element3D's
 * (Element3D.C:242-333), full integration, with Material::getHookeMatrix (Material.C:270-331):
 * the axisymmetric 4x4, the plane-strain 3x3 (its upper-left block) or the 3D 6x6.
 * Ke is row-major (nd x nd). */
static void elem_stiffness(const dnlo *h, long e, double *Ke)
{
  const int nen = h->nen, dim = h->dim, nd = nen * dim;
  const double Nu = h->mNu[MATOF(h, e)], E = h->mE[MATOF(h, e)];
  double C[6][6];
  memset(C, 0, sizeof C);
  const int axi = h->etype == 0;
  if (h->dim == 2) {
    C[0][0] = 1; C[1][1] = 1;
    C[1][0] = Nu / (1. - Nu); C[0][1] = Nu / (1. - Nu);
    if (axi) {
      C[3][3] = 1;
      C[3][0] = Nu / (1. - Nu); C[3][1] = Nu / (1. - Nu);
      C[0][3] = Nu / (1. - Nu); C[1][3] = Nu / (1. - Nu);
    }
    C[2][2] = (1.0 - 2.0 * Nu) / (2. * (1.0 - Nu));
    const double f = (E * (1.0 - Nu) / ((1.0 + Nu) * (1.0 - 2.0 * Nu)));
    for (int i = 0; i < 4; i++)
      for (int j = 0; j < 4; j++) C[i][j] *= f;
  } else {
    C[0][0] = 1; C[1][1] = 1; C[2][2] = 1;
    C[3][3] = (1.0 - 2.0 * Nu) / (2. * (1.0 - Nu));
    C[4][4] = (1.0 - 2.0 * Nu) / (2. * (1.0 - Nu));
    C[5][5] = (1.0 - 2.0 * Nu) / (2. * (1.0 - Nu));
    C[0][1] = C[1][0] = Nu / (1. - Nu);
    C[0][2] = C[2][0] = Nu / (1. - Nu);
    C[1][2] = C[2][1] = Nu / (1. - Nu);
    const double f = (E * (1.0 - Nu) / ((1.0 + Nu) * (1.0 - 2.0 * Nu)));
    for (int i = 0; i < 6; i++)
      for (int j = 0; j < 6; j++) C[i][j] *= f;
  }
  for (int k = 0; k < nd * nd; k++) Ke[k] = 0;
  double CB[6][30];
  for (int pt = 0; pt < h->nip; pt++) {
    const long ix = IPX(h, e, pt);
    double WxdJ = h->weight[pt] * h->detJ[ix];
    double R = 0.;
    if (h->dim == 2) {
      if (axi) {
        R = elem_radius(h, e, pt);
        WxdJ *= 2 * DNL_PI * R;
      }
      for (int i = 0; i < 4; i++) {
        const int I = 2 * i;
        const double d0 = DN(h, e, pt, i, 0), d1 = DN(h, e, pt, i, 1), Ni = h->Nt[pt][i];
        CB[0][I] = (C[0][0] * d0 + C[0][2] * d1);
        CB[1][I] = (C[1][0] * d0 + C[1][2] * d1);
        CB[2][I] = (C[2][0] * d0 + C[2][2] * d1);
        CB[0][I + 1] = (C[0][1] * d1 + C[0][2] * d0);
        CB[1][I + 1] = (C[1][1] * d1 + C[1][2] * d0);
        CB[2][I + 1] = (C[2][1] * d1 + C[2][2] * d0);
        if (!axi) continue;
        CB[3][I] = (C[3][0] * d0 + C[3][2] * d1);
        CB[3][I + 1] = (C[3][1] * d1 + C[3][2] * d0);
        CB[0][I] += C[0][3] * Ni / R;
        CB[1][I] += C[1][3] * Ni / R;
        CB[2][I] += C[2][3] * Ni / R;
        CB[3][I] += C[3][3] * Ni / R;
      }
      for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
          const int I = 2 * i, J = 2 * j;
          const double d0 = DN(h, e, pt, i, 0), d1 = DN(h, e, pt, i, 1), Ni = h->Nt[pt][i];
          Ke[I * nd + J] += (d0 * CB[0][J] + d1 * CB[2][J]) * WxdJ;
          Ke[I * nd + J + 1] += (d0 * CB[0][J + 1] + d1 * CB[2][J + 1]) * WxdJ;
          Ke[(I + 1) * nd + J] += (d1 * CB[1][J] + d0 * CB[2][J]) * WxdJ;
          Ke[(I + 1) * nd + J + 1] += (d1 * CB[1][J + 1] + d0 * CB[2][J + 1]) * WxdJ;
          if (!axi) continue;
          Ke[I * nd + J] += CB[3][J] * Ni / R * WxdJ;
          Ke[I * nd + J + 1] += CB[3][J + 1] * Ni / R * WxdJ;
        }
    } else {
      for (int i = 0; i < nen; i++) {
        const int I = 3 * i;
        const double d0 = DN(h, e, pt, i, 0), d1 = DN(h, e, pt, i, 1), d2 = DN(h, e, pt, i, 2);
        for (int r = 0; r < 6; r++) {
          CB[r][I] = (C[r][0] * d0 + C[r][3] * d1 + C[r][5] * d2);
          CB[r][I + 1] = (C[r][1] * d1 + C[r][3] * d0 + C[r][4] * d2);
          CB[r][I + 2] = (C[r][2] * d2 + C[r][4] * d1 + C[r][5] * d0);
        }
      }
      for (int i = 0; i < nen; i++)
        for (int j = 0; j < nen; j++) {
          const int I = 3 * i, J = 3 * j;
          const double d0 = DN(h, e, pt, i, 0), d1 = DN(h, e, pt, i, 1), d2 = DN(h, e, pt, i, 2);
          for (int c = 0; c < 3; c++) {
            Ke[I * nd + J + c] += (d0 * CB[0][J + c] + d1 * CB[3][J + c] + d2 * CB[5][J + c]) * WxdJ;
            Ke[(I + 1) * nd + J + c] += (d1 * CB[1][J + c] + d0 * CB[3][J + c] + d2 * CB[4][J + c]) * WxdJ;
            Ke[(I + 2) * nd + J + c] += (d2 * CB[2][J + c] + d1 * CB[4][J + c] + d0 * CB[5][J + c]) * WxdJ;
          }
        }
    }
  }
}

/* Domain::getMaximumFrequency (Domain.C:817-945): power iteration on M^-1 K, warm-started from the
 * previous call's vector and fmax0 (Domain members). Returns sqrt(fmax). */
int dnlo_max_frequency(dnlo *h, double *out)
{
  const int nd = h->nen * h->dim;
  const long noddl = (long)h->dim * h->N;
#pragma omp parallel for schedule(static)
  for (long e = 0; e < h->E; e++) elem_stiffness(h, e, h->Ke + e * (long)nd * nd);
  if (h->fmax0 == 0) {
    h->EV[0] = 1.0;
    for (long i = 1; i < noddl; i++) h->EV[i] = h->EV[i - 1] - 2. / (noddl - 1);
  }
  int iteration = 0, ok = 0;
  double fmax = 0.0;
  double *EV0 = (double *)malloc(sizeof(double) * noddl);
  while (!ok) {
    iteration++;
    memcpy(EV0, h->EV, sizeof(double) * noddl);
#pragma omp parallel for schedule(static)
    for (long e = 0; e < h->E; e++) {
      const double *Ke = h->Ke + e * (long)nd * nd;
      const long *cn = h->conn + e * h->nen;
      double loc[30];
      for (int I = 0; I < h->nen; I++)
        for (int j = 0; j < h->dim; j++) loc[I * h->dim + j] = 0. + EV0[cn[I] * h->dim + j];
      double *y = h->kx + e * nd; /* dgemv: y = sum_j Ke(:,j) loc_j, skipping loc_j == 0 */
      for (int i = 0; i < nd; i++) y[i] = 0.;
      for (int j = 0; j < nd; j++)
        if (loc[j] != 0.) {
          const double temp = 1.0 * loc[j];
          for (int i = 0; i < nd; i++) y[i] += temp * Ke[i * nd + j];
        }
    }
    double fm = 0.0;
#pragma omp parallel for schedule(static) reduction(max : fm)
    for (long n = 0; n < h->N; n++)
      for (int j = 0; j < h->dim; j++) {
        double val = 0.0;
        for (long q = h->n2e_start[n]; q < h->n2e_start[n + 1]; q++) {
          const long ent = h->n2e[q];
          val += h->kx[(ent / h->nen) * nd + (ent % h->nen) * h->dim + j];
        }
        val /= h->Mass[n * h->dim + j];
        if (fabs(val) > fm) fm = fabs(val);
        h->EV[n * h->dim + j] = val;
      }
    fmax = fm;
    for (long i = 0; i < noddl; i++) h->EV[i] /= fmax;
    const double convergence = ABS(fmax - h->fmax0) / fmax;
    if (convergence < DNL_PULSE_CONV) ok = 1;
    h->fmax0 = fmax;
    if (iteration > DNL_PULSE_MAXIT) {
      free(EV0);
      return DNLO_ERR_PULSE_NOCONV;
    }
  }
  free(EV0);
  h->pulse_iter = iteration;
  h->pulse_total += iteration;
  *out = sqrt(fmax);
  return 0;
}

/* Solver::computeTimeStep (Solver.C:220-267) */
int dnlo_time_step(dnlo *h, int force)
{
  if (force || (h->increment % h->freq == 0)) {
    double fmax = 0;
    if (h->method == 0) {
      fmax = 2.0 / dnlo_courant(h);
    } else {
      int r = dnlo_max_frequency(h, &fmax);
      if (r) return r;
    }
    h->timeStep = h->safety * h->omegaS / fmax;
    h->lastTsDate = h->tsDate;
    h->lastTimeStep = h->computedTimeStep;
    h->tsDate = h->currentTime;
    h->computedTimeStep = h->timeStep;
  } else {
    if (h->tsDate != h->lastTsDate) {
      const double dx = (h->currentTime - h->lastTsDate) / (h->tsDate - h->lastTsDate);
      h->timeStep = ((dx) * (h->computedTimeStep) + (1.0 - (dx)) * (h->lastTimeStep)); /* LINEARdbl */
    }
  }
  if (!(h->timeStep > 0) || !isfinite(h->timeStep)) return DNLO_ERR_DT;
  return 0;
}

/* BoundaryCondition::applyConstant (Boundary.C:200-214) -> BoundaryRestrain::applyConstant
 * (Boundary.C:636-665) / BoundarySpeed::applyConstant with constant speed (Boundary.C:478-525). */
static void apply_bc(dnlo *h, long n)
{
  double *cdu = h->fld[h->cur][0] + n * 3, *cv = h->fld[h->cur][1] + n * 3, *ca = h->fld[h->cur][2] + n * 3;
  double *ndu = h->fld[1 - h->cur][0] + n * 3, *nv = h->fld[1 - h->cur][1] + n * 3, *na = h->fld[1 - h->cur][2] + n * 3;
  for (long q = h->bcn_start[n]; q < h->bcn_start[n + 1]; q++) {
    const double *val = h->bcn_val + q * 3;
    if (h->bcn_kind[q] == 0) {
      for (int i = 0; i < 3; i++)
        if (val[i] == 1.) {
          cdu[i] = 0.; ndu[i] = 0.;
          cv[i] = 0.; nv[i] = 0.;
          ca[i] = 0.; na[i] = 0.;
        }
    } else {
      for (int i = 0; i < 3; i++)
        if (val[i] != 0.) {
          ca[i] = 0.; na[i] = 0.;
          cv[i] = val[i]; nv[i] = val[i];
          cdu[i] = cv[i] * h->timeStep;
          ndu[i] = nv[i] * h->timeStep;
        }
    }
  }
}

/* ExplicitSolverCH::computePredictions (ExplicitSolverCH.C:387-431) */
static void predictions(dnlo *h)
{
  const double dt = h->timeStep;
  const double c1 = dt * (0.5 - h->beta), c2 = dt * (1 - h->gamma);
#pragma omp parallel for schedule(static)
  for (long n = 0; n < h->N; n++) {
    double *cdu = h->fld[h->cur][0] + n * 3, *cv = h->fld[h->cur][1] + n * 3;
    double *ca = h->fld[h->cur][2] + n * 3, *cd = h->fld[h->cur][3] + n * 3;
    double *ndu = h->fld[1 - h->cur][0] + n * 3, *nv = h->fld[1 - h->cur][1] + n * 3;
    double *na = h->fld[1 - h->cur][2] + n * 3, *nd = h->fld[1 - h->cur][3] + n * 3;
    (void)cdu;
    for (int i = 0; i < 3; i++) {
      double du = ca[i];
      du *= c1;
      du += cv[i];
      du *= dt;
      ndu[i] = du;
      nd[i] = cd[i] + ndu[i];
      double v = ca[i];
      v *= c2;
      v += cv[i];
      nv[i] = v;
      na[i] = 0.0;
    }
    apply_bc(h, n);
  }
}

/* ExplicitSolverCH::explicitSolve (ExplicitSolverCH.C:490-545) + updateGrid (:555-567) with
 * lagMotion::updateNode (lagMotion.C:52-57); MatrixDiag::Solve is Fint(i) / Mass(i). */
static void explicit_solve(dnlo *h)
{
  const double dt = h->timeStep;
  const double cg = dt * h->gamma, cb = (dt * dt) * h->beta;
#pragma omp parallel for schedule(static)
  for (long n = 0; n < h->N; n++) {
    double *ca = h->fld[h->cur][2] + n * 3, *cd = h->fld[h->cur][3] + n * 3;
    double *ndu = h->fld[1 - h->cur][0] + n * 3, *nv = h->fld[1 - h->cur][1] + n * 3;
    double *na = h->fld[1 - h->cur][2] + n * 3, *nd = h->fld[1 - h->cur][3] + n * 3;
    for (int j = 0; j < h->dim; j++) na[j] = h->fint[n * h->dim + j] / h->Mass[n * h->dim + j];
    for (int i = 0; i < 3; i++) {
      na[i] -= h->alphaM * ca[i];
      na[i] /= (1.0 - h->alphaM);
      nv[i] += cg * na[i];
      ndu[i] += cb * na[i];
    }
    apply_bc(h, n);
    for (int i = 0; i < 3; i++) nd[i] = cd[i] + ndu[i];
    for (int i = 0; i < 3; i++) h->coords[n * 3 + i] += ndu[i];
  }
}

/* ExplicitSolverCH::solve prologue (ExplicitSolverCH.C:115-172) */
int dnlo_prologue(dnlo *h)
{
  int r;
  h->upTime = h->tend;
  if ((r = dnlo_internal_matrices(h, 0))) return r;
  dnlo_mass(h);
  if ((r = dnlo_internal_forces(h))) return r;
  return dnlo_time_step(h, 1);
}

/* One pass of the ExplicitSolverCH::solve loop (ExplicitSolverCH.C:179-274) per step; stops at
 * the end time (Solver::betweenTimeBounds, Solver.C:151-159). */
int dnlo_steps(dnlo *h, long nsteps, long *done)
{
  long k = 0;
  int r = 0;
  const double up = h->upTime;
  while (k < nsteps) {
    if (!(h->currentTime >= h->startTime && h->currentTime < (h->tend < up ? h->tend : up))) break;
    if (h->currentTime + h->timeStep > up) h->timeStep = up - h->currentTime; /* initStep */
    h->nextTime = h->currentTime + h->timeStep;
    h->increment++;
    predictions(h);
    if ((r = dnlo_internal_forces(h))) break;
    explicit_solve(h);
    h->currentTime += h->timeStep; /* endStep: updateTime, then swap New/Current */
    h->cur = 1 - h->cur;
    k++;
    if (h->currentTime >= h->startTime && h->currentTime < (h->tend < up ? h->tend : up)) {
      if ((r = dnlo_internal_matrices(h, 0))) break;
      if ((r = dnlo_time_step(h, 0))) break;
    }
  }
  if (done) *done = k;
  return r;
}

/* ---------------------------------------------------------------------- creation / access */
static double *zalloc(long n)
{
  double *p = (double *)calloc((size_t)(n > 0 ? n : 1), sizeof(double));
  return p;
}

dnlo *dnlo_create(int etype, long N, long E, const double *coords, const long *conn,
                  const double *mat, const double *v0, long nbc, const long *bc_kind,
                  const double *bc_val, const long *bc_start, const long *bc_nodes,
                  const double *solver)
{
  if (etype < 0 || etype > 5 || N <= 0 || E <= 0) return NULL;
  if (etype == 5 && (int)solver[4] == 1) return NULL; /* the one-point hexahedron: Courant only */
  dnlo *h = (dnlo *)calloc(1, sizeof(dnlo));
  h->etype = etype;
  h->dim = (etype == 0 || etype == 2) ? 2 : 3;
  h->nen = (etype == 1 || etype == 5) ? 8 : (etype == 4 ? 10 : 4);
  h->nip = etype == 1 ? 8 : ((etype == 3 || etype == 5) ? 1 : 4);
  h->hourglass = 0.05;
  h->N = N;
  h->E = E;
  h->conn = (long *)malloc(sizeof(long) * E * h->nen);
  memcpy(h->conn, conn, sizeof(long) * E * h->nen);
  for (long i = 0; i < E * h->nen; i++)
    if (h->conn[i] < 0 || h->conn[i] >= N) {
      free(h->conn);
      free(h);
      return NULL;
    }
  h->coords = zalloc(N * 3);
  h->coords0 = zalloc(N * 3);
  memcpy(h->coords, coords, sizeof(double) * N * 3);
  memcpy(h->coords0, coords, sizeof(double) * N * 3);
  for (int b = 0; b < 2; b++) {
    for (int f = 0; f < 4; f++) h->fld[b][f] = zalloc(N * 3);
    h->ro[b] = zalloc(N);
  }
  h->cur = 0;
  h->mass = zalloc(N);
  h->Mass = zalloc(N * h->dim);
  h->fint = zalloc(N * h->dim);
  h->fe = zalloc(E * h->nen * h->dim);
  const long nI = E * h->nip;
  h->S = zalloc(nI * 9);
  h->Eps = zalloc(nI * 9);
  h->EpsPlas = zalloc(nI * 9);
  h->Sig = zalloc(nI * 9);
  h->dEps = zalloc(nI * 9);
  h->R = zalloc(nI * 9);
  h->p = zalloc(nI);
  h->evp = zalloc(nI);
  h->detJ = zalloc(nI);
  h->detJ0 = zalloc(nI);
  h->dN = zalloc(nI * h->nen * 3);
  for (long i = 0; i < nI; i++) h->evp[i] = 1e-10; /* IntegrationPoint::flush, IntegrationPoint.C:117 */
  h->young = mat[0]; h->nu = mat[1]; h->rho = mat[2];
  h->A = mat[3]; h->B = mat[4]; h->n = mat[5];
  h->nmat = 1;
  h->mE = zalloc(1); h->mNu = zalloc(1); h->mRho = zalloc(1); h->mP = zalloc(8);
  h->mLaw = (int *)calloc(1, sizeof(int));
  h->mTab = (long *)calloc(2, sizeof(long));
  h->tabX = zalloc(1); h->tabY = zalloc(1);
  h->mE[0] = mat[0]; h->mNu[0] = mat[1]; h->mRho[0] = mat[2];
  h->mP[0] = mat[3]; h->mP[1] = mat[4]; h->mP[2] = mat[5];
  h->elemMat = NULL;
  for (int i = 0; i < 3; i++) h->v0[i] = v0[i];
  /* Domain::initSolve: Current->ro = density (Domain.C:1076-1091); initial speed on both fields
   * (BoundarySpeed::applyInitial_V0, Boundary.C:378-385) */
  for (long n = 0; n < N; n++) {
    h->ro[0][n] = h->rho;
    for (int i = 0; i < 3; i++) {
      h->fld[0][1][n * 3 + i] = v0[i];
      h->fld[1][1][n * 3 + i] = v0[i];
    }
  }
  /* per-node BC lists in attachment order */
  h->bcn_start = (long *)calloc(N + 1, sizeof(long));
  for (long g = 0; g < nbc; g++)
    for (long q = bc_start[g]; q < bc_start[g + 1]; q++) h->bcn_start[bc_nodes[q] + 1]++;
  for (long n = 0; n < N; n++) h->bcn_start[n + 1] += h->bcn_start[n];
  const long nb = h->bcn_start[N];
  h->bcn_kind = (int *)malloc(sizeof(int) * (nb > 0 ? nb : 1));
  h->bcn_val = zalloc(nb * 3);
  long *fill = (long *)calloc(N, sizeof(long));
  for (long g = 0; g < nbc; g++)
    for (long q = bc_start[g]; q < bc_start[g + 1]; q++) {
      const long n = bc_nodes[q];
      const long at = h->bcn_start[n] + fill[n]++;
      h->bcn_kind[at] = (int)bc_kind[g];
      for (int i = 0; i < 3; i++) h->bcn_val[at * 3 + i] = bc_val[g * 3 + i];
    }
  free(fill);
  /* node -> (element, local node) in ascending element order */
  h->n2e_start = (long *)calloc(N + 1, sizeof(long));
  for (long i = 0; i < E * h->nen; i++) h->n2e_start[h->conn[i] + 1]++;
  for (long n = 0; n < N; n++) h->n2e_start[n + 1] += h->n2e_start[n];
  h->n2e = (long *)malloc(sizeof(long) * E * h->nen);
  fill = (long *)calloc(N, sizeof(long));
  for (long i = 0; i < E * h->nen; i++) {
    const long n = h->conn[i];
    h->n2e[h->n2e_start[n] + fill[n]++] = i;
  }
  free(fill);
  h->tend = solver[0];
  h->rho_b = solver[1];
  h->safety = solver[2];
  h->freq = (long)solver[3];
  h->method = (int)solver[4];
  if (h->freq < 1) h->freq = 1;
  /* ExplicitSolverCH::computeIntegrationParameters (ExplicitSolverCH.C:336-343) */
  const double rb = h->rho_b;
  h->alphaM = (2.0 * rb - 1.0) / (1.0 + rb);
  h->beta = (5.0 - 3.0 * rb) / ((1.0 + rb) * (1.0 + rb) * (2.0 - rb));
  h->gamma = 1.5 - h->alphaM;
  h->omegaS = sqrt((12.0 * pow((1 + rb), 3) * (2.0 - rb)) / (10 + 15 * rb - rb * rb + pow(rb, 3) - pow(rb, 4)));
  h->upTime = h->tend;
  h->EV = zalloc(N * h->dim);
  h->kx = zalloc(E * h->nen * h->dim);
  h->Ke = h->method == 1 ? zalloc(E * (long)(h->nen * h->dim) * (h->nen * h->dim)) : NULL;
  h->bad_elem = -1;
  build_tables(h);
  /* Domain::initSolve ends with computeInternalMatrices(True) (Domain.C:1219-1223) */
  dnlo_internal_matrices(h, 1);
  return h;
}

void dnlo_destroy(dnlo *h)
{
  if (!h) return;
  free(h->conn); free(h->coords); free(h->coords0);
  for (int b = 0; b < 2; b++) {
    for (int f = 0; f < 4; f++) free(h->fld[b][f]);
    free(h->ro[b]);
  }
  free(h->mass); free(h->Mass); free(h->fint); free(h->fe);
  free(h->S); free(h->Eps); free(h->EpsPlas); free(h->Sig); free(h->dEps); free(h->R);
  free(h->p); free(h->evp); free(h->detJ); free(h->detJ0); free(h->dN);
  free(h->bcn_start); free(h->bcn_kind); free(h->bcn_val);
  free(h->EV); free(h->kx); free(h->Ke);
  free(h->n2e_start); free(h->n2e);
  free(h->mE); free(h->mNu); free(h->mRho); free(h->mP); free(h->mLaw); free(h->mTab);
  free(h->tabX); free(h->tabY); free(h->elemMat);
  free(h);
}

/* Several materials (Structure::attachMaterialToElements per ElementSet): props is nmat x 12
 * {E, nu, rho, law, P1..P8}; material m's table (tabular law) is tab_x/tab_y[tab_start[m] ..
 * tab_start[m+1]); elem_mat gives each element's material (NULL: all material 0).  The nodal
 * density on the Current field becomes that of the last element, in element order, that holds the
 * node (Domain::initSolve, Domain.C:1073-1106).  Before the prologue. */
int dnlo_set_materials(dnlo *h, int nmat, const double *props, const long *tab_start,
                       const double *tab_x, const double *tab_y, const long *elem_mat)
{
  if (nmat < 1 || !props || h->mass_done) return DNLO_ERR_ARG;
  if (elem_mat)
    for (long e = 0; e < h->E; e++)
      if (elem_mat[e] < 0 || elem_mat[e] >= nmat) return DNLO_ERR_ARG;
  free(h->mE); free(h->mNu); free(h->mRho); free(h->mP); free(h->mLaw); free(h->mTab);
  free(h->tabX); free(h->tabY); free(h->elemMat);
  h->nmat = nmat;
  h->mE = zalloc(nmat); h->mNu = zalloc(nmat); h->mRho = zalloc(nmat); h->mP = zalloc(8 * nmat);
  h->mLaw = (int *)calloc(nmat, sizeof(int));
  h->mTab = (long *)calloc(nmat + 1, sizeof(long));
  for (int m = 0; m < nmat; m++) {
    const double *q = props + 12 * m;
    h->mE[m] = q[0]; h->mNu[m] = q[1]; h->mRho[m] = q[2];
    h->mLaw[m] = (int)q[3];
    for (int k = 0; k < 8; k++) h->mP[8 * m + k] = q[4 + k];
    h->mTab[m + 1] = tab_start ? tab_start[m + 1] : 0;
  }
  const long nt = h->mTab[nmat];
  h->tabX = zalloc(nt); h->tabY = zalloc(nt);
  for (long i = 0; i < nt; i++) {
    h->tabX[i] = tab_x[i];
    h->tabY[i] = tab_y[i];
  }
  h->elemMat = NULL;
  if (elem_mat) {
    h->elemMat = (int *)malloc(sizeof(int) * h->E);
    for (long e = 0; e < h->E; e++) h->elemMat[e] = (int)elem_mat[e];
  }
  h->young = h->mE[0]; h->nu = h->mNu[0]; h->rho = h->mRho[0];
  h->A = h->mP[0]; h->B = h->mP[1]; h->n = h->mP[2];
  for (long e = 0; e < h->E; e++)
    for (int k = 0; k < h->nen; k++) h->ro[0][h->conn[e * h->nen + k]] = h->mRho[MATOF(h, e)];
  return 0;
}

/* Initial velocities per node (BoundarySpeed::applyInitial_V0 on node sets, Boundary.C:378-385):
 * v (N x 3) on both nodal fields. */
int dnlo_set_hourglass(dnlo *h, double coefficient)
{
  h->hourglass = coefficient;
  return 0;
}

int dnlo_set_velocity(dnlo *h, const double *v)
{
  for (long n = 0; n < h->N; n++)
    for (int i = 0; i < 3; i++) h->fld[0][1][n * 3 + i] = h->fld[1][1][n * 3 + i] = v[n * 3 + i];
  return 0;
}

double *dnlo_array(dnlo *h, const char *nm, long *count)
{
  const long nI = h->E * h->nip;
  struct { const char *name; double *ptr; long n; } tab[] = {
      {"coords", h->coords, h->N * 3},
      {"coords0", h->coords0, h->N * 3},
      {"du", h->fld[h->cur][0], h->N * 3},
      {"v", h->fld[h->cur][1], h->N * 3},
      {"a", h->fld[h->cur][2], h->N * 3},
      {"disp", h->fld[h->cur][3], h->N * 3},
      {"new_du", h->fld[1 - h->cur][0], h->N * 3},
      {"new_v", h->fld[1 - h->cur][1], h->N * 3},
      {"new_a", h->fld[1 - h->cur][2], h->N * 3},
      {"new_disp", h->fld[1 - h->cur][3], h->N * 3},
      {"ro", h->ro[h->cur], h->N},
      {"mass", h->mass, h->N},
      {"Mass", h->Mass, h->N * h->dim},
      {"fint", h->fint, h->N * h->dim},
      {"S", h->S, nI * 9},
      {"Eps", h->Eps, nI * 9},
      {"EpsPlas", h->EpsPlas, nI * 9},
      {"Sig", h->Sig, nI * 9},
      {"dEps", h->dEps, nI * 9},
      {"R", h->R, nI * 9},
      {"p", h->p, nI},
      {"evp", h->evp, nI},
      {"detJ", h->detJ, nI},
      {"dN", h->dN, nI * h->nen * 3},
      {"EV", h->EV, h->N * h->dim},
  };
  for (size_t i = 0; i < sizeof tab / sizeof tab[0]; i++)
    if (!strcmp(tab[i].name, nm)) {
      if (count) *count = tab[i].n;
      return tab[i].ptr;
    }
  if (count) *count = 0;
  return NULL;
}

double dnlo_get(dnlo *h, const char *nm)
{
  if (!strcmp(nm, "time")) return h->currentTime;
  if (!strcmp(nm, "dt")) return h->timeStep;
  if (!strcmp(nm, "increment")) return (double)h->increment;
  if (!strcmp(nm, "computed_dt")) return h->computedTimeStep;
  if (!strcmp(nm, "fmax0")) return h->fmax0;
  if (!strcmp(nm, "pulse_iterations")) return (double)h->pulse_iter;
  if (!strcmp(nm, "pulse_total")) return (double)h->pulse_total;
  if (!strcmp(nm, "alphaM")) return h->alphaM;
  if (!strcmp(nm, "beta")) return h->beta;
  if (!strcmp(nm, "gamma")) return h->gamma;
  if (!strcmp(nm, "omegaS")) return h->omegaS;
  if (!strcmp(nm, "kinetic")) { /* Domain::getTotalKineticEnergy (Domain.C:1330-1344), New field */
    double energy = 0.;
    const double *v = h->fld[1 - h->cur][1];
    for (long n = 0; n < h->N; n++)
      energy += .5 * h->mass[n] * (v[n * 3] * v[n * 3] + v[n * 3 + 1] * v[n * 3 + 1] + v[n * 3 + 2] * v[n * 3 + 2]);
    return energy;
  }
  if (!strcmp(nm, "kinetic_current")) {
    double energy = 0.;
    const double *v = h->fld[h->cur][1];
    for (long n = 0; n < h->N; n++)
      energy += .5 * h->mass[n] * (v[n * 3] * v[n * 3] + v[n * 3 + 1] * v[n * 3 + 1] + v[n * 3 + 2] * v[n * 3 + 2]);
    return energy;
  }
  return NAN;
}

int dnlo_set(dnlo *h, const char *nm, double value)
{
  if (!strcmp(nm, "dt")) h->timeStep = value;
  else if (!strcmp(nm, "time")) h->currentTime = value;
  else if (!strcmp(nm, "up_time")) h->upTime = value;
  else if (!strcmp(nm, "increment")) h->increment = (long)value;
  else if (!strcmp(nm, "computed_dt")) h->computedTimeStep = value;
  else if (!strcmp(nm, "last_dt")) h->lastTimeStep = value;
  else if (!strcmp(nm, "ts_date")) h->tsDate = value;
  else if (!strcmp(nm, "last_ts_date")) h->lastTsDate = value;
  else return DNLO_ERR_ARG;
  return 0;
}

int dnlo_bad_element(dnlo *h) { return h->bad_elem; }

/* the element tables built by build_tables, for comparison with the reference's */
int dnlo_tables(int etype, double *N, double *dN)
{
  dnlo t;
  memset(&t, 0, sizeof t);
  t.etype = etype;
  t.dim = (etype == 0 || etype == 2) ? 2 : 3;
  t.nen = (etype == 1 || etype == 5) ? 8 : (etype == 4 ? 10 : 4);
  t.nip = etype == 1 ? 8 : ((etype == 3 || etype == 5) ? 1 : 4);
  build_tables(&t);
  for (int pt = 0; pt < t.nip; pt++)
    for (int k = 0; k < t.nen; k++) {
      N[pt * t.nen + k] = t.Nt[pt][k];
      for (int c = 0; c < t.dim; c++) dN[(pt * t.nen + k) * t.dim + c] = t.dNxi[pt][k][c];
    }
  return 0;
}

void dnlo_set_threads(int n)
{
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

int dnlo_get_threads(void)
{
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
