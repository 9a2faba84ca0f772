/* ElTet10n3D's tables (ElTet10n3D.C:45-72) as the compiled reference holds them, shared by the
 * primal oracle (dnl_oracle.c) and the dual-number oracle (dnl_sens.cc).  Test infrastructure only.
 *
 * At Gauss point p (0: (a,a,a), 1: (b,a,a), 2: (a,b,a), 3: (a,a,b)) the barycentric coordinate L_p
 * is b and the others a; the corner shape functions L_i (2 L_i - 1) are +-0.1, the mid-edge ones
 * 4 L_i L_j (nodes 4..9 on the edges 01 12 02 03 13 23) are (1 + sqrt 5)/10 or (3 - sqrt 5)/10.
 * The derivatives are the reference's named constants 3/sqrt5, 1/sqrt5, 4/sqrt5, 1 - 1/sqrt5 (4a)
 * and 1 + 3/sqrt5 (4b); the last two are unparenthesised macros, so where the reference negates
 * them the stored values are -1 - 1/sqrt5 and -1 + 3/sqrt5 instead of -4a and -4b. */
#ifndef DNL_TET10_TABLES_H
#define DNL_TET10_TABLES_H

#include <math.h>

static inline void dnl_tet10_tables(double Nt[][10], double dNxi[][10][3], double *weight)
{
  const double r5 = sqrt(5.0);
  const int e0[6] = {0, 1, 0, 0, 1, 2}, e1[6] = {1, 2, 2, 3, 3, 3};
  for (int p = 0; p < 4; p++) {
    weight[p] = 1.0 / 24.0;
    for (int i = 0; i < 4; i++) Nt[p][i] = i == p ? 0.1 : -0.1;
    for (int m = 0; m < 6; m++)
      Nt[p][4 + m] = (e0[m] == p || e1[m] == p) ? (1.0 + r5) / 10.0 : (3.0 - r5) / 10.0;
    for (int c = 0; c < 3; c++) {
      /* d L_0 / d xi_c = -1, d L_i / d xi_c = 1 if c == i - 1 */
      dNxi[p][0][c] = p == 0 ? -(3.0 / r5) : 1.0 / r5;
      for (int i = 1; i < 4; i++)
        dNxi[p][i][c] = c != i - 1 ? 0.0 : (p == i ? 3.0 / r5 : -(1.0 / r5));
      for (int m = 0; m < 6; m++) {
        const int A = e0[m], B = e1[m];
        const int gA = A == 0 ? -1 : (c == A - 1), gB = c == B - 1;
        double v;
        if (!gA && !gB)
          v = 0.0;
        else if (gA == -1 && gB) /* 4 (L0 - L_B) */
          v = p == 0 ? 4.0 / r5 : (p == B ? -(4.0 / r5) : 0.0);
        else if (gA == -1) /* -4 L_B, as the macro expansion evaluates it */
          v = p == B ? -1.0 + 3.0 / r5 : -1.0 - 1.0 / r5;
        else /* 4 L_B or 4 L_A */
          v = p == (gA ? B : A) ? 1.0 + 3.0 / r5 : 1.0 - 1.0 / r5;
        dNxi[p][4 + m][c] = v;
      }
    }
  }
}

#endif
