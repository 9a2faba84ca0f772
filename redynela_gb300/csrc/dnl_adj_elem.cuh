// Adjoint (reverse mode) of the element pass, included by dnl_elem.cu (it shares the shape-function
// tables).  Given the adjoints of the pass's outputs -- the assembled nodal forces (through the
// node-centric gather, each element node reads its node's adjoint force) and the integration-point
// state after the pass -- it forms the adjoints of the pass's inputs: the state before the pass,
// the coordinates and Current delta_disp of the element's nodes (per element node, summed per node
// by the reverse gather), and the derivative of the loss with respect to the hardening parameters
// A, B, n accumulated per integration point.
//
// It is the transpose of the tangent pass (dnl_sens_elem.cuh), step by step in reverse order, read
// from the record the primal pass writes (TapeLayout) and the state after the pass:
//   forces M = J^-1 Sig W, Fe_k = -sum_q dN_k(q) M(q) (+ the hoop term)   (Element.C:164-214)
//   RFI X' = R X R^T:  adj(X) = R^T adj(X') R,  adj(R) += 2 adj(X') X' R    (Element.C:386-388)
//   pressure p' = p + K mean(tr dEps) over the element's points            (Element.C:254, 351)
//   J2 return at the converged multiplier (implicit function of
//     sqrt(6) G gamma - Strial + sigma_y(evp + sqrt(2/3) gamma; A, B, n) = 0)  (Element.C:282-345)
//   trial stress S + 2 G dev(ln U), strain Eps + ln U                      (Element.C:245-260)
//   ln U, U^-1 of C = F^T F: the spectral (Daleckii-Krein) derivative is self-adjoint,
//     adj(C) = V (G o (V^T adj(ln U) V) + H o (V^T adj(U^-1) V)) V^T       (Tensor2.C:1154-1259)
//   R = F U^-1, C = F^T F, F = I + G_u J^-1 (+ u_r / R), J^-1, det J, J = sum dN/dxi x_k
// Adjoints of symmetric tensors are held as symmetric matrices G paired with a perturbation by
// the full Frobenius product sum_ij G_ij dX_ij (stored components xx yy zz xy [xz yz] of G).
// Threading as k_elem: the NIP points of an element on adjacent lanes of one warp.

template <int ET> struct AdjSlot {
  static constexpr int DIM = Elem<ET>::DIM, NIP = Elem<ET>::NIP;
  static constexpr int PER = 2 * DIM * DIM + 2;  // adj(J), adj(G_u), adj(radius), adj(vR) per point
  static constexpr int SIZE = NIP * PER;
};

template <int ET>
__device__ __forceinline__ void elem_adj(const AdjElemArgs &a, int e, int pt, bool valid, int lane,
                                         double *red)
{
  using T = Elem<ET>;
  using SH = Shape<ET>;
  using TL = TapeLayout<ET>;
  using TN = TanLayout<ET>;
  using L = IpLayout<ET>;
  constexpr int NIP = T::NIP, NEN = T::NEN, DIM = T::DIM, NS = T::NS;
  constexpr bool AXI = ET == DNL_ELQUA4NAX;
  constexpr bool TWO_D = DIM == 2;
  const long nIP = (long)a.E * NIP, ipx = (long)e * NIP + pt, N = a.N;
  const Material &m = a.mat;
  auto tp = [&](int slot) { return a.tape[(long)slot * nIP + ipx]; };
  const int I0[6] = {0, 1, 2, 0, 0, 1}, I1[6] = {0, 1, 2, 1, 2, 2};
  // (i, j) entries that are identically zero in the 2 + 1 block structure of the quads
  auto zero = [](int i, int j) { return TWO_D && ((i == 2) != (j == 2)); };
  auto symload = [&](double X[3][3], auto get) {
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) X[i][j] = 0.;
#pragma unroll
    for (int k = 0; k < NS; k++) X[I0[k]][I1[k]] = X[I1[k]][I0[k]] = get(k);
  };

  int node[NEN];
#pragma unroll
  for (int k = 0; k < NEN; k++) node[k] = __ldg(a.conn + (long)k * a.E + e);

  double Ji[DIM][DIM];
#pragma unroll
  for (int l = 0; l < DIM; l++)
#pragma unroll
    for (int c = 0; c < DIM; c++) Ji[l][c] = tp(TL::JI + l * DIM + c);
  const double detJ = tp(TL::DETJ), Rad = tp(TL::RAD);

  // ---- forces: adj(M(q))[l][i] = -sum_k dN_k(q)[l] adj(Fe_k)[i], adj(hoop) = -sum_k N_k(q) adj(Fe_k)[0]
  double Mb[DIM][DIM], hb = 0.;
#pragma unroll
  for (int l = 0; l < DIM; l++)
#pragma unroll
    for (int i = 0; i < DIM; i++) Mb[l][i] = 0.;
#pragma unroll
  for (int k = 0; k < NEN; k++) {
    double fb[DIM];
#pragma unroll
    for (int i = 0; i < DIM; i++) fb[i] = __ldg(a.fbar + (long)i * N + node[k]);
#pragma unroll
    for (int l = 0; l < DIM; l++) {
      const double d = SH::dN(pt, k, l);
#pragma unroll
      for (int i = 0; i < DIM; i++) Mb[l][i] = fma(-d, fb[i], Mb[l][i]);
    }
    if (AXI) hb = fma(-SH::N(pt, k), fb[0], hb);
  }
  double S2[3][3], E2[3][3], P2[3][3];
  symload(S2, [&](int k) { return a.ipOut[(L::S + k) * nIP + ipx]; });
  symload(E2, [&](int k) { return a.ipOut[(L::EPS + k) * nIP + ipx]; });
  symload(P2, [&](int k) { return a.ipOut[(L::EPSP + k) * nIP + ipx]; });
  const double p1 = a.ipOut[L::P * nIP + ipx];
  // M = W B, B = J^-1 Sig, Sig = S' + p' I (the point's DIM x DIM block)
  double W = weighted<ET>(detJ);
  if (AXI) W = W * (kDeuxPi * Rad);
  double Wb = 0., Jib[DIM][DIM], Sigb[DIM][DIM];
#pragma unroll
  for (int l = 0; l < DIM; l++)
#pragma unroll
    for (int i = 0; i < DIM; i++) {
      double s = 0.;
#pragma unroll
      for (int j = 0; j < DIM; j++) s = fma(Ji[l][j], i == j ? S2[j][i] + p1 : S2[j][i], s);
      Wb = fma(Mb[l][i], s, Wb);
    }
#pragma unroll
  for (int l = 0; l < DIM; l++)
#pragma unroll
    for (int j = 0; j < DIM; j++) {
      double s = 0.;
#pragma unroll
      for (int i = 0; i < DIM; i++) s = fma(Mb[l][i], i == j ? S2[j][i] + p1 : S2[j][i], s);
      Jib[l][j] = W * s;
    }
#pragma unroll
  for (int j = 0; j < DIM; j++)
#pragma unroll
    for (int i = 0; i < DIM; i++) {
      double s = 0.;
#pragma unroll
      for (int l = 0; l < DIM; l++) s = fma(Ji[l][j], Mb[l][i], s);
      Sigb[j][i] = W * s;
    }
  // adjoints of the state after the pass (symmetric adjoint of S', of p') plus the force's share
  double GS[3][3], GE[3][3], GP[3][3];
  symload(GS, [&](int k) { return a.ipAdj[(TN::S + k) * nIP + ipx]; });
  symload(GE, [&](int k) { return a.ipAdj[(TN::EPS + k) * nIP + ipx]; });
  symload(GP, [&](int k) { return a.ipAdj[(TN::EPSP + k) * nIP + ipx]; });
  double pb = a.ipAdj[TN::P * nIP + ipx];
  const double evpb = a.ipAdj[TN::EVP * nIP + ipx];
#pragma unroll
  for (int i = 0; i < DIM; i++) {
    pb += Sigb[i][i];
#pragma unroll
    for (int j = 0; j < DIM; j++) GS[i][j] = fma(0.5, Sigb[i][j] + Sigb[j][i], GS[i][j]);
  }
  double detJb = 0., Radb = 0.;
  if (AXI) {
    // hoop = (S'_tt + p') detJ 2 pi; W = detJ 2 pi R
    const double hk = hb * (detJ * kDeuxPi);
    GS[2][2] += hk;
    pb += hk;
    detJb = fma(hb * kDeuxPi, S2[2][2] + p1, fma(Wb * kDeuxPi, Rad, detJb));
    Radb = Wb * (detJ * kDeuxPi);
  } else {
    detJb = Wb * weighted<ET>(1.0);
  }

  // ---- RFI: adj(X) = R^T adj(X') R, adj(R) += 2 adj(X') X' R for S, Eps, EpsPlas
  double R[3][3], Rb[3][3];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      R[i][j] = tp(TL::R + i * 3 + j);
      Rb[i][j] = 0.;
    }
  auto rfi_adj = [&](double G[3][3], const double X2[3][3]) {
    double GX[3][3];  // adj(X') X'
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) {
        double s = 0.;
        if (!zero(i, j)) {
#pragma unroll
          for (int k = 0; k < 3; k++)
            if (!zero(i, k) && !zero(k, j)) s = fma(G[i][k], X2[k][j], s);
        }
        GX[i][j] = s;
      }
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) {
        if (zero(i, j)) continue;
        double s = 0.;
#pragma unroll
        for (int k = 0; k < 3; k++)
          if (!zero(i, k) && !zero(k, j)) s = fma(GX[i][k], R[k][j], s);
        Rb[i][j] = fma(2.0, s, Rb[i][j]);
      }
    double T1[3][3];  // adj(X') R
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) {
        double s = 0.;
        if (!zero(i, j)) {
#pragma unroll
          for (int k = 0; k < 3; k++)
            if (!zero(i, k) && !zero(k, j)) s = fma(G[i][k], R[k][j], s);
        }
        T1[i][j] = s;
      }
#pragma unroll
    for (int q = 0; q < 6; q++) {
      const int i = I0[q], j = I1[q];
      double s = 0.;
      if (!zero(i, j)) {
#pragma unroll
        for (int k = 0; k < 3; k++)
          if (!zero(k, i) && !zero(k, j)) s = fma(R[k][i], T1[k][j], s);
      }
      G[i][j] = G[j][i] = s;
    }
  };
  rfi_adj(GS, S2);
  rfi_adj(GE, E2);
  rfi_adj(GP, P2);

  // ---- element-mean pressure: adj(tr dEps) of this point = K / NIP sum over the element's adj(p')
  double trb = 0.;
  {
    const int base = lane - pt;
#pragma unroll
    for (int k = 0; k < NIP; k++) trb += __shfl_sync(0xffffffffu, pb, base + k);
    trb *= m.K * (1.0 / NIP);
  }

  // ---- J2 return at the converged multiplier
  double GStr[3][3], evp0b = evpb;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) GStr[i][j] = GS[i][j];
  const double gam = tp(TL::GAM);
  double gA = 0., gB = 0., gN = 0.;
  if (gam > 0.) {
    const double normS = tp(TL::NORMS), xv = tp(TL::XV), xn = tp(TL::XN), rnorm = nr_rcp(normS);
    double nh[3][3];
    symload(nh, [&](int k) { return tp(TL::STR + k) * rnorm; });
    double gsn = 0., gpn = 0.;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) {
        gsn = fma(GS[i][j], nh[i][j], gsn);
        gpn = fma(GP[i][j], nh[i][j], gpn);
      }
    // S = Str - 2 G gamma n, EpsPlas += gamma n, evp += sqrt(2/3) gamma, n = Str / |Str|
    const double gamb = fma(-m.G2, gsn, fma(kSqrt23, evpb, gpn));
    double nb[3][3], nbn = 0.;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) {
        nb[i][j] = gam * fma(-m.G2, GS[i][j], GP[i][j]);
        nbn = fma(nb[i][j], nh[i][j], nbn);
      }
    const double h = m.nB * xn * nr_rcp(xv);  // n B xv^(n-1)
    const double D = fma(kSqrt23, h, m.dfun0);
    const double lam = gamb * nr_rcp(D);
    // d gamma = (sqrt(3/2) d|Str| - h d evp - d sigma_y / d p) / D
    const double cn = kSqrt32 * lam;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) GStr[i][j] = fma(cn, nh[i][j], fma(rnorm, fma(-nbn, nh[i][j], nb[i][j]), GS[i][j]));
    evp0b = fma(-h, lam, evpb);
    gA = -lam;
    gB = -lam * xn;
    gN = -lam * m.B * xn * tp(TL::LXV);
  }

  // ---- trial stress and strain: adj(ln U) = adj(Eps') + 2 G dev(adj(Str)) + adj(tr) I
  double GL[3][3];
  {
    const double tg = (GStr[0][0] + GStr[1][1] + GStr[2][2]) * (1.0 / 3.0);
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++)
        GL[i][j] = fma(m.G2, i == j ? GStr[i][j] - tg : GStr[i][j], GE[i][j]) + (i == j ? trb : 0.);
  }

  // ---- the state before the pass: adj(S) = adj(Str), adj(Eps) = adj(Eps'), adj(EpsPlas), p, evp
  if (valid) {
#pragma unroll
    for (int k = 0; k < NS; k++) {
      a.ipAdj[(TN::S + k) * nIP + ipx] = GStr[I0[k]][I1[k]];
      a.ipAdj[(TN::EPS + k) * nIP + ipx] = GE[I0[k]][I1[k]];
      a.ipAdj[(TN::EPSP + k) * nIP + ipx] = GP[I0[k]][I1[k]];
    }
    a.ipAdj[TN::P * nIP + ipx] = pb;
    a.ipAdj[TN::EVP * nIP + ipx] = evp0b;
    if (gam > 0.) {
      a.gpar[ipx] += gA;
      a.gpar[a.gStride + ipx] += gB;
      a.gpar[2 * a.gStride + ipx] += gN;
    }
  }

  // ---- polar decomposition: adj(U^-1) = sym(F^T adj(R)); adj(C) by the spectral formula
  double F[3][3];
#pragma unroll
  for (int k = 0; k < 9; k++) F[k / 3][k % 3] = tp(TL::F + k);
  double GU_[3][3];  // sym(F^T adj(R))
  {
    double T1[3][3];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) {
        double s = 0.;
        if (!zero(i, j)) {
#pragma unroll
          for (int k = 0; k < 3; k++)
            if (!zero(k, i) && !zero(k, j)) s = fma(F[k][i], Rb[k][j], s);
        }
        T1[i][j] = s;
      }
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) GU_[i][j] = 0.5 * (T1[i][j] + T1[j][i]);
  }
  double V[3][3];
#pragma unroll
  for (int k = 0; k < 9; k++) V[k / 3][k % 3] = tp(TL::V + k);
  double Cb[3][3];
  {
    // A = V^T G V for both adjoints, B = GD o A1 + HD o A2, adj(C) = V B V^T
    double T1[3][3], T2[3][3];  // G V
#pragma unroll
    for (int k = 0; k < 3; k++)
#pragma unroll
      for (int j = 0; j < 3; j++) {
        double s1 = 0., s2 = 0.;
#pragma unroll
        for (int l = 0; l < 3; l++)
          if (!zero(k, l) && !zero(l, j)) {
            s1 = fma(GL[k][l], V[l][j], s1);
            s2 = fma(GU_[k][l], V[l][j], s2);
          }
        T1[k][j] = s1;
        T2[k][j] = s2;
      }
    double Bm[3][3];
#pragma unroll
    for (int q = 0; q < 6; q++) {
      const int i = I0[q], j = I1[q];
      double s1 = 0., s2 = 0.;
      if (!zero(i, j)) {
#pragma unroll
        for (int k = 0; k < 3; k++)
          if (!zero(k, i) && !zero(k, j)) {
            s1 = fma(V[k][i], T1[k][j], s1);
            s2 = fma(V[k][i], T2[k][j], s2);
          }
      }
      Bm[i][j] = Bm[j][i] = fma(tp(TL::GD + q), s1, tp(TL::HD + q) * s2);
    }
    double T3[3][3];  // V B
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int l = 0; l < 3; l++) {
        double s = 0.;
#pragma unroll
        for (int k = 0; k < 3; k++)
          if (!zero(i, k) && !zero(k, l)) s = fma(V[i][k], Bm[k][l], s);
        T3[i][l] = s;
      }
#pragma unroll
    for (int q = 0; q < 6; q++) {
      const int i = I0[q], j = I1[q];
      double s = 0.;
      if (!zero(i, j)) {
#pragma unroll
        for (int l = 0; l < 3; l++)
          if (!zero(i, l) && !zero(j, l)) s = fma(T3[i][l], V[j][l], s);
      }
      Cb[i][j] = Cb[j][i] = s;
    }
  }
  // adj(F) = 2 F adj(C) + adj(R) U^-1
  double Fb[3][3];
  {
    double Ui[3][3];
#pragma unroll
    for (int q = 0; q < 6; q++) Ui[I0[q]][I1[q]] = Ui[I1[q]][I0[q]] = tp(TL::UI + q);
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) {
        double s = 0.;
        if (!zero(i, j)) {
#pragma unroll
          for (int k = 0; k < 3; k++)
            if (!zero(i, k) && !zero(k, j)) s = fma(2.0 * F[i][k], Cb[k][j], fma(Rb[i][k], Ui[k][j], s));
        }
        Fb[i][j] = s;
      }
  }

  // ---- F = I + G_u J^-1 (+ u_r / R): adj(G_u) = adj(F) J^-T, adj(J^-1) += G_u^T adj(F)
  double GUb[DIM][DIM];
  {
    double GU[DIM][DIM];
#pragma unroll
    for (int r = 0; r < DIM; r++)
#pragma unroll
      for (int l = 0; l < DIM; l++) GU[r][l] = tp(TL::GU + r * DIM + l);
#pragma unroll
    for (int r = 0; r < DIM; r++)
#pragma unroll
      for (int l = 0; l < DIM; l++) {
        double s = 0.;
#pragma unroll
        for (int c = 0; c < DIM; c++) s = fma(Fb[r][c], Ji[l][c], s);
        GUb[r][l] = s;
      }
#pragma unroll
    for (int l = 0; l < DIM; l++)
#pragma unroll
      for (int c = 0; c < DIM; c++) {
        double s = Jib[l][c];
#pragma unroll
        for (int r = 0; r < DIM; r++) s = fma(GU[r][l], Fb[r][c], s);
        Jib[l][c] = s;
      }
  }
  double vRb = 0.;
  if (AXI) {
    const double rRad = nr_rcp(Rad);
    vRb = Fb[2][2] * rRad;
    Radb = fma(-vRb, tp(TL::VRR), Radb);
  }
  // ---- J^-1 and det J: adj(J) = -J^-T adj(J^-1) J^-T + adj(detJ) detJ J^-T
  double Jb[DIM][DIM];
  {
    double T1[DIM][DIM];  // adj(J^-1) J^-T
#pragma unroll
    for (int l = 0; l < DIM; l++)
#pragma unroll
      for (int r = 0; r < DIM; r++) {
        double s = 0.;
#pragma unroll
        for (int c = 0; c < DIM; c++) s = fma(Jib[l][c], Ji[r][c], s);
        T1[l][r] = s;
      }
    const double dd = detJb * detJ;
#pragma unroll
    for (int r = 0; r < DIM; r++)
#pragma unroll
      for (int c = 0; c < DIM; c++) {
        double s = 0.;
#pragma unroll
        for (int l = 0; l < DIM; l++) s = fma(Ji[l][r], T1[l][c], s);
        Jb[r][c] = fma(dd, Ji[c][r], -s);
      }
  }

  // ---- J = sum_k dN_k/dxi x_k, G_u = sum_k dN_k/dxi du_k, R = sum N_k x_k,r, vR = sum N_k du_k,r:
  // every point's adjoints through the element's shared memory, each lane assembling its node(s)
  using AS = AdjSlot<ET>;
  double *mine = red + pt * AS::PER;
#pragma unroll
  for (int r = 0; r < DIM; r++)
#pragma unroll
    for (int c = 0; c < DIM; c++) {
      mine[r * DIM + c] = Jb[r][c];
      mine[DIM * DIM + r * DIM + c] = GUb[r][c];
    }
  mine[2 * DIM * DIM] = Radb;
  mine[2 * DIM * DIM + 1] = vRb;
  __syncwarp();
  if (!valid) return;
#pragma unroll
  for (int j = 0; j < (NEN + NIP - 1) / NIP; j++) {
    const int k = pt + j * NIP;
    if (k >= NEN) break;
    double sx[DIM], su[DIM];
#pragma unroll
    for (int r = 0; r < DIM; r++) sx[r] = su[r] = 0.;
#pragma unroll
    for (int q = 0; q < NIP; q++) {
      const double *o = red + q * AS::PER;
#pragma unroll
      for (int c = 0; c < DIM; c++) {
        const double d = SH::dN(q, k, c);
#pragma unroll
        for (int r = 0; r < DIM; r++) {
          sx[r] = fma(d, o[r * DIM + c], sx[r]);
          su[r] = fma(d, o[DIM * DIM + r * DIM + c], su[r]);
        }
      }
      if (AXI) {
        const double nk = SH::N(q, k);
        sx[0] = fma(nk, o[2 * DIM * DIM], sx[0]);
        su[0] = fma(nk, o[2 * DIM * DIM + 1], su[0]);
      }
    }
#pragma unroll
    for (int r = 0; r < DIM; r++) {
      a.xe[(long)r * a.feStride + (long)e * NEN + k] = sx[r];
      a.ue[(long)r * a.feStride + (long)e * NEN + k] = su[r];
    }
  }
}

template <int ET>
__global__ void __launch_bounds__(128) k_elem_adj(AdjElemArgs a)
{
  constexpr int NIP = Elem<ET>::NIP;
  constexpr int EPW = 32 / NIP;
  __shared__ double red[128 / 32][EPW][AdjSlot<ET>::SIZE];
  const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
  if ((gtid & ~31) / NIP >= a.E) return;
  const int eRaw = gtid / NIP;
  const bool valid = eRaw < a.E;
  const int lane = threadIdx.x & 31;
  const int e = valid ? eRaw : a.E - 1;
  elem_adj<ET>(a, e, gtid % NIP, valid, lane, red[threadIdx.x >> 5][lane / NIP]);
}

int launch_elem_adj(int etype, const AdjElemArgs &a, cudaStream_t s)
{
  if (!etype_has_sens(etype) || etype == DNL_ELHEX8N3D_1PT) return DNL_ERR_ARG;
  const long threads = (long)a.E * etype_nip(etype);
  const int grid = (int)((threads + 127) / 128);
  if (etype == DNL_ELQUA4NAX)
    k_elem_adj<DNL_ELQUA4NAX><<<grid, 128, 0, s>>>(a);
  else if (etype == DNL_ELQUA4N2D)
    k_elem_adj<DNL_ELQUA4N2D><<<grid, 128, 0, s>>>(a);
  else if (etype == DNL_ELHEX8N3D)
    k_elem_adj<DNL_ELHEX8N3D><<<grid, 128, 0, s>>>(a);
  else if (etype == DNL_ELTET4N3D)
    k_elem_adj<DNL_ELTET4N3D><<<grid, 128, 0, s>>>(a);
  else
    k_elem_adj<DNL_ELTET10N3D><<<grid, 128, 0, s>>>(a);
  launch_counter()++;
  return cudaPeekAtLastError() == cudaSuccess ? 0 : DNL_ERR_CUDA;
}

// The tape instance of the element pass on caller-built arguments (the adjoint's recomputation of
// one step's record from a saved state)
int launch_elem_tape_raw(int etype, const ElemArgs &a, cudaStream_t s)
{
  if (!etype_has_sens(etype)) return DNL_ERR_ARG;
  const long threads = (long)a.E * etype_nip(etype);
  const int grid = (int)((threads + 127) / 128);
  DNL_BY_ETYPE(etype, (k_elem<ET, true><<<grid, 128, 0, s>>>(a)));
  launch_counter()++;
  return cudaPeekAtLastError() == cudaSuccess ? 0 : DNL_ERR_CUDA;
}
