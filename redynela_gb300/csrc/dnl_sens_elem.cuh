// Tangent of the element pass: forward-mode sensitivities of one explicit step with respect to the
// hardening parameters (A, B, n) and the initial-velocity magnitude, included by dnl_elem.cu
// (it shares the shape-function tables).
//
// The primal pass (k_elem<ET, true>) records per integration point the quantities the derivative
// needs (TapeLayout); this pass reads them with the tangents of its inputs and propagates:
//   J, J^-1, det J      from the coordinate tangents          (Element2D.C:53-126, Element3D.C:53-113)
//   F = I + grad du     with the Current delta_disp tangents  (ElementAx.C:114-136, Element3D.C:182-205)
//   ln U, U^-1, R       spectral derivative at the computed eigenpairs of C = F^T F (Daleckii-Krein:
//                       d f(C) = V (F o (V^T dC V)) V^T, F_ij divided differences of f, recorded
//                       by the primal pass)                 (Tensor2.C:1154-1259)
//   trial stress, J2 return: implicit-function derivative of the converged return equation
//                       sqrt(6) G gamma - Strial + sigma_y(evp + sqrt(2/3) gamma; A, B, n) = 0
//                                                           (Element.C:245-345, IsoHardElastoplastic.C:171-184)
//   pressure, RFI rotation (d(R X R^T) = R dX R^T + Omega X' + (Omega X')^T, Omega = dR R^T,
//   X' the rotated state the primal pass stored), B^T sigma  (Element.C:164-214, 351-401)
// Work that does not depend on the parameter (the divided differences, U^-1, G_u) is formed once
// per point by the primal pass; in the axisymmetric case the 2 + 1 block structure of F, C, V, R
// skips the identically zero entries.
// Threading: NIP adjacent lanes per (element, direction) group, the four directions of an element
// in consecutive groups, so the pressure average and the force sum stay warp-local as in k_elem.

template <int ET>
__device__ __forceinline__ void elem_tan(const SensElemArgs &a, int e, int dir, int pt, bool valid,
                                         int lane, double *red)
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
  const Material &m = a.elemInst ? a.mats[a.elemInst[e]] : a.mat;
  auto tp = [&](int slot) { return a.tape[(long)slot * nIP + ipx]; };
  const double *tx = a.tx + (long)dir * 3 * N, *tdu = a.tdu + (long)dir * 3 * N;
  double *tip = a.tip + (long)dir * TN::NCOMP * nIP;
  const int I0[6] = {0, 1, 2, 0, 0, 1}, I1[6] = {0, 1, 2, 1, 2, 2};
  // (i, j) entries that are identically zero in the axisymmetric block structure (2 + 1)
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

  // ---- dJ, dRad from the coordinate tangents; the tangent of G_u from the Current du tangents
  double dJ[DIM][DIM], GT[DIM][DIM], dRad = 0., dvR = 0.;
#pragma unroll
  for (int r = 0; r < DIM; r++)
#pragma unroll
    for (int c = 0; c < DIM; c++) dJ[r][c] = GT[r][c] = 0.;
  constexpr bool EDGES = ET == DNL_ELHEX8N3D || ET == DNL_ELQUA4NAX || ET == DNL_ELQUA4N2D;
  if constexpr (EDGES) {
    // the group's edge differences of the tangents, a few per lane, through its shared memory
    // (as the primal pass's J and G_u)
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
          ex[eg * DIM + r] = tx[(long)r * N + hi] - tx[(long)r * N + lo];
          eu[eg * DIM + r] = tdu[(long)r * N + hi] - tdu[(long)r * N + lo];
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
          dJ[r][c] = fma(w, ex[eg * DIM + r], dJ[r][c]);
          GT[r][c] = fma(w, eu[eg * DIM + r], GT[r][c]);
        }
      }
    __syncwarp();  // the force assembly reuses the buffer
    if (AXI) {
#pragma unroll
      for (int k = 0; k < NEN; k++) {
        dRad = fma(SH::N(pt, k), tx[node[k]], dRad);
        dvR = fma(SH::N(pt, k), tdu[node[k]], dvR);
      }
    }
  } else {
#pragma unroll
  for (int k = 0; k < NEN; k++) {
    double t[DIM], tu[DIM];
#pragma unroll
    for (int r = 0; r < DIM; r++) {
      t[r] = tx[(long)r * N + node[k]];
      tu[r] = tdu[(long)r * N + node[k]];
    }
#pragma unroll
    for (int r = 0; r < DIM; r++)
#pragma unroll
      for (int c = 0; c < DIM; c++) {
        const double d = SH::dN(pt, k, c);
        dJ[r][c] = fma(d, t[r], dJ[r][c]);
        GT[r][c] = fma(d, tu[r], GT[r][c]);
      }
    if (AXI) {
      dRad = fma(SH::N(pt, k), t[0], dRad);
      dvR = fma(SH::N(pt, k), tu[0], dvR);
    }
  }
  }
  // ---- dJ^-1 = -J^-1 dJ J^-1, d det J = det J tr(J^-1 dJ)
  double Ji[DIM][DIM];
#pragma unroll
  for (int l = 0; l < DIM; l++)
#pragma unroll
    for (int c = 0; c < DIM; c++) Ji[l][c] = tp(TL::JI + l * DIM + c);
  const double detJ = tp(TL::DETJ), Rad = tp(TL::RAD);
  double JdJ[DIM][DIM], dJi[DIM][DIM];
#pragma unroll
  for (int l = 0; l < DIM; l++)
#pragma unroll
    for (int c = 0; c < DIM; c++) {
      double s = 0.;
#pragma unroll
      for (int r = 0; r < DIM; r++) s = fma(Ji[l][r], dJ[r][c], s);
      JdJ[l][c] = s;
    }
  double trJ = 0.;
#pragma unroll
  for (int l = 0; l < DIM; l++) {
    trJ += JdJ[l][l];
#pragma unroll
    for (int c = 0; c < DIM; c++) {
      double s = 0.;
#pragma unroll
      for (int q = 0; q < DIM; q++) s = fma(JdJ[l][q], Ji[q][c], s);
      dJi[l][c] = -s;
    }
  }
  const double ddetJ = detJ * trJ;

  // ---- dF = d(G_u J^-1) = G_t J^-1 + G_u dJ^-1  (F - I = G_u J^-1); axisymmetric hoop term
  double F[3][3], dF[3][3];
#pragma unroll
  for (int k = 0; k < 9; k++) {
    F[k / 3][k % 3] = tp(TL::F + k);
    dF[k / 3][k % 3] = 0.;
  }
  {
    double GU[DIM][DIM];
#pragma unroll
    for (int r = 0; r < DIM; r++)
#pragma unroll
      for (int l = 0; l < DIM; l++) GU[r][l] = tp(TL::GU + r * DIM + l);
#pragma unroll
    for (int r = 0; r < DIM; r++)
#pragma unroll
      for (int c = 0; c < DIM; c++) {
        double s = 0.;
#pragma unroll
        for (int l = 0; l < DIM; l++) s = fma(GT[r][l], Ji[l][c], fma(GU[r][l], dJi[l][c], s));
        dF[r][c] = s;
      }
  }
  const double rRad = AXI ? nr_rcp(Rad) : 0.;  // tangents need no correctly rounded quotients
  if (AXI) dF[2][2] = fma(-tp(TL::VRR), dRad, dvR) * rRad;

  // ---- dC = dF^T F + F^T dF (symmetric)
  double dC[3][3];
#pragma unroll
  for (int q = 0; q < 6; q++) {
    const int i = I0[q], j = I1[q];
    double s = 0.;
    if (!zero(i, j)) {
#pragma unroll
      for (int k = 0; k < 3; k++)
        if (!zero(k, i) && !zero(k, j)) s = fma(dF[k][i], F[k][j], fma(F[k][i], dF[k][j], s));
    }
    dC[i][j] = dC[j][i] = s;
  }
  // ---- spectral derivative: Ah = V^T dC V; d ln U = V (G o Ah) V^T; d U^-1 = V (H o Ah) V^T
  double V[3][3];
#pragma unroll
  for (int k = 0; k < 9; k++) V[k / 3][k % 3] = tp(TL::V + k);
  double Bg[3][3], Bh[3][3];
  {
    double T1[3][3];
#pragma unroll
    for (int k = 0; k < 3; k++)
#pragma unroll
      for (int j = 0; j < 3; j++) {
        double s = 0.;
#pragma unroll
        for (int l = 0; l < 3; l++)
          if (!zero(k, l) && !zero(l, j)) s = fma(dC[k][l], V[l][j], s);
        T1[k][j] = s;
      }
#pragma unroll
    for (int q = 0; q < 6; q++) {
      const int i = I0[q], j = I1[q];
      double s = 0.;
      if (!zero(i, j)) {
#pragma unroll
        for (int k = 0; k < 3; k++)
          if (!zero(k, i) && !zero(k, j)) s = fma(V[k][i], T1[k][j], s);
      }
      Bg[i][j] = Bg[j][i] = tp(TL::GD + q) * s;
      Bh[i][j] = Bh[j][i] = tp(TL::HD + q) * s;
    }
  }
  double dLn[3][3], dUi[3][3];
  {
    double Tg[3][3], Th[3][3];  // V B
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int l = 0; l < 3; l++) {
        double sg = 0., sh = 0.;
#pragma unroll
        for (int k = 0; k < 3; k++)
          if (!zero(i, k) && !zero(k, l)) {
            sg = fma(V[i][k], Bg[k][l], sg);
            sh = fma(V[i][k], Bh[k][l], sh);
          }
        Tg[i][l] = sg;
        Th[i][l] = sh;
      }
#pragma unroll
    for (int q = 0; q < 6; q++) {
      const int i = I0[q], j = I1[q];
      double sg = 0., sh = 0.;
      if (!zero(i, j)) {
#pragma unroll
        for (int l = 0; l < 3; l++)
          if (!zero(i, l) && !zero(j, l)) {
            sg = fma(Tg[i][l], V[j][l], sg);
            sh = fma(Th[i][l], V[j][l], sh);
          }
      }
      dLn[i][j] = dLn[j][i] = sg;
      dUi[i][j] = dUi[j][i] = sh;
    }
  }
  // ---- dR = dF U^-1 + F dU^-1, and Omega = dR R^T
  double R[3][3], Om[3][3];
  {
    double Ui[3][3], dR[3][3];
#pragma unroll
    for (int q = 0; q < 6; q++) Ui[I0[q]][I1[q]] = Ui[I1[q]][I0[q]] = tp(TL::UI + q);
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) {
        R[i][j] = tp(TL::R + i * 3 + j);
        double s = 0.;
        if (!zero(i, j)) {
#pragma unroll
          for (int k = 0; k < 3; k++)
            if (!zero(i, k) && !zero(k, j)) s = fma(dF[i][k], Ui[k][j], fma(F[i][k], dUi[k][j], s));
        }
        dR[i][j] = s;
      }
    // Omega = dR R^T is skew (R R^T = I): its upper entries (and, in 2D, Omega_22) suffice
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) Om[i][j] = 0.;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = i; j < 3; j++) {
        if (zero(i, j) || (i == j && !(TWO_D && i == 2))) continue;
        double s = 0.;
#pragma unroll
        for (int k = 0; k < 3; k++)
          if (!zero(i, k) && !zero(j, k)) s = fma(dR[i][k], R[j][k], s);
        Om[i][j] = s;
        if (i != j) Om[j][i] = -s;
      }
  }

  // ---- strain, trial stress
  double dS[3][3], dE[3][3], dP[3][3];
  symload(dS, [&](int k) { return tip[(TN::S + k) * nIP + ipx]; });
  symload(dE, [&](int k) { return tip[(TN::EPS + k) * nIP + ipx]; });
  symload(dP, [&](int k) { return tip[(TN::EPSP + k) * nIP + ipx]; });
  const double dp0 = tip[TN::P * nIP + ipx], devp0 = tip[TN::EVP * nIP + ipx];
  const double dtr = dLn[0][0] + dLn[1][1] + dLn[2][2];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      dE[i][j] += dLn[i][j];
      dS[i][j] = fma(m.G2, i == j ? fma(-dtr, 1. / 3., dLn[i][j]) : dLn[i][j], dS[i][j]);
    }

  // ---- J2 return: d gamma from the converged return equation
  double devp = devp0;
  const double gam = tp(TL::GAM);
  if (gam > 0.) {
    const double normS = tp(TL::NORMS), xv = tp(TL::XV), xn = tp(TL::XN), rnorm = nr_rcp(normS);
    double nh[3][3];
    symload(nh, [&](int k) { return tp(TL::STR + k) * rnorm; });
    double dnorm = 0.;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) dnorm = fma(nh[i][j], dS[i][j], dnorm);
    const double h = m.nB * xn * nr_rcp(xv);  // n B xv^(n-1)
    const double D = fma(kSqrt23, h, m.dfun0);
    const double dsig = dir == 0 ? 1. : (dir == 1 ? xn : (dir == 2 ? m.B * xn * tp(TL::LXV) : 0.));
    const double dgam = fma(kSqrt32, dnorm, -fma(h, devp0, dsig)) * nr_rcp(D);
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) {
        if (zero(i, j)) continue;
        const double dn = fma(-nh[i][j], dnorm, dS[i][j]) * rnorm;
        const double dflow = fma(dgam, nh[i][j], gam * dn);
        dS[i][j] = fma(-m.G2, dflow, dS[i][j]);
        dP[i][j] += dflow;
      }
    devp = fma(kSqrt23, dgam, devp0);
  }

  // ---- element-mean pressure
  double dpres = 0.;
  {
    const int base = lane - pt;
#pragma unroll
    for (int k = 0; k < NIP; k++) dpres += __shfl_sync(0xffffffffu, dtr, base + k);
    dpres *= 1.0 / NIP;
  }
  const double dpn = fma(m.K, dpres, dp0);

  // ---- RFI: X' = R X R^T, d X' = R dX R^T + Omega X' + (Omega X')^T (R^T R = I), with X' the
  // rotated state the primal pass stored
  auto rfi_t = [&](int comp, double dX[3][3]) {
    double Xp[3][3];
    symload(Xp, [&](int k) { return a.ip[(comp + k) * nIP + ipx]; });
    if (comp == L::EPSP) {  // a point that never yielded: EpsPlas and its tangent are 0
      unsigned long long nz = 0;
#pragma unroll
      for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = i; j < 3; j++) nz |= abits(Xp[i][j]) | abits(dX[i][j]);
      if (!nz) return;
    }
    if constexpr (TWO_D) {
      // Omega = dR R^T is skew (R R^T = I): in the block one rate w, so Omega X' + (Omega X')^T is
      // 2 w X'01 on the diagonal and w (X'11 - X'00) off it; R dX R^T by two 2x2 products
      const double w = 0.5 * (Om[0][1] - Om[1][0]);
      const double t00 = fma(dX[0][0], R[0][0], dX[0][1] * R[0][1]);
      const double t01 = fma(dX[0][0], R[1][0], dX[0][1] * R[1][1]);
      const double t10 = fma(dX[1][0], R[0][0], dX[1][1] * R[0][1]);
      const double t11 = fma(dX[1][0], R[1][0], dX[1][1] * R[1][1]);
      const double y00 = fma(R[0][0], t00, R[0][1] * t10);
      const double y01 = fma(R[0][0], t01, R[0][1] * t11);
      const double y11 = fma(R[1][0], t01, R[1][1] * t11);
      const double w2x = 2. * w * Xp[0][1];
      dX[0][0] = y00 + w2x;
      dX[1][1] = y11 - w2x;
      dX[0][1] = dX[1][0] = fma(w, Xp[1][1] - Xp[0][0], y01);
      dX[2][2] = fma(2. * Om[2][2], Xp[2][2], R[2][2] * (dX[2][2] * R[2][2]));
      return;
    } else {
      // R dX R^T, then Omega X' + (Omega X')^T written out for the skew Omega (a, b, c) =
      // (Omega_01, Omega_02, Omega_12)
      double dXRt[3][3];
#pragma unroll
      for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) dXRt[i][j] = fma(dX[i][0], R[j][0], fma(dX[i][1], R[j][1], dX[i][2] * R[j][2]));
      double Y[3][3];
#pragma unroll
      for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = i; j < 3; j++) Y[i][j] = fma(R[i][0], dXRt[0][j], fma(R[i][1], dXRt[1][j], R[i][2] * dXRt[2][j]));
      const double oa = Om[0][1], ob = Om[0][2], oc = Om[1][2];
      dX[0][0] = fma(2. * oa, Xp[1][0], fma(2. * ob, Xp[2][0], Y[0][0]));
      dX[1][1] = fma(-2. * oa, Xp[0][1], fma(2. * oc, Xp[2][1], Y[1][1]));
      dX[2][2] = fma(-2. * ob, Xp[0][2], fma(-2. * oc, Xp[1][2], Y[2][2]));
      dX[0][1] = dX[1][0] = fma(oa, Xp[1][1] - Xp[0][0], fma(ob, Xp[2][1], fma(oc, Xp[2][0], Y[0][1])));
      dX[0][2] = dX[2][0] = fma(oa, Xp[1][2], fma(ob, Xp[2][2] - Xp[0][0], fma(-oc, Xp[1][0], Y[0][2])));
      dX[1][2] = dX[2][1] = fma(-oa, Xp[0][2], fma(-ob, Xp[0][1], fma(oc, Xp[2][2] - Xp[1][1], Y[1][2])));
    }
  };
  rfi_t(L::S, dS);
  rfi_t(L::EPS, dE);
  rfi_t(L::EPSP, dP);
  if (valid) {
#pragma unroll
    for (int k = 0; k < NS; k++) {
      tip[(TN::S + k) * nIP + ipx] = dS[I0[k]][I1[k]];
      tip[(TN::EPS + k) * nIP + ipx] = dE[I0[k]][I1[k]];
      tip[(TN::EPSP + k) * nIP + ipx] = dP[I0[k]][I1[k]];
    }
    tip[TN::P * nIP + ipx] = dpn;
    tip[TN::EVP * nIP + ipx] = devp;
  }

  // ---- forces: Fe_k = - sum_pt dN_k . Sig W (+ hoop term)
  double sig[3][3];
  symload(sig, [&](int k) { return a.ip[(L::S + k) * nIP + ipx]; });
  const double pf = a.ip[L::P * nIP + ipx];
#pragma unroll
  for (int i = 0; i < 3; i++) {
    sig[i][i] += pf;
    dS[i][i] += dpn;  // now d Sig
  }
  // the Gauss weight (1 for the quads and the hexahedron; 1/6, 1/24, 8 for the others)
  double W = weighted<ET>(detJ), dW = weighted<ET>(ddetJ), dhoop = 0.;
  if (AXI) {
    W = detJ * (kDeuxPi * Rad);
    dW = kDeuxPi * fma(ddetJ, Rad, detJ * dRad);
    // the primal hoop force is sigma_tt / R x W = sigma_tt detJ 2 pi
    dhoop = kDeuxPi * fma(dS[2][2], detJ, sig[2][2] * ddetJ);
  }
  double dM[DIM][DIM];
#pragma unroll
  for (int l = 0; l < DIM; l++)
#pragma unroll
    for (int i = 0; i < DIM; i++) {
      double s = 0., ds = 0.;
#pragma unroll
      for (int j = 0; j < DIM; j++) {
        s = fma(Ji[l][j], sig[j][i], s);
        ds = fma(dJi[l][j], sig[j][i], fma(Ji[l][j], dS[j][i], ds));
      }
      dM[l][i] = fma(ds, W, s * dW);
    }
  // every point's dM (and hoop tangent) through the group's shared memory
  constexpr int ST = DIM * DIM + (AXI ? 1 : 0);
  double *mine = red + pt * ST;
#pragma unroll
  for (int l = 0; l < DIM; l++)
#pragma unroll
    for (int i = 0; i < DIM; i++) mine[l * DIM + i] = dM[l][i];
  if (AXI) mine[DIM * DIM] = dhoop;
  __syncwarp();
  if (!valid) return;
  double *tfe = a.tfe + (long)dir * DIM * a.feStride;
  if constexpr (NEN == NIP) {
    // the quads and the hexahedron: lane k assembles node k
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
    for (int i = 0; i < DIM; i++) tfe[(long)i * a.feStride + (long)e * NEN + pt] = ineg(s[i]);
  } else {
    // the tetrahedra and the one-point hexahedron: lane pt assembles nodes pt, pt + NIP, ...
    constexpr bool HG = ET == DNL_ELHEX8N3D_1PT;
    // hourglass force f_k = a_h sum_a gamma_ak (gamma_a . v) (added to the row, as in the primal
    // pass) and its tangent: gamma_ak = h_ak - sum_i (h_a . x_i) b_ki with b_k = J^-T dN_k/dxi, so
    // d gamma_ak = - sum_i (h_a . dx_i) b_ki + (h_a . x_i) db_ki; d a_h = (2/3) a_h dV / V
    double hx[4][3], dhx[4][3], qv[4][3], dqv[4][3], ah = 0., dah = 0.;
    auto hs = [](int q, int k) {
      const int sx = sgx(k), sy = sgy(k), sz = sgz(k);
      const int par = q == 0 ? sx ^ sy : (q == 1 ? sy ^ sz : (q == 2 ? sz ^ sx : sx ^ sy ^ sz));
      return (q == 3 ? par : !par) ? 1. : -1.;
    };
    auto gam_k = [&](int k, double g[4], double dg[4]) {
      double b[3], db[3];
#pragma unroll
      for (int i = 0; i < 3; i++) {
        double u = 0., du = 0.;
#pragma unroll
        for (int l = 0; l < 3; l++) {
          u = fma(Ji[l][i], SH::dN(0, k, l), u);
          du = fma(dJi[l][i], SH::dN(0, k, l), du);
        }
        b[i] = u;
        db[i] = du;
      }
#pragma unroll
      for (int q = 0; q < 4; q++) {
        double u = hs(q, k), du = 0.;
#pragma unroll
        for (int i = 0; i < 3; i++) {
          u = fma(-hx[q][i], b[i], u);
          du = fma(-dhx[q][i], b[i], fma(-hx[q][i], db[i], du));
        }
        g[q] = u;
        dg[q] = du;
      }
    };
    if constexpr (HG) {
#pragma unroll
      for (int q = 0; q < 4; q++)
#pragma unroll
        for (int i = 0; i < 3; i++) hx[q][i] = dhx[q][i] = qv[q][i] = dqv[q][i] = 0.;
#pragma unroll
      for (int k = 0; k < NEN; k++)
#pragma unroll
        for (int i = 0; i < 3; i++) {
          const double xk = a.x[i][node[k]], txk = tx[(long)i * N + node[k]];
#pragma unroll
          for (int q = 0; q < 4; q++) {
            hx[q][i] = fma(hs(q, k), xk, hx[q][i]);
            dhx[q][i] = fma(hs(q, k), txk, dhx[q][i]);
          }
        }
      const double *tv = a.tv + (long)dir * 3 * N;
#pragma unroll
      for (int k = 0; k < NEN; k++) {
        double g[4], dg[4];
        gam_k(k, g, dg);
#pragma unroll
        for (int i = 0; i < 3; i++) {
          const double vk = a.v[i][node[k]], tvk = tv[(long)i * N + node[k]];
#pragma unroll
          for (int q = 0; q < 4; q++) {
            qv[q][i] = fma(g[q], vk, qv[q][i]);
            dqv[q][i] = fma(dg[q], vk, fma(g[q], tvk, dqv[q][i]));
          }
        }
      }
      const double cv = cbrt(weighted<ET>(detJ));
      ah = 0.25 * a.hourglass * m.rho * m.Cs * (cv * cv);
      dah = ah * (2. / 3.) * ddetJ * nr_rcp(detJ);
    }
#pragma unroll
    for (int j = 0; j < (NEN + NIP - 1) / NIP; j++) {
      const int k = pt + j * NIP;
      if (k >= NEN) break;
      double s[DIM];
#pragma unroll
      for (int i = 0; i < DIM; i++) s[i] = 0.0;
#pragma unroll
      for (int q = 0; q < NIP; q++) {
        const double *Mq = red + q * ST;
#pragma unroll
        for (int l = 0; l < DIM; l++) {
          const double d = SH::dN(q, k, l);
#pragma unroll
          for (int i = 0; i < DIM; i++) s[i] = fma(d, Mq[l * DIM + i], s[i]);
        }
      }
      if constexpr (HG) {
        double g[4], dg[4];
        gam_k(k, g, dg);
#pragma unroll
        for (int i = 0; i < DIM; i++) {
          double f = 0., df = 0.;
#pragma unroll
          for (int q = 0; q < 4; q++) {
            f = fma(g[q], qv[q][i], f);
            df = fma(dg[q], qv[q][i], fma(g[q], dqv[q][i], df));
          }
          s[i] = fma(dah, f, fma(ah, df, s[i]));
        }
      }
#pragma unroll
      for (int i = 0; i < DIM; i++) tfe[(long)i * a.feStride + (long)e * NEN + k] = ineg(s[i]);
    }
  }
}

template <int ET>
__global__ void __launch_bounds__(128) k_elem_tan(SensElemArgs a)
{
  constexpr int NIP = Elem<ET>::NIP, NEN = Elem<ET>::NEN, DIM = Elem<ET>::DIM;
  constexpr int GPW = 32 / NIP;  // (element, direction) groups per warp
  __shared__ double red[128 / 32][GPW][NIP * NEN * DIM];
  if (!a.elemInst && a.tm->status) return;
  const long groups = (long)a.E * kSensParams;
  const long gtid = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if ((gtid & ~31L) / NIP >= groups) return;
  const long group = gtid / NIP;
  const bool valid = group < groups;
  const long g = valid ? group : groups - 1;
  const int lane = threadIdx.x & 31;
  elem_tan<ET>(a, (int)(g / kSensParams), (int)(g % kSensParams), (int)(gtid % NIP), valid, lane,
               red[threadIdx.x >> 5][lane / NIP]);
}

int launch_elem_tan(int etype, const SensElemArgs &a, cudaStream_t s)
{
  if (!etype_has_sens(etype)) return DNL_ERR_ARG;
  const long threads = (long)a.E * kSensParams * etype_nip(etype);
  const int grid = (int)((threads + 127) / 128);
  DNL_BY_ETYPE(etype, (k_elem_tan<ET><<<grid, 128, 0, s>>>(a)));
  launch_counter()++;
  return cudaPeekAtLastError() == cudaSuccess ? 0 : DNL_ERR_CUDA;
}
