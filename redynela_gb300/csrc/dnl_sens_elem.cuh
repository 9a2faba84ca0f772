// Tangent of the element pass: forward-mode sensitivities of one explicit step with respect to the
// hardening parameters (A, B, n) and the initial-velocity magnitude, included by dnl_elem.cu
// (it shares the shape-function tables).
//
// The primal pass (k_elem<ET, true>) records per integration point the quantities the derivative
// needs (TapeLayout); this pass reads them with the tangents of its inputs and propagates:
//   J, J^-1, det J      from the coordinate tangents          (Element2D.C:53-126, Element3D.C:53-113)
//   F = I + grad du     with the Current delta_disp tangents  (ElementAx.C:114-136, Element3D.C:182-205)
//   ln U, U^-1, R       spectral derivative at the computed eigenpairs of C = F^T F (Daleckii-Krein:
//                       d f(C) = V (F o (V^T dC V)) V^T, F_ij divided differences of f)
//                                                           (Tensor2.C:1154-1259)
//   trial stress, J2 return: implicit-function derivative of the converged return equation
//                       sqrt(6) G gamma - Strial + sigma_y(evp + sqrt(2/3) gamma; A, B, n) = 0
//                                                           (Element.C:245-345, IsoHardElastoplastic.C:171-184)
//   pressure, RFI rotation, B^T sigma                       (Element.C:164-214, 351-401)
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
  const long nIP = (long)a.E * NIP, ipx = (long)e * NIP + pt, N = a.N;
  const Material &m = a.elemInst ? a.mats[a.elemInst[e]] : a.mat;
  auto tp = [&](int slot) { return a.tape[(long)slot * nIP + ipx]; };
  const double *tx = a.tx + (long)dir * 3 * N, *tdu = a.tdu + (long)dir * 3 * N;
  double *tip = a.tip + (long)dir * TN::NCOMP * nIP;
  const int I0[6] = {0, 1, 2, 0, 0, 1}, I1[6] = {0, 1, 2, 1, 2, 2};
  auto sym = [&](double X[3][3], auto get) {
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

  // ---- J^-1, det J and their tangents
  double Ji[DIM][DIM];
#pragma unroll
  for (int l = 0; l < DIM; l++)
#pragma unroll
    for (int c = 0; c < DIM; c++) Ji[l][c] = tp(TL::JI + l * DIM + c);
  const double detJ = tp(TL::DETJ), Rad = tp(TL::RAD);
  double dJ[DIM][DIM], dRad = 0.;
#pragma unroll
  for (int r = 0; r < DIM; r++)
#pragma unroll
    for (int c = 0; c < DIM; c++) dJ[r][c] = 0.;
#pragma unroll
  for (int k = 0; k < NEN; k++) {
    double t[DIM];
#pragma unroll
    for (int r = 0; r < DIM; r++) t[r] = tx[(long)r * N + node[k]];
#pragma unroll
    for (int r = 0; r < DIM; r++)
#pragma unroll
      for (int c = 0; c < DIM; c++) dJ[r][c] = fma(SH::dN(pt, k, c), t[r], dJ[r][c]);
    if (AXI) dRad = fma(SH::N(pt, k), t[0], dRad);
  }
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

  // ---- F (recorded) and dF
  double F[3][3], dF[3][3];
#pragma unroll
  for (int k = 0; k < 9; k++) {
    F[k / 3][k % 3] = tp(TL::F + k);
    dF[k / 3][k % 3] = 0.;
  }
  double vR = 0., dvR = 0.;
#pragma unroll
  for (int k = 0; k < NEN; k++) {
    double dNk[DIM], ddNk[DIM], u[DIM], tu[DIM];
#pragma unroll
    for (int c = 0; c < DIM; c++) {
      double s = 0., ds = 0.;
#pragma unroll
      for (int l = 0; l < DIM; l++) {
        s = fma(Ji[l][c], SH::dN(pt, k, l), s);
        ds = fma(dJi[l][c], SH::dN(pt, k, l), ds);
      }
      dNk[c] = s;
      ddNk[c] = ds;
    }
#pragma unroll
    for (int r = 0; r < DIM; r++) {
      u[r] = a.du[r][node[k]];
      tu[r] = tdu[(long)r * N + node[k]];
    }
#pragma unroll
    for (int r = 0; r < DIM; r++)
#pragma unroll
      for (int c = 0; c < DIM; c++) dF[r][c] = fma(ddNk[c], u[r], fma(dNk[c], tu[r], dF[r][c]));
    if (AXI) {
      vR = fma(SH::N(pt, k), u[0], vR);
      dvR = fma(SH::N(pt, k), tu[0], dvR);
    }
  }
  if (AXI) dF[2][2] = fma(-(vR / Rad), dRad, dvR) / Rad;

  // ---- dC, and the spectral derivatives of ln U = ln(C)/2 and U^-1 = C^-1/2
  double dC[3][3];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      double s = 0.;
#pragma unroll
      for (int k = 0; k < 3; k++) s = fma(dF[k][i], F[k][j], fma(F[k][i], dF[k][j], s));
      dC[i][j] = s;
    }
  double V[3][3], lam[3], lg[3], il[3];
#pragma unroll
  for (int k = 0; k < 9; k++) V[k / 3][k % 3] = tp(TL::V + k);
#pragma unroll
  for (int c = 0; c < 3; c++) {
    lam[c] = tp(TL::LAM + c);
    lg[c] = tp(TL::LG + c);
    il[c] = tp(TL::IL + c);
  }
  double Ah[3][3];  // V^T dC V
  {
    double T1[3][3];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) {
        double s = 0.;
#pragma unroll
        for (int k = 0; k < 3; k++) s = fma(dC[i][k], V[k][j], s);
        T1[i][j] = s;
      }
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) {
        double s = 0.;
#pragma unroll
        for (int k = 0; k < 3; k++) s = fma(V[k][i], T1[k][j], s);
        Ah[i][j] = s;
      }
  }
  double Bg[3][3], Bh[3][3];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      const double li = lam[i], lj = lam[j];
      const double mean = 0.5 * (li + lj), q = (li - lj) / mean;
      // (ln li - ln lj) / (2 (li - lj)); near-equal pair: 2 atanh(q/2) / (2 q mean) series
      const double g = fabs(q) < 1e-3 ? 0.5 * fma(q * q, fma(q * q, 1. / 80., 1. / 12.), 1.) / mean
                                       : (lg[i] - lg[j]) / (li - lj);
      const double hh = -il[i] * il[j] / fma(li, il[i], lj * il[j]);
      Bg[i][j] = g * Ah[i][j];
      Bh[i][j] = hh * Ah[i][j];
    }
  double dLn[3][3], dUi[3][3], Ui[3][3];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      double sg = 0., sh = 0., su = 0.;
#pragma unroll
      for (int k = 0; k < 3; k++) {
        double tg = 0., th = 0.;
#pragma unroll
        for (int l = 0; l < 3; l++) {
          tg = fma(Bg[k][l], V[j][l], tg);
          th = fma(Bh[k][l], V[j][l], th);
        }
        sg = fma(V[i][k], tg, sg);
        sh = fma(V[i][k], th, sh);
        su = fma(V[i][k] * il[k], V[j][k], su);
      }
      dLn[i][j] = sg;
      dUi[i][j] = sh;
      Ui[i][j] = su;
    }
  double R[3][3], dR[3][3];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      R[i][j] = tp(TL::R + i * 3 + j);
      double s = 0.;
#pragma unroll
      for (int k = 0; k < 3; k++) s = fma(dF[i][k], Ui[k][j], fma(F[i][k], dUi[k][j], s));
      dR[i][j] = s;
    }

  // ---- strain, trial stress
  double dS[3][3], dE[3][3], dP[3][3];
  sym(dS, [&](int k) { return tip[(TN::S + k) * nIP + ipx]; });
  sym(dE, [&](int k) { return tip[(TN::EPS + k) * nIP + ipx]; });
  sym(dP, [&](int k) { return tip[(TN::EPSP + k) * nIP + ipx]; });
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
    const double normS = tp(TL::NORMS), xv = tp(TL::XV), xn = tp(TL::XN);
    double nh[3][3];
    sym(nh, [&](int k) { return tp(TL::STR + k) / normS; });
    double dnorm = 0.;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) dnorm = fma(nh[i][j], dS[i][j], dnorm);
    const double h = m.nB * xn / xv;  // n B xv^(n-1)
    const double D = fma(kSqrt23, h, m.dfun0);
    const double dsig = dir == 0 ? 1. : (dir == 1 ? xn : (dir == 2 ? m.B * xn * log(xv) : 0.));
    const double dgam = fma(kSqrt32, dnorm, -fma(h, devp0, dsig)) / D;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) {
        const double dn = fma(-nh[i][j], dnorm, dS[i][j]) / normS;
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

  // ---- RFI: d(R X R^T) = R dX R^T + T + T^T, T = dR X R^T
  auto rfi_t = [&](int slot, double dX[3][3]) {
    double X[3][3];
    sym(X, [&](int k) { return tp(slot + k); });
    double XRt[3][3], dXRt[3][3];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) {
        double s = 0., t = 0.;
#pragma unroll
        for (int k = 0; k < 3; k++) {
          s = fma(X[i][k], R[j][k], s);
          t = fma(dX[i][k], R[j][k], t);
        }
        XRt[i][j] = s;
        dXRt[i][j] = t;
      }
    double Tm[3][3], Y[3][3];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) {
        double s = 0., t = 0.;
#pragma unroll
        for (int k = 0; k < 3; k++) {
          s = fma(dR[i][k], XRt[k][j], s);
          t = fma(R[i][k], dXRt[k][j], t);
        }
        Tm[i][j] = s;
        Y[i][j] = t;
      }
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) dX[i][j] = Y[i][j] + Tm[i][j] + Tm[j][i];
  };
  rfi_t(TL::SPRE, dS);
  rfi_t(TL::EPRE, dE);
  rfi_t(TL::PPRE, dP);
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
  sym(sig, [&](int k) { return a.ip[(L::S + k) * nIP + ipx]; });
  const double pf = a.ip[L::P * nIP + ipx];
#pragma unroll
  for (int i = 0; i < 3; i++) {
    sig[i][i] += pf;
    dS[i][i] += dpn;  // now d Sig
  }
  double W = detJ, dW = ddetJ, dhoop = 0.;
  if (AXI) {
    W = detJ * (kDeuxPi * Rad);
    dW = kDeuxPi * fma(ddetJ, Rad, detJ * dRad);
    const double hb = sig[2][2] / Rad;
    dhoop = fma(fma(-hb, dRad, dS[2][2]) / Rad, W, hb * dW);
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
  double *row = red + pt * (NEN * DIM);
#pragma unroll
  for (int k = 0; k < NEN; k++)
#pragma unroll
    for (int i = 0; i < DIM; i++) {
      double s = 0.;
#pragma unroll
      for (int l = 0; l < DIM; l++) s = fma(SH::dN(pt, k, l), dM[l][i], s);
      if (AXI && i == 0) s = fma(SH::N(pt, k), dhoop, s);
      row[k * DIM + i] = s;
    }
  __syncwarp();
  if (valid) {
    double *tfe = a.tfe + (long)dir * DIM * a.E * NEN;
#pragma unroll
    for (int i = 0; i < DIM; i++) {
      double s = 0.0;
#pragma unroll
      for (int q = 0; q < NIP; q++) s -= red[q * (NEN * DIM) + pt * DIM + i];
      tfe[(long)i * a.E * NEN + (long)e * NEN + pt] = s;
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
  const long threads = (long)a.E * kSensParams * (etype == DNL_ELQUA4NAX ? 4 : 8);
  const int grid = (int)((threads + 127) / 128);
  if (etype == DNL_ELQUA4NAX)
    k_elem_tan<DNL_ELQUA4NAX><<<grid, 128, 0, s>>>(a);
  else
    k_elem_tan<DNL_ELHEX8N3D><<<grid, 128, 0, s>>>(a);
  launch_counter()++;
  return cudaPeekAtLastError() == cudaSuccess ? 0 : DNL_ERR_CUDA;
}
