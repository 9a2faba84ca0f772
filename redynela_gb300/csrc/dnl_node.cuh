// Nodal update and time-step logic of one node / one instance, shared by the nodal kernels
// (dnl_host.cu) and the batch's persistent step kernel (dnl_elem.cu):
//   node_update  the CSR gather of the element forces + ExplicitSolverCH::computePredictions
//                (ExplicitSolverCH.C:387-431), explicitSolve (:490-545), updateGrid (:555-567) and
//                the constant boundary conditions (Boundary.C:478-525, 636-665), with the
//                reference's rounding (__dmul_rn/__dadd_rn in its operation order);
//   dt_update    Solver::computeTimeStep (Solver.C:220-267), ExplicitSolverCH::initStep
//                (:434-447), updateTime and Solver::betweenTimeBounds.
// Every product and sum is written with an explicit rounding intrinsic or fma, so the code rounds
// the same in every translation unit whatever its contraction flags.
#pragma once

#include "dnl_common.cuh"

namespace dnl {

// ----------------------------------------------------------------------------- nodal update
__device__ __forceinline__ void apply_bc(int code, const double *spd, double dt, double cdu[3],
                                         double ndu[3], double cv[3], double nv[3], double ca[3],
                                         double na[3])
{
#pragma unroll
  for (int i = 0; i < 3; i++) {
    const int act = (code >> (2 * i)) & 3;
    if (act == 1) {
      cdu[i] = ndu[i] = cv[i] = nv[i] = ca[i] = na[i] = 0.;
    } else if (act == 2) {
      ca[i] = na[i] = 0.;
      cv[i] = nv[i] = spd[i];
      cdu[i] = __dmul_rn(cv[i], dt);
      ndu[i] = __dmul_rn(nv[i], dt);
    }
  }
}

// one node of the Chung-Hulbert update; dt and the integration constants of its mesh.  In 2D the
// third components of the nodal fields stay 0 (nothing writes them), so only DIM are read and
// written.  The two divisions of the corrector, F/M and (. - alphaM a)/(1 - alphaM), go through
// a reciprocal and one residual correction (quot): the FP64 pipe bounds this kernel too.
template <int DIM>
__device__ __forceinline__ void node_update(const NodeArgs &g, int n, double dt, double alphaM,
                                            double beta, double gamma)
{
  double cdu[3] = {0., 0., 0.}, cv[3] = {0., 0., 0.}, ca[3] = {0., 0., 0.}, cd[3] = {0., 0., 0.};
  double ndu[3] = {0., 0., 0.}, nv[3] = {0., 0., 0.}, na[3] = {0., 0., 0.}, nd[3] = {0., 0., 0.};
#pragma unroll
  for (int i = 0; i < DIM; i++) {
    cdu[i] = g.cur.du[i][n];
    cv[i] = g.cur.v[i][n];
    ca[i] = g.cur.a[i][n];
    cd[i] = g.cur.disp[i][n];
  }
  // computePredictions
  const double c1 = __dmul_rn(dt, __dsub_rn(0.5, beta)), c2 = __dmul_rn(dt, __dsub_rn(1., gamma));
#pragma unroll
  for (int i = 0; i < DIM; i++) {
    ndu[i] = __dmul_rn(__dadd_rn(__dmul_rn(ca[i], c1), cv[i]), dt);
    nd[i] = __dadd_rn(cd[i], ndu[i]);
    nv[i] = __dadd_rn(__dmul_rn(ca[i], c2), cv[i]);
    na[i] = 0.0;
  }
  const int bc = g.bcIdx[n];
  int code = 0;
  const double *spd = nullptr;
  if (bc >= 0) {
    code = g.bcCode[bc];
    spd = g.bcSpeed + 3 * bc;
    apply_bc(code, spd, dt, cdu, ndu, cv, nv, ca, na);
  }
  // assembled internal forces of this node
  double f[DIM];
#pragma unroll
  for (int c = 0; c < DIM; c++) f[c] = 0.0;
  for (int q = g.start[n]; q < g.start[n + 1]; q++) {
    const int ent = __ldg(g.entry + q);
#pragma unroll
    for (int c = 0; c < DIM; c++) f[c] = __dadd_rn(f[c], __ldg(g.fe + (long)c * g.EN + ent));
  }
  if (g.fint) {
#pragma unroll
    for (int c = 0; c < DIM; c++) g.fint[(long)n * DIM + c] = f[c];
  }
  // explicitSolve
  const double m = g.mass[n], rm = nr_rcp(m);
#pragma unroll
  for (int c = 0; c < DIM; c++) na[c] = quot(f[c], m, rm);
  const double cg = __dmul_rn(dt, gamma), cb = __dmul_rn(__dmul_rn(dt, dt), beta);
  const double oma = __dsub_rn(1.0, alphaM), roma = nr_rcp(oma);
#pragma unroll
  for (int i = 0; i < DIM; i++) {
    na[i] = __dsub_rn(na[i], __dmul_rn(alphaM, ca[i]));
    na[i] = quot(na[i], oma, roma);
    nv[i] = __dadd_rn(nv[i], __dmul_rn(cg, na[i]));
    ndu[i] = __dadd_rn(ndu[i], __dmul_rn(cb, na[i]));
  }
  if (bc >= 0) apply_bc(code, spd, dt, cdu, ndu, cv, nv, ca, na);
#pragma unroll
  for (int i = 0; i < DIM; i++) {
    nd[i] = __dadd_rn(cd[i], ndu[i]);
    g.nxt.du[i][n] = ndu[i];
    g.nxt.v[i][n] = nv[i];
    g.nxt.a[i][n] = na[i];
    g.nxt.disp[i][n] = nd[i];
    g.x[i][n] = __dadd_rn(g.x[i][n], ndu[i]);
  }
}

enum { DT_FORCE = 1, DT_POST = 2, DT_PRE = 4 };


__device__ __forceinline__ bool in_bounds(const DevTime *tm)
{
  const double up = tm->endTime < tm->upTime ? tm->endTime : tm->upTime;
  return tm->currentTime >= tm->startTime && tm->currentTime < up;
}

static __device__ void recompute_dt(DevTime *tm, int method, double safetyOmega, double Cs)
{
  double fmax;
  if (method == DNL_COURANT) {
    const double crit = __longlong_as_double((long long)tm->lenMinBits) / Cs;
    fmax = 2.0 / crit;
    tm->lenMinBits = 0x7ff0000000000000ull;  // +inf for the next reduction
  } else {
    fmax = tm->fmax;
  }
  tm->timeStep = safetyOmega / fmax;
  tm->lastTsDate = tm->tsDate;
  tm->lastTimeStep = tm->computedTimeStep;
  tm->tsDate = tm->currentTime;
  tm->computedTimeStep = tm->timeStep;
}

static __device__ void dt_update(DevTime *tm, int mode, int freq, int method, double safetyOmega, double Cs)
{
  if (tm->status) return;
  if (mode & DT_FORCE) recompute_dt(tm, method, safetyOmega, Cs);
  if ((mode & DT_POST) && !tm->done) {
    tm->currentTime = __dadd_rn(tm->currentTime, tm->timeStep);  // ExplicitSolverCH::updateTime
    if (!in_bounds(tm)) {
      tm->done = 1;
    } else if (tm->increment % freq == 0) {
      recompute_dt(tm, method, safetyOmega, Cs);
    } else if (tm->tsDate != tm->lastTsDate) {  // LINEARdbl extrapolation (Math.h:91)
      const double dx = __dsub_rn(tm->currentTime, tm->lastTsDate) / __dsub_rn(tm->tsDate, tm->lastTsDate);
      tm->timeStep = __dadd_rn(__dmul_rn(dx, tm->computedTimeStep), __dmul_rn(__dsub_rn(1.0, dx), tm->lastTimeStep));
    }
  }
  if ((mode & DT_PRE) && !tm->done) {
    if (!in_bounds(tm)) {
      tm->done = 1;
    } else {
      if (__dadd_rn(tm->currentTime, tm->timeStep) > tm->upTime) tm->timeStep = __dsub_rn(tm->upTime, tm->currentTime);
      tm->nextTime = __dadd_rn(tm->currentTime, tm->timeStep);
      tm->increment++;
    }
  }
  if (!tm->done && !(tm->timeStep > 0. && tm->timeStep < 1e300)) {
    tm->status = DNL_ERR_DT;
    tm->badElem = -1;
  }
}


}  // namespace dnl
