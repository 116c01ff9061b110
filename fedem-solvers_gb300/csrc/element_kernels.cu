// element_kernels.cu -- per-model control, per-DOF vector, per-element and
// per-equation kernels of the batched FEDEM HHT-alpha Newton iteration.
//
// Reference behaviour (paths relative to fedem-solvers):
//   predictor/corrector   src/vpmSolver/newmarkRoutinesModule.f90:85-187 (PredictVelAcc, IncVelAcc),
//                         :705-708 (SSTIF/SDAMP/SMASS), :751-805 (eqs. 7.53/7.55), :826-842 (tangent policy)
//   element update        src/vpmSolver/supElRoutinesModule.f90:47-85 (SetSupElsVelAcc), :231-456 (UpdateSupEls),
//                         src/vpmCommon/supElTypeModule.f90:912-992 (updateSupElCorot), :1067-1114 (BuildFinit)
//   Newton matrix         src/vpmSolver/supElRoutinesModule.f90:1254-1320 (BuildSupNewtonMat), :1127-1187 (AddInSupMat)
//   force vectors         src/vpmSolver/addInSysModule.f90:626-840 (GetForceVectors)
//   triad update          src/vpmCommon/triadTypeModule.f90:677-722, src/vpmUtilities/rotationModule.f90:355-500
//   norms/convergence     src/vpmSolver/solverRoutinesModule.f90:285-380, normRoutinesModule.f90:83-340,
//                         normTypeModule.f90:196-249
//   step end              src/vpmSolver/solverRoutinesModule.f90:728-827 (terminateStep, orthonorm3)
//   static equilibrium    src/vpmSolver/staticEquilibriumModule.f90:50-437, :919-1216
//
// All arithmetic here is FP64.  Summation orders are fixed (no atomics on
// floating-point data), so results are bitwise reproducible run to run.

#include <cmath>

#include "kernels.h"

namespace fgpu {
namespace {

constexpr int TPB = 256;

inline int blocksFor(long long n, int tpb = TPB) { return (int)((n + tpb - 1) / tpb); }

// 3x4 position matrices, column-major: T[r + 3c]
__device__ inline void compose34(const double* a, const double* b, double* o) {
#pragma unroll
  for (int c = 0; c < 4; ++c)
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      double s = a[r] * b[3 * c] + a[r + 3] * b[3 * c + 1] + a[r + 6] * b[3 * c + 2];
      if (c == 3) s += a[r + 9];
      o[r + 3 * c] = s;
    }
}

__device__ inline void crossd(const double* a, const double* b, double* c) {
  double x = a[1] * b[2] - a[2] * b[1], y = a[2] * b[0] - a[0] * b[2], z = a[0] * b[1] - a[1] * b[0];
  c[0] = x; c[1] = y; c[2] = z;
}

// rotation tensor from a rotation vector through a unit quaternion
__device__ inline void rotvecToMat(const double* rv, double* R /* col-major 3x3 */) {
  const double epsTh2 = 0.0005;
  double thh = 0.5 * sqrt(rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2]);
  double sthh, cthh;
  sincos(thh, &sthh, &cthh);
  double fac;
  if (thh < epsTh2) {
    double f1 = thh / epsTh2;
    fac = f1 * sin(epsTh2) / epsTh2 + 1.0 - f1;
  } else {
    fac = sthh / thh;
  }
  double q0 = cthh, q1 = rv[0] * fac * 0.5, q2 = rv[1] * fac * 0.5, q3 = rv[2] * fac * 0.5;
  double n = sqrt(q0 * q0 + q1 * q1 + q2 * q2 + q3 * q3);
  q0 /= n; q1 /= n; q2 /= n; q3 /= n;
  n = sqrt(q0 * q0 + q1 * q1 + q2 * q2 + q3 * q3);
  q0 /= n; q1 /= n; q2 /= n; q3 /= n;
  R[0] = 2.0 * (q1 * q1 + q0 * q0) - 1.0;
  R[4] = 2.0 * (q2 * q2 + q0 * q0) - 1.0;
  R[8] = 2.0 * (q3 * q3 + q0 * q0) - 1.0;
  R[3] = 2.0 * (q1 * q2 - q3 * q0);
  R[6] = 2.0 * (q1 * q3 + q2 * q0);
  R[7] = 2.0 * (q2 * q3 - q1 * q0);
  R[1] = 2.0 * (q2 * q1 + q3 * q0);
  R[2] = 2.0 * (q3 * q1 - q2 * q0);
  R[5] = 2.0 * (q3 * q2 + q1 * q0);
}

// re-orthonormalise a rotation tensor through its quaternion (Spurrier)
__device__ inline void orthonormRot(double* R /* col-major 3x3 */) {
  auto r = [&](int i, int j) { return R[i + 3 * j]; };
  double q[4];
  double tr = r(0, 0) + r(1, 1) + r(2, 2);
  int imax = 0;
  if (r(1, 1) > r(imax, imax)) imax = 1;
  if (r(2, 2) > r(imax, imax)) imax = 2;
  if (tr > r(imax, imax)) {
    q[0] = sqrt(1.0 + tr) * 0.5;
    q[1] = (r(2, 1) - r(1, 2)) / (4.0 * q[0]);
    q[2] = (r(0, 2) - r(2, 0)) / (4.0 * q[0]);
    q[3] = (r(1, 0) - r(0, 1)) / (4.0 * q[0]);
  } else {
    int i = imax, j = (imax + 1) % 3, k = (imax + 2) % 3;
    q[i + 1] = sqrt(r(i, i) * 0.5 + (1.0 - tr) * 0.25);
    q[0] = (r(k, j) - r(j, k)) / (4.0 * q[i + 1]);
    q[j + 1] = (r(j, i) + r(i, j)) / (4.0 * q[i + 1]);
    q[k + 1] = (r(k, i) + r(i, k)) / (4.0 * q[i + 1]);
  }
  double n = sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  for (int a = 0; a < 4; ++a) q[a] /= n;
  R[0] = 2.0 * (q[1] * q[1] + q[0] * q[0]) - 1.0;
  R[4] = 2.0 * (q[2] * q[2] + q[0] * q[0]) - 1.0;
  R[8] = 2.0 * (q[3] * q[3] + q[0] * q[0]) - 1.0;
  R[3] = 2.0 * (q[1] * q[2] - q[3] * q[0]);
  R[6] = 2.0 * (q[1] * q[3] + q[2] * q[0]);
  R[7] = 2.0 * (q[2] * q[3] - q[1] * q[0]);
  R[1] = 2.0 * (q[2] * q[1] + q[3] * q[0]);
  R[2] = 2.0 * (q[3] * q[1] - q[2] * q[0]);
  R[5] = 2.0 * (q[3] * q[2] + q[1] * q[0]);
}

// ---------------------------------------------------------------------------
// per-model control at the start of a batched iteration
// ---------------------------------------------------------------------------
__global__ void kBeginStep(DevModels m, int* activeCount, long long* activeEl) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m.n) return;
  int st = m.state[i], fl = 0;
  if (st == ST_NEED_STEP) {
    if (m.nStep[i] >= m.stepLimit[i]) { m.flags[i] = 0; return; }
    double t = m.time[i];
    if (m.tStart[i] <= m.tEnd[i] && t + 0.1 * m.minInc[i] > m.tEnd[i]) {
      m.state[i] = ST_DONE;
      m.flags[i] = 0;
      return;
    }
    double dt = m.dt[i], be = m.beta[i], ga = m.gamma[i];
    m.time[i] = t + dt;
    m.iter[i] = 0;
    m.nSeqNoUpd[i] = 0;
    m.negPiv[i] = 0;
    m.pc[4 * i + 0] = ga / be - 1.0;
    m.pc[4 * i + 1] = (0.5 * ga / be - 1.0) * dt;
    m.pc[4 * i + 2] = 1.0 / (be * dt);
    m.pc[4 * i + 3] = 0.5 / be - 1.0;
    m.sacc[i] = 1.0 / (be * dt * dt);
    m.svel[i] = ga / (be * dt);
    m.state[i] = ST_ITER;
    fl = FL_ACTIVE | FL_PRED;
  } else if (st == ST_ITER) {
    fl = FL_ACTIVE;
  } else {
    m.flags[i] = 0;
    return;
  }
  int it = m.iter[i];
  bool tangent = it < max(1, m.nUpdat[i]) || m.nSeqNoUpd[i] >= m.maxSeq[i];
  if (tangent) {
    fl |= FL_TANGENT;
    double sK = m.alpha[i] + 1.0, sC = m.svel[i] * sK, sM = m.sacc[i];
    double* sn = m.scaleN + 3 * i;
    if (fabs(sM - sn[0]) + fabs(sK - sn[1]) + fabs(sC - sn[2]) > 1.0e-16) {
      sn[0] = sM; sn[1] = sK; sn[2] = sC;
      fl |= FL_REBUILD;
    }
  }
  m.flags[i] = fl;
  atomicAdd(activeCount, 1);
  atomicAdd(reinterpret_cast<unsigned long long*>(activeEl), (unsigned long long)m.nel[i]);
}

// predicted velocity/acceleration increments and the actual inertia force
__global__ void kPredictDofs(DevData d) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < d.ndofTot) {
    int m = d.dofModel[i];
    if (d.m.flags[m] & FL_PRED) {
      const double* pc = d.m.pc + 4 * m;
      double v = d.urd[i], a = d.urdd[i];
      d.dk[i] = pc[0] * v + pc[1] * a;
      d.ak[i] = pc[2] * v + pc[3] * a;
      d.rinc[i] = 0.0;
    }
  }
  if (i < d.neqTot) {
    int m = d.eqModel[i];
    if (d.m.flags[m] & FL_PRED) {
      // FIactual = FIk of the converged previous step (NewmarkFlag = 0)
      double s = 0.0;
      const double* FI = d.Fel + (size_t)24 * d.nelTot;
      for (int k = d.eqPtr[i]; k < d.eqPtr[i + 1]; ++k) s += FI[d.eqSrc[k]];
      d.FIact[i] = s;
    }
  }
}

// ---------------------------------------------------------------------------
// element pass: corotated frame, deformation, internal and inertia forces
// ---------------------------------------------------------------------------
__device__ inline void matvecSoA(const double* __restrict__ A, int nel, int e, const double* x, double s,
                                 double* y) {
#pragma unroll
  for (int r = 0; r < 12; ++r) y[r] = 0.0;
#pragma unroll
  for (int c = 0; c < 12; ++c) {
    double xc = x[c];
#pragma unroll
    for (int r = 0; r < 12; ++r) y[r] += A[(size_t)(r + 12 * c) * nel + e] * xc;
  }
#pragma unroll
  for (int r = 0; r < 12; ++r) y[r] *= s;
}

// Beam elements whose superelement axes are the beam's principal axes (the
// usual FEDEM set-up) have exactly 40 structural nonzeros in K, M and C
// (axial, torsion and the two bending planes).  They are stored as the 26
// upper-triangle values of kBeamPattern; the product visits each row's
// nonzeros in ascending column order, so it rounds exactly like the dense one.
__device__ inline void matvecBeam(const double* __restrict__ A26, int nel, int e, const double* x, double s,
                                  double* y) {
  double a[26];
#pragma unroll
  for (int k = 0; k < 26; ++k) a[k] = A26[(size_t)k * nel + e];
  // row -> (value index, column) pairs, ascending column
  y[0] = a[0] * x[0];   y[0] += a[1] * x[6];
  y[1] = a[2] * x[1];   y[1] += a[3] * x[5];   y[1] += a[4] * x[7];   y[1] += a[5] * x[11];
  y[2] = a[6] * x[2];   y[2] += a[7] * x[4];   y[2] += a[8] * x[8];   y[2] += a[9] * x[10];
  y[3] = a[10] * x[3];  y[3] += a[11] * x[9];
  y[4] = a[7] * x[2];   y[4] += a[12] * x[4];  y[4] += a[13] * x[8];  y[4] += a[14] * x[10];
  y[5] = a[3] * x[1];   y[5] += a[15] * x[5];  y[5] += a[16] * x[7];  y[5] += a[17] * x[11];
  y[6] = a[1] * x[0];   y[6] += a[18] * x[6];
  y[7] = a[4] * x[1];   y[7] += a[16] * x[5];  y[7] += a[19] * x[7];  y[7] += a[20] * x[11];
  y[8] = a[8] * x[2];   y[8] += a[13] * x[4];  y[8] += a[21] * x[8];  y[8] += a[22] * x[10];
  y[9] = a[11] * x[3];  y[9] += a[23] * x[9];
  y[10] = a[9] * x[2];  y[10] += a[14] * x[4]; y[10] += a[22] * x[8]; y[10] += a[24] * x[10];
  y[11] = a[5] * x[1];  y[11] += a[17] * x[5]; y[11] += a[20] * x[7]; y[11] += a[25] * x[11];
#pragma unroll
  for (int r = 0; r < 12; ++r) y[r] *= s;
}

// y = s * A x for element matrix 0 = K, 1 = M, 2 = C (compressed when the batch allows)
__device__ inline void elemMatvec(const DevData& d, int which, int e, const double* x, double s, double* y) {
  if (d.beamSparse) {
    const double* A = which == 0 ? d.K26 : which == 1 ? d.M26 : d.C26;
    matvecBeam(A, d.nelTot, e, x, s, y);
  } else {
    const double* A = which == 0 ? d.K : which == 1 ? d.M : d.C;
    matvecSoA(A, d.nelTot, e, x, s, y);
  }
}

__device__ inline void rotateStore(const double* S, const double* f, double* out, int nel, int e) {
#pragma unroll
  for (int g = 0; g < 4; ++g)
#pragma unroll
    for (int r = 0; r < 3; ++r)
      out[(size_t)(3 * g + r) * nel + e] = S[r] * f[3 * g] + S[r + 3] * f[3 * g + 1] + S[r + 6] * f[3 * g + 2];
}

__global__ void __launch_bounds__(128) kElements(DevData d, int mode) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  const int nel = d.nelTot;
  if (e >= nel) return;
  int m = d.elModel[e];
  int fl = d.m.flags[m];
  if (mode == EM_PRED) {
    if (!(fl & FL_PRED)) return;
  } else if (mode == EM_INC) {
    if (!(fl & FL_ACTIVE)) return;
  } else if (mode == EM_STATIC || mode == EM_STATIC_INIT) {
    if (!(fl & FL_STATIC)) return;
  }  // EM_FINAL: every model
  const bool isStatic = mode == EM_STATIC || mode == EM_STATIC_INIT;
  double S[12];
#pragma unroll
  for (int k = 0; k < 12; ++k) S[k] = d.supTr[(size_t)k * nel + e];
  int tri[2] = {d.elTri[e], d.elTri[nel + e]};
  double uld[12], uldd[12];
  if (!isStatic) {
    const double* vs = mode == EM_PRED ? d.dk : d.urd;
    const double* as = mode == EM_PRED ? d.ak : d.urdd;
#pragma unroll
    for (int n = 0; n < 2; ++n) {
      int d0 = d.triFirstDof[tri[n]];
#pragma unroll
      for (int g = 0; g < 2; ++g) {
        double v0 = vs[d0 + 3 * g], v1 = vs[d0 + 3 * g + 1], v2 = vs[d0 + 3 * g + 2];
        double a0 = as[d0 + 3 * g], a1 = as[d0 + 3 * g + 1], a2 = as[d0 + 3 * g + 2];
#pragma unroll
        for (int r = 0; r < 3; ++r) {
          uld[6 * n + 3 * g + r] = S[3 * r] * v0 + S[3 * r + 1] * v1 + S[3 * r + 2] * v2;
          uldd[6 * n + 3 * g + r] = S[3 * r] * a0 + S[3 * r + 1] * a1 + S[3 * r + 2] * a2;
        }
      }
    }
  }
  const bool newPositions = mode == EM_INC || mode == EM_STATIC || mode == EM_FINAL;
  double fin[12];
  if (newPositions) {
    // corotated frame through the three reference points (shadowPosAlg = 1)
    double p[3][3];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      int node = d.elRef[(size_t)j * nel + e];
      const double* U = d.ur + 12 * (size_t)(node ? tri[1] : tri[0]);
      double o0 = d.offset[(size_t)(3 * j) * nel + e], o1 = d.offset[(size_t)(3 * j + 1) * nel + e],
             o2 = d.offset[(size_t)(3 * j + 2) * nel + e];
#pragma unroll
      for (int q = 0; q < 3; ++q) p[j][q] = U[q] * o0 + U[q + 3] * o1 + U[q + 6] * o2 + U[q + 9];
    }
    double ex[3], v2[3], ez[3], ey[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) { ex[k] = p[1][k] - p[0][k]; v2[k] = p[2][k] - p[0][k]; }
    crossd(ex, v2, ez);
    double lx = ex[0] * ex[0] + ex[1] * ex[1] + ex[2] * ex[2];
    double lz = ez[0] * ez[0] + ez[1] * ez[1] + ez[2] * ez[2];
    if (!(lx > 1.0e-16) || !(lz > 1.0e-16)) {
      atomicOr(&d.m.status[m], SS_COROT);
      return;
    }
    lx = sqrt(lx);
    lz = sqrt(lz);
#pragma unroll
    for (int k = 0; k < 3; ++k) { ex[k] /= lx; ez[k] /= lz; }
    crossd(ez, ex, ey);
    double T[12] = {ex[0], ex[1], ex[2], ey[0], ey[1], ey[2], ez[0], ez[1], ez[2], p[0][0], p[0][1], p[0][2]};
    double Rel[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) Rel[k] = d.triRelSup[(size_t)k * nel + e];
    compose34(T, Rel, S);
#pragma unroll
    for (int k = 0; k < 12; ++k) d.supTr[(size_t)k * nel + e] = S[k];
  }
  if (newPositions || mode == EM_STATIC_INIT) {
    // deformation vector in the corotated axes
    double inv[12];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 3; ++c) inv[r + 3 * c] = S[c + 3 * r];
#pragma unroll
    for (int r = 0; r < 3; ++r) inv[9 + r] = -(inv[r] * S[9] + inv[r + 3] * S[10] + inv[r + 6] * S[11]);
#pragma unroll
    for (int n = 0; n < 2; ++n) {
      const double* U = d.ur + 12 * (size_t)tri[n];
      double Uc[12], loc[12];
#pragma unroll
      for (int k = 0; k < 12; ++k) Uc[k] = U[k];
      compose34(inv, Uc, loc);
      double Tu[12];
#pragma unroll
      for (int k = 0; k < 12; ++k) Tu[k] = d.trUnd[(size_t)(12 * n + k) * nel + e];
#pragma unroll
      for (int r = 0; r < 3; ++r) fin[6 * n + r] = loc[9 + r] - Tu[9 + r];
      // dR = loc(:,1:3) * Tu(:,1:3); entries (3,2), (1,3), (2,1)
      auto dR = [&](int r, int c) { return loc[r] * Tu[3 * c] + loc[r + 3] * Tu[3 * c + 1] + loc[r + 6] * Tu[3 * c + 2]; };
      fin[6 * n + 3] = dR(2, 1);
      fin[6 * n + 4] = dR(0, 2);
      fin[6 * n + 5] = dR(1, 0);
    }
#pragma unroll
    for (int k = 0; k < 12; ++k) d.finit[(size_t)k * nel + e] = fin[k];
  } else {
#pragma unroll
    for (int k = 0; k < 12; ++k) fin[k] = d.finit[(size_t)k * nel + e];
  }
  const double ss = d.stifScl[e];
  double y[12];
  double* FSo = d.Fel;
  double* FDo = d.Fel + (size_t)12 * nel;
  double* FIo = d.Fel + (size_t)24 * nel;
  double* Qo = d.Fel + (size_t)36 * nel;
  // Fs = stifScl * K * finit.  The predictor pass keeps the frame and the
  // deformation of the converged previous step, so FS and Q stored by the
  // last pass are already the values UpdateSupEls would recompute.
  const bool keepFsQ = mode == EM_PRED;
  if (!keepFsQ) {
    elemMatvec(d, 0, e, fin, ss, y);
    rotateStore(S, y, FSo, nel, e);
  }
  if (isStatic) {
#pragma unroll
    for (int k = 0; k < 12; ++k) { FDo[(size_t)k * nel + e] = 0.0; FIo[(size_t)k * nel + e] = 0.0; }
  } else {
    // Fi = M * uldd
    elemMatvec(d, 1, e, uldd, 1.0, y);
    rotateStore(S, y, FIo, nel, e);
    // Fd = stifScl * C * uld  (- kDmp * stifScl * K * (uld - vld)); exactly zero without damping
    const double dt = d.m.dt[m];
    const bool vldActive = mode == EM_INC && d.hasVld[e] && dt > 0.0;
    if (d.hasC[e] || vldActive) {
      if (d.hasC[e]) {
        elemMatvec(d, 2, e, uld, ss, y);
      } else {
#pragma unroll
        for (int k = 0; k < 12; ++k) y[k] = 0.0;
      }
      if (vldActive) {
        double tmp[12], yk[12];
#pragma unroll
        for (int k = 0; k < 12; ++k) tmp[k] = uld[k] - (fin[k] - d.finitPrev[(size_t)k * nel + e]) / dt;
        elemMatvec(d, 0, e, tmp, ss, yk);
        double kd = d.kDmp[e];
#pragma unroll
        for (int k = 0; k < 12; ++k) y[k] -= kd * yk[k];
      }
      rotateStore(S, y, FDo, nel, e);
    } else {
#pragma unroll
      for (int k = 0; k < 12; ++k) FDo[(size_t)k * nel + e] = 0.0;
    }
  }
  if (keepFsQ) return;
  // gravity: Q = stifScl * fg * (supTr^T g); exactly zero without gravity
  const double* gv = d.m.gravity + 3 * m;
  if (gv[0] == 0.0 && gv[1] == 0.0 && gv[2] == 0.0) {
#pragma unroll
    for (int k = 0; k < 12; ++k) Qo[(size_t)k * nel + e] = 0.0;
    return;
  }
  double gl0 = gv[0] * S[0] + gv[1] * S[1] + gv[2] * S[2];
  double gl1 = gv[0] * S[3] + gv[1] * S[4] + gv[2] * S[5];
  double gl2 = gv[0] * S[6] + gv[1] * S[7] + gv[2] * S[8];
#pragma unroll
  for (int r = 0; r < 12; ++r)
    y[r] = ss * (d.fg[(size_t)r * nel + e] * gl0 + d.fg[(size_t)(r + 12) * nel + e] * gl1 +
                 d.fg[(size_t)(r + 24) * nel + e] * gl2);
  rotateStore(S, y, Qo, nel, e);
}

// residual: force predictor (7.53) or corrector (7.55); RHS del = residual
__global__ void kResidual(DevData d) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.neqTot) return;
  int m = d.eqModel[i];
  int fl = d.m.flags[m];
  if (!(fl & FL_ACTIVE)) return;
  const size_t blk = (size_t)12 * d.nelTot;
  double fs = 0.0, fd = 0.0, fi = 0.0, q = 0.0;
  for (int k = d.eqPtr[i]; k < d.eqPtr[i + 1]; ++k) {
    size_t s = d.eqSrc[k];
    fs += d.Fel[s];
    fd += d.Fel[s + blk];
    fi += d.Fel[s + 2 * blk];
    q += d.Fel[s + 3 * blk];
  }
  q += d.qext[i];
  d.FSk[i] = fs;
  d.FDk[i] = fd;
  d.FIk[i] = fi;
  d.Qk[i] = q;
  double a = d.m.alpha[m], sstif = a + 1.0, r;
  if (fl & FL_PRED)
    r = sstif * (q - fs + fd) + fi - a * d.FIact[i];
  else
    r = sstif * (q - fs - fd) - fi - a * d.FIact[i];
  d.res[i] = r;
  d.del[i] = r;
}

// element Newton matrix N = sM*M + sC*stifScl*C + sK*stifScl*K (rebuilt when the scales change)
__global__ void kBuildElementNewton(DevData d) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  const int nel = d.nelTot;
  if (e >= nel) return;
  int m = d.elModel[e];
  if (!(d.m.flags[m] & FL_REBUILD)) return;
  const double* sn = d.m.scaleN + 3 * m;
  double ss = d.stifScl[e];
  double sM = sn[0], sK = sn[1] * ss, sC = sn[2] * ss;
  bool hc = d.hasC[e];
  for (int k = 0; k < 144; ++k) {
    size_t ix = (size_t)k * nel + e;
    double v = sM * d.M[ix];
    if (hc) v += sC * d.C[ix];
    v += sK * d.K[ix];
    d.N[ix] = v;
  }
}

// rotate the element Newton matrix to system axes: Ns = R N R^T blockwise
__global__ void __launch_bounds__(128) kRotateElementNewton(DevData d) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  const int nel = d.nelTot;
  if (e >= nel) return;
  int m = d.elModel[e];
  if (!(d.m.flags[m] & FL_TANGENT)) return;
  double R[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) R[k] = d.supTr[(size_t)k * nel + e];
  for (int bj = 0; bj < 4; ++bj)
    for (int bi = 0; bi < 4; ++bi) {
      double B[9], W[9];
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int r = 0; r < 3; ++r) B[r + 3 * c] = d.N[(size_t)((3 * bi + r) + 12 * (3 * bj + c)) * nel + e];
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int r = 0; r < 3; ++r) W[r + 3 * c] = R[r] * B[3 * c] + R[r + 3] * B[3 * c + 1] + R[r + 6] * B[3 * c + 2];
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int r = 0; r < 3; ++r)
          d.elMat[(size_t)((3 * bi + r) + 12 * (3 * bj + c)) * nel + e] =
              W[r] * R[c] + W[r + 3] * R[c + 3] + W[r + 6] * R[c + 6];
    }
}

// CSR slot gather (deterministic segmented reduction over element contributions)
__global__ void kCsrGather(DevData d) {
  long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= d.nslotTot) return;
  if (!(d.m.flags[d.slotModel[s]] & FL_TANGENT)) return;
  double v = 0.0;
  for (long long k = d.slotPtr[s]; k < d.slotPtr[s + 1]; ++k) v += d.elMat[d.slotSrc[k]];
  d.csrVal[s] = v;
}

// increment: expand the solution, update velocities/accelerations and triads
__global__ void kIncrement(DevData d) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < d.ndofTot) {
    int m = d.dofModel[i];
    if (d.m.flags[m] & FL_ACTIVE) {
      int eq = d.meqn[i];
      // corrector steps replace prescribed values by zero; fixed DOFs are zero
      double s0 = eq >= 0 ? d.del[eq] : 0.0;
      double sv = d.m.svel[m], sa = d.m.sacc[m];
      d.sinc0[i] = s0;
      d.sinc1[i] = s0 * sv;
      d.sinc2[i] = s0 * sa;
      double ri = d.rinc[i] + s0;
      d.rinc[i] = ri;
      d.urd[i] = sv * ri - d.dk[i];
      d.urdd[i] = sa * ri - d.ak[i];
    }
  }
  if (i < d.ntriTot) {
    int m = d.triModel[i];
    if ((d.m.flags[m] & FL_ACTIVE) && d.triNdof[i] > 0) {
      double inc[6] = {0, 0, 0, 0, 0, 0};
      int d0 = d.triFirstDof[i], nd = d.triNdof[i];
      for (int k = 0; k < nd && k < 6; ++k) {
        int eq = d.meqn[d0 + k];
        inc[k] = eq >= 0 ? d.del[eq] : 0.0;
      }
      double* U = d.ur + 12 * (size_t)i;
      for (int r = 0; r < 3; ++r) U[9 + r] += inc[r];
      if (nd == 6) {
        double R[9], O[9];
        rotvecToMat(inc + 3, R);
        for (int c = 0; c < 3; ++c)
          for (int r = 0; r < 3; ++r) O[r + 3 * c] = R[r] * U[3 * c] + R[r + 3] * U[3 * c + 1] + R[r + 6] * U[3 * c + 2];
        for (int k = 0; k < 9; ++k) U[k] = O[k];
      }
    }
  }
}

// ---------------------------------------------------------------------------
// block reductions with a fixed tree (deterministic)
// ---------------------------------------------------------------------------
constexpr int NTPB = 128;

__device__ inline double blockSum(double v, double* sh) {
  int t = threadIdx.x;
  sh[t] = v;
  __syncthreads();
  for (int s = NTPB / 2; s > 0; s >>= 1) {
    if (t < s) sh[t] += sh[t + s];
    __syncthreads();
  }
  double r = sh[0];
  __syncthreads();
  return r;
}

__device__ inline double blockMax(double v, double* sh) {
  int t = threadIdx.x;
  sh[t] = v;
  __syncthreads();
  for (int s = NTPB / 2; s > 0; s >>= 1) {
    if (t < s) sh[t] = fmax(sh[t], sh[t + s]);
    __syncthreads();
  }
  double r = sh[0];
  __syncthreads();
  return r;
}

__device__ inline bool isBad(double v) { return !(fabs(v) <= 1.0e300); }

// Iteration norms in two deterministic stages: every chunk of DOFs (one model
// each) reduces 21 partial values with a fixed tree; one thread per model then
// combines its chunks in order, applies the convergence test and the step-end
// bookkeeping flags.  Partials: 0 sw, 1 swf, 2-4 disp/vel/acc sums of squares,
// 5 residual, 6 energy sum, 7 energy max, 8-19 inf norms (4 vectors x 3 DOF
// types), 20 NaN/Inf seen.
constexpr int NPART = 21;
constexpr int CHUNK_TPB = 256;

__global__ void __launch_bounds__(CHUNK_TPB) kNormsPartial(DevData d) {
  __shared__ double sh[CHUNK_TPB / 32][NPART];
  const int c = blockIdx.x;
  const int m = d.chunkModel[c];
  if (!(d.m.flags[m] & FL_ACTIVE)) return;
  const double* wD = d.m.wDisp + 3 * m;
  const double* wF = d.m.wForce + 3 * m;
  double v[NPART];
#pragma unroll
  for (int k = 0; k < NPART; ++k) v[k] = 0.0;
  for (int i = d.chunkStart[c] + threadIdx.x; i < d.chunkEnd[c]; i += CHUNK_TPB) {
    int eq = d.meqn[i];
    if (eq < 0) continue;
    int t = d.dofType[i] - 1;
    double wd = wD[t], wf = wF[t];
    double s0 = d.sinc0[i], s1 = d.sinc1[i], s2 = d.sinc2[i], r = d.res[eq];
    if (isBad(s0) || isBad(r)) v[20] = 1.0;
    v[0] += wd * wd;
    v[1] += wf * wf;
    v[2] += (wd * s0) * (wd * s0);
    v[3] += (wd * s1) * (wd * s1);
    v[4] += (wd * s2) * (wd * s2);
    v[5] += (wf * r) * (wf * r);
    double en = fabs(s0 * r);
    v[6] += en;
    v[7] = fmax(v[7], en);
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      if (q != t) continue;
      v[8 + q] = fmax(v[8 + q], fabs(s0));
      v[11 + q] = fmax(v[11 + q], fabs(s1));
      v[14 + q] = fmax(v[14 + q], fabs(s2));
      v[17 + q] = fmax(v[17 + q], fabs(r));
    }
  }
  // warp tree (fixed pattern), then warps in order
#pragma unroll
  for (int k = 0; k < NPART; ++k) {
    double x = v[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      double y = __shfl_down_sync(0xffffffffu, x, o);
      x = (k <= 6) ? x + y : fmax(x, y);
    }
    v[k] = x;
  }
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < NPART; ++k) sh[w][k] = v[k];
  __syncthreads();
  if (threadIdx.x < NPART) {
    const int k = threadIdx.x;
    double x = sh[0][k];
    for (int ww = 1; ww < CHUNK_TPB / 32; ++ww) x = (k <= 6) ? x + sh[ww][k] : fmax(x, sh[ww][k]);
    d.partial[(size_t)c * NPART + k] = x;
  }
}

// norms, convergence test (normTypeModule.f90:196-249) and iteration counters
__global__ void kControl(DevData d) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= d.m.n) return;
  const int fl = d.m.flags[m];
  if (!(fl & FL_ACTIVE)) return;
  double v[NPART];
  const int c0 = d.modelChunkOff[m], nc = d.modelNchunk[m];
  for (int k = 0; k < NPART; ++k) v[k] = nc > 0 ? d.partial[(size_t)c0 * NPART + k] : 0.0;
  for (int c = 1; c < nc; ++c)
    for (int k = 0; k < NPART; ++k) {
      double x = d.partial[(size_t)(c0 + c) * NPART + k];
      v[k] = (k <= 6) ? v[k] + x : fmax(v[k], x);
    }
  double* nv = d.m.normVal + 18 * m;
  nv[0] = v[0] > 0 ? sqrt(v[2] / v[0]) : 0.0;
  nv[4] = v[0] > 0 ? sqrt(v[3] / v[0]) : 0.0;
  nv[8] = v[0] > 0 ? sqrt(v[4] / v[0]) : 0.0;
  nv[12] = v[1] > 0 ? sqrt(v[5] / v[1]) : 0.0;
  for (int t = 0; t < 3; ++t) {
    nv[1 + t] = v[8 + t];
    nv[5 + t] = v[11 + t];
    nv[9 + t] = v[14 + t];
    nv[13 + t] = v[17 + t];
  }
  const int neq = d.m.neq[m], nd = d.m.ndof[m];
  nv[16] = v[7];
  nv[17] = (nd > 1 && neq > 0) ? v[6] / (double)neq : v[6];
  const int it = d.m.iter[m] + 1;
  d.m.iter[m] = it;
  d.m.nIter[m] += 1;
  if (fl & FL_TANGENT) d.m.nSeqNoUpd[m] = 0;
  else d.m.nSeqNoUpd[m] += 1;
  bool conv = false;
  if (d.errFlag && *d.errFlag) d.m.status[m] |= SS_TIMEOUT;
  if (v[20] > 0.0 || (d.m.status[m] & (SS_SINGULAR | SS_COROT | SS_TIMEOUT))) {
    d.m.status[m] |= v[20] > 0.0 ? SS_NAN : 0;
    d.m.state[m] = ST_ERROR;
  } else if (d.m.fixedIt[m] > 0) {
    conv = it == d.m.fixedIt[m];
  } else if (it > d.m.maxIt[m]) {
    d.m.status[m] |= SS_MAXIT;
    d.m.state[m] = ST_ERROR;
  } else if (it >= max(2, d.m.minIt[m])) {
    bool exists1 = false, exists2 = false, oneOf = false, allOf = true;
    const int* code = d.m.tolCode + 18 * m;
    const double* tol = d.m.tolVal + 18 * m;
    for (int k = 0; k < 18; ++k) {
      if (code[k] == 2) { exists2 = true; if (nv[k] < tol[k]) oneOf = true; }
      else if (code[k] == 1) { exists1 = true; if (nv[k] >= tol[k]) allOf = false; }
    }
    conv = true;
    if (exists2) conv = conv && oneOf;
    if (exists1) conv = conv && allOf;
  }
  if (conv) {
    d.m.nStep[m] += 1;
    d.m.state[m] = ST_NEED_STEP;
    d.m.flags[m] = fl | FL_STEPDONE;
  }
}

// terminateStep (solverRoutinesModule.f90:728-827): orthonormalise the triad
// rotations of models that finished a step; keep their deformation for the next one
__global__ void kStepEnd(DevData d) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < d.ntriTot) {
    if ((d.m.flags[d.triModel[i]] & FL_STEPDONE) && d.triNdof[i] == 6) orthonormRot(d.ur + 12 * (size_t)i);
  }
  if (i < d.nelTot) {
    if (d.m.flags[d.elModel[i]] & FL_STEPDONE)
#pragma unroll
      for (int c = 0; c < 12; ++c) {
        size_t ix = (size_t)c * d.nelTot + i;
        d.finitPrev[ix] = d.finit[ix];
      }
  }
}

// ---------------------------------------------------------------------------
// static equilibrium iterations
// ---------------------------------------------------------------------------
__global__ void kStaticBegin(DevModels m, int* activeCount) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m.n) return;
  if (m.staticDone[i] || m.state[i] == ST_ERROR) { m.flags[i] = 0; return; }
  int fl = FL_ACTIVE | FL_STATIC | FL_TANGENT;
  double* sn = m.scaleN + 3 * i;
  if (fabs(0.0 - sn[0]) + fabs(1.0 - sn[1]) + fabs(0.0 - sn[2]) > 1.0e-16) {
    sn[0] = 0.0; sn[1] = 1.0; sn[2] = 0.0;
    fl |= FL_REBUILD;
  }
  m.flags[i] = fl;
  atomicAdd(activeCount, 1);
}

__global__ void kStaticResidual(DevData d) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.neqTot) return;
  int m = d.eqModel[i];
  if (!(d.m.flags[m] & FL_STATIC)) return;
  double fs = 0.0, q = 0.0;
  const size_t blk = (size_t)12 * d.nelTot;
  for (int k = d.eqPtr[i]; k < d.eqPtr[i + 1]; ++k) {
    size_t s = d.eqSrc[k];
    fs += d.Fel[s];
    q += d.Fel[s + 3 * blk];
  }
  q += d.qext[i];
  d.FSk[i] = fs;
  d.Qk[i] = q;
  d.res[i] = q - fs;
  d.del[i] = q - fs;
}

__global__ void __launch_bounds__(NTPB) kStaticNorm(DevData d) {
  __shared__ double sh[NTPB];
  int m = blockIdx.x;
  if (!(d.m.flags[m] & FL_STATIC)) return;
  const int d0 = d.m.dofOff[m], nd = d.m.ndof[m];
  const double* wD = d.m.wDisp + 3 * m;
  double sw = 0.0, q = 0.0;
  for (int k = threadIdx.x; k < nd; k += NTPB) {
    int i = d0 + k, eq = d.meqn[i];
    if (eq < 0) continue;
    double w = wD[d.dofType[i] - 1], v = d.del[eq];
    sw += w * w;
    q += (w * v) * (w * v);
  }
  sw = blockSum(sw, sh);
  q = blockSum(q, sh);
  if (threadIdx.x == 0) {
    double deln = sw > 0.0 ? sqrt(q / sw) : 0.0;
    d.m.deln[m] = deln;
    double f = 1.0;
    if (d.m.staticMode[m] == 2 && deln > d.m.equLim[m]) f = d.m.equLim[m] / deln;
    d.m.staticScale[m] = f;
  }
}

__global__ void kStaticIncrement(DevData d) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < d.ndofTot) {
    int m = d.dofModel[i];
    if (d.m.flags[m] & FL_STATIC) {
      int eq = d.meqn[i];
      double s0 = eq >= 0 ? d.del[eq] * d.m.staticScale[m] : 0.0;
      d.sinc0[i] = s0;
      d.rinc[i] += s0;
    }
  }
  if (i < d.ntriTot) {
    int m = d.triModel[i];
    if ((d.m.flags[m] & FL_STATIC) && d.triNdof[i] > 0) {
      double f = d.m.staticScale[m];
      double inc[6] = {0, 0, 0, 0, 0, 0};
      int d0 = d.triFirstDof[i], nd = d.triNdof[i];
      for (int k = 0; k < nd && k < 6; ++k) {
        int eq = d.meqn[d0 + k];
        inc[k] = eq >= 0 ? d.del[eq] * f : 0.0;
      }
      double* U = d.ur + 12 * (size_t)i;
      for (int r = 0; r < 3; ++r) U[9 + r] += inc[r];
      if (nd == 6) {
        double R[9], O[9];
        rotvecToMat(inc + 3, R);
        for (int c = 0; c < 3; ++c)
          for (int r = 0; r < 3; ++r) O[r + 3 * c] = R[r] * U[3 * c] + R[r + 3] * U[3 * c + 1] + R[r + 6] * U[3 * c + 2];
        for (int k = 0; k < 9; ++k) U[k] = O[k];
      }
    }
  }
}

// convergence logic of the static iterations (staticEquilibriumModule.f90:262-371)
__global__ void kStaticFinish(DevModels m) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m.n) return;
  if (!(m.flags[i] & FL_STATIC)) return;
  if (m.status[i] & (SS_SINGULAR | SS_COROT)) { m.state[i] = ST_ERROR; m.staticDone[i] = 1; return; }
  int it = m.staticIter[i] + 1;
  m.staticIter[i] = it;
  double deln = m.deln[i];
  if (!(deln <= 1.0e300)) { m.status[i] |= SS_NAN; m.state[i] = ST_ERROR; m.staticDone[i] = 1; return; }
  if (m.staticMode[i] == 1) { m.staticDone[i] = 1; return; }
  if (deln < m.equTol[i] && it >= m.minIt[i]) { m.staticDone[i] = 1; return; }
  if (deln > m.equLim[i]) {  // restart the iteration loop with the scaled step
    m.staticIter[i] = 0;
    int ninc = m.staticNinc[i] + 1;
    m.staticNinc[i] = ninc;
    if (ninc >= m.maxIt[i]) { m.status[i] |= SS_MAXIT; m.state[i] = ST_ERROR; m.staticDone[i] = 1; }
    return;
  }
  if (it >= m.maxIt[i]) m.staticDone[i] = 1;  // accepted without full convergence
}

}  // namespace

void launchBeginStep(const DevData& d, int* activeCount, long long* activeEl, cudaStream_t s) {
  kBeginStep<<<blocksFor(d.m.n, 128), 128, 0, s>>>(d.m, activeCount, activeEl);
}
void launchPredictDofs(const DevData& d, cudaStream_t s) {
  long long n = d.ndofTot > d.neqTot ? d.ndofTot : d.neqTot;
  kPredictDofs<<<blocksFor(n), TPB, 0, s>>>(d);
}
void launchElements(const DevData& d, int mode, cudaStream_t s) {
  if (d.nelTot > 0) kElements<<<blocksFor(d.nelTot, 128), 128, 0, s>>>(d, mode);
}
void launchResidual(const DevData& d, cudaStream_t s) {
  if (d.neqTot > 0) kResidual<<<blocksFor(d.neqTot), TPB, 0, s>>>(d);
}
void launchBuildElementNewton(const DevData& d, cudaStream_t s) {
  if (d.nelTot > 0) kBuildElementNewton<<<blocksFor(d.nelTot), TPB, 0, s>>>(d);
}
void launchRotateElementNewton(const DevData& d, cudaStream_t s) {
  if (d.nelTot > 0) kRotateElementNewton<<<blocksFor(d.nelTot, 128), 128, 0, s>>>(d);
}
void launchCsrGather(const DevData& d, cudaStream_t s) {
  if (d.nslotTot > 0) kCsrGather<<<blocksFor(d.nslotTot), TPB, 0, s>>>(d);
}
void launchIncrement(const DevData& d, cudaStream_t s) {
  long long n = d.ndofTot > d.ntriTot ? d.ndofTot : d.ntriTot;
  kIncrement<<<blocksFor(n), TPB, 0, s>>>(d);
}
void launchNormsControl(const DevData& d, cudaStream_t s) {
  if (d.nchunkTot > 0) kNormsPartial<<<d.nchunkTot, CHUNK_TPB, 0, s>>>(d);
  kControl<<<blocksFor(d.m.n, 128), 128, 0, s>>>(d);
  long long n = d.ntriTot > d.nelTot ? d.ntriTot : d.nelTot;
  kStepEnd<<<blocksFor(n), TPB, 0, s>>>(d);
}
void launchStaticBegin(const DevData& d, int* activeCount, cudaStream_t s) {
  kStaticBegin<<<blocksFor(d.m.n, 128), 128, 0, s>>>(d.m, activeCount);
}
void launchStaticResidual(const DevData& d, cudaStream_t s) {
  if (d.neqTot > 0) kStaticResidual<<<blocksFor(d.neqTot), TPB, 0, s>>>(d);
}
void launchStaticNorm(const DevData& d, cudaStream_t s) { kStaticNorm<<<d.m.n, NTPB, 0, s>>>(d); }
void launchStaticIncrement(const DevData& d, cudaStream_t s) {
  long long n = d.ndofTot > d.ntriTot ? d.ndofTot : d.ntriTot;
  kStaticIncrement<<<blocksFor(n), TPB, 0, s>>>(d);
}
void launchStaticFinish(const DevData& d, cudaStream_t s) {
  kStaticFinish<<<blocksFor(d.m.n, 128), 128, 0, s>>>(d.m);
}

}  // namespace fgpu
