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

#include <algorithm>
#include <mutex>

#include "kernels.h"
#include "rotation.cuh"

namespace fgpu {
namespace {

constexpr int TPB = 256;

inline int blocksFor(long long n, int tpb = TPB) { return (int)((n + tpb - 1) / tpb); }

// re-orthonormalise a rotation tensor through its quaternion (Spurrier)
__device__ inline void orthonormRot(double* R /* col-major 3x3 */) {
  auto r = [&](int i, int j) { return R[i + 3 * j]; };
  double q[4];
  double tr = r(0, 0) + r(1, 1) + r(2, 2);
  int imax = 0;
  if (r(1, 1) > r(imax, imax)) imax = 1;
  if (r(2, 2) > r(imax, imax)) imax = 2;
  // one reciprocal for the three off-diagonal components and one reciprocal
  // square root for the normalisation
  if (tr > r(imax, imax)) {
    q[0] = sqrt(1.0 + tr) * 0.5;
    const double f = 1.0 / (4.0 * q[0]);
    q[1] = (r(2, 1) - r(1, 2)) * f;
    q[2] = (r(0, 2) - r(2, 0)) * f;
    q[3] = (r(1, 0) - r(0, 1)) * f;
  } else {
    int i = imax, j = (imax + 1) % 3, k = (imax + 2) % 3;
    q[i + 1] = sqrt(r(i, i) * 0.5 + (1.0 - tr) * 0.25);
    const double f = 1.0 / (4.0 * q[i + 1]);
    q[0] = (r(k, j) - r(j, k)) * f;
    q[j + 1] = (r(j, i) + r(i, j)) * f;
    q[k + 1] = (r(k, i) + r(i, k)) * f;
  }
  const double inv = rsqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  for (int a = 0; a < 4; ++a) q[a] *= inv;
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

// value of a dependent DOF (a joint's slave triad) from the equation vector eqv
// scaled by f: its row of the joint's constraint coefficients (csExpand,
// solExtensionModule.f90:1352-1387; the constant term of a joint is zero)
__device__ inline double dependentValue(const DevData& d, int dd, const double* eqv, double f) {
  const int j = dd / 6, r = dd % 6;
  const double* T = d.jT + 72 * (size_t)j + 12 * r;
  const int* ce = d.jColEq + 12 * j;
  const int nc = d.jNcol[j];
  double s = 0.0;
  for (int c = 0; c < nc; ++c) {
    const int q = ce[c];
    if (q >= 0) s += T[c] * (eqv[q] * f);
  }
  return s;
}

// ---------------------------------------------------------------------------
// per-model control at the start of a batched iteration
// ---------------------------------------------------------------------------
// the roots of model i into every backward queue, and its chain count
__device__ inline void seedBackward(const BackwardSeed& b, int i) {
  for (int q = 0; q < b.nq; ++q) {
    const int r0 = b.rootOff[i], nr = b.rootOff[i + 1] - r0;
    int* ctr = b.ctr + 4 * q;
    int* queue = b.queue + (size_t)q * b.stride;
    const int base = atomicAdd(ctr + 1, nr);
    for (int k = 0; k < nr; ++k) queue[base + k] = b.roots[r0 + k];
    atomicAdd(ctr + 2, b.slotCnt[i]);
    if (b.strideL > 0) {  // the large roots into the large-front queue
      const int l0 = b.rootOffL[i], nl = b.rootOffL[i + 1] - l0;
      int* ctrL = b.ctrL + 4 * q;
      int* queueL = b.queueL + (size_t)q * b.strideL;
      const int baseL = atomicAdd(ctrL + 1, nl);
      for (int k = 0; k < nl; ++k) queueL[baseL + k] = b.rootsL[l0 + k];
      atomicAdd(ctrL + 2, b.slotCntL[i]);
    }
  }
}

__global__ void kBeginStep(DevModels m, int* activeCount, long long* activeEl, BackwardSeed bs) {
  pdlEntry();
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
    fl = FL_ACTIVE | FL_PRED;
    if (t + dt < m.tQs[i] + 0.1 * m.minInc[i]) {
      // quasi-static load step (solverModule.f90:826-841, isQuasiStatic)
      fl |= FL_QSTATIC;
      if (m.fixedIt[i] == -1) fl |= FL_LINEAR;
      m.qsCount[i] += 1;
    } else {
      if (m.qsCount[i] > 0) fl |= FL_QS2DYN;
      m.qsCount[i] = 0;
      m.pc[4 * i + 0] = ga / be - 1.0;
      m.pc[4 * i + 1] = (0.5 * ga / be - 1.0) * dt;
      m.pc[4 * i + 2] = 1.0 / (be * dt);
      m.pc[4 * i + 3] = 0.5 / be - 1.0;
      m.sacc[i] = 1.0 / (be * dt * dt);
      m.svel[i] = ga / (be * dt);
    }
    m.state[i] = ST_ITER;
  } else if (st == ST_ITER) {
    fl = FL_ACTIVE | (m.flags[i] & (FL_QSTATIC | FL_LINEAR));
  } else {
    m.flags[i] = 0;
    return;
  }
  int it = m.iter[i];
  bool tangent = it < max(1, m.nUpdat[i]) || m.nSeqNoUpd[i] >= m.maxSeq[i];
  if (tangent) {
    fl |= FL_TANGENT;
    double sK = m.alpha[i] + 1.0, sC = m.svel[i] * sK, sM = m.sacc[i];
    if (fl & FL_QSTATIC) { sM = 0.0; sK = 1.0; sC = 0.0; }  // stiffness only
    double* sn = m.scaleN + 3 * i;
    if (fabs(sM - sn[0]) + fabs(sK - sn[1]) + fabs(sC - sn[2]) > 1.0e-16) {
      sn[0] = sM; sn[1] = sK; sn[2] = sC;
      fl |= FL_REBUILD;
    }
  }
  m.flags[i] = fl;
  atomicAdd(activeCount, 1);
  atomicAdd(reinterpret_cast<unsigned long long*>(activeEl), (unsigned long long)m.nel[i]);
  seedBackward(bs, i);
}

// predicted velocity/acceleration increments and the actual inertia force
__global__ void kPredictDofs(DevData d) {
  pdlEntry();
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < d.ndofTot) {
    int m = d.dofModel[i];
    const int fl = d.m.flags[m];
    if ((fl & FL_PRED) && !(fl & FL_QSTATIC)) {
      const double* pc = d.m.pc + 4 * m;
      double v = d.urd[i], a = d.urdd[i];
      if (fl & FL_QS2DYN) {
        // starting velocity after quasi-static steps (solverModule.f90:850)
        v = d.rinc[i] / d.m.dt[m];
        d.urd[i] = v;
      }
      d.dk[i] = pc[0] * v + pc[1] * a;
      d.ak[i] = pc[2] * v + pc[3] * a;
      d.rinc[i] = 0.0;
    } else if (fl & FL_PRED) {
      d.rinc[i] = 0.0;
    }
  }
  if (i < d.neqTot) {
    int m = d.eqModel[i];
    if (d.m.flags[m] & FL_PRED) {
      // FIactual = FIk of the converged previous step (NewmarkFlag = 0)
      double s = 0.0;
      const double* FI = d.Fel + (size_t)24 * d.nelTot;
      const int beamLim = 12 * d.nelTot;  // axial elements have no inertia forces
      const int xLim = beamLim + 6 * d.naxTot;  // expanded forces of elements with a dependent triad
      for (int k = d.eqPtr[i]; k < d.eqPtr[i + 1]; ++k) {
        const int src = d.eqSrc[k];
        if (src < beamLim) s += FI[src];
        else if (src >= xLim) s += d.FelX[src - xLim + 2];
      }
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
  pdlEntry();
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
  // quasi-static steps: no velocity terms; pure linear ones keep the frame
  const bool qs = (mode == EM_PRED || mode == EM_INC) && (fl & FL_QSTATIC);
  const bool isStatic = mode == EM_STATIC || mode == EM_STATIC_INIT || qs;
  double S[12];
#pragma unroll
  for (int k = 0; k < 12; ++k) S[k] = d.supTr[(size_t)k * nel + e];
  int tri[2] = {d.elTri[e], d.elTri[nel + e]};
  double uld[12], uldd[12];
  // the damping force is the only user of the local velocities (stiffness-proportional
  // damping C, or the kDmp term of the pass after the increment)
  const bool needUld =
      !isStatic && (d.hasC[e] || ((mode == EM_INC || mode == EM_PRED) && d.hasVld[e] && d.m.dt[m] > 0.0));
  if (!isStatic) {
    const double* vs = mode == EM_PRED ? d.dk : d.urd;
    const double* as = mode == EM_PRED ? d.ak : d.urdd;
#pragma unroll
    for (int n = 0; n < 2; ++n) {
      int d0 = d.triFirstDof[tri[n]];
#pragma unroll
      for (int g = 0; g < 2; ++g) {
        double a0 = as[d0 + 3 * g], a1 = as[d0 + 3 * g + 1], a2 = as[d0 + 3 * g + 2];
#pragma unroll
        for (int r = 0; r < 3; ++r)
          uldd[6 * n + 3 * g + r] = S[3 * r] * a0 + S[3 * r + 1] * a1 + S[3 * r + 2] * a2;
        if (needUld) {
          double v0 = vs[d0 + 3 * g], v1 = vs[d0 + 3 * g + 1], v2 = vs[d0 + 3 * g + 2];
#pragma unroll
          for (int r = 0; r < 3; ++r)
            uld[6 * n + 3 * g + r] = S[3 * r] * v0 + S[3 * r + 1] * v1 + S[3 * r + 2] * v2;
        }
      }
    }
  }
  const bool newPositions = (mode == EM_INC || mode == EM_STATIC || mode == EM_FINAL) && !(qs && (fl & FL_LINEAR));
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
    // unit vectors: one reciprocal square root per length, then products
    const double ilx = rsqrt(lx), ilz = rsqrt(lz);
#pragma unroll
    for (int k = 0; k < 3; ++k) { ex[k] *= ilx; ez[k] *= ilz; }
    crossd(ez, ex, ey);
    double T[12] = {ex[0], ex[1], ex[2], ey[0], ey[1], ey[2], ez[0], ez[1], ez[2], p[0][0], p[0][1], p[0][2]};
    double Rel[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) Rel[k] = d.triRelSup[(size_t)k * nel + e];
    compose34(T, Rel, S);
#pragma unroll
    for (int k = 0; k < 12; ++k) d.supTr[(size_t)k * nel + e] = S[k];
  }
  if (newPositions || mode == EM_STATIC_INIT || qs) {
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
  const bool keepFsQ = mode == EM_PRED && !qs;
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
    // Fd = stifScl * C * uld  (- kDmp * stifScl * K * (uld - vld)); exactly zero without damping.
    // The rigid-body filtering applies in the predictor too (UpdateSupEls is
    // called with the step size there), where the deformation is the previous
    // step's and vld is zero.
    const double dt = d.m.dt[m];
    const bool vldActive = (mode == EM_INC || mode == EM_PRED) && d.hasVld[e] && dt > 0.0;
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

// axial springs and dampers: direction, length, forces (UpdateSprings/UpdateDampers,
// calcSpringForces, addInDampingForces, calcDamperForces); same pass gating as kElements
__global__ void kAxial(DevData d, int mode) {
  pdlEntry();
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  const int nax = d.naxTot;
  if (a >= nax) return;
  const int m = d.axModel[a], fl = d.m.flags[m];
  if (mode == EM_PRED) {
    if (!(fl & FL_PRED)) return;
  } else if (mode == EM_INC) {
    if (!(fl & FL_ACTIVE)) return;
  } else if (mode == EM_STATIC || mode == EM_STATIC_INIT) {
    if (!(fl & FL_STATIC)) return;
  }
  const bool qs = (mode == EM_PRED || mode == EM_INC) && (fl & FL_QSTATIC);
  const bool isStatic = mode == EM_STATIC || mode == EM_STATIC_INIT || qs;
  const int t1 = d.axTri[a], t2 = d.axTri[nax + a];
  const double* U1 = d.ur + 12 * (size_t)t1;
  const double* U2 = d.ur + 12 * (size_t)t2;
  double dv[3] = {U2[9] - U1[9], U2[10] - U1[10], U2[11] - U1[11]}, n[3];
  const double l2 = dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2];
  const double L = sqrt(l2);
  const bool spring = d.axKind[a] == 0;
  if (l2 < 1.0e-16) {
    if (spring) {
      atomicOr(&d.m.status[m], SS_COROT);  // the two points defining the spring coincide
      return;
    }
    n[0] = n[1] = n[2] = 0.0;
  } else {
#pragma unroll
    for (int k = 0; k < 3; ++k) n[k] = dv[k] / L;
  }
  double v1[3] = {0, 0, 0}, v2[3] = {0, 0, 0};
  if (!isStatic) {
    const double* vs = mode == EM_PRED ? d.dk : d.urd;  // predicted velocities in the predictor
    const int f1 = d.triFirstDof[t1], f2 = d.triFirstDof[t2];
#pragma unroll
    for (int k = 0; k < 3; ++k) { v1[k] = vs[f1 + k]; v2[k] = vs[f2 + k]; }
  }
  double fs[6] = {0, 0, 0, 0, 0, 0}, fd[6] = {0, 0, 0, 0, 0, 0};
  if (spring) {
    const double F = d.axS0[a] * (L - d.axL0[a]);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      fs[k] = 0.0 - F * n[k];
      fs[3 + k] = 0.0 + F * n[k];
    }
    const double al = d.axAlpha2[a];
    if (!isStatic && fabs(al) > 1.0e-16) {
      const double km = d.axS0[a] * al * L / L;
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        double f1 = 0.0, f2 = 0.0;
#pragma unroll
        for (int j = 0; j < 3; ++j) f1 += n[i] * n[j] * km * v1[j];
#pragma unroll
        for (int j = 0; j < 3; ++j) f1 += -(n[i] * n[j] * km) * v2[j];
#pragma unroll
        for (int j = 0; j < 3; ++j) f2 += -(n[i] * n[j] * km) * v1[j];
#pragma unroll
        for (int j = 0; j < 3; ++j) f2 += n[i] * n[j] * km * v2[j];
        fd[i] = f1;
        fd[3 + i] = f2;
      }
    }
  } else {
    const double vr[3] = {v2[0] - v1[0], v2[1] - v1[1], v2[2] - v1[2]};
    const double F = d.axD0[a] * (n[0] * vr[0] + n[1] * vr[1] + n[2] * vr[2]);
    if (!isStatic)
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        fd[k] = -F * n[k];
        fd[3 + k] = -fd[k];
      }
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) d.axN[(size_t)k * nax + a] = n[k];
  d.axLen[a] = L;
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    d.FelA[(size_t)k * nax + a] = fs[k];
    d.FelA[(size_t)(6 + k) * nax + a] = fd[k];
  }
}

// axial element Newton matrices [A -A; -A A], A = n n^T (s0 (sK + sC alpha2)) for a
// spring (calcSpringStiffness, no geometric stiffness) or n n^T d0 sC for a damper
// (addInDamperMat)
__global__ void kAxialNewton(DevData d) {
  pdlEntry();
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  const int nax = d.naxTot;
  if (a >= nax) return;
  const int m = d.axModel[a];
  if (!(d.m.flags[m] & FL_TANGENT)) return;
  const double* sn = d.m.scaleN + 3 * m;  // sM, sK, sC
  const double sK = sn[1], sC = sn[2];
  double n[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) n[k] = d.axN[(size_t)k * nax + a];
  const double L = d.axLen[a];
  double A[9];
  if (d.axKind[a] == 0) {
    const double km = (d.axS0[a] * (sK + sC * d.axAlpha2[a])) * L / L;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) A[i + 3 * j] = n[i] * n[j] * km;
  } else {
    const double c = d.axD0[a];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) A[i + 3 * j] = n[i] * n[j] * c * sC;
  }
#pragma unroll
  for (int j = 0; j < 6; ++j)
#pragma unroll
    for (int i = 0; i < 6; ++i) {
      const double v = A[(i % 3) + 3 * (j % 3)];
      d.elMatA[(size_t)(i + 6 * j) * nax + a] = (i / 3 == j / 3) ? v : -v;
    }
}

// residual: force predictor (7.53) or corrector (7.55); RHS del = residual
__global__ void kResidual(DevData d) {
  pdlEntry();
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.neqTot) return;
  // the list of the equation's first two contributions is read with the model's
  // flags, before the activity test, to save a dependent round trip
  const int m = d.eqModel[i];
  const int k0 = d.eqPtr[i], k1 = d.eqPtr[i + 1];
  const size_t s0 = k0 < k1 ? (size_t)d.eqSrc[k0] : 0, s1 = k0 + 1 < k1 ? (size_t)d.eqSrc[k0 + 1] : 0;
  const int fl = d.m.flags[m];
  if (!(fl & FL_ACTIVE)) return;
  const size_t blk = (size_t)12 * d.nelTot, ablk = (size_t)6 * d.naxTot;
  double fs = 0.0, fd = 0.0, fi = 0.0, q = 0.0;
  // one contribution: element forces FS, FD, FI, Q, or FS, FD of an axial spring/damper
  auto add = [&](double v0, double v1, double v2, double v3, bool el) {
    fs += v0;
    fd += v1;
    if (el) {
      fi += v2;
      q += v3;
    }
  };
  auto load = [&](size_t s, double& v0, double& v1, double& v2, double& v3) {
    if (s >= blk + ablk) {  // expanded forces (FS, FD, FI, Q interleaved)
      const double* b = d.FelX + (s - blk - ablk);
      v0 = b[0];
      v1 = b[1];
      v2 = b[2];
      v3 = b[3];
      return true;
    }
    const bool el = s < blk;
    const double* b = el ? d.Fel + s : d.FelA + (s - blk);
    const size_t st = el ? blk : ablk;
    v0 = b[0];
    v1 = b[st];
    v2 = el ? b[2 * st] : 0.0;
    v3 = el ? b[3 * st] : 0.0;
    return el;
  };
  // equations of beam chains have one or two contributions: the loads of the first
  // two are issued together; the sums keep the order of the list
  double a0 = 0, a1 = 0, a2 = 0, a3 = 0, b0 = 0, b1 = 0, b2 = 0, b3 = 0;
  bool ea = false, eb = false;
  if (k0 < k1) ea = load(s0, a0, a1, a2, a3);
  if (k0 + 1 < k1) eb = load(s1, b0, b1, b2, b3);
  if (k0 < k1) add(a0, a1, a2, a3, ea);
  if (k0 + 1 < k1) add(b0, b1, b2, b3, eb);
  for (int k = k0 + 2; k < k1; ++k) {
    double c0, c1, c2, c3;
    const bool ec = load((size_t)d.eqSrc[k], c0, c1, c2, c3);
    add(c0, c1, c2, c3, ec);
  }
  q += d.qext[i];
  // forces set by an external process (newmarkRoutinesModule.f90:747-749, 792-794);
  // they apply to the iterations of one step (solverModule.f90:880-882)
  if (fl & FL_PRED)
    d.extRhs[i] = 0.0;
  else
    q += d.extRhs[i];
  d.FSk[i] = fs;
  d.FDk[i] = fd;
  d.FIk[i] = fi;
  d.Qk[i] = q;
  double a = d.m.alpha[m], sstif = a + 1.0, r;
  if (fl & FL_QSTATIC)  // staticEquilibriumModule.f90 (staticInt): Q alone in a pure linear step
    r = ((fl & FL_LINEAR) && (fl & FL_PRED)) ? q : q - fs;
  else if (fl & FL_PRED)
    r = sstif * (q - fs + fd) + fi - a * d.FIact[i];
  else
    r = sstif * (q - fs - fd) - fi - a * d.FIact[i];
  d.res[i] = r;
  d.del[i] = r;
}

// element Newton matrix N = sM*M + sC*stifScl*C + sK*stifScl*K (rebuilt when the scales change)
__global__ void kBuildElementNewton(DevData d) {
  pdlEntry();
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
  pdlEntry();
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

// Beam batches in principal axes (26-value pattern): N = sM*M + sC*stifScl*C +
// sK*stifScl*K built on the fly and rotated block by block.  Each 3x3 block of
// N is diagonal (translations/rotations of one direction) or holds one
// off-diagonal pair (bending coupling), so R B R^T costs 2-3 products per
// entry instead of 6 for a dense block; only the 10 upper blocks are computed
// and the lower ones written as their transposes (an exactly symmetric Ns).
__device__ inline void storeBlock(double* out, int nel, int e, int bi, int bj, const double* S) {
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      out[(size_t)((3 * bi + r) + 12 * (3 * bj + c)) * nel + e] = S[r + 3 * c];
      if (bi != bj) out[(size_t)((3 * bj + c) + 12 * (3 * bi + r)) * nel + e] = S[r + 3 * c];
    }
}

// R diag(b) R^T (symmetric)
__device__ inline void rotDiag(const double* R, double b0, double b1, double b2, double* S) {
  double W[9];
#pragma unroll
  for (int r = 0; r < 3; ++r) { W[r] = R[r] * b0; W[r + 3] = R[r + 3] * b1; W[r + 6] = R[r + 6] * b2; }
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int r = 0; r <= c; ++r) {
      double v = W[r] * R[c] + W[r + 3] * R[c + 3] + W[r + 6] * R[c + 6];
      S[r + 3 * c] = v;
      S[c + 3 * r] = v;
    }
}

// R B R^T with B_12 = p, B_21 = q (0-based rows/cols 1 and 2), all else zero
__device__ inline void rotPair(const double* R, double p, double q, double* S) {
  double W1[3], W2[3];
#pragma unroll
  for (int r = 0; r < 3; ++r) { W1[r] = R[r + 6] * q; W2[r] = R[r + 3] * p; }
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int r = 0; r < 3; ++r) S[r + 3 * c] = W1[r] * R[c + 3] + W2[r] * R[c + 6];
}

__global__ void __launch_bounds__(128) kNewtonBeam(DevData d) {
  pdlEntry();
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  const int nel = d.nelTot;
  if (e >= nel) return;
  const int m = d.elModel[e];
  if (!(d.m.flags[m] & FL_TANGENT)) return;
  const double* sn = d.m.scaleN + 3 * m;
  const double ss = d.stifScl[e];
  const double sM = sn[0], sK = sn[1] * ss, sC = sn[2] * ss;
  const bool hc = d.hasC[e];
  double a[26];
#pragma unroll
  for (int k = 0; k < 26; ++k) {
    const size_t ix = (size_t)k * nel + e;
    double v = sM * d.M26[ix];
    if (hc) v += sC * d.C26[ix];
    v += sK * d.K26[ix];
    a[k] = v;
  }
  double R[9], S[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) R[k] = d.supTr[(size_t)k * nel + e];
  double* out = d.elMat;
  rotDiag(R, a[0], a[2], a[6], S);    storeBlock(out, nel, e, 0, 0, S);
  rotPair(R, a[3], a[7], S);          storeBlock(out, nel, e, 0, 1, S);
  rotDiag(R, a[1], a[4], a[8], S);    storeBlock(out, nel, e, 0, 2, S);
  rotPair(R, a[5], a[9], S);          storeBlock(out, nel, e, 0, 3, S);
  rotDiag(R, a[10], a[12], a[15], S); storeBlock(out, nel, e, 1, 1, S);
  rotPair(R, a[13], a[16], S);        storeBlock(out, nel, e, 1, 2, S);
  rotDiag(R, a[11], a[14], a[17], S); storeBlock(out, nel, e, 1, 3, S);
  rotDiag(R, a[18], a[19], a[21], S); storeBlock(out, nel, e, 2, 2, S);
  rotPair(R, a[20], a[22], S);        storeBlock(out, nel, e, 2, 3, S);
  rotDiag(R, a[23], a[24], a[25], S); storeBlock(out, nel, e, 3, 3, S);
}

// CSR slot gather (deterministic segmented reduction over element contributions)
// The block of kSlotBlock slots runs on kSlotBlock / 4 threads, four slots a thread.
// Each CSR slot of a beam chain has one or two contributions, so the slot pointers,
// the first two source indices and their values are loaded in three rounds with
// every load of a round independent; longer lists continue one by one. The sum keeps
// the order of the list (v = 0, then += each contribution).
constexpr int kGatherSlotsPerThread = 4;

__device__ __forceinline__ double gatherEntry(const DevData& d, int src, int64_t lim) {
  if (src < lim) return d.elMat[src];
  const int64_t lim2 = lim + (int64_t)36 * d.naxTot;  // expanded matrices of elements with a dependent triad
  return src < lim2 ? d.elMatA[src - lim] : d.elMatX[src - lim2];
}

// Grid-stride over the blocks of kSlotBlock slots with a grid of resident blocks only:
// in iterations where few or no models update the tangent, the slot blocks of the
// other models are skipped by a flag test (32 slot blocks per round of loads)
// instead of a block launch each.
__global__ void __launch_bounds__(kSlotBlock / kGatherSlotsPerThread) kCsrGather(DevData d, int nSlotBlocks) {
  pdlEntry();
  constexpr int R = kGatherSlotsPerThread;
  const int64_t lim = (int64_t)144 * d.nelTot;
  const int lane = threadIdx.x & 31;
  for (int b0 = blockIdx.x; b0 < nSlotBlocks; b0 += 32 * gridDim.x) {
    // lane j of each warp tests slot block b0 + j * gridDim.x (its model's flags, or
    // every slot's when the block spans several models); the ballot is the same in
    // every warp of the block, which then works through the selected slot blocks
    const int bj = b0 + lane * gridDim.x;
    int bmj = -1;
    bool sel = false;
    if (bj < nSlotBlocks) {
      bmj = d.slotBlockModel[bj];
      sel = bmj < 0 || (d.m.flags[bmj] & FL_TANGENT);
    }
    unsigned pending = __ballot_sync(0xffffffffu, sel);
    while (pending) {
      const int j = __ffs(pending) - 1;
      pending &= pending - 1;
      const int b = b0 + j * (int)gridDim.x;
      const int bm = __shfl_sync(0xffffffffu, bmj, j);
      int64_t sl[R];
      int p0[R], p1[R], at[R], i0[R], i1[R];
      double c0[R], c1[R];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        sl[r] = (int64_t)b * kSlotBlock + r * (kSlotBlock / R) + threadIdx.x;
        p0[r] = p1[r] = 0;
        at[r] = -1;
        if (sl[r] < d.nslotTot && (bm >= 0 || (d.m.flags[d.slotModel[sl[r]]] & FL_TANGENT))) {
          p0[r] = d.slotPtr[sl[r]];
          p1[r] = d.slotPtr[sl[r] + 1];
          at[r] = d.slotAsm[sl[r]];
        } else {
          sl[r] = -1;
        }
      }
#pragma unroll
      for (int r = 0; r < R; ++r) {
        i0[r] = p0[r] < p1[r] ? d.slotSrc[p0[r]] : 0;
        i1[r] = p0[r] + 1 < p1[r] ? d.slotSrc[p0[r] + 1] : 0;
      }
#pragma unroll
      for (int r = 0; r < R; ++r) {
        c0[r] = p0[r] < p1[r] ? gatherEntry(d, i0[r], lim) : 0.0;
        c1[r] = p0[r] + 1 < p1[r] ? gatherEntry(d, i1[r], lim) : 0.0;
      }
#pragma unroll
      for (int r = 0; r < R; ++r) {
        if (sl[r] < 0) continue;
        double v = 0.0;
        if (p0[r] < p1[r]) v += c0[r];
        if (p0[r] + 1 < p1[r]) v += c1[r];
        for (int k = p0[r] + 2; k < p1[r]; ++k) v += gatherEntry(d, d.slotSrc[k], lim);
        d.csrVal[sl[r]] = v;
        // front-ordered copy for the factorisation, in its precision
        if (at[r] >= 0) {
          if (d.asmVal32) d.asmVal32[at[r]] = (float)v;
          else d.asmVal64[at[r]] = v;
        }
      }
    }
  }
}

// increment: expand the solution, update velocities/accelerations and triads
// threads [0, ntriTot) update a triad each (rotation increments: the heavier
// work, in the first blocks), threads [ntriTot, ntriTot + ndofTot) a DOF each
__global__ void kIncrement(DevData d) {
  pdlEntry();
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long i = t - d.ntriTot;
  if (t >= d.ntriTot && i < d.ndofTot) {
    int m = d.dofModel[i];
    const int fl = d.m.flags[m];
    if (fl & FL_ACTIVE) {
      int eq = d.meqn[i];
      // prescribed DOFs take their constraint value in the predictor and zero in
      // corrector steps (solExtensionModule.f90:1352-1387); fixed DOFs are zero;
      // dependent DOFs their joint's constraint equation
      double s0 = eq >= 0 ? d.del[eq]
                          : (eq <= -2 && (fl & FL_PRED)) ? d.motCc[d.modelMotOff[m] - 2 - eq] : 0.0;
      if (eq == -1 && d.dofDep && d.dofDep[i] >= 0) s0 = dependentValue(d, d.dofDep[i], d.del, 1.0);
      d.sinc0[i] = s0;
      double ri = d.rinc[i] + s0;
      d.rinc[i] = ri;
      if (fl & FL_QSTATIC) {
        d.sinc1[i] = 0.0;
        d.sinc2[i] = 0.0;
      } else {
        double sv = d.m.svel[m], sa = d.m.sacc[m];
        d.sinc1[i] = s0 * sv;
        d.sinc2[i] = s0 * sa;
        d.urd[i] = sv * ri - d.dk[i];
        d.urdd[i] = sa * ri - d.ak[i];
      }
    }
  }
  if (t < d.ntriTot) {
    const long long i = t;
    int m = d.triModel[i];
    if ((d.m.flags[m] & FL_ACTIVE) && d.triNdof[i] > 0) {
      double inc[6] = {0, 0, 0, 0, 0, 0};
      int d0 = d.triFirstDof[i], nd = d.triNdof[i];
      const bool pred = d.m.flags[m] & FL_PRED;
      for (int k = 0; k < nd && k < 6; ++k) {
        int eq = d.meqn[d0 + k];
        inc[k] = eq >= 0 ? d.del[eq] : (eq <= -2 && pred) ? d.motCc[d.modelMotOff[m] - 2 - eq] : 0.0;
        if (eq == -1 && d.dofDep && d.dofDep[d0 + k] >= 0) inc[k] = dependentValue(d, d.dofDep[d0 + k], d.del, 1.0);
      }
      double* U = d.ur + 12 * (size_t)i;
      for (int r = 0; r < 3; ++r) U[9 + r] += inc[r];
      if (nd == 6) {
        double R[9], O[9];
        rotvecToMat(inc + 3, d.sinEpsOverEps, R);
        for (int c = 0; c < 3; ++c)
          for (int r = 0; r < 3; ++r) O[r + 3 * c] = R[r] * U[3 * c] + R[r + 3] * U[3 * c + 1] + R[r + 6] * U[3 * c + 2];
        for (int k = 0; k < 9; ++k) U[k] = O[k];
      }
    }
  }
}

// prescribed deflections at the start of a step (motionRoutinesModule.f90:58-193):
// cc = D - Dprev, or the total D in a linear quasi-static step
__global__ void kMotions(DevData d) {
  pdlEntry();
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= d.nmotTot) return;
  const int m = d.motModel[k], fl = d.m.flags[m];
  if (!(fl & FL_PRED)) return;
  const int ch = d.motCh[k];
  const double D = d.motD0[k] + d.motD1[k] * (ch >= 0 ? d.extVal[ch] : d.motEA[k] * d.m.time[m] + d.motEB[k]);
  d.motCc[k] = (fl & FL_LINEAR) ? D : D - d.motD[k];
  d.motD[k] = D;
}

// engine-driven point loads at the new time (forceRoutinesModule.f90:52-131)
__global__ void kLoads(DevData d) {
  pdlEntry();
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= d.nldTot) return;
  const int eq = d.ldEq[k], m = d.eqModel[eq];
  if (!(d.m.flags[m] & FL_PRED)) return;
  const double t = d.m.time[m];
  double q = d.qextBase[eq];
  for (int j = d.ldPtr[k]; j < d.ldPtr[k + 1]; ++j) {
    const int ch = d.ldCh[j];
    double ev = ch >= 0 ? d.extVal[ch] : d.ldEA[j] * t + d.ldEB[j];
    const double* sp = d.ldSin + 4 * (size_t)j;
    if (sp[2] != 0.0 || sp[3] != 0.0) ev += sp[3] + sp[2] * sin(2.0 * M_PI * (sp[0] * t - sp[1]));
    q += d.ldF0[j] + d.ldF1[j] * ev;
  }
  d.qext[eq] = q;
}

// predictor right-hand side: the prescribed values times the Newton matrix
// columns of the prescribed DOFs, moved to the right-hand side (terms with
// |cc| <= 1e-15 skipped, sysMatrixTypeModule.f90:2099-2259)
__global__ void kMotionRhs(DevData d) {
  pdlEntry();
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= d.nmrTot) return;
  const int eq = d.mrEq[k];
  if (!(d.m.flags[d.eqModel[eq]] & FL_PRED)) return;
  double b = d.del[eq];
  for (int64_t q = d.mrPtr[k]; q < d.mrPtr[k + 1]; ++q) {
    const double c = d.motCc[d.mrMot[q]];
    const int64_t src = d.mrSrc[q], lim = (int64_t)144 * d.nelTot;
    if (fabs(c) > 1.0e-15) b -= c * gatherEntry(d, (int)src, lim);
  }
  d.del[eq] = b;
}

// a pure linear quasi-static step restarts from the state after the initial
// configuration (restoreLastStep, solverRoutinesModule.f90:920-970)
__global__ void kQsRestore(DevData d) {
  pdlEntry();
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int want = FL_PRED | FL_QSTATIC | FL_LINEAR;
  if (i < d.ntriTot && (d.m.flags[d.triModel[i]] & want) == want)
    for (int k = 0; k < 12; ++k) d.ur[12 * i + k] = d.urQs[12 * i + k];
  if (i < d.nelTot && (d.m.flags[d.elModel[i]] & want) == want)
    for (int k = 0; k < 12; ++k) {
      size_t ix = (size_t)k * d.nelTot + i;
      d.supTr[ix] = d.supTrQs[ix];
      d.finit[ix] = d.finitPrev[ix];
    }
  if (i < d.ndofTot && (d.m.flags[d.dofModel[i]] & want) == want) {
    d.urd[i] = d.urdQs[i];
    d.urdd[i] = d.urddQs[i];
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

// |x| as a bit pattern: for non-negative doubles the order of the patterns is
// the numeric order (NaN patterns are above infinity), so the maxima and the
// finiteness test run on the integer pipe and leave the FP64 pipe to the sums
__device__ inline unsigned long long absBits(double x) {
  return (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
}
__device__ inline unsigned long long umax64(unsigned long long a, unsigned long long b) { return a > b ? a : b; }

__global__ void __launch_bounds__(CHUNK_TPB) kNormsPartial(DevData d) {
  pdlEntry();
  __shared__ double sh[CHUNK_TPB / 32][NPART];
  const int c = blockIdx.x;
  const int m = d.chunkModel[c];
  if (!(d.m.flags[m] & FL_ACTIVE)) return;
  const double* wD = d.m.wDisp + 3 * m;
  const double* wF = d.m.wForce + 3 * m;
  const unsigned long long badBits = absBits(1.0e300);
  // sums: 2-4 disp/vel/acc, 5 residual, 6 energy; maxima as bit patterns:
  // mx[0] energy, mx[1 + 3 q + t] vector q of DOF type t; (the weight sums
  // 0 and 1 are per-model constants)
  double v2 = 0.0, v3 = 0.0, v4 = 0.0, v5 = 0.0, v6 = 0.0;
  unsigned long long mx[13];
#pragma unroll
  for (int k = 0; k < 13; ++k) mx[k] = 0ull;
  bool bad = false;
  const int cEnd = d.chunkEnd[c];
  for (int i0 = d.chunkStart[c] + threadIdx.x; i0 < cEnd; i0 += 4 * CHUNK_TPB) {
    // four DOFs per pass: all loads issued before the ordered accumulation
    int eqs[4], ts[4];
    double a0[4], a1[4], a2[4], rr[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int i = i0 + u * CHUNK_TPB;
      eqs[u] = i < cEnd ? d.meqn[i] : -1;
      ts[u] = i < cEnd ? d.dofType[i] - 1 : 0;
      a0[u] = i < cEnd ? d.sinc0[i] : 0.0;
      a1[u] = i < cEnd ? d.sinc1[i] : 0.0;
      a2[u] = i < cEnd ? d.sinc2[i] : 0.0;
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) rr[u] = eqs[u] >= 0 ? d.res[eqs[u]] : 0.0;
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      if (eqs[u] < 0) continue;
      const int t = ts[u];
      const double wd = wD[t], wf = wF[t];
      const double s0 = a0[u], s1 = a1[u], s2 = a2[u], r = rr[u];
      const unsigned long long b0 = absBits(s0), b1 = absBits(s1), b2 = absBits(s2), br = absBits(r);
      bad |= b0 > badBits || br > badBits;
      v2 += (wd * s0) * (wd * s0);
      v3 += (wd * s1) * (wd * s1);
      v4 += (wd * s2) * (wd * s2);
      v5 += (wf * r) * (wf * r);
      const double en = fabs(s0 * r);
      v6 += en;
      mx[0] = umax64(mx[0], absBits(en));
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        if (q != t) continue;
        mx[1 + q] = umax64(mx[1 + q], b0);
        mx[4 + q] = umax64(mx[4 + q], b1);
        mx[7 + q] = umax64(mx[7 + q], b2);
        mx[10 + q] = umax64(mx[10 + q], br);
      }
    }
  }
  // warp tree (fixed pattern), then warps in order
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    v2 += __shfl_down_sync(0xffffffffu, v2, o);
    v3 += __shfl_down_sync(0xffffffffu, v3, o);
    v4 += __shfl_down_sync(0xffffffffu, v4, o);
    v5 += __shfl_down_sync(0xffffffffu, v5, o);
    v6 += __shfl_down_sync(0xffffffffu, v6, o);
#pragma unroll
    for (int k = 0; k < 13; ++k) mx[k] = umax64(mx[k], __shfl_down_sync(0xffffffffu, mx[k], o));
  }
  bad = __any_sync(0xffffffffu, bad);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) {
    sh[w][0] = 0.0;
    sh[w][1] = 0.0;
    sh[w][2] = v2;
    sh[w][3] = v3;
    sh[w][4] = v4;
    sh[w][5] = v5;
    sh[w][6] = v6;
#pragma unroll
    for (int k = 0; k < 13; ++k) sh[w][7 + k] = __longlong_as_double((long long)mx[k]);
    sh[w][20] = bad ? 1.0 : 0.0;
  }
  __syncthreads();
  if (threadIdx.x < NPART) {
    const int k = threadIdx.x;
    double x = sh[0][k];
    for (int ww = 1; ww < CHUNK_TPB / 32; ++ww)
      x = (k <= 6) ? x + sh[ww][k] : __longlong_as_double((long long)umax64(absBits(x), absBits(sh[ww][k])));
    d.partial[(size_t)c * NPART + k] = x;
  }
}

// norms, convergence test (normTypeModule.f90:196-249) and iteration counters
// one warp per model: lane k combines partial value k over the model's chunks
// in chunk order, lane 0 evaluates the norms and the test
__global__ void kControl(DevData d) {
  pdlEntry();
  const int m = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (m >= d.m.n) return;
  const int fl = d.m.flags[m];
  if (!(fl & FL_ACTIVE)) return;
  const int c0 = d.modelChunkOff[m], nc = d.modelNchunk[m];
  double acc = 0.0;
  if (lane < NPART) {
    acc = nc > 0 ? d.partial[(size_t)c0 * NPART + lane] : 0.0;
    for (int c = 1; c < nc; ++c) {
      double x = d.partial[(size_t)(c0 + c) * NPART + lane];
      // maxima (and the NaN flag) as |x| bit patterns: a NaN stays in the norm
      acc = (lane <= 6) ? acc + x : __longlong_as_double((long long)umax64(absBits(acc), absBits(x)));
    }
  }
  double v[NPART];
#pragma unroll
  for (int k = 0; k < NPART; ++k) v[k] = __shfl_sync(0xffffffffu, acc, k);
  if (lane != 0) return;
  double* nv = d.m.normVal + 18 * m;
  v[0] = d.m.sumWd2[m];
  v[1] = d.m.sumWf2[m];
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
  } else if (fl & FL_LINEAR) {
    conv = it == d.linearIters;  // pure linear quasi-static step: one solve (+ refinement)
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
// threads [0, ntriTot) a triad each, threads [ntriTot, ntriTot + nelTot) an element each
__global__ void kStepEnd(DevData d) {
  pdlEntry();
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < d.ntriTot) {
    if ((d.m.flags[d.triModel[t]] & FL_STEPDONE) && d.triNdof[t] == 6) orthonormRot(d.ur + 12 * (size_t)t);
    return;
  }
  const long long i = t - d.ntriTot;
  if (i < d.nelTot) {
    const int fl = d.m.flags[d.elModel[i]];
    if ((fl & FL_STEPDONE) && !(fl & FL_LINEAR))
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
// backward queues of the active models, for solves outside a step start
__global__ void kSeedBackward(DevModels m, BackwardSeed bs) {
  pdlEntry();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m.n && (m.flags[i] & FL_ACTIVE)) seedBackward(bs, i);
}

__global__ void kStaticBegin(DevModels m, int* activeCount, BackwardSeed bs) {
  pdlEntry();
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
  seedBackward(bs, i);
}

__global__ void kStaticResidual(DevData d) {
  pdlEntry();
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.neqTot) return;
  int m = d.eqModel[i];
  if (!(d.m.flags[m] & FL_STATIC)) return;
  double fs = 0.0, q = 0.0;
  const size_t blk = (size_t)12 * d.nelTot;
  const size_t xlim = blk + (size_t)6 * d.naxTot;
  for (int k = d.eqPtr[i]; k < d.eqPtr[i + 1]; ++k) {
    size_t s = d.eqSrc[k];
    if (s < blk) {
      fs += d.Fel[s];
      q += d.Fel[s + 3 * blk];
    } else if (s >= xlim) {
      fs += d.FelX[s - xlim];
      q += d.FelX[s - xlim + 3];
    } else {
      fs += d.FelA[s - blk];
    }
  }
  q += d.qext[i];
  d.FSk[i] = fs;
  d.Qk[i] = q;
  d.res[i] = q - fs;
  d.del[i] = q - fs;
}

__global__ void __launch_bounds__(NTPB) kStaticNorm(DevData d) {
  pdlEntry();
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
  pdlEntry();
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < d.ndofTot) {
    int m = d.dofModel[i];
    if (d.m.flags[m] & FL_STATIC) {
      int eq = d.meqn[i];
      double s0 = eq >= 0 ? d.del[eq] * d.m.staticScale[m] : 0.0;
      if (eq == -1 && d.dofDep && d.dofDep[i] >= 0) s0 = dependentValue(d, d.dofDep[i], d.del, d.m.staticScale[m]);
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
        if (eq == -1 && d.dofDep && d.dofDep[d0 + k] >= 0) inc[k] = dependentValue(d, d.dofDep[d0 + k], d.del, f);
      }
      double* U = d.ur + 12 * (size_t)i;
      for (int r = 0; r < 3; ++r) U[9 + r] += inc[r];
      if (nd == 6) {
        double R[9], O[9];
        rotvecToMat(inc + 3, d.sinEpsOverEps, R);
        for (int c = 0; c < 3; ++c)
          for (int r = 0; r < 3; ++r) O[r + 3 * c] = R[r] * U[3 * c] + R[r + 3] * U[3 * c + 1] + R[r + 6] * U[3 * c + 2];
        for (int k = 0; k < 9; ++k) U[k] = O[k];
      }
    }
  }
}

// convergence logic of the static iterations (staticEquilibriumModule.f90:262-371)
__global__ void kStaticFinish(DevModels m) {
  pdlEntry();
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

void launchBeginStep(const DevData& d, int* activeCount, long long* activeEl, const BackwardSeed& seed,
                     cudaStream_t s) {
  pdlLaunch(kBeginStep, blocksFor(d.m.n, 128), 128, 0, s, d.m, activeCount, activeEl, seed);
}
void launchPredictDofs(const DevData& d, cudaStream_t s) {
  long long n = d.ndofTot > d.neqTot ? d.ndofTot : d.neqTot;
  pdlLaunch(kPredictDofs, blocksFor(n), TPB, 0, s, d);
}
void launchElements(const DevData& d, int mode, cudaStream_t s) {
  launchJoints(d, mode, s);  // dependent triads first, as UpdateMechanism updates the joints first
  if (d.nelTot > 0) pdlLaunch(kElements, blocksFor(d.nelTot, 128), 128, 0, s, d, mode);
  launchParts(d, mode, s);
  if (d.naxTot > 0) pdlLaunch(kAxial, blocksFor(d.naxTot, 128), 128, 0, s, d, mode);
  launchExpandForces(d, mode, s);
}
void launchResidual(const DevData& d, cudaStream_t s) {
  if (d.neqTot > 0) pdlLaunch(kResidual, blocksFor(d.neqTot), TPB, 0, s, d);
}
void launchBuildElementNewton(const DevData& d, cudaStream_t s) {
  // compressed beam batches build N inside kNewtonBeam
  if (d.nelTot > 0 && !d.beamSparse) pdlLaunch(kBuildElementNewton, blocksFor(d.nelTot), TPB, 0, s, d);
}
void launchRotateElementNewton(const DevData& d, cudaStream_t s) {
  if (d.nelTot > 0 && d.beamSparse) pdlLaunch(kNewtonBeam, blocksFor(d.nelTot, 128), 128, 0, s, d);
  else if (d.nelTot > 0) pdlLaunch(kRotateElementNewton, blocksFor(d.nelTot, 128), 128, 0, s, d);
  if (d.naxTot > 0) pdlLaunch(kAxialNewton, blocksFor(d.naxTot, 128), 128, 0, s, d);
  launchExpandElements(d, s);
  launchPartsNewton(d, s);
}
void launchCsrGather(const DevData& d, cudaStream_t s) {
  if (d.nslotTot <= 0) return;
  // resident blocks of the device this launch runs on (queried once per device)
  static int perSm[64] = {0}, sms[64] = {0};
  static std::mutex mu;
  int dev = 0;
  cudaGetDevice(&dev);
  int bps = 0, nsm = 0;
  {
    std::lock_guard<std::mutex> lk(mu);
    if (dev < 64 && perSm[dev] == 0) {
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm[dev], kCsrGather, kSlotBlock / kGatherSlotsPerThread, 0);
      cudaDeviceGetAttribute(&sms[dev], cudaDevAttrMultiProcessorCount, dev);
    }
    if (dev < 64) { bps = perSm[dev]; nsm = sms[dev]; }
  }
  const int nb = blocksFor(d.nslotTot, kSlotBlock);
  const int grid = bps > 0 && nsm > 0 ? std::min(nb, bps * nsm) : nb;
  pdlLaunch(kCsrGather, grid, kSlotBlock / kGatherSlotsPerThread, 0, s, d, nb);
}
void launchIncrement(const DevData& d, cudaStream_t s) {
  pdlLaunch(kIncrement, blocksFor(d.ntriTot + d.ndofTot), TPB, 0, s, d);
}
void launchNormsControl(const DevData& d, cudaStream_t s) {
  launchNormsPartial(d, s);
  launchControlStepEnd(d, s);
}
void launchNormsPartial(const DevData& d, cudaStream_t s) {
  if (d.nchunkTot > 0) pdlLaunch(kNormsPartial, d.nchunkTot, CHUNK_TPB, 0, s, d);
}
void launchControlStepEnd(const DevData& d, cudaStream_t s) {
  pdlLaunch(kControl, blocksFor(32LL * d.m.n, 128), 128, 0, s, d);
  pdlLaunch(kStepEnd, blocksFor(d.ntriTot + d.nelTot), TPB, 0, s, d);
  launchPartsStepEnd(d, s);
}
void launchLoads(const DevData& d, cudaStream_t s) {
  if (d.nldTot > 0) pdlLaunch(kLoads, blocksFor(d.nldTot, 128), 128, 0, s, d);
}
void launchMotions(const DevData& d, cudaStream_t s) {
  if (d.nmotTot > 0) pdlLaunch(kMotions, blocksFor(d.nmotTot, 128), 128, 0, s, d);
}
void launchMotionRhs(const DevData& d, cudaStream_t s) {
  if (d.nmrTot > 0) pdlLaunch(kMotionRhs, blocksFor(d.nmrTot, 128), 128, 0, s, d);
}
void launchQsRestore(const DevData& d, cudaStream_t s) {
  if (!d.urQs) return;
  long long n = std::max<long long>(std::max<long long>(d.ntriTot, d.nelTot), d.ndofTot);
  pdlLaunch(kQsRestore, blocksFor(n), TPB, 0, s, d);
}
void launchSeedBackward(const DevData& d, const BackwardSeed& seed, cudaStream_t s) {
  pdlLaunch(kSeedBackward, blocksFor(d.m.n, 128), 128, 0, s, d.m, seed);
}
void launchStaticBegin(const DevData& d, int* activeCount, const BackwardSeed& seed, cudaStream_t s) {
  pdlLaunch(kStaticBegin, blocksFor(d.m.n, 128), 128, 0, s, d.m, activeCount, seed);
}
void launchStaticResidual(const DevData& d, cudaStream_t s) {
  if (d.neqTot > 0) pdlLaunch(kStaticResidual, blocksFor(d.neqTot), TPB, 0, s, d);
}
void launchStaticNorm(const DevData& d, cudaStream_t s) { pdlLaunch(kStaticNorm, d.m.n, NTPB, 0, s, d); }
void launchStaticIncrement(const DevData& d, cudaStream_t s) {
  long long n = d.ndofTot > d.ntriTot ? d.ndofTot : d.ntriTot;
  pdlLaunch(kStaticIncrement, blocksFor(n), TPB, 0, s, d);
}
void launchStaticFinish(const DevData& d, cudaStream_t s) {
  pdlLaunch(kStaticFinish, blocksFor(d.m.n, 128), 128, 0, s, d.m);
}

}  // namespace fgpu
