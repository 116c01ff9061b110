// part_kernels.cu -- reduced parts (superelements with component modes) on the
// GPU: the element pass and the Newton matrix of parts with any number of
// triads and generalized DOFs, one thread block per part.
//
// Reference behaviour (paths relative to fedem-solvers):
//   corotated frame      src/vpmCommon/supElTypeModule.f90:912-954 (updateSupElCorot, shadowPosAlg 1)
//   deformation vector   :1067-1114 (BuildFinit; the generalized DOFs copy genDOFs%ur)
//   local velocities     src/vpmSolver/supElRoutinesModule.f90:47-85 (SetSupElsVelAcc)
//   generalized DOFs     :168-200 (IncSupElsGenDofs)
//   forces               :231-456 (UpdateSupEls: Fi = M uldd, Fd = stifScl C uld with the
//                        rigid-body filtering of the stiffness-proportional part on the
//                        triad DOFs, Fs = stifScl K finit, Q = stifScl fg (g R))
//   Newton matrix        :1127-1187, 1254-1320 (BuildSupNewtonMat, AddInSupMat/MATTRA on the
//                        triad DOF groups only)
//   constraint expansion src/vpmCommon/vpmLinAlg/sysMatrixTypeModule.f90:2099-2259 (a dependent
//                        triad's DOFs through its joint's coefficients)
//
// A part's forces and Newton matrix are written straight in expanded form (B^T F
// and B^T N B, B the identity on free triads and generalized DOFs and the
// joint coefficients T on a dependent triad) into the expanded region the
// deterministic gather maps read, so the residual and slot gathers take them
// like any other source.  FP64 throughout, fixed summation order.

#include "kernels.h"
#include "rotation.cuh"

namespace fgpu {
namespace {

constexpr int kPartThreads = 128;

__device__ inline bool partModeActive(int mode, int fl) {
  if (mode == EM_PRED) return fl & FL_PRED;
  if (mode == EM_INC) return fl & FL_ACTIVE;
  if (mode == EM_STATIC || mode == EM_STATIC_INIT) return fl & FL_STATIC;
  return true;  // EM_FINAL: every model
}

// column q of B for part p: the part DOFs i0..i0+5 with coefficients b (nb = 6),
// or the single part DOF i0 (nb = -1)
__device__ inline void partColumn(const DevData& d, int p, int q, int& i0, double* b, int& nb) {
  const int nt = d.pNtri[p], t0 = d.pTriOff[p];
  int base = 0;
  for (int t = 0; t < nt; ++t) {
    const int j = d.pTriJoint[t0 + t];
    const int nc = j >= 0 ? d.jNcol[j] : 6;
    if (q < base + nc) {
      if (j < 0) {
        nb = -1;
        i0 = 6 * t + (q - base);
      } else {
        nb = 6;
        i0 = 6 * t;
        const double* T = d.jT + 72 * (size_t)j;
#pragma unroll
        for (int r = 0; r < 6; ++r) b[r] = T[12 * r + (q - base)];
      }
      return;
    }
    base += nc;
  }
  nb = -1;
  i0 = 6 * nt + (q - base);  // a generalized DOF
}

// Element pass of the parts (same modes and gating as the beam element pass):
// generalized DOF increments, frame, deformation, local velocities, the four
// force vectors rotated to system axes on the triad groups, expanded into FelX.
__global__ void __launch_bounds__(kPartThreads) kParts(DevData d, int mode) {
  pdlEntry();
  extern __shared__ double sh[];
  const int p = blockIdx.x, tid = threadIdx.x, nth = blockDim.x;
  const int m = d.pModel[p];
  const int fl = d.m.flags[m];
  if (!partModeActive(mode, fl)) return;
  const int n = d.pN[p], nt = d.pNtri[p], ng = d.pNgen[p], nd = 6 * nt, t0 = d.pTriOff[p];
  const int gfd = d.pGenFirstDof[p], go = d.pGenOff[p];
  const int64_t mo = d.pMatOff[p];
  const int vo = d.pVecOff[p];
  double* S = sh;            // 12: the frame
  double* fin = sh + 12;     // n
  double* uld = fin + n;     // n
  double* uldd = uld + n;    // n
  double* F = uldd + n;      // 4 n: FS, FD, FI, Q
  __shared__ int bad;
  const bool qs = (mode == EM_PRED || mode == EM_INC) && (fl & FL_QSTATIC);
  const bool isStatic = mode == EM_STATIC || mode == EM_STATIC_INIT || qs;
  const bool newPositions = (mode == EM_INC || mode == EM_STATIC || mode == EM_FINAL) && !(qs && (fl & FL_LINEAR));
  // generalized DOFs follow the solution increment (IncSupElsGenDofs)
  if (mode == EM_INC || mode == EM_STATIC)
    for (int g = tid; g < ng; g += nth) d.pGen[go + g] += d.sinc0[gfd + g];
  if (tid == 0) bad = 0;
  for (int k = tid; k < 12; k += nth) S[k] = d.pSupTr[12 * (size_t)p + k];
  __syncthreads();
  // local velocities and accelerations with the frame of the last update, as
  // SetSupElsVelAcc runs before the frame is updated: triad DOFs in part axes,
  // generalized DOFs as they are
  const double* vs = mode == EM_PRED ? d.dk : d.urd;
  const double* as = mode == EM_PRED ? d.ak : d.urdd;
  for (int i = tid; i < n; i += nth) {
    double v = 0.0, a = 0.0;
    if (!isStatic) {
      if (i < nd) {
        const int t = i / 6, g = (i % 6) / 3, r = i % 3;
        const int d0 = d.triFirstDof[d.pTri[t0 + t]] + 3 * g;
        a = S[3 * r] * as[d0] + S[3 * r + 1] * as[d0 + 1] + S[3 * r + 2] * as[d0 + 2];
        v = S[3 * r] * vs[d0] + S[3 * r + 1] * vs[d0 + 1] + S[3 * r + 2] * vs[d0 + 2];
      } else {
        a = as[gfd + (i - nd)];
        v = vs[gfd + (i - nd)];
      }
    }
    uld[i] = v;
    uldd[i] = a;
  }
  __syncthreads();
  if (tid == 0 && newPositions) {
    // corotated frame through the three reference points (shadowPosAlg = 1)
    double pt[3][3];
    for (int j = 0; j < 3; ++j) {
      const double* U = d.ur + 12 * (size_t)d.pTri[t0 + d.pRef[3 * p + j]];
      const double* o = d.pOffset + 9 * (size_t)p + 3 * j;
      for (int q = 0; q < 3; ++q) pt[j][q] = U[q] * o[0] + U[q + 3] * o[1] + U[q + 6] * o[2] + U[q + 9];
    }
    double ex[3], v2[3], ez[3], ey[3];
    for (int k = 0; k < 3; ++k) { ex[k] = pt[1][k] - pt[0][k]; v2[k] = pt[2][k] - pt[0][k]; }
    crossd(ex, v2, ez);
    const double lx = ex[0] * ex[0] + ex[1] * ex[1] + ex[2] * ex[2];
    const double lz = ez[0] * ez[0] + ez[1] * ez[1] + ez[2] * ez[2];
    if (!(lx > 1.0e-16) || !(lz > 1.0e-16)) {
      atomicOr(&d.m.status[m], SS_COROT);
      bad = 1;
    } else {
      const double ilx = rsqrt(lx), ilz = rsqrt(lz);
      for (int k = 0; k < 3; ++k) { ex[k] *= ilx; ez[k] *= ilz; }
      crossd(ez, ex, ey);
      double T[12] = {ex[0], ex[1], ex[2], ey[0], ey[1], ey[2], ez[0], ez[1], ez[2], pt[0][0], pt[0][1], pt[0][2]};
      double Rel[12], Snew[12];
      for (int k = 0; k < 12; ++k) Rel[k] = d.pTriRelSup[12 * (size_t)p + k];
      compose34(T, Rel, Snew);
      for (int k = 0; k < 12; ++k) {
        S[k] = Snew[k];
        d.pSupTr[12 * (size_t)p + k] = Snew[k];
      }
    }
  }
  __syncthreads();
  if (bad) return;
  // deformation vector in the corotated axes
  if (newPositions || mode == EM_STATIC_INIT || qs) {
    double inv[12];
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) inv[r + 3 * c] = S[c + 3 * r];
    for (int r = 0; r < 3; ++r) inv[9 + r] = -(inv[r] * S[9] + inv[r + 3] * S[10] + inv[r + 6] * S[11]);
    for (int t = tid; t < nt; t += nth) {
      const double* U = d.ur + 12 * (size_t)d.pTri[t0 + t];
      double Uc[12], loc[12], Tu[12];
      for (int k = 0; k < 12; ++k) { Uc[k] = U[k]; Tu[k] = d.pTrUnd[12 * (size_t)(t0 + t) + k]; }
      compose34(inv, Uc, loc);
      for (int r = 0; r < 3; ++r) fin[6 * t + r] = loc[9 + r] - Tu[9 + r];
      auto dR = [&](int r, int c) { return loc[r] * Tu[3 * c] + loc[r + 3] * Tu[3 * c + 1] + loc[r + 6] * Tu[3 * c + 2]; };
      fin[6 * t + 3] = dR(2, 1);
      fin[6 * t + 4] = dR(0, 2);
      fin[6 * t + 5] = dR(1, 0);
    }
    for (int g = tid; g < ng; g += nth) fin[nd + g] = d.pGen[go + g];
    __syncthreads();
    for (int i = tid; i < n; i += nth) d.pFinit[vo + i] = fin[i];
  } else {
    for (int i = tid; i < n; i += nth) fin[i] = d.pFinit[vo + i];
  }
  __syncthreads();
  // force vectors, one row per thread
  const double ss = d.pStifScl[p], dt = d.m.dt[m];
  const double* K = d.pK + mo;
  const double* M = d.pM + mo;
  const double* C = d.pC + mo;
  const bool hasC = d.pHasC[p];
  // the stiffness-proportional damping is filtered of rigid-body motion on the
  // triad DOFs in every dynamic pass (the deformation rate is zero in the
  // predictor, whose deformation is the previous step's)
  const bool vldActive = (mode == EM_INC || mode == EM_PRED) && !isStatic && d.pHasVld[p] && dt > 0.0;
  const double* gv = d.m.gravity + 3 * m;
  const double gl0 = gv[0] * S[0] + gv[1] * S[1] + gv[2] * S[2];
  const double gl1 = gv[0] * S[3] + gv[1] * S[4] + gv[2] * S[5];
  const double gl2 = gv[0] * S[6] + gv[1] * S[7] + gv[2] * S[8];
  const double* fg = d.pFg + 3 * (size_t)vo;
  const double* fprev = d.pFinitPrev + vo;
  for (int i = tid; i < n; i += nth) {
    double fs = 0.0, fi = 0.0, fd = 0.0;
    for (int j = 0; j < n; ++j) fs += K[i + (size_t)n * j] * fin[j];
    fs *= ss;
    if (!isStatic) {
      for (int j = 0; j < n; ++j) fi += M[i + (size_t)n * j] * uldd[j];
      if (hasC) {
        for (int j = 0; j < n; ++j) fd += C[i + (size_t)n * j] * uld[j];
        fd *= ss;
      }
      if (vldActive && i < nd) {
        double y = 0.0;
        for (int j = 0; j < nd; ++j) y += K[i + (size_t)n * j] * (uld[j] - (fin[j] - fprev[j]) / dt);
        fd -= d.pKDmp[p] * (ss * y);
      }
    }
    F[i] = fs;
    F[n + i] = fd;
    F[2 * n + i] = fi;
    F[3 * n + i] = ss * (fg[i] * gl0 + fg[i + n] * gl1 + fg[i + 2 * n] * gl2);
  }
  __syncthreads();
  // triad groups to system axes
  for (int w = tid; w < 4 * 2 * nt; w += nth) {
    const int v = w / (2 * nt), g = w % (2 * nt);
    double* f = F + (size_t)v * n + 3 * g;
    const double x0 = f[0], x1 = f[1], x2 = f[2];
    for (int r = 0; r < 3; ++r) f[r] = S[r] * x0 + S[r + 3] * x1 + S[r + 6] * x2;
  }
  __syncthreads();
  // expanded forces B^T F
  const int nx = d.pNx[p];
  double* out = d.FelX + d.pXVecOff[p];
  for (int q = tid; q < nx; q += nth) {
    int i0, nb;
    double b[6];
    partColumn(d, p, q, i0, b, nb);
    for (int v = 0; v < 4; ++v) {
      const double* f = F + (size_t)v * n;
      double s = 0.0;
      if (nb < 0) s = f[i0];
      else
        for (int r = 0; r < 6; ++r) s += b[r] * f[i0 + r];
      out[4 * q + v] = s;
    }
  }
}

// Newton matrices of the parts of models that update their tangent:
// N = sM M + sC stifScl C + sK stifScl K, rotated to system axes on the triad
// DOF groups, expanded B^T N B into elMatX (column-major nx x nx).
__global__ void __launch_bounds__(kPartThreads) kPartsNewton(DevData d) {
  pdlEntry();
  extern __shared__ double sh[];
  const int p = blockIdx.x, tid = threadIdx.x, nth = blockDim.x;
  const int m = d.pModel[p];
  if (!(d.m.flags[m] & FL_TANGENT)) return;
  const int n = d.pN[p], nd = 6 * d.pNtri[p], nx = d.pNx[p];
  const int64_t mo = d.pMatOff[p];
  const double* sn = d.m.scaleN + 3 * m;
  const double ss = d.pStifScl[p];
  const double sM = sn[0], sK = sn[1] * ss, sC = sn[2] * ss;
  const bool hasC = d.pHasC[p];
  double* A = sh;                                    // n x n: local N, then W = Nrot B (n x nx)
  double* Nr = sh + (size_t)n * (n > nx ? n : nx);   // n x n: rotated N
  double S[9];
  for (int k = 0; k < 9; ++k) S[k] = d.pSupTr[12 * (size_t)p + k];
  for (int k = tid; k < n * n; k += nth) {
    double v = sM * d.pM[mo + k];
    if (hasC) v += sC * d.pC[mo + k];
    v += sK * d.pK[mo + k];
    A[k] = v;
  }
  __syncthreads();
  // R N R^T on the triad groups (R = supTr(:,1:3), S[r + 3c] = R(r, c))
  for (int k = tid; k < n * n; k += nth) {
    const int i = k % n, j = k / n;
    double v;
    if (i < nd && j < nd) {
      const int gi = i - i % 3, ri = i % 3, gj = j - j % 3, rj = j % 3;
      v = 0.0;
      for (int a = 0; a < 3; ++a) {
        double w = 0.0;
        for (int b = 0; b < 3; ++b) w += A[(gi + a) + (size_t)n * (gj + b)] * S[rj + 3 * b];
        v += S[ri + 3 * a] * w;
      }
    } else if (i < nd) {
      const int gi = i - i % 3, ri = i % 3;
      v = S[ri] * A[gi + (size_t)n * j] + S[ri + 3] * A[gi + 1 + (size_t)n * j] + S[ri + 6] * A[gi + 2 + (size_t)n * j];
    } else if (j < nd) {
      const int gj = j - j % 3, rj = j % 3;
      v = A[i + (size_t)n * gj] * S[rj] + A[i + (size_t)n * (gj + 1)] * S[rj + 3] + A[i + (size_t)n * (gj + 2)] * S[rj + 6];
    } else {
      v = A[k];
    }
    Nr[k] = v;
  }
  __syncthreads();
  // W(:, q) = Nr B(:, q)
  for (int w = tid; w < n * nx; w += nth) {
    const int i = w % n, q = w / n;
    int i0, nb;
    double b[6];
    partColumn(d, p, q, i0, b, nb);
    double s = 0.0;
    if (nb < 0) s = Nr[i + (size_t)n * i0];
    else
      for (int r = 0; r < 6; ++r) s += Nr[i + (size_t)n * (i0 + r)] * b[r];
    A[w] = s;
  }
  __syncthreads();
  // out(p, q) = B(:, p)^T W(:, q) for p >= q, mirrored: the expanded matrix is
  // exactly symmetric whatever the rounding of the rotation
  double* out = d.elMatX + d.pXMatOff[p];
  for (int w = tid; w < nx * nx; w += nth) {
    const int pp = w % nx, q = w / nx;
    if (pp < q) continue;
    int i0, nb;
    double b[6];
    partColumn(d, p, pp, i0, b, nb);
    double s = 0.0;
    if (nb < 0) s = A[i0 + (size_t)n * q];
    else
      for (int r = 0; r < 6; ++r) s += b[r] * A[i0 + r + (size_t)n * q];
    out[w] = s;
    out[q + (size_t)nx * pp] = s;
  }
}

// terminateStep: the deformation of a finished step becomes the previous one
// (the rigid-body filtering of the next step measures from it)
__global__ void kPartsStepEnd(DevData d) {
  pdlEntry();
  const int p = blockIdx.x;
  const int fl = d.m.flags[d.pModel[p]];
  if (!(fl & FL_STEPDONE) || (fl & FL_LINEAR)) return;
  const int vo = d.pVecOff[p], n = d.pN[p];
  for (int i = threadIdx.x; i < n; i += blockDim.x) d.pFinitPrev[vo + i] = d.pFinit[vo + i];
}

size_t partSmem(const DevData& d) { return sizeof(double) * (12 + 7 * (size_t)d.partMaxN); }

size_t partNewtonSmem(const DevData& d) {
  const size_t n = (size_t)d.partMaxN, nx = (size_t)d.partMaxNx;
  return sizeof(double) * (n * (n > nx ? n : nx) + n * n);
}

}  // namespace

int preparePartKernels(const DevData& d) {
  if (d.npartTot <= 0) return 0;
  if (cudaFuncSetAttribute(kParts, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)partSmem(d)) != cudaSuccess)
    return -1;
  if (cudaFuncSetAttribute(kPartsNewton, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)partNewtonSmem(d)) !=
      cudaSuccess)
    return -1;
  return 0;
}

void launchParts(const DevData& d, int mode, cudaStream_t s) {
  if (d.npartTot > 0) pdlLaunch(kParts, d.npartTot, kPartThreads, partSmem(d), s, d, mode);
}

void launchPartsNewton(const DevData& d, cudaStream_t s) {
  if (d.npartTot > 0) pdlLaunch(kPartsNewton, d.npartTot, kPartThreads, partNewtonSmem(d), s, d);
}

void launchPartsStepEnd(const DevData& d, cudaStream_t s) {
  if (d.npartTot > 0) pdlLaunch(kPartsStepEnd, d.npartTot, 64, 0, s, d);
}

}  // namespace fgpu
