// joint_kernels.cu -- master-slave joints on the GPU: the per-joint update of
// the dependent triad and of the constraint coefficients, and the expansion of
// the element matrices and forces of elements that hold a dependent triad.
//
// Reference behaviour (paths relative to fedem-solvers):
//   joint variables      src/vpmSolver/masterSlaveJointRoutinesModule.f90:40-99 (IncJointsVar)
//   dependent triad      :218-299 (moveJointInPosition, SetLinearDependencies)
//   coefficients TTCC    :374-577 (updateDependencies)
//   constraint assembly  src/vpmCommon/vpmLinAlg/sysMatrixTypeModule.f90:2099-2259 (asmSparse,
//                        MEEN < 0 through MPMCEQ/MMCEQ/TTCC); csAddEV for the forces
//
// A joint has one master triad; the slave triad's six DOFs are dependent:
// u_s = T [u_master; q_joint], T = 6 x (nM + nJ).  An element holding a
// dependent triad contributes B^T N B and B^T F, B the block-diagonal map from
// its expanded DOFs (free triad: identity; dependent triad: T) to its 12 DOFs.
// All arithmetic is FP64 in a fixed order.

#include "kernels.h"
#include "rotation.cuh"

namespace fgpu {
namespace {

constexpr int kMaxLevels = 7;  // position-matrix levels of a joint (1..6 used)

// joint variables of level im (1-based) as a 3x4 position matrix
__device__ void jointLevel(const DevData& d, int j, int im, double* F) {
  double th[3] = {0.0, 0.0, 0.0};
#pragma unroll
  for (int k = 0; k < 12; ++k) F[k] = 0.0;
  const int n0 = d.jDofOff[j], nv = d.jNdof[j];
  for (int k = 0; k < nv; ++k) {
    if (d.jImat[n0 + k] != im) continue;
    const int l = d.jLdof[n0 + k];
    if (l <= 3) F[9 + l - 1] = d.jVar[n0 + k];
    else th[l - 4] = d.jVar[n0 + k];
  }
  rotvecToMat(th, d.sinEpsOverEps, F);
}

__device__ inline bool modeActive(int mode, int fl) {
  if (mode == EM_PRED) return fl & FL_PRED;
  if (mode == EM_INC) return fl & FL_ACTIVE;
  if (mode == EM_STATIC || mode == EM_STATIC_INIT) return fl & FL_STATIC;
  return true;  // EM_FINAL: every model
}

// One thread per joint: increment of the joint variables (after an increment
// pass), the dependent triad on its kinematic position, the coefficients T.
__global__ void kJoints(DevData d, int mode) {
  pdlEntry();
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= d.njointTot) return;
  if (!modeActive(mode, d.m.flags[d.jModel[j]])) return;
  const int n0 = d.jDofOff[j], nv = d.jNdof[j], nmats = d.jNmats[j];
  if (mode == EM_INC || mode == EM_STATIC)
    for (int k = 0; k < nv; ++k) d.jVar[n0 + k] += d.sinc0[d.jFirstDof[j] + k];
  double* US = d.ur + 12 * (size_t)d.jSlave[j];
  const double* UM = d.ur + 12 * (size_t)d.jMaster[j];
  double M[12], JG[12], JT[12];
#pragma unroll
  for (int k = 0; k < 12; ++k) { M[k] = UM[k]; JT[k] = d.jPosInT[12 * j + k]; }
  compose34(M, JT, JG);  // joint frame follows the master triad
  // TR = -spin(e), e the dependent triad's position relative to the master
  // before the dependent triad is moved (SetLinearDependencies)
  const double e0 = US[9] - M[9], e1 = US[10] - M[10], e2 = US[11] - M[11];
  double P[12], Q[12], F[12];
#pragma unroll
  for (int k = 0; k < 12; ++k) P[k] = d.jSTPos0[12 * j + k];
  for (int im = 1; im <= nmats; ++im) {
    jointLevel(d, j, im, F);
    compose34(F, P, Q);
#pragma unroll
    for (int k = 0; k < 12; ++k) P[k] = Q[k];
  }
  compose34(JG, P, Q);
#pragma unroll
  for (int k = 0; k < 12; ++k) US[k] = Q[k];
  // constraint coefficients (updateDependencies): master block, then joint DOFs
  double* T = d.jT + 72 * (size_t)j;
#pragma unroll
  for (int k = 0; k < 72; ++k) T[k] = 0.0;
  const int nM = d.jNM[j];
  // TR columns: TR(:,c) = -spin(e) e_c = e x e_c
  const double TR[9] = {0.0, -e2, e1, e2, 0.0, -e0, -e1, e0, 0.0};  // column-major, TR[r + 3c]
  for (int lm = 0; lm < nM; ++lm)
    for (int ls = 0; ls < 6; ++ls) {
      double v = 0.0;
      if (ls < 3 && lm < 3) v = ls == lm ? 1.0 : 0.0;
      else if (ls < 3) v = TR[ls + 3 * (lm - 3)];
      else if (lm >= 3) v = ls == lm ? 1.0 : 0.0;
      T[12 * ls + lm] = v;
    }
  // accumulated level frames: csys(im) = rotation of the frame the level's DOFs
  // act in, png(im) = position of level im (global)
  double csys[kMaxLevels][9], png[kMaxLevels][3];
  double Pacc[12];
#pragma unroll
  for (int k = 0; k < 12; ++k) Pacc[k] = JG[k];
  for (int im = nmats; im >= 1; --im) {
#pragma unroll
    for (int k = 0; k < 9; ++k) csys[im][k] = Pacc[k];
    jointLevel(d, j, im, F);
    compose34(Pacc, F, Q);
#pragma unroll
    for (int k = 0; k < 12; ++k) Pacc[k] = Q[k];
    png[im][0] = Pacc[9]; png[im][1] = Pacc[10]; png[im][2] = Pacc[11];
  }
  for (int k = 0; k < nv; ++k) {
    const int lm = d.jLdof[n0 + k], im = d.jImat[n0 + k];
    double dUS[6];
    if (lm <= 3) {
#pragma unroll
      for (int r = 0; r < 3; ++r) { dUS[r] = csys[im][r + 3 * (lm - 1)]; dUS[3 + r] = 0.0; }
    } else {
      double dOm[3], ecc[3], dUG[3];
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        dOm[r] = csys[im][r + 3 * (lm - 4)];
        ecc[r] = US[9 + r] - png[im][r];
      }
      crossd(dOm, ecc, dUG);
#pragma unroll
      for (int r = 0; r < 3; ++r) { dUS[r] = dUG[r]; dUS[3 + r] = dOm[r]; }
    }
#pragma unroll
    for (int ls = 0; ls < 6; ++ls) T[12 * ls + nM + k] = dUS[ls];
  }
}

// the column of B (12 x nx) at expanded DOF q of constrained element c:
// rows i0..i0+5 with coefficients b[0..5] (a free triad's DOF has one entry)
__device__ inline void bColumn(const DevData& d, int c, int q, int& i0, double* b, int& nb) {
  const int ja = d.cxNode[2 * c], jb = d.cxNode[2 * c + 1];
  const int na = ja >= 0 ? d.jNcol[ja] : 6;
  const int n = q < na ? 0 : 1;
  const int jn = n == 0 ? ja : jb;
  const int col = q - (n == 0 ? 0 : na);
  i0 = 6 * n;
  if (jn < 0) {
    nb = -1;  // identity: row i0 + col only
    b[0] = 1.0;
    i0 += col;
    return;
  }
  nb = 6;
  const double* T = d.jT + 72 * (size_t)jn;
#pragma unroll
  for (int r = 0; r < 6; ++r) b[r] = T[12 * r + col];
}

// Expanded Newton matrices B^T N B of the constrained elements of the models
// that update their tangent: one block per element, thread q builds column q
__global__ void kExpandElements(DevData d) {
  pdlEntry();
  const int c = blockIdx.x, q = threadIdx.x;
  const int e = d.cxEl[c];
  if (!(d.m.flags[d.elModel[e]] & FL_TANGENT)) return;
  const int nx = d.cxNx[c];
  if (q >= nx) return;
  const int nel = d.nelTot;
  int iq;
  double bq[6];
  int nbq;
  bColumn(d, c, q, iq, bq, nbq);
  // W = N B(:, q)
  double W[12];
#pragma unroll
  for (int i = 0; i < 12; ++i) {
    double s = 0.0;
    if (nbq < 0) {
      s = d.elMat[(size_t)(i + 12 * iq) * nel + e];
    } else {
      for (int r = 0; r < 6; ++r) s += d.elMat[(size_t)(i + 12 * (iq + r)) * nel + e] * bq[r];
    }
    W[i] = s;
  }
  double* out = d.elMatX + d.cxMatOff[c] + (size_t)nx * q;
  for (int p = 0; p < nx; ++p) {
    int ip;
    double bp[6];
    int nbp;
    bColumn(d, c, p, ip, bp, nbp);
    double s = 0.0;
    if (nbp < 0) s = W[ip];
    else
      for (int r = 0; r < 6; ++r) s += bp[r] * W[ip + r];
    out[p] = s;
  }
}

// Expanded forces B^T F (FS, FD, FI, Q) of the constrained elements, with the
// same model gating as the element pass of this mode
__global__ void kExpandForces(DevData d, int mode) {
  pdlEntry();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = t >> 5, p = t & 31;
  if (c >= d.ncxTot) return;
  const int e = d.cxEl[c];
  if (!modeActive(mode, d.m.flags[d.elModel[e]])) return;
  const int nx = d.cxNx[c];
  if (p >= nx) return;
  const int nel = d.nelTot;
  int ip;
  double b[6];
  int nb;
  bColumn(d, c, p, ip, b, nb);
  double* out = d.FelX + d.cxVecOff[c] + 4 * p;
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    const double* F = d.Fel + (size_t)(12 * v) * nel;
    double s = 0.0;
    if (nb < 0) s = F[(size_t)ip * nel + e];
    else
      for (int r = 0; r < 6; ++r) s += b[r] * F[(size_t)(ip + r) * nel + e];
    out[v] = s;
  }
}

}  // namespace

void launchJoints(const DevData& d, int mode, cudaStream_t s) {
  if (d.njointTot > 0) pdlLaunch(kJoints, (d.njointTot + 63) / 64, 64, 0, s, d, mode);
}

void launchExpandElements(const DevData& d, cudaStream_t s) {
  if (d.ncxTot > 0) pdlLaunch(kExpandElements, d.ncxTot, 32, 0, s, d);
}

void launchExpandForces(const DevData& d, int mode, cudaStream_t s) {
  if (d.ncxTot > 0) pdlLaunch(kExpandForces, (d.ncxTot * 32 + 127) / 128, 128, 0, s, d, mode);
}

}  // namespace fgpu
