// front_kernels.cu -- multifrontal LDL^T factorisation and triangular solves,
// one warp per front, level by level over the assembly trees of all models.
//
// This replaces the factor and solve of the absent SAM/SPR solver that the
// reference calls from csSolve (src/vpmCommon/vpmLinAlg/solExtensionModule.f90:
// 153-505: SPRFC1/SPRFC3 factor, SPRFS1/SPRBS1 forward/back substitution).
// Semantics kept: LDL^T without pivoting, a pivot counts as singular when
// |d_k| <= tolFactorize * |a_kk| (error -3), negative pivots are counted.
//
// Fronts are dense column-major nrow x nrow tiles in shared memory (lower
// triangle used); a front's first npiv rows are its pivots.  Children's update
// matrices and forward-solve vectors are extend-added by the parent in child
// order, so every sum has a fixed order (bitwise reproducible, no atomics on
// floating-point data).
//
// Mixed precision: the factor and the correction solves run in FP32; the
// refinement residual r = b - A x uses the FP64 Newton matrix and FP64 x.

#include "kernels.h"

namespace fgpu {
namespace {

constexpr int TPB = 256;
inline int blocksFor(long long n, int tpb = TPB) { return (int)((n + tpb - 1) / tpb); }

template <typename T>
__global__ void kFactorLevel(DevData d, const int* __restrict__ fronts, int count, int maxRow, T* Lbase,
                             T* Ubase, double tolFact) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int wpb = blockDim.x >> 5, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int fi = blockIdx.x * wpb + w;
  if (fi >= count) return;
  const int f = fronts[fi];
  const int m = d.fModel[f];
  if (!(d.m.flags[m] & FL_TANGENT)) return;
  const int nr = d.fNrow[f], np = d.fNpiv[f], nu = nr - np;
  T* F = reinterpret_cast<T*>(smraw) + (size_t)w * ((size_t)maxRow * maxRow + 2 * maxRow);
  T* lcol = F + (size_t)maxRow * maxRow;
  T* diag0 = lcol + maxRow;
  for (int k = lane; k < nr * nr; k += 32) F[k] = T(0);
  __syncwarp();
  // original matrix entries of the pivot columns (unique positions)
  const int64_t ao = d.fAsmOff[f];
  const int na = d.fNasm[f];
  for (int k = lane; k < na; k += 32) F[d.asmPos[ao + k]] = (T)d.csrVal[d.asmSlot[ao + k]];
  __syncwarp();
  for (int k = lane; k < np; k += 32) diag0[k] = F[k + nr * k];
  __syncwarp();
  // extend-add the children's update matrices
  const int nc = d.fNchild[f];
  const int64_t co = d.fChildOff[f];
  for (int c = 0; c < nc; ++c) {
    const int ch = d.childList[co + c];
    const int cu = d.fNrow[ch] - d.fNpiv[ch];
    const T* Uc = Ubase + d.fUOff[ch];
    const int* rel = d.relIndex + d.fRelOff[ch];
    for (int k = lane; k < cu * cu; k += 32) {
      int a = k % cu, b = k / cu;
      if (a >= b) F[rel[a] + nr * rel[b]] += Uc[k];
    }
    __syncwarp();
  }
  // partial LDL^T of the pivot columns
  int neg = 0;
  bool sing = false;
  for (int k = 0; k < np; ++k) {
    const T dk = F[k + nr * k];
    const bool bad = !(fabs((double)dk) > tolFact * fabs((double)diag0[k]));
    sing |= bad;
    if (dk < T(0)) ++neg;
    const T inv = bad ? T(0) : T(1) / dk;
    for (int i = k + 1 + lane; i < nr; i += 32) lcol[i] = F[i + nr * k] * inv;
    __syncwarp();
    const int mrem = nr - k - 1;
    for (int t = lane; t < mrem * mrem; t += 32) {
      int ii = t % mrem, jj = t / mrem;
      if (ii >= jj) {
        int i = k + 1 + ii, j = k + 1 + jj;
        F[i + nr * j] -= F[i + nr * k] * lcol[j];
      }
    }
    __syncwarp();
    for (int i = k + 1 + lane; i < nr; i += 32) F[i + nr * k] = lcol[i];
    __syncwarp();
  }
  T* Lout = Lbase + d.fLOff[f];
  for (int k = lane; k < nr * np; k += 32) Lout[k] = F[k];
  T* Uout = Ubase + d.fUOff[f];
  for (int k = lane; k < nu * nu; k += 32) {
    int a = k % nu, b = k / nu;
    Uout[k] = F[(np + a) + nr * (np + b)];
  }
  if (lane == 0) {
    if (neg) atomicAdd(&d.m.negPiv[m], neg);
    if (sing) atomicOr(&d.m.status[m], SS_SINGULAR);
  }
}

template <typename T>
__global__ void kForwardLevel(DevData d, const int* __restrict__ fronts, int count, int maxRow, const T* Lbase,
                              T* X, T* W) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int wpb = blockDim.x >> 5, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int fi = blockIdx.x * wpb + w;
  if (fi >= count) return;
  const int f = fronts[fi];
  const int m = d.fModel[f];
  if (!(d.m.flags[m] & FL_ACTIVE)) return;
  const int nr = d.fNrow[f], np = d.fNpiv[f], nu = nr - np;
  T* v = reinterpret_cast<T*>(smraw) + (size_t)w * maxRow;
  const int* rows = d.frontRows + d.fRowOff[f];
  for (int r = lane; r < nr; r += 32) v[r] = r < np ? X[rows[r]] : T(0);
  __syncwarp();
  const int nc = d.fNchild[f];
  const int64_t co = d.fChildOff[f];
  for (int c = 0; c < nc; ++c) {
    const int ch = d.childList[co + c];
    const int cu = d.fNrow[ch] - d.fNpiv[ch];
    const T* wc = W + d.fWOff[ch];
    const int* rel = d.relIndex + d.fRelOff[ch];
    for (int a = lane; a < cu; a += 32) v[rel[a]] += wc[a];
    __syncwarp();
  }
  const T* L = Lbase + d.fLOff[f];
  for (int k = 0; k < np; ++k) {
    const T yk = v[k];
    __syncwarp();
    for (int i = k + 1 + lane; i < nr; i += 32) v[i] -= L[i + (size_t)nr * k] * yk;
    __syncwarp();
  }
  for (int r = lane; r < np; r += 32) X[rows[r]] = v[r] / L[r + (size_t)nr * r];
  T* wo = W + d.fWOff[f];
  for (int a = lane; a < nu; a += 32) wo[a] = v[np + a];
}

template <typename T>
__global__ void kBackwardLevel(DevData d, const int* __restrict__ fronts, int count, int maxRow, const T* Lbase,
                               T* X) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int wpb = blockDim.x >> 5, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int fi = blockIdx.x * wpb + w;
  if (fi >= count) return;
  const int f = fronts[fi];
  const int m = d.fModel[f];
  if (!(d.m.flags[m] & FL_ACTIVE)) return;
  const int nr = d.fNrow[f], np = d.fNpiv[f];
  T* xs = reinterpret_cast<T*>(smraw) + (size_t)w * maxRow;
  const int* rows = d.frontRows + d.fRowOff[f];
  for (int r = lane; r < nr; r += 32) xs[r] = X[rows[r]];
  __syncwarp();
  const T* L = Lbase + d.fLOff[f];
  for (int k = np - 1; k >= 0; --k) {
    T s = T(0);
    for (int i = k + 1 + lane; i < nr; i += 32) s += L[i + (size_t)nr * k] * xs[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) xs[k] -= s;
    __syncwarp();
  }
  for (int r = lane; r < np; r += 32) X[rows[r]] = xs[r];
}

__global__ void kSolveSetup(DevData d, int fp32, int sweep) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.neqTot) return;
  if (!(d.m.flags[d.eqModel[i]] & FL_ACTIVE)) return;
  if (!fp32) {
    d.x64[i] = d.del[i];
  } else if (sweep == 0) {
    d.x32[i] = (float)d.del[i];
    d.xref[i] = 0.0;
  } else {
    d.x32[i] = (float)d.rref[i];
  }
}

__global__ void kSolveAccumulate(DevData d, int fp32) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.neqTot) return;
  if (!(d.m.flags[d.eqModel[i]] & FL_ACTIVE)) return;
  if (fp32) d.xref[i] += (double)d.x32[i];
  else d.del[i] = d.x64[i];
}

__global__ void kSolveFinalize(DevData d) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.neqTot) return;
  if (!(d.m.flags[d.eqModel[i]] & FL_ACTIVE)) return;
  d.del[i] = d.xref[i];
}

// refinement residual r = b - A x with the FP64 Newton matrix (full symmetric CSR)
__global__ void kRefineResidual(DevData d) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.neqTot) return;
  if (!(d.m.flags[d.eqModel[i]] & FL_ACTIVE)) return;
  double s = 0.0;
  for (int64_t k = d.rowPtr[i]; k < d.rowPtr[i + 1]; ++k) s += d.csrVal[k] * d.xref[d.colInd[k]];
  d.rref[i] = d.del[i] - s;
}

template <typename T>
int warpsPerBlock(int maxRow, size_t perWarpElems) {
  size_t bytes = perWarpElems * sizeof(T);
  int w = (int)(96 * 1024 / (bytes > 0 ? bytes : 1));
  if (w > 8) w = 8;
  if (w < 1) w = 1;
  return w;
}

template <typename K>
void allowSmem(K kernel, size_t bytes) {
  if (bytes > 48 * 1024) cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

}  // namespace

void launchFactorLevel(const DevData& d, const LevelPlan& lv, bool fp32, cudaStream_t s) {
  if (lv.count <= 0) return;
  const double tol = 1.0e-12;
  size_t perWarp = (size_t)lv.maxRow * lv.maxRow + 2 * lv.maxRow;
  if (fp32) {
    int wpb = warpsPerBlock<float>(lv.maxRow, perWarp);
    size_t sm = (size_t)wpb * perWarp * sizeof(float);
    allowSmem(kFactorLevel<float>, sm);
    kFactorLevel<float><<<(lv.count + wpb - 1) / wpb, 32 * wpb, sm, s>>>(d, lv.fronts, lv.count, lv.maxRow, d.L32,
                                                                        d.U32, tol);
  } else {
    int wpb = warpsPerBlock<double>(lv.maxRow, perWarp);
    size_t sm = (size_t)wpb * perWarp * sizeof(double);
    allowSmem(kFactorLevel<double>, sm);
    kFactorLevel<double><<<(lv.count + wpb - 1) / wpb, 32 * wpb, sm, s>>>(d, lv.fronts, lv.count, lv.maxRow,
                                                                          d.L64, d.U64, tol);
  }
}

void launchForwardLevel(const DevData& d, const LevelPlan& lv, bool fp32, cudaStream_t s) {
  if (lv.count <= 0) return;
  const int wpb = 8;
  if (fp32) {
    size_t sm = (size_t)wpb * lv.maxRow * sizeof(float);
    kForwardLevel<float><<<(lv.count + wpb - 1) / wpb, 32 * wpb, sm, s>>>(d, lv.fronts, lv.count, lv.maxRow, d.L32,
                                                                         d.x32, d.w32);
  } else {
    size_t sm = (size_t)wpb * lv.maxRow * sizeof(double);
    kForwardLevel<double><<<(lv.count + wpb - 1) / wpb, 32 * wpb, sm, s>>>(d, lv.fronts, lv.count, lv.maxRow,
                                                                           d.L64, d.x64, d.w64);
  }
}

void launchBackwardLevel(const DevData& d, const LevelPlan& lv, bool fp32, cudaStream_t s) {
  if (lv.count <= 0) return;
  const int wpb = 8;
  if (fp32) {
    size_t sm = (size_t)wpb * lv.maxRow * sizeof(float);
    kBackwardLevel<float><<<(lv.count + wpb - 1) / wpb, 32 * wpb, sm, s>>>(d, lv.fronts, lv.count, lv.maxRow,
                                                                          d.L32, d.x32);
  } else {
    size_t sm = (size_t)wpb * lv.maxRow * sizeof(double);
    kBackwardLevel<double><<<(lv.count + wpb - 1) / wpb, 32 * wpb, sm, s>>>(d, lv.fronts, lv.count, lv.maxRow,
                                                                            d.L64, d.x64);
  }
}

void launchSolveSetup(const DevData& d, bool fp32, int sweep, cudaStream_t s) {
  if (d.neqTot > 0) kSolveSetup<<<blocksFor(d.neqTot), TPB, 0, s>>>(d, fp32 ? 1 : 0, sweep);
}
void launchSolveAccumulate(const DevData& d, bool fp32, cudaStream_t s) {
  if (d.neqTot > 0) kSolveAccumulate<<<blocksFor(d.neqTot), TPB, 0, s>>>(d, fp32 ? 1 : 0);
}
void launchSolveFinalize(const DevData& d, cudaStream_t s) {
  if (d.neqTot > 0) kSolveFinalize<<<blocksFor(d.neqTot), TPB, 0, s>>>(d);
}
void launchRefineResidual(const DevData& d, cudaStream_t s) {
  if (d.neqTot > 0) kRefineResidual<<<blocksFor(d.neqTot), TPB, 0, s>>>(d);
}

}  // namespace fgpu
