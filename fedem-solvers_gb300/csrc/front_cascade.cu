// front_cascade.cu -- one-launch multifrontal factorisation and solves over
// the assembly trees of all models, without co-residency assumptions.
//
// Factor and forward solve run bottom-up as a cascade: warps start at the
// leaves; a front's counter is incremented (release) when one of its children
// is done, and the warp whose increment completes the count goes on with the
// parent itself.  Nothing ever waits, so the launch is correct whatever the
// residency (several engines may run concurrently on their own streams).
// The backward solve runs top-down: blocks grab consecutive ranges of the
// fronts sorted by decreasing height from a global counter, so every awaited
// parent was grabbed earlier by a running block; each wait is bounded and
// sets errFlag when it runs out.
//
// Front arithmetic is that of front_kernels.cu (SPRFC1/SPRFS1/SPRBS1
// semantics, src/vpmCommon/vpmLinAlg/solExtensionModule.f90:153-505).

#include "kernels.h"

namespace fgpu {
namespace {

constexpr long long kSpinLimit = 1LL << 22;

// partial LDL^T of front f in shared memory (F: maxRow^2, lcol/diag0: maxRow)
template <typename T>
__device__ void factorOneFront(const DevData& d, int f, T* F, T* lcol, T* diag0, const T* Ubase, T* Lbase,
                               T* Uout0, double tolFact, int lane) {
  const int m = d.fModel[f];
  const int nr = d.fNrow[f], np = d.fNpiv[f], nu = nr - np;
  for (int k = lane; k < nr * nr; k += 32) F[k] = T(0);
  __syncwarp();
  const int64_t ao = d.fAsmOff[f];
  const int na = d.fNasm[f];
  for (int k = lane; k < na; k += 32) F[d.asmPos[ao + k]] = (T)d.csrVal[d.asmSlot[ao + k]];
  __syncwarp();
  for (int k = lane; k < np; k += 32) diag0[k] = F[k + nr * k];
  __syncwarp();
  const int nc = d.fNchild[f];
  const int64_t co = d.fChildOff[f];
  for (int c = 0; c < nc; ++c) {
    const int ch = d.childList[co + c];
    const int cu = d.fNrow[ch] - d.fNpiv[ch];
    const T* Uc = Ubase + d.fUOff[ch];
    const int* rel = d.relIndex + d.fRelOff[ch];
    for (int k = lane; k < cu * cu; k += 32) {
      int a = k % cu, b = k / cu;
      if (a >= b) F[rel[a] + nr * rel[b]] += __ldcg(Uc + k);
    }
    __syncwarp();
  }
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
  T* Uout = Uout0 + d.fUOff[f];
  for (int k = lane; k < nu * nu; k += 32) {
    int a = k % nu, b = k / nu;
    Uout[k] = F[(np + a) + nr * (np + b)];
  }
  if (lane == 0) {
    if (neg) atomicAdd(&d.m.negPiv[m], neg);
    if (sing) atomicOr(&d.m.status[m], SS_SINGULAR);
  }
}

// forward elimination of front f: v = [b_p; 0] + children's updates, y = L11^-1 v_p,
// w = v_u - L21 y; X(pivots) = D^-1 y
template <typename T>
__device__ void forwardOneFront(const DevData& d, int f, T* v, const T* Lbase, T* X, T* W, int lane) {
  const int nr = d.fNrow[f], np = d.fNpiv[f], nu = nr - np;
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
    for (int a = lane; a < cu; a += 32) v[rel[a]] += __ldcg(wc + a);
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

// After a front is done: release its data and count it at the parent; returns
// the parent if this warp completed the parent's count (and must go on), else -1.
__device__ inline int climb(const DevData& d, int f, int* cnt, int lane) {
  __threadfence();
  __syncwarp();
  int next = -1;
  if (lane == 0) {
    const int p = d.fParent[f];
    if (p >= 0) {
      int old = atomicAdd(cnt + p, 1);
      if (old == d.fNchild[p] - 1) next = p;
    }
  }
  next = __shfl_sync(0xffffffffu, next, 0);
  if (next >= 0) __threadfence();
  return next;
}

template <typename T>
__global__ void kFactorCascade(DevData d, const int* __restrict__ leaves, int nLeaves, int maxRow, T* Lbase,
                               T* Ubase, double tolFact, int* cnt) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int wpb = blockDim.x >> 5, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int W = gridDim.x * wpb;
  T* F = reinterpret_cast<T*>(smraw) + (size_t)w * ((size_t)maxRow * maxRow + 2 * maxRow);
  T* lcol = F + (size_t)maxRow * maxRow;
  T* diag0 = lcol + maxRow;
  for (int idx = blockIdx.x * wpb + w; idx < nLeaves; idx += W) {
    int f = leaves[idx];
    if (!(d.m.flags[d.fModel[f]] & FL_TANGENT)) continue;
    while (f >= 0) {
      factorOneFront<T>(d, f, F, lcol, diag0, Ubase, Lbase, Ubase, tolFact, lane);
      f = climb(d, f, cnt, lane);
    }
  }
}

template <typename T>
__global__ void kForwardCascade(DevData d, const int* __restrict__ leaves, int nLeaves, int maxRow, const T* Lbase,
                                T* X, T* W, int* cnt) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int wpb = blockDim.x >> 5, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int Wt = gridDim.x * wpb;
  T* v = reinterpret_cast<T*>(smraw) + (size_t)w * maxRow;
  for (int idx = blockIdx.x * wpb + w; idx < nLeaves; idx += Wt) {
    int f = leaves[idx];
    if (!(d.m.flags[d.fModel[f]] & FL_ACTIVE)) continue;
    while (f >= 0) {
      forwardOneFront<T>(d, f, v, Lbase, X, W, lane);
      f = climb(d, f, cnt, lane);
    }
  }
}

// top-down: blocks grab ranges of the fronts sorted by decreasing height
template <typename T>
__global__ void kBackwardDynamic(DevData d, const int* __restrict__ order, int n, int maxRow, const T* Lbase, T* X,
                                 int* ready, int* work, int perWarp, int* errFlag) {
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ int base;
  const int wpb = blockDim.x >> 5, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  T* xs = reinterpret_cast<T*>(smraw) + (size_t)w * maxRow;
  for (;;) {
    if (threadIdx.x == 0) base = atomicAdd(work, wpb * perWarp);
    __syncthreads();
    const int b = base;
    __syncthreads();
    if (b >= n) break;
    for (int j = 0; j < perWarp; ++j) {
      const int idx = b + w * perWarp + j;
      if (idx >= n) break;
      const int f = order[n - 1 - idx];  // decreasing height: parents first
      if (!(d.m.flags[d.fModel[f]] & FL_ACTIVE)) continue;
      int ok = 1;
      if (lane == 0 && d.fParent[f] >= 0) {
        long long spins = 0;
        while (*(volatile const int*)(ready + f) == 0) {
          __nanosleep(32);
          if (++spins > kSpinLimit) {
            atomicOr(errFlag, 1);
            ok = 0;
            break;
          }
        }
        __threadfence();
      }
      ok = __shfl_sync(0xffffffffu, ok, 0);
      if (!ok) continue;
      const int nr = d.fNrow[f], np = d.fNpiv[f];
      const int* rows = d.frontRows + d.fRowOff[f];
      for (int r = lane; r < nr; r += 32) xs[r] = __ldcg(X + rows[r]);
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
      __threadfence();
      __syncwarp();
      const int nc = d.fNchild[f];
      const int64_t co = d.fChildOff[f];
      for (int c = lane; c < nc; c += 32) atomicExch(ready + d.childList[co + c], 1);
      __syncwarp();
    }
  }
}

int smCountCached() {
  static int n = 0;
  if (n == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 1;
  }
  return n;
}

template <typename K>
int occupancyBlocks(K kernel, int threads, size_t smem, int needed) {
  int perSm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, kernel, threads, smem) != cudaSuccess || perSm < 1)
    perSm = 1;
  int cap = perSm * smCountCached();
  return needed < cap ? (needed > 0 ? needed : 1) : cap;
}

template <typename K>
void allowBigSmem(K kernel, size_t bytes) {
  if (bytes > 48 * 1024) cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

int factorWarpsPerBlock(size_t perWarpBytes) {
  int w = (int)(96 * 1024 / (perWarpBytes > 0 ? perWarpBytes : 1));
  return w > 8 ? 8 : (w < 1 ? 1 : w);
}

}  // namespace

void launchFactorCascade(const DevData& d, const PersistentPlan& p, bool fp32, cudaStream_t s) {
  if (p.nLeaves <= 0) return;
  const double tol = 1.0e-12;
  const size_t perWarp = (size_t)p.maxRow * p.maxRow + 2 * p.maxRow;
  cudaMemsetAsync(p.cntFactor, 0, sizeof(int) * (size_t)d.nfrontTot, s);
  if (fp32) {
    const int wpb = factorWarpsPerBlock(perWarp * sizeof(float));
    const size_t sm = (size_t)wpb * perWarp * sizeof(float);
    allowBigSmem(kFactorCascade<float>, sm);
    const int blocks = occupancyBlocks(kFactorCascade<float>, 32 * wpb, sm, (p.nLeaves + wpb - 1) / wpb);
    kFactorCascade<float><<<blocks, 32 * wpb, sm, s>>>(d, p.leaves, p.nLeaves, p.maxRow, d.L32, d.U32, tol,
                                                      p.cntFactor);
  } else {
    const int wpb = factorWarpsPerBlock(perWarp * sizeof(double));
    const size_t sm = (size_t)wpb * perWarp * sizeof(double);
    allowBigSmem(kFactorCascade<double>, sm);
    const int blocks = occupancyBlocks(kFactorCascade<double>, 32 * wpb, sm, (p.nLeaves + wpb - 1) / wpb);
    kFactorCascade<double><<<blocks, 32 * wpb, sm, s>>>(d, p.leaves, p.nLeaves, p.maxRow, d.L64, d.U64, tol,
                                                        p.cntFactor);
  }
}

void launchForwardCascade(const DevData& d, const PersistentPlan& p, bool fp32, cudaStream_t s) {
  if (p.nLeaves <= 0) return;
  const int wpb = 8;
  cudaMemsetAsync(p.cntForward, 0, sizeof(int) * (size_t)d.nfrontTot, s);
  if (fp32) {
    const size_t sm = (size_t)wpb * p.maxRow * sizeof(float);
    const int blocks = occupancyBlocks(kForwardCascade<float>, 32 * wpb, sm, (p.nLeaves + wpb - 1) / wpb);
    kForwardCascade<float><<<blocks, 32 * wpb, sm, s>>>(d, p.leaves, p.nLeaves, p.maxRow, d.L32, d.x32, d.w32,
                                                       p.cntForward);
  } else {
    const size_t sm = (size_t)wpb * p.maxRow * sizeof(double);
    const int blocks = occupancyBlocks(kForwardCascade<double>, 32 * wpb, sm, (p.nLeaves + wpb - 1) / wpb);
    kForwardCascade<double><<<blocks, 32 * wpb, sm, s>>>(d, p.leaves, p.nLeaves, p.maxRow, d.L64, d.x64, d.w64,
                                                         p.cntForward);
  }
}

void launchBackwardDynamic(const DevData& d, const PersistentPlan& p, bool fp32, cudaStream_t s) {
  if (p.n <= 0) return;
  const int wpb = 8, perWarp = 4;
  cudaMemsetAsync(p.readyBackward, 0, sizeof(int) * (size_t)d.nfrontTot, s);
  cudaMemsetAsync(p.workCounter, 0, sizeof(int), s);
  const int needed = (p.n + wpb * perWarp - 1) / (wpb * perWarp);
  if (fp32) {
    const size_t sm = (size_t)wpb * p.maxRow * sizeof(float);
    const int blocks = occupancyBlocks(kBackwardDynamic<float>, 32 * wpb, sm, needed);
    kBackwardDynamic<float><<<blocks, 32 * wpb, sm, s>>>(d, p.order, p.n, p.maxRow, d.L32, d.x32, p.readyBackward,
                                                        p.workCounter, perWarp, p.errFlag);
  } else {
    const size_t sm = (size_t)wpb * p.maxRow * sizeof(double);
    const int blocks = occupancyBlocks(kBackwardDynamic<double>, 32 * wpb, sm, needed);
    kBackwardDynamic<double><<<blocks, 32 * wpb, sm, s>>>(d, p.order, p.n, p.maxRow, d.L64, d.x64,
                                                          p.readyBackward, p.workCounter, perWarp, p.errFlag);
  }
}

}  // namespace fgpu
