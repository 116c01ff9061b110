// front_large.cu -- multifrontal factorisation and solves of the large fronts
// (more rows than one warp's shared-memory front holds), one thread block per
// front.
//
// Large fronts are marked upward-closed on the host (every ancestor of a large
// front is large), so the warp kernels of front_cascade.cu finish every small
// subtree first and these kernels take the tops of the assembly trees:
//   factor + forward: a cascade over the large fronts (blocks start at large
//     fronts whose children are all small, a parent's counter completes on its
//     last large child, the completing block climbs to it; nothing waits);
//   forward (refinement sweeps): the same cascade without the factorisation;
//   backward: a top-down work queue of large fronts seeded with the large roots
//     (a block waits only for a slot that a running block fills), before the
//     warp queue takes the small fronts below them.
// A large front is factored in place in its outputs: its pivot columns in its
// L block (nrow x npiv, column-major) and its trailing lower triangle in its
// packed update matrix (column by column, inside the parent's segment), so no
// workspace is needed.  Blocked right-looking LDL^T, panels of kPanel pivots:
// the panel is factored column by column (the unscaled column in shared
// memory), then the trailing lower triangle is updated with the panel,
// C -= L_p D_p L_p^T.  Semantics as the warp kernels and the reference's
// SPRFC1/SPRFS1/SPRBS1 seam (solExtensionModule.f90:153-505): no pivoting, a
// pivot is singular when |d_k| <= tolFactorize |a_kk|, negative pivots counted,
// children's update matrices added in child order (fixed summation order).
// Data other blocks wrote (children's updates, solution values) are read
// through L2 (__ldcg), and a block's own front data too, since its threads
// read back what others of the block wrote.

#include "kernels.h"

namespace fgpu {
namespace {

constexpr int kLT = 256;    // threads per large-front block
constexpr int kPanel = 32;  // pivots per panel

// lower-triangle entry (ii >= jj) of an nu x nu matrix packed column by column
__device__ inline int64_t packedAt(int ii, int jj, int nu) {
  return (int64_t)jj * nu - (int64_t)jj * (jj - 1) / 2 + (ii - jj);
}

template <typename T>
struct Front {
  T* L;  // nr x np, column-major
  T* U;  // packed lower triangle of the trailing nu x nu block
  int nr, np, nu;
  __device__ T* at(int i, int j) const {  // i >= j
    return j < np ? L + i + (int64_t)nr * j : U + packedAt(i - np, j - np, nu);
  }
};

__device__ inline bool singularPivot(float dk, float d0, double tol) { return !(fabsf(dk) > (float)tol * fabsf(d0)); }
__device__ inline bool singularPivot(double dk, double d0, double tol) { return !(fabs(dk) > tol * fabs(d0)); }

template <typename T>
__device__ inline T ld(const T* p) {
  return __ldcg(p);
}
template <typename T>
__device__ inline void st(T* p, T v) {
  __stcg(p, v);
}

// assembly (original entries, then the children's update matrices in child
// order) and the blocked partial LDL^T of large front f; shared: ucol (nr),
// diag0 (np), dpan (kPanel)
template <typename T>
__device__ void factorLarge(const DevData& d, int f, const T* asmVal, T* Lbase, T* Ubase, double tolFact, T* ucol,
                            T* diag0, T* dpan) {
  const int tid = threadIdx.x;
  Front<T> F{Lbase + d.fLOff[f], Ubase + d.fUOff[f], d.fNrow[f], d.fNpiv[f], d.fNrow[f] - d.fNpiv[f]};
  const int nr = F.nr, np = F.np, nu = F.nu;
  const int64_t nL = (int64_t)nr * np, nU = (int64_t)nu * (nu + 1) / 2;
  for (int64_t k = tid; k < nL; k += kLT) st(F.L + k, T(0));
  for (int64_t k = tid; k < nU; k += kLT) st(F.U + k, T(0));
  __syncthreads();
  const int64_t ao = d.fAsmOff[f];
  const int na = d.fNasm[f];
  for (int k = tid; k < na; k += kLT) {  // original entries: pivot columns only, distinct positions
    const int p = __ldg(d.asmPos + ao + k);
    st(F.L + p, __ldg(asmVal + ao + k));
  }
  __syncthreads();
  for (int k = tid; k < np; k += kLT) diag0[k] = ld(F.L + k + (int64_t)nr * k);
  // extend-add, child by child (positions are distinct within one child)
  const T* seg = Ubase + d.fSegOff[f];
  const int* spos = d.segPos + d.fSegOff[f];
  const int nch = d.fNchild[f];
  const int64_t co = d.fChildOff[f];
  int64_t off = 0;
  for (int c = 0; c < nch; ++c) {
    const int ch = d.childList[co + c];
    const int cu = d.fNrow[ch] - d.fNpiv[ch];
    const int64_t len = (int64_t)cu * (cu + 1) / 2;
    __syncthreads();
    for (int64_t k = tid; k < len; k += kLT) {
      const int p = __ldg(spos + off + k) & 0xfffff;
      T* q = F.at(p % nr, p / nr);
      st(q, ld(q) + ld(seg + off + k));
    }
    off += len;
  }
  __syncthreads();
  int neg = 0;
  bool sing = false;
  for (int k0 = 0; k0 < np; k0 += kPanel) {
    const int kb = min(kPanel, np - k0);
    // panel: pivots k0 .. k0 + kb - 1, right-looking inside the panel
    for (int k = k0; k < k0 + kb; ++k) {
      const T dk = ld(F.L + k + (int64_t)nr * k);
      for (int i = k + 1 + tid; i < nr; i += kLT) ucol[i] = ld(F.L + i + (int64_t)nr * k);
      if (tid == 0) {
        const bool bad = singularPivot(dk, diag0[k], tolFact);
        sing |= bad;
        if (dk < T(0)) ++neg;
        dpan[k - k0] = dk;
      }
      __syncthreads();
      const bool bad = singularPivot(dk, diag0[k], tolFact);
      const T inv = bad ? T(0) : T(1) / dk;
      const int je = k0 + kb - 1;
      for (int i = k + 1 + tid; i < nr; i += kLT) {
        const T l = ucol[i] * inv;
        st(F.L + i + (int64_t)nr * k, l);
        const int jm = i < je ? i : je;
        for (int j = k + 1; j <= jm; ++j) {
          T* q = F.L + i + (int64_t)nr * j;
          st(q, ld(q) - l * ucol[j]);
        }
      }
      __syncthreads();
    }
    // trailing lower triangle: columns j >= j0, C(i, j) -= sum_k L(i, k) d_k L(j, k)
    const int j0 = k0 + kb, nt = nr - j0;
    int b = 0, t = tid;
    while (b < nt && t >= nt - b) { t -= nt - b; ++b; }
    while (b < nt) {
      const int j = j0 + b, i = j + t;
      T acc = T(0);
      for (int kk = 0; kk < kb; ++kk) {
        const int k = k0 + kk;
        acc += ld(F.L + i + (int64_t)nr * k) * (ld(F.L + j + (int64_t)nr * k) * dpan[kk]);
      }
      T* q = F.at(i, j);
      st(q, ld(q) - acc);
      t += kLT;
      while (b < nt && t >= nt - b) { t -= nt - b; ++b; }
    }
    __syncthreads();
  }
  if (tid == 0) {
    const int m = d.fModel[f];
    if (neg) atomicAdd(&d.m.negPiv[m], neg);
    if (sing) atomicOr(&d.m.status[m], SS_SINGULAR);
  }
}

// forward elimination of large front f (v: nr values in shared memory)
template <typename T>
__device__ void forwardLarge(const DevData& d, int f, const T* Lbase, const double* rhs, T* X, T* W, T* v) {
  const int tid = threadIdx.x;
  const int nr = d.fNrow[f], np = d.fNpiv[f], nu = nr - np;
  const T* L = Lbase + d.fLOff[f];
  const int* rows = d.frontRows + d.fRowOff[f];
  __syncthreads();
  for (int r = tid; r < nr; r += kLT) v[r] = r < np ? (T)rhs[__ldg(rows + r)] : T(0);
  const int nc = d.fNchild[f];
  const int64_t co = d.fChildOff[f];
  for (int c = 0; c < nc; ++c) {
    __syncthreads();
    const int ch = d.childList[co + c];
    const int cu = d.fNrow[ch] - d.fNpiv[ch];
    const T* wc = W + d.fWOff[ch];
    const int* rel = d.relIndex + d.fRelOff[ch];
    for (int a = tid; a < cu; a += kLT) v[__ldg(rel + a)] += ld(wc + a);
  }
  __syncthreads();
  for (int k = 0; k < np; ++k) {
    const T yk = v[k];
    __syncthreads();
    for (int i = k + 1 + tid; i < nr; i += kLT) v[i] -= ld(L + i + (int64_t)nr * k) * yk;
    __syncthreads();
  }
  for (int r = tid; r < np; r += kLT) X[__ldg(rows + r)] = v[r] / ld(L + r + (int64_t)nr * r);
  T* wo = W + d.fWOff[f];
  for (int a = tid; a < nu; a += kLT) st(wo + a, v[np + a]);
}

// after large front f: count it at its (large) parent; returns the parent when
// this block completed the count, else -1
__device__ inline int climbLarge(const DevData& d, const PersistentPlan& p, int f, int* cnt, int* shNext) {
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    int next = -1;
    const int par = d.fParent[f];
    if (par >= 0) {
      int old;
      asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], 1;\n" : "=r"(old) : "l"(cnt + par) : "memory");
      if (old == p.fNlarge[par] - 1) next = par;
    }
    *shNext = next;
  }
  __syncthreads();
  return *shNext;
}

template <typename T>
__global__ void __launch_bounds__(kLT) kLargeFactorForward(DevData d, PersistentPlan p, const T* asmVal, T* Lbase,
                                                            T* Ubase, double tolFact, const double* rhs, T* X, T* W,
                                                            int* cnt, int doFactor) {
  extern __shared__ __align__(16) unsigned char smraw[];
  T* v = reinterpret_cast<T*>(smraw);
  T* ucol = v + p.maxRowLarge;
  T* diag0 = ucol + p.maxRowLarge;
  T* dpan = diag0 + p.maxRowLarge;
  __shared__ int shIdx, shNext;
  int* const next = cnt + d.nfrontTot;
  for (;;) {
    if (threadIdx.x == 0) shIdx = atomicAdd(next, 1);
    __syncthreads();
    const int idx = shIdx;
    __syncthreads();
    if (idx >= p.nLargeTasks) break;
    int f = p.largeTasks[idx];
    const int fl = d.m.flags[d.fModel[f]];
    const bool factor = doFactor && (fl & FL_TANGENT);
    while ((fl & FL_ACTIVE) && f >= 0) {
      if (factor) factorLarge<T>(d, f, asmVal, Lbase, Ubase, tolFact, ucol, diag0, dpan);
      forwardLarge<T>(d, f, Lbase, rhs, X, W, v);
      f = climbLarge(d, p, f, cnt, &shNext);
    }
  }
}

// Top-down queue of large fronts (see front_cascade.cu's kBackwardQueue for
// the protocol): a block takes the next slot, waits (bounded) until a front is
// stored there, solves it, stores its large children but the first in fresh
// slots and continues with the first; the small children are left to the warp
// queue launched afterwards.  acc as kBackwardQueue.
template <typename T>
__global__ void __launch_bounds__(kLT) kLargeBackward(DevData d, PersistentPlan p, const T* Lbase, T* X, int* queue,
                                                       int* ctr, int* errFlag, int acc, int finalize) {
  extern __shared__ __align__(16) unsigned char smraw[];
  T* xs = reinterpret_cast<T*>(smraw);
  __shared__ int shSlot, shF, shOk;
  const int tid = threadIdx.x;
  const int total = *(volatile const int*)(ctr + 2);
  for (;;) {
    if (tid == 0) shSlot = atomicAdd(ctr, 1);
    __syncthreads();
    const int slot = shSlot;
    __syncthreads();
    if (slot >= total) break;
    if (tid == 0) {
      int f = -1, ok = 1;
      long long spins = 0;
      while ((f = *(volatile const int*)(queue + slot)) < 0) {
        __nanosleep(32);
        if (++spins > p.spinLimit) {
          atomicOr(errFlag, 1);
          ok = 0;
          break;
        }
      }
      __threadfence();
      shF = f;
      shOk = ok;
    }
    __syncthreads();
    int f = shF;
    if (!shOk) break;
    while (f >= 0) {
      const int nr = d.fNrow[f], np = d.fNpiv[f];
      const T* L = Lbase + d.fLOff[f];
      const int* rows = d.frontRows + d.fRowOff[f];
      for (int r = tid; r < nr; r += kLT) xs[r] = ld(X + __ldg(rows + r));
      __syncthreads();
      // the update rows' contribution for every pivot, then the unit triangle
      for (int k = tid; k < np; k += kLT) {
        T a = xs[k];
        for (int i = np; i < nr; ++i) a -= ld(L + i + (int64_t)nr * k) * xs[i];
        xs[k] = a;
      }
      __syncthreads();
      for (int j = np - 1; j > 0; --j) {
        const T xj = xs[j];
        for (int k = tid; k < j; k += kLT) xs[k] -= ld(L + j + (int64_t)nr * k) * xj;
        __syncthreads();
      }
      for (int r = tid; r < np; r += kLT) {
        const int row = __ldg(rows + r);
        const T x = xs[r];
        st(X + row, x);
        if (acc == 0) {
          d.del[row] = (double)x;
        } else {
          const double xr = acc == 1 ? (double)x : d.xref[row] + (double)x;
          d.xref[row] = xr;
          if (finalize) d.del[row] = xr;
        }
      }
      __threadfence();
      __syncthreads();
      // large children: the first continues here, the others go to fresh slots
      const int nch = d.fNchild[f];
      const int* chl = d.childList + d.fChildOff[f];
      int first = -1;
      if (tid == 0) {
        int nl = 0;
        for (int c = 0; c < nch; ++c)
          if (p.fLarge[chl[c]]) {
            if (first < 0) first = chl[c];
            else ++nl;
          }
        if (nl > 0) {
          int base = atomicAdd(ctr + 1, nl);
          bool skip = true;
          for (int c = 0; c < nch; ++c)
            if (p.fLarge[chl[c]]) {
              if (skip) { skip = false; continue; }
              atomicExch(queue + base++, chl[c]);
            }
        }
        shF = first;
      }
      __syncthreads();
      f = shF;
      __syncthreads();
    }
  }
}

int smCount() {
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
int gridFor(K kernel, size_t smem, int needed) {
  int perSm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, kernel, kLT, smem) != cudaSuccess || perSm < 1) perSm = 1;
  const int cap = perSm * smCount();
  return needed < 1 ? 1 : (needed < cap ? needed : cap);
}

template <typename K>
void bigSmem(K kernel, size_t bytes) {
  if (bytes > 48 * 1024) cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

template <typename T>
void factorForwardLarge(const DevData& d, const PersistentPlan& p, const T* asmVal, T* L, T* U, const double* rhs,
                        T* X, T* W, int* cnt, bool factor, cudaStream_t s) {
  const size_t sm = (3 * (size_t)p.maxRowLarge + kPanel) * sizeof(T);
  bigSmem(kLargeFactorForward<T>, sm);
  const int grid = gridFor(kLargeFactorForward<T>, sm, p.nLargeTasks);
  kLargeFactorForward<T><<<grid, kLT, sm, s>>>(d, p, asmVal, L, U, 1.0e-12, rhs, X, W, cnt, factor ? 1 : 0);
}

}  // namespace

void launchLargeFactorForward(const DevData& d, const PersistentPlan& p, bool fp32, const double* rhs,
                              cudaStream_t s) {
  if (p.nLargeTasks <= 0) return;
  if (fp32) factorForwardLarge<float>(d, p, d.asmVal32, d.L32, d.U32, rhs, d.x32, d.w32, p.cntLargeFactor, true, s);
  else factorForwardLarge<double>(d, p, d.asmVal64, d.L64, d.U64, rhs, d.x64, d.w64, p.cntLargeFactor, true, s);
}

void launchLargeForward(const DevData& d, const PersistentPlan& p, bool fp32, const double* rhs, int sweep,
                        cudaStream_t s) {
  if (p.nLargeTasks <= 0) return;
  int* cnt = p.cntLargeForward + (size_t)(sweep - 1) * ((size_t)d.nfrontTot + 1);
  if (fp32) factorForwardLarge<float>(d, p, d.asmVal32, d.L32, d.U32, rhs, d.x32, d.w32, cnt, false, s);
  else factorForwardLarge<double>(d, p, d.asmVal64, d.L64, d.U64, rhs, d.x64, d.w64, cnt, false, s);
}

void launchLargeBackward(const DevData& d, const PersistentPlan& p, bool fp32, int sweep, bool last, cudaStream_t s) {
  if (p.nLargeTasks <= 0) return;
  const int acc = !fp32 ? 0 : (sweep == 0 ? 1 : 2);
  const int fin = (fp32 && last) ? 1 : 0;
  int* queue = p.bwLQueue + (size_t)sweep * p.largeStride;
  int* ctr = p.bwLCtr + 4 * sweep;
  if (fp32) {
    const size_t sm = (size_t)p.maxRowLarge * sizeof(float);
    bigSmem(kLargeBackward<float>, sm);
    const int grid = gridFor(kLargeBackward<float>, sm, p.nLargeTasks);
    kLargeBackward<float><<<grid, kLT, sm, s>>>(d, p, d.L32, d.x32, queue, ctr, p.errFlag, acc, fin);
  } else {
    const size_t sm = (size_t)p.maxRowLarge * sizeof(double);
    bigSmem(kLargeBackward<double>, sm);
    const int grid = gridFor(kLargeBackward<double>, sm, p.nLargeTasks);
    kLargeBackward<double><<<grid, kLT, sm, s>>>(d, p, d.L64, d.x64, queue, ctr, p.errFlag, acc, fin);
  }
}

}  // namespace fgpu
