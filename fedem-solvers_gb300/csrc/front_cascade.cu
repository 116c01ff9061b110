// front_cascade.cu -- one-launch multifrontal factorisation and solves over
// the assembly trees of all models, without co-residency assumptions.
//
// Factor and forward solve run bottom-up as a cascade: warps start at the
// leaves; a front's counter is incremented (release) when one of its children
// is done, and the warp whose increment completes the count goes on with the
// parent itself.  Nothing ever waits, so the launch is correct whatever the
// residency (several engines may run concurrently on their own streams).
// The backward solve runs top-down through a work queue of fronts whose
// parents are solved (kBackwardQueue); a warp waits only for a queue slot to
// be filled, by warps that are running and never wait themselves, so the wait
// ends whatever the residency.  Each wait is still bounded and sets errFlag
// when it runs out.
// The forward and backward solves stage each front's L block in shared memory
// first (one burst of loads instead of one load latency per pivot).
//
// These kernels replace the factor and solve of the absent SAM/SPR solver that
// the reference calls from csSolve (src/vpmCommon/vpmLinAlg/
// solExtensionModule.f90:153-505: SPRFC1/SPRFC3, SPRFS1/SPRBS1).  Semantics
// kept: LDL^T without pivoting, a pivot counts as singular when
// |d_k| <= tolFactorize * |a_kk| (error -3), negative pivots are counted.
// Fronts are dense column-major nrow x nrow tiles in shared memory (lower
// triangle used), pivots first; children's contributions are added in child
// order, so every sum has a fixed order (no atomics on floating-point data).
// Mixed precision: FP32 factor and correction solves; the FP64 refinement
// residual is in front_kernels.cu.

#include <atomic>

#include "kernels.h"

namespace fgpu {
namespace {


// Partial LDL^T of a front, blocked: the pivot panel (all rows, the np
// pivot columns) is factored right-looking within the panel, one row per lane;
// the update matrix (the Schur complement of the update block) is then formed
// in one rank-np pass over its lower triangle, one entry per lane, and stored
// packed column by column at Uout.  F afterwards holds D on the diagonal and
// the unit L below it in the panel; the unscaled panel values of the update
// rows (L d) are kept in the unused upper triangle (row k, column i) for the
// rank-np pass.
// a pivot counts as singular when |d_k| <= tolFactorize * |a_kk| (the FP32
// factor tests in FP32, keeping the FP64 pipe free)
__device__ inline bool singularPivot(float dk, float d0, double tol) { return !(fabsf(dk) > (float)tol * fabsf(d0)); }
__device__ inline bool singularPivot(double dk, double d0, double tol) { return !(fabs(dk) > tol * fabs(d0)); }

// Panel factorisations of the small fronts, all with the same arithmetic in
// the same order (so the same factor to the last bit), picked per batch by the
// engine's autotuner: pivot by pivot with the multipliers passed by shuffles
// and the rows kept in shared memory (few registers, high occupancy), or
// register-blocked (fewer instructions and shared-memory accesses, more
// registers) in blocks of 8 or 4 pivots.
constexpr int kPanelShuffle = 0;
constexpr int kPanelRegisters = 1;   // blocks of 8 pivots, fronts up to 64 rows
constexpr int kPanelRegisters4 = 2;  // blocks of 4 pivots, one row per lane (fronts up to 32 rows)

// pivot by pivot: rows lane and lane + 32 in shared memory; the multipliers of
// the pivot rows (lanes below np) are passed by shuffles, one barrier per pivot
template <typename T>
__device__ void panelShuffle(T* F, const T* diag0, int nr, int np, int lane, double tolFact, int& neg, bool& sing) {
  const int i0 = lane, i1 = lane + 32;
  for (int k = 0; k < np; ++k) {
    const T dk = F[k + nr * k];
    const bool bad = singularPivot(dk, diag0[k], tolFact);
    sing |= bad;
    if (dk < T(0)) ++neg;
    const T inv = bad ? T(0) : T(1) / dk;
    const bool r0 = i0 > k && i0 < nr, r1 = i1 > k && i1 < nr;
    const T f0 = r0 ? F[i0 + nr * k] : T(0), f1 = r1 ? F[i1 + nr * k] : T(0);
    const T l0 = f0 * inv, l1 = f1 * inv;
    for (int j = k + 1; j < np; ++j) {
      const T lj = __shfl_sync(0xffffffffu, l0, j);
      if (r0 && j <= i0) F[i0 + nr * j] -= f0 * lj;
      if (r1) F[i1 + nr * j] -= f1 * lj;
    }
    if (r0) {
      if (i0 >= np) F[k + nr * i0] = f0;
      F[i0 + nr * k] = l0;
    }
    if (r1) {
      if (i1 >= np) F[k + nr * i1] = f1;
      F[i1 + nr * k] = l1;
    }
    __syncwarp();
  }
}

// register-blocked in blocks of PB pivots (TWO: a second row per lane, fronts
// of up to 64 rows; else at most 32 rows)
template <typename T, int PB, bool TWO>
__device__ void panelRegisters(T* F, const T* diag0, int nr, int np, int lane, double tolFact, int& neg,
                               bool& sing) {
  // Register-blocked panel: lane r owns rows r and r + 32; the pivot columns
  // are taken PB at a time.  Inside a block the row values sit in
  // registers and each multiplier l_jk is passed by a shuffle from the lane
  // owning row j; the block's columns are then stored (l_ik below the
  // diagonal, the unscaled value of an update row in its upper position),
  // and the later pivot columns receive the block's updates all at once,
  // l_jk read from shared memory (one broadcast load per value).  Every
  // entry receives the same multiply-subtracts in the same order as in a
  // right-looking elimination one pivot at a time, so the factor is the same
  // to the last bit, with a fraction of the shared-memory traffic and no
  // barrier per pivot.
  const int i0 = lane, i1 = lane + 32;
  const bool two = TWO && nr > 32;     // warp-uniform: a second row per lane
  const bool h1 = two && i1 < nr;      // row i1 exists (it is below every pivot: np <= 32)
  for (int k0 = 0; k0 < np; k0 += PB) {
    const int kb = min(PB, np - k0);
    const bool h0 = i0 >= k0 && i0 < nr;
    T a0[PB], a1[PB];
#pragma unroll
    for (int kk = 0; kk < PB; ++kk) {
      a0[kk] = (kk < kb && h0) ? F[i0 + nr * (k0 + kk)] : T(0);
      a1[kk] = (kk < kb && h1) ? F[i1 + nr * (k0 + kk)] : T(0);
    }
#pragma unroll
    for (int kk = 0; kk < PB; ++kk) {
      if (kk >= kb) break;  // warp-uniform
      const int k = k0 + kk;
      const T dk = __shfl_sync(0xffffffffu, a0[kk], k);  // row k < 32 is lane k's first row
      const bool bad = singularPivot(dk, diag0[k], tolFact);
      sing |= bad;
      if (dk < T(0)) ++neg;
      const T inv = bad ? T(0) : T(1) / dk;
      const bool r0 = i0 > k && i0 < nr;
      const T f0 = r0 ? a0[kk] : T(0), f1 = h1 ? a1[kk] : T(0);
      const T l0 = f0 * inv, l1 = f1 * inv;
#pragma unroll
      for (int jj = kk + 1; jj < PB; ++jj) {
        if (jj >= kb) break;
        const T lj = __shfl_sync(0xffffffffu, l0, k0 + jj);
        if (r0 && k0 + jj <= i0) a0[jj] -= f0 * lj;
        if (h1) a1[jj] -= f1 * lj;
      }
      if (i0 == k) F[k + nr * k] = dk;
      if (r0) {
        F[i0 + nr * k] = l0;
        if (i0 >= np) F[k + nr * i0] = f0;
        a0[kk] = f0;
      }
      if (h1) {
        F[i1 + nr * k] = l1;
        if (i1 >= np) F[k + nr * i1] = f1;
        a1[kk] = f1;
      }
    }
    __syncwarp();
    // the later pivot columns j (row i >= j): C(i, j) -= f_i,k l_j,k over the block's k in order
    for (int j = k0 + kb; j < np; ++j) {
      T lj[PB];
#pragma unroll
      for (int kk = 0; kk < PB; ++kk) lj[kk] = kk < kb ? F[j + nr * (k0 + kk)] : T(0);
      if (i0 >= j && i0 < nr) {
        T c = F[i0 + nr * j];
#pragma unroll
        for (int kk = 0; kk < PB; ++kk)
          if (kk < kb) c -= a0[kk] * lj[kk];
        F[i0 + nr * j] = c;
      }
      if (h1) {
        T c = F[i1 + nr * j];
#pragma unroll
        for (int kk = 0; kk < PB; ++kk)
          if (kk < kb) c -= a1[kk] * lj[kk];
        F[i1 + nr * j] = c;
      }
    }
    __syncwarp();
  }
}

template <typename T, int PANEL>
__device__ void factorBlocked(T* F, T* lcol, const T* diag0, int nr, int np, int lane, double tolFact, int& neg,
                              bool& sing, T* Uout) {
  if (np <= 32 && nr <= 64) {
    if constexpr (PANEL == kPanelRegisters) {
      panelRegisters<T, 8, true>(F, diag0, nr, np, lane, tolFact, neg, sing);
    } else if constexpr (PANEL == kPanelRegisters4) {
      if (nr <= 32) panelRegisters<T, 4, false>(F, diag0, nr, np, lane, tolFact, neg, sing);
      else panelShuffle<T>(F, diag0, nr, np, lane, tolFact, neg, sing);
    } else {
      panelShuffle<T>(F, diag0, nr, np, lane, tolFact, neg, sing);
    }
  } else {
    for (int k = 0; k < np; ++k) {
      const T dk = F[k + nr * k];
      const bool bad = singularPivot(dk, diag0[k], tolFact);
      sing |= bad;
      if (dk < T(0)) ++neg;
      const T inv = bad ? T(0) : T(1) / dk;
      for (int i = k + 1 + lane; i < nr; i += 32) lcol[i] = F[i + nr * k] * inv;
      __syncwarp();
      for (int i = k + 1 + lane; i < nr; i += 32) {
        const T fik = F[i + nr * k];
        const int je = i < np - 1 ? i : np - 1;
        for (int j = k + 1; j <= je; ++j) F[i + nr * j] -= fik * lcol[j];
        if (i >= np) F[k + nr * i] = fik;
        F[i + nr * k] = lcol[i];
      }
      __syncwarp();
    }
  }
  // update matrix, lower triangle packed column by column: entry e = lane + 32 q
  // is (row np + b + t, column np + b)
  const int nu = nr - np;
  int b = 0, t = lane;
  while (b < nu && t >= nu - b) { t -= nu - b; ++b; }
  for (int e = lane; b < nu; e += 32) {
    const int i = np + b + t, j = np + b;
    T acc = T(0);
    for (int k = 0; k < np; ++k) acc += F[k + nr * i] * F[j + nr * k];
    Uout[e] = F[i + nr * j] - acc;
    t += 32;
    while (b < nu && t >= nu - b) { t -= nu - b; ++b; }
  }
  __syncwarp();
}

// partial LDL^T of front f in shared memory (F: maxRow^2, lcol/diag0: maxRow).
// The original entries (front-ordered copy of the CSR values) and the
// children's packed update matrices are contiguous per front and loaded
// kFrontBatch per lane before use; the rank-1 updates run one row per lane.
constexpr int kFrontBatch = 4;
// Uout: the front's packed update matrix (its place in the parent's
// segment); segIn: the front's own children segment
template <typename T, int PANEL>
__device__ void factorOneFront(const DevData& d, int f, T* F, T* lcol, T* diag0, const T* asmVal, T* Lbase,
                               T* Uout, const T* segIn, double tolFact, int lane) {
  const int m = d.fModel[f];
  const int nr = d.fNrow[f], np = d.fNpiv[f];
  const int64_t ao = d.fAsmOff[f], so = d.fSegOff[f];
  const int na = d.fNasm[f], ns = d.fSegLen[f], nch = d.fNchild[f];
  for (int k = lane; k < nr * nr; k += 32) F[k] = T(0);
  for (int k0 = 0; k0 < na; k0 += 32 * kFrontBatch) {
    T val[kFrontBatch];
    int pos[kFrontBatch];
#pragma unroll
    for (int u = 0; u < kFrontBatch; ++u) {
      const int k = k0 + 32 * u + lane;
      pos[u] = k < na ? __ldg(d.asmPos + ao + k) : -1;
      val[u] = k < na ? __ldg(asmVal + ao + k) : T(0);
    }
    __syncwarp();
#pragma unroll
    for (int u = 0; u < kFrontBatch; ++u)
      if (pos[u] >= 0) F[pos[u]] = val[u];
  }
  __syncwarp();
  for (int k = lane; k < np; k += 32) diag0[k] = F[k + nr * k];
  __syncwarp();
  // extend-add of the children's update matrices, child by child
  for (int k0 = 0; k0 < ns; k0 += 32 * kFrontBatch) {
    T val[kFrontBatch];
    int pc[kFrontBatch];
#pragma unroll
    for (int u = 0; u < kFrontBatch; ++u) {
      const int k = k0 + 32 * u + lane;
      pc[u] = k < ns ? __ldg(d.segPos + so + k) : -1;
      val[u] = k < ns ? __ldcg(segIn + k) : T(0);
    }
    for (int c = 0; c < nch; ++c) {
#pragma unroll
      for (int u = 0; u < kFrontBatch; ++u)
        if (pc[u] >= 0 && (pc[u] >> 20) == c) F[pc[u] & 0xfffff] += val[u];
      __syncwarp();
    }
  }
  int neg = 0;
  bool sing = false;
  factorBlocked<T, PANEL>(F, lcol, diag0, nr, np, lane, tolFact, neg, sing, Uout);
  T* Lout = Lbase + d.fLOff[f];
  for (int k = lane; k < nr * np; k += 32) Lout[k] = F[k];
  if (lane == 0) {
    if (neg) atomicAdd(&d.m.negPiv[m], neg);
    if (sing) atomicOr(&d.m.status[m], SS_SINGULAR);
  }
}

// forward elimination of front f: v = [b_p; 0] + children's updates, y = L11^-1 v_p,
// w = v_u - L21 y; X(pivots) = D^-1 y
// copies the nr x np block L of a front into the warp's staging area Ls when
// it fits (capL values), else returns the global block
// asynchronous global -> shared copies of single elements (cp.async): every
// copy of a block is in flight at once and none occupies a register
template <typename T>
__device__ inline void copyAsync(T* dstShared, const T* srcGlobal) {
  static_assert(sizeof(T) == 4 || sizeof(T) == 8, "4- or 8-byte elements");
  const unsigned dst = (unsigned)__cvta_generic_to_shared(dstShared);
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(dst), "l"(srcGlobal), "n"(sizeof(T)));
}
__device__ inline void copyAsyncWait() {
  asm volatile("cp.async.commit_group;\n" ::);
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}

// copies the L block into Ls (callers wait with copyAsyncWait and __syncwarp
// before reading Ls); returns the global block when it does not fit
template <typename T>
__device__ inline const T* stageL(const T* Lg, int cnt, T* Ls, int capL, int lane) {
  if (cnt > capL) return Lg;
  for (int k = lane; k < cnt; k += 32) copyAsync(Ls + k, Lg + k);
  return Ls;
}

template <typename T>
__device__ void forwardOneFront(const DevData& d, int f, T* v, T* Ls, int capL, const T* Lbase, const double* rhs,
                                T* X, T* W, int lane, const T* Lres = nullptr) {
  const int nr = d.fNrow[f], np = d.fNpiv[f], nu = nr - np;
  const int* rows = d.frontRows + d.fRowOff[f];
  // the factor block first (independent loads; or the front just factored in
  // shared memory), then the right-hand side of the pivot rows rounded to the
  // solve precision
  const T* L = Lres ? Lres : stageL(Lbase + d.fLOff[f], nr * np, Ls, capL, lane);
  for (int r = lane; r < nr; r += 32) v[r] = r < np ? (T)rhs[__ldg(rows + r)] : T(0);
  copyAsyncWait();
  __syncwarp();
  const int nc = d.fNchild[f];
  const int64_t co = d.fChildOff[f];
  for (int c = 0; c < nc; ++c) {
    const int ch = d.childList[co + c];
    const int cu = d.fNrow[ch] - d.fNpiv[ch];
    const T* wc = W + d.fWOff[ch];
    const int* rel = d.relIndex + d.fRelOff[ch];
    for (int a = lane; a < cu; a += 32) v[__ldg(rel + a)] += __ldcg(wc + a);
    __syncwarp();
  }
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

// Forward elimination with few dependent memory round trips (fronts of at most
// 64 rows and 64 child update rows): the front's descriptors, then its L block
// (asynchronous copies), row list and child gather list together, then the
// right-hand side and the children's update values together.

// Wout: where the front's update vector goes; Win: the children's update
// vectors concatenated in child order in shared memory (their gather list
// order), or null to read them from W
// Descriptors a solve of front f reads, loaded together in one round of
// independent loads (every lane the same address: broadcasts).  The caller
// loads them early, the parent's climb data right after (ParentLink), so that
// neither costs a round trip of its own later.
struct SolveDesc {
  int f, nr, np, cg0, ncg, nch, parent;
  int64_t lOff, rowOff, wOff;
};
__device__ inline SolveDesc solveDesc(const DevData& d, int f) {
  SolveDesc q;
  q.f = f;
  q.nr = d.fNrow[f];
  q.np = d.fNpiv[f];
  q.cg0 = d.cgOff[f];
  q.ncg = d.cgOff[f + 1] - q.cg0;
  q.nch = d.fNchild[f];
  q.parent = d.fParent[f];
  q.lOff = d.fLOff[f];
  q.rowOff = d.fRowOff[f];
  q.wOff = d.fWOff[f];
  return q;
}

template <typename T>
__device__ bool forwardOneFrontFast(const DevData& d, const SolveDesc& q, T* v, T* Ls, int capL, const T* Lbase,
                                    const double* rhs, T* X, const T* W, int lane, const T* Lres, T* Wout,
                                    const T* Win = nullptr) {
  const int nr = q.nr, np = q.np;
  const int cg0 = q.cg0, ncg = q.ncg, nch = q.nch;
  const int cnt = nr * np;
  if (nr > 64 || ncg > 64 || (!Lres && cnt > capL)) return false;
  const int* rows = d.frontRows + q.rowOff;
  // second round of loads: independent loads (the L block asynchronously into shared memory)
  if (!Lres) {
    const T* Lg = Lbase + q.lOff;
    for (int k = lane; k < cnt; k += 32) copyAsync(Ls + k, Lg + k);
  }
  int row[2], src[2], dst[2];
#pragma unroll
  for (int u = 0; u < 2; ++u) {
    const int r = lane + 32 * u;
    row[u] = r < np ? __ldg(rows + r) : -1;
    src[u] = r < ncg ? __ldg(d.cgSrc + cg0 + r) : -1;
    dst[u] = r < ncg ? __ldg(d.cgDst + cg0 + r) : 0;
  }
  // third round of loads: values through the indices
  double b[2];
  T wv[2];
#pragma unroll
  for (int u = 0; u < 2; ++u) {
    b[u] = row[u] >= 0 ? rhs[row[u]] : 0.0;
    wv[u] = src[u] < 0 ? T(0) : Win ? Win[lane + 32 * u] : __ldcg(W + src[u]);
  }
  if (!Lres) copyAsyncWait();
  const T* L = Lres ? Lres : Ls;
#pragma unroll
  for (int u = 0; u < 2; ++u) {
    const int r = lane + 32 * u;
    if (r < nr) v[r] = r < np ? (T)b[u] : T(0);
  }
  __syncwarp();
  for (int c = 0; c < nch; ++c) {
#pragma unroll
    for (int u = 0; u < 2; ++u)
      if (src[u] >= 0 && (dst[u] >> 16) == c) v[dst[u] & 0xffff] += wv[u];
    __syncwarp();
  }
  // the elimination with the rows in registers (lane r: rows r and r + 32), the
  // pivot value of each step passed by a shuffle: no barrier between steps
  T v0 = lane < nr ? v[lane] : T(0), v1 = lane + 32 < nr ? v[lane + 32] : T(0);
  for (int k = 0; k < np; ++k) {
    const T yk = __shfl_sync(0xffffffffu, k < 32 ? v0 : v1, k & 31);
    const T* Lk = L + (size_t)nr * k;
    if (lane > k && lane < nr) v0 -= Lk[lane] * yk;
    if (lane + 32 > k && lane + 32 < nr) v1 -= Lk[lane + 32] * yk;
  }
  if (lane >= np && lane < nr) Wout[lane - np] = v0;
  if (lane + 32 >= np && lane + 32 < nr) Wout[lane + 32 - np] = v1;
  if (lane < np) X[row[0]] = v0 / L[lane + (size_t)nr * lane];
  if (lane + 32 < np) X[row[1]] = v1 / L[(lane + 32) + (size_t)nr * (lane + 32)];
  return true;
}

// After a front is done: release its data and count it at the parent; true
// if this warp completed the parent's count (and must go on with the parent),
// false otherwise (also for a large parent: the large-front kernels take it up
// afterwards).  The parent's id, size class and child count (ParentLink) are
// loaded while the front is still being processed, so the climb itself is one
// atomic.  The warp barrier orders every lane's stores before lane 0's counter
// update, a release-acquire RMW at GPU scope (no full fence): the warp that
// completes the count acquires the children's stores, and its barrier passes
// them on to its other lanes.
struct ParentLink {
  int p, nch;
  bool large;
};
__device__ inline ParentLink parentLink(const DevData& d, int p) {
  ParentLink l{p, 0, true};
  if (p >= 0) {
    l.large = d.fLarge[p] != 0;
    l.nch = d.fNchild[p];
  }
  return l;
}
__device__ inline bool climb(const ParentLink& l, int* cnt, int lane) {
  __syncwarp();
  int go = 0;
  if (lane == 0 && l.p >= 0 && !l.large) {
    int old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], 1;\n" : "=r"(old) : "l"(cnt + l.p) : "memory");
    go = old == l.nch - 1;
  }
  go = __shfl_sync(0xffffffffu, go, 0);
  __syncwarp();
  return go != 0;
}

// A root's elimination is complete: its counter gets kRootDone added with
// release semantics (after the warp barrier that orders every lane's stores),
// which the fused back substitution acquires before it solves the root.
constexpr int kRootDone = 1 << 24;
__device__ inline void releaseRoot(int* cnt, int f, int lane) {
  __syncwarp();
  if (lane == 0) asm volatile("red.release.gpu.global.add.s32 [%0], %1;\n" ::"l"(cnt + f), "r"(kRootDone) : "memory");
  __syncwarp();
}
__device__ inline int acquireCount(const int* c) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];\n" : "=r"(v) : "l"(c) : "memory");
  return v;
}

// Leaves are taken in their stored order (longest root paths first) from a
// launch-wide counter, cnt[nfrontTot]; lane 0 asks for the next leaf before
// the current one is processed, so the request's latency is hidden.
__device__ inline int requestLeaf(int* next, int lane) { return lane == 0 ? atomicAdd(next, 1) : 0; }

// Forward-elimination tasks are single leaves or groups: a group is a front
// whose children are all leaves (kGroupBit set in the task), eliminated by one
// warp -- the children first, their update vectors kept in shared memory, then
// the front itself -- so that inside a group nothing goes through global
// memory or a counter.  After a task the warp climbs as from a leaf.  (The
// factorisation keeps one task per leaf: there the leaves are the most
// expensive fronts, and factoring siblings one after the other lengthens the
// critical path more than the saved climbs shorten it.)
constexpr int kGroupBit = 1 << 30;

// factorisation (models with a tangent update) fused with the forward
// elimination of the first solve (all active models): one climb per front, and
// the forward elimination reads L from the front still in shared memory
template <typename T>
__device__ void backwardQueueLoop(const DevData& d, int maxRow, int capL, const T* Lbase, T* X, int* queue, int* ctr,
                                  const unsigned char* bwInline, int* errFlag, int acc, int finalize,
                                  long long spinLimit, T* xs, T* Ls, int lane, const int* rootDone);
template <typename T, int PANEL>
__global__ void kFactorForwardCascade(DevData d, const int* __restrict__ leaves, int nLeaves, int maxRow,
                                      const T* asmVal, T* Lbase, T* Ubase, double tolFact, const double* rhs, T* X,
                                      T* Wv, int* cnt, FusedBackward fb) {
  pdlEntry();
  extern __shared__ __align__(16) unsigned char smraw[];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int capL = maxRow * maxRow;  // F doubles as the staging area of L
  T* F = reinterpret_cast<T*>(smraw) + (size_t)w * ((size_t)maxRow * maxRow + 3 * maxRow);
  T* lcol = F + (size_t)maxRow * maxRow;
  T* diag0 = lcol + maxRow;
  T* v = diag0 + maxRow;
  int* const next = cnt + d.nfrontTot;
  int idx = __shfl_sync(0xffffffffu, requestLeaf(next, lane), 0);
  while (idx < nLeaves) {
    const int pending = requestLeaf(next, lane);
    int f = leaves[idx];
    const int fl = d.m.flags[d.fModel[f]];
    const bool factor = fl & FL_TANGENT;
    while ((fl & FL_ACTIVE) && f >= 0) {
      const SolveDesc q = solveDesc(d, f);
      const ParentLink pl = parentLink(d, q.parent);
      const T* Lres = nullptr;
      if (factor) {
        factorOneFront<T, PANEL>(d, f, F, lcol, diag0, asmVal, Lbase, Ubase + d.fUOff[f], Ubase + d.fSegOff[f],
                                 tolFact, lane);
        __syncwarp();
        Lres = F;
      }
      if (!forwardOneFrontFast<T>(d, q, v, F, capL, Lbase, rhs, X, Wv, lane, Lres, Wv + q.wOff))
        forwardOneFront<T>(d, f, v, F, capL, Lbase, rhs, X, Wv, lane, Lres);
      if (fb.queue && q.parent < 0) releaseRoot(cnt, f, lane);
      f = climb(pl, cnt, lane) ? q.parent : -1;
    }
    idx = __shfl_sync(0xffffffffu, pending, 0);
  }
  // Fused first back substitution: once every leaf is taken, the warp serves
  // the back-substitution queue.  Every front still to be eliminated belongs to
  // a running warp that never waits, so a root the queue hands out completes;
  // the warp waits for it (bounded) before solving it.
  if (fb.queue)
    backwardQueueLoop<T>(d, maxRow, fb.capL, Lbase, X, fb.queue, fb.ctr, fb.bwInline, fb.errFlag, fb.acc, fb.finalize,
                         fb.spinLimit, v, F, lane, cnt);
}

template <typename T>
__global__ void kForwardCascade(DevData d, const int* __restrict__ tasks, int nTasks, int maxRow, int capL,
                                const T* Lbase, const double* rhs, T* X, T* W, int* cnt) {
  pdlEntry();
  extern __shared__ __align__(16) unsigned char smraw[];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  T* v = reinterpret_cast<T*>(smraw) + (size_t)w * (maxRow + capL + 64);
  T* Ls = v + maxRow;
  T* wsm = Ls + capL;
  int* const next = cnt + d.nfrontTot;
  int idx = __shfl_sync(0xffffffffu, requestLeaf(next, lane), 0);
  while (idx < nTasks) {
    const int pending = requestLeaf(next, lane);
    const int task = tasks[idx];
    int f = task & ~kGroupBit;
    const bool active = d.m.flags[d.fModel[f]] & FL_ACTIVE;
    if (!active) f = -1;
    SolveDesc q;
    if (f >= 0) q = solveDesc(d, f);
    if (f >= 0 && (task & kGroupBit)) {
      const ParentLink pl = parentLink(d, q.parent);
      const int* ch = d.childList + d.fChildOff[f];
      int wo = 0;
      SolveDesc cq = solveDesc(d, ch[0]);
      for (int c = 0; c < q.nch; ++c) {
        // the next child's descriptors are loaded while this one is eliminated
        const SolveDesc nq = solveDesc(d, ch[c + 1 < q.nch ? c + 1 : c]);
        forwardOneFrontFast<T>(d, cq, v, Ls, capL, Lbase, rhs, X, W, lane, nullptr, wsm + wo);
        wo += cq.nr - cq.np;
        __syncwarp();
        cq = nq;
      }
      forwardOneFrontFast<T>(d, q, v, Ls, capL, Lbase, rhs, X, W, lane, nullptr, W + q.wOff, wsm);
      f = climb(pl, cnt, lane) ? q.parent : -1;
      if (f >= 0) q = solveDesc(d, f);
    }
    while (f >= 0) {
      // the parent's climb data and descriptors are loaded ahead of this
      // front's elimination; they are used only if this warp goes on to it
      const ParentLink pl = parentLink(d, q.parent);
      const SolveDesc pq = solveDesc(d, q.parent >= 0 ? q.parent : f);
      if (!forwardOneFrontFast<T>(d, q, v, Ls, capL, Lbase, rhs, X, W, lane, nullptr, W + q.wOff))
        forwardOneFront<T>(d, f, v, Ls, capL, Lbase, rhs, X, W, lane);
      f = climb(pl, cnt, lane) ? q.parent : -1;
      q = pq;
    }
    idx = __shfl_sync(0xffffffffu, pending, 0);
  }
}

// backward substitution of front f (parent values already in X): the update
// rows' contribution for every pivot at once (one lane per pivot), then the
// unit triangle column by column; writes the pivot values to X
// accumulation of the solved pivot values: ACC_SET del = x (FP64 solve), ACC_FIRST
// xref = x, ACC_ADD xref += x (FP32 refinement sweeps); finalize: del = xref
enum { ACC_SET = 0, ACC_FIRST = 1, ACC_ADD = 2 };

// Descriptors of a back substitution, loaded together: the front's, and with
// them those of its first child (the front the warp goes on to), so that the
// next front starts without a descriptor round trip.
struct BackDesc {
  int f, nr, np, nch;
  bool inl;  // children all leaves, solved by this warp
  int64_t lOff, rowOff, childOff;
};
__device__ inline BackDesc backDesc(const DevData& d, const unsigned char* bwInline, int f) {
  BackDesc q;
  q.f = f;
  q.nr = d.fNrow[f];
  q.np = d.fNpiv[f];
  q.nch = d.fNchild[f];
  q.inl = bwInline[f] != 0;
  q.lOff = d.fLOff[f];
  q.rowOff = d.fRowOff[f];
  q.childOff = d.fChildOff[f];
  return q;
}

// l2Only: L was written in the same launch (fused back substitution), so it
// is staged through L2 loads; an L1 line filled earlier in the launch by a
// neighbouring front's solve could hold its old values (fusableBackward
// guarantees that every block fits the staging area)
template <typename T>
__device__ void backwardOneFront(const DevData& d, const BackDesc& q, T* xs, T* Ls, int capL, const T* Lbase, T* X,
                                 int acc, bool finalize, int lane, bool l2Only = false) {
  const int nr = q.nr, np = q.np;
  const int* rows = d.frontRows + q.rowOff;
  const T* L;
  if (l2Only) {
    const T* Lg = Lbase + q.lOff;
    const int cnt = nr * np;
    if (cnt > capL) {
      L = Lg;
    } else {
      for (int k = lane; k < cnt; k += 32) Ls[k] = __ldcg(Lg + k);
      L = Ls;
    }
  } else {
    L = stageL(Lbase + q.lOff, nr * np, Ls, capL, lane);
  }
  for (int r = lane; r < nr; r += 32) xs[r] = __ldcg(X + __ldg(rows + r));
  copyAsyncWait();
  __syncwarp();
  if (np <= 32) {
    // one pivot per lane in a register; the back substitution passes each
    // solved value by a shuffle (no barrier between steps)
    T a = T(0);
    if (lane < np) {
      a = xs[lane];
      for (int i = np; i < nr; ++i) a -= L[i + (size_t)nr * lane] * xs[i];
    }
    for (int j = np - 1; j > 0; --j) {
      const T xj = __shfl_sync(0xffffffffu, a, j);
      if (lane < j) a -= L[j + (size_t)nr * lane] * xj;
    }
    if (lane < np) xs[lane] = a;
    __syncwarp();
  } else {
    for (int k = lane; k < np; k += 32) {
      T a = xs[k];
      for (int i = np; i < nr; ++i) a -= L[i + (size_t)nr * k] * xs[i];
      xs[k] = a;
    }
    __syncwarp();
    for (int j = np - 1; j > 0; --j) {
      const T xj = xs[j];
      for (int k = lane; k < j; k += 32) xs[k] -= L[j + (size_t)nr * k] * xj;
      __syncwarp();
    }
  }
  for (int r = lane; r < np; r += 32) {
    const int row = rows[r];
    const T x = xs[r];
    X[row] = x;
    if (acc == ACC_SET) {
      d.del[row] = (double)x;
    } else {
      const double xr = acc == ACC_FIRST ? (double)x : d.xref[row] + (double)x;
      d.xref[row] = xr;
      if (finalize) d.del[row] = xr;
    }
  }
}

// Top-down work queue.  The step-start kernel puts the roots of the active
// models in the first queue slots and sets the slot total to their number of
// chains; a warp takes the next slot, waits until a front is stored there,
// solves it and goes on with its first child, storing the other children in
// fresh slots, until it reaches a leaf; a front whose children are all leaves
// (bwInline) has them solved by the same warp, one after the other, which ends
// the chain.  Every chain ends at a distinct leaf or such front, so the slots
// are exactly the chains of the active models: a warp whose slot number
// reaches the total is done.  A front is stored only after its parent is
// solved (fence, then the slot write; the taker fences after reading it).  A
// waiting warp holds no front, and every stored slot below the one it waits
// for is held by a running warp that solves without waiting, so each wait
// ends; it is still bounded and sets errFlag when it runs out.
// ctr: [0] next slot to take, [1] next free slot, [2] slot total.
// rootDone: the fused factorisation's counters (a root may still be in
// elimination in the same launch), or null when the roots are complete
template <typename T>
__device__ void backwardQueueLoop(const DevData& d, int maxRow, int capL, const T* Lbase, T* X, int* queue, int* ctr,
                                  const unsigned char* bwInline, int* errFlag, int acc, int finalize,
                                  long long spinLimit, T* xs, T* Ls, int lane, const int* rootDone) {
  const int total = *(volatile const int*)(ctr + 2);
  for (;;) {
    const int slot = __shfl_sync(0xffffffffu, lane == 0 ? atomicAdd(ctr, 1) : 0, 0);
    if (slot >= total) break;
    int f = -1, ok = 1;
    if (lane == 0) {
      long long spins = 0;
      while ((f = *(volatile const int*)(queue + slot)) < 0) {
        __nanosleep(32);
        if (++spins > spinLimit) {
          atomicOr(errFlag, 1);
          ok = 0;
          break;
        }
      }
      __threadfence();
      // a root of an active model: wait until its elimination is released
      if (ok && rootDone && d.fParent[f] < 0 && (d.m.flags[d.fModel[f]] & FL_ACTIVE)) {
        while (acquireCount(rootDone + f) < kRootDone) {
          __nanosleep(32);
          if (++spins > spinLimit) {
            atomicOr(errFlag, 1);
            ok = 0;
            break;
          }
        }
      }
    }
    f = __shfl_sync(0xffffffffu, f, 0);
    ok = __shfl_sync(0xffffffffu, ok, 0);
    __syncwarp();
    if (!ok) break;
    BackDesc q = backDesc(d, bwInline, f);
    while (f >= 0) {
      // the first child and its descriptors are loaded ahead of this front's solve
      const int* ch = d.childList + q.childOff;
      const int c0 = q.nch > 0 ? ch[0] : -1;
      const BackDesc cq = backDesc(d, bwInline, c0 >= 0 ? c0 : f);
      backwardOneFront<T>(d, q, xs, Ls, capL, Lbase, X, acc, finalize != 0, lane, rootDone != nullptr);
      __threadfence();
      __syncwarp();
      const int nch = q.nch;
      int next = -1;
      if (nch > 0) {
        if (q.inl) {
          // children that are all leaves: solved here, one after the other
          BackDesc lq = cq;
          for (int c = 0; c < nch; ++c) {
            const BackDesc nq = backDesc(d, bwInline, ch[c + 1 < nch ? c + 1 : c]);
            backwardOneFront<T>(d, lq, xs, Ls, capL, Lbase, X, acc, finalize != 0, lane, rootDone != nullptr);
            __syncwarp();
            lq = nq;
          }
        } else {
          next = c0;
          if (lane == 0 && nch > 1) {
            const int base = atomicAdd(ctr + 1, nch - 1);
            for (int k = 1; k < nch; ++k) atomicExch(queue + base + k - 1, ch[k]);
          }
        }
      }
      __syncwarp();
      f = next;
      q = cq;
    }
  }
}

template <typename T>
__global__ void kBackwardQueue(DevData d, int maxRow, int capL, const T* Lbase, T* X, int* queue, int* ctr,
                               const unsigned char* __restrict__ bwInline, int* errFlag, int acc, int finalize,
                               long long spinLimit) {
  pdlEntry();
  extern __shared__ __align__(16) unsigned char smraw[];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  T* xs = reinterpret_cast<T*>(smraw) + (size_t)w * (maxRow + capL);
  T* Ls = xs + maxRow;
  backwardQueueLoop<T>(d, maxRow, capL, Lbase, X, queue, ctr, bwInline, errFlag, acc, finalize, spinLimit, xs, Ls,
                       lane, nullptr);
}

int smCountCached() {
  // engines may be built on several host threads at once
  static std::atomic<int> cached{0};
  int n = cached.load(std::memory_order_relaxed);
  if (n == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 1;
    cached.store(n, std::memory_order_relaxed);
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

// one launch of a factor cascade kernel (either panel variant)
template <typename T>
void factorCascade(void (*kernel)(DevData, const int*, int, int, const T*, T*, T*, double, const double*, T*, T*,
                                  int*, FusedBackward),
                   int wpb, size_t sm, const DevData& d, const PersistentPlan& p, const T* asmVal, T* L, T* U,
                   double tol, const double* rhs, T* X, T* W, const FusedBackward& fb, cudaStream_t s) {
  allowBigSmem(kernel, sm);
  const int blocks = occupancyBlocks(kernel, 32 * wpb, sm, (p.nLeaves + wpb - 1) / wpb);
  pdlLaunch(kernel, blocks, 32 * wpb, sm, s, d, p.leaves, p.nLeaves, p.maxRow, asmVal, L, U, tol, rhs, X, W, p.cntFactor,
            fb);
}

int factorWarpsPerBlock(size_t perWarpBytes) {
  int w = (int)(96 * 1024 / (perWarpBytes > 0 ? perWarpBytes : 1));
  return w > 8 ? 8 : (w < 1 ? 1 : w);
}

// Synthetic original entries for the autotuner's timing probe: a dominant
// diagonal and small off-diagonal values of alternating sign (pivots stay
// positive and far from singular, like a Newton matrix's), one thread per front.
template <typename T>
__global__ void kProbeEntries(DevData d, T* asmVal) {
  pdlEntry();
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= d.nfrontTot) return;
  const int nr = d.fNrow[f], na = d.fNasm[f];
  const int64_t ao = d.fAsmOff[f];
  for (int k = 0; k < na; ++k) {
    const int pos = d.asmPos[ao + k];
    const int i = pos % nr, j = pos / nr;
    asmVal[ao + k] = i == j ? T(4 + nr) : (((i + j) & 1) ? T(0.01) : T(-0.01));
  }
}

}  // namespace

void launchProbeEntries(const DevData& d, bool fp32, cudaStream_t s) {
  if (d.nfrontTot <= 0) return;
  const int blocks = (d.nfrontTot + 127) / 128;
  if (fp32) pdlLaunch(kProbeEntries<float>, blocks, 128, 0, s, d, d.asmVal32);
  else pdlLaunch(kProbeEntries<double>, blocks, 128, 0, s, d, d.asmVal64);
}

void launchFactorForwardCascade(const DevData& d, const PersistentPlan& p, bool fp32, const double* rhs,
                                cudaStream_t s, bool withBackward, bool lastSweep) {
  if (p.nLeaves <= 0) return;
  const double tol = 1.0e-12;
  const size_t perWarp = (size_t)p.maxRow * p.maxRow + 3 * p.maxRow;
  // the fused back substitution of solve 0 (launchBackward's arguments); its
  // solve vector and L staging reuse the warp's v and F areas
  FusedBackward fb;
  if (withBackward) {
    fb.queue = p.bwQueue;
    fb.ctr = p.bwCtr;
    fb.bwInline = p.bwInline;
    fb.errFlag = p.errFlag;
    fb.spinLimit = p.spinLimit;
    fb.acc = fp32 ? ACC_FIRST : ACC_SET;
    fb.finalize = (fp32 && lastSweep) ? 1 : 0;
    fb.capL = stagingCapacity(p, fp32 ? sizeof(float) : sizeof(double));
  }
  if (fp32) {
    const int wpb = factorWarpsPerBlock(perWarp * sizeof(float));
    const size_t sm = (size_t)wpb * perWarp * sizeof(float);
    if (p.factorPanel == kPanelRegisters)
      factorCascade(kFactorForwardCascade<float, kPanelRegisters>, wpb, sm, d, p, d.asmVal32, d.L32, d.U32, tol, rhs,
                    d.x32, d.w32, fb, s);
    else if (p.factorPanel == kPanelRegisters4)
      factorCascade(kFactorForwardCascade<float, kPanelRegisters4>, wpb, sm, d, p, d.asmVal32, d.L32, d.U32, tol,
                    rhs, d.x32, d.w32, fb, s);
    else
      factorCascade(kFactorForwardCascade<float, kPanelShuffle>, wpb, sm, d, p, d.asmVal32, d.L32, d.U32, tol, rhs,
                    d.x32, d.w32, fb, s);
  } else {
    const int wpb = factorWarpsPerBlock(perWarp * sizeof(double));
    const size_t sm = (size_t)wpb * perWarp * sizeof(double);
    if (p.factorPanel == kPanelRegisters)
      factorCascade(kFactorForwardCascade<double, kPanelRegisters>, wpb, sm, d, p, d.asmVal64, d.L64, d.U64, tol,
                    rhs, d.x64, d.w64, fb, s);
    else if (p.factorPanel == kPanelRegisters4)
      factorCascade(kFactorForwardCascade<double, kPanelRegisters4>, wpb, sm, d, p, d.asmVal64, d.L64, d.U64, tol,
                    rhs, d.x64, d.w64, fb, s);
    else
      factorCascade(kFactorForwardCascade<double, kPanelShuffle>, wpb, sm, d, p, d.asmVal64, d.L64, d.U64, tol, rhs,
                    d.x64, d.w64, fb, s);
  }
}

// staging capacity (values) of one front's L block per warp
int stagingCapacity(const PersistentPlan& p, size_t elemBytes) {
  long long want = (long long)p.maxRow * p.maxNpiv;
  long long cap = (long long)(12 * 1024 / elemBytes);
  return (int)(want < cap ? want : cap);
}

bool fusableBackward(const PersistentPlan& p, bool fp32) {
  return p.nLeaves > 0 && p.nLargeTasks == 0 &&
         (long long)stagingCapacity(p, fp32 ? sizeof(float) : sizeof(double)) >= (long long)p.maxRow * p.maxNpiv;
}

void launchForwardCascade(const DevData& d, const PersistentPlan& p, bool fp32, const double* rhs, int sweep,
                          cudaStream_t s) {
  if (p.nTasks <= 0) return;
  const int wpb = p.forwardWarps;
  int* cnt = p.cntForward + (size_t)(sweep - 1) * ((size_t)d.nfrontTot + 1);
  if (fp32) {
    const int capL = stagingCapacity(p, sizeof(float));
    const size_t sm = (size_t)wpb * (p.maxRow + capL + 64) * sizeof(float);
    allowBigSmem(kForwardCascade<float>, sm);
    const int blocks = occupancyBlocks(kForwardCascade<float>, 32 * wpb, sm, (p.nTasks + wpb - 1) / wpb);
    pdlLaunch(kForwardCascade<float>, blocks, 32 * wpb, sm, s, d, p.tasks, p.nTasks, p.maxRow, capL, d.L32, rhs, d.x32,
                                                       d.w32, cnt);
  } else {
    const int capL = stagingCapacity(p, sizeof(double));
    const size_t sm = (size_t)wpb * (p.maxRow + capL + 64) * sizeof(double);
    allowBigSmem(kForwardCascade<double>, sm);
    const int blocks = occupancyBlocks(kForwardCascade<double>, 32 * wpb, sm, (p.nTasks + wpb - 1) / wpb);
    pdlLaunch(kForwardCascade<double>, blocks, 32 * wpb, sm, s, d, p.tasks, p.nTasks, p.maxRow, capL, d.L64, rhs, d.x64,
                                                         d.w64, cnt);
  }
}

void launchBackward(const DevData& d, const PersistentPlan& p, bool fp32, int sweep, bool last, cudaStream_t s) {
  const int acc = !fp32 ? ACC_SET : (sweep == 0 ? ACC_FIRST : ACC_ADD);
  const int fin = (fp32 && last) ? 1 : 0;
  if (p.nLeaves <= 0) return;
  const int wpb = p.backwardWarps;
  int* queue = p.bwQueue + (size_t)sweep * p.nLeaves;
  int* ctr = p.bwCtr + 4 * sweep;
  const int needed = (p.nLeaves + wpb - 1) / wpb;
  if (fp32) {
    const int capL = stagingCapacity(p, sizeof(float));
    const size_t sm = (size_t)wpb * (p.maxRow + capL) * sizeof(float);
    allowBigSmem(kBackwardQueue<float>, sm);
    const int blocks = occupancyBlocks(kBackwardQueue<float>, 32 * wpb, sm, needed);
    pdlLaunch(kBackwardQueue<float>, blocks, 32 * wpb, sm, s, d, p.maxRow, capL, d.L32, d.x32, queue, ctr, p.bwInline,
                                                      p.errFlag, acc, fin, p.spinLimit);
  } else {
    const int capL = stagingCapacity(p, sizeof(double));
    const size_t sm = (size_t)wpb * (p.maxRow + capL) * sizeof(double);
    allowBigSmem(kBackwardQueue<double>, sm);
    const int blocks = occupancyBlocks(kBackwardQueue<double>, 32 * wpb, sm, needed);
    pdlLaunch(kBackwardQueue<double>, blocks, 32 * wpb, sm, s, d, p.maxRow, capL, d.L64, d.x64, queue, ctr, p.bwInline,
                                                        p.errFlag, acc, fin, p.spinLimit);
  }
}

void launchBackwardWaitProbe(const DevData& d, const PersistentPlan& p, int* queue, int* ctr, long long spins,
                             cudaStream_t s) {
  // one warp; it waits on slot 0 and touches no front (the wait gives up first)
  const int capL = stagingCapacity(p, sizeof(double));
  const size_t sm = (size_t)(p.maxRow + capL) * sizeof(double);
  allowBigSmem(kBackwardQueue<double>, sm);
  pdlLaunch(kBackwardQueue<double>, 1, 32, sm, s, d, p.maxRow, capL, d.L64, d.x64, queue, ctr, p.bwInline, p.errFlag,
                                           ACC_SET, 0, spins);
}

void launchRootWaitProbe(const DevData& d, const PersistentPlan& p, int* queue, int* ctr, int* cnt, long long spins,
                         cudaStream_t s) {
  // one warp of the fused factorisation with no leaf: it goes straight to the
  // back substitution, takes slot 0 (a root) and waits for a release that no
  // elimination makes (cnt is zero); the wait gives up before any front is touched
  const size_t perWarp = (size_t)p.maxRow * p.maxRow + 3 * p.maxRow;
  const size_t sm = perWarp * sizeof(double);
  FusedBackward fb;
  fb.queue = queue;
  fb.ctr = ctr;
  fb.bwInline = p.bwInline;
  fb.errFlag = p.errFlag;
  fb.spinLimit = spins;
  fb.acc = ACC_SET;
  fb.capL = stagingCapacity(p, sizeof(double));
  allowBigSmem(kFactorForwardCascade<double, kPanelShuffle>, sm);
  pdlLaunch(kFactorForwardCascade<double, kPanelShuffle>, 1, 32, sm, s, d, p.leaves, 0, p.maxRow,
            (const double*)d.asmVal64, d.L64, d.U64, 1.0e-12, (const double*)d.del, d.x64, d.w64, cnt, fb);
}

}  // namespace fgpu
