// front_large.cu -- multifrontal factorisation and solves of the large fronts
// (more rows than one warp's shared-memory front holds).
//
// Large fronts are marked upward-closed on the host (every ancestor of a large
// front is large), so the warp kernels of front_cascade.cu finish every small
// subtree first and these kernels take the tops of the assembly trees:
//   factor + forward: a cascade over the large fronts (clusters of blocks start
//     at large fronts whose children are all small, a parent's counter
//     completes on its last large child, the completing cluster climbs to it;
//     nothing waits on another cluster);
//   forward (refinement sweeps): the same cascade without the factorisation,
//     one block per front;
//   backward: a top-down work queue of large fronts seeded with the large roots
//     (a block waits only for a slot that a running block fills), before the
//     warp queue takes the small fronts below them.
// A large front is factored in place in its outputs: its pivot columns in its
// L block (nrow x npiv, column-major) and its trailing lower triangle in its
// packed update matrix (column by column, inside the parent's segment), so no
// workspace is needed.  Blocked right-looking LDL^T in panels of up to 32
// pivots: each panel is factored in shared memory (its diagonal block by one
// warp, the rows below it one per thread, no barrier inside), then the
// trailing lower triangle is updated with it, C -= L_p D_p L_p^T, in 64 x 64
// tiles (FP32 fronts: mma.sync TF32 products on the tensor cores in the 3xTF32
// split; FP64 fronts: 4 x 4 register blocks), the tiles shared out over the blocks of a
// thread-block cluster (GB300's FP64 units are thin: one front's update on one
// SM would set the pace).  Semantics as the warp kernels and the reference's
// SPRFC1/SPRFS1/SPRBS1 seam (solExtensionModule.f90:153-505): no pivoting, a
// pivot is singular when |d_k| <= tolFactorize |a_kk|, negative pivots counted,
// children's update matrices added in child order (fixed summation order).
// Front data written by other threads or blocks are read through L2 (__ldcg).

#include <cooperative_groups.h>

#include <algorithm>
#include <type_traits>

#include <atomic>

#include "kernels.h"

namespace fgpu {
namespace {

namespace cg = cooperative_groups;

constexpr int kLT = 256;         // threads per large-front block
constexpr int kTile = 64;        // trailing-update tile (rows and columns)

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

// a barrier of all threads of the cluster, their global writes visible to
// every thread of the cluster afterwards (each thread fences first)
__device__ inline void clusterBarrier() {
  __threadfence();
  cg::this_cluster().sync();
}

// ---- FP32 trailing tiles on the tensor cores --------------------------------
// C(64 x 64 tile) -= A B with A(m, k) = P(r0 + m, k) and B(k, n) = P(c0 + n, k) d_k
// (k < kb <= 32, zero beyond kb), as mma.sync m16n8k8 TF32 products with FP32
// accumulation in the 3xTF32 split (x = hi + lo, both TF32; a b = hi hi + hi lo
// + lo hi), which keeps the FP32 accuracy of the update.  Warp w takes rows
// 16 (w & 3) .. +15 and columns 32 (w >> 2) .. +31 of the tile (four 16 x 8
// products); fragment layouts of m16n8k8.row.col: lane = 4 g + t holds
// A(g, t), A(g + 8, t), A(g, t + 4), A(g + 8, t + 4); B(t, g), B(t + 4, g);
// C(g, 2t), C(g, 2t + 1), C(g + 8, 2t), C(g + 8, 2t + 1).
__device__ inline uint32_t tf32Of(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

__device__ inline void split3(float x, uint32_t& hi, uint32_t& lo) {
  hi = tf32Of(x);
  lo = tf32Of(x - __uint_as_float(hi));
}

__device__ inline void mmaTf32(float* c, const uint32_t* a, const uint32_t* b) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
      "{%0, %1, %2, %3};"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// acc[j][q]: this thread's C fragment of the warp's j-th 16 x 8 product
__device__ inline void tileUpdateMma(const float* P, int ldp, const float* dpan, int kb, int pr, int r0, int c0,
                                     float acc[4][4]) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int g = lane >> 2, t = lane & 3;
  const int rb = r0 + 16 * (w & 3), cb = c0 + 32 * (w >> 2);
#pragma unroll
  for (int j = 0; j < 4; ++j)
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[j][q] = 0.0f;
  for (int k0 = 0; k0 < kb; k0 += 8) {
    const int ka = k0 + t, kc = k0 + t + 4;
    auto av = [&](int r, int k) { return (r < pr && k < kb) ? P[k * ldp + r] : 0.0f; };
    uint32_t ah[4], al[4];
    split3(av(rb + g, ka), ah[0], al[0]);
    split3(av(rb + g + 8, ka), ah[1], al[1]);
    split3(av(rb + g, kc), ah[2], al[2]);
    split3(av(rb + g + 8, kc), ah[3], al[3]);
    const float da = ka < kb ? dpan[ka] : 0.0f, dc = kc < kb ? dpan[kc] : 0.0f;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int c = cb + 8 * j + g;
      uint32_t bh[2], bl[2];
      split3(av(c, ka) * da, bh[0], bl[0]);
      split3(av(c, kc) * dc, bh[1], bl[1]);
      mmaTf32(acc[j], al, bh);
      mmaTf32(acc[j], ah, bl);
      mmaTf32(acc[j], ah, bh);
    }
  }
}

// Assembly (original entries, then the children's update matrices in child
// order) and the blocked partial LDL^T of large front f by the blocks of a
// cluster (crank of csize): the assembly is split over all their threads,
// every block factors each panel itself (the same arithmetic, so the same
// values) and takes its share of the trailing tiles; block 0 writes the panel
// back and reports the pivots.  Shared memory: the panel P (kb <= 32 columns of
// ldp rows, column-major: the panel's rows k0 .. nr-1), diag0 (np), dpan (kb).
template <typename T>
__device__ void factorLarge(const DevData& d, int f, const T* asmVal, T* Lbase, T* Ubase, double tolFact, T* P,
                            int ldp, int kbMax, T* diag0, T* dpan, int crank, int csize) {
  const int tid = threadIdx.x;
  const int gtid = crank * kLT + tid, gstride = csize * kLT;
  Front<T> F{Lbase + d.fLOff[f], Ubase + d.fUOff[f], d.fNrow[f], d.fNpiv[f], d.fNrow[f] - d.fNpiv[f]};
  const int nr = F.nr, np = F.np, nu = F.nu;
  const int64_t nL = (int64_t)nr * np, nU = (int64_t)nu * (nu + 1) / 2;
  clusterBarrier();
  for (int64_t k = gtid; k < nL; k += gstride) st(F.L + k, T(0));
  for (int64_t k = gtid; k < nU; k += gstride) st(F.U + k, T(0));
  clusterBarrier();
  const int64_t ao = d.fAsmOff[f];
  const int na = d.fNasm[f];
  for (int k = gtid; k < na; k += gstride) {  // original entries: pivot columns only, distinct positions
    const int p = __ldg(d.asmPos + ao + k);
    st(F.L + p, __ldg(asmVal + ao + k));
  }
  clusterBarrier();
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
    if (c > 0) clusterBarrier();
    // four entries per thread at a time, every load issued before the stores
    // (positions are distinct within one child)
    for (int64_t k0 = gtid; k0 < len; k0 += 4 * (int64_t)gstride) {
      T* q[4];
      T sv[4], cur[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int64_t k = k0 + (int64_t)u * gstride;
        const int p = k < len ? (__ldg(spos + off + k) & 0xfffff) : -1;
        q[u] = p >= 0 ? F.at(p % nr, p / nr) : nullptr;
        sv[u] = p >= 0 ? ld(seg + off + k) : T(0);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) cur[u] = q[u] ? ld(q[u]) : T(0);
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (q[u]) st(q[u], cur[u] + sv[u]);
    }
    off += len;
  }
  int neg = 0;
  bool sing = false;
  for (int k0 = 0; k0 < np; k0 += kbMax) {
    clusterBarrier();  // the panel's columns complete (assembly, earlier trailing updates)
    const int kb = min(kbMax, np - k0), pr = nr - k0;  // panel columns and rows
    for (int kk = 0; kk < kb; ++kk)
      for (int r = tid; r < pr; r += kLT) P[kk * ldp + r] = ld(F.L + (k0 + r) + (int64_t)nr * (k0 + kk));
    __syncthreads();
    // the panel's kb x kb diagonal block, right-looking, by warp 0 alone: lane
    // r owns row r; the unscaled value of each scaled entry (row r, column k) is
    // kept in the unused upper triangle (row k, column r)
    if (tid < 32) {
      const int r = tid;
      for (int kk = 0; kk < kb; ++kk) {
        const T dk = P[kk * ldp + kk];
        const bool bad = singularPivot(dk, diag0[k0 + kk], tolFact);
        if (r == 0) {
          sing |= bad;
          if (dk < T(0)) ++neg;
          dpan[kk] = dk;
        }
        const T inv = bad ? T(0) : T(1) / dk;
        T l = T(0);
        if (r > kk && r < kb) {
          const T u = P[kk * ldp + r];
          P[r * ldp + kk] = u;
          l = u * inv;
          P[kk * ldp + r] = l;
        }
        __syncwarp();
        if (r > kk && r < kb)
          for (int j = kk + 1; j <= r; ++j) P[j * ldp + r] -= l * P[j * ldp + kk];
        __syncwarp();
      }
    }
    __syncthreads();
    // the panel's rows below the block, each on its own: for k in order,
    // a = P(r, k) - sum_{j < k} l_rj u_kj, l_rk = a / d_k (the right-looking
    // updates of the row, in the same order)
    for (int r = kb + tid; r < pr; r += kLT) {
      T lr[32];
#pragma unroll
      for (int kk = 0; kk < 32; ++kk) {
        if (kk >= kb) break;
        T a = P[kk * ldp + r];
#pragma unroll
        for (int j = 0; j < kk; ++j) a -= lr[j] * P[kk * ldp + j];
        const bool bad = singularPivot(dpan[kk], diag0[k0 + kk], tolFact);
        lr[kk] = a * (bad ? T(0) : T(1) / dpan[kk]);
      }
#pragma unroll
      for (int kk = 0; kk < 32; ++kk) {
        if (kk >= kb) break;
        P[kk * ldp + r] = lr[kk];
      }
    }
    __syncthreads();
    if (crank == 0)
      for (int kk = 0; kk < kb; ++kk)
        for (int r = kk + tid; r < pr; r += kLT) st(F.L + (k0 + r) + (int64_t)nr * (k0 + kk), P[kk * ldp + r]);
    // trailing lower triangle, rows and columns k0 + kb .. nr-1 (panel-local
    // kb .. pr-1): C(i, j) -= sum_k P(i, k) d_k P(j, k), tile by tile; a
    // thread's 4 x 4 block is rows lr + 16 a and columns lc + 16 b of the tile
    const int nt = pr - kb;
    const int ntiles = (nt + kTile - 1) / kTile;
    const int lr = tid & 15, lc = tid >> 4;
    int tcount = 0;
    for (int tj = 0; tj < ntiles; ++tj)
      for (int ti = tj; ti < ntiles; ++ti) {
        if (tcount++ % csize != crank) continue;  // this block's share of the tiles
        const int r0 = kb + ti * kTile, c0 = kb + tj * kTile;
        if constexpr (std::is_same<T, float>::value) {
          // FP32 fronts: the tile's product on the tensor cores (3xTF32)
          float acc[4][4];
          tileUpdateMma(P, ldp, dpan, kb, pr, r0, c0, acc);
          const int lane = tid & 31, w = tid >> 5, g = lane >> 2, t = lane & 3;
          // the tile's sixteen entries of this thread: every load before the stores
          T* dst[4][4];
          T cur[4][4];
#pragma unroll
          for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              const int r = r0 + 16 * (w & 3) + g + 8 * (q >> 1), c = c0 + 32 * (w >> 2) + 8 * j + 2 * t + (q & 1);
              dst[j][q] = (r < pr && c < pr && r >= c) ? F.at(k0 + r, k0 + c) : nullptr;
              cur[j][q] = dst[j][q] ? ld(dst[j][q]) : T(0);
            }
#pragma unroll
          for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int q = 0; q < 4; ++q)
              if (dst[j][q]) st(dst[j][q], cur[j][q] - acc[j][q]);
        } else {
          // FP64 fronts: 4 x 4 register blocks on the FP64 units
          T acc[4][4];
#pragma unroll
          for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b) acc[a][b] = T(0);
          for (int kk = 0; kk < kb; ++kk) {
            const T* Pk = P + kk * ldp;
            const T dk = dpan[kk];
            T av[4], bv[4];
#pragma unroll
            for (int a = 0; a < 4; ++a) {
              const int r = r0 + lr + 16 * a;
              av[a] = r < pr ? Pk[r] : T(0);
            }
#pragma unroll
            for (int b = 0; b < 4; ++b) {
              const int c = c0 + lc + 16 * b;
              bv[b] = c < pr ? Pk[c] * dk : T(0);
            }
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
              for (int b = 0; b < 4; ++b) acc[a][b] += av[a] * bv[b];
          }
          T* dst[4][4];
          T cur[4][4];
#pragma unroll
          for (int b = 0; b < 4; ++b) {
            const int c = c0 + lc + 16 * b;
#pragma unroll
            for (int a = 0; a < 4; ++a) {
              const int r = r0 + lr + 16 * a;
              dst[a][b] = (r < pr && c < pr && r >= c) ? F.at(k0 + r, k0 + c) : nullptr;
              cur[a][b] = dst[a][b] ? ld(dst[a][b]) : T(0);
            }
          }
#pragma unroll
          for (int b = 0; b < 4; ++b)
#pragma unroll
            for (int a = 0; a < 4; ++a)
              if (dst[a][b]) st(dst[a][b], cur[a][b] - acc[a][b]);
        }
      }
  }
  if (tid == 0 && crank == 0) {
    const int m = d.fModel[f];
    if (neg) atomicAdd(&d.m.negPiv[m], neg);
    if (sing) atomicOr(&d.m.status[m], SS_SINGULAR);
  }
  clusterBarrier();  // L block and update matrix complete
}

// forward elimination of large front f (v: nr values in shared memory), in
// blocks of 32 pivots: warp 0 eliminates the block's unit lower triangle with
// shuffles, then every thread updates its rows below the block with it
template <typename T>
__device__ void forwardLarge(const DevData& d, int f, const T* Lbase, const double* rhs, T* X, T* W, T* v,
                             T* Ltri) {
  const int tid = threadIdx.x, lane = tid & 31;
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
  for (int b0 = 0; b0 < np; b0 += 32) {
    const int bs = min(32, np - b0);
    if (tid < 32) {  // the block's triangle: lane r holds v[b0 + r]
      // the triangle is staged in shared memory first (eight independent loads
      // at a time), so that no step of the dependent chain below waits on a load
      for (int k0 = 0; k0 < bs - 1; k0 += 8) {
        T t[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int k = k0 + u;
          t[u] = (k < bs - 1 && lane > k && lane < bs) ? ld(L + (b0 + lane) + (int64_t)nr * (b0 + k)) : T(0);
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) Ltri[(k0 + u) * 32 + lane] = t[u];
      }
      __syncwarp();
      T x = lane < bs ? v[b0 + lane] : T(0);
      for (int k = 0; k < bs - 1; ++k) {
        const T yk = __shfl_sync(0xffffffffu, x, k);
        if (lane > k && lane < bs) x -= Ltri[k * 32 + lane] * yk;
      }
      if (lane < bs) v[b0 + lane] = x;
    }
    __syncthreads();
    for (int i = b0 + bs + tid; i < nr; i += kLT) {
      T s = v[i];
      for (int k0 = 0; k0 < bs; k0 += 8) {  // eight loads in flight, then the ordered updates
        T t[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) t[u] = k0 + u < bs ? ld(L + i + (int64_t)nr * (b0 + k0 + u)) : T(0);
#pragma unroll
        for (int u = 0; u < 8; ++u)
          if (k0 + u < bs) s -= t[u] * v[b0 + k0 + u];
      }
      v[i] = s;
    }
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
                                                            int* cnt, int doFactor, int panel) {
  pdlEntry();
  extern __shared__ __align__(16) unsigned char smraw[];
  const int ldp = (p.maxRowLarge + 3) & ~3;
  T* v = reinterpret_cast<T*>(smraw);
  T* diag0 = v + ldp;
  T* dpan = diag0 + ldp;
  T* Ltri = dpan + 32;  // 32 x 32 staging of a forward elimination's triangle
  T* P = Ltri + 32 * 32;
  __shared__ int shIdx, shNext;
  cg::cluster_group cluster = cg::this_cluster();
  const int crank = (int)cluster.block_rank(), csize = (int)cluster.num_blocks();
  int* const next = cnt + d.nfrontTot;
  for (;;) {
    // block 0 of the cluster takes the task; every block reads it from there
    if (crank == 0 && threadIdx.x == 0) shIdx = atomicAdd(next, 1);
    cluster.sync();
    const int idx = *cluster.map_shared_rank(&shIdx, 0);
    cluster.sync();
    if (idx >= p.nLargeTasks) break;
    int f = p.largeTasks[idx];
    const int fl = d.m.flags[d.fModel[f]];
    const bool factor = doFactor && (fl & FL_TANGENT);
    while ((fl & FL_ACTIVE) && f >= 0) {
      if (factor) factorLarge<T>(d, f, asmVal, Lbase, Ubase, tolFact, P, ldp, panel, diag0, dpan, crank, csize);
      if (crank == 0) {
        forwardLarge<T>(d, f, Lbase, rhs, X, W, v, Ltri);
        f = climbLarge(d, p, f, cnt, &shNext);
      }
      cluster.sync();
      f = *cluster.map_shared_rank(&shNext, 0);
      cluster.sync();
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
  pdlEntry();
  extern __shared__ __align__(16) unsigned char smraw[];
  T* xs = reinterpret_cast<T*>(smraw);
  T* Ltri = xs + ((p.maxRowLarge + 3) & ~3);  // 32 x 32 staging of a block's triangle
  __shared__ int shSlot, shF, shOk;
  const int tid = threadIdx.x;
  const int w = tid >> 5, lane = tid & 31;
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
      // the update rows' contribution for every pivot: one warp per pivot, the
      // lanes over the rows in a fixed pattern, a fixed shuffle tree
      for (int k = w; k < np; k += kLT / 32) {
        T a = T(0);
        for (int i = np + lane; i < nr; i += 32) a += ld(L + i + (int64_t)nr * k) * xs[i];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
        if (lane == 0) xs[k] -= a;
      }
      __syncthreads();
      // the unit upper triangle L11^T, blocks of 32 pivots from the last: warp
      // 0 solves the block with shuffles, then the pivots above it are updated
      // with the block's values (one warp per pivot)
      for (int bEnd = np; bEnd > 0; bEnd -= 32) {
        const int b0 = bEnd > 32 ? bEnd - 32 : 0, bs = bEnd - b0;
        if (tid < 32) {
          // lane r's column of the triangle staged first (rows j > r), eight
          // independent loads at a time
          for (int j0 = 0; j0 < bs; j0 += 8) {
            T t[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
              const int j = j0 + u;
              t[u] = (j < bs && lane < j) ? ld(L + (b0 + j) + (int64_t)nr * (b0 + lane)) : T(0);
            }
#pragma unroll
            for (int u = 0; u < 8; ++u) Ltri[(j0 + u) * 32 + lane] = t[u];
          }
          __syncwarp();
          T x = lane < bs ? xs[b0 + lane] : T(0);
          for (int j = bs - 1; j > 0; --j) {
            const T xj = __shfl_sync(0xffffffffu, x, j);
            if (lane < j) x -= Ltri[j * 32 + lane] * xj;
          }
          if (lane < bs) xs[b0 + lane] = x;
        }
        __syncthreads();
        for (int k = w; k < b0; k += kLT / 32) {
          T a = lane < bs ? ld(L + (b0 + lane) + (int64_t)nr * k) * xs[b0 + lane] : T(0);
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
          if (lane == 0) xs[k] -= a;
        }
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
      if (tid == 0) {
        int first = -1, nl = 0;
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

// panel width: 32 pivots, fewer when the panel of the largest front would not
// fit the shared memory (about 200 KB)
template <typename T>
int panelWidth(int maxRow) {
  const size_t ldp = (size_t)((maxRow + 3) & ~3);
  int kb = 32;
  while (kb > 4 && (2 * ldp + 32 + 32 * 32 + (size_t)kb * ldp) * sizeof(T) > 200 * 1024) kb -= 4;
  return kb;
}

// clusters of csize blocks the device can hold at once with the factorisation's
// shared memory (0: none; sizes above 8 need the non-portable cluster opt-in)
template <typename T>
int largeClusterCapacity(const PersistentPlan& p, int csize) {
  const size_t ldp = (size_t)((p.maxRowLarge + 3) & ~3);
  const int kb = panelWidth<T>(p.maxRowLarge);
  const size_t sm = (2 * ldp + 32 + 32 * 32 + (size_t)kb * ldp) * sizeof(T);
  bigSmem(kLargeFactorForward<T>, sm);
  if (csize > 8 && cudaFuncSetAttribute(kLargeFactorForward<T>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
                       cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = csize;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.blockDim = dim3(kLT);
  cfg.dynamicSmemBytes = sm;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cfg.gridDim = dim3(csize);
  int clusters = 0;
  if (cudaOccupancyMaxActiveClusters(&clusters, kLargeFactorForward<T>, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return clusters;
}

// Factorisations run as clusters of p.largeCluster blocks per front (a grid of
// as many clusters as fit at once, at most one per start task); forward
// eliminations alone as single blocks.
template <typename T>
void factorForwardLarge(const DevData& d, const PersistentPlan& p, const T* asmVal, T* L, T* U, const double* rhs,
                        T* X, T* W, int* cnt, bool factor, cudaStream_t s) {
  const size_t ldp = (size_t)((p.maxRowLarge + 3) & ~3);
  const int kb = panelWidth<T>(p.maxRowLarge);
  const size_t sm = (2 * ldp + 32 + 32 * 32 + (factor ? (size_t)kb * ldp : 0)) * sizeof(T);
  bigSmem(kLargeFactorForward<T>, sm);
  if (!factor) {
    const int grid = gridFor(kLargeFactorForward<T>, sm, p.nLargeTasks);
    pdlLaunch(kLargeFactorForward<T>, grid, kLT, sm, s, d, p, asmVal, L, U, 1.0e-12, rhs, X, W, cnt, 0, kb);
    return;
  }
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[2];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  int csize = p.largeCluster;
  // 16 blocks per cluster is beyond the portable size: allowed per kernel, and
  // only taken when the device can hold such a cluster with this shared memory
  if (csize > 8 && largeClusterCapacity<T>(p, csize) < 1) csize = 8;
  attr[0].val.clusterDim.x = csize;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[1].val.programmaticStreamSerializationAllowed = 1;
  cfg.blockDim = dim3(kLT);
  cfg.dynamicSmemBytes = sm;
  cfg.stream = s;
  cfg.attrs = attr;
  cfg.numAttrs = 2;
  cfg.gridDim = dim3(csize * p.nLargeTasks);
  int clusters = 0;
  if (cudaOccupancyMaxActiveClusters(&clusters, kLargeFactorForward<T>, &cfg) != cudaSuccess || clusters < 1)
    clusters = 1;
  clusters = std::min(clusters, p.nLargeTasks);
  cfg.gridDim = dim3(csize * clusters);
  cudaLaunchKernelEx(&cfg, kLargeFactorForward<T>, d, p, asmVal, L, U, 1.0e-12, rhs, X, W, cnt, 1, kb);
}

}  // namespace

int largeClusterCapacity(const PersistentPlan& p, bool fp32, int csize) {
  if (p.nLargeTasks <= 0) return 0;
  return fp32 ? largeClusterCapacity<float>(p, csize) : largeClusterCapacity<double>(p, csize);
}

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
    const size_t sm = ((size_t)((p.maxRowLarge + 3) & ~3) + 32 * 32) * sizeof(float);
    bigSmem(kLargeBackward<float>, sm);
    const int grid = gridFor(kLargeBackward<float>, sm, p.nLargeTasks);
    pdlLaunch(kLargeBackward<float>, grid, kLT, sm, s, d, p, d.L32, d.x32, queue, ctr, p.errFlag, acc, fin);
  } else {
    const size_t sm = ((size_t)((p.maxRowLarge + 3) & ~3) + 32 * 32) * sizeof(double);
    bigSmem(kLargeBackward<double>, sm);
    const int grid = gridFor(kLargeBackward<double>, sm, p.nLargeTasks);
    pdlLaunch(kLargeBackward<double>, grid, kLT, sm, s, d, p, d.L64, d.x64, queue, ctr, p.errFlag, acc, fin);
  }
}

}  // namespace fgpu
