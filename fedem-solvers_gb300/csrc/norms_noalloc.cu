// norms_noalloc.cu -- convergence norms of one model of a batch, computed
// again on the device without allocating any memory.
//
// Who needs it: callers that may not allocate device memory at the moment they
// ask for the norms -- a co-simulation or control loop that checks convergence
// between its own stream-ordered kernels (cudaMalloc/cudaFree synchronise the
// whole device and would stall that loop), or a process whose device memory is
// already committed to resident batches and served engines.  The batch's own
// norms pass reduces into a buffer allocated with the batch; this variant of
// that pass reduces into a fixed scratch array compiled into the library.
//
// Limits and rules:
//  * the scratch holds kMaxChunks chunks of 2048 DOFs: models with more than
//    kMaxChunks * 2048 = 524,288 DOFs are refused with an error message;
//  * the first call on each device does the set-up (makes the batch's device
//    current and looks up the scratch address with cudaGetSymbolAddress):
//    make it before any stream capture begins on that device;
//  * the completion counter at the head of the scratch must start at zero: each
//    call clears it on the batch's stream before its launch, and nothing else
//    of the scratch is read before the same call has written it;
//  * there is one scratch per device, so calls that overlap in time on one
//    device (from several host threads) race on it: serialise them.
//
// The arithmetic is the batch's two-stage norms pass (kNormsPartial + kControl
// in element_kernels.cu): the same chunk boundaries, thread-to-DOF mapping,
// expressions, warp tree and chunk order, maxima compared as |x| bit patterns
// (a NaN shows as it does there) and the model's constant weight sums, so the
// 18 values equal what the batch stored for the same vectors.  The launch runs
// on the batch's device (made current first).  Norm definitions:
// src/vpmSolver/normTypeModule.f90:196-249.

#include <cstdint>
#include <mutex>
#include <string>

#include "kernels.h"

namespace fgpu {
namespace {

constexpr int kTpb = 256;        // threads per chunk block (as the batch's pass)
constexpr int kParts = 20;       // partial values per chunk (see kNormsOneModel)
constexpr int kMaxChunks = 256;  // 256 chunks x 2048 DOFs = 524,288 DOFs
constexpr int kMaxDevices = 64;
constexpr size_t kHeadBytes = 256;             // completion counter (must start at 0)
constexpr size_t kOutOffset = kHeadBytes;      // 18 norms
constexpr size_t kPartOffset = kHeadBytes + 256;
constexpr size_t kScratchBytes = kPartOffset + sizeof(double) * kParts * kMaxChunks;  // 41,472 bytes

static __device__ __align__(256) unsigned char g_normScratch[kScratchBytes];

std::mutex g_setupMutex;
void* g_scratchPtr[kMaxDevices] = {};

// |x| as a bit pattern: for non-negative doubles the order of the patterns is
// the numeric order and NaN patterns lie above infinity, so a NaN anywhere
// shows in the maxima exactly as in the batch's own pass
__device__ inline unsigned long long absBits(double x) {
  return (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
}
__device__ inline unsigned long long umax64(unsigned long long a, unsigned long long b) { return a > b ? a : b; }

// one block per chunk of the model; the block that completes the count
// combines the chunks in order and writes the 18 norms.  Partials per chunk:
// 0-4 the sums of squares of the weighted increment, velocity and acceleration
// increments and residual, and the energy sum (same order and expressions as
// the batch's pass), 5-17 the maxima as |x| bit patterns (energy, then the four
// vectors per DOF type), 18 unused, 19 a NaN/Inf flag.
__global__ void __launch_bounds__(kTpb) kNormsOneModel(DevData d, int m, int c0, int nc, unsigned char* scratch) {
  __shared__ double sh[kTpb / 32][kParts];
  __shared__ bool lastBlock;
  unsigned int* counter = reinterpret_cast<unsigned int*>(scratch);
  double* out = reinterpret_cast<double*>(scratch + kOutOffset);
  double* part = reinterpret_cast<double*>(scratch + kPartOffset);
  const int c = c0 + blockIdx.x;
  const double* wD = d.m.wDisp + 3 * m;
  const double* wF = d.m.wForce + 3 * m;
  const unsigned long long badBits = absBits(1.0e300);
  double v2 = 0.0, v3 = 0.0, v4 = 0.0, v5 = 0.0, v6 = 0.0;
  unsigned long long mx[13];
#pragma unroll
  for (int k = 0; k < 13; ++k) mx[k] = 0ull;
  bool bad = false;
  const int cEnd = d.chunkEnd[c];
  // thread t visits DOFs t, t + kTpb, t + 2 kTpb, ... of the chunk: the order
  // in which the batch's pass accumulates them
  for (int i = d.chunkStart[c] + threadIdx.x; i < cEnd; i += kTpb) {
    const int eq = d.meqn[i];
    if (eq < 0) continue;
    const int t = d.dofType[i] - 1;
    const double wd = wD[t], wf = wF[t];
    const double s0 = d.sinc0[i], s1 = d.sinc1[i], s2 = d.sinc2[i], r = d.res[eq];
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
    sh[w][0] = v2;
    sh[w][1] = v3;
    sh[w][2] = v4;
    sh[w][3] = v5;
    sh[w][4] = v6;
#pragma unroll
    for (int k = 0; k < 13; ++k) sh[w][5 + k] = __longlong_as_double((long long)mx[k]);
    sh[w][18] = 0.0;
    sh[w][19] = bad ? 1.0 : 0.0;
  }
  __syncthreads();
  // warps in order: sums added, maxima compared as bit patterns
  if (threadIdx.x < kParts) {
    const int k = threadIdx.x;
    double x = sh[0][k];
    for (int ww = 1; ww < kTpb / 32; ++ww) {
      const double y = sh[ww][k];
      if (k <= 4) x = x + y;
      else x = __longlong_as_double((long long)umax64(absBits(x), absBits(y)));
    }
    part[(size_t)blockIdx.x * kParts + k] = x;
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) lastBlock = atomicAdd(counter, 1u) == (unsigned int)nc - 1u;
  __syncthreads();
  if (!lastBlock || threadIdx.x != 0) return;
  __threadfence();
  double s[kParts];
  for (int k = 0; k < kParts; ++k) s[k] = __ldcg(part + k);
  for (int b = 1; b < nc; ++b)
    for (int k = 0; k < kParts; ++k) {
      const double x = __ldcg(part + (size_t)b * kParts + k);
      s[k] = (k <= 4) ? s[k] + x : __longlong_as_double((long long)umax64(absBits(s[k]), absBits(x)));
    }
  // the weight sums are the model's constants, as the batch's convergence test reads them
  const double sw = d.m.sumWd2[m], swf = d.m.sumWf2[m];
  out[0] = sw > 0 ? sqrt(s[0] / sw) : 0.0;
  out[4] = sw > 0 ? sqrt(s[1] / sw) : 0.0;
  out[8] = sw > 0 ? sqrt(s[2] / sw) : 0.0;
  out[12] = swf > 0 ? sqrt(s[3] / swf) : 0.0;
  for (int t = 0; t < 3; ++t) {
    out[1 + t] = s[6 + t];
    out[5 + t] = s[9 + t];
    out[9 + t] = s[12 + t];
    out[13 + t] = s[15 + t];
  }
  const int neq = d.m.neq[m], nd = d.m.ndof[m];
  out[16] = s[5];
  out[17] = (nd > 1 && neq > 0) ? s[4] / (double)neq : s[4];
  *counter = 0u;
}

// scratch address on device `dev` (made current here), looked up once per device
int scratchAddress(int dev, unsigned char** ptr, std::string& err) {
  if (dev < 0 || dev >= kMaxDevices) {
    err = "device ordinal " + std::to_string(dev) + " outside 0.." + std::to_string(kMaxDevices - 1);
    return -1;
  }
  cudaError_t e = cudaSetDevice(dev);
  if (e != cudaSuccess) {
    err = std::string("cannot make the batch's device current: ") + cudaGetErrorString(e);
    return -1;
  }
  std::lock_guard<std::mutex> lock(g_setupMutex);
  if (!g_scratchPtr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_normScratch);
    if (e != cudaSuccess || !p) {
      err = std::string("cudaGetSymbolAddress of the norms scratch failed: ") + cudaGetErrorString(e);
      return -2;
    }
    g_scratchPtr[dev] = p;
  }
  *ptr = static_cast<unsigned char*>(g_scratchPtr[dev]);
  return 0;
}

}  // namespace

int normsNoAlloc(const DevData& d, int m, int c0, int nc, int dev, cudaStream_t s, double* out18, std::string& err) {
  if (nc > kMaxChunks) {
    err = "model has " + std::to_string(nc) + " norm chunks of 2048 DOFs; the no-allocation path holds at most " +
          std::to_string(kMaxChunks) + " (524,288 DOFs)";
    return -3;
  }
  unsigned char* scratch = nullptr;
  if (int rc = scratchAddress(dev, &scratch, err)) return rc;
  cudaError_t e = cudaMemsetAsync(scratch, 0, kHeadBytes + 18 * sizeof(double), s);
  if (e == cudaSuccess && nc > 0) {
    kNormsOneModel<<<nc, kTpb, 0, s>>>(d, m, c0, nc, scratch);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(out18, scratch + kOutOffset, 18 * sizeof(double), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    err = std::string("norms without allocation failed: ") + cudaGetErrorString(e);
    return -4;
  }
  return 0;
}

}  // namespace fgpu
