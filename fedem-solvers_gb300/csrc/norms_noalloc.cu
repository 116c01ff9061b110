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
//  * the first call on each device does the set-up (looks up the scratch
//    address with cudaGetSymbolAddress, that device current): make it before
//    any stream capture begins on that device;
//  * the completion counter at the head of the scratch must start at zero: each
//    call clears it on the batch's stream before its launch, and nothing else
//    of the scratch is read before the same call has written it;
//  * there is one scratch per device, so calls that overlap in time on one
//    device (from several host threads) race on it: serialise them.
//
// The arithmetic is the batch's two-stage norms pass (kNormsPartial + kControl
// in element_kernels.cu): the same chunk boundaries, thread-to-DOF mapping,
// warp tree and chunk order, so the 18 values equal what the batch stored for
// the same vectors.  Norm definitions: src/vpmSolver/normTypeModule.f90:196-249.

#include <cstdint>
#include <mutex>
#include <string>

#include "kernels.h"

namespace fgpu {
namespace {

constexpr int kTpb = 256;        // threads per chunk block (as the batch's pass)
constexpr int kParts = 20;       // partial values per chunk
constexpr int kMaxChunks = 256;  // 256 chunks x 2048 DOFs = 524,288 DOFs
constexpr int kMaxDevices = 64;
constexpr size_t kHeadBytes = 256;             // completion counter (must start at 0)
constexpr size_t kOutOffset = kHeadBytes;      // 18 norms
constexpr size_t kPartOffset = kHeadBytes + 256;
constexpr size_t kScratchBytes = kPartOffset + sizeof(double) * kParts * kMaxChunks;  // 41,472 bytes

static __device__ __align__(256) unsigned char g_normScratch[kScratchBytes];

std::mutex g_setupMutex;
void* g_scratchPtr[kMaxDevices] = {};

// one block per chunk of the model; the block that completes the count
// combines the chunks in order and writes the 18 norms
__global__ void __launch_bounds__(kTpb) kNormsOneModel(DevData d, int m, int c0, int nc, unsigned char* scratch) {
  __shared__ double sh[kTpb / 32][kParts];
  __shared__ bool lastBlock;
  unsigned int* counter = reinterpret_cast<unsigned int*>(scratch);
  double* out = reinterpret_cast<double*>(scratch + kOutOffset);
  double* part = reinterpret_cast<double*>(scratch + kPartOffset);
  const int c = c0 + blockIdx.x;
  const double* wD = d.m.wDisp + 3 * m;
  const double* wF = d.m.wForce + 3 * m;
  double v[kParts];
#pragma unroll
  for (int k = 0; k < kParts; ++k) v[k] = 0.0;
  for (int i = d.chunkStart[c] + threadIdx.x; i < d.chunkEnd[c]; i += kTpb) {
    int eq = d.meqn[i];
    if (eq < 0) continue;
    int t = d.dofType[i] - 1;
    double wd = wD[t], wf = wF[t];
    double s0 = d.sinc0[i], s1 = d.sinc1[i], s2 = d.sinc2[i], r = d.res[eq];
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
#pragma unroll
  for (int k = 0; k < kParts; ++k) {
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
    for (int k = 0; k < kParts; ++k) sh[w][k] = v[k];
  __syncthreads();
  if (threadIdx.x < kParts) {
    const int k = threadIdx.x;
    double x = sh[0][k];
    for (int ww = 1; ww < kTpb / 32; ++ww) x = (k <= 6) ? x + sh[ww][k] : fmax(x, sh[ww][k]);
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
      double x = __ldcg(part + (size_t)b * kParts + k);
      s[k] = (k <= 6) ? s[k] + x : fmax(s[k], x);
    }
  out[0] = s[0] > 0 ? sqrt(s[2] / s[0]) : 0.0;
  out[4] = s[0] > 0 ? sqrt(s[3] / s[0]) : 0.0;
  out[8] = s[0] > 0 ? sqrt(s[4] / s[0]) : 0.0;
  out[12] = s[1] > 0 ? sqrt(s[5] / s[1]) : 0.0;
  for (int t = 0; t < 3; ++t) {
    out[1 + t] = s[8 + t];
    out[5 + t] = s[11 + t];
    out[9 + t] = s[14 + t];
    out[13 + t] = s[17 + t];
  }
  const int neq = d.m.neq[m], nd = d.m.ndof[m];
  out[16] = s[7];
  out[17] = (nd > 1 && neq > 0) ? s[6] / (double)neq : s[6];
  *counter = 0u;
}

// scratch address on the current device, looked up once per device
int scratchAddress(unsigned char** ptr, std::string& err) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    err = std::string("no usable current CUDA device: ") + cudaGetErrorString(e);
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

int normsNoAlloc(const DevData& d, int m, int c0, int nc, cudaStream_t s, double* out18, std::string& err) {
  if (nc > kMaxChunks) {
    err = "model has " + std::to_string(nc) + " norm chunks of 2048 DOFs; the no-allocation path holds at most " +
          std::to_string(kMaxChunks) + " (524,288 DOFs)";
    return -3;
  }
  unsigned char* scratch = nullptr;
  if (int rc = scratchAddress(&scratch, err)) return rc;
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
