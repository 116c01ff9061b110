// front_kernels.cu -- FP64 refinement residual of the mixed-precision solves.
//
// The multifrontal factorisation and the triangular solves replace the factor
// and solve of the absent SAM/SPR solver that the reference calls from csSolve
// (src/vpmCommon/vpmLinAlg/solExtensionModule.f90:153-505); they live in
// front_cascade.cu.  With FP32 fronts, each further solve of a Newton
// iteration corrects the accumulated FP64 solution x with the residual
// r = b - A x of the FP64 Newton matrix computed here.

#include "kernels.h"

namespace fgpu {
namespace {

constexpr int TPB = 256;
inline int blocksFor(long long n, int tpb = TPB) { return (int)((n + tpb - 1) / tpb); }

// r = b - A x with the FP64 Newton matrix (full symmetric CSR), one row per thread
__global__ void kRefineResidual(DevData d) {
  pdlEntry();
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.neqTot) return;
  // the row's extent is read with the model index, before the activity test
  const int64_t kb = d.rowPtr[i], ke = d.rowPtr[i + 1];
  if (!(d.m.flags[d.eqModel[i]] & FL_ACTIVE)) return;
  double s = 0.0;
  for (int64_t k = kb; k < ke; ++k) s += d.csrVal[k] * d.xref[d.colInd[k]];
  d.rref[i] = d.del[i] - s;
}

}  // namespace

void launchRefineResidual(const DevData& d, cudaStream_t s) {
  if (d.neqTot > 0) pdlLaunch(kRefineResidual, blocksFor(d.neqTot), TPB, 0, s, d);
}

}  // namespace fgpu
