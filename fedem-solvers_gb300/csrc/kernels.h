// kernels.h -- launch wrappers of the batched FEDEM Newton engine kernels.
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "engine_dev.cuh"

namespace fgpu {

// Programmatic dependent launch.  Every kernel of the engine is launched with
// programmatic stream serialization (pdlLaunch) and calls pdlEntry() first:
// it waits until the previous kernel of its stream has completed and its
// memory is visible (griddepcontrol.wait), then lets the next kernel's blocks
// be scheduled (griddepcontrol.launch_dependents), which then wait the same
// way.  Ordering and results are those of plain stream order; only the launch
// of each kernel overlaps the end of the one before.
#ifdef __CUDACC__
__device__ __forceinline__ void pdlEntry() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

template <typename... KArgs, typename... Args>
inline void pdlLaunch(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                      Args... args) {
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, kernel, args...);
}
#endif

// element pass modes
enum ElemMode : int {
  EM_PRED = 0,         // predictor: velocities from dk/ak, no position update
  EM_INC = 1,          // after an increment: corotation, deformation, forces
  EM_STATIC_INIT = 2,  // static, initial frame kept (linInc = 1)
  EM_STATIC = 3,       // static after an increment (corotated update)
  EM_FINAL = 4         // final static update: corotation, zero velocities, no vld
};

// --- element_kernels.cu ----------------------------------------------------
// Seeding of the backward work queues by the step-start kernels: for each
// solve q of the iteration, queue q receives the roots of the active models
// and ctr[4 q + 2] their number of chains (ctr[4 q] and ctr[4 q + 1] are the
// take and fill positions); nq = 0 seeds nothing.
struct BackwardSeed {
  int nq = 0;      // queues (solves per iteration)
  int stride = 0;  // slots per queue
  // per model: the tops of its small-front subtrees (fronts whose parent is a
  // large front, or roots) in roots[rootOff[m]..rootOff[m+1]), and its number
  // of chains
  const int* rootOff = nullptr;
  const int* roots = nullptr;
  const int* slotCnt = nullptr;
  int* queue = nullptr;
  int* ctr = nullptr;
  // the same for the large-front queues (seeded with the large roots; chains
  // end at large fronts without large children); strideL = 0: no large fronts
  int strideL = 0;
  const int* rootOffL = nullptr;
  const int* rootsL = nullptr;
  const int* slotCntL = nullptr;
  int* queueL = nullptr;
  int* ctrL = nullptr;
};
void launchBeginStep(const DevData& d, int* activeCount, long long* activeEl, const BackwardSeed& seed,
                     cudaStream_t s);
void launchPredictDofs(const DevData& d, cudaStream_t s);
void launchElements(const DevData& d, int mode, cudaStream_t s);
void launchResidual(const DevData& d, cudaStream_t s);
void launchBuildElementNewton(const DevData& d, cudaStream_t s);
void launchRotateElementNewton(const DevData& d, cudaStream_t s);
void launchCsrGather(const DevData& d, cudaStream_t s);
void launchIncrement(const DevData& d, cudaStream_t s);
void launchNormsControl(const DevData& d, cudaStream_t s);
// the same in two parts: the per-chunk partial norms (reading the increments
// and the residual only), then the convergence test and the step end
void launchNormsPartial(const DevData& d, cudaStream_t s);
void launchControlStepEnd(const DevData& d, cudaStream_t s);
// static equilibrium helpers
void launchStaticBegin(const DevData& d, int* activeCount, const BackwardSeed& seed, cudaStream_t s);
void launchSeedBackward(const DevData& d, const BackwardSeed& seed, cudaStream_t s);
void launchStaticResidual(const DevData& d, cudaStream_t s);
void launchStaticNorm(const DevData& d, cudaStream_t s);
void launchStaticIncrement(const DevData& d, cudaStream_t s);
void launchStaticFinish(const DevData& d, cudaStream_t s);

// --- joint_kernels.cu: master-slave joints ----------------------------------
// per joint: joint variables incremented (EM_INC, EM_STATIC), dependent triad
// placed, constraint coefficients rebuilt; same model gating as the element pass
void launchJoints(const DevData& d, int mode, cudaStream_t s);
// expanded Newton matrices of the elements with a dependent triad (tangent models)
void launchExpandElements(const DevData& d, cudaStream_t s);
// expanded forces of those elements after an element pass of this mode
void launchExpandForces(const DevData& d, int mode, cudaStream_t s);

// reduced parts (part_kernels.cu): the element pass, the Newton matrices and
// the end-of-step copy of the deformation; preparePartKernels sets the shared
// memory the batch's largest part needs (0, or < 0 on error)
int preparePartKernels(const DevData& d);
void launchParts(const DevData& d, int mode, cudaStream_t s);
void launchPartsNewton(const DevData& d, cudaStream_t s);
void launchPartsStepEnd(const DevData& d, cudaStream_t s);

// --- front_cascade.cu: one launch per phase over all fronts of all models ----
struct PersistentPlan {
  const int* leaves;  // fronts without children, longest root path first (factorisation)
  int nLeaves;
  // forward-elimination tasks, longest root path first: a leaf, or a front
  // whose children are all leaves with bit 30 set (a group, eliminated by one
  // warp)
  const int* tasks;
  int nTasks;
  int maxRow;         // largest front of the batch (rows)
  int maxNpiv;        // largest pivot block of the batch
  int maxAsm;         // largest number of original entries of one front
  int maxSeg;         // largest children update segment of one front (packed lower values)
  // per-front counters, each followed by the launch's leaf counter: one set for
  // the factorisation, one per refinement forward elimination (nfrontTot + 1
  // apart); zeroed with the other iteration counters at the iteration start
  int *cntFactor, *cntForward, *errFlag;
  // backward work queues, one per solve of the iteration (nLeaves slots apart),
  // and their counters (4 per queue), seeded by the step-start kernels; the
  // fronts whose leaf children are solved inline
  const unsigned char* bwInline;
  int *bwQueue, *bwCtr;
  // polls of a bounded wait in the back substitution before it gives up and
  // sets errFlag (about 1-2 s at the default)
  long long spinLimit = 1LL << 23;
  // large fronts (more than kLargeFrontRows rows, and all their ancestors),
  // one thread block each (front_large.cu): the number of large children of
  // every front (d.fNlarge, global), the cascade's start tasks (large fronts
  // without large children, longest root path first), the largest large front,
  // their counters (factor, then one set per refinement forward elimination,
  // nfrontTot + 1 apart) and backward queues (largeStride slots per solve, 4
  // counters per solve)
  const unsigned char* fLarge = nullptr;
  const int* fNlarge = nullptr;
  const int* largeTasks = nullptr;
  int nLargeTasks = 0;
  int maxRowLarge = 0;
  int *cntLargeFactor = nullptr, *cntLargeForward = nullptr;
  int *bwLQueue = nullptr, *bwLCtr = nullptr;
  int largeStride = 0;
  // Launch shapes, picked per batch by the engine's autotuner.  No choice
  // changes a result bit: tasks are taken dynamically, and each front's
  // arithmetic is the same whichever warp, block or cluster does it.
  int factorPanel = 0;     // small-front panel factorisation: 0 shuffles, 1 register-blocked
                           // (blocks of 8), 2 register-blocked (blocks of 4, fronts up to 32 rows)
  int forwardWarps = 8;    // warps per block of the forward-elimination cascade
  int backwardWarps = 8;   // warps per block of the back-substitution queue
  int largeCluster = 8;    // blocks per cluster of the large-front factorisation (2, 4, 8 or 16)
};
// fronts with more rows than this are factored and solved by a thread block
// each (front_large.cu); smaller ones by one warp each in shared memory
constexpr int kLargeFrontRows = 96;
// the large-front kernels: factorisation (tangent models) fused with the first
// forward elimination, a further forward elimination (refinement sweep), and
// the back substitution of the large fronts (before the warp queue's)
void launchLargeFactorForward(const DevData& d, const PersistentPlan& p, bool fp32, const double* rhs,
                              cudaStream_t s);
// clusters of csize blocks (2 to 16) the device can hold at once for the
// large-front factorisation of this plan (0: none)
int largeClusterCapacity(const PersistentPlan& p, bool fp32, int csize);
void launchLargeForward(const DevData& d, const PersistentPlan& p, bool fp32, const double* rhs, int sweep,
                        cudaStream_t s);
void launchLargeBackward(const DevData& d, const PersistentPlan& p, bool fp32, int sweep, bool last, cudaStream_t s);
// values of one front's L block the solve kernels stage in shared memory
int stagingCapacity(const PersistentPlan& p, size_t elemBytes);
// The first solve's back substitution run by the factorisation's own launch
// (its warps serve the solve's queue once every leaf is taken); queue null:
// not fused.  Batches without large fronts only.
struct FusedBackward {
  int* queue = nullptr;
  int* ctr = nullptr;
  const unsigned char* bwInline = nullptr;
  int* errFlag = nullptr;
  long long spinLimit = 0;
  int acc = 0, finalize = 0, capL = 0;
};
// whether the factorisation's launch can run the first back substitution: no
// large fronts, and every front's L block fits the warp's staging area (the
// fused solve reads L through L2 into shared memory)
bool fusableBackward(const PersistentPlan& p, bool fp32);
// factorisation of the models with a tangent update fused with the forward
// elimination of rhs for every active model (first solve of an iteration);
// withBackward: the back substitution of that solve too (lastSweep: it is the
// iteration's last solve), in place of launchBackward for sweep 0
void launchFactorForwardCascade(const DevData& d, const PersistentPlan& p, bool fp32, const double* rhs,
                                cudaStream_t s, bool withBackward = false, bool lastSweep = false);
// forward elimination of the right-hand side rhs (FP64, rounded to the solve precision)
void launchForwardCascade(const DevData& d, const PersistentPlan& p, bool fp32, const double* rhs, int sweep,
                          cudaStream_t s);
// back substitution; stores the solution in del (FP64 solve) or accumulates it in xref
// (FP32 refinement sweep `sweep`; the last sweep also copies xref to del)
void launchBackward(const DevData& d, const PersistentPlan& p, bool fp32, int sweep, bool last, cudaStream_t s);
// One warp of the back-substitution queue kernel on a private queue (4 ints of
// counters at ctr, the slots at queue), waiting at most `spins` polls: with an
// empty slot 0 and a slot total of 1 the wait runs out and sets p.errFlag.
void launchBackwardWaitProbe(const DevData& d, const PersistentPlan& p, int* queue, int* ctr, long long spins,
                             cudaStream_t s);
// One warp of the fused factorisation without leaves on a private queue whose
// slot 0 holds a root of an active model and private counters cnt (zeroed,
// nfrontTot + 1): the root's release never comes, so the bounded wait runs out
// after `spins` polls and sets p.errFlag.
void launchRootWaitProbe(const DevData& d, const PersistentPlan& p, int* queue, int* ctr, int* cnt, long long spins,
                         cudaStream_t s);
// prescribed deflections (step start), their predictor right-hand side (after the
// element Newton matrices), and the restart state of pure linear quasi-static steps
void launchMotions(const DevData& d, cudaStream_t s);
void launchLoads(const DevData& d, cudaStream_t s);
void launchMotionRhs(const DevData& d, cudaStream_t s);
void launchQsRestore(const DevData& d, cudaStream_t s);
// synthetic, diagonally dominant original entries of every front (the
// autotuner's timing probe, before the first iteration gathers the real ones)
void launchProbeEntries(const DevData& d, bool fp32, cudaStream_t s);
// results database of the primary response (results.cu): per model a ring of
// kRecordRing records (step, time, triad positions, superelement frames and
// generalized DOFs, as doubles) in buf, written at each completed step
struct RecordPlan {
  double* buf = nullptr;       // the rings, model after model
  long long* off = nullptr;    // per model: first value of its ring
  int* vals = nullptr;         // per model: values per record (2 + data)
  int* triRec = nullptr;       // per triad (global): offset of its values in its model's record
  int* elRec = nullptr;        // per model: offset of its beam frames (12 per element)
  int* partFirst = nullptr;    // per model, + 1: first reduced part (global)
  int* partRec = nullptr;      // per part: offset of its frame and generalized DOFs
  long long* count = nullptr;  // per model: records written so far
  int ring = 0;
};
constexpr int kRecordRing = 8;
// all: a record of every model's current state; otherwise of the models whose
// step has just completed
void launchRecordStep(const DevData& d, const RecordPlan& r, bool all, cudaStream_t s);
// FP64 refinement residual r = b - A x (front_kernels.cu)
void launchRefineResidual(const DevData& d, cudaStream_t s);

// Convergence norms of model m recomputed into a fixed scratch array compiled
// into the library (no device allocation); blocks until the 18 values are in
// out18 (host).  c0/nc: the model's first norm chunk and chunk count; dev: the
// batch's device (made current for the launch).
int normsNoAlloc(const DevData& d, int m, int c0, int nc, int dev, cudaStream_t s, double* out18, std::string& err);

}  // namespace fgpu
