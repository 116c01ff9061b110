// engine.h -- the batched GB300 Newton engine: many FEDEM models resident in
// HBM, advanced one Newton iteration per model per batched iteration.
#pragma once

#include <cuda_runtime.h>

#include <cstdio>
#include <string>
#include <array>
#include <vector>

#include "engine_dev.cuh"
#include "host_model.h"
#include "kernels.h"

namespace fgpu {

struct EngineOptions {
  bool fp32Factor = false;  // mixed precision: FP32 fronts + FP64 iterative refinement
  int refineSweeps = 3;     // solves per Newton iteration in mixed precision (1 + refinements)
  bool useGraph = true;     // capture the batched iteration in a CUDA graph
  bool compressBeams = true;  // 26-value beam matrices when every element has the principal-axes pattern
};

struct RunStats {
  long long newtonIterations = 0;  // sum over models of Newton iterations performed
  long long timeSteps = 0;         // sum over models of completed time steps
  long long batchedIterations = 0;
  int modelsDone = 0, modelsFailed = 0;
};

class Engine {
 public:
  Engine() = default;
  ~Engine();
  Engine(const Engine&) = delete;
  Engine& operator=(const Engine&) = delete;

  // Uploads the models (host arrays -> HBM) and prepares the level schedule.
  int upload(const std::vector<const HostModel*>& models, const EngineOptions& opt, std::string& err);
  // Initial static equilibrium (when requested) and the final static update.
  int initialState(std::string& err);
  // Runs batched iterations until no model is active or maxBatched is reached.
  int run(long long maxBatched, RunStats* stats);
  // Non-blocking driving (serving): enqueue n batched iterations followed by an
  // asynchronous read of the active-model count and of every model's state;
  // poll reports whether that chunk finished (*ready) and whether any model is
  // still active; chunkStates() then holds the states (ModelState per model).
  int launchChunk(int n);
  int pollChunk(bool* ready, int* active);
  const int* chunkStates() const { return hStates_; }
  // Device bytes this engine allocated.
  size_t deviceBytes() const { return deviceBytes_; }
  // The CUDA device the engine was uploaded to (the calling thread's current
  // device at upload); every later call on the engine must run with it current.
  int device() const { return device_; }
  // Sum of Newton iterations over all models (blocking read).
  long long totalIterations();
  // Advances model `m` by exactly one time step (other models may advance too).
  int advanceOneStep(int m, int* state);

  // accessors (blocking device -> host copies)
  int numModels() const { return (int)hm_.size(); }
  int modelState(int m);
  int modelStatus(int m);
  double modelTime(int m);
  double modelDt(int m);
  long long modelSteps(int m);
  long long modelIterations(int m);
  int getTriadUr(int m, double* ur);  // 12 per triad of the model
  int getNorms(int m, double* norms18);
  int getElementFrames(int m, double* supTr12);  // current 3x4 frames, 12 per element
  int getCsrValues(int m, double* vals);  // full symmetric CSR values of the last tangent
  int getEqVector(int m, int which, double* v);  // 0 FS, 1 FD, 2 FI, 3 Q, 4 residual, 5 del
  const HostModel& host(int m) const { return *hm_[m]; }
  cudaStream_t stream() const { return stream_; }
  const DevData& devData() const { return d_; }
  // first norm chunk and chunk count (2048 DOFs each) of model m
  int normChunkOffset(int m) const { return normChunkOff_[m]; }
  int normChunkCount(int m) const { return normChunkCnt_[m]; }
  // Device counters for the launch count claim: kernels enqueued per batched iteration.
  int launchesPerIteration() const { return launchesPerIter_; }
  double lastRunSeconds() const { return lastRunSec_; }
  double lastRunDeviceSeconds() const { return lastRunDevSec_; }  // CUDA events on the engine stream
  long long uploadedBytes() const { return uploadedBytes_; }
  void setStepLimit(long long lim);
  // Externally driven stepping (solverInterface startStep / solveIteration):
  // the two halves of a Newton iteration, launched directly and completed.
  int assembleIteration();
  int solveUpdateIteration();
  void setStepLimitOf(int m, long long lim);
  int setTimeStep(int m, double dt);
  // Solves with the stiffness matrix at the current configuration (eigenmodes):
  // prepareStiffnessSolves assembles and factors K of every model (Newton matrix
  // scales 0, 1, 0), solveStiffness solves K x = b for model m (b, x: its
  // equations; the other models' vectors are scratch), endStiffnessSolves puts the
  // flags back and makes the next tangent iteration rebuild the Newton matrices.
  // Only between steps: the factors of the step in progress are overwritten.
  int prepareStiffnessSolves();
  int solveStiffness(int m, const double* b, double* x);
  int endStiffnessSolves();
  // The linear-solver seam of one model, between its steps (csAddEM + csSolve
  // granularity): its Newton matrix N = sM M + sC C + sK K assembled on the GPU
  // (element matrices, constraint expansion, CSR); factored (returns the
  // number of negative pivots, -3 when a pivot is singular); solved for nrhs
  // right-hand sides of its equations, in place.  The model's next batched
  // iteration starts a step and so refactors its own tangent.
  int seamAssemble(int m, double sM, double sC, double sK);
  int seamFactor(int m);
  int seamSolve(int m, double* rhs, int nrhs);
  // external function channel ch (0-based) of model m: its value for the next step
  int setExtValue(int m, int ch, double v);
  double extValue(int m, int ch);
  // replaces (add = false) or adds to the right-hand side of the assembled iteration
  int setRhs(int m, const double* v, bool add);
  // the mutable state as one host byte array (in-core restart)
  size_t stateBytes() const;
  int saveStateTo(void* host);
  int restoreStateFrom(const void* host);
  // One model's share of the mutable state (its slices of every state array):
  // a model built from the same host model in another engine takes it and
  // continues from there bitwise as it would have here (continuous batching
  // moves running models into a new engine with it).  Only between steps.
  int extractModelState(int m, std::vector<char>& out);
  int injectModelState(int m, const std::vector<char>& in);
  // The models in `ms` stop at the end of their current step (a model between
  // steps at once): their step limit becomes the current step count (+ 1 when a
  // step is in progress).  Blocking.
  int parkModels(const std::vector<int>& ms);
  // Saves / restores the mutable device state (device-to-device copies), so a
  // timed run can start again from the initial state already resident in HBM.
  int snapshot();
  int restore();
  // Phase timings sampled with CUDA events inside the captured iteration:
  // phase 0 = element pass after the increment, 1 = factorisation with the
  // first forward elimination, 2 = the rest of the solves, 3 = the forward
  // elimination of the second solve (mixed-precision batches; else 0),
  // 4 = the back substitution of the first solve.
  // Returns samples; ms[n] (n <= 5) = summed milliseconds, elems = summed active elements.
  long long phaseTimings(double* ms, long long* activeElems, int n = 4);
  // Times `reps` launches of the factorisation fused with the first forward
  // elimination with every model factoring (CUDA events on the engine stream);
  // the flags, status and pivot counters are restored afterwards, the factors
  // and solve vectors are scratch.  *bytes: algorithmic bytes of one launch.
  int timeFactor(int reps, double* msPerLaunch, double* bytes);
  void resetPhaseTimings();
  // Test hook: a bounded wait of `spins` polls that nothing ends (see engine.cu).
  int probeWaitTimeout(long long spins, int* flag);
  // the same for the fused back substitution's wait for a root's elimination
  int probeRootWaitTimeout(long long spins, int* flag);

  // Launch shapes of the multifrontal kernels (PersistentPlan: factor panel
  // variant, forward and backward warps per block, large-front cluster size).
  // Before the first batched iteration the autotuner times the candidates on
  // this batch's own fronts and keeps the fastest; shapes already tuned for a
  // batch of the same structure are reused.  setLaunchShape (before the first
  // iteration) fixes them instead.  No shape changes a result bit.
  int setLaunchShape(const int* shape4);
  // shape4 as above; *probeMs: wall time of this engine's probe (0 when the
  // shapes came from setLaunchShape or the cache); returns 1 if tuned, 0 if not yet
  int launchShape(int* shape4, double* probeMs) const;

  // Results database of the primary response (results.cu): from now on every
  // model appends one record per completed time step to <dir>/model<k>.res
  // (a record of the current state first).  resultsClose flushes and closes.
  // paths: one file per model instead of <dir>/model<k>.res; records of times
  // before saveStart are not written (the reference's -savestart)
  int resultsOpen(const std::string& dir, bool asDouble, std::string& err,
                  const std::vector<std::string>* paths = nullptr, double saveStart = -1.0e300);
  int resultsClose(std::string& err);

 private:
  template <typename T>
  T* alloc(size_t n);
  void enqueueIteration(cudaStream_t s);
  void enqueueAssembly(cudaStream_t s);
  void enqueueSolveUpdate(cudaStream_t s);
  // backwardDone: the first solve's back substitution already ran in the
  // factorisation's launch (enqueueFactor with withBackward)
  void enqueueSolve(cudaStream_t s, bool timedForward = false, bool backwardDone = false);
  void enqueueFactor(cudaStream_t s, bool withBackward = false);
  int readActive();
  // the autotuner: runs once, before the first batched iteration
  void ensureTuned();
  int autotune();
  bool tuned_ = false, shapeFixed_ = false, iterated_ = false;
  double probeMs_ = 0.0;
  // results database: ring plan, files and the records already written per model
  struct Results {
    bool on = false, asDouble = true;
    double saveStart = -1.0e300, epsT = 0.0;
    RecordPlan plan;
    std::vector<FILE*> files;
    std::vector<int> vals;
    std::vector<long long> off, written;
    std::vector<double> host;
  } rec_;
  int resultsDrain(std::string& err);

  std::vector<const HostModel*> hm_;
  EngineOptions opt_;
  DevData d_{};
  std::vector<void*> allocs_;
  PersistentPlan pplan_{};
  int* dActive_ = nullptr;
  int* hActive_ = nullptr;  // pinned
  int* hStates_ = nullptr;  // pinned: every model's state after the last chunk
  cudaStream_t stream_ = nullptr;
  // beam-only batches: the Newton-matrix assembly (element matrices, CSR
  // gather) runs on a second stream beside the predictor, element pass and
  // residual, which it does not depend on; fork and join events
  cudaStream_t side_ = nullptr;
  cudaEvent_t evFork_ = nullptr, evJoin_ = nullptr;
  bool forkAssembly_ = false;
  bool fuseBackward_ = false;  // first back substitution inside the factorisation's launch
  // every batch: the partial norms run on the side stream beside the element
  // pass after the increment (they read the increments and the residual only)
  cudaEvent_t evFork2_ = nullptr, evJoin2_ = nullptr;
  bool sideReady();
  cudaGraph_t graph_ = nullptr;
  cudaGraphExec_t graphExec_ = nullptr;
  std::vector<int> modelTriOff_, modelDofOff_, modelEqOff_, modelElOff_;
  std::vector<int64_t> modelSlotOff_;
  std::vector<int> normChunkOff_, normChunkCnt_;
  int launchesPerIter_ = 0;
  double lastRunSec_ = 0.0;
  bool allocFailed_ = false;
  // snapshot of mutable arrays: (device pointer, bytes) and the backup buffer
  std::vector<std::pair<void*, size_t>> mutable_;
  // the same arrays with the layout their per-model slices follow
  enum StateKind : int { SK_TRIAD, SK_DOF, SK_EQ, SK_MODEL, SK_ELEM, SK_AXIAL, SK_MOTION, SK_EXT, SK_PART,
                         SK_PARTVEC, SK_PARTGEN, SK_JVAR, SK_JOINT, SK_XVEC };
  struct StateArray {
    char* p;
    size_t elem;  // bytes of one value
    int kind;
    int width;    // values per object (per model for SK_MODEL; rows for the SoA kinds)
    std::string tag;  // names the array in a model's state blob
  };
  std::vector<StateArray> stateArrays_;
  // per model and kind: first object and object count (SK_MODEL: the model itself)
  std::vector<std::array<int64_t, 2>> mRange_[14];
  int64_t stride_[14] = {0};  // objects per SoA row (elements, axial elements)
  void modelSlices(const StateArray& a, int m, std::vector<std::pair<size_t, size_t>>& out) const;
  std::vector<double> scaleSentinel_;
  std::vector<int> modelExtOff_, modelExtCnt_;
  std::vector<int> savedFlags_;
  double factorBytes_ = 0.0;  // algorithmic bytes of one factor + first forward launch, all models
  int* ctrBlock_ = nullptr;   // the iteration counters (see upload)
  size_t ctrInts_ = 0, queueInts_ = 0, largeQueueInts_ = 0;
  BackwardSeed seed_;
  void resetIterationCounters(cudaStream_t s);
  void invalidateNewtonScales();
  void recordPhase(cudaEvent_t ev, cudaStream_t s);
  char* backup_ = nullptr;
  // phase timing events (recorded as external event nodes inside the graph)
  cudaEvent_t ev_[9] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  long long* dActiveEl_ = nullptr;
  long long* hActiveEl_ = nullptr;
  cudaEvent_t evRun_[2] = {nullptr, nullptr};
  double lastRunDevSec_ = 0.0;
  long long uploadedBytes_ = 0;
  size_t partVecTot_ = 0;  // DOF-vector entries of all parts (pFinit, pFinitPrev)
  cudaEvent_t evChunk_ = nullptr;
  bool chunkPending_ = false;
  size_t deviceBytes_ = 0;
  int device_ = 0;
  double phaseMs_[5] = {0, 0, 0, 0, 0};
  long long phaseSamples_ = 0, phaseElems_ = 0;
};

}  // namespace fgpu
