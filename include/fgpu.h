/*
 * fgpu.h -- batched and served GB300 FEDEM Newton engine (handle-based C ABI,
 * exported by libfedem_solver_core.so next to the legacy ABI).
 *
 * The reference core is a process-wide singleton (src/vpmSolver/solverModule.f90:
 * 40-49, solverInterface.C:49) and has no batch or serving interface, so these
 * entry points have no direct reference counterpart.  Their per-model semantics
 * are exactly solverInit + solveNext-until-the-end of the reference
 * (src/vpmSolver/solverInterface.h:65, :247): same input text, same options,
 * same time integration; only many models advance together on one GPU.
 *
 * All pointers are caller-owned host memory, read or written during the call.
 * Return codes: 0 success, < 0 error (fgpu_last_error() gives the text).
 */
#ifndef FGPU_H
#define FGPU_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fgpu_model fgpu_model;  /* host-side set-up of one model */
typedef struct fgpu_batch fgpu_batch;  /* models resident on the GPU    */

/* Device selection.  The library carries its own CUDA runtime, so the device a
 * caller selected through another runtime (e.g. a deep-learning framework) is
 * not seen here.  fgpu_set_device makes `ordinal` current on the calling thread
 * and the device of every batch, server and legacy solverInit created
 * afterwards (from any thread); without it they use the creating thread's
 * current device of this runtime (device 0 unless set).  Every later call on a
 * handle runs on the handle's device, whichever thread makes it.  A process per
 * GPU calls fgpu_set_device(local rank) once before creating anything. */
int fgpu_set_device(int ordinal);
/* The selected device (or the calling thread's current one) and its PCI bus id
 * ("0000:1b:00.0" style, len bytes at most; pciBusId may be NULL). */
int fgpu_get_device(int* ordinal, char* pciBusId, int len);
/* The device a batch was uploaded to. */
int fgpu_batch_device(const fgpu_batch* b);

/* Host set-up of one model (the preprocessing part of solverInit,
 * solverInterface.h:65): parses the solver-input text and options, builds
 * the element matrices, equation numbering, sparsity pattern, gather maps and
 * the multifrontal symbolic factorisation.  No GPU work. */
int fgpu_model_create(const char* fsi, int argc, const char* const* argv, fgpu_model** out);
void fgpu_model_destroy(fgpu_model* m);
/* ntri, ndof, neq, nel, nnz (full CSR), nfront, max front rows, tree height */
int fgpu_model_sizes(const fgpu_model* m, long long* sizes8);
/* equation numbering (1-based, 0 = fixed), ndof entries */
int fgpu_model_meqn(const fgpu_model* m, int* meqn);
/* full symmetric CSR pattern in equation order: rowptr[neq+1], cols[nnz] (0-based) */
int fgpu_model_csr_pattern(const fgpu_model* m, int* rowptr, int* cols);
/* elimination order (position -> 0-based equation) and front partition:
 * for each front: npiv, nrow, parent (-1 root), height */
int fgpu_model_symbolic(const fgpu_model* m, int* perm, int* frontInfo4);
/* element matrix (0 = K, 1 = M, 2 = C), 12x12 column-major, superelement axes */
int fgpu_model_element_matrix(const fgpu_model* m, int iel, int which, double* mat);

/* Uploads the models to the GPU (host -> HBM copies), solves each model's
 * initial static equilibrium if requested and prepares the batched iteration.
 * mixed != 0: FP32 frontal factorisation + FP64 iterative refinement with
 * `sweeps` solves per Newton iteration (0: default 2); mixed == 0: plain FP64. */
int fgpu_batch_create(int nmodels, fgpu_model* const* models, int mixed, int sweeps, fgpu_batch** out);
void fgpu_batch_destroy(fgpu_batch* b);
/* Runs batched Newton iterations until every model reached its end time (or
 * maxBatched iterations).  stats10: newton iterations, time steps, batched
 * iterations, models done, models failed, kernels per batched iteration,
 * wall microseconds, device microseconds (CUDA events), bytes uploaded by
 * fgpu_batch_create, 0. */
int fgpu_batch_run(fgpu_batch* b, long long maxBatched, long long* stats10);
/* per-model results: state (0 stepping, 1 iterating, 2 done, 3 error),
 * status bits (1 singular, 2 max iterations, 4 NaN, 8 corotation, 16 a bounded
 * wait ran out), time, steps, Newton iterations.  A model that fails (in its
 * initial static equilibrium or in a step) stops in state 3 with its bits set;
 * the other models of the batch go on unaffected. */
int fgpu_batch_model_info(fgpu_batch* b, int model, int* state, int* status, double* time, long long* steps,
                          long long* iters);
/* triad position matrices of one model, 12 doubles (3x4 column-major) each */
int fgpu_batch_get_triads(fgpu_batch* b, int model, double* ur);
/* triad position matrices of all models, concatenated in model order */
long long fgpu_batch_get_all_triads(fgpu_batch* b, double* ur);
/* FP64 Newton matrix values (full CSR, last tangent update) of one model */
int fgpu_batch_get_newton_values(fgpu_batch* b, int model, double* vals);
/* equation vectors of one model: 0 FS, 1 FD, 2 FI, 3 Q, 4 residual, 5 last solution */
int fgpu_batch_get_vector(fgpu_batch* b, int model, int which, double* v);
/* last iteration norms (18: displacement, velocity, acceleration, residual
 * L2 + inf per DOF type, energy max/sum) */
int fgpu_batch_get_norms(fgpu_batch* b, int model, double* norms18);
/* The same 18 norms recomputed on the device from the model's current
 * increment and residual vectors WITHOUT ALLOCATING anything: for callers that
 * may not allocate device memory when they check convergence (a control or
 * co-simulation loop between its own stream-ordered kernels, where cudaMalloc
 * and cudaFree would synchronise the device; a process whose device memory is
 * committed to resident batches).  It reduces into a fixed scratch array of
 * about 41 KB per device compiled into the library, so models above 524,288
 * DOFs are refused (error code, message in fgpu_last_error).  The first call on
 * a device looks up that scratch's address: make it before any stream capture
 * begins on the device.  Calls that overlap in time on one device race on the
 * shared scratch: serialise them.  Blocks until the values are in norms18.
 * No reference counterpart (the reference computes norms inside its own
 * iteration loop only). */
int fgpu_batch_norms_noalloc(fgpu_batch* b, int model, double* norms18);
/* Advances only `model` by one time step (step-at-a-time driving). */
int fgpu_batch_step(fgpu_batch* b, int model, int* state);
/* Saves / restores the batch's mutable device state with device-to-device
 * copies (a rerun from the initial state without host transfers). */
int fgpu_batch_snapshot(fgpu_batch* b);
int fgpu_batch_restore(fgpu_batch* b);
/* CUDA-event samples of phases of the batched iteration, taken inside
 * fgpu_batch_run: ms4 = summed milliseconds of {element pass after the
 * increment, multifrontal factorisation with the first forward elimination
 * (and the first back substitution in batches without large fronts), the
 * remaining solve launches incl. refinement, the forward elimination of
 * the second solve (0 with one solve)}; elems = summed active elements of the
 * sampled iterations.  Returns the number of samples; reset != 0 clears the
 * accumulators afterwards. */
long long fgpu_batch_phase_timings(fgpu_batch* b, double* ms4, long long* elems, int reset);
/* The same with n (1..5) phases: the four above, then the back substitution
 * launched on its own -- the first solve's, or, in batches without large
 * fronts (where the first solve's back substitution runs inside the
 * factorisation's launch), the second solve's (0 with one solve). */
long long fgpu_batch_phase_timings_n(fgpu_batch* b, double* ms, int n, long long* elems, int reset);
/* Times reps launches of the factorisation fused with the first forward
 * elimination with every model factoring (CUDA events on the batch's stream).
 * out2[0]: milliseconds per launch, out2[1]: algorithmic bytes of one launch.
 * The factors and solve vectors are scratch afterwards (the models' flags,
 * status and pivot counts are kept); time it after a run or restore a
 * snapshot before the next one.  Returns 0, or < 0 on error. */
int fgpu_batch_time_factor(fgpu_batch* b, int reps, double* out2);

/* Launch shapes of the multifrontal kernels, shape4 = {small-front panel
 * factorisation (0: pivot by pivot with shuffles, 1: register-blocked in
 * blocks of 8 pivots, 2: register-blocked in blocks of 4 for fronts of up to
 * 32 rows),
 * warps per block of the forward-elimination cascade (4, 8 or 16), warps per
 * block of the back-substitution queue (4, 8 or 16), blocks per cluster of the
 * large-front factorisation (2, 4, 8, or 16 where the device holds such
 * clusters; else 8 is used)}.  The autotuner picks them before a
 * batch's first batched iteration by timing the candidates on the batch's own
 * fronts (a few milliseconds; a batch of the same structure reuses the
 * choice).  Every shape gives the same results to the last bit, so the
 * timing-dependent choice never changes a result.  set: before the first
 * iteration only, and it replaces the probe.  get: returns 1 once the shapes
 * are chosen (0 before); *probeMs (may be NULL) = wall time of the batch's
 * probe, 0 when set or reused.  No reference counterpart (the reference has
 * no GPU kernels to shape). */
int fgpu_batch_set_launch_shape(fgpu_batch* b, const int* shape4);
int fgpu_batch_launch_shape(fgpu_batch* b, int* shape4, double* probeMs);

/* The linear-solver seam of one model, at the granularity of the reference's
 * csAddEM + csSolve (src/vpmCommon/vpmLinAlg/asmExtensionModule.f90:1227,
 * solExtensionModule.f90:153-505), for a host that drives its own Newton
 * loop and wants the GPU's assembly and sparse LDL^T.  Between the model's
 * time steps only (-2 inside one); the model's next batched iteration starts a
 * step and refactors its own tangent.
 * assemble_newton: N = sM M + sC C + sK K of the model's current state on the
 *   GPU (element matrices in system axes, constraint expansion of joints and
 *   prescribed DOFs as in the batched iteration, CSR in equation order);
 *   fgpu_batch_get_newton_values reads it.
 * factor: LDL^T of N (FP32 fronts for a mixed batch, FP64 otherwise); returns
 *   the number of negative pivots (>= 0), -3 when a pivot is singular
 *   (|d_k| <= 1e-12 |a_kk|, the reference's tolFactorize), < 0 on error.
 * solve: N x = b for nrhs right-hand sides (each neq values in equation order,
 *   overwritten by its solution); a mixed batch refines each solution against
 *   the FP64 N (its solves-per-iteration count). */
int fgpu_batch_assemble_newton(fgpu_batch* b, int model, double sM, double sC, double sK);
int fgpu_batch_factor(fgpu_batch* b, int model);
int fgpu_batch_solve(fgpu_batch* b, int model, double* rhs, int nrhs);

/* Results database of the primary response (the reference's writeSolverDB1,
 * src/vpmSolver/saveModule.f90:615-663, called for the initial configuration
 * and after every time step, solverModule.f90:512-513, :929-931): every model
 * of the batch writes <dir>/model<k>.res, a text header naming the record
 * layout, then one binary record per saved state -- the step number (int32),
 * the time (float64), each triad's position matrix (3 x 4, column by column;
 * the translation only for three-DOF triads), each beam superelement's frame
 * (3 x 4) and each reduced part's frame and generalized DOF values -- in
 * double precision, or single precision when doublePrecision is 0 (the
 * reference's -double1 option).  The first record is the models' current
 * state; then one per completed time step.  Records are packed on the GPU at
 * the end of each step into a small ring in device memory and appended to the
 * files at the next synchronisation point of fgpu_batch_run, fgpu_batch_step
 * or an externally driven iteration.  close flushes and closes the files
 * (also done by fgpu_batch_destroy).  The header layout is this library's own
 * (the reference's lives in a results-database library that is not part of
 * its source tree); the record contents and order follow the reference. */
int fgpu_batch_results_open(fgpu_batch* b, const char* dir, int doublePrecision);
int fgpu_batch_results_close(fgpu_batch* b);

/* Failure-path test hook: runs one warp of the back-substitution queue kernel
 * on a private queue whose only slot is never filled, with a wait limit of
 * `spins` polls (about 32 ns each), so the bounded wait runs out and sets the
 * batch's wait-error flag, which *flag receives (1).  No fault, trap or hang:
 * the kernel returns and the context stays usable.  Every model of the batch
 * still running then fails with status 16 (wait timed out) at its next
 * convergence test, as after a real wait that ran out. */
int fgpu_batch_probe_wait_timeout(fgpu_batch* b, long long spins, int* flag);
/* The same for the other bounded wait of the back substitution: where it runs
 * inside the factorisation's launch, a warp waits for the elimination of the
 * root it takes from the queue.  One warp of that launch, with no leaf to
 * factor, takes a root of the batch's first model from a private queue and
 * waits for a release that nothing makes; the wait runs out after `spins`
 * polls and sets the wait-error flag (*flag = 1).  No front is touched; the
 * running models then fail with status 16 as above. */
int fgpu_batch_probe_root_wait_timeout(fgpu_batch* b, long long spins, int* flag);

/* Measured FP64 fused multiply-add rate of the library's current device:
 * eight independent FMA chains per thread, eight 256-thread blocks per SM,
 * best of five timed launches after three warm-up launches (CUDA events).
 * *tflops: FP64 TFLOP/s (2 flops per FMA); *ms: the best launch's time.
 * Returns 0, or < 0 on error.  The peak that FP64-bound kernels are quoted
 * against. */
int fgpu_measure_fp64_peak(double* tflops, double* ms);

/* Measured TF32 tensor rate of the warp-level mma.sync m16n8k8 instruction
 * (FP32 accumulation) on the library's current device: eight independent
 * accumulator fragments per warp, eight 256-thread blocks per SM, best of
 * five timed launches after three warm-up launches.  *tflops: TF32 TFLOP/s
 * (2 flops per multiply-add; a 3xTF32 split product costs three of them);
 * *ms: the best launch's time.  Returns 0, or < 0 on error.  The peak that
 * the FP32 large-front trailing tiles are quoted against.  No counterpart in
 * the reference (a measurement helper). */
int fgpu_measure_tf32_mma_peak(double* tflops, double* ms);

/* ---- serving: continuous batching of simulation requests ------------------
 * Requests are admitted into new GPU batches (own stream each) as soon as the
 * HBM budget allows, after a short batching window (min_batch requests or
 * max_wait seconds, immediately when the GPU is idle); their work overlaps on
 * the device with the batches already running.  Times are seconds on the
 * server's steady clock (arrival stamped at submit). */
typedef struct fgpu_server fgpu_server;
int fgpu_server_create(double budget_bytes, int mixed, int sweeps, int max_models_per_batch, int min_batch,
                       double max_wait, fgpu_server** out);
void fgpu_server_destroy(fgpu_server* s);
/* the model handle must stay alive until the request finished */
int fgpu_server_submit(fgpu_server* s, fgpu_model* m, int* request_id);
/* one admission/launch/collection pass; returns requests finished in it (< 0 error) */
int fgpu_server_pump(fgpu_server* s);
/* counts: requests, pending, live batches; bytes in use */
int fgpu_server_status(fgpu_server* s, long long* status4);
/* Slot reuse: when this share (0..1) of an engine's models has finished and
 * requests wait, the engine's running models stop at the end of their current
 * step and move, with their whole state, into a new engine together with the
 * waiting requests that fit the freed memory; they continue there exactly as
 * they would have.  share < 0 leaves the setting (default 0.25), 0 disables
 * it.  *rebatches: engines rebuilt this way so far. */
int fgpu_server_slot_reuse(fgpu_server* s, double share, long long* rebatches);
/* At most n engines run at a time (n <= 0: as many as the memory budget allows). */
int fgpu_server_set_max_engines(fgpu_server* s, int n);
double fgpu_server_now(fgpu_server* s);
/* per request: state (0 pending, 1 running, 2 done, 3 failed), arrival, admitted,
 * finished times, Newton iterations, time steps */
int fgpu_server_request(fgpu_server* s, int id, int* state, double* times3, long long* iters, long long* steps);
/* final triad positions of a finished request (12 doubles per triad) */
int fgpu_server_result(fgpu_server* s, int id, double* ur);

/* Text of the last error of this thread. */
const char* fgpu_last_error(void);

#ifdef __cplusplus
}
#endif

#endif
