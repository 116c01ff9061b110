/*
 * fedem_solver_core.h -- the drop-in C ABI of the GB300 FEDEM dynamics solver
 * core (library libfedem_solver_core.so).
 *
 * Every entry point keeps the name, signature, argument meaning and return
 * convention of the reference's src/vpmSolver/solverInterface.h (cited per
 * declaration), so that fedempy (PythonAPI/src/fedempy/solver.py:154-191,
 * ctypes.cdll.LoadLibrary + restype setup) loads this library unchanged.
 *
 * Like the reference, this ABI drives ONE model per process (a process-wide
 * singleton, not thread safe).  The batched, many-model API is fgpu.h.
 *
 * Hot path implemented on the GPU: initial static equilibrium and the
 * HHT-alpha Newton time steps of beam models (solverInit, solveNext,
 * startStep, solveIteration, setTime, getStateVar, getTime, getSystemSize,
 * getEquations, getSystemMatrix, getNewtonMatrix, getStiffness/Mass/
 * DampingMatrix, get/set/addRhsVector, getElementStiffnessMatrix, in-core
 * state save and restart, external functions (setExtFunc, evalFunc,
 * getFuncId, solveWindow), eigenmodes (solveEigenModes), solverDone,
 * solverClose).  Entry points for features
 * outside that path (inverse analysis, strain/beam-force recovery, part and
 * gauge states) exist
 * so the library loads as a drop-in, and return the reference's failure value
 * (false, 0 or a negative status, with *ierr = -1 where present).
 */
#ifndef FEDEM_SOLVER_CORE_H
#define FEDEM_SOLVER_CORE_H

#include <stdbool.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* solverInterface.h:65 -- reads the model (cfsi text, or -fsifile=<path> in
 * argv), sets it up on the GPU and solves the initial equilibrium when
 * -initEquilibrium is given; with stateData (ndat >= getStateSize()) the
 * state saved by saveState for the same model is restored afterwards.
 * Returns >= 0 on success, < 0 on error.
 * Extra option understood here: -gpuMixed (FP32 factor + FP64 refinement). */
int solverInit(int argc, char** argv, const char* cfsi, const double* stateData, int ndat,
               const double* gagesData, int ngda, const double* extInput, int* nxinp);

/* solverInterface.h:87 -- in-core restart: restores a saveState array of the
 * current model (positions, velocities, accelerations, element frames and
 * forces, time, step counters); writeToRDB is ignored (no results database).
 * Returns 0, or < 0 when there is no model or ndat < getStateSize(). */
int restartFromState(const double* stateData, const int ndat, const int writeToRDB);

/* solverInterface.h:110 -- nStep steps; before each, the step time (times,
 * when nInc >= nStep) and the values of external function channels 1..nIn
 * (inputs, nIn per step) are applied; after each, the engines with user ids
 * fOut are evaluated into outputs (nOut per step); with nDat > 0 the state is
 * saved into stateData at the end.  False at the end of the simulation or on
 * error (*ierr != 0; nInc - nStep for a too short times array). */
bool solveWindow(int nStep, int nInc, int nIn, int nOut, const int* fOut, const double* times,
                 const double* inputs, double* outputs, int nDat, double* stateData, int* ierr);

/* solverInterface.h:118 -- doubles saveState needs; :124-144 (transformation,
 * part and gauge states, not kept by this solver) return 0. */
int getStateSize(void);
int getTransformationStateSize(void);
int getPartDeformationStateSize(int bid);
int getPartStressStateSize(int bid);
int getGagesSize(void);

/* solverInterface.h:156 -- the solver state between steps into stateData;
 * false within a started step or when ndat < getStateSize().
 * :162-170, :226-238 (transformation, gauge and part states): false. */
bool saveState(double* stateData, const int ndat);
bool saveTransformationState(double* stateData, const int ndat);
bool saveGages(double* stateData, const int ndat);
bool savePartDeformationState(int bid, double* stateData, const int ndat);
bool savePartStressState(int bid, double* stateData, const int ndat);

/* solverInterface.h:180-213 -- recovery from a given displacement field: unsupported. */
bool getStrainsFromDisp(const double* disp, const int* gageIDs, double* eps, const int ndof, const int nGage);
bool getBeamForcesFromDisp(const double* disp, const int* beamIDs, double* forces, const int ndof,
                           const int nBeam);
bool getRelDisp(const double* disp, const int* Ids, double* relDis, const int ndof, const int nId);
bool getRespVars(const double* disp, const int* Ids, double* resVar, const int ndof, const int nId);

/* solverInterface.h:247 -- advances one time step on the GPU (or completes
 * the step startStep began).  Returns false at the end of the simulation or
 * on error; *ierr != 0 tells them apart. */
bool solveNext(int* ierr);

/* solverInterface.h:262 -- predictor of the next step and its first linear
 * system (Newton matrix and right-hand side), which get/set/addRhsVector and
 * getNewtonMatrix then see.  False at the end of the simulation or on error
 * (*ierr = -999 when a step is already started).
 * solverInterface.h:278 -- solves the assembled system, updates the state and
 * assembles the next iteration; returns false when the step has converged
 * (all = false) or, with all = true (iterate to convergence), at the end of
 * the simulation; on error false with *ierr != 0 (-999: no step started). */
bool startStep(int* ierr);
bool solveIteration(int* ierr, bool all);

/* solverInterface.h:293 -- the nmod lowest eigenmodes of K phi = lambda M phi at
 * the current state (Lanczos on the GPU-factored stiffness matrix): eval in Hz
 * (sqrt|lambda| / 2 pi), evec M-orthonormal, nmod columns in equation order or
 * (dofOrder) DOF order.  *ierr = number of negative eigenvalues (+1 when the
 * iteration did not converge every mode), < 0 on error; useLaPack is ignored.
 * Between steps only.
 * solverInterface.h:309 -- inverse analysis: unsupported. */
bool solveEigenModes(const int nmod, double* eval, double* evec, bool dofOrder, int useLaPack, int* ierr);
bool solveInverse(const double* x, const int* xeqs, const int* feqs, int ndis, int nfrs, int* ierr);

/* solverInterface.h:323 -- releases the model and the GPU memory; returns 0. */
int solverDone(bool removeSingletons);
/* solverInterface.h:330 */
void solverClose(void);

/* solverInterface.h:342 -- value of external function channel funcId
 * (1-based: a DEVICE_FUNCTION without a file and with that channel) for the
 * next step; false when the model has no such channel. */
bool setExtFunc(int funcId, double value);
/* solverInterface.h:349 -- current (or next) physical time. */
double getTime(bool nextStep, int* ierr);
/* solverInterface.h:355 -- time of the next step: increment nextTime - time,
 * raised to the minimum increment; false for a negative increment or within
 * a started step. */
bool setTime(double nextTime);
/* solverInterface.h:361, :369 */
static inline double getCurrentTime(int* ierr) { return getTime(false, ierr); }
static inline double getNextTime(int* ierr) { return getTime(true, ierr); }
/* solverInterface.h:383 -- value of the engine with user id uid, or with a tag
 * of the first engine with that tag (a user id match wins, no match gives 0);
 * x >= 0 (without a tag) evaluates the engine's function at x.  Engines of
 * SCALE, CONSTANT and external functions of the TIME sensor (or none). */
double evalFunc(int uid, const char* tag, double x, int* ierr);
/* solverInterface.h:398 -- user id of the first engine with the tag, -1 if none. */
int getFuncId(const char* tag);

/* solverInterface.h:407 -- 1-based equation numbers of the DOFs of the triad
 * with base id bid (0 for a fixed DOF); returns the number of DOFs. */
int getEquations(int bid, int* meqn);
/* solverInterface.h:420 -- triad position (3 values); returns 3, or 0. */
int getStateVar(int bid, double* var);
/* solverInterface.h:426 -- number of equations (dofs = false) or DOFs. */
int getSystemSize(bool dofs);
/* solverInterface.h:433 -- dense column-major neq x neq matrix: iMat = 0 the
 * Newton matrix of the last tangent update, 1 stiffness, 2 mass, 3 damping at
 * the current configuration (element matrices rotated with the current frames,
 * axial spring/damper blocks included). */
bool getSystemMatrix(double* Smat, int iMat);
/* solverInterface.h:439-457 -- getSystemMatrix with iMat = 0, 1, 2, 3 */
bool getNewtonMatrix(double* Nmat);
bool getStiffnessMatrix(double* Kmat);
bool getMassMatrix(double* Mmat);
bool getDampingMatrix(double* Cmat);
/* solverInterface.h:465 -- 12x12 beam stiffness in element axes. */
bool getElementStiffnessMatrix(double* Kmat, int bid);
/* solverInterface.h:472 -- iVec < 5: the right-hand side of the current
 * linear system, 5: the external force vector Q. */
bool getRhsVector(double* Rvec, int iVec);
/* solverInterface.h:478, :484 -- replaces / adds to the right-hand side of the
 * system assembled by startStep or solveIteration.  Given in the first
 * iteration of a step, the vector is also applied as external forces in the
 * step's later iterations (the reference's keepDuringIterations).  False
 * outside a started step. */
bool setRhsVector(const double* Rvec);
bool addRhsVector(const double* Rvec);
/* solverInterface.h:491 -- unsupported, returns false. */
bool getJointSprCoeff(double* sprCoeff, int bid);

#ifdef __cplusplus
}
#endif

#endif
