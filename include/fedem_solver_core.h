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
 * getStateVar, getTime, getSystemSize, getEquations, getSystemMatrix with
 * iMat = 0, getNewtonMatrix, getRhsVector, getElementStiffnessMatrix,
 * solverDone, solverClose).  Entry points for features outside that path
 * (restart state, windowed stepping with external functions, eigenmodes,
 * inverse analysis, strain/beam-force recovery, externally driven iterations)
 * exist so the library loads as a drop-in, and return the reference's failure
 * value (false, 0 or a negative status, with *ierr = -1 where present).
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
 * -initEquilibrium is given.  Returns >= 0 on success, < 0 on error.
 * Extra option understood here: -gpuMixed (FP32 factor + FP64 refinement). */
int solverInit(int argc, char** argv, const char* cfsi, const double* stateData, int ndat,
               const double* gagesData, int ngda, const double* extInput, int* nxinp);

/* solverInterface.h:87 -- in-core restart: unsupported, returns -1. */
int restartFromState(const double* stateData, const int ndat, const int writeToRDB);

/* solverInterface.h:110 -- windowed stepping with external inputs: unsupported. */
bool solveWindow(int nStep, int nInc, int nIn, int nOut, const int* fOut, const double* times,
                 const double* inputs, double* outputs, int nDat, double* stateData, int* ierr);

/* solverInterface.h:118-144 -- state vector sizes: no restart state, returns 0. */
int getStateSize(void);
int getTransformationStateSize(void);
int getPartDeformationStateSize(int bid);
int getPartStressStateSize(int bid);
int getGagesSize(void);

/* solverInterface.h:156-170, :226-238 -- state saving: unsupported, returns false. */
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

/* solverInterface.h:247 -- advances one time step on the GPU.  Returns false
 * at the end of the simulation or on error; *ierr != 0 tells them apart. */
bool solveNext(int* ierr);

/* solverInterface.h:262, :278 -- externally driven Newton iterations: unsupported. */
bool startStep(int* ierr);
bool solveIteration(int* ierr, bool all);

/* solverInterface.h:293, :309 -- eigenmodes and inverse analysis: unsupported. */
bool solveEigenModes(const int nmod, double* eval, double* evec, bool dofOrder, int useLaPack, int* ierr);
bool solveInverse(const double* x, const int* xeqs, const int* feqs, int ndis, int nfrs, int* ierr);

/* solverInterface.h:323 -- releases the model and the GPU memory; returns 0. */
int solverDone(bool removeSingletons);
/* solverInterface.h:330 */
void solverClose(void);

/* solverInterface.h:342 -- external function values: unsupported, returns false. */
bool setExtFunc(int funcId, double value);
/* solverInterface.h:349 -- current (or next) physical time. */
double getTime(bool nextStep, int* ierr);
/* solverInterface.h:355 -- unsupported, returns false. */
bool setTime(double nextTime);
/* solverInterface.h:361, :369 */
static inline double getCurrentTime(int* ierr) { return getTime(false, ierr); }
static inline double getNextTime(int* ierr) { return getTime(true, ierr); }
/* solverInterface.h:383 -- general functions: unsupported, *ierr = -1. */
double evalFunc(int uid, const char* tag, double x, int* ierr);
/* solverInterface.h:398 -- unsupported, returns -1. */
int getFuncId(const char* tag);

/* solverInterface.h:407 -- 1-based equation numbers of the DOFs of the triad
 * with base id bid (0 for a fixed DOF); returns the number of DOFs. */
int getEquations(int bid, int* meqn);
/* solverInterface.h:420 -- triad position (3 values); returns 3, or 0. */
int getStateVar(int bid, double* var);
/* solverInterface.h:426 -- number of equations (dofs = false) or DOFs. */
int getSystemSize(bool dofs);
/* solverInterface.h:433 -- dense column-major neq x neq matrix; iMat = 0
 * (Newton matrix of the last tangent update) is supported. */
bool getSystemMatrix(double* Smat, int iMat);
/* solverInterface.h:439-457 */
bool getNewtonMatrix(double* Nmat);
bool getStiffnessMatrix(double* Kmat);
bool getMassMatrix(double* Mmat);
bool getDampingMatrix(double* Cmat);
/* solverInterface.h:465 -- 12x12 beam stiffness in element axes. */
bool getElementStiffnessMatrix(double* Kmat, int bid);
/* solverInterface.h:472 -- iVec = 0: the current right-hand side (residual). */
bool getRhsVector(double* Rvec, int iVec);
/* solverInterface.h:478, :484 -- unsupported (needs startStep), returns false. */
bool setRhsVector(const double* Rvec);
bool addRhsVector(const double* Rvec);
/* solverInterface.h:491 -- unsupported, returns false. */
bool getJointSprCoeff(double* sprCoeff, int bid);

#ifdef __cplusplus
}
#endif

#endif
