// engine_dev.cuh -- device-side data layout of the batched FEDEM Newton engine.
//
// All models of a batch live in one set of flat arrays in HBM.  Every object
// class has a global index (triad, DOF, equation, element, CSR slot, front)
// and a reverse map to its model, so that one launch per phase covers every
// model.  Element data are stored entry-major ("SoA"): entry k of element e
// is at [k * nelTot + e], so thread-per-element loads are coalesced.
#pragma once

#include <cstdint>

namespace fgpu {

// per-model state machine
enum ModelState : int { ST_NEED_STEP = 0, ST_ITER = 1, ST_DONE = 2, ST_ERROR = 3 };
// per-model flags for the current batched iteration
enum ModelFlag : int { FL_ACTIVE = 1, FL_PRED = 2, FL_TANGENT = 4, FL_STATIC = 8, FL_REBUILD = 16, FL_STEPDONE = 32 };
// per-model status bits
enum ModelStatus : int { SS_SINGULAR = 1, SS_MAXIT = 2, SS_NAN = 4, SS_COROT = 8, SS_TIMEOUT = 16 };

struct DevModels {
  int n = 0;
  // object ranges
  int *triOff, *ntri, *dofOff, *ndof, *eqOff, *neq, *elOff, *nel;
  // control scalars
  double *time, *dt, *tStart, *tEnd, *minInc, *alpha, *beta, *gamma, *sacc, *svel;
  double *scaleN;   // 3 per model: scale factors the element Newton matrices were built with
  double *pc;       // 4 per model: predictor coefficients DD, DA, AD, AA
  double *gravity;  // 3 per model
  double *wDisp, *wForce;  // 3 per model
  double *tolVal, *normVal;  // 18 per model
  int *tolCode;             // 18 per model
  int *maxIt, *minIt, *fixedIt, *nUpdat, *maxSeq;
  int *state, *flags, *status, *iter, *nSeqNoUpd, *negPiv;
  long long *nStep, *stepLimit, *nIter;
  // static equilibrium
  double *deln, *equTol, *equLim, *staticScale;
  int *staticIter, *staticNinc, *staticDone, *staticMode;  // staticMode: 0 none, 1 linear, 2 iterate
};

struct DevData {
  DevModels m;
  int ntriTot = 0, ndofTot = 0, neqTot = 0, nelTot = 0;
  int64_t nslotTot = 0;
  // triads
  double* ur;            // 12 per triad, column-major 3x4
  int *triFirstDof, *triNdof, *triModel;
  // DOF vectors
  double *urd, *urdd, *dk, *ak, *rinc, *sinc0, *sinc1, *sinc2;
  int *meqn, *dofType, *dofModel;  // meqn: global equation or -1
  // equation vectors
  double *FSk, *FDk, *FIk, *Qk, *qext, *FIact, *res, *del, *xref, *rref;
  float* rhs32;
  int* eqModel;
  // elements (SoA)
  double *K, *M, *C, *N, *fg, *supTr, *triRelSup, *trUnd, *offset, *finit, *finitPrev, *Fel;
  double *stifScl, *kDmp;
  int *elTri, *elRef, *elModel;
  uint8_t *hasC, *hasVld;
  double* elMat;  // rotated element Newton matrices, SoA 144
  // compressed beam matrices (26 upper values of the principal-axes pattern),
  // used by the element pass when every element of the batch has that pattern
  int beamSparse = 0;
  double *K26, *M26, *C26;
  // CSR (full symmetric), global slots; column indices are global equations
  int64_t* rowPtr;  // neqTot + 1
  int* colInd;
  double* csrVal;
  int64_t* slotPtr;
  int64_t* slotSrc;  // SoA index into elMat
  int* slotModel;
  int *eqPtr, *eqSrc;  // eqSrc = local * nelTot + element
  // fronts (global indices)
  int nfrontTot = 0;
  int *fNpiv, *fNrow, *fParent, *fModel, *fNchild, *fNasm;
  int64_t *fRowOff, *fLOff, *fUOff, *fWOff, *fChildOff, *fRelOff, *fAsmOff;
  int *frontRows, *childList, *relIndex;
  int64_t* asmSlot;
  int* asmPos;
  double *L64, *U64;
  float *L32, *U32;
  double* w64;
  float* w32;
  double* x64;  // solve vector, global equations
  float* x32;
  int* errFlag;  // set by a kernel whose bounded wait ran out
  // DOF chunks for the two-stage norm reduction (each chunk within one model)
  int nchunkTot = 0;
  int *chunkModel, *chunkStart, *chunkEnd, *modelChunkOff, *modelNchunk;
  double* partial;  // 21 per chunk
};

}  // namespace fgpu
