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

constexpr int kSlotBlock = 256;  // CSR slots per block of the slot gather

// per-model state machine
enum ModelState : int { ST_NEED_STEP = 0, ST_ITER = 1, ST_DONE = 2, ST_ERROR = 3 };
// per-model flags for the current batched iteration
// FL_QSTATIC: a quasi-static load step (staticInt), FL_LINEAR: pure linear one
// (numit = -1, restarted from the initial state), FL_QS2DYN: first dynamic step
// after quasi-static ones (starting velocity rinc / dt)
enum ModelFlag : int {
  FL_ACTIVE = 1, FL_PRED = 2, FL_TANGENT = 4, FL_STATIC = 8, FL_REBUILD = 16, FL_STEPDONE = 32,
  FL_QSTATIC = 64, FL_LINEAR = 128, FL_QS2DYN = 256
};
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
  double *sumWd2, *sumWf2;   // sums of the squared displacement / force weights over the free DOFs
  int *tolCode;             // 18 per model
  int *maxIt, *minIt, *fixedIt, *nUpdat, *maxSeq;
  int *state, *flags, *status, *iter, *nSeqNoUpd, *negPiv;
  long long *nStep, *stepLimit, *nIter;
  // quasi-static load steps while time + dt < tQs; qsCount: such steps since the last dynamic one
  double* tQs;
  int* qsCount;
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
  int *meqn, *dofType, *dofModel;  // meqn: global equation, -1 fixed, -2 - k prescribed by model motion k
  // equation vectors
  double *FSk, *FDk, *FIk, *Qk, *qext, *FIact, *res, *del, *xref, *rref;
  // forces set by an external process for the iterations of the current step
  // (added to Q in the corrector residuals, cleared by the next predictor)
  double* extRhs;
  float* rhs32;
  int* eqModel;
  // elements (SoA)
  double *K, *M, *C, *N, *fg, *supTr, *triRelSup, *trUnd, *offset, *finit, *finitPrev, *Fel;
  double *stifScl, *kDmp;
  int *elTri, *elRef, *elModel;
  uint8_t *hasC, *hasVld;
  double* elMat;  // rotated element Newton matrices, SoA 144 (entry i + 12 j of element e at (i + 12 j) * nelTot + e)
  // compressed beam matrices (26 upper values of the principal-axes pattern),
  // used by the element pass when every element of the batch has that pattern
  int beamSparse = 0;
  double *K26, *M26, *C26;
  // CSR (full symmetric), global slots; column indices are global equations
  int64_t* rowPtr;  // neqTot + 1
  int* colInd;
  double* csrVal;
  int* slotPtr;      // 32-bit: a batch keeps its slot contributions below 2^31
  int* slotSrc;      // index into elMat (elMatA above 144 * nelTot)
  int* slotModel;
  int* slotBlockModel;  // per block of kSlotBlock slots: their model, or -1 when they span several
  int *eqPtr, *eqSrc;  // eqSrc = local * nelTot + element
  // fronts (global indices)
  int nfrontTot = 0;
  int *fNpiv, *fNrow, *fParent, *fModel, *fNchild, *fNasm;
  int64_t *fRowOff, *fLOff, *fUOff, *fWOff, *fChildOff, *fRelOff, *fAsmOff;  // fUOff: the front's packed
                                                                            // update matrix in its parent's segment
  int *frontRows, *childList, *relIndex;
  // large fronts (one thread block each) and every front's number of large children
  uint8_t* fLarge;
  int* fNlarge;
  // children's update rows of each front, in child order: W index and
  // (child ordinal << 16 | destination row), cgOff[f]..cgOff[f+1]
  int *cgOff, *cgSrc, *cgDst;
  int64_t* asmSlot;
  int* asmPos;
  // the original entries again in front-assembly order, written with the CSR
  // values (slotAsm[s]: assembly index of CSR slot s, or -1), in the factor precision
  int* slotAsm;
  float* asmVal32;
  double* asmVal64;
  // children's update matrices, lower triangles packed column by column, one
  // contiguous segment per parent front in child order: fSegOff/fSegLen, and
  // for each segment entry (child ordinal << 20 | position in the parent front)
  int64_t* fSegOff;
  int* fSegLen;
  int* segPos;
  double *L64, *U64;
  float *L32, *U32;
  double* w64;
  float* w32;
  double* x64;  // solve vector, global equations
  float* x32;
  int* errFlag;  // set by a kernel whose bounded wait ran out
  // engine-driven point loads: equation ldEq[k] holds qextBase (its constant loads)
  // + sum over ldPtr[k]..ldPtr[k+1] of f0 + f1 * (eA * t + eB), refreshed in qext at step start
  int nldTot = 0;
  int *ldEq, *ldPtr;
  double *ldF0, *ldF1, *ldEA, *ldEB, *qextBase;
  double* ldSin;  // 4 per load term: SINUSOIDAL frequency, delay, amplitude, mean (zeros otherwise)
  // external functions: a load term or motion whose engine is one (ldCh / motCh
  // >= 0, a global channel) takes extVal[ch] instead of eA * t + eB
  int* ldCh;
  int nextTot = 0;
  double* extVal;
  // axial springs and dampers (SoA): kind (0 spring, 1 damper), triads [k * naxTot + a],
  // model, constants; current direction axN (3) and length; element forces FelA
  // (FS 6, FD 6) and Newton matrices elMatA (6x6, translational DOFs of both triads).
  // Gather sources: eqSrc >= 12 * nelTot and slotSrc/mrSrc >= 144 * nelTot address
  // FelA / elMatA with that offset removed.
  int naxTot = 0;
  uint8_t* axKind;
  int *axTri, *axModel;
  double *axS0, *axL0, *axAlpha2, *axD0, *axN, *axLen, *FelA, *elMatA;
  // prescribed deflections: D(t) = d0 + d1 * (eA * t + eB); cc = constraint value of the
  // current step (increment, or total in linear quasi-static steps)
  int nmotTot = 0;
  int *motModel, *modelMotOff;
  double *motD0, *motD1, *motEA, *motEB, *motD, *motCc;
  int* motCh;
  // predictor right-hand-side terms: del[mrEq[k]] -= cc[mrMot[q]] * elMat[mrSrc[q]]
  int nmrTot = 0;
  int *mrEq, *mrMot;
  int64_t *mrPtr, *mrSrc;
  // state linear quasi-static steps restart from (null when no model has such steps)
  double *urQs, *supTrQs, *urdQs, *urddQs;
  // iterations of a pure linear step: 1 with FP64 solves; with FP32 solves the
  // single reference solve is followed by corrections against the FP64 residual
  // Q - FS (iterative refinement of the same linear system)
  int linearIters = 1;
  // sin(5e-4) / 5e-4 for the small-angle branch of the rotation update
  double sinEpsOverEps = 1.0;
  // master-slave joints (one master triad each; see host_model.h): slave and
  // master triad, master DOFs in T, columns of T, first joint DOF, joint DOF
  // count, position-matrix levels, first entry in the per-joint-DOF arrays,
  // model; joint frame in the master's axes and the slave's start position in
  // the joint frame (12 each); constraint coefficients T (6 rows x 12 columns
  // per joint, row-major) and the global equation of each column (12, -1 fixed)
  int njointTot = 0;
  int *jSlave, *jMaster, *jNM, *jNcol, *jFirstDof, *jNdof, *jNmats, *jDofOff, *jModel;
  int *jLdof, *jImat;  // per joint DOF: 1..6 and level (1-based)
  double* jVar;        // per joint DOF: current value
  double *jPosInT, *jSTPos0, *jT;
  int* jColEq;
  int* dofDep;  // per DOF: 6 * joint + row of a dependent DOF, else -1 (null without joints)
  // elements with a dependent triad: their element, expanded DOF count, offsets
  // of the expanded Newton matrix (elMatX, nx x nx column-major) and of the
  // expanded forces (FelX: FS, FD, FI, Q interleaved per expanded DOF), and per
  // node the joint whose dependent triad it is (-1 for a free triad).  Gather
  // sources at or above 144 * nelTot + 36 * naxTot (matrix) and 12 * nelTot +
  // 6 * naxTot (forces) address these with that offset removed.
  int ncxTot = 0;
  int *cxEl, *cxNx, *cxMatOff, *cxVecOff, *cxNode;
  double *elMatX, *FelX;
  // reduced parts (one thread block each): model, DOF count n (6 per triad,
  // then the generalized DOFs), triad count, generalized DOF count, first entry
  // of their triads (pTri: triad, pTriJoint: joint whose dependent triad it is
  // or -1; pTrUnd: 12 per part triad), reference triads (3, local index),
  // first generalized DOF (global), first generalized value (pGen), offsets of
  // the DOF vectors (pFinit, pFinitPrev: n apart; pFg: 3 n at 3 * pVecOff) and
  // of the matrices (pK, pM, pC: n^2 apart), the expanded DOF count and the
  // expanded matrix and force offsets in elMatX / FelX.  12 per part: frame
  // pSupTr, pTriRelSup; 9: reference-point offsets.
  int npartTot = 0, partMaxN = 0, partMaxNx = 0;
  int *pModel, *pN, *pNtri, *pNgen, *pTriOff, *pTri, *pTriJoint, *pRef, *pGenFirstDof, *pGenOff, *pVecOff, *pNx,
      *pXMatOff, *pXVecOff;
  int64_t* pMatOff;
  double *pOffset, *pSupTr, *pTriRelSup, *pTrUnd, *pK, *pM, *pC, *pFg, *pStifScl, *pKDmp, *pFinit, *pFinitPrev,
      *pGen;
  uint8_t *pHasC, *pHasVld;
  // DOF chunks for the two-stage norm reduction (each chunk within one model)
  int nchunkTot = 0;
  int *chunkModel, *chunkStart, *chunkEnd, *modelChunkOff, *modelNchunk;
  double* partial;  // 21 per chunk
};

}  // namespace fgpu
