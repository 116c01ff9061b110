// host_model.h -- host-side set-up of one FEDEM beam model for the GB300
// solver: input reading, element matrices, SAM numbering, sparsity pattern,
// deterministic gather maps and the multifrontal symbolic analysis.
//
// Everything here runs once per model (set-up); the per-iteration work is in
// engine.cu.  Arrays are flat so they upload to HBM without repacking.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace fgpu {

// Integration and convergence control (initiateSystemTypeModule.f90:41-185,
// normTypeModule.f90:93-193).  Norm test codes: 1 = all-of, 2 = one-of, 0 = off.
struct Control {
  double alpha = -0.1, beta = 0.3025, gamma = 0.6;
  double tStart = 0.0, tEnd = 0.0, tInc = 0.0, minInc = 0.001, maxInc = 0.1;
  int maxIt = 15, minIt = 1, fixedIt = 0, nUpdat = 0, maxSeqNoUpdate = 100;
  int stiffDampFiltering = 1;
  bool initEquilibrium = false;
  double tolInitEquil = 1.0e-3, limInitEquilStep = 1.0;
  double tolFactorize = 1.0e-12;
  // 18 convergence tests: dis[4], vel[4], acc[4], res[4], ener[2] (max, sum)
  int tolCode[18] = {0};
  double tolVal[18] = {0.0};
  double wDisp[3] = {1, 1, 1}, wForce[3] = {1, 1, 1};
  double gravity[3] = {0, 0, 0};
  // quasi-static load steps while time + dt < tQStatic (-quasiStatic; none when <= tStart)
  double tQStatic = -1.0e99;
};

struct Front {            // one supernode of the assembly tree
  int npiv = 0, nrow = 0; // pivots p and front size f (p pivots first)
  int parent = -1;        // front index within the model, -1 for a root
  int height = 0;         // 0 for leaves
  int64_t rowOff = 0;     // offset into frontRows (f entries: equation numbers)
  int64_t lOff = 0;       // offset of the f x p factor block (column-major)
  int64_t uOff = 0;       // offset of the (f-p)^2 update matrix
  int64_t wOff = 0;       // offset of the (f-p) forward-solve update vector
  int64_t childOff = 0;   // offset into childList
  int nchild = 0;
  int64_t relOff = 0;     // offset into relIndex (f-p entries: row in parent front)
  int64_t asmOff = 0;     // offset into asmSlot/asmPos (original entries)
  int nasm = 0;
};

struct HostModel {
  Control ctl;
  // triads (initiateTriadTypeModule.f90): ur is 3x4 column-major
  int ntri = 0;
  std::vector<int> triId, triNdof, triFirstDof;
  std::vector<double> ur;
  // DOFs and equations (samSolverModule.f90:95-250): meqn 0-based, -1 fixed,
  // -2 - k prescribed by motion k
  int ndof = 0, neq = 0;
  std::vector<int> meqn, dofType;
  // beam superelements: matrices column-major 12x12 in superelement axes
  int nel = 0;
  std::vector<int> elId, elTri, elRef, elEq;  // elTri: triad index x2, elRef x3, elEq x12
  std::vector<double> elOffset, supTr, triRelSup, trUnd;  // 9, 12, 12, 24 per element
  std::vector<double> K, M, C, fg;                        // 144, 144, 144, 36 per element
  std::vector<double> stifScl, kDmp;
  std::vector<uint8_t> hasC, hasVld;
  // axial springs (constant stiffness s0, stress-free length l0, stiffness-proportional
  // damping alpha2) and axial dampers (coefficient d0) between two triads, springs first;
  // they act on the translational DOFs (springRoutinesModule.f90, damperRoutinesModule.f90)
  int nax = 0;
  std::vector<uint8_t> axKind;  // 0 spring, 1 damper
  std::vector<int> axTri, axEq; // 2 and 6 per axial element
  std::vector<double> axS0, axL0, axAlpha2, axD0;
  // external point loads in equation order: constant ones summed in qext; loads
  // driven by an engine, F = f0 + f1 * (eA * t + eB), listed per equation in input
  // order (forceRoutinesModule.f90:52-131): equation ldEq[k] gets ldPtr[k]..ldPtr[k+1]
  std::vector<double> qext;
  std::vector<int> ldEq, ldPtr;
  std::vector<double> ldF0, ldF1, ldEA, ldEB;
  std::vector<int> ldCh;  // external channel of the load's engine (value ext[ch] instead of eA t + eB), -1 none
  // a load term whose engine is a SINUSOIDAL function adds mean + amplitude *
  // sin(2 pi (frequency x - delay)), x the time for a TIME sensor, else 0: 4
  // values per load term (frequency (0 without a TIME sensor), delay,
  // amplitude, mean; all 0 for other engines)
  std::vector<double> ldSin;
  // engines: base id, user id, tag, value eA t + eB (+ ext[ch] when ch >= 0), the
  // function (0 none, 1 SCALE fc x, 2 CONSTANT fc, 3 external, 4 SINUSOIDAL) and whether its
  // argument is the time; nExt: external channels used
  std::vector<int> engId, engUserId, engCh, engFType, engTimeArg;
  std::vector<std::string> engTag;
  std::vector<double> engEA, engEB, engFc;
  std::vector<double> engSin;  // 4 per engine: SINUSOIDAL parameters as for ldSin
  int nExt = 0;
  std::vector<double> extInit;  // initial external function values (empty: zero)
  // prescribed deflections (motionRoutinesModule.f90:58-193): D(t) = d0 + d1 * (eA * t + eB)
  // (engine = function of the TIME sensor); a prescribed DOF has meqn = -2 - motion index
  std::vector<int> motDof;
  std::vector<double> motD0, motD1, motEA, motEB;
  std::vector<int> motCh;  // external channel of the motion's engine, -1 none
  // predictor right-hand-side terms of the prescribed DOFs: equation mrEq[k] gets
  // -cc(motion mrMot[q]) * elMat[mrSrc[q]] for q in mrPtr[k]..mrPtr[k+1] (mrSrc = 144*e + entry)
  std::vector<int> mrEq, mrPtr, mrSrc, mrMot;
  // master-slave joints with one master triad (masterSlaveJointTypeModule.f90):
  // the slave triad's 6 DOFs are dependent, u_s = T [u_master; joint DOFs], T
  // (6 x ncol, ncol = nM master DOFs + the joint DOFs) rebuilt from the current
  // geometry after every increment.  Joint DOFs follow all triad DOFs (SAM
  // order).  Per joint: slave and master triad, master DOFs in T (0 for a
  // grounded master), first joint DOF, its DOF count and position-matrix levels,
  // first entry in the per-joint-DOF arrays; joint frame in the master's axes and
  // the slave's start position in the joint frame (3x4 column-major each); the
  // 0-based equation of every column of T (-1 for a fixed DOF).
  int njoint = 0;
  std::vector<int> jSlave, jMaster, jNM, jFirstDof, jNdof, jNmats, jDofOff;
  std::vector<int> jLdof, jImat;      // per joint DOF: 1..6 and level (1-based)
  std::vector<double> jVar0;          // per joint DOF: start value
  std::vector<double> jPosInT, jSTPos0;  // 12 per joint
  std::vector<int> jColEq;            // 12 per joint
  std::vector<int> dofDep;            // per DOF: 6 * joint + row of a dependent DOF, else -1
  // elements with a dependent triad: their DOFs expand through T.  Per such
  // element: the element, its expanded DOF count nx (6 per free triad, ncol per
  // dependent one) and the offsets of its expanded equations (cxEq), of its
  // expanded Newton matrix (nx x nx, column-major) and of its expanded force
  // vectors (FS, FD, FI, Q interleaved, 4 per expanded DOF)
  std::vector<int> cxEl, cxNx, cxEqOff, cxMatOff, cxVecOff, cxEq;
  std::vector<int> elCx;  // per element: its index in cxEl, or -1
  int cxMatSize = 0, cxVecSize = 0;
  // reduced parts (superelements whose K, M and gravity force vectors come from
  // binary matrix files; SupElType with genDOFs): nTri triads with six DOFs and
  // nGen generalized (component-mode) DOFs each, n = 6 nTri + nGen, matrices
  // n x n column-major in part axes.  Generalized DOFs follow all triad DOFs,
  // part by part, and precede the joint DOFs (initSAM_dofStatus).  Per part:
  // triad count, generalized DOF count, first entry in pTri (its triads), the
  // three reference triads (local index), first generalized DOF, offsets of its
  // matrices (n^2 apart), of its DOF vectors (n apart; gravity vectors 3n at
  // 3 * pVecOff) and of its generalized DOF values (pGenOff).  A part's forces
  // and Newton matrix reach the gather maps in expanded form, after the beam
  // elements' in the expanded region: expanded DOFs per triad 6, or its joint's
  // columns when it is dependent, then the generalized DOFs; pXEqOff into cxEq.
  int npart = 0;
  std::vector<int> pNtri, pNgen, pTriOff, pTri, pRef, pGenFirstDof, pGenOff, pVecOff, pXEqOff, pNx, pXMatOff,
      pXVecOff;
  std::vector<int64_t> pMatOff;
  std::vector<double> pOffset, pSupTr, pTriRelSup, pTrUnd;  // 9, 12, 12 per part; 12 per part triad
  std::vector<double> pK, pM, pC, pFg, pStifScl, pKDmp;
  std::vector<uint8_t> pHasC, pHasVld;
  // full symmetric CSR pattern of the Newton matrix, equation order
  std::vector<int> rowPtr, colInd;
  // deterministic gather maps: CSR slot <- (element, entry); equation <- (element, local dof)
  // (axial elements follow the beams: slotSrc = 144*nel + 36*axial + entry,
  // eqSrc = 12*nel + 6*axial + local, mrSrc like slotSrc)
  // (expanded elements follow the axial ones: slotSrc = 144*nel + 36*nax +
  // cxMatOff + p + nx*q, eqSrc = 12*nel + 6*nax + cxVecOff + 4*p)
  std::vector<int> slotPtr, slotSrc;   // slotSrc = 144*element + entry
  std::vector<int> eqPtr, eqSrc;       // eqSrc = 12*element + local dof
  // multifrontal symbolic factorisation
  std::vector<Front> fronts;
  std::vector<int> frontRows, childList, relIndex, asmSlot, asmPos;
  int maxHeight = 0, maxFront = 0;
  int64_t lSize = 0, uSize = 0, wSize = 0;
  std::vector<int> perm;  // elimination position -> equation
};

// Parses the solver-input text and command-line options; returns 0 or < 0.
int buildModel(const char* fsi, int argc, const char* const* argv, HostModel& m, std::string& err);
// Nested-dissection ordering, assembly tree and front maps (symbolic.cpp).
int symbolicAnalysis(HostModel& m, std::string& err);

}  // namespace fgpu
