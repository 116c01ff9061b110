/*
 * fedem_oracle.h -- C interface of the CPU oracle for the FEDEM implicit
 * HHT-alpha/Newmark Newton time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker that the CUDA
 * solver is compared against, and the timed CPU baseline.  Nothing in the
 * product library links or calls it.
 *
 * The oracle restates, in plain FP64 C++, the reference algorithm of
 *   src/vpmSolver/newmarkRoutinesModule.f90   (NewmarkInt, PredictVelAcc, IncVelAcc)
 *   src/vpmSolver/supElRoutinesModule.f90     (UpdateSupEls, BuildSupNewtonMat, AddInSupMat)
 *   src/vpmCommon/supElTypeModule.f90         (updateSupElCorot, BuildFinit)
 *   src/vpmSolver/staticEquilibriumModule.f90 (staticEquilibrium)
 *   src/Femlib/beam.f, src/Femlib/beamaux.f   (BEAM31, BELS31, BEAM35, DCOS30, MPRO30, TRIX30)
 * with a skyline (profile) LDL^T in place of the absent SAM/SPR solver.
 */
#ifndef FEDEM_ORACLE_H
#define FEDEM_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct OracleModel OracleModel;

/* Parses the model text (solver input file subset) and the command-line style
 * options, sets up the model and runs the initial static equilibrium when
 * -initEquilibrium is given.  Returns NULL and a negative *ierr on failure. */
OracleModel* oracle_create(const char* fsi, int argc, const char* const* argv, int* ierr);
void oracle_destroy(OracleModel* m);

/* Advances one time step (one NewmarkInt call).  Returns 1 while more steps
 * remain, 0 when the end time was reached or on error (*ierr != 0). */
int oracle_solve_next(OracleModel* m, int* ierr);

/* Triad position (ur(:,4)) of the triad with the given id; returns 3, or 0. */
int oracle_get_state_var(OracleModel* m, int id, double* var);
double oracle_get_time(OracleModel* m);

/* Sizes: ndof = total DOFs, neq = number of equations (free DOFs). */
int oracle_get_ndof(OracleModel* m);
int oracle_get_neq(OracleModel* m);
int oracle_get_ntriads(OracleModel* m);
int oracle_get_nelements(OracleModel* m);
/* Equation number (1-based, 0 = fixed) of every DOF, DOF order. */
int oracle_get_meqn(OracleModel* m, int* meqn);
/* All triad position matrices, 12 doubles (3x4 column-major) per triad. */
int oracle_get_triad_ur(OracleModel* m, double* ur);
/* Largest triad displacement from the start positions at the end of any
 * step so far: the response scale of the run, for relative errors. */
double oracle_get_max_displacement(OracleModel* m);
/* Total Newton iterations done so far in the time integration. */
long long oracle_get_iterations(OracleModel* m);
/* Newton iterations in the last step and the last iteration norms
 * (displacement, velocity, acceleration, residual). */
int oracle_get_last_norms(OracleModel* m, double* norms4);

/* Upper-triangle CSR pattern of the Newton matrix in equation order
 * (0-based): rowptr[neq+1], cols[nnz].  Returns nnz (call with NULL to size). */
int oracle_get_csr_pattern(OracleModel* m, int* rowptr, int* cols);
/* Assembles the Newton matrix sM*M + sC*C + sK*K at the current configuration
 * into the upper CSR pattern above.  Returns nnz. */
int oracle_assemble_newton(OracleModel* m, double sM, double sC, double sK, double* values);
/* Element n x n matrices (column-major, superelement axes): 0=K, 1=M, 2=C.
 * Returns n * n. */
int oracle_get_element_matrix(OracleModel* m, int iel, int which, double* mat);
/* DOFs of element iel: 6 per triad, then its generalized DOFs. */
int oracle_get_element_size(OracleModel* m, int iel);
/* Generalized DOF values of element iel; returns their number. */
int oracle_get_gen_dofs(OracleModel* m, int iel, double* v);
/* System force vectors in equation order: 0=FS, 1=FD, 2=FI, 3=Q. */
int oracle_get_force_vector(OracleModel* m, int which, double* vec);

#ifdef __cplusplus
}
#endif

#endif
