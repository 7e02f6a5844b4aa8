/* Stand-in for the four UMFPACK calls made by the reference's Poisson solver
 * (fields.cpp:273-275, 311, 347, 352, 364), for the oracle build only.
 *
 * SuiteSparse is not in the reference tree and its version is unpinned
 * (INSTALL:10).  The reference assembles its 5-point operator in CSC arrays
 * filled row by row and solves with UMFPACK_At, i.e. it solves the
 * row-stencil system S u = b with S = (CSC matrix)^T.  This stand-in builds S
 * from the same arrays and factors it with a banded LU (no pivoting; S is a
 * weakly diagonally dominant M-matrix for every geometry the reference
 * builds).  Solve times measured with it are this banded LU's, not UMFPACK's.
 */
#ifndef ORACLE_UMFPACK_SHIM_H
#define ORACLE_UMFPACK_SHIM_H
#ifdef __cplusplus
extern "C" {
#endif

#define UMFPACK_A 0
#define UMFPACK_At 1
#define UMFPACK_OK 0
#define UMFPACK_ERROR_invalid_system -13

int umfpack_di_symbolic(int n_row, int n_col, const int* Ap, const int* Ai,
                        const double* Ax, void** Symbolic,
                        const double* Control, double* Info);
int umfpack_di_numeric(const int* Ap, const int* Ai, const double* Ax,
                       void* Symbolic, void** Numeric,
                       const double* Control, double* Info);
int umfpack_di_solve(int sys, const int* Ap, const int* Ai, const double* Ax,
                     double* X, const double* B, void* Numeric,
                     const double* Control, double* Info);
void umfpack_di_free_symbolic(void** Symbolic);
void umfpack_di_free_numeric(void** Numeric);

#ifdef __cplusplus
}
#endif
#endif
