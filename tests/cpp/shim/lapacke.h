/* Declarations-only LAPACKE stand-in so the reference's math/math.hpp parses
 * when compiled as the oracle.  Nothing on the filter path calls LAPACK
 * (only utility/covariance.hpp and rng/normal_mv_distribution.hpp do). */
#ifndef VSMC_ORACLE_SHIM_LAPACKE_H
#define VSMC_ORACLE_SHIM_LAPACKE_H

#define LAPACK_ROW_MAJOR 101
#define LAPACK_COL_MAJOR 102
typedef int lapack_int;

#ifdef __cplusplus
extern "C" {
#endif
lapack_int LAPACKE_spptrf(int, char, lapack_int, float *);
lapack_int LAPACKE_dpptrf(int, char, lapack_int, double *);
lapack_int LAPACKE_spotrf(int, char, lapack_int, float *, lapack_int);
lapack_int LAPACKE_dpotrf(int, char, lapack_int, double *, lapack_int);
#ifdef __cplusplus
}
#endif

#endif
