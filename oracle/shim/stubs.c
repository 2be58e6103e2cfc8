/* Link stubs for off-path CBLAS / LAPACKE routines that the reference's
 * lib/src/vsmc_rng.cpp pulls in through rng/normal_mv_distribution.hpp.  The
 * particle-filter path never calls them; calling one aborts. */
#include <stdlib.h>
#include "cblas.h"
#include "lapacke.h"

void cblas_ssyr(const enum CBLAS_LAYOUT a, const enum CBLAS_UPLO b, const int c,
    const float d, const float *e, const int f, float *g, const int h)
{ (void)a; (void)b; (void)c; (void)d; (void)e; (void)f; (void)g; (void)h; abort(); }
void cblas_dsyr(const enum CBLAS_LAYOUT a, const enum CBLAS_UPLO b, const int c,
    const double d, const double *e, const int f, double *g, const int h)
{ (void)a; (void)b; (void)c; (void)d; (void)e; (void)f; (void)g; (void)h; abort(); }
void cblas_ssyrk(const enum CBLAS_LAYOUT a, const enum CBLAS_UPLO b,
    const enum CBLAS_TRANSPOSE c, const int d, const int e, const float f,
    const float *g, const int h, const float i, float *j, const int k)
{ (void)a; (void)b; (void)c; (void)d; (void)e; (void)f; (void)g; (void)h; (void)i; (void)j; (void)k; abort(); }
void cblas_dsyrk(const enum CBLAS_LAYOUT a, const enum CBLAS_UPLO b,
    const enum CBLAS_TRANSPOSE c, const int d, const int e, const double f,
    const double *g, const int h, const double i, double *j, const int k)
{ (void)a; (void)b; (void)c; (void)d; (void)e; (void)f; (void)g; (void)h; (void)i; (void)j; (void)k; abort(); }
void cblas_stpmv(const enum CBLAS_LAYOUT a, const enum CBLAS_UPLO b,
    const enum CBLAS_TRANSPOSE c, const enum CBLAS_DIAG d, const int e,
    const float *f, float *g, const int h)
{ (void)a; (void)b; (void)c; (void)d; (void)e; (void)f; (void)g; (void)h; abort(); }
void cblas_dtpmv(const enum CBLAS_LAYOUT a, const enum CBLAS_UPLO b,
    const enum CBLAS_TRANSPOSE c, const enum CBLAS_DIAG d, const int e,
    const double *f, double *g, const int h)
{ (void)a; (void)b; (void)c; (void)d; (void)e; (void)f; (void)g; (void)h; abort(); }
void cblas_strmm(const enum CBLAS_LAYOUT a, const enum CBLAS_SIDE b,
    const enum CBLAS_UPLO c, const enum CBLAS_TRANSPOSE d, const enum CBLAS_DIAG e,
    const int f, const int g, const float h, const float *i, const int j, float *k,
    const int l)
{ (void)a; (void)b; (void)c; (void)d; (void)e; (void)f; (void)g; (void)h; (void)i; (void)j; (void)k; (void)l; abort(); }
void cblas_dtrmm(const enum CBLAS_LAYOUT a, const enum CBLAS_SIDE b,
    const enum CBLAS_UPLO c, const enum CBLAS_TRANSPOSE d, const enum CBLAS_DIAG e,
    const int f, const int g, const double h, const double *i, const int j, double *k,
    const int l)
{ (void)a; (void)b; (void)c; (void)d; (void)e; (void)f; (void)g; (void)h; (void)i; (void)j; (void)k; (void)l; abort(); }
lapack_int LAPACKE_spptrf(int a, char b, lapack_int c, float *d)
{ (void)a; (void)b; (void)c; (void)d; abort(); }
lapack_int LAPACKE_dpptrf(int a, char b, lapack_int c, double *d)
{ (void)a; (void)b; (void)c; (void)d; abort(); }
lapack_int LAPACKE_spotrf(int a, char b, lapack_int c, float *d, lapack_int e)
{ (void)a; (void)b; (void)c; (void)d; (void)e; abort(); }
lapack_int LAPACKE_dpotrf(int a, char b, lapack_int c, double *d, lapack_int e)
{ (void)a; (void)b; (void)c; (void)d; (void)e; abort(); }
