/* Minimal CBLAS stand-in for compiling the reference's headers: the oracle's
 * reference build (oracle/Makefile) and the Sampler<T> programs of
 * tests/cpp.  No system CBLAS exists on either machine.
 *
 * Only the two routines on the particle-filter path are defined, with the
 * plain sequential summation order a reference BLAS would use:
 *   cblas_ddot   <- Weight::normalize ESS       (core/weight.hpp:46, 220)
 *   cblas_dgemv  <- Monitor::eval weighted mean (core/monitor.hpp:263)
 * The rest are declared so off-path inline code in the headers parses. */
#ifndef VSMC_ORACLE_SHIM_CBLAS_H
#define VSMC_ORACLE_SHIM_CBLAS_H

#ifdef __cplusplus
extern "C" {
#endif

enum CBLAS_LAYOUT { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };
enum CBLAS_UPLO { CblasUpper = 121, CblasLower = 122 };
enum CBLAS_DIAG { CblasNonUnit = 131, CblasUnit = 132 };
enum CBLAS_SIDE { CblasLeft = 141, CblasRight = 142 };
typedef enum CBLAS_LAYOUT CBLAS_ORDER;

static inline double cblas_ddot(const int n, const double *x, const int incx,
    const double *y, const int incy)
{
    double s = 0;
    for (int i = 0; i < n; ++i)
        s += x[i * incx] * y[i * incy];
    return s;
}

/* y = alpha * op(A) * x + beta * y, sequential accumulation over columns */
static inline void cblas_dgemv(const enum CBLAS_LAYOUT layout,
    const enum CBLAS_TRANSPOSE trans, const int m, const int n,
    const double alpha, const double *a, const int lda, const double *x,
    const int incx, const double beta, double *y, const int incy)
{
    int rows = m, cols = n;
    int col_major_notrans =
        (layout == CblasColMajor) == (trans == CblasNoTrans);
    if (trans != CblasNoTrans) {
        rows = n;
        cols = m;
    }
    for (int r = 0; r < rows; ++r) {
        double s = 0;
        for (int c = 0; c < cols; ++c) {
            double av = col_major_notrans ? a[c * lda + r] : a[r * lda + c];
            s += av * x[c * incx];
        }
        y[r * incy] = alpha * s + (beta == 0 ? 0 : beta * y[r * incy]);
    }
}

void cblas_ssyr(const enum CBLAS_LAYOUT, const enum CBLAS_UPLO, const int,
    const float, const float *, const int, float *, const int);
void cblas_dsyr(const enum CBLAS_LAYOUT, const enum CBLAS_UPLO, const int,
    const double, const double *, const int, double *, const int);
void cblas_ssyrk(const enum CBLAS_LAYOUT, const enum CBLAS_UPLO,
    const enum CBLAS_TRANSPOSE, const int, const int, const float,
    const float *, const int, const float, float *, const int);
void cblas_dsyrk(const enum CBLAS_LAYOUT, const enum CBLAS_UPLO,
    const enum CBLAS_TRANSPOSE, const int, const int, const double,
    const double *, const int, const double, double *, const int);
void cblas_stpmv(const enum CBLAS_LAYOUT, const enum CBLAS_UPLO,
    const enum CBLAS_TRANSPOSE, const enum CBLAS_DIAG, const int,
    const float *, float *, const int);
void cblas_dtpmv(const enum CBLAS_LAYOUT, const enum CBLAS_UPLO,
    const enum CBLAS_TRANSPOSE, const enum CBLAS_DIAG, const int,
    const double *, double *, const int);
void cblas_strmm(const enum CBLAS_LAYOUT, const enum CBLAS_SIDE,
    const enum CBLAS_UPLO, const enum CBLAS_TRANSPOSE, const enum CBLAS_DIAG,
    const int, const int, const float, const float *, const int, float *,
    const int);
void cblas_dtrmm(const enum CBLAS_LAYOUT, const enum CBLAS_SIDE,
    const enum CBLAS_UPLO, const enum CBLAS_TRANSPOSE, const enum CBLAS_DIAG,
    const int, const int, const double, const double *, const int, double *,
    const int);

#ifdef __cplusplus
}
#endif

#endif
