/* MAGMA 2.2.0 subset used by calcIR.cu, implemented on the host (refshim.cpp):
 * ssyevd (FP64 cyclic Jacobi, eigenvalues ascending), sgemv, cgemv, cdotu, cgemm, ccopy
 * with column-major BLAS semantics and FP32 accumulation.  Test infrastructure only. */
#ifndef REFSHIM_MAGMA_V2_H
#define REFSHIM_MAGMA_V2_H
#include "shim_types.h"
typedef long long magma_int_t;
typedef refshim_cfloat magmaFloatComplex;
typedef void *magma_queue_t;
typedef enum { MagmaNoVec = 301, MagmaVec = 302 } magma_vec_t;
typedef enum { MagmaUpper = 121, MagmaLower = 122 } magma_uplo_t;
typedef enum { MagmaNoTrans = 111, MagmaTrans = 112, MagmaConjTrans = 113 } magma_trans_t;
#define MAGMA_SUCCESS 0

static inline magmaFloatComplex refshim_cmake(double r, double i) { magmaFloatComplex z = {(float)r, (float)i}; return z; }
static inline magmaFloatComplex refshim_cadd(magmaFloatComplex a, magmaFloatComplex b) { return refshim_cmake(a.x + b.x, a.y + b.y); }
static inline magmaFloatComplex refshim_cmul(magmaFloatComplex a, magmaFloatComplex b) {
    magmaFloatComplex z = {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; return z; }
static inline magmaFloatComplex refshim_cdiv(magmaFloatComplex a, magmaFloatComplex b) {
    float d = b.x * b.x + b.y * b.y;
    magmaFloatComplex z = {(a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d}; return z; }
#define MAGMA_C_MAKE(r, i) refshim_cmake((r), (i))
#define MAGMA_C_ADD(a, b) refshim_cadd((a), (b))
#define MAGMA_C_MUL(a, b) refshim_cmul((a), (b))
#define MAGMA_C_DIV(a, b) refshim_cdiv((a), (b))
#define MAGMA_C_REAL(a) ((a).x)
#define MAGMA_C_IMAG(a) ((a).y)
#define MAGMA_C_ONE refshim_cmake(1.0, 0.0)
#define MAGMA_C_ZERO refshim_cmake(0.0, 0.0)

int magma_init(void);
int magma_finalize(void);
void magma_queue_create(int device, magma_queue_t *queue);
void magma_queue_destroy(magma_queue_t queue);
const char *magma_strerror(int err);
int magma_imalloc_cpu(magma_int_t **p, magma_int_t n);
int magma_smalloc_pinned(float **p, magma_int_t n);
int magma_free_pinned(void *p);
int magma_free(void *p);
magma_int_t magma_ssyevd_gpu(magma_vec_t jobz, magma_uplo_t uplo, magma_int_t n, float *dA, magma_int_t ldda,
                             float *w, float *wA, magma_int_t ldwa, float *work, magma_int_t lwork,
                             magma_int_t *iwork, magma_int_t liwork, magma_int_t *info);
void magma_sgemv(magma_trans_t t, magma_int_t m, magma_int_t n, float alpha, const float *A, magma_int_t lda,
                 const float *x, magma_int_t incx, float beta, float *y, magma_int_t incy, magma_queue_t q);
void magma_cgemv(magma_trans_t t, magma_int_t m, magma_int_t n, magmaFloatComplex alpha, const magmaFloatComplex *A,
                 magma_int_t lda, const magmaFloatComplex *x, magma_int_t incx, magmaFloatComplex beta,
                 magmaFloatComplex *y, magma_int_t incy, magma_queue_t q);
magmaFloatComplex magma_cdotu(magma_int_t n, const magmaFloatComplex *x, magma_int_t incx,
                              const magmaFloatComplex *y, magma_int_t incy, magma_queue_t q);
void magma_cgemm(magma_trans_t ta, magma_trans_t tb, magma_int_t m, magma_int_t n, magma_int_t k,
                 magmaFloatComplex alpha, const magmaFloatComplex *A, magma_int_t lda, const magmaFloatComplex *B,
                 magma_int_t ldb, magmaFloatComplex beta, magmaFloatComplex *C, magma_int_t ldc, magma_queue_t q);
void magma_ccopy(magma_int_t n, const magmaFloatComplex *x, magma_int_t incx, magmaFloatComplex *y,
                 magma_int_t incy, magma_queue_t q);
#endif
