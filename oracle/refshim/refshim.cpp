/* Host implementations behind the shim headers (test infrastructure only):
 *   magma_ssyevd_gpu  cyclic Jacobi in double precision on the upper triangle, eigenvalues
 *                     ascending, eigenvectors as columns (LAPACK/MAGMA layout);
 *   BLAS calls        straightforward loops with column-major semantics, FP32 sums;
 *   cufftExecC2R      y_k = Re X_0 + 2 sum_{0<j<n/2} Re(X_j e^{+2 pi i jk/n}) [+ (-1)^k Re X_{n/2}]
 *                     in double precision (cuFFT's unnormalised C2R convention);
 *   xdrfile / xtc     CIRTRJ01 raw trajectories. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "cufft.h"
#include "magma_v2.h"
#include "xdrfile_xtc.h"
#include "xtc_seek.h"

int magma_init(void) { return 0; }
int magma_finalize(void) { return 0; }
void magma_queue_create(int, magma_queue_t *q) { *q = nullptr; }
void magma_queue_destroy(magma_queue_t) {}
const char *magma_strerror(int) { return "shim"; }
int magma_imalloc_cpu(magma_int_t **p, magma_int_t n) { *p = (magma_int_t *)calloc(n > 0 ? n : 1, sizeof(magma_int_t)); return *p ? 0 : -1; }
int magma_smalloc_pinned(float **p, magma_int_t n) { *p = (float *)calloc(n > 0 ? n : 1, sizeof(float)); return *p ? 0 : -1; }
int magma_free_pinned(void *p) { free(p); return 0; }
int magma_free(void *p) { free(p); return 0; }

magma_int_t magma_ssyevd_gpu(magma_vec_t, magma_uplo_t, magma_int_t n, float *dA, magma_int_t ldda, float *w,
                             float *, magma_int_t, float *work, magma_int_t lwork, magma_int_t *iwork,
                             magma_int_t liwork, magma_int_t *info) {
    *info = 0;
    if (lwork == -1 || liwork == -1) {   // workspace query
        if (work) work[0] = 1;
        if (iwork) iwork[0] = 1;
        return 0;
    }
    std::vector<double> a(n * n), v(n * n, 0.0);
    for (magma_int_t j = 0; j < n; j++)
        for (magma_int_t i = 0; i <= j; i++) a[i + j * n] = a[j + i * n] = dA[i + j * ldda];   // upper triangle
    for (magma_int_t i = 0; i < n; i++) v[i + i * n] = 1.0;
    for (int sweep = 0; sweep < 100; sweep++) {
        double off = 0, tot = 0;
        for (magma_int_t j = 0; j < n; j++)
            for (magma_int_t i = 0; i < n; i++) {
                tot += a[i + j * n] * a[i + j * n];
                if (i != j) off += a[i + j * n] * a[i + j * n];
            }
        if (off <= 1e-30 * tot) break;
        for (magma_int_t p = 0; p < n - 1; p++)
            for (magma_int_t q = p + 1; q < n; q++) {
                const double apq = a[p + q * n];
                if (fabs(apq) < 1e-300) continue;
                const double theta = (a[q + q * n] - a[p + p * n]) / (2 * apq);
                const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1));
                const double c = 1 / sqrt(t * t + 1), s = t * c;
                for (magma_int_t k = 0; k < n; k++) {   // columns p, q
                    const double akp = a[k + p * n], akq = a[k + q * n];
                    a[k + p * n] = c * akp - s * akq;
                    a[k + q * n] = s * akp + c * akq;
                }
                for (magma_int_t k = 0; k < n; k++) {   // rows p, q
                    const double apk = a[p + k * n], aqk = a[q + k * n];
                    a[p + k * n] = c * apk - s * aqk;
                    a[q + k * n] = s * apk + c * aqk;
                }
                for (magma_int_t k = 0; k < n; k++) {
                    const double vkp = v[k + p * n], vkq = v[k + q * n];
                    v[k + p * n] = c * vkp - s * vkq;
                    v[k + q * n] = s * vkp + c * vkq;
                }
            }
    }
    std::vector<magma_int_t> idx(n);
    for (magma_int_t i = 0; i < n; i++) idx[i] = i;
    std::stable_sort(idx.begin(), idx.end(), [&](magma_int_t x, magma_int_t y) { return a[x + x * n] < a[y + y * n]; });
    for (magma_int_t j = 0; j < n; j++) {
        w[j] = (float)a[idx[j] + idx[j] * n];
        for (magma_int_t i = 0; i < n; i++) dA[i + j * ldda] = (float)v[i + idx[j] * n];
    }
    return 0;
}

void magma_sgemv(magma_trans_t t, magma_int_t m, magma_int_t n, float alpha, const float *A, magma_int_t lda,
                 const float *x, magma_int_t incx, float beta, float *y, magma_int_t incy, magma_queue_t) {
    if (t == MagmaNoTrans) {
        for (magma_int_t i = 0; i < m; i++) {
            float s = 0;
            for (magma_int_t j = 0; j < n; j++) s += A[i + j * lda] * x[j * incx];
            y[i * incy] = alpha * s + (beta != 0 ? beta * y[i * incy] : 0.f);
        }
    } else {
        for (magma_int_t j = 0; j < n; j++) {
            float s = 0;
            for (magma_int_t i = 0; i < m; i++) s += A[i + j * lda] * x[i * incx];
            y[j * incy] = alpha * s + (beta != 0 ? beta * y[j * incy] : 0.f);
        }
    }
}

static inline magmaFloatComplex cfma(magmaFloatComplex a, magmaFloatComplex b, magmaFloatComplex c) {
    c.x += a.x * b.x - a.y * b.y;
    c.y += a.x * b.y + a.y * b.x;
    return c;
}

void magma_cgemv(magma_trans_t t, magma_int_t m, magma_int_t n, magmaFloatComplex alpha, const magmaFloatComplex *A,
                 magma_int_t lda, const magmaFloatComplex *x, magma_int_t incx, magmaFloatComplex beta,
                 magmaFloatComplex *y, magma_int_t incy, magma_queue_t) {
    if (t != MagmaNoTrans) { fprintf(stderr, "refshim: cgemv only implements NoTrans\n"); exit(1); }
    for (magma_int_t i = 0; i < m; i++) {
        magmaFloatComplex s = {0, 0};
        for (magma_int_t j = 0; j < n; j++) s = cfma(A[i + j * lda], x[j * incx], s);
        magmaFloatComplex r = refshim_cmul(alpha, s);
        if (beta.x != 0 || beta.y != 0) r = refshim_cadd(r, refshim_cmul(beta, y[i * incy]));
        y[i * incy] = r;
    }
}

magmaFloatComplex magma_cdotu(magma_int_t n, const magmaFloatComplex *x, magma_int_t incx,
                              const magmaFloatComplex *y, magma_int_t incy, magma_queue_t) {
    magmaFloatComplex s = {0, 0};
    for (magma_int_t i = 0; i < n; i++) s = cfma(x[i * incx], y[i * incy], s);
    return s;
}

void magma_cgemm(magma_trans_t ta, magma_trans_t tb, magma_int_t m, magma_int_t n, magma_int_t k,
                 magmaFloatComplex alpha, const magmaFloatComplex *A, magma_int_t lda, const magmaFloatComplex *B,
                 magma_int_t ldb, magmaFloatComplex beta, magmaFloatComplex *C, magma_int_t ldc, magma_queue_t) {
    if (ta != MagmaNoTrans || (tb != MagmaNoTrans && tb != MagmaTrans)) {
        fprintf(stderr, "refshim: cgemm transpose mode not implemented\n");
        exit(1);
    }
    std::vector<magmaFloatComplex> out((size_t)m * n);
    for (magma_int_t j = 0; j < n; j++)
        for (magma_int_t i = 0; i < m; i++) {
            magmaFloatComplex s = {0, 0};
            for (magma_int_t l = 0; l < k; l++) {
                const magmaFloatComplex b = tb == MagmaNoTrans ? B[l + j * ldb] : B[j + l * ldb];
                s = cfma(A[i + l * lda], b, s);
            }
            magmaFloatComplex r = refshim_cmul(alpha, s);
            if (beta.x != 0 || beta.y != 0) r = refshim_cadd(r, refshim_cmul(beta, C[i + j * ldc]));
            out[i + j * (size_t)m] = r;
        }
    for (magma_int_t j = 0; j < n; j++)
        for (magma_int_t i = 0; i < m; i++) C[i + j * ldc] = out[i + j * (size_t)m];
}

void magma_ccopy(magma_int_t n, const magmaFloatComplex *x, magma_int_t incx, magmaFloatComplex *y,
                 magma_int_t incy, magma_queue_t) {
    for (magma_int_t i = 0; i < n; i++) y[i * incy] = x[i * incx];
}

static std::vector<int> g_plan_n;
int cufftPlan1d(cufftHandle *plan, int nx, cufftType, int) {
    g_plan_n.push_back(nx);
    *plan = (int)g_plan_n.size() - 1;
    return 0;
}
int cufftDestroy(cufftHandle) { return 0; }
int cufftExecC2R(cufftHandle plan, cufftComplex *in, cufftReal *out) {
    const long long n = g_plan_n[plan];
    const long long h = n / 2;
    std::vector<double> y(n, 0.0);
    for (long long j = 0; j <= h; j++) {
        const double re = in[j].x, im = (j == 0 || 2 * j == n) ? 0.0 : in[j].y;
        if (re == 0.0 && im == 0.0) continue;
        const double wgt = (j == 0 || 2 * j == n) ? 1.0 : 2.0;
        for (long long k = 0; k < n; k++) {
            const double ang = 2.0 * M_PI * (double)((j * k) % n) / (double)n;
            y[k] += wgt * (re * cos(ang) - im * sin(ang));
        }
    }
    for (long long k = 0; k < n; k++) out[k] = (float)y[k];
    return 0;
}

struct refshim_xdrfile {
    FILE *f;
    int natoms;
};

XDRFILE *xdrfile_open(const char *path, const char *) {
    FILE *f = fopen(path, "rb");
    if (!f) return nullptr;
    char magic[8];
    int hdr[4];
    if (fread(magic, 1, 8, f) != 8 || memcmp(magic, "CIRTRJ01", 8) || fread(hdr, 4, 4, f) != 4) {
        fclose(f);
        return nullptr;
    }
    XDRFILE *x = new XDRFILE;
    x->f = f;
    x->natoms = hdr[0];
    return x;
}

int xdrfile_close(XDRFILE *x) {
    if (x) { fclose(x->f); delete x; }
    return 0;
}

int read_xtc_natoms(char *fn, int *natoms) {
    XDRFILE *x = xdrfile_open(fn, "r");
    if (!x) return exdrFILENOTFOUND;
    *natoms = x->natoms;
    xdrfile_close(x);
    return exdrOK;
}

int read_xtc(XDRFILE *xd, int natoms, int *step, float *time, matrix box, rvec *x, float *prec) {
    float t, b[3];
    if (fread(&t, 4, 1, xd->f) != 1 || fread(b, 4, 3, xd->f) != 3) return exdrENDOFFILE;
    if (fread(x, 12, natoms, xd->f) != (size_t)natoms) return exdrENDOFFILE;
    memset(box, 0, sizeof(matrix));
    box[0][0] = b[0]; box[1][1] = b[1]; box[2][2] = b[2];
    *time = t;
    *step = 0;
    *prec = 1000.f;
    return exdrOK;
}

int read_xtc_n_frames(char *fn, int *n_frames, int *est_nframes, int64_t **offsets) {
    FILE *f = fopen(fn, "rb");
    if (!f) return exdrFILENOTFOUND;
    char magic[8];
    int hdr[4];
    if (fread(magic, 1, 8, f) != 8 || fread(hdr, 4, 4, f) != 4) { fclose(f); return exdrHEADER; }
    fclose(f);
    *n_frames = hdr[1];
    *est_nframes = hdr[1];
    *offsets = (int64_t *)malloc(sizeof(int64_t) * (hdr[1] > 0 ? hdr[1] : 1));
    for (int i = 0; i < hdr[1]; i++) (*offsets)[i] = 24 + (int64_t)i * (16 + 12LL * hdr[0]);
    return exdrOK;
}

int xdr_seek(XDRFILE *xd, int64_t pos, int whence) { return fseek(xd->f, (long)pos, whence) == 0 ? exdrOK : exdrENDOFFILE; }
