// Device-side helpers and the kernel entry points shared by the .cu files.
#ifndef CIR_DEVICE_CUH_
#define CIR_DEVICE_CUH_

#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include "cir_internal.h"

// minImage (calcIR.cu:1459-1463): dx - L*round(dx/L), round half away from zero, evaluated
// as the reference's float expression is, one rounding per operation (no fused multiply-add),
// so that the image chosen at the box's half-width rounds as the reference rounds it.
__device__ __forceinline__ float cir_mi(float dx, float L) {
    return __fsub_rn(dx, __fmul_rn(L, roundf(__fdiv_rn(dx, L))));
}
// mag3 (calcIR.cu:1464-1476): sqrt(x*x + y*y + z*z) with the reference's order of operations
// and one rounding each; the field's cutoff test compares it with 0.7831 nm, a discontinuous
// decision that a contracted evaluation would take differently for pairs within an ulp of it.
__device__ __forceinline__ float cir_mag3(float x, float y, float z) {
    return __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)), __fmul_rn(z, z)));
}

__device__ __forceinline__ float warp_sum(float v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_sum_d(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Strict total order on (value, index) with NaN after every number: ranks counted with it
// form a permutation whatever the values, so non-finite input can never turn a rank into an
// out-of-range index.  cir_lt / cir_le are x < v and x <= v in the same order (no index).
template <typename T>
__device__ __forceinline__ bool cir_before(T a, int i, T b, int j) {
    const bool na = a != a, nb = b != b;
    if (na || nb) return na && nb ? i < j : nb;
    return a < b || (a == b && i < j);
}
template <typename T>
__device__ __forceinline__ bool cir_lt(T x, T v) { return x == x && (v != v || x < v); }
template <typename T>
__device__ __forceinline__ bool cir_le(T x, T v) { return v != v || (x == x && x <= v); }

// Per-chromophore quantities produced by the field kernel, struct-of-arrays per frame:
// row r of a frame's [CT_NROW][ld] block.
enum {
    CT_E = 0,     // field projection (a.u.)
    CT_W,         // map frequency omega (cm^-1)
    CT_X,         // map x
    CT_P,         // map p
    CT_MUP,       // map mu'
    CT_UX, CT_UY, CT_UZ,   // OH unit vector
    CT_TX, CT_TY, CT_TZ,   // transition dipole position, wrapped by minImage
    CT_NROW
};

struct BuildArgs {
    const float *xyz;     // [nframes][natoms][3]
    const float *box;     // [nframes][3]
    float *ct;            // [nframes][CT_NROW][ld] chromophore table
    float *H;             // [nframes][n][ldh]
    float *eproj;         // [nframes][n]  or null
    float *dip;           // frame f: rows x,y,z at dip + f*dip_fstride + {0,1,2}*ldv, or null
    float *pol;           // frame f: rows xx,yy,zz,xy,yz,zx at pol + f*pol_fstride + r*ldv, or null
    long long dip_fstride, pol_fstride;
    int natoms, natom_mol, nchrom_mol, nmol, n;
    int ld;               // leading dimension of the chromophore table rows
    int ldh;              // row stride of H
    int ldv;              // row stride of dip/pol
    int imodel, ispecies;
    float avef;
    CirMaps maps;
};

constexpr int CIR_EIG_PROF_SLOTS = 20;

struct EighArgs {
    float *A;             // [nmat] matrices, column j of matrix m at A + m*mstride + j*ld
    float *W;             // [nmat][wstride] eigenvalues
    float *Z;             // scratch, same shape as A
    float2 *rot;          // scratch, cir_eigh_rot_bytes(n) per matrix
    float *DE;            // scratch, cir_eigh_de_bytes(ld) per matrix (tridiagonal d, e, tau)
    cudaEvent_t tq_done;  // recorded after the tridiagonalisation kernel when not null
    int precision;        // CIR_PREC_*: FP32, or the tensor-core form of the final V = Q_H Q_T product
    int *err;             // tensor-core kernels: set to 1 when a bounded wait gives up
    float *DC;            // divide-and-conquer scratch, cir_dc_bytes(n, ld) per matrix, laid out
                          // [3][nmat][mstride]; null selects the implicit-QR path (rot needed)
    long long mstride;
    int wstride;
    int n, ld;
    int *status;          // [nmat] 0 ok, 1 sweep cap reached
    unsigned long long *sweeps;   // accumulated QR sweeps (may be null)
    // frequency distribution (calcIR.cu:493-538); hist_count == null disables it
    int hist_group;       // matrices per histogram set (consecutive matrices; 0: one set for all);
                          // set g uses hist_*[g*nomega ..] and out_of_range[g]
    unsigned long long *hist_count;
    double *hist_ipr, *hist_mipr;
    const int *hist_weight;       // [nmat] times each matrix counts in the distributions (null: once)
    unsigned long long *out_of_range;
    int nomega, omegaStep, nchrom_mol;
    float avef, omegaStart;
    // optional [nmat][CIR_EIG_PROF_SLOTS]: %globaltimer at the start and end of the
    // tridiagonalisation, of forming Q, of the QR iteration and of the ordering (0-6), then the
    // chase and apply times (ns), rotations, the chase's block-search time (ns) and sweeps
    // (7-11; on the divide-and-conquer path: the merges' time in setup and deflation, secular
    // roots, z and norms, ranking and rotation, summed over a matrix's merges), then the blocked
    // tridiagonalisation's time (ns) in its column fetch, reflector, symmetric matrix-vector
    // product, panel dot products, w and trailing update (12-17), then the secular equation's
    // iterations and roots (18-19)
    unsigned long long *phase_ns;
    // optional FP64 refinement of the eigenpairs on the divide-and-conquer path (k_refine.cu),
    // on when Href is not null: Href holds a copy of the input matrices (same strides as A), RW
    // is scratch of cir_refine_bytes(n, ld) per matrix for refine_chunk matrices at a time
    const float *Href;
    void *RW;
    int refine_iters, refine_chunk;
    // fault drills (tests only, 0 = off): the split-BF16 GEMMs' stall (SplitGemmArgs::test_stall)
    // and a cap on the QR sweeps of each divide-and-conquer leaf
    int test_stall, test_sweep_cap;
    // set by the launcher: 1 walks the tiles of the tridiagonalisation's matrix-vector
    // products in reverse order on alternate columns (CIR_TQ_ORDER=0 keeps one order)
    int tq_order;
    // thread blocks of the tridiagonalisation per SM: 0 the kernel's own occupancy, or a
    // smaller count enforced through its shared-memory request (the autotuner's choice)
    int tq_blocks;
    // per-matrix stride of Z in the tridiagonalisation (0: mstride), which keeps only the
    // panel's W there (cir_tridiag_w_floats(ld) floats per matrix)
    long long zstride;
    // 1: cir_launch_eigh starts after the tridiagonalisation (d, e, tau already in DE and the
    // reflectors in A, as cir_launch_tridiag_multi leaves them)
    int skip_tridiag;
};

// kernel launchers (return cudaError_t of the launch)
cudaError_t cir_launch_build(const BuildArgs &a, int nframes, cudaStream_t s, int *launches);
cudaError_t cir_launch_eigh(const EighArgs &a, int nmat, cudaStream_t s, int *launches);
// the tridiagonalisation kernel alone (phase 1 of cir_launch_eigh), for the autotuner
cudaError_t cir_launch_tridiag(const EighArgs &a, int nmat, cudaStream_t s);
// thread blocks per SM the tridiagonalisation of order n runs with by default
int cir_tridiag_blocks(int n);
// The tridiagonalisations of up to CIR_TQ_MAXP batches of orders 257-1024 (boxes of different
// size) in one launch, the longest matrices first; a[i] as for cir_launch_tridiag (tq_blocks
// is not applied: the kernel's own occupancy).
constexpr int CIR_TQ_MAXP = 4;
cudaError_t cir_launch_tridiag_multi(const EighArgs *a, const int *nmat, int np, cudaStream_t s, int *launches);
size_t cir_tridiag_w_floats(int ld);   // the tridiagonalisation's use of Z per matrix
size_t cir_eigh_rot_bytes(int n);
size_t cir_eigh_de_bytes(int ld);
size_t cir_dc_bytes(int n, int ld);
cudaError_t cir_launch_dc(const EighArgs &a, int nmat, cudaStream_t s, int *launches);
// V = Q_H Q into a.A by blocked compact-WY application of the tridiagonalisation's
// reflectors (in a.A) to Q; Q is overwritten, P and U are scratch (a.mstride floats per
// matrix), a.Z holds the blocks' T^T V^T.
cudaError_t cir_launch_backtransform(const EighArgs &a, float *Q, float *P, float *U, int nmat, cudaStream_t s,
                                     int *launches,
                                     bool q_split = false);
// FP64 refinement of eigenpairs (k_refine.cu): iters steps on the eigenvectors Z (row j =
// eigenvector j, mstride / ld as A) of the matrices H (same strides) with eigenvalues w
// (stride wstride), chunk matrices at a time in ws (cir_refine_bytes(n, ld) per matrix).
size_t cir_refine_bytes(int n, int ld);
cudaError_t cir_launch_refine(const float *H, float *Z, long long mstride, int ld, int n, float *w, long long wstride,
                              int nmat, int iters, void *ws, int chunk, cudaStream_t s, int *launches);
int cir_eigh_max_n();

// batched SIMT FP32 GEMM, C = A * B (row-major B, C); A row- or column-major.
// epilogue 1: rotate column pairs (2q, 2q+1) of row i by exp(+i w[i] dt/hbar).
struct GemmArgs {
    const float *A, *B;
    float *C;
    int M, N, K;
    int lda, ldb, ldc;
    long long sA, sB, sC;  // batch strides (elements)
    bool a_colmajor;
    bool b_kmajor;         // B element (k, n) at B[n*ldb + k] instead of B[k*ldb + n]
    int epilogue;          // 0 none, 1 phase rotation, 2 C = D - A B
    const float *D;        // epilogue 2 (may equal C)
    int ldd;
    long long sD;
    const float *w;        // [batch][wstride] for epilogue 1
    int wstride;
    float dt_over_hbar;
    int *err;              // tensor-core kernels: set to 1 when a bounded wait gives up
    // k_tc_gemm only, epilogue 0: when set, C is written as a BF16 hi/lo pair at the same
    // element offsets instead (batch stride 2 sC elements)
    __nv_bfloat16 *Chi, *Clo;
};
// SIMT tile shapes: 128 x 128 x 8, or 64 x 64 x 16 (more blocks for small products)
constexpr int CIR_GEMM_TILE_128 = 0, CIR_GEMM_TILE_64 = 1;
cudaError_t cir_launch_gemm(const GemmArgs &g, int batch, cudaStream_t s, int *launches, int tile = CIR_GEMM_TILE_128);
// the same product on the tensor cores (tcgen05), precision CIR_PREC_TF32
cudaError_t cir_launch_tc_gemm(const GemmArgs &g, int batch, int precision, cudaStream_t s, int *launches);
size_t cir_tc_gemm_smem_bytes();

// ---- split-BF16 propagation on pre-split operands (k_tc_split.cu) ----
// A matrix held as two BF16 matrices, hi = bf16(x) and lo = bf16(x - hi).
struct SplitMat {
    __nv_bfloat16 *hi, *lo;
};
// C = A B (hi*hi + hi*lo + lo*hi, FP32 accumulation) with K-major operands:
// A(i, k) at A[i*lda + k], B(k, j) at B[j*ldb + k].  out_mode 0: C(i, j) written as a
// hi/lo pair at C[j*ldc + i]; 1: as a pair at C[i*ldc + j]; 2: in FP32 at Cf[i*ldc + j].
// lda, ldb and the batch strides are multiples of 8, the operand pointers 16-byte aligned.
// epilogue 1: columns (2q, 2q+1) of row i rotated by exp(+i w[i] dt/hbar) before the split;
// epilogue 2: C = D - A B, D a row-major pair (D[i*ldd + j], batch stride sD; may be C).
struct SplitGemmArgs {
    const __nv_bfloat16 *Ahi, *Alo, *Bhi, *Blo;
    __nv_bfloat16 *Chi, *Clo;
    float *Cf;
    int out_mode;
    const __nv_bfloat16 *Dhi, *Dlo;
    int ldd;
    long long sD;
    int M, N, K;
    int lda, ldb, ldc;
    long long sA, sB, sC;
    int epilogue;
    const float *w;
    int wstride;
    float dt_over_hbar;
    int *err;
    // fused correlation contraction for the propagation product F' = V G (out_mode 0): when
    // tcf_out is set, row r of the product contracts with m(0) over the tile's complex columns
    // and with m(k) at row r (the terms of k_tcf), and each block adds its six sums to
    // tcf_out[batch * tcf_sout ..]
    const float *tcf_m0, *tcf_mt;
    long long tcf_sm0, tcf_smt;
    int tcf_ldv;
    double *tcf_out;
    long long tcf_sout;
    int bz0;              // batch entry of blockIdx.z == 0 (set by the launcher when it splits a batch)
    int test_stall;       // fault drill (tests only): 1 withholds the first tile's completion and
                          // shortens the pipeline waits, so that they run out and raise err
    int tile_n;           // tile width: 0 picks by shape; 128 or 256 forces it (the autotuner's choice)
};
size_t cir_split_ld(int n);   // leading dimension of the split operands (n rounded up to 8)
cudaError_t cir_launch_split_gemm(const SplitGemmArgs &g, int batch, cudaStream_t s, int *launches);
// Several split-BF16 products in one persistent launch (the tiles of problem 0 first, then
// problem 1, ...): each problem a batch of one shape with its own operands, epilogue and
// tensor maps, all in the widest tile width any of them takes; bz0 must be 0.
constexpr int CIR_SPLIT_MAXP = 4;
cudaError_t cir_launch_split_gemm_multi(const SplitGemmArgs *g, const int *batch, int np, cudaStream_t s,
                                        int *launches);
// Vc = V (V[k][i] at A[i*ld + k]) and Vr = V^T, both as Vc[i*ldh + k]-style K-major pairs
cudaError_t cir_launch_split_v(const float *A, int ld, long long sA, int n, SplitMat Vc, SplitMat Vr, int ldh,
                               long long sV, int batch, cudaStream_t s, int *launches);
// Ft = I for the transposed complex F (real column c = 2q + {0: re, 1: im} at Ft[c*ldh ..])
cudaError_t cir_launch_identity_t(SplitMat F, int n, int ldh, long long sF, int batch, cudaStream_t s, int *launches);

// ---- two-stage reduction to tridiagonal form (k_sbr.cu): dense -> band on the split-BF16
// tcgen05 GEMM, band -> tridiagonal by bulge chasing; d and e only (no eigenvectors) ----
int cir_sbr_max_n();
size_t cir_sbr_bytes(int n, int ld);   // work area per matrix (ld a multiple of 8)
cudaError_t cir_launch_sbr(const float *H, long long sH, int nmat, int n, int ld, float *d, float *e, void *work,
                           int *err, cudaStream_t s, float *ms, int *launches);

// TCF terms: out[b][6] += (IR, VV, VH) for batch element b
struct TcfArgs {
    const float *F;        // [batch] complex row-major, row stride ldf floats (2 per element)
    long long sF;
    const float *m0;       // [batch][9][ldv] dip0 (3) then pol0 (6)
    const float *mt;       // [batch][9][ldv]
    long long sm0, smt;
    double *out;           // [batch][6]
    long long sout;
    int n, ldf, ldv;
    SplitMat Ft;           // when Ft.hi is set: F stored transposed as a split pair, F[r][c] at
    long long sFt;         // Ft[c*ldft + r], instead of F
    int ldft;
};
cudaError_t cir_launch_tcf(const TcfArgs &t, int batch, cudaStream_t s, int *launches);

// spectral density of one frame: Sw[nomega] += ...
cudaError_t cir_launch_spectral(const float *V, int ld, const float *w, const float *dip, int ldv, int n,
                                float *mu2_scratch, double *Sw, int nomega, float omegaStart, int omegaStep,
                                float t1, float avef, cudaStream_t s, int *launches);

// unnormalised inverse real DFT (cuFFT C2R convention) of X[0..n/2] (complex double)
// into y[n], by a mixed-radix Stockham FFT in double precision
cudaError_t cir_launch_c2r(const double *X, int nx, int n, double *work0, double *work1, double *y,
                           cudaStream_t s, int *launches);

// F = I for nprop complex matrices
cudaError_t cir_launch_identity(float *F, int n, int ldf, long long sF, int batch, cudaStream_t s, int *launches);


// ---- differentiation form (k_adjoint.cu) ----
constexpr int CIR_PSI_LD = 18;   // psi / lambda: n x 9 complex, row-major (re, im) pairs
struct DthetaArgs {
    const float *ct;      // chromophore table of the step's frame of origin 0; origin s at + s*sct
    long long sct;
    const float *box;     // box of that frame; origin s at + s*sbox
    long long sbox;
    const float *G;       // dL/dH of the step (row-major, ldg; origin s at + s*sG), or null at step 0
    int ldg;
    long long sG;
    const float *psi;     // psi(k), n x 18 per origin
    const float *lam0;    // lambda(0) at step 0, else null
    float gir_r, gir_i, gvv_r, gvv_i;   // dL/dTCF of the step (IR, VV)
    CirMaps maps;
    int n, ld, nchrom_mol, ispecies;
    double *out;          // [13] accumulated
};
// one step psi <- V e^{i L dt/hbar} V^T psi of S origins (psi, tmp: n x CIR_PSI_LD per origin)
cudaError_t cir_psi_step(const float *V, int ld, long long sV, int n, const float *w, long long sw, float dt_over_hbar,
                         float *psi, float *tmp, int S, cudaStream_t s);
cudaError_t cir_adj_psi_init(const float *M, long long sM, int ld, int n, int S, float *psi, cudaStream_t s);
cudaError_t cir_adj_tcf(const float *psi, const float *M, long long sM, int ld, int n, int S, double *out, long long sout,
                        cudaStream_t s);
cudaError_t cir_adj_lambda_src(float *lam, const float *M, long long sM, int ld, int n, int S, float gir_r, float gir_i,
                               float gvv_r, float gvv_i, int zero, cudaStream_t s);
cudaError_t cir_adj_build_R(const float *a, const float *b, const float *W, long long sW, int n, int S, float tau, float *R,
                            int ldr, long long sR, cudaStream_t s);
cudaError_t cir_adj_dtheta(const DthetaArgs &d, int S, cudaStream_t s);

#endif
