// Two-stage reduction of the batched symmetric eigenproblem to tridiagonal form (the
// successive band reduction of ELPA / MAGMA's two-stage ssyevd; the one-stage path is
// k_eigh_tq, which replaces the sytrd step of magma_ssyevd_gpu, calcIR.cu:420-448):
//
//  stage 1, dense -> band of width SB_B, by panels of SB_B columns: the panel below the band
//   is factored by Householder QR (k_sb_panel, one thread per panel row, the panel in
//   registers), and the trailing block gets the two-sided update of the compact WY form,
//     X = A22 V,  Y = X T,  W = Y - 1/2 V (T^T V^T Y),  A22 <- A22 - V W^T - W V^T,
//   both products on the persistent split-BF16 tcgen05 GEMM (k_tc_split.cu), A kept as a
//   BF16 hi/lo pair (full symmetric storage); W in k_sb_w.  The matrix is shifted by the mean
//   of its diagonal first, so the pairs' 16-bit precision is relative to the spread of the
//   spectrum rather than to its centre.
//  stage 2, band -> tridiagonal, by bulge chasing (k_sb_chase, one thread block per matrix,
//   the band in global memory, lower storage of 2*SB_B+1 offsets for the fill): sweep c
//   annihilates column c below the subdiagonal with a reflector of length <= SB_B, then chases
//   the bulge it creates down the band, one SB_B-row block per step; sweep c+1 follows
//   sweep c four steps behind, so the tasks of one time step touch disjoint index ranges
//   and run on separate warps (at most eight at once at SB_B = 32, order <= 1025).
//
// The reflectors of both stages are not kept: this path gives the tridiagonal (d, e) whose
// eigenvalues are the matrix's; the eigenvectors would need the two back-transforms.
#include "cir_device.cuh"

#include <vector>

namespace {

constexpr int SB_B = 32;                 // band width
constexpr int SB_LDB = 2 * SB_B + 1;     // band storage: element (r, c), 0 <= r - c <= 2 SB_B, at c*SB_LDB + r - c
constexpr int SB_NT = 1024;              // panel and W kernels: one thread per panel row
constexpr int SB_LAG = 4;                // steps between consecutive sweeps of the chase
constexpr int SB_CW = 8;                 // warps of the chase

__device__ __forceinline__ float pair_get(const __nv_bfloat16 *h, const __nv_bfloat16 *l, size_t o) {
    return __bfloat162float(h[o]) + __bfloat162float(l[o]);
}
__device__ __forceinline__ void pair_put(__nv_bfloat16 *h, __nv_bfloat16 *l, size_t o, float x) {
    const __nv_bfloat16 hi = __float2bfloat16_rn(x);
    h[o] = hi;
    l[o] = __float2bfloat16_rn(x - __bfloat162float(hi));
}

}  // namespace

// Work areas of the two-stage reduction, per matrix (strides in elements of each array).
struct SbArgs {
    int n, ld;
    SplitMat S;           // the shifted matrix as a pair, column-major, hi and lo S.lo - S.hi apart
    long long sS;
    SplitMat Vc;          // the panel's reflectors, column j at Vc + j*ld (panel rows)
    long long sVc;
    SplitMat L, R;        // [V W] and [W V], row-major, panel rows x 2 SB_B
    long long sLR;
    float *Vf, *X;        // the reflectors and X = A22 V in FP32, row-major, panel rows x SB_B
    long long sVX;
    float *T;             // SB_B x SB_B per matrix
    float *Bd;            // the band, n x SB_LDB per matrix
    long long sBd;
    float *sig;           // the diagonal shift of each matrix
    int *err;
};

namespace {

// sig = mean of the diagonal; Bd cleared
__global__ void __launch_bounds__(256) k_sb_shift(const float *H, long long sH, SbArgs g) {
    __shared__ float red[8];
    const int mat = blockIdx.x, t = threadIdx.x, n = g.n, ld = g.ld;
    const float *A = H + (size_t)mat * sH;
    float s = 0.f;
    for (int i = t; i < n; i += 256) s += A[(size_t)i * ld + i];
    s = warp_sum(s);
    if ((t & 31) == 0) red[t >> 5] = s;
    __syncthreads();
    if (t == 0) {
        float x = 0.f;
        for (int w = 0; w < 8; w++) x += red[w];
        g.sig[mat] = x / (float)n;
    }
    float *Bd = g.Bd + (size_t)mat * g.sBd;
    for (size_t i = t; i < (size_t)n * SB_LDB; i += 256) Bd[i] = 0.f;
}

// S = H - sig I as a pair (same column-major layout); grid (columns / 8, matrices)
__global__ void __launch_bounds__(256) k_sb_split(const float *H, long long sH, SbArgs g) {
    const int mat = blockIdx.y, n = g.n, ld = g.ld;
    const float sg = g.sig[mat];
    const float *A = H + (size_t)mat * sH;
    __nv_bfloat16 *sh = g.S.hi + (size_t)mat * g.sS, *sl = g.S.lo + (size_t)mat * g.sS;
    for (int idx = threadIdx.x; idx < 8 * n; idx += 256) {
        const int c = blockIdx.x * 8 + idx / n, r = idx % n;
        if (c >= n) break;
        const size_t o = (size_t)c * ld + r;
        pair_put(sh, sl, o, A[o] - (r == c ? sg : 0.f));
    }
}

// Panel p (columns k .. k+SB_B-1): the diagonal block into the band, then (when rows remain
// below the band) the QR of the m x SB_B panel below it, m = n - k - SB_B: thread t holds row
// t in registers; per column a norm (block sum) and one block sum of 32 values (the
// products of v with every column: the update's w for the columns to the right, V^T v for
// T's column to the left).  Writes R into the band, V (pairs: column layout and the V halves of
// L and R; FP32 row-major) and T.
__global__ void __launch_bounds__(SB_NT, 1) k_sb_panel(SbArgs g, int k) {
    __shared__ float red[32][33];
    __shared__ float wsum[32], Ts[32][33], betas[32], sc[4];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5, mat = blockIdx.x;
    const int n = g.n, ld = g.ld, m = n - k - SB_B;
    const __nv_bfloat16 *Sh = g.S.hi + (size_t)mat * g.sS, *Sl = g.S.lo + (size_t)mat * g.sS;
    float *Bd = g.Bd + (size_t)mat * g.sBd;
    {   // the diagonal block, lower part
        const int db = min(SB_B, n - k), i = t >> 5, j = t & 31;
        if (i < db && j <= i) Bd[(size_t)(k + j) * SB_LDB + i - j] = pair_get(Sh, Sl, (size_t)(k + j) * ld + k + i);
    }
    if (m < 1) return;
    const bool own = t < m;
    float P[SB_B];
    #pragma unroll
    for (int j = 0; j < SB_B; j++) P[j] = own ? pair_get(Sh, Sl, (size_t)(k + j) * ld + k + SB_B + t) : 0.f;
    for (int i = t; i < 32 * 33; i += SB_NT) (&Ts[0][0])[i] = 0.f;
    const int nr = min(SB_B, m);
    #pragma unroll
    for (int j = 0; j < SB_B; j++) {
        if (j >= nr) break;
        // the reflector of column j (rows j.. of the panel)
        float part = (own && t > j) ? P[j] * P[j] : 0.f;
        part = warp_sum(part);
        if (lane == 0) red[warp][32] = part;
        if (t == j) sc[1] = P[j];
        __syncthreads();
        if (t == 0) {
            float xn2 = 0.f;
            for (int w = 0; w < 32; w++) xn2 += red[w][32];
            const float alpha = sc[1];
            float tau = 0.f, beta = alpha, scale = 0.f;
            if (xn2 > 0.f) {
                beta = -copysignf(sqrtf(alpha * alpha + xn2), alpha);
                tau = (beta - alpha) / beta;
                scale = 1.f / (alpha - beta);
            }
            sc[2] = tau;
            sc[3] = scale;
            betas[j] = beta;
        }
        __syncthreads();
        const float tau = sc[2], scale = sc[3];
        const float v = t == j ? 1.f : ((own && t > j) ? P[j] * scale : 0.f);
        // u_c = v * P[c] summed over the rows: lane l of each warp ends with its warp's sum of u_l
        float u[SB_B / 2];
        {   // the first halving exchange straight from P, so that only 16 partial sums are live
            const bool up = (lane & 16) != 0;
            #pragma unroll
            for (int c = 0; c < 16; c++) {
                const float lo = v * P[c], hi = v * P[c + 16];
                u[c] = (up ? hi : lo) + __shfl_xor_sync(0xffffffffu, up ? lo : hi, 16);
            }
        }
        #pragma unroll
        for (int h = 8; h >= 1; h >>= 1) {
            const bool up = (lane & h) != 0;
            #pragma unroll
            for (int c = 0; c < h; c++) {
                const float send = up ? u[c] : u[c + h], keep = up ? u[c + h] : u[c];
                u[c] = keep + __shfl_xor_sync(0xffffffffu, send, h);
            }
        }
        red[warp][lane] = u[0];
        __syncthreads();
        if (t < 32) {
            float s = 0.f;
            for (int w = 0; w < 32; w++) s += red[w][t];
            wsum[t] = s;
        }
        __syncthreads();
        // T[0:j, j] = -tau T[0:j, 0:j] (V^T v)[0:j], T[j][j] = tau
        if (t < j) {
            float s = 0.f;
            for (int l = t; l < j; l++) s = fmaf(Ts[t][l], wsum[l], s);
            Ts[t][j] = -tau * s;
        } else if (t == j) {
            Ts[j][j] = tau;
        }
        #pragma unroll
        for (int c = j + 1; c < SB_B; c++) P[c] = fmaf(-tau * v, wsum[c], P[c]);
        if (t > j) P[j] = v;
        __syncthreads();
    }
    // R (upper trapezoidal, rows < nr) into the band: (k+SB_B+t, k+c) at offset SB_B + t - c
    if (own && t < nr) {
        #pragma unroll
        for (int c = 0; c < SB_B; c++)
            if (c >= t) Bd[(size_t)(k + c) * SB_LDB + SB_B + t - c] = c == t ? betas[t] : P[c];
    }
    if (own) {
        __nv_bfloat16 *vh = g.Vc.hi + (size_t)mat * g.sVc, *vl = g.Vc.lo + (size_t)mat * g.sVc;
        const size_t olr = (size_t)mat * g.sLR + (size_t)t * 2 * SB_B;
        float *vf = g.Vf + (size_t)mat * g.sVX + (size_t)t * SB_B;
        #pragma unroll
        for (int j = 0; j < SB_B; j++) {
            const float x = j < nr ? (t > j ? P[j] : (t == j ? 1.f : 0.f)) : 0.f;
            pair_put(vh, vl, (size_t)j * ld + t, x);
            pair_put(g.L.hi, g.L.lo, olr + j, x);
            pair_put(g.R.hi, g.R.lo, olr + SB_B + j, x);
            vf[j] = x;
        }
    }
    for (int i = t; i < SB_B * SB_B; i += SB_NT) g.T[(size_t)mat * SB_B * SB_B + i] = Ts[i / SB_B][i % SB_B];
}

// W = Y - 1/2 V (T^T V^T Y), Y = X T, for the panel at column k: thread t owns panel row t
// (Y and W rows in registers); V^T Y through shared memory, 256 rows at a time, thread
// (i, j) summing entry (i, j).  W goes into the W halves of L and R as pairs.
constexpr int SB_WCH = 256;
constexpr size_t sb_w_smem() { return sizeof(float) * 2 * SB_WCH * (SB_B + 1); }

__global__ void __launch_bounds__(SB_NT, 1) k_sb_w(SbArgs g, int k) {
    extern __shared__ __align__(16) float wsm[];
    float *Vs = wsm, *Ys = wsm + SB_WCH * (SB_B + 1);
    __shared__ float Ts[32][33], Zs[32][33], Ms[32][33];
    const int t = threadIdx.x, mat = blockIdx.x, m = g.n - k - SB_B;
    const bool own = t < m;
    const float *Tg = g.T + (size_t)mat * SB_B * SB_B;
    Ts[t >> 5][t & 31] = Tg[t];
    __syncthreads();
    float y[SB_B];
    const float *vf = g.Vf + (size_t)mat * g.sVX + (size_t)t * SB_B;
    {
        const float *x = g.X + (size_t)mat * g.sVX + (size_t)t * SB_B;
        #pragma unroll
        for (int j = 0; j < SB_B; j++) y[j] = 0.f;
        #pragma unroll 4
        for (int l = 0; l < SB_B; l++) {
            const float xl = own ? x[l] : 0.f;
            #pragma unroll
            for (int j = 0; j < SB_B; j++) y[j] = fmaf(xl, Ts[l][j], y[j]);
        }
    }
    const int zi = t >> 5, zj = t & 31;
    float z = 0.f;
    for (int r0 = 0; r0 < m; r0 += SB_WCH) {
        if (own && t >= r0 && t < r0 + SB_WCH) {
            #pragma unroll
            for (int j = 0; j < SB_B; j++) {
                Vs[(t - r0) * (SB_B + 1) + j] = vf[j];
                Ys[(t - r0) * (SB_B + 1) + j] = y[j];
            }
        }
        __syncthreads();
        const int rows = min(SB_WCH, m - r0);
        for (int r = 0; r < rows; r++) z = fmaf(Vs[r * (SB_B + 1) + zi], Ys[r * (SB_B + 1) + zj], z);
        __syncthreads();
    }
    Zs[zi][zj] = z;
    __syncthreads();
    float mm = 0.f;   // M = T^T Z
    for (int l = 0; l < SB_B; l++) mm = fmaf(Ts[l][zi], Zs[l][zj], mm);
    Ms[zi][zj] = mm;
    __syncthreads();
    if (!own) return;
    const size_t olr = (size_t)mat * g.sLR + (size_t)t * 2 * SB_B;
    #pragma unroll 4
    for (int i = 0; i < SB_B; i++) {
        const float hv = -0.5f * vf[i];
        #pragma unroll
        for (int j = 0; j < SB_B; j++) y[j] = fmaf(hv, Ms[i][j], y[j]);
    }
    #pragma unroll
    for (int j = 0; j < SB_B; j++) {
        pair_put(g.L.hi, g.L.lo, olr + SB_B + j, y[j]);
        pair_put(g.R.hi, g.R.lo, olr + j, y[j]);
    }
}

// Bulge chasing (stage 2), one block of SB_CW warps per matrix.  Time step tt: sweep c runs
// step kk = tt - SB_LAG c on warp c % SB_CW (sweeps c and c + SB_CW never overlap in time
// while a sweep has at most SB_LAG * SB_CW steps).  Step kk of sweep c, rows rk = c+1+kk*SB_B
// .. rk+L-1: the reflector that annihilates column c (kk = 0) or the first column of the
// bulge block B_kk = A[rk.., rk-SB_B..rk-1] below row rk; it is applied from the left to B_kk,
// from both sides to the diagonal block D = A[rk.., rk..] and from the right to the block
// below, B_kk+1 = A[rk+L.., rk..].
__device__ __forceinline__ float &bd_at(float *Bd, int r, int c) { return Bd[(size_t)c * SB_LDB + (r - c)]; }

// Sum over the 32 lanes of u[c] * (lane's value), for c = 0..31 at once: lane l ends with
// the sum for c = l (halving exchanges, 31 shuffles).
__device__ __forceinline__ float col_sums(const float (&a)[SB_B], float f, int lane) {
    float u[SB_B / 2];
    {
        const bool up = (lane & 16) != 0;
        #pragma unroll
        for (int c = 0; c < 16; c++) {
            const float lo = f * a[c], hi = f * a[c + 16];
            u[c] = (up ? hi : lo) + __shfl_xor_sync(0xffffffffu, up ? lo : hi, 16);
        }
    }
    #pragma unroll
    for (int h = 8; h >= 1; h >>= 1) {
        const bool up = (lane & h) != 0;
        #pragma unroll
        for (int c = 0; c < h; c++) {
            const float send = up ? u[c] : u[c + h], keep = up ? u[c + h] : u[c];
            u[c] = keep + __shfl_xor_sync(0xffffffffu, send, h);
        }
    }
    return u[0];
}

__global__ void __launch_bounds__(32 * SB_CW, 3) k_sb_chase(SbArgs g) {
    __shared__ float vs[SB_CW][32], zs[SB_CW][32];
    const int n = g.n, mat = blockIdx.x, lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    float *Bd = g.Bd + (size_t)mat * g.sBd;
    const int nsw = n - 2;
    auto nsteps = [&](int c) { return (n - 1 - c + SB_B - 1) / SB_B; };
    const int tmax = nsw > 0 ? SB_LAG * (nsw - 1) + nsteps(0) : 0;
    for (int tt = 0; tt < tmax; tt++) {
        int c = -1, kk = 0;
        if (tt >= SB_LAG * w) {
            const int q = (tt - SB_LAG * w) / (SB_LAG * SB_CW);
            c = w + SB_CW * q;
            kk = tt - SB_LAG * c;
            if (c >= nsw || kk >= nsteps(c)) c = -1;
        }
        if (c >= 0) {
            // lane i works on row i of each block: every load and store covers consecutive
            // offsets of one column of the band
            const int rk = c + 1 + kk * SB_B, L = min(SB_B, n - rk), r2 = rk + L, L2 = min(SB_B, n - r2);
            const int col = kk == 0 ? c : rk - SB_B;
            const int nbc = rk - col;   // columns of B_kk (1 when kk = 0: column c itself)
            const bool row = lane < L;
            float a[SB_B];
            #pragma unroll
            for (int j = 0; j < SB_B; j++) a[j] = (row && j < nbc) ? bd_at(Bd, rk + lane, col + j) : 0.f;
            // the reflector from column 0 of B_kk
            const float xi = a[0];
            const float xn2 = warp_sum((lane >= 1 && row) ? xi * xi : 0.f);
            const float alpha = __shfl_sync(0xffffffffu, xi, 0);
            float tau = 0.f, beta = alpha, scale = 0.f;
            if (xn2 > 0.f) {
                beta = -copysignf(sqrtf(alpha * alpha + xn2), alpha);
                tau = (beta - alpha) / beta;
                scale = 1.f / (alpha - beta);
            }
            const float vl = lane == 0 ? 1.f : (row ? xi * scale : 0.f);
            vs[w][lane] = vl;
            // B_kk <- H B_kk: s_j = v . column j, row i -= tau v_i s_j; column 0 becomes beta e_0
            zs[w][lane] = col_sums(a, vl, lane);
            __syncwarp();
            if (row) {
                bd_at(Bd, rk + lane, col) = lane == 0 ? beta : 0.f;
                #pragma unroll
                for (int j = 1; j < SB_B; j++)
                    if (j < nbc) bd_at(Bd, rk + lane, col + j) = fmaf(-tau * vl, zs[w][j], a[j]);
            }
            __syncwarp();
            // D <- H D H: row i of the lower part in lane i (D[i][j], j <= i); p = tau D v with
            // the part above the diagonal, D[i][j] = D[j][i], as column sums of the rows below
            #pragma unroll
            for (int j = 0; j < SB_B; j++) a[j] = (row && j <= lane) ? bd_at(Bd, rk + lane, rk + j) : 0.f;
            float p = 0.f;
            #pragma unroll
            for (int j = 0; j < SB_B; j++) p = fmaf(a[j], vs[w][j], p);
            {
                float b[SB_B];
                #pragma unroll
                for (int j = 0; j < SB_B; j++) b[j] = j < lane ? a[j] : 0.f;
                p += col_sums(b, vl, lane);
            }
            p *= tau;
            const float vp = warp_sum(vl * p);
            const float zl = fmaf(-0.5f * tau * vp, vl, p);
            zs[w][lane] = zl;
            __syncwarp();
            if (row) {
                #pragma unroll
                for (int j = 0; j < SB_B; j++)
                    if (j <= lane) bd_at(Bd, rk + lane, rk + j) = a[j] - (vl * zs[w][j] + zl * vs[w][j]);
            }
            // B_kk+1 <- B_kk+1 H, lane = row
            if (lane < L2) {
                #pragma unroll
                for (int j = 0; j < SB_B; j++) a[j] = j < L ? bd_at(Bd, r2 + lane, rk + j) : 0.f;
                float s2 = 0.f;
                #pragma unroll
                for (int j = 0; j < SB_B; j++) s2 = fmaf(a[j], vs[w][j], s2);
                #pragma unroll
                for (int j = 0; j < SB_B; j++)
                    if (j < L) bd_at(Bd, r2 + lane, rk + j) = fmaf(-tau * s2, vs[w][j], a[j]);
            }
            __syncwarp();
        }
        __syncthreads();
    }
}

__global__ void k_sb_out(SbArgs g, int nmat, float *d, float *e) {
    const int n = g.n;
    for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < (size_t)nmat * n;
         idx += (size_t)gridDim.x * blockDim.x) {
        const int mat = (int)(idx / n), c = (int)(idx % n);
        const float *Bd = g.Bd + (size_t)mat * g.sBd;
        d[idx] = Bd[(size_t)c * SB_LDB] + g.sig[mat];
        e[idx] = c + 1 < n ? Bd[(size_t)c * SB_LDB + 1] : 0.f;
    }
}

}  // namespace

int cir_sbr_max_n() { return SB_LAG * SB_CW * SB_B + 1; }

// bytes of work area per matrix of order n (leading dimension ld, a multiple of 8)
size_t cir_sbr_bytes(int n, int ld) {
    auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
    return al((size_t)4 * n * ld) + al((size_t)4 * SB_B * ld) + 2 * al((size_t)8 * n * SB_B) + 2 * al((size_t)4 * n * SB_B) +
           al((size_t)4 * SB_B * SB_B) + al((size_t)4 * n * SB_LDB) + 256;
}

// The two-stage reduction of nmat matrices (H: column-major, leading dimension ld, a multiple
// of 8, batch stride sH) to tridiagonal form: d and e (n per matrix) receive the diagonal and
// subdiagonal.  work: cir_sbr_bytes(n, ld) per matrix.  ms (optional, 2): the device time of
// stage 1 and stage 2 in ms (the call then waits for the stream).
cudaError_t cir_launch_sbr(const float *H, long long sH, int nmat, int n, int ld, float *d, float *e, void *work,
                           int *err, cudaStream_t s, float *ms, int *launches) {
    if (n < 3 || n > cir_sbr_max_n() || (ld & 7) || ld < n || nmat < 1 || nmat > 65535) return cudaErrorInvalidValue;
    auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
    unsigned char *q = static_cast<unsigned char *>(work);
    auto take = [&](size_t per) {
        unsigned char *r = q;
        q += al(per) * nmat;
        return r;
    };
    SbArgs g{};
    g.n = n;
    g.ld = ld;
    g.sS = (long long)n * ld;
    __nv_bfloat16 *sb = reinterpret_cast<__nv_bfloat16 *>(take((size_t)4 * n * ld));
    g.S = SplitMat{sb, sb + (size_t)nmat * g.sS};
    g.sVc = (long long)SB_B * ld;
    __nv_bfloat16 *vb = reinterpret_cast<__nv_bfloat16 *>(take((size_t)4 * SB_B * ld));
    g.Vc = SplitMat{vb, vb + (size_t)nmat * g.sVc};
    g.sLR = (long long)n * 2 * SB_B;
    __nv_bfloat16 *lb = reinterpret_cast<__nv_bfloat16 *>(take((size_t)8 * n * SB_B));
    __nv_bfloat16 *rb = reinterpret_cast<__nv_bfloat16 *>(take((size_t)8 * n * SB_B));
    g.L = SplitMat{lb, lb + (size_t)nmat * g.sLR};
    g.R = SplitMat{rb, rb + (size_t)nmat * g.sLR};
    g.sVX = (long long)n * SB_B;
    g.Vf = reinterpret_cast<float *>(take((size_t)4 * n * SB_B));
    g.X = reinterpret_cast<float *>(take((size_t)4 * n * SB_B));
    g.T = reinterpret_cast<float *>(take((size_t)4 * SB_B * SB_B));
    g.sBd = (long long)n * SB_LDB;
    g.Bd = reinterpret_cast<float *>(take((size_t)4 * n * SB_LDB));
    g.sig = reinterpret_cast<float *>(take(4));
    g.err = err;
    cudaEvent_t ev[3] = {};
    cudaError_t e0 = cudaSuccess;
    if (ms)
        for (auto &x : ev)
            if ((e0 = cudaEventCreate(&x)) != cudaSuccess) return e0;
    auto fin = [&](cudaError_t r) {
        if (ms)
            for (auto &x : ev) cudaEventDestroy(x);
        return r;
    };
    int nl = 0;
    if (ms) cudaEventRecord(ev[0], s);
    k_sb_shift<<<nmat, 256, 0, s>>>(H, sH, g);
    k_sb_split<<<dim3((n + 7) / 8, nmat), 256, 0, s>>>(H, sH, g);
    nl += 2;
    if ((e0 = cudaFuncSetAttribute(k_sb_w, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sb_w_smem())) != cudaSuccess)
        return fin(e0);
    for (int k = 0;; k += SB_B) {
        const int m = n - k - SB_B;
        k_sb_panel<<<nmat, SB_NT, 0, s>>>(g, k);
        nl++;
        if ((e0 = cudaGetLastError()) != cudaSuccess) return fin(e0);
        if (m < 1) break;
        SplitGemmArgs x{};                                         // X = A22 V
        x.Ahi = g.S.hi + (size_t)(k + SB_B) * ld + k + SB_B; x.Alo = g.S.lo + (size_t)(k + SB_B) * ld + k + SB_B;
        x.lda = ld; x.sA = g.sS;
        x.Bhi = g.Vc.hi; x.Blo = g.Vc.lo; x.ldb = ld; x.sB = g.sVc;
        x.Cf = g.X; x.ldc = SB_B; x.sC = g.sVX; x.out_mode = 2;
        x.M = m; x.N = SB_B; x.K = m;
        x.err = err;
        x.tile_n = 128;
        if ((e0 = cir_launch_split_gemm(x, nmat, s, &nl)) != cudaSuccess) return fin(e0);
        k_sb_w<<<nmat, SB_NT, sb_w_smem(), s>>>(g, k);
        nl++;
        if ((e0 = cudaGetLastError()) != cudaSuccess) return fin(e0);
        SplitGemmArgs u{};                                         // A22 -= V W^T + W V^T
        u.Ahi = g.L.hi; u.Alo = g.L.lo; u.lda = 2 * SB_B; u.sA = g.sLR;
        u.Bhi = g.R.hi; u.Blo = g.R.lo; u.ldb = 2 * SB_B; u.sB = g.sLR;
        u.epilogue = 2;
        u.Dhi = u.Chi = g.S.hi + (size_t)(k + SB_B) * ld + k + SB_B;
        u.Dlo = u.Clo = g.S.lo + (size_t)(k + SB_B) * ld + k + SB_B;
        u.ldd = u.ldc = ld; u.sD = u.sC = g.sS; u.out_mode = 1;
        u.M = u.N = m; u.K = 2 * SB_B;
        u.err = err;
        if ((e0 = cir_launch_split_gemm(u, nmat, s, &nl)) != cudaSuccess) return fin(e0);
    }
    if (ms) cudaEventRecord(ev[1], s);
    k_sb_chase<<<nmat, 32 * SB_CW, 0, s>>>(g);
    nl++;
    if ((e0 = cudaGetLastError()) != cudaSuccess) return fin(e0);
    if (ms) cudaEventRecord(ev[2], s);
    k_sb_out<<<256, 256, 0, s>>>(g, nmat, d, e);
    nl++;
    if ((e0 = cudaGetLastError()) != cudaSuccess) return fin(e0);
    if (launches) *launches += nl;
    if (ms) {
        if ((e0 = cudaEventSynchronize(ev[2])) != cudaSuccess) return fin(e0);
        cudaEventElapsedTime(ms, ev[0], ev[1]);
        cudaEventElapsedTime(ms + 1, ev[1], ev[2]);
    }
    return fin(cudaSuccess);
}
