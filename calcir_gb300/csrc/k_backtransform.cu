// Householder back-transform of the divide-and-conquer eigensolver: the eigenvectors of H
// are V = Q_H Q_T, where Q_H = H_0 H_1 ... H_{n-3} holds the reflectors of the
// tridiagonalisation (H_k = I - tau_k v_k v_k^T, v_k stored below the subdiagonal of
// column k of A with v_k[k+1] = 1 implied, tau in DE row 2; LAPACK ssytrd lower storage)
// and Q_T the eigenvectors of the tridiagonal matrix.  magma_ssyevd (calcIR.cu:420-448)
// does the same with sormtr after stedc.  Q_H is never formed: the reflectors are applied
// to Q_T in blocks of BT_NB in the compact WY form (LAPACK slarft, forward, columnwise),
//     H_kb ... H_kb+nb-1 = I - V T V^T,   Z <- Z - V (T (V^T Z)),
// from the last block to the first.  Q_T is column-major, so its transpose is a row-major
// view in which each block is two batched GEMMs (tensor cores in the mixed forms):
//     P = Z^T[:, kb:] V_b                   n x nb, K = n - kb, V_b read K-major from A
//     Z^T[:, kb:] = Z^T[:, kb:] - P Y_b     Y_b = T^T V_b^T, nb x (n - kb)
// The first block's update (kb = 0 covers the whole matrix) writes its result into A.
// 2 n^3 flops in all, against 4/3 n^3 to form Q_H and 2 n^3 to multiply it out.
//
// k_bt_prep (one thread block per reflector block and matrix) runs first: it writes the
// implied zeros and unit of V_b into A (rows kb..k+1 of column k), forms G = V_b^T V_b,
// T by the slarft recursion T[i][j] = -tau_j sum_{i <= l < j} T[i][l] G[l][j],
// T[j][j] = tau_j, and Y_b into rows kb.. of Z (Y[kb+j][r] for r >= kb).
#include "cir_device.cuh"

#include <cstdlib>
#include <vector>

namespace {

constexpr int BT_NB = 128;              // reflectors per block
constexpr int BT_RC = 64;               // rows of V_b staged per step
constexpr int BT_NT = 256;
constexpr int BT_LDM = BT_NB + 4;       // shared row strides (float4 aligned, conflict-free)
constexpr int BT_LDV = BT_RC + 4;

constexpr size_t bt_prep_smem() { return sizeof(float) * ((size_t)BT_NB * BT_LDM + (size_t)BT_NB * BT_LDV + BT_NB); }

// Stage rows r0..r0+BT_RC-1 of V_b as Vt[j][r - r0] (j = reflector of the block), with the
// implied entries: 0 above row k+1, 1 at row k+1, 0 for rows >= n and for j >= nbb.  When
// `clean`, the implied entries are also written into A, so that the GEMMs can read V_b
// from A directly.  Thread t covers rows r0 + 4 (t & 15) .. +3 of columns (t >> 4) + 16 q:
// 16 threads read one column's 64 rows as 256 contiguous bytes.
__device__ __forceinline__ void bt_stage(float *A, int ld, int n, int kb, int nbb, int r0, bool clean, float *Vt) {
    const int t = threadIdx.x;
    const int rr = 4 * (t & 15), r = r0 + rr;
    #pragma unroll 2
    for (int q = 0; q < BT_NB / 16; q++) {
        const int j = (t >> 4) + 16 * q, k = kb + j;
        float x[4] = {0.f, 0.f, 0.f, 0.f};
        if (j < nbb) {
            float *col = A + (size_t)k * ld;
            if (r + 3 < n) {
                const float4 g = *reinterpret_cast<const float4 *>(col + r);
                x[0] = g.x; x[1] = g.y; x[2] = g.z; x[3] = g.w;
            } else {
                #pragma unroll
                for (int i = 0; i < 4; i++) x[i] = r + i < n ? col[r + i] : 0.f;
            }
            #pragma unroll
            for (int i = 0; i < 4; i++) {
                const int row = r + i;
                if (row <= k + 1) {
                    x[i] = row == k + 1 ? 1.f : 0.f;
                    if (clean && row < n) col[row] = x[i];
                }
            }
        }
        *reinterpret_cast<float4 *>(Vt + j * BT_LDV + rr) = make_float4(x[0], x[1], x[2], x[3]);
    }
}

// Outputs of the split form of the prep (the mixed forms): V_b and Y_b^T as BF16 hi/lo pairs.
struct BtSplit {
    SplitMat V;        // V[(kb + j)*ldq + r]: column kb + j of the cleaned reflectors, rows kb..
    SplitMat Yt;       // block b at Yt + bt_yoff(b, n, ldy): Y_b^T, (n - kb) rows of ldy
    int ldq, ldy;      // ldy = min(BT_NB, n - 2 rounded up to 8): the width of a block
    long long sV, sY;  // per-matrix strides (elements)
};

// offset of block b's Y_b^T: the (n - kb') x ldy blocks of the blocks before it
__host__ __device__ inline long long bt_yoff(int b, int n, int ldy) {
    return (long long)ldy * ((long long)b * n - (long long)BT_NB * b * (b - 1) / 2);
}

// The paired layout (blocks 2q and 2q+1 applied as one block of 2*BT_NB reflectors): pair q's
// Y^T is (n - 2*BT_NB*q) x (2*BT_NB), row-major, from row 2*BT_NB*q; block 2q fills its left
// half, block 2q+1 its right half (zero in the first BT_NB rows, above its reflectors)
__host__ __device__ inline long long bt_yoff2(int q, int n) {
    return 2LL * BT_NB * ((long long)q * n - 2LL * BT_NB * q * (q - 1) / 2);
}

template <bool SPLIT>
__global__ void __launch_bounds__(BT_NT, 2) k_bt_prep(EighArgs a, BtSplit sp) {
    extern __shared__ __align__(16) float bsm[];
    float *M = bsm;                           // [BT_NB][BT_LDM]: G, then T^T (M[j][i] = T[i][j])
    float *Vt = M + BT_NB * BT_LDM;           // [BT_NB][BT_LDV]
    float *tau = Vt + BT_NB * BT_LDV;         // [BT_NB]
    const int n = a.n, ld = a.ld, mat = blockIdx.y;
    const int kb = blockIdx.x * BT_NB, nbb = min(BT_NB, n - 2 - kb);
    float *A = a.A + (size_t)mat * a.mstride;
    float *Y = a.Z + (size_t)mat * a.mstride;
    const float *tau_g = a.DE + (size_t)mat * 3 * ld + 2 * ld;
    const int t = threadIdx.x;
    if (t < BT_NB) tau[t] = t < nbb ? tau_g[kb + t] : 0.f;

    // G = V_b^T V_b: thread (tx, ty) accumulates G[ty + 16 p][tx + 16 q] for p <= q only: the
    // T recursion reads G above the diagonal, and the tiles p > q lie strictly below it
    {
        const int tx = t & 15, ty = t >> 4;
        float acc[8][8];
        #pragma unroll
        for (int p = 0; p < 8; p++)
            #pragma unroll
            for (int q = 0; q < 8; q++) acc[p][q] = 0.f;
        for (int r0 = kb; r0 < n; r0 += BT_RC) {
            __syncthreads();
            bt_stage(A, ld, n, kb, nbb, r0, !SPLIT, Vt);
            __syncthreads();
            if (SPLIT) {   // the cleaned chunk as a split pair: column kb + j, rows r0..
                const size_t ov = (size_t)mat * sp.sV;
                for (int idx = t; idx < BT_NB * BT_RC; idx += BT_NT) {
                    const int j = idx / BT_RC, rr = idx - j * BT_RC, r = r0 + rr;
                    if (j < nbb && r < n) {
                        const float x = Vt[j * BT_LDV + rr];
                        const __nv_bfloat16 h = __float2bfloat16_rn(x);
                        const size_t o = ov + (size_t)(kb + j) * sp.ldq + r;
                        sp.V.hi[o] = h;
                        sp.V.lo[o] = __float2bfloat16_rn(x - __bfloat162float(h));
                    }
                }
            }
            #pragma unroll 1
            for (int rr = 0; rr < BT_RC; rr += 4) {
                float4 va[8];
                #pragma unroll
                for (int p = 0; p < 8; p++) va[p] = *reinterpret_cast<const float4 *>(Vt + (ty + 16 * p) * BT_LDV + rr);
                #pragma unroll
                for (int q = 0; q < 8; q++) {
                    const float4 vb = *reinterpret_cast<const float4 *>(Vt + (tx + 16 * q) * BT_LDV + rr);
                    #pragma unroll
                    for (int p = 0; p <= q; p++)
                        acc[p][q] = fmaf(va[p].x, vb.x, fmaf(va[p].y, vb.y, fmaf(va[p].z, vb.z, fmaf(va[p].w, vb.w, acc[p][q]))));
                }
            }
        }
        #pragma unroll
        for (int p = 0; p < 8; p++)
            #pragma unroll
            for (int q = p; q < 8; q++) M[(ty + 16 * p) * BT_LDM + tx + 16 * q] = acc[p][q];
    }
    __syncthreads();
    // T, column by column; T[i][l] (i <= l) is kept at M[l][i], which the recursion never
    // reads as G (it reads G[l][j], l < j, from the untouched upper part M[l][j])
    for (int j = 0; j < BT_NB; j++) {
        if (t < j) {
            float s = 0.f;
            for (int l = 0; l < j; l++) s = fmaf(l >= t ? M[l * BT_LDM + t] : 0.f, M[l * BT_LDM + j], s);
            M[j * BT_LDM + t] = -tau[j] * s;
        } else if (t == j) {
            M[j * BT_LDM + j] = tau[j];
        }
        __syncthreads();
    }
    for (int idx = t; idx < BT_NB * BT_NB; idx += BT_NT) {   // T[i][j] = 0 for i > j
        const int j = idx / BT_NB, i = idx - j * BT_NB;
        if (i > j) M[j * BT_LDM + i] = 0.f;
    }
    // Y[kb + j][r] = sum_i T[i][j] V[r][i] = sum_i M[j][i] Vt[i][r]: thread (tr, tj) computes
    // rows j = tj + 16 q, columns r0 + 4 tr .. +3 of each chunk
    const int tr = t & 15, tj = t >> 4;
    for (int r0 = kb; r0 < n; r0 += BT_RC) {
        __syncthreads();
        bt_stage(A, ld, n, kb, nbb, r0, false, Vt);
        __syncthreads();
        float acc[8][4];
        #pragma unroll
        for (int q = 0; q < 8; q++)
            #pragma unroll
            for (int c = 0; c < 4; c++) acc[q][c] = 0.f;
        #pragma unroll 1
        for (int i = 0; i < BT_NB; i += 4) {
            float4 v[4];
            #pragma unroll
            for (int p = 0; p < 4; p++) v[p] = *reinterpret_cast<const float4 *>(Vt + (i + p) * BT_LDV + 4 * tr);
            #pragma unroll
            for (int q = 0; q < 8; q++) {
                const float4 m = *reinterpret_cast<const float4 *>(M + (tj + 16 * q) * BT_LDM + i);
                const float mm[4] = {m.x, m.y, m.z, m.w};
                #pragma unroll
                for (int p = 0; p < 4; p++) {
                    acc[q][0] = fmaf(mm[p], v[p].x, acc[q][0]);
                    acc[q][1] = fmaf(mm[p], v[p].y, acc[q][1]);
                    acc[q][2] = fmaf(mm[p], v[p].z, acc[q][2]);
                    acc[q][3] = fmaf(mm[p], v[p].w, acc[q][3]);
                }
            }
        }
        if (SPLIT) {
            // Y_b^T rows r0..r0+63 through shared memory (Vt is free once every thread has
            // its products), then 32 values of one row per thread as a split pair
            __syncthreads();
            float *Ts = Vt;   // [BT_RC][BT_NB + 1]
            #pragma unroll
            for (int q = 0; q < 8; q++)
                #pragma unroll
                for (int c = 0; c < 4; c++) Ts[(4 * tr + c) * (BT_NB + 1) + tj + 16 * q] = acc[q][c];
            __syncthreads();
            const int rl = t >> 2, j0 = (t & 3) * 32, r = r0 + rl;
            if (r < n) {
                const size_t o = (size_t)mat * sp.sY + bt_yoff(blockIdx.x, n, sp.ldy) + (size_t)(r - kb) * sp.ldy + j0;
                #pragma unroll
                for (int q = 0; q < 32; q += 8) {
                    if (j0 + q >= sp.ldy) break;
                    uint32_t ph[4], pl[4];
                    #pragma unroll
                    for (int u = 0; u < 8; u += 2) {
                        const float x0 = j0 + q + u < nbb ? Ts[rl * (BT_NB + 1) + j0 + q + u] : 0.f;
                        const float x1 = j0 + q + u + 1 < nbb ? Ts[rl * (BT_NB + 1) + j0 + q + u + 1] : 0.f;
                        const __nv_bfloat16 h0 = __float2bfloat16_rn(x0), h1 = __float2bfloat16_rn(x1);
                        const __nv_bfloat16 l0 = __float2bfloat16_rn(x0 - __bfloat162float(h0));
                        const __nv_bfloat16 l1 = __float2bfloat16_rn(x1 - __bfloat162float(h1));
                        ph[u / 2] = (uint32_t)__bfloat16_as_ushort(h0) | ((uint32_t)__bfloat16_as_ushort(h1) << 16);
                        pl[u / 2] = (uint32_t)__bfloat16_as_ushort(l0) | ((uint32_t)__bfloat16_as_ushort(l1) << 16);
                    }
                    *reinterpret_cast<uint4 *>(sp.Yt.hi + o + q) = make_uint4(ph[0], ph[1], ph[2], ph[3]);
                    *reinterpret_cast<uint4 *>(sp.Yt.lo + o + q) = make_uint4(pl[0], pl[1], pl[2], pl[3]);
                }
            }
        } else {
            const int r = r0 + 4 * tr;
            #pragma unroll
            for (int q = 0; q < 8; q++) {
                const int j = tj + 16 * q;
                if (j >= nbb) continue;
                float *y = Y + (size_t)(kb + j) * ld + r;
                if (r + 3 < n) {
                    *reinterpret_cast<float4 *>(y) = make_float4(acc[q][0], acc[q][1], acc[q][2], acc[q][3]);
                } else {
                    #pragma unroll
                    for (int c = 0; c < 4; c++)
                        if (r + c < n) y[c] = acc[q][c];
                }
            }
        }
    }
}

// Q as a split pair in the same layout (column c at Q[c*ld ..], rows 0..n-1).
// Q as a split pair (the same layout, rows of ld), eight rows per block: 16-byte loads and
// 8-byte stores of four BF16; values past n are zero.  ld is a multiple of 8 on this path.
constexpr int BT_SQ_ROWS = 8;

__global__ void __launch_bounds__(256) k_bt_split_q(const float *Q, long long sQ, int n, int ld, SplitMat Qs,
                                                    long long sS) {
    const int mat = blockIdx.y, n4 = (n + 3) >> 2, c0 = blockIdx.x * BT_SQ_ROWS;
    for (int idx = threadIdx.x; idx < BT_SQ_ROWS * n4; idx += blockDim.x) {
        const int cr = idx / n4, r = 4 * (idx - cr * n4), c = c0 + cr;
        if (c >= n) break;
        float4 x = *reinterpret_cast<const float4 *>(Q + (size_t)mat * sQ + (size_t)c * ld + r);
        if (r + 1 >= n) x.y = 0.f;
        if (r + 2 >= n) x.z = 0.f;
        if (r + 3 >= n) x.w = 0.f;
        const __nv_bfloat162 h0 = __floats2bfloat162_rn(x.x, x.y), h1 = __floats2bfloat162_rn(x.z, x.w);
        const __nv_bfloat162 l0 = __floats2bfloat162_rn(x.x - __bfloat162float(h0.x), x.y - __bfloat162float(h0.y));
        const __nv_bfloat162 l1 = __floats2bfloat162_rn(x.z - __bfloat162float(h1.x), x.w - __bfloat162float(h1.y));
        const size_t o = (size_t)mat * sS + (size_t)c * ld + r;
        uint2 hv, lv;
        hv.x = *reinterpret_cast<const uint32_t *>(&h0);
        hv.y = *reinterpret_cast<const uint32_t *>(&h1);
        lv.x = *reinterpret_cast<const uint32_t *>(&l0);
        lv.y = *reinterpret_cast<const uint32_t *>(&l1);
        *reinterpret_cast<uint2 *>(Qs.hi + o) = hv;
        *reinterpret_cast<uint2 *>(Qs.lo + o) = lv;
    }
}

// The split form's preparation on tensor cores, in four launches instead of k_bt_prep<1>:
//   k_bt_clean  V_b with its implied zeros and unit as a split pair in two layouts: columns
//               (the product P = Z^T V_b and G read it K-major over rows) and rows (the
//               block's Y_b^T region, which the product Y_b^T = V_b T reads K-major over
//               reflectors and then overwrites in place)
//   G_b = V_b^T V_b on the persistent split-BF16 GEMM (FP32 out)
//   k_bt_tmat   T by the slarft recursion from G_b and tau, stored transposed as a pair
//   Y_b^T = V_b T on the persistent GEMM, in place over V_b's row layout
// One thread block per reflector block and matrix: rows kb.. in chunks of BT_RC staged
// like k_bt_prep's, written as pairs column-wise and, transposed through shared memory,
// row-wise (columns j >= nbb of the row layout are zero).
// eight values as BF16 hi and lo words at 16-byte aligned hi and lo
__device__ __forceinline__ void store_pair8(__nv_bfloat16 *hi, __nv_bfloat16 *lo, const float (&x)[8]) {
    uint32_t h[4], l[4];
    #pragma unroll
    for (int e = 0; e < 8; e += 2) {
        const __nv_bfloat162 hh = __floats2bfloat162_rn(x[e], x[e + 1]);
        const __nv_bfloat162 ll = __floats2bfloat162_rn(x[e] - __bfloat162float(hh.x), x[e + 1] - __bfloat162float(hh.y));
        h[e / 2] = *reinterpret_cast<const uint32_t *>(&hh);
        l[e / 2] = *reinterpret_cast<const uint32_t *>(&ll);
    }
    *reinterpret_cast<uint4 *>(hi) = make_uint4(h[0], h[1], h[2], h[3]);
    *reinterpret_cast<uint4 *>(lo) = make_uint4(l[0], l[1], l[2], l[3]);
}

// PAIRED: the row layout in the paired form (bt_yoff2), and both layouts from the pair's first
// row, so that the second block's columns hold zeros above its reflectors.
template <bool PAIRED>
__global__ void __launch_bounds__(BT_NT) k_bt_clean(EighArgs a, BtSplit sp) {
    extern __shared__ __align__(16) float bsm[];
    float *Vt = bsm;                          // [BT_NB][BT_LDV]
    const int n = a.n, ld = a.ld, mat = blockIdx.y, b = blockIdx.x;
    const int kb = b * BT_NB, nbb = min(BT_NB, n - 2 - kb);
    const int rs = PAIRED ? (b & ~1) * BT_NB : kb;         // first row written
    const int ldy = PAIRED ? 2 * BT_NB : sp.ldy, wy = PAIRED ? BT_NB : sp.ldy;   // row stride, columns
    float *A = a.A + (size_t)mat * a.mstride;
    const size_t ov = (size_t)mat * sp.sV;
    const size_t oy = (size_t)mat * sp.sY + (PAIRED ? bt_yoff2(b >> 1, n) + (b & 1) * BT_NB : bt_yoff(b, n, sp.ldy));
    const int t = threadIdx.x;
    for (int r0 = rs; r0 < n; r0 += BT_RC) {
        __syncthreads();
        bt_stage(A, ld, n, kb, nbb, r0, false, Vt);
        __syncthreads();
        // the column layout 8 rows a thread, stored as 16-byte hi and lo words (ld is a multiple
        // of 8 and the rows start on 8-row boundaries; rows past n, zero in Vt, fall in the
        // column's padding below n)
        for (int idx = t; idx < BT_NB * (BT_RC / 8); idx += BT_NT) {   // column layout, rows contiguous
            const int j = idx / (BT_RC / 8), rr = 8 * (idx - j * (BT_RC / 8)), r = r0 + rr;
            if (j < nbb && r < n) {
                const float4 x0 = *reinterpret_cast<const float4 *>(Vt + j * BT_LDV + rr);
                const float4 x1 = *reinterpret_cast<const float4 *>(Vt + j * BT_LDV + rr + 4);
                const float x[8] = {x0.x, x0.y, x0.z, x0.w, x1.x, x1.y, x1.z, x1.w};
                const size_t o = ov + (size_t)(kb + j) * sp.ldq + r;
                store_pair8(sp.V.hi + o, sp.V.lo + o, x);
            }
        }
        for (int idx = t; idx < BT_RC * wy; idx += BT_NT) {  // row layout, reflectors contiguous
            const int rr = idx / wy, j = idx - rr * wy, r = r0 + rr;
            if (r < n) {
                const float x = j < nbb ? Vt[j * BT_LDV + rr] : 0.f;
                const __nv_bfloat16 h = __float2bfloat16_rn(x);
                const size_t o = oy + (size_t)(r - rs) * ldy + j;
                sp.Yt.hi[o] = h;
                sp.Yt.lo[o] = __float2bfloat16_rn(x - __bfloat162float(h));
            }
        }
    }
}

// T of one reflector block (LAPACK slarft, forward, columnwise) from G = V_b^T V_b (FP32,
// row-major BT_NB x BT_NB at Gb) and tau, written transposed as a pair, Tt[j*BT_NB + i] =
// T[i][j] (zero for i > j and for rows or columns past the block's reflectors).  Blocked:
// the four diagonal 32 x 32 blocks by the column recursion T[i][j] = -tau_j sum_{i <= l < j}
// T[i][l] G[l][j], T[j][j] = tau_j (a warp each), then the blocks above them by
// T_AB = -T_A G_AB T_B (the product of two compact-WY blocks), for the 32-column pairs (0,1),
// (2,3) and then the 64-column halves; the same T, with the long dependent chains of the
// plain recursion turned into products.  T[i][j] (i <= j) is kept at M[j][i], below the
// diagonal, where G (read above the diagonal only) is no longer needed.
constexpr size_t bt_tmat_smem() { return sizeof(float) * ((size_t)BT_NB * BT_LDM + BT_NB + 64 * 64); }

__global__ void __launch_bounds__(BT_NB) k_bt_tmat(EighArgs a, const float *Gb, SplitMat Tt, long long sG,
                                                  long long sT) {
    extern __shared__ __align__(16) float bsm[];
    float *M = bsm;                           // [BT_NB][BT_LDM]: G above the diagonal, T^T below
    float *tau = M + BT_NB * BT_LDM;          // [BT_NB]
    float *Ws = tau + BT_NB;                  // [64][64]: G_AB T_B
    const int n = a.n, ld = a.ld, mat = blockIdx.y, b = blockIdx.x;
    const int kb = b * BT_NB, nbb = min(BT_NB, n - 2 - kb);
    const float *G = Gb + (size_t)mat * sG + (size_t)b * BT_NB * BT_NB;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    tau[t] = t < nbb ? a.DE[(size_t)mat * 3 * ld + 2 * ld + kb + t] : 0.f;
    for (int l = 0; l < BT_NB; l++) M[l * BT_LDM + t] = (l < nbb && t < nbb) ? G[(size_t)l * BT_NB + t] : 0.f;
    __syncthreads();
    // the diagonal blocks: warp w, columns 32w + j, lane = row within the block
    {
        const int o = 32 * warp;
        for (int j = 0; j < 32; j++) {
            if (lane < j) {
                float s = 0.f;
                for (int l = lane; l < j; l++) s = fmaf(M[(o + l) * BT_LDM + o + lane], M[(o + l) * BT_LDM + o + j], s);
                M[(o + j) * BT_LDM + o + lane] = -tau[o + j] * s;
            } else if (lane == j) {
                M[(o + j) * BT_LDM + o + j] = tau[o + j];
            }
            __syncwarp();
        }
    }
    __syncthreads();
    // T_AB = -T_A (G_AB T_B) for blocks A = [a0, a0 + w), B = [a0 + w, a0 + 2w); thread u of
    // the NU threads on it computes column c = u % w of rows r0 .. r0 + R - 1, R = w*w / NU
    auto combine = [&](int a0, int w, int u, int NU, float *W) {
        constexpr int RMAX = 32;
        const int R = w * w / NU, c = u % w, r0 = (u / w) * R, b0 = a0 + w;
        float acc[RMAX];
        #pragma unroll
        for (int i = 0; i < RMAX; i++) acc[i] = 0.f;
        for (int k = 0; k <= c; k++) {          // W = G_AB T_B, T_B upper triangular
            const float tb = M[(b0 + c) * BT_LDM + b0 + k];
            #pragma unroll
            for (int i = 0; i < RMAX; i++)
                if (i < R) acc[i] = fmaf(M[(a0 + r0 + i) * BT_LDM + b0 + k], tb, acc[i]);
        }
        #pragma unroll
        for (int i = 0; i < RMAX; i++)
            if (i < R) W[(r0 + i) * w + c] = acc[i];
        __syncthreads();
        #pragma unroll
        for (int i = 0; i < RMAX; i++) acc[i] = 0.f;
        for (int k = r0; k < w; k++) {          // T_AB = -T_A W, T_A upper triangular
            const float wk = W[k * w + c];
            #pragma unroll
            for (int i = 0; i < RMAX; i++)
                if (i < R && r0 + i <= k) acc[i] = fmaf(M[(a0 + k) * BT_LDM + a0 + r0 + i], wk, acc[i]);
        }
        #pragma unroll
        for (int i = 0; i < RMAX; i++)
            if (i < R) M[(b0 + c) * BT_LDM + a0 + r0 + i] = -acc[i];
        __syncthreads();
    };
    combine(64 * (t >> 6), 32, t & 63, 64, Ws + (t >> 6) * 1024);   // pairs (0,1) and (2,3)
    combine(0, 64, t, BT_NB, Ws);                                     // halves
    const size_t o = (size_t)mat * sT + (size_t)b * BT_NB * BT_NB;
    for (int j = 0; j < BT_NB; j++) {   // thread t writes Tt[j][t] = T[t][j]: row j, contiguous in t
        const float x = t <= j ? M[j * BT_LDM + t] : 0.f;
        const __nv_bfloat16 h = __float2bfloat16_rn(x);
        Tt.hi[o + (size_t)j * BT_NB + t] = h;
        Tt.lo[o + (size_t)j * BT_NB + t] = __float2bfloat16_rn(x - __bfloat162float(h));
    }
}

// Pair q of reflector blocks (b1 = 2q, b2 = 2q + 1) applied as one block: with X = V_2^T V_1,
// T = [[T_1, -T_1 X^T T_2], [0, T_2]] and Y = T^T V^T = [Y_1; Y_2 - C Y_1], C = T_2^T X.
// k_bt_cross forms C (X in FP32 at X + q*BT_NB^2, row-major; T_2 from its pair in Tt) and
// writes it as a pair, row-major, at Cs + q*BT_NB^2.  Thread t computes column t % BT_NB of
// rows 64 (t / BT_NB) .. +63; X is masked to the blocks' nbb2 x nbb1 part, T_2 holds zeros
// outside its triangle.
constexpr int BT_CX_NT = 2 * BT_NB;
constexpr int BT_CX_LDT = BT_NB + 4;
constexpr size_t bt_cross_smem() { return sizeof(float) * ((size_t)BT_NB * BT_CX_LDT + (size_t)BT_NB * BT_NB); }

__global__ void __launch_bounds__(BT_CX_NT) k_bt_cross(EighArgs a, const float *X, SplitMat Tt, SplitMat Cs,
                                                      long long sX, long long sT) {
    extern __shared__ __align__(16) float bsm[];
    float *Ts = bsm;                          // Ts[l][i] = T_2[l][i]
    float *Xs = Ts + BT_NB * BT_CX_LDT;       // Xs[l][j] = X[l][j]
    const int q = blockIdx.x, mat = blockIdx.y, t = threadIdx.x, nrefl = a.n - 2;
    const int nbb1 = min(BT_NB, nrefl - 2 * q * BT_NB), nbb2 = min(BT_NB, nrefl - (2 * q + 1) * BT_NB);
    const float *Xg = X + (size_t)mat * sX + (size_t)q * BT_NB * BT_NB;
    const size_t to = (size_t)mat * sT + (size_t)(2 * q + 1) * BT_NB * BT_NB;
    for (int idx = t; idx < BT_NB * BT_NB; idx += BT_CX_NT) {
        const int r = idx / BT_NB, c = idx - r * BT_NB;   // Tt[r*BT_NB + c] = T_2[c][r]
        Ts[c * BT_CX_LDT + r] = __bfloat162float(Tt.hi[to + idx]) + __bfloat162float(Tt.lo[to + idx]);
        Xs[idx] = (r < nbb2 && c < nbb1) ? Xg[idx] : 0.f;
    }
    __syncthreads();
    const int j = t % BT_NB, i0 = 64 * (t / BT_NB);
    float acc[64];
    #pragma unroll
    for (int i = 0; i < 64; i++) acc[i] = 0.f;
    #pragma unroll 2
    for (int l = 0; l < BT_NB; l++) {
        const float x = Xs[l * BT_NB + j];
        const float4 *tr = reinterpret_cast<const float4 *>(Ts + l * BT_CX_LDT + i0);
        #pragma unroll
        for (int i4 = 0; i4 < 16; i4++) {
            const float4 tv = tr[i4];
            acc[4 * i4] = fmaf(tv.x, x, acc[4 * i4]);
            acc[4 * i4 + 1] = fmaf(tv.y, x, acc[4 * i4 + 1]);
            acc[4 * i4 + 2] = fmaf(tv.z, x, acc[4 * i4 + 2]);
            acc[4 * i4 + 3] = fmaf(tv.w, x, acc[4 * i4 + 3]);
        }
    }
    const size_t oc = (size_t)mat * sT + (size_t)q * BT_NB * BT_NB;
    #pragma unroll
    for (int i = 0; i < 64; i++) {
        const __nv_bfloat16 h = __float2bfloat16_rn(acc[i]);
        Cs.hi[oc + (size_t)(i0 + i) * BT_NB + j] = h;
        Cs.lo[oc + (size_t)(i0 + i) * BT_NB + j] = __float2bfloat16_rn(acc[i] - __bfloat162float(h));
    }
}

}  // namespace

// CIR_BT_TC=0: the split form's preparation in the one SIMT kernel k_bt_prep<1> (for comparison)
static bool bt_tc_enabled() {
    static const bool on = [] {
        const char *v = getenv("CIR_BT_TC");
        return !(v && v[0] == '0');
    }();
    return on;
}

// CIR_BT_PAIR=0: blocks of BT_NB reflectors in the split form's updates, not pairs of them
static bool bt_pair_enabled() {
    static const bool on = [] {
        const char *v = getenv("CIR_BT_PAIR");
        return !(v && v[0] == '0');
    }();
    return on;
}

static cudaError_t multi_gemm(std::vector<SplitGemmArgs> &g, int nmat, cudaStream_t s, int &nl) {
    std::vector<int> batch(g.size(), nmat);
    for (size_t i = 0; i < g.size(); i += CIR_SPLIT_MAXP) {
        const int np = (int)std::min<size_t>(CIR_SPLIT_MAXP, g.size() - i);
        const cudaError_t e = cir_launch_split_gemm_multi(g.data() + i, batch.data() + i, np, s, &nl);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// The split form in pairs of reflector blocks: blocks 2q and 2q+1 are applied as one block of
// 2*BT_NB reflectors (k_bt_cross), so Z is read and written half as often.  Per block as in
// backtransform_split's single-block preparation (clean, G, T, Y_b^T = V_b T), the row layout
// of V_b and so Y_b^T in the paired layout; then per pair X = V_2^T V_1, C = T_2^T X and the
// second half of Y^T less Y_1^T C^T; then per pair from the last, P = Z^T[:, kq:] V_q and
// Z^T[:, kq:] -= P Y_q.  G, T, X and C live in U, which the products P need only afterwards.
// Returns cudaErrorNotSupported when the work areas do not fit (the caller falls back).
static cudaError_t backtransform_paired(const EighArgs &a, const SplitMat &Qs, const SplitMat &Vs, const SplitMat &Ys,
                                        float *U, int nmat, int nblk, cudaStream_t s, int &nl) {
    const int n = a.n, ld = a.ld, nrefl = n - 2, npair = (nblk + 1) / 2, npf = nblk / 2;
    const long long ms = a.mstride, ss = 2 * a.mstride, B2 = (long long)BT_NB * BT_NB;
    if (nblk < 2 || ld < 2 * BT_NB || (2LL * nblk + 2LL * npf) * B2 > ms || bt_yoff2(npair, n) > ms ||
        (long long)n * 2 * BT_NB > ms)
        return cudaErrorNotSupported;
    auto nbb = [&](int b) { return min(BT_NB, nrefl - b * BT_NB); };
    float *Gb = U, *Xq = U + 2LL * nblk * B2;
    __nv_bfloat16 *tb = reinterpret_cast<__nv_bfloat16 *>(U + (long long)nblk * B2);
    __nv_bfloat16 *cb = reinterpret_cast<__nv_bfloat16 *>(U + (2LL * nblk + npf) * B2);
    const SplitMat Tt{tb, tb + nblk * B2}, Cs{cb, cb + npf * B2};
    const SplitMat Ps{reinterpret_cast<__nv_bfloat16 *>(U), reinterpret_cast<__nv_bfloat16 *>(U) + ms};
    const int ldy = 2 * BT_NB;
    auto yoff = [&](int b) { return bt_yoff2(b >> 1, n) + (b & 1) * BT_NB; };   // block b's row layout
    auto base = [&](SplitGemmArgs &g) {
        g = SplitGemmArgs{};
        g.err = a.err;
        g.test_stall = a.test_stall;
        g.tile_n = 128;
    };
    cudaError_t e;
    k_bt_clean<true><<<dim3(nblk, nmat), BT_NT, sizeof(float) * (size_t)BT_NB * BT_LDV, s>>>(
        a, BtSplit{Vs, Ys, ld, ldy, ss, ss});
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    nl += 1;
    std::vector<SplitGemmArgs> gx, ys, cr;
    for (int b = 0; b < nblk; b++) {   // G_b = V_b^T V_b
        const int kb = b * BT_NB;
        SplitGemmArgs g;
        base(g);
        g.Ahi = g.Bhi = Vs.hi + (size_t)kb * ld + kb; g.Alo = g.Blo = Vs.lo + (size_t)kb * ld + kb;
        g.lda = g.ldb = ld; g.sA = g.sB = ss;
        g.Cf = Gb + (size_t)b * B2; g.ldc = BT_NB; g.sC = ms; g.out_mode = 2;
        g.M = g.N = nbb(b); g.K = n - kb;
        gx.push_back(g);
    }
    for (int q = 0; q < npf; q++) {    // X_q = V_2^T V_1 over the rows of V_2
        const int k1 = 2 * q * BT_NB, k2 = k1 + BT_NB;
        SplitGemmArgs g;
        base(g);
        g.Ahi = Vs.hi + (size_t)k2 * ld + k2; g.Alo = Vs.lo + (size_t)k2 * ld + k2; g.lda = ld; g.sA = ss;
        g.Bhi = Vs.hi + (size_t)k1 * ld + k2; g.Blo = Vs.lo + (size_t)k1 * ld + k2; g.ldb = ld; g.sB = ss;
        g.Cf = Xq + (size_t)q * B2; g.ldc = BT_NB; g.sC = ms; g.out_mode = 2;
        g.M = nbb(2 * q + 1); g.N = nbb(2 * q); g.K = n - k2;
        gx.push_back(g);
    }
    if ((e = multi_gemm(gx, nmat, s, nl)) != cudaSuccess) return e;
    const size_t tsm = bt_tmat_smem();
    if ((e = cudaFuncSetAttribute(k_bt_tmat, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tsm)) != cudaSuccess)
        return e;
    k_bt_tmat<<<dim3(nblk, nmat), BT_NB, tsm, s>>>(a, Gb, Tt, ms, ss);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    nl += 1;
    if (npf > 0) {
        if ((e = cudaFuncSetAttribute(k_bt_cross, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bt_cross_smem())) !=
            cudaSuccess)
            return e;
        k_bt_cross<<<dim3(npf, nmat), BT_CX_NT, bt_cross_smem(), s>>>(a, Xq, Tt, Cs, ms, ss);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        nl += 1;
    }
    for (int b = 0; b < nblk; b++) {   // Y_b^T = V_b T_b in place over V_b's row layout
        const int rs = (b & ~1) * BT_NB;
        SplitGemmArgs y;
        base(y);   // 128-wide tiles span every column: a tile's rows are read before it writes them
        y.Ahi = y.Chi = Ys.hi + yoff(b); y.Alo = y.Clo = Ys.lo + yoff(b); y.lda = y.ldc = ldy; y.sA = y.sC = ss;
        y.Bhi = Tt.hi + (size_t)b * B2; y.Blo = Tt.lo + (size_t)b * B2; y.ldb = BT_NB; y.sB = ss;
        y.out_mode = 1;
        y.M = n - rs; y.N = y.K = nbb(b);
        ys.push_back(y);
    }
    if ((e = multi_gemm(ys, nmat, s, nl)) != cudaSuccess) return e;
    for (int q = 0; q < npf; q++) {    // Y_2^T -= Y_1^T C^T, in place (the right half of the pair's rows)
        SplitGemmArgs g;
        base(g);
        const long long o = bt_yoff2(q, n);
        g.Ahi = Ys.hi + o; g.Alo = Ys.lo + o; g.lda = ldy; g.sA = ss;
        g.Bhi = Cs.hi + (size_t)q * B2; g.Blo = Cs.lo + (size_t)q * B2; g.ldb = BT_NB; g.sB = ss;
        g.epilogue = 2;
        g.Dhi = g.Chi = Ys.hi + o + BT_NB; g.Dlo = g.Clo = Ys.lo + o + BT_NB; g.ldd = g.ldc = ldy; g.sD = g.sC = ss;
        g.out_mode = 1;
        g.M = n - 2 * q * BT_NB; g.N = nbb(2 * q + 1); g.K = nbb(2 * q);
        cr.push_back(g);
    }
    if ((e = multi_gemm(cr, nmat, s, nl)) != cudaSuccess) return e;
    for (int q = npair - 1; q >= 0; q--) {
        const int kq = 2 * q * BT_NB, m = n - kq, wq = nbb(2 * q) + (2 * q + 1 < nblk ? nbb(2 * q + 1) : 0);
        SplitGemmArgs g1;                                          // P = Z^T[:, kq:] V_q
        base(g1);
        g1.tile_n = 0;
        g1.Ahi = Qs.hi + kq; g1.Alo = Qs.lo + kq; g1.lda = ld; g1.sA = ss;
        g1.Bhi = Vs.hi + (size_t)kq * ld + kq; g1.Blo = Vs.lo + (size_t)kq * ld + kq; g1.ldb = ld; g1.sB = ss;
        g1.Chi = Ps.hi; g1.Clo = Ps.lo; g1.ldc = ldy; g1.sC = ss; g1.out_mode = 1;
        g1.M = n; g1.N = wq; g1.K = m;
        SplitGemmArgs g2;                                          // Z^T[:, kq:] -= P Y_q
        base(g2);
        g2.tile_n = 0;
        g2.Ahi = Ps.hi; g2.Alo = Ps.lo; g2.lda = ldy; g2.sA = ss;
        g2.Bhi = Ys.hi + bt_yoff2(q, n); g2.Blo = Ys.lo + bt_yoff2(q, n); g2.ldb = ldy; g2.sB = ss;
        g2.epilogue = 2;
        g2.Dhi = Qs.hi + kq; g2.Dlo = Qs.lo + kq; g2.ldd = ld; g2.sD = ss;
        if (q > 0) {
            g2.Chi = Qs.hi + kq; g2.Clo = Qs.lo + kq; g2.ldc = ld; g2.sC = ss; g2.out_mode = 1;
        } else {
            g2.Cf = a.A; g2.ldc = ld; g2.sC = ms; g2.out_mode = 2;
        }
        g2.M = n; g2.N = m; g2.K = wq;
        if ((e = cir_launch_split_gemm(g1, nmat, s, &nl)) != cudaSuccess) return e;
        if ((e = cir_launch_split_gemm(g2, nmat, s, &nl)) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// The mixed forms with ld a multiple of 8: every operand as a BF16 split pair and the
// products on the pre-split tensor-core GEMM (k_tc_split.cu).  Q is first split into Qs
// (in P's buffer); the prep writes V_b (into Q's buffer) and Y_b^T (into a.Z) as pairs; P_b
// goes to U; the updates of Qs stay split and the last one writes V in FP32 into a.A.
static cudaError_t backtransform_split(const EighArgs &a, float *Q, float *P, float *U, int nmat, int nblk,
                                       cudaStream_t s, int &nl, bool q_split) {
    const int n = a.n, ld = a.ld, nrefl = n - 2;
    const long long ms = a.mstride, ss = 2 * a.mstride;   // per-matrix stride of a pair (BF16 elements)
    auto pair = [&](float *buf) {
        __nv_bfloat16 *b = reinterpret_cast<__nv_bfloat16 *>(buf);
        return SplitMat{b, b + ms};
    };
    // q_split: Q arrives as a pair already (the top merge's product wrote it so) and P is free
    const SplitMat Qs = q_split ? pair(Q) : pair(P), Vs = q_split ? pair(P) : pair(Q), Ys = pair(a.Z), Ps = pair(U);
    cudaError_t e = cudaSuccess;
    if (!q_split) {
        k_bt_split_q<<<dim3((n + BT_SQ_ROWS - 1) / BT_SQ_ROWS, nmat), 256, 0, s>>>(Q, ms, n, ld, Qs, ss);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    const int bw = min(BT_NB, (nrefl + 7) & ~7);   // width of P and of the Y_b^T blocks (<= ld)
    BtSplit sp{Vs, Ys, ld, bw, ss, ss};
    if (!q_split) nl += 1;
    if (bt_tc_enabled() && bt_pair_enabled() && bw == BT_NB) {
        e = backtransform_paired(a, Qs, Vs, Ys, U, nmat, nblk, s, nl);
        if (e != cudaErrorNotSupported) return e;
    }
    if (bt_tc_enabled() && bw == BT_NB && (long long)nblk * 2 * BT_NB * BT_NB <= ms) {
        // the preparation on tensor cores: V_b in both layouts, G_b = V_b^T V_b, T, Y_b^T = V_b T.
        // G_b (FP32) and T^T (a pair) live in U, which the products P only need afterwards.
        float *Gb = U;                                              // [nblk][BT_NB][BT_NB] per matrix
        const SplitMat Tt{reinterpret_cast<__nv_bfloat16 *>(U + (size_t)nblk * BT_NB * BT_NB),
                          reinterpret_cast<__nv_bfloat16 *>(U + (size_t)nblk * BT_NB * BT_NB) + (size_t)nblk * BT_NB * BT_NB};
        const size_t csm = sizeof(float) * (size_t)BT_NB * BT_LDV;
        k_bt_clean<false><<<dim3(nblk, nmat), BT_NT, csm, s>>>(a, sp);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        std::vector<SplitGemmArgs> gs(nblk), ys(nblk);
        std::vector<int> batch(nblk, nmat);
        for (int b = 0; b < nblk; b++) {
            const int kb = b * BT_NB, nbb = min(BT_NB, nrefl - kb), m = n - kb;
            SplitGemmArgs &g = gs[b];                               // G_b = V_b^T V_b
            g = SplitGemmArgs{};
            g.Ahi = g.Bhi = Vs.hi + (size_t)kb * ld + kb; g.Alo = g.Blo = Vs.lo + (size_t)kb * ld + kb;
            g.lda = g.ldb = ld; g.sA = g.sB = ss;
            g.Cf = Gb + (size_t)b * BT_NB * BT_NB; g.ldc = BT_NB; g.sC = ms; g.out_mode = 2;
            g.M = g.N = nbb; g.K = m;
            g.err = a.err;
            g.test_stall = a.test_stall;
            g.tile_n = 128;
            SplitGemmArgs &y = ys[b];                               // Y_b^T = V_b T, over V_b's row layout
            y = SplitGemmArgs{};
            y.Ahi = Ys.hi + bt_yoff(b, n, bw); y.Alo = Ys.lo + bt_yoff(b, n, bw); y.lda = bw; y.sA = ss;
            y.Bhi = Tt.hi + (size_t)b * BT_NB * BT_NB; y.Blo = Tt.lo + (size_t)b * BT_NB * BT_NB; y.ldb = BT_NB; y.sB = ss;
            y.Chi = Ys.hi + bt_yoff(b, n, bw); y.Clo = Ys.lo + bt_yoff(b, n, bw); y.ldc = bw; y.sC = ss; y.out_mode = 1;
            y.M = m; y.N = nbb; y.K = nbb;
            y.err = a.err;
            y.test_stall = a.test_stall;
            y.tile_n = 128;   // one tile spans every column: a tile's rows are read before it writes them
        }
        for (int b0 = 0; b0 < nblk; b0 += CIR_SPLIT_MAXP) {
            const int np = min(CIR_SPLIT_MAXP, nblk - b0);
            if ((e = cir_launch_split_gemm_multi(gs.data() + b0, batch.data() + b0, np, s, &nl)) != cudaSuccess) return e;
        }
        const size_t tsm = bt_tmat_smem();
        if ((e = cudaFuncSetAttribute(k_bt_tmat, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tsm)) != cudaSuccess)
            return e;
        k_bt_tmat<<<dim3(nblk, nmat), BT_NB, tsm, s>>>(a, Gb, Tt, ms, ss);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        nl += 2;
        for (int b0 = 0; b0 < nblk; b0 += CIR_SPLIT_MAXP) {
            const int np = min(CIR_SPLIT_MAXP, nblk - b0);
            if ((e = cir_launch_split_gemm_multi(ys.data() + b0, batch.data() + b0, np, s, &nl)) != cudaSuccess) return e;
        }
    } else {
        const size_t smem = bt_prep_smem();
        if ((e = cudaFuncSetAttribute(k_bt_prep<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) !=
            cudaSuccess)
            return e;
        k_bt_prep<true><<<dim3(nblk, nmat), BT_NT, smem, s>>>(a, sp);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        nl += 1;
    }
    for (int b = nblk - 1; b >= 0; b--) {
        const int kb = b * BT_NB, nbb = min(BT_NB, nrefl - kb), m = n - kb;
        SplitGemmArgs g1{};                                        // P = Z^T[:, kb:] V_b
        g1.Ahi = Qs.hi + kb; g1.Alo = Qs.lo + kb; g1.lda = ld; g1.sA = ss;
        g1.Bhi = Vs.hi + (size_t)kb * ld + kb; g1.Blo = Vs.lo + (size_t)kb * ld + kb; g1.ldb = ld; g1.sB = ss;
        g1.Chi = Ps.hi; g1.Clo = Ps.lo; g1.ldc = bw; g1.sC = ss; g1.out_mode = 1;
        g1.M = n; g1.N = nbb; g1.K = m;
        g1.err = a.err;
        g1.test_stall = a.test_stall;
        SplitGemmArgs g2{};                                        // Z^T[:, kb:] -= P Y_b
        g2.Ahi = Ps.hi; g2.Alo = Ps.lo; g2.lda = bw; g2.sA = ss;
        g2.Bhi = Ys.hi + bt_yoff(b, n, bw); g2.Blo = Ys.lo + bt_yoff(b, n, bw); g2.ldb = bw; g2.sB = ss;
        g2.epilogue = 2;
        g2.Dhi = Qs.hi + kb; g2.Dlo = Qs.lo + kb; g2.ldd = ld; g2.sD = ss;
        if (b > 0) {
            g2.Chi = Qs.hi + kb; g2.Clo = Qs.lo + kb; g2.ldc = ld; g2.sC = ss; g2.out_mode = 1;
        } else {
            g2.Cf = a.A; g2.ldc = ld; g2.sC = ms; g2.out_mode = 2;
        }
        g2.M = n; g2.N = m; g2.K = nbb;
        g2.err = a.err;
        g2.test_stall = a.test_stall;
        if ((e = cir_launch_split_gemm(g1, nmat, s, &nl)) != cudaSuccess) return e;
        if ((e = cir_launch_split_gemm(g2, nmat, s, &nl)) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// V = Q_H Q into a.A.  Q (the tridiagonal eigenvectors, column-major, a.mstride per
// matrix) is overwritten; P and U are scratch of a.mstride floats per matrix; a.Z receives Y.
// a.A must hold the reflectors of the tridiagonalisation.
cudaError_t cir_launch_backtransform(const EighArgs &a, float *Q, float *P, float *U, int nmat, cudaStream_t s,
                                     int *launches, bool q_split) {
    const int n = a.n, ld = a.ld, nrefl = n - 2;
    if ((ld & 3) || (reinterpret_cast<uintptr_t>(a.A) & 15) || (reinterpret_cast<uintptr_t>(a.Z) & 15))
        return cudaErrorInvalidValue;
    if (nrefl <= 0)
        return cudaMemcpyAsync(a.A, Q, sizeof(float) * (size_t)nmat * a.mstride, cudaMemcpyDeviceToDevice, s);
    const int nblk = (nrefl + BT_NB - 1) / BT_NB;
    if (q_split && !(a.precision == CIR_PREC_BF16X3 && (ld & 7) == 0)) return cudaErrorInvalidValue;
    if (a.precision == CIR_PREC_BF16X3 && (ld & 7) == 0) {
        int nl = 0;
        const cudaError_t e = backtransform_split(a, Q, P, U, nmat, nblk, s, nl, q_split);
        if (launches) *launches += nl;
        return e;
    }
    const int pld = min(BT_NB, (nrefl + 3) & ~3);   // P: n x pld, pld <= ld
    const size_t smem = bt_prep_smem();
    cudaError_t e = cudaFuncSetAttribute(k_bt_prep<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_bt_prep<false><<<dim3(nblk, nmat), BT_NT, smem, s>>>(a, BtSplit{});
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    int nl = 1;
    for (int b = nblk - 1; b >= 0; b--) {
        const int kb = b * BT_NB, nbb = min(BT_NB, nrefl - kb), m = n - kb;
        GemmArgs g1{};
        g1.A = Q + kb;                               // Z^T[:, kb:]
        g1.lda = ld;
        g1.sA = a.mstride;
        g1.B = a.A + (size_t)kb * ld + kb;           // V_b, element (r, j) at column kb + j
        g1.ldb = ld;
        g1.sB = a.mstride;
        g1.b_kmajor = true;
        g1.C = P;
        g1.ldc = pld;
        g1.sC = a.mstride;
        g1.M = n;
        g1.N = nbb;
        g1.K = m;
        g1.err = a.err;
        GemmArgs g2{};
        g2.A = P;
        g2.lda = pld;
        g2.sA = a.mstride;
        g2.B = a.Z + (size_t)kb * ld + kb;           // Y_b
        g2.ldb = ld;
        g2.sB = a.mstride;
        g2.C = (b == 0 ? a.A : Q) + kb;
        g2.ldc = ld;
        g2.sC = a.mstride;
        g2.D = Q + kb;
        g2.ldd = ld;
        g2.sD = a.mstride;
        g2.M = n;
        g2.N = m;
        g2.K = nbb;
        g2.epilogue = 2;
        g2.err = a.err;
        for (const GemmArgs *g : {&g1, &g2}) {
            e = a.precision == CIR_PREC_FP32 ? cir_launch_gemm(*g, nmat, s, nullptr)
                                             : cir_launch_tc_gemm(*g, nmat, a.precision, s, nullptr);
            if (e != cudaSuccess) return e;
        }
        nl += 2;
    }
    if (launches) *launches += nl;
    return cudaSuccess;
}
