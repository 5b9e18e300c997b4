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

__global__ void __launch_bounds__(BT_NT, 2) k_bt_prep(EighArgs a) {
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

    // G = V_b^T V_b: thread (tx, ty) accumulates G[ty + 16 p][tx + 16 q]
    {
        const int tx = t & 15, ty = t >> 4;
        float acc[8][8];
        #pragma unroll
        for (int p = 0; p < 8; p++)
            #pragma unroll
            for (int q = 0; q < 8; q++) acc[p][q] = 0.f;
        for (int r0 = kb; r0 < n; r0 += BT_RC) {
            __syncthreads();
            bt_stage(A, ld, n, kb, nbb, r0, true, Vt);
            __syncthreads();
            #pragma unroll 1
            for (int rr = 0; rr < BT_RC; rr += 4) {
                float4 va[8];
                #pragma unroll
                for (int p = 0; p < 8; p++) va[p] = *reinterpret_cast<const float4 *>(Vt + (ty + 16 * p) * BT_LDV + rr);
                #pragma unroll
                for (int q = 0; q < 8; q++) {
                    const float4 vb = *reinterpret_cast<const float4 *>(Vt + (tx + 16 * q) * BT_LDV + rr);
                    #pragma unroll
                    for (int p = 0; p < 8; p++)
                        acc[p][q] = fmaf(va[p].x, vb.x, fmaf(va[p].y, vb.y, fmaf(va[p].z, vb.z, fmaf(va[p].w, vb.w, acc[p][q]))));
                }
            }
        }
        #pragma unroll
        for (int p = 0; p < 8; p++)
            #pragma unroll
            for (int q = 0; q < 8; q++) M[(ty + 16 * p) * BT_LDM + tx + 16 * q] = acc[p][q];
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

}  // namespace

// V = Q_H Q into a.A.  Q (the tridiagonal eigenvectors, column-major, a.mstride per
// matrix) is overwritten; P is scratch of a.mstride floats per matrix; a.Z receives Y.
// a.A must hold the reflectors of the tridiagonalisation.
cudaError_t cir_launch_backtransform(const EighArgs &a, float *Q, float *P, int nmat, cudaStream_t s, int *launches) {
    const int n = a.n, ld = a.ld, nrefl = n - 2;
    if ((ld & 3) || (reinterpret_cast<uintptr_t>(a.A) & 15) || (reinterpret_cast<uintptr_t>(a.Z) & 15))
        return cudaErrorInvalidValue;
    if (nrefl <= 0)
        return cudaMemcpyAsync(a.A, Q, sizeof(float) * (size_t)nmat * a.mstride, cudaMemcpyDeviceToDevice, s);
    const int nblk = (nrefl + BT_NB - 1) / BT_NB;
    const int pld = min(BT_NB, (nrefl + 3) & ~3);   // P: n x pld, pld <= ld
    const size_t smem = bt_prep_smem();
    cudaError_t e = cudaFuncSetAttribute(k_bt_prep, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_bt_prep<<<dim3(nblk, nmat), BT_NT, smem, s>>>(a);
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
