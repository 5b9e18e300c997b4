// Correlation-function contraction and spectral density.
//
// k_tcf: psi_a = F m_a(0) for the 9 dipole/polarisability vectors (one warp per row of
// F), then the 15 unconjugated dot products with m_b(t) the reference evaluates as
// separate magma_cgemv + magma_cdotu pairs (calcIR.cu:628-745), combined directly into
//     IR = sum_a mu_a(t).F.mu_a(0)
//     VV = (3 iiFii + iiFjj + 4 ijFij) / 15,   VH = (2 iiFii - iiFjj + 6 ijFij) / 30.
// Row sums are accumulated in double and stay on the device.
//
// k_spec_mu2 / k_spec_sum: M = V^T mu (calcIR.cu:462-467) and the Lorentzian sum
// S(w_i) += sum_j |M_j|^2 g / ((w_i - l_j - avef)^2 + g^2) / pi, g = hbar/(2 T1)
// (get_spectral_density, calcIR.cu:1414-1444).
#include "cir_device.cuh"

namespace {

constexpr int TCF_WARPS = 8;
constexpr int TCF_ROWS = 64;   // rows of F per block

__global__ void __launch_bounds__(TCF_WARPS * 32) k_tcf(TcfArgs t) {
    extern __shared__ float m0s[];   // [9][n]
    __shared__ double part[TCF_WARPS][6];
    const int b = blockIdx.y;
    const float *F = t.F + (size_t)b * t.sF;
    const float *m0 = t.m0 + (size_t)b * t.sm0;
    const float *mt = t.mt + (size_t)b * t.smt;
    const int n = t.n;
    for (int i = threadIdx.x; i < 9 * n; i += blockDim.x) m0s[i] = m0[(size_t)(i / n) * t.ldv + i % n];
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double acc[6] = {0, 0, 0, 0, 0, 0};
    const int rend = min(n, (int)(blockIdx.x + 1) * TCF_ROWS);
    for (int r = blockIdx.x * TCF_ROWS + warp; r < rend; r += TCF_WARPS) {
        const float2 *row = reinterpret_cast<const float2 *>(F + (size_t)r * t.ldf);
        float pr[9], pi[9];
        #pragma unroll
        for (int a = 0; a < 9; a++) pr[a] = pi[a] = 0.f;
        for (int q = lane; q < n; q += 32) {
            const float2 f = row[q];
            #pragma unroll
            for (int a = 0; a < 9; a++) {
                const float m = m0s[a * n + q];
                pr[a] = fmaf(f.x, m, pr[a]);
                pi[a] = fmaf(f.y, m, pi[a]);
            }
        }
        #pragma unroll
        for (int a = 0; a < 9; a++) {
            pr[a] = warp_sum(pr[a]);
            pi[a] = warp_sum(pi[a]);
        }
        if (lane == 0) {
            float c[9];
            #pragma unroll
            for (int a = 0; a < 9; a++) c[a] = mt[(size_t)a * t.ldv + r];
            // IR: x, y, z
            float ir_r = c[0] * pr[0] + c[1] * pr[1] + c[2] * pr[2];
            float ir_i = c[0] * pi[0] + c[1] * pi[1] + c[2] * pi[2];
            // iiFii: xx->xx, yy->yy, zz->zz (psi index 3,4,5 = xx,yy,zz)
            float ii_r = c[3] * pr[3] + c[4] * pr[4] + c[5] * pr[5];
            float ii_i = c[3] * pi[3] + c[4] * pi[4] + c[5] * pi[5];
            // ijFij: xy->xy, yz->yz, zx->zx
            float ij_r = c[6] * pr[6] + c[7] * pr[7] + c[8] * pr[8];
            float ij_i = c[6] * pi[6] + c[7] * pi[7] + c[8] * pi[8];
            // iiFjj: xx->yy, xx->zz, yy->xx, yy->zz, zz->xx, zz->yy
            float jj_r = (c[4] + c[5]) * pr[3] + (c[3] + c[5]) * pr[4] + (c[3] + c[4]) * pr[5];
            float jj_i = (c[4] + c[5]) * pi[3] + (c[3] + c[5]) * pi[4] + (c[3] + c[4]) * pi[5];
            acc[0] += ir_r;
            acc[1] += ir_i;
            acc[2] += (3.0 * ii_r + jj_r + 4.0 * ij_r) / 15.0;
            acc[3] += (3.0 * ii_i + jj_i + 4.0 * ij_i) / 15.0;
            acc[4] += (2.0 * ii_r - jj_r + 6.0 * ij_r) / 30.0;
            acc[5] += (2.0 * ii_i - jj_i + 6.0 * ij_i) / 30.0;
        }
    }
    if (lane == 0)
        #pragma unroll
        for (int q = 0; q < 6; q++) part[warp][q] = acc[q];
    __syncthreads();
    if (threadIdx.x < 6) {
        double s = 0;
        for (int w = 0; w < TCF_WARPS; w++) s += part[w][threadIdx.x];
        atomicAdd(t.out + (size_t)b * t.sout + threadIdx.x, s);
    }
}

// The same contraction with F stored transposed as a split BF16 pair (the mixed form's
// pre-split propagation): F[r][q] = Ft[(2q)*ldft + r] + i Ft[(2q+1)*ldft + r], hi + lo.
// The correlation terms are linear in psi, so each block takes 64 rows and a quarter of the
// q range and contracts its partial psi with m(t) directly.  Thread (rr, ql) = (t & 63,
// t >> 6) handles row r = 64 blockIdx.x + rr and every fourth q of the block's range.
constexpr int TT_ROWS = 64, TT_QSPLIT = 4;

__device__ __forceinline__ void tcf_terms(const float (&pr)[9], const float (&pi)[9], const float (&c)[9],
                                          double (&acc)[6]) {
    const float ir_r = c[0] * pr[0] + c[1] * pr[1] + c[2] * pr[2];
    const float ir_i = c[0] * pi[0] + c[1] * pi[1] + c[2] * pi[2];
    const float ii_r = c[3] * pr[3] + c[4] * pr[4] + c[5] * pr[5];
    const float ii_i = c[3] * pi[3] + c[4] * pi[4] + c[5] * pi[5];
    const float ij_r = c[6] * pr[6] + c[7] * pr[7] + c[8] * pr[8];
    const float ij_i = c[6] * pi[6] + c[7] * pi[7] + c[8] * pi[8];
    const float jj_r = (c[4] + c[5]) * pr[3] + (c[3] + c[5]) * pr[4] + (c[3] + c[4]) * pr[5];
    const float jj_i = (c[4] + c[5]) * pi[3] + (c[3] + c[5]) * pi[4] + (c[3] + c[4]) * pi[5];
    acc[0] += ir_r;
    acc[1] += ir_i;
    acc[2] += (3.0 * ii_r + jj_r + 4.0 * ij_r) / 15.0;
    acc[3] += (3.0 * ii_i + jj_i + 4.0 * ij_i) / 15.0;
    acc[4] += (2.0 * ii_r - jj_r + 6.0 * ij_r) / 30.0;
    acc[5] += (2.0 * ii_i - jj_i + 6.0 * ij_i) / 30.0;
}

__global__ void __launch_bounds__(256) k_tcf_t(TcfArgs t) {
    extern __shared__ float mq[];    // [9][qchunk]
    __shared__ double part[8][6];
    const int b = blockIdx.z, n = t.n;
    const int qchunk = (n + TT_QSPLIT - 1) / TT_QSPLIT;
    const int qb = blockIdx.y * qchunk, qe = min(n, qb + qchunk);
    const float *m0 = t.m0 + (size_t)b * t.sm0;
    const float *mt = t.mt + (size_t)b * t.smt;
    for (int i = threadIdx.x; i < 9 * qchunk; i += blockDim.x) {
        const int a = i / qchunk, q = qb + i % qchunk;
        mq[i] = q < n ? m0[(size_t)a * t.ldv + q] : 0.f;
    }
    __syncthreads();
    const int rr = threadIdx.x & 63, ql = threadIdx.x >> 6;
    const int r = blockIdx.x * TT_ROWS + rr;
    double acc[6] = {0, 0, 0, 0, 0, 0};
    if (r < n) {
        const __nv_bfloat16 *fh = t.Ft.hi + (size_t)b * t.sFt + r, *fl = t.Ft.lo + (size_t)b * t.sFt + r;
        float pr[9], pi[9], c[9];
        #pragma unroll
        for (int a = 0; a < 9; a++) pr[a] = pi[a] = 0.f;
        for (int q = qb + ql; q < qe; q += TT_QSPLIT) {
            const size_t o = (size_t)(2 * q) * t.ldft;
            const float re = __bfloat162float(fh[o]) + __bfloat162float(fl[o]);
            const float im = __bfloat162float(fh[o + t.ldft]) + __bfloat162float(fl[o + t.ldft]);
            #pragma unroll
            for (int a = 0; a < 9; a++) {
                const float m = mq[a * qchunk + (q - qb)];
                pr[a] = fmaf(re, m, pr[a]);
                pi[a] = fmaf(im, m, pi[a]);
            }
        }
        #pragma unroll
        for (int a = 0; a < 9; a++) c[a] = mt[(size_t)a * t.ldv + r];
        tcf_terms(pr, pi, c, acc);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    #pragma unroll
    for (int q = 0; q < 6; q++) acc[q] = warp_sum_d(acc[q]);
    if (lane == 0)
        #pragma unroll
        for (int q = 0; q < 6; q++) part[warp][q] = acc[q];
    __syncthreads();
    if (threadIdx.x < 6) {
        double s = 0;
        for (int w = 0; w < 8; w++) s += part[w][threadIdx.x];
        atomicAdd(t.out + (size_t)b * t.sout + threadIdx.x, s);
    }
}

__global__ void k_spec_mu2(const float *V, int ld, const float *dip, int ldv, int n, float *mu2) {
    const int lane = threadIdx.x & 31;
    const int j = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
    if (j >= n) return;
    const float *col = V + (size_t)j * ld;
    float mx = 0, my = 0, mz = 0;
    for (int i = lane; i < n; i += 32) {
        const float v = col[i];
        mx = fmaf(v, dip[i], mx);
        my = fmaf(v, dip[ldv + i], my);
        mz = fmaf(v, dip[2 * ldv + i], mz);
    }
    mx = warp_sum(mx); my = warp_sum(my); mz = warp_sum(mz);
    if (lane == 0) mu2[j] = mx * mx + my * my + mz * mz;
}

__global__ void k_spec_sum(const float *mu2, const float *w, int n, double *Sw, int nomega, float omegaStart,
                           int omegaStep, float gamma, float avef) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nomega) return;
    const float wi = (float)(omegaStart + omegaStep * i);
    float s = 0.f;
    for (int j = 0; j < n; j++) {
        const float dw = wi - (w[j] + avef);
        s += mu2[j] * gamma / (dw * dw + gamma * gamma) / (float)CIR_PI;
    }
    Sw[i] += (double)s;
}

}  // namespace

cudaError_t cir_launch_tcf(const TcfArgs &t, int batch, cudaStream_t s, int *launches) {
    if (t.Ft.hi) {
        const size_t sm = sizeof(float) * 9 * (size_t)((t.n + TT_QSPLIT - 1) / TT_QSPLIT);
        cudaError_t e = cudaFuncSetAttribute(k_tcf_t, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        k_tcf_t<<<dim3((t.n + TT_ROWS - 1) / TT_ROWS, TT_QSPLIT, batch), 256, sm, s>>>(t);
        if (launches) *launches += 1;
        return cudaGetLastError();
    }
    const size_t smem = sizeof(float) * 9 * (size_t)t.n;
    cudaError_t e = cudaFuncSetAttribute(k_tcf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grid((t.n + TCF_ROWS - 1) / TCF_ROWS, batch);
    k_tcf<<<grid, TCF_WARPS * 32, smem, s>>>(t);
    if (launches) *launches += 1;
    return cudaGetLastError();
}

cudaError_t cir_launch_spectral(const float *V, int ld, const float *w, const float *dip, int ldv, int n,
                                float *mu2, double *Sw, int nomega, float omegaStart, int omegaStep, float t1,
                                float avef, cudaStream_t s, int *launches) {
    k_spec_mu2<<<(n + 7) / 8, 256, 0, s>>>(V, ld, dip, ldv, n, mu2);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const float gamma = (float)(CIR_HBAR / (t1 * 2.0));
    k_spec_sum<<<(nomega + 127) / 128, 128, 0, s>>>(mu2, w, n, Sw, nomega, omegaStart, omegaStep, gamma, avef);
    if (launches) *launches += 2;
    return cudaGetLastError();
}
