// Kernels of the differentiation form: the gradient of a spectrum-mismatch loss with respect
// to the 13 map and coupling coefficients (calcIR.cu:1207-1242) by the adjoint of the
// propagation and of the eigendecomposition.
//
// Only F m_c(0) enters the correlation functions (calcIR.cu:628-745), so the forward state
// is psi_c(k) = F(k) m_c(0) for the nine vectors c (dipole x, y, z; polarisability xx .. zx),
// stored per origin as an n x 18 row-major array of (re, im) pairs and propagated with the
// same GEMM pair as F (U_k = V_k exp(i L_k dt/hbar) V_k^T).  The adjoint lambda_c obeys
// lambda_c(k) = w_c(k) + U_{k+1} lambda_c(k+1) (U is complex symmetric), w_c(k) being the
// coefficient vector of psi_c(k) in dL.  The gradient with respect to H_k is
// G_k = V_k R_k V_k^T, R_k = Re(Phi o sum_c (V_k^T lambda_c(k)) (V_k^T psi_c(k-1))^T), where
// Phi_mn = i tau exp(i tau (l_m + l_n)/2) sinc(tau (l_m - l_n)/2) is the divided difference of
// exp(i tau l) (Daleckii-Krein), exact and finite for equal eigenvalues.  k_dtheta contracts
// G_k and dL/dm(k) with the derivatives of the maps.
#include "cir_device.cuh"

#include <algorithm>

namespace {

constexpr int PSI_LD = CIR_PSI_LD;   // 9 complex columns

__device__ __forceinline__ double dblock_sum(double v, double *red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    double r = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) r += red[w];
    return r;
}

// psi(0) = m(0): grid (ceil(n/256), S)
__global__ void k_psi_init(const float *M, long long sM, int ld, int n, float *psi) {
    const int s = blockIdx.y, i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float *m = M + (size_t)s * sM;
    float *p = psi + ((size_t)s * n + i) * PSI_LD;
    #pragma unroll
    for (int c = 0; c < 9; c++) {
        p[2 * c] = m[(size_t)c * ld + i];
        p[2 * c + 1] = 0.f;
    }
}

// IR, VV, VH of one step for every origin from psi(k) and m(k) (the terms of
// calcIR.cu:628-745 with psi_a = F m_a(0)): out[s*sout + 0..5] = (re, im) of each.
__global__ void __launch_bounds__(256) k_tcf_psi(const float *psi, const float *M, long long sM, int ld, int n,
                                                 double *out, long long sout) {
    __shared__ double red[8];
    const int s = blockIdx.x;
    const float *m = M + (size_t)s * sM;
    const float *p = psi + (size_t)s * n * PSI_LD;
    double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};   // ir, ii, jj, ij (re, im)
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        float mv[9], pr[9], pi[9];
        #pragma unroll
        for (int c = 0; c < 9; c++) {
            mv[c] = m[(size_t)c * ld + i];
            pr[c] = p[(size_t)i * PSI_LD + 2 * c];
            pi[c] = p[(size_t)i * PSI_LD + 2 * c + 1];
        }
        // term(a, b) = m_b . psi_a
        acc[0] += (double)(mv[0] * pr[0] + mv[1] * pr[1] + mv[2] * pr[2]);
        acc[1] += (double)(mv[0] * pi[0] + mv[1] * pi[1] + mv[2] * pi[2]);
        acc[2] += (double)(mv[3] * pr[3] + mv[4] * pr[4] + mv[5] * pr[5]);
        acc[3] += (double)(mv[3] * pi[3] + mv[4] * pi[4] + mv[5] * pi[5]);
        acc[4] += (double)(mv[4] * pr[3] + mv[5] * pr[3] + mv[3] * pr[4] + mv[5] * pr[4] + mv[3] * pr[5] + mv[4] * pr[5]);
        acc[5] += (double)(mv[4] * pi[3] + mv[5] * pi[3] + mv[3] * pi[4] + mv[5] * pi[4] + mv[3] * pi[5] + mv[4] * pi[5]);
        acc[6] += (double)(mv[6] * pr[6] + mv[7] * pr[7] + mv[8] * pr[8]);
        acc[7] += (double)(mv[6] * pi[6] + mv[7] * pi[7] + mv[8] * pi[8]);
    }
    double v[8];
    for (int q = 0; q < 8; q++) v[q] = dblock_sum(acc[q], red);
    if (threadIdx.x == 0) {
        double *o = out + (size_t)s * sout;
        o[0] = v[0];
        o[1] = v[1];
        o[2] = (3 * v[2] + v[4] + 4 * v[6]) / 15.0;
        o[3] = (3 * v[3] + v[5] + 4 * v[7]) / 15.0;
        o[4] = (2 * v[2] - v[4] + 6 * v[6]) / 30.0;
        o[5] = (2 * v[3] - v[5] + 6 * v[7]) / 30.0;
    }
}

// lambda += w(k): w_c = conj(g_ir) m_c (c < 3), conj(g_vv) (2 m_c + m3 + m4 + m5)/15
// (c = 3..5), conj(g_vv) 4 m_c/15 (c = 6..8).  With zero set, lambda = w(k).
__global__ void k_lambda_src(float *lam, const float *M, long long sM, int ld, int n, float gir_r, float gir_i,
                             float gvv_r, float gvv_i, int zero) {
    const int s = blockIdx.y, i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float *m = M + (size_t)s * sM;
    float *l = lam + ((size_t)s * n + i) * PSI_LD;
    float mv[9];
    #pragma unroll
    for (int c = 0; c < 9; c++) mv[c] = m[(size_t)c * ld + i];
    const float s3 = mv[3] + mv[4] + mv[5];
    #pragma unroll
    for (int c = 0; c < 9; c++) {
        float v, gr, gi;
        if (c < 3) { v = mv[c]; gr = gir_r; gi = gir_i; }
        else if (c < 6) { v = (2.f * mv[c] + s3) / 15.f; gr = gvv_r; gi = gvv_i; }
        else { v = 4.f * mv[c] / 15.f; gr = gvv_r; gi = gvv_i; }
        l[2 * c] = (zero ? 0.f : l[2 * c]) + gr * v;          // conj(g) v
        l[2 * c + 1] = (zero ? 0.f : l[2 * c + 1]) - gi * v;
    }
}

// R[s][m][n'] = Re(Phi_mn' sum_c a[s][m][c] b[s][n'][c]), a = V^T lambda, b = V^T psi(k-1)
// (n x 18 each), Phi from the eigenvalues l of the step's frame (W + s*sW).  32 x 32 tiles,
// grid (tiles, tiles, S); R row-major with leading dimension ldr.
__global__ void __launch_bounds__(256) k_build_R(const float *a, const float *b, const float *W, long long sW,
                                                 int n, float tau, float *R, int ldr, long long sR) {
    __shared__ float as[32][PSI_LD + 1], bs[32][PSI_LD + 1];
    __shared__ float la[32], lb[32];
    const int s = blockIdx.z;
    const int m0 = blockIdx.y * 32, n0 = blockIdx.x * 32;
    const float *A = a + (size_t)s * n * PSI_LD, *B = b + (size_t)s * n * PSI_LD, *w = W + (size_t)s * sW;
    for (int q = threadIdx.x; q < 32 * PSI_LD; q += blockDim.x) {
        const int r = q / PSI_LD, c = q % PSI_LD;
        as[r][c] = m0 + r < n ? A[(size_t)(m0 + r) * PSI_LD + c] : 0.f;
        bs[r][c] = n0 + r < n ? B[(size_t)(n0 + r) * PSI_LD + c] : 0.f;
    }
    if (threadIdx.x < 32) {
        la[threadIdx.x] = m0 + (int)threadIdx.x < n ? w[m0 + threadIdx.x] : 0.f;
        lb[threadIdx.x] = n0 + (int)threadIdx.x < n ? w[n0 + threadIdx.x] : 0.f;
    }
    __syncthreads();
    float *Rs = R + (size_t)s * sR;
    for (int q = threadIdx.x; q < 32 * 32; q += blockDim.x) {
        const int r = q >> 5, c = q & 31;
        if (m0 + r >= n || n0 + c >= n) continue;
        float sr = 0.f, si = 0.f;
        #pragma unroll
        for (int k = 0; k < 9; k++) {
            const float ar = as[r][2 * k], ai = as[r][2 * k + 1], br = bs[c][2 * k], bi = bs[c][2 * k + 1];
            sr += ar * br - ai * bi;
            si += ar * bi + ai * br;
        }
        const float x = 0.5f * tau * (la[r] - lb[c]);
        const float sinc = fabsf(x) < 1e-3f ? 1.f - x * x * (1.f / 6.f) : sinf(x) / x;
        float sp, cp;
        sincosf(0.5f * tau * (la[r] + lb[c]), &sp, &cp);
        // Phi = i tau (cp + i sp) sinc = tau sinc (-sp + i cp); Re(Phi S) = tau sinc (-sp sr - cp si)
        Rs[(size_t)(m0 + r) * ldr + n0 + c] = tau * sinc * (-sp * sr - cp * si);
    }
}

// the geometric factor of the transition dipole coupling between chromophores i and j of a
// frame's table (calcIR.cu:1352-1399 without the x and mu' factors)
__device__ __forceinline__ float tdc_kappa(const float *ct, int ld, int i, int j, float bx, float by, float bz) {
    float dx = cir_mi(ct[CT_TX * ld + i] - ct[CT_TX * ld + j], bx);
    float dy = cir_mi(ct[CT_TY * ld + i] - ct[CT_TY * ld + j], by);
    float dz = cir_mi(ct[CT_TZ * ld + i] - ct[CT_TZ * ld + j], bz);
    float r = sqrtf(dx * dx + dy * dy + dz * dz);
    dx /= r; dy /= r; dz /= r;
    r *= CIR_BOHR_NM;
    const float uix = ct[CT_UX * ld + i], uiy = ct[CT_UY * ld + i], uiz = ct[CT_UZ * ld + i];
    const float ujx = ct[CT_UX * ld + j], ujy = ct[CT_UY * ld + j], ujz = ct[CT_UZ * ld + j];
    const float uu = uix * ujx + uiy * ujy + uiz * ujz;
    const float un = uix * dx + uiy * dy + uiz * dz;
    const float vn = ujx * dx + ujy * dy + ujz * dz;
    return (uu - 3.0f * un * vn) / (r * r * r) * CIR_CM_HARTREE;
}

// Contraction of one step's gradients with the map derivatives, for every origin (blockIdx.y).
// Thread i (chromophore i of its frame) gathers
//   cw = G_ii (on d omega), a_i = sum_j inter (G_ij + G_ji) kappa_ij q_j (q = mu' x),
//   the intramolecular sums, and dL/dm_b,i (the correlation terms at this step, plus
//   Re lambda_c(0) at step 0, where psi(0) = m(0)),
// folds them into coefficients on d omega, d x, d p and d mu', and adds the 13 products with
// the derivatives of those four maps (plus the direct intramolecular ones) to out[13].
__global__ void __launch_bounds__(128) k_dtheta(DthetaArgs d) {
    __shared__ double red[8];
    const int s = blockIdx.y, i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = d.n, ld = d.ld;
    const float *ct = d.ct + (size_t)s * d.sct;
    const float *bx3 = d.box + (size_t)s * d.sbox;
    const float bx = bx3[0], by = bx3[1], bz = bx3[2];
    const CirMaps &mp = d.maps;
    double th[13];
    #pragma unroll
    for (int q = 0; q < 13; q++) th[q] = 0.0;
    if (i < n) {
        const float E = ct[CT_E * ld + i], w = ct[CT_W * ld + i], x = ct[CT_X * ld + i], p = ct[CT_P * ld + i];
        const float mup = ct[CT_MUP * ld + i];
        const float ux = ct[CT_UX * ld + i], uy = ct[CT_UY * ld + i], uz = ct[CT_UZ * ld + i];
        const int mol = i / d.nchrom_mol;
        float cw = 0.f, a = 0.f, ax = 0.f, bp = 0.f, d10 = 0.f, d11 = 0.f, d12 = 0.f;
        if (d.G) {
            const float *G = d.G + (size_t)s * d.sG;
            cw = G[(size_t)i * d.ldg + i];
            if (d.ispecies != 1 && d.ispecies != 2) {
                for (int j = 0; j < n; j++) {
                    if (j == i) continue;
                    const float gs = G[(size_t)i * d.ldg + j] + G[(size_t)j * d.ldg + i];
                    const float xj = ct[CT_X * ld + j];
                    if (j / d.nchrom_mol == mol) {          // intramolecular map (calcIR.cu:1339)
                        const float Ej = ct[CT_E * ld + j], pj = ct[CT_P * ld + j];
                        const float gij = G[(size_t)i * d.ldg + j];
                        ax += gs * (mp.wi[0] + mp.wi[1] * (E + Ej)) * xj;
                        bp += gs * mp.wi[2] * pj;
                        d10 += gij * x * xj;
                        d11 += gij * (E + Ej) * x * xj;
                        d12 += gij * p * pj;
                    } else {                                 // transition dipole coupling
                        a += gs * tdc_kappa(ct, ld, i, j, bx, by, bz) * ct[CT_MUP * ld + j] * xj;
                    }
                }
            }
        }
        // dL/dm_b,i: the correlation terms of this step, plus Re lambda(0) at step 0
        const float *ps = d.psi + ((size_t)s * n + i) * PSI_LD;
        float gm[9];
        {
            float pr[9], pi[9];
            #pragma unroll
            for (int c = 0; c < 9; c++) { pr[c] = ps[2 * c]; pi[c] = ps[2 * c + 1]; }
            // Re(conj(g) v) = gr vr + gi vi
            #pragma unroll
            for (int c = 0; c < 3; c++) gm[c] = d.gir_r * pr[c] + d.gir_i * pi[c];
            const float sr = pr[3] + pr[4] + pr[5], si = pi[3] + pi[4] + pi[5];
            #pragma unroll
            for (int c = 3; c < 6; c++)
                gm[c] = (d.gvv_r * (2.f * pr[c] + sr) + d.gvv_i * (2.f * pi[c] + si)) / 15.f;
            #pragma unroll
            for (int c = 6; c < 9; c++) gm[c] = 4.f * (d.gvv_r * pr[c] + d.gvv_i * pi[c]) / 15.f;
            if (d.lam0) {
                const float *l0 = d.lam0 + ((size_t)s * n + i) * PSI_LD;
                #pragma unroll
                for (int c = 0; c < 9; c++) gm[c] += l0[2 * c];
            }
        }
        const float sq = gm[0] * ux + gm[1] * uy + gm[2] * uz;
        const float sx = gm[3] * (4.6f * ux * ux + 1.f) + gm[4] * (4.6f * uy * uy + 1.f) + gm[5] * (4.6f * uz * uz + 1.f) +
                         gm[6] * 4.6f * ux * uy + gm[7] * 4.6f * uy * uz + gm[8] * 4.6f * uz * ux;
        // coefficients on d omega, d x, d p, d mu' (q = mu' x: dq = dmu' x + mu' dx)
        const double cx = (double)ax + sx + (double)mup * (a + sq);
        const double cp = bp, cm = (double)x * (a + sq);
        const double e1 = E, e2 = (double)E * E;
        const double base = cw + cx * mp.x[1] + cp * mp.p[1];   // d omega feeds omega, x and p
        th[0] = base; th[1] = base * e1; th[2] = base * e2;
        th[3] = cx; th[4] = cx * w;
        th[5] = cp; th[6] = cp * w;
        th[7] = cm; th[8] = cm * e1; th[9] = cm * e2;
        th[10] = d10; th[11] = d11; th[12] = d12;
    }
    #pragma unroll
    for (int q = 0; q < 13; q++) {
        const double v = dblock_sum(th[q], red);
        if (threadIdx.x == 0) atomicAdd(d.out + q, v);
    }
}

// One propagation step of every origin's nine vectors, psi <- V e^{i L dt/hbar} V^T psi (the
// F propagation of calcIR.cu:596-617 applied to psi = F m(0)), as two streaming passes over
// the step's eigenvectors (row j of V = eigenvector j, stride ld, a multiple of 4):
//   k_psi_rows: X[j][.] = e^{i w_j dt/hbar} sum_k V[j][k] psi[k][.]   (a warp per 4 rows j,
//               16-byte loads along k against psi transposed in shared memory)
//   k_psi_cols: psi[i][.] = sum_j V[j][i] X[j][.]   (32 columns i per block; its 8 warps take
//               every 8th row j and add their partial sums in shared memory)
// psi and X are n x 18 floats per origin (nine complex vectors, (re, im) pairs).
constexpr int PSI_NT = 512;                  // threads of k_psi_rows (16 warps)
constexpr int PSI_RW = 4;                    // rows per warp of k_psi_rows
constexpr int PSI_ROWS = 16 * PSI_RW;        // rows of V per block of k_psi_rows
constexpr int PSI_COLS = 32;                 // columns of V per block of k_psi_cols

__host__ __device__ inline int psi_tld(int n) { return ((n + 3) & ~3) + 4; }   // row stride of psi^T

__global__ void __launch_bounds__(PSI_NT) k_psi_rows(const float *V, int ld, long long sV, int n, const float *w,
                                                     long long sw, float dtoh, const float *psi, float *X) {
    extern __shared__ __align__(16) float pt[];       // psi^T: pt[q * tld + k], zero for k >= n
    const int b = blockIdx.y, warp = threadIdx.x >> 5, lane = threadIdx.x & 31, tld = psi_tld(n);
    const float *P = psi + (size_t)b * n * PSI_LD;
    for (int t = threadIdx.x; t < n * PSI_LD; t += blockDim.x) {
        const int k = t / PSI_LD, q = t - k * PSI_LD;
        pt[q * tld + k] = P[t];
    }
    for (int t = threadIdx.x; t < PSI_LD * (tld - n); t += blockDim.x) {
        const int q = t / (tld - n), k = n + t - q * (tld - n);
        pt[q * tld + k] = 0.f;
    }
    __syncthreads();
    const int j0 = blockIdx.x * PSI_ROWS + warp * PSI_RW;
    if (j0 >= n) return;
    const float *Vb = V + (size_t)b * sV;
    float acc[PSI_RW][PSI_LD];
    #pragma unroll
    for (int r = 0; r < PSI_RW; r++)
        #pragma unroll
        for (int q = 0; q < PSI_LD; q++) acc[r][q] = 0.f;
    const int n4 = (n + 3) >> 2;
    for (int k4 = lane; k4 < n4; k4 += 32) {
        const int k = 4 * k4;
        float4 z[PSI_RW];
        #pragma unroll
        for (int r = 0; r < PSI_RW; r++) {
            z[r] = j0 + r < n ? *reinterpret_cast<const float4 *>(Vb + (size_t)(j0 + r) * ld + k)
                              : make_float4(0.f, 0.f, 0.f, 0.f);
            // the row's padding past n is not part of V: clear it (0 * a non-finite pad is NaN)
            if (k + 1 >= n) z[r].y = 0.f;
            if (k + 2 >= n) z[r].z = 0.f;
            if (k + 3 >= n) z[r].w = 0.f;
        }
        #pragma unroll
        for (int q = 0; q < PSI_LD; q++) {
            const float4 p = *reinterpret_cast<const float4 *>(pt + q * tld + k);
            #pragma unroll
            for (int r = 0; r < PSI_RW; r++)
                acc[r][q] = fmaf(z[r].x, p.x, fmaf(z[r].y, p.y, fmaf(z[r].z, p.z, fmaf(z[r].w, p.w, acc[r][q]))));
        }
    }
    #pragma unroll
    for (int r = 0; r < PSI_RW; r++)
        #pragma unroll
        for (int q = 0; q < PSI_LD; q++) acc[r][q] = warp_sum(acc[r][q]);
    if (lane == 0) {
        #pragma unroll
        for (int r = 0; r < PSI_RW; r++) {
            const int j = j0 + r;
            if (j >= n) break;
            float sn, cs;
            sincosf(w[(size_t)b * sw + j] * dtoh, &sn, &cs);
            float *x = X + ((size_t)b * n + j) * PSI_LD;
            #pragma unroll
            for (int q = 0; q < PSI_LD; q += 2) {   // (re, im) times exp(+i phase)
                x[q] = cs * acc[r][q] - sn * acc[r][q + 1];
                x[q + 1] = sn * acc[r][q] + cs * acc[r][q + 1];
            }
        }
    }
}

__global__ void __launch_bounds__(256) k_psi_cols(const float *V, int ld, long long sV, int n, const float *X,
                                                  float *psi) {
    extern __shared__ __align__(16) float xs[];       // X[j * 18 + q] (three blocks per SM at n = 1024),
                                                      // then partial sums
    const int b = blockIdx.y, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const float *Xb = X + (size_t)b * n * PSI_LD;
    for (int t = threadIdx.x; t < n * PSI_LD; t += blockDim.x) xs[t] = Xb[t];
    __syncthreads();
    const int i = blockIdx.x * PSI_COLS + lane;
    float acc[PSI_LD];
    #pragma unroll
    for (int q = 0; q < PSI_LD; q++) acc[q] = 0.f;
    if (i < n) {
        const float *Vb = V + (size_t)b * sV + i;
        #pragma unroll 4
        for (int j = warp; j < n; j += 8) {
            const float z = Vb[(size_t)j * ld];
            const float2 *x2 = reinterpret_cast<const float2 *>(xs + j * PSI_LD);   // 8-byte aligned rows
            #pragma unroll
            for (int u = 0; u < PSI_LD / 2; u++) {
                const float2 x = x2[u];
                acc[2 * u] = fmaf(z, x.x, acc[2 * u]);
                acc[2 * u + 1] = fmaf(z, x.y, acc[2 * u + 1]);
            }
        }
    }
    __syncthreads();                                  // xs is reused for the partial sums
    float *part = xs + (warp * PSI_COLS + lane) * (PSI_LD + 1);
    #pragma unroll
    for (int q = 0; q < PSI_LD; q++) part[q] = acc[q];
    __syncthreads();
    for (int t = threadIdx.x; t < PSI_COLS * PSI_LD; t += blockDim.x) {
        const int c = t / PSI_LD, q = t - c * PSI_LD, ic = blockIdx.x * PSI_COLS + c;
        if (ic >= n) continue;
        float sum = 0.f;
        for (int wv = 0; wv < 8; wv++) sum += xs[(wv * PSI_COLS + c) * (PSI_LD + 1) + q];
        psi[((size_t)b * n + ic) * PSI_LD + q] = sum;
    }
}

}  // namespace

cudaError_t cir_psi_step(const float *V, int ld, long long sV, int n, const float *w, long long sw, float dt_over_hbar,
                         float *psi, float *tmp, int S, cudaStream_t s) {
    if (n < 1 || S < 1 || S > 65535 || ld < n || (ld & 3) || (sV & 3) || (reinterpret_cast<uintptr_t>(V) & 15))
        return cudaErrorInvalidValue;
    const size_t smem_r = sizeof(float) * PSI_LD * (size_t)psi_tld(n);
    const size_t smem_c = sizeof(float) * std::max((size_t)PSI_LD * n, (size_t)8 * PSI_COLS * (PSI_LD + 1));
    cudaError_t e = cudaFuncSetAttribute(k_psi_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_r);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_psi_cols, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_c);
    if (e != cudaSuccess) return e;
    k_psi_rows<<<dim3((n + PSI_ROWS - 1) / PSI_ROWS, S), PSI_NT, smem_r, s>>>(V, ld, sV, n, w, sw, dt_over_hbar, psi,
                                                                             tmp);
    k_psi_cols<<<dim3((n + PSI_COLS - 1) / PSI_COLS, S), 256, smem_c, s>>>(V, ld, sV, n, tmp, psi);
    return cudaGetLastError();
}

cudaError_t cir_adj_psi_init(const float *M, long long sM, int ld, int n, int S, float *psi, cudaStream_t s) {
    k_psi_init<<<dim3((n + 255) / 256, S), 256, 0, s>>>(M, sM, ld, n, psi);
    return cudaGetLastError();
}

cudaError_t cir_adj_tcf(const float *psi, const float *M, long long sM, int ld, int n, int S, double *out, long long sout,
                        cudaStream_t s) {
    k_tcf_psi<<<S, 256, 0, s>>>(psi, M, sM, ld, n, out, sout);
    return cudaGetLastError();
}

cudaError_t cir_adj_lambda_src(float *lam, const float *M, long long sM, int ld, int n, int S, float gir_r, float gir_i,
                               float gvv_r, float gvv_i, int zero, cudaStream_t s) {
    k_lambda_src<<<dim3((n + 255) / 256, S), 256, 0, s>>>(lam, M, sM, ld, n, gir_r, gir_i, gvv_r, gvv_i, zero);
    return cudaGetLastError();
}

cudaError_t cir_adj_build_R(const float *a, const float *b, const float *W, long long sW, int n, int S, float tau, float *R,
                            int ldr, long long sR, cudaStream_t s) {
    const int t = (n + 31) / 32;
    k_build_R<<<dim3(t, t, S), 256, 0, s>>>(a, b, W, sW, n, tau, R, ldr, sR);
    return cudaGetLastError();
}

cudaError_t cir_adj_dtheta(const DthetaArgs &d, int S, cudaStream_t s) {
    k_dtheta<<<dim3((d.n + 127) / 128, S), 128, 0, s>>>(d);
    return cudaGetLastError();
}
