// Batched symmetric eigensolver for the exciton Hamiltonians (replaces magma_ssyevd_gpu,
// calcIR.cu:420-448).  One thread block solves one matrix; a launch solves a batch of
// frames, so the SMs work on independent frames at once.
//
//  1. Householder tridiagonalisation Q^T H Q = T (reflectors stored below the
//     subdiagonal, as LAPACK sytd2).  The rank-2 update of step k-1 and the
//     matrix-vector product of step k share one read/write pass over the trailing
//     block; each thread streams four consecutive rows with 16-byte accesses.
//  2. Q is formed explicitly in Z by backward accumulation of the reflectors, in blocks
//     of EIG_NB reflectors staged in shared memory; each warp keeps one column segment of
//     Z in registers while a block is applied.
//  3. Implicit symmetric QR on T with the Wilkinson shift (Golub & Van Loan, Alg. 8.3.2).
//     Lane 0 of warp 0 chases the bulges of a group of EIG_KS sweeps while the other
//     warps apply the previous group to the rows of Z.  A group is applied as a
//     wavefront: sweep s trails sweep s-1 by one column, so each row keeps a window of
//     EIG_KS+1 columns in registers and reads and writes every column once per group
//     instead of once per sweep.
//  4. Eigenvalues are ranked ascending; column j of Z is written to column rank(j) of A,
//     and, when enabled, the inverse participation ratios of every eigenvector are binned
//     into the frequency distributions (calcIR.cu:493-538).
//
// Every loop is bounded: the QR phase stops after 30*n sweeps and reports status 1.
// The leading dimension must be a multiple of 4 and A 16-byte aligned.
#include "cir_device.cuh"
#include <float.h>

namespace {

constexpr int EIG_NB = 8;      // reflectors per block in phase 2
constexpr int EIG_KS = 16;     // QR sweeps per wavefront group in phase 3
constexpr int EIG_W = EIG_KS + 1;

template <int NT>
__device__ __forceinline__ float block_sum(float v, float *red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    v = warp_sum(v);
    __syncthreads();               // red may still be read from the previous call
    if (lane == 0) red[warp] = v;
    __syncthreads();
    if (warp == 0) {
        float t = lane < NT / 32 ? red[lane] : 0.f;
        t = warp_sum(t);
        if (lane == 0) red[32] = t;
    }
    __syncthreads();
    return red[32];
}

__device__ __forceinline__ bool negligible(float e, float d0, float d1, float tiny) {
    return fabsf(e) <= 5.9604645e-8f * (fabsf(d0) + fabsf(d1)) || fabsf(e) <= tiny;
}

struct Chaser {
    int cm, nsweep, status, cap;
    float tiny;
};

// One implicit QR sweep with the Wilkinson shift on the trailing unreduced block of
// (d, e); its rotations go to rot[l..cm-1] (rotation i acts on columns i, i+1).
// Returns false when T is diagonal or the sweep cap is reached.
__device__ bool qr_sweep(Chaser &ch, float *d, float *e, float2 *rot, int *lo, int *hi) {
    int cm = ch.cm;
    while (cm > 0 && negligible(e[cm - 1], d[cm - 1], d[cm], ch.tiny)) { e[cm - 1] = 0.f; cm--; }
    ch.cm = cm;
    if (cm == 0) return false;
    if (ch.nsweep >= ch.cap) { ch.status = 1; return false; }
    int l = cm - 1;
    while (l > 0 && !negligible(e[l - 1], d[l - 1], d[l], ch.tiny)) l--;
    const float t = 0.5f * (d[cm - 1] - d[cm]);
    const float bb = e[cm - 1];
    const float den = t + copysignf(sqrtf(t * t + bb * bb), t);
    const float mu = d[cm] - (den != 0.f ? bb * bb / den : 0.f);
    float x = d[l] - mu, z = e[l];
    for (int k = l; k < cm; k++) {
        const float r = sqrtf(x * x + z * z);
        float c = 1.f, s = 0.f;
        if (r > 0.f) { c = x / r; s = z / r; }
        if (k > l) e[k - 1] = r;
        const float a0 = d[k], a1 = d[k + 1], be = e[k];
        const float g = s * (a0 - a1) - 2.f * c * be;
        d[k] = a0 - s * g;
        d[k + 1] = a1 + s * g;
        e[k] = c * s * (a1 - a0) + (c * c - s * s) * be;
        if (k + 1 < cm) {
            const float b2 = e[k + 1];
            z = s * b2;
            e[k + 1] = c * b2;
            x = e[k];
        }
        rot[k] = make_float2(c, s);
    }
    *lo = l;
    *hi = cm;
    ch.nsweep++;
    return true;
}

// Apply a group of `cnt` sweeps (rotations rot[s*n + i], i in [lo[s], hi[s])) to rows
// ra and rb of Z as a wavefront (see the file comment).
__device__ __forceinline__ void apply_group(float *Z, int ld, int ra, int rb, bool va, bool vb,
                                            const float2 *rot, int n, const int *lo, const int *hi, int cnt) {
    int T0 = 1 << 30, T1 = -1, cmin = 1 << 30, cmax = -1;
    for (int s = 0; s < cnt; s++) {
        T0 = min(T0, lo[s] + s);
        T1 = max(T1, hi[s] - 1 + s);
        cmin = min(cmin, lo[s]);
        cmax = max(cmax, hi[s]);
    }
    if (T1 < 0) return;
    int los[EIG_KS], his[EIG_KS];
    #pragma unroll
    for (int s = 0; s < EIG_KS; s++) {
        los[s] = s < cnt ? lo[s] : 0;
        his[s] = s < cnt ? hi[s] : 0;
    }
    float wa[EIG_W], wb[EIG_W];
    const int tb = (T0 / EIG_W) * EIG_W;
    #pragma unroll
    for (int v = 1; v <= EIG_KS; v++) {
        const int c = tb - EIG_KS + v;
        const bool ok = c >= cmin && c <= cmax;
        wa[(v + 1) % EIG_W] = (ok && va) ? Z[(size_t)c * ld + ra] : 0.f;
        wb[(v + 1) % EIG_W] = (ok && vb) ? Z[(size_t)c * ld + rb] : 0.f;
    }
    int tc = tb;
    for (; tc <= T1; tc += EIG_W) {
        #pragma unroll
        for (int u = 0; u < EIG_W; u++) {
            const int tau = tc + u;
            {
                const int c = tau + 1;
                if (c >= cmin && c <= cmax) {
                    if (va) wa[(u + 1) % EIG_W] = Z[(size_t)c * ld + ra];
                    if (vb) wb[(u + 1) % EIG_W] = Z[(size_t)c * ld + rb];
                }
            }
            #pragma unroll
            for (int s = 0; s < EIG_KS; s++) {
                const int i = tau - s;
                if (i >= los[s] && i < his[s]) {
                    const float2 cs = rot[s * n + i];
                    const int ia = (u - s + 2 * EIG_W) % EIG_W, ib = (u - s + 1 + 2 * EIG_W) % EIG_W;
                    const float a0 = wa[ia], a1 = wa[ib];
                    wa[ia] = cs.x * a0 + cs.y * a1;
                    wa[ib] = cs.x * a1 - cs.y * a0;
                    const float b0 = wb[ia], b1 = wb[ib];
                    wb[ia] = cs.x * b0 + cs.y * b1;
                    wb[ib] = cs.x * b1 - cs.y * b0;
                }
            }
            {
                const int c = tau - EIG_KS + 1;
                if (c >= cmin && c <= cmax) {
                    if (va) Z[(size_t)c * ld + ra] = wa[(u + 2) % EIG_W];
                    if (vb) Z[(size_t)c * ld + rb] = wb[(u + 2) % EIG_W];
                }
            }
        }
    }
    const int tl = tc - 1;   // last time step processed, congruent to EIG_KS mod EIG_W
    #pragma unroll
    for (int v = 1; v < EIG_W; v++) {
        const int c = tl - EIG_KS + 1 + v;
        if (c >= cmin && c <= cmax) {
            if (va) Z[(size_t)c * ld + ra] = wa[(v + 1) % EIG_W];
            if (vb) Z[(size_t)c * ld + rb] = wb[(v + 1) % EIG_W];
        }
    }
}

template <int NT, int NMAX>
__global__ void __launch_bounds__(NT) k_eigh(EighArgs a) {
    constexpr int RMAX = (NMAX + 31) / 32;            // rows per lane, phase 2
    constexpr int QG = (NMAX + 4 * NT - 1) / (4 * NT); // 4-row groups per thread, phase 1
    constexpr int NW = NT / 32;
    extern __shared__ __align__(16) float smem[];
    const int n = a.n, ld = a.ld;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    float *A = a.A + (size_t)blockIdx.x * a.mstride;
    float *Z = a.Z + (size_t)blockIdx.x * a.mstride;
    float2 *rotg = a.rot + (size_t)blockIdx.x * 2 * EIG_KS * n;

    const int n4 = (n + 3) & ~3;
    float *d = smem;             // [n4]
    float *e = d + n4;           // [n4]
    float *tau = e + n4;         // [n4]
    float *U = tau + n4;         // union region, EIG_NB*n4 floats (>= 4*n4)
    float *red = U + (size_t)EIG_NB * n4;   // [64]
    int *isc = reinterpret_cast<int *>(red + 64);   // [4*EIG_KS + 8]

    // ---------------- phase 1: tridiagonalisation ----------------
    {
        float *vp = U, *wp = U + n4, *vc = U + 2 * n4, *wc = U + 3 * n4;
        bool pending = false;
        for (int k = 0; k + 2 < n; k++) {
            // (a) column k below the diagonal with the pending rank-2 update applied
            float part = 0.f;
            for (int i = k + tid; i < n; i += NT) {
                float v = A[(size_t)k * ld + i];
                if (pending) v -= vp[i] * wp[k] + wp[i] * vp[k];
                if (i == k) d[k] = v;
                else if (i == k + 1) red[48] = v;   // alpha
                else { vc[i] = v; part += v * v; }
            }
            const float xn2 = block_sum<NT>(part, red);
            // (b) the reflector (slarfg convention: v[0] = 1, beta = -sign(alpha)*norm)
            if (tid == 0) {
                const float alpha = red[48];
                float t = 0.f, beta = alpha, scale = 0.f;
                if (xn2 > 0.f) {
                    beta = -copysignf(sqrtf(alpha * alpha + xn2), alpha);
                    t = (beta - alpha) / beta;
                    scale = 1.f / (alpha - beta);
                }
                tau[k] = t;
                e[k] = beta;
                red[49] = scale;
            }
            __syncthreads();
            const float scale = red[49];
            const float tk = tau[k];
            for (int i = k + 2 + tid; i < n; i += NT) {
                const float v = vc[i] * scale;
                vc[i] = v;
                A[(size_t)k * ld + i] = v;
            }
            if (tid == 0) vc[k + 1] = 1.f;
            __syncthreads();
            // (c) one pass over the trailing block: apply update k-1, accumulate p = A v_k.
            // Thread t owns the 4-row groups starting at r_al + 4*(t + q*NT).
            const int r0 = k + 1;
            const int r_al = r0 & ~3;
            float p[QG][4];
            float vr[QG][4], wr[QG][4];
            #pragma unroll
            for (int q = 0; q < QG; q++)
                #pragma unroll
                for (int j = 0; j < 4; j++) {
                    const int r = r_al + 4 * (tid + q * NT) + j;
                    const bool in = r >= r0 && r < n;
                    p[q][j] = 0.f;
                    vr[q][j] = (pending && in) ? vp[r] : 0.f;
                    wr[q][j] = (pending && in) ? wp[r] : 0.f;
                }
            int c = r0;
            for (; c + 3 < n; c += 4) {
                float4 col[4][QG];
                #pragma unroll
                for (int cc = 0; cc < 4; cc++)
                    #pragma unroll
                    for (int q = 0; q < QG; q++) {
                        const int rb = r_al + 4 * (tid + q * NT);
                        col[cc][q] = rb < n ? *reinterpret_cast<const float4 *>(A + (size_t)(c + cc) * ld + rb)
                                            : make_float4(0.f, 0.f, 0.f, 0.f);
                    }
                #pragma unroll
                for (int cc = 0; cc < 4; cc++) {
                    const float vpc = vp[c + cc], wpc = wp[c + cc], vcc = vc[c + cc];
                    #pragma unroll
                    for (int q = 0; q < QG; q++) {
                        const int rb = r_al + 4 * (tid + q * NT);
                        if (rb >= n) continue;
                        float x[4] = {col[cc][q].x, col[cc][q].y, col[cc][q].z, col[cc][q].w};
                        #pragma unroll
                        for (int j = 0; j < 4; j++) {
                            const float v = x[j] - (vr[q][j] * wpc + wr[q][j] * vpc);
                            x[j] = v;
                            p[q][j] += v * vcc;
                        }
                        if (pending)
                            *reinterpret_cast<float4 *>(A + (size_t)(c + cc) * ld + rb) = make_float4(x[0], x[1], x[2], x[3]);
                    }
                }
            }
            for (; c < n; c++) {
                const float vpc = vp[c], wpc = wp[c], vcc = vc[c];
                #pragma unroll
                for (int q = 0; q < QG; q++) {
                    const int rb = r_al + 4 * (tid + q * NT);
                    if (rb >= n) continue;
                    float4 v4 = *reinterpret_cast<const float4 *>(A + (size_t)c * ld + rb);
                    float x[4] = {v4.x, v4.y, v4.z, v4.w};
                    #pragma unroll
                    for (int j = 0; j < 4; j++) {
                        const float v = x[j] - (vr[q][j] * wpc + wr[q][j] * vpc);
                        x[j] = v;
                        p[q][j] += v * vcc;
                    }
                    if (pending) *reinterpret_cast<float4 *>(A + (size_t)c * ld + rb) = make_float4(x[0], x[1], x[2], x[3]);
                }
            }
            // rows below r0 saw vr = wr = 0 and contribute nothing
            float dpart = 0.f;
            #pragma unroll
            for (int q = 0; q < QG; q++)
                #pragma unroll
                for (int j = 0; j < 4; j++) {
                    const int r = r_al + 4 * (tid + q * NT) + j;
                    if (r >= r0 && r < n) {
                        p[q][j] *= tk;
                        dpart += p[q][j] * vc[r];
                    }
                }
            const float dot = block_sum<NT>(dpart, red);
            const float half = 0.5f * tk * dot;
            #pragma unroll
            for (int q = 0; q < QG; q++)
                #pragma unroll
                for (int j = 0; j < 4; j++) {
                    const int r = r_al + 4 * (tid + q * NT) + j;
                    if (r >= r0 && r < n) wc[r] = p[q][j] - half * vc[r];
                }
            __syncthreads();
            float *t0 = vp; vp = vc; vc = t0;
            float *t1 = wp; wp = wc; wc = t1;
            pending = true;
        }
        if (tid == 0) {
            if (n >= 2) {
                float a00 = A[(size_t)(n - 2) * ld + n - 2], a10 = A[(size_t)(n - 2) * ld + n - 1];
                float a11 = A[(size_t)(n - 1) * ld + n - 1];
                if (pending) {
                    a00 -= 2.f * vp[n - 2] * wp[n - 2];
                    a10 -= vp[n - 1] * wp[n - 2] + wp[n - 1] * vp[n - 2];
                    a11 -= 2.f * vp[n - 1] * wp[n - 1];
                }
                d[n - 2] = a00;
                d[n - 1] = a11;
                e[n - 2] = a10;
                tau[n - 2] = 0.f;
            } else {
                d[0] = A[0];
            }
            e[n - 1] = 0.f;
        }
        __syncthreads();
    }

    // ---------------- phase 2: Q = H_0 H_1 ... H_{n-3} into Z ----------------
    for (size_t idx = tid; idx < (size_t)n * ld; idx += NT) {
        const int j = (int)(idx / ld), i = (int)(idx % ld);
        Z[idx] = (i == j) ? 1.f : 0.f;
    }
    __syncthreads();
    {
        const int nrefl = n - 2;
        float *vb = U;   // [EIG_NB][n - r0]
        for (int kb = nrefl > 0 ? ((nrefl - 1) / EIG_NB) * EIG_NB : -1; kb >= 0; kb -= EIG_NB) {
            const int kend = min(kb + EIG_NB, nrefl);
            const int r0 = kb + 1;
            const int m = n - r0;
            const int nb = kend - kb;
            for (int idx = tid; idx < nb * m; idx += NT) {
                const int kk = idx / m, i = r0 + idx % m, k = kb + kk;
                vb[kk * m + (i - r0)] = i < k + 1 ? 0.f : (i == k + 1 ? 1.f : A[(size_t)k * ld + i]);
            }
            __syncthreads();
            for (int j = r0 + warp; j < n; j += NW) {
                float *col = Z + (size_t)j * ld + r0;
                float q[RMAX];
                #pragma unroll
                for (int t = 0; t < RMAX; t++) {
                    const int i = lane + 32 * t;
                    q[t] = i < m ? col[i] : 0.f;
                }
                for (int kk = nb - 1; kk >= 0; kk--) {
                    const float *v = vb + kk * m;
                    float s = 0.f;
                    #pragma unroll
                    for (int t = 0; t < RMAX; t++) {
                        const int i = lane + 32 * t;
                        if (i < m) s += v[i] * q[t];
                    }
                    s = warp_sum(s) * tau[kb + kk];
                    #pragma unroll
                    for (int t = 0; t < RMAX; t++) {
                        const int i = lane + 32 * t;
                        if (i < m) q[t] -= s * v[i];
                    }
                }
                #pragma unroll
                for (int t = 0; t < RMAX; t++) {
                    const int i = lane + 32 * t;
                    if (i < m) col[i] = q[t];
                }
            }
            __syncthreads();
        }
    }

    // ---------------- phase 3: implicit QR on (d, e), rotations applied to Z ----------------
    {
        int *g_lo = isc;                 // [2][EIG_KS]
        int *g_hi = isc + 2 * EIG_KS;    // [2][EIG_KS]
        int *g_cnt = isc + 4 * EIG_KS;   // [2]
        Chaser ch;
        ch.cm = n - 1;
        ch.nsweep = 0;
        ch.status = 0;
        ch.cap = 30 * n;
        ch.tiny = 0.f;
        if (tid == 0) {
            float tn = 0.f;
            for (int i = 0; i < n; i++) tn = fmaxf(tn, fabsf(d[i]) + 2.f * fabsf(e[i]));
            ch.tiny = 1e-12f * tn + FLT_MIN;
        }
        // produce a group of up to EIG_KS sweeps into buffer b
        auto produce = [&](int b) {
            int cnt = 0;
            while (cnt < EIG_KS &&
                   qr_sweep(ch, d, e, rotg + (size_t)(b * EIG_KS + cnt) * n, &g_lo[b * EIG_KS + cnt], &g_hi[b * EIG_KS + cnt]))
                cnt++;
            g_cnt[b] = cnt;
        };
        if (tid == 0) produce(0);
        __syncthreads();
        int b = 0;
        const int napp = NT - 32;
        while (g_cnt[b] > 0) {
            if (warp == 0) {
                if (lane == 0) produce(b ^ 1);
            } else {
                const int t = tid - 32;
                const float2 *rb = rotg + (size_t)b * EIG_KS * n;
                for (int r0 = 0; r0 < n; r0 += 2 * napp) {
                    const int ra = r0 + t, rb2 = r0 + napp + t;
                    if (ra >= n) break;
                    apply_group(Z, ld, ra, rb2 < n ? rb2 : ra, true, rb2 < n, rb, n, g_lo + b * EIG_KS,
                                g_hi + b * EIG_KS, g_cnt[b]);
                }
            }
            __syncthreads();
            b ^= 1;
        }
        if (tid == 0) {
            if (a.status) a.status[blockIdx.x] = ch.status;
            if (a.sweeps) atomicAdd(a.sweeps, (unsigned long long)ch.nsweep);
        }
        __syncthreads();
    }

    // ---------------- phase 4: ascending order, output, frequency distribution ----------------
    {
        int *rank = reinterpret_cast<int *>(U);
        for (int j = tid; j < n; j += NT) {
            const float dj = d[j];
            int r = 0;
            for (int i = 0; i < n; i++) {
                const float di = d[i];
                r += (di < dj) || (di == dj && i < j);
            }
            rank[j] = r;
            a.W[(size_t)blockIdx.x * a.wstride + r] = dj;
        }
        __syncthreads();
        for (int j = warp; j < n; j += NW) {
            const float *src = Z + (size_t)j * ld;
            float *dst = A + (size_t)rank[j] * ld;
            float s4 = 0.f, m4 = 0.f;
            for (int i0 = 0; i0 < n; i0 += 32) {
                const int i = i0 + lane;
                const float v = i < n ? src[i] : 0.f;
                if (i < n) dst[i] = v;
                const float v2 = v * v;
                s4 += v2 * v2;
                if (a.nchrom_mol == 2) {
                    const float pair = v2 + __shfl_xor_sync(0xffffffffu, v2, 1);
                    if ((lane & 1) == 0) m4 += pair * pair;
                } else {
                    m4 += v2 * v2;
                }
            }
            if (a.hist_count) {
                s4 = warp_sum(s4);
                m4 = warp_sum(m4);
                if (lane == 0) {
                    const float wi = d[j] + a.avef;
                    const int bin = (int)roundf((wi - a.omegaStart) / (float)a.omegaStep);
                    if (bin >= 0 && bin < a.nomega) {
                        atomicAdd(a.hist_count + bin, 1ull);
                        atomicAdd(a.hist_ipr + bin, (double)(1.f / s4));
                        atomicAdd(a.hist_mipr + bin, (double)(1.f / m4));
                    } else {
                        atomicAdd(a.out_of_range, 1ull);
                    }
                }
            }
        }
    }
}

template <int NT, int NMAX>
cudaError_t launch_one(const EighArgs &a, int nmat, cudaStream_t s, size_t smem) {
    auto kern = k_eigh<NT, NMAX>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<nmat, NT, smem, s>>>(a);
    return cudaGetLastError();
}

}  // namespace

size_t cir_eigh_smem_bytes(int n) {
    const size_t n4 = (size_t)((n + 3) & ~3);
    return sizeof(float) * (3 * n4 + EIG_NB * n4 + 64) + sizeof(int) * (4 * EIG_KS + 8);
}

size_t cir_eigh_rot_bytes(int n) { return sizeof(float2) * 2 * EIG_KS * (size_t)n; }

int cir_eigh_max_n() { return 2048; }

cudaError_t cir_launch_eigh(const EighArgs &a, int nmat, cudaStream_t s, int *launches) {
    if (a.n < 1 || a.n > cir_eigh_max_n() || nmat < 1 || (a.ld & 3) || a.ld < a.n) return cudaErrorInvalidValue;
    if ((reinterpret_cast<uintptr_t>(a.A) & 15) || (reinterpret_cast<uintptr_t>(a.Z) & 15) || !a.rot)
        return cudaErrorInvalidValue;
    const size_t smem = cir_eigh_smem_bytes(a.n);
    cudaError_t e;
    if (a.n <= 256) e = launch_one<128, 256>(a, nmat, s, smem);
    else if (a.n <= 512) e = launch_one<256, 512>(a, nmat, s, smem);
    else if (a.n <= 1024) e = launch_one<256, 1024>(a, nmat, s, smem);
    else e = launch_one<256, 2048>(a, nmat, s, smem);
    if (launches) *launches += 1;
    return e;
}
