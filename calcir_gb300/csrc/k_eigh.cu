// Batched symmetric eigensolver for the exciton Hamiltonians (replaces magma_ssyevd_gpu,
// calcIR.cu:420-448).  Two kernels, each with one thread block per matrix, so the SMs
// work on independent frames at once: k_eigh_tq (phases 1-2, 256 threads) and k_eigh_qr
// (phases 3-4, 128 threads: one chasing warp and three applying warps, four blocks per SM
// so that four bulge chases overlap on every SM).
//
//  1. Householder tridiagonalisation Q^T H Q = T (reflectors stored below the
//     subdiagonal, as LAPACK sytd2).  The rank-2 update of step k-1 and the
//     matrix-vector product of step k share one read/write pass over the trailing
//     block; each thread streams four consecutive rows with 16-byte accesses.
//  2. Q is formed explicitly in Z by backward accumulation of the reflectors, in blocks
//     of EIG_NB reflectors staged in shared memory; each warp keeps one column segment of
//     Z in registers while a block is applied.
//  3. Implicit symmetric QR on T with the Wilkinson shift (Golub & Van Loan, Alg. 8.3.2).
//     Lane 0 of warp 0 chases the bulges of a group of EIG_KS sweeps (the bulge state is
//     carried in registers) while the other warps apply the previous group to the rows
//     of Z.  A group is applied as a
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
#include <cstring>
#include <mutex>

namespace {

__device__ __forceinline__ unsigned long long globaltimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

constexpr int EIG_NB = 8;      // reflectors per block in phase 2
constexpr int EIG_KS = 16;     // QR sweeps per wavefront group in phase 3
constexpr int EIG_W = EIG_KS + 1;
constexpr int QR_PREFETCH = 4;  // Z columns loaded ahead of the wavefront in phase 3

size_t tq_smem_bytes(int n) {
    const size_t n4 = (size_t)((n + 3) & ~3);
    return sizeof(float) * (3 * n4 + EIG_NB * n4 + 64);
}

size_t qr_smem_bytes(int n) {
    const size_t n4 = (size_t)((n + 3) & ~3);
    return sizeof(float) * 3 * n4 + sizeof(int) * (4 * EIG_KS + 8);
}

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
    long long nrot;
};

// One implicit QR sweep with the Wilkinson shift on the trailing unreduced block of
// (d, e); rotation i (acting on columns i, i+1) goes to rot[(i + s_slot) * EIG_KS].
// Returns false when T is diagonal or the sweep cap is reached.
// rot points at slot s of a time-major group buffer: rotation i of this sweep is stored at
// rot[(i + s) * EIG_KS], so the EIG_KS rotations applied at one wavefront step share one
// 128-byte line.
__device__ bool qr_sweep(Chaser &ch, float *d, float *e, float2 *rot, int s_slot, int *lo, int *hi) {
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
    // bulge state in registers: dk = current d[k], ek = current e[k]; dk1/ek1 are the
    // untouched d[k+1], e[k+1], loaded one iteration ahead
    float x = d[l] - mu, z = e[l];
    float dk = d[l], ek = e[l];
    float dk1 = d[l + 1], ek1 = (l + 1 < cm) ? e[l + 1] : 0.f;
    for (int k = l; k < cm; k++) {
        const float dk2 = (k + 2 <= cm) ? d[k + 2] : 0.f;
        const float ek2 = (k + 2 < cm) ? e[k + 2] : 0.f;
        const float r2 = x * x + z * z;
        float c = 1.f, s = 0.f, r = 0.f;
        if (r2 >= 1e-30f) {
            // reciprocal square root refined by one FMA-based Newton step (as accurate as a
            // correctly rounded rsqrt for the orthogonality of the rotations)
            const float i0 = rsqrtf(r2);
            const float res = fmaf(-(r2 * i0), i0, 1.0f);
            const float inv = fmaf(0.5f * i0, res, i0);
            c = x * inv;
            s = z * inv;
            r = r2 * inv;
        } else if (r2 > 0.f) {
            r = sqrtf(r2);
            c = x / r;
            s = z / r;
        }
        if (k > l) e[k - 1] = r;
        const float g = s * (dk - dk1) - 2.f * c * ek;
        d[k] = dk - s * g;
        const float dk1n = dk1 + s * g;
        const float ekn = c * s * (dk1 - dk) + (c * c - s * s) * ek;
        e[k] = ekn;
        float ek_next = 0.f;
        if (k + 1 < cm) {
            z = s * ek1;
            ek_next = c * ek1;
            x = ekn;
        }
        rot[(size_t)(k + s_slot) * EIG_KS] = make_float2(c, s);
        dk = dk1n;
        ek = ek_next;
        dk1 = dk2;
        ek1 = ek2;
    }
    d[cm] = dk;
    *lo = l;
    *hi = cm;
    ch.nsweep++;
    ch.nrot += cm - l;
    return true;
}

// Apply a group of `cnt` sweeps to R rows of Z as a wavefront.  Rotation i of sweep s
// lives at rot[(i + s) * EIG_KS + s]; every other slot of the group buffer holds the
// identity rotation (c = 1, s = 0), so the EIG_KS rotations of step tau are one 128-byte
// line rot[tau * EIG_KS ..] and are applied without predicates.  At step tau, sweep s
// applies its rotation i = tau - s.  Each row keeps the columns tau-EIG_KS+1 .. tau+1 in
// registers w[0..EIG_KS] (slot j holds column tau-EIG_KS+1+j); rotation (s, tau-s) acts
// on slots EIG_KS-1-s and EIG_KS-s and the window shifts by one slot per step, so every
// column is read and written once per group.  Slots EIG_KS+1 .. EIG_KS+P hold columns
// loaded P steps ahead.  row[j] < 0 marks an unused row slot.
template <int R, int P>
__device__ __forceinline__ void apply_group(float *Z, int ld, const int (&row)[R], const float2 *rot,
                                            int T0, int T1, int cmin, int cmax) {
    constexpr int S = EIG_W + P;   // window slots
    float w[R][S];
    // columns T0-EIG_KS+1 .. T0+P into slots 0 .. EIG_KS-1+P
    #pragma unroll
    for (int v = 0; v < EIG_KS + P; v++) {
        const int c = T0 - EIG_KS + 1 + v;
        const bool ok = c >= cmin && c <= cmax;
        #pragma unroll
        for (int j = 0; j < R; j++) w[j][v] = (ok && row[j] >= 0) ? __ldcg(Z + (size_t)c * ld + row[j]) : 0.f;
    }
    float4 nxt[EIG_KS / 2];
    #pragma unroll
    for (int q = 0; q < EIG_KS / 2; q++) nxt[q] = reinterpret_cast<const float4 *>(rot + (size_t)T0 * EIG_KS)[q];
    for (int tau = T0; tau <= T1; tau++) {
        float4 cur[EIG_KS / 2];
        #pragma unroll
        for (int q = 0; q < EIG_KS / 2; q++) cur[q] = nxt[q];
        if (tau < T1) {
            #pragma unroll
            for (int q = 0; q < EIG_KS / 2; q++) nxt[q] = reinterpret_cast<const float4 *>(rot + (size_t)(tau + 1) * EIG_KS)[q];
        }
        {   // column tau+1+P into the last slot
            const int c = tau + 1 + P;
            const bool ok = c >= cmin && c <= cmax;
            #pragma unroll
            for (int j = 0; j < R; j++) w[j][S - 1] = (ok && row[j] >= 0) ? __ldcg(Z + (size_t)c * ld + row[j]) : 0.f;
        }
        #pragma unroll
        for (int s = 0; s < EIG_KS; s++) {
            const float cc = (s & 1) ? cur[s / 2].z : cur[s / 2].x;
            const float ss = (s & 1) ? cur[s / 2].w : cur[s / 2].y;
            #pragma unroll
            for (int j = 0; j < R; j++) {
                const float a0 = w[j][EIG_KS - 1 - s], a1 = w[j][EIG_KS - s];
                w[j][EIG_KS - 1 - s] = cc * a0 + ss * a1;
                w[j][EIG_KS - s] = cc * a1 - ss * a0;
            }
        }
        {
            const int c = tau - EIG_KS + 1;
            if (c >= cmin && c <= cmax) {
                #pragma unroll
                for (int j = 0; j < R; j++)
                    if (row[j] >= 0) __stcg(Z + (size_t)c * ld + row[j], w[j][0]);
            }
        }
        #pragma unroll
        for (int j = 0; j < R; j++)
            #pragma unroll
            for (int v = 0; v < S - 1; v++) w[j][v] = w[j][v + 1];
    }
    // after the last step the window holds columns T1-EIG_KS+2 .. T1+1 in slots 0..EIG_KS-1
    #pragma unroll
    for (int v = 0; v < EIG_KS; v++) {
        const int c = T1 - EIG_KS + 2 + v;
        if (c >= cmin && c <= cmax) {
            #pragma unroll
            for (int j = 0; j < R; j++)
                if (row[j] >= 0) __stcg(Z + (size_t)c * ld + row[j], w[j][v]);
        }
    }
}

template <int NT, int NMAX, int MINB>
__global__ void __launch_bounds__(NT, MINB) k_eigh_tq(EighArgs a) {
    constexpr int RMAX = (NMAX + 31) / 32;            // rows per lane, phase 2
    constexpr int QG = (NMAX + 4 * NT - 1) / (4 * NT); // 4-row groups per thread, phase 1
    constexpr int NW = NT / 32;
    extern __shared__ __align__(16) float smem[];
    const int n = a.n, ld = a.ld;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    float *A = a.A + (size_t)blockIdx.x * a.mstride;
    float *Z = a.Z + (size_t)blockIdx.x * a.mstride;

    const int n4 = (n + 3) & ~3;
    float *d = smem;             // [n4]
    float *e = d + n4;           // [n4]
    float *tau = e + n4;         // [n4]
    float *U = tau + n4;         // union region, EIG_NB*n4 floats (>= 4*n4)
    float *red = U + (size_t)EIG_NB * n4;   // [64]

    unsigned long long *pt = a.phase_ns ? a.phase_ns + (size_t)blockIdx.x * 8 : nullptr;
    if (pt && tid == 0) pt[0] = globaltimer_ns();
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

    if (pt && tid == 0) pt[1] = globaltimer_ns();
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

    // d and e for the QR kernel
    for (int i = tid; i < n; i += NT) {
        a.DE[(size_t)blockIdx.x * 2 * ld + i] = d[i];
        a.DE[(size_t)blockIdx.x * 2 * ld + ld + i] = e[i];
    }
    if (pt && tid == 0) pt[2] = globaltimer_ns();
}

template <int NT, int R>
__global__ void __launch_bounds__(NT, 3) k_eigh_qr(EighArgs a) {
    constexpr int NW = NT / 32;
    extern __shared__ __align__(16) float smem[];
    const int n = a.n, ld = a.ld;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    float *A = a.A + (size_t)blockIdx.x * a.mstride;
    float *Z = a.Z + (size_t)blockIdx.x * a.mstride;
    float2 *rotg = a.rot + (size_t)blockIdx.x * 2 * (n + EIG_KS) * EIG_KS;
    const int n4 = (n + 3) & ~3;
    float *d = smem;                                 // [n4]
    float *e = d + n4;                               // [n4]
    float *U = e + n4;                               // [n4] ranks
    int *isc = reinterpret_cast<int *>(U + n4);      // [4*EIG_KS + 8]
    unsigned long long *pt = a.phase_ns ? a.phase_ns + (size_t)blockIdx.x * 8 : nullptr;
    for (int i = tid; i < n; i += NT) {
        d[i] = a.DE[(size_t)blockIdx.x * 2 * ld + i];
        e[i] = a.DE[(size_t)blockIdx.x * 2 * ld + ld + i];
    }
    for (int q = tid; q < 2 * (n + EIG_KS) * EIG_KS; q += NT) rotg[q] = make_float2(1.f, 0.f);
    __syncthreads();
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
        ch.nrot = 0;
        unsigned long long t_chase = 0, t_apply = 0;
        if (tid == 0) {
            float tn = 0.f;
            for (int i = 0; i < n; i++) tn = fmaxf(tn, fabsf(d[i]) + 2.f * fabsf(e[i]));
            ch.tiny = 1e-12f * tn + FLT_MIN;
        }
        // produce a group of up to EIG_KS sweeps into buffer b
        auto produce = [&](int b) {
            int cnt = 0;
            while (cnt < EIG_KS &&
                   qr_sweep(ch, d, e, rotg + (size_t)b * (n + EIG_KS) * EIG_KS + cnt, cnt, &g_lo[b * EIG_KS + cnt],
                            &g_hi[b * EIG_KS + cnt]))
                cnt++;
            g_cnt[b] = cnt;
        };
        if (tid == 0) produce(0);
        __syncthreads();
        int b = 0;
        const int napp = NT - 32;
        while (g_cnt[b] > 0) {
            const unsigned long long tg = pt ? globaltimer_ns() : 0ull;
            if (warp == 0) {
                if (lane == 0) {
                    produce(b ^ 1);
                    if (pt) t_chase += globaltimer_ns() - tg;
                }
            } else {
                const int t = tid - 32;
                float2 *rb = rotg + (size_t)b * (n + EIG_KS) * EIG_KS;
                int T0 = 1 << 30, T1 = -1, cmin = 1 << 30, cmax = -1;
                for (int s = 0; s < g_cnt[b]; s++) {
                    T0 = min(T0, g_lo[b * EIG_KS + s] + s);
                    T1 = max(T1, g_hi[b * EIG_KS + s] - 1 + s);
                    cmin = min(cmin, g_lo[b * EIG_KS + s]);
                    cmax = max(cmax, g_hi[b * EIG_KS + s]);
                }
                for (int r0 = 0; r0 < n; r0 += R * napp) {
                    if (r0 + t >= n) break;
                    int row[R];
                    #pragma unroll
                    for (int j = 0; j < R; j++) row[j] = (r0 + j * napp + t < n) ? r0 + j * napp + t : -1;
                    apply_group<R, QR_PREFETCH>(Z, ld, row, rb, T0, T1, cmin, cmax);
                }
                // back to identity for the group after next (the __syncthreads below orders
                // this before the chase writes into the buffer again)
                asm volatile("bar.sync 1, %0;" ::"r"(NT - 32));
                for (int q = T0 * EIG_KS + t; q <= T1 * EIG_KS + EIG_KS - 1; q += napp) rb[q] = make_float2(1.f, 0.f);
                if (pt && tid == 32) t_apply += globaltimer_ns() - tg;
            }
            __syncthreads();
            b ^= 1;
        }
        if (pt && tid == 0) { pt[5] = t_chase; pt[7] = (unsigned long long)ch.nrot; }
        if (pt && tid == 32) pt[6] = t_apply;
        if (tid == 0) {
            if (a.status) a.status[blockIdx.x] = ch.status;
            if (a.sweeps) atomicAdd(a.sweeps, (unsigned long long)ch.nsweep);
        }
        __syncthreads();
    }

    if (pt && tid == 0) pt[3] = globaltimer_ns();
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
    if (pt) {
        __syncthreads();
        if (tid == 0) pt[4] = globaltimer_ns();
    }
}

// MINB: resident blocks per SM the register budget is fitted to (3 while the spill stays
// negligible; the order-2048 variant is fitted to 2 blocks).
template <int NT, int NMAX, int MINB>
cudaError_t launch_tq(const EighArgs &a, int nmat, cudaStream_t s) {
    auto kern = k_eigh_tq<NT, NMAX, MINB>;
    const size_t smem = tq_smem_bytes(a.n);
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<nmat, NT, smem, s>>>(a);
    return cudaGetLastError();
}

constexpr int QR_THREADS = 128;
constexpr int QR_ROWS = 3;   // rows per applying thread; 3 blocks per SM without spills

cudaError_t launch_qr(const EighArgs &a, int nmat, cudaStream_t s) {
    auto kern = k_eigh_qr<QR_THREADS, QR_ROWS>;
    const size_t smem = qr_smem_bytes(a.n);
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<nmat, QR_THREADS, smem, s>>>(a);
    return cudaGetLastError();
}

}  // namespace

size_t cir_eigh_rot_bytes(int n) { return sizeof(float2) * 2 * EIG_KS * (size_t)(n + EIG_KS); }

size_t cir_eigh_de_bytes(int ld) { return sizeof(float) * 2 * (size_t)ld; }

int cir_eigh_max_n() { return 2048; }

cudaError_t cir_launch_eigh(const EighArgs &a, int nmat, cudaStream_t s, int *launches) {
    if (a.n < 1 || a.n > cir_eigh_max_n() || nmat < 1 || (a.ld & 3) || a.ld < a.n) return cudaErrorInvalidValue;
    if ((reinterpret_cast<uintptr_t>(a.A) & 15) || (reinterpret_cast<uintptr_t>(a.Z) & 15) || !a.rot || !a.DE)
        return cudaErrorInvalidValue;
    cudaError_t e;
    if (a.n <= 256) e = launch_tq<128, 256, 4>(a, nmat, s);
    else if (a.n <= 512) e = launch_tq<256, 512, 3>(a, nmat, s);
    else if (a.n <= 1024) e = launch_tq<256, 1024, 3>(a, nmat, s);
    else e = launch_tq<256, 2048, 2>(a, nmat, s);
    if (e != cudaSuccess) return e;
    e = launch_qr(a, nmat, s);
    if (launches) *launches += 2;
    return e;
}

// ---------------------------------------------------------------------------------------
// Allocation-free entry point.  Some callers cannot allocate device memory: a simulation
// engine that calls this per frame from inside its own time step owns the GPU memory
// budget, and cudaMalloc/cudaFree synchronise the whole device and may fail in the middle
// of a run.  cir_eigh_noalloc takes the caller's device buffers for A and w and keeps all
// of its scratch (the eigenvector workspace, the QR rotation groups, the tridiagonal and
// the per-matrix status) in one statically sized device array that the library holds
// for as long as it is loaded.
// ---------------------------------------------------------------------------------------
namespace {

constexpr size_t NOALLOC_SCRATCH_BYTES = size_t(8) << 20;   // 8 MiB on every device that loads the library
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

constexpr int NOALLOC_MAX_DEVICES = 64;
std::mutex g_noalloc_mu;
void *g_noalloc_ptr[NOALLOC_MAX_DEVICES];   // device address of g_noalloc_scratch, per device

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace

extern "C" int cir_eigh_noalloc(int nmat, int n, float *A, float *w, void *cuda_stream) {
    if (nmat < 1 || n < 1 || n > cir_eigh_max_n() || !A || !w)
        return cir_fail(CIR_ERR_ARG, "cir_eigh_noalloc: need nmat >= 1, 1 <= n <= %d and device buffers A, w",
                        cir_eigh_max_n());
    cudaPointerAttributes pa, pw;
    if (cudaPointerGetAttributes(&pa, A) != cudaSuccess || cudaPointerGetAttributes(&pw, w) != cudaSuccess) {
        cudaGetLastError();
        return cir_fail(CIR_ERR_ARG, "cir_eigh_noalloc: A and w must be device pointers");
    }
    if (pa.type != cudaMemoryTypeDevice || pw.type != cudaMemoryTypeDevice)
        return cir_fail(CIR_ERR_ARG, "cir_eigh_noalloc: A and w must be device pointers");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cir_fail(CIR_ERR_CUDA, "cir_eigh_noalloc: cudaGetDevice: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) return cir_fail(CIR_ERR_ARG, "cir_eigh_noalloc: device %d unsupported", dev);
    unsigned char *scratch = nullptr;
    {
        // one-time set-up per device, with that device current: the array's device address
        std::lock_guard<std::mutex> lock(g_noalloc_mu);
        if (!g_noalloc_ptr[dev]) {
            void *p = nullptr;
            e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess)
                return cir_fail(CIR_ERR_CUDA, "cir_eigh_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
            g_noalloc_ptr[dev] = p;
        }
        scratch = static_cast<unsigned char *>(g_noalloc_ptr[dev]);
    }
    const int ld = (n + 3) & ~3;
    const bool pad = (ld != n) || (reinterpret_cast<uintptr_t>(A) & 15);
    const size_t mat = (size_t)n * ld * sizeof(float);
    const size_t need = align256(nmat * mat)                                   // Z
                        + align256(nmat * cir_eigh_rot_bytes(n))               // rotation groups
                        + align256(nmat * cir_eigh_de_bytes(ld))               // d, e
                        + align256((size_t)nmat * sizeof(int))                 // status
                        + (pad ? align256(nmat * mat) : 0);                    // 16-byte aligned copy of A
    if (need > NOALLOC_SCRATCH_BYTES)
        return cir_fail(CIR_ERR_ARG,
                        "cir_eigh_noalloc: %d matrices of order %d need %zu bytes of scratch; the allocation-free "
                        "scratch holds %zu bytes (call it with fewer matrices at a time)",
                        nmat, n, need, NOALLOC_SCRATCH_BYTES);
    cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
    unsigned char *q = scratch;
    EighArgs a;
    memset(&a, 0, sizeof a);
    a.Z = reinterpret_cast<float *>(q); q += align256(nmat * mat);
    a.rot = reinterpret_cast<float2 *>(q); q += align256(nmat * cir_eigh_rot_bytes(n));
    a.DE = reinterpret_cast<float *>(q); q += align256(nmat * cir_eigh_de_bytes(ld));
    a.status = reinterpret_cast<int *>(q); q += align256((size_t)nmat * sizeof(int));
    a.A = pad ? reinterpret_cast<float *>(q) : A;
    a.W = w;
    a.mstride = (long long)n * ld;
    a.wstride = n;
    a.n = n;
    a.ld = ld;
    a.nchrom_mol = 2;
    if (pad) {
        e = cudaMemcpy2DAsync(a.A, (size_t)ld * 4, A, (size_t)n * 4, (size_t)n * 4, (size_t)nmat * n,
                              cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess) return cir_fail(CIR_ERR_CUDA, "cir_eigh_noalloc: %s", cudaGetErrorString(e));
    }
    e = cir_launch_eigh(a, nmat, s, nullptr);
    if (e != cudaSuccess) return cir_fail(CIR_ERR_CUDA, "cir_eigh_noalloc: launch: %s", cudaGetErrorString(e));
    if (pad) {
        e = cudaMemcpy2DAsync(A, (size_t)n * 4, a.A, (size_t)ld * 4, (size_t)n * 4, (size_t)nmat * n,
                              cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess) return cir_fail(CIR_ERR_CUDA, "cir_eigh_noalloc: %s", cudaGetErrorString(e));
    }
    // the per-matrix convergence flags, read back through a small stack buffer
    int st[256];
    for (int m0 = 0; m0 < nmat; m0 += 256) {
        const int cnt = nmat - m0 < 256 ? nmat - m0 : 256;
        e = cudaMemcpyAsync(st, a.status + m0, (size_t)cnt * sizeof(int), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return cir_fail(CIR_ERR_CUDA, "cir_eigh_noalloc: %s", cudaGetErrorString(e));
        for (int i = 0; i < cnt; i++)
            if (st[i]) return cir_fail(CIR_ERR_NOCONVERGE, "cir_eigh_noalloc: sweep cap reached on matrix %d", m0 + i);
    }
    return CIR_OK;
}
