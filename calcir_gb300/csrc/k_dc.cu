// Divide-and-conquer eigensolver for the symmetric tridiagonal T = Q^T H Q left by the
// tridiagonalisation (the method magma_ssyevd uses, calcIR.cu:420-448: LAPACK stedc /
// laed0-laed4 in FP32), batched over matrices and run level by level:
//
//   * The index range [0, n) is halved recursively to a uniform depth D (block b of level
//     l is [b n >> l, (b+1) n >> l)), leaves of at most DC_LEAF rows.  At every internal
//     boundary m the coupling beta = e[m-1] is torn out (Cuppen): d[m-1] and d[m] lose |beta|
//     and the merge that joins the two sides adds back rho u u^T, rho = |beta|,
//     u = e_{m-1} + sign(beta) e_m.
//   * k_dc_leaf: one warp per leaf solves its block by implicit QR (Wilkinson shift), every
//     lane applying the rotations to its row of the leaf's eigenvector block, and writes the
//     eigenvalues ascending with their vectors.
//   * k_dc_merge (one block per merge): z = (last row of Q1, sign(beta) first row of Q2)/sqrt2,
//     rho = 2|beta|; the two sorted eigenvalue lists are merged; small components of z and
//     close pairs are deflated (close pairs by a Givens rotation, LAPACK laed2 rules with
//     tol = 8 eps max(|D|, |z|)); the secular equation 1/rho + sum z_j^2/(D_j - lambda) = 0
//     is solved for each root by a safeguarded rational (Gragg "middle way") iteration on
//     tau = lambda - D_origin, origin the nearer pole, so D_j - lambda is formed as
//     (D_j - D_origin) - tau without cancellation; z is recomputed from the roots
//     (Gu-Eisenstat), which keeps the vectors orthogonal; the block's K x K rotation
//     U = P G W (merge permutation, deflation rotations, secular vectors) is written
//     row-major, and the eigenvalues ascending.
//   * k_dc_gemm: Q_new = diag(Q1, Q2) U for every merge, as two products of the diagonal
//     blocks with the matching rows of U (64 x 64 tiles, FP32).
// The eigenvectors of H are then V = Q_H Q_T, the reflectors of the tridiagonalisation
// applied to Q_T in compact WY blocks (k_backtransform.cu): FP32 GEMMs in the plain form,
// the tensor-core GEMM (a.precision) in the mixed forms.
#include "cir_device.cuh"

#include <cstdlib>
#include <float.h>

namespace {

constexpr int DC_LEAF = 32;
constexpr int DC_NT = 256;          // threads of a merge block of 129-512 rows (fewer below, twice above)
constexpr float DC_EPS = 5.9604645e-8f;   // 2^-24

__host__ __device__ inline int dc_off(int level, int b, int n) { return (int)(((long long)b * n) >> level); }

// ---------------------------------------------------------------------------------------
// Leaves: warp w of the block handles leaf blockIdx.x * 4 + w of matrix blockIdx.y.
// ---------------------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_dc_leaf(EighArgs a, int depth, float *Qout) {
    __shared__ float Zs[4][DC_LEAF][DC_LEAF + 1];
    __shared__ float dS[4][DC_LEAF + 1], eS[4][DC_LEAF + 1];
    __shared__ int rk[4][DC_LEAF];
    const int n = a.n, ld = a.ld;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int leaf = blockIdx.x * 4 + warp;
    if (leaf >= (1 << depth)) return;
    const int m = blockIdx.y;
    float *dw = a.DE + (size_t)m * 3 * ld;          // d in, eigenvalues out
    const float *ev = dw + ld;                      // e
    float *Q = Qout + (size_t)m * a.mstride;
    const int a0 = dc_off(depth, leaf, n), a1 = dc_off(depth, leaf + 1, n);
    const int s = a1 - a0;
    float *d = dS[warp], *e = eS[warp];
    float(*Z)[DC_LEAF + 1] = Zs[warp];
    if (lane < s) {
        float v = dw[a0 + lane];
        if (lane == 0 && a0 > 0) v -= fabsf(ev[a0 - 1]);
        if (lane == s - 1 && a1 < n) v -= fabsf(ev[a1 - 1]);
        d[lane] = v;
        e[lane] = lane < s - 1 ? ev[a0 + lane] : 0.f;
    }
    for (int c = 0; c < s; c++)
        if (lane < s) Z[lane][c] = lane == c ? 1.f : 0.f;
    __syncwarp();
    // implicit QR with the Wilkinson shift; every lane runs the same scalar recurrence
    float tn = 0.f;
    for (int i = 0; i < s; i++) tn = fmaxf(tn, fabsf(d[i]) + 2.f * fabsf(e[i]));
    const float tiny = 1e-12f * tn + FLT_MIN;
    int cm = s - 1, nsweep = 0;
    const int cap = a.test_sweep_cap > 0 ? a.test_sweep_cap : 30 * s + 30;
    while (cm > 0 && nsweep < cap) {
        if (fabsf(e[cm - 1]) <= DC_EPS * (fabsf(d[cm - 1]) + fabsf(d[cm])) || fabsf(e[cm - 1]) <= tiny) {
            cm--;
            continue;
        }
        int l = cm - 1;
        while (l > 0 && !(fabsf(e[l - 1]) <= DC_EPS * (fabsf(d[l - 1]) + fabsf(d[l])) || fabsf(e[l - 1]) <= tiny)) l--;
        const float t = 0.5f * (d[cm - 1] - d[cm]);
        const float bb = e[cm - 1];
        const float den = t + copysignf(sqrtf(t * t + bb * bb), t);
        const float mu = d[cm] - (den != 0.f ? bb * bb / den : 0.f);
        float x = d[l] - mu, z = e[l];
        for (int k = l; k < cm; k++) {
            // every lane reads the same scalars, then lane 0 alone writes them back
            const float dk = d[k], dk1 = d[k + 1], ek = e[k], ek1 = k + 1 < cm ? e[k + 1] : 0.f;
            __syncwarp();
            const float r = sqrtf(x * x + z * z);
            const float c = r > 0.f ? x / r : 1.f, sn = r > 0.f ? z / r : 0.f;
            const float g = sn * (dk - dk1) - 2.f * c * ek;
            const float ekn = c * sn * (dk1 - dk) + (c * c - sn * sn) * ek;
            if (lane == 0) {
                if (k > l) e[k - 1] = r;
                d[k] = dk - sn * g;
                d[k + 1] = dk1 + sn * g;
                e[k] = ekn;
                if (k + 1 < cm) e[k + 1] = c * ek1;
            }
            if (k + 1 < cm) {
                z = sn * ek1;
                x = ekn;
            }
            if (lane < s) {
                const float z0 = Z[lane][k], z1 = Z[lane][k + 1];
                Z[lane][k] = c * z0 + sn * z1;
                Z[lane][k + 1] = c * z1 - sn * z0;
            }
            __syncwarp();
        }
        nsweep++;
    }
    if (lane == 0 && nsweep >= cap && a.status) a.status[m] = 1;
    // ascending order (ties by index)
    if (lane < s) {
        int r = 0;
        for (int i = 0; i < s; i++) r += cir_before(d[i], i, d[lane], lane);
        rk[warp][lane] = r;
    }
    __syncwarp();
    if (lane < s) dw[a0 + rk[warp][lane]] = d[lane];
    for (int c = 0; c < s; c++)
        if (lane < s) Q[(size_t)(a0 + rk[warp][c]) * ld + a0 + lane] = Z[lane][c];
}

// ---------------------------------------------------------------------------------------
// Merges of one level.
// ---------------------------------------------------------------------------------------
struct DcSmem {      // offsets (floats) of the merge block's arrays for a merge of size <= KM
    int D, Ds, zs, z2, Dn, tau, zh, inv, vals, perm, kind, nidx, defl, org, src, rot, red, total;
    __host__ __device__ DcSmem(int KM) {
        int o = 0;
        D = o; o += KM;
        Ds = o; o += KM;
        zs = o; o += KM;
        z2 = o; o += KM;
        Dn = o; o += KM;
        tau = o; o += KM;
        zh = o; o += KM;
        inv = o; o += KM;
        vals = o; o += KM;
        perm = o; o += KM;     // int
        kind = o; o += KM;     // int: index among the non-deflated, or -1
        nidx = o; o += KM;     // int: sorted index of non-deflated i
        defl = o; o += KM;     // int: sorted index of deflated q
        org = o; o += KM;      // int
        src = o; o += KM;      // int: final column -> value index
        rot = o; o += 4 * KM;  // rotations (p, j as int; c, s)
        red = o; o += 64;
        total = o;
    }
};

template <int NT>
__device__ float dc_block_max(float v, float *red) {
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    float r = 0.f;
    for (int w = 0; w < NT / 32; w++) r = fmaxf(r, red[w]);
    return r;
}

template <int NT>
__device__ float dc_block_sum(float v, float *red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[32 + (threadIdx.x >> 5)] = v;
    __syncthreads();
    float r = 0.f;
    for (int w = 0; w < NT / 32; w++) r += red[32 + w];
    return r;
}

// root i of 1/rho + sum_j z2_j / (Dn_j - lambda); returns the origin index, *tau = lambda - Dn[origin]
__device__ int dc_root(int i, int Kp, const float *Dn, const float *z2, float rho, float z2sum, float *tau_out,
                       int *iters) {
    const float rinv = 1.f / rho;
    int o;
    float lo, hi;
    if (i < Kp - 1) {
        const float gap = Dn[i + 1] - Dn[i];
        const float mid = 0.5f * gap;
        const float base = Dn[i];
        float g = rinv;
        for (int j = 0; j < Kp; j++) g += z2[j] / ((Dn[j] - base) - mid);
        if (g >= 0.f) { o = i; lo = 0.f; hi = mid; }
        else { o = i + 1; lo = mid - gap; hi = 0.f; }
    } else {
        o = i; lo = 0.f; hi = rho * z2sum;
    }
    const float dorg = Dn[o];
    const int ip = i < Kp - 1 ? i : Kp - 2;   // poles ip, ip+1 of the local model
    float t = 0.5f * (lo + hi);
    int it = 0;
    for (; it < 64; it++) {
        // the poles up to ip (psi) and beyond (phi) in two loops; one reciprocal per term,
        // approximate (1 ulp), well inside the 8 eps sum(|terms|) convergence bound below
        float psi = 0.f, phi = 0.f, dpsi = 0.f, dphi = 0.f;
        for (int j = 0; j <= ip; j++) {
            const float rl = __fdividef(1.f, (Dn[j] - dorg) - t);
            const float q = z2[j] * rl;
            psi += q;
            dpsi = fmaf(q, rl, dpsi);
        }
        for (int j = ip + 1; j < Kp; j++) {
            const float rl = __fdividef(1.f, (Dn[j] - dorg) - t);
            const float q = z2[j] * rl;
            phi += q;
            dphi = fmaf(q, rl, dphi);
        }
        const float di = ip >= 0 ? (Dn[ip] - dorg) - t : 0.f;
        const float dj = ip + 1 < Kp ? (Dn[ip + 1] - dorg) - t : 0.f;
        const float g = rinv + psi + phi;
        const float errb = 8.f * (fabsf(psi) + fabsf(phi)) + 2.f * rinv;
        if (fabsf(g) <= DC_EPS * errb) break;
        if (g < 0.f) lo = t;
        else hi = t;
        float eta;
        if (Kp == 1) {
            eta = -g / (dpsi + dphi);
        } else {
            const float C = g - di * dpsi - dj * dphi;
            const float A = (di + dj) * g - di * dj * (dpsi + dphi);
            const float B = di * dj * g;
            const float disc = sqrtf(fabsf(A * A - 4.f * B * C));
            if (C == 0.f) eta = A != 0.f ? B / A : -g / (dpsi + dphi);
            else if (A <= 0.f) eta = (A - disc) / (2.f * C);
            else eta = 2.f * B / (A + disc);
            if (g * eta >= 0.f) eta = -g / (dpsi + dphi);
        }
        float tn = t + eta;
        if (!(tn > lo && tn < hi)) tn = 0.5f * (lo + hi);
        const bool done = tn == t || hi - lo <= DC_EPS * fmaxf(fabsf(lo), fabsf(hi));
        t = tn;
        if (done) break;
    }
    *tau_out = t;
    *iters = it + 1;
    return o;
}

template <int NT>
__global__ void __launch_bounds__(NT) k_dc_merge(EighArgs a, int level, int KM, const float *Qin, float *Uout) {
    extern __shared__ __align__(16) float sm[];
    const DcSmem L(KM);
    float *D = sm + L.D, *Ds = sm + L.Ds, *zs = sm + L.zs, *z2 = sm + L.z2, *Dn = sm + L.Dn, *tau = sm + L.tau;
    float *zh = sm + L.zh, *inv = sm + L.inv, *vals = sm + L.vals, *red = sm + L.red;
    int *perm = reinterpret_cast<int *>(sm + L.perm), *kind = reinterpret_cast<int *>(sm + L.kind);
    int *nidx = reinterpret_cast<int *>(sm + L.nidx), *defl = reinterpret_cast<int *>(sm + L.defl);
    int *org = reinterpret_cast<int *>(sm + L.org), *src = reinterpret_cast<int *>(sm + L.src);
    float *rot = sm + L.rot;
    __shared__ int s_kp, s_m, s_nd;
    // optional per-phase timers of the merges (EighArgs.phase_ns slots 7-11, summed over merges)
    unsigned long long *pt = a.phase_ns ? a.phase_ns + (size_t)blockIdx.y * CIR_EIG_PROF_SLOTS : nullptr;
    unsigned long long tl = 0;
    auto mark = [&](int slot) {
        if (!pt) return;
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned long long t;
            asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
            if (slot >= 0) atomicAdd(pt + slot, t - tl);
            tl = t;
        }
    };
    mark(-1);
    const int n = a.n, ld = a.ld, tid = threadIdx.x;
    const int mat = blockIdx.y, b = blockIdx.x;
    if (b >= (1 << level)) return;
    const int a0 = dc_off(level, b, n), a1 = dc_off(level, b + 1, n), mid = dc_off(level + 1, 2 * b + 1, n);
    const int K = a1 - a0, k1 = mid - a0;
    float *dw = a.DE + (size_t)mat * 3 * ld;
    const float beta = dw[ld + mid - 1];
    const float *Q = Qin + (size_t)mat * a.mstride;
    float *U = Uout + (size_t)mat * a.mstride;
    const float rho = 2.f * fabsf(beta);
    const float sgn = beta >= 0.f ? 1.f : -1.f;
    // z and the two sorted lists
    for (int i = tid; i < K; i += NT) {
        D[i] = dw[a0 + i];
        zs[i] = (i < k1 ? Q[(size_t)(a0 + i) * ld + mid - 1] : sgn * Q[(size_t)(a0 + i) * ld + mid]) * 0.70710678118654752f;
    }
    __syncthreads();
    for (int i = tid; i < K; i += NT) {
        int rnk;
        const float v = D[i];
        // (both halves ascend in the order of cir_before, NaN last, so the ranks are a permutation)
        if (i < k1) {   // number of D2 < v
            int lo = k1, hi = K;
            while (lo < hi) { const int md = (lo + hi) >> 1; if (cir_lt(D[md], v)) lo = md + 1; else hi = md; }
            rnk = i + (lo - k1);
        } else {        // number of D1 <= v
            int lo = 0, hi = k1;
            while (lo < hi) { const int md = (lo + hi) >> 1; if (cir_le(D[md], v)) lo = md + 1; else hi = md; }
            rnk = (i - k1) + lo;
        }
        perm[rnk] = i;
    }
    __syncthreads();
    float mx = 0.f;
    for (int r = tid; r < K; r += NT) {
        const int i = perm[r];
        Ds[r] = D[i];
        z2[r] = zs[i];       // z in sorted order (z2 reused below for z^2)
        mx = fmaxf(mx, fmaxf(fabsf(D[i]), fabsf(zs[i])));
    }
    const float tol = 8.f * DC_EPS * dc_block_max<NT>(mx, red);
    __syncthreads();
    for (int r = tid; r < K; r += NT) zs[r] = z2[r];
    __syncthreads();
    // deflation (LAPACK laed2): sequential scan over the sorted entries
    if (tid == 0) {
        int kp = 0, nd = 0, m = 0, pj = -1;
        for (int j = 0; j < K; j++) {
            if (rho * fabsf(zs[j]) <= tol) { kind[j] = -1; defl[nd++] = j; continue; }
            if (pj < 0) { pj = j; continue; }
            // close pair test |t c s| <= tol with c = z_j / tt, s = -z_pj / tt, tt^2 = z_j^2 + z_pj^2,
            // multiplied through by tt^2 (no division unless the pair deflates)
            const float zj = zs[j], zp = zs[pj], t = Ds[j] - Ds[pj];
            if (fabsf(t * zj * zp) <= tol * fmaf(zj, zj, zp * zp)) {
                const float tt = hypotf(zj, zp);
                const float c = zj / tt, s = -zp / tt;
                zs[j] = tt;
                zs[pj] = 0.f;
                reinterpret_cast<int *>(rot)[4 * m] = pj;
                reinterpret_cast<int *>(rot)[4 * m + 1] = j;
                rot[4 * m + 2] = c;
                rot[4 * m + 3] = s;
                m++;
                const float t2 = Ds[pj] * c * c + Ds[j] * s * s;
                Ds[j] = Ds[pj] * s * s + Ds[j] * c * c;
                Ds[pj] = t2;
                kind[pj] = -1;
                defl[nd++] = pj;
                pj = j;
            } else {
                kind[pj] = kp;
                nidx[kp++] = pj;
                pj = j;
            }
        }
        if (pj >= 0) { kind[pj] = kp; nidx[kp++] = pj; }
        s_kp = kp;
        s_m = m;
        s_nd = nd;
    }
    __syncthreads();
    const int Kp = s_kp, nrot = s_m, nd = s_nd;
    float zpart = 0.f;
    for (int i = tid; i < Kp; i += NT) {
        const int r = nidx[i];
        Dn[i] = Ds[r];
        const float zz = zs[r];
        z2[i] = zz * zz;
        zh[i] = zz;          // sign carrier until the recomputation below
        zpart += zz * zz;
    }
    const float z2sum = dc_block_sum<NT>(zpart, red);
    __syncthreads();
    mark(7);
    // secular roots
    int nit = 0;
    for (int i = tid; i < Kp; i += NT) {
        float t;
        int itc;
        org[i] = dc_root(i, Kp, Dn, z2, rho, z2sum, &t, &itc);
        tau[i] = t;
        nit += itc;
    }
    if (pt && nit) {
        atomicAdd(pt + 18, (unsigned long long)nit);
        atomicAdd(pt + 19, (unsigned long long)((Kp - tid + NT - 1) / NT > 0 ? (Kp - tid + NT - 1) / NT : 0));
    }
    __syncthreads();
    mark(8);
    // Gu-Eisenstat: zh_j^2 = -prod_i (Dn_j - lambda_i) / prod_{i != j} (Dn_j - Dn_i)
    for (int j = tid; j < Kp; j += NT) {
        const float dj = Dn[j];
        float p = (dj - Dn[org[j]]) - tau[j];
        for (int i = 0; i < Kp; i++)
            if (i != j) p *= ((dj - Dn[org[i]]) - tau[i]) / (dj - Dn[i]);
        vals[j] = copysignf(sqrtf(fmaxf(-p, 0.f)), zh[j]);
    }
    __syncthreads();
    for (int j = tid; j < Kp; j += NT) zh[j] = vals[j];
    __syncthreads();
    for (int i = tid; i < Kp; i += NT) {
        const float base = Dn[org[i]], ti = tau[i];
        float sq = 0.f;
        for (int j = 0; j < Kp; j++) {
            const float u = __fdividef(zh[j], (Dn[j] - base) - ti);
            sq = fmaf(u, u, sq);
        }
        inv[i] = 1.f / sqrtf(sq);
    }
    mark(9);
    // eigenvalues: roots then deflated values; ascending rank (ties by index)
    for (int q = tid; q < K; q += NT) vals[q] = q < Kp ? Dn[org[q]] + tau[q] : Ds[defl[q - Kp]];
    __syncthreads();
    for (int q = tid; q < K; q += NT) {
        const float v = vals[q];
        int r = 0;
        for (int i = 0; i < K; i++) r += cir_before(vals[i], i, v, q);
        src[r] = q;
        dw[a0 + r] = v;
    }
    __syncthreads();
    mark(10);
    // U = P G W without an intermediate: G = G_0 G_1 ... G_{nrot-1} are the deflation
    // rotations (G_t mixes the sorted rows p_t, j_t: p' = c p - s j, j' = s p + c j), W the
    // secular vectors in the sorted basis; rows that no rotation touches take W directly.
    // The deflation scan leaves the rotations in chains: rotation t+1 continues the chain of
    // rotation t when p_{t+1} = j_t, and no other rotation touches p_t or j_t.  Applied from
    // the last to the first, rotation t therefore reads row p_t from W and row j_t from the
    // previous step's p row (or from W at the end of a chain); row j_t is then final, and
    // row p_t is carried to rotation t-1 or, at the start of a chain, written.  The values
    // and the order of the operations are those of applying every rotation to a full copy.
    int *touched = reinterpret_cast<int *>(D);   // D is free once the two lists are merged
    const int *rotp = reinterpret_cast<const int *>(rot);
    for (int r = tid; r < K; r += NT) touched[r] = 0;
    __syncthreads();
    for (int t = tid; t < nrot; t += NT) {
        touched[rotp[4 * t]] = 1;
        touched[rotp[4 * t + 1]] = 1;
    }
    __syncthreads();
    for (int c = tid; c < K; c += NT) {
        const int q = src[c];
        const bool root = q < Kp;
        const float base = root ? Dn[org[q]] : 0.f, ti = root ? tau[q] : 0.f, sc = root ? inv[q] : 0.f;
        const int pd = root ? -1 : defl[q - Kp];
        auto w = [&](int r) -> float {   // W[r][c]: secular vector entry, or the deflated unit vector
            if (!root) return r == pd ? 1.f : 0.f;
            const int jn = kind[r];
            return jn >= 0 ? zh[jn] / ((Dn[jn] - base) - ti) * sc : 0.f;
        };
        float *Uc = U + (size_t)a0 * ld + a0 + c;
        for (int r = 0; r < K; r++)
            if (!touched[r]) Uc[(size_t)perm[r] * ld] = w(r);
        float carry = 0.f;
        for (int t = nrot - 1; t >= 0; t--) {
            const int p = rotp[4 * t], j = rotp[4 * t + 1];
            const float cc = rot[4 * t + 2], ss = rot[4 * t + 3];
            const float rp = w(p), rj = (t + 1 < nrot && rotp[4 * (t + 1)] == j) ? carry : w(j);
            carry = cc * rp - ss * rj;
            Uc[(size_t)perm[j] * ld] = ss * rp + cc * rj;
            if (t == 0 || rotp[4 * (t - 1) + 1] != p) Uc[(size_t)perm[p] * ld] = carry;
        }
    }
    mark(11);
    (void)nd;
}

// Q_new = diag(Q1, Q2) U for every merge of a level: blockIdx.y = matrix, blockIdx.x =
// (merge, half, tile over (rows of the half) x (K columns)).  Q column-major (ld), U row-major
// (ld), 64 x 64 tiles, 16-deep k steps, 4 x 4 outputs per thread.
__global__ void __launch_bounds__(256) k_dc_gemm(EighArgs a, int level, int tiles, const float *Qin, const float *Uin,
                                                 float *Qout) {
    __shared__ float As[16][64 + 4];
    __shared__ float Bs[16][64 + 4];
    const int n = a.n, ld = a.ld;
    const int z = blockIdx.x / tiles, half = z & 1, b = z >> 1;
    const int mat = blockIdx.y;
    const int a0 = dc_off(level, b, n), a1 = dc_off(level, b + 1, n), mid = dc_off(level + 1, 2 * b + 1, n);
    const int K = a1 - a0;
    const int h0 = half ? mid : a0, hK = half ? a1 - mid : mid - a0;   // rows/k range of this half
    const int tr = (hK + 63) / 64, tc = (K + 63) / 64;
    const int tile = blockIdx.x - z * tiles;
    if (tile >= tr * tc) return;
    const int r0 = (tile % tr) * 64, c0 = (tile / tr) * 64;
    const float *Q = Qin + (size_t)mat * a.mstride;
    const float *U = Uin + (size_t)mat * a.mstride;
    float *C = Qout + (size_t)mat * a.mstride;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    float acc[4][4] = {};
    for (int k0 = 0; k0 < hK; k0 += 16) {
        for (int q = threadIdx.x; q < 16 * 64; q += 256) {
            const int kk = q >> 6, i = q & 63;
            const int k = k0 + kk;
            As[kk][i] = (k < hK && r0 + i < hK) ? Q[(size_t)(h0 + k) * ld + h0 + r0 + i] : 0.f;
            Bs[kk][i] = (k < hK && c0 + i < K) ? U[(size_t)(h0 + k) * ld + a0 + c0 + i] : 0.f;
        }
        __syncthreads();
        #pragma unroll
        for (int kk = 0; kk < 16; kk++) {
            float av[4], bv[4];
            #pragma unroll
            for (int i = 0; i < 4; i++) av[i] = As[kk][ty + 16 * i];
            #pragma unroll
            for (int j = 0; j < 4; j++) bv[j] = Bs[kk][tx + 16 * j];
            #pragma unroll
            for (int i = 0; i < 4; i++)
                #pragma unroll
                for (int j = 0; j < 4; j++) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
        }
        __syncthreads();
    }
    #pragma unroll
    for (int j = 0; j < 4; j++) {
        const int c = c0 + tx + 16 * j;
        if (c >= K) continue;
        #pragma unroll
        for (int i = 0; i < 4; i++) {
            const int r = r0 + ty + 16 * i;
            if (r < hK) C[(size_t)(a0 + c) * ld + h0 + r] = acc[i][j];
        }
    }
}

// W (ascending eigenvalues) and the IPR histograms (calcIR.cu:493-538) of V's columns.
__global__ void __launch_bounds__(256) k_dc_finish(EighArgs a) {
    const int n = a.n, ld = a.ld, mat = blockIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const float *dw = a.DE + (size_t)mat * 3 * ld;
    const float *V = a.A + (size_t)mat * a.mstride;
    for (int i = threadIdx.x; i < n; i += blockDim.x) a.W[(size_t)mat * a.wstride + i] = dw[i];
    if (!a.hist_count) return;
    for (int j = warp; j < n; j += blockDim.x / 32) {
        const float *col = V + (size_t)j * ld;
        float s4 = 0.f, m4 = 0.f;
        for (int i0 = 0; i0 < n; i0 += 32) {
            const int i = i0 + lane;
            const float v = i < n ? col[i] : 0.f;
            const float v2 = v * v;
            s4 += v2 * v2;
            if (a.nchrom_mol == 2) {
                const float pair = v2 + __shfl_xor_sync(0xffffffffu, v2, 1);
                if ((lane & 1) == 0) m4 += pair * pair;
            } else {
                m4 += v2 * v2;
            }
        }
        s4 = warp_sum(s4);
        m4 = warp_sum(m4);
        if (lane == 0) {
            const float wi = dw[j] + a.avef;
            const int bin = (int)roundf((wi - a.omegaStart) / (float)a.omegaStep);
            const size_t grp = a.hist_group > 0 ? (size_t)(mat / a.hist_group) : 0;
            const int wgt = a.hist_weight ? a.hist_weight[mat] : 1;   // a frame shared by origins counts for each
            if (bin >= 0 && bin < a.nomega) {
                atomicAdd(a.hist_count + grp * a.nomega + bin, (unsigned long long)wgt);
                atomicAdd(a.hist_ipr + grp * a.nomega + bin, (double)wgt * (double)(1.f / s4));
                atomicAdd(a.hist_mipr + grp * a.nomega + bin, (double)wgt * (double)(1.f / m4));
            } else {
                atomicAdd(a.out_of_range + grp, (unsigned long long)wgt);
            }
        }
    }
}

// CIR_Q_PAIR=0: the top merge writes Q_T in FP32 and the back-transform splits it (for comparison)
bool pair_q_enabled() {
    static const bool on = [] {
        const char *v = getenv("CIR_Q_PAIR");
        return !(v && v[0] == '0');
    }();
    return on;
}

int dc_depth(int n) {
    int D = 0;
    while (((n + (1 << D) - 1) >> D) > DC_LEAF) D++;
    return D;
}

}  // namespace

size_t cir_dc_bytes(int n, int ld) { return sizeof(float) * 3 * (size_t)n * ld; }

// Stage 2 of the divide-and-conquer eigensolver: everything after the tridiagonalisation
// (DE holds d, e, tau; A the reflectors).  a.DC: 3 buffers of a.mstride floats per matrix
// (Q_T ping, pong, U), laid out [buffer][matrix]; a.Z is scratch of the back-transform.
cudaError_t cir_launch_dc(const EighArgs &a, int nmat, cudaStream_t s, int *launches) {
    const int n = a.n, ld = a.ld;
    const int D = dc_depth(n);
    float *buf[3] = {a.DC, a.DC + (size_t)nmat * a.mstride, a.DC + 2 * (size_t)nmat * a.mstride};
    const int nleaf = 1 << D;
    k_dc_leaf<<<dim3((nleaf + 3) / 4, nmat), 128, 0, s>>>(a, D, buf[0]);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    int nl = 1;
    int cur = 0;
    // the split-BF16 back-transform takes Q_T as a BF16 pair: the top merge's tensor-core
    // product writes it so directly, and the back-transform skips its own split of Q_T
    const bool q_pair = a.precision == CIR_PREC_BF16X3 && (ld & 7) == 0 && n > 2 && pair_q_enabled();
    bool q_split = false;
    for (int level = D - 1; level >= 0; level--) {
        const int KM = ((n + (1 << level) - 1) >> level);
        const DcSmem L(KM);
        const size_t smem = sizeof(float) * L.total;
        const int other = cur ^ 1;
        // small merges in small blocks, so that many of them share an SM
        auto merge = [&](auto kern, int nt) -> cudaError_t {
            cudaError_t r = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (r != cudaSuccess) return r;
            kern<<<dim3(1 << level, nmat), nt, smem, s>>>(a, level, KM, buf[cur], buf[2]);
            return cudaSuccess;
        };
        e = KM <= 64 ? merge(k_dc_merge<64>, 64) : KM <= 128 ? merge(k_dc_merge<128>, 128)
          : KM <= 512 ? merge(k_dc_merge<DC_NT>, DC_NT) : merge(k_dc_merge<2 * DC_NT>, 2 * DC_NT);
        if (e != cudaSuccess) return e;
        // the top three levels of the mixed forms on the tensor cores: one batched product per
        // merge half when every offset keeps 16-byte alignment
        bool tc = a.precision != CIR_PREC_FP32 && level <= 2;
        for (int b = 0; tc && b < (1 << level); b++)
            tc = (dc_off(level, b, n) & 3) == 0 && (dc_off(level + 1, 2 * b + 1, n) & 3) == 0;
        if (tc) {
            for (int b = 0; b < (1 << level); b++) {
                const int a0 = dc_off(level, b, n), a1 = dc_off(level, b + 1, n), mid = dc_off(level + 1, 2 * b + 1, n);
                for (int half = 0; half < 2; half++) {
                    const int h0 = half ? mid : a0, hK = half ? a1 - mid : mid - a0;
                    // column-major Q_new block = Q_half U_half; in the row-major view the
                    // transpose: C^T = U_half^T Q_half^T
                    GemmArgs g{};
                    g.A = buf[2] + (size_t)h0 * ld + a0;        // U rows h0.., columns a0.. (row-major)
                    g.B = buf[cur] + (size_t)h0 * ld + h0;      // Q block (column-major)
                    g.C = buf[other] + (size_t)a0 * ld + h0;
                    g.M = a1 - a0;
                    g.N = hK;
                    g.K = hK;
                    g.lda = g.ldb = g.ldc = ld;
                    g.sA = g.sB = g.sC = a.mstride;
                    g.a_colmajor = true;
                    g.epilogue = 0;
                    g.err = a.err;
                    if (level == 0 && q_pair) {
                        __nv_bfloat16 *pb = reinterpret_cast<__nv_bfloat16 *>(buf[other]) + (size_t)a0 * ld + h0;
                        g.Chi = pb;
                        g.Clo = pb + a.mstride;
                    }
                    e = cir_launch_tc_gemm(g, nmat, a.precision, s, nullptr);
                    if (e != cudaSuccess) return e;
                    nl++;
                }
            }
            nl++;
            if (level == 0 && q_pair) q_split = true;
        } else {
            const int tiles = ((KM / 2 + 1 + 63) / 64) * ((KM + 63) / 64);
            k_dc_gemm<<<dim3(tiles * (1 << level) * 2, nmat), 256, 0, s>>>(a, level, tiles, buf[cur], buf[2], buf[other]);
            nl += 2;
        }
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        cur = other;
    }
    // V = Q_H Q_T into a.A: the reflectors applied to Q_T (buf[cur]) in compact WY blocks,
    // with the free ping-pong buffer as scratch
    e = cir_launch_backtransform(a, buf[cur], buf[cur ^ 1], buf[2], nmat, s, &nl, q_split);
    if (e != cudaSuccess) return e;
    // optional FP64 refinement of the eigenpairs (eigenvalues in DE row 0) before W and the
    // distributions are written
    if (a.Href) {
        e = cir_launch_refine(a.Href, a.A, a.mstride, ld, n, a.DE, 3LL * ld, nmat, a.refine_iters, a.RW,
                              a.refine_chunk, s, &nl);
        if (e != cudaSuccess) return e;
    }
    k_dc_finish<<<nmat, 256, 0, s>>>(a);
    nl += 1;
    if (launches) *launches += nl;
    return cudaGetLastError();
}
