// Batched symmetric eigensolver for the exciton Hamiltonians (replaces magma_ssyevd_gpu,
// calcIR.cu:420-448).  Three kernels, each with one thread block per matrix, so the SMs
// work on independent frames at once: k_eigh_tq (phase 1), k_eigh_formq (phase 2) and
// k_eigh_qr (phases 3-4, 128 threads: one chasing warp and three applying warps, three
// blocks per SM so that three bulge chases overlap on every SM).
//
//  1. Householder tridiagonalisation Q^T H Q = T (reflectors stored below the subdiagonal,
//     as LAPACK sytrd).  Orders above 256: blocked, lower storage, panels of TB_NB columns
//     (tiled symmetric matrix-vector products, one rank-2*TB_NB update per panel).  Smaller
//     orders: the rank-2 update of step k-1 and the matrix-vector product of step k share
//     one read/write pass over the trailing block.
//  2. Q is formed explicitly in Z by backward accumulation of the reflectors in compact WY
//     blocks, each warp holding its rows of the block's reflectors in registers.  (The
//     divide-and-conquer path, a.DC set, skips phases 2-4: it solves the tridiagonal
//     problem in k_dc.cu and applies the reflectors to its eigenvectors afterwards,
//     k_backtransform.cu.)
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
#include <algorithm>
#include <cstring>
#include <mutex>

namespace {

__device__ __forceinline__ unsigned long long globaltimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

constexpr int EIG_KS = 16;     // QR sweeps per wavefront group in phase 3
constexpr int EIG_W = EIG_KS + 1;
constexpr int QR_AHEAD = 12;    // Z columns copied ahead of the wavefront in phase 3

// 4-byte asynchronous global-to-shared copy (src_size 0: zero fill), group commit and wait
__device__ __forceinline__ void cp_async4(float *dst, const float *src, bool valid) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    const int sz = valid ? 4 : 0;   // 0: fill with zeros
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(d), "l"(src), "r"(sz) : "memory");
}
// 16-byte asynchronous global-to-shared copy (zero fill when !valid)
__device__ __forceinline__ void cp_async16(float *dst, const float *src, bool valid) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    const int sz = valid ? 16 : 0;
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(d), "l"(src), "r"(sz) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
// request the 128-byte line holding p into L2 (no data returned, no register held)
__device__ __forceinline__ void prefetch_l2(const float *p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// Blocked tridiagonalisation (orders above 256): panels of TB_NB columns, LAPACK sytrd/latrd
// with lower storage.  Within a panel each column's matrix-vector product reads the lower
// triangle of the trailing block as it stood at the start of the panel and corrects for the
// panel's earlier columns with V and W; after the panel the trailing block is updated once,
// A -= V W^T + W V^T, in TB_KC-column steps staged in shared memory.
constexpr int TB_NB = 32;      // panel width
constexpr int TB_KC = 8;       // panel columns per staged step of the trailing update
constexpr int TB_ROWS = 128;   // rows of a trailing-update tile

__host__ __device__ constexpr int tb_cols(int nt) { return 4 * (nt / 16); }   // its columns
__host__ __device__ constexpr int tb_stage(int nt) { return TB_KC * (2 * TB_ROWS + 2 * tb_cols(nt)); }

// floats of phase 1's shared work area: the four vectors of the unblocked path, or the
// blocked state (x, one partial product per warp, the staging tiles aliasing those, 4 panel
// vectors)
__host__ __device__ inline size_t tq_union_floats(int n, int nt, bool blocked) {
    const size_t n4 = (size_t)((n + 3) & ~3), n32 = (size_t)((n + 31) & ~31);
    if (!blocked) return 4 * n4;
    const size_t yw = n32 * (nt / 32), st = 2 * (size_t)tb_stage(nt);   // two staging buffers
    return n32 + (yw > st ? yw : st) + 4 * TB_NB;
}

size_t tq_smem_bytes(int n, int nt, bool blocked) {
    const size_t n4 = (size_t)((n + 3) & ~3);
    return sizeof(float) * (3 * n4 + tq_union_floats(n, nt, blocked) + 64);
}

// d, e, ranks, the group bookkeeping, then the appliers' column ring (QR_AHEAD+1 slots of
// rows x applying threads)
__host__ __device__ inline size_t qr_ring_offset_floats(int n) {
    const size_t n4 = (size_t)((n + 3) & ~3);
    return 3 * n4 + 4 * EIG_KS + 8;
}

size_t qr_smem_bytes(int n, int nt, int rows) {
    return sizeof(float) * (qr_ring_offset_floats(n) + (size_t)(QR_AHEAD + 1) * rows * (nt - 32));
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
    int l;                         // start of the block of the previous sweep (-1: none yet)
    int js;                        // largest split found during the previous sweep (-1: none)
    float tiny;
    long long nrot;
    bool timed;                    // accumulate t_search (profiling only)
    unsigned long long t_search;   // ns spent locating the unreduced block and the shift
};

// One implicit QR sweep with the Wilkinson shift on the trailing unreduced block of
// (d, e); rotation i (acting on columns i, i+1) goes to rot[(i + s_slot) * EIG_KS].
// Returns false when T is diagonal or the sweep cap is reached.
// rot points at slot s of a time-major group buffer: rotation i of this sweep is stored at
// rot[(i + s) * EIG_KS], so the EIG_KS rotations applied at one wavefront step share one
// 128-byte line.
// The block [l, cm] is found without rescanning it: a sweep records the largest index whose
// new off-diagonal is negligible, and a split, once used, is set to zero (as LAPACK ssteqr
// does) so that it stays one when d[l] moves; only when the bottom deflates past every known
// split is the block below scanned.
__device__ bool qr_sweep(Chaser &ch, float *d, float *e, float2 *rot, int s_slot, int *lo, int *hi) {
    const unsigned long long ts = ch.timed ? globaltimer_ns() : 0ull;
    int cm = ch.cm;
    while (cm > 0 && negligible(e[cm - 1], d[cm - 1], d[cm], ch.tiny)) { e[cm - 1] = 0.f; cm--; }
    ch.cm = cm;
    if (cm == 0) return false;
    if (ch.nsweep >= ch.cap) { ch.status = 1; return false; }
    int l;
    if (ch.js >= 0 && cm > ch.js + 1) l = ch.js + 1;
    else if (ch.js < 0 && ch.l >= 0 && cm > ch.l) l = ch.l;
    else {
        l = cm - 1;
        while (l > 0 && !negligible(e[l - 1], d[l - 1], d[l], ch.tiny)) l--;
    }
    if (l > 0) e[l - 1] = 0.f;
    ch.l = l;
    const float t = 0.5f * (d[cm - 1] - d[cm]);
    const float bb = e[cm - 1];
    const float den = t + copysignf(sqrtf(t * t + bb * bb), t);
    const float mu = d[cm] - (den != 0.f ? bb * bb / den : 0.f);
    if (ch.timed) ch.t_search += globaltimer_ns() - ts;
    // bulge state in registers: dk = current d[k], ek = current e[k]; dk1/ek1 are the
    // untouched d[k+1], e[k+1], loaded one iteration ahead
    float x = d[l] - mu, z = e[l];
    float dk = d[l], ek = e[l];
    float dk1 = d[l + 1], ek1 = (l + 1 < cm) ? e[l + 1] : 0.f;
    float dprev = 0.f;
    int js = -1;
    for (int k = l; k < cm; k++) {
        const float dk2 = (k + 2 <= cm) ? d[k + 2] : 0.f;
        const float ek2 = (k + 2 < cm) ? e[k + 2] : 0.f;
        const float r2 = x * x + z * z;
        // reciprocal square root refined by one FMA-based Newton step (as accurate as a
        // correctly rounded rsqrt for the orthogonality of the rotations), computed without
        // a branch; r2 below 1e-30 takes sqrt and division
        const float i0 = rsqrtf(r2);
        const float res = fmaf(-(r2 * i0), i0, 1.0f);
        const float inv = fmaf(0.5f * i0, res, i0);
        const bool big = r2 >= 1e-30f;
        float c = big ? x * inv : 1.f, s = big ? z * inv : 0.f, r = big ? r2 * inv : 0.f;
        if (!big && r2 > 0.f) {
            r = sqrtf(r2);
            c = x / r;
            s = z / r;
        }
        if (k > l) e[k - 1] = r;
        const float g = s * (dk - dk1) - 2.f * c * ek;
        const float dkn = dk - s * g;
        d[k] = dkn;
        if (k > l && negligible(r, dprev, dkn, ch.tiny)) js = k - 1;
        dprev = dkn;
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
    if (negligible(e[cm - 1], dprev, dk, ch.tiny)) js = cm - 1;
    ch.js = js;
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
// column is read and written once per group.  Columns are streamed QR_AHEAD steps ahead
// through a per-thread ring of QR_AHEAD+1 slots in shared memory (cp.async, so the DRAM
// latency is covered without registers); ring + (slot * R + j) * stride is this thread's
// element for row j.  row[j] < 0 marks an unused row slot.
template <int R>
__device__ __forceinline__ void apply_group(float *Z, int ld, const int (&row)[R], const float2 *rot,
                                            int T0, int T1, int cmin, int cmax, float *ring, int stride) {
    constexpr int NS = QR_AHEAD + 1;
    float w[R][EIG_W];
    // columns T0-EIG_KS+1 .. T0 into slots 0 .. EIG_KS-1
    #pragma unroll
    for (int v = 0; v < EIG_KS; v++) {
        const int c = T0 - EIG_KS + 1 + v;
        const bool ok = c >= cmin && c <= cmax;
        #pragma unroll
        for (int j = 0; j < R; j++) w[j][v] = (ok && row[j] >= 0) ? __ldcg(Z + (size_t)c * ld + row[j]) : 0.f;
    }
    // columns T0+1 .. T0+QR_AHEAD into the ring (column c in slot c mod NS)
    auto fetch = [&](int c) {
        const int slot = c % NS;
        const bool okc = c >= cmin && c <= cmax;
        #pragma unroll
        for (int j = 0; j < R; j++) {
            const bool ok = okc && row[j] >= 0;
            cp_async4(ring + (slot * R + j) * stride, ok ? Z + (size_t)c * ld + row[j] : Z, ok);
        }
        cp_async_commit();
    };
    #pragma unroll 1
    for (int q = 1; q <= QR_AHEAD; q++) fetch(T0 + q);
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
        {   // column tau+1 from the ring into the last slot; its slot's previous column (tau)
            // was consumed a step ago, so column tau+1+QR_AHEAD may be fetched into ...(tau) mod NS
            cp_async_wait<QR_AHEAD - 1>();
            const int slot = (tau + 1) % NS;
            #pragma unroll
            for (int j = 0; j < R; j++) w[j][EIG_KS] = ring[(slot * R + j) * stride];
            fetch(tau + 1 + QR_AHEAD);
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
            for (int v = 0; v < EIG_KS; v++) w[j][v] = w[j][v + 1];
    }
    cp_async_wait<0>();
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

// ---- blocked tridiagonalisation (phase 1 for orders above 256) ----

// y += A x on one 32 x 32 tile (I, J), I >= J, of the lower triangle, for both halves of
// the symmetric matrix: A_IJ x_J into rows 32I.., A_IJ^T x_I into rows 32J...  Lane
// (g, h) = (lane & 7, lane >> 3) loads rows 32I+4g..+3 of columns 32J+8h..+7 with 16-byte
// accesses (each load instruction covers four whole 128-byte column segments).  The row
// sums are reduced over h and the column sums over g by halving exchanges, after which lane
// (g, h) owns row 32I+4g+h and column 32J+8h+g; both are added to this warp's own partial
// product ywp, so no two lanes or warps write one word.  CHECK: diagonal tile (only r >= c
// counted, the diagonal once) or a tile reaching past row n-1 (rows/columns >= n masked;
// the padding rows below n may hold anything).
template <bool CHECK>
__device__ __forceinline__ void symv_tile(const float *__restrict__ A, int ld, int n, int I, int J,
                                          const float *x, float *ywp, int lane) {
    const int g = lane & 7, h = lane >> 3;
    const int r0 = 32 * I + 4 * g, c0 = 32 * J + 8 * h;
    float4 a[8];
    #pragma unroll
    for (int t = 0; t < 8; t++) {
        if (!CHECK || (r0 < n && c0 + t < n)) a[t] = __ldcg(reinterpret_cast<const float4 *>(A + (size_t)(c0 + t) * ld + r0));
        else a[t] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    const float4 xr4 = *reinterpret_cast<const float4 *>(x + r0);
    const float4 xc0 = *reinterpret_cast<const float4 *>(x + c0);
    const float4 xc1 = *reinterpret_cast<const float4 *>(x + c0 + 4);
    const float xr[4] = {xr4.x, xr4.y, xr4.z, xr4.w};
    const float xc[8] = {xc0.x, xc0.y, xc0.z, xc0.w, xc1.x, xc1.y, xc1.z, xc1.w};
    float yr[4] = {0.f, 0.f, 0.f, 0.f}, yc[8];
    #pragma unroll
    for (int t = 0; t < 8; t++) {
        float av[4] = {a[t].x, a[t].y, a[t].z, a[t].w};
        float s = 0.f;
        #pragma unroll
        for (int q = 0; q < 4; q++) {
            float ar = av[q], ac = av[q];
            if (CHECK) {
                const int r = r0 + q, c = c0 + t;
                const bool ok = r < n && c < n;
                ar = (ok && (I != J || r >= c)) ? ar : 0.f;
                ac = (ok && (I != J || r > c)) ? ac : 0.f;
            }
            yr[q] = fmaf(ar, xc[t], yr[q]);
            s = fmaf(ac, xr[q], s);
        }
        yc[t] = s;
    }
    // column sums over g (lane bits 0-2): keep the upper half where the bit is set
    #pragma unroll
    for (int i = 0; i < 4; i++) {
        const bool up = lane & 4;
        const float send = up ? yc[i] : yc[i + 4], keep = up ? yc[i + 4] : yc[i];
        yc[i] = keep + __shfl_xor_sync(0xffffffffu, send, 4);
    }
    #pragma unroll
    for (int i = 0; i < 2; i++) {
        const bool up = lane & 2;
        const float send = up ? yc[i] : yc[i + 2], keep = up ? yc[i + 2] : yc[i];
        yc[i] = keep + __shfl_xor_sync(0xffffffffu, send, 2);
    }
    {
        const bool up = lane & 1;
        const float send = up ? yc[0] : yc[1], keep = up ? yc[1] : yc[0];
        yc[0] = keep + __shfl_xor_sync(0xffffffffu, send, 1);
    }
    // row sums over h (lane bits 3-4)
    #pragma unroll
    for (int i = 0; i < 2; i++) {
        const bool up = lane & 16;
        const float send = up ? yr[i] : yr[i + 2], keep = up ? yr[i + 2] : yr[i];
        yr[i] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
    }
    {
        const bool up = lane & 8;
        const float send = up ? yr[0] : yr[1], keep = up ? yr[1] : yr[0];
        yr[0] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
    }
    ywp[r0 + h] += yr[0];
    ywp[c0 + g] += yc[0];
}

// Trailing update after a panel: A[r][c] -= sum_j V[r][j] W[c][j] + W[r][j] V[c][j] for
// q0 <= c <= r < n (lower triangle only), V = the panel's reflectors (columns p0.. of A,
// with the unit element stored), W = the panel's W columns (Wb, leading dimension ld).
// Tiles of TB_ROWS x BC on a grid starting at q0 rounded down to 4; thread (tr, tc) owns
// rows 4tr..+3 and 64+4tr..+3 and columns 4tc..+3 of a tile.  V and W rows of the tile's
// rows and columns are staged TB_KC panel columns at a time.
template <int NT>
__device__ void trail_update(float *__restrict__ A, const float *__restrict__ Wb, int n, int ld, int p0,
                             int nb, float *stage) {
    constexpr int BC = tb_cols(NT);
    constexpr int F4 = (2 * TB_ROWS + 2 * BC) / 4;     // staged float4 per panel column
    const int tid = threadIdx.x, tr = tid & 15, tc = tid >> 4;
    const int q0 = p0 + nb;
    const int R0 = q0 & ~3;
    const int mr = n - R0;
    const int ti = (mr + TB_ROWS - 1) / TB_ROWS, tj = (mr + BC - 1) / BC;
    constexpr int TBS = tb_stage(NT);                 // floats of one staging buffer
    for (int I = 0; I < ti; I++) {
        const int jmax = min(tj - 1, (TB_ROWS * I + TB_ROWS - 1) / BC);
        for (int J = 0; J <= jmax; J++) {
            const int rb = R0 + TB_ROWS * I, cb = R0 + BC * J;
            const bool full = rb + TB_ROWS <= n && cb + BC <= n && cb >= q0 && cb + BC - 1 <= rb;
            float a[8][4];
            #pragma unroll
            for (int j = 0; j < 4; j++) {
                const int c = cb + 4 * tc + j;
                #pragma unroll
                for (int hh = 0; hh < 2; hh++) {
                    const int r = rb + 64 * hh + 4 * tr;
                    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (full || (r < n && c < n)) v = __ldcg(reinterpret_cast<const float4 *>(A + (size_t)c * ld + r));
                    a[4 * hh + 0][j] = v.x; a[4 * hh + 1][j] = v.y; a[4 * hh + 2][j] = v.z; a[4 * hh + 3][j] = v.w;
                }
            }
            // V and W rows of the tile's rows and columns, TB_KC panel columns at a time, copied
            // by cp.async into one of two buffers while the other is in use
            auto stage_chunk = [&](int j0, int buf) {
                const int kc = min(TB_KC, nb - j0);
                float *Vr = stage + buf * TBS, *Wr = Vr + TB_KC * TB_ROWS, *Vc = Wr + TB_KC * TB_ROWS, *Wc = Vc + TB_KC * BC;
                for (int idx = tid; idx < kc * F4; idx += NT) {
                    const int jj = idx / F4, o = idx - jj * F4;
                    int row, part;
                    if (o < TB_ROWS / 4) { part = 0; row = rb + 4 * o; }
                    else if (o < TB_ROWS / 2) { part = 1; row = rb + 4 * (o - TB_ROWS / 4); }
                    else if (o < TB_ROWS / 2 + BC / 4) { part = 2; row = cb + 4 * (o - TB_ROWS / 2); }
                    else { part = 3; row = cb + 4 * (o - TB_ROWS / 2 - BC / 4); }
                    const float *src = (part == 0 || part == 2) ? A + (size_t)(p0 + j0 + jj) * ld
                                                                : Wb + (size_t)(j0 + jj) * ld;
                    float *dst = part == 0 ? Vr + jj * TB_ROWS + (row - rb)
                               : part == 1 ? Wr + jj * TB_ROWS + (row - rb)
                               : part == 2 ? Vc + jj * BC + (row - cb)
                                           : Wc + jj * BC + (row - cb);
                    cp_async16(dst, row < n ? src + row : src, row < n);
                }
                cp_async_commit();
            };
            __syncthreads();   // the previous tile's reads of both buffers are done
            stage_chunk(0, 0);
            for (int j0 = 0, buf = 0; j0 < nb; j0 += TB_KC, buf ^= 1) {
                const int kc = min(TB_KC, nb - j0);
                if (j0 + TB_KC < nb) {
                    stage_chunk(j0 + TB_KC, buf ^ 1);
                    cp_async_wait<1>();
                } else {
                    cp_async_wait<0>();
                }
                __syncthreads();   // every thread's copies of this chunk are in
                const float *Vr = stage + buf * TBS, *Wr = Vr + TB_KC * TB_ROWS, *Vc = Wr + TB_KC * TB_ROWS,
                            *Wc = Vc + TB_KC * BC;
                for (int jj = 0; jj < kc; jj++) {
                    const float4 v0 = *reinterpret_cast<const float4 *>(Vr + jj * TB_ROWS + 4 * tr);
                    const float4 v1 = *reinterpret_cast<const float4 *>(Vr + jj * TB_ROWS + 64 + 4 * tr);
                    const float4 w0 = *reinterpret_cast<const float4 *>(Wr + jj * TB_ROWS + 4 * tr);
                    const float4 w1 = *reinterpret_cast<const float4 *>(Wr + jj * TB_ROWS + 64 + 4 * tr);
                    const float4 vc4 = *reinterpret_cast<const float4 *>(Vc + jj * BC + 4 * tc);
                    const float4 wc4 = *reinterpret_cast<const float4 *>(Wc + jj * BC + 4 * tc);
                    const float vr[8] = {v0.x, v0.y, v0.z, v0.w, v1.x, v1.y, v1.z, v1.w};
                    const float wr[8] = {w0.x, w0.y, w0.z, w0.w, w1.x, w1.y, w1.z, w1.w};
                    const float vc[4] = {vc4.x, vc4.y, vc4.z, vc4.w};
                    const float wc[4] = {wc4.x, wc4.y, wc4.z, wc4.w};
                    #pragma unroll
                    for (int i = 0; i < 8; i++)
                        #pragma unroll
                        for (int j = 0; j < 4; j++) a[i][j] = fmaf(-vr[i], wc[j], fmaf(-wr[i], vc[j], a[i][j]));
                }
                __syncthreads();   // this buffer is refilled by the next chunk's copies
            }
            #pragma unroll
            for (int j = 0; j < 4; j++) {
                const int c = cb + 4 * tc + j;
                #pragma unroll
                for (int hh = 0; hh < 2; hh++) {
                    const int r = rb + 64 * hh + 4 * tr;
                    float *dst = A + (size_t)c * ld + r;
                    if (full) {
                        __stcg(reinterpret_cast<float4 *>(dst),
                               make_float4(a[4 * hh][j], a[4 * hh + 1][j], a[4 * hh + 2][j], a[4 * hh + 3][j]));
                    } else if (c < n && c >= q0) {
                        #pragma unroll
                        for (int q = 0; q < 4; q++)
                            if (r + q < n && r + q >= c) dst[q] = a[4 * hh + q][j];
                    }
                }
            }
        }
    }
}

// Phase 1 for orders above 256 (LAPACK ssytrd with lower storage, panels of TB_NB columns;
// the same reflectors, d, e and tau conventions as the unblocked path).  Wb (TB_NB columns
// of leading dimension ld) holds the panel's W; x, ywall (one partial product of order n32
// per warp), pv (4 x TB_NB) and stage (aliasing ywall) are shared memory.
template <int NT, int NMAX>
__device__ void tridiag_blocked(float *__restrict__ A, float *__restrict__ Wb, int n, int ld, float *d, float *e,
                                float *tau, float *x, float *ywall, float *pv, float *red, unsigned long long *pt,
                                int tq_order) {
    constexpr int NW = NT / 32;
    constexpr int RW = (NMAX + NT - 1) / NT;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int n32 = (n + 31) & ~31;
    const int tn = n32 >> 5;
    float *sv = pv, *sw = pv + TB_NB, *t1 = pv + 2 * TB_NB, *t2 = pv + 3 * TB_NB;
    float *ywp = ywall + (size_t)warp * n32;
    for (int i = tid; i < n32; i += NT) x[i] = 0.f;
    __syncthreads();
    // optional per-phase timers (pt[12..17]), read by thread 0 after a block-wide barrier
    unsigned long long tlast = (pt && tid == 0) ? globaltimer_ns() : 0ull;
    auto mark = [&](int slot) {
        if (!pt) return;
        __syncthreads();
        if (tid == 0) {
            const unsigned long long t = globaltimer_ns();
            pt[slot] += t - tlast;
            tlast = t;
        }
    };
    const int nref = n - 2;       // columns 0 .. n-3 carry reflectors
    for (int p0 = 0; p0 < nref; p0 += TB_NB) {
        const int nb = min(TB_NB, nref - p0);
        float xn2 = 0.f;   // |column k below k+1|^2; after the first column of a panel it comes
                           // from the previous column's step (d), which also leaves d[k], the
                           // alpha in red[48] and the rest of the column in x
        for (int kk = 0; kk < nb; kk++) {
            const int k = p0 + kk;
            if (kk == 0) {
                // (a) column k (rows k..n-1): the panel's first, unaffected by its reflectors
                float part = 0.f;
                for (int r = k + tid; r < n; r += NT) {
                    const float v = A[(size_t)k * ld + r];
                    if (r == k) d[k] = v;
                    else if (r == k + 1) red[48] = v;
                    else { x[r] = v; part += v * v; }
                }
                xn2 = block_sum<NT>(part, red);
            }
            mark(12);
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
            // v (unit element at k+1, stored in A during the panel) into x; x[k] cleared
            for (int r = k + tid; r < n; r += NT) {
                const float v = r == k ? 0.f : (r == k + 1 ? 1.f : x[r] * scale);
                x[r] = v;
                if (r > k) A[(size_t)k * ld + r] = v;
            }
            const int j0 = (k + 1) >> 5;
            for (int i = 32 * j0 + lane; i < n32; i += 32) ywp[i] = 0.f;
            __syncthreads();
            mark(13);
            // (c) y = A22 v on the panel-start trailing block, plus t1 = W^T v, t2 = V^T v.
            // Within a panel consecutive columns read the same tiles (A is not updated until the
            // panel ends), so alternate columns walk them in opposite orders: a column starts on
            // the tiles the previous column (or the trailing update, for a panel's first column)
            // read last, which are the ones most likely still in L2.
            {
                const int tt = tn - j0;
                const int ntiles = tt * (tt + 1) / 2;
                const bool rev = tq_order && (kk & 1) == 0;
                // tile of position L of the row-major enumeration of the lower triangle
                auto tile_of = [&](int L, int &Ii, int &Jj) {
                    int i = (int)((sqrtf(8.f * (float)L + 1.f) - 1.f) * 0.5f);
                    while (i * (i + 1) / 2 > L) i--;
                    while ((i + 1) * (i + 2) / 2 <= L) i++;
                    Ii = i;
                    Jj = L - i * (i + 1) / 2;
                };
                for (int q = warp; q < ntiles; q += NW) {
                    int Ii, Jj;
                    tile_of(rev ? ntiles - 1 - q : q, Ii, Jj);
                    if (q + NW < ntiles) {   // this warp's next tile: its lines are requested into L2
                        int In, Jn;
                        tile_of(rev ? ntiles - 1 - (q + NW) : q + NW, In, Jn);
                        const int c = 32 * (j0 + Jn) + lane;
                        if (c < n) prefetch_l2(A + (size_t)c * ld + 32 * (j0 + In));
                    }
                    const int I = j0 + Ii, J = j0 + Jj;
                    if (I == J || 32 * I + 32 > n) symv_tile<true>(A, ld, n, I, J, x, ywp, lane);
                    else symv_tile<false>(A, ld, n, I, J, x, ywp, lane);
                }
            }
            mark(14);
            for (int dq = warp; dq < 2 * kk; dq += NW) {
                const float *col = dq < kk ? Wb + (size_t)dq * ld : A + (size_t)(p0 + dq - kk) * ld;
                float s = 0.f;
                float s2 = 0.f;            // two chains, four loads in flight per lane
                int r = k + 1 + lane;
                for (; r + 32 < n; r += 64) {
                    s = fmaf(col[r], x[r], s);
                    s2 = fmaf(col[r + 32], x[r + 32], s2);
                }
                if (r < n) s = fmaf(col[r], x[r], s);
                s += s2;
                s = warp_sum(s);
                if (lane == 0) {
                    if (dq < kk) t1[dq] = s;
                    else t2[dq - kk] = s;
                }
            }
            __syncthreads();
            mark(15);
            // (d) w = tau (y - V t1 - W t2), then w -= (tau/2)(w.v) v, into column kk of Wb.
            // When the next column is in this panel, the same pass over the panel's first kk
            // columns also applies them to column k+1 (its step (a): rows k+1.., held by the
            // threads that own those rows in step (b)), and the kk-th term v_k w_k[k+1] + w_k
            // (v_k[k+1] = 1) follows once w is final.
            const bool fuse = kk + 1 < nb;
            if (fuse) {
                if (tid < kk) {                     // row k+1 of the panel's V and W
                    sv[tid] = A[(size_t)(p0 + tid) * ld + k + 1];
                    sw[tid] = Wb[(size_t)tid * ld + k + 1];
                }
                __syncthreads();
            }
            float wr[RW], cr[RW];
            float dpart = 0.f;
            #pragma unroll
            for (int i = 0; i < RW; i++) {
                const int r = k + 1 + tid + i * NT;
                float w = 0.f, c = 0.f;
                if (r < n) {
                    float y = 0.f;
                    #pragma unroll
                    for (int ww = 0; ww < NW; ww++) y += ywall[(size_t)ww * n32 + r];
                    if (fuse) {
                        c = A[(size_t)(k + 1) * ld + r];
                        for (int jj = 0; jj < kk; jj++) {
                            const float vj = A[(size_t)(p0 + jj) * ld + r], wj = Wb[(size_t)jj * ld + r];
                            y -= vj * t1[jj] + wj * t2[jj];
                            c -= vj * sw[jj] + wj * sv[jj];
                        }
                    } else {
                        for (int jj = 0; jj < kk; jj++)
                            y -= A[(size_t)(p0 + jj) * ld + r] * t1[jj] + Wb[(size_t)jj * ld + r] * t2[jj];
                    }
                    w = tk * y;
                    dpart += w * x[r];
                }
                wr[i] = w;
                cr[i] = c;
            }
            const float dot = block_sum<NT>(dpart, red);
            const float half = -0.5f * tk * dot;
            #pragma unroll
            for (int i = 0; i < RW; i++) {
                const int r = k + 1 + tid + i * NT;
                if (r < n) {
                    wr[i] += half * x[r];
                    Wb[(size_t)kk * ld + r] = wr[i];
                    if (r == k + 1) red[50] = wr[i];
                }
            }
            if (fuse) {
                __syncthreads();                   // w_k[k+1] in red[50]
                const float wk1 = red[50];
                float part = 0.f;
                #pragma unroll
                for (int i = 0; i < RW; i++) {
                    const int r = k + 1 + tid + i * NT;
                    if (r < n) {
                        const float c = cr[i] - x[r] * wk1 - wr[i];
                        if (r == k + 1) d[k + 1] = c;
                        else if (r == k + 2) red[48] = c;
                        else { x[r] = c; part += c * c; }
                    }
                }
                xn2 = block_sum<NT>(part, red);
            }
            __syncthreads();
            mark(16);
        }
        // (e) the trailing block beyond the panel
        trail_update<NT>(A, Wb, n, ld, p0, nb, ywall);
        __syncthreads();
        mark(17);
    }
    if (tid == 0) {
        d[n - 2] = A[(size_t)(n - 2) * ld + n - 2];
        e[n - 2] = A[(size_t)(n - 2) * ld + n - 1];
        d[n - 1] = A[(size_t)(n - 1) * ld + n - 1];
        tau[n - 2] = 0.f;
        e[n - 1] = 0.f;
    }
    __syncthreads();
}

// Phase 1 of matrix `mat` of a (the body of k_eigh_tq and of k_eigh_tq_multi).
template <int NT, int NMAX, bool BLK>
__device__ __forceinline__ void tq_body(const EighArgs &a, int mat) {
    constexpr int QG = (NMAX + 4 * NT - 1) / (4 * NT); // 4-row groups per thread, phase 1
    constexpr int NW = NT / 32;
    extern __shared__ __align__(16) float smem[];
    const int n = a.n, ld = a.ld;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    float *A = a.A + (size_t)mat * a.mstride;
    float *Z = a.Z + (size_t)mat * (a.zstride ? a.zstride : a.mstride);

    const int n4 = (n + 3) & ~3;
    float *d = smem;             // [n4]
    float *e = d + n4;           // [n4]
    float *tau = e + n4;         // [n4]
    float *U = tau + n4;         // union region (tq_union_floats)
    float *red = U + tq_union_floats(n, NT, BLK);   // [64]

    unsigned long long *pt = a.phase_ns ? a.phase_ns + (size_t)mat * CIR_EIG_PROF_SLOTS : nullptr;
    if (pt && tid == 0) pt[0] = globaltimer_ns();
    if (a.status && tid == 0) a.status[mat] = 0;
    // ---------------- phase 1: tridiagonalisation ----------------
    if constexpr (BLK) {
        // W of the current panel lives in Z, which phase 2 overwrites
        const int n32 = (n + 31) & ~31;
        const int yws = max(n32 * NW, 2 * tb_stage(NT));
        tridiag_blocked<NT, NMAX>(A, Z, n, ld, d, e, tau, U, U + n32, U + n32 + yws, red, pt, a.tq_order);
    } else {
        float *vp = U, *wp = U + n4, *vc = U + 2 * n4, *wc = U + 3 * n4;
        // the first column reads vp / wp (scaled by zero) before any update has written them:
        // clear them, since 0 * (a NaN or infinity left in shared memory) is NaN
        for (int i = tid; i < 4 * n4; i += NT) U[i] = 0.f;
        __syncthreads();
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

    // d, e and tau for the next two kernels
    float *de = a.DE + (size_t)mat * 3 * ld;
    for (int i = tid; i < n; i += NT) {
        de[i] = d[i];
        de[ld + i] = e[i];
        de[2 * ld + i] = tau[i];
    }
    if (pt) {
        __syncthreads();
        if (tid == 0) pt[1] = globaltimer_ns();
    }
}

template <int NT, int NMAX, int MINB, bool BLK>
__global__ void __launch_bounds__(NT, MINB) k_eigh_tq(EighArgs a) {
    tq_body<NT, NMAX, BLK>(a, blockIdx.x);
}

// Several batches of the blocked form in one launch (orders 257-1024, the order-1024
// instantiation for all): problem p covers blocks start[p] .. start[p+1]-1, the problems in
// descending order, so that the longest matrices start first and the shorter ones fill
// the last wave.
struct TqPlan {
    EighArgs a[CIR_TQ_MAXP];
    int start[CIR_TQ_MAXP + 1];
    int np;
};

template <int NT, int NMAX, int MINB>
__global__ void __launch_bounds__(NT, MINB) k_eigh_tq_multi(const __grid_constant__ TqPlan plan) {
    int p = 0;
    while (p + 1 < plan.np && (int)blockIdx.x >= plan.start[p + 1]) p++;
    tq_body<NT, NMAX, true>(plan.a[p], (int)blockIdx.x - plan.start[p]);
}

// Sum NV per-lane values over the warp by halving exchanges (lane bit 4 first): lane L ends
// with the warp sum of value xr_index<NV>(L), held by the 32/NV lanes that share it.
template <int NV>
__device__ __forceinline__ float xreduce(float (&y)[NV], int lane) {
    constexpr int LG = NV == 32 ? 5 : NV == 16 ? 4 : NV == 8 ? 3 : NV == 4 ? 2 : NV == 2 ? 1 : 0;
    #pragma unroll
    for (int L = 0; L < LG; L++) {
        const int o = 16 >> L, h = NV >> (L + 1);
        const bool up = lane & o;
        #pragma unroll
        for (int i = 0; i < h; i++) {
            const float send = up ? y[i] : y[i + h], keep = up ? y[i + h] : y[i];
            y[i] = keep + __shfl_xor_sync(0xffffffffu, send, o);
        }
    }
    #pragma unroll
    for (int L = LG; L < 5; L++) y[0] += __shfl_xor_sync(0xffffffffu, y[0], 16 >> L);
    return y[0];
}

template <int NV>
__device__ __forceinline__ int xr_index(int lane) {
    int idx = 0;
    #pragma unroll
    for (int L = 0; (NV >> (L + 1)) >= 1; L++)
        if (lane & (16 >> L)) idx += NV >> (L + 1);
    return idx;
}

// Phase 2: Q = H_0 H_1 ... H_{n-3} into Z by backward accumulation, NBQ reflectors at a
// time in compact WY form (LAPACK slarft, forward, columnwise):
// H_kb ... H_kb+NBQ-1 = I - V T V^T, applied as Z <- Z - V (T (V^T Z)) to the trailing
// rows and columns.  Each warp owns interleaved 32-row chunks of the trailing rows and keeps
// their NBQ reflector values in registers for the whole block, so a column costs NBQ FMAs
// per element for V^T z and NBQ for the update with no shared-memory operand traffic; the
// NBQ partial dots per column are summed over lanes by exchanges and over warps through
// shared memory, CB columns at a time.  The next CB columns are copied into shared memory
// (cp.async, each lane its own elements, so a per-thread wait suffices) while the current
// ones are processed.  d, e, tau come from the tridiagonalisation kernel (DE rows 0-2).
template <int NT, int NMAX, int NBQ, int CB>
__host__ __device__ constexpr int fq_smem_floats() {
    constexpr int NW = NT / 32, S = (NMAX + 32 * NW - 1) / (32 * NW);
    return 2 * NW * CB * S * 32                                    // z double buffer
           + NW * CB * NBQ + 2 * CB * NBQ + 2 * NBQ * NBQ + NBQ;
}


template <int NT, int NMAX, int NBQ, int CB, int MINB>
__global__ void __launch_bounds__(NT, MINB) k_eigh_formq(EighArgs a) {
    constexpr int NW = NT / 32;
    constexpr int S = (NMAX + 32 * NW - 1) / (32 * NW);   // row slots per lane
    extern __shared__ __align__(16) float fsm[];
    float *zb = fsm;                                 // [2][NW][CB][S][32]
    float *part = zb + 2 * NW * CB * S * 32;         // [NW][CB][NBQ] per-warp partial V^T z
    float *yfull = part + NW * CB * NBQ;             // [CB][NBQ] V^T z
    float *uu = yfull + CB * NBQ;                    // [CB][NBQ] T V^T z
    float *Gm = uu + CB * NBQ;                       // [NBQ][NBQ] V^T V (strict upper part)
    float *Tm = Gm + NBQ * NBQ;                      // [NBQ][NBQ]
    float *taus = Tm + NBQ * NBQ;                    // [NBQ]
    const int n = a.n, ld = a.ld;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const float *A = a.A + (size_t)blockIdx.x * a.mstride;
    float *Z = a.Z + (size_t)blockIdx.x * a.mstride;
    const float *tau_g = a.DE + (size_t)blockIdx.x * 3 * ld + 2 * ld;
    unsigned long long *pt = a.phase_ns ? a.phase_ns + (size_t)blockIdx.x * CIR_EIG_PROF_SLOTS : nullptr;
    if (pt && tid == 0) pt[2] = globaltimer_ns();
    for (size_t idx = tid; idx < (size_t)n * ld; idx += NT) {
        const int j = (int)(idx / ld), i = (int)(idx % ld);
        Z[idx] = (i == j) ? 1.f : 0.f;
    }
    __syncthreads();
    const int nrefl = n - 2;
    const int myidx = xr_index<NBQ>(lane);
    const bool writer = (lane & ((32 / NBQ) - 1)) == 0;
    float *zw = zb + (size_t)warp * CB * S * 32 + lane;   // this lane's slots: zw[buf*NW*CB*S*32 + (cc*S + t)*32]
    for (int kb = nrefl > 0 ? ((nrefl - 1) / NBQ) * NBQ : -1; kb >= 0; kb -= NBQ) {
        const int nb = min(NBQ, nrefl - kb);
        const int r0 = kb + 1, m = n - r0;
        // copy one batch of CB columns (this lane's rows) into buffer bf
        auto fetch = [&](int c0, int bf) {
            float *dst = zw + (size_t)bf * NW * CB * S * 32;
            #pragma unroll
            for (int cc = 0; cc < CB; cc++) {
                const int j = c0 + cc;
                #pragma unroll
                for (int t = 0; t < S; t++) {
                    const int rho = lane + 32 * (warp + NW * t);
                    const bool ok = j < n && rho < m;
                    cp_async4(dst + (cc * S + t) * 32, ok ? Z + (size_t)j * ld + r0 + rho : Z, ok);
                }
            }
            cp_async_commit();
        };
        fetch(r0, 0);
        // this warp's rows of V: row r0 + rho, rho = lane + 32 (warp + NW t)
        float vr[S][NBQ];
        #pragma unroll
        for (int t = 0; t < S; t++) {
            const int rho = lane + 32 * (warp + NW * t);
            const int r = r0 + rho;
            #pragma unroll
            for (int kk = 0; kk < NBQ; kk++) {
                const int k = kb + kk;
                float v = 0.f;
                if (kk < nb && rho < m) v = r < k + 1 ? 0.f : (r == k + 1 ? 1.f : A[(size_t)k * ld + r]);
                vr[t][kk] = v;
            }
        }
        // V^T V: G[l][j] = A[l'][j'+1] + sum_{r >= j'+2} A[l'][r] A[j'][r] (l < j, primes: +kb)
        for (int pq = warp; pq < NBQ * (NBQ - 1) / 2; pq += NW) {
            int l = 0, j = pq;
            while (j >= NBQ - 1 - l) { j -= NBQ - 1 - l; l++; }
            j += l + 1;
            float g = 0.f;
            if (j < nb) {
                const float *cl = A + (size_t)(kb + l) * ld, *cj = A + (size_t)(kb + j) * ld;
                for (int r = kb + j + 2 + lane; r < n; r += 32) g += cl[r] * cj[r];
                g = warp_sum(g);
                g += cl[kb + j + 1];
            }
            if (lane == 0) Gm[l * NBQ + j] = g;
        }
        if (tid < NBQ) taus[tid] = tid < nb ? tau_g[kb + tid] : 0.f;
        __syncthreads();
        if (warp == 0 && lane < NBQ) {
            // row i = lane of T: T[i][i] = tau_i, T[i][j] = -tau_j sum_{l=i}^{j-1} T[i][l] G[l][j]
            const int i = lane;
            for (int j = 0; j < NBQ; j++) {
                float t = 0.f;
                if (j == i) t = taus[i];
                else if (j > i) {
                    float acc = 0.f;
                    for (int l = i; l < j; l++) acc += Tm[i * NBQ + l] * Gm[l * NBQ + j];
                    t = -taus[j] * acc;
                }
                Tm[i * NBQ + j] = t;
            }
        }
        __syncthreads();
        int bf = 0;
        for (int c0 = r0; c0 < n; c0 += CB, bf ^= 1) {
            if (c0 + CB < n) {
                fetch(c0 + CB, bf ^ 1);
                cp_async_wait<1>();
            } else {
                cp_async_wait<0>();
            }
            const float *zc = zw + (size_t)bf * NW * CB * S * 32;
            // V^T z for CB columns: this warp's partial sums
            #pragma unroll 1
            for (int cc = 0; cc < CB; cc++) {
                float y[NBQ];
                #pragma unroll
                for (int kk = 0; kk < NBQ; kk++) y[kk] = 0.f;
                #pragma unroll
                for (int t = 0; t < S; t++) {
                    const float z = zc[(cc * S + t) * 32];
                    #pragma unroll
                    for (int kk = 0; kk < NBQ; kk++) y[kk] = fmaf(vr[t][kk], z, y[kk]);
                }
                const float ys = xreduce<NBQ>(y, lane);
                if (writer) part[(warp * CB + cc) * NBQ + myidx] = ys;
            }
            __syncthreads();
            for (int q = tid; q < CB * NBQ; q += NT) {
                float sacc = 0.f;
                #pragma unroll
                for (int w = 0; w < NW; w++) sacc += part[w * CB * NBQ + q];
                yfull[q] = sacc;
            }
            __syncthreads();
            for (int q = tid; q < CB * NBQ; q += NT) {
                const int cc = q / NBQ, i = q - cc * NBQ;
                float sacc = 0.f;
                for (int jj = i; jj < NBQ; jj++) sacc += Tm[i * NBQ + jj] * yfull[cc * NBQ + jj];
                uu[q] = sacc;
            }
            __syncthreads();
            // z -= V u
            #pragma unroll 1
            for (int cc = 0; cc < CB; cc++) {
                const int j = c0 + cc;
                if (j >= n) break;
                float u[NBQ];
                #pragma unroll
                for (int kk = 0; kk < NBQ; kk++) u[kk] = uu[cc * NBQ + kk];
                float *col = Z + (size_t)j * ld + r0;
                #pragma unroll
                for (int t = 0; t < S; t++) {
                    const int rho = lane + 32 * (warp + NW * t);
                    if (rho < m) {
                        float zz = zc[(cc * S + t) * 32];
                        #pragma unroll
                        for (int kk = 0; kk < NBQ; kk++) zz = fmaf(-vr[t][kk], u[kk], zz);
                        col[rho] = zz;
                    }
                }
            }
        }
        __syncthreads();
    }
    if (pt) {
        __syncthreads();
        if (tid == 0) pt[3] = globaltimer_ns();
    }
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
    unsigned long long *pt = a.phase_ns ? a.phase_ns + (size_t)blockIdx.x * CIR_EIG_PROF_SLOTS : nullptr;
    if (pt && tid == 0) pt[4] = globaltimer_ns();
    for (int i = tid; i < n; i += NT) {
        d[i] = a.DE[(size_t)blockIdx.x * 3 * ld + i];
        e[i] = a.DE[(size_t)blockIdx.x * 3 * ld + ld + i];
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
        ch.timed = pt != nullptr;
        ch.t_search = 0;
        ch.l = -1;
        ch.js = -1;
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
                    apply_group<R>(Z, ld, row, rb, T0, T1, cmin, cmax, smem + qr_ring_offset_floats(n) + t, napp);
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
        if (pt && tid == 0) {
            pt[7] = t_chase;
            pt[9] = (unsigned long long)ch.nrot;
            pt[10] = ch.t_search;
            pt[11] = (unsigned long long)ch.nsweep;
        }
        if (pt && tid == 32) pt[8] = t_apply;
        if (tid == 0) {
            if (a.status) a.status[blockIdx.x] = ch.status;
            if (a.sweeps) atomicAdd(a.sweeps, (unsigned long long)ch.nsweep);
        }
        __syncthreads();
    }

    if (pt && tid == 0) pt[5] = globaltimer_ns();
    // ---------------- phase 4: ascending order, output, frequency distribution ----------------
    {
        int *rank = reinterpret_cast<int *>(U);
        for (int j = tid; j < n; j += NT) {
            const float dj = d[j];
            int r = 0;
            for (int i = 0; i < n; i++) {
                r += cir_before(d[i], i, dj, j);
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
                    const size_t grp = a.hist_group > 0 ? (size_t)(blockIdx.x / a.hist_group) : 0;
                    const int wgt = a.hist_weight ? a.hist_weight[blockIdx.x] : 1;
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
    }
    if (pt) {
        __syncthreads();
        if (tid == 0) pt[6] = globaltimer_ns();
    }
}

// MINB: resident blocks per SM the register budget is fitted to (3 while the spill stays
// negligible; the order-2048 variant is fitted to 2 blocks).
template <int NT, int NMAX, int MINB, bool BLK>
cudaError_t launch_tq(const EighArgs &a, int nmat, cudaStream_t s) {
    auto kern = k_eigh_tq<NT, NMAX, MINB, BLK>;
    const size_t smem = tq_smem_bytes(a.n, NT, BLK);
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    static const int order = [] {
        const char *v = getenv("CIR_TQ_ORDER");
        return v ? atoi(v) : 1;
    }();
    EighArgs b = a;
    b.tq_order = order;
    size_t req = smem;
    if (a.tq_blocks > 0 && a.tq_blocks < MINB) {
        // fewer blocks per SM: ask for enough shared memory that only tq_blocks fit
        int dev = 0, per_sm = 0, reserved = 0;
        if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
        if ((e = cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev)) != cudaSuccess ||
            (e = cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev)) != cudaSuccess)
            return e;
        const size_t want = (size_t)per_sm / (a.tq_blocks + 1) - (size_t)reserved + 1024;
        if (want > req) req = want;
        if ((e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)req)) != cudaSuccess)
            return e;
    }
    kern<<<nmat, NT, req, s>>>(b);
    return cudaGetLastError();
}

template <int NT, int NMAX, int NBQ, int CB, int MINB>
cudaError_t launch_formq(const EighArgs &a, int nmat, cudaStream_t s) {
    auto kern = k_eigh_formq<NT, NMAX, NBQ, CB, MINB>;
    const size_t smem = sizeof(float) * fq_smem_floats<NT, NMAX, NBQ, CB>();
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<nmat, NT, smem, s>>>(a);
    return cudaGetLastError();
}

constexpr int QR_THREADS = 128;
constexpr int QR_ROWS = 3;   // rows per applying thread; 3 blocks per SM without spills

cudaError_t launch_qr(const EighArgs &a, int nmat, cudaStream_t s) {
    auto kern = k_eigh_qr<QR_THREADS, QR_ROWS>;
    const size_t smem = qr_smem_bytes(a.n, QR_THREADS, QR_ROWS);
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<nmat, QR_THREADS, smem, s>>>(a);
    return cudaGetLastError();
}

}  // namespace

size_t cir_eigh_rot_bytes(int n) { return sizeof(float2) * 2 * EIG_KS * (size_t)(n + EIG_KS); }

size_t cir_eigh_de_bytes(int ld) { return sizeof(float) * 3 * (size_t)ld; }

int cir_eigh_max_n() { return 2048; }

int cir_tridiag_blocks(int n) { return n <= 256 ? 4 : (n <= 1024 ? 3 : 2); }

size_t cir_tridiag_w_floats(int ld) { return (size_t)TB_NB * ld; }

cudaError_t cir_launch_tridiag_multi(const EighArgs *a, const int *nmat, int np, cudaStream_t s, int *launches) {
    if (np < 1 || np > CIR_TQ_MAXP) return cudaErrorInvalidValue;
    int order[CIR_TQ_MAXP];
    for (int i = 0; i < np; i++) {
        const EighArgs &x = a[i];
        if (x.n <= 256 || x.n > 1024 || nmat[i] < 1 || nmat[i] > 65535 || (x.ld & 3) || x.ld < x.n || !x.DE ||
            (reinterpret_cast<uintptr_t>(x.A) & 15) || (reinterpret_cast<uintptr_t>(x.Z) & 15))
            return cudaErrorInvalidValue;
        order[i] = i;
    }
    std::sort(order, order + np, [&](int x, int y) { return a[x].n > a[y].n; });
    static const int tq_order = [] {
        const char *v = getenv("CIR_TQ_ORDER");
        return v ? atoi(v) : 1;
    }();
    TqPlan plan;
    memset(&plan, 0, sizeof plan);
    plan.np = np;
    size_t smem = 0;
    int total = 0;
    for (int k = 0; k < np; k++) {
        plan.a[k] = a[order[k]];
        plan.a[k].tq_order = tq_order;
        plan.start[k] = total;
        total += nmat[order[k]];
        smem = std::max(smem, tq_smem_bytes(plan.a[k].n, 256, true));
    }
    plan.start[np] = total;
    auto kern = k_eigh_tq_multi<256, 1024, 3>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<total, 256, smem, s>>>(plan);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if (launches) *launches += 1;
    return cudaSuccess;
}

cudaError_t cir_launch_tridiag(const EighArgs &a, int nmat, cudaStream_t s) {
    if (a.n <= 256) return launch_tq<128, 256, 4, false>(a, nmat, s);
    if (a.n <= 512) return launch_tq<256, 512, 3, true>(a, nmat, s);
    if (a.n <= 1024) return launch_tq<256, 1024, 3, true>(a, nmat, s);
    return launch_tq<256, 2048, 2, true>(a, nmat, s);
}

cudaError_t cir_launch_eigh(const EighArgs &a, int nmat, cudaStream_t s, int *launches) {
    if (a.n < 1 || a.n > cir_eigh_max_n() || nmat < 1 || nmat > 65535 || (a.ld & 3) || a.ld < a.n)
        return cudaErrorInvalidValue;
    if ((reinterpret_cast<uintptr_t>(a.A) & 15) || (reinterpret_cast<uintptr_t>(a.Z) & 15) || !a.DE ||
        (!a.rot && !a.DC) || (a.DC && (reinterpret_cast<uintptr_t>(a.DC) & 15)))
        return cudaErrorInvalidValue;
    cudaError_t e = cudaSuccess;
    if (!a.skip_tridiag) {
        if ((e = cir_launch_tridiag(a, nmat, s)) != cudaSuccess) return e;
        if (launches) *launches += 1;
    }
    if (a.tq_done && (e = cudaEventRecord(a.tq_done, s)) != cudaSuccess) return e;
    // divide and conquer: the reflectors are applied to the tridiagonal eigenvectors at the end
    if (a.DC) return cir_launch_dc(a, nmat, s, launches);
    if (a.n <= 512) e = launch_formq<256, 512, 16, 8, 2>(a, nmat, s);
    else if (a.n <= 1024) e = launch_formq<256, 1024, 16, 8, 2>(a, nmat, s);
    else e = launch_formq<256, 2048, 8, 4, 2>(a, nmat, s);
    if (e != cudaSuccess) return e;
    if (launches) *launches += 1;
    e = launch_qr(a, nmat, s);
    if (launches) *launches += 1;
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

// scratch bytes of a call on nmat matrices of order n (pad: A is copied to a 16-byte
// aligned, ld-strided buffer first)
size_t noalloc_need(int nmat, int n, bool pad) {
    const int ld = (n + 3) & ~3;
    const size_t mat = (size_t)n * ld * sizeof(float);
    return align256(nmat * mat)                                   // Z
           + align256(nmat * cir_eigh_rot_bytes(n))               // rotation groups
           + align256(nmat * cir_eigh_de_bytes(ld))               // d, e, tau
           + align256((size_t)nmat * sizeof(int))                 // status
           + (pad ? align256(nmat * mat) : 0);                    // 16-byte aligned copy of A
}

// the largest order one call can take: a single matrix, with the aligned copy (pad) or
// without it (then n is a multiple of 4)
int noalloc_max_order(bool pad) {
    int n = cir_eigh_max_n();
    while (n > 1 && ((!pad && (n & 3)) || noalloc_need(1, n, pad) > NOALLOC_SCRATCH_BYTES)) n--;
    return n;
}

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
    const size_t need = noalloc_need(nmat, n, pad);
    if (noalloc_need(1, n, pad) > NOALLOC_SCRATCH_BYTES)
        return cir_fail(CIR_ERR_ARG,
                        "cir_eigh_noalloc: order %d needs %zu bytes of scratch for one matrix; the allocation-free "
                        "scratch holds %zu bytes, enough for orders up to %d (%d when n is not a multiple of 4 or "
                        "A is not 16-byte aligned)",
                        n, noalloc_need(1, n, pad), NOALLOC_SCRATCH_BYTES, noalloc_max_order(false),
                        noalloc_max_order(true));
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
