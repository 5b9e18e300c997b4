// FP64 refinement of a batch of eigendecompositions: Rayleigh quotients for the eigenvalues,
// a first-order correction and re-orthogonalisation of the eigenvectors, after T. Ogita and
// K. Aishima, "Iterative refinement for symmetric eigenvalue decomposition", Japan J. Indust.
// Appl. Math. 35 (2018) 1007-1035 (Algorithm 1, RefSyEv).  Clusters of close eigenvalues (the
// subject of their sequel, "... II: clustered eigenvalues", ibid. 36 (2019) 435-459) are
// separated here by Rayleigh-Ritz on each cluster.  The reference takes magma_ssyevd's FP32 eigenpairs as they are
// (calcIR.cu:420-448); this is an opt-in step on top of the FP32 / split-BF16 eigensolver that
// takes the eigenpairs of the FP32 Hamiltonian to the accuracy that FP32 storage allows.
//
// With X the approximate eigenvectors (columns) of the symmetric A:
//     G = X^T X,  S = X^T A X                 (FP64 accumulation of exact FP32 products)
//     lambda_j = s_jj / g_jj                    (Rayleigh quotient)
//     E_kj = (s_kj - lambda_j g_kj) / (lambda_j - lambda_k)     (k != j)
//     E_jj = (1 - g_jj) / 2,   X <- X + X E
// squares the eigenvector error of well-separated pairs.  A pair whose coefficient would
// exceed tau (1/64; 1/4096 when a single step is asked for, so that one step never leaves
// more than tau^2 of non-orthogonality) is close.  Clusters are the closure of the close
// relation over the eigenvalue ranks; each cluster of up to RF_KMAX is solved exactly
// (Loewdin orthonormalisation, then Jacobi on its projected matrix), and the first-order
// step runs in the basis rotated by the clusters' Ritz vectors (k_rf_coef).  Larger clusters
// are only re-orthogonalised.
//
// Storage: eigenvector j is row j of the matrix (A + j*ld), so with Z the row-major array
//     Y^T = Z A^T (A symmetric),  S = Z Y,  G = Z Z^T,  Z' = Z + E^T Z
// The three products of the form P Q^T take Z (and A) as FP32 and Y as FP64; S and G are
// symmetric, so only their upper tiles are formed.  The update writes row j of Z' to row
// rank(lambda_j), which keeps the eigenvalues ascending.
// GB300's FP64 rate is a small fraction of its FP32 and tensor rates: these are SIMT FP64
// products (3 n^3 multiply-adds per step with S and G at half), which is why the step is
// opt-in.
#include "cir_device.cuh"

#include <algorithm>

namespace {

constexpr int RF_T = 64;              // output tile
constexpr int RF_K = 16;              // k per stage
constexpr int RF_LDS = RF_T + 1;      // shared row stride in doubles (conflict-free transposed stores)
constexpr double RF_TAU = 1.0 / 64;         // close: first-order coefficient above this
constexpr double RF_TAU_ONE = 1.0 / 4096;    // ... when a single step is asked for
constexpr int RF_KMAX = 16;                  // largest cluster given Rayleigh-Ritz

struct RfGemm {
    const void *P;        // [batch] n x n, row-major, element (r, k) at P[r*ldp + k]
    long long sP;
    int ldp;
    const void *Q;        // QN: element (k, c) at Q[k*ldq + c]; else (k, c) at Q[c*ldq + k]
    long long sQ;
    int ldq;
    double *C;            // MODE 0: C[r*ldc + c]
    long long sC;
    int ldc;
    int n;
    int upper;            // MODE 0: form only the tiles on and above the diagonal
    const float *Z0;      // MODE 1: Zo[pos[r]*ldz + c] = Z0[r*ldz + c] + (P Q)[r][c]
    float *Zo;
    long long sZ0, sZ;    // batch strides of Z0 and Zo
    int ldz;
    const int *pos;
    int spos;
};

template <typename T>
__device__ __forceinline__ double ld64(const T *p, long long i) {
    return (double)p[i];
}

// 64 x 64 output tile per 256 threads; thread (tx, ty) = (t & 15, t >> 4) holds rows
// ty + 16 i and columns tx + 16 j (i, j < 4).  Operands are converted to FP64 when staged.
template <typename TP, typename TQ, bool QN, int MODE>
__global__ void __launch_bounds__(256) k_rf_gemm(RfGemm g) {
    if (MODE == 0 && g.upper && blockIdx.y > blockIdx.x) return;
    __shared__ double Ps[RF_K][RF_LDS], Qs[RF_K][RF_LDS];
    const int n = g.n, b = blockIdx.z;
    const int r0 = blockIdx.y * RF_T, c0 = blockIdx.x * RF_T;
    const int t = threadIdx.x, tx = t & 15, ty = t >> 4;
    const TP *P = static_cast<const TP *>(g.P) + (size_t)b * g.sP;
    const TQ *Q = static_cast<const TQ *>(g.Q) + (size_t)b * g.sQ;
    double acc[4][4];
    #pragma unroll
    for (int i = 0; i < 4; i++)
        #pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = 0.0;
    double pr[4], qr[4];
    // staging: P rows r0 + (t >> 4) + 16 i at k = t & 15 (16 threads read 16 consecutive k);
    // Q the same for Q^T, or k = (t >> 6) + 4 i at column c0 + (t & 63) for QN
    auto fetch = [&](int k0) {
        #pragma unroll
        for (int i = 0; i < 4; i++) {
            const int r = r0 + ty + 16 * i, k = k0 + tx;
            pr[i] = (r < n && k < n) ? ld64(P, (long long)r * g.ldp + k) : 0.0;
            if (QN) {
                const int kq = k0 + (t >> 6) + 4 * i, c = c0 + (t & 63);
                qr[i] = (kq < n && c < n) ? ld64(Q, (long long)kq * g.ldq + c) : 0.0;
            } else {
                const int c = c0 + ty + 16 * i;
                qr[i] = (c < n && k < n) ? ld64(Q, (long long)c * g.ldq + k) : 0.0;
            }
        }
    };
    fetch(0);
    for (int k0 = 0; k0 < n; k0 += RF_K) {
        __syncthreads();
        #pragma unroll
        for (int i = 0; i < 4; i++) {
            Ps[tx][ty + 16 * i] = pr[i];
            if (QN) Qs[(t >> 6) + 4 * i][t & 63] = qr[i];
            else Qs[tx][ty + 16 * i] = qr[i];
        }
        __syncthreads();
        if (k0 + RF_K < n) fetch(k0 + RF_K);
        #pragma unroll
        for (int kk = 0; kk < RF_K; kk++) {
            double a[4], q[4];
            #pragma unroll
            for (int i = 0; i < 4; i++) {
                a[i] = Ps[kk][ty + 16 * i];
                q[i] = Qs[kk][tx + 16 * i];
            }
            #pragma unroll
            for (int i = 0; i < 4; i++)
                #pragma unroll
                for (int j = 0; j < 4; j++) acc[i][j] = fma(a[i], q[j], acc[i][j]);
        }
    }
    #pragma unroll
    for (int i = 0; i < 4; i++) {
        const int r = r0 + ty + 16 * i;
        if (r >= n) continue;
        #pragma unroll
        for (int j = 0; j < 4; j++) {
            const int c = c0 + tx + 16 * j;
            if (c >= n) continue;
            if (MODE == 0) {
                g.C[(size_t)b * g.sC + (size_t)r * g.ldc + c] = acc[i][j];
            } else {
                const int pr_ = g.pos[(size_t)b * g.spos + r];
                g.Zo[(size_t)b * g.sZ + (size_t)pr_ * g.ldz + c] =
                    (float)((double)g.Z0[(size_t)b * g.sZ0 + (size_t)r * g.ldz + c] + acc[i][j]);
            }
        }
    }
}

// Rayleigh quotients lambda_j = s_jj / g_jj.
__global__ void k_rf_lambda(const double *S, const double *G, long long sM, int n, double *lam) {
    const int b = blockIdx.y, j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const size_t d = (size_t)b * sM + (size_t)j * n + j;
    lam[(size_t)b * n + j] = S[d] / G[d];
}

// Symmetric entry (j, k) of S or G, formed in the upper triangle only.
__device__ __forceinline__ double rf_sym(const double *M, int n, int j, int k) {
    return M[(size_t)min(j, k) * n + max(j, k)];
}

// A pair (j, k) is close when its first-order coefficient would exceed tau (symmetric in j, k).
__device__ __forceinline__ bool rf_close(double s, double g, double lj, double lk, double tau) {
    return !(fabs(lj - lk) * tau > fabs(s) + fmax(fabs(lj), fabs(lk)) * fabs(g));
}

__device__ __forceinline__ int rf_block_sum(int a) {
    __shared__ int red_i[8];
    for (int o = 16; o; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    if ((threadIdx.x & 31) == 0) red_i[threadIdx.x >> 5] = a;
    __syncthreads();
    a = 0;
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) a += red_i[i];
    return a;
}

__device__ __forceinline__ double rf_block_sum_d(double a) {
    __shared__ double red_d[8];
    a = warp_sum_d(a);
    if ((threadIdx.x & 31) == 0) red_d[threadIdx.x >> 5] = a;
    __syncthreads();
    a = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) a += red_d[i];
    return a;
}

// Rank of the Rayleigh quotient lambda_j (ties by index, NaN last) into pos[j], and inv[rank] = j.
__global__ void __launch_bounds__(256) k_rf_rank(const double *lam, int n, int *pos, int *inv) {
    const int j = blockIdx.x, b = blockIdx.y;
    const double *lb = lam + (size_t)b * n;
    const double lj = lb[j];
    int below = 0;
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const double lk = lb[k];
        below += cir_before(lk, k, lj, j) ? 1 : 0;
    }
    below = rf_block_sum(below);
    if (threadIdx.x == 0) {
        pos[(size_t)b * n + j] = below;
        inv[(size_t)b * n + below] = j;
    }
}

__device__ __forceinline__ int rf_block_max(int a) {
    __shared__ int red_m[8];
    for (int o = 16; o; o >>= 1) a = max(a, __shfl_xor_sync(0xffffffffu, a, o));
    if ((threadIdx.x & 31) == 0) red_m[threadIdx.x >> 5] = a;
    __syncthreads();
    a = -1;
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) a = max(a, red_m[i]);
    return a;
}

// The highest rank among row j's close partners (at least j's own rank) into reach[pos[j]].
__global__ void __launch_bounds__(256) k_rf_reach(const double *S, const double *G, long long sM, int n,
                                                  const double *lam, const int *pos, int *reach, double tau) {
    const int j = blockIdx.x, b = blockIdx.y;
    const size_t o = (size_t)b * n;
    const double *Sb = S + (size_t)b * sM, *Gb = G + (size_t)b * sM;
    const double lj = lam[o + j];
    int hi = pos[o + j];
    for (int k = threadIdx.x; k < n; k += blockDim.x)
        if (k != j && rf_close(rf_sym(Sb, n, j, k), rf_sym(Gb, n, j, k), lj, lam[o + k], tau)) hi = max(hi, pos[o + k]);
    hi = rf_block_max(hi);
    if (threadIdx.x == 0) reach[o + pos[o + j]] = hi;
}

// Clusters: the closure of the close relation over ranks -- a close pair at ranks r1 < r2
// joins every rank between them.  For rank u, cst[u] is its cluster's first rank and csz[u]
// the cluster's size.  One thread per matrix (a scan over n ranks).
__global__ void k_rf_runs(const int *reach, int n, int nmat, int *cst, int *csz) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nmat) return;
    const size_t o = (size_t)b * n;
    int start = 0, far = -1;
    for (int u = 0; u < n; u++) {
        far = max(far, reach[o + u]);
        cst[o + u] = start;
        if (far <= u) {                 // no close pair crosses from u to u + 1
            for (int v = start; v <= u; v++) csz[o + v] = u - start + 1;
            start = u + 1;
        }
    }
}

// Rayleigh-Ritz on every cluster of 2..RF_KMAX ranks (one warp per rank; the warp at a
// cluster's first rank does the work, lane r holding row / column r): G_c and S_c, the
// cluster's entries of G and S; first-order Loewdin orthonormalisation W = I + (I - G_c)/2;
// cyclic Jacobi on W S_c W (Golub and Van Loan, sym.schur2 rotations, |angle| <= pi/4) to J;
// eigenvalues in ascending order.  The new vector at rank u + a is
// sum_b (W J)[b][a] x_{inv[u + b]}: its coefficients go to mco[j][0..size) and its
// eigenvalue to lam2[j], j = inv[u + a].  Every other row keeps lam2[j] = lambda_j.
__global__ void __launch_bounds__(32) k_rf_rr(const double *S, const double *G, long long sM, int n,
                                              const double *lam, const int *inv, const int *cst, const int *csz,
                                              double *lam2, double *mco) {
    constexpr int L = RF_KMAX + 1;
    __shared__ double W[RF_KMAX][L], T[RF_KMAX][L], J[RF_KMAX][L];
    __shared__ int m[RF_KMAX], ord[RF_KMAX];
    const int b = blockIdx.y, u = blockIdx.x, lane = threadIdx.x;
    const size_t o = (size_t)b * n;
    const int sz = csz[o + u];
    if (sz < 2 || sz > RF_KMAX) {
        if (lane == 0) lam2[o + inv[o + u]] = lam[o + inv[o + u]];
        return;
    }
    if (cst[o + u] != u) return;
    const double *Sb = S + (size_t)b * sM, *Gb = G + (size_t)b * sM;
    const bool act = lane < sz;
    if (act) m[lane] = inv[o + u + lane];
    __syncwarp();
    if (act)
        for (int c = 0; c < sz; c++) {
            W[lane][c] = (lane == c ? 1.5 : 0.0) - 0.5 * rf_sym(Gb, n, m[lane], m[c]);
            J[lane][c] = lane == c ? 1.0 : 0.0;
        }
    __syncwarp();
    double row[RF_KMAX];                       // row `lane` of S_c W
    if (act)
        for (int c = 0; c < sz; c++) {
            double t = 0.0;
            for (int d = 0; d < sz; d++) t += rf_sym(Sb, n, m[lane], m[d]) * W[d][c];
            row[c] = t;
        }
    if (act)
        for (int c = 0; c < sz; c++) T[lane][c] = row[c];
    __syncwarp();
    if (act)                                   // row `lane` of W (S_c W)
        for (int c = 0; c < sz; c++) {
            double t = 0.0;
            for (int d = 0; d < sz; d++) t += W[lane][d] * T[d][c];
            row[c] = t;
        }
    __syncwarp();
    if (act)
        for (int c = 0; c < sz; c++) T[lane][c] = row[c];
    __syncwarp();
    if (act)                                   // exact symmetry
        for (int c = 0; c < lane; c++) {
            const double t = 0.5 * (T[lane][c] + T[c][lane]);
            row[c] = t;
        }
    __syncwarp();
    if (act)
        for (int c = 0; c < lane; c++) T[lane][c] = T[c][lane] = row[c];
    __syncwarp();
    for (int sweep = 0; sweep < 30; sweep++) {
        double off = 0.0, dia = 0.0;
        if (act) {
            dia = T[lane][lane] * T[lane][lane];
            for (int c = lane + 1; c < sz; c++) off += T[lane][c] * T[lane][c];
        }
        off = warp_sum_d(off);
        dia = warp_sum_d(dia);
        if (!(off > 1e-34 * dia)) break;
        for (int p = 0; p < sz - 1; p++)
            for (int q = p + 1; q < sz; q++) {
                const double tpq = T[p][q];
                if (tpq == 0.0) continue;
                const double z = (T[q][q] - T[p][p]) / (2.0 * tpq);
                const double t = (z >= 0.0 ? 1.0 : -1.0) / (fabs(z) + sqrt(1.0 + z * z));
                const double c = 1.0 / sqrt(1.0 + t * t), s = t * c;
                __syncwarp();
                if (act) {                     // columns p, q of T and of J
                    const double x = T[lane][p], y = T[lane][q];
                    T[lane][p] = c * x - s * y;
                    T[lane][q] = s * x + c * y;
                    const double xj = J[lane][p], yj = J[lane][q];
                    J[lane][p] = c * xj - s * yj;
                    J[lane][q] = s * xj + c * yj;
                }
                __syncwarp();
                if (act) {                     // rows p, q of T
                    const double x = T[p][lane], y = T[q][lane];
                    T[p][lane] = c * x - s * y;
                    T[q][lane] = s * x + c * y;
                }
                __syncwarp();
            }
    }
    if (lane == 0) {                           // eigenvalues ascending
        for (int a = 0; a < sz; a++) ord[a] = a;
        for (int a = 0; a < sz; a++)
            for (int c = a + 1; c < sz; c++)
                if (T[ord[c]][ord[c]] < T[ord[a]][ord[a]]) {
                    const int x = ord[a];
                    ord[a] = ord[c];
                    ord[c] = x;
                }
    }
    __syncwarp();
    if (act) {                                 // lane a: the vector at rank u + a
        const int j = m[lane], col = ord[lane];
        lam2[o + j] = T[col][col];
        for (int c = 0; c < sz; c++) {
            double t = 0.0;
            for (int d = 0; d < sz; d++) t += W[c][d] * J[d][col];
            mco[(o + j) * RF_KMAX + c] = t;
        }
    }
}

// Coefficients of the new vector x_j' in the old basis, row j of E^T (one block per row and
// matrix), and lam2[j] (as FP32) into w[rank j].  The step runs in the basis rotated by the
// clusters' Rayleigh-Ritz vectors, X M (M block diagonal: W J per cluster, the 1 x 1 Loewdin
// factor 1.5 - g_jj / 2 for every other row), so that a cluster and the rows around it see
// the same vectors:
//   s~_ca = sum_{b in c} M_bc t_b,  t_b = sum_{d in a} M_da s_bd  (and the same for g)
//   e~_ca = (s~_ca - lam2_a g~_ca) / (lam2_a - lam2_c)      c outside a's cluster
//         = -g~_ca / 2                                     c close to a, or in a cluster too
//                                                          large for Rayleigh-Ritz
//         = 0                                              c in a's cluster
//   x_j' = sigma_a X M (e_a + e~_a),  sigma_a = 1 - sum_c e~_ca^2 / 2  (the second-order term
//          that keeps x_j' at unit length)
// so E^T[j][k] = sum_{c in k's cluster} M_kc sigma_a (delta_ca + e~_ca) - delta_jk.
// Shared memory: t (for s and g) and e~, 3 n doubles.
__device__ __forceinline__ int rf_cluster(const int *pos, const int *cst, const int *csz, size_t o, int j, int &u0) {
    const int r = pos[o + j];
    u0 = cst[o + r];
    return csz[o + r];
}

__global__ void __launch_bounds__(256) k_rf_coef(const double *S, const double *G, long long sM, int n,
                                                 const double *lam2, const double *mco, const int *pos,
                                                 const int *inv, const int *cst, const int *csz, double *Et, float *w,
                                                 long long wstride, double tau) {
    extern __shared__ double rf_sm[];
    double *ts = rf_sm, *tg = rf_sm + n, *ee = rf_sm + 2 * n;
    __shared__ int mem[RF_KMAX];
    __shared__ double cf[RF_KMAX];
    const int j = blockIdx.x, b = blockIdx.y;
    const size_t o = (size_t)b * n;
    const double *Sb = S + (size_t)b * sM, *Gb = G + (size_t)b * sM;
    double *row = Et + (size_t)b * sM + (size_t)j * n;
    int u0;
    const int sz = rf_cluster(pos, cst, csz, o, j, u0);
    const bool rrj = sz >= 2 && sz <= RF_KMAX, ovj = sz > RF_KMAX;
    const int na = rrj ? sz : 1;
    if (threadIdx.x < na) {
        if (rrj) {
            mem[threadIdx.x] = inv[o + u0 + threadIdx.x];
            cf[threadIdx.x] = mco[(o + j) * RF_KMAX + threadIdx.x];
        } else {
            mem[0] = j;
            cf[0] = 1.5 - 0.5 * Gb[(size_t)j * n + j];
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        double s = 0.0, g = 0.0;
        for (int a = 0; a < na; a++) {
            s += cf[a] * rf_sym(Sb, n, mem[a], k);
            g += cf[a] * rf_sym(Gb, n, mem[a], k);
        }
        ts[k] = s;
        tg[k] = g;
    }
    __syncthreads();
    const double la = lam2[o + j];
    double sq = 0.0;
    for (int c = threadIdx.x; c < n; c += blockDim.x) {
        int uc;
        const int szc = rf_cluster(pos, cst, csz, o, c, uc);
        const bool same = uc == u0;
        double e = 0.0;
        if (c != j && !(same && rrj)) {
            double s, g;
            if (szc >= 2 && szc <= RF_KMAX) {
                s = 0.0;
                g = 0.0;
                const double *mc = mco + (o + c) * RF_KMAX;
                for (int d = 0; d < szc; d++) {
                    const int kd = inv[o + uc + d];
                    s += mc[d] * ts[kd];
                    g += mc[d] * tg[kd];
                }
            } else {
                const double m = 1.5 - 0.5 * Gb[(size_t)c * n + c];
                s = m * ts[c];
                g = m * tg[c];
            }
            const double lc = lam2[o + c];
            e = ((same && ovj) || rf_close(s, g, la, lc, tau)) ? -0.5 * g : (s - la * g) / (la - lc);
            sq += e * e;
        }
        ee[c] = e;
    }
    const double sig = 1.0 - 0.5 * rf_block_sum_d(sq);   // (its barrier also publishes ee)
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        int uk;
        const int szk = rf_cluster(pos, cst, csz, o, k, uk);
        double t;
        if (szk >= 2 && szk <= RF_KMAX) {
            const int lk = pos[o + k] - uk;
            t = 0.0;
            for (int d = 0; d < szk; d++) {
                const int c = inv[o + uk + d];
                t += mco[(o + c) * RF_KMAX + lk] * ((c == j ? 1.0 : 0.0) + ee[c]);
            }
        } else {
            t = (1.5 - 0.5 * Gb[(size_t)k * n + k]) * ((k == j ? 1.0 : 0.0) + ee[k]);
        }
        row[k] = sig * t - (k == j ? 1.0 : 0.0);
    }
    if (threadIdx.x == 0) w[(size_t)b * wstride + pos[o + j]] = (float)la;
}

template <typename TP, typename TQ, bool QN, int MODE>
cudaError_t rf_gemm(const RfGemm &g, int batch, cudaStream_t s) {
    const int tiles = (g.n + RF_T - 1) / RF_T;
    k_rf_gemm<TP, TQ, QN, MODE><<<dim3(tiles, tiles, batch), 256, 0, s>>>(g);
    return cudaGetLastError();
}

}  // namespace

// Per matrix: Y^T, S and G (n x n doubles each; E^T reuses Y^T's space), the Rayleigh
// quotients, the refined eigenvalues and the cluster coefficients ((2 + RF_KMAX) n doubles),
// a copy of the eigenvectors, and the ranks, their inverse, the reach of each rank and the
// clusters (5 n ints).
size_t cir_refine_bytes(int n, int ld) {
    return (size_t)3 * n * n * 8 + (size_t)(2 + RF_KMAX) * n * 8 + (size_t)n * ld * 4 + (size_t)5 * n * 4 + 64;
}

cudaError_t cir_launch_refine(const float *H, float *Z, long long mstride, int ld, int n, float *w, long long wstride,
                              int nmat, int iters, void *ws, int chunk, cudaStream_t s, int *launches) {
    if (!H || !Z || !w || !ws || n < 1 || ld < n || mstride < (long long)n * ld || chunk < 1 || nmat < 1 ||
        iters < 1 || chunk > 65535)
        return cudaErrorInvalidValue;
    const long long sM = (long long)n * n;
    const size_t smem = (size_t)3 * n * 8;
    cudaError_t e0 = cudaFuncSetAttribute(k_rf_coef, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e0 != cudaSuccess) return e0;
    int nl = 0;
    for (int m0 = 0; m0 < nmat; m0 += chunk) {
        const int c = std::min(chunk, nmat - m0);
        char *p = static_cast<char *>(ws);
        double *Y = reinterpret_cast<double *>(p);
        double *S = Y + (size_t)c * sM;
        double *G = S + (size_t)c * sM;
        double *lam = G + (size_t)c * sM;
        double *lam2 = lam + (size_t)c * n;
        double *mco = lam2 + (size_t)c * n;                      // RF_KMAX per row
        float *Z0 = reinterpret_cast<float *>(mco + (size_t)RF_KMAX * c * n);
        int *pos = reinterpret_cast<int *>(Z0 + (size_t)c * n * ld);
        int *inv = pos + (size_t)c * n, *cst = inv + (size_t)c * n, *csz = cst + (size_t)c * n;
        int *reach = csz + (size_t)c * n;
        const float *Hc = H + (size_t)m0 * mstride;
        float *Zc = Z + (size_t)m0 * mstride;
        float *wc = w + (size_t)m0 * wstride;
        for (int it = 0; it < iters; it++) {
            cudaError_t e;
            RfGemm g{};
            g.n = n;
            // Y^T = Z A^T
            g.P = Zc; g.sP = mstride; g.ldp = ld;
            g.Q = Hc; g.sQ = mstride; g.ldq = ld;
            g.C = Y; g.sC = sM; g.ldc = n;
            if ((e = rf_gemm<float, float, false, 0>(g, c, s)) != cudaSuccess) return e;
            // S = Z Y (upper tiles)
            g.Q = Y; g.sQ = sM; g.ldq = n;
            g.C = S; g.upper = 1;
            if ((e = rf_gemm<float, double, false, 0>(g, c, s)) != cudaSuccess) return e;
            // G = Z Z^T (upper tiles)
            g.Q = Zc; g.sQ = mstride; g.ldq = ld;
            g.C = G;
            if ((e = rf_gemm<float, float, false, 0>(g, c, s)) != cudaSuccess) return e;
            const double tau = iters == 1 ? RF_TAU_ONE : RF_TAU;
            k_rf_lambda<<<dim3((n + 255) / 256, c), 256, 0, s>>>(S, G, sM, n, lam);
            k_rf_rank<<<dim3(n, c), 256, 0, s>>>(lam, n, pos, inv);
            k_rf_reach<<<dim3(n, c), 256, 0, s>>>(S, G, sM, n, lam, pos, reach, tau);
            k_rf_runs<<<(c + 127) / 128, 128, 0, s>>>(reach, n, c, cst, csz);
            k_rf_rr<<<dim3(n, c), 32, 0, s>>>(S, G, sM, n, lam, inv, cst, csz, lam2, mco);
            k_rf_coef<<<dim3(n, c), 256, smem, s>>>(S, G, sM, n, lam2, mco, pos, inv, cst, csz, Y, wc, wstride, tau);
            if ((e = cudaGetLastError()) != cudaSuccess) return e;
            // Z' = Z + E^T Z, row j to row pos[j]
            const size_t zb = (size_t)n * ld * 4;
            if ((e = cudaMemcpy2DAsync(Z0, zb, Zc, (size_t)mstride * 4, zb, c, cudaMemcpyDeviceToDevice, s)) !=
                cudaSuccess)
                return e;
            RfGemm u{};
            u.n = n;
            u.P = Y; u.sP = sM; u.ldp = n;
            u.Q = Z0; u.sQ = (long long)n * ld; u.ldq = ld;
            u.Z0 = Z0; u.Zo = Zc; u.sZ0 = (long long)n * ld; u.sZ = mstride; u.ldz = ld;
            u.pos = pos; u.spos = n;
            if ((e = rf_gemm<double, float, true, 1>(u, c, s)) != cudaSuccess) return e;
            nl += 10;
        }
    }
    if (launches) *launches += nl;
    return cudaSuccess;
}
