// Batched FP32 SIMT GEMM for the propagation step of the plain form.
// The reference builds a dense diagonal propagator and multiplies three complex
// matrices per frame (Pinit + 3 x magma_cgemm, calcIR.cu:596-613, 24 N^3 real flops).
// Here the complex F is a real N x 2N matrix of interleaved (re, im) columns and one step
// is two real GEMMs, 8 N^3 flops:
//     G  = V^T F                  (epilogue: row j of G times exp(+i w_j dt/hbar))
//     F' = V G
// 128x128x8 or 64x64x16 block tiles, 256 threads, 8x8 or 4x4 outputs per thread,
// double-buffered shared memory; edges are predicated so any N works.
#include "cir_device.cuh"

namespace {

// Tile shapes (256 threads, a 16 x 16 thread grid, TM x TN outputs per thread in 4 x 4 groups
// 64 rows / columns apart): 128 x 128 x 8 for large products, 64 x 64 x 16 for products
// whose 128 x 128 grid would not fill the SMs.  The autotuner of the library picks one.
template <int BM_, int BN_, int BK_>
struct Tile {
    static constexpr int BM = BM_, BN = BN_, BK = BK_, TM = BM_ / 16, TN = BN_ / 16;
};
using TileL = Tile<128, 128, 8>;
using TileS = Tile<64, 64, 16>;
constexpr int GT = 256;

template <class T, bool ACOL>
__device__ __forceinline__ void load_a(const GemmArgs &g, const float *A, int m0, int k0, float (&ra)[4]) {
    const int t = threadIdx.x;
    if (ACOL) {   // element (i, k) at A[k*lda + i]; thread loads 4 consecutive i of one k
        const int kk = t / (T::BM / 4), i = (t % (T::BM / 4)) * 4;
        const int gk = k0 + kk, gi = m0 + i;
        const float *p = A + (size_t)gk * g.lda + gi;
        if (gk < g.K && gi + 3 < g.M && ((reinterpret_cast<uintptr_t>(p) & 15) == 0)) {
            const float4 v = *reinterpret_cast<const float4 *>(p);
            ra[0] = v.x; ra[1] = v.y; ra[2] = v.z; ra[3] = v.w;
        } else {
            #pragma unroll
            for (int q = 0; q < 4; q++) ra[q] = (gk < g.K && gi + q < g.M) ? p[q] : 0.f;
        }
    } else {      // element (i, k) at A[i*lda + k]; thread loads 4 consecutive k of one i
        const int i = t / (T::BK / 4), kk = (t % (T::BK / 4)) * 4;
        const int gi = m0 + i, gk = k0 + kk;
        const float *p = A + (size_t)gi * g.lda + gk;
        if (gi < g.M && gk + 3 < g.K && ((reinterpret_cast<uintptr_t>(p) & 15) == 0)) {
            const float4 v = *reinterpret_cast<const float4 *>(p);
            ra[0] = v.x; ra[1] = v.y; ra[2] = v.z; ra[3] = v.w;
        } else {
            #pragma unroll
            for (int q = 0; q < 4; q++) ra[q] = (gi < g.M && gk + q < g.K) ? p[q] : 0.f;
        }
    }
}

template <class T, bool ACOL>
__device__ __forceinline__ void store_a(float (*As)[T::BM], const float (&ra)[4]) {
    const int t = threadIdx.x;
    if (ACOL) {
        const int kk = t / (T::BM / 4), i = (t % (T::BM / 4)) * 4;
        *reinterpret_cast<float4 *>(&As[kk][i]) = make_float4(ra[0], ra[1], ra[2], ra[3]);
    } else {
        const int i = t / (T::BK / 4), kk = (t % (T::BK / 4)) * 4;
        #pragma unroll
        for (int q = 0; q < 4; q++) As[kk + q][i] = ra[q];
    }
}

template <class T, bool BKC>
__device__ __forceinline__ void load_b(const GemmArgs &g, const float *B, int k0, int n0, float (&rb)[4]) {
    const int t = threadIdx.x;
    if (BKC) {    // element (k, j) at B[j*ldb + k]; thread loads 4 consecutive k of one j
        const int j = t / (T::BK / 4), kk = (t % (T::BK / 4)) * 4;
        const int gj = n0 + j, gk = k0 + kk;
        const float *p = B + (size_t)gj * g.ldb + gk;
        if (gj < g.N && gk + 3 < g.K && ((reinterpret_cast<uintptr_t>(p) & 15) == 0)) {
            const float4 v = *reinterpret_cast<const float4 *>(p);
            rb[0] = v.x; rb[1] = v.y; rb[2] = v.z; rb[3] = v.w;
        } else {
            #pragma unroll
            for (int q = 0; q < 4; q++) rb[q] = (gj < g.N && gk + q < g.K) ? p[q] : 0.f;
        }
        return;
    }
    const int kk = t / (T::BN / 4), j = (t % (T::BN / 4)) * 4;
    const int gk = k0 + kk, gj = n0 + j;
    const float *p = B + (size_t)gk * g.ldb + gj;
    if (gk < g.K && gj + 3 < g.N && ((reinterpret_cast<uintptr_t>(p) & 15) == 0)) {
        const float4 v = *reinterpret_cast<const float4 *>(p);
        rb[0] = v.x; rb[1] = v.y; rb[2] = v.z; rb[3] = v.w;
    } else {
        #pragma unroll
        for (int q = 0; q < 4; q++) rb[q] = (gk < g.K && gj + q < g.N) ? p[q] : 0.f;
    }
}

template <class T, bool BKC>
__device__ __forceinline__ void store_b(float (*Bs)[T::BN], const float (&rb)[4]) {
    const int t = threadIdx.x;
    if (BKC) {
        const int j = t / (T::BK / 4), kk = (t % (T::BK / 4)) * 4;
        #pragma unroll
        for (int q = 0; q < 4; q++) Bs[kk + q][j] = rb[q];
    } else {
        const int kk = t / (T::BN / 4), j = (t % (T::BN / 4)) * 4;
        *reinterpret_cast<float4 *>(&Bs[kk][j]) = make_float4(rb[0], rb[1], rb[2], rb[3]);
    }
}

template <class T, bool ACOL, bool BKC>
__global__ void __launch_bounds__(GT) k_sgemm(GemmArgs g) {
    constexpr int BM = T::BM, BN = T::BN, BK = T::BK, TM = T::TM, TN = T::TN;
    __shared__ __align__(16) float As[2][BK][BM];
    __shared__ __align__(16) float Bs[2][BK][BN];
    const int bz = blockIdx.z;
    const float *A = g.A + (size_t)bz * g.sA;
    const float *B = g.B + (size_t)bz * g.sB;
    float *C = g.C + (size_t)bz * g.sC;
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;

    float acc[TM][TN];
    #pragma unroll
    for (int i = 0; i < TM; i++)
        #pragma unroll
        for (int j = 0; j < TN; j++) acc[i][j] = 0.f;

    float ra[4], rb[4];
    load_a<T, ACOL>(g, A, m0, 0, ra);
    load_b<T, BKC>(g, B, 0, n0, rb);
    store_a<T, ACOL>(As[0], ra);
    store_b<T, BKC>(Bs[0], rb);
    __syncthreads();
    int buf = 0;
    for (int k0 = 0; k0 < g.K; k0 += BK) {
        const bool more = k0 + BK < g.K;
        if (more) {
            load_a<T, ACOL>(g, A, m0, k0 + BK, ra);
            load_b<T, BKC>(g, B, k0 + BK, n0, rb);
        }
        #pragma unroll
        for (int kk = 0; kk < BK; kk++) {
            float af[TM], bf[TN];
            #pragma unroll
            for (int q = 0; q < TM / 4; q++) {
                const float4 a4 = *reinterpret_cast<const float4 *>(&As[buf][kk][ty * 4 + 64 * q]);
                af[4 * q] = a4.x; af[4 * q + 1] = a4.y; af[4 * q + 2] = a4.z; af[4 * q + 3] = a4.w;
            }
            #pragma unroll
            for (int q = 0; q < TN / 4; q++) {
                const float4 b4 = *reinterpret_cast<const float4 *>(&Bs[buf][kk][tx * 4 + 64 * q]);
                bf[4 * q] = b4.x; bf[4 * q + 1] = b4.y; bf[4 * q + 2] = b4.z; bf[4 * q + 3] = b4.w;
            }
            #pragma unroll
            for (int i = 0; i < TM; i++)
                #pragma unroll
                for (int j = 0; j < TN; j++) acc[i][j] = fmaf(af[i], bf[j], acc[i][j]);
        }
        if (more) {
            store_a<T, ACOL>(As[buf ^ 1], ra);
            store_b<T, BKC>(Bs[buf ^ 1], rb);
        }
        __syncthreads();
        buf ^= 1;
    }
    // rows ty*4 + {0..3} (+ 64); columns tx*4 + {0..3} (+ 64)
    #pragma unroll
    for (int i = 0; i < TM; i++) {
        const int r = m0 + 64 * (i / 4) + ty * 4 + (i % 4);
        if (r >= g.M) continue;
        float cph = 1.f, sph = 0.f;
        if (g.epilogue == 1) {
            const float ph = g.w[(size_t)bz * g.wstride + r] * g.dt_over_hbar;
            sincosf(ph, &sph, &cph);
        }
        #pragma unroll
        for (int h = 0; h < TN / 4; h++) {
            const int c = n0 + h * 64 + tx * 4;
            float v[4] = {acc[i][4 * h], acc[i][4 * h + 1], acc[i][4 * h + 2], acc[i][4 * h + 3]};
            if (g.epilogue == 1) {   // (re, im) pairs times exp(+i ph)
                #pragma unroll
                for (int q = 0; q < 4; q += 2) {
                    const float re = v[q], im = v[q + 1];
                    v[q] = cph * re - sph * im;
                    v[q + 1] = sph * re + cph * im;
                }
            }
            if (g.epilogue == 2) {   // C = D - A B
                const float *d = g.D + (size_t)bz * g.sD + (size_t)r * g.ldd + c;
                #pragma unroll
                for (int q = 0; q < 4; q++) v[q] = (c + q < g.N ? d[q] : 0.f) - v[q];
            }
            float *p = C + (size_t)r * g.ldc + c;
            if (c + 3 < g.N && ((reinterpret_cast<uintptr_t>(p) & 15) == 0)) {
                *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]);
            } else {
                #pragma unroll
                for (int q = 0; q < 4; q++)
                    if (c + q < g.N) p[q] = v[q];
            }
        }
    }
}

__global__ void k_identity(float *F, int n, int ldf, long long sF) {
    float *f = F + (size_t)blockIdx.y * sF;
    const int r = blockIdx.x;
    for (int c = threadIdx.x; c < 2 * n; c += blockDim.x) f[(size_t)r * ldf + c] = (c == 2 * r) ? 1.f : 0.f;
}

template <class T>
cudaError_t launch_sgemm(const GemmArgs &g, int batch, cudaStream_t s) {
    dim3 grid((g.N + T::BN - 1) / T::BN, (g.M + T::BM - 1) / T::BM, batch);
    if (g.a_colmajor && g.b_kmajor) return cudaErrorInvalidValue;
    if (g.a_colmajor) k_sgemm<T, true, false><<<grid, GT, 0, s>>>(g);
    else if (g.b_kmajor) k_sgemm<T, false, true><<<grid, GT, 0, s>>>(g);
    else k_sgemm<T, false, false><<<grid, GT, 0, s>>>(g);
    return cudaGetLastError();
}

}  // namespace

cudaError_t cir_launch_gemm(const GemmArgs &g, int batch, cudaStream_t s, int *launches, int tile) {
    if ((g.epilogue == 1 && (g.N & 1)) || (g.epilogue == 2 && !g.D)) return cudaErrorInvalidValue;
    if (batch < 1 || batch > 65535) return cudaErrorInvalidValue;
    const cudaError_t e = tile == CIR_GEMM_TILE_64 ? launch_sgemm<TileS>(g, batch, s) : launch_sgemm<TileL>(g, batch, s);
    if (launches) *launches += 1;
    return e;
}

cudaError_t cir_launch_identity(float *F, int n, int ldf, long long sF, int batch, cudaStream_t s, int *launches) {
    k_identity<<<dim3(n, batch), 256, 0, s>>>(F, n, ldf, sF);
    if (launches) *launches += 1;
    return cudaGetLastError();
}
