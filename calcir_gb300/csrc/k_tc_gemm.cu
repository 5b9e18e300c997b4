// Tensor-core (tcgen05) GEMM for the propagation step of the mixed-precision form:
// C[b] = A[b] * B[b] with FP32 accumulation in tensor memory, B row-major (N contiguous),
// A row-major (K contiguous) or column-major (M contiguous), optional fused phase
// rotation of (re, im) column pairs in the epilogue (see k_gemm.cu for the step).
//
// One CTA computes a 128 x 128 tile with 128 threads:
//   * all threads stage 32-deep K slices of A and B from global memory into shared
//     memory, rounded to TF32 (round to nearest), in the non-swizzled K-major
//     core-matrix layout: core matrix (r/8, k/4) at (r/8)*SBO + (k/4)*LBO, 8 rows of 16
//     bytes inside.  LBO = 144 and SBO = 1168 bytes are padded so the 16-byte stores
//     of a warp spread over all bank groups;
//   * one thread issues the tcgen05.mma instructions (K = 8 each) of a stage and
//     signals their completion to the stage's mbarrier with tcgen05.commit; two stages
//     let the loads of the next slice overlap the MMAs of the current one;
//   * the accumulator lives in 128 TMEM columns; each warp reads its 32 lanes with
//     tcgen05.ld, applies the epilogue and stores.
// BF16X3 mode splits each operand into bf16 hi + lo parts and accumulates
// hi*hi + hi*lo + lo*hi (kind::f16, K = 16 per MMA), which keeps about 16 mantissa bits.
//
// Every mbarrier wait is bounded; on timeout the kernel records an error, waits (again
// bounded) for its own MMAs, frees its tensor memory and returns.
#include "cir_device.cuh"

#include <cuda_bf16.h>
#include <stdint.h>

namespace {

constexpr int TM = 128, TN = 128, TK = 32;   // tile; TK in elements per stage (TF32)
constexpr int LBO = 144, SBO = 1168;          // bytes, see above
constexpr int TILE_BYTES = (TM / 8) * SBO;    // 18688 bytes per operand tile
constexpr int NTHREADS = 128;
constexpr long long WAIT_LIMIT = 1ll << 24;

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
    for (long long i = 0; i < WAIT_LIMIT; i++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
    // start address >> 4, leading (K) byte offset >> 4, stride (M/N) byte offset >> 4,
    // fixed field 0b001 at bit 46, no swizzle
    return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)(LBO >> 4) << 16) | ((uint64_t)(SBO >> 4) << 32) |
           (1ull << 46);
}

// instruction descriptor: D f32, A/B format, K-major A and B, N = 128, M = 128
__host__ __device__ constexpr uint32_t make_idesc(uint32_t ab_format) {
    return (1u << 4) | (ab_format << 7) | (ab_format << 10) | ((uint32_t)(TN >> 3) << 17) | ((uint32_t)(TM >> 4) << 24);
}

__device__ __forceinline__ void mma_tf32(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void mma_f16(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void mma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
                 : "memory");
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ uint32_t to_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}

// 16 consecutive fp32 columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    #pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// offset in bytes of element (r, k) of a K-major tile; k counts 4-byte units
__device__ __forceinline__ uint32_t tile_off(int r, int k) {
    return (uint32_t)((r >> 3) * SBO + (k >> 2) * LBO + (r & 7) * 16 + (k & 3) * 4);
}

// One operand slice (rows r0..r0+127 of the MN dimension, k0..k0+TK-1) staged into
// registers.  KC: K contiguous in global memory (element (r, k) at p[r*ld + k]); else MN
// contiguous (element (r, k) at p[k*ld + r]).  Out-of-range elements read as zero.
template <bool KC>
struct Slice {
    float4 v[8];
    __device__ __forceinline__ void load(const float *p, int ld, int rdim, int kdim, int r0, int k0) {
        const int t = threadIdx.x;
        #pragma unroll
        for (int i = 0; i < 8; i++) {
            int r, k;
            if (KC) {   // 8 float4 per thread: row r = i*16 + t/8, k = 4*(t%8)
                r = r0 + i * 16 + t / 8;
                k = k0 + 4 * (t % 8);
            } else {    // 4x4 blocks: block b = t + 128*(i/4), 4 rows of k; i%4 selects the k row
                const int b = t + NTHREADS * (i / 4);
                r = r0 + 4 * (b % 32);
                k = k0 + 4 * (b / 32) + (i % 4);
            }
            float4 x = make_float4(0.f, 0.f, 0.f, 0.f);
            if (KC) {
                const float *q = p + (size_t)r * ld + k;
                if (r < rdim) {
                    if (k + 3 < kdim && ((reinterpret_cast<uintptr_t>(q) & 15) == 0)) x = *reinterpret_cast<const float4 *>(q);
                    else {
                        if (k < kdim) x.x = q[0];
                        if (k + 1 < kdim) x.y = q[1];
                        if (k + 2 < kdim) x.z = q[2];
                        if (k + 3 < kdim) x.w = q[3];
                    }
                }
            } else {
                const float *q = p + (size_t)k * ld + r;
                if (k < kdim) {
                    if (r + 3 < rdim && ((reinterpret_cast<uintptr_t>(q) & 15) == 0)) x = *reinterpret_cast<const float4 *>(q);
                    else {
                        if (r < rdim) x.x = q[0];
                        if (r + 1 < rdim) x.y = q[1];
                        if (r + 2 < rdim) x.z = q[2];
                        if (r + 3 < rdim) x.w = q[3];
                    }
                }
            }
            v[i] = x;
        }
    }
    // write as TF32 into the K-major tile at byte address base
    __device__ __forceinline__ void store_tf32(unsigned char *base) const {
        const int t = threadIdx.x;
        #pragma unroll
        for (int i = 0; i < 8; i++) {
            if (KC) {
                const int r = i * 16 + t / 8, k = 4 * (t % 8);
                const uint4 u = make_uint4(to_tf32(v[i].x), to_tf32(v[i].y), to_tf32(v[i].z), to_tf32(v[i].w));
                *reinterpret_cast<uint4 *>(base + tile_off(r, k)) = u;
            } else if (i % 4 == 3) {
                // v[i-3..i] are 4 k rows x 4 consecutive r: transpose to 4 r rows x 4 consecutive k
                const int b = t + NTHREADS * (i / 4);
                const int r = 4 * (b % 32), k = 4 * (b / 32);
                const float4 a0 = v[i - 3], a1 = v[i - 2], a2 = v[i - 1], a3 = v[i];
                *reinterpret_cast<uint4 *>(base + tile_off(r + 0, k)) = make_uint4(to_tf32(a0.x), to_tf32(a1.x), to_tf32(a2.x), to_tf32(a3.x));
                *reinterpret_cast<uint4 *>(base + tile_off(r + 1, k)) = make_uint4(to_tf32(a0.y), to_tf32(a1.y), to_tf32(a2.y), to_tf32(a3.y));
                *reinterpret_cast<uint4 *>(base + tile_off(r + 2, k)) = make_uint4(to_tf32(a0.z), to_tf32(a1.z), to_tf32(a2.z), to_tf32(a3.z));
                *reinterpret_cast<uint4 *>(base + tile_off(r + 3, k)) = make_uint4(to_tf32(a0.w), to_tf32(a1.w), to_tf32(a2.w), to_tf32(a3.w));
            }
        }
    }
};

template <bool ACOL>
__global__ void __launch_bounds__(NTHREADS) k_tc_gemm_tf32(GemmArgs g) {
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char *sA[2] = {smem, smem + TILE_BYTES};
    unsigned char *sB[2] = {smem + 2 * TILE_BYTES, smem + 3 * TILE_BYTES};
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + 4 * TILE_BYTES);    // [2]
    uint32_t *tslot = reinterpret_cast<uint32_t *>(smem + 4 * TILE_BYTES + 16);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int bz = blockIdx.z;
    const float *A = g.A + (size_t)bz * g.sA;
    const float *B = g.B + (size_t)bz * g.sB;
    float *C = g.C + (size_t)bz * g.sC;
    const int m0 = blockIdx.y * TM, n0 = blockIdx.x * TN;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tslot)),
                     "r"(TN));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tslot;
    constexpr uint32_t IDESC = make_idesc(2);   // TF32

    Slice<!ACOL> la;    // A: K contiguous unless column-major
    Slice<false> lb;    // B: N contiguous
    const int KT = (g.K + TK - 1) / TK;
    bool ok = true;
    la.load(g.A + (size_t)bz * g.sA, g.lda, g.M, g.K, m0, 0);
    lb.load(B, g.ldb, g.N, g.K, n0, 0);
    for (int kt = 0; kt < KT; kt++) {
        const int s = kt & 1;
        if (kt >= 2) ok = mbar_wait(&bar[s], ((kt >> 1) - 1) & 1) && ok;   // MMAs that read stage s are done
        la.store_tf32(sA[s]);
        lb.store_tf32(sB[s]);
        fence_proxy_async();
        __syncthreads();
        if (tid == 0) {
            fence_after();
            const uint32_t a0 = smem_addr(sA[s]), b0 = smem_addr(sB[s]);
            #pragma unroll
            for (int ks = 0; ks < TK / 8; ks++)
                mma_tf32(tmem, smem_desc(a0 + 2 * ks * LBO), smem_desc(b0 + 2 * ks * LBO), IDESC, (kt | ks) != 0);
            mma_commit(&bar[s]);
        }
        if (kt + 1 < KT) {
            la.load(A, g.lda, g.M, g.K, m0, (kt + 1) * TK);
            lb.load(B, g.ldb, g.N, g.K, n0, (kt + 1) * TK);
        }
    }
    {   // the last commit covers every MMA issued before it
        const int last = KT - 1;
        ok = mbar_wait(&bar[last & 1], (last >> 1) & 1) && ok;
    }
    fence_after();
    if (!ok) {
        if (g.err && lane == 0) atomicExch(g.err, 1);
    } else {
        const int r = m0 + warp * 32 + lane;
        float cph = 1.f, sph = 0.f;
        if (g.epilogue == 1 && r < g.M) {
            const float ph = g.w[(size_t)bz * g.wstride + r] * g.dt_over_hbar;
            sincosf(ph, &sph, &cph);
        }
        #pragma unroll 1
        for (int c0 = 0; c0 < TN; c0 += 16) {
            float v[16];
            tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
            if (r >= g.M) continue;
            if (g.epilogue == 1) {
                #pragma unroll
                for (int q = 0; q < 16; q += 2) {
                    const float re = v[q], im = v[q + 1];
                    v[q] = cph * re - sph * im;
                    v[q + 1] = sph * re + cph * im;
                }
            }
            const int c = n0 + c0;
            float *p = C + (size_t)r * g.ldc + c;
            if (c + 15 < g.N && ((reinterpret_cast<uintptr_t>(p) & 15) == 0)) {
                #pragma unroll
                for (int q = 0; q < 16; q += 4) *reinterpret_cast<float4 *>(p + q) = make_float4(v[q], v[q + 1], v[q + 2], v[q + 3]);
            } else {
                #pragma unroll
                for (int q = 0; q < 16; q++)
                    if (c + q < g.N) p[q] = v[q];
            }
        }
    }
    fence_before();
    __syncthreads();
    if (warp == 0) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TN));
    }
}

}  // namespace

size_t cir_tc_gemm_smem_bytes() { return 4 * (size_t)TILE_BYTES + 64; }

cudaError_t cir_launch_tc_gemm(const GemmArgs &g, int batch, int precision, cudaStream_t s, int *launches) {
    if (g.epilogue == 1 && (g.N & 1)) return cudaErrorInvalidValue;
    if (precision != CIR_PREC_TF32) return cudaErrorInvalidValue;
    const size_t smem = cir_tc_gemm_smem_bytes();
    dim3 grid((g.N + TN - 1) / TN, (g.M + TM - 1) / TM, batch);
    cudaError_t e;
    if (g.a_colmajor) {
        e = cudaFuncSetAttribute(k_tc_gemm_tf32<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e == cudaSuccess) k_tc_gemm_tf32<true><<<grid, NTHREADS, smem, s>>>(g);
    } else {
        e = cudaFuncSetAttribute(k_tc_gemm_tf32<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e == cudaSuccess) k_tc_gemm_tf32<false><<<grid, NTHREADS, smem, s>>>(g);
    }
    if (e != cudaSuccess) return e;
    if (launches) *launches += 1;
    return cudaGetLastError();
}
