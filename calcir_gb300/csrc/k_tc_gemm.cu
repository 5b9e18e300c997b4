// Tensor-core (tcgen05) GEMM for the propagation step of the mixed-precision form:
// C[b] = A[b] * B[b] with FP32 accumulation in tensor memory, B row-major (N contiguous) or
// K-major, A row-major (K contiguous) or column-major (M contiguous), optional fused phase
// rotation of (re, im) column pairs in the epilogue (see k_gemm.cu for the step) or
// C = D - A B (the Householder back-transform of the eigensolver).
//
// One CTA computes a 128 x 128 tile with 128 threads:
//   * all threads stage 32-deep K slices of A and B from global memory into shared
//     memory, converted to the operand type (TF32 rounded to nearest, or BF16 hi/lo
//     pairs), in the non-swizzled K-major core-matrix layout: core matrix (r/8, k/CK)
//     at (r/8)*SBO + (k/CK)*LBO, 8 rows of 16 bytes inside.  The strides are padded
//     (TF32: 144/1168 bytes, BF16: 128/528) so a warp's stores spread over the banks;
//   * one thread issues the tcgen05.mma instructions of a stage and
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
#include "cir_tcgen05.cuh"

#include <cuda_bf16.h>
#include <stdint.h>

namespace {

constexpr int TM = 128, TN = 128, TK = 32;   // tile; TK elements of K per stage
constexpr int NTHREADS = 128;

// Shared-memory tile layouts (K-major, no swizzle): core matrix (r/8, k/CK) at
// (r/8)*SBO + (k/CK)*LBO, rows of 16 bytes inside; CK = elements per 16 bytes.
// TF32: 8 core matrices along K per stage; BF16: 4, stored as separate hi and lo tiles.
template <int MODE> struct Cfg;
template <> struct Cfg<CIR_PREC_TF32> {
    static constexpr int LBO = 144, SBO = 1168, CK = 4, KSTEP = 8, PARTS = 1;
    static constexpr uint32_t FMT = 2;   // TF32
};
template <> struct Cfg<CIR_PREC_BF16X3> {
    static constexpr int LBO = 128, SBO = 528, CK = 8, KSTEP = 16, PARTS = 2;
    static constexpr uint32_t FMT = 1;   // BF16
};
template <int MODE> __host__ __device__ constexpr int tile_bytes() { return (TM / 8) * Cfg<MODE>::SBO; }
template <int MODE>
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
    // start address >> 4, leading (K) byte offset >> 4, stride (M/N) byte offset >> 4,
    // fixed field 0b001 at bit 46, no swizzle
    return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)(Cfg<MODE>::LBO >> 4) << 16) |
           ((uint64_t)(Cfg<MODE>::SBO >> 4) << 32) | (1ull << 46);
}

// instruction descriptor: D f32, A/B format, K-major A and B, N = 128, M = 128
__host__ __device__ constexpr uint32_t make_idesc(uint32_t ab_format) {
    return (1u << 4) | (ab_format << 7) | (ab_format << 10) | ((uint32_t)(TN >> 3) << 17) | ((uint32_t)(TM >> 4) << 24);
}

// offset in bytes of element (r, k) of a K-major tile
template <int MODE>
__device__ __forceinline__ uint32_t tile_off(int r, int k) {
    using C = Cfg<MODE>;
    return (uint32_t)((r >> 3) * C::SBO + (k / C::CK) * C::LBO + (r & 7) * 16 + (k % C::CK) * (16 / C::CK));
}

// four consecutive K values of one row, converted and stored at tile offset o
template <int MODE>
__device__ __forceinline__ void put4(unsigned char *const (&t)[2], uint32_t o, float a, float b, float c, float d) {
    if (MODE == CIR_PREC_TF32) {
        *reinterpret_cast<uint4 *>(t[0] + o) = make_uint4(to_tf32(a), to_tf32(b), to_tf32(c), to_tf32(d));
    } else {
        const __nv_bfloat16 ha = __float2bfloat16_rn(a), hb = __float2bfloat16_rn(b);
        const __nv_bfloat16 hc = __float2bfloat16_rn(c), hd = __float2bfloat16_rn(d);
        const __nv_bfloat16 la = __float2bfloat16_rn(a - __bfloat162float(ha));
        const __nv_bfloat16 lb = __float2bfloat16_rn(b - __bfloat162float(hb));
        const __nv_bfloat16 lc = __float2bfloat16_rn(c - __bfloat162float(hc));
        const __nv_bfloat16 ld = __float2bfloat16_rn(d - __bfloat162float(hd));
        uint2 hi, lo;
        hi.x = (uint32_t)__bfloat16_as_ushort(ha) | ((uint32_t)__bfloat16_as_ushort(hb) << 16);
        hi.y = (uint32_t)__bfloat16_as_ushort(hc) | ((uint32_t)__bfloat16_as_ushort(hd) << 16);
        lo.x = (uint32_t)__bfloat16_as_ushort(la) | ((uint32_t)__bfloat16_as_ushort(lb) << 16);
        lo.y = (uint32_t)__bfloat16_as_ushort(lc) | ((uint32_t)__bfloat16_as_ushort(ld) << 16);
        *reinterpret_cast<uint2 *>(t[0] + o) = hi;
        *reinterpret_cast<uint2 *>(t[1] + o) = lo;
    }
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
    // write into the K-major tile(s) of the mode (TF32, or BF16 hi and lo)
    template <int MODE>
    __device__ __forceinline__ void store(unsigned char *const (&base)[2]) const {
        const int t = threadIdx.x;
        #pragma unroll
        for (int i = 0; i < 8; i++) {
            if (KC) {
                const int r = i * 16 + t / 8, k = 4 * (t % 8);
                put4<MODE>(base, tile_off<MODE>(r, k), v[i].x, v[i].y, v[i].z, v[i].w);
            } else if (i % 4 == 3) {
                // v[i-3..i] are 4 k rows x 4 consecutive r: transpose to 4 r rows x 4 consecutive k
                const int b = t + NTHREADS * (i / 4);
                const int r = 4 * (b % 32), k = 4 * (b / 32);
                const float4 a0 = v[i - 3], a1 = v[i - 2], a2 = v[i - 1], a3 = v[i];
                put4<MODE>(base, tile_off<MODE>(r + 0, k), a0.x, a1.x, a2.x, a3.x);
                put4<MODE>(base, tile_off<MODE>(r + 1, k), a0.y, a1.y, a2.y, a3.y);
                put4<MODE>(base, tile_off<MODE>(r + 2, k), a0.z, a1.z, a2.z, a3.z);
                put4<MODE>(base, tile_off<MODE>(r + 3, k), a0.w, a1.w, a2.w, a3.w);
            }
        }
    }
};

template <bool ACOL, bool BKC, int MODE>
__global__ void __launch_bounds__(NTHREADS) k_tc_gemm(GemmArgs g) {
    using C_ = Cfg<MODE>;
    constexpr int TB = tile_bytes<MODE>();
    constexpr int STAGE = 2 * C_::PARTS * TB;   // A and B parts of one stage
    extern __shared__ __align__(1024) unsigned char smem[];
    // stage s: A parts at smem + s*STAGE, B parts after them
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + 2 * STAGE);    // [2]
    uint32_t *tslot = reinterpret_cast<uint32_t *>(smem + 2 * STAGE + 16);
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
    constexpr uint32_t IDESC = make_idesc(C_::FMT);

    // two K slices in flight in registers: slice kt + 2 is requested right after slice kt is
    // stored, so a load has two slices' MMA and staging time to arrive
    Slice<!ACOL> la0, la1;   // A: K contiguous unless column-major
    Slice<BKC> lb0, lb1;     // B: N contiguous unless K-major
    const int KT = (g.K + TK - 1) / TK;
    bool ok = true;
    la0.load(A, g.lda, g.M, g.K, m0, 0);
    lb0.load(B, g.ldb, g.N, g.K, n0, 0);
    if (KT > 1) {
        la1.load(A, g.lda, g.M, g.K, m0, TK);
        lb1.load(B, g.ldb, g.N, g.K, n0, TK);
    }
    auto step = [&](int kt, Slice<!ACOL> &la, Slice<BKC> &lb) {
        const int s = kt & 1;
        if (kt >= 2) ok = mbar_wait(&bar[s], ((kt >> 1) - 1) & 1) && ok;   // MMAs that read stage s are done
        unsigned char *const pa[2] = {smem + s * STAGE, smem + s * STAGE + (C_::PARTS - 1) * TB};
        unsigned char *const pb[2] = {smem + s * STAGE + C_::PARTS * TB, smem + s * STAGE + (2 * C_::PARTS - 1) * TB};
        la.template store<MODE>(pa);
        lb.template store<MODE>(pb);
        if (kt + 2 < KT) {
            la.load(A, g.lda, g.M, g.K, m0, (kt + 2) * TK);
            lb.load(B, g.ldb, g.N, g.K, n0, (kt + 2) * TK);
        }
        fence_proxy_async();
        __syncthreads();
        if (tid == 0) {
            fence_after();
            #pragma unroll
            for (int ks = 0; ks < TK / C_::KSTEP; ks++) {
                const uint32_t o = 2 * ks * C_::LBO;   // two core matrices of K per instruction
                const uint64_t ah = smem_desc<MODE>(smem_addr(pa[0]) + o), bh = smem_desc<MODE>(smem_addr(pb[0]) + o);
                if (MODE == CIR_PREC_TF32) {
                    mma_tf32(tmem, ah, bh, IDESC, (kt | ks) != 0);
                } else {   // hi*hi + hi*lo + lo*hi
                    const uint64_t al = smem_desc<MODE>(smem_addr(pa[1]) + o), bl = smem_desc<MODE>(smem_addr(pb[1]) + o);
                    mma_f16(tmem, ah, bh, IDESC, (kt | ks) != 0);
                    mma_f16(tmem, ah, bl, IDESC, 1u);
                    mma_f16(tmem, al, bh, IDESC, 1u);
                }
            }
            mma_commit(&bar[s]);
        }
    };
    for (int kt = 0; kt < KT; kt += 2) {
        step(kt, la0, lb0);
        if (kt + 1 < KT) step(kt + 1, la1, lb1);
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
            if (g.epilogue == 2) {   // C = D - A B
                const float *d = g.D + (size_t)bz * g.sD + (size_t)r * g.ldd + c;
                #pragma unroll
                for (int q = 0; q < 16; q++) v[q] = (c + q < g.N ? d[q] : 0.f) - v[q];
            }
            if (g.Chi) {   // as a BF16 hi/lo pair
                const size_t o = (size_t)bz * 2 * g.sC + (size_t)r * g.ldc + c;
                __nv_bfloat16 *ph = g.Chi + o, *pl = g.Clo + o;
                if (c + 15 < g.N && ((reinterpret_cast<uintptr_t>(ph) | reinterpret_cast<uintptr_t>(pl)) & 15) == 0) {
                    uint32_t wh[8], wl[8];
                    #pragma unroll
                    for (int q = 0; q < 16; q += 2) {
                        const __nv_bfloat162 h = __floats2bfloat162_rn(v[q], v[q + 1]);
                        const __nv_bfloat162 l = __floats2bfloat162_rn(v[q] - __bfloat162float(h.x), v[q + 1] - __bfloat162float(h.y));
                        wh[q / 2] = *reinterpret_cast<const uint32_t *>(&h);
                        wl[q / 2] = *reinterpret_cast<const uint32_t *>(&l);
                    }
                    *reinterpret_cast<uint4 *>(ph) = make_uint4(wh[0], wh[1], wh[2], wh[3]);
                    *reinterpret_cast<uint4 *>(ph + 8) = make_uint4(wh[4], wh[5], wh[6], wh[7]);
                    *reinterpret_cast<uint4 *>(pl) = make_uint4(wl[0], wl[1], wl[2], wl[3]);
                    *reinterpret_cast<uint4 *>(pl + 8) = make_uint4(wl[4], wl[5], wl[6], wl[7]);
                } else {
                    #pragma unroll
                    for (int q = 0; q < 16; q++)
                        if (c + q < g.N) {
                            const __nv_bfloat16 h = __float2bfloat16_rn(v[q]);
                            ph[q] = h;
                            pl[q] = __float2bfloat16_rn(v[q] - __bfloat162float(h));
                        }
                }
                continue;
            }
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

template <int MODE>
__host__ __device__ constexpr size_t smem_bytes() { return 4 * (size_t)Cfg<MODE>::PARTS * tile_bytes<MODE>() + 64; }

template <bool ACOL, bool BKC, int MODE>
cudaError_t launch(const GemmArgs &g, int batch, cudaStream_t s) {
    const size_t smem = smem_bytes<MODE>();
    dim3 grid((g.N + TN - 1) / TN, (g.M + TM - 1) / TM, batch);
    cudaError_t e = cudaFuncSetAttribute(k_tc_gemm<ACOL, BKC, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_tc_gemm<ACOL, BKC, MODE><<<grid, NTHREADS, smem, s>>>(g);
    return cudaGetLastError();
}

template <int MODE>
cudaError_t launch_mode(const GemmArgs &g, int batch, cudaStream_t s) {
    if (g.a_colmajor && g.b_kmajor) return cudaErrorInvalidValue;
    if (g.a_colmajor) return launch<true, false, MODE>(g, batch, s);
    if (g.b_kmajor) return launch<false, true, MODE>(g, batch, s);
    return launch<false, false, MODE>(g, batch, s);
}

}  // namespace

size_t cir_tc_gemm_smem_bytes() { return smem_bytes<CIR_PREC_BF16X3>(); }

cudaError_t cir_launch_tc_gemm(const GemmArgs &g, int batch, int precision, cudaStream_t s, int *launches) {
    if ((g.epilogue == 1 && (g.N & 1)) || (g.epilogue == 2 && !g.D)) return cudaErrorInvalidValue;
    if (batch < 1 || batch > 65535) return cudaErrorInvalidValue;
    cudaError_t e;
    if (precision == CIR_PREC_TF32) e = launch_mode<CIR_PREC_TF32>(g, batch, s);
    else if (precision == CIR_PREC_BF16X3) e = launch_mode<CIR_PREC_BF16X3>(g, batch, s);
    else return cudaErrorInvalidValue;
    if (e != cudaSuccess) return e;
    if (launches) *launches += 1;
    return cudaSuccess;
}
