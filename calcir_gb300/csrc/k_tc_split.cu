// Propagation step of the split-BF16 mixed form on pre-split operands.
//
// The step F <- V exp(i L dt/hbar) V^T F (calcIR.cu:596-613) is two real GEMMs.  Every
// operand is kept in global memory as a pair of BF16 matrices (hi = bf16(x),
// lo = bf16(x - hi)), K-major, and each product is hi*hi + hi*lo + lo*hi accumulated in
// FP32 tensor memory (tcgen05.mma kind::f16):
//     G = V^T F      A = V (column-major: A(i, k) = V[k][i] at Vc[i*ldh + k]),
//                    B = F stored transposed (B(k, c) = F[k][c] at Ft[c*ldh + k]),
//                    epilogue: row i of G times exp(+i w_i dt/hbar), written transposed (Gt)
//     F' = V G       A = V row-major (Vr[i*ldh + k] = V[i][k]), B = Gt, written as Ft
// so the output of each product is the K-major operand of the next.  k_split_v writes
// Vc and Vr from the eigensolver's FP32 eigenvectors once per step.
//
// One CTA computes a 128 x 128 tile: thread 0 streams 32-deep K slices of A hi, A lo,
// B hi and B lo with TMA (cp.async.bulk.tensor, 64-byte swizzle, one 8 KB box each) into
// a 3-stage ring, counting the bytes on the stage's full barrier; thread 32 issues the
// 6 MMAs of a stage and commits them to the stage's empty barrier, which the producer
// waits on before refilling it.  At 97 KB of shared memory two CTAs share an SM, so one
// CTA's epilogue overlaps the other's MMAs (measured faster than 64-deep 128-byte-swizzled
// stages at one CTA per SM).  The epilogue reads the accumulator with tcgen05.ld
// (lane = row) and stores each column's 32 rows of a warp as 64 contiguous bytes.  Every
// mbarrier wait is bounded; a timeout sets the error flag.
#include "cir_device.cuh"
#include "cir_tcgen05.cuh"

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <algorithm>
#include <climits>
#include <cstdlib>
#include <mutex>

namespace {

struct SplitMaps {
    CUtensorMap a_hi, a_lo, b_hi, b_lo;
};

constexpr int QM = 128;                       // tile rows
constexpr int QT = 128;                       // threads

// QK BF16 of K per stage = one swizzled row of 2 QK bytes (128-byte swizzle for QK = 64,
// 64-byte for QK = 32), QS stages of A hi, A lo (QM rows) and B hi, B lo (QN rows)
template <int QK, int QS, int QN> struct QCfg {
    static constexpr int TILE_A = QM * QK * 2, TILE_B = QN * QK * 2;
    static constexpr int STAGE = 2 * TILE_A + 2 * TILE_B;
    static constexpr size_t SMEM = (size_t)QS * STAGE + 1024 + 256;   // + alignment slack, barriers
};

// shared-memory descriptor of a K-major tile in the swizzled layout a TMA box of QK BF16
// x rows writes: 8-row atoms of 16 QK bytes (the stride byte offset), leading byte offset
// unused (1), the layout type at bit 61 (2: 128-byte swizzle, 4: 64-byte)
template <int QK>
__device__ __forceinline__ uint64_t desc_sw(uint32_t addr) {
    constexpr uint64_t layout = QK == 64 ? 2ull : 4ull;
    return (uint64_t)((addr >> 4) & 0x3FFF) | (1ull << 16) | ((uint64_t)((16 * QK) >> 4) << 32) | (1ull << 46) |
           (layout << 61);
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}

// 3-D tiled TMA load (x = K, y = row, z = matrix) into shared memory, completing on bar
__device__ __forceinline__ void tma_load3(uint32_t dst, const CUtensorMap *map, int x, int y, int z, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
        ::"r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
        : "memory");
}

// One CTA per 128 x 128 tile of C.  Thread 0 is the TMA producer (stage s is refilled once
// the MMAs that read it have committed to empty[s]), thread 32 issues the MMAs of a stage
// once full[s] has received its bytes, and all four warps run the epilogue.
template <int QK, int QS, int QN>
__global__ void __launch_bounds__(QT) k_tc_split(const __grid_constant__ SplitMaps maps, SplitGemmArgs g) {
    using C = QCfg<QK, QS, QN>;
    constexpr int TA = C::TILE_A, TB = C::TILE_B, Q_STAGE = C::STAGE;
    constexpr uint32_t Q_IDESC = make_idesc_mn(1u, QM, QN);   // BF16 operands
    extern __shared__ unsigned char smem_raw[];
    const uint32_t raw = smem_addr(smem_raw);
    const uint32_t sbase = (raw + 1023) & ~1023u;             // 1024-byte aligned stages
    unsigned char *smem = smem_raw + (sbase - raw);
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + QS * Q_STAGE);   // [QS]
    uint64_t *empty = full + QS;                                        // [QS]
    uint64_t *done = empty + QS;
    uint32_t *tslot = reinterpret_cast<uint32_t *>(done + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int bz = blockIdx.z + g.bz0;
    const int m0 = blockIdx.y * QM, n0 = blockIdx.x * QN;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tslot)),
                     "r"(QN));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        for (int s = 0; s < QS; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tslot;

    const int KT = (g.K + QK - 1) / QK;
    bool ok = true;
    if (tid == 0) {
        for (int kt = 0; kt < KT && ok; kt++) {
            const int s = kt % QS;
            if (kt >= QS) ok = mbar_wait(&empty[s], ((kt / QS) - 1) & 1);
            if (!ok) break;
            const uint32_t st = sbase + s * Q_STAGE;
            mbar_expect_tx(&full[s], Q_STAGE);
            tma_load3(st, &maps.a_hi, kt * QK, m0, bz, &full[s]);
            tma_load3(st + TA, &maps.a_lo, kt * QK, m0, bz, &full[s]);
            tma_load3(st + 2 * TA, &maps.b_hi, kt * QK, n0, bz, &full[s]);
            tma_load3(st + 2 * TA + TB, &maps.b_lo, kt * QK, n0, bz, &full[s]);
        }
    } else if (tid == 32) {
        for (int kt = 0; kt < KT && ok; kt++) {
            const int s = kt % QS;
            ok = mbar_wait(&full[s], (kt / QS) & 1);
            if (!ok) break;
            fence_after();
            const uint32_t st = sbase + s * Q_STAGE;
            #pragma unroll
            for (int ks = 0; ks < QK / 16; ks++) {
                const uint32_t o = 32 * ks;                  // 16 BF16 of K inside the swizzled row
                const uint64_t ah = desc_sw<QK>(st + o), al = desc_sw<QK>(st + TA + o);
                const uint64_t bh = desc_sw<QK>(st + 2 * TA + o), bl = desc_sw<QK>(st + 2 * TA + TB + o);
                mma_f16(tmem, ah, bh, Q_IDESC, (kt | ks) != 0);
                mma_f16(tmem, ah, bl, Q_IDESC, 1u);
                mma_f16(tmem, al, bh, Q_IDESC, 1u);
            }
            mma_commit(&empty[s]);
        }
        mma_commit(done);   // arrives once every MMA issued above has completed
    }
    __syncwarp();
    ok = mbar_wait(done, 0) && ok;
    fence_after();
    ok = __syncthreads_and(ok);   // one branch for the whole block (the epilogue reduces over it)
    if (!ok) {
        if (g.err && lane == 0) atomicExch(g.err, 1);
    } else {
        const int r = m0 + warp * 32 + lane;
        const bool fuse = g.tcf_out != nullptr;
        float pr[9], pi[9];
        #pragma unroll
        for (int a = 0; a < 9; a++) pr[a] = pi[a] = 0.f;
        float cph = 1.f, sph = 0.f;
        if (g.epilogue == 1 && r < g.M) {
            const float ph = g.w[(size_t)bz * g.wstride + r] * g.dt_over_hbar;
            sincosf(ph, &sph, &cph);
        }
        __nv_bfloat16 *Ch = g.Chi + (size_t)bz * g.sC, *Cl = g.Clo + (size_t)bz * g.sC;
        // epilogue 2 loads its row's D chunk one chunk ahead (16 values of hi and lo as four
        // 16-byte words), so that the load's latency overlaps the previous chunk's work
        const bool dpre = g.epilogue == 2 && r < g.M;
        auto dload = [&](int cc, uint4 *d) -> bool {
            const int c = n0 + cc;
            const __nv_bfloat16 *dh = g.Dhi + (size_t)bz * g.sD + (size_t)r * g.ldd + c;
            const __nv_bfloat16 *dl = g.Dlo + (size_t)bz * g.sD + (size_t)r * g.ldd + c;
            if (c + 15 >= g.N || ((reinterpret_cast<uintptr_t>(dh) | reinterpret_cast<uintptr_t>(dl)) & 15)) return false;
            d[0] = *reinterpret_cast<const uint4 *>(dh);
            d[1] = *reinterpret_cast<const uint4 *>(dh + 8);
            d[2] = *reinterpret_cast<const uint4 *>(dl);
            d[3] = *reinterpret_cast<const uint4 *>(dl + 8);
            return true;
        };
        uint4 dnext[4];
        bool dnext_ok = dpre && dload(0, dnext);
        #pragma unroll 1
        for (int c0 = 0; c0 < QN; c0 += 16) {
            uint4 dcur[4] = {dnext[0], dnext[1], dnext[2], dnext[3]};
            const bool dcur_ok = dnext_ok;
            if (dpre && c0 + 16 < QN) dnext_ok = dload(c0 + 16, dnext);
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
            if (g.epilogue == 2) {   // C = D - A B, D a row-major split pair
                const __nv_bfloat16 *dh = g.Dhi + (size_t)bz * g.sD + (size_t)r * g.ldd + c;
                const __nv_bfloat16 *dl = g.Dlo + (size_t)bz * g.sD + (size_t)r * g.ldd + c;
                if (dcur_ok) {
                    #pragma unroll
                    for (int h = 0; h < 2; h++) {
                        const uint4 a = dcur[h], b = dcur[2 + h];
                        const uint32_t wa[4] = {a.x, a.y, a.z, a.w}, wb[4] = {b.x, b.y, b.z, b.w};
                        #pragma unroll
                        for (int u = 0; u < 8; u++) {
                            const float xh = __uint_as_float((wa[u / 2] >> (16 * (u & 1))) << 16);
                            const float xl = __uint_as_float((wb[u / 2] >> (16 * (u & 1))) << 16);
                            v[8 * h + u] = (xh + xl) - v[8 * h + u];
                        }
                    }
                } else {
                    #pragma unroll
                    for (int q = 0; q < 16; q++)
                        v[q] = (c + q < g.N ? __bfloat162float(dh[q]) + __bfloat162float(dl[q]) : 0.f) - v[q];
                }
            }
            if (g.out_mode == 0) {           // transposed split pair
                #pragma unroll
                for (int q = 0; q < 16; q++) {
                    if (c + q < g.N) {
                        const __nv_bfloat16 h = __float2bfloat16_rn(v[q]);
                        Ch[(size_t)(c + q) * g.ldc + r] = h;
                        Cl[(size_t)(c + q) * g.ldc + r] = __float2bfloat16_rn(v[q] - __bfloat162float(h));
                    }
                }
            } else if (g.out_mode == 1) {    // row-major split pair
                uint32_t wh[8], wl[8];   // 16 values as packed BF16 pairs
                #pragma unroll
                for (int q = 0; q < 16; q += 2) {
                    const __nv_bfloat16 h0 = __float2bfloat16_rn(v[q]), h1 = __float2bfloat16_rn(v[q + 1]);
                    const __nv_bfloat16 l0 = __float2bfloat16_rn(v[q] - __bfloat162float(h0));
                    const __nv_bfloat16 l1 = __float2bfloat16_rn(v[q + 1] - __bfloat162float(h1));
                    wh[q / 2] = (uint32_t)__bfloat16_as_ushort(h0) | ((uint32_t)__bfloat16_as_ushort(h1) << 16);
                    wl[q / 2] = (uint32_t)__bfloat16_as_ushort(l0) | ((uint32_t)__bfloat16_as_ushort(l1) << 16);
                }
                __nv_bfloat16 *ph = Ch + (size_t)r * g.ldc + c, *pl = Cl + (size_t)r * g.ldc + c;
                if (c + 15 < g.N && ((reinterpret_cast<uintptr_t>(ph) | reinterpret_cast<uintptr_t>(pl)) & 15) == 0) {
                    #pragma unroll
                    for (int q = 0; q < 8; q += 4) {
                        *reinterpret_cast<uint4 *>(ph + 2 * q) = make_uint4(wh[q], wh[q + 1], wh[q + 2], wh[q + 3]);
                        *reinterpret_cast<uint4 *>(pl + 2 * q) = make_uint4(wl[q], wl[q + 1], wl[q + 2], wl[q + 3]);
                    }
                } else {
                    #pragma unroll
                    for (int q = 0; q < 16; q++)
                        if (c + q < g.N) {
                            ph[q] = __ushort_as_bfloat16((unsigned short)(wh[q / 2] >> (16 * (q & 1))));
                            pl[q] = __ushort_as_bfloat16((unsigned short)(wl[q / 2] >> (16 * (q & 1))));
                        }
                }
            } else {                         // row-major FP32
                float *pf = g.Cf + (size_t)bz * g.sC + (size_t)r * g.ldc + c;
                if (c + 15 < g.N && (reinterpret_cast<uintptr_t>(pf) & 15) == 0) {
                    #pragma unroll
                    for (int q = 0; q < 16; q += 4) *reinterpret_cast<float4 *>(pf + q) = make_float4(v[q], v[q + 1], v[q + 2], v[q + 3]);
                } else {
                    #pragma unroll
                    for (int q = 0; q < 16; q++)
                        if (c + q < g.N) pf[q] = v[q];
                }
            }
            if (fuse) {   // psi_a[r] += F'[r][q] m_a(0)[q] over the chunk's 8 complex columns
                const float *m0p = g.tcf_m0 + (size_t)bz * g.tcf_sm0;
                #pragma unroll
                for (int u = 0; u < 8; u++) {
                    const int q = (c >> 1) + u;
                    if (2 * q + 1 < g.N) {
                        #pragma unroll
                        for (int a = 0; a < 9; a++) {
                            const float m = __ldg(m0p + (size_t)a * g.tcf_ldv + q);
                            pr[a] = fmaf(v[2 * u], m, pr[a]);
                            pi[a] = fmaf(v[2 * u + 1], m, pi[a]);
                        }
                    }
                }
            }
        }
        if (fuse) {
            // the row's six terms (k_tcf's combination), then a block sum into the step's slot
            __shared__ double tred[QT / 32][6];
            float t6[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            if (r < g.M) {
                const float *mtp = g.tcf_mt + (size_t)bz * g.tcf_smt;
                float cm[9];
                #pragma unroll
                for (int a = 0; a < 9; a++) cm[a] = mtp[(size_t)a * g.tcf_ldv + r];
                const float ii_r = cm[3] * pr[3] + cm[4] * pr[4] + cm[5] * pr[5];
                const float ii_i = cm[3] * pi[3] + cm[4] * pi[4] + cm[5] * pi[5];
                const float ij_r = cm[6] * pr[6] + cm[7] * pr[7] + cm[8] * pr[8];
                const float ij_i = cm[6] * pi[6] + cm[7] * pi[7] + cm[8] * pi[8];
                const float jj_r = (cm[4] + cm[5]) * pr[3] + (cm[3] + cm[5]) * pr[4] + (cm[3] + cm[4]) * pr[5];
                const float jj_i = (cm[4] + cm[5]) * pi[3] + (cm[3] + cm[5]) * pi[4] + (cm[3] + cm[4]) * pi[5];
                t6[0] = cm[0] * pr[0] + cm[1] * pr[1] + cm[2] * pr[2];
                t6[1] = cm[0] * pi[0] + cm[1] * pi[1] + cm[2] * pi[2];
                t6[2] = (3.f * ii_r + jj_r + 4.f * ij_r) * (1.f / 15.f);
                t6[3] = (3.f * ii_i + jj_i + 4.f * ij_i) * (1.f / 15.f);
                t6[4] = (2.f * ii_r - jj_r + 6.f * ij_r) * (1.f / 30.f);
                t6[5] = (2.f * ii_i - jj_i + 6.f * ij_i) * (1.f / 30.f);
            }
            #pragma unroll
            for (int q = 0; q < 6; q++) {
                const double d = warp_sum_d((double)t6[q]);
                if (lane == 0) tred[warp][q] = d;
            }
            __syncthreads();
            if (threadIdx.x < 6) {
                double s = 0.0;
                #pragma unroll
                for (int w = 0; w < QT / 32; w++) s += tred[w][threadIdx.x];
                atomicAdd(g.tcf_out + (size_t)bz * g.tcf_sout + threadIdx.x, s);
            }
        }
    }
    fence_before();
    __syncthreads();
    if (warp == 0) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(QN));
    }
}

// Persistent, warp-specialised form of the same product (every epilogue and output form of
// k_tc_split, the fused correlation terms optional): one CTA per SM walks
// the tiles t = blockIdx.x, + gridDim.x, ... (column tile fastest, then row tile, then
// matrix).  Warp 0 lane 0 streams every tile's K slices through one QS-stage ring; warp 1
// lane 0 issues the MMAs of tile i into tensor-memory accumulator i & 1 and commits it to
// tfull; warps 2..9 drain accumulator i & 1 while tile i + 1 is loaded and multiplied
// (warp w reads TMEM lane quarter w & 3, and the first or second half of the columns),
// then release it on tempty.  Every wait is bounded: a
// timeout raises the CTA's abort flag and the error flag, every role leaves its loop, the
// producer waits for its copies in flight, and the accumulators are freed.
constexpr int PT = 320;                       // threads: producer, MMA, eight epilogue warps
constexpr int PEW = 8;                        // epilogue warps

// The products one persistent launch walks: up to CIR_SPLIT_MAXP problems (each a batch of
// one shape, e.g. the origins of one box size), their tiles numbered problem after problem.
struct PersistPlan {
    SplitMaps maps[CIR_SPLIT_MAXP];
    SplitGemmArgs g[CIR_SPLIT_MAXP];
    int tiles_n[CIR_SPLIT_MAXP], tiles_mn[CIR_SPLIT_MAXP], first[CIR_SPLIT_MAXP + 1];
    int np;
};

// problem, batch entry and tile origin of tile t of a plan
__device__ __forceinline__ int plan_tile(const PersistPlan &plan, int t, int &bz, int &m0, int &n0, int qn) {
    int pi = 0;
    while (pi + 1 < plan.np && t >= plan.first[pi + 1]) pi++;
    const int lt = t - plan.first[pi], rem = lt % plan.tiles_mn[pi];
    bz = lt / plan.tiles_mn[pi] + plan.g[pi].bz0;
    m0 = (rem / plan.tiles_n[pi]) * QM;
    n0 = (rem % plan.tiles_n[pi]) * qn;
    return pi;
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

template <int QK, int QS, int QN>
__global__ void __launch_bounds__(PT, 1) k_tc_persist(const __grid_constant__ PersistPlan plan) {
    const int ntiles = plan.first[plan.np];
    using C = QCfg<QK, QS, QN>;
    constexpr int TA = C::TILE_A, TB = C::TILE_B, Q_STAGE = C::STAGE;
    constexpr uint32_t Q_IDESC = make_idesc_mn(1u, QM, QN);
    extern __shared__ unsigned char smem_raw[];
    const uint32_t raw = smem_addr(smem_raw);
    const uint32_t sbase = (raw + 1023) & ~1023u;
    unsigned char *smem = smem_raw + (sbase - raw);
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + QS * Q_STAGE);   // [QS]
    uint64_t *empty = full + QS;                                        // [QS]
    uint64_t *tfull = empty + QS;                                       // [2]
    uint64_t *tempty = tfull + 2;                                       // [2]
    uint64_t *drain = tempty + 2;
    uint32_t *tslot = reinterpret_cast<uint32_t *>(drain + 1);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(tslot + 1);
    // the fused contraction's per-tile sums: the epilogue warps of accumulator a add into
    // tred[a], and the last of them adds the six totals to the step's slots in FP64
    __shared__ double tred[2][6];
    __shared__ int tcnt[2];
    // the fused contraction's m(0) values of each epilogue warp's columns of the current tile
    // (complex columns, nine vectors), staged once per tile
    __shared__ __align__(16) float msm[PEW][9][QN / 4];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tslot)),
                     "r"(2 * QN));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        for (int s = 0; s < QS; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int a = 0; a < 2; a++) {
            mbar_init(&tfull[a], 1);
            mbar_init(&tempty[a], PEW);
        }
        mbar_init(drain, 1);
        *abort_flag = 0;
        for (int a = 0; a < 2; a++) {
            tcnt[a] = 0;
            for (int q = 0; q < 6; q++) tred[a][q] = 0.0;
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tslot;
    // the pipeline's waits; the fault drill shortens them so that they run out quickly (the
    // waits for copies and MMAs in flight before the CTA exits always keep the full limit)
    const bool stall = plan.g[0].test_stall != 0;
    const long long lim = stall ? (1ll << 14) : WAIT_LIMIT;
    auto fail = [&]() {
        *abort_flag = 1;
        if (plan.g[0].err) atomicExch(plan.g[0].err, 1);
    };

    if (warp == 0) {
        if (lane == 0) {
            uint32_t it = 0;
            bool ok = true;
            for (int t = blockIdx.x; t < ntiles && ok && !*abort_flag; t += gridDim.x) {
                int bz, m0, n0;
                const int pi = plan_tile(plan, t, bz, m0, n0, QN);
                const SplitMaps &maps = plan.maps[pi];
                const int KT = (plan.g[pi].K + QK - 1) / QK;
                for (int kt = 0; kt < KT; kt++, it++) {
                    const int s = it % QS;
                    if (it >= QS && !(ok = mbar_wait(&empty[s], ((it / QS) & 1) ^ 1, lim))) break;
                    if (*abort_flag) break;
                    const uint32_t st = sbase + s * Q_STAGE;
                    mbar_expect_tx(&full[s], Q_STAGE);
                    tma_load3(st, &maps.a_hi, kt * QK, m0, bz, &full[s]);
                    tma_load3(st + TA, &maps.a_lo, kt * QK, m0, bz, &full[s]);
                    tma_load3(st + 2 * TA, &maps.b_hi, kt * QK, n0, bz, &full[s]);
                    tma_load3(st + 2 * TA + TB, &maps.b_lo, kt * QK, n0, bz, &full[s]);
                }
            }
            if (!ok) fail();
            // the copies of the last QS slices may still be in flight: wait for them
            for (uint32_t j = it > QS ? it - QS : 0; j < it; j++) mbar_wait(&full[j % QS], (j / QS) & 1);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            uint32_t it = 0;
            bool ok = true, issued = false;
            int li = 0;
            for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x, li++) {
                const int a = li & 1;
                int bz_, m0_, n0_;
                const int KT = (plan.g[plan_tile(plan, t, bz_, m0_, n0_, QN)].K + QK - 1) / QK;
                if (li >= 2 && !(ok = mbar_wait(&tempty[a], ((li >> 1) & 1) ^ 1, lim))) break;
                if (*abort_flag) break;
                fence_after();
                const uint32_t d = tmem + (uint32_t)(a * QN);
                for (int kt = 0; kt < KT; kt++, it++) {
                    const int s = it % QS;
                    if (!(ok = mbar_wait(&full[s], (it / QS) & 1, lim))) break;
                    fence_after();
                    const uint32_t st = sbase + s * Q_STAGE;
                    #pragma unroll
                    for (int ks = 0; ks < QK / 16; ks++) {
                        const uint32_t o = 32 * ks;
                        const uint64_t ah = desc_sw<QK>(st + o), al = desc_sw<QK>(st + TA + o);
                        const uint64_t bh = desc_sw<QK>(st + 2 * TA + o), bl = desc_sw<QK>(st + 2 * TA + TB + o);
                        mma_f16(d, ah, bh, Q_IDESC, (kt | ks) != 0);
                        mma_f16(d, ah, bl, Q_IDESC, 1u);
                        mma_f16(d, al, bh, Q_IDESC, 1u);
                    }
                    issued = true;
                    mma_commit(&empty[s]);
                }
                if (!ok) break;
                // fault drill: the first tile's completion is never signalled, so the epilogue's
                // wait on it (and then every other role's) runs out
                if (!(stall && li == 0)) mma_commit(&tfull[a]);
            }
            if (!ok) fail();
            if (issued) {   // every MMA issued has completed before the accumulators are freed
                mma_commit(drain);
                mbar_wait(drain, 0);
            }
        }
    } else {
        const int quarter = warp & 3, row = quarter * 32 + lane;
        const int cbeg = ((warp - 2) >> 2) * (QN / 2), cend = cbeg + QN / 2;   // this warp's columns
        int li = 0;
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x, li++) {
            const int a = li & 1;
            if (!mbar_wait(&tfull[a], (li >> 1) & 1, lim)) {
                fail();
                break;
            }
            if (*abort_flag) break;
            fence_after();
            int bz, m0, n0;
            const SplitGemmArgs &g = plan.g[plan_tile(plan, t, bz, m0, n0, QN)];
            const bool fuse = g.tcf_out != nullptr;
            const int r = m0 + row;
            float pr[9], pi[9];
            #pragma unroll
            for (int q = 0; q < 9; q++) pr[q] = pi[q] = 0.f;
            float cph = 1.f, sph = 0.f;
            if (g.epilogue == 1 && r < g.M) sincosf(g.w[(size_t)bz * g.wstride + r] * g.dt_over_hbar, &sph, &cph);
            __nv_bfloat16 *Ch = g.Chi + (size_t)bz * g.sC, *Cl = g.Clo + (size_t)bz * g.sC;
            const float *m0p = fuse ? g.tcf_m0 + (size_t)bz * g.tcf_sm0 : nullptr;
            float *mw = &msm[warp - 2][0][0];
            if (fuse) {   // all of this warp's m(0) values for the tile in one round of loads
                const int qb = (n0 + cbeg) >> 1;
                __syncwarp();                     // the previous tile's reads are done
                #pragma unroll
                for (int b9 = 0; b9 < 9; b9++) {
                    #pragma unroll
                    for (int u = lane; u < QN / 4; u += 32) {
                        const int q = qb + u;
                        mw[b9 * (QN / 4) + u] = 2 * q + 1 < g.N ? __ldg(m0p + (size_t)b9 * g.tcf_ldv + q) : 0.f;
                    }
                }
                __syncwarp();
            }
            // epilogue 2 loads its row's D chunk one chunk ahead (hi and lo as four 16-byte words)
            const bool dpre = g.epilogue == 2 && r < g.M;
            auto dload = [&](int cc, uint4 *dd) -> bool {
                const int c = n0 + cc;
                const __nv_bfloat16 *dh = g.Dhi + (size_t)bz * g.sD + (size_t)r * g.ldd + c;
                const __nv_bfloat16 *dl = g.Dlo + (size_t)bz * g.sD + (size_t)r * g.ldd + c;
                if (c + 15 >= g.N || ((reinterpret_cast<uintptr_t>(dh) | reinterpret_cast<uintptr_t>(dl)) & 15))
                    return false;
                dd[0] = *reinterpret_cast<const uint4 *>(dh);
                dd[1] = *reinterpret_cast<const uint4 *>(dh + 8);
                dd[2] = *reinterpret_cast<const uint4 *>(dl);
                dd[3] = *reinterpret_cast<const uint4 *>(dl + 8);
                return true;
            };
            // three chunks in flight: the loads of chunk c0 + 48 are issued while c0 is processed
            uint4 dnext[4], dnext2[4], dnext3[4];
            bool dnext_ok = dpre && dload(cbeg, dnext);
            bool dnext2_ok = dpre && cbeg + 16 < cend && dload(cbeg + 16, dnext2);
            bool dnext3_ok = dpre && cbeg + 32 < cend && dload(cbeg + 32, dnext3);
            #pragma unroll 1
            for (int c0 = cbeg; c0 < cend; c0 += 16) {
                uint4 dcur[4] = {dnext[0], dnext[1], dnext[2], dnext[3]};
                const bool dcur_ok = dnext_ok;
                #pragma unroll
                for (int q = 0; q < 4; q++) {
                    dnext[q] = dnext2[q];
                    dnext2[q] = dnext3[q];
                }
                dnext_ok = dnext2_ok;
                dnext2_ok = dnext3_ok;
                if (dpre && c0 + 48 < cend) dnext3_ok = dload(c0 + 48, dnext3);
                float v[16];
                tmem_ld16(tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(a * QN + c0), v);
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
                if (g.epilogue == 2) {   // C = D - A B, D a row-major split pair
                    if (dcur_ok) {
                        #pragma unroll
                        for (int h = 0; h < 2; h++) {
                            const uint32_t wa[4] = {dcur[h].x, dcur[h].y, dcur[h].z, dcur[h].w};
                            const uint32_t wb[4] = {dcur[2 + h].x, dcur[2 + h].y, dcur[2 + h].z, dcur[2 + h].w};
                            #pragma unroll
                            for (int u = 0; u < 8; u++) {
                                const float xh = __uint_as_float((wa[u / 2] >> (16 * (u & 1))) << 16);
                                const float xl = __uint_as_float((wb[u / 2] >> (16 * (u & 1))) << 16);
                                v[8 * h + u] = (xh + xl) - v[8 * h + u];
                            }
                        }
                    } else {
                        const __nv_bfloat16 *dh = g.Dhi + (size_t)bz * g.sD + (size_t)r * g.ldd + c;
                        const __nv_bfloat16 *dl = g.Dlo + (size_t)bz * g.sD + (size_t)r * g.ldd + c;
                        #pragma unroll
                        for (int q = 0; q < 16; q++)
                            v[q] = (c + q < g.N ? __bfloat162float(dh[q]) + __bfloat162float(dl[q]) : 0.f) - v[q];
                    }
                }
                if (g.out_mode == 0) {           // transposed split pair
                    #pragma unroll
                    for (int q = 0; q < 16; q++) {
                        if (c + q < g.N) {
                            const __nv_bfloat16 h = __float2bfloat16_rn(v[q]);
                            Ch[(size_t)(c + q) * g.ldc + r] = h;
                            Cl[(size_t)(c + q) * g.ldc + r] = __float2bfloat16_rn(v[q] - __bfloat162float(h));
                        }
                    }
                } else if (g.out_mode == 1) {    // row-major split pair
                    uint32_t wh[8], wl[8];
                    #pragma unroll
                    for (int q = 0; q < 16; q += 2) {
                        const __nv_bfloat16 h0 = __float2bfloat16_rn(v[q]), h1 = __float2bfloat16_rn(v[q + 1]);
                        const __nv_bfloat16 l0 = __float2bfloat16_rn(v[q] - __bfloat162float(h0));
                        const __nv_bfloat16 l1 = __float2bfloat16_rn(v[q + 1] - __bfloat162float(h1));
                        wh[q / 2] = (uint32_t)__bfloat16_as_ushort(h0) | ((uint32_t)__bfloat16_as_ushort(h1) << 16);
                        wl[q / 2] = (uint32_t)__bfloat16_as_ushort(l0) | ((uint32_t)__bfloat16_as_ushort(l1) << 16);
                    }
                    __nv_bfloat16 *ph = Ch + (size_t)r * g.ldc + c, *pl = Cl + (size_t)r * g.ldc + c;
                    if (c + 15 < g.N && ((reinterpret_cast<uintptr_t>(ph) | reinterpret_cast<uintptr_t>(pl)) & 15) == 0) {
                        #pragma unroll
                        for (int q = 0; q < 8; q += 4) {
                            *reinterpret_cast<uint4 *>(ph + 2 * q) = make_uint4(wh[q], wh[q + 1], wh[q + 2], wh[q + 3]);
                            *reinterpret_cast<uint4 *>(pl + 2 * q) = make_uint4(wl[q], wl[q + 1], wl[q + 2], wl[q + 3]);
                        }
                    } else {
                        #pragma unroll
                        for (int q = 0; q < 16; q++)
                            if (c + q < g.N) {
                                ph[q] = __ushort_as_bfloat16((unsigned short)(wh[q / 2] >> (16 * (q & 1))));
                                pl[q] = __ushort_as_bfloat16((unsigned short)(wl[q / 2] >> (16 * (q & 1))));
                            }
                    }
                } else {                         // row-major FP32
                    float *pf = g.Cf + (size_t)bz * g.sC + (size_t)r * g.ldc + c;
                    if (c + 15 < g.N && (reinterpret_cast<uintptr_t>(pf) & 15) == 0) {
                        #pragma unroll
                        for (int q = 0; q < 16; q += 4)
                            *reinterpret_cast<float4 *>(pf + q) = make_float4(v[q], v[q + 1], v[q + 2], v[q + 3]);
                    } else {
                        #pragma unroll
                        for (int q = 0; q < 16; q++)
                            if (c + q < g.N) pf[q] = v[q];
                    }
                }
                if (fuse) {   // psi_a[r] += F'[r][q] m_a(0)[q] over the chunk's 8 complex columns
                    const float *mc = mw + ((c0 - cbeg) >> 1);   // zero past the last column
                    #pragma unroll
                    for (int b9 = 0; b9 < 9; b9++) {
                        const float4 x = *reinterpret_cast<const float4 *>(mc + b9 * (QN / 4));
                        const float4 y = *reinterpret_cast<const float4 *>(mc + b9 * (QN / 4) + 4);
                        const float m[8] = {x.x, x.y, x.z, x.w, y.x, y.y, y.z, y.w};
                        #pragma unroll
                        for (int u = 0; u < 8; u++) {
                            pr[b9] = fmaf(v[2 * u], m[u], pr[b9]);
                            pi[b9] = fmaf(v[2 * u + 1], m[u], pi[b9]);
                        }
                    }
                }
            }
            if (fuse) {   // the row's six terms (k_tcf's combination): a warp's 32 rows summed in FP32
                          // (GB300's FP64 shuffles and adds would stall the epilogue), added in FP64
                float t6[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
                if (r < g.M) {
                    const float *mtp = g.tcf_mt + (size_t)bz * g.tcf_smt;
                    float cm[9];
                    #pragma unroll
                    for (int b9 = 0; b9 < 9; b9++) cm[b9] = mtp[(size_t)b9 * g.tcf_ldv + r];
                    const float ii_r = cm[3] * pr[3] + cm[4] * pr[4] + cm[5] * pr[5];
                    const float ii_i = cm[3] * pi[3] + cm[4] * pi[4] + cm[5] * pi[5];
                    const float ij_r = cm[6] * pr[6] + cm[7] * pr[7] + cm[8] * pr[8];
                    const float ij_i = cm[6] * pi[6] + cm[7] * pi[7] + cm[8] * pi[8];
                    const float jj_r = (cm[4] + cm[5]) * pr[3] + (cm[3] + cm[5]) * pr[4] + (cm[3] + cm[4]) * pr[5];
                    const float jj_i = (cm[4] + cm[5]) * pi[3] + (cm[3] + cm[5]) * pi[4] + (cm[3] + cm[4]) * pi[5];
                    t6[0] = cm[0] * pr[0] + cm[1] * pr[1] + cm[2] * pr[2];
                    t6[1] = cm[0] * pi[0] + cm[1] * pi[1] + cm[2] * pi[2];
                    t6[2] = (3.f * ii_r + jj_r + 4.f * ij_r) * (1.f / 15.f);
                    t6[3] = (3.f * ii_i + jj_i + 4.f * ij_i) * (1.f / 15.f);
                    t6[4] = (2.f * ii_r - jj_r + 6.f * ij_r) * (1.f / 30.f);
                    t6[5] = (2.f * ii_i - jj_i + 6.f * ij_i) * (1.f / 30.f);
                }
                float ws[6];
                #pragma unroll
                for (int q = 0; q < 6; q++) ws[q] = warp_sum(t6[q]);
                if (lane == 0) {
                    #pragma unroll
                    for (int q = 0; q < 6; q++) atomicAdd(&tred[a][q], (double)ws[q]);
                    __threadfence_block();
                    if (atomicAdd(&tcnt[a], 1) == PEW - 1) {   // the tile's last epilogue warp
                        __threadfence_block();
                        #pragma unroll
                        for (int q = 0; q < 6; q++) {   // every other warp's add precedes its count
                            volatile double *slot = &tred[a][q];
                            const double tot = *slot;
                            *slot = 0.0;
                            atomicAdd(g.tcf_out + (size_t)bz * g.tcf_sout + q, tot);
                        }
                        atomicExch(&tcnt[a], 0);
                    }
                }
            }
            // the accumulator (and tred[a]) is free for tile i + 2 once every warp is done
            fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&tempty[a]);
        }
    }
    fence_before();
    __syncthreads();
    if (warp == 1) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * QN));
    }
}

// Vc = V and Vr = V^T as BF16 hi/lo pairs; V column-major (V[k][i] at A[i*ld + k]).
// 64 x 64 tiles through shared memory, block (32, 8): a thread reads two adjacent values
// (8 bytes) and stores each output as a pair of BF16 (4 bytes); values past n are zero.
__global__ void __launch_bounds__(256) k_split_v(const float *A, int ld, long long sA, int n, SplitMat Vc, SplitMat Vr,
                                                 int ldh, long long sV) {
    __shared__ float t[64][65];
    const int b = blockIdx.z;
    const int i0 = blockIdx.y * 64, k0 = blockIdx.x * 64;
    const float *a = A + (size_t)b * sA;
    const size_t ob = (size_t)b * sV;
    auto store2 = [](__nv_bfloat16 *hi, __nv_bfloat16 *lo, float x0, float x1) {
        const __nv_bfloat162 h = __floats2bfloat162_rn(x0, x1);
        *reinterpret_cast<__nv_bfloat162 *>(hi) = h;
        *reinterpret_cast<__nv_bfloat162 *>(lo) =
            __floats2bfloat162_rn(x0 - __bfloat162float(h.x), x1 - __bfloat162float(h.y));
    };
    const int kx = k0 + 2 * threadIdx.x;
    for (int y = threadIdx.y; y < 64; y += 8) {
        const int i = i0 + y;
        float2 x = make_float2(0.f, 0.f);
        if (i < n && kx < n) {
            x = *reinterpret_cast<const float2 *>(a + (size_t)i * ld + kx);   // ld and kx even
            if (kx + 1 >= n) x.y = 0.f;
            store2(Vc.hi + ob + (size_t)i * ldh + kx, Vc.lo + ob + (size_t)i * ldh + kx, x.x, x.y);
        }
        t[y][2 * threadIdx.x] = x.x;
        t[y][2 * threadIdx.x + 1] = x.y;
    }
    __syncthreads();
    const int ix = i0 + 2 * threadIdx.x;
    for (int y = threadIdx.y; y < 64; y += 8) {
        const int k = k0 + y;                           // Vr[k][i] = V[k][i] = A[i*ld + k]
        if (k < n && ix < n)
            store2(Vr.hi + ob + (size_t)k * ldh + ix, Vr.lo + ob + (size_t)k * ldh + ix, t[2 * threadIdx.x][y],
                   ix + 1 < n ? t[2 * threadIdx.x + 1][y] : 0.f);
    }
}

// Ft = I: F[r][c] = 1 for c = 2r (the real part of the diagonal), stored at Ft[c*ldh + r].
__global__ void k_identity_t(SplitMat F, int n, int ldh, long long sF) {
    const size_t ob = (size_t)blockIdx.y * sF;
    const int c = blockIdx.x;
    const __nv_bfloat16 one = __float2bfloat16_rn(1.f), zero = __float2bfloat16_rn(0.f);
    for (int r = threadIdx.x; r < ldh; r += blockDim.x) {
        F.hi[ob + (size_t)c * ldh + r] = (c == 2 * r) ? one : zero;
        F.lo[ob + (size_t)c * ldh + r] = zero;
    }
}

}  // namespace

size_t cir_split_ld(int n) { return (size_t)((n + 7) & ~7); }

template <int QK, int QS, int QN>
static cudaError_t launch_split(const SplitMaps &maps, const SplitGemmArgs &g, int batch, cudaStream_t s) {
    constexpr size_t smem = QCfg<QK, QS, QN>::SMEM;
    cudaError_t e = cudaFuncSetAttribute(k_tc_split<QK, QS, QN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grid((g.N + QN - 1) / QN, (g.M + QM - 1) / QM, batch);
    k_tc_split<QK, QS, QN><<<grid, QT, smem, s>>>(maps, g);
    return cudaGetLastError();
}

// streaming multiprocessors of the current device (looked up once per device)
static int sm_count() {
    static int cache[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 148;
    if (!cache[dev]) {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n < 1) n = 148;
        cache[dev] = n;
    }
    return cache[dev];
}

// The persistent propagation kernel, unless CIR_SPLIT_PERSIST=0 (the one-tile-per-CTA kernel).
static bool persist_enabled() {
    static const bool on = [] {
        const char *v = getenv("CIR_SPLIT_PERSIST");
        return !(v && v[0] == '0');
    }();
    return on;
}

// cuTensorMapEncodeTiled from the driver, looked up once
static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

// Tensor map of one K-major BF16 operand: x = K (contiguous), y = rows (stride ld), z = matrix
// (stride sb); boxes of 64 x 128 x 1 in the 128-byte swizzle, zero fill outside.
static bool make_map(CUtensorMap *m, const __nv_bfloat16 *base, int K, int rows, int ld, long long sb, int batch, int QK,
                     int box_rows) {
    auto fn = encode_fn();
    if (!fn) return false;
    const cuuint64_t dim[3] = {(cuuint64_t)K, (cuuint64_t)rows, (cuuint64_t)batch};
    const cuuint64_t stride[2] = {(cuuint64_t)ld * 2, (cuuint64_t)sb * 2};
    const cuuint32_t box[3] = {(cuuint32_t)QK, (cuuint32_t)box_rows, 1};
    const cuuint32_t es[3] = {1, 1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<__nv_bfloat16 *>(base), dim, stride, box, es,
              CU_TENSOR_MAP_INTERLEAVE_NONE, QK == 64 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
              CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// checks of one split-BF16 problem
static bool split_ok(const SplitGemmArgs &g, int batch) {
    if (batch < 1 || batch > 65535 || g.M < 1 || g.N < 1 || g.K < 1 || (g.epilogue == 1 && (g.N & 1))) return false;
    if ((g.lda & 7) || (g.ldb & 7) || (g.sA & 7) || (g.sB & 7) || g.lda < g.K || g.ldb < g.K) return false;
    if ((long long)g.lda * g.M > g.sA && batch > 1) return false;
    if ((long long)g.ldb * g.N > g.sB && batch > 1) return false;
    for (const void *p : {(const void *)g.Ahi, (const void *)g.Alo, (const void *)g.Bhi, (const void *)g.Blo})
        if (reinterpret_cast<uintptr_t>(p) & 15) return false;
    return true;
}

// the tile width a problem takes by itself
static int split_width(const SplitGemmArgs &g) {
    constexpr int QK = 32;
    if (g.tile_n == 128 || g.tile_n == 256) return g.tile_n;
    // 128 x 256 tiles for the wide products (the propagation) and the back-transform updates
    // (C = D - A B): a quarter less operand traffic per flop
    return ((g.N >= 1024 && g.K > 4 * QK) || (g.epilogue == 2 && g.N >= 256)) ? 256 : 128;
}

static bool split_maps(const SplitGemmArgs &g, int batch, int qn, SplitMaps &maps) {
    constexpr int QK = 32;
    const long long sA = batch > 1 ? g.sA : (long long)g.lda * g.M, sB = batch > 1 ? g.sB : (long long)g.ldb * g.N;
    return make_map(&maps.a_hi, g.Ahi, g.K, g.M, g.lda, sA, batch, QK, QM) &&
           make_map(&maps.a_lo, g.Alo, g.K, g.M, g.lda, sA, batch, QK, QM) &&
           make_map(&maps.b_hi, g.Bhi, g.K, g.N, g.ldb, sB, batch, QK, qn) &&
           make_map(&maps.b_lo, g.Blo, g.K, g.N, g.ldb, sB, batch, QK, qn);
}

// One persistent launch over np problems (the tiles of problem 0 first), all in tiles of width qn.
static cudaError_t launch_persist(const SplitGemmArgs *g, const int *batch, int np, int qn, cudaStream_t s,
                                  int *launches) {
    constexpr int QK = 32;
    PersistPlan plan;
    memset(&plan, 0, sizeof plan);
    plan.np = np;
    long long ntl = 0;
    for (int i = 0; i < np; i++) {
        if (!split_maps(g[i], batch[i], qn, plan.maps[i])) return cudaErrorInvalidValue;
        plan.g[i] = g[i];
        plan.tiles_n[i] = (g[i].N + qn - 1) / qn;
        plan.tiles_mn[i] = plan.tiles_n[i] * ((g[i].M + QM - 1) / QM);
        plan.first[i] = (int)ntl;
        ntl += (long long)plan.tiles_mn[i] * batch[i];
        if (ntl > INT32_MAX) return cudaErrorInvalidValue;
    }
    plan.first[np] = (int)ntl;
    const int grid = (int)std::min<long long>(ntl, sm_count());
    auto go = [&](auto kern, size_t smem) -> cudaError_t {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        kern<<<grid, PT, smem, s>>>(plan);
        return cudaGetLastError();
    };
    const cudaError_t e = qn == 256 ? go(k_tc_persist<QK, 4, 256>, QCfg<QK, 4, 256>::SMEM)
                                    : go(k_tc_persist<QK, 6, 128>, QCfg<QK, 6, 128>::SMEM);
    if (e == cudaSuccess && launches) *launches += 1;
    return e;
}

cudaError_t cir_launch_split_gemm_multi(const SplitGemmArgs *g, const int *batch, int np, cudaStream_t s,
                                        int *launches) {
    if (np < 1 || np > CIR_SPLIT_MAXP) return cudaErrorInvalidValue;
    int qn = 0;
    for (int i = 0; i < np; i++) {
        if (!split_ok(g[i], batch[i]) || g[i].bz0 != 0) return cudaErrorInvalidValue;
        qn = std::max(qn, split_width(g[i]));
    }
    return launch_persist(g, batch, np, qn, s, launches);
}

cudaError_t cir_launch_split_gemm(const SplitGemmArgs &g, int batch, cudaStream_t s, int *launches) {
    if (!split_ok(g, batch)) return cudaErrorInvalidValue;
    constexpr int QK = 32;   // 64-byte swizzle; 3 x 32 KB stages (two CTAs per SM), or for
                             // products of at most 4 K slices 2 stages (three CTAs per SM)
    const int qn = split_width(g);
    SplitMaps maps;
    if (!split_maps(g, batch, qn, maps)) return cudaErrorInvalidValue;
    const long long sB = batch > 1 ? g.sB : (long long)g.ldb * g.N;
    // persistent warp-specialised CTAs (one per SM), the epilogue of one tile overlapping the
    // loads and MMAs of the next: 128 x 256 tiles in a 4-stage ring for the propagation,
    // 128 x 128 tiles in a 6-stage ring otherwise
    if (g.bz0 == 0 && persist_enabled()) {
        const long long ntl = (long long)((g.N + qn - 1) / qn) * ((g.M + QM - 1) / QM) * batch;
        if (ntl <= INT32_MAX) return launch_persist(&g, &batch, 1, qn, s, launches);
    }
    if (qn == 256) {
        // Wave quantisation: two 128 x 256 CTAs per SM.  When the last wave of the batch would
        // hold less than half the slots, the batch entries that fill whole waves run in this
        // shape and the rest in 128 x 64 tiles (four times the CTAs, a quarter of the work each,
        // three per SM), so the tail costs about a quarter of a wave instead of a whole one.
        const long long per = (long long)((g.N + 255) / 256) * ((g.M + QM - 1) / QM);
        const long long slots = 2LL * sm_count();
        const long long waves = per * batch / slots, rem = per * batch - waves * slots;
        const int bmain = waves >= 1 ? (int)(waves * slots / per) : 0;
        if (rem > 0 && 2 * rem < slots && bmain >= 1 && bmain < batch) {
            SplitMaps tail = maps;
            if (!make_map(&tail.b_hi, g.Bhi, g.K, g.N, g.ldb, sB, batch, QK, 64) ||
                !make_map(&tail.b_lo, g.Blo, g.K, g.N, g.ldb, sB, batch, QK, 64))
                return cudaErrorInvalidValue;
            cudaError_t e = launch_split<QK, 2, 256>(maps, g, bmain, s);
            if (e != cudaSuccess) return e;
            SplitGemmArgs gt = g;
            gt.bz0 = g.bz0 + bmain;
            if ((e = launch_split<QK, 3, 64>(tail, gt, batch - bmain, s)) != cudaSuccess) return e;
            if (launches) *launches += 2;
            return cudaSuccess;
        }
    }
    const cudaError_t e = qn == 256 ? launch_split<QK, 2, 256>(maps, g, batch, s)
                        : g.K <= 4 * QK ? launch_split<QK, 2, 128>(maps, g, batch, s)
                                        : launch_split<QK, 3, 128>(maps, g, batch, s);
    if (e != cudaSuccess) return e;
    if (launches) *launches += 1;
    return cudaSuccess;
}

cudaError_t cir_launch_split_v(const float *A, int ld, long long sA, int n, SplitMat Vc, SplitMat Vr, int ldh,
                               long long sV, int batch, cudaStream_t s, int *launches) {
    if ((ld & 1) || (ldh & 1) || (sA & 1) || (sV & 1) || (reinterpret_cast<uintptr_t>(A) & 7))
        return cudaErrorInvalidValue;
    dim3 grid((n + 63) / 64, (n + 63) / 64, batch);
    k_split_v<<<grid, dim3(32, 8), 0, s>>>(A, ld, sA, n, Vc, Vr, ldh, sV);
    if (launches) *launches += 1;
    return cudaGetLastError();
}

cudaError_t cir_launch_identity_t(SplitMat F, int n, int ldh, long long sF, int batch, cudaStream_t s, int *launches) {
    k_identity_t<<<dim3(2 * n, batch), 256, 0, s>>>(F, n, ldh, sF);
    if (launches) *launches += 1;
    return cudaGetLastError();
}
