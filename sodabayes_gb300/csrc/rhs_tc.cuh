// rhs_tc.cuh — tensor-core right-hand sides of one SODA subset for FP8 mode
// with several chains (models.f90:154 for every chain at once), included by
// sweep.cu after rhs_kernel.cuh.
//
//   rhs[j][c] = x_j' r_c + u_j' ra_c,   x_j = x0_j + code_j / sd_j
//             = (code_j' r_c + (sd_j u_j)' ra_c) / sd_j + x0_j sum(r_c)
//
// Both products run on tcgen05 into one FP32 accumulator in tensor memory
// (M = 128 SNPs per tile, N = 3 * chains padded to 16):
//   genotype stages (K = 128 individuals): codes 0/1/2 are exact in bf16;
//     B is the bf16 hi/mid/lo split of the FP32 residuals (about 24
//     significant bits), kept in HBM by every kernel that writes r;
//   augmenting stages (K = 64 rows of U): A is one of the three bf16 terms
//     of sd_j u_j (split once when the chains are set up), B the split of ra.
// The centring x0_j sum(r_c) and the scaling by 1/sd_j are applied by the
// draw kernel.  A CTA owns one M tile and a contiguous range of its stages
// (genotype stages first) and runs a warp-specialised pipeline synchronised
// by mbarriers:
//   warp 8 (one thread) TMA: each stage's B tile (the residual split) and,
//           for U stages, its A tile (128 x 64 bf16), 128-byte swizzled, into
//           a raw buffer (NS buffers in flight);
//   warp 10 (one thread) streams each genotype stage's 2-bit packed codes
//           (4 KB) into a ring of shared-memory slots by bulk copy, the first
//           ones before the dependency wait (the codes are written once,
//           before the sweep);
//   warps 0-7 take their 16 bytes (64 codes) of a stage from that ring and
//           widen them into one of four bf16 operands in tensor memory
//           (lane = SNP, tcgen05.st); they take no part in the raw buffers'
//           hand-offs;
//   warp 9 runs the issue loop on warp-uniform values and one elected lane
//           issues the stage's MMAs (A from tensor memory or, for U stages,
//           from the raw buffer; B always from the raw buffer) once the
//           operands are in place, and commits their completion, which frees
//           the buffers.
// With programmatic dependent launch the prologue (barriers, tensor memory,
// the first U tiles, which are constant, and the first code words) overlaps
// the previous kernel; the residual splits are read after it completes.  Each
// thread lets the draw kernel launch only after its own dependency wait, so
// that the draw's prologue may read what the previous residual update wrote.
// The accumulator rows go to rpx as FP32 partial sums, one slot per K split,
// added by k_draw.
#pragma once
#include <cuda.h>

namespace soda {

constexpr int TC_TM = 128;       // SNPs per M tile
constexpr int TC_KC = 128;       // individuals per genotype stage
constexpr int TC_KU = 64;        // U rows per augmenting stage
constexpr int TC_THREADS = 352;  // 8 converter warps, the TMA warp, the MMA warp, the code loader
constexpr int TC_CONV = 256;     // converter threads
constexpr int TC_CONV_WARPS = TC_CONV / 32;   // each converter warp arrives once per stage
constexpr int TC_NOB = 4;        // bf16 codes operands in tensor memory (converters run up to 4 stages ahead)
constexpr int TC_NC = 6;         // shared-memory slots of packed codes (4 KB: one genotype stage each)
constexpr int TC_WARP_TMA = 8, TC_WARP_MMA = 9, TC_WARP_CODES = 10;

template <int CT>
struct RhsTc {
    static constexpr int NB = ((3 * CT + 15) / 16) * 16;   // MMA N: hi, mid, lo per chain
    static constexpr int RAW_A = TC_TM * TC_KU * 2;        // U box 128 x 64 bf16 (U stages)
    static constexpr int RAW_B = NB * TC_KC * 2;           // residual split: two 64-wide K regions
    static constexpr int RAW = RAW_A + RAW_B;
    static constexpr uint32_t TX_G = RAW_B;                // bytes a genotype stage loads
    static constexpr uint32_t TX_U = RAW_A + NB * TC_KU * 2;   // bytes an augmenting stage loads
    static constexpr int CODE = 2 * 64 * 16 * 2;            // packed codes of a stage: 128 SNPs x 128 individuals
    static constexpr int NS_FIT = (220 * 1024 - 1024 - TC_NC * CODE) / RAW;
    static constexpr int NS = NS_FIT > 8 ? 8 : NS_FIT;     // raw buffers in flight
    static constexpr int CODE0 = NS * RAW;
    static constexpr size_t SMEM = 1024 + (size_t)CODE0 + (size_t)TC_NC * CODE;
    static_assert(RAW % 1024 == 0 && (NB * 128) % 1024 == 0, "buffers and K regions must keep 1024-byte alignment");
    static_assert(NS >= 4, "pipeline too shallow");
};

// Stages of tile mt of subset b: the genotype stages, then three per 64 U
// rows (terms hi, mid, lo); upper-triangular factors stop at the tile's last
// column.
__host__ __device__ inline int rhs_tc_stages(int nG, int N, int mt, bool pd, int *nUq)
{
    const int npad = (N + 7) & ~7;
    const int rows = pd ? (npad < TC_TM * (mt + 1) ? npad : TC_TM * (mt + 1)) : npad;
    const int q = (rows + TC_KU - 1) / TC_KU;
    if (nUq) *nUq = q;
    return nG + 3 * q;
}

// First stage of K split ks of ksplit over a tile's T stages (nG genotype
// stages of weight 2, then U stages of weight 1), in equal shares of weight.
__host__ __device__ inline int rhs_tc_split(int nG, int T, int ks, int ksplit)
{
    const long long wt = 2LL * nG + (T - nG);
    const long long x = (wt * ks) / ksplit;
    if (x <= 2LL * nG) return (int)((x + 1) / 2);
    return nG + (int)(x - 2LL * nG);
}

template <int CT>
__global__ void __launch_bounds__(TC_THREADS, 1)
    k_rhs_tc(const __grid_constant__ CUtensorMap tm_rsp, const __grid_constant__ CUtensorMap tm_usp,
             const __grid_constant__ CUtensorMap tm_rasp, Dev D, int b)
{
    using T = RhsTc<CT>;
    constexpr int NB = T::NB, NS = T::NS;
    extern __shared__ __align__(1024) unsigned char smem_dyn[];
    __shared__ uint64_t s_full[NS], s_empty[NS], s_conv[TC_NOB], s_opfree[TC_NOB], s_done;
    __shared__ uint64_t s_cfull[TC_NC], s_cfree[TC_NC];
    __shared__ uint32_t s_tmem;
    __shared__ int s_err;
    unsigned char *raw0 = smem_dyn + ((1024u - (tc::smem_u32(smem_dyn) & 1023u)) & 1023u);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int ls = D.blk_ls[b];
    const int N = D.blk_ls[b + 1] - ls;
    // this CTA's SNP tile and K split: tiles get splits in proportion to their MMAs, and a tile's
    // stages are split in equal shares of MMA work (a genotype stage has twice the MMAs of a U stage)
    const int32_t *rt = D.rtab + (size_t)b * D.tstride;
    const int mtiles = (N + TC_TM - 1) / TC_TM;
    int mt = 0;
    while (mt + 1 < mtiles && rt[mt + 1] <= (int)blockIdx.x) ++mt;
    const int ksplit = rt[mt + 1] - rt[mt], ks = (int)blockIdx.x - rt[mt];
    const int j0 = mt * TC_TM;
    if (j0 >= N || ks >= ksplit) return;
    const int nG = D.ldx / TC_KC;
    const int T_ = rhs_tc_stages(nG, N, mt, D.blk_pd[b] != 0, nullptr);
    const int t0 = rhs_tc_split(nG, T_, ks, ksplit), t1 = rhs_tc_split(nG, T_, ks + 1, ksplit);
    const int ns = t1 - t0;                              // stages of this CTA
    const int nck = max(0, min(t1, nG) - t0);            // of which genotype stages (first)

    if (tid == 0) {
        for (int i = 0; i < NS; ++i) {
            tc::mbar_init(&s_full[i], 1);
            tc::mbar_init(&s_empty[i], 1);   // the MMAs reading B (and a U stage's A)
        }
        for (int i = 0; i < TC_NOB; ++i) {
            tc::mbar_init(&s_conv[i], TC_CONV_WARPS);
            tc::mbar_init(&s_opfree[i], 1);
        }
        tc::mbar_init(&s_done, 1);
        for (int i = 0; i < TC_NC; ++i) {
            tc::mbar_init(&s_cfull[i], 1);                // a stage's packed codes landed
            tc::mbar_init(&s_cfree[i], TC_CONV_WARPS);    // every converter warp has read them
        }
        tc::mbar_fence_init();
        s_err = 0;
    }
    if (warp == TC_WARP_MMA) tc::tmem_alloc(&s_tmem, 512);   // accumulator 0-63, codes operands 64-319
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tm = s_tmem;

    if (warp == TC_WARP_TMA) {
        if (lane == 0) {
            tc::tma_prefetch_desc(&tm_rsp);
            tc::tma_prefetch_desc(&tm_usp);
            tc::tma_prefetch_desc(&tm_rasp);
            // U stages' A tiles do not depend on the previous kernel; B tiles do
            auto load_a = [&](int s) {
                const int t = t0 + s;
                if (t < nG) return;   // genotype stages: the converters load the codes
                unsigned char *rw = raw0 + (size_t)(s % NS) * T::RAW;
                uint64_t *bar = &s_full[s % NS];
                const int u = t - nG;
                tc::mbar_expect_tx(bar, T::TX_U);
                tc::tma_load_2d(rw, &tm_usp, (u / 3) * TC_KU, (u % 3) * D.p + ls + j0, bar);
            };
            auto load_b = [&](int s) {
                const int t = t0 + s;
                unsigned char *rw = raw0 + (size_t)(s % NS) * T::RAW + T::RAW_A;
                uint64_t *bar = &s_full[s % NS];
                if (t < nG) {
                    tc::mbar_expect_tx(bar, T::TX_G);
                    tc::tma_load_2d(rw, &tm_rsp, t * TC_KC, 0, bar);
                    tc::tma_load_2d(rw + NB * 128, &tm_rsp, t * TC_KC + 64, 0, bar);
                } else {
                    tc::tma_load_2d(rw, &tm_rasp, ((t - nG) / 3) * TC_KU, 0, bar);
                }
            };
            const int pre = ns < NS ? ns : NS;
            for (int s = 0; s < pre; ++s) load_a(s);
            tc::pdl_wait();
            tc::pdl_trigger();
            for (int s = 0; s < pre; ++s) load_b(s);
            for (int s = pre; s < ns; ++s) {
                // the buffer's previous stage has been consumed
                if (!tc::mbar_wait(&s_empty[s % NS], ((s / NS) - 1) & 1)) {
                    s_err = 1;
                    break;
                }
                load_a(s);
                load_b(s);
            }
            // no copy may still be in flight into this CTA's shared memory when it exits
            for (int s = max(0, ns - NS); s < ns; ++s)
                if (!tc::mbar_wait(&s_full[s % NS], (s / NS) & 1)) s_err = 1;
        } else {
            tc::pdl_wait();
            tc::pdl_trigger();
        }
    } else if (warp == TC_WARP_MMA) {
        tc::pdl_wait();
        tc::pdl_trigger();
        // the whole warp runs the loop on warp-uniform values; one elected lane issues (its
        // operands stay in uniform registers)
        const bool leader = tc::elect_one();
        if (ns > 0) {
            const uint32_t idesc = tc::idesc_bf16(TC_TM, NB);
            for (int s = 0; s < ns; ++s) {
                const int buf = s % NS;
                const uint32_t rb = tc::smem_u32(raw0 + (size_t)buf * T::RAW);
                if (s < nck) {
                    const int ob = s % TC_NOB;
                    bool ok = tc::mbar_wait(&s_conv[ob], (s / TC_NOB) & 1) && tc::mbar_wait(&s_full[buf], (s / NS) & 1);
                    if (!__all_sync(0xffffffffu, ok)) {
                        s_err = 1;
                        break;
                    }
                    tc::fence_after_sync();
                    const uint32_t ta = tm + 64 + 64 * ob;
                    if (leader) {
#pragma unroll
                        for (int kk = 0; kk < TC_KC / 16; ++kk) {
                            const uint32_t kb = (kk >> 2) * (NB * 128) + (kk & 3) * 32;
                            tc::mma_bf16_ta(tm, ta + 8 * kk, tc::desc_sw128(rb + T::RAW_A + kb, 1024), idesc,
                                            (s | kk) != 0 ? 1u : 0u);
                        }
                        tc::mma_commit(&s_opfree[ob]);
                    }
                } else {
                    if (!__all_sync(0xffffffffu, tc::mbar_wait(&s_full[buf], (s / NS) & 1))) {
                        s_err = 1;
                        break;
                    }
                    tc::fence_after_sync();
                    if (leader) {
#pragma unroll
                        for (int kk = 0; kk < TC_KU / 16; ++kk)
                            tc::mma_bf16(tm, tc::desc_sw128(rb + kk * 32, 1024), tc::desc_sw128(rb + T::RAW_A + kk * 32, 1024),
                                         idesc, (s | kk) != 0 ? 1u : 0u);
                    }
                }
                if (leader) tc::mma_commit(&s_empty[buf]);
                __syncwarp();
            }
            if (leader) tc::mma_commit(&s_done);
        }
    } else if (warp == TC_WARP_CODES) {
        // code loader: one bulk copy (4 KB) of a genotype stage's packed codes per stage into the
        // ring, issued as slots free.  A packed block is [4 groups of 64 individuals][128 positions]
        // [16 bytes]; stage t covers individuals 128 (t % 2) .. of tile t / 2, groups 2 (t % 2) and
        // 2 (t % 2) + 1: one contiguous 4 KB.  The codes are not written by any kernel of the sweep,
        // so the first copies run before the dependency wait.  Bulk copies stream at DRAM rates that
        // per-thread loads of the same bytes do not reach (each SM caps its outstanding loads).
        if (lane == 0) {
            const unsigned char *blk0 = D.gpk + (size_t)(D.qoff[b] + mt) * D.nvt * TC_PACKED_BLOCK;
            int issued = 0;
            for (int s = 0; s < nck; ++s) {
                const int cs = s % TC_NC, t = t0 + s;
                if (s == TC_NC) {
                    // the draw kernel launches once every thread has passed its dependency wait
                    tc::pdl_wait();
                    tc::pdl_trigger();
                }
                if (s >= TC_NC && !tc::mbar_wait(&s_cfree[cs], ((s / TC_NC) - 1) & 1)) {
                    s_err = 1;
                    break;
                }
                tc::mbar_expect_tx(&s_cfull[cs], T::CODE);
                tc::bulk_load(raw0 + T::CODE0 + cs * T::CODE, blk0 + (size_t)(t >> 1) * TC_PACKED_BLOCK + (t & 1) * T::CODE,
                              T::CODE, &s_cfull[cs]);
                issued = s + 1;
            }
            // no copy may still be in flight into this CTA's shared memory when it exits
            for (int s = max(0, issued - TC_NC); s < issued; ++s)
                if (!tc::mbar_wait(&s_cfull[s % TC_NC], (s / TC_NC) & 1)) s_err = 1;
        }
        tc::pdl_wait();
        tc::pdl_trigger();
    } else {
        // converters: thread (SNP m of the tile, individuals 64 g .. 64 g + 63 of each stage) takes
        // 16 bytes of packed codes per genotype stage from the code ring and widens them into one
        // of four bf16 operands in tensor memory (32 columns); they take no part in the raw buffers'
        // hand-offs.  Few, wide converter threads: each stage costs a warp one tensor-memory store,
        // its wait and an arrival, whatever the number of codes it carries.
        const int m = 32 * (warp & 3) + lane, g = warp >> 2;
        const unsigned char *codes0 = raw0 + T::CODE0 + (g * TC_TM + m) * 16;
        tc::pdl_wait();
        tc::pdl_trigger();
        const uint32_t tl = tm + ((uint32_t)(32 * (warp & 3)) << 16) + 64 + 32 * g;
        for (int s = 0; s < nck; ++s) {
            const int ob = s % TC_NOB, cs = s % TC_NC;
            bool ok = tc::mbar_wait(&s_cfull[cs], (s / TC_NC) & 1);
            ok = __all_sync(0xffffffffu, ok);
            if (!ok) {
                s_err = 1;
                break;
            }
            const uint4 w = *reinterpret_cast<const uint4 *>(codes0 + (size_t)cs * T::CODE);
            // the next bulk copy (async proxy) overwrites what these generic loads read: order
            // them first, or the copy can land before the reads (results then vary run to run)
            tc::fence_async_smem();
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(&s_cfree[cs]);   // the slot may be refilled
            // the operand buffer was last read by the MMAs of stage s - TC_NOB
            ok = s < TC_NOB || tc::mbar_wait(&s_opfree[ob], ((s - TC_NOB) / TC_NOB) & 1);
            ok = __all_sync(0xffffffffu, ok);   // the warp arrives as one
            if (!ok) {
                s_err = 1;
                break;
            }
            tc::fence_after_sync();
            uint32_t o[32];
            tc::codes64_to_bf16(w, o);   // individuals of the stage, two per column
            uint32_t lo[16], hi[16];
#pragma unroll
            for (int e = 0; e < 16; ++e) {
                lo[e] = o[e];
                hi[e] = o[16 + e];
            }
            tc::tmem_st16(tl + 64 * ob, lo);
            tc::tmem_st16(tl + 64 * ob + 16, hi);
            tc::tmem_wait_st();
            tc::fence_before_sync();
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(&s_conv[ob]);
        }
        if (ns > 0 && !tc::mbar_wait(&s_done, 0)) s_err = 1;
    }
    __syncthreads();
    tc::fence_after_sync();
    const bool have = ns > 0 && !s_err;
    if (s_err && tid == 0) flag_err(D, 4);
    // partial sums: row m of the accumulator (tensor-memory lane m), hi + mid + lo per chain
    if (warp < 4) {
        const int m = warp * 32 + lane, jk = j0 + m;
        float acc[NB];
#pragma unroll
        for (int g = 0; g < NB / 8; ++g) {
            float v[8];
            if (have) {
                tc::tmem_ld8(tm + ((uint32_t)(warp * 32) << 16) + g * 8, v);
                tc::tmem_wait_ld();
            } else {
#pragma unroll
                for (int e = 0; e < 8; ++e) v[e] = 0.0f;
            }
#pragma unroll
            for (int e = 0; e < 8; ++e) acc[g * 8 + e] = v[e];
        }
        if (jk < N) {
            float *px32 = reinterpret_cast<float *>(D.rpx);
#pragma unroll
            for (int c = 0; c < CT; ++c) px32[((size_t)ks * CT + c) * D.bs + jk] = (acc[c] + acc[CT + c]) + acc[2 * CT + c];
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == TC_WARP_MMA) {
        tc::fence_after_sync();
        tc::tmem_dealloc(tm, 512);
    }
}

}  // namespace soda
