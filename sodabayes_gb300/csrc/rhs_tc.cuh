// rhs_tc.cuh — tensor-core right-hand sides of one SODA subset for FP8 mode
// with several chains (models.f90:154 for every chain at once), included by
// sweep.cu after rhs_kernel.cuh.
//
//   rhs[j][c] = x_j' r_c + u_j' ra_c,   x_j = x0_j + code_j / sd_j
//
// The genotype part G_b' R (M = 128 SNPs per tile, N = chains, K =
// individuals) runs on tcgen05: codes 0/1/2 are exact in bf16, and each FP32
// residual column is split into three bf16 terms (hi + mid + lo carry about
// 24 significant bits), so one MMA of N = 3 * chains (padded to 16) gives
// FP32-accurate products with FP32 accumulation in tensor memory.  A CTA owns
// one M tile and one K split of 128-individual stages and runs a
// warp-specialised pipeline synchronised by mbarriers:
//   warp 16 (one thread) TMA: the stage's 128 x 128 code tile (hardware
//           128-byte swizzle) and the chains' 128 residuals into a raw buffer
//           (TC_NS buffers in flight);
//   warps 0-15 convert the raw buffer into the double-buffered bf16 operands
//           (codes: tensor memory, lane = SNP, written with tcgen05.st;
//           residual hi/mid/lo rows: shared memory) and release both;
//   warp 17 (one thread) issues the eight K=16 MMAs of the stage and commits
//           their completion, which frees the operand buffer.
// With programmatic dependent launch the prologue (barriers, tensor memory,
// the first code tiles) overlaps the previous kernel; residuals are read
// after it completes.
// The augmenting part u_j' ra_c (5% of the work) then runs on the FP32 cores
// from staged windows of U.  Partial sums go to rpx/rpu (as FP32), added and
// drawn by k_draw.
#pragma once
#include <cuda.h>

namespace soda {

constexpr int TC_TM = 128;       // SNPs per M tile
constexpr int TC_KC = 128;       // individuals per stage
constexpr int TC_NS = 6;         // raw stages in flight
constexpr int TC_THREADS = 576;  // 16 converter warps, the TMA warp, the MMA warp
constexpr int TC_CONV = 512;     // converter threads
constexpr int TC_WARP_TMA = 16, TC_WARP_MMA = 17;

template <int CT>
struct RhsTc {
    static constexpr int NB = ((3 * CT + 15) / 16) * 16;   // MMA N: hi, mid, lo per chain
    static constexpr int RAW_A = TC_TM * TC_KC;            // codes (TMA box 128 x 128, 128-byte swizzle)
    static constexpr int RAW_B = CT * TC_KC * 4;           // FP32 residuals (TMA box 128 x CT)
    static constexpr int RAW = RAW_A + RAW_B;
    static constexpr int OP_B = NB * TC_KC * 2;            // bf16 residual split, two 64-wide K regions
    static constexpr int OP = OP_B;                        // (the codes operand lives in tensor memory)
    static constexpr size_t SMEM = 1024 + 2 * (size_t)OP + (size_t)TC_NS * RAW;
    static_assert(OP % 1024 == 0 && RAW % 1024 == 0, "operand and raw buffers must keep 1024-byte alignment");
    // U part: a window of UWR rows of the tile's 128 U columns and the chains' ra, plus the partial sums
    static constexpr size_t PIPE = 2 * (size_t)OP + (size_t)TC_NS * RAW;
    static constexpr size_t upart(int rows) { return (size_t)(TC_TM + CT) * rows * 4 + (size_t)TC_TM * CT * 4; }
    static constexpr int UWR = upart(256) <= PIPE ? 256 : (upart(192) <= PIPE ? 192 : 128);
    static_assert(upart(UWR) <= PIPE, "U window must fit the pipeline buffers");
};

// Transposing butterfly: V values per lane summed over the warp's 32 lanes.
// Each round with CNT > 1 exchanges half of the values with lane ^ OFF and
// keeps the other half (upper half when lane & OFF); once one value is left
// the remaining rounds add it across lanes.  Afterwards a lane holds the
// totals of values xreduce_base(lane) + 0 .. FIN-1 (FIN = V/32, or 1 with
// V < 32, where lanes differing in the low bits hold the same totals).
template <int CNT, int OFF, int V>
__device__ __forceinline__ void xreduce_round(float (&v)[V], int lane)
{
    if constexpr (OFF >= 1) {
        if constexpr (CNT > 1) {
            constexpr int H = CNT / 2;
            const bool up = (lane & OFF) != 0;
#pragma unroll
            for (int i = 0; i < H; ++i) {
                const float send = up ? v[i] : v[i + H];
                const float keep = up ? v[i + H] : v[i];
                v[i] = keep + __shfl_xor_sync(0xffffffffu, send, OFF);
            }
            xreduce_round<H, OFF / 2, V>(v, lane);
        } else {
            v[0] += __shfl_xor_sync(0xffffffffu, v[0], OFF);
            xreduce_round<1, OFF / 2, V>(v, lane);
        }
    }
}

template <int V>
__device__ __forceinline__ int xreduce_base(int lane)
{
    int base = 0, cnt = V;
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) {
        if (cnt > 1) {
            cnt >>= 1;
            if (lane & off) base += cnt;
        }
    }
    return base;
}

template <int CT>
__global__ void __launch_bounds__(TC_THREADS, 1)
    k_rhs_tc(const __grid_constant__ CUtensorMap tm_codes, const __grid_constant__ CUtensorMap tm_r, Dev D, int b)
{
    using T = RhsTc<CT>;
    constexpr int NB = T::NB;
    extern __shared__ __align__(1024) unsigned char smem_dyn[];
    __shared__ uint64_t s_full[TC_NS], s_empty[TC_NS], s_conv[2], s_opfree[2], s_done;
    __shared__ uint32_t s_tmem;
    __shared__ int s_err;
    unsigned char *base = smem_dyn + ((1024u - (tc::smem_u32(smem_dyn) & 1023u)) & 1023u);
    unsigned char *op0 = base;
    unsigned char *raw0 = base + 2 * T::OP;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int ls = D.blk_ls[b];
    const int N = D.blk_ls[b + 1] - ls;
    // this CTA's SNP tile and K split (tiles get splits in proportion to their work)
    const int32_t *rt = D.rtab + (size_t)b * D.tstride;
    const int mtiles = (N + TC_TM - 1) / TC_TM;
    int mt = 0;
    while (mt + 1 < mtiles && rt[mt + 1] <= (int)blockIdx.x) ++mt;
    const int ksplit = rt[mt + 1] - rt[mt], ks = (int)blockIdx.x - rt[mt];
    const int j0 = mt * TC_TM;
    if (j0 >= N || ks >= ksplit) return;
    const int nG = D.ldx / TC_KC;
    const int c0 = (int)(((long long)nG * ks) / ksplit), c1 = (int)(((long long)nG * (ks + 1)) / ksplit);
    const int nck = c1 - c0;

    // padding rows of B (n >= 3*CT) stay zero in both operand buffers
    if constexpr (NB > 3 * CT) {
        for (int t = tid; t < 2 * (NB - 3 * CT) * (TC_KC / 8); t += TC_THREADS) {
            const int ob = t / ((NB - 3 * CT) * (TC_KC / 8)), r = t % ((NB - 3 * CT) * (TC_KC / 8));
            const int n = 3 * CT + r / (TC_KC / 8), q = r % (TC_KC / 8);
            *reinterpret_cast<uint4 *>(op0 + ob * T::OP + tc::sw128_off(n, 8 * q, NB)) = make_uint4(0, 0, 0, 0);
        }
    }
    if (tid == 0) {
        for (int i = 0; i < TC_NS; ++i) {
            tc::mbar_init(&s_full[i], 1);
            tc::mbar_init(&s_empty[i], TC_CONV);
        }
        for (int i = 0; i < 2; ++i) {
            tc::mbar_init(&s_conv[i], TC_CONV);
            tc::mbar_init(&s_opfree[i], 1);
        }
        tc::mbar_init(&s_done, 1);
        tc::mbar_fence_init();
        s_err = 0;
    }
    if (warp == TC_WARP_MMA) tc::tmem_alloc(&s_tmem, 256);   // accumulator 0-63, codes operand 64-191
    tc::pdl_trigger();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tm = s_tmem;

    if (warp == TC_WARP_TMA) {
        if (lane == 0) {
            tc::tma_prefetch_desc(&tm_codes);
            tc::tma_prefetch_desc(&tm_r);
            // the first code tiles do not depend on the previous kernel
            const int pre = nck < TC_NS ? nck : TC_NS;
            for (int s = 0; s < pre; ++s) {
                tc::mbar_expect_tx(&s_full[s], T::RAW);
                tc::tma_load_2d(raw0 + (size_t)s * T::RAW, &tm_codes, (c0 + s) * TC_KC, ls + j0, &s_full[s]);
            }
            tc::pdl_wait();
            for (int s = 0; s < pre; ++s)
                tc::tma_load_2d(raw0 + (size_t)s * T::RAW + T::RAW_A, &tm_r, (c0 + s) * TC_KC, 0, &s_full[s]);
            for (int s = pre; s < nck; ++s) {
                const int buf = s % TC_NS;
                // the buffer's previous stage has been converted
                if (!tc::mbar_wait(&s_empty[buf], ((s / TC_NS) - 1) & 1)) {
                    s_err = 1;
                    break;
                }
                unsigned char *rw = raw0 + (size_t)buf * T::RAW;
                const int i0 = (c0 + s) * TC_KC;
                tc::mbar_expect_tx(&s_full[buf], T::RAW);
                tc::tma_load_2d(rw, &tm_codes, i0, ls + j0, &s_full[buf]);
                tc::tma_load_2d(rw + T::RAW_A, &tm_r, i0, 0, &s_full[buf]);
            }
        } else {
            tc::pdl_wait();
        }
    } else if (warp == TC_WARP_MMA) {
        tc::pdl_wait();
        if (lane == 0 && nck > 0) {
            const uint32_t idesc = tc::idesc_bf16(TC_TM, NB);
            for (int s = 0; s < nck; ++s) {
                const int ob = s & 1;
                if (!tc::mbar_wait(&s_conv[ob], (s >> 1) & 1)) {
                    s_err = 1;
                    break;
                }
                tc::fence_after_sync();
                const uint32_t ta = tm + 64 + 64 * ob, b0 = tc::smem_u32(op0 + ob * T::OP);
#pragma unroll
                for (int kk = 0; kk < TC_KC / 16; ++kk) {
                    const uint32_t kb = (kk >> 2) * (NB * 128) + (kk & 3) * 32;
                    tc::mma_bf16_ta(tm, ta + 8 * kk, tc::desc_sw128(b0 + kb, 1024), idesc, (s | kk) != 0 ? 1u : 0u);
                }
                tc::mma_commit(&s_opfree[ob]);
            }
            tc::mma_commit(&s_done);
        }
    } else {
        tc::pdl_wait();
        // converters: raw stage -> bf16 operand tiles
        for (int s = 0; s < nck; ++s) {
            const int buf = s % TC_NS, ob = s & 1;
            bool ok = tc::mbar_wait(&s_full[buf], (s / TC_NS) & 1);
            // the operand buffer was last read by the MMAs of stage s-2
            if (ok && s >= 2) ok = tc::mbar_wait(&s_opfree[ob], ((s - 2) >> 1) & 1);
            if (!ok) {
                s_err = 1;
                break;
            }
            const unsigned char *ra_ = raw0 + (size_t)buf * T::RAW;
            unsigned char *opb = op0 + ob * T::OP;
            // codes -> tensor memory: warp w writes lanes 32*(w%4).. (SNP rows), 32 codes of K
            // (columns 16*(w/4) .. +15 of the stage's operand block)
            {
                const int m = 32 * (warp & 3) + lane, s4 = warp >> 2;
                const uint4 wa = *reinterpret_cast<const uint4 *>(ra_ + m * 128 + (((2 * s4) ^ (m & 7)) << 4));
                const uint4 wb = *reinterpret_cast<const uint4 *>(ra_ + m * 128 + (((2 * s4 + 1) ^ (m & 7)) << 4));
                uint32_t v[16];
                tc::codes_to_bf16x4(wa.x, v[0], v[1]);
                tc::codes_to_bf16x4(wa.y, v[2], v[3]);
                tc::codes_to_bf16x4(wa.z, v[4], v[5]);
                tc::codes_to_bf16x4(wa.w, v[6], v[7]);
                tc::codes_to_bf16x4(wb.x, v[8], v[9]);
                tc::codes_to_bf16x4(wb.y, v[10], v[11]);
                tc::codes_to_bf16x4(wb.z, v[12], v[13]);
                tc::codes_to_bf16x4(wb.w, v[14], v[15]);
                tc::tmem_st16(tm + ((uint32_t)(32 * (warp & 3)) << 16) + 64 + 64 * ob + 16 * s4, v);
            }
            // residuals -> three bf16 rows per chain
            for (int t = tid; t < CT * (TC_KC / 8); t += TC_CONV) {
                const int c = t / (TC_KC / 8), q = t % (TC_KC / 8);
                const float4 a = *reinterpret_cast<const float4 *>(ra_ + T::RAW_A + c * 512 + q * 32);
                const float4 bq = *reinterpret_cast<const float4 *>(ra_ + T::RAW_A + c * 512 + q * 32 + 16);
                uint4 h, md, l;
                tc::split3x2(a.x, a.y, h.x, md.x, l.x);
                tc::split3x2(a.z, a.w, h.y, md.y, l.y);
                tc::split3x2(bq.x, bq.y, h.z, md.z, l.z);
                tc::split3x2(bq.z, bq.w, h.w, md.w, l.w);
                *reinterpret_cast<uint4 *>(opb + tc::sw128_off(c, 8 * q, NB)) = h;
                *reinterpret_cast<uint4 *>(opb + tc::sw128_off(CT + c, 8 * q, NB)) = md;
                *reinterpret_cast<uint4 *>(opb + tc::sw128_off(2 * CT + c, 8 * q, NB)) = l;
            }
            tc::tmem_wait_st();
            tc::fence_async_smem();
            tc::fence_before_sync();
            tc::mbar_arrive(&s_conv[ob]);
            tc::mbar_arrive(&s_empty[buf]);
        }
        if (nck > 0 && !tc::mbar_wait(&s_done, 0)) s_err = 1;
    }
    __syncthreads();
    tc::fence_after_sync();
    const bool have = nck > 0 && !s_err;
    if (s_err && tid == 0) flag_err(D, 4);
    // genotype partial sums: row m of the accumulator (tensor-memory lane m)
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
        if (jk < N) {   // FP32 partial sums (the accumulators are FP32)
            float *px32 = reinterpret_cast<float *>(D.rpx);
#pragma unroll
            for (int c = 0; c < CT; ++c) px32[((size_t)ks * CT + c) * D.bs + jk] = (acc[c] + acc[CT + c]) + acc[2 * CT + c];
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == TC_WARP_MMA) {
        tc::fence_after_sync();
        tc::tmem_dealloc(tm, 256);
    }

    // augmenting part on the FP32 cores: this split's share of the U rows of
    // the tile's columns (upper triangular: rows up to the tile's last
    // column), staged by windows of UWR rows with cp.async; converter warp
    // w owns 8 columns (four at a time), lanes run over rows, and the 4 x CT
    // lane sums are reduced by a transposing butterfly.
    const int npad = (N + 7) & ~7;
    const int rowsU = D.blk_pd[b] ? min(npad, j0 + TC_TM) : npad;
    const int nUc = (rowsU + 31) / 32;
    const int l0 = 32 * (int)(((long long)nUc * ks) / ksplit);
    const int l1 = min(rowsU, 32 * (int)(((long long)nUc * (ks + 1)) / ksplit));
    float *sU = reinterpret_cast<float *>(base);      // [TC_TM][T::UWR]
    float *sRa = sU + TC_TM * T::UWR;                 // [CT][T::UWR]
    float *s_u = sRa + CT * T::UWR;                   // [TC_TM][CT]
    for (int t = tid; t < TC_TM * CT; t += TC_THREADS) s_u[t] = 0.0f;
    for (int w0 = l0; w0 < l1; w0 += T::UWR) {
        const int len = min(T::UWR, l1 - w0);        // a multiple of 8
        __syncthreads();
        for (int t = tid; t < TC_TM * (len / 4); t += TC_THREADS) {
            const int jj = t / (len / 4), q = t % (len / 4);
            const int jk = j0 + jj;
            float *dst = sU + jj * T::UWR + 4 * q;
            if (jk < N) __pipeline_memcpy_async(dst, D.U32 + D.uoff[ls + jk] + w0 + 4 * q, 16);
            else *reinterpret_cast<float4 *>(dst) = make_float4(0.f, 0.f, 0.f, 0.f);
        }
        for (int t = tid; t < CT * (len / 4); t += TC_THREADS) {
            const int c = t / (len / 4), q = t % (len / 4);
            __pipeline_memcpy_async(sRa + c * T::UWR + 4 * q, D.ra32 + (size_t)c * D.ldra + w0 + 4 * q, 16);
        }
        __pipeline_commit();
        __pipeline_wait_prior(0);
        __syncthreads();
#pragma unroll 1
        for (int g = 0; g < (warp < TC_CONV / 32 ? TC_TM / (4 * (TC_CONV / 32)) : 0); ++g) {
            const int jq = warp * (TC_TM / (TC_CONV / 32)) + g * 4;
            float acc[4 * CT];
#pragma unroll
            for (int v = 0; v < 4 * CT; ++v) acc[v] = 0.0f;
            for (int l = lane; l < len; l += 32) {
                float u[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) u[q] = sU[(jq + q) * T::UWR + l];
#pragma unroll
                for (int c = 0; c < CT; ++c) {
                    const float rv = sRa[c * T::UWR + l];
#pragma unroll
                    for (int q = 0; q < 4; ++q) acc[q * CT + c] = fmaf(u[q], rv, acc[q * CT + c]);
                }
            }
            xreduce_round<4 * CT, 16>(acc, lane);
            constexpr int FIN = 4 * CT >= 32 ? 4 * CT / 32 : 1;
            const int vb = xreduce_base<4 * CT>(lane);
            if (4 * CT >= 32 || (lane & (32 / (4 * CT) - 1)) == 0) {
#pragma unroll
                for (int f = 0; f < FIN; ++f) {
                    const int v = vb + f;
                    s_u[(jq + v / CT) * CT + v % CT] += acc[f];
                }
            }
        }
    }
    __syncthreads();
    for (int t = tid; t < TC_TM * CT; t += TC_THREADS) {
        const int m = t / CT, c = t % CT, jk = j0 + m;
        if (jk < N) reinterpret_cast<float *>(D.rpu)[((size_t)ks * CT + c) * D.bs + jk] = s_u[t];
    }
}

}  // namespace soda
