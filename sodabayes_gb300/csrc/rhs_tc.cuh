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
// one M tile and one K split of 128-individual stages; per stage, cp.async
// brings the tile's codes (XOR-swizzled 16-byte chunks, conflict-free reads)
// and the chains' FP32 residuals into a raw buffer, the CTA converts them into
// a double-buffered 128-byte-swizzled operand buffer, and one thread issues
// eight K=16 MMAs whose completion an mbarrier reports when the operand buffer
// is needed again.  The augmenting part u_j' ra_c (5% of the work) runs on
// the FP32 cores.  Partial sums, the ticket and the draws are those of
// rhs_finish; the last CTA of a tile also leaves the bf16 split of delta/sd
// for the tensor-core update.
#pragma once

namespace soda {

constexpr int TC_TM = 128;   // SNPs per M tile
constexpr int TC_KC = 128;   // individuals per stage
constexpr int TC_NS = 4;     // raw stages in flight
constexpr int TC_UW = 1024;  // augmented rows per ra staging window

template <int CT>
struct RhsTc {
    static constexpr int NB = ((3 * CT + 15) / 16) * 16;   // MMA N: hi, mid, lo per chain
    static constexpr int RAW_A = TC_TM * TC_KC;            // codes
    static constexpr int RAW_B = CT * TC_KC * 4;           // FP32 residuals
    static constexpr int RAW = RAW_A + RAW_B;
    static constexpr int OP_A = TC_TM * TC_KC * 2;         // bf16 codes, two 64-wide K regions
    static constexpr int OP_B = NB * TC_KC * 2;
    static constexpr int OP = OP_A + OP_B;
    static constexpr size_t SMEM = 1024 + 2 * (size_t)OP + (size_t)TC_NS * RAW;
    static_assert(OP % 1024 == 0, "operand buffers must keep 1024-byte alignment");
    static_assert((size_t)CT * TC_UW * 4 <= (size_t)TC_NS * RAW, "ra window must fit the raw buffers");
    static_assert((size_t)TC_TM * CT * 4 <= 2 * (size_t)OP, "u partials must fit the operand buffers");
};

template <int CT>
__global__ void __launch_bounds__(256, 1) k_rhs_tc(Dev D, int b, int ksplit)
{
    using T = RhsTc<CT>;
    constexpr int NB = T::NB;
    extern __shared__ __align__(1024) unsigned char smem_dyn[];
    __shared__ uint64_t s_bar[2];
    __shared__ uint32_t s_tmem;
    __shared__ int s_err;
    unsigned char *base = smem_dyn + ((1024u - (tc::smem_u32(smem_dyn) & 1023u)) & 1023u);
    unsigned char *op0 = base;
    unsigned char *raw0 = base + 2 * T::OP;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int ls = D.blk_ls[b];
    const int N = D.blk_ls[b + 1] - ls;
    const int mt = blockIdx.x / ksplit, ks = blockIdx.x % ksplit;
    const int j0 = mt * TC_TM;
    if (j0 >= N) return;
    const int nG = D.ldx / TC_KC;
    const int c0 = (int)(((long long)nG * ks) / ksplit), c1 = (int)(((long long)nG * (ks + 1)) / ksplit);
    const int nck = c1 - c0;

    // padding rows of B (n >= 3*CT) stay zero in both operand buffers
    if constexpr (NB > 3 * CT) {
        for (int t = tid; t < 2 * (NB - 3 * CT) * (TC_KC / 8); t += 256) {
            const int ob = t / ((NB - 3 * CT) * (TC_KC / 8)), r = t % ((NB - 3 * CT) * (TC_KC / 8));
            const int n = 3 * CT + r / (TC_KC / 8), q = r % (TC_KC / 8);
            *reinterpret_cast<uint4 *>(op0 + ob * T::OP + T::OP_A + tc::sw128_off(n, 8 * q, NB)) =
                make_uint4(0, 0, 0, 0);
        }
    }
    if (tid == 0) {
        tc::mbar_init(&s_bar[0], 1);
        tc::mbar_init(&s_bar[1], 1);
        tc::mbar_fence_init();
        s_err = 0;
    }
    if (warp == 0) tc::tmem_alloc(&s_tmem, 64);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tm = s_tmem;

    auto issue = [&](int s, int buf) {
        unsigned char *ra_ = raw0 + (size_t)buf * T::RAW;
        const int i0 = (c0 + s) * TC_KC;
        for (int t = tid; t < TC_TM * 8; t += 256) {   // codes: 128 SNPs x 8 chunks of 16
            const int m = t >> 3, ch = t & 7;
            unsigned char *dst = ra_ + m * 128 + ((ch ^ (m & 7)) << 4);
            const int jk = j0 + m;
            if (jk < N) __pipeline_memcpy_async(dst, D.G + (size_t)(ls + jk) * D.ldx + i0 + ch * 16, 16);
            else *reinterpret_cast<uint4 *>(dst) = make_uint4(0, 0, 0, 0);
        }
        for (int t = tid; t < CT * 32; t += 256) {     // residuals: CT rows of 128 floats
            const int c = t >> 5, ch = t & 31;
            __pipeline_memcpy_async(ra_ + T::RAW_A + c * 512 + ch * 16, D.r32 + (size_t)c * D.ldr + i0 + ch * 4, 16);
        }
        __pipeline_commit();
    };

#pragma unroll
    for (int pp = 0; pp < TC_NS - 1; ++pp) {
        if (pp < nck) issue(pp, pp);
        else __pipeline_commit();
    }
    const uint32_t idesc = tc::idesc_bf16(TC_TM, NB);
    for (int s = 0; s < nck; ++s) {
        if (s + TC_NS - 1 < nck) issue(s + TC_NS - 1, (s + TC_NS - 1) % TC_NS);
        else __pipeline_commit();
        __pipeline_wait_prior(TC_NS - 1);
        const int ob = s & 1;
        // the operand buffer was last read by the MMAs of stage s-2
        if (s >= 2 && !tc::mbar_wait(&s_bar[ob], ((s - 2) >> 1) & 1)) s_err = 1;
        __syncthreads();
        const unsigned char *ra_ = raw0 + (size_t)(s % TC_NS) * T::RAW;
        unsigned char *opa = op0 + ob * T::OP;
        unsigned char *opb = opa + T::OP_A;
        // codes -> bf16: a warp converts 4 SNP rows x 8 chunks of 16 codes
#pragma unroll
        for (int it = 0; it < TC_TM * 8 / 256; ++it) {
            const int t = tid + 256 * it;
            const int m = t >> 3, ch = t & 7;
            const uint4 w = *reinterpret_cast<const uint4 *>(ra_ + m * 128 + ((ch ^ (m & 7)) << 4));
            uint4 lo, hi;
            tc::codes_to_bf16x4(w.x, lo.x, lo.y);
            tc::codes_to_bf16x4(w.y, lo.z, lo.w);
            tc::codes_to_bf16x4(w.z, hi.x, hi.y);
            tc::codes_to_bf16x4(w.w, hi.z, hi.w);
            *reinterpret_cast<uint4 *>(opa + tc::sw128_off(m, 16 * ch, TC_TM)) = lo;
            *reinterpret_cast<uint4 *>(opa + tc::sw128_off(m, 16 * ch + 8, TC_TM)) = hi;
        }
        // residuals -> three bf16 rows per chain
        for (int t = tid; t < CT * (TC_KC / 8); t += 256) {
            const int c = t / (TC_KC / 8), q = t % (TC_KC / 8);
            const float4 a = *reinterpret_cast<const float4 *>(ra_ + T::RAW_A + c * 512 + q * 32);
            const float4 bq = *reinterpret_cast<const float4 *>(ra_ + T::RAW_A + c * 512 + q * 32 + 16);
            const float v[8] = {a.x, a.y, a.z, a.w, bq.x, bq.y, bq.z, bq.w};
            uint32_t h[8], md[8], l[8];
#pragma unroll
            for (int e = 0; e < 8; ++e) tc::split3(v[e], h[e], md[e], l[e]);
            *reinterpret_cast<uint4 *>(opb + tc::sw128_off(c, 8 * q, NB)) =
                make_uint4(h[0] | h[1] << 16, h[2] | h[3] << 16, h[4] | h[5] << 16, h[6] | h[7] << 16);
            *reinterpret_cast<uint4 *>(opb + tc::sw128_off(CT + c, 8 * q, NB)) =
                make_uint4(md[0] | md[1] << 16, md[2] | md[3] << 16, md[4] | md[5] << 16, md[6] | md[7] << 16);
            *reinterpret_cast<uint4 *>(opb + tc::sw128_off(2 * CT + c, 8 * q, NB)) =
                make_uint4(l[0] | l[1] << 16, l[2] | l[3] << 16, l[4] | l[5] << 16, l[6] | l[7] << 16);
        }
        tc::fence_async_smem();
        __syncthreads();
        if (tid == 0 && !s_err) {
            tc::fence_after_sync();
            const uint32_t a0 = tc::smem_u32(opa), b0 = tc::smem_u32(opb);
#pragma unroll
            for (int kk = 0; kk < TC_KC / 16; ++kk) {
                const uint32_t ka = (kk >> 2) * (TC_TM * 128) + (kk & 3) * 32;
                const uint32_t kb = (kk >> 2) * (NB * 128) + (kk & 3) * 32;
                tc::mma_bf16(tm, tc::desc_sw128(a0 + ka, 1024), tc::desc_sw128(b0 + kb, 1024), idesc,
                             (s | kk) != 0 ? 1u : 0u);
            }
            tc::mma_commit(&s_bar[ob]);
        }
    }
    __pipeline_wait_prior(0);
    bool have = nck > 0;
    if (have) {
        const int last = nck - 1;
        if (!tc::mbar_wait(&s_bar[last & 1], (last >> 1) & 1)) s_err = 1;
    }
    __syncthreads();
    if (s_err) {
        have = false;
        if (tid == 0) flag_err(D, 4);
    }
    tc::fence_after_sync();
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
        if (jk < N) {
#pragma unroll
            for (int c = 0; c < CT; ++c)
                D.rpx[((size_t)ks * CT + c) * D.bs + jk] = (double)((acc[c] + acc[CT + c]) + acc[2 * CT + c]);
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        tc::fence_after_sync();
        tc::tmem_dealloc(tm, 64);
    }

    // augmenting part on the FP32 cores: this split's share of the U rows of
    // the tile's columns (upper triangular: rows up to the tile's last column)
    const int npad = (N + 7) & ~7;
    const int rowsU = D.blk_pd[b] ? min(npad, j0 + TC_TM) : npad;
    const int nUc = (rowsU + 31) / 32;
    const int l0 = 32 * (int)(((long long)nUc * ks) / ksplit);
    const int l1 = min(rowsU, 32 * (int)(((long long)nUc * (ks + 1)) / ksplit));
    float *s_u = reinterpret_cast<float *>(op0);     // [TC_TM][CT] partial u'ra
    float *s_ra = reinterpret_cast<float *>(raw0);   // [CT][TC_UW] window of ra
    for (int t = tid; t < TC_TM * CT; t += 256) s_u[t] = 0.0f;
    for (int w0 = l0; w0 < l1; w0 += TC_UW) {
        const int len = min(TC_UW, l1 - w0);
        __syncthreads();
        for (int t = tid; t < CT * len; t += 256) {
            const int c = t / len, l = t % len;
            s_ra[c * TC_UW + l] = D.ra32[(size_t)c * D.ldra + w0 + l];
        }
        __syncthreads();
        // warp w: tile columns 16w .. 16w+15, four at a time; lanes over rows
#pragma unroll 1
        for (int g = 0; g < 4; ++g) {
            const int jq = warp * 16 + g * 4;
            float acc[4][CT];
#pragma unroll
            for (int q = 0; q < 4; ++q)
#pragma unroll
                for (int c = 0; c < CT; ++c) acc[q][c] = 0.0f;
            const float *ucol[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int jk = j0 + jq + q;
                ucol[q] = jk < N ? D.U32 + D.uoff[ls + jk] + w0 : nullptr;
            }
            for (int l = lane; l < len; l += 32) {
                float u[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) u[q] = ucol[q] ? ucol[q][l] : 0.0f;
#pragma unroll
                for (int c = 0; c < CT; ++c) {
                    const float rv = s_ra[c * TC_UW + l];
#pragma unroll
                    for (int q = 0; q < 4; ++q) acc[q][c] = fmaf(u[q], rv, acc[q][c]);
                }
            }
#pragma unroll
            for (int q = 0; q < 4; ++q)
#pragma unroll
                for (int c = 0; c < CT; ++c) {
                    const float v = warp_sumf(acc[q][c]);
                    if (lane == 0) s_u[(jq + q) * CT + c] += v;
                }
        }
    }
    __syncthreads();
    for (int t = tid; t < TC_TM * CT; t += 256) {
        const int m = t / CT, c = t % CT, jk = j0 + m;
        if (jk < N) D.rpu[((size_t)ks * CT + c) * D.bs + jk] = (double)s_u[t];
    }
    rhs_finish<SODAGPU_FP8, CT, true>(D, b, mt, ksplit, j0, TC_TM);
}

}  // namespace soda
