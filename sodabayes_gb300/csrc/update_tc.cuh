// update_tc.cuh — tensor-core residual update of one subset for FP8 mode with
// several chains (models.f90:164-174 for every chain at once), included by
// sweep.cu after rhs_tc.cuh.
//
//   r  += X_b delta = sum_j x0_j delta_j + G_b (delta / sd)
//   ra += U_b delta
//
// Row tiles of r (128 individuals, one CTA each) run on tcgen05: A = the
// tile's codes of 64 subset positions per stage, transposed to individual-major
// bf16 in tensor memory (lane = individual, written with tcgen05.st), B = the
// three-way bf16 split of delta/sd written by the draws (k_draw), D = 128 x
// 3*chains FP32 in tensor memory.  Stages whose 64 positions have no
// non-zero delta in any chain are skipped.  The pipeline is the one of
// k_rhs_tc: warp 8 loads each stage's code tile and delta-split tile by TMA
// (both 128-byte swizzled; the MMA reads the delta split straight from the
// raw buffer), warps 0-7 gather and convert the codes, warp 9 issues the
// MMAs.  The centring term sum_j x0_j delta_j is added in FP64 from the
// per-CTA sums of the draws.  The augmented rows ra (U_b is FP32; a tile of
// 128 rows is split over column ranges, D.atab giving wider tiles more CTAs)
// run on the FP32 cores; the last CTA of a row tile adds the split partial
// sums in split order (deterministic).
#pragma once

namespace soda {

constexpr int TU_KC = 64;          // subset positions per stage
constexpr int TU_NS = 6;           // raw stages in flight
constexpr int TU_MAXQ = 256;       // stages per subset (subsets up to 16384 SNPs)
constexpr int TU_RA_SPLIT = 8;     // ra-update CTAs per 128-row tile, on average
constexpr int TU_UNR = 8;          // U columns in flight per warp
constexpr int TU_THREADS = 320;    // 8 converter warps, the TMA warp, the MMA warp
constexpr int TU_CONV = 256;
constexpr int TU_WARP_TMA = 8, TU_WARP_MMA = 9;

template <int CT>
struct UpdTc {
    static constexpr int NB = RhsTc<CT>::NB;
    static constexpr int RAW_A = TU_KC * 128;          // codes: 64 positions x 128 individuals (TMA, swizzled)
    static constexpr int RAW_B = NB * TU_KC * 2;       // bf16 split of delta/sd (TMA, swizzled; MMA operand B)
    static constexpr int RAW = RAW_A + RAW_B;
    static constexpr int PIPE = TU_NS * RAW;           // (the codes operand lives in tensor memory)
    static constexpr int RED = 4 * CT * 128 * 4;       // column-group partials of the ra tiles
    static constexpr size_t SMEM = 1024 + (size_t)(PIPE > RED ? PIPE : RED);
    static_assert(RAW % 1024 == 0 && RAW_A % 1024 == 0, "buffers must keep 1024-byte alignment");
};

template <int CT>
__device__ __forceinline__ void update_tc_rows(const CUtensorMap *tm_codes, const CUtensorMap *tm_d, const Dev &D,
                                               int b, unsigned char *base)
{
    using T = UpdTc<CT>;
    constexpr int NB = T::NB;
    constexpr int NW = TU_THREADS / 32;
    __shared__ uint64_t s_full[TU_NS], s_empty[TU_NS], s_conv[2], s_opfree[2], s_done;
    __shared__ uint32_t s_tmem;
    __shared__ int s_err, s_nact, s_wcnt[NW + 1];
    __shared__ int s_act[TU_MAXQ];
    __shared__ double s_k0[CT];
    __shared__ double s_k0p[TU_CONV];
    __shared__ double s_rsw[8][CT];
    unsigned char *raw0 = base;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int ls = D.blk_ls[b];
    const int N = D.blk_ls[b + 1] - ls;
    const int tile = blockIdx.x, t0 = tile * 128;
    const int nq = (N + TU_KC - 1) / TU_KC;
    tc::pdl_trigger();
    tc::pdl_wait();   // the draws of this subset are complete

    // stages with a non-zero delta, in subset order (nq <= 256)
    {
        bool f = false;
        if (tid < nq) {
            const int jb = tid * TU_KC, e = min(N, jb + TU_KC);
            if (e - jb == TU_KC) {   // full stage: four 16-byte loads
                const uint4 *q = reinterpret_cast<const uint4 *>(D.nzflag + jb);
                const uint4 a = q[0], bq = q[1], c2 = q[2], d2 = q[3];
                f = ((a.x | a.y | a.z | a.w) | (bq.x | bq.y | bq.z | bq.w) | (c2.x | c2.y | c2.z | c2.w) |
                     (d2.x | d2.y | d2.z | d2.w)) != 0u;
            } else {
                uint32_t o = 0;
                for (int jk = jb; jk < e; ++jk) o |= D.nzflag[jk];
                f = o != 0u;
            }
        }
        const unsigned m = __ballot_sync(0xffffffffu, f);
        if (lane == 0) s_wcnt[warp] = __popc(m);
        // the centring term: 256/CT threads per chain over interleaved draw CTAs, then in part order
        constexpr int PARTS = TU_CONV / CT;
        if (tid < TU_CONV) {
            const int c = tid / PARTS, part = tid % PARTS;
            const int ntl = (((N + TC_TM - 1) / TC_TM) * TC_TM * CT + 255) / 256;
            double a = 0.0;
            for (int q0 = part; q0 < ntl; q0 += 8 * PARTS) {
                double v[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    const int q = q0 + u * PARTS;
                    v[u] = q < ntl ? D.k0part[(size_t)q * CT + c] : 0.0;
                }
#pragma unroll
                for (int u = 0; u < 8; ++u) a += v[u];
            }
            s_k0p[tid] = a;
        }
        __syncthreads();
        if (tid == 0) {
            int acc = 0;
            for (int q = 0; q < NW; ++q) {
                const int t = s_wcnt[q];
                s_wcnt[q] = acc;
                acc += t;
            }
            s_nact = acc;
        }
        if (tid < CT) {
            double t = 0.0;
            for (int q = 0; q < PARTS; ++q) t += s_k0p[tid * PARTS + q];
            s_k0[tid] = t;
        }
        __syncthreads();
        if (f) s_act[s_wcnt[warp] + __popc(m & ((1u << lane) - 1u))] = tid;
        __syncthreads();
    }
    const int nact = s_nact;
    if (nact == 0) return;   // nothing changed: r, r32 and rsum stay valid

    if (tid == 0) {
        for (int i = 0; i < TU_NS; ++i) {
            tc::mbar_init(&s_full[i], 1);
            tc::mbar_init(&s_empty[i], TU_CONV + 1);   // converters + the MMAs reading the delta split
        }
        for (int i = 0; i < 2; ++i) {
            tc::mbar_init(&s_conv[i], TU_CONV);
            tc::mbar_init(&s_opfree[i], 1);
        }
        tc::mbar_init(&s_done, 1);
        tc::mbar_fence_init();
        s_err = 0;
    }
    if (warp == TU_WARP_MMA) tc::tmem_alloc(&s_tmem, 128);   // accumulator 0-63, codes operand 64-127
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tm = s_tmem;

    if (warp == TU_WARP_TMA) {
        if (lane == 0) {
            tc::tma_prefetch_desc(tm_codes);
            tc::tma_prefetch_desc(tm_d);
            for (int s = 0; s < nact; ++s) {
                const int buf = s % TU_NS;
                if (s >= TU_NS && !tc::mbar_wait(&s_empty[buf], ((s / TU_NS) - 1) & 1)) {
                    s_err = 1;
                    break;
                }
                unsigned char *rw = raw0 + (size_t)buf * T::RAW;
                const int k0 = s_act[s] * TU_KC;
                tc::mbar_expect_tx(&s_full[buf], T::RAW);
                tc::tma_load_2d(rw, tm_codes, t0, ls + k0, &s_full[buf]);
                tc::tma_load_2d(rw + T::RAW_A, tm_d, k0, 0, &s_full[buf]);
            }
        }
    } else if (warp == TU_WARP_MMA) {
        if (lane == 0) {
            const uint32_t idesc = tc::idesc_bf16(128, NB);
            for (int s = 0; s < nact; ++s) {
                const int ob = s & 1, buf = s % TU_NS;
                if (!tc::mbar_wait(&s_conv[ob], (s >> 1) & 1)) {
                    s_err = 1;
                    break;
                }
                tc::fence_after_sync();
                const uint32_t ta = tm + 64 + 32 * ob;
                const uint32_t b0 = tc::smem_u32(raw0 + (size_t)buf * T::RAW + T::RAW_A);
#pragma unroll
                for (int kk = 0; kk < TU_KC / 16; ++kk)
                    tc::mma_bf16_ta(tm, ta + 8 * kk, tc::desc_sw128(b0 + kk * 32, 1024), idesc, (s | kk) != 0 ? 1u : 0u);
                tc::mma_commit(&s_opfree[ob]);
                tc::mma_commit(&s_empty[buf]);
            }
            tc::mma_commit(&s_done);
        }
    } else {
        // converters: warp w writes tensor-memory lanes 32*(w%4).. (individuals), positions 32*(w/4) ..
        // +31 of the stage (16 columns): a thread gathers its individual's byte from 32 rows of the
        // 128-byte-swizzled code tile (a warp reads 32 consecutive bytes of one row at a time)
        const int ind = 32 * (warp & 3) + lane, kh = warp >> 2;
        for (int s = 0; s < nact; ++s) {
            const int buf = s % TU_NS, ob = s & 1;
            bool ok = tc::mbar_wait(&s_full[buf], (s / TU_NS) & 1);
            if (ok && s >= 2) ok = tc::mbar_wait(&s_opfree[ob], ((s - 2) >> 1) & 1);
            if (!ok) {
                s_err = 1;
                break;
            }
            const unsigned char *ra_ = raw0 + (size_t)buf * T::RAW;
            uint32_t v[16];
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const int k = 32 * kh + 2 * j;
                const uint32_t c0 = ra_[k * 128 + ((((ind >> 4) ^ (k & 7))) << 4) + (ind & 15)];
                const uint32_t c1 = ra_[(k + 1) * 128 + ((((ind >> 4) ^ ((k + 1) & 7))) << 4) + (ind & 15)];
                v[j] = tc::bf16x2_sub128(c0 | (c1 << 16) | 0x43004300u);
            }
            tc::tmem_st16(tm + ((uint32_t)(32 * (warp & 3)) << 16) + 64 + 32 * ob + 16 * kh, v);
            tc::tmem_wait_st();
            tc::fence_before_sync();
            tc::mbar_arrive(&s_conv[ob]);
            tc::mbar_arrive(&s_empty[buf]);
        }
        if (!tc::mbar_wait(&s_done, 0)) s_err = 1;
    }
    __syncthreads();
    const bool ok = !s_err;
    if (!ok && tid == 0) flag_err(D, 4);
    tc::fence_after_sync();
    // epilogue: warps w and w+4 read the same 32 accumulator rows, each for half of the chains
    constexpr int HALF = CT >= 8 ? CT / 2 : CT;
    const int h = warp >> 2;
    if (warp < 8 && h * HALF < CT) {
        const int i = t0 + (warp & 3) * 32 + lane;
        const bool row_ok = i < D.n;
        double rv[HALF];
#pragma unroll
        for (int c = 0; c < HALF; ++c) rv[c] = row_ok ? D.r[(size_t)(h * HALF + c) * D.ldr + i] : 0.0;
#pragma unroll
        for (int g = 0; g < (HALF + 7) / 8; ++g) {
            // chains h*HALF + 8g ..: their hi, mid and lo accumulator columns
            float hi[8], md[8], lo[8];
            const uint32_t ta = tm + ((uint32_t)((warp & 3) * 32) << 16) + h * HALF + 8 * g;
            tc::tmem_ld8(ta, hi);
            tc::tmem_ld8(ta + CT, md);
            tc::tmem_ld8(ta + 2 * CT, lo);
            tc::tmem_wait_ld();
#pragma unroll
            for (int e = 0; e < 8; ++e) {
                const int cl = 8 * g + e;
                if (cl < HALF && ok && row_ok) rv[cl] += (double)((hi[e] + md[e]) + lo[e]) + s_k0[h * HALF + cl];
            }
        }
        if (ok && row_ok) {
#pragma unroll
            for (int c = 0; c < HALF; ++c) store_r(D, h * HALF + c, i, rv[c]);
        }
#pragma unroll
        for (int c = 0; c < HALF; ++c) {
            const double v = warp_sum(rv[c]);
            if (lane == 0) s_rsw[warp][c] = v;
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == TU_WARP_MMA) {
        tc::fence_after_sync();
        tc::tmem_dealloc(tm, 128);
    }
    // this tile's partial sum of r (the centring of the next subset)
    if (tid < CT) {
        const int hh = tid / HALF, cl = tid % HALF;
        D.rsum[(size_t)tid * D.nr_ctas + tile] =
            ((s_rsw[4 * hh][cl] + s_rsw[4 * hh + 1][cl]) + s_rsw[4 * hh + 2][cl]) + s_rsw[4 * hh + 3][cl];
    }
}

template <int CT>
__device__ __forceinline__ void update_tc_ra(const Dev &D, int b, unsigned char *base)
{
    __shared__ int s_last;
    float *s_red = reinterpret_cast<float *>(base);   // [4 column groups][CT][128 rows]
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    tc::pdl_trigger();
    tc::pdl_wait();   // the draws of this subset are complete
    const int ls = D.blk_ls[b];
    const int N = D.blk_ls[b + 1] - ls;
    const int npad = (N + 7) & ~7;
    // this CTA's row tile and column split (tiles get splits in proportion to their width)
    const int idx = blockIdx.x - D.nr_ctas;
    const int32_t *at = D.atab + (size_t)b * D.tstride;
    const int ntr = (N + 127) / 128;
    int tr = 0;
    while (tr + 1 < ntr && at[tr + 1] <= idx) ++tr;
    const int ra_split = at[tr + 1] - at[tr], sp = idx - at[tr];
    const int i0 = tr * 128;
    const int kbeg = D.blk_pd[b] ? min(i0, N) : 0;   // upper triangular: rows i only meet columns k >= i
    const int ka = kbeg + (int)(((long long)(N - kbeg) * sp) / ra_split);
    const int kb = kbeg + (int)(((long long)(N - kbeg) * (sp + 1)) / ra_split);
    // warp w of 8: rows i0 + 64*(w&1) + 2*lane (+1), columns ka + (w>>1) + 4q; the TMA/MMA warps idle here
    const int rh = warp & 1, cg = warp >> 1;
    const int ii = i0 + 64 * rh + 2 * lane;
    const bool rows_ok = ii + 2 <= npad;
    float acc[2][CT];
#pragma unroll
    for (int e = 0; e < 2; ++e)
#pragma unroll
        for (int c = 0; c < CT; ++c) acc[e][c] = 0.0f;
    for (int k0 = ka + cg; warp < 8 && k0 < kb; k0 += 4 * TU_UNR) {
        float2 u[TU_UNR];
        int kk[TU_UNR];
#pragma unroll
        for (int q = 0; q < TU_UNR; ++q) {
            const int k = k0 + 4 * q;
            kk[q] = (k < kb && D.nzflag[k]) ? k : -1;
            u[q] = make_float2(0.f, 0.f);
            if (kk[q] >= 0 && rows_ok) u[q] = *reinterpret_cast<const float2 *>(D.U32 + D.uoff[ls + k] + ii);
        }
#pragma unroll
        for (int q = 0; q < TU_UNR; ++q) {
            if (kk[q] < 0) continue;
#pragma unroll
            for (int c = 0; c < CT; c += 4) {
                const float4 v = *reinterpret_cast<const float4 *>(D.delta32 + (size_t)kk[q] * CT + c);
                acc[0][c] = fmaf(u[q].x, v.x, acc[0][c]);
                acc[1][c] = fmaf(u[q].y, v.x, acc[1][c]);
                acc[0][c + 1] = fmaf(u[q].x, v.y, acc[0][c + 1]);
                acc[1][c + 1] = fmaf(u[q].y, v.y, acc[1][c + 1]);
                acc[0][c + 2] = fmaf(u[q].x, v.z, acc[0][c + 2]);
                acc[1][c + 2] = fmaf(u[q].y, v.z, acc[1][c + 2]);
                acc[0][c + 3] = fmaf(u[q].x, v.w, acc[0][c + 3]);
                acc[1][c + 3] = fmaf(u[q].y, v.w, acc[1][c + 3]);
            }
        }
    }
    if (warp < 8) {
#pragma unroll
        for (int c = 0; c < CT; ++c) {
            s_red[(cg * CT + c) * 128 + 64 * rh + 2 * lane] = acc[0][c];
            s_red[(cg * CT + c) * 128 + 64 * rh + 2 * lane + 1] = acc[1][c];
        }
    }
    __syncthreads();
    float *part = D.rapart + ((size_t)idx * CT) * 128;
    for (int t = tid; t < CT * 128; t += TU_THREADS) {
        const int c = t >> 7, rl = t & 127;
        part[c * 128 + rl] = ((s_red[(0 * CT + c) * 128 + rl] + s_red[(1 * CT + c) * 128 + rl]) +
                              s_red[(2 * CT + c) * 128 + rl]) + s_red[(3 * CT + c) * 128 + rl];
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) s_last = atomicAdd(&D.raticket[tr], 1) == ra_split - 1;
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    // the last CTA of the row tile: split partial sums in split order
    const float *p0 = D.rapart + ((size_t)at[tr] * CT) * 128;
    for (int t = tid; t < CT * 128; t += TU_THREADS) {
        const int c = t >> 7, rl = t & 127, i = i0 + rl;
        if (i >= D.bs) continue;
        float sum = 0.0f;
        for (int q0 = 0; q0 < ra_split; q0 += 8) {
            float pv[8];
#pragma unroll
            for (int q = 0; q < 8; ++q)
                pv[q] = q0 + q < ra_split ? __ldcg(p0 + ((size_t)(q0 + q) * CT + c) * 128 + rl) : 0.0f;
#pragma unroll
            for (int q = 0; q < 8; ++q)
                if (q0 + q < ra_split) sum += pv[q];
        }
        store_ra(D, c, i, D.ra[(size_t)c * D.ldra + i] + (double)sum);
    }
    if (tid == 0) D.raticket[tr] = 0;
}

template <int CT>
__global__ void __launch_bounds__(TU_THREADS, 2)
    k_update_tc(const __grid_constant__ CUtensorMap tm_codes, const __grid_constant__ CUtensorMap tm_d, Dev D, int b)
{
    extern __shared__ __align__(1024) unsigned char smem_dyn[];
    unsigned char *base = smem_dyn + ((1024u - (tc::smem_u32(smem_dyn) & 1023u)) & 1023u);
    if ((int)blockIdx.x < D.nr_ctas) update_tc_rows<CT>(&tm_codes, &tm_d, D, b, base);
    else update_tc_ra<CT>(D, b, base);
}

}  // namespace soda
