// rhs_kernel.cuh — right-hand sides of one SODA subset (models.f90:154) on
// the FP32/FP64 cores, and the per-SNP draws (models.f90:146-162, 211-256,
// 350-413), included by sweep.cu.
//
//   rhs[j][c] = x_j' r_c + u_j' ra_c (+ d g_j)
//
// is a tall-skinny GEMM: M = the subset's SNPs, N = chains, K = individuals
// followed by the augmented rows.  The grid is (M tiles of 8*SPT SNPs) x
// (K splits), sized to one wave.  Each CTA streams its share of both K
// ranges through shared memory in one NS-stage cp.async pipeline — genotype
// stages (codes or FP32 columns with r) first, then augmenting-matrix stages
// (U columns with ra; the factor is upper triangular, so a tile needs only
// the rows up to its last column) — keeping an SPT x CT accumulator block per
// thread.  Partial sums go to scratch (one slice per K split), which k_draw
// adds in split order before the draws.  FP8 mode: codes 0/1/2 are exact in
// FP32 and the centring is applied once per SNP, x'r = (G'r)/sd - 2p/sd *
// sum(r).
#pragma once
#include <cuda_pipeline_primitives.h>

namespace soda {

template <int MODE>
struct RhsCfg;
template <>
struct RhsCfg<SODAGPU_FP8> {       // int8 codes, FP32 residual, FP32 U
    static constexpr int KST = 512;            // genotype elements per row per stage
    static constexpr int XB = 1;               // bytes per genotype element
    static constexpr int RB = 4;               // bytes per residual element
    static constexpr int UB = 4;               // bytes per U / ra element
};
template <>
struct RhsCfg<SODAGPU_FP32> {      // FP32 columns, FP32 residual, FP32 U
    static constexpr int KST = 256;
    static constexpr int XB = 4;
    static constexpr int RB = 4;
    static constexpr int UB = 4;
};
template <>
struct RhsCfg<SODAGPU_FP64> {      // int8 codes looked up as FP64, FP64 residual and U
    static constexpr int KST = 512;
    static constexpr int XB = 1;
    static constexpr int RB = 8;
    static constexpr int UB = 8;
};

template <int CT>
struct SptOf { static constexpr int v = CT >= 8 ? 4 : 8; };

template <int MODE>
constexpr int rhs_ku() { return RhsCfg<MODE>::KST * RhsCfg<MODE>::XB / RhsCfg<MODE>::UB; }   // U rows per stage

template <int MODE, int CT>
constexpr size_t rhs_xpart_bytes() { return (size_t)8 * SptOf<CT>::v * RhsCfg<MODE>::KST * RhsCfg<MODE>::XB; }
template <int MODE, int CT>
constexpr size_t rhs_rpart_bytes()
{
    return (size_t)CT * (RhsCfg<MODE>::KST * RhsCfg<MODE>::RB > rhs_ku<MODE>() * RhsCfg<MODE>::UB
                             ? RhsCfg<MODE>::KST * RhsCfg<MODE>::RB
                             : rhs_ku<MODE>() * RhsCfg<MODE>::UB);
}
template <int MODE, int CT>
constexpr size_t rhs_stage_bytes() { return rhs_xpart_bytes<MODE, CT>() + rhs_rpart_bytes<MODE, CT>(); }
template <int MODE, int CT>
constexpr int rhs_nstage()
{
    return 4 * rhs_stage_bytes<MODE, CT>() <= 200 * 1024 ? 4 : (3 * rhs_stage_bytes<MODE, CT>() <= 200 * 1024 ? 3 : 2);
}
template <int MODE, int CT>
constexpr size_t rhs_smem_bytes() { return rhs_nstage<MODE, CT>() * rhs_stage_bytes<MODE, CT>(); }

__device__ __forceinline__ float code_to_f32(uint32_t w, int k)
{
    // 0x4B000000 | byte is the float 2^23 + byte; subtracting 2^23 is exact
    return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7540u | (uint32_t)k)) - 8388608.0f;
}

// Per-SNP draws of one subset (models.f90:146-162, 211-256, 350-413) after
// the rhs kernel left its split partial sums in rpx/rpu: one thread per
// (SNP, chain) pair; a CTA takes 256/CT consecutive SNPs, its threads
// SNP-fastest so that the chain-major arrays (partial sums, g, class, delta
// and its split) are read and written in contiguous runs.
// Every load a draw needs is issued up front: the SNP's metadata and state,
// and the partial sums of all splits at once (added in split order).  With
// TC the kernel also writes what the tensor-core update reads (and takes the
// split count of each SNP's tile from D.rtab): the bf16
// three-way split of delta/sd per chain (dsplit; pairs up to `span`, past the
// subset's end, write zeros) and per-CTA sums of x0_j delta_j (k0part).
template <int MODE, int CT, bool TC>
__device__ __forceinline__ void draw_body(const Dev &D, const VB &vb, int b, int ksplit, int span)
{
    __shared__ double s_rs[CT];   // sum(r) per chain (FP8 centring)
    __shared__ double s_k[256];
    __shared__ float s_kf[256];   // tensor-core path: x0_j delta_j in FP32
    __shared__ DrawPre s_pre[CT];   // chain constants in FP32 (the FP64 pipe is narrow)
    __shared__ float s_zzv[CT];
    __shared__ float s_d32[256];
    __shared__ int s_nzf[256 / CT];
    constexpr int SPC = 256 / CT;   // SNPs per CTA
    const int tid = threadIdx.x;
    const int jloc = tid % SPC, c = tid / SPC;
    const int jl = vb.x * SPC + jloc;
    if (tid < SPC) s_nzf[tid] = 0;
    const int ls = D.blk_ls[b];
    const int N = D.blk_ls[b + 1] - ls;
    const bool act = jl < N;
    const int k = ls + (act ? jl : 0);
    const double zz = D.xxd[b];
    // prologue, overlapping the rhs kernel: chain constants (fixed within an
    // iteration), the SNP's metadata and state (not written by the rhs kernel)
    if (MODE != SODAGPU_FP64 && tid < CT) {
        draw_prefetch(D, &D.scal[tid], tid, 0, 0, s_pre[tid]);
        s_zzv[tid] = (float)(zz / D.scal[tid].vare);
    }
    const int snp = act && !D.skip[k] ? D.perm[k] : -1;
    double inv = 0.0, x0 = 0.0, gold = 0.0;
    float inv32 = 0.0f;
    int cl = 0, sg = 0;
    float vs = 0.0f;
    if (snp >= 0) {
        if (MODE == SODAGPU_FP8 || TC) {
            inv = D.xv[(size_t)k * 4 + 3];
            x0 = D.xv[(size_t)k * 4 + 0];
            inv32 = D.xv32[(size_t)k * 4 + 3];
        }
        if (MODE != SODAGPU_FP64) {
            gold = D.g[(size_t)c * D.p + snp];
            cl = D.cls[(size_t)c * D.p + snp];
            sg = D.grp[snp] - 1;
            if (D.method == SODAGPU_BAYES_A || D.method == SODAGPU_BAYES_B)
                vs = (float)D.vara_s[(size_t)c * D.p + snp];
        }
    }
    // the SNP's draw site and its first Philox block, ahead of the dependency wait
    CRng R;
    if (snp >= 0 && !D.rhs_out) {
        crng_site(R, D, c, cur_rep(D), snp, P_SNP);
        crng_warm(R);
    }
    if (TC && act) {   // the tensor-core rhs gives each 128-SNP tile its own number of splits
        const int32_t *rt = D.rtab + (size_t)b * D.tstride + jl / 128;
        ksplit = rt[1] - rt[0];
    }
    if (MODE == SODAGPU_FP8 || TC) {
        // sum(r) per chain from the row-tile partial sums of the previous residual update, before
        // the dependency wait: that update is complete once this kernel runs, because the rhs
        // kernel lets it launch only after its own dependency wait.  256/CT threads per chain
        // take interleaved tiles, loaded 16 at a time in one batch, then added in part order
        constexpr int PARTS = 256 / CT;
        const int cc = tid / PARTS, part = tid % PARTS;
        double a = 0.0;
        for (int q0 = part; q0 < D.nr_ctas; q0 += 16 * PARTS) {
            double v[16];
#pragma unroll
            for (int u = 0; u < 16; ++u) {
                const int q = q0 + u * PARTS;
                v[u] = q < D.nr_ctas ? __ldcg(D.rsum + (size_t)cc * D.nr_ctas + q) : 0.0;
            }
#pragma unroll
            for (int u = 0; u < 16; ++u) a += v[u];
        }
        s_k[tid] = a;
    }
    __syncthreads();
    if ((MODE == SODAGPU_FP8 || TC) && tid < CT) {
        constexpr int PARTS = 256 / CT;
        double tt = 0.0;
        for (int q = 0; q < PARTS; ++q) tt += s_k[tid * PARTS + q];
        s_rs[tid] = tt;
    }
    __syncthreads();
    // tensor-core path: the rhs is assembled in FP32 (its split sums are FP32; the FP64 pipe of
    // GB300 is narrow and also runs every double <-> float conversion)
    const float x0f = (float)x0, rsf = TC ? (float)s_rs[c] : 0.0f;
    tc::pdl_trigger();
    tc::pdl_wait();
    // the rhs partial sums of all splits, added in split order (the tensor-core rhs
    // gives one FP32 sum per split: codes' r + (sd u)' ra)
    double xr = 0.0, ur = 0.0;
    float xf = 0.0f;
    if (TC) {
        const float *px32 = reinterpret_cast<const float *>(D.rpx);
        float px[RHS_KSPLIT_MAX];
#pragma unroll
        for (int sp = 0; sp < RHS_KSPLIT_MAX; ++sp) {
            px[sp] = 0.0f;
            if (act && sp < ksplit) px[sp] = __ldcg(px32 + ((size_t)sp * CT + c) * D.bs + jl);
        }
        float xs = 0.0f;
#pragma unroll
        for (int sp = 0; sp < RHS_KSPLIT_MAX; ++sp) xs += px[sp];
        // columns with sd = 0 (zero codes) carry U unscaled
        xf = __fmaf_rn(x0f, rsf, __fmul_rn(xs, inv32 != 0.0f ? inv32 : 1.0f));
    } else {
        double px[RHS_KSPLIT_MAX], pu[RHS_KSPLIT_MAX];
#pragma unroll
        for (int sp = 0; sp < RHS_KSPLIT_MAX; ++sp) {
            px[sp] = pu[sp] = 0.0;
            if (act && sp < ksplit) {
                const size_t o = ((size_t)sp * CT + c) * D.bs + jl;
                px[sp] = __ldcg(D.rpx + o);
                pu[sp] = __ldcg(D.rpu + o);
            }
        }
#pragma unroll
        for (int sp = 0; sp < RHS_KSPLIT_MAX; ++sp) {
            if (sp < ksplit) {
                xr += px[sp];
                ur += pu[sp];
            }
        }
    }
    if (D.rhs_out) {   // the same for every thread: the whole CTA leaves here
        if (act) {
            double v = 0.0;
            if (snp >= 0) {
                double x = xr;
                if (MODE == SODAGPU_FP8 && !TC) x = x * inv + x0 * s_rs[c];
                // what the draw consumes
                v = TC ? (double)xf : MODE == SODAGPU_FP64 ? x + ur : (double)(float)(x + ur);
            }
            D.rhs_out[(size_t)c * D.bs + jl] = v;
        }
        return;
    }
    double delta = 0.0;
    if (snp >= 0) {
        if (MODE == SODAGPU_FP8 && !TC) xr = xr * inv + x0 * s_rs[c];
        const ChainScal *S = &D.scal[c];
        int err = 0;
        if (MODE == SODAGPU_FP64) {
            delta = draw_snp(D, S, c, cur_rep(D), snp, xr + ur, zz, zz / S->vare, R, &err);
        } else {
            DrawPre pre = s_pre[c];
            pre.vs = vs;
            if (D.ngroup > 1) {
#pragma unroll
                for (int q = 0; q < DRAW_PRE; ++q)
                    pre.logp[q] = q < D.nmix ? (float)S->log_p[sg + q * D.ngroup] : 0.0f;
            }
            const float rhs = TC ? xf : (float)(xr + ur);
            delta = draw_snp_f(D, S, c, snp, rhs, (float)zz, s_zzv[c], R, &err, gold, cl, sg, pre);
        }
        if (err) flag_err(D, 1);
    }
    float delta32 = 0.0f;
    if (act) {
        delta32 = (float)delta;
        if (!TC) D.delta[(size_t)c * D.bs + jl] = delta;
        if (delta != 0.0) s_nzf[jloc] = 1;
    }
    s_d32[jloc * CT + c] = delta32;
    if (TC) {
        if (jl < span) {
            uint32_t hi = 0, mid = 0, lo = 0;
            // delta / sd; columns with sd = 0 (zero codes) carry delta for the unscaled U
            if (delta32 != 0.0f) tc::split3(delta32 * (inv32 != 0.0f ? inv32 : 1.0f), hi, mid, lo);
            D.dsplit[(size_t)c * D.ldd + jl] = (uint16_t)hi;
            D.dsplit[(size_t)(CT + c) * D.ldd + jl] = (uint16_t)mid;
            D.dsplit[(size_t)(2 * CT + c) * D.ldd + jl] = (uint16_t)lo;
        }
        // this CTA's sum of x0_j delta_j per chain, SNPs in order (FP32: the update adds the
        // centring term to FP32 segment sums)
        s_kf[jloc * CT + c] = __fmul_rn(x0f, delta32);
    }
    __syncthreads();
    if (TC && tid < CT) {
        float tt = 0.0f;
        for (int q = 0; q < SPC; ++q) tt += s_kf[q * CT + tid];
        D.k0part[(size_t)vb.x * CT + tid] = (double)tt;
    }
    // delta32 chain-contiguous per SNP (the CTA's block of 256 values), and the flags of SNPs whose
    // delta is non-zero in some chain
    if (MODE != SODAGPU_FP64) {
        const int j = vb.x * SPC + tid / CT;
        if (j < N) D.delta32[(size_t)vb.x * 256 + tid] = s_d32[tid];
    }
    if (tid < SPC && vb.x * SPC + tid < N) D.nzflag[vb.x * SPC + tid] = s_nzf[tid];
}

template <int MODE, int CT, bool TC>
__global__ void __launch_bounds__(256, 1) k_draw(Dev D, int b, int ksplit, int span)
{
    draw_body<MODE, CT, TC>(D, vb_native(), b, ksplit, span);
}


template <int MODE, int CT>
__device__ __forceinline__ void rhs_body(const Dev &D, const VB &vb, int b, int ksplit)
{
    using Cfg = RhsCfg<MODE>;
    constexpr int SPT = SptOf<CT>::v;
    constexpr int MTS = 8 * SPT;                 // SNPs per M tile (8 warps)
    constexpr int KST = Cfg::KST;
    constexpr int KU = rhs_ku<MODE>();
    constexpr int NS = rhs_nstage<MODE, CT>();
    constexpr size_t XPART = rhs_xpart_bytes<MODE, CT>();
    constexpr size_t SBYTES = rhs_stage_bytes<MODE, CT>();
    typedef typename std::conditional<MODE == SODAGPU_FP64, double, float>::type acc_t;
    extern __shared__ __align__(16) unsigned char smem[];

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // the draw kernel launches only after this wait (its prologue reads what the previous
    // residual update wrote)
    tc::pdl_wait();
    tc::pdl_trigger();
    const int ls = D.blk_ls[b];
    const int N = D.blk_ls[b + 1] - ls;
    const int mt = vb.x / ksplit, ks = vb.x % ksplit;
    const int j0 = mt * MTS;
    if (j0 >= N) return;
    const int npad = (N + 7) & ~7;             // spacing of the subset's U columns
    // K ranges of this split: genotype stages, then augmenting-matrix stages
    const int nG = (D.ldx + KST - 1) / KST;
    const int rowsU = D.blk_pd[b] ? min(npad, j0 + MTS) : npad;   // triangular: rows up to the tile's last column
    const int nU = (rowsU + KU - 1) / KU;
    const int g0 = (int)(((long long)nG * ks) / ksplit), g1 = (int)(((long long)nG * (ks + 1)) / ksplit);
    const int u0 = (int)(((long long)nU * ks) / ksplit), u1 = (int)(((long long)nU * (ks + 1)) / ksplit);
    const int ng = g1 - g0, nv = ng + (u1 - u0);

    auto issue = [&](int v, int buf) {
        unsigned char *dx = smem + (size_t)buf * SBYTES;
        unsigned char *dr = dx + XPART;
        if (v < ng) {     // genotype stage
            const int k0 = (g0 + v) * KST;
            constexpr int XCH = KST * Cfg::XB / 16;
            for (int t = tid; t < MTS * XCH; t += 256) {
                const int row = t / XCH, ch = t % XCH;
                unsigned char *dst = dx + (size_t)row * KST * Cfg::XB + ch * 16;
                const int jk = j0 + row;
                const int e0 = k0 + ch * (16 / Cfg::XB);
                if (jk < N && e0 + 16 / Cfg::XB <= D.ldx) {
                    const void *src = MODE == SODAGPU_FP32
                                          ? (const void *)(D.X32 + (size_t)(ls + jk) * D.ldx + e0)
                                          : (const void *)(D.G + (size_t)(ls + jk) * D.ldx + e0);
                    __pipeline_memcpy_async(dst, src, 16);
                } else {
                    *reinterpret_cast<uint4 *>(dst) = make_uint4(0, 0, 0, 0);
                }
            }
            constexpr int RCH = KST * Cfg::RB / 16;
            for (int t = tid; t < CT * RCH; t += 256) {
                const int c = t / RCH, ch = t % RCH;
                unsigned char *dst = dr + (size_t)c * KST * Cfg::RB + ch * 16;
                const int e0 = k0 + ch * (16 / Cfg::RB);
                if (e0 + 16 / Cfg::RB <= D.ldr) {
                    const void *src = MODE == SODAGPU_FP64 ? (const void *)(D.r + (size_t)c * D.ldr + e0)
                                                           : (const void *)(D.r32 + (size_t)c * D.ldr + e0);
                    __pipeline_memcpy_async(dst, src, 16);
                } else {
                    *reinterpret_cast<uint4 *>(dst) = make_uint4(0, 0, 0, 0);
                }
            }
        } else {          // augmenting-matrix stage: rows [i0, i0+KU) of the tile's U columns
            const int i0 = (u0 + v - ng) * KU;
            constexpr int UCH = KU * Cfg::UB / 16;
            for (int t = tid; t < MTS * UCH; t += 256) {
                const int row = t / UCH, ch = t % UCH;
                unsigned char *dst = dx + (size_t)row * KU * Cfg::UB + ch * 16;
                const int jk = j0 + row;
                const int e0 = i0 + ch * (16 / Cfg::UB);
                if (jk < N && e0 + 16 / Cfg::UB <= npad) {
                    const int64_t off = D.uoff[ls + jk] + e0;
                    const void *src = MODE == SODAGPU_FP64 ? (const void *)(D.U64 + off) : (const void *)(D.U32 + off);
                    __pipeline_memcpy_async(dst, src, 16);
                } else {
                    *reinterpret_cast<uint4 *>(dst) = make_uint4(0, 0, 0, 0);
                }
            }
            constexpr int RCH = KU * Cfg::UB / 16;
            for (int t = tid; t < CT * RCH; t += 256) {
                const int c = t / RCH, ch = t % RCH;
                unsigned char *dst = dr + (size_t)c * KU * Cfg::UB + ch * 16;
                const int e0 = i0 + ch * (16 / Cfg::UB);
                if (e0 + 16 / Cfg::UB <= D.ldra) {
                    const void *src = MODE == SODAGPU_FP64 ? (const void *)(D.ra + (size_t)c * D.ldra + e0)
                                                           : (const void *)(D.ra32 + (size_t)c * D.ldra + e0);
                    __pipeline_memcpy_async(dst, src, 16);
                } else {
                    *reinterpret_cast<uint4 *>(dst) = make_uint4(0, 0, 0, 0);
                }
            }
        }
        __pipeline_commit();
    };

    acc_t acc[SPT][CT];
#pragma unroll
    for (int s = 0; s < SPT; ++s)
#pragma unroll
        for (int c = 0; c < CT; ++c) acc[s][c] = 0;
    double xl[SPT][3];
    if (MODE == SODAGPU_FP64) {
#pragma unroll
        for (int s = 0; s < SPT; ++s) {
            const int jk = j0 + warp * SPT + s;
            const int k = ls + (jk < N ? jk : 0);
            xl[s][0] = D.xv[(size_t)k * 4 + 0];
            xl[s][1] = D.xv[(size_t)k * 4 + 1];
            xl[s][2] = D.xv[(size_t)k * 4 + 2];
        }
    }
    // publishes the accumulators as this split's genotype (is_u = false) or
    // augmenting (is_u = true) partial sums and clears them
    auto publish = [&](bool is_u) {
        double *dstp = is_u ? D.rpu : D.rpx;
#pragma unroll
        for (int s = 0; s < SPT; ++s) {
            const int jk = j0 + warp * SPT + s;
#pragma unroll
            for (int c = 0; c < CT; ++c) {
                // FP32 modes reduce in FP32; only lane 0 widens (the FP64 pipe is narrow)
                if (MODE == SODAGPU_FP64) {
                    const double a = warp_sum((double)acc[s][c]);
                    if (lane == 0 && jk < N) dstp[((size_t)ks * CT + c) * D.bs + jk] = a;
                } else {
                    const float a = warp_sumf((float)acc[s][c]);
                    if (lane == 0 && jk < N) dstp[((size_t)ks * CT + c) * D.bs + jk] = (double)a;
                }
                acc[s][c] = 0;
            }
        }
    };

#pragma unroll
    for (int pp = 0; pp < NS - 1; ++pp) {
        if (pp < nv) issue(pp, pp);
        else __pipeline_commit();
    }
    for (int v = 0; v < nv; ++v) {
        const int buf = v % NS;
        // the buffer of stage v+NS-1 was last read in iteration v-1, which
        // ended with a barrier: refill it before waiting for stage v
        if (v + NS - 1 < nv) issue(v + NS - 1, (v + NS - 1) % NS);
        else __pipeline_commit();
        __pipeline_wait_prior(NS - 1);
        __syncthreads();
        if (v == ng) publish(false);
        const unsigned char *bx = smem + (size_t)buf * SBYTES;
        const unsigned char *br = bx + XPART;
        if (v < ng && MODE == SODAGPU_FP8) {
            // lane covers individuals q*128 + 4*lane + {0..3}: genotype words
            // and residual float4s are contiguous across lanes
#pragma unroll
            for (int q = 0; q < KST / 128; ++q) {
                float x[SPT][4];
#pragma unroll
                for (int s = 0; s < SPT; ++s) {
                    const uint32_t w = *reinterpret_cast<const uint32_t *>(bx + (size_t)(warp * SPT + s) * KST +
                                                                           q * 128 + lane * 4);
                    x[s][0] = code_to_f32(w, 0);
                    x[s][1] = code_to_f32(w, 1);
                    x[s][2] = code_to_f32(w, 2);
                    x[s][3] = code_to_f32(w, 3);
                }
#pragma unroll
                for (int c = 0; c < CT; ++c) {
                    const float4 rr = *reinterpret_cast<const float4 *>(br + ((size_t)c * KST + q * 128 + lane * 4) * 4);
#pragma unroll
                    for (int s = 0; s < SPT; ++s) {
                        acc[s][c] = fmaf(x[s][0], rr.x, acc[s][c]);
                        acc[s][c] = fmaf(x[s][1], rr.y, acc[s][c]);
                        acc[s][c] = fmaf(x[s][2], rr.z, acc[s][c]);
                        acc[s][c] = fmaf(x[s][3], rr.w, acc[s][c]);
                    }
                }
            }
        } else if (MODE != SODAGPU_FP64) {
            // FP32 columns (FP32 mode genotype stages) or FP32 U columns (both modes)
            constexpr int KF = KST * Cfg::XB / 4;    // floats per row of the stage
            const int rstride = v < ng ? KST : KU;
#pragma unroll
            for (int q = 0; q < KF / 128; ++q) {
                float4 xx[SPT];
#pragma unroll
                for (int s = 0; s < SPT; ++s)
                    xx[s] = *reinterpret_cast<const float4 *>(bx + ((size_t)(warp * SPT + s) * KF + q * 128 + lane * 4) * 4);
#pragma unroll
                for (int c = 0; c < CT; ++c) {
                    const float4 rr = *reinterpret_cast<const float4 *>(br + ((size_t)c * rstride + q * 128 + lane * 4) * 4);
#pragma unroll
                    for (int s = 0; s < SPT; ++s) {
                        acc[s][c] = fmaf(xx[s].x, rr.x, acc[s][c]);
                        acc[s][c] = fmaf(xx[s].y, rr.y, acc[s][c]);
                        acc[s][c] = fmaf(xx[s].z, rr.z, acc[s][c]);
                        acc[s][c] = fmaf(xx[s].w, rr.w, acc[s][c]);
                    }
                }
            }
        } else if (v < ng) {   // FP64 genotype stage: codes looked up in the column's exact x values
#pragma unroll 4
            for (int q = 0; q < KST / 32; ++q) {
                const int idx = q * 32 + lane;
                double x[SPT];
#pragma unroll
                for (int s = 0; s < SPT; ++s) {
                    const int code = bx[(size_t)(warp * SPT + s) * KST + idx] & 3;
                    x[s] = code == 0 ? xl[s][0] : (code == 1 ? xl[s][1] : xl[s][2]);
                }
#pragma unroll
                for (int c = 0; c < CT; ++c) {
                    const double rv = *reinterpret_cast<const double *>(br + ((size_t)c * KST + idx) * 8);
#pragma unroll
                    for (int s = 0; s < SPT; ++s) acc[s][c] = fma(x[s], rv, acc[s][c]);
                }
            }
        } else {               // FP64 augmenting stage
#pragma unroll
            for (int q = 0; q < KU / 32; ++q) {
                const int idx = q * 32 + lane;
                double x[SPT];
#pragma unroll
                for (int s = 0; s < SPT; ++s)
                    x[s] = *reinterpret_cast<const double *>(bx + ((size_t)(warp * SPT + s) * KU + idx) * 8);
#pragma unroll
                for (int c = 0; c < CT; ++c) {
                    const double rv = *reinterpret_cast<const double *>(br + ((size_t)c * KU + idx) * 8);
#pragma unroll
                    for (int s = 0; s < SPT; ++s) acc[s][c] = fma(x[s], rv, acc[s][c]);
                }
            }
        }
        __syncthreads();
    }
    __pipeline_wait_prior(0);
    if (nv == ng) publish(false);   // no augmenting stage in this split
    publish(true);

}

template <int MODE, int CT>
__global__ void __launch_bounds__(256, 1) k_rhs(Dev D, int b, int ksplit)
{
    rhs_body<MODE, CT>(D, vb_native(), b, ksplit);
}


}  // namespace soda
