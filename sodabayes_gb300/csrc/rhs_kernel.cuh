// rhs_kernel.cuh — right-hand sides of one SODA subset and the per-SNP draws
// (models.f90:146-162, 211-256, 350-413), included by sweep.cu.
//
//   rhs[j][c] = x_j' r_c + u_j' ra_c (+ d g_j)
//
// is a tall-skinny GEMM (M = subset SNPs, N = chains, K = individuals).  The
// grid is (M tiles of 8*SPT SNPs) x (K splits): each CTA streams its genotype
// rows and the chains' residual rows through shared memory with cp.async
// (double-buffered), keeps an SPT x CT accumulator block per thread, and adds
// its share of the augmenting-matrix dots.  Partial sums go to scratch; the
// last CTA of an M tile to finish (atomic ticket, no waiting) sums them in
// split order and performs the draws of that tile, so the draws are spread
// over the M tiles.  FP8 mode: the codes 0/1/2 are exact in FP32, the centring
// is applied afterwards as x'r = (G'r) / sd - 2p/sd * sum(r).
#pragma once
#include <cuda_pipeline_primitives.h>

namespace soda {

template <int MODE>
struct RhsCfg;
template <>
struct RhsCfg<SODAGPU_FP8> {       // int8 codes, FP32 residual
    static constexpr int KST = 512;            // individuals per stage
    static constexpr int XB = 1;               // bytes per genotype element in smem
    static constexpr int RB = 4;               // bytes per residual element
};
template <>
struct RhsCfg<SODAGPU_FP32> {      // FP32 columns, FP32 residual
    static constexpr int KST = 256;
    static constexpr int XB = 4;
    static constexpr int RB = 4;
};
template <>
struct RhsCfg<SODAGPU_FP64> {      // int8 codes looked up as FP64, FP64 residual
    static constexpr int KST = 512;
    static constexpr int XB = 1;
    static constexpr int RB = 8;
};

template <int CT>
struct SptOf { static constexpr int v = CT >= 8 ? 4 : 8; };

// smem bytes of k_rhs for a mode / chain count
template <int MODE, int CT>
constexpr size_t rhs_smem_bytes()
{
    return 2 * ((size_t)8 * SptOf<CT>::v * RhsCfg<MODE>::KST * RhsCfg<MODE>::XB +
                (size_t)CT * RhsCfg<MODE>::KST * RhsCfg<MODE>::RB);
}

__device__ __forceinline__ float code_to_f32(uint32_t w, int k)
{
    // 0x4B000000 | byte is the float 2^23 + byte; subtracting 2^23 is exact
    return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7540u | (uint32_t)k)) - 8388608.0f;
}

template <int MODE, int CT>
__global__ void __launch_bounds__(256, 1) k_rhs(Dev D, int b, int ksplit)
{
    using Cfg = RhsCfg<MODE>;
    constexpr int SPT = SptOf<CT>::v;
    constexpr int MTS = 8 * SPT;                 // SNPs per M tile (8 warps)
    constexpr int KST = Cfg::KST;
    typedef typename std::conditional<MODE == SODAGPU_FP64, double, float>::type acc_t;
    extern __shared__ __align__(16) unsigned char smem[];
    unsigned char *sX = smem;                                        // [2][MTS][KST*XB]
    unsigned char *sR = smem + 2 * (size_t)MTS * KST * Cfg::XB;      // [2][CT][KST*RB]
    __shared__ int s_last;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int ls = D.blk_ls[b];
    const int N = D.blk_ls[b + 1] - ls;
    const int mt = blockIdx.x / ksplit, ks = blockIdx.x % ksplit;
    const int j0 = mt * MTS;
    if (j0 >= N) return;
    // K range of this split, in whole stages
    const int nst_tot = (D.ldx + KST - 1) / KST;
    const int st0 = (int)(((long long)nst_tot * ks) / ksplit);
    const int st1 = (int)(((long long)nst_tot * (ks + 1)) / ksplit);

    auto issue = [&](int stage, int buf) {
        const int k0 = stage * KST;
        // genotype rows: MTS rows of KST*XB bytes, 16-byte chunks
        constexpr int XCH = KST * Cfg::XB / 16;
        unsigned char *dx = sX + (size_t)buf * MTS * KST * Cfg::XB;
        for (int t = tid; t < MTS * XCH; t += 256) {
            const int row = t / XCH, ch = t % XCH;
            unsigned char *dst = dx + (size_t)row * KST * Cfg::XB + ch * 16;
            const int jk = j0 + row;
            const long long e0 = (long long)k0 + (long long)ch * 16 / Cfg::XB;   // first element of the chunk
            if (jk < N && e0 + 16 / Cfg::XB <= D.ldx) {
                const unsigned char *src;
                if (MODE == SODAGPU_FP32)
                    src = reinterpret_cast<const unsigned char *>(D.X32 + (size_t)(ls + jk) * D.ldx + e0);
                else
                    src = reinterpret_cast<const unsigned char *>(D.G + (size_t)(ls + jk) * D.ldx + e0);
                __pipeline_memcpy_async(dst, src, 16);
            } else {
                *reinterpret_cast<uint4 *>(dst) = make_uint4(0, 0, 0, 0);
            }
        }
        constexpr int RCH = KST * Cfg::RB / 16;
        unsigned char *dr = sR + (size_t)buf * CT * KST * Cfg::RB;
        for (int t = tid; t < CT * RCH; t += 256) {
            const int c = t / RCH, ch = t % RCH;
            unsigned char *dst = dr + (size_t)c * KST * Cfg::RB + ch * 16;
            const long long e0 = (long long)k0 + (long long)ch * 16 / Cfg::RB;
            if (e0 + 16 / Cfg::RB <= D.ldr) {
                const unsigned char *src;
                if (MODE == SODAGPU_FP64)
                    src = reinterpret_cast<const unsigned char *>(D.r + (size_t)c * D.ldr + e0);
                else
                    src = reinterpret_cast<const unsigned char *>(D.r32 + (size_t)c * D.ldr + e0);
                __pipeline_memcpy_async(dst, src, 16);
            } else {
                *reinterpret_cast<uint4 *>(dst) = make_uint4(0, 0, 0, 0);
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

    if (st0 < st1) issue(st0, 0);
    for (int st = st0; st < st1; ++st) {
        const int buf = (st - st0) & 1;
        if (st + 1 < st1) {
            issue(st + 1, buf ^ 1);
            __pipeline_wait_prior(1);
        } else {
            __pipeline_wait_prior(0);
        }
        __syncthreads();
        const unsigned char *bx = sX + (size_t)buf * MTS * KST * Cfg::XB;
        const unsigned char *br = sR + (size_t)buf * CT * KST * Cfg::RB;
        if (MODE == SODAGPU_FP8) {
            // lane covers individuals q*128 + 4*lane + {0..3}, q = 0..3:
            // genotype words and residual float4s are contiguous across lanes
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
        } else if (MODE == SODAGPU_FP32) {
#pragma unroll
            for (int q = 0; q < KST / 128; ++q) {
                float4 xx[SPT];
#pragma unroll
                for (int s = 0; s < SPT; ++s)
                    xx[s] = *reinterpret_cast<const float4 *>(bx + ((size_t)(warp * SPT + s) * KST + q * 128 + lane * 4) * 4);
#pragma unroll
                for (int c = 0; c < CT; ++c) {
                    const float4 rr = *reinterpret_cast<const float4 *>(br + ((size_t)c * KST + q * 128 + lane * 4) * 4);
#pragma unroll
                    for (int s = 0; s < SPT; ++s) {
                        acc[s][c] = fmaf(xx[s].x, rr.x, acc[s][c]);
                        acc[s][c] = fmaf(xx[s].y, rr.y, acc[s][c]);
                        acc[s][c] = fmaf(xx[s].z, rr.z, acc[s][c]);
                        acc[s][c] = fmaf(xx[s].w, rr.w, acc[s][c]);
                    }
                }
            }
        } else {   // FP64: codes looked up in the column's exact x values
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
        }
        __syncthreads();
    }

    // publish this split's genotype partial sums
#pragma unroll
    for (int s = 0; s < SPT; ++s) {
        const int jk = j0 + warp * SPT + s;
#pragma unroll
        for (int c = 0; c < CT; ++c) {
            const double a = MODE == SODAGPU_FP64 ? warp_sum((double)acc[s][c]) : (double)warp_sumf((float)acc[s][c]);
            if (lane == 0 && jk < N) D.rpx[((size_t)ks * CT + c) * D.bs + jk] = a;
        }
    }
    // augmenting-matrix share: rows [ks*RS, (ks+1)*RS) of each column
    {
        const int RS = (D.bs + ksplit - 1) / ksplit;
        const int r0 = ks * RS, r1 = min(D.bs, r0 + RS);
#pragma unroll
        for (int s = 0; s < SPT; ++s) {
            const int jk = j0 + warp * SPT + s;
            acc_t accu[CT];
#pragma unroll
            for (int c = 0; c < CT; ++c) accu[c] = 0;
            if (jk < N) {
                const int k = ls + jk;
                const int64_t off = D.uoff[k];
                const int len = min(D.ulen[k], r1);
                for (int i = r0 + lane; i < len; i += 32) {
                    acc_t u;
                    if (MODE == SODAGPU_FP64) u = (acc_t)D.U64[off + i];
                    else if (MODE == SODAGPU_FP32) u = (acc_t)D.U32[off + i];
                    else u = (acc_t)(__bfloat162float(D.Uhi[off + i]) + __bfloat162float(D.Ulo[off + i]));
#pragma unroll
                    for (int c = 0; c < CT; ++c) accu[c] += u * (acc_t)D.ra[(size_t)c * D.bs + i];
                }
            }
#pragma unroll
            for (int c = 0; c < CT; ++c) {
                const double u = MODE == SODAGPU_FP64 ? warp_sum((double)accu[c]) : (double)warp_sumf((float)accu[c]);
                if (lane == 0 && jk < N) D.rpu[((size_t)ks * CT + c) * D.bs + jk] = u;
            }
        }
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) s_last = atomicAdd(&D.rticket[mt], 1) == ksplit - 1;
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    // the last CTA of the M tile: totals in split order, then the draws
    const int rep = cur_rep(D);
    const double zz = D.xxd[b];
    const int cnt = min(MTS, N - j0);
    for (int t = tid; t < ((cnt * CT + 31) & ~31); t += 256) {
        const int jl = t / CT, c = t % CT;
        const int jk = j0 + jl;
        const bool act = jl < cnt;
        double delta = 0.0;
        if (act) {
            const int k = ls + jk;
            if (D.skip[k]) {
                delta = 0.0;
            } else {
                double xr = 0.0, ur = 0.0;
                for (int sp = 0; sp < ksplit; ++sp) {
                    const size_t o = ((size_t)sp * CT + c) * D.bs + jk;
                    xr += __ldcg(D.rpx + o);
                    ur += __ldcg(D.rpu + o);
                }
                if (MODE == SODAGPU_FP8) {
                    double rs = 0.0;
                    for (int q = 0; q < D.nr_ctas; ++q) rs += D.rsum[(size_t)c * D.nr_ctas + q];
                    xr = xr * D.xv[(size_t)k * 4 + 3] + D.xv[(size_t)k * 4 + 0] * rs;
                }
                const ChainScal *S = &D.scal[c];
                CRng R;
                crng_init(R, D.seed, c, rep, D.perm[k], P_SNP);
                int err = 0;
                delta = draw_snp(D, S, c, rep, D.perm[k], xr + ur, zz, zz / S->vare, R, &err);
                if (err) flag_err(D, 1);
            }
            D.delta[(size_t)c * D.bs + jk] = delta;
        }
        // chains of one SNP are CT consecutive lanes (CT divides 32)
        const unsigned m = __ballot_sync(0xffffffffu, act && delta != 0.0);
        const unsigned grp = CT >= 32 ? 0xffffffffu : (((1u << CT) - 1u) << ((lane / CT) * CT));
        if (act && c == 0) D.nzflag[jk] = (m & grp) != 0u;
    }
    if (tid == 0) D.rticket[mt] = 0;
}

}  // namespace soda
