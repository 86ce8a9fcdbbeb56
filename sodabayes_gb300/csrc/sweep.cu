// sweep.cu — per-iteration kernels of the SODA Gibbs sampler.
//
// One iteration (models.f90:129-574) is, per chain:
//   mu draw                              k_mu_partial + k_mu_apply   (models.f90:130-132)
//   for each subset b (sequential):
//     rhs_j = x_j'r + u_j'ra (+d g_j) and the per-SNP draw
//                                        k_rhs (rhs_kernel.cuh)      (models.f90:146-162, 211-256, 350-413)
//     r += X_b delta, ra += U_b delta    k_update                    (models.f90:164-174, 258-272, 415-430)
//   single-site updates of skipped SNPs  k_skipped                   (models.f90:178-193, 276-320, 433-495)
//   class counts, sum g^2, sum r^2       k_stats
//   sigma2_g, sigma2_e, pi draws, trace  k_hyper                     (models.f90:194, 321-325, 496-522, 549-569)
//   ra redraw, posterior accumulators    k_post                      (models.f90:523-548)
//   residual recalibration               k_recal_partial/_apply      (models.f90:571-573)
// All chains of the context advance together inside each launch.
#include <cuda_runtime.h>
#include <stdint.h>
#include "rng.cuh"
#include "state.cuh"
#include "sweep.cuh"
#include "tc.cuh"
#include <algorithm>
#include <vector>

namespace soda {

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ float warp_sumf(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Deterministic block sum; every thread gets the total.  blockDim.x % 32 == 0.
__device__ double block_sum(double v, double *sh /* >= 33 doubles */)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    v = warp_sum(v);
    __syncthreads();
    if (lane == 0) sh[w] = v;
    __syncthreads();
    if (w == 0) {
        double t = lane < nw ? sh[lane] : 0.0;
        t = warp_sum(t);
        if (lane == 0) sh[32] = t;
    }
    __syncthreads();
    return sh[32];
}

__device__ __forceinline__ int cur_rep(const Dev &D) { return *((volatile int32_t *)&D.ctl->rep); }

// Residual stores: the FP64 master and, for the FP32-core rhs, its FP32 copy,
// or, when the tensor-core rhs runs, the bf16 hi/mid/lo split of the FP32
// value that it loads by TMA.
__device__ __forceinline__ void split_store(uint16_t *sp, size_t o, size_t part, float f)
{
    uint32_t h, m, l;
    tc::split3(f, h, m, l);
    sp[o] = (uint16_t)h;
    sp[o + part] = (uint16_t)m;
    sp[o + 2 * part] = (uint16_t)l;
}
__device__ __forceinline__ void store_r(const Dev &D, int c, int i, double v)
{
    const size_t o = (size_t)c * D.ldr + i;
    D.r[o] = v;
    if (!D.tc) D.r32[o] = (float)v;   // read only by the FP32-core dot products
    if (D.rsp) split_store(D.rsp, o, (size_t)D.chains * D.ldr, (float)v);
}
__device__ __forceinline__ void store_ra(const Dev &D, int c, int i, double v)
{
    const size_t o = (size_t)c * D.ldra + i;
    D.ra[o] = v;
    D.ra32[o] = (float)v;
    if (D.rasp) split_store(D.rasp, o, (size_t)D.chains * D.ldra, (float)v);
}

__device__ __forceinline__ void flag_err(const Dev &D, int code)
{
    atomicExch(&D.ctl->err, code);
}

// A draw past the end of an injected-draw tape sets the same error code as a
// site needing more uniforms than its record holds.
constexpr int ERR_TAPE = CRNG_TAPE_OVERRUN;

// The draw stream of one site: Philox keyed by (seed, chain, rep, slot,
// purpose), or, with an injected-draw tape, the site's record (chain 0; site
// numbering of sodagpu_set_tape).
__device__ __forceinline__ void crng_site(CRng &R, const Dev &D, int c, int rep, int slot, int purpose)
{
    crng_init(R, D.seed, c, rep, slot, purpose);
    if (!D.tape) return;
    int site;
    switch (purpose) {
    case P_MU: site = 0; break;
    case P_VARA: site = 1; break;
    case P_VARE: site = 2; break;
    case P_PI: site = 3 + slot; break;
    case P_RA: site = 3 + D.ngroup + slot; break;
    default: site = D.tape_snp0 + slot; break;   // P_SNP, P_SKIP: by SNP id
    }
    R.tover = &D.ctl->err;
    if (rep >= 0 && rep < D.tape_reps && site < D.tape_sites) {
        R.tape = D.tape + ((size_t)rep * D.tape_sites + site) * SODAGPU_TAPE_W;
    } else {
        flag_err(D, ERR_TAPE);
    }
}

// ---------------------------------------------------------------------------
// Per-SNP conditional draw inside a subset.  Returns delta = g_old - g_new.
// Restates models.f90:146-161 (BayesA), 211-255 (BayesB), 350-412 (C/Cpi/R/Rc).
// ---------------------------------------------------------------------------
__device__ __forceinline__ double draw_snp(const Dev &D, const ChainScal *S, int c, int rep, int snploc,
                           double rhs, double zz, double zz_vare, CRng &R, int *err)
{
    const size_t o = (size_t)c * D.p + snploc;
    const double vare = S->vare;
    double gk = D.g[o];
    const double gold = gk;
    const int m = D.method;
    if (m == SODAGPU_BAYES_A) {
        rhs = rhs + zz * gk;
        const double vs = D.vara_s[o];
        const double v1 = zz + vare / vs;
        gk = d_rnorm(rhs / v1, sqrt(vare / v1), R);
        D.g[o] = gk;
        const double scale = (gk * gk + S->scale_va * D.df_va) / (D.df_va + 1.0);
        D.vara_s[o] = d_rscinvchi2(D.df_va + 1.0, scale, R, err);
        return gold - gk;
    }
    const int cl = D.cls[o];
    if (cl > 1) rhs = rhs + zz * gk;
    const int ng = D.ngroup;
    if (m == SODAGPU_BAYES_B) {
        const double vs = D.vara_s[o];
        const double s1 = S->log_p[0];
        const double logdetV = log(vs * zz_vare + 1.0);
        const double uhat = rhs / (zz + vare / vs);
        const double s2 = -0.5 * (logdetV - (rhs * uhat / vare)) + S->log_p[ng];
        const double clike = s1 - s2;
        double sk;
        if (clike > 700) sk = 0.0;
        else if (clike < -700) sk = 1.0;
        else sk = 1.0 / (1.0 + exp(clike));
        const double u = crng_unit(R);
        const int flag = u < sk ? 2 : 1;
        double gnew;
        if (flag == 1) {
            gk = d_rnorm(0.0, sqrt(vs), R);
            gnew = 0.0;
        } else {
            const double v1 = zz + vare / vs;
            gk = d_rnorm(rhs / v1, sqrt(vare / v1), R);
            gnew = gk;
        }
        D.g[o] = gnew;
        D.cls[o] = flag;
        const double scale = (gk * gk + S->scale_va * D.df_va) / (D.df_va + 1.0);
        D.vara_s[o] = d_rscinvchi2(D.df_va + 1.0, scale, R, err);
        return gold - gnew;
    }
    // BayesC / Cpi / R / Rc
    const int nm = D.nmix;
    const int sg = D.grp[snploc] - 1;
    double s[MAXDIST];
    s[0] = S->log_p[sg];
    for (int kk = 1; kk < nm; ++kk) {
        const double logdetV = log(S->gp[kk] * zz_vare + 1.0);
        const double uhat = rhs / (zz + S->vare_gp[kk]);
        s[kk] = -0.5 * (logdetV - (rhs * uhat / vare)) + S->log_p[sg + kk * ng];
    }
    const double u = crng_unit(R);
    double ssculm = 0.0;
    int flag = 1;
    for (int kk = 0; kk < nm; ++kk) {
        const double skk = s[kk];
        double sk = 0.0;
        bool overflow = false;
        for (int j = 0; j < nm; ++j) {
            if (j == kk) continue;
            const double clike = s[j] - skk;
            if (clike < -700) continue;
            if (clike > 700) { overflow = true; break; }
            sk = sk + exp(clike);
        }
        const double st = overflow ? 0.0 : 1.0 / (1.0 + sk);
        ssculm = ssculm + st;
        if (u < ssculm) { flag = kk + 1; break; }
    }
    double gnew = 0.0;
    if (flag != 1) {
        const double v1 = zz + vare / S->gp[flag - 1];
        gnew = d_rnorm(rhs / v1, sqrt(vare / v1), R);
    }
    D.cls[o] = flag;
    D.g[o] = gnew;
    return gold - gnew;
}

// The same draw in FP32 arithmetic, for the FP32/FP8 sweeps: GB300 executes
// FP64 at a small fraction of its FP32 rate, and the draws of a subset sit on
// the critical path of every subset.  State stays FP64.
// Chain state a draw reads, loaded by the caller ahead of the draw (for up
// to DRAW_PRE mixture classes; the state changes only between iterations):
// the residual variance, the prior scale, the SNP's locus variance (BayesA/B)
// and, per class k, log pi of the SNP's group, gamma_k sigma2_g and
// sigma2_e / (gamma_k sigma2_g).
constexpr int DRAW_PRE = 4;
struct DrawPre {
    float vare, scale_va, vs;
    float logp[DRAW_PRE], gp[DRAW_PRE], vgp[DRAW_PRE];
};

__device__ __forceinline__ void draw_prefetch(const Dev &D, const ChainScal *S, int c, int snploc, int sg, DrawPre &q)
{
    q.vare = (float)S->vare;
    q.scale_va = (float)S->scale_va;
    q.vs = (D.method == SODAGPU_BAYES_A || D.method == SODAGPU_BAYES_B) ? (float)D.vara_s[(size_t)c * D.p + snploc]
                                                                          : 0.0f;
#pragma unroll
    for (int k = 0; k < DRAW_PRE; ++k) {
        const bool in = k < D.nmix;
        q.logp[k] = in ? (float)S->log_p[sg + k * D.ngroup] : 0.0f;
        q.gp[k] = in ? (float)S->gp[k] : 0.0f;
        q.vgp[k] = in ? (float)S->vare_gp[k] : 0.0f;
    }
}

// gold = g and cl = class of the SNP in this chain, sg = its group - 1, all
// loaded by the caller ahead of the draw (they sit on its critical path);
// pre: the prefetched chain state (used when nmix <= DRAW_PRE).
__device__ __forceinline__ double draw_snp_f(const Dev &D, const ChainScal *S, int c, int snploc, float rhs, float zz,
                                             float zz_vare, CRng &R, int *err, double gold, int cl, int sg,
                                             const DrawPre &pre)
{
    const size_t o = (size_t)c * D.p + snploc;
    const bool use_pre = D.nmix <= DRAW_PRE;
    const float vare = pre.vare;
    float gk = (float)gold;
    const int m = D.method;
    const float df_va = (float)D.df_va, scale_va = pre.scale_va;
    if (m == SODAGPU_BAYES_A) {
        rhs = rhs + zz * gk;
        const float vs = pre.vs;
        const float v1 = zz + vare / vs;
        gk = d_rnorm_f(rhs / v1, sqrtf(vare / v1), R);
        D.g[o] = (double)gk;
        const float scale = (gk * gk + scale_va * df_va) / (df_va + 1.0f);
        D.vara_s[o] = (double)d_rscinvchi2_f(df_va + 1.0f, scale, R, err);
        return gold - (double)gk;
    }
    if (cl > 1) rhs = rhs + zz * gk;
    const int ng = D.ngroup;
    if (m == SODAGPU_BAYES_B) {
        const float vs = pre.vs;
        const float s1 = pre.logp[0];
        const float logdetV = logf(vs * zz_vare + 1.0f);
        const float uhat = rhs / (zz + vare / vs);
        const float s2 = -0.5f * (logdetV - (rhs * uhat / vare)) + pre.logp[1];
        const float clike = s1 - s2;
        float sk;
        if (clike > 700.0f) sk = 0.0f;
        else if (clike < -700.0f) sk = 1.0f;
        else sk = 1.0f / (1.0f + expf(clike));
        const float u = crng_unit_f(R);
        const int flag = u < sk ? 2 : 1;
        double gnew;
        if (flag == 1) {
            gk = d_rnorm_f(0.0f, sqrtf(vs), R);
            gnew = 0.0;
        } else {
            const float v1 = zz + vare / vs;
            gk = d_rnorm_f(rhs / v1, sqrtf(vare / v1), R);
            gnew = (double)gk;
        }
        D.g[o] = gnew;
        D.cls[o] = flag;
        const float scale = (gk * gk + scale_va * df_va) / (df_va + 1.0f);
        D.vara_s[o] = (double)d_rscinvchi2_f(df_va + 1.0f, scale, R, err);
        return gold - gnew;
    }
    const int nm = D.nmix;
    int flag = 1;
    if (use_pre) {
        // up to DRAW_PRE classes with every loop unrolled: the scores stay in registers
        float sv[DRAW_PRE];
        sv[0] = pre.logp[0];
#pragma unroll
        for (int kk = 1; kk < DRAW_PRE; ++kk) {
            sv[kk] = 0.0f;
            if (kk < nm) {
                const float logdetV = logf(pre.gp[kk] * zz_vare + 1.0f);
                const float uhat = rhs / (zz + pre.vgp[kk]);
                sv[kk] = -0.5f * (logdetV - (rhs * uhat / vare)) + pre.logp[kk];
            }
        }
        const float u = crng_unit_f(R);
        float ssculm = 0.0f;
        bool done = false;
#pragma unroll
        for (int kk = 0; kk < DRAW_PRE; ++kk) {
            if (kk < nm && !done) {
                float sk = 0.0f;
                bool overflow = false;
#pragma unroll
                for (int j = 0; j < DRAW_PRE; ++j) {
                    if (j < nm && j != kk && !overflow) {
                        const float clike = sv[j] - sv[kk];
                        if (clike > 700.0f) overflow = true;
                        else if (clike >= -700.0f) sk = sk + expf(clike);
                    }
                }
                ssculm = ssculm + (overflow ? 0.0f : 1.0f / (1.0f + sk));
                if (u < ssculm) {
                    flag = kk + 1;
                    done = true;
                }
            }
        }
    } else {
        float sv[MAXDIST];
        sv[0] = (float)S->log_p[sg];
        for (int kk = 1; kk < nm; ++kk) {
            const float logdetV = logf((float)S->gp[kk] * zz_vare + 1.0f);
            const float uhat = rhs / (zz + (float)S->vare_gp[kk]);
            sv[kk] = -0.5f * (logdetV - (rhs * uhat / vare)) + (float)S->log_p[sg + kk * ng];
        }
        const float u = crng_unit_f(R);
        float ssculm = 0.0f;
        for (int kk = 0; kk < nm; ++kk) {
            const float skk = sv[kk];
            float sk = 0.0f;
            bool overflow = false;
            for (int j = 0; j < nm; ++j) {
                if (j == kk) continue;
                const float clike = sv[j] - skk;
                if (clike < -700.0f) continue;
                if (clike > 700.0f) { overflow = true; break; }
                sk = sk + expf(clike);
            }
            ssculm = ssculm + (overflow ? 0.0f : 1.0f / (1.0f + sk));
            if (u < ssculm) { flag = kk + 1; break; }
        }
    }
    double gnew = 0.0;
    if (flag != 1) {
        float gsel = 0.0f;
#pragma unroll
        for (int k = 0; k < DRAW_PRE; ++k)
            if (k == flag - 1) gsel = pre.gp[k];
        const float v1 = zz + vare / (use_pre ? gsel : (float)S->gp[flag - 1]);
        gnew = (double)d_rnorm_f(rhs / v1, sqrtf(vare / v1), R);
    }
    D.cls[o] = flag;
    D.g[o] = gnew;
    return gold - gnew;
}

}  // namespace soda

#include "rhs_kernel.cuh"

namespace soda {

// ---------------------------------------------------------------------------
// iteration start and the mu draw
// ---------------------------------------------------------------------------
__device__ __forceinline__ void iter_begin_body(const Dev &D, const VB &vb)
{
    RunCtl *ctl = D.ctl;
    const int rep = ctl->rep + 1;
    ctl->rep = rep;
    if (rep % D.thin == 0) ctl->trace_iter += 1;
}

__global__ void  k_iter_begin(Dev D)
{
    iter_begin_body(D, vb_native());
}


__device__ __forceinline__ void mu_partial_body(const Dev &D, const VB &vb)
{
    __shared__ double sh[33];
    const int c = vb.y, rep = cur_rep(D);
    const double mu_old = D.scal[c].mu[(rep - 1) & 1];
    double v = 0.0;
#pragma unroll
    for (int q = 0; q < ROWS_PER_THREAD; ++q) {
        const int i = vb.x * ROW_TILE + q * ROW_THREADS + threadIdx.x;
        if (i < D.n) v += D.r[(size_t)c * D.ldr + i] + mu_old;
    }
    const double t = block_sum(v, sh);
    if (threadIdx.x == 0) D.rpart[(size_t)c * D.nr_ctas + vb.x] = t;
}

__global__ void __launch_bounds__(ROW_THREADS) k_mu_partial(Dev D)
{
    mu_partial_body(D, vb_native());
}


__device__ __forceinline__ void mu_apply_body(const Dev &D, const VB &vb)
{
    __shared__ double sh[33];
    __shared__ double s_mu;
    const int c = vb.y, rep = cur_rep(D);
    ChainScal *S = &D.scal[c];
    const double mu_old = S->mu[(rep - 1) & 1];
    if (threadIdx.x == 0) {
        double tot = 0.0;
        for (int t = 0; t < D.nr_ctas; ++t) tot += D.rpart[(size_t)c * D.nr_ctas + t];
        CRng R;
        crng_site(R, D, c, rep, 0, P_MU);
        const double nn = (double)D.n;
        const double mu = d_rnorm(tot / nn, sqrt(S->vare / nn), R);
        s_mu = mu;
        if (vb.x == 0) S->mu[rep & 1] = mu;
    }
    __syncthreads();
    const double mu = s_mu;
    double vs = 0.0;
#pragma unroll
    for (int q = 0; q < ROWS_PER_THREAD; ++q) {
        const int i = vb.x * ROW_TILE + q * ROW_THREADS + threadIdx.x;
        if (i < D.n) {
            const double v = (D.r[(size_t)c * D.ldr + i] + mu_old) - mu;
            store_r(D, c, i, v);
            vs += v;
        }
    }
    if (D.precision == SODAGPU_FP8) {
        const double t = block_sum(vs, sh);
        if (threadIdx.x == 0) D.rsum[(size_t)c * D.nr_ctas + vb.x] = t;
    }
}

__global__ void __launch_bounds__(ROW_THREADS) k_mu_apply(Dev D)
{
    mu_apply_body(D, vb_native());
}


}  // namespace soda

#include "update_kernel.cuh"
#include "rhs_tc.cuh"
#include "update_tc.cuh"

namespace soda {

// ---------------------------------------------------------------------------
// Single-site updates, one CTA per chain, SNPs in order: the SNPs the pivoted
// fallback skips (models.f90:178-193, 276-320, 433-495) and, for the regular
// sampler, every SNP (regular_bayes, models.f90:717-859).  The residual is
// held in shared memory when it fits (each thread owns the same individuals
// in the dot product and in the update, so only the reduction and the draw
// need barriers); the mixture-class scores and the exponentials of their
// differences are computed by parallel lanes of warp 0 and added by lane 0 in
// the reference's order.  The reference reads module copies of log_p /
// vare_gp for skipped SNPs that its parallel regions never assign; the
// current values are used.
// ---------------------------------------------------------------------------
constexpr int SS_THREADS = 512;
constexpr int SS_SMEM_MAX = 200 * 1024;   // residual in shared memory up to 25,600 individuals

// Lane 0 returns the update delta = g_old - g_new of SNP snploc of chain c
// (its new effect, class and locus variance written); all 32 lanes enter.
__device__ __forceinline__ double single_site_draw(const Dev &D, ChainScal *S, int c, int rep, int snploc, double dot)
{
    const int lane = threadIdx.x & 31;
    const size_t o = (size_t)c * D.p + snploc;
    const double vare = S->vare, zz = D.xpx[snploc], zz_vare = zz / vare;
    const int m = D.method, ng = D.ngroup, nm = D.nmix;
    double rhs = dot, upd = 0.0;
    int err = 0;
    if (m != SODAGPU_BAYES_A && m != SODAGPU_BAYES_B) {
        // BayesC/Cpi/R/Rc: scores by lanes 0..nm-1, exponentials of their differences by lanes (kk, j)
        const double gk = D.g[o];
        const int cl = D.cls[o];
        if (cl > 1) rhs = rhs + zz * gk;
        const int sg = D.grp[snploc] - 1;
        double sv = 0.0;
        if (lane == 0) sv = S->log_p[sg];
        else if (lane < nm) {
            const double logdetV = log(S->gp[lane] * zz_vare + 1.0);
            const double uhat = rhs / (zz + S->vare_gp[lane]);
            sv = -0.5 * (logdetV - (rhs * uhat / vare)) + S->log_p[sg + lane * ng];
        }
        const bool par = nm * nm <= 32;
        const int kq = lane / (nm > 0 ? nm : 1), jq = lane % (nm > 0 ? nm : 1);
        const double skq = __shfl_sync(0xffffffffu, sv, par ? kq : 0);
        const double sjq = __shfl_sync(0xffffffffu, sv, par ? jq : 0);
        double ev = 0.0;
        if (par && lane < nm * nm && kq != jq) {
            const double clike = sjq - skq;
            if (clike >= -700 && clike <= 700) ev = exp(clike);
        }
        double s[MAXDIST];
        double e[MAXDIST * MAXDIST > 32 ? 32 : MAXDIST * MAXDIST];
#pragma unroll
        for (int t = 0; t < MAXDIST; ++t) s[t] = __shfl_sync(0xffffffffu, sv, t < 32 ? t : 0);
#pragma unroll
        for (int t = 0; t < 32; ++t) {
            const double v = __shfl_sync(0xffffffffu, ev, t);
            if (t < (int)(sizeof(e) / sizeof(e[0]))) e[t] = v;
        }
        if (lane == 0) {
            CRng R;
            crng_site(R, D, c, rep, snploc, P_SKIP);
            const double u = crng_unit(R);
            double ssculm = 0.0;
            int flag = 1;
            for (int kk = 0; kk < nm; ++kk) {
                const double skk = s[kk];
                double sk = 0.0;
                bool overflow = false;
                for (int j = 0; j < nm; ++j) {
                    if (j == kk) continue;
                    const double clike = s[j] - skk;
                    if (clike < -700) continue;
                    if (clike > 700) { overflow = true; break; }
                    sk = sk + (par ? e[kk * nm + j] : exp(clike));
                }
                ssculm = ssculm + (overflow ? 0.0 : 1.0 / (1.0 + sk));
                if (u < ssculm) { flag = kk + 1; break; }
            }
            double gt = 0.0;
            if (flag == 1) {
                upd = cl > 1 ? gk : 0.0;
            } else {
                const double v1 = zz + vare / S->gp[flag - 1];
                gt = d_rnorm(rhs / v1, sqrt(vare / v1), R);
                upd = gk - gt;
            }
            D.g[o] = gt;
            D.cls[o] = flag;
        }
        return upd;
    }
    if (lane == 0) {
        const double gk = D.g[o];
        double gt = 0.0;
        CRng R;
        crng_site(R, D, c, rep, snploc, P_SKIP);
        if (m == SODAGPU_BAYES_A) {
            rhs = rhs + zz * gk;
            const double v1 = zz + vare / D.vara_s[o];
            gt = d_rnorm(rhs / v1, sqrt(vare / v1), R);
            upd = gk - gt;
            D.g[o] = gt;
        } else {
            if (D.cls[o] > 1) rhs = rhs + zz * gk;
            const double vs = D.vara_s[o];
            const double s1 = S->log_p[0];
            const double logdetV = log(vs * zz_vare + 1.0);
            const double uhat = rhs / (zz + vare / vs);
            const double s2 = -0.5 * (logdetV - (rhs * uhat / vare)) + S->log_p[ng];
            const double clike = s1 - s2;
            double sk;
            if (clike > 700) sk = 0.0;
            else if (clike < -700) sk = 1.0;
            else sk = 1.0 / (1.0 + exp(clike));
            const double u = crng_unit(R);
            const int flag = u < sk ? 2 : 1;
            if (flag == 1) {
                gt = d_rnorm(0.0, sqrt(vs), R);
                upd = D.cls[o] > 1 ? gk : 0.0;
                D.g[o] = 0.0;
            } else {
                const double v1 = zz + vare / vs;
                gt = d_rnorm(rhs / v1, sqrt(vare / v1), R);
                upd = gk - gt;
                D.g[o] = gt;
            }
            D.cls[o] = flag;
        }
        const double scale = (gt * gt + S->scale_va * D.df_va) / (D.df_va + 1.0);
        D.vara_s[o] = d_rscinvchi2(D.df_va + 1.0, scale, R, &err);
        if (err) flag_err(D, 1);
    }
    return upd;
}

__device__ __forceinline__ void skipped_body(const Dev &D, const VB &vb)
{
    extern __shared__ double s_r[];
    __shared__ double s_part[SS_THREADS / 32];
    __shared__ double s_upd;
    const int c = vb.x, rep = cur_rep(D);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    ChainScal *S = &D.scal[c];
    double *rg = D.r + (size_t)c * D.ldr;
    const bool in_smem = (size_t)D.n * sizeof(double) <= (size_t)SS_SMEM_MAX;
    double *r = in_smem ? s_r : rg;
    if (in_smem) {
        for (int i = tid; i < D.n; i += SS_THREADS) s_r[i] = rg[i];
        __syncthreads();
    }
    for (int t = 0; t < D.nskipped; ++t) {
        const int snploc = D.iskipped[t];
        const int k = D.pos_of[snploc];
        const int8_t *col = D.G + (size_t)k * D.ldx;
        const double *xv = D.xv + (size_t)k * 4;
        const double x0 = xv[0], x1 = xv[1], x2 = xv[2];
        double part = 0.0;
        for (int i = tid; i < D.n; i += SS_THREADS) {
            const int g = col[i];
            part += r[i] * (g == 0 ? x0 : (g == 1 ? x1 : x2));
        }
        part = warp_sum(part);
        if (lane == 0) s_part[warp] = part;
        __syncthreads();
        if (warp == 0) {
            double d = lane < SS_THREADS / 32 ? s_part[lane] : 0.0;
            d = warp_sum(d);
            const double upd = single_site_draw(D, S, c, rep, snploc, d);
            if (lane == 0) s_upd = upd;
        }
        __syncthreads();
        const double upd = s_upd;
        if (upd != 0.0) {
            for (int i = tid; i < D.n; i += SS_THREADS) {
                const int g = col[i];
                r[i] = r[i] + (g == 0 ? x0 : (g == 1 ? x1 : x2)) * upd;
            }
        }
    }
    if (in_smem) {
        __syncthreads();
        for (int i = tid; i < D.n; i += SS_THREADS) rg[i] = s_r[i];
    }
}

__global__ void __launch_bounds__(SS_THREADS) k_skipped(Dev D)
{
    skipped_body(D, vb_native());
}


// ---------------------------------------------------------------------------
// per-iteration statistics: class counts and sum g^2 per (group, class),
// sum r^2 (models.f90:194, 321-325, 496-503, 515)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void stats_body(const Dev &D, const VB &vb)
{
    __shared__ double sh[33];
    const int c = vb.y;
    if (vb.x < NSTAT) {
        const int ngm = D.ngroup * D.nmix;
        const size_t base = (size_t)c * D.p;
        for (int e = 0; e < ngm; ++e) {
            const int eg = e % D.ngroup, em = e / D.ngroup;
            double v = 0.0;
            int cnt = 0;
            for (int j = vb.x * 256 + threadIdx.x; j < D.p; j += NSTAT * 256) {
                const int cl = D.cls[base + j];
                if (D.grp[j] - 1 == eg && cl - 1 == em) {
                    const double gj = D.g[base + j];
                    v += gj * gj;
                    ++cnt;
                }
            }
            const double tv = block_sum(v, sh);
            const double tc = block_sum((double)cnt, sh);
            if (threadIdx.x == 0) {
                const size_t o = ((size_t)c * NSTAT + vb.x) * ngm + e;
                D.statpart[o] = tv;
                D.cntpart[o] = (int32_t)tc;
            }
        }
    } else {
        const int rb = vb.x - NSTAT;
        double v2 = 0.0;
        const int i = rb * ROW_TILE + threadIdx.x;
        if (threadIdx.x < ROW_TILE && i < D.n) {
            const double v = D.r[(size_t)c * D.ldr + i];
            v2 = v * v;
        }
        const double t = block_sum(v2, sh);
        if (threadIdx.x == 0) D.rpart[(size_t)c * D.nr_ctas + rb] = t;
    }
}

__global__ void __launch_bounds__(256) k_stats(Dev D)
{
    stats_body(D, vb_native());
}


__device__ __forceinline__ void hyper_body(const Dev &D, const VB &vb)
{
    __shared__ double s_vara;
    const int c = vb.x, rep = cur_rep(D);
    ChainScal *S = &D.scal[c];
    const int ng = D.ngroup, nm = D.nmix, ngm = ng * nm, m = D.method;
    for (int e = threadIdx.x; e < ngm; e += blockDim.x) {
        double v = 0.0;
        int cnt = 0;
        for (int t = 0; t < NSTAT; ++t) {
            const size_t o = ((size_t)c * NSTAT + t) * ngm + e;
            v += D.statpart[o];
            cnt += D.cntpart[o];
        }
        S->varindist[e] = v;
        // BayesA tracks no class counts (models.f90:194): its trace shows none
        S->snpindist[e] = m == SODAGPU_BAYES_A ? 0 : cnt;
    }
    __syncthreads();
    int err = 0;
    if (threadIdx.x == 0) {
        if (m == SODAGPU_BAYES_B) {
            S->included = S->snpindist[ng];
            S->varindist[0] = 0.0;
        } else if (m != SODAGPU_BAYES_A) {
            int excl = 0;
            for (int i = 0; i < ng; ++i) excl += S->snpindist[i];
            S->included = D.p - excl;
            double scale = 0.0;
            for (int i = 0; i < ng; ++i)
                for (int j = 1; j < nm; ++j) scale = scale + S->varindist[i + j * ng] / D.mix[j];
            scale = (scale + S->scale_va * D.df_va) / (D.df_va + (double)S->included);
            CRng R;
            crng_site(R, D, c, rep, 0, P_VARA);
            S->vara = d_rscinvchi2((double)S->included + D.df_va, scale, R, &err);
            for (int j = 0; j < nm; ++j) S->gp[j] = D.mix[j] * S->vara;
        }
        double rr = 0.0;
        for (int t = 0; t < D.nr_ctas; ++t) rr += D.rpart[(size_t)c * D.nr_ctas + t];
        const double nn = (double)D.n;
        const double scale = (rr + D.scale_ve * D.df_ve) / (nn + D.df_ve);
        CRng R;
        crng_site(R, D, c, rep, 0, P_VARE);
        S->vare = d_rscinvchi2(nn + D.df_ve, scale, R, &err);
        s_vara = S->vara;
    }
    __syncthreads();
    // pi ~ Dirichlet(counts + alpha), one thread per group (models.f90:517-522)
    if (m == SODAGPU_BAYES_CPI || m == SODAGPU_BAYES_R || m == SODAGPU_BAYES_RC) {
        for (int i = threadIdx.x; i < ng; i += blockDim.x) {
            CRng R;
            crng_site(R, D, c, rep, i, P_PI);
            double x[MAXDIST], sx = 0.0;
            for (int j = 0; j < nm; ++j)
                x[j] = d_rgamma((double)S->snpindist[i + j * ng] + D.alpha[j], 1.0, R, &err);
            for (int j = 0; j < nm; ++j) sx = sx + x[j];
            for (int j = 0; j < nm; ++j) S->p[i + j * ng] = x[j] / sx;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const bool keep = rep > D.burnin && rep % D.thin == 0;
        S->keep = keep;
        const double mu = S->mu[rep & 1];
        if (keep) {
            S->counter += 1;
            S->mu_store = S->mu_store + mu;
            // soda_bayes keeps varstore for every method (models.f90:530), regular_bayes
            // not for BayesA (models.f90:893-896)
            if (!(D.regular && m == SODAGPU_BAYES_A))
                for (int e = 0; e < ngm; ++e) S->varstore[e] = S->varstore[e] + S->varindist[e];
            S->vare_store = S->vare_store + S->vare;
            if (m != SODAGPU_BAYES_A) {
                S->included_store = S->included_store + S->included;
                for (int e = 0; e < ngm; ++e) S->snpstore[e] = S->snpstore[e] + S->snpindist[e];
                if (m != SODAGPU_BAYES_B && m != SODAGPU_BAYES_C)
                    for (int e = 0; e < ngm; ++e) S->pstore[e] = S->pstore[e] + S->p[e];
            }
            if (m != SODAGPU_BAYES_A && m != SODAGPU_BAYES_B) S->vara_store = S->vara_store + s_vara;
        }
        if (rep % D.thin == 0) {
            RunCtl *ctl = D.ctl;
            const int row = (ctl->trace_iter - 1) * D.chains + c;
            if (ctl->trace && row >= 0 && row < ctl->trace_cap) {
                sodagpu_trace_row *tr = ctl->trace + row;
                tr->chain = c;
                tr->rep = rep;
                tr->included = S->included;
                tr->pad = 0;
                tr->mu = mu;
                tr->vare = S->vare;
                tr->vara = S->vara;
                for (int j = 0; j < MAXDIST; ++j) {
                    tr->snpindist[j] = j < nm ? S->snpindist[j * ng] : 0;
                    tr->varindist[j] = j < nm ? S->varindist[j * ng] : 0.0;
                }
            }
        }
        // log_p and vare/gp for the next iteration (models.f90:198-199, 330-338)
        if (m != SODAGPU_BAYES_A) {
            for (int e = 0; e < ngm; ++e) S->log_p[e] = log(S->p[e]);
            for (int j = 1; j < nm; ++j) S->vare_gp[j] = S->vare / S->gp[j];
        }
        if (err) flag_err(D, 1);
    }
}

__global__ void __launch_bounds__(128) k_hyper(Dev D)
{
    hyper_body(D, vb_native());
}


// ra redraw (models.f90:523-525) and the per-SNP accumulators (528, 535-538, 544)
__device__ __forceinline__ void post_body(const Dev &D, const VB &vb)
{
    const int c = vb.y, rep = cur_rep(D);
    const ChainScal *S = &D.scal[c];
    const int t0 = vb.x * blockDim.x + threadIdx.x, stride = vb.nx * blockDim.x;
    const double sd = sqrt(S->vare);
    for (int i = t0; i < D.naind; i += stride) {
        CRng R;
        crng_site(R, D, c, rep, i, P_RA);
        store_ra(D, c, i, d_rnorm(0.0, sd, R));
    }
    if (!S->keep) return;
    const int m = D.method;
    for (int j = t0; j < D.p; j += stride) {
        const size_t o = (size_t)c * D.p + j;
        D.gstore[o] = D.gstore[o] + D.g[o];
        if (m != SODAGPU_BAYES_A) D.indist[o * D.nmix + (D.cls[o] - 1)] += 1u;
        if (m == SODAGPU_BAYES_A || m == SODAGPU_BAYES_B)
            D.vara_sstore[o] = D.vara_sstore[o] + D.vara_s[o];
    }
}

__global__ void __launch_bounds__(256) k_post(Dev D)
{
    post_body(D, vb_native());
}


// compute_residuals (utilities.f90:609-614), every `recal` iterations
__device__ __forceinline__ void recal_partial_body(const Dev &D, const VB &vb, int force)
{
    const int rep = cur_rep(D);
    if (!force && (D.recal <= 0 || rep % D.recal != 0)) return;
    const int c = vb.z, split = vb.y;
    const int i = vb.x * 256 + threadIdx.x;
    if (i >= D.n) return;
    const int per = (D.p + RECAL_SPLIT - 1) / RECAL_SPLIT;
    const int k0 = split * per, k1 = min(D.p, k0 + per);
    double acc = 0.0;
    const double *g = D.g + (size_t)c * D.p;
    for (int k = k0; k < k1; ++k) {
        const double gj = g[D.perm[k]];
        if (gj == 0.0) continue;
        acc = acc + D.xv[(size_t)k * 4 + D.G[(size_t)k * D.ldx + i]] * gj;
    }
    D.recal_part[((size_t)c * RECAL_SPLIT + split) * D.ldr + i] = acc;
}

__global__ void __launch_bounds__(256) k_recal_partial(Dev D, int force)
{
    recal_partial_body(D, vb_native(), force);
}


__device__ __forceinline__ void recal_apply_body(const Dev &D, const VB &vb, int force, int mu_slot)
{
    const int rep = cur_rep(D);
    if (!force && (D.recal <= 0 || rep % D.recal != 0)) return;
    const int c = vb.y;
    const int i = vb.x * 256 + threadIdx.x;
    if (i >= D.n) return;
    double d = 0.0;
    for (int s = 0; s < RECAL_SPLIT; ++s) d = d + D.recal_part[((size_t)c * RECAL_SPLIT + s) * D.ldr + i];
    const int slot = mu_slot >= 0 ? mu_slot : (rep & 1);
    store_r(D, c, i, D.y[i] - d - D.scal[c].mu[slot]);
}

__global__ void __launch_bounds__(256) k_recal_apply(Dev D, int force, int mu_slot)
{
    recal_apply_body(D, vb_native(), force, mu_slot);
}


// ---------------------------------------------------------------------------
// chain initialisation (models.f90:56-128)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_init_chain(Dev D, double vara0, double scale_va0)
{
    __shared__ double sh[33];
    const int c = blockIdx.x, m = D.method, ng = D.ngroup, nm = D.nmix;
    ChainScal *S = &D.scal[c];
    const double nn = (double)D.n;
    double sy = 0.0;
    for (int i = threadIdx.x; i < D.n; i += blockDim.x) sy += D.y[i];
    sy = block_sum(sy, sh);
    const double mu = sy / nn;
    double rr = 0.0, vy = 0.0;
    for (int i = threadIdx.x; i < D.n; i += blockDim.x) {
        const double v = (D.y[i] - 0.0) - mu;
        store_r(D, c, i, v);
        rr += v * v;
        vy += (D.y[i] - mu) * (D.y[i] - mu);
    }
    rr = block_sum(rr, sh);
    vy = block_sum(vy, sh);
    if (threadIdx.x == 0) {
        S->mu[0] = mu;
        S->mu[1] = mu;
        S->scale_va = scale_va0;
        S->vara = vara0;
        S->counter = 0;
        S->keep = 0;
        S->err = 0;
        S->included = 0;
        S->mu_store = S->vare_store = S->vara_store = S->included_store = 0.0;
        for (int e = 0; e < MAXGM; ++e) {
            S->snpstore[e] = S->pstore[e] = S->varstore[e] = 0.0;
            S->varindist[e] = 0.0;
            S->snpindist[e] = 0;
            S->p[e] = 0.0;
            S->log_p[e] = 0.0;
        }
        if (m != SODAGPU_BAYES_A) {
            if (m == SODAGPU_BAYES_B || m == SODAGPU_BAYES_C) {
                for (int i = 0; i < ng; ++i) {
                    S->p[i] = D.pizero;
                    S->p[i + ng] = 1.0 - D.pizero;
                }
            } else {
                for (int i = 0; i < ng; ++i) {
                    S->p[i] = 0.5;
                    double s = 0.0;
                    for (int j = 1; j < nm; ++j) S->p[i + j * ng] = 1.0 / D.mix[j];
                    for (int j = 1; j < nm; ++j) s = s + S->p[i + j * ng];
                    for (int j = 1; j < nm; ++j) S->p[i + j * ng] = 0.5 * S->p[i + j * ng] / s;
                }
            }
        }
        if (D.df_va <= 0.0) {
            const double vary = vy / (nn - 1.0);
            if (m == SODAGPU_BAYES_A) {
                S->vara = S->scale_va * vary / D.p;
            } else if (m == SODAGPU_BAYES_B) {
                S->vara = S->scale_va * vary / D.p / S->p[ng];
            } else {
                for (int i = 0; i < ng; ++i) {
                    double dp = 0.0;
                    for (int j = 0; j < nm; ++j) dp = dp + S->p[i + j * ng] * D.mix[j];
                    S->vara = S->vara + dp;
                }
                S->vara = S->scale_va * vary / D.p / S->vara;
            }
            S->scale_va = 0.0;
        } else {
            S->vara = S->scale_va * D.df_va / (D.df_va + 2.0);
        }
        for (int j = 0; j < nm; ++j) S->gp[j] = D.mix[j] * S->vara;
        const double scale = (rr + D.scale_ve * D.df_ve) / (nn + D.df_ve);
        CRng R;
        crng_site(R, D, c, 0, 0, P_VARE);
        int err = 0;
        S->vare = d_rscinvchi2(nn + D.df_ve, scale, R, &err);
        if (err) flag_err(D, 1);
        if (m != SODAGPU_BAYES_A) {
            for (int e = 0; e < ng * nm; ++e) S->log_p[e] = log(S->p[e]);
            for (int j = 1; j < nm; ++j) S->vare_gp[j] = S->vare / S->gp[j];
        }
    }
    __syncthreads();
    const double sd = sqrt(S->vare);
    for (int i = threadIdx.x; i < D.bs; i += blockDim.x) {
        double v = 0.0;
        if (i < D.naind) {
            CRng R;
            crng_site(R, D, c, 0, i, P_RA);
            v = d_rnorm(0.0, sd, R);
        }
        store_ra(D, c, i, v);
    }
}

__global__ void __launch_bounds__(256) k_init_snp(Dev D)
{
    const int c = blockIdx.y;
    const double vara = D.scal[c].vara;
    const int m = D.method;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < D.p; j += gridDim.x * blockDim.x) {
        const size_t o = (size_t)c * D.p + j;
        D.g[o] = 0.0;
        D.cls[o] = m == SODAGPU_BAYES_A ? 1 : 2;
        D.vara_s[o] = (m == SODAGPU_BAYES_A || m == SODAGPU_BAYES_B) ? vara : 0.0;
        D.gstore[o] = 0.0;
        D.vara_sstore[o] = 0.0;
        for (int q = 0; q < D.nmix; ++q) D.indist[o * D.nmix + q] = 0u;
    }
}

// ---------------------------------------------------------------------------
// host-side launch helpers
// ---------------------------------------------------------------------------
struct ProfScope {
    ProfHook *h;
    cudaStream_t st;
    int slot;
    ProfScope(ProfHook *h_, cudaStream_t st_, int cls) : h(h_), st(st_), slot(-1)
    {
        if (h && h->n < h->cap) {
            slot = h->n++;
            h->cls[slot] = cls;
            cudaEventRecord(h->ev[2 * slot], st);
        }
    }
    ~ProfScope()
    {
        if (slot >= 0) cudaEventRecord(h->ev[2 * slot + 1], st);
    }
};

// Launch with programmatic stream serialization: the kernel may start while
// the previous one in the stream finishes; it calls griddepcontrol.wait before
// reading that kernel's results.
template <typename... KArgs, typename... Args>
static cudaError_t launch_pdl(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                              Args... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, args...);
}

// Tensor-core subset: rhs tiles of 128 SNPs x K splits (one wave of one CTA
// per SM), then the update (row tiles of r on the tensor cores, ra tiles on
// the FP32 cores; two CTAs per SM).
template <int CT>
static cudaError_t launch_block_tc(const Dev &D, int b, int nblk_snps, int sm_count, const TcMaps *maps,
                                   cudaStream_t st, ProfHook *prof, bool rhs_only)
{
    const int mtiles = (nblk_snps + TC_TM - 1) / TC_TM;
    const int nrhs = maps->h_rtab[(size_t)b * D.tstride + mtiles];
    cudaError_t e;
    {
        ProfScope ps(prof, st, PROF_RHS);
        e = launch_pdl(k_rhs_tc<CT>, dim3(nrhs), dim3(TC_THREADS), RhsTc<CT>::SMEM, st, maps->rsp, maps->usp,
                       maps->rasp, D, b);
    }
    if (e != cudaSuccess) return e;
    {
        const int span = mtiles * TC_TM;
        ProfScope ps(prof, st, PROF_DRAW);
        e = launch_pdl(k_draw<SODAGPU_FP8, CT, true>, dim3((span * CT + 255) / 256), dim3(256), 0, st, D, b, 0, span);
    }
    if (e != cudaSuccess || rhs_only) return e != cudaSuccess ? e : cudaGetLastError();
    {
        ProfScope ps(prof, st, PROF_UPDATE);
        e = launch_pdl(k_update_tc<CT>, dim3(std::min(sm_count, TV_MAXG)), dim3(TV_THREADS), UpdTc<CT>::SMEM, st,
                       maps->d, maps->usp64, D, b);

    }
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

template <int MODE, int CT>
static cudaError_t launch_block(const Dev &D, int b, int nblk_snps, int sm_count, const TcMaps *maps, cudaStream_t st,
                               ProfHook *prof, bool rhs_only)
{
    if constexpr (MODE == SODAGPU_FP8 && CT >= 4) {
        if (D.tc) return launch_block_tc<CT>(D, b, nblk_snps, sm_count, maps, st, prof, rhs_only);
    }
    constexpr int MTS = 8 * SptOf<CT>::v;
    const int mtiles = (nblk_snps + MTS - 1) / MTS;
    const int nst = (D.ldx + RhsCfg<MODE>::KST - 1) / RhsCfg<MODE>::KST;
    // one wave: a CTA per SM (the pipeline fills most of its shared memory)
    int ks = sm_count / mtiles;
    ks = ks < 1 ? 1 : (ks > RHS_KSPLIT_MAX ? RHS_KSPLIT_MAX : ks);
    ks = ks > nst ? nst : ks;
    cudaError_t e;
    {
        ProfScope ps(prof, st, PROF_RHS);
        e = launch_pdl(k_rhs<MODE, CT>, dim3(mtiles * ks), dim3(256), rhs_smem_bytes<MODE, CT>(), st, D, b, ks);
    }
    if (e != cudaSuccess) return e;
    {
        ProfScope ps(prof, st, PROF_DRAW);
        e = launch_pdl(k_draw<MODE, CT, false>, dim3((nblk_snps * CT + 255) / 256), dim3(256), 0, st, D, b, ks,
                       nblk_snps);
    }
    if (e != cudaSuccess || rhs_only) return e != cudaSuccess ? e : cudaGetLastError();
    const int ntile = D.nr_ctas + (D.bs + UT - 1) / UT;
    {
        ProfScope ps(prof, st, PROF_UPDATE);
        e = launch_pdl(k_update<MODE, CT>, dim3(ntile), dim3(32 * UpdWarps<MODE, CT>::v),
                       update_smem_bytes_ct<MODE, CT>(D.bs), st, D, b);
    }
    return e != cudaSuccess ? e : cudaGetLastError();
}

template <int MODE>
static cudaError_t launch_block_mode(const Dev &D, int b, int nsnp, int sm_count, const TcMaps *maps, cudaStream_t st,
                                    ProfHook *prof, bool rhs_only = false)
{
    switch (D.chains) {
    case 1: return launch_block<MODE, 1>(D, b, nsnp, sm_count, maps, st, prof, rhs_only);
    case 2: return launch_block<MODE, 2>(D, b, nsnp, sm_count, maps, st, prof, rhs_only);
    case 4: return launch_block<MODE, 4>(D, b, nsnp, sm_count, maps, st, prof, rhs_only);
    case 8: return launch_block<MODE, 8>(D, b, nsnp, sm_count, maps, st, prof, rhs_only);
    case 16: return launch_block<MODE, 16>(D, b, nsnp, sm_count, maps, st, prof, rhs_only);
    default: return cudaErrorInvalidValue;
    }
}

int sweep_chain_count_supported(int c) { return c == 1 || c == 2 || c == 4 || c == 8 || c == 16; }

// Every kernel of an iteration asks for the largest shared-memory carveout,
// so that consecutive kernels never wait for the SMs to repartition L1 and
// shared memory (microseconds per kernel boundary otherwise).
template <typename K>
static cudaError_t max_carveout(K *kern)
{
    return cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                                (int)cudaSharedmemCarveoutMaxShared);
}

template <int MODE, bool TC>
static cudaError_t carve_draw()
{
    cudaError_t e = cudaSuccess;
    if constexpr (!TC) {
        e = max_carveout(k_draw<MODE, 1, false>);
        if (e == cudaSuccess) e = max_carveout(k_draw<MODE, 2, false>);
    }
    if (e == cudaSuccess) e = max_carveout(k_draw<MODE, 4, TC>);
    if (e == cudaSuccess) e = max_carveout(k_draw<MODE, 8, TC>);
    if (e == cudaSuccess) e = max_carveout(k_draw<MODE, 16, TC>);
    return e;
}

static cudaError_t carve_all()
{
    cudaError_t e = carve_draw<SODAGPU_FP64, false>();
    if (e == cudaSuccess) e = carve_draw<SODAGPU_FP32, false>();
    if (e == cudaSuccess) e = carve_draw<SODAGPU_FP8, false>();
    if (e == cudaSuccess) e = carve_draw<SODAGPU_FP8, true>();
    if (e == cudaSuccess) e = max_carveout(k_iter_begin);
    if (e == cudaSuccess) e = max_carveout(k_mu_partial);
    if (e == cudaSuccess) e = max_carveout(k_mu_apply);
    if (e == cudaSuccess) e = max_carveout(k_skipped);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_skipped, cudaFuncAttributeMaxDynamicSharedMemorySize, SS_SMEM_MAX);
    if (e == cudaSuccess) e = max_carveout(k_stats);
    if (e == cudaSuccess) e = max_carveout(k_hyper);
    if (e == cudaSuccess) e = max_carveout(k_post);
    if (e == cudaSuccess) e = max_carveout(k_recal_partial);
    if (e == cudaSuccess) e = max_carveout(k_recal_apply);
    return e;
}

template <int MODE, int CT>
static cudaError_t set_update_smem(int bs)
{
    cudaError_t e = cudaFuncSetAttribute(k_update<MODE, CT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)update_smem_bytes_ct<MODE, CT>(bs));
    return e == cudaSuccess ? max_carveout(k_update<MODE, CT>) : e;
}

template <int MODE>
static cudaError_t set_update_smem_mode(int bs)
{
    cudaError_t e = set_update_smem<MODE, 1>(bs);
    if (e == cudaSuccess) e = set_update_smem<MODE, 2>(bs);
    if (e == cudaSuccess) e = set_update_smem<MODE, 4>(bs);
    if (e == cudaSuccess) e = set_update_smem<MODE, 8>(bs);
    if (e == cudaSuccess) e = set_update_smem<MODE, 16>(bs);
    return e;
}

template <int MODE, int CT>
static cudaError_t set_rhs_smem()
{
    cudaError_t e = cudaFuncSetAttribute(k_rhs<MODE, CT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)rhs_smem_bytes<MODE, CT>());
    return e == cudaSuccess ? max_carveout(k_rhs<MODE, CT>) : e;
}

template <int MODE>
static cudaError_t set_rhs_smem_mode()
{
    cudaError_t e = set_rhs_smem<MODE, 1>();
    if (e == cudaSuccess) e = set_rhs_smem<MODE, 2>();
    if (e == cudaSuccess) e = set_rhs_smem<MODE, 4>();
    if (e == cudaSuccess) e = set_rhs_smem<MODE, 8>();
    if (e == cudaSuccess) e = set_rhs_smem<MODE, 16>();
    return e;
}

template <int CT>
static cudaError_t set_tc_smem()
{
    cudaError_t e = cudaFuncSetAttribute(k_rhs_tc<CT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)RhsTc<CT>::SMEM);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_update_tc<CT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)UpdTc<CT>::SMEM);
    if (e == cudaSuccess) e = max_carveout(k_rhs_tc<CT>);
    if (e == cudaSuccess) e = max_carveout(k_update_tc<CT>);

    return e;
}

int sweep_tc_supported(int precision, int chains, int bs)
{
    return precision == SODAGPU_FP8 && (chains == 4 || chains == 8 || chains == 16) && bs <= TV_MAXQ * TV_K;
}

int sweep_tc_update_tiles(int n) { return (n + TV_N - 1) / TV_N; }

size_t sweep_tc_vpart_floats(int n, int bs, int chains, int sm_count)
{
    const size_t slots = (size_t)sweep_tc_update_tiles(n) + (size_t)((bs + TV_N - 1) / TV_N) + (size_t)sm_count;
    return slots * (size_t)chains * TV_N;
}

int sweep_tc_rows(int chains) { return ((3 * chains + 15) / 16) * 16; }

__global__ void __launch_bounds__(256) k_tc_prepare(int8_t *G, Dev D, uint16_t *usp)
{
    for (int k = blockIdx.x; k < D.p; k += gridDim.x) {
        const double inv = D.xv[(size_t)k * 4 + 3];
        const double sc = inv != 0.0 ? 1.0 / inv : 1.0;
        const int len = D.ulen[k];
        const int64_t off = D.uoff[k];
        for (int i = threadIdx.x; i < D.ldu; i += blockDim.x) {
            const double v = i < len ? D.U64[off + i] * sc : 0.0;
            const __nv_bfloat16 h = __double2bfloat16(v);
            const double r1 = v - (double)__bfloat162float(h);
            const __nv_bfloat16 m = __double2bfloat16(r1);
            const __nv_bfloat16 l = __double2bfloat16(r1 - (double)__bfloat162float(m));
            usp[(size_t)k * D.ldu + i] = __bfloat16_as_ushort(h);
            usp[((size_t)D.p + k) * D.ldu + i] = __bfloat16_as_ushort(m);
            usp[((size_t)2 * D.p + k) * D.ldu + i] = __bfloat16_as_ushort(l);
        }
        if (inv == 0.0)
            for (int i = threadIdx.x; i < D.ldx; i += blockDim.x) G[(size_t)k * D.ldx + i] = 0;
    }
}

cudaError_t sweep_tc_prepare(int8_t *G, const Dev &D, cudaStream_t st)
{
    if (!D.usp || D.ldu <= 0) return cudaErrorInvalidValue;
    k_tc_prepare<<<std::min(D.p, 4096), 256, 0, st>>>(G, D, const_cast<uint16_t *>(D.usp));
    return cudaGetLastError();
}

int sweep_tc_code_blocks(const int *blk_sizes, int nb, int32_t *qoff)
{
    int tot = 0;
    for (int b = 0; b < nb; ++b) {
        qoff[b] = tot;
        tot += (blk_sizes[b] + TC_TM - 1) / TC_TM;
    }
    qoff[nb] = tot;
    return tot;
}

// Packed code block (q2, t): positions 128 (q2 - qoff[b]) .. of subset b x individuals 256 t .. (see
// TC_PACKED_BLOCK); positions past the subset and individuals past n hold 0.  One thread per 16-byte word
// (group g of 64 individuals, position k): four 16-byte loads of the position's column of G (64 bytes never
// straddle ldx, a multiple of 128), each folded into one 32-bit word.
__global__ void __launch_bounds__(256) k_tile_codes(const int8_t *G, Dev D, uint8_t *Gt, long long nblocks)
{
    constexpr int WORDS = TC_PACKED_BLOCK / 16;
    const long long total = nblocks * WORDS;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const long long blk = idx / WORDS;
        const int wi = (int)(idx - blk * WORDS), g = wi / TC_TM, k = wi - g * TC_TM;
        const int q2 = (int)(blk / D.nvt), t = (int)(blk - (long long)q2 * D.nvt);
        int lo = 0, hi = D.nb - 1;   // the subset: last b with qoff[b] <= q2
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (D.qoff[mid] <= q2) lo = mid;
            else hi = mid - 1;
        }
        const int ls = D.blk_ls[lo], N = D.blk_ls[lo + 1] - ls, r = (q2 - D.qoff[lo]) * TC_TM + k;
        const int i0 = t * TV_N + 64 * g;
        uint32_t out[4] = {0u, 0u, 0u, 0u};
        if (r < N && i0 + 64 <= D.ldx) {
            const uint4 *src = reinterpret_cast<const uint4 *>(G + (size_t)(ls + r) * D.ldx + i0);
#pragma unroll
            for (int w = 0; w < 4; ++w) {
                const uint4 v = src[w];   // individuals 16 w + 4 b + j: byte j of word b
                out[w] = (v.x & 0x03030303u) | ((v.y & 0x03030303u) << 2) | ((v.z & 0x03030303u) << 4) |
                         ((v.w & 0x03030303u) << 6);
            }
        }
        *reinterpret_cast<uint4 *>(Gt + blk * TC_PACKED_BLOCK + (size_t)wi * 16) =
            make_uint4(out[0], out[1], out[2], out[3]);
    }
}

// The individual-major copy: one thread per (block, stage, individual) writes
// that individual's 16 bytes, reading its 64 codes of the stage one position
// (column of G) at a time; a warp's 32 individuals read 32 consecutive bytes
// of each column.
__global__ void __launch_bounds__(256) k_tile_codes_ind(const int8_t *G, Dev D, uint8_t *Gu, long long nblocks)
{
    constexpr int WORDS = TC_PACKED_BLOCK / 16;   // 2 stages x 256 individuals
    const long long total = nblocks * WORDS;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const long long blk = idx / WORDS;
        const int wi = (int)(idx - blk * WORDS), st = wi / TV_N, il = wi - st * TV_N;
        const int q2 = (int)(blk / D.nvt), t = (int)(blk - (long long)q2 * D.nvt);
        int lo = 0, hi = D.nb - 1;   // the subset: last b with qoff[b] <= q2
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (D.qoff[mid] <= q2) lo = mid;
            else hi = mid - 1;
        }
        const int ls = D.blk_ls[lo], N = D.blk_ls[lo + 1] - ls, r0 = (q2 - D.qoff[lo]) * TC_TM + st * TV_K;
        const int i = t * TV_N + il;
        uint32_t out[4] = {0u, 0u, 0u, 0u};
        if (i < D.n) {
            for (int k = 0; k < TV_K && r0 + k < N; ++k) {
                const uint32_t c = (uint32_t)G[(size_t)(ls + r0 + k) * D.ldx + i] & 3u;
                out[k >> 4] |= c << (8 * (k & 3) + 2 * ((k >> 2) & 3));
            }
        }
        *reinterpret_cast<uint4 *>(Gu + blk * TC_PACKED_BLOCK + (size_t)wi * 16) =
            make_uint4(out[0], out[1], out[2], out[3]);
    }
}

cudaError_t sweep_tc_tile_codes(const int8_t *G, const Dev &D, uint8_t *Gt, uint8_t *Gu, long long nblocks,
                                int sm_count, cudaStream_t st)
{
    if (!Gt || !D.qoff || nblocks <= 0) return cudaErrorInvalidValue;
    const long long words = nblocks * (TC_PACKED_BLOCK / 16);
    const long long grid = std::min<long long>((words + 255) / 256, 16LL * sm_count);
    k_tile_codes<<<(unsigned)grid, 256, 0, st>>>(G, D, Gt, nblocks);
    if (Gu) k_tile_codes_ind<<<(unsigned)grid, 256, 0, st>>>(G, D, Gu, nblocks);
    return cudaGetLastError();
}

int sweep_tc_table_stride(int bs) { return (bs + TC_TM - 1) / TC_TM + 1; }

void sweep_tc_tables(const int *blk_sizes, int nb, int bs, int ldx, int sm_count, int32_t *rtab)
{
    const int stride = sweep_tc_table_stride(bs);
    const int nst = ldx / TC_KC;
    for (int b = 0; b < nb; ++b) {
        const int N = blk_sizes[b], tiles = (N + TC_TM - 1) / TC_TM;
        int32_t *rt = rtab + (size_t)b * stride;
        // K splits in proportion to each tile's MMAs (8 per genotype stage, 4 per U stage), largest
        // remainders first, so that the CTAs (one per SM, all of them) get equal MMA work
        std::vector<long long> w(tiles);
        std::vector<int> ks(tiles), cap(tiles);
        long long W = 0;
        for (int m = 0; m < tiles; ++m) {
            const int T = rhs_tc_stages(nst, N, m, true, nullptr);
            w[m] = 8LL * nst + 4LL * (T - nst);
            cap[m] = std::min(RHS_KSPLIT_MAX, T);
            W += w[m];
        }
        int total = 0;
        for (int m = 0; m < tiles; ++m) {
            ks[m] = std::max(1, std::min(cap[m], (int)(((long long)sm_count * w[m]) / W)));
            total += ks[m];
        }
        while (total < sm_count) {
            int best = -1;
            double bf = -1.0;
            for (int m = 0; m < tiles; ++m) {
                if (ks[m] >= cap[m]) continue;
                const double f = (double)sm_count * (double)w[m] / (double)W - ks[m];
                if (f > bf) {
                    bf = f;
                    best = m;
                }
            }
            if (best < 0) break;
            ++ks[best];
            ++total;
        }
        int acc = 0;
        for (int m = 0; m < tiles; ++m) {
            rt[m] = acc;
            acc += ks[m];
        }
        rt[tiles] = acc;
    }
}

// Raises the dynamic shared-memory limits of the rhs and update kernels (the
// update's for the largest subset size asked for so far in this process:
// the limit is per kernel, and every job's launches must stay within it).
cudaError_t sweep_prepare(int bs)
{
    static int s_max_bs = 0;
    if (bs < s_max_bs) bs = s_max_bs;
    s_max_bs = bs;
    {
        cudaError_t e = carve_all();
        if (e == cudaSuccess) e = set_tc_smem<4>();
        if (e == cudaSuccess) e = set_tc_smem<8>();
        if (e == cudaSuccess) e = set_tc_smem<16>();
        if (e != cudaSuccess) return e;
    }
    cudaError_t e = set_rhs_smem_mode<SODAGPU_FP64>();
    if (e == cudaSuccess) e = set_rhs_smem_mode<SODAGPU_FP32>();
    if (e == cudaSuccess) e = set_rhs_smem_mode<SODAGPU_FP8>();
    if (e != cudaSuccess) return e;
    if (update_smem_bytes_ct<SODAGPU_FP64, 16>(bs) > 220 * 1024) return cudaErrorInvalidValue;
    e = set_update_smem_mode<SODAGPU_FP64>(bs);
    if (e == cudaSuccess) e = set_update_smem_mode<SODAGPU_FP32>(bs);
    if (e == cudaSuccess) e = set_update_smem_mode<SODAGPU_FP8>(bs);
    return e;
}

cudaError_t sweep_enqueue_iteration(const Dev &D, const int *blk_sizes, int sm_count, const TcMaps *maps,
                                    cudaStream_t st, ProfHook *prof)
{
    if (D.tc && !maps) return cudaErrorInvalidValue;
    const int C = D.chains;
    {
        ProfScope ps(prof, st, PROF_MU);
        k_iter_begin<<<1, 1, 0, st>>>(D);
        k_mu_partial<<<dim3(D.nr_ctas, C), ROW_THREADS, 0, st>>>(D);
        k_mu_apply<<<dim3(D.nr_ctas, C), ROW_THREADS, 0, st>>>(D);
    }
    for (int b = 0; b < D.nb; ++b) {
        const int nsnp = blk_sizes[b];
        cudaError_t e;
        if (D.precision == SODAGPU_FP64) e = launch_block_mode<SODAGPU_FP64>(D, b, nsnp, sm_count, maps, st, prof);
        else if (D.precision == SODAGPU_FP32)
            e = launch_block_mode<SODAGPU_FP32>(D, b, nsnp, sm_count, maps, st, prof);
        else e = launch_block_mode<SODAGPU_FP8>(D, b, nsnp, sm_count, maps, st, prof);
        if (e != cudaSuccess) return e;
    }
    {
        ProfScope ps(prof, st, PROF_OTHER);
        if (D.nskipped > 0) {
            const size_t sm = (size_t)D.n * sizeof(double) <= (size_t)SS_SMEM_MAX ? (size_t)D.n * sizeof(double) : 0;
            k_skipped<<<C, SS_THREADS, sm, st>>>(D);
        }
        k_stats<<<dim3(NSTAT + D.nr_ctas, C), 256, 0, st>>>(D);
        k_hyper<<<C, 128, 0, st>>>(D);
        const int pgrid = (D.p + 255) / 256 < 4 * sm_count ? (D.p + 255) / 256 : 4 * sm_count;
        k_post<<<dim3(pgrid > 0 ? pgrid : 1, C), 256, 0, st>>>(D);
        k_recal_partial<<<dim3((D.n + 255) / 256, RECAL_SPLIT, C), 256, 0, st>>>(D, 0);
        k_recal_apply<<<dim3((D.n + 255) / 256, C), 256, 0, st>>>(D, 0, -1);
    }
    return cudaGetLastError();
}

cudaError_t sweep_enqueue_init(const Dev &D, double vara0, double scale_va0, int sm_count, cudaStream_t st)
{
    k_init_chain<<<D.chains, 256, 0, st>>>(D, vara0, scale_va0);
    const int pgrid = (D.p + 255) / 256 < 4 * sm_count ? (D.p + 255) / 256 : 4 * sm_count;
    k_init_snp<<<dim3(pgrid > 0 ? pgrid : 1, D.chains), 256, 0, st>>>(D);
    return cudaGetLastError();
}

cudaError_t sweep_enqueue_subset(const Dev &D, int b, int nsnp, int sm_count, const TcMaps *maps, cudaStream_t st,
                                 bool rhs_only)
{
    if (D.tc && !maps) return cudaErrorInvalidValue;
    if (D.precision == SODAGPU_FP64) return launch_block_mode<SODAGPU_FP64>(D, b, nsnp, sm_count, maps, st, nullptr, rhs_only);
    if (D.precision == SODAGPU_FP32) return launch_block_mode<SODAGPU_FP32>(D, b, nsnp, sm_count, maps, st, nullptr, rhs_only);
    return launch_block_mode<SODAGPU_FP8>(D, b, nsnp, sm_count, maps, st, nullptr, rhs_only);
}

// ---------------------------------------------------------------------------
// Loading one chain's state (the inverse of sodagpu_get_state): the residuals
// with every copy derived from them (FP32 copy or bf16 split, and the 128-row
// partial sums of r that the FP8 centring reads), the per-SNP state, and the
// chain scalars with the tables the draws read (models.f90:198-199, 330-338).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(ROW_THREADS) k_set_rows(Dev D, int c, const double *r)
{
    __shared__ double sh[33];
    const int i = blockIdx.x * ROW_TILE + threadIdx.x;
    double v = 0.0;
    if (i < D.n) {
        v = r[i];
        store_r(D, c, i, v);
    }
    const double t = block_sum(v, sh);
    if (threadIdx.x == 0) D.rsum[(size_t)c * D.nr_ctas + blockIdx.x] = t;
}

__global__ void __launch_bounds__(256) k_set_snps(Dev D, int c, const double *g, const int32_t *cls, const double *vs,
                                                  const double *ra, const double *pi, double mu, double vare,
                                                  double vara, int included)
{
    const int t0 = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
    for (int j = t0; j < D.p; j += stride) {
        const size_t o = (size_t)c * D.p + j;
        D.g[o] = g[j];
        D.cls[o] = cls[j];
        D.vara_s[o] = vs[j];
    }
    for (int i = t0; i < D.bs; i += stride) store_ra(D, c, i, i < D.naind ? ra[i] : 0.0);
    if (t0 == 0) {
        ChainScal *S = &D.scal[c];
        S->mu[0] = S->mu[1] = mu;
        S->vare = vare;
        S->vara = vara;
        S->included = included;
        const int ngm = D.ngroup * D.nmix;
        if (pi)
            for (int e = 0; e < ngm; ++e) S->p[e] = pi[e];
        for (int j = 0; j < D.nmix; ++j) S->gp[j] = D.mix[j] * vara;
        if (D.method != SODAGPU_BAYES_A) {
            for (int e = 0; e < ngm; ++e) S->log_p[e] = log(S->p[e]);
            for (int j = 1; j < D.nmix; ++j) S->vare_gp[j] = vare / S->gp[j];
        }
    }
}

cudaError_t sweep_set_state(const Dev &D, int c, const double *g, const int32_t *cls, const double *vs,
                            const double *r, const double *ra, const double *pi, double mu, double vare, double vara,
                            int included, cudaStream_t st)
{
    k_set_rows<<<D.nr_ctas, ROW_THREADS, 0, st>>>(D, c, r);
    const int grid = std::max(1, std::min((D.p + 255) / 256, 1024));
    k_set_snps<<<grid, 256, 0, st>>>(D, c, g, cls, vs, ra, pi, mu, vare, vara, included);
    return cudaGetLastError();
}

cudaError_t sweep_enqueue_recal(const Dev &D, double mu_slot_unused, cudaStream_t st)
{
    (void)mu_slot_unused;
    k_recal_partial<<<dim3((D.n + 255) / 256, RECAL_SPLIT, D.chains), 256, 0, st>>>(D, 1);
    k_recal_apply<<<dim3((D.n + 255) / 256, D.chains), 256, 0, st>>>(D, 1, -1);
    return cudaGetLastError();
}

}  // namespace soda

// ---------------------------------------------------------------------------
// Several jobs in one launch per kernel (the CUDA-core kernels; every job of a
// batch has the same precision and chain count).  Each wrapper finds its job
// and block coordinates (jg_locate) and runs the same body as the plain
// kernel, so a job's results do not depend on the batch it runs in.
// ---------------------------------------------------------------------------
namespace soda {

__global__ void k_iter_begin_m(const __grid_constant__ JobGrid G)
{
    VB vb;
    const int j = jg_locate(G, vb);
    iter_begin_body(G.dev[j], vb);
}

__global__ void __launch_bounds__(ROW_THREADS) k_mu_partial_m(const __grid_constant__ JobGrid G)
{
    VB vb;
    const int j = jg_locate(G, vb);
    mu_partial_body(G.dev[j], vb);
}

__global__ void __launch_bounds__(ROW_THREADS) k_mu_apply_m(const __grid_constant__ JobGrid G)
{
    VB vb;
    const int j = jg_locate(G, vb);
    mu_apply_body(G.dev[j], vb);
}

__global__ void __launch_bounds__(SS_THREADS) k_skipped_m(const __grid_constant__ JobGrid G)
{
    VB vb;
    const int j = jg_locate(G, vb);
    skipped_body(G.dev[j], vb);
}

__global__ void __launch_bounds__(256) k_stats_m(const __grid_constant__ JobGrid G)
{
    VB vb;
    const int j = jg_locate(G, vb);
    stats_body(G.dev[j], vb);
}

__global__ void __launch_bounds__(128) k_hyper_m(const __grid_constant__ JobGrid G)
{
    VB vb;
    const int j = jg_locate(G, vb);
    hyper_body(G.dev[j], vb);
}

__global__ void __launch_bounds__(256) k_post_m(const __grid_constant__ JobGrid G)
{
    VB vb;
    const int j = jg_locate(G, vb);
    post_body(G.dev[j], vb);
}

__global__ void __launch_bounds__(256) k_recal_partial_m(const __grid_constant__ JobGrid G)
{
    VB vb;
    const int j = jg_locate(G, vb);
    recal_partial_body(G.dev[j], vb, 0);
}

__global__ void __launch_bounds__(256) k_recal_apply_m(const __grid_constant__ JobGrid G)
{
    VB vb;
    const int j = jg_locate(G, vb);
    recal_apply_body(G.dev[j], vb, 0, -1);
}

template <int MODE, int CT>
__global__ void __launch_bounds__(256, 1) k_rhs_m(const __grid_constant__ JobGrid G)
{
    VB vb;
    const int j = jg_locate(G, vb);
    rhs_body<MODE, CT>(G.dev[j], vb, G.arg[j][0], G.arg[j][1]);
}

template <int MODE, int CT>
__global__ void __launch_bounds__(256, 1) k_draw_m(const __grid_constant__ JobGrid G)
{
    VB vb;
    const int j = jg_locate(G, vb);
    draw_body<MODE, CT, false>(G.dev[j], vb, G.arg[j][0], G.arg[j][1], G.arg[j][2]);
}

template <int MODE, int CT>
__global__ void __launch_bounds__(32 * UpdWarps<MODE, CT>::v) k_update_m(const __grid_constant__ JobGrid G)
{
    VB vb;
    const int j = jg_locate(G, vb);
    update_body<MODE, CT>(G.dev[j], vb, G.arg[j][0]);
}

namespace {

// Builds the JobGrid of one launch from each job's grid (x, y, z; all zero
// for a job that sits the launch out) and arguments.
struct GridBuilder {
    JobGrid g;
    explicit GridBuilder(const Dev *ddev, int njobs)
    {
        memset(&g, 0, sizeof g);
        g.dev = ddev;
        g.njobs = njobs;
    }
    void set(int j, int gx, int gy, int gz, int a0 = 0, int a1 = 0, int a2 = 0)
    {
        const int n = gx > 0 && gy > 0 && gz > 0 ? gx * gy * gz : 0;
        g.gx[j] = gx > 0 ? gx : 1;
        g.gy[j] = gy > 0 ? gy : 1;
        g.off[j + 1] = g.off[j] + n;
        g.arg[j][0] = a0;
        g.arg[j][1] = a1;
        g.arg[j][2] = a2;
    }
    int total() const { return g.off[g.njobs]; }
};

template <int MODE, int CT>
static cudaError_t multi_step(const BatchPlan &P, int t, cudaStream_t st)
{
    const int nj = P.njobs;
    constexpr int MTS = 8 * SptOf<CT>::v;
    GridBuilder rhs(P.ddev, nj), draw(P.ddev, nj), upd(P.ddev, nj);
    size_t usmem = 0;
    for (int j = 0; j < nj; ++j) {
        const Dev &D = P.hdev[j];
        if (t >= D.nb) {
            rhs.set(j, 0, 0, 0);
            draw.set(j, 0, 0, 0);
            upd.set(j, 0, 0, 0);
            continue;
        }
        const int N = P.blk_sizes[j][t];
        const int mtiles = (N + MTS - 1) / MTS;
        const int ks = P.ksplit[j];
        rhs.set(j, mtiles * ks, 1, 1, t, ks);
        draw.set(j, (N * CT + 255) / 256, 1, 1, t, ks, N);
        upd.set(j, D.nr_ctas + (D.bs + UT - 1) / UT, 1, 1, t);
        usmem = std::max(usmem, update_smem_bytes_ct<MODE, CT>(D.bs));
    }
    if (rhs.total() == 0) return cudaSuccess;
    cudaError_t e = launch_pdl(k_rhs_m<MODE, CT>, dim3(rhs.total()), dim3(256), rhs_smem_bytes<MODE, CT>(), st, rhs.g);
    if (e == cudaSuccess) e = launch_pdl(k_draw_m<MODE, CT>, dim3(draw.total()), dim3(256), 0, st, draw.g);
    if (e == cudaSuccess)
        e = launch_pdl(k_update_m<MODE, CT>, dim3(upd.total()), dim3(32 * UpdWarps<MODE, CT>::v), usmem, st, upd.g);
    return e;
}

template <int MODE>
static cudaError_t multi_step_mode(const BatchPlan &P, int t, cudaStream_t st)
{
    switch (P.hdev[0].chains) {
    case 1: return multi_step<MODE, 1>(P, t, st);
    case 2: return multi_step<MODE, 2>(P, t, st);
    case 4: return multi_step<MODE, 4>(P, t, st);
    case 8: return multi_step<MODE, 8>(P, t, st);
    case 16: return multi_step<MODE, 16>(P, t, st);
    default: return cudaErrorInvalidValue;
    }
}

template <int MODE, int CT>
static cudaError_t multi_attrs(size_t usmem)
{
    cudaError_t e = cudaFuncSetAttribute(k_rhs_m<MODE, CT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)rhs_smem_bytes<MODE, CT>());
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_update_m<MODE, CT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)usmem);
    if (e == cudaSuccess) e = max_carveout(k_rhs_m<MODE, CT>);
    if (e == cudaSuccess) e = max_carveout(k_draw_m<MODE, CT>);
    if (e == cudaSuccess) e = max_carveout(k_update_m<MODE, CT>);
    return e;
}

template <int MODE>
static cudaError_t multi_attrs_mode(int chains, int max_bs)
{
    switch (chains) {
    case 1: return multi_attrs<MODE, 1>(update_smem_bytes_ct<MODE, 1>(max_bs));
    case 2: return multi_attrs<MODE, 2>(update_smem_bytes_ct<MODE, 2>(max_bs));
    case 4: return multi_attrs<MODE, 4>(update_smem_bytes_ct<MODE, 4>(max_bs));
    case 8: return multi_attrs<MODE, 8>(update_smem_bytes_ct<MODE, 8>(max_bs));
    case 16: return multi_attrs<MODE, 16>(update_smem_bytes_ct<MODE, 16>(max_bs));
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace

cudaError_t sweep_multi_prepare(int precision, int chains, int max_bs)
{
    cudaError_t e = sweep_prepare(max_bs);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_skipped_m, cudaFuncAttributeMaxDynamicSharedMemorySize, SS_SMEM_MAX);
    if (e != cudaSuccess) return e;
    if (precision == SODAGPU_FP64) return multi_attrs_mode<SODAGPU_FP64>(chains, max_bs);
    if (precision == SODAGPU_FP32) return multi_attrs_mode<SODAGPU_FP32>(chains, max_bs);
    return multi_attrs_mode<SODAGPU_FP8>(chains, max_bs);
}

template <int MODE, int CT>
static int multi_split(int N, int ldx, int cta_share)
{
    constexpr int MTS = 8 * SptOf<CT>::v;
    const int mtiles = (N + MTS - 1) / MTS;
    const int nst = (ldx + RhsCfg<MODE>::KST - 1) / RhsCfg<MODE>::KST;
    int ks = cta_share / std::max(1, mtiles);
    ks = std::max(1, std::min(ks, RHS_KSPLIT_MAX));
    return std::min(ks, std::max(1, nst));
}

template <int MODE>
static int multi_split_mode(int N, int chains, int ldx, int cta_share)
{
    switch (chains) {
    case 1: return multi_split<MODE, 1>(N, ldx, cta_share);
    case 2: return multi_split<MODE, 2>(N, ldx, cta_share);
    case 4: return multi_split<MODE, 4>(N, ldx, cta_share);
    case 8: return multi_split<MODE, 8>(N, ldx, cta_share);
    default: return multi_split<MODE, 16>(N, ldx, cta_share);
    }
}

int sweep_multi_rhs_split(int precision, int N, int chains, int ldx, int cta_share)
{
    if (precision == SODAGPU_FP64) return multi_split_mode<SODAGPU_FP64>(N, chains, ldx, cta_share);
    if (precision == SODAGPU_FP32) return multi_split_mode<SODAGPU_FP32>(N, chains, ldx, cta_share);
    return multi_split_mode<SODAGPU_FP8>(N, chains, ldx, cta_share);
}

cudaError_t sweep_enqueue_iteration_multi(const BatchPlan &P, int sm_count, cudaStream_t st)
{
    const int nj = P.njobs;
    if (nj < 1 || nj > MAXJOBS) return cudaErrorInvalidValue;
    const int prec = P.hdev[0].precision;
    GridBuilder one(P.ddev, nj), rows(P.ddev, nj);
    int maxnb = 0;
    for (int j = 0; j < nj; ++j) {
        const Dev &D = P.hdev[j];
        one.set(j, 1, 1, 1);
        rows.set(j, D.nr_ctas, D.chains, 1);
        maxnb = std::max(maxnb, D.nb);
    }
    k_iter_begin_m<<<one.total(), 1, 0, st>>>(one.g);
    k_mu_partial_m<<<rows.total(), ROW_THREADS, 0, st>>>(rows.g);
    k_mu_apply_m<<<rows.total(), ROW_THREADS, 0, st>>>(rows.g);
    for (int t = 0; t < maxnb; ++t) {
        cudaError_t e = prec == SODAGPU_FP64   ? multi_step_mode<SODAGPU_FP64>(P, t, st)
                        : prec == SODAGPU_FP32 ? multi_step_mode<SODAGPU_FP32>(P, t, st)
                                               : multi_step_mode<SODAGPU_FP8>(P, t, st);
        if (e != cudaSuccess) return e;
    }
    GridBuilder skp(P.ddev, nj), stats(P.ddev, nj), hyp(P.ddev, nj), post(P.ddev, nj), rp(P.ddev, nj),
        ra(P.ddev, nj);
    size_t ssm = 0;
    for (int j = 0; j < nj; ++j) {
        const Dev &D = P.hdev[j];
        const int C = D.chains;
        skp.set(j, D.nskipped > 0 ? C : 0, 1, 1);
        if (D.nskipped > 0 && (size_t)D.n * sizeof(double) <= (size_t)SS_SMEM_MAX)
            ssm = std::max(ssm, (size_t)D.n * sizeof(double));
        stats.set(j, NSTAT + D.nr_ctas, C, 1);
        hyp.set(j, C, 1, 1);
        const int pgrid = (D.p + 255) / 256 < 4 * sm_count ? (D.p + 255) / 256 : 4 * sm_count;
        post.set(j, pgrid > 0 ? pgrid : 1, C, 1);
        rp.set(j, (D.n + 255) / 256, RECAL_SPLIT, C);
        ra.set(j, (D.n + 255) / 256, C, 1);
    }
    if (skp.total() > 0) k_skipped_m<<<skp.total(), SS_THREADS, ssm, st>>>(skp.g);
    k_stats_m<<<stats.total(), 256, 0, st>>>(stats.g);
    k_hyper_m<<<hyp.total(), 128, 0, st>>>(hyp.g);
    k_post_m<<<post.total(), 256, 0, st>>>(post.g);
    k_recal_partial_m<<<rp.total(), 256, 0, st>>>(rp.g);
    k_recal_apply_m<<<ra.total(), 256, 0, st>>>(ra.g);
    return cudaGetLastError();
}

}  // namespace soda
