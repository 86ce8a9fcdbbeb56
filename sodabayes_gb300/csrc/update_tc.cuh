// update_tc.cuh — tensor-core residual update of one subset for FP8 mode with
// several chains (models.f90:164-174 for every chain at once), included by
// sweep.cu after rhs_tc.cuh.
//
//   r  += X_b delta = sum_j x0_j delta_j + G_b (delta / sd)
//   ra += U_b delta = (U_b sd) (delta / sd)
//
// Both products run on tcgen05 as D (M = 128 individuals or rows of U, N =
// the 3 * chains rows of the delta split) = A B':
//   A for r = the genotype codes of 128 individuals x 16 subset positions per
//     MMA, in tensor memory: the converter warps load them 2-bit packed
//     (individual-major, 16 bytes per individual and 64-position stage)
//     straight from global memory into registers, several units ahead, widen
//     them to bf16 and store them with tcgen05.st (lane = individual), so the
//     codes never pass through shared memory;
//   A for ra = one bf16 term of sd * U (128 rows of U), loaded by TMA into an
//     MN-major shared-memory operand (the factor is stored column by column);
//   B (K-major, TMA) = the bf16 hi/mid/lo split of delta/sd written by the
//     draws (delta itself for columns with sd = 0, whose codes are zero):
//     rows term * chains + c, K = subset positions, 64 per stage;
//   D = 128 x 3C FP32 in tensor memory (lane = individual, column = term and
//     chain), two per unit (256 individuals), double-buffered by segment.
// Measured on GB300: an N = 48 MMA costs 44 cycles against 128 for an N = 256
// one, and a 32 KB widened operand costs about as many cycles to store in
// shared memory as the MMAs that read it; in tensor memory both costs drop.
//
// Work units: (row tile of 256 individuals, stage of 64 positions) and, for
// ra, (tile of 256 rows of U, stage, U term); an upper-triangular factor meets
// an ra tile only from its first row on.  The plan depends on the subset's
// shape alone, so it is made, and the first code words are loaded, before
// the draws of this subset complete.  The units are laid out row tiles first
// and split over the CTAs (stream-K, one CTA per SM) in equal shares of
// weight, an ra unit weighing 6/5 of a row unit; a CTA's consecutive units of
// one tile form a segment, whose accumulator rows go to vpart as FP32 partial
// sums (hi + mid + lo per chain).  After a grid-wide barrier (one CTA per SM,
// all resident; the wait is bounded) the non-epilogue warps of every CTA take
// an equal share of the (128-element half tile, chain) pairs, whose old
// residuals each loaded as soon as its own role ended: it adds the pair's segments in
// segment order (deterministic) and the centring term sum_j x0_j delta_j, and
// writes the FP64 residuals.  Spreading this over every SM matters: GB300
// runs FP64 at a small fraction of its FP32 rate, and a tile's residuals take
// about as long on one SM's FP64 pipe as a third of the unit loop.
//
// Warp roles (mbarrier hand-offs, every wait bounded): warp 8 issues the TMA
// loads, warps 0-7 widen the codes, warp 9 runs the MMA loop on warp-uniform
// values with one elected lane issuing, warps 10-13 reduce the centring term
// and move finished accumulators to vpart; warps 0-9 then take part in the
// reductions.  A CTA's row units come before its ra units.  Unit s uses slot
// s % TV_NS of both operands, and one commit of its MMAs frees both:
//   producer: wait free (MMAs of s - TV_NS); load the delta tile (+ tx) on
//     fulla; for an ra unit also load the U tile (+ tx) on fullb (the U
//     tiles of the first TV_NS units load before the dependency wait);
//   converters (row units only): wait free; write the codes into the slot's
//     tensor-memory operand; arrive on conv;
//   MMA: wait conv (row unit) or fullb (ra unit), and fulla; 8 MMAs; commit
//     to free.
// Every wait is at most one phase behind its barrier, so the parity waits are
// exact (checked by a CPU model of this protocol in the tests).
#pragma once

namespace soda {

constexpr int TV_N = 256;          // individuals per row tile / rows of U per ra tile (two MMA M halves)
constexpr int TV_K = 64;           // subset positions per stage
constexpr int TV_NS = 5;           // operand slots: delta-split tile, and the codes or the U tile
constexpr int TV_NC = 6;           // shared-memory slots of packed codes (4 KB: one row unit each)
constexpr int TV_MAXQ = 256;       // stages per subset (subsets up to 16384 SNPs)
constexpr int TV_MAXRA = 64;       // ra tiles per subset
constexpr int TV_THREADS = 480;    // 8 converter warps, TMA, MMA, 4 epilogue warps, code loader
constexpr int TV_NW = TV_THREADS / 32;
constexpr int TV_NPW = 10;         // warps that take part in the reductions (all but the epilogue warps)
constexpr int TV_WROW = 5, TV_WRA = 6;   // weights of a row unit and an ra unit in the split (ra
                                         // units stream their U tile from DRAM: ~1.2x the time)
constexpr int TV_MAXG = 512;       // CTAs (one per SM)
constexpr int TV_CONV = 256;
constexpr int TV_CONV_WARPS = TV_CONV / 32;   // each converter warp arrives once per unit
constexpr int TV_WARP_TMA = 8, TV_WARP_MMA = 9, TV_WARP_EPI = 10, TV_WARP_CODES = 14;

template <int CT>
struct UpdTc {
    static constexpr int NB = RhsTc<CT>::NB;           // MMA N: 3 * chains rounded up to 16
    static constexpr int ROWS = 3 * CT;                // delta-split rows in use
    static constexpr int RAW_A = NB * TV_K * 2;        // delta split tile: NB rows x 64 bf16, 128-byte swizzle
    static constexpr int ASTRIDE = RAW_A;              // the MMAs read exactly the NB rows the TMA writes
    static constexpr int AREG = TV_NS * ASTRIDE;
    static constexpr int BOP = TV_K * TV_N * 2;        // U tile of an ra unit: 256 rows x 64 bf16
    static constexpr int BOP0 = AREG;
    static constexpr int CODE = TV_N * 16;             // packed codes of one row unit (256 individuals)
    static constexpr int CODE0 = BOP0 + TV_NS * BOP;
    static constexpr size_t SMEM = 1024 + (size_t)CODE0 + (size_t)TV_NC * CODE;
    // tensor memory: accumulators (segment parity p, half h) at columns NB (2p + h), the codes
    // operands (slot sl, half h) at 192 + 64 sl + 32 h (32 columns: 64 positions, two bf16 each)
    static constexpr int TM_ACC = NB;
    static constexpr int TM_OPS = 192;
    static_assert(RAW_A % 1024 == 0 && AREG % 1024 == 0 && BOP % 1024 == 0, "buffer alignment");
    static_assert(4 * NB <= TM_OPS && TM_OPS + 64 * TV_NS <= 512, "tensor memory");
    static_assert(SMEM <= 227 * 1024, "shared memory");
};

// Units of one subset, as every role decodes them.
struct UnitPlan {
    int nq, nvt, nra, R, W;          // stages, row tiles, ra tiles, row units, all units
    int qs[TV_MAXRA];                // first stage of each ra tile
    int pref[TV_MAXRA + 1];          // first ra unit of each ra tile (relative to R)
};

struct Unit {
    int kind, tile, q, term;         // kind 0: r, 1: ra; tile; stage; U term
};

__device__ __forceinline__ Unit decode_unit(const UnitPlan &P, int u, int &ra_hint)
{
    Unit x;
    if (u < P.R) {
        x.kind = 0;
        x.tile = u / P.nq;
        x.q = u - x.tile * P.nq;
        x.term = 0;
        return x;
    }
    const int v = u - P.R;
    int a = ra_hint;
    while (a + 1 < P.nra && P.pref[a + 1] <= v) ++a;
    ra_hint = a;
    const int w = v - P.pref[a];
    x.kind = 1;
    x.tile = a;
    x.q = P.qs[a] + w / 3;
    x.term = w % 3;
    return x;
}

// Phase index of fullb of slot s % TV_NS for ra unit s: the slot's earlier
// units less its row units (the CTA's nrow row units come first).
__device__ __forceinline__ int ra_phase(int s, int nrow)
{
    const int sl = s % TV_NS;
    return s / TV_NS - (nrow > sl ? (nrow - 1 - sl) / TV_NS + 1 : 0);
}

// decode_unit without a hint (binary search over the ra tiles), for lanes that
// decode different units at once.
__device__ __forceinline__ Unit decode_unit_bs(const UnitPlan &P, int u)
{
    Unit x;
    if (u < P.R) {
        x.kind = 0;
        x.tile = u / P.nq;
        x.q = u - x.tile * P.nq;
        x.term = 0;
        return x;
    }
    const int v = u - P.R;
    int lo = 0, hi = P.nra - 1;   // last a with pref[a] <= v
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (P.pref[mid] <= v) lo = mid;
        else hi = mid - 1;
    }
    const int w = v - P.pref[lo];
    x.kind = 1;
    x.tile = lo;
    x.q = P.qs[lo] + w / 3;
    x.term = w % 3;
    return x;
}

// First unit of CTA q when the W units (R row units, then ra units) are split
// over G CTAs in equal shares of weight (TV_WROW per row unit, TV_WRA per ra
// unit): the first unit whose cumulative weight reaches q / G of the total.
__device__ __forceinline__ int split_bound(const UnitPlan &P, int q, int G)
{
    const long long wr = (long long)TV_WROW * P.R;
    const long long tw = wr + (long long)TV_WRA * (P.W - P.R);
    const long long target = (q * tw) / G;
    if (target <= wr) return (int)((target + TV_WROW - 1) / TV_WROW);
    return P.R + (int)((target - wr + TV_WRA - 1) / TV_WRA);
}

// CTA holding unit u: the last q with bnd[q] <= u.
__device__ __forceinline__ int unit_cta(const int *bnd, int u, int G)
{
    int lo = 0, hi = G - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (bnd[mid] <= u) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// The centring term sum_j x0_j delta_j of the subset per chain into s_k0,
// from the per-CTA sums of the draws (parts in a fixed order), by the 128
// threads of the epilogue warps.
template <int CT>
__device__ __forceinline__ void update_k0(const Dev &D, int b, int t, double *s_k0p, double *s_k0)
{
    constexpr int PARTS = 128 / CT;
    const int N = D.blk_ls[b + 1] - D.blk_ls[b];
    const int c = t / PARTS, part = t % PARTS;
    const int ntl = (((N + TC_TM - 1) / TC_TM) * TC_TM * CT + 255) / 256;
    double a = 0.0;
    for (int q0 = part; q0 < ntl; q0 += 8 * PARTS) {
        double v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int q = q0 + u * PARTS;
            v[u] = q < ntl ? __ldcg(D.k0part + (size_t)q * CT + c) : 0.0;
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) a += v[u];
    }
    s_k0p[t] = a;
    asm volatile("bar.sync 1, 128;" ::: "memory");
    if (t < CT) {
        double s = 0.0;
        for (int q = 0; q < PARTS; ++q) s += s_k0p[t * PARTS + q];
        s_k0[t] = s;
    }
    asm volatile("bar.sync 1, 128;" ::: "memory");
}

// Units [u0, u1) of global tile tg (row tiles, then ra tiles).
__device__ __forceinline__ void tile_units(const UnitPlan &P, int tg, int &u0, int &u1)
{
    if (tg < P.nvt) {
        u0 = tg * P.nq;
        u1 = u0 + P.nq;
    } else {
        u0 = P.R + P.pref[tg - P.nvt];
        u1 = P.R + P.pref[tg - P.nvt + 1];
    }
}

// One (128-element half tile, chain) pair of the reductions: global tile tg
// (row tiles, then ra tiles), half h, chain c, the CTAs sl..sh whose segments
// cover the tile (sl > sh: no unit touched it, nothing changes) and the old
// values (r or ra) of the half, lane l holding elements l + 32k.  Everything
// here is known before the grid barrier: nothing else writes those values
// during the update.
struct PairJob {
    int tg, h, c, sl, sh;
    double rold[4];
};

template <int CT>
__device__ __forceinline__ void pair_prepare(const Dev &D, const UnitPlan &P, const int *bnd, int G, int pr, int npair,
                                             int N, PairJob &j)
{
    j.tg = j.h = j.c = 0;
    j.sl = 1;
    j.sh = 0;
    if (pr >= npair) return;
    const int hh = pr / CT;
    j.c = pr - hh * CT;
    j.tg = hh >> 1;
    j.h = hh & 1;
    int u0, u1;
    tile_units(P, j.tg, u0, u1);
    if (u1 <= u0) return;
    j.sl = unit_cta(bnd, u0, G);
    j.sh = unit_cta(bnd, u1 - 1, G);
    const int lane = threadIdx.x & 31;
    const bool is_r = j.tg < P.nvt;
    const int tile = is_r ? j.tg : j.tg - P.nvt;
    const int lim = is_r ? D.n : min(N, D.bs);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int i = tile * TV_N + j.h * 128 + lane + 32 * k;
        j.rold[k] = 0.0;
        if (i < lim) j.rold[k] = is_r ? __ldcg(D.r + (size_t)j.c * D.ldr + i) : __ldcg(D.ra + (size_t)j.c * D.ldra + i);
    }
}

// The segments of job j from CTA q0 + u (u < 4) of its range: loads only.
template <int CT>
__device__ __forceinline__ void pair_load4(const Dev &D, const int *bnd, const PairJob &j, int q0, float (&v)[4][4])
{
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int q = q0 + u;
        const bool ok = q <= j.sh && bnd[q] < bnd[q + 1];   // CTAs without units have no slot
        const float *pp = D.vpart + ((size_t)(j.tg + q) * CT + j.c) * TV_N + j.h * 128 + lane;
#pragma unroll
        for (int k = 0; k < 4; ++k) v[u][k] = ok ? __ldcg(pp + 32 * k) : 0.0f;
    }
}

// Applies the update of job j from its segment sum acc: r, its bf16 split and
// the 128-row partial sum of r for a row tile, ra and its split for an ra
// tile.  The centring term is added to the FP32 segment sum (it is of the
// size of the other terms), leaving one FP64 conversion and one FP64
// addition per element.
template <int CT>
__device__ __forceinline__ void pair_finish(const Dev &D, const UnitPlan &P, const PairJob &j, const float (&acc)[4],
                                            const float *s_k0f, int N)
{
    const int lane = threadIdx.x & 31;
    const bool is_r = j.tg < P.nvt;
    const int tile = is_r ? j.tg : j.tg - P.nvt;
    const int lim = is_r ? D.n : min(N, D.bs);
    float part = 0.0f;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int i = tile * TV_N + j.h * 128 + lane + 32 * k;
        if (is_r) {
            const double rn = j.rold[k] + (double)(acc[k] + s_k0f[j.c]);
            if (i < lim) {
                const size_t o = (size_t)j.c * D.ldr + i;
                const float rf = (float)rn;
                D.r[o] = rn;
                split_store(D.rsp, o, (size_t)D.chains * D.ldr, rf);
                part += rf;
            }
        } else if (i < lim) {
            store_ra(D, j.c, i, j.rold[k] + (double)acc[k]);
        }
    }
    if (is_r) {
        const float ws = warp_sumf(part);
        if (lane == 0 && 2 * tile + j.h < D.nr_ctas) D.rsum[(size_t)j.c * D.nr_ctas + 2 * tile + j.h] = (double)ws;
    }
}

// Two jobs of one warp: the segments of each are added in segment order (the
// same order for any grouping), with the loads of both jobs issued together.
template <int CT>
__device__ __forceinline__ void pair_reduce2(const Dev &D, const UnitPlan &P, const int *bnd, const PairJob &ja,
                                             const PairJob &jb, const float *s_k0f, int N)
{
    float aa[4] = {0.0f, 0.0f, 0.0f, 0.0f}, ab[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    const int na = ja.sh - ja.sl + 1, nb_ = jb.sh - jb.sl + 1, nmax = max(na, nb_);
    for (int q0 = 0; q0 < nmax; q0 += 4) {
        float va[4][4], vb[4][4];
        pair_load4<CT>(D, bnd, ja, ja.sl + q0, va);
        pair_load4<CT>(D, bnd, jb, jb.sl + q0, vb);
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                aa[k] += va[u][k];
                ab[k] += vb[u][k];
            }
    }
    if (na > 0) pair_finish<CT>(D, P, ja, aa, s_k0f, N);
    if (nb_ > 0) pair_finish<CT>(D, P, jb, ab, s_k0f, N);
}

// Grid-wide barrier of the G CTAs of one launch on a monotonic counter (each
// launch adds G); bounded by %globaltimer (20 ms), false on time-out.
__device__ __forceinline__ bool update_grid_sync(unsigned long long *ctr, unsigned G)
{
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned long long old = atomicAdd(ctr, 1ull);
        const unsigned long long target = (old / G + 1) * G;
        const uint64_t t0 = tc::globaltimer_ns();
        int ok = 1;
        for (;;) {
            unsigned long long v;
            asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(ctr) : "memory");
            if (v >= target) break;
            if (tc::globaltimer_ns() - t0 > 20000000ull) {
                ok = 0;
                break;
            }
            __nanosleep(64);
        }
        __threadfence();
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

template <int CT>
__global__ void __launch_bounds__(TV_THREADS, 1)
    k_update_tc(const __grid_constant__ CUtensorMap tm_d, const __grid_constant__ CUtensorMap tm_u, Dev D, int b)
{
    using T = UpdTc<CT>;
    extern __shared__ __align__(1024) unsigned char smem_dyn[];
    __shared__ uint64_t s_fulla[TV_NS], s_fullb[TV_NS], s_conv[TV_NS], s_free[TV_NS];
    __shared__ uint64_t s_cfull[TV_NC], s_cfree[TV_NC];
    __shared__ uint64_t s_segdone[2], s_dfree[2];
    __shared__ uint32_t s_tmem;
    __shared__ int s_err;
    __shared__ UnitPlan s_plan;
    __shared__ double s_k0p[128], s_k0[CT];
    __shared__ float s_k0f[CT];
    __shared__ int s_bnd[TV_MAXG + 1];
    unsigned char *raw0 = smem_dyn + ((1024u - (tc::smem_u32(smem_dyn) & 1023u)) & 1023u);
    unsigned char *bop0 = raw0 + T::BOP0;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int ls = D.blk_ls[b];
    const int N = D.blk_ls[b + 1] - ls;
    const int nq = (N + TV_K - 1) / TV_K;
    const bool pd = D.blk_pd[b] != 0;
    const int cblk = D.qoff[b];   // the subset's first code block row (set up before the sweep)

    // the unit plan: the subset's shape only (set up before the sweep), so it overlaps the draws
    if (warp == 0) {
        // ra tile a (<= 64 of them, two per lane): its first stage (upper triangular: rows 256a ..
        // meet positions from 256a on, stages >= 4a) and an exclusive scan of its units
        UnitPlan &P = s_plan;
        const int nra = (N + TV_N - 1) / TV_N;
        int cnt[2], qs[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int a = 2 * lane + h;
            qs[h] = pd ? min(4 * a, nq) : 0;
            cnt[h] = a < nra ? 3 * (nq - qs[h]) : 0;
        }
        const int pair = cnt[0] + cnt[1];
        int incl = pair;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        const int excl = incl - pair;
        P.qs[2 * lane] = qs[0];
        P.pref[2 * lane] = excl;
        P.qs[2 * lane + 1] = qs[1];
        P.pref[2 * lane + 1] = excl + cnt[0];
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        if (lane == 0) {
            P.nq = nq;
            P.nvt = D.nvt;
            P.nra = nra;
            P.R = D.nvt * nq;
            P.pref[TV_MAXRA] = total;
            P.pref[nra] = total;
            P.W = P.R + total;
            s_err = 0;
        }
    }
    __syncthreads();
    const UnitPlan &P = s_plan;
    const int G = gridDim.x;
    for (int q = tid; q <= G; q += TV_THREADS) s_bnd[q] = split_bound(P, q, G);
    __syncthreads();
    tc::pdl_trigger();
    const int u_begin = s_bnd[blockIdx.x], u_end = s_bnd[blockIdx.x + 1];
    const int nu = u_end - u_begin;
    // this warp's first two reduction pairs (pr0 and pr0 + stride), prepared as soon as its role
    // ends (the epilogue warps, the last to finish, take none)
    const int npair = 2 * (P.nvt + P.nra) * CT;
    const int pr0 = blockIdx.x * TV_NPW + warp, stride = G * TV_NPW;
    PairJob ja, jb;
    auto prepare = [&]() {
        if (warp < TV_NPW) {
            tc::pdl_wait();   // r and ra of the previous update
            pair_prepare<CT>(D, P, s_bnd, G, pr0, npair, N, ja);
            pair_prepare<CT>(D, P, s_bnd, G, pr0 + stride, npair, N, jb);
        }
    };
    if (nu > 0) {
        if (tid == 0) {
            for (int i = 0; i < TV_NS; ++i) {
                tc::mbar_init(&s_fulla[i], 1);    // A tile landed
                tc::mbar_init(&s_fullb[i], 1);    // U tile of an ra unit landed
                tc::mbar_init(&s_conv[i], TV_CONV_WARPS);
                tc::mbar_init(&s_free[i], 1);     // the MMAs reading the slot are complete
            }
            for (int i = 0; i < 2; ++i) {
                tc::mbar_init(&s_segdone[i], 1);
                tc::mbar_init(&s_dfree[i], 1);
            }
            for (int i = 0; i < TV_NC; ++i) {
                tc::mbar_init(&s_cfull[i], 1);                // a row unit's packed codes landed
                tc::mbar_init(&s_cfree[i], TV_CONV_WARPS);    // every converter warp has read them
            }
            tc::mbar_fence_init();
        }
        if (warp == TV_WARP_MMA) tc::tmem_alloc(&s_tmem, 512);   // accumulators and codes operands
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
        const uint32_t tm = s_tmem;

        if (warp == TV_WARP_TMA) {
            // the warp decodes 32 units at a time into registers (lane l: unit s0 + l); lane 0 issues
            // their loads, taking each unit's coordinates by shuffle
            if (lane == 0) {
                tc::tma_prefetch_desc(&tm_d);
                tc::tma_prefetch_desc(&tm_u);
            }
            bool ok = true;
            int issued = 0;
            int kind = 0, ax = 0, cy = 0, cz = 0;
            auto decode = [&](int s0) {
                kind = ax = cy = cz = 0;
                if (s0 + lane < nu) {
                    const Unit x = decode_unit_bs(P, u_begin + s0 + lane);
                    kind = x.kind;
                    ax = x.q * TV_K;
                    cy = x.tile * TV_N;                 // ra: four boxes of 64 rows of U x 64 positions
                    cz = x.term * D.p + ls + ax;        //     from row 256 tile, term's plane
                }
            };
            auto load_u = [&](int sl, int y, int z) {
                unsigned char *bo = bop0 + (size_t)sl * T::BOP;   // MN atoms 8 KB apart
                tc::mbar_expect_tx(&s_fullb[sl], T::BOP);
#pragma unroll
                for (int h = 0; h < 4; ++h) tc::tma_load_2d(bo + h * 8192, &tm_u, y + 64 * h, z, &s_fullb[sl]);
            };
            // the U tiles of the first slots' ra units do not depend on the draws: they stream from
            // DRAM while the draws run
            decode(0);
            const int npre = min(nu, TV_NS);
            for (int i = 0; i < npre; ++i) {
                const int kd = __shfl_sync(0xffffffffu, kind, i);
                const int y = __shfl_sync(0xffffffffu, cy, i), z = __shfl_sync(0xffffffffu, cz, i);
                if (lane == 0 && kd == 1) load_u(i, y, z);
            }
            tc::pdl_wait();   // the delta tiles are the draws' split
            for (int s0 = 0; s0 < nu && ok; s0 += 32) {
                if (s0 > 0) decode(s0);
                const int m = min(32, nu - s0);
                for (int i = 0; i < m; ++i) {
                    const int s = s0 + i;
                    const int kd = __shfl_sync(0xffffffffu, kind, i), k0 = __shfl_sync(0xffffffffu, ax, i);
                    const int y = __shfl_sync(0xffffffffu, cy, i), z = __shfl_sync(0xffffffffu, cz, i);
                    if (lane == 0) {
                        const int sl = s % TV_NS;
                        // the slot's previous operands are consumed by the MMAs of unit s - TV_NS
                        ok = s < TV_NS || tc::mbar_wait(&s_free[sl], ((s / TV_NS) - 1) & 1);
                        if (!ok) {
                            s_err = 11;
                        } else {
                            tc::mbar_expect_tx(&s_fulla[sl], T::RAW_A);
                            tc::tma_load_2d(raw0 + (size_t)sl * T::ASTRIDE, &tm_d, k0, 0, &s_fulla[sl]);
                            if (kd == 1 && s >= TV_NS) load_u(sl, y, z);
                            issued = s + 1;
                        }
                    }
                    ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
                    if (!ok) break;
                }
            }
            // no copy may still be in flight into this CTA's shared memory when it exits: wait (bounded)
            // for the last loads issued into every slot (already complete unless a wait above gave up),
            // the U tiles issued before the dependency wait included
            if (lane == 0) {
                const int nrow = max(0, min(u_end, P.R) - u_begin);
                const int last = max(issued, npre);
                for (int s = max(0, last - TV_NS); s < last; ++s) {
                    if (s < issued && !tc::mbar_wait(&s_fulla[s % TV_NS], (s / TV_NS) & 1)) s_err = 21;
                    if (s >= nrow && !tc::mbar_wait(&s_fullb[s % TV_NS], ra_phase(s, nrow) & 1)) s_err = 21;
                }
            }
        } else if (warp == TV_WARP_MMA) {
            // nothing to issue before the draws' delta tiles: block in the dependency wait rather than
            // in mbarrier polls, which would take issue slots from the draw kernel on this SM
            tc::pdl_wait();
            // The loop keeps the tensor pipe fed only if it does little between MMA issues (the pipe
            // queues about one unit ahead): the whole warp runs it on warp-uniform values and one
            // elected lane issues, the descriptors are built once per slot and advanced by constants,
            // and a row unit is decoded from registers.  Descriptor start addresses are 16-byte units
            // in bits 0-13; every address here is below 256 KB, so the additions never carry out of
            // that field.
            const bool leader = tc::elect_one();
            const uint32_t id_row = tc::idesc_bf16(128, T::NB);               // A in tensor memory
            const uint32_t id_ra = tc::idesc_bf16(128, T::NB) | (1u << 15);   // A MN-major in smem
            const int nrow = max(0, min(u_end, P.R) - u_begin);
            const int pnq = P.nq, pR = P.R;
            const uint64_t bd0 = tc::desc_sw128(tc::smem_u32(raw0), 1024);          // delta split (B)
            const uint64_t ud0 = tc::desc_sw128_mn(tc::smem_u32(bop0), 8192, 1024);  // U tile (A)
            int hint = 0, seg = -1, pkind = -1, ptile = -1;
            int rtile = u_begin / pnq, rq = u_begin - rtile * pnq;   // the next row unit
            bool ok = true;
            for (int s = 0; s < nu && ok; ++s) {
                const int sl = s % TV_NS;
                int kind, tile;
                if (u_begin + s < pR) {
                    kind = 0;
                    tile = rtile;
                    if (++rq == pnq) {
                        rq = 0;
                        ++rtile;
                    }
                } else {
                    const Unit x = decode_unit(P, u_begin + s, hint);
                    kind = 1;
                    tile = x.tile;
                }
                const bool first = kind != pkind || tile != ptile;
                if (first) {
                    if (seg >= 0 && leader) tc::mma_commit(&s_segdone[seg & 1]);
                    ++seg;
                    pkind = kind;
                    ptile = tile;
                    // these accumulators were last used by segment seg - 2
                    if (seg >= 2) ok = tc::mbar_wait(&s_dfree[seg & 1], ((seg - 2) >> 1) & 1);
                    ok = __all_sync(0xffffffffu, ok);
                    if (!ok) s_err = 17;
                }
                if (ok) {
                    // A: widened codes of a row unit, or the U tile of an ra unit
                    ok = s < nrow ? tc::mbar_wait(&s_conv[sl], (s / TV_NS) & 1)
                                  : tc::mbar_wait(&s_fullb[sl], ra_phase(s, nrow) & 1);
                    ok = __all_sync(0xffffffffu, ok);
                    if (!ok) s_err = 12;
                }
                if (ok) {
                    ok = tc::mbar_wait(&s_fulla[sl], (s / TV_NS) & 1);
                    ok = __all_sync(0xffffffffu, ok);
                    if (!ok) s_err = 18;
                }
                if (!ok) break;
                tc::fence_after_sync();
                const uint64_t bd = bd0 + (uint64_t)((sl * T::ASTRIDE) >> 4);
                const uint32_t acc = tm + T::TM_ACC * 2 * (seg & 1);
                if (leader) {
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const uint32_t dt = acc + T::TM_ACC * h;
                        if (kind == 0) {
                            // codes of individuals 128 h ..: 8 columns (16 positions) per MMA
                            const uint32_t ta = tm + T::TM_OPS + 64 * sl + 32 * h;
#pragma unroll
                            for (int kk = 0; kk < TV_K / 16; ++kk)
                                tc::mma_bf16_ta(dt, ta + 8 * kk, bd + (uint64_t)(kk * (32 >> 4)), id_row,
                                                (first && kk == 0) ? 0u : 1u);
                        } else {
                            // rows 128 h .. of the U tile: two 64-row atoms (8 KB each), K groups 1 KB apart
                            const uint64_t ad = ud0 + (uint64_t)((sl * T::BOP + h * 16384) >> 4);
#pragma unroll
                            for (int kk = 0; kk < TV_K / 16; ++kk)
                                tc::mma_bf16(dt, ad + (uint64_t)(kk * (2048 >> 4)), bd + (uint64_t)(kk * (32 >> 4)),
                                             id_ra, (first && kk == 0) ? 0u : 1u);
                        }
                    }
                    tc::mma_commit(&s_free[sl]);
                }
                __syncwarp();
            }
            if (seg >= 0 && leader) tc::mma_commit(&s_segdone[seg & 1]);
        } else if (warp < TV_WARP_TMA) {
            // converters.  Row units come first in the unit order, so this CTA's row units are
            // u_begin .. min(u_end, R) - 1; the code loader streams their packed codes into a ring
            // of shared-memory slots, and each thread takes its 16 bytes from there.  Warp w writes
            // tensor-memory lanes 32 (w % 4) .. of half h = w / 4: the thread's individual is
            // 128 h + 32 (w % 4) + lane.
            const int nrow = max(0, min(u_end, P.R) - u_begin);
            const int ind = 128 * (warp >> 2) + 32 * (warp & 3) + lane;
            const unsigned char *codes0 = raw0 + T::CODE0 + ind * 16;
            const uint32_t tl = tm + ((uint32_t)(32 * (warp & 3)) << 16) + T::TM_OPS + 32 * (warp >> 2);
            for (int s = 0; s < nrow; ++s) {
                const int ob = s % TV_NS, cs = s % TV_NC;
                bool ok = tc::mbar_wait(&s_cfull[cs], (s / TV_NC) & 1);
                ok = __all_sync(0xffffffffu, ok);
                if (!ok) {
                    s_err = 13;
                    break;
                }
                const uint4 w = *reinterpret_cast<const uint4 *>(codes0 + (size_t)cs * T::CODE);
                // the next bulk copy (async proxy) overwrites what these generic loads read: order
                // them first, or the copy can land before the reads (results then vary run to run)
                tc::fence_async_smem();
                __syncwarp();
                if (lane == 0) tc::mbar_arrive(&s_cfree[cs]);   // the slot may be refilled
                // the first TV_NS units are widened while the draws still run; the next ones wait
                // for MMAs that need the draws' output, so block in the dependency wait first
                // (mbarrier polls would take issue slots from the draw kernel on this SM)
                if (s == TV_NS) tc::pdl_wait();
                // the operand was last read by the MMAs of unit s - TV_NS
                ok = s < TV_NS || tc::mbar_wait(&s_free[ob], ((s / TV_NS) - 1) & 1);
                ok = __all_sync(0xffffffffu, ok);   // the warp arrives as one
                if (!ok) {
                    s_err = 13;
                    break;
                }
                tc::fence_after_sync();
                uint32_t o[32];
                tc::codes64_to_bf16(w, o);   // positions of the stage, two per column
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
        } else if (warp == TV_WARP_CODES) {
            // code loader: one bulk copy (4 KB, individual-major packed codes) per row unit into the
            // ring, issued as slots free; the codes are not written by any kernel of the sweep, so
            // the first copies run while the draws still do.  Bulk copies stream at DRAM rates that
            // per-thread loads of the same bytes do not reach (each SM caps its outstanding loads).
            if (lane == 0) {
                const int nrow = max(0, min(u_end, P.R) - u_begin);
                const int pnq = P.nq, pnvt = P.nvt;
                int tile = u_begin / pnq, q = u_begin - tile * pnq;
                int issued = 0;
                for (int s = 0; s < nrow; ++s) {
                    const int cs = s % TV_NC;
                    if (s >= TV_NC && !tc::mbar_wait(&s_cfree[cs], ((s / TV_NC) - 1) & 1)) {
                        s_err = 14;
                        break;
                    }
                    const size_t blk = (size_t)(cblk + (q >> 1)) * pnvt + tile;
                    tc::mbar_expect_tx(&s_cfull[cs], T::CODE);
                    tc::bulk_load(raw0 + T::CODE0 + cs * T::CODE, D.gpu + blk * TC_PACKED_BLOCK + (q & 1) * T::CODE,
                                  T::CODE, &s_cfull[cs]);
                    issued = s + 1;
                    if (++q == pnq) {
                        q = 0;
                        ++tile;
                    }
                }
                // no copy may still be in flight into this CTA's shared memory when it exits
                for (int s = max(0, issued - TV_NC); s < issued; ++s)
                    if (!tc::mbar_wait(&s_cfull[s % TV_NC], (s / TV_NC) & 1)) s_err = 21;
            }
        } else {
            // epilogue: per finished segment, warp w reads tensor-memory lanes 32 (w % 4) .. (individuals
            // or rows of U 128 h + 32 (w % 4) + lane) of both halves h, and stores hi + mid + lo per chain
            // to the segment's slot of vpart
            tc::pdl_wait();   // the draws' centring sums; r of the previous update
            const int t = tid - 32 * TV_WARP_EPI;
            const int qd = warp & 3;
            update_k0<CT>(D, b, t, s_k0p, s_k0);
            int hint = 0, seg = -1, pkind = -1, ptile = -1;
            for (int s = 0; s <= nu; ++s) {
                Unit x;
                x.kind = -2;
                x.tile = -2;
                if (s < nu) x = decode_unit(P, u_begin + s, hint);
                if (s < nu && x.kind == pkind && x.tile == ptile) continue;
                if (seg >= 0) {
                    // segment seg (pkind, ptile) is complete once its MMAs are
                    const bool ok = tc::mbar_wait(&s_segdone[seg & 1], (seg >> 1) & 1);
                    if (!ok) s_err = 15;
                    tc::fence_after_sync();
                    const int tg = pkind == 0 ? ptile : P.nvt + ptile;
                    float *dst = D.vpart + (size_t)(tg + blockIdx.x) * CT * TV_N + 32 * qd + lane;
                    const uint32_t ta = tm + ((uint32_t)(32 * qd) << 16) + T::TM_ACC * 2 * (seg & 1);
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        float v[T::NB];
                        if (ok) {
#pragma unroll
                            for (int g = 0; g < T::NB / 8; ++g) {
                                float u8[8];
                                tc::tmem_ld8(ta + T::TM_ACC * h + 8 * g, u8);
#pragma unroll
                                for (int e = 0; e < 8; ++e) v[8 * g + e] = u8[e];
                            }
                            tc::tmem_wait_ld();
                        } else {
#pragma unroll
                            for (int e = 0; e < T::NB; ++e) v[e] = 0.0f;
                        }
#pragma unroll
                        for (int c = 0; c < CT; ++c) dst[c * TV_N + 128 * h] = (v[c] + v[CT + c]) + v[2 * CT + c];
                    }
                    tc::fence_before_sync();
                    __threadfence();   // the slot is read after the grid barrier
                    asm volatile("bar.sync 1, 128;" ::: "memory");
                    // the accumulators are free once every lane has read them
                    if (t == 0) tc::mbar_arrive(&s_dfree[seg & 1]);
                }
                if (s == nu) break;
                ++seg;
                pkind = x.kind;
                ptile = x.tile;
            }
        }
        prepare();
        __syncthreads();
        if (warp == TV_WARP_MMA) {
            tc::fence_after_sync();
            tc::tmem_dealloc(tm, 512);
        }
    } else {
        if (warp >= TV_WARP_EPI && warp < TV_WARP_EPI + 4) {
            tc::pdl_wait();
            update_k0<CT>(D, b, tid - 32 * TV_WARP_EPI, s_k0p, s_k0);   // the centring term
        }
        prepare();
    }
    __syncthreads();   // s_k0 is complete
    if (tid < CT) s_k0f[tid] = (float)s_k0[tid];   // read after the grid barrier's __syncthreads
    // every segment is in vpart once all CTAs are here; then the reductions, an equal share of the
    // (half tile, chain) pairs per CTA, one pair per warp at a time
    if (!update_grid_sync(D.ugrid, (unsigned)G)) s_err = 16;
    if (s_err) {
        if (tid == 0) flag_err(D, s_err);
        return;
    }
    if (warp >= TV_NPW) return;
    for (int pr = pr0; pr < npair; pr += 2 * stride) {
        if (pr != pr0) {
            pair_prepare<CT>(D, P, s_bnd, G, pr, npair, N, ja);
            pair_prepare<CT>(D, P, s_bnd, G, pr + stride, npair, N, jb);
        }
        pair_reduce2<CT>(D, P, s_bnd, ja, jb, s_k0f, N);
    }
}

}  // namespace soda
