// state.cuh — device-side layout of one SODA job.
//
// HBM layout (all arrays 256-byte aligned):
//   G      int8   [nloci][ldx]   genotype codes 0/1/2, one column per subset
//                                position k (SNP perm[k]), padded to ldx
//   X32    float  [nloci][ldx]   centred/scaled columns (FP32 mode only)
//   xv     double [nloci][4]     the three values (code - 2p)/sqrt(2p(1-p))
//                                of each column and 1/sqrt(2p(1-p)); all 0
//                                for monomorphic SNPs
//   U*     columns of the augmenting matrix: column k holds rows
//          0..ulen[k]-1 at uoff[k]; columns of a subset are spaced
//          round_up(N,8) apart (16-byte aligned, zero below ulen), FP64 in the
//          FP64 mode, FP32 otherwise
//   r      double [C][ldr]       residual yadj (master copy, FP64)
//   r32    float  [C][ldr]       FP32 copy read by the FP32/FP8 dot products
//   ra     double [C][ldra]      augmented residual yAadj (ra32: FP32 copy)
//   g, vara_s double [C][nloci], cls int32 [C][nloci] (by SNP id)
//   tensor-core sweep only: rsp / rasp, the bf16 hi/mid/lo split of r32 /
//   ra32 (written with them), and usp, the same split of U scaled by sd_k
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>
#include "../../include/sodagpu.h"

namespace soda {

constexpr int MAXDIST = SODAGPU_MAXDIST;
constexpr int MAXGRP = SODAGPU_MAXGRP;
constexpr int MAXGM = MAXDIST * MAXGRP;

// Per-chain scalars and small tables (device memory, one per chain).
struct ChainScal {
    double mu[2];              // mu of the previous / current iteration (by rep parity)
    double vara, vare, scale_va;
    double gp[MAXDIST], vare_gp[MAXDIST];
    double mu_store, vare_store, vara_store, included_store;
    int32_t included, counter, keep, err;
    double p[MAXGM];           // (ngroup, nmix) column-major
    double log_p[MAXGM];
    double varindist[MAXGM];
    double snpstore[MAXGM], pstore[MAXGM], varstore[MAXGM];
    int32_t snpindist[MAXGM];
};

// Control block written by the host before a run and by the kernels.
struct RunCtl {
    int32_t rep;               // iteration counter (1-based once running)
    int32_t trace_iter;        // thinned iterations seen in this run
    int32_t trace_cap;         // rows available in trace
    int32_t trace_count;       // rows written
    int32_t err;               // sticky device error flag
    sodagpu_trace_row *trace;  // device trace buffer
};

// Everything the kernels read, passed by value.
struct Dev {
    // sizes
    int n, p, bs, nb, bt, method, nmix, ngroup, chains, precision;
    int ldx;                   // column stride of G / X32 (elements)
    int ldr;                   // chain stride of r / r32
    int nskipped, naind;
    int nr_ctas;               // row tiles (ROW_TILE rows) of the residual kernels
    int recal;
    int regular;               // 1: regular_bayes (every SNP single-site, no augmented data)
    int burnin, thin;
    uint64_t seed;
    double pizero, scale_ve, df_va, df_ve;
    double mix[MAXDIST], alpha[MAXDIST];
    // data (shared by chains)
    const int8_t *G;
    const float *X32;
    const double *xv;          // [p][4]: x for codes 0,1,2 and 1/sd (0 if monomorphic)
    const float *xv32;         // the same table in FP32 (FP32/FP8 inner loops)
    const double *y;
    const int64_t *uoff;
    const int32_t *ulen;
    const double *U64;
    const float *U32;
    const __nv_bfloat16 *Uhi, *Ulo;
    const double *xxd;         // d per subset
    const double *xpx;         // x'x by SNP (skipped SNPs)
    const int32_t *perm;       // position -> SNP (0-based)
    const int32_t *pos_of;     // SNP -> position
    const uint8_t *skip;       // by position
    const int32_t *iskipped;   // skipped SNP ids
    const int32_t *grp;        // by SNP, 1-based
    const int32_t *blk_ls;     // [nb+1] first position of each subset
    const int32_t *blk_pd;     // [nb] 1 when the subset's factor is the unpivoted one
    // chain state
    double *r;
    float *r32;
    double *ra;                // [C][ldra]
    float *ra32;               // [C][ldra] FP32 copy read by the FP32/FP8 dot products
    int ldra;                  // chain stride of ra / ra32 (bs rounded up to 8)
    double *g;
    int32_t *cls;
    double *vara_s;
    double *gstore, *vara_sstore;
    uint32_t *indist;          // [C][p][nmix] kept-sample class counts
    ChainScal *scal;
    RunCtl *ctl;
    // scratch
    double *delta;             // [C][bs]
    float *delta32;            // [bs][C] FP32 copy for the FP32/FP8 update (chain-contiguous)
    uint8_t *nzflag;           // [bs]
    double *rpart;             // [C][nr_ctas] row-CTA partial sums (mu, rsum, r^2)
    double *rsum;              // [C][nr_ctas] partial sums of r for the FP8 centring
    double *statpart;          // [C][NSTAT][ngroup*nmix] sum g^2
    int32_t *cntpart;          // [C][NSTAT][ngroup*nmix] counts
    double *recal_part;        // [C][RECAL_SPLIT][ldr]
    double *rpx, *rpu;         // [RHS_KSPLIT_MAX][C][bs] rhs partial sums (genotype / augmented part)
    // tensor-core sweep (FP8 mode, 4/8/16 chains)
    int tc;                    // 1 when the tensor-core kernels run
    int ldd;                   // row stride of dsplit (bs rounded up to 128)
    uint16_t *dsplit;          // [round_up(3C,16)][ldd] bf16 hi/mid/lo of delta/sd per chain
    double *k0part;            // [draw CTAs][C] per-CTA sums of x0_j delta_j
    float *vpart;              // [tiles + update CTAs][C][256] update partial sums, one slot per segment
    unsigned long long *ugrid; // grid-barrier counter of the update (each launch adds its CTA count)
    const uint8_t *gpk;        // 2-bit packed code blocks, position-major (the rhs; see TC_PACKED_BLOCK)
    const uint8_t *gpu;        // the same codes individual-major (the residual update)
    int nvt;                   // row tiles of 256 individuals of the update
    const int32_t *qoff;       // [nb+1] first 128-position code block of each subset (tiled codes)
    const int32_t *rtab;       // [nb][tstride] first rhs CTA of each 128-SNP tile, then the total
    int tstride;
    uint16_t *rsp;             // [round_up(3C,16)][ldr] bf16 hi/mid/lo of r32 (rows c, C+c, 2C+c), or null
    uint16_t *rasp;            // [round_up(3C,16)][ldra] the same split of ra32, or null
    const uint16_t *usp;       // [3][nloci][ldu] bf16 hi/mid/lo of U column k times sd_k (1 if sd_k = 0)
    int ldu;                   // row stride of usp (bs rounded up to 8)
    // conditional right-hand sides only: when set, k_draw writes the rhs of
    // (chain c, subset SNP jl) to rhs_out[c * bs + jl] (exactly the value its
    // draw would consume) and draws nothing
    double *rhs_out;
    // injected-draw tape (sodagpu_set_tape): tape_reps iterations of
    // tape_sites records of SODAGPU_TAPE_W uniforms; SNP records start at
    // site tape_snp0 (3 + ngroup + the configured blocksize)
    const double *tape;
    int tape_reps, tape_sites, tape_snp0;
};

// Block coordinates of a CTA in its own job's grid.  A plain launch takes the
// hardware's; a batched launch (the grids of several jobs laid end to end
// along x, JobGrid) maps blockIdx.x to (job, x, y, z) first.
struct VB {
    int x, y, z, nx, ny, nz;
};

__device__ __forceinline__ VB vb_native()
{
    return VB{(int)blockIdx.x, (int)blockIdx.y, (int)blockIdx.z, (int)gridDim.x, (int)gridDim.y, (int)gridDim.z};
}

// One launch over several jobs: job j owns CTAs off[j] .. off[j+1]-1 of a
// 1-D grid, its own grid being gx[j] x gy[j] x (the rest), and the kernel's
// integer arguments for it are arg[j][0..2].  Passed by value (grid constant).
constexpr int MAXJOBS = 64;
struct JobGrid {
    const Dev *dev;            // [njobs] the jobs' descriptors in device memory
    int njobs;
    int off[MAXJOBS + 1];
    int gx[MAXJOBS], gy[MAXJOBS];
    int arg[MAXJOBS][3];
};

// The job of this CTA (the last j with off[j] <= blockIdx.x, so jobs without
// CTAs are passed over) and its block coordinates in that job's grid.
__device__ __forceinline__ int jg_locate(const JobGrid &G, VB &vb)
{
    const int bid = (int)blockIdx.x;
    int lo = 0, hi = G.njobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (G.off[mid] <= bid) lo = mid;
        else hi = mid - 1;
    }
    const int l = bid - G.off[lo], gx = G.gx[lo], gy = G.gy[lo];
    vb.nx = gx;
    vb.ny = gy;
    vb.nz = (G.off[lo + 1] - G.off[lo]) / (gx * gy);
    vb.x = l % gx;
    vb.y = (l / gx) % gy;
    vb.z = l / (gx * gy);
    return lo;
}

constexpr int RHS_KSPLIT_MAX = 16;

constexpr int NSTAT = 64;          // CTAs of the per-iteration SNP statistics
constexpr int ROW_THREADS = 128;   // threads of the row kernels
constexpr int ROWS_PER_THREAD = 1;
constexpr int ROW_TILE = ROW_THREADS * ROWS_PER_THREAD;   // rows per row tile (= the update's tile)
constexpr int RECAL_SPLIT = 32;    // column splits of the residual recalibration

}  // namespace soda
