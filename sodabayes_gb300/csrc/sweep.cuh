// sweep.cuh — host-side entry points of the sweep kernels (sweep.cu).
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include "state.cuh"

namespace soda {

int sweep_chain_count_supported(int chains);
cudaError_t sweep_prepare(int bs);
// Tensor-core sweep: whether it applies and the rows of its delta split
// (3 * chains rounded up to 16).
int sweep_tc_supported(int precision, int chains, int bs);
int sweep_tc_rows(int chains);
// The residual update's row tiles (256 individuals) and the floats of its
// partial-sum slots (one per tile segment: tiles + CTAs slots of C x 256).
int sweep_tc_update_tiles(int n);
size_t sweep_tc_vpart_floats(int n, int bs, int chains, int sm_count);
// Work tables of the tensor-core rhs (host side), per subset b of blk_sizes:
// rtab[b*stride + m] = first rhs CTA of 128-SNP tile m, rtab[b*stride + tiles]
// = rhs CTAs; tiles get K splits in proportion to their pipeline stages
// (genotype stages plus the U stages of the upper-triangular factor).
int sweep_tc_table_stride(int bs);
void sweep_tc_tables(const int *blk_sizes, int nb, int bs, int ldx, int sm_count, int32_t *rtab);
// Set-up of the tensor-core rhs, once per job after the Z build: writes the
// bf16 hi/mid/lo split of every U column k times sd_k into D.usp ([3][p][ldu];
// sd_k = 1 where 1/sd_k is 0) and zeroes the codes of those columns in G (their
// x values are all 0, so no product changes).
cudaError_t sweep_tc_prepare(int8_t *G, const Dev &D, cudaStream_t st);
// Packed copy of the codes for the tensor-core kernels: per subset b, code
// blocks qoff[b] .. qoff[b+1]-1 of 128 positions (the last one zero-padded);
// block (q2, t) covers 128 positions x 256 individuals (individuals past n
// hold 0) as TC_PACKED_BLOCK bytes at Gt + (q2 * D.nvt + t) * TC_PACKED_BLOCK:
// [4 groups of 64 individuals][128 positions][16 bytes], 2 bits per code, and
// in each 32-bit word of a 16-byte entry the code of individual 16 w + 4 b + j
// of the group (w the word) sits at bits 8 j + 2 b, so that
// (word >> 2b) & 0x03030303 holds four consecutive codes as bytes.  An update
// unit (64 positions of one block) is 4 KB, one word per converter thread; an
// rhs stage (128 positions x 128 individuals) is 8 bytes per converter thread.
// sweep_tc_code_blocks fills qoff[0..nb] and returns the block rows;
// sweep_tc_tile_codes writes all nblocks = rows * D.nvt blocks from G (after
// sweep_tc_prepare, on the same stream).
// The update reads a second copy, individual-major: block (q2, t) holds
// [2 stages of 64 positions][256 individuals][16 bytes], and in word w of an
// individual's 16 bytes the code of position 16 w + 4 b + j of the stage sits
// at bits 8 j + 2 b (one 16-byte load per individual and update unit).
// sweep_tc_tile_codes writes both copies (Gu may be null).
constexpr int TC_PACKED_BLOCK = 4 * 128 * 16;   // bytes of one packed code block
int sweep_tc_code_blocks(const int *blk_sizes, int nb, int32_t *qoff);
cudaError_t sweep_tc_tile_codes(const int8_t *G, const Dev &D, uint8_t *Gt, uint8_t *Gu, long long nblocks,
                                int sm_count, cudaStream_t st);
// Optional per-launch event recording (eager profiling, never inside a graph):
// before/after every launch an event pair is recorded and its kernel class
// stored.  Classes: 0 rhs, 1 residual update, 2 mu, 3 everything else, 4 draws.
enum { PROF_RHS = 0, PROF_UPDATE = 1, PROF_MU = 2, PROF_OTHER = 3, PROF_DRAW = 4, PROF_NCLASS = 5 };
struct ProfHook {
    cudaEvent_t *ev;   // 2 * cap events
    int *cls;          // cap classes
    int n, cap;
};

// TMA descriptors of the tensor-core sweep: the bf16 splits of delta, r and
// ra in 64 x rows boxes; the bf16 U terms in 64 x 128 and 64 x 64 (U rows x
// SNPs) boxes (all 128-byte swizzle); and the host copy of the rhs work table.
struct TcMaps {
    CUtensorMap d;                      // delta split
    CUtensorMap rsp, usp, usp64, rasp;  // residual split, U-term split (two box heights), ra split
    const int32_t *h_rtab;              // host copy of D.rtab
};

// Enqueues one Gibbs iteration of every chain on `st` (graph-capturable when
// prof == nullptr).  `maps` is required when D.tc is set.
cudaError_t sweep_enqueue_iteration(const Dev &D, const int *blk_sizes, int sm_count, const TcMaps *maps,
                                    cudaStream_t st, ProfHook *prof = nullptr);
cudaError_t sweep_enqueue_init(const Dev &D, double vara0, double scale_va0, int sm_count, cudaStream_t st);
// One subset b (nsnp SNPs) of the current iteration, eagerly: rhs, draws and
// residual update, or with rhs_only the rhs and the draw kernel in its
// rhs-only mode (D.rhs_out set by the caller), which changes no state.
cudaError_t sweep_enqueue_subset(const Dev &D, int b, int nsnp, int sm_count, const TcMaps *maps, cudaStream_t st,
                                 bool rhs_only);
// Loads chain c's state from device arrays: g, cls, vs by SNP id (nloci), r
// (nind), ra (naind used), pi ((ngroup, nmix) column-major, or null to keep
// the chain's current pi), and its scalars.
cudaError_t sweep_set_state(const Dev &D, int c, const double *g, const int32_t *cls, const double *vs,
                            const double *r, const double *ra, const double *pi, double mu, double vare, double vara,
                            int included, cudaStream_t st);
cudaError_t sweep_enqueue_recal(const Dev &D, double unused, cudaStream_t st);

// Several jobs per launch (CUDA-core kernels; the jobs share precision and
// chain count).  hdev / ddev: the jobs' descriptors on the host and in device
// memory; blk_sizes[j]: job j's subset sizes; ksplit[j]: the K splits of its
// rhs tiles.  Step t of an iteration runs subset t of every job that has one.
struct BatchPlan {
    int njobs;
    const Dev *hdev;
    const Dev *ddev;
    const int *const *blk_sizes;
    const int *ksplit;
};
cudaError_t sweep_multi_prepare(int precision, int chains, int max_bs);
// K splits of the rhs of a subset of N SNPs so that its CTAs number about
// cta_share (at least one per 128-SNP tile, at most the stages of ldx).
int sweep_multi_rhs_split(int precision, int N, int chains, int ldx, int cta_share);
cudaError_t sweep_enqueue_iteration_multi(const BatchPlan &P, int sm_count, cudaStream_t st);

}  // namespace soda
