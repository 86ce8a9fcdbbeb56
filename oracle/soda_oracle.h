/*
 * soda_oracle.h — CPU FP64 restatement of SODABayes' SODA path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker the GPU library is compared
 * against; only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline /
 * reference arm load it.  Nothing in the product links or calls it.
 *
 * Parity status: the Gibbs sweep and the Z build are restated from the Fortran
 * sources; the reference ships no tests and cannot be compiled here (no Fortran
 * compiler), so only the prediction path (bed decode, xscale, compute_dgv) is
 * pinned against the reference's own shipped outputs.  The sweep itself is
 * "parity unpinned" against reference runs; its checks are algebraic
 * identities and distribution tests.
 */
#ifndef SODA_ORACLE_H
#define SODA_ORACLE_H

#include <stdint.h>
#include "../include/sodagpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* RNG modes: COUNTER draws from Philox4x32-10 keyed like the GPU sampler, so
 * both codes consume identical uniforms (injected-draw parity).  REFERENCE
 * replays the reference's per-thread xoroshiro128+ streams
 * (parallelrng.f90:54-149) with OpenMP static chunking for `ref_threads`. */
enum { ORACLE_RNG_COUNTER = 0, ORACLE_RNG_REFERENCE = 1 };

typedef struct oracle_ctx oracle_ctx;

int oracle_create(const sodagpu_config *cfg, int32_t rng_mode, int32_t ref_threads,
                  oracle_ctx **out);
void oracle_destroy(oracle_ctx *o);
int oracle_set_omp_threads(int32_t nthreads);

int oracle_decode_bed(int32_t nind, int32_t nloci, const uint8_t *payload, int8_t *codes);
int oracle_load_genotypes(oracle_ctx *o, const int8_t *codes);
int oracle_get_freq(oracle_ctx *o, double *freq);
int oracle_get_x(oracle_ctx *o, double *x);
int oracle_load_pheno(oracle_ctx *o, const double *y);
int oracle_set_groups(oracle_ctx *o, const int32_t *group);
int oracle_permutate(oracle_ctx *o, int32_t *permvec);
int oracle_gram(oracle_ctx *o, const int32_t *cols, int32_t ncols, double *A);
int oracle_build_z(oracle_ctx *o, const int32_t *permvec, int64_t power_maxit,
                   double d_offset, int32_t *nskipped);
int oracle_get_z(oracle_ctx *o, double *xa, double *xxd, int32_t *skip);
int oracle_set_z(oracle_ctx *o, const double *xa, const double *xxd);
/* Injected-draw tape (layout of sodagpu_set_tape, one chain): with record = 1
 * every draw site of iterations 0 .. reps-1 (0 = chain initialisation) writes
 * the uniforms it draws into `tape` (reps x sites x SODAGPU_TAPE_W doubles,
 * owned by the caller); with record = 0 the sites read them from it instead. */
int oracle_set_tape(oracle_ctx *o, double *tape, int32_t reps, int32_t record);
int oracle_tape_sites(const oracle_ctx *o);
int oracle_init_chains(oracle_ctx *o);
int oracle_run(oracle_ctx *o, int32_t iters, sodagpu_trace_cb cb, void *user);
int oracle_run_blocks(oracle_ctx *o, int32_t first_block, int32_t nblocks_run,
                      int32_t reps);
int oracle_set_sparse_state(oracle_ctx *o, double incl, int64_t seed);
int oracle_get_state(oracle_ctx *o, int32_t chain, double *g, int32_t *cls,
                     double *vara_s, double *yadj, double *yaadj, double *scalars);
int oracle_get_results(oracle_ctx *o, int32_t chain, double *gstore,
                       double *indiststore, double *vara_sstore, double *scalars,
                       double *snpstore, double *pstore, double *varstore);
int oracle_compute_dgv(oracle_ctx *o, double mu, const double *effects, double *pred);
int oracle_predict(int32_t nind, int32_t nloci, const int8_t *codes,
                   const double *freq, double mu, const double *effects, double *pred);

/* Building blocks exported for unit tests. */
void oracle_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
int oracle_ref_uniforms(int64_t seed, int32_t stream, int32_t count, double *out);
int oracle_counter_uniforms(int64_t seed, int32_t chain, int32_t iter, int32_t slot,
                            int32_t purpose, int32_t count, double *out);
int oracle_sample(int32_t dist, int32_t mode, int64_t seed, int32_t count,
                  double a, double b, double *out);
int oracle_cholesky_pd(int32_t n, const double *A, double *U);
int oracle_cholesky_psd(int32_t n, double *A, int32_t *piv, int32_t *rank);
int oracle_power_method(int32_t n, const double *A, const double *start,
                        int64_t maxit, double *lambda, int64_t *iters);

#ifdef __cplusplus
}
#endif
#endif
