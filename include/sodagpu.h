/*
 * sodagpu.h — C ABI of the GB300 SODA Gibbs sampler (libsodagpu.so).
 *
 * The reference program (SODABayes, Fortran 2018 + OpenMP) has no plugin or FFI
 * layer: its modules talk through the `globals` module (globals.f90:1-53) and the
 * SODA sampler is the argument-less `subroutine soda_bayes` (models.f90:9), run
 * from `run_program_sodaBayes` (SODABayes.f90:112-165) after `setup_soda`
 * (SODABayes.f90:139).  Each entry point below replaces one step of that call
 * chain; the comment on each names the reference code it stands in for.
 *
 * Conventions
 *   - Plain C types only; every array is allocated and owned by the caller.
 *   - Matrices are column-major (Fortran order).  Index arguments that the
 *     reference keeps 1-based (permvec, SNP groups, mixture classes) stay
 *     1-based at this boundary.
 *   - Every function returns 0 on success and a negative SODAGPU_E* code on
 *     failure; nothing calls exit/abort/stop.  sodagpu_errstr() names the code,
 *     sodagpu_last_error() gives the message of the last failure on the calling
 *     thread.
 *   - One context per host thread.  A context owns one CUDA stream on the
 *     device that was current when it was created.
 */
#ifndef SODAGPU_H
#define SODAGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SODAGPU_ABI_VERSION 1

#define SODAGPU_MAXDIST 20 /* globals.f90:8  maxdist: mixture classes */
#define SODAGPU_MAXGRP 100 /* globals.f90:35 maxgrp:  SNP groups       */

/* globals.f90:22  BayesA=1 ... BayesRc=6 */
enum sodagpu_method {
    SODAGPU_BAYES_A = 1,
    SODAGPU_BAYES_B = 2,
    SODAGPU_BAYES_C = 3,
    SODAGPU_BAYES_CPI = 4,
    SODAGPU_BAYES_R = 5,
    SODAGPU_BAYES_RC = 6
};

/* Arithmetic of the per-iteration sweep.  The Z build is FP64 in every mode.
 *   FP64: genotypes as centred/scaled FP64 columns, U in FP64 — the parity mode.
 *   FP32: genotypes as centred/scaled FP32 columns, U in FP32 — the plain path.
 *   FP8 : genotypes as exact 8-bit 0/1/2 codes with the centring applied as an
 *         FP32 rank-1 correction, U as BF16 hi+lo pairs.                      */
enum sodagpu_precision { SODAGPU_FP64 = 0, SODAGPU_FP32 = 1, SODAGPU_FP8 = 2 };

/* Sweep kernels.  AUTO puts the genotype products of the FP8 mode with 4, 8
   or 16 chains on the tensor cores (tcgen05); CUDA_CORES keeps every product
   on the FP32/FP64 cores.  Results agree to rounding. */
enum sodagpu_kernels { SODAGPU_KERNELS_AUTO = 0, SODAGPU_KERNELS_CUDA_CORES = 1 };

/* Sampler.  SODA is soda_bayes (models.f90:9-605): subsets drawn in parallel
   against the augmented data.  REGULAR is regular_bayes (models.f90:607-962,
   the -SODAOff path, SODABayes.f90:137): single-site Gibbs over the SNPs in
   order, no augmenting matrix; it needs no sodagpu_build_z factorisation (the
   call only lays out the genotypes) and always runs in FP64. */
enum sodagpu_sampler { SODAGPU_SAMPLER_SODA = 0, SODAGPU_SAMPLER_REGULAR = 1 };

/* Genotype input layouts for sodagpu_load_genotypes(). */
enum sodagpu_geno_layout {
    /* int8 codes 0/1/2, column-major nind x nloci (one SNP per column);
     * missing calls already mapped to 1 as load_geno does (utilities.f90:446-451). */
    SODAGPU_GENO_CODES = 0,
    /* PLINK .bed SNP-major payload without the 3-byte magic header:
     * nloci records of ceil(nind/4) bytes, decoded like utilities.f90:438-454. */
    SODAGPU_GENO_BED = 1,
    /* OR-ed flag: the pointer is device memory on the context's device. */
    SODAGPU_GENO_DEVICE_PTR = 0x100
};

/* Error codes (negative). */
enum sodagpu_status {
    SODAGPU_OK = 0,
    SODAGPU_E_ARG = -1,        /* invalid argument or configuration          */
    SODAGPU_E_STATE = -2,      /* call out of order (e.g. run before build_z) */
    SODAGPU_E_NOMEM = -3,      /* device or host allocation failed           */
    SODAGPU_E_CUDA = -4,       /* CUDA runtime / launch error                */
    SODAGPU_E_NOTPSD = -5,     /* d*I - X'X not positive semidefinite (soda.f90:496-499) */
    SODAGPU_E_TIMEOUT = -6,    /* a bounded device wait gave up              */
    SODAGPU_E_NODEVICE = -7,   /* no CUDA device / unsupported architecture  */
    SODAGPU_E_UNSUPPORTED = -8 /* option combination not implemented         */
};

/* Job configuration: the values the reference reads from its option table
 * (useroptions.f90:22-55) after parse() (useroptions.f90:554-572), plus the
 * GPU-only knobs at the end.  Floating options are passed as the reference holds
 * them: cast_float() reads them as default REAL (utilities.f90:168-171), so a
 * drop-in host rounds them through float before widening to double.          */
typedef struct sodagpu_config {
    int32_t nind;       /* individuals (get_size, utilities.f90:256-267)        */
    int32_t nloci;      /* SNPs        (get_size, utilities.f90:268-275)        */
    int32_t method;     /* enum sodagpu_method (parse_method)                   */
    int32_t nmix;       /* mixture classes (parse_nmix, useroptions.f90:375-400) */
    int32_t ngroup;     /* SNP groups, 1 unless BayesRc (get_size 276-301)      */
    int32_t blocksize;  /* SODA subset size  (setup_soda, soda.f90:407-417)     */
    int32_t nblocks;    /* number of subsets                                    */
    int32_t blockt;     /* subsets of full size; the rest hold blocksize-1 SNPs */
    int32_t numit;      /* -numit  */
    int32_t burnin;     /* -burnin */
    int32_t thin;       /* -thin   */
    int32_t precision;  /* enum sodagpu_precision                                */
    int32_t chains;     /* independent chains sharing X and Z (>=1)             */
    int32_t recal_every;/* residual recalibration period, 1000 in models.f90:571 */
    int64_t seed;       /* -seed (set_random_seed, utilities.f90:504-517)       */
    double pizero;      /* -pi: fraction of zero-effect SNPs (BayesB/C)         */
    double scale_va, scale_ve, df_va, df_ve; /* priors (parse_priors)            */
    double mix[SODAGPU_MAXDIST];   /* -mix   (class variances as share of Va)   */
    double alpha[SODAGPU_MAXDIST]; /* -alpha (Dirichlet prior)                  */
    double vara0;       /* value of the module variable `vara` on entry: the
                           df_va<=0 branch adds to it (models.f90:99-102)       */
    int32_t kernels;    /* enum sodagpu_kernels: which sweep kernels run        */
    int32_t sampler;    /* enum sodagpu_sampler (-SODAOn / -SODAOff)            */
    int32_t reserved[6];
} sodagpu_config;

/* One thinned iteration of the .hyp trace (models.f90:549-569). */
typedef struct sodagpu_trace_row {
    int32_t chain;
    int32_t rep;        /* iteration, 1-based                                  */
    int32_t included;   /* ModelSize                                           */
    int32_t pad;
    double mu, vare, vara;
    int32_t snpindist[SODAGPU_MAXDIST]; /* counts for group 1 (ngroup==1 rows)   */
    double varindist[SODAGPU_MAXDIST];  /* sum g^2 per class, group 1           */
} sodagpu_trace_row;

typedef void (*sodagpu_trace_cb)(void *user, const sodagpu_trace_row *row);

typedef struct sodagpu_ctx sodagpu_ctx;

/* ---- setup ------------------------------------------------------------- */

/* Block sizing of setup_soda (soda.f90:407-421).  blocksize_opt/nblocks_opt are
 * the -blocksize/-nblocks options (0 = unset), nthreads the resolved thread
 * count.  Returns 1 when SODA has to be switched off (blocksize<=1, soda.f90:418),
 * 0 otherwise. */
int sodagpu_block_layout(int32_t nloci, int32_t nthreads, int32_t blocksize_opt,
                         int32_t nblocks_opt, int32_t *blocksize, int32_t *nblocks,
                         int32_t *blockt);

/* Allocates the device state for one job (allocate_data, utilities.f90:558-586;
 * the SODA arrays of setup_soda, soda.f90:422-428). */
int sodagpu_create(const sodagpu_config *cfg, sodagpu_ctx **out);

/* Genotypes (load_geno, utilities.f90:402-460) and their centring and scaling
 * (xscale, utilities.f90:519-534).  Allele frequencies are computed on the
 * device; sodagpu_get_freq returns them for the .frq writer. */
int sodagpu_load_genotypes(sodagpu_ctx *ctx, const void *geno, int32_t layout);
int sodagpu_get_freq(sodagpu_ctx *ctx, double *freq /* nloci */);

/* Phenotypes (load_pheno, utilities.f90:329-400): nind doubles. */
int sodagpu_load_pheno(sodagpu_ctx *ctx, const double *y);

/* BayesRc SNP groups (load_snp_grp, utilities.f90:304-327): nloci 1-based ids. */
int sodagpu_set_groups(sodagpu_ctx *ctx, const int32_t *group);

/* Augmenting matrix (get_aug_matrix, soda.f90:445-518): per subset the exact
 * genotype Gram (xxproduct, soda.f90:520-556), d = lambda_max + 0.001
 * (power_method, soda.f90:378-401, 484-486) and the upper Cholesky factor of
 * d*I - X'X (choleskyPD, soda.f90:8-47) with the pivoted fallback
 * (choleskyPSD, soda.f90:49-124).  permvec is the 1-based SNP order of
 * setup_soda (soda.f90:429-435); NULL means identity.  *nskipped receives the
 * number of SNPs dropped by the pivoted fallback (may be NULL). */
int sodagpu_build_z(sodagpu_ctx *ctx, const int32_t *permvec, int32_t *nskipped);

/* Test hook: add `delta` to every d_b before the factorisation, which makes
 * d*I - X'X indefinite for negative delta and exercises the pivoted path. */
int sodagpu_set_d_offset(sodagpu_ctx *ctx, double delta);

/* Injected draws (the reference's per-thread xoroshiro128+ streams,
 * parallelrng.f90:100-149, or any other source of uniforms in [0,1)).
 * Without a tape every draw is a counter-based Philox draw keyed by (seed,
 * chain, iteration, site); with one, each draw site of chain 0 takes the
 * uniforms its distribution transforms consume (rand_normal two per normal,
 * parallelrng.f90:264-277; rand_gamma's rejection loop as many as it needs,
 * 294-333) from its record instead.
 * Layout: draws[(rep * sites + site) * SODAGPU_TAPE_W + k], k-th uniform of
 * `site` in iteration rep (rep 0 = chain initialisation, models.f90:56-128),
 * sites = 3 + ngroup + blocksize + nloci:
 *   0 mu (models.f90:130-132), 1 sigma2_g (505-513), 2 sigma2_e (515-516; at
 *   rep 0 the initial draw, models.f90:118), 3 + i pi of group i (517-522),
 *   3 + ngroup + i yAadj(i) (523-525; at rep 0, models.f90:124-127),
 *   3 + ngroup + blocksize + j SNP j by id (its draw in its subset,
 *   models.f90:146-162, 211-256, 350-413, or its single-site draw).
 * n doubles cover n / (sites * SODAGPU_TAPE_W) iterations from rep 0; a draw
 * past them, or one needing more than SODAGPU_TAPE_W uniforms, makes
 * sodagpu_run / sodagpu_init_chains fail with SODAGPU_E_ARG.  One chain only;
 * call before sodagpu_init_chains (draws == NULL, n == 0 removes the tape). */
#define SODAGPU_TAPE_W 32
int sodagpu_set_tape(sodagpu_ctx *ctx, const double *draws, size_t n);

/* Chain initialisation (models.f90:56-128) for all chains. */
int sodagpu_init_chains(sodagpu_ctx *ctx);

/* Runs `iters` Gibbs iterations of every chain (models.f90:129-574), continuing
 * the iteration count across calls.  When cb is non-NULL it is called after the
 * iterations finish, once per chain and thinned iteration, in order. */
int sodagpu_run(sodagpu_ctx *ctx, int32_t iters, sodagpu_trace_cb cb, void *user);

/* Posterior means (models.f90:575-594) of one chain, any pointer may be NULL:
 *   gstore[nloci], indiststore[nloci*nmix] (column-major), vara_sstore[nloci],
 *   scalars[4] = {mu_store, vare_store, vara_store, included_store},
 *   snpstore/pstore/varstore [ngroup*nmix] (column-major). */
int sodagpu_get_results(sodagpu_ctx *ctx, int32_t chain, double *gstore,
                        double *indiststore, double *vara_sstore, double *scalars,
                        double *snpstore, double *pstore, double *varstore);

/* Current sampler state of one chain (any pointer may be NULL):
 *   g[nloci], cls[nloci] (1-based class = snptracker(:,2)), vara_s[nloci],
 *   yadj[nind], yaadj[blocksize], scalars[4] = {mu, vare, vara, included}. */
int sodagpu_get_state(sodagpu_ctx *ctx, int32_t chain, double *g, int32_t *cls,
                      double *vara_s, double *yadj, double *yaadj, double *scalars);

/* Loads the sampler state of one chain, the inverse of sodagpu_get_state:
 * g, cls (1-based classes), vara_s by SNP id (nloci each), yadj (nind),
 * yaadj (blocksize; entries past naind are ignored), scalars[4] = {mu, vare,
 * vara, included} and pi, the mixture proportions p(ngroup, nmix) column-major
 * (globals.f90: p; NULL keeps the chain's current ones).  The module state
 * soda_bayes carries from one iteration to the next (models.f90:129-574) is
 * exactly this plus the iteration counter (sodagpu_set_iteration), so a chain
 * restarted from it draws what it would have drawn; the posterior
 * accumulators are not touched. */
int sodagpu_set_state(sodagpu_ctx *ctx, int32_t chain, const double *g, const int32_t *cls,
                      const double *vara_s, const double *yadj, const double *yaadj,
                      const double *scalars, const double *pi);

/* Sets the iteration counter `rep` (models.f90:129): the draws of
 * sodagpu_run_subset / sodagpu_subset_rhs belong to iteration rep, and the
 * next sodagpu_run iteration is rep + 1. */
int sodagpu_set_iteration(sodagpu_ctx *ctx, int32_t rep);

/* The conditional right-hand side of every SNP of subset b (0-based) on the
 * current state, for every chain: rhs[chain * N_b + j] = x_j'yadj + u_j'yAadj
 * (models.f90:154, 219, 358), before the d*g term, exactly as the draw of
 * this context's precision consumes it (rounded to FP32 in the FP32/FP8
 * modes); 0 for SNPs the pivoted fallback skipped.  Draws nothing and changes
 * no state. */
int sodagpu_subset_rhs(sodagpu_ctx *ctx, int32_t b, double *rhs);

/* One subset b (0-based) of the current iteration for every chain: the
 * per-SNP draws (models.f90:349-414) and the residual update (415-430),
 * without the mu and hyper-parameter draws around the subset loop. */
int sodagpu_run_subset(sodagpu_ctx *ctx, int32_t b);

/* The augmenting matrix as the reference stores it: XA(blocksize, nloci)
 * column-major (globals.f90:52) and xxd(nblocks) (any pointer may be NULL),
 * plus skip flags by position (1 = skipped). */
int sodagpu_get_z(sodagpu_ctx *ctx, double *xa, double *xxd, int32_t *skip);

/* Genomic values pred = mu + X*effects (compute_dgv, utilities.f90:616-622)
 * with the context's own genotypes and centring. */
int sodagpu_compute_dgv(sodagpu_ctx *ctx, double mu, const double *effects,
                        double *pred /* nind */);

/* Prediction with external frequencies (setup_prediction + xscale's
 * prediction branch, utilities.f90:540-553, 616-622): genotypes as in
 * sodagpu_load_genotypes, freq[nloci] from a .frq file. Needs no context. */
int sodagpu_predict(int32_t nind, int32_t nloci, const void *geno, int32_t layout,
                    const double *freq, double mu, const double *effects,
                    double *pred);

/* Seconds spent in the last sodagpu_build_z and sodagpu_run calls (host
 * clock), and the device time of the last run's iterations in milliseconds
 * (CUDA events on the context's stream around the iteration launches). */
int sodagpu_timings(sodagpu_ctx *ctx, double *build_z_s, double *run_s, double *run_device_ms);

/* Measurement hook: runs `iters` iterations (advancing the chains exactly like
 * sodagpu_run) with kernels launched one by one and a CUDA-event pair around
 * each launch.  ms[c] receives the summed device time and launches[c] the
 * launch count of kernel class c: 0 rhs products, 1 residual update,
 * 2 mu draw, 3 hyper-parameter draws and accumulators, 4 per-SNP draws. */
#define SODAGPU_NPROF 5
int sodagpu_profile_kernels(sodagpu_ctx *ctx, int32_t iters, double *ms, int32_t *launches);

/* Genomic values pred = mu + X*effects for callers that cannot let this
 * library allocate device memory (a host that owns the GPU through its own
 * memory pool, or a latency-bound loop that must avoid cudaMalloc/cudaFree).
 * No counterpart in the reference: it computes what compute_dgv does
 * (utilities.f90:616-622) but allocates nothing, device or host.
 *   codes   device, int8 0/1/2, column-major nind x nloci with leading dim ldg
 *   freq    device, nloci allele frequencies (xscale centring, 0 if monomorphic)
 *   effects device, nloci; pred device, nind (written)
 *   stream  a cudaStream_t, or NULL for the default stream; the call only
 *           enqueues work there, results are ready when the stream is.
 * Scratch is one fixed array of SODAGPU_NOALLOC_SCRATCH doubles (16 MiB) in
 * the library's device memory, held by every GPU that loads the library until
 * the process exits; nind may not exceed SODAGPU_NOALLOC_SCRATCH
 * (SODAGPU_E_ARG otherwise).  The first call on each device looks up the
 * array's device address (cudaGetSymbolAddress, with that device current), so
 * make that first call before any stream capture.  All calls share the array
 * and leave their partial sums in it: calls that overlap on the GPU race and
 * must be serialised by the caller.  cudaDeviceReset invalidates the address
 * looked up for that device: after a reset, do not call this again on that
 * device in the same process.  The columns are summed in min(32,
 * SODAGPU_NOALLOC_SCRATCH / nind, nloci) splits: up to nind = 65,536 the same
 * order as sodagpu_predict, above it the last bits may differ.  Codes outside
 * 0..2 count as 1 (a missing call, utilities.f90:446-449), where
 * sodagpu_predict returns SODAGPU_E_ARG.  Errors are reported by the return
 * code only (sodagpu_last_error is not updated); a launch error the caller
 * left pending is neither reported nor cleared. */
#define SODAGPU_NOALLOC_SCRATCH (2 * 1024 * 1024)
int sodagpu_compute_dgv_noalloc(int32_t nind, int32_t nloci, const int8_t *codes, int32_t ldg,
                                const double *freq, double mu, const double *effects, double *pred,
                                void *stream);

/* ---- many analyses in one launch per kernel ------------------------------
 * A batch runs the iterations of several independent jobs (analyses of their
 * own n, p, phenotype, priors and seed) together: every kernel of an
 * iteration is launched once over all jobs (each CTA finds its job in a
 * table), and step t of the subset loop runs subset t of every job that has
 * one.  No counterpart in the reference, which runs one analysis per .par job
 * (SODABayes.f90:35-97) with soda_bayes (models.f90:9-605) each time; each
 * job in a batch takes exactly the draws, and gives exactly the results, it
 * would give on its own.  The jobs are ordinary contexts, created, loaded,
 * Z-built and initialised one by one (sodagpu_init_chains), on one device,
 * with one precision and chain count, and run on the CUDA-core kernels
 * (SODAGPU_KERNELS_CUDA_CORES, or fewer than 4 chains); after a batch run
 * their state and results are read with the per-job calls.  A job may belong
 * to one batch at a time and must not be run on its own meanwhile.  The batch
 * copies each job's device layout when it is created: destroy the batch
 * before any of its jobs, and create it again after re-initialising a job
 * (sodagpu_init_chains). */
#define SODAGPU_MAXJOBS 64
/* flags of sodagpu_batch_create.  By default each job's rhs products get K
 * splits in proportion to its share of the batch's genotype bytes, so that
 * the batch's CTAs make about one wave; the partial sums of a split are then
 * added in another grouping than in a job run on its own (results equal to
 * rounding).  SOLO_SPLITS keeps every job's own splits: bit-identical
 * results to the job run on its own. */
#define SODAGPU_BATCH_SOLO_SPLITS 1
typedef struct sodagpu_batch sodagpu_batch;
int sodagpu_batch_create(sodagpu_batch **out, sodagpu_ctx *const *jobs, int32_t njobs, int32_t flags);
/* `iters` iterations of every job (no trace rows are gathered). */
int sodagpu_batch_run(sodagpu_batch *batch, int32_t iters);
/* Device time of the last sodagpu_batch_run, in milliseconds (CUDA events on
 * the batch's stream around the iteration launches), and the subset steps of
 * one iteration (the largest subset count of the jobs). */
int sodagpu_batch_timings(sodagpu_batch *batch, double *run_device_ms, int32_t *steps);
void sodagpu_batch_destroy(sodagpu_batch *batch);

/* Subset sizes for a batch of njobs analyses (n[j] individuals, p[j] SNPs)
 * that will run `iters` iterations.  All jobs share one step count S (the
 * subset loop runs in lock step), job j gets blocksize[j] = ceil(p[j] / S),
 * capped at max_blocksize, and S is the candidate of least modelled time:
 *   iters * (S * step_us + sum_j stream_bytes_j(S) / bw)  +  sum_j zbuild_j(S)
 * where stream_bytes_j reads job j's codes and its factor's triangle twice
 * per iteration (rhs and update; e_x and e_u bytes per element), and
 * zbuild_j = p[j] * (n[j] * N_j / gram_ops + N_j^2 / (3 * fp64_flops)) is the
 * Gram and Cholesky of its subsets (N_j = blocksize[j]).  model[] holds
 * {step_us, bw (bytes/s), e_x, e_u, gram_ops (int8 multiply-adds/s),
 * fp64_flops}; NULL takes values measured on GB300 for the FP8 mode
 * {30, 2.6e12, 1, 4, 5e13, 6e11} (the bandwidth as measured on a batch of
 * 32 BayesB analyses, n up to 20,000 and p up to 200,000: 90 GB per
 * iteration in 35.6 ms).  *steps receives S and *model_s the modelled
 * seconds of the choice. */
int sodagpu_autotune_batch(int32_t njobs, const int32_t *n, const int32_t *p, int32_t iters,
                           int32_t max_blocksize, const double *model, int32_t *blocksize, int32_t *steps,
                           double *model_s);

void sodagpu_destroy(sodagpu_ctx *ctx);
const char *sodagpu_errstr(int code);
const char *sodagpu_last_error(void);
int sodagpu_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif /* SODAGPU_H */
