/*
 * soda_oracle.c — CPU FP64 restatement of SODABayes' SODA path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker): loaded by tests/, smoke() and the CPU
 * baseline legs of bench.py, never by the product.  Build with
 * -ffp-contract=off so that x86-64 and aarch64 hosts round identically.
 *
 * What is restated, with the reference lines each part follows:
 *   RNG            parallelrng.f90:54-149 (xoroshiro128+, 2^64 jumps),
 *                  242-249 (u64 -> [0,1)), 264-277 (normal), 294-333 (gamma),
 *                  348-362 (scaled inverse chi-square), 445-455 (Dirichlet)
 *   seed           utilities.f90:504-517
 *   genotypes      utilities.f90:438-454 (bed decode), 519-534 (xscale),
 *                  462-502 (2-bit words)
 *   SODA setup     soda.f90:403-443 (blocks), utilities.f90:588-607 (permutate),
 *                  soda.f90:445-518 (get_aug_matrix), 520-556 (xxproduct),
 *                  378-401 (power_method), 8-47 (choleskyPD), 49-124 and
 *                  128-376 (choleskyPSD with its LAPACK helpers)
 *   sampler        models.f90:56-128 (initialisation), 129-574 (iterations),
 *                  575-594 (posterior means); the regular (-SODAOff) sampler
 *                  models.f90:607-962 as the same iteration with every SNP
 *                  drawn single-site in order (draw_skipped restates 717-859)
 *                  and no augmented data
 *   products       utilities.f90:609-622 (compute_residuals, compute_dgv)
 *
 * Parity status: unpinned for the sweep and the Z build (the reference has no
 * tests and no Fortran compiler is available to run it); the prediction path
 * is pinned by the reference's shipped example outputs.
 */
#include "soda_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Counter-RNG purposes; the GPU sampler uses the same numbering. */
enum {
    P_SNP = 1, P_MU = 2, P_VARA = 3, P_VARE = 4, P_PI = 5, P_RA = 6,
    P_SKIP = 7, P_PERM = 8, P_POWER = 9
};

#define REF_PI ((double)3.141592653589793238462f) /* parallelrng.f90:20, a REAL literal */
#define POWER_TOL ((double)1.0e-14f)               /* soda.f90:385, a REAL literal      */
#define D_SHIFT ((double)0.001f)                    /* soda.f90:485, a REAL literal      */

/* ------------------------------------------------------------------------ */
/* xoroshiro128+ streams (parallelrng.f90:100-149)                          */
/* ------------------------------------------------------------------------ */
typedef struct { uint64_t s1, s2; } xo_state;

static inline uint64_t rotl64(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

static inline uint64_t xo_next(xo_state *s)
{
    uint64_t s1 = s->s1, s2 = s->s2;
    uint64_t r = s1 + s2;
    s2 ^= s1;
    s->s1 = rotl64(s1, 55) ^ s2 ^ (s2 << 14);
    s->s2 = rotl64(s2, 36);
    return r;
}

static void xo_jump(xo_state *s)
{
    static const uint64_t jmp[2] = {0xbeac0467eba5facbULL, 0xd86b048b86aa9922ULL};
    uint64_t a = 0, b = 0;
    for (int i = 0; i < 2; ++i)
        for (int bit = 0; bit < 64; ++bit) {
            if (jmp[i] & (1ULL << bit)) { a ^= s->s1; b ^= s->s2; }
            xo_next(s);
        }
    s->s1 = a;
    s->s2 = b;
}

/* rng_zigset: stream k is the seed jumped k+1 times (parallelrng.f90:54-78);
 * the seed pair is (|seed|, |seed|+1) (utilities.f90:508-510). */
static void xo_streams(int64_t seed, int n, xo_state *out)
{
    xo_state s;
    uint64_t a = (uint64_t)(seed < 0 ? -seed : seed);
    s.s1 = a;
    s.s2 = a + 1;
    for (int k = 0; k < n; ++k) { xo_jump(&s); out[k] = s; }
}

/* rng_int64_to_real64 (parallelrng.f90:242-249) */
static inline double u64_to_unit(uint64_t x)
{
    uint64_t bits = 0x3FF0000000000000ULL | (x >> 12);
    double d;
    memcpy(&d, &bits, sizeof d);
    return d - 1.0;
}

/* ------------------------------------------------------------------------ */
/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11)                        */
/* ------------------------------------------------------------------------ */
void oracle_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        if (r) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        c1 = (uint32_t)p1;
        c3 = (uint32_t)p0;
        c0 = n0;
        c2 = n2;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

typedef struct {
    uint32_t key[2], ctr[4], out[4];
    int have;
} ctr_rng;

static void ctr_init(ctr_rng *s, int64_t seed, int chain, int iter, int slot, int purpose)
{
    uint64_t a = (uint64_t)(seed < 0 ? -seed : seed);
    s->key[0] = (uint32_t)a;
    s->key[1] = (uint32_t)(a >> 32);
    s->ctr[0] = (uint32_t)iter;
    s->ctr[1] = (uint32_t)slot;
    s->ctr[2] = (uint32_t)purpose;
    s->ctr[3] = (uint32_t)chain << 20;
    s->have = 0;
}

static inline uint64_t ctr_next(ctr_rng *s)
{
    if (s->have == 0) {
        oracle_philox4x32_10(s->ctr, s->key, s->out);
        s->ctr[3]++;
        s->have = 2;
        return ((uint64_t)s->out[1] << 32) | s->out[0];
    }
    s->have = 0;
    return ((uint64_t)s->out[3] << 32) | s->out[2];
}

/* ------------------------------------------------------------------------ */
/* Uniform source and the reference distributions                          */
/* ------------------------------------------------------------------------ */
typedef struct {
    int mode;        /* ORACLE_RNG_* */
    xo_state *xo;    /* reference: the stream in use */
    ctr_rng c;       /* counter */
    /* injected-draw tape: the record of the current draw site (tmode 1:
     * the uniforms drawn are written to it, 2: they are read from it instead
     * of the RNG), tn uniforms used so far */
    double *tp;
    int tn, tmode;
} rng_t;

static inline double rng_u(rng_t *r)
{
    if (r->tmode == 2) {
        double u = r->tn < SODAGPU_TAPE_W ? r->tp[r->tn] : 0.5;
        r->tn++;
        return u;
    }
    double u = r->mode == ORACLE_RNG_REFERENCE ? u64_to_unit(xo_next(r->xo))
                                               : u64_to_unit(ctr_next(&r->c));
    if (r->tmode == 1) {
        if (r->tn < SODAGPU_TAPE_W) r->tp[r->tn] = u;
        r->tn++;
    }
    return u;
}

/* rand_normal (parallelrng.f90:264-277): Box-Muller, sine branch, REAL pi */
static double rnorm(double mean, double sd, rng_t *r)
{
    if (sd <= 0.0) return mean;
    double u1 = rng_u(r), u2 = rng_u(r);
    double rr = pow(-2.0 * log(u1), 0.5);
    double th = 2.0 * REF_PI * u2;
    return mean + sd * rr * sin(th);
}

/* rand_gamma (parallelrng.f90:294-333): Marsaglia & Tsang (2000) */
static double rgamma_(double shape, double scale, rng_t *r)
{
    if (shape >= 1.0) {
        double d = shape - 1.0 / 3.0;
        double c = 1.0 / pow(9.0 * d, 0.5);
        for (;;) {
            double x = rnorm(0.0, 1.0, r);
            double v = 1.0 + c * x;
            while (v <= 0.0) {
                x = rnorm(0.0, 1.0, r);
                v = 1.0 + c * x;
            }
            v = v * v * v;
            double u = rng_u(r);
            double xsq = x * x;
            if ((u < 1.0 - 0.0331 * xsq * xsq) ||
                (log(u) < 0.5 * xsq + d * (1.0 - v + log(v))))
                return scale * d * v;
        }
    }
    double g = rgamma_(shape + 1.0, 1.0, r);
    double w = rng_u(r);
    return scale * g * pow(w, 1.0 / shape);
}

/* rand_scaled_inverse_chi_square -> rand_inverse_gamma (parallelrng.f90:348-362) */
static double rscinvchi2(double dof, double scale, rng_t *r)
{
    double shape = 0.5 * dof, sc = 0.5 * dof * scale;
    return 1.0 / rgamma_(shape, 1.0 / sc, r);
}

/* rand_dirichlet (parallelrng.f90:445-455) */
static void rdirichlet(int n, const double *irx, double *x, rng_t *r)
{
    double sx = 0.0;
    for (int i = 0; i < n; ++i) x[i] = rgamma_(irx[i], 1.0, r);
    for (int i = 0; i < n; ++i) sx += x[i];
    for (int i = 0; i < n; ++i) x[i] = x[i] / sx;
}

/* ------------------------------------------------------------------------ */
/* Context                                                                  */
/* ------------------------------------------------------------------------ */
typedef struct {
    double *g, *r, *ra, *vara_s, *gtemp;
    int32_t *cls;                       /* snptracker(:,2), 1-based           */
    int32_t *gflag;
    double mu, vara, vare, scale_va;
    double *p, *log_p;                  /* (ngroup, nmix) column-major        */
    double gp[SODAGPU_MAXDIST], vare_gp[SODAGPU_MAXDIST];
    int32_t *snpindist;                 /* (ngroup, nmix)                      */
    double *varindist;                  /* (ngroup, nmix)                      */
    int32_t included;
    int32_t counter, rep;
    double mu_store, vare_store, vara_store, included_store;
    double *gstore, *indiststore, *vara_sstore, *snpstore, *pstore, *varstore;
} chain_t;

struct oracle_ctx {
    sodagpu_config cfg;
    int n, p, method, nmix, ngroup, nchain, bs, nb, bt;
    int regular;                        /* regular_bayes (models.f90:607-962) */
    int rng_mode, ref_threads;
    xo_state *xo;                       /* reference streams                   */
    int8_t *G;                          /* n*p codes                           */
    double *X;                          /* n*p centred/scaled                  */
    double *freq, *y, *xpx;
    int32_t *grp;                       /* snptracker(:,1), 1-based            */
    int32_t *perm;                      /* 0-based SNP at each position        */
    double *XA, *xxd;
    uint8_t *skip;                      /* by position                         */
    int32_t *iskipped;                  /* 0-based SNP ids                     */
    int nskipped, naind, naless;
    int have_geno, have_pheno, have_z, have_chain;
    chain_t *ch;
    /* injected-draw tape (oracle_set_tape) */
    double *tape;
    int tape_reps, tape_sites, tape_play, tape_over;
};

#define IDX2(i, j, ld) ((size_t)(i) + (size_t)(j) * (size_t)(ld))

static void block_bounds(const oracle_ctx *o, int b /*0-based*/, int *ls, int *le)
{
    /* models.f90:136-142 / soda.f90:463-469 (1-based ls, le) */
    int blocki = b + 1;
    if (blocki <= o->bt) {
        *ls = (blocki - 1) * o->bs + 1;
        *le = *ls + o->bs - 1;
        if (*le > o->p) *le = o->p;
    } else {
        *ls = o->bs * o->bt + (blocki - o->bt - 1) * (o->bs - 1) + 1;
        *le = *ls + o->bs - 2;
        if (*le > o->p) *le = o->p;
    }
}

int oracle_set_omp_threads(int32_t nthreads)
{
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
    return omp_get_max_threads();
#else
    (void)nthreads;
    return 1;
#endif
}

int oracle_create(const sodagpu_config *cfg, int32_t rng_mode, int32_t ref_threads,
                  oracle_ctx **out)
{
    if (!cfg || !out) return SODAGPU_E_ARG;
    const int regular = cfg->sampler == SODAGPU_SAMPLER_REGULAR;
    if (cfg->nind < 2 || cfg->nloci < 1 || cfg->method < 1 || cfg->method > 6 ||
        cfg->nmix < 1 || cfg->nmix > SODAGPU_MAXDIST || cfg->ngroup < 1 ||
        cfg->ngroup > SODAGPU_MAXGRP || (!regular && (cfg->blocksize < 2 || cfg->nblocks < 1)) ||
        cfg->thin < 1 || cfg->chains < 1 || (cfg->sampler != SODAGPU_SAMPLER_SODA && !regular))
        return SODAGPU_E_ARG;
    if (rng_mode == ORACLE_RNG_REFERENCE && cfg->chains != 1) return SODAGPU_E_ARG;
    oracle_ctx *o = (oracle_ctx *)calloc(1, sizeof *o);
    if (!o) return SODAGPU_E_NOMEM;
    o->cfg = *cfg;
    o->n = cfg->nind;
    o->p = cfg->nloci;
    o->method = cfg->method;
    o->nmix = cfg->nmix;
    o->ngroup = cfg->ngroup;
    o->nchain = cfg->chains;
    /* the regular sampler has no subsets and no augmented data */
    o->regular = regular;
    o->bs = regular ? 1 : cfg->blocksize;
    o->nb = regular ? 0 : cfg->nblocks;
    o->bt = regular ? 0 : cfg->blockt;
    o->rng_mode = rng_mode;
    o->ref_threads = ref_threads < 1 ? 1 : ref_threads;
    size_t np = (size_t)o->n * o->p;
    o->G = (int8_t *)calloc(np, 1);
    o->X = (double *)calloc(np, sizeof(double));
    o->freq = (double *)calloc(o->p, sizeof(double));
    o->y = (double *)calloc(o->n, sizeof(double));
    o->xpx = (double *)calloc(o->p, sizeof(double));
    o->grp = (int32_t *)malloc(sizeof(int32_t) * o->p);
    o->perm = (int32_t *)malloc(sizeof(int32_t) * o->p);
    o->XA = (double *)calloc((size_t)o->bs * o->p, sizeof(double));
    o->xxd = (double *)calloc(o->nb > 0 ? o->nb : 1, sizeof(double));
    o->skip = (uint8_t *)calloc(o->p, 1);
    o->iskipped = (int32_t *)calloc(o->p, sizeof(int32_t));
    o->xo = (xo_state *)calloc(o->ref_threads, sizeof(xo_state));
    if (!o->G || !o->X || !o->freq || !o->y || !o->xpx || !o->grp || !o->perm || !o->XA ||
        !o->xxd || !o->skip || !o->iskipped || !o->xo) {
        oracle_destroy(o);
        return SODAGPU_E_NOMEM;
    }
    for (int j = 0; j < o->p; ++j) { o->grp[j] = 1; o->perm[j] = j; }
    xo_streams(cfg->seed, o->ref_threads, o->xo);
    *out = o;
    return 0;
}

static void free_chain(chain_t *c)
{
    free(c->g); free(c->r); free(c->ra); free(c->vara_s); free(c->gtemp);
    free(c->cls); free(c->gflag); free(c->p); free(c->log_p); free(c->snpindist);
    free(c->varindist); free(c->gstore); free(c->indiststore); free(c->vara_sstore);
    free(c->snpstore); free(c->pstore); free(c->varstore);
}

void oracle_destroy(oracle_ctx *o)
{
    if (!o) return;
    if (o->ch) {
        for (int c = 0; c < o->nchain; ++c) free_chain(&o->ch[c]);
        free(o->ch);
    }
    free(o->G); free(o->X); free(o->freq); free(o->y); free(o->xpx); free(o->grp);
    free(o->perm); free(o->XA); free(o->xxd); free(o->skip); free(o->iskipped); free(o->xo);
    free(o);
}

/* ------------------------------------------------------------------------ */
/* Genotypes                                                                */
/* ------------------------------------------------------------------------ */

/* load_geno's per-SNP decode (utilities.f90:438-454): b - ((b>>1)&0x55) maps
 * the 2-bit codes 00,01,10,11 to 0,1,1,2 (missing 01 becomes 1). */
int oracle_decode_bed(int32_t nind, int32_t nloci, const uint8_t *payload, int8_t *codes)
{
    if (nind < 1 || nloci < 1 || !payload || !codes) return SODAGPU_E_ARG;
    size_t nbytes = ((size_t)nind + 3) / 4;
    for (int j = 0; j < nloci; ++j) {
        const uint8_t *rec = payload + (size_t)j * nbytes;
        for (int i = 0; i < nind; ++i) {
            uint8_t b = rec[i >> 2];
            b = (uint8_t)(b - ((b >> 1) & 0x55));
            codes[IDX2(i, j, nind)] = (int8_t)((b >> (2 * (i & 3))) & 3);
        }
    }
    return 0;
}

/* xscale, MCMC branch (utilities.f90:525-534) */
int oracle_load_genotypes(oracle_ctx *o, const int8_t *codes)
{
    if (!o || !codes) return SODAGPU_E_ARG;
    const int n = o->n;
    const double eps = 2.220446049250313e-16;
    memcpy(o->G, codes, (size_t)n * o->p);
    for (int j = 0; j < o->p; ++j) {
        const int8_t *gc = codes + (size_t)j * n;
        double *xc = o->X + (size_t)j * n;
        double s = 0.0;
        for (int i = 0; i < n; ++i) s = s + (double)gc[i];
        double p = s / (2.0 * n);
        if (p < eps || (1.0 - p) < eps) {
            for (int i = 0; i < n; ++i) xc[i] = 0.0;
        } else {
            double sd = sqrt(2.0 * p * (1.0 - p));
            for (int i = 0; i < n; ++i) xc[i] = ((double)gc[i] - 2.0 * p) / sd;
        }
        o->freq[j] = p;
    }
    o->have_geno = 1;
    return 0;
}

int oracle_get_freq(oracle_ctx *o, double *freq)
{
    if (!o || !freq || !o->have_geno) return SODAGPU_E_ARG;
    memcpy(freq, o->freq, sizeof(double) * o->p);
    return 0;
}

int oracle_get_x(oracle_ctx *o, double *x)
{
    if (!o || !x || !o->have_geno) return SODAGPU_E_ARG;
    memcpy(x, o->X, sizeof(double) * (size_t)o->n * o->p);
    return 0;
}

int oracle_load_pheno(oracle_ctx *o, const double *y)
{
    if (!o || !y) return SODAGPU_E_ARG;
    memcpy(o->y, y, sizeof(double) * o->n);
    o->have_pheno = 1;
    return 0;
}

int oracle_set_groups(oracle_ctx *o, const int32_t *group)
{
    if (!o || !group) return SODAGPU_E_ARG;
    for (int j = 0; j < o->p; ++j) {
        if (group[j] < 1 || group[j] > o->ngroup) return SODAGPU_E_ARG;
        o->grp[j] = group[j];
    }
    return 0;
}

/* permutate (utilities.f90:588-607), uniforms from stream 0. */
int oracle_permutate(oracle_ctx *o, int32_t *permvec)
{
    if (!o || !permvec) return SODAGPU_E_ARG;
    const int n = o->p, s = o->bs;
    double *u = (double *)malloc(sizeof(double) * s);
    if (!u) return SODAGPU_E_NOMEM;
    for (int i = 0; i < n; ++i) permvec[i] = i + 1;
    int chunk = 0;
    for (int i = 1; i <= n; i += s, ++chunk) {
        int m = n - i + 1 < s ? n - i + 1 : s;
        rng_t r;
        r.mode = o->rng_mode;
        r.tmode = 0;
        r.xo = &o->xo[0];
        ctr_init(&r.c, o->cfg.seed, 0, 0, chunk, P_PERM);
        for (int k = 0; k < s; ++k) u[k] = rng_u(&r);
        for (int j = 1; j <= m; ++j) {
            int ipj = i + j - 1;
            int k = (int)(u[j - 1] * (double)(n - ipj + 1)) + ipj;
            int t = permvec[ipj - 1];
            permvec[ipj - 1] = permvec[k - 1];
            permvec[k - 1] = t;
        }
    }
    free(u);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Z build                                                                  */
/* ------------------------------------------------------------------------ */

/* 2-bit genotype words as load_geno_bits leaves them (utilities.f90:462-502):
 * 32 individuals per 64-bit word, individual i in bits 2(i%32)..2(i%32)+1. */
static uint64_t *make_genbits(const oracle_ctx *o, int *nbatch_out)
{
    int nbatch = (o->n + 31) / 32;
    uint64_t *gb = (uint64_t *)calloc((size_t)nbatch * o->p, sizeof(uint64_t));
    if (!gb) return NULL;
    for (int j = 0; j < o->p; ++j)
        for (int i = 0; i < o->n; ++i)
            gb[IDX2(i / 32, j, nbatch)] |= (uint64_t)(uint8_t)o->G[IDX2(i, j, o->n)]
                                           << (2 * (i % 32));
    *nbatch_out = nbatch;
    return gb;
}

static inline int popc64(uint64_t x) { return __builtin_popcountll(x); }

/* xxproduct (soda.f90:520-556) */
static double xxproduct(const oracle_ctx *o, const uint64_t *gb, int nbatch, int jj, int kk)
{
    const double ep = 2.220446049250313e-16;
    const uint64_t FIVE = 0x5555555555555555ULL;
    double pj = o->freq[jj], pk = o->freq[kk];
    double qj = 1.0 - pj, qk = 1.0 - pk;
    if (pj <= ep || qj <= ep || pk <= ep || qk <= ep) return 0.0;
    pj = pj * 2.0;
    pk = pk * 2.0;
    int nc = 0, nd = 0, ng = 0;
    const uint64_t *a_ = gb + (size_t)jj * nbatch, *b_ = gb + (size_t)kk * nbatch;
    for (int i = 0; i < nbatch; ++i) {
        uint64_t a = a_[i], b = b_[i];
        uint64_t c = a & b;
        uint64_t d = (c >> 1) & FIVE;
        uint64_t e = ((a >> 1) & b) & FIVE;
        uint64_t f = (a & (b >> 1)) & FIVE;
        uint64_t g = e | f;
        nc += popc64(c);
        nd += popc64(d);
        ng += popc64(g);
    }
    double res = (double)(nd * 3 + ng * 2 + nc);
    res = (res - (double)o->n * pj * pk) / sqrt(pj * pk * qj * qk);
    return res;
}

int oracle_gram(oracle_ctx *o, const int32_t *cols, int32_t ncols, double *A)
{
    if (!o || !cols || ncols < 1 || !A || !o->have_geno) return SODAGPU_E_ARG;
    int nbatch;
    uint64_t *gb = make_genbits(o, &nbatch);
    if (!gb) return SODAGPU_E_NOMEM;
    for (int j = 0; j < ncols; ++j)
        for (int k = 0; k <= j; ++k) {
            double v = xxproduct(o, gb, nbatch, cols[j], cols[k]);
            A[IDX2(k, j, ncols)] = v;
            A[IDX2(j, k, ncols)] = v;
        }
    free(gb);
    return 0;
}

/* power_method (soda.f90:378-401) */
int oracle_power_method(int32_t n, const double *A, const double *start, int64_t maxit,
                        double *lambda, int64_t *iters)
{
    double *y = (double *)malloc(sizeof(double) * n), *v = (double *)malloc(sizeof(double) * n);
    if (!y || !v) { free(y); free(v); return SODAGPU_E_NOMEM; }
    memcpy(y, start, sizeof(double) * n);
    double lam = 0.0;
    int64_t it;
    for (it = 1; it <= maxit; ++it) {
        double ss = 0.0;
        for (int i = 0; i < n; ++i) ss = ss + y[i] * y[i];
        double nrm = sqrt(ss);
        for (int i = 0; i < n; ++i) v[i] = y[i] / nrm;
        for (int i = 0; i < n; ++i) y[i] = 0.0;
        for (int j = 0; j < n; ++j) {
            double vj = v[j];
            const double *Aj = A + (size_t)j * n;
            for (int i = 0; i < n; ++i) y[i] = y[i] + Aj[i] * vj;
        }
        lam = 0.0;
        for (int i = 0; i < n; ++i) lam = lam + y[i] * v[i];
        double del = 0.0;
        for (int i = 0; i < n; ++i) {
            double t = y[i] - lam * v[i];
            del = del + t * t;
        }
        del = del / fabs(lam);
        if (del <= POWER_TOL) break;
    }
    *lambda = fabs(lam);
    if (iters) *iters = it > maxit ? maxit : it;
    free(y);
    free(v);
    return 0;
}

/* choleskyPD (soda.f90:8-47): U upper, A read from its lower triangle. Returns
 * 0 on success, -1 for a bad diagonal, i (1-based) for failure at row i. */
static int cholesky_pd_ld(int n, const double *A, double *U, int ldu)
{
    if (n <= 0) return -1;
    for (int i = 0; i < n; ++i)
        if (A[IDX2(i, i, n)] <= 0.0) return -1;
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) U[IDX2(i, j, ldu)] = 0.0;
    for (int i = 0; i < n; ++i) {
        double dd = 0.0;
        for (int k = 0; k < i; ++k) dd = dd + U[IDX2(k, i, ldu)] * U[IDX2(k, i, ldu)];
        double tmp = A[IDX2(i, i, n)] - dd;
        if (tmp <= 0.0 || isnan(tmp)) return i + 1;
        double uii = sqrt(tmp);
        U[IDX2(i, i, ldu)] = uii;
#pragma omp parallel for schedule(static) if (n - i > 256)
        for (int j = i + 1; j < n; ++j) {
            double dj = 0.0;
            for (int k = 0; k < i; ++k) dj = dj + U[IDX2(k, j, ldu)] * U[IDX2(k, i, ldu)];
            U[IDX2(i, j, ldu)] = (A[IDX2(j, i, n)] - dj) / uii;
        }
    }
    return 0;
}

int oracle_cholesky_pd(int32_t n, const double *A, double *U)
{
    return cholesky_pd_ld(n, A, U, n);
}

/* IDMAX (soda.f90 helper): smallest index of the maximum, stride incx. */
static int idmax(int n, const double *x, int incx)
{
    if (n < 1 || incx <= 0) return 0;
    int k = 1;
    if (n == 1) return 1;
    double r = x[0];
    for (int i = 2; i <= n; ++i) {
        double v = x[(size_t)(i - 1) * incx];
        if (v > r) { k = i; r = v; }
    }
    return k;
}

static void dswap_(int n, double *dx, int incx, double *dy, int incy)
{
    for (int i = 0; i < n; ++i) {
        double t = dx[(size_t)i * incx];
        dx[(size_t)i * incx] = dy[(size_t)i * incy];
        dy[(size_t)i * incy] = t;
    }
}

/* choleskyPSD (soda.f90:49-124): pivoted upper Cholesky in place. Returns 0
 * (rank in *rank, 1-based pivots in piv) or -1. */
int oracle_cholesky_psd(int32_t n, double *A, int32_t *piv, int32_t *rank)
{
#define A_(i, j) A[IDX2((i) - 1, (j) - 1, n)]
    if (n <= 0) return -1;
    double *work = (double *)calloc((size_t)2 * n, sizeof(double));
    if (!work) return SODAGPU_E_NOMEM;
    for (int p = 1; p <= n; ++p) piv[p - 1] = p;
    const double EPS = 2.220446049250313e-16;
    int pvt = idmax(n, A, n + 1);
    double Ajj = A_(pvt, pvt);
    if (Ajj <= EPS) { *rank = 0; free(work); return -1; }
    double DSTOP = n * EPS * Ajj;
    for (int p = 1; p <= n; ++p) work[p - 1] = 0;
    for (int j = 1; j <= n; ++j) {
        for (int p = j; p <= n; ++p) {
            if (j > 1) work[p - 1] = work[p - 1] + A_(j - 1, p) * A_(j - 1, p);
            work[n + p - 1] = A_(p, p) - work[p - 1];
        }
        if (j > 1) {
            int itemp = idmax(n - j + 1, &work[n + j - 1], 1);
            pvt = itemp + j - 1;
            Ajj = work[n + pvt - 1];
            if (Ajj <= DSTOP) {
                A_(j, j) = Ajj;
                *rank = j - 1;
                free(work);
                return 0;
            }
        }
        if (j != pvt) {
            A_(pvt, pvt) = A_(j, j);
            dswap_(j - 1, &A_(1, j), 1, &A_(1, pvt), 1);
            if (pvt - j - 1 > 0) dswap_(pvt - j - 1, &A_(j, j + 1), n, &A_(j + 1, pvt), 1);
            if (pvt < n) dswap_(n - pvt, &A_(j, pvt + 1), n, &A_(pvt, pvt + 1), n);
            double dt = work[j - 1];
            work[j - 1] = work[pvt - 1];
            work[pvt - 1] = dt;
            int it = piv[pvt - 1];
            piv[pvt - 1] = piv[j - 1];
            piv[j - 1] = it;
        }
        Ajj = sqrt(Ajj);
        A_(j, j) = Ajj;
        if (j < n) {
            /* DGEMV('Trans', j-1, n-j, -1, A(1,j+1), n, A(1,j), 1, 1, A(j,j+1), n) */
            for (int jc = 1; jc <= n - j; ++jc) {
                double temp = 0.0;
                for (int i = 1; i <= j - 1; ++i) temp = temp + A_(i, j + jc) * A_(i, j);
                A_(j, j + jc) = A_(j, j + jc) + (-1.0) * temp;
            }
            /* DSCAL(n-j, 1.0/Ajj, A(j,j+1), n) */
            double sc = 1.0 / Ajj;
            for (int jc = 1; jc <= n - j; ++jc) A_(j, j + jc) = sc * A_(j, j + jc);
        }
    }
    *rank = n;
    free(work);
    return 0;
#undef A_
}

/* get_aug_matrix (soda.f90:445-518) and the tail of setup_soda (436-441). */
int oracle_build_z(oracle_ctx *o, const int32_t *permvec, int64_t power_maxit,
                   double d_offset, int32_t *nskipped_out)
{
    if (!o || !o->have_geno) return SODAGPU_E_STATE;
    const int bs = o->bs, p = o->p;
    if (o->regular) {
        /* regular_bayes: every SNP single-site, in order (permvec(i) = i, models.f90:675-678) */
        for (int k = 0; k < p; ++k) {
            o->perm[k] = k;
            o->iskipped[k] = k;
        }
        memset(o->skip, 0, p);
        o->nskipped = p;
        o->naless = 1;
        o->naind = 0;
        o->have_z = 1;
        if (nskipped_out) *nskipped_out = 0;
        (void)permvec;
        (void)power_maxit;
        (void)d_offset;
        return 0;
    }
    for (int k = 0; k < p; ++k) {
        int v = permvec ? permvec[k] - 1 : k;
        if (v < 0 || v >= p) return SODAGPU_E_ARG;
        o->perm[k] = v;
    }
    int nbatch;
    uint64_t *gb = make_genbits(o, &nbatch);
    double *xx = (double *)malloc(sizeof(double) * (size_t)bs * bs);
    double *start = (double *)malloc(sizeof(double) * bs);
    int32_t *piv = (int32_t *)malloc(sizeof(int32_t) * bs);
    if (!gb || !xx || !start || !piv) {
        free(gb); free(xx); free(start); free(piv);
        return SODAGPU_E_NOMEM;
    }
    memset(o->skip, 0, p);
    memset(o->iskipped, 0, sizeof(int32_t) * p);
    o->nskipped = 0;
    o->naless = p;
    memset(o->XA, 0, sizeof(double) * (size_t)bs * p);
    int rc = 0;
    for (int b = 0; b < o->nb && rc == 0; ++b) {
        int ls, le;
        block_bounds(o, b, &ls, &le);
        const int nn = le - ls + 1;
#pragma omp parallel for schedule(dynamic, 4)
        for (int j = 0; j < nn; ++j) {
            int jj = o->perm[ls + j - 1];
            for (int k = 0; k <= j; ++k) {
                int kk = o->perm[ls + k - 1];
                double v = xxproduct(o, gb, nbatch, jj, kk);
                xx[IDX2(k, j, nn)] = v;
                xx[IDX2(j, k, nn)] = v;
            }
        }
        rng_t r;
        r.mode = o->rng_mode;
        r.tmode = 0;
        r.xo = &o->xo[0];
        ctr_init(&r.c, o->cfg.seed, 0, 0, b, P_POWER);
        for (int i = 0; i < nn; ++i) start[i] = rng_u(&r);
        double lam;
        if (power_maxit < 0) {
            /* timing samples only: Gershgorin upper bound instead of lambda_max */
            lam = 0.0;
            for (int j = 0; j < nn; ++j) {
                double rs = 0.0;
                for (int k = 0; k < nn; ++k) rs += fabs(xx[IDX2(k, j, nn)]);
                if (rs > lam) lam = rs;
            }
        } else {
            int64_t maxit = power_maxit > 0 ? power_maxit : (int64_t)1000 * nn;
            oracle_power_method(nn, xx, start, maxit, &lam, NULL);
        }
        double d = lam + D_SHIFT + d_offset;
        o->xxd[b] = d;
        for (size_t t = 0; t < (size_t)nn * nn; ++t) xx[t] = -xx[t];
        for (int j = 0; j < nn; ++j) xx[IDX2(j, j, nn)] = d + xx[IDX2(j, j, nn)];
        double *U = o->XA + (size_t)(ls - 1) * bs;
        int st = cholesky_pd_ld(nn, xx, U, bs);
        if (st != 0) {
            int rank = 0;
            int ps = oracle_cholesky_psd(nn, xx, piv, &rank);
            if (ps != 0) { rc = SODAGPU_E_NOTPSD; break; }
            for (int j = 1; j <= nn; ++j) {
                int jj = piv[j - 1];
                if (j <= rank) {
                    double *col = o->XA + (size_t)(ls + jj - 2) * bs;
                    for (int i = 0; i < j; ++i) col[i] = xx[IDX2(i, j - 1, nn)];
                } else {
                    o->skip[ls + jj - 2] = 1;
                    o->iskipped[o->nskipped++] = o->perm[ls + jj - 2];
                }
            }
        } else {
            o->naless = 0;
        }
        int cand = bs - nn + o->nskipped;
        if (cand < o->naless) o->naless = cand;
    }
    free(gb); free(xx); free(start); free(piv);
    if (rc) return rc;
    o->naind = bs - o->naless;
    o->have_z = 1;
    if (nskipped_out) *nskipped_out = o->nskipped;
    return 0;
}

/* Takes the augmenting matrix from elsewhere (XA(bs, p) column-major and
 * xxd(nb), identity SNP order, no skipped SNPs) instead of building it, so
 * that a sweep can be compared on the same Z.  The factor's conditioning
 * (its smallest eigenvalue is the 0.001 of soda.f90:485) turns a 1e-12
 * relative difference in d into ~1e-9 in U, which would otherwise reach
 * the sweep. */
int oracle_set_z(oracle_ctx *o, const double *xa, const double *xxd)
{
    if (!o || !o->have_geno || !xa || !xxd || o->regular) return SODAGPU_E_STATE;
    for (int k = 0; k < o->p; ++k) o->perm[k] = k;
    memcpy(o->XA, xa, sizeof(double) * (size_t)o->bs * o->p);
    memcpy(o->xxd, xxd, sizeof(double) * o->nb);
    memset(o->skip, 0, o->p);
    memset(o->iskipped, 0, sizeof(int32_t) * o->p);
    o->nskipped = 0;
    o->naless = 0;
    o->naind = o->bs;
    o->have_z = 1;
    return 0;
}

int oracle_get_z(oracle_ctx *o, double *xa, double *xxd, int32_t *skip)
{
    if (!o || !o->have_z) return SODAGPU_E_STATE;
    if (xa) memcpy(xa, o->XA, sizeof(double) * (size_t)o->bs * o->p);
    if (xxd) memcpy(xxd, o->xxd, sizeof(double) * o->nb);
    if (skip)
        for (int k = 0; k < o->p; ++k) skip[k] = o->skip[k];
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Sampler                                                                  */
/* ------------------------------------------------------------------------ */

/* Injected-draw tape sites (layout of sodagpu_set_tape): 0 mu, 1 sigma2_g,
 * 2 sigma2_e, 3 + i pi of group i, 3 + ngroup + i ra_i, 3 + ngroup +
 * blocksize + j SNP j (block draw or single-site draw). */
static void tape_site(oracle_ctx *o, rng_t *R, int rep, int site)
{
    R->tmode = 0;
    if (!o->tape) return;
    if (rep >= o->tape_reps) {
        if (o->tape_play) o->tape_over = 1;   /* playing past the end of the tape */
        return;
    }
    R->tp = o->tape + ((size_t)rep * o->tape_sites + site) * SODAGPU_TAPE_W;
    R->tn = 0;
    R->tmode = o->tape_play ? 2 : 1;
}

static void tape_end(oracle_ctx *o, rng_t *R)
{
    if (R->tmode && R->tn > SODAGPU_TAPE_W) o->tape_over = 1;
    R->tmode = 0;
}

static int snp_site(const oracle_ctx *o, int snploc) { return 3 + o->ngroup + o->cfg.blocksize + snploc; }

int oracle_set_tape(oracle_ctx *o, double *tape, int32_t reps, int32_t record)
{
    if (!o || (tape && reps < 1) || o->nchain != 1) return SODAGPU_E_ARG;
    o->tape = tape;
    o->tape_reps = tape ? reps : 0;
    o->tape_sites = 3 + o->ngroup + o->cfg.blocksize + o->p;
    o->tape_play = !record;
    o->tape_over = 0;
    return 0;
}

int oracle_tape_sites(const oracle_ctx *o) { return o ? 3 + o->ngroup + o->cfg.blocksize + o->p : 0; }

/* compute_residuals (utilities.f90:609-614) */
static void compute_residuals(const oracle_ctx *o, chain_t *c)
{
    const int n = o->n, p = o->p;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        double d = 0.0;
        for (int j = 0; j < p; ++j) d = d + o->X[IDX2(i, j, n)] * c->g[j];
        c->r[i] = o->y[i] - d - c->mu;
    }
}

static int is_ab(int m) { return m == SODAGPU_BAYES_A || m == SODAGPU_BAYES_B; }

static int init_chains_(oracle_ctx *o);

int oracle_init_chains(oracle_ctx *o)
{
    int rc = init_chains_(o);
    return rc ? rc : (o->tape_over ? SODAGPU_E_ARG : 0);
}

static int init_chains_(oracle_ctx *o)
{
    if (!o || !o->have_geno || !o->have_pheno || !o->have_z) return SODAGPU_E_STATE;
    const int n = o->n, p = o->p, nm = o->nmix, ng = o->ngroup, m = o->method;
    if (!o->ch) {
        o->ch = (chain_t *)calloc(o->nchain, sizeof(chain_t));
        if (!o->ch) return SODAGPU_E_NOMEM;
        for (int ci = 0; ci < o->nchain; ++ci) {
            chain_t *c = &o->ch[ci];
            c->g = calloc(p, sizeof(double));
            c->r = calloc(n, sizeof(double));
            c->ra = calloc(o->bs, sizeof(double));
            c->vara_s = calloc(p, sizeof(double));
            c->gtemp = calloc(o->bs, sizeof(double));
            c->cls = calloc(p, sizeof(int32_t));
            c->gflag = calloc(o->bs, sizeof(int32_t));
            c->p = calloc((size_t)ng * nm, sizeof(double));
            c->log_p = calloc((size_t)ng * nm, sizeof(double));
            c->snpindist = calloc((size_t)ng * nm, sizeof(int32_t));
            c->varindist = calloc((size_t)ng * nm, sizeof(double));
            c->gstore = calloc(p, sizeof(double));
            c->indiststore = calloc((size_t)p * nm, sizeof(double));
            c->vara_sstore = calloc(p, sizeof(double));
            c->snpstore = calloc((size_t)ng * nm, sizeof(double));
            c->pstore = calloc((size_t)ng * nm, sizeof(double));
            c->varstore = calloc((size_t)ng * nm, sizeof(double));
            if (!c->g || !c->r || !c->ra || !c->vara_s || !c->gtemp || !c->cls || !c->gflag ||
                !c->p || !c->log_p || !c->snpindist || !c->varindist || !c->gstore ||
                !c->indiststore || !c->vara_sstore || !c->snpstore || !c->pstore || !c->varstore)
                return SODAGPU_E_NOMEM;
        }
    }
    const double nn = (double)n;
    /* xpx of skipped SNPs (models.f90:82-85) */
    for (int t = 0; t < o->nskipped; ++t) {
        int j = o->iskipped[t];
        double s = 0.0;
        for (int i = 0; i < n; ++i) s = s + o->X[IDX2(i, j, n)] * o->X[IDX2(i, j, n)];
        o->xpx[j] = s;
    }
    for (int ci = 0; ci < o->nchain; ++ci) {
        chain_t *c = &o->ch[ci];
        c->counter = 0;
        c->rep = 0;
        c->scale_va = o->cfg.scale_va;
        c->vara = o->cfg.vara0;
        c->included = 0;
        c->included_store = 0;
        memset(c->snpstore, 0, sizeof(double) * ng * nm);
        memset(c->indiststore, 0, sizeof(double) * (size_t)p * nm);
        memset(c->varstore, 0, sizeof(double) * ng * nm);
        memset(c->pstore, 0, sizeof(double) * ng * nm);
        memset(c->vara_sstore, 0, sizeof(double) * p);
        c->vara_store = 0;
        memset(c->gflag, 0, sizeof(int32_t) * o->bs);
        if (m != SODAGPU_BAYES_A) {
            for (int j = 0; j < p; ++j) c->cls[j] = 2;
            if (m == SODAGPU_BAYES_B || m == SODAGPU_BAYES_C) {
                for (int i = 0; i < ng; ++i) {
                    c->p[IDX2(i, 0, ng)] = o->cfg.pizero;
                    c->p[IDX2(i, 1, ng)] = 1.0 - o->cfg.pizero;
                }
            } else {
                for (int i = 0; i < ng; ++i) {
                    c->p[IDX2(i, 0, ng)] = 0.5;
                    double s = 0.0;
                    for (int j = 1; j < nm; ++j) c->p[IDX2(i, j, ng)] = 1.0 / o->cfg.mix[j];
                    for (int j = 1; j < nm; ++j) s = s + c->p[IDX2(i, j, ng)];
                    for (int j = 1; j < nm; ++j)
                        c->p[IDX2(i, j, ng)] = 0.5 * c->p[IDX2(i, j, ng)] / s;
                }
            }
        } else {
            for (int j = 0; j < p; ++j) c->cls[j] = 1;
        }
        double sy = 0.0;
        for (int i = 0; i < n; ++i) sy = sy + o->y[i];
        c->mu = sy / nn;
        memset(c->g, 0, sizeof(double) * p);
        memset(c->gstore, 0, sizeof(double) * p);
        c->mu_store = 0;
        compute_residuals(o, c);
        if (o->cfg.df_va <= 0.0) {
            double yhat = sy / nn, vary = 0.0;
            for (int i = 0; i < n; ++i) vary = vary + (o->y[i] - yhat) * (o->y[i] - yhat);
            vary = vary / (nn - 1.0);
            if (m == SODAGPU_BAYES_A) {
                c->vara = c->scale_va * vary / p;
            } else if (m == SODAGPU_BAYES_B) {
                c->vara = c->scale_va * vary / p / c->p[IDX2(0, 1, ng)];
            } else {
                for (int i = 0; i < ng; ++i) {
                    double dp = 0.0;
                    for (int j = 0; j < nm; ++j) dp = dp + c->p[IDX2(i, j, ng)] * o->cfg.mix[j];
                    c->vara = c->vara + dp;
                }
                c->vara = c->scale_va * vary / p / c->vara;
            }
            c->scale_va = 0.0;
        } else {
            c->vara = c->scale_va * o->cfg.df_va / (o->cfg.df_va + 2.0);
        }
        if (is_ab(m)) {
            for (int j = 0; j < p; ++j) c->vara_s[j] = c->vara;
        } else {
            for (int j = 0; j < nm; ++j) c->gp[j] = o->cfg.mix[j] * c->vara;
        }
        double rr = 0.0;
        for (int i = 0; i < n; ++i) rr = rr + c->r[i] * c->r[i];
        double scale = (rr + o->cfg.scale_ve * o->cfg.df_ve) / (nn + o->cfg.df_ve);
        rng_t R;
        R.mode = o->rng_mode;
        R.tmode = 0;
        R.xo = &o->xo[0];
        ctr_init(&R.c, o->cfg.seed, ci, 0, 0, P_VARE);
        tape_site(o, &R, 0, 2);
        c->vare = rscinvchi2(nn + o->cfg.df_ve, scale, &R);
        tape_end(o, &R);
        c->vare_store = 0;
        memset(c->ra, 0, sizeof(double) * o->bs);
        for (int i = 0; i < o->naind; ++i) {
            if (o->rng_mode == ORACLE_RNG_COUNTER) ctr_init(&R.c, o->cfg.seed, ci, 0, i, P_RA);
            tape_site(o, &R, 0, 3 + o->ngroup + i);
            c->ra[i] = rnorm(0.0, sqrt(c->vare), &R);
            tape_end(o, &R);
        }
    }
    o->have_chain = 1;
    return 0;
}

/* Per-SNP conditional draw of one SNP inside a block (models.f90:146-161,
 * 211-255, 350-412).  Returns the new g and writes gtemp/gflag. */
static void draw_in_block(const oracle_ctx *o, chain_t *c, int k /*0-based pos*/,
                          int jk, double zz, double zz_vare, rng_t *R)
{
    const int n = o->n, m = o->method, nm = o->nmix, ng = o->ngroup;
    const int snploc = o->perm[k];
    const double *z = o->X + (size_t)snploc * n;
    const double *za = o->XA + (size_t)k * o->bs;
    const double vare = c->vare;
    double gk = c->g[snploc];
    double d1 = 0.0, d2 = 0.0;
    for (int i = 0; i < n; ++i) d1 = d1 + c->r[i] * z[i];
    for (int i = 0; i < o->bs; ++i) d2 = d2 + c->ra[i] * za[i];
    double rhs = d1 + d2;
    if (m == SODAGPU_BAYES_A) {
        rhs = rhs + zz * gk;
        c->gtemp[jk] = gk;
        double v1 = zz + vare / c->vara_s[snploc];
        gk = rnorm(rhs / v1, sqrt(vare / v1), R);
        c->g[snploc] = gk;
        double scale = (gk * gk + c->scale_va * o->cfg.df_va) / (o->cfg.df_va + 1.0);
        c->vara_s[snploc] = rscinvchi2(o->cfg.df_va + 1.0, scale, R);
        return;
    }
    if (c->cls[snploc] > 1) rhs = rhs + zz * gk;
    if (m == SODAGPU_BAYES_B) {
        double s1 = c->log_p[IDX2(0, 0, ng)];
        double logdetV = log(c->vara_s[snploc] * zz_vare + 1.0);
        double uhat = rhs / (zz + vare / c->vara_s[snploc]);
        double s2 = -0.5 * (logdetV - (rhs * uhat / vare)) + c->log_p[IDX2(0, 1, ng)];
        double clike = s1 - s2, sk;
        if (clike > 700) sk = 0.0;
        else if (clike < -700) sk = 1.0;
        else sk = 1.0 / (1.0 + exp(clike));
        double r = rng_u(R);
        int flag = r < sk ? 2 : 1;
        c->gtemp[jk] = gk;
        if (flag == 1) {
            gk = rnorm(0.0, sqrt(c->vara_s[snploc]), R);
            c->g[snploc] = 0.0;
            if (c->cls[snploc] == 1) c->gflag[jk] = 1;
        } else {
            double v1 = zz + vare / c->vara_s[snploc];
            gk = rnorm(rhs / v1, sqrt(vare / v1), R);
            c->g[snploc] = gk;
        }
        c->cls[snploc] = flag;
        double scale = (gk * gk + c->scale_va * o->cfg.df_va) / (o->cfg.df_va + 1.0);
        c->vara_s[snploc] = rscinvchi2(o->cfg.df_va + 1.0, scale, R);
        return;
    }
    /* BayesC / Cpi / R / Rc */
    int sg = o->grp[snploc] - 1;
    double s[SODAGPU_MAXDIST], stemp[SODAGPU_MAXDIST];
    s[0] = c->log_p[IDX2(sg, 0, ng)];
    for (int kk = 1; kk < nm; ++kk) {
        double logdetV = log(c->gp[kk] * zz_vare + 1.0);
        double uhat = rhs / (zz + c->vare_gp[kk]);
        s[kk] = -0.5 * (logdetV - (rhs * uhat / vare)) + c->log_p[IDX2(sg, kk, ng)];
    }
    for (int kk = 0; kk < nm; ++kk) {
        double skk = s[kk], sk = 0.0;
        int overflow = 0;
        for (int j = 0; j < nm; ++j) {
            if (j == kk) continue;
            double clike = s[j] - skk;
            if (clike < -700) continue;
            else if (clike > 700) { overflow = 1; break; }
            sk = sk + exp(clike);
        }
        stemp[kk] = overflow ? 0.0 : 1.0 / (1.0 + sk);
    }
    double ssculm = 0.0, r = rng_u(R);
    int flag = 1;
    for (int kk = 0; kk < nm; ++kk) {
        ssculm = ssculm + stemp[kk];
        if (r < ssculm) { flag = kk + 1; break; }
    }
    c->gtemp[jk] = gk;
    if (flag == 1) {
        if (c->cls[snploc] == 1) c->gflag[jk] = 1;
        gk = 0.0;
    } else {
        double v1 = zz + vare / c->gp[flag - 1];
        gk = rnorm(rhs / v1, sqrt(vare / v1), R);
    }
    c->cls[snploc] = flag;
    c->g[snploc] = gk;
}

/* Single-site update of a SNP dropped by the pivoted fallback
 * (models.f90:178-193, 276-320, 433-495).  The reference reads the module
 * arrays log_p and vare_gp here, which its parallel regions never assign
 * (they are private there); the current values are used instead. */
static void draw_skipped(const oracle_ctx *o, chain_t *c, int snploc, rng_t *R)
{
    const int n = o->n, m = o->method, nm = o->nmix, ng = o->ngroup;
    const double *z = o->X + (size_t)snploc * n;
    const double vare = c->vare;
    double zz = o->xpx[snploc], zz_vare = zz / vare;
    double gk = c->g[snploc], gt;
    double rhs = 0.0;
    for (int i = 0; i < n; ++i) rhs = rhs + c->r[i] * z[i];
    if (m == SODAGPU_BAYES_A) {
        rhs = rhs + zz * gk;
        double v1 = zz + vare / c->vara_s[snploc];
        gt = rnorm(rhs / v1, sqrt(vare / v1), R);
        gk = gk - gt;
        for (int i = 0; i < n; ++i) c->r[i] = c->r[i] + z[i] * gk;
        c->g[snploc] = gt;
        double scale = (gt * gt + c->scale_va * o->cfg.df_va) / (o->cfg.df_va + 1.0);
        c->vara_s[snploc] = rscinvchi2(o->cfg.df_va + 1.0, scale, R);
        return;
    }
    if (c->cls[snploc] > 1) rhs = rhs + zz * gk;
    if (m == SODAGPU_BAYES_B) {
        double s1 = c->log_p[IDX2(0, 0, ng)];
        double logdetV = log(c->vara_s[snploc] * zz_vare + 1.0);
        double uhat = rhs / (zz + vare / c->vara_s[snploc]);
        double s2 = -0.5 * (logdetV - (rhs * uhat / vare)) + c->log_p[IDX2(0, 1, ng)];
        double clike = s1 - s2, sk;
        if (clike > 700) sk = 0.0;
        else if (clike < -700) sk = 1.0;
        else sk = 1.0 / (1.0 + exp(clike));
        double r = rng_u(R);
        int flag = r < sk ? 2 : 1;
        if (flag == 1) {
            gt = rnorm(0.0, sqrt(c->vara_s[snploc]), R);
            if (c->cls[snploc] > 1)
                for (int i = 0; i < n; ++i) c->r[i] = c->r[i] + z[i] * gk;
            c->g[snploc] = 0.0;
        } else {
            double v1 = zz + vare / c->vara_s[snploc];
            gt = rnorm(rhs / v1, sqrt(vare / v1), R);
            gk = gk - gt;
            for (int i = 0; i < n; ++i) c->r[i] = c->r[i] + z[i] * gk;
            c->g[snploc] = gt;
        }
        c->cls[snploc] = flag;
        double scale = (gt * gt + c->scale_va * o->cfg.df_va) / (o->cfg.df_va + 1.0);
        c->vara_s[snploc] = rscinvchi2(o->cfg.df_va + 1.0, scale, R);
        return;
    }
    int sg = o->grp[snploc] - 1;
    double s[SODAGPU_MAXDIST], stemp[SODAGPU_MAXDIST];
    s[0] = c->log_p[IDX2(sg, 0, ng)];
    for (int kk = 1; kk < nm; ++kk) {
        double logdetV = log(c->gp[kk] * zz_vare + 1.0);
        double uhat = rhs / (zz + c->vare_gp[kk]);
        s[kk] = -0.5 * (logdetV - (rhs * uhat / vare)) + c->log_p[IDX2(sg, kk, ng)];
    }
    for (int kk = 0; kk < nm; ++kk) {
        double skk = s[kk], sk = 0.0;
        int overflow = 0;
        for (int j = 0; j < nm; ++j) {
            if (j == kk) continue;
            double clike = s[j] - skk;
            if (clike < -700) continue;
            else if (clike > 700) { overflow = 1; break; }
            sk = sk + exp(clike);
        }
        stemp[kk] = overflow ? 0.0 : 1.0 / (1.0 + sk);
    }
    double ssculm = 0.0, r = rng_u(R);
    int flag = 1;
    for (int kk = 0; kk < nm; ++kk) {
        ssculm = ssculm + stemp[kk];
        if (r < ssculm) { flag = kk + 1; break; }
    }
    if (flag == 1) {
        gt = 0.0;
        if (c->cls[snploc] > 1)
            for (int i = 0; i < n; ++i) c->r[i] = c->r[i] + z[i] * gk;
    } else {
        double v1 = zz + vare / c->gp[flag - 1];
        gt = rnorm(rhs / v1, sqrt(vare / v1), R);
        gk = gk - gt;
        for (int i = 0; i < n; ++i) c->r[i] = c->r[i] + z[i] * gk;
    }
    c->g[snploc] = gt;
    c->cls[snploc] = flag;
}

/* static OpenMP chunk of iteration `t` among `T` threads for N iterations */
static void static_chunk(int N, int T, int t, int *lo, int *hi)
{
    int q = N / T, rem = N % T;
    *lo = t * q + (t < rem ? t : rem);
    *hi = *lo + q + (t < rem ? 1 : 0);
}

/* One block of the sweep: rhs + draws (the first `!$omp do`) and the residual
 * update (the second `!$omp do reduction(+:yadj,yAadj)`). */
static void sweep_block(oracle_ctx *o, chain_t *c, int ci, int b, int rep)
{
    const int n = o->n, bs = o->bs, m = o->method;
    int ls, le;
    block_bounds(o, b, &ls, &le);
    const int N = le - ls + 1;
    const double zz = o->xxd[b], zz_vare = zz / c->vare;
    if (o->rng_mode == ORACLE_RNG_REFERENCE) {
        for (int t = 0; t < o->ref_threads; ++t) {
            int lo, hi;
            static_chunk(N, o->ref_threads, t, &lo, &hi);
            rng_t R;
            R.mode = ORACLE_RNG_REFERENCE;
            R.tmode = 0;
            R.xo = &o->xo[t];
            for (int jk = lo; jk < hi; ++jk) {
                int k = ls - 1 + jk;
                if (o->skip[k]) continue;
                tape_site(o, &R, rep, snp_site(o, o->perm[k]));
                draw_in_block(o, c, k, jk, zz, zz_vare, &R);
                tape_end(o, &R);
            }
        }
    } else {
#pragma omp parallel for schedule(static)
        for (int jk = 0; jk < N; ++jk) {
            int k = ls - 1 + jk;
            if (o->skip[k]) continue;
            rng_t R;
            R.mode = ORACLE_RNG_COUNTER;
            R.tmode = 0;
            R.xo = NULL;
            ctr_init(&R.c, o->cfg.seed, ci, rep, o->perm[k], P_SNP);
            tape_site(o, &R, rep, snp_site(o, o->perm[k]));
            draw_in_block(o, c, k, jk, zz, zz_vare, &R);
            tape_end(o, &R);
        }
    }
    /* residual update, SNP order within each element (models.f90:164-174) */
    int *nz = (int *)malloc(sizeof(int) * N);
    double *dl = (double *)malloc(sizeof(double) * N);
    int nnz = 0;
    for (int jk = 0; jk < N; ++jk) {
        int k = ls - 1 + jk;
        if (o->skip[k]) continue;
        if (m != SODAGPU_BAYES_A && c->gflag[jk] == 1) {
            c->gflag[jk] = 0;
            continue;
        }
        double gdiff = c->gtemp[jk] - c->g[o->perm[k]];
        nz[nnz] = k;
        dl[nnz] = gdiff;
        ++nnz;
    }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        double ri = c->r[i];
        for (int t = 0; t < nnz; ++t) ri = ri + o->X[IDX2(i, o->perm[nz[t]], n)] * dl[t];
        c->r[i] = ri;
    }
    for (int i = 0; i < bs; ++i) {
        double ai = c->ra[i];
        for (int t = 0; t < nnz; ++t) ai = ai + o->XA[IDX2(i, nz[t], bs)] * dl[t];
        c->ra[i] = ai;
    }
    free(nz);
    free(dl);
}

/* One Gibbs iteration of one chain (models.f90:129-574). */
static void iterate(oracle_ctx *o, chain_t *c, int ci, int rep, sodagpu_trace_cb cb,
                    void *user)
{
    const int n = o->n, p = o->p, nm = o->nmix, ng = o->ngroup, m = o->method;
    const double nn = (double)n;
    rng_t R0;
    R0.mode = o->rng_mode;
    R0.tmode = 0;
    R0.xo = &o->xo[0];
    /* mu (130-132) */
    double s = 0.0;
    for (int i = 0; i < n; ++i) { c->r[i] = c->r[i] + c->mu; s = s + c->r[i]; }
    ctr_init(&R0.c, o->cfg.seed, ci, rep, 0, P_MU);
    tape_site(o, &R0, rep, 0);
    c->mu = rnorm(s / nn, sqrt(c->vare / nn), &R0);
    tape_end(o, &R0);
    for (int i = 0; i < n; ++i) c->r[i] = c->r[i] - c->mu;
    /* log_p / vare_gp of the parallel region (198-199, 330-338) */
    if (m != SODAGPU_BAYES_A) {
        for (int i = 0; i < ng; ++i)
            for (int j = 0; j < nm; ++j) c->log_p[IDX2(i, j, ng)] = log(c->p[IDX2(i, j, ng)]);
        for (int j = 1; j < nm; ++j) c->vare_gp[j] = c->vare / c->gp[j];
    }
    for (int b = 0; b < o->nb; ++b) sweep_block(o, c, ci, b, rep);
    for (int t = 0; t < o->nskipped; ++t) {
        int snploc = o->iskipped[t];
        if (o->rng_mode == ORACLE_RNG_COUNTER) ctr_init(&R0.c, o->cfg.seed, ci, rep, snploc, P_SKIP);
        tape_site(o, &R0, rep, snp_site(o, snploc));
        draw_skipped(o, c, snploc, &R0);
        tape_end(o, &R0);
    }
    /* counts and variances (194, 321-325, 496-513) */
    if (m == SODAGPU_BAYES_A) {
        double v = 0.0;
        for (int j = 0; j < p; ++j) v = v + c->g[j] * c->g[j];
        c->varindist[0] = v;
    } else if (m == SODAGPU_BAYES_B) {
        int inc = 0;
        double v = 0.0;
        for (int j = 0; j < p; ++j)
            if (c->cls[j] == 2) { inc++; v = v + c->g[j] * c->g[j]; }
        c->included = inc;
        c->snpindist[0] = p - inc;
        c->snpindist[1] = inc;
        c->varindist[0] = 0.0;
        c->varindist[1] = v;
    } else {
        int excl = 0;
        for (int i = 0; i < ng; ++i) {
            for (int j = 0; j < nm; ++j) {
                int cnt = 0;
                double v = 0.0;
                for (int l = 0; l < p; ++l)
                    if (o->grp[l] == i + 1 && c->cls[l] == j + 1) { cnt++; v = v + c->g[l] * c->g[l]; }
                c->snpindist[IDX2(i, j, ng)] = cnt;
                c->varindist[IDX2(i, j, ng)] = v;
            }
            excl += c->snpindist[IDX2(i, 0, ng)];
        }
        c->included = p - excl;
        double scale = 0.0;
        for (int i = 0; i < ng; ++i)
            for (int j = 1; j < nm; ++j) scale = scale + c->varindist[IDX2(i, j, ng)] / o->cfg.mix[j];
        scale = (scale + c->scale_va * o->cfg.df_va) / (o->cfg.df_va + (double)c->included);
        ctr_init(&R0.c, o->cfg.seed, ci, rep, 0, P_VARA);
        tape_site(o, &R0, rep, 1);
        c->vara = rscinvchi2((double)c->included + o->cfg.df_va, scale, &R0);
        tape_end(o, &R0);
        for (int j = 0; j < nm; ++j) c->gp[j] = o->cfg.mix[j] * c->vara;
    }
    /* vare (515-516) */
    double rr = 0.0;
    for (int i = 0; i < n; ++i) rr = rr + c->r[i] * c->r[i];
    double scale = (rr + o->cfg.scale_ve * o->cfg.df_ve) / (nn + o->cfg.df_ve);
    ctr_init(&R0.c, o->cfg.seed, ci, rep, 0, P_VARE);
    tape_site(o, &R0, rep, 2);
    c->vare = rscinvchi2(nn + o->cfg.df_ve, scale, &R0);
    tape_end(o, &R0);
    /* pi (517-522) */
    if (m == SODAGPU_BAYES_CPI || m == SODAGPU_BAYES_R || m == SODAGPU_BAYES_RC) {
        double dirx[SODAGPU_MAXDIST], pi[SODAGPU_MAXDIST];
        for (int i = 0; i < ng; ++i) {
            for (int j = 0; j < nm; ++j)
                dirx[j] = (double)c->snpindist[IDX2(i, j, ng)] + o->cfg.alpha[j];
            ctr_init(&R0.c, o->cfg.seed, ci, rep, i, P_PI);
            tape_site(o, &R0, rep, 3 + i);
            rdirichlet(nm, dirx, pi, &R0);
            tape_end(o, &R0);
            for (int j = 0; j < nm; ++j) c->p[IDX2(i, j, ng)] = pi[j];
        }
    }
    /* augmented residual redraw (523-525) */
    for (int i = 0; i < o->naind; ++i) {
        if (o->rng_mode == ORACLE_RNG_COUNTER) ctr_init(&R0.c, o->cfg.seed, ci, rep, i, P_RA);
        tape_site(o, &R0, rep, 3 + ng + i);
        c->ra[i] = rnorm(0.0, sqrt(c->vare), &R0);
        tape_end(o, &R0);
    }
    /* accumulators (526-548) */
    if (rep > o->cfg.burnin && rep % o->cfg.thin == 0) {
        c->counter++;
        for (int j = 0; j < p; ++j) c->gstore[j] = c->gstore[j] + c->g[j];
        c->mu_store = c->mu_store + c->mu;
        /* soda_bayes keeps varstore for every method (models.f90:530), regular_bayes not
           for BayesA (models.f90:893-896) */
        if (!(o->regular && m == SODAGPU_BAYES_A))
            for (int t = 0; t < ng * nm; ++t) c->varstore[t] = c->varstore[t] + c->varindist[t];
        c->vare_store = c->vare_store + c->vare;
        if (m != SODAGPU_BAYES_A) {
            c->included_store = c->included_store + c->included;
            for (int t = 0; t < ng * nm; ++t) c->snpstore[t] = c->snpstore[t] + c->snpindist[t];
            for (int j = 0; j < p; ++j) c->indiststore[IDX2(j, c->cls[j] - 1, p)] += 1.0;
            if (m != SODAGPU_BAYES_B && m != SODAGPU_BAYES_C)
                for (int t = 0; t < ng * nm; ++t) c->pstore[t] = c->pstore[t] + c->p[t];
        }
        if (is_ab(m)) {
            for (int j = 0; j < p; ++j) c->vara_sstore[j] = c->vara_sstore[j] + c->vara_s[j];
        } else {
            c->vara_store = c->vara_store + c->vara;
        }
    }
    if (cb && rep % o->cfg.thin == 0) {
        sodagpu_trace_row row;
        memset(&row, 0, sizeof row);
        row.chain = ci;
        row.rep = rep;
        row.included = c->included;
        row.mu = c->mu;
        row.vare = c->vare;
        row.vara = c->vara;
        for (int j = 0; j < nm; ++j) {
            row.snpindist[j] = c->snpindist[IDX2(0, j, ng)];
            row.varindist[j] = c->varindist[IDX2(0, j, ng)];
        }
        cb(user, &row);
    }
    if (o->cfg.recal_every > 0 && rep % o->cfg.recal_every == 0) compute_residuals(o, c);
}

int oracle_run(oracle_ctx *o, int32_t iters, sodagpu_trace_cb cb, void *user)
{
    if (!o || !o->have_chain) return SODAGPU_E_STATE;
    if (iters < 0) return SODAGPU_E_ARG;
    for (int t = 0; t < iters; ++t)
        for (int ci = 0; ci < o->nchain; ++ci) {
            chain_t *c = &o->ch[ci];
            c->rep++;
            iterate(o, c, ci, c->rep, cb, user);
        }
    return o->tape_over ? SODAGPU_E_ARG : 0;   /* a draw site used more uniforms than a tape record holds */
}

/* Timing helper for the CPU baseline: sweeps `nblocks_run` blocks starting at
 * `first_block`, `reps` times, for chain 0, without the hyper-parameter draws. */
int oracle_run_blocks(oracle_ctx *o, int32_t first_block, int32_t nblocks_run, int32_t reps)
{
    if (!o || !o->have_chain) return SODAGPU_E_STATE;
    if (first_block < 0 || nblocks_run < 1 || first_block + nblocks_run > o->nb) return SODAGPU_E_ARG;
    chain_t *c = &o->ch[0];
    const int nm = o->nmix, ng = o->ngroup;
    for (int t = 0; t < reps; ++t) {
        c->rep++;
        if (o->method != SODAGPU_BAYES_A) {
            for (int i = 0; i < ng; ++i)
                for (int j = 0; j < nm; ++j) c->log_p[IDX2(i, j, ng)] = log(c->p[IDX2(i, j, ng)]);
            for (int j = 1; j < nm; ++j) c->vare_gp[j] = c->vare / c->gp[j];
        }
        for (int b = first_block; b < first_block + nblocks_run; ++b) sweep_block(o, c, 0, b, c->rep);
    }
    return 0;
}

/* Timing helper: puts chain 0 in the sparse state of a settled BayesC-type
 * chain — a random fraction `incl` of SNPs in class 2 (with g = 0, so the
 * residuals stay consistent) and pi = (1-incl, incl). */
int oracle_set_sparse_state(oracle_ctx *o, double incl, int64_t seed)
{
    if (!o || !o->have_chain) return SODAGPU_E_STATE;
    if (o->method == SODAGPU_BAYES_A || o->method == SODAGPU_BAYES_B) return SODAGPU_E_ARG;
    chain_t *c = &o->ch[0];
    xo_state st;
    xo_streams(seed, 1, &st);
    for (int j = 0; j < o->p; ++j) c->cls[j] = u64_to_unit(xo_next(&st)) < incl ? 2 : 1;
    for (int i = 0; i < o->ngroup; ++i) {
        c->p[IDX2(i, 0, o->ngroup)] = 1.0 - incl;
        for (int k = 1; k < o->nmix; ++k) c->p[IDX2(i, k, o->ngroup)] = incl / (o->nmix - 1);
        for (int k = 0; k < o->nmix; ++k)
            c->log_p[IDX2(i, k, o->ngroup)] = log(c->p[IDX2(i, k, o->ngroup)]);
    }
    return 0;
}

int oracle_get_state(oracle_ctx *o, int32_t chain, double *g, int32_t *cls, double *vara_s,
                     double *yadj, double *yaadj, double *scalars)
{
    if (!o || !o->have_chain) return SODAGPU_E_STATE;
    if (chain < 0 || chain >= o->nchain) return SODAGPU_E_ARG;
    chain_t *c = &o->ch[chain];
    if (g) memcpy(g, c->g, sizeof(double) * o->p);
    if (cls) memcpy(cls, c->cls, sizeof(int32_t) * o->p);
    if (vara_s) memcpy(vara_s, c->vara_s, sizeof(double) * o->p);
    if (yadj) memcpy(yadj, c->r, sizeof(double) * o->n);
    if (yaadj) memcpy(yaadj, c->ra, sizeof(double) * o->bs);
    if (scalars) {
        scalars[0] = c->mu;
        scalars[1] = c->vare;
        scalars[2] = c->vara;
        scalars[3] = c->included;
    }
    return 0;
}

/* Posterior means (models.f90:575-594) */
int oracle_get_results(oracle_ctx *o, int32_t chain, double *gstore, double *indiststore,
                       double *vara_sstore, double *scalars, double *snpstore,
                       double *pstore, double *varstore)
{
    if (!o || !o->have_chain) return SODAGPU_E_STATE;
    if (chain < 0 || chain >= o->nchain) return SODAGPU_E_ARG;
    chain_t *c = &o->ch[chain];
    const int p = o->p, nm = o->nmix, ng = o->ngroup;
    const double cnt = (double)c->counter;
    if (gstore)
        for (int j = 0; j < p; ++j) gstore[j] = c->gstore[j] / cnt;
    if (indiststore)
        for (size_t t = 0; t < (size_t)p * nm; ++t) indiststore[t] = c->indiststore[t] / cnt;
    if (vara_sstore)
        for (int j = 0; j < p; ++j) vara_sstore[j] = c->vara_sstore[j] / cnt;
    if (scalars) {
        scalars[0] = c->mu_store / cnt;
        scalars[1] = c->vare_store / cnt;
        scalars[2] = c->vara_store / cnt;
        scalars[3] = c->included_store / cnt;
    }
    for (int t = 0; t < ng * nm; ++t) {
        if (snpstore) snpstore[t] = c->snpstore[t] / cnt;
        if (pstore) pstore[t] = c->pstore[t] / cnt;
        if (varstore) varstore[t] = c->varstore[t] / cnt;
    }
    return 0;
}

/* compute_dgv (utilities.f90:616-622) */
int oracle_compute_dgv(oracle_ctx *o, double mu, const double *effects, double *pred)
{
    if (!o || !o->have_geno || !effects || !pred) return SODAGPU_E_ARG;
    const int n = o->n, p = o->p;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        double d = 0.0;
        for (int j = 0; j < p; ++j) d = d + o->X[IDX2(i, j, n)] * effects[j];
        pred[i] = mu + d;
    }
    return 0;
}

/* Prediction: xscale with frequencies from a .frq file (utilities.f90:540-553)
 * followed by compute_dgv. */
int oracle_predict(int32_t nind, int32_t nloci, const int8_t *codes, const double *freq,
                   double mu, const double *effects, double *pred)
{
    if (nind < 1 || nloci < 1 || !codes || !freq || !effects || !pred) return SODAGPU_E_ARG;
    const double eps = 2.220446049250313e-16;
    for (int i = 0; i < nind; ++i) pred[i] = 0.0;
    double *acc = (double *)calloc(nind, sizeof(double));
    if (!acc) return SODAGPU_E_NOMEM;
    /* row-wise dot products in SNP order, as dot_product(X(i,:), gstore) */
    for (int j = 0; j < nloci; ++j) {
        double p = freq[j];
        int mono = (p < eps || (1.0 - p) < eps);
        double sd = mono ? 1.0 : sqrt(2.0 * p * (1.0 - p));
        for (int i = 0; i < nind; ++i) {
            double x = mono ? 0.0 : ((double)codes[IDX2(i, j, nind)] - 2.0 * p) / sd;
            acc[i] = acc[i] + x * effects[j];
        }
    }
    for (int i = 0; i < nind; ++i) pred[i] = mu + acc[i];
    free(acc);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Unit-test exports                                                        */
/* ------------------------------------------------------------------------ */
int oracle_ref_uniforms(int64_t seed, int32_t stream, int32_t count, double *out)
{
    if (stream < 0 || count < 0 || !out) return SODAGPU_E_ARG;
    xo_state *st = (xo_state *)malloc(sizeof(xo_state) * (stream + 1));
    if (!st) return SODAGPU_E_NOMEM;
    xo_streams(seed, stream + 1, st);
    for (int i = 0; i < count; ++i) out[i] = u64_to_unit(xo_next(&st[stream]));
    free(st);
    return 0;
}

int oracle_counter_uniforms(int64_t seed, int32_t chain, int32_t iter, int32_t slot,
                            int32_t purpose, int32_t count, double *out)
{
    if (count < 0 || !out) return SODAGPU_E_ARG;
    ctr_rng c;
    ctr_init(&c, seed, chain, iter, slot, purpose);
    for (int i = 0; i < count; ++i) out[i] = u64_to_unit(ctr_next(&c));
    return 0;
}

/* dist: 0 uniform, 1 normal(a,b), 2 gamma(a,b), 3 scaled-inv-chi2(a,b),
 *       4 dirichlet with a classes of prior b (out holds count*a values). */
int oracle_sample(int32_t dist, int32_t mode, int64_t seed, int32_t count, double a, double b,
                  double *out)
{
    if (count < 0 || !out) return SODAGPU_E_ARG;
    xo_state st;
    xo_streams(seed, 1, &st);
    rng_t R;
    R.mode = mode;
    R.tmode = 0;
    R.xo = &st;
    ctr_init(&R.c, seed, 0, 0, 0, 0);
    for (int i = 0; i < count; ++i) {
        switch (dist) {
        case 0: out[i] = rng_u(&R); break;
        case 1: out[i] = rnorm(a, b, &R); break;
        case 2: out[i] = rgamma_(a, b, &R); break;
        case 3: out[i] = rscinvchi2(a, b, &R); break;
        case 4: {
            int k = (int)a;
            double irx[SODAGPU_MAXDIST];
            if (k < 1 || k > SODAGPU_MAXDIST) return SODAGPU_E_ARG;
            for (int j = 0; j < k; ++j) irx[j] = b;
            rdirichlet(k, irx, out + (size_t)i * k, &R);
            break;
        }
        default: return SODAGPU_E_ARG;
        }
    }
    return 0;
}
