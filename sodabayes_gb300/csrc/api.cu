// api.cu — the C ABI of libsodagpu.so (declared in include/sodagpu.h).
//
// Host-side orchestration only: every array operation runs in the kernels of
// zbuild.cu and sweep.cu.  The host computes block bounds, prefix sums of the
// factor column lengths, the top eigenvalue of the small Lanczos tridiagonal
// matrices, and formats results.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/sodagpu.h"
#include "state.cuh"
#include "sweep.cuh"
#include "zbuild.cuh"

using namespace soda;

namespace {

// cuTensorMapEncodeTiled from the driver, looked up once through the runtime
// (no link-time dependency on libcuda).
PFN_cuTensorMapEncodeTiled_v12000 tmap_encoder()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
        cudaGetLastError();
    });
    return fn;
}

// 2-D tile map over a row-major array of d1 rows of d0 elements (row stride
// `stride` bytes), loaded in boxes of b0 x b1 elements.
CUresult make_tmap_2d(CUtensorMap *m, CUtensorMapDataType dt, const void *base, uint64_t d0, uint64_t d1,
                      uint64_t stride, uint32_t b0, uint32_t b1, CUtensorMapSwizzle sw)
{
    PFN_cuTensorMapEncodeTiled_v12000 fn = tmap_encoder();
    if (!fn) return CUDA_ERROR_NOT_SUPPORTED;
    const cuuint64_t dims[2] = {d0, d1};
    const cuuint64_t strides[1] = {stride};
    const cuuint32_t box[2] = {b0, b1};
    const cuuint32_t es[2] = {1, 1};
    return fn(m, dt, 2, const_cast<void *>(base), dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, sw,
              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
}

thread_local std::string g_last_error;

int fail(int code, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

#define CUDA_TRY(expr)                                                                     \
    do {                                                                                   \
        cudaError_t _e = (expr);                                                           \
        if (_e != cudaSuccess)                                                             \
            return fail(SODAGPU_E_CUDA, "%s failed: %s (%s:%d)", #expr, cudaGetErrorString(_e), \
                        __FILE__, __LINE__);                                               \
    } while (0)

inline size_t round_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Largest eigenvalue of the symmetric tridiagonal matrix (a[0..m), b[0..m-1))
// by Sturm-sequence bisection.
double tridiag_max_eig(const double *a, const double *b, int m)
{
    double lo = a[0], hi = a[0];
    for (int i = 0; i < m; ++i) {
        const double r = (i > 0 ? fabs(b[i - 1]) : 0.0) + (i + 1 < m ? fabs(b[i]) : 0.0);
        lo = std::min(lo, a[i] - r);
        hi = std::max(hi, a[i] + r);
    }
    auto count_below = [&](double x) {
        int cnt = 0;
        double q = a[0] - x;
        if (q < 0) ++cnt;
        for (int i = 1; i < m; ++i) {
            const double qq = q != 0.0 ? q : 1e-300;
            q = a[i] - x - b[i - 1] * b[i - 1] / qq;
            if (q < 0) ++cnt;
        }
        return cnt;
    };
    for (int it = 0; it < 200; ++it) {
        const double mid = 0.5 * (lo + hi);
        if (mid <= lo || mid >= hi) break;
        if (count_below(mid) == m) hi = mid;
        else lo = mid;
    }
    return hi;
}

}  // namespace

struct sodagpu_ctx {
    sodagpu_config cfg;
    int dev = 0, sm_count = 0;
    cudaStream_t st = nullptr;
    int n = 0, p = 0, bs = 0, nb = 0, bt = 0, C = 0, ldx = 0, ldr = 0, nr_ctas = 0;
    int nskipped = 0, naind = 0, nsplit = 1;
    double d_offset = 0.0;
    bool have_geno = false, have_pheno = false, have_z = false, have_chain = false;
    bool regular = false;   // regular_bayes (models.f90:607-962): no subsets, no Z
    std::vector<void *> allocs;
    std::vector<int32_t> blk_sizes, h_blk_ls;
    // device
    int8_t *Gsnp = nullptr, *G = nullptr;
    float *X32 = nullptr;
    double *xv = nullptr, *freq = nullptr, *y = nullptr;
    int64_t *uoff = nullptr;
    int32_t *ulen = nullptr;
    double *U64 = nullptr;
    float *U32 = nullptr;
    __nv_bfloat16 *Uhi = nullptr, *Ulo = nullptr;
    double *xxd = nullptr, *xpx = nullptr;
    int32_t *perm = nullptr, *pos_of = nullptr, *iskipped = nullptr, *grp = nullptr, *blk_ls = nullptr;
    uint8_t *skip = nullptr;
    float *ra32 = nullptr, *xv32 = nullptr, *delta32 = nullptr;
    int32_t *blk_pd = nullptr;
    int ldra = 0;
    double *r = nullptr, *ra = nullptr, *g = nullptr, *vara_s = nullptr, *gstore = nullptr,
           *vara_sstore = nullptr;
    float *r32 = nullptr;
    int32_t *cls = nullptr;
    uint32_t *indist = nullptr;
    ChainScal *scal = nullptr;
    RunCtl *ctl = nullptr;
    double *delta = nullptr, *rpart = nullptr, *rsum = nullptr, *statpart = nullptr, *recal_part = nullptr,
           *upart = nullptr, *rpx = nullptr, *rpu = nullptr;
    int32_t *cntpart = nullptr, *ucount = nullptr;
    uint8_t *nzflag = nullptr;
    int tc = 0, ldd = 0;                 // tensor-core sweep
    uint16_t *dsplit = nullptr;
    uint16_t *rsp = nullptr, *rasp = nullptr, *usp = nullptr;   // tensor-core rhs operands
    int ldu = 0;
    bool usp_ready = false;
    double *k0part = nullptr;
    float *vpart = nullptr;              // residual-update partial sums
    unsigned long long *ugrid = nullptr; // grid-barrier counter of the residual update
    TcMaps maps{};
    std::vector<int32_t> h_rtab;         // work table of the tensor-core rhs
    int32_t *rtab = nullptr;
    std::vector<int32_t> h_qoff;         // first code block of each subset (tiled codes)
    int32_t *qoff = nullptr;
    uint8_t *Gt = nullptr;               // packed codes: [blocks][TC_PACKED_BLOCK], position-major (rhs)
    uint8_t *Gu = nullptr;               // the same blocks individual-major (residual update)
    long long ncblk = 0;
    sodagpu_trace_row *trace = nullptr;
    int trace_cap = 0;
    // staging of sodagpu_set_state and the output of sodagpu_subset_rhs
    double *st_g = nullptr, *st_vs = nullptr, *st_r = nullptr, *st_ra = nullptr, *st_pi = nullptr;
    int32_t *st_cls = nullptr;
    double *rhs_buf = nullptr;
    double *tape = nullptr;              // injected-draw tape (sodagpu_set_tape)
    int tape_reps = 0;
    cudaGraphExec_t graph = nullptr;
    double t_build = 0.0, t_run = 0.0, t_run_dev_ms = 0.0;
    Dev D;

    template <class T>
    int alloc(T **ptr, size_t count, bool zero = true)
    {
        void *p_ = nullptr;
        const size_t bytes = std::max<size_t>(count, 1) * sizeof(T);
        cudaError_t e = cudaMalloc(&p_, bytes);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return fail(SODAGPU_E_NOMEM, "cudaMalloc of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
        }
        if (zero) {
            e = cudaMemsetAsync(p_, 0, bytes, st);
            if (e != cudaSuccess) return fail(SODAGPU_E_CUDA, "cudaMemset failed: %s", cudaGetErrorString(e));
        }
        allocs.push_back(p_);
        *ptr = (T *)p_;
        return 0;
    }
    void release(void *p_)
    {
        if (!p_) return;
        auto it = std::find(allocs.begin(), allocs.end(), p_);
        if (it != allocs.end()) allocs.erase(it);
        cudaFree(p_);
    }
};

#define TRY(expr)                 \
    do {                          \
        int _rc = (expr);         \
        if (_rc != 0) return _rc; \
    } while (0)

extern "C" {

int sodagpu_abi_version(void) { return SODAGPU_ABI_VERSION; }

const char *sodagpu_errstr(int code)
{
    switch (code) {
    case SODAGPU_OK: return "ok";
    case SODAGPU_E_ARG: return "invalid argument";
    case SODAGPU_E_STATE: return "call out of order";
    case SODAGPU_E_NOMEM: return "out of memory";
    case SODAGPU_E_CUDA: return "CUDA error";
    case SODAGPU_E_NOTPSD: return "d*I - X'X is not positive semidefinite";
    case SODAGPU_E_TIMEOUT: return "device wait timed out";
    case SODAGPU_E_NODEVICE: return "no usable CUDA device";
    case SODAGPU_E_UNSUPPORTED: return "unsupported option combination";
    default: return "unknown error";
    }
}

const char *sodagpu_last_error(void) { return g_last_error.c_str(); }

int sodagpu_block_layout(int32_t nloci, int32_t nthreads, int32_t blocksize_opt, int32_t nblocks_opt,
                         int32_t *blocksize, int32_t *nblocks, int32_t *blockt)
{
    if (nloci < 1 || !blocksize || !nblocks || !blockt) return fail(SODAGPU_E_ARG, "bad block layout arguments");
    int32_t bsz, nbk, bt;
    if (blocksize_opt > 0) {            // soda.f90:407-409
        bsz = blocksize_opt;
        nbk = (int32_t)ceil((double)nloci / bsz);
        bt = nbk;
    } else if (nblocks_opt > 0) {       // soda.f90:410-412
        nbk = nblocks_opt;
        bsz = (int32_t)ceil((double)nloci / nbk);
        bt = nloci - (bsz - 1) * nbk;
    } else {                            // soda.f90:413-416
        bsz = nthreads;
        nbk = (int32_t)ceil((double)nloci / (bsz > 0 ? bsz : 1));
        bt = nbk;
    }
    *blocksize = bsz;
    *nblocks = nbk;
    *blockt = bt;
    return bsz <= 1 ? 1 : 0;           // soda.f90:418-421
}

int sodagpu_create(const sodagpu_config *cfg, sodagpu_ctx **out)
{
    if (!cfg || !out) return fail(SODAGPU_E_ARG, "null argument");
    *out = nullptr;
    if (cfg->nind < 2 || cfg->nloci < 1) return fail(SODAGPU_E_ARG, "nind must be >= 2 and nloci >= 1");
    if (cfg->method < 1 || cfg->method > 6) return fail(SODAGPU_E_ARG, "method %d out of range", cfg->method);
    if (cfg->nmix < 1 || cfg->nmix > SODAGPU_MAXDIST) return fail(SODAGPU_E_ARG, "nmix out of range");
    if (cfg->ngroup < 1 || cfg->ngroup > SODAGPU_MAXGRP) return fail(SODAGPU_E_ARG, "ngroup out of range");
    if (cfg->method == SODAGPU_BAYES_A && cfg->nmix != 1) return fail(SODAGPU_E_ARG, "BayesA needs nmix=1");
    if ((cfg->method >= SODAGPU_BAYES_B && cfg->method <= SODAGPU_BAYES_CPI) && cfg->nmix != 2)
        return fail(SODAGPU_E_ARG, "BayesB/C/Cpi need nmix=2");
    if (cfg->method != SODAGPU_BAYES_RC && cfg->ngroup != 1) return fail(SODAGPU_E_ARG, "ngroup>1 needs BayesRc");
    if (cfg->sampler != SODAGPU_SAMPLER_SODA && cfg->sampler != SODAGPU_SAMPLER_REGULAR)
        return fail(SODAGPU_E_ARG, "sampler %d out of range", cfg->sampler);
    const bool regular = cfg->sampler == SODAGPU_SAMPLER_REGULAR;
    if (!regular && (cfg->blocksize < 2 || cfg->nblocks < 1 || cfg->blockt < 0 || cfg->blockt > cfg->nblocks))
        return fail(SODAGPU_E_ARG, "invalid SODA block layout");
    if (cfg->thin < 1 || cfg->numit < 0 || cfg->burnin < 0) return fail(SODAGPU_E_ARG, "bad numit/burnin/thin");
    if (cfg->precision < 0 || cfg->precision > 2) return fail(SODAGPU_E_ARG, "precision out of range");
    if (cfg->chains < 1 || !sweep_chain_count_supported(cfg->chains))
        return fail(SODAGPU_E_UNSUPPORTED, "chains must be 1, 2, 4, 8 or 16");
    if (cfg->kernels != SODAGPU_KERNELS_AUTO && cfg->kernels != SODAGPU_KERNELS_CUDA_CORES)
        return fail(SODAGPU_E_ARG, "kernels %d out of range", cfg->kernels);
    for (int j = 1; j < cfg->nmix; ++j)
        if (cfg->method >= SODAGPU_BAYES_C && !(cfg->mix[j] > 0.0))
            return fail(SODAGPU_E_ARG, "mix[%d] must be > 0", j);
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(SODAGPU_E_NODEVICE, "no CUDA device visible");
    }
    sodagpu_ctx *c = new (std::nothrow) sodagpu_ctx();
    if (!c) return fail(SODAGPU_E_NOMEM, "host allocation failed");
    c->cfg = *cfg;
    cudaGetDevice(&c->dev);
    cudaDeviceProp prop;
    cudaGetDeviceProperties(&prop, c->dev);
    if (prop.major != 10 || prop.minor != 3) {
        delete c;
        return fail(SODAGPU_E_NODEVICE, "libsodagpu is built for sm_103a; device %d is sm_%d%d (%s)", c->dev,
                    prop.major, prop.minor, prop.name);
    }
    c->sm_count = prop.multiProcessorCount;
    if (cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking) != cudaSuccess) {
        delete c;
        return fail(SODAGPU_E_CUDA, "stream creation failed");
    }
    c->n = cfg->nind;
    c->p = cfg->nloci;
    // the regular sampler has no subsets: one nominal subset of all SNPs, a small scratch size
    c->regular = regular;
    c->bs = regular ? 8 : cfg->blocksize;
    c->nb = regular ? 1 : cfg->nblocks;
    c->bt = regular ? 1 : cfg->blockt;
    c->C = cfg->chains;
    c->ldx = (int)round_up((size_t)c->n, 128);
    c->ldr = c->ldx;
    c->nr_ctas = (c->n + ROW_TILE - 1) / ROW_TILE;
    // block bounds (models.f90:136-142), 0-based first positions
    c->h_blk_ls.resize(c->nb + 1);
    c->blk_sizes.resize(c->nb);
    for (int b = 0; b < c->nb && !regular; ++b) {
        const int blocki = b + 1;
        int ls, le;
        if (blocki <= c->bt) {
            ls = (blocki - 1) * c->bs + 1;
            le = std::min(ls + c->bs - 1, c->p);
        } else {
            ls = c->bs * c->bt + (blocki - c->bt - 1) * (c->bs - 1) + 1;
            le = std::min(ls + c->bs - 2, c->p);
        }
        if (le < ls) {
            sodagpu_destroy(c);
            return fail(SODAGPU_E_ARG, "empty SODA block %d", blocki);
        }
        c->h_blk_ls[b] = ls - 1;
        c->blk_sizes[b] = le - ls + 1;
    }
    if (regular) {
        c->h_blk_ls[0] = 0;
        c->blk_sizes[0] = c->p;
    }
    c->h_blk_ls[c->nb] = c->h_blk_ls[c->nb - 1] + c->blk_sizes[c->nb - 1];
    if (c->h_blk_ls[c->nb] != c->p) {
        sodagpu_destroy(c);
        return fail(SODAGPU_E_ARG, "blocks cover %d of %d SNPs", c->h_blk_ls[c->nb], c->p);
    }
    if (sweep_prepare(c->bs) != cudaSuccess) {
        sodagpu_destroy(c);
        return fail(SODAGPU_E_UNSUPPORTED, "blocksize %d too large", c->bs);
    }
    int rc = 0;
    rc = rc ? rc : c->alloc(&c->Gsnp, (size_t)c->p * c->ldx);
    rc = rc ? rc : c->alloc(&c->freq, c->p);
    rc = rc ? rc : c->alloc(&c->y, c->n);
    rc = rc ? rc : c->alloc(&c->grp, c->p);
    rc = rc ? rc : c->alloc(&c->blk_ls, c->nb + 1);
    rc = rc ? rc : c->alloc(&c->ctl, 1);
    if (rc) {
        sodagpu_destroy(c);
        return rc;
    }
    std::vector<int32_t> ones(c->p, 1);
    cudaMemcpyAsync(c->grp, ones.data(), sizeof(int32_t) * c->p, cudaMemcpyHostToDevice, c->st);
    cudaMemcpyAsync(c->blk_ls, c->h_blk_ls.data(), sizeof(int32_t) * (c->nb + 1), cudaMemcpyHostToDevice, c->st);
    if (cudaStreamSynchronize(c->st) != cudaSuccess) {
        sodagpu_destroy(c);
        return fail(SODAGPU_E_CUDA, "initial copies failed");
    }
    *out = c;
    return 0;
}

int sodagpu_load_genotypes(sodagpu_ctx *c, const void *geno, int32_t layout)
{
    if (!c || !geno) return fail(SODAGPU_E_ARG, "null argument");
    if (!c->Gsnp) return fail(SODAGPU_E_STATE, "genotypes already consumed by sodagpu_build_z");
    const bool on_dev = (layout & SODAGPU_GENO_DEVICE_PTR) != 0;
    const int kind = layout & 0xff;
    const cudaMemcpyKind mk = on_dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    if (kind == SODAGPU_GENO_CODES) {
        CUDA_TRY(cudaMemcpy2DAsync(c->Gsnp, c->ldx, geno, c->n, c->n, c->p, mk, c->st));
    } else if (kind == SODAGPU_GENO_BED) {
        const size_t rec = ((size_t)c->n + 3) / 4;
        uint8_t *tmp = nullptr;
        TRY(c->alloc(&tmp, rec * c->p, false));
        CUDA_TRY(cudaMemcpyAsync(tmp, geno, rec * c->p, mk, c->st));
        CUDA_TRY(zb_decode_bed(tmp, c->n, c->p, c->Gsnp, c->ldx, c->st));
        CUDA_TRY(cudaStreamSynchronize(c->st));
        c->release(tmp);
    } else {
        return fail(SODAGPU_E_ARG, "unknown genotype layout %d", layout);
    }
    int *bad = nullptr, h_bad = 0;
    TRY(c->alloc(&bad, 1));
    CUDA_TRY(zb_freq(c->Gsnp, c->n, c->p, c->ldx, c->freq, bad, c->st));
    CUDA_TRY(cudaMemcpyAsync(&h_bad, bad, sizeof(int), cudaMemcpyDeviceToHost, c->st));
    CUDA_TRY(cudaStreamSynchronize(c->st));
    c->release(bad);
    if (h_bad) return fail(SODAGPU_E_ARG, "%d genotype codes outside 0..2", h_bad);
    c->have_geno = true;
    return 0;
}

int sodagpu_get_freq(sodagpu_ctx *c, double *freq)
{
    if (!c || !freq) return fail(SODAGPU_E_ARG, "null argument");
    if (!c->have_geno) return fail(SODAGPU_E_STATE, "no genotypes loaded");
    CUDA_TRY(cudaMemcpyAsync(freq, c->freq, sizeof(double) * c->p, cudaMemcpyDeviceToHost, c->st));
    CUDA_TRY(cudaStreamSynchronize(c->st));
    return 0;
}

int sodagpu_load_pheno(sodagpu_ctx *c, const double *y)
{
    if (!c || !y) return fail(SODAGPU_E_ARG, "null argument");
    for (int i = 0; i < c->n; ++i)
        if (!std::isfinite(y[i])) return fail(SODAGPU_E_ARG, "phenotype %d is not finite", i + 1);
    CUDA_TRY(cudaMemcpyAsync(c->y, y, sizeof(double) * c->n, cudaMemcpyHostToDevice, c->st));
    CUDA_TRY(cudaStreamSynchronize(c->st));
    c->have_pheno = true;
    return 0;
}

int sodagpu_set_groups(sodagpu_ctx *c, const int32_t *group)
{
    if (!c || !group) return fail(SODAGPU_E_ARG, "null argument");
    for (int j = 0; j < c->p; ++j)
        if (group[j] < 1 || group[j] > c->cfg.ngroup)
            return fail(SODAGPU_E_ARG, "group of SNP %d is %d, outside 1..%d", j + 1, group[j], c->cfg.ngroup);
    CUDA_TRY(cudaMemcpyAsync(c->grp, group, sizeof(int32_t) * c->p, cudaMemcpyHostToDevice, c->st));
    CUDA_TRY(cudaStreamSynchronize(c->st));
    return 0;
}

int sodagpu_set_d_offset(sodagpu_ctx *c, double delta)
{
    if (!c) return fail(SODAGPU_E_ARG, "null argument");
    c->d_offset = delta;
    return 0;
}

}  // extern "C"

namespace {

// The regular sampler's set-up in place of the Z build: genotypes in SNP order
// (permvec(i) = i, models.f90:675-678), every SNP drawn single-site in order by
// k_skipped, no augmented data.
int regular_layout(sodagpu_ctx *c, int32_t *nskipped_out, std::chrono::steady_clock::time_point t0)
{
    const int p = c->p;
    std::vector<int32_t> h_id(p);
    for (int k = 0; k < p; ++k) h_id[k] = k;
    TRY(c->alloc(&c->perm, p, false));
    TRY(c->alloc(&c->pos_of, p, false));
    TRY(c->alloc(&c->G, (size_t)p * c->ldx, false));
    TRY(c->alloc(&c->xv, (size_t)p * 4, false));
    TRY(c->alloc(&c->xxd, c->nb));
    TRY(c->alloc(&c->ulen, p));
    TRY(c->alloc(&c->uoff, p + 1));
    TRY(c->alloc(&c->skip, p));
    TRY(c->alloc(&c->blk_pd, c->nb));
    TRY(c->alloc(&c->U64, 1));
    TRY(c->alloc(&c->U32, 1));
    TRY(c->alloc(&c->iskipped, p, false));
    TRY(c->alloc(&c->xpx, p));
    CUDA_TRY(cudaMemcpyAsync(c->perm, h_id.data(), sizeof(int32_t) * p, cudaMemcpyHostToDevice, c->st));
    CUDA_TRY(cudaMemcpyAsync(c->pos_of, h_id.data(), sizeof(int32_t) * p, cudaMemcpyHostToDevice, c->st));
    CUDA_TRY(cudaMemcpyAsync(c->iskipped, h_id.data(), sizeof(int32_t) * p, cudaMemcpyHostToDevice, c->st));
    CUDA_TRY(zb_gather(c->Gsnp, c->G, c->perm, p, c->ldx, c->st));
    CUDA_TRY(zb_xv(c->freq, c->perm, p, c->xv, c->st));
    TRY(c->alloc(&c->xv32, (size_t)p * 4, false));
    CUDA_TRY(zb_xv32(c->xv, p, c->xv32, c->st));
    CUDA_TRY(cudaStreamSynchronize(c->st));
    c->release(c->Gsnp);
    c->Gsnp = nullptr;
    c->nskipped = p;
    c->naind = 0;
    c->have_z = true;
    if (nskipped_out) *nskipped_out = 0;
    c->t_build = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return 0;
}

}  // namespace

extern "C" {

int sodagpu_build_z(sodagpu_ctx *c, const int32_t *permvec, int32_t *nskipped_out)
{
    if (!c) return fail(SODAGPU_E_ARG, "null argument");
    if (!c->have_geno || !c->Gsnp) return fail(SODAGPU_E_STATE, "load genotypes before sodagpu_build_z");
    if (c->have_z) return fail(SODAGPU_E_STATE, "sodagpu_build_z already ran on this context");
    const auto t0 = std::chrono::steady_clock::now();
    if (c->regular) return regular_layout(c, nskipped_out, t0);
    const int p = c->p, n = c->n, bs = c->bs, nb = c->nb;
    std::vector<int32_t> h_perm(p), h_pos(p, -1);
    for (int k = 0; k < p; ++k) {
        const int v = permvec ? permvec[k] - 1 : k;
        if (v < 0 || v >= p || h_pos[v] != -1) return fail(SODAGPU_E_ARG, "permvec is not a permutation of 1..nloci");
        h_perm[k] = v;
        h_pos[v] = k;
    }
    TRY(c->alloc(&c->perm, p, false));
    TRY(c->alloc(&c->pos_of, p, false));
    TRY(c->alloc(&c->G, (size_t)p * c->ldx, false));
    TRY(c->alloc(&c->xv, (size_t)p * 4, false));
    TRY(c->alloc(&c->xxd, nb));
    TRY(c->alloc(&c->ulen, p));
    TRY(c->alloc(&c->uoff, p + 1));
    TRY(c->alloc(&c->skip, p));
    CUDA_TRY(cudaMemcpyAsync(c->perm, h_perm.data(), sizeof(int32_t) * p, cudaMemcpyHostToDevice, c->st));
    CUDA_TRY(cudaMemcpyAsync(c->pos_of, h_pos.data(), sizeof(int32_t) * p, cudaMemcpyHostToDevice, c->st));
    CUDA_TRY(zb_gather(c->Gsnp, c->G, c->perm, p, c->ldx, c->st));
    CUDA_TRY(zb_xv(c->freq, c->perm, p, c->xv, c->st));
    TRY(c->alloc(&c->xv32, (size_t)p * 4, false));
    CUDA_TRY(zb_xv32(c->xv, p, c->xv32, c->st));
    CUDA_TRY(cudaStreamSynchronize(c->st));
    c->release(c->Gsnp);
    c->Gsnp = nullptr;
    if (c->cfg.precision == SODAGPU_FP32) {
        TRY(c->alloc(&c->X32, (size_t)p * c->ldx, false));
        CUDA_TRY(zb_x32(c->G, c->xv, c->X32, n, p, c->ldx, c->st));
    }
    // FP64 work matrices of every subset
    std::vector<int64_t> wofs(nb);
    int64_t wtot = 0;
    int maxN = 0;
    for (int b = 0; b < nb; ++b) {
        wofs[b] = wtot;
        wtot += (int64_t)c->blk_sizes[b] * c->blk_sizes[b];
        maxN = std::max(maxN, c->blk_sizes[b]);
    }
    double *W = nullptr;
    int64_t *d_wofs = nullptr;
    TRY(c->alloc(&W, (size_t)wtot, false));
    TRY(c->alloc(&d_wofs, nb, false));
    CUDA_TRY(cudaMemcpyAsync(d_wofs, wofs.data(), sizeof(int64_t) * nb, cudaMemcpyHostToDevice, c->st));
    const int BATCH = std::min(nb, 64);
    const int mmax = std::min(maxN, 400);
    CUDA_TRY(zb_lz_prepare(maxN, mmax));
    double *V = nullptr, *wvec = nullptr, *alpha = nullptr, *beta = nullptr;
    int64_t *d_vofs = nullptr;
    int32_t *d_batch = nullptr, *d_status = nullptr;
    uint8_t *d_done = nullptr;
    TRY(c->alloc(&V, (size_t)BATCH * mmax * maxN));
    TRY(c->alloc(&wvec, (size_t)BATCH * maxN));
    TRY(c->alloc(&alpha, (size_t)BATCH * mmax));
    TRY(c->alloc(&beta, (size_t)BATCH * mmax));
    TRY(c->alloc(&d_vofs, BATCH, false));
    TRY(c->alloc(&d_batch, BATCH, false));
    TRY(c->alloc(&d_status, nb));
    TRY(c->alloc(&d_done, BATCH));
    std::vector<int64_t> vofs(BATCH);
    for (int i = 0; i < BATCH; ++i) vofs[i] = (int64_t)i * mmax * maxN;
    CUDA_TRY(cudaMemcpyAsync(d_vofs, vofs.data(), sizeof(int64_t) * BATCH, cudaMemcpyHostToDevice, c->st));
    std::vector<double> h_xxd(nb), ha((size_t)BATCH * mmax), hb((size_t)BATCH * mmax);
    std::vector<int32_t> h_status(nb, 0);
    std::vector<int32_t> batch_ids;
    const float shift_f = 0.001f;   // soda.f90:485 adds a REAL literal
    for (int b0 = 0; b0 < nb; b0 += BATCH) {
        const int nbat = std::min(BATCH, nb - b0);
        batch_ids.resize(nbat);
        int bmax = 0;
        for (int i = 0; i < nbat; ++i) {
            batch_ids[i] = b0 + i;
            bmax = std::max(bmax, c->blk_sizes[b0 + i]);
        }
        CUDA_TRY(cudaMemcpyAsync(d_batch, batch_ids.data(), sizeof(int32_t) * nbat, cudaMemcpyHostToDevice, c->st));
        CUDA_TRY(zb_gram(c->G, c->ldx, c->blk_ls, d_batch, nbat, bmax, d_wofs, c->freq, c->perm, n, W, c->st));
        // Lanczos for lambda_max of each subset
        CUDA_TRY(cudaMemsetAsync(d_done, 0, BATCH, c->st));
        CUDA_TRY(cudaMemsetAsync(alpha, 0, sizeof(double) * BATCH * mmax, c->st));
        CUDA_TRY(cudaMemsetAsync(beta, 0, sizeof(double) * BATCH * mmax, c->st));
        CUDA_TRY(zb_lz_init(c->blk_ls, d_batch, nbat, d_vofs, V, (uint64_t)llabs(c->cfg.seed), c->st));
        std::vector<uint8_t> done(nbat, 0);
        std::vector<double> theta(nbat, 0.0), theta_prev(nbat, -1.0);
        std::vector<int> steps(nbat, 0);
        const int bmm = std::min(bmax, mmax);
        for (int j = 0; j < bmm; ++j) {
            CUDA_TRY(zb_lz_step(W, d_wofs, c->blk_ls, d_batch, nbat, bmax, d_vofs, V, wvec, maxN, alpha, beta, mmax,
                                j, d_done, c->st));
            const bool check = ((j + 1) % 8 == 0) || j + 1 == bmm;
            if (!check) continue;
            CUDA_TRY(cudaMemcpyAsync(ha.data(), alpha, sizeof(double) * nbat * mmax, cudaMemcpyDeviceToHost, c->st));
            CUDA_TRY(cudaMemcpyAsync(hb.data(), beta, sizeof(double) * nbat * mmax, cudaMemcpyDeviceToHost, c->st));
            CUDA_TRY(cudaStreamSynchronize(c->st));
            bool all = true;
            for (int i = 0; i < nbat; ++i) {
                if (done[i]) continue;
                const int Nb = c->blk_sizes[b0 + i];
                const int m = std::min(j + 1, Nb);
                const double *a = &ha[(size_t)i * mmax];
                const double *bb = &hb[(size_t)i * mmax];
                theta[i] = tridiag_max_eig(a, bb, m);
                steps[i] = m;
                const double scale = std::max(fabs(theta[i]), 1e-300);
                bool conv = false;
                if (m >= Nb) conv = true;   // full Krylov space: exact
                for (int t = 0; t < m && !conv; ++t)
                    if (bb[t] <= 1e-13 * scale) conv = true;   // invariant subspace
                if (!conv && theta_prev[i] >= 0.0 && fabs(theta[i] - theta_prev[i]) <= 1e-15 * scale) conv = true;
                theta_prev[i] = theta[i];
                if (conv) done[i] = 1;
                else all = false;
            }
            CUDA_TRY(cudaMemcpyAsync(d_done, done.data(), nbat, cudaMemcpyHostToDevice, c->st));
            if (all) break;
        }
        for (int i = 0; i < nbat; ++i)
            h_xxd[b0 + i] = fabs(theta[i]) + (double)shift_f + c->d_offset;
        CUDA_TRY(cudaMemcpyAsync(c->xxd + b0, &h_xxd[b0], sizeof(double) * nbat, cudaMemcpyHostToDevice, c->st));
        CUDA_TRY(zb_form_m(W, d_wofs, c->blk_ls, d_batch, nbat, c->xxd, c->st));
        CUDA_TRY(zb_cholesky(W, d_wofs, c->blk_ls, d_batch, nbat, bmax, d_status, c->st));
        CUDA_TRY(zb_pd_lengths(c->blk_ls, d_batch, nbat, d_status, c->ulen, c->skip, c->st));
        CUDA_TRY(cudaStreamSynchronize(c->st));
    }
    CUDA_TRY(cudaMemcpyAsync(h_status.data(), d_status, sizeof(int32_t) * nb, cudaMemcpyDeviceToHost, c->st));
    CUDA_TRY(cudaStreamSynchronize(c->st));
    // pivoted fallback for the subsets whose factorisation failed (soda.f90:492-510)
    std::vector<int32_t> h_iskipped;
    int naless = p;
    {
        double *M = nullptr, *work = nullptr;
        int32_t *piv = nullptr, *rank = nullptr, *pst = nullptr;
        bool any_fail = false;
        for (int b = 0; b < nb; ++b) any_fail |= h_status[b] != 0;
        if (any_fail) {
            TRY(c->alloc(&M, (size_t)maxN * maxN, false));
            TRY(c->alloc(&work, (size_t)2 * maxN));
            TRY(c->alloc(&piv, maxN));
            TRY(c->alloc(&rank, 1));
            TRY(c->alloc(&pst, 1));
        }
        std::vector<int32_t> hpiv(maxN);
        int nsk = 0;
        for (int b = 0; b < nb; ++b) {
            const int N = c->blk_sizes[b];
            if (h_status[b] != 0) {
                int32_t one = b;
                CUDA_TRY(cudaMemcpyAsync(d_batch, &one, sizeof(int32_t), cudaMemcpyHostToDevice, c->st));
                CUDA_TRY(zb_gram(c->G, c->ldx, c->blk_ls, d_batch, 1, N, d_wofs, c->freq, c->perm, n, W, c->st));
                CUDA_TRY(zb_form_m(W, d_wofs, c->blk_ls, d_batch, 1, c->xxd, c->st));
                CUDA_TRY(cudaMemcpyAsync(M, W + wofs[b], sizeof(double) * N * N, cudaMemcpyDeviceToDevice, c->st));
                CUDA_TRY(zb_psd_block(W + wofs[b], M, N, c->h_blk_ls[b], c->ulen, c->skip, piv, rank, pst, work, c->st));
                int32_t h_rank = 0, h_pst = 0;
                CUDA_TRY(cudaMemcpyAsync(&h_rank, rank, sizeof(int32_t), cudaMemcpyDeviceToHost, c->st));
                CUDA_TRY(cudaMemcpyAsync(&h_pst, pst, sizeof(int32_t), cudaMemcpyDeviceToHost, c->st));
                CUDA_TRY(cudaMemcpyAsync(hpiv.data(), piv, sizeof(int32_t) * N, cudaMemcpyDeviceToHost, c->st));
                CUDA_TRY(cudaStreamSynchronize(c->st));
                if (h_pst != 0) return fail(SODAGPU_E_NOTPSD, "subset %d: d*I - X'X is not positive semidefinite", b + 1);
                for (int j = h_rank; j < N; ++j) {
                    const int jj = hpiv[j] - 1;
                    h_iskipped.push_back(h_perm[c->h_blk_ls[b] + jj]);
                    ++nsk;
                }
            } else {
                naless = 0;
            }
            naless = std::min(naless, bs - N + nsk);
        }
        if (M) { c->release(M); c->release(work); c->release(piv); c->release(rank); c->release(pst); }
    }
    c->nskipped = (int)h_iskipped.size();
    c->naind = bs - naless;
    // ragged offsets and packing
    std::vector<int32_t> h_len(p);
    CUDA_TRY(cudaMemcpyAsync(h_len.data(), c->ulen, sizeof(int32_t) * p, cudaMemcpyDeviceToHost, c->st));
    CUDA_TRY(cudaStreamSynchronize(c->st));
    // columns of subset b spaced round_up(N_b, 8) apart: every column starts
    // 16-byte aligned (FP32) and rows ulen..N-1 stay zero
    std::vector<int64_t> h_off(p + 1);
    int64_t tot = 0;
    for (int b = 0; b < nb; ++b) {
        const int N = c->blk_sizes[b];
        const int64_t npad = (int64_t)round_up((size_t)N, 8);
        for (int jj = 0; jj < N; ++jj) h_off[c->h_blk_ls[b] + jj] = tot + jj * npad;
        tot += npad * N;
    }
    h_off[p] = tot;
    {
        std::vector<int32_t> pd(nb);
        for (int b = 0; b < nb; ++b) pd[b] = h_status[b] == 0;
        TRY(c->alloc(&c->blk_pd, nb, false));
        CUDA_TRY(cudaMemcpyAsync(c->blk_pd, pd.data(), sizeof(int32_t) * nb, cudaMemcpyHostToDevice, c->st));
    }
    CUDA_TRY(cudaMemcpyAsync(c->uoff, h_off.data(), sizeof(int64_t) * (p + 1), cudaMemcpyHostToDevice, c->st));
    TRY(c->alloc(&c->U64, (size_t)tot));
    if (c->cfg.precision != SODAGPU_FP64) TRY(c->alloc(&c->U32, (size_t)tot));
    for (int b0 = 0; b0 < nb; b0 += BATCH) {
        const int nbat = std::min(BATCH, nb - b0);
        batch_ids.resize(nbat);
        for (int i = 0; i < nbat; ++i) batch_ids[i] = b0 + i;
        CUDA_TRY(cudaMemcpyAsync(d_batch, batch_ids.data(), sizeof(int32_t) * nbat, cudaMemcpyHostToDevice, c->st));
        CUDA_TRY(zb_pack(W, d_wofs, c->blk_ls, d_batch, nbat, c->uoff, c->ulen, c->U64, c->U32, c->Uhi, c->Ulo, c->st));
        CUDA_TRY(cudaStreamSynchronize(c->st));
    }
    c->release(W);
    c->release(V);
    c->release(wvec);
    c->release(alpha);
    c->release(beta);
    c->release(d_vofs);
    c->release(d_batch);
    c->release(d_status);
    c->release(d_done);
    c->release(d_wofs);
    TRY(c->alloc(&c->iskipped, std::max(1, c->nskipped), false));
    TRY(c->alloc(&c->xpx, p));
    if (c->nskipped)
        CUDA_TRY(cudaMemcpyAsync(c->iskipped, h_iskipped.data(), sizeof(int32_t) * c->nskipped, cudaMemcpyHostToDevice,
                                 c->st));
    CUDA_TRY(cudaStreamSynchronize(c->st));
    c->have_z = true;
    if (nskipped_out) *nskipped_out = c->nskipped;
    c->t_build = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return 0;
}

}  // extern "C"

namespace {

__global__ void k_xpx(const int8_t *G, int ldx, const double *xv, const int32_t *pos_of, const int32_t *isk, int nsk,
                      int n, double *xpx)
{
    __shared__ double sh[32];
    for (int t = blockIdx.x; t < nsk; t += gridDim.x) {
        const int snp = isk[t], k = pos_of[snp];
        double s = 0.0;
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const double x = xv[(size_t)k * 4 + G[(size_t)k * ldx + i]];
            s += x * x;
        }
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
        __syncthreads();
        if (threadIdx.x == 0) {
            double tsum = 0.0;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tsum += sh[w];
            xpx[snp] = tsum;
        }
        __syncthreads();
    }
}

int build_dev(sodagpu_ctx *c)
{
    Dev &D = c->D;
    memset(&D, 0, sizeof D);
    D.n = c->n;
    D.p = c->p;
    D.bs = c->bs;
    D.nb = c->regular ? 0 : c->nb;   // the regular sampler's SNPs all run through k_skipped
    D.regular = c->regular ? 1 : 0;
    D.bt = c->bt;
    D.method = c->cfg.method;
    D.nmix = c->cfg.nmix;
    D.ngroup = c->cfg.ngroup;
    D.chains = c->C;
    D.precision = c->cfg.precision;
    D.ldx = c->ldx;
    D.ldr = c->ldr;
    D.nskipped = c->nskipped;
    D.naind = c->naind;
    D.nr_ctas = c->nr_ctas;
    D.recal = c->cfg.recal_every;
    D.burnin = c->cfg.burnin;
    D.thin = c->cfg.thin;
    D.seed = (uint64_t)llabs(c->cfg.seed);
    D.pizero = c->cfg.pizero;
    D.scale_ve = c->cfg.scale_ve;
    D.df_va = c->cfg.df_va;
    D.df_ve = c->cfg.df_ve;
    for (int j = 0; j < MAXDIST; ++j) {
        D.mix[j] = c->cfg.mix[j];
        D.alpha[j] = c->cfg.alpha[j];
    }
    D.G = c->G;
    D.X32 = c->X32;
    D.xv = c->xv;
    D.xv32 = c->xv32;
    D.delta32 = c->delta32;
    D.y = c->y;
    D.uoff = c->uoff;
    D.ulen = c->ulen;
    D.U64 = c->U64;
    D.U32 = c->U32;
    D.Uhi = c->Uhi;
    D.Ulo = c->Ulo;
    D.xxd = c->xxd;
    D.xpx = c->xpx;
    D.perm = c->perm;
    D.pos_of = c->pos_of;
    D.skip = c->skip;
    D.iskipped = c->iskipped;
    D.grp = c->grp;
    D.blk_ls = c->blk_ls;
    D.r = c->r;
    D.r32 = c->r32;
    D.ra = c->ra;
    D.ra32 = c->ra32;
    D.ldra = c->ldra;
    D.blk_pd = c->blk_pd;
    D.g = c->g;
    D.cls = c->cls;
    D.vara_s = c->vara_s;
    D.gstore = c->gstore;
    D.vara_sstore = c->vara_sstore;
    D.indist = c->indist;
    D.scal = c->scal;
    D.ctl = c->ctl;
    D.delta = c->delta;
    D.nzflag = c->nzflag;
    D.rpart = c->rpart;
    D.rsum = c->rsum;
    D.statpart = c->statpart;
    D.cntpart = c->cntpart;
    D.recal_part = c->recal_part;
    D.rpx = c->rpx;
    D.rpu = c->rpu;
    D.tc = c->tc;
    D.ldd = c->ldd;
    D.dsplit = c->dsplit;
    D.k0part = c->k0part;
    D.vpart = c->vpart;
    D.ugrid = c->ugrid;
    D.gpk = c->Gt;
    D.gpu = c->Gu;
    D.nvt = sweep_tc_update_tiles(c->n);
    D.rtab = c->rtab;
    D.qoff = c->qoff;
    D.tstride = sweep_tc_table_stride(c->bs);
    D.rsp = c->rsp;
    D.rasp = c->rasp;
    D.usp = c->usp;
    D.ldu = c->ldu;
    D.tape = c->tape;
    D.tape_reps = c->tape_reps;
    D.tape_snp0 = 3 + c->cfg.ngroup + c->cfg.blocksize;
    D.tape_sites = D.tape_snp0 + c->p;
    return 0;
}

}  // namespace

extern "C" {

int sodagpu_set_tape(sodagpu_ctx *c, const double *draws, size_t n)
{
    if (!c) return fail(SODAGPU_E_ARG, "null argument");
    if (c->have_chain) return fail(SODAGPU_E_STATE, "set the tape before sodagpu_init_chains");
    if (c->C != 1) return fail(SODAGPU_E_UNSUPPORTED, "an injected-draw tape drives one chain");
    if (c->tape) {
        c->release(c->tape);
        c->tape = nullptr;
        c->tape_reps = 0;
    }
    if (!draws && n == 0) return 0;
    const size_t rec = (size_t)(3 + c->cfg.ngroup + c->cfg.blocksize + c->p) * SODAGPU_TAPE_W;
    if (!draws || n < rec || n % rec != 0)
        return fail(SODAGPU_E_ARG, "tape length %zu is not a positive multiple of %zu (sites x SODAGPU_TAPE_W)", n, rec);
    if (n / rec > (size_t)INT32_MAX) return fail(SODAGPU_E_ARG, "tape too long");
    TRY(c->alloc(&c->tape, n, false));
    CUDA_TRY(cudaMemcpyAsync(c->tape, draws, sizeof(double) * n, cudaMemcpyHostToDevice, c->st));
    CUDA_TRY(cudaStreamSynchronize(c->st));
    c->tape_reps = (int)(n / rec);
    return 0;
}

int sodagpu_init_chains(sodagpu_ctx *c)
{
    if (!c) return fail(SODAGPU_E_ARG, "null argument");
    if (!c->have_z || !c->have_pheno) return fail(SODAGPU_E_STATE, "build Z and load phenotypes first");
    const int C = c->C, p = c->p, nm = c->cfg.nmix, ngm = c->cfg.ngroup * nm;
    if (!c->r) {
        TRY(c->alloc(&c->r, (size_t)C * c->ldr));
        TRY(c->alloc(&c->r32, (size_t)C * c->ldr));
        c->ldra = (int)round_up((size_t)c->bs, 8);
        TRY(c->alloc(&c->ra, (size_t)C * c->ldra));
        TRY(c->alloc(&c->ra32, (size_t)C * c->ldra));
        TRY(c->alloc(&c->g, (size_t)C * p));
        TRY(c->alloc(&c->cls, (size_t)C * p));
        TRY(c->alloc(&c->vara_s, (size_t)C * p));
        TRY(c->alloc(&c->gstore, (size_t)C * p));
        TRY(c->alloc(&c->vara_sstore, (size_t)C * p));
        TRY(c->alloc(&c->indist, (size_t)C * p * nm));
        TRY(c->alloc(&c->scal, C));
        TRY(c->alloc(&c->delta, (size_t)C * c->bs));
        TRY(c->alloc(&c->delta32, (size_t)C * c->bs));
        TRY(c->alloc(&c->nzflag, c->bs));
        TRY(c->alloc(&c->rpart, (size_t)C * c->nr_ctas));
        TRY(c->alloc(&c->rsum, (size_t)C * c->nr_ctas));
        TRY(c->alloc(&c->statpart, (size_t)C * NSTAT * ngm));
        TRY(c->alloc(&c->cntpart, (size_t)C * NSTAT * ngm));
        TRY(c->alloc(&c->recal_part, (size_t)C * RECAL_SPLIT * c->ldr));
        TRY(c->alloc(&c->rpx, (size_t)RHS_KSPLIT_MAX * C * c->bs));
        TRY(c->alloc(&c->rpu, (size_t)RHS_KSPLIT_MAX * C * c->bs));
        c->tc = !c->regular && c->cfg.kernels == SODAGPU_KERNELS_AUTO &&
                sweep_tc_supported(c->cfg.precision, C, c->bs);
        if (c->tc) {
            c->ldd = (int)round_up((size_t)c->bs, 128);
            TRY(c->alloc(&c->dsplit, (size_t)sweep_tc_rows(C) * c->ldd));
            TRY(c->alloc(&c->k0part, (((size_t)c->ldd * C + 255) / 256) * C));
            TRY(c->alloc(&c->vpart, sweep_tc_vpart_floats(c->n, c->bs, C, c->sm_count), false));
            TRY(c->alloc(&c->ugrid, 1));
            const int NB = sweep_tc_rows(C);
            c->ldu = (int)round_up((size_t)c->bs, 8);
            TRY(c->alloc(&c->rsp, (size_t)NB * c->ldr));
            TRY(c->alloc(&c->rasp, (size_t)NB * c->ldra));
            TRY(c->alloc(&c->usp, (size_t)3 * p * c->ldu, false));
            const int ts = sweep_tc_table_stride(c->bs);
            c->h_rtab.assign((size_t)c->nb * ts, 0);
            sweep_tc_tables(c->blk_sizes.data(), c->nb, c->bs, c->ldx, c->sm_count, c->h_rtab.data());
            TRY(c->alloc(&c->rtab, c->h_rtab.size(), false));
            CUDA_TRY(cudaMemcpyAsync(c->rtab, c->h_rtab.data(), c->h_rtab.size() * 4, cudaMemcpyHostToDevice, c->st));
            c->maps.h_rtab = c->h_rtab.data();
            c->h_qoff.assign((size_t)c->nb + 1, 0);
            c->ncblk = (long long)sweep_tc_code_blocks(c->blk_sizes.data(), c->nb, c->h_qoff.data()) *
                       sweep_tc_update_tiles(c->n);
            TRY(c->alloc(&c->qoff, c->h_qoff.size(), false));
            CUDA_TRY(cudaMemcpyAsync(c->qoff, c->h_qoff.data(), c->h_qoff.size() * 4, cudaMemcpyHostToDevice, c->st));
            TRY(c->alloc(&c->Gt, (size_t)c->ncblk * TC_PACKED_BLOCK, false));
            TRY(c->alloc(&c->Gu, (size_t)c->ncblk * TC_PACKED_BLOCK, false));
        }
    }
    build_dev(c);
    if (c->tc) {
        const int NB = sweep_tc_rows(C);
        CUresult r = make_tmap_2d(&c->maps.rsp, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, c->rsp, c->ldr, NB, (uint64_t)c->ldr * 2,
                             64, NB, CU_TENSOR_MAP_SWIZZLE_128B);
        if (r == CUDA_SUCCESS)
            r = make_tmap_2d(&c->maps.rasp, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, c->rasp, c->ldra, NB,
                             (uint64_t)c->ldra * 2, 64, NB, CU_TENSOR_MAP_SWIZZLE_128B);
        if (r == CUDA_SUCCESS)
            r = make_tmap_2d(&c->maps.usp, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, c->usp, c->ldu, (uint64_t)3 * p,
                             (uint64_t)c->ldu * 2, 64, 128, CU_TENSOR_MAP_SWIZZLE_128B);
        if (r == CUDA_SUCCESS)
            r = make_tmap_2d(&c->maps.usp64, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, c->usp, c->ldu, (uint64_t)3 * p,
                             (uint64_t)c->ldu * 2, 64, 64, CU_TENSOR_MAP_SWIZZLE_128B);
        if (r == CUDA_SUCCESS)
            r = make_tmap_2d(&c->maps.d, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, c->dsplit, c->ldd, NB, (uint64_t)c->ldd * 2,
                             64, NB, CU_TENSOR_MAP_SWIZZLE_128B);
        if (r != CUDA_SUCCESS) return fail(SODAGPU_E_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
        if (!c->usp_ready) {
            CUDA_TRY(sweep_tc_prepare(c->G, c->D, c->st));
            CUDA_TRY(sweep_tc_tile_codes(c->G, c->D, c->Gt, c->Gu, c->ncblk, c->sm_count, c->st));
            c->usp_ready = true;
        }
    }
    RunCtl h{};
    CUDA_TRY(cudaMemcpyAsync(c->ctl, &h, sizeof h, cudaMemcpyHostToDevice, c->st));
    if (c->nskipped)
        k_xpx<<<std::min(c->nskipped, 1024), 256, 0, c->st>>>(c->G, c->ldx, c->xv, c->pos_of, c->iskipped,
                                                               c->nskipped, c->n, c->xpx);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(sweep_enqueue_init(c->D, c->cfg.vara0, c->cfg.scale_va, c->sm_count, c->st));
    CUDA_TRY(cudaStreamSynchronize(c->st));
    {
        RunCtl hc{};
        CUDA_TRY(cudaMemcpy(&hc, c->ctl, sizeof hc, cudaMemcpyDeviceToHost));
        if (hc.err == 19) return fail(SODAGPU_E_ARG, "a draw of the chain initialisation overran the injected-draw tape");
        if (hc.err) return fail(SODAGPU_E_TIMEOUT, "a bounded device loop gave up (code %d)", hc.err);
    }
    // capture one iteration of every chain as a CUDA graph
    if (c->graph) {
        cudaGraphExecDestroy(c->graph);
        c->graph = nullptr;
    }
    cudaGraph_t gr;
    CUDA_TRY(cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = sweep_enqueue_iteration(c->D, c->blk_sizes.data(), c->sm_count, &c->maps, c->st);
    cudaError_t e2 = cudaStreamEndCapture(c->st, &gr);
    if (e != cudaSuccess) return fail(SODAGPU_E_CUDA, "capturing the iteration failed: %s", cudaGetErrorString(e));
    if (e2 != cudaSuccess) return fail(SODAGPU_E_CUDA, "cudaStreamEndCapture: %s", cudaGetErrorString(e2));
    e = cudaGraphInstantiate(&c->graph, gr, 0);
    cudaGraphDestroy(gr);
    if (e != cudaSuccess) return fail(SODAGPU_E_CUDA, "cudaGraphInstantiate: %s", cudaGetErrorString(e));
    c->have_chain = true;
    return 0;
}

int sodagpu_run(sodagpu_ctx *c, int32_t iters, sodagpu_trace_cb cb, void *user)
{
    if (!c) return fail(SODAGPU_E_ARG, "null argument");
    if (!c->have_chain) return fail(SODAGPU_E_STATE, "call sodagpu_init_chains first");
    if (iters < 0) return fail(SODAGPU_E_ARG, "iters < 0");
    if (iters == 0) return 0;
    const auto t0 = std::chrono::steady_clock::now();
    RunCtl h{};
    CUDA_TRY(cudaMemcpyAsync(&h, c->ctl, sizeof h, cudaMemcpyDeviceToHost, c->st));
    CUDA_TRY(cudaStreamSynchronize(c->st));
    const int rep0 = h.rep;
    const int thin = c->cfg.thin;
    const int rows = (cb ? ((rep0 + iters) / thin - rep0 / thin) : 0) * c->C;
    if (rows > c->trace_cap) {
        if (c->trace) c->release(c->trace);
        c->trace = nullptr;
        TRY(c->alloc(&c->trace, rows, false));
        c->trace_cap = rows;
    }
    h.trace_iter = 0;
    h.trace_cap = cb ? rows : 0;
    h.trace_count = 0;
    h.trace = cb ? c->trace : nullptr;
    CUDA_TRY(cudaMemcpyAsync(c->ctl, &h, sizeof h, cudaMemcpyHostToDevice, c->st));
    cudaEvent_t e0, e1;
    CUDA_TRY(cudaEventCreate(&e0));
    CUDA_TRY(cudaEventCreate(&e1));
    CUDA_TRY(cudaEventRecord(e0, c->st));
    for (int t = 0; t < iters; ++t) CUDA_TRY(cudaGraphLaunch(c->graph, c->st));
    CUDA_TRY(cudaEventRecord(e1, c->st));
    CUDA_TRY(cudaMemcpyAsync(&h, c->ctl, sizeof h, cudaMemcpyDeviceToHost, c->st));
    CUDA_TRY(cudaStreamSynchronize(c->st));
    float dev_ms = 0.f;
    cudaEventElapsedTime(&dev_ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    c->t_run_dev_ms = dev_ms;
    c->t_run = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (h.err == 19)
        return fail(SODAGPU_E_ARG, "a draw overran the injected-draw tape (iteration past its end, or a draw site "
                                   "needing more than %d uniforms)", SODAGPU_TAPE_W);
    if (h.err) return fail(SODAGPU_E_TIMEOUT, "a bounded device loop gave up (code %d)", h.err);
    if (cb && rows > 0) {
        std::vector<sodagpu_trace_row> hr(rows);
        CUDA_TRY(cudaMemcpy(hr.data(), c->trace, sizeof(sodagpu_trace_row) * rows, cudaMemcpyDeviceToHost));
        for (int i = 0; i < rows; ++i) cb(user, &hr[i]);
    }
    return 0;
}

int sodagpu_get_results(sodagpu_ctx *c, int32_t chain, double *gstore, double *indiststore, double *vara_sstore,
                        double *scalars, double *snpstore, double *pstore, double *varstore)
{
    if (!c) return fail(SODAGPU_E_ARG, "null argument");
    if (!c->have_chain) return fail(SODAGPU_E_STATE, "no chain");
    if (chain < 0 || chain >= c->C) return fail(SODAGPU_E_ARG, "chain out of range");
    const int p = c->p, nm = c->cfg.nmix, ng = c->cfg.ngroup, ngm = ng * nm;
    ChainScal *S = new ChainScal;
    cudaError_t e = cudaMemcpyAsync(S, c->scal + chain, sizeof(ChainScal), cudaMemcpyDeviceToHost, c->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
    if (e != cudaSuccess) {
        delete S;
        return fail(SODAGPU_E_CUDA, "reading chain scalars: %s", cudaGetErrorString(e));
    }
    const double cnt = (double)S->counter;
    const size_t off = (size_t)chain * p;
    if (gstore) {
        CUDA_TRY(cudaMemcpy(gstore, c->gstore + off, sizeof(double) * p, cudaMemcpyDeviceToHost));
        for (int j = 0; j < p; ++j) gstore[j] = gstore[j] / cnt;
    }
    if (vara_sstore) {
        CUDA_TRY(cudaMemcpy(vara_sstore, c->vara_sstore + off, sizeof(double) * p, cudaMemcpyDeviceToHost));
        for (int j = 0; j < p; ++j) vara_sstore[j] = vara_sstore[j] / cnt;
    }
    if (indiststore) {
        std::vector<uint32_t> h((size_t)p * nm);
        CUDA_TRY(cudaMemcpy(h.data(), c->indist + off * nm, sizeof(uint32_t) * p * nm, cudaMemcpyDeviceToHost));
        for (int j = 0; j < p; ++j)
            for (int q = 0; q < nm; ++q) indiststore[(size_t)j + (size_t)q * p] = (double)h[(size_t)j * nm + q] / cnt;
    }
    if (scalars) {
        scalars[0] = S->mu_store / cnt;
        scalars[1] = S->vare_store / cnt;
        scalars[2] = S->vara_store / cnt;
        scalars[3] = S->included_store / cnt;
    }
    for (int t = 0; t < ngm; ++t) {
        if (snpstore) snpstore[t] = S->snpstore[t] / cnt;
        if (pstore) pstore[t] = S->pstore[t] / cnt;
        if (varstore) varstore[t] = S->varstore[t] / cnt;
    }
    delete S;
    return 0;
}

int sodagpu_get_state(sodagpu_ctx *c, int32_t chain, double *g, int32_t *cls, double *vara_s, double *yadj,
                      double *yaadj, double *scalars)
{
    if (!c) return fail(SODAGPU_E_ARG, "null argument");
    if (!c->have_chain) return fail(SODAGPU_E_STATE, "no chain");
    if (chain < 0 || chain >= c->C) return fail(SODAGPU_E_ARG, "chain out of range");
    const int p = c->p;
    const size_t off = (size_t)chain * p;
    if (g) CUDA_TRY(cudaMemcpy(g, c->g + off, sizeof(double) * p, cudaMemcpyDeviceToHost));
    if (cls) CUDA_TRY(cudaMemcpy(cls, c->cls + off, sizeof(int32_t) * p, cudaMemcpyDeviceToHost));
    if (vara_s) CUDA_TRY(cudaMemcpy(vara_s, c->vara_s + off, sizeof(double) * p, cudaMemcpyDeviceToHost));
    if (yadj) CUDA_TRY(cudaMemcpy(yadj, c->r + (size_t)chain * c->ldr, sizeof(double) * c->n, cudaMemcpyDeviceToHost));
    if (yaadj) CUDA_TRY(cudaMemcpy(yaadj, c->ra + (size_t)chain * c->ldra, sizeof(double) * c->bs, cudaMemcpyDeviceToHost));
    if (scalars) {
        ChainScal *S = new ChainScal;
        RunCtl h{};
        cudaError_t e = cudaMemcpy(S, c->scal + chain, sizeof(ChainScal), cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(&h, c->ctl, sizeof h, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) {
            delete S;
            return fail(SODAGPU_E_CUDA, "reading chain scalars: %s", cudaGetErrorString(e));
        }
        scalars[0] = S->mu[h.rep & 1];
        scalars[1] = S->vare;
        scalars[2] = S->vara;
        scalars[3] = S->included;
        delete S;
    }
    return 0;
}

int sodagpu_set_state(sodagpu_ctx *c, int32_t chain, const double *g, const int32_t *cls, const double *vara_s,
                      const double *yadj, const double *yaadj, const double *scalars, const double *pi)
{
    if (!c || !g || !cls || !vara_s || !yadj || !yaadj || !scalars) return fail(SODAGPU_E_ARG, "null argument");
    if (!c->have_chain) return fail(SODAGPU_E_STATE, "call sodagpu_init_chains first");
    if (chain < 0 || chain >= c->C) return fail(SODAGPU_E_ARG, "chain out of range");
    const int p = c->p, nm = c->cfg.nmix, ngm = c->cfg.ngroup * nm;
    for (int j = 0; j < p; ++j)
        if (cls[j] < 1 || cls[j] > nm) return fail(SODAGPU_E_ARG, "class of SNP %d is %d, not in 1..%d", j + 1, cls[j], nm);
    if (!(scalars[1] > 0.0)) return fail(SODAGPU_E_ARG, "vare must be positive");
    if (c->cfg.method != SODAGPU_BAYES_A && !(scalars[2] > 0.0)) return fail(SODAGPU_E_ARG, "vara must be positive");
    if (pi)
        for (int e = 0; e < ngm; ++e)
            if (!(pi[e] > 0.0)) return fail(SODAGPU_E_ARG, "pi entries must be positive");
    if (!c->st_g) {
        TRY(c->alloc(&c->st_g, p, false));
        TRY(c->alloc(&c->st_vs, p, false));
        TRY(c->alloc(&c->st_cls, p, false));
        TRY(c->alloc(&c->st_r, c->n, false));
        TRY(c->alloc(&c->st_ra, c->bs, false));
        TRY(c->alloc(&c->st_pi, ngm, false));
    }
    CUDA_TRY(cudaMemcpyAsync(c->st_g, g, sizeof(double) * p, cudaMemcpyHostToDevice, c->st));
    CUDA_TRY(cudaMemcpyAsync(c->st_cls, cls, sizeof(int32_t) * p, cudaMemcpyHostToDevice, c->st));
    CUDA_TRY(cudaMemcpyAsync(c->st_vs, vara_s, sizeof(double) * p, cudaMemcpyHostToDevice, c->st));
    CUDA_TRY(cudaMemcpyAsync(c->st_r, yadj, sizeof(double) * c->n, cudaMemcpyHostToDevice, c->st));
    CUDA_TRY(cudaMemcpyAsync(c->st_ra, yaadj, sizeof(double) * c->bs, cudaMemcpyHostToDevice, c->st));
    if (pi) CUDA_TRY(cudaMemcpyAsync(c->st_pi, pi, sizeof(double) * ngm, cudaMemcpyHostToDevice, c->st));
    CUDA_TRY(sweep_set_state(c->D, chain, c->st_g, c->st_cls, c->st_vs, c->st_r, c->st_ra, pi ? c->st_pi : nullptr,
                             scalars[0], scalars[1], scalars[2], (int)scalars[3], c->st));
    CUDA_TRY(cudaStreamSynchronize(c->st));
    return 0;
}

int sodagpu_set_iteration(sodagpu_ctx *c, int32_t rep)
{
    if (!c) return fail(SODAGPU_E_ARG, "null argument");
    if (!c->have_chain) return fail(SODAGPU_E_STATE, "call sodagpu_init_chains first");
    if (rep < 0) return fail(SODAGPU_E_ARG, "rep < 0");
    RunCtl h{};
    CUDA_TRY(cudaMemcpyAsync(&h, c->ctl, sizeof h, cudaMemcpyDeviceToHost, c->st));
    CUDA_TRY(cudaStreamSynchronize(c->st));
    h.rep = rep;
    CUDA_TRY(cudaMemcpyAsync(c->ctl, &h, sizeof h, cudaMemcpyHostToDevice, c->st));
    CUDA_TRY(cudaStreamSynchronize(c->st));
    return 0;
}

namespace {
int subset_call(sodagpu_ctx *c, int32_t b, bool rhs_only)
{
    if (!c) return fail(SODAGPU_E_ARG, "null argument");
    if (!c->have_chain) return fail(SODAGPU_E_STATE, "call sodagpu_init_chains first");
    if (c->regular) return fail(SODAGPU_E_UNSUPPORTED, "the regular sampler has no subsets");
    if (b < 0 || b >= c->nb) return fail(SODAGPU_E_ARG, "subset %d out of range 0..%d", b, c->nb - 1);
    Dev D = c->D;
    if (rhs_only) {
        if (!c->rhs_buf) TRY(c->alloc(&c->rhs_buf, (size_t)c->C * c->bs));
        D.rhs_out = c->rhs_buf;
    }
    CUDA_TRY(sweep_enqueue_subset(D, b, c->blk_sizes[b], c->sm_count, &c->maps, c->st, rhs_only));
    RunCtl h{};
    CUDA_TRY(cudaMemcpyAsync(&h, c->ctl, sizeof h, cudaMemcpyDeviceToHost, c->st));
    CUDA_TRY(cudaStreamSynchronize(c->st));
    if (h.err) return fail(SODAGPU_E_TIMEOUT, "a bounded device loop gave up (code %d)", h.err);
    return 0;
}
}  // namespace

int sodagpu_subset_rhs(sodagpu_ctx *c, int32_t b, double *rhs)
{
    if (!rhs) return fail(SODAGPU_E_ARG, "null argument");
    TRY(subset_call(c, b, true));
    const int N = c->blk_sizes[b];
    for (int ch = 0; ch < c->C; ++ch)
        CUDA_TRY(cudaMemcpy(rhs + (size_t)ch * N, c->rhs_buf + (size_t)ch * c->bs, sizeof(double) * N,
                            cudaMemcpyDeviceToHost));
    return 0;
}

int sodagpu_run_subset(sodagpu_ctx *c, int32_t b) { return subset_call(c, b, false); }

int sodagpu_get_z(sodagpu_ctx *c, double *xa, double *xxd, int32_t *skip)
{
    if (!c) return fail(SODAGPU_E_ARG, "null argument");
    if (!c->have_z) return fail(SODAGPU_E_STATE, "no Z built");
    if (xa) {
        double *dxa = nullptr;
        TRY(c->alloc(&dxa, (size_t)c->bs * c->p, false));
        CUDA_TRY(zb_unpack_dense(c->U64, c->uoff, c->ulen, c->p, c->bs, dxa, c->st));
        CUDA_TRY(cudaMemcpyAsync(xa, dxa, sizeof(double) * c->bs * c->p, cudaMemcpyDeviceToHost, c->st));
        CUDA_TRY(cudaStreamSynchronize(c->st));
        c->release(dxa);
    }
    if (xxd) CUDA_TRY(cudaMemcpy(xxd, c->xxd, sizeof(double) * c->nb, cudaMemcpyDeviceToHost));
    if (skip) {
        std::vector<uint8_t> h(c->p);
        CUDA_TRY(cudaMemcpy(h.data(), c->skip, c->p, cudaMemcpyDeviceToHost));
        for (int k = 0; k < c->p; ++k) skip[k] = h[k];
    }
    return 0;
}

int sodagpu_compute_dgv(sodagpu_ctx *c, double mu, const double *effects, double *pred)
{
    if (!c || !effects || !pred) return fail(SODAGPU_E_ARG, "null argument");
    if (!c->have_z) return fail(SODAGPU_E_STATE, "no genotypes in subset order (run sodagpu_build_z)");
    const int nsplit = 32;
    double *deff = nullptr, *part = nullptr, *dpred = nullptr;
    TRY(c->alloc(&deff, c->p, false));
    TRY(c->alloc(&part, (size_t)nsplit * c->ldx, false));
    TRY(c->alloc(&dpred, c->n, false));
    CUDA_TRY(cudaMemcpyAsync(deff, effects, sizeof(double) * c->p, cudaMemcpyHostToDevice, c->st));
    CUDA_TRY(zb_dgv(c->G, c->ldx, c->xv, c->perm, deff, c->n, c->p, mu, part, nsplit, dpred, c->st));
    CUDA_TRY(cudaMemcpyAsync(pred, dpred, sizeof(double) * c->n, cudaMemcpyDeviceToHost, c->st));
    CUDA_TRY(cudaStreamSynchronize(c->st));
    c->release(deff);
    c->release(part);
    c->release(dpred);
    return 0;
}

int sodagpu_predict(int32_t nind, int32_t nloci, const void *geno, int32_t layout, const double *freq, double mu,
                    const double *effects, double *pred)
{
    if (nind < 1 || nloci < 1 || !geno || !freq || !effects || !pred) return fail(SODAGPU_E_ARG, "bad argument");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(SODAGPU_E_NODEVICE, "no CUDA device visible");
    }
    cudaStream_t st;
    CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    const int n = nind, p = nloci;
    const int ldx = (int)round_up((size_t)n, 128);
    int8_t *G = nullptr;
    double *dfreq = nullptr, *xv = nullptr, *deff = nullptr, *part = nullptr, *dpred = nullptr;
    int32_t *perm = nullptr;
    uint8_t *tmp = nullptr;
    const int nsplit = 32;
    std::vector<int32_t> ident(p);
    for (int k = 0; k < p; ++k) ident[k] = k;
    cudaError_t e = cudaSuccess;
    auto chk = [&](cudaError_t x) { if (e == cudaSuccess) e = x; };
    chk(cudaMalloc(&G, (size_t)p * ldx));
    chk(cudaMalloc(&dfreq, sizeof(double) * p));
    chk(cudaMalloc(&xv, sizeof(double) * 4 * p));
    chk(cudaMalloc(&deff, sizeof(double) * p));
    chk(cudaMalloc(&part, sizeof(double) * nsplit * ldx));
    chk(cudaMalloc(&dpred, sizeof(double) * n));
    chk(cudaMalloc(&perm, sizeof(int32_t) * p));
    if (e == cudaSuccess) chk(cudaMemsetAsync(G, 0, (size_t)p * ldx, st));
    const bool on_dev = (layout & SODAGPU_GENO_DEVICE_PTR) != 0;
    const cudaMemcpyKind mk = on_dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    if (e == cudaSuccess) {
        if ((layout & 0xff) == SODAGPU_GENO_CODES) {
            chk(cudaMemcpy2DAsync(G, ldx, geno, n, n, p, mk, st));
        } else {
            const size_t rec = ((size_t)n + 3) / 4;
            chk(cudaMalloc(&tmp, rec * p));
            if (e == cudaSuccess) chk(cudaMemcpyAsync(tmp, geno, rec * p, mk, st));
            if (e == cudaSuccess) chk(zb_decode_bed(tmp, n, p, G, ldx, st));
        }
    }
    // codes outside 0..2 are an error, as in sodagpu_load_genotypes: counted on the device (k_freq, into
    // the xv buffer, which is written again below)
    int *bad = nullptr, h_bad = 0;
    chk(cudaMalloc(&bad, sizeof(int)));
    if (e == cudaSuccess) chk(cudaMemsetAsync(bad, 0, sizeof(int), st));
    if (e == cudaSuccess) chk(zb_freq(G, n, p, ldx, xv, bad, st));
    if (e == cudaSuccess) chk(cudaMemcpyAsync(&h_bad, bad, sizeof(int), cudaMemcpyDeviceToHost, st));
    if (e == cudaSuccess) chk(cudaStreamSynchronize(st));
    if (e == cudaSuccess) chk(cudaMemcpyAsync(dfreq, freq, sizeof(double) * p, cudaMemcpyHostToDevice, st));
    if (e == cudaSuccess) chk(cudaMemcpyAsync(deff, effects, sizeof(double) * p, cudaMemcpyHostToDevice, st));
    if (e == cudaSuccess) chk(cudaMemcpyAsync(perm, ident.data(), sizeof(int32_t) * p, cudaMemcpyHostToDevice, st));
    if (e == cudaSuccess) chk(zb_xv(dfreq, perm, p, xv, st));
    if (e == cudaSuccess) chk(zb_dgv(G, ldx, xv, nullptr, deff, n, p, mu, part, nsplit, dpred, st));
    if (e == cudaSuccess) chk(cudaMemcpyAsync(pred, dpred, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
    if (e == cudaSuccess) chk(cudaStreamSynchronize(st));
    cudaFree(G); cudaFree(dfreq); cudaFree(xv); cudaFree(deff); cudaFree(part); cudaFree(dpred); cudaFree(perm);
    cudaFree(tmp);
    cudaFree(bad);
    cudaStreamDestroy(st);
    if (e != cudaSuccess) return fail(SODAGPU_E_CUDA, "prediction failed: %s", cudaGetErrorString(e));
    if (h_bad) return fail(SODAGPU_E_ARG, "%d genotype codes outside 0..2", h_bad);
    return 0;
}

int sodagpu_timings(sodagpu_ctx *c, double *build_z_s, double *run_s, double *run_device_ms)
{
    if (!c) return fail(SODAGPU_E_ARG, "null argument");
    if (build_z_s) *build_z_s = c->t_build;
    if (run_s) *run_s = c->t_run;
    if (run_device_ms) *run_device_ms = c->t_run_dev_ms;
    return 0;
}

int sodagpu_profile_kernels(sodagpu_ctx *c, int32_t iters, double *ms, int32_t *launches)
{
    if (!c || !ms || !launches) return fail(SODAGPU_E_ARG, "null argument");
    if (!c->have_chain) return fail(SODAGPU_E_STATE, "call sodagpu_init_chains first");
    for (int k = 0; k < PROF_NCLASS; ++k) { ms[k] = 0.0; launches[k] = 0; }
    RunCtl h{};
    CUDA_TRY(cudaMemcpyAsync(&h, c->ctl, sizeof h, cudaMemcpyDeviceToHost, c->st));
    CUDA_TRY(cudaStreamSynchronize(c->st));
    h.trace = nullptr;
    h.trace_cap = 0;
    h.trace_iter = 0;
    CUDA_TRY(cudaMemcpyAsync(c->ctl, &h, sizeof h, cudaMemcpyHostToDevice, c->st));
    const int cap = 4 * c->nb + 16;   // rhs, draws and update per subset, plus the iteration kernels
    std::vector<cudaEvent_t> ev(2 * cap);
    std::vector<int> cls(cap);
    for (auto &e : ev) CUDA_TRY(cudaEventCreate(&e));
    int rc = 0;
    for (int t = 0; t < iters && rc == 0; ++t) {
        ProfHook hook{ev.data(), cls.data(), 0, cap};
        cudaError_t e = sweep_enqueue_iteration(c->D, c->blk_sizes.data(), c->sm_count, &c->maps, c->st, &hook);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
        if (e != cudaSuccess) {
            rc = fail(SODAGPU_E_CUDA, "profiled iteration failed: %s", cudaGetErrorString(e));
            break;
        }
        for (int q = 0; q < hook.n; ++q) {
            float x = 0.f;
            cudaEventElapsedTime(&x, ev[2 * q], ev[2 * q + 1]);
            ms[cls[q]] += x;
            launches[cls[q]] += 1;
        }
    }
    for (auto &e : ev) cudaEventDestroy(e);
    return rc;
}

}  // extern "C"

struct sodagpu_batch {
    std::vector<sodagpu_ctx *> jobs;
    int dev = 0, sm_count = 0, steps = 0;
    cudaStream_t st = nullptr;
    cudaGraphExec_t graph = nullptr;
    Dev *ddev = nullptr;
    double last_ms = 0.0;
};

extern "C" {

void sodagpu_batch_destroy(sodagpu_batch *b)
{
    if (!b) return;
    if (b->st) cudaStreamSynchronize(b->st);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    if (b->ddev) cudaFree(b->ddev);
    if (b->st) cudaStreamDestroy(b->st);
    delete b;
}

int sodagpu_batch_create(sodagpu_batch **out, sodagpu_ctx *const *jobs, int32_t njobs, int32_t flags)
{
    if (flags & ~SODAGPU_BATCH_SOLO_SPLITS) return fail(SODAGPU_E_ARG, "unknown flags 0x%x", flags);
    if (!out || !jobs) return fail(SODAGPU_E_ARG, "null argument");
    *out = nullptr;
    if (njobs < 1 || njobs > SODAGPU_MAXJOBS) return fail(SODAGPU_E_ARG, "njobs %d outside 1..%d", njobs, SODAGPU_MAXJOBS);
    for (int j = 0; j < njobs; ++j) {
        const sodagpu_ctx *c = jobs[j];
        if (!c) return fail(SODAGPU_E_ARG, "job %d is null", j);
        for (int k = 0; k < j; ++k)
            if (jobs[k] == c) return fail(SODAGPU_E_ARG, "job %d appears twice", j);
        if (!c->have_chain) return fail(SODAGPU_E_STATE, "job %d: call sodagpu_init_chains first", j);
        if (c->tc) return fail(SODAGPU_E_UNSUPPORTED, "job %d runs the tensor-core kernels; batches run the CUDA-core "
                                                      "kernels (SODAGPU_KERNELS_CUDA_CORES or fewer than 4 chains)", j);
        if (c->regular) return fail(SODAGPU_E_UNSUPPORTED, "job %d: the regular sampler is not batched", j);
        if (c->tape) return fail(SODAGPU_E_UNSUPPORTED, "job %d has an injected-draw tape", j);
        if (c->dev != jobs[0]->dev || c->C != jobs[0]->C || c->D.precision != jobs[0]->D.precision)
            return fail(SODAGPU_E_ARG, "job %d: every job of a batch needs the same device, chain count and precision", j);
    }
    CUDA_TRY(cudaSetDevice(jobs[0]->dev));
    for (int j = 0; j < njobs; ++j) CUDA_TRY(cudaStreamSynchronize(jobs[j]->st));
    sodagpu_batch *b = new sodagpu_batch;
    b->jobs.assign(jobs, jobs + njobs);
    b->dev = jobs[0]->dev;
    b->sm_count = jobs[0]->sm_count;
    int max_bs = 0;
    for (auto *c : b->jobs) {
        max_bs = std::max(max_bs, c->bs);
        b->steps = std::max(b->steps, c->nb);
    }
    const int prec = jobs[0]->D.precision, C = jobs[0]->C;
    if (sweep_multi_prepare(prec, C, max_bs) != cudaSuccess) {
        sodagpu_batch_destroy(b);
        return fail(SODAGPU_E_UNSUPPORTED, "blocksize %d too large", max_bs);
    }
    // the rhs of every job gets a share of one wave of CTAs in proportion to its genotype bytes per step
    std::vector<Dev> hdev(njobs);
    std::vector<const int *> bsz(njobs);
    std::vector<int> ks(njobs);
    double wsum = 0.0;
    for (auto *c : b->jobs) wsum += (double)c->n * c->bs;
    for (int j = 0; j < njobs; ++j) {
        sodagpu_ctx *c = b->jobs[j];
        hdev[j] = c->D;
        bsz[j] = c->blk_sizes.data();
        // a job on its own takes one wave of CTAs for its rhs
        const int share = (flags & SODAGPU_BATCH_SOLO_SPLITS)
                              ? b->sm_count
                              : std::max(1, (int)std::lround(b->sm_count * (double)c->n * c->bs / wsum));
        ks[j] = sweep_multi_rhs_split(prec, c->bs, C, c->ldx, share);
    }
    cudaError_t e = cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&b->ddev, sizeof(Dev) * njobs);
    if (e == cudaSuccess) e = cudaMemcpy(b->ddev, hdev.data(), sizeof(Dev) * njobs, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        sodagpu_batch_destroy(b);
        return fail(SODAGPU_E_CUDA, "batch set-up: %s", cudaGetErrorString(e));
    }
    BatchPlan P{njobs, hdev.data(), b->ddev, bsz.data(), ks.data()};
    cudaGraph_t gr;
    e = cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        cudaError_t e1 = sweep_enqueue_iteration_multi(P, b->sm_count, b->st);
        cudaError_t e2 = cudaStreamEndCapture(b->st, &gr);
        e = e1 != cudaSuccess ? e1 : e2;
        if (e == cudaSuccess) {
            e = cudaGraphInstantiate(&b->graph, gr, 0);
            cudaGraphDestroy(gr);
        }
    }
    if (e != cudaSuccess) {
        sodagpu_batch_destroy(b);
        return fail(SODAGPU_E_CUDA, "capturing the batched iteration: %s", cudaGetErrorString(e));
    }
    *out = b;
    return 0;
}

int sodagpu_batch_run(sodagpu_batch *b, int32_t iters)
{
    if (!b) return fail(SODAGPU_E_ARG, "null argument");
    if (iters < 0) return fail(SODAGPU_E_ARG, "iters < 0");
    if (iters == 0) return 0;
    CUDA_TRY(cudaSetDevice(b->dev));
    // each job's control block: no trace rows; the job's own stream drained first
    for (auto *c : b->jobs) {
        RunCtl h{};
        CUDA_TRY(cudaMemcpyAsync(&h, c->ctl, sizeof h, cudaMemcpyDeviceToHost, c->st));
        CUDA_TRY(cudaStreamSynchronize(c->st));
        h.trace_iter = 0;
        h.trace_cap = 0;
        h.trace_count = 0;
        h.trace = nullptr;
        CUDA_TRY(cudaMemcpyAsync(c->ctl, &h, sizeof h, cudaMemcpyHostToDevice, c->st));
        CUDA_TRY(cudaStreamSynchronize(c->st));
    }
    cudaEvent_t e0, e1;
    CUDA_TRY(cudaEventCreate(&e0));
    CUDA_TRY(cudaEventCreate(&e1));
    CUDA_TRY(cudaEventRecord(e0, b->st));
    for (int t = 0; t < iters; ++t) CUDA_TRY(cudaGraphLaunch(b->graph, b->st));
    CUDA_TRY(cudaEventRecord(e1, b->st));
    CUDA_TRY(cudaStreamSynchronize(b->st));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b->last_ms = ms;
    for (size_t j = 0; j < b->jobs.size(); ++j) {
        RunCtl h{};
        CUDA_TRY(cudaMemcpy(&h, b->jobs[j]->ctl, sizeof h, cudaMemcpyDeviceToHost));
        if (h.err) return fail(SODAGPU_E_TIMEOUT, "job %zu: a bounded device loop gave up (code %d)", j, h.err);
    }
    return 0;
}

int sodagpu_batch_timings(sodagpu_batch *b, double *run_device_ms, int32_t *steps)
{
    if (!b) return fail(SODAGPU_E_ARG, "null argument");
    if (run_device_ms) *run_device_ms = b->last_ms;
    if (steps) *steps = b->steps;
    return 0;
}

int sodagpu_autotune_batch(int32_t njobs, const int32_t *n, const int32_t *p, int32_t iters, int32_t max_blocksize,
                           const double *model, int32_t *blocksize, int32_t *steps, double *model_s)
{
    if (!n || !p || !blocksize) return fail(SODAGPU_E_ARG, "null argument");
    if (njobs < 1 || njobs > SODAGPU_MAXJOBS) return fail(SODAGPU_E_ARG, "njobs %d outside 1..%d", njobs, SODAGPU_MAXJOBS);
    if (iters < 1 || max_blocksize < 2) return fail(SODAGPU_E_ARG, "iters < 1 or max_blocksize < 2");
    static const double dflt[6] = {30.0, 2.6e12, 1.0, 4.0, 5e13, 6e11};
    const double *m = model ? model : dflt;
    for (int q = 0; q < 6; ++q)
        if (!(m[q] > 0.0)) return fail(SODAGPU_E_ARG, "model[%d] must be positive", q);
    int pmax = 0;
    for (int j = 0; j < njobs; ++j) {
        if (n[j] < 1 || p[j] < 1) return fail(SODAGPU_E_ARG, "job %d: n and p must be positive", j);
        pmax = std::max(pmax, p[j]);
    }
    // S from the smallest that respects max_blocksize up to one SNP per subset; candidates grow by 1/16
    int s_lo = 1;
    for (int j = 0; j < njobs; ++j) s_lo = std::max(s_lo, (p[j] + max_blocksize - 1) / max_blocksize);
    auto cost = [&](int S) {
        double per_iter = S * m[0] * 1e-6, build = 0.0;
        for (int j = 0; j < njobs; ++j) {
            const double N = std::min<double>(max_blocksize, std::ceil((double)p[j] / S));
            const double bytes = 2.0 * ((double)n[j] * p[j] * m[2] + (double)p[j] * (N + 1.0) / 2.0 * m[3]);
            per_iter += bytes / m[1];
            build += (double)p[j] * ((double)n[j] * N / m[4] + N * N / (3.0 * m[5]));
        }
        return iters * per_iter + build;
    };
    int best = s_lo;
    double best_c = cost(s_lo);
    for (int S = s_lo; S <= pmax;) {
        const double cst = cost(S);
        if (cst < best_c) {
            best_c = cst;
            best = S;
        }
        const int nx = S + std::max(1, S / 16);
        if (nx > pmax && S < pmax) S = pmax;
        else S = nx;
    }
    int smax = 0;
    for (int j = 0; j < njobs; ++j) {
        blocksize[j] = std::min(max_blocksize, (p[j] + best - 1) / best);
        smax = std::max(smax, (p[j] + blocksize[j] - 1) / blocksize[j]);
    }
    if (steps) *steps = smax;
    if (model_s) *model_s = best_c;
    return 0;
}

void sodagpu_destroy(sodagpu_ctx *c)
{
    if (!c) return;
    if (c->st) cudaStreamSynchronize(c->st);
    if (c->graph) cudaGraphExecDestroy(c->graph);
    for (void *p_ : c->allocs) cudaFree(p_);
    c->allocs.clear();
    if (c->st) cudaStreamDestroy(c->st);
    delete c;
}

}  // extern "C"
