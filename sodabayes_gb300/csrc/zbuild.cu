// zbuild.cu — construction of the SODA augmenting matrix on the GPU.
//
// Per subset b of N SNPs (get_aug_matrix, soda.f90:445-518):
//   A   = X_b'X_b from the exact integer Gram of the 0/1/2 codes, centred and
//         scaled like xxproduct (soda.f90:520-556)              k_gram
//   d   = lambda_max(A) + 0.001 (soda.f90:484-486); lambda_max from a
//         fully reorthogonalised Lanczos run (k_lz_*) instead of the
//         reference's power iteration (soda.f90:378-401): both converge to
//         the same eigenvalue, Lanczos in far fewer products with A.
//   U   = chol(d I - A), upper (choleskyPD, soda.f90:8-47)     k_chol_*
//   fallback for a failed factorisation: the reference's own sequence —
//         the unpivoted attempt up to the failing row, then the pivoted
//         factorisation (choleskyPSD, soda.f90:49-124) — in k_psd_block.
// All kernels work on a batch of subsets at once; each subset's FP64 work
// matrix W_b (N x N, column-major, ld N) lives at wofs[b].
#include <cuda_runtime.h>
#include <stdint.h>
#include "rng.cuh"
#include "state.cuh"
#include "zbuild.cuh"

namespace soda {

// ---------------------------------------------------------------------------
// genotype ingest: bed decode, allele frequencies, centring tables
// ---------------------------------------------------------------------------

// load_geno's decode (utilities.f90:438-454): b - ((b>>1)&0x55) maps the
// 2-bit codes 00,01,10,11 to 0,1,1,2.  One thread per output byte quad.
__global__ void k_decode_bed(const uint8_t *bed, int n, int p, size_t rec_bytes, int8_t *G, int ldx)
{
    const size_t tot = (size_t)p * rec_bytes;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < tot; t += (size_t)gridDim.x * blockDim.x) {
        const int j = (int)(t / rec_bytes);
        const int q = (int)(t % rec_bytes);
        uint8_t b = bed[t];
        b = (uint8_t)(b - ((b >> 1) & 0x55));
        for (int s = 0; s < 4; ++s) {
            const int i = q * 4 + s;
            if (i < n) G[(size_t)j * ldx + i] = (int8_t)((b >> (2 * s)) & 3);
        }
    }
}

// freq_j = sum(codes)/(2n) (xscale, utilities.f90:527).  One warp per SNP.
// Codes outside 0..2 are counted in *bad and replaced by 1 (a missing call).
__global__ void k_freq(int8_t *G, int n, int p, int ldx, double *freq, int *bad)
{
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= p) return;
    int8_t *col = G + (size_t)warp * ldx;
    long long s = 0;
    int nbad = 0;
    for (int i = lane; i < n; i += 32) {
        int v = col[i];
        if (v < 0 || v > 2) {
            ++nbad;
            v = 1;
            col[i] = 1;
        }
        s += v;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_xor_sync(0xffffffffu, s, o);
        nbad += __shfl_xor_sync(0xffffffffu, nbad, o);
    }
    if (lane == 0) {
        freq[warp] = (double)s / (2.0 * (double)n);
        if (nbad) atomicAdd(bad, nbad);
    }
}

// Gather SNP columns into subset order and build the centring table.
__global__ void k_gather(const int8_t *Gsnp, int8_t *Gpos, const int32_t *perm, int p, int ldx)
{
    const size_t tot = (size_t)p * (ldx / 16);
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < tot; t += (size_t)gridDim.x * blockDim.x) {
        const int k = (int)(t / (ldx / 16));
        const int q = (int)(t % (ldx / 16));
        reinterpret_cast<uint4 *>(Gpos + (size_t)k * ldx)[q] =
            reinterpret_cast<const uint4 *>(Gsnp + (size_t)perm[k] * ldx)[q];
    }
}

__global__ void k_xv32(const double *xv, int p, float *xv32)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < 4 * p) xv32[t] = (float)xv[t];
}

__global__ void k_xv(const double *freq, const int32_t *perm, int p, double *xv)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= p) return;
    const double eps = 2.220446049250313e-16;
    const double f = freq[perm[k]];
    double *o = xv + (size_t)k * 4;
    if (f < eps || (1.0 - f) < eps) {
        o[0] = o[1] = o[2] = o[3] = 0.0;
        return;
    }
    const double sd = sqrt(__dmul_rn(__dmul_rn(2.0, f), __dsub_rn(1.0, f)));
    const double twop = __dmul_rn(2.0, f);
    o[0] = __ddiv_rn(__dsub_rn(0.0, twop), sd);
    o[1] = __ddiv_rn(__dsub_rn(1.0, twop), sd);
    o[2] = __ddiv_rn(__dsub_rn(2.0, twop), sd);
    o[3] = __ddiv_rn(1.0, sd);
}

__global__ void k_x32(const int8_t *G, const double *xv, float *X32, int n, int p, int ldx)
{
    const size_t tot = (size_t)p * ldx;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < tot; t += (size_t)gridDim.x * blockDim.x) {
        const int k = (int)(t / ldx);
        const int i = (int)(t % ldx);
        X32[t] = i < n ? (float)xv[(size_t)k * 4 + G[t]] : 0.0f;
    }
}

// ---------------------------------------------------------------------------
// Gram: S = G_b'G_b with dp4a on 64x64 tiles, then the xxproduct scaling
// ---------------------------------------------------------------------------
constexpr int GT = 64;   // output tile
constexpr int GK = 64;   // bytes of K per stage

__global__ void __launch_bounds__(256) k_gram(const int8_t *G, int ldx, const int32_t *blk_ls,
                                              const int32_t *batch_blocks, const int64_t *wofs,
                                              const double *freq, const int32_t *perm, int n,
                                              double *W)
{
    __shared__ int sA[GT][GK / 4 + 1];
    __shared__ int sB[GT][GK / 4 + 1];
    const int b = batch_blocks[blockIdx.y];
    const int ls = blk_ls[b], N = blk_ls[b + 1] - ls;
    const int nt = (N + GT - 1) / GT;
    // decode the upper-triangular tile index
    int t = blockIdx.x, ti = 0;
    while (ti < nt && t >= nt - ti) { t -= nt - ti; ++ti; }
    if (ti >= nt) return;
    const int tj = ti + t;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    int acc[4][4] = {};
    const int lr = threadIdx.x >> 2;          // column of the tile this thread loads
    const int lq = (threadIdx.x & 3) * 4;     // first word of the 16-byte chunk
    const int ca = ti * GT + lr, cb = tj * GT + lr;
    for (int k0 = 0; k0 < ldx; k0 += GK) {
        uint4 va = make_uint4(0, 0, 0, 0), vb = make_uint4(0, 0, 0, 0);
        if (ca < N) va = *reinterpret_cast<const uint4 *>(G + (size_t)(ls + ca) * ldx + k0 + lq * 4);
        if (cb < N) vb = *reinterpret_cast<const uint4 *>(G + (size_t)(ls + cb) * ldx + k0 + lq * 4);
        __syncthreads();
        sA[lr][lq + 0] = (int)va.x; sA[lr][lq + 1] = (int)va.y; sA[lr][lq + 2] = (int)va.z; sA[lr][lq + 3] = (int)va.w;
        sB[lr][lq + 0] = (int)vb.x; sB[lr][lq + 1] = (int)vb.y; sB[lr][lq + 2] = (int)vb.z; sB[lr][lq + 3] = (int)vb.w;
        __syncthreads();
#pragma unroll
        for (int w = 0; w < GK / 4; ++w) {
            int a[4], bb[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) { a[q] = sA[ty * 4 + q][w]; bb[q] = sB[tx * 4 + q][w]; }
#pragma unroll
            for (int q = 0; q < 4; ++q)
#pragma unroll
                for (int r = 0; r < 4; ++r) acc[q][r] = __dp4a(a[q], bb[r], acc[q][r]);
        }
    }
    const double ep = 2.220446049250313e-16;
    double *Wb = W + wofs[b];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int j = ti * GT + ty * 4 + q;
        if (j >= N) continue;
        const double fj = freq[perm[ls + j]];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int k = tj * GT + tx * 4 + r;
            if (k >= N) continue;
            const double fk = freq[perm[ls + k]];
            // the scaling takes the frequency of the later position first, like xxproduct's
            // (jj, kk) with kk <= jj (soda.f90:474-481, 553-554): products of doubles are not
            // associative, and in a diagonal tile the two threads holding (j, k) and (k, j) both
            // write both entries, so they must compute the same value
            const double fa = k > j ? fk : fj, fb = k > j ? fj : fk;
            const double qa = __dsub_rn(1.0, fa), qb = __dsub_rn(1.0, fb);
            double res;
            if (fa <= ep || qa <= ep || fb <= ep || qb <= ep) {
                res = 0.0;
            } else {
                const double pa = __dmul_rn(fa, 2.0), pb = __dmul_rn(fb, 2.0);
                const double t1 = __dmul_rn(__dmul_rn((double)n, pa), pb);
                const double den = sqrt(__dmul_rn(__dmul_rn(__dmul_rn(pa, pb), qa), qb));
                res = __ddiv_rn(__dsub_rn((double)acc[q][r], t1), den);
            }
            Wb[(size_t)j + (size_t)k * N] = res;
            Wb[(size_t)k + (size_t)j * N] = res;
        }
    }
}

// ---------------------------------------------------------------------------
// Lanczos with full reorthogonalisation (two classical Gram-Schmidt passes)
// V_b: [mmax][N] at vofs[b]; alpha/beta: [batch][mmax]
// ---------------------------------------------------------------------------
__device__ double blk_sum(double v, double *sh)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if (lane == 0) sh[w] = v;
    __syncthreads();
    if (w == 0) {
        double t = lane < nw ? sh[lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (lane == 0) sh[32] = t;
    }
    __syncthreads();
    return sh[32];
}

__global__ void __launch_bounds__(1024) k_lz_init(const int32_t *blk_ls, const int32_t *batch_blocks,
                                                  const int64_t *vofs, double *V, uint64_t seed)
{
    __shared__ double sh[33];
    const int b = batch_blocks[blockIdx.x];
    const int N = blk_ls[b + 1] - blk_ls[b];
    double *v = V + vofs[blockIdx.x];
    double ss = 0.0;
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        // the i-th uniform of the (seed, subset, P_POWER) stream, like the
        // reference's random start vector (soda.f90:390)
        CRng R;
        crng_init(R, seed, 0, 0, b, P_POWER);
        R.c3 += (uint32_t)(i >> 1);
        double x = crng_unit(R);
        if (i & 1) x = crng_unit(R);
        v[i] = x;
        ss += x * x;
    }
    ss = blk_sum(ss, sh);
    const double inv = 1.0 / sqrt(ss);
    for (int i = threadIdx.x; i < N; i += blockDim.x) v[i] *= inv;
}

// w = A v_j ; one thread per row, v_j staged in shared memory
__global__ void __launch_bounds__(128) k_lz_matvec(const double *W, const int64_t *wofs,
                                                   const int32_t *blk_ls, const int32_t *batch_blocks,
                                                   const int64_t *vofs, const double *V, double *Wvec,
                                                   int ldw, int j)
{
    extern __shared__ double sv[];
    const int b = batch_blocks[blockIdx.y];
    const int N = blk_ls[b + 1] - blk_ls[b];
    const double *v = V + vofs[blockIdx.y] + (size_t)j * N;
    for (int k = threadIdx.x; k < N; k += blockDim.x) sv[k] = v[k];
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const double *A = W + wofs[b];
    double acc0 = 0.0, acc1 = 0.0;
    int k = 0;
    for (; k + 1 < N; k += 2) {
        acc0 += A[(size_t)i + (size_t)k * N] * sv[k];
        acc1 += A[(size_t)i + (size_t)(k + 1) * N] * sv[k + 1];
    }
    if (k < N) acc0 += A[(size_t)i + (size_t)k * N] * sv[k];
    Wvec[(size_t)blockIdx.y * ldw + i] = acc0 + acc1;
}

// alpha, three-term recurrence, two CGS passes, beta, v_{j+1}
__global__ void __launch_bounds__(1024) k_lz_orth(const int32_t *blk_ls, const int32_t *batch_blocks,
                                                  const int64_t *vofs, double *V, double *Wvec, int ldw,
                                                  double *alpha, double *beta, int mmax, int j,
                                                  const uint8_t *done)
{
    __shared__ double sh[33];
    extern __shared__ double sw[];   // [N] w, then [mmax] h
    const int bi = blockIdx.x;
    if (done[bi]) return;
    const int b = batch_blocks[bi];
    const int N = blk_ls[b + 1] - blk_ls[b];
    double *Vb = V + vofs[bi];
    double *h = sw + N;
    const double *vj = Vb + (size_t)j * N;
    for (int i = threadIdx.x; i < N; i += blockDim.x) sw[i] = Wvec[(size_t)bi * ldw + i];
    __syncthreads();
    double part = 0.0;
    for (int i = threadIdx.x; i < N; i += blockDim.x) part += sw[i] * vj[i];
    const double a = blk_sum(part, sh);
    const double bprev = j > 0 ? beta[(size_t)bi * mmax + j - 1] : 0.0;
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        double x = sw[i] - a * vj[i];
        if (j > 0) x -= bprev * Vb[(size_t)(j - 1) * N + i];
        sw[i] = x;
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int pass = 0; pass < 2; ++pass) {
        for (int t = warp; t <= j; t += nw) {
            const double *vt = Vb + (size_t)t * N;
            double s = 0.0;
            for (int i = lane; i < N; i += 32) s += vt[i] * sw[i];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if (lane == 0) h[t] = s;
        }
        __syncthreads();
        for (int i = threadIdx.x; i < N; i += blockDim.x) {
            double x = sw[i];
            for (int t = 0; t <= j; ++t) x -= h[t] * Vb[(size_t)t * N + i];
            sw[i] = x;
        }
        __syncthreads();
    }
    double ss = 0.0;
    for (int i = threadIdx.x; i < N; i += blockDim.x) ss += sw[i] * sw[i];
    const double bt = sqrt(blk_sum(ss, sh));
    if (threadIdx.x == 0) {
        alpha[(size_t)bi * mmax + j] = a;
        beta[(size_t)bi * mmax + j] = bt;
    }
    if (j + 1 < mmax && j + 1 < N) {
        double *vn = Vb + (size_t)(j + 1) * N;
        const double inv = bt > 0.0 ? 1.0 / bt : 0.0;
        for (int i = threadIdx.x; i < N; i += blockDim.x) vn[i] = sw[i] * inv;
    }
}

// M = d I - A in place (soda.f90:487-490)
__global__ void k_form_m(double *W, const int64_t *wofs, const int32_t *blk_ls,
                         const int32_t *batch_blocks, const double *xxd)
{
    const int b = batch_blocks[blockIdx.y];
    const int N = blk_ls[b + 1] - blk_ls[b];
    double *A = W + wofs[b];
    const double d = xxd[b];
    const size_t tot = (size_t)N * N;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < tot; t += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(t % N), j = (int)(t / N);
        const double v = -A[t];
        A[t] = i == j ? d + v : v;
    }
}

// ---------------------------------------------------------------------------
// blocked right-looking Cholesky M = U'U (upper), batched over subsets
// ---------------------------------------------------------------------------
constexpr int CB = 32;   // panel width

// factor the diagonal tile of panel kb; status[b] = failing row (1-based)
__global__ void __launch_bounds__(1024) k_chol_diag(double *W, const int64_t *wofs, const int32_t *blk_ls,
                                                    const int32_t *batch_blocks, int32_t *status, int kb)
{
    __shared__ double T[CB][CB + 1];
    __shared__ int s_fail;
    const int b = batch_blocks[blockIdx.x];
    const int N = blk_ls[b + 1] - blk_ls[b];
    if (kb >= N || status[b] != 0) return;
    const int nbk = min(CB, N - kb);
    double *A = W + wofs[b];
    const int r = threadIdx.x >> 5, c = threadIdx.x & 31;
    if (r < nbk && c < nbk) T[r][c] = A[(size_t)(kb + r) + (size_t)(kb + c) * N];
    if (threadIdx.x == 0) s_fail = 0;
    __syncthreads();
    for (int j = 0; j < nbk; ++j) {
        if (threadIdx.x == 0) {
            const double v = T[j][j];
            if (!(v > 0.0)) s_fail = kb + j + 1;
            else T[j][j] = sqrt(v);
        }
        __syncthreads();
        if (s_fail) break;
        if (r == 0 && c > j && c < nbk) T[j][c] = T[j][c] / T[j][j];
        __syncthreads();
        if (r > j && c >= r && c < nbk) T[r][c] -= T[j][r] * T[j][c];
        __syncthreads();
    }
    if (s_fail) {
        if (threadIdx.x == 0) status[b] = s_fail;
        return;
    }
    if (r < nbk && c < nbk && c >= r) A[(size_t)(kb + r) + (size_t)(kb + c) * N] = T[r][c];
}

// row panel: U[kb:kb+nbk, c] = U_kk'^{-1} M[kb:kb+nbk, c] for c >= kb+nbk
__global__ void __launch_bounds__(256) k_chol_trsm(double *W, const int64_t *wofs, const int32_t *blk_ls,
                                                   const int32_t *batch_blocks, const int32_t *status, int kb)
{
    __shared__ double T[CB][CB + 1];
    const int b = batch_blocks[blockIdx.y];
    const int N = blk_ls[b + 1] - blk_ls[b];
    if (kb >= N || status[b] != 0) return;
    const int nbk = min(CB, N - kb);
    double *A = W + wofs[b];
    for (int t = threadIdx.x; t < CB * CB; t += blockDim.x) {
        const int r = t % CB, c = t / CB;
        if (r < nbk && c < nbk) T[r][c] = A[(size_t)(kb + r) + (size_t)(kb + c) * N];
    }
    __syncthreads();
    const int col = kb + nbk + blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= N) return;
    double x[CB];
    double *ac = A + (size_t)col * N + kb;
#pragma unroll
    for (int r = 0; r < CB; ++r) x[r] = r < nbk ? ac[r] : 0.0;
#pragma unroll
    for (int r = 0; r < CB; ++r) {
        if (r < nbk) {
            double s = x[r];
#pragma unroll
            for (int t = 0; t < r; ++t) s -= T[t][r] * x[t];
            x[r] = s / T[r][r];
        }
    }
#pragma unroll
    for (int r = 0; r < CB; ++r)
        if (r < nbk) ac[r] = x[r];
}

// trailing update of the upper triangle: M[i,j] -= sum_t U[t,i] U[t,j]
constexpr int UT = 64;
__global__ void __launch_bounds__(256) k_chol_update(double *W, const int64_t *wofs, const int32_t *blk_ls,
                                                     const int32_t *batch_blocks, const int32_t *status, int kb)
{
    __shared__ double Pi[CB][UT + 1];
    __shared__ double Pj[CB][UT + 1];
    const int b = batch_blocks[blockIdx.y];
    const int N = blk_ls[b + 1] - blk_ls[b];
    if (status[b] != 0) return;
    const int k1 = kb + CB;
    if (k1 >= N) return;
    const int M = N - k1;
    const int nt = (M + UT - 1) / UT;
    int t = blockIdx.x, ti = 0;
    while (ti < nt && t >= nt - ti) { t -= nt - ti; ++ti; }
    if (ti >= nt) return;
    const int tj = ti + t;
    double *A = W + wofs[b];
    const int i0 = k1 + ti * UT, j0 = k1 + tj * UT;
    for (int q = threadIdx.x; q < CB * UT; q += blockDim.x) {
        const int r = q % CB, c = q / CB;
        const int ci = i0 + c, cj = j0 + c;
        Pi[r][c] = ci < N ? A[(size_t)(kb + r) + (size_t)ci * N] : 0.0;
        Pj[r][c] = cj < N ? A[(size_t)(kb + r) + (size_t)cj * N] : 0.0;
    }
    __syncthreads();
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    double acc[4][4] = {};
#pragma unroll 4
    for (int r = 0; r < CB; ++r) {
        double a[4], bb[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) { a[q] = Pi[r][ty + 16 * q]; bb[q] = Pj[r][tx + 16 * q]; }
#pragma unroll
        for (int q = 0; q < 4; ++q)
#pragma unroll
            for (int s = 0; s < 4; ++s) acc[q][s] += a[q] * bb[s];
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int i = i0 + ty + 16 * q;
        if (i >= N) continue;
#pragma unroll
        for (int s = 0; s < 4; ++s) {
            const int j = j0 + tx + 16 * s;
            if (j >= N || j < i) continue;
            A[(size_t)i + (size_t)j * N] -= acc[q][s];
        }
    }
}

// column lengths of PD subsets: column jj of the subset holds rows 0..jj
__global__ void k_pd_lengths(const int32_t *blk_ls, const int32_t *batch_blocks, const int32_t *status,
                             int32_t *ulen, uint8_t *skip)
{
    const int b = batch_blocks[blockIdx.y];
    if (status[b] != 0) return;
    const int ls = blk_ls[b], N = blk_ls[b + 1] - ls;
    for (int jj = blockIdx.x * blockDim.x + threadIdx.x; jj < N; jj += gridDim.x * blockDim.x) {
        ulen[ls + jj] = jj + 1;
        skip[ls + jj] = 0;
    }
}

// ---------------------------------------------------------------------------
// failed factorisation: the reference's sequence on one subset, one CTA.
// M (N x N) holds d I - A on entry (scratch, destroyed).  W_b receives the
// columns the reference leaves in XA(1:N, ls:le): rows of the unpivoted
// attempt before the failing row, overwritten by the pivoted factor.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(1024) k_psd_block(double *Wb, double *M, int N, int ls,
                                                    int32_t *ulen, uint8_t *skip, int32_t *piv_out,
                                                    int32_t *rank_out, int32_t *status_out, double *work)
{
    __shared__ double sh[33];
    __shared__ int s_fail, s_pvt, s_stop;
    __shared__ double s_ajj;
    const int tid = threadIdx.x;
    // (1) choleskyPD attempt (soda.f90:8-47), up-looking, into Wb
    if (tid == 0) s_fail = 0;
    __syncthreads();
    for (int i = tid; i < N; i += blockDim.x)
        if (M[(size_t)i * N + i] <= 0.0) s_fail = -1;
    __syncthreads();
    int ifail = 0;   // rows [0, ifail) of the attempt are written
    if (s_fail == 0) {
        for (size_t t = tid; t < (size_t)N * N; t += blockDim.x) Wb[t] = 0.0;
        __syncthreads();
        for (int i = 0; i < N; ++i) {
            double part = 0.0;
            for (int k = tid; k < i; k += blockDim.x) part += Wb[k + (size_t)i * N] * Wb[k + (size_t)i * N];
            const double dd = blk_sum(part, sh);
            const double tmp = M[i + (size_t)i * N] - dd;
            if (tmp <= 0.0 || isnan(tmp)) { ifail = i; break; }
            const double uii = sqrt(tmp);
            if (tid == 0) Wb[i + (size_t)i * N] = uii;
            for (int j = i + 1 + tid; j < N; j += blockDim.x) {
                double dj = 0.0;
                for (int k = 0; k < i; ++k) dj += Wb[k + (size_t)j * N] * Wb[k + (size_t)i * N];
                Wb[i + (size_t)j * N] = (M[j + (size_t)i * N] - dj) / uii;
            }
            __syncthreads();
            ifail = i + 1;
        }
    } else {
        for (size_t t = tid; t < (size_t)N * N; t += blockDim.x) Wb[t] = 0.0;
    }
    __syncthreads();
    // (2) choleskyPSD (soda.f90:49-124) on M in place
    double *wk = work;   // [2N]
    const double EPS = 2.220446049250313e-16;
    if (tid == 0) {
        int pvt = 0;
        double best = M[0];
        for (int t = 1; t < N; ++t)
            if (M[(size_t)t * N + t] > best) { best = M[(size_t)t * N + t]; pvt = t; }
        s_pvt = pvt;
        s_ajj = best;
        s_stop = 0;
    }
    for (int t = tid; t < N; t += blockDim.x) { piv_out[t] = t + 1; wk[t] = 0.0; }
    __syncthreads();
    if (s_ajj <= EPS) {
        if (tid == 0) { *status_out = -1; *rank_out = 0; }
        return;
    }
    const double DSTOP = N * EPS * s_ajj;
    int rank = N;
    for (int j = 0; j < N; ++j) {
        for (int p = j + tid; p < N; p += blockDim.x) {
            if (j > 0) wk[p] = wk[p] + M[(j - 1) + (size_t)p * N] * M[(j - 1) + (size_t)p * N];
            wk[N + p] = M[p + (size_t)p * N] - wk[p];
        }
        __syncthreads();
        if (tid == 0) {
            if (j > 0) {
                int pv = j;
                double best = wk[N + j];
                for (int p = j + 1; p < N; ++p)
                    if (wk[N + p] > best) { best = wk[N + p]; pv = p; }
                s_pvt = pv;
                s_ajj = best;
                if (best <= DSTOP) {
                    M[j + (size_t)j * N] = best;
                    s_stop = 1;
                }
            }
        }
        __syncthreads();
        if (s_stop) { rank = j; break; }
        const int pvt = s_pvt;
        if (j != pvt) {
            if (tid == 0) M[pvt + (size_t)pvt * N] = M[j + (size_t)j * N];
            __syncthreads();
            for (int t = tid; t < j; t += blockDim.x) {   // rows 0..j-1 of columns j and pvt
                const double a = M[t + (size_t)j * N];
                M[t + (size_t)j * N] = M[t + (size_t)pvt * N];
                M[t + (size_t)pvt * N] = a;
            }
            for (int t = tid; t < pvt - j - 1; t += blockDim.x) {   // row j (cols j+1..) <-> col pvt (rows j+1..)
                const double a = M[j + (size_t)(j + 1 + t) * N];
                M[j + (size_t)(j + 1 + t) * N] = M[(j + 1 + t) + (size_t)pvt * N];
                M[(j + 1 + t) + (size_t)pvt * N] = a;
            }
            for (int t = tid; t < N - pvt - 1; t += blockDim.x) {   // rows j and pvt, cols pvt+1..
                const double a = M[j + (size_t)(pvt + 1 + t) * N];
                M[j + (size_t)(pvt + 1 + t) * N] = M[pvt + (size_t)(pvt + 1 + t) * N];
                M[pvt + (size_t)(pvt + 1 + t) * N] = a;
            }
            if (tid == 0) {
                const double dt = wk[j];
                wk[j] = wk[pvt];
                wk[pvt] = dt;
                const int it = piv_out[pvt];
                piv_out[pvt] = piv_out[j];
                piv_out[j] = it;
            }
            __syncthreads();
        }
        const double ajj = sqrt(s_ajj);
        if (tid == 0) M[j + (size_t)j * N] = ajj;
        __syncthreads();
        if (j < N - 1) {
            const double sc = 1.0 / ajj;
            for (int jc = j + 1 + tid; jc < N; jc += blockDim.x) {
                double temp = 0.0;
                for (int i = 0; i < j; ++i) temp = temp + M[i + (size_t)jc * N] * M[i + (size_t)j * N];
                const double v = M[j + (size_t)jc * N] + (-1.0) * temp;
                M[j + (size_t)jc * N] = sc * v;
            }
        }
        __syncthreads();
    }
    __syncthreads();
    // (3) scatter: XA(1:j, ls+jj-1) = factor(1:j, j) for j <= rank, else skip
    for (int j = tid; j < N; j += blockDim.x) {
        const int jj = piv_out[j] - 1;   // 0-based subset column
        const int jj_stale = ifail < (jj + 1) ? ifail : (jj + 1);   // rows written by the attempt
        if (j < rank) {
            for (int i = 0; i <= j; ++i) Wb[i + (size_t)jj * N] = M[i + (size_t)j * N];
            ulen[ls + jj] = (j + 1) > jj_stale ? (j + 1) : jj_stale;
            skip[ls + jj] = 0;
        } else {
            // skipped column: XA keeps the rows of the unpivoted attempt
            ulen[ls + jj] = jj_stale;
            skip[ls + jj] = 1;
        }
    }
    if (tid == 0) { *rank_out = rank; *status_out = 0; }
}

// ---------------------------------------------------------------------------
// pack the factors into ragged columns in the sweep's precision
// ---------------------------------------------------------------------------
__global__ void k_pack(const double *W, const int64_t *wofs, const int32_t *blk_ls,
                       const int32_t *batch_blocks, const int64_t *uoff, const int32_t *ulen,
                       double *U64, float *U32, __nv_bfloat16 *Uhi, __nv_bfloat16 *Ulo)
{
    const int b = batch_blocks[blockIdx.y];
    const int ls = blk_ls[b], N = blk_ls[b + 1] - ls;
    const double *Wb = W + wofs[b];
    for (int jj = blockIdx.x; jj < N; jj += gridDim.x) {
        const int len = ulen[ls + jj];
        const int64_t off = uoff[ls + jj];
        for (int i = threadIdx.x; i < len; i += blockDim.x) {
            const double v = Wb[(size_t)i + (size_t)jj * N];
            if (U64) U64[off + i] = v;
            if (U32) U32[off + i] = (float)v;
            if (Uhi) {
                const __nv_bfloat16 hi = __double2bfloat16(v);
                const double rem = v - (double)__bfloat162float(hi);
                Uhi[off + i] = hi;
                Ulo[off + i] = __double2bfloat16(rem);
            }
        }
    }
}

// dense XA(bs, nloci) from the ragged columns (for inspection)
__global__ void k_unpack_dense(const double *U64, const int64_t *uoff, const int32_t *ulen, int p, int bs,
                               double *xa)
{
    const size_t tot = (size_t)p * bs;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < tot; t += (size_t)gridDim.x * blockDim.x) {
        const int k = (int)(t / bs), i = (int)(t % bs);
        xa[t] = i < ulen[k] ? U64[uoff[k] + i] : 0.0;
    }
}

// pred = mu + sum_k xv[k][G[k][i]] * eff[perm[k]], rows split over columns
__global__ void __launch_bounds__(256) k_dgv_partial(const int8_t *G, int ldx, const double *xv, const int32_t *perm,
                                                     const double *eff, int n, int p, int nsplit, double *part)
{
    const int i = blockIdx.x * 256 + threadIdx.x, s = blockIdx.y;
    if (i >= n) return;
    const int per = (p + nsplit - 1) / nsplit;
    const int k0 = s * per, k1 = min(p, k0 + per);
    double acc = 0.0;
    for (int k = k0; k < k1; ++k) {
        const double e = eff[perm ? perm[k] : k];
        if (e == 0.0) continue;
        const int code = G[(size_t)k * ldx + i];
        acc = acc + xv[(size_t)k * 4 + ((unsigned)code <= 2u ? code : 1)] * e;   // codes are validated on entry
    }
    part[(size_t)s * ldx + i] = acc;
}

__global__ void k_dgv_final(const double *part, int ldx, int n, int nsplit, double mu, double *pred)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double d = 0.0;
    for (int s = 0; s < nsplit; ++s) d = d + part[(size_t)s * ldx + i];
    pred[i] = mu + d;
}

// ---------------------------------------------------------------------------
// host wrappers
// ---------------------------------------------------------------------------
cudaError_t zb_decode_bed(const uint8_t *bed, int n, int p, int8_t *G, int ldx, cudaStream_t st)
{
    const size_t rec = ((size_t)n + 3) / 4;
    k_decode_bed<<<1024, 256, 0, st>>>(bed, n, p, rec, G, ldx);
    return cudaGetLastError();
}

cudaError_t zb_freq(int8_t *G, int n, int p, int ldx, double *freq, int *bad, cudaStream_t st)
{
    k_freq<<<(int)(((size_t)p * 32 + 255) / 256), 256, 0, st>>>(G, n, p, ldx, freq, bad);
    return cudaGetLastError();
}

cudaError_t zb_gather(const int8_t *Gsnp, int8_t *Gpos, const int32_t *perm, int p, int ldx, cudaStream_t st)
{
    k_gather<<<2048, 256, 0, st>>>(Gsnp, Gpos, perm, p, ldx);
    return cudaGetLastError();
}

cudaError_t zb_xv(const double *freq, const int32_t *perm, int p, double *xv, cudaStream_t st)
{
    k_xv<<<(p + 255) / 256, 256, 0, st>>>(freq, perm, p, xv);
    return cudaGetLastError();
}

cudaError_t zb_xv32(const double *xv, int p, float *xv32, cudaStream_t st)
{
    k_xv32<<<(4 * p + 255) / 256, 256, 0, st>>>(xv, p, xv32);
    return cudaGetLastError();
}

cudaError_t zb_x32(const int8_t *G, const double *xv, float *X32, int n, int p, int ldx, cudaStream_t st)
{
    k_x32<<<4096, 256, 0, st>>>(G, xv, X32, n, p, ldx);
    return cudaGetLastError();
}

cudaError_t zb_gram(const int8_t *G, int ldx, const int32_t *blk_ls, const int32_t *batch_blocks, int nbatch,
                    int maxN, const int64_t *wofs, const double *freq, const int32_t *perm, int n, double *W,
                    cudaStream_t st)
{
    const int nt = (maxN + GT - 1) / GT;
    k_gram<<<dim3(nt * (nt + 1) / 2, nbatch), 256, 0, st>>>(G, ldx, blk_ls, batch_blocks, wofs, freq, perm, n, W);
    return cudaGetLastError();
}

cudaError_t zb_lz_init(const int32_t *blk_ls, const int32_t *batch_blocks, int nbatch, const int64_t *vofs,
                       double *V, uint64_t seed, cudaStream_t st)
{
    k_lz_init<<<nbatch, 1024, 0, st>>>(blk_ls, batch_blocks, vofs, V, seed);
    return cudaGetLastError();
}

cudaError_t zb_lz_step(const double *W, const int64_t *wofs, const int32_t *blk_ls, const int32_t *batch_blocks,
                       int nbatch, int maxN, const int64_t *vofs, double *V, double *wvec, int ldw, double *alpha,
                       double *beta, int mmax, int j, const uint8_t *done, cudaStream_t st)
{
    k_lz_matvec<<<dim3((maxN + 127) / 128, nbatch), 128, sizeof(double) * maxN, st>>>(W, wofs, blk_ls, batch_blocks,
                                                                                      vofs, V, wvec, ldw, j);
    k_lz_orth<<<nbatch, 1024, sizeof(double) * (maxN + mmax), st>>>(blk_ls, batch_blocks, vofs, V, wvec, ldw, alpha,
                                                                    beta, mmax, j, done);
    return cudaGetLastError();
}

cudaError_t zb_lz_prepare(int maxN, int mmax)
{
    cudaError_t e = cudaFuncSetAttribute(k_lz_matvec, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)(sizeof(double) * maxN));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_lz_orth, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(sizeof(double) * (maxN + mmax)));
    return e;
}

cudaError_t zb_form_m(double *W, const int64_t *wofs, const int32_t *blk_ls, const int32_t *batch_blocks, int nbatch,
                      const double *xxd, cudaStream_t st)
{
    k_form_m<<<dim3(256, nbatch), 256, 0, st>>>(W, wofs, blk_ls, batch_blocks, xxd);
    return cudaGetLastError();
}

cudaError_t zb_cholesky(double *W, const int64_t *wofs, const int32_t *blk_ls, const int32_t *batch_blocks,
                        int nbatch, int maxN, int32_t *status, cudaStream_t st)
{
    for (int kb = 0; kb < maxN; kb += CB) {
        k_chol_diag<<<nbatch, 1024, 0, st>>>(W, wofs, blk_ls, batch_blocks, status, kb);
        const int rest = maxN - kb - CB;
        if (rest > 0) {
            k_chol_trsm<<<dim3((rest + 255) / 256, nbatch), 256, 0, st>>>(W, wofs, blk_ls, batch_blocks, status, kb);
            const int nt = (rest + UT - 1) / UT;
            k_chol_update<<<dim3(nt * (nt + 1) / 2, nbatch), 256, 0, st>>>(W, wofs, blk_ls, batch_blocks, status, kb);
        }
    }
    return cudaGetLastError();
}

cudaError_t zb_pd_lengths(const int32_t *blk_ls, const int32_t *batch_blocks, int nbatch, const int32_t *status,
                          int32_t *ulen, uint8_t *skip, cudaStream_t st)
{
    k_pd_lengths<<<dim3(8, nbatch), 256, 0, st>>>(blk_ls, batch_blocks, status, ulen, skip);
    return cudaGetLastError();
}

cudaError_t zb_psd_block(double *Wb, double *M, int N, int ls, int32_t *ulen, uint8_t *skip, int32_t *piv,
                         int32_t *rank, int32_t *status, double *work, cudaStream_t st)
{
    k_psd_block<<<1, 1024, 0, st>>>(Wb, M, N, ls, ulen, skip, piv, rank, status, work);
    return cudaGetLastError();
}

cudaError_t zb_pack(const double *W, const int64_t *wofs, const int32_t *blk_ls, const int32_t *batch_blocks,
                    int nbatch, const int64_t *uoff, const int32_t *ulen, double *U64, float *U32,
                    __nv_bfloat16 *Uhi, __nv_bfloat16 *Ulo, cudaStream_t st)
{
    k_pack<<<dim3(512, nbatch), 256, 0, st>>>(W, wofs, blk_ls, batch_blocks, uoff, ulen, U64, U32, Uhi, Ulo);
    return cudaGetLastError();
}

cudaError_t zb_unpack_dense(const double *U64, const int64_t *uoff, const int32_t *ulen, int p, int bs, double *xa,
                            cudaStream_t st)
{
    k_unpack_dense<<<2048, 256, 0, st>>>(U64, uoff, ulen, p, bs, xa);
    return cudaGetLastError();
}

cudaError_t zb_dgv(const int8_t *G, int ldx, const double *xv, const int32_t *perm, const double *eff, int n, int p,
                   double mu, double *part, int nsplit, double *pred, cudaStream_t st)
{
    k_dgv_partial<<<dim3((n + 255) / 256, nsplit), 256, 0, st>>>(G, ldx, xv, perm, eff, n, p, nsplit, part);
    k_dgv_final<<<(n + 255) / 256, 256, 0, st>>>(part, ldx, n, nsplit, mu, pred);
    return cudaGetLastError();
}

}  // namespace soda
