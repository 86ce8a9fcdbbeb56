// update_kernel.cuh — residual update of one subset, included by sweep.cu:
//   r  += X_b delta   (rows of the residual)
//   ra += U_b delta   (rows of the augmented residual)      (models.f90:164-174)
// Only the positions whose delta is non-zero in some chain contribute; every
// CTA compacts their list in subset order.  A CTA owns UT = 128 rows of r (or
// of ra) and all listed columns: warp w of NW takes the columns w, w+NW, ...
// and lane l the rows 4l..4l+3, so each column is one coalesced 128-byte (or
// 512-byte) line, loaded UNR columns at a time for memory-level parallelism.
// The NW warps' partial sums are added in warp order in shared memory
// (deterministic), then added to the FP64 master residual.  FP64 mode
// accumulates in FP64, the FP32/FP8 modes in FP32.
#pragma once

namespace soda {

constexpr int UT = 128;     // rows per CTA
constexpr int UNR = 8;      // columns in flight per warp

// warps per CTA: enough to hide the load latency with few chains, fewer
// (with more FMAs each) with many chains
template <int MODE, int CT>
struct UpdWarps { static constexpr int v = MODE == SODAGPU_FP64 ? 8 : (CT <= 2 ? 32 : (CT <= 4 ? 16 : 8)); };

__host__ __device__ inline size_t update_list_bytes(int bs) { return ((sizeof(int) * ((size_t)bs + 32)) + 15) & ~(size_t)15; }

template <int MODE, int CT>
static inline size_t update_smem_bytes_ct(int bs)
{
    const size_t acc = MODE == SODAGPU_FP64 ? 8 : 4;
    return update_list_bytes(bs) + UpdWarps<MODE, CT>::v * (size_t)CT * UT * acc;
}

template <int MODE, int CT>
__device__ __forceinline__ void update_body(const Dev &D, const VB &vb, int b)
{
    typedef typename std::conditional<MODE == SODAGPU_FP64, double, float>::type acc_t;
    constexpr int NW = UpdWarps<MODE, CT>::v;
    extern __shared__ __align__(16) unsigned char smem[];
    int *s_list = reinterpret_cast<int *>(smem);
    acc_t *s_red = reinterpret_cast<acc_t *>(smem + update_list_bytes(D.bs));   // [NW][CT][UT]
    __shared__ int s_wcnt[NW + 1];
    __shared__ int s_n;
    __shared__ double sh[33];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    tc::pdl_trigger();
    tc::pdl_wait();
    const int ls = D.blk_ls[b];
    const int N = D.blk_ls[b + 1] - ls;
    const int npad = (N + 7) & ~7;
    // positions with a non-zero delta in any chain, in subset order
    if (tid == 0) s_n = 0;
    __syncthreads();
    for (int base = 0; base < N; base += 32 * NW) {
        const int jk = base + tid;
        const bool f = jk < N && D.nzflag[jk];
        const unsigned m = __ballot_sync(0xffffffffu, f);
        if (lane == 0) s_wcnt[w] = __popc(m);
        __syncthreads();
        if (tid == 0) {
            int acc = s_n;
            for (int q = 0; q < NW; ++q) {
                const int t = s_wcnt[q];
                s_wcnt[q] = acc;
                acc += t;
            }
            s_wcnt[NW] = acc;
        }
        __syncthreads();
        if (f) s_list[s_wcnt[w] + __popc(m & ((1u << lane) - 1u))] = jk;
        __syncthreads();
        if (tid == 0) s_n = s_wcnt[NW];
        __syncthreads();
    }
    const int nlist = s_n;
    if (nlist == 0) return;   // nothing changed: r, r32 and rsum stay valid
    const int ntile_r = D.nr_ctas;
    const bool rows = (int)vb.x < ntile_r;
    const int t0 = (rows ? vb.x : vb.x - ntile_r) * UT;
    const int nrow = rows ? D.n : D.bs;
    const int i0 = t0 + lane * 4;

    acc_t acc[4][CT];
#pragma unroll
    for (int e = 0; e < 4; ++e)
#pragma unroll
        for (int c = 0; c < CT; ++c) acc[e][c] = 0;
    // columns w, w+NW, ... of the list, UNR at a time; every load of a column
    // (codes, its three x values, the deltas) is independent of the others
    for (int q0 = w; q0 < nlist; q0 += NW * UNR) {
        acc_t x[UNR][4];
        int kk[UNR];
#pragma unroll
        for (int u = 0; u < UNR; ++u) kk[u] = q0 + NW * u < nlist ? s_list[q0 + NW * u] : -1;
#pragma unroll
        for (int u = 0; u < UNR; ++u) {
            x[u][0] = x[u][1] = x[u][2] = x[u][3] = 0;
            if (kk[u] < 0 || i0 >= nrow) continue;
            const int k = ls + kk[u];
            if (rows) {
                if (MODE == SODAGPU_FP32) {
                    const float4 v = *reinterpret_cast<const float4 *>(D.X32 + (size_t)k * D.ldx + i0);
                    x[u][0] = v.x; x[u][1] = v.y; x[u][2] = v.z; x[u][3] = v.w;
                } else {
                    const uint32_t wv = *reinterpret_cast<const uint32_t *>(D.G + (size_t)k * D.ldx + i0);
                    acc_t x0, x1, x2;
                    if (MODE == SODAGPU_FP64) {
                        const double2 x01 = *reinterpret_cast<const double2 *>(D.xv + (size_t)k * 4);
                        x0 = (acc_t)x01.x;
                        x1 = (acc_t)x01.y;
                        x2 = (acc_t)D.xv[(size_t)k * 4 + 2];
                    } else {   // FP32 table: no FP64-pipe conversions in the inner loop
                        const float4 xf = *reinterpret_cast<const float4 *>(D.xv32 + (size_t)k * 4);
                        x0 = (acc_t)xf.x;
                        x1 = (acc_t)xf.y;
                        x2 = (acc_t)xf.z;
                    }
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        const uint32_t code = (wv >> (8 * e)) & 3u;
                        x[u][e] = code == 0u ? x0 : (code == 1u ? x1 : x2);
                    }
                }
            } else if (i0 + 4 <= npad) {
                const int64_t o = D.uoff[k] + i0;
                if (MODE == SODAGPU_FP64) {
                    const double2 a = *reinterpret_cast<const double2 *>(D.U64 + o);
                    const double2 bq = *reinterpret_cast<const double2 *>(D.U64 + o + 2);
                    x[u][0] = a.x; x[u][1] = a.y; x[u][2] = bq.x; x[u][3] = bq.y;
                } else {
                    const float4 v = *reinterpret_cast<const float4 *>(D.U32 + o);
                    x[u][0] = v.x; x[u][1] = v.y; x[u][2] = v.z; x[u][3] = v.w;
                }
            }
        }
#pragma unroll
        for (int u = 0; u < UNR; ++u) {
            if (kk[u] < 0) continue;
            acc_t dl[CT];
            if (MODE == SODAGPU_FP64) {
#pragma unroll
                for (int c = 0; c < CT; ++c) dl[c] = (acc_t)D.delta[(size_t)c * D.bs + kk[u]];
            } else if (CT >= 4) {   // chain-contiguous FP32 copy: 16-byte loads
#pragma unroll
                for (int c = 0; c < CT; c += 4) {
                    const float4 v = *reinterpret_cast<const float4 *>(D.delta32 + (size_t)kk[u] * CT + c);
                    dl[c] = v.x; dl[c + 1] = v.y; dl[c + 2] = v.z; dl[c + 3] = v.w;
                }
            } else {
#pragma unroll
                for (int c = 0; c < CT; ++c) dl[c] = D.delta32[(size_t)kk[u] * CT + c];
            }
#pragma unroll
            for (int c = 0; c < CT; ++c)
#pragma unroll
                for (int e = 0; e < 4; ++e) acc[e][c] += x[u][e] * dl[c];
        }
    }
    // the warps' partial sums, added in warp order
#pragma unroll
    for (int c = 0; c < CT; ++c)
#pragma unroll
        for (int e = 0; e < 4; ++e) s_red[((size_t)w * CT + c) * UT + lane * 4 + e] = acc[e][c];
    __syncthreads();
    for (int c = 0; c < CT; ++c) {
        double v = 0.0;
        const int rl = tid;                 // row within the tile (tid < UT)
        const int i = t0 + rl;
        if (tid < UT && i < nrow) {
            acc_t dsum = 0;   // the warps' partial sums, in warp order
#pragma unroll
            for (int ww = 0; ww < NW; ++ww) dsum += s_red[((size_t)ww * CT + c) * UT + rl];
            const double d = (double)dsum;
            if (rows) {
                v = D.r[(size_t)c * D.ldr + i] + d;
                store_r(D, c, i, v);
            } else {
                store_ra(D, c, i, D.ra[(size_t)c * D.ldra + i] + d);
            }
        }
        if (MODE == SODAGPU_FP8 && rows) {
            // refresh this tile's partial sum of r (the centring of the next subset)
            const double t = block_sum(v, sh);
            if (tid == 0) D.rsum[(size_t)c * D.nr_ctas + vb.x] = t;
        }
    }
}

template <int MODE, int CT>
__global__ void __launch_bounds__(32 * UpdWarps<MODE, CT>::v) k_update(Dev D, int b)
{
    update_body<MODE, CT>(D, vb_native(), b);
}


}  // namespace soda
