// zbuild.cuh — host entry points of the Z-build and genotype kernels (zbuild.cu).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace soda {

cudaError_t zb_decode_bed(const uint8_t *bed, int n, int p, int8_t *G, int ldx, cudaStream_t st);
cudaError_t zb_freq(int8_t *G, int n, int p, int ldx, double *freq, int *bad, cudaStream_t st);
cudaError_t zb_gather(const int8_t *Gsnp, int8_t *Gpos, const int32_t *perm, int p, int ldx, cudaStream_t st);
cudaError_t zb_xv(const double *freq, const int32_t *perm, int p, double *xv, cudaStream_t st);
cudaError_t zb_xv32(const double *xv, int p, float *xv32, cudaStream_t st);
cudaError_t zb_x32(const int8_t *G, const double *xv, float *X32, int n, int p, int ldx, cudaStream_t st);
cudaError_t zb_gram(const int8_t *G, int ldx, const int32_t *blk_ls, const int32_t *batch_blocks, int nbatch,
                    int maxN, const int64_t *wofs, const double *freq, const int32_t *perm, int n, double *W,
                    cudaStream_t st);
cudaError_t zb_lz_prepare(int maxN, int mmax);
cudaError_t zb_lz_init(const int32_t *blk_ls, const int32_t *batch_blocks, int nbatch, const int64_t *vofs,
                       double *V, uint64_t seed, cudaStream_t st);
cudaError_t zb_lz_step(const double *W, const int64_t *wofs, const int32_t *blk_ls, const int32_t *batch_blocks,
                       int nbatch, int maxN, const int64_t *vofs, double *V, double *wvec, int ldw, double *alpha,
                       double *beta, int mmax, int j, const uint8_t *done, cudaStream_t st);
cudaError_t zb_form_m(double *W, const int64_t *wofs, const int32_t *blk_ls, const int32_t *batch_blocks, int nbatch,
                      const double *xxd, cudaStream_t st);
cudaError_t zb_cholesky(double *W, const int64_t *wofs, const int32_t *blk_ls, const int32_t *batch_blocks,
                        int nbatch, int maxN, int32_t *status, cudaStream_t st);
cudaError_t zb_pd_lengths(const int32_t *blk_ls, const int32_t *batch_blocks, int nbatch, const int32_t *status,
                          int32_t *ulen, uint8_t *skip, cudaStream_t st);
cudaError_t zb_psd_block(double *Wb, double *M, int N, int ls, int32_t *ulen, uint8_t *skip, int32_t *piv,
                         int32_t *rank, int32_t *status, double *work, cudaStream_t st);
cudaError_t zb_pack(const double *W, const int64_t *wofs, const int32_t *blk_ls, const int32_t *batch_blocks,
                    int nbatch, const int64_t *uoff, const int32_t *ulen, double *U64, float *U32,
                    __nv_bfloat16 *Uhi, __nv_bfloat16 *Ulo, cudaStream_t st);
cudaError_t zb_unpack_dense(const double *U64, const int64_t *uoff, const int32_t *ulen, int p, int bs, double *xa,
                            cudaStream_t st);
cudaError_t zb_dgv(const int8_t *G, int ldx, const double *xv, const int32_t *perm, const double *eff, int n, int p,
                   double mu, double *part, int nsplit, double *pred, cudaStream_t st);

}  // namespace soda
