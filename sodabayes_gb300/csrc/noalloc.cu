// noalloc.cu — genomic values pred = mu + X * effects without any allocation.
//
// Some hosts cannot let this library allocate device memory: a Fortran or C
// host that already owns the GPU through its own memory pool (CUDA Fortran /
// OpenACC runtimes, frameworks with caching allocators), or a latency-bound
// loop that must not pay cudaMalloc/cudaFree and the device-wide
// synchronisation they can imply.  For them sodagpu_compute_dgv_noalloc
// computes the same values as compute_dgv (utilities.f90:616-622, with the
// centring of xscale, utilities.f90:545-552) from device buffers the caller
// owns, using as scratch only the fixed array below.
//
// The scratch is a file-scope __device__ array of SODAGPU_NOALLOC_SCRATCH
// doubles (16 MiB): every GPU that loads this library keeps it until the
// process exits.  Host code cannot use the array's name as a device address,
// so the first call on each device looks the address up with
// cudaGetSymbolAddress (with that device current) and caches it; later calls
// reuse it.  Every call shares the one array: calls that overlap on the GPU
// (different streams, or different host threads on the same device) race on
// it and must be serialised by the caller.  cudaDeviceReset destroys the
// context that holds the array; the cached address is then stale, so a host
// that resets a device must not call this entry point on it again in the
// same process.
//
// The columns are summed in nsplit = min(32, SCRATCH / nind, nloci) splits,
// the same 32 as sodagpu_predict up to nind = 65,536; above that the
// summation order differs and so can the last bits of the result.  Codes
// outside 0..2 count as 1, the value load_geno gives a missing call
// (utilities.f90:446-449); sodagpu_predict rejects them instead.
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "../../include/sodagpu.h"

namespace {

constexpr int kSplitMax = 32;     // column splits of the partial sums
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_dgv_scratch[SODAGPU_NOALLOC_SCRATCH];

std::mutex g_scratch_mu;
double *g_scratch_ptr[kMaxDevices];   // device address per device, 0 until looked up

// partial[s][i] = sum over the columns of split s of x_ij * effects_j, with
// x_ij = (code - 2p_j) / sqrt(2p_j(1-p_j)) (0 for monomorphic SNPs); the
// three values of each column are formed in shared memory per chunk.
__global__ void __launch_bounds__(256) k_dgv_noalloc_partial(const int8_t *codes, int ldg, const double *freq,
                                                             const double *eff, int n, int p, int nsplit,
                                                             double *part)
{
    __shared__ double s_x[256][3];
    __shared__ double s_e[256];
    const int i = blockIdx.x * 256 + threadIdx.x, s = blockIdx.y;
    const int per = (p + nsplit - 1) / nsplit;
    const int k0 = s * per, k1 = min(p, k0 + per);
    const double eps = 2.220446049250313e-16;
    double acc = 0.0;
    for (int c0 = k0; c0 < k1; c0 += 256) {
        const int cnt = min(256, k1 - c0);
        __syncthreads();
        if (threadIdx.x < cnt) {
            const int k = c0 + threadIdx.x;
            const double f = freq[k];
            s_e[threadIdx.x] = eff[k];
            if (f < eps || (1.0 - f) < eps) {
                s_x[threadIdx.x][0] = s_x[threadIdx.x][1] = s_x[threadIdx.x][2] = 0.0;
            } else {
                const double twop = __dmul_rn(2.0, f);
                const double sd = sqrt(__dmul_rn(twop, __dsub_rn(1.0, f)));
                s_x[threadIdx.x][0] = __ddiv_rn(__dsub_rn(0.0, twop), sd);
                s_x[threadIdx.x][1] = __ddiv_rn(__dsub_rn(1.0, twop), sd);
                s_x[threadIdx.x][2] = __ddiv_rn(__dsub_rn(2.0, twop), sd);
            }
        }
        __syncthreads();
        if (i < n) {
            for (int q = 0; q < cnt; ++q) {
                const double e = s_e[q];
                if (e == 0.0) continue;
                const int code = codes[(size_t)(c0 + q) * ldg + i];
                acc = acc + s_x[q][code < 0 ? 1 : (code > 2 ? 1 : code)] * e;
            }
        }
    }
    if (i < n) part[(size_t)s * n + i] = acc;
}

__global__ void k_dgv_noalloc_final(const double *part, int n, int nsplit, double mu, double *pred)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double d = 0.0;
    for (int s = 0; s < nsplit; ++s) d = d + part[(size_t)s * n + i];
    pred[i] = mu + d;
}

}  // namespace

extern "C" int sodagpu_compute_dgv_noalloc(int32_t nind, int32_t nloci, const int8_t *codes, int32_t ldg,
                                           const double *freq, double mu, const double *effects, double *pred,
                                           void *stream)
{
    if (nind < 1 || nloci < 1 || ldg < nind || !codes || !freq || !effects || !pred) return SODAGPU_E_ARG;
    if ((int64_t)nind > (int64_t)SODAGPU_NOALLOC_SCRATCH) return SODAGPU_E_ARG;   // beyond the scratch maximum
    int nsplit = (int)((int64_t)SODAGPU_NOALLOC_SCRATCH / nind);
    nsplit = nsplit > kSplitMax ? kSplitMax : nsplit;
    nsplit = nsplit > nloci ? nloci : nsplit;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return SODAGPU_E_NODEVICE;
    }
    if (dev < 0 || dev >= kMaxDevices) return SODAGPU_E_UNSUPPORTED;
    double *scratch = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_scratch_mu);
        if (!g_scratch_ptr[dev]) {
            void *ptr = nullptr;
            const cudaError_t e = cudaGetSymbolAddress(&ptr, g_dgv_scratch);
            if (e != cudaSuccess || !ptr) {
                cudaGetLastError();
                return SODAGPU_E_CUDA;
            }
            g_scratch_ptr[dev] = (double *)ptr;
        }
        scratch = g_scratch_ptr[dev];
    }
    // cudaLaunchKernel reports a failed launch in its own return value, so an error the caller left
    // pending from earlier work is neither reported as this call's failure nor cleared
    cudaStream_t st = (cudaStream_t)stream;
    {
        void *args[] = {(void *)&codes, (void *)&ldg, (void *)&freq, (void *)&effects, (void *)&nind,
                        (void *)&nloci, (void *)&nsplit, (void *)&scratch};
        if (cudaLaunchKernel((const void *)k_dgv_noalloc_partial, dim3((nind + 255) / 256, nsplit), dim3(256), args,
                             0, st) != cudaSuccess) {
            cudaGetLastError();
            return SODAGPU_E_CUDA;
        }
    }
    {
        const double *part = scratch;
        void *args[] = {(void *)&part, (void *)&nind, (void *)&nsplit, (void *)&mu, (void *)&pred};
        if (cudaLaunchKernel((const void *)k_dgv_noalloc_final, dim3((nind + 255) / 256), dim3(256), args, 0, st) !=
            cudaSuccess) {
            cudaGetLastError();
            return SODAGPU_E_CUDA;
        }
    }
    return 0;
}
