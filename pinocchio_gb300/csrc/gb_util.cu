// Device scratch from the stream-ordered memory pool, and the SOA -> instance
// transpose that lets the per-thread kernels write their nv x nv matrices
// coalesced ([element][configuration]: a warp's 32 configurations side by
// side) when the caller asked for the reference's instance layout (every
// configuration's matrix contiguous), instead of 32 scattered 8-byte stores
// per warp instruction.
#include "gb_internal.h"

namespace gbi {

int scratch_alloc(void** p, size_t bytes, cudaStream_t st) {
  static bool pool_tuned = false;
  if (!pool_tuned) {  // keep freed blocks in the pool: repeated calls reuse them
    int dev = 0;
    cudaMemPool_t pool;
    if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
      unsigned long long thr = ~0ull;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    pool_tuned = true;
  }
  *p = nullptr;
  return cuda_error(cudaMallocAsync(p, bytes, st), "workspace allocation");
}

void scratch_free(void* p, cudaStream_t st) {
  if (p) cudaFreeAsync(p, st);
}

namespace {
// 32 elements x 32 configurations per CTA through shared memory: reads along the
// configurations, writes along the elements, both coalesced
__global__ void __launch_bounds__(256) k_soa_to_instance(const double* __restrict__ src, long B, long n,
                                                          double* __restrict__ dst, long is) {
  __shared__ double tile[32][33];
  const long e0 = (long)blockIdx.y * 32, b0 = (long)blockIdx.x * 32;
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const long e = e0 + k, b = b0 + threadIdx.x;
    if (e < n && b < B) tile[k][threadIdx.x] = src[e * B + b];
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const long b = b0 + k, e = e0 + threadIdx.x;
    if (e < n && b < B) dst[b * is + e] = tile[threadIdx.x][k];
  }
}
}  // namespace

int launch_soa_to_instance(const double* src, long B, long n, Arr dst, cudaStream_t st) {
  if (B == 0 || n == 0) return GB_OK;
  if (dst.es != 1) return set_error(GB_ERR_INVALID_ARGUMENT, "transpose target must be the instance layout");
  const dim3 grid((unsigned)((B + 31) / 32), (unsigned)((n + 31) / 32)), block(32, 8);
  k_soa_to_instance<<<grid, block, 0, st>>>(src, B, n, const_cast<double*>(dst.p), dst.is);
  return cuda_error(cudaGetLastError(), "k_soa_to_instance");
}

}  // namespace gbi
