// Warp-per-instance layout of RNEA and ABA: the 32 lanes of a warp evaluate
// one configuration together (gb_warp.cuh), for batches too small to fill the
// GPU with one thread per configuration (a real-time controller's handful of
// states, a planner's few hundred).
#include <algorithm>

#include "gb_warp.cuh"

namespace gbi {
namespace {
using namespace warp;

constexpr int kWarpThreads = 256;  // 8 instances per CTA at most

__device__ __forceinline__ gb::MView stage_blob(const unsigned char* __restrict__ blob, int bytes,
                                                unsigned char* smem) {
  const uint4* src = reinterpret_cast<const uint4*>(blob);
  uint4* dst = reinterpret_cast<uint4*>(smem);
  for (int k = threadIdx.x; k < bytes / 16; k += blockDim.x) dst[k] = src[k];
  __syncthreads();
  return gb::make_view(smem);
}

template <class S>
__global__ void __launch_bounds__(kWarpThreads) k_rnea_warp(const unsigned char* blob, int bytes, long B, Arr q,
                                                             Arr v, Arr a, Arr tau) {
  extern __shared__ __align__(16) unsigned char smem[];
  const gb::MView m = stage_blob(blob, bytes, smem);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  S* ws = reinterpret_cast<S*>(smem + align16(bytes)) + (long)warp * rnea_words<S>() * m.nj;
  for (long b = (long)blockIdx.x * nw + warp; b < B; b += (long)gridDim.x * nw) {
    rnea_warp_one<S>(m, w_in(q, b), w_in(v, b), w_in(a, b), w_out(tau, b), ws, lane);
    __syncwarp();
  }
}

template <class S, class SS>
__global__ void __launch_bounds__(kWarpThreads) k_aba_warp(const unsigned char* blob, int bytes, long B, Arr q,
                                                            Arr v, Arr tau, Arr ddq) {
  extern __shared__ __align__(16) unsigned char smem[];
  const gb::MView m = stage_blob(blob, bytes, smem);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const size_t per_s = align16(sizeof(S) * aba_words_s<S, SS>() * (size_t)m.nj);
  const size_t per_ss = align16(sizeof(SS) * ((size_t)m.nj + 78));
  unsigned char* base = smem + align16(bytes) + (size_t)warp * (per_s + per_ss);
  S* ws = reinterpret_cast<S*>(base);
  SS* wss = reinterpret_cast<SS*>(base + per_s);
  for (long b = (long)blockIdx.x * nw + warp; b < B; b += (long)gridDim.x * nw) {
    aba_warp_one<S, SS>(m, w_in(q, b), w_in(v, b), w_in(tau, b), w_out(ddq, b), ws, wss, lane);
    __syncwarp();
  }
}

// warps per CTA that fit the shared-memory budget (blob + per-warp regions), and the launch
template <class Kern>
int warp_launch_shape(const gb_model* M, size_t per_warp, Kern kernel, const char* name, int* nw, size_t* smem) {
  const size_t limit = 200 * 1024;
  const size_t blob = align16((size_t)M->stage_bytes);
  if (blob + per_warp > limit) return set_error(GB_ERR_UNSUPPORTED, std::string(name) + ": model too large for the warp layout");
  *nw = (int)std::min<size_t>(kWarpThreads / 32, (limit - blob) / per_warp);
  *smem = blob + (size_t)(*nw) * per_warp;
  if (*smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)*smem);
    if (e != cudaSuccess) return cuda_error(e, name);
  }
  return GB_OK;
}

template <class S>
int launch_rnea_warp_t(const gb_model* M, long B, Arr q, Arr v, Arr a, Arr tau, cudaStream_t st) {
  int nw;
  size_t smem;
  const size_t per_warp = rnea_warp_bytes<S>(M->nj);
  int rc = warp_launch_shape(M, per_warp, k_rnea_warp<S>, "k_rnea_warp", &nw, &smem);
  if (rc != GB_OK) return rc;
  const long grid = std::min<long>((B + nw - 1) / nw, 152L * 16);
  k_rnea_warp<S><<<(unsigned)grid, 32 * nw, smem, st>>>(M->d_blob, M->stage_bytes, B, q, v, a, tau);
  return cuda_error(cudaGetLastError(), "k_rnea_warp");
}

template <class S, class SS>
int launch_aba_warp_t(const gb_model* M, long B, Arr q, Arr v, Arr tau, Arr ddq, cudaStream_t st) {
  int nw;
  size_t smem;
  const size_t per_warp = aba_warp_bytes<S, SS>(M->nj);
  int rc = warp_launch_shape(M, per_warp, k_aba_warp<S, SS>, "k_aba_warp", &nw, &smem);
  if (rc != GB_OK) return rc;
  const long grid = std::min<long>((B + nw - 1) / nw, 152L * 16);
  k_aba_warp<S, SS><<<(unsigned)grid, 32 * nw, smem, st>>>(M->d_blob, M->stage_bytes, B, q, v, tau, ddq);
  return cuda_error(cudaGetLastError(), "k_aba_warp");
}

}  // namespace

int launch_rnea_warp(const gb_model* M, int precision, long B, Arr q, Arr v, Arr a, Arr tau, cudaStream_t st) {
  if (precision == GB_FP64) return launch_rnea_warp_t<double>(M, B, q, v, a, tau, st);
  return launch_rnea_warp_t<float>(M, B, q, v, a, tau, st);
}

int launch_aba_warp(const gb_model* M, int precision, long B, Arr q, Arr v, Arr tau, Arr ddq, cudaStream_t st) {
  if (precision == GB_FP64) return launch_aba_warp_t<double, double>(M, B, q, v, tau, ddq, st);
  return launch_aba_warp_t<float, double>(M, B, q, v, tau, ddq, st);
}

}  // namespace gbi
