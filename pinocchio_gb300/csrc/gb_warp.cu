// Warp-per-instance and lane-per-branch layouts of RNEA and ABA (gb_warp.cuh):
// the 32 lanes of a warp, or a team of 4-32 lanes (one per chain of the tree),
// evaluate one configuration together, for batches too small to fill the GPU
// with one thread per configuration (a real-time controller's handful of
// states, a planner's few hundred or thousand).
#include <algorithm>

#include "gb_warp.cuh"

namespace gbi {
namespace {
using namespace warp;

constexpr int kWarpThreads = 256;  // 8 instances per CTA at most
// the RNEA warp layout gathers children's forces by warp shuffles (1) or shared memory (0)
#ifndef GB_WARP_SHFL
#define GB_WARP_SHFL 0
#endif

__device__ __forceinline__ gb::MView stage_blob(const unsigned char* __restrict__ blob, int bytes,
                                                unsigned char* smem) {
  const uint4* src = reinterpret_cast<const uint4*>(blob);
  uint4* dst = reinterpret_cast<uint4*>(smem);
  for (int k = threadIdx.x; k < bytes / 16; k += blockDim.x) dst[k] = src[k];
  __syncthreads();
  gb::MView m = gb::make_view(smem);
  gb::attach_status(m, blob);
  return m;
}

template <class S, bool SHFL>
__global__ void __launch_bounds__(kWarpThreads) k_rnea_warp(const unsigned char* blob, int bytes, long B, Arr q,
                                                             Arr v, Arr a, Arr tau) {
  extern __shared__ __align__(16) unsigned char smem[];
  const gb::MView m = stage_blob(blob, bytes, smem);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  S* ws = reinterpret_cast<S*>(smem + align16(bytes)) + (long)warp * rnea_words<S>() * m.nj;
  for (long b = (long)blockIdx.x * nw + warp; b < B; b += (long)gridDim.x * nw) {
    rnea_warp_one<S, LevelSched, SHFL>(m, w_in(q, b), w_in(v, b), w_in(a, b), w_out(tau, b), ws, LevelSched{lane});
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
    aba_warp_one<S, SS>(m, w_in(q, b), w_in(v, b), w_in(tau, b), w_out(ddq, b), ws, wss, LevelSched{lane});
    __syncwarp();
  }
}

// Lane-per-branch layout: a team of TS lanes per configuration (BranchSched), teams of one
// CTA share the staged model, each team its shared-memory region.
template <int TS> __device__ __forceinline__ unsigned team_mask() {
  return TS == 32 ? 0xffffffffu : ((1u << TS) - 1u) << ((threadIdx.x & 31) & ~(TS - 1));
}
template <class S, int TS>
__global__ void __launch_bounds__(kWarpThreads) k_rnea_branch(const unsigned char* blob, int bytes, long B, Arr q,
                                                               Arr v, Arr a, Arr tau, int region_bytes) {
  extern __shared__ __align__(16) unsigned char smem[];
  const gb::MView m = stage_blob(blob, bytes, smem);
  const int team = threadIdx.x / TS, nt = blockDim.x / TS;
  const BranchSched<TS> sc{(int)(threadIdx.x % TS), team_mask<TS>()};
  S* ws = reinterpret_cast<S*>(smem + align16(bytes) + (size_t)team * region_bytes);
  for (long b = (long)blockIdx.x * nt + team; b < B; b += (long)gridDim.x * nt) {
    rnea_warp_one<S>(m, w_in(q, b), w_in(v, b), w_in(a, b), w_out(tau, b), ws, sc);
    sc.sync();
  }
}
template <class S, class SS, int TS>
__global__ void __launch_bounds__(kWarpThreads) k_aba_branch(const unsigned char* blob, int bytes, long B, Arr q,
                                                              Arr v, Arr tau, Arr ddq, int region_bytes) {
  extern __shared__ __align__(16) unsigned char smem[];
  const gb::MView m = stage_blob(blob, bytes, smem);
  const int team = threadIdx.x / TS, nt = blockDim.x / TS;
  const BranchSched<TS> sc{(int)(threadIdx.x % TS), team_mask<TS>()};
  const size_t per_s = align16(sizeof(S) * aba_words_s<S, SS>() * (size_t)m.nj);
  unsigned char* base = smem + align16(bytes) + (size_t)team * region_bytes;
  for (long b = (long)blockIdx.x * nt + team; b < B; b += (long)gridDim.x * nt) {
    aba_warp_one<S, SS>(m, w_in(q, b), w_in(v, b), w_in(tau, b), w_out(ddq, b), reinterpret_cast<S*>(base),
                        reinterpret_cast<SS*>(base + per_s), sc);
    sc.sync();
  }
}

// teams per CTA (a multiple of the teams of one warp) that fit the shared-memory budget, and the launch
template <class Kern>
int branch_launch_shape(const gb_model* M, int ts, size_t region, Kern kernel, const char* name, int* threads,
                        size_t* smem) {
  const size_t limit = 200 * 1024;
  const size_t blob = align16((size_t)M->stage_bytes);
  if (blob + region > limit) return set_error(GB_ERR_UNSUPPORTED, std::string(name) + ": model too large for the branch layout");
  const int per_warp = 32 / ts;
  int teams = (int)std::min<size_t>(kWarpThreads / ts, (limit - blob) / region);
  if (teams >= per_warp) teams -= teams % per_warp;  // whole warps when they fit, else part of one
  *threads = teams * ts;
  *smem = blob + (size_t)teams * region;
  if (*smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)*smem);
    if (e != cudaSuccess) return cuda_error(e, name);
  }
  return GB_OK;
}

template <class S, int TS>
int launch_rnea_branch_t(const gb_model* M, long B, Arr q, Arr v, Arr a, Arr tau, cudaStream_t st) {
  int threads;
  size_t smem;
  const size_t region = rnea_warp_bytes<S>(M->nj);
  int rc = branch_launch_shape(M, TS, region, k_rnea_branch<S, TS>, "k_rnea_branch", &threads, &smem);
  if (rc != GB_OK) return rc;
  const int teams = threads / TS;
  const long grid = std::min<long>((B + teams - 1) / teams, (long)M->sm_count * 16);
  k_rnea_branch<S, TS><<<(unsigned)grid, threads, smem, st>>>(M->d_blob, M->stage_bytes, B, q, v, a, tau, (int)region);
  return cuda_error(cudaGetLastError(), "k_rnea_branch");
}
template <class S, class SS, int TS>
int launch_aba_branch_t(const gb_model* M, long B, Arr q, Arr v, Arr tau, Arr ddq, cudaStream_t st) {
  int threads;
  size_t smem;
  const size_t region = aba_warp_bytes<S, SS>(M->nj);
  int rc = branch_launch_shape(M, TS, region, k_aba_branch<S, SS, TS>, "k_aba_branch", &threads, &smem);
  if (rc != GB_OK) return rc;
  const int teams = threads / TS;
  const long grid = std::min<long>((B + teams - 1) / teams, (long)M->sm_count * 16);
  k_aba_branch<S, SS, TS><<<(unsigned)grid, threads, smem, st>>>(M->d_blob, M->stage_bytes, B, q, v, tau, ddq,
                                                                  (int)region);
  return cuda_error(cudaGetLastError(), "k_aba_branch");
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
  const bool shfl = GB_WARP_SHFL && M->nj - 1 <= 32;  // one joint per lane
  int rc = shfl ? warp_launch_shape(M, per_warp, k_rnea_warp<S, true>, "k_rnea_warp", &nw, &smem)
                : warp_launch_shape(M, per_warp, k_rnea_warp<S, false>, "k_rnea_warp", &nw, &smem);
  if (rc != GB_OK) return rc;
  const long grid = std::min<long>((B + nw - 1) / nw, (long)M->sm_count * 16);
  if (shfl) k_rnea_warp<S, true><<<(unsigned)grid, 32 * nw, smem, st>>>(M->d_blob, M->stage_bytes, B, q, v, a, tau);
  else k_rnea_warp<S, false><<<(unsigned)grid, 32 * nw, smem, st>>>(M->d_blob, M->stage_bytes, B, q, v, a, tau);
  return cuda_error(cudaGetLastError(), "k_rnea_warp");
}

template <class S, class SS>
int launch_aba_warp_t(const gb_model* M, long B, Arr q, Arr v, Arr tau, Arr ddq, cudaStream_t st) {
  int nw;
  size_t smem;
  const size_t per_warp = aba_warp_bytes<S, SS>(M->nj);
  int rc = warp_launch_shape(M, per_warp, k_aba_warp<S, SS>, "k_aba_warp", &nw, &smem);
  if (rc != GB_OK) return rc;
  const long grid = std::min<long>((B + nw - 1) / nw, (long)M->sm_count * 16);
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

#define GB_TEAM_SWITCH(TSV, CALL)               \
  switch (TSV) {                                \
    case 4: { constexpr int T = 4; CALL; }       \
    case 8: { constexpr int T = 8; CALL; }       \
    case 16: { constexpr int T = 16; CALL; }     \
    default: { constexpr int T = 32; CALL; }     \
  }

int launch_rnea_branch(const gb_model* M, int precision, long B, Arr q, Arr v, Arr a, Arr tau, cudaStream_t st) {
  if (precision == GB_FP64) {
    GB_TEAM_SWITCH(M->chain_team, return (launch_rnea_branch_t<double, T>(M, B, q, v, a, tau, st)));
  }
  GB_TEAM_SWITCH(M->chain_team, return (launch_rnea_branch_t<float, T>(M, B, q, v, a, tau, st)));
}

int launch_aba_branch(const gb_model* M, int precision, long B, Arr q, Arr v, Arr tau, Arr ddq, cudaStream_t st) {
  if (precision == GB_FP64) {
    GB_TEAM_SWITCH(M->chain_team, return (launch_aba_branch_t<double, double, T>(M, B, q, v, tau, ddq, st)));
  }
  GB_TEAM_SWITCH(M->chain_team, return (launch_aba_branch_t<float, double, T>(M, B, q, v, tau, ddq, st)));
}

}  // namespace gbi
