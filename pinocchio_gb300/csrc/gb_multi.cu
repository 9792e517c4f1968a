// Heterogeneous batch: RNEA and ABA tasks over several models in one
// persistent launch.
//
// Every task (model, function, batch, arrays) is cut into tiles of one CTA's
// worth of configurations.  A grid of (number of SMs x CTAs per SM) persistent
// CTAs walks the tile list with a static stride (no atomics, so the launch can
// be captured in a CUDA graph and replayed); the list is ordered by model
// cost so that the heavy trees start first.  A CTA re-stages the model blob in
// shared memory only when its next tile belongs to another model, then each
// thread evaluates one configuration with the per-instance code of
// gb_dyn.cuh instantiated for the largest capacity class of the batch.
#include <algorithm>
#include <vector>

#include "gb_dyn.cuh"
#include "gb_internal.h"

namespace gbi {
namespace {

constexpr int kMaxTasks = 16;

struct DevTask {
  const unsigned char* blob;
  int blob_bytes;
  int function;
  long batch;
  long tile_begin;  // first global tile index of the task
  const double* q;
  const double* v;
  const double* x;
  double* out;
  int nq, nv;
};

struct TaskTable {
  DevTask t[kMaxTasks];
  int ntasks;
  long ntiles;
};

template <class S, class SS, int CAP>
__global__ void k_multi(TaskTable tab, int tile) {
  extern __shared__ __align__(16) unsigned char smem[];
  const unsigned char* staged = nullptr;
  for (long g = blockIdx.x; g < tab.ntiles; g += gridDim.x) {
    int ti = 0;
    while (ti + 1 < tab.ntasks && g >= tab.t[ti + 1].tile_begin) ++ti;
    const DevTask& T = tab.t[ti];
    if (T.blob != staged) {  // uniform across the CTA
      __syncthreads();
      const uint4* src = reinterpret_cast<const uint4*>(T.blob);
      uint4* dst = reinterpret_cast<uint4*>(smem);
      for (int k = threadIdx.x; k < T.blob_bytes / 16; k += blockDim.x) dst[k] = src[k];
      __syncthreads();
      staged = T.blob;
    }
    const gb::MView m = gb::make_view(smem);
    const long b = (g - T.tile_begin) * tile + threadIdx.x;
    if (b >= T.batch) continue;
    const gb::In q{T.q + b * T.nq, 1}, v{T.v + b * T.nv, 1}, x{T.x + b * T.nv, 1};
    const gb::Out o{T.out + b * T.nv, 1};
    if (T.function == GB_FUNC_RNEA) gb::rnea_one<S, CAP>(m, q, v, x, o);
    else gb::aba_one<S, SS, CAP>(m, q, v, x, o);
  }
}

template <class S, class SS, int CAP>
int launch_multi_cap(const TaskTable& tab, int tile, int max_blob, cudaStream_t st) {
  auto kernel = k_multi<S, SS, CAP>;
  cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, max_blob);
  if (e != cudaSuccess) return cuda_error(e, "k_multi");
  int dev = 0, nsm = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, tile, max_blob);
  if (e != cudaSuccess) return cuda_error(e, "k_multi occupancy");
  const long grid = std::min<long>(tab.ntiles, (long)nsm * std::max(per_sm, 1));
  kernel<<<(unsigned)grid, tile, max_blob, st>>>(tab, tile);
  return cuda_error(cudaGetLastError(), "k_multi");
}

}  // namespace
}  // namespace gbi

extern "C" int gb_batch_multi(const gb_task* tasks, int ntasks, int precision, int threads_per_block, void* stream) {
  using namespace gbi;
  if (tasks == nullptr || ntasks <= 0) return set_error(GB_ERR_INVALID_ARGUMENT, "no tasks");
  if (ntasks > kMaxTasks) return set_error(GB_ERR_SIZE, "at most 16 tasks per launch");
  if (precision != GB_FP64 && precision != GB_MIXED) return set_error(GB_ERR_INVALID_ARGUMENT, "unknown precision");
  const int tile = threads_per_block > 0 ? threads_per_block : 128;
  if (tile % 32 != 0 || tile > 512) return set_error(GB_ERR_INVALID_ARGUMENT, "threads_per_block must be a multiple of 32, <= 512");
  // order by model cost (joints x dofs), heaviest first
  std::vector<int> order(ntasks);
  for (int k = 0; k < ntasks; ++k) order[k] = k;
  for (int k = 0; k < ntasks; ++k) {
    const gb_task& t = tasks[k];
    if (t.model == nullptr) return set_error(GB_ERR_INVALID_ARGUMENT, "task model is NULL");
    if (t.function != GB_FUNC_RNEA && t.function != GB_FUNC_ABA) return set_error(GB_ERR_INVALID_ARGUMENT, "unknown task function");
    if (t.batch < 0) return set_error(GB_ERR_SIZE, "task batch must be >= 0");
    if (t.batch > 0) {
      int rc = check_ptr(t.q, "task q");
      if (rc == GB_OK) rc = check_ptr(t.v, "task v");
      if (rc == GB_OK) rc = check_ptr(t.x, "task x");
      if (rc == GB_OK) rc = check_ptr(t.out, "task out");
      if (rc != GB_OK) return rc;
    }
  }
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    return (long)tasks[a].model->nj * tasks[a].model->nv > (long)tasks[b].model->nj * tasks[b].model->nv;
  });
  TaskTable tab;
  tab.ntasks = 0;
  tab.ntiles = 0;
  int cap = 8, max_blob = 0;
  for (int k : order) {
    const gb_task& t = tasks[k];
    if (t.batch == 0) continue;
    DevTask& d = tab.t[tab.ntasks++];
    d.blob = t.model->d_blob;
    d.blob_bytes = t.model->stage_bytes;
    d.function = t.function;
    d.batch = t.batch;
    d.tile_begin = tab.ntiles;
    d.q = t.q; d.v = t.v; d.x = t.x; d.out = t.out;
    d.nq = t.model->nq; d.nv = t.model->nv;
    tab.ntiles += (t.batch + tile - 1) / tile;
    cap = std::max(cap, t.model->cap);
    max_blob = std::max(max_blob, t.model->stage_bytes);
  }
  if (tab.ntasks == 0) return GB_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const bool f64 = precision == GB_FP64;
  switch (cap) {
    case 8: return f64 ? launch_multi_cap<double, double, 8>(tab, tile, max_blob, st) : launch_multi_cap<float, double, 8>(tab, tile, max_blob, st);
    case 16: return f64 ? launch_multi_cap<double, double, 16>(tab, tile, max_blob, st) : launch_multi_cap<float, double, 16>(tab, tile, max_blob, st);
    case 32: return f64 ? launch_multi_cap<double, double, 32>(tab, tile, max_blob, st) : launch_multi_cap<float, double, 32>(tab, tile, max_blob, st);
    case 64: return f64 ? launch_multi_cap<double, double, 64>(tab, tile, max_blob, st) : launch_multi_cap<float, double, 64>(tab, tile, max_blob, st);
    case 128: return f64 ? launch_multi_cap<double, double, 128>(tab, tile, max_blob, st) : launch_multi_cap<float, double, 128>(tab, tile, max_blob, st);
    default: return set_error(GB_ERR_UNSUPPORTED, "model too large");
  }
}
