// Heterogeneous batch: RNEA and ABA tasks over several models in one
// persistent launch.
//
// Every task (model, function, batch, arrays) is cut into tiles of one CTA's
// worth of configurations, in the layout chosen for its model and function
// (gb_model_set_layout, the autotuner's choice per tree): one configuration per
// thread, or one per warp (the warp-layout code of gb_warp.cuh, per-warp state
// in shared memory after the staged model).  A grid of (number of SMs x CTAs per SM) persistent
// CTAs walks the tile list with a static stride (no atomics, so the launch can
// be captured in a CUDA graph and replayed); the list is ordered by model
// cost so that the heavy trees start first.  A CTA re-stages the model blob in
// shared memory only when its next tile belongs to another model, then each
// thread evaluates one configuration with the per-instance code of
// gb_dyn.cuh instantiated for the largest capacity class of the batch.
#include <algorithm>
#include <vector>

#include "gb_warp.cuh"

namespace gbi {
namespace {

constexpr int kMaxTasks = 16;

struct DevTask {
  const unsigned char* blob;
  int blob_bytes;
  int function;
  int warp;      // 1: one warp per configuration
  int per_tile;  // configurations per tile: the CTA's threads, or its warps
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

// J3: some task's model has spherical / planar joints (the ABA's three-dof steps are compiled in
// only then, so that the launches of the other models keep their registers)
template <class S, class SS, int CAP, bool J3>
__global__ void k_multi(TaskTable tab, int tile, int blob_region, int warp_region) {
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
    gb::MView m = gb::make_view(smem);
    gb::attach_status(m, T.blob);
    if (T.warp) {  // warp-uniform
      const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
      const long b = (g - T.tile_begin) * T.per_tile + w;
      if (b >= T.batch) continue;
      unsigned char* region = smem + blob_region + (size_t)w * warp_region;
      const gb::In q = warp::w_in(Arr{T.q, T.nq, 1}, b), v = warp::w_in(Arr{T.v, T.nv, 1}, b);
      const gb::In x = warp::w_in(Arr{T.x, T.nv, 1}, b);
      const gb::Out o = warp::w_out(Arr{T.out, T.nv, 1}, b);
      if (T.function == GB_FUNC_RNEA) {
        warp::rnea_warp_one<S>(m, q, v, x, o, reinterpret_cast<S*>(region), warp::LevelSched{lane});
      } else {
        const size_t per_s = warp::align16(sizeof(S) * warp::aba_words_s<S, SS>() * (size_t)m.nj);
        warp::aba_warp_one<S, SS>(m, q, v, x, o, reinterpret_cast<S*>(region), reinterpret_cast<SS*>(region + per_s),
                                  warp::LevelSched{lane});
      }
      __syncwarp();
      continue;
    }
    const long b = (g - T.tile_begin) * tile + threadIdx.x;
    if (b >= T.batch) continue;
    const gb::In q{T.q + b * T.nq, 1}, v{T.v + b * T.nv, 1}, x{T.x + b * T.nv, 1};
    const gb::Out o{T.out + b * T.nv, 1};
    if (T.function == GB_FUNC_RNEA) gb::rnea_one<S, CAP>(m, q, v, x, o);
    else gb::aba_one<S, SS, CAP, J3>(m, q, v, x, o);
  }
}

template <class S, class SS, int CAP>
int launch_multi_cap(const TaskTable& tab, int tile, int blob_region, int warp_region, bool j3, cudaStream_t st) {
  auto kernel = j3 ? k_multi<S, SS, CAP, true> : k_multi<S, SS, CAP, false>;
  const int smem = blob_region + (tile / 32) * warp_region;
  cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return cuda_error(e, "k_multi");
  int dev = 0, nsm = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, tile, smem);
  if (e != cudaSuccess) return cuda_error(e, "k_multi occupancy");
  const long grid = std::min<long>(tab.ntiles, (long)nsm * std::max(per_sm, 1));
  kernel<<<(unsigned)grid, tile, smem, st>>>(tab, tile, blob_region, warp_region);
  return cuda_error(cudaGetLastError(), "k_multi");
}

// shared memory of one warp-layout task's per-warp region
size_t warp_region_bytes(const gb_model* M, int function, bool f64) {
  if (function == GB_FUNC_RNEA) return f64 ? warp::rnea_warp_bytes<double>(M->nj) : warp::rnea_warp_bytes<float>(M->nj);
  return f64 ? warp::aba_warp_bytes<double, double>(M->nj) : warp::aba_warp_bytes<float, double>(M->nj);
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
    if (t.model->has_mimic)
      return set_error(GB_ERR_UNSUPPORTED, "mimic joints: the heterogeneous launch does not take them (gb_rnea does)");
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
  const bool f64 = precision == GB_FP64;
  // shared memory: the largest staged model, then one region per warp for the warp-layout tasks
  // (a task whose layout does not fit runs one configuration per thread)
  int max_blob = 0;
  for (int k = 0; k < ntasks; ++k) max_blob = std::max(max_blob, tasks[k].model->stage_bytes);
  const int blob_region = (int)warp::align16((size_t)max_blob);
  constexpr size_t kSmemLimit = 200 * 1024;
  size_t warp_region = 0;
  std::vector<bool> use_warp(ntasks, false);
  for (int k = 0; k < ntasks; ++k) {
    const gb_task& t = tasks[k];
    if (t.model->layout[t.function] != GB_INSTANCE_PER_WARP) continue;
    const size_t r = std::max(warp_region, warp_region_bytes(t.model, t.function, f64));
    if (blob_region + (size_t)(tile / 32) * r > kSmemLimit) continue;
    warp_region = r;
    use_warp[k] = true;
  }
  TaskTable tab;
  tab.ntasks = 0;
  tab.ntiles = 0;
  int cap = 8;
  bool j3 = false;  // spherical / planar joints in a task (they run one configuration per thread)
  for (int k : order) {
    const gb_task& t = tasks[k];
    if (t.batch == 0) continue;
    DevTask& d = tab.t[tab.ntasks++];
    d.blob = t.model->d_blob;
    d.blob_bytes = t.model->stage_bytes;
    d.function = t.function;
    d.warp = use_warp[k] ? 1 : 0;
    d.per_tile = use_warp[k] ? tile / 32 : tile;
    d.batch = t.batch;
    d.tile_begin = tab.ntiles;
    d.q = t.q; d.v = t.v; d.x = t.x; d.out = t.out;
    d.nq = t.model->nq; d.nv = t.model->nv;
    tab.ntiles += (t.batch + d.per_tile - 1) / d.per_tile;
    if (!use_warp[k]) cap = std::max(cap, t.model->cap);
    j3 = j3 || t.model->has_three;
  }
  if (tab.ntasks == 0) return GB_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const int wr = (int)warp_region;
  switch (cap) {
    case 8: return f64 ? launch_multi_cap<double, double, 8>(tab, tile, blob_region, wr, j3, st) : launch_multi_cap<float, double, 8>(tab, tile, blob_region, wr, j3, st);
    case 16: return f64 ? launch_multi_cap<double, double, 16>(tab, tile, blob_region, wr, j3, st) : launch_multi_cap<float, double, 16>(tab, tile, blob_region, wr, j3, st);
    case 32: return f64 ? launch_multi_cap<double, double, 32>(tab, tile, blob_region, wr, j3, st) : launch_multi_cap<float, double, 32>(tab, tile, blob_region, wr, j3, st);
    case 64: return f64 ? launch_multi_cap<double, double, 64>(tab, tile, blob_region, wr, j3, st) : launch_multi_cap<float, double, 64>(tab, tile, blob_region, wr, j3, st);
    case 128: return f64 ? launch_multi_cap<double, double, 128>(tab, tile, blob_region, wr, j3, st) : launch_multi_cap<float, double, 128>(tab, tile, blob_region, wr, j3, st);
    default: return set_error(GB_ERR_UNSUPPORTED, "model too large");
  }
}
