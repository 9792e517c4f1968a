// Batched sweep kernels: RNEA, ABA, CRBA (+ FP64 Cholesky), forward kinematics,
// joint Jacobians, integrate.
//
// One thread evaluates one configuration; a CTA of kThreads threads first
// copies the model blob (joint tables, placements, inertias) from global to
// shared memory with 16-byte loads, then every thread walks the tree reading
// the tables as broadcasts.  Per-joint state lives in thread-local arrays of
// the model's capacity class.
#include "gb_dyn.cuh"
#include "gb_internal.h"

namespace gbi {
namespace {

constexpr int kThreads = 128;
// resident CTAs of kThreads per SM the ABA kernel is compiled for (caps registers per thread)
#ifndef GB_ABA_MINB
#define GB_ABA_MINB 4
#endif

__device__ __forceinline__ gb::MView stage_model(const unsigned char* __restrict__ blob, int bytes,
                                                 unsigned char* smem) {
  const uint4* src = reinterpret_cast<const uint4*>(blob);
  uint4* dst = reinterpret_cast<uint4*>(smem);
  for (int k = threadIdx.x; k < bytes / 16; k += blockDim.x) dst[k] = src[k];
  __syncthreads();
  gb::MView m = gb::make_view(smem);
  gb::attach_status(m, blob);
  return m;
}

__device__ __forceinline__ gb::In in_at(const Arr& a, long b) { return gb::In{a.p + b * a.is, a.es}; }
__device__ __forceinline__ gb::Out out_at(const Arr& a, long b) {
  return gb::Out{const_cast<double*>(a.p) + b * a.is, a.es};
}

template <class S, int CAP>
__global__ void __launch_bounds__(kThreads) k_rnea(const unsigned char* blob, int bytes, long B, Arr q, Arr v, Arr a,
                                                   Arr tau) {
  extern __shared__ __align__(16) unsigned char smem[];
  const gb::MView m = stage_model(blob, bytes, smem);
  const long b = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  gb::rnea_one<S, CAP>(m, in_at(q, b), in_at(v, b), in_at(a, b), out_at(tau, b));
}

template <class S, class SS, int CAP, bool J3>
__global__ void __launch_bounds__(kThreads, GB_ABA_MINB) k_aba(const unsigned char* blob, int bytes, long B, Arr q, Arr v, Arr tau,
                                                  Arr ddq) {
  extern __shared__ __align__(16) unsigned char smem[];
  const gb::MView m = stage_model(blob, bytes, smem);
  const long b = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  gb::aba_one<S, SS, CAP, J3>(m, in_at(q, b), in_at(v, b), in_at(tau, b), out_at(ddq, b));
}

// RNEA / ABA with external forces fext (njoints x 6 per configuration, in the
// joint frames): one thread per configuration, whatever layout the model has.
template <class S, int CAP>
__global__ void __launch_bounds__(kThreads) k_rnea_fext(const unsigned char* blob, int bytes, long B, Arr q, Arr v,
                                                        Arr a, Arr fext, Arr tau) {
  extern __shared__ __align__(16) unsigned char smem[];
  const gb::MView m = stage_model(blob, bytes, smem);
  const long b = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const gb::In fe = in_at(fext, b);
  gb::rnea_one<S, CAP>(m, in_at(q, b), in_at(v, b), in_at(a, b), out_at(tau, b), &fe);
}

template <class S, class SS, int CAP, bool J3>
__global__ void __launch_bounds__(kThreads, GB_ABA_MINB) k_aba_fext(const unsigned char* blob, int bytes, long B,
                                                                    Arr q, Arr v, Arr tau, Arr fext, Arr ddq) {
  extern __shared__ __align__(16) unsigned char smem[];
  const gb::MView m = stage_model(blob, bytes, smem);
  const long b = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const gb::In fe = in_at(fext, b);
  gb::aba_one<S, SS, CAP, J3>(m, in_at(q, b), in_at(v, b), in_at(tau, b), out_at(ddq, b), &fe);
}

template <class S, int CAP>
__global__ void __launch_bounds__(kThreads) k_crba(const unsigned char* blob, int bytes, long B, bool symmetric, Arr q,
                                                   Arr M, Arr U, Arr D) {
  extern __shared__ __align__(16) unsigned char smem[];
  const gb::MView m = stage_model(blob, bytes, smem);
  const long b = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const gb::Out Uo = out_at(U, b), Do = out_at(D, b);
  gb::crba_one<S, CAP>(m, in_at(q, b), out_at(M, b), symmetric, U.p ? &Uo : nullptr, U.p ? &Do : nullptr, true);
}

template <class S, int CAP>
__global__ void __launch_bounds__(kThreads) k_fk(const unsigned char* blob, int bytes, long B, Arr q, Arr v, Arr a,
                                                 Arr oMi, Arr vo, Arr ao) {
  extern __shared__ __align__(16) unsigned char smem[];
  const gb::MView m = stage_model(blob, bytes, smem);
  const long b = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const gb::In qi = in_at(q, b), vi = in_at(v, b), ai = in_at(a, b);
  const gb::Out vout = out_at(vo, b), aout = out_at(ao, b);
  gb::fk_one<S, CAP>(m, qi, v.p ? &vi : nullptr, a.p ? &ai : nullptr, out_at(oMi, b), vo.p ? &vout : nullptr,
                     ao.p ? &aout : nullptr);
}

template <class S, int CAP>
__global__ void __launch_bounds__(kThreads) k_jacobians(const unsigned char* blob, int bytes, long B, Arr q, Arr J) {
  extern __shared__ __align__(16) unsigned char smem[];
  const gb::MView m = stage_model(blob, bytes, smem);
  const long b = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  gb::jacobians_one<S, CAP>(m, in_at(q, b), out_at(J, b));
}

__global__ void __launch_bounds__(kThreads) k_integrate(const unsigned char* blob, int bytes, long B, Arr q, Arr v,
                                                        Arr qo) {
  extern __shared__ __align__(16) unsigned char smem[];
  const gb::MView m = stage_model(blob, bytes, smem);
  const long b = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  gb::integrate_one(m, in_at(q, b), in_at(v, b), out_at(qo, b));
}

template <class K>
int launch_common(const gb_model* M, long B, cudaStream_t st, K kernel, const char* name) {
  static_assert(sizeof(K) > 0, "");
  const int bytes = M->stage_bytes;
  if (bytes > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e != cudaSuccess) return cuda_error(e, name);
  }
  (void)st;
  return GB_OK;
}

#define GB_LAUNCH(kernel, ...)                                                              \
  do {                                                                                      \
    const int rc__ = launch_common(M, B, st, kernel, #kernel);                              \
    if (rc__ != GB_OK) return rc__;                                                         \
    const int tpb__ = M->tpb[GB_FUNC_ID];                                                   \
    const long grid__ = (B + tpb__ - 1) / tpb__;                                            \
    kernel<<<(unsigned)grid__, tpb__, M->stage_bytes, st>>>(M->d_blob, M->stage_bytes, B, __VA_ARGS__); \
    return cuda_error(cudaGetLastError(), #kernel);                                         \
  } while (0)

#define GB_CAP_SWITCH(CAPV, BODY)           \
  switch (CAPV) {                           \
    case 8: { constexpr int C = 8; BODY; }   \
    case 16: { constexpr int C = 16; BODY; } \
    case 32: { constexpr int C = 32; BODY; } \
    case 64: { constexpr int C = 64; BODY; } \
    case 128: { constexpr int C = 128; BODY; } \
    default: return set_error(GB_ERR_UNSUPPORTED, "model too large"); \
  }

}  // namespace

int launch_rnea(const gb_model* M, int precision, long B, Arr q, Arr v, Arr a, Arr tau, cudaStream_t st) {
  constexpr int GB_FUNC_ID = GB_FUNC_RNEA;
  if (M->layout[GB_FUNC_ID] == GB_INSTANCE_PER_WARP) return launch_rnea_warp(M, precision, B, q, v, a, tau, st);
  if (M->layout[GB_FUNC_ID] == GB_INSTANCE_PER_BRANCH) return launch_rnea_branch(M, precision, B, q, v, a, tau, st);
  if (precision == GB_FP64) {
    GB_CAP_SWITCH(M->cap, GB_LAUNCH((k_rnea<double, C>), q, v, a, tau));
  } else {
    GB_CAP_SWITCH(M->cap, GB_LAUNCH((k_rnea<float, C>), q, v, a, tau));
  }
}

int launch_aba(const gb_model* M, int precision, long B, Arr q, Arr v, Arr tau, Arr ddq, cudaStream_t st) {
  constexpr int GB_FUNC_ID = GB_FUNC_ABA;
  if (M->layout[GB_FUNC_ID] == GB_INSTANCE_PER_WARP) return launch_aba_warp(M, precision, B, q, v, tau, ddq, st);
  if (M->layout[GB_FUNC_ID] == GB_INSTANCE_PER_BRANCH) return launch_aba_branch(M, precision, B, q, v, tau, ddq, st);
  if (M->has_three) {  // spherical / planar joints: the kernels with the three-dof steps
    if (precision == GB_FP64) {
      GB_CAP_SWITCH(M->cap, GB_LAUNCH((k_aba<double, double, C, true>), q, v, tau, ddq));
    } else {
      GB_CAP_SWITCH(M->cap, GB_LAUNCH((k_aba<float, double, C, true>), q, v, tau, ddq));
    }
  }
  if (precision == GB_FP64) {
    GB_CAP_SWITCH(M->cap, GB_LAUNCH((k_aba<double, double, C, false>), q, v, tau, ddq));
  } else {
    GB_CAP_SWITCH(M->cap, GB_LAUNCH((k_aba<float, double, C, false>), q, v, tau, ddq));
  }
}

int launch_rnea_fext(const gb_model* M, int precision, long B, Arr q, Arr v, Arr a, Arr fext, Arr tau,
                     cudaStream_t st) {
  constexpr int GB_FUNC_ID = GB_FUNC_RNEA;
  if (precision == GB_FP64) {
    GB_CAP_SWITCH(M->cap, GB_LAUNCH((k_rnea_fext<double, C>), q, v, a, fext, tau));
  } else {
    GB_CAP_SWITCH(M->cap, GB_LAUNCH((k_rnea_fext<float, C>), q, v, a, fext, tau));
  }
}

int launch_aba_fext(const gb_model* M, int precision, long B, Arr q, Arr v, Arr tau, Arr fext, Arr ddq,
                    cudaStream_t st) {
  constexpr int GB_FUNC_ID = GB_FUNC_ABA;
  if (M->has_three) {
    if (precision == GB_FP64) {
      GB_CAP_SWITCH(M->cap, GB_LAUNCH((k_aba_fext<double, double, C, true>), q, v, tau, fext, ddq));
    } else {
      GB_CAP_SWITCH(M->cap, GB_LAUNCH((k_aba_fext<float, double, C, true>), q, v, tau, fext, ddq));
    }
  }
  if (precision == GB_FP64) {
    GB_CAP_SWITCH(M->cap, GB_LAUNCH((k_aba_fext<double, double, C, false>), q, v, tau, fext, ddq));
  } else {
    GB_CAP_SWITCH(M->cap, GB_LAUNCH((k_aba_fext<float, double, C, false>), q, v, tau, fext, ddq));
  }
}

int launch_crba(const gb_model* M, int precision, bool symmetric, long B, Arr q, Arr Mo, Arr U, Arr D,
                cudaStream_t st) {
  constexpr int GB_FUNC_ID = GB_FUNC_CRBA;
  // instance-layout matrices of a large batch are written coalesced into an SOA scratch, then transposed
  if (Mo.es == 1 && B >= kSoaStagingMin) {
    const long nn = (long)M->nv * M->nv;
    void* scratch = nullptr;
    int rc = scratch_alloc(&scratch, sizeof(double) * (U.p ? 2 : 1) * (size_t)nn * B, st);
    if (rc != GB_OK) return rc;
    double* ms = static_cast<double*>(scratch);
    const Arr Ms{ms, 1, B}, Us{U.p ? ms + (size_t)nn * B : nullptr, 1, B};
    rc = launch_crba(M, precision, symmetric, B, q, Ms, Us, D, st);
    if (rc == GB_OK) rc = launch_soa_to_instance(Ms.p, B, nn, Mo, st);
    if (rc == GB_OK && U.p) rc = launch_soa_to_instance(Us.p, B, nn, U, st);
    scratch_free(scratch, st);
    return rc;
  }
  // M and U are cleared here with full-bandwidth memsets; the kernel writes their non-zero entries
  const size_t nn = (size_t)M->nv * M->nv * sizeof(double) * (size_t)B;
  int rc = cuda_error(cudaMemsetAsync(const_cast<double*>(Mo.p), 0, nn, st), "cudaMemsetAsync(M)");
  if (rc == GB_OK && U.p) rc = cuda_error(cudaMemsetAsync(const_cast<double*>(U.p), 0, nn, st), "cudaMemsetAsync(U)");
  if (rc != GB_OK) return rc;
  // the factorisation is FP64 in both precisions, and so is the M it factorises
  if (precision == GB_FP64 || U.p != nullptr) {
    GB_CAP_SWITCH(M->cap, GB_LAUNCH((k_crba<double, C>), symmetric, q, Mo, U, D));
  } else {
    GB_CAP_SWITCH(M->cap, GB_LAUNCH((k_crba<float, C>), symmetric, q, Mo, U, D));
  }
}

int launch_fk(const gb_model* M, int precision, long B, Arr q, Arr v, Arr a, Arr oMi, Arr vo, Arr ao, cudaStream_t st) {
  constexpr int GB_FUNC_ID = GB_FUNC_RNEA;
  if (precision == GB_FP64) {
    GB_CAP_SWITCH(M->cap, GB_LAUNCH((k_fk<double, C>), q, v, a, oMi, vo, ao));
  } else {
    GB_CAP_SWITCH(M->cap, GB_LAUNCH((k_fk<float, C>), q, v, a, oMi, vo, ao));
  }
}

int launch_jacobians(const gb_model* M, int precision, long B, Arr q, Arr J, cudaStream_t st) {
  constexpr int GB_FUNC_ID = GB_FUNC_RNEA;
  if (precision == GB_FP64) {
    GB_CAP_SWITCH(M->cap, GB_LAUNCH((k_jacobians<double, C>), q, J));
  } else {
    GB_CAP_SWITCH(M->cap, GB_LAUNCH((k_jacobians<float, C>), q, J));
  }
}

int launch_integrate(const gb_model* M, long B, Arr q, Arr v, Arr qo, cudaStream_t st) {
  constexpr int GB_FUNC_ID = GB_FUNC_RNEA;
  GB_LAUNCH(k_integrate, q, v, qo);
}

}  // namespace gbi
