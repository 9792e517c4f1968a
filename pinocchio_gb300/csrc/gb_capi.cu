// C ABI of the engine: model flattening / validation, argument checks, the
// ModelPool-shaped batch entry points.  No entry point computes on the CPU.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>

#include "gb_internal.h"

namespace {
thread_local std::string g_err;
}  // namespace

namespace gbi {

int set_error(int code, const std::string& msg) {
  g_err = msg;
  return code;
}
int cuda_error(cudaError_t e, const char* where) {
  if (e == cudaSuccess) return GB_OK;
  return set_error(GB_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}
int check_ptr(const void* p, const char* name) {
  if (p == nullptr) return set_error(GB_ERR_INVALID_ARGUMENT, std::string(name) + " is NULL");
  if (reinterpret_cast<uintptr_t>(p) % alignof(double) != 0)
    return set_error(GB_ERR_INVALID_ARGUMENT, std::string(name) + " is not 8-byte aligned");
  return GB_OK;
}
int check_common_mimic(const gb_model* m, int precision, int layout, long batch) {
  if (m == nullptr) return set_error(GB_ERR_INVALID_ARGUMENT, "model is NULL");
  if (precision != GB_FP64 && precision != GB_MIXED) return set_error(GB_ERR_INVALID_ARGUMENT, "unknown precision");
  if (layout != GB_LAYOUT_INSTANCE && layout != GB_LAYOUT_SOA)
    return set_error(GB_ERR_INVALID_ARGUMENT, "unknown layout");
  if (batch < 0) return set_error(GB_ERR_SIZE, "batch must be >= 0");
  return GB_OK;
}
// the reference rejects mimic joints outside RNEA, CRBA and the kinematics (MimicChecker:
// aba.hxx:250, rnea-derivatives.hxx:157, cholesky.hxx:37)
int check_common(const gb_model* m, int precision, int layout, long batch) {
  const int rc = check_common_mimic(m, precision, layout, batch);
  if (rc == GB_OK && m->has_mimic) return set_error(GB_ERR_UNSUPPORTED, "Function does not support mimic joints");
  return rc;
}

}  // namespace gbi

using gbi::set_error;

extern "C" {

const char* gb_last_error(void) { return g_err.c_str(); }

int gb_model_create(const gb_model_desc* desc, gb_model** out) {
  if (out == nullptr || desc == nullptr) return set_error(GB_ERR_INVALID_ARGUMENT, "desc/out is NULL");
  *out = nullptr;
  if (!desc->parents || !desc->jtype || !desc->placement || !desc->inertia)
    return set_error(GB_ERR_INVALID_ARGUMENT, "model tables must not be NULL");
  gb_model* M = new (std::nothrow) gb_model();
  if (!M) return set_error(GB_ERR_INVALID_ARGUMENT, "out of host memory");
  std::string err;
  int rc = gbm::build_model(M, desc, &err);
  if (rc != GB_OK) {
    delete M;
    return set_error(rc, err);
  }
  cudaError_t e = cudaGetDevice(&M->device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&M->sm_count, cudaDevAttrMultiProcessorCount, M->device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&M->smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, M->device);
  if (e == cudaSuccess) e = cudaMalloc(&M->d_blob, M->blob_bytes);
  if (e == cudaSuccess) e = cudaMemcpy(M->d_blob, M->blob.data(), M->blob_bytes, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    if (M->d_blob) cudaFree(M->d_blob);
    delete M;
    return gbi::cuda_error(e, "gb_model_create");
  }
  if (M->has_mimic) {
    const size_t qb = sizeof(gb::MimicQ) * M->qmap.size(), vb = sizeof(gb::MimicV) * M->vmap.size();
    e = cudaMalloc(&M->d_mimic, qb + vb);
    if (e == cudaSuccess) e = cudaMemcpy(M->d_mimic, M->qmap.data(), qb, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
      e = cudaMemcpy(static_cast<unsigned char*>(M->d_mimic) + qb, M->vmap.data(), vb, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      if (M->d_mimic) cudaFree(M->d_mimic);
      cudaFree(M->d_blob);
      delete M;
      return gbi::cuda_error(e, "gb_model_create");
    }
  }
  rc = gbi::prepare_model_launches(M);
  if (rc != GB_OK) {
    if (M->d_mimic) cudaFree(M->d_mimic);
    cudaFree(M->d_blob);
    delete M;
    return rc;
  }
  *out = M;
  return GB_OK;
}

int gb_model_destroy(gb_model* M) {
  if (!M) return GB_OK;
  if (M->d_blob) cudaFree(M->d_blob);
  if (M->d_mimic) cudaFree(M->d_mimic);
  delete M;
  return GB_OK;
}

int gb_numeric_status(const gb_model* M, unsigned int* flags, int reset) {
  if (!M || !flags) return set_error(GB_ERR_INVALID_ARGUMENT, "model/flags is NULL");
  static_assert(GB_NUMERIC_PIVOT == gb::NUM_PIVOT && GB_NUMERIC_NONFINITE == gb::NUM_NONFINITE, "status bits");
  const gb::BlobHeader* h = reinterpret_cast<const gb::BlobHeader*>(M->blob.data());
  unsigned* word = reinterpret_cast<unsigned*>(M->d_blob + h->o_status);
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(flags, word, sizeof(unsigned), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && reset) e = cudaMemset(word, 0, sizeof(unsigned));
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return gbi::cuda_error(e, "gb_numeric_status");
  if (*flags == 0) return GB_OK;
  std::string msg = "numeric failure in a kernel:";
  if (*flags & GB_NUMERIC_PIVOT) msg += " a pivot was not positive (singular or indefinite inertia, or NaN input);";
  if (*flags & GB_NUMERIC_NONFINITE) msg += " an output was NaN or infinite;";
  return set_error(GB_ERR_NUMERIC, msg);
}

int gb_memcpy_async(void* dst, const void* src, size_t bytes, void* stream) {
  if (bytes == 0) return GB_OK;
  if (!dst || !src) return set_error(GB_ERR_INVALID_ARGUMENT, "dst/src is NULL");
  return gbi::cuda_error(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, (cudaStream_t)stream), "gb_memcpy_async");
}

int gb_model_dims(const gb_model* M, int* nq, int* nv, int* nj) {
  if (!M) return set_error(GB_ERR_INVALID_ARGUMENT, "model is NULL");
  if (nq) *nq = M->nq_red;
  if (nv) *nv = M->nv_red;
  if (nj) *nj = M->nj_user;
  return GB_OK;
}

int gb_model_nv_extended(const gb_model* M, int* nv_extended) {
  if (!M || !nv_extended) return set_error(GB_ERR_INVALID_ARGUMENT, "model/nv_extended is NULL");
  *nv_extended = M->nv;
  return GB_OK;
}

#define GB_TRY(x)               \
  do {                          \
    const int rc__ = (x);       \
    if (rc__ != GB_OK) return rc__; \
  } while (0)

int gb_rnea(const gb_model* M, int precision, int layout, long B, const double* q, const double* v, const double* a,
            double* tau, void* stream) {
  GB_TRY(gbi::check_common_mimic(M, precision, layout, B));
  if (B == 0) return GB_OK;
  GB_TRY(gbi::check_ptr(q, "q")); GB_TRY(gbi::check_ptr(v, "v")); GB_TRY(gbi::check_ptr(a, "a"));
  GB_TRY(gbi::check_ptr(tau, "tau"));
  return (M->has_mimic ? gbi::launch_rnea_mimic : gbi::launch_rnea)(
      M, precision, B, gbi::arr(q, layout, B, M->nq_red), gbi::arr(v, layout, B, M->nv_red),
      gbi::arr(a, layout, B, M->nv_red), gbi::arr(tau, layout, B, M->nv_red), (cudaStream_t)stream);
}

int gb_rnea_fext(const gb_model* M, int precision, int layout, long B, const double* q, const double* v,
                 const double* a, const double* fext, double* tau, void* stream) {
  GB_TRY(gbi::check_common_mimic(M, precision, layout, B));
  if (B == 0) return GB_OK;
  GB_TRY(gbi::check_ptr(q, "q")); GB_TRY(gbi::check_ptr(v, "v")); GB_TRY(gbi::check_ptr(a, "a"));
  GB_TRY(gbi::check_ptr(fext, "fext")); GB_TRY(gbi::check_ptr(tau, "tau"));
  return (M->has_mimic ? gbi::launch_rnea_fext_mimic : gbi::launch_rnea_fext)(
      M, precision, B, gbi::arr(q, layout, B, M->nq_red), gbi::arr(v, layout, B, M->nv_red),
      gbi::arr(a, layout, B, M->nv_red), gbi::arr(fext, layout, B, 6L * M->nj_user),
      gbi::arr(tau, layout, B, M->nv_red), (cudaStream_t)stream);
}

// nonLinearEffects = rnea(q, v, 0) and computeGeneralizedGravity = rnea(q, 0, 0)
// (reference algorithm/rnea.hxx:221-336, 346-446): the RNEA kernel reading a zero vector
// (16 zero bytes of the model blob, stride 0) for the absent arguments.
static gbi::Arr zero_arr(const gb_model* M) {
  const gb::BlobHeader* h = reinterpret_cast<const gb::BlobHeader*>(M->blob.data());
  return gbi::Arr{reinterpret_cast<const double*>(M->d_blob + h->o_zero), 0, 0};
}

int gb_nonlinear_effects(const gb_model* M, int precision, int layout, long B, const double* q, const double* v,
                         double* nle, void* stream) {
  GB_TRY(gbi::check_common_mimic(M, precision, layout, B));
  if (B == 0) return GB_OK;
  GB_TRY(gbi::check_ptr(q, "q")); GB_TRY(gbi::check_ptr(v, "v")); GB_TRY(gbi::check_ptr(nle, "nle"));
  return (M->has_mimic ? gbi::launch_rnea_mimic : gbi::launch_rnea)(
      M, precision, B, gbi::arr(q, layout, B, M->nq_red), gbi::arr(v, layout, B, M->nv_red), zero_arr(M),
      gbi::arr(nle, layout, B, M->nv_red), (cudaStream_t)stream);
}

int gb_generalized_gravity(const gb_model* M, int precision, int layout, long B, const double* q, double* g,
                           void* stream) {
  GB_TRY(gbi::check_common_mimic(M, precision, layout, B));
  if (B == 0) return GB_OK;
  GB_TRY(gbi::check_ptr(q, "q")); GB_TRY(gbi::check_ptr(g, "g"));
  return (M->has_mimic ? gbi::launch_rnea_mimic : gbi::launch_rnea)(
      M, precision, B, gbi::arr(q, layout, B, M->nq_red), zero_arr(M), zero_arr(M),
      gbi::arr(g, layout, B, M->nv_red), (cudaStream_t)stream);
}

int gb_static_torque(const gb_model* M, int precision, int layout, long B, const double* q, const double* fext,
                     double* tau, void* stream) {
  GB_TRY(gbi::check_common_mimic(M, precision, layout, B));
  if (B == 0) return GB_OK;
  GB_TRY(gbi::check_ptr(q, "q")); GB_TRY(gbi::check_ptr(fext, "fext")); GB_TRY(gbi::check_ptr(tau, "tau"));
  return (M->has_mimic ? gbi::launch_rnea_fext_mimic : gbi::launch_rnea_fext)(
      M, precision, B, gbi::arr(q, layout, B, M->nq_red), zero_arr(M), zero_arr(M),
      gbi::arr(fext, layout, B, 6L * M->nj_user), gbi::arr(tau, layout, B, M->nv_red),
                               (cudaStream_t)stream);
}

// forwardDynamics / impulseDynamics with a constraint Jacobian: J is nc x nv
// row-major per configuration (nc * nv values in `layout`), gamma / lambda nc values.
static int contact_entry(const gb_model* M, int precision, int layout, long B, int nc, bool impulse,
                         const double* q, const double* v, const double* tau, const double* J, const double* gamma,
                         double r_coeff, double inv_damping, double* out, double* lam, void* stream) {
  GB_TRY(gbi::check_common(M, precision, layout, B));
  if (nc < 0 || nc > 1024) return set_error(GB_ERR_SIZE, "the number of constraint rows must be in 0..1024");
  if (!(inv_damping >= 0.0)) return set_error(GB_ERR_INVALID_ARGUMENT, "mu must be positive.");
  if (B == 0) return GB_OK;
  GB_TRY(gbi::check_ptr(q, "q")); GB_TRY(gbi::check_ptr(v, impulse ? "v_before" : "v"));
  GB_TRY(gbi::check_ptr(out, impulse ? "dq_after" : "ddq"));
  if (!impulse) GB_TRY(gbi::check_ptr(tau, "tau"));
  if (nc > 0) {
    GB_TRY(gbi::check_ptr(J, "J"));
    GB_TRY(gbi::check_ptr(lam, impulse ? "impulse_c" : "lambda_c"));
    if (!impulse) GB_TRY(gbi::check_ptr(gamma, "gamma"));
  }
  const gbi::Arr none{nullptr, 0, 0};
  const long nv = M->nv;
  return gbi::launch_contact(M, precision, impulse, B, nc, gbi::arr(q, layout, B, M->nq), gbi::arr(v, layout, B, nv),
                             gbi::arr(impulse ? v : tau, layout, B, nv),
                             nc > 0 ? gbi::arr(J, layout, B, (long)nc * nv) : none,
                             nc > 0 && !impulse ? gbi::arr(gamma, layout, B, nc) : none, r_coeff, inv_damping,
                             gbi::arr(out, layout, B, nv), nc > 0 ? gbi::arr(lam, layout, B, nc) : none,
                             (cudaStream_t)stream);
}

int gb_forward_dynamics(const gb_model* M, int precision, int layout, long B, int nc, const double* q, const double* v,
                        const double* tau, const double* J, const double* gamma, double inv_damping, double* ddq,
                        double* lambda_c, void* stream) {
  return contact_entry(M, precision, layout, B, nc, false, q, v, tau, J, gamma, 0.0, inv_damping, ddq, lambda_c,
                       stream);
}

int gb_impulse_dynamics(const gb_model* M, int precision, int layout, long B, int nc, const double* q,
                        const double* v_before, const double* J, double r_coeff, double inv_damping, double* dq_after,
                        double* impulse_c, void* stream) {
  return contact_entry(M, precision, layout, B, nc, true, q, v_before, nullptr, J, nullptr, r_coeff, inv_damping,
                       dq_after, impulse_c, stream);
}

int gb_kkt_contact_inverse(const gb_model* M, int precision, int layout, long B, int nc, const double* q,
                           const double* J, double inv_damping, double* K, void* stream) {
  GB_TRY(gbi::check_common(M, precision, layout, B));
  if (nc < 0 || nc > 1024) return set_error(GB_ERR_SIZE, "the number of constraint rows must be in 0..1024");
  if (!(inv_damping >= 0.0)) return set_error(GB_ERR_INVALID_ARGUMENT, "mu must be positive.");
  if (B == 0) return GB_OK;
  GB_TRY(gbi::check_ptr(q, "q")); GB_TRY(gbi::check_ptr(K, "KKTMatrix_inv"));
  if (nc > 0) GB_TRY(gbi::check_ptr(J, "J"));
  const long nv = M->nv, n = nv + nc;
  return gbi::launch_kkt_inverse(M, B, nc, gbi::arr(q, layout, B, M->nq),
                                 nc > 0 ? gbi::arr(J, layout, B, (long)nc * nv) : gbi::Arr{nullptr, 0, 0}, inv_damping,
                                 gbi::arr(K, layout, B, n * n), (cudaStream_t)stream);
}

int gb_constraint_set_create(const gb_model* M, int n, const gb_constraint_desc* cs, gb_constraint_set** out) {
  if (!M || !out) return set_error(GB_ERR_INVALID_ARGUMENT, "model/out is NULL");
  *out = nullptr;
  if (M->has_mimic) return set_error(GB_ERR_UNSUPPORTED, "Function does not support mimic joints");
  if (n < 0 || n > 64) return set_error(GB_ERR_SIZE, "the number of constraint models must be in 0..64");
  if (n > 0 && !cs) return set_error(GB_ERR_INVALID_ARGUMENT, "constraints is NULL");
  std::vector<int> internal(M->nj_user, -1);  // the caller's joint -> the internal joint carrying it
  for (int i = 0; i < M->nj; ++i)
    if (M->ujoint[i] >= 0) internal[M->ujoint[i]] = i;
  internal[0] = 0;
  auto* S = new gb_constraint_set;
  S->model = M;
  S->n = n;
  const int nv = M->nv;
  S->sparsity.assign((size_t)n * nv, 0);
  for (int e = 0; e < n; ++e) {
    const gb_constraint_desc& c = cs[e];
    std::string bad;
    if (c.type != GB_CONTACT_3D && c.type != GB_CONTACT_6D) bad = "unknown constraint type";
    else if (c.reference_frame != GB_FRAME_LOCAL && c.reference_frame != GB_FRAME_LOCAL_WORLD_ALIGNED)
      bad = "constraintDynamics is only operating from LOCAL or LOCAL_WORLD_ALIGNED reference frames";
    else if (c.joint1_id < 0 || c.joint1_id >= M->nj_user || c.joint2_id < 0 || c.joint2_id >= M->nj_user)
      bad = "constraint joint index out of range";
    if (!bad.empty()) {
      delete S;
      return set_error(GB_ERR_INVALID_ARGUMENT, "constraint " + std::to_string(e) + ": " + bad);
    }
    gbi::ConstraintDev d{};
    const int size = c.type == GB_CONTACT_3D ? 3 : 6;
    d.type = c.type;
    d.frame = c.reference_frame;
    d.j1 = internal[c.joint1_id];
    d.j2 = internal[c.joint2_id];
    d.row = S->nc;
    S->nc += size;
    // placements relative to the internal (folded) frames: the caller's frame i is frame_i' F^T
    for (int side = 0; side < 2; ++side) {
      const double* P = side == 0 ? c.joint1_placement : c.joint2_placement;
      double* Q = side == 0 ? d.P1 : d.P2;
      const double* F = M->fix.data() + 9 * (side == 0 ? d.j1 : d.j2);
      for (int r = 0; r < 3; ++r) {
        for (int col = 0; col < 3; ++col)
          Q[3 * r + col] = F[r] * P[col] + F[3 + r] * P[3 + col] + F[6 + r] * P[6 + col];
        Q[9 + r] = F[r] * P[9] + F[3 + r] * P[10] + F[6 + r] * P[11];
      }
    }
    for (int k = 0; k < 6; ++k) {
      d.des[k] = c.desired_acceleration[k];
      d.Kp[k] = k < size ? c.Kp[k] : 0.0;
      d.Kd[k] = k < size ? c.Kd[k] : 0.0;
      if (d.Kp[k] != 0.0 || d.Kd[k] != 0.0) d.gains = 1;
    }
    // the columns each side moves (RigidConstraintModel::init, contact-info.hpp:712-790), on the
    // internal tree: joints up to the common ancestor, and for a point constraint the ancestor's support
    signed char* sp = S->sparsity.data() + (size_t)e * nv;
    auto mark = [&](int j, int bit) {
      for (int k = 0; k < M->nvs[j]; ++k) sp[M->idx_v[j] + k] |= bit;
    };
    int c1 = d.j1, c2 = d.j2;
    while (c1 != c2) {
      if (c1 > c2) {
        mark(c1, 1);
        c1 = M->parents[c1];
      } else {
        mark(c2, 2);
        c2 = M->parents[c2];
      }
    }
    if (c.type == GB_CONTACT_3D)
      for (int j = c1; j > 0; j = M->parents[j]) mark(j, 3);
    S->host.push_back(d);
  }
  // the dofs whose rows of U^-1 J^T can be non-zero: the ancestor closure of each constraint's
  // columns (both joints' supports), as a mask and as a sorted list [count, dofs...]
  std::vector<signed char> closure((size_t)n * nv, 0);
  std::vector<short> lists((size_t)n * (nv + 1), 0);
  for (int e = 0; e < n; ++e) {
    signed char* cm = closure.data() + (size_t)e * nv;
    for (int j : {S->host[e].j1, S->host[e].j2})
      for (; j > 0; j = M->parents[j])
        for (int k = 0; k < M->nvs[j]; ++k) cm[M->idx_v[j] + k] = 1;
    short* L = lists.data() + (size_t)e * (nv + 1);
    for (int k = 0; k < nv; ++k)
      if (cm[k]) L[1 + L[0]++] = (short)k;
  }
  const size_t o_lists = (sizeof(gbi::ConstraintDev) * (size_t)n + 2 * S->sparsity.size() + 1) & ~(size_t)1;
  const size_t bytes = n > 0 ? o_lists + sizeof(short) * lists.size() : 0;
  if (bytes > 0) {
    std::vector<unsigned char> h(bytes, 0);
    std::memcpy(h.data(), S->host.data(), sizeof(gbi::ConstraintDev) * (size_t)n);
    unsigned char* codes = h.data() + sizeof(gbi::ConstraintDev) * (size_t)n;
    std::memcpy(codes, S->sparsity.data(), S->sparsity.size());
    std::memcpy(codes + S->sparsity.size(), closure.data(), closure.size());
    std::memcpy(h.data() + o_lists, lists.data(), sizeof(short) * lists.size());
    cudaError_t e = cudaMalloc(&S->d_mem, bytes);
    if (e == cudaSuccess) e = cudaMemcpy(S->d_mem, h.data(), bytes, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      if (S->d_mem) cudaFree(S->d_mem);
      delete S;
      return gbi::cuda_error(e, "gb_constraint_set_create");
    }
  }
  *out = S;
  return GB_OK;
}

int gb_constraint_set_destroy(gb_constraint_set* S) {
  if (!S) return GB_OK;
  if (S->d_mem) cudaFree(S->d_mem);
  delete S;
  return GB_OK;
}

int gb_constraint_set_dims(const gb_constraint_set* S, int* n, int* constraint_dim) {
  if (!S) return set_error(GB_ERR_INVALID_ARGUMENT, "set is NULL");
  if (n) *n = S->n;
  if (constraint_dim) *constraint_dim = S->nc;
  return GB_OK;
}

int gb_constraint_dynamics(const gb_model* M, int precision, const gb_constraint_set* S,
                           const gb_proximal_settings* settings, int layout, long B, const double* q, const double* v,
                           const double* tau, double* ddq, double* lambda_c, int* iterations, double* residuals,
                           void* stream) {
  GB_TRY(gbi::check_common(M, precision, layout, B));
  if (!S || !settings) return set_error(GB_ERR_INVALID_ARGUMENT, "set/settings is NULL");
  if (S->model != M) return set_error(GB_ERR_INVALID_ARGUMENT, "the constraint set belongs to another model");
  if (!(settings->mu >= 0.0)) return set_error(GB_ERR_INVALID_ARGUMENT, "mu has to be positive");
  if (!(settings->absolute_accuracy >= 0.0) || !(settings->relative_accuracy >= 0.0))
    return set_error(GB_ERR_INVALID_ARGUMENT, "Accuracy must be positive.");
  if (settings->max_iter < 1) return set_error(GB_ERR_INVALID_ARGUMENT, "max_iter must be greater or equal to 1");
  if (B == 0) return GB_OK;
  GB_TRY(gbi::check_ptr(q, "q")); GB_TRY(gbi::check_ptr(v, "v")); GB_TRY(gbi::check_ptr(tau, "tau"));
  GB_TRY(gbi::check_ptr(ddq, "ddq"));
  if (S->nc > 0) GB_TRY(gbi::check_ptr(lambda_c, "lambda_c"));
  const long nv = M->nv;
  return gbi::launch_constraint(M, precision, B, S, *settings, gbi::arr(q, layout, B, M->nq), gbi::arr(v, layout, B, nv),
                                gbi::arr(tau, layout, B, nv), gbi::arr(ddq, layout, B, nv),
                                S->nc > 0 ? gbi::arr(lambda_c, layout, B, S->nc) : gbi::Arr{nullptr, 0, 0}, iterations,
                                residuals, (cudaStream_t)stream);
}

int gb_contact_cholesky(const gb_model* M, int precision, const gb_constraint_set* S, double mu, int layout, long B,
                        const double* q, double* kkt, double* kkt_inverse, double* osim_inverse, double* osim,
                        double* minv, double* jminv, void* stream) {
  GB_TRY(gbi::check_common(M, precision, layout, B));
  if (!S) return set_error(GB_ERR_INVALID_ARGUMENT, "set is NULL");
  if (S->model != M) return set_error(GB_ERR_INVALID_ARGUMENT, "the constraint set belongs to another model");
  if (!(mu >= 0.0)) return set_error(GB_ERR_INVALID_ARGUMENT, "mu must be positive.");
  if (B == 0) return GB_OK;
  GB_TRY(gbi::check_ptr(q, "q"));
  const long nv = M->nv, nc = S->nc, n = nv + nc;
  auto a = [&](double* p, long k) { return p && k > 0 ? gbi::arr(p, layout, B, k) : gbi::Arr{nullptr, 0, 0}; };
  return gbi::launch_contact_cholesky(M, B, S, mu, gbi::arr(q, layout, B, M->nq), a(kkt, n * n), a(kkt_inverse, n * n),
                                      a(osim_inverse, nc * nc), a(osim, nc * nc), a(minv, nv * nv), a(jminv, nc * nv),
                                      (cudaStream_t)stream);
}

int gb_constraint_dynamics_derivatives(const gb_model* M, int precision, const gb_constraint_set* S,
                                       const gb_proximal_settings* settings, int layout, long B, const double* q,
                                       const double* v, const double* tau, double* ddq, double* lambda_c,
                                       double* ddq_dq, double* ddq_dv, double* ddq_dtau, double* dl_dq, double* dl_dv,
                                       double* dl_dtau, int* iterations, void* stream) {
  GB_TRY(gbi::check_common(M, precision, layout, B));
  if (!S || !settings) return set_error(GB_ERR_INVALID_ARGUMENT, "set/settings is NULL");
  if (S->model != M) return set_error(GB_ERR_INVALID_ARGUMENT, "the constraint set belongs to another model");
  if (!(settings->mu >= 0.0)) return set_error(GB_ERR_INVALID_ARGUMENT, "mu has to be positive");
  if (!(settings->absolute_accuracy >= 0.0) || !(settings->relative_accuracy >= 0.0))
    return set_error(GB_ERR_INVALID_ARGUMENT, "Accuracy must be positive.");
  if (settings->max_iter < 1) return set_error(GB_ERR_INVALID_ARGUMENT, "max_iter must be greater or equal to 1");
  for (const gbi::ConstraintDev& c : S->host)
    if (c.j2 != 0 || (c.gains && c.frame != GB_FRAME_LOCAL))
      return set_error(GB_ERR_UNSUPPORTED,
                       "the constraint dynamics derivatives take constraints to the world (joint2_id = 0), with "
                       "Baumgarte gains on LOCAL contacts only");
  GB_TRY(gbi::check_gravity(M));
  if (B == 0) return GB_OK;
  GB_TRY(gbi::check_ptr(q, "q")); GB_TRY(gbi::check_ptr(v, "v")); GB_TRY(gbi::check_ptr(tau, "tau"));
  GB_TRY(gbi::check_ptr(ddq, "ddq"));
  GB_TRY(gbi::check_ptr(ddq_dq, "ddq_dq")); GB_TRY(gbi::check_ptr(ddq_dv, "ddq_dv"));
  GB_TRY(gbi::check_ptr(ddq_dtau, "ddq_dtau"));
  if (S->nc > 0) {
    GB_TRY(gbi::check_ptr(lambda_c, "lambda_c"));
    GB_TRY(gbi::check_ptr(dl_dq, "dlambda_dq")); GB_TRY(gbi::check_ptr(dl_dv, "dlambda_dv"));
    GB_TRY(gbi::check_ptr(dl_dtau, "dlambda_dtau"));
  }
  const long nv = M->nv, nn = nv * nv, cn = (long)S->nc * nv;
  using gbi::arr;
  const gbi::Arr none{nullptr, 0, 0};
  return gbi::launch_constraint_derivs(
      M, precision, B, S, *settings, arr(q, layout, B, M->nq), arr(v, layout, B, nv), arr(tau, layout, B, nv),
      arr(ddq, layout, B, nv), S->nc > 0 ? arr(lambda_c, layout, B, S->nc) : none, arr(ddq_dq, layout, B, nn),
      arr(ddq_dv, layout, B, nn), arr(ddq_dtau, layout, B, nn), S->nc > 0 ? arr(dl_dq, layout, B, cn) : none,
      S->nc > 0 ? arr(dl_dv, layout, B, cn) : none, S->nc > 0 ? arr(dl_dtau, layout, B, cn) : none, iterations,
      (cudaStream_t)stream);
}

int gb_forward_kinematics(const gb_model* M, int precision, int layout, long B, const double* q, const double* v,
                          const double* a, double* oMi, double* vout, double* aout, void* stream) {
  GB_TRY(gbi::check_common_mimic(M, precision, layout, B));
  if (a && !v) return set_error(GB_ERR_INVALID_ARGUMENT, "an acceleration needs a velocity");
  if ((vout && !v) || (aout && !a)) return set_error(GB_ERR_INVALID_ARGUMENT, "velocity / acceleration output without input");
  if (B == 0) return GB_OK;
  GB_TRY(gbi::check_ptr(q, "q")); GB_TRY(gbi::check_ptr(oMi, "oMi"));
  if (v) GB_TRY(gbi::check_ptr(v, "v"));
  if (a) GB_TRY(gbi::check_ptr(a, "a"));
  if (vout) GB_TRY(gbi::check_ptr(vout, "v output"));
  if (aout) GB_TRY(gbi::check_ptr(aout, "a output"));
  const long nj = M->nj_user;
  return (M->has_mimic ? gbi::launch_fk_mimic : gbi::launch_fk)(
      M, precision, B, gbi::arr(q, layout, B, M->nq_red), gbi::arr(v, layout, B, M->nv_red),
      gbi::arr(a, layout, B, M->nv_red), gbi::arr(oMi, layout, B, 12 * nj), gbi::arr(vout, layout, B, 6 * nj),
      gbi::arr(aout, layout, B, 6 * nj), (cudaStream_t)stream);
}

int gb_compute_joint_jacobians(const gb_model* M, int precision, int layout, long B, const double* q, double* J,
                               void* stream) {
  GB_TRY(gbi::check_common_mimic(M, precision, layout, B));
  if (B == 0) return GB_OK;
  GB_TRY(gbi::check_ptr(q, "q")); GB_TRY(gbi::check_ptr(J, "J"));
  // 6 x nvExtended (data.J of a model with mimic joints has their columns too)
  return (M->has_mimic ? gbi::launch_jacobians_mimic : gbi::launch_jacobians)(
      M, precision, B, gbi::arr(q, layout, B, M->nq_red), gbi::arr(J, layout, B, 6L * M->nv), (cudaStream_t)stream);
}

int gb_aba(const gb_model* M, int precision, int convention, int layout, long B, const double* q, const double* v,
           const double* tau, double* ddq, void* stream) {
  GB_TRY(gbi::check_common(M, precision, layout, B));
  if (convention != GB_LOCAL && convention != GB_WORLD) return set_error(GB_ERR_INVALID_ARGUMENT, "unknown convention");
  if (B == 0) return GB_OK;
  GB_TRY(gbi::check_ptr(q, "q")); GB_TRY(gbi::check_ptr(v, "v")); GB_TRY(gbi::check_ptr(tau, "tau"));
  GB_TRY(gbi::check_ptr(ddq, "ddq"));
  return gbi::launch_aba(M, precision, B, gbi::arr(q, layout, B, M->nq), gbi::arr(v, layout, B, M->nv),
                         gbi::arr(tau, layout, B, M->nv), gbi::arr(ddq, layout, B, M->nv), (cudaStream_t)stream);
}

int gb_aba_fext(const gb_model* M, int precision, int convention, int layout, long B, const double* q,
                const double* v, const double* tau, const double* fext, double* ddq, void* stream) {
  GB_TRY(gbi::check_common(M, precision, layout, B));
  if (convention != GB_LOCAL && convention != GB_WORLD) return set_error(GB_ERR_INVALID_ARGUMENT, "unknown convention");
  if (B == 0) return GB_OK;
  GB_TRY(gbi::check_ptr(q, "q")); GB_TRY(gbi::check_ptr(v, "v")); GB_TRY(gbi::check_ptr(tau, "tau"));
  GB_TRY(gbi::check_ptr(fext, "fext")); GB_TRY(gbi::check_ptr(ddq, "ddq"));
  return gbi::launch_aba_fext(M, precision, B, gbi::arr(q, layout, B, M->nq), gbi::arr(v, layout, B, M->nv),
                              gbi::arr(tau, layout, B, M->nv), gbi::arr(fext, layout, B, 6L * M->nj_user),
                              gbi::arr(ddq, layout, B, M->nv), (cudaStream_t)stream);
}

int gb_crba(const gb_model* M, int precision, int convention, int matrix_mode, int layout, long B, const double* q,
            double* Mout, double* U, double* D, void* stream) {
  GB_TRY(gbi::check_common_mimic(M, precision, layout, B));
  if (M->has_mimic && U) return set_error(GB_ERR_UNSUPPORTED, "the Cholesky decomposition does not support mimic joints");
  if (convention != GB_LOCAL && convention != GB_WORLD) return set_error(GB_ERR_INVALID_ARGUMENT, "unknown convention");
  if (matrix_mode != GB_MATRIX_UPPER && matrix_mode != GB_MATRIX_SYMMETRIC)
    return set_error(GB_ERR_INVALID_ARGUMENT, "unknown matrix mode");
  if ((U == nullptr) != (D == nullptr)) return set_error(GB_ERR_INVALID_ARGUMENT, "U and D must both be set or both NULL");
  if (B == 0) return GB_OK;
  GB_TRY(gbi::check_ptr(q, "q")); GB_TRY(gbi::check_ptr(Mout, "M"));
  if (U) { GB_TRY(gbi::check_ptr(U, "U")); GB_TRY(gbi::check_ptr(D, "D")); }
  if (M->has_mimic)
    return gbi::launch_crba_mimic(M, precision, matrix_mode == GB_MATRIX_SYMMETRIC, B, gbi::arr(q, layout, B, M->nq_red),
                                  gbi::arr(Mout, layout, B, (long)M->nv_red * M->nv_red), (cudaStream_t)stream);
  const long nn = (long)M->nv * M->nv;
  return gbi::launch_crba(M, precision, matrix_mode == GB_MATRIX_SYMMETRIC, B, gbi::arr(q, layout, B, M->nq),
                          gbi::arr(Mout, layout, B, nn), gbi::arr(U, layout, B, nn), gbi::arr(D, layout, B, M->nv),
                          (cudaStream_t)stream);
}

int gb_integrate(const gb_model* M, int layout, long B, const double* q, const double* v, double* qout, void* stream) {
  GB_TRY(gbi::check_common_mimic(M, GB_FP64, layout, B));
  if (B == 0) return GB_OK;
  GB_TRY(gbi::check_ptr(q, "q")); GB_TRY(gbi::check_ptr(v, "v")); GB_TRY(gbi::check_ptr(qout, "qout"));
  return (M->has_mimic ? gbi::launch_integrate_mimic : gbi::launch_integrate)(
      M, B, gbi::arr(q, layout, B, M->nq_red), gbi::arr(v, layout, B, M->nv_red), gbi::arr(qout, layout, B, M->nq_red),
      (cudaStream_t)stream);
}

int gb_model_set_launch(gb_model* M, int function, int threads_per_block) {
  if (!M) return set_error(GB_ERR_INVALID_ARGUMENT, "model is NULL");
  if (function < GB_FUNC_RNEA || function > GB_FUNC_ABA_DERIVATIVES) return set_error(GB_ERR_INVALID_ARGUMENT, "unknown function");
  if (threads_per_block != 32 && threads_per_block != 64 && threads_per_block != 96 && threads_per_block != 128)
    return set_error(GB_ERR_INVALID_ARGUMENT, "threads_per_block must be 32, 64, 96 or 128");
  M->tpb[function] = threads_per_block;
  return GB_OK;
}

int gb_model_set_layout(gb_model* M, int function, int layout) {
  if (!M) return set_error(GB_ERR_INVALID_ARGUMENT, "model is NULL");
  if (function < GB_FUNC_RNEA || function > GB_FUNC_ABA_DERIVATIVES) return set_error(GB_ERR_INVALID_ARGUMENT, "unknown function");
  if (layout < GB_INSTANCE_PER_THREAD || layout > GB_INSTANCE_PER_BRANCH)
    return set_error(GB_ERR_INVALID_ARGUMENT, "unknown layout");
  if (M->has_three && layout != GB_INSTANCE_PER_THREAD)
    return set_error(GB_ERR_UNSUPPORTED, "spherical and planar joints run one configuration per thread");
  if (layout == GB_INSTANCE_PER_BRANCH && function != GB_FUNC_RNEA && function != GB_FUNC_ABA)
    return set_error(GB_ERR_UNSUPPORTED, "the lane-per-branch layout exists for RNEA and ABA");
  if (layout == GB_INSTANCE_PER_WARP && function != GB_FUNC_RNEA && function != GB_FUNC_ABA &&
      function != GB_FUNC_ABA_DERIVATIVES)
    return set_error(GB_ERR_UNSUPPORTED, "the warp-per-instance layout exists for RNEA, ABA and the ABA derivatives");
  if ((layout == GB_INSTANCE_PER_4_LANES || layout == GB_INSTANCE_PER_8_LANES) && function != GB_FUNC_ABA_DERIVATIVES)
    return set_error(GB_ERR_UNSUPPORTED, "lane teams of 4 or 8 exist for the ABA derivatives only");
  M->layout[function] = layout;
  return GB_OK;
}

// ---- ModelPool and the *InParallel entry points ------------------------------------------
int gb_pool_create(const gb_model* M, long size, gb_pool** out) {
  if (!M || !out) return set_error(GB_ERR_INVALID_ARGUMENT, "model/out is NULL");
  *out = nullptr;
  if (size <= 0) return set_error(GB_ERR_POOL, "The pool should have at least one element");
  gb_pool* P = new (std::nothrow) gb_pool();
  if (!P) return set_error(GB_ERR_INVALID_ARGUMENT, "out of host memory");
  P->model = M;
  P->size = size;
  cudaError_t e = cudaStreamCreateWithFlags(&P->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete P;
    return gbi::cuda_error(e, "gb_pool_create");
  }
  *out = P;
  return GB_OK;
}
int gb_pool_destroy(gb_pool* P) {
  if (!P) return GB_OK;
  if (P->d_buf) cudaFree(P->d_buf);
  if (P->stream) cudaStreamDestroy(P->stream);
  delete P;
  return GB_OK;
}
int gb_pool_size(const gb_pool* P, long* size) {
  if (!P || !size) return set_error(GB_ERR_INVALID_ARGUMENT, "pool/size is NULL");
  *size = P->size;
  return GB_OK;
}
int gb_pool_set_precision(gb_pool* P, int precision) {
  if (!P) return set_error(GB_ERR_INVALID_ARGUMENT, "pool is NULL");
  if (precision != GB_FP64 && precision != GB_MIXED) return set_error(GB_ERR_INVALID_ARGUMENT, "unknown precision");
  P->precision = precision;
  return GB_OK;
}

static int pool_buffers(gb_pool* P, size_t bytes) {
  if (bytes <= P->d_bytes) return GB_OK;
  if (P->d_buf) cudaFree(P->d_buf);
  P->d_buf = nullptr;
  P->d_bytes = 0;
  cudaError_t e = cudaMalloc(&P->d_buf, bytes);
  if (e != cudaSuccess) return gbi::cuda_error(e, "pool buffers");
  P->d_bytes = bytes;
  return GB_OK;
}

// checks of algorithm/parallel/{rnea,aba}.hpp:53-69
static int parallel_checks(long num_threads, gb_pool* P, long B) {
  if (!P) return set_error(GB_ERR_INVALID_ARGUMENT, "pool is NULL");
  if (P->size <= 0) return set_error(GB_ERR_POOL, "The pool should have at least one element");
  if (num_threads > P->size) return set_error(GB_ERR_POOL, "The pool is too small");
  if (num_threads < 1) return set_error(GB_ERR_POOL, "num_threads must be >= 1");
  if (B < 0) return set_error(GB_ERR_SIZE, "batch must be >= 0");
  return GB_OK;
}

typedef int (*launch3_fn)(const gb_model*, int, long, gbi::Arr, gbi::Arr, gbi::Arr, gbi::Arr, cudaStream_t);

static int in_parallel(gb_pool* P, long B, const double* q, const double* v, const double* x, double* out,
                       launch3_fn fn) {
  const gb_model* M = P->model;
  if (B == 0) return GB_OK;
  GB_TRY(gbi::check_ptr(q, "q")); GB_TRY(gbi::check_ptr(v, "v")); GB_TRY(gbi::check_ptr(x, "x"));
  GB_TRY(gbi::check_ptr(out, "out"));
  const size_t nq = M->nq_red, nv = M->nv_red;
  const size_t bytes = sizeof(double) * (size_t)B * (nq + 3 * nv);
  GB_TRY(pool_buffers(P, bytes));
  double* dq = P->d_buf;
  double* dv = dq + (size_t)B * nq;
  double* dx = dv + (size_t)B * nv;
  double* dout = dx + (size_t)B * nv;
  cudaStream_t st = P->stream;
  cudaError_t e = cudaMemcpyAsync(dq, q, sizeof(double) * B * nq, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dv, v, sizeof(double) * B * nv, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dx, x, sizeof(double) * B * nv, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return gbi::cuda_error(e, "host-to-device copy");
  GB_TRY(fn(M, P->precision, B, gbi::arr(dq, GB_LAYOUT_INSTANCE, B, nq), gbi::arr(dv, GB_LAYOUT_INSTANCE, B, nv),
            gbi::arr(dx, GB_LAYOUT_INSTANCE, B, nv), gbi::arr(dout, GB_LAYOUT_INSTANCE, B, nv), st));
  e = cudaMemcpyAsync(out, dout, sizeof(double) * B * nv, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return gbi::cuda_error(e, "device-to-host copy");
}

int gb_rnea_in_parallel(long num_threads, gb_pool* P, long B, const double* q, const double* v, const double* a,
                        double* tau) {
  GB_TRY(parallel_checks(num_threads, P, B));
  return in_parallel(P, B, q, v, a, tau, P->model->has_mimic ? gbi::launch_rnea_mimic : gbi::launch_rnea);
}

int gb_aba_in_parallel(long num_threads, gb_pool* P, long B, const double* q, const double* v, const double* tau,
                       double* a) {
  GB_TRY(parallel_checks(num_threads, P, B));
  if (P->model->has_mimic) return set_error(GB_ERR_UNSUPPORTED, "Function does not support mimic joints");
  return in_parallel(P, B, q, v, tau, a, gbi::launch_aba);
}

}  // extern "C"
