// Mimic joints (JointModelMimic, reference multibody/joint/joint-mimic.hpp:557-760) on the
// batched path.  The kernels run the extended tree, in which every mimic joint is a joint with
// its own dof; around them, one thread per configuration maps the caller's arrays:
//   q_ext: copies of the caller's entries, q_i = scaling q_j + offset for a mimic joint i of
//          joint j (LinearAffineTransform), or (cos, sin) of scaling * atan2(s, c) + offset for an
//          unbounded one (UnboundedRevoluteAffineTransform, joint-common-operations.hpp:52-90);
//   v_ext = G v, a_ext = G a  (G: one entry per extended dof, 1 or the mimic's scaling);
//   tau = G^T tau_ext  (the reference's RNEA adds S_i^T f_i of a mimic joint to its mimicked
//          joint's torque: JointMappedVelocitySelector, rnea.hxx:102-104);
//   M = G^T M_ext G  (the reduced joint-space inertia; the reference's CRBA builds the same
//          matrix in place, crba.hxx:112-215, and its unit tests check it against this product).
// The extended arrays are [element][configuration] scratch, so the maps' reads and writes of them
// coalesce; the caller's arrays keep their layout.
#include <cuda_runtime.h>

#include "gb_internal.h"

#define GB_TRY(x)                   \
  do {                              \
    const int rc__ = (x);           \
    if (rc__ != GB_OK) return rc__; \
  } while (0)

namespace gbi {
namespace {

constexpr int kThreads = 128;

__device__ inline double at(const Arr& x, long b, long k) { return x.p[b * x.is + k * x.es]; }
__device__ inline double& at_mut(const Arr& x, long b, long k) { return const_cast<double*>(x.p)[b * x.is + k * x.es]; }

__global__ void __launch_bounds__(kThreads)
    k_mimic_expand(long B, int nq, int nv, const gb::MimicQ* __restrict__ qm, const gb::MimicV* __restrict__ vm,
                   Arr q, Arr v, Arr a, double* qe, double* ve, double* ae) {
  const long b = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  if (qe)
    for (int e = 0; e < nq; ++e) {
      const gb::MimicQ m = qm[e];
      if (m.kind == 0) {
        qe[(long)e * B + b] = at(q, b, m.src);
      } else if (m.kind == 1) {
        qe[(long)e * B + b] = m.scaling * at(q, b, m.src) + m.offset;
      } else if (m.kind == 2) {
        const double th = m.scaling * atan2(at(q, b, m.src + 1), at(q, b, m.src)) + m.offset;
        double s, c;
        sincos(th, &s, &c);
        qe[(long)e * B + b] = c;
        qe[(long)(e + 1) * B + b] = s;
      }
    }
  for (int e = 0; e < nv; ++e) {
    const gb::MimicV m = vm[e];
    if (ve) ve[(long)e * B + b] = m.g * at(v, b, m.src);
    if (ae) ae[(long)e * B + b] = m.g * at(a, b, m.src);
  }
}

// out = G^T x (x extended, [element][configuration]); out has nv_red entries
__global__ void __launch_bounds__(kThreads)
    k_mimic_reduce_vec(long B, int nv, int nv_red, const gb::MimicV* __restrict__ vm, const double* x, Arr out) {
  const long b = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  for (int r = 0; r < nv_red; ++r) at_mut(out, b, r) = 0.0;
  for (int e = 0; e < nv; ++e) at_mut(out, b, vm[e].src) += vm[e].g * x[(long)e * B + b];
}

// out = G^T X G (X extended nv x nv row-major, [element][configuration]); upper: the caller's
// strictly lower triangle is left zero
__global__ void __launch_bounds__(kThreads)
    k_mimic_reduce_mat(long B, int nv, int nv_red, const gb::MimicV* __restrict__ vm, const double* X, Arr out,
                       int upper) {
  const long b = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const long nn = (long)nv_red * nv_red;
  for (long k = 0; k < nn; ++k) at_mut(out, b, k) = 0.0;
  for (int r = 0; r < nv; ++r) {
    const gb::MimicV mr = vm[r];
    for (int c = 0; c < nv; ++c) {
      const gb::MimicV mc = vm[c];
      if (upper && mc.src < mr.src) continue;
      at_mut(out, b, (long)mr.src * nv_red + mc.src) += mr.g * mc.g * X[((long)r * nv + c) * B + b];
    }
  }
}

// the caller's configuration from an extended one: the entries the caller owns
__global__ void __launch_bounds__(kThreads)
    k_mimic_compress_q(long B, int nq, const gb::MimicQ* __restrict__ qm, const double* qe, Arr out) {
  const long b = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  for (int e = 0; e < nq; ++e)
    if (qm[e].kind == 0) at_mut(out, b, qm[e].src) = qe[(long)e * B + b];
}

const gb::MimicQ* qmap(const gb_model* M) { return static_cast<const gb::MimicQ*>(M->d_mimic); }
const gb::MimicV* vmap(const gb_model* M) {
  return reinterpret_cast<const gb::MimicV*>(static_cast<const unsigned char*>(M->d_mimic) +
                                             sizeof(gb::MimicQ) * (size_t)M->nq);
}
bool is_zero(const Arr& x) { return x.is == 0 && x.es == 0; }
unsigned grid_of(long B) { return (unsigned)((B + kThreads - 1) / kThreads); }

// extended scratch of q (nq), v, a (nv each, when given and not the zero vector) and an output
// of `nout` doubles per configuration
struct Ext {
  void* mem = nullptr;
  double *q = nullptr, *v = nullptr, *a = nullptr, *out = nullptr;
};
int expand(const gb_model* M, long B, Arr q, const Arr* v, const Arr* a, long nout, Ext& x, cudaStream_t st) {
  const bool hv = v && !is_zero(*v) && v->p, ha = a && !is_zero(*a) && a->p;
  const size_t doubles = (size_t)B * ((size_t)M->nq + (hv ? M->nv : 0) + (ha ? M->nv : 0) + (size_t)nout);
  GB_TRY(scratch_alloc(&x.mem, sizeof(double) * doubles, st));
  double* p = static_cast<double*>(x.mem);
  x.q = p;
  p += (size_t)B * M->nq;
  if (hv) { x.v = p; p += (size_t)B * M->nv; }
  if (ha) { x.a = p; p += (size_t)B * M->nv; }
  x.out = nout > 0 ? p : nullptr;
  k_mimic_expand<<<grid_of(B), kThreads, 0, st>>>(B, M->nq, M->nv, qmap(M), vmap(M), q, hv ? *v : q, ha ? *a : q,
                                                   x.q, x.v, x.a);
  const int rc = cuda_error(cudaGetLastError(), "k_mimic_expand");
  if (rc != GB_OK) scratch_free(x.mem, st);
  return rc;
}
Arr soa(const double* p, long B) { return Arr{p, 1, B}; }
Arr ext_or(const double* p, const Arr& given, long B) { return p ? soa(p, B) : given; }

}  // namespace

int launch_rnea_mimic(const gb_model* M, int precision, long B, Arr q, Arr v, Arr a, Arr tau, cudaStream_t st) {
  Ext x;
  GB_TRY(expand(M, B, q, &v, &a, M->nv, x, st));
  int rc = launch_rnea(M, precision, B, soa(x.q, B), ext_or(x.v, v, B), ext_or(x.a, a, B), soa(x.out, B), st);
  if (rc == GB_OK) {
    k_mimic_reduce_vec<<<grid_of(B), kThreads, 0, st>>>(B, M->nv, M->nv_red, vmap(M), x.out, tau);
    rc = cuda_error(cudaGetLastError(), "k_mimic_reduce_vec");
  }
  scratch_free(x.mem, st);
  return rc;
}

int launch_rnea_fext_mimic(const gb_model* M, int precision, long B, Arr q, Arr v, Arr a, Arr fext, Arr tau,
                           cudaStream_t st) {
  Ext x;
  GB_TRY(expand(M, B, q, &v, &a, M->nv, x, st));
  int rc = launch_rnea_fext(M, precision, B, soa(x.q, B), ext_or(x.v, v, B), ext_or(x.a, a, B), fext, soa(x.out, B),
                            st);
  if (rc == GB_OK) {
    k_mimic_reduce_vec<<<grid_of(B), kThreads, 0, st>>>(B, M->nv, M->nv_red, vmap(M), x.out, tau);
    rc = cuda_error(cudaGetLastError(), "k_mimic_reduce_vec");
  }
  scratch_free(x.mem, st);
  return rc;
}

int launch_crba_mimic(const gb_model* M, int precision, bool symmetric, long B, Arr q, Arr Mout, cudaStream_t st) {
  Ext x;
  GB_TRY(expand(M, B, q, nullptr, nullptr, (long)M->nv * M->nv, x, st));
  const Arr none{nullptr, 0, 0};
  int rc = launch_crba(M, precision, true, B, soa(x.q, B), soa(x.out, B), none, none, st);
  if (rc == GB_OK) {
    k_mimic_reduce_mat<<<grid_of(B), kThreads, 0, st>>>(B, M->nv, M->nv_red, vmap(M), x.out, Mout, symmetric ? 0 : 1);
    rc = cuda_error(cudaGetLastError(), "k_mimic_reduce_mat");
  }
  scratch_free(x.mem, st);
  return rc;
}

int launch_fk_mimic(const gb_model* M, int precision, long B, Arr q, Arr v, Arr a, Arr oMi, Arr vout, Arr aout,
                    cudaStream_t st) {
  Ext x;
  GB_TRY(expand(M, B, q, &v, &a, 0, x, st));
  const int rc = launch_fk(M, precision, B, soa(x.q, B), ext_or(x.v, v, B), ext_or(x.a, a, B), oMi, vout, aout, st);
  scratch_free(x.mem, st);
  return rc;
}

int launch_jacobians_mimic(const gb_model* M, int precision, long B, Arr q, Arr J, cudaStream_t st) {
  Ext x;
  GB_TRY(expand(M, B, q, nullptr, nullptr, 0, x, st));
  const int rc = launch_jacobians(M, precision, B, soa(x.q, B), J, st);
  scratch_free(x.mem, st);
  return rc;
}

int launch_integrate_mimic(const gb_model* M, long B, Arr q, Arr v, Arr qout, cudaStream_t st) {
  Ext x;
  GB_TRY(expand(M, B, q, &v, nullptr, M->nq, x, st));
  int rc = launch_integrate(M, B, soa(x.q, B), soa(x.v, B), soa(x.out, B), st);
  if (rc == GB_OK) {
    k_mimic_compress_q<<<grid_of(B), kThreads, 0, st>>>(B, M->nq, qmap(M), x.out, qout);
    rc = cuda_error(cudaGetLastError(), "k_mimic_compress_q");
  }
  scratch_free(x.mem, st);
  return rc;
}

}  // namespace gbi
