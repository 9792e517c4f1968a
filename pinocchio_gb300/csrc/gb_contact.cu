// Contact dynamics with a given constraint Jacobian: forwardDynamics and
// impulseDynamics (reference algorithm/contact-dynamics.hxx:81-165, 255-327).
//
// Three launches per call: the CRBA with its FP64 tree factorisation
// M = U D U^T (k_crba), the bias forces nle = rnea(q, v, 0) (forward dynamics
// only; FP32 sweeps in mixed precision), then k_contact: one thread per
// configuration forms sDUiJt = D^-1/2 U^-1 J^T, the Delassus matrix
// J M^-1 J^T = sDUiJt^T sDUiJt (+ inv_damping I), its LLT, the multipliers and
// the accelerations (velocities after impact) with the tree-sparse solves of
// cholesky.hxx.  U, D, nle and the per-configuration matrices live in a
// stream-ordered scratch laid out [element][configuration], so the lanes of a
// warp touch consecutive addresses; everything after the CRBA is FP64.
#include "gb_dyn.cuh"
#include "gb_internal.h"

namespace gbi {
namespace {

constexpr int kThreads = 128;

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

// One configuration's view of an [element][configuration] scratch array.
struct Col {
  double* p;
  long s;
  __device__ double& operator[](long k) const { return p[k * s]; }
};

// v <- U^-1 v (cholesky.hxx:210-235); U unit upper, row-major nv x nv; row k has
// non-zeros right of the diagonal only in its subtree (nvSubtree_fromRow[k] - 1 entries)
__device__ void chol_uiv(const gb::MView& m, const Col& U, const Col& v, int vs) {
  const int nv = m.nv;
  for (int k = nv - 2; k >= 0; --k) {
    const int n = m.nsfr[k] - 1;
    double s = 0.0;
    for (int j = 1; j <= n; ++j) s += U[(long)k * nv + k + j] * v[(long)(k + j) * vs];
    v[(long)k * vs] -= s;
  }
}
// v <- U^-T v (cholesky.hxx:275-296)
__device__ void chol_utiv(const gb::MView& m, const Col& U, const Col& v) {
  const int nv = m.nv;
  for (int k = 0; k < nv - 1; ++k) {
    const int n = m.nsfr[k] - 1;
    const double vk = v[k];
    for (int j = 1; j <= n; ++j) v[k + j] -= U[(long)k * nv + k + j] * vk;
  }
}
// v <- M^-1 v = U^-T D^-1 U^-1 v (cholesky.hxx:483-500)
__device__ void chol_solve(const gb::MView& m, const Col& U, const Col& D, const Col& v) {
  chol_uiv(m, U, v, 1);
  for (int k = 0; k < m.nv; ++k) v[k] *= 1.0 / D[k];
  chol_utiv(m, U, v);
}

// sDUiJt = D^-1/2 U^-1 J^T (nv x nc row-major, in Y), the Delassus matrix
// J M^-1 J^T + inv_damping I and its lower LLT in place (in G, nc x nc)
__device__ void delassus_llt(const gb::MView& m, const Col& U, const Col& D, const gb::In& Ji, int nc,
                             double inv_damping, const Col& Y, const Col& G) {
  const int nv = m.nv;
  const long B = Y.s;
  for (int r = 0; r < nv; ++r)
    for (int c = 0; c < nc; ++c) Y[(long)r * nc + c] = Ji[c * nv + r];
  for (int c = 0; c < nc; ++c) chol_uiv(m, U, Col{Y.p + (long)c * B, B}, nc);
  for (int r = 0; r < nv; ++r) {
    gb::check_pivot(m, D[r]);
    const double sd = sqrt(D[r]);
    for (int c = 0; c < nc; ++c) Y[(long)r * nc + c] /= sd;
  }
  for (int i = 0; i < nc; ++i)
    for (int j = 0; j <= i; ++j) {
      double s = 0.0;
      for (int r = 0; r < nv; ++r) s += Y[(long)r * nc + i] * Y[(long)r * nc + j];
      G[(long)i * nc + j] = s + (i == j ? inv_damping : 0.0);
    }
  for (int j = 0; j < nc; ++j) {
    double s = G[(long)j * nc + j];
    for (int k = 0; k < j; ++k) s -= G[(long)j * nc + k] * G[(long)j * nc + k];
    gb::check_pivot(m, s);
    const double ljj = sqrt(s);
    G[(long)j * nc + j] = ljj;
    for (int i = j + 1; i < nc; ++i) {
      double t = G[(long)i * nc + j];
      for (int k = 0; k < j; ++k) t -= G[(long)i * nc + k] * G[(long)j * nc + k];
      G[(long)i * nc + j] = t / ljj;
    }
  }
}
// x <- (L L^T)^-1 x with the factor of delassus_llt
__device__ void llt_solve(const Col& G, int nc, const Col& x) {
  for (int i = 0; i < nc; ++i) {
    double t = x[i];
    for (int k = 0; k < i; ++k) t -= G[(long)i * nc + k] * x[k];
    x[i] = t / G[(long)i * nc + i];
  }
  for (int i = nc - 1; i >= 0; --i) {
    double t = x[i];
    for (int k = i + 1; k < nc; ++k) t -= G[(long)k * nc + i] * x[k];
    x[i] = t / G[(long)i * nc + i];
  }
}

// computeKKTContactDynamicMatrixInverse (contact-dynamics.hxx:166-225): the inverse of
// [[M, J^T], [J, -inv_damping I]] (n = nv + nc, row-major), built in the output itself:
// bottomRight = -(J M^-1 J^T + mu I)^-1, topLeft = M^-1, bottomLeft = J M^-1, topRight =
// bottomLeft^T (-bottomRight), topLeft -= topRight bottomLeft, bottomLeft = topRight^T.
__global__ void __launch_bounds__(kThreads)
    k_kkt_inverse(const unsigned char* blob, int bytes, long B, int nc, const double* Us, const double* Ds, double* Ys,
                  double* Gs, Arr J, double inv_damping, Arr K) {
  extern __shared__ __align__(16) unsigned char smem[];
  const gb::MView m = stage_model(blob, bytes, smem);
  const long b = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const int nv = m.nv, n = nv + nc;
  const Col U{const_cast<double*>(Us) + b, B}, D{const_cast<double*>(Ds) + b, B};
  const Col Y{Ys + b, B}, G{Gs + b, B};
  const gb::In Ji{J.p + b * J.is, J.es};
  double* o = const_cast<double*>(K.p) + b * K.is;
  const long es = K.es;
  auto at = [&](int r, int c) -> double& { return o[((long)r * n + c) * es]; };
  if (nc > 0) delassus_llt(m, U, D, Ji, nc, inv_damping, Y, G);
  for (int c = 0; c < nv; ++c) {  // topLeft = M^-1, column by column
    const Col col{o + (long)c * es, (long)n * es};
    for (int k = 0; k < nv; ++k) col[k] = k == c ? 1.0 : 0.0;
    chol_solve(m, U, D, col);
  }
  for (int j = 0; j < nc; ++j) {  // bottomRight = -G^-1
    const Col col{o + ((long)nv * n + nv + j) * es, (long)n * es};
    for (int i = 0; i < nc; ++i) col[i] = i == j ? -1.0 : 0.0;
    llt_solve(G, nc, col);
  }
  for (int i = 0; i < nc; ++i)  // bottomLeft = J topLeft
    for (int c = 0; c < nv; ++c) {
      double s = 0.0;
      for (int k = 0; k < nv; ++k) s += Ji[i * nv + k] * at(k, c);
      at(nv + i, c) = s;
    }
  for (int r = 0; r < nv; ++r)  // topRight = bottomLeft^T (-bottomRight)
    for (int j = 0; j < nc; ++j) {
      double s = 0.0;
      for (int i = 0; i < nc; ++i) s += at(nv + i, r) * -at(nv + i, nv + j);
      at(r, nv + j) = s;
    }
  for (int r = 0; r < nv; ++r)  // topLeft -= topRight bottomLeft
    for (int c = 0; c < nv; ++c) {
      double s = 0.0;
      for (int j = 0; j < nc; ++j) s += at(r, nv + j) * at(nv + j, c);
      at(r, c) -= s;
    }
  for (int r = 0; r < nv; ++r)  // bottomLeft = topRight^T
    for (int j = 0; j < nc; ++j) at(nv + j, r) = at(r, nv + j);
}

// IMPULSE: impulseDynamics (x = v_before); otherwise forwardDynamics (x = tau,
// nle and gamma read, r = M^-1 (tau - nle) kept in the scratch R).
template <bool IMPULSE>
__global__ void __launch_bounds__(kThreads)
    k_contact(const unsigned char* blob, int bytes, long B, int nc, const double* Us, const double* Ds,
              const double* nles, double* Rs, double* Ys, double* Gs, Arr x, Arr J, Arr gamma, double r_coeff,
              double inv_damping, Arr out, Arr lam) {
  extern __shared__ __align__(16) unsigned char smem[];
  const gb::MView m = stage_model(blob, bytes, smem);
  const long b = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const int nv = m.nv;
  const Col U{const_cast<double*>(Us) + b, B}, D{const_cast<double*>(Ds) + b, B};
  const Col Y{Ys + b, B}, G{Gs + b, B};
  const gb::In xi{x.p + b * x.is, x.es}, Ji{J.p + b * J.is, J.es};
  const gb::Out o{const_cast<double*>(out.p) + b * out.is, out.es}, l{const_cast<double*>(lam.p) + b * lam.is, lam.es};
  // the free term: r = M^-1 (tau - nle) (forward) or v_before (impulse)
  const Col R{Rs + b, B};
  if (!IMPULSE) {
    const Col nle{const_cast<double*>(nles) + b, B};
    for (int k = 0; k < nv; ++k) R[k] = xi[k] - nle[k];
    chol_solve(m, U, D, R);
  } else {
    for (int k = 0; k < nv; ++k) R[k] = xi[k];
  }
  if (nc > 0) {
    delassus_llt(m, U, D, Ji, nc, inv_damping, Y, G);
    // right-hand side: -J r - gamma (forward) or -(1 + r_coeff) J v_before (impulse)
    for (int c = 0; c < nc; ++c) {
      double s = 0.0;
      for (int k = 0; k < nv; ++k) s += Ji[c * nv + k] * R[k];
      l[c] = IMPULSE ? (-r_coeff - 1.0) * s : -s - gamma.p[b * gamma.is + (long)c * gamma.es];
    }
    llt_solve(G, nc, Col{l.p, l.es});
  }
  // out = M^-1 J^T lambda + r; the product is formed in the scratch column, then written
  const Col A{Y.p, B};  // sDUiJt is no longer needed: its first nv entries hold J^T lambda
  for (int k = 0; k < nv; ++k) {
    double s = 0.0;
    for (int c = 0; c < nc; ++c) s += Ji[c * nv + k] * l[c];
    A[k] = s;
  }
  chol_solve(m, U, D, A);
  for (int k = 0; k < nv; ++k) o[k] = A[k] + R[k];
}

}  // namespace

int launch_contact(const gb_model* M, int precision, bool impulse, long B, int nc, Arr q, Arr v, Arr x, Arr J,
                   Arr gamma, double r_coeff, double inv_damping, Arr out, Arr lam, cudaStream_t st) {
  const long nv = M->nv, nn = nv * nv;
  // scratch, [element][configuration]: M, U (nn), D, nle, r (nv), sDUiJt (nv * max(nc, 1)), G (nc * nc)
  const long ny = nv * (nc > 0 ? nc : 1), ng = (long)nc * nc;
  void* scratch = nullptr;
  int rc = scratch_alloc(&scratch, sizeof(double) * (size_t)B * (2 * nn + 3 * nv + ny + ng), st);
  if (rc != GB_OK) return rc;
  double* base = static_cast<double*>(scratch);
  double *Ms = base, *Us = Ms + nn * B, *Ds = Us + nn * B, *nles = Ds + nv * B, *Rs = nles + nv * B,
         *Ys = Rs + nv * B, *Gs = Ys + ny * B;
  rc = launch_crba(M, GB_FP64, false, B, q, Arr{Ms, 1, B}, Arr{Us, 1, B}, Arr{Ds, 1, B}, st);
  if (rc == GB_OK && !impulse) {
    const gb::BlobHeader* h = reinterpret_cast<const gb::BlobHeader*>(M->blob.data());
    const Arr zero{reinterpret_cast<const double*>(M->d_blob + h->o_zero), 0, 0};
    rc = launch_rnea(M, precision, B, q, v, zero, Arr{nles, 1, B}, st);
  }
  if (rc == GB_OK) {
    const void* kern = impulse ? (const void*)k_contact<true> : (const void*)k_contact<false>;
    if (M->stage_bytes > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, M->stage_bytes);
      if (e != cudaSuccess) rc = cuda_error(e, "k_contact");
    }
  }
  if (rc == GB_OK) {
    const long grid = (B + kThreads - 1) / kThreads;
    if (impulse)
      k_contact<true><<<(unsigned)grid, kThreads, M->stage_bytes, st>>>(M->d_blob, M->stage_bytes, B, nc, Us, Ds, nles,
                                                                        Rs, Ys, Gs, x, J, gamma, r_coeff, inv_damping,
                                                                        out, lam);
    else
      k_contact<false><<<(unsigned)grid, kThreads, M->stage_bytes, st>>>(M->d_blob, M->stage_bytes, B, nc, Us, Ds,
                                                                         nles, Rs, Ys, Gs, x, J, gamma, r_coeff,
                                                                         inv_damping, out, lam);
    rc = cuda_error(cudaGetLastError(), "k_contact");
  }
  scratch_free(scratch, st);
  return rc;
}

int launch_kkt_inverse(const gb_model* M, long B, int nc, Arr q, Arr J, double inv_damping, Arr K, cudaStream_t st) {
  const long nv = M->nv, nn = nv * nv;
  const long ny = nv * (nc > 0 ? nc : 1), ng = (long)nc * nc;
  void* scratch = nullptr;
  int rc = scratch_alloc(&scratch, sizeof(double) * (size_t)B * (2 * nn + nv + ny + ng), st);
  if (rc != GB_OK) return rc;
  double* base = static_cast<double*>(scratch);
  double *Ms = base, *Us = Ms + nn * B, *Ds = Us + nn * B, *Ys = Ds + nv * B, *Gs = Ys + ny * B;
  rc = launch_crba(M, GB_FP64, false, B, q, Arr{Ms, 1, B}, Arr{Us, 1, B}, Arr{Ds, 1, B}, st);
  if (rc == GB_OK && M->stage_bytes > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute((const void*)k_kkt_inverse, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         M->stage_bytes);
    if (e != cudaSuccess) rc = cuda_error(e, "k_kkt_inverse");
  }
  if (rc == GB_OK) {
    const long grid = (B + kThreads - 1) / kThreads;
    k_kkt_inverse<<<(unsigned)grid, kThreads, M->stage_bytes, st>>>(M->d_blob, M->stage_bytes, B, nc, Us, Ds, Ys, Gs,
                                                                     J, inv_damping, K);
    rc = cuda_error(cudaGetLastError(), "k_kkt_inverse");
  }
  scratch_free(scratch, st);
  return rc;
}

}  // namespace gbi
