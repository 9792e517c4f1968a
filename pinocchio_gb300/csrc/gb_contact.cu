// Contact dynamics with a given constraint Jacobian: forwardDynamics and
// impulseDynamics (reference algorithm/contact-dynamics.hxx:81-165, 255-327); and
// constraintDynamics with rigid constraint models (constrained-dynamics.hxx:188-520).
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


// ---- constraintDynamics with rigid constraint models (algorithm/constrained-dynamics.hxx:188-520) ----
// Two more launches after the CRBA and the bias forces: k_constraint_setup (world-frame kinematics,
// the constraint Jacobian rows and drifts of every constraint model) and k_constraint_solve (the
// Delassus factorisation and the proximal iterations).  The reference factorises the whole KKT matrix
// [[-mu I, J], [J^T, M]] (contact-cholesky.hxx:152-304); here M = U D U^T and the Delassus matrix
// J M^-1 J^T + mu I = L L^T are factorised apart, which gives the same iterates.

using X3d = gb::X3<double>;
using M6d = gb::M6<double>;

__device__ void load_se3(const double* P, X3d& X) {
#pragma unroll
  for (int k = 0; k < 9; ++k) X.R[k] = P[k];
#pragma unroll
  for (int k = 0; k < 3; ++k) X.t[k] = P[9 + k];
}
__device__ void se3_actinv(const X3d& A, const X3d& B, X3d& o) {  // A^-1 B
  double d[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) d[k] = B.t[k] - A.t[k];
  gb::mtv3(A.R, d, o.t);
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) o.R[3 * r + c] = A.R[r] * B.R[c] + A.R[3 + r] * B.R[3 + c] + A.R[6 + r] * B.R[6 + c];
}
// the angle-axis vector of a rotation, angle in [0, pi] (spatial/log.hxx:58-170): theta =
// atan2(|a|, (tr - 1) / 2) with a = unskew(R) = sin(theta) n; w = theta / sin(theta) a away from pi
// (a series of theta / sin(theta) near 0), near pi the axis from (R + R^T) / 2 - cos(theta) I =
// (1 - cos(theta)) n n^T with the sign of a
__device__ void log3(const double* R, double* w, double& theta) {
  const double a[3] = {0.5 * (R[7] - R[5]), 0.5 * (R[2] - R[6]), 0.5 * (R[3] - R[1])};
  const double s = sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
  const double c = fmin(1.0, fmax(-1.0, 0.5 * (R[0] + R[4] + R[8] - 1.0)));
  theta = atan2(s, c);
  if (theta < 3.0) {
    const double t2 = theta * theta;
    const double k = s < 1e-4 ? 1.0 + t2 / 6.0 + 7.0 * t2 * t2 / 360.0 : theta / s;
#pragma unroll
    for (int i = 0; i < 3; ++i) w[i] = k * a[i];
    return;
  }
  const double omc = 1.0 - c;
  int j = 0;
  if (R[4] > R[0]) j = 1;
  if (R[8] > R[4 * j]) j = 2;
  double n[3];
  n[j] = sqrt((R[4 * j] - c) / omc);
#pragma unroll
  for (int i = 0; i < 3; ++i)
    if (i != j) n[i] = (R[3 * i + j] + R[3 * j + i]) / (2.0 * omc * n[j]);
  const double sg = n[0] * a[0] + n[1] * a[1] + n[2] * a[2] < 0.0 ? -1.0 : 1.0;
#pragma unroll
  for (int i = 0; i < 3; ++i) w[i] = sg * theta * n[i];
}
// log6 of a placement (spatial/log.hxx:189-230): [alpha p - w x p / 2 + beta (w . p) w; w]
__device__ void log6(const X3d& M, M6d& o) {
  double w[3], theta;
  log3(M.R, w, theta);
  const double a[3] = {0.5 * (M.R[7] - M.R[5]), 0.5 * (M.R[2] - M.R[6]), 0.5 * (M.R[3] - M.R[1])};
  const double t2 = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
  double alpha, beta;
  if (M.R[0] + M.R[4] + M.R[8] >= 3.0 - 6.0554544523933395e-06) {  // 3 - eps^(1/3)
    alpha = 1.0 - t2 / 12.0 - t2 * t2 / 720.0;
    beta = 1.0 / 12.0 + t2 / 720.0;
  } else {
    double st, ct;
    sincos(theta, &st, &ct);
    alpha = theta * st / (2.0 * (1.0 - ct));
    beta = 1.0 / (theta * theta) - st / (2.0 * theta * (1.0 - ct));
  }
  double wxp[3];
  gb::cross3(w, M.t, wxp);
  const double wp = w[0] * M.t[0] + w[1] * M.t[1] + w[2] * M.t[2];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    o.v[k] = alpha * M.t[k] - 0.5 * wxp[k] + beta * wp * w[k];
    o.v[3 + k] = w[k];
  }
}

// Jlog6 = d log6(M exp6(d)) / dd at d = 0 (row-major 6 x 6, [linear; angular]): the inverse of SE(3)'s
// right Jacobian at (rho, phi) = log6(M), from the published closed form (Barfoot, State Estimation
// for Robotics, 7.1.5): [[Jr^-1, -Jr^-1 Qr Jr^-1], [0, Jr^-1]] with Jr^-1 = I + phi^ / 2 + c phi^2 and
// Qr the right-Jacobian coupling block (a1, a2, a3 below; Taylor series for small angles)
__device__ void jlog6(const X3d& M, double* J) {
  M6d xi;
  log6(M, xi);
  const double* rho = xi.v;
  const double* phi = xi.v + 3;
  const double t2 = phi[0] * phi[0] + phi[1] * phi[1] + phi[2] * phi[2], t = sqrt(t2);
  double c, a1, a2, a3;
  if (t < 1e-3) {
    c = 1.0 / 12.0 + t2 / 720.0;
    a1 = 1.0 / 6.0 - t2 / 120.0;
    a2 = 1.0 / 24.0 - t2 / 720.0;
    a3 = 1.0 / 120.0 - t2 / 2520.0;
  } else {
    double st, ct;
    sincos(t, &st, &ct);
    c = 1.0 / t2 - (1.0 + ct) / (2.0 * t * st);
    a1 = (t - st) / (t2 * t);
    a2 = (t2 + 2.0 * ct - 2.0) / (2.0 * t2 * t2);
    a3 = (2.0 * t - 3.0 * st + t * ct) / (2.0 * t2 * t2 * t);
  }
  auto skew = [](const double* v, double* S) {
    S[0] = 0.0; S[1] = -v[2]; S[2] = v[1];
    S[3] = v[2]; S[4] = 0.0; S[5] = -v[0];
    S[6] = -v[1]; S[7] = v[0]; S[8] = 0.0;
  };
  auto mul = [](const double* A, const double* B, double* C) {
    for (int r = 0; r < 3; ++r)
      for (int q = 0; q < 3; ++q) C[3 * r + q] = A[3 * r] * B[q] + A[3 * r + 1] * B[3 + q] + A[3 * r + 2] * B[6 + q];
  };
  double P[9], R[9], PP[9], PR[9], RP[9], PRP[9], X[9], Y[9], Jr[9], Q[9];
  skew(phi, P);
  skew(rho, R);
  mul(P, P, PP);
  mul(P, R, PR);
  mul(R, P, RP);
  mul(PR, P, PRP);
  for (int k = 0; k < 9; ++k) {
    Jr[k] = (k % 4 == 0 ? 1.0 : 0.0) + 0.5 * P[k] + c * PP[k];
    Q[k] = -0.5 * R[k] + a1 * (PR[k] + RP[k] - PRP[k]);
  }
  mul(PP, R, X);  // phi^ phi^ rho^, then + rho^ phi^ phi^ - 3 phi^ rho^ phi^
  mul(RP, P, Y);
  for (int k = 0; k < 9; ++k) Q[k] -= a2 * (X[k] + Y[k] - 3.0 * PRP[k]);
  mul(PRP, P, X);  // phi^ rho^ phi^ phi^ + phi^ phi^ rho^ phi^
  mul(PP, R, Y);
  mul(Y, P, R);
  for (int k = 0; k < 9; ++k) Q[k] += a3 * (X[k] + R[k]);
  mul(Jr, Q, X);
  mul(X, Jr, Y);
  for (int r = 0; r < 3; ++r)
    for (int q = 0; q < 3; ++q) {
      J[6 * r + q] = Jr[3 * r + q];
      J[6 * r + 3 + q] = -Y[3 * r + q];
      J[6 * (3 + r) + q] = 0.0;
      J[6 * (3 + r) + 3 + q] = Jr[3 * r + q];
    }
}
// ov.ang x (ov.lin + ov.ang x p): the velocity-product part of a point's classical acceleration
__device__ void point_drift(const M6d& ov, const double* p, double* o) {
  double wxp[3], vp[3];
  gb::cross3(ov.v + 3, p, wxp);
#pragma unroll
  for (int k = 0; k < 3; ++k) vp[k] = ov.v[k] + wxp[k];
  gb::cross3(ov.v + 3, vp, o);
}

// Per configuration: the world placements, velocities and velocity-product accelerations of every
// joint (ContactAndImpulseDynamicsForwardStep, constrained-dynamics.hxx:63-135), then per constraint
// model its placements (RigidConstraintModel::calc, contact-info.hpp:426-446), Jacobian rows
// (RigidConstraintModel::jacobian, contact-info.hpp:551-672) into Js and the right-hand side
// (-drift_1 + drift_2 + Baumgarte correction + desired acceleration, constrained-dynamics.hxx:282-432)
// into Rh, both [element][configuration].
template <int CAP>
__global__ void __launch_bounds__(kThreads)
    k_constraint_setup(const unsigned char* blob, int bytes, long B, Arr q, Arr v,
                       const ConstraintDev* __restrict__ tab, const signed char* __restrict__ sparsity, int ncon,
                       double* Js, double* Rh) {
  extern __shared__ __align__(16) unsigned char smem[];
  const gb::MView m = stage_model(blob, bytes, smem);
  const long b = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const int nv = m.nv;
  const gb::In qi{q.p + b * q.is, q.es}, vi{v.p + b * v.is, v.es};
  X3d oM[CAP];
  M6d ov[CAP], oa[CAP];
  gb::zero(ov[0]);
  gb::zero(oa[0]);
  for (int i = 1; i < m.nj; ++i) {
    const int p = m.parent[i];
    X3d X;
    gb::joint_transform(m, i, qi, X);
    if (p > 0) gb::compose(oM[p], X, oM[i]);
    else oM[i] = X;
    M6d vJ, w;
    gb::joint_motion(m.jtype[i], vi, m.idx_v[i], vJ);
    gb::act_motion(oM[i], vJ, w);
#pragma unroll
    for (int k = 0; k < 6; ++k) ov[i].v[k] = w.v[k] + ov[p].v[k];
    gb::cross_motion(ov[p], ov[i], w);  // zero for a root joint (ov[0] = 0)
#pragma unroll
    for (int k = 0; k < 6; ++k) oa[i].v[k] = w.v[k] + oa[p].v[k];
  }
  const Col J{Js + b, B}, Rhs{Rh + b, B};
  for (int e = 0; e < ncon; ++e) {
    const ConstraintDev& c = tab[e];
    const int n = c.type == GB_CONTACT_3D ? 3 : 6, j1 = c.j1, j2 = c.j2;
    X3d P1, P2, oMc1, oMc2, c12;
    load_se3(c.P1, P1);
    load_se3(c.P2, P2);
    if (j1 > 0) gb::compose(oM[j1], P1, oMc1);
    else oMc1 = P1;
    if (j2 > 0) gb::compose(oM[j2], P2, oMc2);
    else oMc2 = P2;
    se3_actinv(oMc1, oMc2, c12);
    const bool local = c.frame == GB_FRAME_LOCAL;
    // Jacobian rows: column jj of the world Jacobian, by the side(s) of the loop it moves
    for (int jj = 0; jj < nv; ++jj) {
      const int code = sparsity[(long)e * nv + jj];
      double col[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
      if (code != 0) {
        const int i = m.dof_joint[jj];
        M6d Jc;
        gb::world_axis_column(oM[i], gb::jt_col(m.jtype[i], jj - m.idx_v[i]), Jc.v);
        const double sign = code == 1 ? 1.0 : code == 2 ? -1.0 : 0.0;
        if (n == 3) {
          if (local) {
            if (code == 3) {
              M6d l1, l2;
              double r2[3];
              gb::actinv_motion(oMc1, Jc, l1);
              gb::actinv_motion(oMc2, Jc, l2);
              gb::mv3(c12.R, l2.v, r2);
#pragma unroll
              for (int k = 0; k < 3; ++k) col[k] = l1.v[k] - r2[k];
            } else if (code == 1) {
              M6d l1;
              gb::actinv_motion(oMc1, Jc, l1);
#pragma unroll
              for (int k = 0; k < 3; ++k) col[k] = l1.v[k];
            } else {
              M6d l2;
              double r2[3];
              gb::actinv_motion(oMc2, Jc, l2);
              gb::mv3(c12.R, l2.v, r2);
#pragma unroll
              for (int k = 0; k < 3; ++k) col[k] = -r2[k];
            }
          } else if (code == 3) {
            double d[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) d[k] = oMc2.t[k] - oMc1.t[k];
            gb::cross3(d, Jc.v + 3, col);
          } else {
            double pxw[3];
            gb::cross3(code == 1 ? oMc1.t : oMc2.t, Jc.v + 3, pxw);
#pragma unroll
            for (int k = 0; k < 3; ++k) col[k] = (Jc.v[k] - pxw[k]) * sign;
          }
        } else if (local) {
          M6d l1;
          gb::actinv_motion(oMc1, Jc, l1);
#pragma unroll
          for (int k = 0; k < 6; ++k) col[k] = l1.v[k] * sign;
        } else {
          double pxw[3];
          gb::cross3(oMc1.t, Jc.v + 3, pxw);
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            col[k] = (Jc.v[k] - pxw[k]) * sign;
            col[3 + k] = Jc.v[3 + k] * sign;
          }
        }
      }
      for (int k = 0; k < n; ++k) J[(long)(c.row + k) * nv + jj] = col[k];
    }
    // velocities and errors of the constraint (constrained-dynamics.hxx:296-350)
    M6d vc1, vc2, vc21, pe, ve, ae, a1, a2;
    gb::zero(vc1);
    gb::zero(vc2);
    if (j1 > 0) gb::actinv_motion(oMc1, ov[j1], vc1);
    if (j2 > 0) gb::actinv_motion(oMc2, ov[j2], vc2);
    gb::act_motion(c12, vc2, vc21);
    gb::zero(pe);
    gb::zero(ve);
    gb::zero(ae);
    if (n == 6) {
      M6d lg;
      log6(c12, lg);
#pragma unroll
      for (int k = 0; k < 6; ++k) {
        pe.v[k] = -lg.v[k];
        ve.v[k] = vc1.v[k] - vc21.v[k];
      }
    } else {
      double r2[3];
      gb::mv3(c12.R, vc2.v, r2);
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        pe.v[k] = -c12.t[k];
        ve.v[k] = vc1.v[k] - r2[k];
      }
    }
    if (c.gains)
      for (int k = 0; k < n; ++k) ae.v[k] = -c.Kp[k] * pe.v[k] - c.Kd[k] * ve.v[k];
    const M6d& oa1 = oa[j1];
    const M6d& oa2 = oa[j2];
    double t[3], u[3];
    if (!local) {  // LOCAL_WORLD_ALIGNED
      gb::cross3(oa1.v + 3, oMc1.t, t);
#pragma unroll
      for (int k = 0; k < 3; ++k) a1.v[k] = oa1.v[k] + t[k];
      if (n == 3) {
        point_drift(ov[j1], oMc1.t, t);
#pragma unroll
        for (int k = 0; k < 3; ++k) a1.v[k] += t[k];
      }
#pragma unroll
      for (int k = 0; k < 3; ++k) a1.v[3 + k] = oa1.v[3 + k];
      if (n == 3) {
        gb::cross3(oa2.v + 3, oMc2.t, t);
        point_drift(ov[j2], oMc2.t, u);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          a2.v[k] = oa2.v[k] + t[k] + u[k];
          a2.v[3 + k] = 0.0;
        }
      } else {
        gb::cross3(oa2.v + 3, oMc1.t, t);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          a2.v[k] = oa2.v[k] + t[k];
          a2.v[3 + k] = oa2.v[3 + k];
        }
      }
      double rl[3], ra[3];
      gb::mv3(oMc1.R, ae.v, rl);
      gb::mv3(oMc1.R, ae.v + 3, ra);
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        ae.v[k] = rl[k];
        ae.v[3 + k] = ra[k];
      }
    } else {
      gb::actinv_motion(oMc1, oa1, a1);
      if (n == 3) {
        gb::cross3(vc1.v + 3, vc1.v, t);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          a1.v[k] += t[k];
          a1.v[3 + k] = 0.0;
        }
        double w[3];
        gb::cross3(oa2.v + 3, oMc2.t, t);
        point_drift(ov[j2], oMc2.t, u);
#pragma unroll
        for (int k = 0; k < 3; ++k) w[k] = oa2.v[k] + t[k] + u[k];
        gb::mtv3(oMc1.R, w, a2.v);
#pragma unroll
        for (int k = 0; k < 3; ++k) a2.v[3 + k] = 0.0;
      } else {
        M6d x;
        gb::cross_motion(ve, vc21, x);
#pragma unroll
        for (int k = 0; k < 6; ++k) a1.v[k] += x.v[k];
        gb::actinv_motion(oMc1, oa2, a2);
      }
    }
    for (int k = 0; k < n; ++k) Rhs[c.row + k] = -a1.v[k] + a2.v[k] + ae.v[k] + c.des[k];
  }
}

// The Delassus matrix J M^-1 J^T + mu I = Y^T Y + mu I by columns, one thread per (configuration,
// constraint row c): Y(:, c) = D^-1/2 U^-1 J(c, :)^T on the ancestor closure of row c's constraint
// (the rows of U^-1 J^T that can be non-zero: U^-1 keeps a vector inside such a set; the entries
// outside it are neither written nor read; clist holds the closure of each constraint as [count,
// dofs...], cmask as a mask), then G(i, c) for i >= c over the two rows' common dofs + mu [i == c]
// (its LLT: k_llt).  Y is nv x nc and G nc x nc, [element][configuration].
__global__ void __launch_bounds__(kThreads)
    k_delassus_y_cols(const unsigned char* blob, int bytes, long B, int nc, const double* Us, const double* Ds,
                      const double* Js, double* Ys, const ConstraintDev* __restrict__ tab, int ncon,
                      const short* __restrict__ clist) {
  extern __shared__ __align__(16) unsigned char smem[];
  const gb::MView m = stage_model(blob, bytes, smem);
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= B * nc) return;
  const long b = t % B;
  const int c = (int)(t / B), nv = m.nv;
  int e = 0;
  while (e + 1 < ncon && tab[e + 1].row <= c) ++e;
  const short* L = clist + (long)e * (nv + 1);
  const int len = L[0];
  auto U = [&](int r, int k) { return Us[((long)r * nv + k) * B + b]; };
  auto Y = [&](int k) -> double& { return Ys[((long)k * nc + c) * B + b]; };
  for (int p = 0; p < len; ++p) Y(L[1 + p]) = Js[((long)c * nv + L[1 + p]) * B + b];
  for (int p = len - 2; p >= 0; --p) {  // U^-1 restricted to the set (subtree rows k..k+nsfr-1)
    const int k = L[1 + p], end = k + m.nsfr[k];
    double acc = 0.0;
    for (int p2 = p + 1; p2 < len && L[1 + p2] < end; ++p2) acc += U(k, L[1 + p2]) * Y(L[1 + p2]);
    Y(k) -= acc;
  }
  for (int p = 0; p < len; ++p) Y(L[1 + p]) /= sqrt(Ds[(long)L[1 + p] * B + b]);
}
__global__ void __launch_bounds__(kThreads)
    k_delassus_gram_cols(long B, int nc, int nv, const double* Ys, double* Gs, double mu,
                         const ConstraintDev* __restrict__ tab, int ncon, const signed char* __restrict__ cmask,
                         const short* __restrict__ clist) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= B * nc) return;
  const long b = t % B;
  const int c = (int)(t / B);
  int ec = 0;
  while (ec + 1 < ncon && tab[ec + 1].row <= c) ++ec;
  const short* L = clist + (long)ec * (nv + 1);
  int ei = ec;
  for (int i = c; i < nc; ++i) {
    while (ei + 1 < ncon && tab[ei + 1].row <= i) ++ei;
    const signed char* mi = cmask + (long)ei * nv;
    double acc = 0.0;
    for (int p = 0; p < L[0]; ++p) {
      const int k = L[1 + p];
      if (mi[k]) acc += Ys[((long)k * nc + i) * B + b] * Ys[((long)k * nc + c) * B + b];
    }
    Gs[((long)i * nc + c) * B + b] = acc + (i == c ? mu : 0.0);
  }
}

// The proximal iterations (constrained-dynamics.hxx:434-486) on the factorisations M = U D U^T and
// J M^-1 J^T + mu I = L L^T: lambda_k = L^-T L^-1 (c0 + mu lambda_{k-1}) with c0 = rhs - J M^-1 (tau -
// nle); the reference's residuals: absolute ||(J M^-1 J^T) y - rhs||_inf and relative ||y - y_prev||_inf
// for y = -lambda_k; then ddq = M^-1 (tau - nle + J^T lambda).
__global__ void __launch_bounds__(kThreads, 1)  // a single wave at these batches: no register cap
    k_constraint_solve(const unsigned char* blob, int bytes, long B, int nc, const double* Us, const double* Ds,
                       const double* nles, double* Rs, double* Ys, double* Gs, const double* Js, const double* Rh,
                       double* C0s, double* LPs, double* Ts, Arr tau, gb_proximal_settings s, Arr ddq, Arr lam,
                       int* iters, double* residuals, const ConstraintDev* __restrict__ tab, int ncon,
                       const short* __restrict__ clist) {
  extern __shared__ __align__(16) unsigned char smem[];
  const gb::MView m = stage_model(blob, bytes, smem);
  const long b = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const int nv = m.nv;
  const Col U{const_cast<double*>(Us) + b, B}, D{const_cast<double*>(Ds) + b, B};
  const Col Y{Ys + b, B}, G{Gs + b, B}, R{Rs + b, B};
  const Col C0{C0s + b, B}, LP{LPs + b, B}, T{Ts + b, B}, Rhs{const_cast<double*>(Rh) + b, B};
  const gb::In taui{tau.p + b * tau.is, tau.es}, Ji{Js + b, B};
  const gb::Out o{const_cast<double*>(ddq.p) + b * ddq.is, ddq.es};
  const Col nle{const_cast<double*>(nles) + b, B};
  for (int k = 0; k < nv; ++k) R[k] = taui[k] - nle[k];
  chol_solve(m, U, D, R);
  int it = 0;
  double ar = 0.0, rr = 0.0;
  const Col L{nc > 0 ? const_cast<double*>(lam.p) + b * lam.is : nullptr, nc > 0 ? lam.es : 0};
  if (nc > 0) {
    for (int r = 0; r < nv; ++r) gb::check_pivot(m, D[r]);  // G and its LLT: the column kernels
    for (int e = 0; e < ncon; ++e) {
      const short* Ls = clist + (long)e * (nv + 1);
      const int r0 = tab[e].row, r1 = r0 + (tab[e].type == GB_CONTACT_3D ? 3 : 6);
      for (int c = r0; c < r1; ++c) {
        double t = 0.0;
        for (int p = 0; p < Ls[0]; ++p) t += Ji[c * nv + Ls[1 + p]] * R[Ls[1 + p]];
        C0[c] = Rhs[c] - t;
        LP[c] = 0.0;
      }
    }
    while (it < s.max_iter) {
      ++it;
      for (int c = 0; c < nc; ++c) L[c] = C0[c] + s.mu * LP[c];
      llt_solve(G, nc, L);
      for (int i = 0; i < nc; ++i) {  // T = L_f^T lambda (L_f the lower factor in G)
        double t = 0.0;
        for (int k = i; k < nc; ++k) t += G[(long)k * nc + i] * L[k];
        T[i] = t;
      }
      ar = 0.0;
      rr = 0.0;
      for (int i = 0; i < nc; ++i) {
        double t = 0.0;
        for (int k = 0; k <= i; ++k) t += G[(long)i * nc + k] * T[k];
        ar = fmax(ar, fabs(t - s.mu * L[i] + Rhs[i]));
        rr = fmax(rr, fabs(L[i] - LP[i]));
      }
      for (int c = 0; c < nc; ++c) LP[c] = L[c];
      if (ar <= s.absolute_accuracy || rr <= s.relative_accuracy) break;
    }
  } else {
    it = 1;
  }
  if (iters) iters[b] = it;
  if (residuals) {
    residuals[2 * b] = ar;
    residuals[2 * b + 1] = rr;
  }
  const Col A{Y.p, B};
  for (int k = 0; k < nv; ++k) A[k] = 0.0;
  for (int e = 0; e < ncon; ++e) {
    const short* Ls = clist + (long)e * (nv + 1);
    const int r0 = tab[e].row, r1 = r0 + (tab[e].type == GB_CONTACT_3D ? 3 : 6);
    for (int p = 0; p < Ls[0]; ++p) {
      const int k = Ls[1 + p];
      double t = 0.0;
      for (int c = r0; c < r1; ++c) t += Ji[c * nv + k] * L[c];
      A[k] += t;
    }
  }
  chol_solve(m, U, D, A);
  bool finite = true;
  for (int k = 0; k < nv; ++k) {
    const double x = A[k] + R[k];
    finite = finite && gb::finite_value(x);
    o[k] = x;
  }
  if (!finite) gb::flag_numeric(m, gb::NUM_NONFINITE);
}

// ---- computeConstraintDynamicsDerivatives for constraints to the world without Baumgarte gains ----
// (algorithm/constrained-dynamics-derivatives.hxx:344-1050).  After constraintDynamics (ddq, lambda)
// and before the inverse dynamics derivatives: k_cd_setup, per configuration, the world kinematics
// at ddq, per constraint its Jacobian rows (dac_da), the derivatives of its frame acceleration
// (dac_dq, dac_dv: getFrameAccelerationDerivatives, frames-derivatives.hxx:85-176, over
// JointAccelerationDerivativesBackwardStep, kinematics-derivatives.hxx:285-440; point constraints:
// PointClassicAccelerationDerivativesBackwardStep, kinematics-derivatives.hxx:700-880), the force
// derivative term of world-aligned constraints (hxx:1000-1040) and the constraint forces as forces
// on the constraint joints (ContactForceContribution, hxx:225-342) for the inverse dynamics
// derivatives; then the assembly as column-parallel steps (M^-1, the operational-space inertia,
// the proximal recursion, hxx:815-990: k_tree_solve_cols, k_jprod_rows, k_delassus_cols, k_llt, k_osim_cols, k_prox_cols,
// k_out_rows).

__device__ void translate_motion(const double* p, M6d& m) {  // linear -= p x angular
  double w[3];
  gb::cross3(p, m.v + 3, w);
#pragma unroll
  for (int k = 0; k < 3; ++k) m.v[k] -= w[k];
}
__device__ void cross_lin_ang(const M6d& a, const M6d& b, double* o) {  // a.ang x b.lin + a.lin x b.ang
  double t1[3], t2[3];
  gb::cross3(a.v + 3, b.v, t1);
  gb::cross3(a.v, b.v + 3, t2);
#pragma unroll
  for (int k = 0; k < 3; ++k) o[k] = t1[k] + t2[k];
}
__device__ void cross_lin_ang_minus(const M6d& a, const M6d& b, double* o) {  // a.ang x b.lin - a.lin x b.ang
  double t1[3], t2[3];
  gb::cross3(a.v + 3, b.v, t1);
  gb::cross3(a.v, b.v + 3, t2);
#pragma unroll
  for (int k = 0; k < 3; ++k) o[k] = t1[k] - t2[k];
}

template <int CAP>
__global__ void __launch_bounds__(kThreads)
    k_cd_setup(const unsigned char* blob, int bytes, long B, Arr q, Arr v, Arr ddq, Arr lam,
               const ConstraintDev* __restrict__ tab, int ncon, int nj_user, double* Js, double* Aqs, double* Avs,
               double* Cqs, double* Fes) {
  extern __shared__ __align__(16) unsigned char smem[];
  const gb::MView m = stage_model(blob, bytes, smem);
  const long b = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const int nv = m.nv;
  const gb::In qi{q.p + b * q.is, q.es}, vi{v.p + b * v.is, v.es}, ai{ddq.p + b * ddq.is, ddq.es};
  const gb::In li{lam.p + b * lam.is, lam.es};
  X3d oM[CAP];
  M6d ov[CAP], oa[CAP];
  gb::zero(ov[0]);
  gb::zero(oa[0]);
  for (int i = 1; i < m.nj; ++i) {  // world placements, velocities, accelerations at ddq
    const int p = m.parent[i];
    X3d X;
    gb::joint_transform(m, i, qi, X);
    if (p > 0) gb::compose(oM[p], X, oM[i]);
    else oM[i] = X;
    M6d vJ, aJ, w, t;
    gb::joint_motion(m.jtype[i], vi, m.idx_v[i], vJ);
    gb::joint_motion(m.jtype[i], ai, m.idx_v[i], aJ);
    gb::act_motion(oM[i], vJ, w);
    gb::act_motion(oM[i], aJ, t);
    M6d x;
    gb::cross_motion(ov[p], w, x);  // ov_p x vJ (world); zero for a root joint
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      ov[i].v[k] = ov[p].v[k] + w.v[k];
      oa[i].v[k] = oa[p].v[k] + x.v[k] + t.v[k];
    }
  }
  const Col J{Js + b, B}, Aq{Aqs + b, B}, Av{Avs + b, B}, Cq{Cqs + b, B}, Fe{Fes + b, B};
  for (int k = 0; k < 6 * nj_user; ++k) Fe[k] = 0.0;
  for (int e = 0; e < ncon; ++e) {
    const ConstraintDev& c = tab[e];
    const int n = c.type == GB_CONTACT_3D ? 3 : 6, j = c.j1, row = c.row;
    const bool local = c.frame == GB_FRAME_LOCAL;
    for (int k = 0; k < n; ++k)
      for (int jj = 0; jj < nv; ++jj) {
        const long o = (long)(row + k) * nv + jj;
        J[o] = 0.0;
        Aq[o] = 0.0;
        Av[o] = 0.0;
        Cq[o] = 0.0;
      }
    X3d P, oMc;
    load_se3(c.P1, P);
    gb::compose(oM[j], P, oMc);
    // Baumgarte gains (LOCAL contacts: the host refuses the others): the point contact's placement
    // error pe = -c1Mc2.translation = -R_c^T (t_anchor - t_c), the frame contact's Jlog6(c1Mc2^-1)
    const bool gains3 = n == 3 && c.gains, gains6 = n == 6 && c.gains;
    double pe[3] = {0.0, 0.0, 0.0};
    double Jl[36];
    if (gains3) {
      const double dpos[3] = {c.P2[9] - oMc.t[0], c.P2[10] - oMc.t[1], c.P2[11] - oMc.t[2]};
      gb::mtv3(oMc.R, dpos, pe);
#pragma unroll
      for (int k = 0; k < 3; ++k) pe[k] = -pe[k];
    }
    if (gains6) {  // c2Mc1 = anchor^-1 oMc
      X3d A, c21;
      load_se3(c.P2, A);
      se3_actinv(A, oMc, c21);
      jlog6(c21, Jl);
    }
    M6d f;
    gb::zero(f);
    for (int k = 0; k < n; ++k) f.v[k] = li[row + k];
    // the constraint force on joint j, in the caller's frame of that joint
    {
      M6d fi;
      if (local) {
        gb::act_force(P, f, fi);
      } else {
        M6d fw = f;
        double w[3], nn[3];
        gb::cross3(oMc.t, f.v, w);
#pragma unroll
        for (int k = 0; k < 3; ++k) fw.v[3 + k] += w[k];
        gb::mtv3(oM[j].R, fw.v, fi.v);
        gb::cross3(oM[j].t, fw.v, w);
#pragma unroll
        for (int k = 0; k < 3; ++k) nn[k] = fw.v[3 + k] - w[k];
        gb::mtv3(oM[j].R, nn, fi.v + 3);
      }
      M6d fu = fi;
      if (m.fix_d) {  // the caller's frame of an unaligned joint is the kernels' frame F^T
        gb::mv3(m.fix_d + 9 * j, fi.v, fu.v);
        gb::mv3(m.fix_d + 9 * j, fi.v + 3, fu.v + 3);
      }
      const int u = m.ujoint[j];
#pragma unroll
      for (int k = 0; k < 6; ++k) Fe[6 * u + k] += fu.v[k];
    }
    const X3d& oMl = oM[j];
    M6d vloc;  // the local velocity of joint j
    gb::actinv_motion(oMl, ov[j], vloc);
    M6d vl, al;  // point constraints: the contact point's spatial velocity / acceleration
    double pacc[3], trans[3];
    gb::actinv_motion(oMc, ov[j], vl);
    gb::actinv_motion(oMc, oa[j], al);
    gb::cross3(vl.v + 3, vl.v, pacc);
#pragma unroll
    for (int k = 0; k < 3; ++k) pacc[k] += al.v[k];
    gb::mv3(oMl.R, P.t, trans);
    for (int i = j; i > 0; i = m.parent[i]) {
      const int p = m.parent[i], jt = m.jtype[i];
      for (int k = 0; k < gb::jt_nv(jt); ++k) {
        const int col = m.idx_v[i] + k;
        M6d Jc, dJc;
        gb::world_axis_column(oM[i], gb::jt_col(jt, k), Jc.v);
        gb::cross_motion(ov[i], Jc, dJc);
        double rj[6], rq[6], rv[6];
        if (n == 6) {
          M6d da, vdq, adq, adv;
          gb::zero(vdq);
          gb::zero(adq);
          if (local) {
            M6d vtmp, t;
            gb::actinv_motion(oMl, Jc, da);
            gb::zero(vtmp);
            if (p > 0) {
              gb::actinv_motion(oMl, ov[p], vtmp);
              gb::cross_motion(vtmp, da, vdq);
            }
#pragma unroll
            for (int r = 0; r < 6; ++r) vtmp.v[r] -= vloc.v[r];
            gb::cross_motion(vtmp, da, adv);
            gb::actinv_motion(oMl, dJc, t);
#pragma unroll
            for (int r = 0; r < 6; ++r) adv.v[r] += t.v[r];
            if (p > 0) {
              M6d atmp, x1, x2;
              gb::actinv_motion(oMl, oa[p], atmp);
              gb::cross_motion(atmp, da, x1);
              gb::cross_motion(vtmp, vdq, x2);
#pragma unroll
              for (int r = 0; r < 6; ++r) adq.v[r] = x1.v[r] + x2.v[r];
            }
          } else {
            M6d vtmp, atmp;
            da = Jc;
            translate_motion(oMl.t, da);
#pragma unroll
            for (int r = 0; r < 6; ++r) {
              vtmp.v[r] = (p > 0 ? ov[p].v[r] : 0.0) - ov[j].v[r];
              atmp.v[r] = (p > 0 ? oa[p].v[r] : 0.0) - oa[j].v[r];
            }
            double w[3];
            gb::cross3(vtmp.v + 3, oMl.t, w);
#pragma unroll
            for (int r = 0; r < 3; ++r) vtmp.v[r] += w[r];
            gb::cross3(atmp.v + 3, oMl.t, w);
#pragma unroll
            for (int r = 0; r < 3; ++r) atmp.v[r] += w[r];
            gb::cross_motion(vtmp, da, vdq);
            adv = dJc;
            translate_motion(oMl.t, adv);
            gb::cross_motion(atmp, da, adq);
            if (p > 0) {
              M6d x;
              gb::cross_motion(vtmp, adv, x);
#pragma unroll
              for (int r = 0; r < 6; ++r) adq.v[r] += x.v[r];
            }
#pragma unroll
            for (int r = 0; r < 6; ++r) adv.v[r] += vdq.v[r];
          }
          // the frame's placement in the joint (frames-derivatives.hxx:137-172)
          M6d* mats[4] = {&da, &adq, &adv, &vdq};
          for (int t = 0; t < (gains6 ? 4 : 3); ++t) {
            if (local) {
              M6d y;
              gb::actinv_motion(P, *mats[t], y);
              *mats[t] = y;
            } else {
              translate_motion(trans, *mats[t]);
            }
          }
#pragma unroll
          for (int r = 0; r < 6; ++r) {
            rj[r] = da.v[r];
            rq[r] = adq.v[r];
            rv[r] = adv.v[r];
          }
          if (gains6)  // the corrector (hxx:758-782): dac_dq += Kd dvc_dq + Kp Jlog6 dac_da, dac_dv += Kd dac_da
            for (int r = 0; r < 6; ++r) {
              double acc = 0.0;
#pragma unroll
              for (int i2 = 0; i2 < 6; ++i2) acc += Jl[6 * r + i2] * da.v[i2];
              rq[r] += c.Kd[r] * vdq.v[r] + c.Kp[r] * acc;
              rv[r] += c.Kd[r] * da.v[r];
            }
        } else {
          M6d sda, svdq, vtmp;
          gb::actinv_motion(oMc, Jc, sda);
          gb::zero(svdq);
          gb::zero(vtmp);
          double vdq[3] = {0.0, 0.0, 0.0}, adq[3] = {0.0, 0.0, 0.0}, adv[3], t1[3], t2[3];
          if (p > 0) {
            gb::actinv_motion(oMc, ov[p], vtmp);
            gb::cross_motion(vtmp, sda, svdq);
#pragma unroll
            for (int r = 0; r < 3; ++r) vdq[r] = svdq.v[r];
          }
#pragma unroll
          for (int r = 0; r < 6; ++r) vtmp.v[r] -= vl.v[r];
          cross_lin_ang(vtmp, sda, adv);
          double dl[3];
          gb::cross3(dJc.v + 3, oMc.t, t1);
#pragma unroll
          for (int r = 0; r < 3; ++r) dl[r] = dJc.v[r] + t1[r];
          gb::mtv3(oMc.R, dl, t1);
          cross_lin_ang_minus(vl, sda, t2);
#pragma unroll
          for (int r = 0; r < 3; ++r) adv[r] += t1[r] + t2[r];
          if (p > 0) {
            M6d atmp;
            gb::actinv_motion(oMc, oa[p], atmp);
            cross_lin_ang(atmp, sda, adq);
            cross_lin_ang(vtmp, svdq, t1);
            cross_lin_ang_minus(vl, svdq, t2);
#pragma unroll
            for (int r = 0; r < 3; ++r) adq[r] += t1[r] + t2[r];
          }
          double ada[3] = {sda.v[0], sda.v[1], sda.v[2]};
          if (!local) {
            double x[3], y[3];
            gb::cross3(sda.v + 3, pacc, x);
#pragma unroll
            for (int r = 0; r < 3; ++r) x[r] += adq[r];
            gb::mv3(oMc.R, x, adq);
            gb::mv3(oMc.R, adv, y);
#pragma unroll
            for (int r = 0; r < 3; ++r) adv[r] = y[r];
            gb::mv3(oMc.R, ada, y);
#pragma unroll
            for (int r = 0; r < 3; ++r) ada[r] = y[r];
          }
#pragma unroll
          for (int r = 0; r < 3; ++r) {
            rj[r] = ada[r];
            rq[r] = adq[r];
            rv[r] = adv[r];
          }
          if (gains3) {  // the corrector (hxx:753-830): dac_dq += Kd dvc_dq + Kp (dac_da + pe x (R_c^T J_ang)),
                         // dac_dv += Kd dac_da
            double wa[3], x[3];
            gb::mtv3(oMc.R, Jc.v + 3, wa);
            gb::cross3(pe, wa, x);
#pragma unroll
            for (int r = 0; r < 3; ++r) {
              rq[r] += c.Kd[r] * vdq[r] + c.Kp[r] * (ada[r] + x[r]);
              rv[r] += c.Kd[r] * ada[r];
            }
          }
        }
        for (int r = 0; r < n; ++r) {
          const long o = (long)(row + r) * nv + col;
          J[o] = rj[r];
          Aq[o] = rq[r];
          Av[o] = rv[r];
        }
        if (!local) {  // world-aligned: d(force)/dq += J.ang x f (hxx:1000-1040)
          double w[3];
          gb::cross3(Jc.v + 3, f.v, w);
#pragma unroll
          for (int r = 0; r < 3; ++r) Cq[(long)(row + r) * nv + col] = w[r];
          if (n == 6) {
            gb::cross3(Jc.v + 3, f.v + 3, w);
#pragma unroll
            for (int r = 0; r < 3; ++r) Cq[(long)(row + 3 + r) * nv + col] = w[r];
          }
        }
      }
    }
  }
}

// ---- the assembly as column-parallel steps: one thread per (configuration, column or row) ----
// Thread t covers configuration b = t % B and column (or row) c = t / B: the 32 threads of a warp are
// consecutive configurations of one column, so every [element][configuration] array they touch is
// read and written in 256-byte lines, and a batch of B configurations gives B x nv threads instead
// of B.  Element (k, c) of an m x n per-configuration matrix X sits at X[(k * n + c) * B + b].

// X[:, c] <- M^-1 X[:, c] for the columns c < ncols of an nv x ncols matrix (identity: from the unit
// columns, i.e. X = M^-1), by the tree factorisation M = U D U^T (cholesky.hxx:483-500)
__global__ void __launch_bounds__(kThreads)
    k_tree_solve_cols(const unsigned char* blob, int bytes, long B, int ncols, const double* Us, const double* Ds,
                      double* X, int identity) {
  extern __shared__ __align__(16) unsigned char smem[];
  const gb::MView m = stage_model(blob, bytes, smem);
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= B * ncols) return;
  const long b = t % B;
  const int c = (int)(t / B);
  const Col U{const_cast<double*>(Us) + b, B}, D{const_cast<double*>(Ds) + b, B};
  const Col x{X + (long)c * B + b, (long)ncols * B};
  if (identity)
    for (int k = 0; k < m.nv; ++k) x[k] = k == c ? 1.0 : 0.0;
  chol_solve(m, U, D, x);
}

// Y(r, c) = (A(r, c) if A) + sign * sum over row r's constraint dofs k of J(r, k) S(k, c), c < ncols,
// one thread per (configuration, row r < nc); J nc x nv, S nv x ncols, A and Y nc x ncols
__global__ void __launch_bounds__(kThreads)
    k_jprod_rows(long B, int nc, int nv, int ncols, const ConstraintDev* __restrict__ tab, int ncon,
                 const short* __restrict__ clist, const double* Js, const double* S, const double* A, double sign,
                 double* Y) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= B * nc) return;
  const long b = t % B;
  const int r = (int)(t / B);
  int e = 0;
  while (e + 1 < ncon && tab[e + 1].row <= r) ++e;
  const short* L = clist + (long)e * (nv + 1);
  const int len = L[0];
  for (int c = 0; c < ncols; ++c) {
    double acc = 0.0;
    for (int p = 0; p < len; ++p) {
      const int k = L[1 + p];
      acc += Js[((long)r * nv + k) * B + b] * S[((long)k * ncols + c) * B + b];
    }
    const long o = ((long)r * ncols + c) * B + b;
    Y[o] = (A ? A[o] : 0.0) + sign * acc;
  }
}

// G(r, c) = JMinv(r, :) J(c, :)^T + mu [r == c] for r >= c (the damped Delassus matrix, lower part;
// the sum over column c's constraint dofs): one thread per (configuration, column c < nc); oinv
// (optional) takes the symmetric matrix
__global__ void __launch_bounds__(kThreads)
    k_delassus_cols(long B, int nc, int nv, const ConstraintDev* __restrict__ tab, int ncon,
                    const short* __restrict__ clist, const double* Js, const double* JMs, double mu, double* Gs,
                    Arr oinv) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= B * nc) return;
  const long b = t % B;
  const int c = (int)(t / B);
  int e = 0;
  while (e + 1 < ncon && tab[e + 1].row <= c) ++e;
  const short* L = clist + (long)e * (nv + 1);
  for (int r = c; r < nc; ++r) {
    double acc = 0.0;
    for (int p = 0; p < L[0]; ++p)
      acc += JMs[((long)r * nv + L[1 + p]) * B + b] * Js[((long)c * nv + L[1 + p]) * B + b];
    acc += r == c ? mu : 0.0;
    Gs[((long)r * nc + c) * B + b] = acc;
    if (oinv.p) {
      double* o = const_cast<double*>(oinv.p) + b * oinv.is;
      o[((long)r * nc + c) * oinv.es] = acc;
      o[((long)c * nc + r) * oinv.es] = acc;
    }
  }
}

// G = L L^T in place (lower), per configuration (pivots checked)
__global__ void __launch_bounds__(kThreads)
    k_llt(const unsigned char* blob, int bytes, long B, int nc, double* Gs) {
  extern __shared__ __align__(16) unsigned char smem[];
  const gb::MView m = stage_model(blob, bytes, smem);
  const long b = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const Col G{Gs + b, B};
  for (int j = 0; j < nc; ++j) {
    double t = G[(long)j * nc + j];
    for (int k = 0; k < j; ++k) t -= G[(long)j * nc + k] * G[(long)j * nc + k];
    gb::check_pivot(m, t);
    const double l = sqrt(t);
    G[(long)j * nc + j] = l;
    for (int i = j + 1; i < nc; ++i) {
      double u = G[(long)i * nc + j];
      for (int k = 0; k < j; ++k) u -= G[(long)i * nc + k] * G[(long)j * nc + k];
      G[(long)i * nc + j] = u / l;
    }
  }
}

// O(:, c) = (L L^T)^-1 e_c (osim, the operational-space inertia): one thread per (configuration,
// column c < nc); osim (optional) takes it
__global__ void __launch_bounds__(kThreads)
    k_osim_cols(long B, int nc, const double* Gs, double* Os, Arr osim) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= B * nc) return;
  const long b = t % B;
  const int c = (int)(t / B);
  const Col G{const_cast<double*>(Gs) + b, B};
  const Col x{Os + (long)c * B + b, (long)nc * B};
  for (int k = 0; k < nc; ++k) x[k] = k == c ? 1.0 : 0.0;
  llt_solve(G, nc, x);
  if (osim.p)
    for (int k = 0; k < nc; ++k)
      const_cast<double*>(osim.p)[b * osim.is + ((long)k * nc + c) * osim.es] = x[k];
}

// X[:, c] = s1 O R[:, c], then it - 1 times X[:, c] = O (mu X[:, c] - R[:, c]) (the proximal
// recursion of the derivatives, hxx:869-990, per column); one thread per (configuration, column
// c < ncols), O nc x nc, R, X, Tm (scratch) nc x ncols; dl (optional): X + C (C optional)
__global__ void __launch_bounds__(kThreads)
    k_prox_cols(long B, int nc, int ncols, const double* Os, const int* iters, double mu, double s1, const double* R,
                double* X, double* Tm, Arr dl, const double* C) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= B * ncols) return;
  const long b = t % B;
  const int c = (int)(t / B), it = iters ? iters[b] : 1;
  auto at = [&](int k) { return ((long)k * ncols + c) * B + b; };
  for (int r = 0; r < nc; ++r) {
    double acc = 0.0;
    for (int k = 0; k < nc; ++k) acc += Os[((long)r * nc + k) * B + b] * R[at(k)];
    X[at(r)] = s1 * acc;
  }
  for (int k2 = 1; k2 < it; ++k2) {
    for (int k = 0; k < nc; ++k) Tm[at(k)] = mu * X[at(k)] - R[at(k)];
    for (int r = 0; r < nc; ++r) {
      double acc = 0.0;
      for (int k = 0; k < nc; ++k) acc += Os[((long)r * nc + k) * B + b] * Tm[at(k)];
      X[at(r)] = acc;
    }
  }
  if (dl.p)
    for (int r = 0; r < nc; ++r)
      const_cast<double*>(dl.p)[b * dl.is + ((long)r * ncols + c) * dl.es] = X[at(r)] + (C ? C[at(r)] : 0.0);
}

// Out(r, c) = bsign Base(r, c) + sum_k JM(k, r) X(k, c) for c < nv: one thread per (configuration,
// row r < nv); Base nv x nv, JM and X nc x nv; Out in the caller's layout, at column offset
// (ro, co) of an ld-wide matrix (ld = nv for the derivative outputs)
__global__ void __launch_bounds__(kThreads)
    k_out_rows(const unsigned char* blob, int bytes, long B, int nc, const double* Base, double bsign,
               const double* JMs, const double* X, Arr out, int ld, int ro, int co) {
  extern __shared__ __align__(16) unsigned char smem[];
  const gb::MView m = stage_model(blob, bytes, smem);
  const int nv = m.nv;
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= B * nv) return;
  const long b = t % B;
  const int r = (int)(t / B);
  double* o = const_cast<double*>(out.p) + b * out.is;
  bool finite = true;
  for (int c = 0; c < nv; ++c) {
    double acc = bsign * Base[((long)r * nv + c) * B + b];
    for (int k = 0; k < nc; ++k) acc += JMs[((long)k * nv + r) * B + b] * X[((long)k * nv + c) * B + b];
    finite = finite && gb::finite_value(acc);
    o[((long)(ro + r) * ld + co + c) * out.es] = acc;
  }
  if (!finite) gb::flag_numeric(m, gb::NUM_NONFINITE);
}

// The contact Cholesky's row-wise outputs, one thread per (configuration, row r < nc + nv), from
// M^-1, J, JMinv, osim and Tn = -osim JMinv: the KKT matrix [[-mu I, J], [J^T, M]] (constraint rows
// first, as the reference's matrix()), the blocks of its inverse other than the bottom-right one
// ([[-osim, osim JMinv], [M^-1 J^T osim, .]]), M^-1 and JMinv; every output optional
__global__ void __launch_bounds__(kThreads)
    k_cc_rows(long B, int nc, int nv, double mu, const double* Ms, const double* Mis, const double* Js,
              const double* JMs, const double* Os, const double* Tn, Arr kkt, Arr kinv, Arr minv, Arr jminv) {
  const int n = nc + nv;
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= B * n) return;
  const long b = t % B;
  const int r = (int)(t / B);
  auto at = [&](const double* X, int ld, int i, int j) { return X[((long)i * ld + j) * B + b]; };
  auto put = [&](const Arr& a, long k, double x) { const_cast<double*>(a.p)[b * a.is + k * a.es] = x; };
  if (r < nc) {
    if (kkt.p)
      for (int c = 0; c < n; ++c) put(kkt, (long)r * n + c, c < nc ? (r == c ? -mu : 0.0) : at(Js, nv, r, c - nc));
    if (kinv.p)
      for (int c = 0; c < n; ++c) put(kinv, (long)r * n + c, c < nc ? -at(Os, nc, r, c) : -at(Tn, nv, r, c - nc));
    if (jminv.p)
      for (int c = 0; c < nv; ++c) put(jminv, (long)r * nv + c, at(JMs, nv, r, c));
  } else {
    const int i = r - nc;
    if (kkt.p)
      for (int c = 0; c < n; ++c) put(kkt, (long)r * n + c, c < nc ? at(Js, nv, c, i) : at(Ms, nv, i, c - nc));
    if (kinv.p)
      for (int c = 0; c < nc; ++c) put(kinv, (long)r * n + c, -at(Tn, nv, c, i));
    if (minv.p)
      for (int c = 0; c < nv; ++c) put(minv, (long)i * nv + c, at(Mis, nv, i, c));
  }
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

// the constraint set's device table: the models, their side codes, the ancestor-closure masks and
// then (2-byte aligned) the closure lists [count, dofs...] of nv + 1 entries per model
const short* closure_lists(const gb_constraint_set* set, int nv) {
  return reinterpret_cast<const short*>(
      static_cast<const unsigned char*>(set->d_mem) +
      ((sizeof(ConstraintDev) * (size_t)set->n + 2 * (size_t)set->n * nv + 1) & ~(size_t)1));
}

int launch_constraint(const gb_model* M, int precision, long B, const gb_constraint_set* set,
                      const gb_proximal_settings& s, Arr q, Arr v, Arr tau, Arr ddq, Arr lam, int* iters,
                      double* residuals, cudaStream_t st, double* U_keep, double* D_keep) {
  const long nv = M->nv, nn = nv * nv, nc = set->nc;
  // scratch, [element][configuration]: M, U (nn), D, nle, r (nv), sDUiJt (nv * max(nc, 1)), G (nc * nc),
  // J (nc * nv), rhs, c0, lambda_prev, tmp (nc)
  const long ny = nv * (nc > 0 ? nc : 1), ng = nc * nc;
  void* scratch = nullptr;
  int rc = scratch_alloc(&scratch, sizeof(double) * (size_t)B * (2 * nn + 3 * nv + ny + ng + nc * nv + 4 * nc), st);
  if (rc != GB_OK) return rc;
  double* base = static_cast<double*>(scratch);
  double *Ms = base, *Us = Ms + nn * B, *Ds = Us + nn * B, *nles = Ds + nv * B, *Rs = nles + nv * B,
         *Ys = Rs + nv * B, *Gs = Ys + ny * B, *Js = Gs + ng * B, *Rh = Js + nc * nv * B, *C0 = Rh + nc * B,
         *LP = C0 + nc * B, *Ts = LP + nc * B;
  if (U_keep) Us = U_keep;  // the caller keeps the factorisation of M ([element][configuration])
  if (D_keep) Ds = D_keep;
  const ConstraintDev* tab = static_cast<const ConstraintDev*>(set->d_mem);
  const signed char* sp = reinterpret_cast<const signed char*>(tab + (set->n > 0 ? set->n : 0));
  const signed char* cmask = sp + (long)set->n * nv;
  const short* clist = closure_lists(set, (int)nv);
  rc = launch_crba(M, GB_FP64, false, B, q, Arr{Ms, 1, B}, Arr{Us, 1, B}, Arr{Ds, 1, B}, st);
  if (rc == GB_OK) {
    const gb::BlobHeader* h = reinterpret_cast<const gb::BlobHeader*>(M->blob.data());
    const Arr zero{reinterpret_cast<const double*>(M->d_blob + h->o_zero), 0, 0};
    rc = launch_rnea(M, precision, B, q, v, zero, Arr{nles, 1, B}, st);
  }
  const long grid = (B + kThreads - 1) / kThreads;
  auto opt_in = [&](const void* kern, const char* name) -> int {
    if (M->stage_bytes <= 48 * 1024) return GB_OK;
    const cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, M->stage_bytes);
    return e == cudaSuccess ? GB_OK : cuda_error(e, name);
  };
  if (rc == GB_OK && set->n > 0) {
    switch (M->cap) {
#define GB_SETUP(C)                                                                                         \
  case C:                                                                                                   \
    rc = opt_in((const void*)k_constraint_setup<C>, "k_constraint_setup");                                  \
    if (rc == GB_OK)                                                                                        \
      k_constraint_setup<C><<<(unsigned)grid, kThreads, M->stage_bytes, st>>>(M->d_blob, M->stage_bytes, B, q, v, \
                                                                               tab, sp, set->n, Js, Rh);    \
    break;
      GB_SETUP(8)
      GB_SETUP(16)
      GB_SETUP(32)
      GB_SETUP(64)
      GB_SETUP(128)
#undef GB_SETUP
      default:
        rc = set_error(GB_ERR_UNSUPPORTED, "model too large");
    }
    if (rc == GB_OK) rc = cuda_error(cudaGetLastError(), "k_constraint_setup");
  }
  // the Delassus matrix and its factor by columns (one thread per configuration and constraint row),
  // then the per-configuration solve: R = M^-1 (tau - nle), the proximal iterations, ddq
  if (rc == GB_OK && nc > 0) {
    const unsigned gr = (unsigned)((B * nc + kThreads - 1) / kThreads);
    rc = opt_in((const void*)k_delassus_y_cols, "k_delassus_y_cols");
    if (rc == GB_OK) rc = opt_in((const void*)k_llt, "k_llt");
    if (rc == GB_OK) {
      k_delassus_y_cols<<<gr, kThreads, M->stage_bytes, st>>>(M->d_blob, M->stage_bytes, B, (int)nc, Us, Ds, Js, Ys,
                                                             tab, set->n, clist);
      k_delassus_gram_cols<<<gr, kThreads, 0, st>>>(B, (int)nc, (int)nv, Ys, Gs, s.mu, tab, set->n, cmask, clist);
      k_llt<<<(unsigned)grid, kThreads, M->stage_bytes, st>>>(M->d_blob, M->stage_bytes, B, (int)nc, Gs);
      rc = cuda_error(cudaGetLastError(), "the Delassus kernels");
    }
  }
  if (rc == GB_OK) rc = opt_in((const void*)k_constraint_solve, "k_constraint_solve");
  if (rc == GB_OK) {
    k_constraint_solve<<<(unsigned)grid, kThreads, M->stage_bytes, st>>>(M->d_blob, M->stage_bytes, B, (int)nc, Us, Ds,
                                                                        nles, Rs, Ys, Gs, Js, Rh, C0, LP, Ts, tau, s,
                                                                        ddq, lam, iters, residuals, tab, set->n, clist);
    rc = cuda_error(cudaGetLastError(), "k_constraint_solve");
  }
  scratch_free(scratch, st);
  return rc;
}

int launch_contact_cholesky(const gb_model* M, long B, const gb_constraint_set* set, double mu, Arr q, Arr kkt,
                            Arr kinv, Arr oinv, Arr osim, Arr minv, Arr jminv, cudaStream_t st) {
  const long nv = M->nv, nn = nv * nv, nc = set->nc;
  // scratch, [element][configuration]: M, U, M^-1 (nn), D (nv), J, J M^-1, OSIM J M^-1 (nc nv),
  // the Delassus factor, OSIM (nc nc), the constraint right-hand sides (nc, unused here)
  void* scratch = nullptr;
  int rc = scratch_alloc(&scratch, sizeof(double) * (size_t)B * (3 * nn + nv + 3 * nc * nv + 2 * nc * nc + nc), st);
  if (rc != GB_OK) return rc;
  double* base = static_cast<double*>(scratch);
  double *Ms = base, *Us = Ms + nn * B, *Mis = Us + nn * B, *Ds = Mis + nn * B, *Js = Ds + nv * B,
         *JMs = Js + nc * nv * B, *Ts = JMs + nc * nv * B, *Gs = Ts + nc * nv * B, *Os = Gs + nc * nc * B,
         *Rh = Os + nc * nc * B;
  const ConstraintDev* tab = static_cast<const ConstraintDev*>(set->d_mem);
  const signed char* sp = reinterpret_cast<const signed char*>(tab + (set->n > 0 ? set->n : 0));
  rc = launch_crba(M, GB_FP64, true, B, q, Arr{Ms, 1, B}, Arr{Us, 1, B}, Arr{Ds, 1, B}, st);
  const long grid = (B + kThreads - 1) / kThreads;
  auto opt_in = [&](const void* kern, const char* name) -> int {
    if (M->stage_bytes <= 48 * 1024) return GB_OK;
    const cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, M->stage_bytes);
    return e == cudaSuccess ? GB_OK : cuda_error(e, name);
  };
  if (rc == GB_OK && set->n > 0) {
    const gb::BlobHeader* h = reinterpret_cast<const gb::BlobHeader*>(M->blob.data());
    const Arr zero{reinterpret_cast<const double*>(M->d_blob + h->o_zero), 0, 0};
    switch (M->cap) {
#define GB_SETUP(C)                                                                                         \
  case C:                                                                                                   \
    rc = opt_in((const void*)k_constraint_setup<C>, "k_constraint_setup");                                  \
    if (rc == GB_OK)                                                                                        \
      k_constraint_setup<C><<<(unsigned)grid, kThreads, M->stage_bytes, st>>>(M->d_blob, M->stage_bytes, B, q, zero, \
                                                                               tab, sp, set->n, Js, Rh);    \
    break;
      GB_SETUP(8)
      GB_SETUP(16)
      GB_SETUP(32)
      GB_SETUP(64)
      GB_SETUP(128)
#undef GB_SETUP
      default:
        rc = set_error(GB_ERR_UNSUPPORTED, "model too large");
    }
    if (rc == GB_OK) rc = cuda_error(cudaGetLastError(), "k_constraint_setup");
  }
  // M^-1 by tree solves, JMinv over each constraint's dofs, the Delassus factor (+ its matrix and
  // osim as outputs), Tn = -osim JMinv, the row-wise outputs and the inverse's bottom-right block
  // M^-1 + JMinv^T Tn = M^-1 - M^-1 J^T osim J M^-1
  const unsigned gc = (unsigned)((B * nv + kThreads - 1) / kThreads), gr = (unsigned)((B * nc + kThreads - 1) / kThreads);
  const unsigned gn = (unsigned)((B * (nv + nc) + kThreads - 1) / kThreads);
  const short* clist = closure_lists(set, (int)nv);
  if (rc == GB_OK) rc = opt_in((const void*)k_tree_solve_cols, "k_tree_solve_cols");
  if (rc == GB_OK) rc = opt_in((const void*)k_llt, "k_llt");
  if (rc == GB_OK) rc = opt_in((const void*)k_out_rows, "k_out_rows");
  if (rc == GB_OK) {
    k_tree_solve_cols<<<gc, kThreads, M->stage_bytes, st>>>(M->d_blob, M->stage_bytes, B, (int)nv, Us, Ds, Mis, 1);
    if (nc > 0) {
      k_jprod_rows<<<gr, kThreads, 0, st>>>(B, (int)nc, (int)nv, (int)nv, tab, set->n, clist, Js, Mis, nullptr, 1.0,
                                            JMs);
      k_delassus_cols<<<gr, kThreads, 0, st>>>(B, (int)nc, (int)nv, tab, set->n, clist, Js, JMs, mu, Gs, oinv);
      k_llt<<<(unsigned)grid, kThreads, M->stage_bytes, st>>>(M->d_blob, M->stage_bytes, B, (int)nc, Gs);
      k_osim_cols<<<gr, kThreads, 0, st>>>(B, (int)nc, Gs, Os, osim);
      k_prox_cols<<<gc, kThreads, 0, st>>>(B, (int)nc, (int)nv, Os, nullptr, mu, -1.0, JMs, Ts, Rh, Arr{nullptr, 0, 0},
                                           nullptr);
    }
    k_cc_rows<<<gn, kThreads, 0, st>>>(B, (int)nc, (int)nv, mu, Ms, Mis, Js, JMs, Os, Ts, kkt, kinv, minv, jminv);
    if (kinv.p)
      k_out_rows<<<gc, kThreads, M->stage_bytes, st>>>(M->d_blob, M->stage_bytes, B, (int)nc, Mis, 1.0, JMs, Ts, kinv,
                                                      (int)(nv + nc), (int)nc, (int)nc);
    rc = cuda_error(cudaGetLastError(), "contact Cholesky kernels");
  }
  scratch_free(scratch, st);
  return rc;
}

int launch_constraint_derivs(const gb_model* M, int precision, long B, const gb_constraint_set* set,
                             const gb_proximal_settings& s, Arr q, Arr v, Arr tau, Arr ddq, Arr lam, Arr ddq_dq,
                             Arr ddq_dv, Arr ddq_dtau, Arr dl_dq, Arr dl_dv, Arr dl_dtau, int* iters_out,
                             cudaStream_t st) {
  const long nv = M->nv, nn = nv * nv, nc = set->nc, cn = nc * nv, nju = M->nj_user;
  // scratch, [element][configuration]: M, U, M^-1, dtau_dq, dtau_dv, dM (nn); D (nv); J, dac_dq, dac_dv,
  // the force term, JMinv, R, X, tmp (nc * nv each); G, osim (nc * nc); fext (6 per caller joint);
  // and the iteration counts (ints)
  const size_t doubles = (size_t)B * (6 * nn + nv + 8 * cn + 2 * nc * nc + 6 * nju);
  void* scratch = nullptr;
  int rc = scratch_alloc(&scratch, sizeof(double) * doubles + sizeof(int) * (size_t)B + 256, st);
  if (rc != GB_OK) return rc;
  double* base = static_cast<double*>(scratch);
  double *Ms = base, *Us = Ms + nn * B, *Mis = Us + nn * B, *dtq = Mis + nn * B, *dtv = dtq + nn * B,
         *dMs = dtv + nn * B, *Ds = dMs + nn * B, *Js = Ds + nv * B, *Aq = Js + cn * B, *Av = Aq + cn * B,
         *Cq = Av + cn * B, *JMs = Cq + cn * B, *Rs = JMs + cn * B, *Xs = Rs + cn * B, *Ts = Xs + cn * B,
         *Gs = Ts + cn * B, *Os = Gs + nc * nc * B, *Fe = Os + nc * nc * B;
  int* its = reinterpret_cast<int*>(base + doubles);
  // the constraint dynamics it differentiates, which leaves the factorisation of M in Us / Ds
  rc = launch_constraint(M, precision, B, set, s, q, v, tau, ddq, lam, its, nullptr, st, Us, Ds);
  const long grid = (B + kThreads - 1) / kThreads;
  auto opt_in = [&](const void* kern, const char* name) -> int {
    if (M->stage_bytes <= 48 * 1024) return GB_OK;
    const cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, M->stage_bytes);
    return e == cudaSuccess ? GB_OK : cuda_error(e, name);
  };
  const ConstraintDev* tab = static_cast<const ConstraintDev*>(set->d_mem);
  const short* clist = closure_lists(set, (int)nv);
  if (rc == GB_OK && set->n > 0) {
    switch (M->cap) {
#define GB_CD_SETUP(C)                                                                                       \
  case C:                                                                                                    \
    rc = opt_in((const void*)k_cd_setup<C>, "k_cd_setup");                                                   \
    if (rc == GB_OK)                                                                                         \
      k_cd_setup<C><<<(unsigned)grid, kThreads, M->stage_bytes, st>>>(M->d_blob, M->stage_bytes, B, q, v, ddq, lam, \
                                                                       tab, set->n, (int)nju, Js, Aq, Av, Cq, Fe); \
    break;
      GB_CD_SETUP(8)
      GB_CD_SETUP(16)
      GB_CD_SETUP(32)
      GB_CD_SETUP(64)
      GB_CD_SETUP(128)
#undef GB_CD_SETUP
      default:
        rc = set_error(GB_ERR_UNSUPPORTED, "model too large");
    }
    if (rc == GB_OK) rc = cuda_error(cudaGetLastError(), "k_cd_setup");
  } else if (rc == GB_OK) {
    rc = cuda_error(cudaMemsetAsync(Fe, 0, sizeof(double) * 6 * nju * B, st), "cudaMemsetAsync");
  }
  if (rc == GB_OK)
    rc = launch_rnea_derivs_fext(M, precision, B, q, v, ddq, Arr{Fe, 1, B}, Arr{dtq, 1, B}, Arr{dtv, 1, B},
                                 Arr{dMs, 1, B}, st);
  // the assembly (hxx:815-990), column-parallel: M^-1 and W = M^-1 dtau_dx by tree solves,
  // JMinv = J M^-1 and R = dac_dx - J W over each constraint's dofs, the Delassus factor and osim,
  // the proximal recursion per column, then ddq_dtau = M^-1 + JMinv^T dlambda_dtau and
  // ddq_dx = -W + JMinv^T dlambda_dx (= -M^-1 (dtau_dx - J^T dlambda_dx))
  const unsigned gc = (unsigned)((B * nv + kThreads - 1) / kThreads), gr = (unsigned)((B * nc + kThreads - 1) / kThreads);
  if (rc == GB_OK) rc = opt_in((const void*)k_tree_solve_cols, "k_tree_solve_cols");
  if (rc == GB_OK) rc = opt_in((const void*)k_llt, "k_llt");
  if (rc == GB_OK) rc = opt_in((const void*)k_out_rows, "k_out_rows");
  const Arr none{nullptr, 0, 0};
  if (rc == GB_OK) {
    k_tree_solve_cols<<<gc, kThreads, M->stage_bytes, st>>>(M->d_blob, M->stage_bytes, B, (int)nv, Us, Ds, Mis, 1);
    k_tree_solve_cols<<<gc, kThreads, M->stage_bytes, st>>>(M->d_blob, M->stage_bytes, B, (int)nv, Us, Ds, dtq, 0);
    k_tree_solve_cols<<<gc, kThreads, M->stage_bytes, st>>>(M->d_blob, M->stage_bytes, B, (int)nv, Us, Ds, dtv, 0);
    rc = cuda_error(cudaGetLastError(), "k_tree_solve_cols");
  }
  if (rc == GB_OK && nc > 0) {
    k_jprod_rows<<<gr, kThreads, 0, st>>>(B, (int)nc, (int)nv, (int)nv, tab, set->n, clist, Js, Mis, nullptr, 1.0, JMs);
    k_delassus_cols<<<gr, kThreads, 0, st>>>(B, (int)nc, (int)nv, tab, set->n, clist, Js, JMs, s.mu, Gs, none);
    k_llt<<<(unsigned)grid, kThreads, M->stage_bytes, st>>>(M->d_blob, M->stage_bytes, B, (int)nc, Gs);
    k_osim_cols<<<gr, kThreads, 0, st>>>(B, (int)nc, Gs, Os, none);
    k_prox_cols<<<gc, kThreads, 0, st>>>(B, (int)nc, (int)nv, Os, its, s.mu, -1.0, JMs, Xs, Ts, dl_dtau, nullptr);
    rc = cuda_error(cudaGetLastError(), "the Delassus kernels");
  }
  if (rc == GB_OK) {
    k_out_rows<<<gc, kThreads, M->stage_bytes, st>>>(M->d_blob, M->stage_bytes, B, (int)nc, Mis, 1.0, JMs, Xs,
                                                    ddq_dtau, (int)nv, 0, 0);
    rc = cuda_error(cudaGetLastError(), "k_out_rows");
  }
  for (int pass = 0; pass < 2 && rc == GB_OK; ++pass) {
    double* W = pass == 0 ? dtq : dtv;
    if (nc > 0) {
      k_jprod_rows<<<gr, kThreads, 0, st>>>(B, (int)nc, (int)nv, (int)nv, tab, set->n, clist, Js, W,
                                            pass == 0 ? Aq : Av, -1.0, Rs);
      k_prox_cols<<<gc, kThreads, 0, st>>>(B, (int)nc, (int)nv, Os, its, s.mu, -1.0, Rs, Xs, Ts,
                                           pass == 0 ? dl_dq : dl_dv, pass == 0 ? Cq : nullptr);
    }
    k_out_rows<<<gc, kThreads, M->stage_bytes, st>>>(M->d_blob, M->stage_bytes, B, (int)nc, W, -1.0, JMs, Xs,
                                                    pass == 0 ? ddq_dq : ddq_dv, (int)nv, 0, 0);
    rc = cuda_error(cudaGetLastError(), "k_out_rows");
  }
  if (rc == GB_OK && iters_out)
    rc = cuda_error(cudaMemcpyAsync(iters_out, its, sizeof(int) * B, cudaMemcpyDefault, st), "cudaMemcpyAsync");
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
