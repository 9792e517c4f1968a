// Test infrastructure: CPU oracle for the batched rigid-body dynamics path.
//
// This header is a plain-C++ restatement (no Eigen) of the reference algorithms
// that the GPU kernels must reproduce.  It is used only by the tests, by the
// smoke check and by the CPU baseline leg of the benchmark; the product path
// never links it.  Every function names the reference file:line it follows.
//
// Parity status: the reference (Pinocchio 3.7.0) cannot be compiled in this
// environment (Eigen and Boost are absent), and its tests hold no golden
// vectors.  The oracle is therefore pinned by the reference's own identity
// tests (ABA∘RNEA round trip, M·a + nle = tau, CRBA vs RNEA columns,
// Minv·M = I, UDU^T = M, finite-difference derivative checks, batch == serial)
// and by analytic known-answer cases.  Against reference *outputs* it is
// "parity unpinned".
//
// Scalar T may be double, long double, float, or the FLOP-counting scalar
// FlopScalar (flop_scalar.hpp).  Storage conventions:
//   * SE3: rotation R row-major (R[3*r+c]) and translation t.
//   * Motion / Force 6-vectors: [linear(0:3); angular(3:6)]
//     (reference spatial/force-tpl.hpp:27, motion-tpl.hpp).
//   * Inertia: mass m, lever c (COM), rotational inertia about the COM as a
//     packed symmetric [xx, xy, yy, xz, yz, zz] (spatial/symmetric3.hpp:46-49).
//   * 6x6 matrices row-major; 6 x nv sets column-major (column k at 6*k);
//     nv x nv matrices row-major (the reference's RowMatrixXs,
//     multibody/data.hpp:401-416).
#pragma once

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <stdexcept>
#include <string>
#include <vector>

namespace orc {

enum JointType {
  JT_NONE = 0, JT_RX = 1, JT_RY = 2, JT_RZ = 3, JT_FF = 4, JT_PX = 5, JT_PY = 6, JT_PZ = 7,
  JT_RU = 8,  // JointModelRevoluteUnaligned (multibody/joint/joint-revolute-unaligned.hpp)
  JT_PU = 9,  // JointModelPrismaticUnaligned (multibody/joint/joint-prismatic-unaligned.hpp)
  JT_TR = 10,   // JointModelTranslation (multibody/joint/joint-translation.hpp): nq = nv = 3
  JT_SPH = 11,  // JointModelSpherical (multibody/joint/joint-spherical.hpp): quaternion, nq 4, nv 3
  JT_PL = 12,   // JointModelPlanar (multibody/joint/joint-planar.hpp): (x, y, cos, sin), nq 4, nv 3
  // JointModelRevoluteUnboundedTpl<axis> (multibody/joint/joint-revolute-unbounded.hpp):
  // q = (cos, sin), nq 2, nv 1; the unaligned form (joint-revolute-unbounded-unaligned.hpp)
  JT_RUBX = 13, JT_RUBY = 14, JT_RUBZ = 15, JT_RUBU = 16
};
inline bool three_dof(int jt) { return jt == JT_TR || jt == JT_SPH || jt == JT_PL; }
inline bool unbounded(int jt) { return jt >= JT_RUBX && jt <= JT_RUBU; }
enum Convention { LOCAL = 0, WORLD = 1 };  // reference multibody/fwd.hpp:73-81

// ---------------------------------------------------------------------------
// scalar helpers (overloaded for every scalar type the oracle is built for)
// ---------------------------------------------------------------------------
inline double o_sqrt(double x) { return std::sqrt(x); }
inline long double o_sqrt(long double x) { return std::sqrt(x); }
inline float o_sqrt(float x) { return std::sqrt(x); }
inline void o_sincos(double a, double* s, double* c) { *s = std::sin(a); *c = std::cos(a); }
inline void o_sincos(long double a, long double* s, long double* c) { *s = std::sin(a); *c = std::cos(a); }
inline void o_sincos(float a, float* s, float* c) { *s = std::sin(a); *c = std::cos(a); }
template <class T> inline T o_max(const T& a, const T& b) { return (a < b) ? b : a; }
template <class T> inline T o_eps() { return std::numeric_limits<T>::epsilon(); }

// ---------------------------------------------------------------------------
// Model description (double storage) and the tree tables of DataTpl
// ---------------------------------------------------------------------------
struct Model {
  int njoints = 0, nq = 0, nv = 0;
  std::vector<int> parents, jtype, idx_q, idx_v, nqs, nvs;
  std::vector<double> placement;  // 12 per joint: R (row-major 9), t (3)
  std::vector<double> inertia;    // 10 per joint: m, c[3], I[6]
  std::vector<double> armature;   // nv
  std::vector<double> axis;       // 3 per joint: the unit axis of a JT_RU / JT_PU joint
  double gravity[6] = {0, 0, -9.81, 0, 0, 0};
  // derived tables (multibody/data.hxx:195-306)
  std::vector<int> lastChild, nvSubtree, parents_fromRow, nvSubtree_fromRow;

  static int joint_nq(int jt) {
    return jt == JT_FF ? 7 : jt == JT_NONE ? 0 : jt == JT_TR ? 3 : (jt == JT_SPH || jt == JT_PL) ? 4 : unbounded(jt) ? 2 : 1;
  }
  static int joint_nv(int jt) { return jt == JT_FF ? 6 : jt == JT_NONE ? 0 : three_dof(jt) ? 3 : 1; }

  // Validates the description and fills the derived tables.
  // lastChild / nvSubtree: data.hxx:195-225 (no mimic joints).
  // parents_fromRow / nvSubtree_fromRow: data.hxx:250-306.
  void finalize() {
    if (njoints < 1) throw std::invalid_argument("njoints must be >= 1");
    nqs.assign(njoints, 0);
    nvs.assign(njoints, 0);
    idx_q.assign(njoints, 0);
    idx_v.assign(njoints, 0);
    int cq = 0, cv = 0;
    for (int i = 0; i < njoints; ++i) {
      if (i == 0) {
        if (jtype[0] != JT_NONE) throw std::invalid_argument("joint 0 must be the universe");
        continue;
      }
      if (jtype[i] < JT_RX || jtype[i] > JT_RUBU) throw std::invalid_argument("unsupported joint type");
      if (jtype[i] == JT_RU || jtype[i] == JT_PU || jtype[i] == JT_RUBU) {
        if ((int)axis.size() != 3 * njoints) throw std::invalid_argument("unaligned joints need the axis table");
        const double n = std::sqrt(axis[3 * i] * axis[3 * i] + axis[3 * i + 1] * axis[3 * i + 1] +
                                   axis[3 * i + 2] * axis[3 * i + 2]);
        if (!(n > 0.0)) throw std::invalid_argument("zero joint axis");
        for (int k = 0; k < 3; ++k) axis[3 * i + k] /= n;
      }
      if (parents[i] < 0 || parents[i] >= i) throw std::invalid_argument("parents[i] must be < i");
      nqs[i] = joint_nq(jtype[i]);
      nvs[i] = joint_nv(jtype[i]);
      idx_q[i] = cq;
      idx_v[i] = cv;
      cq += nqs[i];
      cv += nvs[i];
    }
    nq = cq;
    nv = cv;
    if ((int)armature.size() != nv) armature.assign(nv, 0.0);
    lastChild.assign(njoints, -1);
    nvSubtree.assign(njoints, 0);
    for (int i = njoints - 1; i >= 0; --i) {
      if (lastChild[i] == -1) lastChild[i] = i;
      const int parent = i > 0 ? parents[i] : 0;
      lastChild[parent] = std::max(lastChild[i], lastChild[parent]);
      const int lc = lastChild[i];
      nvSubtree[i] = idx_v[lc] + nvs[lc] - idx_v[i];
    }
    parents_fromRow.assign(nv, -1);
    nvSubtree_fromRow.assign(nv, 0);
    for (int j = 1; j < njoints; ++j) {
      const int parent = parents[j];
      const int iv = idx_v[j];
      parents_fromRow[iv] = parent > 0 ? idx_v[parent] + nvs[parent] - 1 : -1;
      nvSubtree_fromRow[iv] = nvSubtree[j];
      for (int row = 1; row < nvs[j]; ++row) {
        parents_fromRow[iv + row] = iv + row - 1;
        nvSubtree_fromRow[iv + row] = nvSubtree[j] - row;
      }
    }
    // CRBA requires compact (depth-first) subtrees: crba.hxx:573-595.
    for (int i = 1; i < njoints; ++i) {
      for (int k = i + 1; k <= lastChild[i]; ++k) {
        int a = k;
        while (a > i) a = parents[a];
        if (a != i) throw std::invalid_argument("joints are not in depth-first order");
      }
    }
  }
};

// ---------------------------------------------------------------------------
// spatial algebra (restated from the reference spatial/ headers)
// ---------------------------------------------------------------------------
template <class T> struct SE3 { T R[9]; T t[3]; };
template <class T> struct Vec6 { T v[6]; };  // motion or force, [lin; ang]
template <class T> struct Iner { T m; T c[3]; T I[6]; };
template <class T> struct Mat6 { T a[36]; };

template <class T> inline void cross3(const T* a, const T* b, T* o) {
  T x = a[1] * b[2] - a[2] * b[1];
  T y = a[2] * b[0] - a[0] * b[2];
  T z = a[0] * b[1] - a[1] * b[0];
  o[0] = x; o[1] = y; o[2] = z;
}
template <class T> inline void matvec(const T* R, const T* x, T* o) {
  T a = R[0] * x[0] + R[1] * x[1] + R[2] * x[2];
  T b = R[3] * x[0] + R[4] * x[1] + R[5] * x[2];
  T c = R[6] * x[0] + R[7] * x[1] + R[8] * x[2];
  o[0] = a; o[1] = b; o[2] = c;
}
template <class T> inline void matTvec(const T* R, const T* x, T* o) {
  T a = R[0] * x[0] + R[3] * x[1] + R[6] * x[2];
  T b = R[1] * x[0] + R[4] * x[1] + R[7] * x[2];
  T c = R[2] * x[0] + R[5] * x[1] + R[8] * x[2];
  o[0] = a; o[1] = b; o[2] = c;
}
template <class T> inline void matmul3(const T* A, const T* B, T* C) {  // C = A B
  T tmp[9];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c)
      tmp[3 * r + c] = A[3 * r + 0] * B[0 + c] + A[3 * r + 1] * B[3 + c] + A[3 * r + 2] * B[6 + c];
  for (int k = 0; k < 9; ++k) C[k] = tmp[k];
}
template <class T> inline void matmul3_ABt(const T* A, const T* B, T* C) {  // C = A B^T
  T tmp[9];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c)
      tmp[3 * r + c] = A[3 * r + 0] * B[3 * c + 0] + A[3 * r + 1] * B[3 * c + 1] + A[3 * r + 2] * B[3 * c + 2];
  for (int k = 0; k < 9; ++k) C[k] = tmp[k];
}

// SE3 composition A*B (spatial/se3-tpl.hpp:314-330).
template <class T> inline SE3<T> se3_mul(const SE3<T>& A, const SE3<T>& B) {
  SE3<T> C;
  matmul3(A.R, B.R, C.R);
  T rt[3];
  matvec(A.R, B.t, rt);
  for (int k = 0; k < 3; ++k) C.t[k] = A.t[k] + rt[k];
  return C;
}
// Motion M.act(m): spatial/motion-dense.hpp:259-263.
template <class T> inline Vec6<T> act_motion(const SE3<T>& M, const Vec6<T>& m) {
  Vec6<T> o;
  matvec(M.R, m.v + 3, o.v + 3);
  T rl[3], txw[3];
  matvec(M.R, m.v, rl);
  cross3(M.t, o.v + 3, txw);
  for (int k = 0; k < 3; ++k) o.v[k] = rl[k] + txw[k];
  return o;
}
// Motion M.actInv(m): spatial/motion-dense.hpp:274-279.
template <class T> inline Vec6<T> actinv_motion(const SE3<T>& M, const Vec6<T>& m) {
  Vec6<T> o;
  T txw[3], d[3];
  cross3(M.t, m.v + 3, txw);
  for (int k = 0; k < 3; ++k) d[k] = m.v[k] - txw[k];
  matTvec(M.R, d, o.v);
  matTvec(M.R, m.v + 3, o.v + 3);
  return o;
}
// Force M.act(f): spatial/force-dense.hpp:214-219.
template <class T> inline Vec6<T> act_force(const SE3<T>& M, const Vec6<T>& f) {
  Vec6<T> o;
  matvec(M.R, f.v, o.v);
  matvec(M.R, f.v + 3, o.v + 3);
  T txf[3];
  cross3(M.t, o.v, txf);
  for (int k = 0; k < 3; ++k) o.v[3 + k] += txf[k];
  return o;
}
// Motion cross v ^ w (spatial/motion-dense.hpp:217-227): w.motionAction(v).
template <class T> inline Vec6<T> cross_motion(const Vec6<T>& v, const Vec6<T>& w) {
  Vec6<T> o;
  T a[3], b[3];
  cross3(v.v, w.v + 3, a);
  cross3(v.v + 3, w.v, b);
  for (int k = 0; k < 3; ++k) o.v[k] = a[k] + b[k];
  cross3(v.v + 3, w.v + 3, o.v + 3);
  return o;
}
// Force cross v.cross(f) (spatial/force-dense.hpp:178-182): f.motionAction(v).
template <class T> inline Vec6<T> cross_force(const Vec6<T>& v, const Vec6<T>& f) {
  Vec6<T> o;
  cross3(v.v + 3, f.v, o.v);
  T a[3], b[3];
  cross3(v.v + 3, f.v + 3, a);
  cross3(v.v, f.v, b);
  for (int k = 0; k < 3; ++k) o.v[3 + k] = a[k] + b[k];
  return o;
}
template <class T> inline Vec6<T> add6(const Vec6<T>& a, const Vec6<T>& b) {
  Vec6<T> o;
  for (int k = 0; k < 6; ++k) o.v[k] = a.v[k] + b.v[k];
  return o;
}
template <class T> inline Vec6<T> zero6() {
  Vec6<T> o;
  for (int k = 0; k < 6; ++k) o.v[k] = T(0);
  return o;
}

// Symmetric3 right multiplication (spatial/symmetric3.hpp:490-499).
template <class T> inline void sym3_mul(const T* S, const T* x, T* o) {
  T a = S[0] * x[0] + S[1] * x[1] + S[3] * x[2];
  T b = S[1] * x[0] + S[2] * x[1] + S[4] * x[2];
  T c = S[3] * x[0] + S[4] * x[1] + S[5] * x[2];
  o[0] = a; o[1] = b; o[2] = c;
}
// Symmetric3 R*S*R^T via the L-decomposition (spatial/symmetric3.hpp:552-600).
template <class T> inline void sym3_rotate(const T* d, const T* R, T* out) {
  const T L00 = d[0] - d[5], L01 = d[1];
  const T L10 = d[1], L11 = d[2] - d[5];
  const T L20 = T(2) * d[3], L21 = d[4] + d[4];
  // Y = R.block<2,3>(1,0) * L
  const T Y00 = R[3] * L00 + R[4] * L10 + R[5] * L20;
  const T Y01 = R[3] * L01 + R[4] * L11 + R[5] * L21;
  const T Y10 = R[6] * L00 + R[7] * L10 + R[8] * L20;
  const T Y11 = R[6] * L01 + R[7] * L11 + R[8] * L21;
  T s[6];
  s[1] = Y00 * R[0] + Y01 * R[1];
  s[2] = Y00 * R[3] + Y01 * R[4];
  s[3] = Y10 * R[0] + Y11 * R[1];
  s[4] = Y10 * R[3] + Y11 * R[4];
  s[5] = Y10 * R[6] + Y11 * R[7];
  const T r0 = -R[0] * d[4] + R[1] * d[3];
  const T r1 = -R[3] * d[4] + R[4] * d[3];
  const T r2 = -R[6] * d[4] + R[7] * d[3];
  s[0] = L00 + L11 - s[2] - s[5];
  s[0] += d[5];
  s[1] += r2;
  s[2] += d[5];
  s[3] -= r1;
  s[4] += r0;
  s[5] += d[5];
  for (int k = 0; k < 6; ++k) out[k] = s[k];
}

// Inertia * motion (spatial/inertia.hpp:729-735).
template <class T> inline Vec6<T> iner_mul(const Iner<T>& Y, const Vec6<T>& v) {
  Vec6<T> f;
  T cxw[3];
  cross3(Y.c, v.v + 3, cxw);
  for (int k = 0; k < 3; ++k) f.v[k] = Y.m * (v.v[k] - cxw[k]);
  sym3_mul(Y.I, v.v + 3, f.v + 3);
  T cxf[3];
  cross3(Y.c, f.v, cxf);
  for (int k = 0; k < 3; ++k) f.v[3 + k] += cxf[k];
  return f;
}
// M.act(Y) (spatial/inertia.hpp:873-880).
template <class T> inline Iner<T> iner_act(const SE3<T>& M, const Iner<T>& Y) {
  Iner<T> o;
  o.m = Y.m;
  T rc[3];
  matvec(M.R, Y.c, rc);
  for (int k = 0; k < 3; ++k) o.c[k] = M.t[k] + rc[k];
  sym3_rotate(Y.I, M.R, o.I);
  return o;
}
// Ya += Yb (spatial/inertia.hpp:659-673).
template <class T> inline void iner_add(Iner<T>& Ya, const Iner<T>& Yb) {
  const T eps = o_eps<T>();
  const T mab = Ya.m + Yb.m;
  const T mab_inv = T(1) / o_max(mab, eps);
  T AB[3];
  for (int k = 0; k < 3; ++k) AB[k] = Ya.c[k] - Yb.c[k];
  const T sa = Ya.m * mab_inv, sb = Yb.m * mab_inv;
  for (int k = 0; k < 3; ++k) Ya.c[k] *= sa;
  for (int k = 0; k < 3; ++k) Ya.c[k] += sb * Yb.c[k];
  for (int k = 0; k < 6; ++k) Ya.I[k] += Yb.I[k];
  const T al = Ya.m * Yb.m * mab_inv;
  const T x = AB[0], y = AB[1], z = AB[2];
  Ya.I[0] += al * (y * y + z * z);
  Ya.I[1] -= al * x * y;
  Ya.I[2] += al * (x * x + z * z);
  Ya.I[3] -= al * x * z;
  Ya.I[4] -= al * y * z;
  Ya.I[5] += al * (x * x + y * y);
  Ya.m = mab;
}
// (I - m [c]x^2) packed (Symmetric3 operator-(AlphaSkewSquare), symmetric3.hpp:252-259).
template <class T> inline void sym3_minus_mskewsq(const T* I, T m, const T* c, T* o) {
  const T x = c[0], y = c[1], z = c[2];
  o[0] = I[0] + m * (y * y + z * z);
  o[1] = I[1] - m * x * y;
  o[2] = I[2] + m * (x * x + z * z);
  o[3] = I[3] - m * x * z;
  o[4] = I[4] - m * y * z;
  o[5] = I[5] + m * (x * x + y * y);
}
template <class T> inline void sym3_full(const T* s, T* M) {  // packed -> 3x3
  M[0] = s[0]; M[1] = s[1]; M[2] = s[3];
  M[3] = s[1]; M[4] = s[2]; M[5] = s[4];
  M[6] = s[3]; M[7] = s[4]; M[8] = s[5];
}
// Y.matrix() (spatial/inertia.hpp:481-491).
template <class T> inline Mat6<T> iner_matrix(const Iner<T>& Y) {
  Mat6<T> M;
  for (int k = 0; k < 36; ++k) M.a[k] = T(0);
  for (int k = 0; k < 3; ++k) M.a[6 * k + k] = Y.m;
  // ANGULAR,LINEAR = alphaSkew(m, c) (spatial/skew.hpp:134-150)
  T S[9];
  S[0] = T(0);
  S[1] = -Y.c[2] * Y.m;
  S[2] = Y.c[1] * Y.m;
  S[3] = -S[1];
  S[4] = T(0);
  S[5] = -Y.c[0] * Y.m;
  S[6] = -S[2];
  S[7] = -S[5];
  S[8] = T(0);
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) {
      M.a[6 * (3 + r) + c] = S[3 * r + c];
      M.a[6 * r + 3 + c] = -S[3 * r + c];
    }
  T p[6], F[9];
  sym3_minus_mskewsq(Y.I, Y.m, Y.c, p);
  sym3_full(p, F);
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) M.a[6 * (3 + r) + 3 + c] = F[3 * r + c];
  return M;
}
template <class T> inline void skew3(const T* v, T* M) {
  M[0] = T(0); M[1] = -v[2]; M[2] = v[1];
  M[3] = v[2]; M[4] = T(0); M[5] = -v[0];
  M[6] = -v[1]; M[7] = v[0]; M[8] = T(0);
}
// skewSquare(u, v) = v u^T - (u.v) I (spatial/skew.hpp:181-200).
template <class T> inline void skewsq3(const T* u, const T* v, T* C) {
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) C[3 * r + c] = v[r] * u[c];
  const T d = u[0] * v[0] + u[1] * v[1] + u[2] * v[2];
  C[0] -= d; C[4] -= d; C[8] -= d;
}
// Y.variation(v) (spatial/inertia.hpp:750-770).
template <class T> inline Mat6<T> iner_variation(const Iner<T>& Y, const Vec6<T>& v) {
  Mat6<T> res;
  T mvl[3], mva[3];
  for (int k = 0; k < 3; ++k) { mvl[k] = v.v[k] * Y.m; mva[k] = v.v[3 + k] * Y.m; }
  T A[9], B[9], C[9], Bla[9];
  skew3(mvl, A);
  skewsq3(mva, Y.c, B);
  skewsq3(Y.c, mva, C);
  for (int k = 0; k < 9; ++k) Bla[k] = -A[k] - B[k] + C[k];  // LINEAR,ANGULAR block
  T D1[9], D2[9], Daa[9];
  skewsq3(mvl, Y.c, D1);
  skewsq3(Y.c, mvl, D2);
  for (int k = 0; k < 9; ++k) Daa[k] = -D1[k] - D2[k];
  T p[6], Ll[9];
  sym3_minus_mskewsq(Y.I, Y.m, Y.c, p);
  sym3_full(p, Ll);
  T Sw[9], P[9];
  skew3(v.v + 3, Sw);
  matmul3(Ll, Sw, P);
  for (int k = 0; k < 9; ++k) Daa[k] -= P[k];
  // cross(v.ang, Ll): rows = v x (columns) (spatial/skew.hpp:228-245)
  const T* w = v.v + 3;
  for (int c = 0; c < 3; ++c) {
    Daa[0 * 3 + c] += w[1] * Ll[6 + c] - w[2] * Ll[3 + c];
    Daa[1 * 3 + c] += w[2] * Ll[0 + c] - w[0] * Ll[6 + c];
    Daa[2 * 3 + c] += w[0] * Ll[3 + c] - w[1] * Ll[0 + c];
  }
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) {
      res.a[6 * r + c] = T(0);
      res.a[6 * r + 3 + c] = Bla[3 * r + c];
      res.a[6 * (3 + r) + c] = Bla[3 * c + r];
      res.a[6 * (3 + r) + 3 + c] = Daa[3 * r + c];
    }
  return res;
}
// addForceCrossMatrix (algorithm/rnea-derivatives.hxx:358-367).
template <class T> inline void add_force_cross_matrix(const Vec6<T>& f, Mat6<T>& M) {
  auto add_skew = [&](const T* v, int r0, int c0) {  // spatial/skew.hpp:68-82
    M.a[6 * (r0 + 0) + c0 + 1] -= v[2];
    M.a[6 * (r0 + 0) + c0 + 2] += v[1];
    M.a[6 * (r0 + 1) + c0 + 0] += v[2];
    M.a[6 * (r0 + 1) + c0 + 2] -= v[0];
    M.a[6 * (r0 + 2) + c0 + 0] -= v[1];
    M.a[6 * (r0 + 2) + c0 + 1] += v[0];
  };
  T nl[3] = {-f.v[0], -f.v[1], -f.v[2]};
  T na[3] = {-f.v[3], -f.v[4], -f.v[5]};
  add_skew(nl, 0, 3);
  add_skew(nl, 3, 0);
  add_skew(na, 3, 3);
}
template <class T> inline Vec6<T> mat6_vec(const Mat6<T>& M, const T* x) {
  Vec6<T> o;
  for (int r = 0; r < 6; ++r) {
    T s = M.a[6 * r] * x[0];
    for (int c = 1; c < 6; ++c) s += M.a[6 * r + c] * x[c];
    o.v[r] = s;
  }
  return o;
}
// SE3actOn(M, I) for a 6x6 matrix (algorithm/aba.hxx:22-76).
template <class T> inline Mat6<T> se3_act_on(const SE3<T>& M, const Mat6<T>& I) {
  T Ai[9], Bi[9], Di[9];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) {
      Ai[3 * r + c] = I.a[6 * r + c];
      Bi[3 * r + c] = I.a[6 * r + 3 + c];
      Di[3 * r + c] = I.a[6 * (3 + r) + 3 + c];
    }
  const T* R = M.R;
  const T* t = M.t;
  T Ao[9], Bo[9], Co[9], Do[9];
  matmul3(R, Ai, Do);
  matmul3_ABt(Do, R, Ao);
  matmul3(R, Bi, Do);
  matmul3_ABt(Do, R, Bo);
  matmul3(R, Di, Co);
  matmul3_ABt(Co, R, Do);
  for (int k = 0; k < 3; ++k) {  // Do.row(k) += t x Bo.col(k)
    T col[3] = {Bo[k], Bo[3 + k], Bo[6 + k]}, o[3];
    cross3(t, col, o);
    for (int c = 0; c < 3; ++c) Do[3 * k + c] += o[c];
  }
  for (int k = 0; k < 3; ++k) {  // Co.col(k) = t x Ao.col(k)
    T col[3] = {Ao[k], Ao[3 + k], Ao[6 + k]}, o[3];
    cross3(t, col, o);
    for (int r = 0; r < 3; ++r) Co[3 * r + k] = o[r];
  }
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) Co[3 * r + c] += Bo[3 * c + r];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) Bo[3 * r + c] = Co[3 * c + r];
  for (int k = 0; k < 3; ++k) {  // Do.col(k) += t x Bo.col(k)
    T col[3] = {Bo[k], Bo[3 + k], Bo[6 + k]}, o[3];
    cross3(t, col, o);
    for (int r = 0; r < 3; ++r) Do[3 * r + k] += o[r];
  }
  Mat6<T> res;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) {
      res.a[6 * r + c] = Ao[3 * r + c];
      res.a[6 * r + 3 + c] = Bo[3 * r + c];
      res.a[6 * (3 + r) + c] = Co[3 * r + c];
      res.a[6 * (3 + r) + 3 + c] = Do[3 * r + c];
    }
  return res;
}

// Inverse of a small SPD matrix through an unblocked LLT followed by two
// triangular solves on the identity, as PerformStYSInversion does
// (multibody/joint/joint-common-operations.hpp:20-33 with Eigen 3.4 LLT).
template <class T> inline void llt_inverse(int n, const T* A, T* Ainv) {
  T L[36];
  for (int k = 0; k < n * n; ++k) L[k] = A[k];
  for (int k = 0; k < n; ++k) {
    T x = L[n * k + k];
    for (int j = 0; j < k; ++j) x -= L[n * k + j] * L[n * k + j];
    x = o_sqrt(x);
    L[n * k + k] = x;
    for (int i = k + 1; i < n; ++i) {
      T s = L[n * i + k];
      for (int j = 0; j < k; ++j) s -= L[n * i + j] * L[n * k + j];
      L[n * i + k] = s / x;
    }
  }
  for (int c = 0; c < n; ++c) {
    T y[6];
    for (int i = 0; i < n; ++i) {  // L y = e_c
      T s = (i == c) ? T(1) : T(0);
      for (int j = 0; j < i; ++j) s -= L[n * i + j] * y[j];
      y[i] = s / L[n * i + i];
    }
    for (int i = n - 1; i >= 0; --i) {  // L^T x = y
      T s = y[i];
      for (int j = i + 1; j < n; ++j) s -= L[n * j + i] * y[j];
      y[i] = s / L[n * i + i];
    }
    for (int i = 0; i < n; ++i) Ainv[n * i + c] = y[i];
  }
}

// ---------------------------------------------------------------------------
// joint models: revolute about x/y/z and free-flyer
// ---------------------------------------------------------------------------
template <class T> inline SE3<T> placement_of(const Model& m, int i) {
  SE3<T> M;
  for (int k = 0; k < 9; ++k) M.R[k] = T(m.placement[12 * i + k]);
  for (int k = 0; k < 3; ++k) M.t[k] = T(m.placement[12 * i + 9 + k]);
  return M;
}
template <class T> inline Iner<T> inertia_of(const Model& m, int i) {
  Iner<T> Y;
  Y.m = T(m.inertia[10 * i]);
  for (int k = 0; k < 3; ++k) Y.c[k] = T(m.inertia[10 * i + 1 + k]);
  for (int k = 0; k < 6; ++k) Y.I[k] = T(m.inertia[10 * i + 4 + k]);
  return Y;
}
// Joint transform M(q).
//  * revolute: TransformRevoluteTpl::_setRotation (joint-revolute.hpp:213-235),
//    angle through SINCOS (math/sincos.hpp:27-55); calc at joint-revolute.hpp:811-821.
//  * prismatic: translation q[0] along the axis, identity rotation
//    (TransformPrismaticTpl, joint-prismatic.hpp:232-284; calc at 700-704).
//  * free-flyer: translation q[0:3], rotation = Eigen Quaternion::matrix()
//    of (x,y,z,w) = q[3:7], not normalised (joint-free-flyer.hpp:333-375).
//  * translation: (I, q[0:3]) (TransformTranslationTpl, joint-translation.hpp; calc);
//  * spherical: rotation = Quaternion::matrix() of q[0:4] = (x,y,z,w), no translation
//    (joint-spherical.hpp:504-531);
//  * planar: rotation about z with (cos, sin) = q[2:4], translation (q[0], q[1], 0)
//    (joint-planar.hpp:586-609).
template <class T> inline void quat_rotation(const T* qv, T* R) {
  const T x = qv[0], y = qv[1], z = qv[2], w = qv[3];
  const T tx = T(2) * x, ty = T(2) * y, tz = T(2) * z;
  const T twx = tx * w, twy = ty * w, twz = tz * w;
  const T txx = tx * x, txy = ty * x, txz = tz * x;
  const T tyy = ty * y, tyz = tz * y, tzz = tz * z;
  R[0] = T(1) - (tyy + tzz); R[1] = txy - twz; R[2] = txz + twy;
  R[3] = txy + twz; R[4] = T(1) - (txx + tzz); R[5] = tyz - twx;
  R[6] = txz - twy; R[7] = tyz + twx; R[8] = T(1) - (txx + tyy);
}
template <class T> inline SE3<T> joint_transform(int jt, const T* q) {
  SE3<T> M;
  for (int k = 0; k < 9; ++k) M.R[k] = T(0);
  for (int k = 0; k < 3; ++k) M.t[k] = T(0);
  if (jt == JT_TR) {
    for (int k = 0; k < 3; ++k) { M.R[4 * k] = T(1); M.t[k] = q[k]; }
    return M;
  }
  if (jt == JT_SPH) {
    quat_rotation(q, M.R);
    return M;
  }
  if (jt == JT_PL) {
    const T c = q[2], s = q[3];
    M.R[0] = c; M.R[1] = -s; M.R[3] = s; M.R[4] = c; M.R[8] = T(1);
    M.t[0] = q[0]; M.t[1] = q[1];
    return M;
  }
  if (jt == JT_FF) {
    const T x = q[3], y = q[4], z = q[5], w = q[6];
    const T tx = T(2) * x, ty = T(2) * y, tz = T(2) * z;
    const T twx = tx * w, twy = ty * w, twz = tz * w;
    const T txx = tx * x, txy = ty * x, txz = tz * x;
    const T tyy = ty * y, tyz = tz * y, tzz = tz * z;
    M.R[0] = T(1) - (tyy + tzz); M.R[1] = txy - twz; M.R[2] = txz + twy;
    M.R[3] = txy + twz; M.R[4] = T(1) - (txx + tzz); M.R[5] = tyz - twx;
    M.R[6] = txz - twy; M.R[7] = tyz + twx; M.R[8] = T(1) - (txx + tyy);
    for (int k = 0; k < 3; ++k) M.t[k] = q[k];
    return M;
  }
  for (int k = 0; k < 3; ++k) M.R[4 * k] = T(1);
  if (jt >= JT_PX && jt <= JT_PZ) {
    M.t[jt - JT_PX] = q[0];
    return M;
  }
  T s, c;
  int ax = jt - JT_RX;
  if (unbounded(jt)) {  // the unbounded joint's (cos, sin) taken as they are (joint-revolute-unbounded.hpp:154-162)
    c = q[0];
    s = q[1];
    ax = jt - JT_RUBX;
  } else {
    o_sincos(q[0], &s, &c);
  }
  if (ax == 0) { M.R[4] = c; M.R[5] = -s; M.R[7] = s; M.R[8] = c; }
  if (ax == 1) { M.R[0] = c; M.R[2] = s; M.R[6] = -s; M.R[8] = c; }
  if (ax == 2) { M.R[0] = c; M.R[1] = -s; M.R[3] = s; M.R[4] = c; }
  return M;
}
// The motion-subspace entry of a one-dof joint: the angular axis 3 + a of a
// revolute joint (SpatialAxis<ANGULAR + axis>, joint-revolute.hpp:429-543), the
// linear axis a of a prismatic one (SpatialAxis<LINEAR + axis>, joint-prismatic.hpp:353-461).
inline int motion_index(int jt) {
  return unbounded(jt) ? 3 + (jt - JT_RUBX) : jt >= JT_PX ? jt - JT_PX : 3 + (jt - JT_RX);
}
// Column k of the joint motion subspace S (local frame).
// The three-dof joints have unit columns too: translation the linear axes
// (JointMotionSubspaceTranslationTpl), spherical the angular axes
// (JointMotionSubspaceSphericalTpl), planar (vx, vy, wz) (JointMotionSubspacePlanarTpl,
// joint-planar.hpp:380-470); multi_col gives the spatial index of column k.
inline int multi_col(int jt, int k) { return jt == JT_TR ? k : jt == JT_SPH ? 3 + k : (k < 2 ? k : 5); }
template <class T> inline Vec6<T> S_col(int jt, int k) {
  Vec6<T> s = zero6<T>();
  if (jt == JT_FF) s.v[k] = T(1);
  else if (three_dof(jt)) s.v[multi_col(jt, k)] = T(1);
  else s.v[motion_index(jt)] = T(1);
  return s;
}
// Joint velocity vJ = S * qdot_j.
template <class T> inline Vec6<T> joint_velocity(int jt, const T* v) {
  Vec6<T> o = zero6<T>();
  if (jt == JT_FF) for (int k = 0; k < 6; ++k) o.v[k] = v[k];
  else if (three_dof(jt)) for (int k = 0; k < 3; ++k) o.v[multi_col(jt, k)] = v[k];
  else o.v[motion_index(jt)] = v[0];
  return o;
}

// Joint i of a model, unaligned joints included.
//  * revolute unaligned: M = (toRotationMatrix(axis, q), 0) (joint-revolute-unaligned.hpp:668-673;
//    math/rotation.hpp:26-73, the Eigen AngleAxis formula), S = (0, axis);
//  * prismatic unaligned: M = (I, axis q) (joint-prismatic-unaligned.hpp:643-647), S = (axis, 0).
inline bool unaligned(int jt) { return jt == JT_RU || jt == JT_PU || jt == JT_RUBU; }
//  * revolute unbounded unaligned: the same rotation from (cos, sin) = q (no sincos),
//    S = (0, axis) (joint-revolute-unbounded-unaligned.hpp).
template <class T> inline SE3<T> joint_transform(const Model& m, int i, const T* q) {
  const int jt = m.jtype[i];
  if (!unaligned(jt)) return joint_transform<T>(jt, q);
  const T a[3] = {T(m.axis[3 * i]), T(m.axis[3 * i + 1]), T(m.axis[3 * i + 2])};
  SE3<T> M;
  for (int k = 0; k < 9; ++k) M.R[k] = T(0);
  for (int k = 0; k < 3; ++k) M.t[k] = T(0);
  if (jt == JT_PU) {
    for (int k = 0; k < 3; ++k) { M.R[4 * k] = T(1); M.t[k] = a[k] * q[0]; }
    return M;
  }
  T s, c;
  if (jt == JT_RUBU) {
    c = q[0];
    s = q[1];
  } else {
    o_sincos(q[0], &s, &c);
  }
  const T sa[3] = {s * a[0], s * a[1], s * a[2]};
  const T ca[3] = {(T(1) - c) * a[0], (T(1) - c) * a[1], (T(1) - c) * a[2]};
  T t = ca[0] * a[1];
  M.R[1] = t - sa[2]; M.R[3] = t + sa[2];
  t = ca[0] * a[2];
  M.R[2] = t + sa[1]; M.R[6] = t - sa[1];
  t = ca[1] * a[2];
  M.R[5] = t - sa[0]; M.R[7] = t + sa[0];
  for (int k = 0; k < 3; ++k) M.R[4 * k] = ca[k] * a[k] + c;
  return M;
}
template <class T> inline Vec6<T> S_col(const Model& m, int i, int k) {
  const int jt = m.jtype[i];
  if (!unaligned(jt)) return S_col<T>(jt, k);
  Vec6<T> s = zero6<T>();
  const int o = jt == JT_PU ? 0 : 3;
  for (int r = 0; r < 3; ++r) s.v[o + r] = T(m.axis[3 * i + r]);
  return s;
}
template <class T> inline Vec6<T> joint_velocity(const Model& m, int i, const T* v) {
  if (!unaligned(m.jtype[i])) return joint_velocity<T>(m.jtype[i], v);
  Vec6<T> s = S_col<T>(m, i, 0);
  for (int r = 0; r < 6; ++r) s.v[r] *= v[0];
  return s;
}

// ---------------------------------------------------------------------------
// Data workspace (the subset of DataTpl the hot-path algorithms use)
// ---------------------------------------------------------------------------
template <class T> struct Data {
  int nj, nv;
  std::vector<SE3<T>> liMi, oMi;
  std::vector<Vec6<T>> v, a, a_gf, f, h, ov, oa, oa_gf, oh, of;
  std::vector<Iner<T>> Ycrb, oYcrb, oinertias;
  std::vector<Mat6<T>> Yaba, doYcrb;
  std::vector<std::vector<T>> Ujoint, Dinvjoint, UDinvjoint;  // 6 x nvj, nvj x nvj, 6 x nvj
  std::vector<T> J, dJ, dVdq, dAdq, dAdv, dFdq, dFdv, dFda, SDinv;  // 6 x nv col-major
  std::vector<std::vector<T>> Fcrb;                                  // nj x (6 x nv)
  std::vector<T> tau, ddq, u;
  std::vector<T> M, Minv, dtau_dq, dtau_dv, ddq_dq, ddq_dv;  // nv x nv row-major
  std::vector<T> U, D, Dinv, tmp;                            // Cholesky
  explicit Data(const Model& m) : nj(m.njoints), nv(m.nv) {
    liMi.resize(nj); oMi.resize(nj);
    for (auto* vec : {&v, &a, &a_gf, &f, &h, &ov, &oa, &oa_gf, &oh, &of}) vec->assign(nj, zero6<T>());
    Ycrb.resize(nj); oYcrb.resize(nj); oinertias.resize(nj);
    Yaba.resize(nj); doYcrb.resize(nj);
    Ujoint.assign(nj, std::vector<T>(36, T(0)));
    Dinvjoint.assign(nj, std::vector<T>(36, T(0)));
    UDinvjoint.assign(nj, std::vector<T>(36, T(0)));
    for (auto* mat : {&J, &dJ, &dVdq, &dAdq, &dAdv, &dFdq, &dFdv, &dFda, &SDinv}) mat->assign(6 * nv, T(0));
    Fcrb.assign(nj, std::vector<T>(6 * nv, T(0)));
    tau.assign(nv, T(0)); ddq.assign(nv, T(0)); u.assign(nv, T(0));
    for (auto* mat : {&M, &Minv, &dtau_dq, &dtau_dv, &ddq_dq, &ddq_dv}) mat->assign((size_t)nv * nv, T(0));
    U.assign((size_t)nv * nv, T(0));
    for (int k = 0; k < nv; ++k) U[(size_t)k * nv + k] = T(1);
    D.assign(nv, T(0)); Dinv.assign(nv, T(0)); tmp.assign(nv, T(0));
  }
};

template <class T> inline Vec6<T> col6(const std::vector<T>& X, int k) {
  Vec6<T> o;
  for (int r = 0; r < 6; ++r) o.v[r] = X[6 * k + r];
  return o;
}
template <class T> inline void set_col6(std::vector<T>& X, int k, const Vec6<T>& c) {
  for (int r = 0; r < 6; ++r) X[6 * k + r] = c.v[r];
}
template <class T> inline T dot6(const Vec6<T>& a, const Vec6<T>& b) {
  T s = a.v[0] * b.v[0];
  for (int k = 1; k < 6; ++k) s += a.v[k] * b.v[k];
  return s;
}
template <class T> inline T dot6p(const T* a, const T* b) {
  T s = a[0] * b[0];
  for (int k = 1; k < 6; ++k) s += a[k] * b[k];
  return s;
}

// External forces: fext holds njoints x 6 values [linear; angular], the force on
// joint i expressed in joint i's frame (the reference's aligned_vector<Force> of
// size njoints, algorithm/rnea.hpp:60-79); NULL for none.  f -= fext_i
// (joint frame) or f -= oMi.act(fext_i) (world frame).
template <class T> inline void sub_fext_local(const T* fext, int i, Vec6<T>& f) {
  if (!fext) return;
  for (int k = 0; k < 6; ++k) f.v[k] -= fext[6 * i + k];
}
template <class T> inline void sub_fext_world(const T* fext, int i, const SE3<T>& oMi, Vec6<T>& f) {
  if (!fext) return;
  Vec6<T> fl;
  for (int k = 0; k < 6; ++k) fl.v[k] = fext[6 * i + k];
  const Vec6<T> fw = act_force(oMi, fl);
  for (int k = 0; k < 6; ++k) f.v[k] -= fw.v[k];
}

// ---------------------------------------------------------------------------
// RNEA (algorithm/rnea.hxx:24-161); with fext rnea.hxx:164-218 (f_i -= fext_i,
// line 205)
// ---------------------------------------------------------------------------
template <class T>
void rnea(const Model& m, Data<T>& d, const T* q, const T* v, const T* a, const T* fext = nullptr) {
  std::fill(d.tau.begin(), d.tau.end(), T(0));
  d.v[0] = zero6<T>();
  for (int k = 0; k < 6; ++k) d.a_gf[0].v[k] = -T(m.gravity[k]);
  for (int i = 1; i < m.njoints; ++i) {  // RneaForwardStep (rnea.hxx:24-80)
    const int p = m.parents[i];
    const int iq = m.idx_q[i], iv = m.idx_v[i];
    const SE3<T> jM = joint_transform<T>(m, i, q + iq);
    d.liMi[i] = se3_mul(placement_of<T>(m, i), jM);
    const Vec6<T> vJ = joint_velocity<T>(m, i, v + iv);
    d.v[i] = vJ;
    if (p > 0) d.v[i] = add6(d.v[i], actinv_motion(d.liMi[i], d.v[p]));
    d.a_gf[i] = cross_motion(d.v[i], vJ);  // c() = 0 for these joints
    d.a_gf[i] = add6(d.a_gf[i], joint_velocity<T>(m, i, a + iv));
    d.a_gf[i] = add6(d.a_gf[i], actinv_motion(d.liMi[i], d.a_gf[p]));
    const Iner<T> Y = inertia_of<T>(m, i);
    d.h[i] = iner_mul(Y, d.v[i]);
    d.f[i] = iner_mul(Y, d.a_gf[i]);
    d.f[i] = add6(d.f[i], cross_force(d.v[i], d.h[i]));
    sub_fext_local(fext, i, d.f[i]);
  }
  for (int i = m.njoints - 1; i > 0; --i) {  // RneaBackwardStep (rnea.hxx:83-108)
    const int p = m.parents[i], iv = m.idx_v[i];
    for (int k = 0; k < m.nvs[i]; ++k) d.tau[iv + k] += dot6(S_col<T>(m, i, k), d.f[i]);
    if (p > 0) d.f[p] = add6(d.f[p], act_force(d.liMi[i], d.f[i]));
  }
  for (int k = 0; k < m.nv; ++k) d.tau[k] += T(m.armature[k]) * a[k];  // rnea.hxx:158
}

// ---------------------------------------------------------------------------
// ABA, LOCAL convention (algorithm/aba.hxx:360-540)
// ---------------------------------------------------------------------------
// with fext: aba.hxx:543-605 (f_i -= fext_i after the forward step, line 584)
template <class T>
void aba_local(const Model& m, Data<T>& d, const T* q, const T* v, const T* tau, const T* fext = nullptr) {
  d.v[0] = zero6<T>();
  for (int k = 0; k < 6; ++k) d.a_gf[0].v[k] = -T(m.gravity[k]);
  d.f[0] = zero6<T>();
  for (int k = 0; k < m.nv; ++k) d.u[k] = tau[k];
  for (int i = 1; i < m.njoints; ++i) {  // AbaLocalConventionForwardStep1 (aba.hxx:360-399)
    const int p = m.parents[i];
    const SE3<T> jM = joint_transform<T>(m, i, q + m.idx_q[i]);
    d.liMi[i] = se3_mul(placement_of<T>(m, i), jM);
    const Vec6<T> vJ = joint_velocity<T>(m, i, v + m.idx_v[i]);
    d.v[i] = vJ;
    if (p > 0) d.v[i] = add6(d.v[i], actinv_motion(d.liMi[i], d.v[p]));
    d.a_gf[i] = cross_motion(d.v[i], vJ);
    const Iner<T> Y = inertia_of<T>(m, i);
    d.Yaba[i] = iner_matrix(Y);
    d.h[i] = iner_mul(Y, d.v[i]);
    d.f[i] = cross_force(d.v[i], d.h[i]);
    sub_fext_local(fext, i, d.f[i]);
  }
  for (int i = m.njoints - 1; i > 0; --i) {  // AbaLocalConventionBackwardStep (aba.hxx:402-434)
    const int p = m.parents[i], jt = m.jtype[i], iv = m.idx_v[i], nvj = m.nvs[i];
    Mat6<T>& Ia = d.Yaba[i];
    for (int k = 0; k < nvj; ++k) d.u[iv + k] -= dot6(S_col<T>(m, i, k), d.f[i]);
    std::vector<T>& U = d.Ujoint[i];
    std::vector<T>& Dinv = d.Dinvjoint[i];
    std::vector<T>& UDinv = d.UDinvjoint[i];
    if (jt == JT_FF) {  // JointModelFreeFlyer::calc_aba (joint-free-flyer.hpp:377-391)
      T StU[36];
      for (int k = 0; k < 36; ++k) { U[k] = Ia.a[k]; StU[k] = Ia.a[k]; }
      for (int k = 0; k < 6; ++k) StU[7 * k] += T(m.armature[iv + k]);
      llt_inverse(6, StU, Dinv.data());
      for (int r = 0; r < 6; ++r)
        for (int c = 0; c < 6; ++c) {
          T s = Ia.a[6 * r] * Dinv[c];
          for (int k = 1; k < 6; ++k) s += Ia.a[6 * r + k] * Dinv[6 * k + c];
          UDinv[6 * r + c] = s;
        }
      if (p > 0)
        for (int r = 0; r < 6; ++r)
          for (int c = 0; c < 6; ++c) {
            T s = UDinv[6 * r] * U[6 * c];
            for (int k = 1; k < 6; ++k) s += UDinv[6 * r + k] * U[6 * c + k];
            Ia.a[6 * r + c] -= s;
          }
    } else if (three_dof(jt)) {  // calc_aba of the three-dof joints with unit columns (translation
                               // joint-translation.hpp, spherical joint-spherical.hpp:572-586, planar
                               // joint-planar.hpp:643-661): U = I S, StU = S^T U + armature, LLT inverse
      int cols[3];
      for (int k = 0; k < 3; ++k) cols[k] = multi_col(jt, k);
      T StU[9];
      for (int r = 0; r < 6; ++r)
        for (int k = 0; k < 3; ++k) U[r * 3 + k] = Ia.a[6 * r + cols[k]];
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) StU[3 * r + c] = U[cols[r] * 3 + c];
      for (int k = 0; k < 3; ++k) StU[4 * k] += T(m.armature[iv + k]);
      llt_inverse(3, StU, Dinv.data());
      for (int r = 0; r < 6; ++r)
        for (int c = 0; c < 3; ++c) {
          T s = U[r * 3] * Dinv[c];
          for (int k = 1; k < 3; ++k) s += U[r * 3 + k] * Dinv[3 * k + c];
          UDinv[r * 3 + c] = s;
        }
      if (p > 0)
        for (int r = 0; r < 6; ++r)
          for (int c = 0; c < 6; ++c) {
            T s = UDinv[r * 3] * U[c * 3];
            for (int k = 1; k < 3; ++k) s += UDinv[r * 3 + k] * U[c * 3 + k];
            Ia.a[6 * r + c] -= s;
          }
    } else if (unaligned(jt)) {  // calc_aba of joint-revolute-unaligned.hpp:695-707 /
                                 // joint-prismatic-unaligned.hpp:671-683: U = I S, Dinv = 1 / (S.U + armature)
      const int o = jt == JT_PU ? 0 : 3;
      T a[3];
      for (int k = 0; k < 3; ++k) a[k] = T(m.axis[3 * i + k]);
      for (int r = 0; r < 6; ++r) U[r] = Ia.a[6 * r + o] * a[0] + Ia.a[6 * r + o + 1] * a[1] + Ia.a[6 * r + o + 2] * a[2];
      Dinv[0] = T(1) / ((a[0] * U[o] + a[1] * U[o + 1] + a[2] * U[o + 2]) + T(m.armature[iv]));
      for (int r = 0; r < 6; ++r) UDinv[r] = U[r] * Dinv[0];
      if (p > 0)
        for (int r = 0; r < 6; ++r)
          for (int c = 0; c < 6; ++c) Ia.a[6 * r + c] -= UDinv[r] * U[c];
    } else {  // JointModelRevolute::calc_aba (joint-revolute.hpp:823-834), prismatic (joint-prismatic.hpp:728-740)
      const int ax = motion_index(jt);
      for (int r = 0; r < 6; ++r) U[r] = Ia.a[6 * r + ax];
      Dinv[0] = T(1) / (Ia.a[6 * ax + ax] + T(m.armature[iv]));
      for (int r = 0; r < 6; ++r) UDinv[r] = U[r] * Dinv[0];
      if (p > 0)
        for (int r = 0; r < 6; ++r)
          for (int c = 0; c < 6; ++c) Ia.a[6 * r + c] -= UDinv[r] * U[c];
    }
    if (p > 0) {
      Vec6<T> pa = mat6_vec(Ia, d.a_gf[i].v);
      for (int r = 0; r < 6; ++r) {
        T s = T(0);
        for (int k = 0; k < nvj; ++k) s += UDinv[r * nvj + k] * d.u[iv + k];
        pa.v[r] += s;
      }
      d.f[i] = add6(d.f[i], pa);
      const Mat6<T> Ip = se3_act_on(d.liMi[i], Ia);
      for (int k = 0; k < 36; ++k) d.Yaba[p].a[k] += Ip.a[k];
      d.f[p] = add6(d.f[p], act_force(d.liMi[i], d.f[i]));
    }
  }
  for (int i = 1; i < m.njoints; ++i) {  // AbaLocalConventionForwardStep2 (aba.hxx:437-468)
    const int p = m.parents[i], iv = m.idx_v[i], nvj = m.nvs[i];
    d.a_gf[i] = add6(d.a_gf[i], actinv_motion(d.liMi[i], d.a_gf[p]));
    const std::vector<T>& Dinv = d.Dinvjoint[i];
    const std::vector<T>& UDinv = d.UDinvjoint[i];
    for (int k = 0; k < nvj; ++k) {
      T s = T(0);
      for (int c = 0; c < nvj; ++c) s += Dinv[k * nvj + c] * d.u[iv + c];
      T w = T(0);
      for (int r = 0; r < 6; ++r) w += UDinv[r * nvj + k] * d.a_gf[i].v[r];
      d.ddq[iv + k] = s - w;
    }
    for (int k = 0; k < nvj; ++k) {
      const Vec6<T> s = S_col<T>(m, i, k);
      for (int r = 0; r < 6; ++r) d.a_gf[i].v[r] += s.v[r] * d.ddq[iv + k];
    }
  }
}

// Shared by the WORLD ABA and the ABA derivatives: the WORLD backward step
// (aba.hxx:142-193 / aba-derivatives.hxx:87-171 Schur part).
template <class T>
void world_schur(const Model& m, Data<T>& d, int i) {
  const int iv = m.idx_v[i], nvj = m.nvs[i];
  Mat6<T>& Ia = d.Yaba[i];
  std::vector<T>& U = d.Ujoint[i];
  std::vector<T>& Dinv = d.Dinvjoint[i];
  std::vector<T>& UDinv = d.UDinvjoint[i];
  for (int k = 0; k < nvj; ++k) d.u[iv + k] -= dot6(col6(d.J, iv + k), d.of[i]);
  for (int k = 0; k < nvj; ++k) {  // U = Ia * Jcols (6 x nvj, row-major)
    const Vec6<T> jc = col6(d.J, iv + k);
    const Vec6<T> uc = mat6_vec(Ia, jc.v);
    for (int r = 0; r < 6; ++r) U[r * nvj + k] = uc.v[r];
  }
  T StU[36];
  for (int r = 0; r < nvj; ++r)
    for (int c = 0; c < nvj; ++c) {
      const Vec6<T> jr = col6(d.J, iv + r);
      T s = jr.v[0] * U[0 * nvj + c];
      for (int k = 1; k < 6; ++k) s += jr.v[k] * U[k * nvj + c];
      StU[r * nvj + c] = s;
    }
  for (int k = 0; k < nvj; ++k) StU[k * nvj + k] += T(m.armature[iv + k]);
  llt_inverse(nvj, StU, Dinv.data());
  for (int r = 0; r < 6; ++r)
    for (int c = 0; c < nvj; ++c) {
      T s = U[r * nvj] * Dinv[c];
      for (int k = 1; k < nvj; ++k) s += U[r * nvj + k] * Dinv[k * nvj + c];
      UDinv[r * nvj + c] = s;
    }
}
template <class T>
void world_schur_update(const Model& m, Data<T>& d, int i) {
  const int p = m.parents[i], iv = m.idx_v[i], nvj = m.nvs[i];
  Mat6<T>& Ia = d.Yaba[i];
  const std::vector<T>& U = d.Ujoint[i];
  const std::vector<T>& UDinv = d.UDinvjoint[i];
  for (int r = 0; r < 6; ++r)
    for (int c = 0; c < 6; ++c) {
      T s = UDinv[r * nvj] * U[c * nvj];
      for (int k = 1; k < nvj; ++k) s += UDinv[r * nvj + k] * U[c * nvj + k];
      Ia.a[6 * r + c] -= s;
    }
  Vec6<T> pa = mat6_vec(Ia, d.oa_gf[i].v);
  for (int r = 0; r < 6; ++r) {
    T s = T(0);
    for (int k = 0; k < nvj; ++k) s += UDinv[r * nvj + k] * d.u[iv + k];
    pa.v[r] += s;
  }
  d.of[i] = add6(d.of[i], pa);
  for (int k = 0; k < 36; ++k) d.Yaba[p].a[k] += Ia.a[k];
  d.of[p] = add6(d.of[p], d.of[i]);
}

// World-frame forward kinematics shared by the WORLD ABA and the ABA
// derivatives (aba.hxx:85-139, aba-derivatives.hxx:22-80).
template <class T>
void world_forward1(const Model& m, Data<T>& d, const T* q, const T* v, int i) {
  const int p = m.parents[i], iv = m.idx_v[i];
  const SE3<T> jM = joint_transform<T>(m, i, q + m.idx_q[i]);
  d.liMi[i] = se3_mul(placement_of<T>(m, i), jM);
  d.oMi[i] = (p > 0) ? se3_mul(d.oMi[p], d.liMi[i]) : d.liMi[i];
  for (int k = 0; k < m.nvs[i]; ++k) set_col6(d.J, iv + k, act_motion(d.oMi[i], S_col<T>(m, i, k)));
  d.ov[i] = act_motion(d.oMi[i], joint_velocity<T>(m, i, v + iv));
  if (p > 0) d.ov[i] = add6(d.ov[i], d.ov[p]);
  d.oa_gf[i] = zero6<T>();  // oMi.act(c()) with c() = 0
  if (p > 0) d.oa_gf[i] = add6(d.oa_gf[i], cross_motion(d.ov[p], d.ov[i]));
  d.oinertias[i] = d.oYcrb[i] = iner_act(d.oMi[i], inertia_of<T>(m, i));
  d.Yaba[i] = iner_matrix(d.oYcrb[i]);
  d.oh[i] = iner_mul(d.oYcrb[i], d.ov[i]);
  d.of[i] = cross_force(d.ov[i], d.oh[i]);
}

// ---------------------------------------------------------------------------
// ABA, WORLD convention (algorithm/aba.hxx:85-293); abaInParallel uses it
// (algorithm/parallel/aba.hpp:82).
// ---------------------------------------------------------------------------
// with fext: aba.hxx:296-352 (of_i -= oMi.act(fext_i) after the forward step, line 336)
template <class T>
void aba_world(const Model& m, Data<T>& d, const T* q, const T* v, const T* tau, const T* fext = nullptr) {
  for (int k = 0; k < 6; ++k) d.oa_gf[0].v[k] = -T(m.gravity[k]);
  d.of[0] = zero6<T>();
  for (int k = 0; k < m.nv; ++k) d.u[k] = tau[k];
  for (int i = 1; i < m.njoints; ++i) {
    world_forward1(m, d, q, v, i);
    sub_fext_world(fext, i, d.oMi[i], d.of[i]);
  }
  for (int i = m.njoints - 1; i > 0; --i) {
    world_schur(m, d, i);
    if (m.parents[i] > 0) world_schur_update(m, d, i);
  }
  for (int i = 1; i < m.njoints; ++i) {  // AbaWorldConventionForwardStep2 (aba.hxx:196-232)
    const int p = m.parents[i], iv = m.idx_v[i], nvj = m.nvs[i];
    d.oa_gf[i] = add6(d.oa_gf[i], d.oa_gf[p]);
    const std::vector<T>& Dinv = d.Dinvjoint[i];
    const std::vector<T>& UDinv = d.UDinvjoint[i];
    for (int k = 0; k < nvj; ++k) {
      T s = T(0);
      for (int c = 0; c < nvj; ++c) s += Dinv[k * nvj + c] * d.u[iv + c];
      T w = T(0);
      for (int r = 0; r < 6; ++r) w += UDinv[r * nvj + k] * d.oa_gf[i].v[r];
      d.ddq[iv + k] = s - w;
    }
    for (int r = 0; r < 6; ++r) {
      T s = T(0);
      for (int k = 0; k < nvj; ++k) s += d.J[6 * (iv + k) + r] * d.ddq[iv + k];
      d.oa_gf[i].v[r] += s;
    }
  }
}

template <class T>
void aba(const Model& m, Data<T>& d, const T* q, const T* v, const T* tau, int conv, const T* fext = nullptr) {
  if (conv == WORLD) aba_world(m, d, q, v, tau, fext);
  else aba_local(m, d, q, v, tau, fext);
}

// ---------------------------------------------------------------------------
// CRBA (algorithm/crba.hxx): LOCAL 224-339 + 454-491, WORLD 25-110 + 498-548.
// Fills the upper triangle of M (row-major) and adds the armature.
// ---------------------------------------------------------------------------
template <class T>
void crba(const Model& m, Data<T>& d, const T* q, int conv) {
  const int nv = m.nv;
  if (conv == LOCAL) {
    for (int i = 1; i < m.njoints; ++i) {
      d.liMi[i] = se3_mul(placement_of<T>(m, i), joint_transform<T>(m, i, q + m.idx_q[i]));
      d.Ycrb[i] = inertia_of<T>(m, i);
    }
    for (int i = m.njoints - 1; i > 0; --i) {
      const int p = m.parents[i], iv = m.idx_v[i], nvj = m.nvs[i];
      const int nst = m.nvSubtree[i];
      std::vector<T>& Fi = d.Fcrb[i];
      for (int k = 0; k < nvj; ++k) set_col6(Fi, iv + k, iner_mul(d.Ycrb[i], S_col<T>(m, i, k)));
      for (int r = 0; r < nvj; ++r)
        for (int c = iv; c < iv + nst; ++c) d.M[(size_t)(iv + r) * nv + c] = dot6(S_col<T>(m, i, r), col6(Fi, c));
      if (p > 0) {
        iner_add(d.Ycrb[p], iner_act(d.liMi[i], d.Ycrb[i]));
        for (int c = iv; c < iv + nst; ++c) set_col6(d.Fcrb[p], c, act_force(d.liMi[i], col6(Fi, c)));
      }
    }
  } else {
    Iner<T> Y0;
    Y0.m = T(0);
    for (int k = 0; k < 3; ++k) Y0.c[k] = T(0);
    for (int k = 0; k < 6; ++k) Y0.I[k] = T(0);
    d.oYcrb[0] = Y0;
    for (int i = 1; i < m.njoints; ++i) {
      const int p = m.parents[i], iv = m.idx_v[i];
      d.liMi[i] = se3_mul(placement_of<T>(m, i), joint_transform<T>(m, i, q + m.idx_q[i]));
      d.oMi[i] = (p > 0) ? se3_mul(d.oMi[p], d.liMi[i]) : d.liMi[i];
      for (int k = 0; k < m.nvs[i]; ++k) set_col6(d.J, iv + k, act_motion(d.oMi[i], S_col<T>(m, i, k)));
      d.oYcrb[i] = iner_act(d.oMi[i], inertia_of<T>(m, i));
    }
    std::vector<T>& Ag = d.dFda;  // plays the role of data.Ag
    for (int i = m.njoints - 1; i > 0; --i) {
      const int p = m.parents[i], iv = m.idx_v[i], nvj = m.nvs[i], nst = m.nvSubtree[i];
      for (int k = 0; k < nvj; ++k) set_col6(Ag, iv + k, iner_mul(d.oYcrb[i], col6(d.J, iv + k)));
      for (int r = 0; r < nvj; ++r)
        for (int c = iv; c < iv + nst; ++c) d.M[(size_t)(iv + r) * nv + c] = dot6(col6(d.J, iv + r), col6(Ag, c));
      iner_add(d.oYcrb[p], d.oYcrb[i]);
    }
  }
  for (int k = 0; k < nv; ++k) d.M[(size_t)k * nv + k] += T(m.armature[k]);
}

// ---------------------------------------------------------------------------
// Tree-sparse U D U^T factorisation of M (algorithm/cholesky.hxx:18-62).
// Reads the upper triangle of d.M; writes d.U (unit upper, row-major), d.D, d.Dinv.
// ---------------------------------------------------------------------------
template <class T>
void cholesky_decompose(const Model& m, Data<T>& d) {
  const int nv = m.nv;
  auto Mij = [&](int i, int j) { return d.M[(size_t)i * nv + j]; };
  auto Uij = [&](int i, int j) -> T& { return d.U[(size_t)i * nv + j]; };
  for (int j = nv - 1; j >= 0; --j) {
    const int NVT = m.nvSubtree_fromRow[j] - 1;
    for (int k = 0; k < NVT; ++k) d.tmp[k] = Uij(j, j + 1 + k) * d.D[j + 1 + k];
    T s = T(0);
    for (int k = 0; k < NVT; ++k) s += Uij(j, j + 1 + k) * d.tmp[k];
    d.D[j] = Mij(j, j) - s;
    d.Dinv[j] = T(1) / d.D[j];
    for (int ii = m.parents_fromRow[j]; ii >= 0; ii = m.parents_fromRow[ii]) {
      T w = T(0);
      for (int k = 0; k < NVT; ++k) w += Uij(ii, j + 1 + k) * d.tmp[k];
      Uij(ii, j) = (Mij(ii, j) - w) * d.Dinv[j];
    }
  }
}

// ---------------------------------------------------------------------------
// RNEA derivatives (algorithm/rnea-derivatives.hxx:242-541).
// Outputs d.dtau_dq, d.dtau_dv (row-major), d.M (upper triangle + armature), d.tau.
// ---------------------------------------------------------------------------
template <class T>
// with fext: rnea-derivatives.hxx:550-633 (of_i -= oMi.act(fext_i) after the forward step, line 596)
void rnea_derivatives(const Model& m, Data<T>& d, const T* q, const T* v, const T* a, const T* fext = nullptr) {
  const int nv = m.nv;
  if (m.gravity[3] != 0.0 || m.gravity[4] != 0.0 || m.gravity[5] != 0.0)
    throw std::invalid_argument("The gravity must be a pure force vector, no angular part");
  for (int k = 0; k < 6; ++k) d.oa_gf[0].v[k] = -T(m.gravity[k]);
  Vec6<T> g;
  for (int k = 0; k < 6; ++k) g.v[k] = T(m.gravity[k]);
  for (int i = 1; i < m.njoints; ++i) {  // ComputeRNEADerivativesForwardStep (hxx:242-352)
    const int p = m.parents[i], iv = m.idx_v[i], nvj = m.nvs[i];
    const SE3<T> jM = joint_transform<T>(m, i, q + m.idx_q[i]);
    d.liMi[i] = se3_mul(placement_of<T>(m, i), jM);
    const Vec6<T> vJ = joint_velocity<T>(m, i, v + iv);
    d.v[i] = vJ;
    if (p > 0) {
      d.oMi[i] = se3_mul(d.oMi[p], d.liMi[i]);
      d.v[i] = add6(d.v[i], actinv_motion(d.liMi[i], d.v[p]));
    } else {
      d.oMi[i] = d.liMi[i];
    }
    d.a[i] = add6(joint_velocity<T>(m, i, a + iv), cross_motion(d.v[i], vJ));
    if (p > 0) d.a[i] = add6(d.a[i], actinv_motion(d.liMi[i], d.a[p]));
    d.oYcrb[i] = d.oinertias[i] = iner_act(d.oMi[i], inertia_of<T>(m, i));
    d.ov[i] = act_motion(d.oMi[i], d.v[i]);
    d.oa[i] = act_motion(d.oMi[i], d.a[i]);
    for (int k = 0; k < 6; ++k) d.oa_gf[i].v[k] = d.oa[i].v[k] - g.v[k];
    d.oh[i] = iner_mul(d.oYcrb[i], d.ov[i]);
    d.of[i] = add6(iner_mul(d.oYcrb[i], d.oa_gf[i]), cross_force(d.ov[i], d.oh[i]));
    sub_fext_world(fext, i, d.oMi[i], d.of[i]);
    for (int k = 0; k < nvj; ++k) {
      const int c = iv + k;
      const Vec6<T> Jc = act_motion(d.oMi[i], S_col<T>(m, i, k));
      set_col6(d.J, c, Jc);
      const Vec6<T> dJc = cross_motion(d.ov[i], Jc);
      set_col6(d.dJ, c, dJc);
      Vec6<T> dAdq = cross_motion(d.oa_gf[p], Jc);
      Vec6<T> dAdv = dJc;
      if (p > 0) {
        const Vec6<T> dVdq = cross_motion(d.ov[p], Jc);
        set_col6(d.dVdq, c, dVdq);
        dAdq = add6(dAdq, cross_motion(d.ov[p], dVdq));
        dAdv = add6(dAdv, dVdq);
      } else {
        set_col6(d.dVdq, c, zero6<T>());
      }
      set_col6(d.dAdq, c, dAdq);
      set_col6(d.dAdv, c, dAdv);
    }
    d.doYcrb[i] = iner_variation(d.oYcrb[i], d.ov[i]);
    add_force_cross_matrix(d.oh[i], d.doYcrb[i]);
  }
  std::vector<T>& dYtJ = d.Fcrb[0];
  for (int i = m.njoints - 1; i > 0; --i) {  // ComputeRNEADerivativesBackwardStep (hxx:361-460)
    const int p = m.parents[i], iv = m.idx_v[i], nvj = m.nvs[i];
    const int nst = m.nvSubtree[i], ivp = iv + nvj, nstp = nst - nvj;
    for (int k = 0; k < nvj; ++k) d.tau[iv + k] = dot6(col6(d.J, iv + k), d.of[i]);
    for (int k = 0; k < nvj; ++k) set_col6(d.dFda, iv + k, iner_mul(d.oYcrb[i], col6(d.J, iv + k)));
    for (int r = 0; r < nvj; ++r)
      for (int c = iv; c < iv + nst; ++c) d.M[(size_t)(iv + r) * nv + c] = dot6(col6(d.J, iv + r), col6(d.dFda, c));
    for (int k = 0; k < nvj; ++k) {
      const int c = iv + k;
      Vec6<T> dFdq;
      if (p > 0) dFdq = add6(mat6_vec(d.doYcrb[i], col6(d.dVdq, c).v), iner_mul(d.oYcrb[i], col6(d.dAdq, c)));
      else dFdq = iner_mul(d.oYcrb[i], col6(d.dAdq, c));
      set_col6(d.dFdq, c, dFdq);
    }
    for (int k = 0; k < nvj; ++k) {  // dYtJ_cols^T = J_cols^T doYcrb
      const Vec6<T> Jc = col6(d.J, iv + k);
      Vec6<T> row;
      for (int c = 0; c < 6; ++c) {
        T s = Jc.v[0] * d.doYcrb[i].a[c];
        for (int r = 1; r < 6; ++r) s += Jc.v[r] * d.doYcrb[i].a[6 * r + c];
        row.v[c] = s;
      }
      set_col6(dYtJ, iv + k, row);
    }
    for (int r = ivp; r < ivp + nstp; ++r)
      for (int k = 0; k < nvj; ++k) {
        const int c = iv + k;
        d.dtau_dq[(size_t)r * nv + c] = dot6(col6(d.dFda, r), col6(d.dAdq, c)) + dot6(col6(dYtJ, r), col6(d.dVdq, c));
      }
    for (int r = 0; r < nvj; ++r)
      for (int c = iv; c < iv + nst; ++c)
        d.dtau_dq[(size_t)(iv + r) * nv + c] = dot6(col6(d.J, iv + r), col6(d.dFdq, c));
    for (int k = 0; k < nvj; ++k) {
      const int c = iv + k;
      set_col6(d.dFdq, c, add6(col6(d.dFdq, c), cross_force(col6(d.J, c), d.of[i])));
    }
    for (int k = 0; k < nvj; ++k) {
      const int c = iv + k;
      set_col6(d.dFdv, c, add6(mat6_vec(d.doYcrb[i], col6(d.J, c).v), iner_mul(d.oYcrb[i], col6(d.dAdv, c))));
    }
    for (int r = ivp; r < ivp + nstp; ++r)
      for (int k = 0; k < nvj; ++k) {
        const int c = iv + k;
        d.dtau_dv[(size_t)r * nv + c] = dot6(col6(d.dFda, r), col6(d.dAdv, c)) + dot6(col6(dYtJ, r), col6(d.J, c));
      }
    for (int r = 0; r < nvj; ++r)
      for (int c = iv; c < iv + nst; ++c)
        d.dtau_dv[(size_t)(iv + r) * nv + c] = dot6(col6(d.J, iv + r), col6(d.dFdv, c));
    if (p > 0) {
      iner_add(d.oYcrb[p], d.oYcrb[i]);
      for (int k = 0; k < 36; ++k) d.doYcrb[p].a[k] += d.doYcrb[i].a[k];
      d.of[p] = add6(d.of[p], d.of[i]);
    }
  }
  for (int k = 0; k < nv; ++k) {  // restore dAdq (hxx:530-535)
    T w[3];
    cross3(g.v, &d.J[6 * k + 3], w);
    for (int r = 0; r < 3; ++r) d.dAdq[6 * k + r] += w[r];
  }
  for (int k = 0; k < nv; ++k) d.tau[k] += T(m.armature[k]) * a[k];
  for (int k = 0; k < nv; ++k) d.M[(size_t)k * nv + k] += T(m.armature[k]);
}

// ---------------------------------------------------------------------------
// ABA derivatives (algorithm/aba-derivatives.hxx:22-453).
// Outputs d.ddq, d.ddq_dq, d.ddq_dv, d.Minv (full symmetric; row-major).
// ---------------------------------------------------------------------------
// with fext: aba-derivatives.hxx:463-541 (of_i -= oMi.act(fext_i) after forward
// steps 1 and 2, lines 513 and 529)
template <class T>
void aba_derivatives(const Model& m, Data<T>& d, const T* q, const T* v, const T* tau, const T* fext = nullptr) {
  const int nv = m.nv;
  if (m.gravity[3] != 0.0 || m.gravity[4] != 0.0 || m.gravity[5] != 0.0)
    throw std::invalid_argument("The gravity must be a pure force vector, no angular part");
  Vec6<T> g;
  for (int k = 0; k < 6; ++k) g.v[k] = T(m.gravity[k]);
  for (int k = 0; k < 6; ++k) d.oa_gf[0].v[k] = -g.v[k];
  for (int k = 0; k < nv; ++k) d.u[k] = tau[k];
  std::vector<T>& Minv = d.Minv;
  for (int r = 0; r < nv; ++r)
    for (int c = r; c < nv; ++c) Minv[(size_t)r * nv + c] = T(0);
  for (int i = 1; i < m.njoints; ++i) {  // ForwardStep1 (22-80)
    world_forward1(m, d, q, v, i);
    sub_fext_world(fext, i, d.oMi[i], d.of[i]);
  }
  std::vector<T>& Fcrb = d.Fcrb[0];
  std::fill(Fcrb.begin(), Fcrb.end(), T(0));
  for (int i = m.njoints - 1; i > 0; --i) {  // BackwardStep1 (87-171)
    const int p = m.parents[i], iv = m.idx_v[i], nvj = m.nvs[i], nst = m.nvSubtree[i];
    world_schur(m, d, i);
    const std::vector<T>& U = d.Ujoint[i];
    const std::vector<T>& Dinv = d.Dinvjoint[i];
    for (int r = 0; r < nvj; ++r)
      for (int c = 0; c < nvj; ++c) Minv[(size_t)(iv + r) * nv + iv + c] = Dinv[r * nvj + c];
    const int nch = nst - nvj;
    if (nch > 0) {
      for (int k = 0; k < nvj; ++k)  // SDinv_cols = J_cols * Dinv
        for (int r = 0; r < 6; ++r) {
          T s = d.J[6 * iv + r] * Dinv[k];
          for (int j = 1; j < nvj; ++j) s += d.J[6 * (iv + j) + r] * Dinv[j * nvj + k];
          d.SDinv[6 * (iv + k) + r] = s;
        }
      for (int r = 0; r < nvj; ++r)
        for (int c = iv + nvj; c < iv + nst; ++c)
          Minv[(size_t)(iv + r) * nv + c] = -dot6p(&d.SDinv[6 * (iv + r)], &Fcrb[6 * c]);
      if (p > 0)
        for (int c = iv; c < iv + nst; ++c)
          for (int r = 0; r < 6; ++r) {
            T s = U[r * nvj] * Minv[(size_t)iv * nv + c];
            for (int k = 1; k < nvj; ++k) s += U[r * nvj + k] * Minv[(size_t)(iv + k) * nv + c];
            Fcrb[6 * c + r] += s;
          }
    } else {
      for (int c = iv; c < iv + nst; ++c)
        for (int r = 0; r < 6; ++r) {
          T s = U[r * nvj] * Minv[(size_t)iv * nv + c];
          for (int k = 1; k < nvj; ++k) s += U[r * nvj + k] * Minv[(size_t)(iv + k) * nv + c];
          Fcrb[6 * c + r] = s;
        }
    }
    if (p > 0) world_schur_update(m, d, i);
  }
  for (int i = 1; i < m.njoints; ++i) {  // ForwardStep2 (178-270)
    const int p = m.parents[i], iv = m.idx_v[i], nvj = m.nvs[i];
    const std::vector<T>& Dinv = d.Dinvjoint[i];
    const std::vector<T>& UDinv = d.UDinvjoint[i];
    d.oa_gf[i] = add6(d.oa_gf[i], d.oa_gf[p]);
    for (int k = 0; k < nvj; ++k) {
      T s = T(0);
      for (int c = 0; c < nvj; ++c) s += Dinv[k * nvj + c] * d.u[iv + c];
      T w = T(0);
      for (int r = 0; r < 6; ++r) w += UDinv[r * nvj + k] * d.oa_gf[i].v[r];
      d.ddq[iv + k] = s - w;
    }
    for (int r = 0; r < 6; ++r) {
      T s = T(0);
      for (int k = 0; k < nvj; ++k) s += d.J[6 * (iv + k) + r] * d.ddq[iv + k];
      d.oa_gf[i].v[r] += s;
    }
    for (int k = 0; k < 6; ++k) d.oa[i].v[k] = d.oa_gf[i].v[k] + g.v[k];
    d.of[i] = add6(iner_mul(d.oYcrb[i], d.oa_gf[i]), cross_force(d.ov[i], d.oh[i]));
    sub_fext_world(fext, i, d.oMi[i], d.of[i]);
    if (p > 0)
      for (int r = 0; r < nvj; ++r)
        for (int c = iv; c < nv; ++c) {
          T s = UDinv[0 * nvj + r] * d.Fcrb[p][6 * c];
          for (int k = 1; k < 6; ++k) s += UDinv[k * nvj + r] * d.Fcrb[p][6 * c + k];
          Minv[(size_t)(iv + r) * nv + c] -= s;
        }
    for (int c = iv; c < nv; ++c)
      for (int r = 0; r < 6; ++r) {
        T s = d.J[6 * iv + r] * Minv[(size_t)iv * nv + c];
        for (int k = 1; k < nvj; ++k) s += d.J[6 * (iv + k) + r] * Minv[(size_t)(iv + k) * nv + c];
        if (p > 0) s += d.Fcrb[p][6 * c + r];
        d.Fcrb[i][6 * c + r] = s;
      }
    for (int k = 0; k < nvj; ++k) {
      const int c = iv + k;
      const Vec6<T> Jc = col6(d.J, c);
      const Vec6<T> dJc = cross_motion(d.ov[i], Jc);
      set_col6(d.dJ, c, dJc);
      Vec6<T> dAdq = cross_motion(d.oa_gf[p], Jc);
      Vec6<T> dAdv = dJc;
      if (p > 0) {
        const Vec6<T> dVdq = cross_motion(d.ov[p], Jc);
        set_col6(d.dVdq, c, dVdq);
        dAdq = add6(dAdq, cross_motion(d.ov[p], dVdq));
        dAdv = add6(dAdv, dVdq);
      } else {
        set_col6(d.dVdq, c, zero6<T>());
      }
      set_col6(d.dAdq, c, dAdq);
      set_col6(d.dAdv, c, dAdv);
    }
    d.doYcrb[i] = iner_variation(d.oYcrb[i], d.ov[i]);
    add_force_cross_matrix(d.oh[i], d.doYcrb[i]);
  }
  for (int i = m.njoints - 1; i > 0; --i) {  // BackwardStep2 (273-368)
    const int p = m.parents[i], iv = m.idx_v[i], nvj = m.nvs[i], nst = m.nvSubtree[i];
    for (int k = 0; k < nvj; ++k) {
      const int c = iv + k;
      set_col6(d.dFdv, c, add6(iner_mul(d.oYcrb[i], col6(d.dAdv, c)), mat6_vec(d.doYcrb[i], col6(d.J, c).v)));
    }
    for (int r = 0; r < nvj; ++r)
      for (int c = iv; c < iv + nst; ++c)
        d.dtau_dv[(size_t)(iv + r) * nv + c] = dot6(col6(d.J, iv + r), col6(d.dFdv, c));
    for (int k = 0; k < nvj; ++k) {
      const int c = iv + k;
      Vec6<T> dFdq = iner_mul(d.oYcrb[i], col6(d.dAdq, c));
      if (p > 0) dFdq = add6(dFdq, mat6_vec(d.doYcrb[i], col6(d.dVdq, c).v));
      set_col6(d.dFdq, c, dFdq);
    }
    for (int r = 0; r < nvj; ++r)
      for (int c = iv; c < iv + nst; ++c)
        d.dtau_dq[(size_t)(iv + r) * nv + c] = dot6(col6(d.J, iv + r), col6(d.dFdq, c));
    for (int k = 0; k < nvj; ++k) {
      const int c = iv + k;
      set_col6(d.dFdq, c, add6(col6(d.dFdq, c), cross_force(col6(d.J, c), d.of[i])));
    }
    for (int k = 0; k < nvj; ++k) set_col6(d.dFda, iv + k, iner_mul(d.oYcrb[i], col6(d.J, iv + k)));
    if (p > 0) {
      for (int r = 0; r < nvj; ++r)
        for (int j = m.parents_fromRow[iv]; j >= 0; j = m.parents_fromRow[j])
          d.dtau_dq[(size_t)(iv + r) * nv + j] = dot6(col6(d.dFda, iv + r), col6(d.dAdq, j));
      for (int r = 0; r < nvj; ++r)
        for (int j = m.parents_fromRow[iv]; j >= 0; j = m.parents_fromRow[j])
          d.dtau_dv[(size_t)(iv + r) * nv + j] = dot6(col6(d.dFda, iv + r), col6(d.dAdv, j));
      for (int r = 0; r < nvj; ++r) {
        const Vec6<T> Jc = col6(d.J, iv + r);
        T StdY[6];
        for (int c = 0; c < 6; ++c) {
          T s = Jc.v[0] * d.doYcrb[i].a[c];
          for (int k = 1; k < 6; ++k) s += Jc.v[k] * d.doYcrb[i].a[6 * k + c];
          StdY[c] = s;
        }
        for (int j = m.parents_fromRow[iv]; j >= 0; j = m.parents_fromRow[j])
          d.dtau_dq[(size_t)(iv + r) * nv + j] += dot6p(StdY, &d.dVdq[6 * j]);
        for (int j = m.parents_fromRow[iv]; j >= 0; j = m.parents_fromRow[j])
          d.dtau_dv[(size_t)(iv + r) * nv + j] += dot6p(StdY, &d.J[6 * j]);
      }
    }
    if (p > 0) {
      iner_add(d.oYcrb[p], d.oYcrb[i]);
      for (int k = 0; k < 36; ++k) d.doYcrb[p].a[k] += d.doYcrb[i].a[k];
      d.of[p] = add6(d.of[p], d.of[i]);
    }
    for (int k = 0; k < nvj; ++k) {
      T w[3];
      cross3(g.v, &d.J[6 * (iv + k) + 3], w);
      for (int r = 0; r < 3; ++r) d.dAdq[6 * (iv + k) + r] += w[r];
    }
  }
  for (int r = 1; r < nv; ++r)  // symmetrise (hxx:448-449)
    for (int c = 0; c < r; ++c) Minv[(size_t)r * nv + c] = Minv[(size_t)c * nv + r];
  for (int r = 0; r < nv; ++r)  // ddq_dq = -Minv dtau_dq, ddq_dv = -Minv dtau_dv (hxx:451-452)
    for (int c = 0; c < nv; ++c) {
      T s1 = T(0), s2 = T(0);
      for (int k = 0; k < nv; ++k) {
        s1 += Minv[(size_t)r * nv + k] * d.dtau_dq[(size_t)k * nv + c];
        s2 += Minv[(size_t)r * nv + k] * d.dtau_dv[(size_t)k * nv + c];
      }
      d.ddq_dq[(size_t)r * nv + c] = -s1;
      d.ddq_dv[(size_t)r * nv + c] = -s2;
    }
}

// ---------------------------------------------------------------------------
// forwardKinematics (algorithm/kinematics.hxx: ForwardKinematicZeroStep
// 42-77 with q, FirstStep 105-178 with q and v, SecondStep 188-272 with q, v
// and a): liMi, oMi, and the joint-frame spatial velocities / accelerations
// (no gravity: data.a[0] = 0).
// ---------------------------------------------------------------------------
// ---------------------------------------------------------------------------
// Tree-sparse solves with M = U D U^T (algorithm/cholesky.hxx): Uiv (210-235,
// v <- U^-1 v), Utiv (275-296, v <- U^-T v) and solve (483-505, v <- M^-1 v).
// ---------------------------------------------------------------------------
template <class T>
void chol_Uiv(const Model& m, const Data<T>& d, T* v, int stride = 1) {
  const int nv = m.nv;
  for (int k = nv - 2; k >= 0; --k) {
    const int n = m.nvSubtree_fromRow[k] - 1;
    T s = T(0);
    for (int j = 0; j < n; ++j) s += d.U[(size_t)k * nv + k + 1 + j] * v[(size_t)(k + 1 + j) * stride];
    v[(size_t)k * stride] -= s;
  }
}
template <class T>
void chol_Utiv(const Model& m, const Data<T>& d, T* v) {
  const int nv = m.nv;
  for (int k = 0; k < nv - 1; ++k) {
    const int n = m.nvSubtree_fromRow[k] - 1;
    for (int j = 0; j < n; ++j) v[k + 1 + j] -= d.U[(size_t)k * nv + k + 1 + j] * v[k];
  }
}
template <class T>
void chol_solve(const Model& m, const Data<T>& d, T* v) {
  chol_Uiv(m, d, v);
  for (int k = 0; k < m.nv; ++k) v[k] *= d.Dinv[k];
  chol_Utiv(m, d, v);
}

// In-place LLT of an n x n row-major SPD matrix (lower factor L, G = L L^T) and
// the solve G x = b (Eigen LLT, Cholesky-Banachiewicz order; the reference's
// PerformCholeskyCompute / PerformCholeskySolveInPlace, contact-dynamics.hxx:19-80).
template <class T>
void llt_factor_solve(int n, T* G, T* b) {
  for (int j = 0; j < n; ++j) {
    T s = G[(size_t)j * n + j];
    for (int k = 0; k < j; ++k) s -= G[(size_t)j * n + k] * G[(size_t)j * n + k];
    const T ljj = o_sqrt(s);
    G[(size_t)j * n + j] = ljj;
    for (int i = j + 1; i < n; ++i) {
      T t = G[(size_t)i * n + j];
      for (int k = 0; k < j; ++k) t -= G[(size_t)i * n + k] * G[(size_t)j * n + k];
      G[(size_t)i * n + j] = t / ljj;
    }
  }
  for (int i = 0; i < n; ++i) {  // L y = b
    T t = b[i];
    for (int k = 0; k < i; ++k) t -= G[(size_t)i * n + k] * b[k];
    b[i] = t / G[(size_t)i * n + i];
  }
  for (int i = n - 1; i >= 0; --i) {  // L^T x = y
    T t = b[i];
    for (int k = i + 1; k < n; ++k) t -= G[(size_t)k * n + i] * b[k];
    b[i] = t / G[(size_t)i * n + i];
  }
}

// ---------------------------------------------------------------------------
// Contact dynamics with a given constraint Jacobian (algorithm/contact-dynamics.hxx):
// forwardDynamics(q, v, tau, J, gamma, inv_damping) (81-165) and
// impulseDynamics(q, v_before, J, r_coeff, inv_damping) (255-327).  J is nc x nv
// row-major.  Outputs: d.ddq (or the velocity after impact) in `out` and the
// multipliers (lambda_c / impulse_c) in `lam`.
// ---------------------------------------------------------------------------
template <class T>
void contact_common(const Model& m, Data<T>& d, const T* q, int nc, const T* J, T inv_damping,
                    std::vector<T>& G) {
  const int nv = m.nv;
  std::fill(d.M.begin(), d.M.end(), T(0));
  crba(m, d, q, WORLD);
  std::fill(d.U.begin(), d.U.end(), T(0));
  for (int k = 0; k < nv; ++k) d.U[(size_t)k * nv + k] = T(1);
  cholesky_decompose(m, d);
  // sDUiJt = D^-1/2 U^-1 J^T (nv x nc, row-major), JMinvJt = sDUiJt^T sDUiJt + inv_damping I
  std::vector<T> Y((size_t)nv * nc);
  for (int r = 0; r < nv; ++r)
    for (int c = 0; c < nc; ++c) Y[(size_t)r * nc + c] = J[(size_t)c * nv + r];
  for (int c = 0; c < nc; ++c) chol_Uiv(m, d, Y.data() + c, nc);
  for (int r = 0; r < nv; ++r) {
    const T sd = o_sqrt(d.D[r]);
    for (int c = 0; c < nc; ++c) Y[(size_t)r * nc + c] /= sd;
  }
  G.assign((size_t)nc * nc, T(0));
  for (int i = 0; i < nc; ++i)
    for (int j = 0; j < nc; ++j) {
      T s = T(0);
      for (int r = 0; r < nv; ++r) s += Y[(size_t)r * nc + i] * Y[(size_t)r * nc + j];
      G[(size_t)i * nc + j] = s + (i == j ? inv_damping : T(0));
    }
}
// computeKKTContactDynamicMatrixInverse(q, J, inv_damping) (contact-dynamics.hxx:166-225):
// the inverse of [[M, J^T], [J, -inv_damping I]], n = nv + nc, row-major in `K`, from the
// factorisations: bottomRight = -(J M^-1 J^T + mu I)^-1, topLeft = M^-1, bottomLeft = J M^-1,
// topRight = bottomLeft^T (-bottomRight), topLeft -= topRight bottomLeft, bottomLeft = topRight^T.
template <class T>
void kkt_inverse_contact(const Model& m, Data<T>& d, const T* q, int nc, const T* J, T inv_damping, T* K) {
  const int nv = m.nv, n = nv + nc;
  std::vector<T> G;
  contact_common(m, d, q, nc, J, inv_damping, G);
  auto at = [&](int r, int c) -> T& { return K[(size_t)r * n + c]; };
  std::vector<T> col(nv);
  for (int c = 0; c < nv; ++c) {  // topLeft = M^-1
    for (int k = 0; k < nv; ++k) col[k] = T(k == c);
    chol_solve(m, d, col.data());
    for (int k = 0; k < nv; ++k) at(k, c) = col[k];
  }
  std::vector<T> BR((size_t)nc * nc), BL((size_t)nc * nv), TR((size_t)nv * nc);
  for (int j = 0; j < nc; ++j) {  // bottomRight = -G^-1, column by column
    std::vector<T> Gc(G), e(nc, T(0));
    e[j] = T(-1);
    llt_factor_solve(nc, Gc.data(), e.data());
    for (int i = 0; i < nc; ++i) BR[(size_t)i * nc + j] = e[i];
  }
  for (int i = 0; i < nc; ++i)  // bottomLeft = J topLeft
    for (int c = 0; c < nv; ++c) {
      T s = T(0);
      for (int k = 0; k < nv; ++k) s += J[(size_t)i * nv + k] * at(k, c);
      BL[(size_t)i * nv + c] = s;
    }
  for (int r = 0; r < nv; ++r)  // topRight = bottomLeft^T (-bottomRight)
    for (int j = 0; j < nc; ++j) {
      T s = T(0);
      for (int i = 0; i < nc; ++i) s += BL[(size_t)i * nv + r] * -BR[(size_t)i * nc + j];
      TR[(size_t)r * nc + j] = s;
    }
  for (int r = 0; r < nv; ++r)  // topLeft -= topRight bottomLeft
    for (int c = 0; c < nv; ++c) {
      T s = T(0);
      for (int j = 0; j < nc; ++j) s += TR[(size_t)r * nc + j] * BL[(size_t)j * nv + c];
      at(r, c) -= s;
    }
  for (int r = 0; r < nv; ++r)
    for (int j = 0; j < nc; ++j) {
      at(r, nv + j) = TR[(size_t)r * nc + j];
      at(nv + j, r) = TR[(size_t)r * nc + j];
    }
  for (int i = 0; i < nc; ++i)
    for (int j = 0; j < nc; ++j) at(nv + i, nv + j) = BR[(size_t)i * nc + j];
}

template <class T>
void forward_dynamics_contact(const Model& m, Data<T>& d, const T* q, const T* v, const T* tau, int nc, const T* J,
                              const T* gamma, T inv_damping, T* out, T* lam) {
  const int nv = m.nv;
  std::vector<T> G;
  contact_common(m, d, q, nc, J, inv_damping, G);
  std::vector<T> zero(nv, T(0)), r(nv);
  rnea(m, d, q, v, zero.data());  // nle = C(q, v) v + g (computeAllTerms)
  for (int k = 0; k < nv; ++k) r[k] = tau[k] - d.tau[k];
  chol_solve(m, d, r.data());  // torque_residual = M^-1 (tau - nle)
  for (int c = 0; c < nc; ++c) {  // lambda = -J torque_residual - gamma
    T s = T(0);
    for (int k = 0; k < nv; ++k) s += J[(size_t)c * nv + k] * r[k];
    lam[c] = -s - gamma[c];
  }
  llt_factor_solve(nc, G.data(), lam);
  for (int k = 0; k < nv; ++k) {  // a = M^-1 J^T lambda + torque_residual
    T s = T(0);
    for (int c = 0; c < nc; ++c) s += J[(size_t)c * nv + k] * lam[c];
    out[k] = s;
  }
  chol_solve(m, d, out);
  for (int k = 0; k < nv; ++k) out[k] += r[k];
}
template <class T>
void impulse_dynamics_contact(const Model& m, Data<T>& d, const T* q, const T* v_before, int nc, const T* J,
                              T r_coeff, T inv_damping, T* out, T* lam) {
  const int nv = m.nv;
  std::vector<T> G;
  contact_common(m, d, q, nc, J, inv_damping, G);
  for (int c = 0; c < nc; ++c) {  // impulse = -(1 + r_coeff) J v_before
    T s = T(0);
    for (int k = 0; k < nv; ++k) s += J[(size_t)c * nv + k] * v_before[k];
    lam[c] = (-r_coeff - T(1)) * s;
  }
  llt_factor_solve(nc, G.data(), lam);
  for (int k = 0; k < nv; ++k) {
    T s = T(0);
    for (int c = 0; c < nc; ++c) s += J[(size_t)c * nv + k] * lam[c];
    out[k] = s;
  }
  chol_solve(m, d, out);
  for (int k = 0; k < nv; ++k) out[k] += v_before[k];
}

template <class T>
void forward_kinematics(const Model& m, Data<T>& d, const T* q, const T* v, const T* a) {
  d.v[0] = zero6<T>();
  d.a[0] = zero6<T>();
  for (int i = 1; i < m.njoints; ++i) {
    const int p = m.parents[i], iq = m.idx_q[i], iv = m.idx_v[i];
    d.liMi[i] = se3_mul(placement_of<T>(m, i), joint_transform<T>(m, i, q + iq));
    d.oMi[i] = p > 0 ? se3_mul(d.oMi[p], d.liMi[i]) : d.liMi[i];
    if (!v) continue;
    const Vec6<T> vJ = joint_velocity<T>(m, i, v + iv);
    d.v[i] = vJ;
    if (p > 0) d.v[i] = add6(d.v[i], actinv_motion(d.liMi[i], d.v[p]));
    if (!a) continue;
    // S a + c + v_i x vJ (c = 0 for these joints), then + liMi.actInv(a_parent)
    d.a[i] = add6(joint_velocity<T>(m, i, a + iv), cross_motion(d.v[i], vJ));
    d.a[i] = add6(d.a[i], actinv_motion(d.liMi[i], d.a[p]));
  }
}

// ---------------------------------------------------------------------------
// computeJointJacobians (algorithm/jacobian.hxx:17-95): oMi and
// J = [oMi.act(S_i)] columns, 6 x nv column-major, about the world origin.
// ---------------------------------------------------------------------------
template <class T>
void joint_jacobians(const Model& m, Data<T>& d, const T* q) {
  for (int i = 1; i < m.njoints; ++i) {
    const int p = m.parents[i], iq = m.idx_q[i], iv = m.idx_v[i];
    d.liMi[i] = se3_mul(placement_of<T>(m, i), joint_transform<T>(m, i, q + iq));
    d.oMi[i] = p > 0 ? se3_mul(d.oMi[p], d.liMi[i]) : d.liMi[i];
    for (int k = 0; k < m.nvs[i]; ++k) set_col6(d.J, iv + k, act_motion(d.oMi[i], S_col<T>(m, i, k)));
  }
}

// ---------------------------------------------------------------------------
// integrate(q, v) for the supported joints: free-flyer through the SE(3)
// exponential (multibody/liegroup/special-euclidean.hpp:660-699,
// spatial/explog-quaternion.hpp:20-147, math/quaternion.hpp:90-111); revolute
// and prismatic joints are a vector space (q + v).
// ---------------------------------------------------------------------------
// exp3 of an angular velocity as a quaternion (x, y, z, w) (spatial/explog-quaternion.hpp:20-60)
template <class T> void exp3_quat(const T* w, T* e) {
  const T eps = o_eps<T>();
  const T ts_prec = T(std::pow((double)eps, 1.0 / 4.0));
  const T s2 = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
  const T th = o_sqrt(s2 + eps * eps);
  if (s2 > ts_prec) {  // AngleAxis(th, w/th) -> quaternion
    T sh, ch;
    o_sincos(T(0.5) * th, &sh, &ch);
    for (int k = 0; k < 3; ++k) e[k] = sh * (w[k] / th);
    e[3] = ch;
  } else {
    const T t2_2 = s2 / T(4);
    const T c = T(0.5) * (T(1) - t2_2 / T(6) + t2_2 * t2_2 / T(120));
    for (int k = 0; k < 3; ++k) e[k] = c * w[k];
    e[3] = T(1) - t2_2 / T(2) + t2_2 * t2_2 / T(24);
  }
}
// SO(3): quat * exp3(v), first-order normalised (liegroup/special-orthogonal.hpp:467-481,
// math/quaternion.hpp:90-111)
template <class T> void integrate_so3(const T* qq, const T* w, T* out) {
  T e[4];
  exp3_quat(w, e);
  T r[4];
  r[3] = qq[3] * e[3] - qq[0] * e[0] - qq[1] * e[1] - qq[2] * e[2];
  r[0] = qq[3] * e[0] + qq[0] * e[3] + qq[1] * e[2] - qq[2] * e[1];
  r[1] = qq[3] * e[1] + qq[1] * e[3] + qq[2] * e[0] - qq[0] * e[2];
  r[2] = qq[3] * e[2] + qq[2] * e[3] + qq[0] * e[1] - qq[1] * e[0];
  const T N2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2] + r[3] * r[3];
  const T alpha = (T(3) - N2) / T(2);
  for (int k = 0; k < 4; ++k) out[k] = r[k] * alpha;
}
// SE(2) on (x, y, cos, sin): exp of (vx, vy, w) in the body frame composed on the right
// (liegroup/special-euclidean.hpp:61-90, 289-306)
template <class T> void integrate_se2(const T* q, const T* v, T* out) {
  const T c0 = q[2], s0 = q[3];
  T sv, cv;
  o_sincos(v[2], &sv, &cv);
  T t[2];
  const T vc0 = -v[1] - (-v[1] * cv + v[0] * (-sv)), vc1 = v[0] - (-v[1] * sv + v[0] * cv);
  const T aw = v[2] < T(0) ? -v[2] : v[2];
  if (aw > T(1e-14)) { t[0] = vc0 / v[2]; t[1] = vc1 / v[2]; }
  else { t[0] = v[0]; t[1] = v[1]; }
  out[0] = c0 * t[0] - s0 * t[1] + q[0];
  out[1] = s0 * t[0] + c0 * t[1] + q[1];
  out[2] = c0 * cv - s0 * sv;
  out[3] = s0 * cv + c0 * sv;
}

// SpecialOrthogonalOperationTpl<2>::integrate (liegroup/special-orthogonal.hpp:164-185): the unit
// complex (cos, sin) turned by v, then its first-order renormalisation (3 - |z|^2) / 2
template <class T> inline void integrate_so2(const T* q, const T* v, T* out) {
  T sw, cw;
  o_sincos(v[0], &sw, &cw);
  out[0] = cw * q[0] - sw * q[1];
  out[1] = sw * q[0] + cw * q[1];
  const T n2 = out[0] * out[0] + out[1] * out[1];
  const T f = (T(3) - n2) / T(2);
  out[0] *= f;
  out[1] *= f;
}

template <class T>
void integrate(const Model& m, const T* q, const T* v, T* qout) {
  for (int i = 1; i < m.njoints; ++i) {
    const int iq = m.idx_q[i], iv = m.idx_v[i], jt = m.jtype[i];
    if (jt == JT_TR) {
      for (int k = 0; k < 3; ++k) qout[iq + k] = q[iq + k] + v[iv + k];
      continue;
    }
    if (jt == JT_SPH) {
      integrate_so3(q + iq, v + iv, qout + iq);
      continue;
    }
    if (jt == JT_PL) {
      integrate_se2(q + iq, v + iv, qout + iq);
      continue;
    }
    if (unbounded(jt)) {
      integrate_so2(q + iq, v + iv, qout + iq);
      continue;
    }
    if (jt != JT_FF) {
      qout[iq] = q[iq] + v[iv];
      continue;
    }
    const T* w = v + iv + 3;
    const T* lv = v + iv;
    const T eps = o_eps<T>();
    // exp6 translation part
    const T t2 = w[0] * w[0] + w[1] * w[1] + w[2] * w[2] + eps * eps;
    const T t = o_sqrt(t2);
    T st, ct;
    o_sincos(t, &st, &ct);
    const T inv_t2 = T(1) / t2;
    const T ts_prec = T(std::pow((double)eps, 1.0 / 4.0));
    T alpha_wxv, alpha_w2;
    if (t < ts_prec) {
      alpha_wxv = T(0.5) - t2 / T(24);
      alpha_w2 = T(1) / T(6) - t2 / T(120);
    } else {
      alpha_wxv = (T(1) - ct) * inv_t2;
      alpha_w2 = (t - st) * inv_t2 / t;
    }
    T wxv[3], wxwxv[3], trans[3];
    cross3(w, lv, wxv);
    cross3(w, wxv, wxwxv);
    for (int k = 0; k < 3; ++k) trans[k] = lv[k] + alpha_wxv * wxv[k] + alpha_w2 * wxwxv[k];
    // exp3 quaternion part
    const T s2 = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
    const T th = o_sqrt(s2 + eps * eps);
    T e[4];  // x, y, z, w
    if (s2 > ts_prec) {  // AngleAxis(th, w/th) -> quaternion
      T sh, ch;
      o_sincos(T(0.5) * th, &sh, &ch);
      for (int k = 0; k < 3; ++k) e[k] = sh * (w[k] / th);
      e[3] = ch;
    } else {
      const T t2_2 = s2 / T(4);
      const T c = T(0.5) * (T(1) - t2_2 / T(6) + t2_2 * t2_2 / T(120));
      for (int k = 0; k < 3; ++k) e[k] = c * w[k];
      e[3] = T(1) - t2_2 / T(2) + t2_2 * t2_2 / T(24);
    }
    const T* qq = q + iq + 3;  // x, y, z, w
    // quat * trans (Eigen _transformVector: uv = 2 (u x v); v + w uv + u x uv)
    T uv[3], uxuv[3];
    cross3(qq, trans, uv);
    for (int k = 0; k < 3; ++k) uv[k] += uv[k];
    cross3(qq, uv, uxuv);
    for (int k = 0; k < 3; ++k) qout[iq + k] = trans[k] + qq[3] * uv[k] + uxuv[k] + q[iq + k];
    // res = quat * quat1 (Hamilton product)
    T r[4];
    r[3] = qq[3] * e[3] - qq[0] * e[0] - qq[1] * e[1] - qq[2] * e[2];
    r[0] = qq[3] * e[0] + qq[0] * e[3] + qq[1] * e[2] - qq[2] * e[1];
    r[1] = qq[3] * e[1] + qq[1] * e[3] + qq[2] * e[0] - qq[0] * e[2];
    r[2] = qq[3] * e[2] + qq[2] * e[3] + qq[0] * e[1] - qq[1] * e[0];
    const T dp = r[0] * qq[0] + r[1] * qq[1] + r[2] * qq[2] + r[3] * qq[3];
    if (dp < T(0))
      for (int k = 0; k < 4; ++k) r[k] = -r[k];
    const T N2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2] + r[3] * r[3];
    const T alpha = (T(3) - N2) / T(2);
    for (int k = 0; k < 4; ++k) qout[iq + 3 + k] = r[k] * alpha;
  }
}

// ---------------------------------------------------------------------------
// constraintDynamics with rigid constraint models and the proximal iterations
// (algorithm/constrained-dynamics.hxx:188-520): the world-frame forward /
// backward sweeps (ContactAndImpulseDynamicsForwardStep / BackwardStep,
// constrained-dynamics.hxx:63-186), the contact Cholesky factorisation of the
// KKT matrix [[-mu I, J], [J^T, M]] (contact-cholesky.hxx:21-330), the contact
// drifts and Baumgarte corrections, and the proximal loop.
// ---------------------------------------------------------------------------
enum ContactType { CONTACT_3D = 0, CONTACT_6D = 1 };                  // contact-info.hpp:19-24
enum ReferenceFrame { RF_WORLD = 0, RF_LOCAL = 1, RF_LOCAL_WORLD_ALIGNED = 2 };  // multibody/fwd.hpp:46-56

// RigidConstraintModel (contact-info.hpp:140-230): placements R row-major + t; the
// desired acceleration and the corrector gains are [linear; angular].
struct ConstraintModel {
  int type = CONTACT_6D, frame = RF_LOCAL, joint1 = 0, joint2 = 0;
  double P1[12] = {1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0}, P2[12] = {1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0};
  double desired_acc[6] = {0, 0, 0, 0, 0, 0}, Kp[6] = {0, 0, 0, 0, 0, 0}, Kd[6] = {0, 0, 0, 0, 0, 0};
  std::vector<int> s1, s2;  // colwise_joint1_sparsity / colwise_joint2_sparsity
  int size() const { return type == CONTACT_3D ? 3 : 6; }
  // RigidConstraintModel::init (contact-info.hpp:712-790): the columns of the joints from
  // joint1 / joint2 up to (excluding) their common ancestor; for CONTACT_3D also the
  // common ancestor's support, in both sets
  void init(const Model& m) {
    if (frame != RF_LOCAL && frame != RF_LOCAL_WORLD_ALIGNED)
      throw std::invalid_argument("reference_frame should be LOCAL or LOCAL_WORLD_ALIGNED");
    if (type != CONTACT_3D && type != CONTACT_6D) throw std::invalid_argument("unknown contact type");
    if (joint1 < 0 || joint1 >= m.njoints || joint2 < 0 || joint2 >= m.njoints)
      throw std::invalid_argument("constraint joint index out of range");
    s1.assign(m.nv, 0);
    s2.assign(m.nv, 0);
    int c1 = joint1, c2 = joint2;
    while (c1 != c2) {
      if (c1 > c2) {
        for (int k = 0; k < m.nvs[c1]; ++k) s1[m.idx_v[c1] + k] = 1;
        c1 = m.parents[c1];
      } else {
        for (int k = 0; k < m.nvs[c2]; ++k) s2[m.idx_v[c2] + k] = 1;
        c2 = m.parents[c2];
      }
    }
    if (type == CONTACT_3D)
      for (int c = c1; c > 0; c = m.parents[c])
        for (int k = 0; k < m.nvs[c]; ++k) s1[m.idx_v[c] + k] = s2[m.idx_v[c] + k] = 1;
  }
};

inline double o_atan2(double y, double x) { return std::atan2(y, x); }
inline long double o_atan2(long double y, long double x) { return std::atan2(y, x); }

template <class T> inline SE3<T> se3_from(const double* P) {
  SE3<T> M;
  for (int k = 0; k < 9; ++k) M.R[k] = T(P[k]);
  for (int k = 0; k < 3; ++k) M.t[k] = T(P[9 + k]);
  return M;
}
template <class T> inline SE3<T> se3_actinv(const SE3<T>& A, const SE3<T>& B) {  // A^-1 B
  SE3<T> o;
  T d[3];
  for (int k = 0; k < 3; ++k) d[k] = B.t[k] - A.t[k];
  matTvec(A.R, d, o.t);
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) o.R[3 * r + c] = A.R[r] * B.R[c] + A.R[3 + r] * B.R[3 + c] + A.R[6 + r] * B.R[6 + c];
  return o;
}

// log3 of a rotation (the angle-axis vector, angle in [0, pi]; reference spatial/log.hxx:58-170):
// theta = atan2(|a|, (tr - 1) / 2) with a = unskew(R) = sin(theta) n; w = theta / sin(theta) a away
// from pi (series of theta / sin(theta) near 0), and near pi the axis from the symmetric part
// (R + R^T) / 2 - cos(theta) I = (1 - cos(theta)) n n^T, its sign taken from a.
template <class T> inline void log3(const T* R, T* w, T& theta) {
  const T a[3] = {(R[7] - R[5]) / T(2), (R[2] - R[6]) / T(2), (R[3] - R[1]) / T(2)};
  const T s = o_sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
  T c = (R[0] + R[4] + R[8] - T(1)) / T(2);
  c = c > T(1) ? T(1) : c < T(-1) ? T(-1) : c;
  theta = o_atan2(s, c);
  if (theta < T(3)) {
    const T t2 = theta * theta;
    const T k = s < T(1e-4) ? T(1) + t2 / T(6) + T(7) * t2 * t2 / T(360) : theta / s;
    for (int i = 0; i < 3; ++i) w[i] = k * a[i];
    return;
  }
  const T omc = T(1) - c;
  int j = 0;
  for (int i = 1; i < 3; ++i)
    if (R[4 * i] > R[4 * j]) j = i;
  T n[3];
  n[j] = o_sqrt((R[4 * j] - c) / omc);
  for (int i = 0; i < 3; ++i)
    if (i != j) n[i] = (R[3 * i + j] + R[3 * j + i]) / (T(2) * omc * n[j]);
  const T dp = n[0] * a[0] + n[1] * a[1] + n[2] * a[2];
  const T sg = dp < T(0) ? T(-1) : T(1);
  for (int i = 0; i < 3; ++i) w[i] = sg * theta * n[i];
}
// log6 of a placement (spatial/log.hxx:189-230): angular = log3(R); linear = alpha p - w x p / 2 +
// beta (w . p) w, alpha = theta sin / (2 (1 - cos)), beta = 1 / theta^2 - sin / (2 theta (1 - cos)),
// their series in |unskew(R)|^2 when tr(R) >= 3 - eps^(1/3)
template <class T> inline Vec6<T> log6(const SE3<T>& M) {
  T w[3], theta;
  log3(M.R, w, theta);
  const T a[3] = {(M.R[7] - M.R[5]) / T(2), (M.R[2] - M.R[6]) / T(2), (M.R[3] - M.R[1]) / T(2)};
  const T t2 = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
  const T tr = M.R[0] + M.R[4] + M.R[8];
  T alpha, beta;
  if (tr >= T(3) - T(std::cbrt(std::numeric_limits<double>::epsilon()))) {
    alpha = T(1) - t2 / T(12) - t2 * t2 / T(720);
    beta = T(1) / T(12) + t2 / T(720);
  } else {
    T st, ct;
    o_sincos(theta, &st, &ct);
    alpha = theta * st / (T(2) * (T(1) - ct));
    beta = T(1) / (theta * theta) - st / (T(2) * theta * (T(1) - ct));
  }
  T wxp[3];
  cross3(w, M.t, wxp);
  const T wp = w[0] * M.t[0] + w[1] * M.t[1] + w[2] * M.t[2];
  Vec6<T> o;
  for (int k = 0; k < 3; ++k) {
    o.v[k] = alpha * M.t[k] - T(0.5) * wxp[k] + beta * wp * w[k];
    o.v[3 + k] = w[k];
  }
  return o;
}

// Jlog6 (spatial/explog.hpp, Jlog6): d log6(M exp6(d)) / dd at d = 0, the inverse of SE(3)'s right
// Jacobian at xi = log6(M) = (rho, phi) ([linear; angular]), written from the published closed form
// (Barfoot, State Estimation for Robotics, 7.1.5; the right Jacobian is the left one at -xi):
//   [[Jr^-1(phi), -Jr^-1(phi) Qr Jr^-1(phi)], [0, Jr^-1(phi)]], row-major 6 x 6,
//   Jr^-1(phi) = I + phi^ / 2 + c phi^ phi^, c = 1 / t^2 - (1 + cos t) / (2 t sin t),
//   Qr = -rho^ / 2 + a1 (phi^ rho^ + rho^ phi^ - phi^ rho^ phi^) - a2 (phi^ phi^ rho^ + rho^ phi^ phi^
//        - 3 phi^ rho^ phi^) + a3 (phi^ rho^ phi^ phi^ + phi^ phi^ rho^ phi^),
//   a1 = (t - sin t) / t^3, a2 = (t^2 + 2 cos t - 2) / (2 t^4), a3 = (2 t - 3 sin t + t cos t) / (2 t^5),
// with their Taylor series for small t.
template <class T> inline void jlog6(const SE3<T>& M, T* J) {
  const Vec6<T> xi = log6(M);
  const T* rho = xi.v;
  const T* phi = xi.v + 3;
  const T t2 = phi[0] * phi[0] + phi[1] * phi[1] + phi[2] * phi[2], t = o_sqrt(t2);
  T c, a1, a2, a3;
  if (t < T(1e-3)) {
    c = T(1) / T(12) + t2 / T(720);
    a1 = T(1) / T(6) - t2 / T(120);
    a2 = T(1) / T(24) - t2 / T(720);
    a3 = T(1) / T(120) - t2 / T(2520);
  } else {
    T st, ct;
    o_sincos(t, &st, &ct);
    c = T(1) / t2 - (T(1) + ct) / (T(2) * t * st);
    a1 = (t - st) / (t2 * t);
    a2 = (t2 + T(2) * ct - T(2)) / (T(2) * t2 * t2);
    a3 = (T(2) * t - T(3) * st + t * ct) / (T(2) * t2 * t2 * t);
  }
  auto skew = [](const T* v, T* S) {
    S[0] = T(0); S[1] = -v[2]; S[2] = v[1];
    S[3] = v[2]; S[4] = T(0); S[5] = -v[0];
    S[6] = -v[1]; S[7] = v[0]; S[8] = T(0);
  };
  auto mul = [](const T* A, const T* B, T* C) {
    for (int r = 0; r < 3; ++r)
      for (int q = 0; q < 3; ++q) C[3 * r + q] = A[3 * r] * B[q] + A[3 * r + 1] * B[3 + q] + A[3 * r + 2] * B[6 + q];
  };
  T P[9], R[9], PP[9], PR[9], RP[9], PRP[9], PPR[9], RPP[9], PRPP[9], PPRP[9], Jr[9], Q[9], tmp[9], B[9];
  skew(phi, P);
  skew(rho, R);
  mul(P, P, PP);
  mul(P, R, PR);
  mul(R, P, RP);
  mul(PR, P, PRP);
  mul(PP, R, PPR);
  mul(RP, P, RPP);
  mul(PRP, P, PRPP);
  mul(PPR, P, PPRP);
  for (int k = 0; k < 9; ++k) {
    Jr[k] = (k % 4 == 0 ? T(1) : T(0)) + T(0.5) * P[k] + c * PP[k];
    Q[k] = -T(0.5) * R[k] + a1 * (PR[k] + RP[k] - PRP[k]) - a2 * (PPR[k] + RPP[k] - T(3) * PRP[k]) +
           a3 * (PRPP[k] + PPRP[k]);
  }
  mul(Jr, Q, tmp);
  mul(tmp, Jr, B);
  for (int r = 0; r < 3; ++r)
    for (int q = 0; q < 3; ++q) {
      J[6 * r + q] = Jr[3 * r + q];
      J[6 * r + 3 + q] = -B[3 * r + q];
      J[6 * (3 + r) + q] = T(0);
      J[6 * (3 + r) + 3 + q] = Jr[3 * r + q];
    }
}

// The contact Cholesky factorisation U D U^T of the KKT matrix (contact-cholesky.hxx:21-330):
// rows / columns 0..nc-1 the constraints, nc..nc+nv-1 the dofs; U unit upper, row-major.
template <class T> struct ContactCholesky {
  int nc = 0, nv = 0, n = 0;
  std::vector<int> pfr, nsfr;  // parents_fromRow / nv_subtree_fromRow shifted by nc
  std::vector<T> U, D, Dinv;
  void allocate(const Model& m, const std::vector<ConstraintModel>& cms) {  // allocate, hxx:21-150
    nv = m.nv;
    nc = 0;
    for (const auto& c : cms) nc += c.size();
    n = nc + nv;
    pfr.assign(n, -1);
    nsfr.assign(n, 0);
    for (int j = 1; j < m.njoints; ++j) {
      const int p = m.parents[j], iv = m.idx_v[j];
      pfr[nc + iv] = p > 0 ? m.idx_v[p] + m.nvs[p] - 1 + nc : -1;
      nsfr[nc + iv] = m.nvSubtree[j];
      for (int r = 1; r < m.nvs[j]; ++r) {
        pfr[nc + iv + r] = nc + iv + r - 1;
        nsfr[nc + iv + r] = m.nvSubtree[j] - r;
      }
    }
    int row = 0;
    for (const auto& c : cms) {
      const int e = std::max(m.idx_v[c.joint1] + m.nvs[c.joint1], m.idx_v[c.joint2] + m.nvs[c.joint2]);
      for (int k = 0; k < c.size(); ++k, ++row) nsfr[row] = e + (nc - row);
    }
    U.assign((size_t)n * n, T(0));
    for (int k = 0; k < n; ++k) U[(size_t)k * n + k] = T(1);
    D.assign(n, T(0));
    Dinv.assign(n, T(0));
  }
  T& u(int r, int c) { return U[(size_t)r * n + c]; }
  // compute (hxx:152-272) after the Jacobian rows are in U's top-right block and M in
  // D.tail / U's bottom-right block; then updateDamping(mu) (hxx:274-304)
  void factor(T mu) {
    std::vector<T> DUt(n);
    for (int j = nv - 1; j >= 0; --j) {
      const int jj = nc + j, NVT = nsfr[jj] - 1;
      for (int k = 0; k < NVT; ++k) DUt[k] = u(jj, jj + 1 + k) * D[jj + 1 + k];
      T s = T(0);
      for (int k = 0; k < NVT; ++k) s += u(jj, jj + 1 + k) * DUt[k];
      D[jj] -= s;
      Dinv[jj] = T(1) / D[jj];
      for (int ii = pfr[jj]; ii >= nc; ii = pfr[ii]) {
        T t = T(0);
        for (int k = 0; k < NVT; ++k) t += u(ii, jj + 1 + k) * DUt[k];
        u(ii, jj) = (u(ii, jj) - t) * Dinv[jj];
      }
      for (int r = nc - 1; r >= 0; --r) {
        T t = T(0);
        for (int k = 0; k < NVT; ++k) t += u(r, jj + 1 + k) * DUt[k];
        u(r, jj) = (u(r, jj) - t) * Dinv[jj];
      }
    }
    for (int j = nc - 1; j >= 0; --j) {
      const int sd = n - j - 1;
      for (int k = 0; k < sd; ++k) DUt[k] = u(j, j + 1 + k) * D[j + 1 + k];
      T s = T(0);
      for (int k = 0; k < sd; ++k) s += u(j, j + 1 + k) * DUt[k];
      D[j] = -mu - s;
      Dinv[j] = T(1) / D[j];
      for (int i = j - 1; i >= 0; --i) {
        T t = T(0);
        for (int k = 0; k < sd; ++k) t += u(i, j + 1 + k) * DUt[k];
        u(i, j) = -t * Dinv[j];
      }
    }
  }
  // solveInPlace (hxx:306-316): Uiv (hxx:512-538), Dinv, Utiv (hxx:570-595)
  void solve(T* x) {
    for (int k = n - 2; k >= nc; --k) {
      T s = T(0);
      for (int j = 1; j < nsfr[k]; ++j) s += u(k, k + j) * x[k + j];
      x[k] -= s;
    }
    for (int k = nc - 1; k >= 0; --k) {
      T s = T(0);
      for (int j = k + 1; j < n; ++j) s += u(k, j) * x[j];
      x[k] -= s;
    }
    for (int k = 0; k < n; ++k) x[k] *= Dinv[k];
    for (int k = 0; k < nc; ++k)
      for (int j = k + 1; j < n; ++j) x[j] -= u(k, j) * x[k];
    for (int k = nc; k <= n - 2; ++k)
      for (int j = 1; j < nsfr[k]; ++j) x[k + j] -= u(k, k + j) * x[k];
  }
  // DelassusCholeskyExpression::applyOnTheRight (contact-cholesky.hpp:536-558):
  // res = U1 (-D1) U1^T x over the constraint block
  void delassus_apply(const T* x, T* res) {
    std::vector<T> t(nc);
    for (int i = 0; i < nc; ++i) {
      T s = x[i];
      for (int k = 0; k < i; ++k) s += u(k, i) * x[k];
      t[i] = -D[i] * s;
    }
    for (int i = 0; i < nc; ++i) {
      T s = t[i];
      for (int k = i + 1; k < nc; ++k) s += u(i, k) * t[k];
      res[i] = s;
    }
  }
};

// The constraint Jacobian rows of one model (RigidConstraintModel::jacobian, contact-info.hpp:551-672)
// from the world-frame columns d.J, written into the KKT factor's top-right block
template <class T>
void constraint_jacobian(const Model& m, const Data<T>& d, const ConstraintModel& c, const SE3<T>& oMc1,
                         const SE3<T>& oMc2, const SE3<T>& c1Mc2, int row, ContactCholesky<T>& ch) {
  for (int jj = 0; jj < m.nv; ++jj) {
    if (!c.s1[jj] && !c.s2[jj]) continue;
    const int sign = c.s1[jj] != c.s2[jj] ? (c.s1[jj] ? 1 : -1) : 0;
    const Vec6<T> Jc = col6(d.J, jj);
    T col[6];
    if (c.type == CONTACT_3D) {
      if (c.frame == RF_LOCAL) {
        if (sign == 0) {
          const Vec6<T> l1 = actinv_motion(oMc1, Jc), l2 = actinv_motion(oMc2, Jc);
          T r2[3];
          matvec(c1Mc2.R, l2.v, r2);
          for (int k = 0; k < 3; ++k) col[k] = l1.v[k] - r2[k];
        } else if (sign == 1) {
          const Vec6<T> l1 = actinv_motion(oMc1, Jc);
          for (int k = 0; k < 3; ++k) col[k] = l1.v[k];
        } else {
          const Vec6<T> l2 = actinv_motion(oMc2, Jc);
          T r2[3];
          matvec(c1Mc2.R, l2.v, r2);
          for (int k = 0; k < 3; ++k) col[k] = -r2[k];
        }
      } else {
        if (sign == 0) {
          T dpos[3];
          for (int k = 0; k < 3; ++k) dpos[k] = oMc2.t[k] - oMc1.t[k];
          cross3(dpos, Jc.v + 3, col);
        } else {
          T pxw[3];
          cross3(sign == 1 ? oMc1.t : oMc2.t, Jc.v + 3, pxw);
          for (int k = 0; k < 3; ++k) col[k] = (Jc.v[k] - pxw[k]) * T(sign);
        }
      }
    } else {
      if (c.frame == RF_LOCAL) {
        const Vec6<T> l1 = actinv_motion(oMc1, Jc);
        for (int k = 0; k < 6; ++k) col[k] = l1.v[k] * T(sign);
      } else {
        T pxw[3];
        cross3(oMc1.t, Jc.v + 3, pxw);
        for (int k = 0; k < 3; ++k) {
          col[k] = (Jc.v[k] - pxw[k]) * T(sign);
          col[3 + k] = Jc.v[3 + k] * T(sign);
        }
      }
    }
    for (int k = 0; k < c.size(); ++k) ch.u(row + k, ch.nc + jj) = col[k];
  }
}

// ContactCholeskyDecomposition::compute at q (contact-cholesky.hxx:152-304: M in the bottom-right
// block, the constraint Jacobian rows in the top-right block, the factorisation with damping mu) and
// its accessors: matrix() = U D U^T (hxx:617-622), inverse() column by column with the strictly lower
// triangle copied from the upper (hxx:746-759), getInverseOperationalSpaceInertiaMatrix() =
// -U1 D1 U1^T, getOperationalSpaceInertiaMatrix() = -U1^-T D1^-1 U1^-1, getInverseMassMatrix() =
// U4^-T D4^-1 U4^-1, getJMinv() = U2 U4^-1 (contact-cholesky.hpp:168-265).  Every output is
// row-major and may be null.
template <class T>
void contact_cholesky(const Model& m, Data<T>& d, const T* q, const std::vector<ConstraintModel>& cms, T mu, T* kkt,
                      T* kkt_inv, T* osim_inv, T* osim, T* minv, T* jminv) {
  const int nv = m.nv;
  for (int i = 1; i < m.njoints; ++i) {  // placements, world columns and inertias (crba.hxx:23-96)
    const int p = m.parents[i], iq = m.idx_q[i], iv = m.idx_v[i];
    d.liMi[i] = se3_mul(placement_of<T>(m, i), joint_transform<T>(m, i, q + iq));
    d.oMi[i] = p > 0 ? se3_mul(d.oMi[p], d.liMi[i]) : d.liMi[i];
    for (int k = 0; k < m.nvs[i]; ++k) set_col6(d.J, iv + k, act_motion(d.oMi[i], S_col<T>(m, i, k)));
    d.oYcrb[i] = iner_act(d.oMi[i], inertia_of<T>(m, i));
  }
  std::fill(d.M.begin(), d.M.end(), T(0));
  for (int i = m.njoints - 1; i > 0; --i) {
    const int p = m.parents[i], iv = m.idx_v[i], nvi = m.nvs[i];
    for (int k = 0; k < nvi; ++k) set_col6(d.dFda, iv + k, iner_mul(d.oYcrb[i], col6(d.J, iv + k)));
    for (int r = 0; r < nvi; ++r)
      for (int c = iv; c < iv + m.nvSubtree[i]; ++c) d.M[(size_t)(iv + r) * nv + c] = dot6(col6(d.J, iv + r), col6(d.dFda, c));
    if (p > 0) iner_add(d.oYcrb[p], d.oYcrb[i]);
  }
  for (int k = 0; k < nv; ++k) d.M[(size_t)k * nv + k] += T(m.armature[k]);
  ContactCholesky<T> ch;
  ch.allocate(m, cms);
  const int nc = ch.nc, n = ch.n;
  for (int k = 0; k < nv; ++k) {
    ch.D[nc + k] = d.M[(size_t)k * nv + k];
    for (int c = k + 1; c < nv; ++c) ch.u(nc + k, nc + c) = d.M[(size_t)k * nv + c];
  }
  int row = 0;
  for (const ConstraintModel& c : cms) {
    const SE3<T> oMc1 = c.joint1 > 0 ? se3_mul(d.oMi[c.joint1], se3_from<T>(c.P1)) : se3_from<T>(c.P1);
    const SE3<T> oMc2 = c.joint2 > 0 ? se3_mul(d.oMi[c.joint2], se3_from<T>(c.P2)) : se3_from<T>(c.P2);
    constraint_jacobian(m, d, c, oMc1, oMc2, se3_actinv(oMc1, oMc2), row, ch);
    row += c.size();
  }
  ch.factor(mu);
  if (kkt)
    for (int r = 0; r < n; ++r)
      for (int c = 0; c < n; ++c) {
        T s = T(0);
        for (int k = std::max(r, c); k < n; ++k) s += ch.u(r, k) * ch.D[k] * ch.u(c, k);
        kkt[(size_t)r * n + c] = s;
      }
  if (kkt_inv) {
    std::vector<T> x(n);
    for (int c = 0; c < n; ++c) {
      std::fill(x.begin(), x.end(), T(0));
      x[c] = T(1);
      ch.solve(x.data());
      for (int r = 0; r <= c; ++r) kkt_inv[(size_t)r * n + c] = x[r];
    }
    for (int r = 0; r < n; ++r)
      for (int c = 0; c < r; ++c) kkt_inv[(size_t)r * n + c] = kkt_inv[(size_t)c * n + r];
  }
  if (osim_inv)
    for (int r = 0; r < nc; ++r)
      for (int c = 0; c < nc; ++c) {
        T s = T(0);
        for (int k = std::max(r, c); k < nc; ++k) s += ch.u(r, k) * ch.D[k] * ch.u(c, k);
        osim_inv[(size_t)r * nc + c] = -s;
      }
  // the inverse of a unit upper triangular block U[o.., o..] of size s: W (row-major, s x s)
  auto unit_upper_inverse = [&](int o, int s, std::vector<T>& W) {
    W.assign((size_t)s * s, T(0));
    for (int c = 0; c < s; ++c) {
      W[(size_t)c * s + c] = T(1);
      for (int r = c - 1; r >= 0; --r) {
        T t = T(0);
        for (int k = r + 1; k <= c; ++k) t += ch.u(o + r, o + k) * W[(size_t)k * s + c];
        W[(size_t)r * s + c] = -t;
      }
    }
  };
  std::vector<T> W;
  if (osim) {
    unit_upper_inverse(0, nc, W);
    for (int r = 0; r < nc; ++r)
      for (int c = 0; c < nc; ++c) {
        T s = T(0);
        for (int k = 0; k <= std::min(r, c); ++k) s += W[(size_t)k * nc + r] * ch.Dinv[k] * W[(size_t)k * nc + c];
        osim[(size_t)r * nc + c] = -s;
      }
  }
  if (minv || jminv) {
    unit_upper_inverse(nc, nv, W);
    if (minv)
      for (int r = 0; r < nv; ++r)
        for (int c = 0; c < nv; ++c) {
          T s = T(0);
          for (int k = 0; k <= std::min(r, c); ++k) s += W[(size_t)k * nv + r] * ch.Dinv[nc + k] * W[(size_t)k * nv + c];
          minv[(size_t)r * nv + c] = s;
        }
    if (jminv)
      for (int r = 0; r < nc; ++r)
        for (int c = 0; c < nv; ++c) {
          T s = T(0);
          for (int k = 0; k <= c; ++k) s += ch.u(r, nc + k) * W[(size_t)k * nv + c];
          jminv[(size_t)r * nv + c] = s;
        }
  }
}

struct ProximalResult {
  int iter = 0;
  double absolute_residual = -1.0, relative_residual = -1.0;
};

// constraintDynamics (constrained-dynamics.hxx:188-520).  ddq: nv; lambda: the stacked
// multipliers lambda_c (sum of the constraint sizes); the contact forces are lambda's segments.
template <class T>
ProximalResult constraint_dynamics(const Model& m, Data<T>& d, const T* q, const T* v, const T* tau,
                                   const std::vector<ConstraintModel>& cms, T mu, int max_iter, T abs_acc,
                                   T rel_acc, T* ddq, T* lambda) {
  const int nv = m.nv;
  // ContactAndImpulseDynamicsForwardStep (hxx:63-135) with ContactMode
  d.ov[0] = zero6<T>();
  d.oa[0] = zero6<T>();
  d.of[0] = zero6<T>();
  d.oYcrb[0] = Iner<T>{T(0), {T(0), T(0), T(0)}, {T(0), T(0), T(0), T(0), T(0), T(0)}};
  for (int i = 1; i < m.njoints; ++i) {
    const int p = m.parents[i], iq = m.idx_q[i], iv = m.idx_v[i];
    d.liMi[i] = se3_mul(placement_of<T>(m, i), joint_transform<T>(m, i, q + iq));
    d.oMi[i] = p > 0 ? se3_mul(d.oMi[p], d.liMi[i]) : d.liMi[i];
    d.ov[i] = act_motion(d.oMi[i], joint_velocity<T>(m, i, v + iv));
    if (p > 0) d.ov[i] = add6(d.ov[i], d.ov[p]);
    for (int k = 0; k < m.nvs[i]; ++k) set_col6(d.J, iv + k, act_motion(d.oMi[i], S_col<T>(m, i, k)));
    d.oinertias[i] = iner_act(d.oMi[i], inertia_of<T>(m, i));
    d.oYcrb[i] = d.oinertias[i];
    d.oh[i] = iner_mul(d.oinertias[i], d.ov[i]);
    d.oa[i] = zero6<T>();  // oMi.act(c) with c = 0 for these joints
    if (p > 0) d.oa[i] = add6(add6(d.oa[i], cross_motion(d.ov[p], d.ov[i])), d.oa[p]);
    for (int k = 0; k < 6; ++k) d.oa_gf[i].v[k] = d.oa[i].v[k] - T(m.gravity[k]);
    d.of[i] = add6(iner_mul(d.oinertias[i], d.oa_gf[i]), cross_force(d.ov[i], d.oh[i]));
  }
  // ContactAndImpulseDynamicsBackwardStep (hxx:137-186): M rows from dFda = oYcrb J, nle = J^T of
  std::fill(d.M.begin(), d.M.end(), T(0));
  std::vector<T> nle(nv);
  for (int i = m.njoints - 1; i > 0; --i) {
    const int p = m.parents[i], iv = m.idx_v[i], nvi = m.nvs[i];
    for (int k = 0; k < nvi; ++k) set_col6(d.dFda, iv + k, iner_mul(d.oYcrb[i], col6(d.J, iv + k)));
    for (int r = 0; r < nvi; ++r)
      for (int c = iv; c < iv + m.nvSubtree[i]; ++c) d.M[(size_t)(iv + r) * nv + c] = dot6(col6(d.J, iv + r), col6(d.dFda, c));
    iner_add(d.oYcrb[p], d.oYcrb[i]);
    for (int r = 0; r < nvi; ++r) nle[iv + r] = dot6(col6(d.J, iv + r), d.of[i]);
    d.of[p] = add6(d.of[p], d.of[i]);
  }
  for (int k = 0; k < nv; ++k) d.M[(size_t)k * nv + k] += T(m.armature[k]);
  // contact_chol.compute (contact-cholesky.hxx:152-272)
  ContactCholesky<T> ch;
  ch.allocate(m, cms);
  const int nc = ch.nc;
  for (int k = 0; k < nv; ++k) {
    ch.D[nc + k] = d.M[(size_t)k * nv + k];
    for (int c = k + 1; c < nv; ++c) ch.u(nc + k, nc + c) = d.M[(size_t)k * nv + c];
  }
  std::vector<SE3<T>> oMc1(cms.size()), oMc2(cms.size()), c1Mc2(cms.size());
  int row = 0;
  for (size_t e = 0; e < cms.size(); ++e) {  // RigidConstraintModel::calc (contact-info.hpp:426-446)
    const ConstraintModel& c = cms[e];
    oMc1[e] = c.joint1 > 0 ? se3_mul(d.oMi[c.joint1], se3_from<T>(c.P1)) : se3_from<T>(c.P1);
    oMc2[e] = c.joint2 > 0 ? se3_mul(d.oMi[c.joint2], se3_from<T>(c.P2)) : se3_from<T>(c.P2);
    c1Mc2[e] = se3_actinv(oMc1[e], oMc2[e]);
    constraint_jacobian(m, d, c, oMc1[e], oMc2[e], c1Mc2[e], row, ch);
    row += c.size();
  }
  ch.factor(mu);
  // the right-hand side: contact drifts and Baumgarte corrections (hxx:282-432)
  std::vector<T> rhs(nc);
  row = 0;
  for (size_t e = 0; e < cms.size(); ++e) {
    const ConstraintModel& c = cms[e];
    const int j1 = c.joint1, j2 = c.joint2;
    const Vec6<T> vc1 = j1 > 0 ? actinv_motion(oMc1[e], d.ov[j1]) : zero6<T>();
    const Vec6<T> vc2 = j2 > 0 ? actinv_motion(oMc2[e], d.ov[j2]) : zero6<T>();
    const Vec6<T> vc2_1 = act_motion(c1Mc2[e], vc2);
    Vec6<T> pe = zero6<T>(), ve = zero6<T>(), ae = zero6<T>(), a1, a2;
    if (c.type == CONTACT_6D) {
      const Vec6<T> lg = log6(c1Mc2[e]);
      for (int k = 0; k < 6; ++k) {
        pe.v[k] = -lg.v[k];
        ve.v[k] = vc1.v[k] - vc2_1.v[k];
      }
    } else {
      T r2[3];
      matvec(c1Mc2[e].R, vc2.v, r2);
      for (int k = 0; k < 3; ++k) {
        pe.v[k] = -c1Mc2[e].t[k];
        ve.v[k] = vc1.v[k] - r2[k];
      }
    }
    bool gains = false;
    for (int k = 0; k < 6; ++k) gains = gains || c.Kp[k] != 0.0 || c.Kd[k] != 0.0;
    if (gains)
      for (int k = 0; k < (c.type == CONTACT_6D ? 6 : 3); ++k) ae.v[k] = -T(c.Kp[k]) * pe.v[k] - T(c.Kd[k]) * ve.v[k];
    const Vec6<T>& oa1 = d.oa[j1];
    const Vec6<T>& oa2 = d.oa[j2];
    const Vec6<T>& ov1 = d.ov[j1];
    const Vec6<T>& ov2 = d.ov[j2];
    // the classical acceleration part of a point p: ov.ang x (ov.lin + ov.ang x p)
    auto point_drift = [](const Vec6<T>& ov, const T* pt, T* o) {
      T wxp[3], vp[3];
      cross3(ov.v + 3, pt, wxp);
      for (int k = 0; k < 3; ++k) vp[k] = ov.v[k] + wxp[k];
      cross3(ov.v + 3, vp, o);
    };
    if (c.frame == RF_LOCAL_WORLD_ALIGNED) {
      T t[3];
      cross3(oa1.v + 3, oMc1[e].t, t);
      for (int k = 0; k < 3; ++k) a1.v[k] = oa1.v[k] + t[k];
      if (c.type == CONTACT_3D) {
        point_drift(ov1, oMc1[e].t, t);
        for (int k = 0; k < 3; ++k) a1.v[k] += t[k];
      }
      for (int k = 0; k < 3; ++k) a1.v[3 + k] = oa1.v[3 + k];
      if (c.type == CONTACT_3D) {
        T u[3];
        cross3(oa2.v + 3, oMc2[e].t, t);
        point_drift(ov2, oMc2[e].t, u);
        for (int k = 0; k < 3; ++k) {
          a2.v[k] = oa2.v[k] + t[k] + u[k];
          a2.v[3 + k] = T(0);
        }
      } else {
        cross3(oa2.v + 3, oMc1[e].t, t);
        for (int k = 0; k < 3; ++k) {
          a2.v[k] = oa2.v[k] + t[k];
          a2.v[3 + k] = oa2.v[3 + k];
        }
      }
      T rl[3], ra[3];
      matvec(oMc1[e].R, ae.v, rl);
      matvec(oMc1[e].R, ae.v + 3, ra);
      for (int k = 0; k < 3; ++k) {
        ae.v[k] = rl[k];
        ae.v[3 + k] = ra[k];
      }
    } else {
      a1 = actinv_motion(oMc1[e], oa1);
      if (c.type == CONTACT_3D) {
        T t[3];
        cross3(vc1.v + 3, vc1.v, t);
        for (int k = 0; k < 3; ++k) {
          a1.v[k] += t[k];
          a1.v[3 + k] = T(0);
        }
        T u[3], w[3];
        cross3(oa2.v + 3, oMc2[e].t, t);
        point_drift(ov2, oMc2[e].t, u);
        for (int k = 0; k < 3; ++k) w[k] = oa2.v[k] + t[k] + u[k];
        matTvec(oMc1[e].R, w, a2.v);
        for (int k = 0; k < 3; ++k) a2.v[3 + k] = T(0);
      } else {
        a1 = add6(a1, cross_motion(ve, vc2_1));
        a2 = actinv_motion(oMc1[e], oa2);
      }
    }
    for (int k = 0; k < c.size(); ++k) rhs[row + k] = -a1.v[k] + a2.v[k] + ae.v[k] + T(c.desired_acc[k]);
    row += c.size();
  }
  // the proximal iterations (hxx:434-486)
  ProximalResult res;
  std::vector<T> x(nc + nv), lprox(nc, T(0)), tmp(nc);
  int it = 0;
  for (; it < max_iter;) {
    ++it;
    for (int k = 0; k < nc; ++k) x[k] = rhs[k] + lprox[k] * mu;
    for (int k = 0; k < nv; ++k) x[nc + k] = tau[k] - nle[k];
    ch.solve(x.data());
    ch.delassus_apply(x.data(), tmp.data());
    T ar = T(0), rr = T(0);
    for (int k = 0; k < nc; ++k) {
      tmp[k] -= mu * x[k] + rhs[k];
      ar = o_max(ar, tmp[k] < T(0) ? -tmp[k] : tmp[k]);
      const T dk = x[k] + lprox[k];
      rr = o_max(rr, dk < T(0) ? -dk : dk);
    }
    res.absolute_residual = (double)ar;
    res.relative_residual = (double)rr;
    for (int k = 0; k < nc; ++k) lprox[k] = -x[k];
    if (ar <= abs_acc || rr <= rel_acc) break;
  }
  res.iter = it;
  for (int k = 0; k < nv; ++k) ddq[k] = x[nc + k];
  for (int k = 0; k < nc; ++k) lambda[k] = -x[k];
  return res;
}

// ---------------------------------------------------------------------------
// computeConstraintDynamicsDerivatives for constraints to the world (joint2 = 0) without Baumgarte
// gains (algorithm/constrained-dynamics-derivatives.hxx:344-1050): the inverse dynamics
// derivatives at (q, v, ddq) with the contact forces as forces on the contact joints
// (ContactForceContribution, hxx:225-342), the contact frames' acceleration derivatives
// (getFrameAccelerationDerivatives, frames-derivatives.hxx:85-176, on
// JointAccelerationDerivativesBackwardStep, kinematics-derivatives.hxx:285-440; for point
// contacts getPointClassicAccelerationDerivatives, kinematics-derivatives.hxx:700-940), and the
// assembly with the operational-space inertia and the proximal recursion (hxx:815-1045).
// Outputs nv x nv (ddq_dq, ddq_dv, ddq_dtau) and nc x nv (dlambda_dq, dlambda_dv, dlambda_dtau),
// row-major.
// ---------------------------------------------------------------------------
template <class T>
void translate_motion(const T* p, Vec6<T>& m) {  // linear -= p x angular
  T w[3];
  cross3(p, m.v + 3, w);
  for (int k = 0; k < 3; ++k) m.v[k] -= w[k];
}

// rows 0..5 of a 6 x nv column-major set written column by column: o[6 * col + r]
template <class T>
void frame_acceleration_derivatives(const Model& m, const Data<T>& d, int joint, const SE3<T>& P, int rf,
                                    std::vector<T>& v_dq, std::vector<T>& a_dq, std::vector<T>& a_dv,
                                    std::vector<T>& a_da) {
  const int nv = m.nv;
  for (auto* x : {&v_dq, &a_dq, &a_dv, &a_da}) x->assign(6 * (size_t)nv, T(0));
  const SE3<T>& oMl = d.oMi[joint];
  const Vec6<T>& alast = d.oa[joint];
  for (int i = joint; i > 0; i = m.parents[i]) {  // JointAccelerationDerivativesBackwardStep
    const int p = m.parents[i];
    for (int k = 0; k < m.nvs[i]; ++k) {
      const int c = m.idx_v[i] + k;
      const Vec6<T> Jc = col6(d.J, c), dJc = col6(d.dJ, c);
      Vec6<T> da, vdq = zero6<T>(), adq = zero6<T>(), adv;
      if (rf == RF_LOCAL) {
        da = actinv_motion(oMl, Jc);
        Vec6<T> vtmp = zero6<T>();
        if (p > 0) {
          vtmp = actinv_motion(oMl, d.ov[p]);
          vdq = cross_motion(vtmp, da);
        }
        for (int r = 0; r < 6; ++r) vtmp.v[r] -= d.v[joint].v[r];
        adv = add6(cross_motion(vtmp, da), actinv_motion(oMl, dJc));
        if (p > 0) adq = add6(cross_motion(actinv_motion(oMl, d.oa[p]), da), cross_motion(vtmp, vdq));
      } else {
        da = Jc;
        translate_motion(oMl.t, da);
        Vec6<T> vtmp, atmp;
        for (int r = 0; r < 6; ++r) {
          vtmp.v[r] = (p > 0 ? d.ov[p].v[r] : T(0)) - d.ov[joint].v[r];
          atmp.v[r] = (p > 0 ? d.oa[p].v[r] : T(0)) - alast.v[r];
        }
        T w[3];
        cross3(vtmp.v + 3, oMl.t, w);
        for (int r = 0; r < 3; ++r) vtmp.v[r] += w[r];
        cross3(atmp.v + 3, oMl.t, w);
        for (int r = 0; r < 3; ++r) atmp.v[r] += w[r];
        vdq = cross_motion(vtmp, da);
        adv = dJc;
        translate_motion(oMl.t, adv);
        adq = cross_motion(atmp, da);
        if (p > 0) adq = add6(adq, cross_motion(vtmp, adv));
        adv = add6(adv, vdq);
      }
      set_col6(v_dq, c, vdq);
      set_col6(a_dq, c, adq);
      set_col6(a_dv, c, adv);
      set_col6(a_da, c, da);
    }
  }
  // getFrameAccelerationDerivatives' frame transform (frames-derivatives.hxx:137-172)
  T trans[3];
  matvec(oMl.R, P.t, trans);
  for (int i = joint; i > 0; i = m.parents[i])
    for (int k = 0; k < m.nvs[i]; ++k) {
      const int c = m.idx_v[i] + k;
      for (auto* x : {&v_dq, &a_dq, &a_dv, &a_da}) {
        Vec6<T> col = col6(*x, c);
        if (rf == RF_LOCAL_WORLD_ALIGNED) translate_motion(trans, col);
        else col = actinv_motion(P, col);
        set_col6(*x, c, col);
      }
    }
}

// PointClassicAccelerationDerivativesBackwardStep over the support of `joint`; 3 x nv outputs
// (o[3 * col + r])
template <class T>
void point_acceleration_derivatives(const Model& m, const Data<T>& d, int joint, const SE3<T>& P, int rf,
                                    std::vector<T>& v_dq, std::vector<T>& a_dq, std::vector<T>& a_dv,
                                    std::vector<T>& a_da) {
  const int nv = m.nv;
  for (auto* x : {&v_dq, &a_dq, &a_dv, &a_da}) x->assign(3 * (size_t)nv, T(0));
  const SE3<T> oMp = se3_mul(d.oMi[joint], P);
  const Vec6<T> vl = actinv_motion(oMp, d.ov[joint]);
  const Vec6<T> al = actinv_motion(oMp, d.oa[joint]);
  T pacc[3];
  cross3(vl.v + 3, vl.v, pacc);
  for (int r = 0; r < 3; ++r) pacc[r] += al.v[r];
  auto put = [&](std::vector<T>& x, int c, const T* v3) {
    for (int r = 0; r < 3; ++r) x[3 * (size_t)c + r] = v3[r];
  };
  for (int i = joint; i > 0; i = m.parents[i]) {
    const int p = m.parents[i];
    for (int k = 0; k < m.nvs[i]; ++k) {
      const int c = m.idx_v[i] + k;
      const Vec6<T> Jc = col6(d.J, c), dJc = col6(d.dJ, c);
      const Vec6<T> sda = actinv_motion(oMp, Jc);
      Vec6<T> svdq = zero6<T>(), vtmp = zero6<T>();
      T vdq[3] = {T(0), T(0), T(0)}, adq[3] = {T(0), T(0), T(0)}, adv[3], t1[3], t2[3];
      if (p > 0) {
        vtmp = actinv_motion(oMp, d.ov[p]);
        svdq = cross_motion(vtmp, sda);
        for (int r = 0; r < 3; ++r) vdq[r] = svdq.v[r];
      }
      for (int r = 0; r < 6; ++r) vtmp.v[r] -= vl.v[r];
      cross3(vtmp.v + 3, sda.v, t1);
      cross3(vtmp.v, sda.v + 3, t2);
      for (int r = 0; r < 3; ++r) adv[r] = t1[r] + t2[r];
      T dl[3], wxt[3];
      cross3(dJc.v + 3, oMp.t, wxt);
      for (int r = 0; r < 3; ++r) dl[r] = dJc.v[r] + wxt[r];
      matTvec(oMp.R, dl, t1);
      for (int r = 0; r < 3; ++r) adv[r] += t1[r];
      cross3(vl.v + 3, sda.v, t1);
      cross3(vl.v, sda.v + 3, t2);
      for (int r = 0; r < 3; ++r) adv[r] += t1[r] - t2[r];
      if (p > 0) {
        const Vec6<T> atmp = actinv_motion(oMp, d.oa[p]);
        cross3(atmp.v + 3, sda.v, t1);
        cross3(atmp.v, sda.v + 3, t2);
        for (int r = 0; r < 3; ++r) adq[r] = t1[r] + t2[r];
        cross3(vtmp.v + 3, svdq.v, t1);
        cross3(vtmp.v, svdq.v + 3, t2);
        for (int r = 0; r < 3; ++r) adq[r] += t1[r] + t2[r];
        cross3(vl.v + 3, svdq.v, t1);
        cross3(vl.v, svdq.v + 3, t2);
        for (int r = 0; r < 3; ++r) adq[r] += t1[r] - t2[r];
      }
      T ada[3] = {sda.v[0], sda.v[1], sda.v[2]};
      if (rf == RF_LOCAL_WORLD_ALIGNED) {
        T x[3], y[3];
        cross3(sda.v + 3, vl.v, x);
        for (int r = 0; r < 3; ++r) x[r] += vdq[r];
        matvec(oMp.R, x, vdq);
        cross3(sda.v + 3, pacc, x);
        for (int r = 0; r < 3; ++r) x[r] += adq[r];
        matvec(oMp.R, x, adq);
        matvec(oMp.R, adv, y);
        for (int r = 0; r < 3; ++r) adv[r] = y[r];
        matvec(oMp.R, ada, y);
        for (int r = 0; r < 3; ++r) ada[r] = y[r];
      }
      put(v_dq, c, vdq);
      put(a_dq, c, adq);
      put(a_dv, c, adv);
      put(a_da, c, ada);
    }
  }
}

template <class T>
ProximalResult constraint_dynamics_derivatives(const Model& m, Data<T>& d, const T* q, const T* v, const T* tau,
                                               const std::vector<ConstraintModel>& cms, T mu, int max_iter,
                                               T abs_acc, T rel_acc, T* ddq, T* lambda, T* ddq_dq, T* ddq_dv,
                                               T* ddq_dtau, T* dl_dq, T* dl_dv, T* dl_dtau) {
  for (const auto& c : cms) {
    bool gains = false;
    for (int k = 0; k < 6; ++k) gains = gains || c.Kp[k] != 0.0 || c.Kd[k] != 0.0;
    if (c.joint2 != 0 || (gains && c.frame != RF_LOCAL))
      throw std::invalid_argument(
          "the derivatives take constraints to the world, with Baumgarte gains on LOCAL contacts only");
  }
  const int nv = m.nv;
  const ProximalResult res = constraint_dynamics(m, d, q, v, tau, cms, mu, max_iter, abs_acc, rel_acc, ddq, lambda);
  int nc = 0;
  for (const auto& c : cms) nc += c.size();
  // the contact forces as forces on the contact joints, in their frames (fext of rnea_derivatives):
  // ContactForceContribution subtracts them from of[joint1] in the world frame
  std::vector<T> fext(6 * (size_t)m.njoints, T(0));
  std::vector<SE3<T>> oMc(cms.size());
  int row = 0;
  for (size_t e = 0; e < cms.size(); ++e) {
    const ConstraintModel& c = cms[e];
    const SE3<T> P = se3_from<T>(c.P1);
    oMc[e] = se3_mul(d.oMi[c.joint1], P);
    Vec6<T> f = zero6<T>();
    for (int k = 0; k < c.size(); ++k) f.v[k] = lambda[row + k];
    Vec6<T> fj;
    if (c.frame == RF_LOCAL) {
      fj = act_force(P, f);
    } else {  // world-aligned force at the contact point -> world force about the origin -> joint frame
      Vec6<T> fw = f;
      T w[3];
      cross3(oMc[e].t, f.v, w);
      for (int r = 0; r < 3; ++r) fw.v[3 + r] += w[r];
      const SE3<T>& oMi = d.oMi[c.joint1];
      // oMi^-1 . act(force): linear R^T f, angular R^T (n - t x f)
      T fl[3], tmp[3], nn[3];
      matTvec(oMi.R, fw.v, fl);
      cross3(oMi.t, fw.v, tmp);
      for (int r = 0; r < 3; ++r) nn[r] = fw.v[3 + r] - tmp[r];
      matTvec(oMi.R, nn, fj.v + 3);
      for (int r = 0; r < 3; ++r) fj.v[r] = fl[r];
    }
    for (int k = 0; k < 6; ++k) fext[6 * (size_t)c.joint1 + k] += fj.v[k];
    row += c.size();
  }
  rnea_derivatives(m, d, q, v, ddq, fext.data());  // J, dJ, ov, oa at ddq; dtau_dq, dtau_dv
  std::vector<T> dtq(d.dtau_dq), dtv(d.dtau_dv);
  // M^-1 (the KKT factor's bottom-right block: M with the armature)
  crba(m, d, q, LOCAL);
  std::fill(d.U.begin(), d.U.end(), T(0));
  for (int k = 0; k < nv; ++k) d.U[(size_t)k * nv + k] = T(1);
  cholesky_decompose(m, d);
  std::vector<T> Minv((size_t)nv * nv);
  for (int c = 0; c < nv; ++c) {
    std::vector<T> col(nv, T(0));
    col[c] = T(1);
    chol_solve(m, d, col.data());
    for (int r = 0; r < nv; ++r) Minv[(size_t)r * nv + c] = col[r];
  }
  // the contact rows: dac_da (= the constraint Jacobian), dac_dq, dac_dv
  std::vector<T> Jc((size_t)nc * nv, T(0)), Aq((size_t)nc * nv, T(0)), Av((size_t)nc * nv, T(0));
  row = 0;
  std::vector<T> vdq, adq, adv, ada;
  for (size_t e = 0; e < cms.size(); ++e) {
    const ConstraintModel& c = cms[e];
    const SE3<T> P = se3_from<T>(c.P1);
    const int n = c.size();
    if (c.type == CONTACT_6D) frame_acceleration_derivatives(m, d, c.joint1, P, c.frame, vdq, adq, adv, ada);
    else point_acceleration_derivatives(m, d, c.joint1, P, c.frame, vdq, adq, adv, ada);
    const int stride = c.type == CONTACT_6D ? 6 : 3;
    for (int k = 0; k < n; ++k)
      for (int col = 0; col < nv; ++col) {
        Jc[(size_t)(row + k) * nv + col] = ada[(size_t)stride * col + k];
        Aq[(size_t)(row + k) * nv + col] = adq[(size_t)stride * col + k];
        Av[(size_t)(row + k) * nv + col] = adv[(size_t)stride * col + k];
      }
    bool gains = false;
    for (int k = 0; k < 6; ++k) gains = gains || c.Kp[k] != 0.0 || c.Kd[k] != 0.0;
    if (gains && c.type == CONTACT_6D) {  // the corrector's derivative for a LOCAL frame contact
      // (hxx:758-782): dac_dq += Kd dvc_dq + Kp Jlog6(c1Mc2^-1) dac_da, dac_dv += Kd dac_da
      const SE3<T> oMc1 = se3_mul(d.oMi[c.joint1], P);
      const SE3<T> c1Mc2 = se3_actinv(oMc1, se3_from<T>(c.P2));
      SE3<T> c2Mc1;  // the inverse placement (R^T, -R^T t)
      for (int r = 0; r < 3; ++r)
        for (int q2 = 0; q2 < 3; ++q2) c2Mc1.R[3 * r + q2] = c1Mc2.R[3 * q2 + r];
      matTvec(c1Mc2.R, c1Mc2.t, c2Mc1.t);
      for (int r = 0; r < 3; ++r) c2Mc1.t[r] = -c2Mc1.t[r];
      T Jl[36];
      jlog6(c2Mc1, Jl);
      for (int col = 0; col < nv; ++col)
        for (int k = 0; k < 6; ++k) {
          T acc = T(0);
          for (int i = 0; i < 6; ++i) acc += Jl[6 * k + i] * ada[(size_t)6 * col + i];
          Aq[(size_t)(row + k) * nv + col] += T(c.Kd[k]) * vdq[(size_t)6 * col + k] + T(c.Kp[k]) * acc;
          Av[(size_t)(row + k) * nv + col] += T(c.Kd[k]) * ada[(size_t)6 * col + k];
        }
    } else if (gains) {  // the corrector's derivative for a LOCAL point contact to the world (hxx:753-830):
      // dac_dq += Kd dvc_dq + Kp dac_da + Kp pe x (R1^T J_ang) on joint 1's support (pe =
      // -c1Mc2.translation the placement error), dac_dv += Kd dac_da.  (In LOCAL_WORLD_ALIGNED axes
      // the reference's same terms miss the rotation of the corrector into world axes: central
      // differences disagree, so those are refused.)
      const SE3<T> oMc1 = se3_mul(d.oMi[c.joint1], P);
      const SE3<T> c1Mc2 = se3_actinv(oMc1, se3_from<T>(c.P2));
      const T pe[3] = {-c1Mc2.t[0], -c1Mc2.t[1], -c1Mc2.t[2]};
      for (int j = m.idx_v[c.joint1] + m.nvs[c.joint1] - 1; j >= 0; j = m.parents_fromRow[j]) {
          const Vec6<T> Jcol = col6(d.J, j);
          T wa[3], x[3];
          matTvec(oMc1.R, Jcol.v + 3, wa);
          cross3(pe, wa, x);
          for (int k = 0; k < 3; ++k) Aq[(size_t)(row + k) * nv + j] += T(c.Kp[k]) * x[k];
        }
      for (int k = 0; k < 3; ++k)
        for (int col = 0; col < nv; ++col) {
          const T da = ada[(size_t)3 * col + k];
          Aq[(size_t)(row + k) * nv + col] += T(c.Kd[k]) * vdq[(size_t)3 * col + k] + T(c.Kp[k]) * da;
          Av[(size_t)(row + k) * nv + col] += T(c.Kd[k]) * da;
        }
    }
    row += n;
  }
  // JMinv, osim = (J M^-1 J^T + mu I)^-1
  std::vector<T> JMinv((size_t)nc * nv, T(0)), G((size_t)nc * nc), osim((size_t)nc * nc);
  for (int r = 0; r < nc; ++r)
    for (int c = 0; c < nv; ++c) {
      T s = T(0);
      for (int k = 0; k < nv; ++k) s += Jc[(size_t)r * nv + k] * Minv[(size_t)k * nv + c];
      JMinv[(size_t)r * nv + c] = s;
    }
  for (int r = 0; r < nc; ++r)
    for (int c = 0; c < nc; ++c) {
      T s = T(0);
      for (int k = 0; k < nv; ++k) s += JMinv[(size_t)r * nv + k] * Jc[(size_t)c * nv + k];
      G[(size_t)r * nc + c] = s + (r == c ? mu : T(0));
    }
  for (int c = 0; c < nc; ++c) {
    std::vector<T> Gc(G), e(nc, T(0));
    e[c] = T(1);
    llt_factor_solve(nc, Gc.data(), e.data());
    for (int r = 0; r < nc; ++r) osim[(size_t)r * nc + c] = e[r];
  }
  // the proximal recursion of a right-hand side R (nc x nv): X_1 = -osim R, X_k = osim (mu X_{k-1} - R)
  auto prox = [&](const std::vector<T>& R, T* X) {
    std::vector<T> prev((size_t)nc * nv), t((size_t)nc * nv);
    for (int r = 0; r < nc; ++r)
      for (int c = 0; c < nv; ++c) {
        T s = T(0);
        for (int k = 0; k < nc; ++k) s += osim[(size_t)r * nc + k] * R[(size_t)k * nv + c];
        X[(size_t)r * nv + c] = -s;
      }
    for (int it = 1; it < res.iter; ++it) {
      for (size_t k = 0; k < prev.size(); ++k) t[k] = mu * X[k] - R[k];
      for (int r = 0; r < nc; ++r)
        for (int c = 0; c < nv; ++c) {
          T s = T(0);
          for (int k = 0; k < nc; ++k) s += osim[(size_t)r * nc + k] * t[(size_t)k * nv + c];
          X[(size_t)r * nv + c] = s;
        }
    }
  };
  prox(JMinv, dl_dtau);
  for (int r = 0; r < nv; ++r)  // ddq_dtau = M^-1 + JMinv^T dl_dtau
    for (int c = 0; c < nv; ++c) {
      T s = Minv[(size_t)r * nv + c];
      for (int k = 0; k < nc; ++k) s += JMinv[(size_t)k * nv + r] * dl_dtau[(size_t)k * nv + c];
      ddq_dtau[(size_t)r * nv + c] = s;
    }
  for (int pass = 0; pass < 2; ++pass) {
    std::vector<T>& dt = pass == 0 ? dtq : dtv;
    const std::vector<T>& A = pass == 0 ? Aq : Av;
    T* dl = pass == 0 ? dl_dq : dl_dv;
    T* out = pass == 0 ? ddq_dq : ddq_dv;
    std::vector<T> R((size_t)nc * nv);
    for (int r = 0; r < nc; ++r)  // R = dac_dx - JMinv dtau_dx
      for (int c = 0; c < nv; ++c) {
        T s = T(0);
        for (int k = 0; k < nv; ++k) s += JMinv[(size_t)r * nv + k] * dt[(size_t)k * nv + c];
        R[(size_t)r * nv + c] = A[(size_t)r * nv + c] - s;
      }
    prox(R, dl);
    for (int r = 0; r < nv; ++r)  // dtau_dx -= J^T dl_dx
      for (int c = 0; c < nv; ++c) {
        T s = T(0);
        for (int k = 0; k < nc; ++k) s += Jc[(size_t)k * nv + r] * dl[(size_t)k * nv + c];
        dt[(size_t)r * nv + c] -= s;
      }
    for (int r = 0; r < nv; ++r)  // ddq_dx = -M^-1 dtau_dx
      for (int c = 0; c < nv; ++c) {
        T s = T(0);
        for (int k = 0; k < nv; ++k) s += Minv[(size_t)r * nv + k] * dt[(size_t)k * nv + c];
        out[(size_t)r * nv + c] = -s;
      }
  }
  // world-aligned contacts: the force rotates with nothing (hxx:1000-1040)
  row = 0;
  for (size_t e = 0; e < cms.size(); ++e) {
    const ConstraintModel& c = cms[e];
    if (c.frame == RF_LOCAL_WORLD_ALIGNED) {
      const int colRef = m.idx_v[c.joint1] + m.nvs[c.joint1] - 1;
      for (int j = colRef; j >= 0; j = m.parents_fromRow[j]) {
        const Vec6<T> J = col6(d.J, j);
        T w[3];
        cross3(J.v + 3, lambda + row, w);
        for (int r = 0; r < 3; ++r) dl_dq[(size_t)(row + r) * nv + j] += w[r];
        if (c.type == CONTACT_6D) {
          cross3(J.v + 3, lambda + row + 3, w);
          for (int r = 0; r < 3; ++r) dl_dq[(size_t)(row + 3 + r) * nv + j] += w[r];
        }
      }
    }
    row += c.size();
  }
  return res;
}

}  // namespace orc
