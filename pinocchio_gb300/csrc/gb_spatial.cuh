// Spatial algebra for the per-instance dynamics sweeps, host/device templated
// on the scalar.  Conventions (shared with the reference):
//   motion / force 6-vectors [linear(0:3); angular(3:6)];
//   SE3 (R row-major, t); act(m) = (R m_lin + t x R m_ang, R m_ang);
//   inertia (m, c, Ic packed [xx, xy, yy, xz, yz, zz]);
//   6x6 symmetric matrices stored by 3x3 blocks: A = lin-lin (packed sym3),
//   B = lin-ang (full 3x3 row-major), D = ang-ang (packed sym3); the ang-lin
//   block is B^T.
#pragma once

#if defined(__CUDACC__)
#define GB_HD __host__ __device__ __forceinline__
#else
#define GB_HD inline
#endif

#include <math.h>

namespace gb {

// FP32 <-> FP64 conversions.  On the device the hardware conversions issue on
// the FP64 pipe (a small fraction of the FP32 rate on GB300), so the exact
// FP32 -> FP64 widening and the round-to-nearest-even FP64 -> FP32 narrowing
// are done with integer instructions on the bit patterns (IEEE 754 binary32 /
// binary64 layouts), branch-free: zero, infinity and NaN map exactly; values
// below the normal FP32 range (subnormal inputs of widen, results of narrow
// smaller than 2^-126) become a signed zero, a change below 1.2e-38.
GB_HD double widen(float x) {
#if defined(__CUDA_ARCH__)
  const unsigned u = __float_as_uint(x);
  const unsigned ex = (u >> 23) & 0xffu;
  const unsigned mant = (u & 0x7fffffu) >> 3;
  const unsigned ex64 = ex == 0u ? 0u : (ex == 0xffu ? 0x7ffu : ex + 896u);
  const unsigned hi = (u & 0x80000000u) | (ex64 << 20) | (ex == 0u ? 0u : mant);
  const unsigned lo = ex == 0u ? 0u : (u << 29);
  return __hiloint2double((int)hi, (int)lo);
#else
  return (double)x;
#endif
}
GB_HD float narrow(double x) {
#if defined(__CUDA_ARCH__)
  const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  const unsigned sign = hi & 0x80000000u;
  const unsigned ex = (hi >> 20) & 0x7ffu;
  const unsigned mant = ((hi & 0xfffffu) << 3) | (lo >> 29);  // top 23 of the 52 fraction bits
  const unsigned rest = lo & 0x1fffffffu;                      // the 29 bits dropped
  unsigned r = sign | (((ex - 896u) & 0xffu) << 23) | mant;
  r += (rest > 0x10000000u || (rest == 0x10000000u && (mant & 1u))) ? 1u : 0u;  // carries into the exponent
  const bool nan = ex == 0x7ffu && (((hi & 0xfffffu) | lo) != 0u);
  r = ex < 897u ? sign : r;                                                        // zero / below FP32's range
  r = ex > 1150u ? (sign | 0x7f800000u | (nan ? 0x400000u : 0u)) : r;              // overflow, inf, NaN
  return __uint_as_float(r);
#else
  return (float)x;
#endif
}
// T(x) with the integer conversions between FP32 and FP64
template <class T, class U> GB_HD T cvt(U x) { return T(x); }
template <> GB_HD double cvt<double, float>(float x) { return widen(x); }
template <> GB_HD float cvt<float, double>(double x) { return narrow(x); }


// packed symmetric 3x3 index (xx, xy, yy, xz, yz, zz)
GB_HD constexpr int s3(int r, int c) {
  return (r == 0 && c == 0) ? 0 : (r + c == 1) ? 1 : (r == 1 && c == 1) ? 2 : (r + c == 2) ? 3 : (r + c == 3) ? 4 : 5;
}

template <class S> GB_HD S sqr(S x) { return x * x; }

template <class S> struct M6 { S v[6]; };   // motion or force
template <class S> struct X3 { S R[9]; S t[3]; };

// column `ax` (0, 1, 2) of a rotation, chosen by selects rather than a
// run-time array index (which would move the matrix to local memory)
template <class S> GB_HD void axis_column(const X3<S>& O, int ax, S* w) {
#pragma unroll
  for (int k = 0; k < 3; ++k) w[k] = ax == 0 ? O.R[3 * k] : (ax == 1 ? O.R[3 * k + 1] : O.R[3 * k + 2]);
}
// x[ax] of a 3-vector by selects
template <class S> GB_HD S pick3(const S* x, int ax) { return ax == 0 ? x[0] : (ax == 1 ? x[1] : x[2]); }
// x[k] of a 6-vector by selects
template <class S> GB_HD S pick6(const S* x, int k) { return k < 3 ? pick3(x, k) : pick3(x + 3, k - 3); }
// x[k] += a for a run-time k, by selects
template <class S> GB_HD void add_at6(S* x, int k, S a) {
#pragma unroll
  for (int r = 0; r < 6; ++r) x[r] += r == k ? a : S(0);
}
template <class S> struct Sym6 { S A[6]; S B[9]; S D[6]; };

template <class S> GB_HD void zero(M6<S>& m) {
#pragma unroll
  for (int k = 0; k < 6; ++k) m.v[k] = S(0);
}
// Short dot products.  The double-float scalar overloads them with one
// compensated accumulation per dot product instead of a normalised sum per term.
template <class S> GB_HD S dot2(S a0, S b0, S a1, S b1) { return a0 * b0 + a1 * b1; }
template <class T> GB_HD T dot6(const T* a, const T* b) {
  T s = a[0] * b[0];
#pragma unroll
  for (int k = 1; k < 6; ++k) s += a[k] * b[k];
  return s;
}
template <class S> GB_HD S dot3(S a0, S b0, S a1, S b1, S a2, S b2) { return a0 * b0 + a1 * b1 + a2 * b2; }
template <class S> GB_HD void cross3(const S* a, const S* b, S* o) {
  const S x = dot2(a[1], b[2], -a[2], b[1]);
  const S y = dot2(a[2], b[0], -a[0], b[2]);
  const S z = dot2(a[0], b[1], -a[1], b[0]);
  o[0] = x; o[1] = y; o[2] = z;
}
template <class S> GB_HD void mv3(const S* R, const S* x, S* o) {
  const S a = dot3(R[0], x[0], R[1], x[1], R[2], x[2]);
  const S b = dot3(R[3], x[0], R[4], x[1], R[5], x[2]);
  const S c = dot3(R[6], x[0], R[7], x[1], R[8], x[2]);
  o[0] = a; o[1] = b; o[2] = c;
}
template <class S> GB_HD void mtv3(const S* R, const S* x, S* o) {
  const S a = dot3(R[0], x[0], R[3], x[1], R[6], x[2]);
  const S b = dot3(R[1], x[0], R[4], x[1], R[7], x[2]);
  const S c = dot3(R[2], x[0], R[5], x[1], R[8], x[2]);
  o[0] = a; o[1] = b; o[2] = c;
}
template <class S> GB_HD void sym3_mv(const S* s, const S* x, S* o) {
  const S a = dot3(s[0], x[0], s[1], x[1], s[3], x[2]);
  const S b = dot3(s[1], x[0], s[2], x[1], s[4], x[2]);
  const S c = dot3(s[3], x[0], s[4], x[1], s[5], x[2]);
  o[0] = a; o[1] = b; o[2] = c;
}

// --- rigid transforms ---------------------------------------------------------------------
// Rotation of a joint about a unit axis, composed on the right of a placement:
// liMi = placement * (Rax(c, s), 0)  (revolute joint, reference joint-revolute.hpp:213-235).
template <int AX, class S> GB_HD void compose_axis_ax(const S* PR, const S* Pt, S c, S s, X3<S>& out) {
  // columns i, j rotated: col_i' = c col_i + s col_j ; col_j' = -s col_i + c col_j (i,j cyclic after axis)
  constexpr int i = (AX + 1) % 3, j = (AX + 2) % 3;
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    const S pi = PR[3 * r + i], pj = PR[3 * r + j];
    out.R[3 * r + AX] = PR[3 * r + AX];
    out.R[3 * r + i] = c * pi + s * pj;
    out.R[3 * r + j] = c * pj - s * pi;
    out.t[r] = Pt[r];
  }
}
// The axis is the same for every thread of a warp (all run the same joint): one
// branch, each case with compile-time indices, so that the transform stays in
// registers (a run-time index into it would move it to local memory).
template <class S> GB_HD void compose_axis(const S* PR, const S* Pt, int axis, S c, S s, X3<S>& out) {
  if (axis == 0) compose_axis_ax<0>(PR, Pt, c, s, out);
  else if (axis == 1) compose_axis_ax<1>(PR, Pt, c, s, out);
  else compose_axis_ax<2>(PR, Pt, c, s, out);
}
// Translation of a joint along a unit axis, composed on the right of a placement:
// liMi = placement * (I, d e_axis)  (prismatic joint, reference joint-prismatic.hpp:232-284,
// calc 700-704).
template <class S> GB_HD void compose_slide(const S* PR, const S* Pt, int axis, S d, X3<S>& out) {
#pragma unroll
  for (int r = 0; r < 3; ++r) {
#pragma unroll
    for (int k = 0; k < 3; ++k) out.R[3 * r + k] = PR[3 * r + k];
    out.t[r] = Pt[r] + PR[3 * r + axis] * d;
  }
}
// Free-flyer joint transform from (x, y, z, qx, qy, qz, qw) composed after a
// placement; quaternion to matrix as Eigen's Quaternion::matrix() (not normalised,
// reference joint-free-flyer.hpp:333-375).
template <class S> GB_HD void quat_matrix(S x, S y, S z, S w, S* R) {
  const S tx = S(2) * x, ty = S(2) * y, tz = S(2) * z;
  const S twx = tx * w, twy = ty * w, twz = tz * w;
  const S txx = tx * x, txy = ty * x, txz = tz * x;
  const S tyy = ty * y, tyz = tz * y, tzz = tz * z;
  R[0] = S(1) - (tyy + tzz); R[1] = txy - twz; R[2] = txz + twy;
  R[3] = txy + twz; R[4] = S(1) - (txx + tzz); R[5] = tyz - twx;
  R[6] = txz - twy; R[7] = tyz + twx; R[8] = S(1) - (txx + tyy);
}
template <class S> GB_HD void compose(const X3<S>& A, const X3<S>& B, X3<S>& C) {  // C = A * B
  S R[9], t[3];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) R[3 * r + c] = dot3(A.R[3 * r], B.R[c], A.R[3 * r + 1], B.R[3 + c], A.R[3 * r + 2], B.R[6 + c]);
  mv3(A.R, B.t, t);
#pragma unroll
  for (int k = 0; k < 9; ++k) C.R[k] = R[k];
#pragma unroll
  for (int k = 0; k < 3; ++k) C.t[k] = A.t[k] + t[k];
}
template <class S> GB_HD void act_motion(const X3<S>& M, const M6<S>& m, M6<S>& o) {
  S w[3], l[3], txw[3];
  mv3(M.R, m.v + 3, w);
  mv3(M.R, m.v, l);
  cross3(M.t, w, txw);
#pragma unroll
  for (int k = 0; k < 3; ++k) { o.v[k] = l[k] + txw[k]; o.v[3 + k] = w[k]; }
}
template <class S> GB_HD void actinv_motion(const X3<S>& M, const M6<S>& m, M6<S>& o) {
  S txw[3], d[3], l[3], w[3];
  cross3(M.t, m.v + 3, txw);
#pragma unroll
  for (int k = 0; k < 3; ++k) d[k] = m.v[k] - txw[k];
  mtv3(M.R, d, l);
  mtv3(M.R, m.v + 3, w);
#pragma unroll
  for (int k = 0; k < 3; ++k) { o.v[k] = l[k]; o.v[3 + k] = w[k]; }
}
template <class S> GB_HD void act_force(const X3<S>& M, const M6<S>& f, M6<S>& o) {
  S l[3], a[3], txl[3];
  mv3(M.R, f.v, l);
  mv3(M.R, f.v + 3, a);
  cross3(M.t, l, txl);
#pragma unroll
  for (int k = 0; k < 3; ++k) { o.v[k] = l[k]; o.v[3 + k] = a[k] + txl[k]; }
}
// motion cross v ^ w
template <class S> GB_HD void cross_motion(const M6<S>& v, const M6<S>& w, M6<S>& o) {
  S a[3], b[3], c[3];
  cross3(v.v, w.v + 3, a);
  cross3(v.v + 3, w.v, b);
  cross3(v.v + 3, w.v + 3, c);
#pragma unroll
  for (int k = 0; k < 3; ++k) { o.v[k] = a[k] + b[k]; o.v[3 + k] = c[k]; }
}
// force cross v x* f
template <class S> GB_HD void cross_force(const M6<S>& v, const M6<S>& f, M6<S>& o) {
  S a[3], b[3], c[3];
  cross3(v.v + 3, f.v, a);
  cross3(v.v + 3, f.v + 3, b);
  cross3(v.v, f.v, c);
#pragma unroll
  for (int k = 0; k < 3; ++k) { o.v[k] = a[k]; o.v[3 + k] = b[k] + c[k]; }
}

// --- rigid-body inertia (m, c, Ic) ------------------------------------------------------
template <class S> struct Iner { S m; S c[3]; S I[6]; };

// f = Y v  (reference spatial/inertia.hpp:729-735)
template <class S> GB_HD void iner_mul(const Iner<S>& Y, const M6<S>& v, M6<S>& f) {
  S cxw[3], l[3], a[3], cxl[3];
  cross3(Y.c, v.v + 3, cxw);
#pragma unroll
  for (int k = 0; k < 3; ++k) l[k] = Y.m * (v.v[k] - cxw[k]);
  sym3_mv(Y.I, v.v + 3, a);
  cross3(Y.c, l, cxl);
#pragma unroll
  for (int k = 0; k < 3; ++k) { f.v[k] = l[k]; f.v[3 + k] = a[k] + cxl[k]; }
}
// R S R^T for a packed symmetric S (the L-decomposition of
// reference spatial/symmetric3.hpp:552-600)
template <class S> GB_HD void sym3_rotate(const S* d, const S* R, S* out) {
  const S L00 = d[0] - d[5], L01 = d[1];
  const S L10 = d[1], L11 = d[2] - d[5];
  const S L20 = S(2) * d[3], L21 = d[4] + d[4];
  const S Y00 = dot3(R[3], L00, R[4], L10, R[5], L20);
  const S Y01 = dot3(R[3], L01, R[4], L11, R[5], L21);
  const S Y10 = dot3(R[6], L00, R[7], L10, R[8], L20);
  const S Y11 = dot3(R[6], L01, R[7], L11, R[8], L21);
  S s1 = dot2(Y00, R[0], Y01, R[1]);
  S s2 = dot2(Y00, R[3], Y01, R[4]);
  S s3v = dot2(Y10, R[0], Y11, R[1]);
  S s4 = dot2(Y10, R[3], Y11, R[4]);
  S s5 = dot2(Y10, R[6], Y11, R[7]);
  const S r0 = dot2(-R[0], d[4], R[1], d[3]);
  const S r1 = dot2(-R[3], d[4], R[4], d[3]);
  const S r2 = dot2(-R[6], d[4], R[7], d[3]);
  S s0 = L00 + L11 - s2 - s5;
  out[0] = s0 + d[5];
  out[1] = s1 + r2;
  out[2] = s2 + d[5];
  out[3] = s3v - r1;
  out[4] = s4 + r0;
  out[5] = s5 + d[5];
}
// M.act(Y) (reference spatial/inertia.hpp:873-880)
template <class S> GB_HD void iner_act(const X3<S>& M, const Iner<S>& Y, Iner<S>& o) {
  S rc[3], I[6];
  mv3(M.R, Y.c, rc);
  sym3_rotate(Y.I, M.R, I);
  o.m = Y.m;
#pragma unroll
  for (int k = 0; k < 3; ++k) o.c[k] = M.t[k] + rc[k];
#pragma unroll
  for (int k = 0; k < 6; ++k) o.I[k] = I[k];
}
// Ya += Yb (reference spatial/inertia.hpp:659-673)
template <class S> GB_HD void iner_add(Iner<S>& Ya, const Iner<S>& Yb, S eps) {
  const S mab = Ya.m + Yb.m;
  const S mab_inv = S(1) / (mab > eps ? mab : eps);
  S AB[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) AB[k] = Ya.c[k] - Yb.c[k];
  const S sa = Ya.m * mab_inv, sb = Yb.m * mab_inv;
#pragma unroll
  for (int k = 0; k < 3; ++k) Ya.c[k] = Ya.c[k] * sa + sb * Yb.c[k];
  const S al = Ya.m * Yb.m * mab_inv;
  const S x = AB[0], y = AB[1], z = AB[2];
  Ya.I[0] += Yb.I[0] + al * (y * y + z * z);
  Ya.I[1] += Yb.I[1] - al * x * y;
  Ya.I[2] += Yb.I[2] + al * (x * x + z * z);
  Ya.I[3] += Yb.I[3] - al * x * z;
  Ya.I[4] += Yb.I[4] - al * y * z;
  Ya.I[5] += Yb.I[5] + al * (x * x + y * y);
  Ya.m = mab;
}
// Y.matrix() in block form (reference spatial/inertia.hpp:481-491), evaluated
// in T: the parallel-axis terms m [c]x^2 must not be rounded to S before the
// Schur complement that cancels them.
template <class S, class T> GB_HD void iner_to_sym6(const Iner<S>& Y, Sym6<T>& M) {
  const T m = T(Y.m), x = T(Y.c[0]), y = T(Y.c[1]), z = T(Y.c[2]);
  M.A[0] = m; M.A[1] = T(0); M.A[2] = m; M.A[3] = T(0); M.A[4] = T(0); M.A[5] = m;
  // LINEAR,ANGULAR = -m [c]x
  M.B[0] = T(0);   M.B[1] = z * m;  M.B[2] = -y * m;
  M.B[3] = -z * m; M.B[4] = T(0);   M.B[5] = x * m;
  M.B[6] = y * m;  M.B[7] = -x * m; M.B[8] = T(0);
  M.D[0] = T(Y.I[0]) + m * (y * y + z * z);
  M.D[1] = T(Y.I[1]) - m * x * y;
  M.D[2] = T(Y.I[2]) + m * (x * x + z * z);
  M.D[3] = T(Y.I[3]) - m * x * z;
  M.D[4] = T(Y.I[4]) - m * y * z;
  M.D[5] = T(Y.I[5]) + m * (x * x + y * y);
}
// f = I x for a block-symmetric 6x6
template <class S, class X> GB_HD void sym6_mv(const Sym6<S>& I, const X* x, S* f) {
  const S xv[6] = {S(x[0]), S(x[1]), S(x[2]), S(x[3]), S(x[4]), S(x[5])};
  const S r0[6] = {I.A[0], I.A[1], I.A[3], I.B[0], I.B[1], I.B[2]};
  const S r1[6] = {I.A[1], I.A[2], I.A[4], I.B[3], I.B[4], I.B[5]};
  const S r2[6] = {I.A[3], I.A[4], I.A[5], I.B[6], I.B[7], I.B[8]};
  const S r3[6] = {I.B[0], I.B[3], I.B[6], I.D[0], I.D[1], I.D[3]};
  const S r4[6] = {I.B[1], I.B[4], I.B[7], I.D[1], I.D[2], I.D[4]};
  const S r5[6] = {I.B[2], I.B[5], I.B[8], I.D[3], I.D[4], I.D[5]};
  f[0] = dot6(r0, xv); f[1] = dot6(r1, xv); f[2] = dot6(r2, xv);
  f[3] = dot6(r3, xv); f[4] = dot6(r4, xv); f[5] = dot6(r5, xv);
}
// column k (0..5) of a block-symmetric 6x6
template <class S> GB_HD void sym6_col(const Sym6<S>& I, int k, S* u) {
  if (k < 3) {
    u[0] = I.A[s3(0, k)]; u[1] = I.A[s3(1, k)]; u[2] = I.A[s3(2, k)];
    u[3] = I.B[3 * k]; u[4] = I.B[3 * k + 1]; u[5] = I.B[3 * k + 2];
  } else {
    const int a = k - 3;
    u[0] = I.B[a]; u[1] = I.B[3 + a]; u[2] = I.B[6 + a];
    u[3] = I.D[s3(0, a)]; u[4] = I.D[s3(1, a)]; u[5] = I.D[s3(2, a)];
  }
}
// I -= w u^T  where w = alpha u  (rank-1 symmetric update)
template <class S> GB_HD void sym6_rank1_sub(Sym6<S>& I, const S* u, const S* w) {
  I.A[0] -= w[0] * u[0]; I.A[1] -= w[1] * u[0]; I.A[2] -= w[1] * u[1];
  I.A[3] -= w[2] * u[0]; I.A[4] -= w[2] * u[1]; I.A[5] -= w[2] * u[2];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) I.B[3 * r + c] -= w[r] * u[3 + c];
  I.D[0] -= w[3] * u[3]; I.D[1] -= w[4] * u[3]; I.D[2] -= w[4] * u[4];
  I.D[3] -= w[5] * u[3]; I.D[4] -= w[5] * u[4]; I.D[5] -= w[5] * u[5];
}
template <class S, class T> GB_HD void sym6_add(Sym6<S>& a, const Sym6<T>& b) {
#pragma unroll
  for (int k = 0; k < 6; ++k) { a.A[k] += S(b.A[k]); a.D[k] += S(b.D[k]); }
#pragma unroll
  for (int k = 0; k < 9; ++k) a.B[k] += S(b.B[k]);
}
template <class S, class T> GB_HD void sym6_convert(const Sym6<T>& b, Sym6<S>& a) {
#pragma unroll
  for (int k = 0; k < 6; ++k) { a.A[k] = cvt<S>(b.A[k]); a.D[k] = cvt<S>(b.D[k]); }
#pragma unroll
  for (int k = 0; k < 9; ++k) a.B[k] = cvt<S>(b.B[k]);
}
// R S R^T for a packed symmetric 3x3, straightforward two-stage product
template <class S> GB_HD void sym3_rrt(const S* s, const S* R, S* o) {
  S T[9];  // T = R S  (3x3)
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    T[3 * r + 0] = R[3 * r] * s[0] + R[3 * r + 1] * s[1] + R[3 * r + 2] * s[3];
    T[3 * r + 1] = R[3 * r] * s[1] + R[3 * r + 1] * s[2] + R[3 * r + 2] * s[4];
    T[3 * r + 2] = R[3 * r] * s[3] + R[3 * r + 1] * s[4] + R[3 * r + 2] * s[5];
  }
  o[0] = T[0] * R[0] + T[1] * R[1] + T[2] * R[2];
  o[1] = T[3] * R[0] + T[4] * R[1] + T[5] * R[2];
  o[2] = T[3] * R[3] + T[4] * R[4] + T[5] * R[5];
  o[3] = T[6] * R[0] + T[7] * R[1] + T[8] * R[2];
  o[4] = T[6] * R[3] + T[7] * R[4] + T[8] * R[5];
  o[5] = T[6] * R[6] + T[7] * R[7] + T[8] * R[8];
}
// X* I X^{-1} for X = (R, t) acting from the child to the parent frame:
// the effect of SE3actOn (reference algorithm/aba.hxx:22-76) written for the
// block-symmetric storage:
//   A' = R A R^T,  B'' = R B R^T,  B' = B'' - A' [t]x,
//   D' = R D R^T - B''^T [t]x + [t]x B'' - [t]x A' [t]x.
template <class S> GB_HD void sym6_transform(const Sym6<S>& I, const X3<S>& X, Sym6<S>& O) {
  const S* R = X.R;
  const S t0 = X.t[0], t1 = X.t[1], t2 = X.t[2];
  S A[6], Dd[6], B2[9];
  sym3_rrt(I.A, R, A);
  sym3_rrt(I.D, R, Dd);
  {  // B2 = R B R^T
    S T[9];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 3; ++c) T[3 * r + c] = R[3 * r] * I.B[c] + R[3 * r + 1] * I.B[3 + c] + R[3 * r + 2] * I.B[6 + c];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 3; ++c) B2[3 * r + c] = T[3 * r] * R[3 * c] + T[3 * r + 1] * R[3 * c + 1] + T[3 * r + 2] * R[3 * c + 2];
  }
  // P = A' [t]x  (3x3), columns: [t]x = [[0,-t2,t1],[t2,0,-t0],[-t1,t0,0]]
  S Af[9] = {A[0], A[1], A[3], A[1], A[2], A[4], A[3], A[4], A[5]};
  S P[9];
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    P[3 * r + 0] = Af[3 * r + 1] * t2 - Af[3 * r + 2] * t1;
    P[3 * r + 1] = Af[3 * r + 2] * t0 - Af[3 * r + 0] * t2;
    P[3 * r + 2] = Af[3 * r + 0] * t1 - Af[3 * r + 1] * t0;
  }
  // B' = B2 - P
#pragma unroll
  for (int k = 0; k < 9; ++k) O.B[k] = B2[k] - P[k];
  // Q = B2^T [t]x ; G = [t]x B2 = -(B2^T [t]x)^T... compute W = [t]x B2 - B2^T [t]x - [t]x P  (symmetric)
  // [t]x X (rows): row0 = t1 X.row2 - t2 X.row1 ; row1 = t2 X.row0 - t0 X.row2 ; row2 = t0 X.row1 - t1 X.row0
  S H[9];  // H = B2 - P/2 ... use E = B2 - P (=B'), then D' = Dd + [t]x E - B2^T [t]x
  // [t]x E
  S TE[9];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    TE[0 + c] = t1 * O.B[6 + c] - t2 * O.B[3 + c];
    TE[3 + c] = t2 * O.B[0 + c] - t0 * O.B[6 + c];
    TE[6 + c] = t0 * O.B[3 + c] - t1 * O.B[0 + c];
  }
  // B2^T [t]x : (B2^T [t]x)(r,c) = sum_k B2(k,r) [t]x(k,c)
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    H[3 * r + 0] = B2[3 * 1 + r] * t2 - B2[3 * 2 + r] * t1;
    H[3 * r + 1] = B2[3 * 2 + r] * t0 - B2[3 * 0 + r] * t2;
    H[3 * r + 2] = B2[3 * 0 + r] * t1 - B2[3 * 1 + r] * t0;
  }
  O.D[0] = Dd[0] + TE[0] - H[0];
  O.D[1] = Dd[1] + TE[3] - H[3];
  O.D[2] = Dd[2] + TE[4] - H[4];
  O.D[3] = Dd[3] + TE[6] - H[6];
  O.D[4] = Dd[4] + TE[7] - H[7];
  O.D[5] = Dd[5] + TE[8] - H[8];
#pragma unroll
  for (int k = 0; k < 6; ++k) O.A[k] = A[k];
}

// Inverse of a small SPD matrix by an LLT and two triangular solves
// (the PerformStYSInversion of reference multibody/joint/joint-common-operations.hpp:20-33).
// Returns false when a pivot is not > 0 (A not positive definite, or NaN).
template <class S, int N> GB_HD bool llt_inverse(const S* A, S* Ainv) {
  S L[N * N];
  bool ok = true;
#pragma unroll
  for (int k = 0; k < N * N; ++k) L[k] = A[k];
#pragma unroll
  for (int k = 0; k < N; ++k) {
    S x = L[N * k + k];
#pragma unroll
    for (int j = 0; j < k; ++j) x -= L[N * k + j] * L[N * k + j];
    ok = ok && x > S(0);
    x = sqrt(x);
    L[N * k + k] = x;
    const S ix = S(1) / x;
#pragma unroll
    for (int i = k + 1; i < N; ++i) {
      S s = L[N * i + k];
#pragma unroll
      for (int j = 0; j < k; ++j) s -= L[N * i + j] * L[N * k + j];
      L[N * i + k] = s * ix;
    }
  }
#pragma unroll
  for (int c = 0; c < N; ++c) {
    S y[N];
#pragma unroll
    for (int i = 0; i < N; ++i) {
      S s = (i == c) ? S(1) : S(0);
#pragma unroll
      for (int j = 0; j < i; ++j) s -= L[N * i + j] * y[j];
      y[i] = s / L[N * i + i];
    }
#pragma unroll
    for (int i = N - 1; i >= 0; --i) {
      S s = y[i];
#pragma unroll
      for (int j = i + 1; j < N; ++j) s -= L[N * j + i] * y[j];
      y[i] = s / L[N * i + i];
    }
#pragma unroll
    for (int i = 0; i < N; ++i) Ainv[N * i + c] = y[i];
  }
  return ok;
}

}  // namespace gb
