// Per-instance analytical derivatives (one thread = one configuration), host/device.
//
// computeRNEADerivatives (reference algorithm/rnea-derivatives.hxx:242-541) and
// the sweeps of computeABADerivatives (reference algorithm/aba-derivatives.hxx:22-453).
// Besides the per-joint arrays, these algorithms need 6 x nv column sets
// (J, dVdq, dAdq, dAdv, dFda, dFdq, dFdv, ...) and, for ABA, the Fcrb blocks of
// the Minv recursion: they live in a workspace laid out structure-of-arrays
// over the batch (element e of instance b at ws[e * batch + b]), so that the
// threads of a warp touch consecutive addresses.
//
// Kinematics run in a world frame as in the reference's derivative passes;
// the forward velocity / acceleration recursions are written directly in that
// frame (ov_i = ov_p + oMi.act(vJ)), which is the same quantity as the
// reference's local-then-transform evaluation up to rounding.  The frame of
// each root subtree is translated to its root joint (see world_forward).
#pragma once

#include "gb_dfloat.cuh"
#include "gb_dyn.cuh"

namespace gb {
template <> GB_HD dfloat eps_of<dfloat>() { return dfloat(1.1920929e-07f); }
}  // namespace gb

namespace gb {

template <class T> struct Ws {
  T* p;
  long st;
  GB_HD T& operator[](long e) const { return p[e * st]; }
};
// Who runs one configuration's sweeps.  Solo: one thread (every loop serial).
// LaneTeam<TS>: TS consecutive lanes of a warp; every lane runs the per-joint
// work (same values), the loops over matrix columns are split by column (rank
// c % TS owns column c in every pass, so a column's workspace entries are
// written and read by one lane; a walk up the ancestors gives every lane every
// TS-th one), and sync() orders the team's workspace
// accesses where one lane's store could otherwise overtake another lane's load
// of the same entry (before the stores of a read-modify-write, at the end of
// every joint).
struct Solo {
  static constexpr int size = 1;
  GB_HD int rank() const { return 0; }
  GB_HD int first(int c0) const { return c0; }  // the first column >= c0 this member owns
  GB_HD int advance(const int* next, int j) const { return next[j]; }  // size steps along a chain
  GB_HD void sync() const {}
};
#if defined(__CUDACC__)
template <int TS> struct LaneTeam {
  static_assert(TS > 1 && TS <= 32 && (TS & (TS - 1)) == 0, "a team is a power-of-two group of lanes");
  static constexpr int size = TS;
  int r;
  unsigned mask;  // the team's lanes
  __device__ explicit LaneTeam(int lane)
      : r(lane & (TS - 1)), mask(TS == 32 ? 0xffffffffu : ((1u << TS) - 1u) << (lane & ~(TS - 1))) {}
  __device__ int rank() const { return r; }
  __device__ int first(int c0) const { return c0 + ((r - c0) & (TS - 1)); }
  __device__ int advance(const int* next, int j) const {
#pragma unroll 1
    for (int s = 0; s < TS && j >= 0; ++s) j = next[j];
    return j;
  }
  __device__ void sync() const { __syncwarp(mask); }
};
#endif

template <class T> GB_HD void ld6(const Ws<T>& w, long e, T* x) {
#pragma unroll
  for (int k = 0; k < 6; ++k) x[k] = w[e + k];
}
template <class T, class U> GB_HD void st6(const Ws<T>& w, long e, const U* x) {
#pragma unroll
  for (int k = 0; k < 6; ++k) w[e + k] = T(x[k]);
}
// a . x + b . y for 6-vectors (one compensated accumulation for double-float)
template <class T> GB_HD T dot6x2(const T* a, const T* x, const T* b, const T* y) { return dot6(a, x) + dot6(b, y); }
GB_HD dfloat dot6x2(const dfloat* a, const dfloat* x, const dfloat* b, const dfloat* y) {
  dacc d;
  d.first(a[0], x[0]);
#pragma unroll
  for (int k = 1; k < 6; ++k) d.add(a[k], x[k]);
#pragma unroll
  for (int k = 0; k < 6; ++k) d.add(b[k], y[k]);
  return d.result();
}

// Element offsets of the per-instance workspace.
// "K" arrays are the world-frame forward kinematics (root-origin frame): oMi,
// ov, oa, oh, of, the link inertias oY and the joint columns J.  "C" arrays are
// the derivative column sets and the composite quantities of the backward
// pass.  The RNEA derivatives keep everything in region S (scalar S).  The
// ABA derivatives keep K and the Schur / Minv data in region SS (FP64) and C
// in region S: their first two sweeps feed the Schur complement and Minv,
// whose conditioning (cond(M) ~ 1e3-1e4 on the humanoid) would amplify FP32
// kinematics beyond 1e-5 in ddq_dq.
struct DerivLayout {
  // K (per joint / per dof)
  int oM, ov, oa, oh, of, oY, J;
  // C (per joint: composite inertia, its variation, force; per dof: column sets)
  int coY, doY, cof, cJ, dVdq, dAdq, dAdv, dFda, dFdq, dFdv, dYtJ;
  int dtq, dtv;  // nv x nv in region P (ABA only: dtau_dq, dtau_dv feeding -Minv * dtau)
  int nS, nP;
  // ABA only: region SS (articulated inertias and the bias u of the Schur
  // complement) and region K (kinematics, the Fcrb columns of the Minv
  // recursion, U Dinv and Dinv u); Minv itself (a packed upper triangle of
  // nv (nv + 1) / 2 values in K) has a region of its own
  int Ia, u, F0, Fslot, nslot, UD, Du;
  int nSS, nK;
};

// index of (r, c), r <= c, in a packed row-major upper triangle of an nv x nv matrix
GB_HD int upk(int nv, int r, int c) { return r * nv - (r * (r - 1)) / 2 + (c - r); }

// Fills the layout for a model; `aba` selects the ABA-derivative arrangement.
inline DerivLayout make_deriv_layout(int nj, int nv, int nslot, bool aba) {
  DerivLayout L;
  int oS = 0, oSS = 0, oK = 0;
  auto takeS = [&](int n) { const int r = oS; oS += n; return r; };
  auto takeSS = [&](int n) { const int r = oSS; oSS += n; return r; };
  auto takeKr = [&](int n) { const int r = oK; oK += n; return r; };
  auto takeK = [&](int n) { return aba ? takeKr(n) : takeS(n); };
  L.oM = takeK(12 * nj); L.ov = takeK(6 * nj); L.oa = takeK(6 * nj); L.oh = takeK(6 * nj); L.of = takeK(6 * nj);
  L.oY = takeK(10 * nj); L.J = takeK(6 * nv);
  L.coY = aba ? takeS(10 * nj) : L.oY;
  L.cof = aba ? takeS(6 * nj) : L.of;
  L.cJ = aba ? takeS(6 * nv) : L.J;
  L.doY = takeS(36 * nj);
  L.dVdq = takeS(6 * nv); L.dAdq = takeS(6 * nv); L.dAdv = takeS(6 * nv);
  L.dFda = takeS(6 * nv); L.dFdq = takeS(6 * nv); L.dFdv = takeS(6 * nv); L.dYtJ = aba ? 0 : takeS(6 * nv);
  L.nS = oS;
  L.dtq = 0;
  L.dtv = aba ? nv * nv : 0;
  L.nP = aba ? 2 * nv * nv : 0;
  L.Ia = aba ? takeSS(21 * nj) : 0;
  L.u = aba ? takeSS(nv) : 0;
  L.F0 = aba ? takeKr(6 * nv) : 0;
  L.nslot = nslot;
  L.Fslot = aba ? takeKr(6 * nv * nslot) : 0;
  L.UD = aba ? takeKr(6 * nv) : 0;
  L.Du = aba ? takeKr(nv) : 0;
  L.nSS = oSS;
  L.nK = oK;
  return L;
}

// load 6 values stored as S into the compute scalar T
template <class T, class S> GB_HD void ldc6(const Ws<S>& w, long e, T* x) {
#pragma unroll
  for (int k = 0; k < 6; ++k) x[k] = T(w[e + k]);
}
template <class T, class S> GB_HD void ldc_iner(const Ws<S>& w, long e, Iner<T>& Y) {
  Y.m = T(w[e]);
#pragma unroll
  for (int k = 0; k < 3; ++k) Y.c[k] = T(w[e + 1 + k]);
#pragma unroll
  for (int k = 0; k < 6; ++k) Y.I[k] = T(w[e + 4 + k]);
}
template <class T, class S> GB_HD void stc_iner(const Ws<S>& w, long e, const Iner<T>& Y) {
  w[e] = S(Y.m);
#pragma unroll
  for (int k = 0; k < 3; ++k) w[e + 1 + k] = S(Y.c[k]);
#pragma unroll
  for (int k = 0; k < 6; ++k) w[e + 4 + k] = S(Y.I[k]);
}
template <class S> GB_HD void ld_iner(const Ws<S>& w, long e, Iner<S>& Y) {
  Y.m = w[e];
#pragma unroll
  for (int k = 0; k < 3; ++k) Y.c[k] = w[e + 1 + k];
#pragma unroll
  for (int k = 0; k < 6; ++k) Y.I[k] = w[e + 4 + k];
}
template <class S> GB_HD void st_iner(const Ws<S>& w, long e, const Iner<S>& Y) {
  w[e] = Y.m;
#pragma unroll
  for (int k = 0; k < 3; ++k) w[e + 1 + k] = Y.c[k];
#pragma unroll
  for (int k = 0; k < 6; ++k) w[e + 4 + k] = Y.I[k];
}
template <class S> GB_HD void ld_x3(const Ws<S>& w, long e, X3<S>& X) {
#pragma unroll
  for (int k = 0; k < 9; ++k) X.R[k] = w[e + k];
#pragma unroll
  for (int k = 0; k < 3; ++k) X.t[k] = w[e + 9 + k];
}
template <class S> GB_HD void st_x3(const Ws<S>& w, long e, const X3<S>& X) {
#pragma unroll
  for (int k = 0; k < 9; ++k) w[e + k] = X.R[k];
#pragma unroll
  for (int k = 0; k < 3; ++k) w[e + 9 + k] = X.t[k];
}
// y = M x for a full row-major 6x6 stored at e
template <class T, class S> GB_HD void mat6_mv(const Ws<S>& w, long e, const T* x, T* y) {
#pragma unroll
  for (int r = 0; r < 6; ++r) {
    T row[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) row[k] = T(w[e + 6 * r + k]);
    y[r] = dot6(row, x);
  }
}
// y = M^T x
template <class T, class S> GB_HD void mat6_tmv(const Ws<S>& w, long e, const T* x, T* y) {
#pragma unroll
  for (int c = 0; c < 6; ++c) {
    T col[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) col[k] = T(w[e + 6 * k + c]);
    y[c] = dot6(col, x);
  }
}

// Y.variation(v) + the force-cross matrix of h (reference spatial/inertia.hpp:750-770,
// algorithm/rnea-derivatives.hxx:358-367), written row-major into M[36].
template <class S> GB_HD void variation_plus_fcross(const Iner<S>& Y, const S* v, const S* h, S* M) {
  const S m = Y.m;
  const S mvl[3] = {v[0] * m, v[1] * m, v[2] * m};
  const S mva[3] = {v[3] * m, v[4] * m, v[5] * m};
  const S* c = Y.c;
  // skewSquare(u, w) = w u^T - (u.w) I
  auto skewsq = [](const S* u, const S* w, S* C) {
    const S d = u[0] * w[0] + u[1] * w[1] + u[2] * w[2];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int cc = 0; cc < 3; ++cc) C[3 * r + cc] = w[r] * u[cc] - (r == cc ? d : S(0));
  };
  S B1[9], B2[9], Bla[9];
  skewsq(mva, c, B1);
  skewsq(c, mva, B2);
  // -skew(mv.lin) - skewSquare(mv.ang, c) + skewSquare(c, mv.ang)
  Bla[0] = -B1[0] + B2[0];          Bla[1] = mvl[2] - B1[1] + B2[1];  Bla[2] = -mvl[1] - B1[2] + B2[2];
  Bla[3] = -mvl[2] - B1[3] + B2[3]; Bla[4] = -B1[4] + B2[4];          Bla[5] = mvl[0] - B1[5] + B2[5];
  Bla[6] = mvl[1] - B1[6] + B2[6];  Bla[7] = -mvl[0] - B1[7] + B2[7]; Bla[8] = -B1[8] + B2[8];
  S D1[9], D2[9], Daa[9];
  skewsq(mvl, c, D1);
  skewsq(c, mvl, D2);
#pragma unroll
  for (int k = 0; k < 9; ++k) Daa[k] = -D1[k] - D2[k];
  const S x = c[0], y = c[1], z = c[2];
  const S L[9] = {Y.I[0] + m * (y * y + z * z), Y.I[1] - m * x * y, Y.I[3] - m * x * z,
                  Y.I[1] - m * x * y,           Y.I[2] + m * (x * x + z * z), Y.I[4] - m * y * z,
                  Y.I[3] - m * x * z,           Y.I[4] - m * y * z, Y.I[5] + m * (x * x + y * y)};
  const S* w = v + 3;
  // Daa -= L skew(w) ; Daa += skew(w) L
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    Daa[3 * r + 0] -= L[3 * r + 1] * w[2] - L[3 * r + 2] * w[1];
    Daa[3 * r + 1] -= L[3 * r + 2] * w[0] - L[3 * r + 0] * w[2];
    Daa[3 * r + 2] -= L[3 * r + 0] * w[1] - L[3 * r + 1] * w[0];
  }
#pragma unroll
  for (int cc = 0; cc < 3; ++cc) {
    Daa[0 + cc] += w[1] * L[6 + cc] - w[2] * L[3 + cc];
    Daa[3 + cc] += w[2] * L[0 + cc] - w[0] * L[6 + cc];
    Daa[6 + cc] += w[0] * L[3 + cc] - w[1] * L[0 + cc];
  }
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int cc = 0; cc < 3; ++cc) {
      M[6 * r + cc] = S(0);
      M[6 * r + 3 + cc] = Bla[3 * r + cc];
      M[6 * (3 + r) + cc] = Bla[3 * cc + r];
      M[6 * (3 + r) + 3 + cc] = Daa[3 * r + cc];
    }
  // force-cross matrix of h: addSkew(-h.lin) on (lin,ang) and (ang,lin), addSkew(-h.ang) on (ang,ang)
  auto add_skew = [&](const S* u, int r0, int c0) {
    M[6 * (r0 + 0) + c0 + 1] += u[2];
    M[6 * (r0 + 0) + c0 + 2] -= u[1];
    M[6 * (r0 + 1) + c0 + 0] -= u[2];
    M[6 * (r0 + 1) + c0 + 2] += u[0];
    M[6 * (r0 + 2) + c0 + 0] += u[1];
    M[6 * (r0 + 2) + c0 + 1] -= u[0];
  };
  add_skew(h, 0, 3);
  add_skew(h, 3, 0);
  add_skew(h + 3, 3, 3);
}

// world-frame joint columns J = oMi.act(S)
template <int NVJ, class S> GB_HD void joint_columns(int jt, const X3<S>& O, S (*Jc)[6]) {
  if constexpr (NVJ == 6) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const S w[3] = {O.R[k], O.R[3 + k], O.R[6 + k]};
      S tw[3];
      cross3(O.t, w, tw);
      Jc[k][0] = w[0]; Jc[k][1] = w[1]; Jc[k][2] = w[2]; Jc[k][3] = S(0); Jc[k][4] = S(0); Jc[k][5] = S(0);
      Jc[3 + k][0] = tw[0]; Jc[3 + k][1] = tw[1]; Jc[3 + k][2] = tw[2];
      Jc[3 + k][3] = w[0]; Jc[3 + k][4] = w[1]; Jc[3 + k][5] = w[2];
    }
  } else if constexpr (NVJ == 3) {  // spherical / planar: unit axes of the joint frame
#pragma unroll
    for (int k = 0; k < 3; ++k) world_axis_column(O, jt_col(jt, k), Jc[k]);
  } else {
    S w[3];
    axis_column(O, jt_axis(jt), w);
    if (jt_slides(jt)) {  // prismatic: (R e_axis, 0)
      Jc[0][0] = w[0]; Jc[0][1] = w[1]; Jc[0][2] = w[2]; Jc[0][3] = S(0); Jc[0][4] = S(0); Jc[0][5] = S(0);
    } else {  // revolute: (t x R e_axis, R e_axis)
      S tw[3];
      cross3(O.t, w, tw);
      Jc[0][0] = tw[0]; Jc[0][1] = tw[1]; Jc[0][2] = tw[2]; Jc[0][3] = w[0]; Jc[0][4] = w[1]; Jc[0][5] = w[2];
    }
  }
}

// motion cross v ^ w on raw 6-arrays
template <class S> GB_HD void mcross(const S* v, const S* w, S* o) {
  M6<S> a, b, c;
#pragma unroll
  for (int k = 0; k < 6; ++k) { a.v[k] = v[k]; b.v[k] = w[k]; }
  cross_motion(a, b, c);
#pragma unroll
  for (int k = 0; k < 6; ++k) o[k] = c.v[k];
}
template <class S> GB_HD void fcross(const S* v, const S* f, S* o) {
  M6<S> a, b, c;
#pragma unroll
  for (int k = 0; k < 6; ++k) { a.v[k] = v[k]; b.v[k] = f[k]; }
  cross_force(a, b, c);
#pragma unroll
  for (int k = 0; k < 6; ++k) o[k] = c.v[k];
}
template <class S> GB_HD void imul(const Iner<S>& Y, const S* v, S* f) {
  M6<S> a, b;
#pragma unroll
  for (int k = 0; k < 6; ++k) a.v[k] = v[k];
  iner_mul(Y, a, b);
#pragma unroll
  for (int k = 0; k < 6; ++k) f[k] = b.v[k];
}

// The world-frame forward pass shared by both derivative algorithms: oMi, ov,
// oa_gf, link inertia oY, oh, of, J, and for `with_derivs` the column sets
// dVdq / dAdq / dAdv and doYcrb.  `acc` selects the RNEA form (joint
// accelerations a given: oa_gf is the full acceleration minus gravity) or the
// ABA form (oa_gf holds only the velocity-product bias ov_p x ov_i, and of the
// gyroscopic force).
// One joint of the world-frame forward pass (NVJ: its degrees of freedom).
template <int NVJ, class S>
GB_HD void world_forward_joint(const MView& m, const DerivLayout& L, const Ws<S>& w, const In& q, const In& v,
                               const In* acc, bool with_derivs, const S* g, int i, const In* fext) {
  const int p = m.parent[i], jt = m.jtype[i], iv = m.idx_v[i];
  X3<S> X, O;
  joint_transform(m, i, q, X);
  if (p > 0) {
    X3<S> Op;
    ld_x3(w, L.oM + 12 * p, Op);
    compose(Op, X, O);
  } else {
    // The inertial frame of a root subtree is placed at its root joint: every
    // output is a joint-space quantity, invariant to a translation of that
    // frame, and world-frame inertias then carry no parallel-axis terms from a
    // distant floating base (which FP32 rounding would amplify).
    O = X;
    O.t[0] = O.t[1] = O.t[2] = S(0);
  }
  st_x3(w, L.oM + 12 * i, O);
  S Jc[NVJ][6];
  joint_columns<NVJ>(jt, O, Jc);
#pragma unroll 1
  for (int k = 0; k < NVJ; ++k) st6(w, L.J + 6 * (iv + k), Jc[k]);
  // ov_i = ov_p + oMi.act(vJ)
  S ovJ[6] = {0, 0, 0, 0, 0, 0}, ov[6], ovp[6] = {0, 0, 0, 0, 0, 0};
#pragma unroll 1
  for (int k = 0; k < NVJ; ++k) {
    const S vk = S(v[iv + k]);
#pragma unroll
    for (int r = 0; r < 6; ++r) ovJ[r] += Jc[k][r] * vk;
  }
  if (p > 0) ld6(w, L.ov + 6 * p, ovp);
#pragma unroll
  for (int r = 0; r < 6; ++r) ov[r] = ovp[r] + ovJ[r];
  st6(w, L.ov + 6 * i, ov);
  S oa[6];
  if (acc) {
    // oa_gf_i = oa_gf_p + oMi.act(S a) + ov_i x oMi.act(vJ)   (oa_gf_0 = -g)
    S oap[6], vx[6];
    if (p > 0) ld6(w, L.oa + 6 * p, oap);
    else
#pragma unroll
      for (int r = 0; r < 6; ++r) oap[r] = -g[r];
    mcross(ov, ovJ, vx);
#pragma unroll
    for (int r = 0; r < 6; ++r) oa[r] = oap[r] + vx[r];
#pragma unroll 1
  for (int k = 0; k < NVJ; ++k) {
      const S ak = S((*acc)[iv + k]);
#pragma unroll
      for (int r = 0; r < 6; ++r) oa[r] += Jc[k][r] * ak;
    }
  } else {
    // velocity-product bias ov_p x ov_i (aba.hxx:126-128)
    if (p > 0) mcross(ovp, ov, oa);
    else
#pragma unroll
      for (int r = 0; r < 6; ++r) oa[r] = S(0);
  }
  st6(w, L.oa + 6 * i, oa);
  Iner<S> Y, oY;
  load_inertia(m, i, Y);
  iner_act(O, Y, oY);
  st_iner(w, L.oY + 10 * i, oY);
  S oh[6], of[6], t6[6];
  imul(oY, ov, oh);
  fcross(ov, oh, t6);
  if (acc) {
    imul(oY, oa, of);
#pragma unroll
    for (int r = 0; r < 6; ++r) of[r] += t6[r];
  } else {
#pragma unroll
    for (int r = 0; r < 6; ++r) of[r] = t6[r];
  }
  if (fext) {  // of -= oMi.act(fext_i) (rnea-derivatives.hxx:596, aba-derivatives.hxx:513)
    M6<S> fe, fw;
    load_fext(m, *fext, i, fe.v);
    act_force(O, fe, fw);
#pragma unroll
    for (int r = 0; r < 6; ++r) of[r] -= fw.v[r];
  }
  st6(w, L.oh + 6 * i, oh);
  st6(w, L.of + 6 * i, of);
  if (!with_derivs) return;
  S oap[6];
  if (p > 0) ld6(w, L.oa + 6 * p, oap);
  else
#pragma unroll
    for (int r = 0; r < 6; ++r) oap[r] = -g[r];
#pragma unroll 1
  for (int k = 0; k < NVJ; ++k) {
    S dJ[6], dAdq[6], dAdv[6], dVdq[6];
    mcross(ov, Jc[k], dJ);
    mcross(oap, Jc[k], dAdq);
#pragma unroll
    for (int r = 0; r < 6; ++r) dAdv[r] = dJ[r];
    if (p > 0) {
      mcross(ovp, Jc[k], dVdq);
      S t[6];
      mcross(ovp, dVdq, t);
#pragma unroll
      for (int r = 0; r < 6; ++r) { dAdq[r] += t[r]; dAdv[r] += dVdq[r]; }
    } else {
#pragma unroll
      for (int r = 0; r < 6; ++r) dVdq[r] = S(0);
    }
    st6(w, L.dVdq + 6 * (iv + k), dVdq);
    st6(w, L.dAdq + 6 * (iv + k), dAdq);
    st6(w, L.dAdv + 6 * (iv + k), dAdv);
  }
  S dY[36];
  variation_plus_fcross(oY, ov, oh, dY);
#pragma unroll
  for (int k = 0; k < 36; ++k) w[L.doY + 36 * i + k] = dY[k];
}

// J3: the model has spherical / planar joints (their three-dof steps are compiled in only then,
// so that the kernels of the other models keep their registers)
template <class S, bool J3 = false>
GB_HD void world_forward(const MView& m, const DerivLayout& L, const Ws<S>& w, const In& q, const In& v,
                         const In* acc, bool with_derivs, const In* fext = nullptr) {
  const S* g = ModelScalar<S>::grav(m);
#pragma unroll 1
  for (int i = 1; i < m.nj; ++i) {
    if (m.jtype[i] == JT_FF) world_forward_joint<6, S>(m, L, w, q, v, acc, with_derivs, g, i, fext);
    else if (J3 && jt_three(m.jtype[i])) world_forward_joint<3, S>(m, L, w, q, v, acc, with_derivs, g, i, fext);
    else world_forward_joint<1, S>(m, L, w, q, v, acc, with_derivs, g, i, fext);
  }
}

// ------------------------------------------------------------------------------------------
// computeRNEADerivatives (rnea-derivatives.hxx:472-541).  Writes dtau_dq, dtau_dv, M (=dtau/da,
// upper or symmetric) and optionally tau; every other matrix entry is written as zero.
// ------------------------------------------------------------------------------------------
template <class S, bool J3 = false>
GB_HD void rnea_derivs_one(const MView& m, const DerivLayout& L, const Ws<S>& w, const In& q, const In& v,
                           const In& a, const Out& dq, const Out& dv, const Out& Mo, const Out* tau, bool symmetric,
                           bool zeroed, const In* fext = nullptr) {
  const int nv = m.nv;
  world_forward<S, J3>(m, L, w, q, v, &a, true, fext);
  if (!zeroed)  // otherwise the outputs arrive zero-filled: only non-zero entries are written
    for (int r = 0; r < nv * nv; ++r) { dq[r] = 0.0; dv[r] = 0.0; Mo[r] = 0.0; }
  const S eps = eps_of<S>();
  for (int i = m.nj - 1; i > 0; --i) {  // ComputeRNEADerivativesBackwardStep (hxx:361-460)
    const int p = m.parent[i], iv = m.idx_v[i], nst = m.nvsub[i];
    const int nvj = jt_nv(m.jtype[i]);
    Iner<S> oY;
    ld_iner(w, L.oY + 10 * i, oY);
    S of[6];
    ld6(w, L.of + 6 * i, of);
    for (int k = 0; k < nvj; ++k) {
      const int c = iv + k;
      S Jc[6], dFda[6], t[6], dFdq[6], dFdv[6], dYtJ[6], x[6];
      ld6(w, L.J + 6 * c, Jc);
      if (tau) (*tau)[c] = double(dot6(Jc, of) + m.arm_d[c] * 0.0);
      imul(oY, Jc, dFda);
      st6(w, L.dFda + 6 * c, dFda);
      ld6(w, L.dAdq + 6 * c, x);
      imul(oY, x, dFdq);
      if (p > 0) {
        ld6(w, L.dVdq + 6 * c, x);
        mat6_mv(w, L.doY + 36 * i, x, t);
#pragma unroll
        for (int r = 0; r < 6; ++r) dFdq[r] = t[r] + dFdq[r];
      }
      st6(w, L.dFdq + 6 * c, dFdq);
      mat6_tmv(w, L.doY + 36 * i, Jc, dYtJ);
      st6(w, L.dYtJ + 6 * c, dYtJ);
      ld6(w, L.dAdv + 6 * c, x);
      imul(oY, x, dFdv);
      mat6_mv(w, L.doY + 36 * i, Jc, t);
#pragma unroll
      for (int r = 0; r < 6; ++r) dFdv[r] = t[r] + dFdv[r];
      st6(w, L.dFdv + 6 * c, dFdv);
    }
    // row blocks: M(i, subtree), dtau_dq(i, subtree), dtau_dv(i, subtree)
    for (int r = 0; r < nvj; ++r) {
      S Jr[6];
      ld6(w, L.J + 6 * (iv + r), Jr);
      for (int c = iv; c < iv + nst; ++c) {
        S x[6];
        ld6(w, L.dFda + 6 * c, x);
        const S mval = dot6(Jr, x);
        Mo[(iv + r) * nv + c] = double(mval);
        if (symmetric) Mo[c * nv + iv + r] = double(mval);
        ld6(w, L.dFdq + 6 * c, x);
        dq[(iv + r) * nv + c] = double(dot6(Jr, x));
        ld6(w, L.dFdv + 6 * c, x);
        dv[(iv + r) * nv + c] = double(dot6(Jr, x));
      }
    }
    // column blocks below the joint: dtau_d*(subtree+, i)
    for (int k = 0; k < nvj; ++k) {
      const int c = iv + k;
      S dAdq[6], dVdq[6], dAdv[6], Jc[6];
      ld6(w, L.dAdq + 6 * c, dAdq);
      ld6(w, L.dVdq + 6 * c, dVdq);
      ld6(w, L.dAdv + 6 * c, dAdv);
      ld6(w, L.J + 6 * c, Jc);
      for (int r = iv + nvj; r < iv + nst; ++r) {
        S fa[6], yt[6];
        ld6(w, L.dFda + 6 * r, fa);
        ld6(w, L.dYtJ + 6 * r, yt);
        dq[r * nv + c] = double(dot6(fa, dAdq) + dot6(yt, dVdq));
        dv[r * nv + c] = double(dot6(fa, dAdv) + dot6(yt, Jc));
      }
      // dFdq += J x* of (kept for the ancestors' rows)
      S x[6], t[6];
      ld6(w, L.dFdq + 6 * c, x);
      fcross(Jc, of, t);
#pragma unroll
      for (int r = 0; r < 6; ++r) x[r] += t[r];
      st6(w, L.dFdq + 6 * c, x);
    }
    if (p > 0) {
      Iner<S> oYp;
      ld_iner(w, L.oY + 10 * p, oYp);
      iner_add(oYp, oY, eps);
      st_iner(w, L.oY + 10 * p, oYp);
      for (int k = 0; k < 36; ++k) w[L.doY + 36 * p + k] += w[L.doY + 36 * i + k];
      S ofp[6];
      ld6(w, L.of + 6 * p, ofp);
#pragma unroll
      for (int r = 0; r < 6; ++r) ofp[r] += of[r];
      st6(w, L.of + 6 * p, ofp);
    }
  }
  for (int k = 0; k < nv; ++k) {
    Mo[k * nv + k] += m.arm_d[k];
    if (tau) (*tau)[k] += m.arm_d[k] * a[k];
  }
}

// ---- translations of the reference point (world orientation kept) --------------------------
// motion about P -> about P + d: (v - d x w, w)
template <class S> GB_HD void shift_motion(const S* m, const S* d, S* o) {
  S dxw[3];
  cross3(d, m + 3, dxw);
#pragma unroll
  for (int k = 0; k < 3; ++k) { o[k] = m[k] - dxw[k]; o[3 + k] = m[3 + k]; }
}
// force about C -> about C - r (i.e. r = C - P for the new point P): (f, n + r x f)
template <class S> GB_HD void shift_force(const S* f, const S* r, S* o) {
  S rxf[3];
  cross3(r, f, rxf);
#pragma unroll
  for (int k = 0; k < 3; ++k) { o[k] = f[k]; o[3 + k] = f[3 + k] + rxf[k]; }
}
// force about the origin -> about point t: (f, n - t x f)
template <class S> GB_HD void shift_force_from_origin(const S* f, const S* t, S* o) {
  S txf[3];
  cross3(t, f, txf);
#pragma unroll
  for (int k = 0; k < 3; ++k) { o[k] = f[k]; o[3 + k] = f[3 + k] - txf[k]; }
}
// The composite inertia variation doY = sum over the subtree of shifted
// (Y.variation(v) + force-cross(h)) has a zero linear-linear block: each
// link's term does (its lin-lin block is zero) and a shift keeps that block.
// The operators below read and write only the other three blocks B (lin-ang),
// C (ang-lin) and D (ang-ang) of such a row-major 6x6.
template <class T, class S> GB_HD void op0_mv(const Ws<S>& w, long e, const T* x, T* y) {  // y = M x
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    y[r] = dot3(T(w[e + 6 * r + 3]), x[3], T(w[e + 6 * r + 4]), x[4], T(w[e + 6 * r + 5]), x[5]);
    T row[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) row[k] = T(w[e + 6 * (3 + r) + k]);
    y[3 + r] = dot6(row, x);
  }
}
template <class T, class S> GB_HD void op0_tmv(const Ws<S>& w, long e, const T* x, T* y) {  // y = M^T x
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    y[c] = dot3(T(w[e + 18 + c]), x[3], T(w[e + 24 + c]), x[4], T(w[e + 30 + c]), x[5]);
    T col[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) col[k] = T(w[e + 6 * k + 3 + c]);
    y[3 + c] = dot6(col, x);
  }
}
// dst += the operator at src (about C) re-expressed about P, r = C - P:
// [[0, B], [C, D + R B - C R]], R = [r]x
template <class T, class S, class Team = Solo>
GB_HD void op0_shift_add(const Ws<S>& w, long src, long dst, const T* r, const Team& tm = Team()) {
  T Bm[9], Cm[9], Dacc[9];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      Bm[3 * a + b] = T(w[src + 6 * a + 3 + b]);
      Cm[3 * a + b] = T(w[src + 6 * (3 + a) + b]);
      Dacc[3 * a + b] = T(w[src + 6 * (3 + a) + 3 + b]);
    }
#pragma unroll
  for (int b = 0; b < 3; ++b) {  // + R B (column b: r x B_b) and - C R (row a: C_a x r)
    Dacc[0 + b] += dot2(r[1], Bm[6 + b], -r[2], Bm[3 + b]);
    Dacc[3 + b] += dot2(r[2], Bm[0 + b], -r[0], Bm[6 + b]);
    Dacc[6 + b] += dot2(r[0], Bm[3 + b], -r[1], Bm[0 + b]);
  }
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    Dacc[3 * a + 0] -= dot2(Cm[3 * a + 1], r[2], -Cm[3 * a + 2], r[1]);
    Dacc[3 * a + 1] -= dot2(Cm[3 * a + 2], r[0], -Cm[3 * a + 0], r[2]);
    Dacc[3 * a + 2] -= dot2(Cm[3 * a + 0], r[1], -Cm[3 * a + 1], r[0]);
  }
  if constexpr (Team::size > 1) {  // every lane loads before any lane stores
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = 0; b < 3; ++b) {
        Bm[3 * a + b] = T(w[dst + 6 * a + 3 + b]) + Bm[3 * a + b];
        Cm[3 * a + b] = T(w[dst + 6 * (3 + a) + b]) + Cm[3 * a + b];
        Dacc[3 * a + b] = T(w[dst + 6 * (3 + a) + 3 + b]) + Dacc[3 * a + b];
      }
    tm.sync();
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = 0; b < 3; ++b) {
        w[dst + 6 * a + 3 + b] = S(Bm[3 * a + b]);
        w[dst + 6 * (3 + a) + b] = S(Cm[3 * a + b]);
        w[dst + 6 * (3 + a) + 3 + b] = S(Dacc[3 * a + b]);
      }
  } else {
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = 0; b < 3; ++b) {
        const long eb = dst + 6 * a + 3 + b, ec = dst + 6 * (3 + a) + b, ed = dst + 6 * (3 + a) + 3 + b;
        w[eb] = S(T(w[eb]) + Bm[3 * a + b]);
        w[ec] = S(T(w[ec]) + Cm[3 * a + b]);
        w[ed] = S(T(w[ed]) + Dacc[3 * a + b]);
      }
  }
}

// ------------------------------------------------------------------------------------------
// The four sweeps of computeABADerivatives (aba-derivatives.hxx:380-449): ddq,
// Minv (packed upper triangle, workspace zm) and dtau_dq / dtau_dv (at
// (q, v, ddq), workspace wp); the products -Minv dtau_dq, -Minv dtau_dv and the
// symmetric Minv output are written by a separate batched kernel.
// `slot[i]` is the Fcrb slot of joint i (a last child reuses its parent's slot).
//
// Scalar types: SS for the Schur complement Ia - U Dinv U^T with Dinv and the
// bias u (pass 2); K for the kinematics of pass 1, Minv and its Fcrb columns,
// U Dinv, Dinv u and the velocity / acceleration recursion of pass 3; T for
// the column sets of pass 3 and the backward pass 4, stored between the
// passes as S; P for dtau_dq / dtau_dv.  The quantities of passes 3-4 are in
// floating origins: every quantity of joint i is expressed about joint i's
// position t_i (world orientation), so that no reduced-precision value
// carries the lever arm of a distant origin; contributions move between
// joints by translation (shift_motion / shift_force / op0_shift_add).
// ------------------------------------------------------------------------------------------
template <class SS> GB_HD void ld_sym6(const Ws<SS>& zs, long e, Sym6<SS>& I6) {
#pragma unroll
  for (int k = 0; k < 6; ++k) { I6.A[k] = zs[e + k]; I6.D[k] = zs[e + 15 + k]; }
#pragma unroll
  for (int k = 0; k < 9; ++k) I6.B[k] = zs[e + 6 + k];
}
template <class SS> GB_HD void st_sym6(const Ws<SS>& zs, long e, const Sym6<SS>& I6) {
#pragma unroll
  for (int k = 0; k < 6; ++k) { zs[e + k] = I6.A[k]; zs[e + 15 + k] = I6.D[k]; }
#pragma unroll
  for (int k = 0; k < 9; ++k) zs[e + 6 + k] = I6.B[k];
}

// Minv(r, c) from the packed upper triangle (symmetric)
template <class K> GB_HD K minv_at(const Ws<K>& zm, int nv, int r, int c) {
  return r <= c ? zm[upk(nv, r, c)] : zm[upk(nv, c, r)];
}

// One joint of pass 2 (ComputeABADerivativesBackwardStep1, hxx:87-171) with
// NVJ degrees of freedom: the Schur complement in SS, the Minv rows and Fcrb
// columns in K.  Minv rows of the joint: the diagonal block Dinv and the
// columns of its subtree (-SDinv^T Fcrb); the columns right of the subtree are
// first written by pass 3.  In a lane team every lane runs the per-joint work
// (one lane and shuffles measured slower: the work is latency-bound, not
// FP64-throughput-bound) and the column loops are split over the team.
template <int NVJ, class K, class SS, class Team = Solo>
GB_HD void aba_derivs_pass2_joint(const MView& m, const DerivLayout& L, const Ws<K>& zk, const Ws<SS>& zs,
                                  const Ws<K>& zm, int i, const Team& tm = Team()) {
  const int nv = m.nv;
  const int p = m.parent[i], iv = m.idx_v[i], nst = m.nvsub[i];
  K Jk[NVJ][6];
#pragma unroll 1
  for (int k = 0; k < NVJ; ++k) ld6(zk, L.J + 6 * (iv + k), Jk[k]);
  Sym6<SS> Ia;
  SS U[NVJ][6];  // per joint dof k: U column
  SS Dinv[NVJ * NVJ];
  SS UD[NVJ][6];  // UDinv columns
  K UDk[NVJ][6];
  {
    ld_sym6(zs, L.Ia + 21 * i, Ia);
    K of[6];
    ld6(zk, L.of + 6 * i, of);
#pragma unroll 1
    for (int k = 0; k < NVJ; ++k) {
      SS Jc[6];
#pragma unroll
      for (int r = 0; r < 6; ++r) Jc[r] = SS(Jk[k][r]);
      const SS uk = zs[L.u + iv + k] - SS(dot6(Jk[k], of));
      tm.sync();  // every lane has read u before any lane writes it
      zs[L.u + iv + k] = uk;
      sym6_mv(Ia, Jc, U[k]);
    }
    {
      SS StU[NVJ * NVJ];
#pragma unroll 1
      for (int r = 0; r < NVJ; ++r)
#pragma unroll 1
        for (int c = 0; c < NVJ; ++c) {
          SS d = SS(Jk[r][0]) * U[c][0];
#pragma unroll
          for (int e = 1; e < 6; ++e) d += SS(Jk[r][e]) * U[c][e];
          StU[r * NVJ + c] = d;
        }
#pragma unroll 1
      for (int k = 0; k < NVJ; ++k) StU[k * NVJ + k] += SS(m.arm_d[iv + k]);
      if constexpr (NVJ > 1) {
        if (!llt_inverse<SS, NVJ>(StU, Dinv)) flag_numeric(m, NUM_PIVOT);
      } else {
        check_pivot(m, StU[0]);
        Dinv[0] = SS(1) / StU[0];
      }
    }
#pragma unroll 1
    for (int k = 0; k < NVJ; ++k)
#pragma unroll
      for (int r = 0; r < 6; ++r) {
        SS sum = U[0][r] * Dinv[k];
#pragma unroll 1
        for (int j = 1; j < NVJ; ++j) sum += U[j][r] * Dinv[j * NVJ + k];
        UD[k][r] = sum;
      }
    // U Dinv and Dinv u (u is final here: every child has been folded in) for pass 3, in K
#pragma unroll 1
    for (int k = 0; k < NVJ; ++k) {
#pragma unroll
      for (int r = 0; r < 6; ++r) UDk[k][r] = K(UD[k][r]);
      st6(zk, L.UD + 6 * (iv + k), UDk[k]);
      SS du = SS(0);
#pragma unroll 1
      for (int c = 0; c < NVJ; ++c) du += Dinv[k * NVJ + c] * zs[L.u + iv + c];
      zk[L.Du + iv + k] = K(du);
    }
#pragma unroll 1
    for (int r = 0; r < NVJ; ++r)
#pragma unroll 1
      for (int c = r; c < NVJ; ++c) zm[upk(nv, iv + r, iv + c)] = K(Dinv[r * NVJ + c]);
  }
  const int nch = nst - NVJ;
  if (nch > 0) {
    K SD[NVJ][6];  // SDinv columns = J Dinv
#pragma unroll 1
    for (int k = 0; k < NVJ; ++k)
#pragma unroll
      for (int r = 0; r < 6; ++r) {
        K sum = Jk[0][r] * K(Dinv[k]);
#pragma unroll 1
        for (int j = 1; j < NVJ; ++j) sum += Jk[j][r] * K(Dinv[j * NVJ + k]);
        SD[k][r] = sum;
      }
#pragma unroll 1
    for (int c = tm.first(iv + NVJ); c < iv + nst; c += Team::size) {
      K F[6];
      ld6(zk, L.F0 + 6 * c, F);
#pragma unroll 1
      for (int r = 0; r < NVJ; ++r) zm[upk(nv, iv + r, c)] = -dot6(SD[r], F);
    }
  }
  if (!(nch > 0 && p == 0)) {  // leaf: F = U Minv_rows; inner joint with a parent: F += U Minv_rows
    K Uk[NVJ][6];
#pragma unroll 1
    for (int k = 0; k < NVJ; ++k)
#pragma unroll
      for (int r = 0; r < 6; ++r) Uk[k][r] = K(U[k][r]);
#pragma unroll 1
    for (int c = tm.first(iv); c < iv + nst; c += Team::size) {
      K F[6] = {K(0), K(0), K(0), K(0), K(0), K(0)};
      if (nch > 0) ld6(zk, L.F0 + 6 * c, F);
#pragma unroll 1
      for (int k = 0; k < NVJ; ++k) {
        const K mk = minv_at(zm, nv, iv + k, c);
#pragma unroll
        for (int r = 0; r < 6; ++r) F[r] += Uk[k][r] * mk;
      }
      st6(zk, L.F0 + 6 * c, F);
    }
  }
  if (p > 0) {
    // Ia -= UDinv U^T (SS); the bias pa = of + Ia oa_gf + UDinv u, accumulated
    // into the parent, is not part of the Schur complement: formed in K
#pragma unroll 1
    for (int k = 0; k < NVJ; ++k) sym6_rank1_sub(Ia, U[k], UD[k]);
    K pa[6];
    {
      K oak[6];
      Sym6<K> Iak;
      sym6_convert(Ia, Iak);
      ld6(zk, L.oa + 6 * i, oak);
      sym6_mv(Iak, oak, pa);
    }
#pragma unroll 1
    for (int k = 0; k < NVJ; ++k) {
      const K uk = K(zs[L.u + iv + k]);
#pragma unroll
      for (int r = 0; r < 6; ++r) pa[r] += UDk[k][r] * uk;
    }
    K of[6], ofp[6];
    ld6(zk, L.of + 6 * i, of);
    ld6(zk, L.of + 6 * p, ofp);
#pragma unroll
    for (int r = 0; r < 6; ++r) ofp[r] += of[r] + pa[r];
    Sym6<SS> Ip;
    ld_sym6(zs, L.Ia + 21 * p, Ip);
    sym6_add(Ip, Ia);
    tm.sync();  // every lane has read the parent's entries before any lane writes them
    st6(zk, L.of + 6 * p, ofp);
    st_sym6(zs, L.Ia + 21 * p, Ip);
  }
}

template <class K, class SS, bool J3 = false, class Team = Solo>
GB_HD void aba_derivs_pass12(const MView& m, const DerivLayout& L, const Ws<K>& zk, const Ws<SS>& zs,
                             const Ws<K>& zm, const In& q, const In& v, const In& tau, const In* fext,
                             const Team& tm = Team()) {
  const int nv = m.nv;
  // ---- pass 1: ComputeABADerivativesForwardStep1 (hxx:22-80), kinematics in K;
  // external forces enter the bias force (hxx:513)
  world_forward<K, J3>(m, L, zk, q, v, nullptr, false, fext);
#pragma unroll 1
  for (int i = 1; i < m.nj; ++i) {  // Ia = oYcrb.matrix(), formed in K and stored in SS
    Iner<K> oY;
    ld_iner(zk, L.oY + 10 * i, oY);
    Sym6<K> Ik;
    iner_to_sym6(oY, Ik);
    Sym6<SS> I6;
    sym6_convert(Ik, I6);
    st_sym6(zs, L.Ia + 21 * i, I6);
  }
  for (int k = 0; k < nv; ++k) zs[L.u + k] = SS(tau[k]);
  for (int c = tm.first(0); c < nv; c += Team::size)
    for (int r = 0; r < 6; ++r) zk[L.F0 + 6 * c + r] = K(0);
  // ---- pass 2: ComputeABADerivativesBackwardStep1 (hxx:87-171)
#pragma unroll 1
  for (int i = m.nj - 1; i > 0; --i) {
    if (m.jtype[i] == JT_FF) aba_derivs_pass2_joint<6, K, SS>(m, L, zk, zs, zm, i, tm);
    else if (J3 && jt_three(m.jtype[i])) aba_derivs_pass2_joint<3, K, SS>(m, L, zk, zs, zm, i, tm);
    else aba_derivs_pass2_joint<1, K, SS>(m, L, zk, zs, zm, i, tm);
    tm.sync();
  }
}

// One joint of pass 3 (ComputeABADerivativesForwardStep2, hxx:178-270) with NVJ
// degrees of freedom.
// MINV: the Minv recursion only (computeMinverse's ComputeMinverseForwardStep2,
// aba.hxx:789-836): no velocity / acceleration recursion, no column sets.
template <int NVJ, class S, class T, class K, bool MINV = false, class Team = Solo>
GB_HD void aba_derivs_pass3_joint(const MView& m, const DerivLayout& L, const int* slot, const Ws<S>& w,
                                  const Ws<K>& zk, const Ws<K>& zm, const In& v, const Out* ddq_out, const K* gk,
                                  const In* fext, int i, const Team& tm = Team()) {
  const int nv = m.nv;
  const int p = m.parent[i], iv = m.idx_v[i], nst = m.nvsub[i];
  K ti[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) ti[k] = zk[L.oM + 12 * i + 9 + k];
  // joint columns about t_i: a revolute axis passes through t_i, a prismatic column has no
  // angular part (the same about every point); the root free-flyer sits at the origin
  K Jo[NVJ][6], Jc[NVJ][6];
#pragma unroll 1
  for (int k = 0; k < NVJ; ++k) {
    ld6(zk, L.J + 6 * (iv + k), Jo[k]);
#pragma unroll
    for (int r = 0; r < 6; ++r) Jc[k][r] = Jo[k][r];
  }
  if constexpr (NVJ == 1)
    if (!jt_slides(m.jtype[i])) Jc[0][0] = Jc[0][1] = Jc[0][2] = K(0);
  if constexpr (NVJ == 3)  // angular axes of a spherical / planar joint pass through t_i
#pragma unroll
    for (int k = 0; k < 3; ++k)
      if (jt_col(m.jtype[i], k) >= 3) Jc[k][0] = Jc[k][1] = Jc[k][2] = K(0);
  K ovp[6] = {K(0), K(0), K(0), K(0), K(0), K(0)}, oap[6], ov[6], oa[6];
  if constexpr (!MINV) {
    if (p > 0) {
      K r[3], x[6];
#pragma unroll
      for (int k = 0; k < 3; ++k) r[k] = ti[k] - zk[L.oM + 12 * p + 9 + k];
      ld6(zk, L.ov + 6 * p, x);
      shift_motion(x, r, ovp);
      ld6(zk, L.oa + 6 * p, x);
      shift_motion(x, r, oap);
    } else {
#pragma unroll
      for (int k = 0; k < 6; ++k) oap[k] = -gk[k];  // uniform field: invariant to the shift
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) ov[k] = ovp[k];
#pragma unroll 1
    for (int k = 0; k < NVJ; ++k) {
      const K vk = K(v[iv + k]);
#pragma unroll
      for (int r = 0; r < 6; ++r) ov[r] += Jc[k][r] * vk;
    }
    mcross(ovp, ov, oa);  // velocity-product bias (aba.hxx:126-128) + the parent's acceleration
#pragma unroll
    for (int k = 0; k < 6; ++k) oa[k] += oap[k];
    K dd[NVJ];
#pragma unroll 1
    for (int k = 0; k < NVJ; ++k) {
      K ud[6], udi[6];
      ld6(zk, L.UD + 6 * (iv + k), ud);
      shift_force_from_origin(ud, ti, udi);  // UDinv (a force about the root origin) about t_i
      dd[k] = zk[L.Du + iv + k] - dot6(udi, oa);
      if (ddq_out) {
        const double x = double(dd[k]);
        if (!finite_value(x)) flag_numeric(m, NUM_NONFINITE);
        (*ddq_out)[iv + k] = x;
      }
    }
#pragma unroll 1
    for (int k = 0; k < NVJ; ++k)
#pragma unroll
      for (int r = 0; r < 6; ++r) oa[r] += Jc[k][r] * dd[k];
    st6(zk, L.ov + 6 * i, ov);
    st6(zk, L.oa + 6 * i, oa);
  }
  // Minv rows of the joint: -= UDinv^T Fcrb[parent] (columns right of the
  // subtree start from zero); Fcrb[i] = J Minv_rows (+ Fcrb[parent]).  A
  // free-flyer is a root joint (no parent); a spherical / planar joint with a parent
  // updates its own NVJ x NVJ block first (every lane, all of it, before its columns).
  const long Fi = L.Fslot + 6L * nv * slot[i];
  const long Fp = p > 0 ? L.Fslot + 6L * nv * slot[p] : -1;
  if constexpr (NVJ == 3) {  // (a free-flyer has no parent: only three-dof joints take this)
   if (p > 0) {
    K ud[NVJ][6], Fo[NVJ][6], Bn[NVJ][NVJ];
#pragma unroll 1
    for (int k = 0; k < NVJ; ++k) {
      ld6(zk, L.UD + 6 * (iv + k), ud[k]);
      ld6(zk, Fp + 6 * (iv + k), Fo[k]);
    }
#pragma unroll 1
    for (int r = 0; r < NVJ; ++r)
#pragma unroll 1
      for (int c = 0; c < NVJ; ++c) Bn[r][c] = minv_at(zm, nv, iv + r, iv + c) - dot6(ud[r], Fo[c]);
    tm.sync();  // every lane has read the block before any lane writes it
#pragma unroll 1
    for (int c = tm.first(iv); c < iv + NVJ; c += Team::size) {
      K F[6];
#pragma unroll
      for (int r = 0; r < 6; ++r) F[r] = Fo[c - iv][r];
#pragma unroll 1
      for (int k = 0; k < NVJ; ++k) {
        if (iv + k <= c) zm[upk(nv, iv + k, c)] = Bn[k][c - iv];
#pragma unroll
        for (int r = 0; r < 6; ++r) F[r] += Jo[k][r] * Bn[k][c - iv];
      }
      st6(zk, Fi + 6 * c, F);
    }
#pragma unroll 1
    for (int c = tm.first(iv + NVJ); c < nv; c += Team::size) {
      K Fpc[6], F[6];
      ld6(zk, Fp + 6 * c, Fpc);
#pragma unroll
      for (int r = 0; r < 6; ++r) F[r] = Fpc[r];
#pragma unroll 1
      for (int k = 0; k < NVJ; ++k) {
        const long e = upk(nv, iv + k, c);
        const K mk = (c < iv + nst ? zm[e] : K(0)) - dot6(ud[k], Fpc);
        zm[e] = mk;
#pragma unroll
        for (int r = 0; r < 6; ++r) F[r] += Jo[k][r] * mk;
      }
      st6(zk, Fi + 6 * c, F);
    }
   }
  }
  if (NVJ == 3 && p > 0) {
  } else if (p > 0) {
    K udk[6];
    ld6(zk, L.UD + 6 * iv, udk);
#pragma unroll 1
    for (int c = tm.first(iv); c < nv; c += Team::size) {
      K Fpc[6];
      ld6(zk, Fp + 6 * c, Fpc);
      const long e = upk(nv, iv, c);
      const K mk = (c < iv + nst ? zm[e] : K(0)) - dot6(udk, Fpc);
      zm[e] = mk;
#pragma unroll
      for (int r = 0; r < 6; ++r) Fpc[r] += Jo[0][r] * mk;
      st6(zk, Fi + 6 * c, Fpc);
    }
  } else {  // a root joint: its rows are final; zero right of its subtree (another root's)
#pragma unroll 1
    for (int c = tm.first(iv); c < nv; c += Team::size) {
      K Fn[6] = {K(0), K(0), K(0), K(0), K(0), K(0)};
      if (c < iv + nst) {
#pragma unroll 1
        for (int k = 0; k < NVJ; ++k) {
          const K mk = minv_at(zm, nv, iv + k, c);
#pragma unroll
          for (int r = 0; r < 6; ++r) Fn[r] += Jo[k][r] * mk;
        }
      } else {
#pragma unroll 1
        for (int k = 0; k < NVJ; ++k) zm[upk(nv, iv + k, c)] = K(0);
      }
      st6(zk, Fi + 6 * c, Fn);
    }
  }
  if constexpr (MINV) return;
  // C quantities about t_i, computed in T and stored as S
  T ovs[6], ovps[6], oaps[6], oas[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) { ovs[k] = T(ov[k]); ovps[k] = T(ovp[k]); oaps[k] = T(oap[k]); oas[k] = T(oa[k]); }
#pragma unroll 1
  for (int k = 0; k < NVJ; ++k) {
    T J[6], dJ[6], dAdq[6], dAdv[6], dVdq[6];
#pragma unroll
    for (int r = 0; r < 6; ++r) J[r] = T(Jc[k][r]);
    mcross(ovs, J, dJ);
    mcross(oaps, J, dAdq);
#pragma unroll
    for (int r = 0; r < 6; ++r) dAdv[r] = dJ[r];
    if (p > 0) {
      mcross(ovps, J, dVdq);
      T t[6];
      mcross(ovps, dVdq, t);
#pragma unroll
      for (int r = 0; r < 6; ++r) { dAdq[r] += t[r]; dAdv[r] += dVdq[r]; }
    } else {
#pragma unroll
      for (int r = 0; r < 6; ++r) dVdq[r] = T(0);
    }
    st6(w, L.cJ + 6 * (iv + k), J);
    st6(w, L.dVdq + 6 * (iv + k), dVdq);
    st6(w, L.dAdq + 6 * (iv + k), dAdq);
    st6(w, L.dAdv + 6 * (iv + k), dAdv);
  }
  Iner<T> oY;
  {
    Iner<K> oYd;
    ld_iner(zk, L.oY + 10 * i, oYd);
    oY.m = T(oYd.m);
#pragma unroll
    for (int k = 0; k < 3; ++k) oY.c[k] = T(oYd.c[k] - ti[k]);
#pragma unroll
    for (int k = 0; k < 6; ++k) oY.I[k] = T(oYd.I[k]);
  }
  stc_iner(w, L.coY + 10 * i, oY);
  T oh[6], of[6], t6[6];
  imul(oY, ovs, oh);
  imul(oY, oas, of);
  fcross(ovs, oh, t6);
#pragma unroll
  for (int k = 0; k < 6; ++k) of[k] += t6[k];
  if (fext) {  // of -= oMi.act(fext_i) (hxx:529), about t_i: the rotation part only
    K R[9], fe[6];
#pragma unroll
    for (int k = 0; k < 9; ++k) R[k] = zk[L.oM + 12 * i + k];
    load_fext(m, *fext, i, fe);
#pragma unroll
    for (int h = 0; h < 6; h += 3)
#pragma unroll
      for (int r = 0; r < 3; ++r) of[h + r] -= T(R[3 * r] * fe[h] + R[3 * r + 1] * fe[h + 1] + R[3 * r + 2] * fe[h + 2]);
  }
  st6(w, L.cof + 6 * i, of);
  T dY[36];
  variation_plus_fcross(oY, ovs, oh, dY);
#pragma unroll
  for (int k = 0; k < 36; ++k)
    if (k >= 18 || k % 6 >= 3) w[L.doY + 36 * i + k] = S(dY[k]);  // the lin-lin block is zero
}

template <class S, class T, class K, bool MINV = false, bool J3 = false, class Team = Solo>
GB_HD void aba_derivs_pass3(const MView& m, const DerivLayout& L, const int* slot, const Ws<S>& w,
                            const Ws<K>& zk, const Ws<K>& zm, const In& v, const Out* ddq_out, const In* fext,
                            const Team& tm = Team()) {
  // ---- pass 3: ComputeABADerivativesForwardStep2 (hxx:178-270).  The
  // velocity / acceleration recursion runs in K in floating origins and
  // replaces ov / oa in K; the column sets, link inertia, momentum, force and
  // inertia variation of joint i are computed in T about t_i and stored as S.
  const K* gk = ModelScalar<K>::grav(m);
#pragma unroll 1
  for (int i = 1; i < m.nj; ++i) {
    if (m.jtype[i] == JT_FF) aba_derivs_pass3_joint<6, S, T, K, MINV>(m, L, slot, w, zk, zm, v, ddq_out, gk, fext, i, tm);
    else if (J3 && jt_three(m.jtype[i]))
      aba_derivs_pass3_joint<3, S, T, K, MINV>(m, L, slot, w, zk, zm, v, ddq_out, gk, fext, i, tm);
    else aba_derivs_pass3_joint<1, S, T, K, MINV>(m, L, slot, w, zk, zm, v, ddq_out, gk, fext, i, tm);
  }
}

// unroll factor of the row-block loop of pass 4 (independent iterations: more loads in flight)
#ifndef GB_P4_UNROLL
#define GB_P4_UNROLL 1
#endif
constexpr int kRowBlockUnroll = GB_P4_UNROLL;

// One joint of pass 4 with NVJ degrees of freedom (1: revolute or prismatic, 6: the root
// free-flyer, whose parent is the universe), so that every per-dof loop has a
// compile-time bound and the per-dof arrays stay in registers.
template <int NVJ, class S, class T, class K, class P, class Team = Solo>
GB_HD void aba_derivs_pass4_joint(const MView& m, const DerivLayout& L, const Ws<S>& w, const Ws<K>& zk,
                                  const Ws<P>& wp, int i, T eps, const Team& tm = Team()) {
  const int nv = m.nv;
  const int p = m.parent[i], iv = m.idx_v[i], nst = m.nvsub[i];
  K ti[3];  // t_i, loaded once (the dtau stores would otherwise force reloads)
#pragma unroll
  for (int k = 0; k < 3; ++k) ti[k] = zk[L.oM + 12 * i + 9 + k];
  auto offset_from = [&](int a, T* d) {  // t_a - t_i
#pragma unroll
    for (int k = 0; k < 3; ++k) d[k] = T(zk[L.oM + 12 * a + 9 + k] - ti[k]);
  };
  {
    Iner<T> oY;
    ldc_iner(w, L.coY + 10 * i, oY);
#pragma unroll 1
    for (int k = 0; k < NVJ; ++k) {
      const int c = iv + k;
      T Jc[6], x[6], t[6], y[6];
      ldc6(w, L.cJ + 6 * c, Jc);
      ldc6(w, L.dAdv + 6 * c, x);
      imul(oY, x, y);
      op0_mv(w, L.doY + 36 * i, Jc, t);
#pragma unroll
      for (int r = 0; r < 6; ++r) y[r] += t[r];
      st6(w, L.dFdv + 6 * c, y);  // dFdv
      ldc6(w, L.dAdq + 6 * c, x);
      imul(oY, x, y);
      if (p > 0) {
        ldc6(w, L.dVdq + 6 * c, x);
        op0_mv(w, L.doY + 36 * i, x, t);
#pragma unroll
        for (int r = 0; r < 6; ++r) y[r] += t[r];
      }
      st6(w, L.dFdq + 6 * c, y);  // dFdq
      imul(oY, Jc, y);
      st6(w, L.dFda + 6 * c, y);  // dFda
    }
  }
  // row block: dtau(i, subtree) = J_i^T dF_c, with dF_c moved from its joint's
  // position to t_i: J . (f_lin, f_ang + d x f_lin) = (J_lin + J_ang x d, J_ang) . f
#pragma unroll 1
  for (int r = 0; r < NVJ; ++r) {
    T Jr[6];
    ldc6(w, L.cJ + 6 * (iv + r), Jr);
#pragma unroll (kRowBlockUnroll)
    for (int c = tm.first(iv); c < iv + nst; c += Team::size) {
      T d[3], u[6], x[6];
      offset_from(m.dof_joint[c], d);
      cross3(Jr + 3, d, u);
#pragma unroll
      for (int k = 0; k < 3; ++k) { u[k] += Jr[k]; u[3 + k] = Jr[3 + k]; }
      ldc6(w, L.dFdv + 6 * c, x);
      wp[L.dtv + (iv + r) * nv + c] = P(dot6(u, x));
      ldc6(w, L.dFdq + 6 * c, x);
      wp[L.dtq + (iv + r) * nv + c] = P(dot6(u, x));
    }
  }
  {
    T of[6];
    ldc6(w, L.cof + 6 * i, of);
#pragma unroll 1
    for (int k = 0; k < NVJ; ++k) {
      const int c = iv + k;
      T Jc[6], x[6], t[6];
      ldc6(w, L.cJ + 6 * c, Jc);
      ldc6(w, L.dFdq + 6 * c, x);
      fcross(Jc, of, t);
#pragma unroll
      for (int r = 0; r < 6; ++r) x[r] += t[r];
      tm.sync();  // the row block's readers of dFdq (column owners) are done
      st6(w, L.dFdq + 6 * c, x);
    }
  }
  if (NVJ == 6 || p == 0) return;  // a free-flyer is a root joint: nothing above it
  // ancestor columns: motion quantities of ancestor j moved from t_j to t_i
#pragma unroll 1
  for (int r = 0; r < NVJ; ++r) {
    T fa[6], StdY[6];
    {
      T Jr[6];
      ldc6(w, L.dFda + 6 * (iv + r), fa);
      ldc6(w, L.cJ + 6 * (iv + r), Jr);
      op0_tmv(w, L.doY + 36 * i, Jr, StdY);
    }
    // f . (m_lin - d x m_ang, m_ang) = (f_lin, f_ang - f_lin x d) . m for the
    // motion m of ancestor j moved from t_j to t_i (d = t_i - t_j)
    // a team's lanes take every size-th ancestor in rounds (the body runs once per
    // round for the whole team)
    int j = m.pfr[iv];
#pragma unroll 1
    for (int s = 0; s < tm.rank() && j >= 0; ++s) j = m.pfr[j];
#pragma unroll 1
    for (; j >= 0; j = tm.advance(m.pfr, j)) {
      T d[3], fs[6], Ss[6], x[6], y[6];
      offset_from(m.dof_joint[j], d);  // t_j - t_i
#pragma unroll
      for (int k = 0; k < 3; ++k) d[k] = -d[k];  // t_i - t_j
      cross3(fa, d, fs + 3);
      cross3(StdY, d, Ss + 3);
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        fs[k] = fa[k];
        fs[3 + k] = fa[3 + k] - fs[3 + k];
        Ss[k] = StdY[k];
        Ss[3 + k] = StdY[3 + k] - Ss[3 + k];
      }
      ldc6(w, L.dAdq + 6 * j, x);
      ldc6(w, L.dVdq + 6 * j, y);
      wp[L.dtq + (iv + r) * nv + j] = P(dot6x2(fs, x, Ss, y));
      ldc6(w, L.dAdv + 6 * j, x);
      ldc6(w, L.cJ + 6 * j, y);
      wp[L.dtv + (iv + r) * nv + j] = P(dot6x2(fs, x, Ss, y));
    }
  }
  // accumulate into the parent, moved from t_i to t_p
  T rr[3];
  offset_from(p, rr);
#pragma unroll
  for (int k = 0; k < 3; ++k) rr[k] = -rr[k];  // t_i - t_p
  {
    Iner<T> oYp, oYs;
    ldc_iner(w, L.coY + 10 * i, oYs);
    ldc_iner(w, L.coY + 10 * p, oYp);
#pragma unroll
    for (int k = 0; k < 3; ++k) oYs.c[k] += rr[k];
    iner_add(oYp, oYs, eps);
    tm.sync();
    stc_iner(w, L.coY + 10 * p, oYp);
  }
  op0_shift_add(w, L.doY + 36 * i, L.doY + 36 * p, rr, tm);
  {
    T of[6], ofs[6], ofp[6];
    ldc6(w, L.cof + 6 * i, of);
    shift_force(of, rr, ofs);
    ldc6(w, L.cof + 6 * p, ofp);
#pragma unroll
    for (int r = 0; r < 6; ++r) ofp[r] += ofs[r];
    tm.sync();
    st6(w, L.cof + 6 * p, ofp);
  }
}

// ---- pass 4: ComputeABADerivativesBackwardStep2 (hxx:273-368), in T, floating
// origins: a joint's composite oY / doY / of are about its own position; a
// child adds its contributions moved to the parent's position.  Only the
// structurally non-zero entries of dtau_dq / dtau_dv (row k of column c for k
// an ancestor of c or in its subtree) are written: the products read no other.
template <class S, class T, class K, class P, bool J3 = false, class Team = Solo>
GB_HD void aba_derivs_pass4(const MView& m, const DerivLayout& L, const Ws<S>& w, const Ws<K>& zk,
                            const Ws<P>& wp, const Team& tm = Team()) {
  const T eps = eps_of<T>();
#pragma unroll 1
  for (int i = m.nj - 1; i > 0; --i) {
    if (m.jtype[i] == JT_FF) aba_derivs_pass4_joint<6, S, T, K, P>(m, L, w, zk, wp, i, eps, tm);
    else if (J3 && jt_three(m.jtype[i])) aba_derivs_pass4_joint<3, S, T, K, P>(m, L, w, zk, wp, i, eps, tm);
    else aba_derivs_pass4_joint<1, S, T, K, P>(m, L, w, zk, wp, i, eps, tm);
    tm.sync();
  }
}

// T3: arithmetic of the column sets in pass 3; T: arithmetic of pass 4
template <class S, class T3, class T, class K, class SS, class P, bool J3 = false>
GB_HD void aba_derivs_sweeps(const MView& m, const DerivLayout& L, const int* slot, const Ws<S>& w,
                             const Ws<K>& zk, const Ws<SS>& zs, const Ws<K>& zm, const Ws<P>& wp, const In& q,
                             const In& v, const In& tau, const Out* ddq_out, const In* fext = nullptr) {
  aba_derivs_pass12<K, SS, J3>(m, L, zk, zs, zm, q, v, tau, fext);
  aba_derivs_pass3<S, T3, K, false, J3>(m, L, slot, w, zk, zm, v, ddq_out, fext);
  aba_derivs_pass4<S, T, K, P, J3>(m, L, w, zk, wp);
}

}  // namespace gb
