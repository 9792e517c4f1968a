// Per-instance dynamics sweeps (one thread = one configuration), host/device.
//
// Template parameters:
//   S   -- scalar of the kinematic sweeps and spatial transforms
//          (double for the FP64 kernels, float for the mixed kernels);
//   SS  -- scalar of the articulated-inertia Schur complement
//          Ia - U D^-1 U^T, its D^-1 pivots and its accumulation into the
//          parent (double in both precisions);
//   CAP -- compile-time capacity (>= njoints and >= nv) of the per-joint
//          local arrays.
//
// The algorithms are the reference's (file:line on each function) written
// for the GPU: revolute joints use their axis-aligned motion subspace
// directly (U is a column of Ia, D a diagonal entry), articulated inertias
// are kept as block-symmetric 6x6 (21 entries), and the free-flyer is only
// allowed as the root joint (parent = universe), which every supported
// model satisfies and the host checks.
#pragma once

#include "gb_model.cuh"

namespace gb {

GB_HD void ssincos(double x, double* s, double* c) { sincos(x, s, c); }
GB_HD void ssincos(float x, float* s, float* c) { sincosf(x, s, c); }
// double-float angle: sine and cosine through FP64 (the reference for sincos_df below)
GB_HD void ssincos(dfloat x, dfloat* s, dfloat* c) {
  double sd, cd;
  sincos(double(x), &sd, &cd);
  *s = dfloat(sd);
  *c = dfloat(cd);
}

// 1 / n!, folded at compile time
constexpr double inv_fact(int n) { return n <= 1 ? 1.0 : inv_fact(n - 1) / n; }
// a double-float constant from an FP64 value known at compile time
#define GB_DF_CONST(x) dfloat(float(x), float((x) - double(float(x))), 0)

// Sine and cosine of an FP64 angle as double-floats with three FP64 operations: the
// Cody-Waite reduction r = x - k pi/2 (k the nearest integer to x 2/pi, found in FP32;
// pi/2 in two FP64 parts, two fused multiply-adds) and the split of r into a double-float.
// The rest runs on the FP32 pipe: the Taylor series of sin and cos on |r| <= pi/4 (the
// quotient can be off by one near a quadrant boundary, which only widens the interval a
// little), Horner steps in double-float for the terms above ~1e-9 and plain FP32 for the
// smaller ones, whose rounding stays below 1e-16; truncation after r^17 / 17! and
// r^16 / 16! leaves < 1e-17.  The quadrant (k mod 4) then selects +-sin / +-cos.
GB_HD void sincos_df(double x, dfloat* s, dfloat* c) {
  constexpr double kPio2Hi = 1.5707963267948966, kPio2Lo = 6.123233995736766e-17;  // pi/2 = hi + lo
  const float kf = rintf(narrow(x) * 0.636619772f);
  const double kd = widen(kf);
#if defined(__CUDA_ARCH__)
  const double r = __fma_rn(-kd, kPio2Lo, __fma_rn(-kd, kPio2Hi, x));
#else
  const double r = fma(-kd, kPio2Lo, fma(-kd, kPio2Hi, x));
#endif
  const dfloat rd(r);
  const dfloat z = rd * rd;
  const float zf = z.hi;
  // sin r = r + r z (-1/3! + z (1/5! + z (-1/7! + z (1/9! + z T(z))))), T in FP32
  const float ts = float(-inv_fact(11)) +
                   zf * (float(inv_fact(13)) + zf * (float(-inv_fact(15)) + zf * float(inv_fact(17))));
  dfloat hs = GB_DF_CONST(inv_fact(9)) + z * dfloat(ts);
  hs = GB_DF_CONST(-inv_fact(7)) + z * hs;
  hs = GB_DF_CONST(inv_fact(5)) + z * hs;
  hs = GB_DF_CONST(-inv_fact(3)) + z * hs;
  const dfloat sn = rd + (rd * z) * hs;
  // cos r = 1 + z (-1/2 + z (1/4! + z (-1/6! + z (1/8! + z (-1/10! + z U(z)))))), U in FP32
  const float uc = float(inv_fact(12)) + zf * (float(-inv_fact(14)) + zf * float(inv_fact(16)));
  dfloat hc = GB_DF_CONST(-inv_fact(10)) + z * dfloat(uc);
  hc = GB_DF_CONST(inv_fact(8)) + z * hc;
  hc = GB_DF_CONST(-inv_fact(6)) + z * hc;
  hc = GB_DF_CONST(inv_fact(4)) + z * hc;
  hc = dfloat(-0.5f) + z * hc;
  const dfloat cs = dfloat(1.0f) + z * hc;
  const int q = (int)kf & 3;
  const dfloat a = (q & 1) ? cs : sn, b = (q & 1) ? sn : cs;  // sin, cos of x up to signs
  *s = (q & 2) ? -a : a;
  *c = ((q + 1) & 2) ? -b : b;
}

// strided view of one instance's vector / matrix in the batch arrays
struct In {
  const double* p;
  long es;
  GB_HD double operator[](int k) const { return p[(long)k * es]; }
};
struct Out {
  double* p;
  long es;
  GB_HD double& operator[](int k) const { return p[(long)k * es]; }
};

template <class S> GB_HD S eps_of();
template <> GB_HD double eps_of<double>() { return 2.220446049250313e-16; }
template <> GB_HD float eps_of<float>() { return 1.1920929e-07f; }

// The configuration parameters of a one-dof joint: (sin, cos) of a revolute
// angle, (displacement, 1) of a prismatic joint.
template <class S> GB_HD void joint_params(int jt, S x, S* s, S* c) {
  if (jt_slides(jt)) {
    *s = x;
    *c = S(1);
  } else {
    ssincos(x, s, c);
  }
}
// joint_params from the FP64 configuration q[iq]; a double-float revolute angle takes
// sincos_df (no FP64 sincos); an unbounded revolute joint's (cos, sin) = (q[iq], q[iq + 1]) are
// taken as they are (JointModelRevoluteUnboundedTpl::calc, joint-revolute-unbounded.hpp:154-162)
template <class S> GB_HD void joint_params_q(int jt, const In& q, int iq, S* s, S* c) {
  if (jt_unbounded(jt)) {
    *c = S(q[iq]);
    *s = S(q[iq + 1]);
  } else {
    joint_params(jt, S(q[iq]), s, c);
  }
}
template <> GB_HD void joint_params_q<dfloat>(int jt, const In& q, int iq, dfloat* s, dfloat* c) {
  if (jt_unbounded(jt)) {
    *c = dfloat(q[iq]);
    *s = dfloat(q[iq + 1]);
  } else if (jt_slides(jt)) {
    *s = dfloat(q[iq]);
    *c = dfloat(1.0f);
  } else {
    sincos_df(q[iq], s, c);
  }
}
// liMi = placement * M_joint of a one-dof joint from its parameters
template <class S> GB_HD void compose_joint(const S* PR, const S* Pt, int jt, S c, S s, X3<S>& X) {
  if (jt_slides(jt)) compose_slide(PR, Pt, jt_axis(jt), s, X);
  else compose_axis(PR, Pt, jt_axis(jt), c, s, X);
}

// liMi = jointPlacements[i] * M_joint(q)   (rnea.hxx:60, joint calc:
// revolute joint-revolute.hpp:811-821, prismatic joint-prismatic.hpp:700-704,
// free-flyer joint-free-flyer.hpp:333-375, spherical joint-spherical.hpp:504-531 (the
// quaternion's matrix, no translation), planar joint-planar.hpp:586-609 (rotation about z
// with (cos, sin) = q[2:4], translation (q[0], q[1], 0)))
template <class S> GB_HD void joint_transform(const MView& m, int i, const In& q, X3<S>& X) {
  const S* P = ModelScalar<S>::place(m, i);
  const int jt = m.jtype[i], iq = m.idx_q[i];
  if (jt == JT_FF || jt_three(jt)) {
    X3<S> Pl, J;
    load_placement(m, i, Pl);
    if (jt == JT_FF) {
      quat_matrix(S(q[iq + 3]), S(q[iq + 4]), S(q[iq + 5]), S(q[iq + 6]), J.R);
      J.t[0] = S(q[iq]); J.t[1] = S(q[iq + 1]); J.t[2] = S(q[iq + 2]);
    } else if (jt == JT_SPH) {
      quat_matrix(S(q[iq]), S(q[iq + 1]), S(q[iq + 2]), S(q[iq + 3]), J.R);
      J.t[0] = J.t[1] = J.t[2] = S(0);
    } else {
      const S c = S(q[iq + 2]), s = S(q[iq + 3]);
      J.R[0] = c; J.R[1] = -s; J.R[2] = S(0);
      J.R[3] = s; J.R[4] = c; J.R[5] = S(0);
      J.R[6] = S(0); J.R[7] = S(0); J.R[8] = S(1);
      J.t[0] = S(q[iq]); J.t[1] = S(q[iq + 1]); J.t[2] = S(0);
    }
    compose(Pl, J, X);
  } else {
    S s, c;
    joint_params_q(jt, q, iq, &s, &c);
    compose_joint(P, P + 9, jt, c, s, X);
  }
}
// S * x for the joint (x = one value per dof)
template <class S> GB_HD void joint_motion(int jt, const In& x, int iv, M6<S>& o) {
  if (jt == JT_FF) {
#pragma unroll
    for (int k = 0; k < 6; ++k) o.v[k] = S(x[iv + k]);
  } else if (jt_three(jt)) {
    const S x0 = S(x[iv]), x1 = S(x[iv + 1]), x2 = S(x[iv + 2]);
    const int c2 = jt_col(jt, 2), c0 = jt_col(jt, 0);  // spherical 3, 4, 5; planar 0, 1, 5
#pragma unroll
    for (int k = 0; k < 6; ++k) o.v[k] = k == c0 ? x0 : k == c0 + 1 ? x1 : k == c2 ? x2 : S(0);
  } else {
    const S val = S(x[iv]);
    const int k0 = jt_sidx(jt);
#pragma unroll
    for (int k = 0; k < 6; ++k) o.v[k] = k == k0 ? val : S(0);
  }
}

// External force on joint i as the reference takes it: a force [linear; angular]
// expressed in the joint's own frame (fext[i], algorithm/rnea.hpp:60-79); fe
// holds njoints x 6 values per configuration, joint 0's are not read.  Inside the
// kernels an unaligned joint's frame is the joint frame turned by F (a rotation
// about the same origin, folded in at model build): f' = F^T f.
// The forces are per caller joint: an intermediate joint of an expanded translation joint
// takes none, the last one the caller joint's.
template <class S> GB_HD void load_fext(const MView& m, const In& fe, int i, S* f) {
  const int u = m.ujoint[i];
  if (u < 0) {
#pragma unroll
    for (int k = 0; k < 6; ++k) f[k] = S(0);
    return;
  }
  if (!m.fix_d) {
#pragma unroll
    for (int k = 0; k < 6; ++k) f[k] = S(fe[6 * u + k]);
    return;
  }
  const double* F = m.fix_d + 9 * i;
#pragma unroll
  for (int h = 0; h < 6; h += 3)
#pragma unroll
    for (int r = 0; r < 3; ++r)
      f[h + r] = S(F[r] * fe[6 * u + h] + F[3 + r] * fe[6 * u + h + 1] + F[6 + r] * fe[6 * u + h + 2]);
}

// ------------------------------------------------------------------------------------------
// RNEA (reference algorithm/rnea.hxx:24-161); with external forces fext
// (rnea.hxx:170-215: f_i -= fext_i after the forward step of joint i).
// ------------------------------------------------------------------------------------------
template <class S, int CAP>
GB_HD void rnea_one(const MView& m, const In& q, const In& v, const In& a, const Out& tau,
                    const In* fext = nullptr) {
  X3<S> X[CAP];
  M6<S> vel[CAP], acc[CAP], f[CAP];
  const S* g = ModelScalar<S>::grav(m);
  const S* arm = ModelScalar<S>::arm(m);
  for (int i = 1; i < m.nj; ++i) {
    const int p = m.parent[i], jt = m.jtype[i], iv = m.idx_v[i];
    joint_transform(m, i, q, X[i]);
    M6<S> vJ, aJ, t, ap;
    joint_motion(jt, v, iv, vJ);
    joint_motion(jt, a, iv, aJ);
    if (p > 0) {
      actinv_motion(X[i], vel[p], t);
#pragma unroll
      for (int k = 0; k < 6; ++k) vel[i].v[k] = vJ.v[k] + t.v[k];
      actinv_motion(X[i], acc[p], ap);
    } else {
      vel[i] = vJ;
      M6<S> mg;
#pragma unroll
      for (int k = 0; k < 6; ++k) mg.v[k] = -g[k];
      actinv_motion(X[i], mg, ap);
    }
    cross_motion(vel[i], vJ, t);
#pragma unroll
    for (int k = 0; k < 6; ++k) acc[i].v[k] = (t.v[k] + aJ.v[k]) + ap.v[k];
    Iner<S> Y;
    load_inertia(m, i, Y);
    M6<S> h, fa, fx;
    iner_mul(Y, vel[i], h);
    iner_mul(Y, acc[i], fa);
    cross_force(vel[i], h, fx);
#pragma unroll
    for (int k = 0; k < 6; ++k) f[i].v[k] = fa.v[k] + fx.v[k];
    if (fext) {
      S fe[6];
      load_fext(m, *fext, i, fe);
#pragma unroll
      for (int k = 0; k < 6; ++k) f[i].v[k] -= fe[k];
    }
  }
  for (int i = m.nj - 1; i > 0; --i) {
    const int p = m.parent[i], jt = m.jtype[i], iv = m.idx_v[i];
    if (jt == JT_FF) {
#pragma unroll
      for (int k = 0; k < 6; ++k) {
        const double t = double(f[i].v[k] + arm[iv + k] * S(a[iv + k]));
        if (!finite_value(t)) flag_numeric(m, NUM_NONFINITE);
        tau[iv + k] = t;
      }
    } else {
      const int nvj = jt_nv(jt);
      for (int k = 0; k < nvj; ++k) {
        const double t = double(pick6(f[i].v, jt_col(jt, k)) + arm[iv + k] * S(a[iv + k]));
        if (!finite_value(t)) flag_numeric(m, NUM_NONFINITE);
        tau[iv + k] = t;
      }
    }
    if (p > 0) {
      M6<S> fp;
      act_force(X[i], f[i], fp);
#pragma unroll
      for (int k = 0; k < 6; ++k) f[p].v[k] += fp.v[k];
    }
  }
}

// ------------------------------------------------------------------------------------------
// ABA, LOCAL convention (reference algorithm/aba.hxx:360-540); the revolute
// calc_aba is joint-revolute.hpp:823-834, the free-flyer one
// joint-free-flyer.hpp:377-391 with the LLT inverse of
// joint-common-operations.hpp:20-33.
//
// Per joint only what crosses passes is stored: the velocity, the joint
// transform (FP64 kernels) or its sine / cosine (mixed kernels, which rebuild
// the transform in FP32), UDinv and Dinv*u.  The articulated inertia, the bias
// force and the acceleration travel in registers from a joint to its first
// child (forward) / from a first child to its parent (backward); only joints
// with two or more children keep them in a branch slot.
// ------------------------------------------------------------------------------------------
//
// With external forces fext (aba.hxx:550-590): the bias force of joint i is
// v_i x* (I_i v_i) - fext_i.
// J3: the model has spherical / planar joints (their three-dof steps are compiled in only
// then, so that the kernels of the other models keep their registers).
template <class S, class SS, int CAP, bool J3 = false>
GB_HD void aba_one(const MView& m, const In& q, const In& v, const In& tau, const Out& ddq,
                   const In* fext = nullptr) {
  constexpr bool kStoreX = sizeof(S) == sizeof(double);
  constexpr int NB = CAP / 2 + 1;
  M6<S> vel[CAP];
  X3<S> Xs[kStoreX ? CAP : 1];
  S cs[kStoreX ? 1 : CAP][2];
  X3<S> Xff;  // root free-flyer transform
  S UDs[CAP][6];
  SS du[CAP];
  SS D6[36], UD6[36], u6[6];
  Sym6<SS> Islot[NB];
  M6<S> fslot[NB], aslot[NB];
  const S* g = ModelScalar<S>::grav(m);
  const double* arm = m.arm_d;
  auto transform = [&](int i, X3<S>& X) {
    if (kStoreX) {
      X = Xs[i];
    } else if (m.jtype[i] == JT_FF) {
      X = Xff;
    } else if (J3 && jt_three(m.jtype[i])) {  // rebuilt from q (spherical / planar)
      joint_transform(m, i, q, X);
    } else {
      const S* P = ModelScalar<S>::place(m, i);
      compose_joint(P, P + 9, m.jtype[i], cs[i][1], cs[i][0], X);
    }
  };
  // pass 1 (AbaLocalConventionForwardStep1, aba.hxx:360-399): transforms and velocities
  for (int i = 1; i < m.nj; ++i) {
    const int p = m.parent[i], jt = m.jtype[i], iv = m.idx_v[i];
    X3<S> X;
    if (jt == JT_FF) {
      joint_transform(m, i, q, X);
      Xff = X;
    } else if (J3 && jt_three(jt)) {
      joint_transform(m, i, q, X);
    } else {
      S sn, cn;
      joint_params_q(jt, q, m.idx_q[i], &sn, &cn);
      const S* P = ModelScalar<S>::place(m, i);
      compose_joint(P, P + 9, jt, cn, sn, X);
      if (!kStoreX) { cs[i][0] = sn; cs[i][1] = cn; }
    }
    if (kStoreX) Xs[kStoreX ? i : 0] = X;
    M6<S> vJ, t;
    joint_motion(jt, v, iv, vJ);
    if (p > 0) {
      actinv_motion(X, vel[p], t);
#pragma unroll
      for (int k = 0; k < 6; ++k) vel[i].v[k] = vJ.v[k] + t.v[k];
    } else {
      vel[i] = vJ;
    }
  }
  for (int b = 0; b < m.nbranch; ++b) {
#pragma unroll
    for (int k = 0; k < 6; ++k) { Islot[b].A[k] = SS(0); Islot[b].D[k] = SS(0); fslot[b].v[k] = S(0); }
#pragma unroll
    for (int k = 0; k < 9; ++k) Islot[b].B[k] = SS(0);
  }
  // pass 2 (AbaLocalConventionBackwardStep, aba.hxx:402-434)
  Sym6<SS> Icar;
  M6<S> fcar;
  for (int i = m.nj - 1; i > 0; --i) {
    const int p = m.parent[i], jt = m.jtype[i], iv = m.idx_v[i];
    X3<S> X;
    transform(i, X);
    Iner<S> Y;
    load_inertia(m, i, Y);
    Sym6<SS> Ia;
    load_sym6(m, i, Ia);
    M6<S> vJ, c, h, f;
    joint_motion(jt, v, iv, vJ);
    cross_motion(vel[i], vJ, c);
    iner_mul(Y, vel[i], h);
    cross_force(vel[i], h, f);
    if (fext) {
      S fe[6];
      load_fext(m, *fext, i, fe);
#pragma unroll
      for (int k = 0; k < 6; ++k) f.v[k] -= fe[k];
    }
    if (i + 1 < m.nj && m.parent[i + 1] == i) {  // first child's contribution, carried
      sym6_add(Ia, Icar);
#pragma unroll
      for (int k = 0; k < 6; ++k) f.v[k] += fcar.v[k];
    }
    const int bs = m.bslot[i];
    if (bs >= 0) {  // the other children's contributions
      sym6_add(Ia, Islot[bs]);
#pragma unroll
      for (int k = 0; k < 6; ++k) f.v[k] += fslot[bs].v[k];
    }
    if (jt == JT_FF) {  // root only: no parent update
      SS StU[36], Ifull[36];
#pragma unroll
      for (int k = 0; k < 6; ++k) {
        SS col[6];
        sym6_col(Ia, k, col);
#pragma unroll
        for (int r = 0; r < 6; ++r) Ifull[6 * r + k] = col[r];
      }
#pragma unroll
      for (int k = 0; k < 36; ++k) StU[k] = Ifull[k];
#pragma unroll
      for (int k = 0; k < 6; ++k) {
        StU[7 * k] += SS(arm[iv + k]);
        u6[k] = SS(tau[iv + k]) - cvt<SS>(f.v[k]);
      }
      if (!llt_inverse<SS, 6>(StU, D6)) flag_numeric(m, NUM_PIVOT);
#pragma unroll
      for (int r = 0; r < 6; ++r)
#pragma unroll
        for (int cc = 0; cc < 6; ++cc) {
          SS s = Ifull[6 * r] * D6[cc];
#pragma unroll
          for (int k = 1; k < 6; ++k) s += Ifull[6 * r + k] * D6[6 * k + cc];
          UD6[6 * r + cc] = s;
        }
      continue;
    }
    // the Schur-updated Ia and the bias pa = f + Ia c + U Dinv u moved to the parent
    auto to_parent = [&](const SS* UDu) {
      Sym6<S> Iaf, Ip;
      sym6_convert(Ia, Iaf);
      S t6[6];
      sym6_mv(Iaf, c.v, t6);
      M6<S> pa, fp;
#pragma unroll
      for (int k = 0; k < 6; ++k) pa.v[k] = f.v[k] + (t6[k] + cvt<S>(UDu[k]));
      sym6_transform(Iaf, X, Ip);
      act_force(X, pa, fp);
      if (p == i - 1) {  // i is the first child of p: processed next
        sym6_convert(Ip, Icar);
        fcar = fp;
      } else {
        const int pb = m.bslot[p];
        sym6_add(Islot[pb], Ip);
#pragma unroll
        for (int k = 0; k < 6; ++k) fslot[pb].v[k] += fp.v[k];
      }
    };
    if (J3 && jt_three(jt)) {  // calc_aba of the spherical (joint-spherical.hpp:572-586) and planar
                         // (joint-planar.hpp:643-661) joints: U = Ia S, Dinv = (S^T U + armature)^-1
      SS U[3][6], UD[3][6], StU[9], D3[9], u3[3];
      for (int k = 0; k < 3; ++k) {
        const int col = jt_col(jt, k);
        sym6_col(Ia, col, U[k]);
        u3[k] = SS(tau[iv + k]) - cvt<SS>(pick6(f.v, col));
      }
      for (int r = 0; r < 3; ++r)
        for (int cc = 0; cc < 3; ++cc) StU[3 * r + cc] = pick6(U[cc], jt_col(jt, r));
      for (int k = 0; k < 3; ++k) StU[4 * k] += SS(arm[iv + k]);
      if (!llt_inverse<SS, 3>(StU, D3)) flag_numeric(m, NUM_PIVOT);
      for (int k = 0; k < 3; ++k) {
#pragma unroll
        for (int r = 0; r < 6; ++r) {
          UD[k][r] = U[0][r] * D3[k] + U[1][r] * D3[3 + k] + U[2][r] * D3[6 + k];
          UDs[iv + k][r] = cvt<S>(UD[k][r]);
        }
        du[iv + k] = D3[3 * k] * u3[0] + D3[3 * k + 1] * u3[1] + D3[3 * k + 2] * u3[2];
      }
      if (p > 0) {
        SS UDu[6];
        for (int k = 0; k < 3; ++k) sym6_rank1_sub(Ia, U[k], UD[k]);
#pragma unroll
        for (int r = 0; r < 6; ++r) UDu[r] = UD[0][r] * u3[0] + UD[1][r] * u3[1] + UD[2][r] * u3[2];
        to_parent(UDu);
      }
      continue;
    }
    // revolute calc_aba (joint-revolute.hpp:823-834), prismatic (joint-prismatic.hpp:728-740)
    const int sx = jt_sidx(jt);
    const SS u = SS(tau[iv]) - cvt<SS>(pick6(f.v, sx));
    SS U[6], UD[6];
    sym6_col(Ia, sx, U);
    const SS Dpiv = pick6(U, sx) + SS(arm[iv]);
    check_pivot(m, Dpiv);
    const SS Dinv = SS(1) / Dpiv;
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      UD[k] = U[k] * Dinv;
      UDs[iv][k] = cvt<S>(UD[k]);
    }
    du[iv] = Dinv * u;
    if (p > 0) {
      sym6_rank1_sub(Ia, U, UD);
      SS UDu[6];
#pragma unroll
      for (int k = 0; k < 6; ++k) UDu[k] = UD[k] * u;
      to_parent(UDu);
    }
  }
  // pass 3 (AbaLocalConventionForwardStep2, aba.hxx:437-468)
  M6<S> acar;
  for (int i = 1; i < m.nj; ++i) {
    const int p = m.parent[i], jt = m.jtype[i], iv = m.idx_v[i];
    X3<S> X;
    transform(i, X);
    M6<S> ap, a, vJ, c;
    if (p == 0) {
#pragma unroll
      for (int k = 0; k < 6; ++k) ap.v[k] = -g[k];
    } else {
      ap = (p == i - 1) ? acar : aslot[m.bslot[p]];
    }
    actinv_motion(X, ap, a);
    joint_motion(jt, v, iv, vJ);
    cross_motion(vel[i], vJ, c);
#pragma unroll
    for (int k = 0; k < 6; ++k) a.v[k] += c.v[k];
    if (jt == JT_FF) {
      SS dd[6];
#pragma unroll
      for (int r = 0; r < 6; ++r) {
        SS s = D6[6 * r] * u6[0];
#pragma unroll
        for (int k = 1; k < 6; ++k) s += D6[6 * r + k] * u6[k];
        SS w = UD6[r] * cvt<SS>(a.v[0]);
#pragma unroll
        for (int k = 1; k < 6; ++k) w += UD6[6 * k + r] * cvt<SS>(a.v[k]);
        dd[r] = s - w;
        if (!finite_value(dd[r])) flag_numeric(m, NUM_NONFINITE);
        ddq[iv + r] = double(dd[r]);
      }
#pragma unroll
      for (int r = 0; r < 6; ++r) a.v[r] += cvt<S>(dd[r]);
    } else if (J3 && jt_three(jt)) {  // the three dofs from the same a
      SS dd[3];
      for (int k = 0; k < 3; ++k) {
        S w = UDs[iv + k][0] * a.v[0];
#pragma unroll
        for (int r = 1; r < 6; ++r) w += UDs[iv + k][r] * a.v[r];
        dd[k] = du[iv + k] - cvt<SS>(w);
        if (!finite_value(dd[k])) flag_numeric(m, NUM_NONFINITE);
        ddq[iv + k] = double(dd[k]);
      }
      for (int k = 0; k < 3; ++k) add_at6(a.v, jt_col(jt, k), cvt<S>(dd[k]));
    } else {
      S w = UDs[iv][0] * a.v[0];
#pragma unroll
      for (int k = 1; k < 6; ++k) w += UDs[iv][k] * a.v[k];
      const SS dd = du[iv] - cvt<SS>(w);
      if (!finite_value(dd)) flag_numeric(m, NUM_NONFINITE);
      ddq[iv] = double(dd);
      add_at6(a.v, jt_sidx(jt), cvt<S>(dd));
    }
    const int bs = m.bslot[i];
    if (bs >= 0) aslot[bs] = a;
    acar = a;
  }
}

// ------------------------------------------------------------------------------------------
// CRBA, WORLD convention (reference algorithm/crba.hxx:25-110, 498-548), writes
// M (upper or symmetric; every other entry zero) and adds the armature; then
// optionally the tree-sparse U D U^T factorisation of cholesky::decompose
// (reference algorithm/cholesky.hxx:18-62) in FP64.
// ------------------------------------------------------------------------------------------
// The world-frame column oMi.act(e_col) of a unit spatial axis col ([linear; angular]) of
// joint i's frame O: (R e_col, 0) for a linear axis, (t x R e_a, R e_a) for angular axis a.
template <class S> GB_HD void world_axis_column(const X3<S>& O, int col, S* Jc) {
  S w[3];
  axis_column(O, col < 3 ? col : col - 3, w);
  if (col < 3) {
    Jc[0] = w[0]; Jc[1] = w[1]; Jc[2] = w[2]; Jc[3] = S(0); Jc[4] = S(0); Jc[5] = S(0);
  } else {
    S tw[3];
    cross3(O.t, w, tw);
    Jc[0] = tw[0]; Jc[1] = tw[1]; Jc[2] = tw[2]; Jc[3] = w[0]; Jc[4] = w[1]; Jc[5] = w[2];
  }
}

template <class S, int CAP>
// `zeroed`: M (and U) arrive zero-filled (the device launcher clears them with
// one bandwidth-bound memset), so only the structurally non-zero entries are written.
GB_HD void crba_one(const MView& m, const In& q, const Out& M, bool symmetric, const Out* U, const Out* D,
                    bool zeroed) {
  const int nv = m.nv;
  X3<S> oM[CAP];
  Iner<S> Yc[CAP];
  S J[CAP][6], Ag[CAP][6];
  for (int i = 1; i < m.nj; ++i) {
    const int p = m.parent[i], jt = m.jtype[i], iv = m.idx_v[i];
    X3<S> X;
    joint_transform(m, i, q, X);
    if (p > 0) {
      compose(oM[p], X, oM[i]);
    } else {  // frame of the root subtree at its root joint (M is invariant to it)
      oM[i] = X;
      oM[i].t[0] = oM[i].t[1] = oM[i].t[2] = S(0);
    }
    const X3<S>& O = oM[i];
    if (jt == JT_FF) {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        S w[3] = {O.R[k], O.R[3 + k], O.R[6 + k]}, tw[3];
        J[iv + k][0] = w[0]; J[iv + k][1] = w[1]; J[iv + k][2] = w[2];
        J[iv + k][3] = S(0); J[iv + k][4] = S(0); J[iv + k][5] = S(0);
        cross3(O.t, w, tw);
        J[iv + 3 + k][0] = tw[0]; J[iv + 3 + k][1] = tw[1]; J[iv + 3 + k][2] = tw[2];
        J[iv + 3 + k][3] = w[0]; J[iv + 3 + k][4] = w[1]; J[iv + 3 + k][5] = w[2];
      }
    } else {
      for (int k = 0; k < jt_nv(jt); ++k) world_axis_column(O, jt_col(jt, k), J[iv + k]);
    }
    Iner<S> Y;
    load_inertia(m, i, Y);
    iner_act(O, Y, Yc[i]);
  }
  if (!zeroed)
    for (int r = 0; r < nv; ++r)
      for (int cidx = 0; cidx < nv; ++cidx) M[r * nv + cidx] = 0.0;
  const S eps = eps_of<S>();
  for (int i = m.nj - 1; i > 0; --i) {
    const int p = m.parent[i], iv = m.idx_v[i], nst = m.nvsub[i];
    const int nvj = jt_nv(m.jtype[i]);
    for (int k = 0; k < nvj; ++k) {
      M6<S> jc, ag;
#pragma unroll
      for (int r = 0; r < 6; ++r) jc.v[r] = J[iv + k][r];
      iner_mul(Yc[i], jc, ag);
#pragma unroll
      for (int r = 0; r < 6; ++r) Ag[iv + k][r] = ag.v[r];
    }
    for (int r = 0; r < nvj; ++r)
      for (int cidx = iv; cidx < iv + nst; ++cidx) {
        S s = J[iv + r][0] * Ag[cidx][0];
#pragma unroll
        for (int k = 1; k < 6; ++k) s += J[iv + r][k] * Ag[cidx][k];
        M[(iv + r) * nv + cidx] = double(s);
        if (symmetric) M[cidx * nv + iv + r] = double(s);
      }
    if (p > 0) iner_add(Yc[p], Yc[i], eps);
  }
  for (int k = 0; k < nv; ++k) M[k * nv + k] += m.arm_d[k];
  if (U == nullptr) return;
  // cholesky::decompose (cholesky.hxx:46-59), FP64 on the just-written M
  const Out& Uo = *U;
  const Out& Do = *D;
  if (zeroed)
    for (int r = 0; r < nv; ++r) Uo[r * nv + r] = 1.0;
  else
    for (int r = 0; r < nv; ++r)
      for (int cidx = 0; cidx < nv; ++cidx) Uo[r * nv + cidx] = (r == cidx) ? 1.0 : 0.0;
  for (int j = nv - 1; j >= 0; --j) {
    const int NVT = m.nsfr[j] - 1;
    double s = 0.0;
    for (int k = 0; k < NVT; ++k) {
      const double ujk = Uo[j * nv + j + 1 + k];
      s += ujk * (ujk * Do[j + 1 + k]);
    }
    const double Dj = M[j * nv + j] - s;
    Do[j] = Dj;
    check_pivot(m, Dj);
    const double Dinv = 1.0 / Dj;
    for (int ii = m.pfr[j]; ii >= 0; ii = m.pfr[ii]) {
      double w = 0.0;
      for (int k = 0; k < NVT; ++k) w += Uo[ii * nv + j + 1 + k] * (Uo[j * nv + j + 1 + k] * Do[j + 1 + k]);
      Uo[ii * nv + j] = (M[ii * nv + j] - w) * Dinv;
    }
  }
}

// ------------------------------------------------------------------------------------------
// forwardKinematics (reference algorithm/kinematics.hxx: ZeroStep 42-77, FirstStep 105-178,
// SecondStep 188-272): oMi (R row-major, then t; joint 0 the identity) and, when v (and a)
// are given, the joint-frame spatial velocities (and accelerations, without gravity).
// computeJointJacobians (reference algorithm/jacobian.hxx:17-95): J = [oMi.act(S_i)],
// 6 x nv column-major about the world origin.
// ------------------------------------------------------------------------------------------
template <class S>
GB_HD void store_placement(const Out& o, int i, const X3<S>& X) {
#pragma unroll
  for (int k = 0; k < 9; ++k) o[12 * i + k] = double(X.R[k]);
#pragma unroll
  for (int k = 0; k < 3; ++k) o[12 * i + 9 + k] = double(X.t[k]);
}
template <class S> GB_HD void store_placement_fixed(const MView& m, const Out& o, int i, const X3<S>& X);
template <class S> GB_HD void store_motion_fixed(const MView& m, const Out& o, int i, const M6<S>& x);
// the joint-i output written at slot u of the caller's joints
template <class S>
GB_HD void store_placement_fixed_at(const MView& m, const Out& o, int i, int u, const X3<S>& X) {
  store_placement_fixed(m, Out{o.p + (long)12 * (u - i) * o.es, o.es}, i, X);
}
template <class S>
GB_HD void store_motion_fixed_at(const MView& m, const Out& o, int i, int u, const M6<S>& x) {
  store_motion_fixed(m, Out{o.p + (long)6 * (u - i) * o.es, o.es}, i, x);
}
// The frame of an unaligned joint i is frame_i F_i inside the kernels (the model
// build folds the axis into the placements): the outputs map back with
// oMi = oMi' F^T and a joint-frame motion m = F m'.
template <class S>
GB_HD void store_placement_fixed(const MView& m, const Out& o, int i, const X3<S>& X) {
  if (!m.fix_d) {
    store_placement(o, i, X);
    return;
  }
  const double* F = m.fix_d + 9 * i;
  X3<S> Y;
#pragma unroll
  for (int r = 0; r < 3; ++r) {
#pragma unroll
    for (int c = 0; c < 3; ++c)
      Y.R[3 * r + c] = X.R[3 * r] * S(F[3 * c]) + X.R[3 * r + 1] * S(F[3 * c + 1]) + X.R[3 * r + 2] * S(F[3 * c + 2]);
    Y.t[r] = X.t[r];
  }
  store_placement(o, i, Y);
}
template <class S>
GB_HD void store_motion_fixed(const MView& m, const Out& o, int i, const M6<S>& x) {
  if (!m.fix_d) {
#pragma unroll
    for (int k = 0; k < 6; ++k) o[6 * i + k] = double(x.v[k]);
    return;
  }
  const double* F = m.fix_d + 9 * i;
#pragma unroll
  for (int h = 0; h < 6; h += 3)
#pragma unroll
    for (int r = 0; r < 3; ++r)
      o[6 * i + h + r] =
          double(S(F[3 * r]) * x.v[h] + S(F[3 * r + 1]) * x.v[h + 1] + S(F[3 * r + 2]) * x.v[h + 2]);
}
template <class S, int CAP>
GB_HD void fk_one(const MView& m, const In& q, const In* v, const In* a, const Out& oMi, const Out* vo,
                  const Out* ao) {
  X3<S> oM[CAP];
  M6<S> vel[CAP], acc[CAP];
  {
    X3<S> I;
#pragma unroll
    for (int k = 0; k < 9; ++k) I.R[k] = (k == 0 || k == 4 || k == 8) ? S(1) : S(0);
    I.t[0] = I.t[1] = I.t[2] = S(0);
    store_placement(oMi, 0, I);
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      if (vo) (*vo)[k] = 0.0;
      if (ao) (*ao)[k] = 0.0;
    }
  }
  for (int i = 1; i < m.nj; ++i) {
    const int p = m.parent[i], jt = m.jtype[i], iv = m.idx_v[i];
    X3<S> X;
    joint_transform(m, i, q, X);
    if (p > 0) compose(oM[p], X, oM[i]);
    else oM[i] = X;
    const int u = m.ujoint[i];  // outputs per caller joint (-1: inside an expanded translation joint)
    if (u > 0) store_placement_fixed_at(m, oMi, i, u, oM[i]);
    if (!v) continue;
    M6<S> vJ, t;
    joint_motion(jt, *v, iv, vJ);
    if (p > 0) {
      actinv_motion(X, vel[p], t);
#pragma unroll
      for (int k = 0; k < 6; ++k) vel[i].v[k] = vJ.v[k] + t.v[k];
    } else {
      vel[i] = vJ;
    }
    if (u > 0) store_motion_fixed_at(m, *vo, i, u, vel[i]);
    if (!a) continue;
    M6<S> aJ, ap;
    joint_motion(jt, *a, iv, aJ);
    cross_motion(vel[i], vJ, t);
    if (p > 0) actinv_motion(X, acc[p], ap);
#pragma unroll
    for (int k = 0; k < 6; ++k) acc[i].v[k] = p > 0 ? (aJ.v[k] + t.v[k]) + ap.v[k] : aJ.v[k] + t.v[k];
    if (u > 0) store_motion_fixed_at(m, *ao, i, u, acc[i]);
  }
}
template <class S, int CAP>
GB_HD void jacobians_one(const MView& m, const In& q, const Out& J) {
  X3<S> oM[CAP];
  for (int i = 1; i < m.nj; ++i) {
    const int p = m.parent[i], jt = m.jtype[i], iv = m.idx_v[i];
    X3<S> X;
    joint_transform(m, i, q, X);
    if (p > 0) compose(oM[p], X, oM[i]);
    else oM[i] = X;
    const int nvj = jt_nv(jt);
    for (int k = 0; k < nvj; ++k) {
      M6<S> sk, c;
      const int col = jt_col(jt, k);
#pragma unroll
      for (int r = 0; r < 6; ++r) sk.v[r] = r == col ? S(1) : S(0);
      act_motion(oM[i], sk, c);
#pragma unroll
      for (int r = 0; r < 6; ++r) J[6 * (iv + k) + r] = double(c.v[r]);
    }
  }
}

// ------------------------------------------------------------------------------------------
// integrate(q, v): revolute and prismatic joints q + v; free-flyer through the SE(3)
// exponential with the quaternion renormalised to first order (reference
// multibody/liegroup/special-euclidean.hpp:660-699, spatial/explog-quaternion.hpp:20-147,
// math/quaternion.hpp:90-111).  Always FP64.
// ------------------------------------------------------------------------------------------
// exp3 of an angular velocity w as a quaternion (x, y, z, w) (spatial/explog-quaternion.hpp:20-60)
GB_HD void exp3_quaternion(const double* w, double* e) {
  const double eps = eps_of<double>();
  const double ts_prec = 1.2207031250000000e-04;  // eps^(1/4)
  const double s2 = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
  const double th = sqrt(s2 + eps * eps);
  if (s2 > ts_prec) {
    double sh, ch;
    sincos(0.5 * th, &sh, &ch);
    for (int k = 0; k < 3; ++k) e[k] = sh * (w[k] / th);
    e[3] = ch;
  } else {
    const double t22 = s2 / 4.0;
    const double cc = 0.5 * (1.0 - t22 / 6.0 + t22 * t22 / 120.0);
    for (int k = 0; k < 3; ++k) e[k] = cc * w[k];
    e[3] = 1.0 - t22 / 2.0 + t22 * t22 / 24.0;
  }
}
// spherical: q * exp3(v), first-order normalised (liegroup/special-orthogonal.hpp:467-481);
// planar: the SE(2) exponential of (vx, vy, w) in the body frame composed on the right
// (liegroup/special-euclidean.hpp:61-90, 289-306)
GB_HD void integrate_three(int jt, const In& q, const In& v, int iq, int iv, const Out& qo) {
  if (jt == JT_SPH) {
    const double qq[4] = {q[iq], q[iq + 1], q[iq + 2], q[iq + 3]};
    const double w[3] = {v[iv], v[iv + 1], v[iv + 2]};
    double e[4], r[4];
    exp3_quaternion(w, e);
    r[3] = qq[3] * e[3] - qq[0] * e[0] - qq[1] * e[1] - qq[2] * e[2];
    r[0] = qq[3] * e[0] + qq[0] * e[3] + qq[1] * e[2] - qq[2] * e[1];
    r[1] = qq[3] * e[1] + qq[1] * e[3] + qq[2] * e[0] - qq[0] * e[2];
    r[2] = qq[3] * e[2] + qq[2] * e[3] + qq[0] * e[1] - qq[1] * e[0];
    const double alpha = (3.0 - (r[0] * r[0] + r[1] * r[1] + r[2] * r[2] + r[3] * r[3])) / 2.0;
    for (int k = 0; k < 4; ++k) qo[iq + k] = r[k] * alpha;
    return;
  }
  const double c0 = q[iq + 2], s0 = q[iq + 3], vx = v[iv], vy = v[iv + 1], w = v[iv + 2];
  double sv, cv;
  sincos(w, &sv, &cv);
  double t0 = vx, t1 = vy;
  if (fabs(w) > 1e-14) {
    t0 = (-vy - (-vy * cv + vx * (-sv))) / w;
    t1 = (vx - (-vy * sv + vx * cv)) / w;
  }
  qo[iq] = c0 * t0 - s0 * t1 + q[iq];
  qo[iq + 1] = s0 * t0 + c0 * t1 + q[iq + 1];
  qo[iq + 2] = c0 * cv - s0 * sv;
  qo[iq + 3] = s0 * cv + c0 * sv;
}
GB_HD void integrate_one(const MView& m, const In& q, const In& v, const Out& qo) {
  const double eps = eps_of<double>();
  const double ts_prec = 1.2207031250000000e-04;  // eps^(1/4): Taylor switch of exp3 / exp6
  for (int i = 1; i < m.nj; ++i) {
    const int iq = m.idx_q[i], iv = m.idx_v[i];
    if (jt_three(m.jtype[i])) {
      integrate_three(m.jtype[i], q, v, iq, iv, qo);
      continue;
    }
    if (jt_unbounded(m.jtype[i])) {  // SpecialOrthogonalOperationTpl<2>::integrate
      // (liegroup/special-orthogonal.hpp:164-185): (cos, sin) turned by v, then the
      // first-order renormalisation (3 - |z|^2) / 2
      double sw, cw;
      sincos(v[iv], &sw, &cw);
      const double c = cw * q[iq] - sw * q[iq + 1], s = sw * q[iq] + cw * q[iq + 1];
      const double f = (3.0 - (c * c + s * s)) / 2.0;
      qo[iq] = c * f;
      qo[iq + 1] = s * f;
      continue;
    }
    if (m.jtype[i] != JT_FF) {
      qo[iq] = q[iq] + v[iv];
      continue;
    }
    const double lv[3] = {v[iv], v[iv + 1], v[iv + 2]};
    const double w[3] = {v[iv + 3], v[iv + 4], v[iv + 5]};
    const double t2 = w[0] * w[0] + w[1] * w[1] + w[2] * w[2] + eps * eps;
    const double t = sqrt(t2);
    double st, ct;
    sincos(t, &st, &ct);
    const double inv_t2 = 1.0 / t2;
    double a_wxv, a_w2;
    if (t < ts_prec) {
      a_wxv = 0.5 - t2 / 24.0;
      a_w2 = 1.0 / 6.0 - t2 / 120.0;
    } else {
      a_wxv = (1.0 - ct) * inv_t2;
      a_w2 = (t - st) * inv_t2 / t;
    }
    double wxv[3], wxwxv[3], tr[3];
    cross3(w, lv, wxv);
    cross3(w, wxv, wxwxv);
    for (int k = 0; k < 3; ++k) tr[k] = lv[k] + a_wxv * wxv[k] + a_w2 * wxwxv[k];
    const double s2 = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
    const double th = sqrt(s2 + eps * eps);
    double e[4];
    if (s2 > ts_prec) {
      double sh, ch;
      sincos(0.5 * th, &sh, &ch);
      for (int k = 0; k < 3; ++k) e[k] = sh * (w[k] / th);
      e[3] = ch;
    } else {
      const double t22 = s2 / 4.0;
      const double cc = 0.5 * (1.0 - t22 / 6.0 + t22 * t22 / 120.0);
      for (int k = 0; k < 3; ++k) e[k] = cc * w[k];
      e[3] = 1.0 - t22 / 2.0 + t22 * t22 / 24.0;
    }
    const double qq[4] = {q[iq + 3], q[iq + 4], q[iq + 5], q[iq + 6]};
    double uv[3], uxuv[3];
    cross3(qq, tr, uv);
    for (int k = 0; k < 3; ++k) uv[k] += uv[k];
    cross3(qq, uv, uxuv);
    for (int k = 0; k < 3; ++k) qo[iq + k] = tr[k] + qq[3] * uv[k] + uxuv[k] + q[iq + k];
    double r[4];
    r[3] = qq[3] * e[3] - qq[0] * e[0] - qq[1] * e[1] - qq[2] * e[2];
    r[0] = qq[3] * e[0] + qq[0] * e[3] + qq[1] * e[2] - qq[2] * e[1];
    r[1] = qq[3] * e[1] + qq[1] * e[3] + qq[2] * e[0] - qq[0] * e[2];
    r[2] = qq[3] * e[2] + qq[2] * e[3] + qq[0] * e[1] - qq[1] * e[0];
    const double dp = r[0] * qq[0] + r[1] * qq[1] + r[2] * qq[2] + r[3] * qq[3];
    if (dp < 0.0)
      for (int k = 0; k < 4; ++k) r[k] = -r[k];
    const double N2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2] + r[3] * r[3];
    const double alpha = (3.0 - N2) / 2.0;
    for (int k = 0; k < 4; ++k) qo[iq + 3 + k] = r[k] * alpha;
  }
}

}  // namespace gb
