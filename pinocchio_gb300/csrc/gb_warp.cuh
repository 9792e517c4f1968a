// Warp-per-instance RNEA and ABA: the per-instance device code shared by the
// warp-layout kernels (gb_warp.cu) and the heterogeneous launch (gb_multi.cu).
//
// Lane j takes joint j (j, j + 32, ...).  The joint transforms are independent
// and computed in parallel; the recursions run level by level over the tree
// depth (every joint of one depth at once: the four limbs of a humanoid in
// parallel), the backward sweeps from the deepest level up, each parent folding
// in its children's contributions itself.  Per-joint state lives in shared
// memory, one region per warp.  Every joint runs the per-instance code of
// gb_dyn.cuh operation for operation, and a parent adds its children's
// contributions in the order the one-thread kernels do (the first child, then
// the others from the last one down), so both layouts give identical bits.
#pragma once

#include "gb_dyn.cuh"
#include "gb_internal.h"

namespace gbi {
namespace warp {

__device__ __forceinline__ gb::In w_in(const Arr& a, long b) { return gb::In{a.p + b * a.is, a.es}; }
__device__ __forceinline__ gb::Out w_out(const Arr& a, long b) {
  return gb::Out{const_cast<double*>(a.p) + b * a.is, a.es};
}
__host__ __device__ __forceinline__ size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

// Who evaluates which joint when.  LevelSched: a warp per configuration, lane j
// takes joints j, j + 32, ...; one step per tree depth (all joints of a depth at
// once).  BranchSched<TS>: a team of TS lanes per configuration, one lane per
// chain (a maximal run of joints each the only child of the previous one); one
// step per chain level, each lane walking its chain joint by joint (down the
// chain in the forward passes, up in the backward ones).  In both, a joint's
// parent and children are done in an earlier step or earlier by the same lane,
// and the per-joint code is the same.
struct LevelSched {
  int lane;
  __device__ int steps(const gb::MView& m) const { return m.max_depth; }
  template <class F> __device__ void all(const gb::MView& m, F f) const {
    for (int i = 1 + lane; i < m.nj; i += 32) f(i);
  }
  template <class F> __device__ void down(const gb::MView& m, int step, F f) const {
    for (int i = 1 + lane; i < m.nj; i += 32)
      if (m.depth[i] == step) f(i);
  }
  template <class F> __device__ void up(const gb::MView& m, int step, F f) const { down(m, step, f); }
  __device__ void sync() const { __syncwarp(); }
};
template <int TS> struct BranchSched {
  int rank;
  unsigned mask;  // the team's lanes
  __device__ int steps(const gb::MView& m) const { return m.nclevel; }
  template <class F> __device__ void all(const gb::MView& m, F f) const {
    for (int i = 1 + rank; i < m.nj; i += TS) f(i);
  }
  template <class F> __device__ void down(const gb::MView& m, int step, F f) const {
    for (int c = rank; c < m.nchain; c += TS)
      if (m.chain[3 * c + 2] == step - 1)
        for (int i = m.chain[3 * c]; i <= m.chain[3 * c + 1]; ++i) f(i);
  }
  template <class F> __device__ void up(const gb::MView& m, int step, F f) const {
    for (int c = rank; c < m.nchain; c += TS)
      if (m.chain[3 * c + 2] == step - 1)
        for (int i = m.chain[3 * c + 1]; i >= m.chain[3 * c]; --i) f(i);
  }
  __device__ void sync() const { __syncwarp(mask); }
};

// shared-memory scalars per joint of one warp's region
template <class S> constexpr int rnea_words() { return 12 + 6 * 4; }  // X, vel, acc, f, child force

// SHFL (one joint per lane, nj - 1 <= 32, LevelSched): the backward sweep gathers the
// children's forces with warp shuffles from the lanes that computed them (kept in registers)
// instead of through shared memory; same children, same order, same bits.
template <class S, class Sched, bool SHFL = false>
__device__ void rnea_warp_one(const gb::MView& m, const gb::In& q, const gb::In& v, const gb::In& a,
                              const gb::Out& tau, S* ws, const Sched& sc) {
  using namespace gb;
  const int nj = m.nj;
  X3<S>* X = reinterpret_cast<X3<S>*>(ws);
  M6<S>* vel = reinterpret_cast<M6<S>*>(ws + 12 * nj);
  M6<S>* acc = vel + nj;
  M6<S>* f = acc + nj;
  M6<S>* cf = f + nj;
  const S* g = ModelScalar<S>::grav(m);
  const S* arm = ModelScalar<S>::arm(m);
  sc.all(m, [&](int i) { joint_transform(m, i, q, X[i]); });
  sc.sync();
  for (int d = 1; d <= sc.steps(m); ++d) {  // forward (rnea_one's first loop)
    sc.down(m, d, [&](int i) {
      const int p = m.parent[i], jt = m.jtype[i], iv = m.idx_v[i];
      M6<S> vJ, aJ, t, ap, vi, ai;
      joint_motion(jt, v, iv, vJ);
      joint_motion(jt, a, iv, aJ);
      if (p > 0) {
        actinv_motion(X[i], vel[p], t);
#pragma unroll
        for (int k = 0; k < 6; ++k) vi.v[k] = vJ.v[k] + t.v[k];
        actinv_motion(X[i], acc[p], ap);
      } else {
        vi = vJ;
        M6<S> mg;
#pragma unroll
        for (int k = 0; k < 6; ++k) mg.v[k] = -g[k];
        actinv_motion(X[i], mg, ap);
      }
      cross_motion(vi, vJ, t);
#pragma unroll
      for (int k = 0; k < 6; ++k) ai.v[k] = (t.v[k] + aJ.v[k]) + ap.v[k];
      Iner<S> Y;
      load_inertia(m, i, Y);
      M6<S> h, fa, fx;
      iner_mul(Y, vi, h);
      iner_mul(Y, ai, fa);
      cross_force(vi, h, fx);
#pragma unroll
      for (int k = 0; k < 6; ++k) f[i].v[k] = fa.v[k] + fx.v[k];
      vel[i] = vi;
      acc[i] = ai;
    });
    sc.sync();
  }
  if constexpr (SHFL) {
    const int i = sc.lane + 1;
    M6<S> mine;  // the joint's force moved to its parent, valid after its level
#pragma unroll
    for (int k = 0; k < 6; ++k) mine.v[k] = S(0);
    for (int d = sc.steps(m); d >= 1; --d) {
      const bool active = i < nj && m.depth[i] == d;
      M6<S> fi;
      if (active) fi = f[i];
      for (int s = 0; s < m.max_child; ++s) {  // warp-uniform: every lane takes part in the shuffles
        const int c = active ? m.child[i * m.max_child + s] : -1;
        const int src = c > 0 ? c - 1 : sc.lane;
#pragma unroll
        for (int k = 0; k < 6; ++k) {
          const S x = __shfl_sync(0xffffffffu, mine.v[k], src);
          if (c > 0) fi.v[k] += x;
        }
      }
      if (active) {
        const int p = m.parent[i], jt = m.jtype[i], iv = m.idx_v[i];
        if (jt == JT_FF) {
#pragma unroll
          for (int k = 0; k < 6; ++k) {
            const double t = double(fi.v[k] + arm[iv + k] * S(a[iv + k]));
            if (!gb::finite_value(t)) gb::flag_numeric(m, gb::NUM_NONFINITE);
            tau[iv + k] = t;
          }
        } else {
          const double t = double(pick6(fi.v, jt_sidx(jt)) + arm[iv] * S(a[iv]));
          if (!gb::finite_value(t)) gb::flag_numeric(m, gb::NUM_NONFINITE);
          tau[iv] = t;
        }
        if (p > 0) act_force(X[i], fi, mine);
      }
      __syncwarp();
    }
    return;
  }
  for (int d = sc.steps(m); d >= 1; --d) {  // backward: children folded in by decreasing index
    sc.up(m, d, [&](int i) {
      const int p = m.parent[i], jt = m.jtype[i], iv = m.idx_v[i];
      M6<S> fi = f[i];
      for (int c = nj - 1; c > i; --c)
        if (m.parent[c] == i)
#pragma unroll
          for (int k = 0; k < 6; ++k) fi.v[k] += cf[c].v[k];
      if (jt == JT_FF) {
#pragma unroll
        for (int k = 0; k < 6; ++k) {
          const double t = double(fi.v[k] + arm[iv + k] * S(a[iv + k]));
          if (!gb::finite_value(t)) gb::flag_numeric(m, gb::NUM_NONFINITE);
          tau[iv + k] = t;
        }
      } else {
        const double t = double(pick6(fi.v, jt_sidx(jt)) + arm[iv] * S(a[iv]));
        if (!gb::finite_value(t)) gb::flag_numeric(m, gb::NUM_NONFINITE);
        tau[iv] = t;
      }
      if (p > 0) act_force(X[i], fi, cf[i]);
    });
    sc.sync();
  }
}

// per joint: X (12 S), vel (6), child inertia (21), child force (6), UDinv (6), acc (6) in S; du in SS
template <class S, class SS> constexpr int aba_words_s() { return 12 + 6 + 21 + 6 + 6 + 6; }

template <class S, class SS, class Sched>
__device__ void aba_warp_one(const gb::MView& m, const gb::In& q, const gb::In& v, const gb::In& tau,
                             const gb::Out& ddq, S* ws, SS* wss, const Sched& sc) {
  using namespace gb;
  const int nj = m.nj;
  X3<S>* X = reinterpret_cast<X3<S>*>(ws);
  M6<S>* vel = reinterpret_cast<M6<S>*>(ws + 12 * nj);
  Sym6<S>* cI = reinterpret_cast<Sym6<S>*>(ws + 18 * nj);
  M6<S>* cf = reinterpret_cast<M6<S>*>(ws + 39 * nj);
  M6<S>* UDs = reinterpret_cast<M6<S>*>(ws + 45 * nj);
  M6<S>* acc = reinterpret_cast<M6<S>*>(ws + 51 * nj);
  SS* du = wss;              // nj
  SS* D6 = wss + nj;         // 36, the root free-flyer's
  SS* UD6 = D6 + 36;         // 36
  SS* u6 = UD6 + 36;         // 6
  const S* g = ModelScalar<S>::grav(m);
  const double* arm = m.arm_d;
  // pass 1 (AbaLocalConventionForwardStep1, aba.hxx:360-399)
  sc.all(m, [&](int i) {
    if (m.jtype[i] == JT_FF) {
      joint_transform(m, i, q, X[i]);
    } else {
      S sn, cn;
      joint_params_q(m.jtype[i], q, m.idx_q[i], &sn, &cn);
      const S* P = ModelScalar<S>::place(m, i);
      compose_joint(P, P + 9, m.jtype[i], cn, sn, X[i]);
    }
  });
  sc.sync();
  for (int d = 1; d <= sc.steps(m); ++d) {
    sc.down(m, d, [&](int i) {
      const int p = m.parent[i];
      M6<S> vJ, t;
      joint_motion(m.jtype[i], v, m.idx_v[i], vJ);
      if (p > 0) {
        actinv_motion(X[i], vel[p], t);
#pragma unroll
        for (int k = 0; k < 6; ++k) vel[i].v[k] = vJ.v[k] + t.v[k];
      } else {
        vel[i] = vJ;
      }
    });
    sc.sync();
  }
  // pass 2 (AbaLocalConventionBackwardStep, aba.hxx:402-434), deepest level first
  for (int d = sc.steps(m); d >= 1; --d) {
    sc.up(m, d, [&](int i) {
      const int p = m.parent[i], jt = m.jtype[i], iv = m.idx_v[i];
      Iner<S> Y;
      load_inertia(m, i, Y);
      Sym6<SS> Ia;
      load_sym6(m, i, Ia);
      M6<S> vJ, c, h, f;
      joint_motion(jt, v, iv, vJ);
      cross_motion(vel[i], vJ, c);
      iner_mul(Y, vel[i], h);
      cross_force(vel[i], h, f);
      if (i + 1 < nj && m.parent[i + 1] == i) {  // first child
        Sym6<SS> Icar;
        sym6_convert(cI[i + 1], Icar);
        sym6_add(Ia, Icar);
#pragma unroll
        for (int k = 0; k < 6; ++k) f.v[k] += cf[i + 1].v[k];
      }
      if (m.bslot[i] >= 0) {  // the other children, from the last one down
        Sym6<SS> Isl;
        M6<S> fsl;
#pragma unroll
        for (int k = 0; k < 6; ++k) { Isl.A[k] = SS(0); Isl.D[k] = SS(0); fsl.v[k] = S(0); }
#pragma unroll
        for (int k = 0; k < 9; ++k) Isl.B[k] = SS(0);
        for (int cj = nj - 1; cj > i + 1; --cj)
          if (m.parent[cj] == i) {
            sym6_add(Isl, cI[cj]);
#pragma unroll
            for (int k = 0; k < 6; ++k) fsl.v[k] += cf[cj].v[k];
          }
        sym6_add(Ia, Isl);
#pragma unroll
        for (int k = 0; k < 6; ++k) f.v[k] += fsl.v[k];
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
        SS D[36];
#pragma unroll
        for (int k = 0; k < 6; ++k) {
          StU[7 * k] += SS(arm[iv + k]);
          u6[k] = SS(tau[iv + k]) - cvt<SS>(f.v[k]);
        }
        if (!llt_inverse<SS, 6>(StU, D)) gb::flag_numeric(m, gb::NUM_PIVOT);
#pragma unroll
        for (int k = 0; k < 36; ++k) D6[k] = D[k];
#pragma unroll
        for (int r = 0; r < 6; ++r)
#pragma unroll
          for (int cc = 0; cc < 6; ++cc) {
            SS s = Ifull[6 * r] * D[cc];
#pragma unroll
            for (int k = 1; k < 6; ++k) s += Ifull[6 * r + k] * D[6 * k + cc];
            UD6[6 * r + cc] = s;
          }
        return;
      }
      const int sx = jt_sidx(jt);
      const SS u = SS(tau[iv]) - cvt<SS>(pick6(f.v, sx));
      SS U[6], UD[6];
      sym6_col(Ia, sx, U);
      const SS Dpiv = pick6(U, sx) + SS(arm[iv]);
      gb::check_pivot(m, Dpiv);
      const SS Dinv = SS(1) / Dpiv;
#pragma unroll
      for (int k = 0; k < 6; ++k) {
        UD[k] = U[k] * Dinv;
        UDs[i].v[k] = cvt<S>(UD[k]);
      }
      du[i] = Dinv * u;
      if (p > 0) {
        sym6_rank1_sub(Ia, U, UD);
        Sym6<S> Iaf;
        sym6_convert(Ia, Iaf);
        S t6[6];
        sym6_mv(Iaf, c.v, t6);
        M6<S> pa;
#pragma unroll
        for (int k = 0; k < 6; ++k) pa.v[k] = f.v[k] + (t6[k] + cvt<S>(UD[k] * u));
        sym6_transform(Iaf, X[i], cI[i]);
        act_force(X[i], pa, cf[i]);
      }
    });
    sc.sync();
  }
  // pass 3 (AbaLocalConventionForwardStep2, aba.hxx:437-468)
  for (int d = 1; d <= sc.steps(m); ++d) {
    sc.down(m, d, [&](int i) {
      const int p = m.parent[i], jt = m.jtype[i], iv = m.idx_v[i];
      M6<S> ap, a, vJ, c;
      if (p == 0) {
#pragma unroll
        for (int k = 0; k < 6; ++k) ap.v[k] = -g[k];
      } else {
        ap = acc[p];
      }
      actinv_motion(X[i], ap, a);
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
          if (!gb::finite_value(dd[r])) gb::flag_numeric(m, gb::NUM_NONFINITE);
          ddq[iv + r] = double(dd[r]);
        }
#pragma unroll
        for (int r = 0; r < 6; ++r) a.v[r] += cvt<S>(dd[r]);
      } else {
        S w = UDs[i].v[0] * a.v[0];
#pragma unroll
        for (int k = 1; k < 6; ++k) w += UDs[i].v[k] * a.v[k];
        const SS dd = du[i] - cvt<SS>(w);
        if (!gb::finite_value(dd)) gb::flag_numeric(m, gb::NUM_NONFINITE);
        ddq[iv] = double(dd);
        add_at6(a.v, jt_sidx(jt), cvt<S>(dd));
      }
      acc[i] = a;
    });
    sc.sync();
  }
}

// bytes of one warp's shared-memory region
template <class S> __host__ __device__ inline size_t rnea_warp_bytes(int nj) {
  return align16(sizeof(S) * rnea_words<S>() * (size_t)nj);
}
template <class S, class SS> __host__ __device__ inline size_t aba_warp_bytes(int nj) {
  return align16(sizeof(S) * aba_words_s<S, SS>() * (size_t)nj) + align16(sizeof(SS) * ((size_t)nj + 78));
}

}  // namespace warp
}  // namespace gbi
