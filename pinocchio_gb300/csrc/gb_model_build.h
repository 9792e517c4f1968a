// Host-side flattening of a kinematic tree into the tables and the device
// blob of gb_model.cuh.  Pure C++ (no CUDA runtime), shared by the C ABI and
// by the host build of the kernels used in the CPU tests.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/pinocchio_gb300.h"
#include "gb_model.cuh"

struct gb_model {
  int nj = 0, nq = 0, nv = 0, cap = 0, max_depth = 0;
  int device = 0;
  std::vector<int> parents, jtype, idx_q, idx_v, nvs, nvsub, depth, pfr, nsfr, rel_off, rel_list, slot;
  int nslot = 0;
  int tpb[8] = {128, 128, 128, 128, 128, 128, 128, 128};  // configurations per CTA, per GB_FUNC_*
  int layout[8] = {0, 0, 0, 0, 0, 0, 0, 0};  // GB_INSTANCE_PER_THREAD / _PER_WARP, per GB_FUNC_*
  std::vector<double> placement, inertia, armature;
  // per joint, the rotation F of an unaligned joint's frame (identity otherwise); has_fix: any
  std::vector<double> fix;
  bool has_fix = false;
  double gravity[6];
  std::vector<unsigned char> blob;  // host copy of the device blob
  unsigned char* d_blob = nullptr;  // device copy (owned by the C ABI)
  int blob_bytes = 0;
  int stage_bytes = 0;  // prefix of the blob the per-instance kernels copy into shared memory
  int chain_team = 4;   // lanes per configuration of the lane-per-branch layout
  // the caller's joints (the reference's model) and, per internal joint, the caller's joint it
  // carries (-1 for the intermediate joints of an expanded translation joint)
  int nj_user = 0;
  std::vector<int> ujoint;
  bool has_three = false;  // spherical or planar joints (three dofs along unit axes of the joint frame)
  // the model's device, read once at creation: multiprocessors (grid sizes of the
  // persistent kernels) and the opt-in shared memory per block
  int sm_count = 0, smem_optin = 0;
  // the warp-task plan of the pipelined -Minv*dtau product kernel (built once per model;
  // prod_plan_ok false: that kernel does not apply to this model)
  unsigned short prod_woff[33] = {};
  unsigned short prod_task[256] = {};
  bool prod_plan_ok = false;
  // mimic joints: the kernels run the extended tree (every mimic joint a joint with its own dof,
  // nq / nv above are its sizes); the caller's q, v, tau, M have nq_red / nv_red entries.  Each
  // extended configuration entry comes from a caller entry (qmap: copy, linear affine, or the
  // (cos, sin) pair of an unbounded revolute joint) and each extended velocity entry is a caller
  // entry times a factor (vmap: 1, or the mimic's scaling): v_ext = G v, tau = G^T tau_ext,
  // M = G^T M_ext G
  bool has_mimic = false;
  int nq_red = 0, nv_red = 0;
  std::vector<gb::MimicQ> qmap;
  std::vector<gb::MimicV> vmap;
  void* d_mimic = nullptr;  // device copy: qmap then vmap
};

namespace gbm {

inline size_t align16(size_t x) { return (x + 15) & ~size_t(15); }
// capacity class used to instantiate the kernels (>= njoints and >= nv)
inline int cap_class(int n) { return n <= 8 ? 8 : n <= 16 ? 16 : n <= 32 ? 32 : n <= 64 ? 64 : n <= 128 ? 128 : 0; }

// A rotation F with F e_z = a (a unit): the smallest rotation taking e_z to a
// (Rodrigues' formula about e_z x a) when a_z >= 0; otherwise the half-turn
// about x composed with the smallest rotation taking e_z to diag(1,-1,-1) a.
inline void rotation_to_axis(const double* a, double* F) {
  const double s = a[2] >= 0.0 ? 1.0 : -1.0;
  const double b0 = a[0], b1 = s * a[1], c = s * a[2];  // b = diag(1, s, s) a, b_z >= 0
  const double k = 1.0 / (1.0 + c);
  const double G[9] = {1.0 - k * b0 * b0, -k * b0 * b1, b0, -k * b0 * b1, 1.0 - k * b1 * b1, b1, -b0, -b1, c};
  for (int r = 0; r < 3; ++r)
    for (int q = 0; q < 3; ++q) F[3 * r + q] = (r == 0 ? 1.0 : s) * G[3 * r + q];
}

// Unaligned joints (JointModelRevoluteUnaligned / JointModelPrismaticUnaligned,
// reference multibody/joint/joint-revolute-unaligned.hpp:611-735 and
// joint-prismatic-unaligned.hpp:586-711) become z-axis joints of a rotated frame:
// with F e_z = a, rotation about (translation along) a in frame i is rotation
// about (along) z in frame i' = frame i * F.  So jointPlacement_i <- jointPlacement_i F,
// and the body of joint i and the placements of its children are expressed in
// frame i' (F^T on the left).  Every joint-space quantity is unchanged; forward
// kinematics maps its frame-i' outputs back to frame i (the blob's fix table).
inline int fold_unaligned(gb_model* M, const gb_model_desc* d, std::string* err) {
  const int nj = M->nj;
  M->fix.assign(9 * (size_t)nj, 0.0);
  for (int i = 0; i < nj; ++i) M->fix[9 * i] = M->fix[9 * i + 4] = M->fix[9 * i + 8] = 1.0;
  M->has_fix = false;
  for (int i = 1; i < nj; ++i) {
    const int jt = M->jtype[i];
    if (jt != GB_JOINT_REVOLUTE_UNALIGNED && jt != GB_JOINT_PRISMATIC_UNALIGNED &&
        jt != GB_JOINT_REVOLUTE_UNBOUNDED_UNALIGNED)
      continue;
    if (!d->axis) {
      *err = "unaligned joints need gb_model_desc.axis";
      return GB_ERR_INVALID_ARGUMENT;
    }
    double a[3] = {d->axis[3 * i], d->axis[3 * i + 1], d->axis[3 * i + 2]};
    const double n = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
    if (!(n > 0.0) || !std::isfinite(n)) {
      *err = "joint " + std::to_string(i) + ": the axis must be finite and non-zero";
      return GB_ERR_INVALID_ARGUMENT;
    }
    for (double& x : a) x /= n;
    double F[9];
    rotation_to_axis(a, F);
    M->jtype[i] = jt == GB_JOINT_REVOLUTE_UNALIGNED ? GB_JOINT_RZ
                  : jt == GB_JOINT_PRISMATIC_UNALIGNED ? GB_JOINT_PZ
                                                       : GB_JOINT_RUBZ;
    double* P = &M->placement[12 * (size_t)i];  // R <- R F
    double R[9];
    std::memcpy(R, P, sizeof(R));
    for (int r = 0; r < 3; ++r)
      for (int q = 0; q < 3; ++q) P[3 * r + q] = R[3 * r] * F[q] + R[3 * r + 1] * F[3 + q] + R[3 * r + 2] * F[6 + q];
    double* Y = &M->inertia[10 * (size_t)i];  // lever <- F^T c, I <- F^T I F
    const double c[3] = {Y[1], Y[2], Y[3]};
    const double I[9] = {Y[4], Y[5], Y[7], Y[5], Y[6], Y[8], Y[7], Y[8], Y[9]};
    double FI[9], J[9];
    for (int r = 0; r < 3; ++r) {
      Y[1 + r] = F[r] * c[0] + F[3 + r] * c[1] + F[6 + r] * c[2];
      for (int q = 0; q < 3; ++q) FI[3 * r + q] = F[r] * I[q] + F[3 + r] * I[3 + q] + F[6 + r] * I[6 + q];
    }
    for (int r = 0; r < 3; ++r)
      for (int q = 0; q < 3; ++q) J[3 * r + q] = FI[3 * r] * F[q] + FI[3 * r + 1] * F[3 + q] + FI[3 * r + 2] * F[6 + q];
    Y[4] = J[0]; Y[5] = 0.5 * (J[1] + J[3]); Y[6] = J[4];
    Y[7] = 0.5 * (J[2] + J[6]); Y[8] = 0.5 * (J[5] + J[7]); Y[9] = J[8];
    for (int j = i + 1; j < nj; ++j) {  // children: placement <- F^T placement
      if (M->parents[j] != i) continue;
      double* Q = &M->placement[12 * (size_t)j];
      double Rq[12];
      std::memcpy(Rq, Q, sizeof(Rq));
      for (int r = 0; r < 3; ++r) {
        for (int q = 0; q < 3; ++q) Q[3 * r + q] = F[r] * Rq[q] + F[3 + r] * Rq[3 + q] + F[6 + r] * Rq[6 + q];
        Q[9 + r] = F[r] * Rq[9] + F[3 + r] * Rq[10] + F[6 + r] * Rq[11];
      }
    }
    std::memcpy(&M->fix[9 * (size_t)i], F, sizeof(F));
    M->has_fix = true;
  }
  return GB_OK;
}

// Translation joints (JointModelTranslation, reference multibody/joint/joint-translation.hpp:
// M = (I, q), S = the three linear axes, nq = nv = 3) become three prismatic joints along x,
// y and z with identity placements between them and the body on the last: the same transform
// placement * (I, q), the same joint velocity (v, 0) in the same frame, the same q and v, and
// positive pivots (each prismatic pivot is a translational inertia of the subtree).  The
// kernels then see only one-dof joints there.  `expanded` is the internal tree; user_of[i] is
// the caller's joint of internal joint i (-1 for the two intermediate ones), last_of[j] the
// internal joint carrying the caller's joint j.
//
// Spherical ZYX joints (JointModelSphericalZYX, joint-spherical-ZYX.hpp:404-470: M = (Rz(q0)
// Ry(q1) Rx(q2), 0), S(q) the angular velocity of the Euler rates in the child frame, c = dS/dt
// v) become three revolute joints about z, y and x the same way: the chain's transform is the
// product of the three rotations, the angular velocity of its last frame is the sum of the three
// axes' rates carried into that frame (the columns of S(q)), and its acceleration adds the
// products of those rates (the bias c), so every joint-space quantity and its derivatives in q
// (a vector space) are the joint's.  The chain is singular where the joint is (cos q1 = 0).
inline bool expanded_three(int jt) { return jt == GB_JOINT_TRANSLATION || jt == GB_JOINT_SPHERICAL_ZYX; }
static_assert((int)GB_JOINT_SPHERICAL == (int)gb::JT_SPH && (int)GB_JOINT_PLANAR == (int)gb::JT_PL &&
                  (int)GB_JOINT_FREEFLYER == (int)gb::JT_FF && (int)GB_JOINT_RUBX == (int)gb::JT_RUX &&
                  (int)GB_JOINT_RUBY == (int)gb::JT_RUY && (int)GB_JOINT_RUBZ == (int)gb::JT_RUZ,
              "the kernels use the C ABI's joint codes");
struct ExpandedTree {
  std::vector<int> parents, jtype, user_of, last_of;
  std::vector<double> placement, inertia, axis;
  gb_model_desc desc{};
};
inline int expand_translations(const gb_model_desc* d, ExpandedTree& t, std::string* err) {
  const int nju = d->njoints;
  t.last_of.assign(nju, 0);
  static const double kIdentity[12] = {1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0};
  static const double kZero[10] = {0};
  auto push = [&](int parent, int jt, const double* place, const double* iner, const double* ax, int user) {
    t.parents.push_back(parent);
    t.jtype.push_back(jt);
    t.placement.insert(t.placement.end(), place, place + 12);
    t.inertia.insert(t.inertia.end(), iner, iner + 10);
    for (int k = 0; k < 3; ++k) t.axis.push_back(ax ? ax[k] : 0.0);
    t.user_of.push_back(user);
    return (int)t.parents.size() - 1;
  };
  for (int j = 0; j < nju; ++j) {
    const double* ax = d->axis ? d->axis + 3 * (size_t)j : nullptr;
    if (j == 0) {
      t.last_of[0] = push(d->parents[0], d->jtype[0], d->placement, d->inertia, ax, 0);
      continue;
    }
    const int pu = d->parents[j];
    if (pu < 0 || pu >= j) {
      *err = "parents[i] must satisfy 0 <= parents[i] < i";
      return GB_ERR_INVALID_ARGUMENT;
    }
    const double* P = d->placement + 12 * (size_t)j;
    const double* Y = d->inertia + 10 * (size_t)j;
    if (d->jtype[j] == GB_JOINT_TRANSLATION) {
      const int a = push(t.last_of[pu], GB_JOINT_PX, P, kZero, nullptr, -1);
      const int b = push(a, GB_JOINT_PY, kIdentity, kZero, nullptr, -1);
      t.last_of[j] = push(b, GB_JOINT_PZ, kIdentity, Y, nullptr, j);
    } else if (d->jtype[j] == GB_JOINT_SPHERICAL_ZYX) {
      const int a = push(t.last_of[pu], GB_JOINT_RZ, P, kZero, nullptr, -1);
      const int b = push(a, GB_JOINT_RY, kIdentity, kZero, nullptr, -1);
      t.last_of[j] = push(b, GB_JOINT_RX, kIdentity, Y, nullptr, j);
    } else {
      t.last_of[j] = push(t.last_of[pu], d->jtype[j], P, Y, ax, j);
    }
  }
  t.desc = *d;
  t.desc.njoints = (int)t.parents.size();
  t.desc.parents = t.parents.data();
  t.desc.jtype = t.jtype.data();
  t.desc.placement = t.placement.data();
  t.desc.inertia = t.inertia.data();
  t.desc.axis = d->axis ? t.axis.data() : nullptr;
  return GB_OK;
}

// Mimic joints (JointModelMimic, reference multibody/joint/joint-mimic.hpp:557-760): the
// mimicking joint is a one-dof joint of the caller's tree whose coordinate follows another
// one-dof joint's, q_i = scaling q_j + offset.
inline bool mimic_capable(int jt) {
  return (jt >= GB_JOINT_RX && jt <= GB_JOINT_RZ) || (jt >= GB_JOINT_PX && jt <= GB_JOINT_PRISMATIC_UNALIGNED) ||
         (jt >= GB_JOINT_RUBX && jt <= GB_JOINT_REVOLUTE_UNBOUNDED_UNALIGNED);
}
inline bool unbounded_type(int jt) { return jt >= GB_JOINT_RUBX && jt <= GB_JOINT_REVOLUTE_UNBOUNDED_UNALIGNED; }
inline int check_mimic(const gb_model_desc* d, std::string* err) {
  if (!d->mimic) return GB_OK;
  for (int i = 1; i < d->njoints; ++i) {
    const int j = d->mimic[i];
    if (j <= 0) continue;
    std::string bad;
    if (j >= i) bad = "a mimic joint must come after the joint it mimics";
    else if (d->mimic[j] > 0) bad = "the mimicked joint is a mimic joint itself";
    else if (!mimic_capable(d->jtype[i]) || !mimic_capable(d->jtype[j]))
      bad = "mimic joints are one-dof joints mimicking one-dof joints";
    else if (unbounded_type(d->jtype[i]) != unbounded_type(d->jtype[j]))
      bad = "a mimic joint and its mimicked joint must have the same nq";
    else if (!d->mimic_scaling || !d->mimic_offset)
      bad = "mimic joints need mimic_scaling and mimic_offset";
    if (!bad.empty()) {
      *err = "joint " + std::to_string(i) + ": " + bad;
      return GB_ERR_INVALID_ARGUMENT;
    }
  }
  return GB_OK;
}
// The caller's indices (mimic joints take none: idx_q / idx_v of the joint they mimic, as the
// reference's setMimicIndexes) and the maps from the extended tree's entries to them.
inline void build_mimic_maps(gb_model* M, const gb_model_desc* du, const ExpandedTree& tree) {
  const int nju = du->njoints;
  std::vector<int> rq(nju, 0), rv(nju, 0);
  int nq = 0, nv = 0;
  for (int j = 1; j < nju; ++j) {
    const int jt = du->jtype[j];
    const int m = du->mimic ? du->mimic[j] : 0;
    if (m > 0) {
      rq[j] = rq[m];
      rv[j] = rv[m];
      M->has_mimic = true;
      continue;
    }
    rq[j] = nq;
    rv[j] = nv;
    nq += jt == GB_JOINT_FREEFLYER ? 7 : (jt == GB_JOINT_SPHERICAL || jt == GB_JOINT_PLANAR) ? 4
          : expanded_three(jt) ? 3 : unbounded_type(jt) ? 2 : 1;
    nv += jt == GB_JOINT_FREEFLYER ? 6 : (jt == GB_JOINT_SPHERICAL || jt == GB_JOINT_PLANAR ||
                                          expanded_three(jt)) ? 3 : 1;
  }
  M->nq_red = nq;
  M->nv_red = nv;
  M->qmap.assign(M->nq, gb::MimicQ{});
  M->vmap.assign(M->nv, gb::MimicV{});
  // internal joints of each caller joint: a translation or ZYX joint's three, otherwise its own
  for (int i = 1; i < M->nj; ++i) {
    int j = tree.user_of[i];
    int k = 0;  // position of internal joint i among its caller joint's internal joints
    if (j < 0) {  // the first two joints of an expanded joint: the caller joint is the last's
      int l = i;
      while (tree.user_of[l] < 0) ++l;
      j = tree.user_of[l];
      k = 2 - (l - i);
    } else if (expanded_three(du->jtype[j])) {
      k = 2;
    }
    const int m = du->mimic ? du->mimic[j] : 0;
    const int iq = M->idx_q[i], iv = M->idx_v[i];
    const int nqi = M->jtype[i] == GB_JOINT_FREEFLYER ? 7 : gb::jt_three(M->jtype[i]) ? 4
                    : gb::jt_unbounded(M->jtype[i]) ? 2 : 1;
    if (m > 0) {
      gb::MimicQ& e = M->qmap[iq];
      e.src = rq[m];
      e.kind = gb::jt_unbounded(M->jtype[i]) ? 2 : 1;
      e.scaling = du->mimic_scaling[j];
      e.offset = du->mimic_offset[j];
      if (e.kind == 2) M->qmap[iq + 1] = gb::MimicQ{rq[m] + 1, 3, 0.0, 0.0};
      M->vmap[iv] = gb::MimicV{rv[m], 0, du->mimic_scaling[j]};
    } else {
      for (int c = 0; c < nqi; ++c) M->qmap[iq + c] = gb::MimicQ{rq[j] + k + c, 0, 1.0, 0.0};
      for (int c = 0; c < M->nvs[i]; ++c) M->vmap[iv + c] = gb::MimicV{rv[j] + k + c, 1, 1.0};
    }
  }
}

// Builds the tree tables of DataTpl (reference multibody/data.hxx:195-306) and
// the device blob.
inline int build_model(gb_model* M, const gb_model_desc* du, std::string* err) {
  auto set_error = [&](int code, const std::string& msg) { *err = msg; return code; };
  if (du->njoints < 2) return set_error(GB_ERR_SIZE, "model needs at least one joint besides the universe");
  ExpandedTree tree;
  if (int rc = expand_translations(du, tree, err)) return rc;
  if (int rc = check_mimic(du, err)) return rc;
  const gb_model_desc* d = &tree.desc;
  M->nj_user = du->njoints;
  M->ujoint = tree.user_of;
  const int nj = d->njoints;
  M->nj = nj;
  M->parents.assign(d->parents, d->parents + nj);
  M->jtype.assign(d->jtype, d->jtype + nj);
  M->placement.assign(d->placement, d->placement + 12 * nj);
  M->inertia.assign(d->inertia, d->inertia + 10 * nj);
  const double g0[6] = {0, 0, -9.81, 0, 0, 0};
  std::memcpy(M->gravity, d->gravity ? d->gravity : g0, sizeof(g0));
  if (M->jtype[0] != GB_JOINT_NONE) return set_error(GB_ERR_UNSUPPORTED, "joint 0 must be the universe");
  M->idx_q.assign(nj, 0);
  M->idx_v.assign(nj, 0);
  M->nvs.assign(nj, 0);
  M->depth.assign(nj, 0);
  int nq = 0, nv = 0, nff = 0;
  for (int i = 1; i < nj; ++i) {
    const int jt = M->jtype[i], p = M->parents[i];
    const bool three = jt == GB_JOINT_SPHERICAL || jt == GB_JOINT_PLANAR;
    const bool unbounded = jt >= GB_JOINT_RUBX && jt <= GB_JOINT_REVOLUTE_UNBOUNDED_UNALIGNED;
    if (!three && !unbounded && (jt < GB_JOINT_RX || jt > GB_JOINT_PRISMATIC_UNALIGNED))
      return set_error(GB_ERR_UNSUPPORTED, "joint " + std::to_string(i) + ": unsupported joint type");
    if (p < 0 || p >= i) return set_error(GB_ERR_INVALID_ARGUMENT, "parents[i] must satisfy 0 <= parents[i] < i");
    if (jt == GB_JOINT_FREEFLYER) {
      ++nff;
      if (i != 1 || p != 0)
        return set_error(GB_ERR_UNSUPPORTED, "a free-flyer is supported only as the root joint (joint 1, parent 0)");
    }
    M->idx_q[i] = nq;
    M->idx_v[i] = nv;
    M->nvs[i] = jt == GB_JOINT_FREEFLYER ? 6 : three ? 3 : 1;
    nq += jt == GB_JOINT_FREEFLYER ? 7 : three ? 4 : unbounded ? 2 : 1;
    M->has_three = M->has_three || three;
    nv += M->nvs[i];
    M->depth[i] = M->depth[p] + 1;
    M->max_depth = std::max(M->max_depth, M->depth[i]);
    if (M->inertia[10 * i] < 0.0) return set_error(GB_ERR_INVALID_ARGUMENT, "negative link mass");
  }
  M->nq = nq;
  M->nv = nv;
  if (int rc = fold_unaligned(M, d, err)) return rc;
  build_mimic_maps(M, du, tree);
  if (d->armature && d->nv_armature != M->nv_red) return set_error(GB_ERR_SIZE, "armature must have nv entries");
  M->armature.assign(nv, 0.0);  // per extended dof: the caller's own dofs' entries, 0 for mimic dofs
  if (d->armature)
    for (int e = 0; e < nv; ++e)
      if (M->vmap[e].own) M->armature[e] = d->armature[M->vmap[e].src];
  M->cap = cap_class(std::max(nj, nv));
  if (M->cap == 0) return set_error(GB_ERR_UNSUPPORTED, "models are limited to 128 joints and 128 dofs");
  // lastChild / nvSubtree (data.hxx:195-225)
  std::vector<int> last(nj, -1);
  M->nvsub.assign(nj, 0);
  for (int i = nj - 1; i >= 0; --i) {
    if (last[i] == -1) last[i] = i;
    const int p = i > 0 ? M->parents[i] : 0;
    last[p] = std::max(last[i], last[p]);
    M->nvsub[i] = M->idx_v[last[i]] + M->nvs[last[i]] - M->idx_v[i];
  }
  for (int i = 1; i < nj; ++i)  // compact subtrees (crba.hxx:573-595)
    for (int k = i + 1; k <= last[i]; ++k) {
      int a = k;
      while (a > i) a = M->parents[a];
      if (a != i) return set_error(GB_ERR_UNSUPPORTED, "joints are not in depth-first order");
    }
  // parents_fromRow / nvSubtree_fromRow (data.hxx:250-306)
  M->pfr.assign(nv, -1);
  M->nsfr.assign(nv, 0);
  for (int j = 1; j < nj; ++j) {
    const int p = M->parents[j], iv = M->idx_v[j];
    M->pfr[iv] = p > 0 ? M->idx_v[p] + M->nvs[p] - 1 : -1;
    M->nsfr[iv] = M->nvsub[j];
    for (int r = 1; r < M->nvs[j]; ++r) {
      M->pfr[iv + r] = iv + r - 1;
      M->nsfr[iv + r] = M->nvsub[j] - r;
    }
  }
  // rows that can be non-zero in column c of dtau/dq: ancestors of c and its subtree
  M->rel_off.assign(nv + 1, 0);
  M->rel_list.clear();
  for (int c = 0; c < nv; ++c) {
    std::vector<int> rows;
    for (int a = M->pfr[c]; a >= 0; a = M->pfr[a]) rows.push_back(a);
    std::sort(rows.begin(), rows.end());
    for (int k = c; k < c + M->nsfr[c]; ++k) rows.push_back(k);
    M->rel_off[c] = (int)M->rel_list.size();
    M->rel_list.insert(M->rel_list.end(), rows.begin(), rows.end());
  }
  M->rel_off[nv] = (int)M->rel_list.size();
  // Fcrb slots of the Minv recursion: the last child of a joint (in depth-first
  // order) overwrites its parent's block in place, any other child takes the next slot.
  std::vector<int> last_child(nj, -1);
  for (int i = 1; i < nj; ++i) last_child[M->parents[i]] = i;
  M->slot.assign(nj, 0);
  M->nslot = 1;
  for (int i = 1; i < nj; ++i) {
    const int p = M->parents[i];
    M->slot[i] = (last_child[p] == i) ? M->slot[p] : M->slot[p] + 1;
    M->nslot = std::max(M->nslot, M->slot[i] + 1);
  }
  // blob
  gb::BlobHeader h;
  std::memset(&h, 0, sizeof(h));
  h.nj = nj; h.nq = nq; h.nv = nv; h.max_depth = M->max_depth; h.has_ff = nff; h.n_rel = (int)M->rel_list.size(); h.nslot = M->nslot;
  size_t off = sizeof(gb::BlobHeader);
  auto take = [&](size_t bytes) { const size_t o = off; off = align16(off + bytes); return (int)o; };
  h.o_parent = take(4 * nj); h.o_jtype = take(4 * nj); h.o_idxq = take(4 * nj); h.o_idxv = take(4 * nj);
  h.o_nvsub = take(4 * nj); h.o_depth = take(4 * nj); h.o_pfr = take(4 * nv); h.o_nsfr = take(4 * nv);
  h.o_rel_off = take(4 * (nv + 1)); h.o_slot = take(4 * nj); h.o_dofj = take(4 * nv); h.o_bslot = take(4 * nj);
  // chains of the lane-per-branch layout
  std::vector<int> chain;
  {
    std::vector<int> nch(nj, 0), chain_of(nj, -1);
    for (int i = 1; i < nj; ++i) ++nch[M->parents[i]];
    int nclevel = 0;
    for (int i = 1; i < nj; ++i) {
      const int p = M->parents[i];
      if (p > 0 && nch[p] == 1) {  // continues the parent's chain (i == p + 1 in depth-first order)
        chain_of[i] = chain_of[p];
        chain[3 * chain_of[i] + 1] = i;
      } else {
        chain_of[i] = (int)chain.size() / 3;
        const int level = p > 0 ? chain[3 * chain_of[p] + 2] + 1 : 0;
        chain.insert(chain.end(), {i, i, level});
        nclevel = std::max(nclevel, level + 1);
      }
    }
    h.nchain = (int)chain.size() / 3;
    h.nclevel = nclevel;
    std::vector<int> per_level(std::max(nclevel, 1), 0);
    for (int c = 0; c < h.nchain; ++c) ++per_level[chain[3 * c + 2]];
    const int widest = *std::max_element(per_level.begin(), per_level.end());
    int ts = 4;  // lanes per configuration: the widest chain level, in powers of two from 4 to 32
    while (ts < widest && ts < 32) ts *= 2;
    h.chain_team = ts;
    M->chain_team = ts;
  }
  h.o_chain = take(4 * chain.size() + 4);
  h.o_ujoint = take(4 * (size_t)nj);
  // children of each joint from the last one down (the order the RNEA backward sweep folds them)
  std::vector<std::vector<int>> kids(nj);
  for (int i = nj - 1; i >= 1; --i) kids[M->parents[i]].push_back(i);
  int maxc = 1;
  for (int i = 0; i < nj; ++i) maxc = std::max(maxc, (int)kids[i].size());
  std::vector<int> child((size_t)nj * maxc, -1);
  for (int i = 0; i < nj; ++i)
    for (size_t k = 0; k < kids[i].size(); ++k) child[(size_t)i * maxc + k] = kids[i][k];
  h.max_child = maxc;
  h.o_child = take(4 * child.size());
  // column groups of the -Minv*dtau products (filled below)
  std::vector<int> grp, grp_rel;
  for (int c = 0; c < nv;) {
    int e = c + 1;
    auto rows_of = [&](int col) { return std::vector<int>(M->rel_list.begin() + M->rel_off[col], M->rel_list.begin() + M->rel_off[col + 1]); };
    const std::vector<int> rc = rows_of(c);
    while (e < nv && e - c < 8 && rows_of(e) == rc) ++e;
    grp.push_back(c); grp.push_back(e - c); grp.push_back((int)grp_rel.size());
    grp_rel.insert(grp_rel.end(), rc.begin(), rc.end());
    grp.push_back((int)grp_rel.size());
    c = e;
  }
  h.ngroup = (int)grp.size() / 4; h.n_grp_rel = (int)grp_rel.size();
  h.o_place_d = take(8 * 12 * nj); h.o_iner_d = take(8 * 10 * nj); h.o_arm_d = take(8 * nv);
  h.o_place_f = take(4 * 12 * nj); h.o_iner_f = take(4 * 10 * nj); h.o_arm_f = take(4 * nv);
  h.o_i6_d = take(8 * 21 * nj); h.o_i6_f = take(4 * 21 * nj);
  h.o_place_df = take(8 * 12 * nj); h.o_iner_df = take(8 * 10 * nj); h.o_arm_df = take(8 * nv);
  h.o_fix = M->has_fix ? take(8 * 9 * nj) : 0;  // frame fixes of forward kinematics
  h.o_zero = take(16);
  // the per-instance kernels stage [0, stage_bytes) in shared memory; the row
  // lists below (O(nv^2) for deep trees) are read from global memory by the
  // product and VJP kernels only
  h.stage_bytes = (int)off;
  h.o_rel_list = take(4 * M->rel_list.size() + 4);
  h.o_grp = take(4 * grp.size()); h.o_grp_rel = take(4 * grp_rel.size() + 4);
  h.o_status = take(16);  // the numeric status word (zero at creation)
  h.bytes = (int)off;
  for (int k = 0; k < 6; ++k) {
    h.grav_d[k] = M->gravity[k];
    h.grav_f[k] = (float)M->gravity[k];
    h.grav_df[k] = gb::dfloat(M->gravity[k]);
  }
  M->blob.assign(off, 0);
  unsigned char* b = M->blob.data();
  std::memcpy(b, &h, sizeof(h));
  auto put_i = [&](int o, const std::vector<int>& v) { if (!v.empty()) std::memcpy(b + o, v.data(), 4 * v.size()); };
  auto put_d = [&](int o, const std::vector<double>& v) { if (!v.empty()) std::memcpy(b + o, v.data(), 8 * v.size()); };
  auto put_f = [&](int o, const std::vector<double>& v) {
    for (size_t k = 0; k < v.size(); ++k) reinterpret_cast<float*>(b + o)[k] = (float)v[k];
  };
  put_i(h.o_parent, M->parents); put_i(h.o_jtype, M->jtype); put_i(h.o_idxq, M->idx_q); put_i(h.o_idxv, M->idx_v);
  put_i(h.o_nvsub, M->nvsub); put_i(h.o_depth, M->depth); put_i(h.o_pfr, M->pfr); put_i(h.o_nsfr, M->nsfr);
  put_i(h.o_rel_off, M->rel_off); put_i(h.o_rel_list, M->rel_list); put_i(h.o_slot, M->slot);
  std::vector<int> dofj(nv, 0);
  for (int i = 1; i < nj; ++i)
    for (int r = 0; r < M->nvs[i]; ++r) dofj[M->idx_v[i] + r] = i;
  put_i(h.o_dofj, dofj);
  // branch slots: joints with two or more children
  std::vector<int> nchild(nj, 0), bslot(nj, -1);
  for (int i = 1; i < nj; ++i) ++nchild[M->parents[i]];
  int nb = 0;
  for (int i = 1; i < nj; ++i)
    if (nchild[i] >= 2) bslot[i] = nb++;
  h.nbranch = nb;
  std::memcpy(b, &h, sizeof(h));
  put_i(h.o_bslot, bslot);
  put_i(h.o_chain, chain);
  put_i(h.o_ujoint, M->ujoint);
  put_i(h.o_child, child);
  put_i(h.o_grp, grp);
  put_i(h.o_grp_rel, grp_rel);
  put_d(h.o_place_d, M->placement); put_d(h.o_iner_d, M->inertia); put_d(h.o_arm_d, M->armature);
  if (M->has_fix) put_d(h.o_fix, M->fix);
  put_f(h.o_place_f, M->placement); put_f(h.o_iner_f, M->inertia); put_f(h.o_arm_f, M->armature);
  {  // Y.matrix() per link (reference spatial/inertia.hpp:481-491), block-symmetric A, B, D
    std::vector<double> i6(21 * (size_t)nj, 0.0);
    for (int i = 0; i < nj; ++i) {
      gb::Iner<double> Y;
      Y.m = M->inertia[10 * i];
      for (int k = 0; k < 3; ++k) Y.c[k] = M->inertia[10 * i + 1 + k];
      for (int k = 0; k < 6; ++k) Y.I[k] = M->inertia[10 * i + 4 + k];
      gb::Sym6<double> S6;
      gb::iner_to_sym6(Y, S6);
      for (int k = 0; k < 6; ++k) { i6[21 * i + k] = S6.A[k]; i6[21 * i + 15 + k] = S6.D[k]; }
      for (int k = 0; k < 9; ++k) i6[21 * i + 6 + k] = S6.B[k];
    }
    put_d(h.o_i6_d, i6);
    put_f(h.o_i6_f, i6);
  }
  auto put_df = [&](int o, const std::vector<double>& v) {
    for (size_t k = 0; k < v.size(); ++k) reinterpret_cast<gb::dfloat*>(b + o)[k] = gb::dfloat(v[k]);
  };
  put_df(h.o_place_df, M->placement); put_df(h.o_iner_df, M->inertia); put_df(h.o_arm_df, M->armature);
  M->blob_bytes = (int)off;
  M->stage_bytes = h.stage_bytes;
  return GB_OK;
}


}  // namespace gbm
