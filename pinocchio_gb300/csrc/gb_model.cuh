// Flattened model tables: the byte blob that is uploaded once per model and
// copied into shared memory by every CTA, and the view the kernels read.
//
// The blob replaces ModelTpl + the tree tables of DataTpl that the hot path
// reads (reference multibody/model.hpp:98-220, multibody/data.hxx:195-306):
// per joint parent / type / idx_q / idx_v / nvSubtree / depth, placements and
// inertias (FP64, FP32 and double-float copies, also as 6x6 block-symmetric
// matrices), per dof armature / parents_fromRow /
// nvSubtree_fromRow, and for the batched products -Minv*X the per-column list
// of rows that can be non-zero (ancestor and subtree dofs), and the Fcrb
// slot of every joint for the Minv recursion of the ABA derivatives, and the
// branch slot of every joint with two or more children (-1 otherwise): the
// sweeps carry a joint's accumulators in registers to its first child / from
// its first child and keep them in a branch slot only where the tree forks.
#pragma once

#include "gb_dfloat.cuh"
#include "gb_spatial.cuh"

namespace gb {

// JT_SPH / JT_PL: spherical (quaternion q, angular velocity v in the joint frame) and planar
// ((x, y, cos, sin), (vx, vy, wz) in the joint frame) joints; JT_RUX / JT_RUY / JT_RUZ: unbounded
// revolute joints (q = (cos, sin) of the angle, nq 2, nv 1); the C ABI's values
enum {
  JT_NONE = 0, JT_RX = 1, JT_RY = 2, JT_RZ = 3, JT_FF = 4, JT_PX = 5, JT_PY = 6, JT_PZ = 7, JT_SPH = 11, JT_PL = 12,
  JT_RUX = 13, JT_RUY = 14, JT_RUZ = 15
};

// One-dof joints (revolute RX/RY/RZ, prismatic PX/PY/PZ, unbounded revolute RUX/RUY/RUZ): the
// coordinate axis, whether the joint slides along it, and its entry of the motion subspace S
// (3 + axis, angular, for a revolute joint; axis, linear, for a prismatic one).
GB_HD bool jt_slides(int jt) { return jt >= JT_PX && jt <= JT_PZ; }
GB_HD bool jt_unbounded(int jt) { return jt >= JT_RUX && jt <= JT_RUZ; }
GB_HD int jt_axis(int jt) { return jt >= JT_RUX ? jt - JT_RUX : jt >= JT_PX ? jt - JT_PX : jt - JT_RX; }
GB_HD int jt_sidx(int jt) { return jt >= JT_RUX ? jt - JT_RUX + 3 : jt >= JT_PX ? jt - JT_PX : jt + 2; }
// Every supported joint's motion subspace is made of unit spatial axes of its frame:
// jt_nv(jt) dofs, dof k along spatial axis jt_col(jt, k) ([linear; angular] index):
// the free-flyer all six (joint-free-flyer.hpp), the spherical joint the angular three
// (JointMotionSubspaceSphericalTpl, joint-spherical.hpp), the planar joint vx, vy, wz
// (JointMotionSubspacePlanarTpl, joint-planar.hpp:380-470), a one-dof joint its axis.
GB_HD bool jt_three(int jt) { return jt == JT_SPH || jt == JT_PL; }
GB_HD int jt_nv(int jt) { return jt == JT_FF ? 6 : jt_three(jt) ? 3 : 1; }
GB_HD int jt_col(int jt, int k) {
  return jt == JT_FF ? k : jt == JT_SPH ? 3 + k : jt == JT_PL ? (k < 2 ? k : 5) : jt_sidx(jt);
}

// Mimic joints: an entry of the extended configuration (src: the caller's entry; kind 0 copy,
// 1 scaling * q + offset, 2 the (cos, sin) pair of an unbounded joint turned to scaling * angle +
// offset, 3 the second entry of such a pair) and of the extended velocity (src, own: the caller's
// own dof, g: 1 or the mimic's scaling)
struct MimicQ {
  int src = 0, kind = 0;
  double scaling = 1.0, offset = 0.0;
};
struct MimicV {
  int src = 0, own = 1;
  double g = 1.0;
};

struct BlobHeader {
  int nj, nq, nv, bytes;
  int max_depth, has_ff, n_rel, nslot;
  int o_parent, o_jtype, o_idxq, o_idxv, o_nvsub, o_depth, o_pfr, o_nsfr;
  int o_place_d, o_iner_d, o_arm_d, o_place_f, o_iner_f, o_arm_f, o_rel_off, o_rel_list;
  int o_slot, o_dofj, o_bslot, nbranch;
  int o_grp, ngroup, o_grp_rel, n_grp_rel;
  int stage_bytes;  // [0, stage_bytes): what the per-instance kernels stage (rel_list and the groups lie beyond)
  int o_i6_d, o_i6_f, o_place_df, o_iner_df;
  int o_arm_df, o_zero;  // o_zero: 16 zero bytes (a zero vector with stride 0)
  int o_fix;             // 9 doubles per joint: F of an unaligned joint's frame (0: no such joint)
  // chains: maximal runs of joints each the only child of the previous one (consecutive in the
  // depth-first order); chain c holds joints chain[3c] .. chain[3c+1] at chain level chain[3c+2]
  int o_chain, nchain, nclevel, chain_team;
  // o_status: the model's numeric status word (GB_NUMERIC_* bits, atomicOr from the kernels), in
  // global memory beyond the staged prefix
  int o_status;
  int o_child, max_child;  // children of each joint, from the last one down (max_child per joint, -1 padded)
  int o_ujoint;            // per joint: the caller's joint it carries (-1: inside an expanded translation)
  double grav_d[6];
  float grav_f[6];
  float padf[2];
  dfloat grav_df[6];
};
static_assert(sizeof(BlobHeader) % 16 == 0, "blob header must keep 16-byte alignment");

struct MView {
  int nj, nq, nv, max_depth, has_ff, nslot;
  const int *parent, *jtype, *idx_q, *idx_v, *nvsub, *depth, *pfr, *nsfr, *rel_off, *rel_list, *slot, *dof_joint, *bslot, *grp, *grp_rel;
  int nbranch, ngroup;
  const int* chain;  // (first joint, last joint, level) per chain
  int nchain, nclevel;
  const double *place_d, *iner_d, *arm_d, *grav_d, *i6_d;
  const float *place_f, *iner_f, *arm_f, *grav_f, *i6_f;
  const dfloat *place_df, *iner_df, *arm_df, *grav_df;
  const double* fix_d;  // nullptr when no joint is unaligned
  unsigned* status;     // the status word in the global copy of the blob (nullptr: not recorded)
  const int* child;     // max_child entries per joint: its children from the last one down, -1 padded
  int max_child;
  const int* ujoint;    // the caller's joint of each joint (per-joint inputs and outputs), -1: none
};

// Numeric failures seen by a kernel (bits of the model's status word, read by gb_numeric_status):
// a pivot of a factorisation that is not > 0 (or NaN): singular or indefinite articulated /
// joint-space inertia; a non-finite output.
enum { NUM_PIVOT = 1u, NUM_NONFINITE = 2u };
GB_HD void flag_numeric(const MView& m, unsigned bits) {
#if defined(__CUDA_ARCH__)
  if (m.status) atomicOr(m.status, bits);
#else
  (void)m;
  (void)bits;
#endif
}
// a pivot d of a factorisation (flagged unless d > 0)
template <class S> GB_HD void check_pivot(const MView& m, S d) {
  if (!(d > S(0))) flag_numeric(m, NUM_PIVOT);
}
GB_HD bool finite_value(double x) { return x - x == 0.0; }  // false for NaN and +-inf
// the status word of a blob staged from `global_blob` (the view was made from the staged copy)
GB_HD void attach_status(MView& m, const unsigned char* global_blob) {
  const BlobHeader* h = reinterpret_cast<const BlobHeader*>(global_blob);
  m.status = reinterpret_cast<unsigned*>(const_cast<unsigned char*>(global_blob) + h->o_status);
}

GB_HD MView make_view(const unsigned char* base) {
  const BlobHeader* h = reinterpret_cast<const BlobHeader*>(base);
  MView m;
  m.nj = h->nj; m.nq = h->nq; m.nv = h->nv; m.max_depth = h->max_depth; m.has_ff = h->has_ff; m.nslot = h->nslot;
  m.parent = reinterpret_cast<const int*>(base + h->o_parent);
  m.jtype = reinterpret_cast<const int*>(base + h->o_jtype);
  m.idx_q = reinterpret_cast<const int*>(base + h->o_idxq);
  m.idx_v = reinterpret_cast<const int*>(base + h->o_idxv);
  m.nvsub = reinterpret_cast<const int*>(base + h->o_nvsub);
  m.depth = reinterpret_cast<const int*>(base + h->o_depth);
  m.pfr = reinterpret_cast<const int*>(base + h->o_pfr);
  m.nsfr = reinterpret_cast<const int*>(base + h->o_nsfr);
  m.rel_off = reinterpret_cast<const int*>(base + h->o_rel_off);
  m.rel_list = reinterpret_cast<const int*>(base + h->o_rel_list);
  m.slot = reinterpret_cast<const int*>(base + h->o_slot);
  m.dof_joint = reinterpret_cast<const int*>(base + h->o_dofj);
  m.bslot = reinterpret_cast<const int*>(base + h->o_bslot);
  m.nbranch = h->nbranch;
  m.grp = reinterpret_cast<const int*>(base + h->o_grp);
  m.grp_rel = reinterpret_cast<const int*>(base + h->o_grp_rel);
  m.ngroup = h->ngroup;
  m.chain = reinterpret_cast<const int*>(base + h->o_chain);
  m.nchain = h->nchain;
  m.nclevel = h->nclevel;
  m.place_d = reinterpret_cast<const double*>(base + h->o_place_d);
  m.iner_d = reinterpret_cast<const double*>(base + h->o_iner_d);
  m.arm_d = reinterpret_cast<const double*>(base + h->o_arm_d);
  m.place_f = reinterpret_cast<const float*>(base + h->o_place_f);
  m.iner_f = reinterpret_cast<const float*>(base + h->o_iner_f);
  m.arm_f = reinterpret_cast<const float*>(base + h->o_arm_f);
  m.i6_d = reinterpret_cast<const double*>(base + h->o_i6_d);
  m.i6_f = reinterpret_cast<const float*>(base + h->o_i6_f);
  m.place_df = reinterpret_cast<const dfloat*>(base + h->o_place_df);
  m.iner_df = reinterpret_cast<const dfloat*>(base + h->o_iner_df);
  m.arm_df = reinterpret_cast<const dfloat*>(base + h->o_arm_df);
  m.grav_df = h->grav_df;
  m.fix_d = h->o_fix ? reinterpret_cast<const double*>(base + h->o_fix) : nullptr;
  m.status = nullptr;
  m.child = reinterpret_cast<const int*>(base + h->o_child);
  m.max_child = h->max_child;
  m.ujoint = reinterpret_cast<const int*>(base + h->o_ujoint);
  m.grav_d = h->grav_d;
  m.grav_f = h->grav_f;
  return m;
}

template <class S> struct ModelScalar;
template <> struct ModelScalar<double> {
  GB_HD static const double* i6(const MView& m, int i) { return m.i6_d + 21 * i; }
  GB_HD static const double* place(const MView& m, int i) { return m.place_d + 12 * i; }
  GB_HD static const double* iner(const MView& m, int i) { return m.iner_d + 10 * i; }
  GB_HD static const double* arm(const MView& m) { return m.arm_d; }
  GB_HD static const double* grav(const MView& m) { return m.grav_d; }
};
template <> struct ModelScalar<float> {
  GB_HD static const float* i6(const MView& m, int i) { return m.i6_f + 21 * i; }
  GB_HD static const float* place(const MView& m, int i) { return m.place_f + 12 * i; }
  GB_HD static const float* iner(const MView& m, int i) { return m.iner_f + 10 * i; }
  GB_HD static const float* arm(const MView& m) { return m.arm_f; }
  GB_HD static const float* grav(const MView& m) { return m.grav_f; }
};

template <> struct ModelScalar<dfloat> {
  GB_HD static const dfloat* place(const MView& m, int i) { return m.place_df + 12 * i; }
  GB_HD static const dfloat* iner(const MView& m, int i) { return m.iner_df + 10 * i; }
  GB_HD static const dfloat* arm(const MView& m) { return m.arm_df; }
  GB_HD static const dfloat* grav(const MView& m) { return m.grav_df; }
};

template <class S> GB_HD void load_placement(const MView& m, int i, X3<S>& P) {
  const S* p = ModelScalar<S>::place(m, i);
#pragma unroll
  for (int k = 0; k < 9; ++k) P.R[k] = p[k];
#pragma unroll
  for (int k = 0; k < 3; ++k) P.t[k] = p[9 + k];
}
// the link's spatial inertia Y.matrix() in block-symmetric form (A, B, D), formed once on the host
template <class S> GB_HD void load_sym6(const MView& m, int i, Sym6<S>& I) {
  const S* p = ModelScalar<S>::i6(m, i);
#pragma unroll
  for (int k = 0; k < 6; ++k) { I.A[k] = p[k]; I.D[k] = p[15 + k]; }
#pragma unroll
  for (int k = 0; k < 9; ++k) I.B[k] = p[6 + k];
}
template <class S> GB_HD void load_inertia(const MView& m, int i, Iner<S>& Y) {
  const S* p = ModelScalar<S>::iner(m, i);
  Y.m = p[0];
#pragma unroll
  for (int k = 0; k < 3; ++k) Y.c[k] = p[1 + k];
#pragma unroll
  for (int k = 0; k < 6; ++k) Y.I[k] = p[4 + k];
}

}  // namespace gb
