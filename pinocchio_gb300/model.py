"""Kinematic-tree model description, shaped like the reference's ``pin.Model``.

The reference builds a ``ModelTpl`` joint by joint with ``addJoint`` and
``appendBodyToJoint`` (reference multibody/model.hxx:61-170); joints are stored
in insertion order with ``parents[i] < i`` and the configuration / velocity
indices ``idx_q`` / ``idx_v`` are cumulative in that order.  This module keeps
that construction API for the joint types on the batched dynamics path
(revolute about the unit x, y or z axis or any unit axis, prismatic along one, and the
free-flyer) and flattens the tree into the plain tables the C ABI takes:

* ``parents`` (int32, njoints), ``jtype`` (int32, njoints; 0 = universe,
  1/2/3 = RX/RY/RZ, 4 = free-flyer, 5/6/7 = PX/PY/PZ, 8 = revolute unaligned,
  9 = prismatic unaligned, 10 = translation, 11 = spherical, 12 = planar, 13/14/15 = unbounded
  revolute RUBX/RUBY/RUBZ, 16 = unbounded revolute unaligned, 17 = spherical ZYX),
* ``axis`` (njoints x 3: the unit axis of an unaligned joint, zero otherwise),
* ``placement`` (njoints x 12: rotation row-major, then translation),
* ``inertia`` (njoints x 10: mass, lever (COM), rotational inertia about the COM
  packed as [xx, xy, yy, xz, yz, zz] -- reference spatial/symmetric3.hpp:46-49),
* ``armature`` (nv) and ``gravity`` (6, [linear; angular]).
"""
from __future__ import annotations

import numpy as np

(JT_NONE, JT_RX, JT_RY, JT_RZ, JT_FF, JT_PX, JT_PY, JT_PZ, JT_RU, JT_PU, JT_TR, JT_SPH, JT_PL, JT_RUBX, JT_RUBY,
 JT_RUBZ, JT_RUBU, JT_ZYX) = range(18)
_ONE_DOF = (JT_RX, JT_RY, JT_RZ, JT_PX, JT_PY, JT_PZ, JT_RU, JT_PU)
UNBOUNDED = (JT_RUBX, JT_RUBY, JT_RUBZ, JT_RUBU)
_JT_NQ = {JT_NONE: 0, JT_FF: 7, JT_TR: 3, JT_ZYX: 3, JT_SPH: 4, JT_PL: 4, **{j: 1 for j in _ONE_DOF},
          **{j: 2 for j in UNBOUNDED}}
_JT_NV = {JT_NONE: 0, JT_FF: 6, JT_TR: 3, JT_ZYX: 3, JT_SPH: 3, JT_PL: 3, **{j: 1 for j in _ONE_DOF + UNBOUNDED}}
PRISMATIC = (JT_PX, JT_PY, JT_PZ, JT_PU)


class Convention:
    """Frame convention of ABA / CRBA (reference multibody/fwd.hpp:73-81)."""

    LOCAL = 0
    WORLD = 1


class JointModel:
    jtype = JT_NONE
    axis = None

    @property
    def nq(self) -> int:
        return _JT_NQ[self.jtype]

    @property
    def nv(self) -> int:
        return _JT_NV[self.jtype]


class JointModelRX(JointModel):
    jtype = JT_RX


class JointModelRY(JointModel):
    jtype = JT_RY


class JointModelRZ(JointModel):
    jtype = JT_RZ


class JointModelFreeFlyer(JointModel):
    jtype = JT_FF


class JointModelPX(JointModel):
    jtype = JT_PX


class JointModelPY(JointModel):
    jtype = JT_PY


class JointModelPZ(JointModel):
    jtype = JT_PZ


class JointModelTranslation(JointModel):
    """Translation along the three axes of the joint frame, q = v in R^3 (reference
    JointModelTranslationTpl, multibody/joint/joint-translation.hpp)."""

    jtype = JT_TR


class JointModelSpherical(JointModel):
    """Rotation with a unit quaternion q = (x, y, z, w), v the angular velocity in the joint
    frame (reference JointModelSphericalTpl, multibody/joint/joint-spherical.hpp)."""

    jtype = JT_SPH


class JointModelSphericalZYX(JointModel):
    """Rotation by the Euler angles q = (z, y, x), R = Rz(q0) Ry(q1) Rx(q2), v = dq/dt (reference
    JointModelSphericalZYXTpl, multibody/joint/joint-spherical-ZYX.hpp); a vector space
    (integrate adds v dt), singular where cos q1 = 0."""

    jtype = JT_ZYX


class JointModelPlanar(JointModel):
    """Motion in the x-y plane: q = (x, y, cos theta, sin theta), v = (vx, vy, wz) in the
    joint frame (reference JointModelPlanarTpl, multibody/joint/joint-planar.hpp)."""

    jtype = JT_PL


class JointModelRUBX(JointModel):
    """Unbounded revolute joint about x: q = (cos theta, sin theta), taken as given (reference
    JointModelRevoluteUnboundedTpl, multibody/joint/joint-revolute-unbounded.hpp); what the URDF
    parser makes of a ``continuous`` joint."""

    jtype = JT_RUBX


class JointModelRUBY(JointModel):
    jtype = JT_RUBY


class JointModelRUBZ(JointModel):
    jtype = JT_RUBZ


def _unit(axis) -> np.ndarray:
    a = np.asarray(axis, dtype=np.float64).reshape(3)
    n = float(np.linalg.norm(a))
    if not n > 0.0:
        raise ValueError("joint axis must be non-zero")
    return a / n


class JointModelRevoluteUnaligned(JointModel):
    """Revolute joint about a unit axis of its frame (reference JointModelRevoluteUnalignedTpl)."""

    jtype = JT_RU

    def __init__(self, axis):
        self.axis = _unit(axis)


class JointModelRevoluteUnboundedUnaligned(JointModel):
    """Unbounded revolute joint about a unit axis of its frame, q = (cos theta, sin theta)
    (reference JointModelRevoluteUnboundedUnalignedTpl)."""

    jtype = JT_RUBU

    def __init__(self, axis):
        self.axis = _unit(axis)


class JointModelPrismaticUnaligned(JointModel):
    """Prismatic joint along a unit axis of its frame (reference JointModelPrismaticUnalignedTpl)."""

    jtype = JT_PU

    def __init__(self, axis):
        self.axis = _unit(axis)


class JointModelComposite(JointModel):
    """A joint made of component joints, each placed relative to the frame of the one before
    (reference JointModelCompositeTpl, multibody/joint/joint-composite.hpp:286-290 addJoint(jmodel,
    placement); joint-composite.hxx:40-77: M = prod_k placement_k M_k(q_k), q and v the components'
    in order).  ``Model.addJoint`` adds it as the chain of its components with massless links
    between them: the same product, q, v, kinematics and dynamics, one model joint per component.
    The last carries the composite's name and bodies and is the index addJoint returns; the others
    are named ``<name>_<k>``."""

    def __init__(self, joint: JointModel | None = None, placement: "SE3 | None" = None):
        self.joints, self.placements = [], []
        if joint is not None:
            self.addJoint(joint, placement)

    def addJoint(self, joint: JointModel, placement: "SE3 | None" = None) -> "JointModelComposite":
        if isinstance(joint, (JointModelComposite, JointModelMimic)):
            raise ValueError("a composite joint's components are plain joint models")
        self.joints.append(joint)
        self.placements.append(SE3.Identity() if placement is None else placement)
        return self

    @property
    def nq(self) -> int:
        return sum(j.nq for j in self.joints)

    @property
    def nv(self) -> int:
        return sum(j.nv for j in self.joints)


class JointModelMimic(JointModel):
    """A joint that follows another one-dof joint (reference JointModelMimicTpl,
    multibody/joint/joint-mimic.hpp:557-760): ``JointModelMimic(joint, mimicked_joint_id, scaling,
    offset)`` adds ``joint`` (a one-dof joint model: revolute, prismatic, unaligned or unbounded)
    with q = scaling * q_mimicked + offset and v = scaling * v_mimicked; it has no entry in q or v
    of its own (nq = nv = 0; nvExtended counts it).  ``mimicked_joint_id`` is the index of a joint
    already in the model (an int, or an object with an ``id`` attribute)."""

    def __init__(self, joint: JointModel, mimicked, scaling: float = 1.0, offset: float = 0.0):
        if isinstance(joint, JointModelMimic):
            raise ValueError("a mimic joint cannot wrap a mimic joint")
        self.joint = joint
        self.jtype = joint.jtype
        self.axis = joint.axis
        self.mimicked = int(getattr(mimicked, "id", mimicked))
        self.scaling = float(scaling)
        self.offset = float(offset)

    @property
    def nq(self) -> int:
        return 0

    @property
    def nv(self) -> int:
        return 0


class SE3:
    """Rigid transform (R, t)."""

    def __init__(self, rotation=None, translation=None):
        self.rotation = np.eye(3) if rotation is None else np.asarray(rotation, dtype=np.float64).reshape(3, 3)
        self.translation = np.zeros(3) if translation is None else np.asarray(translation, dtype=np.float64).reshape(3)

    @staticmethod
    def Identity() -> "SE3":
        return SE3()

    def act_point(self, p):
        return self.rotation @ p + self.translation

    def __mul__(self, other: "SE3") -> "SE3":
        return SE3(self.rotation @ other.rotation, self.rotation @ other.translation + self.translation)


class Inertia:
    """Spatial inertia (mass, lever, rotational inertia about the COM)."""

    def __init__(self, mass: float, lever, inertia):
        self.mass = float(mass)
        self.lever = np.asarray(lever, dtype=np.float64).reshape(3)
        inertia = np.asarray(inertia, dtype=np.float64)
        if inertia.shape == (3, 3):
            inertia = np.array([inertia[0, 0], inertia[1, 0], inertia[1, 1], inertia[2, 0], inertia[2, 1], inertia[2, 2]])
        self.inertia = inertia.reshape(6)

    @staticmethod
    def Zero() -> "Inertia":
        return Inertia(0.0, np.zeros(3), np.zeros(6))

    def matrix3(self):
        s = self.inertia
        return np.array([[s[0], s[1], s[3]], [s[1], s[2], s[4]], [s[3], s[4], s[5]]])

    def se3_action(self, M: SE3) -> "Inertia":
        """M.act(Y) (reference spatial/inertia.hpp:873-880)."""
        R = M.rotation
        return Inertia(self.mass, M.translation + R @ self.lever, R @ self.matrix3() @ R.T)

    def __add__(self, other: "Inertia") -> "Inertia":
        """Y_a + Y_b (reference spatial/inertia.hpp:641-657)."""
        mab = self.mass + other.mass
        inv = 1.0 / max(mab, np.finfo(np.float64).eps)
        c = (self.mass * self.lever + other.mass * other.lever) * inv
        ab = self.lever - other.lever
        skew_sq = np.outer(ab, ab) - ab.dot(ab) * np.eye(3)
        return Inertia(mab, c, self.matrix3() + other.matrix3() - (self.mass * other.mass * inv) * skew_sq)


class Model:
    """Flattened kinematic tree; joint 0 is the universe."""

    def __init__(self):
        self.names = ["universe"]
        self.parents = [0]
        self.jtypes = [JT_NONE]
        self.jointPlacements = [SE3.Identity()]
        self.axes = [np.zeros(3)]
        self.inertias = [Inertia.Zero()]
        self.mimic = [0]  # per joint: the joint it mimics (0: none)
        self.mimic_scaling = [1.0]
        self.mimic_offset = [0.0]
        self.armature = np.zeros(0)
        self.gravity = np.array([0.0, 0.0, -9.81, 0.0, 0.0, 0.0])
        self.name = ""

    # -- construction (reference multibody/model.hxx:61-170) -------------------------------
    def addJoint(self, parent_id: int, joint: JointModel, placement: SE3, name: str = "") -> int:
        if not 0 <= parent_id < self.njoints:
            raise ValueError("parent joint index out of range")
        if isinstance(joint, JointModelComposite):
            if not joint.joints:
                raise ValueError("a composite joint without components")
            jid, n = parent_id, len(joint.joints)
            for k, (jm, P) in enumerate(zip(joint.joints, joint.placements)):
                jid = self.addJoint(jid, jm, placement * P if k == 0 else P, name if k == n - 1 else f"{name}_{k}")
            return jid
        if isinstance(joint, JointModelMimic):
            m = joint.mimicked
            if not 0 < m < self.njoints or self.mimic[m] != 0:
                raise ValueError("the mimicked joint must be a joint of the model that is no mimic itself")
            if joint.jtype not in _ONE_DOF + UNBOUNDED or self.jtypes[m] not in _ONE_DOF + UNBOUNDED:
                raise ValueError("mimic joints are one-dof joints mimicking one-dof joints")
            if (joint.jtype in UNBOUNDED) != (self.jtypes[m] in UNBOUNDED):
                raise ValueError("a mimic joint and its mimicked joint must have the same nq")
            self.mimic.append(m)
            self.mimic_scaling.append(joint.scaling)
            self.mimic_offset.append(joint.offset)
        else:
            self.mimic.append(0)
            self.mimic_scaling.append(1.0)
            self.mimic_offset.append(0.0)
        self.parents.append(int(parent_id))
        self.jtypes.append(int(joint.jtype))
        self.jointPlacements.append(placement)
        self.axes.append(np.zeros(3) if joint.axis is None else np.array(joint.axis, dtype=np.float64))
        self.inertias.append(Inertia.Zero())
        self.names.append(name or f"joint_{self.njoints - 1}")
        self.armature = np.concatenate([self.armature, np.zeros(joint.nv)])
        return self.njoints - 1

    def appendBodyToJoint(self, joint_id: int, inertia: Inertia, placement: SE3 | None = None) -> None:
        placed = inertia if placement is None else inertia.se3_action(placement)
        cur = self.inertias[joint_id]
        self.inertias[joint_id] = placed if cur.mass == 0.0 and not cur.inertia.any() else cur + placed

    # -- sizes ----------------------------------------------------------------------------
    @property
    def njoints(self) -> int:
        return len(self.parents)

    @property
    def nqs(self):
        return [0 if m else _JT_NQ[j] for j, m in zip(self.jtypes, self.mimic)]

    @property
    def nvs(self):
        return [0 if m else _JT_NV[j] for j, m in zip(self.jtypes, self.mimic)]

    def _indices(self, sizes):
        # cumulative in insertion order; a mimic joint takes its mimicked joint's index
        out, n = [], 0
        for i, (k, m) in enumerate(zip(sizes, self.mimic)):
            out.append(out[m] if m else n)
            n += k
        return out

    @property
    def idx_qs(self):
        return self._indices(self.nqs)

    @property
    def idx_vs(self):
        return self._indices(self.nvs)

    @property
    def nvExtended(self) -> int:
        """nv plus one per mimic joint (reference ModelTpl::nvExtended)."""
        return self.nv + sum(1 for m in self.mimic if m)

    def has_mimic(self) -> bool:
        return any(self.mimic)

    @property
    def nq(self) -> int:
        return int(sum(self.nqs))

    @property
    def nv(self) -> int:
        return int(sum(self.nvs))

    def has_free_flyer(self) -> bool:
        return JT_FF in self.jtypes

    # -- flattening for the C ABI ----------------------------------------------------------
    def tables(self) -> dict:
        nj = self.njoints
        placement = np.zeros((nj, 12))
        inertia = np.zeros((nj, 10))
        for i in range(nj):
            placement[i, :9] = self.jointPlacements[i].rotation.reshape(9)
            placement[i, 9:] = self.jointPlacements[i].translation
            Y = self.inertias[i]
            inertia[i, 0] = Y.mass
            inertia[i, 1:4] = Y.lever
            inertia[i, 4:] = Y.inertia
        return dict(
            parents=np.ascontiguousarray(self.parents, dtype=np.int32),
            jtype=np.ascontiguousarray(self.jtypes, dtype=np.int32),
            placement=np.ascontiguousarray(placement),
            inertia=np.ascontiguousarray(inertia),
            armature=np.ascontiguousarray(self.armature, dtype=np.float64),
            gravity=np.ascontiguousarray(self.gravity, dtype=np.float64),
            axis=np.ascontiguousarray(np.array(self.axes, dtype=np.float64).reshape(nj, 3)),
            mimic=np.ascontiguousarray(self.mimic, dtype=np.int32),
            mimic_scaling=np.ascontiguousarray(self.mimic_scaling, dtype=np.float64),
            mimic_offset=np.ascontiguousarray(self.mimic_offset, dtype=np.float64),
        )

    def subtree_tables(self) -> dict:
        """nvSubtree, parents_fromRow, nvSubtree_fromRow (reference multibody/data.hxx:195-306)."""
        nj, nvs, idx_v = self.njoints, self.nvs, self.idx_vs
        last = [-1] * nj
        nvsub = [0] * nj
        for i in range(nj - 1, -1, -1):
            if last[i] == -1:
                last[i] = i
            p = self.parents[i] if i > 0 else 0
            last[p] = max(last[i], last[p])
            nvsub[i] = idx_v[last[i]] + nvs[last[i]] - idx_v[i]
        pfr = [-1] * self.nv
        nsfr = [0] * self.nv
        for j in range(1, nj):
            p = self.parents[j]
            iv = idx_v[j]
            pfr[iv] = idx_v[p] + nvs[p] - 1 if p > 0 else -1
            nsfr[iv] = nvsub[j]
            for r in range(1, nvs[j]):
                pfr[iv + r] = iv + r - 1
                nsfr[iv + r] = nvsub[j] - r
        return dict(lastChild=last, nvSubtree=nvsub, parents_fromRow=pfr, nvSubtree_fromRow=nsfr)

    def check_depth_first(self) -> None:
        """Compact-subtree condition the CRBA needs (reference algorithm/crba.hxx:573-595)."""
        last = self.subtree_tables()["lastChild"]
        for i in range(1, self.njoints):
            for k in range(i + 1, last[i] + 1):
                a = k
                while a > i:
                    a = self.parents[a]
                if a != i:
                    raise ValueError("joints are not in depth-first order")

    def neutral(self) -> np.ndarray:
        """The identity configuration (reference neutral(model), liegroup neutral elements): unit
        quaternions (0, 0, 0, 1), planar and unbounded angles (cos, sin) = (1, 0), zero elsewhere."""
        q = np.zeros(self.nq)
        for jt, iq, m in zip(self.jtypes, self.idx_qs, self.mimic):
            if m:
                continue
            if jt == JT_FF:
                q[iq + 6] = 1.0
            elif jt == JT_SPH:
                q[iq + 3] = 1.0
            elif jt == JT_PL:
                q[iq + 2] = 1.0
            elif jt in UNBOUNDED:
                q[iq] = 1.0
        return q
