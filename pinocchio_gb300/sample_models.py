"""Seeded synthetic models and inputs for the batched dynamics workloads.

The reference builds its test robots with ``buildModels::humanoidRandom`` and
``manipulator`` (reference multibody/sample-models.hxx:20-308) from unseeded
``Inertia::Random`` / ``SE3::Random`` draws.  The workloads here need
reproducible models, so every generator takes an explicit seed and draws from
numpy's PCG64 (``np.random.default_rng(seed)``):

* joint placement: rotation from a uniform random unit quaternion (normalised
  4-D Gaussian), translation U[-0.3, 0.3]^3 m;
* link inertia: mass U[0.5, 5] kg (or the range given), COM U[-0.1, 0.1]^3 m,
  rotational inertia R diag(U[0.01, 0.1]^3) R^T with R a uniform random rotation;
* revolute axes uniform over the unit x / y / z axes; in ``mixed_tree`` each
  one-dof joint is one of RX, RY, RZ, PX, PY, PZ, uniformly.

Workloads:
  ``manipulator6r``  6 revolute joints in series (nq = nv = 6);
  ``humanoid32``     free-flyer root, two torso revolute joints, four limbs of
                     six revolute joints hanging off the torso (nq 33, nv 32);
  ``random_tree``    seeded trees with 0-3 children per node (optional free-flyer root);
  ``chain``          a revolute serial chain (100 links, masses U[0.1, 1] kg);
  ``mixed_tree``     a ``random_tree`` of revolute and prismatic joints;
  ``unaligned_tree`` a ``random_tree`` whose joints are, uniformly, aligned revolute,
                     aligned prismatic, or revolute / prismatic about a random unit axis.
"""
from __future__ import annotations

import numpy as np

from .model import (
    JT_FF,
    JT_PL,
    JT_SPH,
    JT_TR,
    JT_ZYX,
    PRISMATIC,
    UNBOUNDED,
    Inertia,
    JointModelFreeFlyer,
    JointModelPX,
    JointModelPY,
    JointModelPZ,
    JointModelPrismaticUnaligned,
    JointModelRevoluteUnaligned,
    JointModelRevoluteUnboundedUnaligned,
    JointModelRUBX,
    JointModelRUBY,
    JointModelRUBZ,
    JointModelRX,
    JointModelRY,
    JointModelRZ,
    JointModelSphericalZYX,
    JointModelTranslation,
    Model,
    SE3,
)

_REVOLUTE = (JointModelRX, JointModelRY, JointModelRZ)
_ONE_DOF = _REVOLUTE + (JointModelPX, JointModelPY, JointModelPZ)


def quat_to_matrix(x, y, z, w) -> np.ndarray:
    return np.array(
        [
            [1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
            [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
            [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)],
        ]
    )


def random_unit_quaternion(rng: np.random.Generator, n: int | None = None) -> np.ndarray:
    """Uniform unit quaternion(s) (x, y, z, w): a normalised 4-D Gaussian."""
    g = rng.standard_normal((4,) if n is None else (n, 4))
    return g / np.linalg.norm(g, axis=-1, keepdims=True)


def random_rotation(rng: np.random.Generator) -> np.ndarray:
    return quat_to_matrix(*random_unit_quaternion(rng))


def random_placement(rng: np.random.Generator) -> SE3:
    R = random_rotation(rng)
    t = rng.uniform(-0.3, 0.3, 3)
    return SE3(R, t)


def random_inertia(rng: np.random.Generator, mass_range=(0.5, 5.0)) -> Inertia:
    m = rng.uniform(*mass_range)
    c = rng.uniform(-0.1, 0.1, 3)
    R = random_rotation(rng)
    I = R @ np.diag(rng.uniform(0.01, 0.1, 3)) @ R.T
    I = 0.5 * (I + I.T)
    return Inertia(m, c, I)


def _random_revolute(rng: np.random.Generator):
    return _REVOLUTE[int(rng.integers(0, 3))]()


def _random_one_dof(rng: np.random.Generator):
    return _ONE_DOF[int(rng.integers(0, 6))]()


def _random_any_axis(rng: np.random.Generator):
    k = int(rng.integers(0, 4))
    if k == 0:
        return _random_revolute(rng)
    if k == 1:
        return _ONE_DOF[3 + int(rng.integers(0, 3))]()
    axis = rng.standard_normal(3)
    return (JointModelRevoluteUnaligned if k == 2 else JointModelPrismaticUnaligned)(axis / np.linalg.norm(axis))


def _random_unbounded(rng: np.random.Generator):
    """An unbounded revolute joint about x, y, z or a random axis, or (one in five) a revolute one."""
    k = int(rng.integers(0, 5))
    if k < 3:
        return (JointModelRUBX, JointModelRUBY, JointModelRUBZ)[k]()
    if k == 3:
        axis = rng.standard_normal(3)
        return JointModelRevoluteUnboundedUnaligned(axis / np.linalg.norm(axis))
    return _random_revolute(rng)


def _add_link(model: Model, rng, parent: int, joint, name: str, mass_range=(0.5, 5.0)) -> int:
    jid = model.addJoint(parent, joint, random_placement(rng), name)
    model.appendBodyToJoint(jid, random_inertia(rng, mass_range))
    return jid


def manipulator6r(seed: int = 0) -> Model:
    """6-revolute serial manipulator (nq = nv = 6)."""
    rng = np.random.default_rng(seed)
    model = Model()
    model.name = "manipulator6r"
    parent = 0
    for k in range(6):
        parent = _add_link(model, rng, parent, _random_revolute(rng), f"j{k + 1}")
    return model


def humanoid32(seed: int = 1) -> Model:
    """Free-flyer + 2 torso revolute joints + 4 limbs x 6 revolute joints (nq 33, nv 32)."""
    rng = np.random.default_rng(seed)
    model = Model()
    model.name = "humanoid32"
    root = _add_link(model, rng, 0, JointModelFreeFlyer(), "root")
    t1 = _add_link(model, rng, root, _random_revolute(rng), "torso1")
    t2 = _add_link(model, rng, t1, _random_revolute(rng), "torso2")
    for limb in range(4):
        parent = t2
        for k in range(6):
            parent = _add_link(model, rng, parent, _random_revolute(rng), f"limb{limb}_{k}")
    return model


def random_tree(nv: int, free_flyer: bool, seed: int, max_children: int = 3, joint=_random_revolute) -> Model:
    """Seeded tree with 0..max_children children per node and exactly ``nv`` dofs.

    The tree is grown breadth-first (each node draws its number of children),
    then emitted in depth-first order so that ``parents[i] < i`` and every
    subtree is a contiguous joint range, as the reference requires.
    """
    rng = np.random.default_rng(seed)
    n_rev = nv - (6 if free_flyer else 0)
    if n_rev < 1:
        raise ValueError("tree needs at least one revolute joint")
    children: dict[int, list[int]] = {0: []}  # node 0 = root joint (FF or first revolute)
    n_nodes = 1 if free_flyer else 1
    rev_left = n_rev - (0 if free_flyer else 1)
    frontier = [0]
    while rev_left > 0:
        nxt = []
        for node in frontier:
            if rev_left == 0:
                break
            k = int(rng.integers(0, max_children + 1))
            if node == 0 and k == 0:
                k = 1
            k = min(k, rev_left)
            for _ in range(k):
                children[node].append(n_nodes)
                children[n_nodes] = []
                nxt.append(n_nodes)
                n_nodes += 1
                rev_left -= 1
        if not nxt:  # every frontier node drew zero children: force one
            node = frontier[int(rng.integers(0, len(frontier)))]
            children[node].append(n_nodes)
            children[n_nodes] = []
            nxt.append(n_nodes)
            n_nodes += 1
            rev_left -= 1
        frontier = nxt
    model = Model()
    model.name = f"tree{nv}{'ff' if free_flyer else ''}"

    def emit(node: int, parent_jid: int):
        jm = JointModelFreeFlyer() if node == 0 and free_flyer else joint(rng)
        jid = _add_link(model, rng, parent_jid, jm, f"n{node}")
        for ch in children[node]:
            emit(ch, jid)

    emit(0, 0)
    assert model.nv == nv, (model.nv, nv)
    return model


def mixed_tree(nv: int = 24, free_flyer: bool = True, seed: int = 5) -> Model:
    """``random_tree`` whose one-dof joints are revolute or prismatic (x / y / z), uniformly."""
    model = random_tree(nv, free_flyer, seed, joint=_random_one_dof)
    model.name = f"mixedtree{nv}{'ff' if free_flyer else ''}"
    return model


def unaligned_tree(nv: int = 14, free_flyer: bool = False, seed: int = 7) -> Model:
    """``random_tree`` with aligned and unaligned revolute / prismatic joints."""
    model = random_tree(nv, free_flyer, seed, joint=_random_any_axis)
    model.name = f"unalignedtree{nv}{'ff' if free_flyer else ''}"
    return model


def unbounded_tree(nv: int = 15, free_flyer: bool = True, seed: int = 11) -> Model:
    """``random_tree`` whose joints are mostly unbounded revolute joints (JointModelRUBX/Y/Z and
    the unaligned form, q = (cos, sin)): what URDF ``continuous`` joints give."""
    model = random_tree(nv, free_flyer, seed, joint=_random_unbounded)
    model.name = f"unboundedtree{nv}{'ff' if free_flyer else ''}"
    return model


def translation_tree(seed: int = 9) -> Model:
    """A tree with translation joints (JointModelTranslation) at the root, inside a chain and at
    a leaf, among revolute and prismatic joints: nv 14."""
    rng = np.random.default_rng(seed)
    model = Model()
    model.name = "translationtree14"
    root = _add_link(model, rng, 0, JointModelTranslation(), "base")
    a = _add_link(model, rng, root, _random_revolute(rng), "a1")
    a = _add_link(model, rng, a, JointModelTranslation(), "a2")
    a = _add_link(model, rng, a, _random_one_dof(rng), "a3")
    b = _add_link(model, rng, root, _random_revolute(rng), "b1")
    b = _add_link(model, rng, b, _random_revolute(rng), "b2")
    _add_link(model, rng, b, JointModelTranslation(), "b3")
    _add_link(model, rng, root, _random_one_dof(rng), "c1")
    return model


def zyx_tree(seed: int = 12) -> Model:
    """A tree with spherical ZYX joints (JointModelSphericalZYX) at the root, inside a chain and at
    a leaf, among revolute and prismatic joints and a translation joint: nv 16."""
    rng = np.random.default_rng(seed)
    model = Model()
    model.name = "zyxtree16"
    root = _add_link(model, rng, 0, JointModelSphericalZYX(), "base")
    a = _add_link(model, rng, root, _random_revolute(rng), "a1")
    a = _add_link(model, rng, a, JointModelSphericalZYX(), "a2")
    a = _add_link(model, rng, a, _random_one_dof(rng), "a3")
    b = _add_link(model, rng, root, JointModelTranslation(), "b1")
    b = _add_link(model, rng, b, _random_revolute(rng), "b2")
    _add_link(model, rng, b, JointModelSphericalZYX(), "b3")
    _add_link(model, rng, root, _random_one_dof(rng), "c1")
    return model


def multidof_tree(seed: int = 10) -> Model:
    """A tree with every three-dof joint type: a planar root, a spherical torso, a translation
    joint and a spherical leaf among revolute joints: nv 16."""
    from .model import JointModelPlanar, JointModelSpherical

    rng = np.random.default_rng(seed)
    model = Model()
    model.name = "multidoftree16"
    base = _add_link(model, rng, 0, JointModelPlanar(), "base")
    torso = _add_link(model, rng, base, JointModelSpherical(), "torso")
    a = _add_link(model, rng, torso, _random_revolute(rng), "a1")
    a = _add_link(model, rng, a, _random_revolute(rng), "a2")
    _add_link(model, rng, a, JointModelSpherical(), "a3")
    b = _add_link(model, rng, torso, JointModelTranslation(), "b1")
    _add_link(model, rng, b, _random_one_dof(rng), "b2")
    _add_link(model, rng, base, _random_revolute(rng), "c1")
    return model


def mimic_tree(seed: int = 12) -> Model:
    """A floating base with mimic joints (JointModelMimic): a revolute joint about x following a
    revolute joint about z (scaling 0.5, offset 0.1), a parallel gripper (the second finger
    -1 x the first), an unbounded wheel and an unbounded joint about x turning twice as fast
    (offset 0.3), an unaligned revolute joint following a revolute joint (-0.7, 0.2): nv 11,
    nvExtended 15, nq 13."""
    from .model import JointModelMimic, JointModelRUBX, JointModelRUBZ

    rng = np.random.default_rng(seed)
    model = Model()
    model.name = "mimictree"
    base = _add_link(model, rng, 0, JointModelFreeFlyer(), "base")
    a1 = _add_link(model, rng, base, JointModelRZ(), "a1")
    a2 = _add_link(model, rng, a1, JointModelRY(), "a2")
    a3 = _add_link(model, rng, a2, JointModelMimic(JointModelRX(), a1, 0.5, 0.1), "a3")
    f1 = _add_link(model, rng, a3, JointModelPX(), "finger1")
    _add_link(model, rng, a3, JointModelMimic(JointModelPX(), f1, -1.0, 0.0), "finger2")
    w = _add_link(model, rng, base, JointModelRUBZ(), "wheel")
    _add_link(model, rng, w, JointModelMimic(JointModelRUBX(), w, 2.0, 0.3), "wheel2")
    b1 = _add_link(model, rng, base, JointModelRX(), "b1")
    axis = rng.standard_normal(3)
    _add_link(model, rng, b1, JointModelMimic(JointModelRevoluteUnaligned(axis / np.linalg.norm(axis)), b1, -0.7, 0.2),
              "b2")
    return model


def chain(n: int = 100, seed: int = 4, mass_range=(0.1, 1.0)) -> Model:
    """Revolute serial chain of ``n`` links."""
    rng = np.random.default_rng(seed)
    model = Model()
    model.name = f"chain{n}"
    parent = 0
    for k in range(n):
        parent = _add_link(model, rng, parent, _random_revolute(rng), f"l{k}", mass_range)
    return model


def heterogeneous_trees(seed: int = 3):
    """The four trees of the heterogeneous batch: nv 7, 12, 32 (FF), 60 (FF)."""
    return [
        random_tree(7, False, seed * 100 + 7),
        random_tree(12, False, seed * 100 + 12),
        random_tree(32, True, seed * 100 + 32),
        random_tree(60, True, seed * 100 + 60),
    ]


# ---------------------------------------------------------------------------------------------
# inputs
# ---------------------------------------------------------------------------------------------
def random_configurations(model: Model, batch: int, rng: np.random.Generator) -> np.ndarray:
    """q of shape (batch, nq): FF position N(0,1), uniform unit quaternion; revolute angles
    U[-pi, pi] (unbounded revolute joints: their cos and sin); prismatic displacements
    U[-0.5, 0.5] m; spherical ZYX angles U[-pi, pi] with the middle one in U[-1.2, 1.2] (away
    from the joint's singularity at +-pi/2)."""
    q = np.empty((batch, model.nq))
    for jt, iq, m in zip(model.jtypes[1:], model.idx_qs[1:], model.mimic[1:]):
        if m:  # a mimic joint has no entry of its own
            continue
        if jt == JT_FF:
            q[:, iq : iq + 3] = rng.standard_normal((batch, 3))
            q[:, iq + 3 : iq + 7] = random_unit_quaternion(rng, batch)
        elif jt == JT_TR:
            q[:, iq : iq + 3] = rng.uniform(-0.5, 0.5, (batch, 3))
        elif jt == JT_ZYX:
            q[:, iq : iq + 3] = rng.uniform(-np.pi, np.pi, (batch, 3))
            q[:, iq + 1] = rng.uniform(-1.2, 1.2, batch)
        elif jt == JT_SPH:
            q[:, iq : iq + 4] = random_unit_quaternion(rng, batch)
        elif jt == JT_PL:
            th = rng.uniform(-np.pi, np.pi, batch)
            q[:, iq : iq + 2] = rng.uniform(-0.5, 0.5, (batch, 2))
            q[:, iq + 2] = np.cos(th)
            q[:, iq + 3] = np.sin(th)
        elif jt in PRISMATIC:
            q[:, iq] = rng.uniform(-0.5, 0.5, batch)
        elif jt in UNBOUNDED:
            th = rng.uniform(-np.pi, np.pi, batch)
            q[:, iq] = np.cos(th)
            q[:, iq + 1] = np.sin(th)
        else:
            q[:, iq] = rng.uniform(-np.pi, np.pi, batch)
    return q


def random_inputs(model: Model, batch: int, seed: int, v_scale=1.0, x_scale=1.0):
    """(q, v, x) with v ~ N(0, v_scale^2), x ~ N(0, x_scale^2); arrays are (batch, n)."""
    rng = np.random.default_rng(seed)
    q = random_configurations(model, batch, rng)
    v = v_scale * rng.standard_normal((batch, model.nv))
    x = x_scale * rng.standard_normal((batch, model.nv))
    return q, v, x


WORKLOADS = {
    "manipulator6r": manipulator6r,
    "humanoid32": humanoid32,
    "chain100": lambda seed=4: chain(100, seed),
}
