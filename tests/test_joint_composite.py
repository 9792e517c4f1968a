"""JointModelComposite in the construction API (reference multibody/joint/joint-composite.hpp:286-290,
joint-composite.hxx:40-77: M = prod_k placement_k M_k(q_k)) on the CPU: the chain Model.addJoint
makes of it (names, types, sizes, the index it returns), the placement of its frame against the
reference's product, and the errors."""
import numpy as np
import pytest

import pinocchio_gb300 as pg
from oracle.oracle import OracleModel
from pinocchio_gb300 import model as gm
from pinocchio_gb300 import sample_models as sm
from util import rel_err


def _rot(axis, angle):
    a = np.asarray(axis, dtype=np.float64)
    a = a / np.linalg.norm(a)
    K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    return np.eye(3) + np.sin(angle) * K + (1 - np.cos(angle)) * K @ K


def _T(P: pg.SE3):
    T = np.eye(4)
    T[:3, :3], T[:3, 3] = P.rotation, P.translation
    return T


def _J(R=np.eye(3), t=(0.0, 0.0, 0.0)):
    T = np.eye(4)
    T[:3, :3], T[:3, 3] = R, t
    return T


def test_composite_is_the_product_of_its_components():
    rng = np.random.default_rng(8)
    P, P0, P1, P2 = (sm.random_placement(rng) for _ in range(4))
    axis = np.array([0.3, -0.5, 0.8]) / np.linalg.norm([0.3, -0.5, 0.8])
    comp = pg.JointModelComposite(pg.JointModelRZ(), P0)
    comp.addJoint(pg.JointModelPrismaticUnaligned(axis), P1).addJoint(pg.JointModelSphericalZYX(), P2)
    assert (comp.nq, comp.nv) == (5, 5)
    m = pg.Model()
    base = m.addJoint(0, pg.JointModelRY(), pg.SE3.Identity(), "base")
    m.appendBodyToJoint(base, sm.random_inertia(rng))
    jid = m.addJoint(base, comp, P, "hip")
    m.appendBodyToJoint(jid, sm.random_inertia(rng))
    child = m.addJoint(jid, pg.JointModelRX(), sm.random_placement(rng), "knee")
    m.appendBodyToJoint(child, sm.random_inertia(rng))
    assert m.names == ["universe", "base", "hip_0", "hip_1", "hip", "knee"] and jid == 4
    assert m.jtypes[1:] == [gm.JT_RY, gm.JT_RZ, gm.JT_PU, gm.JT_ZYX, gm.JT_RX]
    assert m.parents == [0, 0, 1, 2, 3, 4] and (m.nq, m.nv) == (7, 7)
    assert all(m.inertias[k].mass == 0.0 for k in (2, 3))  # massless links
    q = rng.uniform(-1.0, 1.0, (5, m.nq))
    oMi, _, _ = OracleModel(m).forward_kinematics(q)
    for b in range(5):
        z, y, x = q[b, 3:6]
        M = (_T(P) @ _T(P0) @ _J(_rot([0, 0, 1], q[b, 1])) @ _T(P1) @ _J(t=axis * q[b, 2]) @ _T(P2)
             @ _J(_rot([0, 0, 1], z) @ _rot([0, 1, 0], y) @ _rot([1, 0, 0], x)))
        Mb = _J(_rot([0, 1, 0], q[b, 0])) @ M
        got = np.eye(4)
        got[:3, :3], got[:3, 3] = oMi[b, 4, :9].reshape(3, 3), oMi[b, 4, 9:]
        assert np.allclose(got, Mb, atol=1e-13)
    # the same chain built joint by joint has the same dynamics
    ref = pg.Model()
    r1 = ref.addJoint(0, pg.JointModelRY(), pg.SE3.Identity(), "base")
    ref.appendBodyToJoint(r1, m.inertias[1])
    r2 = ref.addJoint(r1, pg.JointModelRZ(), P * P0, "a")
    r3 = ref.addJoint(r2, pg.JointModelPrismaticUnaligned(axis), P1, "b")
    r4 = ref.addJoint(r3, pg.JointModelSphericalZYX(), P2, "c")
    ref.appendBodyToJoint(r4, m.inertias[4])
    r5 = ref.addJoint(r4, pg.JointModelRX(), m.jointPlacements[5], "d")
    ref.appendBodyToJoint(r5, m.inertias[5])
    qq, v, a = sm.random_inputs(m, 6, 2)
    assert rel_err(OracleModel(m).rnea(qq, v, a), OracleModel(ref).rnea(qq, v, a)) < 1e-14


def test_composite_errors():
    m = pg.Model()
    with pytest.raises(ValueError, match="without components"):
        m.addJoint(0, pg.JointModelComposite(), pg.SE3.Identity(), "c")
    with pytest.raises(ValueError, match="plain joint models"):
        pg.JointModelComposite(pg.JointModelComposite(pg.JointModelRX()))
