"""Mimic joints on the CPU: the model's sizes and indices, the oracle against known answers and
the reference's own check (unittest/rnea.cpp:350-420, unittest/crba.cpp:131-170: the mimic model
against the full model through G), the URDF ``<mimic>`` option, the model file, and the C ABI's
validation of mimic tables (no GPU call)."""
import ctypes as C

import numpy as np
import pytest

import pinocchio_gb300 as pg
from oracle.oracle import MimicOracleModel, OracleModel, symmetrize_upper
from pinocchio_gb300 import _capi
from pinocchio_gb300 import sample_models as sm
from util import rel_err


def test_sizes_and_indices():
    m = sm.mimic_tree()
    assert (m.nq, m.nv, m.nvExtended) == (13, 11, 15)
    for i, p in enumerate(m.mimic):
        if p:
            assert m.idx_qs[i] == m.idx_qs[p] and m.idx_vs[i] == m.idx_vs[p]
            assert m.nqs[i] == 0 and m.nvs[i] == 0
    assert len(m.armature) == m.nv
    q0 = m.neutral()
    assert q0.shape == (13,) and q0[6] == 1.0 and q0[m.idx_qs[7]] == 1.0  # quaternion w, wheel cos
    with pytest.raises(ValueError):
        OracleModel(m)  # the plain oracle refuses mimic tables


def _two_joint_model(mimic_scaling, mimic_offset, as_mimic=True):
    rng = np.random.default_rng(3)
    m = pg.Model()
    j1 = m.addJoint(0, pg.JointModelRZ(), sm.random_placement(rng), "j1")
    m.appendBodyToJoint(j1, sm.random_inertia(rng))
    jm = pg.JointModelMimic(pg.JointModelRX(), j1, mimic_scaling, mimic_offset) if as_mimic else pg.JointModelRX()
    j2 = m.addJoint(j1, jm, sm.random_placement(rng), "j2")
    m.appendBodyToJoint(j2, sm.random_inertia(rng))
    j3 = m.addJoint(j2, pg.JointModelRY(), sm.random_placement(rng), "j3")
    m.appendBodyToJoint(j3, sm.random_inertia(rng))
    return m


def test_scaling_zero_is_a_joint_held_at_its_offset():
    """A mimic with scaling 0 holds its joint at the offset: the dynamics of the tree with that
    joint as an ordinary joint at q = offset, v = a = 0, with its row and column dropped."""
    mm, mf = _two_joint_model(0.0, 0.37), _two_joint_model(0.0, 0.37, as_mimic=False)
    om, of = MimicOracleModel(mm), OracleModel(mf)
    rng = np.random.default_rng(4)
    q, v, a = (rng.standard_normal((8, 2)) for _ in range(3))
    ins = lambda x, val: np.insert(x, 1, val, axis=1)  # noqa: E731
    tau_f = of.rnea(ins(q, 0.37), ins(v, 0.0), ins(a, 0.0))
    assert rel_err(om.rnea(q, v, a), tau_f[:, [0, 2]]) < 1e-12
    Mf = symmetrize_upper(of.crba(ins(q, 0.37)))
    assert rel_err(om.crba(q), Mf[:, [0, 2]][:, :, [0, 2]]) < 1e-12


def test_double_rate_joint_inertia():
    """A mimic with scaling 1 about the same axis and origin as its joint turns its body at twice
    the rate: M = Izz_1 + 4 Izz_2 about the common axis, no gravity or velocity torque."""
    rng = np.random.default_rng(5)
    m = pg.Model()
    j1 = m.addJoint(0, pg.JointModelRZ(), pg.SE3.Identity(), "j1")
    Y1, Y2 = sm.random_inertia(rng), sm.random_inertia(rng)
    m.appendBodyToJoint(j1, Y1)
    j2 = m.addJoint(j1, pg.JointModelMimic(pg.JointModelRZ(), j1, 1.0, 0.0), pg.SE3.Identity(), "j2")
    m.appendBodyToJoint(j2, Y2)
    om = MimicOracleModel(m)
    izz = lambda Y: Y.matrix3()[2, 2] + Y.mass * (Y.lever[0] ** 2 + Y.lever[1] ** 2)  # noqa: E731
    q = rng.uniform(-np.pi, np.pi, (6, 1))
    v, a = rng.standard_normal((6, 1)), rng.standard_normal((6, 1))
    expected = izz(Y1) + 4.0 * izz(Y2)
    assert np.allclose(om.crba(q)[:, 0, 0], expected, rtol=1e-13)
    assert np.allclose(om.rnea(q, v, a)[:, 0], expected * a[:, 0], rtol=1e-12)


def test_two_routes_of_the_reference_recipe_agree():
    """tau = G^T (M_full G a + nle_full) (the reference's test) equals G^T rnea_full(toFull(q), G v,
    G a); the reduced M is symmetric positive definite; integrate keeps the caller's entries."""
    m = sm.mimic_tree()
    om = MimicOracleModel(m)
    q, v, a = sm.random_inputs(m, 16, 6)
    tau = om.rnea(q, v, a)
    assert rel_err(om.rnea(q, v, a, fext=np.zeros((16, m.njoints, 6))), tau) < 1e-12
    M = om.crba(q)
    assert np.allclose(M, np.swapaxes(M, 1, 2)) and np.all(np.linalg.eigvalsh(M) > 0)
    qn = om.integrate(q, 1e-3 * v)
    assert qn.shape == q.shape and rel_err(qn, q) < 1e-2


_GRIPPER = """<robot name="g">
  <link name="base"/>
  <link name="palm"><inertial><mass value="1"/><inertia ixx="0.01" ixy="0" ixz="0" iyy="0.01" iyz="0" izz="0.01"/></inertial></link>
  <link name="f1"><inertial><mass value="0.1"/><inertia ixx="0.001" ixy="0" ixz="0" iyy="0.001" iyz="0" izz="0.001"/></inertial></link>
  <link name="f2"><inertial><mass value="0.1"/><inertia ixx="0.001" ixy="0" ixz="0" iyy="0.001" iyz="0" izz="0.001"/></inertial></link>
  <joint name="wrist" type="revolute"><parent link="base"/><child link="palm"/><axis xyz="0 0 1"/>
    <limit lower="-1" upper="1" effort="1" velocity="1"/></joint>
  <joint name="left" type="prismatic"><parent link="palm"/><child link="f1"/><origin xyz="0 0.05 0"/>
    <axis xyz="0 1 0"/><limit lower="0" upper="0.04" effort="1" velocity="1"/></joint>
  <joint name="right" type="prismatic"><parent link="palm"/><child link="f2"/><origin xyz="0 -0.05 0"/>
    <axis xyz="0 1 0"/><limit lower="-0.04" upper="0" effort="1" velocity="1"/>
    <mimic joint="left" multiplier="-1" offset="0.001"/></joint>
</robot>"""


def test_urdf_mimic_option_and_model_file(tmp_path):
    plain = pg.buildModelFromXML(_GRIPPER)
    assert (plain.nq, plain.nv) == (3, 3) and not plain.has_mimic()
    m = pg.buildModelFromXML(_GRIPPER, mimic=True)
    assert (m.nq, m.nv, m.nvExtended) == (2, 2, 3) and m.mimic == [0, 0, 0, 2]
    assert m.mimic_scaling[3] == -1.0 and m.mimic_offset[3] == 0.001
    path = str(tmp_path / "g.npz")
    pg.save_model(m, path)
    back = pg.load_model(path)
    assert back.mimic == m.mimic and back.mimic_scaling == m.mimic_scaling and back.nv == 2
    # the mimic model is the plain model with right = -left + 0.001
    om, op = MimicOracleModel(m), OracleModel(plain)
    rng = np.random.default_rng(7)
    q, v, a = (rng.standard_normal((8, 2)) for _ in range(3))
    full = lambda x, off: np.concatenate([x, -x[:, 1:2] + off], axis=1)  # noqa: E731
    G = np.array([[1.0, 0.0], [0.0, 1.0], [0.0, -1.0]])
    tau_p = op.rnea(full(q, 0.001), full(v, 0.0), full(a, 0.0))
    assert rel_err(om.rnea(q, v, a), tau_p @ G) < 1e-12
    bad = _GRIPPER.replace('joint="left"', 'joint="nope"')
    with pytest.raises(ValueError):
        pg.buildModelFromXML(bad, mimic=True)


def _create(L, t):
    d, keep = _capi.make_desc(t)
    h = C.c_void_p()
    rc = L.gb_model_create(C.byref(d), C.byref(h))
    return rc, keep


@pytest.mark.parametrize("edit,msg", [
    (lambda t: t["mimic"].__setitem__(2, 5), b"after the joint it mimics"),
    (lambda t: t["mimic"].__setitem__(6, 4), b"mimic joint itself"),  # joint 4 mimics joint 2
    (lambda t: t["mimic"].__setitem__(2, 1), b"one-dof joints"),  # joint 1 is the free-flyer
    (lambda t: t["mimic"].__setitem__(8, 5), b"same nq"),  # an unbounded joint mimicking a prismatic one
])
def test_capi_rejects_bad_mimic_tables(edit, msg):
    L = _capi.lib()
    t = {k: np.array(v, copy=True) for k, v in sm.mimic_tree().tables().items()}
    edit(t)
    rc, _ = _create(L, t)
    assert rc == _capi.GB_ERR_INVALID_ARGUMENT
    assert msg in L.gb_last_error()
