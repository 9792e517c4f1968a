"""URDF loading (reference src/parsers/urdf/model.cpp: depth-first walk from the
root link, moving joints placed through any fixed joints, links appended as
bodies to the joint that moves them, fixed joints merged into the parent body,
an optional free-flyer root joint) and the model's on-disk format, checked on
the CPU against models built with the construction API and through the oracle."""
import numpy as np
import pytest

import pinocchio_gb300 as pg
from oracle.oracle import OracleModel
from pinocchio_gb300 import model as gm
from pinocchio_gb300 import sample_models as sm
from util import MODELS, rel_err

_AX = {gm.JT_RX: "1 0 0", gm.JT_RY: "0 1 0", gm.JT_RZ: "0 0 1", gm.JT_PX: "1 0 0", gm.JT_PY: "0 1 0", gm.JT_PZ: "0 0 1"}


def _axis_text(model, i):
    if model.jtypes[i] in (gm.JT_RU, gm.JT_PU):
        return " ".join(_f(x) for x in model.axes[i])
    return _AX[model.jtypes[i]]


def _rpy_of(R):
    """roll, pitch, yaw with R = Rz(yaw) Ry(pitch) Rx(roll)."""
    pitch = np.arcsin(-np.clip(R[2, 0], -1.0, 1.0))
    roll = np.arctan2(R[2, 1], R[2, 2])
    yaw = np.arctan2(R[1, 0], R[0, 0])
    return roll, pitch, yaw


def _f(x):
    return repr(float(x))


def _origin(P):
    r, p, y = _rpy_of(P.rotation)
    t = P.translation
    return f'<origin xyz="{_f(t[0])} {_f(t[1])} {_f(t[2])}" rpy="{_f(r)} {_f(p)} {_f(y)}"/>'


def _inertial(Y):
    I = Y.matrix3()
    c = Y.lever
    return (f'<inertial><origin xyz="{_f(c[0])} {_f(c[1])} {_f(c[2])}"/><mass value="{_f(Y.mass)}"/>'
            f'<inertia ixx="{_f(I[0, 0])}" ixy="{_f(I[0, 1])}" ixz="{_f(I[0, 2])}" iyy="{_f(I[1, 1])}" '
            f'iyz="{_f(I[1, 2])}" izz="{_f(I[2, 2])}"/></inertial>')


def to_urdf(model, skip_free_flyer=True):
    """URDF of a model of one-dof joints (the root free-flyer, if any, left to root_joint)."""
    out = ['<robot name="exported">', '<link name="base"/>']
    link_of = {0: "base"}
    for i in range(1, model.njoints):
        if model.jtypes[i] == gm.JT_FF:
            assert skip_free_flyer and model.parents[i] == 0
            link_of[i] = "base"
            out[1] = f'<link name="base">{_inertial(model.inertias[i])}</link>'
            continue
        link_of[i] = f"link{i}"
        out.append(f'<link name="link{i}">{_inertial(model.inertias[i])}</link>')
        kind = "prismatic" if model.jtypes[i] in gm.PRISMATIC else "revolute"
        out.append(f'<joint name="{model.names[i]}" type="{kind}"><parent link="{link_of[model.parents[i]]}"/>'
                   f'<child link="link{i}"/>{_origin(model.jointPlacements[i])}<axis xyz="{_axis_text(model, i)}"/>'
                   f'<limit lower="-3" upper="3" effort="1" velocity="1"/></joint>')
    out.append("</robot>")
    return "\n".join(out)


@pytest.mark.parametrize("name", ["manipulator6r", "tree12", "chain100", "mixedtree12", "unaligned14"])
def test_urdf_round_trip(name):
    model = MODELS[name]()
    back = pg.buildModelFromXML(to_urdf(model))
    a, b = model.tables(), back.tables()
    assert np.array_equal(a["parents"], b["parents"]) and np.array_equal(a["jtype"], b["jtype"])
    assert np.abs(a["placement"] - b["placement"]).max() < 1e-12
    assert np.abs(a["inertia"] - b["inertia"]).max() < 1e-12
    assert np.abs(a["axis"] - b["axis"]).max() < 1e-15


def test_urdf_free_flyer_root():
    model = MODELS["humanoid32"]()  # the free-flyer sits at the root with its own placement
    back = pg.buildModelFromXML(to_urdf(model), root_joint=pg.JointModelFreeFlyer())
    a, b = model.tables(), back.tables()
    assert np.array_equal(a["parents"], b["parents"]) and np.array_equal(a["jtype"], b["jtype"])
    assert np.abs(a["placement"][2:] - b["placement"][2:]).max() < 1e-12  # joints below the root
    assert np.abs(a["inertia"] - b["inertia"]).max() < 1e-12
    om, ob = OracleModel(model), OracleModel(back)
    q, v, x = sm.random_inputs(model, 8, 3)
    # the root placement only re-expresses the free-flyer's q: joint-space dynamics in the root frame agree
    assert rel_err(om.crba(q)[:, 6:, 6:], ob.crba(q)[:, 6:, 6:]) < 1e-12


_TWO_LINK = """<robot name="two">
  <link name="base"/>
  <link name="upper"><inertial><origin xyz="0.1 0 -0.2" rpy="0.1 0.2 0.3"/><mass value="1.5"/>
    <inertia ixx="0.02" ixy="0.001" ixz="0" iyy="0.03" iyz="0.002" izz="0.01"/></inertial></link>
  <link name="tool"><inertial><origin xyz="0 0.05 0"/><mass value="0.4"/>
    <inertia ixx="0.001" ixy="0" ixz="0" iyy="0.002" iyz="0" izz="0.003"/></inertial></link>
  <link name="lower"><inertial><origin xyz="0 0 -0.25"/><mass value="0.8"/>
    <inertia ixx="0.01" ixy="0" ixz="0" iyy="0.01" iyz="0" izz="0.004"/></inertial></link>
  <joint name="shoulder" type="continuous"><parent link="base"/><child link="upper"/>
    <origin xyz="0 0 1" rpy="0 0 0.4"/><axis xyz="0 AXIS"/></joint>
  <joint name="mount" type="fixed"><parent link="upper"/><child link="tool"/>
    <origin xyz="0.05 0 -0.1" rpy="0.3 0 0"/></joint>
  <joint name="elbow" type="revolute"><parent link="tool"/><child link="lower"/>
    <origin xyz="0 0.02 -0.3" rpy="0 0.5 0"/><axis xyz="1 0 0"/>
    <limit lower="-2" upper="2" effort="1" velocity="1"/></joint>
</robot>"""


def _unbounded_q(theta, rest):
    return np.concatenate([np.cos(theta)[:, None], np.sin(theta)[:, None], rest], axis=1)


def test_urdf_fixed_joint_and_negative_axis():
    """A fixed joint merges its link into the parent body and carries its origin to
    the next joint; the continuous shoulder is an unbounded revolute joint (q = (cos, sin),
    as the reference's JointModelRUBZ); an axis -z gives the +z joint's dynamics with that joint's
    angle negated (tau_-(q, v, a) = D tau_+(D q, D v, D a), D = diag(-1, 1))."""
    plus = pg.buildModelFromXML(_TWO_LINK.replace("AXIS", "0 1"))
    minus = pg.buildModelFromXML(_TWO_LINK.replace("AXIS", "0 -1"))
    assert plus.njoints == 3 and plus.jtypes[1:] == [gm.JT_RUBZ, gm.JT_RX] and (plus.nq, plus.nv) == (3, 2)
    assert minus.jtypes[1:] == [gm.JT_RUBU, gm.JT_RX]
    assert abs(plus.inertias[1].mass - 1.9) < 1e-15  # upper + tool
    rng = np.random.default_rng(1)
    th, qe = rng.uniform(-np.pi, np.pi, 16), rng.standard_normal((16, 1))
    v, a = (rng.standard_normal((16, 2)) for _ in range(2))
    D = np.array([-1.0, 1.0])
    tp = OracleModel(plus).rnea(_unbounded_q(-th, qe), v * D, a * D)
    tm = OracleModel(minus).rnea(_unbounded_q(th, qe), v, a)
    assert rel_err(tm, tp * D) < 1e-12
    # the same tree from the construction API: the tool merged into the shoulder body
    m = pg.Model()
    j1 = m.addJoint(0, pg.JointModelRZ(), pg.SE3(gm_rz(0.4), [0, 0, 1]), "shoulder")
    upper = pg.Inertia(1.5, [0, 0, 0], [[0.02, 0.001, 0], [0.001, 0.03, 0.002], [0, 0.002, 0.01]])
    m.appendBodyToJoint(j1, upper, pg.SE3(rpy(0.1, 0.2, 0.3), [0.1, 0, -0.2]))
    mount = pg.SE3(rpy(0.3, 0, 0), [0.05, 0, -0.1])
    m.appendBodyToJoint(j1, pg.Inertia(0.4, [0, 0.05, 0], np.diag([0.001, 0.002, 0.003])), mount)
    elbow = pg.SE3(mount.rotation @ rpy(0, 0.5, 0), mount.rotation @ np.array([0, 0.02, -0.3]) + mount.translation)
    j2 = m.addJoint(j1, pg.JointModelRX(), elbow, "elbow")
    m.appendBodyToJoint(j2, pg.Inertia(0.8, [0, 0, -0.25], np.diag([0.01, 0.01, 0.004])))
    q = np.concatenate([th[:, None], qe], axis=1)
    assert rel_err(OracleModel(m).rnea(q, v, a), OracleModel(plus).rnea(_unbounded_q(th, qe), v, a)) < 1e-12


def test_urdf_prismatic_negative_axis():
    """A prismatic joint along -x gives the +x joint's dynamics with its coordinate negated."""
    doc = """<robot name="slide">
  <link name="base"/>
  <link name="cart"><inertial><origin xyz="0.1 0 0.05"/><mass value="2.0"/>
    <inertia ixx="0.02" ixy="0" ixz="0" iyy="0.03" iyz="0" izz="0.04"/></inertial></link>
  <link name="pole"><inertial><origin xyz="0 0 -0.4"/><mass value="0.5"/>
    <inertia ixx="0.01" ixy="0" ixz="0" iyy="0.01" iyz="0" izz="0.002"/></inertial></link>
  <joint name="rail" type="prismatic"><parent link="base"/><child link="cart"/>
    <origin xyz="0 0 0.3" rpy="0 0 0.2"/><axis xyz="AXIS"/>
    <limit lower="-1" upper="1" effort="1" velocity="1"/></joint>
  <joint name="hinge" type="continuous"><parent link="cart"/><child link="pole"/>
    <origin xyz="0.1 0 0"/><axis xyz="0 1 0"/></joint>
</robot>"""
    plus = pg.buildModelFromXML(doc.replace("AXIS", "1 0 0"))
    minus = pg.buildModelFromXML(doc.replace("AXIS", "-1 0 0"))
    assert plus.jtypes[1:] == [gm.JT_PX, gm.JT_RUBY] and minus.jtypes[1:] == [gm.JT_PU, gm.JT_RUBY]
    rng = np.random.default_rng(2)
    x, th = rng.standard_normal((16, 1)), rng.uniform(-np.pi, np.pi, 16)
    v, a = (rng.standard_normal((16, 2)) for _ in range(2))
    D = np.array([-1.0, 1.0])
    hinge = _unbounded_q(th, np.zeros((16, 0)))
    tp = OracleModel(plus).rnea(np.concatenate([-x, hinge], axis=1), v * D, a * D)
    tm = OracleModel(minus).rnea(np.concatenate([x, hinge], axis=1), v, a)
    assert rel_err(tm, tp * D) < 1e-12


def rpy(r, p, y):
    cr, sr, cp, sp, cy, sy = np.cos(r), np.sin(r), np.cos(p), np.sin(p), np.cos(y), np.sin(y)
    return (np.array([[cy, -sy, 0], [sy, cy, 0], [0, 0, 1]]) @ np.array([[cp, 0, sp], [0, 1, 0], [-sp, 0, cp]])
            @ np.array([[1, 0, 0], [0, cr, -sr], [0, sr, cr]]))


def gm_rz(t):
    return rpy(0, 0, t)


@pytest.mark.parametrize("bad,msg", [
    ('<link name="c"/><joint name="r" type="revolute"><parent link="a"/><child link="c"/></joint>'
     '<joint name="s" type="floating"><parent link="c"/><child link="b"/></joint>', "not supported"),
    ('<joint name="s" type="revolute"><parent link="a"/><child link="b"/><axis xyz="0 0 0"/></joint>', "zero axis"),
])
def test_urdf_unsupported(bad, msg):
    xml = f'<robot name="x"><link name="a"/><link name="b"/>{bad}</robot>'
    with pytest.raises(ValueError, match=msg):
        pg.buildModelFromXML(xml)


@pytest.mark.parametrize("kind", ["revolute", "prismatic"])
def test_urdf_unaligned_axis(kind):
    """An axis off the unit axes (negative ones included) gives the unaligned joint with the
    normalised axis, as the reference's extractCartesianAxis; an axis equal to a unit axis
    up to 1e-12 (relative) gives the aligned joint."""
    doc = f"""<robot name="u"><link name="a"/><link name="b"><inertial><mass value="1"/>
      <inertia ixx="0.1" ixy="0" ixz="0" iyy="0.1" iyz="0" izz="0.1"/></inertial></link>
      <joint name="s" type="{kind}"><parent link="a"/><child link="b"/><axis xyz="AXIS"/></joint></robot>"""
    m = pg.buildModelFromXML(doc.replace("AXIS", "0 3 4"))
    assert m.jtypes[1] == (gm.JT_PU if kind == "prismatic" else gm.JT_RU)
    assert np.allclose(m.axes[1], [0, 0.6, 0.8], rtol=0, atol=1e-16)
    m = pg.buildModelFromXML(doc.replace("AXIS", "0 0 -1"))
    assert m.jtypes[1] == (gm.JT_PU if kind == "prismatic" else gm.JT_RU)
    m = pg.buildModelFromXML(doc.replace("AXIS", "0 1e-14 1"))
    assert m.jtypes[1] == (gm.JT_PZ if kind == "prismatic" else gm.JT_RZ)


@pytest.mark.parametrize("name", ["tree12", "unaligned14"])
def test_urdf_file_and_model_file(tmp_path, name):
    model = MODELS[name]()
    path = tmp_path / "tree.urdf"
    path.write_text(to_urdf(model))
    loaded = pg.buildModelFromUrdf(str(path))
    npz = tmp_path / "tree.npz"
    pg.save_model(loaded, str(npz))
    back = pg.load_model(str(npz))
    for k, v in loaded.tables().items():
        assert np.array_equal(v, back.tables()[k]), k
    assert back.names == loaded.names


def test_urdf_planar_and_floating():
    """``planar`` gives the planar joint (the axis ignored), a root ``floating`` joint the
    free-flyer, as the reference's UrdfVisitor::addJointAndBody (model.hxx:255-296); the
    dynamics of the loaded model match the same model built through the construction API."""
    inertial = ('<inertial><origin xyz="0.1 0.2 0.3"/><mass value="2"/>'
                '<inertia ixx="0.3" ixy="0.01" ixz="0" iyy="0.2" iyz="0.02" izz="0.4"/></inertial>')
    doc = f"""<robot name="p"><link name="w"/><link name="a">{inertial}</link><link name="b">{inertial}</link>
      <joint name="f" type="floating"><parent link="w"/><child link="a"/><origin xyz="0 0 1"/></joint>
      <joint name="s" type="planar"><parent link="a"/><child link="b"/><origin xyz="0.5 0 0"/>
      <axis xyz="1 0 0"/></joint></robot>"""
    m = pg.buildModelFromXML(doc)
    assert m.jtypes[1:] == [gm.JT_FF, gm.JT_PL] and m.nq == 11 and m.nv == 9
    Y = gm.Inertia(2.0, np.array([0.1, 0.2, 0.3]), np.array([[0.3, 0.01, 0], [0.01, 0.2, 0.02], [0, 0.02, 0.4]]))
    ref = gm.Model()
    j1 = ref.addJoint(0, gm.JointModelFreeFlyer(), gm.SE3(np.eye(3), np.array([0.0, 0, 1])), "f")
    ref.appendBodyToJoint(j1, Y, gm.SE3.Identity())
    j2 = ref.addJoint(j1, gm.JointModelPlanar(), gm.SE3(np.eye(3), np.array([0.5, 0, 0])), "s")
    ref.appendBodyToJoint(j2, Y, gm.SE3.Identity())
    q, v, a = sm.random_inputs(m, 8, 3)
    assert rel_err(OracleModel(m).rnea(q, v, a), OracleModel(ref).rnea(q, v, a)) < 1e-14
