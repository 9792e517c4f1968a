"""The MJCF loader (a subset of the reference's src/parsers/mjcf/mjcf-graph.cpp) on the CPU:
documents against the same trees built with the construction API (tables equal, and the
oracle's dynamics equal), the orientation forms (quat / axisangle / euler, degrees and
radians), welded bodies, joint positions inside a body, armature, and the features outside
the subset raising ValueError."""
import numpy as np
import pytest

from oracle.oracle import OracleModel
from pinocchio_gb300 import model as gm
from pinocchio_gb300 import sample_models as sm
from pinocchio_gb300.mjcf import buildModelFromMJCF, buildModelFromMJCFXML
from util import rel_err

DOC = """<mujoco model="walker">
  <compiler angle="radian"/>
  <worldbody>
    <body name="base" pos="0 0 1">
      <freejoint name="root"/>
      <inertial pos="0.01 0 0.02" mass="5" diaginertia="0.1 0.2 0.3"/>
      <body name="torso" pos="0 0 0.3" quat="0.9238795325112867 0 0.3826834323650898 0">
        <joint name="waist" type="hinge" axis="0 0 1" armature="0.05"/>
        <inertial pos="0 0 0.1" quat="1 0 0 0" mass="2" diaginertia="0.02 0.03 0.04"/>
        <body name="head" pos="0 0 0.25">
          <inertial pos="0 0 0.05" mass="0.8" fullinertia="0.01 0.012 0.009 0.001 0 0.0005"/>
        </body>
        <body name="arm" pos="0.2 0 0.1" axisangle="1 0 0 0.3">
          <joint name="shoulder" type="hinge" axis="0 1 1" pos="0 0 0.05"/>
          <inertial pos="0 0 -0.1" mass="1" diaginertia="0.01 0.01 0.002"/>
          <body name="forearm" pos="0 0 -0.25" euler="0.1 0.2 0.3">
            <joint name="elbow" type="hinge" axis="1 0 0"/>
            <inertial pos="0 0 -0.1" mass="0.6" diaginertia="0.005 0.005 0.001"/>
          </body>
        </body>
      </body>
      <body name="leg" pos="0 -0.1 -0.1">
        <joint name="hip" type="slide" axis="0 0 -1"/>
        <inertial pos="0 0 -0.2" mass="1.5" diaginertia="0.02 0.02 0.003"/>
        <body name="shin" pos="0 0 -0.4">
          <joint name="knee" type="hinge" axis="0 1 0"/>
          <inertial pos="0 0 -0.2" mass="1" diaginertia="0.01 0.01 0.002"/>
        </body>
      </body>
    </body>
  </worldbody>
</mujoco>"""


def _rot(axis, angle):
    a = np.asarray(axis, dtype=float) / np.linalg.norm(axis)
    K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    return np.eye(3) + np.sin(angle) * K + (1 - np.cos(angle)) * K @ K


def _Y(mass, pos, I, R=np.eye(3)):
    return gm.Inertia(mass, np.zeros(3), R @ I @ R.T).se3_action(gm.SE3(np.eye(3), pos))


def reference_walker():
    """The same tree through the construction API (addJoint / appendBodyToJoint)."""
    m = gm.Model()
    base = m.addJoint(0, gm.JointModelFreeFlyer(), gm.SE3(np.eye(3), [0, 0, 1]), "root")
    m.appendBodyToJoint(base, _Y(5, [0.01, 0, 0.02], np.diag([0.1, 0.2, 0.3])))
    Rt = _rot([0, 1, 0], np.pi / 4)
    waist = m.addJoint(base, gm.JointModelRZ(), gm.SE3(Rt, [0, 0, 0.3]), "waist")
    m.armature[m.idx_vs[waist]] = 0.05
    m.appendBodyToJoint(waist, _Y(2, [0, 0, 0.1], np.diag([0.02, 0.03, 0.04])))
    Ih = np.array([[0.01, 0.001, 0], [0.001, 0.012, 0.0005], [0, 0.0005, 0.009]])
    m.appendBodyToJoint(waist, _Y(0.8, [0, 0, 0.05], Ih), gm.SE3(np.eye(3), [0, 0, 0.25]))
    Ra = _rot([1, 0, 0], 0.3)
    sh = m.addJoint(waist, gm.JointModelRevoluteUnaligned(np.array([0, 1, 1]) / np.sqrt(2)),
                    gm.SE3(Ra, [0.2, 0, 0.1] + Ra @ [0, 0, 0.05]), "shoulder")
    m.appendBodyToJoint(sh, _Y(1, [0, 0, -0.1], np.diag([0.01, 0.01, 0.002])), gm.SE3(np.eye(3), [0, 0, -0.05]))
    Re = _rot([1, 0, 0], 0.1) @ _rot([0, 1, 0], 0.2) @ _rot([0, 0, 1], 0.3)
    el = m.addJoint(sh, gm.JointModelRX(), gm.SE3(Re, [0, 0, -0.3]), "elbow")
    m.appendBodyToJoint(el, _Y(0.6, [0, 0, -0.1], np.diag([0.005, 0.005, 0.001])))
    hip = m.addJoint(base, gm.JointModelPrismaticUnaligned(np.array([0, 0, -1.0])), gm.SE3(np.eye(3), [0, -0.1, -0.1]), "hip")
    m.appendBodyToJoint(hip, _Y(1.5, [0, 0, -0.2], np.diag([0.02, 0.02, 0.003])))
    kn = m.addJoint(hip, gm.JointModelRY(), gm.SE3(np.eye(3), [0, 0, -0.4]), "knee")
    m.appendBodyToJoint(kn, _Y(1, [0, 0, -0.2], np.diag([0.01, 0.01, 0.002])))
    return m


def _same(a, b, tol=1e-12):
    ta, tb = a.tables(), b.tables()
    assert ta.keys() == tb.keys()
    for k in ta:
        assert np.allclose(ta[k], tb[k], rtol=0, atol=tol), k


def test_walker_matches_construction_api(tmp_path):
    m = buildModelFromMJCFXML(DOC)
    ref = reference_walker()
    assert m.names[1:] == ["root", "waist", "shoulder", "elbow", "hip", "knee"]
    _same(m, ref)
    p = tmp_path / "walker.xml"
    p.write_text(DOC)
    _same(buildModelFromMJCF(str(p)), ref)
    om, oref = OracleModel(m), OracleModel(ref)
    q, v, a = sm.random_inputs(m, 8, 3)
    assert rel_err(om.rnea(q, v, a), oref.rnea(q, v, a)) < 1e-13


def test_orientation_forms_and_units():
    def doc(compiler, attr):
        return f"""<mujoco>{compiler}<worldbody>
          <body name="a" {attr}><joint type="hinge" axis="1 0 0"/>
            <inertial pos="0.1 0 0" mass="1" diaginertia="0.1 0.2 0.3"/></body>
        </worldbody></mujoco>"""
    c = np.cos(np.pi / 6 / 2)
    s = np.sin(np.pi / 6 / 2)
    forms = [doc("", f'quat="{c} 0 0 {s}"'), doc("", 'axisangle="0 0 1 30"'), doc("", 'euler="0 0 30"'),
             doc('<compiler angle="radian"/>', f'axisangle="0 0 1 {np.pi / 6}"'),
             doc('<compiler eulerseq="zyx"/>', 'euler="30 0 0"')]
    models = [buildModelFromMJCFXML(x) for x in forms]
    for m in models[1:]:
        _same(m, models[0])
    R = models[0].tables()["placement"][1, :9].reshape(3, 3)
    assert np.allclose(R, _rot([0, 0, 1], np.pi / 6), atol=1e-12)


@pytest.mark.parametrize("snippet, msg", [
    ('<worldbody><body name="a"><freejoint/><joint type="slide"/><inertial mass="1" diaginertia="1 1 1"/></body>'
     '</worldbody>', "composite joint cannot hold a free joint"),
    ('<default><default><joint/></default></default><worldbody/>', "Class does not have a name"),
    ('<worldbody><body name="a" childclass="x"><joint/></body></worldbody>', "unknown class"),
    ('<worldbody><body name="a"><joint/><geom type="box" size="0.1 0.1 0.1" shellinertia="true"/></body></worldbody>',
     "Shell inertia"),
    ('<worldbody><body name="a"><joint/><inertial mass="1" diaginertia="1 1 1"/>'
     '<body name="b"><freejoint/><inertial mass="1" diaginertia="1 1 1"/></body></body></worldbody>', "free"),
    ('<worldbody><body name="a" zaxis="0 1 0"><joint/><inertial mass="1" diaginertia="1 1 1"/></body></worldbody>', "zaxis"),
    ('<worldbody><body name="a"><joint/><inertial mass="1" diaginertia="1 1 1"/>'
     '<frame pos="0 0 1"><body name="b"><joint/><inertial mass="1" diaginertia="1 1 1"/></body></frame>'
     '</body></worldbody>', "frame"),
    ('<worldbody><group><body name="a"><joint/><inertial mass="1" diaginertia="1 1 1"/></body></group></worldbody>',
     "holds bodies"),
])
def test_outside_the_subset_raises(snippet, msg):
    with pytest.raises(ValueError, match=msg):
        buildModelFromMJCFXML(f"<mujoco>{snippet}</mujoco>")
    with pytest.raises(ValueError, match="mujoco"):
        buildModelFromMJCFXML("<robot/>")


def test_inertia_from_geom_false_needs_an_inertial():
    """inertiafromgeom="false" without an <inertial> is an error (mjcf-graph.cpp:416-419)."""
    with pytest.raises(ValueError, match="no inertia was found"):
        buildModelFromMJCFXML("""<mujoco><compiler inertiafromgeom="false"/><worldbody>
          <body name="a"><joint/><geom type="sphere" size="0.1"/></body></worldbody></mujoco>""")


def test_defaults_and_classes():
    """Attribute precedence: top-level default < body childclass (inherited by nested bodies) <
    element class < the element's own attributes; nested classes inherit from their enclosing
    default (mjcf-graph.cpp:35-52, 239-285)."""
    m = buildModelFromMJCFXML("""<mujoco><default>
        <joint type="hinge" axis="0 1 0" armature="0.1"/>
        <default class="slider"><joint type="slide" axis="1 0 0"/>
          <default class="zslider"><joint axis="0 0 1" armature="0.3"/></default></default>
        <default class="heavy"><joint armature="0.5"/></default></default>
      <worldbody>
        <body name="a"><joint/><inertial mass="1" diaginertia="1 1 1"/>
          <body name="b" childclass="slider"><joint/><inertial mass="1" diaginertia="1 1 1"/>
            <body name="c"><joint class="zslider"/><inertial mass="1" diaginertia="1 1 1"/>
              <body name="d"><joint class="heavy" axis="0 0 1" type="hinge"/><inertial mass="1" diaginertia="1 1 1"/>
              </body></body></body></body></worldbody></mujoco>""")
    assert m.jtypes[1:] == [gm.JT_RY, gm.JT_PX, gm.JT_PZ, gm.JT_RZ]
    assert np.allclose(m.armature, [0.1, 0.1, 0.3, 0.5])


def _solid(kind, m, size):
    """Solid inertias about the center (diagonal), by the textbook formulas."""
    if kind == "sphere":
        r = size[0]
        return np.diag([0.4 * m * r * r] * 3)
    if kind == "box":  # full side lengths
        x, y, z = size
        return np.diag([m * (y * y + z * z), m * (x * x + z * z), m * (x * x + y * y)]) / 12
    if kind == "cylinder":  # radius, full length
        r, L = size
        return np.diag([m * (3 * r * r + L * L) / 12] * 2 + [m * r * r / 2])
    raise ValueError(kind)


def test_inertia_from_geoms():
    """A body's inertia from its geoms (inertiafromgeom auto, no <inertial>): a sphere from its
    density (default 1000), a box given its mass, a cylinder placed by fromto; a visual geom
    (contype = conaffinity = 0) does not count; the geom class defaults apply."""
    m = buildModelFromMJCFXML("""<mujoco><default><default class="vis"><geom contype="0" conaffinity="0"/></default>
      </default><worldbody><body name="a"><joint axis="0 0 1"/>
        <geom type="sphere" size="0.1" pos="0.2 0 0"/>
        <geom type="box" size="0.1 0.2 0.3" mass="3" pos="0 0.5 0" euler="0 0 90"/>
        <geom type="cylinder" size="0.05" fromto="0 0 0 0 0 0.4" density="500"/>
        <geom class="vis" type="sphere" size="5"/></body></worldbody></mujoco>""")
    m_s = 1000 * 4.0 / 3 * np.pi * 0.1 ** 3
    m_c = 500 * np.pi * 0.05 ** 2 * 0.4
    Rz = np.array([[0.0, -1, 0], [1, 0, 0], [0, 0, 1]])
    parts = [gm.Inertia(m_s, np.zeros(3), _solid("sphere", m_s, [0.1])).se3_action(gm.SE3(np.eye(3), np.array([0.2, 0, 0]))),
             gm.Inertia(3.0, np.zeros(3), _solid("box", 3.0, [0.2, 0.4, 0.6])).se3_action(gm.SE3(Rz, np.array([0, 0.5, 0]))),
             gm.Inertia(m_c, np.zeros(3), _solid("cylinder", m_c, [0.05, 0.4])).se3_action(gm.SE3(np.eye(3), np.array([0, 0, 0.2])))]
    want = parts[0] + parts[1] + parts[2]
    got = m.inertias[1]
    assert np.isclose(got.mass, m_s + 3.0 + m_c)
    assert np.allclose(got.lever, want.lever, atol=1e-14)
    assert np.allclose(got.matrix3(), want.matrix3(), atol=1e-13)


def test_capsule_inertia_and_fromto_orientation():
    """A capsule along x given by fromto: mass from the volume of a cylinder and two half spheres, the
    reference's capsule inertia (spatial/inertia.hpp FromCapsule) rotated so that its axis is x."""
    m = buildModelFromMJCFXML("""<mujoco><worldbody><body name="a"><joint axis="0 0 1"/>
        <geom type="capsule" size="0.05" fromto="-0.2 0 0 0.2 0 0"/></body></worldbody></mujoco>""")
    r, h = 0.05, 0.4
    vol = np.pi * r * r * h + 4.0 / 3 * np.pi * r ** 3
    Y = m.inertias[1]
    assert np.isclose(Y.mass, 1000 * vol)
    assert np.allclose(Y.lever, 0, atol=1e-15)
    I = Y.matrix3()
    assert np.isclose(I[1, 1], I[2, 2]) and I[0, 0] < I[1, 1]  # the symmetry axis is x
    assert np.allclose(I - np.diag(np.diag(I)), 0, atol=1e-15)


def test_ball_joint():
    """A ``ball`` joint gives the spherical joint at ``body pose * joint pos`` with the armature on
    its three dofs (reference mjcf-graph.cpp:946-970); the dynamics match the same model built
    through the construction API."""
    m = buildModelFromMJCFXML("""<mujoco><worldbody>
      <body name="a" pos="0 0 1"><joint type="hinge" axis="0 1 0"/><inertial mass="1" diaginertia="0.1 0.2 0.3"/>
        <body name="b" pos="0.4 0 0"><joint type="ball" pos="0.1 0 0" armature="0.05"/>
          <inertial pos="0.2 0 0" mass="2" diaginertia="0.2 0.3 0.4"/></body></body></worldbody></mujoco>""")
    assert m.jtypes[1:] == [gm.JT_RY, gm.JT_SPH] and m.nq == 5 and m.nv == 4
    assert np.array_equal(m.armature, [0, 0.05, 0.05, 0.05])
    ref = gm.Model()
    j1 = ref.addJoint(0, gm.JointModelRY(), gm.SE3(np.eye(3), np.array([0.0, 0, 1])), "a")
    ref.appendBodyToJoint(j1, gm.Inertia(1.0, np.zeros(3), np.diag([0.1, 0.2, 0.3])), gm.SE3.Identity())
    j2 = ref.addJoint(j1, gm.JointModelSpherical(), gm.SE3(np.eye(3), np.array([0.5, 0, 0])), "b")
    ref.appendBodyToJoint(j2, gm.Inertia(2.0, np.array([0.1, 0, 0]), np.diag([0.2, 0.3, 0.4])), gm.SE3.Identity())
    ref.armature[1:] = 0.05
    q, v, a = sm.random_inputs(m, 8, 4)
    assert rel_err(OracleModel(m).rnea(q, v, a), OracleModel(ref).rnea(q, v, a)) < 1e-14


def _se3(R, t):
    T = np.eye(4)
    T[:3, :3], T[:3, 3] = R, t
    return T


def test_composite_joint():
    """A body with a hinge about y at (0, 0, 0.1), an unaligned slide at (0.05, 0, 0) and a hinge about
    x: the reference's composite joint (mjcf-graph.cpp:1002-1083) as a chain of three joints with
    massless links, the last named Composite_<first>; the body frame placed by the composite's
    product body pose * pos_0 * M_0(q_0) * (pos_0^-1 pos_1) * M_1(q_1) * (pos_1^-1 pos_2) * M_2(q_2),
    the body at pos_2^-1, each component's armature on its dof."""
    m = buildModelFromMJCFXML("""<mujoco><compiler angle="radian"/><worldbody>
      <body name="base" pos="0 0 1"><joint name="yaw" type="hinge" axis="0 0 1"/>
        <inertial mass="1" diaginertia="0.1 0.2 0.3"/>
        <body name="hip" pos="0.2 0 -0.1" axisangle="0 0 1 0.4">
          <joint name="hy" type="hinge" axis="0 1 0" pos="0 0 0.1" armature="0.02"/>
          <joint name="ext" type="slide" axis="1 1 0" pos="0.05 0 0"/>
          <joint name="hx" type="hinge" axis="1 0 0" armature="0.03"/>
          <inertial pos="0 0 -0.2" mass="2" diaginertia="0.02 0.03 0.04"/>
          <body name="foot" pos="0 0 -0.4"><joint name="ankle" type="hinge" axis="0 1 0"/>
            <inertial mass="0.5" diaginertia="0.01 0.01 0.01"/></body>
        </body></body></worldbody></mujoco>""")
    assert m.names == ["universe", "yaw", "hy", "ext", "Composite_hy", "ankle"]
    assert m.jtypes[1:] == [gm.JT_RZ, gm.JT_RY, gm.JT_PU, gm.JT_RX, gm.JT_RY]
    assert m.parents == [0, 0, 1, 2, 3, 4] and (m.nq, m.nv) == (5, 5)
    assert np.array_equal(m.armature, [0, 0.02, 0, 0.03, 0])
    q = np.random.default_rng(5).uniform(-1, 1, (6, 5))
    oMi, _, _ = OracleModel(m).forward_kinematics(q)
    a = np.array([1.0, 1.0, 0.0]) / np.sqrt(2.0)
    pos = [np.array([0, 0, 0.1]), np.array([0.05, 0, 0]), np.zeros(3)]
    for b in range(6):
        T = _se3(np.eye(3), [0, 0, 1]) @ _se3(_rot([0, 0, 1], q[b, 0]), np.zeros(3))
        T = T @ _se3(_rot([0, 0, 1], 0.4), [0.2, 0, -0.1]) @ _se3(np.eye(3), pos[0])
        T = T @ _se3(_rot([0, 1, 0], q[b, 1]), np.zeros(3)) @ _se3(np.eye(3), pos[1] - pos[0])
        T = T @ _se3(np.eye(3), a * q[b, 2]) @ _se3(np.eye(3), pos[2] - pos[1])
        T = T @ _se3(_rot([1, 0, 0], q[b, 3]), np.zeros(3))
        got = _se3(oMi[b, 4, :9].reshape(3, 3), oMi[b, 4, 9:])
        assert np.allclose(got, T, atol=1e-13)
        foot = T @ _se3(np.eye(3), -pos[2]) @ _se3(np.eye(3), [0, 0, -0.4]) @ _se3(_rot([0, 1, 0], q[b, 4]), np.zeros(3))
        assert np.allclose(_se3(oMi[b, 5, :9].reshape(3, 3), oMi[b, 5, 9:]), foot, atol=1e-13)
    # the body hangs from the last component: its centre of mass at pos_2^-1 * (0, 0, -0.2)
    assert np.allclose(m.tables()["inertia"][4, :4], [2.0, 0.0, 0.0, -0.2])
    assert m.tables()["inertia"][2:4, 0].sum() == 0.0  # massless links between the components
