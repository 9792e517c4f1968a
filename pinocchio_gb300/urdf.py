"""URDF -> Model, and the Model's on-disk format.

``buildModelFromUrdf(path, root_joint=None)`` / ``buildModelFromXML(xml, root_joint=None)`` follow
the reference's URDF parser (src/parsers/urdf/model.cpp, src/parsers/urdf/model.hxx): the tree is
walked depth first from the root link, children in file order; every moving joint becomes a joint of
the model, placed relative to its parent joint by the chain of URDF origins (through any fixed
joints in between); every link becomes a body appended to the joint that moves it (its inertial
frame placed in that joint's frame); a fixed joint adds no degree of freedom and merges its child
link into the parent body (reference: fixed joints become frames, their bodies are appended to the
parent joint).  ``root_joint=JointModelFreeFlyer()`` puts a free-flyer between the universe and the
root link, as the reference's ``buildModel(filename, root_joint, model)`` does.

Joint axes map as in the reference (UrdfVisitor::addJoint and extractCartesianAxis,
include/pinocchio/parsers/urdf/model.hxx:438-576): an axis equal to the unit x, y or z axis (to a
relative 1e-12) gives JointModelRX/RY/RZ (``revolute``), JointModelRUBX/RUBY/RUBZ (``continuous``:
the unbounded revolute joint, nq = 2, q = (cos, sin)) or JointModelPX/PY/PZ (``prismatic``); any
other axis, negative ones included, gives JointModelRevoluteUnaligned /
JointModelRevoluteUnboundedUnaligned / JointModelPrismaticUnaligned with the normalised axis.
``planar`` gives
JointModelPlanar (motion in the joint frame's xy plane, the axis ignored, as the reference's
UrdfVisitor::addJointAndBody, model.hxx:285-290); ``floating`` gives the free-flyer on the root
link (the kernels run the free-flyer as the root joint only; a ``floating`` joint inside the tree
raises ValueError).

``save_model`` / ``load_model`` write and read the flattened tables (``Model.tables()`` plus the joint
names) as one ``.npz`` file: the on-disk format of a model (the reference serialises ModelTpl with
boost archives, serialization/model.hpp).
"""
from __future__ import annotations

import xml.etree.ElementTree as ET

import numpy as np

from .model import (
    JT_FF,
    JT_NONE,
    JT_PU,
    JT_PX,
    JT_PY,
    JT_PZ,
    JT_RU,
    JT_RX,
    JT_RY,
    JT_RZ,
    JT_RUBX,
    JT_RUBY,
    JT_RUBZ,
    JT_RUBU,
    Inertia,
    JointModel,
    JointModelFreeFlyer,
    JointModelMimic,
    JointModelPlanar,
    JointModelPrismaticUnaligned,
    JointModelRevoluteUnaligned,
    JointModelRevoluteUnboundedUnaligned,
    Model,
    SE3,
)


def _floats(text, n, default):
    if text is None:
        return np.array(default, dtype=np.float64)
    vals = [float(x) for x in text.split()]
    if len(vals) != n:
        raise ValueError(f"expected {n} numbers, got {text!r}")
    return np.array(vals)


def _rpy(rpy):
    """Rotation of URDF roll-pitch-yaw angles: Rz(yaw) Ry(pitch) Rx(roll)."""
    r, p, y = rpy
    cr, sr, cp, sp, cy, sy = np.cos(r), np.sin(r), np.cos(p), np.sin(p), np.cos(y), np.sin(y)
    Rx = np.array([[1, 0, 0], [0, cr, -sr], [0, sr, cr]])
    Ry = np.array([[cp, 0, sp], [0, 1, 0], [-sp, 0, cp]])
    Rz = np.array([[cy, -sy, 0], [sy, cy, 0], [0, 0, 1]])
    return Rz @ Ry @ Rx


def _origin(elem):
    o = None if elem is None else elem.find("origin")
    if o is None:
        return SE3.Identity()
    return SE3(_rpy(_floats(o.get("rpy"), 3, [0, 0, 0])), _floats(o.get("xyz"), 3, [0, 0, 0]))


def _mul(A: SE3, B: SE3) -> SE3:
    return SE3(A.rotation @ B.rotation, A.rotation @ B.translation + A.translation)


def _link_inertia(link) -> Inertia:
    """The link's inertia in the link frame (inertial origin applied)."""
    inertial = link.find("inertial")
    if inertial is None:
        return Inertia.Zero()
    mass_el = inertial.find("mass")
    mass = float(mass_el.get("value")) if mass_el is not None else 0.0
    it = inertial.find("inertia")
    I = np.zeros((3, 3))
    if it is not None:
        g = lambda k: float(it.get(k, "0"))  # noqa: E731
        I = np.array([[g("ixx"), g("ixy"), g("ixz")], [g("ixy"), g("iyy"), g("iyz")], [g("ixz"), g("iyz"), g("izz")]])
    return Inertia(mass, np.zeros(3), I).se3_action(_origin(inertial))


_AXIS_JT = {"revolute": (JT_RX, JT_RY, JT_RZ), "continuous": (JT_RUBX, JT_RUBY, JT_RUBZ),
            "prismatic": (JT_PX, JT_PY, JT_PZ)}
_UNALIGNED = {"revolute": JointModelRevoluteUnaligned, "continuous": JointModelRevoluteUnboundedUnaligned,
              "prismatic": JointModelPrismaticUnaligned}


class _OneDof(JointModel):
    def __init__(self, jtype):
        self.jtype = jtype


def _axis_joint(joint) -> JointModel:
    """The joint model of a one-dof URDF joint from its axis (reference extractCartesianAxis:
    Eigen isApprox against the unit axes, precision 1e-12)."""
    ax = _floats(None if joint.find("axis") is None else joint.find("axis").get("xyz"), 3, [1, 0, 0])
    n = float(np.linalg.norm(ax))
    if n == 0:
        raise ValueError(f"joint {joint.get('name')!r}: zero axis")
    kind = joint.get("type")
    for k in range(3):
        e = np.zeros(3)
        e[k] = 1.0
        if np.linalg.norm(ax - e) <= 1e-12 * min(n, 1.0):
            return _OneDof(_AXIS_JT[kind][k])
    return _UNALIGNED[kind](ax / n)


def buildModelFromXML(xml: str, root_joint: JointModel | None = None, mimic: bool = False) -> Model:
    """Model of a URDF document (reference pinocchio::urdf::buildModelFromXML).  With ``mimic``, a
    revolute or prismatic joint carrying ``<mimic joint=... multiplier=... offset=...>`` becomes a
    JointModelMimic of that joint (the reference's ``mimic`` argument, src/parsers/urdf/model.cpp:
    140-160, 213-230; off by default, when such joints are ordinary joints); the mimicked joint
    must come earlier in the depth-first walk."""
    robot = ET.fromstring(xml)
    if robot.tag != "robot":
        raise ValueError("not a URDF document: the root element must be <robot>")
    links = {l.get("name"): l for l in robot.findall("link")}
    joints = robot.findall("joint")
    children: dict[str, list] = {name: [] for name in links}
    is_child = set()
    for j in joints:
        parent, child = j.find("parent").get("link"), j.find("child").get("link")
        if parent not in links or child not in links:
            raise ValueError(f"joint {j.get('name')!r} refers to an unknown link")
        children[parent].append(j)
        is_child.add(child)
    roots = [name for name in links if name not in is_child]
    if len(roots) != 1:
        raise ValueError(f"a URDF tree has one root link, found {roots}")
    model = Model()
    model.name = robot.get("name", "")
    if root_joint is not None:
        if root_joint.jtype != JT_FF:
            raise ValueError("root_joint: only JointModelFreeFlyer is supported")
        frame = (model.addJoint(0, JointModelFreeFlyer(), SE3.Identity(), "root_joint"), SE3.Identity())
    else:
        frame = (0, SE3.Identity())

    def append(joint_id, link_name, placement):
        Y = _link_inertia(links[link_name])
        if joint_id > 0 and (Y.mass > 0.0 or Y.inertia.any()):
            model.appendBodyToJoint(joint_id, Y, placement)

    append(frame[0], roots[0], frame[1])

    def visit(link_name, frame):  # depth first, children in file order (the reference's recursion)
        joint_id, link_in_joint = frame
        for j in children[link_name]:
            child = j.find("child").get("link")
            Pj = _mul(link_in_joint, _origin(j))
            jt = j.get("type")
            if jt == "fixed":
                append(joint_id, child, Pj)
                visit(child, (joint_id, Pj))
            elif jt in _AXIS_JT or jt == "planar" or (jt == "floating" and joint_id == 0):
                jm = _axis_joint(j) if jt in _AXIS_JT else JointModelPlanar() if jt == "planar" else JointModelFreeFlyer()
                mi = j.find("mimic")
                if mimic and mi is not None and jt in ("revolute", "prismatic"):
                    target = mi.get("joint")
                    if target not in model.names:
                        raise ValueError(f"joint {j.get('name')!r} mimics {target!r}, which is not an earlier joint")
                    jm = JointModelMimic(jm, model.names.index(target), float(mi.get("multiplier", "1")),
                                         float(mi.get("offset", "0")))
                new_id = model.addJoint(joint_id, jm, Pj, j.get("name"))
                append(new_id, child, SE3.Identity())
                visit(child, (new_id, SE3.Identity()))
            else:
                raise ValueError(f"joint {j.get('name')!r}: type {jt!r} is not supported by the batched kernels")

    visit(roots[0], frame)
    model.check_depth_first()
    return model


def buildModelFromUrdf(path: str, root_joint: JointModel | None = None, mimic: bool = False) -> Model:
    """Model of a URDF file (reference pinocchio::urdf::buildModel(filename[, root_joint], model[,
    verbose, mimic]))."""
    with open(path, "r", encoding="utf-8") as f:
        return buildModelFromXML(f.read(), root_joint, mimic)


def save_model(model: Model, path: str) -> None:
    """Writes the model's tables and joint names to ``path`` (.npz)."""
    t = model.tables()
    np.savez(path, names=np.array(model.names), name=np.array(model.name), **t)


def load_model(path: str) -> Model:
    """Reads a model written by ``save_model``."""
    with np.load(path, allow_pickle=False) as z:
        parents, jtype = z["parents"], z["jtype"]
        placement, inertia = z["placement"], z["inertia"]
        axis = z["axis"] if "axis" in z.files else np.zeros((len(parents), 3))
        names = [str(n) for n in z["names"]]
        model = Model()
        model.name = str(z["name"])
        for i in range(1, len(parents)):
            jt = int(jtype[i])
            if jt == JT_FF:
                joint = JointModelFreeFlyer()
            elif jt == JT_RU:
                joint = JointModelRevoluteUnaligned(axis[i])
            elif jt == JT_PU:
                joint = JointModelPrismaticUnaligned(axis[i])
            elif jt == JT_RUBU:
                joint = JointModelRevoluteUnboundedUnaligned(axis[i])
            else:
                joint = _OneDof(jt)
            if jt == JT_NONE:
                raise ValueError("joint type 0 (universe) below the root")
            if "mimic" in z.files and int(z["mimic"][i]) > 0:
                joint = JointModelMimic(joint, int(z["mimic"][i]), float(z["mimic_scaling"][i]),
                                        float(z["mimic_offset"][i]))
            P = SE3(placement[i, :9].reshape(3, 3), placement[i, 9:])
            model.addJoint(int(parents[i]), joint, P, names[i])
            model.inertias[i] = Inertia(inertia[i, 0], inertia[i, 1:4], inertia[i, 4:])
        model.armature = np.array(z["armature"], dtype=np.float64)
        model.gravity = np.array(z["gravity"], dtype=np.float64)
    return model
