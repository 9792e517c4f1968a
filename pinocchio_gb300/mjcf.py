"""MJCF -> Model: a subset of MuJoCo's XML format, following the reference's MJCF parser
(src/parsers/mjcf/mjcf-graph.cpp).

``buildModelFromMJCF(path)`` / ``buildModelFromMJCFXML(xml)`` walk ``<worldbody>`` depth first,
children in file order, as MjcfGraph::parseGraph / fillModel do:

* a ``<body>`` with one ``<joint>`` (or ``<freejoint/>``) becomes a joint of the model, placed at
  ``body pose * joint pos`` in the frame of its parent body (addSoloJoint, mjcf-graph.cpp:918-971);
  the body's inertia goes to that joint, expressed in the joint frame (``bodyInJoint = joint
  pos^-1``); ``hinge`` -> revolute, ``slide`` -> prismatic (aligned or unaligned by the axis, as the
  URDF loader maps axes), ``ball`` -> the spherical joint (mjcf-graph.cpp:946-951), ``free`` -> the
  free-flyer (root body only);
* a body without a joint is welded to its parent: its inertia is merged into the parent's joint
  (addFixedJointAndBody);
* body poses: ``pos`` with ``quat`` (w x y z), ``axisangle`` or ``euler`` (the compiler's
  ``eulerseq``, lowercase: rotating axes) in the compiler's ``angle`` unit, degrees by default
  (MjcfCompiler, mjcf-graph.cpp:102-116, 720-770);
* ``<inertial pos quat mass diaginertia|fullinertia>`` gives the body's inertia (the principal
  frame rotated by ``quat``); a joint's ``armature`` becomes the model's armature on each of its
  dofs (mjcf-graph.cpp:966-970).

Outside the subset (each raises ValueError, so that no model is silently different from the
reference's): ``<default>`` classes and ``class`` / ``childclass`` attributes, ``<include>``,
bodies with several joints (the reference's composite joints), free joints below
the root, ``xyaxes`` / ``zaxis`` orientations, uppercase (fixed-axis) Euler sequences, and bodies
whose inertia MuJoCo would infer from their ``<geom>`` elements (``inertiafromgeom``; a body with
geoms needs an ``<inertial>`` unless the compiler sets ``inertiafromgeom="false"``).
"""
from __future__ import annotations

import xml.etree.ElementTree as ET

import numpy as np

from .model import JT_FF, Inertia, JointModelFreeFlyer, JointModelSpherical, Model, SE3
from .urdf import _OneDof, _mul, _floats
from .model import JT_PX, JT_PY, JT_PZ, JT_RX, JT_RY, JT_RZ, JointModelPrismaticUnaligned, JointModelRevoluteUnaligned

_ALIGNED = {"hinge": (JT_RX, JT_RY, JT_RZ), "slide": (JT_PX, JT_PY, JT_PZ)}
_UNALIGNED = {"hinge": JointModelRevoluteUnaligned, "slide": JointModelPrismaticUnaligned}


def _quat_matrix(wxyz):
    w, x, y, z = np.asarray(wxyz, dtype=np.float64) / np.linalg.norm(wxyz)
    return np.array([
        [1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
        [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
        [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)],
    ])


def _axis_angle(axis, angle):
    a = np.asarray(axis, dtype=np.float64)
    a = a / np.linalg.norm(a)
    K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    return np.eye(3) + np.sin(angle) * K + (1 - np.cos(angle)) * (K @ K)


class _Compiler:
    """The <compiler> settings the subset uses (MjcfCompiler)."""

    def __init__(self, el):
        self.scale = np.pi / 180.0  # angle="degree" is MuJoCo's default
        self.seq = "xyz"
        self.inertia_from_geom = "auto"
        if el is None:
            return
        if el.get("angle", "degree") == "radian":
            self.scale = 1.0
        seq = el.get("eulerseq", "xyz")
        if len(seq) != 3 or any(c not in "xyz" for c in seq):
            raise ValueError(f"eulerseq {seq!r}: only rotating-axis (lowercase) sequences are supported")
        self.seq = seq
        self.inertia_from_geom = el.get("inertiafromgeom", "auto")

    def rotation(self, el):
        """The orientation of a body / inertial element (convertPosition, mjcf-graph.cpp:290-330)."""
        for bad in ("xyaxes", "zaxis"):
            if el.get(bad) is not None:
                raise ValueError(f"<{el.tag}> orientation by {bad!r} is not supported")
        if el.get("quat") is not None:
            return _quat_matrix(_floats(el.get("quat"), 4, None))
        if el.get("axisangle") is not None:
            aa = _floats(el.get("axisangle"), 4, None)
            return _axis_angle(aa[:3], aa[3] * self.scale)
        if el.get("euler") is not None:
            ang = _floats(el.get("euler"), 3, None) * self.scale
            R = np.eye(3)
            for c, t in zip(self.seq, ang):  # R = R_a0(t0) R_a1(t1) R_a2(t2): axes that rotate with the frame
                R = R @ _axis_angle(np.eye(3)["xyz".index(c)], t)
            return R
        return np.eye(3)

    def pose(self, el):
        return SE3(self.rotation(el), _floats(el.get("pos"), 3, [0, 0, 0]))


def _body_inertia(body, comp: _Compiler) -> Inertia:
    """The body's spatial inertia in the body frame."""
    inertial = body.find("inertial")
    if inertial is None:
        if body.find("geom") is not None and comp.inertia_from_geom != "false":
            raise ValueError(f"body {body.get('name')!r}: inertia from geoms is not supported; give an <inertial>")
        return Inertia.Zero()
    if comp.inertia_from_geom == "true":
        raise ValueError("inertiafromgeom='true' (inertias computed from geoms) is not supported")
    mass = float(inertial.get("mass", "0"))
    if inertial.get("fullinertia") is not None:
        xx, yy, zz, xy, xz, yz = _floats(inertial.get("fullinertia"), 6, None)
        I = np.array([[xx, xy, xz], [xy, yy, yz], [xz, yz, zz]])
    else:
        I = np.diag(_floats(inertial.get("diaginertia"), 3, [0, 0, 0]))
    P = comp.pose(inertial)
    return Inertia(mass, np.zeros(3), I).se3_action(P)


def _joint_model(j, comp: _Compiler):
    kind = j.get("type", "hinge")
    if kind == "ball":
        return JointModelSpherical()
    if kind not in _ALIGNED:
        raise ValueError(f"joint {j.get('name')!r}: type {kind!r} is not supported by the batched kernels")
    ax = _floats(j.get("axis"), 3, [0, 0, 1])
    n = float(np.linalg.norm(ax))
    if n == 0:
        raise ValueError(f"joint {j.get('name')!r}: zero axis")
    for k in range(3):
        e = np.zeros(3)
        e[k] = 1.0
        if np.linalg.norm(ax / n - e) <= 1e-12:
            return _OneDof(_ALIGNED[kind][k])
    return _UNALIGNED[kind](ax / n)


def buildModelFromMJCFXML(xml: str) -> Model:
    """Model of an MJCF document (reference pinocchio::mjcf::buildModelFromXML)."""
    root = ET.fromstring(xml)
    if root.tag != "mujoco":
        raise ValueError("not an MJCF document: the root element must be <mujoco>")
    for el in root.iter():
        if el.tag in ("default", "include", "frame"):
            raise ValueError(f"<{el.tag}> is not supported")
        if el.get("class") is not None or el.get("childclass") is not None:
            raise ValueError(f"<{el.tag}>: class / childclass attributes are not supported")
    comp = _Compiler(root.find("compiler"))
    world = root.find("worldbody")
    if world is None:
        raise ValueError("no <worldbody>")
    model = Model()
    model.name = root.get("model", "")

    def check_children(el):
        # bodies are read as direct <body> children only: a body nested in any other container
        # would be dropped, so such a container is an error (no model may silently differ)
        for child in el:
            if child.tag != "body" and child.find(".//body") is not None:
                raise ValueError(f"<{child.tag}> inside <{el.tag}> holds bodies: not supported")

    def visit(body, frame):
        """frame: (the joint that carries the parent body, the parent body's frame in that joint's frame)."""
        check_children(body)
        parent_joint, parent_in_joint = frame
        pose = _mul(parent_in_joint, comp.pose(body))
        joints = [("free", j) for j in body.findall("freejoint")] + [(j.get("type", "hinge"), j) for j in body.findall("joint")]
        if len(joints) > 1:
            raise ValueError(f"body {body.get('name')!r}: several joints (a composite joint) are not supported")
        Y = _body_inertia(body, comp)
        if not joints:  # welded to the parent body
            if parent_joint > 0 and (Y.mass > 0.0 or Y.inertia.any()):
                model.appendBodyToJoint(parent_joint, Y, pose)
            child_frame = (parent_joint, pose)
        else:
            kind, j = joints[0]
            name = j.get("name") or (body.get("name", "") + "_joint")
            jpos = SE3(np.eye(3), _floats(j.get("pos"), 3, [0, 0, 0]))
            if kind == "free":
                if parent_joint != 0 or j.get("pos") is not None:
                    raise ValueError(f"joint {name!r}: a free joint is supported on a root body only")
                jid = model.addJoint(0, JointModelFreeFlyer(), pose, name)
            else:
                jid = model.addJoint(parent_joint, _joint_model(j, comp), _mul(pose, jpos), name)
                arm = float(j.get("armature", "0"))
                if arm:
                    iv = model.idx_vs[jid]
                    model.armature[iv:iv + model.nvs[jid]] = arm
            body_in_joint = SE3(np.eye(3), -jpos.translation)
            if Y.mass > 0.0 or Y.inertia.any():
                model.appendBodyToJoint(jid, Y, body_in_joint)
            child_frame = (jid, body_in_joint)
        for child in body.findall("body"):
            visit(child, child_frame)

    check_children(world)
    for body in world.findall("body"):
        visit(body, (0, SE3.Identity()))
    if model.njoints > 1 and any(t == JT_FF for t in model.jtypes[2:]):
        raise ValueError("a free joint is supported on the first root body only")
    model.check_depth_first()
    return model


def buildModelFromMJCF(path: str) -> Model:
    """Model of an MJCF file (reference pinocchio::mjcf::buildModel(filename, model))."""
    with open(path) as f:
        return buildModelFromMJCFXML(f.read())
