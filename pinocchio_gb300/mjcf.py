"""MJCF -> Model: a subset of MuJoCo's XML format, following the reference's MJCF parser
(src/parsers/mjcf/mjcf-graph.cpp, mjcf-graph-geom.cpp).

``buildModelFromMJCF(path)`` / ``buildModelFromMJCFXML(xml)`` walk ``<worldbody>`` depth first,
children in file order, as MjcfGraph::parseGraph / fillModel do:

* a ``<body>`` with one ``<joint>`` (or ``<freejoint/>``) becomes a joint of the model, placed at
  ``body pose * joint pos`` in the frame of its parent body (addSoloJoint, mjcf-graph.cpp:918-971);
  the body's inertia goes to that joint, expressed in the joint frame (``bodyInJoint = joint
  pos^-1``); ``hinge`` -> revolute, ``slide`` -> prismatic (aligned or unaligned by the axis, as the
  URDF loader maps axes), ``ball`` -> the spherical joint (mjcf-graph.cpp:946-951), ``free`` -> the
  free-flyer (root body only);
* a ``<body>`` with several joints (the reference's composite joint, mjcf-graph.cpp:1002-1083: its
  first component at ``body pose * pos_0``, component k at ``pos_{k-1}^-1 pos_k`` from the one
  before, the body at ``pos_last^-1``, the joint's transform the product of the components') becomes
  the same product as a chain of joints with massless links between them: the same q, v,
  kinematics and dynamics, with one joint per component (the last, which carries the body and the
  composite joint's frame, named ``Composite_<first joint's name>`` as the reference's composite
  joint; the others by their own names); each component's armature on its dofs;
* a body without a joint is welded to its parent: its inertia is merged into the parent's joint
  (addFixedJointAndBody);
* body poses: ``pos`` with ``quat`` (w x y z), ``axisangle`` or ``euler`` (the compiler's
  ``eulerseq``, lowercase: rotating axes) in the compiler's ``angle`` unit, degrees by default
  (MjcfCompiler, mjcf-graph.cpp:102-116, 720-770);
* ``<inertial pos quat mass diaginertia|fullinertia>`` gives the body's inertia (the principal
  frame rotated by ``quat``); a joint's ``armature`` becomes the model's armature on each of its
  dofs (mjcf-graph.cpp:966-970);
* ``<default>``: the top-level default and nested ``<default class="...">`` classes, each class
  inheriting the ``joint`` / ``geom`` attributes it does not set from its enclosing default
  (updateClassElement, mjcf-graph.cpp:35-52, parseDefault 657-690); an element's attributes are, in
  increasing precedence, the top-level default's, its body's ``childclass`` (inherited by nested
  bodies), its own ``class``, its own attributes (MjcfJoint::fill, mjcf-graph.cpp:239-285;
  MjcfGeom::fill, mjcf-graph-geom.cpp:428-461); a joint's ``pos`` and a geom's ``pos`` / orientation
  come from the element itself, as in the reference;
* inertia from geoms (the compiler's ``inertiafromgeom``: ``true``, or ``auto`` for a body without
  ``<inertial>``; parseJointAndBody, mjcf-graph.cpp:416-512): the sum over the body's non-visual
  geoms (not ``contype = conaffinity = 0``) of each geom's inertia placed at the geom's pose, the
  geom's mass from ``mass`` or its volume times ``density`` (default 1000); sphere, box, capsule,
  cylinder, ellipsoid sizes and ``fromto`` as in MjcfGeom::computeSize / computeVolume /
  computeInertia (mjcf-graph-geom.cpp:16-46, 318-410) with the reference's solid inertias
  (spatial/inertia.hpp: FromSphere, FromEllipsoid, FromCylinder, FromBox, FromCapsule); mesh, plane
  and hfield geoms keep the unit inertia the reference gives them.

Outside the subset (each raises ValueError, so that no model is silently different from the
reference's): ``<include>`` and ``<frame>``, a free joint among a body's several joints (the
reference refuses it too), free joints below the root, ``xyaxes`` / ``zaxis`` orientations, uppercase (fixed-axis)
Euler sequences, ``shellinertia`` geoms.
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


_DEFAULTED = ("joint", "geom", "site")  # the elements a <default> class sets (ELEMENTS, mjcf-graph.cpp:21)


class _Classes:
    """The <default> classes: class name -> {element tag: attributes}, each class merged with its
    enclosing defaults; "" is the top-level default."""

    def __init__(self, root):
        self.map = {}
        tops = root.findall("default")
        if len(tops) > 1:
            raise ValueError("several top-level <default> elements")
        if tops:
            self._parse(tops[0], {}, top=True)

    def _parse(self, el, parent, top=False):
        name = el.get("class")
        if name is None and not top:
            raise ValueError("Class does not have a name. Cannot parse model.")
        own = {c.tag: dict(c.attrib) for c in el if c.tag in _DEFAULTED}
        merged = {t: {**parent.get(t, {}), **own.get(t, {})} for t in set(parent) | set(own)}
        self.map["" if name is None else name] = merged
        if name is not None and top:
            self.map[""] = merged
        for child in el.findall("default"):
            self._parse(child, merged)

    def attributes(self, el, childclass):
        """The element's attributes: top-level default < body childclass < class < its own."""
        out = dict(self.map.get("", {}).get(el.tag, {}))
        for cls in (childclass, el.get("class")):
            if cls is None:
                continue
            if cls not in self.map:
                raise ValueError(f"unknown class {cls!r}")
            out.update(self.map[cls].get(el.tag, {}))
        out.update({k: v for k, v in el.attrib.items() if k != "class"})
        return out


def _geom_inertia(attrs, comp) -> tuple[Inertia, SE3] | None:
    """A geom's inertia about its center and its pose in the body (MjcfGeom::fill,
    mjcf-graph-geom.cpp:225-461); None for a visual geom."""
    if attrs.get("shellinertia") is not None:
        raise ValueError("Shell inertia computation is not supported yet.")
    if attrs.get("pos") is not None and attrs.get("fromto") is not None:
        raise ValueError("Both pos and fromto are defined in geom object")
    if int(attrs.get("contype", "1")) == 0 and int(attrs.get("conaffinity", "1")) == 0:
        return None  # visual only: not part of the inertia
    gtype = attrs.get("type", "sphere")
    el = ET.Element("geom", {k: v for k, v in attrs.items() if k in ("pos", "quat", "axisangle", "euler",
                                                                        "xyaxes", "zaxis")})
    pose = comp.pose(el)
    fromto = attrs.get("fromto")
    if fromto is not None:
        if gtype in ("plane", "hfield", "mesh", "sphere"):
            raise ValueError("fromto tag can only be used with capsules, boxes, cylinders and ellipsoids")
        ft = _floats(fromto, 6, None)
        z = ft[3:] - ft[:3]
        pose = SE3(_rotation_from_z(z), (ft[:3] + ft[3:]) / 2)
    if gtype in ("mesh", "plane", "hfield"):  # no volume: the reference keeps the unit inertia
        return Inertia(1.0, np.zeros(3), np.eye(3)), pose
    sz = [float(x) for x in attrs.get("size", "").split()]
    if not sz:
        raise ValueError(f"geom of type {gtype!r} without a size")
    zlen = float(np.linalg.norm(_floats(fromto, 6, None)[3:] - _floats(fromto, 6, None)[:3])) if fromto else None
    if gtype == "sphere":
        size = [sz[0]]
    elif gtype == "box":
        size = [2 * sz[0], 2 * sz[1], 2 * sz[2]] if fromto is None else [2 * sz[0], 2 * sz[0], zlen]
    elif gtype == "ellipsoid":
        size = sz[:3] if fromto is None else [sz[0], sz[0], zlen / 2]
    elif gtype in ("cylinder", "capsule"):
        size = sz[:2] if fromto is None else [sz[0], zlen / 2]
    else:
        raise ValueError(f"geomType {gtype!r} does not exist")
    if attrs.get("mass") is not None:
        mass = float(attrs["mass"])
    else:  # computeVolume (mjcf-graph-geom.cpp:19-46)
        r = size[0]
        vol = {"box": lambda: size[0] * size[1] * size[2],
               "cylinder": lambda: 2 * np.pi * r * r * size[1],
               "sphere": lambda: 4.0 / 3 * np.pi * r ** 3,
               "capsule": lambda: 4.0 / 3 * np.pi * r ** 3 + 2 * np.pi * r * r * size[1],
               "ellipsoid": lambda: 4.0 / 3 * np.pi * size[0] * size[1] * size[2]}[gtype]()
        mass = vol * float(attrs.get("density", "1000"))
    m = mass
    if gtype in ("sphere", "ellipsoid"):
        x, y, z = (size[0],) * 3 if gtype == "sphere" else size
        d = [m * (y * y + z * z) / 5, m * (x * x + z * z) / 5, m * (x * x + y * y) / 5]
    elif gtype == "box":
        x, y, z = size
        d = [m * (y * y + z * z) / 12, m * (x * x + z * z) / 12, m * (x * x + y * y) / 12]
    elif gtype == "cylinder":
        r, L = size[0], 2 * size[1]
        a = m * (r * r / 4 + L * L / 12)
        d = [a, a, m * r * r / 2]
    else:  # capsule: cylinder and two half spheres (spatial/inertia.hpp FromCapsule)
        r, h = size[0], 2 * size[1]
        v_cyl = np.pi * r * r * h
        v_hs = 2.0 / 3 * r ** 3 * np.pi
        tot = v_cyl + 2 * v_hs
        m_cyl, m_hs = m * v_cyl / tot, m * v_hs / tot
        dist = h / 2 + 0.375 * r
        ix = m_cyl * (h * h / 12 + r * r / 4) + 2 * (m_hs * r * r * 0.259375 + m_hs * dist * dist)
        iz = m_cyl * r * r / 2 + 2 * m_hs * r * r * 0.4
        d = [ix, ix, iz]
    return Inertia(mass, np.zeros(3), np.diag(d)), pose


def _rotation_from_z(zaxis):
    """The smallest rotation taking e_z onto zaxis (Eigen's Quaternion::FromTwoVectors); for zaxis
    opposite to e_z, the half turn about x."""
    z = np.asarray(zaxis, dtype=np.float64)
    z = z / np.linalg.norm(z)
    c = z[2]
    if c < -1 + 1e-12:
        return np.diag([1.0, -1.0, -1.0])
    ax = np.array([-z[1], z[0], 0.0])  # e_z x z
    K = np.array([[0, -ax[2], ax[1]], [ax[2], 0, -ax[0]], [-ax[1], ax[0], 0]])
    return np.eye(3) + K + K @ K / (1 + c)


def _body_inertia(body, comp: _Compiler, classes=None, childclass=None) -> Inertia:
    """The body's spatial inertia in the body frame."""
    inertial = body.find("inertial")
    from_geoms = comp.inertia_from_geom == "true" or (comp.inertia_from_geom == "auto" and inertial is None)
    if inertial is None and comp.inertia_from_geom == "false":
        if body.find("geom") is not None:
            raise ValueError("Cannot get inertia from geom and no inertia was found")
        return Inertia.Zero()
    if from_geoms:
        total = Inertia.Zero()
        for g in body.findall("geom"):
            attrs = classes.attributes(g, childclass) if classes is not None else dict(g.attrib)
            gi = _geom_inertia(attrs, comp)
            if gi is not None:
                total = total + gi[0].se3_action(gi[1])
        return total
    mass = float(inertial.get("mass", "0"))
    if inertial.get("fullinertia") is not None:
        xx, yy, zz, xy, xz, yz = _floats(inertial.get("fullinertia"), 6, None)
        I = np.array([[xx, xy, xz], [xy, yy, yz], [xz, yz, zz]])
    else:
        I = np.diag(_floats(inertial.get("diaginertia"), 3, [0, 0, 0]))
    P = comp.pose(inertial)
    return Inertia(mass, np.zeros(3), I).se3_action(P)


def _joint_model(j, comp: _Compiler, attrs=None):
    attrs = dict(j.attrib) if attrs is None else attrs
    kind = attrs.get("type", "hinge")
    if kind == "ball":
        return JointModelSpherical()
    if kind not in _ALIGNED:
        raise ValueError(f"joint {j.get('name')!r}: type {kind!r} is not supported by the batched kernels")
    ax = _floats(attrs.get("axis"), 3, [0, 0, 1])
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
        if el.tag in ("include", "frame"):
            raise ValueError(f"<{el.tag}> is not supported")
    classes = _Classes(root)
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

    def visit(body, frame, childclass):
        """frame: (the joint that carries the parent body, the parent body's frame in that joint's frame)."""
        check_children(body)
        childclass = body.get("childclass", childclass)
        parent_joint, parent_in_joint = frame
        pose = _mul(parent_in_joint, comp.pose(body))
        jattrs = {id(j): classes.attributes(j, childclass) for j in body.findall("joint")}
        joints = [("free", j) for j in body.findall("freejoint")] + [
            (jattrs[id(j)].get("type", "hinge"), j) for j in body.findall("joint")]
        if len(joints) > 1 and any(kind == "free" for kind, _ in joints):
            raise ValueError(f"body {body.get('name')!r}: a composite joint cannot hold a free joint")
        Y = _body_inertia(body, comp, classes, childclass)
        if not joints:  # welded to the parent body
            if parent_joint > 0 and (Y.mass > 0.0 or Y.inertia.any()):
                model.appendBodyToJoint(parent_joint, Y, pose)
            child_frame = (parent_joint, pose)
        else:
            jid, prev = parent_joint, None
            first = joints[0][1].get("name") or (body.get("name", "") + "_joint")
            for n, (kind, j) in enumerate(joints):
                name = j.get("name") or (body.get("name", "") + "_joint")
                if len(joints) > 1 and n == len(joints) - 1:
                    name = "Composite_" + first
                jpos = _floats(j.get("pos"), 3, [0, 0, 0])
                if kind == "free":
                    if parent_joint != 0 or j.get("pos") is not None:
                        raise ValueError(f"joint {name!r}: a free joint is supported on a root body only")
                    jid = model.addJoint(0, JointModelFreeFlyer(), pose, name)
                else:
                    # the first component at body pose * pos_0, the next ones at pos_{k-1}^-1 pos_k
                    place = _mul(pose, SE3(np.eye(3), jpos)) if prev is None else SE3(np.eye(3), jpos - prev)
                    jid = model.addJoint(jid, _joint_model(j, comp, jattrs[id(j)]), place, name)
                    arm = float(jattrs[id(j)].get("armature", "0"))
                    if arm:
                        iv = model.idx_vs[jid]
                        model.armature[iv:iv + model.nvs[jid]] = arm
                prev = jpos
            body_in_joint = SE3(np.eye(3), -prev)
            if Y.mass > 0.0 or Y.inertia.any():
                model.appendBodyToJoint(jid, Y, body_in_joint)
            child_frame = (jid, body_in_joint)
        for child in body.findall("body"):
            visit(child, child_frame, childclass)

    check_children(world)
    for body in world.findall("body"):
        visit(body, (0, SE3.Identity()), world.get("childclass"))
    if model.njoints > 1 and any(t == JT_FF for t in model.jtypes[2:]):
        raise ValueError("a free joint is supported on the first root body only")
    model.check_depth_first()
    return model


def buildModelFromMJCF(path: str) -> Model:
    """Model of an MJCF file (reference pinocchio::mjcf::buildModel(filename, model))."""
    with open(path) as f:
        return buildModelFromMJCFXML(f.read())
