"""Rigid constraint models and proximal settings for ``constraintDynamics``.

The classes mirror the reference's constraint API (algorithm/contact-info.hpp:19-230,
algorithm/proximal.hpp:22-110, bindings/python/algorithm/contact-info.hpp):

* ``RigidConstraintModel(type, model, joint1_id, joint1_placement, joint2_id, joint2_placement,
  reference_frame)`` and its shorter forms ``(type, model, joint1_id, joint1_placement,
  reference_frame)`` and ``(type, model, joint1_id, reference_frame)``: a point (CONTACT_3D) or
  frame (CONTACT_6D) constraint between a frame of joint 1 and a frame of joint 2 (joint 0: the
  world), expressed in LOCAL or LOCAL_WORLD_ALIGNED axes, with a desired contact acceleration and
  Baumgarte gains ``corrector.Kp`` / ``corrector.Kd``;
* ``RigidConstraintData(cmodel)``: after a call, ``contact_force`` holds the constraint force of
  every configuration of the batch (B, 6), in the constraint's frame;
* ``ProximalSettings(accuracy, mu, max_iter)`` / ``(absolute_accuracy, relative_accuracy, mu,
  max_iter)``: after a call, ``iter`` and the residuals are the largest over the batch (the
  per-configuration values are in ``data.constraint_iterations`` / ``data.constraint_residuals``).

A model is flattened for the C ABI into 46 doubles (``desc()``): type, reference frame, joint1,
joint2, joint1_placement (R row-major, t), joint2_placement, the desired acceleration
[linear; angular], Kp, Kd (CONTACT_3D uses the first three entries of each).
"""
from __future__ import annotations

from enum import IntEnum

import numpy as np

from .model import SE3, Model


class ContactType(IntEnum):
    """contact-info.hpp:19-24"""

    CONTACT_3D = 0
    CONTACT_6D = 1


class ReferenceFrame(IntEnum):
    """multibody/fwd.hpp:46-56"""

    WORLD = 0
    LOCAL = 1
    LOCAL_WORLD_ALIGNED = 2


CONTACT_3D, CONTACT_6D = ContactType.CONTACT_3D, ContactType.CONTACT_6D
WORLD, LOCAL, LOCAL_WORLD_ALIGNED = ReferenceFrame.WORLD, ReferenceFrame.LOCAL, ReferenceFrame.LOCAL_WORLD_ALIGNED
DESC_SIZE = 46


class BaumgarteCorrectorParameters:
    """Kp, Kd of the constraint's Baumgarte correction (contact-info.hpp:29-90), one gain per row."""

    def __init__(self, size: int):
        self.Kp = np.zeros(size)
        self.Kd = np.zeros(size)


class RigidConstraintModel:
    def __init__(self, contact_type, model: Model, joint1_id: int, *args):
        self.type = ContactType(int(contact_type))
        placements, frame = [], ReferenceFrame.LOCAL
        ids = [int(joint1_id)]
        for a in args:
            if isinstance(a, SE3):
                placements.append(a)
            elif isinstance(a, ReferenceFrame):
                frame = a
            elif isinstance(a, (int, np.integer)):
                if len(ids) == 1 and len(placements) == 1:
                    ids.append(int(a))  # joint2_id after joint1_placement
                else:
                    frame = ReferenceFrame(int(a))
            else:
                raise TypeError(f"unexpected argument {a!r}")
        if len(ids) == 1 and len(placements) > 1:
            raise TypeError("a joint2_placement needs a joint2_id")
        self.joint1_id = ids[0]
        self.joint2_id = ids[1] if len(ids) > 1 else 0
        self.joint1_placement = placements[0] if placements else SE3.Identity()
        self.joint2_placement = placements[1] if len(placements) > 1 else SE3.Identity()
        self.reference_frame = frame
        if frame not in (ReferenceFrame.LOCAL, ReferenceFrame.LOCAL_WORLD_ALIGNED):
            raise ValueError("reference_frame should be LOCAL or LOCAL_WORLD_ALIGNED")
        for j in (self.joint1_id, self.joint2_id):
            if not 0 <= j < model.njoints:
                raise ValueError(f"joint index {j} out of range")
        self.name = ""
        self.desired_contact_acceleration = np.zeros(6)
        self.corrector = BaumgarteCorrectorParameters(self.size())

    def size(self) -> int:
        return 3 if self.type == ContactType.CONTACT_3D else 6

    def desc(self) -> np.ndarray:
        d = np.zeros(DESC_SIZE)
        d[0], d[1], d[2], d[3] = int(self.type), int(self.reference_frame), self.joint1_id, self.joint2_id
        for off, P in ((4, self.joint1_placement), (16, self.joint2_placement)):
            d[off : off + 9] = np.asarray(P.rotation).reshape(9)
            d[off + 9 : off + 12] = P.translation
        d[28:34] = np.asarray(self.desired_contact_acceleration, dtype=np.float64).reshape(6)
        n = self.size()
        d[34 : 34 + n] = np.asarray(self.corrector.Kp, dtype=np.float64).reshape(n)
        d[40 : 40 + n] = np.asarray(self.corrector.Kd, dtype=np.float64).reshape(n)
        return d


class RigidConstraintData:
    def __init__(self, cmodel: RigidConstraintModel):
        self.size = cmodel.size()
        self.contact_force = None


class ProximalSettings:
    def __init__(self, *args):
        if len(args) == 0:
            a, r, mu, it = 1e-12, 1e-12, 0.0, 1
        elif len(args) == 3:
            a, mu, it = args
            r = a
        elif len(args) == 4:
            a, r, mu, it = args
        else:
            raise TypeError("ProximalSettings(), (accuracy, mu, max_iter) or (absolute, relative, mu, max_iter)")
        if a < 0 or r < 0:
            raise ValueError("accuracy must be positive")
        if mu < 0:
            raise ValueError("mu must be positive")
        if int(it) < 1:
            raise ValueError("max_iter must be greater or equal to 1")
        self.absolute_accuracy, self.relative_accuracy, self.mu, self.max_iter = float(a), float(r), float(mu), int(it)
        self.absolute_residual = self.relative_residual = -1.0
        self.iter = 0


def stack_desc(contact_models) -> np.ndarray:
    """The (n, 46) flattened constraint models."""
    if not contact_models:
        return np.zeros((0, DESC_SIZE))
    return np.stack([c.desc() for c in contact_models])
