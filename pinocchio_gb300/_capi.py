"""ctypes binding of the C ABI (``include/pinocchio_gb300.h``) exported by ``libpinocchio_gb300.so``.

The library is built in-tree by ``pinocchio_gb300._build``; importing this
module never compiles anything.  ``lib()`` raises if the library is missing:
there is no CPU fallback behind the ABI.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _build

GB_OK = 0
GB_ERR_INVALID_ARGUMENT, GB_ERR_SIZE, GB_ERR_UNSUPPORTED, GB_ERR_GRAVITY, GB_ERR_POOL, GB_ERR_CUDA, GB_ERR_NUMERIC = range(1, 8)
GB_FP64, GB_MIXED = 0, 1
GB_LOCAL, GB_WORLD = 0, 1
GB_LAYOUT_INSTANCE, GB_LAYOUT_SOA = 0, 1
GB_MATRIX_UPPER, GB_MATRIX_SYMMETRIC = 0, 1
GB_FUNC_RNEA, GB_FUNC_ABA, GB_FUNC_CRBA, GB_FUNC_RNEA_DERIVATIVES, GB_FUNC_ABA_DERIVATIVES = range(5)
GB_INSTANCE_PER_THREAD, GB_INSTANCE_PER_WARP, GB_INSTANCE_PER_4_LANES, GB_INSTANCE_PER_8_LANES = 0, 1, 2, 3
GB_INSTANCE_PER_BRANCH = 4
GB_NUMERIC_PIVOT, GB_NUMERIC_NONFINITE = 1, 2
GB_CONTACT_3D, GB_CONTACT_6D = 0, 1
GB_FRAME_WORLD, GB_FRAME_LOCAL, GB_FRAME_LOCAL_WORLD_ALIGNED = 0, 1, 2

# every symbol declared in include/pinocchio_gb300.h, in declaration order
EXPORTS = (
    "gb_model_create",
    "gb_model_destroy",
    "gb_model_dims",
    "gb_model_nv_extended",
    "gb_last_error",
    "gb_numeric_status",
    "gb_pipeline_timeouts",
    "gb_pipeline_wait_selftest",
    "gb_memcpy_async",
    "gb_rnea",
    "gb_nonlinear_effects",
    "gb_generalized_gravity",
    "gb_rnea_fext",
    "gb_static_torque",
    "gb_aba",
    "gb_aba_fext",
    "gb_crba",
    "gb_rnea_derivatives",
    "gb_rnea_derivatives_fext",
    "gb_aba_derivatives",
    "gb_aba_derivatives_fext",
    "gb_compute_minverse",
    "gb_aba_derivatives_vjp",
    "gb_aba_derivatives_noalloc",
    "gb_forward_dynamics",
    "gb_impulse_dynamics",
    "gb_kkt_contact_inverse",
    "gb_constraint_set_create",
    "gb_constraint_set_destroy",
    "gb_constraint_set_dims",
    "gb_constraint_dynamics",
    "gb_constraint_dynamics_derivatives",
    "gb_contact_cholesky",
    "gb_forward_kinematics",
    "gb_compute_joint_jacobians",
    "gb_integrate",
    "gb_batch_multi",
    "gb_model_set_launch",
    "gb_model_set_layout",
    "gb_pool_create",
    "gb_pool_destroy",
    "gb_pool_size",
    "gb_pool_set_precision",
    "gb_rnea_in_parallel",
    "gb_aba_in_parallel",
)


class GBError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


class Task(C.Structure):
    _fields_ = [
        ("model", C.c_void_p),
        ("function", C.c_int),
        ("batch", C.c_long),
        ("q", C.c_void_p),
        ("v", C.c_void_p),
        ("x", C.c_void_p),
        ("out", C.c_void_p),
    ]


class ModelDesc(C.Structure):
    _fields_ = [
        ("njoints", C.c_int),
        ("parents", C.c_void_p),
        ("jtype", C.c_void_p),
        ("placement", C.c_void_p),
        ("inertia", C.c_void_p),
        ("armature", C.c_void_p),
        ("nv_armature", C.c_int),
        ("gravity", C.c_void_p),
        ("axis", C.c_void_p),
        ("mimic", C.c_void_p),
        ("mimic_scaling", C.c_void_p),
        ("mimic_offset", C.c_void_p),
    ]


class ConstraintDesc(C.Structure):
    """gb_constraint_desc"""

    _fields_ = [
        ("type", C.c_int),
        ("reference_frame", C.c_int),
        ("joint1_id", C.c_int),
        ("joint2_id", C.c_int),
        ("joint1_placement", C.c_double * 12),
        ("joint2_placement", C.c_double * 12),
        ("desired_acceleration", C.c_double * 6),
        ("Kp", C.c_double * 6),
        ("Kd", C.c_double * 6),
    ]


class ProximalSettingsC(C.Structure):
    """gb_proximal_settings"""

    _fields_ = [
        ("absolute_accuracy", C.c_double),
        ("relative_accuracy", C.c_double),
        ("mu", C.c_double),
        ("max_iter", C.c_int),
    ]


def make_desc(tables: dict) -> tuple[ModelDesc, dict]:
    """A gb_model_desc over the arrays of ``Model.tables()`` (kept alive by the returned dict)."""
    keep = {k: np.ascontiguousarray(v) for k, v in tables.items()}
    d = ModelDesc()
    d.njoints = len(keep["parents"])
    d.parents = keep["parents"].ctypes.data
    d.jtype = keep["jtype"].ctypes.data
    d.placement = keep["placement"].ctypes.data
    d.inertia = keep["inertia"].ctypes.data
    d.armature = keep["armature"].ctypes.data if len(keep["armature"]) else None
    d.nv_armature = len(keep["armature"])
    d.gravity = keep["gravity"].ctypes.data
    d.axis = keep["axis"].ctypes.data if "axis" in keep else None
    if "mimic" in keep and keep["mimic"].any():
        d.mimic = keep["mimic"].ctypes.data
        d.mimic_scaling = keep["mimic_scaling"].ctypes.data
        d.mimic_offset = keep["mimic_offset"].ctypes.data
    return d, keep


_lib = None


def lib_path() -> str:
    return _build.LIB


def lib():
    """The loaded library; raises when it has not been built."""
    global _lib
    if _lib is None:
        path = lib_path()
        if not os.path.exists(path):
            raise RuntimeError(
                f"{path} is missing: build the CUDA library first (python -c 'import __graft_entry__ as g; g.build()')"
            )
        L = C.CDLL(path)
        vp, i, l = C.c_void_p, C.c_int, C.c_long
        L.gb_last_error.restype = C.c_char_p
        L.gb_model_create.argtypes = [C.POINTER(ModelDesc), C.POINTER(vp)]
        L.gb_model_destroy.argtypes = [vp]
        L.gb_model_dims.argtypes = [vp, C.POINTER(i), C.POINTER(i), C.POINTER(i)]
        L.gb_model_nv_extended.argtypes = [vp, C.POINTER(i)]
        L.gb_contact_cholesky.argtypes = [vp, i, vp, C.c_double, i, C.c_long] + [vp] * 8
        L.gb_pipeline_timeouts.argtypes = [C.POINTER(C.c_uint), i]
        L.gb_numeric_status.argtypes = [vp, C.POINTER(C.c_uint), i]
        L.gb_pipeline_wait_selftest.argtypes = [C.c_uint, vp]
        L.gb_memcpy_async.argtypes = [vp, vp, C.c_size_t, vp]
        L.gb_rnea.argtypes = [vp, i, i, l, vp, vp, vp, vp, vp]
        L.gb_nonlinear_effects.argtypes = [vp, i, i, l, vp, vp, vp, vp]
        L.gb_generalized_gravity.argtypes = [vp, i, i, l, vp, vp, vp]
        L.gb_aba.argtypes = [vp, i, i, i, l, vp, vp, vp, vp, vp]
        L.gb_rnea_fext.argtypes = [vp, i, i, l, vp, vp, vp, vp, vp, vp]
        L.gb_static_torque.argtypes = [vp, i, i, l, vp, vp, vp, vp]
        L.gb_aba_fext.argtypes = [vp, i, i, i, l, vp, vp, vp, vp, vp, vp]
        L.gb_rnea_derivatives_fext.argtypes = [vp, i, i, i, l, vp, vp, vp, vp, vp, vp, vp, vp, vp]
        L.gb_aba_derivatives_fext.argtypes = [vp, i, i, l, vp, vp, vp, vp, vp, vp, vp, vp, vp]
        L.gb_crba.argtypes = [vp, i, i, i, i, l, vp, vp, vp, vp, vp]
        L.gb_rnea_derivatives.argtypes = [vp, i, i, i, l, vp, vp, vp, vp, vp, vp, vp, vp]
        L.gb_aba_derivatives.argtypes = [vp, i, i, l, vp, vp, vp, vp, vp, vp, vp, vp]
        L.gb_compute_minverse.argtypes = [vp, i, i, i, l, vp, vp, vp]
        L.gb_aba_derivatives_vjp.argtypes = [vp, i, i, l, vp, vp, vp, vp, vp, vp, vp, vp, vp]
        L.gb_aba_derivatives_noalloc.argtypes = [vp, i, i, l, vp, vp, vp, vp, vp, vp, vp, vp]
        L.gb_integrate.argtypes = [vp, i, l, vp, vp, vp, vp]
        L.gb_forward_dynamics.argtypes = [vp, i, i, l, i, vp, vp, vp, vp, vp, C.c_double, vp, vp, vp]
        L.gb_impulse_dynamics.argtypes = [vp, i, i, l, i, vp, vp, vp, C.c_double, C.c_double, vp, vp, vp]
        L.gb_kkt_contact_inverse.argtypes = [vp, i, i, l, i, vp, vp, C.c_double, vp, vp]
        L.gb_constraint_set_create.argtypes = [vp, i, C.POINTER(ConstraintDesc), C.POINTER(vp)]
        L.gb_constraint_set_destroy.argtypes = [vp]
        L.gb_constraint_set_dims.argtypes = [vp, C.POINTER(i), C.POINTER(i)]
        L.gb_constraint_dynamics.argtypes = [vp, i, vp, C.POINTER(ProximalSettingsC), i, l, vp, vp, vp, vp, vp, vp, vp,
                                             vp]
        L.gb_constraint_dynamics_derivatives.argtypes = [vp, i, vp, C.POINTER(ProximalSettingsC), i, l] + [vp] * 13
        L.gb_forward_kinematics.argtypes = [vp, i, i, l, vp, vp, vp, vp, vp, vp, vp]
        L.gb_compute_joint_jacobians.argtypes = [vp, i, i, l, vp, vp, vp]
        L.gb_batch_multi.argtypes = [C.POINTER(Task), i, i, i, vp]
        L.gb_model_set_launch.argtypes = [vp, i, i]
        L.gb_model_set_layout.argtypes = [vp, i, i]
        L.gb_pool_create.argtypes = [vp, l, C.POINTER(vp)]
        L.gb_pool_destroy.argtypes = [vp]
        L.gb_pool_size.argtypes = [vp, C.POINTER(l)]
        L.gb_pool_set_precision.argtypes = [vp, i]
        L.gb_rnea_in_parallel.argtypes = [l, vp, l, vp, vp, vp, vp]
        L.gb_aba_in_parallel.argtypes = [l, vp, l, vp, vp, vp, vp]
        for name in EXPORTS:
            if name != "gb_last_error":
                getattr(L, name).restype = i
        _lib = L
    return _lib


def check(rc: int) -> None:
    if rc != GB_OK:
        raise GBError(rc, lib().gb_last_error().decode())
