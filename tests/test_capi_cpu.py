"""The C ABI library on a machine without a GPU: it loads, exports every symbol
of include/pinocchio_gb300.h, and rejects bad arguments with the reference's
error classes before touching the device."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from pinocchio_gb300 import _build, _capi
from pinocchio_gb300 import model as gm
from pinocchio_gb300 import sample_models as sm

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def L():
    _build.build()
    return _capi.lib()


def header_symbols():
    text = open(os.path.join(ROOT, "include", "pinocchio_gb300.h")).read()
    return re.findall(r"^(?:int|const char\*)\s+(gb_\w+)\s*\(", text, flags=re.M)


def test_header_lists_match_binding():
    assert tuple(header_symbols()) == _capi.EXPORTS


def test_library_exports_every_symbol(L):
    for name in header_symbols():
        assert hasattr(L, name), name


def test_invalid_arguments_are_rejected_on_the_host(L):
    assert L.gb_rnea(None, 0, 0, 1, None, None, None, None, None) == _capi.GB_ERR_INVALID_ARGUMENT
    assert b"model" in L.gb_last_error()
    out = C.c_void_p()
    assert L.gb_model_create(None, C.byref(out)) == _capi.GB_ERR_INVALID_ARGUMENT
    # the external-force entry points check their arguments the same way, and require fext
    assert L.gb_rnea_fext(None, 0, 0, 1, None, None, None, None, None, None) == _capi.GB_ERR_INVALID_ARGUMENT
    assert L.gb_aba_fext(None, 0, 0, 0, 1, None, None, None, None, None, None) == _capi.GB_ERR_INVALID_ARGUMENT
    assert L.gb_static_torque(None, 0, 0, 1, None, None, None, None) == _capi.GB_ERR_INVALID_ARGUMENT
    assert L.gb_rnea_derivatives_fext(None, 0, 0, 0, 1, *([None] * 9)) == _capi.GB_ERR_INVALID_ARGUMENT
    assert b"fext" in L.gb_last_error()
    assert L.gb_aba_derivatives_fext(None, 0, 0, 1, *([None] * 9)) == _capi.GB_ERR_INVALID_ARGUMENT
    assert b"fext" in L.gb_last_error()
    assert L.gb_forward_dynamics(None, 0, 0, 1, 2, *([None] * 5), 0.0, None, None, None) == _capi.GB_ERR_INVALID_ARGUMENT
    assert L.gb_impulse_dynamics(None, 0, 0, 1, 2, None, None, None, 0.0, 0.0, None, None, None) == \
        _capi.GB_ERR_INVALID_ARGUMENT
    assert L.gb_kkt_contact_inverse(None, 0, 0, 1, 2, None, None, 0.0, None, None) == _capi.GB_ERR_INVALID_ARGUMENT


def _create(L, model_tables):
    d, keep = _capi.make_desc(model_tables)
    out = C.c_void_p()
    return L.gb_model_create(C.byref(d), C.byref(out)), out


def test_tree_validation(L):
    # a free-flyer below another joint is outside the supported trees
    m = gm.Model()
    j = m.addJoint(0, gm.JointModelRX(), gm.SE3.Identity(), "a")
    m.addJoint(j, gm.JointModelFreeFlyer(), gm.SE3.Identity(), "b")
    rc, _ = _create(L, m.tables())
    assert rc == _capi.GB_ERR_UNSUPPORTED
    # joints that are not in depth-first order
    m = gm.Model()
    a = m.addJoint(0, gm.JointModelRX(), gm.SE3.Identity(), "a")
    m.addJoint(0, gm.JointModelRY(), gm.SE3.Identity(), "b")
    m.addJoint(a, gm.JointModelRZ(), gm.SE3.Identity(), "c")
    rc, _ = _create(L, m.tables())
    assert rc == _capi.GB_ERR_UNSUPPORTED
    assert b"depth-first" in L.gb_last_error()
    # an unknown joint type code
    t = sm.manipulator6r().tables()
    t["jtype"] = t["jtype"].copy()
    t["jtype"][3] = 18
    rc, _ = _create(L, t)
    assert rc == _capi.GB_ERR_UNSUPPORTED
    # armature of the wrong size
    t = sm.manipulator6r().tables()
    t["armature"] = np.zeros(3)
    rc, _ = _create(L, t)
    assert rc == _capi.GB_ERR_SIZE


def test_pool_checks_before_any_device_work(L):
    assert L.gb_rnea_in_parallel(1, None, 4, None, None, None, None) == _capi.GB_ERR_INVALID_ARGUMENT
