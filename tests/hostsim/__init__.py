"""Test infrastructure: host build of the kernels' per-instance code (see hostsim.cpp)."""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from pinocchio_gb300._capi import ModelDesc, make_desc

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "libhostsim.so")
CSRC = os.path.join(os.path.dirname(os.path.dirname(HERE)), "pinocchio_gb300", "csrc")
_lib = None


def build(force=False):
    deps = [os.path.join(HERE, "hostsim.cpp")] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(map(os.path.getmtime, deps)):
        subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-fopenmp", "-shared", "-o", LIB, os.path.join(HERE, "hostsim.cpp")], check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        vp, l, i = C.c_void_p, C.c_long, C.c_int
        L.hs_last_error.restype = C.c_char_p
        L.hs_model_new.restype = vp
        L.hs_model_new.argtypes = [C.POINTER(ModelDesc)]
        L.hs_model_free.argtypes = [vp]
        L.hs_rnea.argtypes = [vp, i, l, vp, vp, vp, vp, vp]
        L.hs_aba.argtypes = [vp, i, l, vp, vp, vp, vp, vp]
        L.hs_crba.argtypes = [vp, i, i, l, vp, vp, vp, vp]
        L.hs_integrate.argtypes = [vp, l, vp, vp, vp]
        L.hs_rnea_derivs.argtypes = [vp, i, i, l, vp, vp, vp, vp, vp, vp, vp, vp]
        L.hs_aba_derivs.argtypes = [vp, i, l, vp, vp, vp, vp, vp, vp, vp, vp]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _c(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class HostSim:
    def __init__(self, model):
        self.desc, self._keep = make_desc(model.tables())
        h = lib().hs_model_new(C.byref(self.desc))
        if not h:
            raise ValueError(lib().hs_last_error().decode())
        self.h = C.c_void_p(h)
        self.nq, self.nv = model.nq, model.nv

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.hs_model_free(self.h)

    # fext: external forces (B, njoints, 6) in the joint frames, or None
    def rnea(self, q, v, a, mixed=False, fext=None):
        q, v, a = _c(q), _c(v), _c(a)
        tau = np.empty((q.shape[0], self.nv))
        f = None if fext is None else _c(fext)
        lib().hs_rnea(self.h, int(mixed), q.shape[0], _p(q), _p(v), _p(a), _p(tau), _p(f))
        return tau

    def aba(self, q, v, tau, mixed=False, fext=None):
        q, v, tau = _c(q), _c(v), _c(tau)
        ddq = np.empty((q.shape[0], self.nv))
        f = None if fext is None else _c(fext)
        lib().hs_aba(self.h, int(mixed), q.shape[0], _p(q), _p(v), _p(tau), _p(ddq), _p(f))
        return ddq

    def crba(self, q, mixed=False, symmetric=False, cholesky=False):
        q = _c(q)
        B, nv = q.shape[0], self.nv
        M = np.empty((B, nv, nv))
        U = np.empty((B, nv, nv)) if cholesky else None
        D = np.empty((B, nv)) if cholesky else None
        lib().hs_crba(self.h, int(mixed), int(symmetric), B, _p(q), _p(M), _p(U), _p(D))
        return (M, U, D) if cholesky else M

    def integrate(self, q, v):
        q, v = _c(q), _c(v)
        out = np.empty_like(q)
        lib().hs_integrate(self.h, q.shape[0], _p(q), _p(v), _p(out))
        return out

    def rnea_derivatives(self, q, v, a, mixed=False, symmetric=True, fext=None):
        q, v, a = _c(q), _c(v), _c(a)
        B, nv = q.shape[0], self.nv
        dq, dv, M = (np.empty((B, nv, nv)) for _ in range(3))
        tau = np.empty((B, nv))
        f = None if fext is None else _c(fext)
        lib().hs_rnea_derivs(self.h, int(mixed), int(symmetric), B, _p(q), _p(v), _p(a), _p(dq), _p(dv), _p(M), _p(tau), _p(f))
        return tau, dq, dv, M

    def aba_derivatives(self, q, v, tau, mixed=False, fext=None):
        q, v, tau = _c(q), _c(v), _c(tau)
        B, nv = q.shape[0], self.nv
        dq, dv, Minv = (np.empty((B, nv, nv)) for _ in range(3))
        ddq = np.empty((B, nv))
        f = None if fext is None else _c(fext)
        lib().hs_aba_derivs(self.h, int(mixed), B, _p(q), _p(v), _p(tau), _p(dq), _p(dv), _p(Minv), _p(ddq), _p(f))
        return ddq, dq, dv, Minv
