"""Test infrastructure: ctypes front-end of the CPU oracle (liboracle.so).

Only the tests, the smoke check and the CPU-baseline leg of the benchmark use
this module; the product path never imports it.  ``build()`` compiles the
library from ``oracle_capi.cpp`` with the Makefile beside this file.

All batch arrays are numpy float64 of shape (batch, n) -- one instance per
row, i.e. the reference's column-major ``n x batch`` matrices.  Matrix outputs
have shape (batch, nv, nv) (row-major per instance).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

LOCAL, WORLD = 0, 1
F_RNEA, F_ABA_LOCAL, F_ABA_WORLD, F_CRBA_LOCAL, F_CRBA_WORLD, F_CHOL, F_RNEA_D, F_ABA_D, F_INTEGRATE = range(9)

_lib = None
_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")


def build(force: bool = False) -> str:
    srcs = [os.path.join(HERE, f) for f in ("oracle_capi.cpp", "oracle.hpp", "flop_scalar.hpp")]
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < max(map(os.path.getmtime, srcs)):
        subprocess.run(["make", "-s", "-C", HERE, "-B" if force else "all"], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        L.orc_last_error.restype = C.c_char_p
        L.orc_model_new.restype = C.c_void_p
        L.orc_model_new.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                    C.c_void_p, C.c_void_p]
        L.orc_model_free.argtypes = [C.c_void_p]
        L.orc_model_dims.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.orc_model_tables.argtypes = [C.c_void_p] + [C.c_void_p] * 5
        vp = C.c_void_p
        L.orc_rnea.argtypes = [vp, C.c_int, C.c_long, vp, vp, vp, vp, C.c_int]
        L.orc_aba.argtypes = [vp, C.c_int, C.c_int, C.c_long, vp, vp, vp, vp, C.c_int]
        L.orc_crba.argtypes = [vp, C.c_int, C.c_int, C.c_long, vp, vp, C.c_int]
        L.orc_cholesky.argtypes = [vp, C.c_int, C.c_long, vp, vp, vp, C.c_int]
        L.orc_rnea_derivatives.argtypes = [vp, C.c_int, C.c_long, vp, vp, vp, vp, vp, vp, vp, C.c_int]
        L.orc_aba_derivatives.argtypes = [vp, C.c_int, C.c_long, vp, vp, vp, vp, vp, vp, vp, C.c_int]
        L.orc_rnea_fext.argtypes = [vp, C.c_int, C.c_long, vp, vp, vp, vp, vp, C.c_int]
        L.orc_aba_fext.argtypes = [vp, C.c_int, C.c_int, C.c_long, vp, vp, vp, vp, vp, C.c_int]
        L.orc_rnea_derivatives_fext.argtypes = [vp, C.c_int, C.c_long, vp, vp, vp, vp, vp, vp, vp, vp, C.c_int]
        L.orc_aba_derivatives_fext.argtypes = [vp, C.c_int, C.c_long, vp, vp, vp, vp, vp, vp, vp, vp, C.c_int]
        L.orc_forward_dynamics.argtypes = [vp, C.c_int, C.c_long, C.c_int, vp, vp, vp, vp, vp, C.c_double, vp, vp, C.c_int]
        L.orc_kkt_inverse.argtypes = [vp, C.c_long, C.c_int, vp, vp, C.c_double, vp]
        L.orc_constraint_dynamics.argtypes = [vp, C.c_int, C.c_long, C.c_int, vp, vp, vp, vp, C.c_double, C.c_int,
                                              C.c_double, C.c_double, vp, vp, vp, vp, C.c_int]
        L.orc_constraint_dynamics_derivatives.argtypes = [vp, C.c_int, C.c_long, C.c_int, vp, vp, vp, vp, C.c_double,
                                                          C.c_int, C.c_double, C.c_double] + [vp] * 9 + [C.c_int]
        L.orc_log6.argtypes = [vp, vp, vp]
        L.orc_contact_cholesky.argtypes = [vp, C.c_long, C.c_int, vp, vp, C.c_double, vp, vp, vp, vp, vp, vp, C.c_int]
        L.orc_impulse_dynamics.argtypes = [vp, C.c_int, C.c_long, C.c_int, vp, vp, vp, C.c_double, C.c_double, vp, vp, C.c_int]
        L.orc_integrate.argtypes = [vp, C.c_int, C.c_long, vp, vp, vp, C.c_int]
        L.orc_forward_kinematics.argtypes = [vp, C.c_int, C.c_long, vp, vp, vp, vp, vp, vp, C.c_int]
        L.orc_joint_jacobians.argtypes = [vp, C.c_int, C.c_long, vp, vp, C.c_int]
        L.orc_count_flops.argtypes = [vp, C.c_int, vp, vp, vp, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _c(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _out(o, shape):
    """A caller-provided output array (C-contiguous float64 of ``shape``) or a new one."""
    if o is None:
        return np.empty(shape)
    if o.shape != tuple(shape) or o.dtype != np.float64 or not o.flags.c_contiguous:
        raise ValueError(f"output must be a C-contiguous float64 array of shape {tuple(shape)}")
    return o


JT_RX, JT_RY, JT_RZ, JT_ZYX = 1, 2, 3, 17


def expand_spherical_zyx(t):
    """Tables with every spherical ZYX joint (reference JointModelSphericalZYX,
    multibody/joint/joint-spherical-ZYX.hpp:404-470: M = (Rz(q0) Ry(q1) Rx(q2), 0), S(q) the
    angular velocity of the Euler rates in the child frame, c = dS/dt v) replaced by revolute
    joints about z, y and x, the first at the joint's placement, the other two at the identity, the
    body on the last: the same transform, velocity, acceleration and coordinates, a vector space
    like the joint.  Returns (tables, rows): rows[j] the joint carrying the caller's joint j (None
    when the model has no such joint).  The tests pin this against the reference's own known
    answers for the joint (unittest/joint-spherical.cpp:215-300) and against the joint's closed-form
    S(q) and c."""
    jt = [int(j) for j in t["jtype"]]
    if JT_ZYX not in jt:
        return t, None
    nj = len(jt)
    keys = [k for k, v in t.items() if k not in ("armature", "gravity") and len(v) == nj]
    new = {k: [] for k in keys}
    ident = np.array([1.0, 0, 0, 0, 1.0, 0, 0, 0, 1.0, 0, 0, 0])
    rows = []

    def push(row):
        for k in keys:
            new[k].append(row[k])
        return len(new["parents"]) - 1

    for j in range(nj):
        row = {k: np.array(t[k][j], copy=True) for k in keys}
        if j > 0:
            row["parents"] = np.int32(rows[int(t["parents"][j])])
        if jt[j] == JT_ZYX:
            for code in (JT_RZ, JT_RY):
                mid = {k: np.zeros_like(v) for k, v in row.items()}
                mid["parents"], mid["jtype"] = row["parents"], np.int32(code)
                mid["placement"] = row["placement"] if code == JT_RZ else ident
                row["parents"] = np.int32(push(mid))
            row["jtype"], row["placement"] = np.int32(JT_RX), ident
        rows.append(push(row))
    out = dict(t)
    for k in keys:
        out[k] = np.ascontiguousarray(np.stack(new[k]).astype(t[k].dtype))
    return out, np.asarray(rows)


class OracleModel:
    """The oracle's copy of a flattened model (from ``Model.tables()``); spherical ZYX joints run as
    the revolute chain of ``expand_spherical_zyx`` with the caller's joint indices mapped."""

    def __init__(self, model):
        L = lib()
        t = model.tables()
        if "mimic" in t and t["mimic"].any():
            raise ValueError("a model with mimic joints: use MimicOracleModel")
        nj_user = int(len(t["parents"]))
        t, self._rows = expand_spherical_zyx(t)
        self._keep = t
        h = L.orc_model_new(
            int(len(t["parents"])), _ptr(t["parents"]), _ptr(t["jtype"]), _ptr(t["placement"]), _ptr(t["inertia"]),
            _ptr(t["armature"]), int(len(t["armature"])), _ptr(t["gravity"]), _ptr(t.get("axis")),
        )
        if not h:
            raise ValueError(L.orc_last_error().decode())
        self.h = C.c_void_p(h)
        nq, nv = C.c_int(), C.c_int()
        L.orc_model_dims(self.h, C.byref(nq), C.byref(nv))
        self.nq, self.nv = nq.value, nv.value
        self.njoints = nj_user
        self._nj_internal = int(len(t["parents"]))
        self.model = model

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_model_free(self.h)
            self.h = None

    def _check(self, rc):
        if rc != 0:
            raise ValueError(lib().orc_last_error().decode())

    # all methods: prec 0 = double, 1 = long double; nthreads 0 = all cores.
    # fext (rnea, aba and the derivatives): external forces, (B, njoints, 6) [linear;
    # angular] in the joint frames, or None.
    def _fext(self, fext, B):
        f = _c(fext).reshape(B, -1)
        if f.shape[1] != 6 * self.njoints:
            raise ValueError("fext must hold njoints x 6 values per instance")
        if self._rows is not None:
            full = np.zeros((B, self._nj_internal, 6))
            full[:, self._rows] = f.reshape(B, self.njoints, 6)
            return full.reshape(B, -1)
        return f

    def _desc(self, desc):
        d = _c(np.asarray(desc).reshape(-1, 46))
        if self._rows is not None:
            d = d.copy()
            for c in (2, 3):
                d[:, c] = self._rows[d[:, c].astype(np.int64)]
        return d

    def rnea(self, q, v, a, prec=0, nthreads=0, fext=None, out=None):
        q, v, a = _c(q), _c(v), _c(a)
        tau = _out(out, (q.shape[0], self.nv))
        if fext is None:
            self._check(lib().orc_rnea(self.h, prec, q.shape[0], _ptr(q), _ptr(v), _ptr(a), _ptr(tau), nthreads))
        else:
            f = self._fext(fext, q.shape[0])
            self._check(lib().orc_rnea_fext(self.h, prec, q.shape[0], _ptr(q), _ptr(v), _ptr(a), _ptr(f), _ptr(tau), nthreads))
        return tau

    def aba(self, q, v, tau, convention=LOCAL, prec=0, nthreads=0, fext=None, out=None):
        q, v, tau = _c(q), _c(v), _c(tau)
        ddq = _out(out, (q.shape[0], self.nv))
        if fext is None:
            self._check(lib().orc_aba(self.h, prec, convention, q.shape[0], _ptr(q), _ptr(v), _ptr(tau), _ptr(ddq), nthreads))
        else:
            f = self._fext(fext, q.shape[0])
            self._check(lib().orc_aba_fext(self.h, prec, convention, q.shape[0], _ptr(q), _ptr(v), _ptr(tau), _ptr(f), _ptr(ddq), nthreads))
        return ddq

    def crba(self, q, convention=LOCAL, prec=0, nthreads=0):
        """Upper triangle of M (lower part zero), as the reference's crba leaves it."""
        q = _c(q)
        M = np.empty((q.shape[0], self.nv, self.nv))
        self._check(lib().orc_crba(self.h, prec, convention, q.shape[0], _ptr(q), _ptr(M), nthreads))
        return M

    def cholesky(self, M, prec=0, nthreads=0):
        M = _c(M)
        U = np.empty_like(M)
        D = np.empty((M.shape[0], self.nv))
        self._check(lib().orc_cholesky(self.h, prec, M.shape[0], _ptr(M), _ptr(U), _ptr(D), nthreads))
        return U, D

    def rnea_derivatives(self, q, v, a, prec=0, nthreads=0, fext=None):
        """(tau, dtau_dq, dtau_dv, M upper)."""
        q, v, a = _c(q), _c(v), _c(a)
        B, nv = q.shape[0], self.nv
        tau = np.empty((B, nv))
        dq, dv, M = (np.empty((B, nv, nv)) for _ in range(3))
        if fext is None:
            self._check(lib().orc_rnea_derivatives(self.h, prec, B, _ptr(q), _ptr(v), _ptr(a), _ptr(tau), _ptr(dq), _ptr(dv), _ptr(M), nthreads))
        else:
            f = self._fext(fext, B)
            self._check(lib().orc_rnea_derivatives_fext(self.h, prec, B, _ptr(q), _ptr(v), _ptr(a), _ptr(f), _ptr(tau), _ptr(dq), _ptr(dv), _ptr(M), nthreads))
        return tau, dq, dv, M

    def aba_derivatives(self, q, v, tau, prec=0, nthreads=0, fext=None, out=None):
        """(ddq, ddq_dq, ddq_dv, Minv); ``out``: the four arrays to write (reused across calls)."""
        q, v, tau = _c(q), _c(v), _c(tau)
        B, nv = q.shape[0], self.nv
        if out is None:
            ddq = np.empty((B, nv))
            dq, dv, Minv = (np.empty((B, nv, nv)) for _ in range(3))
        else:
            ddq, dq, dv, Minv = (_out(o, shp) for o, shp in zip(out, ((B, nv),) + ((B, nv, nv),) * 3))
        if fext is None:
            self._check(lib().orc_aba_derivatives(self.h, prec, B, _ptr(q), _ptr(v), _ptr(tau), _ptr(ddq), _ptr(dq), _ptr(dv), _ptr(Minv), nthreads))
        else:
            f = self._fext(fext, B)
            self._check(lib().orc_aba_derivatives_fext(self.h, prec, B, _ptr(q), _ptr(v), _ptr(tau), _ptr(f), _ptr(ddq), _ptr(dq), _ptr(dv), _ptr(Minv), nthreads))
        return ddq, dq, dv, Minv

    def forward_dynamics(self, q, v, tau, J, gamma, inv_damping=0.0, prec=0, nthreads=0):
        """(ddq, lambda_c) of forwardDynamics with the constraint Jacobian J (B, nc, nv) and drift gamma (B, nc)."""
        q, v, tau, J, gamma = _c(q), _c(v), _c(tau), _c(J), _c(gamma)
        B, nc = q.shape[0], J.shape[1]
        ddq, lam = np.empty((B, self.nv)), np.empty((B, nc))
        self._check(lib().orc_forward_dynamics(self.h, prec, B, nc, _ptr(q), _ptr(v), _ptr(tau), _ptr(J), _ptr(gamma),
                                               float(inv_damping), _ptr(ddq), _ptr(lam), nthreads))
        return ddq, lam

    def kkt_inverse(self, q, J, inv_damping=0.0):
        """computeKKTContactDynamicMatrixInverse: (B, nv + nc, nv + nc), FP64."""
        q, J = _c(q), _c(J)
        B, nc = q.shape[0], J.shape[1]
        K = np.empty((B, self.nv + nc, self.nv + nc))
        self._check(lib().orc_kkt_inverse(self.h, B, nc, _ptr(q), _ptr(J), float(inv_damping), _ptr(K)))
        return K

    def constraint_dynamics(self, q, v, tau, desc, mu=0.0, max_iter=1, absolute_accuracy=1e-12,
                            relative_accuracy=1e-12, prec=0, nthreads=0):
        """constraintDynamics (reference algorithm/constrained-dynamics.hxx:188-520) with the constraint
        models ``desc`` ((n, 46): type, frame, joint1, joint2, joint1_placement (12), joint2_placement
        (12), desired acceleration (6), Kp (6), Kd (6)).  Returns (ddq (B, nv), lambda_c (B, nc),
        iterations (B,), residuals (B, 2): absolute, relative)."""
        q, v, tau = _c(q), _c(v), _c(tau)
        desc = self._desc(desc)
        B = q.shape[0]
        nc = int(sum(3 if int(d[0]) == 0 else 6 for d in desc))
        ddq, lam = np.empty((B, self.nv)), np.empty((B, nc))
        iters, res = np.empty(B, dtype=np.int32), np.empty((B, 2))
        self._check(lib().orc_constraint_dynamics(self.h, prec, B, len(desc), _ptr(desc), _ptr(q), _ptr(v), _ptr(tau),
                                                  float(mu), int(max_iter), float(absolute_accuracy),
                                                  float(relative_accuracy), _ptr(ddq), _ptr(lam), _ptr(iters),
                                                  _ptr(res), nthreads))
        return ddq, lam, iters, res

    def contact_cholesky(self, q, desc, mu=0.0, nthreads=0):
        """ContactCholeskyDecomposition(model, contact_models).compute(model, data, contact_models,
        contact_datas, mu) at each configuration (reference algorithm/contact-cholesky.hxx:152-304) and
        its accessors (contact-cholesky.hpp:168-265, contact-cholesky.hxx:617-759): a dict of matrix
        (B, n, n), inverse (B, n, n), osim_inverse (B, nc, nc), osim (B, nc, nc), minv (B, nv, nv) and
        jminv (B, nc, nv), n = nc + nv, the constraint rows first."""
        q = _c(q)
        desc = self._desc(desc)
        B, nv = q.shape[0], self.nv
        nc = int(sum(3 if int(d[0]) == 0 else 6 for d in desc))
        n = nc + nv
        out = dict(matrix=np.empty((B, n, n)), inverse=np.empty((B, n, n)), osim_inverse=np.empty((B, nc, nc)),
                   osim=np.empty((B, nc, nc)), minv=np.empty((B, nv, nv)), jminv=np.empty((B, nc, nv)))
        self._check(lib().orc_contact_cholesky(self.h, B, len(desc), _ptr(desc), _ptr(q), float(mu),
                                               *(_ptr(out[k]) for k in ("matrix", "inverse", "osim_inverse", "osim",
                                                                        "minv", "jminv")), nthreads))
        return out

    def constraint_dynamics_derivatives(self, q, v, tau, desc, mu=0.0, max_iter=1, absolute_accuracy=1e-12,
                                        relative_accuracy=1e-12, prec=0, nthreads=0):
        """computeConstraintDynamicsDerivatives (reference algorithm/constrained-dynamics-derivatives.hxx:
        344-1050) for constraints to the world without Baumgarte gains.  Returns (ddq, lambda_c, ddq_dq,
        ddq_dv, ddq_dtau (B, nv, nv), dlambda_dq, dlambda_dv, dlambda_dtau (B, nc, nv), iterations)."""
        q, v, tau = _c(q), _c(v), _c(tau)
        desc = self._desc(desc)
        B, nv = q.shape[0], self.nv
        nc = int(sum(3 if int(d[0]) == 0 else 6 for d in desc))
        ddq, lam = np.empty((B, nv)), np.empty((B, nc))
        a = [np.empty((B, nv, nv)) for _ in range(3)]
        lm = [np.empty((B, nc, nv)) for _ in range(3)]
        iters = np.empty(B, dtype=np.int32)
        self._check(lib().orc_constraint_dynamics_derivatives(
            self.h, prec, B, len(desc), _ptr(desc), _ptr(q), _ptr(v), _ptr(tau), float(mu), int(max_iter),
            float(absolute_accuracy), float(relative_accuracy), _ptr(ddq), _ptr(lam), *(_ptr(x) for x in a),
            *(_ptr(x) for x in lm), _ptr(iters), nthreads))
        return (ddq, lam, *a, *lm, iters)

    def impulse_dynamics(self, q, v_before, J, r_coeff=0.0, inv_damping=0.0, prec=0, nthreads=0):
        """(dq_after, impulse_c) of impulseDynamics with the constraint Jacobian J (B, nc, nv)."""
        q, v, J = _c(q), _c(v_before), _c(J)
        B, nc = q.shape[0], J.shape[1]
        out, lam = np.empty((B, self.nv)), np.empty((B, nc))
        self._check(lib().orc_impulse_dynamics(self.h, prec, B, nc, _ptr(q), _ptr(v), _ptr(J), float(r_coeff),
                                               float(inv_damping), _ptr(out), _ptr(lam), nthreads))
        return out, lam

    def integrate(self, q, v, prec=0, nthreads=0):
        q, v = _c(q), _c(v)
        out = np.empty_like(q)
        self._check(lib().orc_integrate(self.h, prec, q.shape[0], _ptr(q), _ptr(v), _ptr(out), nthreads))
        return out

    def forward_kinematics(self, q, v=None, a=None, prec=0, nthreads=0):
        """(oMi (B, njoints, 12): R row-major then t; v (B, njoints, 6) or None; a (B, njoints, 6) or None),
        joint 0 the identity / zero -- data.oMi, data.v, data.a after forwardKinematics(q[, v[, a]])."""
        q = _c(q)
        B, nj = q.shape[0], self._nj_internal
        v = None if v is None else _c(v)
        a = None if (a is None or v is None) else _c(a)
        oMi = np.empty((B, nj, 12))
        vi = np.empty((B, nj, 6)) if v is not None else None
        ai = np.empty((B, nj, 6)) if a is not None else None
        self._check(lib().orc_forward_kinematics(self.h, prec, B, _ptr(q), _ptr(v), _ptr(a), _ptr(oMi), _ptr(vi),
                                                 _ptr(ai), nthreads))
        if self._rows is not None:
            pick = lambda x: None if x is None else np.ascontiguousarray(x[:, self._rows])  # noqa: E731
            return pick(oMi), pick(vi), pick(ai)
        return oMi, vi, ai

    def joint_jacobians(self, q, prec=0, nthreads=0):
        """data.J after computeJointJacobians(q): (B, nv, 6), column k of the 6 x nv matrix per row."""
        q = _c(q)
        J = np.empty((q.shape[0], self.nv, 6))
        self._check(lib().orc_joint_jacobians(self.h, prec, q.shape[0], _ptr(q), _ptr(J), nthreads))
        return J

    def count_flops(self, func, q, v=None, x=None):
        """(ops, sincos pairs) of one evaluation at a single instance."""
        q = _c(q).reshape(-1)
        v = None if v is None else _c(v).reshape(-1)
        x = None if x is None else _c(x).reshape(-1)
        ops, sc = C.c_double(), C.c_double()
        self._check(lib().orc_count_flops(self.h, func, _ptr(q), _ptr(v), _ptr(x), C.byref(ops), C.byref(sc)))
        return ops.value, sc.value


def symmetrize_upper(M):
    """make_symmetric on the upper triangle (reference bindings/python/algorithm/expose-crba.cpp:22)."""
    U = np.triu(M)
    return U + np.swapaxes(np.triu(M, 1), -1, -2)


def rollout_with_gradients(om, q0, v0, taus, dt=1e-3, nthreads=0):
    """FP64 reference of the differentiable rollout: semi-implicit Euler
    v_{k+1} = v_k + dt ABA(q_k, v_k, tau_k), q_{k+1} = q_k + dt v_{k+1} (vector-space
    configurations, nq == nv), loss ||q_T||^2 per trajectory summed; the gradients of the
    loss with respect to q0, v0 and every tau_k by the adjoint recursion over the oracle's
    analytical ABA derivatives (ddq_dq, ddq_dv, Minv).  Returns (q_T, v_T, g_q0, g_v0, g_taus)."""
    q, v = _c(q0).copy(), _c(v0).copy()
    T = taus.shape[0]
    states = []
    for k in range(T):
        states.append((q, v))
        v = v + dt * om.aba(q, v, taus[k], LOCAL, nthreads=nthreads)
        q = q + dt * v
    qT, vT = q, v
    lq, lv = 2.0 * qT, np.zeros_like(vT)
    gt = np.empty_like(_c(taus))
    for k in range(T - 1, -1, -1):
        qk, vk = states[k]
        lv = lv + dt * lq  # q_{k+1} = q_k + dt v_{k+1}
        g = dt * lv  # adjoint of ddq_k
        _, dq, dv, Minv = om.aba_derivatives(qk, vk, taus[k], nthreads=nthreads)
        lq = lq + np.einsum("bk,bkc->bc", g, dq)
        lv = lv + np.einsum("bk,bkc->bc", g, dv)
        gt[k] = np.einsum("bkc,bk->bc", Minv, g)
    return qT, vT, lq, lv, gt


class _Tables:
    def __init__(self, t):
        self.t = t

    def tables(self):
        return self.t


class MimicOracleModel:
    """Models with mimic joints (reference JointModelMimic, multibody/joint/joint-mimic.hpp:557-760),
    restated as the reference's own unit tests check them (unittest/rnea.cpp:350-420,
    unittest/crba.cpp:131-170, utils/model-generator.hpp MimicTestCases): over the *full* model, in
    which every mimic joint is a joint with its own dof, with q_full = toFull(q) (a mimic's
    coordinate scaling * q + offset; an unbounded joint's angle, LinearAffineTransform /
    UnboundedRevoluteAffineTransform, joint-common-operations.hpp:52-90) and v_full = G v:
    tau = G^T (M_full G a + nle_full), M = G^T M_full G, the kinematics of the full model at
    (toFull(q), G v, G a), data.J the full model's 6 x nvExtended Jacobian."""

    def __init__(self, model):
        t = {k: np.array(v, copy=True) for k, v in model.tables().items()}
        self.model = model
        self.mimic = [int(m) for m in t["mimic"]]
        self.scaling, self.offset = t["mimic_scaling"], t["mimic_offset"]
        nj = len(self.mimic)
        unb = {13, 14, 15, 16}
        full_nq = {0: 0, 4: 7, 10: 3, 11: 4, 12: 4, 17: 3, **{j: 2 for j in unb}}
        full_nv = {0: 0, 4: 6, 10: 3, 11: 3, 12: 3, 17: 3}
        jt = [int(j) for j in t["jtype"]]
        self.fq = np.cumsum([0] + [full_nq.get(j, 1) for j in jt])[:-1]
        self.fv = np.cumsum([0] + [full_nv.get(j, 1) for j in jt])[:-1]
        self.nq_full = int(sum(full_nq.get(j, 1) for j in jt))
        self.nv_full = int(sum(full_nv.get(j, 1) for j in jt))
        self.rq, self.rv = model.idx_qs, model.idx_vs
        self.nq, self.nv = model.nq, model.nv
        self.jt, self.unb = jt, unb
        G = np.zeros((self.nv_full, self.nv))
        arm = np.zeros(self.nv_full)
        for i in range(1, nj):
            nvi = full_nv.get(jt[i], 1)
            if self.mimic[i]:
                G[self.fv[i], self.rv[self.mimic[i]]] = self.scaling[i]
            else:
                for k in range(nvi):
                    G[self.fv[i] + k, self.rv[i] + k] = 1.0
                    arm[self.fv[i] + k] = t["armature"][self.rv[i] + k]
        self.G = G
        t["mimic"][:] = 0
        t["armature"] = arm
        self.full = OracleModel(_Tables(t))

    def to_full(self, q):
        q = np.atleast_2d(np.asarray(q, dtype=np.float64))
        out = np.zeros((q.shape[0], self.nq_full))
        full_nq = lambda j: 7 if j == 4 else 3 if j in (10, 17) else 4 if j in (11, 12) else 2 if j in self.unb else 1  # noqa: E731
        for i in range(1, len(self.mimic)):
            m, f = self.mimic[i], self.fq[i]
            if not m:
                n = full_nq(self.jt[i])
                out[:, f : f + n] = q[:, self.rq[i] : self.rq[i] + n]
            elif self.jt[i] in self.unb:
                th = self.scaling[i] * np.arctan2(q[:, self.rq[m] + 1], q[:, self.rq[m]]) + self.offset[i]
                out[:, f], out[:, f + 1] = np.cos(th), np.sin(th)
            else:
                out[:, f] = self.scaling[i] * q[:, self.rq[m]] + self.offset[i]
        return out

    def _gv(self, v):
        return np.atleast_2d(np.asarray(v, dtype=np.float64)) @ self.G.T

    def crba(self, q):
        """The symmetric reduced joint-space inertia G^T M_full G."""
        Mf = symmetrize_upper(self.full.crba(self.to_full(q)))
        return np.einsum("ki,bkl,lj->bij", self.G, Mf, self.G)

    def rnea(self, q, v, a, fext=None):
        if fext is not None:
            return self.full.rnea(self.to_full(q), self._gv(v), self._gv(a), fext=fext) @ self.G
        qf, vf = self.to_full(q), self._gv(v)
        Mf = symmetrize_upper(self.full.crba(qf))
        nle = self.full.rnea(qf, vf, np.zeros_like(vf))
        return np.einsum("ki,bkl,bl->bi", self.G, Mf, self._gv(a)) + nle @ self.G

    def forward_kinematics(self, q, v=None, a=None):
        return self.full.forward_kinematics(self.to_full(q), None if v is None else self._gv(v),
                                            None if a is None else self._gv(a))

    def joint_jacobians(self, q):
        return self.full.joint_jacobians(self.to_full(q))

    def integrate(self, q, v):
        qf = self.full.integrate(self.to_full(q), self._gv(v))
        out = np.zeros((qf.shape[0], self.nq))
        for i in range(1, len(self.mimic)):
            if not self.mimic[i]:
                n = self.model.nqs[i]
                out[:, self.rq[i] : self.rq[i] + n] = qf[:, self.fq[i] : self.fq[i] + n]
        return out


def log6(M):
    """(log6(M), Jlog6(M)) of a placement M = (R (3, 3), t (3,)) (reference spatial/explog.hpp)."""
    R, t = M
    m = _c(np.concatenate([np.asarray(R, dtype=np.float64).reshape(9), np.asarray(t, dtype=np.float64)]))
    xi, J = np.empty(6), np.empty((6, 6))
    lib().orc_log6(_ptr(m), _ptr(xi), _ptr(J))
    return xi, J

