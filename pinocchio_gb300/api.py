"""Python front end mirroring the reference's ``pin.*`` entry points for the batched dynamics path.

Reference signatures (bindings/python/algorithm/...):
  ``pin.rnea(model, data, q, v, a)``, ``pin.aba(model, data, q, v, tau, convention=LOCAL)``,
  ``pin.crba(model, data, q, convention=LOCAL)`` (symmetrised, expose-crba.cpp:22),
  ``pin.computeRNEADerivatives(model, data, q, v, a) -> (dtau_dq, dtau_dv, M)``,
  ``pin.computeABADerivatives(model, data, q, v, tau) -> (ddq_dq, ddq_dv, Minv)``,
  ``pin.ModelPool(model, size)``, ``pin.rneaInParallel(num_threads, pool, q, v, a)``,
  ``pin.abaInParallel(num_threads, pool, q, v, tau)``, ``pin.integrate(model, q, v)``,
  ``pin.forwardKinematics(model, data, q[, v[, a]])``, ``pin.computeJointJacobians(model, data, q)``.

Here every single-configuration function also takes a batch: a torch CUDA
tensor of shape (batch, n) (one configuration per row, i.e. the reference's
column-major n x batch layout) or a 1-D vector.  numpy inputs are copied to the
device and the result is returned as numpy.  The ``*InParallel`` functions
take numpy arrays of shape (n, batch) exactly as the reference does and go
through the host-memory C entry points.  ``data.precision`` selects the FP64
("fp64", default) or mixed-precision ("mixed") kernels.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _capi
from .model import Convention, Model

_PREC = {"fp64": _capi.GB_FP64, "mixed": _capi.GB_MIXED}


def _torch():
    import torch

    return torch


class DeviceModel:
    """The C ABI's gb_model for one Model (uploaded to the current CUDA device)."""

    def __init__(self, model: Model):
        self.desc, self._keep = _capi.make_desc(model.tables())
        h = C.c_void_p()
        _capi.check(_capi.lib().gb_model_create(C.byref(self.desc), C.byref(h)))
        self.h = h
        self.nq, self.nv, self.njoints = model.nq, model.nv, model.njoints

    def __del__(self):
        h = getattr(self, "h", None)
        if h and _capi._lib is not None:
            _capi._lib.gb_model_destroy(h)
            self.h = None


class Data:
    """Per-model workspace handle (the reference's DataTpl role): holds the device model."""

    def __init__(self, model: Model, precision: str = "fp64"):
        if precision not in _PREC:
            raise ValueError("precision must be 'fp64' or 'mixed'")
        self.model = model
        self.precision = precision
        self.dev = DeviceModel(model)
        # outputs of the last call, as the reference keeps them in data
        self.tau = self.ddq = self.M = self.Minv = None
        self.dtau_dq = self.dtau_dv = self.ddq_dq = self.ddq_dv = None


def createData(model: Model, precision: str = "fp64") -> Data:
    return Data(model, precision)


Model.createData = lambda self, precision="fp64": Data(self, precision)  # pin: model.createData()


def numericStatus(data: Data, reset: bool = True) -> int:
    """The numeric status bits the kernels recorded for this model since it was created or
    last reset (``_capi.GB_NUMERIC_PIVOT``: a factorisation pivot was not > 0, i.e. a
    singular or indefinite inertia or NaN inputs; ``_capi.GB_NUMERIC_NONFINITE``: an output
    was NaN or infinite).  Synchronises the device; 0 means nothing was seen."""
    flags = C.c_uint(0)
    rc = _capi.lib().gb_numeric_status(data.dev.h, C.byref(flags), int(bool(reset)))
    if rc not in (_capi.GB_OK, _capi.GB_ERR_NUMERIC):
        _capi.check(rc)
    return int(flags.value)


def checkNumeric(data: Data, reset: bool = True) -> None:
    """Raises ``GBError`` (code GB_ERR_NUMERIC) when the kernels of this model recorded a
    numeric failure (see ``numericStatus``); the reference raises or asserts at the same
    points of its factorisations."""
    flags = C.c_uint(0)
    _capi.check(_capi.lib().gb_numeric_status(data.dev.h, C.byref(flags), int(bool(reset))))


def _stream_ptr():
    return C.c_void_p(_torch().cuda.current_stream().cuda_stream)


def copyAsync(dst, src) -> None:
    """dst <- src on the current CUDA stream through the library's runtime (gb_memcpy_async):
    tensors of the same number of bytes, contiguous, each on the device or in host memory
    (page-locked host memory makes the copy asynchronous).  A batch's host inputs and outputs
    move next to the calls that use them; measured on GB300, torch's own ``copy_`` between
    pinned host memory and the device stalled for tens of milliseconds every few hundred
    milliseconds while other work ran, this path does not."""
    nb = dst.numel() * dst.element_size()
    if src.numel() * src.element_size() != nb:
        raise ValueError("copyAsync: dst and src sizes differ")
    if not (dst.is_contiguous() and src.is_contiguous()):
        raise ValueError("copyAsync: tensors must be contiguous")
    _capi.check(_capi.lib().gb_memcpy_async(_ptr(dst), _ptr(src), nb, _stream_ptr()))


def _as_batch(x, n: int, name: str):
    """(tensor (B, n) float64 contiguous on CUDA, was_numpy, was_vector)."""
    torch = _torch()
    was_np = isinstance(x, np.ndarray)
    t = torch.as_tensor(x, dtype=torch.float64)
    vec = t.dim() == 1
    if vec:
        t = t.unsqueeze(0)
    if t.dim() != 2 or t.shape[1] != n:
        raise ValueError(f"{name} must have shape (batch, {n}) or ({n},), got {tuple(t.shape)}")
    if not t.is_cuda:
        t = t.cuda()
    return t.contiguous(), was_np, vec


def _ret(t, was_np, vec):
    if vec:
        t = t[0]
    return t.cpu().numpy() if was_np else t


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def _out(out, shape, like, name: str):
    """A preallocated output (``out=``): a contiguous CUDA float64 tensor of ``shape`` (or of
    ``shape[1:]`` for a single configuration) that overlaps no input, else a new one on
    ``like``'s device."""
    torch = _torch()
    if out is None:
        return torch.empty(shape, dtype=torch.float64, device=like.device)
    if isinstance(out, torch.Tensor) and shape[0] == 1 and tuple(out.shape) == tuple(shape[1:]):
        out = out.unsqueeze(0)
    if not (isinstance(out, torch.Tensor) and out.is_cuda and out.dtype == torch.float64 and out.is_contiguous()
            and tuple(out.shape) == tuple(shape)):
        raise ValueError(f"{name} must be a contiguous CUDA float64 tensor of shape {tuple(shape)}")
    return out


def _outs(out, n: int, name: str):
    if out is None:
        return (None,) * n
    if not isinstance(out, (tuple, list)) or len(out) not in (n - 1, n):
        raise ValueError(f"{name}: out must be a tuple of {n - 1} or {n} tensors")
    return tuple(out) + (None,) * (n - len(out))


def _fext(model: Model, fext, B: int):
    """External forces as the reference's Python bindings take them (a list of njoints
    forces, each [linear; angular] in its joint's frame, expressed in the local frame of
    the joints: bindings/python/algorithm/expose-rnea.cpp:38-46): an array (njoints, 6)
    shared by the batch or (B, njoints, 6) per configuration, or a list of njoints 6-vectors
    (objects with .vector, as pin.Force has, are accepted).  Returns a (B, njoints * 6)
    float64 CUDA tensor."""
    torch = _torch()
    if isinstance(fext, (list, tuple)):
        fext = [np.asarray(getattr(f, "vector", f), dtype=np.float64).reshape(6) for f in fext]
    t = torch.as_tensor(np.asarray(fext) if isinstance(fext, list) else fext, dtype=torch.float64)
    if t.dim() == 2:
        t = t.unsqueeze(0).expand(B, -1, -1)
    if t.dim() != 3 or t.shape[1] != model.njoints or t.shape[2] != 6:
        raise ValueError(f"fext must have shape ({model.njoints}, 6) or (batch, {model.njoints}, 6), got {tuple(t.shape)}")
    if t.shape[0] != B:
        raise ValueError(f"fext holds {t.shape[0]} configurations, the batch {B}")
    if not t.is_cuda:
        t = t.cuda()
    return t.reshape(B, -1).contiguous()


def rnea(model: Model, data: Data, q, v, a, fext=None, *, out=None):
    """tau = RNEA(q, v, a) (reference algorithm/rnea.hxx:117-161); with external forces
    fext (njoints forces in the joint frames) rnea(model, data, q, v, a, fext)
    (rnea.hxx:164-218).  ``out``: a preallocated (batch, nv) CUDA tensor for tau."""
    qt, was_np, vec = _as_batch(q, model.nq, "q")
    vt = _as_batch(v, model.nv, "v")[0]
    at = _as_batch(a, model.nv, "a")[0]
    B = qt.shape[0]
    tau = _out(out, (B, model.nv), qt, "out")
    if fext is None:
        _capi.check(
            _capi.lib().gb_rnea(
                data.dev.h, _PREC[data.precision], _capi.GB_LAYOUT_INSTANCE, B, _ptr(qt), _ptr(vt), _ptr(at), _ptr(tau), _stream_ptr()
            )
        )
    else:
        ft = _fext(model, fext, B)
        _capi.check(
            _capi.lib().gb_rnea_fext(
                data.dev.h, _PREC[data.precision], _capi.GB_LAYOUT_INSTANCE, B, _ptr(qt), _ptr(vt), _ptr(at), _ptr(ft), _ptr(tau),
                _stream_ptr(),
            )
        )
    data.tau = tau
    return _ret(tau, was_np, vec)


def computeStaticTorque(model: Model, data: Data, q, fext):
    """tau = g(q) - sum_i J_i^T fext_i, the joint torques that hold the configuration
    against gravity and the external forces (reference algorithm/rnea.hxx:448-489,
    binding expose-rnea.cpp:76-86)."""
    qt, was_np, vec = _as_batch(q, model.nq, "q")
    B = qt.shape[0]
    ft = _fext(model, fext, B)
    out = _torch().empty((B, model.nv), dtype=qt.dtype, device=qt.device)
    _capi.check(
        _capi.lib().gb_static_torque(
            data.dev.h, _PREC[data.precision], _capi.GB_LAYOUT_INSTANCE, B, _ptr(qt), _ptr(ft), _ptr(out), _stream_ptr()
        )
    )
    data.tau = out
    return _ret(out, was_np, vec)


def nonLinearEffects(model: Model, data: Data, q, v):
    """nle = C(q, v) v + g(q) (reference algorithm/rnea.hxx:221-336, 801-808)."""
    qt, was_np, vec = _as_batch(q, model.nq, "q")
    vt = _as_batch(v, model.nv, "v")[0]
    out = _torch().empty((qt.shape[0], model.nv), dtype=qt.dtype, device=qt.device)
    _capi.check(
        _capi.lib().gb_nonlinear_effects(
            data.dev.h, _PREC[data.precision], _capi.GB_LAYOUT_INSTANCE, qt.shape[0], _ptr(qt), _ptr(vt), _ptr(out), _stream_ptr()
        )
    )
    data.nle = out
    return _ret(out, was_np, vec)


def computeGeneralizedGravity(model: Model, data: Data, q):
    """g(q) (reference algorithm/rnea.hxx:346-446, 816-822)."""
    qt, was_np, vec = _as_batch(q, model.nq, "q")
    out = _torch().empty((qt.shape[0], model.nv), dtype=qt.dtype, device=qt.device)
    _capi.check(
        _capi.lib().gb_generalized_gravity(
            data.dev.h, _PREC[data.precision], _capi.GB_LAYOUT_INSTANCE, qt.shape[0], _ptr(qt), _ptr(out), _stream_ptr()
        )
    )
    data.g = out
    return _ret(out, was_np, vec)


def forwardKinematics(model: Model, data: Data, q, v=None, a=None):
    """forwardKinematics(model, data, q[, v[, a]]) (reference algorithm/kinematics.hxx:42-272).

    Fills and returns ``(data.oMi, data.v, data.a)``: oMi (batch, njoints, 12) world placements
    (rotation row-major, then translation; joint 0 the identity), v and a (batch, njoints, 6) the
    joint-frame spatial velocities and accelerations ([linear; angular], no gravity), or None
    when v (a) is not given."""
    torch = _torch()
    qt, was_np, vec = _as_batch(q, model.nq, "q")
    if a is not None and v is None:
        raise ValueError("forwardKinematics: an acceleration needs a velocity")
    vt = None if v is None else _as_batch(v, model.nv, "v")[0]
    at = None if a is None else _as_batch(a, model.nv, "a")[0]
    B, nj = qt.shape[0], model.njoints
    oMi = torch.empty((B, nj, 12), dtype=qt.dtype, device=qt.device)
    vo = None if vt is None else torch.empty((B, nj, 6), dtype=qt.dtype, device=qt.device)
    ao = None if at is None else torch.empty((B, nj, 6), dtype=qt.dtype, device=qt.device)
    p = lambda t: None if t is None else _ptr(t)  # noqa: E731
    _capi.check(
        _capi.lib().gb_forward_kinematics(
            data.dev.h, _PREC[data.precision], _capi.GB_LAYOUT_INSTANCE, B, _ptr(qt), p(vt), p(at), _ptr(oMi), p(vo),
            p(ao), _stream_ptr()
        )
    )
    data.oMi, data.v, data.a = oMi, vo, ao
    return tuple(None if t is None else _ret(t, was_np, vec) for t in (oMi, vo, ao))


def computeJointJacobians(model: Model, data: Data, q):
    """data.J = computeJointJacobians(model, data, q) (reference algorithm/jacobian.hxx:17-95):
    (batch, 6, nvExtended), column k the world-frame motion subspace of dof k about the world
    origin (with mimic joints, data.J has their own columns too: nvExtended = nv + their count)."""
    qt, was_np, vec = _as_batch(q, model.nq, "q")
    B, nv = qt.shape[0], model.nvExtended
    Jc = _torch().empty((B, nv, 6), dtype=qt.dtype, device=qt.device)  # column-major 6 x nv
    _capi.check(
        _capi.lib().gb_compute_joint_jacobians(
            data.dev.h, _PREC[data.precision], _capi.GB_LAYOUT_INSTANCE, B, _ptr(qt), _ptr(Jc), _stream_ptr()
        )
    )
    data.J = Jc.transpose(1, 2)
    return _ret(data.J, was_np, vec)


def computeMinverse(model: Model, data: Data, q, symmetric: bool = True):
    """Minv(q) (reference algorithm/aba.hxx:838-880), symmetrised as the Python binding returns it
    (bindings/python/algorithm/expose-aba.cpp:17-23); ``symmetric=False`` gives the C++ upper triangle."""
    qt, was_np, vec = _as_batch(q, model.nq, "q")
    nv = model.nv
    out = _torch().empty((qt.shape[0], nv, nv), dtype=qt.dtype, device=qt.device)
    mode = _capi.GB_MATRIX_SYMMETRIC if symmetric else _capi.GB_MATRIX_UPPER
    _capi.check(
        _capi.lib().gb_compute_minverse(
            data.dev.h, _PREC[data.precision], mode, _capi.GB_LAYOUT_INSTANCE, qt.shape[0], _ptr(qt), _ptr(out), _stream_ptr()
        )
    )
    data.Minv = out
    return _ret(out, was_np, vec)


def computeStaticTorqueDerivatives(model: Model, data: Data, q, fext):
    """d(computeStaticTorque)/dq (reference algorithm/rnea-derivatives.hxx:185-233, public
    686-697): the RNEA derivative sweeps with external forces at zero velocity and
    acceleration, of which the q-derivative is returned."""
    qt, was_np, vec = _as_batch(q, model.nq, "q")
    z = _torch().zeros((qt.shape[0], model.nv), dtype=qt.dtype, device=qt.device)
    dq = computeRNEADerivatives(model, data, qt, z, z, fext)[0]
    return _ret(dq, was_np, vec)


def aba(model: Model, data: Data, q, v, tau, *args, convention: int | None = None, fext=None, out=None):
    """ddq = ABA(q, v, tau) (reference algorithm/aba.hxx:933-948), called as the
    reference's binding is: aba(model, data, q, v, tau[, convention]) or
    aba(model, data, q, v, tau, fext[, convention]) with external forces in the
    joint frames (aba.hxx:958-973, expose-aba.cpp:60-82).  ``out``: a preallocated
    (batch, nv) CUDA tensor for ddq."""
    if len(args) > 2:
        raise TypeError("aba takes at most fext and convention after tau")
    for x in args:
        if isinstance(x, (int, np.integer)) and not isinstance(x, bool):
            convention = int(x)
        else:
            fext = x
    convention = Convention.LOCAL if convention is None else convention
    qt, was_np, vec = _as_batch(q, model.nq, "q")
    vt = _as_batch(v, model.nv, "v")[0]
    tt = _as_batch(tau, model.nv, "tau")[0]
    B = qt.shape[0]
    ddq = _out(out, (B, model.nv), qt, "out")
    if fext is None:
        _capi.check(
            _capi.lib().gb_aba(
                data.dev.h, _PREC[data.precision], int(convention), _capi.GB_LAYOUT_INSTANCE, B, _ptr(qt), _ptr(vt), _ptr(tt),
                _ptr(ddq), _stream_ptr(),
            )
        )
    else:
        ft = _fext(model, fext, B)
        _capi.check(
            _capi.lib().gb_aba_fext(
                data.dev.h, _PREC[data.precision], int(convention), _capi.GB_LAYOUT_INSTANCE, B, _ptr(qt), _ptr(vt), _ptr(tt),
                _ptr(ft), _ptr(ddq), _stream_ptr(),
            )
        )
    data.ddq = ddq
    return _ret(ddq, was_np, vec)


class _ConstraintSet:
    """The C ABI's gb_constraint_set of a list of RigidConstraintModel (uploaded once)."""

    def __init__(self, data: Data, desc: np.ndarray):
        self.desc = desc.copy()
        n = desc.shape[0]
        arr = (_capi.ConstraintDesc * max(n, 1))()
        for k, d in enumerate(desc):
            c = arr[k]
            c.type, c.reference_frame, c.joint1_id, c.joint2_id = (int(x) for x in d[:4])
            c.joint1_placement[:] = d[4:16].tolist()
            c.joint2_placement[:] = d[16:28].tolist()
            c.desired_acceleration[:] = d[28:34].tolist()
            c.Kp[:] = d[34:40].tolist()
            c.Kd[:] = d[40:46].tolist()
        h = C.c_void_p()
        _capi.check(_capi.lib().gb_constraint_set_create(data.dev.h, n, arr, C.byref(h)))
        self.h = h
        nn, nc = C.c_int(), C.c_int()
        _capi.check(_capi.lib().gb_constraint_set_dims(h, C.byref(nn), C.byref(nc)))
        self.n, self.nc = nn.value, nc.value
        self._data = data  # the set must not outlive its device model

    def __del__(self):
        h = getattr(self, "h", None)
        if h and _capi._lib is not None:
            _capi._lib.gb_constraint_set_destroy(h)
            self.h = None


class ContactCholeskyDecomposition:
    """ContactCholeskyDecomposition(model[, contact_models]) (reference algorithm/contact-cholesky.hpp:
    107-470) over a batch.  ``compute(model, data, contact_models, contact_datas, mu=0.0[, q=])``
    factorises the KKT matrix [[-mu I, J], [J^T, M]] (constraint rows first) at each configuration,
    J the constraint Jacobian of the models: q defaults to the configurations of the last
    ``crba(model, data, q)``, whose data.M the reference's compute reads.  The accessors return
    (batch, ...) arrays: ``matrix()``, ``inverse()``, ``getInverseOperationalSpaceInertiaMatrix()``
    (J M^-1 J^T + mu I), ``getOperationalSpaceInertiaMatrix()``, ``getInverseMassMatrix()``,
    ``getJMinv()``, and ``solve(rhs)`` (the KKT inverse applied to (batch, n) or (batch, n, k)
    right-hand sides); ``updateDamping(mu)`` refactorises with another damping.  FP64 (the CRBA's
    Cholesky is FP64 in both precisions)."""

    _KEYS = ("matrix", "inverse", "osim_inverse", "osim", "minv", "jminv")

    def __init__(self, model: Model, contact_models=()):
        self.nv = model.nv
        self._nc = int(sum(c.size() for c in contact_models))
        self._num_contacts = len(contact_models)
        self._out = None

    def compute(self, model: Model, data: Data, contact_models, contact_datas=None, mu: float = 0.0, *, q=None):
        from .constraints import stack_desc

        if not mu >= 0.0:
            raise ValueError("mu must be positive.")
        if q is None:
            q = getattr(data, "crba_q", None)
            if q is None:
                raise ValueError("compute needs the configurations: call crba(model, data, q) first or pass q=")
        qt, was_np, vec = _as_batch(q, model.nq, "q")
        desc = stack_desc(contact_models)
        cset = getattr(data, "constraint_set", None)
        if cset is None or cset.desc.shape != desc.shape or not np.array_equal(cset.desc, desc):
            data.constraint_set = cset = _ConstraintSet(data, desc)
        torch = _torch()
        B, nv, nc = qt.shape[0], model.nv, cset.nc
        n = nv + nc
        shapes = dict(matrix=(n, n), inverse=(n, n), osim_inverse=(nc, nc), osim=(nc, nc), minv=(nv, nv),
                      jminv=(nc, nv))
        out = {k: torch.empty((B,) + shapes[k], dtype=qt.dtype, device=qt.device) for k in self._KEYS}
        _capi.check(
            _capi.lib().gb_contact_cholesky(
                data.dev.h, _PREC[data.precision], cset.h, float(mu), _capi.GB_LAYOUT_INSTANCE, B, _ptr(qt),
                *(_ptr(out[k]) if out[k].numel() else None for k in self._KEYS), _stream_ptr(),
            )
        )
        self._out, self._was_np, self._vec = out, was_np, vec
        self._args = (model, data, contact_models, contact_datas, qt)
        self._nc, self._num_contacts, self.mu = nc, len(contact_models), float(mu)

    def updateDamping(self, mu: float):
        """contact-cholesky.hxx:274-304: the same factorisation with another damping."""
        model, data, cms, cds, qt = self._args
        self.compute(model, data, cms, cds, mu, q=qt)

    def _get(self, key):
        if self._out is None:
            raise ValueError("call compute first")
        return _ret(self._out[key], self._was_np, self._vec)

    def size(self) -> int:
        return self._nc + self.nv

    def constraintDim(self) -> int:
        return self._nc

    def numContacts(self) -> int:
        return self._num_contacts

    def matrix(self):
        return self._get("matrix")

    def inverse(self):
        return self._get("inverse")

    def getInverseOperationalSpaceInertiaMatrix(self):
        return self._get("osim_inverse")

    def getOperationalSpaceInertiaMatrix(self):
        return self._get("osim")

    def getInverseMassMatrix(self):
        return self._get("minv")

    def getJMinv(self):
        return self._get("jminv")

    def getDelassusCholeskyExpression(self):
        """The damped Delassus matrix J M^-1 J^T + mu I as an operator (DelassusCholeskyExpressionTpl,
        contact-cholesky.hpp:520-620): ``expr @ x`` / ``expr.solve(x)`` for (batch, nc) or (batch, nc, k)
        right-hand sides, ``matrix()``, ``inverse()``, ``size()``, ``updateDamping(mu)``."""
        return _DelassusCholeskyExpression(self)

    def solve(self, rhs):
        """KKT^-1 rhs for (batch, n) or (batch, n, k) right-hand sides (contact-cholesky.hxx:306-330)."""
        if self._out is None:
            raise ValueError("call compute first")
        torch = _torch()
        K = self._out["inverse"]
        r = torch.as_tensor(np.asarray(rhs) if not torch.is_tensor(rhs) else rhs, dtype=K.dtype).to(K.device)
        x = torch.matmul(K, r.unsqueeze(-1)).squeeze(-1) if r.dim() == 2 else torch.matmul(K, r)
        return x.cpu().numpy() if not torch.is_tensor(rhs) else x


class _DelassusCholeskyExpression:
    def __init__(self, chol: ContactCholeskyDecomposition):
        self.chol = chol

    def _apply(self, key, x):
        torch = _torch()
        K = self.chol._out[key]
        r = torch.as_tensor(np.asarray(x) if not torch.is_tensor(x) else x, dtype=K.dtype).to(K.device)
        y = torch.matmul(K, r.unsqueeze(-1)).squeeze(-1) if r.dim() == 2 else torch.matmul(K, r)
        return y.cpu().numpy() if not torch.is_tensor(x) else y

    def __matmul__(self, x):  # applyOnTheRight
        return self._apply("osim_inverse", x)

    def solve(self, x):
        return self._apply("osim", x)

    def matrix(self):
        return self.chol.getInverseOperationalSpaceInertiaMatrix()

    def inverse(self):
        return self.chol.getOperationalSpaceInertiaMatrix()

    def size(self) -> int:
        return self.chol.constraintDim()

    def updateDamping(self, mu: float):
        self.chol.updateDamping(mu)


def initConstraintDynamics(model: Model, data: Data, contact_models) -> None:
    """initConstraintDynamics(model, data, contact_models) (reference
    algorithm/constrained-dynamics.hxx:21-60): uploads the constraint models for the calls of
    constraintDynamics; a later call with different models (or changed gains) uploads them again."""
    from .constraints import stack_desc

    data.constraint_set = _ConstraintSet(data, stack_desc(contact_models))


def constraintDynamics(model: Model, data: Data, q, v, tau, contact_models, contact_datas=None, settings=None, *,
                       out=None):
    """ddq = constraintDynamics(model, data, q, v, tau, contact_models, contact_datas[, settings])
    (reference algorithm/constrained-dynamics.hxx:188-520, constrained-dynamics.hpp:90-110) over a
    batch: data.lambda_c (batch, constraint_dim) the multipliers, contact_datas[k].contact_force
    (batch, 6) each constraint's force in its frame, data.constraint_iterations (batch,) and
    data.constraint_residuals (batch, 2: absolute, relative) per configuration; settings.iter and the
    residuals become the largest over the batch.  ``out``: a preallocated (batch, nv) tensor for ddq."""
    from .constraints import ProximalSettings, stack_desc

    torch = _torch()
    settings = ProximalSettings() if settings is None else settings
    desc = stack_desc(contact_models)
    cset = getattr(data, "constraint_set", None)
    if cset is None or cset.desc.shape != desc.shape or not np.array_equal(cset.desc, desc):
        initConstraintDynamics(model, data, contact_models)
        cset = data.constraint_set
    if contact_datas is not None and len(contact_datas) != len(contact_models):
        raise ValueError("The contact models and data do not have the same vector size.")
    qt, was_np, vec = _as_batch(q, model.nq, "q")
    vt = _as_batch(v, model.nv, "v")[0]
    tt = _as_batch(tau, model.nv, "tau")[0]
    B, nc = qt.shape[0], cset.nc
    ddq = _out(out, (B, model.nv), qt, "out")
    lam = torch.empty((B, nc), dtype=torch.float64, device=qt.device)
    iters = torch.empty(B, dtype=torch.int32, device=qt.device)
    res = torch.empty((B, 2), dtype=torch.float64, device=qt.device)
    ps = _capi.ProximalSettingsC(float(settings.absolute_accuracy), float(settings.relative_accuracy),
                                 float(settings.mu), int(settings.max_iter))
    _capi.check(
        _capi.lib().gb_constraint_dynamics(
            data.dev.h, _PREC[data.precision], cset.h, C.byref(ps), _capi.GB_LAYOUT_INSTANCE, B, _ptr(qt), _ptr(vt),
            _ptr(tt), _ptr(ddq), _ptr(lam) if nc else None, _ptr(iters), _ptr(res), _stream_ptr(),
        )
    )
    data.ddq, data.lambda_c, data.constraint_iterations, data.constraint_residuals = ddq, lam, iters, res
    data.constraint_inputs = (qt, vt, tt, settings)
    if B:
        settings.iter = int(iters.max().item())
        settings.absolute_residual = float(res[:, 0].max().item())
        settings.relative_residual = float(res[:, 1].max().item())
    if contact_datas is not None:
        row = 0
        for cd, cm in zip(contact_datas, contact_models):
            n = cm.size()
            f = torch.zeros((B, 6), dtype=torch.float64, device=qt.device)
            f[:, :n] = lam[:, row : row + n]
            cd.contact_force = _ret(f, was_np, vec)
            row += n
    return _ret(ddq, was_np, vec)


def computeConstraintDynamicsDerivatives(model: Model, data: Data, contact_models, contact_datas=None, settings=None):
    """(ddq_dq, ddq_dv, ddq_dtau, dlambda_dq, dlambda_dv, dlambda_dtau) at the inputs of the last
    constraintDynamics call on ``data`` (reference
    algorithm/constrained-dynamics-derivatives.hxx:344-1050, binding
    expose-constrained-dynamics-derivatives.cpp:23-37): batched (batch, nv, nv) and
    (batch, constraint_dim, nv) tensors, also kept in data.  Constraints to the world, with
    Baumgarte gains on LOCAL contacts only (others raise)."""
    torch = _torch()
    inputs = getattr(data, "constraint_inputs", None)
    if inputs is None:
        raise RuntimeError("call constraintDynamics first")
    qt, vt, tt, last_settings = inputs
    settings = last_settings if settings is None else settings
    from .constraints import stack_desc

    cset = data.constraint_set
    desc = stack_desc(contact_models)
    if cset.desc.shape != desc.shape or not np.array_equal(cset.desc, desc):
        raise ValueError("the constraint models differ from the last constraintDynamics call")
    B, nv, nc = qt.shape[0], model.nv, cset.nc
    dev = qt.device
    ddq = torch.empty((B, nv), dtype=torch.float64, device=dev)
    lam = torch.empty((B, nc), dtype=torch.float64, device=dev)
    mats = [torch.empty((B, nv, nv), dtype=torch.float64, device=dev) for _ in range(3)]
    lmats = [torch.empty((B, nc, nv), dtype=torch.float64, device=dev) for _ in range(3)]
    iters = torch.empty(B, dtype=torch.int32, device=dev)
    ps = _capi.ProximalSettingsC(float(settings.absolute_accuracy), float(settings.relative_accuracy),
                                 float(settings.mu), int(settings.max_iter))
    lp = [_ptr(t) if nc else None for t in [lam] + lmats]
    _capi.check(
        _capi.lib().gb_constraint_dynamics_derivatives(
            data.dev.h, _PREC[data.precision], cset.h, C.byref(ps), _capi.GB_LAYOUT_INSTANCE, B, _ptr(qt), _ptr(vt),
            _ptr(tt), _ptr(ddq), lp[0], *(_ptr(t) for t in mats), *lp[1:], _ptr(iters), _stream_ptr(),
        )
    )
    data.ddq_dq, data.ddq_dv, data.ddq_dtau = mats
    data.dlambda_dq, data.dlambda_dv, data.dlambda_dtau = lmats
    return tuple(mats + lmats)


def _constraint(x, B: int, shape: tuple, name: str):
    """A per-configuration constraint array (B, *shape), or one (shape) shared by the batch,
    as a contiguous float64 CUDA tensor."""
    torch = _torch()
    t = torch.as_tensor(x, dtype=torch.float64)
    if t.dim() == len(shape):
        t = t.unsqueeze(0).expand(B, *shape)
    if tuple(t.shape) != (B, *shape):
        raise ValueError(f"{name} must have shape {shape} or (batch, *{shape}), got {tuple(t.shape)}")
    if not t.is_cuda:
        t = t.cuda()
    return t.contiguous()


def forwardDynamics(model: Model, data: Data, q, v, tau, J, gamma, inv_damping: float = 0.0):
    """ddq of the dynamics under the constraints J ddq + gamma = 0 (J: (nc, nv) or (batch, nc, nv),
    gamma: (nc,) or (batch, nc)), with the multipliers in data.lambda_c (reference
    algorithm/contact-dynamics.hxx:81-165): M ddq + nle = tau + J^T lambda_c."""
    qt, was_np, vec = _as_batch(q, model.nq, "q")
    vt = _as_batch(v, model.nv, "v")[0]
    tt = _as_batch(tau, model.nv, "tau")[0]
    B = qt.shape[0]
    Jt = _torch().as_tensor(J)
    nc = int(Jt.shape[-2])
    Jt = _constraint(J, B, (nc, model.nv), "J")
    gt = _constraint(gamma, B, (nc,), "gamma")
    ddq = _torch().empty((B, model.nv), dtype=qt.dtype, device=qt.device)
    lam = _torch().empty((B, nc), dtype=qt.dtype, device=qt.device)
    _capi.check(
        _capi.lib().gb_forward_dynamics(
            data.dev.h, _PREC[data.precision], _capi.GB_LAYOUT_INSTANCE, B, nc, _ptr(qt), _ptr(vt), _ptr(tt), _ptr(Jt),
            _ptr(gt), float(inv_damping), _ptr(ddq), _ptr(lam), _stream_ptr(),
        )
    )
    data.ddq, data.lambda_c = ddq, _ret(lam, was_np, vec)
    return _ret(ddq, was_np, vec)


def impulseDynamics(model: Model, data: Data, q, v_before, J, r_coeff: float = 0.0, inv_damping: float = 0.0):
    """The velocity after an impact on the constraints J (restitution r_coeff), with the
    impulses in data.impulse_c (reference algorithm/contact-dynamics.hxx:255-327):
    M (dq_after - v_before) = J^T impulse_c, J dq_after = -r_coeff J v_before."""
    qt, was_np, vec = _as_batch(q, model.nq, "q")
    vt = _as_batch(v_before, model.nv, "v_before")[0]
    B = qt.shape[0]
    nc = int(_torch().as_tensor(J).shape[-2])
    Jt = _constraint(J, B, (nc, model.nv), "J")
    out = _torch().empty((B, model.nv), dtype=qt.dtype, device=qt.device)
    imp = _torch().empty((B, nc), dtype=qt.dtype, device=qt.device)
    _capi.check(
        _capi.lib().gb_impulse_dynamics(
            data.dev.h, _PREC[data.precision], _capi.GB_LAYOUT_INSTANCE, B, nc, _ptr(qt), _ptr(vt), _ptr(Jt),
            float(r_coeff), float(inv_damping), _ptr(out), _ptr(imp), _stream_ptr(),
        )
    )
    data.dq_after, data.impulse_c = out, _ret(imp, was_np, vec)
    return _ret(out, was_np, vec)


def computeKKTContactDynamicMatrixInverse(model: Model, data: Data, q, J, inv_damping: float = 0.0):
    """[[M, J^T], [J, -inv_damping I]]^-1, shape (batch, nv + nc, nv + nc) (reference
    algorithm/contact-dynamics.hxx:166-225), FP64."""
    qt, was_np, vec = _as_batch(q, model.nq, "q")
    B = qt.shape[0]
    nc = int(_torch().as_tensor(J).shape[-2])
    Jt = _constraint(J, B, (nc, model.nv), "J")
    n = model.nv + nc
    K = _torch().empty((B, n, n), dtype=qt.dtype, device=qt.device)
    _capi.check(
        _capi.lib().gb_kkt_contact_inverse(
            data.dev.h, _PREC[data.precision], _capi.GB_LAYOUT_INSTANCE, B, nc, _ptr(qt), _ptr(Jt), float(inv_damping),
            _ptr(K), _stream_ptr(),
        )
    )
    return _ret(K, was_np, vec)


def crba(model: Model, data: Data, q, convention: int = Convention.LOCAL, symmetric: bool = True, *, out=None):
    """M(q), symmetrised as the Python binding returns it (reference bindings/python/algorithm/expose-crba.cpp:22).
    ``out``: a preallocated (batch, nv, nv) CUDA tensor for M."""
    qt, was_np, vec = _as_batch(q, model.nq, "q")
    B, nv = qt.shape[0], model.nv
    M = _out(out, (B, nv, nv), qt, "out")
    mode = _capi.GB_MATRIX_SYMMETRIC if symmetric else _capi.GB_MATRIX_UPPER
    _capi.check(
        _capi.lib().gb_crba(
            data.dev.h, _PREC[data.precision], int(convention), mode, _capi.GB_LAYOUT_INSTANCE, B, _ptr(qt), _ptr(M), None, None,
            _stream_ptr(),
        )
    )
    data.M = M
    data.crba_q = qt  # the configurations data.M belongs to (ContactCholeskyDecomposition.compute reads them)
    return _ret(M, was_np, vec)


def crbaCholesky(model: Model, data: Data, q):
    """(M, U, D) with M = U diag(D) U^T, the cholesky::decompose factorisation (reference algorithm/cholesky.hxx:18-62), FP64."""
    qt, was_np, vec = _as_batch(q, model.nq, "q")
    B, nv = qt.shape[0], model.nv
    torch = _torch()
    M = torch.empty((B, nv, nv), dtype=qt.dtype, device=qt.device)
    U = torch.empty_like(M)
    D = torch.empty((B, nv), dtype=qt.dtype, device=qt.device)
    _capi.check(
        _capi.lib().gb_crba(
            data.dev.h, _PREC[data.precision], Convention.LOCAL, _capi.GB_MATRIX_SYMMETRIC, _capi.GB_LAYOUT_INSTANCE, B, _ptr(qt),
            _ptr(M), _ptr(U), _ptr(D), _stream_ptr(),
        )
    )
    return tuple(_ret(t, was_np, vec) for t in (M, U, D))


def computeRNEADerivatives(model: Model, data: Data, q, v, a, fext=None, *, out=None):
    """(dtau_dq, dtau_dv, M) (reference algorithm/rnea-derivatives.hxx:472-541, M symmetrised as the binding does);
    with external forces fext in the joint frames, rnea-derivatives.hxx:550-633.  ``out``: preallocated
    CUDA tensors (dtau_dq, dtau_dv, M[, tau]) of shapes (batch, nv, nv) and (batch, nv)."""
    qt, was_np, vec = _as_batch(q, model.nq, "q")
    vt = _as_batch(v, model.nv, "v")[0]
    at = _as_batch(a, model.nv, "a")[0]
    B, nv = qt.shape[0], model.nv
    o = _outs(out, 4, "computeRNEADerivatives")
    dq, dv, M = (_out(t, (B, nv, nv), qt, "out") for t in o[:3])
    tau = _out(o[3], (B, nv), qt, "out")
    prec, h = _PREC[data.precision], data.dev.h
    if fext is None:
        rc = _capi.lib().gb_rnea_derivatives(
            h, prec, _capi.GB_MATRIX_SYMMETRIC, _capi.GB_LAYOUT_INSTANCE, B, _ptr(qt), _ptr(vt), _ptr(at), _ptr(dq), _ptr(dv),
            _ptr(M), _ptr(tau), _stream_ptr(),
        )
    else:
        ft = _fext(model, fext, B)
        rc = _capi.lib().gb_rnea_derivatives_fext(
            h, prec, _capi.GB_MATRIX_SYMMETRIC, _capi.GB_LAYOUT_INSTANCE, B, _ptr(qt), _ptr(vt), _ptr(at), _ptr(ft), _ptr(dq),
            _ptr(dv), _ptr(M), _ptr(tau), _stream_ptr(),
        )
    _capi.check(rc)
    data.dtau_dq, data.dtau_dv, data.M, data.tau = dq, dv, M, tau
    return tuple(_ret(t, was_np, vec) for t in (dq, dv, M))


def computeABADerivatives(model: Model, data: Data, q, v, tau, fext=None, *, out=None):
    """(ddq_dq, ddq_dv, Minv) (reference algorithm/aba-derivatives.hxx:380-453); with external
    forces fext in the joint frames, aba-derivatives.hxx:463-541.  ``out``: preallocated CUDA
    tensors (ddq_dq, ddq_dv, Minv[, ddq]) of shapes (batch, nv, nv) and (batch, nv)."""
    qt, was_np, vec = _as_batch(q, model.nq, "q")
    vt = _as_batch(v, model.nv, "v")[0]
    tt = _as_batch(tau, model.nv, "tau")[0]
    B, nv = qt.shape[0], model.nv
    o = _outs(out, 4, "computeABADerivatives")
    dq, dv, Minv = (_out(t, (B, nv, nv), qt, "out") for t in o[:3])
    ddq = _out(o[3], (B, nv), qt, "out")
    prec, h = _PREC[data.precision], data.dev.h
    if fext is None:
        rc = _capi.lib().gb_aba_derivatives(
            h, prec, _capi.GB_LAYOUT_INSTANCE, B, _ptr(qt), _ptr(vt), _ptr(tt), _ptr(dq), _ptr(dv), _ptr(Minv), _ptr(ddq),
            _stream_ptr(),
        )
    else:
        ft = _fext(model, fext, B)
        rc = _capi.lib().gb_aba_derivatives_fext(
            h, prec, _capi.GB_LAYOUT_INSTANCE, B, _ptr(qt), _ptr(vt), _ptr(tt), _ptr(ft), _ptr(dq), _ptr(dv), _ptr(Minv),
            _ptr(ddq), _stream_ptr(),
        )
    _capi.check(rc)
    data.ddq_dq, data.ddq_dv, data.Minv, data.ddq = dq, dv, Minv, ddq
    return tuple(_ret(t, was_np, vec) for t in (dq, dv, Minv))


def abaDerivativesVJP(model: Model, data: Data, q, v, tau, g):
    """(q_bar, v_bar, tau_bar) = (ddq_dq^T g, ddq_dv^T g, Minv g) for a gradient g on ddq, without
    forming the Jacobians (gb_aba_derivatives_vjp; used by the autograd wrapper)."""
    qt, was_np, vec = _as_batch(q, model.nq, "q")
    vt = _as_batch(v, model.nv, "v")[0]
    tt = _as_batch(tau, model.nv, "tau")[0]
    gt = _as_batch(g, model.nv, "g")[0]
    torch = _torch()
    qb, vb, tb = (torch.empty_like(vt) for _ in range(3))
    _capi.check(
        _capi.lib().gb_aba_derivatives_vjp(
            data.dev.h, _PREC[data.precision], _capi.GB_LAYOUT_INSTANCE, qt.shape[0], _ptr(qt), _ptr(vt), _ptr(tt),
            _ptr(gt), _ptr(qb), _ptr(vb), _ptr(tb), None, _stream_ptr(),
        )
    )
    return tuple(_ret(t, was_np, vec) for t in (qb, vb, tb))


def integrate(model: Model, q, v, data: Data | None = None):
    """q (+) v on the configuration manifold (reference algorithm/joint-configuration.hpp:41-80), FP64."""
    data = data or Data(model)
    qt, was_np, vec = _as_batch(q, model.nq, "q")
    vt = _as_batch(v, model.nv, "v")[0]
    out = _torch().empty_like(qt)
    _capi.check(
        _capi.lib().gb_integrate(data.dev.h, _capi.GB_LAYOUT_INSTANCE, qt.shape[0], _ptr(qt), _ptr(vt), _ptr(out), _stream_ptr())
    )
    return _ret(out, was_np, vec)


class ModelPool:
    """ModelPool(model, size) (reference multibody/pool/model.hpp:19-165)."""

    def __init__(self, model: Model, size: int | None = None, precision: str = "fp64"):
        import os

        self.model = model
        self._dev = DeviceModel(model)
        size = os.cpu_count() if size is None else int(size)
        h = C.c_void_p()
        _capi.check(_capi.lib().gb_pool_create(self._dev.h, size, C.byref(h)))
        self.h = h
        self.set_precision(precision)

    def set_precision(self, precision: str) -> None:
        _capi.check(_capi.lib().gb_pool_set_precision(self.h, _PREC[precision]))

    def size(self) -> int:
        n = C.c_long()
        _capi.check(_capi.lib().gb_pool_size(self.h, C.byref(n)))
        return n.value

    def getModel(self, index: int = 0) -> Model:
        if not 0 <= index < self.size():
            raise ValueError("Index greater than the size of the model vector.")
        return self.model

    def __del__(self):
        h = getattr(self, "h", None)
        if h and _capi._lib is not None:
            _capi._lib.gb_pool_destroy(h)
            self.h = None


def _colmajor(x, rows: int, name: str):
    a = np.asarray(x, dtype=np.float64)
    if a.ndim == 1:
        a = a.reshape(rows, 1)
    if a.ndim != 2 or a.shape[0] != rows:
        raise ValueError(f"{name} must have {rows} rows (one column per configuration), got {a.shape}")
    return np.asfortranarray(a)


def _in_parallel(fn, num_threads, pool, x1, x2, x3, out, names):
    m = pool.model
    q = _colmajor(x1, m.nq, names[0])
    v = _colmajor(x2, m.nv, names[1])
    x = _colmajor(x3, m.nv, names[2])
    B = q.shape[1]
    if v.shape[1] != B or x.shape[1] != B:
        raise ValueError("all inputs must have the same number of columns")
    res = np.empty((m.nv, B), order="F") if out is None else out
    if res.shape != (m.nv, B) or not res.flags.f_contiguous or res.dtype != np.float64:
        raise ValueError(f"output must be a Fortran-ordered float64 array of shape ({m.nv}, {B})")
    p = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    _capi.check(fn(int(num_threads), pool.h, B, p(q), p(v), p(x), p(res)))
    return res


def rneaInParallel(num_threads: int, pool: ModelPool, q, v, a, tau=None):
    """Batch RNEA over columns (reference algorithm/parallel/rnea.hpp:39-84)."""
    return _in_parallel(_capi.lib().gb_rnea_in_parallel, num_threads, pool, q, v, a, tau, ("q", "v", "a"))


def abaInParallel(num_threads: int, pool: ModelPool, q, v, tau, a=None):
    """Batch ABA over columns, WORLD convention (reference algorithm/parallel/aba.hpp:40-84)."""
    return _in_parallel(_capi.lib().gb_aba_in_parallel, num_threads, pool, q, v, tau, a, ("q", "v", "tau"))


# ------------------------------------------------------------------------------------------
# heterogeneous batch: several models, RNEA / ABA tasks, one persistent launch
# ------------------------------------------------------------------------------------------
_FUNC = {"rnea": _capi.GB_FUNC_RNEA, "aba": _capi.GB_FUNC_ABA}


class MultiBatch:
    """RNEA / ABA tasks over several models evaluated by one persistent launch (gb_batch_multi).

    ``tasks`` is a list of ``(data, function, q, v, x)`` with ``function`` in
    {"rnea", "aba"} and CUDA float64 tensors of shape (batch, nq) / (batch, nv);
    outputs are allocated once.  ``run()`` launches on the current stream;
    ``capture()`` records the launch into a CUDA graph that ``replay()`` re-runs
    (the launch allocates nothing).
    """

    def __init__(self, tasks, precision: str = "fp64", threads_per_block: int = 0):
        torch = _torch()
        if len(tasks) > 16:
            raise ValueError("at most 16 tasks per launch")
        self.precision = precision
        self.threads_per_block = int(threads_per_block)
        self._keep = []
        self.outputs = []
        arr = (_capi.Task * len(tasks))()
        for k, (data, function, q, v, x) in enumerate(tasks):
            m = data.model
            q, v, x = (t.contiguous() for t in (q, v, x))
            out = torch.empty((q.shape[0], m.nv), dtype=torch.float64, device=q.device)
            self._keep += [q, v, x, out, data]
            self.outputs.append(out)
            arr[k].model = data.dev.h.value
            arr[k].function = _FUNC[function]
            arr[k].batch = q.shape[0]
            arr[k].q, arr[k].v, arr[k].x, arr[k].out = (t.data_ptr() for t in (q, v, x, out))
        self._tasks = arr
        self._graph = None

    def run(self):
        _capi.check(
            _capi.lib().gb_batch_multi(self._tasks, len(self._tasks), _PREC[self.precision], self.threads_per_block, _stream_ptr())
        )
        return self.outputs

    def capture(self):
        torch = _torch()
        self.run()  # warm-up outside the capture (sets kernel attributes)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.run()
        self._graph = g
        return g

    def replay(self):
        if self._graph is None:
            self.capture()
        self._graph.replay()
        return self.outputs
