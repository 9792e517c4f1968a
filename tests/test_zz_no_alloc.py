"""gb_aba_derivatives_noalloc: the ABA derivatives for callers that cannot
allocate device memory (real-time control loops that must not wait on an
allocator, plugins whose host owns every device allocation).  Through the
C ABI, two calls in a row must reproduce gb_aba_derivatives on the same
inputs without allocating (the device's free memory and the default memory
pool's high-water mark stay where they were), and a batch beyond the fixed
scratch must be refused.  This file is collected last so that a run stopping
at the first failure has run every other test first; it also passes alone in
a fresh process."""
import ctypes as C

import numpy as np
import pytest

import pinocchio_gb300 as pg
from pinocchio_gb300 import _capi
from pinocchio_gb300 import sample_models as sm
from util import FP64_TOL, MIXED_TOL, rel_err

pytestmark = pytest.mark.gpu


def _call(fn, data, precision, q, v, tau):
    import torch

    B, nv = q.shape[0], q.shape[1] - 1
    outs = [torch.empty((B, nv, nv), dtype=torch.float64, device="cuda") for _ in range(3)]
    ddq = torch.empty((B, nv), dtype=torch.float64, device="cuda")
    p = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    _capi.check(
        fn(data.dev.h, precision, _capi.GB_LAYOUT_INSTANCE, B, p(q), p(v), p(tau), p(outs[0]), p(outs[1]), p(outs[2]), p(ddq),
           C.c_void_p(torch.cuda.current_stream().cuda_stream))
    )
    torch.cuda.synchronize()
    return [t.cpu().numpy() for t in (*outs, ddq)]


def _cudart():
    """The CUDA runtime the library links (the same process-wide device state)."""
    for name in ("libcudart.so.13", "libcudart.so"):
        try:
            return C.CDLL(name)
        except OSError:
            pass
    pytest.skip("libcudart not found by name")


class _AllocationProbe:
    """Free device memory and the default memory pool's used-memory high-water mark
    around a region (the allocating entry point draws its workspace from that pool)."""

    def __init__(self):
        import torch

        self.rt = _cudart()
        self.pool = C.c_void_p()
        dev = torch.cuda.current_device()
        assert self.rt.cudaDeviceGetDefaultMemPool(C.byref(self.pool), dev) == 0

    def _attr(self, attr):
        val = C.c_uint64(0)
        assert self.rt.cudaMemPoolGetAttribute(self.pool, attr, C.byref(val)) == 0
        return val.value

    def _free(self):
        free, total = C.c_size_t(0), C.c_size_t(0)
        assert self.rt.cudaMemGetInfo(C.byref(free), C.byref(total)) == 0
        return free.value

    def __enter__(self):
        import torch

        torch.cuda.synchronize()
        zero = C.c_uint64(0)
        assert self.rt.cudaMemPoolSetAttribute(self.pool, 8, C.byref(zero)) == 0  # reset the used-memory high mark
        self.used0 = self._attr(7)  # cudaMemPoolAttrUsedMemCurrent
        self.free0 = self._free()
        return self

    def __exit__(self, *exc):
        import torch

        torch.cuda.synchronize()
        self.used_high = self._attr(8)  # cudaMemPoolAttrUsedMemHigh
        self.free1 = self._free()
        return False


@pytest.mark.parametrize("precision,tol", [(_capi.GB_FP64, FP64_TOL), (_capi.GB_MIXED, MIXED_TOL)])
def test_noalloc_matches_allocating_entry_point_twice(precision, tol):
    import torch

    model = sm.humanoid32(1)  # nq 33, nv 32
    data = pg.createData(model)
    L = _capi.lib()
    _call(L.gb_aba_derivatives_noalloc, data, precision, *(torch.zeros((8, n), dtype=torch.float64, device="cuda")
                                                           for n in (33, 32, 32)))  # first call: resolves the array
    for call, seed in enumerate((5, 6)):  # two calls in a row, different inputs
        q, v, x = sm.random_inputs(model, 512, seed)
        qd, vd, td = (torch.from_numpy(a).cuda() for a in (q, v, 10.0 * x))
        ref = _call(L.gb_aba_derivatives, data, precision, qd, vd, td)
        outs = [torch.empty((512, 32, 32), dtype=torch.float64, device="cuda") for _ in range(3)]
        ddq = torch.empty((512, 32), dtype=torch.float64, device="cuda")
        p = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
        with _AllocationProbe() as probe:
            _capi.check(L.gb_aba_derivatives_noalloc(data.dev.h, precision, _capi.GB_LAYOUT_INSTANCE, 512, p(qd), p(vd),
                                                     p(td), p(outs[0]), p(outs[1]), p(outs[2]), p(ddq), None))
        assert probe.used_high <= probe.used0, "the call drew memory from the default pool"
        assert probe.free1 >= probe.free0, "the call reduced the device's free memory"
        got = [t.cpu().numpy() for t in (*outs, ddq)]
        for g, r in zip(got, ref):
            assert rel_err(g, r) < tol, f"call {call}"


def test_noalloc_rejects_batches_beyond_the_scratch():
    import torch

    model = sm.humanoid32(1)
    data = pg.createData(model)
    B = 4096  # ~270 MB of workspace in FP64: beyond the fixed 64 MiB array
    t = torch.zeros((B, 33), dtype=torch.float64, device="cuda")
    o = torch.zeros((B, 32, 32), dtype=torch.float64, device="cuda")
    p = lambda x: C.c_void_p(x.data_ptr())  # noqa: E731
    rc = _capi.lib().gb_aba_derivatives_noalloc(data.dev.h, _capi.GB_FP64, _capi.GB_LAYOUT_INSTANCE, B, p(t), p(t), p(t),
                                                p(o), p(o), p(o), None, None)
    assert rc == _capi.GB_ERR_SIZE
    assert b"split the batch" in _capi.lib().gb_last_error()
