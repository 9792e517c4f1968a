"""Launch autotuner: picks, per model and function, the layout and the
configurations per CTA.

Every batched entry point evaluates one configuration per thread by default;
RNEA, ABA (and the functions built on them) and the ABA derivatives also have a
warp-per-instance layout (``gb_model_set_layout``): for RNEA and ABA the 32
lanes of a warp evaluate one configuration with the joints of a tree level in
parallel, and a lane-per-branch layout gives each chain of the tree a lane (a
team of 4-32 lanes per configuration, several configurations per warp); for the ABA derivatives a team of 4, 8 or 32 lanes splits the loops
over matrix columns (subtree, ancestor and Minv-row columns of every joint)
while every lane repeats the per-joint work, which pays on deep trees such as
the 100-link chain at small batches.  They win when the batch is too small to
fill the GPU one thread per configuration.  For the thread layout
the free parameter is how many configurations share a CTA (and so the model
tables staged in its shared memory): small CTAs spread a small batch over more
SMs, large ones amortise the staging.  ``tune`` times the candidates with CUDA
events on the given batch, applies the fastest and records it in a JSON cache
(keyed by GPU name, model tables, function, precision and batch size) so that
later processes reuse it without timing again.  The heterogeneous launch is
tuned over its threads_per_block argument (``tune_multi``).
"""
from __future__ import annotations

import hashlib
import json
import os

import numpy as np

from . import _capi, api
from . import sample_models as sm
from .model import JT_PL, JT_SPH

CANDIDATES = (32, 64, 96, 128)  # configurations per CTA, one thread each
WARP = "warp"  # one warp per configuration (RNEA, ABA, ABA derivatives)
LANES4, LANES8 = "lanes4", "lanes8"  # a team of 4 or 8 lanes per configuration (ABA derivatives)
BRANCH = "branch"  # one lane per chain of the tree (RNEA, ABA)
_LAYOUT = {WARP: _capi.GB_INSTANCE_PER_WARP, LANES4: _capi.GB_INSTANCE_PER_4_LANES,
           LANES8: _capi.GB_INSTANCE_PER_8_LANES, BRANCH: _capi.GB_INSTANCE_PER_BRANCH}
CACHE_PATH = os.environ.get(
    "PINOCCHIO_GB300_AUTOTUNE_CACHE", os.path.join(os.path.expanduser("~"), ".cache", "pinocchio_gb300", "autotune.json")
)
_FUNCS = {
    "rnea": _capi.GB_FUNC_RNEA,
    "aba": _capi.GB_FUNC_ABA,
    "crba": _capi.GB_FUNC_CRBA,
    "rnea_derivatives": _capi.GB_FUNC_RNEA_DERIVATIVES,
    "aba_derivatives": _capi.GB_FUNC_ABA_DERIVATIVES,
}


def model_key(model) -> str:
    h = hashlib.sha1()
    for k, v in sorted(model.tables().items()):
        h.update(k.encode())
        h.update(np.ascontiguousarray(v).tobytes())
    return h.hexdigest()[:16]


def _load():
    try:
        return json.load(open(CACHE_PATH))
    except (OSError, ValueError):
        return {}


def _save(cache):
    try:
        os.makedirs(os.path.dirname(CACHE_PATH), exist_ok=True)
        json.dump(cache, open(CACHE_PATH, "w"), indent=1, sort_keys=True)
    except OSError:
        pass


def _time(fn, reps=5):
    import torch

    fn()
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record()
    for _ in range(reps):
        fn()
    e.record()
    torch.cuda.synchronize()
    return s.elapsed_time(e) / reps


def tune(model, data, functions=("rnea", "aba", "crba", "rnea_derivatives", "aba_derivatives"), batch=16384,
         candidates=CANDIDATES, use_cache=True):
    """Tune ``data``'s device model; returns {function: (threads_per_block or WARP, ms)}."""
    import torch

    dev = torch.cuda.get_device_name()
    key = f"{dev}|{model_key(model)}|{data.precision}|{batch}"
    cache = _load() if use_cache else {}
    q, v, x = (torch.from_numpy(a).cuda() for a in sm.random_inputs(model, batch, 0))
    calls = {
        "rnea": lambda: api.rnea(model, data, q, v, x),
        "aba": lambda: api.aba(model, data, q, v, x),
        "crba": lambda: api.crba(model, data, q),
        "rnea_derivatives": lambda: api.computeRNEADerivatives(model, data, q, v, x),
        "aba_derivatives": lambda: api.computeABADerivatives(model, data, q, v, x),
    }
    def apply(f, setting):
        L = _capi.lib()
        if setting in _LAYOUT:
            _capi.check(L.gb_model_set_layout(data.dev.h, _FUNCS[f], _LAYOUT[setting]))
        else:
            _capi.check(L.gb_model_set_layout(data.dev.h, _FUNCS[f], _capi.GB_INSTANCE_PER_THREAD))
            _capi.check(L.gb_model_set_launch(data.dev.h, _FUNCS[f], int(setting)))

    three_dof = any(jt in (JT_SPH, JT_PL) for jt in model.jtypes)
    result = {}
    for f in functions:
        ck = f"{key}|{f}"
        if ck in cache:
            setting, ms = cache[ck]
        else:
            best = None
            settings = list(candidates)
            if not three_dof:  # spherical and planar joints run one configuration per thread
                settings += [WARP, BRANCH] if f in ("rnea", "aba") else []
                if f == "aba_derivatives":
                    settings += [LANES4, LANES8, WARP]
            for st in settings:
                apply(f, st)
                ms = _time(calls[f])
                if best is None or ms < best[1]:
                    best = (st, ms)
            setting, ms = best
            cache[ck] = [setting, ms]
        apply(f, setting)
        result[f] = (setting if setting in _LAYOUT else int(setting), float(ms))
    if use_cache:
        _save(cache)
    return result


def tune_multi(tasks, precision="fp64", candidates=(64, 128, 256)):
    """Best threads_per_block for a heterogeneous batch (MultiBatch); returns (tpb, ms)."""
    best = None
    for tpb in candidates:
        mb = api.MultiBatch(tasks, precision, tpb)
        ms = _time(mb.run)
        if best is None or ms < best[1]:
            best = (tpb, ms)
    return best
