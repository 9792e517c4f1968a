"""GPU tests of the heterogeneous single-launch batch (RNEA + ABA tasks over the
four seeded random trees, nv 7 / 12 / 32 (free-flyer) / 60 (free-flyer),
instances split 40/30/20/10 %), its CUDA-graph capture, and the autotuner."""
import numpy as np
import pytest

import pinocchio_gb300 as pg
from oracle.oracle import LOCAL, OracleModel
from pinocchio_gb300 import api, autotune
from pinocchio_gb300 import sample_models as sm
from util import FP64_TOL, MIXED_TOL, mixed_tol, rel_err

pytestmark = pytest.mark.gpu


def _tasks(precision, total=4000, seed=0):
    import torch

    models = sm.heterogeneous_trees(3)
    shares = (0.4, 0.3, 0.2, 0.1)
    tasks, ref = [], []
    for k, (model, share) in enumerate(zip(models, shares)):
        B = int(total * share)
        q, v, x = sm.random_inputs(model, B, seed + k)
        data = pg.createData(model, precision)
        d = lambda a: torch.from_numpy(a).cuda()  # noqa: E731
        tasks.append((data, "aba", d(q), d(v), d(10.0 * x)))
        tasks.append((data, "rnea", d(q), d(v), d(x)))
        ref.append((model, q, v, x))
    return tasks, ref


@pytest.mark.parametrize("precision,tol", [("fp64", FP64_TOL), ("mixed", MIXED_TOL)])
def test_multi_matches_oracle_and_single_model_calls(precision, tol):
    import torch

    tasks, ref = _tasks(precision)
    mb = api.MultiBatch(tasks, precision)
    outs = [o.cpu().numpy() for o in mb.run()]
    for k, (model, q, v, x) in enumerate(ref):
        om = OracleModel(model)
        assert rel_err(outs[2 * k], om.aba(q, v, 10.0 * x, LOCAL)) < tol
        assert rel_err(outs[2 * k + 1], om.rnea(q, v, x)) < tol
        data = tasks[2 * k][0]
        single = pg.aba(model, data, torch.from_numpy(q).cuda(), torch.from_numpy(v).cuda(), torch.from_numpy(10.0 * x).cuda())
        assert np.array_equal(single.cpu().numpy(), outs[2 * k])  # same per-instance code


@pytest.mark.parametrize("precision,tol", [("fp64", FP64_TOL), ("mixed", MIXED_TOL)])
def test_multi_per_tree_layouts(precision, tol):
    """Tasks of the same launch in different layouts (the autotuner's choice per
    tree, gb_model_set_layout): warp-layout trees give their single-model calls'
    results (same bits in FP64) and the oracle's."""
    import torch

    tasks, ref = _tasks(precision, 1200, 5)
    L = pg._capi.lib()
    for k in (0, 2):  # nv 7 and 32 (free-flyer) trees: one warp per configuration
        for f in (pg._capi.GB_FUNC_RNEA, pg._capi.GB_FUNC_ABA):
            pg._capi.check(L.gb_model_set_layout(tasks[2 * k][0].dev.h, f, pg._capi.GB_INSTANCE_PER_WARP))
    outs = [o.cpu().numpy() for o in api.MultiBatch(tasks, precision).run()]
    d = lambda a: torch.from_numpy(a).cuda()  # noqa: E731
    for k, (model, q, v, x) in enumerate(ref):
        om = OracleModel(model)
        assert rel_err(outs[2 * k], om.aba(q, v, 10.0 * x, LOCAL)) < tol
        assert rel_err(outs[2 * k + 1], om.rnea(q, v, x)) < tol
        data = tasks[2 * k][0]
        single = [pg.aba(model, data, d(q), d(v), d(10.0 * x)).cpu().numpy(), pg.rnea(model, data, d(q), d(v), d(x)).cpu().numpy()]
        for a, b in zip(single, outs[2 * k : 2 * k + 2]):
            if precision == "fp64":
                assert np.array_equal(a, b)
            else:
                assert rel_err(b, a) < 1e-6


def test_multi_graph_replay():
    tasks, ref = _tasks("mixed", 2000, 7)
    mb = api.MultiBatch(tasks, "mixed", 64)
    first = [o.clone() for o in mb.run()]
    for o in mb.outputs:
        o.zero_()
    mb.capture()
    for o in mb.outputs:
        o.zero_()
    mb.replay()
    for a, b in zip(first, mb.outputs):
        assert bool((a == b).all())


def test_autotuner_keeps_results(tmp_path, monkeypatch):
    import torch

    monkeypatch.setattr(autotune, "CACHE_PATH", str(tmp_path / "tune.json"))
    model = sm.humanoid32(1)
    data = pg.createData(model, "mixed")
    q, v, x = (torch.from_numpy(a).cuda() for a in sm.random_inputs(model, 3000, 2))
    before = pg.aba(model, data, q, v, x).clone()
    res = autotune.tune(model, data, functions=("aba", "rnea"), batch=4096)
    assert set(res) == {"aba", "rnea"} and all(t in autotune.CANDIDATES or t in (autotune.WARP, autotune.BRANCH) for t, _ in res.values())
    assert torch.equal(pg.aba(model, data, q, v, x), before)
    again = autotune.tune(model, data, functions=("aba", "rnea"), batch=4096)  # served from the cache
    assert again == {k: (t, ms) for k, (t, ms) in res.items()}


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", ["manipulator6r", "humanoid32", "tree60ff", "chain100", "mixedtree24ff", "zyxtree16"])
def test_warp_layout_matches_thread_layout_bitwise(name, precision):
    """The warp-per-instance and lane-per-branch layouts (gb_model_set_layout) give
    the thread layout's results for RNEA, ABA, nonLinearEffects and gravity -- the same bits in FP64,
    FP32 rounding in the mixed kernels (the compiler may contract their FP32
    multiply-adds differently in the two kernels) -- and matches the oracle."""
    import torch

    from util import MODELS

    model = MODELS[name]()
    q, v, x = sm.random_inputs(model, 203, 9)
    d = lambda a: torch.from_numpy(a).cuda()  # noqa: E731
    data = pg.createData(model, precision)
    L = pg._capi.lib()
    outs = {}
    layouts = (pg._capi.GB_INSTANCE_PER_THREAD, pg._capi.GB_INSTANCE_PER_WARP, pg._capi.GB_INSTANCE_PER_BRANCH)
    for layout in layouts:
        for f in (pg._capi.GB_FUNC_RNEA, pg._capi.GB_FUNC_ABA):
            pg._capi.check(L.gb_model_set_layout(data.dev.h, f, layout))
        outs[layout] = [
            pg.rnea(model, data, d(q), d(v), d(x)).cpu().numpy(),
            pg.aba(model, data, d(q), d(v), d(10.0 * x)).cpu().numpy(),
            pg.nonLinearEffects(model, data, d(q), d(v)).cpu().numpy(),
            pg.computeGeneralizedGravity(model, data, d(q)).cpu().numpy(),
        ]
    for layout in layouts[1:]:
        for k, (a, b) in enumerate(zip(outs[layouts[0]], outs[layout])):
            if precision == "fp64":
                assert np.array_equal(a, b), (layout, k)
            else:
                assert rel_err(b, a) < 1e-6, (layout, k, rel_err(b, a))
    om = OracleModel(model)
    tol = (1e-10 if name == "chain100" else FP64_TOL) if precision == "fp64" else mixed_tol(name)
    if precision == "fp64" or name != "chain100":
        for layout in layouts[1:]:
            assert rel_err(outs[layout][0], om.rnea(q, v, x)) < tol
            assert rel_err(outs[layout][1], om.aba(q, v, 10.0 * x, LOCAL)) < tol


def test_layout_setting_errors():
    model = sm.manipulator6r(0)
    data = pg.createData(model)
    L = pg._capi.lib()
    assert L.gb_model_set_layout(data.dev.h, pg._capi.GB_FUNC_CRBA, pg._capi.GB_INSTANCE_PER_WARP) == pg._capi.GB_ERR_UNSUPPORTED
    assert L.gb_model_set_layout(data.dev.h, pg._capi.GB_FUNC_RNEA, 5) == pg._capi.GB_ERR_INVALID_ARGUMENT
    assert L.gb_model_set_layout(data.dev.h, pg._capi.GB_FUNC_ABA, pg._capi.GB_INSTANCE_PER_8_LANES) == pg._capi.GB_ERR_UNSUPPORTED
    assert L.gb_model_set_layout(data.dev.h, pg._capi.GB_FUNC_CRBA, pg._capi.GB_INSTANCE_PER_BRANCH) == pg._capi.GB_ERR_UNSUPPORTED
    assert L.gb_model_set_layout(data.dev.h, pg._capi.GB_FUNC_ABA_DERIVATIVES, pg._capi.GB_INSTANCE_PER_4_LANES) == pg._capi.GB_OK


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", ["manipulator6r", "humanoid32", "tree60ff", "chain100", "mixedtree24ff", "zyxtree16"])
def test_team_layouts_aba_derivatives(name, precision):
    """The ABA derivatives with a team of 4, 8 or 32 lanes per configuration
    (the lanes split the column loops of the sweeps) give the thread layout's
    ddq_dq, ddq_dv, Minv, ddq, VJP and computeMinverse: the same bits in FP64,
    FP32 rounding in the mixed kernels."""
    import torch

    from util import MODELS

    model = MODELS[name]()
    q, v, x = sm.random_inputs(model, 77, 4)
    tau = 10.0 * x
    g = np.random.default_rng(2).standard_normal((77, model.nv))
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    data = pg.createData(model, precision)
    L = pg._capi.lib()
    outs = {}
    layouts = (pg._capi.GB_INSTANCE_PER_THREAD, pg._capi.GB_INSTANCE_PER_4_LANES, pg._capi.GB_INSTANCE_PER_8_LANES,
               pg._capi.GB_INSTANCE_PER_WARP)
    for layout in layouts:
        pg._capi.check(L.gb_model_set_layout(data.dev.h, pg._capi.GB_FUNC_ABA_DERIVATIVES, layout))
        res = [t.cpu().numpy() for t in pg.computeABADerivatives(model, data, d(q), d(v), d(tau))]
        res.append(data.ddq.cpu().numpy())
        res += [t.cpu().numpy() for t in pg.abaDerivativesVJP(model, data, d(q), d(v), d(tau), d(g))]
        res.append(pg.computeMinverse(model, data, d(q)).cpu().numpy())
        outs[layout] = res
    for layout in layouts[1:]:
        for k, (a, b) in enumerate(zip(outs[layouts[0]], outs[layout])):
            if precision == "fp64":
                assert np.array_equal(a, b), (layout, k)
            else:
                assert rel_err(b, a) < 1e-6, (layout, k, rel_err(b, a))
    if precision == "fp64" or name != "chain100":
        ddq_o, dq_o, dv_o, Minv_o = OracleModel(model).aba_derivatives(q, v, tau)
        tol = (1e-10 if name == "chain100" else FP64_TOL) if precision == "fp64" else mixed_tol(name)
        w = outs[pg._capi.GB_INSTANCE_PER_WARP]
        assert rel_err(w[0], dq_o) < tol and rel_err(w[1], dv_o) < tol and rel_err(w[2], Minv_o) < tol
        assert rel_err(w[3], ddq_o) < tol


def test_autotuner_chooses_a_derivative_layout(tmp_path, monkeypatch):
    """tune() also times the lane-team layouts of the ABA derivatives; whatever it
    picks, the FP64 results keep their bits."""
    import torch

    from util import MODELS

    monkeypatch.setattr(autotune, "CACHE_PATH", str(tmp_path / "tune.json"))
    model = MODELS["chain100"]()
    data = pg.createData(model)
    q, v, x = (torch.from_numpy(a).cuda() for a in sm.random_inputs(model, 256, 3))
    before = [t.clone() for t in pg.computeABADerivatives(model, data, q, v, x)]
    res = autotune.tune(model, data, functions=("aba_derivatives",), batch=256, use_cache=False)
    setting = res["aba_derivatives"][0]
    assert setting in autotune.CANDIDATES or setting in (autotune.LANES4, autotune.LANES8, autotune.WARP)
    for a, b in zip(before, pg.computeABADerivatives(model, data, q, v, x)):
        assert torch.equal(a, b)


def test_three_dof_joints_run_per_thread(tmp_path, monkeypatch):
    """Models with spherical or planar joints run one configuration per thread: the lane
    layouts are refused, the autotuner keeps to CTA sizes, and gb_batch_multi runs them next to
    other trees (the three-dof steps compiled in for that launch only)."""
    import torch

    from util import MODELS

    monkeypatch.setattr(autotune, "CACHE_PATH", str(tmp_path / "tune.json"))
    model = MODELS["multidoftree16"]()
    data = pg.createData(model)
    L = pg._capi.lib()
    for f, layout in ((pg._capi.GB_FUNC_RNEA, pg._capi.GB_INSTANCE_PER_WARP),
                      (pg._capi.GB_FUNC_ABA, pg._capi.GB_INSTANCE_PER_BRANCH),
                      (pg._capi.GB_FUNC_ABA_DERIVATIVES, pg._capi.GB_INSTANCE_PER_4_LANES)):
        assert L.gb_model_set_layout(data.dev.h, f, layout) == pg._capi.GB_ERR_UNSUPPORTED
    res = autotune.tune(model, data, batch=256, use_cache=False)
    assert all(s in autotune.CANDIDATES for s, _ in res.values())
    q, v, x = (torch.from_numpy(a).cuda() for a in sm.random_inputs(model, 64, 5))
    ddq_o = OracleModel(model).aba(*(t.cpu().numpy() for t in (q, v, x)), LOCAL)
    assert rel_err(pg.aba(model, data, q, v, x).cpu().numpy(), ddq_o) < FP64_TOL
    other = sm.random_tree(12, False, 312)
    d2 = pg.createData(other)
    q2, v2, x2 = (torch.from_numpy(a).cuda() for a in sm.random_inputs(other, 96, 6))
    outs = api.MultiBatch([(data, "aba", q, v, x), (d2, "rnea", q2, v2, x2), (data, "rnea", q, v, x)]).run()
    outs = [o.cpu().numpy() for o in outs]
    assert rel_err(outs[0], ddq_o) < FP64_TOL
    assert rel_err(outs[1], OracleModel(other).rnea(*(t.cpu().numpy() for t in (q2, v2, x2)))) < FP64_TOL
    assert rel_err(outs[2], OracleModel(model).rnea(*(t.cpu().numpy() for t in (q, v, x)))) < FP64_TOL


@pytest.mark.parametrize("precision,tol", [("fp64", FP64_TOL), ("mixed", 1e-4)])
def test_multi_with_spherical_zyx_joints(precision, tol):
    """A launch over the ZYX tree (its joints run as revolute chains) and the humanoid: every task
    against the oracle and the single-model call."""
    import torch

    tasks, ref = [], []
    for k, model in enumerate((sm.zyx_tree(), sm.humanoid32(1))):
        q, v, x = sm.random_inputs(model, 300 + 100 * k, 30 + k)
        data = pg.createData(model, precision)
        d = lambda a: torch.from_numpy(a).cuda()  # noqa: E731
        tasks += [(data, "aba", d(q), d(v), d(10.0 * x)), (data, "rnea", d(q), d(v), d(x))]
        ref.append((model, data, q, v, x))
    outs = [o.cpu().numpy() for o in api.MultiBatch(tasks, precision).run()]
    for k, (model, data, q, v, x) in enumerate(ref):
        om = OracleModel(model)
        assert rel_err(outs[2 * k], om.aba(q, v, 10.0 * x, LOCAL)) < tol
        assert rel_err(outs[2 * k + 1], om.rnea(q, v, x)) < tol
        single = pg.aba(model, data, torch.from_numpy(q).cuda(), torch.from_numpy(v).cuda(),
                        torch.from_numpy(10.0 * x).cuda())
        assert np.array_equal(single.cpu().numpy(), outs[2 * k])
