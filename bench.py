"""Benchmark of the batched dynamics hot path on one GB300 (sm_103a).

Workload (the headline configuration): the 32-dof synthetic humanoid
(free-flyer + 2 torso + 4 limbs x 6 revolute joints, nq 33, nv 32), batch
65536 configurations per GPU (q: random unit quaternion, base N(0,1), joints
U[-pi, pi]; v ~ N(0,1); tau ~ N(0,10)).  One step = ABA (ddq) + ABA
derivatives (ddq_dq, ddq_dv, Minv) of the whole batch.  ``value`` is
configurations per second of the mixed-precision kernels (FP32 sweeps, FP64
Schur complement), inputs resident in HBM; the plain FP64 kernels are timed
beside it (``fp64``) and both are checked against the FP64 oracle on a
sample.  ``e2e`` is the same step through the public API with the inputs in
pinned host memory and the outputs copied back to host memory every step.
Beside the headline the line carries (unless --no-extra) the evals/s of every
batched function per precision (``functions``), the heterogeneous
single-launch batch over four trees (``heterogeneous``) and the differentiable
rollout on the 100-link chain (``rollout``).

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--batch B] [--impl ours|reference]
Under torchrun (N > 1) every rank runs an independent replica on its own GPU
(the instances shard with no exchange step): ``value`` sums all ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ABA/RNEA/derivative evals/s, 1 GB300: mixed vs FP64 plain at ≤1e-5 rel err"
PEAKS_PATH = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=100)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--batch", type=int, default=65536)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-extra", action="store_true",
                   help="skip the per-function, heterogeneous-batch and rollout measurements")
    p.add_argument("--only", choices=["rnea", "aba", "crba", "rnea_derivatives", "aba_derivatives",
                                      "constraint_dynamics", "constraint_dynamics_derivatives", "contact_cholesky"],
                   default=None,
                   help="time one batched call on the humanoid (for profiling), print its timing and exit")
    p.add_argument("--precision", choices=["fp64", "mixed"], default="mixed")
    return p.parse_args()


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist

        import torch

        torch.cuda.set_device(local)
        dist.init_process_group("nccl" if args.impl == "ours" else "gloo")
        pg = dist
    return world, rank, local, pg


# ------------------------------------------------------------------------------------------
# clocks sampled during the timed region
# ------------------------------------------------------------------------------------------
class ClockSampler:
    FIELDS = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(
                    ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits"],
                    capture_output=True, text=True, timeout=5,
                ).stdout.strip()
                if out:
                    self.samples.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *exc):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if len(s) > 5 + k and s[5 + k].lower() == "active"})
        return {
            "sm_mhz": float(np.median(sm)) if sm else None,
            "sm_max_mhz": max(mx) if mx else None,
            "reasons": reasons,
            "samples": len(self.samples),
        }


# ------------------------------------------------------------------------------------------
# reference arm: the reference's CPU algorithm (the oracle port) on all host cores
# ------------------------------------------------------------------------------------------
def _omp_env():
    """Thread binding of the OpenMP batch drivers (OMP_PROC_BIND=true, as the CPU baseline of
    rneaInParallel / abaInParallel is specified); set before the oracle's OpenMP runtime loads."""
    os.environ.setdefault("OMP_PROC_BIND", "true")
    return {"OMP_PROC_BIND": os.environ.get("OMP_PROC_BIND"), "OMP_PLACES": os.environ.get("OMP_PLACES")}


def _cpu_model_name():
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu part")):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return None


def _cpu_step(om, q, v, tau, outs, nthreads):
    """One CPU step of the headline workload: ABA (WORLD, as abaInParallel) + ABA derivatives."""
    from oracle.oracle import WORLD

    om.aba(q, v, tau, WORLD, nthreads=nthreads, out=outs[0])
    om.aba_derivatives(q, v, tau, nthreads=nthreads, out=outs[1:])


def _cpu_outs(B, nv):
    outs = [np.empty((B, nv)), np.empty((B, nv)), np.empty((B, nv, nv)), np.empty((B, nv, nv)), np.empty((B, nv, nv))]
    for o in outs:
        o.fill(0.0)  # touch the pages once, outside any timed region
    return outs


def cpu_single_thread(om, model, sample=1024, reps=3):
    """ABA + ABA derivatives on one thread, on a bounded sample (evals/s)."""
    from pinocchio_gb300 import sample_models as sm

    q, v, x = sm.random_inputs(model, sample, 3)
    tau = 10.0 * x
    outs = _cpu_outs(sample, model.nv)
    _cpu_step(om, q[:64], v[:64], tau[:64], [o[:64] for o in outs], 1)
    t = []
    for _ in range(reps):
        t0 = time.perf_counter()
        _cpu_step(om, q, v, tau, outs, 1)
        t.append(time.perf_counter() - t0)
    return {"value": sample / float(np.median(t)), "unit": "evals/s", "cores": 1,
            "sample": f"{sample} configurations x {reps} repetitions, ABA(WORLD) + ABA derivatives, FP64, 1 thread"}


def cpu_rnea_c0(cores, B=4096):
    """rneaInParallel on the 6R manipulator (batch 4096, FP64): all cores and one thread (evals/s)."""
    from oracle.oracle import OracleModel
    from pinocchio_gb300 import sample_models as sm

    model = sm.manipulator6r(0)
    om = OracleModel(model)
    q, v, a = sm.random_inputs(model, B, 0)
    out = np.zeros((B, model.nv))
    res = {"workload": f"manipulator6r nv=6 RNEA, batch {B}, FP64"}
    for name, nt, reps in (("all_cores", cores, 200), ("single_thread", 1, 20)):
        om.rnea(q, v, a, nthreads=nt, out=out)
        t = []
        for _ in range(reps):
            t0 = time.perf_counter()
            om.rnea(q, v, a, nthreads=nt, out=out)
            t.append(time.perf_counter() - t0)
        res[name] = {"value": B / float(np.median(t)), "unit": "evals/s", "cores": nt,
                     "ms_per_call": 1e3 * float(np.median(t))}
    return res


def run_reference(args, world, rank):
    if rank != 0:
        return
    env = _omp_env()
    from oracle.oracle import OracleModel
    from pinocchio_gb300 import sample_models as sm

    model = sm.humanoid32(1)
    om = OracleModel(model)
    cores = os.cpu_count() or 1
    B = args.batch
    q, v, x = sm.random_inputs(model, B, 0)
    tau = 10.0 * x
    outs = _cpu_outs(B, model.nv)
    for _ in range(max(1, args.warmup)):
        _cpu_step(om, q, v, tau, outs, cores)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        _cpu_step(om, q, v, tau, outs, cores)
        times.append(time.perf_counter() - t0)
    t = float(np.median(times))
    rate = B / t
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": rate,
        "unit": "evals/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * t,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded humanoid32 model and inputs)",
        "config": {
            "workload": f"humanoid32 nv=32 ABA(WORLD)+computeABADerivatives, batch {B}",
            "batch": B,
            "parallelism": "openmp static over instances (rneaInParallel/abaInParallel structure)",
        },
        "cpu_baseline": {
            "value": rate,
            "unit": "evals/s",
            "cores": cores,
            "kind": "port",
            "sample": f"the whole batch of {B} configurations every step (median of {args.steps} steps), ABA(WORLD) + "
                      f"ABA derivatives, FP64, {cores} OpenMP threads, outputs preallocated",
            "cpu": _cpu_model_name(),
            "omp": env,
            "single_thread": cpu_single_thread(om, model),
        },
        "rnea_in_parallel_c0": cpu_rnea_c0(cores),
        "e2e": {"value": rate, "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------------------------------
# our arm
# ------------------------------------------------------------------------------------------
def fp64_peak_tflops(torch):
    """Measured FP64 throughput of this GPU: a cuBLAS DGEMM (4096^3), best of 5."""
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    for _ in range(2):
        torch.mm(a, b)
    torch.cuda.synchronize()
    best = 1e30
    for _ in range(5):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        torch.mm(a, b)
        e.record()
        torch.cuda.synchronize()
        best = min(best, s.elapsed_time(e) / 1e3)
    return 2.0 * n**3 / best / 1e12


def _time_call(torch, fn, reps=5, warmup=2):
    """Milliseconds per call of fn (CUDA events on the current stream, after warm-up)."""
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record()
    for _ in range(reps):
        fn()
    e.record()
    torch.cuda.synchronize()
    return s.elapsed_time(e) / reps


def _per_config_rel_err(got, ref):
    """max and median over configurations of ||got - ref|| / ||ref|| (one row per configuration)."""
    n = ref.shape[0]
    g, r = got.reshape(n, -1), ref.reshape(n, -1)
    e = np.linalg.norm(g - r, axis=1) / np.maximum(np.linalg.norm(r, axis=1), 1e-300)
    return float(e.max()), float(np.median(e))


def _function_reference(om, fname, q, v, x, f, J, g, desc=None):
    """The FP64 oracle's outputs of one benchmarked function, in the order the API returns them."""
    from oracle.oracle import symmetrize_upper

    t, z = 10.0 * x, np.zeros_like(v)
    if fname == "crba_cholesky":
        Mu = om.crba(q)
        return (symmetrize_upper(Mu),) + tuple(om.cholesky(Mu))
    if fname == "rnea_derivatives":
        _, dq, dv, M = om.rnea_derivatives(q, v, x)
        return dq, dv, symmetrize_upper(M)
    return {
        "rnea": lambda: (om.rnea(q, v, x),),
        "aba": lambda: (om.aba(q, v, t),),
        "crba": lambda: (symmetrize_upper(om.crba(q)),),
        "aba_derivatives": lambda: om.aba_derivatives(q, v, t)[1:],
        "compute_minverse": lambda: (om.aba_derivatives(q, v, t)[3],),
        "nonlinear_effects": lambda: (om.rnea(q, v, z),),
        "generalized_gravity": lambda: (om.rnea(q, z, z),),
        "forward_kinematics": lambda: om.forward_kinematics(q, v, x),
        "joint_jacobians": lambda: (np.swapaxes(om.joint_jacobians(q), 1, 2),),
        "rnea_fext": lambda: (om.rnea(q, v, x, fext=f),),
        "aba_fext": lambda: (om.aba(q, v, t, fext=f),),
        "aba_derivatives_fext": lambda: om.aba_derivatives(q, v, t, fext=f)[1:],
        "forward_dynamics_12rows": lambda: (om.forward_dynamics(q, v, t, J, g)[0],),
        "constraint_dynamics_18rows": lambda: (om.constraint_dynamics(q, v, t, desc)[0],),
        "constraint_dynamics_derivatives_18rows": lambda: om.constraint_dynamics_derivatives(q, v, t, desc)[2:8],
        "contact_cholesky_18rows": lambda: tuple(om.contact_cholesky(q, desc).values()),
    }[fname]()


def _contact_cholesky(pg, model, data, contacts, q):
    """ContactCholeskyDecomposition.compute at q and its six accessors."""
    chol = pg.ContactCholeskyDecomposition(model, contacts)
    chol.compute(model, data, contacts, None, 0.0, q=q)
    return (chol.matrix(), chol.inverse(), chol.getInverseOperationalSpaceInertiaMatrix(),
            chol.getOperationalSpaceInertiaMatrix(), chol.getInverseMassMatrix(), chol.getJMinv())


def humanoid_contacts(pg, model):
    """Four contacts of the humanoid's limbs to world anchors: frame contacts (LOCAL) on the two
    legs, point contacts (LOCAL_WORLD_ALIGNED) on the two arms -- 18 constraint rows."""
    rng = np.random.default_rng(17)
    par = set(model.parents[1:])
    leaves = [j for j in range(1, model.njoints) if j not in par]
    out = []
    for k, leaf in enumerate(leaves[:4]):
        R, _ = np.linalg.qr(rng.standard_normal((3, 3)))
        R *= np.sign(np.linalg.det(R))
        P = pg.SE3(R, 0.1 * rng.standard_normal(3))
        anchor = pg.SE3(np.eye(3), rng.standard_normal(3))
        if k < 2:
            out.append(pg.RigidConstraintModel(pg.CONTACT_6D, model, leaf, P, 0, anchor, pg.LOCAL))
        else:
            out.append(pg.RigidConstraintModel(pg.CONTACT_3D, model, leaf, P, 0, anchor, pg.LOCAL_WORLD_ALIGNED))
    return out


def measure_functions(torch, pg, sm):
    """evals/s of every batched function on the humanoid, per precision: RNEA / ABA /
    CRBA (+ tree Cholesky) / computeMinverse / nonLinearEffects / generalized gravity /
    forwardKinematics (q, v, a) / computeJointJacobians at batch 65536, the two derivative
    algorithms at batch 16384; RNEA, ABA and the ABA derivatives with external forces on
    every joint (the fext overloads) at the same batches; forwardDynamics with 12 constraint
    rows (two 6-D contacts) and constraintDynamics with four contacts (18 rows) at batch 65536, and
    constraintDynamics followed by computeConstraintDynamicsDerivatives and the contact Cholesky with
    its six accessors at batch 16384.  Each function's outputs are checked against the
    FP64 oracle on 256 configurations strided over its batch: the max and median over those
    configurations of the relative error of every output."""
    from oracle.oracle import OracleModel

    from pinocchio_gb300.constraints import stack_desc

    model = sm.humanoid32(1)
    om = OracleModel(model)
    contacts = humanoid_contacts(pg, model)
    desc = stack_desc(contacts)
    out = {}
    for prec in ("fp64", "mixed"):
        data = pg.createData(model, prec)
        res = {}
        for fname, B in (("rnea", 65536), ("aba", 65536), ("crba", 65536), ("crba_cholesky", 65536),
                         ("rnea_derivatives", 16384), ("aba_derivatives", 16384), ("compute_minverse", 65536),
                         ("nonlinear_effects", 65536), ("generalized_gravity", 65536),
                         ("forward_kinematics", 65536), ("joint_jacobians", 65536), ("rnea_fext", 65536),
                         ("aba_fext", 65536), ("aba_derivatives_fext", 16384), ("forward_dynamics_12rows", 65536),
                         ("constraint_dynamics_18rows", 65536), ("constraint_dynamics_derivatives_18rows", 16384),
                         ("contact_cholesky_18rows", 16384)):
            q, v, x = (torch.from_numpy(a).cuda() for a in sm.random_inputs(model, B, 11))
            f = torch.randn((B, model.njoints, 6), dtype=torch.float64, device="cuda")
            Jc = torch.randn((B, 12, model.nv), dtype=torch.float64, device="cuda") if fname.startswith("forward_dyn") else None
            gc = torch.randn((B, 12), dtype=torch.float64, device="cuda") if Jc is not None else None
            fn = {
                "rnea": lambda: pg.rnea(model, data, q, v, x),
                "aba": lambda: pg.aba(model, data, q, v, 10.0 * x),
                "crba": lambda: pg.crba(model, data, q),
                "crba_cholesky": lambda: pg.crbaCholesky(model, data, q),
                "rnea_derivatives": lambda: pg.computeRNEADerivatives(model, data, q, v, x),
                "aba_derivatives": lambda: pg.computeABADerivatives(model, data, q, v, 10.0 * x),
                "compute_minverse": lambda: pg.computeMinverse(model, data, q),
                "nonlinear_effects": lambda: pg.nonLinearEffects(model, data, q, v),
                "generalized_gravity": lambda: pg.computeGeneralizedGravity(model, data, q),
                "forward_kinematics": lambda: pg.forwardKinematics(model, data, q, v, x),
                "joint_jacobians": lambda: pg.computeJointJacobians(model, data, q),
                "rnea_fext": lambda: pg.rnea(model, data, q, v, x, f),
                "aba_fext": lambda: pg.aba(model, data, q, v, 10.0 * x, f),
                "aba_derivatives_fext": lambda: pg.computeABADerivatives(model, data, q, v, 10.0 * x, f),
                "forward_dynamics_12rows": lambda: pg.forwardDynamics(model, data, q, v, 10.0 * x, Jc, gc),
                "constraint_dynamics_18rows": lambda: pg.constraintDynamics(model, data, q, v, 10.0 * x, contacts),
                "constraint_dynamics_derivatives_18rows": lambda: (
                    pg.constraintDynamics(model, data, q, v, 10.0 * x, contacts),
                    pg.computeConstraintDynamicsDerivatives(model, data, contacts))[1],
                "contact_cholesky_18rows": lambda: _contact_cholesky(pg, model, data, contacts, q),
            }[fname]
            ms = _time_call(torch, fn)
            res[fname] = {"batch": B, "ms": ms, "evals_per_s": B / ms * 1e3}
            got = fn()
            got = [t for t in (got if isinstance(got, tuple) else (got,)) if t is not None]
            idx = torch.from_numpy(np.unique(np.linspace(0, B - 1, 256).astype(np.int64))).cuda()
            host = lambda t: None if t is None else t[idx].cpu().numpy()  # noqa: E731
            ref = _function_reference(om, fname, host(q), host(v), host(x), host(f), host(Jc), host(gc), desc)
            errs = [_per_config_rel_err(host(a), b) for a, b in zip(got, ref)]
            res[fname]["max_rel_err"] = max(e[0] for e in errs)
            res[fname]["median_rel_err"] = max(e[1] for e in errs)
            del q, v, x, f, Jc, gc, got
        out[prec] = res
    return out


def measure_heterogeneous(torch, pg, sm, total=100000):
    """RNEA + ABA over the four seeded trees (nv 7 / 12 / 32 FF / 60 FF, instances 40/30/20/10 %)
    in one persistent launch captured in a CUDA graph; the autotuner picks the layout per tree (on
    the tree's own batch) and then the launch's threads per block."""
    from pinocchio_gb300 import api, autotune

    models = sm.heterogeneous_trees(3)
    out = {"instances": total, "trees_nv": [m.nv for m in models], "split": [0.4, 0.3, 0.2, 0.1]}
    for prec in ("fp64", "mixed"):
        tasks, layouts = [], []
        for k, (model, share) in enumerate(zip(models, (0.4, 0.3, 0.2, 0.1))):
            B = int(total * share)
            q, v, x = (torch.from_numpy(a).cuda() for a in sm.random_inputs(model, B, 20 + k))
            data = pg.createData(model, prec)
            tuned = autotune.tune(model, data, functions=("rnea", "aba"), batch=B, use_cache=False)
            layouts.append({f: (t if isinstance(t, str) else "thread") for f, (t, _) in tuned.items()})
            tasks.append((data, "aba", q, v, 10.0 * x))
            tasks.append((data, "rnea", q, v, x))
        tpb, _ = autotune.tune_multi(tasks, prec)
        mb = api.MultiBatch(tasks, prec, tpb)
        mb.capture()
        ms = _time_call(torch, mb.replay, reps=20, warmup=3)
        evals = 2 * sum(int(total * s) for s in (0.4, 0.3, 0.2, 0.1))
        out[prec] = {"ms_per_launch": ms, "evals_per_s": evals / ms * 1e3, "threads_per_block": tpb,
                     "evals_per_launch": evals, "layouts": layouts}
    return out


def measure_rollout(torch, pg, sm, B=8192, T=64, n=100):
    """Differentiable rollout: T semi-implicit Euler steps (dt 1e-3) of ABA on the n-link chain,
    batch B, loss ||q_T||^2, backward through the ABA-derivative kernels with checkpoints every 8 steps."""
    from oracle.oracle import OracleModel, rollout_with_gradients
    from pinocchio_gb300 import autograd

    model = sm.chain(n, 4, (0.1, 1.0))
    om = OracleModel(model)
    rng = np.random.default_rng(5)
    d = lambda a: torch.tensor(a, dtype=torch.float64, device="cuda")  # noqa: E731
    q0 = d(rng.uniform(-np.pi, np.pi, (B, n)))
    v0 = d(0.1 * rng.standard_normal((B, n)))
    taus = d(rng.standard_normal((T, B, n)))
    out = {"batch": B, "steps": T, "nv": n, "checkpoint_every": 8}
    from pinocchio_gb300 import autotune

    for prec in ("fp64", "mixed"):
        data = pg.createData(model, prec)
        # layout per function for this model and batch (the deep chain favours a warp per trajectory)
        tuned = autotune.tune(model, data, functions=("aba", "aba_derivatives"), batch=B, use_cache=False)

        def once():
            q0.grad = v0.grad = taus.grad = None
            for t in (q0, v0, taus):
                t.requires_grad_()
            qT, _ = autograd.rollout(model, data, q0, v0, taus, dt=1e-3, checkpoint_every=8)
            (qT**2).sum().backward()

        ms = _time_call(torch, once, reps=2, warmup=1)
        out[prec] = {"ms_per_rollout": ms, "trajectories_per_s": B / ms * 1e3,
                     "aba_evals_per_s": B * T / ms * 1e3,
                     "layouts": {f: (t if isinstance(t, str) else f"thread x{t}") for f, (t, _) in tuned.items()}}
        # accuracy: q_T and the three gradients of 16 trajectories strided over the batch against the
        # FP64 oracle rollout (adjoint recursion over the oracle's ABA derivatives)
        once()
        qT, _ = autograd.rollout(model, data, q0.detach(), v0.detach(), taus.detach(), dt=1e-3, checkpoint_every=8)
        idx = np.unique(np.linspace(0, B - 1, 16).astype(np.int64))
        ti = torch.from_numpy(idx).cuda()
        got = [qT[ti], q0.grad[ti], v0.grad[ti], taus.grad[:, ti].transpose(0, 1)]
        qn, vn, tn = (t.detach().cpu().numpy() for t in (q0[ti], v0[ti], taus[:, ti]))
        qT_o, _, gq_o, gv_o, gt_o = rollout_with_gradients(om, qn, vn, tn, 1e-3)
        refs = [qT_o, gq_o, gv_o, gt_o.transpose(1, 0, 2)]
        out[prec]["accuracy_vs_fp64_oracle"] = {
            k: dict(zip(("max", "median"), _per_config_rel_err(a.detach().cpu().numpy(), b)))
            for k, a, b in zip(("q_T", "grad_q0", "grad_v0", "grad_taus"), got, refs)}
        out[prec]["accuracy_vs_fp64_oracle"]["sample"] = f"{len(idx)} trajectories strided over the batch of {B}"
    return out


def measure_e2e(torch, pg, model, host, B, args, dist, world):
    """The headline step through the public API (``pg.aba`` + ``pg.computeABADerivatives``) with
    the inputs in pinned host memory and every output copied back to pinned host memory, each
    step.  Outputs are double-buffered: step k's device-to-host copies run on a copy stream
    while step k + 1's kernels run on the compute stream (two output sets, preallocated and
    passed as ``out=``, on the device and on the host).  The compute runs on its own stream:
    on the legacy default stream the concurrent device-to-host copies fell to ~20 GB/s after a
    few steps (measured), on a non-default stream they keep the link's rate.  The transfers go
    through the library's ``copyAsync`` (torch's ``copy_`` with pinned memory stalled the
    concurrent copies for tens of milliseconds every ~40 steps, measured).  Beside it, the copy
    floor: the same bytes moved by plain pinned copies alone."""
    nq, nv = model.nq, model.nv
    h2d = B * (nq + 2 * nv) * 8
    d2h = B * (nv + 3 * nv * nv) * 8
    hq = [torch.from_numpy(q).pin_memory() for q, _, _ in host[:2]]
    hv = [torch.from_numpy(v).pin_memory() for _, v, _ in host[:2]]
    ht = [torch.from_numpy(10.0 * x).pin_memory() for _, _, x in host[:2]]
    shapes = {"ddq": (B, nv), "ddq_dq": (B, nv, nv), "ddq_dv": (B, nv, nv), "Minv": (B, nv, nv)}
    ho = [{k: torch.empty(sh, dtype=torch.float64).pin_memory() for k, sh in shapes.items()} for _ in range(2)]
    d = pg.createData(model, "mixed")
    from pinocchio_gb300 import autotune

    autotune.tune(model, d, functions=("aba", "aba_derivatives"), batch=B, use_cache=False)
    comp = torch.cuda.Stream()
    copy = torch.cuda.Stream()
    din = [tuple(torch.empty(t.shape, dtype=torch.float64, device="cuda") for t in (hq[0], hv[0], ht[0]))
           for _ in range(2)]
    dout = [(torch.empty((B, nv), dtype=torch.float64, device="cuda"),)
            + tuple(torch.empty((B, nv, nv), dtype=torch.float64, device="cuda") for _ in range(3))
            + (torch.empty((B, nv), dtype=torch.float64, device="cuda"),) for _ in range(2)]
    done = [torch.cuda.Event() for _ in range(2)]  # the step's kernels finished (outputs ready)
    freed = [torch.cuda.Event() for _ in range(2)]  # the step's outputs are on the host
    keep = [None, None]

    def e2e_step(k):
        s = k % 2
        q, v, t = din[s]
        ddq, dq, dv, Mi, ddq_d = dout[s]
        with torch.cuda.stream(comp):
            comp.wait_event(freed[s])  # the inputs / outputs of step k - 2 are no longer in use
            for dst, src in ((q, hq[s]), (v, hv[s]), (t, ht[s])):
                pg.copyAsync(dst, src)
            pg.aba(model, d, q, v, t, out=ddq)
            pg.computeABADerivatives(model, d, q, v, t, out=(dq, dv, Mi, ddq_d))
            done[s].record(comp)
        with torch.cuda.stream(copy):
            copy.wait_event(done[s])
            for name, src in (("ddq", ddq), ("ddq_dq", dq), ("ddq_dv", dv), ("Minv", Mi)):
                pg.copyAsync(ho[s][name], src)
            freed[s].record(copy)
        keep[s] = (ddq, dq, dv, Mi)

    for k in range(args.warmup):
        e2e_step(k)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for k in range(args.steps):
        e2e_step(k)
    torch.cuda.synchronize()
    t_e2e = (time.perf_counter() - t0) / args.steps
    if dist:
        t = torch.tensor([t_e2e], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_e2e = float(t.item())
    # a host read of the result of the last step (what a caller consumes)
    checksum = float(ho[(args.steps - 1) % 2]["ddq"][0, 0])
    # copy floor: the step's bytes moved by pinned copies alone (no kernels), the outputs split over
    # 1, 2 or 4 streams (each its own copy engine queue); the fastest split, timed with events
    src = [keep[0][1], keep[0][2], keep[0][3], keep[0][0]]
    dst = [ho[0]["ddq_dq"], ho[0]["ddq_dv"], ho[0]["Minv"], ho[0]["ddq"]]
    floor_ms = {}
    for nstreams in (1, 2, 4):
        streams = [torch.cuda.Stream() for _ in range(nstreams)]
        pieces = []  # (dst, src) chunks of about equal size, round-robin over the streams
        for a, b in zip(dst, src):
            fa, fb = a.view(-1), b.view(-1)
            n = fa.numel()
            for k in range(nstreams):
                lo, hi = k * n // nstreams, (k + 1) * n // nstreams
                pieces.append((fa[lo:hi], fb[lo:hi]))
        for a, b in zip(din[0], (hq[0], hv[0], ht[0])):
            pieces.append((a, b))
        times = []
        for rep in range(4):
            torch.cuda.synchronize()
            s0, e0 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s0.record(streams[0])
            ends = []
            for k, st in enumerate(streams):
                st.wait_event(s0)
                with torch.cuda.stream(st):
                    for j in range(k, len(pieces), nstreams):
                        pg.copyAsync(pieces[j][0], pieces[j][1])
                ev = torch.cuda.Event()
                ev.record(st)
                ends.append(ev)
            for ev in ends:
                streams[0].wait_event(ev)
            e0.record(streams[0])
            torch.cuda.synchronize()
            if rep:
                times.append(s0.elapsed_time(e0))
        floor_ms[nstreams] = min(times)
    best = min(floor_ms, key=floor_ms.get)
    ms_copy = floor_ms[best]
    del keep
    floor = world * B / (ms_copy * 1e-3)
    return {"value": world * B / t_e2e, "unit": "evals/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
            "ms_per_step": 1e3 * t_e2e,
            "copy_floor": {"value": floor, "unit": "evals/s", "ms_per_step": ms_copy,
                           "d2h_gbs": d2h / (ms_copy * 1e-3) / 1e9, "streams": best,
                           "ms_by_streams": floor_ms,
                           "note": "the same H2D + D2H bytes as pinned copies alone (no kernels), best of 1/2/4 streams"},
            "fraction_of_copy_floor": (world * B / t_e2e) / floor,
            "overlap": "outputs double-buffered: step k's D2H copies on a copy stream overlap step k+1's kernels",
            "host_checksum": checksum}


def dtau_structural_nonzeros(model):
    """Entries of dtau_dq that can be non-zero: row k of column c with k's joint an ancestor of (or)
    c's joint or in its subtree -- the rows the -Minv * dtau product kernels loop over."""
    par = model.parents
    jv = [j for j, n in enumerate(model.nvs) for _ in range(n)]

    def anc(j):
        out = set()
        while j > 0:
            out.add(j)
            j = par[j]
        return out

    A = [anc(j) for j in range(model.njoints)]
    return sum(1 for c in jv for k in jv if k in A[c] or c in A[k])


def measure_soa(torch, L, _capi, data, dev, B, nq, nv, PREC, sp, P, reps=10):
    """The headline step with GB_LAYOUT_SOA inputs and outputs (element k of every configuration
    contiguous), both precisions, CUDA events: ms per step."""
    q, v, tau = (t.t().contiguous() for t in dev[0])  # (n, B): SOA
    o = {"ddq": torch.empty((nv, B), dtype=torch.float64, device="cuda"),
         "dq": torch.empty((nv * nv, B), dtype=torch.float64, device="cuda"),
         "dv": torch.empty((nv * nv, B), dtype=torch.float64, device="cuda"),
         "Mi": torch.empty((nv * nv, B), dtype=torch.float64, device="cuda"),
         "ddq2": torch.empty((nv, B), dtype=torch.float64, device="cuda")}
    res = {}
    for prec in ("mixed", "fp64"):
        h = data[prec].dev.h

        def fn():
            _capi.check(L.gb_aba(h, PREC[prec], _capi.GB_LOCAL, _capi.GB_LAYOUT_SOA, B, P(q), P(v), P(tau),
                                 P(o["ddq"]), sp))
            _capi.check(L.gb_aba_derivatives(h, PREC[prec], _capi.GB_LAYOUT_SOA, B, P(q), P(v), P(tau), P(o["dq"]),
                                             P(o["dv"]), P(o["Mi"]), P(o["ddq2"]), sp))

        ms = _time_call(torch, fn, reps=reps, warmup=2)
        res[prec] = {"ms_per_step": ms, "evals_per_s": B / ms * 1e3}
    res["note"] = "same step with SOA inputs/outputs (coalesced loads of q, v, tau); the headline uses the reference's layout"
    return res


def measure_c0(torch, pg, sm, B=4096):
    """rneaInParallel's workload (6R manipulator, batch 4096): the batched RNEA kernel on device-resident
    inputs (CUDA events) per precision, and rneaInParallel itself through the host-array entry point
    (wall clock, copies and synchronisation included)."""
    model = sm.manipulator6r(0)
    q, v, a = sm.random_inputs(model, B, 0)
    qd, vd, ad = (torch.from_numpy(x).cuda() for x in (q, v, a))
    out = {"workload": f"manipulator6r nv=6 RNEA, batch {B}"}
    for prec in ("fp64", "mixed"):
        data = pg.createData(model, prec)
        ms = _time_call(torch, lambda: pg.rnea(model, data, qd, vd, ad), reps=50, warmup=5)
        out[prec] = {"ms": ms, "evals_per_s": B / ms * 1e3}
    pool = pg.ModelPool(model, 4)
    qc, vc, ac = (np.asfortranarray(x.T) for x in (q, v, a))
    tau = np.empty((model.nv, B), order="F")
    for _ in range(5):
        pg.rneaInParallel(4, pool, qc, vc, ac, tau)
    t = []
    for _ in range(50):
        t0 = time.perf_counter()
        pg.rneaInParallel(4, pool, qc, vc, ac, tau)
        t.append(time.perf_counter() - t0)
    out["rneaInParallel_host_arrays_fp64"] = {"ms": 1e3 * float(np.median(t)), "evals_per_s": B / float(np.median(t))}
    return out


def run_ours(args, world, rank, local, dist):
    import torch

    import pinocchio_gb300 as pg
    from pinocchio_gb300 import _capi
    from pinocchio_gb300 import sample_models as sm

    torch.cuda.set_device(local)
    B = args.batch
    model = sm.humanoid32(1)
    nq, nv = model.nq, model.nv
    nrot = 4  # input copies rotated across steps: 4 x 51 MB > 129 MB L2
    host = [sm.random_inputs(model, B, 100 * rank + r) for r in range(nrot)]
    dev = [(torch.from_numpy(q).cuda(), torch.from_numpy(v).cuda(), torch.from_numpy(10.0 * x).cuda()) for q, v, x in host]
    stream = torch.cuda.current_stream()
    L = _capi.lib()
    import ctypes

    sp = ctypes.c_void_p(stream.cuda_stream)
    outs = {
        "ddq": torch.empty((B, nv), dtype=torch.float64, device="cuda"),
        "ddq_dq": torch.empty((B, nv, nv), dtype=torch.float64, device="cuda"),
        "ddq_dv": torch.empty((B, nv, nv), dtype=torch.float64, device="cuda"),
        "Minv": torch.empty((B, nv, nv), dtype=torch.float64, device="cuda"),
        "ddq2": torch.empty((B, nv), dtype=torch.float64, device="cuda"),
    }
    data = {p: pg.createData(model, p) for p in ("fp64", "mixed")}
    # both precisions run in the launch settings the autotuner finds best at this batch, so that the
    # plain FP64 kernels are compared at their best
    from pinocchio_gb300 import autotune

    tuned = {p: autotune.tune(model, data[p], functions=("aba", "aba_derivatives"), batch=B, use_cache=False)
             for p in ("fp64", "mixed")}
    P = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    PREC = {"fp64": _capi.GB_FP64, "mixed": _capi.GB_MIXED}

    def step(prec, k):
        q, v, tau = dev[k % nrot]
        h = data[prec].dev.h
        _capi.check(L.gb_aba(h, PREC[prec], _capi.GB_LOCAL, _capi.GB_LAYOUT_INSTANCE, B, P(q), P(v), P(tau), P(outs["ddq"]), sp))
        _capi.check(
            L.gb_aba_derivatives(
                h, PREC[prec], _capi.GB_LAYOUT_INSTANCE, B, P(q), P(v), P(tau), P(outs["ddq_dq"]), P(outs["ddq_dv"]),
                P(outs["Minv"]), P(outs["ddq2"]), sp,
            )
        )

    def timed(prec, steps, warmup, sampler=None):
        for k in range(warmup):
            step(prec, k)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ctx = sampler if sampler is not None else _Null()
        with ctx:
            s.record(stream)
            for k in range(steps):
                step(prec, k)
            e.record(stream)
            torch.cuda.synchronize()
        ms = s.elapsed_time(e) / steps
        if dist:
            t = torch.tensor([ms], device="cuda")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms = float(t.item())
        return ms

    # per-kernel times (dominant kernel for the roofline) with events on the launching stream
    def kernel_times(prec, reps=5):
        q, v, tau = dev[0]
        h = data[prec].dev.h
        res = {}
        for name in ("aba", "aba_derivatives"):
            for _ in range(2):
                step(prec, 0)
            torch.cuda.synchronize()
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record(stream)
            for _ in range(reps):
                if name == "aba":
                    _capi.check(L.gb_aba(h, PREC[prec], _capi.GB_LOCAL, _capi.GB_LAYOUT_INSTANCE, B, P(q), P(v), P(tau), P(outs["ddq"]), sp))
                else:
                    _capi.check(
                        L.gb_aba_derivatives(
                            h, PREC[prec], _capi.GB_LAYOUT_INSTANCE, B, P(q), P(v), P(tau), P(outs["ddq_dq"]),
                            P(outs["ddq_dv"]), P(outs["Minv"]), P(outs["ddq2"]), sp,
                        )
                    )
            e.record(stream)
            torch.cuda.synchronize()
            res[name] = s.elapsed_time(e) / reps
        return res

    sampler = ClockSampler(local)  # samples clocks over both timed regions
    with sampler:
        ms_fp64 = timed("fp64", args.steps, args.warmup)
        ms_mixed = timed("mixed", args.steps, args.warmup)
    clocks = sampler.summary()
    kt_mixed = kernel_times("mixed")
    kt_fp64 = kernel_times("fp64")
    soa_ms = measure_soa(torch, L, _capi, data, dev, B, nq, nv, PREC, sp, P)

    # accuracy of the mixed and FP64 outputs against the FP64 oracle on a sample (rank 0)
    acc = {}
    if rank == 0:
        from oracle.oracle import OracleModel

        om = OracleModel(model)
        # a sample strided over the whole batch (first and last configuration included), so that every
        # part of the grid and of the persistent product pipeline is checked
        idx = np.unique(np.linspace(0, B - 1, min(B, 2048)).astype(np.int64))
        ns = len(idx)
        q, v, x = host[0]
        ref = om.aba_derivatives(q[idx], v[idx], 10.0 * x[idx])
        ref_aba = om.aba(q[idx], v[idx], 10.0 * x[idx])
        tidx = torch.from_numpy(idx).cuda()
        for prec in ("mixed", "fp64"):
            step(prec, 0)
            torch.cuda.synchronize()
            got = [outs["ddq2"][tidx], outs["ddq_dq"][tidx], outs["ddq_dv"][tidx], outs["Minv"][tidx], outs["ddq"][tidx]]
            ref_all = list(ref) + [ref_aba]
            errs = []
            for g, r in zip(got, ref_all):
                g = g.cpu().numpy().reshape(ns, -1)
                r = r.reshape(ns, -1)
                e = np.linalg.norm(g - r, axis=1) / np.linalg.norm(r, axis=1)
                errs.append((float(e.max()), float(np.median(e))))
            acc[prec] = {k: {"max": m, "median": md} for k, (m, md) in
                         zip(("ddq", "ddq_dq", "ddq_dv", "Minv", "aba_ddq"), errs)}
            acc[prec]["sample"] = f"{ns} configurations strided over the batch of {B} (first and last included)"
        # the mixed derivatives over every configuration of the batch (chunks of 8192)
        step("mixed", 0)
        torch.cuda.synchronize()
        errs = {k: [] for k in ("ddq_dq", "ddq_dv", "Minv")}
        for lo in range(0, B, 8192):
            hi = min(B, lo + 8192)
            ref = om.aba_derivatives(q[lo:hi], v[lo:hi], 10.0 * x[lo:hi])
            for k, g, r in (("ddq_dq", outs["ddq_dq"], ref[1]), ("ddq_dv", outs["ddq_dv"], ref[2]),
                            ("Minv", outs["Minv"], ref[3])):
                g = g[lo:hi].cpu().numpy().reshape(hi - lo, -1)
                r = r.reshape(hi - lo, -1)
                errs[k].append(np.linalg.norm(g - r, axis=1) / np.linalg.norm(r, axis=1))
        acc["mixed_full_batch"] = {k: {"max": float(np.concatenate(e).max()), "median": float(np.median(np.concatenate(e))),
                                       "p999": float(np.quantile(np.concatenate(e), 0.999))} for k, e in errs.items()}
        acc["mixed_full_batch"]["sample"] = f"all {B} configurations"

    # end to end through the public API: pinned host inputs -> device -> kernels -> pinned host outputs
    e2e = None
    if not args.no_e2e:
        e2e = measure_e2e(torch, pg, model, host, B, args, dist, world)

    if rank != 0:
        return
    # roofline of the dominant kernel call (mixed): HBM bytes it must move per launch
    peaks = {}
    if os.path.exists(PEAKS_PATH):
        peaks = json.load(open(PEAKS_PATH))
    hbm_peak = peaks.get("hbm_gbs")
    peak_src = "measured" if hbm_peak else "fallback"
    hbm_peak = hbm_peak or FALLBACK_HBM_GBS
    dom = max(kt_mixed, key=kt_mixed.get)
    alg_bytes = {
        "aba": B * (nq + 3 * nv) * 8,  # q, v, tau in; ddq out
        "aba_derivatives": B * (nq + 2 * nv + nv + 3 * nv * nv) * 8,  # q, v, tau in; ddq, ddq_dq, ddq_dv, Minv out
    }[dom]
    achieved = alg_bytes / (kt_mixed[dom] * 1e-3) / 1e9
    # DRAM bytes of one call (sum over its kernels) from an ncu capture, scaled to this batch
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath):
        t = json.load(open(tpath)).get(f"{dom}_mixed")
        if t:
            traffic = t["dram_bytes"] * B / t["batch"]
    # FLOPs per evaluation (humanoid32): the oracle's FLOP-counting scalar over the reference's passes
    # (+, -, *, / = 1 each), with the two dense -Minv * dtau products (4 nv^3) replaced by the products
    # the kernels execute: only the rows of dtau that can be non-zero (4 nv nnz)
    nnz = dtau_structural_nonzeros(model)
    flops_oracle = {"aba": 26417.0, "aba_derivatives": 214728.0}
    flops = {"aba": flops_oracle["aba"],
             "aba_derivatives": flops_oracle["aba_derivatives"] - 4.0 * nv**3 + 4.0 * nv * nnz}
    fp64_tf = fp64_peak_tflops(torch)
    value = world * B / (ms_mixed * 1e-3)
    value_fp64 = world * B / (ms_fp64 * 1e-3)
    line = {
        "metric": METRIC,
        "value": value,
        "unit": "evals/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_mixed,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32+f64 (mixed: FP32 sweeps, FP64 Schur complement / pivots / accumulation)",
        "data": "synthetic (seeded humanoid32 model and inputs)",
        "config": {
            "workload": f"humanoid32 nv=32 ABA + computeABADerivatives, batch {B} per GPU",
            "batch": B,
            "precision": "mixed",
            "parallelism": f"replicas x{world} (instances shard, no exchange step)",
            "l2": "inputs rotate over 4 copies (4 x 51 MB) and every step writes 1.6 GB of outputs (> 129 MB L2)",
            "launch_settings": {p: {f: (t if isinstance(t, str) else f"thread x{t}") for f, (t, _) in tuned[p].items()}
                                for p in tuned},
        },
        "fp64": {"value": value_fp64, "unit": "evals/s", "ms_per_step": ms_fp64},
        "mixed_over_fp64": value / value_fp64,
        "accuracy_vs_fp64_oracle": acc,
        "kernel_ms": {"mixed": kt_mixed, "fp64": kt_fp64},
        "roofline": {
            "bound": "hbm",
            "kernel": f"gb_{dom} (mixed; one call = {'1 kernel' if dom == 'aba' else '3 sweep kernels + 1 product kernel'})",
            "achieved": achieved,
            "peak": hbm_peak,
            "unit": "GB/s",
            "frac": achieved / hbm_peak,
            "peak_source": peak_src,
            "traffic": traffic,
            "algorithmic_bytes_per_launch": alg_bytes,
            "limiter": ("latency (mixed: few warps per SM at this batch, long-scoreboard stalls on workspace "
                        "loads, FP64 Schur complement in the first sweep); FP64 pipe (fp64 kernels)"),
            "fp64_pipe": {
                "fp64_kernel_tflops": flops[dom] * B / (kt_fp64[dom] * 1e-3) / 1e12,
                "measured_dgemm_tflops": fp64_tf,
                "frac": flops[dom] * B / (kt_fp64[dom] * 1e-3) / 1e12 / fp64_tf,
                "flops_per_eval": flops[dom],
                "dtau_structural_nonzeros": nnz,
                "note": "FP64 kernels: FLOPs the kernels execute (oracle-counted sweeps + the sparse products) / "
                        "kernel time vs a measured cuBLAS DGEMM",
            },
        },
        "clocks": clocks,
        # per step: gb_aba (1 kernel) + gb_aba_derivatives (3 sweep kernels + 1 product kernel)
        "gpu_launches": args.steps * (1 + 4),
        "e2e": e2e,
    }
    line["layout_soa"] = soa_ms
    if not args.no_extra:
        line["rnea_in_parallel_c0"] = measure_c0(torch, pg, sm)
        line["functions"] = measure_functions(torch, pg, sm)
        line["heterogeneous"] = measure_heterogeneous(torch, pg, sm)
        line["rollout"] = measure_rollout(torch, pg, sm)
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(model, args)
    print(json.dumps(line), flush=True)


def cpu_baseline(model, args):
    """The oracle port (FP64, OpenMP over instances) on this host's cores, bounded sample."""
    env = _omp_env()
    from oracle.oracle import OracleModel
    from pinocchio_gb300 import sample_models as sm

    om = OracleModel(model)
    cores = os.cpu_count() or 1
    sample = 8192
    q, v, x = sm.random_inputs(model, sample, 3)
    tau = 10.0 * x
    outs = _cpu_outs(sample, model.nv)
    _cpu_step(om, q, v, tau, outs, cores)
    t = []
    while len(t) < 3 or (sum(t) < 10.0 and len(t) < 50):
        t0 = time.perf_counter()
        _cpu_step(om, q, v, tau, outs, cores)
        t.append(time.perf_counter() - t0)
    return {
        "value": sample / float(np.median(t)),
        "unit": "evals/s",
        "cores": cores,
        "kind": "port",
        "sample": f"{sample} configurations x {len(t)} repetitions (median) of ABA(WORLD) + ABA derivatives, FP64, "
                  "outputs preallocated",
        "cpu": _cpu_model_name(),
        "omp": env,
        "single_thread": cpu_single_thread(om, model),
        "rnea_in_parallel_c0": cpu_rnea_c0(cores),
    }


class _Null:
    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False


def run_only(args):
    """Warm-up + timed repetitions of one batched call (used for ncu captures)."""
    import ctypes

    import torch

    import pinocchio_gb300 as pg
    from pinocchio_gb300 import sample_models as sm

    model = sm.humanoid32(1)
    B = args.batch
    q, v, x = sm.random_inputs(model, B, 0)
    qd, vd, xd = (torch.from_numpy(a).cuda() for a in (q, v, 10.0 * x))
    data = pg.createData(model, args.precision)
    contacts = humanoid_contacts(pg, model)
    fn = {
        "constraint_dynamics": lambda: pg.constraintDynamics(model, data, qd, vd, xd, contacts),
        "constraint_dynamics_derivatives": lambda: (pg.constraintDynamics(model, data, qd, vd, xd, contacts),
                                                    pg.computeConstraintDynamicsDerivatives(model, data, contacts)),
        "rnea": lambda: pg.rnea(model, data, qd, vd, xd),
        "aba": lambda: pg.aba(model, data, qd, vd, xd),
        "crba": lambda: pg.crba(model, data, qd),
        "rnea_derivatives": lambda: pg.computeRNEADerivatives(model, data, qd, vd, xd),
        "aba_derivatives": lambda: pg.computeABADerivatives(model, data, qd, vd, xd),
        "contact_cholesky": lambda: _contact_cholesky(pg, model, data, contacts, qd),
    }[args.only]
    for _ in range(args.warmup):
        fn()
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record()
    for _ in range(args.steps):
        fn()
    e.record()
    torch.cuda.synchronize()
    ms = s.elapsed_time(e) / max(1, args.steps)
    print(json.dumps({"only": args.only, "precision": args.precision, "batch": B, "ms": ms, "evals_per_s": B / ms * 1e3}))
    del ctypes


def main():
    args = parse()
    if args.only:
        run_only(args)
        return
    world, rank, local, dist = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local, dist)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
