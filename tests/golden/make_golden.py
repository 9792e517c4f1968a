"""Generate the golden fixtures of tests/golden from the CPU oracle.

The reference's own tests carry no numerical golden vectors (they pin results
by identities), so these fixtures freeze the oracle's FP64 outputs on seeded
inputs: every test platform (x86 development host, Arm GPU host) must reproduce
them, and the GPU kernels are compared with them.  Each fixture also stores the
long-double oracle run of the vector outputs and, for every matrix output, the
largest difference between the FP64 and the long-double runs.

    python tests/golden/make_golden.py        # rewrites tests/golden/*.npz
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle.oracle import LOCAL, WORLD, OracleModel  # noqa: E402
from pinocchio_gb300 import sample_models as sm  # noqa: E402

# (fixture name, model factory, batch, input seed)
CASES = [
    ("manipulator6r", lambda: sm.manipulator6r(0), 16, 101),
    ("humanoid32", lambda: sm.humanoid32(1), 3, 102),
    ("tree12", lambda: sm.random_tree(12, False, 3), 8, 103),
]


def make(name, factory, B, seed):
    model = factory()
    om = OracleModel(model)
    q, v, x = sm.random_inputs(model, B, seed)
    tau = 10.0 * x
    out = {"q": q, "v": v, "a": x, "tau_in": tau}
    full = {}
    for prec, tag in ((0, ""), (1, "_ld")):
        out["rnea" + tag] = om.rnea(q, v, x, prec=prec)
        out["aba_local" + tag] = om.aba(q, v, tau, LOCAL, prec=prec)
        out["aba_world" + tag] = om.aba(q, v, tau, WORLD, prec=prec)
        M = om.crba(q, LOCAL, prec=prec)
        out["crba" + tag] = M
        U, D = om.cholesky(M, prec=prec)
        out["chol_U" + tag], out["chol_D" + tag] = U, D
        t, dq, dv, Mr = om.rnea_derivatives(q, v, x, prec=prec)
        out["rneaD_tau" + tag], out["rneaD_dq" + tag], out["rneaD_dv" + tag], out["rneaD_M" + tag] = t, dq, dv, Mr
        dd, Aq, Av, Mi = om.aba_derivatives(q, v, tau, prec=prec)
        out["abaD_ddq" + tag], out["abaD_dq" + tag], out["abaD_dv" + tag], out["abaD_Minv" + tag] = dd, Aq, Av, Mi
        out["integrate" + tag] = om.integrate(q, v, prec=prec)
        if tag:  # keep the long-double matrices only as a difference bound
            for k in [k for k in out if k.endswith("_ld") and out[k].ndim == 3]:
                full[k] = out.pop(k)
    for k, m in full.items():
        out["maxdiff_" + k[:-3]] = np.array(np.abs(out[k[:-3]] - m).max())
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    return out


def main():
    for name, factory, B, seed in CASES:
        make(name, factory, B, seed)
        print("wrote", name)


if __name__ == "__main__":
    main()
