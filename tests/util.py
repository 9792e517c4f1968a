"""Shared helpers of the tests: error metrics and the workload models."""
import numpy as np

from pinocchio_gb300 import sample_models as sm


def rel_err(x, ref):
    """Max over instances of ||x - ref|| / ||ref|| (Frobenius per instance), the
    isApprox-style relative error the reference's tests use."""
    x = np.asarray(x, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    x = x.reshape(x.shape[0], -1)
    ref = ref.reshape(ref.shape[0], -1)
    den = np.maximum(np.linalg.norm(ref, axis=1), 1e-300)
    return float((np.linalg.norm(x - ref, axis=1) / den).max())


def med_rel_err(x, ref):
    x = np.asarray(x, dtype=np.float64).reshape(len(x), -1)
    ref = np.asarray(ref, dtype=np.float64).reshape(len(ref), -1)
    return float(np.median(np.linalg.norm(x - ref, axis=1) / np.maximum(np.linalg.norm(ref, axis=1), 1e-300)))


MODELS = {
    "manipulator6r": lambda: sm.manipulator6r(0),
    "humanoid32": lambda: sm.humanoid32(1),
    "tree7": lambda: sm.random_tree(7, False, 307),
    "tree12": lambda: sm.random_tree(12, False, 312),
    "tree32ff": lambda: sm.random_tree(32, True, 332),
    "tree60ff": lambda: sm.random_tree(60, True, 360),
    "chain100": lambda: sm.chain(100, 4),
    "mixedtree12": lambda: sm.mixed_tree(12, False, 6),
    "mixedtree24ff": lambda: sm.mixed_tree(24, True, 5),
    "unaligned14": lambda: sm.unaligned_tree(14, False, 7),
    "unaligned20ff": lambda: sm.unaligned_tree(20, True, 8),
    "translationtree14": lambda: sm.translation_tree(9),
    "multidoftree16": lambda: sm.multidof_tree(10),
    "unbounded15ff": lambda: sm.unbounded_tree(15, True, 11),
    "zyxtree16": lambda: sm.zyx_tree(12),
}
# models the oracle covers beyond the kernels (none at present)
ORACLE_ONLY_MODELS = {}
# FP64 parity bar of the batched kernels against the FP64 oracle (relative, per instance)
FP64_TOL = 1e-12
# mixed-precision bar (max relative error against the FP64 oracle)
MIXED_TOL = 1e-5
# the models that cover joint types (prismatic, unaligned axes) rather than a benchmark
# workload: their FP64 results meet FP64_TOL; their mixed-precision error, which scales with
# each random model's conditioning, is held to 1e-4
JOINT_TYPE_MODELS = ("mixedtree12", "mixedtree24ff", "unaligned14", "unaligned20ff", "translationtree14",
                     "multidoftree16", "unbounded15ff", "zyxtree16")


def mixed_tol(name: str) -> float:
    return 1e-4 if name in JOINT_TYPE_MODELS else MIXED_TOL
