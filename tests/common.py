"""Shared helpers of the parity tests."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "kronmult_golden.npz")


def golden():
    return np.load(GOLDEN)


def blockwise_rel_err(y, yref):
    """max over blocks of ||y - yref||_2 / ||yref||_2 (rows are blocks)."""
    y = np.atleast_2d(np.asarray(y, dtype=np.float64))
    yref = np.atleast_2d(np.asarray(yref, dtype=np.float64))
    # scale each block by its largest magnitude so the norms cannot overflow
    s = np.max(np.abs(yref), axis=1, keepdims=True)
    s = np.where(s == 0, 1.0, s)
    num = np.linalg.norm((y - yref) / s, axis=1)
    den = np.linalg.norm(yref / s, axis=1)
    den = np.where(den == 0, 1.0, den)
    return float(np.max(num / den))


def ref_test_err(y, yref):
    """The reference tests' metric: max over elements of min(abs, rel) with
    rel = abs / (1 + max(|y|, |yref|)) (test_kronmult6_xbatched.cpp:612-626)."""
    y = np.asarray(y, dtype=np.float64).ravel()
    yref = np.asarray(yref, dtype=np.float64).ravel()
    a = np.abs(y - yref)
    r = a / (1 + np.maximum(np.abs(y), np.abs(yref)))
    return float(min(a.max(initial=0), r.max(initial=0)))


def vb_cases():
    """(case index, d) of the vbatched golden cases."""
    return [(ci, ci // 2 + 1) for ci in range(12)]
