"""Generate tests/golden/kgemm_golden.npz from the REFERENCE's own CPU build.

Runs hipdac-lab/kronmult's kgemm_nn_batched / kgemm_nt_batched templates
(compiled from its source tree into oracle/_ref/libkron_ref.so by
oracle/Makefile) on the closed-form inputs of its tests
(test_kgemm_nn_batched.cpp:181-217: A(i,j) = 1+i+j*nrowA+ib,
B(i,j) = 1/(1+i+j*nrowB+ib), C = 1, alpha = 1.3) and stores every output C.
beta = 1.2 is the tests' value (test_kgemm_nn_batched.cpp:85-86); beta = 0
and beta = 1 cover the other two epilogue branches.  One more case per
transpose makes every entry accumulate into the same C (beta = 1).

    python tests/golden/make_kgemm_golden.py      # needs the reference source tree
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))

from oracle import pyoracle as po  # noqa: E402

OUT = os.path.join(HERE, "kgemm_golden.npz")
ALPHA = 1.3
SHAPES = [(1, 1, 1, 1), (8, 15, 22, 8), (29, 36, 57, 3), (64, 1, 65, 2), (4, 256, 4, 2),
          (5, 625, 5, 2), (256, 4, 4, 2), (65, 65, 65, 1)]
BETAS = [("b12", 1.2), ("b0", 0.0), ("b1", 1.0)]
ALL_BETAS = {(1, 1, 1, 1), (8, 15, 22, 8), (4, 256, 4, 2)}  # other shapes: beta = 1.2 only


def case_key(trans, tag, mm, nn, kk, batch, bname):
    return f"{trans}_{tag}_{mm}x{nn}x{kk}_b{batch}_{bname}"


def ld_b(trans, nn, kk):
    return kk if trans == "nn" else nn


def run(trans, T, mm, nn, kk, batch, beta, shared_c=False, lib="ref"):
    A, B, Cm = po.ramp_kgemm(trans, mm, nn, kk, batch, dtype=T)
    if shared_c:
        Cm = Cm[:1].copy()
    coff = [0] * batch if shared_c else [i * mm * nn for i in range(batch)]
    po.kgemm_batched(trans, mm, nn, kk, ALPHA, A.reshape(-1), [i * mm * kk for i in range(batch)],
                     [mm] * batch, B.reshape(-1), [i * B.shape[1] for i in range(batch)],
                     [ld_b(trans, nn, kk)] * batch, beta, Cm.reshape(-1), coff, [mm] * batch,
                     lib=lib)
    return Cm


def main():
    po.build(ref=True)
    if po.ref_lib() is None:
        raise SystemExit("oracle/_ref/libkron_ref.so was not built: reference tree absent")
    po.set_threads(1)
    data = {}
    for trans in ("nn", "nt"):
        for T, tag in ((np.float64, "f64"), (np.float32, "f32")):
            for (mm, nn, kk, batch) in SHAPES:
                for bname, beta in BETAS:
                    if bname != "b12" and (mm, nn, kk, batch) not in ALL_BETAS:
                        continue
                    data[case_key(trans, tag, mm, nn, kk, batch, bname)] = run(
                        trans, T, mm, nn, kk, batch, beta)
            data[f"{trans}_{tag}_shared_8x15x22_b8"] = run(trans, T, 8, 15, 22, 8, 1.0,
                                                           shared_c=True)
    np.savez_compressed(OUT, **data)
    print(f"wrote {OUT}: {len(data)} arrays")


if __name__ == "__main__":
    main()
