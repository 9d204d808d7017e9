"""Generate tests/golden/kronmult_golden.npz from the REFERENCE's own CPU build.

Runs hipdac-lab/kronmult's OpenMP templates (compiled from its source tree into
oracle/_ref/libkron_ref.so by oracle/Makefile) on the input generators of the
reference tests, single-threaded so that overlapping-Y sums are reproducible,
and stores inputs that are not closed-form plus every output.

    python tests/golden/make_golden.py      # needs the reference source tree

Cases (reference test they follow):
  batched   d=1..6, n=1..4, batch 1 and 3, ramp inputs, Y starts at zero
            (test_kronmult6_batched.cpp:148-175, 515-529)
  pbatched  same, batch 4, every Y pointer aliases Y(:,1)
            (test_kronmult6_pbatched.cpp, use_overlap_in_Y)
  xbatched  d=1..6, n=1..4, batch 1 and 4, lda = n+3, overlapping Y, FP64 and FP32
            (test_kronmult6_xbatched.cpp:106-110, 253-312)
  vbatched  d=1..6, rectangular m_l x n_l in 1..3, batch 3, seeded uniform inputs,
            FP64 and FP32 (test_kronmult6_vbatched.cpp; its own table never
            exercises m != n, so these shapes are new)
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))

from oracle import pyoracle as po  # noqa: E402

OUT = os.path.join(HERE, "kronmult_golden.npz")


def vb_shapes(seed):
    rng = np.random.default_rng(seed)
    out = []
    for d in range(1, 7):
        for t in range(2):
            m = rng.integers(1, 4, size=d)
            n = rng.integers(1, 4, size=d)
            out.append((d, m.astype(np.int32), n.astype(np.int32)))
    return out


def main():
    po.build(ref=True)
    if po.ref_lib() is None:
        raise SystemExit("oracle/_ref/libkron_ref.so was not built: reference tree absent")
    po.set_threads(1)
    data = {}
    for d in range(1, 7):
        for n in (1, 2, 3, 4):
            N = n ** d
            for batch in (1, 3):
                A = po.ramp_a(n, d, batch)
                X = po.ramp_x(N, batch)
                Y = np.zeros_like(X)
                W = np.zeros_like(X)
                po.batched(d, n, A, X.copy(), Y, W, batch, lib="ref")
                data[f"batched_d{d}_n{n}_b{batch}"] = Y
            batch = 4
            A = po.ramp_a(n, d, batch)
            X = po.ramp_x(N, batch)
            Y = np.zeros((batch, N))
            W = np.zeros((batch, N))
            po.pbatched(d, n, A, X.copy(), [b * N for b in range(batch)], Y, [0] * batch, W,
                        [b * N for b in range(batch)], lib="ref")
            data[f"pbatched_d{d}_n{n}_b{batch}"] = Y[0].copy()
            for T, tag in ((np.float64, "f64"), (np.float32, "f32")):
                for batch in (1, 4):
                    lda = n + 3
                    A = po.ramp_a(n, d, batch, lda=lda, dtype=T)
                    X = po.ramp_x(N, batch, dtype=T)
                    aoff = [[(b * d + l) * n * lda for l in range(d)] for b in range(batch)]
                    Y = np.zeros(N, dtype=T)
                    W = np.zeros((max(batch, 2), N), dtype=T)
                    po.xbatched(d, n, A, aoff, lda, X.copy(), [b * N for b in range(batch)], Y,
                                [0] * batch, W, [b * N for b in range(W.shape[0])], lib="ref")
                    data[f"xbatched_{tag}_d{d}_n{n}_b{batch}"] = Y
    for ci, (d, m, nn) in enumerate(vb_shapes(1234)):
        batch = 3
        rng = np.random.default_rng(100 + ci)
        fsz = [int(m[l] * nn[l]) for l in range(d)]
        Nx, Ny = int(np.prod(nn)), int(np.prod(m))
        A = rng.uniform(-1, 1, size=batch * sum(fsz))
        X = rng.uniform(-1, 1, size=(batch, Nx))
        Y0 = rng.uniform(-1, 1, size=(batch, Ny))
        data[f"vbatched_c{ci}_m"] = m
        data[f"vbatched_c{ci}_n"] = nn
        data[f"vbatched_c{ci}_A"] = A
        data[f"vbatched_c{ci}_X"] = X
        data[f"vbatched_c{ci}_Y0"] = Y0
        aoff, o = [], 0
        for b in range(batch):
            row = []
            for l in range(d):
                row.append(o)
                o += fsz[l]
            aoff.append(row)
        for T, tag in ((np.float64, "f64"), (np.float32, "f32")):
            Y = Y0.astype(T).copy()
            W = np.zeros(2 * po.size_xw(d, m, nn) * 2, dtype=T)
            po.vbatched(d, m, nn, A.astype(T), aoff, X.astype(T), [b * Nx for b in range(batch)],
                        Y, [b * Ny for b in range(batch)], W, lib="ref")
            data[f"vbatched_{tag}_c{ci}"] = Y
    np.savez_compressed(OUT, **data)
    print(f"wrote {OUT}: {len(data)} arrays, {os.path.getsize(OUT)} bytes")


if __name__ == "__main__":
    main()
