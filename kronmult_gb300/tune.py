"""Autotuner: measure every kernel family for each (form, d, n) on the
current GPU and write the committed tuning table ``tune_table.json``.

    python -m kronmult_gb300.tune [--out kronmult_gb300/tune_table.json] [--quick]

For each form (FP64 plain, FP64 split, FP32) and square shape (d = 1..6,
n = 2..8 and 16 where an entry has at most 2^18 elements) the batched entry
point is timed with each engine (per-mode kernels, register-tiled kernels,
small-entry kernels) on about 256 MiB of X; the fastest engine is recorded.
FP32 rows time FP32 fused multiply-add (form PLAIN), the kernels they tune.  For FP64 the
automatic form is the faster of plain and split.  ``build.py`` compiles the
table into ``csrc/kmx_tune_table.h``; the library consults it whenever the
caller leaves ``engine`` / ``form`` on their automatic settings.
"""
from __future__ import annotations

import argparse
import datetime
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
TABLE = os.path.join(HERE, "tune_table.json")

FORM_CODES = {"plain": 1, "split": 2, "f32": 3}
ENGINE_CODES = {"per_mode": 1, "tiled": 2, "small": 3}


def shapes():
    for d in range(1, 7):
        for n in (2, 3, 4, 5, 6, 7, 8, 16):
            if n ** d <= 1 << 18:
                yield d, n


def time_one(kmx, torch, d, n, form, engine, target_bytes, reps):
    N = n ** d
    dt = torch.float32 if form == "f32" else torch.float64
    esz = 4 if form == "f32" else 8
    batch = max(1, min(1 << 20, target_bytes // (N * esz)))
    A = torch.randn((batch, d, n, n), dtype=dt, device="cuda") / 2
    X = torch.randn((batch, N), dtype=dt, device="cuda")
    Y = torch.zeros_like(X)
    W = torch.zeros_like(X) if N * esz > 200 * 1024 else None
    f = "plain" if form == "f32" else form  # FP32 rows time the FMA kernels they tune

    def call():
        kmx.kronmult_batched(d, n, A, X, Y, W, batch, form=f, engine=engine)

    call()
    call()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        call()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    return batch * 2.0 * d * n ** (d + 1) / (ms * 1e-3) / 1e9


def has_tile(d, n):
    return (3 <= d <= 6 and 2 <= n <= 8) or (d == 3 and n == 16)


def has_small(d, n):
    return d <= 3 and n ** d <= 256


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=TABLE)
    ap.add_argument("--quick", action="store_true", help="smaller batches, fewer repetitions")
    args = ap.parse_args(argv)
    sys.path.insert(0, os.path.dirname(HERE))
    import torch

    import kronmult_gb300 as kmx

    target = (64 << 20) if args.quick else (256 << 20)
    reps = 3 if args.quick else 5
    rows, auto = [], []
    best_by_form = {}
    for form in ("plain", "split", "f32"):
        for d, n in shapes():
            if form == "split" and not (2 <= n <= 8 or n == 16):
                continue
            res = {}
            for engine in ("per_mode", "tiled", "small"):
                if engine == "tiled" and not has_tile(d, n):
                    continue
                if engine == "small" and not has_small(d, n):
                    continue
                try:
                    res[engine] = time_one(kmx, torch, d, n, form, engine, target, reps)
                except Exception as ex:  # a shape this engine cannot run
                    res[engine] = None
                    print(f"skip {form} d={d} n={n} {engine}: {ex}", file=sys.stderr)
            ok = {k: v for k, v in res.items() if v}
            if not ok:
                continue
            best = max(ok, key=ok.get)
            rows.append({"form": form, "d": d, "n": n, "engine": best,
                         "gflops": {k: round(v, 1) for k, v in ok.items()}})
            best_by_form[(form, d, n)] = ok[best]
            print(form, d, n, best, {k: round(v, 1) for k, v in ok.items()}, flush=True)
    for d, n in shapes():
        p = best_by_form.get(("plain", d, n))
        s = best_by_form.get(("split", d, n))
        if p and s:
            auto.append({"d": d, "n": n, "form": "split" if s > p else "plain"})
    table = {
        "device": torch.cuda.get_device_name(0),
        "measured": datetime.datetime.now(datetime.timezone.utc).isoformat(timespec="seconds"),
        "method": "batched entry point, ~256 MiB of X per call, CUDA events, best engine",
        "rows": rows,
        "auto_form_f64": auto,
    }
    with open(args.out, "w") as f:
        json.dump(table, f, indent=1)
    print(f"wrote {args.out}: {len(rows)} rows")


def header_from_table(path: str = TABLE) -> str:
    """C++ header with the table's choices (generated by build.py)."""
    rows, auto = [], []
    if os.path.exists(path):
        with open(path) as f:
            t = json.load(f)
        rows = t.get("rows", [])
        auto = t.get("auto_form_f64", [])
    lines = [
        "// Generated by kronmult_gb300/build.py from tune_table.json -- do not edit.",
        "#pragma once",
        "namespace kmx {",
        "struct TuneRow { int form; int d; int n; int engine; };",
        "struct AutoRow { int d; int n; int form; };",
        f"constexpr int kTuneRows = {len(rows)};",
        f"constexpr int kAutoRows = {len(auto)};",
        "static const TuneRow kTuneTable[] = {",
    ]
    for r in rows:
        lines.append(f"  {{{FORM_CODES[r['form']]}, {r['d']}, {r['n']}, {ENGINE_CODES[r['engine']]}}},")
    if not rows:
        lines.append("  {0, 0, 0, 0},")
    lines.append("};")
    lines.append("static const AutoRow kAutoTable[] = {")
    for a in auto:
        lines.append(f"  {{{a['d']}, {a['n']}, {1 if a['form'] == 'plain' else 2}}},")
    if not auto:
        lines.append("  {0, 0, 0},")
    lines.append("};")
    lines.append("}  // namespace kmx")
    return "\n".join(lines) + "\n"


if __name__ == "__main__":
    main()
