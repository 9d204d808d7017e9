"""Autotuner: measure every kernel family and launch shape for each (form,
layout, d, n) on the current GPU and write the committed tuning table
``tune_table.json``.

    python -m kronmult_gb300.tune [--out kronmult_gb300/tune_table.json] [--quick]

For each form (FP64 plain, FP64 split, FP32), square shape (d = 1..6,
n = 2..8 and 16 where an entry has at most 2^18 elements) and layout
(``batched``: disjoint Y blocks, plain stores; ``pointer``: xbatched with
eight entries per Y block on average, atomic accumulation) it times, on about
128 MiB of X (at least 4 entries per SM where that fits in 3 GiB), every
engine (per-mode, register-tiled, small-entry kernels) with each of its
launch shapes:

* per-mode kernels: threads per entry group G in {default, 64, 128, 256, 512};
* register-tiled kernels: entry groups per CTA E in {default, 1}, and the
  grid sized for one CTA per SM instead of the occupancy limit;
* small-entry kernels: their fixed shape.

The fastest (engine, G, E, CTAs per SM) is recorded with every candidate's
GFLOP/s.  FP32 rows time FP32 fused multiply-add (form PLAIN), the kernels
they tune.  For FP64 the automatic form is the faster of plain and split on
the batched layout.  ``build.py`` compiles the table into
``csrc/kmx_tune_table.h``; the library consults it whenever the caller
leaves ``engine`` (and the launch shape) on their automatic settings.

What the table does not cover, because it is fixed at compile time: the
register-tiled kernels' group size (one first-phase tile per thread) and
phase order (chosen so that the first phase reads X and the last writes Y in
whole sectors), and their arithmetic policy (packed FP32 pairs for even n with
one tile per thread, scalar otherwise: measured per shape when the packed
kernels were introduced).
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
ENGINE_CODES = {"per_mode": 1, "tiled": 2, "small": 3, "lane": 6}
LAYOUT_CODES = {"batched": 0, "pointer": 1}
LAYOUTS = ("batched", "pointer")


def shapes():
    for d in range(1, 7):
        for n in (2, 3, 4, 5, 6, 7, 8, 16):
            if n ** d <= 1 << 18:
                yield d, n


def has_tile(d, n):
    return (3 <= d <= 6 and 2 <= n <= 8) or (d == 3 and n == 16)


def has_small(d, n):
    return d <= 3 and n ** d <= 256


def has_lane(d, n):
    """The lane engine (kmx_lane.cuh): one entry per thread for n^2 <= 16 and
    n^d <= 16, one group of n lanes per entry for d = 2 with n = 5..8, one
    group of n^(d-1) <= 32 lanes per entry for d >= 3."""
    return ((d <= 3 and n * n <= 16 and n ** d <= 16) or (d == 2 and 5 <= n <= 8) or
            (3 <= d <= 6 and n ** (d - 1) <= 32))


def split_allowed(d, n):
    """Whether the automatic FP64 form may be double-float: blocks of n >= 3
    with 8 or more elements.  On smaller blocks (n = 2, and d = 1 with n = 3)
    the guarded double-float form measured up to 4e-13 per block on cancelling
    entries, above the 1e-13 that plain FP64 holds."""
    return n >= 3 and n ** d >= 8


def candidates(d, n):
    """(engine, (group_threads, groups_per_cta, ctas_per_sm)) to time."""
    out = [("per_mode", (g, 0, 0)) for g in (0, 64, 128, 256, 512)]
    if has_tile(d, n):
        out += [("tiled", (0, 0, 0)), ("tiled", (0, 1, 0)), ("tiled", (0, 0, 1))]
    if has_small(d, n):
        out.append(("small", (0, 0, 0)))
    if has_lane(d, n):
        out.append(("lane", (0, 0, 0)))
    return out


def label(engine, launch):
    g, e, s = launch
    parts = [engine] + ([f"G{g}"] if g else []) + ([f"E{e}"] if e else []) + ([f"S{s}"] if s else [])
    return "/".join(parts)


class Case:
    """Device inputs of one (form, layout, d, n): about target_bytes of X."""

    def __init__(self, kmx, torch, d, n, form, layout, target_bytes):
        self.kmx, self.torch = kmx, torch
        self.d, self.n, self.layout = d, n, layout
        N = n ** d
        dt = torch.float32 if form == "f32" else torch.float64
        esz = 4 if form == "f32" else 8
        # at least 4 entries per SM (152 SMs) where three such batches fit in
        # 3 GiB, so that entries beyond one SM's shared memory fill the GPU
        b = max(1, min(1 << 20, target_bytes // (N * esz)))
        b = max(b, min(608, (3 << 30) // (3 * N * esz)))
        self.batch = b
        self.form = "plain" if form == "f32" else form  # FP32 rows time the FMA kernels
        self.A = torch.randn((b, d, n, n), dtype=dt, device="cuda") / 2
        self.X = torch.randn((b, N), dtype=dt, device="cuda")
        self.W = torch.zeros_like(self.X) if N * esz > 200 * 1024 else None
        self.dtype = dt
        if layout == "batched":
            self.Y = torch.zeros_like(self.X)
        else:
            ny = max(1, b // 8)
            self.Y = torch.zeros((ny, N), dtype=dt, device="cuda")
            idx = torch.arange(b, device="cuda", dtype=torch.int64)
            self.pA = kmx.pointer_array(self.A, (idx[:, None] * d + torch.arange(d, device="cuda"))
                                        .reshape(-1).cpu().numpy() * n * n)
            self.pX = kmx.pointer_array(self.X, idx.cpu().numpy() * N)
            self.pY = kmx.pointer_array(self.Y, (idx % ny).cpu().numpy() * N)
            self.pW = None
            if self.W is not None:
                self.pW = kmx.pointer_array(self.W, idx.cpu().numpy() * N)
        self.flops = b * 2.0 * d * n ** (d + 1)

    def call(self, engine, launch):
        k = self.kmx
        if self.layout == "batched":
            k.kronmult_batched(self.d, self.n, self.A, self.X, self.Y, self.W, self.batch,
                               form=self.form, engine=engine, launch=launch)
        else:
            k.kronmult_xbatched(self.d, self.n, self.pA, self.n, self.pX, self.pY, self.pW,
                                self.batch, dtype=self.dtype, form=self.form, engine=engine,
                                launch=launch)

    def gflops(self, engine, launch, reps):
        torch = self.torch
        self.call(engine, launch)
        self.call(engine, launch)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            self.call(engine, launch)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        return self.flops / (ms * 1e-3) / 1e9


def time_one(kmx, torch, d, n, form, engine, target_bytes, reps, layout="batched",
             launch=(0, 0, 0)):
    """GFLOP/s of one (form, engine, launch shape) on one layout."""
    return Case(kmx, torch, d, n, form, layout, target_bytes).gflops(engine, launch, reps)


def auto_forms(best_by):
    """The automatic FP64 form per shape: the faster of plain and double-float
    on the batched layout (best_by[(form, layout, d, n)] = GFLOP/s), plain
    where split_allowed says no."""
    auto = []
    for d, n in shapes():
        p = best_by.get(("plain", "batched", d, n))
        s = best_by.get(("split", "batched", d, n))
        if p and s:
            auto.append({"d": d, "n": n,
                         "form": "split" if s > p and split_allowed(d, n) else "plain"})
    return auto


def build_table(rows, auto, device, method, now, only=frozenset(), old=None):
    """The table a run writes.  A partial run (only: the re-tuned (d, n)
    shapes) keeps the other shapes' rows and automatic forms from the old
    table, sorted in the table's order, keeps the full run's date and appends
    its own shapes and date to the "retuned" record."""
    table = {"device": device, "measured": now, "method": method, "rows": rows,
             "auto_form_f64": auto}
    if only:
        old = old or {}
        kept_rows = [r for r in old.get("rows", []) if (r["d"], r["n"]) not in only]
        kept_auto = [a for a in old.get("auto_form_f64", []) if (a["d"], a["n"]) not in only]
        key = lambda r: (list(FORM_CODES).index(r["form"]), r["d"], r["n"],
                         LAYOUTS.index(r.get("layout", "batched")))
        table["rows"] = sorted(kept_rows + rows, key=key)
        table["auto_form_f64"] = sorted(kept_auto + auto, key=lambda a: (a["d"], a["n"]))
        table["measured"] = old.get("measured", now)
        runs = old.get("retuned", [])
        runs = [runs] if isinstance(runs, dict) else list(runs)
        runs.append({"shapes": [f"{d}-{n}" for d, n in sorted(only)], "measured": now})
        table["retuned"] = runs
    return table


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=TABLE)
    ap.add_argument("--quick", action="store_true", help="smaller batches, fewer repetitions")
    ap.add_argument("--shapes", default="",
                    help="comma-separated d-n shapes to tune (default: every shape); the rows "
                         "and AUTO choices of the other shapes are kept from --out")
    args = ap.parse_args(argv)
    sys.path.insert(0, os.path.dirname(HERE))
    import torch

    import kronmult_gb300 as kmx

    target = (32 << 20) if args.quick else (128 << 20)
    reps = 3 if args.quick else 5
    only = {tuple(int(v) for v in t.split("-")) for t in args.shapes.split(",") if t}
    old = None
    if only and os.path.exists(args.out):
        with open(args.out) as f:
            old = json.load(f)
    rows, best_by = [], {}
    for form in ("plain", "split", "f32"):
        for d, n in shapes():
            if only and (d, n) not in only:
                continue
            if form == "split" and not (2 <= n <= 8 or n == 16):
                continue
            for layout in LAYOUTS:
                case = Case(kmx, torch, d, n, form, layout, target)
                res = {}
                for engine, launch in candidates(d, n):
                    try:
                        res[(engine, launch)] = case.gflops(engine, launch, reps)
                    except Exception as ex:  # a shape this engine cannot run
                        print(f"skip {form} {layout} d={d} n={n} {label(engine, launch)}: {ex}",
                              file=sys.stderr)
                del case
                if not res:
                    continue
                (engine, launch), g = max(res.items(), key=lambda kv: kv[1])
                rows.append({"form": form, "layout": layout, "d": d, "n": n, "engine": engine,
                             "group_threads": launch[0], "groups_per_cta": launch[1],
                             "ctas_per_sm": launch[2], "gflops": round(g, 1),
                             "candidates": {label(*k): round(v, 1) for k, v in res.items()}})
                best_by[(form, layout, d, n)] = g
                print(form, layout, d, n, label(engine, launch), round(g, 1), flush=True)
    method = (f"batched and pointer (xbatched, 8 entries per Y block) layouts, "
              f"~{target >> 20} MiB of X per call, CUDA events, {reps} calls after 2; "
              "best engine and launch shape")
    now = datetime.datetime.now(datetime.timezone.utc).isoformat(timespec="seconds")
    table = build_table(rows, auto_forms(best_by), torch.cuda.get_device_name(0), method, now,
                        only, old)
    with open(args.out, "w") as f:
        json.dump(table, f, indent=1)
    print(f"wrote {args.out}: {len(table['rows'])} rows ({len(rows)} measured)")


def header_from_table(path: str = TABLE) -> str:
    """C++ header with the table's choices (generated by build.py).  Rows
    without a layout (older tables) apply to the batched layout; missing
    launch-shape fields are 0 (the built-in default)."""
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
        "struct TuneRow {",
        "  int form, layout, d, n, engine;",
        "  int group_threads, groups_per_cta, ctas_per_sm;",
        "};",
        "struct AutoRow { int d; int n; int form; };",
        f"constexpr int kTuneRows = {len(rows)};",
        f"constexpr int kAutoRows = {len(auto)};",
        "static const TuneRow kTuneTable[] = {",
    ]
    for r in rows:
        vals = [FORM_CODES[r["form"]], LAYOUT_CODES[r.get("layout", "batched")], r["d"], r["n"],
                ENGINE_CODES[r["engine"]], int(r.get("group_threads", 0)),
                int(r.get("groups_per_cta", 0)), int(r.get("ctas_per_sm", 0))]
        lines.append("  {" + ", ".join(str(v) for v in vals) + "},")
    if not rows:
        lines.append("  {0, 0, 0, 0, 0, 0, 0, 0},")
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
