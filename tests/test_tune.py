"""CPU tests of the autotuner's committed table: well formed, covering every
tuned (form, layout, shape), each row's choice the fastest candidate it
measured, and compiled into the header the library reads."""
import json
import os
import re

from kronmult_gb300 import tune

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _table():
    with open(tune.TABLE) as f:
        return json.load(f)


def test_table_covers_every_tuned_shape_and_layout():
    t = _table()
    have = {(r["form"], r["layout"], r["d"], r["n"]) for r in t["rows"]}
    for form in ("plain", "split", "f32"):
        for d, n in tune.shapes():
            for layout in tune.LAYOUTS:
                assert (form, layout, d, n) in have, (form, layout, d, n)
    assert {(a["d"], a["n"]) for a in t["auto_form_f64"]} == set(tune.shapes())


def test_each_row_records_its_fastest_candidate():
    for r in _table()["rows"]:
        assert r["engine"] in tune.ENGINE_CODES
        assert r["layout"] in tune.LAYOUT_CODES
        launch = (r["group_threads"], r["groups_per_cta"], r["ctas_per_sm"])
        assert all(v >= 0 for v in launch)
        assert r["group_threads"] % 32 == 0 and r["group_threads"] <= 512
        cand = r["candidates"]
        key = tune.label(r["engine"], launch)
        assert key in cand, r
        assert cand[key] == max(cand.values()) == r["gflops"], r
        # every candidate the tuner times for this shape was timed (or skipped)
        assert set(cand) <= {tune.label(e, l) for e, l in tune.candidates(r["d"], r["n"])}


def test_automatic_form_is_the_faster_fp64_form():
    """The faster FP64 form, except that blocks where the double-float form
    does not hold 1e-13 (n = 2, fewer than 8 elements) always get FP64."""
    t = _table()
    best = {}
    for r in t["rows"]:
        if r["form"] in ("plain", "split") and r["layout"] == "batched":
            best[(r["form"], r["d"], r["n"])] = r["gflops"]
    for a in t["auto_form_f64"]:
        d, n = a["d"], a["n"]
        faster = "split" if best[("split", d, n)] > best[("plain", d, n)] else "plain"
        assert a["form"] == (faster if tune.split_allowed(d, n) else "plain"), a


def test_candidates_cover_every_engine_of_the_shape():
    for d, n in tune.shapes():
        engines = {e for e, _ in tune.candidates(d, n)}
        assert "per_mode" in engines
        assert ("tiled" in engines) == tune.has_tile(d, n)
        assert ("small" in engines) == tune.has_small(d, n)
        assert ("lane" in engines) == tune.has_lane(d, n)
        # the default launch shape of every engine is always among them
        for e in engines:
            assert (e, (0, 0, 0)) in tune.candidates(d, n)


def test_generated_header_matches_the_table():
    text = tune.header_from_table()
    t = _table()
    assert re.search(r"kTuneRows = (\d+);", text).group(1) == str(len(t["rows"]))
    assert re.search(r"kAutoRows = (\d+);", text).group(1) == str(len(t["auto_form_f64"]))
    for r in t["rows"]:
        row = "{%d, %d, %d, %d, %d, %d, %d, %d}" % (
            tune.FORM_CODES[r["form"]], tune.LAYOUT_CODES[r["layout"]], r["d"], r["n"],
            tune.ENGINE_CODES[r["engine"]], r["group_threads"], r["groups_per_cta"],
            r["ctas_per_sm"])
        assert row in text, row
    path = os.path.join(ROOT, "kronmult_gb300", "csrc", "kmx_tune_table.h")
    if os.path.exists(path):  # written by the build from the same table
        with open(path) as f:
            assert f.read() == text


def test_header_accepts_rows_without_layout(tmp_path):
    """Tables written before the layout column apply to the batched layout
    with the default launch shape."""
    p = tmp_path / "old.json"
    p.write_text(json.dumps({"rows": [{"form": "split", "d": 6, "n": 4, "engine": "tiled"}],
                             "auto_form_f64": []}))
    text = tune.header_from_table(str(p))
    assert "{2, 0, 6, 4, 2, 0, 0, 0}" in text


def _row(form, layout, d, n, g):
    return {"form": form, "layout": layout, "d": d, "n": n, "engine": "per_mode",
            "group_threads": 0, "groups_per_cta": 0, "ctas_per_sm": 0, "gflops": g,
            "candidates": {"per_mode": g}}


def test_partial_run_replaces_its_shapes_and_appends_the_record():
    old = {"measured": "T0", "rows": [_row("f32", "batched", 2, 3, 1.0),
                                      _row("plain", "pointer", 1, 2, 2.0),
                                      _row("plain", "batched", 2, 3, 3.0),
                                      _row("plain", "batched", 1, 2, 4.0)],
           "auto_form_f64": [{"d": 2, "n": 3, "form": "split"}, {"d": 1, "n": 2, "form": "plain"}],
           "retuned": {"shapes": ["1-2"], "measured": "T1"}}  # a single record, older format
    new = [_row("plain", "batched", 2, 3, 9.0)]
    t = tune.build_table(new, [{"d": 2, "n": 3, "form": "plain"}], "dev", "m", "T2",
                         {(2, 3)}, old)
    got = [(r["form"], r["layout"], r["d"], r["n"], r["gflops"]) for r in t["rows"]]
    assert got == [("plain", "batched", 1, 2, 4.0), ("plain", "pointer", 1, 2, 2.0),
                   ("plain", "batched", 2, 3, 9.0)]  # the old (2, 3) rows are gone
    assert t["auto_form_f64"] == [{"d": 1, "n": 2, "form": "plain"},
                                  {"d": 2, "n": 3, "form": "plain"}]
    assert t["measured"] == "T0"  # the full run's date
    assert t["retuned"] == [{"shapes": ["1-2"], "measured": "T1"},
                            {"shapes": ["2-3"], "measured": "T2"}]
    full = tune.build_table(new, [], "dev", "m", "T3")
    assert full["measured"] == "T3" and "retuned" not in full and full["rows"] == new
    # a partial run without an old table starts an empty one
    assert tune.build_table(new, [], "dev", "m", "T4", {(2, 3)})["retuned"][0]["measured"] == "T4"


def test_auto_forms_keep_plain_where_double_float_misses_the_bound():
    best = {("plain", "batched", 6, 2): 1.0, ("split", "batched", 6, 2): 2.0,
            ("plain", "batched", 3, 4): 1.0, ("split", "batched", 3, 4): 2.0,
            ("plain", "batched", 2, 8): 3.0, ("split", "batched", 2, 8): 2.0}
    forms = {(a["d"], a["n"]): a["form"] for a in tune.auto_forms(best)}
    assert forms == {(6, 2): "plain", (3, 4): "split", (2, 8): "plain"}


def test_committed_retune_records_name_tuned_shapes():
    t = _table()
    runs = t.get("retuned", [])
    assert isinstance(runs, list)
    valid = {f"{d}-{n}" for d, n in tune.shapes()}
    for run in runs:
        assert run["shapes"] and set(run["shapes"]) <= valid, run
        assert run["measured"] >= t["measured"], run


def test_lane_shapes_match_the_launcher():
    """tune.has_lane names exactly the shapes kmx_launch.cuh's pick_lane
    dispatches (a mismatch would time another engine under the lane label)."""
    src = open(os.path.join(ROOT, "kronmult_gb300", "csrc", "kmx_launch.cuh")).read()
    body = src[src.index("LaneKernel pick_lane("):]
    body = body[:body.index("default:")]
    cases = {(int(d), int(n)) for n, d in
             re.findall(r"case \d+: return lane_entry<T, FORM, (\d+), (\d+)>", body)}
    assert cases, "pick_lane switch not found"
    assert cases == {(d, n) for d, n in tune.shapes() if tune.has_lane(d, n)}
