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
