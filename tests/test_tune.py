"""CPU tests of the autotuner's committed table: well formed, covering every
tuned shape, each row's choice the fastest engine it measured, and compiled
into the header the library reads."""
import json
import os
import re

from kronmult_gb300 import tune

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _table():
    with open(tune.TABLE) as f:
        return json.load(f)


def test_table_covers_every_tuned_shape():
    t = _table()
    have = {(r["form"], r["d"], r["n"]) for r in t["rows"]}
    for form in ("plain", "split", "f32"):
        for d, n in tune.shapes():
            assert (form, d, n) in have, (form, d, n)
    assert {(a["d"], a["n"]) for a in t["auto_form_f64"]} == set(tune.shapes())


def test_each_row_records_its_fastest_engine():
    for r in _table()["rows"]:
        g = r["gflops"]
        assert r["engine"] in tune.ENGINE_CODES
        assert r["engine"] in g
        assert g[r["engine"]] == max(g.values()), r


def test_automatic_form_is_the_faster_fp64_form():
    t = _table()
    best = {}
    for r in t["rows"]:
        if r["form"] in ("plain", "split"):
            best[(r["form"], r["d"], r["n"])] = max(r["gflops"].values())
    for a in t["auto_form_f64"]:
        d, n = a["d"], a["n"]
        faster = "split" if best[("split", d, n)] >= best[("plain", d, n)] else "plain"
        assert a["form"] == faster, a


def test_generated_header_matches_the_table():
    text = tune.header_from_table()
    t = _table()
    assert re.search(r"kTuneRows = (\d+);", text).group(1) == str(len(t["rows"]))
    assert re.search(r"kAutoRows = (\d+);", text).group(1) == str(len(t["auto_form_f64"]))
    for r in t["rows"]:
        row = "{%d, %d, %d, %d}" % (tune.FORM_CODES[r["form"]], r["d"], r["n"],
                                   tune.ENGINE_CODES[r["engine"]])
        assert row in text, row
    path = os.path.join(ROOT, "kronmult_gb300", "csrc", "kmx_tune_table.h")
    if os.path.exists(path):  # written by the build from the same table
        with open(path) as f:
            assert f.read() == text
