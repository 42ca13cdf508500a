"""CPU tests of the shipped tune table (gpufinitefieldmatrices.jl_gb300/gffm/tuning.json):
every entry is well formed, the GEMM entries' work ranges tile each modulus band, and
the library's own check (gffm_tune_table_set, host code) accepts the whole table."""
import ctypes
import json
import os

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TABLE = os.path.join(ROOT, "gpufinitefieldmatrices.jl_gb300", "gffm", "tuning.json")


@pytest.fixture(scope="module")
def table():
    with open(TABLE) as f:
        return json.load(f)


def test_gemm_entries_are_well_formed(table):
    ents = table["gemm"]
    assert ents
    for e in ents:
        assert e["digit_bits"] in (7, 8)
        assert e["form"] in (0, 1, 2)
        assert e.get("tile_n", 0) in (0, 32, 64)
        assert e.get("max_ctas", 0) >= 0
        assert 2 <= e["N_lo"] <= e["N_hi"] < 2 ** 26
        assert 0 <= e["work_lo"] < e["work_hi"]


def test_gemm_work_ranges_tile_each_band(table):
    bands = {}
    for e in table["gemm"]:
        bands.setdefault((e["N_lo"], e["N_hi"]), []).append((e["work_lo"], e["work_hi"]))
    keys = sorted(bands)
    for (lo1, hi1), (lo2, hi2) in zip(keys, keys[1:]):
        assert hi1 < lo2                                  # modulus bands do not overlap
    for key, ranges in bands.items():
        ranges.sort()
        assert ranges[0][0] == 0.0
        for (a0, a1), (b0, b1) in zip(ranges, ranges[1:]):
            assert a1 == b0                               # contiguous, no overlap
        assert ranges[-1][1] >= 1e30


def test_batched_entries_are_well_formed(table):
    for key, e in table.get("batched", {}).items():
        assert len(key) == 16 and int(key, 16) >= 0       # batch_signature: 16 hex digits
        assert e["pluq_panel"] in (0, 8, 16, 32)
        assert e["overlap"] in (0, 1, 2)
        assert e["digit_bits"] in (0, 7, 8)
        assert e["gemm_ctas"] >= 0 and e["pluq_ctas"] >= 0


def test_library_accepts_the_table(table, tmp_path):
    import gffm
    from gffm import autotune
    gffm.build()
    L = gffm.load_library()
    assert autotune.apply(table) == len(table["gemm"])
    count = ctypes.c_int64(-1)
    assert L.gffm_tune_table_size(ctypes.byref(count)) == 0
    assert count.value == len(table["gemm"])
    # a digit width the library does not know is refused, and the table stays as it was
    bad = {"gemm": [dict(table["gemm"][0], digit_bits=9)]}
    with pytest.raises(Exception):
        autotune.apply(bad)
    assert L.gffm_tune_table_size(ctypes.byref(count)) == 0
    assert count.value == len(table["gemm"])
    # save / load round trip
    path = tmp_path / "t.json"
    autotune.save_table(table, str(path))
    assert autotune.load_table(str(path)) == table
