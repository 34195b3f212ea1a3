"""Autotuner cache logic (CPU only: a fake measurement stands in for the GPU)."""
from synkrotomo_gb300 import autotune


def test_bucket_rounds_to_powers_of_two():
    assert autotune.bucket(128, 128, 182, 1) == "N128_a128_d256_s1"
    assert autotune.bucket(100, 60, 142, 3) == "N128_a64_d256_s4"


def test_candidates_respect_minimum_work():
    c = autotune.candidates(32, 16, 304)
    assert {x["fp_split"] for x in c} == {1, 2}          # 32 rows: at least 16 rows per part
    assert {x["bp_split"] for x in c} == {1, 2}          # 16 angles: at least 8 per part
    assert {x["grid_blocks"] for x in c} == {152, 304, -1}   # -1: the phase-split engine


def test_choose_measures_once_then_reads_the_cache(tmp_path):
    path = str(tmp_path / "t.json")
    calls = []

    def measure(c):
        calls.append(c)
        return 1.0 + c["fp_split"] - 0.1 * c["bp_split"]

    cands = autotune.candidates(256, 256, 100)
    best = autotune.choose("k", cands, measure, path=path)
    assert best["fp_split"] == 1 and best["bp_split"] == 8
    n = len(calls)
    assert n == len(cands)
    again = autotune.choose("k", cands, measure, path=path)
    assert again == best and len(calls) == n
    assert autotune.load_cache(path)["k"]["fp_split"] == 1
