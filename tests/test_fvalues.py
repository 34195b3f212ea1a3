"""Futhark value files (text and binary) and the futhark-bench-style harness
logic: CPU only."""
import hashlib
import io
import os

import numpy as np
import pytest

from synkrotomo_gb300 import fbench, fvalues
from tests.conftest import GOLDEN, load_fpinput512

# directory holding the reference's own dataset files (optional: the exact
# copy under tests/golden/ is what the tests run on)
REF_DATA_DIR = os.environ.get("SYNK_REFERENCE_DATA", "")


def test_text_scalars_and_suffixes():
    v = fvalues.read_values("1 1.5 -2i8 3u8 4i64 2.5f32 -0.25f64 true false 1_000 0x10i64 0b101u16 1e3f32")
    assert [np.asarray(x).dtype for x in v] == [np.int32, np.float64, np.int8, np.uint8, np.int64, np.float32,
                                                np.float64, np.bool_, np.bool_, np.int32, np.int64, np.uint16,
                                                np.float32]
    assert [x.item() for x in v] == [1, 1.5, -2, 3, 4, 2.5, -0.25, True, False, 1000, 16, 5, 1000.0]


def test_text_specials_comments_empty_and_nesting():
    v = fvalues.read_values("-- a comment\n f32.nan -f64.inf f32.inf [[1i32, 2i32], [3i32, 4i32]]"
                            " empty([0][3]f32) -- trailing\n [true, false]")
    assert np.isnan(v[0]) and v[0].dtype == np.float32
    assert v[1] == -np.inf and v[2] == np.inf
    np.testing.assert_array_equal(v[3], np.array([[1, 2], [3, 4]], np.int32))
    assert v[4].shape == (0, 3) and v[4].dtype == np.float32
    np.testing.assert_array_equal(v[5], [True, False])


@pytest.mark.parametrize("bad", ["[1i32, 2i64]", "[[1], [2, 3]]", "[]", "300u8", "1.5i32", "[1f32, 2f32",
                                 "empty([2]f32)", "x"])
def test_text_rejects_malformed(bad):
    with pytest.raises(fvalues.FormatError):
        fvalues.read_values(bad)


def _sample_values():
    rng = np.random.default_rng(3)
    return [rng.standard_normal(7).astype(np.float32), np.float32(-362.0), np.int32(725),
            rng.integers(-5, 5, (2, 3)).astype(np.int64), np.array([True, False, True]), np.uint8(200),
            np.zeros((0, 4), np.float32), np.array([np.nan, np.inf, -np.inf, -0.0], np.float32),
            np.float64(1.0 / 3.0), rng.random(5).astype(np.float16)]


def _same(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return a.dtype == b.dtype and a.shape == b.shape and np.array_equal(a, b, equal_nan=a.dtype.kind == "f")


def test_text_round_trip_is_exact():
    vals = _sample_values()
    back = fvalues.read_values(fvalues.write_text(vals))
    assert len(back) == len(vals)
    assert all(_same(a, b) for a, b in zip(vals, back))


def test_binary_round_trip_and_header():
    vals = _sample_values()
    blob = fvalues.write_binary(vals)
    assert blob[:7] == b"b\x02\x01 f32"               # 'b', version 2, rank 1, type " f32"
    assert blob[7:15] == (7).to_bytes(8, "little")
    back = fvalues.read_values(blob)
    assert all(_same(a, b) for a, b in zip(vals, back))


def test_mixed_text_and_binary_stream():
    blob = b"1.0f32 " + fvalues.write_binary([np.arange(4, dtype=np.int32)]) + b" 725i32\n"
    v = fvalues.read_values(blob)
    assert v[0] == np.float32(1.0) and v[2] == np.int32(725)
    np.testing.assert_array_equal(v[1], np.arange(4))


def test_binary_rejects_bad_version_and_truncation():
    blob = fvalues.write_binary([np.arange(4, dtype=np.float32)])
    with pytest.raises(fvalues.FormatError):
        fvalues.read_values(blob[:1] + b"\x02" + blob[2:-1])
    with pytest.raises(fvalues.FormatError):
        fvalues.read_values(b"b\x02\x01 f99" + blob[7:])


def test_argument_check_follows_entry_point_types():
    good = [np.zeros(3, np.float32), np.float32(-1.0), np.float32(1.0), np.int32(4), np.zeros(16, np.float32)]
    out = fbench.parse_args_for("forwardprojection", good)
    assert out[3] == 4 and out[4].dtype == np.float32
    with pytest.raises(fvalues.FormatError):      # numrhos given as f32
        fbench.parse_args_for("forwardprojection", good[:3] + [np.float32(4)] + good[4:])
    with pytest.raises(fvalues.FormatError):      # wrong arity
        fbench.parse_args_for("SIRT", good)
    assert len(fbench.parse_args_for("diff", [np.zeros(2, np.float32), np.ones(2, np.float32)])) == 2


def test_dataset_size_and_csv(tmp_path):
    assert fbench.dataset_size("data/fpinputf32rad512") == 512
    assert fbench.dataset_size("bpsparseinputf32rad45") == 45
    p = tmp_path / "fut_fp.csv"
    fbench.write_csv([(64, 225.4, []), (128, 348.104, [])], str(p))
    assert p.read_text() == "64;225.40\n128;348.10\n"


def _check_fpinput512(vals):
    args = fbench.parse_args_for("forwardprojection", vals)
    angles, rz, dr, nr, img = args
    assert angles.shape == (805,) and angles.dtype == np.float32
    assert abs(angles[0] - np.pi / 4) < 1e-6 and angles[-1] < 3 * np.pi / 4
    assert (rz, dr, nr) == (np.float32(-362.0), np.float32(1.0), np.int32(725))
    assert img.shape == (512 * 512,) and np.count_nonzero(img) == 205859
    back = fvalues.read_values(fvalues.write_binary(vals))
    assert all(_same(a, b) for a, b in zip(vals, back))
    return args


def test_reference_dataset_copy_round_trips():
    """The exact copy of data/fpinputf32rad512 (forwardprojection.main's five
    arguments) written in both value formats and read back."""
    angles, rz, dr, nr, img = load_fpinput512()
    vals = [angles, rz, dr, nr, img]
    _check_fpinput512(vals)
    text = fvalues.write_text(vals)
    assert all(_same(a, b) for a, b in zip(vals, fvalues.read_values(text)))


@pytest.mark.skipif(not REF_DATA_DIR, reason="SYNK_REFERENCE_DATA (the reference's futhark/data directory) not set")
def test_reads_the_reference_dataset():
    """data/fpinputf32rad512 itself, when its directory is given: it parses to
    the values of the committed copy."""
    path = os.path.join(REF_DATA_DIR, "fpinputf32rad512")
    raw = open(path, "rb").read()
    args = _check_fpinput512(fvalues.read_values(raw))
    copy = load_fpinput512()
    assert all(_same(a, b) for a, b in zip(args, copy))
    z = np.load(os.path.join(GOLDEN, "fpinputf32rad512.npz"))
    assert str(z["source_sha256"]) == hashlib.sha256(raw).hexdigest()
