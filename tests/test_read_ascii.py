"""The library's ASCII field reader (lbm_read_ascii, the replacement for the
np.loadtxt inside init_geo) returns exactly what np.loadtxt returns, on the
number formats and layouts such files use, across the chunk boundaries of its
parallel parse, and rejects what is not a number.  Host code only: no GPU."""
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "taichi_lbm3d_gb300", "liblbm_gb300.so")


@pytest.fixture(scope="module")
def native():
    if not os.path.exists(LIB):
        from taichi_lbm3d_gb300 import build
        build.build()
    from taichi_lbm3d_gb300 import _native
    return _native


def write(tmp_path, name, text):
    p = tmp_path / name
    p.write_bytes(text.encode())
    return str(p)


TOKENS = ["0", "1", "-0.5", "+2.25", "1e-3", "-7.125E+02", "3.", ".5", "0.1", "12345678901234567890",
          "1.0000000000000002", "-0", "9", "4.9406564584124654e-324", "1.7976931348623157e308"]


def test_formats_match_loadtxt(native, tmp_path):
    p = write(tmp_path, "one_per_line.dat", "\n".join(TOKENS) + "\n")
    got = native.read_ascii(p)
    assert got.dtype == np.float64 and np.array_equal(got, np.loadtxt(p))
    assert np.signbit(got[TOKENS.index("-0")])           # "-0" keeps its sign, as np.loadtxt's does
    # several per line, tabs, CRLF, blank lines: the same numbers as Python's float()
    text = "\n\n" + " ".join(TOKENS[:5]) + "\r\n\t" + "\t".join(TOKENS[5:]) + "  \r\n"
    got = native.read_ascii(write(tmp_path, "layout.dat", text))
    assert np.array_equal(got, np.array([float(t) for t in TOKENS]))


def test_large_file_across_chunk_boundaries(native, tmp_path):
    rng = np.random.default_rng(7)
    n = 400_000
    vals = np.where(rng.random(n) < 0.5, rng.integers(0, 2, n).astype(np.float64),
                    rng.standard_normal(n) * 10.0 ** rng.integers(-6, 6, n))
    p = str(tmp_path / "big.dat")
    np.savetxt(p, vals, fmt="%.17g")
    assert os.path.getsize(p) > (1 << 20)               # the parallel path
    got = native.read_ascii(p, n)
    assert np.array_equal(got, np.loadtxt(p))
    assert np.array_equal(got, vals)                     # %.17g round-trips exactly


def test_geometry_reader_uses_it_and_checks_the_count(native, tmp_path):
    from taichi_lbm3d_gb300 import geometry
    solid = (np.random.default_rng(3).random((5, 4, 3)) < 0.4).astype(np.int8)
    p = str(tmp_path / "geo.dat")
    geometry.write_ascii_geometry(p, solid)
    assert np.array_equal(geometry.read_ascii_geometry(p, solid.shape), solid)
    with pytest.raises(ValueError, match="holds 60 values"):
        geometry.read_ascii_geometry(p, (5, 4, 4))


def test_bad_tokens_and_edge_files(native, tmp_path):
    with pytest.raises(native.LbmError, match="not a number at byte 4"):
        native.read_ascii(write(tmp_path, "bad.dat", "0\n1\nx1\n"))
    with pytest.raises(native.LbmError, match="not a number"):
        native.read_ascii(write(tmp_path, "comment.dat", "# header\n1\n"))
    with pytest.raises(native.LbmError, match="cannot open"):
        native.read_ascii(str(tmp_path / "absent.dat"))
    assert native.read_ascii(write(tmp_path, "empty.dat", "")).size == 0
    assert np.array_equal(native.read_ascii(write(tmp_path, "nonl.dat", "1 0 1")), [1.0, 0.0, 1.0])
