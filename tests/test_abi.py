"""CPU-side checks of the C ABI library: it loads, exports every declared symbol, and its
host-only entry points (initgrid) agree with the oracle.  No GPU calls."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = []
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", h)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names += re.findall(r"\b(cans_[a-z0-9_]+)\s*\(", txt)
    return sorted(set(names))


@pytest.fixture(scope="module")
def so():
    from cans_gb300 import build
    path = build.build()
    return C.CDLL(path)


def test_exports_every_declared_symbol(so):
    names = _declared()
    assert len(names) >= 20
    for n in names:
        assert hasattr(so, n), n


def test_initgrid_matches_oracle(so):
    from oracle import oracle as O
    P = C.POINTER(C.c_double)
    so.cans_initgrid.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_int, P, P, P, P]
    for gtype, n, gr, lz, per in ((1, 256, 1.4, 2.0, 0), (1, 384, 1.4, 2.0, 0), (2, 33, 2.0, 1.0, 0),
                                  (3, 17, 1.5, 1.0, 0), (4, 40, 1.2, 3.0, 0), (1, 16, 0.0, 1.0, 1)):
        arrs = [np.zeros(n + 2) for _ in range(4)]
        assert so.cans_initgrid(gtype, n, gr, lz, per, *[a.ctypes.data_as(P) for a in arrs]) == 0
        for got, want in zip(arrs, O.initgrid(gtype, n, gr, lz, per)):
            assert np.array_equal(got, want)


def test_strerror_and_version(so):
    so.cans_strerror.restype = C.c_char_p
    so.cans_version.restype = C.c_char_p
    assert b"sm_103a" in so.cans_version()
    assert so.cans_strerror(1) == b"invalid argument"


def test_null_arguments_are_rejected_without_a_gpu(so):
    """Argument checks run before any CUDA call, so they work on a machine without a GPU."""
    assert so.cans_fillps(None, None, None, C.c_double(1.0), None, None, None, None, None) == 1
    assert so.cans_solver(None, None) == 1


def test_checkpoint_file_reader_checks_size(tmp_path):
    """The host reader of the checkpoint layout (interior in Fortran order + [time, istep])."""
    from cans_gb300 import cans
    n = (4, 3, 2)
    vals = np.arange(24, dtype=np.float64)
    np.concatenate([vals, [0.5, 7.0]]).tofile(tmp_path / "f.bin")
    inner, t, it = cans.read_field_file(tmp_path / "f.bin", n)
    assert inner.shape == n and inner[1, 0, 0] == 1.0 and inner[0, 1, 0] == 4.0 and (t, it) == (0.5, 7)
    vals.tofile(tmp_path / "g.bin")
    with pytest.raises(ValueError):
        cans.read_field_file(tmp_path / "g.bin", n)
