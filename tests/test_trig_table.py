"""The sin / cos tables the FP64 update reads (csrc/trig_table.inc and
csrc/trig_table_f.inc, written by csrc/gen_trig_table.py): every entry of
the first the correctly rounded double of cos, sin and cos - 1 at j / 128;
every entry of the second the float pair (hi, lo) of cos and sin at j / 512
with hi the correctly rounded float and lo the correctly rounded remainder;
and the generator reproduces both files."""
import math
import os
import re
import struct

import numpy as np
import pytest

CSRC = os.path.join(os.path.dirname(__file__), "..", "stochasticsampling_gb300", "csrc")


def _table():
    src = open(os.path.join(CSRC, "trig_table.inc")).read()
    n = int(re.search(r"kTrigN = (\d+);", src).group(1))
    key = int(re.search(r"kTrigMaxKey = 0x([0-9A-F]+)ll", src).group(1), 16)
    body = src.split("kTrig[kTrigN] = {")[1].split("};")[0]
    pairs = re.findall(r"\{(\S+), (\S+)\}", body)
    cm1 = src.split("kTrigCm1[kTrigN] = {")[1].split("};")[0]
    cm1 = [float.fromhex(v.strip().rstrip(",")) for v in cm1.strip().splitlines()]
    return n, key, [(float.fromhex(c), float.fromhex(s)) for c, s in pairs], cm1


def _table_f():
    src = open(os.path.join(CSRC, "trig_table_f.inc")).read()
    n = int(re.search(r"kTrigFN = (\d+);", src).group(1))
    key = int(re.search(r"kTrigFMaxKey = 0x([0-9A-F]+)ll", src).group(1), 16)
    body = src.split("kTrigF[kTrigFN] = {")[1].split("};")[0]
    rows = re.findall(r"\{(\S+), (\S+), (\S+), (\S+)\}", body)
    return n, key, [tuple(float.fromhex(v.rstrip("f")) for v in r) for r in rows]


def test_pair_table_shape_and_range_key():
    n, key, rows = _table_f()
    assert len(rows) == n
    assert struct.unpack("<d", struct.pack("<q", key))[0] == 6.3
    assert round(512 * 6.3) < n and (n - 1) / 512 > 6.3 + 2 ** -10
    assert all(np.float32(v) == v for r in rows for v in r)  # every literal is a float


def test_pair_entries_correctly_rounded():
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.dps = 40
    n, key, rows = _table_f()

    def rn32(x):
        with mpmath.workprec(24):
            return float(+x)

    for j in range(0, n, 5):
        a = mpmath.mpf(j) / 512
        for (h, l), exact in ((rows[j][0:2], mpmath.cos(a)), (rows[j][2:4], mpmath.sin(a))):
            assert h == rn32(exact), j
            assert l == rn32(exact - mpmath.mpf(h)), j


def test_table_shape_and_range_key():
    n, key, cs, cm1 = _table()
    assert len(cs) == n and len(cm1) == n
    # the table path covers a in [0, 6.3): round(128 a) <= 806 < n
    assert struct.unpack("<d", struct.pack("<q", key))[0] == 6.3
    assert round(128 * 6.3) < n
    assert (n - 1) / 128 > 2 * math.pi + 2 ** -8


def test_entries_correctly_rounded():
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.dps = 40
    n, key, cs, cm1 = _table()
    for j in range(0, n, 7):
        a = mpmath.mpf(j) / 128
        for got, exact in ((cs[j][0], mpmath.cos(a)), (cs[j][1], mpmath.sin(a)),
                           (cm1[j], -2 * mpmath.sin(a / 2) ** 2)):
            err = abs(mpmath.mpf(got) - exact)
            assert err <= mpmath.mpf(math.ulp(float(exact)) if exact != 0 else 0) / 2, (j, got)


def test_entries_within_an_ulp_of_libm():
    n, key, cs, cm1 = _table()
    a = np.arange(n) / 128.0
    c = np.array([v[0] for v in cs])
    s = np.array([v[1] for v in cs])
    ulp = np.spacing(np.maximum(np.abs(np.cos(a)), np.abs(np.sin(a))))
    assert np.all(np.abs(c - np.cos(a)) <= ulp) and np.all(np.abs(s - np.sin(a)) <= ulp)


def test_generator_reproduces_the_file(tmp_path):
    pytest.importorskip("mpmath")
    import importlib.util
    spec = importlib.util.spec_from_file_location("gen_trig_table", os.path.join(CSRC, "gen_trig_table.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    out = tmp_path / "trig_table.inc"
    mod.main(str(out))
    assert out.read_text() == open(os.path.join(CSRC, "trig_table.inc")).read()
    out_f = tmp_path / "trig_table_f.inc"
    mod.main_f(str(out_f))
    assert out_f.read_text() == open(os.path.join(CSRC, "trig_table_f.inc")).read()
