"""The committed tables of the FP64 viscosity power (csrc/pow_tables.h) are what their
generator writes, and they hold what the generator's docstring says: r_i close to 1/c_i,
-ln r_i and 2^(i/64) as double-doubles accurate to well below an ulp of the head."""
import contextlib
import importlib.util
import io
import os
import re

import pytest

CSRC = os.path.join(os.path.dirname(__file__), "..", "cudanavierstokes_gb300", "csrc")


def committed():
    with open(os.path.join(CSRC, "pow_tables.h")) as f:
        return f.read()


def test_header_is_the_generator_output():
    pytest.importorskip("mpmath")
    spec = importlib.util.spec_from_file_location("gen_pow_tables", os.path.join(CSRC, "gen_pow_tables.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    out = io.StringIO()
    with contextlib.redirect_stdout(out):
        mod.main()
    assert out.getvalue() == committed()


def test_table_values():
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.dps = 50
    src = committed()
    tab = {m.group(1): [float.fromhex(v.strip()) for v in m.group(2).split(",")]
           for m in re.finditer(r"double (\w+)\[64\] = \{([^}]*)\}", src, re.S)}
    assert sorted(tab) == ["kPowExpHi", "kPowExpLo", "kPowLnHi", "kPowLnLo", "kPowRcp"]
    for i in range(64):
        c = 1 + (mpmath.mpf(i) + 0.5) / 64
        r = tab["kPowRcp"][i]
        assert abs(r * c - 1) < 2.0 ** -52
        ln = mpmath.mpf(tab["kPowLnHi"][i]) + mpmath.mpf(tab["kPowLnLo"][i])
        assert abs(ln + mpmath.log(mpmath.mpf(r))) < mpmath.mpf(2) ** -100
        ex = mpmath.mpf(tab["kPowExpHi"][i]) + mpmath.mpf(tab["kPowExpLo"][i])
        assert abs(ex - mpmath.power(2, mpmath.mpf(i) / 64)) < mpmath.mpf(2) ** -100
    defs = {m.group(1): float.fromhex(m.group(2)) for m in re.finditer(r"#define (\w+) (\S+)", src)}
    for name, v in (("POW_LN2", mpmath.log(2)), ("POW_LN2_64", mpmath.log(2) / 64)):
        hi, lo = defs[name + "_HI"], defs[name + "_LO"]
        assert abs(mpmath.mpf(hi) + mpmath.mpf(lo) - v) < mpmath.mpf(2) ** -100
        # the head has trailing zero bits, so k * hi (|k| < 2^11) and j * hi (|j| < 2^13) are exact
        m, _ = mpmath.frexp(mpmath.mpf(hi))
        assert mpmath.ldexp(m, 42) == int(mpmath.ldexp(m, 42))
