"""Output path (postprocess.rs:15-67): the number format of the CSV writers,
checked on the CPU against the oracle's restatement of Rust's f64 Display
(shortest round-trip digits, positional notation).  The writers themselves
and the `bem` program are checked in tests/test_gpu_output.py."""
import struct

import numpy as np

import cc_abstemious_gb300 as bem
from oracle.oracle import rust_f64_display


def test_known_rust_strings():
    # what `x.to_string()` gives in Rust for these f64 values
    known = [(1.0, "1"), (-0.0, "-0"), (0.0, "0"), (0.1, "0.1"), (1e-7, "0.0000001"), (100.0, "100"),
             (-12.5, "-12.5"), (1e23, "100000000000000000000000"), (0.30000000000000004, "0.30000000000000004"),
             (123456789.125, "123456789.125"), (float("nan"), "NaN"), (float("inf"), "inf"),
             (float("-inf"), "-inf"), (5e-324, "0." + "0" * 323 + "5"),
             (1.7976931348623157e308, "17976931348623157" + "0" * 292)]
    for v, s in known:
        assert bem.format_f64(v) == s, (v, bem.format_f64(v), s)
        assert rust_f64_display(v) == s


def test_format_matches_oracle_on_random_doubles():
    rng = np.random.default_rng(7)
    bits = rng.integers(0, 2 ** 63, size=5000, dtype=np.int64)
    vals = [struct.unpack("<d", struct.pack("<q", int(x)))[0] for x in bits]
    vals += [-v for v in vals[:1000]]
    vals += list(rng.standard_normal(2000) * 10.0 ** rng.integers(-40, 40, 2000))
    bad = [(v, bem.format_f64(v), rust_f64_display(v)) for v in vals if bem.format_f64(v) != rust_f64_display(v)]
    assert not bad, bad[:5]
