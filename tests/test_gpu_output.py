"""The CSV writers through the C ABI and the `bem input.json` program
(main.rs:1-9): files compared byte for byte with the oracle's restatement of
postprocess.rs:15-67 on the same results, and the values with the oracle's
own run of the reference algorithm."""
import csv
import json
import os
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import ROOT, sphere_input
from oracle import oracle as O

pytestmark = pytest.mark.gpu
bem = pytest.importorskip("cc_abstemious_gb300")


def _inp(path, freqs=(100.0,)):
    d = sphere_input(frequency={"List": {"values": list(freqs)}})
    d["output"]["file"] = path
    d["output"]["field_points"] = [[10.0, 0.0, 0.0], [0.0, -7.5, 2.25], [1e-3, 3.0, -4.0]]
    return d


def test_write_results_at_frequency_bytes_and_values():
    wd = tempfile.mkdtemp(prefix="bem_out_")
    out = os.path.join(wd, "out.csv")
    inp = _inp(out)
    a = bem.Analysis()
    a.set_input(inp)
    a.run()
    a.write_results_at_frequency(0)
    r = a.get_result()[0]
    got = open(out, "rb").read()
    assert got == O.csv_results_at_frequency(inp["output"]["field_points"], r.scattered, r.incident)
    # the values against the oracle's run of the reference algorithm
    ref = O.Problem(inp).run()[0]
    rows = list(csv.DictReader(open(out)))
    sc = np.array([float(x["pre_re"]) + 1j * float(x["pre_im"]) for x in rows])
    assert np.max(np.abs(sc - ref["scattered"])) <= 1e-10 * np.max(np.abs(ref["scattered"]))


def test_write_results_at_point_bytes():
    wd = tempfile.mkdtemp(prefix="bem_out_")
    out = os.path.join(wd, "pt.csv")
    inp = _inp(out, freqs=(80.0, 100.0, 125.5))
    inp["output"]["field"] = "VelocityPotential"
    a = bem.Analysis()
    a.set_input(inp)
    a.run()
    a.write_results_at_point(1)
    res = a.get_result()
    want = O.csv_results_at_point([x.frequency for x in res], [x.scattered for x in res],
                                  [x.incident for x in res], 1, pressure=False)
    assert open(out, "rb").read() == want
    with pytest.raises(bem.BemError):
        a.write_results_at_point(3)


def test_cli_writes_first_frequency():
    """`bem input.json` runs every frequency and writes the first one to
    output.file, as main.rs does."""
    wd = tempfile.mkdtemp(prefix="bem_cli_")
    out = os.path.join(wd, "cli.csv")
    inp = _inp(out, freqs=(100.0, 150.0))
    path = os.path.join(wd, "input.json")
    with open(path, "w") as f:
        json.dump(inp, f)
    exe = os.path.join(ROOT, "cc_abstemious_gb300", "bem")
    r = subprocess.run([exe, path], capture_output=True, text=True, cwd=wd)
    assert r.returncode == 0, r.stderr
    a = bem.Analysis()
    a.set_input(inp)
    a.run()
    res = a.get_result()[0]
    assert open(out, "rb").read() == O.csv_results_at_frequency(inp["output"]["field_points"], res.scattered,
                                                               res.incident)
    bad = os.path.join(wd, "missing.json")
    r = subprocess.run([exe, bad], capture_output=True, text=True, cwd=wd)
    assert r.returncode == 1 and "cannot open input file" in r.stderr
