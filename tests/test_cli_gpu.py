"""The drop-in command lines keep the reference drivers' argv and output lines."""
import json
import os
import re
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BIN = os.path.join(ROOT, "fortkernels-_gb300")
GOLD = os.path.join(os.path.dirname(__file__), "golden", "reference_drivers.json")
CPLX = re.compile(r"\(\s*([-+0-9.eE]+)\s*,\s*([-+0-9.eE]+)\s*\)")


def run(exe, *args):
    out = subprocess.run([os.path.join(BIN, exe)] + [str(a) for a in args], capture_output=True, text=True,
                         check=True, timeout=300).stdout
    vals = {}
    for line in out.splitlines():
        m = re.match(r"\s*(\w+(?:\[\d\])?)\s*=\s*(\(.*)$", line)
        if m:
            c = CPLX.search(m.group(2))
            vals[m.group(1)] = complex(float(c.group(1)), float(c.group(2)))
    return out, vals


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_gppKer_cli_prints_reference_values(prec):
    with open(GOLD) as f:
        e = [x for x in json.load(f)["gppKer_bgw"] if x["args"] == [512, 2, 2048, 32]][0]
    out, v = run("gppKer", *e["args"], f"--precision={prec}")
    assert "Chrono Time Taken" in out and "ngpown = 64" in out
    got = np.array([v[f"achtemp[{i}]"] for i in range(3)])
    want = np.array([complex(*z) for z in e["achtemp_exact"]])
    # 15 printed digits; the mixed path is within 1e-6
    assert np.max(np.abs(got - want)) / np.max(np.abs(want)) <= (1e-13 if prec == "fp64" else 1e-6)


def test_gppKer_cli_half_sum_prints_seq_driver_values():
    """Five arguments: gppKerSeq.cpp's command line; gppsum = 1 is the half sum."""
    with open(GOLD) as f:
        e = json.load(f)["gppKer_seq"][0]
    out, v = run("gppKer", *e["args"])
    assert "gppsum = 1" in out
    got = np.array([v[f"achtemp[{i}]"] for i in range(3)])
    want = np.array([complex(*z) for z in e["achtemp"]])
    assert np.max(np.abs(got - want)) / np.max(np.abs(want)) <= 1e-13
    r = subprocess.run([os.path.join(BIN, "gppKer")] + [str(a) for a in e["args"][:4]] + ["0"],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 1 and "gppsum = 0" in r.stderr


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_gppKer_real_cli_prints_reference_values(prec):
    with open(GOLD) as f:
        e = json.load(f)["gppKer_real"][1]
    out = subprocess.run([os.path.join(BIN, "gppKer_real")] + [str(a) for a in e["args"]] + [f"--precision={prec}"],
                         capture_output=True, text=True, check=True, timeout=300).stdout
    assert "Chrono Time Taken" in out
    got = np.array([float(re.search(rf"achtemp\[{i}\] = (\S+)", out).group(1)) for i in range(3)])
    want = np.array(e["achtemp_exact"])
    assert np.max(np.abs(got - want)) / np.max(np.abs(want)) <= (1e-13 if prec == "fp64" else 1e-6)


def test_gppKer_cli_usage_line():
    out = subprocess.run([os.path.join(BIN, "gppKer")], capture_output=True, text=True).stdout
    assert "The correct form of input is" in out


def test_ffKernel_cli_prints_reference_values():
    with open(GOLD) as f:
        e = [x for x in json.load(f)["ffKernel"] if x["args"] == [64, 2, 512, 64, 15, 10]][0]
    out, v = run("ffKernel", *e["args"])
    assert abs(v["achsDtemp"] - complex(*e["achsDtemp"])) <= 1e-6 * abs(complex(*e["achsDtemp"]))
    assert abs(v["asxDtemp"] - complex(*e["asxDtemp0"])) <= 1e-6 * abs(complex(*e["asxDtemp0"]))
    assert abs(v["achDtemp_cor"] - complex(*e["achDtemp_cor0"])) <= 1e-6 * abs(complex(*e["achDtemp_cor0"]))
