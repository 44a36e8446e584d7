"""CPU tests of bench.py's roofline arithmetic: the term counts, the
algorithmic bytes and flops of the dominant kernel, and the choice of bound."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

PEAKS = {"hbm_gbs": 6786.2, "bf16_tflops": 1900.0}


@pytest.fixture(scope="module")
def bench():
    import bench as b
    return b


def test_gpp_default_workload_is_hbm_bound(bench):
    w = dict(bench.WORKLOADS["gpp"], name="gpp")
    assert bench.terms(w) == 512 * 20 * 32768 * 3
    byts, flops = bench.algorithmic(w)
    # every aqsntemp row once (16 B per complex; the occupied bands' sch terms go through
    # the contraction too) and the D image (8 B per complex)
    assert byts == 16 * 512 * 32768 + 8 * 60 * 32768 == 284164096
    assert flops == 8 * 512 * 60 * 32768
    r = bench.roofline(w, "mixed", byts, flops, 0.070, 1, PEAKS)
    assert r["bound"] == "hbm" and r["unit"] == "GB/s" and r["peak"] == PEAKS["hbm_gbs"]
    assert r["achieved"] == pytest.approx(byts / 70e-6 / 1e9)
    assert r["frac"] == pytest.approx(r["achieved"] / PEAKS["hbm_gbs"])
    assert 0.5 < r["frac"] < 0.7


def test_half_sum_counts_both_contractions(bench):
    w = dict(bench.WORKLOADS["gpphalf"], name="gpphalf")
    full = dict(w, half=False)
    # the bands n1 >= nvband, once per A operand (aqsntemp, aqsmtemp)
    M, N, K = 510, 60, 32768
    assert bench.algorithmic(w) == (2 * (16 * M * K + 8 * N * K), 2 * 8 * M * N * K)
    # ig < igp for the baseline columns igp = i * ncouls / ngpown: about half the full sum
    assert 0.4 < bench.terms(w) / bench.terms(full) < 0.5


def test_ff_config_is_tensor_bound(bench):
    w = dict(bench.WORKLOADS["ff"], name="ff")
    byts, flops = bench.algorithmic(w)
    assert flops == 8 * 15 * 512 * 512 * 4096
    r = bench.roofline(w, "mixed", byts, flops, 1.204, 2, PEAKS)
    assert r["bound"] == "tensor" and r["unit"] == "TFLOP/s"
    assert r["duration_ms"] == pytest.approx(0.602)
    assert r["frac"] == pytest.approx(flops / 1.204e-3 / 1e12 / PEAKS["bf16_tflops"])
    assert r["piece_products"] == 3  # FF: FP16 hi/lo pieces
    assert r["executed_tensor_tflops"] == pytest.approx(3 * r["achieved"])


def test_fp64_precision_is_reported_against_hbm_and_without_traffic(bench):
    w = dict(bench.WORKLOADS["ff"], name="ff")
    byts, flops = bench.algorithmic(w)
    r = bench.roofline(w, "fp64", byts, flops, 100.0, 2, PEAKS)
    assert r["bound"] == "hbm" and r["traffic"] is None


def test_fallback_peaks_are_named(bench):
    w = dict(bench.WORKLOADS["gpp"], name="gpp")
    byts, flops = bench.algorithmic(w)
    r = bench.roofline(w, "mixed", byts, flops, 0.070, 1, {})
    assert r["peak_source"] == "fallback" and r["peak"] == 6800.0


def test_reference_ff_program_timing(bench, monkeypatch):
    """The reference's FF program is timed only for FF shapes whose epsilon planes
    fit in 4 GB of host memory; where it was built here it reports its own kernel
    time for a small shape."""
    for name in ("gpp", "ff4", "ffsigma"):
        assert bench.reference_ff_binary(dict(bench.WORKLOADS[name], name=name)) is None
    if not os.access(bench.REF_FF, os.X_OK):
        pytest.skip("the reference's FF program is not built on this machine")
    monkeypatch.setattr(os, "cpu_count", lambda: 2)
    w = dict(kind="ff", nb=16, nv=2, nc=256, ng=64, nf=4, ne=3)
    r = bench.reference_ff_binary(w, runs=1, warmup=0)
    assert r is not None and r["runs"] == 1 and r["cores"] == 2 and r["args"] == [16, 2, 256, 64, 4, 3]
    assert 0 <= r["kernel_s"] < 60


def test_served_stream_roofline(bench):
    """The served stream's roofline: every request's contraction (bands nvband..nb-1
    against 3*ngpown columns, ngpown = ncouls/64) over the burst's wall time."""
    w = dict(bench.WORKLOADS["serve"], name="serve")
    levels, reqs, _ = bench.serve_stream(w, seed=2024)
    assert len(reqs) == 256 and all(nb in w["nb_choices"] and nc in levels for nb, nc in reqs)
    byts = sum(16 * (nb - 2) * nc + 8 * 3 * (nc // 64) * nc for nb, nc in reqs)
    flops = sum(8 * (nb - 2) * 3 * (nc // 64) * nc for nb, nc in reqs)
    r = bench.serve_roofline(reqs, w["nv"], 0.125, 350, PEAKS)
    assert r["algorithmic_bytes"] == byts and r["algorithmic_flops"] == flops
    # large requests make the stream tensor-bound: six BF16 piece products per complex MAC
    assert 6 * flops / (PEAKS["bf16_tflops"] * 1e12) > byts / (PEAKS["hbm_gbs"] * 1e9)
    assert r["bound"] == "tensor" and r["unit"] == "TFLOP/s" and r["piece_products"] == 6
    assert r["achieved"] == pytest.approx(flops / 0.125 / 1e12)
    assert r["duration_ms"] == pytest.approx(125.0 / 350) and r["traffic"] is None
    assert "lower bound" in r["basis"]
