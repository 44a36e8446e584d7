"""Benchmark: GPP / FF self-energy terms/s on GB300 (one JSON line on rank 0).

Default workload: the GPP sum at full mini-app size, number_bands=512,
nvband=2, ncouls=32768, ngpown=20 (synthetic inputs with the benchmark value
distributions), mixed precision, with the FP64 path measured beside it.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload gpp|gpp1638|gpphalf|gppreal|ff|ff4|ffsigma|serve]
                  [--precision mixed|fp64] [--no-cpu] [--headline-only]

A step is one call of the hot path over one set of inputs.  `value` is the
device throughput with inputs resident in HBM (CUDA events on the library's
stream); `e2e` repeats the step through the C ABI with pinned HOST buffers,
so the host->device staging and the device->host read of the outputs are
inside the timed region.  Under torchrun every rank runs its own replica
(the path has no exchange step), and the slowest rank's time is used.
`--impl reference` times the reference's own GPP program built from its
sources (oracle/_ref) on all host cores where the workload can be expressed
in its arguments, else the CPU restatement of the reference loop nest
(oracle/, OpenMP on all host cores), on the same workload.  FF lines also
carry the reference's own FF program's time (`reference_program`), which
covers a subset of the call's outputs.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # GPP at full mini-app size: 512 bands, 2 valence, ncouls 32768, ngpown 20
    "gpp": dict(kind="gpp", nb=512, nv=2, nc=32768, ng=20),
    # the reference's canonical run `gppKer 512 2 32768 20` (ngpown = 32768/20)
    "gpp1638": dict(kind="gpp", nb=512, nv=2, nc=32768, ng=1638),
    # gppKerSeq.cpp's half sum (gppsum = 1) at 512 x 2 x 32768 x 20; its inverted noflag mask keeps only
    # near-pole terms, which the uniform draw never produces, so wtilde comes from the branch-stress draw
    "gpphalf": dict(kind="gpp", nb=512, nv=2, nc=32768, ng=20, half=True, dist="branch"),
    # gppKer_real.cpp's real-valued sum at 512 x 2 x 32768 x 20; branch-stress wtilde so that the
    # reference program's carried noflag values (masked terms) occur
    "gppreal": dict(kind="gpp", nb=512, nv=2, nc=32768, ng=20, real=True, dist="branch"),
    # FF full-frequency contraction: 512 bands, ncouls 4096, ngpown 512, 15 frequencies
    "ff": dict(kind="ff", nb=512, nv=2, nc=4096, ng=512, nf=15, ne=10),
    # large FF contraction: 2048 bands, ncouls 8192, ngpown 4096, 32 frequencies (I_epsR/I_epsA ~17 GB each, drawn on the GPU)
    "ff4": dict(kind="ff", nb=2048, nv=2, nc=8192, ng=4096, nf=32, ne=10, device_inputs=True),
    # the FF shape whose (band, frequency, evaluation frequency) epilogue dominates
    # (ffkernel.deslippe.best.f90's compute-bound example 8 2 1000 60 20000 30000)
    "ffsigma": dict(kind="ff", nb=8, nv=2, nc=1000, ng=60, nf=20000, ne=30000, device_inputs=True),
    # a served, uneven GPP request stream: 256 requests of 128-1024 bands, ncouls 2048-32768
    "serve": dict(kind="serve", requests=256, nb_choices=(128, 256, 512, 1024), nc_lo=2048, nc_hi=32768,
                  nc_levels=8, nv=2, load=0.8),
}


def terms(w):
    if w["kind"] == "gpp" and w.get("half"):
        # the (n1, igp, ig, iw) the half sum visits: ig < igp for the evenly spread columns igp = i*ncouls/ngpown
        return w["nb"] * 3 * sum(i * w["nc"] // w["ng"] for i in range(w["ng"]))
    if w["kind"] == "gpp":
        return w["nb"] * w["ng"] * w["nc"] * 3
    return w["nb"] * w["ng"] * w["nc"] * w["nf"]


def algorithmic(w):
    """(bytes, flops) of the dominant contraction kernel over one call (the
    half sum launches it twice, once per A operand)."""
    if w["kind"] == "gpp" and w.get("real"):
        # FP64 reals of aqsntemp once, the operand at 4 B per real; a real MAC is 2 flops
        M, N, K = w["nb"] - w["nv"], 3 * w["ng"], w["nc"]
        return 8 * M * K + 4 * N * K, 2 * M * N * K
    if w["kind"] == "gpp":
        # the mixed full sum contracts every band (the occupied bands' sch terms too);
        # the half sum the bands n1 >= nvband, twice
        M = w["nb"] - w["nv"] if w.get("half") else w["nb"]
        N, K = 3 * w["ng"], w["nc"]
        n = 2 if w.get("half") else 1
        return n * (16 * M * K + 8 * N * K), n * 8 * M * N * K
    return 16 * w["nb"] * w["nc"] + 16 * w["nf"] * w["ng"] * w["nc"], 8 * w["nf"] * w["nb"] * w["ng"] * w["nc"]


def piece_products(w):
    """Tensor-core products per complex multiply-add of the mixed path: GPP's
    BF16 hi/mid/lo pieces six, FF's FP16 hi/lo pieces three."""
    return 3 if w["kind"] == "ff" else 6


def roofline(w, prec, byts, flops, kms, launches, peaks):
    """Roofline block for the dominant kernel (the contraction).  kms is its
    device time over one call, summed over its launches (CUDA events the
    library records on its stream right around each launch); byts/flops are
    the algorithmic work of those launches, so achieved = work / time is the
    launch-weighted average rate.  The bound is the higher floor: algorithmic
    bytes at the copy peak (GPP at small ngpown), or algorithmic flops, which
    the emulation executes as piece_products(w) products each (GPP 6, FF 3),
    at the bf16 peak (FF; GPP at large ngpown).  A tensor-bound frac is
    algorithmic flops over the bf16 peak, so 1/piece_products is the
    emulation's ceiling."""
    t = kms * 1e-3 if kms and kms > 0 else None
    common = {"kernel": "contraction", "algorithmic_bytes": byts, "algorithmic_flops": flops,
              "traffic": measured_traffic(w) if prec == "mixed" else None,
              "launches_per_call": launches, "duration_ms": kms / launches if kms and launches else None}
    # the bound is whichever floor is higher: the algorithmic bytes at the copy peak, or the
    # executed piece products at the bf16 peak
    npp = piece_products(w)
    hbm_floor = byts / (peaks.get("hbm_gbs", 6800.0) * 1e9)
    tensor_floor = npp * flops / (peaks.get("bf16_tflops", 1900.0) * 1e12)
    if prec == "mixed" and tensor_floor > hbm_floor:
        peak = peaks.get("bf16_tflops", 1900.0)
        ach = flops / t / 1e12 if t else None
        return dict(common, bound="tensor", achieved=ach, peak=peak, unit="TFLOP/s", frac=ach / peak if ach else None,
                    executed_tensor_tflops=npp * ach if ach else None, piece_products=npp,
                    peak_source="measured bf16_tflops (burst)" if "bf16_tflops" in peaks else "fallback")
    peak = peaks.get("hbm_gbs", 6800.0)
    ach = byts / t / 1e9 if t else None
    return dict(common, bound="hbm", achieved=ach, peak=peak, unit="GB/s", frac=ach / peak if ach else None,
                achieved_tflops=flops / t / 1e12 if t else None,
                peak_source="measured hbm_gbs" if "hbm_gbs" in peaks else "fallback")


def make_inputs(fk, w, seed=2024):
    if w["kind"] == "gpp" and w.get("real"):
        return fk.inputs.gpp_real_synthetic(w["nb"], w["nv"], w["nc"], w["ng"], seed=seed, dist=w.get("dist", "uniform"),
                                            index="even", wx="e10")
    if w["kind"] == "gpp":
        return fk.inputs.gpp_synthetic(w["nb"], w["nv"], w["nc"], w["ng"], seed=seed, dist=w.get("dist", "uniform"),
                                       index="even", wx="e10")
    if w.get("device_inputs"):
        return fk.inputs.ff_synthetic_device(w["nb"], w["nv"], w["nc"], w["ng"], w["nf"], w["ne"], seed=seed)
    return fk.inputs.ff_synthetic(w["nb"], w["nv"], w["nc"], w["ng"], w["nf"], w["ne"], seed=seed)


def to_np(v):
    """numpy view of an input array (torch tensors are copied to the host)."""
    if type(v).__module__.startswith("torch"):
        return v.detach().cpu().numpy()
    return v


class ClockSampler:
    """nvidia-smi samples (200 ms) of SM clock and throttle reasons."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index, self.rows, self.proc = index, [], None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm = [float(r[0]) for r in self.rows if r and r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if len(r) > 1 and r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if len(r) > 3 + i and r[3 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(sm)}


class NvmlSampler:
    """SM clock, power and clock-event reasons read through NVML
    (libnvidia-ml, by ctypes) every ~0.5 ms while the timed region runs."""
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown",
               0x80: "hw_power_brake_slowdown"}

    def __init__(self, cuda_index=0):
        import ctypes
        self.ct = ctypes
        self.lib = ctypes.CDLL("libnvidia-ml.so.1")
        if self.lib.nvmlInit_v2() != 0:
            raise OSError("nvmlInit failed")
        self.h = ctypes.c_void_p()
        ok = False
        try:
            import torch
            pr = torch.cuda.get_device_properties(cuda_index)
            bus = "%08x:%02x:%02x.0" % (pr.pci_domain_id, pr.pci_bus_id, pr.pci_device_id)
            ok = self.lib.nvmlDeviceGetHandleByPciBusId_v2(bus.encode(), ctypes.byref(self.h)) == 0
        except Exception:
            ok = False
        if not ok and self.lib.nvmlDeviceGetHandleByIndex_v2(cuda_index, ctypes.byref(self.h)) != 0:
            raise OSError("no NVML handle")
        self.rows, self.stop = [], threading.Event()
        v = ctypes.c_uint()
        self.max_mhz = float(v.value) if self.lib.nvmlDeviceGetMaxClockInfo(self.h, 1, ctypes.byref(v)) == 0 else None

    def _read(self):
        ct, L = self.ct, self.lib
        clk, pw, rs = ct.c_uint(), ct.c_uint(), ct.c_ulonglong()
        if L.nvmlDeviceGetClockInfo(self.h, 1, ct.byref(clk)) == 0:
            L.nvmlDeviceGetPowerUsage(self.h, ct.byref(pw))
            r = rs.value if L.nvmlDeviceGetCurrentClocksEventReasons(self.h, ct.byref(rs)) == 0 else 0
            self.rows.append((float(clk.value), pw.value / 1000.0, r))

    def _sample(self):
        while not self.stop.is_set():
            self._read()
            time.sleep(0.0005)

    def __enter__(self):
        # one reading as the region starts and one as it ends, so that even a
        # region of a few milliseconds is bracketed; the thread reads in between
        self._read()
        self.t = threading.Thread(target=self._sample, daemon=True)
        self.t.start()
        return self

    def __exit__(self, *a):
        self._read()
        self.stop.set()
        self.t.join(timeout=2)

    def summary(self):
        sm = [r[0] for r in self.rows]
        bits = 0
        for r in self.rows:
            bits |= r[2]
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": self.max_mhz,
                "reasons": sorted(n for b, n in self.REASONS.items() if bits & b),
                "power_w_median": statistics.median(r[1] for r in self.rows) if self.rows else None,
                "samples": len(sm), "source": "nvml"}


def clock_sampler(index):
    try:
        return NvmlSampler(index)
    except (OSError, AttributeError):
        return ClockSampler(index)


def load_peaks():
    """The measured HBM copy and bf16 peaks of this GPU type (MEASURED_PEAKS.json), or {}."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def serve_roofline(reqs, nv, seconds, steps, peaks):
    """Roofline block of a served stream: the algorithmic work of every
    request's contraction (bands nvband .. nb-1 against 3 * ngpown columns over
    ncouls, ngpown = ncouls / 64; bytes: aqsntemp's rows once at 16 B and the
    image at 8 B per complex, flops: 8 per complex multiply-add) over
    `seconds`, the burst's wall time for `steps` steps.  That time holds every
    kernel of the steps (index map, prep, A images, reductions) and the host's
    gaps between steps, so `achieved` is a lower bound on the table
    contraction's own rate."""
    byts = flops = 0
    for nb, nc in reqs:
        M, N, K = nb - nv, 3 * (nc // 64), nc
        byts += 16 * M * K + 8 * N * K
        flops += 8 * M * N * K
    r = roofline({"kind": "gpp", "name": "serve"}, "mixed", byts, flops, seconds * 1e3, max(1, steps), peaks)
    r["kernel"] = "table contraction (the stream's steps)"
    r["basis"] = ("algorithmic work of the stream's contractions over the burst's wall time (every kernel and "
                  "host gap of its steps): a lower bound on the contraction's own rate")
    return r


def measured_traffic(w):
    """DRAM bytes per launch of the dominant kernel from a committed ncu
    capture summary (profiles/traffic.json), or None."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            t = json.load(f)
        return t.get(w["name"], {}).get("dram_bytes_per_launch")
    except (OSError, ValueError):
        return None


def max_over_ranks(x: float, device=None) -> float:
    """The largest of every rank's x (x itself when not distributed).  The
    ranks are independent replicas (no data-path collective): this and the
    barriers around the timed region are the only cross-rank communication."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return x
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(world: int, units_per_rank: float, seconds: float) -> float:
    """Whole-job throughput: the units every rank processed over the slowest rank's time."""
    return world * units_per_rank / seconds


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


REF_GPP = os.path.join(ROOT, "oracle", "_ref", "gppKer_bgw")


def reference_gpp_binary(w, runs, warmup=1):
    """Seconds per run of the reference's own GPP driver, BGW-Kernels/gppKer.cpp
    built unmodified from its sources (oracle/Makefile, target ref), as its own
    chrono line reports them (the loop nest alone, :301,441-446), on all host
    cores: `gppKer_bgw nb nvband ncouls nodes_per_group`, nodes_per_group =
    ncouls / ngpown so that the program's ngpown (:175-176) is the workload's.
    None when the binary was not built on this machine or the shape cannot be
    expressed that way.  The program fills its own constant inputs."""
    if w["kind"] != "gpp" or w.get("half") or w.get("real") or not os.access(REF_GPP, os.X_OK):
        return None
    npg = w["nc"] // w["ng"]
    if npg < 1 or w["nc"] // npg != w["ng"]:
        return None
    cores = os.cpu_count() or 1
    env = dict(os.environ, OMP_NUM_THREADS=str(cores))
    times = []
    for i in range(warmup + runs):
        out = subprocess.run([REF_GPP, str(w["nb"]), str(w["nv"]), str(w["nc"]), str(npg)], capture_output=True,
                             text=True, env=env, timeout=600)
        if out.returncode != 0:
            return None
        t = [float(x.split("=")[1].split()[0]) for x in out.stdout.splitlines() if "Chrono Time Taken" in x]
        if not t:
            return None
        if i >= warmup:
            times.append(t[0])
    return {"times": times, "cores": cores, "args": [w["nb"], w["nv"], w["nc"], npg]}


REF_FF = os.path.join(ROOT, "oracle", "_ref", "ffKernel")


def reference_ff_binary(w, runs=2, warmup=1):
    """Seconds per run of the reference's own FF driver, FFKer_cori/ffKernel.cpp
    built unmodified from its sources (oracle/Makefile, target ref), as its own
    "Total Kernel Time" line reports them (its four kernels, :478-513), on all
    host cores: `ffKernel nb nvband ncouls ngpown nFreq nfreqeval`, its own
    constant inputs.  That program has no band x G x G' contraction (its
    schDt_matrix is filled with a constant, :386,422, and only read by
    achDtemp_Kernel): it computes achsDtemp, asxDtemp,
    achDtemp and achDtemp_cor, a subset of the workload's outputs, so its time
    is reported beside the library's call, not as the workload's rate.  None
    when the binary was not built on this machine, the run fails, or the shape
    would hold more than 4 GB of epsilon planes in host memory."""
    if w["kind"] != "ff" or not os.access(REF_FF, os.X_OK):
        return None
    if 2 * w["nf"] * w["ng"] * w["nc"] * 16 > 4e9 or w["ng"] > w["nc"]:
        return None
    cores = os.cpu_count() or 1
    env = dict(os.environ, OMP_NUM_THREADS=str(cores))
    args = [w["nb"], w["nv"], w["nc"], w["ng"], w["nf"], w["ne"]]
    times = []
    try:
        for i in range(warmup + runs):
            out = subprocess.run([REF_FF] + [str(x) for x in args], capture_output=True, text=True, env=env,
                                 timeout=300)
            t = [float(x.split("=")[1].split()[0]) for x in out.stdout.splitlines() if "Total Kernel Time" in x]
            if out.returncode != 0 or not t:
                return None
            if i >= warmup:
                times.append(t[0])
    except (OSError, ValueError, IndexError, subprocess.TimeoutExpired):
        return None
    return {"kernel_s": statistics.mean(times), "runs": len(times), "cores": cores, "args": args,
            "program": "FFKer_cori/ffKernel.cpp built unmodified (g++ -O3 -fopenmp), its constant inputs",
            "computes": "achsDtemp, asxDtemp, achDtemp, achDtemp_cor, without the band x G x G' contraction "
                        "that the library's call also performs (the program fills schDt_matrix with a constant)"}


def run_reference(a, w):
    """The reference's own CPU implementation of the path on all host cores:
    its GPP driver when it was built here (reference_gpp_binary), else the CPU
    restatement of its loop nest (oracle/)."""
    world, rank, _ = dist_setup()
    if rank != 0:
        return
    ref = reference_gpp_binary(w, a.steps, warmup=a.warmup)
    if ref is not None:
        times = ref["times"]
        tot = sum(times)
        val = terms(w) * len(times) / tot
        sample = ("the reference's GPP driver BGW-Kernels/gppKer.cpp built unmodified with g++ -O3 -fopenmp, "
                  "`gppKer %s` (ngpown %d), its own constant inputs, its own chrono time of the loop nest; "
                  "one full run (%.3g terms) per step, OpenMP %d threads"
                  % (" ".join(map(str, ref["args"])), w["ng"], terms(w), ref["cores"]))
        print(json.dumps({
            "impl": "reference", "metric": METRIC, "value": val, "unit": "terms/s", "n_gpus": a.gpus,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": 1e3 * tot / len(times), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "the reference driver's constant inputs",
            "config": workload_config(a, w),
            "cpu_baseline": {"value": val, "unit": "terms/s", "cores": ref["cores"], "kind": "reference",
                             "sample": sample},
            "e2e": {"value": val, "unit": "terms/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "latency_ms": {"p50": 1e3 * statistics.median(times), "p99": 1e3 * float(np.percentile(times, 99))},
        }), flush=True)
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    import __graft_entry__
    fk = __graft_entry__.load_package()
    cores = os.cpu_count() or 1
    if w["kind"] == "serve":
        # the stream's requests in order, those under 2e9 terms (about a
        # second each on the host), until ~20 s of CPU work per step
        levels, reqs, _ = serve_stream(w)
        small = [(nb, nc) for nb, nc in reqs if 3.0 * nb * nc * (nc // 64) <= 2e9]
        times, done_terms, i = [], [], 0
        for _ in range(a.warmup + a.steps):
            t0 = time.perf_counter()
            tt = 0.0
            while time.perf_counter() - t0 < 20.0 / (a.warmup + a.steps):
                nb, nc = small[i % len(small)]
                i += 1
                oracle.gpp(fk.inputs.gpp_synthetic(nb, w["nv"], nc, nc // 64, seed=i), nthreads=cores)
                tt += 3.0 * nb * nc * (nc // 64)
            times.append(time.perf_counter() - t0)
            done_terms.append(tt)
        times, done_terms = times[a.warmup:], done_terms[a.warmup:]
        val = sum(done_terms) / sum(times)
        sample = (f"the stream's requests of <= 2e9 terms ({len(small)} of {len(reqs)}), in order, "
                  f"one after another, OpenMP {cores} threads; input generation included")
        print(json.dumps({
            "impl": "reference", "metric": METRIC, "value": val, "unit": "terms/s", "n_gpus": a.gpus,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "served GPP stream (CPU: sequential)", "ncouls_levels": levels},
            "cpu_baseline": {"value": val, "unit": "terms/s", "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": val, "unit": "terms/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }), flush=True)
        return
    if w.get("device_inputs"):
        # the 2048 x 8192 x 4096 x 32 contraction is far too large for the host cores: a bounded sample of it
        # (8 bands, 2 frequency planes, full ncouls x ngpown) per step
        w = dict(w, nb=8, nf=2)
        p = fk.inputs.ff_synthetic(w["nb"], w["nv"], w["nc"], w["ng"], w["nf"], w["ne"], seed=2024)
    else:
        p = make_inputs(fk, w)
    gflags = oracle.ORC_GPP_HALF_SUM if w.get("half") else 0
    call = (lambda: oracle.gpp_real(p, nthreads=cores)) if w.get("real") else \
        (lambda: oracle.gpp(p, flags=gflags, nthreads=cores)) if w["kind"] == "gpp" else \
        (lambda: oracle.ff(p, flags=oracle.ORC_FF_SCHDT_GEMM, nthreads=cores))
    for _ in range(a.warmup):
        call()
    times = []
    for _ in range(a.steps):
        t0 = time.perf_counter()
        call()
        times.append(time.perf_counter() - t0)
    tot = sum(times)
    val = terms(w) * a.steps / tot
    sample = (f"{'a sample of the workload: %d bands, %d frequencies' % (w['nb'], w['nf']) if w.get('device_inputs') else 'full workload'}"
              f" per step ({terms(w):.3g} terms), OpenMP {cores} threads")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": val, "unit": "terms/s", "n_gpus": a.gpus,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": 1e3 * tot / a.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(a, w),
        "cpu_baseline": {"value": val, "unit": "terms/s", "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": val, "unit": "terms/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "latency_ms": {"p50": 1e3 * statistics.median(times), "p99": 1e3 * float(np.percentile(times, 99))},
    }), flush=True)


METRIC = "GPP/FF self-energy terms/s + p99 latency, mixed vs FP64 at <=1e-6 rel err"


def workload_config(a, w):
    c = {"workload": ("GPP self-energy %s, number_bands=%d nvband=%d ncouls=%d ngpown=%d" %
                      ("half sum (gppsum=1)" if w.get("half") else "real-valued sum (gppKer_real)" if w.get("real")
                       else "sum", w["nb"], w["nv"], w["nc"], w["ng"]))
         if w["kind"] == "gpp" else
         ("FF full-frequency contraction, number_bands=%d nvband=%d ncouls=%d ngpown=%d nFreq=%d nfreqeval=%d"
          % (w["nb"], w["nv"], w["nc"], w["ng"], w["nf"], w["ne"])),
         "precision": a.precision, "parallelism": f"replicas x{a.gpus}",
         "l2": "inputs larger than L2 (aqsntemp %.0f MB)" % ((8 if w.get("real") else 16) * w["nb"] * w["nc"] / 1e6)}
    if w.get("dist"):
        c["distribution"] = w["dist"]
    return c


def timed(torch, stream, fn, steps, warmup, per_step=False):
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
    evs[0].record(stream)
    for i in range(steps):
        fn()
        if per_step:
            evs[i + 1].record(stream)
    if not per_step:
        evs[steps].record(stream)
    torch.cuda.synchronize()
    if per_step:
        return [evs[i].elapsed_time(evs[i + 1]) for i in range(steps)]
    return [evs[0].elapsed_time(evs[steps]) / steps] * steps


def rel(a, b):
    a, b = np.atleast_1d(np.asarray(a)), np.atleast_1d(np.asarray(b))
    d = float(np.max(np.abs(b)))
    return float(np.max(np.abs(a - b))) / d if d > 0 else float(np.max(np.abs(a)))


def measure_ours(a, w, fk, world, rank, local, sub=False):
    """One workload through the library on this rank's GPU; returns the JSON
    line's fields (rank 0) or None.  sub: a sub-block of the default line --
    fewer steps, the FP64 path run once (for its error and its time), no CPU
    baseline."""
    import torch
    steps = min(a.steps, w.get("sub_steps", 10)) if sub else a.steps
    ctx = fk.Context(local)
    stream = torch.cuda.Stream(local)
    ctx.set_stream(stream.cuda_stream)
    p = make_inputs(fk, w, seed=2024 + rank)
    keys_c = [k for k, v in p.items() if isinstance(v, np.ndarray)]
    d = dict(p)
    for k in keys_c:
        d[k] = torch.from_numpy(np.ascontiguousarray(p[k])).to(f"cuda:{local}")
    if w["kind"] == "gpp" and w.get("real"):
        outs = {k: torch.zeros(n, dtype=torch.float64, device=f"cuda:{local}")
                for k, n in (("achtemp", 3), ("asxtemp", 3), ("acht_n1_loc", w["nb"]))}
        flags = 0
        call = lambda prec: ctx.gpp_real(d, prec, flags, out=outs)
        host_call = lambda prec, hp: ctx.gpp_real(hp, prec, flags)
    elif w["kind"] == "gpp":
        outs = {k: torch.zeros(n, dtype=torch.complex128, device=f"cuda:{local}")
                for k, n in (("achtemp", 3), ("asxtemp", 3), ("acht_n1_loc", w["nb"]))}
        outs["achstemp"] = None
        flags = fk.FK_GPP_HALF_SUM if w.get("half") else 0
        call = lambda prec: ctx.gpp(d, prec, flags, out=outs)
        host_call = lambda prec, hp: ctx.gpp(hp, prec, flags)
    else:
        flags = fk.FK_FF_SCHDT_GEMM | fk.FK_FF_SPLIT_ACHD
        outs = {"achsDtemp": torch.zeros(1, dtype=torch.complex128, device=f"cuda:{local}"),
                "asxDtemp": torch.zeros(w["ne"], dtype=torch.complex128, device=f"cuda:{local}"),
                "achDtemp": torch.zeros(w["ne"], dtype=torch.complex128, device=f"cuda:{local}"),
                "achDtemp_cor": torch.zeros(w["ne"], dtype=torch.complex128, device=f"cuda:{local}"),
                "ach2Dtemp": torch.zeros(w["ne"], dtype=torch.complex128, device=f"cuda:{local}"),
                "schDt_matrix": torch.zeros((w["nb"], w["nf"]), dtype=torch.complex128, device=f"cuda:{local}")}
        call = lambda prec: ctx.ff(d, prec, flags, out=outs)
        host_call = lambda prec, hp: ctx.ff(hp, prec, flags)

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    # accuracy of the mixed path against FP64 (stated for every output)
    def fetch(r):
        torch.cuda.synchronize()
        return {k: (v.cpu().numpy().copy() if v is not None else None) for k, v in r.items()}

    prec = a.precision
    other = "fp64" if prec == "mixed" else "mixed"
    if sub:
        # the FP64 call once, timed by the library's own events
        ctx.set_profiling(True)
        ref64 = fetch(call("fp64"))
        ms_fp64 = sum(ctx.last_timings())
        ctx.set_profiling(False)
    else:
        ref64 = fetch(call("fp64"))
    resm = fetch(call("mixed"))
    errs = {k: rel(resm[k], ref64[k]) for k in ref64 if ref64[k] is not None and np.max(np.abs(ref64[k])) > 0}
    barrier()
    for _ in range(a.warmup):
        call(prec)
    barrier()
    with clock_sampler(local) as clk:
        barrier()
        torch.cuda.nvtx.range_push("timed")
        per = timed(torch, stream, lambda: call(prec), steps, 0, per_step=False)
        torch.cuda.nvtx.range_pop()
        barrier()
    ms = max_over_ranks(per[0], f"cuda:{local}")
    launches = ctx.last_launches()
    # per-step latency distribution (events around each call)
    lat = timed(torch, stream, lambda: call(prec), steps, 1, per_step=True)
    # the other precision, for the mixed-vs-FP64 ratio
    if sub and prec == "mixed":
        ms_other = ms_fp64
    else:
        k_other = max(3, min(steps, 10))
        ms_other = statistics.mean(timed(torch, stream, lambda: call(other), k_other, 1, per_step=True))
    # dominant-kernel duration from the library's events on its stream
    ctx.set_profiling(True)
    ph, kt = [], []
    for _ in range(max(3, min(steps, 10))):
        call(prec)
        ph.append(ctx.last_timings())
        kt.append(ctx.last_kernel_time())
    ctx.set_profiling(False)
    phase = [statistics.mean(x[i] for x in ph) for i in range(4)]
    kernel_ms = statistics.mean(x[0] for x in kt)
    kernel_launches = kt[-1][1]
    # end to end through the C ABI with pinned host buffers
    hp = dict(p)
    # arrays drawn on the GPU (the large FF workload) go through host memory like the others
    keys_h = keys_c + [k for k, v in p.items() if type(v).__module__.startswith("torch")]
    for k in keys_h:
        hp[k] = (p[k].cpu() if k not in keys_c else torch.from_numpy(np.ascontiguousarray(p[k]))).pin_memory()
    # as many warm-up calls as the device-resident timing (the first host calls grow the
    # context's workspace and pinned staging buffer)
    for _ in range(max(1, a.warmup)):
        host_call(prec, hp)
    # the bytes a call moves over the host link, as the library counts them: a
    # host array in full, except the parts the call reads (the igp columns of
    # aqsmtemp, the FF frequency planes the request needs)
    h2d, d2h = ctx.last_transfer()
    barrier()
    # each call timed on its own (host outputs: the call returns after its results
    # are on the host); the median is the line's e2e, the mean is reported beside it
    ke = 5 if sub else max(3, min(steps, 10))
    e2e_calls = []
    for _ in range(ke):
        t0 = time.perf_counter()
        host_call(prec, hp)
        torch.cuda.synchronize()
        e2e_calls.append(time.perf_counter() - t0)
    e2e_s = max_over_ranks(statistics.median(e2e_calls), f"cuda:{local}")
    e2e_mean_s = max_over_ranks(statistics.mean(e2e_calls), f"cuda:{local}")
    cpu = None
    if rank == 0 and world == 1 and not a.no_cpu and not sub:
        cpu = cpu_baseline(fk, w, p)
    ctx.close()
    del d, hp, outs, p
    torch.cuda.empty_cache()
    # FF: the reference's own FF program on the host cores, beside the call (a subset of its outputs)
    refprog = reference_ff_binary(w) if rank == 0 and world == 1 and not a.no_cpu else None
    if rank != 0:
        return None
    peaks = load_peaks()
    byts, flops = algorithmic(w)
    T = terms(w)
    line = {
        "metric": METRIC, "value": job_value(world, T, ms * 1e-3), "unit": "terms/s", "n_gpus": world,
        "steps": steps, "warmup": a.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64 in / fp32 bulk + fp64 branch/reductions" if prec == "mixed" else "f64",
        "data": "synthetic (seeded, benchmark value distributions)", "config": workload_config(a, w),
        "precision": prec,
        "fp64_value" if prec == "mixed" else "mixed_value": job_value(world, T, ms_other * 1e-3),
        "mixed_vs_fp64": (ms_other / ms) if prec == "mixed" else (ms / ms_other),
        "rel_err_mixed_vs_fp64": errs,
        "latency_ms": {"p50": statistics.median(lat), "p99": float(np.percentile(lat, 99))},
        "phase_ms": {"staging": phase[0], "prep": phase[1], "contraction": phase[2], "reduction": phase[3]},
        "roofline": roofline(w, prec, byts, flops, kernel_ms, kernel_launches, peaks),
        "e2e": {"value": job_value(world, T, e2e_s), "unit": "terms/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": e2e_s * 1e3, "calls": len(e2e_calls),
                "statistic": "median of per-call times", "mean_ms_per_step": e2e_mean_s * 1e3,
                "calls_ms": [round(x * 1e3, 4) for x in e2e_calls]},
        "gpu_launches": launches * steps,
        "clocks": clk.summary(),
    }
    if cpu:
        line["cpu_baseline"] = cpu
    if refprog:
        line["reference_program"] = dict(refprog, call_ms=ms)
    return line


# The default line's sub-blocks: the metric's other workloads, each measured
# after the headline (GPP 512 x 2 x 32768 x 20) with a few steps.
SUB_BLOCKS = ("gpp1638", "ff", "serve", "ff4")


def run_ours(a, w):
    import torch
    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    import __graft_entry__
    fk = __graft_entry__.load_package()
    line = measure_ours(a, w, fk, world, rank, local)
    # the default workload carries the metric's other configurations as
    # sub-blocks of the same line (one GPU: the replicas run only the headline)
    if line is not None and world == 1 and a.workload == "gpp" and not a.headline_only:
        for name in SUB_BLOCKS:
            sw = dict(WORKLOADS[name], name=name)
            t0 = time.perf_counter()
            blk = measure_serve(a, sw, fk, sub=True) if sw["kind"] == "serve" else \
                measure_ours(a, sw, fk, world, rank, local, sub=True)
            for k in ("metric", "n_gpus", "higher_is_better", "scaling", "vs_baseline", "data", "warmup"):
                blk.pop(k, None)
            blk["wall_s"] = time.perf_counter() - t0
            line[name] = blk
    if line is not None:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def cpu_baseline(fk, w, p):
    """The reference's own GPP driver on the host cores when it was built here
    (kind "reference"; the CPU restatement's rate beside it), else the CPU
    restatement of the reference loop nest (oracle/, kind "port"), on a
    bounded sample of the same workload."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    cores = os.cpu_count() or 1
    if w["kind"] == "gpp":
        t0 = time.perf_counter()
        if w.get("real"):
            oracle.gpp_real(p, nthreads=cores)
        else:
            oracle.gpp(p, flags=oracle.ORC_GPP_HALF_SUM if w.get("half") else 0, nthreads=cores)
        dt = time.perf_counter() - t0
        port = {"value": terms(w) / dt, "unit": "terms/s", "cores": cores, "kind": "port",
                "sample": f"one full call of the CPU restatement on the seeded inputs ({terms(w):.3g} terms)"}
        ref = reference_gpp_binary(w, runs=3)
        if ref is None:
            return port
        return {"value": terms(w) * len(ref["times"]) / sum(ref["times"]), "unit": "terms/s", "cores": ref["cores"],
                "kind": "reference",
                "sample": ("the reference's GPP driver BGW-Kernels/gppKer.cpp built unmodified (g++ -O3 -fopenmp), "
                           "`gppKer %s`, its constant inputs, its chrono time of the loop nest, mean of %d runs "
                           "(%.3g terms each)" % (" ".join(map(str, ref["args"])), len(ref["times"]), terms(w))),
                "port_value": port["value"], "port_sample": port["sample"]}
    q = dict(p)
    big = w["ng"] * w["nc"] * w["nf"] > 1e9
    nbs, nfs = (8, 4) if big else (64, w["nf"])
    for k in ("aqsmtemp", "aqsntemp"):
        q[k] = np.ascontiguousarray(to_np(p[k][:nbs]))
    for k in ("I_epsR_array", "I_epsA_array"):
        q[k] = np.ascontiguousarray(to_np(p[k][:nfs]))
    for k in ("dFreqGrid", "dFreqBrd", "pref"):
        q[k] = np.ascontiguousarray(p[k][:nfs])
    q["ekq"] = p["ekq"][:nbs]
    q["number_bands"], q["nFreq"] = nbs, nfs
    t0 = time.perf_counter()
    oracle.ff(q, flags=oracle.ORC_FF_SCHDT_GEMM, nthreads=cores)
    dt = time.perf_counter() - t0
    tq = nbs * w["ng"] * w["nc"] * nfs
    return {"value": tq / dt, "unit": "terms/s", "cores": cores, "kind": "port",
            "sample": f"first {nbs} of {w['nb']} bands, {nfs} of {w['nf']} frequencies ({tq:.3g} terms)"}


def serve_stream(w, seed=2024):
    """ncouls levels (log-spaced over [nc_lo, nc_hi], multiples of 64), and per
    request (number_bands, ncouls) plus a unit-rate exponential gap."""
    rng = np.random.default_rng(seed)
    L = w["nc_levels"]
    levels = sorted({int(round(w["nc_lo"] * (w["nc_hi"] / w["nc_lo"]) ** (i / (L - 1)) / 64)) * 64 for i in range(L)})
    reqs = [(int(rng.choice(w["nb_choices"])), int(rng.choice(levels))) for _ in range(w["requests"])]
    return levels, reqs, rng.exponential(1.0, w["requests"])


def measure_serve(a, w, fk, sub=False):
    """The served GPP stream: the request server (fk_server_*) on a stream of
    GPP requests of uneven size.  First a burst (all requests at once:
    saturation throughput), then Poisson arrivals at `load` x that rate
    (latency).  Returns the line's fields (rank 0) or None."""
    import torch
    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    levels, reqs, gaps = serve_stream(w, seed=2024 + rank)
    srv = fk.Server(local, hbm_bytes=24 << 30, max_active=32)
    pools = {}
    for i, nc in enumerate(levels):
        ng = nc // 64
        gen = torch.Generator(device=f"cuda:{local}").manual_seed(1000 * (rank + 1) + i)

        def cu(shape):
            x = torch.rand(shape + (2,), generator=gen, device=f"cuda:{local}", dtype=torch.float64) - 0.5
            return torch.view_as_complex(x).contiguous()
        aqsm, aqsn, eps = cu((1024, nc)), cu((1024, nc)), cu((ng, nc))
        wre = torch.rand((ng, nc), generator=gen, device=f"cuda:{local}", dtype=torch.float64) * 1.5 + 0.5
        wim = (torch.rand((ng, nc), generator=gen, device=f"cuda:{local}", dtype=torch.float64) - 0.5) * 0.1
        wt = torch.complex(wre, wim).contiguous()
        srv.resident_put(2 * i + 1, eps)
        srv.resident_put(2 * i + 2, wt)
        del eps, wt
        r = np.random.default_rng(i)
        pools[nc] = dict(key=i, aqsm=aqsm, aqsn=aqsn, vcoul=r.uniform(0.1, 1.0, nc),
                         inv=np.array([j * nc // ng for j in range(ng)], np.int32), indinv=np.arange(nc, dtype=np.int32))
    wx = np.array([9.0, 10.0, 11.0])

    def submit(nb, nc):
        q = pools[nc]
        p = {"number_bands": nb, "nvband": w["nv"], "ncouls": nc, "ngpown": nc // 64, "aqsmtemp": q["aqsm"][:nb],
             "aqsntemp": q["aqsn"][:nb], "vcoul": q["vcoul"], "inv_igp_index": q["inv"], "indinv": q["indinv"],
             "wx_array": wx}
        return srv.submit(p, eps_key=2 * q["key"] + 1, wtilde_key=2 * q["key"] + 2)

    def terms_of(nb, nc):
        return 3.0 * nb * nc * (nc // 64)

    # autotuned plans for every request shape of the stream, then a warm-up
    shapes = sorted(set(reqs))
    tuned = {f"{nb}x{nc}": srv.tune(nb, w["nv"], nc, nc // 64) for nb, nc in shapes}
    for _ in range(max(1, a.warmup // 3)):
        for t in [submit(128, nc) for nc in levels]:
            srv.wait(t)
    total = sum(terms_of(nb, nc) for nb, nc in reqs)
    steps_before = srv.stats()["steps"]
    # burst: saturation throughput
    with clock_sampler(local) as clk:
        t0 = time.perf_counter()
        tickets = [submit(nb, nc) for nb, nc in reqs]
        for t in tickets:
            srv.wait(t)
        burst_s = time.perf_counter() - t0
    sat = total / burst_s
    steps0 = srv.stats()["steps"] - steps_before
    # Poisson arrivals at `load` x saturation
    rate = w["load"] * sat / (total / len(reqs))
    arrivals = np.cumsum(gaps / rate)
    lat = []
    t0 = time.perf_counter()
    tickets = []
    for (nb, nc), at in zip(reqs, arrivals):
        dt = at - (time.perf_counter() - t0)
        if dt > 0:
            time.sleep(dt)
        tickets.append(submit(nb, nc))
    for t in tickets:
        lat.append(srv.wait(t)[1])
    pois_s = time.perf_counter() - t0
    info = srv.stats()
    srv.close()
    pools.clear()
    torch.cuda.empty_cache()
    cpu = None
    if rank == 0 and not a.no_cpu and not sub:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle
        cores = os.cpu_count() or 1
        q = fk.inputs.gpp_synthetic(128, 2, 2048, 32, seed=5)
        t1 = time.perf_counter()
        n = 0
        while time.perf_counter() - t1 < 5.0:
            oracle.gpp(q, nthreads=cores)
            n += 1
        dt = time.perf_counter() - t1
        cpu = {"value": n * terms_of(128, 2048) / dt, "unit": "terms/s", "cores": cores, "kind": "port",
               "sample": f"{n} calls of the smallest request shape (128 x 2048 x 32), ~5 s"}
    if rank == 0:
        line = {
            "metric": METRIC, "value": world * sat, "unit": "terms/s", "n_gpus": world, "steps": len(reqs),
            "warmup": a.warmup, "ms_per_step": 1e3 * burst_s / len(reqs), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64 in / fp32 bulk + fp64 branch/reductions",
            "data": "synthetic (seeded; wavefunction pools and epsilon/wtilde resident on the device)",
            "config": {"workload": ("served GPP stream: %d requests, number_bands in %s, ncouls in %d log-spaced "
                                    "levels over [%d, %d], ngpown = ncouls/64, nvband = %d; burst for throughput, "
                                    "then Poisson arrivals at %.0f%% of it for latency"
                                    % (len(reqs), list(w["nb_choices"]), len(levels), w["nc_lo"], w["nc_hi"],
                                       w["nv"], 100 * w["load"])),
                       "precision": "mixed", "parallelism": f"replicas x{world}",
                       "l2": "inputs larger than L2 (pools of several GB)", "ncouls_levels": levels},
            "precision": "mixed",
            "latency_ms": {"p50": 1e3 * float(np.percentile(lat, 50)), "p99": 1e3 * float(np.percentile(lat, 99)),
                           "mean": 1e3 * float(np.mean(lat)), "arrival_rate_per_s": rate},
            "served": {"burst_s": burst_s, "poisson_s": pois_s, "poisson_terms_per_s": total / pois_s,
                       "steps_burst": steps0, "steps_total": info["steps"],
                       "mean_requests_per_step": info["mean_active"], "peak_active": info["peak_active"],
                       "hbm_peak_bytes": info["hbm_peak_bytes"], "autotuned_kslices": tuned},
            "roofline": serve_roofline(reqs, w["nv"], burst_s, steps0, load_peaks()),
            "e2e": {"value": world * sat, "unit": "terms/s", "h2d_bytes_per_step": None, "d2h_bytes_per_step": None,
                    "note": "requests through fk_server_submit/fk_server_wait; outputs returned to host"},
            "gpu_launches": 5 * info["steps"],
            "clocks": clk.summary(),
        }
        if cpu:
            line["cpu_baseline"] = cpu
        return line
    return None


def run_serve(a, w):
    import __graft_entry__
    line = measure_serve(a, w, __graft_entry__.load_package())
    if line is not None:
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="gpp", choices=sorted(WORKLOADS))
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--headline-only", action="store_true",
                    help="default workload: skip the sub-blocks of the metric's other configurations")
    a = ap.parse_args()
    a.warmup = max(a.warmup, 3)
    w = dict(WORKLOADS[a.workload], name=a.workload)
    if a.impl == "reference":
        run_reference(a, w)
    elif w["kind"] == "serve":
        run_serve(a, w)
    else:
        run_ours(a, w)


if __name__ == "__main__":
    main()
