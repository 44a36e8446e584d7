"""Regenerate the golden fixtures of tests/golden/ from the reference.

Needs the reference tree, named by the FK_REFERENCE_DIR environment variable
(its drivers and harnesses are compiled into oracle/_ref/ by
`make -C oracle ref-src ref`).  It runs:
  * the unmodified reference drivers (BGW-Kernels/gppKer.cpp, repo-root
    gppKer.cpp, gppKer_orig.cpp, gppKerSeq.cpp, gppKer_real.cpp,
    FFKer_cori/ffKernel.cpp) with their own constant inputs, recording what
    they print;
  * the harnesses that call the reference's own solver functions
    (oracle/ref_harness_gpp.cpp, oracle/ref_harness_gpp_real.cpp,
    oracle/ref_harness_ff.cpp) on small seeded random inputs, stored together
    with the inputs.
The oracle and the CUDA library are then checked against these files on any
machine, without the reference.

usage: python tests/golden/make_golden.py [--big]
  --big also runs gppKer 512 2 32768 20 (about two minutes on 8 cores).
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
import __graft_entry__  # noqa: E402

inputs = __graft_entry__.load_package().inputs

GPP_SIZES = [(64, 2, 512, 4), (32, 2, 1000, 8), (128, 4, 777, 7), (512, 2, 2048, 32), (40, 0, 600, 6),
             (24, 24, 256, 4)]
FF_SIZES = [(16, 3, 300, 40, 6, 7), (64, 2, 512, 64, 15, 10), (512, 2, 4096, 512, 15, 10)]
SEQ_SIZES = [(64, 2, 1024, 4, 1), (32, 3, 2048, 8, 1), (16, 2, 1536, 6, 1)]
REAL_SIZES = [(64, 2, 1024, 4), (512, 2, 2048, 32), (33, 5, 1000, 10), (40, 0, 777, 7)]


def cx(z):
    return [z.real, z.imag]


def exact_constant_gpp(nb, nv, nc, npg):
    """Closed form of achtemp for the reference programs' constant inputs (every array
    0.5+0.5i, vcoul = 1, wx = {3,4,5}): all (n1, igp, ig) terms are equal and
    take the first branch, so achtemp[iw] = nb*ngpown*0.5*nc*t(iw) exactly
    (rational arithmetic)."""
    from fractions import Fraction as F
    h = F(1, 2)

    def mul(a, b):
        return (a[0] * b[0] - a[1] * b[1], a[0] * b[1] + a[1] * b[0])

    ng = nc // npg
    out = []
    for wx in (F(3), F(4), F(5)):
        wd = (wx - h, -h)
        r = wd[0] ** 2 + wd[1] ** 2
        d = mul((h, h), (wd[0], -wd[1]))
        t = mul(mul(mul((h, -h), (h, h)), (d[0] / r, d[1] / r)), (h, h))
        out.append([float(t[0] * h * nc * nb * ng), float(t[1] * h * nc * nb * ng)])
    return out


def exact_constant_gpp_real(nb, nv, nc, npg):
    """Closed form of the real-valued driver's achtemp (every array 0.5,
    vcoul = 1, wx = {3,4,5}): every term takes the first branch, so
    achtemp[iw] = nb*ngpown*nc*delw(iw)/16 with delw = 0.5/(wx - 0.5)."""
    from fractions import Fraction as F
    ng = nc // npg
    return [float(F(nb * ng * nc, 16) * F(1, 2) / (wx - F(1, 2))) for wx in (F(3), F(4), F(5))]


def real_fixtures(out: dict) -> None:
    """gppKer_real.cpp: its driver's prints and its own flagOCC_solver on seeded inputs."""
    out["gppKer_real"] = []
    for s in REAL_SIZES:
        r = oracle.run_ref_driver("gppKer_real", s, threads=1)
        out["gppKer_real"].append({"args": list(s), "achtemp": [r[f"achtemp[{i}]"] for i in range(3)],
                                   "achtemp_exact": exact_constant_gpp_real(*s)})
    p = inputs.gpp_real_synthetic(7, 3, 700, 5, seed=11, dist="branch", index="reference", wx="stress")
    inv, nc = p["inv_igp_index"], p["ncouls"]
    igp = np.array([nc - 1 if i == nc else p["indinv"][i] for i in inv], np.int32)
    h = oracle.ref_gpp_real_pairs(p, igp)
    np.savez_compressed(os.path.join(HERE, "gpp_real_pairs.npz"), sch=h["sch"], ssx=h["ssx"],
                        **{k: np.asarray(v) for k, v in p.items()})


def main(big: bool):
    oracle.build()
    out = {"gppKer_bgw": [], "gppKer_root": [], "gppKer_orig": [], "ffKernel": []}
    sizes = GPP_SIZES + ([(512, 2, 32768, 20)] if big else [])
    for s in sizes:
        r = oracle.run_ref_driver("gppKer_bgw", s)
        out["gppKer_bgw"].append({"args": list(s), "achtemp": [cx(r[f"achtemp[{i}]"]) for i in range(3)],
                                  "achtemp_exact": exact_constant_gpp(*s), "seconds": r.get("seconds")})
        if s[0] <= 128:
            r = oracle.run_ref_driver("gppKer_root", s, threads=1)
            out["gppKer_root"].append({"args": list(s), "achtemp": [cx(r[f"achtemp[{i}]"]) for i in range(3)],
                                       "achtemp_exact": exact_constant_gpp(*s),
                                       "achstemp_printed": cx(r["achstemp"])})
    # gppKerSeq.cpp: the same driver with its gppsum argument (1: the half sum)
    out["gppKer_seq"] = []
    for s in SEQ_SIZES:
        r = oracle.run_ref_driver("gppKer_seq", s, threads=1)
        out["gppKer_seq"].append({"args": list(s), "achtemp": [cx(r[f"achtemp[{i}]"]) for i in range(3)]})
    real_fixtures(out)
    r = oracle.run_ref_driver("gppKer_orig", (512, 2, 2048, 32))
    out["gppKer_orig"].append({"args": [512, 2, 2048, 32], "achtemp": [cx(r[f"achtemp[{i}]"]) for i in range(3)]})
    for s in FF_SIZES:
        r = oracle.run_ref_driver("ffKernel", s)
        out["ffKernel"].append({"args": list(s), "achsDtemp": cx(r["achsDtemp"]), "asxDtemp0": cx(r["asxDtemp"]),
                                "achDtemp_cor0": cx(r["achDtemp_cor"])})
    with open(os.path.join(HERE, "reference_drivers.json"), "w") as f:
        json.dump(out, f, indent=1)

    # per-(n1, my_igp, iw) values of the reference solver functions
    for name, kw in (("gpp_pairs_branch", dict(dist="branch")), ("gpp_pairs_uniform", dict(dist="uniform"))):
        p = inputs.gpp_synthetic(7, 3, 300, 5, seed=11, index="reference", wx="reference", **kw)
        inv, nc = p["inv_igp_index"], p["ncouls"]
        igp = np.array([nc - 1 if i == nc else p["indinv"][i] for i in inv], np.int32)
        h = oracle.ref_gpp_pairs(p, igp)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), sch=h["sch"], ssx=h["ssx"],
                            **{k: np.asarray(v) for k, v in p.items()})
    # gppsum == 1 (gppKerSeq.cpp): ncouls 1536 puts igp 512 and 1024 on the
    # driver's 512-wide blocks (diagonal terms, skipped block ends)
    p = inputs.gpp_synthetic(7, 3, 1536, 6, seed=21, dist="branch", index="reference", wx="stress")
    inv, nc = p["inv_igp_index"], p["ncouls"]
    igp = np.array([nc - 1 if i == nc else p["indinv"][i] for i in inv], np.int32)
    h = oracle.ref_gpp_pairs(p, igp, gppsum=1)
    np.savez_compressed(os.path.join(HERE, "gpp_pairs_halfsum.npz"), sch=h["sch"], ssx=h["ssx"],
                        **{k: np.asarray(v) for k, v in p.items()})
    p = inputs.ff_synthetic(9, 3, 96, 12, 4, 5, seed=5)
    # schDt_matrix from the band x G x G' contraction, fed to the reference's
    # own achDtemp_Kernel (the reference C++ leaves it zero)
    schdt = oracle.ff(p, flags=oracle.ORC_FF_SCHDT_GEMM)["schDt_matrix"]
    h = oracle.ref_ff(p, schDt=schdt)
    np.savez_compressed(os.path.join(HERE, "ff_harness.npz"), ref_achsDtemp=h["achsDtemp"],
                        ref_asxDtemp=h["asxDtemp"], ref_achDtemp_cor=h["achDtemp_cor"], ref_ach2Dtemp=h["ach2Dtemp"],
                        ref_schDt=schdt, **{k: np.asarray(v) for k, v in p.items()})
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main("--big" in sys.argv)
