"""pytest configuration: the `gpu` marker and the package loader.

Tests marked `gpu` need a CUDA device and run the CUDA library; the rest run
on any machine (oracle against golden vectors, host logic, library symbols).
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the sm_103a library")


@pytest.fixture(scope="session")
def fk():
    import __graft_entry__
    return __graft_entry__.load_package()


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def ctx(fk):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    c = fk.Context(0)
    yield c
    c.close()


def rel(a, b):
    import numpy as np
    a, b = np.asarray(a), np.asarray(b)
    den = max(float(np.max(np.abs(b))), 1e-300)
    return float(np.max(np.abs(a - b))) / den


def scaled_err(res, ref, scale):
    """max_i |res_i - ref_i| / max(|ref_i|, scale_i): relative error, with the
    root-sum-square of the output's contributions as the floor of the
    denominator.  For a sum of many random-phase terms the rss is its expected
    magnitude, so this is the relative error at the sum's natural scale even
    when the particular sum happens to cancel."""
    import numpy as np
    res, ref, scale = (np.atleast_1d(np.asarray(x)) for x in (res, ref, scale))
    den = np.maximum(np.abs(ref), scale)
    den = np.where(den > 0, den, 1.0)
    return float(np.max(np.abs(res - ref) / den))


def mixed_gate(res, ref, scales, tol=1e-6, kappa_max=3.0, keys=None):
    """The mixed-precision gate.  Plain relative error (rel: max |res - ref| /
    max |ref| over each output) is asserted for every output that is not a
    cancellation, i.e. whose contributions' root-sum-square is at most
    kappa_max times its magnitude; an output that cancels more is gated by its
    error at the natural scale (scaled_err), with the plain relative error
    recorded beside it.  Returns {output: {rel, scaled, kappa}}."""
    import numpy as np
    errs = {}
    for k in (keys or scales):
        kappa = float(np.max(scales[k])) / max(float(np.max(np.abs(ref[k]))), 1e-300)
        e_rel, e_sc = rel(res[k], ref[k]), scaled_err(res[k], ref[k], scales[k])
        errs[k] = {"rel": e_rel, "scaled": e_sc, "kappa": kappa}
        assert (e_rel if kappa <= kappa_max else e_sc) <= tol, (k, errs[k])
    return errs


def gpp_scales_torch(p):
    """gpp_scales for inputs too large for the oracle: the root-sum-square of
    the per-(n1, igp) contributions to achtemp, asxtemp and acht_n1_loc,
    estimated with torch in FP64 on the GPU (noflag mask and sch of every band,
    so asxtemp's scale is its sch stand-in).  A scale only: it decides which
    outputs count as cancellations, nothing is checked against it."""
    import numpy as np
    import torch
    t = lambda k, dt: (p[k] if type(p[k]).__module__.startswith("torch")
                       else torch.from_numpy(np.ascontiguousarray(p[k]))).to("cuda", dt)
    nb, nc = int(p["number_bands"]), int(p["ncouls"])
    wt, eps = t("wtilde_array", torch.complex128), t("I_eps_array", torch.complex128)
    aqsm, aqsn = t("aqsmtemp", torch.complex128)[:nb], t("aqsntemp", torch.complex128)[:nb]
    vcoul, wx = t("vcoul", torch.float64), t("wx_array", torch.float64).cpu().numpy()
    g = torch.from_numpy(gpp_igp(p)).to("cuda")
    ok = g >= 0
    gg = torch.where(ok, g, torch.zeros_like(g))
    w = torch.conj(aqsm[:, gg]) * (0.5 * vcoul[gg] * ok)[None, :]          # [nb][ng]
    ach, n1loc = [], None
    for iw in range(3):
        wd = float(wx[iw]) - wt
        wdr = (wd * torch.conj(wd)).real
        delw = wt * torch.conj(wd) / wdr
        m = (wdr > 0.25) & ((delw * torch.conj(delw)).real < 1.0 / (1e-6 * 4.0))
        S = aqsn @ (torch.where(m, delw * eps, torch.zeros_like(eps))).T  # [nb][ng]
        c = (torch.abs(w * S) ** 2)
        ach.append(float(torch.sqrt(c.sum())))
        if iw == 2:
            n1loc = torch.sqrt(c.sum(dim=1)).cpu().numpy()
    return {"achtemp": np.array(ach), "asxtemp": np.array(ach), "acht_n1_loc": n1loc}


def host(x):
    """numpy view of an array that may be a torch tensor (copied to the host)."""
    import numpy as np
    return x.detach().cpu().numpy() if type(x).__module__.startswith("torch") else np.asarray(x)


def gpp_igp(p):
    import numpy as np
    nc = p["ncouls"]
    out = []
    indinv = host(p["indinv"])
    for i in host(p["inv_igp_index"]):
        if i == nc:
            out.append(nc - 1)
        elif 0 <= i < nc:
            g = int(indinv[i])
            out.append(g if 0 <= g < nc else -1)
        else:
            out.append(-1)
    return np.array(out)


def gpp_scales(p, orc, flags=0):
    """rss of the per-(n1, igp) contributions to achtemp, asxtemp, acht_n1_loc."""
    import numpy as np
    o = orc.gpp(p, flags=flags, per_pair=True)
    g = gpp_igp(p)
    v = np.where(g >= 0, np.asarray(p["vcoul"])[np.maximum(g, 0)], 0.0)
    t = o["sch"] * v[None, :, None]
    x = o["ssx"] * v[None, :, None]
    return {"achtemp": np.sqrt((np.abs(t) ** 2).sum(axis=(0, 1))),
            "asxtemp": np.sqrt((np.abs(x) ** 2).sum(axis=(0, 1))) if x.size else np.zeros(3),
            "acht_n1_loc": np.sqrt((np.abs(t[:, :, 2]) ** 2).sum(axis=1))}


def ff_scales(p, orc):
    """rss of the contributions to every FF output (numpy, small sizes only)."""
    import numpy as np
    nb, nv, nc, ng, nf, ne = (p[k] for k in ("number_bands", "nvband", "ncouls", "ngpown", "nFreq", "nfreqeval"))
    igp = np.asarray(p["indinv"])[np.asarray(p["inv_igp_index"])]
    w = np.conj(np.asarray(p["aqsmtemp"])[:, igp])
    v = np.asarray(p["vcoul"])[igp]
    R = np.stack([np.asarray(p["aqsntemp"]) @ np.asarray(p["I_epsR_array"])[f].T for f in range(nf)])
    A = np.stack([np.asarray(p["aqsntemp"]) @ np.asarray(p["I_epsA_array"])[f].T for f in range(nf)])
    tR, tA = w[None] * R, w[None] * A                       # [nf][nb][ng]
    rs = lambda z, ax: np.sqrt((np.abs(z) ** 2).sum(axis=ax))
    sch = rs(tR, 2).T                                       # [nb][nf]
    achs = 0.5 * rs(v[None, None] * tR[1:2], (0, 1, 2))
    grid, ekq = np.asarray(p["dFreqGrid"]), np.asarray(p["ekq"])
    asx2, cor2 = 0.0, 0.0
    for n1 in range(nb):
        wx = p["freqevalmin"] - ekq[n1] + p["freqevalstep"]
        if n1 < nv:
            f1, f2, i = orc.compute_fact(wx, grid, 1, False)
            asx2 += (rs(v * (f1 * tR[i, n1] + f2 * tR[i + 1, n1]), 0)) ** 2
        occ = n1 < nv
        f1, f2, i = orc.compute_fact(wx, grid, 2, occ)
        kind = (0 if occ else 1) if wx > 0 else (2 if occ else 0)
        if kind:
            d = f1 * (tR[i, n1] - tA[i, n1]) + f2 * (tR[i + 1, n1] - tA[i + 1, n1])
            cor2 += (rs(v * d, 0) * (0.5 if kind == 2 else 1.0)) ** 2
    brd = np.asarray(p["dFreqBrd"])
    achd = np.zeros(ne)
    for iw in range(ne):
        wxe = p["freqevalmin"] - ekq + (iw - 1) * p["freqevalstep"]
        den = np.abs(wxe[:, None] - (grid[None, :] - brd[None, :]))
        achd[iw] = np.sqrt(((np.asarray(p["pref"])[None, :] / den * sch) ** 2).sum())
    a2 = nb * (0.5 / np.pi) * 10 * np.sqrt(sch[-1, -1] ** 2 + sch[-1, -2] ** 2)
    return {"achsDtemp": achs, "asxDtemp": np.full(ne, np.sqrt(asx2)), "achDtemp": achd,
            "achDtemp_cor": np.full(ne, np.sqrt(cor2)), "ach2Dtemp": np.full(ne, a2), "schDt_matrix": sch}
