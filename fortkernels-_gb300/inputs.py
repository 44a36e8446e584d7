"""Input builders for the GPP (gppKer) and FF (ffKernel) paths.

Two families:

* ``*_reference_init``: the arrays the reference drivers build inside main()
  (constant 0.5+0.5i fills, BGW-Kernels/gppKer.cpp:275-299,310-314 and
  FFKer_cori/ffKernel.cpp:398-456), used for the drop-in command lines and the
  golden vectors those drivers print.
* ``gpp_synthetic`` / ``ff_synthetic``: seeded random inputs with the value
  distributions of the benchmark workloads (no BerkeleyGW data sets exist on
  this machine, so synthetic inputs of the same shapes stand in for them).

All complex arrays are complex128, row-major, in the reference layouts:
aqsmtemp/aqsntemp [number_bands][ncouls], I_eps/wtilde [ngpown][ncouls],
I_epsR/I_epsA [nFreq][ngpown][ncouls].
"""
from __future__ import annotations

import numpy as np

TO1 = 1e-6


def gpp_wx(e_lk: float = 10.0, e_n1kq: float = 6.0, dw: float = 1.0) -> np.ndarray:
    """The three evaluation frequencies, BGW-Kernels/gppKer.cpp:310-314."""
    wx = np.array([e_lk - e_n1kq + dw * ((iw + 1) - 2) for iw in range(3)], np.float64)
    wx[np.abs(wx) < TO1] = TO1
    return wx


def gpp_reference_index(ncouls: int, ngpown: int):
    """inv_igp_index[i] = (i+1)*ncouls/ngpown and indinv = identity,
    BGW-Kernels/gppKer.cpp:294-299."""
    inv = np.array([(i + 1) * ncouls // ngpown for i in range(ngpown)], np.int32)
    indinv = np.arange(ncouls, dtype=np.int32)
    return inv, indinv


def gpp_reference_init(number_bands: int, nvband: int, ncouls: int, nodes_per_group: int) -> dict:
    """Arrays of the gppKer driver main() (BGW-Kernels/gppKer.cpp:170-299)."""
    ngpown = ncouls // nodes_per_group
    expr = 0.5 + 0.5j
    inv, indinv = gpp_reference_index(ncouls, ngpown)
    return {
        "number_bands": number_bands, "nvband": nvband, "ncouls": ncouls, "ngpown": ngpown,
        "aqsmtemp": np.full((number_bands, ncouls), expr, np.complex128),
        "aqsntemp": np.full((number_bands, ncouls), expr, np.complex128),
        "I_eps_array": np.full((ngpown, ncouls), expr, np.complex128),
        "wtilde_array": np.full((ngpown, ncouls), expr, np.complex128),
        "vcoul": np.ones(ncouls, np.float64),
        "inv_igp_index": inv, "indinv": indinv, "wx_array": gpp_wx(),
    }


def gpp_real_reference_init(number_bands: int, nvband: int, ncouls: int, nodes_per_group: int) -> dict:
    """Arrays of the real-valued driver main() (gppKer_real.cpp:212-295): every
    array 0.5, vcoul = 1, the index map and frequencies of the complex driver."""
    ngpown = ncouls // nodes_per_group
    inv, indinv = gpp_reference_index(ncouls, ngpown)
    return {
        "number_bands": number_bands, "nvband": nvband, "ncouls": ncouls, "ngpown": ngpown,
        "aqsmtemp": np.full((number_bands, ncouls), 0.5), "aqsntemp": np.full((number_bands, ncouls), 0.5),
        "I_eps_array": np.full((ngpown, ncouls), 0.5), "wtilde_array": np.full((ngpown, ncouls), 0.5),
        "vcoul": np.ones(ncouls, np.float64), "inv_igp_index": inv, "indinv": indinv, "wx_array": gpp_wx(),
    }


def gpp_real_synthetic(number_bands: int, nvband: int, ncouls: int, ngpown: int, seed: int = 0,
                       dist: str = "uniform", index: str = "even", wx: str = "e10") -> dict:
    """Seeded inputs of the real-valued GPP: the real parts of gpp_synthetic's
    arrays (same options).  With dist="branch" wtilde lies around each
    frequency, so the noflag mask is false for many elements (the real driver
    then re-adds the value left at that block offset) and every branch of the
    real solver is taken."""
    p = gpp_synthetic(number_bands, nvband, ncouls, ngpown, seed=seed, dist=dist, index=index, wx=wx)
    for k in ("aqsmtemp", "aqsntemp", "I_eps_array", "wtilde_array"):
        p[k] = np.ascontiguousarray(p[k].real)
    return p


def _cu(rng, shape, lo=-0.5, hi=0.5):
    return rng.uniform(lo, hi, shape) + 1j * rng.uniform(lo, hi, shape)


def gpp_synthetic(number_bands: int, nvband: int, ncouls: int, ngpown: int, seed: int = 0,
                  dist: str = "uniform", index: str = "even", wx: str = "e10") -> dict:
    """Seeded GPP inputs.

    dist:  "uniform"   aqs*, I_eps re/im U[-0.5,0.5]; wtilde re U[0.5,2], im U[-0.05,0.05];
                       vcoul U[0.1,1]  (the benchmark distributions)
           "branch"    as uniform, but wtilde re is drawn around each wx so that
                       every branch of the GPP solver is taken (|wdiff|^2 near
                       0.25, |delw|^2 near 1e-6 and near 2.5e5)
    index: "even"      inv_igp_index[i] = i*ncouls/ngpown
           "reference" inv_igp_index[i] = (i+1)*ncouls/ngpown (clamped by the kernel)
    wx:    "e10"       e_lk-dw, e_lk, e_lk+dw with e_lk=10, dw=1
           "reference" e_lk - e_n1kq + dw*(iw-1) = {3,4,5}
           "stress"    {0.4, 3, 5}: a frequency below 0.5 makes the third branch
                       (neither sch nor ssx, |delw|^2 <= 1e-6) reachable
           "negative"  {-1.2, -0.7, 1.1}: frequencies below zero, where the Fortran
                       source's sexcut test applies (FK_GPP_PHYSICS)
    """
    rng = np.random.default_rng(seed)
    aqsm = _cu(rng, (number_bands, ncouls))
    aqsn = _cu(rng, (number_bands, ncouls))
    eps = _cu(rng, (ngpown, ncouls))
    wxa = {"e10": np.array([9.0, 10.0, 11.0]), "reference": gpp_wx(),
           "stress": np.array([0.4, 3.0, 5.0]), "negative": np.array([-1.2, -0.7, 1.1])}[wx]
    if dist == "uniform":
        wt = rng.uniform(0.5, 2.0, (ngpown, ncouls)) + 1j * rng.uniform(-0.05, 0.05, (ngpown, ncouls))
    elif dist == "branch":
        centre = wxa[rng.integers(0, 3, (ngpown, ncouls))]
        kind = rng.integers(0, 4, (ngpown, ncouls))
        # kind 0: |wdiff| around 0.5 (the limittwo edge); 1: tiny |wdiff| (pole);
        # 2: large wtilde far away; 3: wtilde near zero (|delw|^2 around to1)
        mag = np.where(kind == 0, rng.uniform(0.3, 0.7, kind.shape),
                       np.where(kind == 1, 10.0 ** rng.uniform(-5, -2, kind.shape), rng.uniform(0.5, 2.0, kind.shape)))
        ang = rng.uniform(0, 2 * np.pi, kind.shape)
        wt = centre + mag * np.exp(1j * ang)
        far = kind == 2
        wt[far] = rng.uniform(0.5, 2.0, far.sum()) + 1j * rng.uniform(-0.05, 0.05, far.sum())
        small = kind == 3
        wt[small] = (10.0 ** rng.uniform(-4, -1, small.sum())) * np.exp(1j * rng.uniform(0, 2 * np.pi, small.sum()))
    else:
        raise ValueError(dist)
    if index == "even":
        inv = np.array([i * ncouls // ngpown for i in range(ngpown)], np.int32)
        indinv = np.arange(ncouls, dtype=np.int32)
    else:
        inv, indinv = gpp_reference_index(ncouls, ngpown)
    return {
        "number_bands": number_bands, "nvband": nvband, "ncouls": ncouls, "ngpown": ngpown,
        "aqsmtemp": aqsm, "aqsntemp": aqsn, "I_eps_array": eps, "wtilde_array": wt.astype(np.complex128),
        "vcoul": rng.uniform(0.1, 1.0, ncouls), "inv_igp_index": inv, "indinv": indinv,
        "wx_array": wxa.astype(np.float64),
    }


def ff_reference_init(number_bands: int, nvband: int, ncouls: int, ngpown: int, nFreq: int, nfreqeval: int) -> dict:
    """Arrays of the ffKernel driver main() (FFKer_cori/ffKernel.cpp:344-456)."""
    expr = 0.5 + 0.5j
    grid = 2.0 * np.arange(nFreq, dtype=np.float64)
    pref = np.empty(nFreq)
    for i in range(nFreq):
        pref[i] = (grid[i + 1] - grid[i]) / 3.14 if i < nFreq - 1 else pref[i - 1]
    pref[0] *= 0.5
    pref[nFreq - 1] *= 0.5
    return {
        "number_bands": number_bands, "nvband": nvband, "ncouls": ncouls, "ngpown": ngpown,
        "nFreq": nFreq, "nfreqeval": nfreqeval,
        "aqsmtemp": np.full((number_bands, ncouls), expr, np.complex128),
        "aqsntemp": np.full((number_bands, ncouls), expr, np.complex128),
        "I_epsR_array": np.full((nFreq, ngpown, ncouls), 0.5 + 0.5j, np.complex128),
        "I_epsA_array": np.full((nFreq, ngpown, ncouls), 0.5 - 0.5j, np.complex128),
        "vcoul": np.ones(ncouls), "ekq": -10.0 + np.arange(number_bands, dtype=np.float64),
        "dFreqGrid": grid, "dFreqBrd": np.full(nFreq, 0.5 + 0.1j, np.complex128), "pref": pref,
        "pref_zb": 0.5 / 3.14, "freqevalmin": 0.0, "freqevalstep": 0.5, "occ": 1.0,
        "inv_igp_index": np.arange(ngpown, dtype=np.int32), "indinv": np.arange(ncouls, dtype=np.int32),
    }


def ff_synthetic(number_bands: int, nvband: int, ncouls: int, ngpown: int, nFreq: int, nfreqeval: int,
                 seed: int = 0) -> dict:
    """Seeded FF inputs with the benchmark distributions: aqs* and I_epsR/I_epsA
    re/im U[-0.5,0.5] plus 1.0 on the G=G' diagonal, band energies U[-1,1],
    nFreq real frequencies on [0, 2] Ry."""
    rng = np.random.default_rng(seed)
    epsR = _cu(rng, (nFreq, ngpown, ncouls))
    epsA = _cu(rng, (nFreq, ngpown, ncouls))
    inv = np.arange(ngpown, dtype=np.int32)
    indinv = np.arange(ncouls, dtype=np.int32)
    epsR[:, inv, indinv[inv]] += 1.0
    epsA[:, inv, indinv[inv]] += 1.0
    grid = np.linspace(0.0, 2.0, nFreq)
    pref = np.empty(nFreq)
    for i in range(nFreq):
        pref[i] = (grid[i + 1] - grid[i]) / 3.14 if i < nFreq - 1 else pref[i - 1]
    pref[0] *= 0.5
    pref[nFreq - 1] *= 0.5
    return {
        "number_bands": number_bands, "nvband": nvband, "ncouls": ncouls, "ngpown": ngpown,
        "nFreq": nFreq, "nfreqeval": nfreqeval,
        "aqsmtemp": _cu(rng, (number_bands, ncouls)), "aqsntemp": _cu(rng, (number_bands, ncouls)),
        "I_epsR_array": epsR, "I_epsA_array": epsA,
        "vcoul": rng.uniform(0.1, 1.0, ncouls), "ekq": rng.uniform(-1.0, 1.0, number_bands),
        "dFreqGrid": grid, "dFreqBrd": 0.5 * np.ones(nFreq) + 0.1j * np.ones(nFreq), "pref": pref,
        "pref_zb": 0.5 / 3.14, "freqevalmin": 0.0, "freqevalstep": 0.5, "occ": 1.0,
        "inv_igp_index": inv, "indinv": indinv,
    }


def ff_synthetic_device(number_bands: int, nvband: int, ncouls: int, ngpown: int, nFreq: int, nfreqeval: int,
                        seed: int = 0, device: str = "cuda") -> dict:
    """ff_synthetic's distributions with the four large arrays (aqsmtemp,
    aqsntemp, I_epsR_array, I_epsA_array) drawn on the GPU as torch tensors
    (2048 x 8192 x 4096 x 32 holds ~17 GB per epsilon array); the small arrays are
    numpy, as in ff_synthetic."""
    import torch
    gen = torch.Generator(device=device).manual_seed(seed)

    def cu(shape):
        x = torch.rand(tuple(shape) + (2,), generator=gen, device=device, dtype=torch.float64)
        x -= 0.5
        return torch.view_as_complex(x)

    p = ff_synthetic(1, nvband, 1, 1, nFreq, nfreqeval, seed=seed)  # small arrays of the right kind
    rng = np.random.default_rng(seed + 1)
    epsR, epsA = cu((nFreq, ngpown, ncouls)), cu((nFreq, ngpown, ncouls))
    idx = torch.arange(ngpown, device=device)
    epsR[:, idx, idx] += 1.0
    epsA[:, idx, idx] += 1.0
    p.update({
        "number_bands": number_bands, "ncouls": ncouls, "ngpown": ngpown,
        "aqsmtemp": cu((number_bands, ncouls)), "aqsntemp": cu((number_bands, ncouls)),
        "I_epsR_array": epsR, "I_epsA_array": epsA,
        "vcoul": rng.uniform(0.1, 1.0, ncouls), "ekq": rng.uniform(-1.0, 1.0, number_bands),
        "inv_igp_index": np.arange(ngpown, dtype=np.int32), "indinv": np.arange(ncouls, dtype=np.int32),
    })
    return p

