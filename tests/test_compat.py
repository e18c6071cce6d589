"""The reference-signature C++ layer (include/microlc_compat.hpp).

A driver in the shape of the reference's driver.cpp (tests/compat/driver_compat.cpp),
written only against the reference's class and function names, must compile and link
against the header and the library (CPU test), and its outputs on two synthetic gerlumph
maps must match the oracle run through the same chain (GPU test): light curves (FP64,
<= 1e-9 relative), map MPDs and their ratio (bit-exact), pair counts per bin (exact),
binned chi2 / exp(-chi2/2) and the likelihood (1e-12 relative).
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle
from microsn_gb300 import synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "compat", "driver_compat.cpp")
BUILD = os.path.join(ROOT, "tests", "compat", "_build")
LIBDIR = os.path.join(ROOT, "microsn_gb300")


def _compile(map_path: str) -> str:
    os.makedirs(BUILD, exist_ok=True)
    exe = os.path.join(BUILD, "driver_compat")
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    subprocess.check_call([nvcc, "-std=c++17", "-O2", "-x", "c++", "-I", os.path.join(ROOT, "include"),
                           f"-DMAP_PATH=\"{map_path}\"", SRC, "-L", LIBDIR, "-lmicrolc_gb300",
                           "-Xlinker", f"-rpath={LIBDIR}", "-o", exe])
    return exe


def test_compat_driver_compiles_and_links(lib_built):
    exe = _compile(os.path.join(BUILD, "maps") + "/")
    assert os.path.exists(exe)


def _maps(n, seeds):
    out = {}
    for i, seed in enumerate(seeds):
        rng = np.random.default_rng(seed)
        # ray counts: smooth heavy-tailed field, Poisson-sampled, like gerlumph int32 maps
        mu = synth.lognormal_map(n, seed=seed, sigma=0.9) * 40.0
        counts = rng.poisson(mu).astype(np.int32)
        meta = {"avgmu": 1.05 + 0.1 * i, "avgN": float(counts.mean()), "width": 12.0, "k": 0.4, "g": 0.35 + 0.05 * i,
                "s": 0.0}
        mid = f"map{seed}"
        synth.write_gerlumph(os.path.join(BUILD, "maps", mid), counts, meta)
        factor = abs(meta["avgmu"] / meta["avgN"])
        muth = abs(1.0 / ((1.0 - meta["k"]) ** 2 - meta["g"] ** 2))
        out[mid] = (counts.astype(np.float64) * factor / muth, meta)
    return out


@pytest.mark.gpu
def test_compat_driver_matches_oracle(lib_built):
    n = 480
    maps = _maps(n, (101, 102))
    (ida, (mpA, meta)), (idb, (mpB, _)) = list(maps.items())
    exe = _compile(os.path.join(BUILD, "maps") + "/")
    outdir = os.path.join(BUILD, "out")
    os.makedirs(outdir, exist_ok=True)
    subprocess.check_call([exe, ida, idb, outdir], cwd=BUILD)
    rd = lambda f: np.loadtxt(os.path.join(outdir, f), ndmin=2)

    # ---- light curves: expanding_source on grid locations
    sizes = [0.0, 0.05, 0.1, 0.2, 0.3]
    Nside, width = 24, meta["width"]
    Noff = int(np.ceil((n / width) * sizes[-1]))
    lx, ly = _grid(Nside, n, Noff)
    pix = 1.0 * width / n
    LCA_o, DLCA_o = oracle.expanding_source(mpA, sizes, "gaussian", lx, ly, pix, width)
    LCB_o, DLCB_o = oracle.expanding_source(mpB, sizes, "gaussian", lx, ly, pix, width)
    LCA, LCB = rd("lcurvesA.dat"), rd("lcurvesB.dat")
    for got, ref in ((LCA, LCA_o), (LCB, LCB_o)):
        ref = ref.reshape(got.shape)
        assert np.max(np.abs(got - ref) / np.maximum(np.abs(ref), 1e-3)) < 1e-9

    # ---- MPDs: getBinnedMpd, normalize, divide_by (bit-exact)
    full = rd("mpd_full.dat")
    bA, cA = oracle.binned_mpd(mpA, 200, 0.02, 200.0)
    bB, cB = oracle.binned_mpd(mpB, 200, 0.02, 200.0)
    cA = oracle.mpd_normalize(bA, cA); cB = oracle.mpd_normalize(bB, cB)
    assert np.array_equal(full[:200, 0], bA) and np.array_equal(full[:200, 1], cA)
    assert np.array_equal(full[:200, 2], bB) and np.array_equal(full[:200, 3], cB)
    eR = oracle.mpd_edges(60, 0.05, 20.0, True)
    cR = oracle.mpd_divide(bA, cA, bB, cB, eR)
    assert np.array_equal(full[200:, 0], eR) and np.array_equal(full[200:, 1], cR)

    # ---- pair stage: counts per bin exact, binned values and likelihood to 1e-12
    d = np.array([0.7, 1.2, 1.4, 1.1, 0.9]); s = np.array([0.1, 0.15, 0.1, 0.1, 0.15])
    t = np.array([5.0, 7.0, 12.0, 14.0, 17.0])
    Dfac = np.sqrt(850 * 1570 / 1750)
    cv = oracle.setup_chi2([0.4, 0.5], [1.0], Dfac, d, t, s, np.array(sizes))
    rank, lower, nper = oracle.pair_rank(LCA_o, LCB_o, eR)
    chi2 = oracle.pair_chi2_ratio(cv, LCA_o, DLCA_o, LCB_o, DLCB_o, rank)
    bchi2, bexp = oracle.bin_chi2(lower, nper, chi2)
    bn = rd("binned_N.dat")
    assert np.array_equal(bn[:, 1].astype(np.int64), nper.astype(np.int64))
    be = rd("binned_exp.dat")
    np.testing.assert_allclose(be[:, 1], bexp, rtol=1e-12, atol=0)
    np.testing.assert_allclose(be[:, 2], bchi2, rtol=1e-12, atol=0)
    like = rd("likelihood.dat")[0]
    integral = oracle.trapezium(bexp, cR, eR)
    np.testing.assert_allclose(like[1], integral, rtol=1e-12)
    np.testing.assert_allclose(like[0], integral * np.exp(-0.5 * cv["const_term"]), rtol=1e-12)


def _grid(Nside, Nmap, Noff):
    import microsn_gb300 as mlc
    return mlc.locations_grid(Nside, Nmap, Noff)
