"""The microlc command-line driver (microsn_gb300/driver/microlc.cpp), the replacement of
the reference's simulating_lcurves/src/driver.cpp:19-275.

CPU: the JSON reader and the input checks through `microlc --check` (resolved locations
against the library's locations_on_grid / locations_random, Dfac, bins), and that every
malformed or inconsistent input stops with exit status 1 and a message naming the key
or the line and column.  GPU: the whole run on two synthetic gerlumph maps against the
oracle -- light curves (<= 1e-9 rel), MPDs (bit-exact), pair counts per bin (exact),
binned chi2 (1e-12 rel), binned exp(-chi2/2) and the likelihood (1e-10 rel), the reference's output formats and the
last line "GPU: <integral>" -- and the tracks mode's light curves and offset chi2.
"""
import copy
import json
import os
import subprocess

import numpy as np
import pytest

import oracle
from microsn_gb300 import build as B
from microsn_gb300 import synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

BASE = {
    "sizes": [0, 0.05, 0.1, 0.2, 0.3],
    "shape": "gaussian",
    "locations": {"type": "grid", "Nmap": 10000, "ss": 25, "Nside": 99},
    "mpds": {"mpd": {"Nbins": 500, "min": 0.0001, "max": 400}, "ratio": {"Nbins": 300, "min": 0.0001, "max": 300}},
    "DL": 1570, "DS": 1750, "DLS": 850,
    "data": [{"d": [0.7, 1.2, 1.4, 1.1, 0.9], "s": [0.1, 0.15, 0.1, 0.1, 0.15], "t": [5, 7, 12, 14, 17]}],
}


@pytest.fixture(scope="module")
def exe(lib_built):
    return B.build_driver()


def _run(exe, cfg, tmp_path, *args, name="in.json"):
    p = tmp_path / name
    p.write_text(cfg if isinstance(cfg, str) else json.dumps(cfg))
    return subprocess.run([exe, str(p), *args], capture_output=True, text=True, cwd=tmp_path)


def _check(exe, cfg, tmp_path):
    r = _run(exe, cfg, tmp_path, "--check")
    assert r.returncode == 0, r.stderr
    return json.loads(r.stdout)


def test_check_grid_and_random(exe, tmp_path):
    import microsn_gb300 as mlc
    got = _check(exe, BASE, tmp_path)
    Noff = int(np.ceil((10000 / 25) * 0.3))
    lx, ly = mlc.locations_grid(99, 10000, Noff)
    assert got["Nloc"] == 99 * 99 and got["Noff"] == Noff
    assert got["x_sum"] == int(np.sum(lx)) and got["y_sum"] == int(np.sum(ly))
    assert got["Dfac"] == np.sqrt(1750 * 850 / 1570)
    assert got["mpd"] == [500, 0.0001, 400] and got["ratio"] == [300, 0.0001, 300]
    assert got["M"] == [0.4, 0.5] and got["V"] == [1] and got["maps"] == ["12123", "11156"]
    cfg = copy.deepcopy(BASE)
    cfg["locations"] = {"type": "random", "Nmap": 10000, "ss": 25, "Nloc": 9216, "seed": 5}
    cfg["M"] = [0.3, 0.7]
    cfg["maps"] = {"path": "/maps/", "A": "1", "B": "2"}
    got = _check(exe, cfg, tmp_path)
    lx, ly = mlc.locations_random(9216, 10000, Noff, 5)
    assert got["Nloc"] == 9216 and got["x_sum"] == int(np.sum(lx)) and got["y_sum"] == int(np.sum(ly))
    assert got["M"] == [0.3, 0.7] and got["maps"] == ["/maps/1", "/maps/2"]


def test_json_reader_accepts(exe, tmp_path):
    # comments (jsoncpp's default reader allows them), exponents, escapes, nested whitespace
    text = json.dumps(BASE, indent=2).replace('"Nmap": 10000', '"Nmap": 1e4').replace('"ss": 25', '"ss": 2.5E+1')
    text = "// input\n/* block\n comment */" + text.replace('"gaussian"', '"gau\\u0073sian"') + "\n"
    got = _check(exe, text, tmp_path)
    assert got["Nmap"] == 10000 and got["shape"] == "gaussian" and got["Nloc"] == 9801
    tr = copy.deepcopy(BASE)
    tr["locations"] = {"type": "tracks", "Nmap": 10000, "ss": 25, "Ntracks": 50, "seed": 3, "v": [0.01, 0.02]}
    a, b = _check(exe, tr, tmp_path), _check(exe, tr, tmp_path)
    assert a == b and a["Ntracks"] == 50 and all(np.isfinite(a["track_sums"]))


def _mutate(path, value):
    cfg = copy.deepcopy(BASE)
    node = cfg
    for k in path[:-1]:
        node = node[k]
    if value is KeyError:
        del node[path[-1]]
    else:
        node[path[-1]] = value
    return cfg


BAD = [
    (json.dumps(BASE)[:-20], "line 1"),                                  # truncated
    (json.dumps(BASE).replace('"Nside": 99', '"Nside": 99,'), "member name"),
    (json.dumps(BASE) + " {}", "after the top-level value"),
    (json.dumps(BASE).replace('"gaussian"', '"gauss\\qian"'), "invalid escape"),
    ("/* open comment " + json.dumps(BASE), "unterminated comment"),
    ("[" * 300 + "]" * 300, "nesting"),
    (json.dumps(BASE).replace('"DL": 1570', '"DL": 1570, "DL": 1'), "duplicate"),
    (json.dumps(BASE).replace("1570", "01570"), "line 1"),
    ("[1, 2]", "top level"),
    (_mutate(["sizes"], KeyError), "sizes: missing"),
    (_mutate(["sizes"], [0.1, 0.2]), "sizes[0]"),
    (_mutate(["sizes"], [0, -0.1]), "sizes[1]"),
    (_mutate(["sizes"], "0 0.1"), "sizes: expected an array"),
    (_mutate(["shape"], "wavy"), "shape"),
    (_mutate(["shape"], "hexagon"), "unknown profile shape"),
    (_mutate(["locations", "type"], "hex"), "locations.type"),
    (_mutate(["locations", "Nside"], 0), "locations.Nside"),
    (_mutate(["locations", "Nside"], 9.5), "expected an integer"),
    (_mutate(["locations", "Nmap"], KeyError), "locations.Nmap: missing"),
    (_mutate(["locations", "ss"], 0.5), "no room"),
    (_mutate(["mpds", "ratio", "min"], 0), "mpds.ratio"),
    (_mutate(["mpds", "mpd"], KeyError), "mpds.mpd: missing"),
    (_mutate(["DLS"], "850"), "DLS: expected a number"),
    (_mutate(["DL"], -1), "DL: must be positive"),
    (_mutate(["data"], []), "data"),
    (_mutate(["data"], [{"d": [1, 2], "s": [0.1], "t": [1, 2]}]), "same length"),
    (_mutate(["data"], [{"d": [1], "s": [0], "t": [1]}]), "data[0].s[0]"),
    (_mutate(["M"], [0.4]), "M: needs at least 2"),
]


@pytest.mark.parametrize("i", range(len(BAD)))
def test_bad_input_is_refused(exe, tmp_path, i):
    cfg, msg = BAD[i]
    r = _run(exe, cfg, tmp_path, "--check")
    assert r.returncode == 1, (r.stdout, r.stderr)
    assert msg in r.stderr, r.stderr
    assert r.stdout == ""


def test_usage_and_missing_file(exe, tmp_path):
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 1 and "json" in r.stdout
    r = subprocess.run([exe, str(tmp_path / "none.json"), "--check"], capture_output=True, text=True)
    assert r.returncode == 1 and "cannot open" in r.stderr


# ---------------------------------------------------------------- GPU runs

def _write_maps(directory, n, seeds):
    maps = []
    for i, seed in enumerate(seeds):
        rng = np.random.default_rng(seed)
        mu = synth.lognormal_map(n, seed=seed, sigma=0.9) * 40.0
        counts = rng.poisson(mu).astype(np.int32)
        meta = {"avgmu": 1.05 + 0.1 * i, "avgN": float(counts.mean()), "width": 12.0, "k": 0.4, "g": 0.35 + 0.05 * i,
                "s": 0.0}
        synth.write_gerlumph(os.path.join(directory, f"m{seed}"), counts, meta)
        factor = abs(meta["avgmu"] / meta["avgN"])
        muth = abs(1.0 / ((1.0 - meta["k"]) ** 2 - meta["g"] ** 2))
        maps.append(counts.astype(np.float64) * factor / muth)
    return maps


def _map_config(tmp_path, n):
    cfg = copy.deepcopy(BASE)
    cfg["locations"] = {"type": "grid", "Nmap": n, "ss": 12.0, "Nside": 24}
    cfg["mpds"] = {"mpd": {"Nbins": 200, "min": 0.02, "max": 200}, "ratio": {"Nbins": 60, "min": 0.05, "max": 20}}
    cfg["maps"] = {"path": str(tmp_path / "maps") + "/", "A": "m101", "B": "m102"}
    return cfg


@pytest.mark.gpu
def test_driver_matches_oracle(exe, tmp_path):
    n = 480
    mpA, mpB = _write_maps(tmp_path / "maps", n, (101, 102))
    cfg = _map_config(tmp_path, n)
    out = tmp_path / "full"
    out.mkdir()
    r = _run(exe, cfg, tmp_path, "--full-precision", "--out", str(out))
    assert r.returncode == 0, r.stdout + r.stderr
    rd = lambda f: np.loadtxt(out / f, ndmin=2)

    sizes = BASE["sizes"]
    width = 12.0
    Noff = int(np.ceil((n / width) * sizes[-1]))
    import microsn_gb300 as mlc
    lx, ly = mlc.locations_grid(24, n, Noff)
    pix = width / n
    LCA_o, DLCA_o = oracle.expanding_source(mpA, sizes, "gaussian", lx, ly, pix, width)
    LCB_o, DLCB_o = oracle.expanding_source(mpB, sizes, "gaussian", lx, ly, pix, width)
    for f, ref in (("lcurvesA.dat", LCA_o), ("lcurvesB.dat", LCB_o)):
        got = rd(f)
        assert np.max(np.abs(got - ref) / np.maximum(np.abs(ref), 1e-3)) < 1e-9

    bA, cA = oracle.binned_mpd(mpA, 200, 0.02, 200.0)
    bB, cB = oracle.binned_mpd(mpB, 200, 0.02, 200.0)
    cA = oracle.mpd_normalize(bA, cA)
    cB = oracle.mpd_normalize(bB, cB)
    eR = oracle.mpd_edges(60, 0.05, 20.0, True)
    cR = oracle.mpd_divide(bA, cA, bB, cB, eR)
    for f, (b, c) in (("mpd_A.dat", (bA, cA)), ("mpd_B.dat", (bB, cB)), ("mpd_R.dat", (eR, cR))):
        got = rd(f)
        assert np.array_equal(got[:, 0], b) and np.array_equal(got[:, 1], c), f

    dat = BASE["data"][0]
    Dfac = np.sqrt(1750 * 850 / 1570)
    cv = oracle.setup_chi2([0.4, 0.5], [1.0], Dfac, np.array(dat["d"], float), np.array(dat["t"], float),
                           np.array(dat["s"], float), np.array(sizes, float))
    rank, lower, nper = oracle.pair_rank(LCA_o, LCB_o, eR)
    chi2 = oracle.pair_chi2_ratio(cv, LCA_o, DLCA_o, LCB_o, DLCB_o, rank)
    bchi2, bexp = oracle.bin_chi2(lower, nper, chi2)
    bn = rd("binned_N.dat")
    assert np.array_equal(bn[:, 1].astype(np.int64), nper.astype(np.int64))
    be = rd("binned_exp.dat")
    np.testing.assert_allclose(be[:, 2], bchi2, rtol=1e-12, atol=0)
    # exp(-chi2/2) turns the last-ulp differences of summation order in chi2 (up to ~1e3
    # here) into relative differences chi2/2 times larger
    np.testing.assert_allclose(be[:, 1], bexp, rtol=1e-10, atol=0)
    integral = oracle.trapezium(bexp, cR, eR)
    like = rd("likelihood.dat")[0]
    np.testing.assert_allclose(like[1], integral, rtol=1e-10)
    np.testing.assert_allclose(like[0], integral * np.exp(-0.5 * cv["const_term"]), rtol=1e-10)

    # the reference's formats and last line, in the working directory by default
    r = _run(exe, cfg, tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    last = r.stdout.strip().splitlines()[-1]
    assert last.startswith("GPU: ")
    np.testing.assert_allclose(float(last[5:]), integral, rtol=1e-5)
    line = (tmp_path / "mpd_R.dat").read_text().splitlines()[0]
    assert line == "%11.6e %11.6e" % (eR[0], cR[0])
    assert (tmp_path / "lcurvesA.dat").read_text().splitlines()[0] == "".join(" %f" % x for x in LCA_o[0])
    assert (tmp_path / "binned_N.dat").read_text().splitlines()[0] == "%11.6e %d" % (eR[0], nper[0])


@pytest.mark.gpu
def test_driver_tracks_match_oracle(exe, tmp_path):
    n = 480
    maps = _write_maps(tmp_path / "maps", n, (103, 104))
    cfg = _map_config(tmp_path, n)
    cfg["maps"].update(A="m103", B="m104")
    cfg["locations"] = {"type": "tracks", "Nmap": n, "ss": 12.0, "Ntracks": 300, "seed": 9, "v": [0.02, 0.1]}
    obsB = {"d": [0.1, -0.2, 0.05, 0.3], "s": [0.05, 0.1, 0.05, 0.08], "t": [3.0, 9.0, 20.0, 31.0]}
    cfg["data"] = [{"d": [0.2, 0.1, -0.1, 0.0, 0.3], "s": [0.05, 0.1, 0.05, 0.08, 0.1], "t": [0, 4, 9, 15, 22]}, obsB]
    out = tmp_path / "tr"
    out.mkdir()
    r = _run(exe, cfg, tmp_path, "--full-precision", "--out", str(out))
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip().splitlines()[-1].startswith("best chi2: ")
    tr = np.loadtxt(out / "tracks.dat", ndmin=2)
    x0, y0, phi, v = (np.ascontiguousarray(col) for col in tr.T)
    sizes = BASE["sizes"]
    width, pix = 12.0, 12.0 / n
    Noff = int(np.ceil((n / width) * sizes[-1]))
    for mp, tag, obs in ((maps[0], "A", cfg["data"][0]), (maps[1], "B", obsB)):
        t = np.array(obs["t"], float)
        T = len(t)
        # every position of every track stays Noff + 1 pixels inside the map
        ts = np.concatenate([cfg["data"][0]["t"], obsB["t"]])
        for tt in (ts.min(), ts.max()):
            xs, ys = x0 + v * tt * np.cos(phi), y0 + v * tt * np.sin(phi)
            assert xs.min() >= Noff + 1 - 1e-9 and xs.max() <= n - Noff - 1 + 1e-9
            assert ys.min() >= Noff + 1 - 1e-9 and ys.max() <= n - Noff - 1 + 1e-9
        off = np.arange(len(x0) + 1, dtype=np.int64) * T
        tt = np.tile(t, len(x0))
        lc = np.loadtxt(out / f"lcurves_tracks_{tag}.dat", ndmin=2).reshape(len(x0), len(sizes), T)
        ch = np.loadtxt(out / f"chi2_tracks_{tag}.dat", ndmin=2).reshape(len(x0), len(sizes), 2)
        w = 1.0 / np.array(obs["s"], float) ** 2
        for k, s in enumerate(sizes):
            cm = mp if s == 0 else oracle.conv_fft(mp, oracle.profile("gaussian", s, pix))
            ref = oracle.sample_tracks(cm, x0, y0, phi, v, off, tt).reshape(len(x0), T)
            assert np.max(np.abs(lc[:, k, :] - ref)) < 1e-9, (tag, k)
            c_ref, dm_ref = oracle.chi2_offset(ref, np.array(obs["d"], float), w)
            np.testing.assert_allclose(ch[:, k, 0], c_ref, rtol=1e-9, atol=1e-12)
            np.testing.assert_allclose(ch[:, k, 1], dm_ref, rtol=1e-9, atol=1e-12)
