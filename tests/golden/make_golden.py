"""Generate tests/golden/*.npz from the reference's own CPU code.

Runs the microLC CPU functions compiled from the reference sources
(oracle/_ref/libmlcref.so, built by oracle/Makefile) on small seeded inputs and
stores inputs and outputs.  The fixtures pin the oracle restatement where the
reference itself cannot run (the GPU machine has no reference sources).

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402


def ref_profile(shape, rhalf, pix):
    R = oracle.ref()
    nx = C.c_int(); ny = C.c_int()
    R.ref_profile(shape.encode(), rhalf, pix, C.byref(nx), C.byref(ny), None, 0)
    buf = np.zeros(nx.value * ny.value)
    st = R.ref_profile(shape.encode(), rhalf, pix, C.byref(nx), C.byref(ny), buf.ctypes.data_as(C.c_void_p), buf.size)
    assert st == 0
    return buf.reshape(ny.value, nx.value)


def main():
    oracle.build()
    R = oracle.ref()
    out = {}

    # profiles at the reference's pixel scale (width 25 R_E over 10000 px) and a coarse one
    cases = []
    for shape in ["uniform", "gaussian", "thermal_hole", "exponential"]:
        for rhalf, pix in [(0.05, 0.0025), (0.0123, 0.0025), (0.31, 0.01), (0.2, 0.05)]:
            cases.append((shape, rhalf, pix))
    for i, (shape, rhalf, pix) in enumerate(cases):
        out[f"profile_{i}"] = ref_profile(shape, rhalf, pix)
    out["profile_cases"] = np.array([f"{s}|{r!r}|{p!r}" for s, r, p in cases])

    # kernel wrap of a gaussian profile into a 96 x 80 array
    k = np.zeros(96 * 80)
    R.ref_kernel(b"gaussian", 0.2, 0.01, 80, 96, k)
    out["kernel_gauss_80x96"] = k.reshape(96, 80)

    # chi2 set-up with the reference's own input files' data (grid_input.json / rand_input.json)
    sizes = np.array([0, 0.05, 0.1, 0.2, 0.3])
    d = np.array([0.7, 1.2, 1.4, 1.1, 0.9]); s = np.array([0.1, 0.15, 0.1, 0.1, 0.15])
    t = np.array([5.0, 7.0, 12.0, 14.0, 17.0])
    Dfac = np.sqrt(1750 * 850 / 1570)
    setups = []
    for (M0, M1, V0, tt) in [(0.4, 0.5, 1.0, t), (0.4, 0.5, 1.0, t * 3), (0.3, 0.9, 2.0, t), (1.0, 0.2, 0.5, t * 2)]:
        Nd = len(d)
        Njp = np.zeros(1, np.int32); iA = np.zeros(Nd, np.int32); iB = np.zeros(Nd, np.int32)
        fA = np.zeros(Nd); fB = np.zeros(Nd); nd = np.zeros(Nd); ns = np.zeros(Nd); ct = np.zeros(1)
        R.ref_setup_chi2(M0, M1, V0, Dfac, Nd, d, np.ascontiguousarray(tt), s, len(sizes), sizes, Njp, iA, iB, fA, fB,
                         nd, ns, ct)
        n = int(Njp[0])
        setups.append(dict(M0=M0, M1=M1, V0=V0, t=tt, Njp=n, indA=iA[:n], indB=iB[:n], facA=fA[:n], facB=fB[:n],
                           const=ct[0]))
    for i, su in enumerate(setups):
        for kk, vv in su.items():
            out[f"setup{i}_{kk}"] = np.asarray(vv)
    out["setup_d"] = d; out["setup_s"] = s; out["setup_sizes"] = sizes; out["setup_Dfac"] = np.array(Dfac)

    # pair stage on synthetic light curves: rank table, ratio chi2, bin means
    rng = np.random.default_rng(7)
    Nloc, Nprof = 40, 5
    LCA = np.exp(rng.normal(0, 0.7, (Nloc, Nprof)))
    LCB = np.exp(rng.normal(0, 0.7, (Nloc, Nprof)))
    LCB[3, 0] = LCB[5, 0]  # ties in z
    LCA[7, 0] = 2 * LCA[9, 0]
    LCB[11, 0] = 2 * LCB[5, 0]
    DLCA = np.diff(LCA, axis=1); DLCB = np.diff(LCB, axis=1)
    rank = np.zeros(Nloc * Nloc, np.uint32)
    R.ref_setup_integral_cpu(Nloc, Nprof, LCA.ravel().copy(), LCB.ravel().copy(), rank)
    su = setups[0]
    chi2 = np.zeros(Nloc * Nloc)
    R.ref_calculate_chi2_cpu(su["Njp"], su["indA"].astype(np.int32), su["indB"].astype(np.int32), su["facA"],
                             su["facB"], d[: su["Njp"]].copy(), s[: su["Njp"]].copy(), Nloc, Nprof, LCA.ravel().copy(),
                             DLCA.ravel().copy(), LCB.ravel().copy(), DLCB.ravel().copy(), rank, chi2)
    edges = np.zeros(30)
    R.ref_mpd_edges(30, 1e-2, 1e2, 1, edges)
    # the reference's CPU twin does not compute bins (cpu_functions.cpp:186); bins come from
    # upper_bound over the sorted z (gpu_functions.cu:384-396), restated with numpy here
    z = (LCA[:, 0][:, None] / LCB[:, 0][None, :]).ravel()
    zs = np.sort(z, kind="stable")
    upper = np.searchsorted(zs, edges, side="right").astype(np.uint32)
    lower = np.concatenate([[0], upper[:-1]]).astype(np.uint32)
    nper = np.diff(np.concatenate([[0], upper])).astype(np.uint32)
    bc = np.zeros(30); be = np.zeros(30)
    R.ref_bin_chi2_cpu(Nloc, 30, lower, nper, chi2, bc, be)
    out.update(pair_LCA=LCA, pair_LCB=LCB, pair_rank=rank, pair_chi2=chi2, pair_edges=edges, pair_lower=lower,
               pair_nper=nper, pair_bchi2=bc, pair_bexp=be)

    # locations and log edges
    x = np.zeros(7 * 7, np.int32); y = np.zeros(7 * 7, np.int32)
    R.ref_locations_grid(7, 1000, 13, x, y)
    out["loc_grid_x"] = x; out["loc_grid_y"] = y
    x = np.zeros(50, np.int32); y = np.zeros(50, np.int32)
    R.ref_locations_random(50, 1000, 13, 5, x, y)
    out["loc_rand_x"] = x; out["loc_rand_y"] = y
    e = np.zeros(300)
    R.ref_mpd_edges(300, 1e-4, 300, 1, e)
    out["mpd_edges_log"] = e
    e = np.zeros(17)
    R.ref_mpd_edges(17, 0.5, 9.0, 0, e)
    out["mpd_edges_lin"] = e
    f1 = rng.random(20); f2 = rng.random(20); xx = np.cumsum(rng.random(20))
    out.update(trap_f1=f1, trap_f2=f2, trap_x=xx, trap_val=np.array(R.ref_trapezium(20, f1, f2, xx)))

    # map magnification-probability distributions: getBinnedMpd of a small heavy-tailed map
    # (values placed exactly on edges, at min and max, and between the last edge and max),
    # normalize, and divide_by into a ratio Mpd -- driver.cpp:173-180
    mp = np.exp(rng.normal(0.0, 1.2, (64, 64)))
    e50 = np.zeros(50)
    R.ref_mpd_edges(50, 0.02, 200.0, 1, e50)
    flat = mp.ravel()
    flat[:10] = e50[[0, 1, 5, 5, 20, 33, 48, 49, 49, 12]]
    flat[10:13] = [0.02, 200.0, np.nextafter(200.0, 0.0)]
    flat[13:16] = [0.0, 1e-3, 1e4]
    bins = np.zeros(50); counts = np.zeros(50)
    R.ref_binned_mpd(flat.copy(), 64, 64, 50, 0.02, 200.0, bins, counts)
    cn = counts.copy()
    R.ref_mpd_normalize(50, bins, cn)
    mpB = np.exp(rng.normal(0.2, 0.9, (64, 64))).ravel()
    binsB = np.zeros(50); countsB = np.zeros(50)
    R.ref_binned_mpd(mpB.copy(), 64, 64, 50, 0.02, 200.0, binsB, countsB)
    R.ref_mpd_normalize(50, binsB, countsB)
    eR = np.zeros(30)
    R.ref_mpd_edges(30, 0.05, 20.0, 1, eR)
    cR = np.zeros(30)
    R.ref_mpd_divide(50, bins, cn, 50, binsB, countsB, 30, eR, cR)
    out.update(mpd_map=flat.reshape(64, 64), mpd_bins=bins, mpd_counts=counts, mpd_counts_norm=cn,
               mpd_mapB=mpB.reshape(64, 64), mpd_binsB=binsB, mpd_countsB_norm=countsB, mpd_ratio_bins=eR,
               mpd_ratio_counts=cR)

    # multi-filter flux-ratio likelihood: getChi2CPU (chi2/chi2_functions.cuh:150-190)
    N, F, T = 40, 3, 7
    fo = rng.uniform(0.6, 1.4, (F, T)).astype(np.float32)
    dfo = rng.uniform(0.05, 0.3, (F, T)).astype(np.float32)
    m1 = rng.uniform(0.5, 2.0, (N, F, T)).astype(np.float32)
    m2 = rng.uniform(0.5, 2.0, (N, F, T)).astype(np.float32)
    like = R.chi2.ref_chi2_cpu(fo.ravel(), dfo.ravel(), m1.ravel(), m2.ravel(), N, F, T)
    out.update(fr_fobs=fo, fr_dfobs=dfo, fr_mu1=m1, fr_mu2=m2, fr_like=np.array(like, np.float32))

    np.savez_compressed(os.path.join(HERE, "reference_cpu.npz"), **out)
    print("wrote", os.path.join(HERE, "reference_cpu.npz"), len(out), "arrays")


if __name__ == "__main__":
    main()
