"""The oracle restatement pinned against the reference's own CPU code: live (where the
reference was compiled from its sources, oracle/_ref) and through the committed golden
vectors (everywhere)."""
import ctypes as C

import numpy as np
import pytest

import oracle

needs_ref = pytest.mark.skipif(not oracle.ref_available(), reason="reference sources not compiled here")


@pytest.fixture(scope="module", autouse=True)
def _build():
    oracle.build()


def test_profiles_match_golden(golden):
    cases = [str(c).split("|") for c in golden["profile_cases"]]
    for i, (shape, rhalf, pix) in enumerate(cases):
        ref = golden[f"profile_{i}"]
        mine = oracle.profile(shape, float(rhalf), float(pix))
        assert mine.shape == ref.shape, (shape, rhalf, pix)
        assert np.array_equal(mine, ref), (shape, rhalf, pix, np.abs(mine - ref).max())


@needs_ref
@pytest.mark.parametrize("shape", ["uniform", "gaussian", "thermal_hole", "exponential"])
@pytest.mark.parametrize("rhalf,pix", [(0.05, 25 / 10000), (0.3, 25 / 10000), (0.017, 20 / 2000), (1.7, 0.1)])
def test_profiles_match_reference_live(shape, rhalf, pix):
    R = oracle.ref()
    nx = C.c_int(); ny = C.c_int()
    R.ref_profile(shape.encode(), rhalf, pix, C.byref(nx), C.byref(ny), None, 0)
    buf = np.zeros(nx.value * ny.value)
    R.ref_profile(shape.encode(), rhalf, pix, C.byref(nx), C.byref(ny), buf.ctypes.data_as(C.c_void_p), buf.size)
    mine = oracle.profile(shape, rhalf, pix)
    assert np.array_equal(mine.ravel(), buf)


def test_kernel_wrap_matches_golden(golden):
    prof = oracle.profile("gaussian", 0.2, 0.01)
    k = oracle.kernel_wrap(prof, 80, 96)
    assert np.array_equal(k, golden["kernel_gauss_80x96"])


def test_setup_chi2_matches_golden(golden):
    d, s, sizes, Dfac = golden["setup_d"], golden["setup_s"], golden["setup_sizes"], float(golden["setup_Dfac"])
    for i in range(4):
        g = {k[len(f"setup{i}_"):]: golden[k] for k in golden.files if k.startswith(f"setup{i}_")}
        v = oracle.setup_chi2((float(g["M0"]), float(g["M1"])), (float(g["V0"]),), Dfac, d, g["t"], s, sizes)
        assert v["Njp"] == int(g["Njp"])
        assert np.array_equal(v["indA"], g["indA"]) and np.array_equal(v["indB"], g["indB"])
        assert np.array_equal(v["facA"], g["facA"]) and np.array_equal(v["facB"], g["facB"])
        assert v["const_term"] == float(g["const"])


def test_pair_rank_chi2_bins_match_golden(golden):
    LCA, LCB = golden["pair_LCA"], golden["pair_LCB"]
    rank, lower, nper = oracle.pair_rank(LCA, LCB, golden["pair_edges"])
    assert np.array_equal(rank, golden["pair_rank"])
    assert np.array_equal(lower, golden["pair_lower"]) and np.array_equal(nper, golden["pair_nper"])
    d, s, sizes, Dfac = golden["setup_d"], golden["setup_s"], golden["setup_sizes"], float(golden["setup_Dfac"])
    v = oracle.setup_chi2((0.4, 0.5), (1.0,), Dfac, d, golden["setup0_t"], s, sizes)
    chi2 = oracle.pair_chi2_ratio(v, LCA, np.diff(LCA, axis=1), LCB, np.diff(LCB, axis=1), rank)
    np.testing.assert_allclose(chi2, golden["pair_chi2"], rtol=1e-13, atol=0)
    bc, be = oracle.bin_chi2(lower, nper, chi2)
    ref_bc, ref_be = golden["pair_bchi2"], golden["pair_bexp"]
    full = nper > 0
    np.testing.assert_allclose(bc[full], ref_bc[full], rtol=1e-12)
    np.testing.assert_allclose(be[full], ref_be[full], rtol=1e-12)
    # empty bins: the CPU twin reports 0, the GPU kernel (and the oracle) 2000 / exp(-1000)
    assert np.all(bc[~full] == 2000.0)


def test_edges_trapezium_match_golden(golden):
    np.testing.assert_array_equal(oracle.mpd_edges(300, 1e-4, 300, True), golden["mpd_edges_log"])
    np.testing.assert_array_equal(oracle.mpd_edges(17, 0.5, 9.0, False), golden["mpd_edges_lin"])
    assert oracle.trapezium(golden["trap_f1"], golden["trap_f2"], golden["trap_x"]) == float(golden["trap_val"])


@needs_ref
def test_setup_chi2_random_inputs_live():
    R = oracle.ref()
    rng = np.random.default_rng(3)
    for trial in range(30):
        Nd = int(rng.integers(1, 49))
        sizes = np.concatenate([[0.0], np.sort(rng.random(int(rng.integers(2, 12))))])
        t = np.sort(rng.random(Nd) * 60)
        d = rng.random(Nd) + 0.5; s = rng.random(Nd) * 0.2 + 0.05
        M0, M1, V0 = rng.random() + 0.1, rng.random() + 0.1, rng.random() * 2 + 0.1
        Dfac = 28.0
        Njp = np.zeros(1, np.int32); iA = np.zeros(Nd, np.int32); iB = np.zeros(Nd, np.int32)
        fA = np.zeros(Nd); fB = np.zeros(Nd); nd = np.zeros(Nd); ns = np.zeros(Nd); ct = np.zeros(1)
        R.ref_setup_chi2(M0, M1, V0, Dfac, Nd, d, t, s, sizes.size, sizes, Njp, iA, iB, fA, fB, nd, ns, ct)
        v = oracle.setup_chi2((M0, M1), (V0,), Dfac, d, t, s, sizes)
        n = int(Njp[0])
        assert v["Njp"] == n
        assert np.array_equal(v["indA"], iA[:n]) and np.array_equal(v["indB"], iB[:n])
        assert np.array_equal(v["facA"], fA[:n]) and np.array_equal(v["facB"], fB[:n])
        assert v["const_term"] == ct[0]


@needs_ref
def test_pair_stage_random_live():
    R = oracle.ref()
    rng = np.random.default_rng(11)
    Nloc, Nprof = 61, 6
    LCA = np.exp(rng.normal(0, 0.5, (Nloc, Nprof))); LCB = np.exp(rng.normal(0, 0.5, (Nloc, Nprof)))
    LCA[:10, 0] = 1.0; LCB[:10, 0] = 1.0  # many equal z: stable tie order matters
    rank_ref = np.zeros(Nloc * Nloc, np.uint32)
    R.ref_setup_integral_cpu(Nloc, Nprof, LCA.ravel().copy(), LCB.ravel().copy(), rank_ref)
    rank, _, _ = oracle.pair_rank(LCA, LCB)
    assert np.array_equal(rank, rank_ref)


def test_mpd_match_golden(golden):
    """getBinnedMpd, normalize and divide_by (driver.cpp:173-180) against the reference's output."""
    b, c = oracle.binned_mpd(golden["mpd_map"], 50, 0.02, 200.0)
    assert np.array_equal(b, golden["mpd_bins"])
    assert np.array_equal(c, golden["mpd_counts"])
    assert np.array_equal(oracle.mpd_normalize(b, c), golden["mpd_counts_norm"])
    cR = oracle.mpd_divide(golden["mpd_bins"], golden["mpd_counts_norm"], golden["mpd_binsB"],
                           golden["mpd_countsB_norm"], golden["mpd_ratio_bins"])
    assert np.array_equal(cR, golden["mpd_ratio_counts"])


@needs_ref
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_mpd_random_live(seed):
    R = oracle.ref()
    rng = np.random.default_rng(seed)
    n = 300
    # ray-shooting-like maps: integer counts times a factor, many exact ties
    mp = rng.poisson(rng.lognormal(1.0, 1.0, (n, n))).astype(np.float64) * 0.37
    nb = int(rng.integers(20, 400))
    lo, hi = 10 ** rng.uniform(-3, -1), 10 ** rng.uniform(1, 3)
    bins = np.zeros(nb); counts = np.zeros(nb)
    R.ref_binned_mpd(mp.ravel().copy(), n, n, nb, lo, hi, bins, counts)
    b, c = oracle.binned_mpd(mp, nb, lo, hi)
    assert np.array_equal(b, bins) and np.array_equal(c, counts)
    cn = counts.copy(); R.ref_mpd_normalize(nb, bins, cn)
    assert np.array_equal(oracle.mpd_normalize(b, c), cn)
    mpB = rng.poisson(rng.lognormal(0.5, 1.2, (n, n))).astype(np.float64) * 0.61
    bB = np.zeros(nb); cB = np.zeros(nb)
    R.ref_binned_mpd(mpB.ravel().copy(), n, n, nb, lo, hi, bB, cB)
    R.ref_mpd_normalize(nb, bB, cB)
    nr = int(rng.integers(10, 300))
    eR = oracle.mpd_edges(nr, 0.01, 50.0, True)
    cR = np.zeros(nr)
    R.ref_mpd_divide(nb, bins, cn, nb, bB, cB, nr, eR, cR)
    assert np.array_equal(oracle.mpd_divide(bins, cn, bB, cB, eR), cR)


def test_flux_ratio_match_golden(golden):
    """getChi2CPU: the FP32 emulation is bit-identical, the FP64 restatement within 1e-5."""
    args = (golden["fr_fobs"], golden["fr_dfobs"], golden["fr_mu1"], golden["fr_mu2"])
    ref = float(golden["fr_like"])
    assert np.float32(oracle.flux_ratio_f32(*args)) == np.float32(ref)
    assert abs(oracle.flux_ratio(*args) - ref) <= 1e-5 * abs(ref)


@needs_ref
@pytest.mark.parametrize("N,F,T,seed", [(25, 7, 10, 1), (60, 2, 3, 2), (1, 1, 1, 3)])
def test_flux_ratio_random_live(N, F, T, seed):
    R = oracle.ref()
    rng = np.random.default_rng(seed)
    fo = rng.uniform(0.6, 1.4, (F, T)).astype(np.float32)
    dfo = rng.uniform(0.2, 0.6, (F, T)).astype(np.float32)
    m1 = rng.uniform(0.5, 2.0, (N, F, T)).astype(np.float32)
    m2 = rng.uniform(0.5, 2.0, (N, F, T)).astype(np.float32)
    ref = R.chi2.ref_chi2_cpu(fo.ravel(), dfo.ravel(), m1.ravel(), m2.ravel(), N, F, T)
    assert np.float32(oracle.flux_ratio_f32(fo, dfo, m1, m2)) == np.float32(ref)
    assert abs(oracle.flux_ratio(fo, dfo, m1, m2) - ref) <= 1e-5 * abs(ref)
