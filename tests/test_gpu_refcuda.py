"""The library's FP64 path pinned to the reference's own CUDA build on the same GPU.

oracle.refcuda() is the reference's gpu_functions.cu / data_structs.cu compiled unchanged
for sm_103a (oracle/refcuda.mk, from the copy of its sources staged beside the repository):
its cuFFT expanding_source, thrust z-sort and pair kernels.  This pins the FFT convolution
to the reference's own cuFFT output (not only to numpy's FFT) and the pair stage to its
GPU kernels.  expanding_source is run only at 10000 x 10000: its multiply kernel's grid is
fixed to that size (gpu_functions.cu:88-89) and indexes out of bounds at any other.
"""
import numpy as np
import pytest
import torch

import oracle

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not oracle.refcuda_available(), reason="reference CUDA sources not staged")]
DEV = "cuda:0"


def _rel(a, b, floor):
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), floor)))


@pytest.mark.parametrize("shape", ["uniform", "gaussian", "exponential"])
def test_expanding_source_matches_reference_cuda(ctx, shape):
    import microsn_gb300 as mlc
    N, width = 10000, 20.0
    pix = width / N
    rng = np.random.default_rng(11)
    mp = rng.lognormal(0.0, 0.7, (N, N))
    sizes = np.array([0.0, 2.0, 8.0, 32.0]) * pix  # half-light radii of 2, 8, 32 pixels, in R_E
    Noff = int(np.ceil((N / width) * sizes[-1])) + 4
    lx, ly = mlc.locations_random(3000, N, Noff, 7)
    LCr, DLCr, _ = oracle.refcuda_expanding_source(mp, sizes, shape, lx, ly, pix, width)
    m = mlc.Map(ctx, mp, "f64")
    LC, DLC = mlc.expanding_source(ctx, m, sizes, mlc.profile(shape, 0.0, pix), width, lx, ly)
    LC = LC.cpu().numpy()
    DLC = DLC.cpu().numpy()
    assert np.array_equal(LC[:, 0], LCr[:, 0])  # the point source is the map itself
    floor = 1e-3 * float(np.mean(LCr))
    assert _rel(LC, LCr, floor) < 1e-9
    assert float(np.max(np.abs(DLC - DLCr))) < 1e-9 * float(np.max(np.abs(LCr)))


@pytest.mark.parametrize("Nloc", [600, 2048])
def test_pair_path_matches_reference_cuda(ctx, golden, Nloc):
    import microsn_gb300 as mlc
    rng = np.random.default_rng(Nloc + 1)
    Nprof = 5
    LCA = np.exp(rng.normal(0, 0.6, (Nloc, Nprof)))
    LCB = np.exp(rng.normal(0, 0.6, (Nloc, Nprof)))
    LCA[: Nloc // 4, 0] = 1.25
    LCB[: Nloc // 4, 0] = 1.25  # ties: the stable order must match
    DLCA, DLCB = np.diff(LCA, axis=1), np.diff(LCB, axis=1)
    edges = mlc.bin_edges(300, 1e-4, 300, True)
    d, s, sizes = golden["setup_d"], golden["setup_s"], golden["setup_sizes"]
    v = mlc.setup_chi2_calculation((0.4, 0.5), (1.0,), float(golden["setup_Dfac"]), d, golden["setup0_t"], s, sizes)
    ref = oracle.refcuda_pair_path(LCA, DLCA, LCB, DLCB,
                                   dict(Njp=v.Njp, indA=v.indA, indB=v.indB, facA=v.facA, facB=v.facB, d=v.d, s=v.s),
                                   edges)
    T = lambda a: torch.as_tensor(np.ascontiguousarray(a), device=DEV)
    rank, lower, nper = mlc.setup_integral(ctx, T(LCA), T(LCB), edges)
    assert np.array_equal(rank.cpu().numpy().view(np.uint32), ref["rank"])
    assert np.array_equal(lower, ref["lower"]) and np.array_equal(nper, ref["nper"])
    chi2 = mlc.calculate_chi2(ctx, v, T(LCA), T(DLCA), T(LCB), T(DLCB), rank)
    bc, be = mlc.bin_chi2(ctx, lower, nper, chi2)
    full = nper > 0
    np.testing.assert_allclose(bc[full], ref["bchi2"][full], rtol=1e-12)
    np.testing.assert_allclose(be[full], ref["bexp"][full], rtol=1e-12, atol=1e-300)
    assert np.array_equal(bc[~full], ref["bchi2"][~full]) and np.array_equal(be[~full], ref["bexp"][~full])
    fb, fe, fn = mlc.pair_bin_fused(ctx, v, T(LCA), T(DLCA), T(LCB), T(DLCB), edges)
    assert np.array_equal(fn, ref["nper"])
    np.testing.assert_allclose(fb[full], ref["bchi2"][full], rtol=1e-10)


@pytest.mark.parametrize("nan_inputs", [False, True])
def test_pair_path_zero_and_nan_quotients_match_reference_cuda(ctx, golden, nan_inputs):
    """z = 0/x (both signs of zero), x/0 and 0/0: the reference's radix sort ranks -0.0 with
    +0.0 in pair order and the GPU's 0/0 NaN (sign bit set) before every other z, so those
    pairs fall in the first bin; with NaN light-curve values of either sign as well, a
    negative NaN joins them and a positive one goes after +inf.  Ranks, bins and bin means
    equal the reference's own CUDA path, and the oracle's ranks and bins equal both."""
    import microsn_gb300 as mlc
    rng = np.random.default_rng(23)
    Nloc, Nprof = 700, 5
    LCA = np.exp(rng.normal(0, 0.6, (Nloc, Nprof)))
    LCB = np.exp(rng.normal(0, 0.6, (Nloc, Nprof)))
    LCA[0:60:2, 0] = -0.0
    LCA[1:60:2, 0] = 0.0
    LCB[100:130, 0] = 0.0
    if nan_inputs:
        LCA[200:203, 0] = np.nan
        LCA[300:303, 0] = np.copysign(np.nan, -1.0)
    DLCA, DLCB = np.diff(LCA, axis=1), np.diff(LCB, axis=1)
    edges = mlc.bin_edges(300, 1e-4, 300, True)
    v = mlc.setup_chi2_calculation((0.4, 0.5), (1.0,), float(golden["setup_Dfac"]), golden["setup_d"],
                                   golden["setup0_t"], golden["setup_s"], golden["setup_sizes"])
    ref = oracle.refcuda_pair_path(LCA, DLCA, LCB, DLCB,
                                   dict(Njp=v.Njp, indA=v.indA, indB=v.indB, facA=v.facA, facB=v.facB, d=v.d, s=v.s),
                                   edges)
    T = lambda a: torch.as_tensor(np.ascontiguousarray(a), device=DEV)
    rank_t, lower, nper = mlc.setup_integral(ctx, T(LCA), T(LCB), edges)
    rank = rank_t.cpu().numpy().view(np.uint32)
    assert np.array_equal(rank, ref["rank"])
    assert np.array_equal(lower, ref["lower"]) and np.array_equal(nper, ref["nper"])
    r_o, l_o, n_o = oracle.pair_rank(LCA, LCB, edges)
    assert np.array_equal(r_o, ref["rank"]) and np.array_equal(l_o, ref["lower"]) and np.array_equal(n_o, ref["nper"])
    nan_first = 60 * 30 + (3 * Nloc if nan_inputs else 0)  # 0/0 pairs, and every pair of a negative-NaN row
    assert nper[0] >= nan_first
    chi2 = mlc.calculate_chi2(ctx, v, T(LCA), T(DLCA), T(LCB), T(DLCB), rank_t)
    bc, be = mlc.bin_chi2(ctx, lower, nper, chi2)
    np.testing.assert_allclose(bc, ref["bchi2"], rtol=1e-12)  # NaN where the reference has NaN
    np.testing.assert_allclose(be, ref["bexp"], rtol=1e-12, atol=1e-300)
    if not nan_inputs:  # the rank-free kernel: the same counts (positive NaN z have no bin there)
        _, _, fn = mlc.pair_bin_fused(ctx, v, T(LCA), T(DLCA), T(LCB), T(DLCB), edges)
        assert np.array_equal(fn, ref["nper"])
