"""Direct tiled convolution for small profiles and the launch autotuner on the GPU.

The direct form computes the same circular convolution with the reference's kernel wrap
as the FFT form (magnification_map.cpp:172-193); every tile shape is checked against the
FP64 oracle (per-pixel relative error: a direct sum of N^2 FP32 products, no FFT-wide
error spreading), on maps whose sides are not multiples of the tiles and with profiles
whose halo wraps around the map.  Where the one-call step and a per-stage call of
the same context take the same form the results are equal bit for bit, and either form
stays within the FP32 bound of the FFT form.
"""
import numpy as np
import pytest
import torch

import oracle
from microsn_gb300 import synth

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def _rel(a, b, floor):
    return np.max(np.abs(a - b) / np.maximum(np.abs(b), floor))


PROFILES = [("gaussian", 0.012), ("uniform", 0.006), ("exponential", 0.01), ("uniform", 0.03), ("exponential", 0.04),
            ("gaussian", 0.05), ("uniform", 0.001)]


@pytest.mark.parametrize("variant", [0, 1, 2, 3])
@pytest.mark.parametrize("Ny,Nx", [(200, 360), (96, 250)])
def test_direct_matches_oracle(ctx, variant, Ny, Nx):
    import microsn_gb300 as mlc
    mp = synth.lognormal_map(max(Ny, Nx), seed=Ny + 7 * Nx)[:Ny, :Nx].astype(np.float32).copy()
    m = mlc.Map(ctx, mp, "f32")
    seen = set()
    for shape, rhalf in PROFILES:
        p = mlc.profile(shape, rhalf, 0.002)
        prof = mlc.profile_raster(p)
        N = prof.shape[0]
        if N > 32:
            continue
        seen.add(N)
        got = mlc.convolve_direct(ctx, m, p, variant).cpu().numpy().astype(np.float64)
        ref = oracle.conv_fft(mp.astype(np.float64), prof)
        # FP32 products of FP32 pixels and the FP32-rounded profile, FP32 accumulation of
        # N^2 <= 1024 non-negative terms
        assert _rel(got, ref, 1e-3 * ref.mean()) < 1e-5, (shape, rhalf, N)
    assert len(seen) >= 4 and min(seen) <= 8 and max(seen) >= 24


def test_direct_refuses_what_it_does_not_cover(ctx):
    import microsn_gb300 as mlc
    mp = synth.lognormal_map(64, seed=3)
    m64 = mlc.Map(ctx, mp, "f64")
    m32 = mlc.Map(ctx, mp.astype(np.float32), "f32")
    small = mlc.profile("gaussian", 0.02, 0.01)
    big = mlc.profile("gaussian", 0.2, 0.01)  # raster wider than 32 pixels
    assert mlc.profile_raster(big).shape[0] > 32
    for args in ((m64, small, 0), (m32, big, 0), (m32, small, 4), (m32, small, -1)):
        with pytest.raises(mlc.MlcError):
            mlc.convolve_direct(ctx, *args)


def _profiles(n):
    import microsn_gb300 as mlc
    shapes = ["uniform", "exponential", "gaussian", "limb_darkened"]
    rh = [1.5, 3.0, 5.0, 8.0, 12.0]
    return [mlc.profile(shapes[i % 4], rh[(i // 4) % 5], 1.0, ref_compat=False, u=0.6) for i in range(n)]


def test_autotune_choices_keep_the_step_equal_to_per_stage_calls(lib_built):
    """With the autotuner on, small profiles may run in the direct form: the one-call step
    (cluster last pass reading the direct form's planar rows) must still equal the
    per-stage calls of the same context bit for bit, and every tuned key is reported."""
    import microsn_gb300 as mlc
    c = mlc.Context(0)
    try:
        c.set_autotune(True)
        N = 2000
        mp = synth.lognormal_map(N, seed=61).astype(np.float32)
        m = mlc.Map(c, mp, "f32")
        profs = _profiles(12)
        x0, y0, phi, v, off, t = synth.tracks(500, N, 3.0, 62, epochs=(0, 40), v_range=(0.01, 0.3))
        tr = {k: torch.as_tensor(np.ascontiguousarray(a, np.int64 if k == "off" else np.float32), device=DEV)
              for k, a in zip(("x0", "y0", "phi", "v", "off", "t"), (x0, y0, phi, v, off, t))}
        got = mlc.convolve_sample_tracks(c, m, profs, tr, mag=True)
        outs = []
        for p in profs:
            cm = mlc.convolve(c, m, p, "fused")
            outs.append(mlc.sample_tracks(c, [cm], N, N, tr["x0"], tr["y0"], tr["phi"], tr["v"], tr["off"], tr["t"],
                                          mag=True)[0])
        rep = c.autotune_report()
        Ns = [mlc.profile_raster(p).shape[0] for p in profs]
        small = {n for n in Ns if 2 <= n <= 32}
        # the step tunes against the FFT form up to the shared last pass, single
        # convolutions against the whole FFT form: one key of each per small size
        want = {f"conv f32 {N}x{N} N{n}{s}" for n in small for s in ("", " spectrum")}
        assert small and want <= set(rep)
        for key, (choice, cands) in rep.items():
            assert set(cands) == {"fft", "direct_4x4", "direct_4x8", "direct_8x4", "direct_8x8"}
            assert choice == min(cands, key=cands.get)
        c.set_autotune(False)
        ref = mlc.convolve_sample_tracks(c, m, profs, tr, mag=True)  # the FFT form everywhere
        form = lambda key: "fft" if key not in rep or rep[key][0] == "fft" else "direct"
        fr_all = 10 ** (-0.4 * ref[torch.isfinite(ref)].double())
        bound = 2e-5 * float(fr_all.pow(2).mean().sqrt()) * np.log2(N)
        for k, n in enumerate(Ns):
            # every direct tile shape sums in the same order: same form, same bits
            if form(f"conv f32 {N}x{N} N{n} spectrum") == form(f"conv f32 {N}x{N} N{n}"):
                assert torch.equal(got[k], outs[k]), k
            fin = torch.isfinite(ref[k])
            assert torch.equal(fin, torch.isfinite(got[k]))
            # either form within the FP32 FFT bound of the convolution tests
            fg, fr = 10 ** (-0.4 * got[k][fin].double()), 10 ** (-0.4 * ref[k][fin].double())
            assert float((fg - fr).abs().max()) < bound, k
    finally:
        c.close()


def test_autotune_off_reports_nothing(lib_built):
    import microsn_gb300 as mlc
    c = mlc.Context(0)
    try:
        c.set_autotune(False)
        m = mlc.Map(c, synth.lognormal_map(200, seed=5).astype(np.float32), "f32")
        mlc.convolve(c, m, mlc.profile("gaussian", 0.02, 0.01), "fused")
        torch.cuda.synchronize()
        assert c.autotune_report() == {}
    finally:
        c.close()
