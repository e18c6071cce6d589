"""The whole light-curve step in one call (mlc_convolve_sample_tracks) on the GPU.

The call chains kernels that the other GPU tests check against the oracle (fused
convolution, interleave, interleaved track sampler), so its output must equal, bit for
bit, the same kernels called one at a time; host-buffer calls (chunked downloads, copy
streams, asynchronous calls back to back) must equal device-buffer calls.  One FP64 case
is also checked against the oracle directly.
"""
import numpy as np
import pytest
import torch

import oracle
from microsn_gb300 import synth

pytestmark = pytest.mark.gpu

DEV = "cuda:0"


def _profiles(n, pix=1.0):
    import microsn_gb300 as mlc
    shapes = ["uniform", "exponential", "gaussian", "limb_darkened"]
    rh = [1.5, 3.0, 5.0, 8.0, 12.0]
    out = []
    for i in range(n):
        out.append(mlc.profile(shapes[i % 4], rh[(i // 4) % 5] * pix, pix, ref_compat=False, u=0.6))
    return out


def _host_tracks(n, N, seed, dtype, epochs=(0, 40)):
    x0, y0, phi, v, off, t = synth.tracks(n, N, 3.0, seed, epochs=epochs, v_range=(0.01, 0.3))
    c = lambda a: np.ascontiguousarray(a, dtype)
    return {"x0": c(x0), "y0": c(y0), "phi": c(phi), "v": c(v), "off": np.ascontiguousarray(off, np.int64),
            "t": c(t)}


def _pinned(tr):
    out = {}
    for k, a in tr.items():
        x = torch.empty(a.shape, dtype=torch.from_numpy(a).dtype, pin_memory=True)
        x.copy_(torch.from_numpy(a))
        out[k] = x
    return out


def _device(tr):
    return {k: torch.as_tensor(a, device=DEV) for k, a in tr.items()}


@pytest.fixture(scope="module")
def bctx(lib_built):
    import microsn_gb300 as mlc
    c = mlc.Context(0)
    c.set_autotune(False)  # the FFT form in every path: the comparisons below are bit for bit
    yield c
    c.close()


def _separate(ctx, m, profs, trd, mag):
    """The same step with one library call per stage (planar sampler)."""
    import microsn_gb300 as mlc
    outs = []
    for p in profs:
        c = mlc.convolve(ctx, m, p, "fused")
        o = mlc.sample_tracks(ctx, [c], m.Nx, m.Ny, trd["x0"], trd["y0"], trd["phi"], trd["v"], trd["off"],
                              trd["t"], mag=mag)
        outs.append(o[0])
    return torch.stack(outs)


@pytest.mark.parametrize("nprof", [1, 5, 20])
def test_device_io_equals_separate_calls(bctx, nprof):
    import microsn_gb300 as mlc
    N = 360
    mp = synth.lognormal_map(N, seed=21).astype(np.float32)
    m = mlc.Map(bctx, mp, "f32")
    profs = _profiles(nprof)
    trd = _device(_host_tracks(700, N, 22, np.float32))
    got = mlc.convolve_sample_tracks(bctx, m, profs, trd, mag=True)
    ref = _separate(bctx, m, profs, trd, True)
    assert got.shape == ref.shape
    assert torch.equal(got, ref)
    m.close()


def test_host_io_chunked_equals_device_io(bctx):
    import microsn_gb300 as mlc
    N = 300
    mp = synth.lognormal_map(N, seed=31).astype(np.float32)
    m = mlc.Map(bctx, mp, "f32")
    profs = _profiles(18)  # two profile groups (16 + 2)
    trh = _host_tracks(900, N, 32, np.float32)
    ref = mlc.convolve_sample_tracks(bctx, m, profs, _device(trh), mag=True).cpu()
    bctx.set_chunk_bytes(64 * 1024)  # 64 KiB: 1024 epochs of 16 profiles per chunk -> many chunks
    try:
        got_pinned = mlc.convolve_sample_tracks(bctx, m, profs, _pinned(trh), mag=True)
        got_pageable = mlc.convolve_sample_tracks(bctx, m, profs, trh, mag=True,
                                                  out=torch.empty(ref.shape, dtype=torch.float32))
    finally:
        bctx.set_chunk_bytes(256 << 20)
    assert torch.equal(got_pinned, ref)
    assert torch.equal(got_pageable, ref)
    m.close()


def test_host_io_async_back_to_back(bctx):
    """Three asynchronous calls with new pixels each: every output matches its own map."""
    import microsn_gb300 as mlc
    N = 240
    base = synth.lognormal_map(N, seed=41).astype(np.float32)
    m = mlc.Map(bctx, base, "f32")
    profs = _profiles(6)
    trh = _host_tracks(800, N, 42, np.float32)
    scales = [1.0, 2.0, 0.5]
    pix = []
    for s in scales:
        h = torch.empty((N, N), dtype=torch.float32, pin_memory=True)
        h.copy_(torch.from_numpy(base * np.float32(s)))
        pix.append(h)
    trp = _pinned(trh)
    bctx.set_chunk_bytes(128 * 1024)
    try:
        outs = [mlc.convolve_sample_tracks(bctx, m, profs, trp, mag=False, pixels=pix[i], async_=True)
                for i in range(3)]
        bctx.synchronize()
    finally:
        bctx.set_chunk_bytes(256 << 20)
    trd = _device(trh)
    for i, s in enumerate(scales):
        ref = mlc.convolve_sample_tracks(bctx, m, profs, trd, mag=False,
                                         pixels=torch.as_tensor(base * np.float32(s), device=DEV)).cpu()
        assert torch.equal(outs[i], ref), i
    m.close()


def test_host_buffers_on_huge_pages(bctx):
    """mlc_host_alloc buffers (2 MB pages, registered): page-locked, zero-filled, and the
    asynchronous host-buffer step through them equals the device-buffer step."""
    import microsn_gb300 as mlc
    N = 240
    mp = synth.lognormal_map(N, seed=45).astype(np.float32)
    m = mlc.Map(bctx, mp, "f32")
    profs = _profiles(5)
    trh = _host_tracks(600, N, 46, np.float32)
    trp = {}
    for k, a in trh.items():
        x = mlc.host_empty(a.shape, torch.from_numpy(a).dtype)
        assert x.is_pinned() and not x.any()
        x.copy_(torch.from_numpy(a))
        trp[k] = x
    pix = mlc.host_empty((N, N), torch.float32)
    pix.copy_(torch.from_numpy(mp))
    E = int(trh["off"][-1])
    out = mlc.host_empty((len(profs), E), torch.float32)
    mlc.convolve_sample_tracks(bctx, m, profs, trp, mag=True, pixels=pix, out=out, async_=True)
    bctx.synchronize()
    ref = mlc.convolve_sample_tracks(bctx, m, profs, _device(trh), mag=True,
                                     pixels=torch.as_tensor(mp, device=DEV)).cpu()
    assert torch.equal(out, ref)
    m.close()
    del trp, pix, out  # released through mlc_host_free
    import ctypes
    L = mlc._lib.load()
    assert L.mlc_host_free(ctypes.c_void_p(None)) == 0
    p = ctypes.c_void_p()
    assert L.mlc_host_alloc(0, ctypes.byref(p)) == 1  # MLC_ERR_ARG


def test_join_orders_copies_on_the_stream(bctx):
    import microsn_gb300 as mlc
    N = 200
    mp = synth.lognormal_map(N, seed=51).astype(np.float32)
    m = mlc.Map(bctx, mp, "f32")
    profs = _profiles(3)
    trp = _pinned(_host_tracks(400, N, 52, np.float32))
    out = mlc.convolve_sample_tracks(bctx, m, profs, trp, mag=True, async_=True)
    bctx.join()
    ev = torch.cuda.Event()
    ev.record(bctx.stream)
    ev.synchronize()  # the copies back are done once the stream passes the join
    ref = mlc.convolve_sample_tracks(bctx, m, profs, _device(_pinned(_host_tracks(400, N, 52, np.float32))),
                                     mag=True).cpu()
    assert torch.equal(out, ref)
    m.close()


def test_f64_matches_oracle(bctx):
    import microsn_gb300 as mlc
    N = 128
    mp = synth.lognormal_map(N, seed=61)
    m = mlc.Map(bctx, mp, "f64")
    profs = _profiles(3)
    trh = _host_tracks(200, N, 62, np.float64, epochs=(1, 30))
    got = mlc.convolve_sample_tracks(bctx, m, profs, trh, mag=True,
                                     out=torch.empty((3, int(trh["off"][-1])), dtype=torch.float64)).numpy()
    for q, p in enumerate(profs):
        conv = oracle.conv_fft(mp, mlc.profile_raster(p))
        ref = oracle.sample_tracks(conv, trh["x0"], trh["y0"], trh["phi"], trh["v"], trh["off"], trh["t"], mag=True)
        assert np.max(np.abs(got[q] - ref)) < 1e-9, (q, np.max(np.abs(got[q] - ref)))
    m.close()


def test_no_tracks_and_errors(bctx):
    import microsn_gb300 as mlc
    N = 120
    m = mlc.Map(bctx, synth.lognormal_map(N, seed=71).astype(np.float32), "f32")
    profs = _profiles(2)
    empty = {"x0": np.zeros(0, np.float32), "y0": np.zeros(0, np.float32), "phi": np.zeros(0, np.float32),
             "v": np.zeros(0, np.float32), "off": np.zeros(1, np.int64), "t": np.zeros(0, np.float32)}
    out = mlc.convolve_sample_tracks(bctx, m, profs, empty)
    assert tuple(out.shape) == (2, 0)
    # one track longer than an output chunk is refused with MLC_ERR_LIMIT
    trh = _host_tracks(10, N, 72, np.float32, epochs=(30, 40))
    bctx.set_chunk_bytes(4096)
    try:
        # 4096 B / (2 profiles x 4 B) = 512 epochs per chunk: every track fits
        mlc.convolve_sample_tracks(bctx, m, profs, trh)
        # 4096 B / (16 profiles x 4 B) = 64 epochs per chunk: tracks of 70..80 epochs do not
        with pytest.raises(mlc.MlcError) as e:
            mlc.convolve_sample_tracks(bctx, m, _profiles(16), _host_tracks(10, N, 73, np.float32, epochs=(70, 80)))
        assert e.value.code == 6
    finally:
        bctx.set_chunk_bytes(256 << 20)
    with pytest.raises(ValueError):
        mixed = dict(trh)
        mixed["t"] = torch.as_tensor(trh["t"], device=DEV)
        mlc.convolve_sample_tracks(bctx, m, profs, mixed)
    m.close()


def test_profile_rasters_reused_only_for_the_same_list(bctx):
    """Back-to-back stream-ordered calls that alternate profile lists (and one repeat of a
    list with new pixels) equal the one-call-per-stage results: the cached rasters of the
    previous list are never used for another list."""
    import microsn_gb300 as mlc
    N = 300
    mp1 = synth.lognormal_map(N, seed=31).astype(np.float32)
    mp2 = synth.lognormal_map(N, seed=32).astype(np.float32)
    m = mlc.Map(bctx, mp1, "f32")
    pa = _profiles(6)
    pb = [mlc.profile("gaussian", r, 1.0, ref_compat=False) for r in (2.0, 4.5, 7.0)]
    trd = _device(_host_tracks(500, N, 33, np.float32))
    outs = []
    for profs in (pa, pb, pa, pa):
        outs.append((profs, mlc.convolve_sample_tracks(bctx, m, profs, trd, mag=True)))
    pix2 = torch.as_tensor(mp2, device=DEV)
    last = mlc.convolve_sample_tracks(bctx, m, pa, trd, mag=True, pixels=pix2)
    torch.cuda.synchronize()
    m1 = mlc.Map(bctx, mp1, "f32")
    for profs, got in outs:
        assert torch.equal(got, _separate(bctx, m1, profs, trd, True))
    m2 = mlc.Map(bctx, mp2, "f32")
    assert torch.equal(last, _separate(bctx, m2, pa, trd, True))


@pytest.mark.parametrize("prec,nprof", [("f32", 3), ("f32", 8), ("f32", 12), ("f32", 16), ("f32", 21), ("f64", 9)])
def test_fused_last_pass_interleave_equals_separate_calls(bctx, prec, nprof):
    """At a row length with a register c2r kernel (2000^2: 1000-point rows) the step runs the
    last inverse pass of a group's profiles as one cluster kernel writing the interleaved
    layout (interleave strides 4, 8 and 16, clusters with empty slots, two groups).  Its
    light curves must equal the one-call-per-stage results bit for bit."""
    import microsn_gb300 as mlc
    N = 2000
    dt = np.float32 if prec == "f32" else np.float64
    mp = synth.lognormal_map(N, seed=41).astype(dt)
    m = mlc.Map(bctx, mp, prec)
    profs = _profiles(nprof)
    trd = _device(_host_tracks(600, N, 42, dt))
    got = mlc.convolve_sample_tracks(bctx, m, profs, trd, mag=True)
    ref = _separate(bctx, m, profs, trd, True)
    assert torch.equal(got, ref)


@pytest.mark.parametrize("prec,fft,nprof", [("f32", "native", 12), ("f32", "f32x2", 12), ("f64", "native", 5)])
def test_step_as_cuda_graph_equals_eager(bctx, prec, fft, nprof):
    """graph=True: the first call runs eagerly and captures the whole step (forward spectrum,
    both convolution chains, the split last pass, sampling); later calls replay it.  Each
    replay -- after new pixels, new track values and new profile values of the same raster
    sizes were written into the same buffers -- equals the eager call on the same inputs,
    and one replay counts the kernels of the captured sequence."""
    import microsn_gb300 as mlc
    N = 2000
    dt = np.float32 if prec == "f32" else np.float64
    m = mlc.Map(bctx, synth.lognormal_map(N, seed=51).astype(dt), prec)
    if fft != "native":
        m.set_fft(fft)
    profs = _profiles(nprof)
    pix = torch.as_tensor(synth.lognormal_map(N, seed=52).astype(dt), device=DEV)
    trd = _device(_host_tracks(800, N, 53, dt))
    out = torch.empty((nprof, trd["t"].numel()), dtype=pix.dtype, device=DEV)
    mlc.convolve_sample_tracks(bctx, m, profs, trd, mag=True, pixels=pix, out=out, graph=True)  # eager + capture
    ref = mlc.convolve_sample_tracks(bctx, m, profs, trd, mag=True, pixels=pix)
    assert torch.equal(out, ref)
    l0 = bctx.launch_count()
    mlc.convolve_sample_tracks(bctx, m, profs, trd, mag=True, pixels=pix, out=out, graph=True)  # replay
    per_call = bctx.launch_count() - l0
    assert per_call > nprof
    assert torch.equal(out, ref)
    # new contents in the same buffers: pixels, tracks, profile values (same raster sizes)
    pix.copy_(torch.as_tensor(synth.lognormal_map(N, seed=54).astype(dt), device=DEV))
    new_tr = _host_tracks(800, N, 55, dt)
    for k in ("x0", "y0", "phi", "v"):
        trd[k].copy_(torch.as_tensor(new_tr[k], device=DEV))
    profs2 = list(profs)
    profs2[0] = mlc.profile("limb_darkened", 1.5, 1.0, ref_compat=False, u=0.2)  # same raster size as profs[0]
    assert mlc.profile_raster(profs2[0]).shape == mlc.profile_raster(profs[0]).shape
    l0 = bctx.launch_count()
    mlc.convolve_sample_tracks(bctx, m, profs2, trd, mag=True, pixels=pix, out=out, graph=True)
    assert bctx.launch_count() - l0 == per_call  # replayed, not recaptured
    ref2 = mlc.convolve_sample_tracks(bctx, m, profs2, trd, mag=True, pixels=pix)
    assert torch.equal(out, ref2)
    # the graph form takes device buffers only
    with pytest.raises(mlc.MlcError):
        mlc.convolve_sample_tracks(bctx, m, profs, {k: a.cpu().numpy() for k, a in trd.items()}, graph=True)
    m.close()


@pytest.mark.parametrize("prec,fft", [("f32", "native"), ("f32", "f32x2"), ("f64", "native")])
def test_profile_spectrum_cache_equals_recomputed(lib_built, prec, fft):
    """At 2000^2 (column split with N2 = 100) the step and convolve_many keep the profiles'
    spectra between calls and start P1 from them: the same light curves and maps, bit for bit,
    as a context that transforms every profile on every call -- also after the profile values
    change (same raster sizes), which must recompute the cached spectra."""
    import microsn_gb300 as mlc
    N = 2000
    dt = np.float32 if prec == "f32" else np.float64
    mp = synth.lognormal_map(N, seed=61).astype(dt)
    trh = _host_tracks(600, N, 62, dt)
    profs = _profiles(10)
    profs2 = list(profs)
    profs2[1] = mlc.profile("exponential", 1.4, 1.0, ref_compat=False)  # same raster size as profs[1]
    assert mlc.profile_raster(profs2[1]).shape == mlc.profile_raster(profs[1]).shape
    outs = {}
    for cache in (-1, 0):
        c = mlc.Context(0)
        c.set_autotune(False)
        c.set_profile_cache(cache)
        m = mlc.Map(c, mp, prec)
        if fft != "native":
            m.set_fft(fft)
        trd = {k: torch.as_tensor(a, device=DEV) for k, a in trh.items()}
        r = [mlc.convolve_sample_tracks(c, m, p, trd, mag=True).cpu() for p in (profs, profs, profs2, profs)]
        r.append(mlc.convolve_many(c, m, profs2[:4]).cpu())
        outs[cache] = r
        m.close()
        c.close()
    for a, b in zip(outs[-1], outs[0]):
        assert torch.equal(a, b)
    assert not torch.equal(outs[0][1], outs[0][2])  # the changed profile changed the curves


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_sampler_cell_order_equals_track_order(lib_built, prec):
    """The interleaved sampler in map-cell order (epoch chunks of 32 sorted by the 128-pixel
    cell they start in; chosen for maps much larger than L2) against the track order, both
    pinned: the same light curves bit for bit, through the device-buffer step and through
    the host-buffer step, whose chunks of tracks start at nonzero epoch offsets."""
    import microsn_gb300 as mlc
    N = 2000
    dt = np.float32 if prec == "f32" else np.float64
    mp = synth.lognormal_map(N, seed=71).astype(dt)
    trh = _host_tracks(3000, N, 72, dt, epochs=(5, 90))
    profs = _profiles(5)
    outs = {}
    for order in (0, 1):
        c = mlc.Context(0)
        c.set_autotune(False)
        c.tune_set("sample_tracks_il cell-order", order)
        m = mlc.Map(c, mp, prec)
        dev = mlc.convolve_sample_tracks(c, m, profs, {k: torch.as_tensor(a, device=DEV) for k, a in trh.items()},
                                         mag=True).cpu()
        c.set_chunk_bytes(64 * 1024)  # many chunks of tracks
        host = mlc.convolve_sample_tracks(c, m, profs, _pinned(trh), mag=True).clone()
        outs[order] = (dev, host)
        m.close()
        c.close()
    assert torch.equal(outs[0][0], outs[1][0])
    assert torch.equal(outs[0][1], outs[1][1])
    assert torch.equal(outs[1][0], outs[1][1])
