"""Seeded synthetic inputs with the shapes and value distributions of the workloads:
magnification maps by inverse ray shooting (equal-mass point lenses, kappa_*, gamma,
width in Einstein radii), straight tracks with seasonal epochs, observed curves.

Maps are returned in the reference's normalisation (magnification_map.cpp:33-38):
pixel = counts * |avgmu / avgN| / |mu_th| with avgmu = mu_th, i.e. counts / avgN, so
the mean is about 1.  The gerlumph writer produces files the reference's reader (and
mlc_read_gerlumph) accept.
"""
from __future__ import annotations

import ctypes as C
import math
import os

import numpy as np


def lens_field(kappa_star: float, gamma: float, width: float, seed: int, margin: float = 2.0):
    """Lens positions covering the image-plane region that maps into the source square."""
    rng = np.random.default_rng(seed)
    half = width / 2 + margin
    l1 = half / abs(1 - kappa_star - gamma)
    l2 = half / abs(1 - kappa_star + gamma)
    R = math.hypot(l1, l2) + 5.0
    n = int(round(kappa_star * R * R))
    r = R * np.sqrt(rng.random(n))
    th = 2 * np.pi * rng.random(n)
    return np.stack([r * np.cos(th), r * np.sin(th)], axis=1), (l1, l2)


def _grid(N, width, kappa_star, gamma, rays_per_pixel):
    mu_th = 1.0 / abs((1 - kappa_star) ** 2 - gamma ** 2)
    pix_area = (width / N) ** 2
    dens = rays_per_pixel / (mu_th * pix_area)  # rays per unit image-plane area
    dx = 1.0 / math.sqrt(dens)
    return mu_th, dx


def rayshoot_numpy(N: int, width: float, kappa_star: float, gamma: float, seed: int, rays_per_pixel: float = 8.0):
    """Small maps on the host (tests): returns (map FP64, counts int32, meta dict)."""
    lenses, (l1, l2) = lens_field(kappa_star, gamma, width, seed)
    mu_th, dx = _grid(N, width, kappa_star, gamma, rays_per_pixel)
    nrx, nry = int(2 * l1 / dx) + 1, int(2 * l2 / dx) + 1
    xs = -l1 + dx * np.arange(nrx)
    ys = -l2 + dx * np.arange(nry)
    counts = np.zeros(N * N, np.int64)
    half = width / 2
    X1, X2 = np.meshgrid(xs, ys)
    X1 = X1.ravel(); X2 = X2.ravel()
    chunk = max(1, 4_000_000 // max(len(lenses), 1))
    for s in range(0, X1.size, chunk):
        x1 = X1[s:s + chunk, None]; x2 = X2[s:s + chunk, None]
        u = x1 - lenses[None, :, 0]; v = x2 - lenses[None, :, 1]
        q = 1.0 / (u * u + v * v)
        y1 = (1 - gamma) * x1[:, 0] - (u * q).sum(1)
        y2 = (1 + gamma) * x2[:, 0] - (v * q).sum(1)
        j = np.floor((y1 + half) * N / width).astype(np.int64)
        i = np.floor((y2 + half) * N / width).astype(np.int64)
        ok = (i >= 0) & (i < N) & (j >= 0) & (j < N)
        np.add.at(counts, i[ok] * N + j[ok], 1)
    counts = counts.astype(np.int32).reshape(N, N)
    avgN = counts.mean()
    meta = dict(avgmu=mu_th, avgN=avgN, Nx=N, width=width, k=kappa_star, g=gamma, s=0.0)
    return counts_to_map(counts, meta), counts, meta


def counts_to_map(counts, meta):
    k, g = meta["k"], meta["g"]
    factor = abs(meta["avgmu"] / meta["avgN"])
    muth = abs(1.0 / ((1.0 - k) ** 2 - g ** 2))
    return counts.astype(np.float64) * factor / muth


def rayshoot_gpu(ctx, N: int, width: float, kappa_star: float, gamma: float, seed: int,
                 rays_per_pixel: float = 4.0, dtype=None):
    """Large maps on the device through mlc_rayshoot; returns (map tensor, meta)."""
    import torch
    lenses, (l1, l2) = lens_field(kappa_star, gamma, width, seed)
    mu_th, dx = _grid(N, width, kappa_star, gamma, rays_per_pixel)
    nrx, nry = int(2 * l1 / dx) + 1, int(2 * l2 / dx) + 1
    dev = f"cuda:{ctx.device}"
    lz = torch.as_tensor(lenses.astype(np.float32), device=dev).contiguous()
    counts = torch.empty((N, N), dtype=torch.int32, device=dev)
    ctx.check(ctx.L.mlc_rayshoot(ctx.h, C.c_void_p(lz.data_ptr()), len(lenses), 0.0, gamma, -l1, -l2, dx, nrx, nry,
                                 width, N, C.c_void_p(counts.data_ptr())))
    avgN = counts.double().mean().item()
    meta = dict(avgmu=mu_th, avgN=avgN, Nx=N, width=width, k=kappa_star, g=gamma, s=0.0)
    scale = abs(meta["avgmu"] / avgN) / abs(1.0 / ((1.0 - kappa_star) ** 2 - gamma ** 2))
    m = counts.to(dtype or torch.float64) * scale
    return m, meta


def write_gerlumph(directory: str, counts: np.ndarray, meta: dict):
    os.makedirs(directory, exist_ok=True)
    with open(os.path.join(directory, "mapmeta.dat"), "w") as f:
        f.write(f"{meta['avgmu']:.17g} {meta['avgN']:.17g}\n{counts.shape[0]}\n{meta['width']:.17g}\n"
                f"{meta['k']:.17g} {meta['g']:.17g} {meta['s']:.17g}\n")
    np.ascontiguousarray(counts, np.int32).tofile(os.path.join(directory, "map.bin"))


def lognormal_map(N: int, seed: int, sigma: float = 0.8):
    """Quick heavy-tailed positive field with mean about 1 (smoothed lognormal)."""
    rng = np.random.default_rng(seed)
    g = rng.standard_normal((N, N))
    F = np.fft.rfft2(g)
    ky = np.fft.fftfreq(N)[:, None]; kx = np.fft.rfftfreq(N)[None, :]
    F *= np.exp(-(kx ** 2 + ky ** 2) * (N / 16.0) ** 2)
    g = np.fft.irfft2(F, s=(N, N))
    g = (g - g.mean()) / (g.std() + 1e-30)
    m = np.exp(sigma * g)
    return m / m.mean()


def tracks(ntracks: int, Nmap: int, margin: float, seed: int, epochs=(20, 200), seasons: int = 3,
           v_range=(0.5, 5.0), season_len: float = 120.0, gap: float = 245.0, equal_epochs: int | None = None,
           uniform_span: float | None = None):
    """Straight tracks: uniform start inside [margin, Nmap - margin), uniform angle, speed
    in pixels/day; epoch counts uniform in [epochs[0], epochs[1]] spread over `seasons`
    observing seasons separated by gaps (or `equal_epochs` uniform epochs over
    `uniform_span` days).  The track is kept inside the map by choosing its start such that
    the end stays inside.  Returns numpy arrays x0, y0, phi, v, off (int64), t."""
    rng = np.random.default_rng(seed)
    if equal_epochs is not None:
        n = np.full(ntracks, equal_epochs, np.int64)
    else:
        n = rng.integers(epochs[0], epochs[1] + 1, size=ntracks)
    off = np.zeros(ntracks + 1, np.int64)
    np.cumsum(n, out=off[1:])
    E = int(off[-1])
    t = np.empty(E)
    span_tot = seasons * season_len + (seasons - 1) * gap
    for k in range(ntracks):
        nk = int(n[k])
        if equal_epochs is not None:
            tk = np.linspace(0.0, uniform_span if uniform_span is not None else 1.0 * nk, nk)
        else:
            s = rng.integers(0, seasons, size=nk)
            tk = np.sort(s * (season_len + gap) + rng.random(nk) * season_len)
        t[off[k]:off[k + 1]] = tk
    phi = rng.random(ntracks) * 2 * np.pi
    v = v_range[0] + (v_range[1] - v_range[0]) * rng.random(ntracks)
    tmax = t[off[1:] - 1] if E else np.zeros(ntracks)
    # keep every track inside [margin, Nmap - margin]: cap the speed where the span is too long
    room = 0.9 * (Nmap - 2 * margin)
    v = np.where(v * tmax > room, room / np.maximum(tmax, 1e-300), v)
    L = v * tmax
    lo = margin + np.maximum(0, -L * np.cos(phi))
    hi = Nmap - margin - np.maximum(0, L * np.cos(phi))
    x0 = lo + (hi - lo) * rng.random(ntracks)
    lo = margin + np.maximum(0, -L * np.sin(phi))
    hi = Nmap - margin - np.maximum(0, L * np.sin(phi))
    y0 = lo + (hi - lo) * rng.random(ntracks)
    _ = span_tot
    return x0, y0, phi, v, off, t
