#!/usr/bin/env python
"""Throughput of the light-curve hot path on one GB300 (light curves/s).

Workload (the batched-profiles-and-tracks configuration): a 10000 x 10000 FP32
magnification map (inverse ray shooting, kappa_* = 0.45, gamma = 0.35, width 20
Einstein radii, seed 2) convolved with 16 profiles -- uniform disc and thin disc
(exponential shape), half-light radii 2, 4, 8, 16, 32, 48, 64, 96 px -- then 10^6
straight tracks (epochs uniform in 20..200 over 3 observing seasons with gaps)
sampled bilinearly on every convolved map and converted to magnitudes.  One light
curve = one track x one profile.  A step = map spectrum + 16 fused convolutions +
sampling of all tracks on all 16 maps.

Also reported: the plain one-launch-per-stage FP64 form of the same step, e2e
throughput through the library with host buffers (H2D of the map and tracks, D2H of
all light curves inside the timed region), per-kernel CUDA-event times, the roofline
of the dominant kernel, GPU clocks during the timed region and an FP64 CPU baseline
(the oracle port on the host cores, on a bounded sample).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl mine|reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "light curves/s and pair-chi2/s on 1 GB300, batched vs plain, at <=1e-5 rel err vs FP64"
UNIT = "light curves/s"

N_MAP, WIDTH, KAPPA, GAMMA, MAP_SEED = 10000, 20.0, 0.45, 0.35, 2
RAYS_PER_PIXEL = 4.0
# The headline form: FP32 map pixels, float-float transforms, FP32 convolved maps and light
# curves, float-float track positions -- within 1e-5 of FP64 in chi2 (FP32 transforms are not:
# their absolute error is up to ~1e-5 relative in faint pixels, ~3e-4 in chi2).
HEADLINE_FFT = "f32x2"
RHALF_PX = [2, 4, 8, 16, 32, 48, 64, 96]
SHAPES = ["uniform", "exponential"]
N_TRACKS, EPOCHS, SEASONS, TRACK_SEED = 1_000_000, (20, 200), 3, 3
V_RANGE = (0.05, 1.0)  # pixels / day
SEASON_LEN, GAP = 120.0, 245.0
MARGIN = 2 * max(RHALF_PX) + 2


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["mine", "reference"], default="mine")
    ap.add_argument("--small", action="store_true", help="reduced sizes (debug only; not a bench number)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain FP64 form")
    ap.add_argument("--no-pair", action="store_true", help="skip the pair-chi2/s, flux-ratio, C1 and C4 workloads")
    ap.add_argument("--no-c5", action="store_true", help="skip the supernova multi-image workload")
    ap.add_argument("--n", "--side", dest="n", type=int, default=None,
                    help="map side (profiling cases only; not a bench number)")
    ap.add_argument("--tracks", type=int, default=None, help="track count (profiling cases only)")
    ap.add_argument("--kernel-case", default=None,
                    choices=["step", "pair_bin_fused", "mpd", "flux_ratio", "track_fit", "sort", "pair_sides", "pair",
                             "c1", "c5"],
                    help="run one workload alone at the given sizes, for an ncu capture (prints its times; not a "
                         "bench line)")
    ap.add_argument("--nprof", type=int, default=None, help="profiles of the step (profiling cases only)")
    ap.add_argument("--fft", choices=["native", "f32x2"], default=None,
                    help="transform arithmetic of the step's FP32 map (profiling cases only)")
    ap.add_argument("--tune", action="append", default=[], metavar="KEY=CHOICE",
                    help="pin an autotuner choice (mlc_ctx_tune_set), e.g. 'conv P1 f32x2->f32 10000x10000=1'")
    ap.add_argument("--no-profile-cache", action="store_true",
                    help="recompute every profile spectrum in every call (profiling cases only)")
    ap.add_argument("--no-autotune", action="store_true",
                    help="FFT form for every profile (for ncu captures, under which the autotuner's first-call "
                         "timings are distorted)")
    return ap.parse_args()


def sizes_for(args):
    n = args.n or (2000 if args.small else N_MAP)
    nt = args.tracks or (20000 if args.small else N_TRACKS)
    return n, nt


def workload_config(args):
    n, nt = sizes_for(args)
    full = (n, nt) == (N_MAP, N_TRACKS)
    return dict(workload="batched profiles and tracks: 10000^2 FP32 map x 16 profiles, 10^6 tracks" if full
                else f"profiling case {n}^2 x {nt} tracks (not the bench workload)", map=f"{n}x{n} ray-shot kappa*={KAPPA} gamma={GAMMA} width={WIDTH} R_E seed {MAP_SEED}",
                profiles=f"{SHAPES} x rhalf {RHALF_PX} px", tracks=nt,
                epochs=f"U{{{EPOCHS[0]}..{EPOCHS[1]}}} in {SEASONS} seasons", velocity_px_per_day=list(V_RANGE),
                l2=(f"inputs larger than L2: every map is {n * n * 4 / 1e6:.0f} MB (FP32), L2 is 129 MB"
                    if n * n * 4 > 129e6 else f"maps of {n * n * 4 / 1e6:.0f} MB (FP32) fit in the 129 MB L2"), n=n)


# ----------------------------------------------------------------------------- tracks on the device

def make_tracks_torch(ntracks, nmap, seed, device, dtype):
    """Vectorised, seeded track set: same distribution as microsn_gb300.synth.tracks."""
    import torch
    g = torch.Generator(device="cpu").manual_seed(seed)
    n = torch.randint(EPOCHS[0], EPOCHS[1] + 1, (ntracks,), generator=g)
    off = torch.zeros(ntracks + 1, dtype=torch.int64)
    off[1:] = torch.cumsum(n, 0)
    E = int(off[-1])
    tid = torch.repeat_interleave(torch.arange(ntracks), n)
    j = torch.arange(E) - off[tid]  # epoch index within its track
    nk = n[tid]
    # epochs spread over the seasons in order; jitter inside each slot keeps them sorted
    season = (j * SEASONS) // nk
    first = (season * nk + SEASONS - 1) // SEASONS
    cnt = ((season + 1) * nk + SEASONS - 1) // SEASONS - first
    u = torch.rand(E, generator=g, dtype=torch.float64)
    q = ((j - first).double() + u) / cnt.double()
    t = season.double() * (SEASON_LEN + GAP) + q * SEASON_LEN
    phi = torch.rand(ntracks, generator=g, dtype=torch.float64) * 2 * 3.141592653589793
    v = V_RANGE[0] + (V_RANGE[1] - V_RANGE[0]) * torch.rand(ntracks, generator=g, dtype=torch.float64)
    tmax = t[off[1:] - 1]
    room = 0.9 * (nmap - 2 * MARGIN)  # keep every track inside the map
    v = torch.where(v * tmax > room, room / tmax.clamp(min=1e-300), v)
    L = v * tmax
    cx, sy = torch.cos(phi), torch.sin(phi)
    lo = MARGIN + torch.clamp(-L * cx, min=0)
    hi = nmap - MARGIN - torch.clamp(L * cx, min=0)
    x0 = lo + (hi - lo) * torch.rand(ntracks, generator=g, dtype=torch.float64)
    lo = MARGIN + torch.clamp(-L * sy, min=0)
    hi = nmap - MARGIN - torch.clamp(L * sy, min=0)
    y0 = lo + (hi - lo) * torch.rand(ntracks, generator=g, dtype=torch.float64)
    host = dict(x0=x0, y0=y0, phi=phi, v=v, off=off, t=t)
    dev = {k: (a.to(device=device, dtype=dtype) if a.dtype == torch.float64 else a.to(device)) for k, a in host.items()}
    return host, dev, E


def profiles_for(n):
    import microsn_gb300 as mlc
    pix = WIDTH / n
    return [mlc.profile(s, r * pix, pix, ref_compat=False) for s in SHAPES for r in RHALF_PX]


# ----------------------------------------------------------------------------- clocks

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.lines = []
        self.p = None
        self.gpu = gpu_index

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                       "-lms", "200", "-i", str(self.gpu)], stdout=subprocess.PIPE,
                                      stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except Exception:
            self.p = None

    def _read(self):
        for line in self.p.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def max_over_ranks(x: float, device) -> float:
    """The slowest rank's x: an all-reduce MAX over the process group (NCCL on the GPUs,
    gloo in the CPU tests); x itself in a single process."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return x
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ----------------------------------------------------------------------------- roofline helpers

def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def bf16_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["bf16_tflops"]), "measured burst"
    except Exception:
        return 1900.0, "fallback"


# Pairwise chi2 workload: images A and B, 10^5 FP32 magnitude curves each, T = 128 shared
# epochs, sigma ~ U(0.02, 0.1) mag, offset-minimised magnitude-difference chi2, 1000-bin
# log10-chi2 histogram and the 10^4 smallest pairs.
PAIR_N, PAIR_T, PAIR_BINS, PAIR_K = 100_000, 128, 1000, 10_000


# The small FP64 end-to-end case: 2000^2 ray-shot map (kappa* = 0.4,
# gamma = 0.4, width 20, seed 0) convolved with a Gaussian of sigma 10 px, 10^4 straight
# tracks of 50 epochs at 5 px per epoch, offset chi2 against one noisy observed curve,
# sort and a 100-bin histogram.
C1_N, C1_TRACKS, C1_T = 2000, 10_000, 50


def c1_workload(args, ctx, dev, rank):
    import numpy as np
    import torch

    import microsn_gb300 as mlc
    from microsn_gb300 import synth
    mp, _ = synth.rayshoot_gpu(ctx, C1_N, 20.0, 0.4, 0.4, seed=0 + rank, rays_per_pixel=4.0, dtype=torch.float64)
    m = mlc.Map(ctx, mp, "f64")
    prof = mlc.profile("gaussian", 1.18 * 10.0, 1.0, ref_compat=False)
    rng = np.random.default_rng(1 + rank)
    L = 5.0 * (C1_T - 1)
    phi = rng.uniform(0, 2 * np.pi, C1_TRACKS)
    lo = 40.0 + np.maximum(-L * np.cos(phi), 0), 40.0 + np.maximum(-L * np.sin(phi), 0)
    x0 = lo[0] + rng.uniform(0, 1, C1_TRACKS) * (C1_N - 80.0 - np.abs(L * np.cos(phi)))
    y0 = lo[1] + rng.uniform(0, 1, C1_TRACKS) * (C1_N - 80.0 - np.abs(L * np.sin(phi)))
    D = lambda a: torch.as_tensor(a, dtype=torch.float64, device=dev)
    tr = [D(x0), D(y0), D(phi), D(np.full(C1_TRACKS, 5.0))]
    t = D(np.arange(C1_T, dtype=np.float64))
    conv = mlc.convolve(ctx, m, prof, "fused")
    off1 = torch.tensor([0, C1_T], dtype=torch.int64, device=dev)
    lc0 = mlc.sample_tracks(ctx, [conv], C1_N, C1_N, tr[0][:1], tr[1][:1], tr[2][:1], tr[3][:1], off1, t, mag=True)
    obs = D(lc0[0].cpu().numpy() + rng.normal(0, 0.05, C1_T))
    w = D(np.full(C1_T, 1 / 0.05 ** 2))
    chi2 = torch.empty((1, C1_TRACKS), dtype=torch.float64, device=dev)
    idx = torch.empty(C1_TRACKS, dtype=torch.int32, device=dev)

    def step(mode):
        m.refresh()
        mlc.convolve(ctx, m, prof, mode, out=conv)
        mlc.track_chi2_offset(ctx, conv, 1, *tr, t, obs, w, out=chi2)
        torch.arange(C1_TRACKS, dtype=torch.int32, device=dev, out=idx)
        mlc.sort_f64_u32(ctx, chi2[0], idx)
        return mlc.histogram_f64(ctx, chi2[0], 100, 0.0, 7.0, log=True)

    def plain_step():
        # one launch per stage, FP64: plain convolution, light curves to memory, offset chi2
        m.refresh()
        mlc.convolve(ctx, m, prof, "plain", out=conv)
        offs = torch.arange(0, (C1_TRACKS + 1) * C1_T, C1_T, dtype=torch.int64, device=dev)
        lc = mlc.sample_tracks(ctx, [conv], C1_N, C1_N, *tr, offs, t.repeat(C1_TRACKS), mag=True)
        c2, _ = mlc.chi2_offset(ctx, lc[0].reshape(C1_TRACKS, C1_T), obs.cpu().numpy(), w.cpu().numpy())
        torch.arange(C1_TRACKS, dtype=torch.int32, device=dev, out=idx)
        mlc.sort_f64_u32(ctx, c2, idx)
        return mlc.histogram_f64(ctx, c2, 100, 0.0, 7.0, log=True)

    def ff_step():
        # the fused step with the map's transforms in float-float arithmetic (FP64 results)
        m.set_fft("f32x2")
        try:
            return step("fused")
        finally:
            m.set_fft("native")

    out = {}
    chis = {}
    chi_u = torch.empty_like(chi2)
    for name, fn in (("fused", lambda: step("fused")), ("fused_f32x2", ff_step), ("plain", plain_step)):
        for _ in range(max(args.warmup, 1)):
            h = fn()
        if name != "plain":
            # per-track chi2 in track order (the step sorts its copy in place) from the
            # convolution this form just wrote
            mlc.track_chi2_offset(ctx, conv, 1, *tr, t, obs, w, out=chi_u)
            chis[name] = chi_u[0].cpu().numpy().copy()
        if name == "fused_f32x2":
            out["f32x2_vs_native_max_rel_chi2"] = float(np.max(np.abs(chis[name] - chis["fused"]) /
                                                               np.abs(chis["fused"])))
        torch.cuda.synchronize()
        steps = max(1, min(args.steps, 10))
        e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            h = fn()
        e1.record(); torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        out[name] = {"ms_per_step": ms, "light_curves_per_s": C1_TRACKS / (ms / 1000.0),
                     "histogram_total": int(np.asarray(h).sum())}
    # the same step on the host cores (oracle FP64: scipy FFT convolution + bilinear + offset
    # chi2), which is also the FP64 oracle every GPU form's chi2 is checked against
    import oracle
    oracle.build()
    mph = mp.cpu().numpy()
    P = oracle.profile("gaussian", 1.18 * 10.0, 1.0, ref_compat=False)
    t0 = time.perf_counter()
    cm = oracle.conv_fft_workers(mph, P)
    offs = np.arange(0, (C1_TRACKS + 1) * C1_T, C1_T, dtype=np.int64)
    lc = oracle.sample_tracks(cm, x0, y0, phi, np.full(C1_TRACKS, 5.0), offs, np.tile(np.arange(C1_T, dtype=float),
                                                                                      C1_TRACKS), mag=True)
    c2, _ = oracle.chi2_offset(lc.reshape(C1_TRACKS, C1_T), obs.cpu().numpy(), w.cpu().numpy())
    np.sort(c2)
    np.histogram(np.log10(c2), bins=100, range=(0.0, 7.0))
    dt_ = time.perf_counter() - t0
    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = {"kind": "port", "cores": os.cpu_count(), "ms_per_step": dt_ * 1000.0,
               "light_curves_per_s": C1_TRACKS / dt_}
    vs_oracle = {k: {"max_rel_chi2": float(np.max(np.abs(v - c2) / np.abs(c2))),
                     "max_abs_chi2": float(np.max(np.abs(v - c2)))} for k, v in chis.items()}
    m.close()
    return {"workload": "small FP64 end to end: 2000^2 FP64 ray-shot map, Gaussian sigma 10 px, 10^4 tracks x 50 epochs, "
                        "offset chi2 vs one noisy curve, radix sort, 100-bin log10 chi2 histogram",
            "fused": out["fused"], "fused_f32x2": out["fused_f32x2"], "plain_fp64": out["plain"],
            "fused_over_plain": out["plain"]["ms_per_step"] / out["fused"]["ms_per_step"],
            "fused_f32x2_over_plain": out["plain"]["ms_per_step"] / out["fused_f32x2"]["ms_per_step"],
            "f32x2_vs_native_max_rel_chi2": out["f32x2_vs_native_max_rel_chi2"], "cpu": cpu, "dtype": "f64",
            "max_rel_err_vs_fp64": max(v["max_rel_chi2"] for v in vs_oracle.values()),
            "vs_fp64_oracle": dict(vs_oracle, what=f"offset chi2 of all {C1_TRACKS} tracks against the FP64 oracle "
                                                   "(scipy FFT convolution, C bilinear magnitudes, offset chi2)"),
            "f32x2": "FP64 map whose forward transform and fused convolution run in float-float arithmetic "
                     "(pairs of FP32); pixels, light curves and chi2 FP64"}


# The differentiable fit: 4000^2 FP32 map, thin-disc radius stack (16 radii,
# 4..32 px), 4096 tracks = 64 targets x 64 perturbed starts, 80 uneven epochs each, fused
# chi2 + gradient kernel with an Adam step, replayed from a CUDA graph.
C4_N, C4_TARGETS, C4_STARTS, C4_T = 4000, 64, 64, 80


def c4_workload(args, ctx, dev, rank):
    import numpy as np
    import torch

    import microsn_gb300 as mlc
    from microsn_gb300 import synth
    mp, _ = synth.rayshoot_gpu(ctx, C4_N, 20.0, 0.45, 0.35, seed=5 + rank, rays_per_pixel=4.0, dtype=torch.float32)
    m = mlc.Map(ctx, mp, "f32")
    radii = list(np.geomspace(4.0, 32.0, 16))
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    stack = mlc.radius_stack(ctx, m, radii)
    e1.record(); torch.cuda.synchronize()
    stack_ms = e0.elapsed_time(e1)
    rng = np.random.default_rng(5 + rank)
    n = C4_TARGETS * C4_STARTS
    t1 = np.sort(rng.integers(0, 3, (C4_TARGETS, C4_T)) * 365.0 + rng.uniform(0, 150, (C4_TARGETS, C4_T)), axis=1)
    v = rng.uniform(0.02, 0.08, C4_TARGETS); phi = rng.uniform(0, 2 * np.pi, C4_TARGETS)
    span = v * t1[:, -1]
    mg = 80.0
    x0 = mg + np.maximum(-span * np.cos(phi), 0) + rng.uniform(0, 1, C4_TARGETS) * (C4_N - 2 * mg - np.abs(span * np.cos(phi)))
    y0 = mg + np.maximum(-span * np.sin(phi), 0) + rng.uniform(0, 1, C4_TARGETS) * (C4_N - 2 * mg - np.abs(span * np.sin(phi)))
    true = np.stack([x0, y0, phi, v, rng.uniform(8, 16, C4_TARGETS), rng.uniform(-0.3, 0.3, C4_TARGETS)], 1)
    D = lambda a, dt=torch.float32: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=dev)
    offT = np.arange(C4_TARGETS + 1, dtype=np.int64) * C4_T
    _, _, model = mlc.track_fit(ctx, stack, radii, D(true), D(offT, torch.int64), D(t1.ravel()),
                                D(np.zeros(C4_TARGETS * C4_T)), D(np.ones(C4_TARGETS * C4_T)), grad=False, model=True)
    obs1 = model.cpu().numpy() + rng.normal(0, 0.02, C4_TARGETS * C4_T)
    idx = np.repeat(np.arange(C4_TARGETS), C4_STARTS)
    scale = np.array([2.0, 2.0, 0.02, 0.002, 1.5, 0.1])
    th0 = true[idx] + rng.normal(0, 1, (n, 6)) * scale
    th0[:, 4] = np.clip(th0[:, 4], radii[0], radii[-1])
    sel = (idx[:, None] * C4_T + np.arange(C4_T)[None, :]).ravel()
    off = D(np.arange(n + 1, dtype=np.int64) * C4_T, torch.int64)
    t = D(t1.ravel()[sel]); obs = D(obs1[sel]); w = D(np.full(n * C4_T, 1 / 0.02 ** 2))
    sc = D(scale)
    u = D(th0 / scale)
    th = torch.empty_like(u)
    c2 = torch.empty(n, dtype=torch.float32, device=dev)
    g = torch.empty((n, 6), dtype=torch.float32, device=dev)
    m1 = torch.zeros_like(u); m2 = torch.zeros_like(u)
    b1, b2, lr, eps = 0.9, 0.999, 0.05, 1e-8
    bc = torch.ones(2, dtype=torch.float32, device=dev)  # running bias corrections
    betas = torch.tensor([b1, b2], dtype=torch.float32, device=dev)

    def it():
        torch.mul(u, sc, out=th)
        mlc.track_fit(ctx, stack, radii, th, off, t, obs, w, out_chi2=c2, out_grad=g)
        gu = g * sc
        m1.mul_(b1).add_(gu, alpha=1 - b1)
        m2.mul_(b2).addcmul_(gu, gu, value=1 - b2)
        bc.mul_(betas)
        u.sub_(lr * (m1 / (1 - bc[0])) / ((m2 / (1 - bc[1])).sqrt() + eps))

    # warm up on a side stream, capture one iteration, replay it
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    old = ctx.stream
    with torch.cuda.stream(s):
        ctx.set_stream(s)
        u0 = u.clone()
        for _ in range(3):
            it()
        u.copy_(u0); m1.zero_(); m2.zero_(); bc.fill_(1.0)
    torch.cuda.current_stream().wait_stream(s)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        ctx.set_stream(torch.cuda.current_stream())
        it()
    ctx.set_stream(old)
    iters = 300
    torch.cuda.synchronize()
    e0.record()
    for _ in range(iters):
        graph.replay()
    e1.record(); torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    # kernel-only throughput of the fused chi2 + gradient kernel
    ctx.set_timing(True)
    for _ in range(20):
        mlc.track_fit(ctx, stack, radii, th, off, t, obs, w, out_chi2=c2, out_grad=g)
    kt = ctx.kernel_times(reset=True)
    ctx.set_timing(False)
    k_ms = kt["track_fit"][0] / kt["track_fit"][1]
    final = c2.cpu().numpy().reshape(C4_TARGETS, C4_STARTS)
    torch.mul(u, sc, out=th)
    mlc.track_fit(ctx, stack, radii, D(true), D(offT, torch.int64), D(t1.ravel()), D(obs1),
                  D(np.full(C4_TARGETS * C4_T, 1 / 0.02 ** 2)), out_chi2=c2[:C4_TARGETS], out_grad=g[:C4_TARGETS])
    true_c2 = c2[:C4_TARGETS].cpu().numpy()
    recovered = float(np.mean(final.min(axis=1) <= 1.2 * true_c2 + 5.0))
    m.close()
    return {"workload": "gradient fit: 4000^2 FP32 map, 16-radius thin-disc stack, 4096 tracks (64 targets x 64 "
                        "starts) x 80 uneven epochs, 6 parameters, Adam from a CUDA graph",
            "stack_build_ms": stack_ms, "iteration_ms": ms / iters,
            "gradient_evaluations_per_s": n / (ms / iters / 1000.0),
            "kernel_ms": k_ms, "track_epochs_per_s_kernel": n * C4_T / (k_ms / 1000.0),
            "iterations": iters, "targets_recovered_fraction": recovered,
            "median_best_over_true_chi2": float(np.median(final.min(axis=1) / true_c2))}


# Supernova, multi-band and multi-image: four 8192^2 FP32 maps (one per lensed
# image, seeds 6..9, distinct kappa* and gamma), an expanding photosphere R(t) from 1 to
# 100 px over 40 epochs in 3 bands (limb-darkened discs, one limb-darkening coefficient
# per band) = 120 convolutions per map, 2x10^5 tracks per image sampled at the epochs,
# then the offset magnitude-difference chi2 of every track pair of the 6 image pairs
# (T = 120) with a 1000-bin log histogram and the 10^4 smallest per pair.
C5_N, C5_EPOCHS, C5_TRACKS = 8192, 40, 200_000
C5_LENS = [(0.40, 0.35), (0.45, 0.40), (0.50, 0.45), (0.55, 0.50)]
C5_U = (0.6, 0.45, 0.3)


def c5_workload(args, ctx, dev, rank):
    import itertools

    import numpy as np
    import torch

    import microsn_gb300 as mlc
    from microsn_gb300 import synth
    N = C5_N
    ntr = min(C5_TRACKS, args.tracks) if args.tracks else C5_TRACKS
    maps = []
    for i, (ks, g) in enumerate(C5_LENS):
        mp, _ = synth.rayshoot_gpu(ctx, N, 20.0, ks, g, seed=6 + i + 10 * rank, rays_per_pixel=4.0,
                                   dtype=torch.float32)
        maps.append(mlc.Map(ctx, mp, "f32"))
        del mp
    R = np.linspace(1.0, 100.0, C5_EPOCHS)
    profs = [mlc.profile("limb_darkened", r / np.sqrt(2.0), 1.0, ref_compat=False, u=u) for r in R for u in C5_U]
    nb = len(C5_U)
    conv = torch.empty((len(profs), N, N), dtype=torch.float32, device=dev)  # 32 GB
    rng = np.random.default_rng(60 + rank)
    t = torch.as_tensor(np.arange(C5_EPOCHS) * 2.0, dtype=torch.float32, device=dev)  # every 2 days
    span = 2.0 * (C5_EPOCHS - 1)
    tracks = []
    for i in range(len(maps)):
        v = rng.uniform(0.2, 1.0, ntr); phi = rng.uniform(0, 2 * np.pi, ntr)
        L = v * span; mg = 110.0
        x0 = mg + np.maximum(-L * np.cos(phi), 0) + rng.uniform(0, 1, ntr) * (N - 2 * mg - np.abs(L * np.cos(phi)))
        y0 = mg + np.maximum(-L * np.sin(phi), 0) + rng.uniform(0, 1, ntr) * (N - 2 * mg - np.abs(L * np.sin(phi)))
        tracks.append([torch.as_tensor(a, dtype=torch.float32, device=dev) for a in (x0, y0, phi, v)])
    T = C5_EPOCHS * nb
    w = 1.0 / rng.uniform(0.02, 0.1, T) ** 2
    pairs = list(itertools.combinations(range(len(maps)), 2))
    e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]

    def step():
        """Per image: its convolutions (one CUDA graph), then its pair side straight from the
        convolved maps (sample -> magnitude -> centre -> sliced integers, no light curve);
        then the tensor-core chi2 of every track pair of every image pair."""
        sides, t_conv, t_side = [], 0.0, 0.0
        for i, m in enumerate(maps):
            m.refresh()
            e[0].record()
            mlc.convolve_many(ctx, m, profs, out=conv, graph=True)
            e[1].record()
            sides.append(mlc.PairSide.expanding(ctx, conv, C5_EPOCHS, nb, *tracks[i], t, w, None, True))
            e[2].record()
            torch.cuda.synchronize()
            t_conv += e[0].elapsed_time(e[1]); t_side += e[1].elapsed_time(e[2])
        e[0].record()
        res = [mlc.pair_chi2_sides(ctx, sides[a], sides[b], nbins=PAIR_BINS, lo=-1.0, hi=9.0, k=PAIR_K)
               for a, b in pairs]
        e[1].record()
        torch.cuda.synchronize()
        for sd in sides:
            sd.close()
        return res, t_conv, t_side, e[0].elapsed_time(e[1])

    step()  # warm-up: captures the convolution graphs, sizes the workspaces
    torch.cuda.synchronize()
    nsteps = max(1, min(args.steps, 2))
    t_conv = t_sides = t_pairs = 0.0
    for _ in range(nsteps):
        res, a, b, c = step()
        t_conv += a; t_sides += b; t_pairs += c
    t_conv /= nsteps; t_sides /= nsteps; t_pairs /= nsteps
    # the same convolutions without the graph, for the launch-overhead comparison
    e[0].record()
    for m in maps:
        mlc.convolve_many(ctx, m, profs, out=conv, graph=False)
    e[1].record(); torch.cuda.synchronize()
    conv_eager = e[0].elapsed_time(e[1])
    e[0].record()
    for m in maps:
        mlc.convolve_many(ctx, m, profs, out=conv, graph=True)
    e[1].record(); torch.cuda.synchronize()
    conv_graph = e[0].elapsed_time(e[1])
    # the two-stage form it replaces (light curves of every image stored, then each image
    # pair prepared from them), timed once with the convolutions of the last image reused
    lc = torch.empty((ntr, T), dtype=torch.float32, device=dev)
    lcs = [lc, torch.empty_like(lc)]
    e[0].record()
    mlc.sample_expanding(ctx, conv, nb, *tracks[len(maps) - 1], t, out=lcs[0])
    e[1].record()
    mlc.sample_expanding(ctx, conv, nb, *tracks[0], t, out=lcs[1])
    mlc.pair_chi2_magdiff(ctx, lcs[0], lcs[1], w, None, True, method="tensor", nbins=PAIR_BINS, lo=-1.0, hi=9.0,
                          k=PAIR_K)
    e[2].record(); torch.cuda.synchronize()
    two_stage_curves_ms = e[0].elapsed_time(e[1])
    two_stage_pair_ms = e[1].elapsed_time(e[2]) - two_stage_curves_ms
    del lcs, lc
    npairs = len(pairs) * float(ntr) * ntr
    total = t_conv + t_sides + t_pairs
    # parity on a fixed subset (1000 tracks of the last image x 1000 of image 0, on the last
    # image's convolved maps): the fused sides equal the two-stage tensor form bit for bit,
    # and the tensor-core chi2 stays within 1e-5 of the FP64 plain kernel on the same curves
    sa = torch.randperm(ntr, generator=torch.Generator().manual_seed(4))[:1000].to(dev)
    sb = torch.randperm(ntr, generator=torch.Generator().manual_seed(5))[:1000].to(dev)
    ta = [a[sa].contiguous() for a in tracks[len(maps) - 1]]
    tb = [a[sb].contiguous() for a in tracks[0]]
    As = mlc.sample_expanding(ctx, conv, nb, *ta, t)
    Bs = mlc.sample_expanding(ctx, conv, nb, *tb, t)
    kw = dict(nbins=PAIR_BINS, lo=-1.0, hi=9.0, k=PAIR_K, want_matrix=True)
    sA = mlc.PairSide.expanding(ctx, conv, C5_EPOCHS, nb, *ta, t, w, None, True)
    sB = mlc.PairSide.expanding(ctx, conv, C5_EPOCHS, nb, *tb, t, w, None, True)
    fused = mlc.pair_chi2_sides(ctx, sA, sB, **kw)
    sA.close(); sB.close()
    two = mlc.pair_chi2_magdiff(ctx, As, Bs, w, None, True, method="tensor", **kw)
    plain = mlc.pair_chi2_magdiff(ctx, As, Bs, w, None, True, method="plain", **kw)["matrix"].double()
    mt = fused["matrix"].double()
    pair_rel = ((mt - plain).abs() / plain.abs().clamp_min(1e-30)).max().item()
    fused_equal = bool(torch.equal(fused["matrix"], two["matrix"]) and np.array_equal(fused["hist"], two["hist"])
                       and np.array_equal(fused["topk_val"], two["topk_val"]))
    del mt, plain, As, Bs, fused, two
    out = {"workload": f"supernova: {len(maps)} x {N}^2 FP32 maps, {len(profs)} limb-darkened expanding-photosphere "
                       f"profiles per map ({C5_EPOCHS} epochs x {nb} bands), {ntr} tracks per image, offset "
                       f"magnitude-difference chi2 of all track pairs of {len(pairs)} image pairs (T = {T})",
           "form": "per image: convolutions as one CUDA graph, then a pair side sampled straight from the convolved "
                   "maps (no light curves in HBM); per image pair: the tensor-core chi2 of the two sides",
           "ms_per_step": total, "conv_ms": t_conv, "sides_ms": t_sides, "pairs_ms": t_pairs,
           "two_stage": {"what": "the form this replaces, for one image pair: light curves written to HBM, then "
                                 "both sides prepared from them inside the pair call",
                         "curves_ms_per_image": two_stage_curves_ms, "pair_ms_per_image_pair": two_stage_pair_ms,
                         "sides_ms_per_image": t_sides / len(maps), "pairs_ms_per_image_pair": t_pairs / len(pairs)},
           "light_curves_per_s": len(maps) * ntr * nb / (total / 1000.0),
           "pair_chi2_per_s": npairs / (t_pairs / 1000.0),
           "convolutions_per_s": len(maps) * len(profs) / (t_conv / 1000.0),
           "conv_ms_graph": conv_graph, "conv_ms_eager": conv_eager,
           "refined_pairs": int(sum(r["stats"]["refined"] for r in res)),
           "histogram_total": float(sum(float(r["hist"].sum()) for r in res)),
           "histogram_below_range": int(sum(r["stats"]["below"] for r in res)),
           "histogram_above_range": int(sum(r["stats"]["above"] for r in res)),
           "pairs_total": npairs,
           "max_rel_err_vs_fp64": pair_rel,
           "parity_subset": {"pairs": 1000 * 1000, "max_rel_err_vs_fp64": pair_rel, "tolerance": 1e-5,
                             "fused_equals_two_stage": fused_equal,
                             "what": "fused sides vs the two-stage tensor form (bit for bit) and the tensor-core "
                                     "pair chi2 vs the FP64 plain kernel on the same FP32 light curves (1000 x 1000 "
                                     "fixed tracks of two images on one image's convolved maps)"}}
    for m in maps:
        m.close()
    del conv
    torch.cuda.empty_cache()
    return out


# Multi-filter flux-ratio likelihood at the reference chi2 driver's size
# (chi2/chi2_driver.cu: N = 10^4 locations per image, F = 7 filters, T = 10 epochs).
FR_N, FR_F, FR_T = 10_000, 7, 10


RATIO_NLOC, RATIO_SIZES, RATIO_SEED = 9216, [0.0, 0.05, 0.1, 0.2, 0.3], 5
RATIO_D, RATIO_S, RATIO_T = [0.7, 1.2, 1.4, 1.1, 0.9], [0.1, 0.15, 0.1, 0.1, 0.15], [5.0, 7.0, 12.0, 14.0, 17.0]


def ratio_pair_workload(args, ctx, m, dev, rank):
    """The reference's own pair path at its own size (driver.cpp:143-234 with random
    locations, Nloc = 9216, 5 sizes, 300 log bins, 5 data points): light curves of two FP64
    maps at fixed locations (expanding_source), the z-rank sort (setup_integral), and per
    likelihood evaluation the ratio chi2 of all Nloc^2 pairs + bin means (reference form:
    calculate_chi2 + bin_chi2) or the rank-free fused kernel; the oracle's C restatement of
    calculate_chi2_CPU + bin_chi2_CPU timed on one core on a subset of locations."""
    import numpy as np
    import torch

    import microsn_gb300 as mlc
    import oracle
    n = m.Nx
    Nloc = RATIO_NLOC if not args.small else 1024
    mA = mlc.Map(ctx, m.tensor().double(), "f64")
    mB = mlc.Map(ctx, torch.flip(m.tensor(), [0, 1]).double().contiguous(), "f64")  # image B: the map turned 180 deg
    mA_host = mA.tensor().cpu().numpy() if oracle.refcuda_available() else None
    mB_host = mB.tensor().cpu().numpy() if oracle.refcuda_available() else None
    Noff = int(np.ceil((n / WIDTH) * RATIO_SIZES[-1]))
    lx, ly = mlc.locations_random(Nloc, n, Noff, RATIO_SEED + rank)
    base = mlc.profile("gaussian", 0.0, WIDTH / n)
    ev = lambda: (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
    e0, e1 = ev()
    e0.record()
    LCA, DLCA = mlc.expanding_source(ctx, mA, RATIO_SIZES, base, WIDTH, lx, ly)
    LCB, DLCB = mlc.expanding_source(ctx, mB, RATIO_SIZES, base, WIDTH, lx, ly)
    e1.record()
    torch.cuda.synchronize()
    es_ms = e0.elapsed_time(e1)
    del mA, mB
    edges = mlc.bin_edges(300, 1e-4, 300.0, True)
    Dfac = np.sqrt(1750.0 * 850.0 / 1570.0)
    v = mlc.setup_chi2_calculation((0.4, 0.5), (1.0,), Dfac, np.array(RATIO_D), np.array(RATIO_T),
                                   np.array(RATIO_S), np.array(RATIO_SIZES))

    def timed(fn, k):
        fn()
        torch.cuda.synchronize()
        a, b = ev()
        a.record()
        for _ in range(k):
            r = fn()
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b) / k, r

    setup_ms, (rank_t, lower, nper) = timed(lambda: mlc.setup_integral(ctx, LCA, LCB, edges), 3)
    ref_ms, (bc, be) = timed(lambda: mlc.bin_chi2(ctx, lower, nper, mlc.calculate_chi2(ctx, v, LCA, DLCA, LCB, DLCB,
                                                                                        rank_t)), 5)
    fused_ms, (fb, fe, fn_) = timed(lambda: mlc.pair_bin_fused(ctx, v, LCA, DLCA, LCB, DLCB, edges), 5)
    full = nper > 0
    agree = bool(np.array_equal(fn_, nper) and np.allclose(fe[full], be[full], rtol=1e-12, atol=0))
    pairs = float(Nloc) * Nloc
    # CPU: the oracle's restatement of calculate_chi2_CPU + bin_chi2_CPU on a subset, one core
    cpu = None
    if rank == 0 and not args.no_cpu:
        sub_n = 1200
        A = LCA[:sub_n].cpu().numpy(); B = LCB[:sub_n].cpu().numpy()
        dA = DLCA[:sub_n].cpu().numpy(); dB = DLCB[:sub_n].cpu().numpy()
        r_o, l_o, n_o = oracle.pair_rank(A, B, edges)
        ov = dict(Njp=v.Njp, indA=v.indA, indB=v.indB, facA=v.facA, facB=v.facB, d=v.d, s=v.s)
        t0 = time.perf_counter()
        c_o = oracle.pair_chi2_ratio(ov, A, dA, B, dB, r_o)
        oracle.bin_chi2(l_o, n_o, c_o)
        dt = time.perf_counter() - t0
        cpu = {"kind": "port", "cores": 1, "pairs_per_s": sub_n * sub_n / dt,
               "sample": f"{sub_n}^2 pairs of the same curves (calculate_chi2 + bin_chi2 restated in C)"}
    # the reference's own CUDA build on the same inputs and GPU (compiled unchanged for sm_103a
    # from the staged sources): its expanding_source on both maps (cuFFT, host rasters and a
    # host-built full-size kernel per profile, as it is written) and its pair path, timed
    # around each call, with its outputs compared with the library's
    refc = None
    if rank == 0 and oracle.refcuda_available() and n == 10000:
        try:
            mpA = mA_host
            mpB = mB_host
            pixr = WIDTH / n
            LCr_A, DLCr_A, msA = oracle.refcuda_expanding_source(mpA, RATIO_SIZES, "gaussian", lx, ly, pixr, WIDTH)
            LCr_B, DLCr_B, msB = oracle.refcuda_expanding_source(mpB, RATIO_SIZES, "gaussian", lx, ly, pixr, WIDTH)
            ov = dict(Njp=v.Njp, indA=v.indA, indB=v.indB, facA=v.facA, facB=v.facB, d=v.d, s=v.s)
            rp = oracle.refcuda_pair_path(LCr_A, DLCr_A, LCr_B, DLCr_B, ov, edges, want_rank=False)
            lA = LCA.cpu().numpy()
            rel_lc = float(np.max(np.abs(lA - LCr_A) / np.maximum(np.abs(LCr_A), 1e-3 * np.mean(LCr_A))))
            fullr = rp["nper"] > 0
            refc = {"what": "the reference's gpu_functions.cu / data_structs.cu built unchanged for sm_103a "
                            "(cuFFT, thrust), on the same maps, locations, sizes and bins",
                    "expanding_source_ms_two_maps": msA + msB,
                    "expanding_source_over_library": (msA + msB) / es_ms,
                    "setup_integral_ms": rp["ms"][0], "calculate_chi2_ms": rp["ms"][1], "bin_chi2_ms": rp["ms"][2],
                    "pairs_per_s": pairs / ((rp["ms"][1] + rp["ms"][2]) / 1000.0),
                    "library_reference_form_over_it": (rp["ms"][1] + rp["ms"][2]) / ref_ms,
                    "library_fused_over_it": (rp["ms"][1] + rp["ms"][2]) / fused_ms,
                    "LC_max_rel_vs_library": rel_lc,
                    "bins_equal": bool(np.array_equal(rp["nper"], nper) and np.array_equal(rp["lower"], lower)),
                    "binned_chi2_max_rel_vs_library": float(np.max(np.abs(rp["bchi2"][fullr] - bc[fullr]) /
                                                                   np.abs(bc[fullr]))) if fullr.any() else None,
                    "timing": "wall clock around each call (each synchronises internally)"}
        except Exception as ex:  # report, do not fail the bench
            refc = {"error": str(ex)[:200]}
    return {"metric": "pair-chi2/s (reference ratio form)", "unit": "pair-chi2/s",
            "reference_cuda": refc,
            "config": {"workload": f"two {n}^2 FP64 maps (the bench map and its 180-degree turn), {Nloc} random "
                                   f"locations, sizes {RATIO_SIZES} R_E gaussian, 300 log z-bins, Nd = 5",
                       "pairs_per_evaluation": pairs},
            "expanding_source_ms_two_maps": es_ms, "setup_integral_ms": setup_ms,
            "reference_form": {"ms_per_evaluation": ref_ms, "value": pairs / (ref_ms / 1000.0)},
            "fused": {"ms_per_evaluation": fused_ms, "value": pairs / (fused_ms / 1000.0)},
            "fused_equals_reference_form": agree, "cpu": cpu}


def mpd_workload(args, ctx, m, rank):
    """The map's binned magnification distribution (getBinnedMpd, magnification_map_gpu.cu:45-87)
    of the bench map in FP64 with the reference input's bins (500 log bins, 1e-4..400): one
    pass with shared-memory counters on the GPU, against the oracle's C restatement of the
    reference's sort-and-upper_bound form on one host core, bins compared bit for bit."""
    import numpy as np
    import torch

    import microsn_gb300 as mlc
    import oracle
    m64 = mlc.Map(ctx, m.tensor().double(), "f64")
    nb, lo, hi = 500, 1e-4, 400.0
    mlc.map_binned_mpd(ctx, m64, nb, lo, hi)
    torch.cuda.synchronize()
    k = 5
    t0 = time.perf_counter()
    for _ in range(k):
        bins, counts = mlc.map_binned_mpd(ctx, m64, nb, lo, hi)  # returns host arrays (synchronous)
    gpu_ms = (time.perf_counter() - t0) * 1000.0 / k
    res = {"workload": f"{m.Nx}^2 FP64 map, {nb} log bins {lo}..{hi}", "gpu_ms": gpu_ms,
           "pixels_per_s": m.Nx * m.Ny / (gpu_ms / 1000.0)}
    if rank == 0 and not args.no_cpu:
        host = m64.tensor().cpu().numpy()
        t0 = time.perf_counter()
        b_o, c_o = oracle.binned_mpd(host, nb, lo, hi)
        res["cpu"] = {"kind": "port", "cores": 1, "ms": (time.perf_counter() - t0) * 1000.0,
                      "sample": "the whole map"}
        res["bins_equal"] = bool(np.array_equal(bins, b_o) and np.array_equal(counts, c_o))
    del m64
    return res


def flux_ratio_workload(args, ctx, dev, rank):
    import numpy as np
    import torch

    import microsn_gb300 as mlc
    rng = np.random.default_rng(13 + rank)
    fo = rng.uniform(0.8, 1.2, (FR_F, FR_T)).astype(np.float32)
    dfo = rng.uniform(0.05, 0.2, (FR_F, FR_T)).astype(np.float32)
    m1 = torch.as_tensor(rng.lognormal(0.0, 0.3, (FR_N, FR_F, FR_T)).astype(np.float32), device=dev)
    m2 = torch.as_tensor(rng.lognormal(0.0, 0.3, (FR_N, FR_F, FR_T)).astype(np.float32), device=dev)
    for _ in range(max(args.warmup, 1)):
        mlc.flux_ratio_chi2(ctx, fo, dfo, m1, m2)
    torch.cuda.synchronize()
    ctx.set_timing(True)
    steps = max(1, min(args.steps, 10))
    for _ in range(steps):
        like = mlc.flux_ratio_chi2(ctx, fo, dfo, m1, m2)
    kt = ctx.kernel_times(reset=True)
    ctx.set_timing(False)
    ms = sum(v[0] for v in kt.values()) / steps
    pairs = FR_N * FR_N
    k_ms = kt["flux_ratio_chi2"][0] / kt["flux_ratio_chi2"][1]
    flops = 3.0 * FR_F * FR_T * pairs  # one FMA + one multiply + one FMA per pair and (filter, epoch)
    return {"metric": "flux-ratio pair likelihood terms/s", "value": pairs / (ms / 1000.0), "unit": "pairs/s",
            "ms_per_call": ms, "config": {"N": FR_N, "F": FR_F, "T": FR_T, "data": "synthetic lognormal fluxes"},
            "likelihood": like, "kernel_ms": k_ms, "fp32_tflops": flops / (k_ms / 1000.0) / 1e12,
            "bound": "FP32 pipe (3 FP32 operations per pair and (filter, epoch))"}


def pair_workload(args, ctx, m, profs, n, dev, world, rank, stream):
    import numpy as np
    import torch

    import microsn_gb300 as mlc
    N = min(PAIR_N, args.tracks or PAIR_N) if args.small or args.tracks else PAIR_N
    # curves: 2N straight tracks with 128 epochs over three seasons, sampled on two
    # convolved maps (thin disc 16 px for image A, uniform 16 px for image B)
    g = torch.Generator(device="cpu").manual_seed(7 + rank)
    T = PAIR_T
    ntr = 2 * N
    season = torch.arange(T) * 3 // T
    base_t = season.double() * (SEASON_LEN + GAP) + (torch.arange(T) % (T // 3 + 1)).double() * (SEASON_LEN / (T // 3 + 1))
    t = base_t.repeat(ntr)
    off = torch.arange(0, ntr + 1, dtype=torch.int64) * T
    phi = torch.rand(ntr, generator=g, dtype=torch.float64) * 6.283185307179586
    v = 0.05 + 0.45 * torch.rand(ntr, generator=g, dtype=torch.float64)
    L = v * base_t[-1]
    x0 = MARGIN + torch.clamp(-L * torch.cos(phi), min=0) + (n - 2 * MARGIN - L.abs()) * torch.rand(ntr, generator=g, dtype=torch.float64)
    y0 = MARGIN + torch.clamp(-L * torch.sin(phi), min=0) + (n - 2 * MARGIN - L.abs()) * torch.rand(ntr, generator=g, dtype=torch.float64)
    f = lambda a: a.to(device=dev, dtype=torch.float32)
    convs = [mlc.convolve(ctx, m, profs[len(RHALF_PX) + 3], "fused"), mlc.convolve(ctx, m, profs[3], "fused")]
    mags = mlc.sample_tracks(ctx, convs, n, n, f(x0), f(y0), f(phi), f(v), off.to(dev), f(t), mag=True)
    del convs
    A = mags[0, : N * T].reshape(N, T).contiguous()
    B = mags[1, N * T:].reshape(N, T).contiguous()
    rng = np.random.default_rng(11 + rank)
    w = 1.0 / rng.uniform(0.02, 0.1, T) ** 2
    d = np.zeros(T)

    def pstep():
        return mlc.pair_chi2_magdiff(ctx, A, B, w, d, True, method="tensor", nbins=PAIR_BINS, lo=-1.0, hi=9.0,
                                     k=PAIR_K)

    for _ in range(max(args.warmup, 1)):
        r = pstep()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
    psteps = max(1, min(args.steps, 5))
    if world > 1:
        torch.distributed.barrier()
    e0.record(stream)
    for _ in range(psteps):
        r = pstep()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = max_over_ranks(e0.elapsed_time(e1) / psteps, dev)
    pairs = float(N) * N
    value = world * pairs / (ms / 1000.0)
    # per-kernel times of one step
    ctx.set_timing(True)
    pstep()
    kt = ctx.kernel_times(reset=True)
    ctx.set_timing(False)
    tc_ms = kt.get("pairdiff_tc", (float("nan"), 1))[0]
    Kp = ((T + 63) // 64) * 64
    napad, nbpad = ((N + 127) // 128) * 128, ((N + 47) // 48) * 48
    executed = 9 * 2.0 * Kp * napad * nbpad  # 9 bf16 slice products per epoch per pair
    peak, pk = bf16_peak()
    ach = executed / (tc_ms / 1000.0) / 1e12
    # plain FP64 form on a subset of rows (same statistic, one launch per stage)
    sub_rows = 1000
    mlc.pair_chi2_magdiff(ctx, A[:sub_rows], B, w, d, True, method="plain", nbins=PAIR_BINS, lo=-1.0, hi=9.0,
                          k=min(PAIR_K, 1000))
    torch.cuda.synchronize()
    e0.record(stream)
    mlc.pair_chi2_magdiff(ctx, A[:sub_rows], B, w, d, True, method="plain", nbins=PAIR_BINS, lo=-1.0, hi=9.0,
                          k=min(PAIR_K, 1000))
    e1.record(stream)
    torch.cuda.synchronize()
    pms = e0.elapsed_time(e1)
    plain_val = world * sub_rows * float(N) / (pms / 1000.0)
    # parity on a fixed 10^6-pair subset at full scale: the tensor-core chi2 matrix against
    # the FP64 plain kernel on the same 1000 x 1000 curves
    sa = torch.randperm(N, generator=torch.Generator().manual_seed(4))[:1000].to(A.device)
    sb = torch.randperm(N, generator=torch.Generator().manual_seed(5))[:1000].to(A.device)
    As, Bs = A[sa].contiguous(), B[sb].contiguous()
    mt = mlc.pair_chi2_magdiff(ctx, As, Bs, w, d, True, method="tensor", nbins=PAIR_BINS, lo=-1.0, hi=9.0,
                               want_matrix=True)["matrix"].double()
    mp_ = mlc.pair_chi2_magdiff(ctx, As, Bs, w, d, True, method="plain", nbins=PAIR_BINS, lo=-1.0, hi=9.0,
                                want_matrix=True)["matrix"].double()
    rel = ((mt - mp_).abs() / mp_.abs().clamp_min(1e-30)).max().item()
    return {"metric": "pair-chi2/s", "value": value, "unit": "pair-chi2/s", "ms_per_step": ms, "steps": psteps,
            "parity_subset": {"pairs": 1000 * 1000, "max_rel_err_vs_fp64": rel, "tolerance": 1e-5},
            "config": {"workload": f"images A, B: {N} x {N} FP32 magnitude curves, T={T} shared epochs, "
                                   f"sigma~U(0.02,0.1), offset-minimised, {PAIR_BINS}-bin log10-chi2 histogram, "
                                   f"top-{PAIR_K}", "pairs_per_step": pairs,
                       "curves": "bilinear samples of two convolved maps of the bench map"},
            "roofline": {"kernel": "pairdiff_tc", "bound": "tensor", "achieved": ach, "peak": peak,
                         "unit": "TFLOP/s", "frac": ach / peak, "traffic": None,
                         "flops_per_launch": executed, "launch_ms": tc_ms,
                         "useful_tflops": 2.0 * T * pairs / (tc_ms / 1000.0) / 1e12,
                         "peak_source": f"{pk} bf16 dense (MEASURED_PEAKS.json bf16_tflops)",
                         "note": "executed = 9 bf16 slice products (exact 24-bit sliced integers) per epoch per pair"},
            "kernels_ms": {k_: v_[0] for k_, v_ in kt.items()},
            "stats": r["stats"],
            "plain_fp64": {"value": plain_val, "unit": "pair-chi2/s", "ms": pms, "pairs": sub_rows * N,
                           "batched_over_plain": value / plain_val}}


def algorithmic_bytes(name, n, E, nprof, e=4, es=None):
    """Algorithmic bytes of one launch of each kernel at this workload: real values of e
    bytes (FP32 maps, light curves, epochs), spectra of complex values of 2 es bytes (es = e
    for FP32 transforms, 8 for float-float transforms)."""
    Wc = n // 2 + 1
    spec = n * Wc * 2 * (es or e)  # complex half spectrum
    real = n * n * e
    table = {
        "fft_rows_r2c": real + spec,           # read a real map, write its row spectra
        "fft_profile_rows": None,              # a profile's 2h rows: L2-resident, a few MB
        "fft_rows_c2r": spec + real,           # read row spectra, write a real map
        "fft_col_A": 2 * spec,                 # in-place column sub-pass: read + write
        "fft_col_B": 2 * spec,
        "conv_fused_spectrum": 2 * spec,       # read map spectrum, write product sub-pass output
        "conv_cached_spectrum": 3 * spec,      # read map and cached profile spectra, write the product pass
        "sample_tracks": E * e + nprof * real + E * nprof * e,  # t in, one read of each map, LCs out
        "sample_tracks_il": E * e + nprof * real + E * nprof * e,
        "interleave": 2 * nprof * real,          # read nprof planar maps, write the interleaved map
        # last inverse pass of a group's profiles with the interleave (one launch per group):
        # read each profile's half spectrum, write its values into the interleaved map
        "fft_rows_c2r_interleave": nprof * (spec + real),
        "conv_direct": 2 * real,                  # read the map, write the convolved map
    }
    return table.get(name)


def load_traffic():
    """DRAM bytes per launch from the committed ncu summary (scaled there to a full launch)."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            return json.load(f)
    except Exception:
        return {}


# ----------------------------------------------------------------------------- chi2 error against FP64

CHI2_SIGMA, CHI2_NOISE_SEED = 0.05, 11


def chi2_errors(forms, ref, off):
    """Offset-minimised chi2 of every track's light curve against an observed curve, from
    each form's light curves (forms: name -> (P, E) tensor) and from the FP64 step's (ref),
    on the same inputs: max relative and absolute chi2 error over all tracks and profiles,
    and the largest magnitude difference.  Two observed curves per track and profile: the
    FP64 curve itself plus N(0, 0.05 mag) noise (chi2 about the epoch count, the most
    demanding case), and the FP64 curve of the other shape at the same radius plus the same
    noise (chi2 a few times larger).  Tracks with a non-finite magnitude are left out and
    counted."""
    import torch
    dev = ref.device
    P, E = ref.shape
    ntr = int(off.numel()) - 1
    cnt = (off[1:] - off[:-1]).to(dev)
    tid = torch.repeat_interleave(torch.arange(ntr, device=dev), cnt)
    g = torch.Generator(device=dev).manual_seed(CHI2_NOISE_SEED)
    noise = torch.randn(E, generator=g, device=dev, dtype=torch.float64) * CHI2_SIGMA
    inv_s2 = 1.0 / CHI2_SIGMA ** 2

    def chi2(m, obs):
        r = obs - m.double()
        mu = torch.zeros(ntr, dtype=torch.float64, device=dev).index_add_(0, tid, r) / cnt.double()
        r = r - mu[tid]
        return torch.zeros(ntr, dtype=torch.float64, device=dev).index_add_(0, tid, r * r) * inv_s2

    res = {k: {"max_rel_chi2": 0.0, "max_abs_chi2": 0.0, "max_abs_mag": 0.0, "per_profile_max_rel_chi2": []}
           for k in forms}
    bad_tracks = 0
    for q in range(P):
        bad = torch.zeros(ntr, dtype=torch.float64, device=dev).index_add_(0, tid, (~torch.isfinite(ref[q])).double())
        for name, out in forms.items():
            bad = bad + torch.zeros(ntr, dtype=torch.float64, device=dev).index_add_(
                0, tid, (~torch.isfinite(out[q])).double())
        ok = bad == 0
        bad_tracks += int((~ok).sum())
        cases = [ref[q] + noise, ref[(q + P // 2) % P] + noise]
        c_ref = [chi2(ref[q], o) for o in cases]
        for name, out in forms.items():
            r = res[name]
            qmax = 0.0
            for o, cr in zip(cases, c_ref):
                c = chi2(out[q], o)
                d = (c - cr).abs()[ok]
                qmax = max(qmax, float((d / cr[ok]).max()))
                r["max_abs_chi2"] = max(r["max_abs_chi2"], float(d.max()))
            r["max_rel_chi2"] = max(r["max_rel_chi2"], qmax)
            r["per_profile_max_rel_chi2"].append(qmax)
            fin = torch.isfinite(out[q]) & torch.isfinite(ref[q])
            r["max_abs_mag"] = max(r["max_abs_mag"], float((out[q].double() - ref[q])[fin].abs().max()))
    for r in res.values():
        r.update({"tolerance_rel": 1e-5, "tracks": ntr, "profiles": P, "tracks_left_out": bad_tracks,
                  "observed": "per track: its FP64 light curve (and the other shape's at the same radius) "
                              f"+ N(0, {CHI2_SIGMA} mag) noise, seed {CHI2_NOISE_SEED}; chi2 over the track's epochs"})
    return res


# ----------------------------------------------------------------------------- CPU leg (oracle port)

def oracle_profiles(n):
    """The workload's 16 profile rasters from the oracle's own rasteriser (no library call)."""
    import oracle
    pix = WIDTH / n
    return [oracle.profile(s, r * pix, pix, ref_compat=False) for s in SHAPES for r in RHALF_PX]


def cpu_steps(mp64, host_tracks, profs, steps, warmup, workers=None, first=0):
    """Steps of the FP64 oracle port on the host cores.  One step = the full map convolved
    with one profile (scipy FFT on all cores; profile first + s mod 16) and the bilinear
    magnitudes of every track on it (the oracle's C sampler, threads over track chunks):
    the light curves of all tracks for that profile, 1/16 of the workload's step, timed
    whole.  Returns the seconds of each timed step and the last convolved map."""
    import concurrent.futures as cf

    import numpy as np

    import oracle
    oracle.build()
    workers = workers or os.cpu_count() or 1
    off = host_tracks["off"].numpy()
    x0 = host_tracks["x0"].numpy(); y0 = host_tracks["y0"].numpy()
    phi = host_tracks["phi"].numpy(); v = host_tracks["v"].numpy()
    t = host_tracks["t"].numpy()
    ntr = len(off) - 1
    bounds = np.linspace(0, ntr, 4 * workers + 1).astype(np.int64)
    out = np.empty(int(off[-1]))

    def run(i):
        a, b = int(bounds[i]), int(bounds[i + 1])
        if b > a:
            out[off[a]:off[b]] = oracle.sample_tracks(cm, x0[a:b], y0[a:b], phi[a:b], v[a:b], off[a:b + 1] - off[a],
                                                      t[off[a]:off[b]])

    times = []
    cm = None
    with cf.ThreadPoolExecutor(workers) as ex:
        for s in range(warmup + steps):
            prof = profs[(first + s) % len(profs)]
            t0 = time.perf_counter()
            cm = oracle.conv_fft_workers(mp64, prof, workers=workers)
            list(ex.map(run, range(len(bounds) - 1)))
            dt = time.perf_counter() - t0
            if s >= warmup:
                times.append(dt)
    return times, cm


def cpu_sample_text(n, ntr, workers):
    return (f"FP64 oracle port, each step: scipy.fft convolution of the full {n}^2 map with one of the 16 "
            f"profiles + bilinear magnitudes of all {ntr} tracks on it ({ntr} light curves), timed whole on "
            f"{workers} threads")


def cpu_baseline(mp64, host_tracks, n, steps=3, workers=None, parity=None):
    """The oracle port timed on the host cores (cpu_steps, every step measured), and with
    parity (the GPU's batched FP64 light curves of the thin-disc 16 px profile for the
    first tracks, and those tracks) the full-size FP64 check of the GPU against the oracle."""
    import numpy as np

    import oracle
    workers = workers or os.cpu_count() or 1
    profs = oracle_profiles(n)
    kpar = len(RHALF_PX) + 3  # thin disc, 16 px
    times, cm = cpu_steps(mp64, host_tracks, profs, steps, 1, workers, first=kpar)
    ntr = len(host_tracks["off"]) - 1
    step_s = statistics.mean(times)
    check = None
    if parity is not None:
        if steps % len(profs) != 0:  # the last step's map is not profile kpar: convolve it
            cm = oracle.conv_fft_workers(mp64, profs[kpar], workers=workers)
        pt = parity["tracks"]
        ref = oracle.sample_tracks(cm, pt["x0"], pt["y0"], pt["phi"], pt["v"], pt["off"], pt["t"])
        got = parity["lc"]
        fin = np.isfinite(ref) & np.isfinite(got)
        dm = np.abs(got[fin] - ref[fin])
        check = {"samples": int(ref.size), "tracks": int(len(pt["x0"])), "finite_agree": bool(np.array_equal(
                     np.isfinite(ref), np.isfinite(got))), "max_abs_mag": float(dm.max()),
                 "max_rel_flux": float(np.max(np.abs(10 ** (-0.4 * (got[fin] - ref[fin])) - 1.0))),
                 "tolerance_rel": 1e-9,
                 "what": f"batched FP64 step on the GPU vs the FP64 oracle, full {n}^2 map, thin disc 16 px"}
    return {"value": ntr / step_s, "unit": UNIT, "cores": workers, "kind": "port", "fp64_parity_full_scale": check,
            "ms_per_step": step_s * 1000.0, "steps_timed": len(times),
            "sample": cpu_sample_text(n, ntr, workers)}


# ----------------------------------------------------------------------------- reference arm

def run_reference(args):
    """The reference arm: the path on the host cores with the oracle port (the reference
    convolves only with cuFFT, so it has no CPU implementation of its own to time), every
    step measured.  The map is the same seeded ray-shot map, shot on the host cores by the
    oracle's generator (operation for operation the library's, so the counts are equal);
    the profiles come from the oracle's rasteriser.  This process loads no library of the
    repository's product."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import torch

    import oracle
    oracle.build()
    n, nt = sizes_for(args)
    workers = os.cpu_count() or 1
    t0 = time.perf_counter()
    _, mp = oracle.rayshoot(n, WIDTH, KAPPA, GAMMA, MAP_SEED, RAYS_PER_PIXEL, threads=workers)
    t_map = time.perf_counter() - t0
    host, _, E = make_tracks_torch(nt, n, TRACK_SEED, "cpu", torch.float64)
    profs = oracle_profiles(n)
    times, _ = cpu_steps(mp, host, profs, args.steps, args.warmup, workers)
    ms = statistics.mean(times) * 1000.0
    value = nt / (ms / 1000.0)
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic: seeded inverse-ray-shot map (shot on the host cores), seeded tracks",
           "config": workload_config(args),
           "cpu_baseline": {"kind": "port", "cores": workers, "sample": cpu_sample_text(n, nt, workers),
                            "value": value, "unit": UNIT},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "map_generation_s": t_map, "light_curves_per_step": nt, "epochs_per_step": E,
           "step_ms": [x * 1000.0 for x in times]}
    print(json.dumps(out), flush=True)


# ----------------------------------------------------------------------------- main arm

def kernel_case(args):
    """One workload alone, on small sizes, for ncu captures of its kernels (-k, -c): the
    step (--side, --tracks, --nprof, --fft), the ratio pair path, the MPD histogram, the
    flux-ratio likelihood, the track fit, the radix sort of 2^24 keys, or the pair sides of
    two images of an expanding source; or one of the bench's side workloads alone (c1, c5).
    Prints one JSON line of times (not a bench line)."""
    import numpy as np
    import torch

    import microsn_gb300 as mlc
    from microsn_gb300 import build as B
    from microsn_gb300 import synth
    B.build()
    dev = "cuda:0"
    ctx = mlc.Context(0)
    if args.no_autotune:
        ctx.set_autotune(False)
    for kv in args.tune:
        key, _, val = kv.rpartition("=")
        ctx.tune_set(key, int(val))
    if args.no_profile_cache:
        ctx.set_profile_cache(0)
    args.no_cpu = True
    case = args.kernel_case
    res = {"kernel_case": case}
    n = args.n or 2000
    if case in ("step", "pair_bin_fused", "mpd", "pair"):
        mp_t, _ = synth.rayshoot_gpu(ctx, n, WIDTH, KAPPA, GAMMA, seed=MAP_SEED, rays_per_pixel=RAYS_PER_PIXEL,
                                     dtype=torch.float32)
        m = mlc.Map(ctx, mp_t, "f32")
        m.set_fft(args.fft or HEADLINE_FFT)
    if case == "step":
        ntr = args.tracks or 100_000
        _, tr, E = make_tracks_torch(ntr, n, TRACK_SEED, dev, torch.float32)
        profs = profiles_for(n)[: args.nprof or 16]
        out = torch.empty((len(profs), E), dtype=torch.float32, device=dev)
        dpix = m.tensor()
        for _ in range(max(args.warmup, 1)):
            mlc.convolve_sample_tracks(ctx, m, profs, tr, mag=True, pixels=dpix, out=out)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            mlc.convolve_sample_tracks(ctx, m, profs, tr, mag=True, pixels=dpix, out=out)
        e1.record(); torch.cuda.synchronize()
        res.update(side=n, tracks=ntr, epochs=E, nprof=len(profs), fft=args.fft or HEADLINE_FFT,
                   ms_per_step=e0.elapsed_time(e1) / args.steps)
    elif case == "pair_bin_fused":  # the reference's size: 9216 locations (--small: 1024)
        res.update(ratio_pair_workload(args, ctx, m, dev, 0))
    elif case == "mpd":
        res.update(mpd_workload(args, ctx, m, 0))
    elif case == "flux_ratio":
        res.update(flux_ratio_workload(args, ctx, dev, 0))
    elif case == "track_fit":
        res.update(c4_workload(args, ctx, dev, 0))
    elif case == "pair":  # the pair-chi2/s workload (10^5 x 10^5 curves; --tracks N: N x N)
        res.update(pair_workload(args, ctx, m, profiles_for(n), n, dev, 1, 0, torch.cuda.current_stream()))
    elif case == "c1":
        args.no_cpu = False
        res.update(c1_workload(args, ctx, dev, 0))
    elif case == "c5":
        res.update(c5_workload(args, ctx, dev, 0))
    elif case == "sort":
        nk = 1 << 24
        g = torch.Generator(device="cpu").manual_seed(7)
        keys0 = torch.rand(nk, generator=g, dtype=torch.float64).to(dev)
        vals0 = torch.arange(nk, dtype=torch.int32, device=dev)
        keys, vals = keys0.clone(), vals0.clone()
        mlc.sort_f64_u32(ctx, keys, vals)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ms = 0.0
        for _ in range(args.steps):
            keys.copy_(keys0); vals.copy_(vals0)
            e0.record()
            mlc.sort_f64_u32(ctx, keys, vals)
            e1.record(); torch.cuda.synchronize()
            ms += e0.elapsed_time(e1)
        res.update(keys=nk, ms_per_sort=ms / args.steps, sorted=bool(torch.all(keys[1:] >= keys[:-1]).item()))
    elif case == "pair_sides":
        N, nep, nb = n, 40, 3
        mp_t, _ = synth.rayshoot_gpu(ctx, N, 20.0, 0.45, 0.4, seed=6, rays_per_pixel=4.0, dtype=torch.float32)
        m = mlc.Map(ctx, mp_t, "f32")
        R = np.linspace(1.0, 100.0 * N / C5_N, nep)
        profs = [mlc.profile("limb_darkened", r / np.sqrt(2.0), 1.0, ref_compat=False, u=u) for r in R for u in C5_U]
        conv = mlc.convolve_many(ctx, m, profs)
        ntr = args.tracks or 20_000
        rng = np.random.default_rng(60)
        t = torch.as_tensor(np.arange(nep) * 2.0, dtype=torch.float32, device=dev)
        mg = 0.3 * N
        trk = [[torch.as_tensor(a, dtype=torch.float32, device=dev) for a in
                (rng.uniform(mg, N - mg, ntr), rng.uniform(mg, N - mg, ntr), rng.uniform(0, 2 * np.pi, ntr),
                 rng.uniform(0.2, 1.0, ntr))] for _ in range(2)]
        w = 1.0 / rng.uniform(0.02, 0.1, nep * nb) ** 2
        for _ in range(max(args.warmup, 1)):
            sA = mlc.PairSide.expanding(ctx, conv, nep, nb, *trk[0], t, w, None, True)
            sB = mlc.PairSide.expanding(ctx, conv, nep, nb, *trk[1], t, w, None, True)
            r = mlc.pair_chi2_sides(ctx, sA, sB, nbins=PAIR_BINS, lo=-1.0, hi=9.0, k=PAIR_K)
            sA.close(); sB.close()
        torch.cuda.synchronize()
        res.update(side=N, tracks=ntr, T=nep * nb, refined=r["stats"]["refined"])
    res["autotune"] = {k: {"choice": c, "ms": t} for k, (c, t) in ctx.autotune_report().items()}
    print(json.dumps(res, default=float), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.kernel_case:
        return kernel_case(args)
    import numpy as np
    import torch

    import microsn_gb300 as mlc
    from microsn_gb300 import build as B
    from microsn_gb300 import synth

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    B.build()
    dev = f"cuda:{local}"
    torch.cuda.set_device(local)
    n, ntracks = sizes_for(args)
    ctx = mlc.Context(local)
    if args.no_autotune:
        ctx.set_autotune(False)
    stream = torch.cuda.current_stream(local)

    # ---- inputs resident in HBM
    mp_t, meta = synth.rayshoot_gpu(ctx, n, WIDTH, KAPPA, GAMMA, seed=MAP_SEED + rank, rays_per_pixel=RAYS_PER_PIXEL,
                                    dtype=torch.float32)
    m = mlc.Map(ctx, mp_t, "f32")
    m.set_fft(HEADLINE_FFT)
    host_tr, tr, E = make_tracks_torch(ntracks, n, TRACK_SEED + rank, dev, torch.float32)
    profs = profiles_for(n)
    out = torch.empty((len(profs), E), dtype=torch.float32, device=dev)
    dpix = m.tensor()

    def step():
        # one library call: forward spectrum of the map's pixels, 16 fused convolutions,
        # interleave, bilinear magnitudes of every track
        mlc.convolve_sample_tracks(ctx, m, profs, tr, mag=True, pixels=dpix, out=out)

    for _ in range(max(args.warmup, 1)):
        step()
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    # ---- timed region (device-resident inputs)
    clocks = ClockSampler(local)
    barrier()
    clocks.start()
    time.sleep(0.3)
    l0 = ctx.launch_count()
    e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
    barrier()
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    barrier()
    clk = clocks.stop()
    launches = ctx.launch_count() - l0
    ms_total = max_over_ranks(e0.elapsed_time(e1), dev)
    ms_step = ms_total / args.steps
    lc_per_step = len(profs) * ntracks
    value = world * lc_per_step / (ms_step / 1000.0)

    # ---- per-kernel CUDA-event times over the same steps (separate pass: events add a little overhead)
    ctx.set_timing(True)
    ksteps = min(args.steps, 3)
    for _ in range(ksteps):
        step()
    kt = ctx.kernel_times(reset=True)
    ctx.set_timing(False)
    per_step = {k: v[0] / ksteps for k, v in kt.items()}
    total_k = sum(per_step.values())
    dom = max(per_step, key=per_step.get)
    dom_launch_ms = kt[dom][0] / kt[dom][1]
    spec_es = 8 if HEADLINE_FFT == "f32x2" else 4
    alg = algorithmic_bytes(dom, n, E, len(profs), es=spec_es)
    hbm, peak_kind = peaks()
    traffic = load_traffic().get(dom)
    roof = None
    if alg is not None:
        ach = alg / (dom_launch_ms / 1000.0) / 1e9
        roof = {"kernel": dom, "bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
                "traffic": traffic, "algorithmic_bytes": alg, "launch_ms": dom_launch_ms,
                "peak_source": f"{peak_kind} copy bandwidth (MEASURED_PEAKS.json hbm_gbs)",
                "share_of_step": per_step[dom] / total_k if total_k else None}
        if HEADLINE_FFT == "f32x2" and dom in ("fft_rows_c2r_interleave", "conv_fused_spectrum", "fft_col_A"):
            roof["note"] = ("float-float transform pass: its DRAM traffic equals the algorithmic bytes, and it is "
                            "bound by the FP32 pipe that carries the float-float arithmetic (65-74 % FMA, ncu: "
                            "profiles/step_ff_10000.md), not by HBM")
    kernels = {k: {"ms_per_step": v, "launches_per_step": kt[k][1] / ksteps,
                   "GB_per_s": (algorithmic_bytes(k, n, E, len(profs), es=spec_es) / (kt[k][0] / kt[k][1] / 1000.0) / 1e9)
                   if algorithmic_bytes(k, n, E, len(profs), es=spec_es) else None} for k, v in per_step.items()}

    # ---- the same step with the profile spectra recomputed in every call (cache off)
    ctx.set_profile_cache(0)
    step()
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    ctx.set_profile_cache(-1)
    step()  # the cache refilled before the timings below
    torch.cuda.synchronize()
    profile_cache = {"ms_per_step": ms_step, "ms_per_step_recomputed": e0.elapsed_time(e1) / args.steps,
                     "what": "the timed step keeps the 16 profiles' spectra between calls (the profile list and map "
                             "size repeat; the map's own spectrum is recomputed every step); recomputed: the same "
                             "step transforming every profile in every call"}

    # ---- the same step as one CUDA graph (captured on its first graph call, then replayed)
    def graph_step():
        mlc.convolve_sample_tracks(ctx, m, profs, tr, mag=True, pixels=dpix, out=out, graph=True)

    graph_step(); graph_step()
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        graph_step()
    e1.record(stream)
    torch.cuda.synchronize()
    cuda_graph = {"ms_per_step": e0.elapsed_time(e1) / args.steps, "eager_ms_per_step": ms_step,
                  "what": "the timed step replayed as one CUDA graph (graph=True): same kernels, one launch"}

    # ---- e2e through the library with host buffers: page-locked on 2 MB pages (mlc_host_alloc),
    # whose copies keep their rate when the host memory is fragmented
    h_map = mlc.host_empty((n, n), torch.float32)
    h_map.copy_(mp_t.cpu())
    h_tr = {k: mlc.host_empty(tuple(tr[k].shape), tr[k].dtype) for k in tr}
    for k in tr:
        h_tr[k].copy_(tr[k].cpu())
    h_out = mlc.host_empty((len(profs), E), torch.float32)
    bi = h_map.numel() * 4 + sum(h_tr[k].numel() * h_tr[k].element_size() for k in h_tr)
    bo = h_out.numel() * 4

    def e2e_step():
        # the same call with host buffers: map pixels and tracks up, light curves down, the
        # copies on the library's own streams; asynchronous, so that one step's download
        # overlaps the next step's convolutions
        mlc.convolve_sample_tracks(ctx, m, profs, h_tr, mag=True, pixels=h_map, out=h_out, async_=True)

    e2e_step()
    ctx.synchronize()
    esteps = args.steps
    # five timed loops of K calls (the host link is shared with other jobs on the machine, so
    # the overlap of uploads, kernels and downloads varies from loop to loop); the median is
    # reported, all five are listed
    reps = []
    for _ in range(5):
        barrier()
        e0.record(stream)
        for _ in range(esteps):
            e2e_step()
        ctx.join()  # the stream waits for the last downloads before e1
        e1.record(stream)
        ctx.synchronize()
        barrier()
        reps.append(e0.elapsed_time(e1) / esteps)
    e2e_ms = max_over_ranks(sorted(reps)[2], dev)  # the slowest rank's time
    e2e_val = world * lc_per_step / (e2e_ms / 1000.0)
    # the host link itself: plain 1 GiB copies between pinned host memory and HBM on this machine
    # (the light curves' download bounds the e2e step); the host memory is shared with other
    # jobs, so three samples of three copies each, the best one reported
    link = {}
    nl = min(1 << 28, h_out.numel())  # up to 1 GiB
    dbuf = torch.empty(nl, dtype=torch.float32, device=dev)
    hbuf = h_out.view(-1)[:nl]
    for name, dst, src in (("d2h_gbs", hbuf, dbuf), ("h2d_gbs", dbuf, hbuf)):
        dst.copy_(src, non_blocking=True)
        samples = []
        for _ in range(3):
            e0.record(stream)
            for _ in range(3):
                dst.copy_(src, non_blocking=True)
            e1.record(stream)
            torch.cuda.synchronize()
            samples.append(3 * 4 * nl / (e0.elapsed_time(e1) / 1000.0) / 1e9)
        link[name] = max(samples)
        link[name + "_samples"] = samples
    link["download_floor_ms"] = bo / (link["d2h_gbs"] * 1e9) * 1000.0
    del h_out, dbuf

    # ---- the plain one-launch-per-stage FP64 form of the same step
    plain = None
    parity_in = None
    accuracy = None
    if not args.no_plain:
        m64 = mlc.Map(ctx, mp_t.double(), "f64")
        convs64 = [torch.empty((n, n), dtype=torch.float64, device=dev) for _ in range(2)]
        tr64 = {k: (a.to(dev, torch.float64) if a.dtype == torch.float64 else a.to(dev)) for k, a in host_tr.items()}
        out64 = torch.empty((1, E), dtype=torch.float64, device=dev)

        def step64():
            m64.refresh()
            for k, p in enumerate(profs):
                c = convs64[k % 2]
                mlc.convolve(ctx, m64, p, "plain", out=c)
                mlc.sample_tracks(ctx, [c], n, n, tr64["x0"], tr64["y0"], tr64["phi"], tr64["v"], tr64["off"],
                                  tr64["t"], mag=True, out=out64)

        step64()
        torch.cuda.synchronize()
        e0.record(stream)
        step64()
        e1.record(stream)
        torch.cuda.synchronize()
        pms = e0.elapsed_time(e1)
        plain = {"value": world * lc_per_step / (pms / 1000.0), "unit": UNIT, "ms_per_step": pms, "dtype": "f64",
                 "form": "full-size wrapped kernel + forward FFT + multiply + inverse FFT + sampling, per profile",
                 "batched_over_plain": value / (world * lc_per_step / (pms / 1000.0))}
        del convs64, out64
        # the batched one-call step in FP64 on the FP32 step's own inputs (the FP32 track
        # parameters upcast, the same map pixels): FP32 and FP64 side by side, and the FP32
        # light curves' error against it over every sample
        out64b = torch.empty((len(profs), E), dtype=torch.float64, device=dev)
        pix64 = m64.tensor()
        tr64f = {k: (a.double() if a.is_floating_point() else a) for k, a in tr.items()}

        def step64b():
            mlc.convolve_sample_tracks(ctx, m64, profs, tr64f, mag=True, pixels=pix64, out=out64b)

        step64b()
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(3):
            step64b()
        e1.record(stream)
        torch.cuda.synchronize()
        bms = e0.elapsed_time(e1) / 3
        # the same FP64 step with float-float transforms
        m64.set_fft("f32x2")
        out64f = torch.empty_like(out64b)

        def step64f():
            mlc.convolve_sample_tracks(ctx, m64, profs, tr64f, mag=True, pixels=pix64, out=out64f)

        step64f()
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(3):
            step64f()
        e1.record(stream)
        torch.cuda.synchronize()
        fms = e0.elapsed_time(e1) / 3
        fdev = 0.0
        for q in range(len(profs)):
            ok = torch.isfinite(out64b[q]) & torch.isfinite(out64f[q])
            fdev = max(fdev, float((out64f[q] - out64b[q]).abs()[ok].max()))
        m64.set_fft("native")
        del out64f
        # the same step with FP32 transforms (the fast form), its time and light curves
        m_fast = mlc.Map(ctx, mp_t, "f32")
        pix_fast = m_fast.tensor()
        out_fast = torch.empty_like(out)

        def step_fast():
            mlc.convolve_sample_tracks(ctx, m_fast, profs, tr, mag=True, pixels=pix_fast, out=out_fast)

        step_fast()
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(3):
            step_fast()
        e1.record(stream)
        torch.cuda.synchronize()
        qms = e0.elapsed_time(e1) / 3
        step()  # the headline light curves of the same inputs
        torch.cuda.synchronize()
        acc = chi2_errors({"headline": out, "fp32_transforms": out_fast}, out64b, tr["off"])
        del out_fast, pix_fast, m_fast
        plain["batched_fp64"] = {"value": world * lc_per_step / (bms / 1000.0), "unit": UNIT, "ms_per_step": bms,
                                 "batched_fp64_over_plain_fp64": pms / bms}
        plain["batched_fp64_f32x2"] = {"value": world * lc_per_step / (fms / 1000.0), "unit": UNIT,
                                       "ms_per_step": fms, "over_plain_fp64": pms / fms,
                                       "max_abs_mag_vs_native_fp64": fdev,
                                       "what": "the batched FP64 step with float-float transforms"}
        plain["fp32_transforms"] = {"value": world * lc_per_step / (qms / 1000.0), "unit": UNIT, "ms_per_step": qms,
                                    "over_plain_fp64": pms / qms, "vs_fp64": acc["fp32_transforms"],
                                    "what": "the same step with FP32 transforms (fast form; fails the 1e-5 chi2 bar)"}
        accuracy = acc["headline"]
        # kept for the full-scale FP64 check against the oracle in the CPU leg: the thin-disc
        # 16 px light curves of the first tracks and those tracks' parameters
        kpar = len(RHALF_PX) + 3
        npar = min(20000, int(tr["off"].numel()) - 1)
        epar = int(tr["off"][npar].item())
        parity_in = {"lc": out64b[kpar, :epar].cpu().numpy(),
                     "tracks": {k: tr64f[k][: (npar + 1 if k == "off" else (epar if k == "t" else npar))].cpu().numpy()
                                for k in tr64f}}
        del m64, tr64, out64b, pix64, tr64f

    # ---- pair-chi2/s workload on the same device
    pair = None
    if not args.no_pair:
        pair = pair_workload(args, ctx, m, profs, n, dev, world, rank, stream)
    flux = c1 = c4 = c5 = ratio = mpd = None
    if not args.no_pair:
        ratio = ratio_pair_workload(args, ctx, m, dev, rank)
        mpd = mpd_workload(args, ctx, m, rank)
        flux = flux_ratio_workload(args, ctx, dev, rank)
        c1 = c1_workload(args, ctx, dev, rank)
        c4 = c4_workload(args, ctx, dev, rank)
    if not args.no_c5:
        c5 = c5_workload(args, ctx, dev, rank)

    # ---- CPU baseline (rank 0, N = 1 only)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_baseline(mp_t.double().cpu().numpy(), host_tr, n, parity=parity_in)

    if rank == 0:
        res = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
               "vs_baseline": None, "dtype": "f32",
               "data": "synthetic: seeded inverse-ray-shot map, seeded tracks (no public dataset)",
               "config": workload_config(args), "roofline": roof, "cpu_baseline": cpu,
               "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": int(bi), "d2h_bytes_per_step": int(bo),
                       "ms_per_step": e2e_ms, "repeats_ms_per_step": reps, "link": link,
                       "host_buffers": "page-locked, 2 MB pages (mlc_host_alloc)"},
               "gpu_launches": int(launches), "clocks": clk,
               "form": ("FP32 map pixels, float-float transforms, FP32 convolved maps and light curves, float-float "
                        "track positions" if HEADLINE_FFT == "f32x2" else "FP32 transforms"),
               "max_rel_err_vs_fp64": accuracy["max_rel_chi2"] if accuracy else None,
               "accuracy_vs_fp64": accuracy,
               "plain_fp64": plain, "kernels": kernels, "cuda_graph": cuda_graph, "profile_cache": profile_cache,
               "sampling_stage": ({"value": world * lc_per_step / (kernels["sample_tracks_il"]["ms_per_step"] / 1000.0),
                                   "unit": UNIT, "ms_per_step": kernels["sample_tracks_il"]["ms_per_step"]}
                                  if "sample_tracks_il" in kernels else None),
               "ratio_pairs": ratio,
               "map_mpd": mpd,
               "autotune": {k: {"choice": c, "ms": m} for k, (c, m) in ctx.autotune_report().items()},
               "light_curves_per_step": lc_per_step, "epochs_per_step": E, "pair_chi2": pair,
               "flux_ratio": flux, "c1_small_fp64": c1, "c4_fit": c4,
               "c5_supernova": c5}
        print(json.dumps(res), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()




if __name__ == "__main__":
    main()
