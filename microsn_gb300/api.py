"""Python host mirror of the reference's hot-path interface, over the C ABI.

Names follow the reference (simulating_lcurves/include/gpu_functions.hpp:11-18,
cpu_functions.hpp:12-15): ``expanding_source``, ``setup_integral``, ``calculate_chi2``,
``bin_chi2``, ``setup_chi2_calculation``, plus the new track / offset-chi2 stages.
Device buffers are torch CUDA tensors (plumbing only); all compute runs in
libmicrolc_gb300.so.  Errors raise :class:`MlcError` with the library's message.
"""
from __future__ import annotations

import ctypes as C
import weakref
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from ._lib import MLC_CONV_FUSED, MLC_CONV_PLAIN, MLC_F32, MLC_F64, MlcError, MlcProfile, SHAPES

_MODES = {"fused": MLC_CONV_FUSED, "plain": MLC_CONV_PLAIN}
_PREC = {"f64": MLC_F64, "f32": MLC_F32, torch.float64: MLC_F64, torch.float32: MLC_F32}


def _ptr(t) -> C.c_void_p:
    if t is None:
        return None
    if isinstance(t, torch.Tensor):
        return C.c_void_p(t.data_ptr())
    if isinstance(t, np.ndarray):
        return t.ctypes.data_as(C.c_void_p)
    raise TypeError(type(t))


def _np(a, dtype):
    return np.ascontiguousarray(np.asarray(a), dtype=dtype)


class Context:
    """A library context bound to one CUDA device and stream (torch's current stream by default)."""

    def __init__(self, device: int = 0, stream: torch.cuda.Stream | None = None):
        self.L = _lib.load()
        self.device = device
        s = stream if stream is not None else torch.cuda.current_stream(device)
        self.stream = s
        h = C.c_void_p()
        st = self.L.mlc_ctx_create(device, C.c_void_p(s.cuda_stream), C.byref(h))
        if st != 0:
            raise MlcError(st, "mlc_ctx_create failed (is this an sm_103 GPU?)")
        self.h = h
        self._maps = weakref.WeakSet()

    def check(self, st: int):
        if st != 0:
            raise MlcError(st, self.L.mlc_ctx_last_error(self.h).decode())

    def set_stream(self, stream: torch.cuda.Stream):
        self.stream = stream
        self.check(self.L.mlc_ctx_set_stream(self.h, C.c_void_p(stream.cuda_stream)))

    def synchronize(self):
        self.check(self.L.mlc_ctx_synchronize(self.h))

    def join(self):
        """Make the context's stream wait (on the device) for the copies of host-buffer calls."""
        self.check(self.L.mlc_ctx_join(self.h))

    def set_chunk_bytes(self, nbytes: int):
        """Output chunk size of host-buffer convolve_sample_tracks calls."""
        self.check(self.L.mlc_ctx_set_chunk_bytes(self.h, int(nbytes)))

    def workspace_bytes(self) -> int:
        return int(self.L.mlc_ctx_workspace_bytes(self.h))

    def launch_count(self) -> int:
        return int(self.L.mlc_ctx_launch_count(self.h))

    def set_timing(self, on: bool):
        self.check(self.L.mlc_ctx_set_timing(self.h, int(on)))

    def set_autotune(self, on: bool):
        """Launch autotuner on (default) or off (FFT form everywhere)."""
        self.check(self.L.mlc_ctx_set_autotune(self.h, int(on)))

    def set_profile_cache(self, max_bytes: int = -1):
        """Device bytes the cached profile spectra may take (-1: a quarter of the device, 0: off)."""
        self.check(self.L.mlc_ctx_set_profile_cache(self.h, int(max_bytes)))

    def tune_set(self, key: str, choice: int):
        """Pin the autotuner's choice for one key (see mlc_ctx_tune_set)."""
        self.check(self.L.mlc_ctx_tune_set(self.h, key.encode(), int(choice)))

    def autotune_report(self) -> dict:
        """{key: (choice, {candidate: ms})} of every tuned key."""
        buf = C.create_string_buffer(1 << 16)
        n = self.L.mlc_ctx_autotune_report(self.h, buf, len(buf))
        if n < 0:
            self.check(-n)
        out = {}
        for line in buf.value.decode().splitlines():
            key, rest = line.split(": ", 1)
            choice, _, cands = rest.partition(" (")
            out[key] = (choice, {c.split("=")[0]: float(c.split("=")[1]) for c in cands.rstrip(")").split()})
        return out

    def kernel_times(self, reset: bool = True) -> dict:
        """{kernel name: (total ms, launches)} from the per-launch CUDA events."""
        names = C.create_string_buffer(1 << 16)
        ms = np.zeros(256); n_l = np.zeros(256, np.int64)
        n = self.L.mlc_ctx_kernel_times(self.h, names, len(names), _ptr(ms), _ptr(n_l), 256, int(reset))
        if n < 0:
            self.check(-n)
        keys = names.value.decode().split("\n")[:n]
        return {k: (float(ms[i]), int(n_l[i])) for i, k in enumerate(keys)}

    def close(self):
        if getattr(self, "h", None):
            for m in list(getattr(self, "_maps", ())):
                m.close()
            self.L.mlc_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def profile(shape: str, rhalf: float, pix: float, incl=0.0, orient=0.0, Rin=0.0, a=1.0, u=0.0,
            ref_compat=True) -> MlcProfile:
    return MlcProfile(SHAPES[shape], int(ref_compat), rhalf, pix, incl, orient, Rin, a, u)


def profile_raster(p: MlcProfile) -> np.ndarray:
    L = _lib.load()
    n = C.c_int()
    st = L.mlc_profile_dims(C.byref(p), C.byref(n))
    if st:
        raise MlcError(st, "invalid profile")
    out = np.zeros(n.value * n.value)
    st = L.mlc_profile_raster(C.byref(p), out.ctypes.data_as(C.c_void_p), out.size, C.byref(n))
    if st:
        raise MlcError(st, "profile raster failed")
    return out.reshape(n.value, n.value)


class _CudaArray:
    """Minimal __cuda_array_interface__ holder to view library-owned device memory in torch."""

    def __init__(self, ptr, shape, typestr):
        self.__cuda_array_interface__ = {"data": (ptr, False), "shape": shape, "typestr": typestr, "version": 2}


def _wrap_device_ptr(ptr, shape, dtype, device):
    typestr = "<f8" if dtype == torch.float64 else "<f4"
    with torch.cuda.device(device):
        return torch.as_tensor(_CudaArray(ptr, shape, typestr), device=f"cuda:{device}")


class Map:
    """A magnification map resident on the device (MagnificationMap::data)."""

    def __init__(self, ctx: Context, data, precision: str = "f64"):
        self.ctx = ctx
        if isinstance(data, torch.Tensor):
            src = data.contiguous()
            on_dev = int(src.is_cuda)
            dt = MLC_F64 if src.dtype == torch.float64 else MLC_F32
            ptr = C.c_void_p(src.data_ptr())
            keep = src
        else:
            keep = np.ascontiguousarray(data)
            if keep.dtype not in (np.float64, np.float32):
                keep = keep.astype(np.float64)
            on_dev = 0
            dt = MLC_F64 if keep.dtype == np.float64 else MLC_F32
            ptr = keep.ctypes.data_as(C.c_void_p)
        self.Ny, self.Nx = keep.shape
        self.prec = _PREC[precision]
        h = C.c_void_p()
        ctx.check(ctx.L.mlc_map_create(ctx.h, ptr, on_dev, dt, self.Nx, self.Ny, self.prec, C.byref(h)))
        self.h = h
        ctx._maps.add(self)
        ctx.synchronize()

    @property
    def dtype(self):
        return torch.float64 if self.prec == MLC_F64 else torch.float32

    def data_ptr(self) -> int:
        p = C.c_void_p()
        self.ctx.check(self.ctx.L.mlc_map_data(self.h, C.byref(p)))
        return p.value

    def prepare(self):
        self.ctx.check(self.ctx.L.mlc_map_prepare(self.ctx.h, self.h))

    def set_fft(self, mode: str):
        """Transforms in the map's own precision ("native") or in float-float arithmetic ("f32x2");
        pixels and outputs keep the map's precision either way."""
        self.ctx.check(self.ctx.L.mlc_map_set_fft(self.h, {"native": 0, "f32x2": 1}[mode]))

    def refresh(self):
        """Recompute the spectrum from the current pixels."""
        self.ctx.check(self.ctx.L.mlc_map_refresh(self.ctx.h, self.h))

    def tensor(self) -> torch.Tensor:
        """A torch view of the map's device pixels (shares memory with the library)."""
        return _wrap_device_ptr(self.data_ptr(), (self.Ny, self.Nx), self.dtype, self.ctx.device)

    def close(self):
        if getattr(self, "h", None):
            self.ctx.L.mlc_map_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def convolve(ctx: Context, m: Map, prof: MlcProfile, mode: str = "fused", out: torch.Tensor | None = None):
    if out is None:
        out = torch.empty((m.Ny, m.Nx), dtype=m.dtype, device=f"cuda:{ctx.device}")
    ctx.check(ctx.L.mlc_convolve(ctx.h, m.h, C.byref(prof), _MODES[mode], _ptr(out)))
    return out


def convolve_direct(ctx: Context, m: Map, prof: MlcProfile, variant: int = 0, out: torch.Tensor | None = None):
    """The direct tiled convolution (FP32 map, profile of 2..32 pixels), tile shape 0..3."""
    if out is None:
        out = torch.empty((m.Ny, m.Nx), dtype=m.dtype, device=f"cuda:{ctx.device}")
    ctx.check(ctx.L.mlc_convolve_direct(ctx.h, m.h, C.byref(prof), int(variant), _ptr(out)))
    return out


def expanding_source(ctx: Context, m: Map, sizes, base: MlcProfile, width: float, loc_x, loc_y,
                     mode: str = "fused"):
    """expanding_source (gpu_functions.cu:82): returns LC (Nloc x Nprof) and DLC
    (Nloc x (Nprof-1)) as FP64 device tensors."""
    dev = f"cuda:{ctx.device}"
    sizes = _np(sizes, np.float64)
    lx = torch.as_tensor(np.asarray(loc_x, np.int32), device=dev)
    ly = torch.as_tensor(np.asarray(loc_y, np.int32), device=dev)
    Nloc, Nprof = lx.numel(), sizes.size
    LC = torch.empty((Nloc, Nprof), dtype=torch.float64, device=dev)
    DLC = torch.empty((Nloc, max(Nprof - 1, 1)), dtype=torch.float64, device=dev)
    ctx.check(ctx.L.mlc_expanding_source(ctx.h, m.h, _ptr(sizes), Nprof, C.byref(base), width, Nloc, _ptr(lx),
                                         _ptr(ly), _MODES[mode], _ptr(LC), _ptr(DLC)))
    return LC, DLC[:, : Nprof - 1]


def sample_tracks(ctx: Context, maps, Nx: int, Ny: int, x0, y0, phi, v, off, t, mag: bool = True,
                  out: torch.Tensor | None = None):
    """Bilinear samples of the maps along straight tracks; returns (len(maps), E)."""
    dt = x0.dtype
    prec = _PREC[dt]
    arr = (C.c_void_p * len(maps))(*[C.c_void_p(mm.data_ptr()) for mm in maps])
    E = int(off[-1].item())
    if out is None:
        out = torch.empty((len(maps), E), dtype=dt, device=x0.device)
    ctx.check(ctx.L.mlc_sample_tracks(ctx.h, arr, len(maps), Nx, Ny, prec, x0.numel(), _ptr(x0), _ptr(y0),
                                      _ptr(phi), _ptr(v), _ptr(off), _ptr(t), int(mag), _ptr(out)))
    return out


def interleave_maps(ctx: Context, maps, Nx: int, Ny: int, stride: int = 16, out: torch.Tensor | None = None):
    """Pixel-interleaved copy of up to 16 maps: (Ny, Nx, stride)."""
    dt = maps[0].dtype
    arr = (C.c_void_p * len(maps))(*[C.c_void_p(mm.data_ptr()) for mm in maps])
    if out is None:
        out = torch.empty((Ny, Nx, stride), dtype=dt, device=maps[0].device)
    ctx.check(ctx.L.mlc_interleave_maps(ctx.h, arr, len(maps), Nx, Ny, _PREC[dt], stride, _ptr(out)))
    return out


def sample_tracks_interleaved(ctx: Context, imap: torch.Tensor, nmaps: int, x0, y0, phi, v, off, t, mag=True,
                              out: torch.Tensor | None = None):
    Ny, Nx, stride = imap.shape
    dt = x0.dtype
    E = int(off[-1].item())
    if out is None:
        out = torch.empty((nmaps, E), dtype=dt, device=x0.device)
    ctx.check(ctx.L.mlc_sample_tracks_interleaved(ctx.h, _ptr(imap), stride, nmaps, Nx, Ny, _PREC[dt], x0.numel(),
                                                  _ptr(x0), _ptr(y0), _ptr(phi), _ptr(v), _ptr(off), _ptr(t),
                                                  int(mag), _ptr(out)))
    return out


# ----------------------------------------------------------------------------- differentiable track fit

FIT_PARAMS = ("x0", "y0", "phi", "v", "R_half", "dm")


def fit_raster(rhalf: float, pix: float, N: int):
    """Smooth thin-disc raster P (N x N) and its derivative rasters dP/dx, dP/dy (per pixel
    of offset) and dP/d(rhalf), as used by the radius stack."""
    out = [np.zeros(N * N) for _ in range(4)]
    st = _lib.load().mlc_fit_raster(rhalf, pix, N, *[_ptr(a) for a in out])
    if st:
        raise MlcError(st, "fit raster: rhalf, pix > 0 and an even N are required")
    return tuple(a.reshape(N, N) for a in out)


def radius_stack(ctx: Context, m: Map, radii, N: int | None = None, pix: float = 1.0) -> torch.Tensor:
    """The map convolved with P(R_k), dP/dx, dP/dy and dP/dR for each radius: (Ny, Nx, K, 4)
    tensor in the map's precision.  N defaults to a raster of 2.2 R_max on each side."""
    r = np.ascontiguousarray(radii, np.float64)
    if N is None:
        N = int(np.ceil(4.4 * r[-1] / pix)) // 2 * 2 + 2
    out = torch.empty((m.Ny, m.Nx, len(r), 4), dtype=m.dtype, device=f"cuda:{ctx.device}")
    ctx.check(ctx.L.mlc_radius_stack(ctx.h, m.h, len(r), _ptr(r), pix, int(N), _ptr(out)))
    return out


def track_fit(ctx: Context, stack: torch.Tensor, radii, theta: torch.Tensor, off: torch.Tensor, t: torch.Tensor,
              obs: torch.Tensor, w: torch.Tensor, grad: bool = True, model: bool = False, out_chi2=None,
              out_grad=None, out_model=None):
    """chi2 (n,), d chi2 / d theta (n, 6) and optionally the model magnitudes of n tracks
    with parameters theta = (x0, y0, phi, v, R_half, dm) against observed curves (obs, w
    per epoch).  One kernel launch, no allocation inside the library (pass out_* to make
    the call capturable in a CUDA graph)."""
    Ny, Nx, K, four = stack.shape
    assert four == 4
    dt = stack.dtype
    prec = _PREC[dt]
    n = theta.shape[0]
    for name, a in (("theta", theta), ("t", t), ("obs", obs), ("w", w)):
        if a.dtype != dt or not a.is_contiguous() or not a.is_cuda:
            raise ValueError(f"{name} must be a contiguous CUDA {dt} tensor")
    if off.dtype != torch.int64 or off.numel() != n + 1:
        raise ValueError("off must be int64 with ntracks + 1 entries")
    c2 = out_chi2 if out_chi2 is not None else torch.empty(n, dtype=dt, device=theta.device)
    g = (out_grad if out_grad is not None else torch.empty((n, 6), dtype=dt, device=theta.device)) if grad else None
    mo = (out_model if out_model is not None else torch.empty(t.shape[0], dtype=dt, device=theta.device)) \
        if model else None
    r = (C.c_double * K)(*[float(x) for x in radii])
    ctx.check(ctx.L.mlc_track_fit(ctx.h, _ptr(stack), Nx, Ny, prec, K, r, n, _ptr(theta), _ptr(off), _ptr(t),
                                  _ptr(obs), _ptr(w), _ptr(c2), _ptr(g), _ptr(mo)))
    return c2, g, mo


class TrackChi2(torch.autograd.Function):
    """chi2 of every track as a differentiable function of theta (n, 6); the forward
    kernel computes the gradient at the same time and backward scales it."""

    @staticmethod
    def forward(fctx, theta, ctx, stack, radii, off, t, obs, w):
        c2, g, _ = track_fit(ctx, stack, radii, theta.detach().contiguous(), off, t, obs, w, grad=True)
        fctx.save_for_backward(g)
        return c2

    @staticmethod
    def backward(fctx, gout):
        (g,) = fctx.saved_tensors
        return gout[:, None] * g, None, None, None, None, None, None, None


def track_chi2(ctx: Context, stack, radii, theta, off, t, obs, w) -> torch.Tensor:
    return TrackChi2.apply(theta, ctx, stack, radii, off, t, obs, w)


def flux_ratio_chi2(ctx: Context, f_obs, df_obs, mu1: torch.Tensor, mu2: torch.Tensor, want_chi2=False):
    """getChi2GPU: likelihood = sum over location pairs of exp(-chi2) (FP64), and the
    N x N chi2 (chi2[y, x], FP32) when want_chi2.  f_obs, df_obs: (F, T); mu1, mu2:
    (N, F, T) FP32 CUDA tensors."""
    fo = np.ascontiguousarray(f_obs, np.float32); dfo = np.ascontiguousarray(df_obs, np.float32)
    F, T = fo.shape
    N = mu1.shape[0]
    if mu1.dtype != torch.float32 or mu2.dtype != torch.float32 or tuple(mu1.shape) != (N, F, T) \
            or tuple(mu2.shape) != (N, F, T):
        raise ValueError("mu1 and mu2 must be (N, F, T) float32 tensors")
    mu1 = mu1.contiguous(); mu2 = mu2.contiguous()
    chi2 = torch.empty((N, N), dtype=torch.float32, device=mu1.device) if want_chi2 else None
    like = C.c_double()
    ctx.check(ctx.L.mlc_flux_ratio_chi2(ctx.h, _ptr(fo), _ptr(dfo), _ptr(mu1), _ptr(mu2), N, F, T, _ptr(chi2),
                                        C.byref(like)))
    return (like.value, chi2) if want_chi2 else like.value


def map_binned_mpd(ctx: Context, m: Map, nbins: int, mn: float = 0.02, mx: float = 200.0):
    """MagnificationMap::getBinnedMpd: (bins, counts) of the map's pixels in log bins."""
    bins = np.zeros(nbins); counts = np.zeros(nbins)
    ctx.check(ctx.L.mlc_map_binned_mpd(ctx.h, m.h, nbins, mn, mx, _ptr(bins), _ptr(counts)))
    return bins, counts


def mpd_normalize(bins, counts) -> np.ndarray:
    """Mpd::normalize (mpd.cpp:64-69): counts / trapezium integral over the bins."""
    b = np.asarray(bins, np.float64); c = np.array(counts, np.float64)
    s = 0.0
    for i in range(1, len(c)):
        s += (c[i] + c[i - 1]) * (b[i] - b[i - 1]) / 2.0
    return c / s


def mpd_divide(ctx: Context, binsA, countsA, binsB, countsB, binsR) -> np.ndarray:
    """Mpd::divide_by: A.divide_by(B, R) -> R's counts."""
    c = lambda a: np.ascontiguousarray(a, np.float64)
    bA, cA, bB, cB, bR = c(binsA), c(countsA), c(binsB), c(countsB), c(binsR)
    out = np.zeros(len(bR))
    ctx.check(ctx.L.mlc_mpd_divide(ctx.h, len(bA), _ptr(bA), _ptr(cA), len(bB), _ptr(bB), _ptr(cB), len(bR),
                                   _ptr(bR), _ptr(out)))
    return out


def convolve_many(ctx: Context, m: Map, profiles, mode: str = "fused", out: torch.Tensor | None = None,
                  graph: bool = False) -> torch.Tensor:
    """The map convolved with every profile: (nprof, Ny, Nx) in the map's precision.
    graph=True captures the kernel sequence as a CUDA graph on the first call and replays
    it on later calls with the same map, raster sizes and output."""
    n = len(profiles)
    if out is None:
        out = torch.empty((n, m.Ny, m.Nx), dtype=m.dtype, device=f"cuda:{ctx.device}")
    P = (_lib.MlcProfile * n)(*profiles)
    ctx.check(ctx.L.mlc_convolve_many(ctx.h, m.h, n, P, _MODES[mode], _ptr(out), m.Ny * m.Nx,
                                      _lib.MLC_GRAPH if graph else 0))
    return out


def sample_expanding(ctx: Context, maps: torch.Tensor, nbands: int, x0, y0, phi, v, t, mag=True,
                     out: torch.Tensor | None = None) -> torch.Tensor:
    """Expanding source: maps (nep*nbands, Ny, Nx), epoch e's band b is map e*nbands + b;
    returns (ntracks, nep*nbands) light curves sampled at the shared epochs t (nep,)."""
    nm, Ny, Nx = maps.shape
    nep = t.numel()
    assert nm == nep * nbands
    n = x0.numel()
    if out is None:
        out = torch.empty((n, nep * nbands), dtype=maps.dtype, device=maps.device)
    ctx.check(ctx.L.mlc_sample_expanding(ctx.h, _ptr(maps), Nx, Ny, _PREC[maps.dtype], nep, nbands, n, _ptr(x0),
                                         _ptr(y0), _ptr(phi), _ptr(v), _ptr(t), int(mag), _ptr(out)))
    return out


TRACK_KEYS = ("x0", "y0", "phi", "v", "off", "t")


def convolve_sample_tracks(ctx: Context, m: Map, profiles, tracks: dict, mag=True, pixels=None, out=None,
                           mode="fused", async_=False, graph=False):
    """The light-curve step of one image in one library call (mlc_convolve_sample_tracks).

    tracks: dict of x0, y0, phi, v (map precision), off (int64, ntracks + 1) and t (map
    precision), either all CUDA tensors (device buffers, everything on the context's
    stream) or all CPU tensors / numpy arrays (host buffers: copies overlap the kernels;
    page-locked tensors let them run asynchronously).  pixels: new map pixels (same
    location as the tracks) or None to keep the map's.  Returns out[nprof, nepochs].
    Device buffers: stream-ordered on the context's stream.  Host buffers: the call returns
    with out filled, or with async_=True once queued (out valid after ctx.synchronize()).
    graph=True (device buffers): the step is captured as one CUDA graph after its first
    eager run and replayed by later calls with the same buffers, sizes and profile raster
    sizes (contents and profile values may change).
    """
    tr = {k: tracks[k] for k in TRACK_KEYS}
    first = tr["x0"]
    host = not (isinstance(first, torch.Tensor) and first.is_cuda)
    for k, a in tr.items():
        is_dev = isinstance(a, torch.Tensor) and a.is_cuda
        if is_dev == host:
            raise ValueError("track arrays must all be on the device or all on the host")
        want = np.int64 if k == "off" else (np.float64 if m.prec == MLC_F64 else np.float32)
        dt = torch.int64 if k == "off" else m.dtype
        if isinstance(a, torch.Tensor):
            if a.dtype != dt or not a.is_contiguous():
                raise ValueError(f"tracks[{k!r}] must be a contiguous {dt} tensor")
        elif isinstance(a, np.ndarray):
            if a.dtype != want or not a.flags.c_contiguous:
                raise ValueError(f"tracks[{k!r}] must be a contiguous {want} array")
        else:
            raise TypeError(type(a))
    off = tr["off"]
    ntr = int(off.shape[0]) - 1
    if host:
        E = int(off[-1])
    else:
        E = int(tr["t"].shape[0])
    nprof = len(profiles)
    if out is None:
        if host:
            out = torch.empty((nprof, E), dtype=m.dtype, pin_memory=torch.cuda.is_available())
        else:
            out = torch.empty((nprof, E), dtype=m.dtype, device=first.device)
    flags = (_lib.MLC_IO_HOST if host else 0) | (_lib.MLC_ASYNC if async_ else 0) | (_lib.MLC_GRAPH if graph else 0)
    T = _lib.MlcTracks(ntr, E, *[_ptr(tr[k]) for k in TRACK_KEYS])
    P = (_lib.MlcProfile * nprof)(*profiles)
    md = _MODES[mode]
    ctx.check(ctx.L.mlc_convolve_sample_tracks(ctx.h, m.h, _ptr(pixels), nprof, P, C.byref(T), md, int(mag),
                                               _ptr(out), flags))
    return out


def track_chi2_offset(ctx: Context, imap: torch.Tensor, nmaps: int, x0, y0, phi, v, t, obs, w, out=None):
    """Fused sample -> magnitude -> offset-minimised chi2 of every track against one
    observed curve on shared epochs t (T,).  imap: (Ny, Nx) map or (Ny, Nx, stride)
    interleaved maps; obs, w: (T,) float64 CUDA tensors.  Returns (chi2, dm), each
    (nmaps, ntracks) float64."""
    if imap.dim() == 2:
        Ny, Nx = imap.shape
        stride = 1
    else:
        Ny, Nx, stride = imap.shape
    n = x0.numel()
    chi2 = out if out is not None else torch.empty((nmaps, n), dtype=torch.float64, device=x0.device)
    dm = torch.empty((nmaps, n), dtype=torch.float64, device=x0.device)
    ctx.check(ctx.L.mlc_track_chi2_offset(ctx.h, _ptr(imap), stride, nmaps, Nx, Ny, _PREC[imap.dtype], n, _ptr(x0),
                                          _ptr(y0), _ptr(phi), _ptr(v), t.numel(), _ptr(t), _ptr(obs), _ptr(w),
                                          _ptr(chi2), _ptr(dm)))
    return chi2, dm


def chi2_offset(ctx: Context, m: torch.Tensor, obs, w):
    """Offset-minimised chi2 of each row of m against obs with weights w."""
    n, T = m.shape
    obs = _np(obs, np.float64)
    w = _np(w, np.float64)
    chi2 = torch.empty(n, dtype=torch.float64, device=m.device)
    dm = torch.empty(n, dtype=torch.float64, device=m.device)
    ctx.check(ctx.L.mlc_chi2_offset(ctx.h, _PREC[m.dtype], n, T, _ptr(m), _ptr(obs), _ptr(w), _ptr(chi2), _ptr(dm)))
    return chi2, dm


@dataclass
class Chi2Vars:
    """Chi2Vars (data_structs.hpp:4-18)."""
    Njp: int
    indA: np.ndarray
    indB: np.ndarray
    facA: np.ndarray
    facB: np.ndarray
    d: np.ndarray
    s: np.ndarray
    const_term: float


def setup_chi2_calculation(M, V, Dfac, d, t, s, x, ref_compat=True) -> Chi2Vars:
    L = _lib.load()
    d = _np(d, np.float64); t = _np(t, np.float64); s = _np(s, np.float64); x = _np(x, np.float64)
    Nd = d.size
    indA = np.zeros(Nd, np.int32); indB = np.zeros(Nd, np.int32)
    facA = np.zeros(Nd); facB = np.zeros(Nd); nd = np.zeros(Nd); ns = np.zeros(Nd)
    Njp = C.c_int(); ct = C.c_double()
    st = L.mlc_setup_chi2(M[0], M[1], V[0], Dfac, Nd, _ptr(d), _ptr(t), _ptr(s), x.size, _ptr(x), int(ref_compat),
                          C.byref(Njp), _ptr(indA), _ptr(indB), _ptr(facA), _ptr(facB), _ptr(nd), _ptr(ns),
                          C.byref(ct))
    if st:
        raise MlcError(st, "mlc_setup_chi2 failed")
    n = Njp.value
    return Chi2Vars(n, indA[:n].copy(), indB[:n].copy(), facA[:n].copy(), facB[:n].copy(), nd[:n].copy(),
                    ns[:n].copy(), ct.value)


def _vars_args(v: Chi2Vars):
    arrs = [_np(v.indA, np.int32), _np(v.indB, np.int32), _np(v.facA, np.float64), _np(v.facB, np.float64),
            _np(v.d, np.float64), _np(v.s, np.float64)]
    return arrs, [_ptr(a) for a in arrs]


def setup_integral(ctx: Context, LCA: torch.Tensor, LCB: torch.Tensor, edges, want_rank: bool = True):
    """setup_integral_GPU: returns (rank as int32 device tensor holding uint32, lower, nper)."""
    Nloc, Nprof = LCA.shape
    edges = _np(edges, np.float64)
    nb = edges.size
    rank = torch.empty(Nloc * Nloc, dtype=torch.int32, device=LCA.device) if want_rank else None
    lower = np.zeros(max(nb, 1), np.uint32); nper = np.zeros(max(nb, 1), np.uint32)
    ctx.check(ctx.L.mlc_pair_setup(ctx.h, Nloc, Nprof, _ptr(LCA), _ptr(LCB), nb, _ptr(edges), _ptr(rank),
                                   _ptr(lower), _ptr(nper)))
    return rank, lower[:nb], nper[:nb]


def calculate_chi2(ctx: Context, v: Chi2Vars, LCA, DLCA, LCB, DLCB, rank=None):
    """calculate_chi2_GPU: FP64 chi2 of all Nloc^2 pairs, at rank order if rank is given."""
    Nloc, Nprof = LCA.shape
    keep, p = _vars_args(v)
    out = torch.empty(Nloc * Nloc, dtype=torch.float64, device=LCA.device)
    ctx.check(ctx.L.mlc_pair_chi2_ratio(ctx.h, v.Njp, *p, Nloc, Nprof, _ptr(LCA.contiguous()),
                                        _ptr(DLCA.contiguous()), _ptr(LCB.contiguous()), _ptr(DLCB.contiguous()),
                                        _ptr(rank), _ptr(out)))
    return out


def bin_chi2(ctx: Context, lower, nper, chi2_sorted: torch.Tensor):
    """bin_chi2_GPU: (binned_chi2, binned_exp) host arrays."""
    lower = _np(lower, np.uint32); nper = _np(nper, np.uint32)
    nb = lower.size
    bc = np.zeros(nb); be = np.zeros(nb)
    ctx.check(ctx.L.mlc_bin_chi2(ctx.h, nb, _ptr(lower), _ptr(nper), _ptr(chi2_sorted), _ptr(bc), _ptr(be)))
    return bc, be


def pair_bin_fused(ctx: Context, v: Chi2Vars, LCA, DLCA, LCB, DLCB, edges):
    Nloc, Nprof = LCA.shape
    keep, p = _vars_args(v)
    edges = _np(edges, np.float64)
    nb = edges.size
    bc = np.zeros(nb); be = np.zeros(nb); nper = np.zeros(nb, np.uint32)
    ctx.check(ctx.L.mlc_pair_bin_fused(ctx.h, v.Njp, *p, Nloc, Nprof, _ptr(LCA.contiguous()),
                                       _ptr(DLCA.contiguous()), _ptr(LCB.contiguous()), _ptr(DLCB.contiguous()), nb,
                                       _ptr(edges), _ptr(bc), _ptr(be), _ptr(nper)))
    return bc, be, nper


def pair_chi2_magdiff(ctx: Context, A: torch.Tensor, B: torch.Tensor, w, d=None, offset: bool = False,
                      method: str = "tensor", nbins: int = 1000, lo: float = -2.0, hi: float = 8.0, k: int = 0,
                      want_matrix: bool = False):
    """Magnitude-difference pair chi2: returns dict(hist, topk_val, topk_i, topk_j, matrix, stats)."""
    from ._lib import MlcPairStats
    NA, T = A.shape
    NB = B.shape[0]
    w = _np(w, np.float64)
    dd = None if d is None else _np(d, np.float64)
    hist = np.zeros(nbins, np.uint64)
    tv = np.zeros(max(k, 1)); ti = np.zeros(max(k, 1), np.int64); tj = np.zeros(max(k, 1), np.int64)
    mat = torch.empty((NA, NB), dtype=torch.float32, device=A.device) if want_matrix else None
    st = MlcPairStats()
    ctx.check(ctx.L.mlc_pair_chi2_magdiff(ctx.h, 1 if method == "tensor" else 0, NA, NB, T, _ptr(A.contiguous()),
                                          _ptr(B.contiguous()), _ptr(w), _ptr(dd), int(offset), nbins, lo, hi,
                                          _ptr(hist), k, _ptr(tv), _ptr(ti), _ptr(tj), _ptr(mat), C.byref(st)))
    return dict(hist=hist, topk_val=tv[:k], topk_i=ti[:k], topk_j=tj[:k], matrix=mat,
                stats=dict(delta=st.delta, threshold=st.threshold, refined=st.refined, candidates=st.candidates,
                           passes=st.passes, below=st.below, above=st.above))


class PairSide:
    """One image's curves made ready for the tensor-core pair stage once (centred, weighted,
    quantised), then paired with any number of sides by pair_chi2_sides.  Built from FP32
    curves (PairSide.curves) or straight from an expanding source's convolved FP32 maps and
    tracks (PairSide.expanding), in which case no light curve is stored."""

    def __init__(self, ctx: Context, h, N: int, T: int):
        self.ctx = ctx
        self.h = h
        self.N, self.T = N, T
        ctx._maps.add(self)

    @classmethod
    def curves(cls, ctx: Context, X: torch.Tensor, w, d=None, offset: bool = False):
        if X.dtype != torch.float32 or not X.is_cuda:
            raise ValueError("pair side curves: a device FP32 tensor")
        X = X.contiguous()
        N, T = X.shape
        w = _np(w, np.float64)
        dd = None if d is None else _np(d, np.float64)
        h = C.c_void_p()
        ctx.check(ctx.L.mlc_pair_side_curves(ctx.h, N, T, _ptr(X), _ptr(w), _ptr(dd), int(offset), C.byref(h)))
        return cls(ctx, h, N, T)

    @classmethod
    def expanding(cls, ctx: Context, maps: torch.Tensor, nep: int, nbands: int, x0, y0, phi, v, t, w, d=None,
                  offset: bool = False):
        """maps: nep*nbands FP32 planes (Ny x Nx) on the device, plane e*nbands + b for epoch e,
        band b; track arrays FP32 device tensors; t: the nep shared epochs."""
        if maps.dtype != torch.float32 or not maps.is_cuda:
            raise ValueError("pair side maps: a device FP32 tensor")
        maps = maps.contiguous()
        Ny, Nx = maps.shape[-2:]
        if maps.numel() != nep * nbands * Nx * Ny:
            raise ValueError("pair side maps: nep*nbands planes")
        trk = [a.contiguous() for a in (x0, y0, phi, v, t)]
        if any(a.dtype != torch.float32 or not a.is_cuda for a in trk):
            raise ValueError("pair side tracks: device FP32 tensors")
        w = _np(w, np.float64)
        dd = None if d is None else _np(d, np.float64)
        h = C.c_void_p()
        ctx.check(ctx.L.mlc_pair_side_expanding(ctx.h, _ptr(maps), Nx, Ny, nep, nbands, trk[0].numel(),
                                                *[_ptr(a) for a in trk], _ptr(w), _ptr(dd), int(offset),
                                                C.byref(h)))
        return cls(ctx, h, trk[0].numel(), nep * nbands)

    def close(self):
        if getattr(self, "h", None):
            self.ctx.L.mlc_pair_side_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def pair_chi2_sides(ctx: Context, A: PairSide, B: PairSide, nbins: int = 1000, lo: float = -2.0, hi: float = 8.0,
                    k: int = 0, want_matrix: bool = False):
    """pair_chi2_magdiff (tensor form) between two prepared sides; same dict of results."""
    from ._lib import MlcPairStats
    hist = np.zeros(nbins, np.uint64)
    tv = np.zeros(max(k, 1)); ti = np.zeros(max(k, 1), np.int64); tj = np.zeros(max(k, 1), np.int64)
    mat = torch.empty((A.N, B.N), dtype=torch.float32, device=f"cuda:{ctx.device}") if want_matrix else None
    st = MlcPairStats()
    ctx.check(ctx.L.mlc_pair_chi2_sides(ctx.h, A.h, B.h, nbins, lo, hi, _ptr(hist), k, _ptr(tv), _ptr(ti), _ptr(tj),
                                        _ptr(mat), C.byref(st)))
    return dict(hist=hist, topk_val=tv[:k], topk_i=ti[:k], topk_j=tj[:k], matrix=mat,
                stats=dict(delta=st.delta, threshold=st.threshold, refined=st.refined, candidates=st.candidates,
                           passes=st.passes, below=st.below, above=st.above))


def pair_chi2_magdiff_list(ctx: Context, A: torch.Tensor, B: torch.Tensor, w, ia, ib, d=None, offset=False):
    NA, T = A.shape
    NB = B.shape[0]
    w = _np(w, np.float64)
    dd = None if d is None else _np(d, np.float64)
    ia = torch.as_tensor(np.asarray(ia, np.int64), device=A.device)
    ib = torch.as_tensor(np.asarray(ib, np.int64), device=A.device)
    out = torch.empty(ia.numel(), dtype=torch.float64, device=A.device)
    ctx.check(ctx.L.mlc_pair_chi2_magdiff_list(ctx.h, NA, NB, T, _ptr(A.contiguous()), _ptr(B.contiguous()), _ptr(w),
                                               _ptr(dd), int(offset), ia.numel(), _ptr(ia), _ptr(ib), _ptr(out)))
    return out


def sort_f64_u32(ctx: Context, keys: torch.Tensor, vals: torch.Tensor):
    """Stable in-place radix sort of FP64 keys with 32-bit values (int32 tensor)."""
    ctx.check(ctx.L.mlc_sort_f64_u32(ctx.h, keys.numel(), _ptr(keys), _ptr(vals)))


def histogram_f64(ctx: Context, v: torch.Tensor, nbins: int, lo: float, hi: float, log: bool = False):
    out = np.zeros(nbins, np.uint64)
    ctx.check(ctx.L.mlc_histogram_f64(ctx.h, v.numel(), _ptr(v), nbins, lo, hi, int(log), _ptr(out)))
    return out


class _HostBuffer:
    """One mlc_host_alloc buffer, released when the last array or tensor on it is gone."""

    def __init__(self, nbytes: int):
        self.L = _lib.load()
        p = C.c_void_p()
        st = self.L.mlc_host_alloc(nbytes, C.byref(p))
        if st:
            raise MlcError(st, "mlc_host_alloc failed (host memory or registration with the CUDA driver)")
        self.ptr = p.value

    def __del__(self):
        if getattr(self, "ptr", None):
            self.L.mlc_host_free(C.c_void_p(self.ptr))
            self.ptr = None


_NP_OF = {torch.float32: np.float32, torch.float64: np.float64, torch.int64: np.int64, torch.int32: np.int32,
          torch.uint8: np.uint8}


def host_empty(shape, dtype=torch.float32) -> torch.Tensor:
    """A zero-filled CPU tensor in page-locked host memory on 2 MB pages (mlc_host_alloc),
    for the host-buffer form of the library calls: its copies to and from the GPU keep
    their rate when the host's memory is fragmented."""
    shape = tuple(shape) if isinstance(shape, (tuple, list)) else (int(shape),)
    numel = int(np.prod(shape)) if shape else 1
    nbytes = max(numel * torch.empty((), dtype=dtype).element_size(), 1)
    owner = _HostBuffer(nbytes)
    raw = (C.c_char * nbytes).from_address(owner.ptr)
    raw._owner = owner
    arr = np.frombuffer(raw, dtype=np.uint8).view(_NP_OF[dtype])[:numel].reshape(shape)
    return torch.from_numpy(arr)


def selftest_wait_timeout(ctx: Context, polls: int = 4096):
    """Runs the bounded-wait self-test (mlc_selftest_wait_timeout).  Returns (status, report):
    status MLC_ERR_TIMEOUT (4) when the wait gave up, as it should; report = [gave up, polls
    used, tensor memory released].  The context stays usable either way."""
    rep = np.zeros(3, np.uint32)
    st = ctx.L.mlc_selftest_wait_timeout(ctx.h, int(polls), _ptr(rep))
    return st, rep


def bin_edges(Nbins: int, mn: float, mx: float, log: bool = True) -> np.ndarray:
    out = np.zeros(Nbins)
    st = _lib.load().mlc_bin_edges(Nbins, mn, mx, int(log), _ptr(out))
    if st:
        raise MlcError(st, "bad bin spec")
    return out


def trapezium(f1, f2, x) -> float:
    f1 = _np(f1, np.float64); f2 = _np(f2, np.float64); x = _np(x, np.float64)
    return _lib.load().mlc_trapezium(x.size, _ptr(f1), _ptr(f2), _ptr(x))


def locations_grid(Nside, Nmap, Noff):
    x = np.zeros(Nside * Nside, np.int32); y = np.zeros(Nside * Nside, np.int32)
    st = _lib.load().mlc_locations_grid(Nside, Nmap, Noff, _ptr(x), _ptr(y))
    if st:
        raise MlcError(st, "bad grid")
    return x, y


def locations_random(Nloc, Nmap, Noff, seed):
    x = np.zeros(Nloc, np.int32); y = np.zeros(Nloc, np.int32)
    st = _lib.load().mlc_locations_random(Nloc, Nmap, Noff, seed, _ptr(x), _ptr(y))
    if st:
        raise MlcError(st, "bad random locations")
    return x, y


def read_gerlumph(directory: str):
    L = _lib.load()
    n = C.c_int(); w = C.c_double(); meta = np.zeros(6)
    st = L.mlc_read_gerlumph(directory.encode(), C.byref(n), C.byref(w), _ptr(meta), None, 0)
    if st:
        raise MlcError(st, f"cannot read {directory}")
    out = np.zeros(n.value * n.value)
    st = L.mlc_read_gerlumph(directory.encode(), C.byref(n), C.byref(w), _ptr(meta), _ptr(out), out.size)
    if st:
        raise MlcError(st, f"cannot read {directory}")
    return out.reshape(n.value, n.value), w.value, meta
