"""CPU oracle for the microLC light-curve hot path -- TEST INFRASTRUCTURE ONLY.

This package is the checker, never the thing measured or shipped.  Only tests/,
``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg (and its reference arm)
may import it.  It wraps

* ``libmlc_oracle.so`` -- a plain-C FP64 restatement of the reference's algorithm
  for each stage (oracle/mlc_oracle.c, each function citing the reference lines it
  follows), built by :func:`build`;
* ``_ref/libmlcref.so`` -- the reference's own CPU code (microLC
  simulating_lcurves/src/*.cpp) compiled from its sources by oracle/Makefile, used
  here only to pin the restatement (present in the build container only);
* numpy FP64 FFT convolution, a restatement of the reference's cuFFT D2Z/Z2D
  sequence (gpu_functions.cu:171-209, 571-577) with the kernel wrap of
  Kernel::setKernel (magnification_map.cpp:172-193).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_bin", "libmlc_oracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libmlcref.so")

def _reference_src():
    """The reference's simulating_lcurves directory: $MLC_REFERENCE (the checkout's root),
    else a checkout named "reference" beside this repository; None when neither exists
    (on machines without the reference the golden vectors in tests/golden pin the oracle)."""
    root = os.environ.get("MLC_REFERENCE") or os.path.join(os.path.dirname(HERE), "..", "reference")
    d = os.path.normpath(os.path.join(root, "simulating_lcurves"))
    return d if os.path.isdir(os.path.join(d, "src")) else None


REFERENCE_SRC = _reference_src()
REFCUDA_MK = os.path.join(HERE, "refcuda.mk")
REFCUDA_DIR = os.path.join(os.path.dirname(HERE), "baseline", "_ref")
REFCUDA_PATH = os.path.join(REFCUDA_DIR, "libmlcref_cuda.so")

SHAPES = {
    "uniform": 0,
    "gaussian": 1,
    "gaussian_hole": 2,
    "thermal_hole": 3,
    "wavy": 4,
    "exponential": 5,
    "limb_darkened": 6,
}

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_fp = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_up = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
_lp = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
_u64p = np.ctypeslib.ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")


def build(force: bool = False) -> None:
    """Compile the C restatement (and, where the reference sources exist, the
    reference's CPU code into _ref/)."""
    os.makedirs(os.path.join(HERE, "_bin"), exist_ok=True)
    src = os.path.join(HERE, "mlc_oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.check_call(["gcc", "-O3", "-ffp-contract=off", "-fPIC", "-shared", "-o", LIB_PATH, src, "-lm"])
    if REFERENCE_SRC:
        subprocess.check_call(["make", "-s", "-C", HERE, "-j8", f"REF={REFERENCE_SRC}"])
        # the reference's CUDA sources, staged where they travel with the repository
        subprocess.check_call(["make", "-s", "-f", REFCUDA_MK, "stage", f"REF={REFERENCE_SRC}"],
                              stdout=subprocess.DEVNULL)


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.orc_profile_dims.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int]
        L.orc_profile_raster.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                         C.c_double, C.c_double, C.c_double, C.c_int, _dp, C.c_long]
        L.orc_kernel_wrap.argtypes = [_dp, C.c_int, C.c_int, C.c_int, _dp]
        L.orc_conv_direct.argtypes = [_dp, C.c_int, C.c_int, _dp, C.c_int, _dp]
        L.orc_sample_nearest.argtypes = [_dp, C.c_int, C.c_int, C.c_int, C.c_int, _ip, _ip, _dp, _dp]
        L.orc_find_indices.argtypes = [_dp, _dp, C.c_int, C.c_int, _ip]
        L.orc_setup_chi2.argtypes = [C.c_double, C.c_double, C.c_double, C.c_double, C.c_int, _dp, _dp,
                                     _dp, C.c_int, _dp, C.c_int, _ip, _ip, _dp, _dp, _dp, _dp, _dp]
        L.orc_flux_ratio.argtypes = [_fp, _fp, _fp, _fp, C.c_int, C.c_int, C.c_int, C.c_void_p]
        L.orc_flux_ratio.restype = C.c_double
        L.orc_flux_ratio_f32.argtypes = [_fp, _fp, _fp, _fp, C.c_int, C.c_int, C.c_int]
        L.orc_flux_ratio_f32.restype = C.c_float
        L.orc_fit_raster.argtypes = [C.c_double, C.c_double, C.c_int, _dp, _dp, _dp, _dp]
        L.orc_track_fit.argtypes = [_dp, C.c_int, C.c_int, C.c_int, _dp, C.c_int, _dp, _lp, _dp, _dp, _dp, _dp,
                                    _dp, C.c_void_p]
        L.orc_binned_mpd.argtypes = [_dp, C.c_long, C.c_int, C.c_double, C.c_double, _dp, _dp]
        L.orc_mpd_divide.argtypes = [C.c_int, _dp, _dp, C.c_int, _dp, _dp, C.c_int, _dp, _dp]
        L.orc_mpd_normalize.argtypes = [C.c_int, _dp, _dp]
        L.orc_pair_rank.argtypes = [C.c_int, C.c_int, _dp, _dp, C.c_int, _dp, _up, _up, _up]
        L.orc_pair_chi2_ratio.argtypes = [C.c_int, _ip, _ip, _dp, _dp, _dp, _dp, C.c_int, C.c_int,
                                          _dp, _dp, _dp, _dp, C.c_void_p, _dp]
        L.orc_bin_chi2.argtypes = [C.c_int, _up, _up, _dp, _dp, _dp]
        L.orc_mpd_edges.argtypes = [C.c_int, C.c_double, C.c_double, C.c_int, _dp]
        L.orc_trapezium.argtypes = [C.c_int, _dp, _dp, _dp]
        L.orc_trapezium.restype = C.c_double
        L.orc_bilinear.argtypes = [_dp, C.c_int, C.c_int, C.c_double, C.c_double]
        L.orc_bilinear.restype = C.c_double
        L.orc_sample_tracks.argtypes = [_dp, C.c_int, C.c_int, C.c_int, _dp, _dp, _dp, _dp, _lp, _dp, C.c_int, _dp]
        L.orc_chi2_offset.argtypes = [C.c_int, C.c_int, _dp, _dp, _dp, _dp, _dp]
        L.orc_pair_chi2_magdiff.argtypes = [C.c_int, C.c_int, C.c_int, _fp, _fp, _dp, C.c_void_p, C.c_int,
                                            C.c_long, C.c_void_p, C.c_void_p, _dp]
        L.orc_histogram.argtypes = [C.c_long, _dp, C.c_int, C.c_double, C.c_double, C.c_int, C.c_double,
                                    _u64p, _u64p]
        L.orc_topk_smallest.argtypes = [C.c_long, _dp, C.c_long, _lp]
        L.orc_rayshoot.argtypes = [_fp, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                                   C.c_long, C.c_long, C.c_double, C.c_int, C.c_long, C.c_long, _ip]
        _lib = L
    return _lib


def ref_available() -> bool:
    """The reference's CPU code is here: compiled on first use where its sources exist (a
    failed build raises instead of skipping the tests that pin the oracle to it)."""
    if not os.path.exists(REF_PATH) and REFERENCE_SRC:
        build()
    return os.path.exists(REF_PATH)


def ref():
    """The reference's own CPU code (only where it was compiled from its sources)."""
    global _ref
    if _ref is None:
        R = C.CDLL(REF_PATH)
        R.ref_setup_chi2.argtypes = [C.c_double, C.c_double, C.c_double, C.c_double, C.c_int, _dp, _dp, _dp,
                                     C.c_int, _dp, _ip, _ip, _ip, _dp, _dp, _dp, _dp, _dp]
        R.ref_setup_integral_cpu.argtypes = [C.c_int, C.c_int, _dp, _dp, _up]
        R.ref_calculate_chi2_cpu.argtypes = [C.c_int, _ip, _ip, _dp, _dp, _dp, _dp, C.c_int, C.c_int,
                                             _dp, _dp, _dp, _dp, _up, _dp]
        R.ref_bin_chi2_cpu.argtypes = [C.c_int, C.c_int, _up, _up, _dp, _dp, _dp]
        R.ref_profile.argtypes = [C.c_char_p, C.c_double, C.c_double, C.POINTER(C.c_int),
                                  C.POINTER(C.c_int), C.c_void_p, C.c_long]
        R.ref_kernel.argtypes = [C.c_char_p, C.c_double, C.c_double, C.c_int, C.c_int, _dp]
        R.ref_locations_grid.argtypes = [C.c_int, C.c_int, C.c_int, _ip, _ip]
        R.ref_locations_random.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _ip, _ip]
        R.ref_mpd_edges.argtypes = [C.c_int, C.c_double, C.c_double, C.c_int, _dp]
        R.ref_trapezium.argtypes = [C.c_int, _dp, _dp, _dp]
        R.ref_trapezium.restype = C.c_double
        R.chi2 = C.CDLL(os.path.join(HERE, "_ref", "libmlcref_chi2.so"))
        R.chi2.ref_chi2_cpu.argtypes = [_fp, _fp, _fp, _fp, C.c_int, C.c_int, C.c_int]
        R.chi2.ref_chi2_cpu.restype = C.c_float
        R.ref_binned_mpd.argtypes = [_dp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, _dp, _dp]
        R.ref_mpd_divide.argtypes = [C.c_int, _dp, _dp, C.c_int, _dp, _dp, C.c_int, _dp, _dp]
        R.ref_mpd_normalize.argtypes = [C.c_int, _dp, _dp]
        R.ref_read_map.argtypes = [C.c_char_p, C.c_double, C.POINTER(C.c_int), C.POINTER(C.c_double),
                                   C.POINTER(C.c_double), C.c_void_p, C.c_long]
        _ref = R
    return _ref


# ----------------------------------------------------------------------------- profiles

def profile(shape: str, rhalf: float, pix: float, incl=0.0, orient=0.0, Rin=0.0, a=1.0, u=0.0,
            ref_compat=True) -> np.ndarray:
    """Normalised N x N profile raster (profile.cpp:143-446)."""
    L = lib()
    s = SHAPES[shape]
    N = L.orc_profile_dims(s, rhalf, pix, Rin, a, int(ref_compat))
    out = np.zeros(N * N, np.float64)
    n = L.orc_profile_raster(s, rhalf, pix, incl, orient, Rin, a, u, int(ref_compat), out, out.size)
    assert n == N, n
    return out.reshape(N, N)


def kernel_wrap(prof: np.ndarray, Nx: int, Ny: int) -> np.ndarray:
    out = np.zeros(Nx * Ny, np.float64)
    lib().orc_kernel_wrap(np.ascontiguousarray(prof, np.float64).ravel(), prof.shape[0], Nx, Ny, out)
    return out.reshape(Ny, Nx)


def conv_fft(mp: np.ndarray, prof: np.ndarray) -> np.ndarray:
    """FP64 FFT convolution: irfft2(rfft2(map) * rfft2(wrapped kernel))."""
    Ny, Nx = mp.shape
    k = kernel_wrap(prof, Nx, Ny)
    F = np.fft.rfft2(mp) * np.fft.rfft2(k)
    return np.fft.irfft2(F, s=(Ny, Nx))


def conv_fft_workers(mp: np.ndarray, prof: np.ndarray, workers: int = -1) -> np.ndarray:
    """Same as conv_fft, multi-threaded via scipy.fft (the CPU-baseline form)."""
    import scipy.fft as sf
    Ny, Nx = mp.shape
    k = kernel_wrap(prof, Nx, Ny)
    F = sf.rfft2(mp, workers=workers)
    F *= sf.rfft2(k, workers=workers)
    return sf.irfft2(F, s=(Ny, Nx), workers=workers)


def conv_direct(mp: np.ndarray, prof: np.ndarray) -> np.ndarray:
    Ny, Nx = mp.shape
    out = np.zeros(Nx * Ny, np.float64)
    lib().orc_conv_direct(np.ascontiguousarray(mp, np.float64).ravel(), Nx, Ny,
                          np.ascontiguousarray(prof, np.float64).ravel(), prof.shape[0], out)
    return out.reshape(Ny, Nx)


# ----------------------------------------------------------------------------- sampling

def sample_nearest(mp: np.ndarray, k: int, Nprof: int, lx: np.ndarray, ly: np.ndarray, LC: np.ndarray,
                   DLC: np.ndarray) -> None:
    lib().orc_sample_nearest(np.ascontiguousarray(mp, np.float64).ravel(), mp.shape[1], k, Nprof, lx.size,
                             lx.astype(np.int32), ly.astype(np.int32), LC, DLC)


def expanding_source(mp: np.ndarray, sizes, shape: str, lx, ly, pix_phys: float, width: float,
                     conv=conv_fft):
    """Restatement of expanding_source (gpu_functions.cu:82-225): LC (Nloc x Nprof) and
    DLC (Nloc x (Nprof-1)).  sizes[0] must be 0 (point source)."""
    Ny, Nx = mp.shape
    Nprof = len(sizes)
    Nloc = len(lx)
    LC = np.zeros(Nloc * Nprof)
    DLC = np.zeros(Nloc * max(Nprof - 1, 1))
    lx = np.asarray(lx, np.int32)
    ly = np.asarray(ly, np.int32)
    sample_nearest(mp, 0, Nprof, lx, ly, LC, DLC)
    for k in range(1, Nprof):
        rhalf = sizes[k] * pix_phys * Nx / width
        prof = profile(shape, rhalf, pix_phys)
        cm = conv(mp, prof)
        sample_nearest(cm, k, Nprof, lx, ly, LC, DLC)
    return LC.reshape(Nloc, Nprof), DLC[: Nloc * (Nprof - 1)].reshape(Nloc, max(Nprof - 1, 0))


def bilinear(mp: np.ndarray, x: float, y: float) -> float:
    return lib().orc_bilinear(np.ascontiguousarray(mp, np.float64).ravel(), mp.shape[1], mp.shape[0], x, y)


def sample_tracks(mp, x0, y0, phi, v, off, t, mag=True):
    mpc = np.ascontiguousarray(mp, np.float64)
    out = np.zeros(int(off[-1]), np.float64)
    lib().orc_sample_tracks(mpc.ravel(), mp.shape[1], mp.shape[0], len(x0), np.asarray(x0, np.float64),
                            np.asarray(y0, np.float64), np.asarray(phi, np.float64), np.asarray(v, np.float64),
                            np.asarray(off, np.int64), np.asarray(t, np.float64), int(mag), out)
    return out


# ----------------------------------------------------------------------------- chi2

def setup_chi2(M, V, Dfac, d, t, s, x, ref_compat=True):
    """setup_chi2_calculation restated -> dict(Njp, indA, indB, facA, facB, d, s, const_term)."""
    Nd = len(d)
    indA = np.zeros(Nd, np.int32); indB = np.zeros(Nd, np.int32)
    facA = np.zeros(Nd); facB = np.zeros(Nd); nd = np.zeros(Nd); ns = np.zeros(Nd)
    ct = np.zeros(1)
    Njp = lib().orc_setup_chi2(M[0], M[1], V[0], Dfac, Nd, np.asarray(d, np.float64), np.asarray(t, np.float64),
                               np.asarray(s, np.float64), len(x), np.asarray(x, np.float64), int(ref_compat),
                               indA, indB, facA, facB, nd, ns, ct)
    return dict(Njp=Njp, indA=indA[:Njp], indB=indB[:Njp], facA=facA[:Njp], facB=facB[:Njp],
                d=nd[:Njp], s=ns[:Njp], const_term=float(ct[0]))


def pair_rank(LCA, LCB, edges=None):
    Nloc, Nprof = LCA.shape
    P = Nloc * Nloc
    rank = np.zeros(P, np.uint32)
    nb = 0 if edges is None else len(edges)
    e = np.zeros(max(nb, 1)) if edges is None else np.asarray(edges, np.float64)
    lower = np.zeros(max(nb, 1), np.uint32); nper = np.zeros(max(nb, 1), np.uint32)
    lib().orc_pair_rank(Nloc, Nprof, np.ascontiguousarray(LCA).ravel(), np.ascontiguousarray(LCB).ravel(),
                        nb, e, rank, lower, nper)
    return rank, lower[:nb], nper[:nb]


def pair_chi2_ratio(v, LCA, DLCA, LCB, DLCB, rank=None):
    Nloc, Nprof = LCA.shape
    out = np.zeros(Nloc * Nloc)
    rp = None if rank is None else np.ascontiguousarray(rank, np.uint32)
    lib().orc_pair_chi2_ratio(v["Njp"], np.ascontiguousarray(v["indA"], np.int32),
                              np.ascontiguousarray(v["indB"], np.int32), np.ascontiguousarray(v["facA"]),
                              np.ascontiguousarray(v["facB"]), np.ascontiguousarray(v["d"]),
                              np.ascontiguousarray(v["s"]), Nloc, Nprof, np.ascontiguousarray(LCA).ravel(),
                              np.ascontiguousarray(DLCA).ravel(), np.ascontiguousarray(LCB).ravel(),
                              np.ascontiguousarray(DLCB).ravel(),
                              None if rp is None else rp.ctypes.data_as(C.c_void_p), out)
    return out


def bin_chi2(lower, nper, chi2_sorted):
    nb = len(lower)
    bc = np.zeros(nb); be = np.zeros(nb)
    lib().orc_bin_chi2(nb, np.ascontiguousarray(lower, np.uint32), np.ascontiguousarray(nper, np.uint32),
                       np.ascontiguousarray(chi2_sorted, np.float64), bc, be)
    return bc, be


def mpd_edges(Nbins, mn, mx, log=True):
    out = np.zeros(Nbins)
    lib().orc_mpd_edges(Nbins, mn, mx, int(log), out)
    return out


def binned_mpd(data, Nbins, mn, mx):
    """getBinnedMpd: (edges, counts) of the map's pixels in log bins (see orc_binned_mpd)."""
    d = np.ascontiguousarray(data, np.float64).ravel()
    edges = mpd_edges(Nbins, mn, mx, True)
    counts = np.zeros(Nbins)
    lib().orc_binned_mpd(d, d.size, Nbins, mn, mx, edges, counts)
    return edges, counts


def mpd_normalize(bins, counts):
    c = np.array(counts, np.float64)
    lib().orc_mpd_normalize(len(c), np.ascontiguousarray(bins, np.float64), c)
    return c


def mpd_divide(bA, cA, bB, cB, bR):
    """Mpd::divide_by: A.divide_by(B, R) -> R's counts."""
    c = lambda a: np.ascontiguousarray(a, np.float64)
    out = np.zeros(len(bR))
    lib().orc_mpd_divide(len(bA), c(bA), c(cA), len(bB), c(bB), c(cB), len(bR), c(bR), out)
    return out


def flux_ratio(f_obs, df_obs, mu1, mu2, want_chi2=False):
    """getChi2CPU in FP64: (likelihood, chi2[y, x] if want_chi2)."""
    fo = np.ascontiguousarray(f_obs, np.float32).ravel(); dfo = np.ascontiguousarray(df_obs, np.float32).ravel()
    m1 = np.ascontiguousarray(mu1, np.float32); m2 = np.ascontiguousarray(mu2, np.float32)
    N, F, T = m1.shape
    chi2 = np.zeros((N, N)) if want_chi2 else None
    like = lib().orc_flux_ratio(fo, dfo, m1.ravel(), m2.ravel(), N, F, T,
                                None if chi2 is None else chi2.ctypes.data_as(C.c_void_p))
    return (like, chi2) if want_chi2 else like


def flux_ratio_f32(f_obs, df_obs, mu1, mu2):
    """getChi2CPU in the reference's own FP32 arithmetic (float likelihood)."""
    fo = np.ascontiguousarray(f_obs, np.float32).ravel(); dfo = np.ascontiguousarray(df_obs, np.float32).ravel()
    m1 = np.ascontiguousarray(mu1, np.float32); m2 = np.ascontiguousarray(mu2, np.float32)
    N, F, T = m1.shape
    return lib().orc_flux_ratio_f32(fo, dfo, m1.ravel(), m2.ravel(), N, F, T)


def fit_raster(rhalf, pix, N):
    """(P, dP/dx, dP/dy, dP/dR) N x N rasters of the smooth thin disc."""
    out = [np.zeros(N * N) for _ in range(4)]
    lib().orc_fit_raster(rhalf, pix, N, *out)
    return tuple(a.reshape(N, N) for a in out)


def radius_stack(mp, radii, pix, N):
    """(Ny, Nx, K, 4) FP64: the map convolved with P, dP/dx, dP/dy, dP/dR for each radius."""
    Ny, Nx = mp.shape
    st = np.zeros((Ny, Nx, len(radii), 4))
    for k, R in enumerate(radii):
        for f, r in enumerate(fit_raster(R, pix, N)):
            st[:, :, k, f] = conv_fft(mp, r)
    return st


def track_fit(stack, radii, theta, off, t, obs, w, model=False):
    """FP64 chi2 (n,), gradient (n, 6) and optionally the model magnitudes."""
    st = np.ascontiguousarray(stack, np.float64)
    Ny, Nx, K, _ = st.shape
    th = np.ascontiguousarray(theta, np.float64)
    n = th.shape[0]
    chi2 = np.zeros(n); grad = np.zeros((n, 6))
    mod = np.zeros(len(t)) if model else None
    lib().orc_track_fit(st.ravel(), Nx, Ny, K, np.ascontiguousarray(radii, np.float64), n, th.ravel(),
                        np.ascontiguousarray(off, np.int64), np.ascontiguousarray(t, np.float64),
                        np.ascontiguousarray(obs, np.float64), np.ascontiguousarray(w, np.float64), chi2, grad,
                        None if mod is None else mod.ctypes.data_as(C.c_void_p))
    return (chi2, grad, mod) if model else (chi2, grad)


def trapezium(f1, f2, x):
    return lib().orc_trapezium(len(x), np.asarray(f1, np.float64), np.asarray(f2, np.float64),
                               np.asarray(x, np.float64))


def chi2_offset(m, o, w):
    m = np.ascontiguousarray(m, np.float64)
    n, T = m.shape
    chi2 = np.zeros(n); dm = np.zeros(n)
    lib().orc_chi2_offset(n, T, m.ravel(), np.asarray(o, np.float64), np.asarray(w, np.float64), chi2, dm)
    return chi2, dm


def pair_chi2_magdiff(A, B, w, d=None, offset=False, ia=None, ib=None):
    A = np.ascontiguousarray(A, np.float32); B = np.ascontiguousarray(B, np.float32)
    NA, T = A.shape
    NB = B.shape[0]
    dd = None if d is None else np.ascontiguousarray(d, np.float64)
    if ia is not None:
        ia = np.ascontiguousarray(ia, np.int64); ib = np.ascontiguousarray(ib, np.int64)
        n = ia.size
    else:
        n = NA * NB
    out = np.zeros(n)
    lib().orc_pair_chi2_magdiff(NA, NB, T, A.ravel(), B.ravel(), np.asarray(w, np.float64),
                                None if dd is None else dd.ctypes.data_as(C.c_void_p), int(offset), n,
                                None if ia is None else ia.ctypes.data_as(C.c_void_p),
                                None if ib is None else ib.ctypes.data_as(C.c_void_p), out)
    return out


def histogram(v, nbins, lo, hi, log=False, rel_tol=0.0):
    v = np.ascontiguousarray(v, np.float64)
    counts = np.zeros(nbins, np.uint64)
    ne = np.zeros(1, np.uint64)
    lib().orc_histogram(v.size, v, nbins, lo, hi, int(log), rel_tol, counts, ne)
    return counts, int(ne[0])


def topk_smallest(v, k):
    v = np.ascontiguousarray(v, np.float64)
    idx = np.zeros(min(k, v.size), np.int64)
    lib().orc_topk_smallest(v.size, v, k, idx)
    return idx


# ----------------------------------------------------------------------------- synthetic maps

def lens_field(kappa_star, gamma, width, seed, margin=2.0):
    """Equal-mass point lenses (unit Einstein radius) uniformly in a disc that covers the
    image-plane region mapping into the source square: the same seeded draws as the
    library's map generator, so both shoot through the same lenses."""
    import math
    rng = np.random.default_rng(seed)
    half = width / 2 + margin
    l1 = half / abs(1 - kappa_star - gamma)
    l2 = half / abs(1 - kappa_star + gamma)
    R = math.hypot(l1, l2) + 5.0
    n = int(round(kappa_star * R * R))
    r = R * np.sqrt(rng.random(n))
    th = 2 * np.pi * rng.random(n)
    return np.stack([r * np.cos(th), r * np.sin(th)], axis=1), (l1, l2)


def rayshoot(N, width, kappa_star, gamma, seed, rays_per_pixel=4.0, threads=None):
    """Inverse ray shooting on the host cores (orc_rayshoot, threads over ray ranges):
    int32 counts (N, N) equal to the library's mlc_rayshoot for the same inputs, and the
    map in the reference's normalisation (magnification_map.cpp:33-38): counts / avgN."""
    import concurrent.futures as cf
    import math
    lenses, (l1, l2) = lens_field(kappa_star, gamma, width, seed)
    mu_th = 1.0 / abs((1 - kappa_star) ** 2 - gamma ** 2)
    dx = 1.0 / math.sqrt(rays_per_pixel / (mu_th * (width / N) ** 2))
    nrx, nry = int(2 * l1 / dx) + 1, int(2 * l2 / dx) + 1
    lz = np.ascontiguousarray(lenses.astype(np.float32).ravel())
    counts = np.zeros(N * N, np.int32)
    total = nrx * nry
    threads = threads or os.cpu_count() or 1
    parts = max(threads * 8, 1)
    bounds = [total * i // parts for i in range(parts + 1)]
    L = lib()

    def run(i):
        L.orc_rayshoot(lz, len(lenses), 0.0, gamma, -l1, -l2, dx, nrx, nry, width, N, bounds[i], bounds[i + 1],
                       counts)

    with cf.ThreadPoolExecutor(threads) as ex:
        list(ex.map(run, range(parts)))
    counts = counts.reshape(N, N)
    avgN = float(counts.mean())
    return counts, counts / avgN


# ----------------------------------------------------------------------------- the reference's CUDA build

_refc = None


def refcuda_available() -> bool:
    """The reference's CUDA sources are staged beside the repository (baseline/_ref)."""
    return os.path.isdir(os.path.join(REFCUDA_DIR, "microlc", "src"))


def refcuda_build_async():
    """Start compiling the reference's CUDA path (where its sources are staged) in the
    background and return the process, else None; refcuda() waits for the same make."""
    if not refcuda_available():
        return None
    return subprocess.Popen(["make", "-s", "-f", REFCUDA_MK, "-j8"], stdout=subprocess.DEVNULL)


def refcuda():
    """The reference's own CUDA path (expanding_source, setup_integral_GPU, calculate_chi2_GPU,
    bin_chi2_GPU) built unchanged for sm_103a by oracle/refcuda.mk (compiled on first use),
    behind the C entry points of oracle/ref_cuda_harness.cu; None when its sources are not
    staged.  Runs on the GPU: only -m gpu tests and bench.py's GPU leg call it."""
    global _refc
    if _refc is None:
        if not refcuda_available():
            return None
        subprocess.check_call(["make", "-s", "-f", REFCUDA_MK, "-j8"], stdout=subprocess.DEVNULL)
        L = C.CDLL(REFCUDA_PATH)
        L.refc_expanding_source.argtypes = [_dp, C.c_int, C.c_int, C.c_double, C.c_double, _dp, C.c_int, C.c_char_p,
                                            C.c_int, _ip, _ip, _dp, _dp, _dp, C.c_int]
        L.refc_pair_path.argtypes = [C.c_int, C.c_int, _dp, _dp, _dp, _dp, C.c_int, _ip, _ip, _dp, _dp, _dp, _dp,
                                     C.c_int, _dp, C.c_void_p, _up, _up, _dp, _dp, _dp, C.c_int]
        _refc = L
    return _refc


def refcuda_expanding_source(mp, sizes, shape, lx, ly, pix_phys, width):
    """expanding_source of the reference's CUDA build on a 10000 x 10000 FP64 map (the only
    size its fixed multiply grid covers): (LC, DLC, ms)."""
    L = refcuda()
    mp = np.ascontiguousarray(mp, np.float64)
    Ny, Nx = mp.shape
    sizes = np.ascontiguousarray(sizes, np.float64)
    lx = np.ascontiguousarray(lx, np.int32); ly = np.ascontiguousarray(ly, np.int32)
    Nloc, Nprof = lx.size, sizes.size
    LC = np.zeros(Nloc * Nprof); DLC = np.zeros(max(Nloc * (Nprof - 1), 1)); ms = np.zeros(1)
    st = L.refc_expanding_source(mp, Nx, Ny, width, pix_phys, sizes, Nprof, shape.encode(), Nloc, lx, ly, LC, DLC, ms,
                                 1)
    if st != 0:
        raise RuntimeError(f"refc_expanding_source: status {st}")
    return LC.reshape(Nloc, Nprof), DLC[: Nloc * (Nprof - 1)].reshape(Nloc, Nprof - 1), float(ms[0])


def refcuda_pair_path(LCA, DLCA, LCB, DLCB, v, edges, want_rank=True):
    """setup_integral_GPU + calculate_chi2_GPU + bin_chi2_GPU of the reference's CUDA build:
    dict(rank, lower, nper, bchi2, bexp, ms=[setup, chi2, bin])."""
    L = refcuda()
    f = lambda a: np.ascontiguousarray(a, np.float64)
    LCA, DLCA, LCB, DLCB = f(LCA), f(DLCA), f(LCB), f(DLCB)
    Nloc, Nprof = LCA.shape
    edges = f(edges)
    nb = edges.size
    rank = np.zeros(Nloc * Nloc, np.uint32) if want_rank else None
    lower = np.zeros(nb, np.uint32); nper = np.zeros(nb, np.uint32)
    bc = np.zeros(nb); be = np.zeros(nb); ms = np.zeros(3)
    st = L.refc_pair_path(Nloc, Nprof, LCA, DLCA, LCB, DLCB, int(v["Njp"]), np.ascontiguousarray(v["indA"], np.int32),
                          np.ascontiguousarray(v["indB"], np.int32), f(v["facA"]), f(v["facB"]), f(v["d"]), f(v["s"]),
                          nb, edges, rank.ctypes.data_as(C.c_void_p) if want_rank else None, lower, nper, bc, be, ms, 1)
    if st != 0:
        raise RuntimeError(f"refc_pair_path: status {st}")
    return dict(rank=rank, lower=lower, nper=nper, bchi2=bc, bexp=be, ms=[float(x) for x in ms])
