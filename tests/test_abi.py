"""The C-ABI library loads and exports every symbol include/*.h declares; host-side
stages (C++, no GPU needed) match the oracle / reference golden vectors."""
import glob
import os
import re

import numpy as np
import pytest

import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(mlc_\w+)\s*\(", src, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_library_exports_every_declared_symbol(lib_built):
    from microsn_gb300 import _lib
    L = _lib.load()
    names = declared_symbols()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert set(names) <= set(_lib.SIGNATURES), set(names) - set(_lib.SIGNATURES)
    assert L.mlc_version() >= 100


def test_profile_raster_host_matches_oracle(lib_built):
    import microsn_gb300 as mlc
    for shape in ["uniform", "gaussian", "gaussian_hole", "thermal_hole", "wavy", "exponential", "limb_darkened"]:
        for rc in (True, False):
            kw = dict(Rin=0.01) if shape == "gaussian_hole" else {}
            if shape == "wavy":
                kw = dict(a=1.3)
            if shape == "limb_darkened":
                kw = dict(u=0.6)
            p = mlc.profile(shape, 0.05, 0.0025, ref_compat=rc, **kw)
            a = mlc.profile_raster(p)
            b = oracle.profile(shape, 0.05, 0.0025, ref_compat=rc, **kw)
            assert np.array_equal(a, b), (shape, rc)


def test_profile_raster_matches_reference_golden(lib_built, golden):
    import microsn_gb300 as mlc
    cases = [str(c).split("|") for c in golden["profile_cases"]]
    for i, (shape, rhalf, pix) in enumerate(cases):
        a = mlc.profile_raster(mlc.profile(shape, float(rhalf), float(pix)))
        assert np.array_equal(a, golden[f"profile_{i}"]), (shape, rhalf, pix)


def test_setup_chi2_host_matches_golden(lib_built, golden):
    import microsn_gb300 as mlc
    d, s, sizes, Dfac = golden["setup_d"], golden["setup_s"], golden["setup_sizes"], float(golden["setup_Dfac"])
    for i in range(4):
        g = {k[len(f"setup{i}_"):]: golden[k] for k in golden.files if k.startswith(f"setup{i}_")}
        v = mlc.setup_chi2_calculation((float(g["M0"]), float(g["M1"])), (float(g["V0"]),), Dfac, d, g["t"], s,
                                       sizes)
        assert v.Njp == int(g["Njp"])
        assert np.array_equal(v.indA, g["indA"]) and np.array_equal(v.facA, g["facA"])
        assert np.array_equal(v.indB, g["indB"]) and np.array_equal(v.facB, g["facB"])
        assert v.const_term == float(g["const"])


def test_locations_edges_trapezium_host(lib_built, golden):
    import microsn_gb300 as mlc
    x, y = mlc.locations_grid(7, 1000, 13)
    assert np.array_equal(x, golden["loc_grid_x"]) and np.array_equal(y, golden["loc_grid_y"])
    x, y = mlc.locations_random(50, 1000, 13, 5)
    assert np.array_equal(x, golden["loc_rand_x"]) and np.array_equal(y, golden["loc_rand_y"])
    np.testing.assert_array_equal(mlc.bin_edges(300, 1e-4, 300, True), golden["mpd_edges_log"])
    np.testing.assert_array_equal(mlc.bin_edges(17, 0.5, 9.0, False), golden["mpd_edges_lin"])
    assert mlc.trapezium(golden["trap_f1"], golden["trap_f2"], golden["trap_x"]) == float(golden["trap_val"])


def test_gerlumph_reader_roundtrip(lib_built, tmp_path):
    import microsn_gb300 as mlc
    from microsn_gb300 import synth
    mp, counts, meta = synth.rayshoot_numpy(32, 4.0, 0.4, 0.4, seed=1, rays_per_pixel=4)
    synth.write_gerlumph(str(tmp_path / "m"), counts, meta)
    got, width, m6 = mlc.read_gerlumph(str(tmp_path / "m"))
    np.testing.assert_array_equal(got, synth.counts_to_map(counts, meta))
    assert width == 4.0
    if oracle.ref_available():
        import ctypes as C
        R = oracle.ref()
        n = C.c_int(); w = C.c_double(); px = C.c_double()
        buf = np.zeros(32 * 32)
        R.ref_read_map(str(tmp_path / "m").encode(), 1.0, C.byref(n), C.byref(w), C.byref(px),
                       buf.ctypes.data_as(C.c_void_p), buf.size)
        np.testing.assert_array_equal(got.ravel(), buf)


def test_errors_are_status_codes(lib_built):
    import microsn_gb300 as mlc
    with pytest.raises(mlc.MlcError):
        mlc.profile_raster(mlc.profile("gaussian", -1.0, 0.01))
    with pytest.raises(mlc.MlcError):
        mlc.bin_edges(0, 1, 2)


def test_host_alloc_argument_errors(lib_built):
    """mlc_host_alloc / mlc_host_free argument handling (no GPU needed): zero bytes and a null
    out-pointer are refused, NULL frees as a no-op, an unknown pointer is refused."""
    import ctypes
    from microsn_gb300 import _lib
    L = _lib.load()
    p = ctypes.c_void_p()
    assert L.mlc_host_alloc(0, ctypes.byref(p)) == 1 and not p.value  # MLC_ERR_ARG
    assert L.mlc_host_alloc(4096, None) == 1
    assert L.mlc_host_free(None) == 0
    buf = ctypes.create_string_buffer(64)
    assert L.mlc_host_free(ctypes.cast(buf, ctypes.c_void_p)) == 1  # not from mlc_host_alloc
