"""microsn_gb300 -- GB300-native light-curve hot path of microLC (gvernard/microSN).

FFT convolution of magnification maps with source profiles, light-curve sampling
(fixed locations and straight tracks) and the chi-squared stage (single target,
pairwise, sort and binning), as hand-written sm_103a CUDA kernels behind the C ABI in
include/microlc_gb300.h.  This package is the Python host mirror of that ABI.
"""
from .api import (Chi2Vars, Context, Map, bin_chi2, bin_edges, calculate_chi2, chi2_offset, convolve, convolve_direct,
                  expanding_source, histogram_f64, interleave_maps, locations_grid, locations_random, pair_bin_fused, profile,
                  profile_raster, read_gerlumph, sample_tracks, sample_tracks_interleaved, setup_chi2_calculation, setup_integral,
                  sort_f64_u32, trapezium)
from .api import PairSide, pair_chi2_magdiff, pair_chi2_magdiff_list, pair_chi2_sides  # noqa: F401
from .api import convolve_sample_tracks, map_binned_mpd, mpd_divide, mpd_normalize  # noqa: F401
from .api import flux_ratio_chi2, track_chi2_offset  # noqa: F401
from .api import convolve_many, sample_expanding  # noqa: F401
from .api import FIT_PARAMS, TrackChi2, fit_raster, radius_stack, track_chi2, track_fit  # noqa: F401
from .api import host_empty, selftest_wait_timeout  # noqa: F401
from ._lib import MlcError

__all__ = [
    "Chi2Vars", "Context", "Map", "MlcError", "bin_chi2", "bin_edges", "calculate_chi2", "chi2_offset", "convolve", "convolve_direct",
    "convolve_sample_tracks", "PairSide", "pair_chi2_sides", "pair_chi2_magdiff", "pair_chi2_magdiff_list", "map_binned_mpd", "mpd_divide",
    "mpd_normalize", "flux_ratio_chi2", "track_chi2_offset", "convolve_many", "sample_expanding", "FIT_PARAMS", "TrackChi2", "fit_raster", "radius_stack", "track_chi2",
    "track_fit",
    "expanding_source", "histogram_f64", "locations_grid", "locations_random", "pair_bin_fused", "profile",
    "profile_raster", "read_gerlumph", "sample_tracks", "sample_tracks_interleaved", "interleave_maps", "setup_chi2_calculation", "setup_integral", "sort_f64_u32",
    "trapezium", "selftest_wait_timeout", "host_empty",
]
