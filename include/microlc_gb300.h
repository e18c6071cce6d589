/*
 * microlc_gb300.h -- C ABI of the GB300-native microLC light-curve hot path.
 *
 * The reference (gvernard/microSN, package microLC) exposes this path as C++ free
 * functions over host structs that own device buffers
 * (simulating_lcurves/include/gpu_functions.hpp:11-18, cpu_functions.hpp:12-15,
 * chi2/chi2_functions.cuh:93).  This header replaces them with plain-pointer C entry
 * points that a cgo / ctypes / C++ caller can bind; the header-only C++ layer
 * include/microlc_compat.hpp rebuilds the reference's own classes and signatures on top.
 *
 * Conventions
 *  - Every entry returns an int status: MLC_OK (0) or one of MLC_ERR_*; the text of
 *    the last failure is available from mlc_ctx_last_error().
 *  - Array arguments are DEVICE pointers unless their name ends in _host.  Device
 *    pointers are borrowed: the library never frees them.
 *  - Work is queued on the context's stream; entries that return host results
 *    synchronise that stream before returning.
 *  - A context is used by one host thread at a time.
 *  - The library is built for sm_103a only and fails with MLC_ERR_CUDA elsewhere.
 */
#ifndef MICROLC_GB300_H
#define MICROLC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define MLC_OK 0
#define MLC_ERR_ARG 1         /* bad argument (null, size, unsupported length) */
#define MLC_ERR_OOM 2         /* device or host allocation failed */
#define MLC_ERR_CUDA 3        /* CUDA runtime / launch failure */
#define MLC_ERR_TIMEOUT 4     /* a bounded device-side wait gave up */
#define MLC_ERR_UNSUPPORTED 5 /* valid request the library does not implement */
#define MLC_ERR_LIMIT 6       /* size beyond a documented limit */

/* ---- precisions ---- */
#define MLC_F64 0
#define MLC_F32 1

/* ---- profile shapes (profile.hpp:112-170 factory keys, plus limb_darkened) ---- */
#define MLC_SHAPE_UNIFORM 0       /* "uniform"       profile.cpp:185-222 */
#define MLC_SHAPE_GAUSSIAN 1      /* "gaussian"      profile.cpp:228-263 */
#define MLC_SHAPE_GAUSSIAN_HOLE 2 /* "gaussian_hole" profile.cpp:269-311 */
#define MLC_SHAPE_THERMAL_HOLE 3  /* "thermal_hole"  profile.cpp:315-354 */
#define MLC_SHAPE_WAVY 4          /* "wavy"          profile.cpp:358-398 */
#define MLC_SHAPE_EXPONENTIAL 5   /* "exponential" (thin disc) profile.cpp:402-446 */
#define MLC_SHAPE_LIMB_DARKENED 6 /* linear limb-darkened disc (no reference counterpart) */

/* ---- convolution modes ---- */
#define MLC_CONV_FUSED 0 /* profile spectrum generated from the small raster, multiply fused */
#define MLC_CONV_PLAIN 1 /* full-size wrapped kernel, forward FFT, multiply, inverse: one launch per stage */

typedef struct mlc_ctx mlc_ctx;
typedef struct mlc_map mlc_map;

/* Source profile description.  Physical units are those of pix (the reference uses
 * 10^14 cm; any consistent unit works).  ref_compat = 1 passes rhalf, pix, incl, orient,
 * Rin and a through the reference's std::to_string / std::stof round trip
 * (gpu_functions.cu:108,184) and keeps its exponential-core overwrite
 * (profile.cpp:435-441), so rasters are bit-identical to the reference's. */
typedef struct {
  int shape;
  int ref_compat;
  double rhalf;  /* half-light radius */
  double pix;    /* pixel size */
  double incl;   /* degrees */
  double orient; /* degrees */
  double Rin;    /* gaussian_hole inner radius */
  double a;      /* wavy amplitude */
  double u;      /* limb-darkening coefficient */
} mlc_profile;

/* ======================================================================= context */

/* New context on `device`, queueing work on `stream` (a cudaStream_t; NULL = the
 * legacy default stream).  No reference counterpart: the reference uses the default
 * stream and global __constant__ state (gpu_functions.cu:25-33). */
int mlc_ctx_create(int device, void* stream, mlc_ctx** out);
int mlc_ctx_destroy(mlc_ctx* ctx);
int mlc_ctx_set_stream(mlc_ctx* ctx, void* stream);
int mlc_ctx_synchronize(mlc_ctx* ctx);
const char* mlc_ctx_last_error(const mlc_ctx* ctx);
/* Bytes of device workspace the context currently holds (grow-only pool). */
size_t mlc_ctx_workspace_bytes(const mlc_ctx* ctx);
/* Library version (major*10000 + minor*100 + patch). */
int mlc_version(void);
/* Number of kernels this context has launched so far. */
unsigned long long mlc_ctx_launch_count(const mlc_ctx* ctx);
/* Per-kernel CUDA-event timing on the context's stream (off by default).  Turning it
 * on brackets every launch with events; mlc_ctx_kernel_times synchronises, then writes
 * up to cap entries of (name, total milliseconds, launches) -- names as a
 * '\n'-separated list into names_host (size name_cap) -- and returns the entry count
 * (or a negative status).  reset != 0 clears the totals afterwards. */
int mlc_ctx_set_timing(mlc_ctx* ctx, int on);

/* Launch autotuner (on by default; no reference counterpart).  For each new (map size,
 * profile size) of an FP32 fused convolution the first call times the FFT form against
 * the direct tiled form's tile shapes (mlc_convolve_direct) on the context's stream and
 * keeps the fastest; likewise the fused convolution's P1 variant per map size and
 * arithmetic, the pair kernel's epilogue width per shape class and the track sampler's
 * order (track or map cell) for large calls.  Later calls reuse the
 * choice.  Tuning synchronises the stream once
 * per key and is skipped while the stream is captured into a CUDA graph.  Off: the FFT
 * form everywhere (results then do not depend on timings).  The report lists every tuned
 * key, its choice and the candidates' times: NUL-terminated text into buf (cap bytes);
 * returns the text length, or a negative status. */
int mlc_ctx_set_autotune(mlc_ctx* ctx, int on);
int mlc_ctx_autotune_report(mlc_ctx* ctx, char* buf, int cap);

/* Pins the autotuner's choice for one key (as the report prints it; used whether or not
 * the autotuner is on), e.g. to compare variants or to fix a run's kernels:
 *   "conv f32 <Nx>x<Ny> N<pN>[ spectrum]": -1 FFT form, 0..3 direct tile shape;
 *   "conv P1 <arithmetic> <Nx>x<Ny>[ two-chain]": 0 map spectrum prefetched into L2, 1
 *     staged in shared memory (float-float and FP64 transforms); " two-chain" is the
 *     batched step's key, where the second convolution chain runs alongside (not timed:
 *     0 unless pinned);
 *   "pairdiff_tc K<64|128>[ matrix] bins<1024|4096> pairs~4^<k>": epilogue warps 12, 16
 *     or 24;
 *   "sample_tracks_il order <Nx>x<Ny> <f32|f64> x<stride> epochs~2^<k>": the track sampler
 *     in track order (0) or in map-cell order (1); "sample_tracks_il cell-order" pins it for
 *     every size.
 * Other values fall back to the default. */
int mlc_ctx_tune_set(mlc_ctx* ctx, const char* key, int choice);

/* Cached profile spectra (no reference counterpart; the reference transforms the full-size
 * kernel of every profile for every map, gpu_functions.cu:183-201).  mlc_convolve_sample_tracks
 * and mlc_convolve_many keep the spectra of their last profile list -- each profile's
 * spectrum as the fused convolution holds it before the product with the map spectrum --
 * and reuse them while the list, the map size and the transform arithmetic repeat: a
 * convolution then skips the profile's transform (P0 and the forward half of P1; the same
 * operations on the same values otherwise, so the same results bit for bit).  They take
 * nprof x (Ny x (Nx/2+1) complex) of the map's transform arithmetic: 800 MB per profile at
 * 10000^2 in float-float.  max_bytes: -1 (default) a quarter of the device memory, 0 never
 * cache, else the limit; lists that do not fit are convolved without the cache.  Map sizes
 * whose column split has N2 = 100 or 128 (e.g. 2000^2 ... 10000^2, 8192^2). */
int mlc_ctx_set_profile_cache(mlc_ctx* ctx, long long max_bytes);
int mlc_ctx_kernel_times(mlc_ctx* ctx, char* names_host, int name_cap, double* ms_host, long* launches_host,
                         int cap, int reset);

/* ======================================================================= profiles (host) */

/* Side length N of the N x N raster (profile.cpp:197, 241, 285, 329, 373, 415). */
int mlc_profile_dims(const mlc_profile* p, int* N);
/* Normalised N x N raster into out_host (capacity cap doubles), FP64 on the host,
 * replacing FactoryProfile::createProfileFromHalfRadius (profile.hpp:142-166). */
int mlc_profile_raster(const mlc_profile* p, double* out_host, long cap, int* N);

/* ======================================================================= maps */

/* A map resident on the device in `precision` (MLC_F64 / MLC_F32), Ny rows of Nx
 * pixels, row-major (the layout of MagnificationMap::data, magnification_map.cpp:33-38).
 * `data` is FP64 (data_dtype MLC_F64) or FP32 (MLC_F32), on the device if data_is_device
 * else on the host.  Nx and Ny must be even and factor into 2, 3 and 5. */
int mlc_map_create(mlc_ctx* ctx, const void* data, int data_is_device, int data_dtype, int Nx, int Ny,
                   int precision, mlc_map** out);
/* Frees the map's device memory (waits for the device); valid after its context was destroyed. */
int mlc_map_destroy(mlc_map* map);
/* Device pointer to the map's pixels (precision of the map). */
int mlc_map_data(mlc_map* map, void** dev_ptr);
/* Forward spectrum of the map (computed once and cached), replacing the
 * cufftExecD2Z of the map (gpu_functions.cu:171-176). */
int mlc_map_prepare(mlc_ctx* ctx, mlc_map* map);
/* Recompute the cached spectrum from the map's current pixels (after they were
 * rewritten through mlc_map_data). */
int mlc_map_refresh(mlc_ctx* ctx, mlc_map* map);

/* Arithmetic of a map's Fourier transforms (no reference counterpart).  With
 * MLC_FFT_F32X2 the map's forward transform and its fused convolutions run in float-float
 * arithmetic (pairs of FP32 values, about 48 significant bits) while pixels, convolved
 * maps, light curves and everything after them keep the map's precision.
 *  - FP64 maps: GB300 runs FP64 at a small fraction of its FP32 rate; float-float
 *    transforms give convolved maps within about 1e-13 relative of FP64 transforms.
 *  - FP32 maps: FP32 transforms carry an absolute error of a few 1e-7 of the map's rms,
 *    which is up to ~1e-5 relative in the faint pixels of a ray-shot map and moves the
 *    offset-minimised chi2 of a light curve by up to ~3e-4 relative; float-float transforms
 *    leave only the FP32 rounding of the convolved pixels (about 1e-7 relative).  The
 *    spectrum takes 16 bytes per complex value instead of 8.
 * The plain form (MLC_CONV_PLAIN) keeps the map's own precision and refuses such a map;
 * the direct tiled form is not used for it.  Changing the mode drops the cached spectrum. */
#define MLC_FFT_NATIVE 0
#define MLC_FFT_F32X2 1
int mlc_map_set_fft(mlc_map* map, int mode);

/* ======================================================================= convolution */

/* Convolve the map with one profile into out (Ny x Nx, the map's precision), the
 * per-profile body of expanding_source (gpu_functions.cu:183-201): kernel wrap
 * (magnification_map.cpp:172-193), forward transform, multiply / (Nx Ny)
 * (kernel_multiplyFFTs :571-577) and inverse transform, with hand-written FFTs. */
int mlc_convolve(mlc_ctx* ctx, mlc_map* map, const mlc_profile* prof, int mode, void* out);

/* The direct tiled convolution (no FFT) of an FP32 map with a profile of 2..32 pixels,
 * tile shape variant 0..3 (4x4, 4x8, 8x4, 8x8 outputs per thread): the same circular
 * convolution with the reference's kernel wrap as mlc_convolve (Kernel::setKernel,
 * magnification_map.cpp:172-193).  No reference counterpart. */
int mlc_convolve_direct(mlc_ctx* ctx, mlc_map* map, const mlc_profile* prof, int variant, void* out);

/* Replaces expanding_source (gpu_functions.cu:82-225) for an FP64 map: LC (Nloc x Nprof)
 * and DLC (Nloc x (Nprof-1)), location-major like SimLC (data_structs.hpp:50-63).
 * sizes_host[k] are half-light radii in Einstein radii (sizes_host[0] must be 0, the
 * point source); the profile for k >= 1 has rhalf = sizes_host[k] * base->pix * Nx / width
 * and base's other fields.  loc_x, loc_y: Nloc int pixel indices.  mode: MLC_CONV_*. */
int mlc_expanding_source(mlc_ctx* ctx, mlc_map* map, const double* sizes_host, int Nprof,
                         const mlc_profile* base, double width, int Nloc, const int* loc_x,
                         const int* loc_y, int mode, double* LC, double* DLC);

/* ======================================================================= sampling */

/* kernel_sample (gpu_functions.cu:604-620): LC[id*Nprof+k] = map[loc_y*Nx+loc_x] and,
 * for k > 0, DLC[id*(Nprof-1)+k-1] = LC[id*Nprof+k] - LC[id*Nprof+k-1]. FP64 map of
 * Ny x Nx; a location outside the map yields NaN instead of an out-of-range read. */
int mlc_sample_nearest(mlc_ctx* ctx, const double* map, int Nx, int Ny, int k, int Nprof, int Nloc,
                       const int* loc_x, const int* loc_y, double* LC, double* DLC);

/* Straight source tracks (no reference counterpart; bilinear formula of
 * RectGrid::interp2d_bilinear, rectGrid.cpp:349-378, pixel centres at j + 1/2).
 * Track k is at (x0 + v t cos phi, y0 + v t sin phi) pixels at each of its epoch times
 * t[off[k] .. off[k+1]).  `maps` holds nmaps device pointers to Ny x Nx maps of
 * `precision`; x0, y0, phi, v, t are in that precision; off is int64 (ntracks+1).
 * out[m * E + e] (E = off[ntracks]) is -2.5 log10(mu) when mag != 0, else mu.
 * A position outside the hull of pixel centres samples 0 (magnitude +inf). */
int mlc_sample_tracks(mlc_ctx* ctx, const void* const* maps_host, int nmaps, int Nx, int Ny, int precision,
                      int ntracks, const void* x0, const void* y0, const void* phi, const void* v,
                      const int64_t* off, const void* t, int mag, void* out);

/* Interleave nmaps (<= 16) maps of Ny x Nx pixels pixel by pixel: out[(y*Nx+x)*stride + q]
 * (stride a power of two >= nmaps, slots q >= nmaps zeroed).  The layout the interleaved
 * sampler reads: one contiguous 4*stride-byte (FP32) read per bilinear corner. */
int mlc_interleave_maps(mlc_ctx* ctx, const void* const* maps_host, int nmaps, int Nx, int Ny, int precision,
                        int stride, void* out);

/* mlc_sample_tracks on an interleaved map (mlc_interleave_maps): same tracks, same
 * arithmetic and output layout out[q*E + e] for q < nmaps. */
int mlc_sample_tracks_interleaved(mlc_ctx* ctx, const void* imap, int stride, int nmaps, int Nx, int Ny,
                                  int precision, int ntracks, const void* x0, const void* y0, const void* phi,
                                  const void* v, const int64_t* off, const void* t, int mag, void* out);

/* ======================================================================= whole step, one call */

/* Straight tracks as in mlc_sample_tracks: start x0, y0 (pixels), angle phi (radians),
 * speed v (pixels per day), epoch offsets off[ntracks + 1] (off[0] = 0) and epochs
 * t[nepochs] (days, nepochs = off[ntracks]).  x0, y0, phi, v and t have the map's
 * precision. */
typedef struct {
  int ntracks;
  int64_t nepochs;
  const void* x0;
  const void* y0;
  const void* phi;
  const void* v;
  const int64_t* off;
  const void* t;
} mlc_tracks;

#define MLC_IO_HOST 1 /* pixels, the track arrays and out are host memory */
#define MLC_ASYNC 2   /* return once queued (see below) */
#define MLC_GRAPH 4   /* capture / replay the call's kernel sequence as a CUDA graph (device buffers) */

/* The light-curve step of one lensed image in one call -- expanding_source
 * (gpu_functions.cu:82-225) with straight tracks in place of fixed locations:
 *   pixels (Ny x Nx, the map's precision; NULL keeps the map's current pixels and cached
 *   spectrum) -> forward spectrum -> convolution with each of the nprof profiles
 *   (mode MLC_CONV_*) -> bilinear sampling of every track at its epochs ->
 *   out[q * nepochs + e] (q < nprof), magnitudes -2.5 log10(mu) when mag != 0.
 * Without MLC_IO_HOST every array is device memory and everything runs on the context's
 * stream.  With MLC_IO_HOST the uploads run on an internal host-to-device stream and the
 * light curves come back in chunks of tracks on an internal device-to-host stream, each
 * chunk's copy overlapping the sampling of the next; host buffers should be page-locked
 * (cudaHostAlloc / cudaHostRegister) for the copies to overlap.
 * With device buffers the call is stream-ordered (it returns once queued; out is ready in
 * the order of the context's stream, like every other device-buffer entry).  With
 * MLC_IO_HOST it returns when out holds the result, unless MLC_ASYNC is given: then it
 * returns once the work is queued, the caller keeps pixels, the tracks and out untouched
 * until mlc_ctx_synchronize (or mlc_ctx_join + a sync of its stream), and the next call's
 * uploads and convolutions overlap this call's copies back.  The profile rasters are
 * computed on host threads and uploaded once per profile list: a call with the same list
 * and map size as the previous call reuses them.  Device memory held: the
 * group's convolved maps and their interleaved copy (2 x min(nprof,16) maps), two track
 * buffers and an output ring of about twice one call's light curves (4 to 64 chunks).
 * MLC_GRAPH (device buffers only) runs the call eagerly the first time and then captures
 * the whole step -- forward spectrum (when pixels is given), both convolution chains, the
 * last passes, sampling -- into one CUDA graph on an internal stream; later calls with the
 * same map, pixel, track and output pointers, sizes, profile raster sizes and workspace
 * replay it with one launch on the context's stream.  The contents of pixels, the track
 * arrays and the profile values may change between calls; any other change recaptures.
 * Per-kernel timing (mlc_ctx_set_timing) runs the call eagerly instead. */
int mlc_convolve_sample_tracks(mlc_ctx* ctx, mlc_map* map, const void* pixels, int nprof,
                               const mlc_profile* profiles_host, const mlc_tracks* tracks, int mode,
                               int mag, void* out, int flags);

/* The map convolved with nprof profiles (mode MLC_CONV_*) into out + k*out_stride
 * elements (device, the map's precision): the profiles of an expanding source or of
 * several bands in one call, rasters staged and uploaded once.  With MLC_GRAPH the
 * kernel sequence is captured into a CUDA graph on its first call and replayed by later
 * calls with the same map, profile raster sizes and output (profile values may change).
 * No reference counterpart beyond the per-profile loop of expanding_source. */
int mlc_convolve_many(mlc_ctx* ctx, mlc_map* map, int nprof, const mlc_profile* profiles_host, int mode, void* out,
                      long long out_stride, int flags);

/* Expanding source (one profile per epoch, the supernova case; no reference counterpart):
 * the nep*nbands maps of the epochs and bands stored contiguously (map e*nbands + b starts
 * at maps + (e*nbands + b)*Nx*Ny, e.g. from mlc_convolve_many), ntracks straight tracks
 * (x0, y0, phi, v in the map's precision) sampled bilinearly at the shared epochs t[nep]:
 * out[i*nep*nbands + e*nbands + b], magnitudes when mag != 0 (rows are the curves the
 * pair stage takes, T = nep*nbands). */
int mlc_sample_expanding(mlc_ctx* ctx, const void* maps, int Nx, int Ny, int precision, int nep, int nbands,
                         int ntracks, const void* x0, const void* y0, const void* phi, const void* v, const void* t,
                         int mag, void* out);

/* Makes the context's stream wait (on the device, without blocking the host) for all
 * copies queued by MLC_IO_HOST calls, so that an event recorded on the stream afterwards
 * covers them. */
int mlc_ctx_join(mlc_ctx* ctx);

/* Bytes of one output chunk of MLC_IO_HOST calls (default 256 MiB; 4 to 64 chunks are held
 * on the device).  Smaller chunks start the download sooner; every track's light curves
 * (min(nprof,16) x its epochs) must fit in one.  Waits for the context's queued work. */
int mlc_ctx_set_chunk_bytes(mlc_ctx* ctx, size_t bytes);

/* ======================================================================= differentiable track fit */
/* No reference counterpart.  Gradients of the chi2 of model light curves with respect to
 * every track's parameters theta = (x0, y0, phi, v, R_half, dm), for gradient-based fits. */

#define MLC_FIT_MAX_RADII 32

/* Smooth thin-disc raster on a fixed N x N grid (N even): the thin-disc law of
 * profile.cpp:402-446, I = min(I_core, 1 / (exp((r/sigma)^(3/4)) - 1)), sigma = 0.4106
 * rhalf, without the truncation at 2 rhalf, normalised to unit sum, and the rasters of its
 * analytic derivatives at the same offsets: dP/dx and dP/dy per pixel of offset (x along
 * a row), dP/d(rhalf) with the normalisation included.  Derivative outputs may be NULL.
 * Host FP64. */
int mlc_fit_raster(double rhalf, double pix, int N, double* P_host, double* dPdx_host, double* dPdy_host,
                   double* dPdR_host);

/* Radius stack of a map for mlc_track_fit: for each radius radii_host[k] (K of them,
 * increasing, 2 <= K <= MLC_FIT_MAX_RADII, in the units of pix) the map convolved with
 * P(R_k), dP/dx, dP/dy and dP/dR (mlc_fit_raster, N x N) -- the values and first
 * derivatives of the continuous convolution at every pixel node -- interleaved per pixel
 * into stack (device, Ny*Nx*K*4 values of the map's precision):
 * stack[((y*Nx + x)*K + k)*4 + {0: M, 1: dM/dx, 2: dM/dy, 3: dM/dR}]. */
int mlc_radius_stack(mlc_ctx* ctx, mlc_map* map, int K, const double* radii_host, double pix, int N, void* stack);

/* chi2 of ntracks model curves and its gradient.  theta: ntracks x 6 (x0, y0 in pixels,
 * phi in radians, v in pixels per unit of t, R_half in the stack's radius units, dm in
 * magnitudes); off: ntracks+1 epoch offsets; t, obs, w: epochs, observed magnitudes and
 * weights (1/sigma^2).  Model: m(t) = -2.5 log10 M(x0 + v t cos phi, y0 + v t sin phi; R)
 * + dm, M the tensor-product cubic Hermite interpolant in (x, y, R) of the stack's node
 * values and derivatives (nodes at pixel centres j + 1/2; C1, so finite differences
 * converge to the gradient everywhere); chi2[i] = sum_e w (obs - m)^2; grad[i*6 + j] = dchi2_i/dtheta_ij (NULL to skip);
 * model[e] = m(t_e) (NULL to skip; NaN where the position leaves the map).  All arrays on
 * the device in `precision`.  Only queues one kernel: no allocation, no synchronisation,
 * so the call can be captured into a CUDA graph. */
int mlc_track_fit(mlc_ctx* ctx, const void* stack, int Nx, int Ny, int precision, int K, const double* radii_host,
                  int ntracks, const void* theta, const int64_t* off, const void* t, const void* obs, const void* w,
                  void* chi2, void* grad, void* model);

/* ======================================================================= multi-filter flux ratios */

/* getChi2GPU / getChi2CPU (chi2/chi2_functions.cuh:93-190): for every location pair
 * (x of image 1, y of image 2)
 *   chi2[x,y] = 1/2 sum_f sum_t ((f_obs[f,t] - mu1[x,f,t] / mu2[y,f,t]) / df_obs[f,t])^2
 * -- the CPU twin's indexing; the reference's kernel reads mu2 at x, so its chi2 ignores
 * y -- and *likelihood_host = sum over pairs of exp(-chi2), accumulated in FP64 in a
 * fixed order.  f_obs_host, df_obs_host: F*T floats (filter-major) on the host; mu1, mu2:
 * N*F*T device floats (location, filter, time).  chi2: device N*N floats stored as the
 * reference's chi2_all[y*N + x], or NULL to skip.  FP32 arithmetic per term. */
int mlc_flux_ratio_chi2(mlc_ctx* ctx, const float* f_obs_host, const float* df_obs_host, const float* mu1,
                        const float* mu2, int N, int F, int T, float* chi2, double* likelihood_host);

/* ======================================================================= map MPDs */

/* MagnificationMap::getBinnedMpd (magnification_map_gpu.cu:45-87) of the map's pixels,
 * in one pass instead of a sort of the whole map.  bins_host[i] = Mpd log edges
 * pow(10, log10(min) + (i+1) dl) (mpd.cpp:8-13); counts_host[i] = the fraction of the
 * Nx*Ny pixels v with min <= v < max and edge[i-1] < v <= edge[i] (a value above the last
 * edge is dropped), 1/(Nx*Ny) for an empty bin.  Exact for FP64 maps; an FP32 map is
 * binned by its FP32 values.  1 <= Nbins <= 16000. */
int mlc_map_binned_mpd(mlc_ctx* ctx, mlc_map* map, int Nbins, double min, double max, double* bins_host,
                       double* counts_host);

/* Mpd::divide_by (mpd.cpp:71-107), A.divide_by(B, R): for each ratio edge z = binsR[i],
 * countsR[i] = trapezium over B's bins of muB * pA(z muB) * pB(muB), pA interpolated
 * linearly between A's edges (1e-8 outside them).  Bit-identical to the reference's
 * host arithmetic. */
int mlc_mpd_divide(mlc_ctx* ctx, int NA, const double* binsA_host, const double* countsA_host, int NB,
                   const double* binsB_host, const double* countsB_host, int NR, const double* binsR_host,
                   double* countsR_host);

/* ======================================================================= chi2 vs one observed curve */

/* Fused sample -> magnitude -> offset-minimised chi2, no light curve written: for each of
 * ntracks straight tracks (x0, y0, phi, v as in mlc_sample_tracks) sampled at the shared
 * epochs t[Tn] on each of the nmaps maps of an interleaved map (mlc_interleave_maps,
 * stride a power of two <= 16; stride 1 is a plain map), m = -2.5 log10(mu) and
 *   dm = sum w (o - m) / sum w,  chi2 = sum w (o - m - dm)^2     (FP64 accumulation)
 * against the observed curve obs[Tn] with weights w[Tn] (FP64).  chi2[q*ntracks + i],
 * dm[q*ntracks + i] (dm may be NULL), FP64 device arrays.  A position outside the map makes
 * that chi2 +inf.  One kernel, no allocation or synchronisation.  No reference
 * counterpart (the reference has no offset solve). */
int mlc_track_chi2_offset(mlc_ctx* ctx, const void* imap, int stride, int nmaps, int Nx, int Ny, int precision,
                          int ntracks, const void* x0, const void* y0, const void* phi, const void* v, int Tn,
                          const void* t, const double* obs, const double* w, double* chi2, double* dm);


/* Offset-minimised chi2 of ncurves magnitude curves of T epochs (m, row-major, the
 * given precision) against one observed curve obs_host / weights w_host (FP64, T):
 * dm = sum w (o - m) / sum w (FP64), chi2 = sum w (o - m - dm)^2.  No reference
 * counterpart (the reference has no offset solve).  chi2, dm: FP64 device arrays. */
int mlc_chi2_offset(mlc_ctx* ctx, int precision, int ncurves, int T, const void* m,
                    const double* obs_host, const double* w_host, double* chi2, double* dm);

/* ======================================================================= pair stage (reference ratio form) */

/* setup_integral_GPU (gpu_functions.cu:351-401): z = LCA[a*Nprof]/LCB[b*Nprof] for all
 * Nloc^2 pairs; rank[a*Nloc+b] = position of that pair in the stable ascending order of
 * z (d_sorted_ind); lower_host / nper_host per right edge (edges_host, ascending) from
 * upper_bound, as Chi2SortBins::lower_ind / n_per_bin.  rank may be NULL (bins only). */
int mlc_pair_setup(mlc_ctx* ctx, int Nloc, int Nprof, const double* LCA, const double* LCB, int Nbins,
                   const double* edges_host, uint32_t* rank, uint32_t* lower_host, uint32_t* nper_host);

/* calculate_chi2_GPU (gpu_functions.cu:428-456, kernel_chi2 :700-750):
 * chi2 = sum_i ((d_i - mA_i/mB_i)/s_i)^2 with mA, mB interpolated on the profile axis
 * (index -1 gives 1), FP64, written to chi2[rank[a*Nloc+b]] (or chi2[a*Nloc+b] when rank
 * is NULL).  indA/indB/facA/facB/d/s are the Chi2Vars arrays (data_structs.hpp:4-18) on
 * the host, Njp entries (no limit of 50). */
int mlc_pair_chi2_ratio(mlc_ctx* ctx, int Njp, const int* indA_host, const int* indB_host,
                        const double* facA_host, const double* facB_host, const double* d_host,
                        const double* s_host, int Nloc, int Nprof, const double* LCA, const double* DLCA,
                        const double* LCB, const double* DLCB, const uint32_t* rank, double* chi2);

/* bin_chi2_GPU (gpu_functions.cu:483-503, kernel_bin_chi2 :772-795): per bin, mean of
 * chi2 and of exp(-chi2/2) over chi2_sorted[lower .. lower+n); empty bins give 2000 and
 * exp(-1000).  Results to the host arrays. */
int mlc_bin_chi2(mlc_ctx* ctx, int Nbins, const uint32_t* lower_host, const uint32_t* nper_host,
                 const double* chi2_sorted, double* binned_chi2_host, double* binned_exp_host);

/* The three calls above fused without the Nloc^2 arrays: each pair's z bin is found
 * from edges_host directly (bin i holds edge[i-1] < z <= edge[i], bin 0 everything
 * <= edge[0], z above the last edge is dropped) and its chi2 and exp(-chi2/2) are summed
 * per bin.  Same outputs as mlc_bin_chi2 plus the counts. */
int mlc_pair_bin_fused(mlc_ctx* ctx, int Njp, const int* indA_host, const int* indB_host,
                       const double* facA_host, const double* facB_host, const double* d_host,
                       const double* s_host, int Nloc, int Nprof, const double* LCA, const double* DLCA,
                       const double* LCB, const double* DLCB, int Nbins, const double* edges_host,
                       double* binned_chi2_host, double* binned_exp_host, uint32_t* nper_host);

/* ======================================================================= pair stage (magnitude-difference form) */

#define MLC_PAIR_PLAIN 0  /* FP64 on CUDA cores, one launch per stage (chi2 chunk, histogram, candidates) */
#define MLC_PAIR_TENSOR 1 /* exact sliced-integer cross term on the tensor cores, fused epilogue */

typedef struct {
  double delta;        /* quantisation step of the centred, weighted curves (tensor form) */
  double threshold;    /* top-k candidate threshold used */
  long long refined;   /* near-identical pairs recomputed in FP64 (tensor form) */
  long long candidates;
  int passes;          /* passes over the pairs (1 unless the threshold had to move) */
  long long below;     /* pairs whose chi2 lies below 10^lo_log10 (zero included): not in hist */
  long long above;     /* pairs whose chi2 lies at or above 10^hi_log10: not in hist */
} mlc_pair_stats;

/* Pairwise magnitude-difference chi2 between NA curves A and NB curves B (device FP32,
 * row-major, T epochs shared by all curves):
 *     chi2_ij = sum_t w_t (d_t - (A_it - B_jt) - c_ij)^2,
 * c_ij = 0, or with offset != 0 the constant magnitude offset that minimises it.
 * w_host: T weights (1/sigma^2); d_host: T observed difference (nullable = 0).  Outputs:
 * hist_host (nbins uint64 counts of log10 chi2 in [lo_log10, hi_log10), nbins <= 4096),
 * the k smallest chi2 with their (i, j) (ascending, ties by i*NB+j; k = 0 skips), and,
 * when chi2_out is not NULL, the NA x NB FP32 chi2 matrix (device).  No reference
 * counterpart: the reference's pair statistic is the flux ratio (kernel_chi2,
 * gpu_functions.cu:700-750; chi2/chi2_functions.cuh:35-68); this is its magnitude form.
 * MLC_PAIR_TENSOR needs T <= 128; its chi2 values are those of the curves quantised to
 * 24 bits (relative error ~1e-6 against FP64). */
int mlc_pair_chi2_magdiff(mlc_ctx* ctx, int method, int NA, int NB, int T, const float* A, const float* B,
                          const double* w_host, const double* d_host, int offset, int nbins, double lo_log10,
                          double hi_log10, uint64_t* hist_host, int k, double* topk_val_host, int64_t* topk_i_host,
                          int64_t* topk_j_host, float* chi2_out, mlc_pair_stats* stats);

/* FP64 chi2 of npairs listed pairs (ia, ib device int64), same statistic. */
int mlc_pair_chi2_magdiff_list(mlc_ctx* ctx, int NA, int NB, int T, const float* A, const float* B,
                               const double* w_host, const double* d_host, int offset, long npairs,
                               const int64_t* ia, const int64_t* ib, double* chi2);

/* Pair sides: one image's curves made ready for the tensor-core pair stage once (centred,
 * weighted, quantised to sliced integers, with norms and steps) and then paired with any
 * number of other sides, so that an image taking part in many pairs is prepared once and
 * an expanding source's curves need never be stored.  No reference counterpart: the
 * reference stores each image's light curves (expanding_source, gpu_functions.cu:82-225)
 * and reads both sets for every pair in kernel_chi2 (gpu_functions.cu:700-750).
 * A side owns one device allocation, made when it is built and freed by
 * mlc_pair_side_destroy.  The statistic is that of mlc_pair_chi2_magdiff with the same
 * w and offset; d_host (nullable) enters the side used as B.  T <= 128. */
typedef struct mlc_pair_side mlc_pair_side;

/* A side from N FP32 curves X (device, N x T row-major). */
int mlc_pair_side_curves(mlc_ctx* ctx, int N, int T, const float* X, const double* w_host, const double* d_host,
                         int offset, mlc_pair_side** side);

/* A side straight from an expanding source's convolved FP32 maps (layout as in
 * mlc_sample_expanding; track arrays FP32): curve r is the magnitudes of track r at the nep
 * shared epochs t, band-minor (T = nep*nbands), sampled, converted, centred and weighted in
 * one pass -- the values mlc_sample_expanding with mag != 0 followed by mlc_pair_side_curves
 * give, bit for bit, without the N x T light curves in memory. */
int mlc_pair_side_expanding(mlc_ctx* ctx, const float* maps, int Nx, int Ny, int nep, int nbands, int ntracks,
                            const float* x0, const float* y0, const float* phi, const float* v, const float* t,
                            const double* w_host, const double* d_host, int offset, mlc_pair_side** side);

int mlc_pair_side_destroy(mlc_pair_side* side);

/* mlc_pair_chi2_magdiff (MLC_PAIR_TENSOR) between two sides built with the same T, w and
 * offset; A must have been built without d.  Same outputs and statistics. */
int mlc_pair_chi2_sides(mlc_ctx* ctx, const mlc_pair_side* A, const mlc_pair_side* B, int nbins, double lo_log10,
                        double hi_log10, uint64_t* hist_host, int k, double* topk_val_host, int64_t* topk_i_host,
                        int64_t* topk_j_host, float* chi2_out, mlc_pair_stats* stats);

/* ======================================================================= sort / histogram */

/* Stable ascending sort of n FP64 keys (in place) carrying uint32 values (in place);
 * hand-written LSD radix sort.  keys and vals are device arrays of n. */
int mlc_sort_f64_u32(mlc_ctx* ctx, long n, double* keys, uint32_t* vals);

/* Histogram of n FP64 values (device) into nbins equal bins on [lo, hi) of the value,
 * or of log10(value) when logscale != 0; values outside are not counted.  counts_host
 * receives nbins uint64 counts. */
int mlc_histogram_f64(mlc_ctx* ctx, long n, const double* v, int nbins, double lo, double hi, int logscale,
                      uint64_t* counts_host);

/* The histogram above without any device allocation.  No counterpart in the reference
 * (its binning allocates with thrust on every call).  For callers that cannot allocate
 * device memory -- code running inside a framework that has reserved the whole device pool
 * for its own allocator, and plugins or callbacks that may only use the buffers they are
 * handed.  The per-bin counters live in a fixed array compiled into the
 * library (96 KB on every device that loads it, held until the process exits), so no
 * cudaMalloc, cudaFree or allocating library routine is called.  nbins is limited to
 * 12000; larger requests return MLC_ERR_LIMIT.  The first call on a device resolves the
 * array's device address (cudaGetSymbolAddress) with that device current.  Every call
 * clears the counters it uses, but all calls
 * on a device share the one array: calls that overlap on the GPU (other streams, other
 * contexts, other host threads) race and must be serialised by the caller.  The call copies
 * the counts to counts_host and waits for its stream before it returns. */
int mlc_histogram_f64_noalloc(mlc_ctx* ctx, long n, const double* v, int nbins, double lo, double hi, int logscale,
                              uint64_t* counts_host);

/* Self-test of the bounded-wait error path of the tensor-core kernels (no reference
 * counterpart).  One CTA allocates tensor memory as k_pairdiff_tc does, waits on an mbarrier
 * that nothing arrives at and that no copy or MMA feeds, gives up after `polls` polls
 * (1 .. 2^24), releases its tensor memory and returns.  report_host[3]: [0] 1 if the wait
 * gave up, [1] polls used, [2] 1 if the tensor memory was released after it.  Returns
 * MLC_ERR_TIMEOUT with the message of a timed-out wait (the expected outcome), after which
 * the context stays usable; waits for its stream before it returns. */
int mlc_selftest_wait_timeout(mlc_ctx* ctx, unsigned polls, unsigned* report_host);

/* ======================================================================= host-side stages (C++, FP64) */

/* setup_chi2_calculation (cpu_functions.cpp:80-144) with find_indices (:28-45), M = {MA, MB},
 * V = {V0}: maps the Nd data times to profile-size indices and interpolation factors for
 * images A and B, cuts at Njp (the first epoch outside the size range in both images) and
 * returns the constant chi2 term of the dropped epochs.  Output arrays hold Nd entries;
 * Njp_out receives their used length.  ref_compat = 1 keeps the reference's constant-term
 * range i = Nd-Njp .. Nd-1; 0 sums the dropped epochs Njp .. Nd-1. */
int mlc_setup_chi2(double MA, double MB, double V0, double Dfac, int Nd, const double* d_host,
                   const double* t_host, const double* s_host, int Nprof, const double* x_host, int ref_compat,
                   int* Njp_out, int* indA, int* indB, double* facA, double* facB, double* d_out, double* s_out,
                   double* const_term);

/* find_indices (cpu_functions.cpp:28-45): for each of the Nd ascending times t_host the
 * profile-size index j with x[j] <= t < x[j+1] (x_host: Nprof ascending sizes), -1 where
 * the reference leaves the entry unset (a time above the last size or before the first). */
int mlc_find_indices(const double* t_host, const double* x_host, int Nd, int Nprof, int* ind_host);

/* locations_on_grid / locations_random (locations.cpp:6-25); host arrays of Nside^2 / Nloc. */
int mlc_locations_grid(int Nside, int Nmap, int Noff, int* x_host, int* y_host);
int mlc_locations_random(int Nloc, int Nmap, int Noff, int seed, int* x_host, int* y_host);

/* Right bin edges of Mpd(Nbins, min, max, "log"|linear) (mpd.cpp:4-21). */
int mlc_bin_edges(int Nbins, double mn, double mx, int logscale, double* out_host);

/* trapezium (integration.cpp:3-9): sum (f1 f2 [i-1] + f1 f2 [i]) (x[i] - x[i-1]) / 2.
 * Returns the integral (not a status). */
double mlc_trapezium(int N, const double* f1, const double* f2, const double* x);

/* gerlumph map reader (magnification_map.cpp:7-40) from the directory dir (mapmeta.dat,
 * map.bin).  meta6 (nullable) receives avgmu, avgN, width, k, g, s.  out_host NULL reads
 * the size only; otherwise it receives the Nx*Nx FP64 magnifications. */
int mlc_read_gerlumph(const char* dir, int* Nx, double* width, double* meta6, double* out_host, long cap);

/* Page-locked host memory for the host-buffer calls (MLC_IO_HOST), on 2 MB pages: anonymous
 * memory advised for transparent huge pages (small pages where the host has none free) and
 * registered with the CUDA driver for every context.  The host-to-GPU copies of such buffers
 * keep their rate when the host memory is fragmented, where buffers pinned on small pages
 * lose part of it.  bytes are rounded up to 2 MB; the memory is zero-filled.  Returns
 * MLC_ERR_OOM when the host is out of memory, MLC_ERR_CUDA when the registration fails (no
 * GPU).  mlc_host_free releases a buffer from mlc_host_alloc (NULL is ignored). */
int mlc_host_alloc(size_t bytes, void** ptr);
int mlc_host_free(void* ptr);

/* ======================================================================= synthetic maps */

/* Inverse ray shooting (no reference counterpart; produces the gerlumph ray counts the
 * reference reads, magnification_map.cpp:27-31): nrx x nry rays on the image-plane grid
 * (x0 + i dx, y0 + j dx) are deflected by nl unit-mass point lenses (lenses_xy: device
 * float pairs, Einstein-radius units), smooth convergence kappa_c and shear gamma, and
 * counted into the N x N source-plane pixels of a square of side `width` centred on 0.
 * counts: device int32 N*N (zeroed here).  ctx is an mlc_ctx*. */
int mlc_rayshoot(void* ctx, const float* lenses_xy, int nl, double kappa_c, double gamma, double x0, double y0,
                 double dx, long nrx, long nry, double width, int N, int* counts);

#ifdef __cplusplus
}
#endif

#endif /* MICROLC_GB300_H */
