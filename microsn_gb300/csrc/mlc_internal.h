// Internal host-side state of the library: context, workspace pool, maps, FFT plans.
#pragma once

#include <functional>
#include <map>
#include <memory>
#include <string>
#include <tuple>
#include <vector>

#include "fft.cuh"
#include "mlc_common.cuh"

namespace mlc {

// Plan for 2-D real transforms of an Ny x Nx image: rows are real FFTs of length Nx
// (a complex FFT of length M = Nx/2 plus the split post-process); columns are complex
// FFTs of length Ny = N1 * N2 done as two in-place sub-passes over row sets.
struct FftPlan2D {
  int Nx = 0, Ny = 0, prec = 0;
  int M = 0;   // Nx / 2
  int Wc = 0;  // Nx / 2 + 1 spectrum columns
  int Wp = 0;  // spectrum pitch (complex elements), multiple of 16
  int N1 = 1, N2 = 1;
  int CW = 16;  // columns per strip: 128 bytes of complex data
  RadixList rlM{}, rlN1{}, rlN2{};
  void* twx = nullptr;  // Nx-entry table exp(-2 pi i m / Nx)
  void* twy = nullptr;  // Ny-entry table exp(-2 pi i m / Ny)
  size_t elem = 0;      // sizeof(C2<T>)
  size_t spec_bytes() const { return (size_t)Ny * Wp * elem; }
  ~FftPlan2D();
};

// Internal plan precisions (mlc_map_set_fft): FFTs in float-float arithmetic of FP64 maps
// (FP64 outputs), and of FP32 maps (float-float spectra, FP32 outputs).
constexpr int PREC_FF = 2;
constexpr int PREC_FFS = 3;
inline bool prec_is_ff(int prec) { return prec == PREC_FF || prec == PREC_FFS; }

enum WsSlot {
  WS_SPEC_TMP = 0,
  WS_KX,
  WS_KX2,         // the profile-row spectra of a second concurrent convolution chain
  WS_PROFILE,
  WS_KREAL,
  WS_KSPEC,
  WS_CONV_OUT,
  WS_SORT_KEYS,
  WS_SORT_VALS,
  WS_SORT_HIST,
  WS_PAIR_ACC,
  WS_SMALL,
  WS_LOC,
  WS_PAIR_CAND,  // pair-stage candidates, refinement list, counters, histogram
  WS_BATCH_MAPS,  // convolved maps of one profile group (mlc_convolve_sample_tracks)
  WS_BATCH_IMAP,  // their profile-interleaved copy
  WS_SAMPLE_ORDER,  // the sampler's epoch chunks in map-cell order
  WS_NSLOTS
};

}  // namespace mlc

namespace mlc {
struct BatchIO;  // copy streams, ring and staging buffers of the whole-step entry (batch.cu)
void batch_release(mlc_ctx* ctx);
void batch_synchronize(mlc_ctx* ctx);
void convolve_sample_tracks(mlc_ctx* ctx, mlc_map* map, const void* pixels, int nprof, const mlc_profile* profs,
                            const mlc_tracks& tr, int mode, int mag, void* out, int flags);
void ctx_join(mlc_ctx* ctx);
void convolve_many(mlc_ctx* ctx, mlc_map* map, int nprof, const mlc_profile* profs, int mode, void* out,
                   long long stride, int flags);
void sample_expanding(mlc_ctx* ctx, const void* maps, int Nx, int Ny, int prec, int nep, int nbands, int ntracks,
                      const void* x0, const void* y0, const void* phi, const void* v, const void* t, int mag,
                      void* out);
void set_chunk_bytes(mlc_ctx* ctx, size_t bytes);
}  // namespace mlc

struct mlc_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  int sm_count = 0;
  std::string err;
  // launch accounting and optional per-kernel CUDA-event timing
  unsigned long long launches = 0;
  bool timing = false;
  struct Pending {
    const char* name;
    cudaEvent_t a, b;
  };
  std::vector<Pending> pending;
  std::map<std::string, std::pair<double, long>> ktimes;  // name -> (ms, launches)
  void* ws_ptr[mlc::WS_NSLOTS] = {};
  size_t ws_size[mlc::WS_NSLOTS] = {};
  std::map<std::tuple<int, int, int>, std::unique_ptr<mlc::FftPlan2D>> plans;
  mlc::BatchIO* batch = nullptr;
  // launch autotuner: key -> choice (-1: FFT form; >= 0: direct tile shape), candidate timings
  bool autotune = true;
  bool two_chains = false;  // set while the batched step runs two convolution chains side by side
  // device bytes the cached profile spectra of the step and of mlc_convolve_many may take:
  // -1 a quarter of the device memory, 0 none (every call recomputes them)
  long long profile_cache_bytes = -1;
  std::map<std::string, int> tune;
  std::map<std::string, std::string> tune_log;
  std::map<std::string, std::string> tune_name;  // the choice as the report prints it
};

struct mlc_map {
  mlc_ctx* ctx = nullptr;
  int device = 0;  // kept here so that destroying a map never touches its context
  int Nx = 0, Ny = 0, prec = 0;
  void* data = nullptr;  // Ny x Nx real
  void* spec = nullptr;  // forward spectrum, digit-transposed row order
  bool spec_valid = false;
  int fft = 0;  // 0 transforms in the map's precision, 1 float-float (MLC_FFT_F32X2)
  size_t spec_cap = 0;  // bytes allocated at spec
};

namespace mlc {
// The map's spectrum buffer with room for `bytes` (a float-float spectrum of an FP32 map is
// twice its FP32 one).  Growing it frees the old buffer, which waits for the device.
inline void* map_spec_buffer(mlc_map* m, size_t bytes) {
  if (m->spec_cap < bytes) {
    if (m->spec) MLC_CUDA(cudaFree(m->spec));
    m->spec = nullptr;
    m->spec_cap = 0;
    MLC_CUDA(cudaMalloc(&m->spec, bytes));
    m->spec_cap = bytes;
  }
  return m->spec;
}
// Precision of a map's transforms: PREC_FF / PREC_FFS for FP64 / FP32 maps with float-float FFTs.
inline int map_fft_prec(const mlc_map* m) {
  if (m->fft == 1) return m->prec == MLC_F64 ? PREC_FF : PREC_FFS;
  return m->prec;
}
}  // namespace mlc

namespace mlc {

struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    cudaGetDevice(&prev);
    if (prev != dev) MLC_CUDA(cudaSetDevice(dev));
  }
  ~DeviceGuard() {
    int cur = -1;
    cudaGetDevice(&cur);
    if (prev >= 0 && cur != prev) cudaSetDevice(prev);
  }
};

void* ws_get(mlc_ctx* ctx, int slot, size_t bytes);

// Scope around one kernel launch: counts it and, when the context's timing is on,
// brackets it with CUDA events on the context's stream.
struct KernelScope {
  mlc_ctx* ctx;
  const char* name;
  cudaEvent_t a = nullptr, b = nullptr;
  KernelScope(mlc_ctx* c, const char* n) : ctx(c), name(n) {
    ctx->launches++;
    if (ctx->timing) {
      cudaEventCreate(&a);
      cudaEventCreate(&b);
      cudaEventRecord(a, ctx->stream);
    }
  }
  ~KernelScope() {
    if (a) {
      cudaEventRecord(b, ctx->stream);
      ctx->pending.push_back({name, a, b});
    }
  }
};
#define MLC_KSCOPE(ctx, name) ::mlc::KernelScope ks_##__LINE__((ctx), (name))

// Raise a kernel's dynamic shared-memory limit once.
void set_max_smem(const void* func, size_t bytes);

// FFT and convolution (fft.cu)
FftPlan2D* plan_get(mlc_ctx* ctx, int Nx, int Ny, int prec);
void fft2_forward(mlc_ctx* ctx, const FftPlan2D& p, const void* in, int in_dtype, void* spec);
void conv_fused(mlc_ctx* ctx, const FftPlan2D& p, const void* Fmap, const double* prof_dev, int pN,
                void* out_real);
// Direct tiled convolution of an FP32 map (real pixels) with a profile of 2..32 pixels, tile
// shape `variant`; and the autotuned choice for (map size, profile size): -1 for the FFT
// form, else the fastest direct tile shape (the first call times every candidate into out).
void conv_direct(mlc_ctx* ctx, const FftPlan2D& p, const void* map, const double* prof, int pN, int variant,
                 void* out);
// spectrum: the FFT alternative is conv_fused_spectrum (the caller runs the last pass of
// several profiles together), so out must hold a half-spectrum.
int conv_direct_choice(mlc_ctx* ctx, const FftPlan2D& p, const void* map, const void* Fmap, const double* prof,
                       int pN, void* out, bool spectrum);
// conv_fused, or the direct form where the autotuner chose it.
void conv_auto(mlc_ctx* ctx, const FftPlan2D& p, const void* map, const void* Fmap, const double* prof, int pN,
               void* out);
std::string autotune_report(mlc_ctx* ctx);
// The fused convolution's P1 variant for this map size and arithmetic: true for the one that
// stages the map-spectrum tile in shared memory.  The autotuner times run(false) and
// run(true) once per key; a pinned or earlier choice is reused.
// Runs k_wait_selftest (pairtc.cu) with the given poll limit; report_host[3] as documented
// at mlc_selftest_wait_timeout.  Throws MLC_ERR_TIMEOUT when the wait gave up.
void selftest_wait_timeout(mlc_ctx* ctx, unsigned polls, unsigned* report_host);
bool p1_staged_choice(mlc_ctx* ctx, const FftPlan2D& p, const std::function<void(bool)>& run);
// Cached profile spectra: the profile's spectrum as the fused convolution's P1 holds it
// before the product with the map spectrum (Ny x Wp complex of the plan's arithmetic, the
// map spectrum's layout), and conv_fused_spectrum starting from it.  Supported where P1 has
// its register form for N2 = 100 or 128.
bool profile_spectrum_supported(const FftPlan2D& p);
void profile_spectrum(mlc_ctx* ctx, const FftPlan2D& p, const double* prof, int pN, void* ks);
void conv_cached_spectrum(mlc_ctx* ctx, const FftPlan2D& p, const void* Fmap, const void* ks, void* spec_out);
void conv_cached(mlc_ctx* ctx, const FftPlan2D& p, const void* Fmap, const void* ks, void* out);
// conv_fused up to P2: the inverse half-spectrum (Ny x Wp complex) into spec_out.
void conv_fused_spectrum(mlc_ctx* ctx, const FftPlan2D& p, const void* Fmap, const double* prof, int pN,
                         void* spec_out, int kx_slot = WS_KX);
// P3 of nm (<= 16) such spectra (spec_stride complex elements apart) written straight into
// the interleaved layout out[(y Nx + x) S + q] (S a power of two >= nm, slots >= nm zero).
// False (nothing launched) when the row length has no register kernel.
bool rows_c2r_interleave_supported(const FftPlan2D& p);
// planar: bit q set = slot q holds the real convolved map (Ny x Nx, from the direct form)
// instead of a half-spectrum.
bool rows_c2r_interleave(mlc_ctx* ctx, const FftPlan2D& p, const void* specs, long spec_stride, int nm, int S,
                         void* out, unsigned planar = 0);
void conv_plain(mlc_ctx* ctx, const FftPlan2D& p, const void* Fmap, const double* prof_dev, int pN,
                void* out_real);
// Their per-precision forms (T = float, double, ff), defined in fft_impl.cuh and
// instantiated explicitly in fft_f32.cu, fft_f64.cu and fft_ff_*.cu.
template <typename T>
void forward_impl(mlc_ctx* ctx, const FftPlan2D& p, const void* in, int in_dtype, void* spec);
template <typename T>
void conv_fused_impl(mlc_ctx* ctx, const FftPlan2D& p, const void* Fmap, const double* prof, int pN, void* out,
                     void* spec_out = nullptr, int kx_slot = WS_KX);
template <typename T>
bool profile_spectrum_supported_impl(const FftPlan2D& p);
template <typename T>
void profile_spectrum_impl(mlc_ctx* ctx, const FftPlan2D& p, const double* prof, int pN, void* ks);
template <typename T>
void conv_cached_impl(mlc_ctx* ctx, const FftPlan2D& p, const void* Fmap, const void* ks, void* spec_out);
template <typename T>
void conv_cached_real_impl(mlc_ctx* ctx, const FftPlan2D& p, const void* Fmap, const void* ks, void* out);
template <typename T>
void conv_plain_impl(mlc_ctx* ctx, const FftPlan2D& p, const void* Fmap, const double* prof, int pN, void* out);
template <typename T, typename TO = typename RealOut<T>::type>
bool c2r_interleave_impl(mlc_ctx* ctx, const FftPlan2D& p, const void* specs, long spec_stride, int nm, int S,
                         void* out, unsigned planar);
template <typename T, typename TO>
void rows_c2r_impl(mlc_ctx* ctx, const FftPlan2D& p, const void* spec, void* out);

// Host profile rasters (profile.cpp)
int profile_dims(const mlc_profile& p);
int profile_raster(const mlc_profile& p, double* out, long cap);

// Multi-filter flux-ratio likelihood (fluxratio.cu)
void flux_ratio_chi2(mlc_ctx* ctx, const float* f_obs_host, const float* df_obs_host, const float* mu1,
                     const float* mu2, int N, int F, int T, float* chi2, double* likelihood_host);

// Spectrum of the map's current pixels, computed once and cached (api.cu).
void map_prepare(mlc_ctx* ctx, mlc_map* map);

// Differentiable track fit (profile.cu, fit.cu)
int thin_disc_fit_raster(double rhalf, double pix, int N, double* P, double* dPdx, double* dPdy, double* dPdR);
void radius_stack(mlc_ctx* ctx, mlc_map* map, int K, const double* radii, double pix, int N, void* stack);
void track_fit(mlc_ctx* ctx, const void* stack, int Nx, int Ny, int prec, int K, const double* radii, int ntracks,
               const void* theta, const int64_t* off, const void* t, const void* obs, const void* w, void* chi2,
               void* grad, void* model);

// Map MPDs (mpd.cu)
void map_binned_mpd(mlc_ctx* ctx, const mlc_map* map, int nb, double mn, double mx, double* bins_host,
                    double* counts_host);
void mpd_divide(mlc_ctx* ctx, int NA, const double* bA, const double* cA, int NB, const double* bB,
                const double* cB, int NR, const double* bR, double* cR);

// Sampling (sample.cu)
void interleave(mlc_ctx* ctx, const void* const* maps_host, int nmaps, long npix, int prec, int stride, void* out);
// out[p * S + off + q] = maps[q][p] for q < nmaps (<= 16); other slots untouched.
void interleave_into(mlc_ctx* ctx, const void* const* maps_host, int nmaps, long npix, int prec, int S, int off,
                     void* out);
// Interleaved-map track sampler: out[q * E + (e - ebase)] for the epochs e of the given
// tracks (off holds global epoch indices; ebase lets a chunk of tracks fill its own buffer).
// nep: at least off[ntracks] - off[0] (the epochs of these tracks).
void sample_tracks_il(mlc_ctx* ctx, const void* imap, int stride, int nmaps, int Nx, int Ny, int prec, int ntracks,
                      const void* x0, const void* y0, const void* phi, const void* v, const int64_t* off,
                      const void* t, int mag, void* out, long E, int64_t ebase, int64_t nep);
// Fused sample -> magnitude -> offset-minimised chi2 against one curve on shared epochs.
void track_chi2_offset(mlc_ctx* ctx, const void* imap, int stride, int nmaps, int Nx, int Ny, int prec, int ntracks,
                       const void* x0, const void* y0, const void* phi, const void* v, int Tn, const void* t,
                       const double* obs, const double* w, double* chi2, double* dm);
void sample_nearest(mlc_ctx* ctx, const double* map, int Nx, int Ny, int k, int Nprof, int Nloc, const int* lx,
                    const int* ly, double* LC, double* DLC);

}  // namespace mlc
