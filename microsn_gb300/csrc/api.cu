// C ABI of the library: argument checks, status codes, context and workspace.
// Every entry point catches mlc::Error (and std::exception) and returns a status; the
// message is kept in the context for mlc_ctx_last_error().
#include <cmath>
#include <algorithm>
#include <cstring>
#include <functional>
#include <vector>

#include "mlc_internal.h"
#include "pairdiff.h"

namespace mlc {
void sample_tracks(mlc_ctx* ctx, const void* const* maps_host, int nmaps, int Nx, int Ny, int prec,
                   int ntracks, const void* x0, const void* y0, const void* phi, const void* v,
                   const int64_t* off, const void* t, int mag, void* out, long E);
void chi2_offset(mlc_ctx* ctx, int prec, int ncurves, int T_, const void* m, const double* obs_dev,
                 const double* w_dev, double W, double* chi2, double* dm);
void pair_setup(mlc_ctx* ctx, int Nloc, int Nprof, const double* LCA, const double* LCB, int Nbins,
                const double* edges_host, uint32_t* rank, uint32_t* lower_host, uint32_t* nper_host);
void pair_chi2_ratio(mlc_ctx* ctx, int Njp, const int* indA, const int* indB, const double* facA,
                     const double* facB, const double* d, const double* s, int Nloc, int Nprof, const double* LCA,
                     const double* DLCA, const double* LCB, const double* DLCB, const uint32_t* rank, double* chi2);
void bin_chi2(mlc_ctx* ctx, int Nbins, const uint32_t* lower_host, const uint32_t* nper_host,
              const double* chi2_sorted, double* bchi2_host, double* bexp_host);
void pair_bin_fused(mlc_ctx* ctx, int Njp, const int* indA, const int* indB, const double* facA,
                    const double* facB, const double* d, const double* s, int Nloc, int Nprof, const double* LCA,
                    const double* DLCA, const double* LCB, const double* DLCB, int Nbins, const double* edges_host,
                    double* bchi2_host, double* bexp_host, uint32_t* nper_host);
void sort_f64_u32(mlc_ctx* ctx, long n, double* keys, uint32_t* vals);

void histogram_f64(mlc_ctx* ctx, long n, const double* v, int nbins, double lo, double hi, int logscale,
                   unsigned long long* counts_dev);

void* ws_get(mlc_ctx* ctx, int slot, size_t bytes) {
  if (bytes == 0) bytes = 16;
  if (ctx->ws_size[slot] >= bytes) return ctx->ws_ptr[slot];
  if (ctx->ws_ptr[slot]) {
    MLC_CUDA(cudaStreamSynchronize(ctx->stream));
    MLC_CUDA(cudaFree(ctx->ws_ptr[slot]));
    ctx->ws_ptr[slot] = nullptr;
    ctx->ws_size[slot] = 0;
  }
  size_t sz = (size_t)round_up((long)bytes, 1 << 20);
  void* p = nullptr;
  MLC_CUDA(cudaMalloc(&p, sz));
  ctx->ws_ptr[slot] = p;
  ctx->ws_size[slot] = sz;
  return p;
}

}  // namespace mlc

using namespace mlc;

namespace {

int fail(mlc_ctx* ctx, int code, const char* msg) {
  if (ctx) ctx->err = msg;
  return code;
}

template <typename F>
int guarded(mlc_ctx* ctx, F&& f) {
  if (!ctx) return MLC_ERR_ARG;
  try {
    DeviceGuard g(ctx->device);
    f();
    return MLC_OK;
  } catch (const Error& e) {
    ctx->err = e.what();
    return e.code;
  } catch (const std::bad_alloc&) {
    ctx->err = "host allocation failed";
    return MLC_ERR_OOM;
  } catch (const std::exception& e) {
    ctx->err = e.what();
    return MLC_ERR_CUDA;
  }
}

}  // namespace

extern "C" {

int mlc_version(void) { return 100; }

int mlc_ctx_create(int device, void* stream, mlc_ctx** out) {
  if (!out) return MLC_ERR_ARG;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) {
    cudaGetLastError();
    return MLC_ERR_CUDA;
  }
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return MLC_ERR_CUDA;
  if (prop.major * 10 + prop.minor != 103) return MLC_ERR_UNSUPPORTED;  // built for sm_103a only
  mlc_ctx* c = new (std::nothrow) mlc_ctx();
  if (!c) return MLC_ERR_OOM;
  c->device = device;
  c->stream = (cudaStream_t)stream;
  c->sm_count = prop.multiProcessorCount;
  *out = c;
  return MLC_OK;
}

int mlc_ctx_destroy(mlc_ctx* ctx) {
  if (!ctx) return MLC_ERR_ARG;
  {
    int prev = -1;
    cudaGetDevice(&prev);
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    batch_release(ctx);
    for (int i = 0; i < WS_NSLOTS; i++)
      if (ctx->ws_ptr[i]) cudaFree(ctx->ws_ptr[i]);
    ctx->plans.clear();
    if (prev >= 0) cudaSetDevice(prev);
  }
  delete ctx;
  return MLC_OK;
}

unsigned long long mlc_ctx_launch_count(const mlc_ctx* ctx) { return ctx ? ctx->launches : 0ull; }

static void resolve_timings(mlc_ctx* ctx) {
  if (ctx->pending.empty()) return;
  MLC_CUDA(cudaStreamSynchronize(ctx->stream));
  for (auto& p : ctx->pending) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, p.a, p.b);
    auto& e = ctx->ktimes[p.name];
    e.first += ms;
    e.second += 1;
    cudaEventDestroy(p.a);
    cudaEventDestroy(p.b);
  }
  ctx->pending.clear();
}

int mlc_ctx_set_autotune(mlc_ctx* ctx, int on) {
  return guarded(ctx, [&] { ctx->autotune = on != 0; });
}

int mlc_ctx_set_profile_cache(mlc_ctx* ctx, long long max_bytes) {
  if (!ctx) return MLC_ERR_ARG;
  if (max_bytes < -1) return fail(ctx, MLC_ERR_ARG, "max_bytes: -1, 0 or a byte count");
  return guarded(ctx, [&] { ctx->profile_cache_bytes = max_bytes; });
}

int mlc_ctx_tune_set(mlc_ctx* ctx, const char* key, int choice) {
  if (!ctx || !key || !*key) return fail(ctx, MLC_ERR_ARG, "null argument");
  return guarded(ctx, [&] {
    ctx->tune[key] = choice;
    ctx->tune_name[key] = "pinned " + std::to_string(choice);
    ctx->tune_log.erase(key);
  });
}

int mlc_ctx_autotune_report(mlc_ctx* ctx, char* buf, int cap) {
  if (!ctx || !buf || cap < 1) return -MLC_ERR_ARG;
  int n = 0;
  const int st = guarded(ctx, [&] {
    const std::string s = autotune_report(ctx);
    n = (int)s.size();
    const int m = std::min(n, cap - 1);
    std::memcpy(buf, s.data(), (size_t)m);
    buf[m] = 0;
  });
  return st == MLC_OK ? n : -st;
}

int mlc_ctx_set_timing(mlc_ctx* ctx, int on) {
  return guarded(ctx, [&] {
    resolve_timings(ctx);
    ctx->timing = on != 0;
  });
}

int mlc_ctx_kernel_times(mlc_ctx* ctx, char* names_host, int name_cap, double* ms_host, long* launches_host, int cap,
                         int reset) {
  if (!ctx || !names_host || !ms_host || !launches_host || cap < 0 || name_cap < 1) return -MLC_ERR_ARG;
  int n = 0;
  int st = guarded(ctx, [&] {
    resolve_timings(ctx);
    std::string names;
    for (auto& kv : ctx->ktimes) {
      if (n >= cap) break;
      names += kv.first + "\n";
      ms_host[n] = kv.second.first;
      launches_host[n] = kv.second.second;
      n++;
    }
    MLC_REQUIRE((int)names.size() < name_cap, MLC_ERR_LIMIT, "names buffer too small");
    std::memcpy(names_host, names.c_str(), names.size() + 1);
    if (reset) ctx->ktimes.clear();
  });
  return st ? -st : n;
}

int mlc_ctx_set_stream(mlc_ctx* ctx, void* stream) {
  if (!ctx) return MLC_ERR_ARG;
  ctx->stream = (cudaStream_t)stream;
  return MLC_OK;
}

int mlc_ctx_synchronize(mlc_ctx* ctx) {
  return guarded(ctx, [&] {
    MLC_CUDA(cudaStreamSynchronize(ctx->stream));
    batch_synchronize(ctx);
  });
}

const char* mlc_ctx_last_error(const mlc_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

size_t mlc_ctx_workspace_bytes(const mlc_ctx* ctx) {
  if (!ctx) return 0;
  size_t s = 0;
  for (int i = 0; i < WS_NSLOTS; i++) s += ctx->ws_size[i];
  return s;
}

int mlc_profile_dims(const mlc_profile* p, int* N) {
  if (!p || !N) return MLC_ERR_ARG;
  int n = profile_dims(*p);
  if (n <= 0) return MLC_ERR_ARG;
  *N = n;
  return MLC_OK;
}

int mlc_profile_raster(const mlc_profile* p, double* out_host, long cap, int* N) {
  if (!p || !out_host || !N) return MLC_ERR_ARG;
  int n = profile_raster(*p, out_host, cap);
  if (n == -2) return MLC_ERR_LIMIT;
  if (n <= 0) return MLC_ERR_ARG;
  *N = n;
  return MLC_OK;
}

int mlc_map_create(mlc_ctx* ctx, const void* data, int data_is_device, int data_dtype, int Nx, int Ny,
                   int precision, mlc_map** out) {
  if (!ctx || !out || !data) return fail(ctx, MLC_ERR_ARG, "null argument");
  if ((data_dtype != MLC_F64 && data_dtype != MLC_F32) || (precision != MLC_F64 && precision != MLC_F32))
    return fail(ctx, MLC_ERR_ARG, "dtype must be MLC_F64 or MLC_F32");
  if (Nx < 4 || Ny < 2 || Nx % 2 || Ny % 2) return fail(ctx, MLC_ERR_ARG, "map sides must be even (Nx >= 4)");
  *out = nullptr;
  mlc_map* m = new (std::nothrow) mlc_map();
  if (!m) return MLC_ERR_OOM;
  int st = guarded(ctx, [&] {
    plan_get(ctx, Nx, Ny, precision);  // validates the sizes
    m->ctx = ctx;
    m->device = ctx->device;
    m->Nx = Nx;
    m->Ny = Ny;
    m->prec = precision;
    const size_t n = (size_t)Nx * Ny;
    const size_t esz = precision == MLC_F64 ? 8 : 4;
    MLC_CUDA(cudaMalloc(&m->data, n * esz));
    if (data_dtype == precision) {
      MLC_CUDA(cudaMemcpyAsync(m->data, data, n * esz, data_is_device ? cudaMemcpyDeviceToDevice
                                                                       : cudaMemcpyHostToDevice,
                               ctx->stream));
    } else {
      // convert on the host side of the copy (rare path: upload in the other precision)
      std::vector<char> h(n * esz);
      std::vector<char> src;
      const void* s = data;
      const size_t isz = data_dtype == MLC_F64 ? 8 : 4;
      if (data_is_device) {
        src.resize(n * isz);
        MLC_CUDA(cudaMemcpyAsync(src.data(), data, n * isz, cudaMemcpyDeviceToHost, ctx->stream));
        MLC_CUDA(cudaStreamSynchronize(ctx->stream));
        s = src.data();
      }
      for (size_t i = 0; i < n; i++) {
        if (precision == MLC_F64) ((double*)h.data())[i] = ((const float*)s)[i];
        else ((float*)h.data())[i] = (float)((const double*)s)[i];
      }
      MLC_CUDA(cudaMemcpyAsync(m->data, h.data(), n * esz, cudaMemcpyHostToDevice, ctx->stream));
      MLC_CUDA(cudaStreamSynchronize(ctx->stream));
    }
  });
  if (st != MLC_OK) {
    if (m->data) cudaFree(m->data);
    delete m;
    return st;
  }
  *out = m;
  return MLC_OK;
}

int mlc_map_destroy(mlc_map* map) {
  if (!map) return MLC_ERR_ARG;
  int prev = -1;
  cudaGetDevice(&prev);
  cudaSetDevice(map->device);
  // cudaFree waits for the device; the context may already be gone
  if (map->data) cudaFree(map->data);
  if (map->spec) cudaFree(map->spec);
  if (prev >= 0) cudaSetDevice(prev);
  delete map;
  return MLC_OK;
}

int mlc_map_data(mlc_map* map, void** dev_ptr) {
  if (!map || !dev_ptr) return MLC_ERR_ARG;
  *dev_ptr = map->data;
  return MLC_OK;
}

extern "C++" {
void mlc::map_prepare(mlc_ctx* ctx, mlc_map* map) {
  if (map->spec_valid) return;
  FftPlan2D* p = plan_get(ctx, map->Nx, map->Ny, map_fft_prec(map));
  map_spec_buffer(map, p->spec_bytes());
  fft2_forward(ctx, *p, map->data, map->prec, map->spec);
  map->spec_valid = true;
}
}  // extern "C++"

int mlc_map_prepare(mlc_ctx* ctx, mlc_map* map) {
  if (!map) return fail(ctx, MLC_ERR_ARG, "null map");
  return guarded(ctx, [&] { map_prepare(ctx, map); });
}

int mlc_map_set_fft(mlc_map* map, int mode) {
  if (!map) return MLC_ERR_ARG;
  if (mode != MLC_FFT_NATIVE && mode != MLC_FFT_F32X2) return fail(map->ctx, MLC_ERR_ARG, "unknown FFT mode");
  if (map->fft != mode) {
    map->fft = mode;
    map->spec_valid = false;  // the spectrum's element type changes (and for FP32 maps its size)
  }
  return MLC_OK;
}

int mlc_map_refresh(mlc_ctx* ctx, mlc_map* map) {
  if (!map) return fail(ctx, MLC_ERR_ARG, "null map");
  return guarded(ctx, [&] {
    map->spec_valid = false;
    map_prepare(ctx, map);
  });
}

static const double* upload_profile(mlc_ctx* ctx, const mlc_profile& pr, int* pN) {
  const int N = profile_dims(pr);
  MLC_REQUIRE(N > 0, MLC_ERR_ARG, "invalid profile parameters");
  std::vector<double> h((size_t)N * N);
  MLC_REQUIRE(profile_raster(pr, h.data(), (long)h.size()) == N, MLC_ERR_ARG, "profile raster failed");
  double* d = (double*)ws_get(ctx, WS_PROFILE, sizeof(double) * h.size());
  // synchronous copy: the host buffer dies with this function
  MLC_CUDA(cudaStreamSynchronize(ctx->stream));
  MLC_CUDA(cudaMemcpy(d, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice));
  *pN = N;
  return d;
}

static void convolve_impl(mlc_ctx* ctx, mlc_map* map, const mlc_profile& pr, int mode, void* out) {
  MLC_REQUIRE(mode == MLC_CONV_FUSED || mode == MLC_CONV_PLAIN, MLC_ERR_ARG, "unknown convolution mode");
  map_prepare(ctx, map);
  FftPlan2D* p = plan_get(ctx, map->Nx, map->Ny, map_fft_prec(map));
  int N = 0;
  const double* prof = upload_profile(ctx, pr, &N);
  if (mode == MLC_CONV_FUSED) conv_auto(ctx, *p, map->data, map->spec, prof, N, out);
  else conv_plain(ctx, *p, map->spec, prof, N, out);
}

int mlc_convolve_direct(mlc_ctx* ctx, mlc_map* map, const mlc_profile* prof, int variant, void* out) {
  if (!ctx || !map || !prof || !out) return fail(ctx, MLC_ERR_ARG, "null argument");
  return guarded(ctx, [&] {
    MLC_REQUIRE(map->prec == MLC_F32, MLC_ERR_ARG, "the direct convolution takes FP32 maps");
    FftPlan2D* p = plan_get(ctx, map->Nx, map->Ny, map->prec);
    int N = 0;
    const double* d = upload_profile(ctx, *prof, &N);
    conv_direct(ctx, *p, map->data, d, N, variant, out);
  });
}

int mlc_convolve(mlc_ctx* ctx, mlc_map* map, const mlc_profile* prof, int mode, void* out) {
  if (!ctx || !map || !prof || !out) return fail(ctx, MLC_ERR_ARG, "null argument");
  return guarded(ctx, [&] { convolve_impl(ctx, map, *prof, mode, out); });
}

int mlc_expanding_source(mlc_ctx* ctx, mlc_map* map, const double* sizes_host, int Nprof, const mlc_profile* base,
                         double width, int Nloc, const int* loc_x, const int* loc_y, int mode, double* LC,
                         double* DLC) {
  if (!ctx || !map || !sizes_host || !base || !loc_x || !loc_y || !LC || (Nprof > 1 && !DLC))
    return fail(ctx, MLC_ERR_ARG, "null argument");
  if (map->prec != MLC_F64) return fail(ctx, MLC_ERR_ARG, "expanding_source needs an FP64 map");
  if (Nprof < 1 || Nloc < 0 || !(width > 0)) return fail(ctx, MLC_ERR_ARG, "bad sizes / width");
  return guarded(ctx, [&] {
    sample_nearest(ctx, (const double*)map->data, map->Nx, map->Ny, 0, Nprof, Nloc, loc_x, loc_y, LC, DLC);
    if (Nprof == 1) return;
    double* conv = (double*)ws_get(ctx, WS_CONV_OUT, sizeof(double) * (size_t)map->Nx * map->Ny);
    for (int k = 1; k < Nprof; k++) {
      mlc_profile pr = *base;
      pr.rhalf = sizes_host[k] * base->pix * map->Nx / width;  // gpu_functions.cu:184
      convolve_impl(ctx, map, pr, mode, conv);
      sample_nearest(ctx, conv, map->Nx, map->Ny, k, Nprof, Nloc, loc_x, loc_y, LC, DLC);
    }
  });
}

int mlc_sample_nearest(mlc_ctx* ctx, const double* map, int Nx, int Ny, int k, int Nprof, int Nloc,
                       const int* loc_x, const int* loc_y, double* LC, double* DLC) {
  if (!ctx || !map || !loc_x || !loc_y || !LC || (k > 0 && !DLC)) return fail(ctx, MLC_ERR_ARG, "null argument");
  if (k < 0 || k >= Nprof || Nx <= 0 || Ny <= 0) return fail(ctx, MLC_ERR_ARG, "bad profile index / size");
  return guarded(ctx, [&] { sample_nearest(ctx, map, Nx, Ny, k, Nprof, Nloc, loc_x, loc_y, LC, DLC); });
}

int mlc_sample_tracks(mlc_ctx* ctx, const void* const* maps_host, int nmaps, int Nx, int Ny, int precision,
                      int ntracks, const void* x0, const void* y0, const void* phi, const void* v,
                      const int64_t* off, const void* t, int mag, void* out) {
  if (!ctx || !maps_host || !x0 || !y0 || !phi || !v || !off || !t || !out)
    return fail(ctx, MLC_ERR_ARG, "null argument");
  if (nmaps < 1 || Nx < 2 || Ny < 2 || ntracks < 0 || (precision != MLC_F64 && precision != MLC_F32))
    return fail(ctx, MLC_ERR_ARG, "bad sizes");
  for (int i = 0; i < nmaps; i++)
    if (!maps_host[i]) return fail(ctx, MLC_ERR_ARG, "null map pointer");
  return guarded(ctx, [&] {
    int64_t E = 0;
    if (ntracks > 0) {
      MLC_CUDA(cudaMemcpyAsync(&E, off + ntracks, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
      MLC_CUDA(cudaStreamSynchronize(ctx->stream));
    }
    sample_tracks(ctx, maps_host, nmaps, Nx, Ny, precision, ntracks, x0, y0, phi, v, off, t, mag, out, (long)E);
  });
}

static bool pow2_le16(int s) { return s == 1 || s == 2 || s == 4 || s == 8 || s == 16; }

int mlc_interleave_maps(mlc_ctx* ctx, const void* const* maps_host, int nmaps, int Nx, int Ny, int precision,
                        int stride, void* out) {
  if (!ctx || !maps_host || !out) return fail(ctx, MLC_ERR_ARG, "null argument");
  if (nmaps < 1 || nmaps > 16 || !pow2_le16(stride) || stride < nmaps || Nx < 1 || Ny < 1 ||
      (precision != MLC_F64 && precision != MLC_F32))
    return fail(ctx, MLC_ERR_ARG, "need 1 <= nmaps <= stride, stride in {1,2,4,8,16}");
  for (int i = 0; i < nmaps; i++)
    if (!maps_host[i]) return fail(ctx, MLC_ERR_ARG, "null map pointer");
  return guarded(ctx, [&] { interleave(ctx, maps_host, nmaps, (long)Nx * Ny, precision, stride, out); });
}

int mlc_track_chi2_offset(mlc_ctx* ctx, const void* imap, int stride, int nmaps, int Nx, int Ny, int precision,
                          int ntracks, const void* x0, const void* y0, const void* phi, const void* v, int Tn,
                          const void* t, const double* obs, const double* w, double* chi2, double* dm) {
  if (!ctx || !imap || !x0 || !y0 || !phi || !v || !t || !obs || !w || !chi2)
    return fail(ctx, MLC_ERR_ARG, "null argument");
  if (nmaps < 1 || !pow2_le16(stride) || stride < nmaps || Nx < 2 || Ny < 2 || ntracks < 0 || Tn < 1 ||
      (precision != MLC_F64 && precision != MLC_F32))
    return fail(ctx, MLC_ERR_ARG, "bad sizes");
  return guarded(ctx, [&] {
    track_chi2_offset(ctx, imap, stride, nmaps, Nx, Ny, precision, ntracks, x0, y0, phi, v, Tn, t, obs, w, chi2, dm);
  });
}

int mlc_convolve_sample_tracks(mlc_ctx* ctx, mlc_map* map, const void* pixels, int nprof,
                               const mlc_profile* profiles_host, const mlc_tracks* tracks, int mode, int mag, void* out,
                               int flags) {
  if (!ctx || !map || !profiles_host || !tracks) return fail(ctx, MLC_ERR_ARG, "null argument");
  if (nprof < 1) return fail(ctx, MLC_ERR_ARG, "need at least one profile");
  if (mode != MLC_CONV_FUSED && mode != MLC_CONV_PLAIN) return fail(ctx, MLC_ERR_ARG, "unknown convolution mode");
  if (flags & ~(MLC_IO_HOST | MLC_ASYNC | MLC_GRAPH)) return fail(ctx, MLC_ERR_ARG, "unknown flags");
  if ((flags & MLC_GRAPH) && (flags & MLC_IO_HOST)) return fail(ctx, MLC_ERR_ARG, "MLC_GRAPH takes device buffers only");
  const mlc_tracks& tr = *tracks;
  if (tr.ntracks < 0 || tr.nepochs < 0) return fail(ctx, MLC_ERR_ARG, "negative track or epoch count");
  if (tr.ntracks > 0 && (!tr.x0 || !tr.y0 || !tr.phi || !tr.v || !tr.off || (tr.nepochs > 0 && !tr.t) || !out))
    return fail(ctx, MLC_ERR_ARG, "null track array or output");
  if (map->device != ctx->device) return fail(ctx, MLC_ERR_ARG, "map lives on another device");
  return guarded(ctx, [&] { convolve_sample_tracks(ctx, map, pixels, nprof, profiles_host, tr, mode, mag, out, flags); });
}

int mlc_fit_raster(double rhalf, double pix, int N, double* P_host, double* dPdx_host, double* dPdy_host,
                   double* dPdR_host) {
  if (!P_host) return MLC_ERR_ARG;
  return thin_disc_fit_raster(rhalf, pix, N, P_host, dPdx_host, dPdy_host, dPdR_host) == N ? MLC_OK : MLC_ERR_ARG;
}

int mlc_radius_stack(mlc_ctx* ctx, mlc_map* map, int K, const double* radii_host, double pix, int N, void* stack) {
  if (!ctx || !map || !radii_host || !stack) return fail(ctx, MLC_ERR_ARG, "null argument");
  if (map->device != ctx->device) return fail(ctx, MLC_ERR_ARG, "map lives on another device");
  if (!(pix > 0)) return fail(ctx, MLC_ERR_ARG, "pix must be positive");
  return guarded(ctx, [&] { radius_stack(ctx, map, K, radii_host, pix, N, stack); });
}

int mlc_track_fit(mlc_ctx* ctx, const void* stack, int Nx, int Ny, int precision, int K, const double* radii_host,
                  int ntracks, const void* theta, const int64_t* off, const void* t, const void* obs, const void* w,
                  void* chi2, void* grad, void* model) {
  if (!ctx || !stack || !radii_host || (ntracks > 0 && (!theta || !off || !t || !obs || !w)))
    return fail(ctx, MLC_ERR_ARG, "null argument");
  if (Nx < 2 || Ny < 2 || ntracks < 0 || (precision != MLC_F64 && precision != MLC_F32))
    return fail(ctx, MLC_ERR_ARG, "bad sizes or precision");
  return guarded(ctx, [&] {
    track_fit(ctx, stack, Nx, Ny, precision, K, radii_host, ntracks, theta, off, t, obs, w, chi2, grad, model);
  });
}

int mlc_flux_ratio_chi2(mlc_ctx* ctx, const float* f_obs_host, const float* df_obs_host, const float* mu1,
                        const float* mu2, int N, int F, int T, float* chi2, double* likelihood_host) {
  if (!ctx || !f_obs_host || !df_obs_host || !mu1 || !mu2 || !likelihood_host)
    return fail(ctx, MLC_ERR_ARG, "null argument");
  return guarded(ctx, [&] { flux_ratio_chi2(ctx, f_obs_host, df_obs_host, mu1, mu2, N, F, T, chi2, likelihood_host); });
}

int mlc_map_binned_mpd(mlc_ctx* ctx, mlc_map* map, int Nbins, double min, double max, double* bins_host,
                       double* counts_host) {
  if (!ctx || !map || !bins_host || !counts_host) return fail(ctx, MLC_ERR_ARG, "null argument");
  if (map->device != ctx->device) return fail(ctx, MLC_ERR_ARG, "map lives on another device");
  return guarded(ctx, [&] { map_binned_mpd(ctx, map, Nbins, min, max, bins_host, counts_host); });
}

int mlc_mpd_divide(mlc_ctx* ctx, int NA, const double* binsA_host, const double* countsA_host, int NB,
                   const double* binsB_host, const double* countsB_host, int NR, const double* binsR_host,
                   double* countsR_host) {
  if (!ctx || !binsA_host || !countsA_host || !binsB_host || !countsB_host || !binsR_host || !countsR_host)
    return fail(ctx, MLC_ERR_ARG, "null argument");
  return guarded(ctx, [&] {
    mpd_divide(ctx, NA, binsA_host, countsA_host, NB, binsB_host, countsB_host, NR, binsR_host, countsR_host);
  });
}

int mlc_convolve_many(mlc_ctx* ctx, mlc_map* map, int nprof, const mlc_profile* profiles_host, int mode, void* out,
                      long long out_stride, int flags) {
  if (!ctx || !map || !profiles_host || !out) return fail(ctx, MLC_ERR_ARG, "null argument");
  if (nprof < 1 || out_stride < (long long)map->Nx * map->Ny) return fail(ctx, MLC_ERR_ARG, "bad count or stride");
  if (mode != MLC_CONV_FUSED && mode != MLC_CONV_PLAIN) return fail(ctx, MLC_ERR_ARG, "unknown convolution mode");
  if (flags & ~MLC_GRAPH) return fail(ctx, MLC_ERR_ARG, "unknown flags");
  if (map->device != ctx->device) return fail(ctx, MLC_ERR_ARG, "map lives on another device");
  return guarded(ctx, [&] { convolve_many(ctx, map, nprof, profiles_host, mode, out, out_stride, flags); });
}

int mlc_sample_expanding(mlc_ctx* ctx, const void* maps, int Nx, int Ny, int precision, int nep, int nbands,
                         int ntracks, const void* x0, const void* y0, const void* phi, const void* v, const void* t,
                         int mag, void* out) {
  if (!ctx || !maps || !out || (ntracks > 0 && (!x0 || !y0 || !phi || !v || !t)))
    return fail(ctx, MLC_ERR_ARG, "null argument");
  if (Nx < 2 || Ny < 2 || nep < 1 || nbands < 1 || ntracks < 0 || (precision != MLC_F64 && precision != MLC_F32))
    return fail(ctx, MLC_ERR_ARG, "bad sizes");
  return guarded(ctx, [&] {
    sample_expanding(ctx, maps, Nx, Ny, precision, nep, nbands, ntracks, x0, y0, phi, v, t, mag, out);
  });
}

int mlc_ctx_join(mlc_ctx* ctx) {
  return guarded(ctx, [&] { ctx_join(ctx); });
}

int mlc_ctx_set_chunk_bytes(mlc_ctx* ctx, size_t bytes) {
  if (!ctx) return MLC_ERR_ARG;
  if (bytes < 4096) return fail(ctx, MLC_ERR_ARG, "chunk must hold at least 4096 bytes");
  return guarded(ctx, [&] { set_chunk_bytes(ctx, bytes); });
}

int mlc_sample_tracks_interleaved(mlc_ctx* ctx, const void* imap, int stride, int nmaps, int Nx, int Ny,
                                  int precision, int ntracks, const void* x0, const void* y0, const void* phi,
                                  const void* v, const int64_t* off, const void* t, int mag, void* out) {
  if (!ctx || !imap || !x0 || !y0 || !phi || !v || !off || !t || !out) return fail(ctx, MLC_ERR_ARG, "null argument");
  if (nmaps < 1 || !pow2_le16(stride) || stride < nmaps || Nx < 2 || Ny < 2 || ntracks < 0 ||
      (precision != MLC_F64 && precision != MLC_F32))
    return fail(ctx, MLC_ERR_ARG, "bad sizes");
  return guarded(ctx, [&] {
    int64_t E = 0;
    if (ntracks > 0) {
      MLC_CUDA(cudaMemcpyAsync(&E, off + ntracks, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
      MLC_CUDA(cudaStreamSynchronize(ctx->stream));
    }
    sample_tracks_il(ctx, imap, stride, nmaps, Nx, Ny, precision, ntracks, x0, y0, phi, v, off, t, mag, out, (long)E,
                     0, E);
  });
}

int mlc_chi2_offset(mlc_ctx* ctx, int precision, int ncurves, int T, const void* m, const double* obs_host,
                    const double* w_host, double* chi2, double* dm) {
  if (!ctx || !m || !obs_host || !w_host || !chi2) return fail(ctx, MLC_ERR_ARG, "null argument");
  if (ncurves < 0 || T < 1 || (precision != MLC_F64 && precision != MLC_F32))
    return fail(ctx, MLC_ERR_ARG, "bad sizes");
  double W = 0.0;
  for (int e = 0; e < T; e++) W += w_host[e];
  if (!(W > 0)) return fail(ctx, MLC_ERR_ARG, "weights must sum to a positive number");
  return guarded(ctx, [&] {
    double* buf = (double*)ws_get(ctx, WS_SMALL, sizeof(double) * 2 * T);
    MLC_CUDA(cudaStreamSynchronize(ctx->stream));
    MLC_CUDA(cudaMemcpy(buf, obs_host, sizeof(double) * T, cudaMemcpyHostToDevice));
    MLC_CUDA(cudaMemcpy(buf + T, w_host, sizeof(double) * T, cudaMemcpyHostToDevice));
    chi2_offset(ctx, precision, ncurves, T, m, buf, buf + T, W, chi2, dm);
  });
}

int mlc_pair_setup(mlc_ctx* ctx, int Nloc, int Nprof, const double* LCA, const double* LCB, int Nbins,
                   const double* edges_host, uint32_t* rank, uint32_t* lower_host, uint32_t* nper_host) {
  if (!ctx || !LCA || !LCB || (Nbins > 0 && (!edges_host || !lower_host || !nper_host)))
    return fail(ctx, MLC_ERR_ARG, "null argument");
  if (Nloc < 1 || Nprof < 1 || Nbins < 0) return fail(ctx, MLC_ERR_ARG, "bad sizes");
  for (int i = 1; i < Nbins; i++)
    if (!(edges_host[i] >= edges_host[i - 1])) return fail(ctx, MLC_ERR_ARG, "edges must be ascending");
  return guarded(ctx, [&] { pair_setup(ctx, Nloc, Nprof, LCA, LCB, Nbins, edges_host, rank, lower_host, nper_host); });
}

static int check_vars(mlc_ctx* ctx, int Njp, const int* iA, const int* iB, const double* fA, const double* fB,
                      const double* d, const double* s, int Nloc, int Nprof) {
  if (Njp < 0 || Nloc < 1 || Nprof < 2) return fail(ctx, MLC_ERR_ARG, "bad sizes");
  if (Njp > 0 && (!iA || !iB || !fA || !fB || !d || !s)) return fail(ctx, MLC_ERR_ARG, "null argument");
  for (int i = 0; i < Njp; i++)
    if (iA[i] < -1 || iA[i] >= Nprof - 1 || iB[i] < -1 || iB[i] >= Nprof - 1)
      return fail(ctx, MLC_ERR_ARG, "interpolation index outside [-1, Nprof-2]");
  return MLC_OK;
}

int mlc_pair_chi2_ratio(mlc_ctx* ctx, int Njp, const int* indA_host, const int* indB_host, const double* facA_host,
                        const double* facB_host, const double* d_host, const double* s_host, int Nloc, int Nprof,
                        const double* LCA, const double* DLCA, const double* LCB, const double* DLCB,
                        const uint32_t* rank, double* chi2) {
  if (!ctx || !LCA || !DLCA || !LCB || !DLCB || !chi2) return fail(ctx, MLC_ERR_ARG, "null argument");
  int st = check_vars(ctx, Njp, indA_host, indB_host, facA_host, facB_host, d_host, s_host, Nloc, Nprof);
  if (st) return st;
  return guarded(ctx, [&] {
    pair_chi2_ratio(ctx, Njp, indA_host, indB_host, facA_host, facB_host, d_host, s_host, Nloc, Nprof, LCA, DLCA,
                    LCB, DLCB, rank, chi2);
  });
}

int mlc_bin_chi2(mlc_ctx* ctx, int Nbins, const uint32_t* lower_host, const uint32_t* nper_host,
                 const double* chi2_sorted, double* binned_chi2_host, double* binned_exp_host) {
  if (!ctx || !lower_host || !nper_host || !chi2_sorted || !binned_chi2_host || !binned_exp_host)
    return fail(ctx, MLC_ERR_ARG, "null argument");
  if (Nbins < 0) return fail(ctx, MLC_ERR_ARG, "bad sizes");
  return guarded(ctx, [&] {
    bin_chi2(ctx, Nbins, lower_host, nper_host, chi2_sorted, binned_chi2_host, binned_exp_host);
  });
}

int mlc_pair_bin_fused(mlc_ctx* ctx, int Njp, const int* indA_host, const int* indB_host, const double* facA_host,
                       const double* facB_host, const double* d_host, const double* s_host, int Nloc, int Nprof,
                       const double* LCA, const double* DLCA, const double* LCB, const double* DLCB, int Nbins,
                       const double* edges_host, double* binned_chi2_host, double* binned_exp_host,
                       uint32_t* nper_host) {
  if (!ctx || !LCA || !DLCA || !LCB || !DLCB || !edges_host || !binned_chi2_host || !binned_exp_host)
    return fail(ctx, MLC_ERR_ARG, "null argument");
  int st = check_vars(ctx, Njp, indA_host, indB_host, facA_host, facB_host, d_host, s_host, Nloc, Nprof);
  if (st) return st;
  for (int i = 1; i < Nbins; i++)
    if (!(edges_host[i] >= edges_host[i - 1])) return fail(ctx, MLC_ERR_ARG, "edges must be ascending");
  return guarded(ctx, [&] {
    pair_bin_fused(ctx, Njp, indA_host, indB_host, facA_host, facB_host, d_host, s_host, Nloc, Nprof, LCA, DLCA,
                   LCB, DLCB, Nbins, edges_host, binned_chi2_host, binned_exp_host, nper_host);
  });
}

int mlc_pair_chi2_magdiff(mlc_ctx* ctx, int method, int NA, int NB, int T, const float* A, const float* B,
                          const double* w_host, const double* d_host, int offset, int nbins, double lo_log10,
                          double hi_log10, uint64_t* hist_host, int k, double* topk_val_host, int64_t* topk_i_host,
                          int64_t* topk_j_host, float* chi2_out, mlc_pair_stats* stats) {
  if (!ctx || !A || !B || !w_host || (k > 0 && (!topk_val_host || !topk_i_host || !topk_j_host)))
    return fail(ctx, MLC_ERR_ARG, "null argument");
  if (method != MLC_PAIR_PLAIN && method != MLC_PAIR_TENSOR) return fail(ctx, MLC_ERR_ARG, "unknown method");
  if (NA < 1 || NB < 1 || T < 1 || k < 0 || nbins < 1 || !(hi_log10 > lo_log10))
    return fail(ctx, MLC_ERR_ARG, "bad sizes");
  if ((long long)NA * NB > (1LL << 40)) return fail(ctx, MLC_ERR_LIMIT, "more than 2^40 pairs");
  return guarded(ctx, [&] {
    PdResult r;
    pairdiff_run(ctx, method, A, B, NA, NB, T, w_host, d_host, offset, nbins, lo_log10, hi_log10, hist_host, k,
                 topk_val_host, topk_i_host, topk_j_host, chi2_out, r);
    if (stats) {
      stats->delta = r.delta;
      stats->threshold = r.thr;
      stats->refined = r.nrefined;
      stats->candidates = r.ncand;
      stats->passes = r.passes;
      stats->below = r.below;
      stats->above = r.above;
    }
  });
}

int mlc_pair_chi2_magdiff_list(mlc_ctx* ctx, int NA, int NB, int T, const float* A, const float* B,
                               const double* w_host, const double* d_host, int offset, long npairs,
                               const int64_t* ia, const int64_t* ib, double* chi2) {
  if (!ctx || !A || !B || !w_host || !ia || !ib || !chi2) return fail(ctx, MLC_ERR_ARG, "null argument");
  if (NA < 1 || NB < 1 || T < 1 || npairs < 0) return fail(ctx, MLC_ERR_ARG, "bad sizes");
  return guarded(ctx, [&] {
    double W = 0.0;
    for (int t = 0; t < T; t++) W += w_host[t];
    MLC_REQUIRE(W > 0, MLC_ERR_ARG, "weights sum to zero");
    double* buf = (double*)ws_get(ctx, WS_SMALL, sizeof(double) * 2 * T);
    MLC_CUDA(cudaStreamSynchronize(ctx->stream));
    MLC_CUDA(cudaMemcpy(buf, w_host, sizeof(double) * T, cudaMemcpyHostToDevice));
    if (d_host) MLC_CUDA(cudaMemcpy(buf + T, d_host, sizeof(double) * T, cudaMemcpyHostToDevice));
    pairdiff_plain(ctx, A, B, NA, NB, T, buf, d_host ? buf + T : nullptr, W, offset, npairs, (const long*)ia,
                   (const long*)ib, chi2);
  });
}

struct mlc_pair_side {
  int device = 0;
  PdSide s;
};

namespace {
int side_new(mlc_ctx* ctx, mlc_pair_side** out, const std::function<void(PdSide&)>& build) {
  mlc_pair_side* sd = new mlc_pair_side;
  sd->device = ctx->device;
  const int st = guarded(ctx, [&] { build(sd->s); });
  if (st != MLC_OK) {
    delete sd;
    return st;
  }
  *out = sd;
  return MLC_OK;
}
}  // namespace

int mlc_pair_side_curves(mlc_ctx* ctx, int N, int T, const float* X, const double* w_host, const double* d_host,
                         int offset, mlc_pair_side** side) {
  if (!ctx || !X || !w_host || !side) return fail(ctx, MLC_ERR_ARG, "null argument");
  *side = nullptr;
  if (N < 1 || T < 1) return fail(ctx, MLC_ERR_ARG, "bad sizes");
  if (T > 128) return fail(ctx, MLC_ERR_LIMIT, "pair sides support T <= 128 epochs");
  return side_new(ctx, side, [&](PdSide& s) { pd_side_from_curves(ctx, X, N, T, w_host, d_host, offset, s); });
}

int mlc_pair_side_expanding(mlc_ctx* ctx, const float* maps, int Nx, int Ny, int nep, int nbands, int ntracks,
                            const float* x0, const float* y0, const float* phi, const float* v, const float* t,
                            const double* w_host, const double* d_host, int offset, mlc_pair_side** side) {
  if (!ctx || !maps || !x0 || !y0 || !phi || !v || !t || !w_host || !side)
    return fail(ctx, MLC_ERR_ARG, "null argument");
  *side = nullptr;
  if (Nx < 2 || Ny < 2 || nep < 1 || nbands < 1 || ntracks < 1) return fail(ctx, MLC_ERR_ARG, "bad sizes");
  if ((long)nep * nbands > 128) return fail(ctx, MLC_ERR_LIMIT, "pair sides support nep*nbands <= 128");
  return side_new(ctx, side, [&](PdSide& s) {
    pd_side_from_expanding(ctx, maps, Nx, Ny, nep, nbands, ntracks, x0, y0, phi, v, t, w_host, d_host, offset, s);
  });
}

int mlc_pair_side_destroy(mlc_pair_side* side) {
  if (!side) return MLC_ERR_ARG;
  int prev = -1;
  cudaGetDevice(&prev);
  cudaSetDevice(side->device);
  pd_side_free(side->s);
  if (prev >= 0) cudaSetDevice(prev);
  delete side;
  return MLC_OK;
}

int mlc_selftest_wait_timeout(mlc_ctx* ctx, unsigned polls, unsigned* report_host) {
  if (!ctx || !report_host) return fail(ctx, MLC_ERR_ARG, "null argument");
  return guarded(ctx, [&] { selftest_wait_timeout(ctx, polls, report_host); });
}

int mlc_pair_chi2_sides(mlc_ctx* ctx, const mlc_pair_side* A, const mlc_pair_side* B, int nbins, double lo_log10,
                        double hi_log10, uint64_t* hist_host, int k, double* topk_val_host, int64_t* topk_i_host,
                        int64_t* topk_j_host, float* chi2_out, mlc_pair_stats* stats) {
  if (!ctx || !A || !B || (k > 0 && (!topk_val_host || !topk_i_host || !topk_j_host)))
    return fail(ctx, MLC_ERR_ARG, "null argument");
  if (A->device != ctx->device || B->device != ctx->device)
    return fail(ctx, MLC_ERR_ARG, "pair side built on another device");
  if (k < 0 || nbins < 1 || !(hi_log10 > lo_log10)) return fail(ctx, MLC_ERR_ARG, "bad sizes");
  if ((long long)A->s.N * B->s.N > (1LL << 40)) return fail(ctx, MLC_ERR_LIMIT, "more than 2^40 pairs");
  return guarded(ctx, [&] {
    PdResult r;
    pairdiff_sides(ctx, A->s, B->s, nbins, lo_log10, hi_log10, hist_host, k, topk_val_host, topk_i_host, topk_j_host,
                   chi2_out, r);
    if (stats) {
      stats->delta = r.delta;
      stats->threshold = r.thr;
      stats->refined = r.nrefined;
      stats->candidates = r.ncand;
      stats->passes = r.passes;
      stats->below = r.below;
      stats->above = r.above;
    }
  });
}

int mlc_sort_f64_u32(mlc_ctx* ctx, long n, double* keys, uint32_t* vals) {
  if (!ctx || (n > 0 && (!keys || !vals))) return fail(ctx, MLC_ERR_ARG, "null argument");
  if (n < 0) return fail(ctx, MLC_ERR_ARG, "bad size");
  return guarded(ctx, [&] { sort_f64_u32(ctx, n, keys, vals); });
}

int mlc_histogram_f64(mlc_ctx* ctx, long n, const double* v, int nbins, double lo, double hi, int logscale,
                      uint64_t* counts_host) {
  if (!ctx || (n > 0 && !v) || !counts_host) return fail(ctx, MLC_ERR_ARG, "null argument");
  if (nbins < 1 || nbins > 12000 || !(hi > lo) || n < 0) return fail(ctx, MLC_ERR_ARG, "bad histogram spec");
  return guarded(ctx, [&] {
    unsigned long long* c = (unsigned long long*)ws_get(ctx, WS_SMALL, sizeof(unsigned long long) * nbins);
    histogram_f64(ctx, n, v, nbins, lo, hi, logscale, c);
    MLC_CUDA(cudaMemcpyAsync(counts_host, c, sizeof(uint64_t) * nbins, cudaMemcpyDeviceToHost, ctx->stream));
    MLC_CUDA(cudaStreamSynchronize(ctx->stream));
  });
}

}  // extern "C"
