// The light-curve step of one lensed image through one call (mlc_convolve_sample_tracks):
// map upload, forward spectrum, convolution with every profile, interleave, track
// sampling and the download of the light curves.
//
// Replaces expanding_source (simulating_lcurves/src/gpu_functions.cu:82-225), which per
// profile builds the kernel on the host, uploads it, transforms, multiplies, transforms
// back, samples and synchronises.  Here every kernel runs on the context's stream and,
// with host buffers, the copies run on two internal streams:
//
//   h2d stream   pixels of call i+1 (once call i's forward transform has read the
//                map), tracks of call i+1 (double-buffered by call parity)
//   compute      profiles upload, forward spectrum, convolutions, interleave, sampling
//                of one chunk of tracks at a time into a ring of output slots
//   d2h stream   each filled slot back to the caller's buffer while the next chunk is
//                sampled; the slot is reused once its copy has run
//
// so that, with MLC_ASYNC, one call's download overlaps the next call's convolutions.
#include <algorithm>
#include <atomic>
#include <cstring>
#include <numeric>
#include <thread>
#include <vector>

#include "mlc_internal.h"

namespace mlc {

// One captured kernel sequence: the key of pointers and sizes it was captured with, the
// executable graph and the number of our kernels in it.
struct GraphSlot {
  std::vector<uint64_t> key;
  cudaGraphExec_t exec = nullptr;
  unsigned long long launches = 0;
};

struct BatchIO {
  // Output ring: enough slots for about two calls' light curves (4 to 64 slots), so that
  // the sampling of one call never waits for its own downloads and the next call's
  // kernels start while this call's chunks are still being copied back.
  static constexpr int NRING = 64;
  int nring = 4;                     // slots in use (grow-only)
  size_t slot_bytes = 256ull << 20;  // one output chunk
  cudaStream_t h2d = nullptr, d2h = nullptr;
  // second compute stream: the odd profiles' P0-P2 run on it, beside the even ones'
  cudaStream_t aux = nullptr;
  cudaEvent_t spec_ready = nullptr, aux_done = nullptr;
  // third compute stream: the last pass of a group's first eight profiles, beside the
  // remaining profiles' P0-P2
  cudaStream_t tail = nullptr;
  cudaEvent_t half_main = nullptr, half_aux = nullptr, half_done = nullptr;
  cudaEvent_t pix_free = nullptr;  // compute: the forward transform has read the map pixels
  cudaEvent_t pix_in = nullptr;    // h2d: pixels uploaded
  cudaEvent_t h2d_last = nullptr, d2h_last = nullptr;
  void* ring[NRING] = {};
  size_t ring_cap[NRING] = {};
  cudaEvent_t ring_full[NRING] = {}, ring_free[NRING] = {};
  int ring_pos = 0;
  void* trk[2] = {};
  size_t trk_cap[2] = {};
  cudaEvent_t trk_in[2] = {}, trk_free[2] = {};
  double* prof_host[2] = {};
  size_t prof_cap[2] = {};
  cudaEvent_t prof_sent[2] = {};
  // device rasters of the last profile list (reused while the list and map size repeat)
  void* prof_dev = nullptr;
  size_t prof_dev_cap = 0;
  std::vector<unsigned char> prof_key;
  std::vector<int> prof_N;
  std::vector<size_t> prof_off;
  int parity = 0;
  // the profiles' spectra (as the fused convolution's P1 holds them before the product with
  // the map spectrum) of the last profile list, map size and transform arithmetic
  void* kcache = nullptr;
  size_t kcache_cap = 0, kcache_stride = 0;
  std::vector<unsigned char> kcache_key;
  // the kernel sequences of the last mlc_convolve_many and mlc_convolve_sample_tracks calls
  // with MLC_GRAPH, each replayed while every pointer and size it baked in stays the same
  cudaStream_t cap = nullptr;
  GraphSlot many, step;
};

static void ev_create(cudaEvent_t* e) { MLC_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming)); }

static BatchIO* batch_get(mlc_ctx* ctx) {
  if (ctx->batch) return ctx->batch;
  BatchIO* b = new BatchIO();
  ctx->batch = b;  // released by batch_release even if a creation below fails
  MLC_CUDA(cudaStreamCreateWithFlags(&b->h2d, cudaStreamNonBlocking));
  MLC_CUDA(cudaStreamCreateWithFlags(&b->d2h, cudaStreamNonBlocking));
  MLC_CUDA(cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking));
  MLC_CUDA(cudaStreamCreateWithFlags(&b->aux, cudaStreamNonBlocking));
  MLC_CUDA(cudaStreamCreateWithFlags(&b->tail, cudaStreamNonBlocking));
  ev_create(&b->spec_ready);
  ev_create(&b->aux_done);
  ev_create(&b->half_main);
  ev_create(&b->half_aux);
  ev_create(&b->half_done);
  ev_create(&b->pix_free);
  ev_create(&b->pix_in);
  ev_create(&b->h2d_last);
  ev_create(&b->d2h_last);
  for (int i = 0; i < BatchIO::NRING; i++) {
    ev_create(&b->ring_full[i]);
    ev_create(&b->ring_free[i]);
  }
  for (int i = 0; i < 2; i++) {
    ev_create(&b->trk_in[i]);
    ev_create(&b->trk_free[i]);
    ev_create(&b->prof_sent[i]);
  }
  return b;
}

static void sync_all(mlc_ctx* ctx, BatchIO* b) {
  MLC_CUDA(cudaStreamSynchronize(ctx->stream));
  MLC_CUDA(cudaStreamSynchronize(b->aux));
  MLC_CUDA(cudaStreamSynchronize(b->tail));
  MLC_CUDA(cudaStreamSynchronize(b->h2d));
  MLC_CUDA(cudaStreamSynchronize(b->d2h));
}

void batch_synchronize(mlc_ctx* ctx) {
  BatchIO* b = ctx->batch;
  if (!b) return;
  if (b->h2d) MLC_CUDA(cudaStreamSynchronize(b->h2d));
  if (b->d2h) MLC_CUDA(cudaStreamSynchronize(b->d2h));
}

void batch_release(mlc_ctx* ctx) {
  BatchIO* b = ctx->batch;
  if (!b) return;
  if (b->h2d) cudaStreamSynchronize(b->h2d);
  if (b->d2h) cudaStreamSynchronize(b->d2h);
  for (int i = 0; i < BatchIO::NRING; i++) {
    if (b->ring[i]) cudaFree(b->ring[i]);
    if (b->ring_full[i]) cudaEventDestroy(b->ring_full[i]);
    if (b->ring_free[i]) cudaEventDestroy(b->ring_free[i]);
  }
  for (int i = 0; i < 2; i++) {
    if (b->trk[i]) cudaFree(b->trk[i]);
    if (b->prof_host[i]) cudaFreeHost(b->prof_host[i]);
    for (cudaEvent_t e : {b->trk_in[i], b->trk_free[i], b->prof_sent[i]})
      if (e) cudaEventDestroy(e);
  }
  if (b->aux) cudaStreamSynchronize(b->aux);
  if (b->tail) cudaStreamSynchronize(b->tail);
  for (cudaEvent_t e : {b->pix_free, b->pix_in, b->h2d_last, b->d2h_last, b->spec_ready, b->aux_done, b->half_main,
                        b->half_aux, b->half_done})
    if (e) cudaEventDestroy(e);
  if (b->aux) cudaStreamDestroy(b->aux);
  if (b->tail) cudaStreamDestroy(b->tail);
  if (b->prof_dev) cudaFree(b->prof_dev);
  if (b->kcache) cudaFree(b->kcache);
  for (GraphSlot* g : {&b->many, &b->step})
    if (g->exec) cudaGraphExecDestroy(g->exec);
  if (b->cap) cudaStreamDestroy(b->cap);
  if (b->h2d) cudaStreamDestroy(b->h2d);
  if (b->d2h) cudaStreamDestroy(b->d2h);
  delete b;
  ctx->batch = nullptr;
}

// Device buffer that may still be in use by queued work on any of the three streams.
static void* grow_dev(mlc_ctx* ctx, BatchIO* b, void*& p, size_t& cap, size_t need) {
  if (cap >= need) return p;
  sync_all(ctx, b);
  if (p) MLC_CUDA(cudaFree(p));
  p = nullptr;
  cap = 0;
  const size_t sz = (size_t)round_up((long)need, 1 << 20);
  MLC_CUDA(cudaMalloc(&p, sz));
  cap = sz;
  return p;
}

static int pow2_at_least(int n) {
  int s = 1;
  while (s < n) s <<= 1;
  return s;
}

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Rasters of nprof profiles into page-locked staging (host threads, largest first: they
// take milliseconds each while the previous call's kernels still run) and one upload into
// the context's profile buffer on its stream; a call with the same profile list and map
// size as the previous one reuses the uploaded rasters.  pN / poff receive the raster
// sides and element offsets.
static const double* stage_profiles(mlc_ctx* ctx, BatchIO* b, int par, int nprof, const mlc_profile* profs, int Nx,
                                    int Ny, std::vector<int>& pN, std::vector<size_t>& poff) {
  std::vector<unsigned char> key(sizeof(int) * 2 + sizeof(mlc_profile) * (size_t)nprof);
  std::memcpy(key.data(), &Nx, sizeof(int));
  std::memcpy(key.data() + sizeof(int), &Ny, sizeof(int));
  if (nprof > 0) std::memcpy(key.data() + 2 * sizeof(int), profs, sizeof(mlc_profile) * (size_t)nprof);
  if (b->prof_dev && key == b->prof_key) {
    pN = b->prof_N;
    poff = b->prof_off;
    return (const double*)b->prof_dev;
  }
  pN.assign(nprof, 0);
  poff.assign(nprof + 1, 0);
  for (int k = 0; k < nprof; k++) {
    pN[k] = profile_dims(profs[k]);
    MLC_REQUIRE(pN[k] > 0, MLC_ERR_ARG, "invalid profile parameters");
    MLC_REQUIRE(pN[k] <= Nx && pN[k] <= Ny, MLC_ERR_LIMIT, "profile raster larger than the map");
    poff[k + 1] = poff[k] + (size_t)pN[k] * pN[k];
  }
  const size_t pbytes = poff[nprof] * sizeof(double);
  MLC_CUDA(cudaEventSynchronize(b->prof_sent[par]));  // the last upload from this staging buffer has run
  if (b->prof_cap[par] < pbytes) {
    if (b->prof_host[par]) MLC_CUDA(cudaFreeHost(b->prof_host[par]));
    b->prof_host[par] = nullptr;
    b->prof_cap[par] = 0;
    MLC_CUDA(cudaMallocHost((void**)&b->prof_host[par], pbytes));
    b->prof_cap[par] = pbytes;
  }
  std::vector<int> order(nprof);
  std::iota(order.begin(), order.end(), 0);
  std::sort(order.begin(), order.end(), [&](int a, int c) { return pN[a] > pN[c]; });
  std::atomic<int> next{0}, bad{0};
  double* host = b->prof_host[par];
  auto work = [&] {
    for (int i = next++; i < nprof; i = next++) {
      const int k = order[i];
      if (profile_raster(profs[k], host + poff[k], (long)(poff[k + 1] - poff[k])) != pN[k]) bad = 1;
    }
  };
  const int nth = std::max(0, std::min<int>(nprof, (int)std::thread::hardware_concurrency()) - 1);
  std::vector<std::thread> pool;
  for (int i = 0; i < nth; i++) pool.emplace_back(work);
  work();
  for (auto& th : pool) th.join();
  MLC_REQUIRE(!bad, MLC_ERR_ARG, "profile raster failed");
  b->prof_key.clear();  // invalid until the new rasters are queued
  double* dprof = (double*)grow_dev(ctx, b, b->prof_dev, b->prof_dev_cap, std::max<size_t>(pbytes, 8));
  // (kernels of earlier calls that read the old rasters precede this copy on the stream)
  MLC_CUDA(cudaMemcpyAsync(dprof, host, pbytes, cudaMemcpyHostToDevice, ctx->stream));
  MLC_CUDA(cudaEventRecord(b->prof_sent[par], ctx->stream));
  b->prof_key = std::move(key);
  b->prof_N = pN;
  b->prof_off = poff;
  return dprof;
}

// The profile spectra of the list just staged (stage_profiles), computed once and kept while
// the list, the map size and the transform arithmetic repeat: a convolution then reads its
// profile's spectrum instead of transforming the profile (P0 and half of P1).  nullptr
// where the plan has no cached form or the spectra would exceed the context's budget.
static const char* profile_cache(mlc_ctx* ctx, BatchIO* b, const FftPlan2D& p, int nprof, const double* dprof,
                                 const std::vector<int>& pN, const std::vector<size_t>& poff) {
  if (ctx->profile_cache_bytes == 0 || !profile_spectrum_supported(p)) return nullptr;
  std::vector<unsigned char> key = b->prof_key;
  key.push_back((unsigned char)p.prec);
  if (b->kcache && key == b->kcache_key) return (const char*)b->kcache;
  size_t budget = (size_t)ctx->profile_cache_bytes;
  if (ctx->profile_cache_bytes < 0) {
    size_t fr = 0, tot = 0;
    MLC_CUDA(cudaMemGetInfo(&fr, &tot));
    budget = tot / 4;
  }
  const size_t stride = (size_t)round_up((long)p.spec_bytes(), 256);
  if ((size_t)nprof * stride > budget) return nullptr;
  b->kcache_key.clear();  // invalid until the new spectra are queued
  char* kc = (char*)grow_dev(ctx, b, b->kcache, b->kcache_cap, (size_t)nprof * stride);
  for (int k = 0; k < nprof; k++) profile_spectrum(ctx, p, dprof + poff[k], pN[k], kc + (size_t)k * stride);
  b->kcache_stride = stride;
  b->kcache_key = std::move(key);
  return kc;
}

template <typename T>
static void run(mlc_ctx* ctx, mlc_map* map, const void* pixels, int nprof, const mlc_profile* profs,
                const mlc_tracks& tr, int mode, int mag, void* out, int flags) {
  const bool host = (flags & MLC_IO_HOST) != 0;
  const size_t es = sizeof(T);
  const int Nx = map->Nx, Ny = map->Ny;
  const long npix = (long)Nx * Ny;
  FftPlan2D* p = plan_get(ctx, Nx, Ny, map_fft_prec(map));
  BatchIO* b = batch_get(ctx);
  const int par = b->parity;
  b->parity ^= 1;
  const int ntr = tr.ntracks;
  const int64_t E = tr.nepochs;

  // ---- profiles: all rasters into page-locked staging, one upload on the compute stream
  std::vector<int> pN;
  std::vector<size_t> poff;
  const double* dprof = stage_profiles(ctx, b, par, nprof, profs, Nx, Ny, pN, poff);

  // ---- map pixels and forward spectrum
  if (pixels) {
    if (host) {
      MLC_CUDA(cudaStreamWaitEvent(b->h2d, b->pix_free, 0));
      MLC_CUDA(cudaMemcpyAsync(map->data, pixels, npix * es, cudaMemcpyHostToDevice, b->h2d));
      MLC_CUDA(cudaEventRecord(b->pix_in, b->h2d));
      MLC_CUDA(cudaStreamWaitEvent(ctx->stream, b->pix_in, 0));
    } else if (pixels != map->data) {
      MLC_CUDA(cudaMemcpyAsync(map->data, pixels, npix * es, cudaMemcpyDeviceToDevice, ctx->stream));
    }
    map->spec_valid = false;
  }
  if (!map->spec_valid) {
    map_spec_buffer(map, p->spec_bytes());
    fft2_forward(ctx, *p, map->data, map->prec, map->spec);
    map->spec_valid = true;
  }
  {
    // (not while the sequence is being captured into a graph: an event recorded in a
    // capture may not be waited on by the uncaptured host-buffer path)
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    MLC_CUDA(cudaStreamIsCapturing(ctx->stream, &cs));
    if (cs == cudaStreamCaptureStatusNone) MLC_CUDA(cudaEventRecord(b->pix_free, ctx->stream));
  }

  // ---- tracks
  const char* x0 = (const char*)tr.x0;
  const char* y0 = (const char*)tr.y0;
  const char* phi = (const char*)tr.phi;
  const char* v = (const char*)tr.v;
  const int64_t* off = tr.off;  // host offsets with MLC_IO_HOST, else device
  const int64_t* doff = tr.off;  // device offsets
  const char* t = (const char*)tr.t;
  std::vector<std::pair<int, int>> chunks;  // track ranges of the output chunks (host IO)
  const int nm_max = std::min(nprof, 16);
  if (host && ntr > 0) {
    MLC_REQUIRE(off[0] == 0 && off[ntr] == E, MLC_ERR_ARG, "track offsets must run from 0 to nepochs");
    const size_t sp = align256(ntr * es), so = align256((ntr + 1) * sizeof(int64_t)), st = align256(E * es);
    char* d = (char*)grow_dev(ctx, b, b->trk[par], b->trk_cap[par], 4 * sp + so + st);
    // the buffer of this parity is free once the sampling two calls back has finished
    MLC_CUDA(cudaStreamWaitEvent(b->h2d, b->trk_free[par], 0));
    MLC_CUDA(cudaMemcpyAsync(d, x0, ntr * es, cudaMemcpyHostToDevice, b->h2d));
    MLC_CUDA(cudaMemcpyAsync(d + sp, y0, ntr * es, cudaMemcpyHostToDevice, b->h2d));
    MLC_CUDA(cudaMemcpyAsync(d + 2 * sp, phi, ntr * es, cudaMemcpyHostToDevice, b->h2d));
    MLC_CUDA(cudaMemcpyAsync(d + 3 * sp, v, ntr * es, cudaMemcpyHostToDevice, b->h2d));
    MLC_CUDA(cudaMemcpyAsync(d + 4 * sp, off, (ntr + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, b->h2d));
    MLC_CUDA(cudaMemcpyAsync(d + 4 * sp + so, t, E * es, cudaMemcpyHostToDevice, b->h2d));
    MLC_CUDA(cudaEventRecord(b->trk_in[par], b->h2d));
    // chunks of whole tracks whose light curves fill at most one ring slot
    const int64_t cap_e = (int64_t)(b->slot_bytes / ((size_t)nm_max * es));
    for (int t0 = 0; t0 < ntr;) {
      MLC_REQUIRE(off[t0 + 1] - off[t0] <= cap_e, MLC_ERR_LIMIT, "one track has more epochs than an output chunk holds");
      const int64_t* lim = std::upper_bound(off + t0 + 1, off + ntr + 1, off[t0] + cap_e);
      const int t1 = (int)(lim - off) - 1;  // last offset within the cap
      chunks.emplace_back(t0, t1);
      t0 = t1;
    }
    const size_t call_bytes = (size_t)nprof * E * es;
    const long want = 2 * (long)((call_bytes + b->slot_bytes - 1) / b->slot_bytes);
    const int nring = (int)std::max<long>(b->nring, std::min<long>(BatchIO::NRING, std::max(4L, want)));
    if (nring != b->nring) {
      sync_all(ctx, b);
      b->nring = nring;
      b->ring_pos = 0;
    }
    for (int i = 0; i < b->nring; i++) grow_dev(ctx, b, b->ring[i], b->ring_cap[i], b->slot_bytes);
    x0 = d;
    y0 = d + sp;
    phi = d + 2 * sp;
    v = d + 3 * sp;
    doff = (const int64_t*)(d + 4 * sp);
    t = d + 4 * sp + so;
  }

  // ---- profile groups of up to 16: convolve, interleave, sample.  Where the row length has
  // a register c2r kernel, each profile stops at its inverse half-spectrum and one
  // cluster kernel runs the last pass of all the group's profiles straight into the
  // interleaved layout (no planar maps, no separate interleave pass).
  const bool fuse_il = ntr > 0 && mode == MLC_CONV_FUSED && rows_c2r_interleave_supported(*p);
  const char* kc = fuse_il ? profile_cache(ctx, b, *p, nprof, dprof, pN, poff) : nullptr;
  const size_t slot = fuse_il ? p->spec_bytes() : (size_t)npix * es;
  char* maps = (char*)ws_get(ctx, WS_BATCH_MAPS, (size_t)nm_max * slot);
  void* imap = ntr > 0 ? ws_get(ctx, WS_BATCH_IMAP, (size_t)pow2_at_least(nm_max) * npix * es) : nullptr;
  bool tracks_ready = false;
  for (int g0 = 0; g0 < nprof; g0 += 16) {
    const int nm = std::min(16, nprof - g0);
    const int stride = pow2_at_least(nm);
    const void* mp[16];
    unsigned planar = 0;  // slots holding a real map from the direct form
    // the odd profiles' P0-P2 on the second stream, after the map spectrum (not under the
    // per-kernel timing, whose event pairs would then span the other stream's kernels)
    const bool two = fuse_il && !ctx->timing;
    // with more than eight profiles, the first eight's last pass (the first 32-byte sector of
    // every 64-byte pixel, so its stores still fill whole sectors) starts on a third stream
    // as soon as both chains are past them
    const bool split = two && stride == 16 && nm > 8;
    // slot stride in spectrum elements (C2 of the transform's type: 16 bytes for float-float
    // spectra, also of FP32 maps) -- a planar slot is read through the same pointer type
    const long spec_stride = (long)(slot / p->elem);
    if (two) {
      MLC_CUDA(cudaEventRecord(b->spec_ready, ctx->stream));
      MLC_CUDA(cudaStreamWaitEvent(b->aux, b->spec_ready, 0));
    }
    struct ChainsFlag {  // the convolutions below know they share the GPU with a second chain
      mlc_ctx* c;
      ~ChainsFlag() { c->two_chains = false; }
    } chains_flag{ctx};
    ctx->two_chains = two;
    for (int q = 0; q < nm; q++) {
      mp[q] = maps + (size_t)q * slot;
      const double* pr = dprof + poff[g0 + q];
      const int dv = mode == MLC_CONV_FUSED
                         ? conv_direct_choice(ctx, *p, map->data, map->spec, pr, pN[g0 + q], (void*)mp[q], fuse_il)
                         : -1;
      if (dv >= 0) {
        conv_direct(ctx, *p, map->data, pr, pN[g0 + q], dv, (void*)mp[q]);
        planar |= 1u << q;
      } else if (two && (q & 1)) {
        cudaStream_t main = ctx->stream;
        ctx->stream = b->aux;
        try {
          if (kc) conv_cached_spectrum(ctx, *p, map->spec, kc + (size_t)(g0 + q) * b->kcache_stride, (void*)mp[q]);
          else conv_fused_spectrum(ctx, *p, map->spec, pr, pN[g0 + q], (void*)mp[q], WS_KX2);
        } catch (...) {
          ctx->stream = main;
          throw;
        }
        ctx->stream = main;
      } else if (fuse_il) {
        if (kc) conv_cached_spectrum(ctx, *p, map->spec, kc + (size_t)(g0 + q) * b->kcache_stride, (void*)mp[q]);
        else conv_fused_spectrum(ctx, *p, map->spec, pr, pN[g0 + q], (void*)mp[q]);
      } else if (mode == MLC_CONV_FUSED) {
        conv_fused(ctx, *p, map->spec, pr, pN[g0 + q], (void*)mp[q]);
      } else {
        conv_plain(ctx, *p, map->spec, pr, pN[g0 + q], (void*)mp[q]);
      }
      if (split && q == 7) {
        MLC_CUDA(cudaEventRecord(b->half_main, ctx->stream));
        MLC_CUDA(cudaEventRecord(b->half_aux, b->aux));
        MLC_CUDA(cudaStreamWaitEvent(b->tail, b->half_main, 0));
        MLC_CUDA(cudaStreamWaitEvent(b->tail, b->half_aux, 0));
        cudaStream_t main = ctx->stream;
        ctx->stream = b->tail;
        try {
          rows_c2r_interleave(ctx, *p, maps, spec_stride, 8, stride, imap, planar & 0xFFu);
        } catch (...) {
          ctx->stream = main;
          throw;
        }
        ctx->stream = main;
        MLC_CUDA(cudaEventRecord(b->half_done, b->tail));
      }
    }
    if (two) {  // the last pass needs both chains
      MLC_CUDA(cudaEventRecord(b->aux_done, b->aux));
      MLC_CUDA(cudaStreamWaitEvent(ctx->stream, b->aux_done, 0));
    }
    if (ntr == 0) continue;
    if (split) {
      MLC_CUDA(cudaStreamWaitEvent(ctx->stream, b->half_done, 0));
      rows_c2r_interleave(ctx, *p, maps + 8 * slot, spec_stride, nm - 8, stride, (char*)imap + 8 * es, planar >> 8);
    } else if (fuse_il) {
      rows_c2r_interleave(ctx, *p, maps, spec_stride, nm, stride, imap, planar);
    } else {
      interleave(ctx, mp, nm, npix, map->prec, stride, imap);
    }
    if (!host) {
      sample_tracks_il(ctx, imap, stride, nm, Nx, Ny, map->prec, ntr, x0, y0, phi, v, off, t, mag,
                       (char*)out + (size_t)g0 * E * es, (long)E, 0, E);
      continue;
    }
    if (!tracks_ready) {
      MLC_CUDA(cudaStreamWaitEvent(ctx->stream, b->trk_in[par], 0));
      tracks_ready = true;
    }
    for (const auto& c : chunks) {
      const int t0 = c.first, t1 = c.second;
      const int64_t e0 = off[t0], Ec = off[t1] - off[t0];
      if (Ec == 0) continue;
      const int s = b->ring_pos++ % b->nring;
      MLC_CUDA(cudaStreamWaitEvent(ctx->stream, b->ring_free[s], 0));
      sample_tracks_il(ctx, imap, stride, nm, Nx, Ny, map->prec, t1 - t0, x0 + t0 * es, y0 + t0 * es,
                       phi + t0 * es, v + t0 * es, doff + t0, t, mag, b->ring[s], (long)Ec, e0, Ec);
      MLC_CUDA(cudaEventRecord(b->ring_full[s], ctx->stream));
      MLC_CUDA(cudaStreamWaitEvent(b->d2h, b->ring_full[s], 0));
      char* dst = (char*)out + ((size_t)g0 * E + e0) * es;
      if ((size_t)E * es < (1ull << 30)) {
        MLC_CUDA(cudaMemcpy2DAsync(dst, E * es, b->ring[s], Ec * es, Ec * es, nm, cudaMemcpyDeviceToHost, b->d2h));
      } else {
        for (int q = 0; q < nm; q++)
          MLC_CUDA(cudaMemcpyAsync(dst + (size_t)q * E * es, (const char*)b->ring[s] + (size_t)q * Ec * es, Ec * es,
                                   cudaMemcpyDeviceToHost, b->d2h));
      }
      MLC_CUDA(cudaEventRecord(b->ring_free[s], b->d2h));
    }
  }
  if (host) {
    if (ntr > 0) MLC_CUDA(cudaEventRecord(b->trk_free[par], ctx->stream));
    MLC_CUDA(cudaEventRecord(b->h2d_last, b->h2d));
    MLC_CUDA(cudaEventRecord(b->d2h_last, b->d2h));
  }
  // device buffers: stream-ordered like every other device entry; host buffers: the call
  // returns with out filled unless MLC_ASYNC
  if (host && !(flags & MLC_ASYNC)) sync_all(ctx, b);
}

// Replays the slot's graph when key() matches the key it was captured with; otherwise runs
// enqueue() eagerly (this call's result, and the run that sizes every workspace and fills
// every cache the sequence consults), then captures a second enqueue() on the internal
// stream -- streams that the sequence forks to through events join the capture -- and
// keeps the instantiated graph for later calls.  Nothing is allocated or synchronised
// while capturing: every buffer exists after the eager run and the key holds their
// addresses.
template <typename Enq, typename Key>
static void run_graph(mlc_ctx* ctx, BatchIO* b, GraphSlot& slot, Enq&& enqueue, Key&& key) {
  if (slot.exec && slot.key == key()) {
    ctx->launches += slot.launches;
    MLC_CUDA(cudaGraphLaunch(slot.exec, ctx->stream));
    return;
  }
  const unsigned long long l0 = ctx->launches;
  enqueue();
  const unsigned long long nl = ctx->launches - l0;
  if (slot.exec) {
    MLC_CUDA(cudaGraphExecDestroy(slot.exec));
    slot.exec = nullptr;
  }
  const unsigned long long launches = ctx->launches;
  // the capture stream starts after the eager run (the graph launch itself goes on the
  // context's stream later; the capture only records)
  cudaStream_t saved = ctx->stream;
  ctx->stream = b->cap;
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    try {
      enqueue();
    } catch (...) {
      cudaStreamEndCapture(b->cap, &g);
      if (g) cudaGraphDestroy(g);
      ctx->stream = saved;
      ctx->launches = launches;
      throw;
    }
    e = cudaStreamEndCapture(b->cap, &g);
  }
  ctx->stream = saved;
  ctx->launches = launches;
  MLC_CUDA(e);
  e = cudaGraphInstantiate(&slot.exec, g, 0);
  cudaGraphDestroy(g);
  MLC_CUDA(e);
  slot.key = key();
  slot.launches = nl;
}

void convolve_sample_tracks(mlc_ctx* ctx, mlc_map* map, const void* pixels, int nprof, const mlc_profile* profs,
                            const mlc_tracks& tr, int mode, int mag, void* out, int flags) {
  auto go = [&] {
    if (map->prec == MLC_F64) run<double>(ctx, map, pixels, nprof, profs, tr, mode, mag, out, flags & ~MLC_GRAPH);
    else run<float>(ctx, map, pixels, nprof, profs, tr, mode, mag, out, flags & ~MLC_GRAPH);
  };
  if (!(flags & MLC_GRAPH) || ctx->timing) {
    go();
    return;
  }
  MLC_REQUIRE(!(flags & MLC_IO_HOST), MLC_ERR_ARG, "MLC_GRAPH takes device buffers only");
  BatchIO* b = batch_get(ctx);
  // the rasters first (host work, and an upload when the list changed): the graph reads
  // them from the same device buffer
  std::vector<int> pN;
  std::vector<size_t> poff;
  const double* dprof = stage_profiles(ctx, b, b->parity, nprof, profs, map->Nx, map->Ny, pN, poff);
  // and the profile spectra, recomputed here (outside the graph) when the list changed
  FftPlan2D* p = plan_get(ctx, map->Nx, map->Ny, map_fft_prec(map));
  const bool fuse_il = tr.ntracks > 0 && mode == MLC_CONV_FUSED && rows_c2r_interleave_supported(*p);
  const char* kc = fuse_il ? profile_cache(ctx, b, *p, nprof, dprof, pN, poff) : nullptr;
  auto key = [&] {
    std::vector<uint64_t> kv = {(uint64_t)map,      (uint64_t)map->data, (uint64_t)map->spec, (uint64_t)pixels,
                                (uint64_t)nprof,    (uint64_t)mode,      (uint64_t)mag,       (uint64_t)out,
                                (uint64_t)tr.x0,    (uint64_t)tr.y0,     (uint64_t)tr.phi,    (uint64_t)tr.v,
                                (uint64_t)tr.off,   (uint64_t)tr.t,      (uint64_t)tr.ntracks, (uint64_t)tr.nepochs,
                                (uint64_t)dprof,    (uint64_t)map_fft_prec(map), (uint64_t)ctx->autotune,
                                (uint64_t)kc};
    for (int s = 0; s < WS_NSLOTS; s++) kv.push_back((uint64_t)ctx->ws_ptr[s]);
    for (int k = 0; k < nprof; k++) kv.push_back((uint64_t)pN[k]);
    return kv;
  };
  run_graph(ctx, b, b->step, go, key);
  if (!pixels) return;
  map->spec_valid = true;  // the replayed forward transform has refreshed the spectrum
}

// Convolutions of one map with many profiles into out + k * stride (the map's precision):
// rasters staged and uploaded once, then the fused (or plain) convolution per profile.
// With MLC_GRAPH the per-profile kernel sequence is captured once into a CUDA graph (on an
// internal stream, after an eager run has sized every workspace) and later calls with the
// same map, profile sizes, output and workspace replay it with one launch.
void convolve_many(mlc_ctx* ctx, mlc_map* map, int nprof, const mlc_profile* profs, int mode, void* out,
                   long long stride, int flags) {
  BatchIO* b = batch_get(ctx);
  const int par = b->parity;
  b->parity ^= 1;
  FftPlan2D* p = plan_get(ctx, map->Nx, map->Ny, map_fft_prec(map));
  map_prepare(ctx, map);
  std::vector<int> pN;
  std::vector<size_t> poff;
  const double* dprof = stage_profiles(ctx, b, par, nprof, profs, map->Nx, map->Ny, pN, poff);
  const size_t es = map->prec == MLC_F64 ? 8 : 4;
  const char* kc = mode == MLC_CONV_FUSED ? profile_cache(ctx, b, *p, nprof, dprof, pN, poff) : nullptr;
  auto enqueue = [&] {
    for (int k = 0; k < nprof; k++) {
      void* o = (char*)out + (size_t)k * stride * es;
      if (mode != MLC_CONV_FUSED) {
        conv_plain(ctx, *p, map->spec, dprof + poff[k], pN[k], o);
      } else if (kc && conv_direct_choice(ctx, *p, map->data, map->spec, dprof + poff[k], pN[k], o, false) < 0) {
        conv_cached(ctx, *p, map->spec, kc + (size_t)k * b->kcache_stride, o);
      } else {
        conv_auto(ctx, *p, map->data, map->spec, dprof + poff[k], pN[k], o);
      }
    }
  };
  auto key = [&] {
    std::vector<uint64_t> kv = {(uint64_t)map, (uint64_t)map->spec, (uint64_t)nprof, (uint64_t)mode, (uint64_t)out,
                                (uint64_t)stride, (uint64_t)dprof, (uint64_t)kc};
    for (int s = 0; s < WS_NSLOTS; s++) kv.push_back((uint64_t)ctx->ws_ptr[s]);
    for (int k = 0; k < nprof; k++) kv.push_back((uint64_t)pN[k]);
    return kv;
  };
  if (!(flags & MLC_GRAPH) || ctx->timing) {
    enqueue();
    return;
  }
  run_graph(ctx, b, b->many, enqueue, key);
}

void ctx_join(mlc_ctx* ctx) {
  BatchIO* b = ctx->batch;
  if (!b) return;
  MLC_CUDA(cudaStreamWaitEvent(ctx->stream, b->h2d_last, 0));
  MLC_CUDA(cudaStreamWaitEvent(ctx->stream, b->d2h_last, 0));
}

void set_chunk_bytes(mlc_ctx* ctx, size_t bytes) {
  BatchIO* b = batch_get(ctx);
  if (b->slot_bytes == bytes) return;
  sync_all(ctx, b);
  for (int i = 0; i < BatchIO::NRING; i++) {
    if (b->ring[i]) MLC_CUDA(cudaFree(b->ring[i]));
    b->ring[i] = nullptr;
    b->ring_cap[i] = 0;
  }
  b->slot_bytes = bytes;
  b->nring = 4;
  b->ring_pos = 0;
}

}  // namespace mlc
