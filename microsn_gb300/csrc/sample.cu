// Light-curve sampling: nearest-pixel reads at fixed locations (the reference's
// kernel_sample) and bilinear sampling along straight source tracks with the
// magnitude conversion fused in; plus the offset-minimised chi2 against one observed
// curve.
#include <cmath>
#include <cstdio>

#include "bilinear.cuh"
#include <algorithm>

#include "mlc_internal.h"
#include "scan.cuh"

namespace mlc {

// kernel_sample (simulating_lcurves/src/gpu_functions.cu:604-620).
__global__ void k_sample_nearest(const double* __restrict__ map, int Nx, int Ny, int k, int Nprof, int Nloc,
                                 const int* __restrict__ lx, const int* __restrict__ ly, double* __restrict__ LC,
                                 double* __restrict__ DLC) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= Nloc) return;
  const int x = lx[id], y = ly[id];
  const double v = (x >= 0 && x < Nx && y >= 0 && y < Ny) ? map[(long)y * Nx + x] : __longlong_as_double(0x7ff8000000000000ll);
  LC[(long)id * Nprof + k] = v;
  if (k > 0) DLC[(long)id * (Nprof - 1) + k - 1] = v - LC[(long)id * Nprof + k - 1];
}

void sample_nearest(mlc_ctx* ctx, const double* map, int Nx, int Ny, int k, int Nprof, int Nloc, const int* lx,
                    const int* ly, double* LC, double* DLC) {
  if (Nloc <= 0) return;
  {
    MLC_KSCOPE(ctx, "sample_nearest");
    k_sample_nearest<<<ceil_div(Nloc, 256), 256, 0, ctx->stream>>>(map, Nx, Ny, k, Nprof, Nloc, lx, ly, LC, DLC);
  }
  MLC_CHECK_LAUNCH();
}



template <typename T>
struct MapList {
  const T* m[16];
};

// One warp per track; lanes walk the track's epochs.  For every epoch the position
// and weights are computed once and reused for each of the nm maps of this launch.
template <typename T>
__global__ void __launch_bounds__(256) k_sample_tracks(MapList<T> maps, int nm, int Nx, int Ny, int ntracks,
                                                       const T* __restrict__ x0, const T* __restrict__ y0,
                                                       const T* __restrict__ phi, const T* __restrict__ v,
                                                       const int64_t* __restrict__ off, const T* __restrict__ t,
                                                       int mag, T* __restrict__ out, long E, int m_base) {
  const int lane = threadIdx.x & 31;
  const long track = (long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (track >= ntracks) return;
  const TrackGeom<T> g(x0[track], y0[track], phi[track], v[track]);
  const int64_t e0 = off[track], e1 = off[track + 1];
  for (int64_t e = e0 + lane; e < e1; e += 32) {
    const Bilin<T> B = g.at(t[e], Nx, Ny);
    for (int q = 0; q < nm; q++) {
      T mu = B.inside ? bilin_read<T>(maps.m[q], B, Nx) : (T)0;
      out[(long)(m_base + q) * E + e] = mag ? (T)-2.5 * mlc_log10(mu) : mu;
    }
  }
}

template <typename T>
static void sample_tracks_impl(mlc_ctx* ctx, const void* const* maps_host, int nmaps, int Nx, int Ny,
                               int ntracks, const void* x0, const void* y0, const void* phi, const void* v,
                               const int64_t* off, const void* t, int mag, void* out, long E) {
  for (int base = 0; base < nmaps; base += 16) {
    MapList<T> ml{};
    const int nm = std::min(16, nmaps - base);
    for (int q = 0; q < nm; q++) ml.m[q] = (const T*)maps_host[base + q];
    const int warps_per_block = 8;
    const int grid = ceil_div(ntracks, warps_per_block);
    {
      MLC_KSCOPE(ctx, "sample_tracks");
      k_sample_tracks<T><<<grid, 256, 0, ctx->stream>>>(ml, nm, Nx, Ny, ntracks, (const T*)x0, (const T*)y0,
                                                      (const T*)phi, (const T*)v, off, (const T*)t, mag,
                                                      (T*)out, E, base);
    }
    MLC_CHECK_LAUNCH();
  }
}

void sample_tracks(mlc_ctx* ctx, const void* const* maps_host, int nmaps, int Nx, int Ny, int prec,
                   int ntracks, const void* x0, const void* y0, const void* phi, const void* v,
                   const int64_t* off, const void* t, int mag, void* out, long E) {
  if (ntracks <= 0 || nmaps <= 0) return;
  if (prec == MLC_F64)
    sample_tracks_impl<double>(ctx, maps_host, nmaps, Nx, Ny, ntracks, x0, y0, phi, v, off, t, mag, out, E);
  else
    sample_tracks_impl<float>(ctx, maps_host, nmaps, Nx, Ny, ntracks, x0, y0, phi, v, off, t, mag, out, E);
}

// ---------------------------------------------------------------- profile-interleaved maps
//
// With nm maps of one source sampled at the same positions, a planar layout costs every
// bilinear corner one random 8-byte read per map, which HBM serves as a 64-byte granule.
// Interleaving the maps pixel by pixel ([y][x][stride], stride >= nm, a power of two)
// makes a corner one contiguous 4*stride-byte read for all maps at once.

// out[p*S + off + q] = maps[q][p] for q < width (0 for nm <= q < width).  A CTA moves a
// tile of 256 pixels: coalesced loads of each map's 256 values into shared memory, then
// the tile's width-long runs are written with consecutive threads on consecutive words
// (a whole contiguous block when width == S).  wshift = log2(width) when width is a power
// of two, else -1.
template <typename T>
__global__ void __launch_bounds__(256) k_interleave(MapList<T> maps, int nm, int width, int wshift, int S, int off,
                                                   long npix, T* __restrict__ out) {
  __shared__ T tile[16][257];
  const long ntiles = (npix + 255) / 256;
  for (long tb = blockIdx.x; tb < ntiles; tb += gridDim.x) {
    const long p0 = tb * 256;
    const int np = (int)min(256L, npix - p0);
    for (int q = 0; q < width; q++) {
      const long p = p0 + threadIdx.x;
      tile[q][threadIdx.x] = (q < nm && threadIdx.x < np) ? __ldg(maps.m[q] + p) : (T)0;
    }
    __syncthreads();
    T* o = out + p0 * S + off;
    const int nout = np * width;
    for (int i = threadIdx.x; i < nout; i += blockDim.x) {
      const int px = wshift >= 0 ? (i >> wshift) : i / width;
      const int q = i - px * width;
      o[(long)px * S + q] = tile[q][px];
    }
    __syncthreads();
  }
}

template <typename T, int NM>
struct Pix {
  T v[NM];
};

template <typename T, int NM>
__device__ __forceinline__ void load_pix(const T* __restrict__ p, T* v) {
  if constexpr (sizeof(T) * NM % 16 == 0) {
    const float4* q = reinterpret_cast<const float4*>(p);
    float4* d = reinterpret_cast<float4*>(v);
#pragma unroll
    for (int i = 0; i < (int)(sizeof(T) * NM / 16); i++) d[i] = __ldg(q + i);
  } else {
#pragma unroll
    for (int i = 0; i < NM; i++) v[i] = __ldg(p + i);
  }
}

// One epoch of one track on an interleaved map: with the bilinear weights of its position
// (TrackGeom::at), every map's value (or magnitude) into out[q * E + o].
template <typename T, int NM>
__device__ __forceinline__ void sample_epoch(const T* __restrict__ imap, int Nx, const Bilin<T>& B, int mag,
                                             T* __restrict__ out, long E, int nm_out, int64_t o) {
  // 16 bytes of maps at a time (4 FP32 / 2 FP64): the four corners of one chunk in
  // registers, not all NM maps of all four corners (which needed 100 registers and left
  // 2 CTAs per SM, too few warps to hide the gather latency)
  constexpr int CH = (NM * (int)sizeof(T) >= 16) ? 16 / (int)sizeof(T) : NM;
  const T* pa = imap + ((long)B.iu * Nx + B.jl) * NM;
  const T* pb = imap + ((long)B.iu * Nx + B.jr) * NM;
  const T* pc = imap + ((long)B.il * Nx + B.jl) * NM;
  const T* pd = imap + ((long)B.il * Nx + B.jr) * NM;
#pragma unroll 1
  for (int c0 = 0; c0 < NM; c0 += CH) {
    T acc[CH];
    if (B.inside) {
      T a[CH], b[CH], c[CH], d[CH];
      load_pix<T, CH>(pa + c0, a);
      load_pix<T, CH>(pb + c0, b);
      load_pix<T, CH>(pc + c0, c);
      load_pix<T, CH>(pd + c0, d);
#pragma unroll
      for (int q = 0; q < CH; q++) {
        T z = B.w0 * a[q];
        z += B.w1 * b[q];
        z += B.w2 * c[q];
        z += B.w3 * d[q];
        acc[q] = z;
      }
    } else {
#pragma unroll
      for (int q = 0; q < CH; q++) acc[q] = (T)0;
    }
#pragma unroll
    for (int q = 0; q < CH; q++)
      if (c0 + q < nm_out) out[(long)(c0 + q) * E + o] = mag ? (T)-2.5 * mlc_log10(acc[q]) : acc[q];
  }
}

// One warp per track, lanes over epochs; each epoch reads 4 corners x NM interleaved
// values and writes nm_out light-curve values out[q*E + e].
template <typename T, int NM>
__global__ void __launch_bounds__(256) k_sample_tracks_il(const T* __restrict__ imap, int Nx, int Ny, int ntracks,
                                                          const T* __restrict__ x0, const T* __restrict__ y0,
                                                          const T* __restrict__ phi, const T* __restrict__ v,
                                                          const int64_t* __restrict__ off, const T* __restrict__ t,
                                                          int mag, T* __restrict__ out, long E, int nm_out,
                                                          int64_t ebase) {
  const int lane = threadIdx.x & 31;
  const long track = (long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (track >= ntracks) return;
  const TrackGeom<T> g(x0[track], y0[track], phi[track], v[track]);
  const int64_t e0 = off[track], e1 = off[track + 1];
  for (int64_t e = e0 + lane; e < e1; e += 32)
    sample_epoch<T, NM>(imap, Nx, g.at(t[e], Nx, Ny), mag, out, E, nm_out, e - ebase);
}

// FP32 with a contiguous output (width == S, off == 0, W in {4, 8, 16}), npix % 4 == 0 and
// 16-byte aligned maps: tiles of 512 pixels moved as float4 on both sides.
template <int W>
__global__ void __launch_bounds__(256) k_interleave_f4(MapList<float> maps, int nm, long npix,
                                                      float* __restrict__ out) {
  __shared__ __align__(16) float tile[W][516];  // 516: rows stay 16-byte aligned
  const long ntiles = (npix + 511) / 512;
  for (long tb = blockIdx.x; tb < ntiles; tb += gridDim.x) {
    const long p0 = tb * 512;
    const int np = (int)min(512L, npix - p0);  // a multiple of 4
    for (int f = threadIdx.x; f < W * 128; f += 256) {
      const int q = f >> 7, c = (f & 127) * 4;
      float4 val = make_float4(0.f, 0.f, 0.f, 0.f);
      if (q < nm && c < np) val = __ldg(reinterpret_cast<const float4*>(maps.m[q] + p0 + c));
      *reinterpret_cast<float4*>(&tile[q][c]) = val;
    }
    __syncthreads();
    float4* o = reinterpret_cast<float4*>(out + p0 * W);
    const int nf = np * (W / 4);
    for (int f = threadIdx.x; f < nf; f += 256) {
      const int px = f / (W / 4), q0 = (f % (W / 4)) * 4;
      o[f] = make_float4(tile[q0][px], tile[q0 + 1][px], tile[q0 + 2][px], tile[q0 + 3][px]);
    }
    __syncthreads();
  }
}

static bool aligned16(const void* p) { return ((uintptr_t)p & 15) == 0; }

static void interleave_impl(mlc_ctx* ctx, const void* const* maps_host, int nmaps, int width, int S, int off,
                            long npix, int prec, void* out) {
  const int grid = (int)std::min<long>((npix + 255) / 256, (long)ctx->sm_count * 16);
  int wshift = -1;
  for (int b = 0; b < 5; b++)
    if (width == (1 << b)) wshift = b;
  bool fast = prec == MLC_F32 && width == S && off == 0 && (width == 4 || width == 8 || width == 16) &&
              npix % 4 == 0 && aligned16(out);
  for (int q = 0; q < nmaps && fast; q++) fast = aligned16(maps_host[q]);
  if (fast) {
    MapList<float> ml{};
    for (int q = 0; q < nmaps; q++) ml.m[q] = (const float*)maps_host[q];
    const int g = (int)std::min<long>((npix + 511) / 512, (long)ctx->sm_count * 8);
    MLC_KSCOPE(ctx, "interleave");
    if (width == 16) k_interleave_f4<16><<<g, 256, 0, ctx->stream>>>(ml, nmaps, npix, (float*)out);
    else if (width == 8) k_interleave_f4<8><<<g, 256, 0, ctx->stream>>>(ml, nmaps, npix, (float*)out);
    else k_interleave_f4<4><<<g, 256, 0, ctx->stream>>>(ml, nmaps, npix, (float*)out);
    MLC_CHECK_LAUNCH();
    return;
  }
  if (prec == MLC_F64) {
    MapList<double> ml{};
    for (int q = 0; q < nmaps; q++) ml.m[q] = (const double*)maps_host[q];
    MLC_KSCOPE(ctx, "interleave");
    k_interleave<double><<<grid, 256, 0, ctx->stream>>>(ml, nmaps, width, wshift, S, off, npix, (double*)out);
  } else {
    MapList<float> ml{};
    for (int q = 0; q < nmaps; q++) ml.m[q] = (const float*)maps_host[q];
    MLC_KSCOPE(ctx, "interleave");
    k_interleave<float><<<grid, 256, 0, ctx->stream>>>(ml, nmaps, width, wshift, S, off, npix, (float*)out);
  }
  MLC_CHECK_LAUNCH();
}

void interleave(mlc_ctx* ctx, const void* const* maps_host, int nmaps, long npix, int prec, int stride, void* out) {
  interleave_impl(ctx, maps_host, nmaps, stride, stride, 0, npix, prec, out);
}

void interleave_into(mlc_ctx* ctx, const void* const* maps_host, int nmaps, long npix, int prec, int S, int off,
                     void* out) {
  interleave_impl(ctx, maps_host, nmaps, nmaps, S, off, npix, prec, out);
}

// ---- cell order: chunks of 32 consecutive epochs sampled in the order of the map cell
// they start in.  Taking whole tracks in index order, the warps in flight at one moment
// gather from all over the map, and a map much larger than L2 is read several times over;
// chunks of a few days' motion sorted by 128 x 128-pixel cell keep the gathers of the
// warps in flight within a few cells.  Every
// epoch is computed as in k_sample_tracks_il (the same geometry and arithmetic per lane),
// so the light curves are the same bit for bit; only the order of the work changes.
constexpr int CHUNK_EPOCHS = 32;
constexpr int CHUNK_CELL = 128;

// Each track's geometry (TrackGeom: pixel base, offsets, V cos phi, V sin phi), formed once
// per call: a chunk's lanes load it instead of evaluating sin and cos per epoch.
template <typename T>
__global__ void k_il_track_geom(const T* __restrict__ x0, const T* __restrict__ y0, const T* __restrict__ phi,
                                const T* __restrict__ v, int ntracks, TrackGeom<T>* __restrict__ geom) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < ntracks; r += gridDim.x * blockDim.x)
    geom[r] = TrackGeom<T>(x0[r], y0[r], phi[r], v[r]);
}

// first[c]: the track holding the chunk's first epoch (off[0] + 32 c).
__global__ void k_il_chunk_tracks(const int64_t* __restrict__ off, int ntracks, int* __restrict__ first) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < ntracks; r += gridDim.x * blockDim.x) {
    const int64_t b = off[0], a0 = off[r] - b, a1 = off[r + 1] - b;
    for (int64_t c = (a0 + CHUNK_EPOCHS - 1) / CHUNK_EPOCHS; c * CHUNK_EPOCHS < a1; c++) first[c] = r;
  }
}

// The cell of each chunk's first epoch (clamped to the map), and the per-cell counts.
template <typename T>
__global__ void k_il_chunk_cells(const TrackGeom<T>* __restrict__ geom, const int64_t* __restrict__ off,
                                 const T* __restrict__ t, const int* __restrict__ first, int ntracks, long nchunks,
                                 int Nx, int Ny, int ncx, int ncy, uint32_t* __restrict__ cell,
                                 uint32_t* __restrict__ count) {
  for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < nchunks; c += (long)gridDim.x * blockDim.x) {
    const int64_t e = off[0] + c * CHUNK_EPOCHS;
    if (e >= off[ntracks]) {  // past the tracks' epochs (nep above their count): an empty chunk
      cell[c] = 0;
      atomicAdd(count, 1u);
      continue;
    }
    const Bilin<T> B = geom[first[c]].at(t[e], Nx, Ny);
    const int cx = min(max(B.jl, 0) / CHUNK_CELL, ncx - 1), cy = min(max(B.il, 0) / CHUNK_CELL, ncy - 1);
    const uint32_t k = (uint32_t)(cy * ncx + cx);
    cell[c] = k;
    atomicAdd(count + k, 1u);
  }
}

// Exclusive prefix sum of the cell counts (one CTA), then the write cursors of the cells.
__global__ void __launch_bounds__(1024) k_il_cell_scan(uint32_t* __restrict__ count, int ncells) {
  __shared__ uint32_t wsum[32];
  uint32_t running = 0;
  for (int c0 = 0; c0 < ncells; c0 += blockDim.x) {
    const int c = c0 + threadIdx.x;
    const uint32_t v = c < ncells ? count[c] : 0u;
    uint32_t agg;
    const uint32_t ex = block_exclusive_sum(v, &agg, wsum);
    if (c < ncells) count[c] = running + ex;
    running += agg;
    __syncthreads();  // wsum is rewritten by the next round
  }
}

__global__ void k_il_cell_scatter(const uint32_t* __restrict__ cell, long nchunks, uint32_t* __restrict__ cursor,
                                  uint32_t* __restrict__ order) {
  for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < nchunks; c += (long)gridDim.x * blockDim.x)
    order[atomicAdd(cursor + cell[c], 1u)] = (uint32_t)c;
}

// One warp per chunk, in cell order: lane l samples epoch off[0] + 32 c + l of whichever
// track holds it (a chunk spans at most a few tracks: the first, then forward by offsets).
template <typename T, int NM>
__global__ void __launch_bounds__(256) k_sample_chunks_il(const T* __restrict__ imap, int Nx, int Ny, int ntracks,
                                                          const TrackGeom<T>* __restrict__ geom,
                                                          const int64_t* __restrict__ off, const T* __restrict__ t,
                                                          const int* __restrict__ first,
                                                          const uint32_t* __restrict__ order, long nchunks, int mag,
                                                          T* __restrict__ out, long E, int nm_out, int64_t ebase) {
  const int lane = threadIdx.x & 31;
  const long j = (long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (j >= nchunks) return;
  const long c = order[j];
  const int64_t e = off[0] + c * CHUNK_EPOCHS + lane;
  if (e >= off[ntracks]) return;
  int r = first[c];
  while (off[r + 1] <= e) r++;
  const TrackGeom<T> g = geom[r];
  sample_epoch<T, NM>(imap, Nx, g.at(t[e], Nx, Ny), mag, out, E, nm_out, e - ebase);
}

// The sampler's order for these sizes: cell order where the interleaved pixels are at most
// 16 bytes, the map is larger than L2 and there are enough epochs to cover it; track order
// otherwise.  Measured at 10000^2 with 10^6 tracks: 4 FP32 profiles (16-byte pixels) read
// 4.4 GB instead of 7.7 GB from DRAM and run 10 % faster in cell order, while 16 profiles
// (64-byte pixels, where track order already reads the map only about twice) run 8 % slower
// -- their 7 GB of light curves are then written in scattered 128-byte pieces instead of
// track after track.  A pinned "sample_tracks_il cell-order" tune key (0 or 1) decides
// instead; with the autotuner on, large calls (a map above L2 and at least 2^20 epochs)
// time both orders once per size class and keep the faster.
static bool il_cell_heuristic(long npix, int stride, size_t es, int64_t nep) {
  return stride * es <= 16 && (double)npix * stride * es > 256e6 &&
         nep >= 4 * npix / (CHUNK_CELL * CHUNK_CELL) * CHUNK_EPOCHS;
}

template <typename T>
static void sample_il_run(mlc_ctx* ctx, bool cell, const void* imap, int stride, int nmaps, int Nx, int Ny,
                          int ntracks, const void* x0, const void* y0, const void* phi, const void* v,
                          const int64_t* off, const void* t, int mag, void* out, long E, int64_t ebase, int64_t nep) {
  if (nep > 0 && cell) {
    const long nchunks = (long)((nep + CHUNK_EPOCHS - 1) / CHUNK_EPOCHS);
    const int ncx = ceil_div(Nx, CHUNK_CELL), ncy = ceil_div(Ny, CHUNK_CELL), ncells = ncx * ncy;
    MLC_REQUIRE(nchunks < (1L << 32), MLC_ERR_LIMIT, "more than 2^37 epochs in one sampling call");
    const size_t gbytes = ((size_t)ntracks * sizeof(TrackGeom<T>) + 255) & ~(size_t)255;
    char* ws = (char*)ws_get(ctx, WS_SAMPLE_ORDER, gbytes + (size_t)nchunks * 12 + (size_t)ncells * 4 + 256);
    TrackGeom<T>* geom = (TrackGeom<T>*)ws;
    int* first = (int*)(ws + gbytes);
    uint32_t* cell = (uint32_t*)(first + nchunks);
    uint32_t* order = cell + nchunks;
    uint32_t* count = order + nchunks;
    MLC_CUDA(cudaMemsetAsync(count, 0, sizeof(uint32_t) * ncells, ctx->stream));
    const int g = std::max(1, std::min(ctx->sm_count * 8, (int)((nchunks + 255) / 256)));
    {
      MLC_KSCOPE(ctx, "sample_cell_order");
      const int gt = std::max(1, std::min(ctx->sm_count * 8, ceil_div(ntracks, 256)));
      k_il_track_geom<T><<<gt, 256, 0, ctx->stream>>>((const T*)x0, (const T*)y0, (const T*)phi, (const T*)v, ntracks,
                                                      geom);
      k_il_chunk_tracks<<<gt, 256, 0, ctx->stream>>>(off, ntracks, first);
      k_il_chunk_cells<T><<<g, 256, 0, ctx->stream>>>(geom, off, (const T*)t, first, ntracks, nchunks, Nx, Ny, ncx,
                                                       ncy, cell, count);
      k_il_cell_scan<<<1, 1024, 0, ctx->stream>>>(count, ncells);
      k_il_cell_scatter<<<g, 256, 0, ctx->stream>>>(cell, nchunks, count, order);
    }
    MLC_CHECK_LAUNCH();
    const long grid = (nchunks + 7) / 8;
    MLC_REQUIRE(grid <= 0x7fffffffL, MLC_ERR_LIMIT, "too many epochs in one sampling call");
#define MLC_CH_LAUNCH(NMV)                                                                                          \
  k_sample_chunks_il<T, NMV><<<(unsigned)grid, 256, 0, ctx->stream>>>(                                              \
      (const T*)imap, Nx, Ny, ntracks, geom, off, (const T*)t, first, order, nchunks, mag, (T*)out, E, nmaps, ebase)
    MLC_KSCOPE(ctx, "sample_tracks_il");
    switch (stride) {
      case 1: MLC_CH_LAUNCH(1); break;
      case 2: MLC_CH_LAUNCH(2); break;
      case 4: MLC_CH_LAUNCH(4); break;
      case 8: MLC_CH_LAUNCH(8); break;
      default: MLC_CH_LAUNCH(16); break;
    }
#undef MLC_CH_LAUNCH
    return;
  }
  const int grid = ceil_div(ntracks, 8);
#define MLC_IL_LAUNCH(NMV)                                                                                    \
  k_sample_tracks_il<T, NMV><<<grid, 256, 0, ctx->stream>>>((const T*)imap, Nx, Ny, ntracks, (const T*)x0,  \
                                                              (const T*)y0, (const T*)phi, (const T*)v, off, \
                                                              (const T*)t, mag, (T*)out, E, nmaps, ebase)
  MLC_KSCOPE(ctx, "sample_tracks_il");
  switch (stride) {
    case 1: MLC_IL_LAUNCH(1); break;
    case 2: MLC_IL_LAUNCH(2); break;
    case 4: MLC_IL_LAUNCH(4); break;
    case 8: MLC_IL_LAUNCH(8); break;
    default: MLC_IL_LAUNCH(16); break;
  }
#undef MLC_IL_LAUNCH
}

template <typename T>
static void sample_il_impl(mlc_ctx* ctx, const void* imap, int stride, int nmaps, int Nx, int Ny, int ntracks,
                           const void* x0, const void* y0, const void* phi, const void* v, const int64_t* off,
                           const void* t, int mag, void* out, long E, int64_t ebase, int64_t nep) {
  auto run = [&](bool cell) {
    sample_il_run<T>(ctx, cell, imap, stride, nmaps, Nx, Ny, ntracks, x0, y0, phi, v, off, t, mag, out, E, ebase,
                     nep);
  };
  const long npix = (long)Nx * Ny;
  auto pin = ctx->tune.find("sample_tracks_il cell-order");
  if (pin != ctx->tune.end()) return run(pin->second != 0);
  bool cell = il_cell_heuristic(npix, stride, sizeof(T), nep);
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  MLC_CUDA(cudaStreamIsCapturing(ctx->stream, &cs));
  if (ctx->autotune && cs == cudaStreamCaptureStatusNone && (double)npix * stride * sizeof(T) > 256e6 &&
      nep >= (1 << 20)) {
    int lg = 0;
    while ((int64_t)1 << (lg + 1) <= nep) lg++;
    char key[96];
    std::snprintf(key, sizeof key, "sample_tracks_il order %dx%d %s x%d epochs~2^%d", Nx, Ny,
                  sizeof(T) == 8 ? "f64" : "f32", stride, lg);
    auto it = ctx->tune.find(key);
    if (it != ctx->tune.end()) return run(it->second != 0);
    // both orders write the same values: time each once, keep the faster
    const bool saved = ctx->timing;
    ctx->timing = false;
    float ms[2] = {0.f, 0.f};
    cudaEvent_t a = nullptr, b = nullptr;
    try {
      MLC_CUDA(cudaEventCreate(&a));
      MLC_CUDA(cudaEventCreate(&b));
      for (int o = 0; o < 2; o++) {
        MLC_CUDA(cudaEventRecord(a, ctx->stream));
        run(o == 1);
        MLC_CUDA(cudaEventRecord(b, ctx->stream));
        MLC_CUDA(cudaEventSynchronize(b));
        MLC_CUDA(cudaEventElapsedTime(&ms[o], a, b));
      }
    } catch (...) {
      if (a) cudaEventDestroy(a);
      if (b) cudaEventDestroy(b);
      ctx->timing = saved;
      throw;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    ctx->timing = saved;
    cell = ms[1] < ms[0];
    ctx->tune[key] = cell ? 1 : 0;
    ctx->tune_name[key] = cell ? "cell-order" : "track-order";
    char rec[80];
    std::snprintf(rec, sizeof rec, "track-order=%.4f cell-order=%.4f", ms[0], ms[1]);
    ctx->tune_log[key] = rec;
    return;  // the outputs are written (by both runs)
  }
  run(cell);
}

void sample_tracks_il(mlc_ctx* ctx, const void* imap, int stride, int nmaps, int Nx, int Ny, int prec, int ntracks,
                      const void* x0, const void* y0, const void* phi, const void* v, const int64_t* off,
                      const void* t, int mag, void* out, long E, int64_t ebase, int64_t nep) {
  if (ntracks <= 0) return;
  if (prec == MLC_F64)
    sample_il_impl<double>(ctx, imap, stride, nmaps, Nx, Ny, ntracks, x0, y0, phi, v, off, t, mag, out, E, ebase,
                           nep);
  else
    sample_il_impl<float>(ctx, imap, stride, nmaps, Nx, Ny, ntracks, x0, y0, phi, v, off, t, mag, out, E, ebase,
                          nep);
  MLC_CHECK_LAUNCH();
}

// Expanding source: epoch e has its own nbands maps (map s = e*nbands + b, npix pixels
// apart), all tracks share the epochs t[nep]; one thread per (track, epoch) reads its
// bands' four bilinear corners and writes out[i*nep*nbands + e*nbands + b] -- curves as
// rows of nep*nbands values, the layout the pair stage reads.
template <typename T>
__global__ void __launch_bounds__(256) k_sample_expanding(const T* __restrict__ maps, long npix, int Nx, int Ny,
                                                          int nbands, int ntracks, int nep, const T* __restrict__ x0,
                                                          const T* __restrict__ y0, const T* __restrict__ phi,
                                                          const T* __restrict__ v, const T* __restrict__ t, int mag,
                                                          T* __restrict__ out) {
  const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long)ntracks * nep) return;
  const long tr = idx / nep;
  const int e = (int)(idx - tr * nep);
  const Bilin<T> B = TrackGeom<T>(x0[tr], y0[tr], phi[tr], v[tr]).at(t[e], Nx, Ny);
  T* o = out + idx * nbands;
  for (int b = 0; b < nbands; b++) {
    const T mu = B.inside ? bilin_read<T>(maps + (long)(e * nbands + b) * npix, B, Nx) : (T)0;
    o[b] = mag ? (T)-2.5 * mlc_log10(mu) : mu;
  }
}

void sample_expanding(mlc_ctx* ctx, const void* maps, int Nx, int Ny, int prec, int nep, int nbands, int ntracks,
                      const void* x0, const void* y0, const void* phi, const void* v, const void* t, int mag,
                      void* out) {
  const long n = (long)ntracks * nep;
  if (n <= 0) return;
  const int grid = (int)((n + 255) / 256);
  const long npix = (long)Nx * Ny;
  MLC_KSCOPE(ctx, "sample_expanding");
  if (prec == MLC_F64)
    k_sample_expanding<double><<<grid, 256, 0, ctx->stream>>>((const double*)maps, npix, Nx, Ny, nbands, ntracks, nep,
                                                              (const double*)x0, (const double*)y0,
                                                              (const double*)phi, (const double*)v,
                                                              (const double*)t, mag, (double*)out);
  else
    k_sample_expanding<float><<<grid, 256, 0, ctx->stream>>>((const float*)maps, npix, Nx, Ny, nbands, ntracks, nep,
                                                             (const float*)x0, (const float*)y0, (const float*)phi,
                                                             (const float*)v, (const float*)t, mag, (float*)out);
  MLC_CHECK_LAUNCH();
}

// Fused sample -> magnitude -> offset-minimised chi2 of every track against one observed
// curve on shared epochs t[T] (no light curve is written): one warp per track, lanes over
// the epochs.  Pass 1 samples the NM interleaved maps and accumulates sum w (o - m) per
// map (FP64) to get the offset dm = sum w (o - m) / W; pass 2 samples again (the same
// addresses, now L1 hits) and accumulates sum w (o - m - dm)^2, so the chi2 never comes
// from the cancellation-prone single-pass form.  An epoch outside the hull samples 0
// (magnitude +inf) and makes that map's chi2 +inf, as the light curve would.
template <typename T, int NM>
__device__ __forceinline__ void sample_mags(const T* __restrict__ imap, int Nx, const Bilin<T>& B, T* m) {
  if (!B.inside) {
#pragma unroll
    for (int q = 0; q < NM; q++) m[q] = (T)INFINITY;
    return;
  }
  T a[NM], b[NM], c[NM], d[NM];
  load_pix<T, NM>(imap + ((long)B.iu * Nx + B.jl) * NM, a);
  load_pix<T, NM>(imap + ((long)B.iu * Nx + B.jr) * NM, b);
  load_pix<T, NM>(imap + ((long)B.il * Nx + B.jl) * NM, c);
  load_pix<T, NM>(imap + ((long)B.il * Nx + B.jr) * NM, d);
#pragma unroll
  for (int q = 0; q < NM; q++) {
    T z = B.w0 * a[q];
    z += B.w1 * b[q];
    z += B.w2 * c[q];
    z += B.w3 * d[q];
    m[q] = (T)-2.5 * mlc_log10(z);
  }
}

template <typename T, int NM>
__global__ void __launch_bounds__(256) k_track_chi2_offset(const T* __restrict__ imap, int nm_out, int Nx, int Ny,
                                                           int ntracks, const T* __restrict__ x0,
                                                           const T* __restrict__ y0, const T* __restrict__ phi,
                                                           const T* __restrict__ v, int Tn, const T* __restrict__ t,
                                                           const double* __restrict__ obs,
                                                           const double* __restrict__ w,
                                                           double* __restrict__ chi2, double* __restrict__ dm) {
  const int lane = threadIdx.x & 31;
  const long tr = (long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (tr >= ntracks) return;
  const TrackGeom<T> g(x0[tr], y0[tr], phi[tr], v[tr]);
  double s1[NM], s2[NM], W = 0.0;
#pragma unroll
  for (int q = 0; q < NM; q++) s1[q] = s2[q] = 0.0;
  for (int e = lane; e < Tn; e += 32) {
    T m[NM];
    sample_mags<T, NM>(imap, Nx, g.at(t[e], Nx, Ny), m);
    const double we = __ldg(w + e), oe = __ldg(obs + e);
    W += we;
#pragma unroll
    for (int q = 0; q < NM; q++) s1[q] += we * (oe - (double)m[q]);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) W += __shfl_xor_sync(0xffffffffu, W, o);
#pragma unroll
  for (int q = 0; q < NM; q++) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s1[q] += __shfl_xor_sync(0xffffffffu, s1[q], o);
    s1[q] /= W;  // the offset
  }
  for (int e = lane; e < Tn; e += 32) {
    T m[NM];
    sample_mags<T, NM>(imap, Nx, g.at(t[e], Nx, Ny), m);
    const double we = __ldg(w + e), oe = __ldg(obs + e);
#pragma unroll
    for (int q = 0; q < NM; q++) {
      const double r = oe - (double)m[q] - s1[q];
      s2[q] += we * r * r;
    }
  }
#pragma unroll
  for (int q = 0; q < NM; q++) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s2[q] += __shfl_xor_sync(0xffffffffu, s2[q], o);
  }
  if (lane < NM && lane < nm_out) {
    double c = 0.0, d = 0.0;
#pragma unroll
    for (int q = 0; q < NM; q++)
      if (q == lane) {
        c = s2[q];
        d = s1[q];
      }
    chi2[(long)lane * ntracks + tr] = c;
    if (dm) dm[(long)lane * ntracks + tr] = d;
  }
}

template <typename T>
static void track_chi2_offset_impl(mlc_ctx* ctx, const void* imap, int stride, int nmaps, int Nx, int Ny,
                                   int ntracks, const void* x0, const void* y0, const void* phi, const void* v,
                                   int Tn, const void* t, const double* obs, const double* w, double* chi2,
                                   double* dm) {
  const int grid = ceil_div(ntracks, 8);
#define MLC_TC_LAUNCH(NMV)                                                                                   \
  k_track_chi2_offset<T, NMV><<<grid, 256, 0, ctx->stream>>>((const T*)imap, nmaps, Nx, Ny, ntracks,          \
                                                            (const T*)x0, (const T*)y0, (const T*)phi,      \
                                                            (const T*)v, Tn, (const T*)t, obs, w, chi2, dm)
  MLC_KSCOPE(ctx, "track_chi2_offset");
  switch (stride) {
    case 1: MLC_TC_LAUNCH(1); break;
    case 2: MLC_TC_LAUNCH(2); break;
    case 4: MLC_TC_LAUNCH(4); break;
    case 8: MLC_TC_LAUNCH(8); break;
    default: MLC_TC_LAUNCH(16); break;
  }
#undef MLC_TC_LAUNCH
}

void track_chi2_offset(mlc_ctx* ctx, const void* imap, int stride, int nmaps, int Nx, int Ny, int prec, int ntracks,
                       const void* x0, const void* y0, const void* phi, const void* v, int Tn, const void* t,
                       const double* obs, const double* w, double* chi2, double* dm) {
  if (ntracks <= 0) return;
  if (prec == MLC_F64)
    track_chi2_offset_impl<double>(ctx, imap, stride, nmaps, Nx, Ny, ntracks, x0, y0, phi, v, Tn, t, obs, w, chi2, dm);
  else
    track_chi2_offset_impl<float>(ctx, imap, stride, nmaps, Nx, Ny, ntracks, x0, y0, phi, v, Tn, t, obs, w, chi2, dm);
  MLC_CHECK_LAUNCH();
}

// Offset-minimised chi2, one warp per curve, FP64 accumulation:
// dm = sum w (o - m) / W ; chi2 = sum w (o - m - dm)^2 (two passes, no cancellation).
template <typename T>
__global__ void __launch_bounds__(256) k_chi2_offset(int ncurves, int T_, const T* __restrict__ m,
                                                     const double* __restrict__ obs, const double* __restrict__ w,
                                                     double W, double* __restrict__ chi2, double* __restrict__ dm) {
  const int lane = threadIdx.x & 31;
  const long k = (long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (k >= ncurves) return;
  const T* mk = m + k * T_;
  double sr = 0.0;
  for (int e = lane; e < T_; e += 32) sr += __ldg(w + e) * (__ldg(obs + e) - (double)mk[e]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) sr += __shfl_xor_sync(0xffffffffu, sr, o);
  const double off = sr / W;
  double c = 0.0;
  for (int e = lane; e < T_; e += 32) {
    const double r = __ldg(obs + e) - (double)mk[e] - off;
    c += __ldg(w + e) * r * r;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if (lane == 0) {
    chi2[k] = c;
    if (dm) dm[k] = off;
  }
}

void chi2_offset(mlc_ctx* ctx, int prec, int ncurves, int T_, const void* m, const double* obs_dev,
                 const double* w_dev, double W, double* chi2, double* dm) {
  if (ncurves <= 0) return;
  const int grid = ceil_div(ncurves, 8);
  if (prec == MLC_F64)
    {
      MLC_KSCOPE(ctx, "chi2_offset");
      k_chi2_offset<double><<<grid, 256, 0, ctx->stream>>>(ncurves, T_, (const double*)m, obs_dev, w_dev, W, chi2, dm);
    }
  else
    {
      MLC_KSCOPE(ctx, "chi2_offset");
      k_chi2_offset<float><<<grid, 256, 0, ctx->stream>>>(ncurves, T_, (const float*)m, obs_dev, w_dev, W, chi2, dm);
    }
  MLC_CHECK_LAUNCH();
}

}  // namespace mlc
