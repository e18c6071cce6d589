// Magnification probability distributions of maps (Mpd) on the GPU.
//
//   mlc_map_binned_mpd  MagnificationMap::getBinnedMpd (magnification_map_gpu.cu:45-87)
//                       sorts every pixel of the map (thrust::sort of Nx*Ny doubles), then
//                       binary-searches the bin edges.  Here one pass over the map: each
//                       pixel in [min, max) goes to the first bin whose right edge is >= it
//                       (what upper_bound + adjacent_difference compute), guessed from
//                       log10 and corrected against the exact edges; shared-memory
//                       counters with warp-aggregated increments.
//   mlc_mpd_divide      Mpd::divide_by (mpd.cpp:71-107), O(NR * NB * NA) on one host core
//                       in the reference: one thread per (ratio bin, B bin) locating the
//                       interval of A by binary search, then one thread per ratio bin for
//                       the trapezium sum in the reference's order.  Every FP64 operation
//                       is rounded on its own (no fused multiply-add), so the result is
//                       bit-identical to the reference's host arithmetic.
#include <cfloat>
#include <cmath>
#include <vector>

#include "mlc_internal.h"

namespace mlc {

constexpr int MPD_MAX_BINS = 16000;

// Largest float <= x and smallest float >= x: for a float v, v <= x  <=>  v <= down(x)
// and v >= x  <=>  v >= up(x), so FP32 pixels are compared exactly with FP64 edges.
static float f32_down(double x) {
  float f = (float)x;
  if ((double)f > x) f = std::nextafter(f, -INFINITY);
  return f;
}
static float f32_up(double x) {
  float f = (float)x;
  if ((double)f < x) f = std::nextafter(f, INFINITY);
  return f;
}

// Positive floating-point values order like their bit patterns read as signed integers,
// and every value outside (0, +inf) falls outside [vmin, vmax) as an integer too (negative
// values and -0.0 read negative, +inf and NaN above vmax's bits): the range test and the
// edge search below are integer compares, with results identical to FP64 compares -- GB300's
// FP64 pipe is narrow, and this kernel made one to three FP64 compares per pixel.
__device__ __forceinline__ long long order_bits(double v) { return __double_as_longlong(v); }
__device__ __forceinline__ int order_bits(float v) { return __float_as_int(v); }

// log2 of a positive value, within 0.09, from its exponent and leading mantissa bits: a
// guess of the bin (off by a few bins) that the exact edge search then corrects.
__device__ __forceinline__ float log2_guess(long long b) {
  return (float)((int)(b >> 32) - (1023 << 20)) * 0x1p-20f;
}
__device__ __forceinline__ float log2_guess(int b) { return (float)(b - (127 << 23)) * 0x1p-23f; }

template <typename T>
__global__ void __launch_bounds__(512) k_binned_mpd(const T* __restrict__ data, long npix, int nb,
                                                    const T* __restrict__ edges, T vmin, T vmax, float logmin,
                                                    float inv_dl, unsigned long long* __restrict__ counts) {
  using B = decltype(order_bits(T()));
  extern __shared__ unsigned char smem_raw[];
  B* e = reinterpret_cast<B*>(smem_raw);
  uint32_t* c = reinterpret_cast<uint32_t*>(e + nb);
  for (int i = threadIdx.x; i < nb; i += blockDim.x) {
    e[i] = order_bits(edges[i]);
    c[i] = 0;
  }
  __syncthreads();
  const B lo = order_bits(vmin), hi = order_bits(vmax);  // vmin > 0
  const float ga = 0.30102999566398120f * inv_dl, gb = -logmin * inv_dl;  // bins per log2, offset
  const unsigned lt = (1u << (threadIdx.x & 31)) - 1u;
  for (long base = blockIdx.x * (long)blockDim.x; base < npix; base += (long)gridDim.x * blockDim.x) {
    const long p = base + threadIdx.x;
    int bin = -1;
    if (p < npix) {
      const B v = order_bits(data[p]);
      if (v >= lo && v < hi) {
        const float g = fmaf(log2_guess(v), ga, gb);
        int i = g < 0.f ? 0 : (g > (float)nb ? nb : (int)g);
        while (i > 0 && v <= e[i - 1]) i--;
        while (i < nb && v > e[i]) i++;
        bin = i < nb ? i : -1;  // above the last edge: dropped, as in the reference
      }
    }
    const unsigned peers = __match_any_sync(0xffffffffu, bin);
    if (bin >= 0 && (peers & lt) == 0) atomicAdd(&c[bin], (uint32_t)__popc(peers));
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nb; i += blockDim.x)
    if (c[i]) atomicAdd(&counts[i], (unsigned long long)c[i]);
}

void map_binned_mpd(mlc_ctx* ctx, const mlc_map* map, int nb, double mn, double mx, double* bins_host,
                    double* counts_host) {
  MLC_REQUIRE(nb >= 1 && nb <= MPD_MAX_BINS, MLC_ERR_LIMIT, "binned MPD supports 1..16000 bins");
  MLC_REQUIRE(mn > 0 && mx > mn, MLC_ERR_ARG, "binned MPD needs 0 < min < max");
  MLC_REQUIRE(mlc_bin_edges(nb, mn, mx, 1, bins_host) == MLC_OK, MLC_ERR_ARG, "bad MPD range");
  const long npix = (long)map->Nx * map->Ny;
  const double lmin = std::log10(mn), dl = (std::log10(mx) - lmin) / nb;
  // device buffers: edges (map precision) then counters
  const size_t es = map->prec == MLC_F64 ? 8 : 4;
  char* ws = (char*)ws_get(ctx, WS_SMALL, round_up((long)nb * es, 256) + (size_t)nb * 8);
  void* d_edges = ws;
  auto* d_counts = reinterpret_cast<unsigned long long*>(ws + round_up((long)nb * es, 256));
  std::vector<float> ef;
  if (map->prec == MLC_F64) {
    MLC_CUDA(cudaMemcpyAsync(d_edges, bins_host, nb * 8, cudaMemcpyHostToDevice, ctx->stream));
  } else {
    ef.resize(nb);
    for (int i = 0; i < nb; i++) ef[i] = f32_down(bins_host[i]);
    MLC_CUDA(cudaMemcpyAsync(d_edges, ef.data(), nb * 4, cudaMemcpyHostToDevice, ctx->stream));
  }
  MLC_CUDA(cudaMemsetAsync(d_counts, 0, (size_t)nb * 8, ctx->stream));
  const size_t smem = (size_t)nb * (es + 4);
  const int grid = (int)std::min<long>((npix + 511) / 512, (long)ctx->sm_count * 4);
  if (map->prec == MLC_F64) {
    set_max_smem((const void*)k_binned_mpd<double>, smem);
    MLC_KSCOPE(ctx, "binned_mpd");
    k_binned_mpd<double><<<grid, 512, smem, ctx->stream>>>((const double*)map->data, npix, nb,
                                                           (const double*)d_edges, mn, mx, (float)lmin,
                                                           (float)(1.0 / dl), d_counts);
  } else {
    set_max_smem((const void*)k_binned_mpd<float>, smem);
    MLC_KSCOPE(ctx, "binned_mpd");
    k_binned_mpd<float><<<grid, 512, smem, ctx->stream>>>((const float*)map->data, npix, nb, (const float*)d_edges,
                                                          f32_up(mn), f32_up(mx), (float)lmin, (float)(1.0 / dl),
                                                          d_counts);
  }
  MLC_CHECK_LAUNCH();
  std::vector<unsigned long long> h(nb);
  MLC_CUDA(cudaMemcpyAsync(h.data(), d_counts, (size_t)nb * 8, cudaMemcpyDeviceToHost, ctx->stream));
  MLC_CUDA(cudaStreamSynchronize(ctx->stream));
  // magnification_map_gpu.cu:76-83
  for (int i = 0; i < nb; i++)
    counts_host[i] = h[i] < 1 ? 1.0 / (double)npix : (double)h[i] / (double)npix;
}

// terms[i * NB + b] = muB * pA(z_i * muB) * pB(muB)  (mpd.cpp:78-97)
__global__ void __launch_bounds__(256) k_mpd_terms(int NA, const double* __restrict__ bA, const double* __restrict__ cA,
                                                   int NB, const double* __restrict__ bB,
                                                   const double* __restrict__ cB, int NR,
                                                   const double* __restrict__ bR, double* __restrict__ terms) {
  const long idx = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (idx >= (long)NR * NB) return;
  const int i = (int)(idx / NB), b = (int)(idx - (long)i * NB);
  const double muB = bB[b];
  const double prod = __dmul_rn(bR[i], muB);
  double pA;
  if (prod <= bA[0] || prod >= bA[NA - 1]) {
    pA = 1e-8;
  } else {
    int lo = 0, hi = NA;  // first edge > prod: the reference's linear scan finds the same k
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (bA[mid] <= prod) lo = mid + 1;
      else hi = mid;
    }
    const int k = lo;
    pA = __dadd_rn(cA[k - 1], __ddiv_rn(__dmul_rn(__dsub_rn(cA[k], cA[k - 1]), __dsub_rn(prod, bA[k - 1])),
                                        __dsub_rn(bA[k], bA[k - 1])));
  }
  terms[idx] = __dmul_rn(__dmul_rn(muB, pA), cB[b]);
}

// ratio[i] = sum_b (t[b-1] + t[b]) (bB[b] - bB[b-1]) / 2 in the reference's order (mpd.cpp:99-103)
__global__ void __launch_bounds__(128) k_mpd_trapz(int NB, const double* __restrict__ bB, int NR,
                                                   const double* __restrict__ terms, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= NR) return;
  const double* t = terms + (long)i * NB;
  double s = 0.0;
  for (int b = 1; b < NB; b++)
    s = __dadd_rn(s, __ddiv_rn(__dmul_rn(__dadd_rn(t[b - 1], t[b]), __dsub_rn(bB[b], bB[b - 1])), 2.0));
  out[i] = s;
}

void mpd_divide(mlc_ctx* ctx, int NA, const double* bA, const double* cA, int NB, const double* bB,
                const double* cB, int NR, const double* bR, double* cR) {
  MLC_REQUIRE(NA >= 1 && NB >= 1 && NR >= 1, MLC_ERR_ARG, "empty Mpd");
  const size_t na = round_up((long)NA * 8, 256), nb = round_up((long)NB * 8, 256), nr = round_up((long)NR * 8, 256);
  const size_t nt = (size_t)NR * NB * 8;
  char* ws = (char*)ws_get(ctx, WS_SMALL, 2 * na + 2 * nb + 2 * nr + nt);
  double* d_bA = (double*)ws;
  double* d_cA = (double*)(ws + na);
  double* d_bB = (double*)(ws + 2 * na);
  double* d_cB = (double*)(ws + 2 * na + nb);
  double* d_bR = (double*)(ws + 2 * na + 2 * nb);
  double* d_out = (double*)(ws + 2 * na + 2 * nb + nr);
  double* d_t = (double*)(ws + 2 * na + 2 * nb + 2 * nr);
  auto up = [&](double* d, const double* h, int n) {
    MLC_CUDA(cudaMemcpyAsync(d, h, (size_t)n * 8, cudaMemcpyHostToDevice, ctx->stream));
  };
  up(d_bA, bA, NA);
  up(d_cA, cA, NA);
  up(d_bB, bB, NB);
  up(d_cB, cB, NB);
  up(d_bR, bR, NR);
  const long n = (long)NR * NB;
  {
    MLC_KSCOPE(ctx, "mpd_divide_terms");
    k_mpd_terms<<<(int)((n + 255) / 256), 256, 0, ctx->stream>>>(NA, d_bA, d_cA, NB, d_bB, d_cB, NR, d_bR, d_t);
  }
  MLC_CHECK_LAUNCH();
  {
    MLC_KSCOPE(ctx, "mpd_divide_sum");
    k_mpd_trapz<<<(NR + 127) / 128, 128, 0, ctx->stream>>>(NB, d_bB, NR, d_t, d_out);
  }
  MLC_CHECK_LAUNCH();
  MLC_CUDA(cudaMemcpyAsync(cR, d_out, (size_t)NR * 8, cudaMemcpyDeviceToHost, ctx->stream));
  MLC_CUDA(cudaStreamSynchronize(ctx->stream));
}

}  // namespace mlc
