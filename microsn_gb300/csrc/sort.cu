// Hand-written stable LSD radix sort (8-bit digits) of 64-bit keys carrying 32-bit
// values, and warp-aggregated shared-memory histograms.
//
// Up front, k_digit_hist counts all eight digits of every tile in one read of the keys;
// their totals give each digit's global start and let passes where all keys share a
// digit be skipped.  Then one pass per remaining digit: (1) per-tile counts of that
// digit in the keys' current order (the up-front counts serve the first pass only,
// since each scatter permutes the keys); (2) k_scan_digit turns them into scatter
// offsets; (3) k_scatter ranks each key inside its tile with __match_any_sync in
// element order (stable) and scatters key and value.  Every scatter address is checked
// against n; a violation sets an error flag instead of writing.

#include <mutex>
#include <unordered_map>

#include "mlc_internal.h"
#include "scan.cuh"

namespace mlc {

static constexpr int SORT_THREADS = 256;
static constexpr int SORT_ITEMS = 16;
static constexpr int SORT_TILE = SORT_THREADS * SORT_ITEMS;  // 4096
static constexpr int SORT_WARPS = SORT_THREADS / 32;

// Order-preserving map of an IEEE double to an unsigned key.
__host__ __device__ __forceinline__ uint64_t f64_key(double d) {
  uint64_t u;
  memcpy(&u, &d, 8);
  return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
}

uint64_t f64_to_key(double d) { return f64_key(d); }

// hist layout: [pass][digit][tile]
__global__ void __launch_bounds__(SORT_THREADS) k_digit_hist(const uint64_t* __restrict__ keys, long n,
                                                             int ntiles, uint32_t* __restrict__ hist) {
  __shared__ uint32_t cnt[8][256];
  for (int i = threadIdx.x; i < 8 * 256; i += blockDim.x) (&cnt[0][0])[i] = 0;
  __syncthreads();
  const long t0 = (long)blockIdx.x * SORT_TILE;
  for (int q = 0; q < SORT_ITEMS; q++) {
    const long i = t0 + (long)q * SORT_THREADS + threadIdx.x;
    if (i < n) {
      const uint64_t k = keys[i];
#pragma unroll
      for (int p = 0; p < 8; p++) atomicAdd(&cnt[p][(k >> (8 * p)) & 0xff], 1u);
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < 8 * 256; i += blockDim.x) {
    const int p = i / 256, d = i % 256;
    hist[((long)p * 256 + d) * ntiles + blockIdx.x] = cnt[p][d];
  }
}

// Exclusive scan, in digit-major order, of hist[pass] (256 x ntiles) -> offsets (same
// layout).  One CTA per digit scans that digit's tiles, starting from the digit's
// global base (the count of all keys with a smaller digit, from the host).
__global__ void __launch_bounds__(1024) k_scan_digit(const uint32_t* __restrict__ hist, int ntiles,
                                                     const uint32_t* __restrict__ digit_base,
                                                     uint32_t* __restrict__ offs) {
  __shared__ uint32_t wsum[32];
  const int d = blockIdx.x;
  uint32_t running = digit_base[d];
  for (int t0 = 0; t0 < ntiles; t0 += blockDim.x) {
    const int t = t0 + threadIdx.x;
    const uint32_t v = (t < ntiles) ? hist[(long)d * ntiles + t] : 0;
    uint32_t agg;
    const uint32_t ex = block_exclusive_sum(v, &agg, wsum);
    if (t < ntiles) offs[(long)d * ntiles + t] = running + ex;
    running += agg;
    __syncthreads();  // wsum is rewritten by the next round
  }
}

// Per-tile counts of one digit position in the current key order: hist [digit][tile].
__global__ void __launch_bounds__(SORT_THREADS) k_tile_hist(const uint64_t* __restrict__ keys, long n, int ntiles,
                                                            int shift, uint32_t* __restrict__ hist) {
  __shared__ uint32_t cnt[256];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) cnt[i] = 0;
  __syncthreads();
  const long t0 = (long)blockIdx.x * SORT_TILE;
  for (int q = 0; q < SORT_ITEMS; q++) {
    const long i = t0 + (long)q * SORT_THREADS + threadIdx.x;
    if (i < n) atomicAdd(&cnt[(keys[i] >> shift) & 0xff], 1u);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < 256; d += blockDim.x) hist[(long)d * ntiles + blockIdx.x] = cnt[d];
}

// totals[p*256 + d] = number of keys whose digit p is d
__global__ void __launch_bounds__(256) k_digit_totals(const uint32_t* __restrict__ hist, int ntiles,
                                                      unsigned long long* __restrict__ totals) {
  const long row = blockIdx.x;  // p*256 + d
  unsigned long long s = 0;
  for (int t = threadIdx.x; t < ntiles; t += blockDim.x) s += hist[row * ntiles + t];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  __shared__ unsigned long long red[8];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long t = 0;
    for (int w = 0; w < 8; w++) t += red[w];
    totals[row] = t;
  }
}

__global__ void __launch_bounds__(SORT_THREADS) k_scatter(const uint64_t* __restrict__ kin,
                                                          const uint32_t* __restrict__ vin, uint64_t* __restrict__ kout,
                                                          uint32_t* __restrict__ vout, long n, int ntiles, int shift,
                                                          const uint32_t* __restrict__ offs, int* __restrict__ err) {
  __shared__ uint32_t wcnt[SORT_WARPS][256];  // per-warp running digit counts, then warp bases
  __shared__ uint32_t gbase[256];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int i = threadIdx.x; i < SORT_WARPS * 256; i += blockDim.x) (&wcnt[0][0])[i] = 0;
  for (int i = threadIdx.x; i < 256; i += blockDim.x) gbase[i] = offs[(long)i * ntiles + blockIdx.x];
  __syncthreads();
  // warp w owns tile elements [w*512, (w+1)*512): item q of lane l is element w*512 + 32q + l
  const long t0 = (long)blockIdx.x * SORT_TILE + (long)warp * (SORT_ITEMS * 32);
  uint64_t key[SORT_ITEMS];
  uint32_t rank[SORT_ITEMS];
  const unsigned lt = (1u << lane) - 1u;
#pragma unroll
  for (int q = 0; q < SORT_ITEMS; q++) {
    const long i = t0 + q * 32 + lane;
    const bool ok = i < n;
    key[q] = ok ? kin[i] : ~0ull;
    const unsigned d = ok ? (unsigned)((key[q] >> shift) & 0xff) : 256u;
    const unsigned act = __ballot_sync(0xffffffffu, ok);
    const unsigned peers = __match_any_sync(0xffffffffu, d) & act;
    uint32_t r = 0;
    if (ok) {
      const uint32_t before = wcnt[warp][d];
      r = before + __popc(peers & lt);
    }
    __syncwarp();
    if (ok && (peers & lt) == 0) wcnt[warp][d] += __popc(peers);
    __syncwarp();
    rank[q] = r;
  }
  __syncthreads();
  // exclusive scan of the per-warp counts for each digit -> warp bases
  for (int d = threadIdx.x; d < 256; d += blockDim.x) {
    uint32_t s = 0;
    for (int w = 0; w < SORT_WARPS; w++) {
      const uint32_t c = wcnt[w][d];
      wcnt[w][d] = s;
      s += c;
    }
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < SORT_ITEMS; q++) {
    const long i = t0 + q * 32 + lane;
    if (i < n) {
      const unsigned d = (unsigned)((key[q] >> shift) & 0xff);
      const uint64_t dst = (uint64_t)gbase[d] + wcnt[warp][d] + rank[q];
      if (dst < (uint64_t)n) {
        kout[dst] = key[q];
        vout[dst] = vin[i];
      } else {
        atomicExch(err, 1);
      }
    }
  }
}

// Sorts keys/vals (device, n) stably; uses two workspace buffers.  Result in place.
void radix_sort_u64_u32(mlc_ctx* ctx, long n, uint64_t* keys, uint32_t* vals) {
  if (n <= 1) return;
  MLC_REQUIRE(n <= 0xFFFFFFFFl, MLC_ERR_LIMIT, "sort length above 2^32-1");
  const int ntiles = (int)((n + SORT_TILE - 1) / SORT_TILE);
  uint64_t* k2 = (uint64_t*)ws_get(ctx, WS_SORT_KEYS, sizeof(uint64_t) * n);
  uint32_t* v2 = (uint32_t*)ws_get(ctx, WS_SORT_VALS, sizeof(uint32_t) * n);
  uint32_t* hist = (uint32_t*)ws_get(ctx, WS_SORT_HIST,
                                     sizeof(uint32_t) * (256 * (size_t)ntiles * 9 + 8 * 256) + 8 * 256 * 8 + 64);
  uint32_t* offs = hist + (size_t)8 * 256 * ntiles;
  uint32_t* dbase = offs + (size_t)256 * ntiles;
  unsigned long long* dtot = reinterpret_cast<unsigned long long*>(dbase + 8 * 256);
  int* derr = reinterpret_cast<int*>(dtot + 8 * 256);
  MLC_CUDA(cudaMemsetAsync(derr, 0, sizeof(int), ctx->stream));
  {
    MLC_KSCOPE(ctx, "sort_digit_hist");
    k_digit_hist<<<ntiles, SORT_THREADS, 0, ctx->stream>>>(keys, n, ntiles, hist);
  }
  MLC_CHECK_LAUNCH();
  {
    MLC_KSCOPE(ctx, "sort_digit_totals");
    k_digit_totals<<<8 * 256, 256, 0, ctx->stream>>>(hist, ntiles, dtot);
  }
  MLC_CHECK_LAUNCH();
  // Digit totals to the host: digit bases, and positions where all keys agree are skipped.
  std::vector<unsigned long long> h(8 * 256);
  MLC_CUDA(cudaMemcpyAsync(h.data(), dtot, h.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                           ctx->stream));
  MLC_CUDA(cudaStreamSynchronize(ctx->stream));
  std::vector<uint32_t> base(8 * 256);
  std::vector<char> trivial(8, 0);
  for (int p = 0; p < 8; p++) {
    uint64_t run = 0;
    for (int d = 0; d < 256; d++) {
      const uint64_t tot = h[p * 256 + d];
      base[p * 256 + d] = (uint32_t)run;
      run += tot;
      if (tot == (uint64_t)n) trivial[p] = 1;
    }
  }
  MLC_CUDA(cudaMemcpy(dbase, base.data(), base.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
  uint64_t* ka = keys;
  uint32_t* va = vals;
  uint64_t* kb = k2;
  uint32_t* vb = v2;
  bool first = true;
  for (int p = 0; p < 8; p++) {
    if (trivial[p]) continue;
    if (!first) {  // per-tile counts of digit p in the current order
      MLC_KSCOPE(ctx, "sort_tile_hist");
      k_tile_hist<<<ntiles, SORT_THREADS, 0, ctx->stream>>>(ka, n, ntiles, 8 * p, hist + (size_t)p * 256 * ntiles);
    }
    MLC_CHECK_LAUNCH();
    first = false;
    {
      MLC_KSCOPE(ctx, "sort_scan");
      k_scan_digit<<<256, 1024, 0, ctx->stream>>>(hist + (size_t)p * 256 * ntiles, ntiles, dbase + p * 256, offs);
    }
    MLC_CHECK_LAUNCH();
    {
      MLC_KSCOPE(ctx, "sort_scatter");
      k_scatter<<<ntiles, SORT_THREADS, 0, ctx->stream>>>(ka, va, kb, vb, n, ntiles, 8 * p, offs, derr);
    }
    MLC_CHECK_LAUNCH();
    std::swap(ka, kb);
    std::swap(va, vb);
  }
  if (ka != keys) {
    MLC_CUDA(cudaMemcpyAsync(keys, ka, sizeof(uint64_t) * n, cudaMemcpyDeviceToDevice, ctx->stream));
    MLC_CUDA(cudaMemcpyAsync(vals, va, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, ctx->stream));
  }
  int herr = 0;
  MLC_CUDA(cudaMemcpyAsync(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  MLC_CUDA(cudaStreamSynchronize(ctx->stream));
  MLC_REQUIRE(herr == 0, MLC_ERR_CUDA, "radix sort: scatter offset out of range (inconsistent digit counts)");
}

__global__ void k_f64_to_keys(double* __restrict__ v, long n) {
  uint64_t* u = reinterpret_cast<uint64_t*>(v);
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    u[i] = f64_key(v[i]);
}
__global__ void k_keys_to_f64(double* __restrict__ v, long n) {
  uint64_t* u = reinterpret_cast<uint64_t*>(v);
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    uint64_t k = u[i];
    uint64_t b = (k & 0x8000000000000000ull) ? (k & 0x7fffffffffffffffull) : ~k;
    double d;
    memcpy(&d, &b, 8);
    v[i] = d;
  }
}

void sort_f64_u32(mlc_ctx* ctx, long n, double* keys, uint32_t* vals) {
  if (n <= 1) return;
  const int grid = (int)std::min<long>((n + 255) / 256, (long)ctx->sm_count * 16);
  {
    MLC_KSCOPE(ctx, "sort_keys_in");
    k_f64_to_keys<<<grid, 256, 0, ctx->stream>>>(keys, n);
  }
  MLC_CHECK_LAUNCH();
  radix_sort_u64_u32(ctx, n, reinterpret_cast<uint64_t*>(keys), vals);
  {
    MLC_KSCOPE(ctx, "sort_keys_out");
    k_keys_to_f64<<<grid, 256, 0, ctx->stream>>>(keys, n);
  }
  MLC_CHECK_LAUNCH();
}

// Histogram with warp-aggregated shared-memory counters; counts (uint64, nbins) must
// be zeroed by the caller.
__global__ void __launch_bounds__(256) k_hist_f64(const double* __restrict__ v, long n, int nbins, double lo,
                                                  double width, int logscale, unsigned long long* __restrict__ counts) {
  extern __shared__ uint32_t hs[];
  for (int i = threadIdx.x; i < nbins; i += blockDim.x) hs[i] = 0;
  __syncthreads();
  const unsigned lt = (1u << (threadIdx.x & 31)) - 1u;
  for (long base = blockIdx.x * (long)blockDim.x; base < n; base += (long)gridDim.x * blockDim.x) {
    const long i = base + threadIdx.x;
    int b = -1;
    if (i < n) {
      double x = v[i];
      bool ok = true;
      if (logscale) {
        ok = x > 0;
        x = ok ? log10(x) : 0.0;
      }
      const double hi = lo + width * nbins;
      if (ok && x >= lo && x < hi) {
        b = (int)floor((x - lo) / width);
        b = b < 0 ? 0 : (b >= nbins ? nbins - 1 : b);
      }
    }
    const unsigned peers = __match_any_sync(0xffffffffu, b);
    if (b >= 0 && (peers & lt) == 0) atomicAdd(&hs[b], (uint32_t)__popc(peers));
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nbins; i += blockDim.x)
    if (hs[i]) atomicAdd(&counts[i], (unsigned long long)hs[i]);
}

void histogram_f64(mlc_ctx* ctx, long n, const double* v, int nbins, double lo, double hi, int logscale,
                   unsigned long long* counts_dev) {
  MLC_CUDA(cudaMemsetAsync(counts_dev, 0, sizeof(unsigned long long) * nbins, ctx->stream));
  if (n <= 0) return;
  const size_t smem = sizeof(uint32_t) * nbins;
  set_max_smem((const void*)k_hist_f64, smem);
  const int grid = (int)std::min<long>((n + 255) / 256, (long)ctx->sm_count * 8);
  {
    MLC_KSCOPE(ctx, "histogram");
    k_hist_f64<<<grid, 256, smem, ctx->stream>>>(v, n, nbins, lo, (hi - lo) / nbins, logscale, counts_dev);
  }
  MLC_CHECK_LAUNCH();
}

}  // namespace mlc

// ---------------------------------------------------------------- histogram without allocation
//
// For callers that must not allocate device memory: code running while another
// framework has reserved the whole device memory pool for its own allocator, and host
// callbacks and plugins that may only use the buffers they were handed.  The per-bin
// counters live in a fixed file-scope device array instead of the
// context's workspace, so this entry point calls no cudaMalloc, cudaFree or allocating
// library routine.  The array is loaded with the library and stays allocated on every
// device that loads it until the process exits.
namespace mlc {
namespace {

constexpr int kNoAllocMaxBins = 12000;  // 96 KB of uint64 counters per device
static __device__ __align__(256) unsigned long long g_noalloc_hist[kNoAllocMaxBins];

std::mutex g_noalloc_mu;
std::unordered_map<int, void*> g_noalloc_addr;  // device ordinal -> device address of the array

// Device address of the array on the current device, resolved once per device.  In host
// code the symbol is only a host-side stand-in, never a device address.
void* noalloc_counters(int device) {
  std::lock_guard<std::mutex> g(g_noalloc_mu);
  auto it = g_noalloc_addr.find(device);
  if (it != g_noalloc_addr.end()) return it->second;
  void* p = nullptr;
  MLC_CUDA(cudaGetSymbolAddress(&p, g_noalloc_hist));
  g_noalloc_addr[device] = p;
  return p;
}

}  // namespace
}  // namespace mlc

extern "C" int mlc_histogram_f64_noalloc(mlc_ctx* ctx, long n, const double* v, int nbins, double lo, double hi,
                                         int logscale, uint64_t* counts_host) {
  using namespace mlc;
  if (!ctx) return MLC_ERR_ARG;
  if ((n > 0 && !v) || !counts_host || n < 0 || !(hi > lo)) {
    ctx->err = "mlc_histogram_f64_noalloc: null pointer, negative n or hi <= lo";
    return MLC_ERR_ARG;
  }
  if (nbins < 1 || nbins > kNoAllocMaxBins) {
    ctx->err = "mlc_histogram_f64_noalloc: nbins must be in [1, 12000] (fixed counter array)";
    return MLC_ERR_LIMIT;
  }
  try {
    DeviceGuard g(ctx->device);
    unsigned long long* counts = (unsigned long long*)noalloc_counters(ctx->device);
    // the array keeps the previous call's counts: clear the bins this call uses
    MLC_CUDA(cudaMemsetAsync(counts, 0, sizeof(unsigned long long) * nbins, ctx->stream));
    if (n > 0) {
      const size_t smem = sizeof(uint32_t) * nbins;
      set_max_smem((const void*)k_hist_f64, smem);
      const int grid = (int)std::min<long>((n + 255) / 256, (long)ctx->sm_count * 8);
      {
        MLC_KSCOPE(ctx, "histogram_noalloc");
        k_hist_f64<<<grid, 256, smem, ctx->stream>>>(v, n, nbins, lo, (hi - lo) / nbins, logscale, counts);
      }
      MLC_CHECK_LAUNCH();
    }
    MLC_CUDA(cudaMemcpyAsync(counts_host, counts, sizeof(uint64_t) * nbins, cudaMemcpyDeviceToHost, ctx->stream));
    MLC_CUDA(cudaStreamSynchronize(ctx->stream));
    return MLC_OK;
  } catch (const Error& e) {
    ctx->err = e.what();
    return e.code;
  }
}
