// Direct tiled convolution for small profiles, and the context's launch autotuner.
//
// The FFT convolution costs the same per profile whatever the profile's size; a profile
// of N x N pixels convolved directly costs N^2 FMAs per pixel.  For N up to a few tens of
// pixels (in FP32: GB300's FP64 rate makes the direct form lose at every size) the direct
// form can win.  It computes the same circular convolution as the FFT path with the
// reference's kernel wrap (magnification_map.cpp:172-193: profile centre at (0,0), half-
// pixel shift included):
//     out[y][x] = sum_{i,j < N} P[i][j] map[(y - i + h) mod Ny][(x - j + h) mod Nx],  h = N/2.
// A CTA of 16 x 16 threads owns an output tile of (16 RX) x (16 RY) pixels: the map tile
// with its wrapped halo and the flipped profile Q[a][b] = P[N-1-a][N-1-b] are staged in
// shared memory, and each thread accumulates RY x RX outputs in registers,
//     out[oy][ox] = sum_{a,b} Q[a][b] S[oy + a][ox + b],
// looping over the tile rows it reads: each 2 RX-wide segment of a tile row, loaded once
// (float4), feeds the RX x RX FMAs of every output row it contributes to (profile row
// a = tile row - output row), so shared-memory traffic per FMA falls with RY.
//
// Which form runs, and which tile shape, is decided per (map size, profile size) by the
// autotuner: the first call with a new key times every candidate once (after one
// warm-up launch, CUDA events on the context's stream) and keeps the fastest; later calls
// reuse the choice.  Candidates differ only in launch shape or in the form of the
// convolution, all within the FP32 tolerance of the FP64 oracle.  Tuning synchronises
// the stream, so it is skipped (FFT form, nothing cached) while the stream is being
// captured into a CUDA graph.  mlc_ctx_set_autotune(ctx, 0) fixes the FFT form.
#include <algorithm>
#include <cstdio>
#include <functional>
#include <string>

#include "mlc_internal.h"

namespace mlc {

constexpr int DIRECT_MAX_N = 32;

template <typename T, int RX, int RY>
__global__ void __launch_bounds__(256) k_conv_direct(const T* __restrict__ map, int Nx, int Ny,
                                                     const double* __restrict__ prof, int N, T* __restrict__ out) {
  static_assert(sizeof(T) == 4 && RX % 4 == 0, "FP32, whole float4 segments");
  constexpr int TW = 16 * RX, TH = 16 * RY;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int NP = (N + RX - 1) / RX * RX;  // profile columns padded with zeros to whole RX blocks
  const int SW = TW + NP;                 // tile row width (>= TW + NP - 1; a multiple of 4)
  T* S = reinterpret_cast<T*>(smem_raw);
  T* Q = S + (size_t)(TH + N - 1) * SW;
  const int tid = threadIdx.y * 16 + threadIdx.x;
  const int x0 = blockIdx.x * TW, y0 = blockIdx.y * TH;
  const int h = N / 2;
  for (int idx = tid; idx < N * NP; idx += 256) {
    const int a = idx / NP, b = idx - a * NP;
    Q[idx] = b < N ? (T)prof[(long)(N - 1 - a) * N + (N - 1 - b)] : T(0);
  }
  // tile with its halo, one warp per tile row (128-byte reads).  The halo starts at most
  // N - 1 < 32 <= Nx, Ny pixels before the map, so one add wraps it; a partial edge tile
  // may run a whole map past the end (its extra rows feed no output), hence the modulo
  // there
  const int oy0 = y0 + h - (N - 1), ox0 = x0 + h - (N - 1);
  const int rows = TH + N - 1;
  // (all loads of two rows issued before their stores: many reads in flight per warp)
  const int lane = tid & 31, wid = tid >> 5;
  constexpr int MAXC = (TW + DIRECT_MAX_N + 31) / 32;  // SW <= TW + 32
  for (int r0 = wid; r0 < rows; r0 += 16) {
    T v[2][MAXC];
#pragma unroll
    for (int k = 0; k < 2; k++) {
      const int r = r0 + 8 * k;
      int gy = oy0 + (r < rows ? r : 0);
      gy += gy < 0 ? Ny : 0;
      if (gy >= Ny) gy %= Ny;
      const T* mrow = map + (long)gy * Nx;
#pragma unroll
      for (int i = 0; i < MAXC; i++) {
        const int c = lane + 32 * i;
        int gx = ox0 + (c < SW ? c : 0);
        gx += gx < 0 ? Nx : 0;
        if (gx >= Nx) gx %= Nx;
        v[k][i] = (r < rows && c < SW) ? __ldg(mrow + gx) : T(0);
      }
    }
#pragma unroll
    for (int k = 0; k < 2; k++) {
      const int r = r0 + 8 * k;
      if (r >= rows) continue;
#pragma unroll
      for (int i = 0; i < MAXC; i++) {
        const int c = lane + 32 * i;
        if (c < SW) S[(size_t)r * SW + c] = v[k][i];
      }
    }
  }
  __syncthreads();
  // thread (tx, ty): outputs rows oy .. oy+RY-1, columns ox .. ox+RX-1.  Loop over the tile
  // rows it reads: tile row oy + ir feeds output row r through profile row a = ir - r, so
  // each loaded segment serves up to RY rows of FMAs.
  const int ox = threadIdx.x * RX, oy = threadIdx.y * RY;
  T acc[RY][RX];
#pragma unroll
  for (int r = 0; r < RY; r++)
#pragma unroll
    for (int c = 0; c < RX; c++) acc[r][c] = T(0);
  for (int ir = 0; ir < RY + N - 1; ir++) {
    const T* srow = S + (size_t)(oy + ir) * SW + ox;
    for (int b0 = 0; b0 < NP; b0 += RX) {
      T w[2 * RX];
#pragma unroll
      for (int u = 0; u < 2 * RX; u += 4) *reinterpret_cast<float4*>(w + u) = *reinterpret_cast<const float4*>(srow + b0 + u);
#pragma unroll
      for (int r = 0; r < RY; r++) {
        const int a = ir - r;
        if (a < 0 || a >= N) continue;  // uniform across the CTA
        T q[RX];
#pragma unroll
        for (int u = 0; u < RX; u += 4) *reinterpret_cast<float4*>(q + u) = *reinterpret_cast<const float4*>(Q + a * NP + b0 + u);
#pragma unroll
        for (int bb = 0; bb < RX; bb++)
#pragma unroll
          for (int c = 0; c < RX; c++) acc[r][c] = fmaf(q[bb], w[c + bb], acc[r][c]);
      }
    }
  }
#pragma unroll
  for (int r = 0; r < RY; r++) {
    const int y = y0 + oy + r;
    if (y >= Ny) continue;
#pragma unroll
    for (int c = 0; c < RX; c++) {
      const int x = x0 + ox + c;
      if (x < Nx) out[(long)y * Nx + x] = acc[r][c];
    }
  }
}

namespace {

using DirectKernel = void (*)(const float*, int, int, const double*, int, float*);

struct DirectVariant {
  DirectKernel k;
  int RX, RY;
  const char* name;
};

const DirectVariant kVariants[] = {
    {k_conv_direct<float, 4, 4>, 4, 4, "direct_4x4"},
    {k_conv_direct<float, 4, 8>, 4, 8, "direct_4x8"},
    {k_conv_direct<float, 8, 4>, 8, 4, "direct_8x4"},
    {k_conv_direct<float, 8, 8>, 8, 8, "direct_8x8"},
};
constexpr int kNumVariants = sizeof(kVariants) / sizeof(kVariants[0]);

size_t direct_smem(const DirectVariant& v, int N) {
  const int NP = (N + v.RX - 1) / v.RX * v.RX;
  return ((size_t)(16 * v.RY + N - 1) * (16 * v.RX + NP) + (size_t)N * NP) * sizeof(float);
}

}  // namespace

void conv_direct(mlc_ctx* ctx, const FftPlan2D& p, const void* map, const double* prof, int pN, int variant,
                 void* out) {
  MLC_REQUIRE(p.prec == MLC_F32 && pN >= 2 && pN <= DIRECT_MAX_N && variant >= 0 && variant < kNumVariants,
              MLC_ERR_ARG, "direct convolution: FP32 maps and profiles of 2..32 pixels");
  MLC_REQUIRE(p.Nx >= DIRECT_MAX_N && p.Ny >= DIRECT_MAX_N, MLC_ERR_LIMIT,
              "direct convolution: maps of at least 32 x 32 pixels");
  const DirectVariant& v = kVariants[variant];
  const size_t smem = direct_smem(v, pN);
  set_max_smem((const void*)v.k, smem);
  dim3 grid(ceil_div(p.Nx, 16 * v.RX), ceil_div(p.Ny, 16 * v.RY));
  {
    MLC_KSCOPE(ctx, "conv_direct");
    v.k<<<grid, dim3(16, 16), smem, ctx->stream>>>((const float*)map, p.Nx, p.Ny, prof, pN, (float*)out);
  }
  MLC_CHECK_LAUNCH();
}

static float time_on_stream(mlc_ctx* ctx, const std::function<void()>& f) {
  cudaEvent_t a, b;
  MLC_CUDA(cudaEventCreate(&a));
  MLC_CUDA(cudaEventCreate(&b));
  f();  // warm-up (workspaces, smem attributes, caches)
  MLC_CUDA(cudaEventRecord(a, ctx->stream));
  f();
  MLC_CUDA(cudaEventRecord(b, ctx->stream));
  MLC_CUDA(cudaEventSynchronize(b));
  float ms = 0.f;
  MLC_CUDA(cudaEventElapsedTime(&ms, a, b));
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return ms;
}

int conv_direct_choice(mlc_ctx* ctx, const FftPlan2D& p, const void* map, const void* Fmap, const double* prof,
                       int pN, void* out, bool spectrum) {
  if (!ctx->autotune || p.prec != MLC_F32 || pN > DIRECT_MAX_N || pN < 2 || !map || p.Nx < DIRECT_MAX_N ||
      p.Ny < DIRECT_MAX_N)
    return -1;
  char key[96];
  std::snprintf(key, sizeof key, "conv f32 %dx%d N%d%s", p.Nx, p.Ny, pN, spectrum ? " spectrum" : "");
  auto it = ctx->tune.find(key);
  if (it != ctx->tune.end()) return it->second >= -1 && it->second < kNumVariants ? it->second : -1;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  MLC_CUDA(cudaStreamIsCapturing(ctx->stream, &cs));
  if (cs != cudaStreamCaptureStatusNone) return -1;
  // candidate -1: the fused FFT convolution; 0..: the direct tile shapes
  struct TimingOff {  // tuning launches stay out of the per-kernel timings
    mlc_ctx* c;
    bool saved;
    ~TimingOff() { c->timing = saved; }
  } off{ctx, ctx->timing};
  ctx->timing = false;
  std::vector<std::pair<int, float>> ms;
  // the FFT form as the caller would run it: through P3, or up to the half-spectrum that a
  // later pass shared by several profiles takes further
  ms.emplace_back(-1, time_on_stream(ctx, [&] {
                    if (spectrum) conv_fused_spectrum(ctx, p, Fmap, prof, pN, out);
                    else conv_fused(ctx, p, Fmap, prof, pN, out);
                  }));
  for (int v = 0; v < kNumVariants; v++)
    ms.emplace_back(v, time_on_stream(ctx, [&] { conv_direct(ctx, p, map, prof, pN, v, out); }));
  const auto best = *std::min_element(ms.begin(), ms.end(),
                                      [](const auto& x, const auto& y) { return x.second < y.second; });
  ctx->tune[key] = best.first;
  ctx->tune_name[key] = best.first < 0 ? "fft" : kVariants[best.first].name;
  std::string rec;
  for (const auto& m : ms) {
    char b[64];
    std::snprintf(b, sizeof b, "%s%s=%.4f", rec.empty() ? "" : " ", m.first < 0 ? "fft" : kVariants[m.first].name,
                  m.second);
    rec += b;
  }
  ctx->tune_log[key] = rec;
  return best.first;
}

bool p1_staged_choice(mlc_ctx* ctx, const FftPlan2D& p, const std::function<void(bool)>& run) {
  char key[96];
  const char* pn = p.prec == MLC_F64 ? "f64" : p.prec == MLC_F32 ? "f32" : p.prec == PREC_FF ? "f32x2" : "f32x2->f32";
  // Beside the second convolution chain of the batched step the staged form's extra shared
  // memory crowds out the other chain's CTAs: measured alone it is the faster form (1.06
  // against 1.11 ms per profile at 10000^2, float-float), in the step the slower one (54.4
  // against 53.5 ms per step).  That context has its own key, not timed, prefetching unless
  // pinned.
  std::snprintf(key, sizeof key, "conv P1 %s %dx%d%s", pn, p.Nx, p.Ny, ctx->two_chains ? " two-chain" : "");
  auto it = ctx->tune.find(key);
  if (it != ctx->tune.end()) return it->second != 0;
  if (!ctx->autotune || ctx->two_chains) return false;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  MLC_CUDA(cudaStreamIsCapturing(ctx->stream, &cs));
  if (cs != cudaStreamCaptureStatusNone) return false;
  struct TimingOff {
    mlc_ctx* c;
    bool saved;
    ~TimingOff() { c->timing = saved; }
  } off{ctx, ctx->timing};
  ctx->timing = false;
  const float t0 = time_on_stream(ctx, [&] { run(false); });
  const float t1 = time_on_stream(ctx, [&] { run(true); });
  const int choice = t1 < t0 ? 1 : 0;
  ctx->tune[key] = choice;
  ctx->tune_name[key] = choice ? "smem-staged" : "l2-prefetch";
  char rec[96];
  std::snprintf(rec, sizeof rec, "l2-prefetch=%.4f smem-staged=%.4f", t0, t1);
  ctx->tune_log[key] = rec;
  return choice != 0;
}

void conv_auto(mlc_ctx* ctx, const FftPlan2D& p, const void* map, const void* Fmap, const double* prof, int pN,
               void* out) {
  const int v = conv_direct_choice(ctx, p, map, Fmap, prof, pN, out, false);
  if (v >= 0) conv_direct(ctx, p, map, prof, pN, v, out);
  else conv_fused(ctx, p, Fmap, prof, pN, out);
}

// "key: choice (candidate=ms ...)" lines of every tuned key.
std::string autotune_report(mlc_ctx* ctx) {
  std::string s;
  for (const auto& kv : ctx->tune) {
    auto nm = ctx->tune_name.find(kv.first);
    s += kv.first + ": " + (nm != ctx->tune_name.end() ? nm->second : std::to_string(kv.second));
    auto l = ctx->tune_log.find(kv.first);
    if (l != ctx->tune_log.end()) s += " (" + l->second + ")";
    s += "\n";
  }
  return s;
}

}  // namespace mlc
