// Pairwise magnitude-difference chi2 between simulated curves of two lensed images.
//
//   chi2_ij = sum_t w_t (d_t - (a_it - b_jt) - c_ij)^2
//
// with c_ij = 0, or (offset form) the magnitude offset that minimises it,
// c_ij = sum w (d - a + b) / sum w.  No counterpart in the reference, whose pair
// statistic is the flux ratio (gpu_functions.cu:739-740, chi2/chi2_functions.cuh:59-64);
// this is the separable form, chi2 = |Q_j - P_i|^2 with P_i = sqrt(w) (a_i - abar_i) and
// Q_j = sqrt(w) (b_j + d - bbar_j) (bars: weighted means, only in the offset form).
//
// This file holds the plain FP64 form (one thread per pair, CUDA cores) and the
// preparation used by the tensor-core form (pairtc.cu): per-curve centring and
// weighting in FP64, a power-of-two quantisation step per curve, 24-bit integers split
// into three signed 8-bit slices stored as bf16 (exact), and the exact squared norms.
#include <cmath>
#include <cstring>
#include <vector>

#include "bilinear.cuh"
#include "mlc_internal.h"
#include "pairdiff.h"

namespace mlc {

// ---------------------------------------------------------------- plain FP64 form

// One thread per pair (i, j): FP64 two-pass form (offset first, then the sum of squares).
__global__ void __launch_bounds__(256) k_pairdiff_plain(const float* __restrict__ A, const float* __restrict__ B,
                                                        int NA, int NB, int T, const double* __restrict__ w,
                                                        const double* __restrict__ d, double W, int offset,
                                                        long npairs, const long* __restrict__ ia,
                                                        const long* __restrict__ ib, double* __restrict__ chi2) {
  const long n = ia ? npairs : (long)NA * NB;
  for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < n; p += (long)gridDim.x * blockDim.x) {
    const long i = ia ? ia[p] : p / NB, j = ia ? ib[p] : p % NB;
    const float* a = A + i * T;
    const float* b = B + j * T;
    double c = 0.0;
    if (offset) {
      double sr = 0.0;
      for (int t = 0; t < T; t++) sr += w[t] * ((d ? d[t] : 0.0) - ((double)a[t] - (double)b[t]));
      c = sr / W;
    }
    double s = 0.0;
    for (int t = 0; t < T; t++) {
      const double r = (d ? d[t] : 0.0) - ((double)a[t] - (double)b[t]) - c;
      s += w[t] * r * r;
    }
    chi2[p] = s;
  }
}

void pairdiff_plain(mlc_ctx* ctx, const float* A, const float* B, int NA, int NB, int T, const double* w_dev,
                    const double* d_dev, double W, int offset, long npairs, const long* ia, const long* ib,
                    double* chi2) {
  const long n = ia ? npairs : (long)NA * NB;
  if (n <= 0) return;
  const int grid = (int)std::max<long>(1, std::min<long>((n + 255) / 256, (long)ctx->sm_count * 32));
  {
    MLC_KSCOPE(ctx, "pairdiff_plain");
    k_pairdiff_plain<<<grid, 256, 0, ctx->stream>>>(A, B, NA, NB, T, w_dev, d_dev, W, offset, npairs, ia, ib, chi2);
  }
  MLC_CHECK_LAUNCH();
}

// ---------------------------------------------------------------- preparation for the tensor-core form

// Centred, weighted curves in FP64: out[r*T + t] = sqrt(w_t) (x_rt + sgn*d_t - mean_r).
// side 0: x = a, no d; side 1: x = b, plus d.  Also the per-row max |.| (for the scale).
__global__ void __launch_bounds__(256) k_pd_center(const float* __restrict__ X, int N, int T,
                                                   const double* __restrict__ sw, const double* __restrict__ w,
                                                   const double* __restrict__ d, double W, int offset,
                                                   double* __restrict__ out, double* __restrict__ rowmax) {
  const int lane = threadIdx.x & 31;
  const long r = (long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (r >= N) return;
  const float* x = X + r * T;
  double mean = 0.0;
  if (offset) {
    double s = 0.0;
    for (int t = lane; t < T; t += 32) s += w[t] * ((double)x[t] + (d ? d[t] : 0.0));
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    mean = s / W;
  }
  double mx = 0.0;
  for (int t = lane; t < T; t += 32) {
    const double v = sw[t] * ((double)x[t] + (d ? d[t] : 0.0) - mean);
    out[r * T + t] = v;
    mx = fmax(mx, fabs(v));
  }
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if (lane == 0) rowmax[r] = mx;
}

__global__ void k_pd_maxreduce(const double* __restrict__ v, long n, unsigned long long* __restrict__ out) {
  double m = 0.0;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    m = fmax(m, v[i]);
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(m));  // m >= 0
}

__device__ __forceinline__ uint16_t bf16_of_small_int(int v) {
  // v in [-128, 127] is exact in bf16; build the bits from the float
  const float f = (float)v;
  return (uint16_t)(__float_as_uint(f) >> 16);
}

// Per row: step exponent e = ceil(log2(rowmax / QMAX)) (clamped to [PD_EMIN, PD_EMAX]), integers
// q = rint(v 2^-e) (|q| <= QMAX), split q = s0*65536 + s1*256 + s2 with balanced digits in
// [-128, 127], slices written to the operand row [slice 0 | slice 1 | slice 2] (Kp = padded T
// each, zeros beyond T), the exact squared norm sum q^2 and its float-float copy.  Rows
// beyond N (padding up to the tile) are zero.
__global__ void __launch_bounds__(256) k_pd_quantize(const double* __restrict__ v, const double* __restrict__ rowmax,
                                                     int N, int Npad, int T, int Kp, uint16_t* __restrict__ ops,
                                                     long long* __restrict__ norm2, float2* __restrict__ norm2_ff,
                                                     int* __restrict__ exps, int* __restrict__ err) {
  const int lane = threadIdx.x & 31;
  const long r = (long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (r >= Npad) return;
  // The smallest e with rowmax 2^-e <= QMAX, from the bits of rowmax = (1 + f 2^-52) 2^E0
  // (GB300's FP64 pipe is narrow; log2 and exp2 here had cost more than the rest of the
  // kernel): QMAX = 8355711 lies in [2^22, 2^23), so e = E0 - 22 when (1 + f 2^-52) 2^22 <=
  // QMAX, i.e. f <= (QMAX - 2^22) 2^30, else E0 - 21.  Subnormal or zero maxima keep PD_EMIN.
  int e = PD_EMIN;
  if (r < N && rowmax[r] > 0) {
    const long long b = __double_as_longlong(rowmax[r]);
    const int E0 = (int)((b >> 52) & 0x7ff) - 1023;
    const long long f = b & 0xFFFFFFFFFFFFFll;
    if (E0 > -1023) e = E0 - 22 + (f > ((long long)(PD_QMAX - (1 << 22)) << 30) ? 1 : 0);
    if (e > PD_EMAX) atomicExch(err, 2);
    e = max(PD_EMIN, min(PD_EMAX, e));
  }
  const double inv_delta = __longlong_as_double((long long)(1023 - e) << 52);  // 2^-e exactly
  uint16_t* row = ops + r * (3L * Kp);
  long long acc = 0;
  for (int t = lane; t < Kp; t += 32) {
    int q = 0;
    if (r < N && t < T) {
      // v 2^-e is exact; rounded to the nearest integer (ties to even, as rint), NaN and
      // infinities convert out of range
      const long long x = __double2ll_rn(v[r * T + t] * inv_delta);
      if (!(x >= -PD_QMAX && x <= PD_QMAX)) atomicExch(err, 1);
      q = (int)max((long long)-PD_QMAX, min((long long)PD_QMAX, x));
    }
    int s2 = ((q % 256) + 256 + 128) % 256 - 128;  // balanced digit
    int r1 = (q - s2) / 256;
    int s1 = ((r1 % 256) + 256 + 128) % 256 - 128;
    int s0 = (r1 - s1) / 256;
    row[t] = bf16_of_small_int(s0);
    row[Kp + t] = bf16_of_small_int(s1);
    row[2 * Kp + t] = bf16_of_small_int(s2);
    acc += (long long)q * q;
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) {
    norm2[r] = acc;
    // |P|^2 in natural units, alpha 2^(2e), as a float-float pair (exact scaling in FP64)
    const double v2 = (double)acc * __longlong_as_double((long long)(1023 + 2 * e) << 52);  // 2^(2e)
    const float hi = (float)v2;
    norm2_ff[r] = make_float2(hi, (float)(v2 - (double)hi));
    exps[r] = e;
  }
}

// Builds both operand sides.  Returns delta (the quantisation step).
double pairdiff_prepare(mlc_ctx* ctx, const float* A, const float* B, int NA, int NB, int T, const double* w_host,
                        const double* d_host, int offset, PdOperands& ops) {
  MLC_REQUIRE(T >= 1 && T <= 4096, MLC_ERR_LIMIT, "T must be in [1, 4096]");
  ops.T = T;
  ops.Kp = (int)round_up(T, 64);
  ops.NA = NA;
  ops.NB = NB;
  ops.NApad = (int)round_up(NA, PD_TILE_M);
  ops.NBpad = (int)round_up(NB, PD_TILE_N);
  std::vector<double> sw(T), w(w_host, w_host + T), d(T, 0.0);
  double W = 0.0;
  for (int t = 0; t < T; t++) {
    MLC_REQUIRE(w[t] >= 0 && std::isfinite(w[t]), MLC_ERR_ARG, "weights must be finite and >= 0");
    sw[t] = std::sqrt(w[t]);
    W += w[t];
    if (d_host) d[t] = d_host[t];
  }
  MLC_REQUIRE(W > 0, MLC_ERR_ARG, "weights sum to zero");
  // small device tables: sw, w, d, then rowmax (NA+NB), then the global max
  char* sm = (char*)ws_get(ctx, WS_SMALL, sizeof(double) * (3 * T + NA + NB) + 64);
  double* dsw = (double*)sm;
  double* dw = dsw + T;
  double* dd = dw + T;
  double* rowmax = dd + T;
  // on the context's stream (which may not synchronise with the legacy default stream),
  // then waited for: the host vectors are freed on return
  MLC_CUDA(cudaMemcpyAsync(dsw, sw.data(), sizeof(double) * T, cudaMemcpyHostToDevice, ctx->stream));
  MLC_CUDA(cudaMemcpyAsync(dw, w.data(), sizeof(double) * T, cudaMemcpyHostToDevice, ctx->stream));
  MLC_CUDA(cudaMemcpyAsync(dd, d.data(), sizeof(double) * T, cudaMemcpyHostToDevice, ctx->stream));
  MLC_CUDA(cudaStreamSynchronize(ctx->stream));
  // centred, weighted curves (FP64), both sides
  double* cen = (double*)ws_get(ctx, WS_KREAL, sizeof(double) * ((size_t)NA + NB) * T);
  {
    MLC_KSCOPE(ctx, "pd_center");
    k_pd_center<<<ceil_div(NA, 8), 256, 0, ctx->stream>>>(A, NA, T, dsw, dw, nullptr, W, offset, cen, rowmax);
  }
  {
    MLC_KSCOPE(ctx, "pd_center");
    k_pd_center<<<ceil_div(NB, 8), 256, 0, ctx->stream>>>(B, NB, T, dsw, dw, d_host ? dd : nullptr, W, offset,
                                                          cen + (size_t)NA * T, rowmax + NA);
  }
  MLC_CHECK_LAUNCH();
  // the largest row maximum sets the reported step; rows keep their own steps
  unsigned long long* gmax = (unsigned long long*)ws_get(ctx, WS_SORT_HIST, 64);
  int* derr = (int*)(gmax + 1);
  MLC_CUDA(cudaMemsetAsync(gmax, 0, 16, ctx->stream));
  {
    MLC_KSCOPE(ctx, "pd_maxreduce");
    k_pd_maxreduce<<<std::max(1, std::min(ceil_div(NA + NB, 256), ctx->sm_count * 4)), 256, 0, ctx->stream>>>(
        rowmax, (long)NA + NB, gmax);
  }
  MLC_CHECK_LAUNCH();
  unsigned long long hm = 0;
  MLC_CUDA(cudaMemcpyAsync(&hm, gmax, 8, cudaMemcpyDeviceToHost, ctx->stream));
  MLC_CUDA(cudaStreamSynchronize(ctx->stream));
  double mx;
  memcpy(&mx, &hm, 8);
  const double delta = mx > 0 ? std::exp2(std::ceil(std::log2(mx / (double)PD_QMAX))) : 1.0;
  ops.delta = delta;
  ops.cenA = cen;
  ops.cenB = cen + (size_t)NA * T;
  // operands, norms, float-float norms and exponents
  const size_t rowsA = ops.NApad, rowsB = ops.NBpad;
  ops.a = (uint16_t*)ws_get(ctx, WS_PAIR_ACC, sizeof(uint16_t) * 3 * ops.Kp * (rowsA + rowsB) +
                                                  (sizeof(long long) + sizeof(float2) + sizeof(int)) * (rowsA + rowsB) +
                                                  512);
  ops.b = ops.a + 3 * (size_t)ops.Kp * rowsA;
  ops.alpha = (long long*)round_up((long)(uintptr_t)(ops.b + 3 * (size_t)ops.Kp * rowsB), 16);
  ops.beta = ops.alpha + rowsA;
  ops.alpha_ff = (float2*)(ops.beta + rowsB);
  ops.beta_ff = ops.alpha_ff + rowsA;
  ops.ea = (int*)(ops.beta_ff + rowsB);
  ops.eb = ops.ea + rowsA;
  {
    MLC_KSCOPE(ctx, "pd_quantize");
    k_pd_quantize<<<ceil_div(ops.NApad, 8), 256, 0, ctx->stream>>>(cen, rowmax, NA, ops.NApad, T, ops.Kp, ops.a,
                                                                   ops.alpha, ops.alpha_ff, ops.ea, derr);
  }
  {
    MLC_KSCOPE(ctx, "pd_quantize");
    k_pd_quantize<<<ceil_div(ops.NBpad, 8), 256, 0, ctx->stream>>>(cen + (size_t)NA * T, rowmax + NA, NB, ops.NBpad, T,
                                                                   ops.Kp, ops.b, ops.beta, ops.beta_ff, ops.eb, derr);
  }
  MLC_CHECK_LAUNCH();
  int herr = 0;
  MLC_CUDA(cudaMemcpyAsync(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  MLC_CUDA(cudaStreamSynchronize(ctx->stream));
  MLC_REQUIRE(herr != 2, MLC_ERR_LIMIT, "curve amplitudes beyond 2^20 * 8355711 (after weighting)");
  MLC_REQUIRE(herr == 0, MLC_ERR_ARG, "non-finite curve values");
  return delta;
}

// ---------------------------------------------------------------- sides built once per image

// The sample -> magnitude -> centre/weight pass of one expanding-source curve per warp, from
// the convolved maps (no light curve stored): curve r = the magnitudes of track r at the nep
// shared epochs t, band-minor (element e nbands + b), sampled like k_sample_expanding
// (sample.cu) and centred and weighted like k_pd_center -- the same arithmetic in the same
// order (lane l takes elements l, l + 32, ...), so the centred curves are those of the
// two-stage path bit for bit.  T = nep nbands <= 128.
__global__ void __launch_bounds__(256) k_pd_center_expanding(const float* __restrict__ maps, long npix, int Nx,
                                                             int Ny, int nbands, int nep, int N,
                                                             const float* __restrict__ x0,
                                                             const float* __restrict__ y0,
                                                             const float* __restrict__ phi,
                                                             const float* __restrict__ v,
                                                             const float* __restrict__ t,
                                                             const double* __restrict__ sw,
                                                             const double* __restrict__ w,
                                                             const double* __restrict__ d, double W, int offset,
                                                             double* __restrict__ out,
                                                             double* __restrict__ rowmax) {
  constexpr int PER = 4;  // elements per lane: T <= 128
  const int lane = threadIdx.x & 31;
  const long r = (long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (r >= N) return;
  const int T = nep * nbands;
  const TrackGeom<float> g(x0[r], y0[r], phi[r], v[r]);
  float x[PER];
#pragma unroll
  for (int i = 0; i < PER; i++) {
    const int q = lane + 32 * i;
    x[i] = 0.f;
    if (q < T) {
      const int e = q / nbands, b = q - e * nbands;
      const Bilin<float> B = g.at(t[e], Nx, Ny);
      const float mu = B.inside ? bilin_read<float>(maps + (long)(e * nbands + b) * npix, B, Nx) : 0.f;
      x[i] = -2.5f * mlc_log10(mu);
    }
  }
  double mean = 0.0;
  if (offset) {
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < PER; i++) {
      const int q = lane + 32 * i;
      if (q < T) s += w[q] * ((double)x[i] + (d ? d[q] : 0.0));
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    mean = s / W;
  }
  double mx = 0.0;
#pragma unroll
  for (int i = 0; i < PER; i++) {
    const int q = lane + 32 * i;
    if (q < T) {
      const double vv = sw[q] * ((double)x[i] + (d ? d[q] : 0.0) - mean);
      out[r * T + q] = vv;
      mx = fmax(mx, fabs(vv));
    }
  }
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if (lane == 0) rowmax[r] = mx;
}

namespace {

// One device allocation for a side: weight tables (sqrt w, w, d), centred curves, row
// maxima, operands, norms, steps and the max/error words; sizes from N and T.
void side_alloc(mlc_ctx* ctx, PdSide& sd, int N, int T, const double* w_host, const double* d_host, int offset, double& W) {
  MLC_REQUIRE(N >= 1 && T >= 1 && T <= 128, MLC_ERR_LIMIT, "pair side: N >= 1 and 1 <= T <= 128");
  sd.N = N;
  sd.T = T;
  sd.Kp = (int)round_up(T, 64);
  sd.Npad = (int)round_up(N, PD_SIDE_PAD);
  sd.offset = offset != 0;
  sd.has_d = d_host != nullptr;
  sd.w.assign(w_host, w_host + T);
  W = 0.0;
  for (int i = 0; i < T; i++) {
    MLC_REQUIRE(sd.w[i] >= 0 && std::isfinite(sd.w[i]), MLC_ERR_ARG, "weights must be finite and >= 0");
    W += sd.w[i];
  }
  MLC_REQUIRE(W > 0, MLC_ERR_ARG, "weights sum to zero");
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const size_t b_tab = al(sizeof(double) * 3 * T), b_cen = al(sizeof(double) * (size_t)N * T),
               b_max = al(sizeof(double) * N), b_ops = al(sizeof(uint16_t) * 3 * (size_t)sd.Kp * sd.Npad),
               b_n2 = al(sizeof(long long) * sd.Npad), b_nff = al(sizeof(float2) * sd.Npad),
               b_ex = al(sizeof(int) * sd.Npad), b_fl = 256;
  sd.bytes = b_tab + b_cen + b_max + b_ops + b_n2 + b_nff + b_ex + b_fl;
  MLC_CUDA(cudaMalloc(&sd.mem, sd.bytes));
  char* p = (char*)sd.mem + b_tab;
  sd.cen = (double*)p;
  p += b_cen;
  sd.rowmax = (double*)p;
  p += b_max;
  sd.ops = (uint16_t*)p;
  p += b_ops;
  sd.norm2 = (long long*)p;
  p += b_n2;
  sd.norm2_ff = (float2*)p;
  p += b_nff;
  sd.exps = (int*)p;
  std::vector<double> tab(3 * (size_t)T, 0.0);
  for (int i = 0; i < T; i++) {
    tab[i] = std::sqrt(sd.w[i]);
    tab[T + i] = sd.w[i];
    if (d_host) tab[2 * T + i] = d_host[i];
  }
  MLC_CUDA(cudaMemcpyAsync(sd.mem, tab.data(), sizeof(double) * tab.size(), cudaMemcpyHostToDevice, ctx->stream));
  MLC_CUDA(cudaStreamSynchronize(ctx->stream));  // tab is freed on return
}

// The reported step from the largest row maximum, then the sliced integers (as in
// pairdiff_prepare; every row keeps its own step).
void side_finish(mlc_ctx* ctx, PdSide& sd) {
  unsigned long long* gmax = (unsigned long long*)((char*)sd.mem + sd.bytes - 256);
  int* derr = (int*)(gmax + 1);
  MLC_CUDA(cudaMemsetAsync(gmax, 0, 16, ctx->stream));
  {
    MLC_KSCOPE(ctx, "pd_maxreduce");
    k_pd_maxreduce<<<std::max(1, std::min(ceil_div(sd.N, 256), ctx->sm_count * 4)), 256, 0, ctx->stream>>>(
        sd.rowmax, (long)sd.N, gmax);
  }
  {
    MLC_KSCOPE(ctx, "pd_quantize");
    k_pd_quantize<<<ceil_div(sd.Npad, 8), 256, 0, ctx->stream>>>(sd.cen, sd.rowmax, sd.N, sd.Npad, sd.T, sd.Kp, sd.ops,
                                                                 sd.norm2, sd.norm2_ff, sd.exps, derr);
  }
  MLC_CHECK_LAUNCH();
  unsigned long long hm[2] = {0, 0};
  MLC_CUDA(cudaMemcpyAsync(hm, gmax, 16, cudaMemcpyDeviceToHost, ctx->stream));
  MLC_CUDA(cudaStreamSynchronize(ctx->stream));
  double mx;
  std::memcpy(&mx, &hm[0], 8);
  int herr;
  std::memcpy(&herr, &hm[1], sizeof herr);
  sd.delta = mx > 0 ? std::exp2(std::ceil(std::log2(mx / (double)PD_QMAX))) : 1.0;
  MLC_REQUIRE(herr != 2, MLC_ERR_LIMIT, "curve amplitudes beyond 2^20 * 8355711 (after weighting)");
  MLC_REQUIRE(herr == 0, MLC_ERR_ARG, "non-finite curve values");
}

}  // namespace

void pd_side_free(PdSide& sd) {
  if (sd.mem) cudaFree(sd.mem);
  sd.mem = nullptr;
}

void pd_side_from_curves(mlc_ctx* ctx, const float* X, int N, int T, const double* w_host, const double* d_host,
                         int offset, PdSide& sd) {
  double W;
  side_alloc(ctx, sd, N, T, w_host, d_host, offset, W);
  try {
    const double* tab = (const double*)sd.mem;
    {
      MLC_KSCOPE(ctx, "pd_center");
      k_pd_center<<<ceil_div(N, 8), 256, 0, ctx->stream>>>(X, N, T, tab, tab + T, d_host ? tab + 2 * T : nullptr, W,
                                                           sd.offset, sd.cen, sd.rowmax);
    }
    MLC_CHECK_LAUNCH();
    side_finish(ctx, sd);
  } catch (...) {
    pd_side_free(sd);
    throw;
  }
}

void pd_side_from_expanding(mlc_ctx* ctx, const float* maps, int Nx, int Ny, int nep, int nbands, int ntracks,
                            const float* x0, const float* y0, const float* phi, const float* v, const float* t,
                            const double* w_host, const double* d_host, int offset, PdSide& sd) {
  MLC_REQUIRE(nep >= 1 && nbands >= 1 && Nx >= 2 && Ny >= 2, MLC_ERR_ARG, "pair side: bad map or epoch sizes");
  double W;
  side_alloc(ctx, sd, ntracks, nep * nbands, w_host, d_host, offset, W);
  try {
    const double* tab = (const double*)sd.mem;
    {
      MLC_KSCOPE(ctx, "pd_center_expanding");
      k_pd_center_expanding<<<ceil_div(ntracks, 8), 256, 0, ctx->stream>>>(
          maps, (long)Nx * Ny, Nx, Ny, nbands, nep, ntracks, x0, y0, phi, v, t, tab, tab + sd.T,
          d_host ? tab + 2 * sd.T : nullptr, W, sd.offset, sd.cen, sd.rowmax);
    }
    MLC_CHECK_LAUNCH();
    side_finish(ctx, sd);
  } catch (...) {
    pd_side_free(sd);
    throw;
  }
}

}  // namespace mlc
