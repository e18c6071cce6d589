// 2-D real FFTs and FFT convolution of a magnification map with a source profile.
//
// Replaces the reference's cuFFT D2Z/Z2D plans and kernel_multiplyFFTs
// (simulating_lcurves/src/gpu_functions.cu:150-200, 522-577) with hand-written passes:
//
//   forward(map):  R  rows, real FFT of length Nx (complex FFT of Nx/2 + split)
//                  A  columns, sub-pass over row sets {n1*N2 + n2}: length-N1 DFT, twiddle
//                  B  columns, sub-pass over row blocks {k1*N2 + n2}: length-N2 DFT
//     The spectrum is left in "digit-transposed" row order (row k1*N2 + k2 holds
//     frequency k1 + N1*k2); every consumer below works in that order, so no
//     reordering pass is ever made.
//
//   fused convolution per profile (MLC_CONV_FUSED):
//     P0  real FFT of the 2h non-zero rows of the wrapped profile only
//     P1  per (k1, strip): the profile's column spectrum for all k2 built in shared
//         memory (sub-pass A of the profile reduces to <= 2*ceil(h/N2) terms because
//         only rows [0,h) and [Ny-h,Ny) are non-zero), multiplied by the map spectrum
//         and by 1/(Nx Ny), then the inverse length-N2 sub-pass and its twiddle
//     P2  inverse sub-pass over row sets (length N1)
//     P3  inverse real FFT of each row (c2r)
//   plain convolution (MLC_CONV_PLAIN): full-size wrapped kernel, full forward,
//     pointwise multiply, full inverse -- one launch per stage, like the reference.
//
// This file holds the plans, the twiddle tables and the dispatch by precision; the
// kernels and launch sequences are in fft_impl.cuh.
#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <unordered_map>

#include "mlc_internal.h"

namespace mlc {

RadixList factor_radices(int L, int tw_stride) {
  RadixList rl{};
  rl.n = 0;
  rl.L = L;
  if (L < 1 || L > 65535) {
    rl.n = -1;
    return rl;
  }
  int n = L;
  while (n % 5 == 0) { rl.r[rl.n++] = 5; n /= 5; }
  while (n % 3 == 0) { rl.r[rl.n++] = 3; n /= 3; }
  int e2 = 0;
  while (n % 2 == 0) { e2++; n /= 2; }
  if (n != 1) {
    rl.n = -1;
    return rl;
  }
  int n8 = e2 / 3, rem = e2 % 3;
  if (rem == 1 && n8 > 0) {  // 8*2 -> 4*4
    n8--;
    rl.r[rl.n++] = 4;
    rl.r[rl.n++] = 4;
  } else if (rem == 1) {
    rl.r[rl.n++] = 2;
  } else if (rem == 2) {
    rl.r[rl.n++] = 4;
  }
  for (int i = 0; i < n8; i++) rl.r[rl.n++] = 8;
  int Ns = 1;
  rl.tlen = 0;
  for (int p = 0; p < rl.n; p++) {
    rl.Ns[p] = Ns;
    rl.toff[p] = rl.tlen;
    rl.tlen += p == 0 ? 0 : Ns * (rl.r[p] - 1);
    // exact j / Ns = umulhi(j, magic) for j * Ns < 2^32 (here j < L <= 65535)
    rl.magic[p] = Ns > 1 ? (uint32_t)((0x100000000ull + Ns - 1) / Ns) : 0u;
    rl.twstep[p] = (L / (Ns * rl.r[p])) * tw_stride;
    Ns *= rl.r[p];
  }
  return rl;
}

// The attribute belongs to the function on the current device: a process holding contexts
// on several GPUs sets it once per (device, function).
void set_max_smem(const void* func, size_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<int, const void*>, size_t> done;
  int dev = 0;
  MLC_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> g(mu);
  const auto key = std::make_pair(dev, func);
  auto it = done.find(key);
  if (it != done.end() && it->second >= bytes) return;
  MLC_CUDA(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  done[key] = bytes;
}

FftPlan2D::~FftPlan2D() {
  if (twx) cudaFree(twx);
  if (twy) cudaFree(twy);
}

// exp(-2 pi i m / N), m in [0, N), evaluated in long double with the angle reduced to
// the first octant so that each entry is correctly rounded to FP64 in practice.
static void twiddle_table(int N, std::vector<double>& re, std::vector<double>& im) {
  re.resize(N);
  im.resize(N);
  const long double TWO_PI = 6.283185307179586476925286766559005768L;
  for (int m = 0; m < N; m++) {
    // reduce m/N to [0, 1/8] using the symmetries of cos/sin
    long q8 = (long)m * 8;  // octant index via integer arithmetic
    int oct = (int)(q8 / N);
    long double frac;  // angle fraction of a full turn within the octant frame
    long double c, s;
    // angle a = 2 pi m / N; write m/N = oct/8 + r with r in [0, 1/8)
    long double r = ((long double)m - (long double)oct * N / 8.0L) / N;
    (void)frac;
    long double a = TWO_PI * r;
    long double ca = cosl(a), sa = sinl(a);
    const long double h = 0.70710678118654752440084436210484903928L;
    // rotate by oct * 45 degrees
    switch (oct & 7) {
      case 0: c = ca; s = sa; break;
      case 1: c = h * (ca - sa); s = h * (ca + sa); break;
      case 2: c = -sa; s = ca; break;
      case 3: c = -h * (ca + sa); s = h * (ca - sa); break;
      case 4: c = -ca; s = -sa; break;
      case 5: c = -h * (ca - sa); s = -h * (ca + sa); break;
      case 6: c = sa; s = -ca; break;
      default: c = h * (ca + sa); s = -h * (ca - sa); break;
    }
    // exact values where they are known
    if ((long)m * 4 % N == 0) {
      long k = (long)m * 4 / N;
      c = (k == 0) ? 1 : (k == 2) ? -1 : 0;
      s = (k == 1) ? 1 : (k == 3) ? -1 : 0;
    }
    re[m] = (double)c;
    im[m] = -(double)s;  // forward sign
  }
}

template <typename T>
static void* upload_twiddles(int N) {
  std::vector<double> re, im;
  twiddle_table(N, re, im);
  std::vector<C2<T>> h(N);
  for (int m = 0; m < N; m++) h[m] = C2<T>{(T)re[m], (T)im[m]};
  void* d = nullptr;
  MLC_CUDA(cudaMalloc(&d, sizeof(C2<T>) * N));
  MLC_CUDA(cudaMemcpy(d, h.data(), sizeof(C2<T>) * N, cudaMemcpyHostToDevice));
  return d;
}

static void split_columns(int Ny, int& N1, int& N2) {
  int best = 1;
  for (int d = 1; (long)d * d <= Ny; d++)
    if (Ny % d == 0) best = d;
  N1 = best;
  N2 = Ny / best;
}

FftPlan2D* plan_get(mlc_ctx* ctx, int Nx, int Ny, int prec) {
  auto key = std::make_tuple(Nx, Ny, prec);
  auto it = ctx->plans.find(key);
  if (it != ctx->plans.end()) return it->second.get();
  MLC_REQUIRE(Nx >= 4 && Ny >= 2 && Nx % 2 == 0, MLC_ERR_ARG, "map sides must be even, Nx >= 4");
  std::unique_ptr<FftPlan2D> p(new FftPlan2D());
  p->Nx = Nx;
  p->Ny = Ny;
  p->prec = prec;
  p->M = Nx / 2;
  p->Wc = Nx / 2 + 1;
  p->Wp = (int)round_up(p->Wc, 16);
  p->elem = prec == MLC_F64 ? sizeof(C2<double>) : prec_is_ff(prec) ? sizeof(C2<ff>) : sizeof(C2<float>);
  p->CW = prec == MLC_F64 ? 8 : 16;  // as strip_width<T>() in fft_impl.cuh
  split_columns(Ny, p->N1, p->N2);
  p->rlM = factor_radices(p->M, 2);
  p->rlN1 = factor_radices(p->N1, p->N2);
  p->rlN2 = factor_radices(p->N2, p->N1);
  MLC_REQUIRE(p->rlM.n >= 0 && p->rlN1.n >= 0 && p->rlN2.n >= 0, MLC_ERR_ARG,
              "map sides must factor into 2, 3 and 5");
  size_t row_smem = 2 * (size_t)(p->M + 1) * p->elem;
  MLC_REQUIRE(row_smem <= 220 * 1024, MLC_ERR_LIMIT,
              "map row too long for one shared-memory row transform (Nx <= 13000 FP64, 26000 FP32)");
  MLC_REQUIRE(2 * (size_t)p->N2 * p->CW * p->elem <= 200 * 1024, MLC_ERR_LIMIT, "column length too large");
  if (prec == MLC_F64) {
    p->twx = upload_twiddles<double>(Nx);
    p->twy = upload_twiddles<double>(Ny);
  } else if (prec_is_ff(prec)) {
    p->twx = upload_twiddles<ff>(Nx);
    p->twy = upload_twiddles<ff>(Ny);
  } else {
    p->twx = upload_twiddles<float>(Nx);
    p->twy = upload_twiddles<float>(Ny);
  }
  FftPlan2D* raw = p.get();
  ctx->plans[key] = std::move(p);
  return raw;
}

// ---------------------------------------------------------------- dispatch by precision

void fft2_forward(mlc_ctx* ctx, const FftPlan2D& p, const void* in, int in_dtype, void* spec) {
  if (prec_is_ff(p.prec)) forward_impl<ff>(ctx, p, in, in_dtype, spec);
  else if (p.prec == MLC_F64) forward_impl<double>(ctx, p, in, in_dtype, spec);
  else forward_impl<float>(ctx, p, in, in_dtype, spec);
}

void conv_fused(mlc_ctx* ctx, const FftPlan2D& p, const void* Fmap, const double* prof, int pN, void* out) {
  if (p.prec == PREC_FFS) {  // P0-P2 to the half-spectrum, then P3 into FP32 pixels
    void* tmp = ws_get(ctx, WS_SPEC_TMP, p.spec_bytes());
    conv_fused_impl<ff>(ctx, p, Fmap, prof, pN, nullptr, tmp, WS_KX);
    rows_c2r_impl<ff, float>(ctx, p, tmp, out);
  } else if (p.prec == PREC_FF) conv_fused_impl<ff>(ctx, p, Fmap, prof, pN, out);
  else if (p.prec == MLC_F64) conv_fused_impl<double>(ctx, p, Fmap, prof, pN, out);
  else conv_fused_impl<float>(ctx, p, Fmap, prof, pN, out);
}

void conv_fused_spectrum(mlc_ctx* ctx, const FftPlan2D& p, const void* Fmap, const double* prof, int pN,
                         void* spec_out, int kx_slot) {
  if (prec_is_ff(p.prec)) conv_fused_impl<ff>(ctx, p, Fmap, prof, pN, nullptr, spec_out, kx_slot);
  else if (p.prec == MLC_F64) conv_fused_impl<double>(ctx, p, Fmap, prof, pN, nullptr, spec_out, kx_slot);
  else conv_fused_impl<float>(ctx, p, Fmap, prof, pN, nullptr, spec_out, kx_slot);
}

bool profile_spectrum_supported(const FftPlan2D& p) {
  if (prec_is_ff(p.prec)) return profile_spectrum_supported_impl<ff>(p);
  if (p.prec == MLC_F64) return profile_spectrum_supported_impl<double>(p);
  return profile_spectrum_supported_impl<float>(p);
}

void profile_spectrum(mlc_ctx* ctx, const FftPlan2D& p, const double* prof, int pN, void* ks) {
  if (prec_is_ff(p.prec)) profile_spectrum_impl<ff>(ctx, p, prof, pN, ks);
  else if (p.prec == MLC_F64) profile_spectrum_impl<double>(ctx, p, prof, pN, ks);
  else profile_spectrum_impl<float>(ctx, p, prof, pN, ks);
}

void conv_cached_spectrum(mlc_ctx* ctx, const FftPlan2D& p, const void* Fmap, const void* ks, void* spec_out) {
  if (prec_is_ff(p.prec)) conv_cached_impl<ff>(ctx, p, Fmap, ks, spec_out);
  else if (p.prec == MLC_F64) conv_cached_impl<double>(ctx, p, Fmap, ks, spec_out);
  else conv_cached_impl<float>(ctx, p, Fmap, ks, spec_out);
}

void conv_cached(mlc_ctx* ctx, const FftPlan2D& p, const void* Fmap, const void* ks, void* out) {
  if (p.prec == PREC_FFS) {
    void* tmp = ws_get(ctx, WS_SPEC_TMP, p.spec_bytes());
    conv_cached_impl<ff>(ctx, p, Fmap, ks, tmp);
    rows_c2r_impl<ff, float>(ctx, p, tmp, out);
  } else if (p.prec == PREC_FF) conv_cached_real_impl<ff>(ctx, p, Fmap, ks, out);
  else if (p.prec == MLC_F64) conv_cached_real_impl<double>(ctx, p, Fmap, ks, out);
  else conv_cached_real_impl<float>(ctx, p, Fmap, ks, out);
}

bool rows_c2r_interleave_supported(const FftPlan2D& p) {
  return (p.M == 5000 || p.M == 4096 || p.M == 2000 || p.M == 1000) && p.Ny <= 65535;  // rows on grid.y
}

bool rows_c2r_interleave(mlc_ctx* ctx, const FftPlan2D& p, const void* specs, long spec_stride, int nm, int S,
                         void* out, unsigned planar) {
  if (p.prec == PREC_FFS) return c2r_interleave_impl<ff, float>(ctx, p, specs, spec_stride, nm, S, out, planar);
  if (p.prec == PREC_FF) return c2r_interleave_impl<ff>(ctx, p, specs, spec_stride, nm, S, out, planar);
  if (p.prec == MLC_F64) return c2r_interleave_impl<double>(ctx, p, specs, spec_stride, nm, S, out, planar);
  return c2r_interleave_impl<float>(ctx, p, specs, spec_stride, nm, S, out, planar);
}

void conv_plain(mlc_ctx* ctx, const FftPlan2D& p, const void* Fmap, const double* prof, int pN, void* out) {
  MLC_REQUIRE(!prec_is_ff(p.prec), MLC_ERR_ARG, "the plain form runs the map's own precision (map in float-float mode)");
  if (p.prec == MLC_F64) conv_plain_impl<double>(ctx, p, Fmap, prof, pN, out);
  else conv_plain_impl<float>(ctx, p, Fmap, prof, pN, out);
}

}  // namespace mlc
