// Differentiable track fit (no reference counterpart): the chi2 of model light curves
// against observed curves, and its gradient with respect to every track's parameters
// theta = (x0, y0, phi, v, R_half, dm), in one kernel.
//
// Radius stack (radius_stack, once per map): for radii R_0 < ... < R_{K-1} the map is
// convolved with the smooth thin-disc raster P(R_k) and with its derivative rasters
// (profile.cu, thin_disc_fit_raster), four fields per radius interleaved per pixel:
//   stack[((y Nx + x) K + k) 4 + f],  f = 0: M = map * P, 1: dM/dx = map * dP/dx,
//                                     2: dM/dy = map * dP/dy, 3: dM/dR = map * dP/dR
// (x, y in pixels, R in the radius units): values and exact first derivatives of the
// continuous convolution sum_j map_j P(p - c_j) at every pixel node.
//
// Model of a track at epoch t (pixel units, nodes at pixel centres j + 1/2):
//   p(t) = (x0 + v t cos phi, y0 + v t sin phi)
//   M(p, R) = tensor-product cubic Hermite interpolant in (x, y, R) of those node values
//             and first derivatives (no cross-derivative terms), which is C1 everywhere
//   m(t) = -2.5 log10 M(p(t), R) + dm,        chi2 = sum_e w_e (o_e - m(t_e))^2
// Being C1, the model's central differences converge to its gradient for every
// parameter (a bilinear model has a derivative jump on every line of pixel centres, which
// long tracks cross for any useful step in phi or v).
// Gradient: dchi2/dm_e = -2 w_e (o_e - m_e), dm/dM = -2.5 / (M ln 10), dM/dx, dM/dy, dM/dR
// from the Hermite basis derivatives, dx/dphi = -v t sin phi, dy/dphi = v t cos phi,
// dx/dv = t cos phi, dy/dv = t sin phi, dm/d(dm) = 1.
// One warp per track, lanes over its epochs, reduced with shuffles: the light curve is
// written only when asked for.  An epoch outside the hull of pixel centres, or with
// M <= 0, contributes nothing (its model magnitude is NaN).  R outside [R_0, R_{K-1}]
// is clamped and gets a zero R-gradient.
#include <cmath>
#include <vector>

#include "bilinear.cuh"
#include "mlc_internal.h"

namespace mlc {

template <typename T>
struct RadiusNodes {
  int K;
  T r[MLC_FIT_MAX_RADII];
};

// The eight values (M, dM/dx, dM/dy, dM/dR) of radii k and k+1 at one pixel.
template <typename T>
__device__ __forceinline__ void load8(const T* p, T* v);
template <>
__device__ __forceinline__ void load8<float>(const float* p, float* v) {
  const float4 a = __ldg(reinterpret_cast<const float4*>(p)), b = __ldg(reinterpret_cast<const float4*>(p) + 1);
  v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
}
template <>
__device__ __forceinline__ void load8<double>(const double* p, double* v) {
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const double2 a = __ldg(reinterpret_cast<const double2*>(p) + i);
    v[2 * i] = a.x;
    v[2 * i + 1] = a.y;
  }
}

// Cubic Hermite basis on [0, 1]: value weights (h00, h01), slope weights (h10, h11) and
// their derivatives.
template <typename T>
struct Herm {
  T v0, v1, t0, t1, dv0, dv1, dt0, dt1;
};
template <typename T>
__device__ __forceinline__ Herm<T> herm(T s) {
  const T s2 = s * s, s3 = s2 * s;
  Herm<T> H;
  H.v0 = (T)2 * s3 - (T)3 * s2 + (T)1;
  H.v1 = (T)3 * s2 - (T)2 * s3;
  H.t0 = s3 - (T)2 * s2 + s;
  H.t1 = s3 - s2;
  H.dv0 = (T)6 * s2 - (T)6 * s;
  H.dv1 = (T)6 * s - (T)6 * s2;
  H.dt0 = (T)3 * s2 - (T)4 * s + (T)1;
  H.dt1 = (T)3 * s2 - (T)2 * s;
  return H;
}

template <typename T>
__global__ void __launch_bounds__(256) k_track_fit(const T* __restrict__ stack, int Nx, int Ny, RadiusNodes<T> rn,
                                                   int ntracks, const T* __restrict__ theta,
                                                   const int64_t* __restrict__ off, const T* __restrict__ t,
                                                   const T* __restrict__ obs, const T* __restrict__ w,
                                                   T* __restrict__ chi2, T* __restrict__ grad,
                                                   T* __restrict__ model) {
  const int lane = threadIdx.x & 31;
  const long tr = (long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (tr >= ntracks) return;
  const T* th = theta + tr * 6;
  const T X0 = th[0], Y0 = th[1], PHI = th[2], V = th[3], R = th[4], DM = th[5];
  T sn, cs;
  if (sizeof(T) == 8) {
    double s_, c_;
    sincos((double)PHI, &s_, &c_);
    sn = (T)s_;
    cs = (T)c_;
  } else {
    float s_, c_;
    sincosf((float)PHI, &s_, &c_);
    sn = (T)s_;
    cs = (T)c_;
  }
  // bracket of R: value weights w*, slope weights u* (slope data per unit R, spacing h)
  // and their R-derivatives
  const int K = rn.K;
  int k = 0;
  while (k < K - 2 && R >= rn.r[k + 1]) k++;
  const T h = rn.r[k + 1] - rn.r[k];
  T s = (R - rn.r[k]) / h;
  bool clamped = false;
  if (s < (T)0) {
    s = (T)0;
    clamped = true;
  } else if (s > (T)1) {
    s = (T)1;
    clamped = true;
  }
  const Herm<T> HR = herm<T>(s);
  const T w0 = HR.v0, w1 = HR.v1, u0 = HR.t0 * h, u1 = HR.t1 * h;
  const T c = clamped ? (T)0 : (T)1;
  const T dw0 = c * HR.dv0 / h, dw1 = c * HR.dv1 / h, du0 = c * HR.dt0, du1 = c * HR.dt1;
  const T LN10INV = (T)0.43429448190325182765;  // 1 / ln 10
  const long bx = (long)floor(X0), by = (long)floor(Y0);
  const T fx0 = X0 - (T)bx, fy0 = Y0 - (T)by;
  T c2 = 0, gx0 = 0, gy0 = 0, gphi = 0, gv = 0, gR = 0, gdm = 0;
  const int64_t e0 = off[tr], e1 = off[tr + 1];
  for (int64_t e = e0 + lane; e < e1; e += 32) {
    const T te = t[e];
    const T vt = V * te;
    const T fx = fx0 + vt * cs, fy = fy0 + vt * sn;
    const Bilin<T> B = bilin_weights<T>(bx, fx, by, fy, Nx, Ny);
    if (!B.inside) {
      if (model) model[e] = (T)NAN;
      continue;
    }
    const Herm<T> Hx = herm<T>(B.a), Hy = herm<T>(B.d);
    // corners: (il, jl) (il, jr) (iu, jl) (iu, jr) = (y-node b, x-node a) = (0,0) (0,1) (1,0) (1,1)
    const int rows[4] = {B.il, B.il, B.iu, B.iu}, cols[4] = {B.jl, B.jr, B.jl, B.jr};
    T F = 0, Fx = 0, Fy = 0, FR = 0;
#pragma unroll
    for (int q = 0; q < 4; q++) {
      T v[8];  // M0 X0 Y0 D0 M1 X1 Y1 D1 (radius k, then k+1)
      load8<T>(stack + (((long)rows[q] * Nx + cols[q]) * K + k) * 4, v);
      const T Mc = w0 * v[0] + w1 * v[4] + u0 * v[3] + u1 * v[7];
      const T McR = dw0 * v[0] + dw1 * v[4] + du0 * v[3] + du1 * v[7];
      const T Xc = w0 * v[1] + w1 * v[5], XcR = dw0 * v[1] + dw1 * v[5];
      const T Yc = w0 * v[2] + w1 * v[6], YcR = dw0 * v[2] + dw1 * v[6];
      const bool ax = q & 1, ay = q >> 1;
      const T vx = ax ? Hx.v1 : Hx.v0, tx = ax ? Hx.t1 : Hx.t0, dvx = ax ? Hx.dv1 : Hx.dv0, dtx = ax ? Hx.dt1 : Hx.dt0;
      const T vy = ay ? Hy.v1 : Hy.v0, ty = ay ? Hy.t1 : Hy.t0, dvy = ay ? Hy.dv1 : Hy.dv0, dty = ay ? Hy.dt1 : Hy.dt0;
      F += vx * vy * Mc + tx * vy * Xc + vx * ty * Yc;
      Fx += dvx * vy * Mc + dtx * vy * Xc + dvx * ty * Yc;
      Fy += vx * dvy * Mc + tx * dvy * Xc + vx * dty * Yc;
      FR += vx * vy * McR + tx * vy * XcR + vx * ty * YcR;
    }
    if (!(F > (T)0)) {
      if (model) model[e] = (T)NAN;
      continue;
    }
    const T m = (T)-2.5 * mlc_log10(F) + DM;
    if (model) model[e] = m;
    const T we = w[e];
    const T r = obs[e] - m;
    c2 += we * r * r;
    const T gm = (T)-2 * we * r;             // dchi2/dm
    const T gq = gm * (T)-2.5 * LN10INV / F;  // dchi2/dM
    const T gx = gq * Fx, gy = gq * Fy;
    gdm += gm;
    gx0 += gx;
    gy0 += gy;
    gphi += vt * (cs * gy - sn * gx);
    gv += te * (cs * gx + sn * gy);
    gR += gq * FR;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    c2 += __shfl_xor_sync(0xffffffffu, c2, o);
    gx0 += __shfl_xor_sync(0xffffffffu, gx0, o);
    gy0 += __shfl_xor_sync(0xffffffffu, gy0, o);
    gphi += __shfl_xor_sync(0xffffffffu, gphi, o);
    gv += __shfl_xor_sync(0xffffffffu, gv, o);
    gR += __shfl_xor_sync(0xffffffffu, gR, o);
    gdm += __shfl_xor_sync(0xffffffffu, gdm, o);
  }
  if (lane == 0) {
    if (chi2) chi2[tr] = c2;
    if (grad) {
      T* g = grad + tr * 6;
      g[0] = gx0;
      g[1] = gy0;
      g[2] = gphi;
      g[3] = gv;
      g[4] = gR;
      g[5] = gdm;
    }
  }
}

void track_fit(mlc_ctx* ctx, const void* stack, int Nx, int Ny, int prec, int K, const double* radii, int ntracks,
               const void* theta, const int64_t* off, const void* t, const void* obs, const void* w, void* chi2,
               void* grad, void* model) {
  MLC_REQUIRE(K >= 2 && K <= MLC_FIT_MAX_RADII, MLC_ERR_LIMIT, "2 <= K <= MLC_FIT_MAX_RADII radii");
  for (int k = 0; k + 1 < K; k++) MLC_REQUIRE(radii[k] < radii[k + 1], MLC_ERR_ARG, "radii must increase");
  if (ntracks <= 0) return;
  const int grid = ceil_div(ntracks, 8);
  if (prec == MLC_F64) {
    RadiusNodes<double> rn{};
    rn.K = K;
    for (int k = 0; k < K; k++) rn.r[k] = radii[k];
    MLC_KSCOPE(ctx, "track_fit");
    k_track_fit<double><<<grid, 256, 0, ctx->stream>>>((const double*)stack, Nx, Ny, rn, ntracks,
                                                       (const double*)theta, off, (const double*)t,
                                                       (const double*)obs, (const double*)w, (double*)chi2,
                                                       (double*)grad, (double*)model);
  } else {
    RadiusNodes<float> rn{};
    rn.K = K;
    for (int k = 0; k < K; k++) rn.r[k] = (float)radii[k];
    MLC_KSCOPE(ctx, "track_fit");
    k_track_fit<float><<<grid, 256, 0, ctx->stream>>>((const float*)stack, Nx, Ny, rn, ntracks, (const float*)theta,
                                                      off, (const float*)t, (const float*)obs, (const float*)w,
                                                      (float*)chi2, (float*)grad, (float*)model);
  }
  MLC_CHECK_LAUNCH();
}

void radius_stack(mlc_ctx* ctx, mlc_map* map, int K, const double* radii, double pix, int N, void* stack) {
  MLC_REQUIRE(K >= 2 && K <= MLC_FIT_MAX_RADII, MLC_ERR_LIMIT, "2 <= K <= MLC_FIT_MAX_RADII radii");
  for (int k = 0; k < K; k++) MLC_REQUIRE(radii[k] > 0 && (k == 0 || radii[k - 1] < radii[k]), MLC_ERR_ARG,
                                          "radii must be positive and increasing");
  MLC_REQUIRE(N >= 2 && N % 2 == 0 && N <= map->Nx && N <= map->Ny, MLC_ERR_ARG,
              "raster side must be even and at most the map side");
  map_prepare(ctx, map);
  FftPlan2D* p = plan_get(ctx, map->Nx, map->Ny, map_fft_prec(map));
  const size_t n2 = (size_t)N * N;
  std::vector<double> h(4 * n2 * K);  // per radius: P, dP/dx, dP/dy, dP/dR
  for (int k = 0; k < K; k++) {
    double* b = h.data() + 4 * k * n2;
    MLC_REQUIRE(thin_disc_fit_raster(radii[k], pix, N, b, b + n2, b + 2 * n2, b + 3 * n2) == N, MLC_ERR_ARG,
                "raster failed");
  }
  double* dprof = (double*)ws_get(ctx, WS_PROFILE, h.size() * sizeof(double));
  MLC_CUDA(cudaStreamSynchronize(ctx->stream));
  MLC_CUDA(cudaMemcpy(dprof, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice));
  const long npix = (long)map->Nx * map->Ny;
  const size_t es = map->prec == MLC_F64 ? 8 : 4;
  constexpr int G = 4;  // radii per group: 16 convolved maps, then one interleave pass
  char* tmp = (char*)ws_get(ctx, WS_BATCH_MAPS, (size_t)4 * G * npix * es);
  for (int g0 = 0; g0 < K; g0 += G) {
    const int ng = std::min(G, K - g0);
    const void* mp[16];
    for (int j = 0; j < 4 * ng; j++) {
      mp[j] = tmp + (size_t)j * npix * es;
      conv_fused(ctx, *p, map->spec, dprof + (size_t)(4 * g0 + j) * n2, N, (void*)mp[j]);
    }
    interleave_into(ctx, mp, 4 * ng, npix, map->prec, 4 * K, 4 * g0, stack);
  }
}

}  // namespace mlc
