// Bilinear sampling weights shared by the track samplers (sample.cu, and the pair sides
// of pairdiff.cu) and the differentiable track fit (fit.cu).
#pragma once

#include "mlc_common.cuh"

namespace mlc {

__device__ __forceinline__ double mlc_log10(double x) { return log10_f32x2(x); }
__device__ __forceinline__ float mlc_log10(float x) { return log10f(x); }

// Bilinear weights of RectGrid::interp2d_bilinear (rectGrid.cpp:349-378) on pixel
// centres j + 1/2.  The position is split into an exact integer base (bx, by) and a
// small offset (fx, fy) so that FP32 keeps sub-pixel precision far from the origin.
template <typename T>
struct Bilin {
  int jl, jr, il, iu;
  T w0, w1, w2, w3;  // (iu,jl) (iu,jr) (il,jl) (il,jr)
  T a, d;            // x - centre(jl), y - centre(il), both in [0, 1]
  bool inside;
};

// Whole numbers to 64-bit integers.  FP32 goes through a 32-bit integer: F2I.S64 runs on
// the FP64 pipe, F2I.S32 does not.  FP32 offsets are fractions here, and FP32 track
// coordinates stay far inside +-2^31 pixels; FP64 ones may not, and convert directly.
__device__ __forceinline__ long floor_to_long(float f) { return (long)(int)f; }
__device__ __forceinline__ long floor_to_long(double f) { return (long)f; }

template <typename T>
__device__ __forceinline__ Bilin<T> bilin_weights(long bx, T fx, long by, T fy, int Nx, int Ny) {
  Bilin<T> B;
  // absolute coordinate = b + f ; hull of centres is [0.5, N - 0.5]
  const T flx = floor(fx), fly = floor(fy);
  const long jx = bx + floor_to_long(flx), iy = by + floor_to_long(fly);  // pixel containing the point
  const T rx = fx - flx, ry = fy - fly;                 // in [0, 1)
  B.inside = !((jx < 0) || (jx == 0 && rx < (T)0.5) || (jx > Nx - 1) || (jx == Nx - 1 && rx > (T)0.5) ||
               (iy < 0) || (iy == 0 && ry < (T)0.5) || (iy > Ny - 1) || (iy == Ny - 1 && ry > (T)0.5));
  const T dx = rx - (T)0.5, dy = ry - (T)0.5;
  const long jl = (dx < 0) ? jx - 1 : jx;
  const long iu = (dy < 0) ? iy : iy + 1;
  // a = x - centre(jl), b = centre(jl+1) - x, c = centre(iu) - y, d = y - centre(iu-1)
  const T a = (dx < 0) ? rx + (T)0.5 : dx;
  const T b = (T)1 - a;
  const T d = (dy < 0) ? ry + (T)0.5 : dy;
  const T c = (T)1 - d;
  B.jl = (int)jl;
  B.jr = (int)min(jl + 1, (long)Nx - 1);
  B.iu = (int)min(iu, (long)Ny - 1);
  B.il = (int)(iu - 1);
  B.a = a;
  B.d = d;
  B.w0 = b * d;
  B.w1 = a * d;
  B.w2 = b * c;
  B.w3 = a * c;
  return B;
}

// The bilinear value of one map at the weights B (points outside the hull are the caller's).
template <typename T>
__device__ __forceinline__ T bilin_read(const T* __restrict__ m, const Bilin<T>& B, int Nx) {
  T z = B.w0 * __ldg(m + (long)B.iu * Nx + B.jl);
  z += B.w1 * __ldg(m + (long)B.iu * Nx + B.jr);
  z += B.w2 * __ldg(m + (long)B.il * Nx + B.jl);
  z += B.w3 * __ldg(m + (long)B.il * Nx + B.jr);
  return z;
}

// sin and cos of an FP32 angle as float-float pairs, our own evaluation: Cody-Waite
// reduction by pi/2 (split into P1 + P2 + P3, the first two of 12 significant bits so that
// k P1 and k P2 are exact products; every step a float-float sum), then the Taylor series of
// sin and cos on |r| <= pi/4 (nine and ten terms, the first omitted term below 1e-16), in
// float-float arithmetic.  About 1e-14 absolute for |phi| < 2^12 pi/2; larger angles take
// the FP32 library values (about 1e-7).
__device__ __forceinline__ void sincos_ff(float phi, ff* sn, ff* cs) {
  if (!(fabsf(phi) < 6433.0f)) {
    float s_, c_;
    sincosf(phi, &s_, &c_);
    *sn = ff(s_, 0.f);
    *cs = ff(c_, 0.f);
    return;
  }
  const float kf = rintf(__fmul_rn(phi, 0.636619772367581343f));  // nearest multiple of pi/2
  const float P1 = 1.5703125f, P2 = 4.837512969970703125e-4f, P3 = 7.549790126404332e-08f;
  const float kp3 = __fmul_rn(kf, P3);
  ff r = ff(phi, 0.f) - ff(__fmul_rn(kf, P1), 0.f);  // k P1, k P2: exact products
  r = r - ff(__fmul_rn(kf, P2), 0.f);
  r = r - ff(kp3, __fmaf_rn(kf, P3, -kp3));            // k P3 as an exact two-product
  r = ff_norm(r);
  const ff z = r * r;
  // sin r = r (1 - z/3! + z^2/5! - ...), cos r = 1 - z/2! + z^2/4! - ...: the
  // coefficients (-1)^n / (2n+1)! and (-1)^n / (2n)! as float-float pairs
  ff p = ff(2.8114573589663704e-15f, -1.0462084739763658e-22f);  // 1/17!
  p = ff(-7.647163609812713e-13f, -1.2200710471178288e-20f) + z * p;
  p = ff(1.6059044372074283e-10f, -5.352526511562726e-18f) + z * p;
  p = ff(-2.5052107943679403e-08f, -4.4176230446483665e-16f) + z * p;
  p = ff(2.7557318844628753e-06f, 3.793571224297229e-14f) + z * p;
  p = ff(-0.00019841270113829523f, 2.725596874933456e-12f) + z * p;
  p = ff(0.008333333767950535f, -4.34617203337595e-10f) + z * p;
  p = ff(-0.1666666716337204f, 4.967053879312289e-09f) + z * p;  // -1/3!
  p = ff(1.0f, 0.f) + z * p;
  const ff s = ff_norm(r * p);
  ff q = ff(-1.5619206814541513e-16f, -1.5404471465941993e-24f);  // -1/18!
  q = ff(4.7794772561329454e-14f, 7.62544404448643e-22f) + z * q;
  q = ff(-1.147074536050896e-11f, -2.372207689231238e-19f) + z * q;
  q = ff(2.0876755879584152e-09f, 1.1082839147459852e-16f) + z * q;
  q = ff(-2.755731998149713e-07f, 7.575112209051195e-15f) + z * q;
  q = ff(2.4801587642286904e-05f, -3.40699609366682e-13f) + z * q;
  q = ff(-0.0013888889225199819f, 3.3631094437103215e-11f) + z * q;
  q = ff(0.0416666679084301f, -1.2417634698280722e-09f) + z * q;
  q = ff(-0.5f, 0.f) + z * q;
  q = ff(1.0f, 0.f) + z * q;
  const ff c = ff_norm(q);
  switch (((int)kf) & 3) {
    case 0: *sn = s; *cs = c; break;
    case 1: *sn = c; *cs = -s; break;
    case 2: *sn = -s; *cs = -c; break;
    default: *sn = -c; *cs = s; break;
  }
}

// Offset f0 + t vc of a track epoch from the track's pixel base (vc = V cos phi or V sin phi
// as a float-float pair), returned as whole pixels *d and a fraction in [0, 1) rounded to
// FP32 (6e-8 px).  The displacement runs to thousands of pixels, where an FP32 sum would be
// off by up to 5e-4 px, so it is formed in float-float arithmetic.
__device__ __forceinline__ float track_offset(float f0, float t, ff vc, long* d) {
  const float ph = __fmul_rn(t, vc.hi);
  const ff x = ff(f0, 0.f) + ff(ph, __fmaf_rn(t, vc.lo, __fmaf_rn(t, vc.hi, -ph)));
  const float fl = floorf(x.hi);
  float r = __fadd_rn(__fsub_rn(x.hi, fl), x.lo);
  long dd = floor_to_long(fl);
  if (r < 0.f) {
    r = __fadd_rn(r, 1.f);
    dd -= 1;
  } else if (r >= 1.f) {
    r = __fsub_rn(r, 1.f);
    dd += 1;
  }
  *d = dd;
  return r;
}

// A straight track x0 + V t (cos phi, sin phi): the bilinear weights at epoch t.  The start
// is split into an exact integer pixel base and an offset in [0, 1).  FP64 tracks form the
// position in FP64; FP32 tracks in float-float (sincos_ff, track_offset), so that FP32 light
// curves are limited by the maps' FP32 values, not by the position arithmetic.
template <typename T>
struct TrackGeom;

template <>
struct TrackGeom<double> {
  long bx, by;
  double fx0, fy0, V, c, s;
  __device__ __forceinline__ TrackGeom(double X0, double Y0, double phi, double V_) : V(V_) {
    sincos(phi, &s, &c);
    bx = (long)floor(X0);
    by = (long)floor(Y0);
    fx0 = X0 - (double)bx;
    fy0 = Y0 - (double)by;
  }
  __device__ __forceinline__ Bilin<double> at(double t, int Nx, int Ny) const {
    const double vt = V * t;
    return bilin_weights<double>(bx, fx0 + vt * c, by, fy0 + vt * s, Nx, Ny);
  }
};

template <>
struct TrackGeom<float> {
  long bx, by;
  float fx0, fy0;
  ff vc, vs;  // V cos phi, V sin phi
  __device__ __forceinline__ TrackGeom(float X0, float Y0, float phi, float V) {
    ff c, s;
    sincos_ff(phi, &s, &c);
    vc = ff_norm(ff(V, 0.f) * c);
    vs = ff_norm(ff(V, 0.f) * s);
    bx = floor_to_long(floorf(X0));
    by = floor_to_long(floorf(Y0));
    fx0 = X0 - (float)bx;  // exact
    fy0 = Y0 - (float)by;
  }
  __device__ __forceinline__ Bilin<float> at(float t, int Nx, int Ny) const {
    long dx, dy;
    const float rx = track_offset(fx0, t, vc, &dx);
    const float ry = track_offset(fy0, t, vs, &dy);
    return bilin_weights<float>(bx + dx, rx, by + dy, ry, Nx, Ny);
  }
};

}  // namespace mlc
