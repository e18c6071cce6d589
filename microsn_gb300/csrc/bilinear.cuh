// Bilinear sampling weights shared by the track sampler (sample.cu) and the
// differentiable track fit (fit.cu).
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

template <typename T>
__device__ __forceinline__ Bilin<T> bilin_weights(long bx, T fx, long by, T fy, int Nx, int Ny) {
  Bilin<T> B;
  // absolute coordinate = b + f ; hull of centres is [0.5, N - 0.5]
  const T flx = floor(fx), fly = floor(fy);
  const long jx = bx + (long)flx, iy = by + (long)fly;  // pixel containing the point
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

}  // namespace mlc
