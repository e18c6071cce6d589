// Host FP64 rasters of the source profiles, replacing the reference's profile classes
// and FactoryProfile::createProfileFromHalfRadius (simulating_lcurves/include/profile.hpp:142-166,
// src/profile.cpp:143-446).  Rasters are small (at most a few hundred pixels a side) and
// are uploaded once per convolution; the full-size wrapped kernel of the reference is
// never built on the host.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "mlc_internal.h"

namespace mlc {

namespace {

// std::to_string then std::stof, the reference's parameter round trip.
double roundtrip(double v) {
  char buf[512];
  std::snprintf(buf, sizeof buf, "%f", v);
  return (double)std::strtof(buf, nullptr);
}

int even(int n) { return (n % 2 != 0) ? n + 1 : n; }

struct Resolved {
  int shape, N;
  double pix, incl, orient, R, sdev, Rin, a, b, sigma, u, Rhalf;
};

bool resolve(const mlc_profile& in, Resolved& r) {
  std::memset(&r, 0, sizeof r);
  double rhalf = in.rhalf, pix = in.pix, incl = in.incl, orient = in.orient, Rin = in.Rin, a = in.a;
  if (in.ref_compat) {
    rhalf = roundtrip(rhalf);
    pix = roundtrip(pix);
    incl = roundtrip(incl);
    orient = roundtrip(orient);
    Rin = roundtrip(Rin);
    a = roundtrip(a);
  }
  if (!(pix > 0) || !(rhalf > 0)) return false;
  r.shape = in.shape;
  r.pix = pix;
  r.incl = incl;
  r.orient = orient;
  switch (in.shape) {
    case MLC_SHAPE_UNIFORM:  // UniformDisc: R = sqrt(2) rhalf, N = 2 (3 + ceil(R/pix))
      r.R = std::sqrt(2.0) * rhalf;
      r.N = even(2 * (3 + (int)std::ceil(r.R / pix)));
      break;
    case MLC_SHAPE_GAUSSIAN:  // sdev = rhalf/1.18, N = ceil(4 Rhalf / pix)
      r.sdev = rhalf / 1.18;
      r.Rhalf = 1.18 * r.sdev;
      r.N = even((int)std::ceil(4.0 * r.Rhalf / pix));
      break;
    case MLC_SHAPE_GAUSSIAN_HOLE:
      r.Rin = Rin;
      r.sdev = std::sqrt((std::pow(rhalf, 2.0) - std::pow(Rin, 2.0)) / (2.0 * std::log(2.0)));
      r.Rhalf = std::sqrt(2.0 * std::log(2.0) * std::pow(r.sdev, 2.0) + std::pow(Rin, 2.0));
      r.N = even((int)std::ceil(4.0 * r.Rhalf / pix));
      if (!(r.sdev > 0)) return false;
      break;
    case MLC_SHAPE_THERMAL_HOLE:
      r.Rin = rhalf / 4.0;
      r.Rhalf = 4.0 * r.Rin;
      r.N = even((int)std::ceil(4.0 * r.Rhalf / pix));
      break;
    case MLC_SHAPE_WAVY:  // three nodes
      r.a = a;
      r.b = 3 * M_PI / (2.0 * rhalf);
      r.Rhalf = 3 * M_PI / (2.0 * r.b);
      r.N = even((int)std::ceil(4.0 * r.Rhalf / pix));
      break;
    case MLC_SHAPE_EXPONENTIAL:  // thin disc 1/(exp((r/sigma)^(3/4)) - 1)
      r.sigma = 0.4106 * rhalf;
      r.Rhalf = r.sigma / 0.4106;
      r.N = even((int)std::ceil(4.0 * r.Rhalf / pix));
      break;
    case MLC_SHAPE_LIMB_DARKENED:  // I = 1 - u (1 - sqrt(1 - (r/R)^2)), R = sqrt(2) rhalf
      r.u = in.u;
      r.R = std::sqrt(2.0) * rhalf;
      r.N = even(2 * (3 + (int)std::ceil(r.R / pix)));
      break;
    default:
      return false;
  }
  return r.N > 0;
}

}  // namespace

int profile_dims(const mlc_profile& p) {
  Resolved r;
  if (!resolve(p, r)) return -1;
  return r.N;
}

int profile_raster(const mlc_profile& p, double* out, long cap) {
  Resolved r;
  if (!resolve(p, r)) return -1;
  const int N = r.N;
  if ((long)N * N > cap) return -2;
  // grid and projection: BaseProfile::createGrid / project (profile.cpp:126-157)
  const double fac = M_PI / 180.0;
  const double costheta = std::cos(fac * r.incl);
  const double cosphi = std::cos(fac * (-r.orient));
  const double sinphi = std::sin(fac * (-r.orient));
  double v_inner = 0.0, r_inner = 0.0;
  if (r.shape == MLC_SHAPE_EXPONENTIAL) {
    v_inner = 10.0 / (std::exp(std::pow(r.Rhalf / r.sigma, 0.75)) - 1.0);
    r_inner = r.sigma * std::pow(std::log(1.0 + 1.0 / v_inner), 4.0 / 3.0);
  }
  const double sg = 2 * std::pow(r.sdev, 2);
  const double thfac = 3.0 * r.Rin / (2.0 * M_PI);
  for (int i = 0; i < N; i++) {
    const double y0 = (i - N / 2) * r.pix + r.pix / 2.0;
    for (int j = 0; j < N; j++) {
      const double x0 = (j - N / 2) * r.pix + r.pix / 2.0;
      const double x = x0 * cosphi / costheta + y0 * sinphi / costheta;
      const double y = -sinphi * x0 + cosphi * y0;
      const double rr = std::hypot(x, y);
      double v = 0.0;
      switch (r.shape) {
        case MLC_SHAPE_UNIFORM: v = (rr < r.R) ? 1.0 : 0.0; break;
        case MLC_SHAPE_GAUSSIAN: v = std::exp(-rr * rr / sg); break;
        case MLC_SHAPE_GAUSSIAN_HOLE: v = (rr < r.Rin) ? 0.0 : std::exp(-rr * rr / sg); break;
        case MLC_SHAPE_THERMAL_HOLE:
          v = (rr > r.Rin) ? (1.0 - std::sqrt(r.Rin / rr)) * thfac / std::pow(rr, 3.0) : 0.0;
          break;
        case MLC_SHAPE_WAVY: v = (rr < 2 * r.Rhalf) ? std::pow(std::sin(r.b * rr), 2) / (r.a * rr) : 0.0; break;
        case MLC_SHAPE_EXPONENTIAL:
          // The reference overwrites the flat core (profile.cpp:435-441); ref_compat keeps that.
          if (!p.ref_compat && rr < r_inner) v = v_inner;
          else if (rr < 2 * r.Rhalf) v = 1.0 / (std::exp(std::pow(rr / r.sigma, 0.75)) - 1.0);
          else v = 0.0;
          break;
        case MLC_SHAPE_LIMB_DARKENED:
          if (rr < r.R) {
            const double q = rr / r.R;
            v = 1.0 - r.u * (1.0 - std::sqrt(1.0 - q * q));
          }
          break;
      }
      out[(long)i * N + j] = v;
    }
  }
  // BaseProfile::normalize (profile.cpp:158-174): row-major sum, then divide
  double sum = 0.0;
  for (long k = 0; k < (long)N * N; k++) sum += out[k];
  for (long k = 0; k < (long)N * N; k++) out[k] /= sum;
  return N;
}

// Thin-disc raster for differentiable fits: the reference's thin-disc law
// (profile.cpp:402-446) I(r) = 1 / (exp((r/sigma)^(3/4)) - 1), sigma = 0.4106 R_half,
// with its flat core (I <= I_core = 10 / (exp((R_half/sigma)^(3/4)) - 1), a constant), but
// on a fixed N x N grid and without the truncation at r = 2 R_half, so that the normalised
// raster P is smooth in R_half.  Pixel centres as in createGrid (profile.cpp:126-157):
// (j - N/2) pix + pix/2.  Also returns the derivative rasters of the same continuous
// profile at the same offsets: dPdx, dPdy per pixel of offset (x = column, y = row) and
// dPdR per unit of R_half, dP/dR = (dI/dR) / S - P sum(dI/dR) / S with S = sum I.
// Any of the derivative outputs may be null.
int thin_disc_fit_raster(double rhalf, double pix, int N, double* P, double* dPdx, double* dPdy, double* dPdR) {
  if (!(rhalf > 0) || !(pix > 0) || N < 2 || (N & 1)) return -1;
  const double sigma = 0.4106 * rhalf;
  const double v_core = 10.0 / (std::exp(std::pow(rhalf / sigma, 0.75)) - 1.0);
  double S = 0.0, SdR = 0.0;
  for (int i = 0; i < N; i++) {
    const double y = (i - N / 2) * pix + pix / 2.0;
    for (int j = 0; j < N; j++) {
      const double x = (j - N / 2) * pix + pix / 2.0;
      const double r = std::hypot(x, y);
      const double u = r / sigma;
      const double e = std::exp(std::pow(u, 0.75));
      const double f = 1.0 / (e - 1.0);
      double v, dx = 0.0, dy = 0.0, dR = 0.0;
      if (f >= v_core) {  // core: constant, independent of position and R
        v = v_core;
      } else {
        v = f;
        const double fp = -0.75 * std::pow(u, -0.25) * e / ((e - 1.0) * (e - 1.0));  // dI/du
        dx = fp * x / (r * sigma) * pix;
        dy = fp * y / (r * sigma) * pix;
        dR = -fp * u / rhalf;
      }
      const long q = (long)i * N + j;
      P[q] = v;
      if (dPdx) dPdx[q] = dx;
      if (dPdy) dPdy[q] = dy;
      if (dPdR) dPdR[q] = dR;
      S += v;
      SdR += dR;
    }
  }
  for (long q = 0; q < (long)N * N; q++) {
    P[q] /= S;
    if (dPdx) dPdx[q] /= S;
    if (dPdy) dPdy[q] /= S;
    if (dPdR) dPdR[q] = dPdR[q] / S - P[q] * SdR / S;
  }
  return N;
}

}  // namespace mlc
