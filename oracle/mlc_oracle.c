/*
 * mlc_oracle.c -- CPU oracle for the microLC light-curve hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file restates, in plain FP64 C, the reference's
 * algorithm for each stage of the path so that the CUDA library can be checked
 * against it.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
 * load it; the product library never does.
 *
 * Parity pins: every function that has a counterpart in the reference's own CPU
 * code (profiles, kernel wrap, chi2 set-up, rank table, ref-ratio chi2, bin means,
 * bin edges, trapezium) is checked in tests/ against that code compiled from the
 * reference sources (oracle/_ref/libmlcref.so) and against committed golden vectors.
 * Functions for capabilities the reference does not have (bilinear tracks,
 * magnitudes, offset-minimised chi2, magnitude-difference pair chi2, histograms,
 * top-k) follow the mathematics stated beside them; their parity is unpinned by the
 * reference, except the bilinear degenerate case, which reduces to kernel_sample.
 *
 * Built with -ffp-contract=off so that x86 and Arm hosts give identical results.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

enum {
  ORC_UNIFORM = 0,
  ORC_GAUSSIAN = 1,
  ORC_GAUSSIAN_HOLE = 2,
  ORC_THERMAL_HOLE = 3,
  ORC_WAVY = 4,
  ORC_EXPONENTIAL = 5,
  ORC_LIMB_DARKENED = 6
};

/* std::to_string(double) followed by std::stof: the reference passes every profile
 * parameter through this string round trip (gpu_functions.cu:108,184; profile.hpp:142-166). */
static double str_round_float(double v) {
  char buf[512];
  snprintf(buf, sizeof buf, "%f", v);
  return (double)strtof(buf, NULL);
}

static int make_even(int n) { return (n % 2 != 0) ? n + 1 : n; } /* profile.cpp:175-179 */

/* Profile parameters after the half-radius conversion (profile.hpp:142-166). */
typedef struct {
  int shape, N;
  double pix, incl, orient;
  double R, sdev, Rin, a, b, sigma, u; /* shape-specific */
  double Rhalf;
} orc_prof;

static int prof_setup(int shape, double rhalf, double pix, double incl, double orient, double Rin,
                      double a, double u, int ref_compat, orc_prof* p) {
  memset(p, 0, sizeof *p);
  p->shape = shape;
  if (ref_compat) {
    rhalf = str_round_float(rhalf);
    pix = str_round_float(pix);
    incl = str_round_float(incl);
    orient = str_round_float(orient);
    Rin = str_round_float(Rin);
    a = str_round_float(a);
  }
  p->pix = pix;
  p->incl = incl;
  p->orient = orient;
  switch (shape) {
    case ORC_UNIFORM: /* profile.cpp:185-199 */
      p->R = sqrt(2.0) * rhalf;
      p->N = make_even(2 * (3 + (int)ceil(p->R / pix)));
      break;
    case ORC_GAUSSIAN: /* profile.cpp:228-245 */
      p->sdev = rhalf / 1.18;
      p->Rhalf = 1.18 * p->sdev;
      p->N = make_even((int)ceil(4.0 * p->Rhalf / pix));
      break;
    case ORC_GAUSSIAN_HOLE: /* profile.cpp:269-291 */
      p->Rin = Rin;
      p->sdev = sqrt((pow(rhalf, 2.0) - pow(Rin, 2.0)) / (2.0 * log(2.0)));
      p->Rhalf = sqrt(2.0 * log(2.0) * pow(p->sdev, 2.0) + pow(Rin, 2.0));
      p->N = make_even((int)ceil(4.0 * p->Rhalf / pix));
      break;
    case ORC_THERMAL_HOLE: /* profile.cpp:315-333 */
      p->Rin = rhalf / 4.0;
      p->Rhalf = 4.0 * p->Rin;
      p->N = make_even((int)ceil(4.0 * p->Rhalf / pix));
      break;
    case ORC_WAVY: /* profile.cpp:358-378, node = 3 */
      p->a = a;
      p->b = 3 * M_PI / (2.0 * rhalf);
      p->Rhalf = 3 * M_PI / (2.0 * p->b);
      p->N = make_even((int)ceil(4.0 * p->Rhalf / pix));
      break;
    case ORC_EXPONENTIAL: /* profile.cpp:402-420 */
      p->sigma = 0.4106 * rhalf;
      p->Rhalf = p->sigma / 0.4106;
      p->N = make_even((int)ceil(4.0 * p->Rhalf / pix));
      break;
    case ORC_LIMB_DARKENED:
      /* No reference counterpart.  Linear limb darkening I = 1 - u (1 - mu),
       * mu = sqrt(1 - (r/R)^2), for r < R; the radius is given directly by rhalf*sqrt(2)
       * (the half-light radius of the u = 0 disc), raster 2*(3+ceil(R/pix)) like the disc. */
      p->u = u;
      p->R = sqrt(2.0) * rhalf;
      p->N = make_even(2 * (3 + (int)ceil(p->R / pix)));
      break;
    default:
      return 1;
  }
  return 0;
}

int orc_profile_dims(int shape, double rhalf, double pix, double Rin, double a, int ref_compat) {
  orc_prof p;
  if (prof_setup(shape, rhalf, pix, 0.0, 0.0, Rin, a, 0.0, ref_compat, &p)) return -1;
  return p.N;
}

/* Raster of the normalised profile, N x N row-major (profile.cpp:143-174 grid,
 * projection and normalisation; values per shape as cited in prof_setup). */
int orc_profile_raster(int shape, double rhalf, double pix, double incl, double orient, double Rin,
                       double a, double u, int ref_compat, double* out, long cap) {
  orc_prof p;
  if (prof_setup(shape, rhalf, pix, incl, orient, Rin, a, u, ref_compat, &p)) return -1;
  int N = p.N;
  if ((long)N * N > cap) return -2;
  double fac = M_PI / 180.0;
  double costheta = cos(fac * p.incl);
  double cosphi = cos(fac * (-p.orient));
  double sinphi = sin(fac * (-p.orient));
  double v_inner = 0.0, r_inner = 0.0;
  if (shape == ORC_EXPONENTIAL) {
    v_inner = 10.0 / (exp(pow(p.Rhalf / p.sigma, 0.75)) - 1.0);
    r_inner = p.sigma * pow(log(1.0 + 1.0 / v_inner), 4.0 / 3.0);
  }
  double sgauss = 2 * pow(p.sdev, 2);
  double thfac = 3.0 * p.Rin / (2.0 * M_PI);
  for (int i = 0; i < N; i++) {
    double y0 = (i - N / 2) * p.pix + p.pix / 2.0;
    for (int j = 0; j < N; j++) {
      double x0 = (j - N / 2) * p.pix + p.pix / 2.0;
      double x = x0 * cosphi / costheta + y0 * sinphi / costheta;
      double y = -sinphi * x0 + cosphi * y0;
      double r = hypot(x, y);
      double v = 0.0;
      switch (shape) {
        case ORC_UNIFORM: v = (r < p.R) ? 1.0 : 0.0; break;
        case ORC_GAUSSIAN: v = exp(-r * r / sgauss); break;
        case ORC_GAUSSIAN_HOLE: v = (r < p.Rin) ? 0.0 : exp(-r * r / sgauss); break;
        case ORC_THERMAL_HOLE: v = (r > p.Rin) ? (1.0 - sqrt(p.Rin / r)) * thfac / pow(r, 3.0) : 0.0; break;
        case ORC_WAVY: v = (r < 2 * p.Rhalf) ? pow(sin(p.b * r), 2) / (p.a * r) : 0.0; break;
        case ORC_EXPONENTIAL:
          /* profile.cpp:435-441: the r < r_inner value is overwritten by the following
           * if/else (missing "else"); ref_compat keeps that, otherwise the core is flat. */
          if (!ref_compat && r < r_inner) v = v_inner;
          else if (r < 2 * p.Rhalf) v = 1.0 / (exp(pow(r / p.sigma, 0.75)) - 1.0);
          else v = 0.0;
          break;
        case ORC_LIMB_DARKENED:
          if (r < p.R) {
            double q = r / p.R;
            v = 1.0 - p.u * (1.0 - sqrt(1.0 - q * q));
          }
          break;
      }
      out[(long)i * N + j] = v;
    }
  }
  double sum = 0.0;
  for (long k = 0; k < (long)N * N; k++) sum += out[k];
  for (long k = 0; k < (long)N * N; k++) out[k] /= sum;
  return N;
}

/* Kernel::setKernel (magnification_map.cpp:172-193): the four quadrants of an
 * N x N profile placed at the corners of a zeroed Nx x Ny array. */
void orc_kernel_wrap(const double* prof, int pN, int Nx, int Ny, double* out) {
  int h = pN / 2;
  memset(out, 0, sizeof(double) * (size_t)Nx * Ny);
  for (int i = 0; i < h; i++)
    for (int j = 0; j < h; j++) {
      out[(long)i * Nx + j] = prof[(long)(h + i) * pN + h + j];
      out[(long)i * Nx + Nx - h + j] = prof[(long)(h + i) * pN + j];
      out[(long)(Ny - h + i) * Nx + j] = prof[(long)i * pN + h + j];
      out[(long)(Ny - h + i) * Nx + Nx - h + j] = prof[(long)i * pN + j];
    }
}

/* Direct circular convolution of a map with the wrapped profile: the same result as
 * the reference's D2Z(map) * D2Z(kernel) / (Nx Ny) -> Z2D (gpu_functions.cu:175-200,
 * 571-577), evaluated without an FFT.  out[y][x] = sum_ij map[y-i+h][x-j+h] prof[i][j]. */
void orc_conv_direct(const double* map, int Nx, int Ny, const double* prof, int pN, double* out) {
  int h = pN / 2;
  for (int y = 0; y < Ny; y++)
    for (int x = 0; x < Nx; x++) {
      double acc = 0.0;
      for (int i = 0; i < pN; i++) {
        int yy = ((y - i + h) % Ny + Ny) % Ny;
        const double* row = map + (long)yy * Nx;
        const double* pr = prof + (long)i * pN;
        for (int j = 0; j < pN; j++) {
          int xx = ((x - j + h) % Nx + Nx) % Nx;
          acc += row[xx] * pr[j];
        }
      }
      out[(long)y * Nx + x] = acc;
    }
}

/* kernel_sample (gpu_functions.cu:604-620): nearest-pixel read into LC[id*Nprof+k]
 * and the adjacent difference into DLC[id*(Nprof-1)+k-1]. */
void orc_sample_nearest(const double* map, int Nx, int k, int Nprof, int Nloc, const int* lx,
                        const int* ly, double* LC, double* DLC) {
  for (int id = 0; id < Nloc; id++) {
    double v = map[(long)ly[id] * Nx + lx[id]];
    LC[(long)id * Nprof + k] = v;
    if (k > 0) DLC[(long)id * (Nprof - 1) + k - 1] = v - LC[(long)id * Nprof + k - 1];
  }
}

/* find_indices (cpu_functions.cpp:28-45).  The reference leaves entries unset when a
 * time equals or falls below the size range; here they are set to -1. */
void orc_find_indices(const double* t, const double* x, int Nd, int Nprof, int* ind) {
  for (int i = 0; i < Nd; i++) ind[i] = -1;
  int i = 0, j = 0;
  while (i < Nd && j < Nprof - 1) {
    double comp = t[i];
    if (x[j] <= comp && comp < x[j + 1]) {
      ind[i] = j;
      i++;
    } else if (comp > x[Nprof - 1]) {
      ind[i] = -1;
      i++;
    } else {
      j++;
    }
  }
}

/* setup_chi2_calculation (cpu_functions.cpp:80-144), M = {MA, MB}, V = {V0}.
 * ref_compat keeps the constant-term loop over i = Nd-Njp .. Nd-1 (:138); otherwise
 * the loop covers the dropped epochs i = Njp .. Nd-1. Returns Njp. */
int orc_setup_chi2(double MA, double MB, double V0, double Dfac, int Nd, const double* d,
                   const double* t, const double* s, int Nprof, const double* x, int ref_compat,
                   int* indA, int* indB, double* facA, double* facB, double* nd, double* ns,
                   double* const_term) {
  double Rfac = 23.92865 * Dfac;
  double t2xA = V0 * 8.64 / (Rfac * sqrt(MA));
  double t2xB = V0 * 8.64 / (Rfac * sqrt(MB));
  double* tA = (double*)malloc(sizeof(double) * (Nd + 1));
  double* tB = (double*)malloc(sizeof(double) * (Nd + 1));
  int* iA = (int*)malloc(sizeof(int) * (Nd + 1));
  int* iB = (int*)malloc(sizeof(int) * (Nd + 1));
  for (int i = 0; i < Nd; i++) {
    tA[i] = t2xA * t[i];
    tB[i] = t2xB * t[i];
  }
  orc_find_indices(tA, x, Nd, Nprof, iA);
  orc_find_indices(tB, x, Nd, Nprof, iB);
  int Njp = Nd;
  for (int i = 0; i < Nd; i++)
    if (iA[i] == -1 && iB[i] == -1) {
      Njp = i;
      break;
    }
  for (int i = 0; i < Njp; i++) {
    indA[i] = iA[i];
    indB[i] = iB[i];
    nd[i] = d[i];
    ns[i] = s[i];
    facA[i] = (iA[i] != -1) ? (tA[i] - x[iA[i]]) / (x[iA[i] + 1] - x[iA[i]]) : 0;
    facB[i] = (iB[i] != -1) ? (tB[i] - x[iB[i]]) / (x[iB[i] + 1] - x[iB[i]]) : 0;
  }
  double c = 0.0;
  if (Njp != Nd) {
    int i0 = ref_compat ? Nd - Njp : Njp;
    for (int i = i0; i < Nd; i++) c += pow((d[i] - 1) / s[i], 2);
  }
  *const_term = c;
  free(tA); free(tB); free(iA); free(iB);
  return Njp;
}

/* ---- pair z, rank table, z bins (gpu_functions.cu:351-401, kernel_z :643-658) ---- */

/* The reference sorts z with thrust::stable_sort_by_key on doubles, a radix sort over the
 * bit patterns: negative values (sign bit set) by their inverted bits, the rest above them;
 * -0.0 ranks as +0.0; NaN ranks by its sign bit (a negative NaN before -inf, a positive
 * one after +inf).  Ties keep the pair order. */
static uint64_t radix_key(double d) {
  uint64_t u;
  memcpy(&u, &d, 8);
  if (u == 0x8000000000000000ull) u = 0;
  return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}

/* z = a / b as kernel_z computes it on the GPU: a NaN operand passes through (sign
 * included); 0/0 and inf/inf give the GPU's default NaN, whose sign bit is set (the host's
 * default NaN differs between machines). */
static double gpu_div(double a, double b) {
  if (a != a) return a;
  if (b != b) return b;
  double z = a / b;
  if (z != z) {
    const uint64_t u = 0xfff8000000000000ull;
    memcpy(&z, &u, 8);
  }
  return z;
}

static const double* g_sort_keys;
static int cmp_key_then_index(const void* pa, const void* pb) {
  uint32_t a = *(const uint32_t*)pa, b = *(const uint32_t*)pb;
  uint64_t ka = radix_key(g_sort_keys[a]), kb = radix_key(g_sort_keys[b]);
  if (ka < kb) return -1;
  if (kb < ka) return 1;
  return (a < b) ? -1 : (a > b); /* stable: original pair index breaks ties */
}

/* z[a*Nloc+b] = LCA[a*Nprof]/LCB[b*Nprof]; rank[p] = position of pair p in the stable
 * ascending order of z (the reference's double stable_sort_by_key, :370-377);
 * lower/n per bin from upper_bound against the right edges (:384-396). */
void orc_pair_rank(int Nloc, int Nprof, const double* LCA, const double* LCB, int Nbins,
                   const double* edges, uint32_t* rank, uint32_t* lower, uint32_t* nper) {
  long P = (long)Nloc * Nloc;
  double* z = (double*)malloc(sizeof(double) * P);
  uint32_t* perm = (uint32_t*)malloc(sizeof(uint32_t) * P);
  for (int a = 0; a < Nloc; a++)
    for (int b = 0; b < Nloc; b++) z[(long)a * Nloc + b] = gpu_div(LCA[(long)a * Nprof], LCB[(long)b * Nprof]);
  for (long p = 0; p < P; p++) perm[p] = (uint32_t)p;
  g_sort_keys = z;
  qsort(perm, P, sizeof(uint32_t), cmp_key_then_index);
  if (rank)
    for (long r = 0; r < P; r++) rank[perm[r]] = (uint32_t)r;
  if (Nbins > 0) {
    /* upper_bound(sorted z, edge_i) = number of z <= edge_i */
    uint32_t prev = 0;
    for (int i = 0; i < Nbins; i++) {
      long lo = 0, hi = P;
      while (lo < hi) {
        long mid = (lo + hi) / 2;
        if (edges[i] < z[perm[mid]]) hi = mid; else lo = mid + 1;
      }
      if (lower) lower[i] = prev;
      if (nper) nper[i] = (uint32_t)lo - prev;
      prev = (uint32_t)lo;
    }
  }
  free(z);
  free(perm);
}

/* kernel_chi2 / calculate_chi2_CPU (gpu_functions.cu:700-750, cpu_functions.cpp:213-249):
 * chi2 = sum_i ((d_i - mA_i/mB_i)/s_i)^2, mA, mB interpolated along the profile axis
 * (or 1 where the index is -1), stored at rank[a*Nloc+b] (or at a*Nloc+b if rank is NULL). */
void orc_pair_chi2_ratio(int Njp, const int* indA, const int* indB, const double* facA,
                         const double* facB, const double* d, const double* s, int Nloc, int Nprof,
                         const double* LCA, const double* DLCA, const double* LCB,
                         const double* DLCB, const uint32_t* rank, double* chi2) {
  double* mA = (double*)malloc(sizeof(double) * (Njp > 0 ? Njp : 1));
  for (int a = 0; a < Nloc; a++) {
    for (int i = 0; i < Njp; i++)
      mA[i] = (indA[i] == -1) ? 1.0
                              : LCA[(long)a * Nprof + indA[i]] + facA[i] * DLCA[(long)a * (Nprof - 1) + indA[i]];
    for (int b = 0; b < Nloc; b++) {
      double c = 0.0;
      for (int i = 0; i < Njp; i++) {
        double mB = (indB[i] == -1) ? 1.0
                                    : LCB[(long)b * Nprof + indB[i]] + facB[i] * DLCB[(long)b * (Nprof - 1) + indB[i]];
        double tmp = (d[i] - (mA[i] / mB)) / s[i];
        c += tmp * tmp;
      }
      long p = (long)a * Nloc + b;
      chi2[rank ? rank[p] : p] = c;
    }
  }
  free(mA);
}

/* kernel_bin_chi2 (gpu_functions.cu:772-795): mean chi2 and mean exp(-chi2/2) over each
 * bin's slice of the rank-ordered chi2; empty bins give 2000 and exp(-1000). */
void orc_bin_chi2(int Nbins, const uint32_t* lower, const uint32_t* nper, const double* chi2_sorted,
                  double* bchi2, double* bexp) {
  for (int i = 0; i < Nbins; i++) {
    if (nper[i] > 0) {
      double se = 0.0, sc = 0.0;
      for (uint32_t k = 0; k < nper[i]; k++) {
        se += exp(-0.5 * chi2_sorted[lower[i] + k]);
        sc += chi2_sorted[lower[i] + k];
      }
      bexp[i] = se / nper[i];
      bchi2[i] = sc / nper[i];
    } else {
      bexp[i] = exp(-2000.0 / 2.0);
      bchi2[i] = 2000.0;
    }
  }
}

/* Mpd(Nbins,min,max,scale) right edges (mpd.cpp:4-21). */
void orc_mpd_edges(int Nbins, double mn, double mx, int logscale, double* out) {
  if (logscale) {
    double lmin = log10(mn), lmax = log10(mx), dl = (lmax - lmin) / Nbins;
    for (int i = 0; i < Nbins; i++) out[i] = pow(10, lmin + (i + 1) * dl);
  } else {
    double db = (mx - mn) / Nbins;
    for (int i = 0; i < Nbins; i++) out[i] = mn + (i + 1) * db;
  }
}

/* MagnificationMap::getBinnedMpd (magnification_map_gpu.cu:45-87), restated without the
 * sort: the reference sorts the pixels, keeps those in [lower_bound(min), lower_bound(max))
 * -- min <= v < max -- and counts, for every right edge, the kept values <= edge
 * (upper_bound) and differences neighbours.  So a kept value lands in the first bin whose
 * edge is >= v, and is dropped when it lies above the last edge.  counts are divided by
 * npix, an empty bin gets 1/npix. */
void orc_binned_mpd(const double* data, long npix, int Nbins, double mn, double mx, const double* edges,
                    double* counts) {
  long* c = (long*)calloc(Nbins, sizeof(long));
  for (long p = 0; p < npix; p++) {
    const double v = data[p];
    if (!(v >= mn) || !(v < mx)) continue;
    int lo = 0, hi = Nbins; /* first edge >= v */
    while (lo < hi) {
      const int mid = (lo + hi) / 2;
      if (edges[mid] < v) lo = mid + 1;
      else hi = mid;
    }
    if (lo < Nbins) c[lo]++;
  }
  for (int i = 0; i < Nbins; i++)
    counts[i] = c[i] < 1 ? 1.0 / (double)npix : (double)c[i] / (double)npix;
  free(c);
}

/* Mpd::divide_by (mpd.cpp:71-107): ratio[i] = trapezium over b of
 * muB pA(z_i muB) pB(muB), pA linearly interpolated in A's bins (1e-8 outside the open
 * range of A's edges); the interval is located by binary search (the reference scans
 * linearly for the first edge above z muB -- the same interval). */
void orc_mpd_divide(int NA, const double* bA, const double* cA, int NB, const double* bB, const double* cB,
                    int NR, const double* bR, double* cR) {
  double* terms = (double*)malloc(sizeof(double) * (NB > 0 ? NB : 1));
  for (int i = 0; i < NR; i++) {
    const double z = bR[i];
    for (int b = 0; b < NB; b++) {
      const double muB = bB[b];
      const double prod = z * muB;
      double pA;
      if (prod <= bA[0] || prod >= bA[NA - 1]) {
        pA = 1e-8;
      } else {
        int lo = 0, hi = NA; /* first edge > prod */
        while (lo < hi) {
          const int mid = (lo + hi) / 2;
          if (bA[mid] <= prod) lo = mid + 1;
          else hi = mid;
        }
        const int k = lo;
        pA = cA[k - 1] + (cA[k] - cA[k - 1]) * (prod - bA[k - 1]) / (bA[k] - bA[k - 1]);
      }
      terms[b] = muB * pA * cB[b];
    }
    double s = 0.0;
    for (int b = 1; b < NB; b++) s += (terms[b - 1] + terms[b]) * (bB[b] - bB[b - 1]) / 2.0;
    cR[i] = s;
  }
  free(terms);
}

/* Mpd::integrate / normalize (mpd.cpp:48-69). */
void orc_mpd_normalize(int N, const double* bins, double* counts) {
  double s = 0.0;
  for (int i = 1; i < N; i++) s += (counts[i] + counts[i - 1]) * (bins[i] - bins[i - 1]) / 2.0;
  for (int i = 0; i < N; i++) counts[i] /= s;
}

/* ---- differentiable track fit (no reference counterpart; restated from the model) ---- */

/* Thin-disc law of profile.cpp:402-446 on a fixed N x N grid, flat core kept, no outer
 * truncation; P normalised; Px, Py = dP/dx, dP/dy per pixel of offset, PR = dP/drhalf
 * (quotient rule for the normalisation). */
int orc_fit_raster(double rhalf, double pix, int N, double* P, double* Px, double* Py, double* PR) {
  const double sig = 0.4106 * rhalf;
  const double core = 10.0 / (exp(pow(1.0 / 0.4106, 0.75)) - 1.0);
  double S = 0.0, T = 0.0;
  for (int i = 0; i < N; i++)
    for (int j = 0; j < N; j++) {
      const double y = (i - N / 2) * pix + pix / 2.0, x = (j - N / 2) * pix + pix / 2.0;
      const double r = sqrt(x * x + y * y), u = r / sig;
      const double E = exp(pow(u, 0.75));
      double v = 1.0 / (E - 1.0), gx = 0.0, gy = 0.0, gr = 0.0;
      if (v >= core) {
        v = core;
      } else {
        /* dv/du = -(3/4) u^(-1/4) E / (E-1)^2 ; du/dx = x / (r sig) ; du/dR = -u / R */
        const double dvdu = -0.75 * pow(u, -0.25) * E / ((E - 1.0) * (E - 1.0));
        gx = dvdu * x / (r * sig) * pix;
        gy = dvdu * y / (r * sig) * pix;
        gr = -dvdu * u / rhalf;
      }
      P[i * N + j] = v;
      Px[i * N + j] = gx;
      Py[i * N + j] = gy;
      PR[i * N + j] = gr;
      S += v;
      T += gr;
    }
  for (int k = 0; k < N * N; k++) {
    P[k] /= S;
    Px[k] /= S;
    Py[k] /= S;
    PR[k] = PR[k] / S - P[k] * T / S;
  }
  return N;
}

/* Cubic Hermite basis on [0,1]: b[0..3] = h00, h01, h10, h11 and d[0..3] their derivatives. */
static void orc_herm(double s, double* b, double* d) {
  b[0] = 2 * s * s * s - 3 * s * s + 1;
  b[1] = -2 * s * s * s + 3 * s * s;
  b[2] = s * s * s - 2 * s * s + s;
  b[3] = s * s * s - s * s;
  d[0] = 6 * s * s - 6 * s;
  d[1] = -6 * s * s + 6 * s;
  d[2] = 3 * s * s - 4 * s + 1;
  d[3] = 3 * s * s - 2 * s;
}

/* Model value and first derivatives at (x, y, R): tensor-product cubic Hermite in x, y
 * (nodes at pixel centres, unit spacing) and R (nodes radii[k]) of the stack's node values
 * M and derivatives Mx, My, MR, st[((i Nx + j) K + k) 4 + f], without cross-derivative
 * terms.  Returns 0 outside the hull of pixel centres. */
static int orc_fit_eval(const double* st, int Nx, int Ny, int K, const double* radii, double x, double y, double R,
                        double* F, double* Fx, double* Fy, double* FR) {
  if (x < 0.5 || x > Nx - 0.5 || y < 0.5 || y > Ny - 0.5) return 0;
  int j0 = (int)floor(x - 0.5), i0 = (int)floor(y - 0.5);
  if (j0 > Nx - 2) j0 = Nx - 2;
  if (i0 > Ny - 2) i0 = Ny - 2;
  const double sx = x - (j0 + 0.5), sy = y - (i0 + 0.5);
  int k = 0;
  while (k < K - 2 && R >= radii[k + 1]) k++;
  const double h = radii[k + 1] - radii[k];
  double sr = (R - radii[k]) / h;
  int cl = 0;
  if (sr < 0) { sr = 0; cl = 1; }
  if (sr > 1) { sr = 1; cl = 1; }
  double bx[4], dx[4], by[4], dy[4], br[4], dr[4];
  orc_herm(sx, bx, dx);
  orc_herm(sy, by, dy);
  orc_herm(sr, br, dr);
  *F = *Fx = *Fy = *FR = 0.0;
  for (int b = 0; b < 2; b++)     /* y node */
    for (int a = 0; a < 2; a++)   /* x node */
      for (int c = 0; c < 2; c++) { /* radius node */
        const double* q = st + (((long)(i0 + b) * Nx + (j0 + a)) * K + k + c) * 4;
        const double vx = bx[a], tx = bx[2 + a], vy = by[b], ty = by[2 + b];
        const double wr = br[c], ur = br[2 + c] * h;
        const double dwr = cl ? 0 : dr[c] / h, dur = cl ? 0 : dr[2 + c];
        *F += vx * vy * (wr * q[0] + ur * q[3]) + tx * vy * wr * q[1] + vx * ty * wr * q[2];
        *Fx += dx[a] * vy * (wr * q[0] + ur * q[3]) + dx[2 + a] * vy * wr * q[1] + dx[a] * ty * wr * q[2];
        *Fy += vx * dy[b] * (wr * q[0] + ur * q[3]) + tx * dy[b] * wr * q[1] + vx * dy[2 + b] * wr * q[2];
        *FR += vx * vy * (dwr * q[0] + dur * q[3]) + tx * vy * dwr * q[1] + vx * ty * dwr * q[2];
      }
  return 1;
}

void orc_track_fit(const double* st, int Nx, int Ny, int K, const double* radii, int n, const double* theta,
                   const long* off, const double* t, const double* obs, const double* w, double* chi2,
                   double* grad, double* model) {
  for (int i = 0; i < n; i++) {
    const double* th = theta + 6 * i;
    double c2 = 0, g[6] = {0, 0, 0, 0, 0, 0};
    for (long e = off[i]; e < off[i + 1]; e++) {
      const double vt = th[3] * t[e];
      const double x = th[0] + vt * cos(th[2]), y = th[1] + vt * sin(th[2]);
      double M, Mx, My, MR;
      if (!orc_fit_eval(st, Nx, Ny, K, radii, x, y, th[4], &M, &Mx, &My, &MR) || !(M > 0)) {
        if (model) model[e] = NAN;
        continue;
      }
      const double m = -2.5 * log10(M) + th[5];
      if (model) model[e] = m;
      const double r = obs[e] - m;
      c2 += w[e] * r * r;
      const double gm = -2.0 * w[e] * r;
      const double gM = gm * (-2.5 / log(10.0)) / M;
      g[0] += gM * Mx;
      g[1] += gM * My;
      g[2] += gM * (-vt * sin(th[2]) * Mx + vt * cos(th[2]) * My);
      g[3] += gM * (t[e] * cos(th[2]) * Mx + t[e] * sin(th[2]) * My);
      g[4] += gM * MR;
      g[5] += gm;
    }
    chi2[i] = c2;
    if (grad)
      for (int j = 0; j < 6; j++) grad[6 * i + j] = g[j];
  }
}

/* getChi2CPU (chi2/chi2_functions.cuh:150-190) restated in FP64: chi2[y*N + x] =
 * 1/2 sum_{f,t} ((fo - m1[x]/m2[y]) / df)^2 and the likelihood sum of exp(-chi2). */
double orc_flux_ratio(const float* fo, const float* dfo, const float* m1, const float* m2, int N, int F, int T,
                      double* chi2) {
  const long K = (long)F * T;
  double like = 0.0;
  for (int x = 0; x < N; x++)
    for (int y = 0; y < N; y++) {
      double c = 0.0;
      for (long k = 0; k < K; k++) {
        const double tmp = ((double)fo[k] - (double)m1[x * K + k] / (double)m2[y * K + k]) / (double)dfo[k];
        c += tmp * tmp / 2;
      }
      if (chi2) chi2[(long)y * N + x] = c;
      like += exp(-c);
    }
  return like;
}

/* The same in the reference CPU twin's own FP32 arithmetic and order (float chi2 and
 * float likelihood accumulators, chi2_functions.cuh:165-183). */
float orc_flux_ratio_f32(const float* fo, const float* dfo, const float* m1, const float* m2, int N, int F, int T) {
  float like = 0.0f;
  for (int x = 0; x < N; x++)
    for (int y = 0; y < N; y++) {
      float c = 0.0f;
      for (int f = 0; f < F; f++)
        for (int t = 0; t < T; t++) {
          const float tmp = (fo[f * T + t] - m1[x * F * T + f * T + t] / m2[y * F * T + f * T + t]) / dfo[f * T + t];
          c += tmp * tmp / 2;
        }
      like += expf(-c);
    }
  return like;
}

/* trapezium (integration.cpp:3-9). */
double orc_trapezium(int N, const double* f1, const double* f2, const double* x) {
  double s = 0.0;
  for (int i = 1; i < N; i++) s += (f1[i - 1] * f2[i - 1] + f1[i] * f2[i]) * (x[i] - x[i - 1]) / 2.0;
  return s;
}

/* ---- tracks (no reference counterpart except the formula source) ---- */

/* RectGrid::interp2d_bilinear (rectGrid.cpp:349-378, match_point_to_closest_4 :238-270)
 * on a grid with pixel centres at j + 0.5 (xmin = 0, step = 1 pixel): 0 outside the
 * hull of the centres, otherwise the four weights w = {b d, a d, b c, a c} summed in
 * corner order.  At the upper hull edge the out-of-range neighbour has weight zero and
 * is clamped to the last column/row instead of being read past the end. */
double orc_bilinear(const double* map, int Nx, int Ny, double x, double y) {
  if (x < 0.5 || x > Nx - 0.5 || y < 0.5 || y > Ny - 0.5) return 0.0;
  int j0 = (int)floor(x), i0 = (int)floor(y);
  double dx = x - (j0 + 0.5), dy = y - (i0 + 0.5);
  int jl = (dx < 0) ? j0 - 1 : j0, jr = jl + 1;
  int iu = (dy < 0) ? i0 : i0 + 1, il = iu - 1;
  double a = x - (jl + 0.5), b = (jr + 0.5) - x;
  double c = (iu + 0.5) - y, d = y - (il + 0.5);
  if (jr > Nx - 1) jr = Nx - 1;
  if (iu > Ny - 1) iu = Ny - 1;
  double z = 0.0;
  z += (b * d) * map[(long)iu * Nx + jl];
  z += (a * d) * map[(long)iu * Nx + jr];
  z += (b * c) * map[(long)il * Nx + jl];
  z += (a * c) * map[(long)il * Nx + jr];
  return z;
}

/* Straight tracks: position x0 + v t cos(phi), y0 + v t sin(phi) (pixels) at each of the
 * track's epoch times (CSR offsets); output magnitude -2.5 log10(mu) (or mu if mag==0).
 * out[e] for e in [off[k], off[k+1]). */
void orc_sample_tracks(const double* map, int Nx, int Ny, int Ntr, const double* x0, const double* y0,
                       const double* phi, const double* v, const long* off, const double* t, int mag,
                       double* out) {
  for (int k = 0; k < Ntr; k++) {
    double c = cos(phi[k]), s = sin(phi[k]);
    for (long e = off[k]; e < off[k + 1]; e++) {
      double px = x0[k] + v[k] * t[e] * c;
      double py = y0[k] + v[k] * t[e] * s;
      double mu = orc_bilinear(map, Nx, Ny, px, py);
      out[e] = mag ? -2.5 * log10(mu) : mu;
    }
  }
}

/* Offset-minimised chi2 of each simulated magnitude curve against one observed curve
 * on the same epochs: dm = sum w (o - m) / sum w; chi2 = sum w (o - m - dm)^2. */
void orc_chi2_offset(int Ncurves, int T, const double* m, const double* o, const double* w,
                     double* chi2, double* dm) {
  double W = 0.0;
  for (int e = 0; e < T; e++) W += w[e];
  for (int k = 0; k < Ncurves; k++) {
    const double* mk = m + (long)k * T;
    double sr = 0.0;
    for (int e = 0; e < T; e++) sr += w[e] * (o[e] - mk[e]);
    double off = sr / W, c = 0.0;
    for (int e = 0; e < T; e++) {
      double r = o[e] - mk[e] - off;
      c += w[e] * r * r;
    }
    chi2[k] = c;
    if (dm) dm[k] = off;
  }
}

/* Magnitude-difference pair chi2 over shared epochs: chi2_ij = sum_t w_t (d_t - (a_it - b_jt) - c)^2
 * with c = 0 (offset 0) or the minimising offset c = sum w (d - a + b) / sum w (offset 1).
 * Pairs listed by (ia, ib) index arrays, or all NA x NB pairs (row-major) when ia is NULL. */
void orc_pair_chi2_magdiff(int NA, int NB, int T, const float* A, const float* B, const double* w,
                           const double* d, int offset, long npairs, const long* ia, const long* ib,
                           double* chi2) {
  double W = 0.0;
  for (int t = 0; t < T; t++) W += w[t];
  long n = ia ? npairs : (long)NA * NB;
  for (long p = 0; p < n; p++) {
    long i = ia ? ia[p] : p / NB, j = ia ? ib[p] : p % NB;
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
      double r = (d ? d[t] : 0.0) - ((double)a[t] - (double)b[t]) - c;
      s += w[t] * r * r;
    }
    chi2[p] = s;
  }
}

/* Histogram with nbins equal bins on [lo, hi) of v (logscale: of log10 v); values outside
 * are not counted.  near_edge counts values within rel_tol (relative, on v) of an edge. */
void orc_histogram(long n, const double* v, int nbins, double lo, double hi, int logscale,
                   double rel_tol, uint64_t* counts, uint64_t* near_edge) {
  memset(counts, 0, sizeof(uint64_t) * nbins);
  uint64_t ne = 0;
  double width = (hi - lo) / nbins;
  for (long k = 0; k < n; k++) {
    double x = v[k];
    if (logscale) {
      if (!(x > 0)) continue;
      x = log10(x);
    }
    if (!(x >= lo && x < hi)) continue;
    long b = (long)floor((x - lo) / width);
    if (b >= nbins) b = nbins - 1;
    if (b < 0) b = 0;
    counts[b]++;
    if (rel_tol > 0) {
      double el = lo + b * width, eh = lo + (b + 1) * width;
      double vl = logscale ? pow(10, el) : el, vh = logscale ? pow(10, eh) : eh;
      double vv = v[k];
      if (fabs(vv - vl) <= rel_tol * fabs(vv) || fabs(vh - vv) <= rel_tol * fabs(vv)) ne++;
    }
  }
  if (near_edge) *near_edge = ne;
}

/* Indices of the k smallest values (ascending, ties by index). */
static const double* g_topk_vals;
static int cmp_val_index(const void* pa, const void* pb) {
  long a = *(const long*)pa, b = *(const long*)pb;
  double va = g_topk_vals[a], vb = g_topk_vals[b];
  if (va < vb) return -1;
  if (vb < va) return 1;
  return (a < b) ? -1 : (a > b);
}
void orc_topk_smallest(long n, const double* v, long k, long* idx) {
  long* all = (long*)malloc(sizeof(long) * n);
  for (long i = 0; i < n; i++) all[i] = i;
  g_topk_vals = v;
  qsort(all, n, sizeof(long), cmp_val_index);
  for (long i = 0; i < k && i < n; i++) idx[i] = all[i];
  free(all);
}

/* Inverse ray shooting for synthetic gerlumph maps: the FP32 arithmetic of the library's
 * generator (mlc_rayshoot), operation for operation, so that both give the same counts.
 * Rays r in [r0, r1) of the nrx x nry image-plane grid x = (x0 + dx i, y0 + dx j), r = j nrx + i,
 * are deflected by the nl point lenses (xy pairs, FP32) in index order:
 *   u = x1 - lx, v = x2 - ly, q = 1 / fma(u, u, v v), a1 = fma(u, q, a1), a2 = fma(v, q, a2),
 *   y1 = (1 - kappa_c - gamma) x1 - a1,  y2 = (1 - kappa_c + gamma) x2 - a2,
 * and counted into pixel (floor((y2 + w/2) N / w), floor((y1 + w/2) N / w)) when inside.
 * Blocks of rays run together so the compiler can vectorise across them; counts are added
 * atomically, so several threads may run disjoint ray ranges into one array. */
#define ORC_RAY_BLOCK 16
void orc_rayshoot(const float* lenses, int nl, double kappa_c, double gamma, double x0, double y0, double dx,
                  long nrx, long nry, double width, int N, long r0, long r1, int32_t* counts) {
  const float kc = (float)kappa_c, g = (float)gamma, half_w = (float)(width / 2);
  const float scale = (float)N / (2.0f * half_w);
  const float c1 = (1.0f - kc) - g, c2 = (1.0f - kc) + g;
  const long total = nrx * nry;
  if (r1 > total) r1 = total;
  for (long rb = r0; rb < r1; rb += ORC_RAY_BLOCK) {
    float x1[ORC_RAY_BLOCK], x2[ORC_RAY_BLOCK], a1[ORC_RAY_BLOCK], a2[ORC_RAY_BLOCK];
    for (int k = 0; k < ORC_RAY_BLOCK; k++) {
      const long r = rb + k < r1 ? rb + k : r1 - 1;
      x1[k] = (float)(x0 + dx * (double)(r % nrx));
      x2[k] = (float)(y0 + dx * (double)(r / nrx));
      a1[k] = 0.0f;
      a2[k] = 0.0f;
    }
    for (int i = 0; i < nl; i++) {
      const float lx = lenses[2 * i], ly = lenses[2 * i + 1];
      for (int k = 0; k < ORC_RAY_BLOCK; k++) {
        const float u = x1[k] - lx, v = x2[k] - ly;
        const float q = 1.0f / fmaf(u, u, v * v);
        a1[k] = fmaf(u, q, a1[k]);
        a2[k] = fmaf(v, q, a2[k]);
      }
    }
    for (int k = 0; k < ORC_RAY_BLOCK && rb + k < r1; k++) {
      const float y1 = c1 * x1[k] - a1[k];
      const float y2 = c2 * x2[k] - a2[k];
      const int jx = (int)floorf((y1 + half_w) * scale);
      const int iy = (int)floorf((y2 + half_w) * scale);
      if (iy >= 0 && iy < N && jx >= 0 && jx < N) __atomic_fetch_add(counts + (long)iy * N + jx, 1, __ATOMIC_RELAXED);
    }
  }
}
