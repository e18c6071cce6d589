// Test infrastructure only: a C entry layer over the reference's own CPU code
// (microLC, simulating_lcurves/src/*.cpp), compiled from the reference's sources
// where they lie into oracle/_ref/libmlcref.so by oracle/Makefile.  Nothing in the
// product links this file; tests use it to pin the oracle restatement.
//
// The reference defines the members of Chi2Vars / SimLC / Chi2SortBins in a CUDA
// file (src/data_structs.cu:8-125, with cudaMalloc for the device halves).  The CPU
// twins only touch the host halves, so host-only definitions are given here.

#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "cpu_functions.hpp"
#include "data_structs.hpp"
#include "integration.hpp"
#include "locations.hpp"
#include "magnification_map.hpp"
#include "mpd.hpp"
#include "profile.hpp"

Chi2Vars::Chi2Vars(int n) : Njp(n) {
  indA = (int*)calloc(n > 0 ? n : 1, sizeof(int));
  indB = (int*)calloc(n > 0 ? n : 1, sizeof(int));
  facA = (double*)calloc(n > 0 ? n : 1, sizeof(double));
  facB = (double*)calloc(n > 0 ? n : 1, sizeof(double));
  new_d = (double*)calloc(n > 0 ? n : 1, sizeof(double));
  new_s = (double*)calloc(n > 0 ? n : 1, sizeof(double));
  const_term = 0.0;
}
Chi2Vars::Chi2Vars(const Chi2Vars& o) : Chi2Vars(o.Njp) {
  size_t n = o.Njp > 0 ? o.Njp : 0;
  memcpy(indA, o.indA, n * sizeof(int));
  memcpy(indB, o.indB, n * sizeof(int));
  memcpy(facA, o.facA, n * sizeof(double));
  memcpy(facB, o.facB, n * sizeof(double));
  memcpy(new_d, o.new_d, n * sizeof(double));
  memcpy(new_s, o.new_s, n * sizeof(double));
  const_term = o.const_term;
}
Chi2Vars::~Chi2Vars() {
  free(indA); free(indB); free(facA); free(facB); free(new_d); free(new_s);
}
SimLC::SimLC(int nl, int np) : Nloc(nl), Nprof(np) {
  LC = (double*)calloc((size_t)nl * np, sizeof(double));
  DLC = (double*)calloc((size_t)nl * (np > 1 ? np - 1 : 1), sizeof(double));
  d_LC = nullptr;
  d_DLC = nullptr;
}
SimLC::~SimLC() { free(LC); free(DLC); }
Chi2SortBins::Chi2SortBins(int nl, int nb) : Nloc(nl), Nbins(nb) {
  sorted_ind = (unsigned*)calloc((size_t)nl * nl, sizeof(unsigned));
  lower_ind = (unsigned*)calloc(nb, sizeof(unsigned));
  n_per_bin = (unsigned*)calloc(nb, sizeof(unsigned));
  d_sorted_ind = nullptr;
}
Chi2SortBins::~Chi2SortBins() { free(sorted_ind); free(lower_ind); free(n_per_bin); }

static std::map<std::string, std::string> profile_pars(const char* shape, double rhalf, double pix) {
  // Same string map as the reference's expanding_source builds (gpu_functions.cu:105-110, :184).
  std::map<std::string, std::string> p;
  p["shape"] = shape;
  p["rhalf"] = std::to_string(rhalf);
  p["pixSizePhys"] = std::to_string(pix);
  p["incl"] = "0";
  p["orient"] = "0";
  return p;
}

extern "C" {

int ref_setup_chi2(double M0, double M1, double V0, double Dfac, int Nd, const double* d,
                   const double* t, const double* s, int Nprof, const double* x, int* Njp,
                   int* indA, int* indB, double* facA, double* facB, double* new_d,
                   double* new_s, double* const_term) {
  std::vector<double> M{M0, M1}, V{V0};
  // find_indices reads t[Nd] after the last match (cpu_functions.cpp:36,40); give it a slot.
  std::vector<double> dd(d, d + Nd), tt(t, t + Nd), ss(s, s + Nd), xx(x, x + Nprof);
  tt.push_back(0.0);
  dd.push_back(0.0);
  ss.push_back(1.0);
  Chi2Vars v = setup_chi2_calculation(M, V, Dfac, Nd, dd.data(), tt.data(), ss.data(), Nprof, xx.data());
  *Njp = v.Njp;
  for (int i = 0; i < v.Njp; i++) {
    indA[i] = v.indA[i];
    indB[i] = v.indB[i];
    facA[i] = v.facA[i];
    facB[i] = v.facB[i];
    new_d[i] = v.new_d[i];
    new_s[i] = v.new_s[i];
  }
  *const_term = v.const_term;
  return 0;
}

int ref_setup_integral_cpu(int Nloc, int Nprof, const double* LCA, const double* LCB, unsigned* sorted_ind) {
  SimLC A(Nloc, Nprof), B(Nloc, Nprof);
  memcpy(A.LC, LCA, sizeof(double) * Nloc * Nprof);
  memcpy(B.LC, LCB, sizeof(double) * Nloc * Nprof);
  Mpd dummy(1);
  Chi2SortBins sb(Nloc, 1);
  setup_integral_CPU(&A, &B, &dummy, &sb);
  memcpy(sorted_ind, sb.sorted_ind, sizeof(unsigned) * (size_t)Nloc * Nloc);
  return 0;
}

int ref_calculate_chi2_cpu(int Njp, const int* indA, const int* indB, const double* facA,
                           const double* facB, const double* new_d, const double* new_s, int Nloc,
                           int Nprof, const double* LCA, const double* DLCA, const double* LCB,
                           const double* DLCB, const unsigned* sorted_ind, double* chi2) {
  Chi2Vars v(Njp);
  for (int i = 0; i < Njp; i++) {
    v.indA[i] = indA[i]; v.indB[i] = indB[i];
    v.facA[i] = facA[i]; v.facB[i] = facB[i];
    v.new_d[i] = new_d[i]; v.new_s[i] = new_s[i];
  }
  SimLC A(Nloc, Nprof), B(Nloc, Nprof);
  memcpy(A.LC, LCA, sizeof(double) * Nloc * Nprof);
  memcpy(B.LC, LCB, sizeof(double) * Nloc * Nprof);
  memcpy(A.DLC, DLCA, sizeof(double) * Nloc * (Nprof - 1));
  memcpy(B.DLC, DLCB, sizeof(double) * Nloc * (Nprof - 1));
  Chi2SortBins sb(Nloc, 1);
  memcpy(sb.sorted_ind, sorted_ind, sizeof(unsigned) * (size_t)Nloc * Nloc);
  calculate_chi2_CPU(&v, chi2, &sb, &A, &B);
  return 0;
}

int ref_bin_chi2_cpu(int Nloc, int Nbins, const unsigned* lower_ind, const unsigned* n_per_bin,
                     const double* chi2, double* binned_chi2, double* binned_exp) {
  Chi2SortBins sb(Nloc, Nbins);
  memcpy(sb.lower_ind, lower_ind, sizeof(unsigned) * Nbins);
  memcpy(sb.n_per_bin, n_per_bin, sizeof(unsigned) * Nbins);
  bin_chi2_CPU(binned_chi2, binned_exp, &sb, const_cast<double*>(chi2));
  return 0;
}

// Profile raster exactly as expanding_source requests it (string round trip included).
int ref_profile(const char* shape, double rhalf, double pix, int* Nx, int* Ny, double* out, long cap) {
  BaseProfile* p = FactoryProfile::getInstance()->createProfileFromHalfRadius(profile_pars(shape, rhalf, pix));
  if (!p) return 1;
  *Nx = p->Nx;
  *Ny = p->Ny;
  long n = (long)p->Nx * p->Ny;
  if (out && cap >= n) memcpy(out, p->data, sizeof(double) * n);
  delete p;
  return (out && cap < n) ? 2 : 0;
}

// Kernel::setKernel quadrant wrap of that profile into an Nx x Ny array.
int ref_kernel(const char* shape, double rhalf, double pix, int Nx, int Ny, double* out) {
  BaseProfile* p = FactoryProfile::getInstance()->createProfileFromHalfRadius(profile_pars(shape, rhalf, pix));
  if (!p) return 1;
  Kernel k(Nx, Ny);
  k.setKernel(p);
  memcpy(out, k.data, sizeof(double) * (size_t)Nx * Ny);
  delete p;
  return 0;
}

int ref_locations_grid(int Nside, int Nmap, int Noff, int* x, int* y) {
  locations_on_grid(Nside, Nmap, Noff, x, y);
  return 0;
}

int ref_locations_random(int Nloc, int Nmap, int Noff, int seed, int* x, int* y) {
  locations_random(Nloc, Nmap, Noff, seed, x, y);
  return 0;
}

int ref_mpd_edges(int Nbins, double mn, double mx, int logscale, double* out) {
  Mpd m(Nbins, mn, mx, logscale ? "log" : "linear");
  memcpy(out, m.bins, sizeof(double) * Nbins);
  return 0;
}

double ref_trapezium(int N, const double* f1, const double* f2, const double* x) {
  return trapezium(N, const_cast<double*>(f1), const_cast<double*>(f2), const_cast<double*>(x));
}

// Reads a gerlumph-format map (mapmeta.dat + map.bin) from dir/ (MAP_PATH is empty here).
int ref_read_map(const char* dir, double Rein, int* Nx, double* width, double* pix, double* out, long cap) {
  MagnificationMap m(std::string(dir), Rein);
  *Nx = m.Nx;
  *width = m.width;
  *pix = m.pixSizePhys;
  long n = (long)m.Nx * m.Ny;
  if (out && cap >= n) memcpy(out, m.data, sizeof(double) * n);
  return (out && cap < n) ? 2 : 0;
}

// MagnificationMap::getBinnedMpd (magnification_map_gpu.cu:45-87) on given pixels, built
// for thrust's sequential host backend.
int ref_binned_mpd(const double* data, int Nx, int Ny, int Nbins, double mn, double mx, double* bins,
                   double* counts) {
  MagnificationMap m;
  m.Nx = Nx;
  m.Ny = Ny;
  m.data = (double*)malloc(sizeof(double) * (size_t)Nx * Ny);  // freed by ~Image
  memcpy(m.data, data, sizeof(double) * (size_t)Nx * Ny);
  Mpd r = m.getBinnedMpd(Nbins, mn, mx);
  memcpy(bins, r.bins, sizeof(double) * Nbins);
  memcpy(counts, r.counts, sizeof(double) * Nbins);
  return 0;
}

// Mpd::normalize then Mpd::divide_by (mpd.cpp:64-107): A.divide_by(B, ratio).
int ref_mpd_divide(int NA, const double* binsA, const double* countsA, int NB, const double* binsB,
                   const double* countsB, int NR, const double* binsR, double* countsR) {
  Mpd A(NA), B(NB), R(NR);
  memcpy(A.bins, binsA, sizeof(double) * NA);
  memcpy(A.counts, countsA, sizeof(double) * NA);
  memcpy(B.bins, binsB, sizeof(double) * NB);
  memcpy(B.counts, countsB, sizeof(double) * NB);
  memcpy(R.bins, binsR, sizeof(double) * NR);
  A.divide_by(&B, &R);
  memcpy(countsR, R.counts, sizeof(double) * NR);
  return 0;
}

int ref_mpd_normalize(int N, const double* bins, double* counts) {
  Mpd A(N);
  memcpy(A.bins, bins, sizeof(double) * N);
  memcpy(A.counts, counts, sizeof(double) * N);
  A.normalize();
  memcpy(counts, A.counts, sizeof(double) * N);
  return 0;
}

}  // extern "C"
