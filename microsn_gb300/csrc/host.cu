// Host-side stages of the path in C++: chi2 set-up (time -> profile-size mapping),
// sample locations, log/linear bin edges, the trapezium integral, and the gerlumph map
// reader.  These are serial FP64 host computations in the reference too.
#include <sys/mman.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <mutex>
#include <random>
#include <string>
#include <vector>

#include "mlc_internal.h"

namespace {

// find_indices (simulating_lcurves/src/cpu_functions.cpp:28-45).  Entries the reference
// leaves unset (a time equal to or below the size range) are set to -1 here.
void find_indices(const double* t, const double* x, int Nd, int Nprof, int* ind) {
  for (int i = 0; i < Nd; i++) ind[i] = -1;
  int i = 0, j = 0;
  while (i < Nd && j < Nprof - 1) {
    const double comp = t[i];
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

}  // namespace

extern "C" {

// setup_chi2_calculation (cpu_functions.cpp:80-144) with M = {MA, MB}, V = {V0}.
int mlc_setup_chi2(double MA, double MB, double V0, double Dfac, int Nd, const double* d_host,
                   const double* t_host, const double* s_host, int Nprof, const double* x_host, int ref_compat,
                   int* Njp_out, int* indA, int* indB, double* facA, double* facB, double* d_out, double* s_out,
                   double* const_term) {
  if (Nd < 0 || Nprof < 2 || !Njp_out || !const_term || (Nd > 0 && (!d_host || !t_host || !s_host)) || !x_host)
    return MLC_ERR_ARG;
  if (!(MA > 0) || !(MB > 0) || !(Dfac > 0)) return MLC_ERR_ARG;
  const double Rfac = 23.92865 * Dfac;
  const double t2xA = V0 * 8.64 / (Rfac * std::sqrt(MA));
  const double t2xB = V0 * 8.64 / (Rfac * std::sqrt(MB));
  std::vector<double> tA(Nd), tB(Nd);
  for (int i = 0; i < Nd; i++) {
    tA[i] = t2xA * t_host[i];
    tB[i] = t2xB * t_host[i];
  }
  std::vector<int> iA(Nd), iB(Nd);
  find_indices(tA.data(), x_host, Nd, Nprof, iA.data());
  find_indices(tB.data(), x_host, Nd, Nprof, iB.data());
  int Njp = Nd;
  for (int i = 0; i < Nd; i++)
    if (iA[i] == -1 && iB[i] == -1) {
      Njp = i;
      break;
    }
  for (int i = 0; i < Njp; i++) {
    indA[i] = iA[i];
    indB[i] = iB[i];
    d_out[i] = d_host[i];
    s_out[i] = s_host[i];
    facA[i] = (iA[i] != -1) ? (tA[i] - x_host[iA[i]]) / (x_host[iA[i] + 1] - x_host[iA[i]]) : 0;
    facB[i] = (iB[i] != -1) ? (tB[i] - x_host[iB[i]]) / (x_host[iB[i] + 1] - x_host[iB[i]]) : 0;
  }
  // Constant term for the epochs dropped after Njp.  The reference loops over
  // i = Nd-Njp .. Nd-1 (cpu_functions.cpp:138); ref_compat keeps that range.
  double c = 0.0;
  if (Njp != Nd) {
    const int i0 = ref_compat ? Nd - Njp : Njp;
    for (int i = i0; i < Nd; i++) c += std::pow((d_host[i] - 1) / s_host[i], 2);
  }
  *const_term = c;
  *Njp_out = Njp;
  return MLC_OK;
}

// locations_on_grid (locations.cpp:6-15): integer spacing dd = (Nmap - 2 Noff) / Nside.
int mlc_locations_grid(int Nside, int Nmap, int Noff, int* x_host, int* y_host) {
  if (Nside < 1 || !x_host || !y_host) return MLC_ERR_ARG;
  const double dd = (Nmap - 2 * Noff) / Nside;  // integer division, as the reference
  for (int i = 0; i < Nside; i++)
    for (int j = 0; j < Nside; j++) {
      x_host[i * Nside + j] = Noff + ((int)std::floor(dd / 2.0 + j * dd));
      y_host[i * Nside + j] = Noff + ((int)std::floor(dd / 2.0 + i * dd));
    }
  return MLC_OK;
}

// locations_random (locations.cpp:17-25): std::mt19937(seed), uniform integers in
// [0, Nmap - 2 Noff], x then y.
int mlc_locations_random(int Nloc, int Nmap, int Noff, int seed, int* x_host, int* y_host) {
  if (Nloc < 0 || !x_host || !y_host) return MLC_ERR_ARG;
  const int Neff = Nmap - 2 * Noff;
  if (Neff < 0) return MLC_ERR_ARG;
  std::mt19937 gen(seed);
  std::uniform_int_distribution<unsigned> distrib(0, Neff);
  for (int i = 0; i < Nloc; i++) {
    x_host[i] = Noff + distrib(gen);
    y_host[i] = Noff + distrib(gen);
  }
  return MLC_OK;
}

// Right bin edges of Mpd(Nbins, min, max, scale) (mpd.cpp:4-21).
int mlc_bin_edges(int Nbins, double mn, double mx, int logscale, double* out_host) {
  if (Nbins < 1 || !out_host || (logscale && !(mn > 0 && mx > 0))) return MLC_ERR_ARG;
  if (logscale) {
    const double lmin = std::log10(mn), lmax = std::log10(mx), dl = (lmax - lmin) / Nbins;
    for (int i = 0; i < Nbins; i++) out_host[i] = std::pow(10, lmin + (i + 1) * dl);
  } else {
    const double db = (mx - mn) / Nbins;
    for (int i = 0; i < Nbins; i++) out_host[i] = mn + (i + 1) * db;
  }
  return MLC_OK;
}

// trapezium (integration.cpp:3-9).
double mlc_trapezium(int N, const double* f1, const double* f2, const double* x) {
  double s = 0.0;
  for (int i = 1; i < N; i++) s += (f1[i - 1] * f2[i - 1] + f1[i] * f2[i]) * (x[i] - x[i - 1]) / 2.0;
  return s;
}

// gerlumph map reader (MagnificationMap::MagnificationMap, magnification_map.cpp:7-40):
// dir/mapmeta.dat holds "avgmu avgN / Nx / width / k g s"; dir/map.bin holds Nx*Nx int32
// ray counts; pixels = counts * |avgmu/avgN| / |1/((1-k)^2 - g^2)|.  Call with out_host
// NULL to read the size only.
int mlc_find_indices(const double* t_host, const double* x_host, int Nd, int Nprof, int* ind_host) {
  if (Nd < 0 || Nprof < 1 || (Nd > 0 && (!t_host || !x_host || !ind_host))) return MLC_ERR_ARG;
  find_indices(t_host, x_host, Nd, Nprof, ind_host);
  return MLC_OK;
}

int mlc_read_gerlumph(const char* dir, int* Nx, double* width, double* meta6, double* out_host, long cap) {
  if (!dir || !Nx || !width) return MLC_ERR_ARG;
  std::string d(dir);
  std::ifstream f(d + "/mapmeta.dat");
  if (!f) return MLC_ERR_ARG;
  double avgmu, avgN, w, k, g, s;
  int n;
  f >> avgmu >> avgN >> n >> w >> k >> g >> s;
  if (!f || n < 1) return MLC_ERR_ARG;
  *Nx = n;
  *width = w;
  if (meta6) {
    meta6[0] = avgmu; meta6[1] = avgN; meta6[2] = w; meta6[3] = k; meta6[4] = g; meta6[5] = s;
  }
  if (!out_host) return MLC_OK;
  const long N = (long)n * n;
  if (cap < N) return MLC_ERR_LIMIT;
  FILE* fp = std::fopen((d + "/map.bin").c_str(), "rb");
  if (!fp) return MLC_ERR_ARG;
  std::vector<int> counts(N);
  const size_t got = std::fread(counts.data(), sizeof(int), N, fp);
  std::fclose(fp);
  if ((long)got != N) return MLC_ERR_ARG;
  const double factor = std::fabs(avgmu / avgN);
  const double muth = std::fabs(1.0 / (std::pow(1.0 - k, 2) - std::pow(g, 2)));
  for (long i = 0; i < N; i++) out_host[i] = (counts[i] * factor / muth);
  return MLC_OK;
}

// Page-locked host buffers on 2 MB pages: anonymous memory advised for transparent huge
// pages, then registered with the CUDA driver.  Copies between such buffers and the GPU keep
// their rate when the host's memory is fragmented; buffers pinned on small pages (as
// cudaHostAlloc gives them after the host has run other large jobs) were measured slower in
// the overlapped light-curve step (42.5 against 45 to 51 ms per 10000^2 step on a box whose
// memory had been churned, 42.5 ms either way on a fresh one).
static std::mutex host_mu;
static std::map<void*, size_t> host_bufs;

int mlc_host_alloc(size_t bytes, void** ptr) {
  if (!ptr || bytes == 0) return MLC_ERR_ARG;
  *ptr = nullptr;
  const size_t huge = (size_t)2 << 20;
  const size_t size = (bytes + huge - 1) / huge * huge;
  void* p = mmap(nullptr, size, PROT_READ | PROT_WRITE, MAP_PRIVATE | MAP_ANONYMOUS, -1, 0);
  if (p == MAP_FAILED) return MLC_ERR_OOM;
  (void)madvise(p, size, MADV_HUGEPAGE);  // advice only: small pages where none are free
  if (cudaHostRegister(p, size, cudaHostRegisterPortable) != cudaSuccess) {
    (void)cudaGetLastError();
    munmap(p, size);
    return MLC_ERR_CUDA;
  }
  std::lock_guard<std::mutex> lk(host_mu);
  host_bufs[p] = size;
  *ptr = p;
  return MLC_OK;
}

int mlc_host_free(void* ptr) {
  if (!ptr) return MLC_OK;
  size_t size = 0;
  {
    std::lock_guard<std::mutex> lk(host_mu);
    auto it = host_bufs.find(ptr);
    if (it == host_bufs.end()) return MLC_ERR_ARG;
    size = it->second;
    host_bufs.erase(it);
  }
  const cudaError_t e = cudaHostUnregister(ptr);
  munmap(ptr, size);
  return e == cudaSuccess ? MLC_OK : MLC_ERR_CUDA;
}

}  // extern "C"
