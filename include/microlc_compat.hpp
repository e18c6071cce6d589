// microlc_compat.hpp -- the reference's C++ interface for the light-curve path, rebuilt
// header-only on the C ABI in microlc_gb300.h.
//
// microLC (gvernard/microSN, simulating_lcurves) drives this path from driver.cpp
// (src/driver.cpp:19-275) through C++ classes and free functions:
//   data_structs.hpp   Chi2Vars, Chi2, Chi2SortBins, SimLC
//   mpd.hpp            Mpd
//   image.hpp          Image (pixel container)
//   magnification_map.hpp  MagnificationMap (gerlumph reader, getBinnedMpd)
//   gpu_functions.hpp  expanding_source, setup_integral_GPU, calculate_chi2_GPU, bin_chi2_GPU
//   cpu_functions.hpp  find_indices, setup_chi2_calculation
//   integration.hpp    trapezium
//   locations.hpp      locations_on_grid, locations_random
//   util.hpp           get_total_gpu_mem, get_free_gpu_mem, get_used_gpu_mem
//   chi2/chi2_functions.cuh  getChi2GPU (multi-filter flux-ratio likelihood)
// This header declares the same names with the same members, argument meaning and
// ownership (the classes allocate their device halves with cudaMalloc in their
// constructors, as data_structs.cu:39-125 does), so such a driver compiles unchanged
// against it and links with -lmicrolc_gb300 -lcudart.  All GPU work runs through one
// library context on the current device and the default stream.
//
// Differences, by design:
//   - a failed library call prints the library's message to stderr (as the reference's
//     cuda_error does) and throws std::runtime_error instead of continuing on bad data;
//   - kernel_chi2's 50-entry __constant__ limit and the fixed 10000^2 grid of
//     kernel_multiplyFFTs do not exist;
//   - the CPU twins (setup_integral_CPU, calculate_chi2_CPU, bin_chi2_CPU), test_chi2,
//     test_setup_integral, getFullMpd, the Kernel / EffectiveMap / profile classes and the
//     PNG / FITS writers are not provided (link the reference's own sources for them; the
//     class layouts here match data_structs.hpp member for member).
//
// Map directory: MagnificationMap(id, Rein) reads MAP_PATH + id + "/mapmeta.dat" and
// "/map.bin", MAP_PATH being a compile-time string as in the reference (default "").
#ifndef MICROLC_COMPAT_HPP
#define MICROLC_COMPAT_HPP

#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "microlc_gb300.h"

#ifndef MAP_PATH
#define MAP_PATH ""
#endif

namespace microlc_compat {

// The library context all calls of this header share: current device, default stream.
inline mlc_ctx* context() {
  static mlc_ctx* ctx = [] {
    int dev = 0;
    cudaGetDevice(&dev);
    mlc_ctx* c = nullptr;
    if (mlc_ctx_create(dev, nullptr, &c) != MLC_OK) {
      std::fprintf(stderr, "microlc: cannot create a library context on device %d (an sm_103 GPU is required)\n",
                   dev);
      throw std::runtime_error("microlc: no usable device");
    }
    return c;
  }();
  return ctx;
}

inline void check(int status, const char* where) {
  if (status == MLC_OK) return;
  const char* msg = mlc_ctx_last_error(context());
  std::fprintf(stderr, "microlc: %s failed (status %d): %s\n", where, status, msg);
  throw std::runtime_error(std::string("microlc: ") + where + ": " + msg);
}

// Library calls that take no context report through their status only.
inline void check_status(int status, const char* where) {
  if (status == MLC_OK) return;
  std::fprintf(stderr, "microlc: %s failed (status %d)\n", where, status);
  throw std::runtime_error(std::string("microlc: ") + where + " failed");
}

inline void check_cuda(cudaError_t e, const char* where) {
  if (e == cudaSuccess) return;
  std::fprintf(stderr, "microlc: %s: %s\n", where, cudaGetErrorString(e));
  throw std::runtime_error(std::string("microlc: ") + where + ": " + cudaGetErrorString(e));
}

template <typename T>
inline T* device_alloc(size_t n, const char* what) {
  void* p = nullptr;
  check_cuda(cudaMalloc(&p, n * sizeof(T) > 0 ? n * sizeof(T) : 1), what);
  return static_cast<T*>(p);
}

// Profile shape names of FactoryProfile (profile.hpp:112-170).
inline int shape_code(const std::string& s) {
  if (s == "uniform") return MLC_SHAPE_UNIFORM;
  if (s == "gaussian") return MLC_SHAPE_GAUSSIAN;
  if (s == "gaussian_hole") return MLC_SHAPE_GAUSSIAN_HOLE;
  if (s == "thermal_hole") return MLC_SHAPE_THERMAL_HOLE;
  if (s == "wavy") return MLC_SHAPE_WAVY;
  if (s == "exponential") return MLC_SHAPE_EXPONENTIAL;
  std::fprintf(stderr, "microlc: unknown profile shape '%s'\n", s.c_str());
  throw std::runtime_error("microlc: unknown profile shape " + s);
}

}  // namespace microlc_compat

// ============================================================================ data_structs.hpp

class Chi2Vars {
 public:
  int Njp;
  int* indA;
  int* indB;
  double* facA;
  double* facB;
  double* new_d;
  double* new_s;
  double const_term;

  Chi2Vars(int Njp) : Njp(Njp) {
    const size_t n = Njp > 0 ? (size_t)Njp : 1;
    indA = (int*)std::malloc(n * sizeof(int));
    indB = (int*)std::malloc(n * sizeof(int));
    facA = (double*)std::malloc(n * sizeof(double));
    facB = (double*)std::malloc(n * sizeof(double));
    new_d = (double*)std::malloc(n * sizeof(double));
    new_s = (double*)std::malloc(n * sizeof(double));
    const_term = 0.0;
  }
  Chi2Vars(const Chi2Vars& o) : Chi2Vars(o.Njp) {
    const size_t n = Njp > 0 ? (size_t)Njp : 0;
    std::memcpy(indA, o.indA, n * sizeof(int));
    std::memcpy(indB, o.indB, n * sizeof(int));
    std::memcpy(facA, o.facA, n * sizeof(double));
    std::memcpy(facB, o.facB, n * sizeof(double));
    std::memcpy(new_d, o.new_d, n * sizeof(double));
    std::memcpy(new_s, o.new_s, n * sizeof(double));
    const_term = o.const_term;
  }
  ~Chi2Vars() {
    std::free(indA);
    std::free(indB);
    std::free(facA);
    std::free(facB);
    std::free(new_d);
    std::free(new_s);
  }
};

class Chi2 {
 public:
  int Nloc;
  double* values;    // Nloc*Nloc on the CPU
  double* d_values;  // Nloc*Nloc on the GPU

  Chi2(int Nloc) : Nloc(Nloc) {
    const size_t n = (size_t)Nloc * Nloc;
    values = (double*)std::malloc(n * sizeof(double));
    d_values = microlc_compat::device_alloc<double>(n, "Chi2: cudaMalloc");
  }
  Chi2(const Chi2& o) : Chi2(o.Nloc) {
    const size_t n = (size_t)Nloc * Nloc;
    std::memcpy(values, o.values, n * sizeof(double));
    microlc_compat::check_cuda(cudaMemcpy(d_values, o.d_values, n * sizeof(double), cudaMemcpyDeviceToDevice),
                               "Chi2: copy");
  }
  ~Chi2() {
    std::free(values);
    cudaFree(d_values);
  }
  void transfer_to_CPU() {
    microlc_compat::check_cuda(
        cudaMemcpy(values, d_values, (size_t)Nloc * Nloc * sizeof(double), cudaMemcpyDeviceToHost),
        "Chi2::transfer_to_CPU");
  }
};

class Chi2SortBins {
 public:
  int Nloc;
  int Nbins;
  unsigned int* sorted_ind;    // Nloc*Nloc on the CPU
  unsigned int* d_sorted_ind;  // Nloc*Nloc on the GPU
  unsigned int* lower_ind;     // Nbins on the CPU
  unsigned int* n_per_bin;     // Nbins on the CPU

  Chi2SortBins(int Nloc, int Nbins) : Nloc(Nloc), Nbins(Nbins) {
    const size_t n = (size_t)Nloc * Nloc;
    sorted_ind = (unsigned int*)std::malloc(n * sizeof(unsigned int));
    d_sorted_ind = microlc_compat::device_alloc<unsigned int>(n, "Chi2SortBins: cudaMalloc");
    lower_ind = (unsigned int*)std::calloc(Nbins > 0 ? Nbins : 1, sizeof(unsigned int));
    n_per_bin = (unsigned int*)std::calloc(Nbins > 0 ? Nbins : 1, sizeof(unsigned int));
  }
  Chi2SortBins(const Chi2SortBins& o) : Chi2SortBins(o.Nloc, o.Nbins) {
    const size_t n = (size_t)Nloc * Nloc;
    std::memcpy(sorted_ind, o.sorted_ind, n * sizeof(unsigned int));
    std::memcpy(lower_ind, o.lower_ind, Nbins * sizeof(unsigned int));
    std::memcpy(n_per_bin, o.n_per_bin, Nbins * sizeof(unsigned int));
    microlc_compat::check_cuda(
        cudaMemcpy(d_sorted_ind, o.d_sorted_ind, n * sizeof(unsigned int), cudaMemcpyDeviceToDevice),
        "Chi2SortBins: copy");
  }
  ~Chi2SortBins() {
    std::free(sorted_ind);
    cudaFree(d_sorted_ind);
    std::free(lower_ind);
    std::free(n_per_bin);
  }
  void transfer_to_CPU() {
    microlc_compat::check_cuda(cudaMemcpy(sorted_ind, d_sorted_ind, (size_t)Nloc * Nloc * sizeof(unsigned int),
                                          cudaMemcpyDeviceToHost),
                               "Chi2SortBins::transfer_to_CPU");
  }
};

class SimLC {
 public:
  int Nloc;
  int Nprof;
  double* LC;     // Nloc*Nprof on the CPU
  double* DLC;    // Nloc*(Nprof-1) on the CPU
  double* d_LC;   // Nloc*Nprof on the GPU
  double* d_DLC;  // Nloc*(Nprof-1) on the GPU

  SimLC(int Nloc, int Nprof) : Nloc(Nloc), Nprof(Nprof) {
    const size_t n = (size_t)Nloc * Nprof, m = (size_t)Nloc * (Nprof > 1 ? Nprof - 1 : 0);
    LC = (double*)std::malloc((n > 0 ? n : 1) * sizeof(double));
    DLC = (double*)std::malloc((m > 0 ? m : 1) * sizeof(double));
    d_LC = microlc_compat::device_alloc<double>(n, "SimLC: cudaMalloc");
    d_DLC = microlc_compat::device_alloc<double>(m, "SimLC: cudaMalloc");
  }
  SimLC(const SimLC& o) : SimLC(o.Nloc, o.Nprof) {
    const size_t n = (size_t)Nloc * Nprof, m = (size_t)Nloc * (Nprof > 1 ? Nprof - 1 : 0);
    std::memcpy(LC, o.LC, n * sizeof(double));
    std::memcpy(DLC, o.DLC, m * sizeof(double));
    microlc_compat::check_cuda(cudaMemcpy(d_LC, o.d_LC, n * sizeof(double), cudaMemcpyDeviceToDevice), "SimLC: copy");
    microlc_compat::check_cuda(cudaMemcpy(d_DLC, o.d_DLC, m * sizeof(double), cudaMemcpyDeviceToDevice),
                               "SimLC: copy");
  }
  ~SimLC() {
    std::free(LC);
    std::free(DLC);
    cudaFree(d_LC);
    cudaFree(d_DLC);
  }
  void transfer_to_CPU() {
    const size_t n = (size_t)Nloc * Nprof, m = (size_t)Nloc * (Nprof > 1 ? Nprof - 1 : 0);
    microlc_compat::check_cuda(cudaMemcpy(LC, d_LC, n * sizeof(double), cudaMemcpyDeviceToHost),
                               "SimLC::transfer_to_CPU");
    microlc_compat::check_cuda(cudaMemcpy(DLC, d_DLC, m * sizeof(double), cudaMemcpyDeviceToHost),
                               "SimLC::transfer_to_CPU");
  }
};

// ============================================================================ mpd.hpp

class Mpd {
 public:
  int Nbins;
  double* bins;    // right bin edges
  double* counts;

  Mpd(int Nbins) : Nbins(Nbins) {
    bins = (double*)std::calloc(Nbins > 0 ? Nbins : 1, sizeof(double));
    counts = (double*)std::calloc(Nbins > 0 ? Nbins : 1, sizeof(double));
  }
  // scale "log": edges 10^(log10 min + (i+1) dlog); anything else: linear (mpd.cpp:4-21).
  Mpd(int Nbins, double min, double max, std::string scale) : Mpd(Nbins) {
    microlc_compat::check_status(mlc_bin_edges(Nbins, min, max, scale == "log" ? 1 : 0, bins),
                                 "Mpd(Nbins,min,max,scale)");
  }
  Mpd(const Mpd& o) : Mpd(o.Nbins) {
    std::memcpy(bins, o.bins, Nbins * sizeof(double));
    std::memcpy(counts, o.counts, Nbins * sizeof(double));
  }
  ~Mpd() {
    std::free(bins);
    std::free(counts);
  }
  void reset(int n) {
    std::free(bins);
    std::free(counts);
    Nbins = n;
    bins = (double*)std::calloc(n > 0 ? n : 1, sizeof(double));
    counts = (double*)std::calloc(n > 0 ? n : 1, sizeof(double));
  }
  // Two columns "%11.6e %11.6e" per bin (mpd.cpp:31-46).
  void writeMpd(const std::string filename) {
    FILE* fh = std::fopen(filename.c_str(), "w");
    if (!fh) throw std::runtime_error("microlc: cannot write " + filename);
    for (int i = 0; i < Nbins; i++) std::fprintf(fh, "%11.6e %11.6e\n", bins[i], counts[i]);
    std::fclose(fh);
  }
  // Trapezium rule over the edges (mpd.cpp:48-54).
  double integrate() {
    double s = 0.0;
    for (int i = 1; i < Nbins; i++) s += (counts[i] + counts[i - 1]) * (bins[i] - bins[i - 1]) / 2.0;
    return s;
  }
  double sum() {
    double s = 0.0;
    for (int i = 0; i < Nbins; i++) s += counts[i];
    return s;
  }
  void normalize() {
    const double norm = integrate();
    for (int i = 0; i < Nbins; i++) counts[i] /= norm;
  }
  // ratio = this / B on ratio's edges (mpd.cpp:71-107), computed on the GPU.
  void divide_by(Mpd* B, Mpd* ratio) {
    microlc_compat::check(mlc_mpd_divide(microlc_compat::context(), Nbins, bins, counts, B->Nbins, B->bins, B->counts,
                                         ratio->Nbins, ratio->bins, ratio->counts),
                          "Mpd::divide_by");
  }
};

// ============================================================================ image.hpp / magnification_map.hpp

class Image {
 public:
  std::string imageType;
  int Nx = 0;
  int Ny = 0;
  double* data = nullptr;
  ~Image() { std::free(data); }
};

struct point {
  double x;
  double y;
};

class MagnificationMap : public Image {
 public:
  std::string id;
  double k = 0, g = 0, s = 0;
  double width = 0, height = 0;  // in Rein
  double avgmu = 0, avgN = 0, mu_th = 0;
  double pixSizePhys = 0;  // in 10^14 cm
  bool convolved = false;
  const std::string path;

  MagnificationMap() : path(MAP_PATH) {}
  // gerlumph map MAP_PATH + id (magnification_map.cpp:7-40).
  MagnificationMap(std::string id, double Rein) : path(MAP_PATH) {
    this->id = id;
    imageType = "map";
    const std::string dir = path + id;
    int n = 0;
    double w = 0, meta[6] = {0, 0, 0, 0, 0, 0};
    microlc_compat::check_status(mlc_read_gerlumph(dir.c_str(), &n, &w, meta, nullptr, 0),
                                 ("MagnificationMap: read " + dir).c_str());
    Nx = Ny = n;
    data = (double*)std::calloc((size_t)n * n, sizeof(double));
    microlc_compat::check_status(mlc_read_gerlumph(dir.c_str(), &n, &w, meta, data, (long)n * n),
                                 ("MagnificationMap: read " + dir).c_str());
    avgmu = meta[0];
    avgN = meta[1];
    width = height = meta[2];
    k = meta[3];
    g = meta[4];
    s = meta[5];
    pixSizePhys = Rein * width / Nx;
    mu_th = 1.0 / (std::pow(1.0 - k, 2) - std::pow(g, 2));
  }
  MagnificationMap(const MagnificationMap& o) : Image(), path(o.path) {
    imageType = o.imageType;
    id = o.id;
    k = o.k;
    g = o.g;
    s = o.s;
    Nx = o.Nx;
    Ny = o.Ny;
    width = o.width;
    height = o.height;
    avgmu = o.avgmu;
    avgN = o.avgN;
    mu_th = o.mu_th;
    pixSizePhys = o.pixSizePhys;
    convolved = o.convolved;
    data = (double*)std::calloc((size_t)Nx * Ny, sizeof(double));
    if (o.data) std::memcpy(data, o.data, (size_t)Nx * Ny * sizeof(double));
  }
  ~MagnificationMap() {
    if (dev_) mlc_map_destroy(dev_);
  }

  static double getPixSizePhys(std::string id, double Rein) {
    int n = 0;
    double w = 0;
    const std::string dir = std::string(MAP_PATH) + id;
    microlc_compat::check_status(mlc_read_gerlumph(dir.c_str(), &n, &w, nullptr, nullptr, 0), "getPixSizePhys");
    return Rein * w / n;
  }

  // Log-binned MPD of the pixels (magnification_map_gpu.cu:45-87), on the GPU without a sort.
  Mpd getBinnedMpd(int Nbins, double min = 0.02, double max = 200) {
    Mpd m(Nbins);
    microlc_compat::check(mlc_map_binned_mpd(microlc_compat::context(), device_map(), Nbins, min, max, m.bins,
                                             m.counts),
                          "getBinnedMpd");
    return m;
  }

  // The library's copy of the current pixels (uploaded again on every call, as the
  // reference uploads the map in every expanding_source / getBinnedMpd).
  mlc_map* device_map() {
    mlc_ctx* ctx = microlc_compat::context();
    if (dev_ && (dev_nx_ != Nx || dev_ny_ != Ny)) {
      mlc_map_destroy(dev_);
      dev_ = nullptr;
    }
    if (!dev_) {
      microlc_compat::check(mlc_map_create(ctx, data, 0, MLC_F64, Nx, Ny, MLC_F64, &dev_), "map upload");
      dev_nx_ = Nx;
      dev_ny_ = Ny;
    } else {
      void* p = nullptr;
      microlc_compat::check(mlc_map_data(dev_, &p), "map upload");
      microlc_compat::check_cuda(cudaMemcpy(p, data, (size_t)Nx * Ny * sizeof(double), cudaMemcpyHostToDevice),
                                 "map upload");
      microlc_compat::check(mlc_map_refresh(ctx, dev_), "map upload");
    }
    return dev_;
  }

 private:
  mlc_map* dev_ = nullptr;
  int dev_nx_ = 0, dev_ny_ = 0;
};

// ============================================================================ gpu_functions.hpp

// Convolve the map with the profile of every size (sizes in Einstein radii, sizes[0] the
// point source) and sample it at the Nloc pixel locations: LC->d_LC, LC->d_DLC
// (gpu_functions.cu:82-225).
inline void expanding_source(MagnificationMap* map, std::vector<double> sizes, std::string shape, int Nloc,
                             int* sample_loc_x, int* sample_loc_y, SimLC* LC) {
  mlc_ctx* ctx = microlc_compat::context();
  mlc_profile base{};
  base.shape = microlc_compat::shape_code(shape);
  base.ref_compat = 1;
  base.pix = map->pixSizePhys;
  int* loc = microlc_compat::device_alloc<int>(2 * (size_t)Nloc, "expanding_source: cudaMalloc");
  cudaError_t e = cudaMemcpy(loc, sample_loc_x, Nloc * sizeof(int), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(loc + Nloc, sample_loc_y, Nloc * sizeof(int), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(loc);
    microlc_compat::check_cuda(e, "expanding_source: locations");
  }
  const int st = mlc_expanding_source(ctx, map->device_map(), sizes.data(), (int)sizes.size(), &base, map->width,
                                      Nloc, loc, loc + Nloc, MLC_CONV_FUSED, LC->d_LC, LC->d_DLC);
  cudaFree(loc);
  microlc_compat::check(st, "expanding_source");
}

// Stable rank of every pair's z = LCA/LCB of the point source and the per-bin ranges of
// mpd_ratio's edges (gpu_functions.cu:351-401).
inline void setup_integral_GPU(SimLC* LCA, SimLC* LCB, Mpd* mpd_ratio, Chi2SortBins* sorted) {
  microlc_compat::check(mlc_pair_setup(microlc_compat::context(), LCA->Nloc, LCA->Nprof, LCA->d_LC, LCB->d_LC,
                                       mpd_ratio->Nbins, mpd_ratio->bins, sorted->d_sorted_ind, sorted->lower_ind,
                                       sorted->n_per_bin),
                        "setup_integral_GPU");
}

// Ratio chi2 of every pair, stored at its rank (gpu_functions.cu:428-456).
inline void calculate_chi2_GPU(Chi2Vars* chi2_vars, double* chi2_d_values, Chi2SortBins* sorted, SimLC* LCA,
                               SimLC* LCB) {
  microlc_compat::check(mlc_pair_chi2_ratio(microlc_compat::context(), chi2_vars->Njp, chi2_vars->indA,
                                            chi2_vars->indB, chi2_vars->facA, chi2_vars->facB, chi2_vars->new_d,
                                            chi2_vars->new_s, LCA->Nloc, LCA->Nprof, LCA->d_LC, LCA->d_DLC,
                                            LCB->d_LC, LCB->d_DLC, sorted->d_sorted_ind, chi2_d_values),
                        "calculate_chi2_GPU");
}

// Mean chi2 and mean exp(-chi2/2) per bin into host arrays (gpu_functions.cu:483-503).
inline void bin_chi2_GPU(double* binned_chi2, double* binned_exp, Chi2SortBins* sort_struct, double* chi2_d_values) {
  microlc_compat::check(mlc_bin_chi2(microlc_compat::context(), sort_struct->Nbins, sort_struct->lower_ind,
                                     sort_struct->n_per_bin, chi2_d_values, binned_chi2, binned_exp),
                        "bin_chi2_GPU");
}

// ============================================================================ cpu_functions.hpp / integration.hpp

// Profile-size index of every data time (cpu_functions.cpp:28-45).
inline void find_indices(double* t, double* x, int Nd, int Nprof, int* ind) {
  microlc_compat::check_status(mlc_find_indices(t, x, Nd, Nprof, ind), "find_indices");
}

// Indices, interpolation factors and constant term of the chi2 for masses M = {MA, MB}
// and velocity V[0] (cpu_functions.cpp:80-144).
inline Chi2Vars setup_chi2_calculation(std::vector<double> M, std::vector<double> V, double Dfac, int Nd, double* d,
                                       double* t, double* s, int Nprof, double* x) {
  std::vector<int> iA(Nd > 0 ? Nd : 1), iB(Nd > 0 ? Nd : 1);
  std::vector<double> fA(Nd > 0 ? Nd : 1), fB(Nd > 0 ? Nd : 1), dd(Nd > 0 ? Nd : 1), ss(Nd > 0 ? Nd : 1);
  int Njp = 0;
  double ct = 0.0;
  microlc_compat::check_status(mlc_setup_chi2(M.at(0), M.at(1), V.at(0), Dfac, Nd, d, t, s, Nprof, x, 1, &Njp,
                                              iA.data(), iB.data(), fA.data(), fB.data(), dd.data(), ss.data(), &ct),
                               "setup_chi2_calculation");
  Chi2Vars cv(Njp);
  for (int i = 0; i < Njp; i++) {
    cv.indA[i] = iA[i];
    cv.indB[i] = iB[i];
    cv.facA[i] = fA[i];
    cv.facB[i] = fB[i];
    cv.new_d[i] = dd[i];
    cv.new_s[i] = ss[i];
  }
  cv.const_term = ct;
  return cv;
}

inline double trapezium(int N, double* f1, double* f2, double* x) { return mlc_trapezium(N, f1, f2, x); }

// ============================================================================ locations.hpp / util.hpp

// Nside x Nside grid of pixel locations inside the Noff margin (locations.cpp:6-16).
inline void locations_on_grid(int Nside, int Nmap, int Noff, int* x, int* y) {
  microlc_compat::check_status(mlc_locations_grid(Nside, Nmap, Noff, x, y), "locations_on_grid");
}
// Nloc seeded random pixel locations inside the Noff margin (locations.cpp:18-25).
inline void locations_random(int Nloc, int Nmap, int Noff, int seed, int* x, int* y) {
  microlc_compat::check_status(mlc_locations_random(Nloc, Nmap, Noff, seed, x, y), "locations_random");
}

// Device memory in MiB (util.cu:125-164).
inline std::size_t get_free_gpu_mem() {
  std::size_t f = 0, t = 0;
  cudaMemGetInfo(&f, &t);
  return f / (1024 * 1024);
}
inline std::size_t get_total_gpu_mem() {
  std::size_t f = 0, t = 0;
  cudaMemGetInfo(&f, &t);
  return t / (1024 * 1024);
}
inline std::size_t get_used_gpu_mem() {
  std::size_t f = 0, t = 0;
  cudaMemGetInfo(&f, &t);
  return (t - f) / (1024 * 1024);
}

// ============================================================================ chi2/chi2_functions.cuh

// Adds sum over location pairs of exp(-chi2) to *likelihood, chi2 the multi-filter
// flux-ratio chi2 (chi2_functions.cuh:93-146) with mu2 taken at the second location (the
// reference's kernel reads it at the first).  f_obs, df_obs must be host-readable and mu1,
// mu2 device-readable (the reference's driver passes managed memory, which is both).
// Prints the reason and returns false on failure, like the reference.
inline bool getChi2GPU(float* f_obs, float* df_obs, float* mu1, float* mu2, int N, int F, int T, float* likelihood) {
  double like = 0.0;
  mlc_ctx* ctx = microlc_compat::context();
  const int st = mlc_flux_ratio_chi2(ctx, f_obs, df_obs, mu1, mu2, N, F, T, nullptr, &like);
  if (st != MLC_OK) {
    std::fprintf(stderr, "microlc: getChi2GPU failed (status %d): %s\n", st, mlc_ctx_last_error(ctx));
    return false;
  }
  *likelihood += (float)like;
  return true;
}

#endif  // MICROLC_COMPAT_HPP
