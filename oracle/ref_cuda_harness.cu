// Test infrastructure only: C entry points over the reference's own CUDA path (microLC
// simulating_lcurves/src/gpu_functions.cu and data_structs.cu), compiled unchanged from a
// staged copy of the reference's sources by oracle/refcuda.mk into
// baseline/_ref/libmlcref_cuda.so.  The tests pin the library's FP64 path to it and
// bench.py reports its times as the reference's CUDA baseline on the same GPU.  Nothing in
// the product links this file.
//
// Only inputs the reference's kernels index in bounds are passed on:
//  * expanding_source launches kernel_multiplyFFTs on a fixed grid of 10 x 5001 blocks of
//    1000 threads (gpu_functions.cu:88-89), which covers the Nx (Ny/2 + 1) spectrum of a
//    10000 x 10000 map exactly and no other size: any other map is refused here;
//  * sample locations must lie inside the map (kernel_sample reads map[y Nx + x]);
//  * the pair kernels index pairs as int a Nloc + b (:654, :742): Nloc <= 46340;
//  * data tables live in 50-entry __constant__ arrays (:25-30) and bin tables in 5120-entry
//    ones (:32-33): Njp <= 50, Nbins <= 5120;
//  * the interpolation indices of kernel_chi2 must stay inside the light curves:
//    -1 <= ind and ind + 1 < Nprof.
#include <fcntl.h>
#include <unistd.h>

#include <chrono>
#include <cstdio>
#include <cstring>
#include <iostream>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "data_structs.hpp"
#include "gpu_functions.hpp"
#include "magnification_map.hpp"
#include "mpd.hpp"

namespace {

// The reference prints progress and memory banners on stdout; the caller's stdout (a
// bench's JSON line) stays clean while a call runs.
struct QuietStdout {
  int saved = -1;
  explicit QuietStdout(bool on) {
    if (!on) return;
    std::cout.flush();
    fflush(stdout);
    saved = dup(1);
    int dn = open("/dev/null", O_WRONLY);
    if (dn >= 0) {
      dup2(dn, 1);
      close(dn);
    }
  }
  ~QuietStdout() {
    if (saved < 0) return;
    std::cout.flush();
    fflush(stdout);
    dup2(saved, 1);
    close(saved);
  }
};

double now_ms() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

}  // namespace

extern "C" {

// expanding_source (gpu_functions.cu:82-225) on a host map: LC (Nloc x Nprof) and DLC
// (Nloc x (Nprof - 1)) copied back to the host.  ms receives the wall time of the call
// (it synchronises after every stage).  Returns 0, or 2 for an input the reference cannot
// index in bounds, 3 for a CUDA error.
int refc_expanding_source(const double* data, int Nx, int Ny, double width, double pix_size_phys,
                          const double* sizes, int Nprof, const char* shape, int Nloc, const int* lx,
                          const int* ly, double* LC, double* DLC, double* ms, int quiet) {
  if (Nx != 10000 || Ny != 10000 || Nprof < 1 || Nloc < 1 || sizes[0] != 0.0) return 2;
  for (int i = 0; i < Nloc; i++)
    if (lx[i] < 0 || lx[i] >= Nx || ly[i] < 0 || ly[i] >= Ny) return 2;
  MagnificationMap map;
  map.Nx = Nx;
  map.Ny = Ny;
  map.width = width;
  map.height = width;
  map.pixSizePhys = pix_size_phys;
  map.data = (double*)malloc(sizeof(double) * (size_t)Nx * Ny);  // freed by ~Image
  if (!map.data) return 3;
  memcpy(map.data, data, sizeof(double) * (size_t)Nx * Ny);
  std::vector<int> x(lx, lx + Nloc), y(ly, ly + Nloc);
  std::vector<double> sz(sizes, sizes + Nprof);
  SimLC lc(Nloc, Nprof);
  double t0 = now_ms();
  {
    QuietStdout q(quiet != 0);
    expanding_source(&map, sz, std::string(shape), Nloc, x.data(), y.data(), &lc);
  }
  if (cudaDeviceSynchronize() != cudaSuccess) return 3;
  *ms = now_ms() - t0;
  if (cudaMemcpy(LC, lc.d_LC, sizeof(double) * (size_t)Nloc * Nprof, cudaMemcpyDeviceToHost) != cudaSuccess) return 3;
  if (Nprof > 1 &&
      cudaMemcpy(DLC, lc.d_DLC, sizeof(double) * (size_t)Nloc * (Nprof - 1), cudaMemcpyDeviceToHost) != cudaSuccess)
    return 3;
  return cudaGetLastError() == cudaSuccess ? 0 : 3;
}

// setup_integral_GPU (:351-401), calculate_chi2_GPU (:428-456) and bin_chi2_GPU (:483-503)
// on host light curves of images A and B and a ratio MPD's bin edges: the rank table
// (Nloc^2), lower_ind / n_per_bin (Nbins) and the binned chi2 and exp(-chi2/2) (Nbins).
// ms[0..2] receive the wall time of each call.  Returns 0, 2 (inputs out of the
// reference's bounds) or 3 (CUDA error).
int refc_pair_path(int Nloc, int Nprof, const double* LCA, const double* DLCA, const double* LCB,
                   const double* DLCB, int Njp, const int* indA, const int* indB, const double* facA,
                   const double* facB, const double* d, const double* s, int Nbins, const double* edges,
                   unsigned* sorted_ind, unsigned* lower_ind, unsigned* n_per_bin, double* binned_chi2,
                   double* binned_exp, double* ms, int quiet) {
  if (Nloc < 1 || Nloc > 46340 || Nprof < 2 || Njp < 1 || Njp > 50 || Nbins < 1 || Nbins > 5120) return 2;
  for (int i = 0; i < Njp; i++) {
    if (indA[i] < -1 || indA[i] + 1 >= Nprof || indB[i] < -1 || indB[i] + 1 >= Nprof) return 2;
  }
  const size_t nl = (size_t)Nloc * Nprof, nd = (size_t)Nloc * (Nprof - 1);
  SimLC A(Nloc, Nprof), B(Nloc, Nprof);
  if (cudaMemcpy(A.d_LC, LCA, sizeof(double) * nl, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(A.d_DLC, DLCA, sizeof(double) * nd, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(B.d_LC, LCB, sizeof(double) * nl, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(B.d_DLC, DLCB, sizeof(double) * nd, cudaMemcpyHostToDevice) != cudaSuccess)
    return 3;
  Mpd ratio(Nbins);
  memcpy(ratio.bins, edges, sizeof(double) * Nbins);
  Chi2Vars vars(Njp);
  memcpy(vars.indA, indA, sizeof(int) * Njp);
  memcpy(vars.indB, indB, sizeof(int) * Njp);
  memcpy(vars.facA, facA, sizeof(double) * Njp);
  memcpy(vars.facB, facB, sizeof(double) * Njp);
  memcpy(vars.new_d, d, sizeof(double) * Njp);
  memcpy(vars.new_s, s, sizeof(double) * Njp);
  Chi2SortBins sb(Nloc, Nbins);
  Chi2 chi2(Nloc);
  {
    QuietStdout q(quiet != 0);
    double t0 = now_ms();
    setup_integral_GPU(&A, &B, &ratio, &sb);
    cudaDeviceSynchronize();
    double t1 = now_ms();
    calculate_chi2_GPU(&vars, chi2.d_values, &sb, &A, &B);
    cudaDeviceSynchronize();
    double t2 = now_ms();
    bin_chi2_GPU(binned_chi2, binned_exp, &sb, chi2.d_values);
    cudaDeviceSynchronize();
    double t3 = now_ms();
    ms[0] = t1 - t0;
    ms[1] = t2 - t1;
    ms[2] = t3 - t2;
  }
  if (cudaGetLastError() != cudaSuccess) return 3;
  if (sorted_ind &&
      cudaMemcpy(sorted_ind, sb.d_sorted_ind, sizeof(unsigned) * (size_t)Nloc * Nloc, cudaMemcpyDeviceToHost) !=
          cudaSuccess)
    return 3;
  memcpy(lower_ind, sb.lower_ind, sizeof(unsigned) * Nbins);
  memcpy(n_per_bin, sb.n_per_bin, sizeof(unsigned) * Nbins);
  return 0;
}

}  // extern "C"
