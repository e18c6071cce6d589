// Shared definitions of the pairwise magnitude-difference chi2 (pairdiff.cu, pairtc.cu).
#pragma once

#include <stdint.h>

#include <vector>

#include "mlc_internal.h"

namespace mlc {

// Largest quantised magnitude: three balanced base-256 digits in [-127, 127].
constexpr int PD_QMAX = 127 * (65536 + 256 + 1);  // 8355711
constexpr int PD_TILE_M = 128;                    // A curves per tile (TMEM lanes)
constexpr int PD_TILE_N = 48;                     // B curves per tile
constexpr int PD_EMIN = -60, PD_EMAX = 20;        // range of the per-curve step exponents

// Operands of the tensor-core form, built by pairdiff_prepare.
// Each curve r is quantised with its own power-of-two step 2^e_r (the smallest that keeps
// |q| <= PD_QMAX), so flat curves keep full relative precision.
struct PdOperands {
  int NA = 0, NB = 0, NApad = 0, NBpad = 0, T = 0, Kp = 0;
  double delta = 1.0;          // largest step 2^e over all curves (reported)
  uint16_t* a = nullptr;       // NApad rows of [s0 | s1 | s2], Kp bf16 each (device)
  uint16_t* b = nullptr;       // NBpad rows of [t0 | t1 | t2]
  long long* alpha = nullptr;  // sum q^2 per A row (device)
  long long* beta = nullptr;   // sum q^2 per B row
  float2* alpha_ff = nullptr;  // |P_i|^2 = alpha 2^(2 e) in natural units, float-float (hi, lo)
  float2* beta_ff = nullptr;
  int* ea = nullptr;           // step exponent per A row
  int* eb = nullptr;           // step exponent per B row
  const double* cenA = nullptr;  // NA x T centred, weighted curves (FP64), for the exact list
  const double* cenB = nullptr;  // NB x T
};

// The operands of one image's curves ("side"), built once and used by every pair it takes
// part in: centred, weighted curves, their sliced integers, norms and steps, in one device
// allocation of `bytes` at `mem` (owned by the side).  Rows are padded to PD_SIDE_PAD, a
// multiple of both tile heights, so a side serves as A or as B.
constexpr int PD_SIDE_PAD = 384;
struct PdSide {
  int N = 0, Npad = 0, T = 0, Kp = 0, offset = 0, has_d = 0;
  double delta = 1.0;     // largest step 2^e of its curves
  std::vector<double> w;  // the weights it was built with (host)
  double* cen = nullptr;
  double* rowmax = nullptr;
  uint16_t* ops = nullptr;
  long long* norm2 = nullptr;
  float2* norm2_ff = nullptr;
  int* exps = nullptr;
  void* mem = nullptr;
  size_t bytes = 0;
};

struct PdResult {
  double delta = 0, thr = 0;
  long long nrefined = 0, ncand = 0;
  int passes = 0;
  long long below = 0, above = 0;  // chi2 below lo / at or above hi of the histogram
};

void pairdiff_run(mlc_ctx* ctx, int method, const float* A, const float* B, int NA, int NB, int T,
                  const double* w_host, const double* d_host, int offset, int nbins, double lo, double hi,
                  uint64_t* hist_host, int k, double* tv, int64_t* ti, int64_t* tj, float* out, PdResult& res);

// A side from FP32 curves (N x T, row-major), or straight from the convolved maps of an
// expanding source (maps: nep x nbands planes of Ny x Nx FP32; curve r of track r is its
// magnitudes at the nep shared epochs t, band-minor): sampled, converted to magnitudes,
// centred and weighted in one pass, no light curve stored.  d_host (nullable): the observed
// difference curve, for a side used as B only.  The side's memory is allocated here.
void pd_side_from_curves(mlc_ctx* ctx, const float* X, int N, int T, const double* w_host, const double* d_host,
                         int offset, PdSide& side);
void pd_side_from_expanding(mlc_ctx* ctx, const float* maps, int Nx, int Ny, int nep, int nbands, int ntracks,
                            const float* x0, const float* y0, const float* phi, const float* v, const float* t,
                            const double* w_host, const double* d_host, int offset, PdSide& side);
void pd_side_free(PdSide& side);
void pairdiff_sides(mlc_ctx* ctx, const PdSide& A, const PdSide& B, int nbins, double lo, double hi,
                    uint64_t* hist_host, int k, double* tv, int64_t* ti, int64_t* tj, float* out, PdResult& res);

double pairdiff_prepare(mlc_ctx* ctx, const float* A, const float* B, int NA, int NB, int T, const double* w_host,
                        const double* d_host, int offset, PdOperands& ops);
void pairdiff_plain(mlc_ctx* ctx, const float* A, const float* B, int NA, int NB, int T, const double* w_dev,
                    const double* d_dev, double W, int offset, long npairs, const long* ia, const long* ib,
                    double* chi2);

}  // namespace mlc
