// Shared definitions of the pairwise magnitude-difference chi2 (pairdiff.cu, pairtc.cu).
#pragma once

#include <stdint.h>

#include "mlc_internal.h"

namespace mlc {

// Largest quantised magnitude: three balanced base-256 digits in [-127, 127].
constexpr int PD_QMAX = 127 * (65536 + 256 + 1);  // 8355711
constexpr int PD_TILE_M = 128;                    // A curves per tile (TMEM lanes)
constexpr int PD_TILE_N = 64;                     // B curves per tile

// Operands of the tensor-core form, built by pairdiff_prepare.
struct PdOperands {
  int NA = 0, NB = 0, NApad = 0, NBpad = 0, T = 0, Kp = 0;
  double delta = 1.0;          // quantisation step: value = delta * q
  uint16_t* a = nullptr;       // NApad rows of [s0 | s1 | s2], Kp bf16 each (device)
  uint16_t* b = nullptr;       // NBpad rows of [t0 | t1 | t2]
  long long* alpha = nullptr;  // sum q^2 per A row (device)
  long long* beta = nullptr;   // sum q^2 per B row
};

struct PdResult {
  double delta = 0, thr = 0;
  long long nrefined = 0, ncand = 0;
  int passes = 0;
};

void pairdiff_run(mlc_ctx* ctx, int method, const float* A, const float* B, int NA, int NB, int T,
                  const double* w_host, const double* d_host, int offset, int nbins, double lo, double hi,
                  uint64_t* hist_host, int k, double* tv, int64_t* ti, int64_t* tj, float* out, PdResult& res);

double pairdiff_prepare(mlc_ctx* ctx, const float* A, const float* B, int NA, int NB, int T, const double* w_host,
                        const double* d_host, int offset, PdOperands& ops);
void pairdiff_plain(mlc_ctx* ctx, const float* A, const float* B, int NA, int NB, int T, const double* w_dev,
                    const double* d_dev, double W, int offset, long npairs, const long* ia, const long* ib,
                    double* chi2);

}  // namespace mlc
