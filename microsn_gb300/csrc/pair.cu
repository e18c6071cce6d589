// Pair stage in the reference's flux-ratio form (simulating_lcurves/src/gpu_functions.cu:
// setup_integral_GPU :351-401, calculate_chi2_GPU :428-456, bin_chi2_GPU :483-503 and
// kernels kernel_z :643, kernel_chi2 :700, kernel_bin_chi2 :772).
//
// GB300 form: no "offset-squares" launch loop and no __constant__ tables.  The
// interpolated curves mA (Nloc x Njp) and mB are built once in FP64; pair kernels read
// them through L1/L2; the z ranking uses the hand-written radix sort; bin means are a
// parallel segmented reduction; and a fused variant computes each pair's z bin directly
// and accumulates chi2 and exp(-chi2/2) per bin without any Nloc^2 array.
#include <algorithm>
#include <cmath>
#include <vector>

#include "mlc_internal.h"

namespace mlc {

void radix_sort_u64_u32(mlc_ctx* ctx, long n, uint64_t* keys, uint32_t* vals);

// The key of the reference's z sort (thrust::stable_sort_by_key on doubles, a radix sort):
// the order of the bit patterns with the sign folded in, -0.0 taken as +0.0 (the radix sort
// keeps the two in pair-index order), and NaN placed by its sign bit -- the GPU's 0/0
// (0xfff8...) and a negative NaN operand before -inf, a positive NaN operand after +inf.
__device__ __forceinline__ uint64_t key_of(double d) {
  uint64_t u = __double_as_longlong(d);
  if (u == 0x8000000000000000ull) u = 0;
  return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
}

// The double a key stands for (-0.0 comes back as +0.0, equal under comparison).
__device__ __forceinline__ double value_of(uint64_t k) {
  return __longlong_as_double((k & 0x8000000000000000ull) ? (k & 0x7fffffffffffffffull) : ~k);
}

// z keys and pair indices for the stable rank sort.
__global__ void k_pair_z(const double* __restrict__ LCA, const double* __restrict__ LCB, int Nloc, int Nprof,
                         uint64_t* __restrict__ keys, uint32_t* __restrict__ idx) {
  const long P = (long)Nloc * Nloc;
  for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < P; p += (long)gridDim.x * blockDim.x) {
    const int a = (int)(p / Nloc), b = (int)(p % Nloc);
    const double z = __ldg(LCA + (long)a * Nprof) / __ldg(LCB + (long)b * Nprof);
    keys[p] = key_of(z);
    idx[p] = (uint32_t)p;
  }
}

// rank[perm[r]] = r
__global__ void k_invert_perm(const uint32_t* __restrict__ perm, long P, uint32_t* __restrict__ rank) {
  for (long r = blockIdx.x * (long)blockDim.x + threadIdx.x; r < P; r += (long)gridDim.x * blockDim.x)
    rank[perm[r]] = (uint32_t)r;
}

// upper_bound of each edge in the sorted z: the reference's binary search
// (thrust::upper_bound, gpu_functions.cu:388) step for step -- the same midpoints and the
// same FP64 comparison edge < z, so that NaN z (never greater than an edge) land where they
// land there: those before -inf count in the first bin, those after +inf in the bins the
// search's path gives them.
__global__ void k_upper_bound(const uint64_t* __restrict__ sorted, long P, const double* __restrict__ edges,
                              int nb, uint32_t* __restrict__ upper) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nb) return;
  const double e = edges[i];
  long lo = 0, hi = P;
  while (lo < hi) {
    const long mid = (lo + hi) >> 1;
    if (e < value_of(sorted[mid])) hi = mid;
    else lo = mid + 1;
  }
  upper[i] = (uint32_t)lo;
}

// mA[i*Nloc + a] = LC[a*Nprof + ind_i] + fac_i * DLC[a*(Nprof-1) + ind_i], or 1 (ind_i = -1);
// with invert, its correctly rounded reciprocal (the B side: one division per (epoch,
// location) instead of one per pair)
__global__ void k_interp(const double* __restrict__ LC, const double* __restrict__ DLC, int Nloc, int Nprof,
                         int Njp, const int* __restrict__ ind, const double* __restrict__ fac, int invert,
                         double* __restrict__ m) {
  const long n = (long)Nloc * Njp;
  for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
    const int i = (int)(q / Nloc), a = (int)(q % Nloc);
    const int k = ind[i];
    const double v = (k == -1) ? 1.0 : LC[(long)a * Nprof + k] + fac[i] * DLC[(long)a * (Nprof - 1) + k];
    m[q] = invert ? 1.0 / v : v;
  }
}

// Point-source values for the fused binning's float pre-search: zA[a] = (float)LCA[a*Nprof],
// zB[b] = (float)(1 / LCB[b*Nprof]).
__global__ void k_zfloat(const double* __restrict__ LCA, const double* __restrict__ LCB, int Nloc, int Nprof,
                         float* __restrict__ zA, float* __restrict__ zB) {
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < Nloc; q += gridDim.x * blockDim.x) {
    zA[q] = (float)LCA[(long)q * Nprof];
    zB[q] = (float)(1.0 / LCB[(long)q * Nprof]);
  }
}

struct Chi2Consts {
  const double* d;
  const double* s;
};

// One pair per thread: chi2 = sum_i ((d_i - mA_i/mB_i)/s_i)^2 in FP64, the divisions as
// products with the correctly rounded reciprocals iB_i = 1/mB_i and is_i = 1/s_i (each term
// within a few ulp of the divided form; GB300's FP64 divide is a long instruction sequence).
__global__ void __launch_bounds__(256) k_pair_chi2_ratio(const double* __restrict__ mA, const double* __restrict__ iB,
                                                         int Nloc, int Njp, const double* __restrict__ d,
                                                         const double* __restrict__ is, const uint32_t* __restrict__ rank,
                                                         double* __restrict__ chi2) {
  const int b = blockIdx.x * 32 + (threadIdx.x & 31);
  const int a = blockIdx.y * 8 + (threadIdx.x >> 5);
  if (a >= Nloc || b >= Nloc) return;
  double c = 0.0;
  for (int i = 0; i < Njp; i++) {
    const double tmp = (__ldg(d + i) - __ldg(mA + (long)i * Nloc + a) * __ldg(iB + (long)i * Nloc + b)) * __ldg(is + i);
    c += tmp * tmp;
  }
  const long p = (long)a * Nloc + b;
  chi2[rank ? rank[p] : p] = c;
}

// Bin means of the rank-ordered chi2 (bin_chi2_GPU): every bin's slice is cut into pieces
// of at most BIN_PIECE values, one CTA per piece sums chi2 and exp(-chi2/2) over it, and a
// second kernel adds each bin's pieces in order -- a fixed summation order (the result does
// not depend on timing), and a bin of millions of pairs is spread over many CTAs (one CTA
// per bin left most SMs idle behind the largest bins).
constexpr uint32_t BIN_PIECE = 1u << 15;
struct BinPiece {
  uint32_t first, count;
};

__global__ void __launch_bounds__(256) k_bin_piece_sums(const double* __restrict__ chi2,
                                                        const BinPiece* __restrict__ pieces,
                                                        double* __restrict__ psum, double* __restrict__ pexp) {
  const BinPiece pc = pieces[blockIdx.x];
  double sc = 0.0, se = 0.0;
  for (uint32_t k = threadIdx.x; k < pc.count; k += blockDim.x) {
    const double c = chi2[(long)pc.first + k];
    sc += c;
    se += exp(-0.5 * c);
  }
  __shared__ double r1[8], r2[8];
  for (int o = 16; o > 0; o >>= 1) {
    sc += __shfl_xor_sync(0xffffffffu, sc, o);
    se += __shfl_xor_sync(0xffffffffu, se, o);
  }
  if ((threadIdx.x & 31) == 0) {
    r1[threadIdx.x >> 5] = sc;
    r2[threadIdx.x >> 5] = se;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
      a += r1[w];
      b += r2[w];
    }
    psum[blockIdx.x] = a;
    pexp[blockIdx.x] = b;
  }
}

// Per bin: the sum of its pieces [pfirst[bin], pfirst[bin + 1]) over its count; an empty bin
// gets the reference's values (chi2 2000, exp(-1000)).
__global__ void k_bin_combine(const uint32_t* __restrict__ pfirst, const uint32_t* __restrict__ nper,
                              const double* __restrict__ psum, const double* __restrict__ pexp, int nb,
                              double* __restrict__ bchi2, double* __restrict__ bexp) {
  const int bin = blockIdx.x * blockDim.x + threadIdx.x;
  if (bin >= nb) return;
  const uint32_t n = nper[bin];
  if (n == 0) {
    bexp[bin] = exp(-2000.0 / 2.0);
    bchi2[bin] = 2000.0;
    return;
  }
  double a = 0.0, b = 0.0;
  for (uint32_t q = pfirst[bin]; q < pfirst[bin + 1]; q++) {
    a += psum[q];
    b += pexp[q];
  }
  bexp[bin] = b / n;
  bchi2[bin] = a / n;
}

// Fused rank-free pair binning.  Bin of z = LCA_a / LCB_b: smallest i with z <= edge_i,
// z above the last edge dropped.  The search runs on float copies (z32 = zA_a * zB_b within
// 1.8e-7 of z, float edges within 6e-8 of the edges): when z32 is more than 2^-20 z32
// away from both neighbouring float edges the float order is the FP64 order; otherwise
// (and for zero, non-finite or extreme z32) the exact FP64 quotient is searched in the
// FP64 edges.  chi2 as k_pair_chi2_ratio.  Sums in FP64 shared-memory accumulators, one
// flush per CTA.  Each CTA covers 16 A curves x 256 B curves.
constexpr int FUSED_A = 16;
__global__ void __launch_bounds__(256) k_pair_bin_fused(const double* __restrict__ mA, const double* __restrict__ iB,
                                                        const float* __restrict__ zA, const float* __restrict__ zB,
                                                        const double* __restrict__ LCA, const double* __restrict__ LCB,
                                                        int Nloc, int Nprof, int Njp, const double* __restrict__ d,
                                                        const double* __restrict__ is, int nb,
                                                        const double* __restrict__ edges, double* __restrict__ gsum,
                                                        double* __restrict__ gexp, unsigned long long* __restrict__ gcnt) {
  extern __shared__ double sm[];
  double* e_s = sm;
  double* sum_s = sm + nb;
  double* exp_s = sum_s + nb;
  float* ef_s = reinterpret_cast<float*>(exp_s + nb);
  unsigned int* cnt_s = reinterpret_cast<unsigned int*>(ef_s + nb);
  for (int i = threadIdx.x; i < nb; i += blockDim.x) {
    e_s[i] = edges[i];
    ef_s[i] = (float)edges[i];
    sum_s[i] = 0.0;
    exp_s[i] = 0.0;
    cnt_s[i] = 0u;
  }
  __syncthreads();
  const int b = blockIdx.x * 256 + threadIdx.x;
  const int a0 = blockIdx.y * FUSED_A;
  if (b < Nloc) {
    const float zb = __ldg(zB + b);
    for (int a = a0; a < a0 + FUSED_A && a < Nloc; a++) {
      const float z32 = __ldg(zA + a) * zb;
      int lo = 0, hi = nb;  // first float edge >= z32
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (ef_s[mid] < z32) lo = mid + 1;
        else hi = mid;
      }
      bool exact = !(z32 > 0x1p-100f && z32 < 0x1p100f);
      if (!exact) {
        const float tol = z32 * 0x1p-20f;
        exact = (lo < nb && ef_s[lo] - z32 <= tol) || (lo > 0 && z32 - ef_s[lo - 1] <= tol);
      }
      if (exact) {
        double z = __ldg(LCA + (long)a * Nprof) / __ldg(LCB + (long)b * Nprof);
        // NaN: the rank order puts a negative one (the GPU's 0/0) before every z, in the
        // first bin, and a positive one (from a NaN light-curve value) after +inf, counted
        // here in no bin
        if (z != z) {
          if (!signbit(z)) continue;
          z = -INFINITY;
        }
        lo = 0;
        hi = nb;
        while (lo < hi) {
          const int mid = (lo + hi) >> 1;
          if (e_s[mid] < z) lo = mid + 1;
          else hi = mid;
        }
      }
      if (lo >= nb) continue;
      double c = 0.0;
      for (int i = 0; i < Njp; i++) {
        const double tmp =
            (__ldg(d + i) - __ldg(mA + (long)i * Nloc + a) * __ldg(iB + (long)i * Nloc + b)) * __ldg(is + i);
        c += tmp * tmp;
      }
      atomicAdd(&sum_s[lo], c);
      atomicAdd(&exp_s[lo], exp(-0.5 * c));
      atomicAdd(&cnt_s[lo], 1u);
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nb; i += blockDim.x) {
    if (cnt_s[i]) {
      atomicAdd(&gsum[i], sum_s[i]);
      atomicAdd(&gexp[i], exp_s[i]);
      atomicAdd(&gcnt[i], (unsigned long long)cnt_s[i]);
    }
  }
}

// ---------------------------------------------------------------- host entry helpers

static int grid_for(mlc_ctx* ctx, long n) {
  return (int)std::max<long>(1, std::min<long>((n + 255) / 256, (long)ctx->sm_count * 16));
}

void pair_setup(mlc_ctx* ctx, int Nloc, int Nprof, const double* LCA, const double* LCB, int Nbins,
                const double* edges_host, uint32_t* rank, uint32_t* lower_host, uint32_t* nper_host) {
  const long P = (long)Nloc * Nloc;
  MLC_REQUIRE(P <= 0xFFFFFFFFl, MLC_ERR_LIMIT, "Nloc^2 above 2^32-1");
  uint64_t* keys = (uint64_t*)ws_get(ctx, WS_PAIR_ACC, sizeof(uint64_t) * P + sizeof(uint32_t) * P + 4096);
  uint32_t* idx = reinterpret_cast<uint32_t*>(keys + P);
  {
    MLC_KSCOPE(ctx, "pair_z");
    k_pair_z<<<grid_for(ctx, P), 256, 0, ctx->stream>>>(LCA, LCB, Nloc, Nprof, keys, idx);
  }
  MLC_CHECK_LAUNCH();
  radix_sort_u64_u32(ctx, P, keys, idx);
  if (rank) {
    {
      MLC_KSCOPE(ctx, "pair_rank");
      k_invert_perm<<<grid_for(ctx, P), 256, 0, ctx->stream>>>(idx, P, rank);
    }
    MLC_CHECK_LAUNCH();
  }
  if (Nbins > 0) {
    double* dedge = (double*)ws_get(ctx, WS_SMALL, sizeof(double) * Nbins + sizeof(uint32_t) * Nbins);
    uint32_t* dup = reinterpret_cast<uint32_t*>(dedge + Nbins);
    MLC_CUDA(cudaMemcpyAsync(dedge, edges_host, sizeof(double) * Nbins, cudaMemcpyHostToDevice, ctx->stream));
    {
      MLC_KSCOPE(ctx, "pair_upper_bound");
      k_upper_bound<<<ceil_div(Nbins, 256), 256, 0, ctx->stream>>>(keys, P, dedge, Nbins, dup);
    }
    MLC_CHECK_LAUNCH();
    std::vector<uint32_t> up(Nbins);
    MLC_CUDA(cudaMemcpyAsync(up.data(), dup, sizeof(uint32_t) * Nbins, cudaMemcpyDeviceToHost, ctx->stream));
    MLC_CUDA(cudaStreamSynchronize(ctx->stream));
    // lower_ind[0] = 0, lower_ind[i] = upper[i-1]; n_per_bin = adjacent difference of upper
    for (int i = 0; i < Nbins; i++) {
      lower_host[i] = i ? up[i - 1] : 0u;
      nper_host[i] = i ? up[i] - up[i - 1] : up[0];
    }
  }
}

struct Interp {
  double* mA;
  double* iB;  // 1 / mB
  double* d;
  double* is;  // 1 / s
};

static Interp build_interp(mlc_ctx* ctx, int Njp, const int* indA, const int* indB, const double* facA,
                           const double* facB, const double* d, const double* s, int Nloc, int Nprof,
                           const double* LCA, const double* DLCA, const double* LCB, const double* DLCB) {
  const long n = (long)Nloc * Njp;
  // small tables: ind A/B (int), fac A/B, d, s
  size_t small = sizeof(double) * 4 * Njp + sizeof(int) * 2 * Njp + 64;
  char* sm = (char*)ws_get(ctx, WS_LOC, sizeof(double) * 2 * n + small);
  Interp I;
  I.mA = (double*)sm;
  I.iB = I.mA + n;
  double* fA = I.iB + n;
  double* fB = fA + Njp;
  I.d = fB + Njp;
  I.is = I.d + Njp;
  int* iA = reinterpret_cast<int*>(I.is + Njp);
  int* iB = iA + Njp;
  std::vector<char> h(sizeof(double) * 4 * Njp + sizeof(int) * 2 * Njp);
  double* hd = reinterpret_cast<double*>(h.data());
  std::copy(facA, facA + Njp, hd);
  std::copy(facB, facB + Njp, hd + Njp);
  std::copy(d, d + Njp, hd + 2 * Njp);
  for (int i = 0; i < Njp; i++) hd[3 * Njp + i] = 1.0 / s[i];
  int* hi = reinterpret_cast<int*>(hd + 4 * Njp);
  std::copy(indA, indA + Njp, hi);
  std::copy(indB, indB + Njp, hi + Njp);
  MLC_CUDA(cudaMemcpy(fA, h.data(), h.size(), cudaMemcpyHostToDevice));
  for (int i = 0; i < Njp; i++) {
    MLC_REQUIRE(indA[i] >= -1 && indA[i] < Nprof - 1 && indB[i] >= -1 && indB[i] < Nprof - 1, MLC_ERR_ARG,
                "interpolation index out of the profile range");
  }
  if (n > 0) {
    {
      MLC_KSCOPE(ctx, "pair_interp");
      k_interp<<<grid_for(ctx, n), 256, 0, ctx->stream>>>(LCA, DLCA, Nloc, Nprof, Njp, iA, fA, 0, I.mA);
    }
    MLC_CHECK_LAUNCH();
    {
      MLC_KSCOPE(ctx, "pair_interp");
      k_interp<<<grid_for(ctx, n), 256, 0, ctx->stream>>>(LCB, DLCB, Nloc, Nprof, Njp, iB, fB, 1, I.iB);
    }
    MLC_CHECK_LAUNCH();
  }
  return I;
}

void pair_chi2_ratio(mlc_ctx* ctx, int Njp, const int* indA, const int* indB, const double* facA,
                     const double* facB, const double* d, const double* s, int Nloc, int Nprof, const double* LCA,
                     const double* DLCA, const double* LCB, const double* DLCB, const uint32_t* rank, double* chi2) {
  Interp I = build_interp(ctx, Njp, indA, indB, facA, facB, d, s, Nloc, Nprof, LCA, DLCA, LCB, DLCB);
  dim3 grid(ceil_div(Nloc, 32), ceil_div(Nloc, 8));
  {
    MLC_KSCOPE(ctx, "pair_chi2_ratio");
    k_pair_chi2_ratio<<<grid, 256, 0, ctx->stream>>>(I.mA, I.iB, Nloc, Njp, I.d, I.is, rank, chi2);
  }
  MLC_CHECK_LAUNCH();
}

void bin_chi2(mlc_ctx* ctx, int Nbins, const uint32_t* lower_host, const uint32_t* nper_host,
              const double* chi2_sorted, double* bchi2_host, double* bexp_host) {
  if (Nbins <= 0) return;
  std::vector<BinPiece> pieces;
  std::vector<uint32_t> pfirst(Nbins + 1), nper(nper_host, nper_host + Nbins);
  for (int b = 0; b < Nbins; b++) {
    pfirst[b] = (uint32_t)pieces.size();
    for (uint32_t k = 0; k < nper_host[b]; k += BIN_PIECE)
      pieces.push_back(BinPiece{lower_host[b] + k, std::min(BIN_PIECE, nper_host[b] - k)});
  }
  pfirst[Nbins] = (uint32_t)pieces.size();
  const size_t np = std::max<size_t>(pieces.size(), 1);
  char* sm = (char*)ws_get(ctx, WS_SMALL, sizeof(double) * (2 * Nbins + 2 * np) + sizeof(BinPiece) * np +
                                              sizeof(uint32_t) * (2 * Nbins + 1) + 256);
  double* bc = (double*)sm;
  double* be = bc + Nbins;
  double* ps = be + Nbins;
  double* pe = ps + np;
  BinPiece* dp = reinterpret_cast<BinPiece*>(pe + np);
  uint32_t* dfirst = reinterpret_cast<uint32_t*>(dp + np);
  uint32_t* dn = dfirst + Nbins + 1;
  if (!pieces.empty())
    MLC_CUDA(cudaMemcpyAsync(dp, pieces.data(), sizeof(BinPiece) * pieces.size(), cudaMemcpyHostToDevice, ctx->stream));
  MLC_CUDA(cudaMemcpyAsync(dfirst, pfirst.data(), sizeof(uint32_t) * (Nbins + 1), cudaMemcpyHostToDevice, ctx->stream));
  MLC_CUDA(cudaMemcpyAsync(dn, nper.data(), sizeof(uint32_t) * Nbins, cudaMemcpyHostToDevice, ctx->stream));
  if (!pieces.empty()) {
    MLC_KSCOPE(ctx, "pair_bin_means");
    k_bin_piece_sums<<<(unsigned)pieces.size(), 256, 0, ctx->stream>>>(chi2_sorted, dp, ps, pe);
  }
  MLC_CHECK_LAUNCH();
  {
    MLC_KSCOPE(ctx, "pair_bin_combine");
    k_bin_combine<<<ceil_div(Nbins, 128), 128, 0, ctx->stream>>>(dfirst, dn, ps, pe, Nbins, bc, be);
  }
  MLC_CHECK_LAUNCH();
  MLC_CUDA(cudaMemcpyAsync(bchi2_host, bc, sizeof(double) * Nbins, cudaMemcpyDeviceToHost, ctx->stream));
  MLC_CUDA(cudaMemcpyAsync(bexp_host, be, sizeof(double) * Nbins, cudaMemcpyDeviceToHost, ctx->stream));
  MLC_CUDA(cudaStreamSynchronize(ctx->stream));  // (also keeps the host vectors alive for the copies)
}

void pair_bin_fused(mlc_ctx* ctx, int Njp, const int* indA, const int* indB, const double* facA,
                    const double* facB, const double* d, const double* s, int Nloc, int Nprof, const double* LCA,
                    const double* DLCA, const double* LCB, const double* DLCB, int Nbins, const double* edges_host,
                    double* bchi2_host, double* bexp_host, uint32_t* nper_host) {
  MLC_REQUIRE(Nbins > 0 && Nbins <= 6000, MLC_ERR_LIMIT, "fused pair binning supports 1..6000 bins");
  Interp I = build_interp(ctx, Njp, indA, indB, facA, facB, d, s, Nloc, Nprof, LCA, DLCA, LCB, DLCB);
  char* sm = (char*)ws_get(ctx, WS_PAIR_ACC, (sizeof(double) * 3 + 8) * Nbins + 2 * sizeof(float) * Nloc + 128);
  double* de = (double*)sm;
  double* gs = de + Nbins;
  double* ge = gs + Nbins;
  unsigned long long* gc = reinterpret_cast<unsigned long long*>(ge + Nbins);
  float* zA = reinterpret_cast<float*>(gc + Nbins);
  float* zB = zA + Nloc;
  {
    MLC_KSCOPE(ctx, "pair_interp");
    k_zfloat<<<grid_for(ctx, Nloc), 256, 0, ctx->stream>>>(LCA, LCB, Nloc, Nprof, zA, zB);
  }
  MLC_CHECK_LAUNCH();
  MLC_CUDA(cudaMemcpyAsync(de, edges_host, sizeof(double) * Nbins, cudaMemcpyHostToDevice, ctx->stream));
  MLC_CUDA(cudaMemsetAsync(gs, 0, (sizeof(double) * 2 + 8) * Nbins, ctx->stream));
  const size_t smem = (sizeof(double) * 3 + sizeof(float) + sizeof(unsigned)) * Nbins;
  set_max_smem((const void*)k_pair_bin_fused, smem);
  dim3 grid(ceil_div(Nloc, 256), ceil_div(Nloc, FUSED_A));
  {
    MLC_KSCOPE(ctx, "pair_bin_fused");
    k_pair_bin_fused<<<grid, 256, smem, ctx->stream>>>(I.mA, I.iB, zA, zB, LCA, LCB, Nloc, Nprof, Njp, I.d, I.is,
                                                      Nbins, de, gs, ge, gc);
  }
  MLC_CHECK_LAUNCH();
  std::vector<double> hs(Nbins), he(Nbins);
  std::vector<unsigned long long> hc(Nbins);
  MLC_CUDA(cudaMemcpyAsync(hs.data(), gs, sizeof(double) * Nbins, cudaMemcpyDeviceToHost, ctx->stream));
  MLC_CUDA(cudaMemcpyAsync(he.data(), ge, sizeof(double) * Nbins, cudaMemcpyDeviceToHost, ctx->stream));
  MLC_CUDA(cudaMemcpyAsync(hc.data(), gc, sizeof(unsigned long long) * Nbins, cudaMemcpyDeviceToHost, ctx->stream));
  MLC_CUDA(cudaStreamSynchronize(ctx->stream));
  for (int i = 0; i < Nbins; i++) {
    if (hc[i]) {
      bchi2_host[i] = hs[i] / (double)hc[i];
      bexp_host[i] = he[i] / (double)hc[i];
    } else {
      bchi2_host[i] = 2000.0;
      bexp_host[i] = std::exp(-2000.0 / 2.0);
    }
    if (nper_host) nper_host[i] = (uint32_t)hc[i];
  }
}

}  // namespace mlc
