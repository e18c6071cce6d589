// Multi-filter flux-ratio likelihood of every pair of simulated locations, replacing
// getChi2GPU / getChi2CPU (chi2/chi2_functions.cuh:93-190):
//
//   chi2[x, y] = 1/2 sum_f sum_t ((f_obs[f,t] - mu1[x,f,t] / mu2[y,f,t]) / df_obs[f,t])^2
//   likelihood = sum over (x, y) of exp(-chi2[x, y])
//
// with the CPU twin's indexing (the reference's kernel reads mu2 at x, so its chi2 never
// depends on y).  The reference runs one thread per (x, y, filter) with a float atomic
// per filter into a managed N^2 array zero-filled on the host, then sums the N^2 exp()
// on one host core.  Here one CTA owns a 64 x 64 tile of pairs (each thread 4 x 4):
// the K = F*T values of its 64 + 64 locations are staged through shared memory in
// chunks of 32 with 1/mu2 and 1/df precomputed, so a pair costs 3 FP32 operations per
// (filter, time); exp(-chi2) is summed per thread relative to its smallest chi2 (FP32
// terms, one FP64-range exp per thread), per CTA in FP64, and the CTA sums are added in a
// fixed order (deterministic).  chi2 is stored only when asked for.
#include <vector>

#include "mlc_internal.h"

namespace mlc {

constexpr int FR_TILE = 64;  // locations per tile side
constexpr int FR_KC = 32;    // (filter, time) values per shared-memory chunk

__global__ void __launch_bounds__(256) k_flux_ratio(const float* __restrict__ mu1, const float* __restrict__ mu2,
                                                    const float* __restrict__ obs, const float* __restrict__ sinv,
                                                    int N, int K, float* __restrict__ chi2,
                                                    double* __restrict__ partial) {
  __shared__ __align__(16) float sa[FR_KC][FR_TILE];  // mu1 of the tile's x locations
  __shared__ __align__(16) float sr[FR_KC][FR_TILE];  // 1 / mu2 of the tile's y locations
  __shared__ float so[FR_KC], ss[FR_KC];
  __shared__ double red[8];
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  const int x0 = blockIdx.x * FR_TILE, y0 = blockIdx.y * FR_TILE;
  float acc[4][4];
#pragma unroll
  for (int j = 0; j < 4; j++)
#pragma unroll
    for (int i = 0; i < 4; i++) acc[j][i] = 0.f;

  for (int k0 = 0; k0 < K; k0 += FR_KC) {
    // stage: 64 locations x 32 values of each image into [k][location] (lanes along the
    // location: conflict-free stores; the 8 values of a 32-byte sector are read by
    // consecutive k steps from L1); padding (k >= K or location >= N) contributes 0
    for (int e = tid; e < FR_TILE * FR_KC; e += 256) {
      const int loc = e % FR_TILE, kk = e / FR_TILE;
      const int k = k0 + kk;
      const bool kin = k < K;
      const int xa = x0 + loc, yb = y0 + loc;
      sa[kk][loc] = (kin && xa < N) ? __ldg(mu1 + (long)xa * K + k) : 0.f;
      sr[kk][loc] = (kin && yb < N) ? 1.0f / __ldg(mu2 + (long)yb * K + k) : 0.f;
    }
    if (tid < FR_KC) {
      const int k = k0 + tid;
      so[tid] = k < K ? __ldg(obs + k) : 0.f;
      ss[tid] = k < K ? __ldg(sinv + k) : 0.f;
    }
    __syncthreads();
    const int kn = min(FR_KC, K - k0);
    for (int kk = 0; kk < kn; kk++) {
      const float4 a = *reinterpret_cast<const float4*>(&sa[kk][tx * 4]);
      const float4 r = *reinterpret_cast<const float4*>(&sr[kk][ty * 4]);
      const float o = so[kk], s = ss[kk];
      const float av[4] = {a.x, a.y, a.z, a.w};
      const float rv[4] = {r.x, r.y, r.z, r.w};
#pragma unroll
      for (int j = 0; j < 4; j++)
#pragma unroll
        for (int i = 0; i < 4; i++) {
          const float d = fmaf(-av[i], rv[j], o) * s;
          acc[j][i] = fmaf(d, d, acc[j][i]);
        }
    }
    __syncthreads();
  }

  // sum of exp(-chi2) over this thread's pairs as exp(-cmin) * sum expf(cmin - chi2): the
  // FP32 terms are in (0, 1] and only those below e^-87 of the largest underflow, and
  // one exp per thread takes the FP64 path when cmin is beyond the FP32 exp range
  float cmin = INFINITY;
#pragma unroll
  for (int j = 0; j < 4; j++)
#pragma unroll
    for (int i = 0; i < 4; i++)
      if (x0 + tx * 4 + i < N && y0 + ty * 4 + j < N) cmin = fminf(cmin, 0.5f * acc[j][i]);
  float esum = 0.f;
#pragma unroll
  for (int j = 0; j < 4; j++) {
    const int y = y0 + ty * 4 + j;
    float c[4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
      c[i] = 0.5f * acc[j][i];
      const int x = x0 + tx * 4 + i;
      if (x < N && y < N) esum += expf(cmin - c[i]);
    }
    if (chi2 && y < N) {
      const int x = x0 + tx * 4;
      float* dst = chi2 + (long)y * N + x;
      if (x + 3 < N && (((long)y * N + x) & 3) == 0) {
        *reinterpret_cast<float4*>(dst) = make_float4(c[0], c[1], c[2], c[3]);
      } else {
        for (int i = 0; i < 4; i++)
          if (x + i < N) dst[i] = c[i];
      }
    }
  }
  double lsum = 0.0;
  if (esum > 0.f) lsum = (cmin < 80.f ? (double)expf(-cmin) : exp(-(double)cmin)) * (double)esum;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
  if ((tid & 31) == 0) red[tid >> 5] = lsum;
  __syncthreads();
  if (tid == 0) {
    double t = 0.0;
    for (int w = 0; w < 8; w++) t += red[w];
    partial[blockIdx.y * gridDim.x + blockIdx.x] = t;
  }
}

// Fixed-order sum of the per-CTA partial likelihoods.
__global__ void __launch_bounds__(1024) k_sum_partials(const double* __restrict__ p, long n, double* __restrict__ out) {
  __shared__ double red[32];
  double s = 0.0;
  for (long i = threadIdx.x; i < n; i += blockDim.x) s += p[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
    *out = t;
  }
}

void flux_ratio_chi2(mlc_ctx* ctx, const float* f_obs_host, const float* df_obs_host, const float* mu1,
                     const float* mu2, int N, int F, int T, float* chi2, double* likelihood_host) {
  MLC_REQUIRE(N >= 1 && F >= 1 && T >= 1, MLC_ERR_ARG, "need N, F, T >= 1");
  MLC_REQUIRE(N <= 200000, MLC_ERR_LIMIT, "N <= 200000 locations");
  const int K = F * T;
  std::vector<float> h(2 * (size_t)K);
  for (int k = 0; k < K; k++) {
    h[k] = f_obs_host[k];
    h[K + k] = 1.0f / df_obs_host[k];
  }
  const int nt = (N + FR_TILE - 1) / FR_TILE;
  const long nblk = (long)nt * nt;
  const size_t hb = round_up((long)(2 * K * sizeof(float)), 256);
  char* ws = (char*)ws_get(ctx, WS_SMALL, hb + (size_t)nblk * sizeof(double) + 256);
  float* d_obs = (float*)ws;
  double* d_part = (double*)(ws + hb);
  double* d_like = d_part + nblk;
  MLC_CUDA(cudaMemcpyAsync(d_obs, h.data(), 2 * K * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
  {
    MLC_KSCOPE(ctx, "flux_ratio_chi2");
    k_flux_ratio<<<dim3(nt, nt), 256, 0, ctx->stream>>>(mu1, mu2, d_obs, d_obs + K, N, K, chi2, d_part);
  }
  MLC_CHECK_LAUNCH();
  {
    MLC_KSCOPE(ctx, "flux_ratio_sum");
    k_sum_partials<<<1, 1024, 0, ctx->stream>>>(d_part, nblk, d_like);
  }
  MLC_CHECK_LAUNCH();
  MLC_CUDA(cudaMemcpyAsync(likelihood_host, d_like, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  MLC_CUDA(cudaStreamSynchronize(ctx->stream));
}

}  // namespace mlc
