// Synthetic magnification maps by inverse ray shooting through a field of equal-mass
// point lenses with external shear (the input the reference reads as gerlumph maps,
// magnification_map.cpp:7-40).  Rays on a regular image-plane grid are deflected by all
// lenses (tiles of lenses staged in shared memory) and counted into the source-plane
// pixel they land in; the counts are the gerlumph int32 ray counts.
#include "mlc_internal.h"

namespace mlc {

// Every operation is an explicitly rounded FP32 (or FP64) intrinsic in a fixed order --
// no contraction into FMAs the compiler might choose -- so that a CPU program doing the
// same IEEE operations in the same order reproduces the counts exactly:
//   x1 = fp32(x0 + dx * i),  u = x1 - lx,  q = 1 / fma(u, u, v * v),  a1 = fma(u, q, a1)
// over the lenses in index order, y1 = (1 - kappa_c - gamma) * x1 - a1, and the pixel
// floor((y1 + w/2) * (N / w)).
__global__ void __launch_bounds__(256) k_rayshoot(const float2* __restrict__ lenses, int nl, float kappa_c,
                                                  float gamma, double x0, double y0, double dx, long nrx, long nry,
                                                  float half_w, int N, int* __restrict__ counts) {
  __shared__ float2 ls[1024];
  const long total = nrx * nry;
  const float scale = __fdiv_rn((float)N, __fmul_rn(2.0f, half_w));
  const float c1 = __fsub_rn(__fsub_rn(1.f, kappa_c), gamma);
  const float c2 = __fadd_rn(__fsub_rn(1.f, kappa_c), gamma);
  for (long base = (long)blockIdx.x * blockDim.x; base < total; base += (long)gridDim.x * blockDim.x) {
    const long r = base + threadIdx.x;
    const bool ok = r < total;
    const float x1 = (float)__dadd_rn(x0, __dmul_rn(dx, (double)(ok ? r % nrx : 0)));
    const float x2 = (float)__dadd_rn(y0, __dmul_rn(dx, (double)(ok ? r / nrx : 0)));
    float a1 = 0.f, a2 = 0.f;
    for (int t = 0; t < nl; t += 1024) {
      const int m = min(1024, nl - t);
      __syncthreads();
      for (int i = threadIdx.x; i < m; i += blockDim.x) ls[i] = lenses[t + i];
      __syncthreads();
#pragma unroll 8
      for (int i = 0; i < m; i++) {
        const float u = __fsub_rn(x1, ls[i].x), v = __fsub_rn(x2, ls[i].y);
        const float q = __frcp_rn(__fmaf_rn(u, u, __fmul_rn(v, v)));
        a1 = __fmaf_rn(u, q, a1);
        a2 = __fmaf_rn(v, q, a2);
      }
    }
    if (ok) {
      const float y1 = __fsub_rn(__fmul_rn(c1, x1), a1);
      const float y2 = __fsub_rn(__fmul_rn(c2, x2), a2);
      const int j = (int)floorf(__fmul_rn(__fadd_rn(y1, half_w), scale));
      const int i = (int)floorf(__fmul_rn(__fadd_rn(y2, half_w), scale));
      if (i >= 0 && i < N && j >= 0 && j < N) atomicAdd(counts + (long)i * N + j, 1);
    }
  }
}

}  // namespace mlc

using namespace mlc;

extern "C" int mlc_rayshoot(void* ctx_, const float* lenses_xy, int nl, double kappa_c, double gamma, double x0,
                            double y0, double dx, long nrx, long nry, double width, int N, int* counts) {
  mlc_ctx* ctx = (mlc_ctx*)ctx_;
  if (!ctx || (nl > 0 && !lenses_xy) || !counts || N < 1 || nrx < 1 || nry < 1 || !(width > 0) || !(dx > 0))
    return MLC_ERR_ARG;
  try {
    DeviceGuard g(ctx->device);
    MLC_CUDA(cudaMemsetAsync(counts, 0, sizeof(int) * (size_t)N * N, ctx->stream));
    const long total = nrx * nry;
    const int grid = (int)std::min<long>((total + 255) / 256, (long)ctx->sm_count * 8);
    {
      MLC_KSCOPE(ctx, "rayshoot");
      k_rayshoot<<<grid, 256, 0, ctx->stream>>>((const float2*)lenses_xy, nl, (float)kappa_c, (float)gamma, x0, y0,
                                              dx, nrx, nry, (float)(width / 2), N, counts);
    }
    MLC_CHECK_LAUNCH();
    return MLC_OK;
  } catch (const Error& e) {
    ctx->err = e.what();
    return e.code;
  }
}
