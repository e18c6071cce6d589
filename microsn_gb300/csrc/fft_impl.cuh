// Kernels and per-precision launch sequences of the 2-D FFT and of the FFT convolution
// (passes R, A, B and P0-P3 as described in fft.cu).  The four entry templates at the end
// are instantiated explicitly, one precision per translation unit (fft_f32.cu, fft_f64.cu;
// the float-float ones split over fft_ff_*.cu), so that their kernels compile in parallel.
#pragma once

#include <cooperative_groups.h>

#include <algorithm>
#include <cmath>
#include <type_traits>

#include "mlc_internal.h"

namespace mlc {

// ---------------------------------------------------------------- row loaders

template <typename T, typename Tin>
struct RealRows {
  const Tin* p;
  long ld;
  __device__ __forceinline__ C2<T> pair(int row, int n) const {
    const Tin* r = p + (long)row * ld + 2 * n;
    return C2<T>{(T)r[0], (T)r[1]};
  }
};

// Row j of the compacted wrapped profile: j < h is kernel row j (profile row h + j);
// j >= h is kernel row Ny - 2h + j (profile row j - h).  Columns follow
// Kernel::setKernel (magnification_map.cpp:186-193).
template <typename T>
struct ProfileRows {
  const double* prof;
  int N, h, Nx;
  __device__ __forceinline__ T at(int pr, int m) const {
    if (m < h) return (T)prof[(long)pr * N + h + m];
    if (m >= Nx - h) return (T)prof[(long)pr * N + m - (Nx - h)];
    return (T)0;
  }
  __device__ __forceinline__ C2<T> pair(int j, int n) const {
    int pr = (j < h) ? h + j : j - h;
    return C2<T>{at(pr, 2 * n), at(pr, 2 * n + 1)};
  }
};

// ---------------------------------------------------------------- row kernels

// Spectrum value k <= M of a real row from Z = FFT_M(x[2n] + i x[2n+1]):
// X[k] = (Z[k] + conj Z[M-k]) / 2 - i W_Nx^k (Z[k] - conj Z[M-k]) / 2, Z[M] = Z[0].
template <typename T>
__device__ __forceinline__ C2<T> r2c_split(const C2<T>* Z, int M, const C2<T>* __restrict__ twx, int k) {
  const C2<T> zk = Z[k == M ? 0 : k];
  const C2<T> zc = cconj(Z[k == 0 ? 0 : M - k]);
  const C2<T> s = cadd(zk, zc);
  const C2<T> wd = cmul(ldc(twx + k), csub(zk, zc));  // W_Nx^k (Z - conj Z')
  return C2<T>{(T)0.5 * (s.x + wd.y), (T)0.5 * (s.y - wd.x)};
}

// Real FFT of one row per CTA; writes Nx/2+1 complex values and zero padding up to Wp.
template <typename T, typename Loader>
__global__ void __launch_bounds__(512) k_rows_r2c(Loader ld, C2<T>* __restrict__ out, long pitch, int M,
                                                  RadixList rl, const C2<T>* __restrict__ twx) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C2<T>* a = reinterpret_cast<C2<T>*>(smem_raw);
  C2<T>* b = a + (M + 1);
  const int row = blockIdx.x;
  for (int n = threadIdx.x; n < M; n += blockDim.x) a[n] = ld.pair(row, n);
  __syncthreads();
  C2<T>* Z = fft_smem<T, false, 1>(a, b, rl, twx);
  C2<T>* o = out + (long)row * pitch;
  for (int k = threadIdx.x; k <= M; k += blockDim.x) o[k] = cfin(r2c_split(Z, M, twx, k));
  for (int k = M + 1 + threadIdx.x; k < pitch; k += blockDim.x) o[k] = C2<T>{(T)0, (T)0};
}

// Real FFT of one row per CTA with M = L1 L2 L3 (J = L2 L3) in three register levels, the
// forward counterpart of c2r3_row below (same item shapes, forward DFTs and twiddles):
//   level 1, item j < J:        z[J a + j] (a < L1) from the loader, DFT_L1 over a,
//                               twiddle W_M^(j k1)                    -> s[k1 J + j]
//   level 2, item (k1, m < L3): DFT_L2 over b of s[k1 J + L3 b + m], twiddle W_J^(m k2)
//                                                                      -> s[k1 J + k2 L3 + m]
//   level 3, item (k1, k2):     DFT_L3 over m                      -> Z[k1 + L1 (k2 + L2 k3)]
// then the split into Nx/2+1 spectrum values and the zero padding up to Wp.  FP32: four
// CTAs per SM (three for 16^3, whose 80 registers would spill at 64), like k_rows_c2r3;
// FP64 keeps the compiler's allocation (its 90 KB rows fit two CTAs per SM anyway).
template <typename T, int L1, int L2, int L3, typename Loader>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? (L1 == 16 ? 3 : 4) : 0)
    k_rows_r2c3(Loader ld, C2<T>* __restrict__ out, long pitch,
                                                   const C2<T>* __restrict__ twx) {
  constexpr int J = L2 * L3, M = L1 * J;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C2<T>* s = reinterpret_cast<C2<T>*>(smem_raw);
  C2<T>* wJ = s + M;  // W_J^e = W_Nx^(2 L1 e), e < J
  const int tid = threadIdx.x, row = blockIdx.x;
  for (int e = tid; e < J; e += blockDim.x) wJ[e] = ldc(twx + 2L * L1 * e);
  for (int j = tid; j < J; j += blockDim.x) {
    C2<T> v[L1];
#pragma unroll
    for (int a = 0; a < L1; a++) v[a] = ld.pair(row, J * a + j);
    Dft<T, L1, false>::run(v);
    s[j] = v[0];
#pragma unroll
    for (int k1 = 1; k1 < L1; k1++) s[k1 * J + j] = cmul(v[k1], ldc(twx + 2L * j * k1));  // W_M^(j k1)
  }
  __syncthreads();
  {
    const bool act = tid < L1 * L3;
    const int k1 = tid / L3, m = tid - k1 * L3;
    C2<T> u[L2];
    if (act) {
#pragma unroll
      for (int b = 0; b < L2; b++) u[b] = s[k1 * J + L3 * b + m];
      Dft<T, L2, false>::run(u);
#pragma unroll
      for (int k2 = 1; k2 < L2; k2++) u[k2] = cmul(u[k2], wJ[m * k2]);
    }
    __syncthreads();
    if (act) {
#pragma unroll
      for (int k2 = 0; k2 < L2; k2++) s[k1 * J + k2 * L3 + m] = u[k2];
    }
  }
  __syncthreads();
  {
    const bool act = tid < L1 * L2;
    const int k2 = tid / L1, k1 = tid - k2 * L1;
    C2<T> w[L3];
    if (act) {
#pragma unroll
      for (int m = 0; m < L3; m++) w[m] = s[k1 * J + k2 * L3 + m];
      Dft<T, L3, false>::run(w);
    }
    __syncthreads();
    if (act) {
#pragma unroll
      for (int k3 = 0; k3 < L3; k3++) s[k1 + L1 * (k2 + L2 * k3)] = w[k3];
    }
  }
  __syncthreads();
  C2<T>* o = out + (long)row * pitch;
  for (int k = tid; k <= M; k += blockDim.x) o[k] = cfin(r2c_split(s, M, twx, k));
  for (int k = M + 1 + tid; k < pitch; k += blockDim.x) o[k] = C2<T>{(T)0, (T)0};
}

// Inverse real FFT (unnormalised, like cuFFT Z2D) of one spectrum row per CTA.
template <typename T, typename TO>
__global__ void __launch_bounds__(512) k_rows_c2r(const C2<T>* __restrict__ in, long pitch,
                                                  TO* __restrict__ out, long ldo, int M,
                                                  RadixList rl, const C2<T>* __restrict__ twx) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C2<T>* a = reinterpret_cast<C2<T>*>(smem_raw);
  C2<T>* b = a + (M + 1);
  const int row = blockIdx.x;
  const C2<T>* src = in + (long)row * pitch;
  for (int k = threadIdx.x; k <= M; k += blockDim.x) a[k] = src[k];
  __syncthreads();
  for (int k = threadIdx.x; k < M; k += blockDim.x) {
    C2<T> xk = a[k];
    C2<T> xm = cconj(a[M - k]);
    C2<T> e = cadd(xk, xm);
    C2<T> o = cmulc(csub(xk, xm), ldc(twx + k));  // (X - conj X') W^-k
    b[k] = C2<T>{e.x - o.y, e.y + o.x};
  }
  __syncthreads();
  C2<T>* z = fft_smem<T, true, 1>(b, a, rl, twx);
  C2<TO>* dst = reinterpret_cast<C2<TO>*>(out + (long)row * ldo);
  for (int n = threadIdx.x; n < M; n += blockDim.x) dst[n] = C2<TO>{out_cvt<TO>(z[n].x), out_cvt<TO>(z[n].y)};
}

// Inverse real FFT of one spectrum row per CTA with M = L1 L2 L3 (J = L2 L3) in three
// register levels.  b[k] = (X[k] + conj X[M-k]) + i (X[k] - conj X[M-k]) W_Nx^-k is the
// complex sequence whose inverse FFT z gives the real row (out[2n], out[2n+1]) = z[n].
//   level 1, item j < J:        b[J a + j] (a < L1) from global memory, DFT^-1_L1 over a,
//                               twiddle W_M^-(j n1)                   -> s[n1 J + j]
//   level 2, item (n1, m < L3): DFT^-1_L2 over b of s[n1 J + L3 b + m], twiddle W_J^-(m n2)
//                                                                      -> s[n1 J + n2 L3 + m]
//   level 3, item (n1, n2):     DFT^-1_L3 over m                      -> z[n1 + L1 (n2 + L2 n3)]
// and one coalesced copy of z to the output row.  Levels 2 and 3 read all their inputs
// before a barrier and then overwrite the same buffer (M complex values, 40 KB at
// M = 5000 in FP32).  Items of levels 2 and 3 fit in one pass of the CTA (L1 L3 and
// L1 L2 <= blockDim).
template <typename T, int L1, int L2, int L3>
__device__ __forceinline__ void c2r3_row(const C2<T>* __restrict__ a, const C2<T>* __restrict__ twx, C2<T>* s) {
  constexpr int J = L2 * L3, M = L1 * J;
  C2<T>* wJ = s + M;  // W_J^e = W_Nx^(2 L1 e), e < J
  const int tid = threadIdx.x;
  for (int e = tid; e < J; e += blockDim.x) wJ[e] = ldc(twx + 2L * L1 * e);
  for (int j = tid; j < J; j += blockDim.x) {
    C2<T> v[L1];
#pragma unroll
    for (int q = 0; q < L1; q++) {
      const int k = J * q + j;
      const C2<T> xk = ldc(a + k), xm = cconj(ldc(a + (M - k)));
      const C2<T> e = cadd(xk, xm);
      const C2<T> o = cmulc(csub(xk, xm), ldc(twx + k));  // (X - conj X') W^-k
      v[q] = C2<T>{e.x - o.y, e.y + o.x};
    }
    Dft<T, L1, true>::run(v);
    s[j] = v[0];
#pragma unroll
    for (int n1 = 1; n1 < L1; n1++) s[n1 * J + j] = cmulc(v[n1], ldc(twx + 2L * j * n1));  // W_M^-(j n1)
  }
  __syncthreads();
  {
    const bool act = tid < L1 * L3;
    const int n1 = tid / L3, m = tid - n1 * L3;
    C2<T> u[L2];
    if (act) {
#pragma unroll
      for (int b = 0; b < L2; b++) u[b] = s[n1 * J + L3 * b + m];
      Dft<T, L2, true>::run(u);
#pragma unroll
      for (int n2 = 1; n2 < L2; n2++) u[n2] = cmulc(u[n2], wJ[m * n2]);
    }
    __syncthreads();
    if (act) {
#pragma unroll
      for (int n2 = 0; n2 < L2; n2++) s[n1 * J + n2 * L3 + m] = u[n2];
    }
  }
  __syncthreads();
  {
    const bool act = tid < L1 * L2;
    const int n2 = tid / L1, n1 = tid - n2 * L1;  // n1 fastest: the writes below are contiguous
    C2<T> w[L3];
    if (act) {
#pragma unroll
      for (int m = 0; m < L3; m++) w[m] = s[n1 * J + n2 * L3 + m];
      Dft<T, L3, true>::run(w);
    }
    __syncthreads();
    if (act) {
#pragma unroll
      for (int n3 = 0; n3 < L3; n3++) s[n1 + L1 * (n2 + L2 * n3)] = w[n3];
    }
  }
  __syncthreads();
}

template <typename T, int L1, int L2, int L3, typename TO>
__global__ void __launch_bounds__(256) k_rows_c2r3(const C2<T>* __restrict__ in, long pitch,
                                                   TO* __restrict__ out, long ldo,
                                                   const C2<T>* __restrict__ twx) {
  constexpr int M = L1 * L2 * L3;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C2<T>* s = reinterpret_cast<C2<T>*>(smem_raw);
  const int row = blockIdx.x;
  c2r3_row<T, L1, L2, L3>(in + (long)row * pitch, twx, s);
  C2<TO>* dst = reinterpret_cast<C2<TO>*>(out + (long)row * ldo);
  for (int n = threadIdx.x; n < M; n += blockDim.x) dst[n] = C2<TO>{out_cvt<TO>(s[n].x), out_cvt<TO>(s[n].y)};
}

// P3 of four profiles with the interleave fused in.  A cluster of four CTAs takes one row
// of four profiles' spectra (CTA rank k: profile 4*quad + k; ranks past nm hold zeros),
// each CTA runs the three-level c2r of its row into its own shared memory, and after a
// cluster barrier CTA k writes pixels [k Nx/4, (k+1) Nx/4) of the interleaved row, reading
// the four rows through distributed shared memory: out[(row Nx + x) S + 4 quad + q], one
// 16-byte store per pixel (FP32).  The clusters of the other profiles of the same row are
// launched next to it, so their stores complete each 32-byte sector in L2 before it is
// written back.  No planar maps and no separate interleave pass; the arithmetic is
// k_rows_c2r3's.  (Measured at 10000^2, 16 profiles: clusters of 4 6.0 ms, of 8 6.1 ms,
// of 2 or 1 (8- or 4-byte strided stores) 9.8 ms.)
template <typename T, int L1, int L2, int L3, typename TO>
__global__ void __cluster_dims__(4, 1, 1) __launch_bounds__(256)
    k_rows_c2r3_il(const C2<T>* __restrict__ specs, long spec_stride, long pitch, int nm,
                   TO* __restrict__ out, int S, const C2<T>* __restrict__ twx, unsigned planar) {
  constexpr int J = L2 * L3, M = L1 * J, NX = 2 * M;
  namespace cg = cooperative_groups;
  cg::cluster_group cl = cg::this_cluster();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C2<T>* s = reinterpret_cast<C2<T>*>(smem_raw);
  const int row = blockIdx.y;
  const int k = (int)cl.block_rank(), quad = blockIdx.x >> 2, q = 4 * quad + k;
  if (q < nm && ((planar >> q) & 1u)) {  // the direct form's real map: copy its row
    const TO* src = reinterpret_cast<const TO*>(specs + (long)q * spec_stride) + (long)row * NX;
    T* d = reinterpret_cast<T*>(s);
    for (int n = threadIdx.x; n < NX; n += blockDim.x) d[n] = T(src[n]);
  } else if (q < nm) {
    c2r3_row<T, L1, L2, L3>(specs + (long)q * spec_stride + (long)row * pitch, twx, s);
  } else {
    for (int n = threadIdx.x; n < M; n += blockDim.x) s[n] = C2<T>{T(0), T(0)};
  }
  cl.sync();  // every row of the cluster is in its CTA's shared memory
  const int W = S - 4 * quad < 4 ? S - 4 * quad : 4;  // values per pixel from this cluster
  constexpr int CH = (NX + 3) / 4;
  const int x0 = k * CH, x1 = x0 + CH < NX ? x0 + CH : NX;
  TO* dst = out + (long)row * NX * S + 4 * quad;
  if (W == 4) {
    const T* src[4];
#pragma unroll
    for (int r = 0; r < 4; r++) src[r] = reinterpret_cast<const T*>(cl.map_shared_rank(s, r));
    for (int x = x0 + threadIdx.x; x < x1; x += blockDim.x) {
      TO v[4];
#pragma unroll
      for (int r = 0; r < 4; r++) v[r] = out_cvt<TO>(src[r][x]);
      float4* d = reinterpret_cast<float4*>(dst + (long)x * S);
      const float4* w = reinterpret_cast<const float4*>(v);
#pragma unroll
      for (int i = 0; i < (int)(4 * sizeof(TO) / 16); i++) d[i] = w[i];
    }
  } else {
    for (int r = 0; r < W; r++) {
      const T* sr = reinterpret_cast<const T*>(cl.map_shared_rank(s, r));
      for (int x = x0 + threadIdx.x; x < x1; x += blockDim.x) dst[(long)x * S + r] = out_cvt<TO>(sr[x]);
    }
  }
  // no CTA leaves while the others still read its shared memory.  Execution order is all
  // this barrier needs (every remote load has returned before the stores that use it), so
  // the arrive is relaxed: no release fence for this CTA's global stores.
  asm volatile("barrier.cluster.arrive.relaxed.aligned;\n\tbarrier.cluster.wait.aligned;" ::: "memory");
}

// The same last pass for float-float rows of M = 5000 = 8 x 5^4 points, with levels small
// enough for 64 registers: a float-float DFT25 item of the three-level form holds 100
// registers of data alone, which left two CTAs of 256 threads (16 warps) per SM, waiting
// on its barriers.  Here the c2r sequence b is formed first, both partners k and M - k of
// one read of the row (into shared memory); level 1 is the three-level form's (DFT8 over
// stride 625, twiddle W_M^-(j n1)), in place; then in-place decimation-in-frequency radix-5 levels on
// blocks of 625, 125, 25 (item (block, m < J'/5): DFT5 over stride J'/5, twiddle
// W_J'^-(m r), written back to the slots it read, so a thread takes its items one after
// another with no barrier between them); the last radix-5 level on blocks of 5 reads its
// items, waits, and writes them in natural order: output r of item
// it = 125 k1 + 25 a + 5 b + c is z[k1 + 8 (a + 5 (b + 5 (c + 5 r)))] = z[n0 + 1000 r].  512 threads, two
// CTAs (32 warps) per SM, the same number of barriers as the three-level form.
template <typename T, int JP, bool INV = true>
__device__ __forceinline__ void c2r5_level(C2<T>* s, const C2<T>* w) {
  constexpr int SP = JP / 5, WS = 625 / JP, NB = 5000 / JP;
  for (int it = threadIdx.x; it < 1000; it += blockDim.x) {
    // Item (blk, m) reads and writes s[blk JP + m + r SP], r < 5.  With runs of SP >= 32 the
    // warp's 32 consecutive m are 32 consecutive elements; shorter runs (JP = 125, 25) would
    // put a warp over blocks JP apart in a few banks (a 5-way conflict at JP = 25), so there
    // consecutive threads take consecutive blocks instead: stride JP (odd) in 16-byte
    // elements spreads them over every bank, and the warp shares its twiddles.
    int blk, m;
    if constexpr (SP >= 32) {
      blk = it / SP;
      m = it - blk * SP;
    } else {
      m = it / NB;
      blk = it - m * NB;
    }
    C2<T>* b = s + blk * JP + m;
    C2<T> u[5];
#pragma unroll
    for (int r = 0; r < 5; r++) u[r] = b[r * SP];
    Dft<T, 5, INV>::run(u);
    b[0] = u[0];
#pragma unroll
    for (int r = 1; r < 5; r++) b[r * SP] = INV ? cmulc(u[r], w[m * r * WS]) : cmul(u[r], w[m * r * WS]);
  }
  __syncthreads();
}

template <typename T>
__device__ __forceinline__ void c2r5_row(const C2<T>* __restrict__ a, const C2<T>* __restrict__ twx, C2<T>* s) {
  constexpr int M = 5000, J = 625;
  C2<T>* w = s + M;  // W_625^e = W_Nx^(16 e), e < 625
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int e = tid; e < J; e += nt) w[e] = ldc(twx + 16L * e);
  // b[k] = e + i o with e = X[k] + conj X[M-k], o = (X[k] - conj X[M-k]) W^-k, and for the
  // partner M - k: e' = conj e and, as W^-(M-k) = -conj W^-k, o' = conj o, so
  // b[M-k] = (e.x + o.y, o.x - e.y).  One thread forms both from one read of each input.
  // two partners' loads in flight per thread at a time (the row comes from DRAM)
  auto form = [&](int k, C2<T> xk, C2<T> xm, C2<T> w) {
    const C2<T> e = cadd(xk, xm);
    const C2<T> o = cmulc(csub(xk, xm), w);  // (X - conj X') W^-k
    s[k] = C2<T>{e.x - o.y, e.y + o.x};
    if (k > 0 && k < M / 2) s[M - k] = C2<T>{e.x + o.y, o.x - e.y};
  };
  int k = tid;
  for (; k + nt <= M / 2; k += 2 * nt) {
    const int k2 = k + nt;
    const C2<T> xk = ldc(a + k), xm = cconj(ldc(a + (M - k))), w = ldc(twx + k);
    const C2<T> xk2 = ldc(a + k2), xm2 = cconj(ldc(a + (M - k2))), w2 = ldc(twx + k2);
    form(k, xk, xm, w);
    form(k2, xk2, xm2, w2);
  }
  if (k <= M / 2) form(k, ldc(a + k), cconj(ldc(a + (M - k))), ldc(twx + k));
  __syncthreads();
  // item j reads b[J q + j] (q < 8) and writes its outputs to the same eight slots
  for (int j = tid; j < J; j += nt) {
    C2<T> v[8];
#pragma unroll
    for (int q = 0; q < 8; q++) v[q] = s[J * q + j];
    Dft<T, 8, true>::run(v);
    // W_M^-(j n1) = conj(W_M^j)^n1: one table load (the other powers read at strides of
    // 2 n1 entries fetched a sector per lane), the powers by products at most three deep,
    // each used as soon as it is formed
    s[j] = v[0];
    const C2<T> p1 = ldc(twx + 2L * j);
    s[J + j] = cmulc(v[1], p1);
    const C2<T> p2 = cmul(p1, p1);
    s[2 * J + j] = cmulc(v[2], p2);
    const C2<T> p3 = cmul(p2, p1);
    s[3 * J + j] = cmulc(v[3], p3);
    const C2<T> p4 = cmul(p2, p2);
    s[4 * J + j] = cmulc(v[4], p4);
    s[5 * J + j] = cmulc(v[5], cmul(p3, p2));
    s[6 * J + j] = cmulc(v[6], cmul(p3, p3));
    s[7 * J + j] = cmulc(v[7], cmul(p4, p3));
  }
  __syncthreads();
  c2r5_level<T, 625>(s, w);
  c2r5_level<T, 125>(s, w);
  c2r5_level<T, 25>(s, w);
  // blocks of 5: every item read (two per thread at most: blockDim >= 500), then written
  // in natural order.  Thread t takes the item whose outputs land at n0 = t (and t + nt),
  // n0 + 1000 r: consecutive threads write consecutive slots (taking items in their own
  // order instead put a warp's writes 200 slots apart, all in one shared-memory bank)
  C2<T> u[2][5];
#pragma unroll
  for (int h = 0; h < 2; h++) {
    const int n0 = tid + h * nt;
    if (n0 < 1000) {
      const int it = 125 * (n0 % 8) + 25 * ((n0 / 8) % 5) + 5 * ((n0 / 40) % 5) + n0 / 200;
#pragma unroll
      for (int r = 0; r < 5; r++) u[h][r] = s[5 * it + r];
      Dft<T, 5, true>::run(u[h]);
    }
  }
  __syncthreads();
#pragma unroll
  for (int h = 0; h < 2; h++) {
    const int n0 = tid + h * nt;
    if (n0 < 1000) {
#pragma unroll
      for (int r = 0; r < 5; r++) s[n0 + 1000 * r] = u[h][r];
    }
  }
  __syncthreads();
}

template <typename T, typename TO>
__global__ void __cluster_dims__(4, 1, 1) __launch_bounds__(512, 2)
    k_rows_c2r5_il(const C2<T>* __restrict__ specs, long spec_stride, long pitch, int nm, TO* __restrict__ out,
                   int S, const C2<T>* __restrict__ twx, unsigned planar) {
  constexpr int NX = 10000;
  namespace cg = cooperative_groups;
  cg::cluster_group cl = cg::this_cluster();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C2<T>* s = reinterpret_cast<C2<T>*>(smem_raw);
  const int row = blockIdx.y;
  const int k = (int)cl.block_rank(), quad = blockIdx.x >> 2, q = 4 * quad + k;
  if (q < nm && ((planar >> q) & 1u)) {  // the direct form's real map: copy its row
    const TO* src = reinterpret_cast<const TO*>(specs + (long)q * spec_stride) + (long)row * NX;
    T* d = reinterpret_cast<T*>(s);
    for (int n = threadIdx.x; n < NX; n += blockDim.x) d[n] = T(src[n]);
  } else if (q < nm) {
    c2r5_row<T>(specs + (long)q * spec_stride + (long)row * pitch, twx, s);
  } else {
    for (int n = threadIdx.x; n < NX / 2; n += blockDim.x) s[n] = C2<T>{T(0), T(0)};
  }
  cl.sync();  // every row of the cluster is in its CTA's shared memory
  const int W = S - 4 * quad < 4 ? S - 4 * quad : 4;
  constexpr int CH = NX / 4;
  const int x0 = k * CH, x1 = x0 + CH;
  TO* dst = out + (long)row * NX * S + 4 * quad;
  if (W == 4) {
    const T* src[4];
#pragma unroll
    for (int r = 0; r < 4; r++) src[r] = reinterpret_cast<const T*>(cl.map_shared_rank(s, r));
    for (int x = x0 + threadIdx.x; x < x1; x += blockDim.x) {
      TO v[4];
#pragma unroll
      for (int r = 0; r < 4; r++) v[r] = out_cvt<TO>(src[r][x]);
      float4* d = reinterpret_cast<float4*>(dst + (long)x * S);
      const float4* wv = reinterpret_cast<const float4*>(v);
#pragma unroll
      for (int i = 0; i < (int)(4 * sizeof(TO) / 16); i++) d[i] = wv[i];
    }
  } else {
    for (int r = 0; r < W; r++) {
      const T* sr = reinterpret_cast<const T*>(cl.map_shared_rank(s, r));
      for (int x = x0 + threadIdx.x; x < x1; x += blockDim.x) dst[(long)x * S + r] = out_cvt<TO>(sr[x]);
    }
  }
  // no CTA leaves while the others still read its shared memory (relaxed: see k_rows_c2r3_il)
  asm volatile("barrier.cluster.arrive.relaxed.aligned;\n\tbarrier.cluster.wait.aligned;" ::: "memory");
}

// The forward counterpart of c2r5_row for float-float rows of M = 5000: level 1 (DFT8 over
// stride 625 of the loader's pairs, twiddles W_M^(j k1) as products of the one loaded
// W_M^j), the three radix-5 levels and the last one in natural order as in c2r5_row (forward
// DFTs, unconjugated twiddles), then the split into Nx/2+1 spectrum values and the zero
// padding up to Wp.  512 threads, two CTAs per SM, like the last pass.
template <typename Loader>
__global__ void __launch_bounds__(512, 2) k_rows_r2c5(Loader ld, C2<ff>* __restrict__ out, long pitch,
                                                      const C2<ff>* __restrict__ twx) {
  constexpr int M = 5000, J = 625;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C2<ff>* s = reinterpret_cast<C2<ff>*>(smem_raw);
  C2<ff>* w = s + M;  // W_625^e = W_Nx^(16 e), e < 625
  const int tid = threadIdx.x, nt = blockDim.x, row = blockIdx.x;
  for (int e = tid; e < J; e += nt) w[e] = ldc(twx + 16L * e);
  for (int j = tid; j < J; j += nt) {
    C2<ff> v[8];
#pragma unroll
    for (int q = 0; q < 8; q++) v[q] = ld.pair(row, J * q + j);
    Dft<ff, 8, false>::run(v);
    s[j] = v[0];
    const C2<ff> p1 = ldc(twx + 2L * j);
    s[J + j] = cmul(v[1], p1);
    const C2<ff> p2 = cmul(p1, p1);
    s[2 * J + j] = cmul(v[2], p2);
    const C2<ff> p3 = cmul(p2, p1);
    s[3 * J + j] = cmul(v[3], p3);
    const C2<ff> p4 = cmul(p2, p2);
    s[4 * J + j] = cmul(v[4], p4);
    s[5 * J + j] = cmul(v[5], cmul(p3, p2));
    s[6 * J + j] = cmul(v[6], cmul(p3, p3));
    s[7 * J + j] = cmul(v[7], cmul(p4, p3));
  }
  __syncthreads();
  c2r5_level<ff, 625, false>(s, w);
  c2r5_level<ff, 125, false>(s, w);
  c2r5_level<ff, 25, false>(s, w);
  C2<ff> u[2][5];
#pragma unroll
  for (int h = 0; h < 2; h++) {
    const int n0 = tid + h * nt;
    if (n0 < 1000) {
      const int it = 125 * (n0 % 8) + 25 * ((n0 / 8) % 5) + 5 * ((n0 / 40) % 5) + n0 / 200;
#pragma unroll
      for (int r = 0; r < 5; r++) u[h][r] = s[5 * it + r];
      Dft<ff, 5, false>::run(u[h]);
    }
  }
  __syncthreads();
#pragma unroll
  for (int h = 0; h < 2; h++) {
    const int n0 = tid + h * nt;
    if (n0 < 1000) {
#pragma unroll
      for (int r = 0; r < 5; r++) s[n0 + 1000 * r] = u[h][r];
    }
  }
  __syncthreads();
  C2<ff>* o = out + (long)row * pitch;
  for (int k = tid; k <= M; k += nt) o[k] = cfin(r2c_split(s, M, twx, k));
  for (int k = M + 1 + tid; k < pitch; k += nt) o[k] = C2<ff>{ff(0), ff(0)};
}

// ---------------------------------------------------------------- column kernels

// In-place sub-pass over the row set {set*set_mul + j*j_mul : j < L} of one strip of CW
// columns.  post_tw multiplies output j by W_Ny^(+/- set*j).
template <typename T, int CW, bool INV>
__global__ void __launch_bounds__(256) k_colpass(C2<T>* __restrict__ buf, long pitch, int L, long set_mul,
                                                 long j_mul, RadixList rl, const C2<T>* __restrict__ twy,
                                                 int tw_stride, int post_tw) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C2<T>* a = reinterpret_cast<C2<T>*>(smem_raw);
  C2<T>* b = a + L * CW;
  C2<T>* tab = b + L * CW;   // stage twiddles (rl.tlen)
  C2<T>* pw = tab + rl.tlen; // post twiddles W_Ny^(set j), j < L
  const int set = blockIdx.y;
  const long col0 = (long)blockIdx.x * CW;
  const long base = (long)set * set_mul;
  for (int idx = threadIdx.x; idx < L * CW; idx += blockDim.x) {
    int j = idx / CW, c = idx % CW;
    a[idx] = buf[(base + j * j_mul) * pitch + col0 + c];
  }
  fill_stage_twiddles<T>(rl, twy, tab);
  if (post_tw)
    for (int j = threadIdx.x; j < L; j += blockDim.x) pw[j] = ldc(twy + (long)set * j);  // set*j < Ny
  __syncthreads();
  C2<T>* r = fft_smem_st<T, INV, CW>(a, b, rl, tab);
  for (int idx = threadIdx.x; idx < L * CW; idx += blockDim.x) {
    int j = idx / CW, c = idx % CW;
    C2<T> v = r[idx];
    if (post_tw) v = INV ? cmulc(v, pw[j]) : cmul(v, pw[j]);
    buf[(base + j * j_mul) * pitch + col0 + c] = cfin(v);
  }
}

// The same sub-pass for L = L1 * L2 with both factors done in registers (four-step):
// thread (n2, c) loads x[L2 n1 + n2] (n1 < L1) straight from global memory, DFT_L1 over n1,
// twiddle W_L^(n2 k1), one transpose through shared memory, then thread (k1, c) does
// DFT_L2 over n2 and writes X[k1 + L1 k2] straight back.  One shared-memory round trip and
// fixed per-thread indices instead of a Stockham stage loop per radix.
template <typename T, int CW, int L1, int L2, bool INV>
__global__ void __launch_bounds__(256) k_colpass2(C2<T>* __restrict__ buf, long pitch, long set_mul, long j_mul,
                                                  const C2<T>* __restrict__ twy, int tw_stride, int post_tw) {
  constexpr int L = L1 * L2;
  __shared__ C2<T> y[L2][L1][CW];
  __shared__ C2<T> wl[L];  // W_L^m
  __shared__ C2<T> pw[L];  // post twiddles W_Ny^(set j)
  const int set = blockIdx.y;
  const long col0 = (long)blockIdx.x * CW;
  const long base = (long)set * set_mul;
  const int c = threadIdx.x % CW, g = threadIdx.x / CW;
  for (int m = threadIdx.x; m < L; m += blockDim.x) {
    wl[m] = ldc(twy + (long)m * tw_stride);
    if (post_tw) pw[m] = ldc(twy + (long)set * m);  // set*m < Ny
  }
  C2<T> v[L1];
  if (g < L2) {
#pragma unroll
    for (int n1 = 0; n1 < L1; n1++) v[n1] = buf[(base + (long)(L2 * n1 + g) * j_mul) * pitch + col0 + c];
  }
  __syncthreads();
  if (g < L2) {
    Dft<T, L1, INV>::run(v);
#pragma unroll
    for (int k1 = 0; k1 < L1; k1++) y[g][k1][c] = (k1 == 0) ? v[0] : (INV ? cmulc(v[k1], wl[g * k1]) : cmul(v[k1], wl[g * k1]));
  }
  __syncthreads();
  if (g < L1) {
    C2<T> u[L2];
#pragma unroll
    for (int n2 = 0; n2 < L2; n2++) u[n2] = y[n2][g][c];
    Dft<T, L2, INV>::run(u);
#pragma unroll
    for (int k2 = 0; k2 < L2; k2++) {
      const int j = g + L1 * k2;
      C2<T> val = u[k2];
      if (post_tw) val = INV ? cmulc(val, pw[j]) : cmul(val, pw[j]);
      // inverse passes store float-float values as they are: the row pass that reads them
      // (the last of the transform) rounds each pixel from both parts
      buf[(base + (long)j * j_mul) * pitch + col0 + c] = INV ? val : cfin(val);
    }
  }
}

// P1 of the fused convolution, one CTA per (strip, k1).
template <typename T, int CW>
__global__ void __launch_bounds__(256) k_conv_fused(const C2<T>* __restrict__ Fmap, C2<T>* __restrict__ out,
                                                    long pitch, const C2<T>* __restrict__ Kx, int h, int Ny,
                                                    int N1, int N2, RadixList rl2,
                                                    const C2<T>* __restrict__ twy, T scale) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C2<T>* a = reinterpret_cast<C2<T>*>(smem_raw);
  C2<T>* b = a + N2 * CW;
  C2<T>* w1 = b + N2 * CW;   // W_N1^(n1 k1) for n1 < N1, this CTA's k1
  C2<T>* w2 = w1 + N1;       // W_Ny^(n2 k1) for n2 < N2
  C2<T>* tab = w2 + N2;      // stage twiddles of the N2 transforms (rl2.tlen)
  const int k1 = blockIdx.y;
  const long col0 = (long)blockIdx.x * CW;
  for (int n1 = threadIdx.x; n1 < N1; n1 += blockDim.x) w1[n1] = ldc(twy + ((n1 * k1) % N1) * N2);
  for (int n2 = threadIdx.x; n2 < N2; n2 += blockDim.x) w2[n2] = ldc(twy + (long)n2 * k1);
  fill_stage_twiddles<T>(rl2, twy, tab);
  __syncthreads();
  // profile: column sub-pass A restricted to its non-zero rows, then twiddle W_Ny^(n2 k1)
  const int lo = Ny - h;  // first non-zero high row
  for (int idx = threadIdx.x; idx < N2 * CW; idx += blockDim.x) {
    const int n2 = idx / CW, c = idx & (CW - 1);
    C2<T> acc{(T)0, (T)0};
    for (int n1 = 0; n1 * N2 + n2 < h; n1++) {
      const long j = (long)n1 * N2 + n2;
      acc = cadd(acc, cmul(Kx[j * pitch + col0 + c], w1[n1]));
    }
    int n1s = (lo - n2 + N2 - 1) / N2;
    if (n1s < 0) n1s = 0;
    for (int n1 = n1s; n1 < N1; n1++) {
      const long j = (long)n1 * N2 + n2 - (Ny - 2L * h);
      acc = cadd(acc, cmul(Kx[j * pitch + col0 + c], w1[n1]));
    }
    a[idx] = cmul(acc, w2[n2]);
  }
  __syncthreads();
  C2<T>* K = fft_smem_st<T, false, CW>(a, b, rl2, tab);
  C2<T>* other = (K == a) ? b : a;
  for (int idx = threadIdx.x; idx < N2 * CW; idx += blockDim.x) {
    const int k2 = idx / CW, c = idx % CW;
    C2<T> f = Fmap[((long)k1 * N2 + k2) * pitch + col0 + c];
    K[idx] = cscale(cmul(f, K[idx]), scale);
  }
  __syncthreads();
  C2<T>* U = fft_smem_st<T, true, CW>(K, other, rl2, tab);
  for (int idx = threadIdx.x; idx < N2 * CW; idx += blockDim.x) {
    const int n2 = idx / CW, c = idx % CW;
    C2<T> v = cmulc(U[idx], w2[n2]);
    out[((long)k1 * N2 + n2) * pitch + col0 + c] = cfin(v);
  }
}

// P1 for N2 = L1 * L2 with both factors in registers.  Forward N2 transform of the profile
// column (built in shared memory as in k_conv_fused) as a four-step: thread (n2, c) DFT_L1
// over x[L2 n1 + n2], twiddle, transpose, thread (k1, c) DFT_L2 -> it now holds frequencies
// k = k1 + L1 k2, multiplies them by the map spectrum (read straight from global memory)
// and 1/(Nx Ny), and starts the inverse as the transposed four-step on the same registers:
// DFT^-1_L2 over k2, twiddle W_N2^-(k1 n2), transpose, thread (n2, c) DFT^-1_L1 over k1 ->
// rows n2 + L2 n1, times W_Ny^-(n kk), stored.  (Staging the map-spectrum tile in shared
// memory with cp.async made this kernel 3 % faster alone but the two-chain step 3 % slower:
// the extra 12.8 KB per CTA crowds out the other chain's P2 CTAs.)  The FP32 kernels of at
// most 160 threads are held to 40 registers (ten CTAs per SM instead of seven for 10 x 10,
// 8 bytes of spills): this pass waits on latency, and the extra CTAs hide more of it
// (4.31 -> 4.13 ms per 16 profiles at 10000^2).
// STAGE: the map-spectrum tile is copied into shared memory (cp.async, 16 bytes per copy,
// issued at the start and waited for before forward stage 2) instead of being prefetched
// into L2 and read from there in stage 2: no global-load latency in stage 2, for
// N2 CW sizeof(C2<T>) more shared memory per CTA (fewer resident CTAs).
// MODE splits the pass around the profile's spectrum, for profiles that are convolved with
// many maps: 1 stops after forward stage 2 and stores the profile's spectrum, already scaled
// by 1/(Nx Ny), in the map spectrum's layout into ks (as the registers hold it, so that
// mode 2 continues exactly as mode 0 would: every mode multiplies the map spectrum by the
// scaled profile spectrum); 2 starts from it (ks times the map spectrum, then the inverse
// stages) -- no profile sub-pass, no forward transform and no scaling.  0 is the whole pass.
template <typename T, int CW, int L1, int L2, bool STAGE = false, int MODE = 0>
__global__ void __launch_bounds__(256, (sizeof(T) == 4 && L1 <= 10 && L2 <= 10) ? 6 : 0) k_conv_fused2(const C2<T>* __restrict__ Fmap, C2<T>* __restrict__ out,
                                                     long pitch, const C2<T>* __restrict__ Kx, int h, int Ny,
                                                     int N1, const C2<T>* __restrict__ twy, T scale,
                                                     C2<T>* __restrict__ ks) {
  static_assert(MODE >= 0 && MODE <= 2 && (!STAGE || MODE == 0), "P1 modes");
  constexpr int N2 = L1 * L2;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C2<T>* a = reinterpret_cast<C2<T>*>(smem_raw);  // [N2][CW] profile column sub-pass
  C2<T>* y = a;                                   // the transposes reuse it ([L2][L1][CW])
  C2<T>* w1 = y + N2 * CW;                        // W_N1^(n1 kk), n1 < N1
  C2<T>* w2 = w1 + N1;                            // W_Ny^(n kk), n < N2
  C2<T>* wl = w2 + N2;                            // W_N2^m, m < N2
  C2<T>* fs = wl + N2;                            // STAGE: [N2][CW] map-spectrum tile
  const int kk = blockIdx.y;
  const long col0 = (long)blockIdx.x * CW;
  const int c = threadIdx.x % CW, g = threadIdx.x / CW;
  if constexpr (STAGE) {
    static_assert(sizeof(C2<T>) == 16, "staged form: 16-byte elements (FP64, float-float)");
    constexpr int Q = CW;  // one 16-byte copy per element; fs starts at a multiple of 16 bytes
    for (int n = threadIdx.x; n < N2 * Q; n += blockDim.x) {
      const char* src = reinterpret_cast<const char*>(Fmap + ((long)kk * N2 + n / Q) * pitch + col0) + (n % Q) * 16;
      const uint32_t dst = (uint32_t)__cvta_generic_to_shared(reinterpret_cast<char*>(fs + (n / Q) * CW) + (n % Q) * 16);
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
  } else if constexpr (MODE != 1) {
    // the map-spectrum tile (N2 rows of CW values, the only DRAM input) is needed in forward
    // stage 2, after two L2 round trips and four barriers: start pulling it into L2 now
    // (without registers or shared memory, which the other chain's P2 CTAs need); mode 2
    // reads the profile's spectrum tile there as well
    constexpr int LINES = (int)(CW * sizeof(C2<T>) / 128);  // 128-byte lines per strip row
    for (int n = threadIdx.x; n < N2 * LINES; n += blockDim.x) {
      const long e = ((long)kk * N2 + n / LINES) * pitch + col0 + (n % LINES) * (128 / (int)sizeof(C2<T>));
      asm volatile("prefetch.global.L2 [%0];" ::"l"(Fmap + e));
      if constexpr (MODE == 2) asm volatile("prefetch.global.L2 [%0];" ::"l"(ks + e));
    }
  }
  if constexpr (MODE != 2)
    for (int n1 = threadIdx.x; n1 < N1; n1 += blockDim.x) w1[n1] = ldc(twy + ((n1 * kk) % N1) * N2);
  for (int n = threadIdx.x; n < N2; n += blockDim.x) {
    w2[n] = ldc(twy + (long)n * kk);
    wl[n] = ldc(twy + (long)n * N1);
  }
  __syncthreads();
  if constexpr (MODE != 2) {
  // profile: column sub-pass A restricted to its non-zero rows, then twiddle W_Ny^(n2 kk).
  // Thread (g, c) owns the rows n2 = g + G i (G = blockDim / CW); the terms run outer and the
  // elements inner, so the loads of all its elements for one term are in flight together.
  {
    constexpr int G = (L1 > L2 ? L1 : L2), NE = N2 / G;
    static_assert(N2 % G == 0, "rows per thread");
    if (h <= N2) {
      // Profiles of at most 2 N2 rows: kernel rows [0, h) lie in n1 = 0 (weight 1) and rows
      // [Ny - h, Ny) in n1 = N1 - 1 (weight W_N1^((N1-1) kk)), so row n2 sums at most one
      // low term (n2 < h) and one high term (n2 >= N2 - h, compacted row n2 - (N2 - h) + h):
      // the general loop below with its zero terms and its unit weight left out (the same
      // values: multiplying by the table's exact 1 and adding zeros round nothing).
      const C2<T> wh = w1[N1 - 1];
      const C2<T>* kx = Kx + col0 + c;
      const int hb = N2 - h;
#pragma unroll
      for (int i = 0; i < NE; i++) {
        const int n2 = g + G * i;
        C2<T> acc = C2<T>{(T)0, (T)0};
        if (n2 < h) acc = kx[(long)n2 * pitch];
        if (n2 >= hb) acc = cadd(acc, cmul(kx[(long)(n2 - hb + h) * pitch], wh));
        a[n2 * CW + c] = cmul(acc, w2[n2]);
      }
    } else {
      C2<T> acc[NE];
#pragma unroll
      for (int i = 0; i < NE; i++) acc[i] = C2<T>{(T)0, (T)0};
      const int tlo = (h + N2 - 1) / N2;  // low rows: kernel rows n1 N2 + n2 < h
      for (int n1 = 0; n1 < tlo; n1++) {
        const C2<T> w = w1[n1];
#pragma unroll
        for (int i = 0; i < NE; i++) {
          const int n2 = g + G * i, j = n1 * N2 + n2;
          if (j < h) acc[i] = cadd(acc[i], cmul(Kx[(long)j * pitch + col0 + c], w));
        }
      }
      // high rows: kernel rows >= Ny - h, in the last thi values of n1 (increasing)
      const int thi = (h + N2 - 1) / N2 + 1;
      for (int t = 0; t < thi; t++) {
        const int n1 = N1 - thi + t;
        if (n1 < 0) continue;
        const C2<T> w = w1[n1];
#pragma unroll
        for (int i = 0; i < NE; i++) {
          const int n2 = g + G * i;
          const long jr = (long)n1 * N2 + n2;  // kernel row
          if (jr >= (long)Ny - h && jr < Ny && (n1 > 0 || jr >= h))
            acc[i] = cadd(acc[i], cmul(Kx[(jr - (Ny - 2L * h)) * pitch + col0 + c], w));
        }
      }
#pragma unroll
      for (int i = 0; i < NE; i++) {
        const int n2 = g + G * i;
        a[n2 * CW + c] = cmul(acc[i], w2[n2]);
      }
    }
  }
  __syncthreads();
  // forward stage 1: thread (n2 = g, c); every input is read before the shared buffer is
  // overwritten with the transposed result
  {
    C2<T> v[L1];
    if (g < L2) {
#pragma unroll
      for (int n1 = 0; n1 < L1; n1++) v[n1] = a[(L2 * n1 + g) * CW + c];
      Dft<T, L1, false>::run(v);
    }
    __syncthreads();
    if (g < L2) {
#pragma unroll
      for (int k1 = 0; k1 < L1; k1++) y[(g * L1 + k1) * CW + c] = k1 == 0 ? v[0] : cmul(v[k1], wl[g * k1]);
    }
  }
  if constexpr (STAGE) asm volatile("cp.async.wait_all;" ::: "memory");  // this thread's copies
  __syncthreads();
  }  // MODE != 2
  // forward stage 2, product, inverse stage A: thread (k1 = g, c)
  if (g < L1) {
    C2<T> u[L2];
    if constexpr (MODE != 2) {
#pragma unroll
      for (int n2 = 0; n2 < L2; n2++) u[n2] = y[(n2 * L1 + g) * CW + c];
      Dft<T, L2, false>::run(u);
    }
    if constexpr (MODE == 1) {  // the profile's spectrum, frequencies k1 + L1 k2 of row block kk
#pragma unroll
      for (int k2 = 0; k2 < L2; k2++) ks[((long)kk * N2 + g + L1 * k2) * pitch + col0 + c] = cscale(u[k2], scale);
    } else {
#pragma unroll
      for (int k2 = 0; k2 < L2; k2++) {
        const long e = ((long)kk * N2 + g + L1 * k2) * pitch + col0 + c;
        const C2<T> f = STAGE ? fs[(g + L1 * k2) * CW + c] : Fmap[e];
        u[k2] = cmul(f, MODE == 2 ? ks[e] : cscale(u[k2], scale));
      }
      Dft<T, L2, true>::run(u);  // over k2 -> n2
      // the thread rewrites exactly the entries of y it read above: no other thread's data
#pragma unroll
      for (int n2 = 0; n2 < L2; n2++) y[(n2 * L1 + g) * CW + c] = n2 == 0 ? u[0] : cmulc(u[n2], wl[g * n2]);
    }
  }
  if constexpr (MODE == 1) return;  // (every thread: no barrier follows)
  __syncthreads();
  // inverse stage B: thread (n2 = g, c) over k1 -> rows n2 + L2 n1
  if (g < L2) {
    C2<T> v[L1];
#pragma unroll
    for (int k1 = 0; k1 < L1; k1++) v[k1] = y[(g * L1 + k1) * CW + c];
    Dft<T, L1, true>::run(v);
#pragma unroll
    for (int n1 = 0; n1 < L1; n1++) {
      const int n = g + L2 * n1;
      // not renormalised (see fin in mlc_common.cuh)
      out[((long)kk * N2 + n) * pitch + col0 + c] = cmulc(v[n1], w2[n]);
    }
  }
}

// ---------------------------------------------------------------- plain-path helpers

template <typename T>
__global__ void k_wrap_full(const double* __restrict__ prof, int N, int Nx, int Ny, T* __restrict__ out) {
  const int h = N / 2;
  const long total = (long)Nx * Ny;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    const int y = (int)(i / Nx), x = (int)(i % Nx);
    int pr = -1, pc = -1;
    if (y < h) pr = h + y;
    else if (y >= Ny - h) pr = y - (Ny - h);
    if (x < h) pc = h + x;
    else if (x >= Nx - h) pc = x - (Nx - h);
    out[i] = (pr >= 0 && pc >= 0) ? (T)prof[(long)pr * N + pc] : (T)0;
  }
}

// kernel_multiplyFFTs (gpu_functions.cu:571-577): Fk = Fmap * Fk / norm, in place.
template <typename T>
__global__ void k_multiply(const C2<T>* __restrict__ Fmap, C2<T>* __restrict__ Fk, long n, T scale) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    C2<T> m = cmul(Fmap[i], Fk[i]);
    Fk[i] = C2<T>{m.x * scale, m.y * scale};
  }
}

// ---------------------------------------------------------------- host orchestration

template <typename T, typename Loader>
static void launch_rows_r2c(mlc_ctx* ctx, const FftPlan2D& p, const Loader& ld, int nrows, void* out) {
  if (nrows <= 0) return;
  // the profile's 2h rows (P0) timed apart from the map's rows
  const char* name = std::is_same<Loader, ProfileRows<T>>::value ? "fft_profile_rows" : "fft_rows_r2c";
  {
    using K3 = void (*)(Loader, C2<T>*, long, const C2<T>*);
    K3 k3 = nullptr;
    int J = 0;
    // float-float: the five-level kernel of 5000-point rows (the three-level ones would
    // double the float-float units' compile time)
    if constexpr (std::is_same<T, ff>::value) {
      if (p.M == 5000) {
        auto k5 = k_rows_r2c5<Loader>;
        const size_t smem5 = (size_t)(5000 + 625) * sizeof(C2<ff>);
        set_max_smem((const void*)k5, smem5);
        {
          MLC_KSCOPE(ctx, name);
          k5<<<nrows, 512, smem5, ctx->stream>>>(ld, (C2<ff>*)out, p.Wp, (const C2<ff>*)p.twx);
        }
        MLC_CHECK_LAUNCH();
        return;
      }
    } else {
      switch (p.M) {
        case 5000: k3 = k_rows_r2c3<T, 8, 25, 25, Loader>; J = 625; break;
        case 4096: k3 = k_rows_r2c3<T, 16, 16, 16, Loader>; J = 256; break;
        case 2000: k3 = k_rows_r2c3<T, 8, 10, 25, Loader>; J = 250; break;
        case 1000: k3 = k_rows_r2c3<T, 10, 10, 10, Loader>; J = 100; break;
        default: break;
      }
    }
    if (k3) {
      const size_t smem3 = ((size_t)p.M + J) * sizeof(C2<T>);
      set_max_smem((const void*)k3, smem3);
      {
        MLC_KSCOPE(ctx, name);
        k3<<<nrows, 256, smem3, ctx->stream>>>(ld, (C2<T>*)out, p.Wp, (const C2<T>*)p.twx);
      }
      MLC_CHECK_LAUNCH();
      return;
    }
  }
  size_t smem = 2 * (size_t)(p.M + 1) * sizeof(C2<T>);
  auto kern = k_rows_r2c<T, Loader>;
  set_max_smem((const void*)kern, smem);
  {
    MLC_KSCOPE(ctx, name);
    kern<<<nrows, 512, smem, ctx->stream>>>(ld, (C2<T>*)out, p.Wp, p.M, p.rlM, (const C2<T>*)p.twx);
  }
  MLC_CHECK_LAUNCH();
}

template <typename T, typename TO = typename RealOut<T>::type>
static void launch_rows_c2r(mlc_ctx* ctx, const FftPlan2D& p, const void* in, void* out) {
  {
    using K3 = void (*)(const C2<T>*, long, TO*, long, const C2<T>*);
    K3 k3 = nullptr;
    int J = 0;
    switch (p.M) {
      case 5000: k3 = k_rows_c2r3<T, 8, 25, 25, TO>; J = 625; break;
      case 4096: k3 = k_rows_c2r3<T, 16, 16, 16, TO>; J = 256; break;
      case 2000: k3 = k_rows_c2r3<T, 8, 10, 25, TO>; J = 250; break;
      case 1000: k3 = k_rows_c2r3<T, 10, 10, 10, TO>; J = 100; break;
      default: break;
    }
    if (k3) {
      const size_t smem3 = ((size_t)p.M + J) * sizeof(C2<T>);
      set_max_smem((const void*)k3, smem3);
      {
        MLC_KSCOPE(ctx, "fft_rows_c2r");
        k3<<<p.Ny, 256, smem3, ctx->stream>>>((const C2<T>*)in, p.Wp, (TO*)out, p.Nx, (const C2<T>*)p.twx);
      }
      MLC_CHECK_LAUNCH();
      return;
    }
  }
  size_t smem = 2 * (size_t)(p.M + 1) * sizeof(C2<T>);
  auto kern = k_rows_c2r<T, TO>;
  set_max_smem((const void*)kern, smem);
  {
    MLC_KSCOPE(ctx, "fft_rows_c2r");
    kern<<<p.Ny, 512, smem, ctx->stream>>>((const C2<T>*)in, p.Wp, (TO*)out, p.Nx, p.M, p.rlM,
                                         (const C2<T>*)p.twx);
  }
  MLC_CHECK_LAUNCH();
}

// Columns per CTA of the column passes: 128 bytes of complex values for FP32 and FP64;
// float-float (16-byte values) takes 16 columns, as FP32 does, so that its arithmetic-bound
// CTAs are whole warps (10 x 16 = 160 threads for a 10 x 10 pass, where 8 columns left the
// third of 80 threads' warps half empty).
template <typename T>
constexpr int strip_width() {
  return (sizeof(T) == 8 && !std::is_same<T, ff>::value) ? 8 : 16;
}

// kind 'A': row sets {n2 + N2*j}, length N1; kind 'B': row blocks {k1*N2 + j}, length N2.
template <typename T, bool INV>
static void launch_colpass(mlc_ctx* ctx, const FftPlan2D& p, void* buf, char kind, int post_tw) {
  constexpr int CW = strip_width<T>();
  const int nstrips = ceil_div(p.Wc, CW);
  int L, nsets, tw_stride;
  long set_mul, j_mul;
  RadixList rl;
  if (kind == 'A') {
    L = p.N1; nsets = p.N2; set_mul = 1; j_mul = p.N2; tw_stride = p.N2; rl = p.rlN1;
  } else {
    L = p.N2; nsets = p.N1; set_mul = p.N2; j_mul = 1; tw_stride = p.N1; rl = p.rlN2;
  }
  if (L == 1 && !post_tw) return;
  // two-level register kernels for the lengths that split into two supported factors
  using K2 = void (*)(C2<T>*, long, long, long, const C2<T>*, int, int);
  K2 k2 = nullptr;
  int nthr = 0;
  switch (L) {
    case 100: k2 = k_colpass2<T, CW, 10, 10, INV>; nthr = 10 * CW; break;
    case 128: k2 = k_colpass2<T, CW, 8, 16, INV>; nthr = 16 * CW; break;
    case 64: k2 = k_colpass2<T, CW, 8, 8, INV>; nthr = 8 * CW; break;
    case 80: k2 = k_colpass2<T, CW, 8, 10, INV>; nthr = 10 * CW; break;
    case 50: k2 = k_colpass2<T, CW, 5, 10, INV>; nthr = 10 * CW; break;
    case 40: k2 = k_colpass2<T, CW, 5, 8, INV>; nthr = 8 * CW; break;
    default: break;
  }
  if (k2) {
    dim3 grid(nstrips, nsets);
    {
      MLC_KSCOPE(ctx, kind == 'A' ? "fft_col_A" : "fft_col_B");
      k2<<<grid, nthr, 0, ctx->stream>>>((C2<T>*)buf, p.Wp, set_mul, j_mul, (const C2<T>*)p.twy, tw_stride, post_tw);
    }
    MLC_CHECK_LAUNCH();
    return;
  }
  size_t smem = (2 * (size_t)L * CW + rl.tlen + L) * sizeof(C2<T>);
  auto kern = k_colpass<T, CW, INV>;
  set_max_smem((const void*)kern, smem);
  dim3 grid(nstrips, nsets);
  {
    MLC_KSCOPE(ctx, kind == 'A' ? "fft_col_A" : "fft_col_B");
    kern<<<grid, 256, smem, ctx->stream>>>((C2<T>*)buf, p.Wp, L, set_mul, j_mul, rl, (const C2<T>*)p.twy,
                                         tw_stride, post_tw);
  }
  MLC_CHECK_LAUNCH();
}

// ---------------------------------------------------------------- entry templates

template <typename T>
void forward_impl(mlc_ctx* ctx, const FftPlan2D& p, const void* in, int in_dtype, void* spec) {
  if (in_dtype == MLC_F64)
    launch_rows_r2c<T>(ctx, p, RealRows<T, double>{(const double*)in, p.Nx}, p.Ny, spec);
  else
    launch_rows_r2c<T>(ctx, p, RealRows<T, float>{(const float*)in, p.Nx}, p.Ny, spec);
  launch_colpass<T, false>(ctx, p, spec, 'A', 1);
  launch_colpass<T, false>(ctx, p, spec, 'B', 0);
}

// spec_out: stop after P2 and leave the inverse half-spectrum there (pitch Wp) instead of
// running P3 into out.
template <typename T>
void conv_fused_impl(mlc_ctx* ctx, const FftPlan2D& p, const void* Fmap, const double* prof, int pN,
                     void* out, void* spec_out, int kx_slot) {
  constexpr int CW = strip_width<T>();
  const int h = pN / 2;
  MLC_REQUIRE(pN % 2 == 0 && 2 * h <= p.Ny && 2 * h <= p.Nx, MLC_ERR_LIMIT,
              "profile raster larger than the map");
  void* kx = ws_get(ctx, kx_slot, (size_t)(2 * h > 0 ? 2 * h : 1) * p.Wp * sizeof(C2<T>));
  void* tmp = spec_out ? spec_out : ws_get(ctx, WS_SPEC_TMP, p.spec_bytes());
  launch_rows_r2c<T>(ctx, p, ProfileRows<T>{prof, pN, h, p.Nx}, 2 * h, kx);
  const int nstrips = ceil_div(p.Wc, CW);
  const T scale = (T)(1.0 / ((double)p.Nx * (double)p.Ny));
  {
    // two-level register kernel where N2 splits into two supported factors
    using K2 = void (*)(const C2<T>*, C2<T>*, long, const C2<T>*, int, int, int, const C2<T>*, T, C2<T>*);
    K2 k2 = nullptr;
    int nthr = 0;
    // float-float and FP64 at N2 = 100: the map-spectrum tile prefetched into L2, or staged in
    // shared memory (chosen per map size by the autotuner, or pinned with mlc_ctx_tune_set)
    K2 k2s = nullptr;
    if constexpr (sizeof(C2<T>) == 16)
      if (p.N2 == 100) k2s = k_conv_fused2<T, CW, 10, 10, true>;
    switch (p.N2) {
      case 100: k2 = k_conv_fused2<T, CW, 10, 10>; nthr = 10 * CW; break;
      case 128: k2 = k_conv_fused2<T, CW, 8, 16>; nthr = 16 * CW; break;
      case 64: k2 = k_conv_fused2<T, CW, 8, 8>; nthr = 8 * CW; break;
      case 80: k2 = k_conv_fused2<T, CW, 8, 10>; nthr = 10 * CW; break;
      case 50: k2 = k_conv_fused2<T, CW, 5, 10>; nthr = 10 * CW; break;
      case 40: k2 = k_conv_fused2<T, CW, 5, 8>; nthr = 8 * CW; break;
      default: break;
    }
    if (k2) {
      const size_t smem2 = ((size_t)p.N2 * CW + p.N1 + 2 * (size_t)p.N2) * sizeof(C2<T>);
      const size_t smem2s = smem2 + (size_t)p.N2 * CW * sizeof(C2<T>);
      auto launch = [&](bool staged) {
        const K2 k = staged ? k2s : k2;
        const size_t sm = staged ? smem2s : smem2;
        set_max_smem((const void*)k, sm);
        k<<<dim3(nstrips, p.N1), nthr, sm, ctx->stream>>>((const C2<T>*)Fmap, (C2<T>*)tmp, p.Wp, (const C2<T>*)kx,
                                                          h, p.Ny, p.N1, (const C2<T>*)p.twy, scale, nullptr);
      };
      const bool staged = k2s && p1_staged_choice(ctx, p, [&](bool st) {
                            launch(st);
                            MLC_CHECK_LAUNCH();
                          });
      {
        MLC_KSCOPE(ctx, "conv_fused_spectrum");
        launch(staged);
      }
      MLC_CHECK_LAUNCH();
      launch_colpass<T, true>(ctx, p, tmp, 'A', 0);
      if (!spec_out) launch_rows_c2r<T>(ctx, p, tmp, out);
      return;
    }
  }
  size_t smem = (2 * (size_t)p.N2 * CW + p.N1 + p.N2 + p.rlN2.tlen) * sizeof(C2<T>);
  auto kern = k_conv_fused<T, CW>;
  set_max_smem((const void*)kern, smem);
  dim3 grid(nstrips, p.N1);
  {
    MLC_KSCOPE(ctx, "conv_fused_spectrum");
    kern<<<grid, 256, smem, ctx->stream>>>((const C2<T>*)Fmap, (C2<T>*)tmp, p.Wp, (const C2<T>*)kx, h, p.Ny,
                                         p.N1, p.N2, p.rlN2, (const C2<T>*)p.twy, scale);
  }
  MLC_CHECK_LAUNCH();
  launch_colpass<T, true>(ctx, p, tmp, 'A', 0);
  if (!spec_out) launch_rows_c2r<T>(ctx, p, tmp, out);
}

// P1's register kernel in mode MODE for the plan's N2 (nullptr where there is none): the
// sizes whose profile spectra are cached (N2 = 100: 2000^2 ... 10000^2; 128: 8192^2 and
// the other multiples of 128).
template <typename T, int MODE>
static auto p1_mode_kernel(int N2, int& nthr) {
  constexpr int CW = strip_width<T>();
  using K = void (*)(const C2<T>*, C2<T>*, long, const C2<T>*, int, int, int, const C2<T>*, T, C2<T>*);
  K k = nullptr;
  switch (N2) {
    case 100: k = k_conv_fused2<T, CW, 10, 10, false, MODE>; nthr = 10 * CW; break;
    case 128: k = k_conv_fused2<T, CW, 8, 16, false, MODE>; nthr = 16 * CW; break;
    default: break;
  }
  return k;
}

template <typename T>
bool profile_spectrum_supported_impl(const FftPlan2D& p) {
  int nthr = 0;
  return p1_mode_kernel<T, 1>(p.N2, nthr) != nullptr;
}

// The profile's spectrum as P1 holds it before the product (P0, then P1 up to forward
// stage 2), in the map spectrum's layout (Ny x Wp) into ks.
template <typename T>
void profile_spectrum_impl(mlc_ctx* ctx, const FftPlan2D& p, const double* prof, int pN, void* ks) {
  constexpr int CW = strip_width<T>();
  const int h = pN / 2;
  MLC_REQUIRE(pN % 2 == 0 && 2 * h <= p.Ny && 2 * h <= p.Nx, MLC_ERR_LIMIT, "profile raster larger than the map");
  int nthr = 0;
  const auto k = p1_mode_kernel<T, 1>(p.N2, nthr);
  MLC_REQUIRE(k != nullptr, MLC_ERR_LIMIT, "no cached profile spectra for this map size");
  void* kx = ws_get(ctx, WS_KX, (size_t)(2 * h > 0 ? 2 * h : 1) * p.Wp * sizeof(C2<T>));
  launch_rows_r2c<T>(ctx, p, ProfileRows<T>{prof, pN, h, p.Nx}, 2 * h, kx);
  const size_t smem = ((size_t)p.N2 * CW + p.N1 + 2 * (size_t)p.N2) * sizeof(C2<T>);
  set_max_smem((const void*)k, smem);
  const T scale = (T)(1.0 / ((double)p.Nx * (double)p.Ny));  // stored with the spectrum
  {
    MLC_KSCOPE(ctx, "conv_profile_spectrum");
    k<<<dim3(ceil_div(p.Wc, CW), p.N1), nthr, smem, ctx->stream>>>(nullptr, nullptr, p.Wp, (const C2<T>*)kx, h,
                                                                     p.Ny, p.N1, (const C2<T>*)p.twy, scale,
                                                                     (C2<T>*)ks);
  }
  MLC_CHECK_LAUNCH();
}

// conv_fused_impl up to P2 (the inverse half-spectrum into spec_out) from a profile
// spectrum made by profile_spectrum_impl: P1 is the product and the inverse stages only.
// The same operations on the same values as the whole pass, so the same results bit for bit.
template <typename T>
void conv_cached_impl(mlc_ctx* ctx, const FftPlan2D& p, const void* Fmap, const void* ks, void* spec_out) {
  constexpr int CW = strip_width<T>();
  int nthr = 0;
  const auto k = p1_mode_kernel<T, 2>(p.N2, nthr);
  MLC_REQUIRE(k != nullptr, MLC_ERR_LIMIT, "no cached profile spectra for this map size");
  const T scale = (T)(1.0 / ((double)p.Nx * (double)p.Ny));
  const size_t smem = ((size_t)p.N2 * CW + p.N1 + 2 * (size_t)p.N2) * sizeof(C2<T>);
  set_max_smem((const void*)k, smem);
  {
    MLC_KSCOPE(ctx, "conv_cached_spectrum");
    k<<<dim3(ceil_div(p.Wc, CW), p.N1), nthr, smem, ctx->stream>>>((const C2<T>*)Fmap, (C2<T>*)spec_out, p.Wp,
                                                                     nullptr, 0, p.Ny, p.N1, (const C2<T>*)p.twy,
                                                                     scale, (C2<T>*)ks);
  }
  MLC_CHECK_LAUNCH();
  launch_colpass<T, true>(ctx, p, spec_out, 'A', 0);
}

// The whole cached convolution into real pixels of T (P3 after conv_cached_impl).
template <typename T>
void conv_cached_real_impl(mlc_ctx* ctx, const FftPlan2D& p, const void* Fmap, const void* ks, void* out) {
  void* tmp = ws_get(ctx, WS_SPEC_TMP, p.spec_bytes());
  conv_cached_impl<T>(ctx, p, Fmap, ks, tmp);
  launch_rows_c2r<T>(ctx, p, tmp, out);
}

template <typename T>
void conv_plain_impl(mlc_ctx* ctx, const FftPlan2D& p, const void* Fmap, const double* prof, int pN,
                     void* out) {
  MLC_REQUIRE(pN % 2 == 0 && pN <= p.Ny && pN <= p.Nx, MLC_ERR_LIMIT, "profile raster larger than the map");
  void* kreal = ws_get(ctx, WS_KREAL, (size_t)p.Nx * p.Ny * sizeof(T));
  void* kspec = ws_get(ctx, WS_KSPEC, p.spec_bytes());
  const long total = (long)p.Nx * p.Ny;
  int grid = (int)std::min<long>((total + 255) / 256, (long)ctx->sm_count * 16);
  {
    MLC_KSCOPE(ctx, "conv_plain_wrap");
    k_wrap_full<T><<<grid, 256, 0, ctx->stream>>>(prof, pN, p.Nx, p.Ny, (T*)kreal);
  }
  MLC_CHECK_LAUNCH();
  forward_impl<T>(ctx, p, kreal, sizeof(T) == 8 ? MLC_F64 : MLC_F32, kspec);
  const long n = (long)p.Ny * p.Wp;
  const T scale = (T)(1.0 / ((double)p.Nx * (double)p.Ny));
  grid = (int)std::min<long>((n + 255) / 256, (long)ctx->sm_count * 16);
  {
    MLC_KSCOPE(ctx, "conv_plain_multiply");
    k_multiply<T><<<grid, 256, 0, ctx->stream>>>((const C2<T>*)Fmap, (C2<T>*)kspec, n, scale);
  }
  MLC_CHECK_LAUNCH();
  launch_colpass<T, true>(ctx, p, kspec, 'B', 1);
  launch_colpass<T, true>(ctx, p, kspec, 'A', 0);
  launch_rows_c2r<T>(ctx, p, kspec, out);
}

// P3 alone: the inverse real row transform of a half-spectrum into a real map of TO.
template <typename T, typename TO>
void rows_c2r_impl(mlc_ctx* ctx, const FftPlan2D& p, const void* spec, void* out) {
  launch_rows_c2r<T, TO>(ctx, p, spec, out);
}

template <typename T, typename TO>
bool c2r_interleave_impl(mlc_ctx* ctx, const FftPlan2D& p, const void* specs, long spec_stride, int nm, int S,
                         void* out, unsigned planar) {
  using K = void (*)(const C2<T>*, long, long, int, TO*, int, const C2<T>*, unsigned);
  K k = nullptr;
  int J = 0, nthr = 256;
  switch (p.M) {
    case 5000:
      if constexpr (std::is_same<T, ff>::value) {
        k = k_rows_c2r5_il<T, TO>;
        nthr = 512;
      } else {
        k = k_rows_c2r3_il<T, 8, 25, 25, TO>;
      }
      J = 625;
      break;
    case 4096: k = k_rows_c2r3_il<T, 16, 16, 16, TO>; J = 256; break;
    case 2000: k = k_rows_c2r3_il<T, 8, 10, 25, TO>; J = 250; break;
    case 1000: k = k_rows_c2r3_il<T, 10, 10, 10, TO>; J = 100; break;
    default: return false;
  }
  if (!rows_c2r_interleave_supported(p)) return false;
  const size_t smem = ((size_t)p.M + J) * sizeof(C2<T>);
  set_max_smem((const void*)k, smem);
  const int quads = (nm + 3) / 4;
  {
    MLC_KSCOPE(ctx, "fft_rows_c2r_interleave");
    k<<<dim3(4 * quads, p.Ny), nthr, smem, ctx->stream>>>((const C2<T>*)specs, spec_stride, p.Wp, nm, (TO*)out, S,
                                                           (const C2<T>*)p.twx, planar);
  }
  MLC_CHECK_LAUNCH();
  return true;
}

}  // namespace mlc
