// Tensor-core form of the pairwise magnitude-difference chi2 (see pairdiff.cu for the
// statistic).  chi2_ij = |Q_j - P_i|^2 on quantised curves P_i = 2^ei p_i, Q_j = 2^ej q_j
// (p, q integers, |p|,|q| <= 8355711, one power-of-two step per curve) held as three signed
// 8-bit slices p = 65536 s0 + 256 s1 + s2 in bf16.  A slice product summed over T <= 128
// epochs stays below 2^24, so every FP32 tensor-core accumulation is exact; the cross term
// is accumulated per diagonal d = a + b of slice exponents (five TMEM accumulators
// d = 0..4, all nine slice pairs), so
//     x = p.q = 2^32 X0 + 2^24 X1 + 2^16 X2 + 2^8 X3 + X4   exactly,
// and chi2 = |P|^2 + |Q|^2 - 2^(ei+ej+1) x is formed from the per-curve norms (natural
// units, float-float) and the exactly scaled accumulators: in FP32 summed from the largest
// term down (within 4e-6 relative) where chi2 >= 2^-14 (|P|^2+|Q|^2), in float-float
// arithmetic below that.  Top-k
// candidates, pairs whose chi2 is below 1e-7 of |P|^2 + |Q|^2 (where the float-float
// rounding could matter) and, with a matrix requested, every pair whose quantisation error
// could exceed 1e-6 relative are recomputed in FP64 by k_pd_refine.
//
// Kernel layout (one persistent CTA per SM, 4 + 12..24 warps):
//   warp 0      TMA producer: the work item's 128 A rows (3 slices x Kp, resident in shared
//               memory) and, double-buffered, each 48-row B tile
//   warp 1      MMA issuer (one thread): 9 slice pairs x Kp/16 tcgen05.mma per tile into one
//               of two TMEM buffers (5 accumulators x 48 columns each; buffers at columns
//               0 and 256 of the 512 allocated)
//   warp 2      TMEM allocation / release
//   warps 4..    epilogue (12, 16 or 24 warps, the same number per TMEM lane quadrant; the
//               autotuner picks the count): TMEM ->
//               registers, chi2 assembly, log10-chi2 histogram in shared memory, top-k
//               candidates below a threshold, refinement list, optional matrix
// Every barrier wait is bounded; a timeout sets the error flag and all roles unwind.
#include <cuda.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "pairdiff.h"
#include "tc_ptx.cuh"

namespace mlc {

void radix_sort_u64_u32(mlc_ctx* ctx, long n, uint64_t* keys, uint32_t* vals);
uint64_t f64_to_key(double d);

namespace {

constexpr int TM = PD_TILE_M, TN = PD_TILE_N;
constexpr int NSTAGE = 2;
// Epilogue shapes: EPIW warps (a multiple of 4: the same number per TMEM lane quadrant, one
// per SM sub-partition each), each taking WCOLS of the 48 tile columns, CCH per TMEM load.
// 12 warps: 16 columns (loads of 8); 16: 12 (loads of 4); 24: 8 (one load of 8).
template <int EPIW>
struct Epi {
  static constexpr int warps = EPIW;
  static constexpr int per_q = EPIW / 4;
  static constexpr int wcols = TN / per_q;
  static constexpr int cch = wcols % 8 == 0 ? 8 : 4;
  static constexpr int threads = (4 + EPIW) * 32;
  static_assert(EPIW % 4 == 0 && wcols * per_q == TN && wcols % cch == 0 && wcols <= 16, "epilogue column split");
};
constexpr int MAX_EPIW = 24;
constexpr int EPI_CHOICES[] = {12, 16, 24};
constexpr int TMEM_COLS = 512;
constexpr int MAX_KP = 128;
constexpr int MAX_BINS = 4096;
constexpr int A_BOX = TM * 128;  // bytes of one 64-element K box of A (128 rows x 128 B)
constexpr int B_BOX = TN * 128;  // 6144 B: a multiple of the 1024-B swizzle atom
constexpr int NACC = 5;
constexpr int TBUF = 256;        // TMEM column stride between the two accumulator buffers
static_assert(NACC * TN <= TBUF && B_BOX % 1024 == 0, "TMEM / smem layout");

struct PdParams {
  int NA, NB, nj, njc, jchunk, nitems, nkb;
  const float2* alpha_ff;
  const float2* beta_ff;
  const int* ea;
  const int* eb;
  int nbins;
  float hscale, hoff;  // bin = floor(log2(chi2) * hscale + hoff)
  unsigned long long* hist;
  float thr;
  unsigned int cap;
  unsigned int* ncand;
  float* cval;
  int* ci;
  int* cj;
  float refine_f;  // matrix mode: quantisation bound factor
  unsigned int rcap;
  unsigned int* nref;
  int* ri;
  int* rj;
  float* out;
  int* err;
};

size_t smem_bytes(int nkb, int nbins) {
  return 1024 + (size_t)3 * nkb * A_BOX + (size_t)NSTAGE * 3 * nkb * B_BOX + 16 * 8 + 16 +
         sizeof(uint32_t) * ((nbins + 2 + 3) & ~3) + (size_t)MAX_EPIW * 16 * sizeof(float4);
}

// 2^k for k in [-126, 127]; 0 below (the terms it scales are then negligible)
__device__ __forceinline__ float pow2f(int k) { return k < -126 ? 0.f : __int_as_float((k + 127) << 23); }

// Error-free sum s + e = a + b.
__device__ __forceinline__ float two_sum(float a, float b, float& e) {
  const float s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
  return s;
}

// chi2 = A + B - (u0 + ... + u4): A, B float-float, u_k exact floats (scaled
// accumulators); the large, cancelling terms go through error-free two-sums.
__device__ __forceinline__ float chi2_assemble(float2 A, float2 B, float u0, float u1, float u2, float u3,
                                               float u4) {
  float e1, e2, e3;
  const float s = two_sum(A.x, B.x, e1);
  const float t = two_sum(s, -u0, e2);
  const float t2 = two_sum(t, -u1, e3);
  return t2 + (((e1 + e2) + e3) + ((A.y + B.y) - ((u2 + u3) + u4)));
}

template <int EPIW>
__device__ __forceinline__ void epi_sync() {
  asm volatile("bar.sync 1, %0;" ::"r"(EPIW * 32) : "memory");
}

// NKB: 64-element K boxes per slice (Kp / 64); OUT: chi2 matrix written; EPIW: epilogue warps
template <int NKB, bool OUT, int EPIW>
__global__ void __launch_bounds__(Epi<EPIW>::threads, 1) k_pairdiff_tc(const __grid_constant__ CUtensorMap tmA,
                                                                        const __grid_constant__ CUtensorMap tmB,
                                                                        PdParams P) {
  constexpr int EPI_WARPS = EPIW, WCOLS = Epi<EPIW>::wcols, CCH = Epi<EPIW>::cch, NTHREADS = Epi<EPIW>::threads;
  extern __shared__ unsigned char smem_raw[];
  unsigned char* sm = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  constexpr int nkb = NKB;
  unsigned char* A_s = sm;
  unsigned char* B_s = A_s + 3 * nkb * A_BOX;
  uint64_t* bars = (uint64_t*)(B_s + NSTAGE * 3 * nkb * B_BOX);
  uint64_t* a_full = bars + 0;
  uint64_t* a_empty = bars + 1;
  uint64_t* b_full = bars + 2;   // [2]
  uint64_t* b_empty = bars + 4;  // [2]
  uint64_t* t_full = bars + 6;   // [2]
  uint64_t* t_empty = bars + 8;  // [2]
  uint32_t* tmem_slot = (uint32_t*)(bars + 16);
  volatile int* abort_s = (volatile int*)(tmem_slot + 1);
  uint32_t* hist_s = tmem_slot + 4;
  // counters: below lo, the nbins bins, at or above hi (flushed to the global layout: bins, below, above)
  float4* colv = (float4*)(hist_s + ((P.nbins + 2 + 3) & ~3));  // [EPIW][16] column constants
  const uint32_t hist_sa = tc::smem_u32(hist_s);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    tc::mbar_init(a_full, 1);
    tc::mbar_init(a_empty, 1);
    for (int s = 0; s < 2; s++) {
      tc::mbar_init(b_full + s, 1);
      tc::mbar_init(b_empty + s, 1);
      tc::mbar_init(t_full + s, 1);
      tc::mbar_init(t_empty + s, EPI_WARPS);
    }
    *abort_s = 0;
    tc::fence_barrier_init();
  }
  for (int i = threadIdx.x; i < P.nbins + 2; i += NTHREADS) hist_s[i] = 0;
  if (warp == 2) tc::tmem_alloc(tmem_slot, TMEM_COLS);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tmem_slot;

  auto fail = [&]() {
    *abort_s = 1;
    atomicExch(P.err, 1);
  };

  if (warp == 0 && lane == 0) {
    // ------------------------------------------------ TMA producer
    tc::prefetch_tmap(&tmA);
    tc::prefetch_tmap(&tmB);
    uint32_t cB = 0, n = 0;
    for (int it = blockIdx.x; it < P.nitems && !*abort_s; it += gridDim.x, n++) {
      const int itile = it / P.njc, jc = it % P.njc;
      const int j0 = jc * P.jchunk, j1 = min(P.nj, j0 + P.jchunk);
      if (!tc::mbar_wait(a_empty, (n & 1) ^ 1)) { fail(); break; }
      tc::mbar_arrive_expect_tx(a_full, 3 * nkb * A_BOX);
      for (int bx = 0; bx < 3 * nkb; bx++) tc::tma_load_2d(A_s + bx * A_BOX, &tmA, a_full, bx * 64, itile * TM);
      for (int jt = j0; jt < j1; jt++, cB++) {
        const uint32_t s = cB & 1, u = cB >> 1;
        if (*abort_s || !tc::mbar_wait(b_empty + s, (u & 1) ^ 1)) { fail(); break; }
        tc::mbar_arrive_expect_tx(b_full + s, 3 * nkb * B_BOX);
        for (int bx = 0; bx < 3 * nkb; bx++)
          tc::tma_load_2d(B_s + (s * 3 * nkb + bx) * B_BOX, &tmB, b_full + s, bx * 64, jt * TN);
      }
    }
  } else if (warp == 1 && lane == 0) {
    // ------------------------------------------------ MMA issuer
    const uint32_t idesc = tc::idesc_bf16(TM, TN);
    uint32_t cB = 0, ct = 0, n = 0;
    // Descriptors of the box starts: the start-address field holds (address >> 4) in its low
    // 14 bits and shared-memory addresses stay below 2^18, so a descriptor for
    // base + offset is the base descriptor plus offset >> 4 (no carry).
    const uint64_t dA = tc::desc_sw128(tc::smem_u32(A_s));
    const uint64_t dB0 = tc::desc_sw128(tc::smem_u32(B_s)), dB1 = tc::desc_sw128(tc::smem_u32(B_s + 3 * nkb * B_BOX));
    for (int it = blockIdx.x; it < P.nitems && !*abort_s; it += gridDim.x, n++) {
      const int jc = it % P.njc;
      const int j0 = jc * P.jchunk, j1 = min(P.nj, j0 + P.jchunk);
      if (!tc::mbar_wait(a_full, n & 1)) { fail(); break; }
      for (int jt = j0; jt < j1; jt++, cB++, ct++) {
        const uint32_t s = cB & 1, u = cB >> 1, tb = ct & 1, tu = ct >> 1;
        if (*abort_s || !tc::mbar_wait(b_full + s, u & 1) || !tc::mbar_wait(t_empty + tb, (tu & 1) ^ 1)) {
          fail();
          break;
        }
        tc::fence_after_sync();
        const uint32_t dbase = tmem + tb * TBUF;
        const uint64_t dBs = s ? dB1 : dB0;
        // slice pairs ordered so that each accumulator's first MMA clears it
#pragma unroll
        for (int a = 0; a < 3; a++)
#pragma unroll
          for (int b = 0; b < 3; b++) {
            const int d = a + b;
            const bool first_of_d = (a == 0) || (b == 2);  // (0,b) opens d <= 2; (a,2) opens d = 3, 4
#pragma unroll
            for (int kk = 0; kk < nkb * 4; kk++) {
              const int kb = kk >> 2, ko = (kk & 3) * 32;
              const uint64_t ad = dA + (uint64_t)((((a * nkb + kb) * A_BOX) + ko) >> 4);
              const uint64_t bd = dBs + (uint64_t)((((b * nkb + kb) * B_BOX) + ko) >> 4);
              tc::mma_bf16(dbase + d * TN, ad, bd, idesc, (first_of_d && kk == 0) ? 0u : 1u);
            }
          }
        tc::mma_commit(b_empty + s);
        tc::mma_commit(t_full + tb);
      }
      tc::mma_commit(a_empty);
    }
  } else if (warp >= 4) {
    // ------------------------------------------------ epilogue
    const int q = warp & 3, h = (warp - 4) >> 2;  // lane quadrant, column group
    const uint32_t lane_addr = (uint32_t)(32 * q) << 16;
    // Every epilogue warp walks the same items and reaches the two named-barrier syncs per
    // item the same number of times; after an abort it only skips the work.
    uint32_t ct = 0;
    for (int it = blockIdx.x; it < P.nitems; it += gridDim.x) {
      const int itile = it / P.njc, jc = it % P.njc;
      const int j0 = jc * P.jchunk, j1 = min(P.nj, j0 + P.jchunk);
      const int i = itile * TM + 32 * q + lane;
      const bool irow = i < P.NA;
      const float2 aff = irow ? P.alpha_ff[i] : make_float2(0.f, 0.f);
      const int ei = irow ? P.ea[i] : PD_EMIN;
      const float pa = pow2f(ei);  // 2^ei
      float4* cv = colv + (warp - 4) * 16;
      // this warp's WCOLS columns h*WCOLS + c of a tile: (beta_ff, 2^(ej+33)) fetched one tile ahead
      // (the loads run while the previous tile is processed), staged in shared memory and read
      // back as one broadcast load per element
      float2 nb = make_float2(0.f, 0.f);
      int ne = PD_EMIN;
      auto fetch = [&](int jt) {
        const int jl = jt * TN + h * WCOLS + lane;
        const bool lok = lane < WCOLS && jt < j1 && jl < P.NB;
        nb = lok ? __ldg(P.beta_ff + jl) : make_float2(0.f, 0.f);
        ne = lok ? __ldg(P.eb + jl) : PD_EMIN;
      };
      fetch(j0);
      for (int jt = j0; jt < j1; jt++, ct++) {
        const uint32_t tb = ct & 1, tu = ct >> 1;
        if (*abort_s) break;
        // (the previous tile's reads of cv ended at the __syncwarp closing it)
        if (lane < WCOLS) cv[lane] = make_float4(nb.x, nb.y, pow2f(ne + 33), 0.f);  // 2 x 2^(ei+ej) x 2^32 with pa
        fetch(jt + 1);
        __syncwarp();
        if (!tc::mbar_wait(t_full + tb, tu & 1)) {
          fail();
          break;
        }
        tc::fence_after_sync();
        // full tiles (every row and column real) skip the per-element range tests
        const bool fast = irow && (jt + 1) * TN <= P.NB;
        for (int ch = 0; ch < WCOLS / CCH; ch++) {
          const int col0 = h * WCOLS + ch * CCH;
          uint32_t r0[CCH], r1[CCH], r2[CCH], r3[CCH], r4[CCH];
          const uint32_t ta = tmem + tb * TBUF + lane_addr + col0;
          tc::tmem_ld<CCH>(ta, r0);
          tc::tmem_ld<CCH>(ta + TN, r1);
          tc::tmem_ld<CCH>(ta + 2 * TN, r2);
          tc::tmem_ld<CCH>(ta + 3 * TN, r3);
          tc::tmem_ld<CCH>(ta + 4 * TN, r4);
          tc::tmem_wait_ld();
#pragma unroll
          for (int c = 0; c < CCH; c++) {
            const int j = jt * TN + col0 + c;
            if (!fast && (!irow || j >= P.NB)) continue;
            const float4 b = cv[ch * CCH + c];
            // 2 x 2^(ei+ej) = sum_d 2^(ei+ej+33-8d) X_d; s0 = 2^(ei+ej+33) is an exact product
            const float s0 = pa * b.z;
            const float X0 = __uint_as_float(r0[c]), X1 = __uint_as_float(r1[c]);
            const float X2 = __uint_as_float(r2[c]), X3 = __uint_as_float(r3[c]);
            // FP32 assembly from the largest term down: ab + e = |P|^2 + |Q|^2 (high parts)
            // exactly; s0 X0 is exact (integer < 2^24 times a power of two), so ab - s0 X0 is
            // rounded once, relative to itself, then the X1 term, then the small rest.  Error
            // about 3 2^-24 chi2 + 2^-32 (|P|^2+|Q|^2) (the left-out X4 term below 2^-30 of it):
            // within 4e-6 of chi2 whenever chi2 >= 2^-14 (|P|^2+|Q|^2)
            float e;
            const float ab = two_sum(aff.x, b.x, e);
            const float t1 = fmaf(-X0, s0, ab);
            const float t2 = fmaf(-X1, s0 * 0x1p-8f, t1);
            const float w = fmaf(X3, 0x1p-8f, X2);
            float chi2 = t2 + fmaf(-w, s0 * 0x1p-16f, e + (aff.y + b.y));
            // One test for the rare cases: lim is at least every bound below, so a value at or
            // above it needs neither the float-float form nor the exact list.
            float lim = fmaxf(0x1p-14f * ab, P.thr);
            float qbound = 0.f;
            if constexpr (OUT) {
              const float q = pa + b.z * 0x1p-33f;
              qbound = P.refine_f * q * q;
              lim = fmaxf(lim, qbound);
            }
            if (chi2 < lim) {
              // below 2^-14 (|P|^2+|Q|^2) the float-float form: with this assembly almost no
              // warp enters it (the earlier form, good to (|P|^2+|Q|^2)/16, sent some lane of
              // most warps there)
              if (chi2 < 0x1p-14f * ab)
                chi2 = chi2_assemble(aff, make_float2(b.x, b.y), X0 * s0, X1 * (s0 * 0x1p-8f), X2 * (s0 * 0x1p-16f),
                                     X3 * (s0 * 0x1p-24f), __uint_as_float(r4[c]) * (s0 * 0x1p-32f));
              // below 1e-7 (|P|^2+|Q|^2) the float-float rounding (about 2^-40 of it) could
              // exceed 1e-5 relative; those, the top-k candidates and (matrix mode) pairs within
              // the quantisation-error bound go to the exact FP64 list (which also histograms
              // them)
              const float bound = fmaxf(fmaxf(1e-7f * ab, P.thr), qbound);
              if (chi2 < bound) {
                const unsigned k = atomicAdd(P.nref, 1u);
                if (k < P.rcap) {
                  P.ri[k] = i;
                  P.rj[k] = j;
                }
                continue;
              }
            }
            if constexpr (OUT) P.out[(long)i * P.NB + j] = chi2;
            // chi2 >= 1e-7 (|P|^2+|Q|^2) > 0 here; a subnormal one (flat curves) falls out of range
            float lg;
            asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(lg) : "f"(chi2));
            const int bin = __float2int_rd(fmaf(lg, P.hscale, P.hoff));
            // shared counters: [below lo, bins 0 .. nbins-1, at or above hi]
            const uint32_t slot = (uint32_t)(min(max(bin, -1), P.nbins) + 1);
            asm volatile("red.shared.add.u32 [%0], 1;" ::"r"(hist_sa + 4u * slot) : "memory");
          }
        }
        tc::fence_before_sync();
        __syncwarp();
        if (lane == 0) tc::mbar_arrive(t_empty + tb);
      }
      // flush this item's histogram (per item, so the 32-bit shared counters cannot overflow)
      epi_sync<EPIW>();
      for (int b = (int)threadIdx.x - 128; b < P.nbins + 2; b += EPI_WARPS * 32) {
        const uint32_t v = hist_s[b];
        if (v) {  // global layout: bins 0 .. nbins-1, then below, then above
          atomicAdd(P.hist + (b == 0 ? P.nbins : (b <= P.nbins ? b - 1 : P.nbins + 1)), (unsigned long long)v);
          hist_s[b] = 0;
        }
      }
      epi_sync<EPIW>();
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 2) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, TMEM_COLS);
  }
}

// Exact FP64 chi2 of listed pairs from the centred, weighted curves (P = cenA[i], Q = cenB[j]).
__global__ void __launch_bounds__(256) k_pd_refine(const double* __restrict__ cenA, const double* __restrict__ cenB,
                                                   int T, const int* __restrict__ ri,
                                                   const int* __restrict__ rj, unsigned n, int nbins, double lo,
                                                   double width, unsigned long long* __restrict__ hist, float thr,
                                                   unsigned cap, unsigned* __restrict__ ncand, float* __restrict__ cval,
                                                   int* __restrict__ ci, int* __restrict__ cj, float* __restrict__ out,
                                                   int NB) {
  for (unsigned p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
    const int i = ri[p], j = rj[p];
    const double* a = cenA + (long)i * T;
    const double* b = cenB + (long)j * T;
    double s = 0.0;
    for (int t = 0; t < T; t++) {
      const double r = b[t] - a[t];
      s += r * r;
    }
    const float chi2 = (float)s;
    if (out) out[(long)i * NB + j] = chi2;
    if (s > 0) {
      const int bin = (int)floor((log10(s) - lo) / width);
      atomicAdd(hist + (bin < 0 ? nbins : (bin < nbins ? bin : nbins + 1)), 1ull);
    } else if (s == 0) {
      atomicAdd(hist + nbins, 1ull);  // below every edge
    }
    if (chi2 < thr) {
      const unsigned k = atomicAdd(ncand, 1u);
      if (k < cap) {
        cval[k] = chi2;
        ci[k] = i;
        cj[k] = j;
      }
    }
  }
}

// chi2 of pseudo-random pairs (integer hash of the sample index) for the top-k threshold.
__global__ void __launch_bounds__(256) k_pd_sample(const double* __restrict__ cenA, const double* __restrict__ cenB,
                                                   int NA, int NB, int T, long S,
                                                   uint64_t* __restrict__ keys, uint32_t* __restrict__ vals) {
  for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < S; p += (long)gridDim.x * blockDim.x) {
    uint64_t z = (uint64_t)p * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    const int i = (int)((z & 0xFFFFFFFFull) % (uint64_t)NA), j = (int)((z >> 32) % (uint64_t)NB);
    const double* a = cenA + (long)i * T;
    const double* b = cenB + (long)j * T;
    double s = 0.0;
    for (int t = 0; t < T; t++) {
      const double r = b[t] - a[t];
      s += r * r;
    }
    uint64_t u = __double_as_longlong(s);  // s >= 0: the bit pattern orders like the value
    keys[p] = u;
    vals[p] = (uint32_t)p;
  }
}

// Plain form, stage 2: log10 histogram and top-k candidates of a chunk of FP64 chi2 values
// (pairs row0*NB + q).  Shared-memory counters, flushed once per CTA.
__global__ void __launch_bounds__(256) k_pd_hist_cand(const double* __restrict__ chi2, long n, long p0, int NB,
                                                      int nbins, double lo, double width,
                                                      unsigned long long* __restrict__ hist, float thr, unsigned cap,
                                                      unsigned* __restrict__ ncand, float* __restrict__ cval,
                                                      int* __restrict__ ci, int* __restrict__ cj) {
  extern __shared__ uint32_t hs[];
  for (int b = threadIdx.x; b < nbins + 2; b += blockDim.x) hs[b] = 0;
  __syncthreads();
  for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
    const double s = chi2[q];
    if (s > 0) {
      const int bin = (int)floor((log10(s) - lo) / width);
      atomicAdd(hs + (bin < 0 ? nbins : (bin < nbins ? bin : nbins + 1)), 1u);
    } else if (s == 0) {
      atomicAdd(hs + nbins, 1u);  // below every edge
    }
    if ((float)s < thr) {
      const unsigned k = atomicAdd(ncand, 1u);
      if (k < cap) {
        cval[k] = (float)s;
        ci[k] = (int)((p0 + q) / NB);
        cj[k] = (int)((p0 + q) % NB);
      }
    }
  }
  __syncthreads();
  for (int b = threadIdx.x; b < nbins + 2; b += blockDim.x)
    if (hs[b]) atomicAdd(hist + b, (unsigned long long)hs[b]);
}

__global__ void k_cand_keys(const float* __restrict__ cval, unsigned n, uint64_t* __restrict__ keys,
                            uint32_t* __restrict__ vals) {
  for (unsigned q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    keys[q] = (uint64_t)__float_as_uint(cval[q]);  // chi2 >= 0: bits order like values
    vals[q] = q;
  }
}

__global__ void k_cand_gather(const uint32_t* __restrict__ order, unsigned m, const float* __restrict__ cval,
                              const int* __restrict__ ci, const int* __restrict__ cj, float* __restrict__ ov,
                              int* __restrict__ oi, int* __restrict__ oj) {
  for (unsigned q = blockIdx.x * blockDim.x + threadIdx.x; q < m; q += gridDim.x * blockDim.x) {
    const uint32_t s = order[q];
    ov[q] = cval[s];
    oi[q] = ci[s];
    oj[q] = cj[s];
  }
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    MLC_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q));
    MLC_REQUIRE(q == cudaDriverEntryPointSuccess && p, MLC_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
    fn = (EncodeTiledFn)p;
  }
  return fn;
}

CUtensorMap make_map(void* base, int rows, int kcols, int box_rows) {
  CUtensorMap m;
  std::memset(&m, 0, sizeof m);
  cuuint64_t dims[2] = {(cuuint64_t)kcols, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)kcols * 2};
  cuuint32_t box[2] = {64, (cuuint32_t)box_rows};
  cuuint32_t es[2] = {1, 1};
  CUresult r = encode_fn()(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, base, dims, strides, box, es,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  MLC_REQUIRE(r == CUDA_SUCCESS, MLC_ERR_CUDA, "cuTensorMapEncodeTiled failed");
  return m;
}

}  // namespace

using PdKernel = decltype(&k_pairdiff_tc<1, false, 16>);

template <int NKB, bool OUT>
static PdKernel pd_kernel_t(int epiw) {
  switch (epiw) {
    case 12: return k_pairdiff_tc<NKB, OUT, 12>;
    case 24: return k_pairdiff_tc<NKB, OUT, 24>;
    default: return k_pairdiff_tc<NKB, OUT, 16>;
  }
}

static PdKernel pd_kernel(int nkb, bool out, int epiw) {
  return nkb == 1 ? (out ? pd_kernel_t<1, true>(epiw) : pd_kernel_t<1, false>(epiw))
                  : (out ? pd_kernel_t<2, true>(epiw) : pd_kernel_t<2, false>(epiw));
}

// The epilogue warp count for this shape class (K boxes, matrix or not, histogram size,
// pair count to the nearest power of four): with the autotuner on, the first call of a
// class times one launch of each count on the real operands (the pass loop that follows
// clears and recomputes every output) and keeps the fastest; otherwise 16.
static int pd_epilogue_choice(mlc_ctx* ctx, int nkb, bool out, int nbins, long long P, int grid, size_t smem,
                              const CUtensorMap& tmA, const CUtensorMap& tmB, const PdParams& prm,
                              unsigned* counters, unsigned long long* hist) {
  if (!ctx->autotune) return 16;
  int lg = 0;
  while ((1LL << (2 * (lg + 1))) <= P) lg++;
  char key[96];
  std::snprintf(key, sizeof key, "pairdiff_tc K%d%s bins%d pairs~4^%d", 64 * nkb, out ? " matrix" : "",
                nbins <= 1024 ? 1024 : 4096, lg);
  auto it = ctx->tune.find(key);
  if (it != ctx->tune.end()) return it->second;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  MLC_CUDA(cudaStreamIsCapturing(ctx->stream, &cs));
  if (cs != cudaStreamCaptureStatusNone) return 16;
  const bool saved = ctx->timing;
  ctx->timing = false;  // tuning launches stay out of the per-kernel timings
  cudaEvent_t a = nullptr, b = nullptr;
  std::vector<std::pair<int, float>> ms;
  try {
    MLC_CUDA(cudaEventCreate(&a));
    MLC_CUDA(cudaEventCreate(&b));
    PdParams q = prm;
    q.thr = -1.f;  // no candidates while timing
    for (int e : EPI_CHOICES) {
      const auto kern = pd_kernel(nkb, out, e);
      set_max_smem((const void*)kern, smem);
      MLC_CUDA(cudaMemsetAsync(counters, 0, 16, ctx->stream));
      MLC_CUDA(cudaMemsetAsync(hist, 0, 8 * (size_t)(nbins + 2), ctx->stream));
      MLC_CUDA(cudaEventRecord(a, ctx->stream));
      kern<<<grid, (4 + e) * 32, smem, ctx->stream>>>(tmA, tmB, q);
      MLC_CHECK_LAUNCH();
      MLC_CUDA(cudaEventRecord(b, ctx->stream));
      MLC_CUDA(cudaEventSynchronize(b));
      unsigned hc[4];
      MLC_CUDA(cudaMemcpy(hc, counters, 16, cudaMemcpyDeviceToHost));
      MLC_REQUIRE(hc[2] == 0, MLC_ERR_TIMEOUT, "tensor-core pair kernel: a pipeline wait timed out");
      float t = 0.f;
      MLC_CUDA(cudaEventElapsedTime(&t, a, b));
      ms.emplace_back(e, t);
    }
  } catch (...) {
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    ctx->timing = saved;
    throw;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  ctx->timing = saved;
  const auto best = *std::min_element(ms.begin(), ms.end(), [](const auto& x, const auto& y) { return x.second < y.second; });
  ctx->tune[key] = best.first;
  ctx->tune_name[key] = "epi" + std::to_string(best.first);
  std::string rec;
  for (const auto& m : ms) {
    char buf[48];
    std::snprintf(buf, sizeof buf, "%sepi%d=%.4f", rec.empty() ? "" : " ", m.first, m.second);
    rec += buf;
  }
  ctx->tune_log[key] = rec;
  return best.first;
}

// Pair chi2 from prepared operands, with the fused log10-chi2 histogram and top-k: the
// tensor-core kernel (method 1) or the plain FP64 chunks (method 0, which reads the FP32
// curves A and B and the tables pairdiff_prepare left in the small workspace).
static void pairdiff_core(mlc_ctx* ctx, int method, const float* A, const float* B, const PdOperands& ops,
                          const double* w_host, const double* d_host, int offset, int nbins, double lo, double hi,
                          uint64_t* hist_host, int k, double* tv, int64_t* ti, int64_t* tj, float* out,
                          PdResult& res) {
  const int NA = ops.NA, NB = ops.NB, T = ops.T;
  res.delta = ops.delta;
  const int nkb = ops.Kp / 64;
  CUtensorMap tmA = make_map(ops.a, ops.NApad, 3 * ops.Kp, TM);
  CUtensorMap tmB = make_map(ops.b, ops.NBpad, 3 * ops.Kp, TN);
  const long long P = (long long)NA * NB;

  // ---- top-k threshold from a sample of pairs
  const unsigned cap = (unsigned)std::min<long long>(P, 8LL * k + (1LL << 20));
  double thr = -1.0;  // no candidates unless k > 0
  if (k > 0) {
    // 2^20 sampled pairs: the threshold only filters candidates (the top-k itself is exact),
    // and with the 4x + 16 rank margin below it stays above the k-th value (a rerun of the
    // pass when it does not); 2^22 samples cost 3.5 ms of a 41 ms 10^10-pair step in FP64
    const long S = 1L << 20;
    uint64_t* sk = (uint64_t*)ws_get(ctx, WS_LOC, (sizeof(uint64_t) + sizeof(uint32_t)) * S);
    uint32_t* sv = (uint32_t*)(sk + S);
    {
      MLC_KSCOPE(ctx, "pd_sample");
      k_pd_sample<<<ctx->sm_count * 8, 256, 0, ctx->stream>>>(ops.cenA, ops.cenB, NA, NB, T, S, sk, sv);
    }
    MLC_CHECK_LAUNCH();
    radix_sort_u64_u32(ctx, S, sk, sv);
    const double expect = (double)k * (double)S / (double)P;
    const long rank = std::min<long>(S - 1, (long)std::ceil(4.0 * expect) + 16);
    uint64_t u = 0;
    MLC_CUDA(cudaMemcpy(&u, sk + rank, 8, cudaMemcpyDeviceToHost));
    double v;
    std::memcpy(&v, &u, 8);
    thr = v;
  }
  // ---- buffers: candidates, refinement list, counters, histogram
  const unsigned rcap = 1u << 22;
  char* buf = (char*)ws_get(ctx, WS_PAIR_CAND, (size_t)cap * 12 + (size_t)rcap * 8 + 64 + 8 * (size_t)(nbins + 2) + 64);
  float* cval = (float*)buf;
  int* ci = (int*)(cval + cap);
  int* cj = ci + cap;
  int* ri = cj + cap;
  int* rj = ri + rcap;
  unsigned* counters = (unsigned*)(rj + rcap);  // ncand, nref, err
  unsigned long long* hist = (unsigned long long*)round_up((long)(uintptr_t)(counters + 4), 16);

  const int nj = ops.NBpad / TN, ni = ops.NApad / TM;
  const int grid_max = ctx->sm_count;
  int njc = 1;
  while ((long)ni * njc < 8L * grid_max && njc < nj) njc *= 2;
  const int jchunk = (nj + njc - 1) / njc;
  njc = (nj + jchunk - 1) / jchunk;
  PdParams prm;
  prm.NA = NA;
  prm.NB = NB;
  prm.nj = nj;
  prm.njc = njc;
  prm.jchunk = jchunk;
  prm.nitems = ni * njc;
  prm.nkb = nkb;
  prm.alpha_ff = ops.alpha_ff;
  prm.beta_ff = ops.beta_ff;
  prm.ea = ops.ea;
  prm.eb = ops.eb;
  prm.nbins = nbins;
  prm.hscale = (float)(0.30102999566398120 * nbins / (hi - lo));  // log10(2) / bin width
  prm.hoff = (float)(-lo * nbins / (hi - lo));
  prm.hist = hist;
  prm.cap = cap;
  prm.ncand = counters;
  prm.cval = cval;
  prm.ci = ci;
  prm.cj = cj;
  // Pairs recomputed exactly besides the top-k candidates (bounds in units of 2^(2m), where
  // the steps of both curves are <= 2^m).  With a matrix requested, every pair whose
  // quantisation error (taken at 2 sqrt(T/6) 2^m sqrt(chi2) for independent uniform errors)
  // could exceed 1e-6 relative; otherwise the pairs within 1e4 times the left-out-diagonal
  // bound 2 T 127^2 of zero (whose sign or log10 bin that bound could change).
  // Matrix mode: recompute every pair whose quantisation error, taken at
  // 2 sqrt(T/6) (2^ei + 2^ej) sqrt(chi2) for independent uniform errors, could exceed 1e-6.
  prm.refine_f = (float)(4.0 * (T / 6.0) * 1e12);
  prm.rcap = rcap;
  prm.nref = counters + 1;
  prm.ri = ri;
  prm.rj = rj;
  prm.out = out;
  prm.err = (int*)(counters + 2);
  const size_t smem = smem_bytes(nkb, nbins);
  MLC_REQUIRE(nkb == 1 || nkb == 2, MLC_ERR_LIMIT, "tensor-core pair chi2 supports T <= 128 epochs");
  const int grid = std::min(grid_max, prm.nitems);
  const int epiw = method == 1 ? pd_epilogue_choice(ctx, nkb, out != nullptr, nbins, P, grid, smem, tmA, tmB, prm,
                                                    counters, hist)
                               : 16;
  const auto kern = pd_kernel(nkb, out != nullptr, epiw);
  const int nthreads = (4 + epiw) * 32;
  set_max_smem((const void*)kern, smem);
  // plain form: FP64 chi2 of row chunks, then histogram / candidates of each chunk
  double* wd = nullptr;
  const long rows_per_chunk = std::max<long>(1, std::min<long>(NA, (1L << 27) / NB));
  double* chunk = nullptr;
  if (method == 0) {
    chunk = (double*)ws_get(ctx, WS_CONV_OUT, sizeof(double) * rows_per_chunk * NB);
    wd = (double*)ctx->ws_ptr[WS_SMALL];  // sw, w, d from pairdiff_prepare
  }
  double W = 0.0;
  for (int t = 0; t < T; t++) W += w_host[t];

  for (int pass = 0; pass < 4; pass++) {
    res.passes = pass + 1;
    prm.thr = (float)std::min(thr, 3.0e38);  // -1: no candidates
    MLC_CUDA(cudaMemsetAsync(counters, 0, 16, ctx->stream));
    MLC_CUDA(cudaMemsetAsync(hist, 0, 8 * (size_t)(nbins + 2), ctx->stream));
    if (method == 1) {
      MLC_KSCOPE(ctx, "pairdiff_tc");
      kern<<<grid, nthreads, smem, ctx->stream>>>(tmA, tmB, prm);
    } else {
      for (long r0 = 0; r0 < NA; r0 += rows_per_chunk) {
        const long nr = std::min<long>(rows_per_chunk, NA - r0);
        pairdiff_plain(ctx, A + r0 * T, B, (int)nr, NB, T, wd + T, d_host ? wd + 2 * T : nullptr, W, offset, 0,
                       nullptr, nullptr, chunk);
        if (out) {
          // matrix output of the plain form as FP32
          std::vector<double> hc((size_t)nr * NB);
          MLC_CUDA(cudaMemcpyAsync(hc.data(), chunk, sizeof(double) * hc.size(), cudaMemcpyDeviceToHost, ctx->stream));
          MLC_CUDA(cudaStreamSynchronize(ctx->stream));
          std::vector<float> hf(hc.begin(), hc.end());
          MLC_CUDA(cudaMemcpy(out + r0 * NB, hf.data(), sizeof(float) * hf.size(), cudaMemcpyHostToDevice));
        }
        const long n = nr * NB;
        const size_t hsm = sizeof(uint32_t) * (nbins + 2);
        set_max_smem((const void*)k_pd_hist_cand, hsm);
        MLC_KSCOPE(ctx, "pd_hist_cand");
        k_pd_hist_cand<<<(int)std::min<long>((n + 255) / 256, (long)ctx->sm_count * 8), 256, hsm, ctx->stream>>>(
            chunk, n, r0 * NB, NB, nbins, lo, (hi - lo) / nbins, hist, prm.thr, cap, counters, cval, ci, cj);
      }
    }
    MLC_CHECK_LAUNCH();
    unsigned hc[4];
    MLC_CUDA(cudaMemcpyAsync(hc, counters, 16, cudaMemcpyDeviceToHost, ctx->stream));
    MLC_CUDA(cudaStreamSynchronize(ctx->stream));
    MLC_REQUIRE(hc[2] == 0, MLC_ERR_TIMEOUT, "tensor-core pair kernel: a pipeline wait timed out");
    if (hc[1] > rcap) {  // the exact list overflowed: with a finite threshold lower it, else give up
      MLC_REQUIRE(std::isfinite(thr) && k > 0 && pass < 3, MLC_ERR_LIMIT,
                  "more than 4M pairs need the exact FP64 path (near-identical curves)");
      thr *= 0.25;
      continue;
    }
    if (hc[1] > 0) {
      MLC_KSCOPE(ctx, "pd_refine");
      k_pd_refine<<<std::max(1u, std::min((hc[1] + 255) / 256, (unsigned)ctx->sm_count * 8)), 256, 0, ctx->stream>>>(
          ops.cenA, ops.cenB, T, ri, rj, hc[1], nbins, lo, (hi - lo) / nbins, hist, prm.thr, cap, counters, cval,
          ci, cj, out, NB);
    }
    MLC_CHECK_LAUNCH();
    MLC_CUDA(cudaMemcpyAsync(hc, counters, 16, cudaMemcpyDeviceToHost, ctx->stream));
    MLC_CUDA(cudaStreamSynchronize(ctx->stream));
    res.nrefined = hc[1];
    res.ncand = hc[0];
    res.thr = thr;
    if (k == 0) break;
    if (hc[0] > cap) {  // too many candidates: lower the threshold
      thr *= 0.5;
      continue;
    }
    if ((long long)hc[0] < std::min<long long>(k, P) && std::isfinite(thr)) {  // too few: raise it
      thr = thr > 0 ? thr * (hc[0] > 0 ? 4.0 : 16.0) : 1e-30;
      if (pass == 2) thr = INFINITY;
      continue;
    }
    break;
  }
  if (hist_host) MLC_CUDA(cudaMemcpy(hist_host, hist, 8 * (size_t)nbins, cudaMemcpyDeviceToHost));
  {
    unsigned long long oor[2];
    MLC_CUDA(cudaMemcpy(oor, hist + nbins, sizeof oor, cudaMemcpyDeviceToHost));
    res.below = (long long)oor[0];
    res.above = (long long)oor[1];
  }
  // ---- top-k from the candidates: sort by value (stable by candidate order), then order
  // ties by pair index on the host
  if (k > 0) {
    const unsigned nc = (unsigned)std::min<long long>(res.ncand, cap);
    const unsigned m = (unsigned)std::min<long long>(nc, (long long)k + 1024);
    const unsigned ncb = std::max(nc, 1u);
    char* kb = (char*)ws_get(ctx, WS_LOC, (sizeof(uint64_t) + sizeof(uint32_t)) * (size_t)ncb + 12 * (size_t)ncb + 64);
    uint64_t* keys = (uint64_t*)kb;
    uint32_t* vals = (uint32_t*)(keys + ncb);
    float* gv = (float*)(vals + ncb);
    int* gi = (int*)(gv + ncb);
    int* gj = gi + ncb;
    if (nc > 0) {
      {
        MLC_KSCOPE(ctx, "pd_topk_keys");
        k_cand_keys<<<std::max(1u, std::min((nc + 255) / 256, (unsigned)ctx->sm_count * 8)), 256, 0, ctx->stream>>>(
            cval, nc, keys, vals);
      }
      MLC_CHECK_LAUNCH();
      radix_sort_u64_u32(ctx, nc, keys, vals);
      {
        MLC_KSCOPE(ctx, "pd_topk_gather");
        k_cand_gather<<<std::max(1u, (m + 255) / 256), 256, 0, ctx->stream>>>(vals, m, cval, ci, cj, gv, gi, gj);
      }
      MLC_CHECK_LAUNCH();
    }
    // the first k + 1024 by value; order ties by pair index on the host
    std::vector<float> hv(m);
    std::vector<int> hi_(m), hj(m);
    MLC_CUDA(cudaMemcpy(hv.data(), gv, 4 * (size_t)m, cudaMemcpyDeviceToHost));
    MLC_CUDA(cudaMemcpy(hi_.data(), gi, 4 * (size_t)m, cudaMemcpyDeviceToHost));
    MLC_CUDA(cudaMemcpy(hj.data(), gj, 4 * (size_t)m, cudaMemcpyDeviceToHost));
    const unsigned ncand_used = m;
    std::vector<uint32_t> idx(ncand_used);
    for (unsigned q = 0; q < ncand_used; q++) idx[q] = q;
    std::sort(idx.begin(), idx.end(), [&](uint32_t x, uint32_t y) {
      if (hv[x] != hv[y]) return hv[x] < hv[y];
      const long long px = (long long)hi_[x] * NB + hj[x], py = (long long)hi_[y] * NB + hj[y];
      return px < py;
    });
    const int kk = (int)std::min<long long>(k, ncand_used);
    for (int q = 0; q < kk; q++) {
      tv[q] = hv[idx[q]];
      ti[q] = hi_[idx[q]];
      tj[q] = hj[idx[q]];
    }
    for (int q = kk; q < k; q++) {
      tv[q] = INFINITY;
      ti[q] = -1;
      tj[q] = -1;
    }
  }
}

void pairdiff_run(mlc_ctx* ctx, int method, const float* A, const float* B, int NA, int NB, int T,
                  const double* w_host, const double* d_host, int offset, int nbins, double lo, double hi,
                  uint64_t* hist_host, int k, double* tv, int64_t* ti, int64_t* tj, float* out, PdResult& res) {
  MLC_REQUIRE(method == 1 || T <= 4096, MLC_ERR_LIMIT, "T <= 4096");
  MLC_REQUIRE(method == 0 || (T >= 1 && T <= MAX_KP), MLC_ERR_LIMIT,
              "tensor-core pair chi2 supports T <= 128 epochs");
  MLC_REQUIRE(nbins >= 1 && nbins <= MAX_BINS && hi > lo, MLC_ERR_ARG, "histogram: 1..4096 bins, hi > lo");
  MLC_REQUIRE(NA >= 1 && NB >= 1 && k >= 0, MLC_ERR_ARG, "bad sizes");
  PdOperands ops;
  pairdiff_prepare(ctx, A, B, NA, NB, T, w_host, d_host, offset, ops);
  pairdiff_core(ctx, method, A, B, ops, w_host, d_host, offset, nbins, lo, hi, hist_host, k, tv, ti, tj, out, res);
}

// Two prepared sides: the operands point into the sides' own memory (rows padded to
// PD_SIDE_PAD, beyond both tile heights, and zero there), so nothing is recomputed.
void pairdiff_sides(mlc_ctx* ctx, const PdSide& A, const PdSide& B, int nbins, double lo, double hi,
                    uint64_t* hist_host, int k, double* tv, int64_t* ti, int64_t* tj, float* out, PdResult& res) {
  MLC_REQUIRE(A.T == B.T && A.offset == B.offset && A.w == B.w, MLC_ERR_ARG,
              "pair sides built with different epochs, weights or offset forms");
  MLC_REQUIRE(!A.has_d, MLC_ERR_ARG, "side A must be built without the observed difference curve d");
  MLC_REQUIRE(A.T >= 1 && A.T <= MAX_KP, MLC_ERR_LIMIT, "tensor-core pair chi2 supports T <= 128 epochs");
  MLC_REQUIRE(nbins >= 1 && nbins <= MAX_BINS && hi > lo, MLC_ERR_ARG, "histogram: 1..4096 bins, hi > lo");
  MLC_REQUIRE(A.N >= 1 && B.N >= 1 && k >= 0, MLC_ERR_ARG, "bad sizes");
  PdOperands ops;
  ops.NA = A.N;
  ops.NB = B.N;
  ops.T = A.T;
  ops.Kp = A.Kp;
  ops.NApad = (int)round_up(A.N, PD_TILE_M);
  ops.NBpad = (int)round_up(B.N, PD_TILE_N);
  ops.delta = std::max(A.delta, B.delta);  // the step pairdiff_prepare reports for both sides together
  ops.a = A.ops;
  ops.b = B.ops;
  ops.alpha = A.norm2;
  ops.beta = B.norm2;
  ops.alpha_ff = A.norm2_ff;
  ops.beta_ff = B.norm2_ff;
  ops.ea = A.exps;
  ops.eb = B.exps;
  ops.cenA = A.cen;
  ops.cenB = B.cen;
  pairdiff_core(ctx, 1, nullptr, nullptr, ops, A.w.data(), nullptr, A.offset, nbins, lo, hi, hist_host, k, tv, ti,
                tj, out, res);
}

// Self-test of the bounded-wait unwinding the pair kernel relies on: one CTA allocates TMEM
// like the pair kernel, waits on an mbarrier that nothing arrives at and that no copy or MMA
// feeds (so nothing asynchronous is in flight when the wait gives up), records that it gave
// up, releases its TMEM and records that too.  report[0]: the wait gave up; report[1]: polls
// used; report[2]: TMEM released after it.
__global__ void __launch_bounds__(64) k_wait_selftest(uint32_t limit, unsigned* report) {
  __shared__ uint64_t bar;
  __shared__ uint32_t tslot;
  const int warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) {
    tc::mbar_init(&bar, 1);
    tc::fence_barrier_init();
  }
  if (warp == 0) tc::tmem_alloc(&tslot, 32);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tslot;
  uint32_t polls = 0;
  bool done = false;
  for (; polls < limit && !done; polls++) done = tc::mbar_try_wait(&bar, 0);
  if (threadIdx.x == 0) {
    report[0] = done ? 0u : 1u;
    report[1] = polls;
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, 32);
  }
  __syncthreads();
  if (threadIdx.x == 0) report[2] = 1u;
}

void selftest_wait_timeout(mlc_ctx* ctx, unsigned polls, unsigned* report_host) {
  MLC_REQUIRE(polls >= 1 && polls <= (1u << 24), MLC_ERR_ARG, "polls: 1 .. 2^24");
  unsigned* rep = (unsigned*)ws_get(ctx, WS_SMALL, 4 * sizeof(unsigned));
  MLC_CUDA(cudaMemsetAsync(rep, 0, 4 * sizeof(unsigned), ctx->stream));
  {
    MLC_KSCOPE(ctx, "wait_selftest");
    k_wait_selftest<<<1, 64, 0, ctx->stream>>>(polls, rep);
  }
  MLC_CHECK_LAUNCH();
  unsigned h[4];
  MLC_CUDA(cudaMemcpyAsync(h, rep, sizeof h, cudaMemcpyDeviceToHost, ctx->stream));
  MLC_CUDA(cudaStreamSynchronize(ctx->stream));
  for (int i = 0; i < 3; i++) report_host[i] = h[i];
  MLC_REQUIRE(h[2] == 1u, MLC_ERR_CUDA, "wait self-test: TMEM was not released");
  MLC_REQUIRE(h[0] == 0u, MLC_ERR_TIMEOUT, "wait self-test: the bounded wait gave up after its poll limit");
}

}  // namespace mlc
