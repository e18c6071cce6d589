// Hand-written mixed-radix Stockham FFT for sm_103a: in-shared-memory batched
// transforms (radix 2, 3, 4, 5, 8) used by the row passes (one image row per CTA) and
// the column passes (a 128-byte strip of columns per CTA, four-step split N = N1*N2).
#pragma once

#include "mlc_common.cuh"

namespace mlc {

// Stage plan of one batched transform length: radix, sub-transform size Ns before the
// stage, the 32-bit multiplier that divides by Ns (j / Ns = umulhi(j, magic) for the
// j < 2^16 used here; Ns == 1 is special-cased), and the twiddle-table step.
struct RadixList {
  int n;
  int L;
  int r[20];
  int Ns[20];
  uint32_t magic[20];
  int twstep[20];
  int toff[20];  // offset of stage p's twiddles in a staged table: Ns[p] * (r[p] - 1) entries
  int tlen;      // entries of the whole staged table
};

// Radix plan for length L (2^a 3^b 5^c) whose twiddles come from a table of
// L*tw_stride entries, or n = -1 when L has another factor.
RadixList factor_radices(int L, int tw_stride);

// ---------------------------------------------------------------- small DFTs

template <typename T, int R, bool INV>
struct Dft;

template <typename T, bool INV>
struct Dft<T, 2, INV> {
  static __device__ __forceinline__ void run(C2<T>* v) {
    C2<T> a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  }
};

template <typename T, bool INV>
struct Dft<T, 3, INV> {
  static __device__ __forceinline__ void run(C2<T>* v) {
    const T h = (T)0.86602540378443864676372317075294;  // sin(2 pi / 3)
    C2<T> s = cadd(v[1], v[2]);
    C2<T> d = csub(v[1], v[2]);
    C2<T> m = C2<T>{v[0].x - (T)0.5 * s.x, v[0].y - (T)0.5 * s.y};
    C2<T> id = mul_mi<T, INV>(d);  // -i d (forward) / +i d (inverse)
    v[0] = cadd(v[0], s);
    v[1] = C2<T>{m.x + h * id.x, m.y + h * id.y};
    v[2] = C2<T>{m.x - h * id.x, m.y - h * id.y};
  }
};

template <typename T, bool INV>
struct Dft<T, 4, INV> {
  static __device__ __forceinline__ void run(C2<T>* v) {
    C2<T> a0 = cadd(v[0], v[2]), a1 = csub(v[0], v[2]);
    C2<T> a2 = cadd(v[1], v[3]), a3 = mul_mi<T, INV>(csub(v[1], v[3]));
    v[0] = cadd(a0, a2);
    v[2] = csub(a0, a2);
    v[1] = cadd(a1, a3);
    v[3] = csub(a1, a3);
  }
};

// The cosine part in Winograd's form: x0 + c1 sa + c2 sb and x0 + c2 sa + c1 sb are
// u +/- m with u = x0 + (c1 + c2)/2 (sa + sb), m = (c1 - c2)/2 (sa - sb), where
// (c1 + c2)/2 = -1/4 exactly (an exact scaling) and (c1 - c2)/2 = sqrt(5)/4: one general
// product per component instead of four.
template <typename T, bool INV>
struct Dft<T, 5, INV> {
  static __device__ __forceinline__ void run(C2<T>* v) {
    const T b = (T)0.55901699437494742410229341718282;    // (cos(2 pi/5) - cos(4 pi/5)) / 2
    const T s1 = (T)0.95105651629515357211643933337938;   // sin(2 pi/5)
    const T s2 = (T)0.58778525229247312916870595463907;   // sin(4 pi/5)
    C2<T> x0 = v[0];
    C2<T> sa = cadd(v[1], v[4]), da = csub(v[1], v[4]);
    C2<T> sb = cadd(v[2], v[3]), db = csub(v[2], v[3]);
    C2<T> t1 = cadd(sa, sb), t2 = csub(sa, sb);
    C2<T> u = C2<T>{x0.x - scale2(t1.x, 0.25f), x0.y - scale2(t1.y, 0.25f)};
    C2<T> m = C2<T>{b * t2.x, b * t2.y};
    C2<T> p1 = cadd(u, m), p2 = csub(u, m);
    C2<T> q1 = C2<T>{s1 * da.x + s2 * db.x, s1 * da.y + s2 * db.y};
    C2<T> q2 = C2<T>{s2 * da.x - s1 * db.x, s2 * da.y - s1 * db.y};
    C2<T> iq1 = mul_mi<T, INV>(q1), iq2 = mul_mi<T, INV>(q2);
    v[0] = cadd(x0, t1);
    v[1] = cadd(p1, iq1);
    v[4] = csub(p1, iq1);
    v[2] = cadd(p2, iq2);
    v[3] = csub(p2, iq2);
  }
};

template <typename T, bool INV>
struct Dft<T, 8, INV> {
  static __device__ __forceinline__ void run(C2<T>* v) {
    const T r = (T)0.70710678118654752440084436210485;
    C2<T> e[4] = {v[0], v[2], v[4], v[6]};
    C2<T> o[4] = {v[1], v[3], v[5], v[7]};
    Dft<T, 4, INV>::run(e);
    Dft<T, 4, INV>::run(o);
    // o[q] *= W8^q ; forward W8 = (1 - i)/sqrt2, inverse (1 + i)/sqrt2
    C2<T> o1 = INV ? C2<T>{r * (o[1].x - o[1].y), r * (o[1].x + o[1].y)}
                   : C2<T>{r * (o[1].x + o[1].y), r * (o[1].y - o[1].x)};
    C2<T> o2 = mul_mi<T, INV>(o[2]);
    C2<T> o3 = INV ? C2<T>{-r * (o[3].x + o[3].y), r * (o[3].x - o[3].y)}
                   : C2<T>{r * (o[3].y - o[3].x), -r * (o[3].x + o[3].y)};
    v[0] = cadd(e[0], o[0]);
    v[4] = csub(e[0], o[0]);
    v[1] = cadd(e[1], o1);
    v[5] = csub(e[1], o1);
    v[2] = cadd(e[2], o2);
    v[6] = csub(e[2], o2);
    v[3] = cadd(e[3], o3);
    v[7] = csub(e[3], o3);
  }
};

// Radix 2 over two half-length DFTs: X[k] = E[k] + W^k O[k], X[k + R/2] = E[k] - W^k O[k],
// W = exp(-/+ 2 pi i / R); wr[k], wi[k] = cos, sin(2 pi k / R).
template <typename T, int H, bool INV>
__device__ __forceinline__ void dft_split2(C2<T>* v, const T* wr, const T* wi) {
  C2<T> e[H], o[H];
#pragma unroll
  for (int i = 0; i < H; i++) {
    e[i] = v[2 * i];
    o[i] = v[2 * i + 1];
  }
  Dft<T, H, INV>::run(e);
  Dft<T, H, INV>::run(o);
  v[0] = cadd(e[0], o[0]);  // W^0 = 1
  v[H] = csub(e[0], o[0]);
#pragma unroll
  for (int k = 1; k < H; k++) {
    // W^k o with W^k = (wr, -wi) forward, (wr, wi) inverse
    const T sr = INV ? -wi[k] : wi[k];
    const C2<T> t = C2<T>{wr[k] * o[k].x + sr * o[k].y, wr[k] * o[k].y - sr * o[k].x};
    v[k] = cadd(e[k], t);
    v[k + H] = csub(e[k], t);
  }
}

// 10 points by the prime-factor (Good-Thomas) split 10 = 2 x 5, which needs no twiddles:
// with n = (5 n1 + 2 n2) mod 10 and k = (5 k1 + 6 k2) mod 10, W10^(n k) = W2^(n1 k1) W5^(n2 k2),
// so five DFT2 over n1, then two DFT5 over n2 (84 real additions and 32 multiplications,
// against 94 and 52 for the radix-2 split with its twiddles).
template <typename T, bool INV>
struct Dft<T, 10, INV> {
  static __device__ __forceinline__ void run(C2<T>* v) {
    C2<T> a[5], b[5];
#pragma unroll
    for (int n2 = 0; n2 < 5; n2++) {
      const C2<T> x0 = v[(2 * n2) % 10], x1 = v[(5 + 2 * n2) % 10];
      a[n2] = cadd(x0, x1);  // k1 = 0
      b[n2] = csub(x0, x1);  // k1 = 1
    }
    Dft<T, 5, INV>::run(a);
    Dft<T, 5, INV>::run(b);
#pragma unroll
    for (int k2 = 0; k2 < 5; k2++) {
      v[(6 * k2) % 10] = a[k2];
      v[(5 + 6 * k2) % 10] = b[k2];
    }
  }
};

template <typename T, bool INV>
struct Dft<T, 16, INV> {
  static __device__ __forceinline__ void run(C2<T>* v) {
    const T c1 = (T)0.92387953251128675612818318939679, s1 = (T)0.38268343236508977172845998403040;
    const T r = (T)0.70710678118654752440084436210485;
    const T wr[8] = {(T)1, c1, r, s1, (T)0, -s1, -r, -c1};
    const T wi[8] = {(T)0, s1, r, c1, (T)1, c1, r, s1};
    dft_split2<T, 8, INV>(v, wr, wi);
  }
};

template <typename T, bool INV>
struct Dft<T, 20, INV> {
  static __device__ __forceinline__ void run(C2<T>* v) {
    // cos, sin(2 pi k / 20), k = 0..9
    const T a = (T)0.95105651629515357211643933337938214, b = (T)0.30901699437494742410229341718281906;
    const T c = (T)0.80901699437494742410229341718281906, d = (T)0.58778525229247312916870595463907277;
    const T wr[10] = {(T)1, a, c, d, b, (T)0, -b, -d, -c, -a};
    const T wi[10] = {(T)0, b, d, c, a, (T)1, a, c, d, b};
    dft_split2<T, 10, INV>(v, wr, wi);
  }
};

// 25 points as 5 x 5 (four-step in registers): DFT5 over n1 of x[5 n1 + n2], twiddle
// W25^(n2 k1), DFT5 over n2 -> X[k1 + 5 k2].
template <typename T, bool INV>
struct Dft<T, 25, INV> {
  static __device__ __forceinline__ void run(C2<T>* v) {
    // cos, sin(2 pi m / 25), m = 0..16
    const T cr[17] = {(T)1,
                      (T)0.96858316112863111949016837546473581,  (T)0.87630668004386358730811590392206258,
                      (T)0.72896862742141152314673031905525911,  (T)0.53582679497899661827130876786763998,
                      (T)0.30901699437494742410229341718281906,  (T)0.062790519529313376076178224565631133,
                      (T)-0.18738131458572463054255073444729147, (T)-0.42577929156507264886250244574425170,
                      (T)-0.63742398974868971017671281167601620, (T)-0.80901699437494742410229341718281906,
                      (T)-0.92977648588825140366094255622199073, (T)-0.99211470131447783104979304278577852,
                      (T)-0.99211470131447783104979304278577852, (T)-0.92977648588825140366094255622199073,
                      (T)-0.80901699437494742410229341718281906, (T)-0.63742398974868971017671281167601620};
    const T ci[17] = {(T)0,
                      (T)0.24868988716485478824228374600644797, (T)0.48175367410171527498719150287212965,
                      (T)0.68454710592868867373228335762120927, (T)0.84432792550201507854855806396668151,
                      (T)0.95105651629515357211643933337938214, (T)0.99802672842827156195233680686345055,
                      (T)0.98228725072868868108564174286526842, (T)0.90482705246601952771366864793269759,
                      (T)0.77051324277578923080300963639617785, (T)0.58778525229247312916870595463907277,
                      (T)0.36812455268467795915694714749296083, (T)0.12533323356430424537311875981650879,
                      (T)-0.12533323356430424537311875981650879, (T)-0.36812455268467795915694714749296083,
                      (T)-0.58778525229247312916870595463907277, (T)-0.77051324277578923080300963639617785};
    C2<T> y[5][5];
#pragma unroll
    for (int n2 = 0; n2 < 5; n2++) {
#pragma unroll
      for (int n1 = 0; n1 < 5; n1++) y[n2][n1] = v[5 * n1 + n2];
      Dft<T, 5, INV>::run(y[n2]);
#pragma unroll
      for (int k1 = 1; k1 < 5; k1++) {
        if (n2 == 0) continue;
        const int m = n2 * k1;
        const T sr = INV ? -ci[m] : ci[m];  // W^m = (cr, -ci) forward, (cr, ci) inverse
        const C2<T> q = y[n2][k1];
        y[n2][k1] = C2<T>{cr[m] * q.x + sr * q.y, cr[m] * q.y - sr * q.x};
      }
    }
#pragma unroll
    for (int k1 = 0; k1 < 5; k1++) {
      C2<T> u[5];
#pragma unroll
      for (int n2 = 0; n2 < 5; n2++) u[n2] = y[n2][k1];
      Dft<T, 5, INV>::run(u);
#pragma unroll
      for (int k2 = 0; k2 < 5; k2++) v[k1 + 5 * k2] = u[k2];
    }
  }
};

// ---------------------------------------------------------------- Stockham stage
// src/dst are [L][CW] complex arrays in shared memory; tw is the length-(L*tw_stride)
// table exp(-2 pi i m / (L*tw_stride)) in global memory.
template <typename T, int R, bool INV, int CW>
__device__ __forceinline__ void stockham_stage(const C2<T>* __restrict__ src, C2<T>* __restrict__ dst, int L,
                                               int Ns, uint32_t magic, int twstep, const C2<T>* __restrict__ tw) {
  const int Lr = L / R;
  const int nb = Lr * CW;
  for (int bt = threadIdx.x; bt < nb; bt += blockDim.x) {
    const int c = bt & (CW - 1);
    const int j = bt / CW;  // CW is a power of two
    int q, k;
    if (Ns == 1) {
      q = j;
      k = 0;
    } else {
      q = (int)__umulhi((uint32_t)j, magic);
      k = j - q * Ns;
    }
    C2<T> v[R];
#pragma unroll
    for (int i = 0; i < R; i++) v[i] = src[(j + i * Lr) * CW + c];
    if (Ns > 1) {
      // one table load per butterfly: W^k; the higher powers W^(ik) by multiplication
      const C2<T> w1 = ldc(tw + k * twstep);
      C2<T> w = w1;
#pragma unroll
      for (int i = 1; i < R; i++) {
        v[i] = INV ? cmulc(v[i], w) : cmul(v[i], w);
        if (i + 1 < R) w = cmul(w, w1);
      }
    }
    Dft<T, R, INV>::run(v);
    const int d = q * Ns * R + k;
#pragma unroll
    for (int i = 0; i < R; i++) dst[(d + i * Ns) * CW + c] = v[i];
  }
}

// The same stage with the twiddles W^(i k) (i = 1 .. R-1) of every k read from a table
// staged in shared memory, tws[k * (R-1) + i - 1] (fill_stage_twiddles): no table reads
// from global memory and no chain of multiplications for the powers.
template <typename T, int R, bool INV, int CW>
__device__ __forceinline__ void stockham_stage_st(const C2<T>* __restrict__ src, C2<T>* __restrict__ dst, int L,
                                                  int Ns, uint32_t magic, const C2<T>* __restrict__ tws) {
  const int Lr = L / R;
  const int nb = Lr * CW;
  for (int bt = threadIdx.x; bt < nb; bt += blockDim.x) {
    const int c = bt & (CW - 1);
    const int j = bt / CW;
    int q, k;
    if (Ns == 1) {
      q = j;
      k = 0;
    } else {
      q = (int)__umulhi((uint32_t)j, magic);
      k = j - q * Ns;
    }
    C2<T> v[R];
#pragma unroll
    for (int i = 0; i < R; i++) v[i] = src[(j + i * Lr) * CW + c];
    if (Ns > 1) {
      const C2<T>* w = tws + k * (R - 1);
#pragma unroll
      for (int i = 1; i < R; i++) v[i] = INV ? cmulc(v[i], w[i - 1]) : cmul(v[i], w[i - 1]);
    }
    Dft<T, R, INV>::run(v);
    const int d = q * Ns * R + k;
#pragma unroll
    for (int i = 0; i < R; i++) dst[(d + i * Ns) * CW + c] = v[i];
  }
}

// Stage twiddle table of a radix plan in shared memory: stage p, index k < Ns, power
// i = 1 .. R-1 -> W^(i k twstep) from the global table tw (i k twstep < L tw_stride).
template <typename T>
__device__ __forceinline__ void fill_stage_twiddles(const RadixList& rl, const C2<T>* __restrict__ tw,
                                                    C2<T>* __restrict__ tab) {
  for (int p = 1; p < rl.n; ++p) {
    const int R = rl.r[p], Ns = rl.Ns[p], ts = rl.twstep[p], o = rl.toff[p];
    for (int e = threadIdx.x; e < Ns * (R - 1); e += blockDim.x) {
      const int k = e / (R - 1), i = e - k * (R - 1) + 1;
      tab[o + e] = ldc(tw + (long)i * k * ts);
    }
  }
}

// fft_smem with the stage twiddles staged in shared memory (tab filled by
// fill_stage_twiddles and synchronised before the call).
template <typename T, bool INV, int CW>
__device__ C2<T>* fft_smem_st(C2<T>* a, C2<T>* b, const RadixList& rl, const C2<T>* __restrict__ tab) {
  const int L = rl.L;
  for (int p = 0; p < rl.n; ++p) {
    const int Ns = rl.Ns[p];
    const uint32_t mg = rl.magic[p];
    const C2<T>* tws = tab + rl.toff[p];
    switch (rl.r[p]) {
      case 2: stockham_stage_st<T, 2, INV, CW>(a, b, L, Ns, mg, tws); break;
      case 3: stockham_stage_st<T, 3, INV, CW>(a, b, L, Ns, mg, tws); break;
      case 4: stockham_stage_st<T, 4, INV, CW>(a, b, L, Ns, mg, tws); break;
      case 5: stockham_stage_st<T, 5, INV, CW>(a, b, L, Ns, mg, tws); break;
      default: stockham_stage_st<T, 8, INV, CW>(a, b, L, Ns, mg, tws); break;
    }
    __syncthreads();
    C2<T>* t = a;
    a = b;
    b = t;
  }
  return a;
}

// Batched length-L transform of the CW columns held in a ([L][CW]); b is scratch of the
// same size.  Returns the buffer that holds the natural-order result.  Ends synchronised.
template <typename T, bool INV, int CW>
__device__ C2<T>* fft_smem(C2<T>* a, C2<T>* b, const RadixList& rl, const C2<T>* __restrict__ tw) {
  const int L = rl.L;
  for (int p = 0; p < rl.n; ++p) {
    const int Ns = rl.Ns[p];
    const uint32_t mg = rl.magic[p];
    const int ts = rl.twstep[p];
    switch (rl.r[p]) {
      case 2: stockham_stage<T, 2, INV, CW>(a, b, L, Ns, mg, ts, tw); break;
      case 3: stockham_stage<T, 3, INV, CW>(a, b, L, Ns, mg, ts, tw); break;
      case 4: stockham_stage<T, 4, INV, CW>(a, b, L, Ns, mg, ts, tw); break;
      case 5: stockham_stage<T, 5, INV, CW>(a, b, L, Ns, mg, ts, tw); break;
      default: stockham_stage<T, 8, INV, CW>(a, b, L, Ns, mg, ts, tw); break;
    }
    __syncthreads();
    C2<T>* t = a;
    a = b;
    b = t;
  }
  return a;
}

}  // namespace mlc
