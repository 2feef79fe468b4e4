// qsf_fft.cuh -- FP64 complex FFT building blocks for sm_103a.
//
// Lines of the wavefunction are staged in shared memory and transformed by in-place
// Stockham passes: each pass reads every butterfly's inputs into registers, barriers,
// then writes the outputs (so one shared buffer suffices).  Radix 2, 3, 4, 5, 8 and
// 16 butterflies keep the FP64 instruction count low: on GB300 the FP64 pipe
// (~1.2 TFLOP/s) is the bottleneck of this step, not HBM, so every butterfly is
// written for the fewest DFMA/DADD/DMUL, twiddles come from precomputed tables
// (exp(-2 pi i t / n), loaded through the read-only path) and no transcendental is
// evaluated per point.
//
// Convention: forward = FFTW_FORWARD (exponent sign -1), unnormalised; the backward
// transform has sign +1.  Pass s with radix R and current sub-length ns reads
// x[j + q n/R], twiddles by w^(jm q) with jm = j mod ns, w = exp(sign 2 pi i/(ns R)),
// does an R-point DFT and writes y[(j - jm) R + jm + q ns].
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace qsf {

__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ double2 cmulc(double2 a, double2 b) {  // a * conj(b)
  return make_double2(fma(a.x, b.x, a.y * b.y), fma(a.y, b.x, -a.x * b.y));
}
__device__ __forceinline__ double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
// multiply by (sign * i): forward sign -1 -> -i
template <bool FWD> __device__ __forceinline__ double2 mul_si(double2 a) {
  return FWD ? make_double2(a.y, -a.x) : make_double2(-a.y, a.x);
}

#define QSF_SQRT1_2 0.70710678118654752440
#define QSF_SQRT3_2 0.86602540378443864676
#define QSF_C5_1 0.30901699437494742410   /* cos(2pi/5) */
#define QSF_C5_2 (-0.80901699437494742410) /* cos(4pi/5) */
#define QSF_S5_1 0.95105651629515357212   /* sin(2pi/5) */
#define QSF_S5_2 0.58778525229247312917   /* sin(4pi/5) */
#define QSF_C16_1 0.92387953251128675613  /* cos(pi/8) */
#define QSF_S16_1 0.38268343236508977173  /* sin(pi/8) */

template <bool FWD> __device__ __forceinline__ void bfly2(double2& a, double2& b) {
  double2 t = a;
  a = cadd(t, b);
  b = csub(t, b);
}

template <bool FWD> __device__ __forceinline__ void bfly4(double2& x0, double2& x1, double2& x2, double2& x3) {
  double2 t0 = cadd(x0, x2), t1 = csub(x0, x2), t2 = cadd(x1, x3), t3 = mul_si<FWD>(csub(x1, x3));
  x0 = cadd(t0, t2);
  x2 = csub(t0, t2);
  x1 = cadd(t1, t3);
  x3 = csub(t1, t3);
}

// w8^1 * a with w8 = exp(sign 2 pi i / 8)
template <bool FWD> __device__ __forceinline__ double2 w8_1(double2 a) {
  return FWD ? make_double2((a.x + a.y) * QSF_SQRT1_2, (a.y - a.x) * QSF_SQRT1_2)
             : make_double2((a.x - a.y) * QSF_SQRT1_2, (a.x + a.y) * QSF_SQRT1_2);
}
template <bool FWD> __device__ __forceinline__ double2 w8_3(double2 a) {
  return FWD ? make_double2((a.y - a.x) * QSF_SQRT1_2, -(a.x + a.y) * QSF_SQRT1_2)
             : make_double2(-(a.x + a.y) * QSF_SQRT1_2, (a.x - a.y) * QSF_SQRT1_2);
}

template <bool FWD> __device__ __forceinline__ void bfly8(double2* v) {
  // radix-2 on (q, q+4), then twiddles w8^q on the odd half, then two radix-4
  double2 a0 = cadd(v[0], v[4]), a4 = csub(v[0], v[4]);
  double2 a1 = cadd(v[1], v[5]), a5 = csub(v[1], v[5]);
  double2 a2 = cadd(v[2], v[6]), a6 = csub(v[2], v[6]);
  double2 a3 = cadd(v[3], v[7]), a7 = csub(v[3], v[7]);
  a5 = w8_1<FWD>(a5);
  a6 = mul_si<FWD>(a6);
  a7 = w8_3<FWD>(a7);
  bfly4<FWD>(a0, a1, a2, a3);
  bfly4<FWD>(a4, a5, a6, a7);
  // outputs: even k from first group, odd k from second (bit-reversed inside groups)
  v[0] = a0; v[4] = a2; v[2] = a1; v[6] = a3;
  v[1] = a4; v[5] = a6; v[3] = a5; v[7] = a7;
}

template <bool FWD> __device__ __forceinline__ void bfly3(double2* v) {
  double2 t1 = cadd(v[1], v[2]), t2 = csub(v[1], v[2]);
  double2 m1 = make_double2(fma(-0.5, t1.x, v[0].x), fma(-0.5, t1.y, v[0].y));
  const double k = FWD ? -QSF_SQRT3_2 : QSF_SQRT3_2;
  v[0] = cadd(v[0], t1);
  // X1 = m1 + i k t2, X2 = m1 - i k t2
  v[1] = make_double2(fma(-k, t2.y, m1.x), fma(k, t2.x, m1.y));
  v[2] = make_double2(fma(k, t2.y, m1.x), fma(-k, t2.x, m1.y));
}

template <bool FWD> __device__ __forceinline__ void bfly5(double2* v) {
  const double s1 = FWD ? -QSF_S5_1 : QSF_S5_1, s2 = FWD ? -QSF_S5_2 : QSF_S5_2;
  double2 t1 = cadd(v[1], v[4]), t2 = cadd(v[2], v[3]), t3 = csub(v[1], v[4]), t4 = csub(v[2], v[3]);
  double2 x0 = v[0];
  double2 a1 = make_double2(fma(QSF_C5_2, t2.x, fma(QSF_C5_1, t1.x, x0.x)), fma(QSF_C5_2, t2.y, fma(QSF_C5_1, t1.y, x0.y)));
  double2 a2 = make_double2(fma(QSF_C5_1, t2.x, fma(QSF_C5_2, t1.x, x0.x)), fma(QSF_C5_1, t2.y, fma(QSF_C5_2, t1.y, x0.y)));
  double2 b1 = make_double2(fma(s2, t4.x, s1 * t3.x), fma(s2, t4.y, s1 * t3.y));
  double2 b2 = make_double2(fma(-s1, t4.x, s2 * t3.x), fma(-s1, t4.y, s2 * t3.y));
  v[0] = make_double2(x0.x + t1.x + t2.x, x0.y + t1.y + t2.y);
  v[1] = make_double2(a1.x - b1.y, a1.y + b1.x);
  v[4] = make_double2(a1.x + b1.y, a1.y - b1.x);
  v[2] = make_double2(a2.x - b2.y, a2.y + b2.x);
  v[3] = make_double2(a2.x + b2.y, a2.y - b2.x);
}

// w16^k * a for k = 1, 3 (general rotations), sign-aware
template <bool FWD> __device__ __forceinline__ double2 rot16(double2 a, double c, double s) {
  // multiply by (c + i*sg*s) with sg = -1 forward
  const double ss = FWD ? -s : s;
  return make_double2(fma(a.x, c, -a.y * ss), fma(a.x, ss, a.y * c));
}

template <bool FWD> __device__ __forceinline__ void bfly16(double2* v) {
  // 16 = 4 x 4: four radix-4 over q = r + 4 p (p = 0..3), twiddles w16^(r k1), four radix-4
  double2 a[16];
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    double2 x0 = v[r], x1 = v[r + 4], x2 = v[r + 8], x3 = v[r + 12];
    bfly4<FWD>(x0, x1, x2, x3);  // outputs k1 = 0,1,2,3
    a[r * 4 + 0] = x0;
    a[r * 4 + 1] = x1;
    a[r * 4 + 2] = x2;
    a[r * 4 + 3] = x3;
  }
  // twiddle a[r*4 + k1] by w16^(r k1)
  a[1 * 4 + 1] = rot16<FWD>(a[1 * 4 + 1], QSF_C16_1, QSF_S16_1);  // w^1
  a[1 * 4 + 2] = w8_1<FWD>(a[1 * 4 + 2]);                         // w^2
  a[1 * 4 + 3] = rot16<FWD>(a[1 * 4 + 3], QSF_S16_1, QSF_C16_1);  // w^3
  a[2 * 4 + 1] = w8_1<FWD>(a[2 * 4 + 1]);                         // w^2
  a[2 * 4 + 2] = mul_si<FWD>(a[2 * 4 + 2]);                       // w^4
  a[2 * 4 + 3] = w8_3<FWD>(a[2 * 4 + 3]);                         // w^6
  a[3 * 4 + 1] = rot16<FWD>(a[3 * 4 + 1], QSF_S16_1, QSF_C16_1);  // w^3
  a[3 * 4 + 2] = w8_3<FWD>(a[3 * 4 + 2]);                         // w^6
  a[3 * 4 + 3] = rot16<FWD>(a[3 * 4 + 3], -QSF_C16_1, -QSF_S16_1); // w^9 = -w^1
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) {
    double2 x0 = a[0 * 4 + k1], x1 = a[1 * 4 + k1], x2 = a[2 * 4 + k1], x3 = a[3 * 4 + k1];
    bfly4<FWD>(x0, x1, x2, x3);  // outputs k2 = 0..3 -> k = k1 + 4 k2
    v[k1 + 0] = x0;
    v[k1 + 4] = x1;
    v[k1 + 8] = x2;
    v[k1 + 12] = x3;
  }
}

template <int R, bool FWD> __device__ __forceinline__ void bfly(double2* v) {
  if constexpr (R == 2) bfly2<FWD>(v[0], v[1]);
  else if constexpr (R == 3) bfly3<FWD>(v);
  else if constexpr (R == 4) bfly4<FWD>(v[0], v[1], v[2], v[3]);
  else if constexpr (R == 5) bfly5<FWD>(v);
  else if constexpr (R == 8) bfly8<FWD>(v);
  else if constexpr (R == 16) bfly16<FWD>(v);
}

// Lines in shared memory: element e of line l sits at buf[l * ls + e * es].
struct LineSet {
  int nlines;
  int ls;
  int es;
  bool line_fastest;  // work-item order: consecutive threads take consecutive lines
};

// ---------------------------------------------------------------------------
// Compile-time radix plans.  A line of N = 2^a 3^b 5^c points is transformed by
// floor(a/4) radix-16 passes, one radix 2/4/8 pass for the rest of 2^a, then the
// radix-3 and radix-5 passes.  The first pass needs no twiddles, so radix 16 goes
// first.  Static plans keep every pass straight-line code with constant strides, so
// register allocation stays per pass (a runtime switch over radices merges live
// ranges and spills).
__host__ __device__ constexpr int count_factor(int n, int f) {
  int c = 0;
  while (n % f == 0) {
    n /= f;
    ++c;
  }
  return c;
}
__host__ __device__ constexpr bool is_smooth(int n) {
  int v = n;
  while (v % 2 == 0) v /= 2;
  while (v % 3 == 0) v /= 3;
  while (v % 5 == 0) v /= 5;
  return v == 1 && n > 1;
}
// log2 of the largest power-of-two radix of the plans (16)
#ifndef QSF_RADIX_LOG2
#define QSF_RADIX_LOG2 4
#endif
// Stage plan of an n-point transform: passes of radix 2^l2 (the main radix), one pass
// of the remaining power of two, then radix-3 and radix-5 passes.
__host__ __device__ constexpr int nstages(int n, int l2 = QSF_RADIX_LOG2) {
  const int a = count_factor(n, 2);
  return a / l2 + (a % l2 ? 1 : 0) + count_factor(n, 3) + count_factor(n, 5);
}
__host__ __device__ constexpr int radix_at(int n, int i, int l2 = QSF_RADIX_LOG2) {
  const int a = count_factor(n, 2);
  const int q = a / l2, r = a % l2;
  if (i < q) return 1 << l2;
  int k = i - q;
  if (r) {
    if (k == 0) return 1 << r;
    k -= 1;
  }
  return k < count_factor(n, 3) ? 3 : 5;
}
__host__ __device__ constexpr int ns_at(int n, int i, int l2 = QSF_RADIX_LOG2) {
  int p = 1;
  for (int j = 0; j < i; ++j) p *= radix_at(n, j, l2);
  return p;
}
// butterflies per thread for radix R when lines * N <= 16 * nth
__host__ __device__ constexpr int maxb_for(int r) { return r == 16 ? 1 : r == 8 ? 2 : r == 5 ? 4 : r == 4 ? 4 : r == 3 ? 6 : 8; }

template <int R, bool FWD, int MAXB, int N, int NS>
__device__ __forceinline__ void stockham_static(double2* __restrict__ buf, const LineSet& L,
                                                const double2* __restrict__ tw, int tid, int nth) {
  constexpr int nr = N / R;
  constexpr int twstep = N / (NS * R);
  const int total = nr * L.nlines;
  double2 v[MAXB][R];
  int dsto[MAXB];
#pragma unroll
  for (int b = 0; b < MAXB; ++b) {
    const int w = tid + b * nth;
    dsto[b] = -1;
    if (w < total) {
      int line, j;
      if (L.line_fastest) {
        line = w % L.nlines;
        j = w / L.nlines;
      } else {
        j = w % nr;
        line = w / nr;
      }
      const double2* src = buf + line * L.ls;
#pragma unroll
      for (int q = 0; q < R; ++q) v[b][q] = src[(j + q * nr) * L.es];
      const int jm = j % NS;
      if constexpr (NS > 1) {
#pragma unroll
        for (int q = 1; q < R; ++q) {
          double2 t = __ldg(&tw[jm * q * twstep]);
          if (!FWD) t.y = -t.y;
          v[b][q] = cmul(v[b][q], t);
        }
      }
      dsto[b] = line * L.ls + ((j - jm) * R + jm) * L.es;
    }
  }
  __syncthreads();
#pragma unroll
  for (int b = 0; b < MAXB; ++b) {
    if (dsto[b] >= 0) {
      bfly<R, FWD>(v[b]);
      double2* dst = buf + dsto[b];
      const int st = NS * L.es;
#pragma unroll
      for (int q = 0; q < R; ++q) dst[q * st] = v[b][q];
    }
  }
  __syncthreads();
}

// In-place transform of every line of the set.  The caller has written the lines and
// barrier'd; requires nlines * N <= 16 * nth.  Data is in `buf` on return.
template <int N, bool FWD, int S = 0>
__device__ __forceinline__ void fft_static(double2* buf, const LineSet& L, const double2* __restrict__ tw, int tid,
                                           int nth) {
  if constexpr (S < nstages(N)) {
    constexpr int R = radix_at(N, S);
    stockham_static<R, FWD, maxb_for(R), N, ns_at(N, S)>(buf, L, tw, tid, nth);
    fft_static<N, FWD, S + 1>(buf, L, tw, tid, nth);
  }
}

}  // namespace qsf
