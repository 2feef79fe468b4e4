// qsf_fxfft.cuh -- block-fixed-point (int64) Stockham FFT for sm_103a.
//
// GB300 issues about 2 FP64 instructions per clock per SM but ~128 integer
// instructions, so the split step's FFTs run on the integer pipes: a line (or a tile
// of lines) is held as 64-bit integers sharing one power-of-two block exponent,
// value = int * 2^-scale.  Additions are exact; products by twiddles and butterfly
// constants (62 fractional bits) keep the top 64 bits of the 124-bit product to within
// 1.5 units, from three 32 x 32 -> 64-bit partial products.  After every radix pass the
// block is renormalised so that its largest component again uses all bits the next
// pass can afford (62 minus the pass's growth), i.e. block floating point with a 55-60
// bit mantissa at every pass.  Against an exact DFT this is ~3.5x more accurate than an
// FP64 FFT (normwise relative error ~6e-17 vs ~2.3e-16 at N = 48 .. 2048); FP64
// storage of psi is unchanged.
//
// Radix plans, pass structure and index maps are those of qsf_fft.cuh.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "qsf_fft.cuh"

namespace qsf {

typedef long long i64;
typedef unsigned long long u64;

// a * w / 2^62 for w in 2^62 fixed point, from three signed 32 x 32 -> 64-bit partial
// products (IMAD.WIDE): both operands are split into a high word and a signed low
// word, x = xh 2^32 + xl with xl in [-2^31, 2^31); the low x low product (at most one
// unit of the result) is dropped and the middle terms are rounded, so the result lies
// within 1.5 units of the exact quotient.  Needs |a|, |w| < 2^62.5.
__device__ __forceinline__ i64 mulq62(i64 a, i64 w) {
  const int al = (int)a, wl = (int)w;
  const int ah = (int)((a - (i64)al) >> 32), wh = (int)((w - (i64)wl) >> 32);
  const i64 mid = (i64)ah * wl + (i64)al * wh + (1LL << 29);
  return (i64)(((u64)((i64)ah * wh) << 2) + (u64)(mid >> 30));
}

__device__ __forceinline__ longlong2 fadd(longlong2 a, longlong2 b) { return make_longlong2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ longlong2 fsub(longlong2 a, longlong2 b) { return make_longlong2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ longlong2 fconj(longlong2 a) { return make_longlong2(a.x, -a.y); }
// a * w with w in 2^62 fixed point (|w| <= 1, components of a below 2^62): three
// rounded products (Gauss / Karatsuba): re = c(a+b) - b(c+d), im = c(a+b) + a(d-c)
__device__ __forceinline__ longlong2 fmul62(longlong2 a, longlong2 w) {
  const i64 k1 = mulq62(a.x + a.y, w.x);
  const i64 k2 = mulq62(a.x, w.y - w.x);
  const i64 k3 = mulq62(a.y, w.x + w.y);
  return make_longlong2(k1 - k3, k1 + k2);
}
// Twiddle products from pre-split tables (QSF_TWQ, the default).  A twiddle w in 2^62
// fixed point is stored as the signed 32-bit halves of each component, w = wh 2^32 + wl
// with wl = (int)w (int4 {re lo, re hi, im lo, im hi}; the host keeps every low half
// away from -2^31 so that it can be negated).  The complex product a * w / 2^64 takes
// the four high x high products exactly, sums the eight middle products of each output
// component in one 64-bit word (rounded at bit 32) and drops the four low x low ones:
// within 1 unit of the exact quotient, from twelve 32 x 32 -> 64-bit multiply-adds and
// no 64-bit shifts.  Callers pre-scale a by 4 (components below 2^61), so the product
// comes out at the scale of an untwiddled element.
#ifndef QSF_TWQ
#define QSF_TWQ 1
#endif
// the high half of the signed split x = hi 2^32 + (int)x
__device__ __forceinline__ int split_hi(i64 x) { return (int)(x >> 32) + (int)((unsigned)x >> 31); }
__device__ __forceinline__ longlong2 fmul_tw(longlong2 a, int4 w) {
  const int axl = (int)a.x, axh = split_hi(a.x), ayl = (int)a.y, ayh = split_hi(a.y);
  const int nyl = -w.z, nyh = -w.w;
  i64 rm = (1LL << 31), im = (1LL << 31);
  rm += (i64)axh * w.x;
  rm += (i64)axl * w.y;
  rm += (i64)ayh * nyl;
  rm += (i64)ayl * nyh;
  im += (i64)axh * w.z;
  im += (i64)axl * w.w;
  im += (i64)ayh * w.x;
  im += (i64)ayl * w.y;
  i64 re = rm >> 32, ii = im >> 32;
  re += (i64)axh * w.y;
  re += (i64)ayh * nyh;
  ii += (i64)axh * w.w;
  ii += (i64)ayh * w.y;
  return make_longlong2(re, ii);
}
// the signed 32-bit halves of a compile-time 64-bit constant
__host__ __device__ constexpr int k_lo(i64 c) {
  return (int)((c & 0xffffffffLL) >= 0x80000000LL ? (c & 0xffffffffLL) - 0x100000000LL : (c & 0xffffffffLL));
}
__host__ __device__ constexpr int k_hi(i64 c) { return (int)((c - (i64)k_lo(c)) >> 32); }
// a * C / 2^64 for a compile-time C (|C| < 2^63, |a| < 2^62): three multiply-adds,
// within 0.75 units
template <i64 C>
__device__ __forceinline__ i64 mulk64(i64 a) {
  constexpr int cl = k_lo(C), ch = k_hi(C);
  const int al = (int)a, ah = split_hi(a);
  const i64 m = (i64)ah * cl + (i64)al * ch + (1LL << 31);
  return (m >> 32) + (i64)ah * ch;
}
// a * c for a constant c = C / 2^63 (|c| < 1): within 1.5 units
template <i64 C>
__device__ __forceinline__ i64 mulk63(i64 a) { return (i64)((u64)mulk64<C>(a) << 1); }
// a * (CR + i CI) / 2^63 for compile-time constants: the complex form of mulk64 (merged
// middle words), doubled; within 2 units per component
template <i64 CR, i64 CI>
__device__ __forceinline__ longlong2 fmulk63(longlong2 a) {
  constexpr int rl = k_lo(CR), rh = k_hi(CR), il = k_lo(CI), ih = k_hi(CI), nl = k_lo(-CI), nh = k_hi(-CI);
  const int axl = (int)a.x, axh = split_hi(a.x), ayl = (int)a.y, ayh = split_hi(a.y);
  i64 rm = (1LL << 31), im = (1LL << 31);
  rm += (i64)axh * rl;
  rm += (i64)axl * rh;
  rm += (i64)ayh * nl;
  rm += (i64)ayl * nh;
  im += (i64)axh * il;
  im += (i64)axl * ih;
  im += (i64)ayh * rl;
  im += (i64)ayl * rh;
  i64 re = rm >> 32, ii = im >> 32;
  re += (i64)axh * rh;
  re += (i64)ayh * nh;
  ii += (i64)axh * ih;
  ii += (i64)ayh * rh;
  return make_longlong2((i64)((u64)re << 1), (i64)((u64)ii << 1));
}
// butterfly constants in 2^63 fixed point (|c| < 1)
#define QSF_K63_SQRT1_2 6521908912666391106LL   /* round(2^63 / sqrt(2)) */
#define QSF_K63_C16_1 8521284645587064995LL     /* round(2^63 cos(pi/8)) */
#define QSF_K63_S16_1 3529631669043774883LL     /* round(2^63 sin(pi/8)) */
#define QSF_K63_SQRT3_2 7987674492471257551LL   /* round(2^63 sqrt(3)/2) */
#define QSF_K63_C5_1 2850178704830799621LL      /* round(2^63 cos(2pi/5)) */
#define QSF_K63_C5_2 (-7461864723258187525LL)   /* round(2^63 cos(4pi/5)) */
#define QSF_K63_S5_1 8771948077865237882LL      /* round(2^63 sin(2pi/5)) */
#define QSF_K63_S5_2 5421362059670026167LL      /* round(2^63 sin(4pi/5)) */

// OR of the component magnitudes (x ^ (x >> 63) is |x| or |x| - 1): its bit length is
// the block maximum's bit length, or one less when that maximum is a negative power of two
__device__ __forceinline__ u64 fmag(longlong2 x) { return (u64)(x.x ^ (x.x >> 63)) | (u64)(x.y ^ (x.y >> 63)); }
__device__ __forceinline__ int bitlen(u64 v) { return 64 - __clzll((long long)v); }
// the same from the high words alone (32-bit operations): 32 + the high words' bit
// length, or 0 when every component is below 2^32 in magnitude
__device__ __forceinline__ unsigned fmag_hi(longlong2 x) {
  const int hx = (int)(x.x >> 32), hy = (int)(x.y >> 32);
  return (unsigned)(hx ^ (hx >> 31)) | (unsigned)(hy ^ (hy >> 31));
}
__device__ __forceinline__ int bitlen_hi(unsigned v) { return v ? 64 - __clz((int)v) : 0; }
template <bool FWD> __device__ __forceinline__ longlong2 fmul_si(longlong2 a) {
  return FWD ? make_longlong2(a.y, -a.x) : make_longlong2(-a.y, a.x);
}

// butterfly constants in 2^62 fixed point
#define QSF_FX_SQRT1_2 3260954456333195553LL   /* round(2^62 / sqrt(2)) */
#define QSF_FX_SQRT3_2 3993837246235628775LL   /* round(2^62 * sqrt(3)/2) */
#define QSF_FX_HALF 2305843009213693952LL      /* 2^61 */
#define QSF_FX_C5_1 1425089352415399811LL      /* round(2^62 * cos(2pi/5)) */
#define QSF_FX_C5_2 (-3730932361629093763LL)   /* round(2^62 * cos(4pi/5)) */
#define QSF_FX_S5_1 4385974038932618941LL      /* round(2^62 * sin(2pi/5)) */
#define QSF_FX_S5_2 2710681029835013083LL      /* round(2^62 * sin(4pi/5)) */
#define QSF_FX_C16_1 4260642322793532497LL     /* round(2^62 * cos(pi/8)) */
#define QSF_FX_S16_1 1764815834521887442LL     /* round(2^62 * sin(pi/8)) */

template <bool FWD> __device__ __forceinline__ void fbfly2(longlong2& a, longlong2& b) {
  const longlong2 t = a;
  a = fadd(t, b);
  b = fsub(t, b);
}
template <bool FWD>
__device__ __forceinline__ void fbfly4(longlong2& x0, longlong2& x1, longlong2& x2, longlong2& x3) {
  const longlong2 t0 = fadd(x0, x2), t1 = fsub(x0, x2), t2 = fadd(x1, x3), t3 = fmul_si<FWD>(fsub(x1, x3));
  x0 = fadd(t0, t2);
  x2 = fsub(t0, t2);
  x1 = fadd(t1, t3);
  x3 = fsub(t1, t3);
}
// w8^1 * a and w8^3 * a, w8 = exp(sign 2 pi i / 8)
#if QSF_TWQ
__device__ __forceinline__ i64 mul_sqrt1_2(i64 a) { return mulk63<QSF_K63_SQRT1_2>(a); }
#else
__device__ __forceinline__ i64 mul_sqrt1_2(i64 a) { return mulq62(a, QSF_FX_SQRT1_2); }
#endif
template <bool FWD> __device__ __forceinline__ longlong2 fw8_1(longlong2 a) {
  return FWD ? make_longlong2(mul_sqrt1_2(a.x + a.y), mul_sqrt1_2(a.y - a.x))
             : make_longlong2(mul_sqrt1_2(a.x - a.y), mul_sqrt1_2(a.x + a.y));
}
template <bool FWD> __device__ __forceinline__ longlong2 fw8_3(longlong2 a) {
  return FWD ? make_longlong2(mul_sqrt1_2(a.y - a.x), -mul_sqrt1_2(a.x + a.y))
             : make_longlong2(-mul_sqrt1_2(a.x + a.y), mul_sqrt1_2(a.x - a.y));
}
template <bool FWD> __device__ __forceinline__ void fbfly8(longlong2* v) {
  longlong2 a0 = fadd(v[0], v[4]), a4 = fsub(v[0], v[4]);
  longlong2 a1 = fadd(v[1], v[5]), a5 = fsub(v[1], v[5]);
  longlong2 a2 = fadd(v[2], v[6]), a6 = fsub(v[2], v[6]);
  longlong2 a3 = fadd(v[3], v[7]), a7 = fsub(v[3], v[7]);
  a5 = fw8_1<FWD>(a5);
  a6 = fmul_si<FWD>(a6);
  a7 = fw8_3<FWD>(a7);
  fbfly4<FWD>(a0, a1, a2, a3);
  fbfly4<FWD>(a4, a5, a6, a7);
  v[0] = a0; v[4] = a2; v[2] = a1; v[6] = a3;
  v[1] = a4; v[5] = a6; v[3] = a5; v[7] = a7;
}
template <bool FWD> __device__ __forceinline__ void fbfly3(longlong2* v) {
  const longlong2 t1 = fadd(v[1], v[2]), t2 = fsub(v[1], v[2]);
  // m1 = v0 - t1/2 ; X1 = m1 + i k t2, X2 = m1 - i k t2, k = sign * sqrt(3)/2
#if QSF_TWQ
  const longlong2 m1 = make_longlong2(v[0].x - ((t1.x + 1) >> 1), v[0].y - ((t1.y + 1) >> 1));
  const i64 kx = mulk63<QSF_K63_SQRT3_2>(t2.x), ky = mulk63<QSF_K63_SQRT3_2>(t2.y);
#else
  const longlong2 m1 = make_longlong2(v[0].x - mulq62(t1.x, QSF_FX_HALF), v[0].y - mulq62(t1.y, QSF_FX_HALF));
  const i64 kx = mulq62(t2.x, QSF_FX_SQRT3_2), ky = mulq62(t2.y, QSF_FX_SQRT3_2);
#endif
  v[0] = fadd(v[0], t1);
  if (FWD) {  // k = -sqrt3/2
    v[1] = make_longlong2(m1.x + ky, m1.y - kx);
    v[2] = make_longlong2(m1.x - ky, m1.y + kx);
  } else {
    v[1] = make_longlong2(m1.x - ky, m1.y + kx);
    v[2] = make_longlong2(m1.x + ky, m1.y - kx);
  }
}
template <bool FWD> __device__ __forceinline__ void fbfly5(longlong2* v) {
  const longlong2 t1 = fadd(v[1], v[4]), t2 = fadd(v[2], v[3]), t3 = fsub(v[1], v[4]), t4 = fsub(v[2], v[3]);
  const longlong2 x0 = v[0];
#if QSF_TWQ
#define QSF_M5(x, K) mulk63<QSF_K63_##K>(x)
#else
#define QSF_M5(x, K) mulq62(x, QSF_FX_##K)
#endif
  const longlong2 a1 = make_longlong2(x0.x + QSF_M5(t1.x, C5_1) + QSF_M5(t2.x, C5_2),
                                      x0.y + QSF_M5(t1.y, C5_1) + QSF_M5(t2.y, C5_2));
  const longlong2 a2 = make_longlong2(x0.x + QSF_M5(t1.x, C5_2) + QSF_M5(t2.x, C5_1),
                                      x0.y + QSF_M5(t1.y, C5_2) + QSF_M5(t2.y, C5_1));
  // b1 = s1 t3 + s2 t4, b2 = s2 t3 - s1 t4 with s = sign * sin
  longlong2 b1 = make_longlong2(QSF_M5(t3.x, S5_1) + QSF_M5(t4.x, S5_2), QSF_M5(t3.y, S5_1) + QSF_M5(t4.y, S5_2));
  longlong2 b2 = make_longlong2(QSF_M5(t3.x, S5_2) - QSF_M5(t4.x, S5_1), QSF_M5(t3.y, S5_2) - QSF_M5(t4.y, S5_1));
#undef QSF_M5
  if (FWD) {
    b1 = make_longlong2(-b1.x, -b1.y);
    b2 = make_longlong2(-b2.x, -b2.y);
  }
  v[0] = make_longlong2(x0.x + t1.x + t2.x, x0.y + t1.y + t2.y);
  v[1] = make_longlong2(a1.x - b1.y, a1.y + b1.x);
  v[4] = make_longlong2(a1.x + b1.y, a1.y - b1.x);
  v[2] = make_longlong2(a2.x - b2.y, a2.y + b2.x);
  v[3] = make_longlong2(a2.x + b2.y, a2.y - b2.x);
}
// multiply by (c + i sign s) in 2^62 fixed point (three products)
template <bool FWD> __device__ __forceinline__ longlong2 frot(longlong2 a, i64 c, i64 s) {
  return fmul62(a, make_longlong2(c, FWD ? -s : s));
}
template <bool FWD> __device__ __forceinline__ void fbfly16(longlong2* v) {
  longlong2 a[16];
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    longlong2 x0 = v[r], x1 = v[r + 4], x2 = v[r + 8], x3 = v[r + 12];
    fbfly4<FWD>(x0, x1, x2, x3);
    a[r * 4 + 0] = x0;
    a[r * 4 + 1] = x1;
    a[r * 4 + 2] = x2;
    a[r * 4 + 3] = x3;
  }
#if QSF_TWQ
  constexpr i64 sg = FWD ? -1 : 1;
  a[1 * 4 + 1] = fmulk63<QSF_K63_C16_1, sg * QSF_K63_S16_1>(a[1 * 4 + 1]);     // w^1
  a[1 * 4 + 3] = fmulk63<QSF_K63_S16_1, sg * QSF_K63_C16_1>(a[1 * 4 + 3]);     // w^3
  a[3 * 4 + 1] = fmulk63<QSF_K63_S16_1, sg * QSF_K63_C16_1>(a[3 * 4 + 1]);     // w^3
  a[3 * 4 + 3] = fmulk63<-QSF_K63_C16_1, -sg * QSF_K63_S16_1>(a[3 * 4 + 3]);   // w^9
#else
  a[1 * 4 + 1] = frot<FWD>(a[1 * 4 + 1], QSF_FX_C16_1, QSF_FX_S16_1);    // w^1
  a[1 * 4 + 3] = frot<FWD>(a[1 * 4 + 3], QSF_FX_S16_1, QSF_FX_C16_1);    // w^3
  a[3 * 4 + 1] = frot<FWD>(a[3 * 4 + 1], QSF_FX_S16_1, QSF_FX_C16_1);    // w^3
  a[3 * 4 + 3] = frot<FWD>(a[3 * 4 + 3], -QSF_FX_C16_1, -QSF_FX_S16_1);  // w^9
#endif
  a[1 * 4 + 2] = fw8_1<FWD>(a[1 * 4 + 2]);                              // w^2
  a[2 * 4 + 1] = fw8_1<FWD>(a[2 * 4 + 1]);                              // w^2
  a[2 * 4 + 2] = fmul_si<FWD>(a[2 * 4 + 2]);                            // w^4
  a[2 * 4 + 3] = fw8_3<FWD>(a[2 * 4 + 3]);                              // w^6
  a[3 * 4 + 2] = fw8_3<FWD>(a[3 * 4 + 2]);                              // w^6
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) {
    longlong2 x0 = a[0 * 4 + k1], x1 = a[1 * 4 + k1], x2 = a[2 * 4 + k1], x3 = a[3 * 4 + k1];
    fbfly4<FWD>(x0, x1, x2, x3);
    v[k1 + 0] = x0;
    v[k1 + 4] = x1;
    v[k1 + 8] = x2;
    v[k1 + 12] = x3;
  }
}
template <int R, bool FWD> __device__ __forceinline__ void fbfly(longlong2* v) {
  if constexpr (R == 2) fbfly2<FWD>(v[0], v[1]);
  else if constexpr (R == 3) fbfly3<FWD>(v);
  else if constexpr (R == 4) fbfly4<FWD>(v[0], v[1], v[2], v[3]);
  else if constexpr (R == 5) fbfly5<FWD>(v);
  else if constexpr (R == 8) fbfly8<FWD>(v);
  else if constexpr (R == 16) fbfly16<FWD>(v);
}

// bit length of |x| (0 for x == 0)
__device__ __forceinline__ int fbits(i64 x) {
  const u64 a = (u64)(x < 0 ? -x : x);
  return 64 - __clzll((long long)a);
}
// x * 2^sh with rounding (sh < 0: arithmetic right shift, round half up)
__device__ __forceinline__ i64 fshift(i64 x, int sh) {
  if (sh >= 0) return x << sh;
  const int r = -sh;
  if (r >= 63) return 0;
  return (x + ((i64)1 << (r - 1))) >> r;
}
// guard bits a radix-R pass needs above the block maximum (growth <= R * sqrt(2))
__host__ __device__ constexpr int fguard(int r) { return r == 16 ? 5 : r == 8 ? 4 : r == 5 ? 4 : r == 4 ? 3 : r == 3 ? 3 : 2; }

// Block-wide max of per-thread values over one barrier: every warp's maximum goes to
// slot[warp], then all threads read the slots.  The slots are reused only after at
// least one further barrier (the FFT passes alternate between two slot arrays).
__device__ __forceinline__ int block_max_once(int v, int* slot) {
  v = __reduce_max_sync(0xffffffffu, (unsigned)v);
  if ((threadIdx.x & 31) == 0) slot[threadIdx.x >> 5] = v;
  __syncthreads();
  const int nw = (blockDim.x + 31) >> 5;
  int m = 0;
  for (int w = 0; w < nw; ++w) m = max(m, slot[w]);
  return m;
}

// Block-wide max of per-thread values (red[0..31]); result returned to all.  The
// shared arrays named red in the kernels hold kRedInts ints: [0, 32) for this function,
// [32, 96) for the alternating slots of the FFT passes.
constexpr int kRedInts = 96;
__device__ __forceinline__ int block_max_int(int v, int* red) {
  v = __reduce_max_sync(0xffffffffu, (unsigned)v);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  if (lane == 0) red[wid] = v;
  __syncthreads();
  int m = 0;
  for (int w = 0; w < nw; ++w) m = max(m, red[w]);
  __syncthreads();
  return m;
}

// One in-place forward Stockham pass in fixed point (an inverse transform is the
// forward one between two conjugations) with stride NS (the product of the earlier
// radices; a runtime value, so that passes of equal radix share one code body).
// Inputs are scaled by 2^shift_in on load; returns, valid in every thread after the
// call, the bit length of the block's largest output component (see fmag).
template <class TW>
struct tw_is_split {
  static constexpr bool value = false;
};
template <>
struct tw_is_split<int4> {
  static constexpr bool value = true;
};
// a pre-split twiddle back in one 64-bit word per component
__device__ __forceinline__ longlong2 tw_join(int4 w) {
  return make_longlong2((i64)((u64)(i64)w.y << 32) + (i64)w.x, (i64)((u64)(i64)w.w << 32) + (i64)w.z);
}

template <int R, int MAXB, int N, class TW>
__device__ __forceinline__ int fx_stockham(longlong2* __restrict__ buf, const LineSet& L, const TW* __restrict__ tw,
                                           int tid, int nth, int shift_in, int* red, int parity, int NS) {
  constexpr int nr = N / R;
  constexpr bool kSplit = tw_is_split<TW>::value && R > 2;
  const int twstep = N / (NS * R);
  const int total = nr * L.nlines;
  // the load-time scaling 2^shift_in without branches: (x << sl + half) >> sr; with
  // pre-split twiddles the elements that get one (q >= 1 of a pass after the first)
  // are loaded 2 bits higher (sl2 / sr2), since their product is a * w / 2^64
  const int sl = shift_in > 0 ? shift_in : 0, sr = shift_in < 0 ? min(-shift_in, 63) : 0;
  const i64 half = sr ? (i64)1 << (sr - 1) : 0;
  const int shift_q = (kSplit && NS > 1) ? shift_in + 2 : shift_in;
  const int sl2 = shift_q > 0 ? shift_q : 0, sr2 = shift_q < 0 ? min(-shift_q, 63) : 0;
  const i64 half2 = sr2 ? (i64)1 << (sr2 - 1) : 0;
  // index maps without divisions where the counts are powers of two
  const bool ns_pow2 = (NS & (NS - 1)) == 0;
  const bool nl_pow2 = (L.nlines & (L.nlines - 1)) == 0;
  const int nl_sh = __ffs(L.nlines) - 1;
  longlong2 v[MAXB][R];
  int dsto[MAXB];
#pragma unroll
  for (int b = 0; b < MAXB; ++b) {
    const int w = tid + b * nth;
    dsto[b] = -1;
    if (w < total) {
      int line, j;
      if (L.line_fastest) {
        line = nl_pow2 ? (w & (L.nlines - 1)) : w % L.nlines;
        j = nl_pow2 ? (w >> nl_sh) : w / L.nlines;
      } else {
        j = w % nr;
        line = w / nr;
      }
      const longlong2* src = buf + line * L.ls;
#pragma unroll
      for (int q = 0; q < R; ++q) {
        const longlong2 x = src[(j + q * nr) * L.es];
        if (q == 0)
          v[b][q] = make_longlong2(((i64)((u64)x.x << sl) + half) >> sr, ((i64)((u64)x.y << sl) + half) >> sr);
        else
          v[b][q] = make_longlong2(((i64)((u64)x.x << sl2) + half2) >> sr2, ((i64)((u64)x.y << sl2) + half2) >> sr2);
      }
      const int jm = ns_pow2 ? (j & (NS - 1)) : j % NS;
      if (NS > 1) {
#pragma unroll
        for (int q = 1; q < R; ++q) {
          if constexpr (kSplit) v[b][q] = fmul_tw(v[b][q], tw[jm * q * twstep]);
          else if constexpr (tw_is_split<TW>::value) v[b][q] = fmul62(v[b][q], tw_join(tw[jm * q * twstep]));
          else v[b][q] = fmul62(v[b][q], tw[jm * q * twstep]);
        }
      }
      dsto[b] = line * L.ls + ((j - jm) * R + jm) * L.es;
    }
  }
  __syncthreads();
  unsigned mag = 0;
#pragma unroll
  for (int b = 0; b < MAXB; ++b) {
    if (dsto[b] >= 0) {
      fbfly<R, true>(v[b]);
      longlong2* dst = buf + dsto[b];
      const int st = NS * L.es;
#pragma unroll
      for (int q = 0; q < R; ++q) {
        dst[q * st] = v[b][q];
        mag |= fmag_hi(v[b][q]);
      }
    }
  }
  int bits = block_max_once(bitlen_hi(mag), red + 32 + 32 * parity);  // its barrier ends the pass
  if (bits == 0) {  // every component below 2^32 (rare): bit length from the full words
    u64 m64 = 0;
#pragma unroll
    for (int b = 0; b < MAXB; ++b)
      if (dsto[b] >= 0)
#pragma unroll
        for (int q = 0; q < R; ++q) m64 |= fmag(v[b][q]);
    bits = block_max_int(bitlen(m64), red);
  }
  return bits;
}

// Full forward fixed-point transform of every line of the set, in place.  On entry
// the data have block exponent `scale` (value = int * 2^-scale) and, after the shift
// 2^shift_in applied on load, fit the first pass's guard; on return `scale` is the
// exponent of the output and its largest component has bit length `bits`.
// Requires nlines * N <= 16 * nth.  The passes run as a loop over the stages with one
// inlined pass body per distinct radix of N (instruction-cache footprint).
// radix_at(N, s, L2) for a runtime stage index, from compile-time stage counts
template <int N, int L2>
__device__ __forceinline__ int radix_rt(int s) {
  constexpr int a = count_factor(N, 2), q = a / L2, rem = a % L2;
  constexpr int c3 = count_factor(N, 3);
  if (s < q) return 1 << L2;
  int k = s - q;
  if (rem) {
    if (k == 0) return 1 << rem;
    k -= 1;
  }
  return k < c3 ? 3 : 5;
}
// butterflies per thread of radix R when every thread holds PPT points of the tile
__host__ __device__ constexpr int maxb_ppt(int r, int ppt) { return (ppt + r - 1) / r; }

// main radix of the plan for PPT points per thread: radix 16 needs 16 per thread,
// radix 8 needs 8, radix 4 four
__host__ __device__ constexpr int plan_l2(int ppt) { return ppt >= 16 ? QSF_RADIX_LOG2 : ppt >= 8 ? 3 : 2; }

// the compile-time stages S.. of fft_fx
template <int N, int S, int PPT, class TW>
__device__ __forceinline__ void fft_fx_tail(longlong2* buf, const LineSet& L, const TW* __restrict__ tw,
                                            int tid, int nth, int& scale, int& bits, int* red, int shift_in) {
  constexpr int L2 = plan_l2(PPT);
  if constexpr (S < nstages(N, L2)) {
    constexpr int R = radix_at(N, S, L2);
    bits = fx_stockham<R, maxb_ppt(R, PPT), N>(buf, L, tw, tid, nth, shift_in, red, S & 1, ns_at(N, S, L2));
    if constexpr (S + 1 < nstages(N, L2)) {
      // renormalise for the next pass: largest component below 2^(62 - guard(next))
      const int target = 62 - fguard(radix_at(N, S + 1, L2));
      const int sh = bits == 0 ? 0 : target - bits;
      scale += sh;
      fft_fx_tail<N, S + 1, PPT>(buf, L, tw, tid, nth, scale, bits, red, sh);
    }
  }
}
// PPT: points of the tile per thread (tile points / threads), which sets the butterflies
// each thread carries per pass.
template <int N, int PPT = 16, class TW = longlong2>
__device__ __forceinline__ void fft_fx(longlong2* buf, const LineSet& L, const TW* __restrict__ tw, int tid,
                                       int nth, int& scale, int& bits, int* red, int shift_in = 0) {
  // the leading passes of the plan's main radix share one code body (a loop); the rest
  // are unrolled
  constexpr int L2 = plan_l2(PPT);
  constexpr int R0 = 1 << L2;
  constexpr int q = count_factor(N, 2) / L2;
  if constexpr (q >= 2) {
    int sh = shift_in, ns = 1;
#pragma unroll 1
    for (int s = 0; s < q; ++s) {
      bits = fx_stockham<R0, maxb_ppt(R0, PPT), N>(buf, L, tw, tid, nth, sh, red, s & 1, ns);
      ns *= R0;
      if (s + 1 < nstages(N, L2)) {
        const int target = 62 - fguard(radix_rt<N, L2>(s + 1));
        sh = bits == 0 ? 0 : target - bits;
        scale += sh;
      }
    }
    fft_fx_tail<N, q, PPT>(buf, L, tw, tid, nth, scale, bits, red, sh);
  } else {
    fft_fx_tail<N, 0, PPT>(buf, L, tw, tid, nth, scale, bits, red, shift_in);
  }
}

// Exponent bits of a double's magnitude (0 for 0 / denormals)
__device__ __forceinline__ int dexp(double x) { return (int)((__double_as_longlong(x) >> 52) & 0x7ff); }

// round(x * 2^s) as int64 using integer operations only (x finite, result < 2^63)
__device__ __forceinline__ i64 d2fx(double x, int s) {
  const u64 b = (u64)__double_as_longlong(x);
  const int e = (int)((b >> 52) & 0x7ff);
  if (e == 0) return 0;  // zero or denormal: below any representable fixed-point step here
  const u64 m = (b & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
  const int sh = e - 1075 + s;  // x * 2^s = m * 2^sh
  i64 r;
  if (sh >= 0) r = (i64)(m << sh);
  else if (sh <= -64) r = 0;
  else r = (i64)((m + (1ull << (-sh - 1))) >> (-sh));
  return (b >> 63) ? -r : r;
}
// x * 2^-s as a double (round to nearest even), integer operations only
__device__ __forceinline__ double fx2d(i64 x, int s) {
  if (x == 0) return 0.0;
  const u64 sign = x < 0 ? 0x8000000000000000ull : 0ull;
  u64 a = (u64)(x < 0 ? -x : x);
  const int lz = __clzll((long long)a);
  a <<= lz;  // top bit set: value = a * 2^(63 - lz - 63)
  u64 mant = a >> 11;
  const u64 rem = a & 0x7ffull;
  int e = (63 - lz) - s + 1023;  // exponent of the leading bit
  if (rem > 0x400ull || (rem == 0x400ull && (mant & 1ull))) {
    ++mant;
    if (mant >> 53) {
      mant >>= 1;
      ++e;
    }
  }
  if (e <= 0) return 0.0;  // underflow below the normal range: negligible here
  return __longlong_as_double((long long)(sign | ((u64)e << 52) | (mant & 0xFFFFFFFFFFFFFull)));
}

}  // namespace qsf
