// qsf_cluster.cuh -- 1D lines longer than one CTA's shared memory (8192 < N <= 16384
// points, 256 KiB as int64 pairs) held by a cluster of two CTAs: each CTA keeps half of
// the line in its shared memory and the Stockham passes reach the other half through
// distributed shared memory (map_shared_rank), with cluster barriers between passes.
// Everything else is the single-CTA line kernel's arithmetic: block fixed point, the
// block exponent and maxima agreed across the pair.
#pragma once
#include <cooperative_groups.h>

namespace qsf {

namespace cg = cooperative_groups;

// The line as two halves of H elements in the shared memory of CTA 0 and CTA 1.
struct SplitLine {
  longlong2* half[2];
  int H;
  __device__ __forceinline__ longlong2& operator[](int i) const { return i < H ? half[0][i] : half[1][i - H]; }
};

// max over both CTAs of a per-thread value (result valid in every thread)
__device__ __forceinline__ int cluster_max_int(int v, int* red, cg::cluster_group& cl) {
  v = block_max_int(v, red);
  if (threadIdx.x == 0) red[31] = v;
  cl.sync();
  const int* peer = cl.map_shared_rank(red, cl.block_rank() ^ 1u);
  const int w = max(v, peer[31]);
  cl.sync();  // the peer has read red[31] before it is reused
  return w;
}

// one forward Stockham pass over the split line; butterflies are shared by the 2 * nth
// threads of the pair (g = rank * nth + tid)
template <int R, int MAXB, int N, int NS>
__device__ __forceinline__ int fx_stockham_split(const SplitLine& buf, const longlong2* __restrict__ tw, int g, int gth,
                                                 int shift_in, int* red, cg::cluster_group& cl) {
  constexpr int nr = N / R;
  constexpr int twstep = N / (NS * R);
  longlong2 v[MAXB][R];
  int dsto[MAXB];
#pragma unroll
  for (int b = 0; b < MAXB; ++b) {
    const int j = g + b * gth;
    dsto[b] = -1;
    if (j < nr) {
#pragma unroll
      for (int q = 0; q < R; ++q) {
        longlong2 x = buf[j + q * nr];
        if (shift_in) x = make_longlong2(fshift(x.x, shift_in), fshift(x.y, shift_in));
        v[b][q] = x;
      }
      const int jm = j % NS;
      if constexpr (NS > 1) {
#pragma unroll
        for (int q = 1; q < R; ++q) v[b][q] = fmul62(v[b][q], tw[jm * q * twstep]);
      }
      dsto[b] = (j - jm) * R + jm;
    }
  }
  cl.sync();
  u64 mag = 0;
#pragma unroll
  for (int b = 0; b < MAXB; ++b) {
    if (dsto[b] >= 0) {
      fbfly<R, true>(v[b]);
#pragma unroll
      for (int q = 0; q < R; ++q) {
        buf[dsto[b] + q * NS] = v[b][q];
        mag |= fmag(v[b][q]);
      }
    }
  }
  return cluster_max_int(bitlen(mag), red, cl);  // its cluster barrier ends the pass
}

template <int N, int S = 0>
__device__ __forceinline__ void fft_fx_split(const SplitLine& buf, const longlong2* __restrict__ tw, int g, int gth,
                                             int& scale, int& bits, int* red, cg::cluster_group& cl,
                                             int shift_in = 0) {
  if constexpr (S < nstages(N)) {
    constexpr int R = radix_at(N, S);
    constexpr int nb = (N / R + 2 * kLineThreads - 1) / (2 * kLineThreads);
    bits = fx_stockham_split<R, nb, N, ns_at(N, S)>(buf, tw, g, gth, shift_in, red, cl);
    if constexpr (S + 1 < nstages(N)) {
      const int target = 62 - fguard(radix_at(N, S + 1));
      const int sh = bits == 0 ? 0 : target - bits;
      scale += sh;
      fft_fx_split<N, S + 1>(buf, tw, g, gth, scale, bits, red, cl, sh);
    }
  }
}

__device__ __forceinline__ SplitLine split_line(longlong2* smx, cg::cluster_group& cl, int H) {
  SplitLine s;
  const unsigned r = cl.block_rank();
  longlong2* peer = cl.map_shared_rank(smx, r ^ 1u);
  s.half[0] = r == 0 ? smx : peer;
  s.half[1] = r == 0 ? peer : smx;
  s.H = H;
  return s;
}

// Whole 1D step on a line held by a CTA pair (the k_line_step arithmetic): this CTA
// opens, closes and reduces its half [rank * H, (rank + 1) * H); the transforms run
// over the pair.  Partials go to slot `rank` (the host sets two row blocks).
template <int N>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(kLineThreads, 1)
    k_line_step_cl(const GridDev* __restrict__ Gs, const StepDev* __restrict__ Ss) {
  const GridDev& g = Gs[blockIdx.y];
  const StepDev& S = Ss[blockIdx.y];
  cg::cluster_group cl = cg::this_cluster();
  if (!pass_active(S)) return;  // uniform over the pair
  const bool ek = ekin_at(S, S.ctl[5]);  // read before any block advances the counters
  if (blockIdx.x % 2 == 0 && threadIdx.x == 0) S.ctl[6] = S.ctl[5] + 1;  // the sub-step's only pass
  extern __shared__ __align__(128) longlong2 smx[];
  __shared__ int red[kRedInts];
  __shared__ double dred[32 * 3];
  constexpr int H = N / 2;
  const int rank = (int)cl.block_rank();
  const long long base = (long long)rank * H;
  const AxisDev& a = g.ax[0];
  const bool real_f = S.mode == 1 && g.gauge != 1;
  // open: psi (double) -> fixed point, pending Normalize, X half
  double2* sd = reinterpret_cast<double2*>(smx);
  int em = 0;
  for (int e = threadIdx.x; e < H; e += blockDim.x) {
    const double2 v = g.psi[base + e];
    sd[e] = v;
    em = max(em, max(dexp(v.x), dexp(v.y)));
  }
  em = cluster_max_int(em, red, cl);
  if (em >= 0x7ff && threadIdx.x == 0) S.ctl[4] = 1;  // Inf or NaN in psi: QSF_ENUMERIC
  const int s_in = scale_from_exponent<N>(em);
  int scale = s_in;
  long long F = 0;
  int k = 0;
  const bool use_s = S.normalize && *S.scale != 1.0;
  if (use_s) {
    split_scale(*S.scale, F, k);
    scale -= k;
  }
  u64 mag = 0;
  for (int e = threadIdx.x; e < H; e += blockDim.x) {
    const double2 v = sd[e];
    longlong2 x = make_longlong2(d2fx(v.x, s_in), d2fx(v.y, s_in));
    if (use_s) x = make_longlong2(mulq62(x.x, F), mulq62(x.y, F));
    const long long p = base + e;
    x = xhalf(g, S, x, p, 0, (int)p, 0, real_f);
    smx[e] = x;
    mag |= fmag(x);
  }
  scale -= xhalf_exp(g, S, 0);
  int bits = cluster_max_int(bitlen(mag), red, cl);
  const SplitLine line = split_line(smx, cl, H);
  const int gid = rank * blockDim.x + threadIdx.x, gth = 2 * blockDim.x;
  int sh = first_pass_shift<N>(bits);
  scale += sh;
  fft_fx_split<N>(line, a.twx, gid, gth, scale, bits, red, cl, sh);
  // P phase (own half), written conjugated for the inverse transform
  {
    const int pre = product_headroom(bits);
    mag = 0;
    for (int e = threadIdx.x; e < H; e += blockDim.x) {
      longlong2 x = smx[e];
      if (pre) x = make_longlong2(fshift(x.x, pre), fshift(x.y, pre));
      x = fconj(fapply(x, S.ptab[base + e], S.mode == 1));
      smx[e] = x;
      mag |= fmag(x);
    }
    scale += pre - S.texp[0] - xshift(1);
    bits = cluster_max_int(bitlen(mag), red, cl);
  }
  sh = first_pass_shift<N>(bits);
  scale += sh;
  fft_fx_split<N>(line, a.twx, gid, gth, scale, bits, red, cl, sh);
  // close: conjugate back, X half, 1/m, store, partial sums (own half)
  const int pre = product_headroom(bits);
  mag = 0;
  for (int e = threadIdx.x; e < H; e += blockDim.x) {
    const long long p = base + e;
    longlong2 x = fconj(smx[e]);
    if (pre) x = make_longlong2(fshift(x.x, pre), fshift(x.y, pre));
    x = xhalf(g, S, x, p, 0, (int)p, 1, real_f);
    smx[e] = x;
    mag |= fmag(x);
  }
  scale += pre - xhalf_exp(g, S, 1) + S.l2m;
  bits = cluster_max_int(bitlen(mag), red, cl);
  const int q = bits > 56 ? bits - 56 : 0;
  Acc128 an{0ull, 0ll}, av{0ull, 0ll};
  const bool epot = (S.obs & 2u) != 0;
  for (int e = threadIdx.x; e < H; e += blockDim.x) {
    const long long p = base + e;
    const longlong2 x = smx[e];
    g.psi[p] = make_double2(fx2d(x.x, scale), fx2d(x.y, scale));
    acc_point(an, av, x, q, S.Vx, p, epot);
  }
  if (S.row_ptr) {  // flux snapshot entries in this half
    const int e1 = S.row_ptr[1];
    for (int e = threadIdx.x; e < e1; e += blockDim.x) {
      const long long i = S.snap_idx[e] - base;
      if (i >= 0 && i < H) S.snap[e] = make_double2(fx2d(smx[i].x, scale), fx2d(smx[i].y, scale));
    }
  }
  double dacc[3] = {acc_value(an), acc_value(av), 0.0};
  const int e_n = 2 * q - 2 * scale, e_v = 2 * q - 2 * scale + 50 - S.vshift;
  if (ek) {  // E_kin: forward transform of psi_n over the pair
    cl.sync();
    int b2 = bits, sc2 = scale + first_pass_shift<N>(bits);
    fft_fx_split<N>(line, a.twx, gid, gth, sc2, b2, red, cl, first_pass_shift<N>(bits));
    double ek = 0.0;
    for (int e = threadIdx.x; e < H; e += blockDim.x) {
      const double kk = kpos(a, (int)(base + e));
      const longlong2 x = smx[e];
      const double xr = fx2d(x.x, sc2), xi = fx2d(x.y, sc2);
      ek = fma(kk * kk, fma(xr, xr, xi * xi), ek);
    }
    dacc[2] = ek;
  }
  block_sum<3>(dacc, dred);
  if (threadIdx.x == 0) {
    S.partials[0 * S.pmax + rank] = ldexp(dacc[0], e_n);
    S.partials[1 * S.pmax + rank] = ldexp(dacc[1], e_v);
    S.partials[2 * S.pmax + rank] = dacc[2];
  }
  cl.sync();  // neither CTA leaves while the other may still read its shared memory
}

// fourier<R>() of a 1D line held by a CTA pair (qsf_fourier)
template <int N, bool FWD>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(kLineThreads, 1)
    k_row_fft_cl(GridDev g, int L, double post_scale) {
  cg::cluster_group cl = cg::this_cluster();
  extern __shared__ __align__(128) longlong2 smx[];
  __shared__ int red[kRedInts];
  constexpr int H = N / 2;
  const int rank = (int)cl.block_rank();
  const long long base = (long long)rank * H;
  double2* sd = reinterpret_cast<double2*>(smx);
  int em = 0;
  for (int e = threadIdx.x; e < H; e += blockDim.x) {
    const double2 v = g.psi[base + e];
    sd[e] = v;
    em = max(em, max(dexp(v.x), dexp(v.y)));
  }
  em = cluster_max_int(em, red, cl);
  int scale = (62 - fguard(radix_at(N, 0))) - (em - 1022);
  for (int e = threadIdx.x; e < H; e += blockDim.x) {
    const double2 v = sd[e];
    const longlong2 x = make_longlong2(d2fx(v.x, scale), d2fx(v.y, scale));
    smx[e] = FWD ? x : fconj(x);
  }
  cl.sync();
  const SplitLine line = split_line(smx, cl, H);
  int bits = 0;
  fft_fx_split<N>(line, g.ax[0].twx, rank * blockDim.x + threadIdx.x, 2 * blockDim.x, scale, bits, red, cl);
  for (int e = threadIdx.x; e < H; e += blockDim.x) {
    const longlong2 x = FWD ? smx[e] : fconj(smx[e]);
    double2 v = make_double2(fx2d(x.x, scale), fx2d(x.y, scale));
    if (post_scale != 1.0) v = cscale(v, post_scale);
    g.psi[base + e] = v;
  }
  cl.sync();
}

}  // namespace qsf

namespace qsf {

// ---------------------------------------------------------------------------
// 1D lines spread over a cluster of C CTAs (C = 2 .. 8, power-of-two N): each CTA
// holds H = N / C consecutive points in its shared memory, the Stockham passes (radix
// 8, one butterfly per thread: the 4096-point line runs on 8 CTAs of 64 threads) read
// and write the other CTAs' parts through distributed shared memory, and the whole
// Strang step -- X half, transform, P phase, inverse, X half, observables, fluxes, the
// step end -- runs in one launch with the work of one line on C SMs instead of one
// (a one-CTA line is latency bound: its passes run one after another on one SM).
// Block maxima are agreed over the cluster through alternating slots, so a pass costs
// two cluster barriers (after its reads, after its writes).

// element i of the line: position i mod H in the shared memory of CTA i / H (the
// address mapped into the cluster window per access)
template <int C>
struct ClusterLine {
  longlong2* smx;
  int hshift;  // log2(H)
  __device__ __forceinline__ longlong2& operator[](int i) const {
    return *cg::this_cluster().map_shared_rank(smx + (i & ((1 << hshift) - 1)), (unsigned)(i >> hshift));
  }
};

// max over the cluster of a per-thread value, through slot `slot` of every CTA's red
// (a slot is written again only after two more cluster barriers); one cluster barrier
template <int C>
__device__ __forceinline__ int cluster_max_c(int v, int* red, int slot, cg::cluster_group& cl) {
  v = __reduce_max_sync(0xffffffffu, (unsigned)v);
  const int nw = (blockDim.x + 31) >> 5;
  if ((threadIdx.x & 31) == 0) red[slot + (threadIdx.x >> 5)] = v;
  cl.sync();
  int m = 0;
#pragma unroll
  for (int r = 0; r < C; ++r) {
    const int* pr = cl.map_shared_rank(red, (unsigned)r);
    for (int w = 0; w < nw; ++w) m = max(m, pr[slot + w]);
  }
  return m;
}

// one forward radix-R Stockham pass over the cluster line; butterflies are shared by
// the C * T threads of the cluster (g = rank * T + tid)
template <int R, int MAXB, int N, int NS, int C>
__device__ __forceinline__ int fx_stockham_mc(const ClusterLine<C>& buf, const longlong2* __restrict__ tw, int g,
                                              int gth, int shift_in, int* red, int parity, cg::cluster_group& cl) {
  constexpr int nr = N / R;
  constexpr int twstep = N / (NS * R);
  longlong2 v[MAXB][R];
  int dsto[MAXB];
#pragma unroll
  for (int b = 0; b < MAXB; ++b) {
    const int j = g + b * gth;
    dsto[b] = -1;
    if (j < nr) {
#pragma unroll
      for (int q = 0; q < R; ++q) {
        longlong2 x = buf[j + q * nr];
        if (shift_in) x = make_longlong2(fshift(x.x, shift_in), fshift(x.y, shift_in));
        v[b][q] = x;
      }
      const int jm = j % NS;
      if constexpr (NS > 1) {
#pragma unroll
        for (int q = 1; q < R; ++q) v[b][q] = fmul62(v[b][q], tw[jm * q * twstep]);
      }
      dsto[b] = (j - jm) * R + jm;
    }
  }
  cl.sync();  // every read of this pass is done before any write
  u64 mag = 0;
#pragma unroll
  for (int b = 0; b < MAXB; ++b) {
    if (dsto[b] >= 0) {
      fbfly<R, true>(v[b]);
#pragma unroll
      for (int q = 0; q < R; ++q) {
        buf[dsto[b] + q * NS] = v[b][q];
        mag |= fmag(v[b][q]);
      }
    }
  }
  return cluster_max_c<C>(bitlen(mag), red, 32 + 32 * parity, cl);  // its barrier ends the pass
}

// the passes of a radix-2^L2 plan over the cluster line (C * T = N / 8 threads)
template <int N, int C, int L2, int S = 0>
__device__ __forceinline__ void fft_fx_mc(const ClusterLine<C>& buf, const longlong2* __restrict__ tw, int g, int gth,
                                          int& scale, int& bits, int* red, int& parity, cg::cluster_group& cl,
                                          int shift_in = 0) {
  if constexpr (S < nstages(N, L2)) {
    constexpr int R = radix_at(N, S, L2);
    constexpr int nb = (N / R + (N / 8) - 1) / (N / 8);
    bits = fx_stockham_mc<R, nb, N, ns_at(N, S, L2), C>(buf, tw, g, gth, shift_in, red, parity, cl);
    parity ^= 1;
    if constexpr (S + 1 < nstages(N, L2)) {
      const int target = 62 - fguard(radix_at(N, S + 1, L2));
      const int sh = bits == 0 ? 0 : target - bits;
      scale += sh;
      fft_fx_mc<N, C, L2, S + 1>(buf, tw, g, gth, scale, bits, red, parity, cl, sh);
    }
  }
}

// threads per CTA of the cluster line kernel: one radix-8 butterfly per thread
template <int N, int C>
__host__ __device__ constexpr int mc_threads() { return N / 8 / C; }

template <int N, int C>
__global__ void __cluster_dims__(C, 1, 1) __launch_bounds__(mc_threads<N, C>(), 1)
    k_line_step_mc(const GridDev* __restrict__ Gs, const StepDev* __restrict__ Ss) {
  constexpr int H = N / C;
  const GridDev& g = Gs[blockIdx.y];
  const StepDev& S = Ss[blockIdx.y];
  cg::cluster_group cl = cg::this_cluster();
  if (!pass_active(S)) return;  // uniform over the cluster
  const long long sub = S.ctl[5];
  const bool ek = ekin_at(S, sub);  // read before any block advances the counters
  extern __shared__ __align__(128) longlong2 smx[];
  __shared__ int red[kRedInts];
  __shared__ double dred[32 * kMaxFluxBorders];
  const int rank = (int)cl.block_rank();
  if (rank == 0 && threadIdx.x == 0) S.ctl[6] = sub + 1;  // the sub-step's only pass
  const long long base = (long long)rank * H;
  const AxisDev& a = g.ax[0];
  const bool real_f = S.mode == 1 && g.gauge != 1;
  int parity = 0;
  // open: psi (double) -> fixed point, pending Normalize, X half
  double2* sd = reinterpret_cast<double2*>(smx);
  int em = 0;
  for (int e = threadIdx.x; e < H; e += blockDim.x) {
    const double2 v = g.psi[base + e];
    sd[e] = v;
    em = max(em, max(dexp(v.x), dexp(v.y)));
  }
  em = cluster_max_c<C>(em, red, 32 + 32 * parity, cl);
  parity ^= 1;
  if (em >= 0x7ff && rank == 0 && threadIdx.x == 0) S.ctl[4] = 1;  // Inf or NaN in psi: QSF_ENUMERIC
  const int s_in = scale_from_exponent<N>(em);
  int scale = s_in;
  long long F = 0;
  int k = 0;
  const bool use_s = S.normalize && *S.scale != 1.0;
  if (use_s) {
    split_scale(*S.scale, F, k);
    scale -= k;
  }
  u64 mag = 0;
  for (int e = threadIdx.x; e < H; e += blockDim.x) {
    const double2 v = sd[e];
    longlong2 x = make_longlong2(d2fx(v.x, s_in), d2fx(v.y, s_in));
    if (use_s) x = make_longlong2(mulq62(x.x, F), mulq62(x.y, F));
    const long long p = base + e;
    x = xhalf(g, S, x, p, 0, (int)p, 0, real_f);
    smx[e] = x;
    mag |= fmag(x);
  }
  scale -= xhalf_exp(g, S, 0);
  int bits = cluster_max_c<C>(bitlen(mag), red, 32 + 32 * parity, cl);
  parity ^= 1;
  ClusterLine<C> line;
  line.smx = smx;
  line.hshift = __ffs(H) - 1;
  const int gid = rank * blockDim.x + threadIdx.x, gth = C * blockDim.x;
  int sh = first_pass_shift<N>(bits);
  scale += sh;
  fft_fx_mc<N, C, 3>(line, a.twx, gid, gth, scale, bits, red, parity, cl, sh);
  // P phase (own part), written conjugated for the inverse transform
  {
    const int pre = product_headroom(bits);
    mag = 0;
    for (int e = threadIdx.x; e < H; e += blockDim.x) {
      longlong2 x = smx[e];
      if (pre) x = make_longlong2(fshift(x.x, pre), fshift(x.y, pre));
      x = fconj(fapply(x, S.ptab[base + e], S.mode == 1));
      smx[e] = x;
      mag |= fmag(x);
    }
    scale += pre - S.texp[0] - xshift(1);
    bits = cluster_max_c<C>(bitlen(mag), red, 32 + 32 * parity, cl);
    parity ^= 1;
  }
  sh = first_pass_shift<N>(bits);
  scale += sh;
  fft_fx_mc<N, C, 3>(line, a.twx, gid, gth, scale, bits, red, parity, cl, sh);
  // close: conjugate back, X half, 1/m, store, partial sums (own part)
  const int pre = product_headroom(bits);
  mag = 0;
  for (int e = threadIdx.x; e < H; e += blockDim.x) {
    const long long p = base + e;
    longlong2 x = fconj(smx[e]);
    if (pre) x = make_longlong2(fshift(x.x, pre), fshift(x.y, pre));
    x = xhalf(g, S, x, p, 0, (int)p, 1, real_f);
    smx[e] = x;
    mag |= fmag(x);
  }
  scale += pre - xhalf_exp(g, S, 1) + S.l2m;
  bits = cluster_max_c<C>(bitlen(mag), red, 32 + 32 * parity, cl);
  parity ^= 1;
  const int q = bits > 56 ? bits - 56 : 0;
  Acc128 an{0ull, 0ll}, av{0ull, 0ll};
  const bool epot = (S.obs & 2u) != 0;
  for (int e = threadIdx.x; e < H; e += blockDim.x) {
    const long long p = base + e;
    const longlong2 x = smx[e];
    g.psi[p] = make_double2(fx2d(x.x, scale), fx2d(x.y, scale));
    acc_point(an, av, x, q, S.Vx, p, epot);
  }
  if (S.row_ptr) {  // flux snapshot entries in this part
    const int e1 = S.row_ptr[1];
    for (int e = threadIdx.x; e < e1; e += blockDim.x) {
      const long long i = S.snap_idx[e] - base;
      if (i >= 0 && i < H) S.snap[e] = make_double2(fx2d(smx[i].x, scale), fx2d(smx[i].y, scale));
    }
  }
  double dacc[3] = {acc_value(an), acc_value(av), 0.0};
  const int e_n = 2 * q - 2 * scale, e_v = 2 * q - 2 * scale + 50 - S.vshift;
  if (ek) {  // E_kin: forward transform of psi_n over the cluster
    cl.sync();
    int b2 = bits, sc2 = scale + first_pass_shift<N>(bits);
    fft_fx_mc<N, C, 3>(line, a.twx, gid, gth, sc2, b2, red, parity, cl, first_pass_shift<N>(bits));
    double ekv = 0.0;
    for (int e = threadIdx.x; e < H; e += blockDim.x) {
      const double kk = kpos(a, (int)(base + e));
      const longlong2 x = smx[e];
      const double xr = fx2d(x.x, sc2), xi = fx2d(x.y, sc2);
      ekv = fma(kk * kk, fma(xr, xr, xi * xi), ekv);
    }
    dacc[2] = ekv;
  }
  block_sum<3>(dacc, dred);
  if (threadIdx.x == 0) {
    S.partials[0 * S.pmax + rank] = ldexp(dacc[0], e_n);
    S.partials[1 * S.pmax + rank] = ldexp(dacc[1], e_v);
    S.partials[2 * S.pmax + rank] = dacc[2];
  }
  // the step end in CTA 0 once every CTA's partials and snapshot entries are in memory;
  // the barrier also keeps every CTA's shared memory alive while others may read it
  __threadfence();
  cl.sync();
  if (rank == 0) {
    const bool step_end = (sub + 1) % S.substeps == 0;
    const long long step = sub / S.substeps;
    const int nb = S.nborders;
    if (S.nfterms > 0 && step_end) {
      const double* A = (g.gauge == 0 && S.coupling && g.n_fields) ? S.coupling + sub * S.coup_stride : nullptr;
      flux_block(g, S.fpts, S.fterms, 0, S.nfterms, S.snap, A, nb, dred, S.fpartials);
    }
    finalize_tail(g, S, sub, step_end, step, nb, 1, dred);
  }
}

}  // namespace qsf
