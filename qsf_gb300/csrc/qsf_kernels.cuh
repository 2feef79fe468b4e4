// qsf_kernels.cuh -- sm_103a kernels of the fused split-operator step.
//
// One Strang step  X(dt/2) . P(dt) . X(dt/2)  (propagator.h:311-346 with Split3Base
// mults {0.5, 1, 0.5}, splitting.h:18-27) runs as a short fixed sequence of passes
// over the wavefunction, ending with psi back in X space:
//
//   k_tables      per-step per-axis phase tables (A(t) / E(t) change every step)
//   k_row_open    [pending Normalize scale] . X half-phase . forward FFT (last axis)
//   k_axis  (3D)  forward FFT axis 1
//   k_axis        forward FFT axis 0 . P phase . inverse FFT axis 0 (1/m folded in)
//   k_axis  (3D)  inverse FFT axis 1
//   k_row_close   inverse FFT (last axis) . X half-phase . norm / E_pot partials,
//                 flux snapshot, E_kin partial of the last axis
//   k_axis  (E_kin only) forward FFT of the other axes of psi_n, sum k^2 |.|^2
//   k_finalize    deterministic reductions, border fluxes, Normalize scale,
//                 imaginary-time convergence, step counter
//
// For dim == 1 the whole step is one kernel (k_line_step) over a line held in
// shared memory.  A device step counter lets one captured CUDA graph replay any step.
// Step kernels read their grid and step descriptors from device arrays indexed by
// blockIdx.y, so one launch per stage advances every solve of a batch that shares
// the line length (a single grid is a batch of one).
// FFT kernels are templates on the line length N (compile-time radix plan); the host
// picks the instantiation for the grid's size.
#pragma once
#include "qsf_fft.cuh"

namespace qsf {

constexpr int kMaxDim = 3;
constexpr int kRowThreads = 256;
constexpr int kLineThreads = 512;
constexpr int kMaxFluxBorders = 16;

struct AxisDev {
  int n, n2;
  long long stride;
  double dx, xmin, dp, inv_2dx;
  const double2* tw;  // exp(-2 pi i t / n), t < n
};

struct GridDev {
  int dim;
  long long m;
  AxisDev ax[kMaxDim];
  double dV, dVm, inv_m, eta;
  long long nCAP;
  int pot;
  double NEcharge, EEcharge, Nsoft, Esoft;
  int gauge, n_fields, p_swap;
  double2* psi;
};

// flux evaluation point: slots into the snapshot of psi_n
struct FluxPoint {
  int c;           // slot of the point itself
  int p[kMaxDim];  // slot of psi[c + stride_d], -1 when the reference's bounds test fails
  int q[kMaxDim];  // slot of psi[c - stride_d]
};
// one (point, border) contribution with the normalised border vector
struct FluxTerm {
  int point;
  int border;
  double w[kMaxDim];
};

struct StepDev {
  int mode;  // 1 IM, 2 RE
  double dt;
  long long nsteps;
  const double* coupling;  // device copy of the per-step coupling rows (may be null)
  int coup_stride;         // 3 (velocity gauge) or 6 (length gauge)
  const double2* xs;       // static X half-step factor per point (dt/2, incl. absorber)
  const double* V;         // potential per point
  double2* ptab;           // [dim][nmax] P-phase tables of the current step
  double2* xdyn;           // [2][dim][nmax] length-gauge factors: open half, close half
  int nmax;
  // reductions
  double* partials;  // [5][pmax]: norm, epot, ekin axis 0..2
  int pmax;
  int nrowblk;          // row blocks of the close pass
  int naxblk[kMaxDim];  // blocks of the E_kin axis passes
  // observables
  unsigned obs;
  int normalize;
  int energy_after_normalize;
  double state_accuracy;
  int nborders;
  double2* snap;              // snapshot slots
  const int* row_ptr;         // CSR over rows: snapshot entries of row r are [row_ptr[r], row_ptr[r+1])
  const long long* snap_idx;  // flat index per snapshot entry (sorted)
  const FluxPoint* fpts;
  const FluxTerm* fterms;
  int nfterms;
  double* fpartials;  // [nblk][kMaxFluxBorders]
  // control (device): ctl[0] step within call, ctl[1] stop-after step (or nsteps),
  // ctl[2] steps done, ctl[3] finalize block counter, ctl[4] NaN flag
  long long* ctl;
  double* energy_state;  // [0] last E
  double* rows;          // [nsteps][3 + nborders]
  double* scale;         // pending Normalize factor (1 when none)
};

__device__ __forceinline__ bool step_active(const StepDev& S) { return S.ctl[0] <= S.ctl[1] && S.ctl[0] < S.nsteps; }

// ------------------------------------------------------------ reductions
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}
// block-wide sum of NV values; result valid in thread 0.  red needs 32 * NV doubles.
template <int NV>
__device__ __forceinline__ void block_sum(double* v, double* red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) v[k] = warp_sum(v[k]);
  __syncthreads();
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < NV; ++k) red[k * 32 + wid] = v[k];
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double t = lane < nw ? red[k * 32 + lane] : 0.0;
      v[k] = warp_sum(t);
    }
  }
  __syncthreads();
}

// ------------------------------------------------------------ geometry
__device__ __forceinline__ double xpos(const AxisDev& a, int i) { return a.xmin + (double)i * a.dx; }
__device__ __forceinline__ double kpos(const AxisDev& a, int i) { return a.dp * (double)(i < a.n2 ? i : i - a.n); }

// potential at a point (potential.h:130-143 and 40-44), same operation order
__device__ __forceinline__ double potential_at(const GridDev& g, const double* c) {
  if (g.pot == 3) return 0.0;
  if (g.pot == 2) {
    double s;
    if (g.dim == 1) s = c[0] * c[0];
    else if (g.dim == 2) s = c[0] * c[0] + c[1] * c[1];
    else s = c[0] * c[0] + (c[1] * c[1] + c[2] * c[2]);
    return g.NEcharge / sqrt(s + g.Nsoft);
  }
  auto ne = [&](double x) { return g.NEcharge / sqrt(x * x + g.Nsoft); };
  auto ee = [&](double x, double y) {
    return g.pot == 1 ? g.EEcharge / sqrt((x - y) * (x - y) + x * y + g.Esoft)
                      : g.EEcharge / sqrt((x - y) * (x - y) + g.Esoft);
  };
  if (g.dim == 1) return ne(c[0]);
  if (g.dim == 2) return ee(c[0], c[1]) + ne(c[0]) + ne(c[1]);
  return ee(c[0], c[1]) + ee(c[1], c[2]) + ee(c[2], c[0]) + ne(c[0]) + ne(c[1]) + ne(c[2]);
}

__device__ __forceinline__ void unflatten(const GridDev& g, long long p, int* idx) {
  for (int d = g.dim - 1; d >= 0; --d) {
    idx[d] = (int)(p % g.ax[d].n);
    p /= g.ax[d].n;
  }
}

// absorbers.h:40-46 with neg_dist_from_edge (grid.h:181-185)
__device__ __forceinline__ double absorb_at(const GridDev& g, double delta, const int* idx) {
  if (g.nCAP <= 0) return 1.0;
  long long nodes[kMaxDim];
  bool all_neg = true;
  for (int d = 0; d < g.dim; ++d) {
    const int i = idx[d];
    const long long nd = i < g.ax[d].n2 ? -(long long)i : (long long)i - g.ax[d].n + 1;
    nodes[d] = g.nCAP + nd;
    if (!(nodes[d] < 0)) all_neg = false;
  }
  if (all_neg) return 1.0;
  long long s = 0;
  for (int d = g.dim - 1; d >= 0; --d) {
    const long long v = nodes[d] > 0 ? nodes[d] * (nodes[d] * (nodes[d] * nodes[d])) : 0;
    s = v + s;
  }
  return exp(-delta * (double)s * g.eta);
}

__device__ __forceinline__ double2 expop(int mode, double val) {
  if (mode == 1) return make_double2(exp(-val), 0.0);
  double sn, cs;
  sincos(-val, &sn, &cs);
  return make_double2(cs, sn);
}

#ifdef QSF_DEFINE_KERNELS
// ------------------------------------------------------------ tables
// Static X factor for delta (per point): expOp(delta V) * absorb(delta)   (IM: real).
__global__ void k_build_static(GridDev g, int mode, double delta, double2* xs, double* V) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < g.m; p += stride) {
    int idx[kMaxDim];
    double c[kMaxDim];
    unflatten(g, p, idx);
    for (int d = 0; d < g.dim; ++d) c[d] = xpos(g.ax[d], idx[d]);
    const double v = potential_at(g, c);
    if (V) V[p] = v;
    if (xs) {
      const double2 f = expop(mode, delta * v);
      const double a = absorb_at(g, delta, idx);
      xs[p] = make_double2(f.x * a, f.y * a);
    }
  }
}

// Per-step tables: P phase per axis (velocity gauge A of this step; 1/m folded into
// axis 0) and, in the length gauge, the x.E factors of both X halves.
__global__ void k_tables(const GridDev* __restrict__ Gs, const StepDev* __restrict__ Ss) {
  const GridDev& g = Gs[blockIdx.y];
  const StepDev& S = Ss[blockIdx.y];
  if (!step_active(S)) return;
  const long long step = S.ctl[0];
  const double* cp = S.coupling ? S.coupling + step * S.coup_stride : nullptr;
  const int D = g.dim;
  const int ntab = D * S.nmax;
  const bool lg = g.gauge == 1;
  const int total = ntab * (lg ? 3 : 1);
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
    const int kind = t / ntab;  // 0: P table, 1: X open, 2: X close
    const int d = (t % ntab) / S.nmax;
    const int i = t % S.nmax;
    const AxisDev& a = g.ax[d];
    if (i >= a.n) continue;
    if (kind == 0) {
      // hamiltonian.h:52-58 kinetic + coupling in P (velocity gauge only)
      double A = 0.0;
      if (!lg && cp && g.n_fields) {
        int dd = d;
        if (g.p_swap && D >= 2 && d < 2) dd = 1 - d;
        A = cp[dd];
      }
      const double k = kpos(a, i);
      const double val = S.dt * (0.5 * k * k + k * A);
      double2 f = expop(S.mode, val);
      if (d == 0) f = cscale(f, g.inv_m);
      S.ptab[d * S.nmax + i] = f;
    } else {
      const double E = (cp && g.n_fields) ? cp[(kind - 1) * 3 + d] : 0.0;
      const double val = (S.dt * 0.5) * (xpos(a, i) * E);
      S.xdyn[((kind - 1) * D + d) * S.nmax + i] = expop(S.mode, val);
    }
  }
}

#endif  // QSF_DEFINE_KERNELS

// X factor at point p (row index r, position j on the last axis); half 0 open, 1 close
__device__ __forceinline__ double2 xfactor(const GridDev& g, const StepDev& S, long long p, long long r, int j,
                                           int half) {
  double2 f = __ldg(&S.xs[p]);
  if (g.gauge == 1) {
    const int D = g.dim;
    const double2* t = S.xdyn + (size_t)half * D * S.nmax;
    double2 d = __ldg(&t[(D - 1) * S.nmax + j]);
    long long rr = r;
    for (int dd = D - 2; dd >= 0; --dd) {
      const int ii = (int)(rr % g.ax[dd].n);
      rr /= g.ax[dd].n;
      d = cmul(d, __ldg(&t[dd * S.nmax + ii]));
    }
    f = cmul(f, d);
  }
  return f;
}

// ------------------------------------------------------------ row passes
// Rows of the last axis: L rows of N points per block, contiguous in memory.
template <int N>
__global__ void __launch_bounds__(kRowThreads) k_row_open(const GridDev* __restrict__ Gs, const StepDev* __restrict__ Ss, int L) {
  const GridDev& g = Gs[blockIdx.y];
  const StepDev& S = Ss[blockIdx.y];
  if (!step_active(S)) return;
  extern __shared__ double2 sm[];
  const AxisDev& a = g.ax[g.dim - 1];
  const long long row0 = (long long)blockIdx.x * L;
  const long long nrows = g.m / N;
  const int Lh = (int)min((long long)L, nrows - row0);
  const long long base = row0 * N;
  const int cnt = Lh * N;
  const double s = (S.normalize && S.scale) ? *S.scale : 1.0;
  const bool use_s = S.normalize && s != 1.0;
  const bool realx = S.mode == 1 && g.gauge != 1;
  for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
    const long long p = base + e;
    double2 v = g.psi[p];
    if (use_s) v = cscale(v, s);
    const double2 f = xfactor(g, S, p, row0 + e / N, e % N, 0);
    sm[e] = realx ? cscale(v, f.x) : cmul(v, f);
  }
  __syncthreads();
  const LineSet ls{Lh, N, 1, false};
  fft_static<N, true>(sm, ls, a.tw, threadIdx.x, blockDim.x);
  for (int e = threadIdx.x; e < cnt; e += blockDim.x) g.psi[base + e] = sm[e];
}

template <int N>
__global__ void __launch_bounds__(kRowThreads) k_row_close(const GridDev* __restrict__ Gs, const StepDev* __restrict__ Ss, int L) {
  const GridDev& g = Gs[blockIdx.y];
  const StepDev& S = Ss[blockIdx.y];
  if (!step_active(S)) return;
  extern __shared__ double2 sm[];
  __shared__ double red[32 * 3];
  const AxisDev& a = g.ax[g.dim - 1];
  const long long row0 = (long long)blockIdx.x * L;
  const long long nrows = g.m / N;
  const int Lh = (int)min((long long)L, nrows - row0);
  const long long base = row0 * N;
  const int cnt = Lh * N;
  const bool realx = S.mode == 1 && g.gauge != 1;
  for (int e = threadIdx.x; e < cnt; e += blockDim.x) sm[e] = g.psi[base + e];
  __syncthreads();
  const LineSet ls{Lh, N, 1, false};
  fft_static<N, false>(sm, ls, a.tw, threadIdx.x, blockDim.x);
  double acc[3] = {0.0, 0.0, 0.0};
  for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
    const long long p = base + e;
    const double2 f = xfactor(g, S, p, row0 + e / N, e % N, 1);
    const double2 v = realx ? cscale(sm[e], f.x) : cmul(sm[e], f);
    sm[e] = v;
    g.psi[p] = v;
    const double nrm = fma(v.x, v.x, v.y * v.y);
    acc[0] += nrm;
    if (S.obs & 2u) acc[1] = fma(nrm, __ldg(&S.V[p]), acc[1]);
  }
  __syncthreads();
  // flux snapshot of psi_n for the entries of these rows (psi_n is still in smem)
  if (S.row_ptr) {
    const int e0 = S.row_ptr[row0], e1 = S.row_ptr[row0 + Lh];
    for (int e = e0 + threadIdx.x; e < e1; e += blockDim.x) S.snap[e] = sm[S.snap_idx[e] - base];
  }
  __syncthreads();
  // E_kin part of the last axis: forward FFT of psi_n rows, sum k^2 |.|^2
  if (S.obs & 4u) {
    fft_static<N, true>(sm, ls, a.tw, threadIdx.x, blockDim.x);
    for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
      const double k = kpos(a, e % N);
      const double2 v = sm[e];
      acc[2] = fma(k * k, fma(v.x, v.x, v.y * v.y), acc[2]);
    }
  }
  block_sum<3>(acc, red);
  if (threadIdx.x == 0) {
    S.partials[0 * S.pmax + blockIdx.x] = acc[0];
    S.partials[1 * S.pmax + blockIdx.x] = acc[1];
    S.partials[(2 + g.dim - 1) * S.pmax + blockIdx.x] = acc[2];
  }
}

// ------------------------------------------------------------ strided axes
// Axis `ax` (not the last): tiles of C adjacent columns; element (i, c) of tile
// (o, c0) is psi[o * N * stride + i * stride + c0 + c].  Modes:
//   0 forward, 1 inverse, 2 forward . P phase . inverse, 3 forward + E_kin partial
template <int MODE, int N>
__global__ void __launch_bounds__(kRowThreads) k_axis(const GridDev* __restrict__ Gs, const StepDev* __restrict__ Ss, int ax, int C) {
  const GridDev& g = Gs[blockIdx.y];
  const StepDev& S = Ss[blockIdx.y];
  if (!step_active(S)) return;
  if (MODE == 3 && !(S.obs & 4u)) return;
  extern __shared__ double2 sm[];
  __shared__ double red[32];
  __shared__ double2 pcol[64];
  const AxisDev& a = g.ax[ax];
  const long long inner = a.stride;
  const long long tiles_per_outer = (inner + C - 1) / C;
  const long long o = blockIdx.x / tiles_per_outer;
  const long long c0 = (blockIdx.x % tiles_per_outer) * C;
  const int Ch = (int)min((long long)C, inner - c0);
  const long long obase = o * (long long)N * inner + c0;
  const int cnt = N * Ch;
  for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
    const int i = e / Ch, c = e % Ch;
    sm[i * C + c] = g.psi[obase + (long long)i * inner + c];
  }
  if (MODE == 2 && threadIdx.x < Ch) {
    // per-column factor: product of the P tables of the axes after `ax`
    long long cc = c0 + threadIdx.x;
    double2 f = make_double2(1.0, 0.0);
    for (int d = g.dim - 1; d > ax; --d) {
      const int i = (int)(cc % g.ax[d].n);
      cc /= g.ax[d].n;
      f = cmul(f, __ldg(&S.ptab[d * S.nmax + i]));
    }
    pcol[threadIdx.x] = f;
  }
  __syncthreads();
  const LineSet ls{Ch, 1, C, true};
  if (MODE == 1) fft_static<N, false>(sm, ls, a.tw, threadIdx.x, blockDim.x);
  else fft_static<N, true>(sm, ls, a.tw, threadIdx.x, blockDim.x);
  if (MODE == 2) {
    for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
      const int i = e / Ch, c = e % Ch;
      const double2 f = cmul(__ldg(&S.ptab[ax * S.nmax + i]), pcol[c]);
      sm[i * C + c] = S.mode == 1 ? cscale(sm[i * C + c], f.x) : cmul(sm[i * C + c], f);
    }
    __syncthreads();
    fft_static<N, false>(sm, ls, a.tw, threadIdx.x, blockDim.x);
  }
  if (MODE == 3) {
    double acc = 0.0;
    for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
      const int i = e / Ch, c = e % Ch;
      const double k = kpos(a, i);
      const double2 v = sm[i * C + c];
      acc = fma(k * k, fma(v.x, v.x, v.y * v.y), acc);
    }
    block_sum<1>(&acc, red);
    if (threadIdx.x == 0) S.partials[(2 + ax) * S.pmax + blockIdx.x] = acc;
    return;
  }
  for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
    const int i = e / Ch, c = e % Ch;
    g.psi[obase + (long long)i * inner + c] = sm[i * C + c];
  }
}

// ------------------------------------------------------------ 1D whole step
// One block per line: X open . FFT . P . IFFT . X close . observables, line in smem.
template <int N>
__global__ void __launch_bounds__(kLineThreads) k_line_step(const GridDev* __restrict__ Gs, const StepDev* __restrict__ Ss) {
  const GridDev& g = Gs[blockIdx.y];
  const StepDev& S = Ss[blockIdx.y];
  if (!step_active(S)) return;
  extern __shared__ double2 sm[];
  __shared__ double red[32 * 3];
  const AxisDev& a = g.ax[0];
  const double s = (S.normalize && S.scale) ? *S.scale : 1.0;
  const bool use_s = S.normalize && s != 1.0;
  const bool realx = S.mode == 1 && g.gauge != 1;
  for (int e = threadIdx.x; e < N; e += blockDim.x) {
    double2 v = g.psi[e];
    if (use_s) v = cscale(v, s);
    const double2 f = xfactor(g, S, e, 0, e, 0);
    sm[e] = realx ? cscale(v, f.x) : cmul(v, f);
  }
  __syncthreads();
  const LineSet ls{1, N, 1, false};
  fft_static<N, true>(sm, ls, a.tw, threadIdx.x, blockDim.x);
  for (int e = threadIdx.x; e < N; e += blockDim.x) {
    const double2 f = __ldg(&S.ptab[e]);
    sm[e] = S.mode == 1 ? cscale(sm[e], f.x) : cmul(sm[e], f);
  }
  __syncthreads();
  fft_static<N, false>(sm, ls, a.tw, threadIdx.x, blockDim.x);
  double acc[3] = {0.0, 0.0, 0.0};
  for (int e = threadIdx.x; e < N; e += blockDim.x) {
    const double2 f = xfactor(g, S, e, 0, e, 1);
    const double2 v = realx ? cscale(sm[e], f.x) : cmul(sm[e], f);
    sm[e] = v;
    g.psi[e] = v;
    const double nrm = fma(v.x, v.x, v.y * v.y);
    acc[0] += nrm;
    if (S.obs & 2u) acc[1] = fma(nrm, __ldg(&S.V[e]), acc[1]);
  }
  __syncthreads();
  if (S.row_ptr) {
    const int e1 = S.row_ptr[1];
    for (int e = threadIdx.x; e < e1; e += blockDim.x) S.snap[e] = sm[S.snap_idx[e]];
  }
  __syncthreads();
  if (S.obs & 4u) {
    fft_static<N, true>(sm, ls, a.tw, threadIdx.x, blockDim.x);
    for (int e = threadIdx.x; e < N; e += blockDim.x) {
      const double k = kpos(a, e);
      const double2 v = sm[e];
      acc[2] = fma(k * k, fma(v.x, v.x, v.y * v.y), acc[2]);
    }
  }
  block_sum<3>(acc, red);
  if (threadIdx.x == 0) {
    S.partials[0 * S.pmax] = acc[0];
    S.partials[1 * S.pmax] = acc[1];
    S.partials[2 * S.pmax] = acc[2];
  }
}

// ------------------------------------------------------------ plain FFT passes
// fourier<R>() without phases (qsf_fourier): rows of the last axis, and strided axes
template <int N, bool FWD>
__global__ void __launch_bounds__(kLineThreads) k_row_fft(GridDev g, int L, double post_scale) {
  extern __shared__ double2 sm[];
  const AxisDev& a = g.ax[g.dim - 1];
  const long long row0 = (long long)blockIdx.x * L;
  const long long nrows = g.m / N;
  const int Lh = (int)min((long long)L, nrows - row0);
  const long long base = row0 * N;
  const int cnt = Lh * N;
  for (int e = threadIdx.x; e < cnt; e += blockDim.x) sm[e] = g.psi[base + e];
  __syncthreads();
  const LineSet ls{Lh, N, 1, false};
  fft_static<N, FWD>(sm, ls, a.tw, threadIdx.x, blockDim.x);
  for (int e = threadIdx.x; e < cnt; e += blockDim.x)
    g.psi[base + e] = post_scale == 1.0 ? sm[e] : cscale(sm[e], post_scale);
}

template <int N, bool FWD>
__global__ void __launch_bounds__(kRowThreads) k_axis_fft(GridDev g, int ax, int C, double post_scale) {
  extern __shared__ double2 sm[];
  const AxisDev& a = g.ax[ax];
  const long long inner = a.stride;
  const long long tiles_per_outer = (inner + C - 1) / C;
  const long long o = blockIdx.x / tiles_per_outer;
  const long long c0 = (blockIdx.x % tiles_per_outer) * C;
  const int Ch = (int)min((long long)C, inner - c0);
  const long long obase = o * (long long)N * inner + c0;
  const int cnt = N * Ch;
  for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
    const int i = e / Ch, c = e % Ch;
    sm[i * C + c] = g.psi[obase + (long long)i * inner + c];
  }
  __syncthreads();
  const LineSet ls{Ch, 1, C, true};
  fft_static<N, FWD>(sm, ls, a.tw, threadIdx.x, blockDim.x);
  for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
    const int i = e / Ch, c = e % Ch;
    const double2 v = sm[i * C + c];
    g.psi[obase + (long long)i * inner + c] = post_scale == 1.0 ? v : cscale(v, post_scale);
  }
}

#ifdef QSF_DEFINE_KERNELS
// ------------------------------------------------------------ flux + finalize
// Block-partial border fluxes over flux terms [t0, t1): each term is one grid point
// and one border type; j_d = inv_2dx Im(conj(psi) (psi_+ - psi_-)) (0 where the
// reference's flat-index bounds test fails, grid.h:470-472) + A_d |psi|^2 (velocity
// gauge), dotted with the normalised border vector.  out[b] written by thread b.
__device__ void flux_block(const GridDev& g, const FluxPoint* __restrict__ fpts, const FluxTerm* __restrict__ fterms,
                           int t0, int t1, const double2* __restrict__ snap, const double* A, int nb, double* red,
                           double* out) {
  double fl[kMaxFluxBorders];
#pragma unroll
  for (int b = 0; b < kMaxFluxBorders; ++b) fl[b] = 0.0;
  for (int t = t0 + threadIdx.x; t < t1; t += blockDim.x) {
    const FluxTerm ft = fterms[t];
    const FluxPoint fp = fpts[ft.point];
    const double2 c = snap[fp.c];
    double dot = 0.0;
    for (int d = 0; d < g.dim; ++d) {
      if (ft.w[d] == 0.0) continue;
      double j = 0.0;
      if (fp.p[d] >= 0) {
        const double2 tt = csub(snap[fp.p[d]], snap[fp.q[d]]);
        j = g.ax[d].inv_2dx * (c.x * tt.y + (-c.y) * tt.x);
      }
      if (A) j += A[d] * (c.x * c.x + c.y * c.y);
      dot += j * ft.w[d];
    }
#pragma unroll
    for (int b = 0; b < kMaxFluxBorders; ++b)
      if (b == ft.border) fl[b] += dot;
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int b = 0; b < kMaxFluxBorders; ++b) {
    if (b < nb) {
      const double v = warp_sum(fl[b]);
      if (lane == 0) red[b * 32 + wid] = v;
    }
  }
  __syncthreads();
  if (threadIdx.x < nb) {
    double v = 0.0;
    for (int w = 0; w < nw; ++w) v += red[threadIdx.x * 32 + w];
    out[threadIdx.x] = v;
  }
  __syncthreads();
}

__global__ void __launch_bounds__(256) k_flux(GridDev g, const FluxPoint* fpts, const FluxTerm* fterms, int nfterms,
                                              const double2* snap, double A0, double A1, double A2, int useA, int nb,
                                              double* out_partials) {
  __shared__ double red[32 * kMaxFluxBorders];
  const double Av[3] = {A0, A1, A2};
  const int chunk = (nfterms + gridDim.x - 1) / gridDim.x;
  const int t0 = blockIdx.x * chunk, t1 = min(nfterms, t0 + chunk);
  flux_block(g, fpts, fterms, t0, t1, snap, useA ? Av : nullptr, nb, red, out_partials + blockIdx.x * kMaxFluxBorders);
}

// Border fluxes (grid.h:519-573, propagator.h:249-265) from the psi_n snapshot,
// deterministic reductions of all partials, Normalize scale and IM convergence.
// Grid: nblk blocks; block b sums flux terms [b*chunk, (b+1)*chunk); the last block
// to finish reduces everything in a fixed order and writes the observables row.
__global__ void __launch_bounds__(256) k_finalize(const GridDev* __restrict__ Gs, const StepDev* __restrict__ Ss) {
  const GridDev& g = Gs[blockIdx.y];
  const StepDev& S = Ss[blockIdx.y];
  if (!step_active(S)) return;
  __shared__ double red[32 * kMaxFluxBorders];
  __shared__ int is_last;
  const long long step = S.ctl[0];
  const int nb = S.nborders;
  if (S.nfterms > 0) {
    const double* A = (g.gauge == 0 && S.coupling && g.n_fields) ? S.coupling + step * S.coup_stride : nullptr;
    const int chunk = (S.nfterms + gridDim.x - 1) / gridDim.x;
    const int t0 = blockIdx.x * chunk, t1 = min(S.nfterms, t0 + chunk);
    flux_block(g, S.fpts, S.fterms, t0, t1, S.snap, A, nb, red, S.fpartials + blockIdx.x * kMaxFluxBorders);
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned long long done = atomicAdd((unsigned long long*)&S.ctl[3], 1ull);
    is_last = (done == (unsigned long long)gridDim.x - 1);
  }
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  // last block: deterministic sums in a fixed order
  double acc[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  for (int i = threadIdx.x; i < S.nrowblk; i += blockDim.x) {
    acc[0] += S.partials[0 * S.pmax + i];
    acc[1] += S.partials[1 * S.pmax + i];
    acc[2 + g.dim - 1] += S.partials[(2 + g.dim - 1) * S.pmax + i];
  }
  if (S.obs & 4u) {
    for (int d = 0; d < g.dim - 1; ++d)
      for (int i = threadIdx.x; i < S.naxblk[d]; i += blockDim.x) acc[2 + d] += S.partials[(2 + d) * S.pmax + i];
  }
  block_sum<5>(acc, red);
  if (threadIdx.x == 0) {
    const double norm = acc[0] * g.dV;
    const double epot = acc[1] * g.dV;
    double ekin = 0.0;
    if (S.obs & 4u) {
      for (int d = 0; d < g.dim; ++d) ekin += (double)(g.m / g.ax[d].n) * acc[2 + d];
      ekin = 0.5 * g.dVm * ekin;
    }
    const int ncol = 3 + nb;
    double* row = S.rows + step * ncol;
    row[0] = norm;
    row[1] = epot;
    row[2] = ekin;
    for (int b = 0; b < nb; ++b) {
      double v = 0.0;
      for (int k = 0; k < (int)gridDim.x; ++k) v += S.fpartials[k * kMaxFluxBorders + b];
      row[3 + b] = v * g.dV / g.ax[0].dx;
    }
    if (!(norm > 0.0) || isnan(epot) || isnan(ekin)) S.ctl[4] = 1;
    if (S.normalize && norm > 0.0) *S.scale = sqrt(1.0 / norm);
    if (S.mode == 1 && S.state_accuracy > 0.0) {
      const double se = (S.energy_after_normalize & 1) ? 1.0 / norm : 1.0;
      const double sk = (S.energy_after_normalize & 2) ? 1.0 / norm : 1.0;
      const double E = epot * se + ekin * sk;
      const double dE = E - S.energy_state[0];
      S.energy_state[0] = E;
      if (S.ctl[1] >= S.nsteps && fabs(dE) <= S.state_accuracy) S.ctl[1] = step + 1;
    }
    S.ctl[2] = step + 1;
    S.ctl[3] = 0;
    S.ctl[0] = step + 1;
  }
}

// apply a pending Normalize factor (end of a qsf_step call / qsf_normalize)
__global__ void k_scale(double2* psi, long long m, const double* scale) {
  const double s = *scale;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < m; p += stride) psi[p] = cscale(psi[p], s);
}

// ------------------------------------------------------------ granular members
// evolve<M,R>(delta) with the reference's per-point formula (grid.h:394-418)
__global__ void k_evolve(GridDev g, int mode, int rep, double delta, double c0, double c1, double c2) {
  double cv[3] = {c0, c1, c2};
  if (rep == 2 && g.p_swap && g.dim >= 2) {
    cv[0] = c1;
    cv[1] = c0;
  }
  const int couples = g.gauge == 0 ? 2 : 1;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < g.m; p += stride) {
    int idx[kMaxDim];
    double c[kMaxDim];
    unflatten(g, p, idx);
    double H;
    if (rep == 2) {
      for (int d = 0; d < g.dim; ++d) c[d] = kpos(g.ax[d], idx[d]);
      if (g.dim == 1) H = 0.5 * c[0] * c[0];
      else if (g.dim == 2) H = 0.5 * c[0] * c[0] + 0.5 * c[1] * c[1];
      else H = 0.5 * c[0] * c[0] + (0.5 * c[1] * c[1] + 0.5 * c[2] * c[2]);
    } else {
      for (int d = 0; d < g.dim; ++d) c[d] = xpos(g.ax[d], idx[d]);
      H = potential_at(g, c);
    }
    double ct = 0.0;
    if (couples == rep && g.n_fields) {
      if (g.dim == 1) ct = c[0] * cv[0];
      else if (g.dim == 2) ct = c[0] * cv[0] + c[1] * cv[1];
      else ct = c[0] * cv[0] + (c[1] * cv[1] + c[2] * cv[2]);
    }
    const double val = delta * (H + ct);
    double2 v = g.psi[p];
    if (mode == 1) v = cscale(v, exp(-val));
    else {
      double sn, cs;
      sincos(-val, &sn, &cs);
      v = make_double2(v.x * cs - v.y * sn, v.x * sn + v.y * cs);
    }
    if (rep == 1 && g.nCAP > 0) v = cscale(v, absorb_at(g, delta, idx));
    g.psi[p] = v;
  }
}

// sum |psi|^2 w(p) per block (average_, grid.h:425-441); op 0 identity, 1 potential, 2 kinetic
__global__ void __launch_bounds__(256) k_average(GridDev g, int rep, int op, double* out_partials) {
  __shared__ double red[32];
  double acc = 0.0;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < g.m; p += stride) {
    const double2 v = g.psi[p];
    double w = 1.0;
    if (op != 0) {
      int idx[kMaxDim];
      double c[kMaxDim];
      unflatten(g, p, idx);
      if (op == 2) {
        for (int d = 0; d < g.dim; ++d) c[d] = kpos(g.ax[d], idx[d]);
        if (g.dim == 1) w = 0.5 * c[0] * c[0];
        else if (g.dim == 2) w = 0.5 * c[0] * c[0] + 0.5 * c[1] * c[1];
        else w = 0.5 * c[0] * c[0] + (0.5 * c[1] * c[1] + 0.5 * c[2] * c[2]);
      } else {
        for (int d = 0; d < g.dim; ++d) c[d] = xpos(g.ax[d], idx[d]);
        w = potential_at(g, c);
      }
    }
    acc = fma(fma(v.x, v.x, v.y * v.y), w, acc);
  }
  block_sum<1>(&acc, red);
  if (threadIdx.x == 0) out_partials[blockIdx.x] = acc;
}

__global__ void k_reduce_partials(const double* part, int n, double scale, double* out) {
  __shared__ double red[32];
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) acc += part[i];
  block_sum<1>(&acc, red);
  if (threadIdx.x == 0) *out = acc * scale;
}

// gather psi at the snapshot indices (granular flux)
__global__ void k_gather(const double2* psi, const long long* idx, int n, double2* out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) out[i] = psi[idx[i]];
}

// maskRegion (grid.h:582-597) with CAP::mask (absorbers.h:48-54)
__global__ void k_mask(GridDev g, int b0, int b1, int b2) {
  const int bounded[3] = {b0, b1, b2};
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < g.m; p += stride) {
    int idx[kMaxDim];
    unflatten(g, p, idx);
    long long nodes[kMaxDim];
    bool all_neg = true;
    for (int d = 0; d < g.dim; ++d) {
      const int i = idx[d];
      const long long nd = bounded[d] ? (i < g.ax[d].n2 ? -(long long)i : (long long)i - g.ax[d].n + 1)
                                      : -(long long)g.ax[d].n2;
      nodes[d] = g.nCAP + nd;
      if (!(nodes[d] < 0)) all_neg = false;
    }
    double mk = 1.0;
    if (!all_neg) {
      long long s = 0;
      for (int d = g.dim - 1; d >= 0; --d) {
        const long long v = nodes[d] > 0 ? nodes[d] * (nodes[d] * (nodes[d] * nodes[d])) : 0;
        s = v + s;
      }
      mk = exp(-(double)s * g.eta);
    }
    g.psi[p] = cscale(g.psi[p], mk);
  }
}

// psi += gaussian(at, delta, x...) (wf/preset.h:5-10)
__global__ void k_add_gaussian(GridDev g, double at, double delta) {
  const double delta_inv = 1.0 / delta;
  const double base = sqrt(delta_inv * sqrt(1.0 / 3.14159265358979323846));
  const double nrm = g.dim == 1 ? base : (g.dim == 2 ? base * base : base * (base * base));
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < g.m; p += stride) {
    int idx[kMaxDim];
    unflatten(g, p, idx);
    double t[kMaxDim];
    for (int d = 0; d < g.dim; ++d) {
      const double x = xpos(g.ax[d], idx[d]);
      t[d] = (x - at) * (x - at) * delta_inv * delta_inv;
    }
    const double s = g.dim == 1 ? t[0] : (g.dim == 2 ? t[0] + t[1] : t[0] + (t[1] + t[2]));
    g.psi[p].x += exp(-0.5 * s) * nrm;
  }
}

#endif  // QSF_DEFINE_KERNELS

// ------------------------------------------------------------ per-size kernel table
struct KernelSet {
  int n;
  void (*row_open)(const GridDev*, const StepDev*, int);
  void (*row_close)(const GridDev*, const StepDev*, int);
  void (*axis_fwd)(const GridDev*, const StepDev*, int, int);
  void (*axis_inv)(const GridDev*, const StepDev*, int, int);
  void (*axis_fpi)(const GridDev*, const StepDev*, int, int);
  void (*axis_ekin)(const GridDev*, const StepDev*, int, int);
  void (*line_step)(const GridDev*, const StepDev*);
  void (*row_fft_f)(GridDev, int, double);
  void (*row_fft_b)(GridDev, int, double);
  void (*axis_fft_f)(GridDev, int, int, double);
  void (*axis_fft_b)(GridDev, int, int, double);
};

// kernel table of the supported sizes (qsf_sizes_*.cu); nullptr when n is not built
const KernelSet* kernels_for(int n);

// sizes up to 4096 get the multi-dimensional passes; up to 8192 the 1D line kernel
template <int N>
KernelSet make_kernel_set() {
  static_assert(is_smooth(N), "grid sizes must be 2^a 3^b 5^c");
  KernelSet k{};
  k.n = N;
  if constexpr (N <= 4096) {
    k.row_open = k_row_open<N>;
    k.row_close = k_row_close<N>;
    k.axis_fwd = k_axis<0, N>;
    k.axis_inv = k_axis<1, N>;
    k.axis_fpi = k_axis<2, N>;
    k.axis_ekin = k_axis<3, N>;
    k.axis_fft_f = k_axis_fft<N, true>;
    k.axis_fft_b = k_axis_fft<N, false>;
  }
  k.line_step = k_line_step<N>;
  k.row_fft_f = k_row_fft<N, true>;
  k.row_fft_b = k_row_fft<N, false>;
  return k;
}

}  // namespace qsf
