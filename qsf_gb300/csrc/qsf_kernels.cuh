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
//
// Arithmetic: psi is stored as complex128 between steps; inside a step every pass
// works in block fixed point (int64 components sharing one power-of-two exponent per
// thread block, qsf_fxfft.cuh), because GB300's integer pipes issue ~64x more
// instructions per clock than its FP64 pipe.  Intermediate passes write int64 pairs
// into psi's own buffer together with their block exponents; the next pass aligns every
// element to the smallest exponent of the producing pass.  Phase tables are stored in
// 2^62 fixed point with magnitude <= 1.  Norm and E_pot partials are exact 128-bit
// integer sums per block.
#pragma once
#include "qsf_fft.cuh"
#include "qsf_fxfft.cuh"
#include "qsf_tuning.h"

namespace qsf {

constexpr int kMaxDim = 3;
// Shape of the row / axis pass kernels per line length, as the autotuner measured it
// (qsf_tuning.h): points per block (a tile of whole lines, 1024-4096 points) and
// threads per block, which together set the points per thread and with them the radix
// plan (16 points: radix 16, 8: radix 8).  The autotuner's candidate builds define
// QSF_TILE and QSF_ROW_THREADS to force one shape everywhere.
#ifdef QSF_ROW_THREADS
__host__ __device__ constexpr int row_threads(int) { return QSF_ROW_THREADS; }
#else
__host__ __device__ constexpr int row_threads(int n) { return tuned_row_threads(n); }
#endif
#ifdef QSF_TILE
__host__ __device__ constexpr int tile_size(int) { return QSF_TILE; }
#else
__host__ __device__ constexpr int tile_size(int n) { return tuned_tile(n); }
#endif
// points per block: the tile, or one whole line when lines are longer
__host__ __device__ constexpr int tile_pts(int n) { return n > tile_size(n) ? n : tile_size(n); }
__host__ __device__ constexpr int row_ppt(int n) { return tile_pts(n) / row_threads(n); }
constexpr int kLinePptDiv = 512;  // threads of the one-CTA line kernel (kLineThreads)
// Points per thread of the one-CTA line kernel (512 threads, one line of n points): a
// line shorter than 8192 points leaves threads idle in radix-16 passes, and with one
// CTA per line the per-thread work sets the step's latency, so shorter lines take
// smaller radices; the choice per length comes from the autotuner (tuned_line_ppt,
// qsf_tuning.h).  At least n / 512 points per thread (the line must fit the threads);
// the autotuner's candidate builds force one value with QSF_LINE_PPT.
#ifdef QSF_LINE_PPT
__host__ __device__ constexpr int line_ppt(int n) { return n / kLinePptDiv > QSF_LINE_PPT ? n / kLinePptDiv : QSF_LINE_PPT; }
#else
__host__ __device__ constexpr int line_ppt(int n) {
  return n / kLinePptDiv > tuned_line_ppt(n) ? n / kLinePptDiv : tuned_line_ppt(n);
}
#endif
constexpr int kLineThreads = 512;
constexpr int kMaxFluxBorders = 16;
// 1D lines of 1024 .. 8192 points (powers of two): one step spread over a cluster of
// CTAs (k_line_step_mc) instead of one CTA.  Off by default: measured on GB300 it was
// slower than the one-CTA line kernel (4096 points 0.095 vs 0.073 ms per step, 1024
// 0.071 ms, 2048 0.080 ms, 8192 0.104 ms; every distributed-shared-memory access and
// the two cluster barriers per pass cost more than the per-SM work they spread)
#ifndef QSF_LINE_CLUSTER
#define QSF_LINE_CLUSTER 0
#endif
// resident blocks per SM the FFT kernels are compiled for (caps registers per thread)
#ifndef QSF_FFT_MIN_BLOCKS
#define QSF_FFT_MIN_BLOCKS 2
#endif
// resident blocks per SM the row / axis pass kernels are compiled for: twice as many
// for blocks of 128 threads or fewer (the registers per thread stay the same)
__host__ __device__ constexpr int row_min_blocks(int n) {
  return row_threads(n) <= 128 ? 2 * QSF_FFT_MIN_BLOCKS : QSF_FFT_MIN_BLOCKS;
}

struct AxisDev {
  int n, n2;
  int shift;  // log2(n) when n is a power of two, else -1
  long long stride;
  double dx, xmin, dp, inv_2dx;
  const double2* tw;     // exp(-2 pi i t / n), t < n
  const longlong2* twx;  // the same twiddles in 2^62 fixed point
#if QSF_TWQ
  const int4* twf;  // the 2^62 twiddles as signed 32-bit halves (fmul_tw), read by fft_fx
#else
  const longlong2* twf;
#endif
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
  int free_mask;  // region of a multi-region grid: axes kept in momentum space (bit d)
  int multi;      // multi-region grid: partial potentials, no absorber in evolve
  int abs_kind;     // QSF_ABS_CAP or QSF_ABS_COS8
  double abs_rate;  // cos^(1/8) mask: applications per unit time (1 / mask_dt)
  double2* psi;
  // TMA tensor maps (CUtensorMap, 128 bytes, 64-byte aligned, in device memory) of psi
  // for the strided-axis passes of axis d < dim - 1: psi as 64-bit words, dims
  // {2 * stride_d, n_d, outer}, box {2 * tile columns, tma_box_rows(n_d), 1}; null when
  // the driver offers no encoder (the passes then copy with cp.async)
  const void* tmap[kMaxDim];
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

// Where a member-operation kernel finds its coupling values when they live on the
// device (a step program replayed from a graph): the row at c + (*step) * stride + off
// for the current step index *step; c == nullptr: the kernel's by-value arguments.
struct CoupDev {
  const double* c;
  const long long* step;
  long long stride;
  int off;
};
__device__ __forceinline__ void coup_load(const CoupDev& cd, double* cv) {
  if (!cd.c) return;
  const double* p = cd.c + (*cd.step) * cd.stride + cd.off;
  cv[0] = p[0];
  cv[1] = p[1];
  cv[2] = p[2];
}

struct StepDev {
  int mode;  // 1 IM, 2 RE
  double dt;
  long long nsteps;
  const double* coupling;  // device copy of the per-step coupling rows (may be null)
  int coup_stride;         // 3 (velocity gauge) or 6 (length gauge)
  // phase tables in the split form (split62: 2^62 fixed point as signed 32-bit halves)
  const int4* xs;          // static X half-step factor per point (dt/2, incl. absorber), * 2^-xs_exp
  const long long* Vx;     // potential per point in 2^vshift fixed point
  int4* ptab;              // [dim][nmax] P-phase tables of the current step (|.| <= 1)
  int4* xdyn;              // [3][dim][nmax] length-gauge factors: open half, close half, next open half
  int xs_exp;              // exponent taken out of xs (imaginary time: factors above 1)
  int vshift;              // Vx = round(V * 2^vshift)
  int l2m;                 // 1/m = m_mant * 2^-l2m, m_mant in (0.5, 1] (folded into axis 0's P table)
  double m_mant;
  int* texp;               // [3][3] exponents taken out of the per-step tables (set by k_tables)
  int* gmin;               // [kGmin] minimum block exponent of each fixed-point pass (gmin_slot)
  int* sc;                 // [4][scmax] block exponents of each fixed-point pass
  int scmax;
  // fused: a sub-step's closing row pass also applies the next sub-step's opening X half
  // and forward transform (ψ stays in fixed point between the steps of a call); the
  // pending Normalize factor then folds into the next sub-step's axis-0 P table
  int fused;
  // E_kin (QSF_OBS_EKIN) at the end of every ekin_every-th step of the call and of its
  // last step; such a step ends with psi_n stored as complex128 (its other transforms
  // need it) and the next one opens from there, the steps between stay fused
  int ekin_every;
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
  // control (device): ctl[0] sub-step within call (k_finalize's), ctl[1] stop after
  // this sub-step (or nsteps), ctl[2] steps done, ctl[3] finalize block counter,
  // ctl[4] NaN flag, ctl[5] sub-step of the pass kernels (k_tables copies it from
  // ctl[6]), ctl[6] next sub-step of the pass kernels (advanced by the sub-step's last
  // pass).  The two counters let k_finalize of one sub-step run beside the next
  // sub-step's tables and first passes.
  // nsteps counts sub-steps: steps * substeps (MultiProductSplit order).
  int substeps;
  long long* ctl;
  double* energy_state;  // [0] last E
  double* rows;          // [nsteps][3 + nborders]
  double* scale;         // pending Normalize factor (1 when none)
};

__device__ __forceinline__ bool step_active(const StepDev& S) { return S.ctl[0] <= S.ctl[1] && S.ctl[0] < S.nsteps; }
// whether sub-step `sub` ends a step whose observables include E_kin
__device__ __forceinline__ bool ekin_at(const StepDev& S, long long sub) {
  if (!(S.obs & 4u) || (sub + 1) % S.substeps) return false;
  const long long step = sub / S.substeps;
  return (step + 1) % S.ekin_every == 0 || sub + 1 >= S.nsteps || sub >= S.ctl[1];
}
// hint: move the 128-byte line holding p from DRAM into L2 (p must be in an allocation)
__device__ __forceinline__ void prefetch_l2(const void* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }
__device__ __forceinline__ bool pass_active(const StepDev& S) { return S.ctl[5] <= S.ctl[1] && S.ctl[5] < S.nsteps; }

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

// ReducedDimInteraction::partial (potential.h:144-178): the interactions of the bounded
// coordinates of region fc (free-axis mask), same operation order
__device__ __forceinline__ double partial_potential(const GridDev& g, int fc, const double* c) {
  auto ne = [&](double x) { return g.NEcharge / sqrt(x * x + g.Nsoft); };
  auto ee = [&](double x, double y) {
    return g.pot == 1 ? g.EEcharge / sqrt((x - y) * (x - y) + x * y + g.Esoft)
                      : g.EEcharge / sqrt((x - y) * (x - y) + g.Esoft);
  };
  if (g.dim == 1) return fc == 0 ? ne(c[0]) : 0.0;
  if (g.dim == 2) {
    if (fc == 0) return ee(c[0], c[1]) + ne(c[0]) + ne(c[1]);
    if (fc == 2) return ne(c[0]);
    if (fc == 1) return ne(c[1]);
    return 0.0;
  }
  switch (fc) {
    case 0: return ee(c[0], c[1]) + ee(c[1], c[2]) + ee(c[2], c[0]) + ne(c[0]) + ne(c[1]) + ne(c[2]);
    case 4: return ee(c[0], c[1]) + ne(c[0]) + ne(c[1]);
    case 2: return ee(c[0], c[2]) + ne(c[0]) + ne(c[2]);
    case 1: return ee(c[1], c[2]) + ne(c[1]) + ne(c[2]);
    case 6: return ne(c[0]);
    case 5: return ne(c[1]);
    case 3: return ne(c[2]);
    default: return 0.0;
  }
}

// potential at a point (potential.h:130-143 and 40-44), same operation order
__device__ __forceinline__ double potential_at(const GridDev& g, const double* c) {
  if (g.pot == 3) return 0.0;
  if (g.multi) return partial_potential(g, g.free_mask, c);
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
  if (g.m <= 0x7fffffffLL) {  // 32-bit index arithmetic; shifts for power-of-two axes
    unsigned q = (unsigned)p;
    for (int d = g.dim - 1; d >= 0; --d) {
      const AxisDev& a = g.ax[d];
      if (a.shift >= 0) {
        idx[d] = (int)(q & ((1u << a.shift) - 1u));
        q >>= a.shift;
      } else {
        idx[d] = (int)(q % (unsigned)a.n);
        q /= (unsigned)a.n;
      }
    }
    return;
  }
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
  if (g.abs_kind == 1) {  // cos^(1/8) mask M = prod_d cos(pi/2 nodes_d / nCAP)^(1/8), to the power delta / mask_dt
    double lsum = 0.0;
    for (int d = 0; d < g.dim; ++d)
      if (nodes[d] > 0) lsum += log(cos(1.5707963267948966 * ((double)nodes[d] / (double)g.nCAP)));
    return exp(delta * g.abs_rate * 0.125 * lsum);
  }
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

// ------------------------------------------------------------ fixed-point helpers
// Rows per block of the last-axis passes and columns per tile of the strided-axis
// passes are compile-time functions of the line length (<= kMaxTile points per block),
// so a consumer pass finds the block that produced an element with a few integer ops.
// 16-byte global -> shared copy that bypasses registers (cp.async, cache-global); the
// copies of a thread are visible to that thread after cp_async_wait_all.
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Contiguous global -> shared copies on the TMA engine (cp.async.bulk completing on an
// mbarrier): one thread issues the copy of a whole tile, the others wait on the barrier.
__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// dst, src 16-byte aligned, bytes a multiple of 16
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned phase) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(phase)
      : "memory");
  return ok != 0;
}
// one box of a 3D tensor map into shared memory, completing on the barrier; the first
// coordinate (64-bit words) is a multiple of 2, so every copy starts on 16 bytes
__device__ __forceinline__ void tma_load3(void* dst, const void* tmap, int x, int y, int z, unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
          smem_u32(dst)),
      "l"(tmap), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}
// bounded wait for phase `phase` of the barrier: false when the limit ran out (the
// caller records the failure; nothing spins without end)
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned phase) {
  for (int it = 0; it < (1 << 20); ++it)
    if (mbar_try_wait(bar, phase)) return true;
  return false;
}

// (i, c) = (e / Ch, e % Ch) for e = e0, e0 + step, e0 + 2 step, ... without a division
// per element (Ch is a runtime tile width in the strided-axis passes)
struct TileWalk {
  int i, c, di, dc, Ch;
  __device__ __forceinline__ TileWalk(int e0, int step, int ch)
      : i(e0 / ch), c(e0 % ch), di(step / ch), dc(step % ch), Ch(ch) {}
  __device__ __forceinline__ void next() {
    i += di;
    c += dc;
    if (c >= Ch) {
      c -= Ch;
      ++i;
    }
  }
};

__host__ __device__ constexpr int row_lines(int n) { return tile_pts(n) / n; }
// rows of one TMA box of a strided-axis tile: the largest divisor of n up to 256 (the
// box limit), so that the boxes cover the n rows exactly and none writes past the tile
__host__ __device__ constexpr int tma_box_rows(int n) {
  int b = n < 256 ? n : 256;
  while (n % b) --b;
  return b;
}
__host__ __device__ constexpr int tile_cols(int n) { return (tile_pts(n) / n) < 64 ? (tile_pts(n) / n) : 64; }

// Passes that leave the wavefunction in fixed point inside a step; each block of a
// pass records its exponent in sc[pass][block] and the pass minimum in gmin[pass]:
// 0 last-axis rows (open), 1 axis-1 tiles forward (3D), 2 axis-0 tiles, 3 axis-1
// tiles inverse (3D).  The next pass aligns every element to gmin of its producer.
template <int N>
__device__ __forceinline__ int producer_block(int pass, int dim, long long p) {
  if (pass == 0) return (int)((p / N) / row_lines(N));
  if (pass == 2) {  // axis 0: a single outer index, inner = m / N
    const long long inner = dim == 2 ? (long long)N : (long long)N * N;
    const long long C = tile_cols(N) < inner ? tile_cols(N) : inner;
    return (int)((p % inner) / C);
  }
  // axis 1 of a 3D grid: outer index i0, inner = N
  constexpr long long C = tile_cols(N) < N ? tile_cols(N) : N;
  constexpr long long tpo = (N + C - 1) / C;
  const long long o = p / ((long long)N * N);
  return (int)(o * tpo + (p % N) / C);
}

// Exponent bookkeeping of the step's fixed-point tables: every table is stored with
// magnitude <= 1 in 2^62 fixed point; a table whose exact values exceed 1 (imaginary
// time) is stored times 2^-e and e is added back to the block exponent.
//   texp[0][d]: P table of axis d, texp[1][d] / texp[2][d]: length-gauge X tables of
//   axis d (open / close half), texp[3][d]: opening half of the next sub-step (fused).
//   The static X table's exponent is StepDev::xs_exp.
constexpr int kTexp = 12;
// Pass minima: [1..3] passes 1-3 of the sub-step; pass 0 alternates between [0] and
// [4] with the parity of the sub-step, because in fused mode the closing pass of
// sub-step k produces pass 0 of sub-step k + 1 while pass 0 of k may still be read.
constexpr int kGmin = 5;
__device__ __forceinline__ int gmin_slot(int pass, long long sub) { return pass ? pass : ((sub & 1) ? 4 : 0); }

// sum |x|^2 and sum V |x|^2 of fixed-point values, exact in 128-bit integers
struct Acc128 {
  unsigned long long lo;
  long long hi;
};
__device__ __forceinline__ void acc_add(Acc128& a, unsigned long long lo, long long hi) {
  const unsigned long long l = a.lo + lo;
  a.hi += hi + (l < lo ? 1 : 0);
  a.lo = l;
}
__device__ __forceinline__ double acc_value(const Acc128& a) {
  return (double)a.hi * 18446744073709551616.0 + (double)a.lo;
}

// Norm and E_pot partial sums of a block of psi_n in fixed point (components below
// 2^56 after the block's common shift q): |x|^2 exactly, V|x|^2 with |x|^2 >> 50 and V
// in 2^vshift fixed point (|V| < 2^50 there).
__device__ __forceinline__ void acc_point_v(Acc128& an, Acc128& av, longlong2 x, int q, long long v, bool epot) {
  const long long xr = q ? fshift(x.x, -q) : x.x, xi = q ? fshift(x.y, -q) : x.y;
  const unsigned long long ar = (unsigned long long)(xr < 0 ? -xr : xr), ai = (unsigned long long)(xi < 0 ? -xi : xi);
  const unsigned long long l1 = ar * ar, l2 = ai * ai;
  const unsigned long long lo = l1 + l2;
  const unsigned long long hi = __umul64hi(ar, ar) + __umul64hi(ai, ai) + (lo < l1 ? 1ull : 0ull);
  acc_add(an, lo, (long long)hi);
  if (epot) {
    const long long n2 = (long long)((hi << 14) | (lo >> 50));
    acc_add(av, (unsigned long long)n2 * (unsigned long long)v, __mul64hi(n2, v));
  }
}
__device__ __forceinline__ void acc_point(Acc128& an, Acc128& av, longlong2 x, int q, const long long* Vx, long long p,
                                          bool epot) {
  const long long xr = q ? fshift(x.x, -q) : x.x, xi = q ? fshift(x.y, -q) : x.y;
  const unsigned long long ar = (unsigned long long)(xr < 0 ? -xr : xr), ai = (unsigned long long)(xi < 0 ? -xi : xi);
  const unsigned long long l1 = ar * ar, l2 = ai * ai;
  const unsigned long long lo = l1 + l2;
  const unsigned long long hi = __umul64hi(ar, ar) + __umul64hi(ai, ai) + (lo < l1 ? 1ull : 0ull);
  acc_add(an, lo, (long long)hi);
  if (epot) {
    const long long n2 = (long long)((hi << 14) | (lo >> 50));
    const long long v = Vx[p];
    acc_add(av, (unsigned long long)n2 * (unsigned long long)v, __mul64hi(n2, v));
  }
}

// Phase factors (|components| <= 1) are stored in 2^62 fixed point as the signed
// 32-bit halves of each component (int4 {re lo, re hi, im lo, im hi}, as the FFT's
// twiddles), with every low half kept away from -2^31 so that it can be negated.  A
// product x * f (fapply) returns x * f / 4 from twelve 32 x 32 -> 64-bit multiply-adds
// (fmul_tw) and needs |x| < 2^61.
__device__ __forceinline__ int4 split62(double2 f) {
  long long a = __double2ll_rn(f.x * 4611686018427387904.0), b = __double2ll_rn(f.y * 4611686018427387904.0);
  if ((a & 0xffffffffLL) == 0x80000000LL) ++a;
  if ((b & 0xffffffffLL) == 0x80000000LL) ++b;
  return make_int4((int)a, split_hi(a), (int)b, split_hi(b));
}
__device__ __forceinline__ int4 split_fx(longlong2 v) {
  if ((v.x & 0xffffffffLL) == 0x80000000LL) ++v.x;
  if ((v.y & 0xffffffffLL) == 0x80000000LL) ++v.y;
  return make_int4((int)v.x, split_hi(v.x), (int)v.y, split_hi(v.y));
}
// a * w / 2^64 for a real w given as its signed halves (wl, wh)
__device__ __forceinline__ i64 mul_re(i64 a, int wl, int wh) {
  const int al = (int)a, ah = split_hi(a);
  const i64 m = (i64)ah * wl + (i64)al * wh + (1LL << 31);
  return (m >> 32) + (i64)ah * wh;
}
// x * f / 4 (real f: imaginary-time X factors, only f's real part is read)
__device__ __forceinline__ longlong2 fapply(longlong2 x, int4 f, bool real_f) {
  return real_f ? make_longlong2(mul_re(x.x, f.x, f.y), mul_re(x.y, f.x, f.y)) : fmul_tw(x, f);
}
// x * 4 (renormalises after two products: the data stay below 2^61)
__device__ __forceinline__ longlong2 fshl2(longlong2 x) {
  return make_longlong2((i64)((u64)x.x << 2), (i64)((u64)x.y << 2));
}
// k factors applied in a row (fapply each, fshl2 after every second one that is
// followed by another): the exponent the value moves by and a bound on the change of
// its bit length (each product adds at most one bit, for the complex modulus)
__host__ __device__ constexpr int xshift(int k) { return 2 * k - 2 * ((k - 1) / 2); }
__host__ __device__ constexpr int xbits(int k) { return 2 * ((k - 1) / 2) - k; }

// Largest exponent shift that brings a block whose largest component has `bits`
// bits below 2^(62 - guard of the first pass of an N-point transform)
template <int N>
__device__ __forceinline__ int first_pass_shift(int bits) {
  return bits == 0 ? 0 : (62 - fguard(radix_at(N, 0))) - bits;
}
// shift that brings a block's largest component to 61 bits before phase products: the
// split products need |x| < 2^61 and return x * f / 4, so starting at the top keeps
// their rounding (1 unit of the output) at 2^-59 of the block maximum
__device__ __forceinline__ int product_headroom(int bits) { return bits ? 61 - bits : 0; }

// value of one per-step table entry: kind 0 P phase (hamiltonian.h:52-58: kinetic and,
// in the velocity gauge, A.k), kind 1 / 2 length-gauge x.E factor of the open / close
// X half (hamiltonian.h:60-66 via DipoleCoupling), kind 3 the open half of the next
// sub-step (coupling row `cn`)
__device__ __forceinline__ double2 table_entry(const GridDev& g, const StepDev& S, const double* cp, const double* cn,
                                               int kind, int d, int i) {
  const AxisDev& a = g.ax[d];
  if (kind == 0) {
    double A = 0.0;
    if (g.gauge != 1 && cp && g.n_fields) {
      int dd = d;
      if (g.p_swap && g.dim >= 2 && d < 2) dd = 1 - d;
      A = cp[dd];
    }
    const double k = kpos(a, i);
    return expop(S.mode, S.dt * (0.5 * k * k + k * A));
  }
  const double* row = kind == 3 ? cn : cp;
  const double E = (row && g.n_fields) ? row[(kind == 2 ? 3 : 0) + d] : 0.0;
  return expop(S.mode, (S.dt * 0.5) * (xpos(a, i) * E));
}

// One (kind, axis) table of a step's per-step tables, or its slice `part` of `tb` (all
// threads of the block call it; red: 32 doubles of shared memory, e_sh: one shared int)
__device__ __forceinline__ void tables_one(const GridDev& g, const StepDev& S, long long sub, int kind, int d, int part,
                                           int tb, double* red, int* e_sh) {
  const int D = g.dim;
  if (kind > 0 && g.gauge != 1) return;
  if (kind == 3 && (!S.fused || sub + 1 >= S.nsteps)) return;
  const double* cp = S.coupling ? S.coupling + sub * S.coup_stride : nullptr;
  const double* cn = (S.coupling && sub + 1 < S.nsteps) ? S.coupling + (sub + 1) * S.coup_stride : nullptr;
  const int n = g.ax[d].n;
  double mant = 1.0;
  if (kind == 0 && d == 0) {
    mant = S.m_mant;
    if (S.fused && S.normalize) mant *= *S.scale;
  }
  double mx = mant;  // real time: phases of modulus 1 times the mantissa
  if (S.mode == 1) {  // imaginary time: real factors, maximum over the table
    mx = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) mx = fmax(mx, table_entry(g, S, cp, cn, kind, d, i).x * mant);
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x == 0)
      for (int w = 1; w < (int)(blockDim.x >> 5); ++w) mx = fmax(mx, red[w]);
  }
  if (threadIdx.x == 0) {
    int e = 0;
    if (mx > 1.0) frexp(mx, &e);  // mx < 2^e
    *e_sh = e;
    if (part == 0) S.texp[kind * 3 + d] = e;
  }
  __syncthreads();
  const double sc = ldexp(mant, -*e_sh);
  int4* out = kind == 0 ? S.ptab + (size_t)d * S.nmax : S.xdyn + ((size_t)(kind - 1) * D + d) * S.nmax;
  const int chunk = (n + tb - 1) / tb;
  const int i1 = min(n, (part + 1) * chunk);
  for (int i = part * chunk + threadIdx.x; i < i1; i += blockDim.x) {
    const double2 f = table_entry(g, S, cp, cn, kind, d, i);
    out[i] = split62(make_double2(fmin(fmax(f.x * sc, -1.0), 1.0), fmin(fmax(f.y * sc, -1.0), 1.0)));
  }
}

__device__ __forceinline__ void flux_block(const GridDev& g, const FluxPoint* __restrict__ fpts, const FluxTerm* __restrict__ fterms,
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

// End of a (sub-)step, run by one block once every block's partials and flux partials
// (nfb blocks of them) are in memory: fixed-order sums, the observables row, the
// Normalize factor, the convergence test and the step counters.  red: 32 *
// kMaxFluxBorders doubles of shared memory.
__device__ __forceinline__ void finalize_tail(const GridDev& g, const StepDev& S, long long sub, bool step_end,
                                              long long step, int nb, int nfb, double* red) {
  if (!step_end) {
    if (threadIdx.x == 0) {
      if (S.normalize) *S.scale = 1.0;  // no Normalize between sub-steps
      S.ctl[3] = 0;
      S.ctl[0] = sub + 1;
    }
    return;
  }
  // last block: deterministic sums in a fixed order
  const bool ek = ekin_at(S, sub);
  double acc[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  for (int i = threadIdx.x; i < S.nrowblk; i += blockDim.x) {
    acc[0] += S.partials[0 * S.pmax + i];
    acc[1] += S.partials[1 * S.pmax + i];
    acc[2 + g.dim - 1] += S.partials[(2 + g.dim - 1) * S.pmax + i];
  }
  if (ek) {
    for (int d = 0; d < g.dim - 1; ++d)
      for (int i = threadIdx.x; i < S.naxblk[d]; i += blockDim.x) acc[2 + d] += S.partials[(2 + d) * S.pmax + i];
  }
  __shared__ double fsum[kMaxFluxBorders];
  if (threadIdx.x < nb) {  // per border, the blocks' partials in block order
    double v = 0.0;
    for (int k = 0; k < nfb; ++k) v += S.fpartials[k * kMaxFluxBorders + threadIdx.x];
    fsum[threadIdx.x] = v;
  }
  block_sum<5>(acc, red);  // its barriers also publish fsum
  if (threadIdx.x == 0) {
    const double norm = acc[0] * g.dV;
    const double epot = acc[1] * g.dV;
    double ekin = 0.0;
    if (ek) {
      for (int d = 0; d < g.dim; ++d) ekin += (double)(g.m / g.ax[d].n) * acc[2 + d];
      ekin = 0.5 * g.dVm * ekin;
    }
    const int ncol = 3 + nb;
    double* row = S.rows + step * ncol;
    row[0] = norm;
    row[1] = epot;
    row[2] = ekin;
    for (int b = 0; b < nb; ++b) row[3 + b] = fsum[b] * g.dV / g.ax[0].dx;
    if (!(norm > 0.0) || isnan(epot) || isnan(ekin)) S.ctl[4] = 1;
    if (S.normalize && norm > 0.0) *S.scale = sqrt(1.0 / norm);
    // the convergence test needs E = E_pot + E_kin: with E_kin on every k-th step only,
    // it runs on those steps (comparing with the previous one that had it)
    if (S.mode == 1 && S.state_accuracy > 0.0 && (ek || !(S.obs & 4u))) {
      const double se = (S.energy_after_normalize & 1) ? 1.0 / norm : 1.0;
      const double sk = (S.energy_after_normalize & 2) ? 1.0 / norm : 1.0;
      const double E = epot * se + ekin * sk;
      const double dE = E - S.energy_state[0];
      S.energy_state[0] = E;
      // converged: one more step runs (its last sub-step is sub + substeps)
      if (S.ctl[1] >= S.nsteps && fabs(dE) <= S.state_accuracy) S.ctl[1] = sub + S.substeps;
    }
    S.ctl[2] = step + 1;
    S.ctl[3] = 0;
    S.ctl[0] = sub + 1;
  }
}

#ifdef QSF_DEFINE_KERNELS
// ------------------------------------------------------------ tables
// Range of the potential (for its fixed-point scale and the imaginary-time X factor
// bound): out[0] = max over points of V (ordered-integer encoding), out[1] = max of -V.
__device__ __forceinline__ long long ordered_bits(double x) {
  long long i = __double_as_longlong(x);
  return i < 0 ? i ^ 0x7fffffffffffffffLL : i;
}
__global__ void k_vrange(GridDev g, long long* out) {
  __shared__ long long r0[32], r1[32];
  long long a = LLONG_MIN, b = LLONG_MIN;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < g.m; p += stride) {
    int idx[kMaxDim];
    double c[kMaxDim];
    unflatten(g, p, idx);
    for (int d = 0; d < g.dim; ++d) c[d] = xpos(g.ax[d], idx[d]);
    const double v = potential_at(g, c);
    a = max(a, ordered_bits(v));
    b = max(b, ordered_bits(-v));
  }
  for (int o = 16; o > 0; o >>= 1) {
    a = max(a, __shfl_down_sync(0xffffffffu, a, o));
    b = max(b, __shfl_down_sync(0xffffffffu, b, o));
  }
  if ((threadIdx.x & 31) == 0) {
    r0[threadIdx.x >> 5] = a;
    r1[threadIdx.x >> 5] = b;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
      a = max(a, r0[w]);
      b = max(b, r1[w]);
    }
    atomicMax(&out[0], a);
    atomicMax(&out[1], b);
  }
}

// Static tables for X(delta): expOp(delta V) * absorb(delta) per point in 2^62 fixed
// point times 2^-xs_exp, and the potential in 2^vshift fixed point.
__global__ void k_build_static(GridDev g, int mode, double delta, int xs_exp, int4* xsx, long long* Vx,
                               int vshift) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  const double vs = ldexp(1.0, vshift), xsc = ldexp(1.0, -xs_exp);
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < g.m; p += stride) {
    int idx[kMaxDim];
    double c[kMaxDim];
    unflatten(g, p, idx);
    for (int d = 0; d < g.dim; ++d) c[d] = xpos(g.ax[d], idx[d]);
    const double v = potential_at(g, c);
    Vx[p] = __double2ll_rn(v * vs);
    const double2 f = expop(mode, delta * v);
    const double a = (g.multi ? 1.0 : absorb_at(g, delta, idx)) * xsc;
    const double2 fa = make_double2(f.x * a, f.y * a);
    xsx[p] = split62(make_double2(fmin(fmax(fa.x, -1.0), 1.0), fmin(fmax(fa.y, -1.0), 1.0)));
  }
}

// Per-step tables: `tb` blocks per (kind, axis) table, each storing a contiguous slice.
// A table whose values exceed 1 in magnitude (imaginary time, or a Normalize factor
// folded in) is stored times 2^-e, e from its maximum (every block of the table
// evaluates that maximum, so the slices agree), and e is recorded in texp.  Axis 0's P
// table carries the mantissa of 1/m (its power of two goes into the exponent) and, in
// fused mode, the pending Normalize factor.  Block 0 resets the pass minima this
// sub-step's passes will produce.
__global__ void __launch_bounds__(256) k_tables(const GridDev* __restrict__ Gs, const StepDev* __restrict__ Ss,
                                                int tb) {
  const GridDev& g = Gs[blockIdx.y];
  const StepDev& S = Ss[blockIdx.y];
  // the sub-step of this step's passes; every block stores the same value, also when
  // the step is inactive (its passes then read an inactive sub-step too)
  const long long sub = S.ctl[6];
  if (threadIdx.x == 0) S.ctl[5] = sub;
  if (!(sub <= S.ctl[1] && sub < S.nsteps)) return;
  __shared__ double red[32];
  __shared__ int e_sh;
  const int D = g.dim;
  const int table = blockIdx.x / tb, part = blockIdx.x % tb;
  const int kind = table / D, d = table % D;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    S.gmin[1] = S.gmin[2] = S.gmin[3] = 0x7fffffff;
    S.gmin[gmin_slot(0, sub + 1)] = 0x7fffffff;               // produced by this sub-step's closing pass
    if (!S.fused || sub == 0) S.gmin[gmin_slot(0, sub)] = 0x7fffffff;  // produced by this sub-step's opening pass
  }
  tables_one(g, S, sub, kind, d, part, tb, red, &e_sh);
}

#endif  // QSF_DEFINE_KERNELS

// Factors of the X half `half` (0 opens the step, 1 closes it, 2 opens the next
// sub-step): the static factor and, in the length gauge, one x.E factor per axis.
__device__ __forceinline__ int xfactors(const GridDev& g) { return 1 + (g.gauge == 1 ? g.dim : 0); }
// The X half applied to x at point p (row r of the last axis, position j on it): the
// factors one after another (fapply; fshl2 after the second when more follow), x below
// 2^61.  NA is the length of the axes before the last one when known at compile time
// (0: read it).  The value moves by xhalf_exp (bits <= in + xbits(xfactors(g))).
template <int NA = 0>
__device__ __forceinline__ longlong2 xhalf(const GridDev& g, const StepDev& S, longlong2 x, long long p, long long r,
                                           int j, int half, bool real_f) {
  x = fapply(x, S.xs[p], real_f);
  if (g.gauge == 1) {
    const int D = g.dim;
    const int4* t = S.xdyn + (size_t)half * D * S.nmax;
    x = fapply(x, t[(D - 1) * S.nmax + j], false);
    long long rr = r;
    int k = 2;
    for (int dd = D - 2; dd >= 0; --dd) {
      const long long n = NA ? NA : g.ax[dd].n;
      const int ii = (int)(rr % n);
      rr /= n;
      if (k % 2 == 0) x = fshl2(x);
      x = fapply(x, t[dd * S.nmax + ii], false);
      ++k;
    }
  }
  return x;
}
// exponent taken out of the factors of one half (their table exponents) plus the
// exponent the k products move the value by
__device__ __forceinline__ int xfactor_exp(const GridDev& g, const StepDev& S, int half) {
  int e = S.xs_exp;
  if (g.gauge == 1)
    for (int d = 0; d < g.dim; ++d) e += S.texp[(1 + half) * 3 + d];
  return e;
}
__device__ __forceinline__ int xhalf_exp(const GridDev& g, const StepDev& S, int half) {
  return xfactor_exp(g, S, half) + xshift(xfactors(g));
}

// psi (double) -> fixed point: the block exponent from the largest biased exponent
// em of the block puts the largest component at 61 bits (below 2^61, as the phase
// products need; the pending Normalize factor is at most 1)
template <int N>
__device__ __forceinline__ int scale_from_exponent(int em) {
  return 61 - (em - 1022);
}

// pending Normalize factor s = F 2^-62 * 2^k with F in [2^61, 2^62)
__device__ __forceinline__ void split_scale(double s, long long& F, int& k) {
  int e;
  const double f = frexp(s, &e);
  F = __double2ll_rn(f * 4611686018427387904.0);
  k = e;
}

// Loads psi (double) of `cnt` contiguous points at `base` into smx (one global read,
// staged in smem as doubles, converted in place) as fixed point times the pending
// Normalize factor and the opening X factor; returns the block exponent and (in bits)
// the bit length of the largest component.
template <int N>
__device__ __forceinline__ int open_block(const GridDev& g, const StepDev& S, longlong2* smx, long long base, int cnt,
                                          long long row0, int* red, int& bits) {
  const bool real_f = S.mode == 1 && g.gauge != 1;
  double2* sd = reinterpret_cast<double2*>(smx);
  int em = 0;
#pragma unroll 4
  for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
    const double2 v = g.psi[base + e];
    sd[e] = v;
    em = max(em, max(dexp(v.x), dexp(v.y)));
  }
  em = block_max_int(em, red);
  // an Inf or NaN component (exponent field all ones) has no fixed-point image: flag
  // the solve (QSF_ENUMERIC) instead of converting garbage
  if (em >= 0x7ff && threadIdx.x == 0) S.ctl[4] = 1;
  const int s_in = scale_from_exponent<N>(em);
  int scale = s_in;
  long long F = 0;
  int k = 0;
  const bool use_s = !S.fused && S.normalize && *S.scale != 1.0;
  if (use_s) {
    split_scale(*S.scale, F, k);
    scale -= k;
  }
  u64 mag = 0;
#pragma unroll 4
  for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
    const long long p = base + e;
    const double2 v = sd[e];  // written by this thread
    longlong2 x = make_longlong2(d2fx(v.x, s_in), d2fx(v.y, s_in));
    if (use_s) x = make_longlong2(mulq62(x.x, F), mulq62(x.y, F));
    x = xhalf<N>(g, S, x, p, row0 + e / N, e % N, 0, real_f);
    smx[e] = x;
    mag |= fmag(x);
  }
  bits = block_max_int(bitlen(mag), red);
  return scale - xhalf_exp(g, S, 0);
}

// psi_n from the block after the last inverse transform (held conjugated in smx when
// conj_in): closing X factor, 1/m's power of two, [store as double], norm / E_pot
// partial sums (exact integers).  On return smx holds psi_n in fixed point with
// exponent `scale` and bit length `bits`.
template <int N>
__device__ __forceinline__ void close_block(const GridDev& g, const StepDev& S, longlong2* smx, long long base, int cnt,
                                            long long row0, int* red, int& scale, int& bits, double* dacc,
                                            bool conj_in, bool store) {
  const bool real_f = S.mode == 1 && g.gauge != 1;
  const int pre = product_headroom(bits);
  u64 mag = 0;
#pragma unroll 4
  for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
    const long long p = base + e;
    longlong2 x = smx[e];
    if (conj_in) x = fconj(x);
    if (pre) x = make_longlong2(fshift(x.x, pre), fshift(x.y, pre));
    x = xhalf<N>(g, S, x, p, row0 + e / N, e % N, 1, real_f);
    smx[e] = x;
    mag |= fmag(x);
  }
  scale += pre - xhalf_exp(g, S, 1) + S.l2m;
  bits = block_max_int(bitlen(mag), red);
  const int q = bits > 56 ? bits - 56 : 0;
  Acc128 an{0ull, 0ll}, av{0ull, 0ll};
  const bool epot = (S.obs & 2u) != 0;
#pragma unroll 4
  for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
    const long long p = base + e;
    const longlong2 x = smx[e];
    if (store) g.psi[p] = make_double2(fx2d(x.x, scale), fx2d(x.y, scale));
    acc_point(an, av, x, q, S.Vx, p, epot);
  }
  dacc[0] = acc_value(an);
  dacc[1] = acc_value(av);
  // block-uniform exponents of the two sums
  dacc[3] = (double)(2 * q - 2 * scale);
  dacc[4] = (double)(2 * q - 2 * scale + 50 - S.vshift);
}

// Fused close of one sub-step and open of the next (no E_kin, psi_n not stored): in one
// sweep over the block (held conjugated in smx after the inverse transform), psi_n =
// f1 x feeds the norm / E_pot sums and becomes f2 psi_n, the next sub-step's opening X
// half, left in smx.  The bit length of psi_n is bounded by that of x plus one (|f1| <=
// 1), which fixes its accumulation shift and product headroom before the sweep.  The
// flux snapshot of psi_n is taken first, at its listed points only.
template <int N>
__device__ __forceinline__ void close_open_block(const GridDev& g, const StepDev& S, longlong2* smx, long long base,
                                                 int cnt, long long row0, int Lh, int* red, int& scale, int& bits,
                                                 double* dacc) {
  const bool real_f = S.mode == 1 && g.gauge != 1;
  // length gauge in 3D: the x.E factors of the first two axes are constant along a row;
  // their product per row and half is formed once, so that a half is three products
  constexpr int kRowPre = 64;
  __shared__ int4 rowpre[2][kRowPre];
  const bool hoist = g.gauge == 1 && g.dim == 3 && Lh <= kRowPre;
  const int4* t1 = S.xdyn + (size_t)1 * 3 * S.nmax;  // close half, axes 0..2
  const int4* t2 = S.xdyn + (size_t)2 * 3 * S.nmax;  // next open half
  if (hoist) {
    for (int t = threadIdx.x; t < 2 * Lh; t += blockDim.x) {
      const int h = t / Lh, rl = t % Lh;
      const long long r = row0 + rl;
      const int4* tab = h ? t2 : t1;
      rowpre[h][rl] = split_fx(fmul62(tw_join(tab[S.nmax + (int)(r % N)]), tw_join(tab[(int)(r / N)])));
    }
    __syncthreads();
  }
  // half h (1: close, 2: next open) at block element e
  auto half = [&](longlong2 x, int e, int h) -> longlong2 {
    const long long p = base + e;
    if (hoist) {
      x = fapply(x, S.xs[p], false);
      x = fapply(x, rowpre[h - 1][e / N], false);
      x = fshl2(x);
      return fapply(x, (h == 1 ? t1 : t2)[2 * S.nmax + e % N], false);
    }
    return xhalf<N>(g, S, x, p, row0 + e / N, e % N, h, real_f);
  };
  const int kf = hoist ? 3 : xfactors(g);  // products per half
  const int pre = product_headroom(bits);
  const int by = min(bits + pre + xbits(kf), 62);
  const int sy = scale + pre - xfactor_exp(g, S, 1) - xshift(kf) + S.l2m;
  const int q = by > 56 ? by - 56 : 0;
  const int pre2 = product_headroom(by);
  if (S.row_ptr) {
    const int e0 = S.row_ptr[row0], e1 = S.row_ptr[row0 + Lh];
    for (int e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
      const int k = (int)(S.snap_idx[e] - base);
      longlong2 x = fconj(smx[k]);
      if (pre) x = make_longlong2(fshift(x.x, pre), fshift(x.y, pre));
      x = half(x, k, 1);
      S.snap[e] = make_double2(fx2d(x.x, sy), fx2d(x.y, sy));
    }
    __syncthreads();
  }
  Acc128 an{0ull, 0ll}, av{0ull, 0ll};
  const bool epot = (S.obs & 2u) != 0;
  u64 mag = 0;
  if (g.gauge != 1) {
    // the velocity gauge and imaginary time: the static factor alone, loaded one
    // element ahead (with the potential) so that the sweep does not wait on memory
    int4 f_next = make_int4(0, 0, 0, 0);
    long long v_next = 0;
    if ((int)threadIdx.x < cnt) {
      f_next = S.xs[base + threadIdx.x];
      if (epot) v_next = S.Vx[base + threadIdx.x];
    }
#pragma unroll 1  // a large body: unrolling costs more in instruction fetch than it gains
    for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
      const int4 f = f_next;
      const long long v = v_next;
      if (e + (int)blockDim.x < cnt) {
        f_next = S.xs[base + e + blockDim.x];
        if (epot) v_next = S.Vx[base + e + blockDim.x];
      }
      longlong2 x = fconj(smx[e]);
      if (pre) x = make_longlong2(fshift(x.x, pre), fshift(x.y, pre));
      x = fapply(x, f, real_f);
      acc_point_v(an, av, x, q, v, epot);
      if (pre2) x = make_longlong2(fshift(x.x, pre2), fshift(x.y, pre2));
      x = fapply(x, f, real_f);
      smx[e] = x;
      mag |= fmag(x);
    }
  } else {
#pragma unroll 1
    for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
      longlong2 x = fconj(smx[e]);
      if (pre) x = make_longlong2(fshift(x.x, pre), fshift(x.y, pre));
      x = half(x, e, 1);
      acc_point(an, av, x, q, S.Vx, base + e, epot);
      if (pre2) x = make_longlong2(fshift(x.x, pre2), fshift(x.y, pre2));
      x = half(x, e, 2);
      smx[e] = x;
      mag |= fmag(x);
    }
  }
  dacc[0] = acc_value(an);
  dacc[1] = acc_value(av);
  dacc[3] = (double)(2 * q - 2 * sy);
  dacc[4] = (double)(2 * q - 2 * sy + 50 - S.vshift);
  scale = sy + pre2 - xfactor_exp(g, S, 2) - xshift(kf);
  bits = block_max_int(bitlen(mag), red);
}

// E_kin part of the last axis: forward transform of psi_n (in smx) and sum k^2 |.|^2
template <int N, int PPT>
__device__ __forceinline__ double ekin_rows(const AxisDev& a, longlong2* smx, const LineSet& ls, int cnt, int scale,
                                            int bits, int* red) {
  const int sh = first_pass_shift<N>(bits);
  int sc = scale + sh, b = 0;
  fft_fx<N, PPT>(smx, ls, a.twf, threadIdx.x, blockDim.x, sc, b, red, sh);
  double ek = 0.0;
  for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
    const double kk = kpos(a, e % N);
    const longlong2 x = smx[e];
    const double xr = fx2d(x.x, sc), xi = fx2d(x.y, sc);
    ek = fma(kk * kk, fma(xr, xr, xi * xi), ek);
  }
  return ek;
}

// ------------------------------------------------------------ row passes
// Rows of the last axis: L rows of N points per block, contiguous in memory.
// Open: psi (double) . [Normalize] . X half . forward FFT -> fixed point (pass 0).
template <int N>
__global__ void __launch_bounds__(row_threads(N), row_min_blocks(N)) k_row_open(const GridDev* __restrict__ Gs,
                                                          const StepDev* __restrict__ Ss, int L) {
  const GridDev& g = Gs[blockIdx.y];
  const StepDev& S = Ss[blockIdx.y];
  if (!pass_active(S)) return;
  const long long sub = S.ctl[5];
  // the previous sub-step's closing pass produced pass 0, unless it ended with psi_n in
  // memory for E_kin
  if (S.fused && sub > 0 && !ekin_at(S, sub - 1)) return;
  extern __shared__ __align__(128) longlong2 smx[];
  __shared__ int red[kRedInts];
  const long long row0 = (long long)blockIdx.x * L;
  const int Lh = (int)min((long long)L, g.m / N - row0);
  const long long base = row0 * N;
  const int cnt = Lh * N;
  int bits = 0;
  int scale = open_block<N>(g, S, smx, base, cnt, row0, red, bits);
  const int sh = first_pass_shift<N>(bits);
  scale += sh;
  const LineSet ls{Lh, N, 1, false};
  fft_fx<N, row_ppt(N)>(smx, ls, g.ax[g.dim - 1].twf, threadIdx.x, blockDim.x, scale, bits, red, sh);
  longlong2* out = reinterpret_cast<longlong2*>(g.psi);
#pragma unroll 4
  for (int e = threadIdx.x; e < cnt; e += blockDim.x) out[base + e] = smx[e];
  if (threadIdx.x == 0) {
    S.sc[blockIdx.x] = scale;
    atomicMin(&S.gmin[gmin_slot(0, sub)], scale);
  }
}

// Loads the elements [obase + i * inner + c] (i < rows, c < Ch) of a fixed-point pass
// output into smx[i * ldc + c] aligned to the pass minimum exponent (conjugated when
// conj); returns the block's common exponent and the bit length of its largest
// component.  With dtab, the alignment shift of element (i, c) is dtab[key], key = i
// (tab_by_row) or (obase + i * inner + c) % N; otherwise it is looked up per element.
template <int N>
__device__ __forceinline__ int load_aligned(const GridDev& g, const StepDev& S, int in_pass, longlong2* smx,
                                            long long obase, long long inner, int rows, int Ch, int ldc, int* red,
                                            int& bits, bool conj, const int* dtab = nullptr,
                                            bool tab_by_row = false, const void* tmap = nullptr,
                                            int tx = 0, int tz = 0) {
  const int gm = S.gmin[gmin_slot(in_pass, S.ctl[5])];
  const int* sc = S.sc + (size_t)in_pass * S.scmax;
  const longlong2* in = reinterpret_cast<const longlong2*>(g.psi);
  const int cnt = rows * Ch;
  u64 mag = 0;
  // on the TMA engine: a contiguous tile (the row passes) as one bulk copy (shared and
  // global addresses on 16 bytes); a strided tile (rows of ldc columns, the axis passes,
  // rows == N) as boxes of tma_box_rows(N) rows of the tensor map, whose columns past
  // the grid's edge arrive as zeros (each box's shared address on 128 bytes).  A tile
  // whose addresses miss those alignments takes the cp.async loads.
  const unsigned sa = smem_u32(smx);
  constexpr int br = tma_box_rows(N);
  const bool contiguous = Ch == 1 && inner == 1 && ldc == 1 && (sa & 15u) == 0 &&
                          ((reinterpret_cast<unsigned long long>(in + obase)) & 15ull) == 0;
  const bool boxes = tmap && rows == N && (sa & 127u) == 0 && ((unsigned)br * (unsigned)ldc * 16u) % 128u == 0;
  if (contiguous || boxes) {
    __shared__ __align__(8) unsigned long long bar;
    if (threadIdx.x == 0) {
      mbar_init(&bar, 1);
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      if (contiguous) {
        mbar_expect_tx(&bar, (unsigned)cnt * 16u);
        bulk_g2s(smx, in + obase, (unsigned)cnt * 16u, &bar);
      } else {
        mbar_expect_tx(&bar, (unsigned)rows * (unsigned)ldc * 16u);
        for (int r0 = 0; r0 < rows; r0 += br) tma_load3(smx + (size_t)r0 * ldc, tmap, tx, r0, tz, &bar);
      }
    }
    if (!mbar_wait(&bar, 0)) {
      S.ctl[4] = 2;  // the copy did not complete in time: the call reports QSF_ETIMEDOUT
      mbar_wait(&bar, 0);
    }
  } else {  // all of this thread's copies in flight at once, then fixed up in place
    TileWalk w(threadIdx.x, blockDim.x, Ch);
    for (int e = threadIdx.x; e < cnt; e += blockDim.x, w.next())
      cp_async16(&smx[w.i * ldc + w.c], in + obase + (long long)w.i * inner + w.c);
    cp_async_wait_all();
  }
  TileWalk w(threadIdx.x, blockDim.x, Ch);
#pragma unroll 4
  for (int e = threadIdx.x; e < cnt; e += blockDim.x, w.next()) {
    const int i = w.i, c = w.c;
    const long long p = obase + (long long)i * inner + c;
    longlong2 x = smx[i * ldc + c];
    const int d = dtab ? dtab[tab_by_row ? i : (int)(p % N)] : gm - sc[producer_block<N>(in_pass, g.dim, p)];
    if (d) x = make_longlong2(fshift(x.x, d), fshift(x.y, d));
    if (conj) x = fconj(x);
    smx[i * ldc + c] = x;
    mag |= fmag(x);
  }
  bits = block_max_int(bitlen(mag), red);
  return gm;
}

// Alignment shifts of a consumer block whose producer depends on one index of N values:
// dtab[k] = gmin - sc[producer(k)], producer(k) = base_block + (kbase + k) / div.
template <int N>
__device__ __forceinline__ void build_dtab(const StepDev& S, int in_pass, int* dtab, long long base_block,
                                           long long kbase, int div) {
  const int gm = S.gmin[gmin_slot(in_pass, S.ctl[5])];
  const int* sc = S.sc + (size_t)in_pass * S.scmax;
  for (int k = threadIdx.x; k < N; k += blockDim.x) dtab[k] = gm - sc[base_block + (kbase + k) / div];
  __syncthreads();
}

// Close: (fixed point, produced by the last strided-axis pass) inverse FFT . X half
// -> psi_n: norm / E_pot partials, flux snapshot, E_kin part of the last axis.  The
// inverse transform is the forward one on conjugated data.  psi_n is stored as double
// at the last sub-step of the call (or always when not fused); otherwise the pass goes
// on into the next sub-step: its opening X half and the forward transform of the last
// axis, leaving pass 0 of that sub-step in fixed point.
template <int N>
__global__ void __launch_bounds__(row_threads(N), row_min_blocks(N)) k_row_close(const GridDev* __restrict__ Gs,
                                                           const StepDev* __restrict__ Ss, int L) {
  const GridDev& g = Gs[blockIdx.y];
  const StepDev& S = Ss[blockIdx.y];
  if (!pass_active(S)) return;
  extern __shared__ __align__(128) longlong2 smx[];
  __shared__ int red[kRedInts];
  __shared__ double dred[32 * 3];
  const AxisDev& a = g.ax[g.dim - 1];
  const long long sub = S.ctl[5];
  if (blockIdx.x == 0 && threadIdx.x == 0) S.ctl[6] = sub + 1;  // the sub-step's last pass
  // the step ends here, psi_n stored as complex128: the call's last sub-step, and steps
  // whose E_kin needs psi_n in memory
  const bool ek = ekin_at(S, sub);
  const bool last = !S.fused || sub >= S.ctl[1] || sub + 1 >= S.nsteps || ek;
  const long long row0 = (long long)blockIdx.x * L;
  const int Lh = (int)min((long long)L, g.m / N - row0);
  const long long base = row0 * N;
  const int cnt = Lh * N;
  // 3D: the sweep after the inverse transform reads this block's slice of the X table
  // (16 B per point) and of the potential (8 B per point, E_pot): start moving it into
  // L2 now, one prefetch per 128-byte line, so that those loads do not wait on DRAM
  // (256^3 step 2.11 -> 2.08 ms; no gain for the 2D passes, so they skip it)
  if (g.dim == 3) {
    for (int e = threadIdx.x * 8; e < cnt; e += blockDim.x * 8) prefetch_l2(S.xs + base + e);
    if (S.obs & 2u)
      for (int e = threadIdx.x * 16; e < cnt; e += blockDim.x * 16) prefetch_l2(S.Vx + base + e);
  }
  int bits = 0;
  // producer of element (row, j): axis-0 tile j / C (2D) or axis-1 tile (i0, j / C) (3D,
  // when the block's rows share i0)
  __shared__ int dtab[N];
  const bool use_tab = g.dim == 2 || N % row_lines(N) == 0;
  if (use_tab) {
    constexpr int C = tile_cols(N) < N ? tile_cols(N) : N;
    const long long i0 = g.dim == 3 ? row0 / N : 0;
    build_dtab<N>(S, g.dim == 3 ? 3 : 2, dtab, g.dim == 3 ? i0 * ((N + C - 1) / C) : 0, 0, C);
  }
  // rows are contiguous: treat the block as one "column" of cnt elements
  int scale = load_aligned<N>(g, S, g.dim == 3 ? 3 : 2, smx, base, 1, cnt, 1, 1, red, bits, true,
                              use_tab ? dtab : nullptr, false);
  int sh = first_pass_shift<N>(bits);
  scale += sh;
  const LineSet ls{Lh, N, 1, false};
  fft_fx<N, row_ppt(N)>(smx, ls, a.twf, threadIdx.x, blockDim.x, scale, bits, red, sh);
  double dacc[5];
  const bool fuse_x = !last;
  if (fuse_x) {
    close_open_block<N>(g, S, smx, base, cnt, row0, Lh, red, scale, bits, dacc);
    dacc[2] = 0.0;
  } else {
    close_block<N>(g, S, smx, base, cnt, row0, red, scale, bits, dacc, true, last);
    if (S.row_ptr) {  // flux snapshot of psi_n (this thread's own elements of smx are not needed)
      const int e0 = S.row_ptr[row0], e1 = S.row_ptr[row0 + Lh];
      for (int e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
        const longlong2 x = smx[S.snap_idx[e] - base];
        S.snap[e] = make_double2(fx2d(x.x, scale), fx2d(x.y, scale));
      }
    }
    dacc[2] = ek ? ekin_rows<N, row_ppt(N)>(a, smx, ls, cnt, scale, bits, red) : 0.0;
  }
  const double e_n = dacc[3], e_v = dacc[4];
  block_sum<3>(dacc, dred);  // its barriers also end the snapshot reads of smx
  if (threadIdx.x == 0) {
    S.partials[0 * S.pmax + blockIdx.x] = ldexp(dacc[0], (int)e_n);
    S.partials[1 * S.pmax + blockIdx.x] = ldexp(dacc[1], (int)e_v);
    S.partials[(2 + g.dim - 1) * S.pmax + blockIdx.x] = dacc[2];
  }
  if (last) return;
  // next sub-step: opening X half (static factor and the length-gauge factors of the
  // next coupling row; already applied when fused) and the forward transform of the last axis
  if (!fuse_x) {
    const bool real_f = S.mode == 1 && g.gauge != 1;
    const int pre = product_headroom(bits);
    u64 mag = 0;
#pragma unroll 4
    for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
      const long long p = base + e;
      longlong2 x = smx[e];
      if (pre) x = make_longlong2(fshift(x.x, pre), fshift(x.y, pre));
      x = xhalf<N>(g, S, x, p, row0 + e / N, e % N, 2, real_f);
      smx[e] = x;
      mag |= fmag(x);
    }
    scale += pre - xhalf_exp(g, S, 2);
    bits = block_max_int(bitlen(mag), red);
  }
  sh = first_pass_shift<N>(bits);
  scale += sh;
  fft_fx<N, row_ppt(N)>(smx, ls, a.twf, threadIdx.x, blockDim.x, scale, bits, red, sh);
  longlong2* out = reinterpret_cast<longlong2*>(g.psi);
#pragma unroll 4
  for (int e = threadIdx.x; e < cnt; e += blockDim.x) out[base + e] = smx[e];
  if (threadIdx.x == 0) {
    S.sc[blockIdx.x] = scale;
    atomicMin(&S.gmin[gmin_slot(0, sub + 1)], scale);
  }
}

// P phase between the forward and the inverse transform of axis `ax` (element (i, c)
// of the tile at smx[i * ldc + c]), written conjugated so that the inverse transform
// runs as a forward one; returns the exponent change and the new bit length.
__device__ __forceinline__ int p_phase(const GridDev& g, const StepDev& S, longlong2* smx, int ax, int rows, int Ch,
                                       int ldc, const int4* pcol, int* red, int& bits) {
  const bool real_f = S.mode == 1;
  const int pre = product_headroom(bits);
  const int cnt = rows * Ch;
  u64 mag = 0;
  TileWalk w(threadIdx.x, blockDim.x, Ch);
#pragma unroll 1
  for (int e = threadIdx.x; e < cnt; e += blockDim.x, w.next()) {
    const int i = w.i, c = w.c;
    longlong2 x = smx[i * ldc + c];
    if (pre) x = make_longlong2(fshift(x.x, pre), fshift(x.y, pre));
    x = fapply(x, S.ptab[(size_t)ax * S.nmax + i], real_f);
    if (pcol) x = fapply(x, pcol[c], real_f);
    x = fconj(x);
    smx[i * ldc + c] = x;
    mag |= fmag(x);
  }
  int pe = xshift(pcol ? 2 : 1);
  for (int d = 0; d < g.dim; ++d) pe += S.texp[d];
  bits = block_max_int(bitlen(mag), red);
  return pre - pe;
}

// ------------------------------------------------------------ strided axes
// Axis `ax` (not the last): tiles of C adjacent columns; element (i, c) of tile
// (o, c0) is psi[o * N * stride + i * stride + c0 + c].  Modes:
//   0 forward (3D axis 1: pass 0 -> 1), 1 inverse (3D axis 1: pass 2 -> 3),
//   2 forward . P phase . inverse (axis 0: pass 0 (2D) or 1 (3D) -> 2),
//   3 forward of psi_n (double) + E_kin partial
// Inverse transforms run as forward ones on conjugated data.
template <int MODE, int N>
__global__ void __launch_bounds__(row_threads(N), row_min_blocks(N)) k_axis(const GridDev* __restrict__ Gs, const StepDev* __restrict__ Ss,
                                                      int ax, int C) {
  const GridDev& g = Gs[blockIdx.y];
  const StepDev& S = Ss[blockIdx.y];
  if (!pass_active(S)) return;
  if (MODE == 3 && !ekin_at(S, S.ctl[5])) return;
  extern __shared__ __align__(128) longlong2 smx[];
  __shared__ int red[kRedInts];
  __shared__ double dred[32];
  __shared__ int4 pcol[64];
  const AxisDev& a = g.ax[ax];
  const long long inner = a.stride;
  const long long tiles_per_outer = (inner + C - 1) / C;
  const long long o = blockIdx.x / tiles_per_outer;
  const long long c0 = (blockIdx.x % tiles_per_outer) * C;
  const int Ch = (int)min((long long)C, inner - c0);
  const long long obase = o * (long long)N * inner + c0;
  const int cnt = N * Ch;
  const LineSet ls{Ch, 1, C, true};
  int scale = 0, bits = 0;
  if (MODE == 3) {
    double2* sd = reinterpret_cast<double2*>(smx);
    int em = 0;
    for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
      const int i = e / Ch, c = e % Ch;
      const double2 v = g.psi[obase + (long long)i * inner + c];
      sd[i * C + c] = v;
      em = max(em, max(dexp(v.x), dexp(v.y)));
    }
    em = block_max_int(em, red);
    scale = (62 - fguard(radix_at(N, 0))) - (em - 1022);
    for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
      const int i = e / Ch, c = e % Ch;
      const double2 v = sd[i * C + c];
      smx[i * C + c] = make_longlong2(d2fx(v.x, scale), d2fx(v.y, scale));
    }
    __syncthreads();
    fft_fx<N, row_ppt(N)>(smx, ls, a.twf, threadIdx.x, blockDim.x, scale, bits, red);
    double acc = 0.0;
    for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
      const int i = e / Ch, c = e % Ch;
      const double k = kpos(a, i);
      const longlong2 x = smx[i * C + c];
      const double xr = fx2d(x.x, scale), xi = fx2d(x.y, scale);
      acc = fma(k * k, fma(xr, xr, xi * xi), acc);
    }
    block_sum<1>(&acc, dred);
    if (threadIdx.x == 0) S.partials[(2 + ax) * S.pmax + blockIdx.x] = acc;
    return;
  }
  const int in_pass = MODE == 0 ? 0 : MODE == 1 ? 2 : (g.dim == 3 ? 1 : 0);
  const int out_pass = MODE == 0 ? 1 : MODE == 1 ? 3 : 2;
  // producer row block of element (i, c) when the input is the row pass: (o N + i) / L
  __shared__ int dtab[N];
  const bool by_row = in_pass == 0;
  if (by_row) build_dtab<N>(S, 0, dtab, 0, o * N, row_lines(N));
  scale = load_aligned<N>(g, S, in_pass, smx, obase, inner, N, Ch, C, red, bits, MODE == 1, by_row ? dtab : nullptr,
                          true, g.tmap[ax], (int)(2 * c0), (int)o);
  const bool multi_col = MODE == 2 && ax + 1 < g.dim;
  if (multi_col && threadIdx.x < Ch) {
    // per-column factor: product of the P tables of the axes after `ax`
    long long cc = c0 + threadIdx.x;
    longlong2 f = make_longlong2(4611686018427387904LL, 0LL);  // 1.0
    for (int d2 = g.dim - 1; d2 > ax; --d2) {
      const int i = (int)(cc % g.ax[d2].n);
      cc /= g.ax[d2].n;
      f = fmul62(f, tw_join(S.ptab[(size_t)d2 * S.nmax + i]));
    }
    pcol[threadIdx.x] = split_fx(f);
  }
  int sh = first_pass_shift<N>(bits);
  scale += sh;
  fft_fx<N, row_ppt(N)>(smx, ls, a.twf, threadIdx.x, blockDim.x, scale, bits, red, sh);
  if (MODE == 2) {
    scale += p_phase(g, S, smx, ax, N, Ch, C, multi_col ? pcol : nullptr, red, bits);
    sh = first_pass_shift<N>(bits);
    scale += sh;
    fft_fx<N, row_ppt(N)>(smx, ls, a.twf, threadIdx.x, blockDim.x, scale, bits, red, sh);
  }
  longlong2* out = reinterpret_cast<longlong2*>(g.psi);
  const bool conj_out = MODE != 0;
  TileWalk w(threadIdx.x, blockDim.x, Ch);
#pragma unroll 4
  for (int e = threadIdx.x; e < cnt; e += blockDim.x, w.next()) {
    const int i = w.i, c = w.c;
    const longlong2 x = smx[i * C + c];
    out[obase + (long long)i * inner + c] = conj_out ? fconj(x) : x;
  }
  if (threadIdx.x == 0) {
    S.sc[(size_t)out_pass * S.scmax + blockIdx.x] = scale;
    atomicMin(&S.gmin[out_pass], scale);
  }
}

// ------------------------------------------------------------ 1D whole step
// One block per line: X open . FFT . P . IFFT . X close . observables, line in smem.
template <int N, bool FULL>
__global__ void __launch_bounds__(kLineThreads, (QSF_FFT_MIN_BLOCKS + 1) / 2) k_line_step(const GridDev* __restrict__ Gs,
                                                            const StepDev* __restrict__ Ss) {
  const GridDev& g = Gs[blockIdx.y];
  const StepDev& S = Ss[blockIdx.y];
  if (!pass_active(S)) return;
  if (threadIdx.x == 0) S.ctl[6] = S.ctl[5] + 1;  // the sub-step's only pass
  extern __shared__ __align__(128) longlong2 smx[];
  __shared__ int red[kRedInts];
  __shared__ double dred[32 * kMaxFluxBorders];
  const AxisDev& a = g.ax[0];
  int bits = 0;
  int scale = open_block<N>(g, S, smx, 0, N, 0, red, bits);
  int sh = first_pass_shift<N>(bits);
  scale += sh;
  const LineSet ls{1, N, 1, false};
  fft_fx<N, line_ppt(N)>(smx, ls, a.twf, threadIdx.x, blockDim.x, scale, bits, red, sh);
  scale += p_phase(g, S, smx, 0, N, 1, 1, nullptr, red, bits);
  sh = first_pass_shift<N>(bits);
  scale += sh;
  fft_fx<N, line_ppt(N)>(smx, ls, a.twf, threadIdx.x, blockDim.x, scale, bits, red, sh);
  double dacc[5];
  close_block<N>(g, S, smx, 0, N, 0, red, scale, bits, dacc, true, true);
  __syncthreads();
  if (S.row_ptr) {
    const int e1 = S.row_ptr[1];
    for (int e = threadIdx.x; e < e1; e += blockDim.x) S.snap[e] = g.psi[S.snap_idx[e]];
  }
  dacc[2] = ekin_at(S, S.ctl[5]) ? ekin_rows<N, line_ppt(N)>(a, smx, ls, N, scale, bits, red) : 0.0;
  const double e_n = dacc[3], e_v = dacc[4];
  block_sum<3>(dacc, dred);
  if (threadIdx.x == 0) {
    S.partials[0 * S.pmax] = ldexp(dacc[0], (int)e_n);
    S.partials[1 * S.pmax] = ldexp(dacc[1], (int)e_v);
    S.partials[2 * S.pmax] = dacc[2];
  }
  if constexpr (FULL) {  // the end of the step in this block: fluxes, row, counters
    __syncthreads();
    const long long sub = S.ctl[5];
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

// ------------------------------------------------------------ plain FFT passes
// fourier<R>() without phases (qsf_fourier), in block fixed point: each block takes
// its exponent from the largest double it loads (one global read, staged in smem),
// converts with integer operations, runs the fixed-point passes (an inverse is the
// forward transform between two conjugations) and converts back (times post_scale).
template <int N, bool FWD>
__global__ void __launch_bounds__(kLineThreads, (QSF_FFT_MIN_BLOCKS + 1) / 2) k_row_fft(GridDev g, int L, double post_scale) {
  extern __shared__ __align__(128) longlong2 smx[];
  __shared__ int red[kRedInts];
  const AxisDev& a = g.ax[g.dim - 1];
  const long long row0 = (long long)blockIdx.x * L;
  const long long nrows = g.m / N;
  const int Lh = (int)min((long long)L, nrows - row0);
  const long long base = row0 * N;
  const int cnt = Lh * N;
  double2* sd = reinterpret_cast<double2*>(smx);
  int em = 0;
  for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
    const double2 v = g.psi[base + e];
    sd[e] = v;
    em = max(em, max(dexp(v.x), dexp(v.y)));
  }
  em = block_max_int(em, red);
  int scale = (62 - fguard(radix_at(N, 0))) - (em - 1022);
  for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
    const double2 v = sd[e];
    const longlong2 x = make_longlong2(d2fx(v.x, scale), d2fx(v.y, scale));
    smx[e] = FWD ? x : fconj(x);
  }
  __syncthreads();
  const LineSet ls{Lh, N, 1, false};
  int bits = 0;
  fft_fx<N>(smx, ls, a.twf, threadIdx.x, blockDim.x, scale, bits, red);
  for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
    const longlong2 x = FWD ? smx[e] : fconj(smx[e]);
    double2 v = make_double2(fx2d(x.x, scale), fx2d(x.y, scale));
    if (post_scale != 1.0) v = cscale(v, post_scale);
    g.psi[base + e] = v;
  }
}

template <int N, bool FWD>
__global__ void __launch_bounds__(row_threads(N), row_min_blocks(N)) k_axis_fft(GridDev g, int ax, int C, double post_scale) {
  extern __shared__ __align__(128) longlong2 smx[];
  __shared__ int red[kRedInts];
  const AxisDev& a = g.ax[ax];
  const long long inner = a.stride;
  const long long tiles_per_outer = (inner + C - 1) / C;
  const long long o = blockIdx.x / tiles_per_outer;
  const long long c0 = (blockIdx.x % tiles_per_outer) * C;
  const int Ch = (int)min((long long)C, inner - c0);
  const long long obase = o * (long long)N * inner + c0;
  const int cnt = N * Ch;
  double2* sd = reinterpret_cast<double2*>(smx);
  int em = 0;
  for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
    const int i = e / Ch, c = e % Ch;
    const double2 v = g.psi[obase + (long long)i * inner + c];
    sd[i * C + c] = v;
    em = max(em, max(dexp(v.x), dexp(v.y)));
  }
  em = block_max_int(em, red);
  int scale = (62 - fguard(radix_at(N, 0))) - (em - 1022);
  for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
    const int i = e / Ch, c = e % Ch;
    const double2 v = sd[i * C + c];
    const longlong2 x = make_longlong2(d2fx(v.x, scale), d2fx(v.y, scale));
    smx[i * C + c] = FWD ? x : fconj(x);
  }
  __syncthreads();
  const LineSet ls{Ch, 1, C, true};
  int bits = 0;
  fft_fx<N, row_ppt(N)>(smx, ls, a.twf, threadIdx.x, blockDim.x, scale, bits, red);
  for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
    const int i = e / Ch, c = e % Ch;
    const longlong2 x = FWD ? smx[i * C + c] : fconj(smx[i * C + c]);
    double2 v = make_double2(fx2d(x.x, scale), fx2d(x.y, scale));
    if (post_scale != 1.0) v = cscale(v, post_scale);
    g.psi[obase + (long long)i * inner + c] = v;
  }
}

#ifdef QSF_DEFINE_KERNELS
// ------------------------------------------------------------ flux + finalize
// Block-partial border fluxes over flux terms [t0, t1): each term is one grid point
// and one border type; j_d = inv_2dx Im(conj(psi) (psi_+ - psi_-)) (0 where the
// reference's flat-index bounds test fails, grid.h:470-472) + A_d |psi|^2 (velocity
// gauge), dotted with the normalised border vector.  out[b] written by thread b.
__global__ void __launch_bounds__(256) k_flux(GridDev g, const FluxPoint* fpts, const FluxTerm* fterms, int nfterms,
                                              const double2* snap, double A0, double A1, double A2, int useA, int nb,
                                              double* out_partials, CoupDev cd) {
  __shared__ double red[32 * kMaxFluxBorders];
  double Av[3] = {A0, A1, A2};
  coup_load(cd, Av);
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
  const long long sub = S.ctl[0];
  // observables, Normalize and the convergence test once per step (its last sub-step)
  const bool step_end = (sub + 1) % S.substeps == 0;
  const long long step = sub / S.substeps;
  const int nb = S.nborders;
  if (S.nfterms > 0 && step_end) {
    const double* A = (g.gauge == 0 && S.coupling && g.n_fields) ? S.coupling + sub * S.coup_stride : nullptr;
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
  finalize_tail(g, S, sub, step_end, step, nb, (int)gridDim.x, red);
}

// apply a pending Normalize factor (end of a qsf_step call / qsf_normalize)
__global__ void k_scale(double2* psi, long long m, const double* scale) {
  const double s = *scale;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < m; p += stride) psi[p] = cscale(psi[p], s);
}

// ------------------------------------------------------------ granular members
// evolve<M,R>(delta) with the reference's per-point formula (grid.h:394-418)
// X-phase factor per point of evolve<M, X>(delta) without an X-space coupling term:
// expOp(delta V) times the absorber (grid.h:394-418), as one complex factor
__global__ void k_evolve_xtab(GridDev g, int mode, double delta, double2* __restrict__ tab) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < g.m; p += stride) {
    int idx[kMaxDim];
    double c[kMaxDim];
    unflatten(g, p, idx);
    for (int d = 0; d < g.dim; ++d) c[d] = xpos(g.ax[d], idx[d]);
    double2 f = expop(mode, delta * potential_at(g, c));
    if (g.nCAP > 0 && !g.multi) f = cscale(f, absorb_at(g, delta, idx));
    tab[p] = f;
  }
}
// per-axis factors of evolve<M, P>(delta): expOp(delta (k^2 / 2 + A_d k)) for axis d
// (the P Hamiltonian is a sum over axes, so its exponential is their product)
__global__ void k_evolve_ptab(GridDev g, int mode, double delta, double c0, double c1, double c2, int nmax,
                              double2* __restrict__ tab, CoupDev cd) {
  double cv[3] = {c0, c1, c2};
  coup_load(cd, cv);
  if (g.p_swap && g.dim >= 2) {
    const double t = cv[0];
    cv[0] = cv[1];
    cv[1] = t;
  }
  const bool coupled = g.gauge == 0 && g.n_fields;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < g.dim * nmax; e += gridDim.x * blockDim.x) {
    const int d = e / nmax, i = e % nmax;
    if (i >= g.ax[d].n) continue;
    const double k = kpos(g.ax[d], i);
    tab[e] = expop(mode, delta * (0.5 * k * k + (coupled ? k * cv[d] : 0.0)));
  }
}
// psi *= tab[p] (X) or psi *= prod_d tab[d][idx_d] (P)
__global__ void k_apply_xtab(double2* __restrict__ psi, const double2* __restrict__ tab, long long m) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < m; p += stride) {
    const double2 a = psi[p], f = tab[p];
    psi[p] = make_double2(a.x * f.x - a.y * f.y, a.x * f.y + a.y * f.x);
  }
}
__global__ void k_apply_ptab(GridDev g, const double2* __restrict__ tab, int nmax) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < g.m; p += stride) {
    int idx[kMaxDim];
    unflatten(g, p, idx);
    double2 f = tab[idx[0]];
    for (int d = 1; d < g.dim; ++d) {
      const double2 t = tab[d * nmax + idx[d]];
      f = make_double2(f.x * t.x - f.y * t.y, f.x * t.y + f.y * t.x);
    }
    const double2 a = g.psi[p];
    g.psi[p] = make_double2(a.x * f.x - a.y * f.y, a.x * f.y + a.y * f.x);
  }
}

__global__ void k_evolve(GridDev g, int mode, int rep, double delta, double c0, double c1, double c2, CoupDev cd) {
  double cv[3] = {c0, c1, c2};
  coup_load(cd, cv);
  if (rep == 2 && g.p_swap && g.dim >= 2) {
    const double t = cv[0];
    cv[0] = cv[1];
    cv[1] = t;
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
    if (rep == 1 && g.nCAP > 0 && !g.multi) v = cscale(v, absorb_at(g, delta, idx));
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

// potential per point (X representation), for the member averages of E_pot
__global__ void k_build_vtab(GridDev g, double* __restrict__ vtab) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < g.m; p += stride) {
    int idx[kMaxDim];
    double c[kMaxDim];
    unflatten(g, p, idx);
    for (int d = 0; d < g.dim; ++d) c[d] = xpos(g.ax[d], idx[d]);
    vtab[p] = potential_at(g, c);
  }
}
// sum |psi|^2 w(p) per block with the weights from a table (E_pot from the potential table)
__global__ void __launch_bounds__(256) k_average_tab(GridDev g, const double* __restrict__ w, double* out_partials) {
  __shared__ double red[32];
  double acc = 0.0;
  const long long stride = (long long)gridDim.x * blockDim.x;
#pragma unroll 4
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < g.m; p += stride) {
    const double2 v = g.psi[p];
    acc = fma(fma(v.x, v.x, v.y * v.y), w[p], acc);
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

// the same into column col of row *step of rows (ncol columns): a step program's row
__global__ void k_reduce_row(const double* part, int n, double scale, double* rows, const long long* step, int ncol,
                             int col) {
  __shared__ double red[32];
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) acc += part[i];
  block_sum<1>(&acc, red);
  if (threadIdx.x == 0) rows[(*step) * ncol + col] = acc * scale;
}

// gather psi at the snapshot indices (granular flux)
__global__ void k_gather(const double2* psi, const long long* idx, int n, double2* out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) out[i] = psi[idx[i]];
}

// maskRegion (grid.h:582-597) with CAP::mask (absorbers.h:48-54)
// CAP::mask of one node (absorbers.h:48-54): 1 outside the margin
__device__ __forceinline__ double mask1(const GridDev& g, long long nd) {
  const long long nodes = g.nCAP + nd;
  if (nodes < 0) return 1.0;
  const double v = nodes > 0 ? (double)(nodes * (nodes * (nodes * nodes))) : 0.0;
  return exp(-(v + 0) * g.eta);
}
__device__ __forceinline__ long long neg_dist(const GridDev& g, int d, int i) {
  return i < g.ax[d].n2 ? -(long long)i : (long long)i - g.ax[d].n + 1;
}

// Per-axis values of the one-node absorber mask, mtab[d * nmax + i] = CAP::mask of axis
// d's node i (absorbers.h:48-54).  The mask of several nodes, exp(-eta sum_d n_d^4), is
// the product of these (to rounding), so the region masks and transfers below need no exp.
__global__ void k_mask_tab(GridDev g, int nmax, double* __restrict__ mtab) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < g.dim * nmax; e += gridDim.x * blockDim.x) {
    const int d = e / nmax, i = e % nmax;
    mtab[e] = i < g.ax[d].n ? mask1(g, neg_dist(g, d, i)) : 1.0;
  }
}

// Slice of a region transfer (getBox + maskSlice, multigrid.h:454-569): src in the
// margins along fc times 1 - mask(fc) and, for a destination in group 1, the corner
// correction (mask_correction, multigrid.h:519-530); zero elsewhere, except in 1D,
// where the whole line is copied and only its margins are masked.  In 3D the sliding
// axis is limited to the n / nCAP boxes (slide_lim planes).
__global__ void k_mg_slice(GridDev g, const double2* __restrict__ src, double2* __restrict__ slice, int fc, int group,
                           long long slide_lim, const double* __restrict__ mtab, int nmax) {
  const int D = g.dim;
  const int slide = D == 3 ? (fc == 1 ? 2 : 1) : -1;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < g.m; p += stride) {
    int idx[kMaxDim];
    unflatten(g, p, idx);
    const int i = idx[fc];
    const bool band = i < g.nCAP || i >= g.ax[fc].n - g.nCAP;
    if (!band || (slide >= 0 && idx[slide] >= slide_lim)) {
      slice[p] = (D == 1 && !band) ? src[p] : make_double2(0.0, 0.0);
      continue;
    }
    const double mv = 1.0 - mtab[fc * nmax + i];
    double f = mv;
    if (group == 1) {
      double corr = 1.0;
      if (D == 2) {
        const int o = 1 - fc;
        const double b0 = fc == 0 ? 1.0 : 1.0 - mtab[o * nmax + idx[o]];
        const double b1 = fc == 1 ? 1.0 : 1.0 - mtab[o * nmax + idx[o]];
        corr = 1 - 0.5 * (b0 * b1);
      } else if (D == 3) {
        double a[3], b[3];
        for (int d = 0; d < 3; ++d) {
          const double mk = mtab[d * nmax + idx[d]];
          a[d] = d == fc ? 0 : mk;
          b[d] = d == fc ? 1.0 : mk;
        }
        corr = 0.5 * (a[0] + (a[1] + (a[2] + 0))) + (1.0 / 6.0) * (1 - (b[0] * (b[1] * b[2])));
      }
      f = mv * corr;
    }
    const double2 v = src[p];
    slice[p] = make_double2(v.x * f, v.y * f);
  }
}

// coherent addition (add, multigrid.h:571-586): dst += slice
__global__ void k_add_slice(double2* __restrict__ dst, const double2* __restrict__ slice, long long m) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < m; p += stride) {
    const double2 a = dst[p], b = slice[p];
    dst[p] = make_double2(a.x + b.x, a.y + b.y);
  }
}

// maskRegion_ (grid.h:582-597): psi *= the mask of the bounded axes' nodes, as the
// product of the per-axis one-node masks (a free axis contributes 1)
__global__ void k_mask(GridDev g, int b0, int b1, int b2, const double* __restrict__ mtab, int nmax) {
  const int bounded[3] = {b0, b1, b2};
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < g.m; p += stride) {
    int idx[kMaxDim];
    unflatten(g, p, idx);
    double mk = 1.0;
    for (int d = 0; d < g.dim; ++d)
      if (bounded[d]) mk *= mtab[d * nmax + idx[d]];
    if (mk != 1.0) g.psi[p] = cscale(g.psi[p], mk);
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
  int line_ctas;     // CTAs holding one 1D line in the step kernel (a cluster of 2 .. 8 CTAs for
                     // power-of-two lines of 1024 or more points)
  int line_threads;  // threads per CTA of the 1D line step kernel
  int fft_ctas;      // CTAs of the plain row transform of one line (2: a cluster pair above 8192 points)
  int row_threads;  // threads per block of the row / axis passes
  bool line_full;   // line_step also ends the step (fluxes, row, counters: no k_finalize)
};

// kernel table of the supported sizes (qsf_sizes_*.cu); nullptr when n is not built
const KernelSet* kernels_for(int n);

}  // namespace qsf
#include "qsf_cluster.cuh"
namespace qsf {

// sizes up to 4096 get the multi-dimensional passes; up to 8192 the 1D line kernel of
// one CTA, up to 16384 the one of a cluster pair
template <int N>
KernelSet make_kernel_set() {
  static_assert(is_smooth(N), "grid sizes must be 2^a 3^b 5^c");
  static_assert(N <= 16384, "1D lines longer than 16384 points are not built");
  KernelSet k{};
  k.n = N;
  k.line_ctas = 1;
  k.line_threads = kLineThreads;
  k.fft_ctas = 1;
  k.row_threads = row_threads(N);
  k.line_full = false;
  if constexpr (N > 8192) {
    k.line_ctas = 2;
    k.fft_ctas = 2;
    k.line_step = k_line_step_cl<N>;
    k.row_fft_f = k_row_fft_cl<N, true>;
    k.row_fft_b = k_row_fft_cl<N, false>;
    return k;
  } else {
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
  k.line_step = k_line_step<N, true>;
  k.line_full = true;
#if QSF_LINE_CLUSTER
  if constexpr (N >= 1024 && (N & (N - 1)) == 0) {  // the line spread over a cluster
    constexpr int C = N / 512 < 8 ? N / 512 : 8;
    k.line_ctas = C;
    k.line_threads = mc_threads<N, C>();
    k.line_step = k_line_step_mc<N, C>;
  }
#endif
  k.row_fft_f = k_row_fft<N, true>;
  k.row_fft_b = k_row_fft<N, false>;
  return k;
  }
}

}  // namespace qsf
