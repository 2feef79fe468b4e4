// qsf_bluestein.cu -- fourier<R>() for axis lengths outside the built kernel list.
//
// The reference's FFTW plans take any n (wf/grid.h:251-274); the fused step kernels of
// this library are compiled for a list of lengths 2^a, 3*2^a and 5*2^a (8 ... 16384,
// the add_sizes_* tables).  For any other n one axis of the transform runs as Bluestein's
// chirp-z convolution: with c[j] = exp(-i pi j^2 / n),
//     X[k] = c[k] * sum_j (x[j] c[j]) conj(c[k - j]),
// a linear convolution evaluated as a cyclic one of length M >= 2n - 1 (a length with
// built kernels) through the library's own M-point transforms:
//     a = pad_M(x * c);  A = FFT_M(a);  A *= B = FFT_M(conj(c), wrapped);  a = IFFT_M(A) / M;
//     X[k] = c[k] a[k], k < n.
// A 1D line of more than 8192 points needs M > 16384, beyond the one-CTA-pair line
// transforms: M = M1 * M2 then runs as a four-step transform (columns, twiddles, rows)
// whose output order is transposed, the same for the kernel B and the data, so the
// pointwise product and the inverse four-step give the cyclic convolution unchanged.
// The inverse transform is the forward one between two conjugations.  The chirp comes
// from exact integer angle reduction (j^2 mod 2n) and sincospi on the device; B is
// transformed once per grid.  Grids of such lengths step through the member operations
// (qsf_step's step programs, replayed from graphs); batches take built lengths only,
// the server runs such solves beside its batch.
#include <array>
#include <cmath>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "qsf_internal.h"

namespace qsf {
namespace {

// psi index (o, j, c) of axis ax with length nj: o * nj * inner + j * inner + c
__global__ void k_bs_pre(const double2* __restrict__ psi, double2* __restrict__ scr, const double2* __restrict__ chirp,
                         long long outer, int n, int M, long long inner, int conj_in) {
  const long long total = outer * M * inner;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < total; p += stride) {
    const long long c = p % inner, t = p / inner;
    const int j = (int)(t % M);
    const long long o = t / M;
    double2 v = make_double2(0.0, 0.0);
    if (j < n) {
      double2 x = psi[(o * n + j) * inner + c];
      if (conj_in) x.y = -x.y;
      v = cmul(x, chirp[j]);
    }
    scr[p] = v;
  }
}

__global__ void k_bs_mul(double2* __restrict__ scr, const double2* __restrict__ bhat, long long outer, int M,
                         long long inner) {
  const long long total = outer * M * inner;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < total; p += stride) {
    const int j = (int)((p / inner) % M);
    scr[p] = cmul(scr[p], bhat[j]);
  }
}

__global__ void k_bs_post(double2* __restrict__ psi, const double2* __restrict__ scr, const double2* __restrict__ chirp,
                          long long outer, int n, int M, long long inner, int conj_out, double post) {
  const long long total = outer * n * inner;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < total; p += stride) {
    const long long c = p % inner, t = p / inner;
    const int k = (int)(t % n);
    const long long o = t / n;
    double2 y = cmul(scr[(o * M + k) * inner + c], chirp[k]);
    if (conj_out) y.y = -y.y;
    psi[p] = make_double2(y.x * post, y.y * post);
  }
}

// four-step twiddles: scr[(o * M1 + k1) * M2 + n2] *= w[k1 * M2 + n2] (conjugated: inverse)
__global__ void k_bs_twiddle(double2* __restrict__ scr, const double2* __restrict__ w, long long total, int M,
                             int conj_w) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < total; p += stride) {
    double2 t = w[p % M];
    if (conj_w) t.y = -t.y;
    scr[p] = cmul(scr[p], t);
  }
}

// chirp[j] = exp(-i pi (j^2 mod 2n) / n) (exact integer angle reduction) and the
// convolution kernel w = conj(chirp) wrapped onto M points (w[j] = w[M - j]), zero
// between
__global__ void k_bs_chirp(double2* __restrict__ chirp, double2* __restrict__ w, int n, int M) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < M; j += gridDim.x * blockDim.x) {
    const int k = j < n ? j : M - j;  // the chirp index w[j] holds, or >= n (zero)
    double2 v = make_double2(0.0, 0.0);
    if (k < n) {
      const long long r = ((long long)k * k) % (2LL * n);
      double sn, cs;
      sincospi((double)r / (double)n, &sn, &cs);
      v = make_double2(cs, sn);  // conj(chirp[k])
      if (j < n) chirp[j] = make_double2(cs, -sn);
    }
    w[j] = v;
  }
}

// four-step twiddles w4[k1 * M2 + n2] = exp(-2 pi i (k1 n2 mod M) / M)
__global__ void k_bs_w4(double2* __restrict__ w4, int M1, int M2) {
  const int M = M1 * M2;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < M; p += gridDim.x * blockDim.x) {
    const long long r = ((long long)(p / M2) * (p % M2)) % M;
    double sn, cs;
    sincospi(2.0 * (double)r / (double)M, &sn, &cs);
    w4[p] = make_double2(cs, -sn);
  }
}

int blocks_for(long long count) {
  const long long b = (count + 255) / 256;
  return (int)std::min<long long>(std::max<long long>(b, 1), (long long)device_sm_count() * 16);
}

// one row transform (length n = S.ax[last].n, kernels K) over all rows of S
void row_pass(const KernelSet& K, const GridDev& S, bool fwd, double post, cudaStream_t st) {
  const int n = S.ax[S.dim - 1].n;
  const long long nrows = S.m / n;
  const int L = (int)std::max<long long>(1, std::min<long long>(nrows, (16LL * kLineThreads) / n));
  int blocks = (int)((nrows + L - 1) / L);
  size_t smem = (size_t)L * n * sizeof(double2);
  if (K.fft_ctas > 1) {
    blocks = K.fft_ctas;
    smem = (size_t)(n / K.fft_ctas) * sizeof(double2);
  }
  if (fwd) K.row_fft_f<<<blocks, kLineThreads, smem, st>>>(S, L, post);
  else K.row_fft_b<<<blocks, kLineThreads, smem, st>>>(S, L, post);
}

// one strided-axis transform (length S.ax[ax].n, kernels K) over all columns of S
void axis_pass(const KernelSet& K, const GridDev& S, int ax, bool fwd, double post, cudaStream_t st) {
  const int n = S.ax[ax].n;
  const long long inner = S.ax[ax].stride;
  // the tile the kernels are compiled for (tile_pts(n) points: C columns of n)
  const int C = (int)std::max<long long>(1, std::min<long long>({64, (long long)tile_pts(n) / n, inner}));
  const long long outer = S.m / ((long long)n * inner);
  const int blocks = (int)(outer * ((inner + C - 1) / C));
  const size_t smem = (size_t)n * C * sizeof(double2);
  if (fwd) K.axis_fft_f<<<blocks, K.row_threads, smem, st>>>(S, ax, C, post);
  else K.axis_fft_b<<<blocks, K.row_threads, smem, st>>>(S, ax, C, post);
}

// the M-point transform along axis ax of the array S.psi (geometry of S), on stream st
int fft_M(const qsf_grid* g, const GridDev& S, int ax, bool fwd, double post, cudaStream_t st) {
  const qsf_grid::Bluestein& b = g->bs;
  const KernelSet& K = *b.ks;
  const int M = b.M;
  if (b.M1) {
    // four-step on the 1D line(s) of S seen as [lines * M1][M2]: columns (M1), twiddles,
    // rows (M2); the inverse undoes them in the opposite order
    GridDev V = S;
    V.dim = 2;
    V.ax[0] = S.ax[0];
    V.ax[0].n = b.M1;
    V.ax[0].n2 = b.M1 / 2;
    V.ax[0].shift = (b.M1 & (b.M1 - 1)) == 0 ? __builtin_ctz((unsigned)b.M1) : -1;
    V.ax[0].stride = b.M2;
    V.ax[0].tw = b.tw1;
    V.ax[0].twx = b.twx1;
    V.ax[0].twf = reinterpret_cast<decltype(V.ax[0].twf)>(b.twf1);
    V.ax[1] = S.ax[0];
    V.ax[1].n = b.M2;
    V.ax[1].n2 = b.M2 / 2;
    V.ax[1].shift = (b.M2 & (b.M2 - 1)) == 0 ? __builtin_ctz((unsigned)b.M2) : -1;
    V.ax[1].stride = 1;
    V.ax[1].tw = b.tw;
    V.ax[1].twx = b.twx;
    V.ax[1].twf = reinterpret_cast<decltype(V.ax[1].twf)>(b.twf);
    for (int k = 0; k < kMaxDim; ++k) V.tmap[k] = nullptr;
    if (fwd) {
      axis_pass(*b.ks1, V, 0, true, 1.0, st);
      k_bs_twiddle<<<blocks_for(V.m), 256, 0, st>>>(V.psi, b.tw4, V.m, M, 0);
      row_pass(K, V, true, post, st);
    } else {
      row_pass(K, V, false, 1.0, st);
      k_bs_twiddle<<<blocks_for(V.m), 256, 0, st>>>(V.psi, b.tw4, V.m, M, 1);
      axis_pass(*b.ks1, V, 0, false, post, st);
    }
    QSF_CU(cudaGetLastError());
    return QSF_OK;
  }
  if (ax == S.dim - 1) row_pass(K, S, fwd, post, st);
  else axis_pass(K, S, ax, fwd, post, st);
  QSF_CU(cudaGetLastError());
  return QSF_OK;
}

// geometry of the scratch: psi's with axis ax of length M
GridDev scratch_view(const qsf_grid* g, int ax) {
  GridDev S = g->G;
  S.psi = g->bs.scratch;
  S.ax[ax].n = g->bs.M;
  S.ax[ax].n2 = g->bs.M / 2;
  S.ax[ax].shift = (g->bs.M & (g->bs.M - 1)) == 0 ? __builtin_ctz((unsigned)g->bs.M) : -1;
  S.ax[ax].tw = g->bs.tw;
  S.ax[ax].twx = g->bs.twx;
  S.ax[ax].twf = reinterpret_cast<decltype(S.ax[ax].twf)>(g->bs.twf);
  long long st = 1;
  for (int k = S.dim - 1; k >= 0; --k) {
    S.ax[k].stride = st;
    st *= S.ax[k].n;
  }
  S.m = st;
  for (int k = 0; k < kMaxDim; ++k) S.tmap[k] = nullptr;
  return S;
}

// The convolution length of an n-point axis: the smallest built length M >= 2n - 1
// (up to 16384 on a 1D line, 4096 on the axes of a 2D / 3D grid), else on a 1D line the
// smallest M1 * M2 >= 2n - 1 with M1-point column kernels (M1 <= 4096) and M2-point
// one-CTA row kernels (M2 <= 8192), the larger M2 first at equal M.
bool bs_plan(int n, int dim, int* M, int* M1, int* M2) {
  *M = *M1 = *M2 = 0;
  const int lim = dim == 1 ? 16384 : 4096;
  for (int c = 2 * n - 1; c <= lim; ++c)
    if (kernels_for(c)) {
      *M = c;
      return true;
    }
  if (dim != 1) return false;
  std::vector<int> cols, rows;
  for (int a = 8; a <= 8192; ++a) {
    const KernelSet* k = kernels_for(a);
    if (k && a <= 4096 && k->axis_fft_f) cols.push_back(a);
    if (k && k->row_fft_f && k->fft_ctas == 1) rows.push_back(a);
  }
  long long best = 0;
  for (int a : cols) {
    for (int r : rows) {
      const long long c = (long long)a * r;
      if (c < 2LL * n - 1) continue;
      if (!best || c < best || (c == best && r > *M2)) {
        best = c;
        *M1 = a;
        *M2 = r;
      }
    }
  }
  if (!best || best > (1LL << 24)) return false;
  *M = (int)best;
  return true;
}

}  // namespace

int bs_size(int n, int dim) {
  int M, M1, M2;
  return bs_plan(n, dim, &M, &M1, &M2) ? M : 0;
}

// four-step twiddles of (M1, M2), made once per process and device and shared
int shared_w4(int M1, int M2, double2** w4) {
  static std::mutex mu;
  static std::map<std::array<int, 3>, double2*> cache;
  int dev = 0;
  QSF_CU(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(mu);
  auto it = cache.find({dev, M1, M2});
  if (it == cache.end()) {
    double2* p = nullptr;
    if (int rc = dev_alloc(p, (size_t)M1 * M2)) return rc;
    k_bs_w4<<<blocks_for((long long)M1 * M2), 256>>>(p, M1, M2);
    QSF_CU(cudaGetLastError());
    QSF_CU(cudaDeviceSynchronize());
    it = cache.emplace(std::array<int, 3>{dev, M1, M2}, p).first;
  }
  *w4 = it->second;
  return QSF_OK;
}

int bs_setup(qsf_grid* g) {
  const GridDev& G = g->G;
  const int n = G.ax[0].n;
  int M = 0, M1 = 0, M2 = 0;
  if (!bs_plan(n, G.dim, &M, &M1, &M2))
    return fail(QSF_EINVAL, "grid size " + std::to_string(n) + " has no kernels and no Bluestein length in this build " +
                                "(1D lines up to 16384 points, other grids up to 2048 points per axis)");
  qsf_grid::Bluestein& b = g->bs;
  b.n = n;
  b.M = M;
  b.M1 = M1;
  b.M2 = M2;
  b.ks = kernels_for(M1 ? M2 : M);
  b.ks1 = M1 ? kernels_for(M1) : nullptr;
  int rc;
  if ((rc = shared_twiddles(M1 ? M2 : M, &b.tw, &b.twx, &b.twf))) return rc;
  if (M1 && ((rc = shared_twiddles(M1, &b.tw1, &b.twx1, &b.twf1)) || (rc = shared_w4(M1, M2, &b.tw4)))) return rc;
  const size_t scr = (size_t)(G.m / n) * (size_t)M;
  if ((rc = dev_alloc(b.chirp, (size_t)n)) || (rc = dev_alloc(b.bhat, (size_t)M)) ||
      (rc = dev_alloc(b.scratch, std::max(scr, (size_t)M))))
    return rc;
  k_bs_chirp<<<blocks_for(M), 256, 0, g->stream>>>(b.chirp, b.bhat, n, M);
  QSF_CU(cudaGetLastError());
  // B = FFT_M(w): the kernel array as a one-line grid of M points
  GridDev L = G;
  L.dim = 1;
  L.psi = b.bhat;
  L.ax[0] = G.ax[0];
  L.ax[0].n = M;
  L.ax[0].n2 = M / 2;
  L.ax[0].stride = 1;
  L.ax[0].tw = b.tw;
  L.ax[0].twx = b.twx;
  L.ax[0].twf = reinterpret_cast<decltype(L.ax[0].twf)>(b.twf);
  L.m = M;
  for (int k = 0; k < kMaxDim; ++k) L.tmap[k] = nullptr;
  return fft_M(g, L, 0, true, 1.0, g->stream);
}

void bs_release(qsf_grid* g) {
  qsf_grid::Bluestein& b = g->bs;
  for (void* p : {(void*)b.chirp, (void*)b.bhat, (void*)b.scratch})  // the twiddles are shared
    if (p) cudaFree(p);
  b = qsf_grid::Bluestein();
}

int bs_axis(qsf_grid* g, double2* arr, int ax, bool fwd, double post) {
  const GridDev& G = g->G;
  const qsf_grid::Bluestein& b = g->bs;
  const int n = b.n, M = b.M;
  const long long inner = G.ax[ax].stride, outer = G.m / ((long long)n * inner);
  const GridDev S = scratch_view(g, ax);
  cudaStream_t st = g->stream;
  const int inv = fwd ? 0 : 1;
  k_bs_pre<<<blocks_for(outer * M * inner), 256, 0, st>>>(arr, b.scratch, b.chirp, outer, n, M, inner, inv);
  QSF_CU(cudaGetLastError());
  int rc;
  if ((rc = fft_M(g, S, ax, true, 1.0, st))) return rc;
  k_bs_mul<<<blocks_for(outer * M * inner), 256, 0, st>>>(b.scratch, b.bhat, outer, M, inner);
  QSF_CU(cudaGetLastError());
  if ((rc = fft_M(g, S, ax, false, 1.0 / (double)M, st))) return rc;
  k_bs_post<<<blocks_for(outer * n * inner), 256, 0, st>>>(arr, b.scratch, b.chirp, outer, n, M, inner, inv, post);
  QSF_CU(cudaGetLastError());
  return QSF_OK;
}

}  // namespace qsf
