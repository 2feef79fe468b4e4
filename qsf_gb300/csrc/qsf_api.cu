// qsf_api.cu -- host side of libqsfgpu.so: the C ABI declared in include/qsf_gpu.h.
//
// Owns the device state of each grid (wavefunction, phase tables, twiddles, flux
// point lists, reduction scratch), plans the FFTs (radix 16/8/4/2 first, then 3, 5),
// evaluates the border vectors once per border set, and launches the kernels of
// qsf_kernels.cuh -- per step through a captured CUDA graph that a device-side step
// counter makes reusable for every step of a call.
#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#define QSF_DEFINE_KERNELS
#include <cuda.h>  // CUtensorMap and its encoder's signature (the encoder comes from the runtime's entry point)

#include "qsf_internal.h"

using namespace qsf;

namespace qsf {
namespace {
thread_local std::string g_err;
}  // namespace
int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}
int device_sm_count() {
  static std::atomic<int> cache[64];  // zero-initialised (static storage); read by any host thread
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return 152;
  if (dev < 64) {
    const int c = cache[dev].load(std::memory_order_relaxed);
    if (c > 0) return c;
  }
  int n = 0;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 152;
  if (dev < 64) cache[dev].store(n, std::memory_order_relaxed);
  return n;
}
}  // namespace qsf

namespace {

// the compile-time radix plan of qsf_fft.cuh, for reporting
bool plan_radices(int64_t n, std::vector<int>& r) {
  r.clear();
  if (n < 2 || n > (1 << 24) || !is_smooth((int)n)) return false;
  for (int i = 0; i < nstages((int)n); ++i) r.push_back(radix_at((int)n, i));
  return true;
}

std::vector<KernelSet>& kernel_table();

// kernel launch geometry
constexpr int kMaxLine1D = 16384;       // 1D line in shared memory (one CTA up to 8192, a cluster pair above)
constexpr int kMaxFluxBlocks = 512;  // blocks of the flux-term sums (256 terms each)
constexpr int kMaxTile = 4096;          // points per block in row / axis passes

}  // namespace

namespace qsf {
void set_error_message(const std::string& msg) { fail(0, msg); }
void add_sizes_p2a(std::vector<KernelSet>& out);
void add_sizes_p2b(std::vector<KernelSet>& out);
void add_sizes_r3(std::vector<KernelSet>& out);
void add_sizes_r5(std::vector<KernelSet>& out);
void add_sizes_long(std::vector<KernelSet>& out);
const KernelSet* kernels_for(int n) {
  for (const KernelSet& k : kernel_table())
    if (k.n == n) return &k;
  return nullptr;
}
}  // namespace qsf


namespace {

// The table of kernel sets, one per supported line length (qsf_sizes_*.cu), with the
// dynamic shared memory limits raised once.
std::vector<KernelSet>& kernel_table() {
  static std::vector<KernelSet> t;
  return t;
}

int init_kernel_table() {
  static std::mutex mu;
  static bool done = false;
  std::lock_guard<std::mutex> lk(mu);
  if (done) return QSF_OK;
  std::vector<KernelSet>& t = kernel_table();
  t.clear();  // a failed earlier attempt starts over
  add_sizes_p2a(t);
  add_sizes_p2b(t);
  add_sizes_r3(t);
  add_sizes_r5(t);
  add_sizes_long(t);
  auto lim = [](const void* f, int bytes) -> int {
    if (!f) return QSF_OK;
    QSF_CU(cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    return QSF_OK;
  };
  // dynamic shared memory actually requested: tiles of kMaxTile points (row / axis
  // passes), lines of up to 16 * kLineThreads points (line kernel, plain row FFT)
  const int tile = kMaxTile * (int)sizeof(double2);
  const int line = 16 * kLineThreads * (int)sizeof(double2);
  for (const KernelSet& k : t) {
    int rc;
    if ((rc = lim((const void*)k.row_open, tile)) || (rc = lim((const void*)k.row_close, tile)) ||
        (rc = lim((const void*)k.axis_fwd, tile)) || (rc = lim((const void*)k.axis_inv, tile)) ||
        (rc = lim((const void*)k.axis_fpi, tile)) || (rc = lim((const void*)k.axis_ekin, tile)) ||
        (rc = lim((const void*)k.axis_fft_f, tile)) || (rc = lim((const void*)k.axis_fft_b, tile)) ||
        (rc = lim((const void*)k.row_fft_f, line)) || (rc = lim((const void*)k.row_fft_b, line)) ||
        (rc = lim((const void*)k.line_step, k.n / k.line_ctas * (int)sizeof(double2))))
      return rc;
  }
  done = true;
  return QSF_OK;
}

int grid_blocks(long long m) {
  long long b = (m + 255) / 256;
  return (int)std::min<long long>(std::max<long long>(b, 1), (long long)device_sm_count() * 16);
}

// One twiddle as the fixed-point FFT reads it.  With pre-split tables (QSF_TWQ) each
// component w becomes its signed 32-bit halves {lo = (int)w, hi} (the bytes of an int4
// {re lo, re hi, im lo, im hi}); a component whose low half would be -2^31 moves one
// unit (2^-62) so that the kernels can negate the halves.
longlong2 split_twiddle(longlong2 w) {
#if QSF_TWQ
  int q[4];
  const long long c[2] = {w.x, w.y};
  for (int k = 0; k < 2; ++k) {
    long long v = c[k];
    if ((v & 0xffffffffLL) == 0x80000000LL) v += 1;
    const int lo = k_lo(v), hi = k_hi(v);
    q[2 * k] = lo;
    q[2 * k + 1] = hi;
  }
  longlong2 out;
  std::memcpy(&out, q, sizeof out);
  return out;
#else
  return w;
#endif
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link against the
// driver library); null when the driver does not offer it
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn encode_tiled() {
  static std::mutex mu;
  static bool tried = false;
  static EncodeTiledFn fn = nullptr;
  std::lock_guard<std::mutex> lk(mu);
  if (!tried) {
    tried = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
    else
      cudaGetLastError();
  }
  return fn;
}

// Tensor maps of psi for the strided-axis passes of axes 0 .. dim-2: psi as 64-bit
// words, dims {2 * stride, n, outer}, box {2 * tile columns, tma_box_rows(n), 1} (the
// boxes the pass's load_aligned issues); left null (cp.async loads) without an encoder.
int make_tensor_maps(qsf_grid* g) {
  GridDev& G = g->G;
  for (int ax = 0; ax < kMaxDim; ++ax) G.tmap[ax] = nullptr;
  EncodeTiledFn fn = encode_tiled();
  if (G.dim < 2 || !fn) return QSF_OK;
  if (int rc = dev_alloc(g->tmaps, (size_t)kMaxDim * 128)) return rc;
  for (int ax = 0; ax + 1 < G.dim; ++ax) {
    const AxisDev& a = G.ax[ax];
    const long long inner = a.stride, outer = G.m / ((long long)a.n * inner);
    const cuuint64_t dims[3] = {(cuuint64_t)(2 * inner), (cuuint64_t)a.n, (cuuint64_t)outer};
    const cuuint64_t strides[2] = {(cuuint64_t)(16 * inner), (cuuint64_t)(16 * inner * a.n)};
    const cuuint32_t box[3] = {(cuuint32_t)(2 * g->ax_C[ax]), (cuuint32_t)tma_box_rows(a.n), 1};
    const cuuint32_t elem[3] = {1, 1, 1};
    alignas(64) CUtensorMap map;
    if (fn(&map, CU_TENSOR_MAP_DATA_TYPE_UINT64, 3, G.psi, dims, strides, box, elem, CU_TENSOR_MAP_INTERLEAVE_NONE,
           CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) !=
        CUDA_SUCCESS)
      continue;  // this axis keeps cp.async loads
    // on the grid's stream and waited for: a pageable copy on another stream may still
    // be in flight when it returns, unordered with the grid's later work
    QSF_CU(cudaMemcpyAsync(g->tmaps + 128 * ax, &map, sizeof(map), cudaMemcpyHostToDevice, g->stream));
    QSF_CU(cudaStreamSynchronize(g->stream));
    G.tmap[ax] = g->tmaps + 128 * ax;
  }
  return QSF_OK;
}

}  // namespace

bool qsf::fused_length(int n) { return init_kernel_table() == QSF_OK && kernels_for(n) != nullptr; }

// FP64, 2^62 fixed-point and split-form twiddles exp(-2 pi i t / n), t < n
int qsf::make_twiddles(int n, double2** tw, longlong2** twx, longlong2** twf) {
  std::vector<double2> h((size_t)n);
  std::vector<longlong2> hx((size_t)n), hf((size_t)n);
  const long double twopi = 6.283185307179586476925286766559005768L;
  const long double q62 = 4611686018427387904.0L;
  for (int t = 0; t < n; ++t) {
    const long double ang = twopi * (long double)t / (long double)n;
    const long double c = cosl(ang), sn = -sinl(ang);
    h[(size_t)t] = make_double2((double)c, (double)sn);
    hx[(size_t)t] = make_longlong2(llroundl(c * q62), llroundl(sn * q62));
    hf[(size_t)t] = split_twiddle(hx[(size_t)t]);
  }
  *tw = nullptr;
  *twx = *twf = nullptr;
  int rc;
  if ((rc = dev_alloc(*tw, h.size())) || (rc = dev_alloc(*twx, hx.size())) || (rc = dev_alloc(*twf, hf.size()))) {
    if (*tw) cudaFree(*tw);
    if (*twx) cudaFree(*twx);
    *tw = nullptr;
    *twx = nullptr;
    return rc;
  }
  QSF_CU(cudaMemcpy(*tw, h.data(), h.size() * sizeof(double2), cudaMemcpyHostToDevice));
  QSF_CU(cudaMemcpy(*twx, hx.data(), hx.size() * sizeof(longlong2), cudaMemcpyHostToDevice));
  QSF_CU(cudaMemcpy(*twf, hf.data(), hf.size() * sizeof(longlong2), cudaMemcpyHostToDevice));
  // a pageable copy may return before its transfer lands; the tables are shared by
  // every stream, so wait for the device
  QSF_CU(cudaDeviceSynchronize());
  return QSF_OK;
}

// Twiddle tables of a length, made once per process and device and shared by every
// grid (never freed: one set per built length, at most a few MB in all).
int qsf::shared_twiddles(int n, double2** tw, longlong2** twx, longlong2** twf) {
  static std::mutex mu;
  static std::map<std::pair<int, int>, std::array<void*, 3>> cache;
  int dev = 0;
  QSF_CU(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(mu);
  auto it = cache.find({dev, n});
  if (it == cache.end()) {
    double2* a = nullptr;
    longlong2 *b = nullptr, *c = nullptr;
    if (int rc = make_twiddles(n, &a, &b, &c)) return rc;
    it = cache.emplace(std::make_pair(dev, n), std::array<void*, 3>{a, b, c}).first;
  }
  *tw = (double2*)it->second[0];
  *twx = (longlong2*)it->second[1];
  *twf = (longlong2*)it->second[2];
  return QSF_OK;
}

namespace {

double decode_ordered(long long i) {
  if (i < 0) i ^= 0x7fffffffffffffffLL;
  double x;
  std::memcpy(&x, &i, sizeof x);
  return x;
}

// Static tables of X(delta) in fixed point.  The potential's range sets its
// fixed-point scale (|V| * 2^vshift < 2^50) and, in imaginary time, the exponent taken
// out of the X factor exp(-delta V) so that the stored factors stay <= 1.
int ensure_static(qsf_grid* g, int mode, double delta) {
  const long long m = g->G.m;
  if (!g->Vx) {
    int rc = dev_alloc(g->Vx, (size_t)m);
    if (rc) return rc;
  }
  if (!g->xs) {
    int rc = dev_alloc(g->xs, (size_t)m);
    if (rc) return rc;
  }
  if (g->xs_mode == mode && g->xs_delta == delta && g->V_ready) return QSF_OK;
  if (!g->V_ready) {
    long long* rng = nullptr;
    int rc = dev_alloc(rng, 2);
    if (rc) return rc;
    const long long init[2] = {-0x7fffffffffffffffLL - 1, -0x7fffffffffffffffLL - 1};
    long long h[2];
    cudaError_t ce = cudaMemcpyAsync(rng, init, sizeof init, cudaMemcpyHostToDevice, g->stream);
    if (ce == cudaSuccess) {
      k_vrange<<<grid_blocks(m), 256, 0, g->stream>>>(g->G, rng);
      ce = cudaGetLastError();
    }
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(h, rng, sizeof h, cudaMemcpyDeviceToHost, g->stream);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(g->stream);
    cudaFree(rng);
    if (ce != cudaSuccess) return fail(QSF_ECUDA, std::string("potential range: ") + cudaGetErrorString(ce));
    g->vmax = decode_ordered(h[0]);
    g->vneg = decode_ordered(h[1]);
    if (!std::isfinite(g->vmax) || !std::isfinite(g->vneg))
      return fail(QSF_EINVAL, "the potential is not finite on the grid");
    const double vabs = std::max(std::fabs(g->vmax), std::fabs(g->vneg));
    int e = 0;
    if (vabs > 0.0) std::frexp(vabs, &e);  // vabs < 2^e
    g->vshift = 50 - e;
  }
  g->xs_exp = 0;
  if (mode == QSF_MODE_IM && g->vneg > 0.0) {
    const double fmax = std::exp(delta * g->vneg);
    if (!std::isfinite(fmax)) return fail(QSF_EINVAL, "imaginary-time X factor overflows (dt * |V| too large)");
    if (fmax > 1.0) std::frexp(fmax, &g->xs_exp);
  }
  k_build_static<<<grid_blocks(m), 256, 0, g->stream>>>(g->G, mode, delta, g->xs_exp, reinterpret_cast<int4*>(g->xs),
                                                        g->Vx, g->vshift);
  QSF_CU(cudaGetLastError());
  g->xs_mode = mode;
  g->xs_delta = delta;
  g->V_ready = true;
  return QSF_OK;
}

int ensure_flux(qsf_grid* g, int nb, const int* types, int64_t box) {
  std::vector<int> want(types, types + nb);
  if (g->fl_ready && want == g->fl_borders && box == g->fl_box) return QSF_OK;
  const int D = g->G.dim;
  const int64_t R = border_reach(g->bn, box);
  int64_t lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1};
  for (int d = 0; d < D; ++d) {
    const int64_t n = g->G.ax[d].n, n2 = g->G.ax[d].n2;
    lo[d] = std::max<int64_t>(0, n2 - R);
    hi[d] = std::min<int64_t>(n, n2 + R + 1);
  }
  struct Pt {
    long long p;
    double w[QSF_MAX_BORDERS][3];
    unsigned mask;
  };
  std::vector<Pt> pts;
  std::vector<long long> need;
  const long long m = g->G.m;
  for (int64_t i0 = lo[0]; i0 < hi[0]; ++i0)
    for (int64_t i1 = lo[1]; i1 < hi[1]; ++i1)
      for (int64_t i2 = lo[2]; i2 < hi[2]; ++i2) {
        const int64_t idx[3] = {i0, i1, i2};
        int64_t ci[3];
        long long p = 0;
        for (int d = 0; d < D; ++d) {
          ci[d] = idx[d] - g->G.ax[d].n2;
          p = p * g->G.ax[d].n + idx[d];
        }
        Pt pt{};
        pt.p = p;
        pt.mask = 0;
        for (int b = 0; b < nb; ++b) {
          double w[3];
          if (!border_vector(types[b], box, D, ci, g->bn, w))
            return fail(QSF_EINVAL, "border type " + std::to_string(types[b]) + " is not defined for dim " +
                                        std::to_string(D));
          bool nz = false;
          for (int d = 0; d < D; ++d) {
            pt.w[b][d] = w[d];
            nz = nz || w[d] != 0.0;
          }
          if (nz) pt.mask |= 1u << b;
        }
        if (pt.mask) pts.push_back(pt);
      }
  // snapshot indices: every point and its valid +-stride neighbours (grid.h:470-472)
  for (const Pt& pt : pts) {
    need.push_back(pt.p);
    for (int d = 0; d < D; ++d) {
      const long long s = g->G.ax[d].stride;
      if (pt.p - s > 0 && pt.p + s < m) {
        need.push_back(pt.p + s);
        need.push_back(pt.p - s);
      }
    }
  }
  std::sort(need.begin(), need.end());
  need.erase(std::unique(need.begin(), need.end()), need.end());
  auto slot = [&](long long p) { return (int)(std::lower_bound(need.begin(), need.end(), p) - need.begin()); };
  std::vector<FluxPoint> fps;
  std::vector<FluxTerm> fts;
  for (const Pt& pt : pts) {
    FluxPoint fp{};
    fp.c = slot(pt.p);
    for (int d = 0; d < 3; ++d) fp.p[d] = fp.q[d] = -1;
    for (int d = 0; d < D; ++d) {
      const long long s = g->G.ax[d].stride;
      if (pt.p - s > 0 && pt.p + s < m) {
        fp.p[d] = slot(pt.p + s);
        fp.q[d] = slot(pt.p - s);
      }
    }
    const int pi = (int)fps.size();
    fps.push_back(fp);
    for (int b = 0; b < nb; ++b)
      if (pt.mask & (1u << b)) {
        FluxTerm ft{};
        ft.point = pi;
        ft.border = b;
        for (int d = 0; d < 3; ++d) ft.w[d] = d < D ? pt.w[b][d] : 0.0;
        fts.push_back(ft);
      }
  }
  const long long nlast = g->G.ax[D - 1].n;
  const long long nrows = m / nlast;
  std::vector<int> rp((size_t)nrows + 1, 0);
  for (long long p : need) rp[(size_t)(p / nlast) + 1]++;
  for (long long r = 0; r < nrows; ++r) rp[(size_t)r + 1] += rp[(size_t)r];
  int rc;
  if ((rc = dev_alloc(g->snap, std::max<size_t>(need.size(), 1)))) return rc;
  if ((rc = dev_alloc(g->snap_idx, std::max<size_t>(need.size(), 1)))) return rc;
  if ((rc = dev_alloc(g->row_ptr, rp.size()))) return rc;
  if ((rc = dev_alloc(g->fpts, std::max<size_t>(fps.size(), 1)))) return rc;
  if ((rc = dev_alloc(g->fterms, std::max<size_t>(fts.size(), 1)))) return rc;
  // on the grid's stream (ordered before its later work) and waited for
  cudaStream_t st = g->stream;
  if (!need.empty())
    QSF_CU(cudaMemcpyAsync(g->snap_idx, need.data(), need.size() * sizeof(long long), cudaMemcpyHostToDevice, st));
  QSF_CU(cudaMemcpyAsync(g->row_ptr, rp.data(), rp.size() * sizeof(int), cudaMemcpyHostToDevice, st));
  if (!fps.empty())
    QSF_CU(cudaMemcpyAsync(g->fpts, fps.data(), fps.size() * sizeof(FluxPoint), cudaMemcpyHostToDevice, st));
  if (!fts.empty())
    QSF_CU(cudaMemcpyAsync(g->fterms, fts.data(), fts.size() * sizeof(FluxTerm), cudaMemcpyHostToDevice, st));
  QSF_CU(cudaStreamSynchronize(st));
  g->nsnap = (int)need.size();
  g->nfpts = (int)fps.size();
  g->nfterms = (int)fts.size();
  // one thread per flux term (each is a chain of dependent loads: latency, not bandwidth)
  g->nfblk = (int)std::min<long long>(kMaxFluxBlocks, std::max<long long>(1, (g->nfterms + 255) / 256));
  g->fl_borders = want;
  g->fl_box = box;
  g->fl_ready = true;
  return QSF_OK;
}

// Optional per-launch event timing (qsf_step_desc.kernel_ms): every launch of a step
// is bracketed by a pair of events from a pool; the pairs are read after the step's
// work is queued and synchronised once, so timing adds no host gaps between kernels.
struct Prof {
  float* ms = nullptr;
  int64_t* count = nullptr;
  cudaStream_t st = nullptr;
  std::vector<cudaEvent_t> ev;
  std::vector<int> kinds;
  int used = 0;
  int init(cudaStream_t s, int pairs) {
    st = s;
    ev.resize((size_t)pairs * 2);
    for (auto& e : ev) QSF_CU(cudaEventCreate(&e));
    return QSF_OK;
  }
  void release() {
    for (auto& e : ev)
      if (e) cudaEventDestroy(e);
    ev.clear();
  }
  int begin() {
    if (!ms) return QSF_OK;
    if ((size_t)(used * 2 + 1) >= ev.size()) return fail(QSF_EINVAL, "profiling event pool exhausted");
    QSF_CU(cudaEventRecord(ev[(size_t)used * 2], st));
    return QSF_OK;
  }
  int end(int kind) {
    if (!ms) return QSF_OK;
    QSF_CU(cudaEventRecord(ev[(size_t)used * 2 + 1], st));
    kinds.push_back(kind);
    ++used;
    return QSF_OK;
  }
  int flush() {
    if (!ms || used == 0) return QSF_OK;
    QSF_CU(cudaEventSynchronize(ev[(size_t)used * 2 - 1]));
    for (int i = 0; i < used; ++i) {
      float t = 0.f;
      QSF_CU(cudaEventElapsedTime(&t, ev[(size_t)i * 2], ev[(size_t)i * 2 + 1]));
      ms[kinds[(size_t)i]] += t;
      if (count) count[kinds[(size_t)i]] += 1;
    }
    used = 0;
    kinds.clear();
    return QSF_OK;
  }
};

// Launch geometry shared by every solve of one (dim, line length) group.
struct Geom {
  int dim = 1, n = 0, nmax = 0, gauge = 0;
  int nrowblk = 1, row_L = 1;
  size_t row_smem = 0;
  int ax_blocks[3] = {0, 0, 0}, ax_C[3] = {1, 1, 1};
  size_t ax_smem[3] = {0, 0, 0};
};

Geom geom_of(const qsf_grid* g) {
  Geom q;
  q.dim = g->G.dim;
  q.n = g->G.ax[0].n;
  q.nmax = g->nmax;
  q.gauge = g->G.gauge;
  q.nrowblk = g->nrowblk;
  q.row_L = g->row_L;
  q.row_smem = g->row_smem;
  for (int k = 0; k < 3; ++k) {
    q.ax_blocks[k] = g->ax_blocks[k];
    q.ax_C[k] = g->ax_C[k];
    q.ax_smem[k] = g->ax_smem[k];
  }
  return q;
}

// k_finalize on a second stream (`side`): it forks from `st` after the sub-step's last
// pass, and the next sub-step waits for it (`done`) only before its pass that rewrites
// the partials and the flux snapshot.  Valid when k_finalize writes nothing the next
// sub-step's earlier kernels read: no pending Normalize factor, no convergence stop.
struct FinOverlap {
  cudaStream_t side = nullptr;
  cudaEvent_t fork = nullptr, done = nullptr;
  bool pending = false;
};

// One step's launches for `count` solves sharing kernels K and geometry q; every
// kernel reads its solve's descriptors (blockIdx.y) and step counter from device memory.
int launch_group(const KernelSet& K, const Geom& q, const GridDev* dG, const StepDev* dS, int count, bool ekin,
                 int nfblk, cudaStream_t st, Prof* P, bool with_open = true, FinOverlap* ov = nullptr) {
  Prof none;
  Prof& pf = P ? *P : none;
  int rc;
#define QSF_TIMED(kind, launch)             \
  do {                                      \
    if ((rc = pf.begin())) return rc;       \
    launch;                                 \
    QSF_CU(cudaGetLastError());             \
    if ((rc = pf.end(kind))) return rc;     \
  } while (0)
  const int D = q.dim;
  // (kind, axis) tables (X tables only in the length gauge), ~128 entries per block
  const int tb = std::max(1, std::min(64, q.nmax / 128));
  const dim3 gt(D * 4 * tb, count);
  // a one-CTA line kernel also ends the step itself (its fluxes, row and counters); the
  // tables stay a kernel of their own: their FP64 phases want many SMs
  const bool full = D == 1 && K.line_full;
  QSF_TIMED(QSF_K_TABLES, (k_tables<<<gt, 256, 0, st>>>(dG, dS, tb)));
  const bool wait_fin = ov && ov->pending;
  if (D == 1) {
    if (wait_fin) QSF_CU(cudaStreamWaitEvent(st, ov->done, 0));
    QSF_TIMED(QSF_K_LINE_STEP, (K.line_step<<<dim3(K.line_ctas, count), K.line_threads,
                                               (size_t)(q.n / K.line_ctas) * sizeof(double2), st>>>(dG, dS)));
  } else {
    const dim3 gr(q.nrowblk, count);
    if (with_open) QSF_TIMED(QSF_K_ROW_OPEN, (K.row_open<<<gr, K.row_threads, q.row_smem, st>>>(dG, dS, q.row_L)));
    if (D == 3)
      QSF_TIMED(QSF_K_AXIS_FWD,
                (K.axis_fwd<<<dim3(q.ax_blocks[1], count), K.row_threads, q.ax_smem[1], st>>>(dG, dS, 1, q.ax_C[1])));
    QSF_TIMED(QSF_K_AXIS_FPI,
              (K.axis_fpi<<<dim3(q.ax_blocks[0], count), K.row_threads, q.ax_smem[0], st>>>(dG, dS, 0, q.ax_C[0])));
    if (D == 3)
      QSF_TIMED(QSF_K_AXIS_INV,
                (K.axis_inv<<<dim3(q.ax_blocks[1], count), K.row_threads, q.ax_smem[1], st>>>(dG, dS, 1, q.ax_C[1])));
    if (wait_fin) QSF_CU(cudaStreamWaitEvent(st, ov->done, 0));
    QSF_TIMED(QSF_K_ROW_CLOSE, (K.row_close<<<gr, K.row_threads, q.row_smem, st>>>(dG, dS, q.row_L)));
    if (ekin)
      for (int ax = 0; ax < D - 1; ++ax)
        QSF_TIMED(QSF_K_AXIS_EKIN,
                  (K.axis_ekin<<<dim3(q.ax_blocks[ax], count), K.row_threads, q.ax_smem[ax], st>>>(dG, dS, ax, q.ax_C[ax])));
  }
  if (ov) ov->pending = false;
  if (!full && ov) {
    QSF_CU(cudaEventRecord(ov->fork, st));
    QSF_CU(cudaStreamWaitEvent(ov->side, ov->fork, 0));
    k_finalize<<<dim3(nfblk, count), 256, 0, ov->side>>>(dG, dS);
    QSF_CU(cudaGetLastError());
    QSF_CU(cudaEventRecord(ov->done, ov->side));
    ov->pending = true;
  } else if (!full) {
    QSF_TIMED(QSF_K_FINALIZE, (k_finalize<<<dim3(nfblk, count), 256, 0, st>>>(dG, dS)));
  }
#undef QSF_TIMED
  return QSF_OK;
}

int launch_step(qsf_grid* g, const StepDev& S, Prof* P = nullptr, bool with_open = true, FinOverlap* ov = nullptr) {
  return launch_group(*g->ks, geom_of(g), g->dG, g->dS, 1, (S.obs & QSF_OBS_EKIN) != 0,
                      S.nfterms > 0 ? g->nfblk : 1, g->stream, P, with_open, ov);
}

// Whether k_finalize may run beside the next sub-step (FinOverlap), and its stream.
bool fin_overlap_ok(const StepDev& S) { return !S.normalize && !(S.mode == 1 && S.state_accuracy > 0.0); }
int ensure_fin_stream(qsf_grid* g, FinOverlap* ov) {
  if (!g->fin_stream) {
    QSF_CU(cudaStreamCreateWithFlags(&g->fin_stream, cudaStreamNonBlocking));
    QSF_CU(cudaEventCreateWithFlags(&g->fin_fork, cudaEventDisableTiming));
    QSF_CU(cudaEventCreateWithFlags(&g->fin_done, cudaEventDisableTiming));
  }
  ov->side = g->fin_stream;
  ov->fork = g->fin_fork;
  ov->done = g->fin_done;
  ov->pending = false;
  return QSF_OK;
}

// Validates a step program and stages everything a run of it needs on the device:
// static tables for dt/2, flux point lists, coupling rows, observables rows, control
// words; fills the step descriptor and uploads it to g->dS.
int prepare_step(qsf_grid* g, const qsf_step_desc* d, StepDev* out, int* ncol_out) {
  if (d->mode != QSF_MODE_IM && d->mode != QSF_MODE_RE) return fail(QSF_EINVAL, "mode must be IM or RE");
  if (d->nsteps < 1) return fail(QSF_EINVAL, "nsteps < 1");
  if (d->nborders < 0 || d->nborders > QSF_MAX_BORDERS) return fail(QSF_EINVAL, "too many borders");
  if (d->substeps < 0 || d->substeps > 64) return fail(QSF_EINVAL, "substeps must be in [0, 64]");
  if (d->ekin_interval < 0) return fail(QSF_EINVAL, "ekin_interval must be >= 0");
  if (g->G.free_mask)
    return fail(QSF_EINVAL, "a region with free axes keeps them in momentum space: step it with the member operations");
  const GridDev& G = g->G;
  const int K = std::max(1, d->substeps);
  const int64_t total = d->nsteps * K;  // sub-steps
  const double dt_sub = d->dt / K;
  int rc;
  if ((rc = ensure_static(g, d->mode, dt_sub * 0.5))) return rc;
  const bool want_flux = (d->obs & QSF_OBS_FLUX) && d->nborders > 0;
  if (want_flux && (rc = ensure_flux(g, d->nborders, d->border_types, d->box_size))) return rc;
  const int nb = want_flux ? d->nborders : 0;
  const int ncol = 3 + nb;
  const int cstride = G.gauge == QSF_GAUGE_LENGTH ? 6 : 3;
  if ((rc = dev_reserve(g->rows_dev, g->rows_cap, (size_t)d->nsteps * ncol))) return rc;
  const double* coup = nullptr;
  if (d->coupling) {
    if ((rc = dev_reserve(g->coup_dev, g->coup_cap, (size_t)total * cstride))) return rc;
    QSF_CU(cudaMemcpyAsync(g->coup_dev, d->coupling, (size_t)total * cstride * sizeof(double),
                           cudaMemcpyHostToDevice, g->stream));
    coup = g->coup_dev;
  }
  long long ctl_h[8] = {0, (long long)total, 0, 0, 0, 0, 0, 0};
  double en_h[2] = {d->last_energy, 0.0};
  double sc_h[2] = {1.0, 1.0};
  QSF_CU(cudaMemcpyAsync(g->ctl, ctl_h, sizeof(ctl_h), cudaMemcpyHostToDevice, g->stream));
  QSF_CU(cudaMemcpyAsync(g->energy, en_h, sizeof(en_h), cudaMemcpyHostToDevice, g->stream));
  QSF_CU(cudaMemcpyAsync(g->scale, sc_h, sizeof(sc_h), cudaMemcpyHostToDevice, g->stream));
  StepDev S{};
  S.mode = d->mode;
  S.dt = dt_sub;
  S.nsteps = total;
  S.substeps = K;
  S.coupling = coup;
  S.coup_stride = cstride;
  S.xs = reinterpret_cast<const int4*>(g->xs);
  S.Vx = g->Vx;
  S.ptab = reinterpret_cast<int4*>(g->ptab);
  S.xdyn = reinterpret_cast<int4*>(g->xdyn);
  S.xs_exp = g->xs_exp;
  S.vshift = g->vshift;
  S.l2m = g->l2m;
  S.m_mant = g->m_mant;
  S.texp = g->ibuf;
  S.gmin = g->ibuf + kTexp;
  S.sc = g->ibuf + kTexp + kGmin;
  S.scmax = g->scmax;
  S.nmax = g->nmax;
  S.partials = g->partials;
  S.pmax = g->pmax;
  S.nrowblk = g->nrowblk;
  for (int ax = 0; ax < 3; ++ax) S.naxblk[ax] = g->ax_blocks[ax];
  S.obs = d->obs | QSF_OBS_NORM;
  if (nb == 0) S.obs &= ~QSF_OBS_FLUX;
  // steps of a call stay in fixed point between steps, except after the steps whose
  // E_kin needs psi_n in memory (every ekin_interval-th step and the last one)
  S.fused = G.dim >= 2 ? 1 : 0;
  S.ekin_every = d->ekin_interval > 1 ? d->ekin_interval : 1;
  S.normalize = d->normalize;
  S.energy_after_normalize = d->energy_after_normalize;
  S.state_accuracy = d->mode == QSF_MODE_IM ? d->state_accuracy : 0.0;
  S.nborders = nb;
  if (want_flux) {
    S.snap = g->snap;
    S.row_ptr = g->row_ptr;
    S.snap_idx = g->snap_idx;
    S.fpts = g->fpts;
    S.fterms = g->fterms;
    S.nfterms = g->nfterms;
  }
  S.fpartials = g->fpartials;
  S.ctl = g->ctl;
  S.energy_state = g->energy;
  S.rows = g->rows_dev;
  S.scale = g->scale;
  QSF_CU(cudaMemcpyAsync(g->dS, &S, sizeof(StepDev), cudaMemcpyHostToDevice, g->stream));
  *out = S;
  *ncol_out = ncol;
  return QSF_OK;
}

// After a run: pending Normalize factor, observables rows and progress back to host.
int finish_step(qsf_grid* g, int normalize, int64_t nsteps, int ncol, double* rows, int64_t* steps_done) {
  if (normalize) {
    k_scale<<<grid_blocks(g->G.m), 256, 0, g->stream>>>(g->G.psi, g->G.m, g->scale);
    QSF_CU(cudaGetLastError());
  }
  long long ctl_h[8];
  QSF_CU(cudaMemcpyAsync(ctl_h, g->ctl, sizeof(ctl_h), cudaMemcpyDeviceToHost, g->stream));
  if (rows)
    QSF_CU(cudaMemcpyAsync(rows, g->rows_dev, (size_t)nsteps * ncol * sizeof(double), cudaMemcpyDeviceToHost,
                           g->stream));
  QSF_CU(cudaStreamSynchronize(g->stream));
  if (steps_done) *steps_done = ctl_h[2];
  if (ctl_h[4] == 2) return fail(QSF_ETIMEDOUT, "a bulk copy into shared memory did not complete in time");
  if (ctl_h[4]) return fail(QSF_ENUMERIC, "non-positive norm or NaN in a step's reductions");
  return QSF_OK;
}

// Captures the launches issued by `body` on `st` into an executable graph.
template <class F>
int capture_graph(cudaStream_t st, F&& body, cudaGraphExec_t* exec) {
  cudaGraph_t graph = nullptr;
  QSF_CU(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  const int rc = body();
  cudaError_t ce = cudaStreamEndCapture(st, &graph);
  if (rc) {
    if (graph) cudaGraphDestroy(graph);
    return rc;
  }
  if (ce != cudaSuccess) return fail(QSF_ECUDA, std::string("graph capture: ") + cudaGetErrorString(ce));
  ce = cudaGraphInstantiate(exec, graph, 0);
  cudaGraphDestroy(graph);
  if (ce != cudaSuccess) return fail(QSF_ECUDA, std::string("graph instantiate: ") + cudaGetErrorString(ce));
  return QSF_OK;
}

struct BatchMember {
  qsf_grid* g = nullptr;
  StepDev S{};
  int64_t nsteps = 0;
  int ncol = 0;
  int normalize = 0;
  bool scaled = false;
};

struct BatchGroup {
  const KernelSet* ks = nullptr;
  Geom q;
  std::vector<int64_t> slots;
  GridDev* dG = nullptr;
  StepDev* dS = nullptr;
  bool ekin = false;
  int nfblk = 1;
};

}  // namespace

struct qsf_batch {
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::map<int64_t, BatchMember> members;
  int64_t next_slot = 0;
  bool dirty = true;
  std::vector<BatchGroup> groups;
  cudaGraphExec_t exec = nullptr;
  long long* ctl_host = nullptr;  // pinned, 8 words per member
  size_t ctl_cap = 0;
  // descriptor arrays of all groups (grow-only, so membership changes do not free device
  // memory, which would synchronise the device)
  GridDev* dG_all = nullptr;
  StepDev* dS_all = nullptr;
  size_t desc_cap = 0, dS_cap = 0;
  // one stream per group while the step graph is captured, so that the groups become
  // parallel branches of the graph (grow-only)
  std::vector<cudaStream_t> gstreams;
  std::vector<cudaEvent_t> gjoin;
  cudaEvent_t gfork = nullptr;
};

namespace {

void free_groups(qsf_batch* b) {
  b->groups.clear();
  if (b->exec) cudaGraphExecDestroy(b->exec);
  b->exec = nullptr;
}

// Regroups members by (dim, line length), uploads the descriptor arrays and captures
// one batch step (every group's launches) into a graph.
int rebuild_batch(qsf_batch* b) {
  free_groups(b);
  std::map<std::pair<int, int>, BatchGroup> by;
  for (auto& kv : b->members) {
    const qsf_grid* g = kv.second.g;
    BatchGroup& gr = by[{g->G.dim, g->G.ax[0].n}];
    if (!gr.ks) {
      gr.ks = g->ks;
      gr.q = geom_of(g);
    }
    gr.q.gauge = std::max(gr.q.gauge, g->G.gauge);
    gr.slots.push_back(kv.first);
    gr.ekin = gr.ekin || (kv.second.S.obs & QSF_OBS_EKIN);
    if (kv.second.S.nfterms > 0) gr.nfblk = std::max(gr.nfblk, g->nfblk);
  }
  const size_t total = b->members.size();
  int rc;
  if ((rc = dev_reserve(b->dG_all, b->desc_cap, total)) || (rc = dev_reserve(b->dS_all, b->dS_cap, total))) return rc;
  std::vector<GridDev> hg;
  std::vector<StepDev> hs;
  hg.reserve(total);
  hs.reserve(total);
  for (auto& kv : by) {
    BatchGroup gr = kv.second;
    gr.dG = b->dG_all + hg.size();
    gr.dS = b->dS_all + hs.size();
    for (int64_t slot : gr.slots) {
      const BatchMember& mb = b->members[slot];
      hg.push_back(mb.g->G);
      hs.push_back(mb.S);
    }
    b->groups.push_back(gr);
  }
  if (total) {
    QSF_CU(cudaMemcpyAsync(b->dG_all, hg.data(), total * sizeof(GridDev), cudaMemcpyHostToDevice, b->stream));
    QSF_CU(cudaMemcpyAsync(b->dS_all, hs.data(), total * sizeof(StepDev), cudaMemcpyHostToDevice, b->stream));
  }
  QSF_CU(cudaStreamSynchronize(b->stream));
  if (!b->groups.empty()) {
    if (!b->gfork) QSF_CU(cudaEventCreateWithFlags(&b->gfork, cudaEventDisableTiming));
    while (b->gstreams.size() < b->groups.size()) {
      cudaStream_t s2 = nullptr;
      cudaEvent_t e2 = nullptr;
      QSF_CU(cudaStreamCreateWithFlags(&s2, cudaStreamNonBlocking));
      QSF_CU(cudaEventCreateWithFlags(&e2, cudaEventDisableTiming));
      b->gstreams.push_back(s2);
      b->gjoin.push_back(e2);
    }
    int rc = capture_graph(
        b->stream,
        [&]() {
          // fork: every group on its own stream, joined back before the graph ends
          QSF_CU(cudaEventRecord(b->gfork, b->stream));
          for (size_t i = 0; i < b->groups.size(); ++i) {
            const BatchGroup& gr = b->groups[i];
            QSF_CU(cudaStreamWaitEvent(b->gstreams[i], b->gfork, 0));
            const int r = launch_group(*gr.ks, gr.q, gr.dG, gr.dS, (int)gr.slots.size(), gr.ekin, gr.nfblk,
                                       b->gstreams[i], nullptr);
            if (r) return r;
            QSF_CU(cudaEventRecord(b->gjoin[i], b->gstreams[i]));
            QSF_CU(cudaStreamWaitEvent(b->stream, b->gjoin[i], 0));
          }
          return QSF_OK;
        },
        &b->exec);
    if (rc) return rc;
  }
  b->dirty = false;
  return QSF_OK;
}

}  // namespace

// ======================================================================== C ABI
extern "C" {

const char* qsf_last_error(void) { return g_err.c_str(); }

int qsf_fft_plan_radices(int64_t n, int* radices, int* count) {
  std::vector<int> r;
  if (!plan_radices(n, r)) return fail(QSF_EINVAL, "size " + std::to_string(n) + " is not 2^a 3^b 5^c");
  if (count) *count = (int)r.size();
  if (radices)
    for (size_t i = 0; i < r.size(); ++i) radices[i] = r[i];
  return QSF_OK;
}

int qsf_grid_create(const qsf_grid_desc* d, void* stream, qsf_grid** out) {
  if (!d || !out) return fail(QSF_EINVAL, "null argument");
  *out = nullptr;
  if (d->dim < 1 || d->dim > 3) return fail(QSF_EINVAL, "dim must be 1, 2 or 3");
  for (int k = 0; k < d->dim; ++k)
    if (d->n[k] < 2 || !(d->dx[k] > 0)) return fail(QSF_EINVAL, "n >= 2 and dx > 0 required on every axis");
  if (d->dim >= 2)
    for (int k = 1; k < d->dim; ++k)
      if (d->n[k] != d->n[0] || d->dx[k] != d->dx[0])
        return fail(QSF_EINVAL, "dim >= 2 needs the same n and dx on every axis (the reference's P layout)");
  if (d->dim == 1 && d->n[0] > kMaxLine1D)
    return fail(QSF_EINVAL, "1D lines longer than " + std::to_string(kMaxLine1D) + " points are not supported");
  if (d->dim >= 2 && d->n[0] > kMaxTile) return fail(QSF_EINVAL, "axes longer than 4096 points are not supported");
  if (d->potential < 0 || d->potential > 3) return fail(QSF_EINVAL, "unknown potential");
  if (d->gauge != QSF_GAUGE_VELOCITY && d->gauge != QSF_GAUGE_LENGTH) return fail(QSF_EINVAL, "unknown gauge");
  if (d->multi_region != 0 && d->multi_region != 1) return fail(QSF_EINVAL, "multi_region must be 0 or 1");
  if (d->free_axes < 0 || d->free_axes >= (1 << d->dim) || (d->free_axes && !d->multi_region))
    return fail(QSF_EINVAL, "free_axes must be a mask of the grid's axes, on a multi-region grid");
  if (d->absorber != QSF_ABS_CAP && d->absorber != QSF_ABS_COS8) return fail(QSF_EINVAL, "unknown absorber");
  if (d->absorber == QSF_ABS_COS8 && (d->nCAP < 1 || 2 * d->nCAP > d->n[0] || !(d->mask_dt > 0) || d->multi_region))
    return fail(QSF_EINVAL, "the cos^(1/8) mask needs 1 <= nCAP <= n / 2, mask_dt > 0 and a single-region grid");
  if (d->multi_region) {
    // multigrid.h:19 (an absorber is required); partial potentials exist for the
    // reduced-dimensionality interactions (potential.h:144-178)
    if (d->nCAP < 1 || 2 * d->nCAP > d->n[0])
      return fail(QSF_EINVAL, "a multi-region grid needs 1 <= nCAP <= n / 2");
    if (d->potential == QSF_POT_COULOMB)
      return fail(QSF_EINVAL, "multi-region grids need a reduced-dimensionality interaction (no partial Coulomb)");
  }
  if (int rc = init_kernel_table()) return rc;
  // lengths without fused kernels (not in the built list, or with a prime factor above
  // 5) take Bluestein transforms and the member-operation step
  const KernelSet* ks = kernels_for((int)d->n[0]);
  if (!ks && !bs_size((int)d->n[0], d->dim))
    return fail(QSF_EINVAL, "grid size " + std::to_string(d->n[0]) + " has no kernels and no Bluestein length in "
                            "this build (1D lines up to 8192 points, other grids up to 2048 points per axis)");
  qsf_grid* g = new qsf_grid();
  g->desc = *d;
  g->ks = ks;
  GridDev& G = g->G;
  G.dim = d->dim;
  G.m = 1;
  for (int k = 0; k < d->dim; ++k) G.m *= d->n[k];
  if (stream) {
    g->stream = (cudaStream_t)stream;
  } else {
    if (cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking) != cudaSuccess) {
      delete g;
      return fail(QSF_ECUDA, "cudaStreamCreate failed");
    }
    g->own_stream = true;
  }
  // coords.h:55-93
  G.dV = 1.0;
  long long s = 1;
  for (int k = d->dim - 1; k >= 0; --k) {
    G.ax[k].stride = s;
    s *= d->n[k];
  }
  std::map<int64_t, double2*> tws;
  std::map<int64_t, longlong2*> twxs, twfs;
  for (int k = 0; k < d->dim; ++k) {
    AxisDev& a = G.ax[k];
    a.n = (int)d->n[k];
    a.n2 = a.n / 2;
    a.shift = (a.n & (a.n - 1)) == 0 ? __builtin_ctz((unsigned)a.n) : -1;
    a.dx = d->dx[k];
    G.dV *= d->dx[k];
    const double L = d->dx[k] * (double)(d->n[k] - 1);
    a.xmin = -0.5 * L;
    a.inv_2dx = (1.0 / d->dx[k]) / 2.0;
    a.dp = 2.0 * M_PI / (double)d->n[k] / d->dx[k];
    auto it = tws.find(a.n);
    if (!ks) {
      // Bluestein lengths run no n-point transform kernel: no n-point twiddles
      a.tw = nullptr;
      a.twx = nullptr;
      a.twf = nullptr;
    } else if (it == tws.end()) {
      double2* dptr = nullptr;
      longlong2 *xptr = nullptr, *fptr = nullptr;
      if (int rc = shared_twiddles(a.n, &dptr, &xptr, &fptr)) {
        qsf_grid_destroy(g);
        return rc;
      }
      tws[a.n] = dptr;
      twxs[a.n] = xptr;
      twfs[a.n] = fptr;
      a.tw = dptr;
      a.twx = xptr;
      a.twf = reinterpret_cast<decltype(a.twf)>(fptr);
    } else {
      a.tw = it->second;
      a.twx = twxs[a.n];
      a.twf = reinterpret_cast<decltype(a.twf)>(twfs[a.n]);
    }
  }
  G.inv_m = 1.0 / (double)G.m;
  G.dVm = G.dV * G.inv_m;
  G.nCAP = d->nCAP;
  if (d->nCAP > 0) {
    const double t = 3.0 / (double)d->nCAP;
    G.eta = t * (t * (t * t));
  }
  G.pot = d->potential;
  G.NEcharge = d->Ncharge * d->Echarge;
  G.EEcharge = d->Echarge * d->Echarge;
  G.Nsoft = d->Nsoft;
  G.Esoft = d->Esoft;
  G.gauge = d->gauge;
  G.n_fields = d->n_fields;
  G.p_swap = d->p_axis_swap ? 1 : 0;
  G.free_mask = d->free_axes;
  G.multi = d->multi_region;
  G.abs_kind = d->absorber;
  G.abs_rate = d->absorber == QSF_ABS_COS8 ? 1.0 / d->mask_dt : 0.0;
  if (d->border_nodes[0] > 0) g->bn.NS = d->border_nodes[0];
  if (d->border_nodes[1] > 0) g->bn.SD = d->border_nodes[1];
  if (d->border_nodes[2] > 0) g->bn.DT = d->border_nodes[2];
  if (d->border_nodes[3] > 0) g->bn.CAP = d->border_nodes[3];
  int rc;
  if ((rc = dev_alloc(G.psi, (size_t)G.m))) { qsf_grid_destroy(g); return rc; }
  cudaMemsetAsync(G.psi, 0, (size_t)G.m * sizeof(double2), g->stream);
  // launch geometry
  const int D = d->dim;
  const int nlast = G.ax[D - 1].n;
  const long long nrows = G.m / nlast;
  if (D >= 2) {
    g->row_L = (int)std::max<long long>(1, std::min<long long>(nrows, tile_pts(nlast) / nlast));
    g->nrowblk = (int)((nrows + g->row_L - 1) / g->row_L);
    g->row_smem = (size_t)g->row_L * nlast * sizeof(double2);
    for (int ax = 0; ax < D - 1; ++ax) {
      const AxisDev& a = G.ax[ax];
      const long long inner = a.stride;
      int C = (int)std::max<long long>(1, std::min<long long>({64, (long long)tile_pts(a.n) / a.n, inner}));
      g->ax_C[ax] = C;
      const long long outer = G.m / ((long long)a.n * inner);
      g->ax_blocks[ax] = (int)(outer * ((inner + C - 1) / C));
      g->ax_smem[ax] = (size_t)a.n * C * sizeof(double2);
    }
  } else {
    g->nrowblk = ks ? ks->line_ctas : 1;  // partial sums per CTA of the line
  }
  g->nmax = 0;
  for (int k = 0; k < D; ++k) g->nmax = std::max(g->nmax, G.ax[k].n);
  g->pmax = std::max({g->nrowblk, g->ax_blocks[0], g->ax_blocks[1], g->ax_blocks[2], 256});
  g->scmax = std::max({g->nrowblk, g->ax_blocks[0], g->ax_blocks[1], g->ax_blocks[2], 1});
  // 1/m = m_mant * 2^-l2m with m_mant in (0.5, 1]
  g->l2m = 0;
  while ((1LL << (g->l2m + 1)) <= G.m) ++g->l2m;
  g->m_mant = std::ldexp(1.0, g->l2m) / (double)G.m;
  if ((rc = dev_alloc(g->partials, (size_t)5 * g->pmax)) || (rc = dev_alloc(g->ctl, 8)) ||
      (rc = dev_alloc(g->energy, 2)) || (rc = dev_alloc(g->scale, 2)) ||
      (rc = dev_alloc(g->fpartials, (size_t)kMaxFluxBlocks * kMaxFluxBorders))) {
    qsf_grid_destroy(g);
    return rc;
  }
  // the fused kernels' exponent slots, per-step tables and device descriptors
  if (ks && ((rc = dev_alloc(g->ibuf, (size_t)kTexp + kGmin + 4 * (size_t)g->scmax)) ||
             (rc = dev_alloc(g->ptab, (size_t)D * g->nmax)) ||
             (rc = dev_alloc(g->xdyn, (size_t)3 * D * g->nmax)) || (rc = dev_alloc(g->dG, 1)) ||
             (rc = dev_alloc(g->dS, 1)))) {
    qsf_grid_destroy(g);
    return rc;
  }
  g->fpmax = (size_t)kMaxFluxBlocks * kMaxFluxBorders;
  if ((rc = ks ? make_tensor_maps(g) : bs_setup(g))) {
    qsf_grid_destroy(g);
    return rc;
  }
  if (ks) cudaMemcpyAsync(g->dG, &g->G, sizeof(GridDev), cudaMemcpyHostToDevice, g->stream);
  cudaMemsetAsync(g->partials, 0, sizeof(double) * 5 * g->pmax, g->stream);
  if (cudaStreamSynchronize(g->stream) != cudaSuccess) {
    qsf_grid_destroy(g);
    return fail(QSF_ECUDA, "grid initialisation failed");
  }
  *out = g;
  return QSF_OK;
}

int qsf_grid_destroy(qsf_grid* g) {
  if (!g) return QSF_OK;
  if (g->batch) qsf_batch_remove(g->batch, g->batch_slot);  // out of the batch's graph first
  if (g->stream) cudaStreamSynchronize(g->stream);
  auto fr = [](void* p) {
    if (p) cudaFree(p);
  };
  fr(g->G.psi);
  fr(g->xs);
  fr(g->Vx);
  fr(g->ibuf);
  fr(g->ptab);
  fr(g->xdyn);
  fr(g->partials);
  fr(g->fpartials);
  fr(g->ctl);
  fr(g->energy);
  fr(g->scale);
  fr(g->rows_dev);
  fr(g->coup_dev);
  fr(g->snap);
  fr(g->snap_idx);
  fr(g->row_ptr);
  fr(g->fpts);
  fr(g->fterms);
  fr(g->dG);
  fr(g->dS);
  fr(g->mg_slice);
  fr(g->etab);
  fr(g->eptab);
  fr(g->obs_log);
  fr(g->vtab);
  fr(g->mtab);
  for (const qsf_grid::StepGraph& sg : g->step_graphs) cudaGraphExecDestroy(sg.exec);
  if (g->gen_exec) cudaGraphExecDestroy(g->gen_exec);
  fr(g->tmaps);
  bs_release(g);
  if (g->mg_event) cudaEventDestroy(g->mg_event);
  if (g->fin_fork) cudaEventDestroy(g->fin_fork);
  if (g->fin_done) cudaEventDestroy(g->fin_done);
  if (g->fin_stream) cudaStreamDestroy(g->fin_stream);
  if (g->own_stream) cudaStreamDestroy(g->stream);
  delete g;
  return QSF_OK;
}

int qsf_grid_size(const qsf_grid* g, int64_t* m) {
  if (!g || !m) return fail(QSF_EINVAL, "null argument");
  *m = g->G.m;
  return QSF_OK;
}

int qsf_psi_device_ptr(qsf_grid* g, void** dptr) {
  if (!g || !dptr) return fail(QSF_EINVAL, "null argument");
  *dptr = g->G.psi;
  return QSF_OK;
}

int qsf_upload(qsf_grid* g, const double* host, int64_t m) {
  if (!g || !host) return fail(QSF_EINVAL, "null argument");
  if (m != g->G.m) return fail(QSF_EINVAL, "size mismatch");
  QSF_CU(cudaMemcpyAsync(g->G.psi, host, (size_t)m * sizeof(double2), cudaMemcpyHostToDevice, g->stream));
  QSF_CU(cudaStreamSynchronize(g->stream));
  return QSF_OK;
}

int qsf_download(qsf_grid* g, double* host, int64_t m) {
  if (!g || !host) return fail(QSF_EINVAL, "null argument");
  if (m != g->G.m) return fail(QSF_EINVAL, "size mismatch");
  QSF_CU(cudaMemcpyAsync(host, g->G.psi, (size_t)m * sizeof(double2), cudaMemcpyDeviceToHost, g->stream));
  QSF_CU(cudaStreamSynchronize(g->stream));
  return QSF_OK;
}

int qsf_synchronize(qsf_grid* g) {
  if (!g) return fail(QSF_EINVAL, "null argument");
  QSF_CU(cudaStreamSynchronize(g->stream));
  return QSF_OK;
}

// the per-axis one-node mask table (k_mask_tab), built once per grid
static int ensure_mtab(qsf_grid* g) {
  if (g->mtab) return QSF_OK;
  if (int rc = dev_alloc(g->mtab, (size_t)g->G.dim * g->nmax)) return rc;
  k_mask_tab<<<(g->G.dim * g->nmax + 255) / 256, 256, 0, g->stream>>>(g->G, g->nmax, g->mtab);
  QSF_CU(cudaGetLastError());
  return QSF_OK;
}

// one-axis transform of the array G.psi (grid geometry of g), scaled by sc on the way out
static void axis_fft(qsf_grid* g, const GridDev& G, int ax, bool fwd, double sc) {
  const KernelSet& K = *g->ks;
  const int D = G.dim;
  cudaStream_t st = g->stream;
  {
    if (ax == D - 1) {
      // rows of the last axis with up to 16 * kLineThreads points per block
      const int n = G.ax[ax].n;
      const long long nrows = G.m / n;
      const int L = (int)std::max<long long>(1, std::min<long long>(nrows, (16LL * kLineThreads) / n));
      int blocks = (int)((nrows + L - 1) / L);
      size_t smem = (size_t)L * n * sizeof(double2);
      if (K.fft_ctas > 1) {  // one 1D line held by a cluster pair
        blocks = K.fft_ctas;
        smem = (size_t)(n / K.fft_ctas) * sizeof(double2);
      }
      if (fwd) K.row_fft_f<<<blocks, kLineThreads, smem, st>>>(G, L, sc);
      else K.row_fft_b<<<blocks, kLineThreads, smem, st>>>(G, L, sc);
    } else {
      if (fwd) K.axis_fft_f<<<g->ax_blocks[ax], K.row_threads, g->ax_smem[ax], st>>>(G, ax, g->ax_C[ax], sc);
      else K.axis_fft_b<<<g->ax_blocks[ax], K.row_threads, g->ax_smem[ax], st>>>(G, ax, g->ax_C[ax], sc);
    }
  }
}

int qsf_fourier(qsf_grid* g, int to_rep) {
  if (!g || (to_rep != QSF_REP_X && to_rep != QSF_REP_P)) return fail(QSF_EINVAL, "bad argument");
  const GridDev& G = g->G;
  const int D = G.dim;
  const bool fwd = to_rep == QSF_REP_P;
  // the axes a region keeps in momentum space are not transformed; the way back scales by
  // the product of the transformed axes' 1/n (fourier_partial, multigrid.h:660-674)
  int last = -1;
  double partial = 1.0;
  for (int ax = 0; ax < D; ++ax) {
    const bool use = !((G.free_mask >> ax) & 1);
    partial *= use ? 1.0 / (double)G.ax[ax].n : 1.0;
    if (use && last < 0) last = ax;
  }
  if (last < 0) return QSF_OK;
  const double back = G.free_mask ? partial : G.inv_m;
  for (int ax = D - 1; ax >= 0; --ax) {
    if ((G.free_mask >> ax) & 1) continue;
    const double post = ax == last && !fwd ? back : 1.0;
    if (g->ks) {
      axis_fft(g, G, ax, fwd, post);
    } else if (int rc = bs_axis(g, g->G.psi, ax, fwd, post)) {
      return rc;
    }
  }
  QSF_CU(cudaGetLastError());
  return QSF_OK;
}

int qsf_region_transfer(qsf_grid* dst, const qsf_grid* src, int axis, int group) {
  if (!dst || !src || dst == src) return fail(QSF_EINVAL, "two distinct grids are needed");
  const GridDev& G = dst->G;
  const GridDev& H = src->G;
  if (!G.multi || !H.multi) return fail(QSF_EINVAL, "region transfers need grids created with multi_region = 1");
  if (axis < 0 || axis >= G.dim) return fail(QSF_EINVAL, "axis out of range");
  if (G.dim != H.dim || G.m != H.m || G.nCAP != H.nCAP) return fail(QSF_EINVAL, "the grids differ in geometry");
  for (int k = 0; k < G.dim; ++k)
    if (G.ax[k].n != H.ax[k].n || G.ax[k].dx != H.ax[k].dx) return fail(QSF_EINVAL, "the grids differ in geometry");
  const int bit = 1 << axis;
  int nfree = 0;
  for (int k = 0; k < G.dim; ++k) nfree += (G.free_mask >> k) & 1;
  if (!(G.free_mask & bit) || H.free_mask != (G.free_mask & ~bit) || group != nfree)
    return fail(QSF_EINVAL, "src must be dst's region with `axis` bounded, and group dst's number of free axes");
  if (!dst->mg_slice)
    if (int rc = dev_alloc(dst->mg_slice, (size_t)G.m)) return rc;
  if (!dst->mg_event) QSF_CU(cudaEventCreateWithFlags(&dst->mg_event, cudaEventDisableTiming));
  qsf_grid* s = const_cast<qsf_grid*>(src);
  if (!s->mg_event) QSF_CU(cudaEventCreateWithFlags(&s->mg_event, cudaEventDisableTiming));
  // dst's stream after src's work; src's after the transfer has read it
  QSF_CU(cudaEventRecord(s->mg_event, s->stream));
  QSF_CU(cudaStreamWaitEvent(dst->stream, s->mg_event, 0));
  // boxes of nCAP planes along the sliding axis (multigrid.h:184, 296-317): n / nCAP of them
  const long long slide_lim = G.dim == 3 ? (G.ax[0].n / G.nCAP) * G.nCAP : 0;
  if (int rc = ensure_mtab(dst)) return rc;
  k_mg_slice<<<grid_blocks(G.m), 256, 0, dst->stream>>>(G, H.psi, dst->mg_slice, axis, group, slide_lim, dst->mtab,
                                                        dst->nmax);
  GridDev Gs = G;
  Gs.psi = dst->mg_slice;
  if (dst->ks) axis_fft(dst, Gs, axis, true, 1.0);
  else if (int rc = bs_axis(dst, dst->mg_slice, axis, true, 1.0)) return rc;
  k_add_slice<<<grid_blocks(G.m), 256, 0, dst->stream>>>(G.psi, dst->mg_slice, G.m);
  QSF_CU(cudaGetLastError());
  QSF_CU(cudaEventRecord(dst->mg_event, dst->stream));
  QSF_CU(cudaStreamWaitEvent(s->stream, dst->mg_event, 0));
  return QSF_OK;
}

static int evolve_impl(qsf_grid* g, int mode, int rep, double delta, const double* c3, CoupDev cd);

int qsf_evolve(qsf_grid* g, int mode, int rep, double delta, const double* c3) {
  if (!g || (mode != 1 && mode != 2) || (rep != 1 && rep != 2)) return fail(QSF_EINVAL, "bad argument");
  return evolve_impl(g, mode, rep, delta, c3, CoupDev{nullptr, nullptr, 0, 0});
}

// evolve<mode, rep>(delta) with the coupling values from c3 (host) or, when cd.c is
// set, from the device rows of a step program
// the X factor table of evolve<mode, X>(delta) without X-space coupling, per point:
// evaluated once and reused while (mode, delta) stay the same
static int ensure_xtab(qsf_grid* g, int mode, double delta) {
  if (g->etab && g->etab_mode == mode && g->etab_delta == delta) return QSF_OK;
  if (!g->etab)
    if (int rc = dev_alloc(g->etab, (size_t)g->G.m)) return rc;
  k_evolve_xtab<<<grid_blocks(g->G.m), 256, 0, g->stream>>>(g->G, mode, delta, g->etab);
  g->etab_mode = mode;
  g->etab_delta = delta;
  QSF_CU(cudaGetLastError());
  return QSF_OK;
}

// the potential per point for E_pot averages (built on first use)
static int ensure_vtab(qsf_grid* g) {
  if (g->vtab) return QSF_OK;
  if (int rc = dev_alloc(g->vtab, (size_t)g->G.m)) return rc;
  k_build_vtab<<<grid_blocks(g->G.m), 256, 0, g->stream>>>(g->G, g->vtab);
  QSF_CU(cudaGetLastError());
  return QSF_OK;
}

static int evolve_impl(qsf_grid* g, int mode, int rep, double delta, const double* c3, CoupDev cd) {
  const double c0 = c3 ? c3[0] : 0.0, c1 = c3 ? c3[1] : 0.0, c2 = c3 ? c3[2] : 0.0;
  const GridDev& G = g->G;
  if (rep == QSF_REP_X && !(G.gauge == QSF_GAUGE_LENGTH && G.n_fields)) {
    if (int rc = ensure_xtab(g, mode, delta)) return rc;
    k_apply_xtab<<<grid_blocks(G.m), 256, 0, g->stream>>>(G.psi, g->etab, G.m);
  } else if (rep == QSF_REP_P) {
    if (!g->eptab)
      if (int rc = dev_alloc(g->eptab, (size_t)3 * g->nmax)) return rc;
    k_evolve_ptab<<<(G.dim * g->nmax + 255) / 256, 256, 0, g->stream>>>(G, mode, delta, c0, c1, c2, g->nmax,
                                                                        g->eptab, cd);
    k_apply_ptab<<<grid_blocks(G.m), 256, 0, g->stream>>>(G, g->eptab, g->nmax);
  } else {
    k_evolve<<<grid_blocks(G.m), 256, 0, g->stream>>>(G, mode, rep, delta, c0, c1, c2, cd);
  }
  QSF_CU(cudaGetLastError());
  return QSF_OK;
}

// the per-block partials of average<rep, op> into g->partials; returns the block count
static int launch_average(qsf_grid* g, int rep, int op, int* nblocks) {
  const int nb = std::min(256, grid_blocks(g->G.m));
  if (rep == QSF_REP_X && op == QSF_OP_POTENTIAL) {
    if (int rc = ensure_vtab(g)) return rc;
    k_average_tab<<<nb, 256, 0, g->stream>>>(g->G, g->vtab, g->partials);
  } else {
    k_average<<<nb, 256, 0, g->stream>>>(g->G, rep, op, g->partials);
  }
  *nblocks = nb;
  return QSF_OK;
}

int qsf_average(qsf_grid* g, int rep, int op, double* out) {
  if (!g || !out || (rep != 1 && rep != 2) || op < 0 || op > 2) return fail(QSF_EINVAL, "bad argument");
  int nb = 0;
  if (int rc = launch_average(g, rep, op, &nb)) return rc;
  const double vol = rep == QSF_REP_X ? g->G.dV : g->G.dVm;
  k_reduce_partials<<<1, 256, 0, g->stream>>>(g->partials, nb, vol, g->energy + 1);
  QSF_CU(cudaGetLastError());
  QSF_CU(cudaMemcpyAsync(out, g->energy + 1, sizeof(double), cudaMemcpyDeviceToHost, g->stream));
  QSF_CU(cudaStreamSynchronize(g->stream));
  return QSF_OK;
}

int qsf_average_log(qsf_grid* g, int rep, int op, int64_t slot) {
  if (!g || (rep != 1 && rep != 2) || op < 0 || op > 2 || slot < 0) return fail(QSF_EINVAL, "bad argument");
  if ((size_t)slot >= g->obs_cap) {
    // grow (keeping what is logged); the copy orders after the stream's earlier work
    const size_t cap = std::max<size_t>((size_t)slot + 1, std::max<size_t>(g->obs_cap * 2, 1024));
    double* nb = nullptr;
    if (int rc = dev_alloc(nb, cap)) return rc;
    QSF_CU(cudaMemsetAsync(nb, 0, cap * sizeof(double), g->stream));
    if (g->obs_log) {
      QSF_CU(cudaMemcpyAsync(nb, g->obs_log, g->obs_cap * sizeof(double), cudaMemcpyDeviceToDevice, g->stream));
      QSF_CU(cudaStreamSynchronize(g->stream));
      cudaFree(g->obs_log);
    }
    g->obs_log = nb;
    g->obs_cap = cap;
  }
  int nbk = 0;
  if (int rc = launch_average(g, rep, op, &nbk)) return rc;
  const double vol = rep == QSF_REP_X ? g->G.dV : g->G.dVm;
  k_reduce_partials<<<1, 256, 0, g->stream>>>(g->partials, nbk, vol, g->obs_log + slot);
  QSF_CU(cudaGetLastError());
  return QSF_OK;
}

int qsf_read_log(qsf_grid* g, double* out, int64_t n) {
  if (!g || !out || n < 0 || (size_t)n > g->obs_cap) return fail(QSF_EINVAL, "bad argument");
  if (n == 0) return QSF_OK;
  QSF_CU(cudaMemcpyAsync(out, g->obs_log, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, g->stream));
  QSF_CU(cudaStreamSynchronize(g->stream));
  return QSF_OK;
}

int qsf_normalize(qsf_grid* g, double* norm_out) {
  double nrm = 0.0;
  if (int rc = qsf_average(g, QSF_REP_X, QSF_OP_IDENTITY, &nrm)) return rc;
  if (!(nrm > 0.0)) return fail(QSF_ENUMERIC, "norm is not positive");
  const double s = std::sqrt(1.0 / nrm);
  QSF_CU(cudaMemcpyAsync(g->scale + 1, &s, sizeof(double), cudaMemcpyHostToDevice, g->stream));
  k_scale<<<grid_blocks(g->G.m), 256, 0, g->stream>>>(g->G.psi, g->G.m, g->scale + 1);
  QSF_CU(cudaGetLastError());
  QSF_CU(cudaStreamSynchronize(g->stream));
  if (norm_out) *norm_out = nrm;
  return QSF_OK;
}

int qsf_flux(qsf_grid* g, const double* A3, int nb, const int* types, int64_t box, double* out) {
  if (!g || !out || nb < 0 || nb > QSF_MAX_BORDERS || (nb && !types)) return fail(QSF_EINVAL, "bad argument");
  if (nb == 0) return QSF_OK;
  if (int rc = ensure_flux(g, nb, types, box)) return rc;
  std::vector<double> res((size_t)nb, 0.0);
  if (g->nfterms > 0) {
    k_gather<<<std::max(1, std::min(1024, (g->nsnap + 255) / 256)), 256, 0, g->stream>>>(g->G.psi, g->snap_idx,
                                                                                         g->nsnap, g->snap);
    k_flux<<<g->nfblk, 256, 0, g->stream>>>(g->G, g->fpts, g->fterms, g->nfterms, g->snap, A3 ? A3[0] : 0.0,
                                            A3 ? A3[1] : 0.0, A3 ? A3[2] : 0.0, A3 ? 1 : 0, nb, g->fpartials,
                                            CoupDev{nullptr, nullptr, 0, 0});
    QSF_CU(cudaGetLastError());
    std::vector<double> part((size_t)g->nfblk * kMaxFluxBorders);
    QSF_CU(cudaMemcpyAsync(part.data(), g->fpartials, part.size() * sizeof(double), cudaMemcpyDeviceToHost,
                           g->stream));
    QSF_CU(cudaStreamSynchronize(g->stream));
    for (int k = 0; k < g->nfblk; ++k)
      for (int b = 0; b < nb; ++b) res[(size_t)b] += part[(size_t)k * kMaxFluxBorders + b];
  }
  for (int b = 0; b < nb; ++b) out[b] = res[(size_t)b] * g->G.dV / g->G.ax[0].dx;
  return QSF_OK;
}

int qsf_mask_region(qsf_grid* g, const int* b3) {
  if (!g || !b3) return fail(QSF_EINVAL, "null argument");
  if (g->G.nCAP <= 0) return QSF_OK;  // no absorber: the mask is 1 everywhere
  if (int rc = ensure_mtab(g)) return rc;
  k_mask<<<grid_blocks(g->G.m), 256, 0, g->stream>>>(g->G, b3[0], g->G.dim > 1 ? b3[1] : 1, g->G.dim > 2 ? b3[2] : 1,
                                                     g->mtab, g->nmax);
  QSF_CU(cudaGetLastError());
  return QSF_OK;
}

int qsf_add_gaussian(qsf_grid* g, double at, double delta) {
  if (!g || !(delta > 0)) return fail(QSF_EINVAL, "bad argument");
  k_add_gaussian<<<grid_blocks(g->G.m), 256, 0, g->stream>>>(g->G, at, delta);
  QSF_CU(cudaGetLastError());
  return QSF_OK;
}

static int generic_step(qsf_grid* g, const qsf_step_desc* d, double* rows, int64_t* steps_done);

int qsf_step(qsf_grid* g, const qsf_step_desc* d, double* rows, int64_t* steps_done) {
  if (!g || !d) return fail(QSF_EINVAL, "null argument");
  if (steps_done) *steps_done = 0;
  if (d->nsteps == 0) return QSF_OK;
  if (!g->ks) return generic_step(g, d, rows, steps_done);
  StepDev S{};
  int ncol = 0, rc;
  if ((rc = prepare_step(g, d, &S, &ncol))) return rc;
  if (d->kernel_ms) {
    // one event pair per launch of the whole call (at most 8 per step), read at the end,
    // so the profiled call has no host synchronisation between its steps
    Prof P;
    P.ms = d->kernel_ms;
    P.count = d->kernel_launches;
    rc = P.init(g->stream, (int)std::min<int64_t>(S.nsteps * 8 + 8, 1 << 20));
    for (int64_t k = 0; k < S.nsteps && rc == QSF_OK; ++k) rc = launch_step(g, S, &P);
    if (rc == QSF_OK) rc = P.flush();
    P.release();
    if (rc) return rc;
  } else if (S.nsteps < 4) {
    for (int64_t k = 0; k < S.nsteps; ++k)
      if ((rc = launch_step(g, S))) return rc;
  } else {
    // one graph holds kGraphSteps steps (the kernels read the step index from the
    // device, so every copy is the same), the remainder runs as single steps.  In a
    // fused call only the first step's opening row pass works, so it runs once, before
    // the graphs, which leave it out.  The executable graph stays with the grid and
    // is replayed by later calls of the same launch shape (no capture per call).
    const bool skip_open = S.fused != 0 && !(S.obs & QSF_OBS_EKIN);
    int64_t first = 0;
    if (skip_open) {
      if ((rc = launch_step(g, S))) return rc;
      first = 1;
    }
    const int64_t rest = S.nsteps - first;
    constexpr int64_t kGraphSteps = 16;
    const int64_t per = std::max<int64_t>(1, std::min<int64_t>(kGraphSteps, rest));
    if (rest > 0) {
      cudaGraphExec_t exec = nullptr;
      FinOverlap ov;
      const bool overlap = fin_overlap_ok(S);
      if (overlap && (rc = ensure_fin_stream(g, &ov))) return rc;
      const int ekin = (S.obs & QSF_OBS_EKIN) ? 1 : 0, nfblk = S.nfterms > 0 ? g->nfblk : 1;
      for (const qsf_grid::StepGraph& sg : g->step_graphs)
        if (sg.per == per && sg.skip_open == (int)skip_open && sg.overlap == (int)overlap && sg.ekin == ekin &&
            sg.nfblk == nfblk)
          exec = sg.exec;
      if (!exec) {
        if ((rc = capture_graph(
                 g->stream,
                 [&]() {
                   for (int64_t k = 0; k < per; ++k)
                     if (int r = launch_step(g, S, nullptr, !skip_open, overlap ? &ov : nullptr)) return r;
                   if (ov.pending) QSF_CU(cudaStreamWaitEvent(g->stream, ov.done, 0));  // join
                   return QSF_OK;
                 },
                 &exec)))
          return rc;
        g->step_graphs.push_back({per, (int)skip_open, (int)overlap, ekin, nfblk, exec});
      }
      for (int64_t k = 0; k + per <= rest; k += per) {
        const cudaError_t ce = cudaGraphLaunch(exec, g->stream);
        if (ce != cudaSuccess) return fail(QSF_ECUDA, std::string("graph launch: ") + cudaGetErrorString(ce));
      }
      for (int64_t k = rest - rest % per; k < rest; ++k)
        if ((rc = launch_step(g, S, nullptr, !skip_open))) return rc;
    }
  }
  return finish_step(g, d->normalize, d->nsteps, ncol, rows, steps_done);
}

// End of one member-operation step: the flux partials summed per border in block order
// (the order qsf_flux sums them in) into row *step, the NaN / non-positive norm flag,
// the Normalize factor, and the step counter advanced, all on the device so that the
// steps of a program need no host synchronisation and replay from a graph.
__global__ void k_generic_row(const double* __restrict__ fpart, int nfblk, int nb, double dV, double dx,
                              double* __restrict__ rows, long long* __restrict__ step, int ncol,
                              long long* __restrict__ flag, double* __restrict__ scale, int normalize) {
  double* row = rows + (*step) * ncol;
  if ((int)threadIdx.x < nb) {
    double v = 0.0;
    for (int k = 0; k < nfblk; ++k) v += fpart[k * kMaxFluxBorders + threadIdx.x];
    row[3 + threadIdx.x] = v * dV / dx;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const double norm = row[0];
    if (!(norm > 0.0) || isnan(row[1]) || isnan(row[2])) *flag = 1;
    *scale = normalize && norm > 0.0 ? sqrt(1.0 / norm) : 1.0;
    *step += 1;
  }
}

// The Strang steps of a grid without fused kernels, through the member operations
// (the reference's own sequence: evolve<X>(dt/2), fourier<P>, evolve<P>(dt),
// fourier<X>, evolve<X>(dt/2), propagator.h:311-346), with the same descriptor, rows,
// Normalize, E_kin interval and convergence rule as the fused path.  Observables
// reduce into device rows; the host waits once per call (and once per step that runs
// the imaginary-time convergence test).
static int generic_check(const qsf_grid* g, const qsf_step_desc* d) {
  if (d->mode != QSF_MODE_IM && d->mode != QSF_MODE_RE) return fail(QSF_EINVAL, "mode must be IM or RE");
  if (d->nsteps < 1) return fail(QSF_EINVAL, "nsteps < 1");
  if (d->nborders < 0 || d->nborders > QSF_MAX_BORDERS) return fail(QSF_EINVAL, "too many borders");
  if (d->substeps < 0 || d->substeps > 64) return fail(QSF_EINVAL, "substeps must be in [0, 64]");
  if (d->ekin_interval < 0) return fail(QSF_EINVAL, "ekin_interval must be >= 0");
  if (g->G.free_mask)
    return fail(QSF_EINVAL, "a region with free axes keeps them in momentum space: step it with the member operations");
  return QSF_OK;
}

static int generic_ncol(const qsf_step_desc* d) {
  return 3 + ((d->obs & QSF_OBS_FLUX) && d->nborders > 0 ? d->nborders : 0);
}

}  // extern "C"

bool qsf::grid_fused(const qsf_grid* g) { return g->ks != nullptr; }

// psi = 0, ordered on the grid's stream (a memset on another stream would not be
// ordered before the grid's later work)
int qsf::grid_clear(qsf_grid* g) {
  QSF_CU(cudaMemsetAsync(g->G.psi, 0, (size_t)g->G.m * sizeof(double2), g->stream));
  return QSF_OK;
}

// the launch-shape key of a step program: what its captured kernels bake in
static std::vector<long long> generic_key(const qsf_grid* g, const qsf_step_desc* d) {
  long long dtb;
  std::memcpy(&dtb, &d->dt, sizeof(dtb));
  return {d->mode, dtb, std::max(1, d->substeps), (long long)d->obs, generic_ncol(d), d->normalize,
          d->coupling != nullptr, (long long)(uintptr_t)g->rows_dev, (long long)(uintptr_t)g->coup_dev,
          (long long)(uintptr_t)g->snap, (long long)(uintptr_t)g->fpts, (long long)(uintptr_t)g->fterms, g->nfterms,
          g->nsnap, g->nfblk, (long long)(uintptr_t)g->etab, (long long)(uintptr_t)g->eptab,
          (long long)(uintptr_t)g->vtab};
}

int qsf::generic_begin(qsf_grid* g, const qsf_step_desc* d) {
  int rc;
  if ((rc = generic_check(g, d))) return rc;
  const int ncol = generic_ncol(d);
  const int K = std::max(1, d->substeps), cs = g->G.gauge == QSF_GAUGE_LENGTH ? 6 : 3;
  if (ncol > 3 && (rc = ensure_flux(g, d->nborders, d->border_types, d->box_size))) return rc;
  if ((rc = dev_reserve(g->rows_dev, g->rows_cap, (size_t)d->nsteps * ncol))) return rc;
  if (d->coupling) {
    const size_t nc = (size_t)d->nsteps * K * cs;
    if ((rc = dev_reserve(g->coup_dev, g->coup_cap, nc))) return rc;
    QSF_CU(cudaMemcpyAsync(g->coup_dev, d->coupling, nc * sizeof(double), cudaMemcpyHostToDevice, g->stream));
  }
  QSF_CU(cudaMemsetAsync(g->rows_dev, 0, (size_t)d->nsteps * ncol * sizeof(double), g->stream));
  QSF_CU(cudaMemsetAsync(g->ctl, 0, 8 * sizeof(long long), g->stream));  // [0] step, [4] NaN flag
  g->gen_primed = false;
  return QSF_OK;
}

// one step of the program d at the device step index ctl[0] (its sub-steps, then the
// observables row, then ctl[0] + 1), queued on the grid's stream; E_kin when ek.  The
// launches do not depend on the step index, so a run of them replays from a graph.
static int generic_one(qsf_grid* g, const qsf_step_desc* d, bool ek) {
  const GridDev& G = g->G;
  const bool lg = G.gauge == QSF_GAUGE_LENGTH;
  const int K = std::max(1, d->substeps), cs = lg ? 6 : 3;
  const double dts = d->dt / K;
  const int ncol = generic_ncol(d), nb = ncol - 3;
  const CoupDev none{nullptr, nullptr, 0, 0};
  const bool has_c = d->coupling != nullptr;
  const long long sstride = (long long)K * cs;
  int rc;
  for (int k = 0; k < K; ++k) {
    // sub-step k of the step: E at its opening / closing X half (length gauge), A at
    // its P sub-step (velocity gauge)
    const CoupDev c1 = has_c ? CoupDev{g->coup_dev, g->ctl, sstride, k * cs} : none;
    const CoupDev c2 = has_c && lg ? CoupDev{g->coup_dev, g->ctl, sstride, k * cs + 3} : none;
    if ((rc = evolve_impl(g, d->mode, QSF_REP_X, 0.5 * dts, nullptr, lg ? c1 : none)) ||
        (rc = qsf_fourier(g, QSF_REP_P)) || (rc = evolve_impl(g, d->mode, QSF_REP_P, dts, nullptr, lg ? none : c1)) ||
        (rc = qsf_fourier(g, QSF_REP_X)) || (rc = evolve_impl(g, d->mode, QSF_REP_X, 0.5 * dts, nullptr, c2)))
      return rc;
  }
  int nbk = 0;
  if ((rc = launch_average(g, QSF_REP_X, QSF_OP_IDENTITY, &nbk))) return rc;
  k_reduce_row<<<1, 256, 0, g->stream>>>(g->partials, nbk, G.dV, g->rows_dev, g->ctl, ncol, 0);
  if (d->obs & QSF_OBS_EPOT) {
    if ((rc = launch_average(g, QSF_REP_X, QSF_OP_POTENTIAL, &nbk))) return rc;
    k_reduce_row<<<1, 256, 0, g->stream>>>(g->partials, nbk, G.dV, g->rows_dev, g->ctl, ncol, 1);
  }
  if (ek) {
    if ((rc = qsf_fourier(g, QSF_REP_P)) || (rc = launch_average(g, QSF_REP_P, QSF_OP_KINETIC, &nbk))) return rc;
    k_reduce_row<<<1, 256, 0, g->stream>>>(g->partials, nbk, G.dVm, g->rows_dev, g->ctl, ncol, 2);
    if ((rc = qsf_fourier(g, QSF_REP_X))) return rc;
  }
  if (nb && g->nfterms > 0) {
    // fluxes of psi_n with the A of the step's last P sub-step (velocity gauge)
    const bool useA = !lg && has_c && G.n_fields;
    const CoupDev ca = useA ? CoupDev{g->coup_dev, g->ctl, sstride, (K - 1) * cs} : none;
    k_gather<<<std::max(1, std::min(1024, (g->nsnap + 255) / 256)), 256, 0, g->stream>>>(G.psi, g->snap_idx,
                                                                                         g->nsnap, g->snap);
    k_flux<<<g->nfblk, 256, 0, g->stream>>>(G, g->fpts, g->fterms, g->nfterms, g->snap, 0.0, 0.0, 0.0, useA ? 1 : 0,
                                            nb, g->fpartials, ca);
  }
  k_generic_row<<<1, 32, 0, g->stream>>>(g->fpartials, g->nfterms > 0 ? g->nfblk : 0, nb, G.dV, G.ax[0].dx,
                                         g->rows_dev, g->ctl, ncol, g->ctl + 4, g->scale + 1, d->normalize);
  if (d->normalize) k_scale<<<grid_blocks(G.m), 256, 0, g->stream>>>(G.psi, G.m, g->scale + 1);
  QSF_CU(cudaGetLastError());
  return QSF_OK;
}

static bool generic_ekin_at(const qsf_step_desc* d, int64_t s, int64_t stop_after) {
  const int every = d->ekin_interval > 1 ? d->ekin_interval : 1;
  return (d->obs & QSF_OBS_EKIN) && ((s + 1) % every == 0 || s + 1 == d->nsteps || s == stop_after);
}

// steps per captured graph of a member-operation step program
#ifndef QSF_GEN_GRAPH_STEPS
#define QSF_GEN_GRAPH_STEPS 16
#endif

// The member operations' tables a step program uses, made before any capture (a
// capture may not allocate): the X factor for (mode, dt/2K) where no coupling acts in X,
// the P factor table, the potential table for E_pot.
static int generic_prime(qsf_grid* g, const qsf_step_desc* d) {
  const GridDev& G = g->G;
  const int K = std::max(1, d->substeps);
  int rc;
  if (!(G.gauge == QSF_GAUGE_LENGTH && G.n_fields) && (rc = ensure_xtab(g, d->mode, 0.5 * (d->dt / K)))) return rc;
  if (!g->eptab && (rc = dev_alloc(g->eptab, (size_t)3 * g->nmax))) return rc;
  if ((d->obs & QSF_OBS_EPOT) && (rc = ensure_vtab(g))) return rc;
  g->gen_primed = true;
  return QSF_OK;
}

// Steps [first, first + count) of the program (the device step index must be `first`):
// without E_kin, runs of kGenGraphSteps steps replay one captured graph per grid (its
// launches bake in the program's shape, so it is recaptured when that changes); the
// remainder runs as plain launches.
int qsf::generic_enqueue(qsf_grid* g, const qsf_step_desc* d, int64_t first, int64_t count) {
  constexpr int kGenGraphSteps = QSF_GEN_GRAPH_STEPS;
  if (first < 0 || count < 0 || first + count > d->nsteps) return fail(QSF_EINVAL, "steps outside the program");
  int rc;
  int64_t s = first;
  const int64_t end = first + count;
  const bool graphs = !(d->obs & QSF_OBS_EKIN);
  if (!g->gen_primed && (rc = generic_prime(g, d))) return rc;
  if (graphs && end - s >= kGenGraphSteps) {
    const std::vector<long long> key = generic_key(g, d);
    if (!g->gen_exec || g->gen_key != key) {
      if (g->gen_exec) cudaGraphExecDestroy(g->gen_exec);
      g->gen_exec = nullptr;
      if ((rc = capture_graph(
               g->stream,
               [&]() {
                 for (int k = 0; k < kGenGraphSteps; ++k)
                   if (int r = generic_one(g, d, false)) return r;
                 return QSF_OK;
               },
               &g->gen_exec)))
        return rc;
      g->gen_key = key;
      g->gen_steps = kGenGraphSteps;
    }
    for (; end - s >= g->gen_steps; s += g->gen_steps) {
      const cudaError_t ce = cudaGraphLaunch(g->gen_exec, g->stream);
      if (ce != cudaSuccess) return fail(QSF_ECUDA, std::string("graph launch: ") + cudaGetErrorString(ce));
    }
  }
  for (; s < end; ++s)
    if ((rc = generic_one(g, d, generic_ekin_at(d, s, d->nsteps)))) return rc;
  return QSF_OK;
}

int qsf::generic_wait(qsf_grid* g, bool* bad) {
  long long flag = 0;
  QSF_CU(cudaMemcpyAsync(&flag, g->ctl + 4, sizeof(flag), cudaMemcpyDeviceToHost, g->stream));
  QSF_CU(cudaStreamSynchronize(g->stream));
  *bad = flag != 0;
  return QSF_OK;
}

int qsf::generic_rows(qsf_grid* g, const qsf_step_desc* d, double* rows, int64_t nsteps) {
  if (nsteps > d->nsteps) return fail(QSF_EINVAL, "more rows than steps");
  if (rows && nsteps > 0)
    QSF_CU(cudaMemcpyAsync(rows, g->rows_dev, (size_t)nsteps * generic_ncol(d) * sizeof(double),
                           cudaMemcpyDeviceToHost, g->stream));
  QSF_CU(cudaStreamSynchronize(g->stream));
  return QSF_OK;
}

extern "C" {

static int generic_step(qsf_grid* g, const qsf_step_desc* d, double* rows, int64_t* steps_done) {
  int rc;
  if ((rc = qsf::generic_begin(g, d))) return rc;
  const bool conv = d->mode == QSF_MODE_IM && d->state_accuracy > 0.0;
  const int ncol = generic_ncol(d);
  double last_e = d->last_energy;
  int64_t stop_after = d->nsteps;  // set by the convergence rule
  int64_t s = 0;
  if (!conv) {
    if ((rc = qsf::generic_enqueue(g, d, 0, d->nsteps))) return rc;
    s = d->nsteps;
  }
  for (; conv && s < d->nsteps && s <= stop_after; ++s) {
    const bool ek = generic_ekin_at(d, s, stop_after);
    if ((rc = generic_one(g, d, ek))) return rc;
    if (ek || !(d->obs & QSF_OBS_EKIN)) {
      double r[3];
      QSF_CU(cudaMemcpyAsync(r, g->rows_dev + (size_t)s * ncol, sizeof(r), cudaMemcpyDeviceToHost, g->stream));
      QSF_CU(cudaStreamSynchronize(g->stream));
      const double se = (d->energy_after_normalize & 1) ? 1.0 / r[0] : 1.0;
      const double sk = (d->energy_after_normalize & 2) ? 1.0 / r[0] : 1.0;
      const double e = r[1] * se + r[2] * sk;
      if (stop_after == d->nsteps && std::fabs(e - last_e) <= d->state_accuracy) stop_after = s + 1;
      last_e = e;
    }
  }
  bool bad = false;
  if ((rc = qsf::generic_wait(g, &bad)) || (rc = qsf::generic_rows(g, d, rows, d->nsteps))) return rc;
  if (steps_done) *steps_done = s;
  if (bad) return fail(QSF_ENUMERIC, "non-positive norm or NaN in a step's reductions");
  return QSF_OK;
}

int qsf_batch_create(void* stream, qsf_batch** out) {
  if (!out) return fail(QSF_EINVAL, "null argument");
  if (int rc = init_kernel_table()) return rc;
  qsf_batch* b = new qsf_batch();
  if (stream) {
    b->stream = (cudaStream_t)stream;
  } else {
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) {
      delete b;
      return fail(QSF_ECUDA, "cudaStreamCreate failed");
    }
    b->own_stream = true;
  }
  *out = b;
  return QSF_OK;
}

int qsf_batch_destroy(qsf_batch* b) {
  if (!b) return QSF_OK;
  cudaStreamSynchronize(b->stream);
  for (auto& kv : b->members) {  // the grids outlive the batch
    kv.second.g->batch = nullptr;
    kv.second.g->batch_slot = -1;
  }
  free_groups(b);
  if (b->dG_all) cudaFree(b->dG_all);
  if (b->dS_all) cudaFree(b->dS_all);
  if (b->ctl_host) cudaFreeHost(b->ctl_host);
  for (cudaStream_t s2 : b->gstreams) cudaStreamDestroy(s2);
  for (cudaEvent_t e2 : b->gjoin) cudaEventDestroy(e2);
  if (b->gfork) cudaEventDestroy(b->gfork);
  if (b->own_stream) cudaStreamDestroy(b->stream);
  delete b;
  return QSF_OK;
}

int qsf_batch_add(qsf_batch* b, qsf_grid* g, const qsf_step_desc* d, int64_t* slot) {
  if (!b) return fail(QSF_EINVAL, "null argument");
  QSF_CU(cudaStreamSynchronize(b->stream));
  return qsf::batch_add_nowait(b, g, d, slot);
}

}  // extern "C"

int qsf::batch_add_nowait(qsf_batch* b, qsf_grid* g, const qsf_step_desc* d, int64_t* slot) {
  if (!b || !g || !d || !slot) return fail(QSF_EINVAL, "null argument");
  if (d->substeps > 1) return fail(QSF_EINVAL, "batched solves run plain Strang steps (substeps <= 1)");
  if (!g->ks) return fail(QSF_EINVAL, "batched grids need a line length with fused kernels in this build");
  if (g->batch) return fail(QSF_ESTATE, "grid is already in a batch");
  BatchMember mb;
  mb.g = g;
  qsf_step_desc dd = *d;
  dd.kernel_ms = nullptr;
  dd.kernel_launches = nullptr;
  int rc;
  if ((rc = prepare_step(g, &dd, &mb.S, &mb.ncol))) return rc;
  QSF_CU(cudaStreamSynchronize(g->stream));
  mb.nsteps = d->nsteps;
  mb.normalize = d->normalize;
  *slot = b->next_slot++;
  b->members[*slot] = mb;
  b->dirty = true;
  g->batch = b;
  g->batch_slot = *slot;
  return QSF_OK;
}

extern "C" {

int qsf_batch_remove(qsf_batch* b, int64_t slot) {
  if (!b) return fail(QSF_EINVAL, "null argument");
  auto it = b->members.find(slot);
  if (it == b->members.end()) return fail(QSF_EINVAL, "unknown slot");
  BatchMember& mb = it->second;
  if (mb.normalize && !mb.scaled) {
    k_scale<<<grid_blocks(mb.g->G.m), 256, 0, b->stream>>>(mb.g->G.psi, mb.g->G.m, mb.g->scale);
    QSF_CU(cudaGetLastError());
  }
  QSF_CU(cudaStreamSynchronize(b->stream));
  mb.g->batch = nullptr;
  mb.g->batch_slot = -1;
  b->members.erase(it);
  b->dirty = true;
  return QSF_OK;
}

int qsf_batch_run(qsf_batch* b, int64_t steps, int64_t* active) {
  int rc;
  if ((rc = qsf::batch_launch(b, steps))) return rc;
  return qsf::batch_finish(b, active);
}

}  // extern "C"

int qsf::batch_launch(qsf_batch* b, int64_t steps) {
  if (!b || steps < 0) return fail(QSF_EINVAL, "bad argument");
  int rc;
  if (b->dirty && (rc = rebuild_batch(b))) return rc;
  if (b->exec)
    for (int64_t k = 0; k < steps; ++k) {
      const cudaError_t ce = cudaGraphLaunch(b->exec, b->stream);
      if (ce != cudaSuccess) return fail(QSF_ECUDA, std::string("graph launch: ") + cudaGetErrorString(ce));
    }
  return QSF_OK;
}

int qsf::batch_finish(qsf_batch* b, int64_t* active) {
  if (!b) return fail(QSF_EINVAL, "null argument");
  const size_t nm = b->members.size();
  if (nm * 8 > b->ctl_cap) {
    if (b->ctl_host) cudaFreeHost(b->ctl_host);
    b->ctl_cap = std::max<size_t>(nm * 8, 64);
    QSF_CU(cudaMallocHost((void**)&b->ctl_host, b->ctl_cap * sizeof(long long)));
  }
  size_t i = 0;
  for (auto& kv : b->members) {
    QSF_CU(cudaMemcpyAsync(b->ctl_host + i * 8, kv.second.g->ctl, 8 * sizeof(long long), cudaMemcpyDeviceToHost,
                           b->stream));
    ++i;
  }
  QSF_CU(cudaStreamSynchronize(b->stream));
  int64_t act = 0;
  i = 0;
  bool bad = false;
  for (auto& kv : b->members) {
    const long long* c = b->ctl_host + i * 8;
    const bool done = c[0] >= kv.second.nsteps || c[0] > c[1];
    if (!done) ++act;
    if (c[4]) bad = true;
    ++i;
  }
  if (active) *active = act;
  if (bad) return fail(QSF_ENUMERIC, "non-positive norm or NaN in a batch member's reductions");
  return QSF_OK;
}

extern "C" {

int qsf_batch_result(qsf_batch* b, int64_t slot, double* rows, int64_t* steps_done) {
  if (!b) return fail(QSF_EINVAL, "null argument");
  auto it = b->members.find(slot);
  if (it == b->members.end()) return fail(QSF_EINVAL, "unknown slot");
  BatchMember& mb = it->second;
  QSF_CU(cudaStreamSynchronize(b->stream));
  long long ctl_h[8];
  QSF_CU(cudaMemcpy(ctl_h, mb.g->ctl, sizeof(ctl_h), cudaMemcpyDeviceToHost));
  const bool done = ctl_h[0] >= mb.nsteps || ctl_h[0] > ctl_h[1];
  if (done && mb.normalize && !mb.scaled) {
    k_scale<<<grid_blocks(mb.g->G.m), 256, 0, b->stream>>>(mb.g->G.psi, mb.g->G.m, mb.g->scale);
    QSF_CU(cudaGetLastError());
    QSF_CU(cudaStreamSynchronize(b->stream));
    mb.scaled = true;
  }
  if (rows)
    QSF_CU(cudaMemcpy(rows, mb.g->rows_dev, (size_t)mb.nsteps * mb.ncol * sizeof(double), cudaMemcpyDeviceToHost));
  if (steps_done) *steps_done = ctl_h[2];
  if (ctl_h[4] == 2) return fail(QSF_ETIMEDOUT, "a bulk copy into shared memory did not complete in time");
  if (ctl_h[4]) return fail(QSF_ENUMERIC, "non-finite psi, NaN or non-positive norm in this member's reductions");
  return QSF_OK;
}

}  // extern "C"
