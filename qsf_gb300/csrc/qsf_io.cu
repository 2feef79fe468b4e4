// qsf_io.cu -- wavefunction files (.psi) with the reference LocalGrid's layout and
// semantics: save in the X or P representation, complex or as |psi|^2 block sums
// (downscaled), load, evolution backup / restore and orthogonalizeWith
// (include/wf/grid.h:789-1153).  The arithmetic (phase shift, transforms, block sums,
// overlaps) runs on the device; the host only formats and moves bytes.
//
// File layout (grid.h:1025-1035): dim u8 | rep u8 | complex u8 | downscale i64 |
// n[dim] i64 | dx[dim] f64 | bounded[dim] u8 | payload (native little-endian).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "qsf_internal.h"

using namespace qsf;

namespace {

constexpr size_t kHeaderFixed = 11;  // dim, rep, complex (1 byte each) + downscale (8)

size_t header_bytes(int dim) { return kHeaderFixed + (size_t)dim * (8 + 8 + 1); }

int io_blocks(long long m) {
  long long b = (m + 255) / 256;
  return (int)std::min<long long>(std::max<long long>(b, 1), (long long)device_sm_count() * 16);
}

// psi *= (-1)^(i0 + i1 + ...)  (phaseShiftTrick, grid.h:1074-1085)
__global__ void k_phase_shift(GridDev g) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < g.m; p += stride) {
    int idx[kMaxDim];
    unflatten(g, p, idx);
    int s = 0;
    for (int d = 0; d < g.dim; ++d) s += idx[d];
    if (s & 1) g.psi[p] = make_double2(-g.psi[p].x, -g.psi[p].y);
  }
}

// linear index of memory coordinates c[] in psi; with transpose01 the memory holds the
// P array the way the reference's transposed-out transform leaves it (axes 0 and 1
// swapped; all axes have the same length)
__device__ __forceinline__ long long mem_index(const GridDev& g, const long long* c, bool transpose01) {
  long long p = 0;
  for (int d = 0; d < g.dim; ++d) {
    int dd = d;
    if (transpose01 && d < 2) dd = 1 - d;
    p += c[dd] * g.ax[d].stride;
  }
  return p;
}

// Payload of coarse() (grid.h:955-992): output o runs in C order over the coarse grid
// (ceil(n / ds) points per axis, last axis fastest).  Complex: psi at the coarse point
// times `scale`; otherwise the sum of |psi|^2 over the ds^dim block (offsets with the
// last axis fastest, the reference's accumulation order, no contraction) times `scale`.
__global__ void k_coarse(GridDev g, int transpose01, int ds, int cplx, double scale, double* out, long long nout) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  long long nc[kMaxDim];
  for (int d = 0; d < g.dim; ++d) nc[d] = (g.ax[d].n + ds - 1) / ds;
  for (long long o = (long long)blockIdx.x * blockDim.x + threadIdx.x; o < nout; o += stride) {
    long long c[kMaxDim], r = o;
    for (int d = g.dim - 1; d >= 0; --d) {
      c[d] = (r % nc[d]) * ds;
      r /= nc[d];
    }
    if (cplx) {
      const double2 v = g.psi[mem_index(g, c, transpose01)];
      out[2 * o] = scale == 1.0 ? v.x : __dmul_rn(v.x, scale);
      out[2 * o + 1] = scale == 1.0 ? v.y : __dmul_rn(v.y, scale);
      continue;
    }
    double tmp = 0.0;
    long long ofs[kMaxDim] = {0, 0, 0};
    for (;;) {
      long long cc[kMaxDim];
      for (int d = 0; d < g.dim; ++d) cc[d] = c[d] + ofs[d];
      const double2 v = g.psi[mem_index(g, cc, transpose01)];
      tmp = __dadd_rn(tmp, __dadd_rn(__dmul_rn(v.x, v.x), __dmul_rn(v.y, v.y)));
      int d = g.dim - 1;
      for (; d >= 0; --d) {
        if (++ofs[d] < ds) break;
        ofs[d] = 0;
      }
      if (d < 0) break;
    }
    out[o] = scale == 1.0 ? tmp : __dmul_rn(tmp, scale);
  }
}

// per-block sums of conj(t) psi (orthogonalizeWith's scalar product)
__global__ void __launch_bounds__(256) k_overlap(GridDev g, const double2* __restrict__ t, double* partials) {
  __shared__ double red[64];
  double acc[2] = {0.0, 0.0};
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < g.m; p += stride) {
    const double2 a = t[p], b = g.psi[p];
    acc[0] += a.x * b.x + a.y * b.y;
    acc[1] += a.x * b.y - a.y * b.x;
  }
  block_sum<2>(acc, red);
  if (threadIdx.x == 0) {
    partials[2 * blockIdx.x] = acc[0];
    partials[2 * blockIdx.x + 1] = acc[1];
  }
}

// psi -= s t
__global__ void k_sub_scaled(GridDev g, const double2* __restrict__ t, double sr, double si) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < g.m; p += stride) {
    const double2 a = t[p];
    double2 v = g.psi[p];
    v.x -= sr * a.x - si * a.y;
    v.y -= sr * a.y + si * a.x;
    g.psi[p] = v;
  }
}

std::string header_of(const qsf_grid* g, int rep, int cplx, int64_t ds) {
  const GridDev& G = g->G;
  std::string h;
  h.push_back((char)(unsigned char)G.dim);
  h.push_back((char)(unsigned char)rep);
  h.push_back((char)(cplx ? 1 : 0));
  h.append((const char*)&ds, 8);
  for (int d = 0; d < G.dim; ++d) {
    const int64_t n = G.ax[d].n;
    h.append((const char*)&n, 8);
  }
  for (int d = 0; d < G.dim; ++d) {
    const double dx = G.ax[d].dx;
    h.append((const char*)&dx, 8);
  }
  for (int d = 0; d < G.dim; ++d) h.push_back((char)1);  // single region: every axis bounded
  return h;
}

int write_file(const std::string& path, const std::string& head, const void* data, size_t bytes) {
  std::remove(path.c_str());
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) return fail(QSF_EINVAL, "cannot open " + path + " for writing");
  bool ok = std::fwrite(head.data(), 1, head.size(), f) == head.size();
  if (ok && bytes) ok = std::fwrite(data, 1, bytes, f) == bytes;
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) return fail(QSF_EINVAL, "short write to " + path);
  return QSF_OK;
}

int save_impl(qsf_grid* g, const std::string& base, const qsf_dump_format& df, const std::string& ext,
              std::string* path) {
  const GridDev& G = g->G;
  if (df.rep != QSF_REP_X && df.rep != QSF_REP_P) return fail(QSF_EINVAL, "dump format: rep must be X or P");
  if (df.downscale < 1) return fail(QSF_EINVAL, "dump format: downscale < 1");
  for (int d = 0; d < G.dim; ++d)
    if (G.ax[d].n % df.downscale) return fail(QSF_EINVAL, "dump format: downscale must divide every axis length");
  int cplx = df.complex_values ? 1 : 0;
  std::string name = base;
  if (!df.evo_backup) {
    if (df.downscale > 1) {
      cplx = 0;
      name += "_scale" + std::to_string(df.downscale);
    }
    name += df.rep == QSF_REP_X ? "_repX" : "_repP";
  }
  name += ext;
  const bool prep = df.rep == QSF_REP_P;
  const bool t01 = prep && G.dim > 1;
  cudaStream_t st = g->stream;
  int rc;
  if (prep) {  // _save_centered: centre the P representation, transform
    k_phase_shift<<<io_blocks(G.m), 256, 0, st>>>(G);
    QSF_CU(cudaGetLastError());
    if ((rc = qsf_fourier(g, QSF_REP_P))) return rc;
  }
  const bool raw = df.evo_backup || (df.downscale == 1 && cplx && !prep);
  long long nout = 1;
  for (int d = 0; d < G.dim; ++d) nout *= (G.ax[d].n + df.downscale - 1) / df.downscale;
  const size_t per = (raw || cplx) ? 2 : 1;
  std::vector<double> host((size_t)nout * per);
  if (raw && !prep) {
    QSF_CU(cudaMemcpyAsync(host.data(), G.psi, host.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
  } else {
    double scale = 1.0;
    if (prep && !df.evo_backup) {
      const double p_scale = G.dV / std::pow(std::sqrt(2 * M_PI), G.dim);
      scale = cplx ? p_scale : p_scale * p_scale;
    }
    double* dout = nullptr;
    if ((rc = dev_alloc(dout, host.size()))) return rc;
    k_coarse<<<io_blocks(nout), 256, 0, st>>>(G, t01 ? 1 : 0, raw ? 1 : (int)df.downscale, (raw || cplx) ? 1 : 0,
                                              scale, dout, nout);
    cudaError_t ce = cudaGetLastError();
    if (ce == cudaSuccess)
      ce = cudaMemcpyAsync(host.data(), dout, host.size() * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
    cudaFree(dout);
    if (ce != cudaSuccess) return fail(QSF_ECUDA, std::string("save: ") + cudaGetErrorString(ce));
  }
  if (prep) {  // back to X, undo the centring (as the reference does)
    if ((rc = qsf_fourier(g, QSF_REP_X))) return rc;
    k_phase_shift<<<io_blocks(G.m), 256, 0, st>>>(G);
    QSF_CU(cudaGetLastError());
  }
  QSF_CU(cudaStreamSynchronize(st));
  if ((rc = write_file(name, header_of(g, prep ? QSF_REP_P : QSF_REP_X, (raw || cplx) ? 1 : 0, df.downscale),
                       host.data(), host.size() * sizeof(double))))
    return rc;
  if (path) *path = name;
  return QSF_OK;
}

int read_header(FILE* f, const std::string& path, int dim_expected, int* dim, int* cplx, int64_t* n, double* dx,
                size_t* offset) {
  unsigned char fixed[kHeaderFixed];
  if (std::fread(fixed, 1, kHeaderFixed, f) != kHeaderFixed) return fail(QSF_EINVAL, path + ": truncated header");
  *dim = fixed[0];
  *cplx = fixed[2] ? 1 : 0;
  if (*dim != dim_expected)
    return fail(QSF_EINVAL, path + ": dimensionality of the file (" + std::to_string(*dim) +
                                ") differs from the grid's (" + std::to_string(dim_expected) + ")");
  const size_t rest = header_bytes(*dim) - kHeaderFixed;
  std::vector<unsigned char> h(rest);
  if (std::fread(h.data(), 1, rest, f) != rest) return fail(QSF_EINVAL, path + ": truncated header");
  std::memcpy(n, h.data(), 8 * (size_t)*dim);
  std::memcpy(dx, h.data() + 8 * (size_t)*dim, 8 * (size_t)*dim);
  *offset = header_bytes(*dim);
  return QSF_OK;
}

}  // namespace

extern "C" {

int qsf_save(qsf_grid* g, const char* base, const qsf_dump_format* df, const char* ext, char* path_out,
             size_t path_cap) {
  if (!g || !base || !df) return fail(QSF_EINVAL, "qsf_save: null argument");
  std::string path;
  int rc = save_impl(g, base, *df, ext ? ext : ".psi", &path);
  if (rc) return rc;
  if (path_out && path_cap) {
    if (path.size() + 1 > path_cap) return fail(QSF_EINVAL, "qsf_save: path buffer too small");
    std::memcpy(path_out, path.c_str(), path.size() + 1);
  }
  return QSF_OK;
}

int qsf_load(qsf_grid* g, const char* base, const char* ext, int* warnings, double* norm) {
  if (!g || !base) return fail(QSF_EINVAL, "qsf_load: null argument");
  const GridDev& G = g->G;
  const std::string path = std::string(base) + (ext ? ext : ".psi");
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return fail(QSF_EINVAL, "cannot open " + path);
  int dim = 0, cplx = 0;
  int64_t n[3] = {0, 0, 0};
  double dx[3] = {0, 0, 0};
  size_t off = 0;
  int rc = read_header(f, path, G.dim, &dim, &cplx, n, dx, &off);
  if (rc) {
    std::fclose(f);
    return rc;
  }
  int warn = 0;
  for (int d = 0; d < dim; ++d) {
    if (n[d] != G.ax[d].n) warn |= 1;
    if (dx[d] != G.ax[d].dx) warn |= 2;
  }
  if (!cplx) warn |= 4;
  // the reader fills the first m elements (complex) or the first 8 m bytes (doubles)
  // of the current buffer and keeps the rest
  const size_t m = (size_t)G.m;
  std::vector<double> host(2 * m);
  QSF_CU(cudaMemcpyAsync(host.data(), G.psi, 2 * m * sizeof(double), cudaMemcpyDeviceToHost, g->stream));
  QSF_CU(cudaStreamSynchronize(g->stream));
  const size_t want = cplx ? 2 * m : m;
  const size_t got = std::fread(host.data(), sizeof(double), want, f);
  std::fclose(f);
  if (got < want) warn |= 8;
  if (!cplx)  // probability file: every element becomes its modulus (grid.h:856-857)
    for (size_t i = 0; i < m; ++i) {
      host[2 * i] = std::hypot(host[2 * i], host[2 * i + 1]);
      host[2 * i + 1] = 0.0;
    }
  QSF_CU(cudaMemcpyAsync(G.psi, host.data(), 2 * m * sizeof(double), cudaMemcpyHostToDevice, g->stream));
  if (warnings) *warnings = warn;
  double nrm = 0.0;
  if ((rc = qsf_average(g, QSF_REP_X, QSF_OP_IDENTITY, &nrm))) return rc;
  if (norm) *norm = nrm;
  return QSF_OK;
}

int qsf_orthogonalize_with(qsf_grid* g, const char* base, const char* ext, double* overlap2, double* norm) {
  if (!g || !base) return fail(QSF_EINVAL, "qsf_orthogonalize_with: null argument");
  const GridDev& G = g->G;
  const std::string path = std::string(base) + (ext ? ext : ".psi");
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return fail(QSF_EINVAL, "cannot open " + path);
  int dim = 0, cplx = 0;
  int64_t n[3];
  double dx[3];
  size_t off = 0;
  int rc = read_header(f, path, G.dim, &dim, &cplx, n, dx, &off);
  if (rc) {
    std::fclose(f);
    return rc;
  }
  const size_t m = (size_t)G.m;
  std::vector<double> host(2 * m);
  const size_t got = std::fread(host.data(), sizeof(double), 2 * m, f);
  std::fclose(f);
  if (!cplx || got < 2 * m) return fail(QSF_EINVAL, path + ": not a complex wavefunction of this grid's size");
  double2* t = nullptr;
  if ((rc = dev_alloc(t, m))) return rc;
  const int nb = std::min(256, io_blocks(G.m));
  double* part = nullptr;
  if ((rc = dev_alloc(part, 2 * (size_t)nb))) {
    cudaFree(t);
    return rc;
  }
  std::vector<double> ph(2 * (size_t)nb);
  cudaStream_t st = g->stream;
  cudaError_t ce = cudaMemcpyAsync(t, host.data(), 2 * m * sizeof(double), cudaMemcpyHostToDevice, st);
  if (ce == cudaSuccess) {
    k_overlap<<<nb, 256, 0, st>>>(G, t, part);
    ce = cudaGetLastError();
  }
  if (ce == cudaSuccess) ce = cudaMemcpyAsync(ph.data(), part, ph.size() * sizeof(double), cudaMemcpyDeviceToHost, st);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
  double sr = 0.0, si = 0.0;
  for (int b = 0; b < nb; ++b) {
    sr += ph[2 * (size_t)b];
    si += ph[2 * (size_t)b + 1];
  }
  sr *= G.dV;
  si *= G.dV;
  if (ce == cudaSuccess) {
    k_sub_scaled<<<io_blocks(G.m), 256, 0, st>>>(G, t, sr, si);
    ce = cudaGetLastError();
  }
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
  cudaFree(t);
  cudaFree(part);
  if (ce != cudaSuccess) return fail(QSF_ECUDA, std::string("orthogonalize: ") + cudaGetErrorString(ce));
  if (overlap2) {
    overlap2[0] = sr;
    overlap2[1] = si;
  }
  double nrm = 0.0;
  if ((rc = qsf_average(g, QSF_REP_X, QSF_OP_IDENTITY, &nrm))) return rc;
  if (norm) *norm = nrm;
  return QSF_OK;
}

int qsf_backup(qsf_grid* g, int64_t step, const char* ext) {
  if (!g) return fail(QSF_EINVAL, "qsf_backup: null grid");
  FILE* f = std::fopen("backup.info", "wb");
  if (!f) return fail(QSF_EINVAL, "cannot open backup.info for writing");
  const bool ok = std::fwrite(&step, sizeof(step), 1, f) == 1;
  if (std::fclose(f) != 0 || !ok) return fail(QSF_EINVAL, "short write to backup.info");
  qsf_dump_format df{QSF_REP_X, 1, 1, 1};
  return save_impl(g, "backup", df, ext ? ext : ".psi", nullptr);
}

int qsf_restore(qsf_grid* g, const char* ext, int64_t* step) {
  if (!g) return fail(QSF_EINVAL, "qsf_restore: null grid");
  if (step) {
    FILE* f = std::fopen("backup.info", "rb");
    if (!f) return fail(QSF_EINVAL, "cannot open backup.info");
    const bool ok = std::fread(step, sizeof(*step), 1, f) == 1;
    std::fclose(f);
    if (!ok) return fail(QSF_EINVAL, "backup.info is truncated");
  }
  return qsf_load(g, "backup", ext, nullptr, nullptr);
}

int qsf_remove_backups(const char* ext) {
  const std::string path = std::string("backup") + (ext ? ext : ".psi");
  std::remove(path.c_str());
  return QSF_OK;
}

}  // extern "C"
