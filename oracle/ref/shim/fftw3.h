/* FFTW-API stand-in, written for this project so that the reference's unmodified
 * headers compile and run without the FFTW library.  Plans record their arguments;
 * fftw_execute performs the unnormalised N-D DFT with the oracle's FFT (orc_fft_nd in
 * oracle/qsf_oracle.c) and honours FFTW_MPI_TRANSPOSED_OUT / _IN for rank >= 2 on a
 * single process (the first two axes of the P-space array are swapped).
 * Test infrastructure for the oracle harness only. */
#pragma once
#include <cstdlib>
#include <cstring>
#include <cstdint>
#include <cstdio>
#include <vector>
#include "qsf_shim_arena.h"

extern "C" void orc_fft_nd(double* data, int dim, const long* n, int sign);

typedef double fftw_complex[2];
struct fftw_iodim64 { std::ptrdiff_t n, is, os; };

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)
#define FFTW_PATIENT (1U << 5)
#define FFTW_EXHAUSTIVE (1U << 3)
#define FFTW_WISDOM_ONLY (1U << 21)
#define FFTW_MPI_DEFAULT_BLOCK (0)
#define FFTW_MPI_TRANSPOSED_IN (1U << 29)
#define FFTW_MPI_TRANSPOSED_OUT (1U << 30)

struct qsf_shim_plan {
  int rank;
  std::vector<long> n;
  double* data;
  int sign;
  unsigned flags;
  bool guru;
  long howmany;                      // FFTW-MPI "many" plans: trailing contiguous batch
  std::vector<fftw_iodim64> dims;     // guru plans: transformed axes (n, stride in elements)
  std::vector<fftw_iodim64> hdims;    // guru plans: batch axes
};
typedef qsf_shim_plan* fftw_plan;

static inline void* fftw_malloc(size_t n) {
  if (void* a = qsf_shim_arena_alloc(n ? n : 64)) return a;  // shared between ranks
  void* p = nullptr;
  if (posix_memalign(&p, 64, n ? n : 64)) return nullptr;
  return p;
}
static inline void fftw_free(void* p) {
  if (qsf_shim_in_arena(p)) return;  // arena space is never reused
  free(p);
}
static inline void fftw_print_plan(const fftw_plan) {}
static inline void fftw_destroy_plan(fftw_plan p) { delete p; }

/* swap the first two axes of a C-ordered complex array in place (via a copy) */
static inline void qsf_shim_swap01(double* d, long n0, long n1, long rest) {
  std::vector<double> tmp((size_t)(n0 * n1 * rest * 2));
  for (long i = 0; i < n0; ++i)
    for (long j = 0; j < n1; ++j)
      memcpy(&tmp[(size_t)((j * n0 + i) * rest * 2)], &d[(size_t)((i * n1 + j) * rest * 2)],
             sizeof(double) * 2 * (size_t)rest);
  memcpy(d, tmp.data(), tmp.size() * sizeof(double));
}

/* gather the sub-array at `base` with the given axes (C order) into buf, or scatter back */
static inline void qsf_shim_strided(double* base, const std::vector<fftw_iodim64>& d, double* buf, bool gather) {
  const size_t r = d.size();
  std::vector<long> idx(r, 0);
  long total = 1;
  for (auto& x : d) total *= (long)x.n;
  for (long k = 0; k < total; ++k) {
    long off = 0;
    for (size_t a = 0; a < r; ++a) off += idx[a] * (long)d[a].is;
    if (gather) memcpy(buf + 2 * k, base + 2 * off, 2 * sizeof(double));
    else memcpy(base + 2 * off, buf + 2 * k, 2 * sizeof(double));
    for (size_t a = r; a-- > 0;) {
      if (++idx[a] < (long)d[a].n) break;
      idx[a] = 0;
    }
  }
}

static inline void fftw_execute(const fftw_plan p) {
  if (p->guru) {
    /* every combination of the batch axes: gather, transform, scatter (in place) */
    std::vector<long> n;
    long len = 1;
    for (auto& x : p->dims) { n.push_back((long)x.n); len *= (long)x.n; }
    std::vector<double> buf((size_t)(2 * len));
    const size_t hr = p->hdims.size();
    std::vector<long> h(hr, 0);
    long batches = 1;
    for (auto& x : p->hdims) batches *= (long)x.n;
    for (long b = 0; b < batches; ++b) {
      long off = 0;
      for (size_t a = 0; a < hr; ++a) off += h[a] * (long)p->hdims[a].is;
      qsf_shim_strided(p->data + 2 * off, p->dims, buf.data(), true);
      orc_fft_nd(buf.data(), (int)n.size(), n.data(), p->sign);
      qsf_shim_strided(p->data + 2 * off, p->dims, buf.data(), false);
      for (size_t a = hr; a-- > 0;) {
        if (++h[a] < (long)p->hdims[a].n) break;
        h[a] = 0;
      }
    }
    return;
  }
  if (p->howmany > 1) {
    /* n[0] x ... x n[rank-1] x howmany, the batch index contiguous: one transform per batch index */
    std::vector<fftw_iodim64> d;
    long stride = p->howmany;
    for (int a = p->rank; a-- > 0;) {
      d.insert(d.begin(), fftw_iodim64{(std::ptrdiff_t)p->n[(size_t)a], (std::ptrdiff_t)stride, (std::ptrdiff_t)stride});
      stride *= p->n[(size_t)a];
    }
    long len = stride / p->howmany;
    std::vector<double> buf((size_t)(2 * len));
    for (long b = 0; b < p->howmany; ++b) {
      qsf_shim_strided(p->data + 2 * b, d, buf.data(), true);
      orc_fft_nd(buf.data(), p->rank, p->n.data(), p->sign);
      qsf_shim_strided(p->data + 2 * b, d, buf.data(), false);
    }
    return;
  }
  long rest = 1;
  for (int i = 2; i < p->rank; ++i) rest *= p->n[(size_t)i];
  if (p->rank >= 2 && (p->flags & FFTW_MPI_TRANSPOSED_IN)) {
    /* input stored as n1 x n0 x rest: bring back to n0 x n1 x rest */
    qsf_shim_swap01(p->data, p->n[1], p->n[0], rest);
  }
  orc_fft_nd(p->data, p->rank, p->n.data(), p->sign);
  if (p->rank >= 2 && (p->flags & FFTW_MPI_TRANSPOSED_OUT)) {
    qsf_shim_swap01(p->data, p->n[0], p->n[1], rest);
  }
}

/* in-place guru plan: `rank` transformed axes and `howmany_rank` batch axes, strides in
 * complex elements (fftw_plan_guru64_dft) */
static inline fftw_plan fftw_plan_guru64_dft(int rank, const fftw_iodim64* dims, int howmany_rank,
                                             const fftw_iodim64* howmany_dims, fftw_complex* in, fftw_complex* out,
                                             int sign, unsigned flags) {
  if (in != out) {
    fprintf(stderr, "FFTW stand-in: only in-place guru plans are available\n");
    abort();
  }
  fftw_plan p = new qsf_shim_plan();
  p->guru = true;
  p->rank = rank;
  p->data = reinterpret_cast<double*>(in);
  p->sign = sign;
  p->flags = flags;
  p->howmany = 1;
  p->dims.assign(dims, dims + rank);
  p->hdims.assign(howmany_dims, howmany_dims + howmany_rank);
  return p;
}
