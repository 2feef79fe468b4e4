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
};
typedef qsf_shim_plan* fftw_plan;

static inline void* fftw_malloc(size_t n) {
  void* p = nullptr;
  if (posix_memalign(&p, 64, n ? n : 64)) return nullptr;
  return p;
}
static inline void fftw_free(void* p) { free(p); }
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

static inline void fftw_execute(const fftw_plan p) {
  if (p->guru) {
    fprintf(stderr, "FFTW stand-in: guru (partial) plans are not available\n");
    abort();
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

static inline fftw_plan fftw_plan_guru64_dft(int, const fftw_iodim64*, int, const fftw_iodim64*, fftw_complex*,
                                             fftw_complex*, int, unsigned) {
  fftw_plan p = new qsf_shim_plan();
  p->guru = true;
  return p;
}
