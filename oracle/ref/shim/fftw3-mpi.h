/* FFTW-MPI API stand-in for a single process (see fftw3.h in this directory).
 * Test infrastructure for the oracle harness only. */
#pragma once
#include "fftw3.h"
#include "mpi.h"

static inline void fftw_mpi_init() {}

static inline fftw_plan fftw_mpi_plan_many_dft(int rnk, const std::ptrdiff_t* n, std::ptrdiff_t howmany,
                                               std::ptrdiff_t, std::ptrdiff_t, fftw_complex* in,
                                               fftw_complex* out, MPI_Comm, int sign, unsigned flags) {
  if (in != out || (howmany != 1 && (flags & (FFTW_MPI_TRANSPOSED_IN | FFTW_MPI_TRANSPOSED_OUT)))) {
    fprintf(stderr, "FFTW-MPI stand-in: only in-place plans, transposed ones with howmany=1, are available\n");
    abort();
  }
  fftw_plan p = new qsf_shim_plan();
  p->rank = rnk;
  p->n.assign(n, n + rnk);
  p->data = reinterpret_cast<double*>(in);
  p->sign = sign;
  p->flags = flags;
  p->guru = false;
  p->howmany = (long)howmany;
  return p;
}

static inline std::ptrdiff_t fftw_mpi_local_size_1d(std::ptrdiff_t n0, MPI_Comm, int, unsigned,
                                                    std::ptrdiff_t* ni, std::ptrdiff_t* si,
                                                    std::ptrdiff_t* no, std::ptrdiff_t* so) {
  *ni = n0; *si = 0; *no = n0; *so = 0;
  return n0;
}

static inline std::ptrdiff_t fftw_mpi_local_size(int rnk, const std::ptrdiff_t* n, MPI_Comm,
                                                 std::ptrdiff_t* n0l, std::ptrdiff_t* s0) {
  std::ptrdiff_t m = 1;
  for (int i = 0; i < rnk; ++i) m *= n[i];
  *n0l = n[0];
  *s0 = 0;
  return m;
}

static inline std::ptrdiff_t fftw_mpi_local_size_2d_transposed(std::ptrdiff_t n0, std::ptrdiff_t n1, MPI_Comm,
                                                               std::ptrdiff_t* l0, std::ptrdiff_t* s0,
                                                               std::ptrdiff_t* l1, std::ptrdiff_t* s1) {
  *l0 = n0; *s0 = 0; *l1 = n1; *s1 = 0;
  return n0 * n1;
}
