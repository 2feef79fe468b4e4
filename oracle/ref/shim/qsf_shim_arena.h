/* Shared allocation arena of the MPI / FFTW stand-ins.  With more than one rank the
 * MPI stand-in maps one shared anonymous region before it forks the ranks and gives
 * each rank a slice of it; fftw_malloc then allocates from that slice, so every
 * rank sees every other rank's wavefunction at the same address (this is how the
 * stand-in serves MPI_Get on a window).  With one rank fftw_malloc uses the heap.
 * Test infrastructure for the oracle harness only. */
#pragma once
#include <cstddef>

inline char* qsf_shim_arena_cur = nullptr;  // this rank's free space
inline char* qsf_shim_arena_end = nullptr;
inline char* qsf_shim_arena_lo = nullptr;   // the whole shared mapping
inline char* qsf_shim_arena_hi = nullptr;

static inline void* qsf_shim_arena_alloc(size_t n) {
  if (!qsf_shim_arena_cur) return nullptr;
  const size_t a = (n + 255) & ~(size_t)255;
  if ((size_t)(qsf_shim_arena_end - qsf_shim_arena_cur) < a) return nullptr;
  void* p = qsf_shim_arena_cur;
  qsf_shim_arena_cur += a;
  return p;
}
static inline bool qsf_shim_in_arena(const void* p) {
  return qsf_shim_arena_lo && (const char*)p >= qsf_shim_arena_lo && (const char*)p < qsf_shim_arena_hi;
}
