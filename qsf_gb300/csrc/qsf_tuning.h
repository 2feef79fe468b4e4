// qsf_tuning.h -- pass kernel shapes per line length: threads per block of the row /
// axis passes, and the radix plan of the one-CTA 1D line kernel.
//
// Written by the autotuner (qsf_gb300/autotune.py) from step times measured on a GB300:
//   python -m qsf_gb300.autotune --write
// 256 threads carry 16 points of a 4096-point tile each (radix-16 plans, 128 registers),
// 512 threads 8 points (radix-8 plans, 64 registers, twice the resident warps).  Line
// lengths not listed take 256.  Measured (one call of graph-replayed steps per
// workload, threads per block: ms per step):
//   2d256   ms/step  256: 0.0690  512: 0.0684
//   2d384   ms/step  256: 0.0856  512: 0.0793
//   2d512   ms/step  256: 0.0878  512: 0.0719
//   2d768   ms/step  256: 0.1040  512: 0.1200
//   2d1024  ms/step  256: 0.1072  512: 0.1266
//   2d2048  ms/step  256: 0.4266  512: 0.4351
//   2d4096  ms/step  256: 1.7265  512: 1.9262
//   3d128   ms/step  256: 0.2970  512: 0.3152
//   3d256   ms/step  256: 1.8341  512: 1.9360
#pragma once

namespace qsf {

__host__ __device__ constexpr int tuned_row_threads(int n) {
  return (n == 384 || n == 512) ? 512 : 256;
}

// Points per thread of the one-CTA 1D line kernel per line length (4: radix-4 plans,
// 8: radix 8, 16: radix 16); a length between measured ones takes the plan of the next
// longer measured length.  Measured (one call of graph-replayed steps, points per
// thread: ms per step):
//   1d1024  ms/step  4: 0.0392  8: 0.0416  16: 0.0452
//   1d1536  ms/step  4: 0.0479  8: 0.0472  16: 0.0568
//   1d2048  ms/step  4: 0.0537  8: 0.0522  16: 0.0543
//   1d3072  ms/step  8: 0.0663  16: 0.0683
//   1d4096  ms/step  8: 0.0733  16: 0.0711
__host__ __device__ constexpr int tuned_line_ppt(int n) {
  return n <= 1024 ? 4 : n <= 3072 ? 8 : 16;
}

}  // namespace qsf
