// qsf_tuning.h -- threads per block of the row / axis pass kernels per line length.
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

}  // namespace qsf
