// qsf_tuning.h -- threads per block of the row / axis pass kernels per line length.
//
// Written by the autotuner (qsf_gb300/autotune.py) from step times measured on a GB300:
//   python -m qsf_gb300.autotune --write
// 256 threads carry 16 points of a 4096-point tile each (radix-16 plans, 128 registers),
// 512 threads 8 points (radix-8 plans, 64 registers, twice the resident warps).  Line
// lengths not listed take 256.  Measured (one call of graph-replayed steps per
// workload, threads per block: ms per step):
//   2d256   ms/step  256: 0.0889  512: 0.0789
//   2d384   ms/step  256: 0.1077  512: 0.0903
//   2d512   ms/step  256: 0.1054  512: 0.0817
//   2d768   ms/step  256: 0.1276  512: 0.1412
//   2d1024  ms/step  256: 0.1292  512: 0.1457
//   2d2048  ms/step  256: 0.6016  512: 0.5108
//   2d4096  ms/step  256: 2.0772  512: 2.1414
//   3d128   ms/step  256: 0.3436  512: 0.3521
//   3d256   ms/step  256: 2.1315  512: 2.2095
#pragma once

namespace qsf {

__host__ __device__ constexpr int tuned_row_threads(int n) {
  return (n == 384 || n == 512 || n == 2048) ? 512 : 256;
}

}  // namespace qsf
