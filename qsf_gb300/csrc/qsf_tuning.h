// qsf_tuning.h -- pass kernel shapes per line length: points and threads per block of
// the row / axis passes, and the radix plan of the one-CTA 1D line kernel.
//
// Written by the autotuner (qsf_gb300/autotune.py) from step times measured on a GB300:
//   python -m qsf_gb300.autotune --write
// Row / axis shapes: points per block x threads per block (16 points per thread:
// radix-16 plans, 128 registers; 8: radix-8 plans); lengths not listed take
// 4096x256.  Measured (one call of graph-replayed steps per workload, ms per step):
//   2d256   ms/step  4096x256: 0.0690  4096x512: 0.0684
//   2d320   ms/step  4096x256: 0.0856  4096x512: 0.0793
//   2d512   ms/step  4096x256: 0.0878  4096x512: 0.0719
//   2d640   ms/step  4096x256: 0.1040  4096x512: 0.1200
//   2d1024  ms/step  4096x256: 0.1072  4096x512: 0.1266
//   2d2048  ms/step  4096x256: 0.4266  4096x512: 0.4351
//   2d4096  ms/step  4096x256: 1.7265  4096x512: 1.9262
//   3d128   ms/step  4096x256: 0.2970  4096x512: 0.3152
//   3d256   ms/step  4096x256: 1.8341  4096x512: 1.9360
#pragma once

namespace qsf {

__host__ __device__ constexpr int tuned_row_threads(int n) {
  return n == 320 ? 512 : n == 512 ? 512 : 256;
}

__host__ __device__ constexpr int tuned_tile(int n) {
  return 4096;
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
