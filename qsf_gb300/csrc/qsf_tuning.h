// qsf_tuning.h -- pass kernel shapes per line length: points and threads per block of
// the row / axis passes, and the radix plan of the one-CTA 1D line kernel.
//
// Written by the autotuner (qsf_gb300/autotune.py) from step times measured on a GB300:
//   python -m qsf_gb300.autotune --write
// Row / axis shapes: points per block x threads per block (16 points per thread:
// radix-16 plans, 128 registers; 8: radix-8 plans); lengths not listed take
// 4096x256.  Chosen among 4096x256, 4096x512; smaller tiles, timed
// beside them, speed up small grids run alone but slow the batched form down.
// Measured (one call of graph-replayed steps per workload, ms per step):
//   2d256   ms/step  4096x256: 0.0693  4096x512: 0.0691  2048x128: 0.0577  2048x256: 0.0511  1024x128: 0.0449
//   2d320   ms/step  4096x256: 0.0904  4096x512: 0.0744  2048x128: 0.0823  2048x256: 0.0552  1024x128: 0.0510
//   2d384   ms/step  4096x256: 0.0860  4096x512: 0.0801  2048x128: 0.0777  2048x256: 0.0608  1024x128: 0.0522
//   2d512   ms/step  4096x256: 0.0889  4096x512: 0.0725  2048x128: 0.0776  2048x256: 0.0513  1024x128: 0.0499
//   2d640   ms/step  4096x256: 0.0921  4096x512: 0.0863  2048x128: 0.0869  2048x256: 0.0765  1024x128: 0.1035
//   2d768   ms/step  4096x256: 0.1050  4096x512: 0.1213  2048x128: 0.0830  2048x256: 0.1095  1024x128: 0.1096
//   2d1024  ms/step  4096x256: 0.1069  4096x512: 0.1276  2048x128: 0.1098  2048x256: 0.1376  1024x128: 0.1306
//   2d2048  ms/step  4096x256: 0.4450  4096x512: 0.4330  2048x128: 0.4477  2048x256: 0.5127  1024x128: 0.4559
//   2d4096  ms/step  4096x256: 1.6895  4096x512: 1.8929  2048x128: 2.6868  2048x256: 1.6912  1024x128: 2.7324
//   3d128   ms/step  4096x256: 0.2978  4096x512: 0.3166  2048x128: 0.2872  2048x256: 0.3250  1024x128: 0.3178
//   3d256   ms/step  4096x256: 1.8134  4096x512: 1.9213  2048x128: 1.8110  2048x256: 2.2277  1024x128: 2.2397
#pragma once

namespace qsf {

__host__ __device__ constexpr int tuned_row_threads(int n) {
  return n == 320 ? 512 : n == 384 ? 512 : n == 512 ? 512 : n == 640 ? 512 : n == 2048 ? 512 : 256;
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
