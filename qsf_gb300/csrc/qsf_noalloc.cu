// qsf_noalloc.cu -- norm of a caller-owned wavefunction without any device allocation.
//
// Some callers cannot allocate device memory: a host program that hands out all
// device memory from its own pool or arena, a language runtime that may only pass
// buffers it already owns across a foreign-function boundary, or code that must not
// let a library allocate behind its back.  For them, qsf_norm_noalloc computes
// <psi|psi> dV (average<X, Identity>, grid.h:425-441) of a wavefunction the caller
// already holds on the device, writing one double into a device buffer the caller
// also owns.  The per-block partial sums that qsf_average keeps in its grid handle
// live here in a fixed file-scope device array instead; no cudaMalloc, cudaFree or
// allocating library routine is called.
//
// Limits and behaviour:
//  - the scratch array holds kNoAllocMaxBlocks partial sums, each block summing
//    kNoAllocChunk points, so m may be at most kNoAllocMaxBlocks * kNoAllocChunk
//    (134,217,728 points, 2 GiB of complex128); larger m is rejected with QSF_EINVAL;
//  - the array (64 KiB) is part of the library image: every GPU that loads the
//    library holds it until the process exits;
//  - all calls share the one array; calls that overlap on the GPU (different streams
//    or threads) race on it, so callers serialise them; nothing in it needs to start
//    at zero because each call writes every entry it later reads;
//  - the first call on a device looks up the array's device address with
//    cudaGetSymbolAddress (with that device current) and caches it; make that first
//    call before any stream capture.
#include <mutex>
#include <string>

#include <cuda_runtime.h>

#include "qsf_gpu.h"

namespace qsf {
// records the message returned by qsf_last_error() (defined with the rest of the ABI)
void set_error_message(const std::string& msg);
}  // namespace qsf

namespace {

constexpr int kNoAllocThreads = 256;
constexpr int kNoAllocMaxBlocks = 8192;
constexpr long long kNoAllocChunk = 16384;  // points per block

// the scratch: one partial sum per block of the first pass
static __device__ __align__(256) double g_noalloc_partials[kNoAllocMaxBlocks];


__device__ __forceinline__ double warp_sum_na(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double block_sum_na(double v) {
  __shared__ double red[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  v = warp_sum_na(v);
  if (lane == 0) red[wid] = v;
  __syncthreads();
  double t = 0.0;
  if (wid == 0) {
    t = lane < nw ? red[lane] : 0.0;
    t = warp_sum_na(t);
  }
  return t;  // valid in thread 0
}

// pass 1: block b sums |psi|^2 over points [b * chunk, min(m, (b + 1) * chunk))
__global__ void __launch_bounds__(kNoAllocThreads) k_norm_partials(const double2* __restrict__ psi, long long m,
                                                                   double* __restrict__ partials) {
  const long long p0 = (long long)blockIdx.x * kNoAllocChunk;
  const long long p1 = p0 + kNoAllocChunk < m ? p0 + kNoAllocChunk : m;
  double acc = 0.0;
  for (long long p = p0 + threadIdx.x; p < p1; p += blockDim.x) {
    const double2 v = psi[p];
    acc = fma(v.x, v.x, fma(v.y, v.y, acc));
  }
  acc = block_sum_na(acc);
  if (threadIdx.x == 0) partials[blockIdx.x] = acc;
}

// pass 2: one block sums the partials in a fixed order and scales by the volume
__global__ void __launch_bounds__(kNoAllocThreads) k_norm_finish(const double* __restrict__ partials, int nblocks,
                                                                 double dV, double* __restrict__ out) {
  double acc = 0.0;
  for (int i = threadIdx.x; i < nblocks; i += blockDim.x) acc += partials[i];
  acc = block_sum_na(acc);
  if (threadIdx.x == 0) out[0] = acc * dV;
}

// device address of the scratch array, looked up once per device
double* scratch_for_current_device(int* rc) {
  static std::mutex mu;
  static double* ptrs[64] = {nullptr};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    qsf::set_error_message(std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    *rc = QSF_ECUDA;
    return nullptr;
  }
  if (dev < 0 || dev >= 64) {
    qsf::set_error_message("qsf_norm_noalloc: device index " + std::to_string(dev) +
                           " exceeds the 64 devices whose scratch address is cached");
    *rc = QSF_EINVAL;
    return nullptr;
  }
  std::lock_guard<std::mutex> lk(mu);
  if (!ptrs[dev]) {
    double* p = nullptr;
    e = cudaGetSymbolAddress((void**)&p, g_noalloc_partials);
    if (e != cudaSuccess || !p) {
      qsf::set_error_message(std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      *rc = QSF_ECUDA;
      return nullptr;
    }
    ptrs[dev] = p;
  }
  *rc = QSF_OK;
  return ptrs[dev];
}

}  // namespace

extern "C" {

int qsf_norm_noalloc(const double* psi_dev, int64_t m, double dV, double* out_dev, void* stream) {
  if (!psi_dev || !out_dev || m < 1) {
    qsf::set_error_message("qsf_norm_noalloc: null buffer or m < 1");
    return QSF_EINVAL;
  }
  const long long max_m = (long long)kNoAllocMaxBlocks * kNoAllocChunk;
  if (m > max_m) {
    qsf::set_error_message("qsf_norm_noalloc: m = " + std::to_string((long long)m) + " exceeds the maximum of " +
                           std::to_string(max_m) + " points that the fixed scratch array can reduce");
    return QSF_EINVAL;
  }
  int rc = QSF_OK;
  double* scratch = scratch_for_current_device(&rc);
  if (rc) return rc;
  const int nblocks = (int)((m + kNoAllocChunk - 1) / kNoAllocChunk);
  cudaStream_t st = (cudaStream_t)stream;
  // clear an earlier, unrelated launch error so that the check below reports this call's own
  cudaGetLastError();
  k_norm_partials<<<nblocks, kNoAllocThreads, 0, st>>>((const double2*)psi_dev, (long long)m, scratch);
  k_norm_finish<<<1, kNoAllocThreads, 0, st>>>(scratch, nblocks, dV, out_dev);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    qsf::set_error_message(std::string("qsf_norm_noalloc launch: ") + cudaGetErrorString(e));
    return QSF_ECUDA;
  }
  return QSF_OK;
}

}  // extern "C"
