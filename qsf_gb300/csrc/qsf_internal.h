// qsf_internal.h -- library-internal declarations shared by the host translation units
// of libqsfgpu.so (not part of the C ABI): the grid handle's device state, error
// reporting and allocation helpers.
#pragma once
#include <algorithm>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "qsf_gpu.h"
#include "qsf_borders.h"
#include "qsf_kernels.cuh"

namespace qsf {

// records msg as the text qsf_last_error() returns on this thread and returns code
int fail(int code, const std::string& msg);

// multiprocessor count of the current device (queried once per device); grid-stride
// kernels size their grids as a multiple of it
int device_sm_count();

template <class T>
int dev_alloc(T*& p, size_t count) {
  if (p) cudaFree(p);
  p = nullptr;
  if (count == 0) return QSF_OK;
  if (cudaMalloc((void**)&p, count * sizeof(T)) != cudaSuccess) {
    cudaGetLastError();
    p = nullptr;
    return fail(QSF_ENOMEM, "cudaMalloc of " + std::to_string(count * sizeof(T)) + " bytes failed");
  }
  return QSF_OK;
}
template <class T>
int dev_reserve(T*& p, size_t& cap, size_t count) {
  if (count <= cap && p) return QSF_OK;
  size_t c = std::max(count, cap * 2);
  int rc = dev_alloc(p, c);
  cap = rc == QSF_OK ? c : 0;
  return rc;
}

}  // namespace qsf

#define QSF_CU(call)                                                                                   \
  do {                                                                                                 \
    cudaError_t e_ = (call);                                                                           \
    if (e_ != cudaSuccess) return qsf::fail(QSF_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

using qsf::AxisDev;
using qsf::GridDev;
using qsf::KernelSet;
using qsf::StepDev;
using qsf::FluxPoint;
using qsf::FluxTerm;
using qsf::BorderNodes;

struct qsf_grid {
  qsf_grid_desc desc{};
  GridDev G{};
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  BorderNodes bn;
  std::vector<double2*> tw_owned;
  std::vector<longlong2*> twx_owned;
  const KernelSet* ks = nullptr;  // kernels for this grid's line length
  GridDev* dG = nullptr;          // device copy of G (step kernels read descriptors from device arrays)
  StepDev* dS = nullptr;          // device copy of the current step descriptor
  // static tables
  longlong2* xs = nullptr;
  long long* Vx = nullptr;
  int xs_mode = 0;
  double xs_delta = 0.0;
  int xs_exp = 0;
  int vshift = 0;
  double vmax = 0.0, vneg = 0.0;  // max V and max -V over the grid
  bool V_ready = false;
  // per-step tables
  longlong2* ptab = nullptr;
  longlong2* xdyn = nullptr;
  int nmax = 0;
  int l2m = 0;
  double m_mant = 1.0;
  // fixed-point pass bookkeeping: [kTexp] table exponents, [4] pass minima, [4][scmax] block exponents
  int* ibuf = nullptr;
  int scmax = 1;
  // reductions
  double* partials = nullptr;
  int pmax = 0;
  double* fpartials = nullptr;
  size_t fpmax = 0;
  long long* ctl = nullptr;
  double* energy = nullptr;
  double* scale = nullptr;
  double* rows_dev = nullptr;
  size_t rows_cap = 0;
  double* coup_dev = nullptr;
  size_t coup_cap = 0;
  // flux structures
  std::vector<int> fl_borders;
  int64_t fl_box = -1;
  bool fl_ready = false;
  double2* snap = nullptr;
  long long* snap_idx = nullptr;
  int* row_ptr = nullptr;
  FluxPoint* fpts = nullptr;
  FluxTerm* fterms = nullptr;
  int nsnap = 0, nfterms = 0, nfpts = 0, nfblk = 1;
  // launch geometry
  int row_L = 1;
  int nrowblk = 1;
  size_t row_smem = 0;
  int ax_C[3] = {1, 1, 1};
  int ax_blocks[3] = {0, 0, 0};
  size_t ax_smem[3] = {0, 0, 0};
  // multi-region transfer: slice buffer (m points) and the event that orders streams
  double2* mg_slice = nullptr;
  // member evolve: cached X-phase factors for (mode, delta) and per-axis P factors
  double2* etab = nullptr;
  int etab_mode = 0;
  double etab_delta = 0.0;
  double2* eptab = nullptr;
  // observables log of qsf_average_log (device, grow-only)
  double* obs_log = nullptr;
  size_t obs_cap = 0;
  double* vtab = nullptr;  // potential per point for member E_pot averages (built on first use)
  double* mtab = nullptr;  // per-axis one-node absorber masks [dim][nmax] (built on first use)
  cudaEvent_t mg_event = nullptr;
  // k_finalize of graph-replayed steps on a second stream, beside the next sub-step's
  // first passes: the stream and its fork / join events (created on first use)
  cudaStream_t fin_stream = nullptr;
  cudaEvent_t fin_fork = nullptr, fin_done = nullptr;
  // executable step graphs of qsf_step, kept per launch shape and replayed by later
  // calls (the kernels read every per-call value from the device descriptors)
  struct StepGraph {
    int64_t per;
    int skip_open, overlap, ekin, nfblk;
    cudaGraphExec_t exec;
  };
  std::vector<StepGraph> step_graphs;
  // TMA tensor maps of psi for the strided-axis passes (GridDev::tmap), 128 bytes each
  unsigned char* tmaps = nullptr;
};
