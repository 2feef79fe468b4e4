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
  const KernelSet* ks = nullptr;  // kernels for this grid's line length
  GridDev* dG = nullptr;          // device copy of G (step kernels read descriptors from device arrays)
  StepDev* dS = nullptr;          // device copy of the current step descriptor
  // the batch this grid is a member of (qsf_batch_add) and its slot there: destroying
  // the grid removes it from that batch first (the batch's graph reads its memory)
  qsf_batch* batch = nullptr;
  int64_t batch_slot = -1;
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
  // member-operation step programs (grids without fused kernels): the executable graph
  // of gen_steps steps, the program it was captured for, and whether the member
  // operations' tables of the current program are made (before any capture)
  cudaGraphExec_t gen_exec = nullptr;
  int gen_steps = 0;
  std::vector<long long> gen_key;
  bool gen_primed = false;
  // TMA tensor maps of psi for the strided-axis passes (GridDev::tmap), 128 bytes each
  unsigned char* tmaps = nullptr;
  // Bluestein transforms of a grid whose axis length has a prime factor above 5 (no
  // fused kernels, ks == nullptr): chirp c[j] = exp(-i pi j^2 / n), the transform of
  // the convolution kernel conj(c) padded to M (a length >= 2n - 1 with built
  // kernels), the M-point kernels and twiddles, and a scratch of (m / n) * M points.
  // A 1D line longer than 8192 points takes M = M1 * M2 above 16384 as a four-step
  // transform: M1-point transforms along the columns of the [M1][M2] view, the twiddles
  // exp(-2 pi i k1 n2 / M), M2-point transforms along its rows (the output in the
  // transposed order [k1][k2] = X[k1 + M1 k2], which the convolution does not mind).
  struct Bluestein {
    int n = 0, M = 0;
    int M1 = 0, M2 = 0;  // four-step factors; 0: one M-point transform per line
    const KernelSet* ks = nullptr;   // M-point kernels (or M2-point row kernels)
    const KernelSet* ks1 = nullptr;  // M1-point column kernels (four-step)
    double2* chirp = nullptr;
    double2* bhat = nullptr;
    double2* scratch = nullptr;
    // shared per-process tables (not owned by the grid)
    double2* tw = nullptr;  // twiddles of M (or M2)
    longlong2* twx = nullptr;
    longlong2* twf = nullptr;
    double2* tw1 = nullptr;  // twiddles of M1
    longlong2* twx1 = nullptr;
    longlong2* twf1 = nullptr;
    double2* tw4 = nullptr;  // four-step twiddles [k1][n2]
  } bs;
};

namespace qsf {
// whether n is a line length with fused step kernels in this build
bool fused_length(int n);
bool grid_fused(const qsf_grid* g);
// psi = 0 on the grid's stream
int grid_clear(qsf_grid* g);
// Member-operation steps of a grid without fused kernels (qsf_step's path for them),
// in parts for the server: begin checks the program and zeroes its device rows and
// NaN flag; enqueue queues steps [first, first + count) on the grid's stream without
// waiting (no convergence test); wait waits for the stream and reads the NaN flag;
// rows copies the first nsteps rows to the host.
int generic_begin(qsf_grid* g, const qsf_step_desc* d);
int generic_enqueue(qsf_grid* g, const qsf_step_desc* d, int64_t first, int64_t count);
int generic_wait(qsf_grid* g, bool* bad);
int generic_rows(qsf_grid* g, const qsf_step_desc* d, double* rows, int64_t nsteps);
// qsf_batch_add without waiting for the batch's stream, for a grid that no queued work
// of the batch touches (a solve the server prepares while a round runs); it joins at
// the next batch_launch
int batch_add_nowait(qsf_batch* b, qsf_grid* g, const qsf_step_desc* d, int64_t* slot);
// qsf_batch_run in two halves: launch (rebuild after membership changes, queue the
// steps' graph launches) and finish (wait, read every member's counters)
int batch_launch(qsf_batch* b, int64_t steps);
int batch_finish(qsf_batch* b, int64_t* active);
// twiddle tables of an n-point transform shared by all grids of the process (not to
// be freed by the caller)
int shared_twiddles(int n, double2** tw, longlong2** twx, longlong2** twf);
// twiddle tables of an n-point transform (FP64, 2^62 fixed point, split form)
int make_twiddles(int n, double2** tw, longlong2** twx, longlong2** twf);
// Bluestein plan of a grid without fused kernels (qsf_bluestein.cu)
int bs_setup(qsf_grid* g);
void bs_release(qsf_grid* g);
// one axis of fourier<R>() by Bluestein's chirp-z convolution, in place on the array
// arr (psi's geometry: psi itself, or a region-transfer slice), scaled by post
int bs_axis(qsf_grid* g, double2* arr, int ax, bool fwd, double post);
// the convolution length M >= 2n - 1 of an n-point axis of a dim-D grid (0: none)
int bs_size(int n, int dim);
}  // namespace qsf
