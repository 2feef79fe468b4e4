/*
 * qsf_gpu.h -- C ABI of libqsfgpu.so, the GB300 (sm_103a) implementation of QSF's
 * split-operator time step for the reduced-dimensionality multi-electron TDSE.
 *
 * The reference (QSF-physics/QSF) is a header-only C++ library whose grid type
 * LocalGrid<Hamiltonian, BaseGrid, ...> (include/wf/grid.h) owns the wavefunction and
 * exposes fourier / evolve / average / current_map / flux / operation / maskRegion to
 * the propagator (include/propagator.h).  This ABI replaces those members with calls
 * that run hand-written CUDA kernels on one GPU; every entry point below names the
 * reference member it stands in for.  The wavefunction lives in device memory owned
 * by a qsf_grid handle and is exchanged as complex128.  Inside a step the transforms
 * and phase products run in block fixed point (int64 components sharing one
 * power-of-two exponent per thread block, 55 or more significant bits), which is more
 * accurate than an FP64 FFT and runs on GB300's integer pipes.
 *
 * Conventions
 *  - Arrays of complex numbers are interleaved doubles (re, im), C order, last axis
 *    contiguous -- the reference's layout (grid.h:226-237, cxd = std::complex<double>).
 *  - Every function returns QSF_OK (0) or a QSF_E* status; nothing aborts and no C++
 *    exception crosses the ABI (the reference instead aborts via logError,
 *    basics/logging.h:114).
 *  - A handle is used from one host thread at a time; calls on one handle are
 *    ordered on that handle's CUDA stream.
 */
#ifndef QSF_GPU_H
#define QSF_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
#define QSF_OK 0
#define QSF_EINVAL 1     /* bad argument or unsupported grid                        */
#define QSF_ENOMEM 2     /* device allocation failed                                */
#define QSF_ECUDA 3      /* a CUDA runtime call failed                              */
#define QSF_ETIMEDOUT 4  /* a bounded wait ran out                                  */
#define QSF_ENUMERIC 5   /* NaN/Inf or a non-positive norm in a reduction           */
#define QSF_ESTATE 6     /* call not valid in the handle's current state            */
#define QSF_EBUSY 7      /* admission refused (no slot or not enough free HBM)      */
#define QSF_ECANCELED 8  /* a served request was cancelled (qsf_server_cancel)      */

/* ------------------------------------------------------ reference enums */
/* MODE (basics/enums.h:15-21), REP (36-42) */
#define QSF_MODE_IM 1
#define QSF_MODE_RE 2
#define QSF_REP_X 1
#define QSF_REP_P 2
/* potentials: ReducedDimInteraction<Eberly|EckhardSacha> (potential.h:97-179),
 * CoulombInteraction (potential.h:21-82) */
#define QSF_POT_EBERLY 0
#define QSF_POT_ECKHARDT_SACHA 1
#define QSF_POT_COULOMB 2
#define QSF_POT_NONE 3
/* gauges: DipoleCoupling<VelocityGauge> couples in P (coupling.h:101-118);
 * the length gauge couples x.E(t) in X */
#define QSF_GAUGE_VELOCITY 0
#define QSF_GAUGE_LENGTH 1

/* absorber kinds (qsf_grid_desc.absorber) */
#define QSF_ABS_CAP 0  /* the reference's quartic CAP (absorbers.h:27-54) */
#define QSF_ABS_COS8 1 /* cos^(1/8) mask over the same margins; no reference counterpart */
/* averaged operators: Identity, PotentialEnergy, KineticEnergy (grid.h:7-22) */
#define QSF_OP_IDENTITY 0
#define QSF_OP_POTENTIAL 1
#define QSF_OP_KINETIC 2
/* flux border types (fluxes/borders.h:39-257) */
#define QSF_B_BOX 0
#define QSF_B_S2CAP 1
#define QSF_B_D2CAP 2
#define QSF_B_N2S 3
#define QSF_B_N2D 4
#define QSF_B_N2D_SYM 5
#define QSF_B_N2D_ASYM 6
#define QSF_B_S2D 7
#define QSF_B_S2D_SYM 8
#define QSF_B_S2D_ASYM 9
#define QSF_B_N2T 10
#define QSF_B_S2T 11
#define QSF_B_D2T 12
#define QSF_B_T2CAP 13
#define QSF_MAX_BORDERS 16

/* ---------------------------------------------------------------- grid */
/* CAP<CartesianGrid<dim>> (wf/coords.h:14-139, wf/absorbers.h:15-60) together with
 * the Spin0 Hamiltonian's potential and coupling (hamiltonian.h:8-98). */
typedef struct qsf_grid_desc {
  int dim;            /* 1, 2 or 3                                                 */
  int64_t n[3];       /* nodes per axis; dim >= 2 needs n and dx equal on all axes  */
  double dx[3];       /* spacing per axis (atomic units)                           */
  int64_t nCAP;       /* absorber margin in nodes (0: no absorber)                 */
  int potential;      /* QSF_POT_*                                                 */
  double Ncharge, Echarge, Nsoft, Esoft;
  int gauge;          /* QSF_GAUGE_*                                               */
  int n_fields;       /* fields in the coupling; 0 makes the coupling term exactly 0 */
  int p_axis_swap;    /* 1: apply the axis-0 coupling to axis 1 and vice versa in P
                         space, as the reference's transposed P layout does
                         (grid.h:242-247); ignored for dim == 1                    */
  int64_t border_nodes[4]; /* p_NS, p_SD, p_DT, p_CAP (borders.h:30-36); 0 = default */
  /* Region of a multi-region grid (CAP<MultiCartesianGrid<D>>, multigrid.h; regions of
   * MultiRegionsReduced<D>, mpi_logic.h:262-278).  multi_region = 0: an ordinary grid
   * (both fields 0).  multi_region = 1: evolve applies no absorber (the region masks of
   * qsf_mask_region take its place after each step) and the potential is the partial
   * one of the region (ReducedDimInteraction::partial, potential.h:144-178);
   * free_axes (bit d = axis d) are the axes the region keeps in momentum space:
   * qsf_fourier transforms the other (bounded) axes only and scales by the product of
   * their 1/n (fourier_partial, multigrid.h:660-674), and the P layout is untransposed
   * (set p_axis_swap = 0) unless free_axes = 0 (the main region).  Regions with free
   * axes step through the member operations; qsf_step rejects them.              */
  int free_axes;
  int multi_region;
  /* Absorber over the nCAP-node margins.  QSF_ABS_CAP (0): the reference's CAP,
   * exp(-delta eta sum_d max(0, nodes_d)^4) per evolve<X>(delta).  QSF_ABS_COS8: the
   * cos^(1/8) mask of the 1D plain configuration (the reference has none): with node
   * depth nodes_d = nCAP + neg_dist_from_edge (grid.h:181-185), M = prod_d
   * cos(pi/2 nodes_d / nCAP)^(1/8) over the margin nodes, applied once per mask_dt of
   * propagation (evolve<X>(delta) multiplies by M^(delta / mask_dt); a Strang step of
   * dt = mask_dt applies M once).  Needs nCAP >= 1, mask_dt > 0, multi_region = 0. */
  int absorber;
  double mask_dt;
} qsf_grid_desc;

typedef struct qsf_grid qsf_grid;

/* LocalGrid constructor (grid.h:115-133, 275-293): allocates the device state.
 * `stream` is a cudaStream_t or NULL (the handle then creates its own stream).
 * Axis lengths: any n >= 2 (the reference's FFTW plans take any n, grid.h:251-274) up
 * to 16384 on a 1D line and 4096 on the axes of a 2D / 3D grid.  The lengths of the
 * built kernel list (2^a, 3*2^a and 5*2^a from 8 to 16384: 33 lengths) take the fused
 * kernels; the others (up to 16384 in 1D, 2048 in 2D / 3D) transform each axis by
 * Bluestein's chirp-z convolution over a built length M >= 2n - 1 (a four-step
 * M1 x M2 transform for 1D lines above 8192 points), and qsf_step runs their steps as
 * the member operations evolve / fourier / average; batches take built lengths only
 * (QSF_EINVAL), the server runs the others beside its batch.  Other lengths:
 * QSF_EINVAL. */
int qsf_grid_create(const qsf_grid_desc* desc, void* stream, qsf_grid** out);
/* Frees the grid's device state; a member of a batch leaves the batch first. */
int qsf_grid_destroy(qsf_grid* g);
/* number of grid points m and the device address of psi (complex128[m]) */
int qsf_grid_size(const qsf_grid* g, int64_t* m);
int qsf_psi_device_ptr(qsf_grid* g, void** dptr);

/* copies between host memory (interleaved complex128, m elements) and the grid.
 * operator[] / save / load of the reference (grid.h:296-297, 789-1153). */
int qsf_upload(qsf_grid* g, const double* host_psi, int64_t m);
int qsf_download(qsf_grid* g, double* host_psi, int64_t m);
int qsf_synchronize(qsf_grid* g);

/* ------------------------------------------------------ granular members */
/* fourier<R>() (grid.h:369-378): forward DFT (FFTW_FORWARD) to P or backward DFT
 * to X followed by the 1/m rescale (normalizeAfterTwoFFT, grid.h:363-367).  P space
 * is kept in natural (untransposed) order. */
int qsf_fourier(qsf_grid* g, int to_rep);
/* evolve<M, R>(delta) (grid.h:394-423): psi *= expOp(delta * H_R(r)) and, in X,
 * the absorber (absorbers.h:40-46).  coupling[3] holds the coupling values per axis
 * (A in the velocity gauge, E in the length gauge, as _coupling[Axis<d>] returns). */
int qsf_evolve(qsf_grid* g, int mode, int rep, double delta, const double* coupling3);
/* Region transfer of a multi-region grid, one source (LocalGrid<..., Slices, true>::
 * transfer / coherentAddition, multigrid.h:454-657): dst += DFT_axis(slice), slice =
 * src in the absorber margins along `axis` (both edges), times 1 - mask of that axis
 * and, when dst is in group 1 (one free axis), the corner correction mask_correction
 * (multigrid.h:519-530); in 3D only the n / nCAP boxes of nCAP planes along the
 * sliding axis take part, in 1D the whole line enters and only its margins are masked
 * (as the reference's getBox / maskSlice do).  The DFT is forward and unnormalised.
 * `group` is dst's number of free axes; src must be the region with `axis` bounded and
 * dst's other free axes free.  Both grids need the same geometry and 2 nCAP <= n.
 * The call orders dst's stream after src's and src's after the transfer. */
int qsf_region_transfer(qsf_grid* dst, const qsf_grid* src, int axis, int group);

/* average<R, Op>() (grid.h:425-441). */
int qsf_average(qsf_grid* g, int rep, int op, double* out);
/* The same average without waiting for it (no counterpart in the reference, whose
 * averages return at once): the value goes into slot `slot` of the grid's observables
 * log on the device (grown as needed), so a host loop can queue many steps ahead;
 * qsf_read_log copies slots 0 .. n-1 to host memory (and waits). */
int qsf_average_log(qsf_grid* g, int rep, int op, int64_t slot);
int qsf_read_log(qsf_grid* g, double* out, int64_t n);
/* operation<M, R, Normalize>() (grid.h:601-606); returns the norm divided out. */
int qsf_normalize(qsf_grid* g, double* norm_out);
/* FLUX<B...> (propagator.h:259-265): current_map (grid.h:467-528), the
 * velocity-gauge correction curr += A |psi|^2 (propagator.h:249-257; pass A = NULL
 * in the length gauge) and flux<X, B>() (grid.h:559-573) for each border type. */
int qsf_flux(qsf_grid* g, const double* A3, int nborders, const int* border_types, int64_t box_size,
             double* out);
/* maskRegion() (grid.h:582-597) with CAP::mask (absorbers.h:48-54). */
int qsf_mask_region(qsf_grid* g, const int* bounded3);
/* addUsingCoordinateFunction(gaussian(at, delta, x...)) (grid.h:775-778,
 * wf/preset.h:5-10): psi += gaussian. */
int qsf_add_gaussian(qsf_grid* g, double at, double delta);

/* ------------------------------------------------------- fused Strang steps */
/* One call runs `nsteps` consecutive makeStep()s of SplitPropagator with
 * Split3Base<X,P,X> (propagator.h:311-346, splitting.h:18-27) plus the per-step
 * computeEach observables (propagator.h:275-300), fused into a few passes per step.
 *
 * coupling (host, read during the call):
 *   velocity gauge: nsteps x 3 doubles, A(t) per axis at the step's P sub-step
 *                   (also the A of the flux correction, propagator.h:263);
 *   length gauge:   nsteps x 6 doubles, E(t) per axis at the first and at the
 *                   second X half-step.
 *   May be NULL when the grid has no fields.
 * rows (host, written): nsteps x (3 + nborders) doubles per step, measured on the
 *   wavefunction right after the step and before any Normalize:
 *   [ <psi|psi> dV, <psi|V|psi> dV, <psi|T|psi> dV/m (0 unless QSF_OBS_EKIN),
 *     flux_0 .. flux_{nborders-1} ].
 * With normalize != 0 the step ends with OPERATION<Normalize> (grid.h:601-606).
 * In imaginary time with state_accuracy > 0 the run follows shouldContinue()
 * (propagator.h:304-309): after the first step whose |E_n - E_{n-1}| <= accuracy
 * exactly one more step runs and the call returns; *steps_done says how many ran.
 * E_n = epot + ekin; bit 0 of energy_after_normalize divides epot, bit 1 divides ekin
 * by the step's norm (the observables declared after OPERATION<Normalize>).
 *
 * substeps = K > 1 is MultiProductSplit<Split3Base<X,P,X>, K> (splitting.h:63-91,
 * propagator.h:331-413).  As the reference completes its chains, a step's result is
 * its last chain: K Strang sub-steps of dt / K with the inner X halves joined.  The
 * coupling then holds nsteps * K rows, one per sub-step, as that chain evaluates them
 * (velocity gauge: A at each P sub-step; length gauge: E at the sub-step's opening
 * and closing X half, the closing one equal to the next sub-step's opening one);
 * observables, Normalize and the convergence test apply once per step. */
#define QSF_OBS_NORM 1u
#define QSF_OBS_EPOT 2u
#define QSF_OBS_EKIN 4u
#define QSF_OBS_FLUX 8u
typedef struct qsf_step_desc {
  int mode;                 /* QSF_MODE_IM or QSF_MODE_RE                     */
  double dt;
  int64_t nsteps;
  const double* coupling;   /* see above                                       */
  uint32_t obs;             /* QSF_OBS_* mask                                  */
  int normalize;            /* OPERATION<Normalize> after each step            */
  int nborders;             /* flux borders (QSF_OBS_FLUX)                     */
  int border_types[QSF_MAX_BORDERS];
  int64_t box_size;         /* BOX<size> parameter                             */
  double state_accuracy;    /* IM convergence threshold (0: run all nsteps)    */
  double last_energy;       /* E before the first step of this call            */
  int energy_after_normalize; /* bit 0: epot, bit 1: ekin seen after Normalize */
  /* diagnostics: when non-NULL, every launch is bracketed by CUDA events on the
   * grid's stream (no graph) and its device time in ms is added to
   * kernel_ms[QSF_K_*]; kernel_launches[QSF_K_*] counts the launches. */
  float* kernel_ms;
  int64_t* kernel_launches;
  int substeps;             /* MultiProductSplit order K (0 or 1: plain Strang) */
  /* QSF_OBS_EKIN on every k-th step only (k = ekin_interval; 0 or 1: every step), as
   * the reference's comp_interval records rows every k steps (wf/buffer.h:6, 391):
   * E_kin (rows' column 2) is computed at the end of steps k-1, 2k-1, ... of the call
   * and of its last step, and is 0 in the other rows.  E_kin needs psi_n in memory for
   * its extra transforms, so those steps end in complex128 while the steps between
   * them stay in fixed point.  With a convergence threshold in imaginary time the
   * energy test runs on the steps that have E_kin (E_n minus the previous such E). */
  int ekin_interval;
} qsf_step_desc;
/* kernel kinds of the fused step (for qsf_step_desc.kernel_ms) */
#define QSF_K_TABLES 0
#define QSF_K_ROW_OPEN 1
#define QSF_K_AXIS_FWD 2
#define QSF_K_AXIS_FPI 3
#define QSF_K_AXIS_INV 4
#define QSF_K_ROW_CLOSE 5
#define QSF_K_AXIS_EKIN 6
#define QSF_K_FINALIZE 7
#define QSF_K_LINE_STEP 8
#define QSF_K_COUNT 9
int qsf_step(qsf_grid* g, const qsf_step_desc* d, double* rows, int64_t* steps_done);

/* ------------------------------------------------------------- batching */
/* Many independent solves (grids of different sizes, each with its own step program
 * and pulse) advanced together: solves sharing (dim, line length) form a group, and
 * one launch per split stage covers every solve of a group; all groups' launches for
 * one step are captured once into a CUDA graph and replayed.  Each solve stops at its
 * own nsteps; results are identical to running it alone through qsf_step (the
 * per-solve work and reduction order do not depend on the batch).  There is no
 * counterpart in the reference, which runs one solve per process group. */
typedef struct qsf_batch qsf_batch;
int qsf_batch_create(void* stream, qsf_batch** out);
/* Destroying a batch leaves its member grids alive and out of any batch. */
int qsf_batch_destroy(qsf_batch* b);
/* Adds grid g (owned by the caller) with the step program d (coupling rows are copied
 * at this call).  d->kernel_ms is ignored.  A grid is in at most one batch
 * (QSF_ESTATE otherwise); qsf_grid_destroy of a member removes it from its batch
 * first, so a later qsf_batch_run does not touch its memory. */
int qsf_batch_add(qsf_batch* b, qsf_grid* g, const qsf_step_desc* d, int64_t* slot);
/* Removes a member; applies its pending Normalize factor first. */
int qsf_batch_remove(qsf_batch* b, int64_t slot);
/* Advances every member by up to `steps` steps; *active = members with steps left.
 * Returns QSF_ENUMERIC when any member's wavefunction held an Inf / NaN or its norm
 * became non-positive (the other members are unaffected: qsf_batch_result says which). */
int qsf_batch_run(qsf_batch* b, int64_t steps, int64_t* active);
/* Observables rows (nsteps x (3 + nborders)) and steps done of one member; returns
 * QSF_ENUMERIC (rows still filled) for a member flagged as above. */
int qsf_batch_result(qsf_batch* b, int64_t slot, double* rows, int64_t* steps_done);

/* -------------------------------------------------------------- serving */
/* A request loop with continuous batching: submitted solves wait in a queue, are
 * admitted while a slot is free and enough HBM stays free, join the running batch
 * between rounds of steps (their wavefunctions stay resident on the device for the
 * whole solve), and leave it when their last step is done, returning yields, flux
 * integrals and latencies.  Admissions are prepared while a round runs.  Solves of
 * axis lengths outside the built kernel list run beside the batch, each on its own
 * stream, as graph-replayed member-operation programs.  No counterpart in the
 * reference. */
typedef struct qsf_request {
  qsf_grid_desc grid;
  int mode;                 /* QSF_MODE_RE or QSF_MODE_IM                               */
  double dt;
  int64_t nsteps;
  const double* coupling;   /* nsteps x (3 | 6) rows as for qsf_step; copied at submit   */
  const double* psi0;       /* initial wavefunction (host, m complex); copied at submit;
                               NULL: gaussian(0, 1) normalised (wf/preset.h:5-10)          */
  uint32_t obs;             /* QSF_OBS_* as for qsf_step                                  */
  int nborders;
  int border_types[QSF_MAX_BORDERS];
  int64_t box_size;
} qsf_request;

typedef struct qsf_result {
  int status;               /* QSF_OK or the error that ended the solve                   */
  int64_t steps;            /* steps run                                                   */
  double final_norm;        /* <psi|psi> dV after the last step                           */
  double yield;             /* 1 - final_norm: probability absorbed at the grid edge       */
  double final_epot;        /* <psi|V|psi> dV after the last step                          */
  double flux_integral[QSF_MAX_BORDERS]; /* sum over steps of flux_b * dt                 */
  double queue_s;           /* submit -> admission                                          */
  double latency_s;         /* submit -> completion                                         */
} qsf_result;

typedef struct qsf_server_config {
  int max_slots;            /* solves resident at once                                    */
  double hbm_reserve_gb;    /* admission keeps at least this much device memory free      */
  int64_t steps_per_round;  /* steps between admission / completion checks                */
  int queue_capacity;       /* pending requests; submit returns QSF_EBUSY beyond it       */
} qsf_server_config;

typedef struct qsf_server_stats {
  int64_t submitted, admitted, completed, queued, in_flight;
  double grid_point_steps;  /* completed solves: sum of m * steps                          */
} qsf_server_stats;

typedef struct qsf_server qsf_server;
/* The server's worker thread runs on the calling thread's current device at start
 * (one process per GPU selects its device first). */
int qsf_server_start(const qsf_server_config* cfg, qsf_server** out);
int qsf_server_submit(qsf_server* s, const qsf_request* r, int64_t* ticket);
/* Admission: a request is admitted while a slot is free and its device bytes fit in
 * the free HBM minus hbm_reserve_gb; one that fits on the device but not now waits in
 * the queue (requests behind it wait too); one larger than the device's total memory
 * minus the reserve finishes at once with status QSF_ENOMEM.  A solve whose
 * wavefunction holds an Inf / NaN (or whose norm turns non-positive) finishes with
 * QSF_ENUMERIC without affecting the others.
 * A finished solve's result is handed out once, by qsf_server_poll (done = 1) or
 * qsf_server_wait, and then forgotten (the server keeps no unbounded result history);
 * later calls for that ticket see it as unknown (poll: done = 0; wait: timeout). */
/* non-blocking: *done = 1 and *out filled once the solve has finished */
int qsf_server_poll(qsf_server* s, int64_t ticket, qsf_result* out, int* done);
/* bounded wait for one solve; QSF_ETIMEDOUT when timeout_s runs out */
int qsf_server_wait(qsf_server* s, int64_t ticket, double timeout_s, qsf_result* out);
/* Cancels a submitted solve: a queued one leaves the queue at once, a running one
 * leaves the batch after the current round; its result (status QSF_ECANCELED, the
 * observables of the steps done) is then collected as usual.  QSF_EINVAL for a ticket
 * that is unknown or already finished. */
int qsf_server_cancel(qsf_server* s, int64_t ticket);
int qsf_server_stats_get(qsf_server* s, qsf_server_stats* out);
/* finishes the solves in flight, drops the queued ones (status QSF_ESTATE), joins */
int qsf_server_stop(qsf_server* s);

/* ------------------------------------------------- other LocalGrid members */
/* average_der<X, dir, PotentialEnergy> (grid.h:443-465), the AVG<DERIVATIVE<dir,
 * PotentialEnergy>> output (computations.h:73, propagator.h:242-247):
 * sum |psi|^2 (V(x + dx e_dir) - V(x - dx e_dir)) dV / (2 dx_dir). */
int qsf_average_der(qsf_grid* g, int dir, double* out);
/* operation<M, R, AntiSymmetrize<particles>> (grid.h:611-723) on one rank:
 * particles 2 in 2D: psi(x, y) -= psi(y, x); particles 2 in 3D: the same for the last
 * two coordinates, psi(x, y, y) = 0; particles 3 in 3D: the full antisymmetrisation,
 * zero wherever two coordinates coincide.  Other combinations leave psi unchanged. */
int qsf_antisymmetrize(qsf_grid* g, int particles);

/* ------------------------------------------------------ wavefunction files */
/* .psi files with the layout of the reference's LocalGrid (grid.h:1025-1035):
 * dim u8 | rep u8 | complex u8 | downscale i64 | n[dim] i64 | dx[dim] f64 |
 * bounded[dim] u8 | payload.  Paths are relative to the process's working directory,
 * as in the reference. */
typedef struct qsf_dump_format { /* DUMP_FORMAT, enums.h:157-164 */
  int rep;            /* QSF_REP_X or QSF_REP_P (P: centred by the (-1)^(i0+i1+..) shift) */
  int complex_values; /* 1: complex128 payload; 0: |psi|^2 (float64) */
  int64_t downscale;  /* >= 1 and dividing every axis; > 1 stores |psi|^2 block sums */
  int evo_backup;     /* 1: raw psi, no name suffixes (evolution backups) */
} qsf_dump_format;
/* save / _save_centered / _save / coarse (grid.h:955-1114): writes
 * base[_scale<d>]_rep{X,P}<ext> (no suffixes for evo_backup) and returns the path in
 * path_out (may be NULL).  A P-representation save transforms psi and back, as the
 * reference does. */
int qsf_save(qsf_grid* g, const char* base, const qsf_dump_format* df, const char* ext, char* path_out,
             size_t path_cap);
/* load / _load (grid.h:789-859): reads base<ext> into psi.  A file of the wrong
 * dimensionality is QSF_EINVAL.  warnings (may be NULL) gets bit 0: n differs,
 * bit 1: dx differs, bit 2: file holds |psi|^2 (each element becomes its modulus, as
 * the reference reads it), bit 3: file shorter than the grid.  norm (may be NULL)
 * gets <psi|psi> dV after loading. */
int qsf_load(qsf_grid* g, const char* base, const char* ext, int* warnings, double* norm);
/* orthogonalizeWith (grid.h:909-946): psi -= <psi_f|psi> dV psi_f for the complex
 * wavefunction psi_f in base<ext>; overlap2 (may be NULL) gets <psi_f|psi> dV as
 * (re, im), norm the norm afterwards.  The payload is read after the header the file
 * actually has (the reference's offset arithmetic is 3 bytes short, grid.h:917-918). */
int qsf_orthogonalize_with(qsf_grid* g, const char* base, const char* ext, double* overlap2, double* norm);
/* _backup (grid.h:1116-1126): backup.info (int64 step) and backup<ext> (raw psi) */
int qsf_backup(qsf_grid* g, int64_t step, const char* ext);
/* restore (grid.h:949-953) plus the step read from backup.info (propagator.h:424-428);
 * step may be NULL */
int qsf_restore(qsf_grid* g, const char* ext, int64_t* step);
/* remove_backups (grid.h:1128-1132) */
int qsf_remove_backups(const char* ext);

/* ------------------------------------------------- norm without allocation */
/* No counterpart in the reference.  For callers that cannot allocate device memory
 * (a host program that hands out all device memory from its own pool, a language
 * runtime that may only pass buffers it already owns across its foreign-function
 * boundary): computes <psi|psi> dV of a complex128 wavefunction of m points that the
 * caller holds on the device (psi_dev, interleaved re/im) and writes the one double
 * into out_dev, a device buffer the caller owns.  Launches on `stream` (NULL: the
 * default stream) and returns without waiting.  It allocates nothing: the per-block
 * partial sums live in a fixed 64 KiB device array inside the library, which every
 * GPU that loads the library holds until the process exits.  m may be at most
 * 134,217,728 points; larger m returns QSF_EINVAL.  All calls share that array, so
 * calls that overlap on the GPU race and must be serialised by the caller.  The first
 * call on a device looks up the array's address (with that device current); make it
 * before any stream capture. */
int qsf_norm_noalloc(const double* psi_dev, int64_t m, double dV, double* out_dev, void* stream);

/* ------------------------------------------------------------ diagnostics */
/* last CUDA error text seen by the library (thread-local, never NULL) */
const char* qsf_last_error(void);
/* FFT radices chosen for a line of n points (for tests and the autotuner) */
int qsf_fft_plan_radices(int64_t n, int* radices, int* count);

#ifdef __cplusplus
}
#endif
#endif /* QSF_GPU_H */
