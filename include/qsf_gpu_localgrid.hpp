// qsf_gpu_localgrid.hpp -- the GB300 grid as a drop-in for the reference's LocalGrid.
//
// Include after the reference's QSF.h.  Replacing the grid type of a Spin0
// Hamiltonian,
//
//     using GType = QSF::CAP<QSF::CartesianGrid<2>>;          // reference, CPU
//     using GType = QSF::GPU::CAP<2>;                          // this header, GPU
//
// selects the LocalGrid partial specialisation below, so the reference's own
// SplitPropagator (include/propagator.h) runs unmodified while every member it calls
// -- fourier, evolve, average, operation<Normalize>, flux -- executes as CUDA kernels
// through the C ABI of libqsfgpu.so (include/qsf_gpu.h).  The wavefunction lives on
// the device; operator[] and addUsingCoordinateFunction see a host copy that is kept
// coherent lazily (downloaded on first host access after device work, uploaded
// before the next device call after host access).  Copies of the grid share one
// device state, as the reference's member-wise copy shares psi (propagator.h:115).
//
// The propagator's FLUX path (propagator.h:259-265) still loops over every point on
// the host for the velocity-gauge correction; the fluxes themselves are computed on
// the device.  For full speed use the fused qsf_step path instead.
#pragma once
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "qsf_gpu.h"

namespace QSF {
namespace GPU {

// Stands in for MPI::Regions: one region, the whole grid on one GPU.  It sets up the
// communicators a one-region run of one rank would have (MPI::Regions,
// basics/mpi_logic.h:140-175 splits MPI_COMM_WORLD into them), because the reference's
// propagator reduces some values itself (MPI::reduceImmediataly over MPI::rComm,
// propagator.h:225, basics/mpi_logic.h:76-83); left unset, rComm is a null communicator.
template <DIMS D> struct Region {
  using MPIDivision = MPI::Slices;
  static constexpr bool many = false;
  static bool calcsEnabled() { return true; }
  bool isMain = true;
  bool bounded[D];
  AXIS freeCoord = AXIS::NO;
  Region() {
    for (DIMS i = 0; i < D; ++i) bounded[i] = true;
    if (MPI::rComm == MPI_Comm()) {
      MPI::gComm = MPI::rComm = MPI::eComm = MPI_COMM_WORLD;
      MPI::gID = MPI::rID = MPI::eID = 0;
      MPI::gSize = MPI::rSize = MPI::eSize = 1;
    }
  }
};

// CAP<CartesianGrid<D>> for the GPU grid: same geometry (coords.h:14-139), same
// absorber parameters (absorbers.h:27-35).
template <DIMS D> struct CAP : CartesianGrid_<D, Region<D>>, AbsorberType {
  using Base = CartesianGrid_<D, Region<D>>;
  ind nCAP;
  CAP(Base base, ind nCAP) : Base(base), nCAP(nCAP) {}
  CAP(double dx, ind n, ind nCAP) : Base(dx, n), nCAP(nCAP) {}
};

inline void check(int rc, const char* where) {
  if (rc != QSF_OK) throw std::runtime_error(std::string(where) + ": " + qsf_last_error());
}

template <class V> struct potential_kind;
template <> struct potential_kind<ReducedDimInteraction<ReducedModel::Eberly>> {
  static constexpr int value = QSF_POT_EBERLY;
};
template <> struct potential_kind<ReducedDimInteraction<ReducedModel::EckhardSacha>> {
  static constexpr int value = QSF_POT_ECKHARDT_SACHA;
};
template <> struct potential_kind<CoulombInteraction> {
  static constexpr int value = QSF_POT_COULOMB;
};

// border type -> (QSF_B_* id, BOX size)
template <class B> struct border_id;
template <int S> struct border_id<BOX<S>> {
  static constexpr int id = QSF_B_BOX, box = S;
};
#define QSF_GPU_BORDER(T, ID)            \
  template <> struct border_id<T> {      \
    static constexpr int id = ID, box = 0; \
  };
QSF_GPU_BORDER(S2CAP, QSF_B_S2CAP)
QSF_GPU_BORDER(D2CAP, QSF_B_D2CAP)
QSF_GPU_BORDER(N2S, QSF_B_N2S)
QSF_GPU_BORDER(N2D, QSF_B_N2D)
QSF_GPU_BORDER(N2D_SYM, QSF_B_N2D_SYM)
QSF_GPU_BORDER(N2D_ASYM, QSF_B_N2D_ASYM)
QSF_GPU_BORDER(S2D, QSF_B_S2D)
QSF_GPU_BORDER(S2D_SYM, QSF_B_S2D_SYM)
QSF_GPU_BORDER(S2D_ASYM, QSF_B_S2D_ASYM)
QSF_GPU_BORDER(N2T, QSF_B_N2T)
QSF_GPU_BORDER(S2T, QSF_B_S2T)
QSF_GPU_BORDER(D2T, QSF_B_D2T)
QSF_GPU_BORDER(T2CAP, QSF_B_T2CAP)
#undef QSF_GPU_BORDER

template <DIMS D> struct State {
  qsf_grid* g = nullptr;
  std::vector<cxd> host;
  bool host_newer = true;  // the host copy holds the latest values (fresh grids start at zero)
  bool dev_newer = false;  // the device holds values the host copy has not seen
  std::vector<borVec<D>> curr;
  ~State() {
    if (g) qsf_grid_destroy(g);
  }
};

}  // namespace GPU

template <class Hamiltonian, DIMS D, uind Components, class MPI_GC>
struct LocalGrid<Hamiltonian, GPU::CAP<D>, Components, MPI_GC, MPI::Slices, false> : GPU::CAP<D> {
  using BaseGrid = GPU::CAP<D>;
  using BaseGrid::DIM;
  using BaseGrid::dx;
  using BaseGrid::n;
  using MPIGridComm = MPI_GC;
  static constexpr auto indices = n_seq<DIM>;
  static constexpr bool hasAbsorber = true;

  MPIGridComm mcomm;
  const ind m = BaseGrid::m * Components;
  ind m_l = BaseGrid::m * Components;
  std::shared_ptr<GPU::State<D>> st;
  cxd* psi = nullptr;  // host copy (operator[], initial conditions)

  explicit LocalGrid(BaseGrid g) : BaseGrid(g), mcomm(), st(std::make_shared<GPU::State<D>>()) {
    st->host.assign((size_t)m, cxd(0.0, 0.0));
    psi = st->host.data();
  }

  Hamiltonian& ham() { return *static_cast<Hamiltonian*>(this); }

  // create the device grid on first use (the Hamiltonian's potential and coupling are
  // constructed after this base class)
  qsf_grid* grid() {
    if (!st->g) {
      qsf_grid_desc d{};
      d.dim = DIM;
      for (DIMS k = 0; k < DIM; ++k) {
        d.n[k] = n[k];
        d.dx[k] = dx[k];
      }
      d.nCAP = BaseGrid::nCAP;
      using V = std::decay_t<decltype(ham()._potential)>;
      d.potential = GPU::potential_kind<V>::value;
      d.Ncharge = ham()._potential.Ncharge;
      d.Echarge = ham()._potential.Echarge;
      d.Nsoft = ham()._potential.Nsoft;
      d.Esoft = ham()._potential.Esoft;
      d.gauge = Hamiltonian::couplesInRep == REP::P ? QSF_GAUGE_VELOCITY : QSF_GAUGE_LENGTH;
      using C = std::decay_t<decltype(ham()._coupling)>;
      d.n_fields = (int)C::size;
      d.p_axis_swap = DIM > 1;
      d.border_nodes[0] = p_NS;
      d.border_nodes[1] = p_SD;
      d.border_nodes[2] = p_DT;
      d.border_nodes[3] = p_CAP;
      GPU::check(qsf_grid_create(&d, nullptr, &st->g), "qsf_grid_create");
    }
    return st->g;
  }
  // host copy -> device, if the host copy is newer
  void push() {
    qsf_grid* g = grid();
    if (st->host_newer) {
      GPU::check(qsf_upload(g, reinterpret_cast<const double*>(st->host.data()), m), "qsf_upload");
      st->host_newer = false;
    }
    st->dev_newer = true;
  }
  // device -> host copy, if the device is newer
  void pull() {
    if (st->dev_newer && st->g) {
      GPU::check(qsf_download(st->g, reinterpret_cast<double*>(st->host.data()), m), "qsf_download");
      st->dev_newer = false;
    }
  }

  cxd& operator[](ind i) {
    pull();
    st->host_newer = true;
    return st->host[(size_t)i];
  }
  ind localSize() { return m; }

  // fourier<R>() (grid.h:369-378)
  template <REP R> void fourier() {
    push();
    GPU::check(qsf_fourier(grid(), R == REP::P ? QSF_REP_P : QSF_REP_X), "qsf_fourier");
  }
  template <REP R, OPTIMS O> void precalc(double time) { ham()._coupling.precalc(time); }

  template <REP R> void coupling_values(double* cv) {
    cv[0] = cv[1] = cv[2] = 0.0;
    using C = std::decay_t<decltype(ham()._coupling)>;
    if constexpr (C::size > 0)
      if (Hamiltonian::couplesInRep == R)
        for (DIMS k = 0; k < DIM; ++k) cv[k] = ham()._coupling[getAxis(k)];
  }

  // evolve<M, R>(delta) (grid.h:394-423)
  template <MODE M, REP R> void evolve(double delta) {
    push();
    double cv[3];
    coupling_values<R>(cv);
    GPU::check(qsf_evolve(grid(), M == MODE::IM ? QSF_MODE_IM : QSF_MODE_RE, R == REP::X ? QSF_REP_X : QSF_REP_P,
                          delta, cv),
               "qsf_evolve");
  }

  // average<R, Op>() (grid.h:425-441)
  template <REP R, class Op> double average() {
    push();
    int op = QSF_OP_IDENTITY;
    if constexpr (std::is_same_v<Op, PotentialEnergy>) op = QSF_OP_POTENTIAL;
    if constexpr (std::is_same_v<Op, KineticEnergy>) op = QSF_OP_KINETIC;
    double out = 0.0;
    GPU::check(qsf_average(grid(), R == REP::X ? QSF_REP_X : QSF_REP_P, op, &out), "qsf_average");
    return out;
  }

  // current_map() (grid.h:519-528): the propagator adds its velocity-gauge correction
  // to this host array; flux<R, B>() below recomputes current, correction and border
  // sum on the device, so the array only has to exist.
  borVec<DIM>* current_map() {
    if (st->curr.size() != (size_t)m) st->curr.assign((size_t)m, borVec<DIM>());
    return st->curr.data();
  }

  // flux<R, B>() (grid.h:559-573) with the propagator's velocity-gauge correction
  // (propagator.h:249-257) done on the device
  template <REP R, class B> double flux() {
    push();
    double A[3];
    coupling_values<REP::P>(A);
    const int id = GPU::border_id<B>::id;
    double out = 0.0;
    GPU::check(qsf_flux(grid(), Hamiltonian::couplesInRep == REP::P ? A : nullptr, 1, &id, GPU::border_id<B>::box,
                        &out),
               "qsf_flux");
    return out;
  }

  // operation<M, R, Op>() (grid.h:599-723): Normalize, AntiSymmetrize<2|3>
  template <MODE M, REP R, class Op> void operation() {
    if constexpr (std::is_same_v<Op, Normalize>) {
      push();
      GPU::check(qsf_normalize(grid(), nullptr), "qsf_normalize");
    }
    if constexpr (std::is_same_v<Op, AntiSymmetrize<2>>) {
      push();
      GPU::check(qsf_antisymmetrize(grid(), 2), "qsf_antisymmetrize");
    }
    if constexpr (std::is_same_v<Op, AntiSymmetrize<3>>) {
      push();
      GPU::check(qsf_antisymmetrize(grid(), 3), "qsf_antisymmetrize");
    }
  }

  // average_der<R, dir, Op>() (grid.h:443-465) for the potential
  template <REP R, uind dir, class Op> double average_der() {
    static_assert(std::is_same_v<Op, PotentialEnergy>, "derivative observables are built for the potential");
    push();
    double out = 0.0;
    GPU::check(qsf_average_der(grid(), (int)dir, &out), "qsf_average_der");
    return out;
  }

  void maskRegion() {
    push();
    int b[3] = {1, 1, 1};
    for (DIMS k = 0; k < DIM; ++k) b[k] = mcomm.bounded[k];
    GPU::check(qsf_mask_region(grid(), b), "qsf_mask_region");
  }

  template <class Op> double getValue() { return ham()._coupling.template getValue<Op>(); }
  template <MODE M, REP R, class BO, class COMP> void compute(BO& bo, COMP&& c) {
    bo.template store<M, COMP>(1.0);
  }
  void postCompute() {}

  // .psi files (grid.h:948-1153), written and read by the library
  static qsf_dump_format dump_of(const DUMP_FORMAT& df) {
    return qsf_dump_format{df.rep == REP::P ? QSF_REP_P : QSF_REP_X, df.complex ? 1 : 0, (int64_t)df.downscale,
                           df.evo_backup ? 1 : 0};
  }
  IO::path save(IO::path file_sub_path = "", DUMP_FORMAT df = {.dim = DIM}) {
    push();
    const qsf_dump_format f = dump_of(df);
    char out[4096];
    GPU::check(qsf_save(grid(), file_sub_path.c_str(), &f, IO::psi_ext, out, sizeof out), "qsf_save");
    return std::filesystem::current_path() / out;
  }
  void load(IO::path input_path) {
    push();
    GPU::check(qsf_load(grid(), input_path.c_str(), IO::psi_ext, nullptr, nullptr), "qsf_load");
  }
  void backup(const ind step) {
    push();
    GPU::check(qsf_backup(grid(), step, IO::psi_ext), "qsf_backup");
  }
  void restore() {
    push();
    GPU::check(qsf_restore(grid(), IO::psi_ext, nullptr), "qsf_restore");
  }
  void remove_backups() { GPU::check(qsf_remove_backups(IO::psi_ext), "qsf_remove_backups"); }
  void snapshot(std::string extra_info, DUMP_FORMAT df = {.dim = DIM}) {
    static ind x_count = 0;
    static ind p_count = 0;
    ind& count = df.rep == REP::X ? x_count : p_count;
    push();
    const qsf_dump_format f = dump_of(df);
    const std::string ext = std::string(IO::psi_ext) + std::to_string(MPI::region);
    GPU::check(qsf_save(grid(), ("snapshot_" + std::to_string(count) + extra_info).c_str(), &f, ext.c_str(),
                        nullptr, 0),
               "qsf_save");
    count++;
  }
  void orthogonalizeWith(IO::path input_path, std::string ext = IO::psi_ext) {
    push();
    GPU::check(qsf_orthogonalize_with(grid(), input_path.c_str(), ext.c_str(), nullptr, nullptr),
               "qsf_orthogonalize_with");
  }

  // addUsingCoordinateFunction (grid.h:775-778): psi += f(x...) on the host copy
  template <class F, REP R = REP::X> void addUsingCoordinateFunction(F&& f) {
    pull();
    add_<F, R>(std::forward<F>(f), indices);
    st->host_newer = true;
  }
  template <class F, REP R, uind... Is> void add_(F&& f, seq<Is...>) {
    ind c[DIM + 1] = {0};
    for (ind p = 0; p < m; ++p) {
      ind r = p;
      for (int k = DIM - 1; k >= 0; --k) {
        c[k] = r % n[k];
        r /= n[k];
      }
      st->host[(size_t)p] += f(BaseGrid::template pos<R, Is>(c[Is])...);
    }
  }
};

}  // namespace QSF
