// The reference's own propagator driving the GB300 grid: a user program written
// against the reference's API (QSF.h, unmodified), with only the grid type changed
// to QSF::GPU::CAP<2>.  Imaginary-time ground state, then a real-time run under a
// sin^2 pulse in the velocity gauge with ZOA_FLUX_2D fluxes, all through the
// reference's SplitPropagator::run.
#include "QSF.h"
#include "qsf_gpu_localgrid.hpp"

using namespace QSF;
using GType = GPU::CAP<2>;
using Eberly = ReducedDimInteraction<ReducedModel::Eberly>;
using F = Field<AXIS::XY, Sin2Envelope<SinPulse>>;
using Split = MultiProductSplit<Split3Base<REP::X, REP::P, REP::X>, 1>;

int main(int argc, char** argv) {
  MPI::init(argc, argv);
  const ind n = argc > 1 ? atoi(argv[1]) : 64;
  GType grid(0.3, n, n / 10);
  Eberly pot(InteractionBase{2.0, -1.0, 1.0, 1.0});
  using HamIM = Schrodinger::Spin0<GType, Eberly>;
  HamIM wf(grid, pot);
  wf.addUsingCoordinateFunction([](auto... x) { return gaussian(0.0, 1.0, x...); });
  SplitPropagator<MODE::IM, Split, HamIM> im(PropagatorBase{.dt = 0.01, .max_steps = 50, .state_accuracy = 0.0},
                                             std::move(wf), "IM");
  using IMOuts = BufferedBinaryOutputs<VALUE<Step>, AVG<Identity>, OPERATION<Normalize>, AVG<PotentialEnergy>,
                                      AVG<KineticEnergy>, ENERGY_TOTAL, ENERGY_DIFFERENCE>;
  im.run(IMOuts(BufferedOutputsBase{1, 1}));
  // .psi files of the ground state: X and centred P representation, a snapshot, an
  // evolution backup read back, and a projection onto the saved state
  im.wf.save("ground");
  im.wf.save("ground", DUMP_FORMAT{.dim = 2, .rep = REP::P});
  im.wf.snapshot("_ground");
  im.wf.backup(0);
  im.wf.restore();
  im.wf.remove_backups();
  _FieldConfig fc{.field = 0.1, .omega = 1.0, .ncycles = 1.0, .FWHM_percent = 0, .phase_in_pi_units = 0,
                  .delay_in_cycles = 0};
  using C = DipoleCoupling<VelocityGauge, F>;
  using HamRE = Schrodinger::Spin0<GType, Eberly, C>;
  HamRE wre(grid, pot, C(F(Sin2Envelope<SinPulse>(fc))));
  SplitPropagator<MODE::RE, Split, HamRE> re(PropagatorBase{.dt = 0.05, .max_steps = 0, .state_accuracy = 0},
                                             std::move(wre), "RE");
  // the real-time run starts from the ground state (operator[] copies, element by element)
  for (ind i = 0; i < re.wf.localSize(); ++i) re.wf[i] = im.wf[i];
  // other members on the ground state: the potential's derivative observable and the
  // exchange antisymmetrisation
  const double dVdx = im.wf.template average_der<REP::X, 0, PotentialEnergy>();
  im.wf.template operation<MODE::IM, REP::X, AntiSymmetrize<2>>();
  printf("<dV/dx0> of the ground state: %.17e\n", dVdx);
  using REOuts = BufferedBinaryOutputs<VALUE<Step, Time>, AVG<Identity>, AVG<PotentialEnergy>, ZOA_FLUX_2D>;
  re.run(REOuts(BufferedOutputsBase{1, 1}));
  re.wf.orthogonalizeWith("ground_repX");
  printf("norm after the pulse: %.17e\n", re.wf.template average<REP::X, Identity>());
  return 0;
}
