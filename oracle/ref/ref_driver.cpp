// Oracle harness: runs the reference's own header-only implementation (QSF.h, compiled
// unmodified from the reference checkout) on small seeded cases and writes its outputs
// (the reference's binary .dat rows and raw complex128 wavefunctions) so that the CPU
// restatement in oracle/qsf_oracle.c and the GPU path can be pinned against it.
//
// Test infrastructure only.  Built by oracle/Makefile (target `ref`) into oracle/_ref/
// against the MPI and FFTW stand-ins in oracle/ref/shim/.
//
// Usage: qsf_ref <case> <outdir> key=value ...
//   cases: prim2d, prim3d, c1 (1D IM + RE), c2 (2D IM + RE VG), c3 (3D RE LG),
//          io1 / io2 / io3 (.psi save / load / backup / orthogonalizeWith / snapshot),
//          mp (1D real time with MultiProductSplit of order 2 and 3, VG and LG),
//          as2 / as3 (average_der of the potential, AntiSymmetrize<2> and <3>),
//          mg1 / mg2 / mg3 (multi-region grid, one process per region: QSF_SHIM_NP=2^D)
#include "QSF.h"

#include <map>
#include <string>

using namespace QSF;

// The reference declares LengthGauge (coupling.h:9-11) but never specialises
// DipoleCoupling for it.  The harness defines it the way the velocity-gauge
// specialisation is written (coupling.h:101-118): the fields are used as E(t)
// directly (no promotion to A) and the coupling acts in X:  H_int = x . E(t).
namespace QSF {
template <class... Fields>
struct DipoleCoupling<LengthGauge, Fields...> : CouplingBase<DipoleApprox, Fields...> {
  using base = CouplingBase<DipoleApprox, Fields...>;
  static constexpr REP couplesInRep = REP::X;
  DipoleCoupling(Fields&&... fields) : base(std::forward<Fields>(fields)...) {}
  template <class F> double getValue() { return base::template getValue<F>(); }
};
}  // namespace QSF

static std::map<std::string, double> P;
static double par(const char* k, double def) {
  auto it = P.find(k);
  return it == P.end() ? def : it->second;
}

static void dump(const std::string& path, const cxd* psi, ind m) {
  FILE* f = fopen(path.c_str(), "wb");
  fwrite(psi, sizeof(cxd), (size_t)m, f);
  fclose(f);
}

// splitmix64 -> uniform [-1, 1)
static uint64_t g_state = 0;
static double urand() {
  uint64_t z = (g_state += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  z = z ^ (z >> 31);
  return (double)(z >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}

static void set_borders() {
  p_NS = (ind)par("p_NS", 25);
  p_SD = (ind)par("p_SD", 14);
  p_DT = (ind)par("p_DT", 10);
  p_CAP = (ind)par("p_CAP", 40);
}

static _FieldConfig field_cfg() {
  return _FieldConfig{.field = par("F0", 0.05),
                      .omega = par("omega", 0.057),
                      .ncycles = par("ncycles", 2.0),
                      .FWHM_percent = 0.0,
                      .phase_in_pi_units = par("phase", 0.0),
                      .delay_in_cycles = par("delay", 0.0)};
}

using Sin2 = Sin2Envelope<SinPulse>;
using Split = MultiProductSplit<Split3Base<REP::X, REP::P, REP::X>, 1>;

template <DIMS D> using CapGrid = CAP<CartesianGrid<D>>;
using Eberly = ReducedDimInteraction<ReducedModel::Eberly>;

template <DIMS D> CapGrid<D> make_grid() {
  return CapGrid<D>(CartesianGrid<D>(par("dx", 0.2), (ind)par("n", 64)), (ind)par("nCAP", 6));
}
static Eberly make_pot() {
  return Eberly(InteractionBase{par("Ncharge", 1.0), par("Echarge", -1.0), par("Nsoft", 1.0), par("Esoft", 1.0)});
}

// ---------------------------------------------------------------- primitives
template <DIMS D> static void prim(const std::string& out) {
  using F = Field<AXIS::XYZ, ConstantPulse>;
  using HamLG = Schrodinger::Spin0<CapGrid<D>, Eberly, DipoleCoupling<LengthGauge, F>>;
  using HamVG = Schrodinger::Spin0<CapGrid<D>, Eberly, DipoleCoupling<VelocityGauge, F>>;
  _FieldConfig fc{.field = par("F0", 0.11), .omega = 1.0, .ncycles = 100.0, .FWHM_percent = 0,
                  .phase_in_pi_units = 0, .delay_in_cycles = 0};
  HamLG lg(make_grid<D>(), make_pot(), DipoleCoupling<LengthGauge, F>(F(ConstantPulse(fc))));
  HamVG vg(make_grid<D>(), make_pot(), DipoleCoupling<VelocityGauge, F>(F(ConstantPulse(fc))));
  g_state = (uint64_t)par("seed", 1);
  ind m = lg.m_l;
  for (ind i = 0; i < m; i++) {
    double re = urand(), im = urand();
    lg[i] = cxd(re, im);
    vg[i] = cxd(re, im);
  }
  dump(out + "/psi_in.bin", &lg[0], m);
  FILE* fo = fopen((out + "/prim.bin").c_str(), "wb");
  auto put = [&](double v) { fwrite(&v, sizeof(double), 1, fo); };
  put(lg.template average<REP::X, Identity>());
  put(lg.template average<REP::X, PotentialEnergy>());
  // currents and every border flux on the input (no velocity-gauge term)
  {
    lg.current_map();
    put(lg.template flux<REP::X, BOX<3>>());
    put(lg.template flux<REP::X, S2CAP>());
    put(lg.template flux<REP::X, D2CAP>());
    put(lg.template flux<REP::X, N2S>());
    put(lg.template flux<REP::X, N2D>());
    put(lg.template flux<REP::X, S2D>());
    if constexpr (D == 2) {
      put(lg.template flux<REP::X, N2D_SYM>());
      put(lg.template flux<REP::X, N2D_ASYM>());
      put(lg.template flux<REP::X, S2D_SYM>());
      put(lg.template flux<REP::X, S2D_ASYM>());
    } else {
      put(lg.template flux<REP::X, N2T>());
      put(lg.template flux<REP::X, S2T>());
      put(lg.template flux<REP::X, D2T>());
      put(lg.template flux<REP::X, T2CAP>());
    }
  }
  // X evolution, real time, length gauge E = F0 at t = 0.5
  lg.template precalc<REP::X, OPTIMS::NONE>(0.5);
  lg.template evolve<MODE::RE, REP::X>(par("delta", 0.37));
  dump(out + "/psi_xre.bin", &lg[0], m);
  lg.template evolve<MODE::IM, REP::X>(par("delta", 0.37));
  dump(out + "/psi_xim.bin", &lg[0], m);
  // forward transform (P layout transposed for D > 1, as in the reference)
  lg.template fourier<REP::P>();
  dump(out + "/psi_p.bin", &lg[0], m);
  put(lg.template average<REP::P, KineticEnergy>());
  lg.template fourier<REP::X>();
  dump(out + "/psi_back.bin", &lg[0], m);
  // P evolution with the velocity gauge: A after precalc(0), precalc(1) = -F0
  vg.template fourier<REP::P>();
  vg.template precalc<REP::P, OPTIMS::NONE>(0.0);
  vg.template precalc<REP::P, OPTIMS::NONE>(1.0);
  vg.template evolve<MODE::RE, REP::P>(par("delta", 0.37));
  vg.template evolve<MODE::IM, REP::P>(par("delta", 0.37) * 0.25);
  vg.template fourier<REP::X>();
  dump(out + "/psi_pvg.bin", &vg[0], m);
  // Normalize
  vg.template operation<MODE::IM, REP::X, Normalize>();
  dump(out + "/psi_norm.bin", &vg[0], m);
  fclose(fo);
}

// ---------------------------------------------------------------- IM stage
template <DIMS D, class Outs>
static void run_im(const std::string& out, cxd* dst, ind m) {
  using HamIM = Schrodinger::Spin0<CapGrid<D>, Eberly>;
  HamIM wf(make_grid<D>(), make_pot());
  wf.addUsingCoordinateFunction([](auto... x) { return gaussian(0.0, 1.0, x...); });
  dump(out + "/im_psi0.bin", &wf[0], m);
  SplitPropagator<MODE::IM, Split, HamIM> im(
      PropagatorBase{.dt = par("im_dt", 0.01), .max_steps = (ind)par("im_steps", 100), .state_accuracy = 0.0},
      std::move(wf), "IM");
  im.run(Outs(BufferedOutputsBase{1, 1}), [&](WHEN when, ind, uind, auto& w) {
    if (when == WHEN::AT_END)
      for (ind i = 0; i < m; i++) dst[i] = w[i];
  });
  dump(out + "/im_psi.bin", dst, m);
}

using IMOuts = BufferedBinaryOutputs<VALUE<Step>, AVG<Identity>, OPERATION<Normalize>, AVG<PotentialEnergy>,
                                     AVG<KineticEnergy>, ENERGY_TOTAL, ENERGY_DIFFERENCE>;

template <class Coupling, class Outs, DIMS D>
static void run_re(const std::string& out, const cxd* src, ind m, Coupling&& c) {
  using Ham = Schrodinger::Spin0<CapGrid<D>, Eberly, std::decay_t<Coupling>>;
  Ham wf(make_grid<D>(), make_pot(), std::forward<Coupling>(c));
  SplitPropagator<MODE::RE, Split, Ham> re(PropagatorBase{.dt = par("re_dt", 0.05), .max_steps = 0, .state_accuracy = 0},
                                           std::move(wf), "RE");
  for (ind i = 0; i < m; i++) re.wf[i] = src[i];
  dump(out + "/re_psi0.bin", src, m);
  re.run(Outs(BufferedOutputsBase{1, 1}), [&](WHEN when, ind, uind, auto& w) {
    if (when == WHEN::AT_END) dump(out + "/re_psi.bin", &w[0], m);
  });
}

template <int BOXSZ> static void c1(const std::string& out) {
  ind n = (ind)par("n", 512);
  std::vector<cxd> psi((size_t)n);
  run_im<1, IMOuts>(out, psi.data(), n);
  using Outs = BufferedBinaryOutputs<VALUE<Step, Time>, AVG<Identity>, AVG<PotentialEnergy>, AVG<KineticEnergy>,
                                     FLUX<BOX<BOXSZ>>>;
  using F = Field<AXIS::X, Sin2>;
  if (par("lg", 0) != 0)
    run_re<DipoleCoupling<LengthGauge, F>, Outs, 1>(out, psi.data(), n,
                                                     DipoleCoupling<LengthGauge, F>(F(Sin2(field_cfg()))));
  else
    run_re<DipoleCoupling<VelocityGauge, F>, Outs, 1>(out, psi.data(), n,
                                                       DipoleCoupling<VelocityGauge, F>(F(Sin2(field_cfg()))));
}

static void c2(const std::string& out) {
  ind n = (ind)par("n", 64);
  ind m = n * n;
  std::vector<cxd> psi((size_t)m);
  run_im<2, IMOuts>(out, psi.data(), m);
  using Outs = BufferedBinaryOutputs<VALUE<Step, Time>, AVG<Identity>, AVG<PotentialEnergy>, AVG<KineticEnergy>,
                                     ZOA_FLUX_2D>;
  using F = Field<AXIS::XY, Sin2>;
  if (par("lg", 0) != 0)
    run_re<DipoleCoupling<LengthGauge, F>, Outs, 2>(out, psi.data(), m,
                                                     DipoleCoupling<LengthGauge, F>(F(Sin2(field_cfg()))));
  else
    run_re<DipoleCoupling<VelocityGauge, F>, Outs, 2>(out, psi.data(), m,
                                                       DipoleCoupling<VelocityGauge, F>(F(Sin2(field_cfg()))));
}

static void c3(const std::string& out) {
  ind n = (ind)par("n", 24);
  ind m = n * n * n;
  std::vector<cxd> psi((size_t)m);
  run_im<3, IMOuts>(out, psi.data(), m);
  using Outs = BufferedBinaryOutputs<VALUE<Step, Time>, AVG<Identity>, AVG<PotentialEnergy>, AVG<KineticEnergy>,
                                     ZOA_FLUX_3D>;
  using F = Field<AXIS::XYZ, Sin2>;
  if (par("lg", 1) != 0)
    run_re<DipoleCoupling<LengthGauge, F>, Outs, 3>(out, psi.data(), m,
                                                     DipoleCoupling<LengthGauge, F>(F(Sin2(field_cfg()))));
  else
    run_re<DipoleCoupling<VelocityGauge, F>, Outs, 3>(out, psi.data(), m,
                                                       DipoleCoupling<VelocityGauge, F>(F(Sin2(field_cfg()))));
}


// ---------------------------------------------------------------- multigrid
// Real-time run on the reference's multi-region grid (MultiCartesianGrid<D>: regions
// NO, X, (Y, XY, ...), multigrid.h) with one process per region (QSF_SHIM_NP = 2^D).
// The main region starts from seeded complex noise, the others from zero; each step
// ends with the region transfer and the region masks (postCompute, multigrid.h:617-657).
// Rank r (region r) writes psi_r<r>.bin; rank 0 also the main region's .dat rows.
template <DIMS D> using MGrid = CAP<MultiCartesianGrid<D>>;

template <DIMS D> static void mg(const std::string& out) {
  using F = Field<D == 1 ? AXIS::X : (D == 2 ? AXIS::XY : AXIS::XYZ), Sin2>;
  using C = DipoleCoupling<VelocityGauge, F>;
  using Ham = Schrodinger::Spin0<MGrid<D>, Eberly, C>;
  using Outs = BufferedBinaryOutputs<VALUE<Step, Time>, AVG<Identity>, AVG<PotentialEnergy>, AVG<KineticEnergy>>;
  MGrid<D> grid(MultiCartesianGrid<D>(par("dx", 0.3), (ind)par("n", 32)), (ind)par("nCAP", 4));
  Ham wf(grid, make_pot(), C(F(Sin2(field_cfg()))));
  SplitPropagator<MODE::RE, Split, Ham> re(PropagatorBase{.dt = par("re_dt", 0.05), .max_steps = 0, .state_accuracy = 0},
                                           std::move(wf), "RE");
  const ind m = re.wf.m_l;
  g_state = (uint64_t)par("seed", 1);
  std::vector<cxd> psi0((size_t)m);
  for (ind i = 0; i < m; i++) {
    const double a = urand(), b = urand();
    psi0[(size_t)i] = cxd(a, b);
  }
  for (ind i = 0; i < m; i++) re.wf[i] = MPI::region == 0 ? psi0[(size_t)i] : cxd(0.0, 0.0);
  if (MPI::region == 0) dump(out + "/psi_in.bin", psi0.data(), m);
  const std::string tag = "/psi_r" + std::to_string(MPI::region) + ".bin";
  re.run(Outs(BufferedOutputsBase{1, 1}), [&](WHEN when, ind, uind, auto& w) {
    if (when == WHEN::AT_END) dump(out + tag, &w[0], m);
  });
}

// ---------------------------------------------------------------- .psi I/O
// Writes the reference's .psi files (grid.h:948-1153) from a seeded state: X and P
// representation, complex and probability (doubles) payloads, downscale 2, the
// evolution backup, a snapshot; then loads files back into fresh grids and runs
// orthogonalizeWith, dumping the resulting wavefunctions.
template <DIMS D> static void io(const std::string& out) {
  using Ham = Schrodinger::Spin0<CapGrid<D>, Eberly>;
  Ham wf(make_grid<D>(), make_pot());
  const ind m = wf.m_l;
  g_state = (uint64_t)par("seed", 3);
  std::vector<cxd> psi0((size_t)m), psi1((size_t)m);
  for (ind i = 0; i < m; i++) psi0[(size_t)i] = cxd(urand(), urand());
  for (ind i = 0; i < m; i++) psi1[(size_t)i] = cxd(urand(), urand());
  auto set = [&](Ham& w, const std::vector<cxd>& v) {
    for (ind i = 0; i < m; i++) w[i] = v[(size_t)i];
  };
  set(wf, psi0);
  dump(out + "/psi_in.bin", psi0.data(), m);
  dump(out + "/psi_b.bin", psi1.data(), m);
  wf.save("sx");
  wf.save("sp", DUMP_FORMAT{.dim = D, .rep = REP::P});
  dump(out + "/psi_after_sp.bin", &wf[0], m);
  set(wf, psi0);
  wf.save("sd", DUMP_FORMAT{.dim = D, .rep = REP::X, .complex = true, .downscale = 2});
  wf.save("sdp", DUMP_FORMAT{.dim = D, .rep = REP::P, .complex = true, .downscale = 2});
  set(wf, psi0);
  wf.save("sn", DUMP_FORMAT{.dim = D, .rep = REP::X, .complex = false});
  wf.backup(7);
  wf.snapshot("_a");
  {
    Ham w2(make_grid<D>(), make_pot());
    set(w2, psi1);
    w2.load("sx_repX");
    dump(out + "/psi_load_sx.bin", &w2[0], m);
  }
  {
    Ham w3(make_grid<D>(), make_pot());
    set(w3, psi1);
    w3.load("sn_repX");
    dump(out + "/psi_load_sn.bin", &w3[0], m);
  }
  {
    Ham w4(make_grid<D>(), make_pot());
    set(w4, psi1);
    w4.orthogonalizeWith("sx_repX");
    dump(out + "/psi_orth.bin", &w4[0], m);
  }
}


// ---------------------------------------------------------------- multi-product
// Real-time 1D runs from the field-free Gaussian with MultiProductSplit<Split3Base, K>
// (splitting.h:63-91, propagator.h:331-413): final psi and the .dat rows.
template <size_t K, class Coupling>
static void mp_run(const std::string& out, const std::string& tag, Coupling&& c) {
  using Ham = Schrodinger::Spin0<CapGrid<1>, Eberly, std::decay_t<Coupling>>;
  using SplitK = MultiProductSplit<Split3Base<REP::X, REP::P, REP::X>, K>;
  Ham wf(make_grid<1>(), make_pot(), std::forward<Coupling>(c));
  wf.addUsingCoordinateFunction([](auto... x) { return gaussian(0.0, 1.0, x...); });
  const ind m = wf.m_l;
  dump(out + "/" + tag + "_psi0.bin", &wf[0], m);
  SplitPropagator<MODE::RE, SplitK, Ham> re(
      PropagatorBase{.dt = par("re_dt", 0.05), .max_steps = 0, .state_accuracy = 0}, std::move(wf), tag);
  using Outs = BufferedBinaryOutputs<VALUE<Step, Time>, AVG<Identity>, AVG<PotentialEnergy>>;
  re.run(Outs(BufferedOutputsBase{1, 1}), [&](WHEN when, ind, uind, auto& w) {
    if (when == WHEN::AT_END) dump(out + "/" + tag + "_psi.bin", &w[0], m);
  });
}
static void mp(const std::string& out) {
  using F = Field<AXIS::X, Sin2>;
  mp_run<2>(out, "MP2VG", DipoleCoupling<VelocityGauge, F>(F(Sin2(field_cfg()))));
  mp_run<3>(out, "MP3VG", DipoleCoupling<VelocityGauge, F>(F(Sin2(field_cfg()))));
  mp_run<2>(out, "MP2LG", DipoleCoupling<LengthGauge, F>(F(Sin2(field_cfg()))));
  mp_run<3>(out, "MP3LG", DipoleCoupling<LengthGauge, F>(F(Sin2(field_cfg()))));
}


// ---------------------------------------------------------------- other members
// average_der<X, d, PotentialEnergy> (grid.h:443-465) on a seeded state, then
// operation<IM, X, AntiSymmetrize<2>> and, in 3D, AntiSymmetrize<3> (grid.h:611-723)
template <DIMS D> static void as_case(const std::string& out) {
  using Ham = Schrodinger::Spin0<CapGrid<D>, Eberly>;
  Ham wf(make_grid<D>(), make_pot());
  const ind m = wf.m_l;
  g_state = (uint64_t)par("seed", 5);
  std::vector<cxd> psi0((size_t)m);
  for (ind i = 0; i < m; i++) psi0[(size_t)i] = cxd(urand(), urand());
  auto set = [&]() {
    for (ind i = 0; i < m; i++) wf[i] = psi0[(size_t)i];
  };
  set();
  dump(out + "/psi_in.bin", psi0.data(), m);
  FILE* fo = fopen((out + "/der.bin").c_str(), "wb");
  double v;
  v = wf.template average_der<REP::X, 0, PotentialEnergy>();
  fwrite(&v, sizeof v, 1, fo);
  if constexpr (D >= 2) {
    v = wf.template average_der<REP::X, 1, PotentialEnergy>();
    fwrite(&v, sizeof v, 1, fo);
  }
  if constexpr (D >= 3) {
    v = wf.template average_der<REP::X, 2, PotentialEnergy>();
    fwrite(&v, sizeof v, 1, fo);
  }
  fclose(fo);
  wf.template operation<MODE::IM, REP::X, AntiSymmetrize<2>>();
  dump(out + "/psi_as2.bin", &wf[0], m);
  if constexpr (D == 3) {
    set();
    wf.template operation<MODE::IM, REP::X, AntiSymmetrize<3>>();
    dump(out + "/psi_as3.bin", &wf[0], m);
  }
}

int main(int argc, char** argv) {
  if (argc < 3) {
    fprintf(stderr, "usage: %s <case> <outdir> key=value...\n", argv[0]);
    return 2;
  }
  std::string cs = argv[1], out = argv[2];
  for (int i = 3; i < argc; ++i) {
    std::string kv = argv[i];
    auto eq = kv.find('=');
    if (eq == std::string::npos) continue;
    P[kv.substr(0, eq)] = atof(kv.substr(eq + 1).c_str());
  }
  MPI::init(argc, argv);
  std::filesystem::current_path(out);
  if (MPI::pID) {  // every rank but 0 in a directory of its own (each opens the .dat file)
    const std::string sub = "rank" + std::to_string(MPI::pID);
    std::filesystem::create_directories(sub);
    std::filesystem::current_path(sub);
  }
  out = ".";
  set_borders();
  if (cs == "prim2d") prim<2>(out);
  else if (cs == "prim3d") prim<3>(out);
  else if (cs == "c1") {
    int b = (int)par("box", 100);
    if (b == 100) c1<100>(out);
    else if (b == 1638) c1<1638>(out);
    else { fprintf(stderr, "box size %d not instantiated\n", b); return 2; }
  } else if (cs == "c2") c2(out);
  else if (cs == "c3") c3(out);
  else if (cs == "mp") mp(out);
  else if (cs == "as2") as_case<2>(out);
  else if (cs == "as3") as_case<3>(out);
  else if (cs == "mg1") mg<1>(out);
  else if (cs == "mg2") mg<2>(out);
  else if (cs == "mg3") mg<3>(out);
  else if (cs == "io1") io<1>(out);
  else if (cs == "io2") io<2>(out);
  else if (cs == "io3") io<3>(out);
  else { fprintf(stderr, "unknown case %s\n", cs.c_str()); return 2; }
  return 0;
}
