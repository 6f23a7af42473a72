// Reference harness -- TEST INFRASTRUCTURE ONLY.
//
// Runs the reference's own classes (ViennaEMC headers, compiled in place by
// oracle/Makefile into oracle/_ref/) and prints their results as exact
// hex-float records, one "key count v0 v1 ..." line each.
// tests/golden/make_golden.py turns these into the committed fixtures.
//
// The harness reads private members of the reference classes (particle state,
// RNG state, normalised tables, simulation internals); oracle/Makefile builds
// it with -fno-access-control for that.
#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <functional>
#include <iostream>
#include <limits>
#include <map>
#include <memory>
#include <numeric>
#include <random>
#include <sstream>
#include <stdexcept>
#include <string>
#include <tuple>
#include <type_traits>
#include <unistd.h>
#include <utility>
#include <vector>

#include <ParticleType/emcElectron.hpp>
#include <ScatterMechanisms/emcAcousticScatterMechanism.hpp>
#include <ScatterMechanisms/emcCoulombScatterMechanism.hpp>
#include <ScatterMechanisms/emcFirstOrderInterValleyScatterMechanism.hpp>
#include <ScatterMechanisms/emcZeroOrderInterValleyScatterMechanism.hpp>
#include <ValleyTypes/emcNonParabolicAnistropValley.hpp>
#include <SurfaceScatterMechanisms/emcConstantSurfaceScatterMechanism.hpp>
#include <SurfaceScatterMechanisms/emcMomentumDependentSurfaceScatterMechanism.hpp>
#include <ScatterMechanisms/emcHotPhononFroehlichMechanism.hpp>
#include <emcPhononBath.hpp>
#include <ParticleHandler/FMM/FP2PRCutoff.hpp>
#include <PMSchemes/emcCICScheme.hpp>
#include <PMSchemes/emcNECScheme.hpp>
#include <PMSchemes/emcNGPScheme.hpp>
#include <ParticleHandler/emcBasicParticleHandler.hpp>
#include <PoissonSolver/emcSORSolver.hpp>
#include <emcDevice.hpp>
#include <emcParticleDrift.hpp>
#include <emcSimulation.hpp>
#include "../examples/bulkSimulation/basicBulkParticleHandler.hpp"
#include "../examples/mosfet2D/NECSchemeVWD.hpp"
#include "../examples/mosfet2D/electronVWD.hpp"

using T = double;
using Dev3 = emcDevice<T, 3>;
using Handler = basicBulkParticleHandler<T, Dev3>;
using Valley = emcNonParabolicAnisotropValley<T>;

static void rec(const char *key, const std::vector<double> &v) {
  std::printf("%s %zu", key, v.size());
  for (double x : v)
    std::printf(" %a", x);
  std::printf("\n");
}
static void reci(const char *key, const std::vector<long long> &v) {
  std::printf("%s %zu", key, v.size());
  for (long long x : v)
    std::printf(" %lld", x);
  std::printf("\n");
}
static void recu(const char *key, const std::vector<unsigned long long> &v) {
  std::printf("%s %zu", key, v.size());
  for (unsigned long long x : v)
    std::printf(" %llu", x);
  std::printf("\n");
}

struct ModelSpec {
  std::string name;   // "refbulk" | "jacoboni"
  double temperature = 300;
  int nLevels = 1000;
  double maxE = 1.;
};

// Silicon X valley: three paired Delta valleys (examples/SiliconFunctions.hpp:
// 62-73); the transverse mass is a parameter (0.196 in the reference example,
// 0.19 in the bulk benchmark model).
template <class PT> void addValley(std::unique_ptr<PT> &pt, double mt) {
  std::unique_ptr<Valley> v(
      new Valley({0.916, mt, mt}, pt->getMass(), 3, 0.5));
  v->setSubValleyEllipseCoordSystem(0, {1, 0, 0}, {0, 1, 0}, {0, 0, 1});
  v->setSubValleyEllipseCoordSystem(1, {0, 1, 0}, {1, 0, 0}, {0, 0, 1});
  v->setSubValleyEllipseCoordSystem(2, {0, 0, 1}, {0, 1, 0}, {1, 0, 0});
  pt->addValley(std::move(v));
}

static const std::map<SizeType, std::vector<SizeType>> kG = {
    {0, {0}}, {1, {1}}, {2, {2}}};
static const std::map<SizeType, std::vector<SizeType>> kF = {
    {0, {1, 1, 2, 2}}, {1, {0, 0, 2, 2}}, {2, {0, 0, 1, 1}}};

// Intervalley phonons of Jacoboni & Reggiani, Rev. Mod. Phys. 55, 645 (1983),
// Si table: phonon temperature [K] and coupling [1e8 eV/cm]; used as zero-order
// couplings (the bulk benchmark model).
struct IvPhonon {
  const char *name;
  bool isF;
  double thetaK;
  double D;
};
static const IvPhonon kJacoboni[6] = {
    {"G1", false, 140., 0.5e10}, {"G2", false, 215., 0.8e10},
    {"G3", false, 720., 11.e10}, {"F1", true, 220., 0.3e10},
    {"F2", true, 550., 2.0e10},  {"F3", true, 685., 2.0e10}};

template <class PT, class Dev>
void addMechanisms(const ModelSpec &spec, std::unique_ptr<PT> &pt,
                   const Dev &device, const std::vector<int> &regions) {
  using Ac = emcAcousticScatterMechanism<T>;
  using ZA = emcZeroOrderInterValleyAbsorptionScatterMechanism<T>;
  using ZE = emcZeroOrderInterValleyEmissionScatterMechanism<T>;
  using FA = emcFirstOrderInterValleyAbsorptionScatterMechanism<T>;
  using FE = emcFirstOrderInterValleyEmissionScatterMechanism<T>;
  if (spec.name == "refbulk") {
    // examples/SiliconFunctions.hpp:224-239, 265-333
    pt->addScatterMechanism(regions, std::make_unique<Ac>(0, 9., device));
    pt->addScatterMechanism(regions, std::make_unique<ZA>("F", 0, kF, 5.23e10, 0.06, device));
    pt->addScatterMechanism(regions, std::make_unique<ZE>("F", 0, kF, 5.23e10, 0.06, device));
    pt->addScatterMechanism(regions, std::make_unique<ZA>("G", 0, kG, 5.23e10, 0.06, device));
    pt->addScatterMechanism(regions, std::make_unique<ZE>("G", 0, kG, 5.23e10, 0.06, device));
    pt->addScatterMechanism(regions, std::make_unique<FA>("F", 0, kF, 2.5, 0.023, device));
    pt->addScatterMechanism(regions, std::make_unique<FE>("F", 0, kF, 2.5, 0.023, device));
    pt->addScatterMechanism(regions, std::make_unique<FA>("G", 0, kG, 4., 0.018, device));
    pt->addScatterMechanism(regions, std::make_unique<FE>("G", 0, kG, 4., 0.018, device));
  } else if (spec.name == "jacoboni") {
    pt->addScatterMechanism(regions, std::make_unique<Ac>(0, 9., device));
    for (const auto &ph : kJacoboni) {
      double e = constants::kB * ph.thetaK / constants::q;
      const auto &fs = ph.isF ? kF : kG;
      pt->addScatterMechanism(regions, std::make_unique<ZA>(ph.name, 0, fs, ph.D, e, device));
      pt->addScatterMechanism(regions, std::make_unique<ZE>(ph.name, 0, fs, ph.D, e, device));
    }
  } else {
    std::fprintf(stderr, "unknown model %s\n", spec.name.c_str());
    std::exit(2);
  }
}

static emcMaterial<T> silicon() {
  // examples/SiliconFunctions.hpp:15-19
  return emcMaterial<T>{11.8, 2329., 1.45e16, 9040., 1.15};
}

template <class PT> static void dumpTablesOf(PT &pt, const char *prefix = "") {
  auto &h = pt.scatterHandler;
  for (auto &[key, tables] : h.scatterTables) {
    auto v = std::get<0>(key), r = std::get<1>(key);
    const auto &mechIdx = h.idxTableToIdxMech.at(key);
    for (size_t t = 0; t < tables.size(); t++) {
      auto &mech = h.scatterMechanisms[mechIdx[t]];
      std::vector<double> raw(h.nrEnergyLevels);
      for (SizeType l = 0; l < h.nrEnergyLevels; l++)
        raw[l] = mech->getScatterRate((l + 1) * h.dE, r);
      char key1[96], key2[96];
      std::snprintf(key1, sizeof key1, "%sraw_v%zu_r%zu_t%zu", prefix, (size_t)v, (size_t)r, t);
      std::snprintf(key2, sizeof key2, "%snorm_v%zu_r%zu_t%zu", prefix, (size_t)v, (size_t)r,
                    t);
      rec(key1, raw);
      rec(key2, tables[t]);
      std::printf("%sname_v%zu_r%zu_t%zu 1 %s\n", prefix, (size_t)v, (size_t)r, t,
                  mech->getName().c_str());
    }
    char kt[64];
    std::snprintf(kt, sizeof kt, "%stau_v%zu_r%zu", prefix, (size_t)v, (size_t)r);
    rec(kt, {h.getTau(r, v)});
  }
}

static void dumpBulkState(const char *tag, Handler &h) {
  auto &P = h.particles[0];
  auto &X = h.positionsParticles[0];
  size_t n = P.size();
  std::vector<double> kx(n), ky(n), kz(n), px(n), py(n), pz(n), E(n), tau(n),
      gt(n);
  std::vector<long long> val(n), sub(n), reg(n);
  for (size_t i = 0; i < n; i++) {
    kx[i] = P[i].k[0];
    ky[i] = P[i].k[1];
    kz[i] = P[i].k[2];
    px[i] = X[i][0];
    py[i] = X[i][1];
    pz[i] = X[i][2];
    E[i] = P[i].energy;
    tau[i] = P[i].tau;
    gt[i] = P[i].grainTau;
    val[i] = P[i].valley;
    sub[i] = P[i].subValley;
    reg[i] = P[i].region;
  }
  std::string t(tag);
  rec((t + "_kx").c_str(), kx);
  rec((t + "_ky").c_str(), ky);
  rec((t + "_kz").c_str(), kz);
  rec((t + "_px").c_str(), px);
  rec((t + "_py").c_str(), py);
  rec((t + "_pz").c_str(), pz);
  rec((t + "_E").c_str(), E);
  rec((t + "_tau").c_str(), tau);
  rec((t + "_gtau").c_str(), gt);
  reci((t + "_valley").c_str(), val);
  reci((t + "_sub").c_str(), sub);
  reci((t + "_region").c_str(), reg);
}

static void dumpMt(const char *tag, const emcRNG &rng) {
  std::stringstream ss;
  ss << rng;
  std::vector<unsigned long long> w;
  unsigned long long x;
  while (ss >> x)
    w.push_back(x);
  recu(tag, w); // 312 state words followed by the position index
}

// usage: ref_driver bulk <model> <T> <nLevels> <maxE> <box> <spacing>
//                   <doping> <seed> <field> <dx> <dy> <dz> <dt> <nSteps> <mt>
//                   [<grain transmission probability> <grain scatter rate>]
static int runBulk(int argc, char **argv) {
  if (argc < 17) {
    std::fprintf(stderr, "bulk: missing arguments\n");
    return 2;
  }
  ModelSpec spec;
  spec.name = argv[2];
  spec.temperature = std::atof(argv[3]);
  spec.nLevels = std::atoi(argv[4]);
  spec.maxE = std::atof(argv[5]);
  double box = std::atof(argv[6]), h = std::atof(argv[7]);
  double doping = std::atof(argv[8]);
  unsigned long seed = std::strtoul(argv[9], nullptr, 10);
  double field = std::atof(argv[10]);
  std::array<T, 3> dir = {std::atof(argv[11]), std::atof(argv[12]),
                          std::atof(argv[13])};
  double dt = std::atof(argv[14]);
  int nSteps = std::atoi(argv[15]);
  double mt = std::atof(argv[16]);

  std::array<T, 3> maxPos = {box, box, box}, spacing = {h, h, h};
  Dev3 device{silicon(), maxPos, spacing, spec.temperature};
  device.addConstantDopingRegion({0, 0, 0}, maxPos, doping);
  Handler::MapIdxToParticleTypes types;
  auto el = std::make_unique<emcElectron<T, Dev3>>(spec.nLevels, spec.maxE, false);
  addValley(el, mt);
  addMechanisms(spec, el, device, {0});
  if (argc > 18)
    el->setGrainScatterMechanism(
        std::make_unique<emcGrainScatterMechanism<T>>(std::atof(argv[17]), std::atof(argv[18])));
  types[0] = std::move(el);
  // tables are written to files by initScatterTables; keep them out of cwd
  Handler handler(device, types, dir, field, seed);
  dumpTablesOf(*types[0]);
  handler.generateInitialParticles();
  rec("appliedField", {handler.appliedField[0], handler.appliedField[1],
                       handler.appliedField[2]});
  rec("appliedFieldDir", {handler.appliedFieldDir[0], handler.appliedFieldDir[1],
                          handler.appliedFieldDir[2]});
  dumpBulkState("s0", handler);
  dumpMt("mt0", handler.rngs[0]);
  auto obs = [&](int s) {
    auto e = handler.getAvgEnergy(0);
    auto v = handler.getAvgDriftVelocity(0);
    auto o = handler.getValleyOccupationProbability(0);
    char k[64];
    std::vector<double> all;
    for (size_t i = 0; i < e.size(); i++) {
      all.push_back(e[i]);
      all.push_back(v[i]);
      all.push_back(o[i]);
    }
    std::snprintf(k, sizeof k, "obs%d", s);
    rec(k, all);
  };
  obs(0);
  for (int s = 1; s <= nSteps; s++) {
    handler.moveParticles(dt);
    char tag[32];
    std::snprintf(tag, sizeof tag, "s%d", s);
    dumpBulkState(tag, handler);
    obs(s);
  }
  dumpMt("mtEnd", handler.rngs[0]);
  return 0;
}

// usage: ref_driver mt <seed> <n>   -- first n words of std::mt19937_64(seed)
static int runMt(int argc, char **argv) {
  if (argc < 4)
    return 2;
  std::mt19937_64 g(std::strtoull(argv[2], nullptr, 10));
  int n = std::atoi(argv[3]);
  std::vector<unsigned long long> w(n);
  for (int i = 0; i < n; i++)
    w[i] = g();
  recu("mt", w);
  std::uniform_real_distribution<double> d01(0., 1.), dlog(1e-6, 1.);
  std::mt19937_64 g2(std::strtoull(argv[2], nullptr, 10));
  std::vector<double> u(n);
  for (int i = 0; i < n; i++)
    u[i] = (i % 2) ? dlog(g2) : d01(g2);
  rec("canon", u);
  return 0;
}


using Dev2 = emcDevice<T, 2>;

template <class Grid> static std::vector<double> gridVec(const Grid &g) {
  return std::vector<double>(g.begin(), g.end());
}

template <class PH> static void dumpDevState(const char *tag, PH &ph) {
  auto &P = ph.particles[0];
  auto &X = ph.positionsParticles[0];
  size_t n = P.size();
  std::vector<double> kx(n), ky(n), kz(n), px(n), py(n), E(n), tau(n), gt(n);
  std::vector<long long> val(n), sub(n), reg(n);
  for (size_t i = 0; i < n; i++) {
    kx[i] = P[i].k[0];
    ky[i] = P[i].k[1];
    kz[i] = P[i].k[2];
    px[i] = X[i][0];
    py[i] = X[i][1];
    E[i] = P[i].energy;
    tau[i] = P[i].tau;
    gt[i] = P[i].grainTau;
    val[i] = P[i].valley;
    sub[i] = P[i].subValley;
    reg[i] = P[i].region;
  }
  std::string t(tag);
  rec((t + "_kx").c_str(), kx);
  rec((t + "_ky").c_str(), ky);
  rec((t + "_kz").c_str(), kz);
  rec((t + "_px").c_str(), px);
  rec((t + "_py").c_str(), py);
  std::vector<double> pz(n, 0.);
  rec((t + "_pz").c_str(), pz);
  rec((t + "_E").c_str(), E);
  rec((t + "_tau").c_str(), tau);
  rec((t + "_gtau").c_str(), gt);
  reci((t + "_valley").c_str(), val);
  reci((t + "_sub").c_str(), sub);
  reci((t + "_region").c_str(), reg);
}

// usage: ref_driver device <resistor|mosfet|resistor_nec|mosfet_vwd> <seed> <dt> <nSteps>
//                          <accV> <width> [outDir]
// resistor: NGP, mosfet: CIC, resistor_nec: emcNECScheme, all with emcElectron;
// resistor_surface: the NGP resistor with surface mechanisms on YMIN and YMAX;
// mosfet_vwd: the mosfet2D example's NEC-VWD scheme with its electronVWD
// With outDir, the reference's own writers put their files there after the
// last step (emcSimulationResults::writeCurrentResults with suffix "Step",
// emcBasicParticleHandler::print, and writeFinalResults averaged over all steps).
template <class PM, class PT>
static int runDeviceT(const std::string &kind, unsigned long seed, double dt, int nSteps,
                      double acc, double width, const std::string &outDir) {
  using PH = emcBasicParticleHandler<T, Dev2, PM>;
  using Solver = emcSORSolver<T, Dev2, PH>;
  using Sim = emcSimulation<T, Dev2, Solver, PH, PM>;
  const bool mos = kind.rfind("mosfet", 0) == 0;
  std::array<T, 2> maxPos = mos ? std::array<T, 2>{30e-9, 20e-9} : std::array<T, 2>{20e-9, 10e-9};
  std::array<T, 2> spacing = {1e-9, 1e-9};
  Dev2 device{silicon(), maxPos, spacing, 300.};
  device.setDeviceWidth(width);
  std::vector<int> regions;
  if (mos) {
    device.addConstantDopingRegion({0, 8e-9}, {30e-9, 20e-9}, -1e24);
    device.addConstantDopingRegion({0, 0}, {10e-9, 8e-9}, 1e26);
    device.addConstantDopingRegion({10e-9, 0}, {20e-9, 8e-9}, -1e24);
    device.addConstantDopingRegion({20e-9, 0}, {30e-9, 8e-9}, 1e26);
    device.addOhmicContact(emcBoundaryPos::YMAX, 0, {0}, {30e-9});
    device.addOhmicContact(emcBoundaryPos::YMIN, 0, {0}, {10e-9});
    device.addGateContact(emcBoundaryPos::YMIN, 1.0, {10e-9}, {20e-9}, 3.9, 1.2e-9,
                          device.getMaterial().getBandGap() / 2.);
    device.addOhmicContact(emcBoundaryPos::YMIN, 0.5, {20e-9}, {30e-9});
    regions = {0, 1, 2, 3};
  } else {
    device.addConstantDopingRegion({0, 0}, maxPos, 1e25);
    device.addOhmicContact(emcBoundaryPos::XMAX, 0, {0}, {maxPos[1]});
    device.addOhmicContact(emcBoundaryPos::XMIN, 0.1, {0}, {maxPos[1]});
    regions = {0};
  }
  Solver solver(device, acc, 1.8);
  PM pm;
  emcSimulationParameter<T, Dev2> param;
  param.setTimes(nSteps * dt, dt, 0.);
  param.setSeed(seed);
  param.setNrStepsBetweenShowProgress(1000000);
  param.setNrStepsForFinalAvg(1);
  if (!outDir.empty())
    param.setNamePrefix(outDir + "/");
  std::unique_ptr<PT> el;
  if constexpr (std::is_same<PT, emcElectron<T, Dev2>>::value)
    el = std::make_unique<PT>(1000, 4., mos);
  else
    el = std::make_unique<PT>(1000, 4.);
  addValley(el, 0.196);
  ModelSpec spec;
  spec.name = "refbulk";
  using Ac = emcAcousticScatterMechanism<T>;
  using ZA = emcZeroOrderInterValleyAbsorptionScatterMechanism<T>;
  using ZE = emcZeroOrderInterValleyEmissionScatterMechanism<T>;
  el->addScatterMechanism(regions, std::make_unique<Ac>(0, 9., device));
  el->addScatterMechanism(regions, std::make_unique<emcCoulombScatterMechanism<T, Dev2>>(0, 11.8, device));
  el->addScatterMechanism(regions, std::make_unique<ZA>("F", 0, kF, 5.23e10, 0.06, device));
  el->addScatterMechanism(regions, std::make_unique<ZE>("F", 0, kF, 5.23e10, 0.06, device));
  el->addScatterMechanism(regions, std::make_unique<ZA>("G", 0, kG, 5.23e10, 0.06, device));
  el->addScatterMechanism(regions, std::make_unique<ZE>("G", 0, kG, 5.23e10, 0.06, device));
  if (kind == "resistor_surface") {
    // surface mechanisms on the two artificial boundaries of the resistor
    el->setSurfaceScatterMechanism(
        emcBoundaryPos::YMIN,
        std::make_unique<emcConstantSurfaceScatterMechanism<T, Dev2>>(0.3, maxPos));
    el->setSurfaceScatterMechanism(
        emcBoundaryPos::YMAX,
        std::make_unique<emcMomentumDependentSurfaceScatterMechanism<T, Dev2>>(0.5e-9, maxPos));
  }
  param.addParticleType(std::move(el));
  Sim sim(param, device, solver, pm);
  // device description
  rec("doping", gridVec(device.getDopingProfile().doping));
  {
    std::vector<long long> r(device.getDopingProfile().idxDopingRegions.begin(),
                             device.getDopingProfile().idxDopingRegions.end());
    reci("region", r);
  }
  auto &surf = device.getSurface();
  for (int b = 0; b < 4; b++) {
    std::vector<long long> g(surf.idxContactGrid[b].begin(), surf.idxContactGrid[b].end());
    char k[32];
    std::snprintf(k, sizeof k, "bnd%d", b);
    reci(k, g);
  }
  std::vector<long long> ct;
  std::vector<double> cv, cp;
  for (size_t c = 0; c < surf.getNrContacts(); c++) {
    auto t = surf.getContactType(c);
    ct.push_back(t == emcContactType::OHMIC ? 0 : t == emcContactType::SCHOTTKY ? 1 : 2);
    cv.push_back(surf.getContactVoltage(c));
    for (int q = 0; q < 3; q++)
      cp.push_back(t == emcContactType::GATE ? surf.getContactFurtherParameter(c, q) : 0.);
  }
  reci("ctype", ct);
  rec("cvolt", cv);
  rec("cpar", cp);
  rec("geom", {maxPos[0], maxPos[1], spacing[0], spacing[1], device.deviceWidth,
               device.getCellVolume(), device.getDebyeLength(), device.getThermalVoltage()});
  auto &type = *param.particleTypes[0];
  dumpTablesOf(type);
  // equilibrium + initial particles (emcSimulation.hpp:139-146), in parts
  auto &res = sim.results;
  rec("pot_init", gridVec(res.currPot));
  sim.solver.calcEquilibriumPotential(res.currPot, device);
  rec("pot_eq", gridVec(res.currPot));
  sim.pmScheme.calcEField(res.eField, res.currPot, device);
  rec("ex_eq", gridVec(res.eField[0]));
  rec("ey_eq", gridVec(res.eField[1]));
  dumpMt("mt_pre", sim.particleHandler.rngs[0]);
  sim.particleHandler.generateInitialParticles(res.currPot);
  sim.assignParticlesToGrid();
  res.updateCurrentParticleConcentrations(device);
  dumpDevState("s0", sim.particleHandler);
  dumpMt("mt0", sim.particleHandler.rngs[0]);
  rec("nr0", gridVec(res.nrPart[0]));
  rec("conc0", gridVec(res.currConc[0]));
  {
    std::vector<double> e(sim.particleHandler.expNrPart[0].begin(),
                          sim.particleHandler.expNrPart[0].end());
    rec("expnr", e);
  }
  for (int s = 1; s <= nSteps; s++) {
    sim.performEMCStep(s == 1, false, true);
    if (!outDir.empty())
      res.updateAverageCharacteristics();
    char k[48];
    std::snprintf(k, sizeof k, "s%d", s);
    dumpDevState(k, sim.particleHandler);
    std::snprintf(k, sizeof k, "pot%d", s);
    rec(k, gridVec(res.currPot));
    std::snprintf(k, sizeof k, "ex%d", s);
    rec(k, gridVec(res.eField[0]));
    std::snprintf(k, sizeof k, "ey%d", s);
    rec(k, gridVec(res.eField[1]));
    std::snprintf(k, sizeof k, "nr%d", s);
    rec(k, gridVec(res.nrPart[0]));
    std::snprintf(k, sizeof k, "conc%d", s);
    rec(k, gridVec(res.currConc[0]));
    std::vector<long long> netto(res.nettoPart[s - 1][0].begin(), res.nettoPart[s - 1][0].end());
    std::snprintf(k, sizeof k, "netto%d", s);
    reci(k, netto);
    std::snprintf(k, sizeof k, "cur%d", s);
    rec(k, std::vector<double>(res.current[s - 1][0].begin(), res.current[s - 1][0].end()));
  }
  if (!outDir.empty()) {
    res.writeCurrentResults("Step", device);
    sim.particleHandler.print(param.namePrefix, "Step");
    res.writeFinalResults(device);
  }
  return 0;
}

static int runDevice(int argc, char **argv) {
  if (argc < 8)
    return 2;
  std::string kind = argv[2];
  unsigned long seed = std::strtoul(argv[3], nullptr, 10);
  double dt = std::atof(argv[4]);
  int n = std::atoi(argv[5]);
  double acc = std::atof(argv[6]);
  double width = std::atof(argv[7]);
  std::string out = argc > 8 ? argv[8] : "";
  using El = emcElectron<T, Dev2>;
  if (kind == "mosfet")
    return runDeviceT<emcCICScheme<T, Dev2>, El>(kind, seed, dt, n, acc, width, out);
  if (kind == "resistor_nec")
    return runDeviceT<emcNECScheme<T, Dev2>, El>(kind, seed, dt, n, acc, width, out);
  if (kind == "mosfet_vwd")
    return runDeviceT<emcNECSchemeVWD<T, Dev2>, electronVWD<T, Dev2>>(kind, seed, dt, n, acc,
                                                                      width, out);
  return runDeviceT<emcNGPScheme<T, Dev2>, El>(kind, seed, dt, n, acc, width, out);
}

// reinitScatterTables with rates that change: acoustic scattering and the
// hot-phonon Froehlich absorption / emission pair sharing one emcPhononBath
// (include/ScatterMechanisms/emcHotPhononFroehlichMechanism.hpp,
// include/emcPhononBath.hpp).  The tables are dumped after initScatterTables
// ("init_"), then the bath records emissions over its q range and is advanced
// by dt, the tables are rebuilt, and dumped again ("re_").
// args: nLevels maxE nEmissions dt
static int runReinit(int argc, char **argv) {
  if (argc < 6)
    return 2;
  const int nLevels = std::atoi(argv[2]);
  const double maxE = std::atof(argv[3]);
  const int nEm = std::atoi(argv[4]);
  const double dtBath = std::atof(argv[5]);
  const double temp = 300.;
  std::array<T, 3> maxPos = {1e-7, 1e-7, 1e-7}, spacing = {1e-8, 1e-8, 1e-8};
  Dev3 device{silicon(), maxPos, spacing, temp};
  auto el = std::make_unique<emcElectron<T, Dev3>>(nLevels, maxE, false);
  addValley(el, 0.19);
  // LO phonon of 36 meV, 200 q bins of 1e7 1/m, 3 ps lifetime, 1e-21 m^3
  auto bath = std::make_shared<emcPhononBath<T>>(200, 1e7, 3e-12, 0.036, temp, 1e-21);
  el->addScatterMechanism({0}, std::make_unique<emcAcousticScatterMechanism<T>>(0, 9., device));
  el->addScatterMechanism(
      {0}, std::make_unique<emcHotPhononFroehlichAbsorption3D<T>>(0, 0.036, 0.26, 10.9, 12.9,
                                                                   bath));
  el->addScatterMechanism(
      {0}, std::make_unique<emcHotPhononFroehlichEmission3D<T>>(0, 0.036, 0.26, 10.9, 12.9,
                                                                 bath));
  el->initScatterTables();
  dumpTablesOf(*el, "init_");
  rec("init_meanNq", {bath->getMeanNq()});
  for (int i = 0; i < nEm; i++) // q over the bath's range, denser at small q
    bath->recordEmission(1e7 * 200. * std::pow((i + 0.5) / nEm, 2.));
  bath->update(dtBath);
  el->reinitScatterTables();
  dumpTablesOf(*el, "re_");
  rec("re_meanNq", {bath->getMeanNq()});
  return 0;
}

// The reference's particle-particle pair kernel with the 1 nm cutoff
// (include/ParticleHandler/FMM/FP2PRCutoff.hpp:18-100), as the FMM handlers'
// P2P evaluates it: n particles in a cube, each target summed over every
// other particle in index order with NonMutualParticles, plus the pairs of a
// MutualParticles call.  args: n box seed
static int runP2P(int argc, char **argv) {
  if (argc < 5)
    return 2;
  const int n = std::atoi(argv[2]);
  const double box = std::atof(argv[3]);
  std::mt19937_64 g(std::strtoull(argv[4], nullptr, 10));
  std::uniform_real_distribution<double> u(0., 1.);
  std::vector<double> x(n), y(n), z(n), q(n);
  for (int i = 0; i < n; i++) {
    x[i] = u(g) * box;
    y[i] = u(g) * box;
    z[i] = u(g) * box;
    q[i] = (i % 3 == 2 ? 1. : -1.) * constants::q;
  }
  // a few pairs closer than the cutoff
  for (int i = 1; i < n; i += 7) {
    x[i] = x[i - 1] + 3e-10 * (u(g) - 0.5);
    y[i] = y[i - 1] + 3e-10 * (u(g) - 0.5);
    z[i] = z[i - 1] + 3e-10 * (u(g) - 0.5);
  }
  std::vector<double> fx(n, 0.), fy(n, 0.), fz(n, 0.), pot(n, 0.);
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++)
      if (j != i)
        FP2PRCutoff::NonMutualParticles<double>(x[i], y[i], z[i], q[i], &fx[i], &fy[i], &fz[i],
                                                &pot[i], x[j], y[j], z[j], q[j]);
  rec("x", x);
  rec("y", y);
  rec("z", z);
  rec("q", q);
  rec("fx", fx);
  rec("fy", fy);
  rec("fz", fz);
  rec("pot", pot);
  // one MutualParticles call per consecutive pair: both sides of a pair
  std::vector<double> m(8 * (n / 2), 0.);
  for (int p = 0; p + 1 < n; p += 2) {
    double *o = &m[8 * (p / 2)];
    FP2PRCutoff::MutualParticles<double>(x[p], y[p], z[p], q[p], o + 0, o + 1, o + 2, o + 3,
                                         x[p + 1], y[p + 1], z[p + 1], q[p + 1], o + 4, o + 5,
                                         o + 6, o + 7);
  }
  rec("mutual", m);
  return 0;
}

int main(int argc, char **argv) {
  if (argc < 2) {
    std::fprintf(stderr, "usage: ref_driver {bulk|mt} ...\n");
    return 2;
  }
  std::string mode = argv[1];
  // initScatterTables writes one file per table into the working directory:
  // the caller runs the harness in a scratch directory (oracle/pyoracle.py)
  std::cout.setf(std::ios::unitbuf);
  // the reference prints progress to stdout; route it to stderr
  std::streambuf *orig = std::cout.rdbuf(std::cerr.rdbuf());
  int rc = 2;
  if (mode == "bulk")
    rc = runBulk(argc, argv);
  else if (mode == "mt")
    rc = runMt(argc, argv);
  else if (mode == "device")
    rc = runDevice(argc, argv);
  else if (mode == "reinit")
    rc = runReinit(argc, argv);
  else if (mode == "p2p")
    rc = runP2P(argc, argv);
  std::cout.rdbuf(orig);
  return rc;
}
