// Reference harness -- TEST INFRASTRUCTURE ONLY.
//
// Runs the reference's own classes (ViennaEMC headers, compiled in place by
// oracle/Makefile into oracle/_ref/) and prints their results as exact
// hex-float records, one "key count v0 v1 ..." line each.
// tests/golden/make_golden.py turns these into the committed fixtures.
//
// The harness reads private members of the reference classes (particle state,
// RNG state, normalised tables); the access macro below is applied after all
// standard headers are included so that only the reference headers see it.
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

#define private public
#define protected public
#include <ParticleType/emcElectron.hpp>
#include <ScatterMechanisms/emcAcousticScatterMechanism.hpp>
#include <ScatterMechanisms/emcCoulombScatterMechanism.hpp>
#include <ScatterMechanisms/emcFirstOrderInterValleyScatterMechanism.hpp>
#include <ScatterMechanisms/emcZeroOrderInterValleyScatterMechanism.hpp>
#include <ValleyTypes/emcNonParabolicAnistropValley.hpp>
#include <emcDevice.hpp>
#include <emcParticleDrift.hpp>
#include "../examples/bulkSimulation/basicBulkParticleHandler.hpp"
#undef private
#undef protected

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

template <class PT> static void dumpTablesOf(PT &pt) {
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
      std::snprintf(key1, sizeof key1, "raw_v%zu_r%zu_t%zu", (size_t)v, (size_t)r, t);
      std::snprintf(key2, sizeof key2, "norm_v%zu_r%zu_t%zu", (size_t)v, (size_t)r, t);
      rec(key1, raw);
      rec(key2, tables[t]);
      std::printf("name_v%zu_r%zu_t%zu 1 %s\n", (size_t)v, (size_t)r, t,
                  mech->getName().c_str());
    }
    char kt[64];
    std::snprintf(kt, sizeof kt, "tau_v%zu_r%zu", (size_t)v, (size_t)r);
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
//                   <doping> <seed> <field> <dx> <dy> <dz> <dt> <nSteps>
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

int main(int argc, char **argv) {
  if (argc < 2) {
    std::fprintf(stderr, "usage: ref_driver {bulk|mt} ...\n");
    return 2;
  }
  std::string mode = argv[1];
  // initScatterTables writes one file per table into the working directory
  char tmpl[] = "/tmp/emcrefXXXXXX";
  if (char *d = mkdtemp(tmpl))
    if (chdir(d) != 0)
      return 3;
  std::cout.setf(std::ios::unitbuf);
  // the reference prints progress to stdout; route it to stderr
  std::streambuf *orig = std::cout.rdbuf(std::cerr.rdbuf());
  int rc = 2;
  if (mode == "bulk")
    rc = runBulk(argc, argv);
  else if (mode == "mt")
    rc = runMt(argc, argv);
  std::cout.rdbuf(orig);
  return rc;
}
