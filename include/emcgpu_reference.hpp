// emcgpu_reference.hpp -- drop-in bindings of libemcgpu for ViennaEMC users.
//
// Header-only C++17, compiled together with the reference's headers
// (ViennaEMC include/ and examples/ on the include path) and linked against
// libemcgpu.  Two pieces:
//
//   emcgpu::ModelBuilder     registers scatter mechanisms on a reference
//                            emcParticleType through factory helpers that also
//                            record each mechanism's final-state parameters
//                            (the reference classes keep phononEnergy,
//                            finalSubValleys, ... private), and produces the
//                            engine's emcg_model_desc with rate tables filled
//                            by the reference's own getScatterRate.
//   emcgpu::GpuBulkParticleHandler
//                            the API of basicBulkParticleHandler
//                            (examples/bulkSimulation/basicBulkParticleHandler.hpp)
//                            with the particles resident on the GPU.
//   emcgpu::DeviceDesc, emcgpu::GpuDeviceSimulation
//                            a 2-D reference emcDevice as the engine's device
//                            description, and emcSimulation's equilibrium /
//                            performEMCStep on the GPU, the engine's fast
//                            path (every grid stays on the GPU).
//   emcgpu::GpuEngine, GpuPMScheme, GpuPoissonSolver, GpuParticleHandler
//                            plugins of the reference's own interfaces
//                            (emcAbstractPMScheme, emcAbstractSolver,
//                            emcAbstractParticleHandler), so that the stock
//                            emcSimulation runs on the GPU with its template
//                            arguments swapped and nothing else changed.
//
// Every status returned by the C ABI other than EMCG_OK is turned into the
// reference's own error path (emcMessage::addError, which aborts).
#ifndef EMCGPU_REFERENCE_HPP
#define EMCGPU_REFERENCE_HPP

#include <algorithm>
#include <array>
#include <cmath>
#include <map>
#include <memory>
#include <string>
#include <utility>
#include <tuple>
#include <vector>

#include <fstream>
#include <iostream>

#include <PMSchemes/emcAbstractPMScheme.hpp>
#include <PMSchemes/emcCICScheme.hpp>
#include <PMSchemes/emcNECScheme.hpp>
#include <PMSchemes/emcNGPScheme.hpp>
#include <ParticleHandler/emcAbstractParticleHandler.hpp>
#include <ParticleType/emcParticleType.hpp>
#include <PoissonSolver/emcAbstractSolver.hpp>
#include <emcParticleInitialization.hpp>
#include <ScatterMechanisms/emcAcousticScatterMechanism.hpp>
#include <ScatterMechanisms/emcCoulombScatterMechanism.hpp>
#include <ScatterMechanisms/emcFirstOrderInterValleyScatterMechanism.hpp>
#include <ScatterMechanisms/emcZeroOrderInterValleyScatterMechanism.hpp>
#include <ValleyTypes/emcNonParabolicAnistropValley.hpp>
#include <emcBoundaryPos.hpp>
#include <emcContact.hpp>
#include <emcGrainScatterMechanism.hpp>
#include <SurfaceScatterMechanisms/emcConstantSurfaceScatterMechanism.hpp>
#include <SurfaceScatterMechanisms/emcMomentumDependentSurfaceScatterMechanism.hpp>
#include <emcMessage.hpp>

#include "emcgpu.h"

namespace emcgpu {

inline void check(int32_t status) {
  if (status != EMCG_OK)
    emcMessage::getInstance()
        .addError(std::string("libemcgpu: ") + emcg_last_error())
        .print();
}

template <class T, class DeviceType> class ModelBuilder {
public:
  using ParticleType = emcParticleType<T, DeviceType>;
  using FinalSubValleys = std::map<SizeType, std::vector<SizeType>>;

  // nrEnergyLevels and maxEnergy: the values the particle type was built with
  // (emcParticleType(nrEnergyLevels, maxEnergy)); the reference keeps them private.
  ModelBuilder(ParticleType &pt, SizeType nrEnergyLevels, T maxEnergy)
      : pt_(pt), nL_(nrEnergyLevels), maxE_(maxEnergy) {}

  // ---- mechanism factories (examples/SiliconFunctions.hpp style) ----------
  void addAcoustic(SizeType valley, T sigma, const DeviceType &device,
                   const std::vector<int> &regions) {
    auto m = std::make_unique<emcAcousticScatterMechanism<T>>(valley, sigma, device);
    record(m.get(), EMCG_MECH_ACOUSTIC, valley, valley, 0., {}, regions);
    pt_.addScatterMechanism(regions, std::move(m));
  }

  template <class Mech>
  void addInterValley(int kind, const std::string &suffix, SizeType valley,
                      SizeType finalValley, const FinalSubValleys &finalSub, T defPot,
                      T phononEnergy, const DeviceType &device,
                      const std::vector<int> &regions) {
    auto m = std::make_unique<Mech>(suffix, valley, finalValley, finalSub, defPot,
                                    phononEnergy, device);
    const bool abs = kind == EMCG_MECH_ZERO_IV_ABS || kind == EMCG_MECH_FIRST_IV_ABS;
    const T dv = valleyOf(finalValley)->getBottomEnergy() - valleyOf(valley)->getBottomEnergy();
    record(m.get(), kind, valley, finalValley, abs ? phononEnergy - dv : -(phononEnergy + dv),
           finalSub, regions);
    pt_.addScatterMechanism(regions, std::move(m));
  }

  void addZeroOrderAbsorption(const std::string &s, SizeType v, const FinalSubValleys &f, T D,
                              T ph, const DeviceType &dev, const std::vector<int> &r) {
    addInterValley<emcZeroOrderInterValleyAbsorptionScatterMechanism<T>>(
        EMCG_MECH_ZERO_IV_ABS, s, v, v, f, D, ph, dev, r);
  }
  void addZeroOrderEmission(const std::string &s, SizeType v, const FinalSubValleys &f, T D,
                            T ph, const DeviceType &dev, const std::vector<int> &r) {
    addInterValley<emcZeroOrderInterValleyEmissionScatterMechanism<T>>(
        EMCG_MECH_ZERO_IV_EMI, s, v, v, f, D, ph, dev, r);
  }
  void addFirstOrderAbsorption(const std::string &s, SizeType v, const FinalSubValleys &f, T D,
                               T ph, const DeviceType &dev, const std::vector<int> &r) {
    addInterValley<emcFirstOrderInterValleyAbsorptionScatterMechanism<T>>(
        EMCG_MECH_FIRST_IV_ABS, s, v, v, f, D, ph, dev, r);
  }
  void addFirstOrderEmission(const std::string &s, SizeType v, const FinalSubValleys &f, T D,
                             T ph, const DeviceType &dev, const std::vector<int> &r) {
    addInterValley<emcFirstOrderInterValleyEmissionScatterMechanism<T>>(
        EMCG_MECH_FIRST_IV_EMI, s, v, v, f, D, ph, dev, r);
  }

  template <class Dev>
  void addCoulomb(SizeType valley, T epsR, Dev &device, const std::vector<int> &regions) {
    auto m = std::make_unique<emcCoulombScatterMechanism<T, Dev>>(valley, epsR, device);
    record(m.get(), EMCG_MECH_COULOMB, valley, valley, 0., {}, regions);
    // 8 eps0 epsR Vt / hbar^2 (emcCoulombScatterMechanism.hpp:31)
    mechs_.back().coulomb_sc2 = 8 * constants::eps0 * epsR * device.getThermalVoltage() /
                                (constants::hbar * constants::hbar);
    const auto &prof = device.getDopingProfile();
    for (int r = 0; r < EMCG_MAX_REGIONS; r++)
      regionDoping_[r] = r < (int)prof.getNrDopingRegions() ? prof.getDoping(r)
                                                             : device.getMaterial().getNi();
    pt_.addScatterMechanism(regions, std::move(m));
  }

  // emcParticleType::setGrainScatterMechanism with an
  // emcGrainScatterMechanism(transmissionProb, scatterRate)
  // (include/emcGrainScatterMechanism.hpp:27-29): forwarded to the particle
  // type; its two parameters are kept for the engine, since the reference
  // keeps them protected.
  void setGrainScatterMechanism(T transmissionProb, T scatterRate) {
    pt_.setGrainScatterMechanism(
        std::make_unique<emcGrainScatterMechanism<T>>(transmissionProb, scatterRate));
    grain_ = true;
    grainProb_ = transmissionProb;
    grainRate_ = scatterRate;
  }

  // emcParticleType::setSurfaceScatterMechanism(boundary, mechanism)
  // (include/ParticleType/emcParticleType.hpp:155-166) with an
  // emcConstantSurfaceScatterMechanism(specularity, maxPos) or an
  // emcMomentumDependentSurfaceScatterMechanism(roughnessHeight, maxPos):
  // forwarded to the particle type, the kind and parameter kept for the
  // engine (device simulations; the reference keeps them private).
  void setConstantSurfaceScatterMechanism(emcBoundaryPos boundary, T specularity,
                                          const std::array<T, DeviceType::Dimension> &maxPos) {
    pt_.setSurfaceScatterMechanism(
        boundary,
        std::make_unique<emcConstantSurfaceScatterMechanism<T, DeviceType>>(specularity, maxPos));
    surface(boundary, EMCG_SURFACE_CONSTANT, specularity);
  }
  void setMomentumDependentSurfaceScatterMechanism(
      emcBoundaryPos boundary, T roughnessHeight,
      const std::array<T, DeviceType::Dimension> &maxPos) {
    pt_.setSurfaceScatterMechanism(
        boundary, std::make_unique<emcMomentumDependentSurfaceScatterMechanism<T, DeviceType>>(
                      roughnessHeight, maxPos));
    surface(boundary, EMCG_SURFACE_ROUGHNESS, roughnessHeight);
  }

  // ---- engine descriptor (after all mechanisms are registered) ------------
  // Rates are the reference's getScatterRate at (L + 1) dE, accumulated and
  // normalised exactly as emcScatterHandler::renormalizeTables
  // (include/emcScatterHandler.hpp:220-273).
  const emcg_model_desc &desc() {
    const SizeType nL = nL_;
    const T dE = maxE_ / nL_; // include/emcScatterHandler.hpp:75
    valleys_.clear();
    for (SizeType v = 0; v < pt_.getNrValleys(); v++)
      valleys_.push_back(valleyDesc(v));
    sets_.clear();
    tables_.clear();
    for (auto &[key, idx] : sets_of_) {
      emcg_tableset_desc s{};
      s.valley = key.first;
      s.region = key.second;
      s.n_tables = (int32_t)idx.size();
      std::vector<std::vector<T>> t(idx.size(), std::vector<T>(nL));
      for (size_t j = 0; j < idx.size(); j++) {
        s.mech[j] = idx[j];
        for (SizeType l = 0; l < nL; l++)
          t[j][l] = ptrs_[idx[j]]->getScatterRate((l + 1) * dE, key.second);
      }
      for (size_t j = 1; j < t.size(); j++)
        for (SizeType l = 0; l < nL; l++)
          t[j][l] = t[j][l] + t[j - 1][l];
      T mx = t.empty() ? T(0) : *std::max_element(t.back().begin(), t.back().end());
      for (auto &row : t)
        for (auto &x : row) {
          x /= mx;
          tables_.push_back(x);
        }
      s.tau_max = t.empty() ? 2e-15 : 1. / mx;
      sets_.push_back(s);
    }
    d_ = emcg_model_desc{};
    d_.n_valleys = (int32_t)valleys_.size();
    d_.n_mechs = (int32_t)mechs_.size();
    d_.n_tablesets = (int32_t)sets_.size();
    d_.n_levels = (int32_t)nL;
    d_.max_energy = maxE_;
    // the grain free-flight constant: 1 / rate with a mechanism
    // (include/emcScatterHandler.hpp:233-234), else the particle type's 1.  A
    // mechanism set on the particle type directly (not through this builder)
    // has parameters the engine cannot read: refuse it rather than run
    // without its scattering.
    if (!grain_ && pt_.getGrainTau() != T(1))
      emcMessage::getInstance().addError(
          "libemcgpu: a grain mechanism was set on the particle type directly; set it "
          "with ModelBuilder::setGrainScatterMechanism so that the engine knows its "
          "transmission probability");
    d_.grain_tau = grain_ ? T(1) / grainRate_ : pt_.getGrainTau();
    d_.grain = grain_ ? 1 : 0;
    d_.grain_transmission = grain_ ? grainProb_ : T(0);
    for (int b = 0; b < 4; b++) {
      d_.surface_kind[b] = surfKind_[b];
      d_.surface_param[b] = surfParam_[b];
    }
    d_.valleys = valleys_.data();
    d_.mechs = mechs_.data();
    d_.tablesets = sets_.data();
    d_.tables = tables_.data();
    for (int r = 0; r < EMCG_MAX_REGIONS; r++)
      d_.region_doping[r] = regionDoping_[r];
    return d_;
  }

  // The rates of every table refilled now from the reference mechanisms
  // (fillScatterTables, include/emcScatterHandler.hpp:220-235), in the table
  // sets' order of desc(), table-major: what emcg_update_rates takes after a
  // dynamic mechanism (e.g. one reading an emcPhononBath) changed.
  std::vector<double> rawRates() const {
    const T dE = maxE_ / nL_;
    std::vector<double> raw;
    for (auto &[key, idx] : sets_of_)
      for (size_t j = 0; j < idx.size(); j++)
        for (SizeType l = 0; l < nL_; l++)
          raw.push_back((double)ptrs_[idx[j]]->getScatterRate((l + 1) * dE, key.second));
    return raw;
  }

  ParticleType &particleType() { return pt_; }

private:
  const emcNonParabolicAnisotropValley<T> *valleyOf(SizeType v) const {
    auto *p = dynamic_cast<const emcNonParabolicAnisotropValley<T> *>(pt_.getValley(v));
    if (!p)
      emcMessage::getInstance()
          .addError("libemcgpu supports emcNonParabolicAnisotropValley valleys only")
          .print();
    return p;
  }

  emcg_valley_desc valleyDesc(SizeType v) const {
    const auto *V = valleyOf(v);
    emcg_valley_desc d{};
    d.deg = (int32_t)V->getDegeneracyFactor();
    d.particle_mass = pt_.getMass();
    d.alpha = V->getNonParabolicity();
    d.bottom = V->getBottomEnergy();
    const auto &vogt = V->getVogtTransformationFactor();
    const T mc = V->getEffMassCond();
    for (int i = 0; i < 3; i++) // vogt_i = sqrt(mc / (m_i m0))
      d.rel_mass[i] = mc / (vogt[i] * vogt[i] * d.particle_mass);
    for (int s = 0; s < d.deg; s++)
      for (int j = 0; j < 3; j++) { // rows of the rotation: R e_j gives column j
        std::array<T, 3> e{0, 0, 0};
        e[j] = 1;
        auto c = V->transformToEllipseCoord(s, e);
        for (int i = 0; i < 3; i++)
          d.rot[s][3 * i + j] = c[i];
      }
    return d;
  }

  void record(const emcScatterMechanism<T> *ptr, int kind, SizeType valley,
              SizeType finalValley, T shift, const FinalSubValleys &finalSub,
              const std::vector<int> &regions) {
    emcg_mech_desc m{};
    m.kind = kind;
    m.valley = (int32_t)valley;
    m.final_valley = (int32_t)finalValley;
    m.shift = shift;
    if (!finalSub.empty()) {
      m.n_final = (int32_t)finalSub.at(0).size();
      for (auto &[s, fs] : finalSub)
        for (size_t f = 0; f < fs.size() && f < EMCG_MAX_NF; f++)
          m.final_sub[s][f] = (int32_t)fs[f];
    }
    const int idx = (int)mechs_.size();
    mechs_.push_back(m);
    ptrs_.push_back(ptr);
    for (int r : regions)
      sets_of_[{(int)valley, r}].push_back(idx);
  }

  ParticleType &pt_;
  SizeType nL_;
  T maxE_;
  std::vector<emcg_mech_desc> mechs_;
  std::vector<const emcScatterMechanism<T> *> ptrs_;
  std::map<std::pair<int, int>, std::vector<int>> sets_of_;
  std::vector<emcg_valley_desc> valleys_;
  std::vector<emcg_tableset_desc> sets_;
  std::vector<T> tables_;
  T regionDoping_[EMCG_MAX_REGIONS] = {1.45e16, 1.45e16, 1.45e16, 1.45e16, 1.45e16, 1.45e16,
                                       1.45e16, 1.45e16, 1.45e16, 1.45e16, 1.45e16, 1.45e16,
                                       1.45e16, 1.45e16, 1.45e16, 1.45e16};
  bool grain_ = false;
  T grainProb_ = 0, grainRate_ = 0;
  int32_t surfKind_[4] = {EMCG_SURFACE_SPECULAR, EMCG_SURFACE_SPECULAR, EMCG_SURFACE_SPECULAR,
                          EMCG_SURFACE_SPECULAR};
  T surfParam_[4] = {0, 0, 0, 0};
  emcg_model_desc d_{};

  void surface(emcBoundaryPos boundary, int32_t kind, T param) {
    const int b = (int)toUnderlying(boundary);
    if (b < 0 || b > 3) {
      emcMessage::getInstance().addError("libemcgpu: a surface mechanism needs a 2-D boundary "
                                         "(XMIN, XMAX, YMIN or YMAX)");
      return;
    }
    surfKind_[b] = kind;
    surfParam_[b] = param;
  }
};

// basicBulkParticleHandler on the GPU (one particle type, index 0).
template <class T, class DeviceType> class GpuBulkParticleHandler {
public:
  using ValueVec = typename DeviceType::ValueVec;

  GpuBulkParticleHandler(DeviceType &device, ModelBuilder<T, DeviceType> &model,
                         const ValueVec &fieldDir, T fieldStrength, unsigned long seed,
                         int precision = EMCG_FP32, int64_t capacity = 1 << 20)
      : device_(device), model_(model), seed_(seed) {
    T n = 0;
    for (int i = 0; i < 3; i++)
      n += fieldDir[i] * fieldDir[i];
    n = std::sqrt(n);
    for (int i = 0; i < 3; i++)
      dir_[i] = n == 0 ? fieldDir[i] : fieldDir[i] / n; // normalize (:100)
    ens_ = emcg_ensemble_desc{};
    ens_.capacity = capacity;
    ens_.charge = model.particleType().getCharge();
    ens_.seed = seed;
    ens_.dt = 1e-15;
    for (int i = 0; i < 3; i++) {
      ens_.field_dir[i] = dir_[i];
      ens_.field[i] = dir_[i] * fieldStrength;
      ens_.box[i] = device.getMaxPos()[i];
    }
    const emcg_model_desc &md = model.desc();
    check(emcg_bulk_create(&md, 1, &ens_, 1, precision, &h_));
  }
  ~GpuBulkParticleHandler() { emcg_destroy(h_); }
  GpuBulkParticleHandler(const GpuBulkParticleHandler &) = delete;
  GpuBulkParticleHandler &operator=(const GpuBulkParticleHandler &) = delete;

  // particleType.reinitScatterTables() (include/emcScatterHandler.hpp:100-108)
  // on the GPU: rates refilled from the reference mechanisms, renormalised by
  // the engine before the next move
  void reinitScatterTables() {
    const std::vector<double> raw = model_.rawRates();
    check(emcg_update_rates(h_, 0, raw.data(), 0));
  }

  void resetAppliedFieldStrength(T f) { // :135-137
    for (int i = 0; i < 3; i++)
      ens_.field[i] = dir_[i] * f;
    check(emcg_bulk_update_ensemble(h_, 0, &ens_));
  }

  // n particles uniformly in the box with the reference's k-space sampling
  void generateInitialParticles(int64_t n) {
    check(emcg_bulk_init(h_, 0, n, nullptr, nullptr, nullptr, device_.getThermalVoltage()));
    n_ = n;
  }

  void moveParticles(T dt, int nSteps = 1) { // :181-225
    if (dt != ens_.dt) {
      ens_.dt = dt;
      check(emcg_bulk_update_ensemble(h_, 0, &ens_));
    }
    const int nV = (int)model_.particleType().getNrValleys();
    obs_.assign((size_t)nSteps * nV * 3, 0.);
    check(emcg_bulk_step(h_, nSteps, step_, obs_.data()));
    step_ += (uint32_t)nSteps;
    last_.assign(obs_.end() - nV * 3, obs_.end());
  }

  SizeType getNrParticles(SizeType = 0) const { return (SizeType)n_; }

  std::vector<T> getAvgEnergy(SizeType = 0) const { return avg(0); }
  std::vector<T> getAvgDriftVelocity(SizeType = 0) const { return avg(1); }
  std::vector<T> getValleyOccupationProbability(SizeType = 0) const {
    std::vector<T> o;
    for (size_t v = 0; v < last_.size() / 3; v++)
      o.push_back(n_ ? last_[3 * v + 2] / (T)n_ : T(0));
    return o;
  }

private:
  std::vector<T> avg(int q) const {
    std::vector<T> o;
    for (size_t v = 0; v < last_.size() / 3; v++) {
      T c = last_[3 * v + 2];
      o.push_back(c > 0 ? last_[3 * v + q] / c : T(0));
    }
    return o;
  }

  DeviceType &device_;
  ModelBuilder<T, DeviceType> &model_;
  unsigned long seed_;
  T dir_[3];
  emcg_ensemble_desc ens_;
  emcg_handle *h_ = nullptr;
  int64_t n_ = 0;
  uint32_t step_ = 0;
  std::vector<double> obs_, last_;
};

// emcg_device_desc of a 2-D reference device (emcDevice<T, 2>), read through
// its public accessors: grid extent and spacing, material, doping and doping
// region per node (emcDopingProfile), the contact index of every boundary
// coordinate and the contacts' types, voltages and gate parameters
// (emcSurface).  emcDevice keeps its width private; it is recovered from the
// cell volume (getCellVolume = hx * hy * width).
template <class T, class DeviceType> class DeviceDesc {
public:
  using SizeVec = typename DeviceType::SizeVec;
  static_assert(std::tuple_size<SizeVec>::value == 2, "the device engine is 2-D");

  explicit DeviceDesc(const DeviceType &dev) {
    const SizeVec ext = dev.getGridExtent();
    const SizeType nx = ext[0], ny = ext[1];
    const auto h = dev.getSpacing();
    const auto mx = dev.getMaxPos();
    d_ = emcg_device_desc{};
    d_.nx = (int32_t)nx;
    d_.ny = (int32_t)ny;
    d_.hx = h[0];
    d_.hy = h[1];
    d_.max_x = mx[0];
    d_.max_y = mx[1];
    d_.width = dev.getCellVolume() / (h[0] * h[1]);
    d_.temperature = dev.getTemperature();
    d_.ni = dev.getMaterial().getNi();
    d_.eps_r = dev.getMaterial().getEpsR();
    doping_.resize(nx * ny);
    region_.resize(nx * ny);
    const auto &dp = dev.getDopingProfile();
    for (SizeType y = 0; y < ny; y++)
      for (SizeType x = 0; x < nx; x++) {
        const SizeVec c = {x, y};
        doping_[y * nx + x] = dp.getDoping(c);
        region_[y * nx + x] = dp.getDopingRegionIdx(c);
      }
    const auto &sf = dev.getSurface();
    for (int b = 0; b < 4; b++) {
      const SizeType len = b < 2 ? ny : nx;
      bnd_[b].resize(len);
      for (SizeType c = 0; c < len; c++)
        bnd_[b][c] = sf.getContactIdx(std::array<SizeType, 1>{c}, (emcBoundaryPos)b);
      d_.boundary_contact[b] = bnd_[b].data();
    }
    const SizeType nc = sf.getNrContacts();
    for (SizeType k = 0; k < nc; k++) {
      const emcContactType t = sf.getContactType(k);
      type_.push_back(t == emcContactType::OHMIC      ? EMCG_CONTACT_OHMIC
                      : t == emcContactType::SCHOTTKY ? EMCG_CONTACT_SCHOTTKY
                                                      : EMCG_CONTACT_GATE);
      volt_.push_back(sf.getContactVoltage(k));
      for (SizeType q = 0; q < 3; q++)
        param_.push_back(t == emcContactType::GATE ? sf.getContactFurtherParameter(k, q) : 0.);
    }
    d_.doping = doping_.data();
    d_.region = region_.data();
    d_.n_contacts = (int32_t)nc;
    d_.contact_type = type_.empty() ? nullptr : type_.data();
    d_.contact_voltage = volt_.empty() ? nullptr : volt_.data();
    d_.contact_param = param_.empty() ? nullptr : param_.data();
  }
  DeviceDesc(const DeviceDesc &) = delete;
  DeviceDesc &operator=(const DeviceDesc &) = delete;

  const emcg_device_desc &desc() const { return d_; }

private:
  emcg_device_desc d_;
  std::vector<double> doping_, volt_, param_;
  std::vector<int32_t> region_, type_;
  std::vector<int32_t> bnd_[4];
};

// emcSimulation (include/emcSimulation.hpp) with particle handler, PM scheme
// and Poisson solver on the GPU, for one particle type on a 2-D device.
template <class T, class DeviceType> class GpuDeviceSimulation {
public:
  // cfg: PM scheme, dt, seed, capacity and the Poisson settings; its charge is
  // taken from the particle type
  GpuDeviceSimulation(const DeviceType &device, ModelBuilder<T, DeviceType> &model,
                      emcg_device_config cfg, int precision = EMCG_FP32)
      : dd_(device) {
    cfg.charge = model.particleType().getCharge();
    const emcg_model_desc &md = model.desc();
    check(emcg_device_create(&md, &dd_.desc(), &cfg, precision, &h_));
    nc_ = dd_.desc().n_contacts;
    model_ = &model;
  }

  // the particle type's reinitScatterTables() (include/emcScatterHandler.hpp:
  // 100-108) on the GPU, before the next performEMCStep
  void reinitScatterTables() {
    const std::vector<double> raw = model_->rawRates();
    check(emcg_update_rates(h_, 0, raw.data(), 0));
  }
  ~GpuDeviceSimulation() { emcg_destroy(h_); }
  GpuDeviceSimulation(const GpuDeviceSimulation &) = delete;
  GpuDeviceSimulation &operator=(const GpuDeviceSimulation &) = delete;

  // calcEquilibriumCharacteristics (emcSimulation.hpp:139-146): equilibrium
  // potential, field, initial particles (from the doping, or from the
  // potential), charge assignment
  void calcEquilibriumCharacteristics(bool potentialBased = false) {
    double rel = 0;
    int32_t cycles = 0;
    check(emcg_device_poisson(h_, 1, 1, &rel, &cycles));
    check(emcg_device_efield(h_));
    check(emcg_device_init(h_, potentialBased ? 1 : 0, 0));
    check(emcg_device_assign(h_));
  }

  // performEMCStep (emcSimulation.hpp:164-193) nSteps times; per step and
  // contact the netto particle count that emcSimulationResults::updateCurrent
  // takes (removed - (injected - deleted)), step-major
  std::vector<int32_t> performEMCStep(int nSteps = 1) {
    std::vector<int32_t> netto((size_t)nSteps * (nc_ > 0 ? nc_ : 1), 0);
    check(emcg_device_step(h_, nSteps, step_, netto.data()));
    step_ += (uint32_t)nSteps;
    return netto;
  }

  // EMCG_GRID_POTENTIAL (phi / Vt), EMCG_GRID_CONC (n / Ni), ...
  std::vector<double> grid(int which) const {
    std::vector<double> v((size_t)dd_.desc().nx * dd_.desc().ny);
    check(emcg_device_get_grid(h_, which, v.data()));
    return v;
  }

  SizeType getNrParticles() const { return (SizeType)emcg_num_particles(h_, 0); }

private:
  DeviceDesc<T, DeviceType> dd_;
  ModelBuilder<T, DeviceType> *model_ = nullptr;
  emcg_handle *h_ = nullptr;
  int nc_ = 0;
  uint32_t step_ = 0;
};

// ---------------------------------------------------------------------------
// Plugins of the reference's interfaces for its stock emcSimulation
// (include/emcSimulation.hpp:28-47 static_asserts these bases):
//
//   using Engine  = emcgpu::GpuEngine<T, Dev>;
//   using PM      = emcgpu::GpuPMScheme<T, Dev, emcNGPScheme<T, Dev>>;
//   using Handler = emcgpu::GpuParticleHandler<T, Dev, PM>;
//   using Solver  = emcgpu::GpuPoissonSolver<T, Dev, Handler>;
//   emcSimulation<T, Dev, Solver, Handler, PM> simulation(param, device, solver, pm);
//
// The three share one device engine (GpuEngine), created at its first use.
// The host grids emcSimulation passes between them (potential, field,
// particle counts, concentration) cross the boundary at every call, so the
// reference's results, averages and output files are its own; the particles
// stay on the GPU.  The initial particles are made by the reference's
// emcAbstractParticleHandler::generateInitialParticles (its counts and its
// random-number stream) through addParticle, and uploaded before the first
// move; moves, contacts and injection then run on the GPU engine.
// ---------------------------------------------------------------------------

// EMCG_PM_* of a reference PM scheme class
template <class S> struct PmKindOf {
  static constexpr int value = -1;
};
template <class T, class D> struct PmKindOf<emcNGPScheme<T, D>> {
  static constexpr int value = EMCG_PM_NGP;
};
template <class T, class D> struct PmKindOf<emcCICScheme<T, D>> {
  static constexpr int value = EMCG_PM_CIC;
};
template <class T, class D> struct PmKindOf<emcNECScheme<T, D>> {
  static constexpr int value = EMCG_PM_NEC;
};

// The device engine behind the plugins: one particle type (index 0) on a 2-D
// device.  cfg: dt (= emcSimulationParameter's step time), Poisson settings,
// capacity (0: from the device's doping); the PM scheme, charge, seed and
// carriers per particle are set by the plugins.
template <class T, class DeviceType> class GpuEngine {
public:
  using Grid = emcGrid<T, 2>;

  GpuEngine(const DeviceType &device, ModelBuilder<T, DeviceType> &model, emcg_device_config cfg,
            int precision = EMCG_FP32)
      : dd_(device), model_(model), cfg_(cfg), precision_(precision) {
    if (cfg_.capacity == 0) { // 1.6 x the doping's carriers, as the Python host
      double sum = 0;
      const emcg_device_desc &d = dd_.desc();
      for (int i = 0; i < d.nx * d.ny; i++)
        sum += std::abs(d.doping[i]);
      cfg_.capacity = (int64_t)(1.6 * std::max(sum, 1.) * device.getCellVolume()) + 4096;
    }
  }
  ~GpuEngine() {
    if (h_)
      emcg_destroy(h_);
  }
  GpuEngine(const GpuEngine &) = delete;
  GpuEngine &operator=(const GpuEngine &) = delete;

  // settings, before the engine's first use
  emcg_device_config &config() {
    if (h_)
      emcMessage::getInstance()
          .addError("libemcgpu: the engine's settings are fixed at its first use")
          .print();
    return cfg_;
  }

  emcg_handle *handle() {
    if (!h_) {
      cfg_.charge = model_.particleType().getCharge();
      const emcg_model_desc &md = model_.desc();
      check(emcg_device_create(&md, &dd_.desc(), &cfg_, precision_, &h_));
    }
    return h_;
  }
  const emcg_device_config &settings() const { return cfg_; }
  int nContacts() const { return dd_.desc().n_contacts; }

  void toGrid(int which, const Grid &g) {
    buf_.assign(g.begin(), g.end());
    check(emcg_device_set_grid(handle(), which, buf_.data()));
  }
  void fromGrid(int which, Grid &g) {
    buf_.resize(g.getSize());
    check(emcg_device_get_grid(handle(), which, buf_.data()));
    std::copy(buf_.begin(), buf_.end(), g.begin());
  }

  uint32_t step = 0; // Philox step counter of moves and injection

private:
  DeviceDesc<T, DeviceType> dd_;
  ModelBuilder<T, DeviceType> &model_;
  emcg_device_config cfg_;
  int precision_;
  emcg_handle *h_ = nullptr;
  std::vector<double> buf_;
};

// emcAbstractPMScheme on the GPU engine: the field from the potential
// (calcEField, include/PMSchemes/emcEFieldCalculation.hpp) on the GPU; the
// single-particle host methods (assignToMesh, interpolateForce), which
// emcSimulation itself never calls, from the reference scheme HostScheme.
// Copies share the engine (emcSimulation keeps a copy).
template <class T, class DeviceType, class HostScheme, int Kind = PmKindOf<HostScheme>::value>
class GpuPMScheme : public emcAbstractPMScheme<T, DeviceType> {
  static_assert(Kind >= 0, "give the engine's EMCG_PM_* kind of this PM scheme");
  static constexpr SizeType Dim = DeviceType::Dimension;

public:
  using Engine = GpuEngine<T, DeviceType>;

  explicit GpuPMScheme(std::shared_ptr<Engine> engine, HostScheme host = HostScheme())
      : engine_(std::move(engine)), host_(std::move(host)) {
    engine_->config().pm_scheme = Kind;
  }

  void assignToMesh(const std::array<T, Dim> &pos, SizeType nrCarriers,
                    const std::array<T, Dim> &spacing,
                    emcGrid<T, Dim> &grid) const override {
    host_.assignToMesh(pos, nrCarriers, spacing, grid);
  }
  void assignToMesh(const std::vector<std::array<T, Dim>> &position, SizeType nrCarriers,
                    const std::array<T, Dim> &spacing,
                    emcGrid<T, Dim> &grid) const override {
    host_.assignToMesh(position, nrCarriers, spacing, grid);
  }
  std::array<T, 3> interpolateForce(const std::vector<emcGrid<T, Dim>> &eField,
                                    const std::array<T, Dim> &pos,
                                    const std::array<T, Dim> &spacing,
                                    T charge) const override {
    return host_.interpolateForce(eField, pos, spacing, charge);
  }
  // the potential to the engine, its field back into eField
  void calcEField(std::vector<emcGrid<T, Dim>> &eField, const emcGrid<T, Dim> &potential,
                  const DeviceType &) const override {
    engine_->toGrid(EMCG_GRID_POTENTIAL, potential);
    check(emcg_device_efield(engine_->handle()));
    engine_->fromGrid(EMCG_GRID_EX, eField[0]);
    engine_->fromGrid(EMCG_GRID_EY, eField[1]);
  }

  std::shared_ptr<Engine> engine() const { return engine_; }

private:
  std::shared_ptr<Engine> engine_;
  HostScheme host_;
};

// emcAbstractSolver on the GPU engine: the multigrid / double-precision
// defect-correction solve of the reference's discrete equation
// (include/PoissonSolver/emcSORSolver.hpp:49-197), on the potential and
// concentration that emcSimulation hands over.
template <class T, class DeviceType, class ParticleHandler>
class GpuPoissonSolver : public emcAbstractSolver<T, DeviceType, ParticleHandler> {
  using GridType = typename emcAbstractSolver<T, DeviceType, ParticleHandler>::GridType;

public:
  using Engine = GpuEngine<T, DeviceType>;

  explicit GpuPoissonSolver(std::shared_ptr<Engine> engine) : engine_(std::move(engine)) {}

  void calcEquilibriumPotential(GridType &pot, const DeviceType &, bool resetBC = true) override {
    engine_->toGrid(EMCG_GRID_POTENTIAL, pot);
    double rel = 0;
    int32_t cycles = 0;
    check(emcg_device_poisson(engine_->handle(), 1, resetBC ? 1 : 0, &rel, &cycles));
    engine_->fromGrid(EMCG_GRID_POTENTIAL, pot);
  }
  void calcNonEquilibriumPotential(GridType &pot, const DeviceType &, const GridType &eConc,
                                   bool resetBC = true) override {
    engine_->toGrid(EMCG_GRID_POTENTIAL, pot);
    engine_->toGrid(EMCG_GRID_CONC, eConc);
    double rel = 0;
    int32_t cycles = 0;
    check(emcg_device_poisson(engine_->handle(), 0, resetBC ? 1 : 0, &rel, &cycles));
    engine_->fromGrid(EMCG_GRID_POTENTIAL, pot);
  }
  // the background potential of the FMM handlers: particle-particle forces
  // are not part of the device engine
  void calcBackgroundPotential(GridType &, const DeviceType &, ParticleHandler &,
                               bool = true) override {
    emcMessage::getInstance()
        .addError("libemcgpu: the device engine has no particle-particle (FMM) interaction")
        .print();
  }

private:
  std::shared_ptr<Engine> engine_;
};

// emcAbstractParticleHandler on the GPU engine, constructed by emcSimulation
// as it constructs emcBasicParticleHandler
// (include/ParticleHandler/emcBasicParticleHandler.hpp:51-59): one particle
// type (index 0) that moves and is injected.
template <class T, class DeviceType, class PMScheme>
class GpuParticleHandler : public emcAbstractParticleHandler<T, DeviceType, PMScheme, 2> {
  using Base = emcAbstractParticleHandler<T, DeviceType, PMScheme, 2>;
  using typename Base::MapIdxToParticleTypes;
  using typename Base::NettoParticleCounter;
  using typename Base::SizeVec;
  using typename Base::ValueVec;

public:
  GpuParticleHandler(const DeviceType &device, PMScheme &pmScheme, MapIdxToParticleTypes &types,
                     SizeType nrCarriersPerParticle, SizeType seed)
      : Base(device, pmScheme, nrCarriersPerParticle, types, seed),
        engine_(pmScheme.engine()), spacing_(device.getSpacing()),
        extent_(device.getGridExtent()) {
    if (types.size() != 1 || !types.count(0) || !types.at(0)->isMoved())
      emcMessage::getInstance()
          .addError("libemcgpu: one moving particle type, with index 0")
          .print();
    emcg_device_config &c = engine_->config();
    c.seed = seed;
    c.carriers_per_particle = (double)nrCarriersPerParticle;
  }

  bool calcsPartPartInteraction() const override { return false; }

  SizeType getNrParticles(SizeType = 0) const {
    return pending_.empty() && engine_ ? (SizeType)emcg_num_particles(engine_->handle(), 0)
                                       : pending_.size();
  }

  void printNrParticles() const override {
    std::cout << "\t" << getNrParticles() << " " << Base::idxTypeToPartType.at(0)->getName()
              << "\n";
  }

  void assignParticlesToMesh(SizeType, emcGrid<T, 2> &gridNrParticles) override {
    upload();
    check(emcg_device_assign(engine_->handle()));
    engine_->fromGrid(EMCG_GRID_NRPART, gridNrParticles);
  }

  // the engine moves its particles in its own field (the one calcEField just
  // computed from the same potential); removed particles per contact
  NettoParticleCounter driftScatterParticles(T tStep, std::vector<emcGrid<T, 2>> &) override {
    upload();
    if (tStep != engine_->settings().dt)
      emcMessage::getInstance()
          .addError("libemcgpu: the step time differs from the engine's dt")
          .print();
    auto counter = Base::initNettoParticleCounter();
    std::vector<int32_t> n((size_t)std::max(engine_->nContacts(), 1), 0);
    check(emcg_device_move(engine_->handle(), engine_->step, n.data()));
    for (size_t c = 0; c < counter[0].size(); c++)
      counter[0][c] = n[c];
    return counter;
  }

  // deletion of excess particles and injection at the ohmic contacts on the
  // GPU; injected minus deleted per contact
  NettoParticleCounter handleOhmicContacts() override {
    auto counter = Base::initNettoParticleCounter();
    std::vector<int32_t> n((size_t)std::max(engine_->nContacts(), 1), 0);
    check(emcg_device_contacts(engine_->handle(), engine_->step, n.data()));
    engine_->step++;
    for (size_t c = 0; c < counter[0].size(); c++)
      counter[0][c] = n[c];
    return counter;
  }

  // the particle dump of emcBasicParticleHandler::print (:194-216)
  void print(std::string namePrefix, std::string nameSuffix) override {
    const auto &type = Base::idxTypeToPartType.at(0);
    const State st = download();
    std::ofstream os(namePrefix + type->getName() + nameSuffix + ".txt");
    os << Base::device.getMaxPos() << "\n";
    for (size_t i = 0; i < st.n; i++) {
      const std::array<T, 2> pos = {st.px[i], st.py[i]};
      const std::array<T, 3> k = {st.kx[i], st.ky[i], st.kz[i]};
      os << i << " " << pos << " " << k << " " << st.energy[i] << " " << st.sub[i] << " "
         << st.valley[i] << " " << st.tau[i];
      if (i + 1 < st.n)
        os << "\n";
    }
  }

  // emcBasicParticleHandler::getChannelDriftCurrent (:224-238), from the
  // downloaded particles
  T getChannelDriftCurrent(SizeType idxType, T x0, T x1, T channelLength) const {
    const auto &type = Base::idxTypeToPartType.at(idxType);
    const State st = download();
    T sumVx = 0;
    for (size_t i = 0; i < st.n; i++) {
      if (st.px[i] < x0 || st.px[i] > x1)
        continue;
      const std::array<T, 3> k = {st.kx[i], st.ky[i], st.kz[i]};
      sumVx += type->getValley(st.valley[i])->getVelocity(k, st.energy[i], st.sub[i])[0];
    }
    return constants::q * Base::nrCarriersPerPart * sumVx / channelLength;
  }

protected:
  // the reference's particle making (initParticlePos and the particle type's
  // generateInitialParticle / generateInjectedParticle), kept on the host
  // until the next call that needs the engine
  void addParticle(SizeType idxType, const SizeVec &coord, emcRNG &rng,
                   bool isInitial) override {
    const std::array<T, 2> pos = initParticlePos(coord, extent_, spacing_, rng);
    const auto &type = Base::idxTypeToPartType.at(idxType);
    emcParticle<T> p = isInitial ? type->generateInitialParticle(coord, Base::device, rng)
                                 : type->generateInjectedParticle(coord, Base::device, rng);
    pending_.push_back({pos, p});
  }

private:
  struct State {
    size_t n = 0;
    std::vector<double> kx, ky, kz, px, py, pz, energy, tau, gtau;
    std::vector<int32_t> valley, sub, region;
    void resize(size_t m) {
      n = m;
      for (auto *v : {&kx, &ky, &kz, &px, &py, &pz, &energy, &tau, &gtau})
        v->assign(m, 0.);
      for (auto *v : {&valley, &sub, &region})
        v->assign(m, 0);
    }
    emcg_state desc() {
      emcg_state s{};
      s.kx = kx.data();
      s.ky = ky.data();
      s.kz = kz.data();
      s.px = px.data();
      s.py = py.data();
      s.pz = pz.data();
      s.energy = energy.data();
      s.tau = tau.data();
      s.grain_tau = gtau.data();
      s.valley = valley.data();
      s.sub = sub.data();
      s.region = region.data();
      s.n = (int64_t)n;
      return s;
    }
  };

  void upload() {
    if (pending_.empty())
      return;
    State st;
    st.resize(pending_.size());
    for (size_t i = 0; i < pending_.size(); i++) {
      const auto &[pos, p] = pending_[i];
      st.kx[i] = p.k[0];
      st.ky[i] = p.k[1];
      st.kz[i] = p.k[2];
      st.px[i] = pos[0];
      st.py[i] = pos[1];
      st.energy[i] = p.energy;
      st.tau[i] = p.tau;
      st.gtau[i] = p.grainTau;
      st.valley[i] = (int32_t)p.valley;
      st.sub[i] = (int32_t)p.subValley;
      st.region[i] = (int32_t)p.region;
    }
    const emcg_state s = st.desc();
    check(emcg_set_state(engine_->handle(), 0, &s));
    pending_.clear();
  }

  State download() const {
    State st;
    const int64_t n = emcg_num_particles(engine_->handle(), 0);
    st.resize((size_t)std::max<int64_t>(n, 0));
    emcg_state s = st.desc();
    check(emcg_get_state(engine_->handle(), 0, &s));
    return st;
  }

  std::shared_ptr<GpuEngine<T, DeviceType>> engine_;
  ValueVec spacing_;
  SizeVec extent_;
  std::vector<std::pair<std::array<T, 2>, emcParticle<T>>> pending_;
};

} // namespace emcgpu

#endif // EMCGPU_REFERENCE_HPP
