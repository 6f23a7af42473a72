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
#include <vector>

#include <ParticleType/emcParticleType.hpp>
#include <ScatterMechanisms/emcAcousticScatterMechanism.hpp>
#include <ScatterMechanisms/emcCoulombScatterMechanism.hpp>
#include <ScatterMechanisms/emcFirstOrderInterValleyScatterMechanism.hpp>
#include <ScatterMechanisms/emcZeroOrderInterValleyScatterMechanism.hpp>
#include <ValleyTypes/emcNonParabolicAnistropValley.hpp>
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
    d_.grain_tau = pt_.getGrainTau();
    d_.valleys = valleys_.data();
    d_.mechs = mechs_.data();
    d_.tablesets = sets_.data();
    d_.tables = tables_.data();
    for (int r = 0; r < EMCG_MAX_REGIONS; r++)
      d_.region_doping[r] = regionDoping_[r];
    return d_;
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
  emcg_model_desc d_{};
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

} // namespace emcgpu

#endif // EMCGPU_REFERENCE_HPP
