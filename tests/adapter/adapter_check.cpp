// Builds the bulk benchmark model through emcgpu::ModelBuilder on the
// reference's own classes and prints the engine descriptor (hex floats), so
// that tests/test_adapter.py can compare it with the Python host builder.
// GpuBulkParticleHandler is instantiated to check that it compiles and links.
#include <cstdio>
#include <memory>
#include <vector>

#include <ParticleType/emcElectron.hpp>
#include <emcDevice.hpp>

#include "emcgpu_reference.hpp"

using T = double;
using Dev3 = emcDevice<T, 3>;
using Dev2 = emcDevice<T, 2>;
template class emcgpu::GpuBulkParticleHandler<T, Dev3>;
template class emcgpu::GpuDeviceSimulation<T, Dev2>;

int main() {
  Dev3 device{emcMaterial<T>{11.8, 2329., 1.45e16, 9040., 1.15}, {5e-7, 5e-7, 5e-7},
              {1e-7, 1e-7, 1e-7}, 300.};
  device.addConstantDopingRegion({0, 0, 0}, {5e-7, 5e-7, 5e-7}, 1e21);
  emcElectron<T, Dev3> el(1000, 1., false);
  std::unique_ptr<emcNonParabolicAnisotropValley<T>> v(
      new emcNonParabolicAnisotropValley<T>({0.916, 0.19, 0.19}, el.getMass(), 3, 0.5));
  v->setSubValleyEllipseCoordSystem(0, {1, 0, 0}, {0, 1, 0}, {0, 0, 1});
  v->setSubValleyEllipseCoordSystem(1, {0, 1, 0}, {1, 0, 0}, {0, 0, 1});
  v->setSubValleyEllipseCoordSystem(2, {0, 0, 1}, {0, 1, 0}, {1, 0, 0});
  el.addValley(std::move(v));
  emcgpu::ModelBuilder<T, Dev3> mb(el, 1000, 1.);
  std::map<SizeType, std::vector<SizeType>> G = {{0, {0}}, {1, {1}}, {2, {2}}};
  std::map<SizeType, std::vector<SizeType>> F = {{0, {1, 1, 2, 2}}, {1, {0, 0, 2, 2}},
                                                 {2, {0, 0, 1, 1}}};
  mb.addAcoustic(0, 9., device, {0});
  const double th[6] = {140., 215., 720., 220., 550., 685.};
  const double D[6] = {0.5e10, 0.8e10, 11.e10, 0.3e10, 2.0e10, 2.0e10};
  const char *nm[6] = {"G1", "G2", "G3", "F1", "F2", "F3"};
  for (int i = 0; i < 6; i++) {
    double e = constants::kB * th[i] / constants::q;
    mb.addZeroOrderAbsorption(nm[i], 0, i < 3 ? G : F, D[i], e, device, {0});
    mb.addZeroOrderEmission(nm[i], 0, i < 3 ? G : F, D[i], e, device, {0});
  }
  const emcg_model_desc &d = mb.desc();
  std::printf("counts %d %d %d %d\n", d.n_valleys, d.n_mechs, d.n_tablesets, d.n_levels);
  std::printf("tau %a\n", d.tablesets[0].tau_max);
  for (int i = 0; i < 3; i++)
    std::printf("relmass %a\n", d.valleys[0].rel_mass[i]);
  for (int m = 0; m < d.n_mechs; m++)
    std::printf("mech %d %d %a %d\n", d.mechs[m].kind, d.mechs[m].n_final, d.mechs[m].shift,
                d.mechs[m].final_sub[1][0]);
  for (int i = 0; i < d.n_mechs * d.n_levels; i += 97)
    std::printf("table %d %a\n", i, d.tables[i]);
  // the refilled rates that reinitScatterTables hands to emcg_update_rates
  const std::vector<double> raw = mb.rawRates();
  std::printf("rawcount %zu\n", raw.size());
  for (size_t i = 0; i < raw.size(); i += 89)
    std::printf("raw %zu %a\n", i, raw[i]);
  // a gated 2-D device described through DeviceDesc
  Dev2 dev2{emcMaterial<T>{11.8, 2329., 1.45e16, 9040., 1.15}, {30e-9, 20e-9}, {1e-9, 1e-9},
            300.};
  dev2.setDeviceWidth(3e-8);
  dev2.addConstantDopingRegion({0, 8e-9}, {30e-9, 20e-9}, -1e24);
  dev2.addConstantDopingRegion({0, 0}, {10e-9, 8e-9}, 1e26);
  dev2.addConstantDopingRegion({10e-9, 0}, {20e-9, 8e-9}, -1e24);
  dev2.addConstantDopingRegion({20e-9, 0}, {30e-9, 8e-9}, 1e26);
  dev2.addOhmicContact(emcBoundaryPos::YMAX, 0, {0}, {30e-9});
  dev2.addOhmicContact(emcBoundaryPos::YMIN, 0, {0}, {10e-9});
  dev2.addGateContact(emcBoundaryPos::YMIN, 1.0, {10e-9}, {20e-9}, 3.9, 1.2e-9, 1.15 / 2.0);
  dev2.addOhmicContact(emcBoundaryPos::YMIN, 0.5, {20e-9}, {30e-9});
  emcgpu::DeviceDesc<T, Dev2> dd(dev2);
  const emcg_device_desc &g = dd.desc();
  std::printf("dev %d %d %a %a %a %a %a %a %a %a\n", g.nx, g.ny, g.hx, g.hy, g.max_x, g.max_y,
              g.width, g.temperature, g.ni, g.eps_r);
  for (int i = 0; i < g.nx * g.ny; i++)
    std::printf("node %d %a %d\n", i, g.doping[i], g.region[i]);
  for (int b = 0; b < 4; b++)
    for (int c = 0; c < (b < 2 ? g.ny : g.nx); c++)
      std::printf("bnd %d %d %d\n", b, c, g.boundary_contact[b][c]);
  for (int k = 0; k < g.n_contacts; k++)
    std::printf("contact %d %d %a %a %a %a\n", k, g.contact_type[k], g.contact_voltage[k],
                g.contact_param[3 * k], g.contact_param[3 * k + 1], g.contact_param[3 * k + 2]);
  // a grain mechanism set through the builder (and forwarded to the type)
  emcElectron<T, Dev3> el2(1000, 1., false);
  std::unique_ptr<emcNonParabolicAnisotropValley<T>> v2(
      new emcNonParabolicAnisotropValley<T>({0.916, 0.19, 0.19}, el2.getMass(), 3, 0.5));
  el2.addValley(std::move(v2));
  emcgpu::ModelBuilder<T, Dev3> mb2(el2, 1000, 1.);
  mb2.addAcoustic(0, 9., device, {0});
  mb2.setGrainScatterMechanism(0.3, 2e14);
  mb2.setConstantSurfaceScatterMechanism(emcBoundaryPos::YMIN, 0.3, {5e-7, 5e-7, 5e-7});
  mb2.setMomentumDependentSurfaceScatterMechanism(emcBoundaryPos::YMAX, 0.5e-9,
                                                  {5e-7, 5e-7, 5e-7});
  const emcg_model_desc &d2 = mb2.desc();
  std::printf("grain %d %a %a\n", d2.grain, d2.grain_transmission, d2.grain_tau);
  std::printf("surface %d %d %d %d %a %a %a %a\n", d2.surface_kind[0], d2.surface_kind[1],
              d2.surface_kind[2], d2.surface_kind[3], d2.surface_param[0], d2.surface_param[1],
              d2.surface_param[2], d2.surface_param[3]);
  std::printf("nograin %d %a\n", d.grain, d.grain_tau);
  return 0;
}
