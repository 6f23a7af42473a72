// The reference's stock emcSimulation with the GPU plugins as its template
// arguments (only those changed): a 2-D n+ resistor, 21 x 11 nodes, NGP,
// acoustic + Coulomb + zero-order f/g phonons, registered through
// emcgpu::ModelBuilder.  Compiling it checks emcSimulation's static_asserts
// on the plugin bases; running it (against the recording stand-in of
// libemcgpu in stub_emcgpu.cpp, or the engine itself) executes the
// reference's own step loop through the plugins and writes the reference's
// output files under the name prefix given as argv[1].
#include <cstdio>
#include <memory>
#include <string>

#include <ParticleType/emcElectron.hpp>
#include <emcDevice.hpp>
#include <emcSimulation.hpp>

#include "emcgpu_reference.hpp"

using T = double;
using Dev = emcDevice<T, 2>;
using Engine = emcgpu::GpuEngine<T, Dev>;
using PM = emcgpu::GpuPMScheme<T, Dev, emcNGPScheme<T, Dev>>;
using Handler = emcgpu::GpuParticleHandler<T, Dev, PM>;
using Solver = emcgpu::GpuPoissonSolver<T, Dev, Handler>;
using Simulation = emcSimulation<T, Dev, Solver, Handler, PM>;

int main(int argc, char **argv) {
  const std::string prefix = argc > 1 ? argv[1] : "gpu_resistor";
  const int steps = argc > 2 ? std::atoi(argv[2]) : 6;
  const T dt = 1e-15;
  emcMaterial<T> si{11.8, 2329., 1.45e16, 9040., 1.15};
  Dev device{si, {20e-9, 10e-9}, {1e-9, 1e-9}, 300.};
  device.setDeviceWidth(3e-7);
  device.addConstantDopingRegion({0, 0}, {20e-9, 10e-9}, 1e25);
  device.addOhmicContact(emcBoundaryPos::XMAX, 0, {0}, {10e-9});
  device.addOhmicContact(emcBoundaryPos::XMIN, 0.1, {0}, {10e-9});

  auto electrons = std::make_unique<emcElectron<T, Dev>>(1000, 4., false);
  std::unique_ptr<emcNonParabolicAnisotropValley<T>> v(
      new emcNonParabolicAnisotropValley<T>({0.916, 0.196, 0.196}, electrons->getMass(), 3, 0.5));
  v->setSubValleyEllipseCoordSystem(0, {1, 0, 0}, {0, 1, 0}, {0, 0, 1});
  v->setSubValleyEllipseCoordSystem(1, {0, 1, 0}, {1, 0, 0}, {0, 0, 1});
  v->setSubValleyEllipseCoordSystem(2, {0, 0, 1}, {0, 1, 0}, {1, 0, 0});
  electrons->addValley(std::move(v));
  emcgpu::ModelBuilder<T, Dev> mb(*electrons, 1000, 4.);
  const std::map<SizeType, std::vector<SizeType>> G = {{0, {0}}, {1, {1}}, {2, {2}}};
  const std::map<SizeType, std::vector<SizeType>> F = {{0, {1, 1, 2, 2}}, {1, {0, 0, 2, 2}},
                                                       {2, {0, 0, 1, 1}}};
  mb.addAcoustic(0, 9., device, {0});
  mb.addCoulomb(0, 11.8, device, {0});
  mb.addZeroOrderAbsorption("F", 0, F, 5.23e10, 0.06, device, {0});
  mb.addZeroOrderEmission("F", 0, F, 5.23e10, 0.06, device, {0});
  mb.addZeroOrderAbsorption("G", 0, G, 5.23e10, 0.06, device, {0});
  mb.addZeroOrderEmission("G", 0, G, 5.23e10, 0.06, device, {0});

  emcSimulationParameter<T, Dev> param;
  param.setTimes(steps * dt, dt, 2 * dt); // two transient steps
  param.setNamePrefix(prefix);
  param.setNrStepsForFinalAvg(steps);
  param.setSeed(42);
  param.addParticleType(std::move(electrons));

  emcg_device_config cfg{};
  cfg.dt = dt;
  cfg.poisson_rtol = 1e-10;
  cfg.poisson_max_cycles = 200;
  cfg.poisson_fp32 = 1;
  auto engine = std::make_shared<Engine>(device, mb, cfg, EMCG_FP64);
  PM pm(engine);
  Solver solver(engine);
  Simulation simulation(param, device, solver, pm);
  simulation.execute();
  std::printf("done %d steps\n", steps);
  return 0;
}
