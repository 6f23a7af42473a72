// Device (2-D) engine: Poisson -> E field -> drift/scatter with boundaries
// -> ohmic contacts -> charge assignment (include/emcSimulation.hpp:164-193).
#include "emcg_host.h"

namespace emcg {
int32_t destroyDevice(emcg_handle *h) {
  (void)h;
  return EMCG_OK;
}
} // namespace emcg
