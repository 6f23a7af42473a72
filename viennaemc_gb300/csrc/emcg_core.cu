// Error reporting and version of libemcgpu.
#include "emcg_host.h"

namespace emcg {

static thread_local std::string g_lastError;

void setError(const char *fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_lastError = buf;
}

const char *statusName(int32_t s) {
  switch (s) {
  case EMCG_OK: return "ok";
  case EMCG_ERR_ARG: return "invalid argument";
  case EMCG_ERR_CUDA: return "CUDA error";
  case EMCG_ERR_TIMEOUT: return "bounded device loop gave up";
  case EMCG_ERR_NONCONVERGED: return "Poisson solve did not converge";
  case EMCG_ERR_OUT_OF_TABLE: return "particle in (valley, region) without rate tables";
  case EMCG_ERR_REPLAY: return "replay word stream does not match";
  case EMCG_ERR_CAPACITY: return "particle capacity exceeded";
  }
  return "unknown status";
}

} // namespace emcg

extern "C" const char *emcg_last_error(void) {
  return emcg::g_lastError.c_str();
}

extern "C" int32_t emcg_version(void) { return 100; }
