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

extern "C" int32_t emcg_host_alloc(int64_t bytes, void **ptr) {
  EMCG_CHECK_ARG(ptr && bytes >= 0, "bad host allocation request");
  *ptr = nullptr;
  if (bytes == 0)
    return EMCG_OK;
  EMCG_CUDA(cudaHostAlloc(ptr, (size_t)bytes, cudaHostAllocDefault));
  return EMCG_OK;
}

extern "C" int32_t emcg_host_free(void *ptr) {
  if (ptr)
    EMCG_CUDA(cudaFreeHost(ptr));
  return EMCG_OK;
}

extern "C" int32_t emcg_update_rates(emcg_handle *h, int32_t model, const double *raw,
                                     int32_t raw_on_device) {
  EMCG_CHECK_ARG(h, "handle is NULL");
  if (h->kind == 2) {
    EMCG_CHECK_ARG(model == 0, "a device engine has one model (index 0)");
    return emcg::deviceUpdateRates(h, raw, raw_on_device != 0);
  }
  return emcg::bulkUpdateRates(h, model, raw, raw_on_device != 0);
}

extern "C" int32_t emcg_get_rates(emcg_handle *h, int32_t model, double *tables, double *tau) {
  EMCG_CHECK_ARG(h, "handle is NULL");
  if (h->kind == 2) {
    EMCG_CHECK_ARG(model == 0, "a device engine has one model (index 0)");
    return emcg::deviceGetRates(h, tables, tau);
  }
  return emcg::bulkGetRates(h, model, tables, tau);
}
