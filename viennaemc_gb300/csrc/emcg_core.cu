// Error reporting, version and page-locked host blocks of libemcgpu.
#include "emcg_host.h"

#include <cstdint>
#include <map>
#include <mutex>

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

// live emcg_host_alloc blocks: start address -> (bytes, device address)
struct HostBlock {
  size_t bytes;
  char *dev;
};
static std::mutex g_hostMu;
static std::map<uintptr_t, HostBlock> g_hostBlocks;

const void *mappedHostRange(const void *p, size_t bytes) {
  const uintptr_t a = reinterpret_cast<uintptr_t>(p);
  std::lock_guard<std::mutex> lk(g_hostMu);
  auto it = g_hostBlocks.upper_bound(a);
  if (it == g_hostBlocks.begin())
    return nullptr;
  --it;
  const uintptr_t off = a - it->first;
  if (off > it->second.bytes || bytes > it->second.bytes - off)
    return nullptr;
  return it->second.dev + off;
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
  EMCG_CUDA(cudaHostAlloc(ptr, (size_t)bytes, cudaHostAllocMapped));
  void *dev = nullptr;
  if (cudaHostGetDevicePointer(&dev, *ptr, 0) != cudaSuccess) {
    cudaGetLastError();
    dev = nullptr; // not readable by kernels: used through copies only
  }
  if (dev) {
    std::lock_guard<std::mutex> lk(emcg::g_hostMu);
    emcg::g_hostBlocks[reinterpret_cast<uintptr_t>(*ptr)] = {(size_t)bytes,
                                                             static_cast<char *>(dev)};
  }
  return EMCG_OK;
}

extern "C" int32_t emcg_host_free(void *ptr) {
  if (!ptr)
    return EMCG_OK;
  {
    std::lock_guard<std::mutex> lk(emcg::g_hostMu);
    emcg::g_hostBlocks.erase(reinterpret_cast<uintptr_t>(ptr));
  }
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
