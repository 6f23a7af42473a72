// Host-side helpers shared by the translation units of libemcgpu.
#pragma once

#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <string>

#include "emcgpu.h"

namespace emcg {

void setError(const char *fmt, ...);

// Return EMCG_ERR_CUDA (with the CUDA message) if a runtime call failed.
#define EMCG_CUDA(call)                                                        \
  do {                                                                         \
    cudaError_t e_ = (call);                                                   \
    if (e_ != cudaSuccess) {                                                   \
      ::emcg::setError("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                       __FILE__, __LINE__);                                    \
      return EMCG_ERR_CUDA;                                                    \
    }                                                                          \
  } while (0)

#define EMCG_CHECK_ARG(cond, ...)                                              \
  do {                                                                         \
    if (!(cond)) {                                                             \
      ::emcg::setError(__VA_ARGS__);                                           \
      return EMCG_ERR_ARG;                                                     \
    }                                                                          \
  } while (0)

#define EMCG_TRY(expr)                                                         \
  do {                                                                         \
    int32_t s_ = (expr);                                                       \
    if (s_ != EMCG_OK)                                                         \
      return s_;                                                               \
  } while (0)

const char *statusName(int32_t s);

// The device address of host bytes [p, p + bytes) when they lie inside one
// live emcg_host_alloc block (page-locked, mapped into the device's address
// space), else nullptr: only such ranges are read by kernels over the host link.
const void *mappedHostRange(const void *p, size_t bytes);

struct BulkImpl;
struct DeviceImpl;


} // namespace emcg

struct emcg_handle;
namespace emcg {
// rate-table rebuild (emcg_bulk.cu, emcg_device.cu)
int32_t bulkUpdateRates(emcg_handle *h, int model, const double *raw, bool onDevice);
int32_t bulkGetRates(emcg_handle *h, int model, double *tables, double *tau);
int32_t deviceUpdateRates(emcg_handle *h, const double *raw, bool onDevice);
int32_t deviceGetRates(emcg_handle *h, double *tables, double *tau);
// emcg_device.cu
int32_t destroyDevice(emcg_handle *h);
int32_t deviceSetState(emcg_handle *h, const emcg_state *s);
int32_t deviceGetState(emcg_handle *h, emcg_state *s);
int64_t deviceNumParticles(emcg_handle *h);
}

struct emcg_handle {
  int kind = 0; // 1 = bulk, 2 = device
  emcg::BulkImpl *bulk = nullptr;
  emcg::DeviceImpl *dev = nullptr;
};
