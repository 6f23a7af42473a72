// Rate-table rebuild on the GPU: emcScatterHandler::reinitScatterTables
// (include/emcScatterHandler.hpp:100-108), which clears the tables, refills
// them from getScatterRate (fillScatterTables, :220-235) and renormalises them
// (renormalizeTables, :248-273).  The caller supplies the refilled rates -- on
// the host, or on the device where a kernel (e.g. a phonon bath) made them --
// and the GPU forms, per (valley, region) table set:
//   cum_0 = rate_0,  cum_t = rate_t + cum_{t-1}      (std::plus, in table order)
//   Gmax  = max over levels of cum_{n-1}
//   table_t = cum_t / Gmax,  tau = 1 / Gmax
// in double, then stores the tables level-major in the engine's precision in
// place of the old ones.  The launch is ordered on the handle's stream, so the
// next step sees the new tables; a captured step graph reads them through the
// same pointers.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "emcg_common.cuh"
#include "emcg_host.h"

namespace emcg {

// Table layout of one model, kept on the host at creation.
struct RateLayout {
  int nTS = 0, nLevels = 0;
  int32_t tsN[EMCG_MAX_TABLESETS] = {};
  int64_t total = 0; // doubles of a raw table array
};

inline RateLayout rateLayoutOf(const emcg_model_desc &m) {
  RateLayout R;
  R.nTS = m.n_tablesets;
  R.nLevels = m.n_levels;
  for (int t = 0; t < m.n_tablesets; t++) {
    R.tsN[t] = m.tablesets[t].n_tables;
    R.total += (int64_t)m.tablesets[t].n_tables * m.n_levels;
  }
  return R;
}

constexpr int kRenormThreads = 256;

// One block per table set.  Pass 1 forms the last cumulative row per level
// and its maximum; pass 2 forms the cumulative rows again (the same
// operations, so the same bits) and stores them divided by the maximum.  A
// set with a non-finite rate or a maximum that is not positive is left as it
// was and EMCG_ERR_ARG is recorded (the reference would divide by it).
template <class T>
__global__ void __launch_bounds__(kRenormThreads)
    renormRatesKernel(const double *__restrict__ raw, ModelK<T> *model, T *tables, int *err) {
  __shared__ double wmax[kRenormThreads / 32];
  __shared__ double gmax;
  const int ts = blockIdx.x;
  const int nT = model->tsN[ts];
  if (nT == 0) // no mechanism: the default free-flight time stays (:250-251)
    return;
  const int L = model->nLevels;
  const int64_t off = model->tsOff[ts];
  const double *r = raw + off;
  double mx = -INFINITY;
  int bad = 0;
  for (int l = threadIdx.x; l < L; l += blockDim.x) {
    double c = r[l];
    bad |= !isfinite(c);
    for (int t = 1; t < nT; t++) {
      const double x = r[(int64_t)t * L + l];
      bad |= !isfinite(x);
      c = x + c;
    }
    mx = fmax(mx, c);
  }
  for (int o = 16; o > 0; o >>= 1)
    mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0)
    wmax[threadIdx.x >> 5] = mx;
  bad = __syncthreads_or(bad);
  if (threadIdx.x == 0) {
    double m = wmax[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); w++)
      m = fmax(m, wmax[w]);
    gmax = m;
  }
  __syncthreads();
  const double g = gmax;
  if (bad || !(g > 0.0) || !isfinite(g)) {
    if (threadIdx.x == 0)
      atomicCAS(err, 0, EMCG_ERR_ARG);
    return;
  }
  T *dst = tables + off;
  for (int l = threadIdx.x; l < L; l += blockDim.x) {
    double c = r[l];
    dst[(int64_t)l * nT] = (T)(c / g);
    for (int t = 1; t < nT; t++) {
      c = r[(int64_t)t * L + l] + c;
      dst[(int64_t)l * nT + t] = (T)(c / g);
    }
  }
  if (threadIdx.x == 0)
    model->tauMax[ts] = (T)(1.0 / g);
}

// Host-side checks of host rates: every rate finite, every set's maximum
// cumulative rate positive.
inline int32_t checkHostRates(const RateLayout &R, const double *raw) {
  int64_t off = 0;
  const int L = R.nLevels;
  for (int s = 0; s < R.nTS; s++) {
    const int nT = R.tsN[s];
    if (nT == 0)
      continue;
    double mx = -INFINITY;
    for (int l = 0; l < L; l++) {
      double c = 0;
      for (int t = 0; t < nT; t++) {
        const double x = raw[off + (int64_t)t * L + l];
        EMCG_CHECK_ARG(std::isfinite(x), "table set %d, table %d, level %d: rate not finite", s,
                       t, l);
        c = t ? x + c : x;
      }
      mx = std::fmax(mx, c);
    }
    EMCG_CHECK_ARG(mx > 0, "table set %d: the maximum cumulative rate is not positive", s);
    off += (int64_t)nT * L;
  }
  return EMCG_OK;
}

// Launch the rebuild of one model.  raw: host or device doubles (onDevice);
// host rates go through the handle's staging buffer (grown on demand).
template <class T>
int32_t launchRateUpdate(void *dModel, void *dTables, const RateLayout &R, const double *raw,
                         bool onDevice, double **stage, int64_t *stageCap, int *dErr,
                         cudaStream_t st) {
  EMCG_CHECK_ARG(raw != nullptr, "rates: raw is NULL");
  if (R.total == 0)
    return EMCG_OK;
  const double *src = raw;
  if (onDevice) {
    cudaPointerAttributes a;
    EMCG_CUDA(cudaPointerGetAttributes(&a, raw));
    int dev = 0;
    EMCG_CUDA(cudaGetDevice(&dev));
    EMCG_CHECK_ARG((a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) &&
                       a.device == dev,
                   "rates: raw is not device memory of the handle's device");
  } else {
    EMCG_TRY(checkHostRates(R, raw));
    if (*stageCap < R.total) {
      EMCG_CUDA(cudaStreamSynchronize(st)); // an earlier rebuild may still read it
      cudaFree(*stage);
      *stage = nullptr;
      *stageCap = 0;
      EMCG_CUDA(cudaMalloc(stage, (size_t)R.total * sizeof(double)));
      *stageCap = R.total;
    }
    EMCG_CUDA(cudaMemcpyAsync(*stage, raw, (size_t)R.total * sizeof(double),
                              cudaMemcpyHostToDevice, st));
    src = *stage;
  }
  renormRatesKernel<T><<<R.nTS, kRenormThreads, 0, st>>>(src, (ModelK<T> *)dModel, (T *)dTables,
                                                         dErr);
  EMCG_CUDA(cudaGetLastError());
  return EMCG_OK;
}

// The engine's current tables of one model, table-major in double (the layout
// of the raw rates), and tau per table set.  Synchronises the stream.
template <class T>
int32_t readRateTables(const void *dModel, const void *dTables, const RateLayout &R,
                       double *tables, double *tau, cudaStream_t st) {
  ModelK<T> K;
  EMCG_CUDA(cudaMemcpyAsync(&K, dModel, sizeof(K), cudaMemcpyDeviceToHost, st));
  std::vector<T> tab((size_t)std::max<int64_t>(R.total, 1));
  if (R.total > 0)
    EMCG_CUDA(cudaMemcpyAsync(tab.data(), dTables, (size_t)R.total * sizeof(T),
                              cudaMemcpyDeviceToHost, st));
  EMCG_CUDA(cudaStreamSynchronize(st));
  const int L = R.nLevels;
  int64_t off = 0;
  for (int s = 0; s < R.nTS; s++) {
    const int nT = R.tsN[s];
    if (tables)
      for (int t = 0; t < nT; t++)
        for (int l = 0; l < L; l++)
          tables[off + (int64_t)t * L + l] = (double)tab[(size_t)(off + (int64_t)l * nT + t)];
    if (tau)
      tau[s] = (double)K.tauMax[s];
    off += (int64_t)nT * L;
  }
  return EMCG_OK;
}

} // namespace emcg
