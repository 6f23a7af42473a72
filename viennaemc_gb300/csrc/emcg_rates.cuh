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
// place of the old ones.  The launches are ordered on the handle's stream, so
// the next step sees the new tables; a captured step graph reads them through
// the same pointers.
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

// Device scratch of a handle's rebuilds: staged host rates and the per-chunk
// maxima of pass 1.
struct RateScratch {
  double *stage = nullptr;
  int64_t stageCap = 0;
  double *part = nullptr;
  int64_t partCap = 0;
};

inline void freeRateScratch(RateScratch &S) {
  cudaFree(S.stage);
  cudaFree(S.part);
  S = RateScratch{};
}

__device__ __forceinline__ double blockMaxOr(double v, int *bad) {
  __shared__ double w[kRenormThreads / 32];
  for (int o = 16; o > 0; o >>= 1)
    v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  if ((threadIdx.x & 31) == 0)
    w[threadIdx.x >> 5] = v;
  *bad = __syncthreads_or(*bad);
  double m = w[0];
  for (int i = 1; i < (int)(blockDim.x >> 5); i++)
    m = fmax(m, w[i]);
  return m;
}

// Pass 1, one thread per (table set, level): the last cumulative row and its
// maximum per chunk of kRenormThreads levels; NaN marks a chunk with a
// non-finite rate.
template <class T>
__global__ void __launch_bounds__(kRenormThreads)
    rateMaxKernel(const double *__restrict__ raw, const ModelK<T> *__restrict__ model,
                  double *__restrict__ part, int nChunks) {
  const int ts = blockIdx.y, ch = blockIdx.x;
  const int nT = model->tsN[ts], L = model->nLevels;
  const int l = ch * kRenormThreads + threadIdx.x;
  double c = -INFINITY;
  int bad = 0;
  if (nT > 0 && l < L) {
    const double *r = raw + model->tsOff[ts] + l;
    c = r[0];
    bad = !isfinite(c);
    for (int t = 1; t < nT; t++) {
      const double x = r[(int64_t)t * L];
      bad |= !isfinite(x);
      c = x + c;
    }
  }
  const double m = blockMaxOr(c, &bad);
  if (threadIdx.x == 0)
    part[(int64_t)ts * nChunks + ch] = bad ? NAN : m;
}

// Pass 2: the set's maximum from the chunk maxima, then the cumulative rows
// again (the same operations, so the same bits) divided by it, stored
// level-major in the engine's precision; tau = 1 / maximum.  A set with a
// non-finite rate or a maximum that is not positive is left as it was and
// EMCG_ERR_ARG is recorded (the reference would divide by it).
template <class T>
__global__ void __launch_bounds__(kRenormThreads)
    rateNormKernel(const double *__restrict__ raw, ModelK<T> *model, T *tables,
                   const double *__restrict__ part, int nChunks, int *err) {
  const int ts = blockIdx.y, ch = blockIdx.x;
  const int nT = model->tsN[ts], L = model->nLevels;
  if (nT == 0) // no mechanism: the default free-flight time stays (:250-251)
    return;
  double g = -INFINITY;
  bool bad = false;
  for (int i = 0; i < nChunks; i++) {
    const double p = part[(int64_t)ts * nChunks + i];
    bad |= isnan(p);
    g = fmax(g, p);
  }
  if (bad || !(g > 0.0) || !isfinite(g)) {
    if (ch == 0 && threadIdx.x == 0)
      atomicCAS(err, 0, EMCG_ERR_ARG);
    return;
  }
  const int l = ch * kRenormThreads + threadIdx.x;
  if (l < L) {
    const int64_t off = model->tsOff[ts];
    const double *r = raw + off + l;
    T *dst = tables + off + (int64_t)l * nT;
    double c = r[0];
    dst[0] = (T)(c / g);
    for (int t = 1; t < nT; t++) {
      c = r[(int64_t)t * L] + c;
      dst[t] = (T)(c / g);
    }
  }
  if (ch == 0 && threadIdx.x == 0)
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

// Grow a scratch buffer of doubles (after the stream has drained: an earlier
// rebuild may still read the old one).
inline int32_t growScratch(double **p, int64_t *cap, int64_t n, cudaStream_t st) {
  if (*cap >= n)
    return EMCG_OK;
  EMCG_CUDA(cudaStreamSynchronize(st));
  cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  EMCG_CUDA(cudaMalloc(p, (size_t)n * sizeof(double)));
  *cap = n;
  return EMCG_OK;
}

// Launch the rebuild of one model: pass 1 and pass 2 over a grid of
// (level chunk, table set).  raw: host or device doubles (onDevice); host
// rates go through the handle's staging buffer.
template <class T>
int32_t launchRateUpdate(void *dModel, void *dTables, const RateLayout &R, const double *raw,
                         bool onDevice, RateScratch &S, int *dErr, cudaStream_t st) {
  EMCG_CHECK_ARG(raw != nullptr, "rates: raw is NULL");
  if (R.total == 0)
    return EMCG_OK;
  const int nChunks = (R.nLevels + kRenormThreads - 1) / kRenormThreads;
  EMCG_TRY(growScratch(&S.part, &S.partCap, (int64_t)R.nTS * nChunks, st));
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
    EMCG_TRY(growScratch(&S.stage, &S.stageCap, R.total, st));
    EMCG_CUDA(cudaMemcpyAsync(S.stage, raw, (size_t)R.total * sizeof(double),
                              cudaMemcpyHostToDevice, st));
    src = S.stage;
  }
  const dim3 grid(nChunks, R.nTS);
  rateMaxKernel<T><<<grid, kRenormThreads, 0, st>>>(src, (const ModelK<T> *)dModel, S.part,
                                                    nChunks);
  EMCG_CUDA(cudaGetLastError());
  rateNormKernel<T><<<grid, kRenormThreads, 0, st>>>(src, (ModelK<T> *)dModel, (T *)dTables,
                                                     S.part, nChunks, dErr);
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
