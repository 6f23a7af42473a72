// Particle-particle Coulomb sums of the reference's FMM particle handlers
// (include/ParticleHandler/emcFMMParticleHandler.hpp,
// examples/bulkSimulationFMM/FMMBulkParticleHandler.hpp), evaluated directly on
// the GPU in place of scalFMM's fast multipole method.
//
// For every target i and every other particle j (and every periodic copy of
// the box), the pair term of FP2PRCutoff::NonMutualParticles
// (include/ParticleHandler/FMM/FP2PRCutoff.hpp:64-100):
//   d = x_i - x_j, 1/r^2 and 1/r; closer than the cutoff radius the separation
//   is rescaled to the cutoff and 1/r, 1/r^2 take the cutoff's values;
//   force_i += -q_i q_j d / r^3,   potential_i += q_j / r.
// These are the sums scalFMM leaves in its particle containers; the handlers
// multiply them by their Coulomb factor (ke / eps_r, with their sign).
//
// Layout: two targets per thread; the sources staged through shared memory in
// tiles of one block as (x, y, z, q) quadruples, one vector load feeding two
// pair terms; when the targets alone give too few blocks, the sources are
// split into chunks over a second grid dimension and the chunks' partial sums
// are added in order afterwards.  The pair arithmetic runs in the engine's
// precision (float: rsqrt), each tile's partial sums go to double
// accumulators.  The work is n^2 pair terms of about 20 operations: bound by
// the FP32 (or FP64) pipes, not by memory.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "emcg_host.h"

namespace emcg {

constexpr int kP2PThreads = 256;
constexpr int kP2PTargets = 2; // targets per thread: one tile entry feeds two pair terms

template <class T> struct Src4 { T x, y, z, q; };
template <> struct __align__(16) Src4<float> { float x, y, z, q; };
template <> struct __align__(16) Src4<double> { double x, y, z, q; };

template <class T> __device__ __forceinline__ void invDistance(T r2, T &inv2, T &inv);
template <> __device__ __forceinline__ void invDistance<double>(double r2, double &inv2,
                                                               double &inv) {
  inv2 = 1.0 / r2; // the reference's order: 1 / r^2, then its square root
  inv = sqrt(inv2);
}
template <> __device__ __forceinline__ void invDistance<float>(float r2, float &inv2,
                                                              float &inv) {
  inv = rsqrtf(r2);
  inv2 = inv * inv;
}

// One pair term of NonMutualParticles (FP2PRCutoff.hpp:64-100) added to acc.
template <class T>
__device__ __forceinline__ void pairTerm(T xi, T yi, T zi, T qi, const Src4<T> &s, T invCut,
                                         T cut, T invCut2, T acc[4]) {
  T dx = xi - s.x, dy = yi - s.y, dz = zi - s.z;
  T inv2, inv;
  invDistance<T>(dx * dx + dy * dy + dz * dz, inv2, inv);
  if (inv > invCut) { // closer than the cutoff (:76-86); invCut = +inf: no cutoff
    const T f = inv * cut;
    dx *= f;
    dy *= f;
    dz *= f;
    inv = invCut;
    inv2 = invCut2;
  }
  inv2 *= inv;
  inv2 *= qi * s.q;
  acc[0] += dx * -inv2;
  acc[1] += dy * -inv2;
  acc[2] += dz * -inv2;
  acc[3] += inv * s.q;
}

// Grid (target blocks, source chunks): each thread sums the sources of its
// chunk (all periodic copies) for kP2PTargets targets and writes the partial
// sums part[chunk][4][n]; p2pReduceKernel adds the chunks in order.
template <class T>
__global__ void __launch_bounds__(kP2PThreads)
    p2pKernel(const double *__restrict__ x, const double *__restrict__ y,
              const double *__restrict__ z, const double *__restrict__ q, int64_t n,
              int64_t chunk, T invCut, T cut, T invCut2, double box, int images,
              double *__restrict__ part) {
  __shared__ Src4<T> tile[kP2PThreads];
  const int64_t base = (int64_t)blockIdx.x * kP2PThreads * kP2PTargets + threadIdx.x;
  const int64_t j0 = (int64_t)blockIdx.y * chunk, j1 = min(n, j0 + chunk);
  T xi[kP2PTargets], yi[kP2PTargets], zi[kP2PTargets], qi[kP2PTargets];
  double F[kP2PTargets][4];
#pragma unroll
  for (int u = 0; u < kP2PTargets; u++) {
    const int64_t i = base + (int64_t)u * kP2PThreads;
    const bool a = i < n;
    xi[u] = a ? (T)x[i] : T(0);
    yi[u] = a ? (T)y[i] : T(0);
    zi[u] = a ? (T)z[i] : T(0);
    qi[u] = a ? (T)q[i] : T(0);
    F[u][0] = F[u][1] = F[u][2] = F[u][3] = 0.;
  }
  for (int a = -images; a <= images; a++)
    for (int b = -images; b <= images; b++)
      for (int c = -images; c <= images; c++) {
        const bool central = a == 0 && b == 0 && c == 0;
        const double ox = a * box, oy = b * box, oz = c * box;
        for (int64_t t0 = j0; t0 < j1; t0 += kP2PThreads) {
          const int cnt = j1 - t0 < kP2PThreads ? (int)(j1 - t0) : kP2PThreads;
          __syncthreads(); // the previous tile is consumed
          if (threadIdx.x < cnt) {
            const int64_t j = t0 + threadIdx.x;
            tile[threadIdx.x] = Src4<T>{(T)(x[j] + ox), (T)(y[j] + oy), (T)(z[j] + oz), (T)q[j]};
          }
          __syncthreads();
          // the self pair (central copy) is left out: its index in this tile
          int self[kP2PTargets];
#pragma unroll
          for (int u = 0; u < kP2PTargets; u++) {
            const int64_t i = base + (int64_t)u * kP2PThreads;
            self[u] = central && i >= t0 && i < t0 + cnt ? (int)(i - t0) : -1;
          }
          T acc[kP2PTargets][4] = {};
          if (self[0] < 0 && self[1] < 0) {
#pragma unroll 4
            for (int k = 0; k < cnt; k++) {
              const Src4<T> s = tile[k];
#pragma unroll
              for (int u = 0; u < kP2PTargets; u++)
                pairTerm<T>(xi[u], yi[u], zi[u], qi[u], s, invCut, cut, invCut2, acc[u]);
            }
          } else {
            for (int k = 0; k < cnt; k++) {
              const Src4<T> s = tile[k];
#pragma unroll
              for (int u = 0; u < kP2PTargets; u++)
                if (k != self[u])
                  pairTerm<T>(xi[u], yi[u], zi[u], qi[u], s, invCut, cut, invCut2, acc[u]);
            }
          }
#pragma unroll
          for (int u = 0; u < kP2PTargets; u++)
#pragma unroll
            for (int v = 0; v < 4; v++)
              F[u][v] += (double)acc[u][v];
        }
      }
  double *out = part + (size_t)blockIdx.y * 4 * n;
#pragma unroll
  for (int u = 0; u < kP2PTargets; u++) {
    const int64_t i = base + (int64_t)u * kP2PThreads;
    if (i < n)
#pragma unroll
      for (int v = 0; v < 4; v++)
        out[(size_t)v * n + i] = F[u][v];
  }
}

// The chunks' partial sums added in chunk order (deterministic).
__global__ void p2pReduceKernel(const double *__restrict__ part, int chunks, int64_t n,
                                double *__restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 4 * n)
    return;
  double s = 0.;
  for (int c = 0; c < chunks; c++)
    s += part[(size_t)c * 4 * n + i];
  out[i] = s;
}

} // namespace emcg

using namespace emcg;

extern "C" int32_t emcg_p2p_coulomb(const double *pos, const double *charge, int64_t n,
                                    double inv_cutoff, double box, int32_t images,
                                    int32_t precision, double *force, double *potential,
                                    double *kernel_ms) {
  EMCG_CHECK_ARG(n >= 0, "n must not be negative");
  EMCG_CHECK_ARG(precision == EMCG_FP64 || precision == EMCG_FP32, "bad precision %d",
                 precision);
  EMCG_CHECK_ARG(inv_cutoff >= 0 && std::isfinite(inv_cutoff), "inv_cutoff must be >= 0");
  EMCG_CHECK_ARG(images >= 0 && images <= 8, "images must be in [0, 8]");
  EMCG_CHECK_ARG(images == 0 || (box > 0 && std::isfinite(box)),
                 "periodic images need a positive box");
  if (kernel_ms)
    *kernel_ms = 0.;
  if (n == 0)
    return EMCG_OK;
  EMCG_CHECK_ARG(pos && charge && force && potential, "NULL array");
  EMCG_CHECK_ARG(n < (int64_t(1) << 31) * kP2PThreads, "n too large");
  // enough blocks for every SM: split the sources into chunks when the
  // targets alone give too few blocks (at least one tile per chunk)
  int dev = 0, sms = 0;
  EMCG_CUDA(cudaGetDevice(&dev));
  EMCG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int64_t perBlock = (int64_t)kP2PThreads * kP2PTargets;
  const int64_t tBlocks = (n + perBlock - 1) / perBlock;
  const int64_t want = 4LL * sms;
  int chunks = (int)std::max<int64_t>(1, std::min<int64_t>((want + tBlocks - 1) / tBlocks,
                                                            (n + kP2PThreads - 1) / kP2PThreads));
  chunks = std::min(chunks, 65535);
  const int64_t chunk = (n + chunks - 1) / chunks;
  double *d = nullptr;
  EMCG_CUDA(cudaMalloc(&d, (size_t)n * (4 + 4 + 4 * (size_t)chunks) * sizeof(double)));
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  auto done = [&](int32_t s) {
    if (e0)
      cudaEventDestroy(e0);
    if (e1)
      cudaEventDestroy(e1);
    cudaFree(d);
    return s;
  };
  double *dx = d, *dq = d + 3 * n, *dout = d + 4 * n, *dpart = d + 8 * n;
  if (cudaMemcpy(dx, pos, (size_t)n * 3 * sizeof(double), cudaMemcpyHostToDevice) ||
      cudaMemcpy(dq, charge, (size_t)n * sizeof(double), cudaMemcpyHostToDevice) ||
      cudaEventCreate(&e0) || cudaEventCreate(&e1)) {
    setError("p2p: %s", cudaGetErrorString(cudaGetLastError()));
    return done(EMCG_ERR_CUDA);
  }
  const dim3 grid((unsigned)tBlocks, (unsigned)chunks);
  // no cutoff: a threshold no 1/r exceeds
  const double ic = inv_cutoff > 0 ? inv_cutoff : INFINITY;
  const double cut = inv_cutoff > 0 ? 1.0 / inv_cutoff : 0.;
  cudaEventRecord(e0);
  if (precision == EMCG_FP64)
    p2pKernel<double><<<grid, kP2PThreads>>>(dx, dx + n, dx + 2 * n, dq, n, chunk, ic, cut,
                                             ic * ic, box, images, dpart);
  else
    p2pKernel<float><<<grid, kP2PThreads>>>(dx, dx + n, dx + 2 * n, dq, n, chunk, (float)ic,
                                            (float)cut, (float)(ic * ic), box, images, dpart);
  p2pReduceKernel<<<(unsigned)((4 * n + 255) / 256), 256>>>(dpart, chunks, n, dout);
  cudaEventRecord(e1);
  cudaError_t err = cudaGetLastError();
  if (err == cudaSuccess)
    err = cudaEventSynchronize(e1);
  if (err != cudaSuccess) {
    setError("p2p kernel: %s", cudaGetErrorString(err));
    return done(EMCG_ERR_CUDA);
  }
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  if (kernel_ms)
    *kernel_ms = ms;
  if (cudaMemcpy(force, dout, (size_t)n * 3 * sizeof(double), cudaMemcpyDeviceToHost) ||
      cudaMemcpy(potential, dout + 3 * n, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost)) {
    setError("p2p: %s", cudaGetErrorString(cudaGetLastError()));
    return done(EMCG_ERR_CUDA);
  }
  return done(EMCG_OK);
}
