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
// accumulators.  The work is n^2 pair terms of about 15 (float) or 20
// (double) operations: bound by the FP32 (or FP64) pipes, not by memory.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

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

// The float form of the same term in fewer operations.  Closer than the
// cutoff the reference rescales d to the cutoff's length and takes 1/r and
// 1/r^2 at the cutoff, so the force factor d / r'^3 becomes d (1/r) (1/cut)^2
// and the potential term q_j / cut: with c = min(1/r, 1/cut) the terms are
// d (1/r) c^2 q_j and c q_j on either side of the cutoff.  The target's charge
// and the force's sign are applied to the tile's sums, not to every pair.
__device__ __forceinline__ void pairTermF(float xi, float yi, float zi, const Src4<float> &s,
                                          float invCut, float acc[4]) {
  const float dx = xi - s.x, dy = yi - s.y, dz = zi - s.z;
  const float inv = rsqrtf(fmaf(dx, dx, fmaf(dy, dy, dz * dz)));
  const float c = fminf(inv, invCut);
  const float w = inv * c * c * s.q;
  acc[0] = fmaf(dx, w, acc[0]);
  acc[1] = fmaf(dy, w, acc[1]);
  acc[2] = fmaf(dz, w, acc[2]);
  acc[3] = fmaf(c, s.q, acc[3]);
}

template <class T>
__device__ __forceinline__ void pairTermAny(T xi, T yi, T zi, T qi, const Src4<T> &s, T invCut,
                                            T cut, T invCut2, T acc[4]) {
  if constexpr (sizeof(T) == 4)
    pairTermF(xi, yi, zi, s, invCut, acc);
  else
    pairTerm<T>(xi, yi, zi, qi, s, invCut, cut, invCut2, acc);
}

// Grid (target blocks, source chunks): each thread sums the sources of its
// chunk (all periodic copies) for kP2PTargets of the first nTgt particles and
// writes the partial sums part[chunk][4][nTgt]; p2pReduceKernel adds the
// chunks in order.
template <class T>
__global__ void __launch_bounds__(kP2PThreads)
    p2pKernel(const double *__restrict__ x, const double *__restrict__ y,
              const double *__restrict__ z, const double *__restrict__ q, int64_t n,
              int64_t nTgt, int64_t chunk, T invCut, T cut, T invCut2, double box, int images,
              double *__restrict__ part) {
  __shared__ Src4<T> tile[kP2PThreads];
  const int64_t base = (int64_t)blockIdx.x * kP2PThreads * kP2PTargets + threadIdx.x;
  const int64_t j0 = (int64_t)blockIdx.y * chunk, j1 = min(n, j0 + chunk);
  T xi[kP2PTargets], yi[kP2PTargets], zi[kP2PTargets], qi[kP2PTargets];
  double F[kP2PTargets][4];
#pragma unroll
  for (int u = 0; u < kP2PTargets; u++) {
    const int64_t i = base + (int64_t)u * kP2PThreads;
    const bool a = i < nTgt;
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
          bool anySelf = false;
#pragma unroll
          for (int u = 0; u < kP2PTargets; u++)
            anySelf |= self[u] >= 0;
          if (!anySelf) {
#pragma unroll 4
            for (int k = 0; k < cnt; k++) {
              const Src4<T> s = tile[k];
#pragma unroll
              for (int u = 0; u < kP2PTargets; u++)
                pairTermAny<T>(xi[u], yi[u], zi[u], qi[u], s, invCut, cut, invCut2, acc[u]);
            }
          } else {
            for (int k = 0; k < cnt; k++) {
              const Src4<T> s = tile[k];
#pragma unroll
              for (int u = 0; u < kP2PTargets; u++)
                if (k != self[u])
                  pairTermAny<T>(xi[u], yi[u], zi[u], qi[u], s, invCut, cut, invCut2, acc[u]);
            }
          }
#pragma unroll
          for (int u = 0; u < kP2PTargets; u++) {
            // float sums leave out the target's charge and the force's sign
            const double g = sizeof(T) == 4 ? -(double)qi[u] : 1.0;
#pragma unroll
            for (int v = 0; v < 3; v++)
              F[u][v] += g * (double)acc[u][v];
            F[u][3] += (double)acc[u][3];
          }
        }
      }
  double *out = part + (size_t)blockIdx.y * 4 * nTgt;
#pragma unroll
  for (int u = 0; u < kP2PTargets; u++) {
    const int64_t i = base + (int64_t)u * kP2PThreads;
    if (i < nTgt)
#pragma unroll
      for (int v = 0; v < 4; v++)
        out[(size_t)v * nTgt + i] = F[u][v];
  }
}

// The chunks' partial sums added in chunk order (deterministic); quantity v
// of target i goes to out[v * stride + i].
static __global__ void __launch_bounds__(256)
    p2pReduceKernel(const double *__restrict__ part, int chunks, int64_t n,
                    double *__restrict__ out, int64_t stride) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 4 * n)
    return;
  double s = 0.;
  for (int c = 0; c < chunks; c++)
    s += part[(size_t)c * 4 * n + t];
  const int64_t v = t / n, i = t - v * n;
  out[v * stride + i] = s;
}

// Source chunks for n targets on this device: enough blocks for every SM,
// at least one tile per chunk.
inline int p2pChunks(int64_t n, int sms) {
  const int64_t perBlock = (int64_t)kP2PThreads * kP2PTargets;
  const int64_t tBlocks = (n + perBlock - 1) / perBlock;
  const int64_t want = 4LL * sms;
  const int64_t c = std::max<int64_t>(
      1, std::min<int64_t>((want + tBlocks - 1) / tBlocks, (n + kP2PThreads - 1) / kP2PThreads));
  return (int)std::min<int64_t>(c, 65535);
}

// Launch the sums over sources (x, y, z, q: n doubles each) for the first
// nTgt of them on stream st: part holds 4 * nTgt * chunks doubles, out
// receives force x, y, z and potential with the given stride.  inv_cutoff 0:
// no cutoff.
template <class T>
inline cudaError_t p2pLaunch(const double *x, const double *y, const double *z, const double *q,
                             int64_t n, int64_t nTgt, double invCutoff, double box, int images,
                             int chunks, double *part, double *out, int64_t stride,
                             cudaStream_t st) {
  if (nTgt <= 0)
    return cudaSuccess;
  const int64_t perBlock = (int64_t)kP2PThreads * kP2PTargets;
  const dim3 grid((unsigned)((nTgt + perBlock - 1) / perBlock), (unsigned)chunks);
  const int64_t chunk = (n + chunks - 1) / chunks;
  const double ic = invCutoff > 0 ? invCutoff : INFINITY; // no cutoff: no 1/r exceeds it
  const double cut = invCutoff > 0 ? 1.0 / invCutoff : 0.;
  p2pKernel<T><<<grid, kP2PThreads, 0, st>>>(x, y, z, q, n, nTgt, chunk, (T)ic, (T)cut,
                                             (T)(ic * ic), box, images, part);
  p2pReduceKernel<<<(unsigned)((4 * nTgt + 255) / 256), 256, 0, st>>>(part, chunks, nTgt, out,
                                                                      stride);
  return cudaGetLastError();
}


} // namespace emcg
