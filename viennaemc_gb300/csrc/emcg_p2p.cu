// C ABI of the particle-particle Coulomb sums (kernels in emcg_p2p.cuh).
#include "emcg_p2p.cuh"

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
  // targets alone give too few blocks
  int dev = 0, sms = 0;
  EMCG_CUDA(cudaGetDevice(&dev));
  EMCG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int chunks = p2pChunks(n, sms);
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
  cudaEventRecord(e0);
  cudaError_t lerr =
      precision == EMCG_FP64
          ? p2pLaunch<double>(dx, dx + n, dx + 2 * n, dq, n, n, inv_cutoff, box, images, chunks,
                              dpart, dout, n, 0)
          : p2pLaunch<float>(dx, dx + n, dx + 2 * n, dq, n, n, inv_cutoff, box, images, chunks,
                             dpart, dout, n, 0);
  if (lerr != cudaSuccess) {
    setError("p2p launch: %s", cudaGetErrorString(lerr));
    return done(EMCG_ERR_CUDA);
  }
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
