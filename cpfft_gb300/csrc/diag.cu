// diag.cu -- measurement helper: the FP64 FMA rate of this GPU, the roofline
// denominator of the FP64-bound kernels (the stress update and the FP64 Green apply).
#include "common.cuh"

namespace {
__global__ void __launch_bounds__(256) dfma_loop(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x * 1e-9, x1 = x0 + 1e-9, x2 = x0 + 2e-9, x3 = x0 + 3e-9;
  double x4 = x0 + 4e-9, x5 = x0 + 5e-9, x6 = x0 + 6e-9, x7 = x0 + 7e-9;
  for (int i = 0; i < iters; i++) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  double s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (s == 1234.5) out[threadIdx.x] = s;  // keeps the chain alive, never true
}
}  // namespace

extern "C" int cpfft_measure_fp64_peak(double* tflops) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cpfft_set_error("no CUDA device");
    return CPFFT_ERR_CUDA;
  }
  double* out = nullptr;
  if (cudaMalloc((void**)&out, 256 * sizeof(double)) != cudaSuccess) return CPFFT_ERR_NO_MEMORY;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int blocks = sms * 8, iters = 1 << 14;
  float best = 1e30f;
  for (int rep = 0; rep < 4; rep++) {
    cudaEventRecord(e0);
    dfma_loop<<<blocks, 256>>>(out, iters, 0.999999, 1e-12);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best) best = ms;
  }
  cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (err != cudaSuccess) {
    cpfft_set_error("fp64 probe: %s", cudaGetErrorString(err));
    return CPFFT_ERR_CUDA;
  }
  double flops = 2.0 * 8.0 * (double)iters * blocks * 256.0;
  *tflops = flops / (best * 1e-3) / 1e12;
  return 0;
}
