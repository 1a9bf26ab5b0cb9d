// green_df.cu -- the FP64-accurate Green operator of mixed precision in double-float
// arithmetic: the register-FFT passes of green_passes.cuh instantiated on the double-float
// type of dfloat.cuh.  N = 32 and 64 here, 128 and 256 in green_df_large.cu (separate
// translation units, compiled in parallel: the double-float passes are large).
#include "green_passes.cuh"

// the large grids (green_df_large.cu)
cudaError_t green_setup_df_large(int N);
cudaError_t green_apply_df_large(const double* x, const float* K4hi, const float* K4lo, int flgK,
                                 double* y, dfl2* S, const dfl2* tw, const GridDesc& g,
                                 cudaStream_t st);

bool green_df_supported(int N) { return N == 32 || N == 64 || N == 128 || N == 256; }

cudaError_t green_setup_df(int N) {
  switch (N) {
    case 32: return wgreen_setup<1, dfl, float, double>();
    case 64: return wgreen_setup<2, dfl, float, double>();
    case 128: case 256: return green_setup_df_large(N);
    default: return cudaErrorNotSupported;
  }
}

cudaError_t green_apply_df(const double* x, const float* K4hi, const float* K4lo, int flgK,
                           double* y, dfl2* S, const dfl2* tw, GridDesc g, cudaStream_t st) {
  g.pre = 0;
  switch (g.N) {
    case 32: wgreen_apply<1, dfl, float, double>(x, K4hi, K4lo, flgK, y, S, tw, g, st, nullptr); break;
    case 64: wgreen_apply<2, dfl, float, double>(x, K4hi, K4lo, flgK, y, S, tw, g, st, nullptr); break;
    case 128: case 256: {
      cudaError_t e = green_apply_df_large(x, K4hi, K4lo, flgK, y, S, tw, g, st);
      if (e != cudaSuccess) return e;
      break;
    }
    default: return cudaErrorNotSupported;
  }
  g_kernel_launches += 5;
  return cudaGetLastError();
}

cudaError_t green_autotune_df(const double* x, const float* K4hi, const float* K4lo, double* y,
                              dfl2* S, const dfl2* tw, GridDesc* g, cudaStream_t st, float* best_ms) {
  if (!green_df_supported(g->N)) return cudaSuccess;
  GridDesc t = *g;
  cudaError_t e = tune_tiles(t, [&](const GridDesc& gg) {
    green_apply_df(x, K4hi, K4lo, 1, y, S, tw, gg, st);
  }, st, best_ms, false);
  if (e == cudaSuccess) { g->wtb = t.wtb; g->wtc = t.wtc; }
  return e;
}
