// green_df_large.cu -- the double-float Green passes for N = 128 and 256 (see green_df.cu).
#include "green_passes.cuh"

cudaError_t green_setup_df_large(int N) {
  switch (N) {
    case 128: return wgreen_setup<4, dfl, float, double>();
    case 256: return wgreen_setup<8, dfl, float, double>();
    default: return cudaErrorNotSupported;
  }
}

cudaError_t green_apply_df_large(const double* x, const float* K4hi, const float* K4lo, int flgK,
                                 double* y, dfl2* S, const dfl2* tw, const GridDesc& g,
                                 cudaStream_t st) {
  switch (g.N) {
    case 128: wgreen_apply<4, dfl, float, double>(x, K4hi, K4lo, flgK, y, S, tw, g, st, nullptr); break;
    case 256: wgreen_apply<8, dfl, float, double>(x, K4hi, K4lo, flgK, y, S, tw, g, st, nullptr); break;
    default: return cudaErrorNotSupported;
  }
  return cudaSuccess;
}
