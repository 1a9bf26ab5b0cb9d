// fft_warp.cuh -- register-resident column FFTs for power-of-two N = 32 M (M = 1..8).
//
// One warp transforms one column.  Four-step factorisation N = M x 32 with
// n = 32 j + l (l = lane) and k = k1 + M k2:
//   X[k1 + M k2] = sum_l W_32^{l k2} W_N^{l k1} ( sum_j x[32 j + l] W_M^{j k1} ).
// Each lane does the M-point DFT of its own elements, applies W_N^{l k1}, then the
// 32-point DFT across lanes runs as five radix-2 decimation-in-frequency stages over
// warp shuffles, which leaves lane l holding X[k1 + M brev5(l)].  No shared memory and
// no block barrier inside the transform.
#pragma once
#include "fft_green.cuh"

namespace warpfft {

template <typename T2>
__device__ __forceinline__ T2 cmul(T2 a, T2 b) {
  T2 r;
  r.x = a.x * b.x - a.y * b.y;
  r.y = a.x * b.y + a.y * b.x;
  return r;
}
template <typename T2>
__device__ __forceinline__ T2 shfl_xor2(T2 v, int m) {
  v.x = __shfl_xor_sync(0xffffffffu, v.x, m);
  v.y = __shfl_xor_sync(0xffffffffu, v.y, m);
  return v;
}
// forward M-point DFT in registers (M = 1, 2, 4, 8)
template <int M, typename T2, typename T>
__device__ __forceinline__ void dft_m(T2* v) {
  if (M == 2) {
    T2 a = v[0], b = v[1];
    v[0].x = a.x + b.x; v[0].y = a.y + b.y;
    v[1].x = a.x - b.x; v[1].y = a.y - b.y;
  } else if (M == 4) {
    T2 a = v[0], b = v[1], c = v[2], d = v[3];
    T2 s0, s1, d0, d1;
    s0.x = a.x + c.x; s0.y = a.y + c.y; d0.x = a.x - c.x; d0.y = a.y - c.y;
    s1.x = b.x + d.x; s1.y = b.y + d.y; d1.x = b.x - d.x; d1.y = b.y - d.y;
    v[0].x = s0.x + s1.x; v[0].y = s0.y + s1.y;
    v[2].x = s0.x - s1.x; v[2].y = s0.y - s1.y;
    v[1].x = d0.x + d1.y; v[1].y = d0.y - d1.x;   // d0 - i d1
    v[3].x = d0.x - d1.y; v[3].y = d0.y + d1.x;   // d0 + i d1
  } else if (M == 8) {
    const T h = (T)0.70710678118654752440;
    T2 e[4] = {v[0], v[2], v[4], v[6]}, o[4] = {v[1], v[3], v[5], v[7]};
    dft_m<4, T2, T>(e);
    dft_m<4, T2, T>(o);
    T2 t1; t1.x = h * (o[1].x + o[1].y); t1.y = h * (o[1].y - o[1].x); o[1] = t1;
    T2 t2; t2.x = o[2].y; t2.y = -o[2].x; o[2] = t2;
    T2 t3; t3.x = h * (o[3].y - o[3].x); t3.y = -h * (o[3].x + o[3].y); o[3] = t3;
#pragma unroll
    for (int k = 0; k < 4; k++) {
      v[k].x = e[k].x + o[k].x; v[k].y = e[k].y + o[k].y;
      v[k + 4].x = e[k].x - o[k].x; v[k + 4].y = e[k].y - o[k].y;
    }
  }
}

// Forward DFT of one column of N = 32 M points held as v[j] = x[32 j + lane].
// On return v[k1] = X[k1 + M brev5(lane)].  tw[k] = exp(-2 pi i k / N).
template <int M, typename T2, typename T>
__device__ __forceinline__ void fft(T2* v, const T2* __restrict__ tw) {
  constexpr int N = 32 * M;
  const int lane = threadIdx.x & 31;
  dft_m<M, T2, T>(v);
#pragma unroll
  for (int k1 = 1; k1 < M; k1++) v[k1] = cmul(v[k1], tw[lane * k1]);
#pragma unroll
  for (int d = 16; d >= 1; d >>= 1) {
    const bool upper = (lane & d) != 0;
    const T2 w = tw[(lane & (d - 1)) * (N / (2 * d))];
#pragma unroll
    for (int k1 = 0; k1 < M; k1++) {
      T2 p = shfl_xor2(v[k1], d);
      T2 r;
      if (upper) {
        T2 diff;
        diff.x = p.x - v[k1].x;
        diff.y = p.y - v[k1].y;
        r = cmul(diff, w);
      } else {
        r.x = v[k1].x + p.x;
        r.y = v[k1].y + p.y;
      }
      v[k1] = r;
    }
  }
}

__device__ __forceinline__ int brev5(int l) { return (int)(__brev((unsigned)l) >> 27); }

}  // namespace warpfft
