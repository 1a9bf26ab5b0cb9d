// fft_warp.cuh -- register column FFTs for power-of-two N in {32, 64, 128, 256}.
//
// A column of N points in shared memory is transformed by P threads of one warp (a warp
// holds 32 / P columns), each thread holding R = N / P points in registers:
//   N = 32: P = 8,  R = 4      N = 64: P = 8, R = 8
//   N = 128: P = 16, R = 8     N = 256: P = 16, R = 16
// Four-step factorisation with n = t + P j and k = k1 + R k2 (t < P, j, k1 < R, k2 < P):
//   Y[k1][t]    = W_N^{t k1} DFT_R(x[t + P j])[k1]                        (step 1)
//   X[k1 + R k2] = DFT_P(Y[k1][.])[k2]                                     (step 2)
// Step 2 runs as one P-point DFT per thread when P == R; when P == 2R two neighbouring
// threads split it into even / odd halves (R-point DFTs) joined by one radix-2 stage
// over a lane shuffle.  The only data exchange is one pass through the column's own
// shared memory between the steps (warp-synchronous: no block barrier).  Output in
// natural order.  Inverse transforms conjugate on the way in and out.  T is float, or the
// double-float type of dfloat.cuh for FP64-accurate transforms on the FP32 pipes.
#pragma once
#include "fft_green.cuh"

namespace regfft {

template <typename T2>
__device__ __forceinline__ T2 cmul(T2 a, T2 b) {
  T2 r;
  r.x = a.x * b.x - a.y * b.y;
  r.y = a.x * b.y + a.y * b.x;
  return r;
}
template <typename T2>
__device__ __forceinline__ T2 shfl_xor2(T2 v, int m) {
  v.x = shfl_xor_val(v.x, m);
  v.y = shfl_xor_val(v.y, m);
  return v;
}
template <typename T2>
__device__ __forceinline__ void bfly(T2& a, T2& b) {
  T2 t = a;
  a.x = t.x + b.x; a.y = t.y + b.y;
  b.x = t.x - b.x; b.y = t.y - b.y;
}

// forward R-point DFT in registers, natural order in and out (R = 2, 4, 8, 16)
template <int R, typename T2, typename T>
__device__ __forceinline__ void dft(T2* v) {
  if (R == 2) {
    bfly(v[0], v[1]);
  } else if (R == 4) {
    T2 a = v[0], b = v[1], c = v[2], d = v[3];
    bfly(a, c);  // a = a + c, c = a - c
    bfly(b, d);  // b = b + d, d = b - d
    v[0].x = a.x + b.x; v[0].y = a.y + b.y;
    v[2].x = a.x - b.x; v[2].y = a.y - b.y;
    v[1].x = c.x + d.y; v[1].y = c.y - d.x;  // c - i d
    v[3].x = c.x - d.y; v[3].y = c.y + d.x;  // c + i d
  } else if (R == 8) {
    const T h = (T)0.70710678118654752440;
    T2 e[4] = {v[0], v[2], v[4], v[6]}, o[4] = {v[1], v[3], v[5], v[7]};
    dft<4, T2, T>(e);
    dft<4, T2, T>(o);
    T2 t1; t1.x = h * (o[1].x + o[1].y); t1.y = h * (o[1].y - o[1].x); o[1] = t1;  // W8^1
    T2 t2; t2.x = o[2].y; t2.y = -o[2].x; o[2] = t2;                               // W8^2
    T2 t3; t3.x = h * (o[3].y - o[3].x); t3.y = -h * (o[3].x + o[3].y); o[3] = t3;  // W8^3
#pragma unroll
    for (int k = 0; k < 4; k++) {
      v[k].x = e[k].x + o[k].x; v[k].y = e[k].y + o[k].y;
      v[k + 4].x = e[k].x - o[k].x; v[k + 4].y = e[k].y - o[k].y;
    }
  } else if (R == 16) {
    // W16^k = cos(k pi / 8) - i sin(k pi / 8)
    const T c1 = (T)0.92387953251128675613, s1 = (T)0.38268343236508977173;
    const T h = (T)0.70710678118654752440;
    T2 e[8], o[8];
#pragma unroll
    for (int k = 0; k < 8; k++) { e[k] = v[2 * k]; o[k] = v[2 * k + 1]; }
    dft<8, T2, T>(e);
    dft<8, T2, T>(o);
    const T wr[8] = {(T)1, c1, h, s1, (T)0, -s1, -h, -c1};
    const T wi[8] = {(T)0, -s1, -h, -c1, (T)-1, -c1, -h, -s1};
#pragma unroll
    for (int k = 1; k < 8; k++) {
      T2 t;
      t.x = o[k].x * wr[k] - o[k].y * wi[k];
      t.y = o[k].x * wi[k] + o[k].y * wr[k];
      o[k] = t;
    }
#pragma unroll
    for (int k = 0; k < 8; k++) {
      v[k].x = e[k].x + o[k].x; v[k].y = e[k].y + o[k].y;
      v[k + 8].x = e[k].x - o[k].x; v[k + 8].y = e[k].y - o[k].y;
    }
  }
}

template <int N> struct Shape;
template <> struct Shape<32> { static constexpr int P = 8, R = 4; };
template <> struct Shape<64> { static constexpr int P = 8, R = 8; };
template <> struct Shape<128> { static constexpr int P = 16, R = 8; };
template <> struct Shape<256> { static constexpr int P = 16, R = 16; };

// Transform the column at col (element k at col[pidx(k)]) with thread t of its P threads;
// tw[k] = exp(-2 pi i k / N) in shared memory.  Every lane of the warp must call this
// (warp-synchronous shuffles and __syncwarp), each on its own column.
template <int N, typename T2, typename T, bool INV>
__device__ __forceinline__ void column(T2* col, const T2* tw, int t) {
  constexpr int P = Shape<N>::P, R = Shape<N>::R;
  T2 v[R > P ? R : P];
#pragma unroll
  for (int j = 0; j < R; j++) {
    v[j] = col[pidx(t + P * j)];
    if (INV) v[j].y = -v[j].y;
  }
  dft<R, T2, T>(v);
#pragma unroll
  for (int k1 = 1; k1 < R; k1++) v[k1] = cmul(v[k1], tw[t * k1]);
  __syncwarp();
#pragma unroll
  for (int k1 = 0; k1 < R; k1++) col[pidx(k1 * P + t)] = v[k1];
  __syncwarp();
  if (P == R) {
#pragma unroll
    for (int m = 0; m < P; m++) v[m] = col[pidx(t * P + m)];
    dft<P, T2, T>(v);
    __syncwarp();
#pragma unroll
    for (int k2 = 0; k2 < P; k2++) {
      T2 o = v[k2];
      if (INV) o.y = -o.y;
      col[pidx(t + R * k2)] = o;
    }
  } else {  // P == 2R: threads (k1, h) hold the even (h = 0) / odd (h = 1) half
    const int k1 = t >> 1, hh = t & 1;
#pragma unroll
    for (int m = 0; m < R; m++) v[m] = col[pidx(k1 * P + 2 * m + hh)];
    dft<R, T2, T>(v);
    __syncwarp();
#pragma unroll
    for (int i = 0; i < R; i++) {
      T2 p = shfl_xor2(v[i], 1);
      T2 e = hh ? p : v[i], od = hh ? v[i] : p;
      T2 w = cmul(od, tw[i * R]);  // W_P^i = W_N^{i R}
      T2 o;
      o.x = hh ? e.x - w.x : e.x + w.x;
      o.y = hh ? e.y - w.y : e.y + w.y;
      if (INV) o.y = -o.y;
      col[pidx(k1 + R * (hh * R + i))] = o;
    }
  }
  __syncwarp();
}

// ---- column transforms with the data in registers at both ends ----------------------
// A team of P consecutive lanes transforms one column; thread t of the team holds the
// column in "space order" v[j] = x[t + P j] (j < R) or in "frequency order":
//   P == R:  v[k2] = X[t + R k2]                        (k2 < P)
//   P == 2R: v[i]  = X[k1 + R (hh R + i)], k1 = t / 2, hh = t % 2   (i < R)
// The forward transform takes space order to frequency order, the inverse (unscaled,
// sum_k X[k] W_N^{-nk}) frequency order back to space order, the inverse being the
// forward's steps transposed (its inverse P-point step runs on the data each thread
// holds).  Each direction exchanges the column once through the team's buffer `xb`
// (xlen<N>() elements, index xidx<N>: rows of P padded so that a half-warp's accesses
// of both the row and the column pattern fall in distinct banks).

template <int N>
constexpr int xpad() { return Shape<N>::P == Shape<N>::R ? 1 : 2; }
template <int N>
__device__ __forceinline__ int xidx(int k) { return k + (k / Shape<N>::P) * xpad<N>(); }
template <int N>
constexpr int xlen() { return N + Shape<N>::R * xpad<N>(); }

// frequency of element e of thread t in frequency order
template <int N>
__device__ __forceinline__ int freq_of(int t, int e) {
  constexpr int P = Shape<N>::P, R = Shape<N>::R;
  if (P == R) return t + R * e;
  return (t >> 1) + R * ((t & 1) * R + e);
}

template <int R, typename T2, typename T>
__device__ __forceinline__ void idft(T2* v) {
#pragma unroll
  for (int k = 0; k < R; k++) v[k].y = -v[k].y;
  dft<R, T2, T>(v);
#pragma unroll
  for (int k = 0; k < R; k++) v[k].y = -v[k].y;
}

template <int N, typename T2, typename T>
__device__ __forceinline__ void fwd_regs(T2* v, T2* xb, const T2* tw, int t) {
  constexpr int P = Shape<N>::P, R = Shape<N>::R;
  dft<R, T2, T>(v);
#pragma unroll
  for (int k1 = 1; k1 < R; k1++) v[k1] = cmul(v[k1], tw[t * k1]);
#pragma unroll
  for (int k1 = 0; k1 < R; k1++) xb[xidx<N>(k1 * P + t)] = v[k1];
  __syncwarp();
  if (P == R) {
#pragma unroll
    for (int m = 0; m < P; m++) v[m] = xb[xidx<N>(t * P + m)];
    __syncwarp();
    dft<P, T2, T>(v);
  } else {
    const int k1 = t >> 1, hh = t & 1;
#pragma unroll
    for (int m = 0; m < R; m++) v[m] = xb[xidx<N>(k1 * P + 2 * m + hh)];
    __syncwarp();
    dft<R, T2, T>(v);
#pragma unroll
    for (int i = 0; i < R; i++) {
      T2 p = shfl_xor2(v[i], 1);
      T2 e = hh ? p : v[i], od = hh ? v[i] : p;
      T2 w = cmul(od, tw[i * R]);  // W_P^i = W_N^{i R}
      v[i].x = hh ? e.x - w.x : e.x + w.x;
      v[i].y = hh ? e.y - w.y : e.y + w.y;
    }
  }
}

template <int N, typename T2, typename T>
__device__ __forceinline__ void inv_regs(T2* v, T2* xb, const T2* tw, int t) {
  constexpr int P = Shape<N>::P, R = Shape<N>::R;
  if (P == R) {
    const int k1 = t;
    idft<P, T2, T>(v);  // over k2: Z[k1][t'] in v[t']
#pragma unroll
    for (int tp = 0; tp < P; tp++) {
      T2 w = tw[tp * k1];
      w.y = -w.y;
      xb[xidx<N>(k1 * P + tp)] = cmul(v[tp], w);
    }
  } else {
    const int k1 = t >> 1, hh = t & 1;
#pragma unroll
    for (int i = 0; i < R; i++) {  // radix-2 across the thread pair, W_P^{-i} on the odd half
      T2 p = shfl_xor2(v[i], 1);
      T2 x0 = hh ? p : v[i], x1 = hh ? v[i] : p;
      T2 u;
      if (hh) {
        T2 d;
        d.x = x0.x - x1.x;
        d.y = x0.y - x1.y;
        T2 w = tw[i * R];
        w.y = -w.y;
        u = cmul(d, w);
      } else {
        u.x = x0.x + x1.x;
        u.y = x0.y + x1.y;
      }
      v[i] = u;
    }
    idft<R, T2, T>(v);  // Z[k1][2m + hh] in v[m]
#pragma unroll
    for (int m = 0; m < R; m++) {
      const int tp = 2 * m + hh;
      T2 w = tw[tp * k1];
      w.y = -w.y;
      xb[xidx<N>(k1 * P + tp)] = cmul(v[m], w);
    }
  }
  __syncwarp();
#pragma unroll
  for (int k1 = 0; k1 < R; k1++) v[k1] = xb[xidx<N>(k1 * P + t)];
  __syncwarp();
  idft<R, T2, T>(v);
}

}  // namespace regfft
