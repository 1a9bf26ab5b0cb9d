// green_passes.cuh -- the kernels of the fused FFT + Green-operator apply (templates),
// shared by the translation units that instantiate them: fft_green.cu (FP64 Stockham,
// FP32 register passes) and green_df.cu (double-float register passes).  Each unit gets
// its own copies in an unnamed namespace.
#pragma once
#include "fft_green.cuh"
#include "fft_warp.cuh"
#include "krylov.cuh"

namespace {

template <typename T2, typename T>
__device__ __forceinline__ T2 cmul(T2 a, T2 b) {
  T2 r;
  r.x = a.x * b.x - a.y * b.y;
  r.y = a.x * b.y + a.y * b.x;
  return r;
}
template <typename T2>
__device__ __forceinline__ T2 conjg(T2 a) { a.y = -a.y; return a; }

// forward radix-2/4/8 butterflies on registers
template <typename T2, typename T>
__device__ __forceinline__ void bfly2(T2& a, T2& b) {
  T2 t = a;
  a.x = t.x + b.x; a.y = t.y + b.y;
  b.x = t.x - b.x; b.y = t.y - b.y;
}
template <typename T2, typename T>
__device__ __forceinline__ T2 mul_mi(T2 a) { T2 r; r.x = a.y; r.y = -a.x; return r; }  // * (-i)

template <typename T2, typename T>
__device__ __forceinline__ void dft4(T2* v) {
  // X0 = a+b+c+d, X1 = a - i b - c + i d, X2 = a - b + c - d, X3 = a + i b - c - i d
  bfly2<T2, T>(v[0], v[2]);
  bfly2<T2, T>(v[1], v[3]);
  v[3] = mul_mi<T2, T>(v[3]);
  bfly2<T2, T>(v[0], v[1]);
  bfly2<T2, T>(v[2], v[3]);
  T2 t = v[1]; v[1] = v[2]; v[2] = t;
}
template <typename T2, typename T>
__device__ __forceinline__ void dft8(T2* v) {
  const T h = (T)0.70710678118654752440;
  T2 e[4] = {v[0], v[2], v[4], v[6]}, o[4] = {v[1], v[3], v[5], v[7]};
  dft4<T2, T>(e);
  dft4<T2, T>(o);
  // twiddles W8^k for k = 1, 2, 3 (forward)
  T2 t1; t1.x = h * (o[1].x + o[1].y); t1.y = h * (o[1].y - o[1].x); o[1] = t1;
  o[2] = mul_mi<T2, T>(o[2]);
  T2 t3; t3.x = h * (o[3].y - o[3].x); t3.y = -h * (o[3].x + o[3].y); o[3] = t3;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    v[k].x = e[k].x + o[k].x; v[k].y = e[k].y + o[k].y;
    v[k + 4].x = e[k].x - o[k].x; v[k + 4].y = e[k].y - o[k].y;
  }
}


// One forward Stockham stage of radix R on `ncols` columns (column stride cs) from
// src to dst; tw[k] = exp(-2 pi i k / N).  Radix 2/4/8 run as register butterflies,
// any other radix evaluates each output as a direct sum (test-only odd sizes).
template <typename T2, typename T>
__device__ void stage(const T2* __restrict__ src, T2* __restrict__ dst, int ncols, int cs,
                      int N, int R, int Ns, const T2* tw) {
  const int NR = N / R;
  const int tstride = N / (Ns * R);
  if (R == 2 || R == 4 || R == 8) {
    const int total = ncols * NR;
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
      int col = t / NR, j = t - col * NR;
      int jm = j % Ns;
      int ts = jm * tstride;
      const T2* s = src + col * cs;
      T2 v[8];
#pragma unroll
      for (int r = 0; r < 8; r++)
        if (r < R) {
          T2 x = s[pidx(j + r * NR)];
          if (r) x = cmul<T2, T>(x, tw[r * ts]);
          v[r] = x;
        }
      if (R == 2) bfly2<T2, T>(v[0], v[1]);
      else if (R == 4) dft4<T2, T>(v);
      else dft8<T2, T>(v);
      T2* d = dst + col * cs;
      const int base = (j / Ns) * Ns * R + jm;
#pragma unroll
      for (int r = 0; r < 8; r++)
        if (r < R) d[pidx(base + r * Ns)] = v[r];
    }
  } else {
    const int total = ncols * N;
    const int NoR = N / R;
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
      int col = t / N, rem = t - col * N;
      int j = rem % NR, sidx = rem / NR;  // output s of butterfly j
      int jm = j % Ns;
      int ts = jm * tstride;
      const T2* s = src + col * cs;
      T2 acc; acc.x = 0; acc.y = 0;
      for (int r = 0; r < R; r++) {
        int e = (r * ts + ((r * sidx) % R) * NoR) % N;
        T2 p = cmul<T2, T>(s[pidx(j + r * NR)], tw[e]);
        acc.x += p.x; acc.y += p.y;
      }
      dst[col * cs + pidx((j / Ns) * Ns * R + jm + sidx * Ns)] = acc;
    }
  }
}

// Forward FFT of ncols columns held in a (ping-pong with b); returns the buffer with
// the result.  Caller synchronises before (data in a) and this leaves a barrier after.
template <typename T2, typename T>
__device__ T2* fft_cols(T2* a, T2* b, int ncols, int cs, const FftPlan& P, const T2* tw) {
  for (int s = 0; s < P.nst; s++) {
    stage<T2, T>(a, b, ncols, cs, P.n, P.R[s], P.Ns[s], tw);
    __syncthreads();
    T2* t = a; a = b; b = t;
  }
  return a;
}

template <typename T2>
__device__ void load_tw(T2* tw_s, const T2* tw_g, int N) {
  for (int k = threadIdx.x; k < N; k += blockDim.x) tw_s[k] = tw_g[k];
}

__device__ __forceinline__ int qmap(int f, int N, int Nhalf, int gmap) {
  if (gmap == CPFFT_G_REF_SHIFT) {
    int k = ((f - Nhalf) % N + N) % N;
    return k + 1 - Nhalf;
  }
  return f <= (N - 1) / 2 ? f : f - N;
}

// (Ghat(q):A)_ij = q_j (sum_l A_il q_l) / |q|^2, zero when |q|^2 <= 1e-10
// (formG, src/FFT_init.f:310-335); A is 9 complex, accumulated into out with weight w
template <typename T2, typename T>
__device__ __forceinline__ void ghat_acc(const T2* A, int q0, int q1, int q2, T w, T2* out) {
  int qq = q0 * q0 + q1 * q1 + q2 * q2;
  if (qq == 0) return;
  T s = w / (T)qq;
  T q[3] = {(T)q0, (T)q1, (T)q2};
#pragma unroll
  for (int i = 0; i < 3; i++) {
    T2 d;
    d.x = A[3 * i].x * q[0] + A[3 * i + 1].x * q[1] + A[3 * i + 2].x * q[2];
    d.y = A[3 * i].y * q[0] + A[3 * i + 1].y * q[1] + A[3 * i + 2].y * q[2];
    d.x *= s; d.y *= s;
#pragma unroll
    for (int j = 0; j < 3; j++) {
      out[3 * i + j].x += q[j] * d.x;
      out[3 * i + j].y += q[j] * d.y;
    }
  }
}


// Reference-medium Green operator: (Ghat0(q):X)_ij = (A0(q)^-1 X q)_i q_j with
// A0(q)_ik = sum_jl K0_ijkl q_j q_l (Moulinec-Suquet's Gamma0 for the stiffness K0),
// accumulated into out with weight w.  A0 is symmetric (K0 has the major symmetry) and
// inverted through its cofactors; a direction where it is not positive definite
// contributes nothing.
template <typename T2, typename T>
__device__ __forceinline__ void ghat0_acc(const float* coef, const T2* A, int q0, int q1, int q2,
                                          T w, T2* out) {
  if (q0 == 0 && q1 == 0 && q2 == 0) return;
  const T q[3] = {(T)q0, (T)q1, (T)q2};
  const T pr[6] = {q[0] * q[0], q[1] * q[1], q[2] * q[2], q[0] * q[1], q[1] * q[2], q[0] * q[2]};
  T a[6];
#pragma unroll
  for (int r = 0; r < 6; r++) {
    T s = 0;
#pragma unroll
    for (int m = 0; m < 6; m++) s += (T)coef[6 * r + m] * pr[m];
    a[r] = s;
  }
  // a = (a00, a11, a22, a01, a12, a02)
  const T c00 = a[1] * a[2] - a[4] * a[4], c01 = a[5] * a[4] - a[3] * a[2];
  const T c02 = a[3] * a[4] - a[5] * a[1], c11 = a[0] * a[2] - a[5] * a[5];
  const T c12 = a[3] * a[5] - a[0] * a[4], c22 = a[0] * a[1] - a[3] * a[3];
  const T det = a[0] * c00 + a[3] * c01 + a[5] * c02;
  if (!(det > (T)0)) return;
  const T s = w / det;
  T2 d[3];
#pragma unroll
  for (int i = 0; i < 3; i++) {
    d[i].x = A[3 * i].x * q[0] + A[3 * i + 1].x * q[1] + A[3 * i + 2].x * q[2];
    d[i].y = A[3 * i].y * q[0] + A[3 * i + 1].y * q[1] + A[3 * i + 2].y * q[2];
  }
  T2 e[3];
  e[0].x = (c00 * d[0].x + c01 * d[1].x + c02 * d[2].x) * s;
  e[0].y = (c00 * d[0].y + c01 * d[1].y + c02 * d[2].y) * s;
  e[1].x = (c01 * d[0].x + c11 * d[1].x + c12 * d[2].x) * s;
  e[1].y = (c01 * d[0].y + c11 * d[1].y + c12 * d[2].y) * s;
  e[2].x = (c02 * d[0].x + c12 * d[1].x + c22 * d[2].x) * s;
  e[2].y = (c02 * d[0].y + c12 * d[1].y + c22 * d[2].y) * s;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      out[3 * i + j].x += e[i].x * q[j];
      out[3 * i + j].y += e[i].y * q[j];
    }
}

// the spectral operator of pass C: the reference medium when selected (FP32 only)
template <typename T2, typename T>
__device__ __forceinline__ void green_acc(bool pre, const float* coef, const T2* A, int q0, int q1,
                                          int q2, T w, T2* out) {
  if constexpr (sizeof(T) == 4) {
    if (pre) {
      ghat0_acc<T2, T>(coef, A, q0, q1, q2, w, out);
      return;
    }
  }
  ghat_acc<T2, T>(A, q0, q1, q2, w, out);
}

// the reference medium's coefficients in shared memory (block-wide; pre only)
__device__ __forceinline__ void load_acoef(const GridDesc& g, float* s_coef) {
  if (g.pre)
    for (int i = threadIdx.x; i < 36; i += blockDim.x) s_coef[i] = g.acoef[i];
}

// an entry of the tangent in the transform's arithmetic type: FP32 / FP64 as stored, or
// the double-float pair (hi, lo) of the FP64 tangent
template <typename T, typename TK>
__device__ __forceinline__ T kval(const TK* __restrict__ K, const float* __restrict__ Klo,
                                  long long i) {
  return (T)K[i];
}
template <>
__device__ __forceinline__ dfl kval<dfl, float>(const float* __restrict__ K,
                                                const float* __restrict__ Klo, long long i) {
  return dfl(K[i], Klo[i]);
}

// one partial sum per block of the per-thread values d (fixed order), into *dst
template <int NT>
__device__ __forceinline__ void block_partial(double d, double* dst) {
  __shared__ double wsum[NT / 32];
  for (int o = 16; o > 0; o >>= 1) d += __shfl_down_sync(0xffffffffu, d, o);
  if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = d;
  __syncthreads();
  if (threadIdx.x == 0) {
    double b = 0.0;
    for (int k = 0; k < NT / 32; k++) b += wsum[k];
    *dst = b;
  }
}

// ---- pass A: K:x + real-to-complex transform along a --------------------------------
// part != nullptr (with flgK): one partial sum per block of <K : x, x> over its voxels
template <typename T, typename TK>
__global__ void __launch_bounds__(256) pass_a(const T* __restrict__ x, const TK* __restrict__ K4,
                                              int flgK, typename Vec2<T>::t* __restrict__ S,
                                              GridDesc g, const typename Vec2<T>::t* __restrict__ twg,
                                              double* __restrict__ part) {
  using T2 = typename Vec2<T>::t;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int N = g.N, H = g.H, Lp = padlen(N);
  const long long N3 = g.N3;
  T2* tw = reinterpret_cast<T2*>(smem_raw);
  T2* b0 = tw + N;
  T2* b1 = b0 + 9 * Lp;
  load_tw(tw, twg, N);
  const int npair = (N + 1) / 2;
  const int bp = blockIdx.x % npair, c = blockIdx.x / npair;
  const int bl0 = 2 * bp, bl1 = 2 * bp + 1;
  T dsum = 0;
  for (int t = threadIdx.x; t < 2 * N; t += blockDim.x) {
    int l = t / N, a = t - l * N;
    int b = l ? bl1 : bl0;
    T y[9];
    if (b < N) {
      long long v = a + (long long)N * b + (long long)N * N * c;
      if (flgK) {
        T xv[9];
#pragma unroll
        for (int j = 0; j < 9; j++) xv[j] = x[j * N3 + v];
#pragma unroll
        for (int i = 0; i < 9; i++) {
          T s = 0;
#pragma unroll
          for (int j = 0; j < 9; j++) s += (T)K4[(9 * i + j) * N3 + v] * xv[j];
          y[i] = s;
          dsum += s * xv[i];
        }
      } else {
#pragma unroll
        for (int i = 0; i < 9; i++) y[i] = x[i * N3 + v];
      }
    } else {
#pragma unroll
      for (int i = 0; i < 9; i++) y[i] = 0;
    }
#pragma unroll
    for (int i = 0; i < 9; i++) {
      if (l == 0) b0[i * Lp + pidx(a)].x = y[i];
      else b0[i * Lp + pidx(a)].y = y[i];
    }
  }
  if (part) block_partial<256>((double)dsum, part + blockIdx.x);
  __syncthreads();
  T2* r = fft_cols<T2, T>(b0, b1, 9, Lp, g.plan, tw);
  // unpack the two real lines: X0 = (Z + conj Z(-k))/2, X1 = (Z - conj Z(-k))/(2i)
  for (int t = threadIdx.x; t < 9 * H; t += blockDim.x) {
    int i = t / H, k = t - i * H;
    T2 z = r[i * Lp + pidx(k)], w = conjg(r[i * Lp + pidx((N - k) % N)]);
    T2 X0, X1;
    X0.x = (T)0.5 * (z.x + w.x); X0.y = (T)0.5 * (z.y + w.y);
    X1.x = (T)0.5 * (z.y - w.y); X1.y = (T)-0.5 * (z.x - w.x);
    long long base = ((long long)i * N + c) * N;
    S[(base + bl0) * H + k] = X0;
    if (bl1 < N) S[(base + bl1) * H + k] = X1;
  }
}

// ---- pass B / D: transform along b ---------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256) pass_b(typename Vec2<T>::t* __restrict__ S, GridDesc g,
                                              const typename Vec2<T>::t* __restrict__ twg,
                                              int inverse) {
  using T2 = typename Vec2<T>::t;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int N = g.N, H = g.H, TK = g.tkb, Lp = padlen(N);
  T2* tw = reinterpret_cast<T2*>(smem_raw);
  T2* b0 = tw + N;
  T2* b1 = b0 + TK * Lp;
  load_tw(tw, twg, N);
  const int ka0 = blockIdx.x * TK;
  const int c = blockIdx.y, i = blockIdx.z;
  T2* plane = S + ((long long)i * N + c) * (long long)N * H;
  for (int t = threadIdx.x; t < TK * N; t += blockDim.x) {
    int row = t / TK, kk = t - row * TK;
    int ka = ka0 + kk;
    T2 v;
    v.x = 0; v.y = 0;
    if (ka < H) v = plane[(long long)row * H + ka];
    if (inverse) v.y = -v.y;
    b0[kk * Lp + pidx(row)] = v;
  }
  __syncthreads();
  T2* r = fft_cols<T2, T>(b0, b1, TK, Lp, g.plan, tw);
  for (int t = threadIdx.x; t < TK * N; t += blockDim.x) {
    int row = t / TK, kk = t - row * TK;
    int ka = ka0 + kk;
    if (ka < H) {
      T2 v = r[kk * Lp + pidx(row)];
      if (inverse) v.y = -v.y;
      plane[(long long)row * H + ka] = v;
    }
  }
}

// ---- pass C: transform along c, Green contraction, inverse along c -------------------
template <typename T>
__global__ void __launch_bounds__(256) pass_c(typename Vec2<T>::t* __restrict__ S, GridDesc g,
                                              const typename Vec2<T>::t* __restrict__ twg) {
  using T2 = typename Vec2<T>::t;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int N = g.N, H = g.H, TK = g.tkc, Lp = padlen(N);
  T2* tw = reinterpret_cast<T2*>(smem_raw);
  T2* b0 = tw + N;
  T2* b1 = b0 + 9 * TK * Lp;
  load_tw(tw, twg, N);
  __shared__ float s_coef[36];
  load_acoef(g, s_coef);
  const int ka0 = blockIdx.x * TK;
  const int kb = blockIdx.y;
  const long long cstr = (long long)N * H;  // stride between c planes
  // column (i, kk) holds the N values along c
  for (int t = threadIdx.x; t < 9 * N * TK; t += blockDim.x) {
    int kk = t % TK, rem = t / TK;
    int c = rem % N, i = rem / N;
    int ka = ka0 + kk;
    T2 v;
    v.x = 0; v.y = 0;
    if (ka < H) v = S[((long long)i * N) * cstr + c * cstr + (long long)kb * H + ka];
    b0[(i * TK + kk) * Lp + pidx(c)] = v;
  }
  __syncthreads();
  T2* r = fft_cols<T2, T>(b0, b1, 9 * TK, Lp, g.plan, tw);
  T2* o = (r == b0) ? b1 : b0;
  // Green contraction at every (kc, kb, ka) of the tile, symmetrised over +-f
  const int Nh = g.Nhalf, gm = g.gmap;
  const T scale = (T)g.inv_n3;
  for (int t = threadIdx.x; t < N * TK; t += blockDim.x) {
    int kc = t / TK, kk = t - kc * TK;
    int ka = ka0 + kk;
    T2 A[9], out[9];
#pragma unroll
    for (int i = 0; i < 9; i++) {
      A[i] = r[(i * TK + kk) * Lp + pidx(kc)];
      out[i].x = 0; out[i].y = 0;
    }
    // centered mapping at even N: the Nyquist frequency has no signed partner and
    // carries no compatible fluctuation (zero Green operator)
    bool nyq = gm == CPFFT_G_CENTERED && (N & 1) == 0 &&
               (2 * kc == N || 2 * kb == N || 2 * ka == N);
    if (ka < H && !nyq) {
      int p0 = qmap(kc, N, Nh, gm), p1 = qmap(kb, N, Nh, gm), p2 = qmap(ka, N, Nh, gm);
      int m0 = qmap((N - kc) % N, N, Nh, gm), m1 = qmap((N - kb) % N, N, Nh, gm),
          m2 = qmap((N - ka) % N, N, Nh, gm);
      if (m0 == -p0 && m1 == -p1 && m2 == -p2) {
        green_acc<T2, T>(g.pre, s_coef, A, p0, p1, p2, scale, out);
      } else {
        green_acc<T2, T>(g.pre, s_coef, A, p0, p1, p2, (T)0.5 * scale, out);
        green_acc<T2, T>(g.pre, s_coef, A, m0, m1, m2, (T)0.5 * scale, out);
      }
    }
    // conjugate for the inverse transform
#pragma unroll
    for (int i = 0; i < 9; i++) {
      out[i].y = -out[i].y;
      o[(i * TK + kk) * Lp + pidx(kc)] = out[i];
    }
  }
  __syncthreads();
  T2* r2 = fft_cols<T2, T>(o, r, 9 * TK, Lp, g.plan, tw);
  for (int t = threadIdx.x; t < 9 * N * TK; t += blockDim.x) {
    int kk = t % TK, rem = t / TK;
    int c = rem % N, i = rem / N;
    int ka = ka0 + kk;
    if (ka < H) {
      T2 v = r2[(i * TK + kk) * Lp + pidx(c)];
      v.y = -v.y;
      S[((long long)i * N) * cstr + c * cstr + (long long)kb * H + ka] = v;
    }
  }
}

// ---- pass E: complex-to-real inverse along a, unpacking line pairs -------------------
template <typename T>
__global__ void __launch_bounds__(256) pass_e(const typename Vec2<T>::t* __restrict__ S,
                                              T* __restrict__ y, GridDesc g,
                                              const typename Vec2<T>::t* __restrict__ twg) {
  using T2 = typename Vec2<T>::t;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int N = g.N, H = g.H, Lp = padlen(N);
  const long long N3 = g.N3;
  T2* tw = reinterpret_cast<T2*>(smem_raw);
  T2* b0 = tw + N;
  T2* b1 = b0 + 9 * Lp;
  load_tw(tw, twg, N);
  const int npair = (N + 1) / 2;
  const int bp = blockIdx.x % npair, c = blockIdx.x / npair;
  const int bl0 = 2 * bp, bl1 = 2 * bp + 1;
  const bool even = (N % 2) == 0;
  for (int t = threadIdx.x; t < 9 * N; t += blockDim.x) {
    int i = t / N, k = t - i * N;
    long long base = ((long long)i * N + c) * N;
    int kk = k < H ? k : N - k;
    T2 X0 = S[(base + bl0) * H + kk], X1;
    if (bl1 < N) X1 = S[(base + bl1) * H + kk];
    else { X1.x = 0; X1.y = 0; }
    if (kk == 0 || (even && kk == N / 2)) { X0.y = 0; X1.y = 0; }
    if (k >= H) { X0.y = -X0.y; X1.y = -X1.y; }
    // Z = X0 + i X1, load conj(Z) for the inverse
    T2 z;
    z.x = X0.x - X1.y;
    z.y = -(X0.y + X1.x);
    b0[i * Lp + pidx(k)] = z;
  }
  __syncthreads();
  T2* r = fft_cols<T2, T>(b0, b1, 9, Lp, g.plan, tw);
  for (int t = threadIdx.x; t < 2 * 9 * N; t += blockDim.x) {
    int l = t / (9 * N), rem = t - l * 9 * N;
    int i = rem / N, a = rem - i * N;
    int b = l ? bl1 : bl0;
    if (b < N) {
      T2 z = r[i * Lp + pidx(a)];  // conj of the unscaled inverse
      long long v = a + (long long)N * b + (long long)N * N * c;
      y[i * N3 + v] = l ? -z.y : z.x;
    }
  }
}

// ---- warp-FFT passes for power-of-two N = 32 M ------------------------------------
// Same data flow and HBM layout as the passes above; each column transform runs in the
// registers of one warp (fft_warp.cuh), shared memory only stages coalesced tiles.

// columns per warp of the register transform and 9 component columns rounded up to it
template <int N>
constexpr int cpw() { return 32 / regfft::Shape<N>::P; }
template <int N>
constexpr int ncols9() { return ((9 + cpw<N>() - 1) / cpw<N>()) * cpw<N>(); }
// columns of pass C's tile: 9 components x TK, rounded up to whole warps of the register
// transform (the extra columns are scratch)
template <int N, int TK>
constexpr int ncols_c() { return ((9 * TK + cpw<N>() - 1) / cpw<N>()) * cpw<N>(); }

// Transform ncols columns (stride Lp; ncols a multiple of cpw<N>()) with every warp of
// the block; inverse through conjugation.  Columns past the data are scratch.
template <int N, typename T, bool INV>
__device__ __forceinline__ void block_columns(typename Vec2<T>::t* base, int ncols, int Lp,
                                              const typename Vec2<T>::t* tw) {
  using T2 = typename Vec2<T>::t;
  constexpr int P = regfft::Shape<N>::P, CPW = cpw<N>();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int g = w; g * CPW < ncols; g += nw)
    regfft::column<N, T2, T, INV>(base + (g * CPW + lane / P) * Lp, tw, lane % P);
}

// part != nullptr (with flgK): one partial sum per block of <K : x, x> over its voxels.
// Resident blocks per SM the FP32 passes A and E are compiled for at N = 128: four
// 288-thread blocks (at most 56 registers a thread) keep more loads in flight than the
// three the default register count allows -- 5 % off the FP32 apply at 128^3, measured.
// 0 (no hint) elsewhere: the double-float passes, N = 256 (the cap would spill) and the
// small grids (whose default counts already fit more blocks).
template <int M, typename T>
constexpr int minblocks_ae() { return (sizeof(T) == 4 && M == 4) ? 4 : 0; }

// TIO: the field type of x (float, or double for the double-float transform T = dfl,
// whose tangent is the pair K4, K4lo)
// FUSEP (FP32 CG iteration): the operand is the CG direction updated in place on load,
// p = r + beta p with beta = sc[SC_BETA] (x is p, rfuse is r), and sc[SC_RR] takes
// sc[SC_RRNEW] -- the work of k_cg_p fused into this pass.
template <int M, typename T, typename TK, typename TIO, bool FUSEP = false>
__global__ void __launch_bounds__(288, minblocks_ae<M, T>()) wpass_a(const TIO* __restrict__ x, const TK* __restrict__ K4,
                                               const float* __restrict__ K4lo,
                                               int flgK, typename Vec2<T>::t* __restrict__ S,
                                               GridDesc g, const typename Vec2<T>::t* __restrict__ twg,
                                               double* __restrict__ part,
                                               const TIO* __restrict__ rfuse = nullptr,
                                               double* scf = nullptr,
                                               TIO* __restrict__ pout = nullptr) {
  using T2 = typename Vec2<T>::t;
  constexpr int N = 32 * M, H = N / 2 + 1;
  const int Lp = padlen(N);
  const long long N3 = g.N3;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T2* tw = reinterpret_cast<T2*>(smem_raw);
  T2* col = tw + N;
  load_tw(tw, twg, N);
  const int bp = blockIdx.x % (N / 2), c = blockIdx.x / (N / 2);
  const int bl0 = 2 * bp;
  T dsum = 0;
  T beta = 0;
  if constexpr (FUSEP) {
    beta = (T)scf[SC_BETA];
    if (blockIdx.x == 0 && threadIdx.x == 0) scf[SC_RR] = scf[SC_RRNEW];
  }
  for (int t = threadIdx.x; t < 2 * N; t += blockDim.x) {
    int l = t / N, a = t - l * N;
    long long v = a + (long long)N * (bl0 + l) + (long long)N * N * c;
    T y[9];
    if (flgK) {
      T xv[9];
      if constexpr (FUSEP) {
        // x (read) and pout (write) are the same field: each element is read, then
        // written, by this thread alone
#pragma unroll
        for (int j = 0; j < 9; j++) xv[j] = rfuse[j * N3 + v] + beta * x[j * N3 + v];
#pragma unroll
        for (int j = 0; j < 9; j++) pout[j * N3 + v] = xv[j];
      } else {
#pragma unroll
        for (int j = 0; j < 9; j++) xv[j] = from_io<T, TIO>(x[j * N3 + v]);
      }
#pragma unroll
      for (int i = 0; i < 9; i++) {
        T s = 0;
#pragma unroll
        for (int j = 0; j < 9; j++) s += kval<T, TK>(K4, K4lo, (9 * i + j) * N3 + v) * xv[j];
        y[i] = s;
        if (part) dsum += s * xv[i];
      }
    } else {
#pragma unroll
      for (int i = 0; i < 9; i++) y[i] = from_io<T, TIO>(x[i * N3 + v]);
    }
#pragma unroll
    for (int i = 0; i < 9; i++) {
      if (l == 0) col[i * Lp + pidx(a)].x = y[i];
      else col[i * Lp + pidx(a)].y = y[i];
    }
  }
  if (part) block_partial<288>(to_io<double, T>(dsum), part + blockIdx.x);
  __syncthreads();
  block_columns<N, T, false>(col, ncols9<N>(), Lp, tw);
  __syncthreads();
  for (int t = threadIdx.x; t < 9 * H; t += blockDim.x) {
    int i = t / H, k = t - i * H;
    T2 z = col[i * Lp + pidx(k)], wv = conjg(col[i * Lp + pidx((N - k) & (N - 1))]);
    T2 X0, X1;
    X0.x = (T)0.5 * (z.x + wv.x); X0.y = (T)0.5 * (z.y + wv.y);
    X1.x = (T)0.5 * (z.y - wv.y); X1.y = (T)-0.5 * (z.x - wv.x);
    long long base = ((long long)i * N + c) * N;
    S[(base + bl0) * H + k] = X0;
    S[(base + bl0 + 1) * H + k] = X1;
  }
}

// TK columns of one (component, c) plane per block, one warp per column
template <int M, typename T, int TK>
__global__ void __launch_bounds__(32 * TK / cpw<32 * M>()) wpass_b(typename Vec2<T>::t* __restrict__ S, GridDesc g,
                                                   const typename Vec2<T>::t* __restrict__ twg,
                                                   int inverse) {
  using T2 = typename Vec2<T>::t;
  constexpr int N = 32 * M, H = N / 2 + 1;
  const int Lp = padlen(N);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T2* tw = reinterpret_cast<T2*>(smem_raw);
  T2* col = tw + N;
  load_tw(tw, twg, N);
  const int ka0 = blockIdx.x * TK;
  const int c = blockIdx.y, i = blockIdx.z;
  T2* plane = S + ((long long)i * N + c) * (long long)N * H;
  // every load of the tile in flight before the first shared-memory store
  constexpr int NT = 32 * TK / cpw<N>(), E = TK * N / NT;
  static_assert(E * NT == TK * N, "tile must divide evenly over the block");
  {
    T2 v[E];
#pragma unroll
    for (int e = 0; e < E; e++) {
      const int t = threadIdx.x + e * NT, row = t / TK, ka = ka0 + t % TK;
      v[e].x = 0; v[e].y = 0;
      if (ka < H) v[e] = plane[(long long)row * H + ka];
    }
#pragma unroll
    for (int e = 0; e < E; e++) {
      const int t = threadIdx.x + e * NT, row = t / TK, kk = t % TK;
      col[kk * Lp + pidx(row)] = v[e];
    }
  }
  __syncthreads();
  if (inverse) block_columns<N, T, true>(col, TK, Lp, tw);
  else block_columns<N, T, false>(col, TK, Lp, tw);
  __syncthreads();
  for (int t = threadIdx.x; t < TK * N; t += blockDim.x) {
    int row = t / TK, kk = t - row * TK;
    int ka = ka0 + kk;
    if (ka < H) plane[(long long)row * H + ka] = col[kk * Lp + pidx(row)];
  }
}

template <int M, typename T, int TK>
__global__ void __launch_bounds__(288) wpass_c(typename Vec2<T>::t* __restrict__ S, GridDesc g,
                                               const typename Vec2<T>::t* __restrict__ twg) {
  using T2 = typename Vec2<T>::t;
  constexpr int N = 32 * M, H = N / 2 + 1;
  const int Lp = padlen(N);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T2* tw = reinterpret_cast<T2*>(smem_raw);
  T2* col = tw + N;
  load_tw(tw, twg, N);
  __shared__ float s_coef[36];
  load_acoef(g, s_coef);
  const int ka0 = blockIdx.x * TK;
  const int kb = blockIdx.y;
  const long long cstr = (long long)N * H;
  constexpr int NT = 288, E = 9 * N * TK / NT;
  static_assert(E * NT == 9 * N * TK, "tile must divide evenly over the block");
  {
    T2 v[E];
#pragma unroll
    for (int e = 0; e < E; e++) {
      const int t = threadIdx.x + e * NT, kk = t % TK, rem = t / TK;
      const int c = rem % N, i = rem / N, ka = ka0 + kk;
      v[e].x = 0; v[e].y = 0;
      if (ka < H) v[e] = S[((long long)i * N) * cstr + c * cstr + (long long)kb * H + ka];
    }
#pragma unroll
    for (int e = 0; e < E; e++) {
      const int t = threadIdx.x + e * NT, kk = t % TK, rem = t / TK;
      const int c = rem % N, i = rem / N;
      col[(i * TK + kk) * Lp + pidx(c)] = v[e];
    }
  }
  __syncthreads();
  block_columns<N, T, false>(col, ncols_c<N, TK>(), Lp, tw);
  __syncthreads();
  const int Nh = g.Nhalf, gm = g.gmap;
  const T scale = (T)g.inv_n3;
  for (int t = threadIdx.x; t < N * TK; t += blockDim.x) {
    int kc = t / TK, kk = t - kc * TK;
    int ka = ka0 + kk;
    T2 A[9], out[9];
#pragma unroll
    for (int i = 0; i < 9; i++) {
      A[i] = col[(i * TK + kk) * Lp + pidx(kc)];
      out[i].x = 0; out[i].y = 0;
    }
    bool nyq = gm == CPFFT_G_CENTERED && (2 * kc == N || 2 * kb == N || 2 * ka == N);
    if (ka < H && !nyq) {
      int p0 = qmap(kc, N, Nh, gm), p1 = qmap(kb, N, Nh, gm), p2 = qmap(ka, N, Nh, gm);
      int m0 = qmap((N - kc) & (N - 1), N, Nh, gm), m1 = qmap((N - kb) & (N - 1), N, Nh, gm),
          m2 = qmap((N - ka) & (N - 1), N, Nh, gm);
      if (m0 == -p0 && m1 == -p1 && m2 == -p2) {
        green_acc<T2, T>(g.pre, s_coef, A, p0, p1, p2, scale, out);
      } else {
        green_acc<T2, T>(g.pre, s_coef, A, p0, p1, p2, (T)0.5 * scale, out);
        green_acc<T2, T>(g.pre, s_coef, A, m0, m1, m2, (T)0.5 * scale, out);
      }
    }
#pragma unroll
    for (int i = 0; i < 9; i++) col[(i * TK + kk) * Lp + pidx(kc)] = out[i];
  }
  __syncthreads();
  block_columns<N, T, true>(col, ncols_c<N, TK>(), Lp, tw);
  __syncthreads();
  for (int t = threadIdx.x; t < 9 * N * TK; t += blockDim.x) {
    int kk = t % TK, rem = t / TK;
    int c = rem % N, i = rem / N;
    int ka = ka0 + kk;
    if (ka < H)
      S[((long long)i * N) * cstr + c * cstr + (long long)kb * H + ka] = col[(i * TK + kk) * Lp + pidx(c)];
  }
}

// ---- pass C, register-resident form ---------------------------------------------------
// The Green contraction acts row by row: (Ghat : A)_ij = q_j (sum_l A_il q_l) / |q|^2 needs
// only row i of A at the same frequency.  A team of P lanes therefore holds the 3
// components of one row (i = 3 row + l) of one (kb, ka) column along c in registers:
// loaded straight from the half spectrum in space order, transformed forward (one
// exchange through the team's buffer), contracted in registers, transformed back (one
// exchange) and stored straight back -- four shared-memory accesses per element instead of
// twelve in wpass_c.  The reference-medium operator couples the rows only through the
// 3-vector d_i = sum_l A_il q_l: the teams of one column trade it through shared memory.
// Block: 3 rows x TK columns of teams (3 TK P threads); grid ((H + TK - 1) / TK, N).
template <typename T2, typename T>
__device__ __forceinline__ void green_row_plain(const T2* A, int q0, int q1, int q2, T w,
                                                T2* out) {
  const int qq = q0 * q0 + q1 * q1 + q2 * q2;
  if (qq == 0) return;
  const T s = w / (T)qq;
  const T q[3] = {(T)q0, (T)q1, (T)q2};
  T2 d;
  d.x = (A[0].x * q[0] + A[1].x * q[1] + A[2].x * q[2]) * s;
  d.y = (A[0].y * q[0] + A[1].y * q[1] + A[2].y * q[2]) * s;
#pragma unroll
  for (int j = 0; j < 3; j++) {
    out[j].x += q[j] * d.x;
    out[j].y += q[j] * d.y;
  }
}

// row `row` of Ghat0(q) : A from the three rows' d = A q (dq[3]), accumulated with weight w
template <typename T2, typename T>
__device__ __forceinline__ void green_row_pre(const float* coef, const T2* dq, int row, int q0,
                                              int q1, int q2, T w, T2* out) {
  if (q0 == 0 && q1 == 0 && q2 == 0) return;
  const T q[3] = {(T)q0, (T)q1, (T)q2};
  const T pr[6] = {q[0] * q[0], q[1] * q[1], q[2] * q[2], q[0] * q[1], q[1] * q[2], q[0] * q[2]};
  T a[6];
#pragma unroll
  for (int r = 0; r < 6; r++) {
    T s = 0;
#pragma unroll
    for (int m = 0; m < 6; m++) s += (T)coef[6 * r + m] * pr[m];
    a[r] = s;
  }
  // a = (a00, a11, a22, a01, a12, a02); cofactors of the symmetric A0(q)
  const T c00 = a[1] * a[2] - a[4] * a[4], c01 = a[5] * a[4] - a[3] * a[2];
  const T c02 = a[3] * a[4] - a[5] * a[1], c11 = a[0] * a[2] - a[5] * a[5];
  const T c12 = a[3] * a[5] - a[0] * a[4], c22 = a[0] * a[1] - a[3] * a[3];
  const T det = a[0] * c00 + a[3] * c01 + a[5] * c02;
  if (!(det > (T)0)) return;
  const T cr0 = row == 0 ? c00 : row == 1 ? c01 : c02;
  const T cr1 = row == 0 ? c01 : row == 1 ? c11 : c12;
  const T cr2 = row == 0 ? c02 : row == 1 ? c12 : c22;
  const T s = w / det;
  T2 e;
  e.x = (cr0 * dq[0].x + cr1 * dq[1].x + cr2 * dq[2].x) * s;
  e.y = (cr0 * dq[0].y + cr1 * dq[1].y + cr2 * dq[2].y) * s;
#pragma unroll
  for (int j = 0; j < 3; j++) {
    out[j].x += e.x * q[j];
    out[j].y += e.y * q[j];
  }
}

template <typename T2, typename T>
__device__ __forceinline__ T2 dot_q(const T2* A, int q0, int q1, int q2) {
  const T a = (T)q0, b = (T)q1, c = (T)q2;
  T2 d;
  d.x = A[0].x * a + A[1].x * b + A[2].x * c;
  d.y = A[0].y * a + A[1].y * b + A[2].y * c;
  return d;
}

template <int N, int TK>
constexpr int c2_threads() { return 3 * TK * regfft::Shape<N>::P; }
template <typename T, int N, int TK>
constexpr size_t smem_c2() {
  // twiddles, one exchange buffer per team, and the d exchange of the reference medium
  // (per column of the tile: N frequencies x {+q, -q} x 3 rows)
  return sizeof(typename Vec2<T>::t) *
         ((size_t)N + (size_t)3 * TK * regfft::xlen<N>() + (size_t)TK * N * 6);
}

template <int M, typename T, int TK>
__global__ void __launch_bounds__(c2_threads<32 * M, TK>()) wpass_c2(
    typename Vec2<T>::t* __restrict__ S, GridDesc g, const typename Vec2<T>::t* __restrict__ twg) {
  using T2 = typename Vec2<T>::t;
  constexpr int N = 32 * M, H = N / 2 + 1;
  constexpr int P = regfft::Shape<N>::P, R = regfft::Shape<N>::R;
  constexpr int XL = regfft::xlen<N>();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T2* tw = reinterpret_cast<T2*>(smem_raw);
  T2* xbuf = tw + N;
  T2* dbuf = xbuf + 3 * TK * XL;
  __shared__ float s_coef[36];
  load_acoef(g, s_coef);
  load_tw(tw, twg, N);
  const int team = threadIdx.x / P, t = threadIdx.x % P;
  const int row = team / TK, kk = team % TK;
  const int ka = blockIdx.x * TK + kk, kb = blockIdx.y;
  const bool valid = ka < H;
  const long long cstr = (long long)N * H;
  T2 v[3][R];
#pragma unroll
  for (int l = 0; l < 3; l++) {
    const T2* src = S + (long long)(3 * row + l) * N * cstr + (long long)kb * H + ka;
#pragma unroll
    for (int j = 0; j < R; j++) {
      v[l][j].x = 0;
      v[l][j].y = 0;
      if (valid) v[l][j] = src[(long long)(t + P * j) * cstr];
    }
  }
  __syncthreads();  // twiddles and coefficients
  T2* xb = xbuf + team * XL;
#pragma unroll
  for (int l = 0; l < 3; l++) regfft::fwd_regs<N, T2, T>(v[l], xb, tw, t);
  const int Nh = g.Nhalf, gm = g.gmap;
  const T scale = (T)g.inv_n3;
  const bool cen_even = gm == CPFFT_G_CENTERED && (N & 1) == 0;
  const bool nyq_ab = cen_even && (2 * kb == N || 2 * ka == N);
  const int p1 = qmap(kb, N, Nh, gm), p2 = qmap(ka, N, Nh, gm);
  const int m1 = qmap((N - kb) & (N - 1), N, Nh, gm), m2 = qmap((N - ka) & (N - 1), N, Nh, gm);
  bool pre = false;
  if constexpr (sizeof(T) == 4) pre = g.pre != 0;
  if (pre) {
    // d = A q of this row at +q and -q, traded with the other rows of the column
#pragma unroll
    for (int e = 0; e < R; e++) {
      const int kc = regfft::freq_of<N>(t, e);
      const int p0 = qmap(kc, N, Nh, gm), m0 = qmap((N - kc) & (N - 1), N, Nh, gm);
      const T2 A[3] = {v[0][e], v[1][e], v[2][e]};
      T2* d = dbuf + ((size_t)kk * N + kc) * 6;
      d[row] = dot_q<T2, T>(A, p0, p1, p2);
      d[3 + row] = dot_q<T2, T>(A, m0, m1, m2);
    }
    __syncthreads();
  }
#pragma unroll
  for (int e = 0; e < R; e++) {
    const int kc = regfft::freq_of<N>(t, e);
    T2 out[3];
#pragma unroll
    for (int l = 0; l < 3; l++) { out[l].x = 0; out[l].y = 0; }
    const bool nyq = nyq_ab || (cen_even && 2 * kc == N);
    if (valid && !nyq) {
      const int p0 = qmap(kc, N, Nh, gm), m0 = qmap((N - kc) & (N - 1), N, Nh, gm);
      const bool sym = m0 == -p0 && m1 == -p1 && m2 == -p2;
      const T w = sym ? scale : (T)0.5 * scale;
      if (pre) {
        const T2* d = dbuf + ((size_t)kk * N + kc) * 6;
        green_row_pre<T2, T>(s_coef, d, row, p0, p1, p2, w, out);
        if (!sym) green_row_pre<T2, T>(s_coef, d + 3, row, m0, m1, m2, w, out);
      } else {
        const T2 A[3] = {v[0][e], v[1][e], v[2][e]};
        green_row_plain<T2, T>(A, p0, p1, p2, w, out);
        if (!sym) green_row_plain<T2, T>(A, m0, m1, m2, w, out);
      }
    }
#pragma unroll
    for (int l = 0; l < 3; l++) v[l][e] = out[l];
  }
#pragma unroll
  for (int l = 0; l < 3; l++) regfft::inv_regs<N, T2, T>(v[l], xb, tw, t);
  if (valid) {
#pragma unroll
    for (int l = 0; l < 3; l++) {
      T2* dst = S + (long long)(3 * row + l) * N * cstr + (long long)kb * H + ka;
#pragma unroll
      for (int j = 0; j < R; j++) dst[(long long)(t + P * j) * cstr] = v[l][j];
    }
  }
}

// dotx != nullptr: also one partial sum per block of dotx . y over the voxels the block
// writes (the CG product p . Ap without re-reading Ap), into part[blockIdx.x]
template <int M, typename T, typename TIO>
__global__ void __launch_bounds__(288, minblocks_ae<M, T>()) wpass_e(const typename Vec2<T>::t* __restrict__ S,
                                               TIO* __restrict__ y, GridDesc g,
                                               const typename Vec2<T>::t* __restrict__ twg,
                                               const TIO* __restrict__ dotx,
                                               double* __restrict__ part) {
  using T2 = typename Vec2<T>::t;
  constexpr int N = 32 * M, H = N / 2 + 1;
  const int Lp = padlen(N);
  const long long N3 = g.N3;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T2* tw = reinterpret_cast<T2*>(smem_raw);
  T2* col = tw + N;
  load_tw(tw, twg, N);
  const int bp = blockIdx.x % (N / 2), c = blockIdx.x / (N / 2);
  const int bl0 = 2 * bp;
  constexpr int NT = 288, E = 9 * N / NT;
  static_assert(E * NT == 9 * N, "lines must divide evenly over the block");
  {
    T2 X0[E], X1[E];
#pragma unroll
    for (int e = 0; e < E; e++) {
      const int t = threadIdx.x + e * NT, i = t / N, k = t - i * N;
      const long long base = ((long long)i * N + c) * N;
      const int kk = k < H ? k : N - k;
      X0[e] = S[(base + bl0) * H + kk];
      X1[e] = S[(base + bl0 + 1) * H + kk];
    }
#pragma unroll
    for (int e = 0; e < E; e++) {
      const int t = threadIdx.x + e * NT, i = t / N, k = t - i * N;
      const int kk = k < H ? k : N - k;
      T2 a = X0[e], b = X1[e];
      if (kk == 0 || kk == N / 2) { a.y = 0; b.y = 0; }
      if (k >= H) { a.y = -a.y; b.y = -b.y; }
      T2 z;  // Z = X0 + i X1 (the inverse is taken as conj(FFT(conj Z)))
      z.x = a.x - b.y;
      z.y = a.y + b.x;
      col[i * Lp + pidx(k)] = z;
    }
  }
  // the other factor of the fused product, loaded before the transform hides its latency
  constexpr int EO = 2 * 9 * N / NT;
  T px[EO];
  if (dotx) {
#pragma unroll
    for (int e = 0; e < EO; e++) {
      const int t = threadIdx.x + e * NT, l = t / (9 * N), rem = t - l * 9 * N;
      const int i = rem / N, a = rem - i * N;
      px[e] = from_io<T, TIO>(dotx[i * N3 + a + (long long)N * (bl0 + l) + (long long)N * N * c]);
    }
  }
  __syncthreads();
  block_columns<N, T, true>(col, ncols9<N>(), Lp, tw);
  __syncthreads();
  T dsum = 0;
#pragma unroll
  for (int e = 0; e < EO; e++) {
    const int t = threadIdx.x + e * NT, l = t / (9 * N), rem = t - l * 9 * N;
    const int i = rem / N, a = rem - i * N;
    T2 z = col[i * Lp + pidx(a)];  // unscaled inverse (scale applied in pass C)
    long long v = a + (long long)N * (bl0 + l) + (long long)N * N * c;
    const T yv = l ? z.y : z.x;
    y[i * N3 + v] = to_io<TIO, T>(yv);
    if (dotx) dsum += px[e] * yv;
  }
  if (dotx) {  // block sum (9 warps), fixed order
    __shared__ double wsum[9];
    double d = to_io<double, T>(dsum);
    for (int o = 16; o > 0; o >>= 1) d += __shfl_down_sync(0xffffffffu, d, o);
    if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = d;
    __syncthreads();
    if (threadIdx.x == 0) {
      double b = 0.0;
      for (int k = 0; k < 9; k++) b += wsum[k];
      part[blockIdx.x] = b;
    }
  }
}

// Pass E fused with the rest of a preconditioned FP32 CG iteration: the inverse transform
// gives Ap = G0(K : p) on the block's two lines, and x += alpha p, r -= alpha Ap and one
// partial sum of <r, r>_K0 per block follow at once, so Ap never reaches memory.  x, r and
// p of the block's voxels are loaded before the transform (their latency hides behind it);
// each thread owns whole voxels (all 9 components, as the K0 form needs them).
template <int M>
__global__ void __launch_bounds__(288, minblocks_ae<M, float>()) wpass_e_xr(
    const float2* __restrict__ S, GridDesc g, const float2* __restrict__ twg,
    float* __restrict__ x, float* __restrict__ r, const float* __restrict__ p,
    const float* __restrict__ k0, const double* __restrict__ sc, double* __restrict__ part) {
  using T = float;
  using T2 = float2;
  constexpr int N = 32 * M, H = N / 2 + 1, NT = 288;
  constexpr int NV = (2 * N + NT - 1) / NT;  // voxels per thread
  const int Lp = padlen(N);
  const long long N3 = g.N3;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T2* tw = reinterpret_cast<T2*>(smem_raw);
  T2* col = tw + N;
  __shared__ float s_k0[81];
  for (int i = threadIdx.x; i < 81; i += blockDim.x) s_k0[i] = k0[i];
  load_tw(tw, twg, N);
  const int bp = blockIdx.x % (N / 2), c = blockIdx.x / (N / 2);
  const int bl0 = 2 * bp;
  constexpr int E = 9 * N / NT;
  static_assert(E * NT == 9 * N, "lines must divide evenly over the block");
  {
    T2 X0[E], X1[E];
#pragma unroll
    for (int e = 0; e < E; e++) {
      const int t = threadIdx.x + e * NT, i = t / N, k = t - i * N;
      const long long base = ((long long)i * N + c) * N;
      const int kk = k < H ? k : N - k;
      X0[e] = S[(base + bl0) * H + kk];
      X1[e] = S[(base + bl0 + 1) * H + kk];
    }
#pragma unroll
    for (int e = 0; e < E; e++) {
      const int t = threadIdx.x + e * NT, i = t / N, k = t - i * N;
      const int kk = k < H ? k : N - k;
      T2 a = X0[e], b = X1[e];
      if (kk == 0 || kk == N / 2) { a.y = 0; b.y = 0; }
      if (k >= H) { a.y = -a.y; b.y = -b.y; }
      T2 z;  // Z = X0 + i X1 (the inverse is taken as conj(FFT(conj Z)))
      z.x = a.x - b.y;
      z.y = a.y + b.x;
      col[i * Lp + pidx(k)] = z;
    }
  }
  float xv[NV][9], rv[NV][9], pv[NV][9];
#pragma unroll
  for (int u = 0; u < NV; u++) {
    const int vt = threadIdx.x + NT * u;
    if (vt < 2 * N) {
      const int l = vt / N, a = vt - l * N;
      const long long v = a + (long long)N * (bl0 + l) + (long long)N * N * c;
#pragma unroll
      for (int i = 0; i < 9; i++) {
        xv[u][i] = x[i * N3 + v];
        rv[u][i] = r[i * N3 + v];
        pv[u][i] = p[i * N3 + v];
      }
    }
  }
  __syncthreads();
  block_columns<N, T, true>(col, ncols9<N>(), Lp, tw);
  __syncthreads();
  const float alpha = (float)sc[SC_ALPHA];
  float s = 0.f;
#pragma unroll
  for (int u = 0; u < NV; u++) {
    const int vt = threadIdx.x + NT * u;
    if (vt < 2 * N) {
      const int l = vt / N, a = vt - l * N;
      const long long v = a + (long long)N * (bl0 + l) + (long long)N * N * c;
#pragma unroll
      for (int i = 0; i < 9; i++) {
        const T2 z = col[i * Lp + pidx(a)];  // unscaled inverse (scale applied in pass C)
        const float ap = l ? z.y : z.x;
        xv[u][i] += alpha * pv[u][i];
        rv[u][i] -= alpha * ap;
        x[i * N3 + v] = xv[u][i];
        r[i * N3 + v] = rv[u][i];
      }
#pragma unroll
      for (int i = 0; i < 9; i++) {
        float t = 0.f;
#pragma unroll
        for (int j = 0; j < 9; j++) t += s_k0[9 * i + j] * rv[u][j];
        s += rv[u][i] * t;
      }
    }
  }
  block_partial<NT>((double)s, part + blockIdx.x);
}

template <typename T>
size_t smem_w(int N, int ncols) { return sizeof(typename Vec2<T>::t) * (size_t)(N + ncols * padlen(N)); }
template <typename T>
constexpr int wtile_c() { return sizeof(T) == 4 ? 4 : 2; }

// Tile shapes of the warp passes, chosen per operator by green_autotune: columns per
// block of passes B / D (TB) and of pass C (TC).
// (the double-float passes, whose code is several times larger, are instantiated for the
// B/D tiles 16 and 32 and the C tile 2 only)
constexpr int TB_CAND[3] = {8, 16, 32};
constexpr int TC_CAND[2] = {2, 4};
// pass C in registers (wpass_c2, FP32 only): its TK.  The slowest-axis algorithm is fixed
// per grid, because the two round differently and contexts of one grid must give identical
// results whatever their timings: in registers up to N = 64 (64^3: 12.9 against 19.4 us a
// launch), in shared memory above (128^3: 120 against 103 us), measured with ncu on a
// GB300; the autotuner then chooses the tiles within that algorithm.  cpfft_set_tiles
// selects either.
constexpr int C2_CAND[2] = {2, 4};
constexpr int C2_MAX_N = 64;

template <int M, typename T, int TB>
cudaError_t wsetup_b() {
  constexpr int N = 32 * M;
  return cudaFuncSetAttribute(wpass_b<M, T, TB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)smem_w<T>(N, TB));
}
template <int M, typename T, int TC>
cudaError_t wsetup_c() {
  constexpr int N = 32 * M;
  return cudaFuncSetAttribute(wpass_c<M, T, TC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)smem_w<T>(N, ncols_c<N, TC>()));
}

template <typename T>
constexpr bool small_code() { return sizeof(T) == 4; }

template <int M, typename T, int TK>
cudaError_t wsetup_c2() {
  return cudaFuncSetAttribute(wpass_c2<M, T, TK>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)smem_c2<T, 32 * M, TK>());
}
template <int M, typename T, int TK>
void wlaunch_c2(typename Vec2<T>::t* S, const GridDesc& g, const typename Vec2<T>::t* tw,
                cudaStream_t st) {
  constexpr int N = 32 * M, H = N / 2 + 1;
  dim3 gc((H + TK - 1) / TK, N);
  wpass_c2<M, T, TK><<<gc, c2_threads<N, TK>(), smem_c2<T, N, TK>(), st>>>(S, g, tw);
}

template <int M, typename T, typename TK = T, typename TIO = T>
cudaError_t wgreen_setup() {
  constexpr int N = 32 * M;
  cudaError_t e;
  if ((e = cudaFuncSetAttribute(wpass_a<M, T, TK, TIO>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)smem_w<T>(N, ncols9<N>())))) return e;
  if ((e = wsetup_b<M, T, 16>()) || (e = wsetup_b<M, T, 32>()) || (e = wsetup_c<M, T, 2>())) return e;
  if constexpr (small_code<T>()) {
    if ((e = wsetup_b<M, T, 8>()) || (e = wsetup_c<M, T, 4>()) || (e = wsetup_c2<M, T, 2>()) ||
        (e = wsetup_c2<M, T, 4>()))
      return e;
    if ((e = cudaFuncSetAttribute(wpass_a<M, T, TK, TIO, true>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem_w<T>(N, ncols9<N>()))))
      return e;
    if ((e = cudaFuncSetAttribute(wpass_e_xr<M>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem_w<T>(N, ncols9<N>()))))
      return e;
  }
  if ((e = cudaFuncSetAttribute(wpass_e<M, T, TIO>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)smem_w<T>(N, ncols9<N>())))) return e;
  return cudaSuccess;
}

template <int M, typename T, int TB>
void wlaunch_b(typename Vec2<T>::t* S, const GridDesc& g, const typename Vec2<T>::t* tw,
               int inverse, cudaStream_t st) {
  constexpr int N = 32 * M, H = N / 2 + 1;
  dim3 gb((H + TB - 1) / TB, N, 9);
  wpass_b<M, T, TB><<<gb, 32 * TB / cpw<N>(), smem_w<T>(N, TB), st>>>(S, g, tw, inverse);
}
template <int M, typename T, int TC>
void wlaunch_c(typename Vec2<T>::t* S, const GridDesc& g, const typename Vec2<T>::t* tw,
               cudaStream_t st) {
  constexpr int N = 32 * M, H = N / 2 + 1;
  dim3 gc((H + TC - 1) / TC, N);
  wpass_c<M, T, TC><<<gc, 288, smem_w<T>(N, ncols_c<N, TC>()), st>>>(S, g, tw);
}
template <int M, typename T>
void wlaunch_b_any(int tb, typename Vec2<T>::t* S, const GridDesc& g,
                   const typename Vec2<T>::t* tw, int inverse, cudaStream_t st) {
  if constexpr (small_code<T>()) {
    if (tb == 8) { wlaunch_b<M, T, 8>(S, g, tw, inverse, st); return; }
  }
  if (tb == 32) wlaunch_b<M, T, 32>(S, g, tw, inverse, st);
  else wlaunch_b<M, T, 16>(S, g, tw, inverse, st);
}

template <int M, typename T, typename TK = T, typename TIO = T>
void wgreen_apply(const TIO* x, const TK* K4, const float* K4lo, int flgK, TIO* y,
                  typename Vec2<T>::t* S, const typename Vec2<T>::t* tw, const GridDesc& g,
                  cudaStream_t st, double* part, const TIO* rfuse = nullptr,
                  double* scf = nullptr) {
  constexpr int N = 32 * M;
  constexpr int NA = ncols9<N>();
  // the fused product: <K : x, x> in pass A for the reference-medium operator (where it
  // equals <x, y> in the K0 inner product), else <x, y> in pass E
  double* part_a = g.pre ? part : nullptr;
  double* part_e = g.pre ? nullptr : part;
  if constexpr (small_code<T>()) {
    if (rfuse)
      wpass_a<M, T, TK, TIO, true><<<(N / 2) * N, 288, smem_w<T>(N, NA), st>>>(
          x, K4, K4lo, flgK, S, g, tw, part_a, rfuse, scf, const_cast<TIO*>(x));
    else
      wpass_a<M, T, TK, TIO><<<(N / 2) * N, 288, smem_w<T>(N, NA), st>>>(x, K4, K4lo, flgK, S, g,
                                                                        tw, part_a);
  } else {
    wpass_a<M, T, TK, TIO><<<(N / 2) * N, 288, smem_w<T>(N, NA), st>>>(x, K4, K4lo, flgK, S, g, tw,
                                                                      part_a);
  }
  wlaunch_b_any<M, T>(g.wtb, S, g, tw, 0, st);
  if constexpr (small_code<T>()) {
    if (g.wc2 == 4) wlaunch_c2<M, T, 4>(S, g, tw, st);
    else if (g.wc2 == 2) wlaunch_c2<M, T, 2>(S, g, tw, st);
    else if ((g.wtc ? g.wtc : wtile_c<T>()) == 4) { wlaunch_c<M, T, 4>(S, g, tw, st); }
    else wlaunch_c<M, T, 2>(S, g, tw, st);
  } else {
    wlaunch_c<M, T, 2>(S, g, tw, st);
  }
  wlaunch_b_any<M, T>(g.wtb, S, g, tw, 1, st);
  wpass_e<M, T, TIO><<<(N / 2) * N, 288, smem_w<T>(N, NA), st>>>(S, y, g, tw,
                                                                 part_e ? x : nullptr, part_e);
}

// One preconditioned FP32 CG iteration's operator and vector work on the register-FFT
// grids: pass A with p = r + beta p fused (and the partials of <K : p, p>), alpha from
// them, passes B-D, pass E fused with x += alpha p, r -= alpha G0(K : p) and the partials
// of <r, r>_K0 (part_e, (N/2) N of them).  g.pre must be set.
template <int M>
void wcg_iteration(float* x, float* r, float* p, const float* K4, float2* S, const float2* tw,
                   const GridDesc& g, cudaStream_t st, double* part_a, double* part_e,
                   const float* k0, double* sc) {
  constexpr int N = 32 * M;
  constexpr int NA = ncols9<N>();
  wpass_a<M, float, float, float, true><<<(N / 2) * N, 288, smem_w<float>(N, NA), st>>>(
      p, K4, nullptr, 1, S, g, tw, part_a, r, sc, p);
  dev_final(part_a, (N / 2) * N, sc, SC_PAP, OP_ALPHA, st);
  wlaunch_b_any<M, float>(g.wtb, S, g, tw, 0, st);
  if (g.wc2 == 4) wlaunch_c2<M, float, 4>(S, g, tw, st);
  else if (g.wc2 == 2) wlaunch_c2<M, float, 2>(S, g, tw, st);
  else if ((g.wtc ? g.wtc : wtile_c<float>()) == 4) wlaunch_c<M, float, 4>(S, g, tw, st);
  else wlaunch_c<M, float, 2>(S, g, tw, st);
  wlaunch_b_any<M, float>(g.wtb, S, g, tw, 1, st);
  wpass_e_xr<M><<<(N / 2) * N, 288, smem_w<float>(N, NA), st>>>(S, g, tw, x, r, p, k0, sc, part_e);
}

template <typename T>
size_t smem_a(int N) { return sizeof(typename Vec2<T>::t) * (size_t)(N + 2 * 9 * padlen(N)); }
template <typename T>
size_t smem_b(int N, int tk) { return sizeof(typename Vec2<T>::t) * (size_t)(N + 2 * tk * padlen(N)); }
template <typename T>
size_t smem_c(int N, int tk) {
  return sizeof(typename Vec2<T>::t) * (size_t)(N + 2 * 9 * tk * padlen(N));
}
// columns per block of pass C: 32-byte rows of the half spectrum per (component, c)
template <typename T>
constexpr int tile_c() { return sizeof(T) == 4 ? 4 : 2; }

// Time one configuration: 2 warm-up and `reps` timed applies, mean milliseconds.
template <typename F>
cudaError_t time_applies(F&& apply, int reps, cudaStream_t st, float* ms) {
  cudaEvent_t e0, e1;
  cudaError_t e;
  if ((e = cudaEventCreate(&e0))) return e;
  if ((e = cudaEventCreate(&e1))) { cudaEventDestroy(e0); return e; }
  for (int i = 0; i < 2; i++) apply();
  cudaEventRecord(e0, st);
  for (int i = 0; i < reps; i++) apply();
  cudaEventRecord(e1, st);
  e = cudaEventSynchronize(e1);
  if (e == cudaSuccess) e = cudaGetLastError();
  float t = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
  *ms = t / reps;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return e;
}

template <typename C>
cudaError_t tune_tiles(GridDesc& g, C&& one_apply, cudaStream_t st, float* best_ms,
                       bool all_shapes) {
  float best = 1e30f;
  int btb = 16, btc = 2, bc2 = 0;
  const bool regs_c = all_shapes && g.N <= C2_MAX_N;  // FP32 only (all_shapes)
  for (int tb : TB_CAND)
    for (int tc : TC_CAND)
      for (int c2 : C2_CAND) {
        if (!all_shapes && (tb == 8 || tc == 4)) continue;
        // one loop over the tiles of the grid's slowest-axis algorithm
        if (regs_c ? tc != TC_CAND[0] : c2 != C2_CAND[0]) continue;
        g.wtb = tb;
        g.wtc = tc;
        g.wc2 = regs_c ? c2 : 0;
        float ms = 0.f;
        cudaError_t e = time_applies([&] { one_apply(g); }, 5, st, &ms);
        if (e != cudaSuccess) return e;
        if (ms < best) { best = ms; btb = tb; btc = tc; bc2 = g.wc2; }
      }
  g.wtb = btb;
  g.wtc = btc;
  g.wc2 = bc2;
  if (best_ms) *best_ms = best;
  return cudaSuccess;
}

}  // namespace
