// krylov.cu -- vector kernels of the device-resident Newton-Krylov loop: CG updates,
// deterministic two-stage reductions (warp shuffles inside a block, one partial per
// block, a single-block final pass), field fills and precision casts.
#include "krylov.cuh"

namespace {

constexpr int RB = 256;  // threads per reduction block

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double block_sum(double v) {
  __shared__ double ws[RB / 32];
  v = warp_sum(v);
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) ws[w] = v;
  __syncthreads();
  v = threadIdx.x < RB / 32 ? ws[threadIdx.x] : 0.0;
  if (w == 0) v = warp_sum(v);
  return v;  // valid in thread 0
}

template <typename TA, typename TB>
__global__ void __launch_bounds__(RB) k_dot(const TA* __restrict__ a, const TB* __restrict__ b,
                                            long long n, double* __restrict__ part) {
  TA s = 0;
  for (long long i = (long long)blockIdx.x * RB + threadIdx.x; i < n; i += (long long)gridDim.x * RB)
    s += a[i] * (TA)b[i];
  double sb = block_sum((double)s);
  if (threadIdx.x == 0) part[blockIdx.x] = sb;
}

// final pass: sc[slot] = sum(part); op-specific scalar follow-ups for CG
__global__ void __launch_bounds__(1024) k_final(const double* __restrict__ part, int np,
                                                double* __restrict__ sc, int slot, int op) {
  __shared__ double ws[32];
  double v = 0.0;
  for (int i = threadIdx.x; i < np; i += 1024) v += part[i];
  v = warp_sum(v);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    v = ws[threadIdx.x];
    v = warp_sum(v);
    if (threadIdx.x == 0) {
      sc[slot] = v;
      if (op == OP_ALPHA) sc[SC_ALPHA] = sc[SC_RR] / v;          // alpha = rr / pAp
      else if (op == OP_BETA) sc[SC_BETA] = v / sc[SC_RR];       // beta = rr_new / rr
    }
  }
}

// x += alpha p ; r -= alpha Ap ; partial r.r
template <typename T>
__global__ void __launch_bounds__(RB) k_cg_xr(T* __restrict__ x, T* __restrict__ r,
                                              const T* __restrict__ p, const T* __restrict__ Ap,
                                              long long n, const double* __restrict__ sc,
                                              double* __restrict__ part) {
  // arithmetic in T: on GB300 an FP64 instruction costs ~64 FP32 ones, so the FP32
  // vectors stay in FP32; per-thread partial sums are promoted only for the block sum
  const T alpha = (T)sc[SC_ALPHA];
  T s = 0;
  for (long long i = (long long)blockIdx.x * RB + threadIdx.x; i < n; i += (long long)gridDim.x * RB) {
    x[i] = x[i] + alpha * p[i];
    T ri = r[i] - alpha * Ap[i];
    r[i] = ri;
    s += ri * ri;
  }
  double sb = block_sum((double)s);
  if (threadIdx.x == 0) part[blockIdx.x] = sb;
}

// FP32 form with 16-byte vector accesses (n % 4 elements handled by a scalar tail)
__global__ void __launch_bounds__(RB) k_cg_xr4(float* __restrict__ x, float* __restrict__ r,
                                               const float* __restrict__ p,
                                               const float* __restrict__ Ap, long long n,
                                               const double* __restrict__ sc,
                                               double* __restrict__ part) {
  const float alpha = (float)sc[SC_ALPHA];
  const long long n4 = n >> 2, stride = (long long)gridDim.x * RB;
  float4* x4 = reinterpret_cast<float4*>(x);
  float4* r4 = reinterpret_cast<float4*>(r);
  const float4* p4 = reinterpret_cast<const float4*>(p);
  const float4* a4 = reinterpret_cast<const float4*>(Ap);
  float s = 0.f;
  const long long t0 = (long long)blockIdx.x * RB + threadIdx.x;
  for (long long i = t0; i < n4; i += stride) {
    float4 xv = x4[i], pv = p4[i], rv = r4[i], av = a4[i];
    xv.x += alpha * pv.x; xv.y += alpha * pv.y; xv.z += alpha * pv.z; xv.w += alpha * pv.w;
    rv.x -= alpha * av.x; rv.y -= alpha * av.y; rv.z -= alpha * av.z; rv.w -= alpha * av.w;
    x4[i] = xv;
    r4[i] = rv;
    s += rv.x * rv.x + rv.y * rv.y + rv.z * rv.z + rv.w * rv.w;
  }
  for (long long i = 4 * n4 + t0; i < n; i += stride) {
    x[i] = x[i] + alpha * p[i];
    float ri = r[i] - alpha * Ap[i];
    r[i] = ri;
    s += ri * ri;
  }
  double sb = block_sum((double)s);
  if (threadIdx.x == 0) part[blockIdx.x] = sb;
}

__global__ void k_cg_p4(float* __restrict__ p, const float* __restrict__ r, long long n,
                        double* __restrict__ sc) {
  const float beta = (float)sc[SC_BETA];
  const long long n4 = n >> 2, stride = (long long)gridDim.x * blockDim.x;
  const long long t0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  float4* p4 = reinterpret_cast<float4*>(p);
  const float4* r4 = reinterpret_cast<const float4*>(r);
  for (long long i = t0; i < n4; i += stride) {
    float4 pv = p4[i], rv = r4[i];
    pv.x = rv.x + beta * pv.x; pv.y = rv.y + beta * pv.y;
    pv.z = rv.z + beta * pv.z; pv.w = rv.w + beta * pv.w;
    p4[i] = pv;
  }
  for (long long i = 4 * n4 + t0; i < n; i += stride) p[i] = r[i] + beta * p[i];
  __syncthreads();
  if (blockIdx.x == 0 && threadIdx.x == 0) sc[SC_RR] = sc[SC_RRNEW];
}

// p = r + beta p ; rr <- rr_new
template <typename T>
__global__ void k_cg_p(T* __restrict__ p, const T* __restrict__ r, long long n,
                       double* __restrict__ sc) {
  const T beta = (T)sc[SC_BETA];
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    p[i] = r[i] + beta * p[i];
  __syncthreads();
  if (blockIdx.x == 0 && threadIdx.x == 0) sc[SC_RR] = sc[SC_RRNEW];
}

__global__ void k_axpy(double* __restrict__ y, const double* __restrict__ x, double a, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    y[i] += a * x[i];
}
__global__ void k_scale(double* __restrict__ y, double a, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    y[i] *= a;
}
__global__ void k_scale_f(float* __restrict__ y, float a, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    y[i] *= a;
}
__global__ void k_sub(double* __restrict__ y, const double* __restrict__ a,
                      const double* __restrict__ b, long long n) {  // y = a - b
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    y[i] = a[i] - b[i];
}
// fill component c of a (9, N3) field with v[c]
__global__ void k_fill9(double* __restrict__ y, long long N3, double v0, double v1, double v2,
                        double v3, double v4, double v5, double v6, double v7, double v8) {
  const double v[9] = {v0, v1, v2, v3, v4, v5, v6, v7, v8};
  long long n = 9 * N3;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    y[i] = v[i / N3];
}
__global__ void k_add_const(double* __restrict__ y, double v, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    y[i] += v;
}
// y_f = (float)(x * s)
__global__ void k_to_f32(float* __restrict__ y, const double* __restrict__ x, double s, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    y[i] = (float)(x[i] * s);
}
// y += s * (double)x_f
__global__ void k_add_f32(double* __restrict__ y, const float* __restrict__ x, double s, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    y[i] += s * (double)x[i];
}
// sums of each of the 9 components of a (9, N3) field (one partial per block and comp)
__global__ void __launch_bounds__(RB) k_sum9(const double* __restrict__ x, long long N3,
                                             double* __restrict__ part) {
  for (int c = 0; c < 9; c++) {
    double s = 0.0;
    for (long long i = (long long)blockIdx.x * RB + threadIdx.x; i < N3; i += (long long)gridDim.x * RB)
      s += x[c * N3 + i];
    s = block_sum(s);
    if (threadIdx.x == 0) part[c * gridDim.x + blockIdx.x] = s;
    __syncthreads();
  }
}

// ---- K0-weighted forms of the reference-medium preconditioned FP32 CG ----------------
// The CG of the preconditioned operator G0(K : .) runs in the inner product
// <a, b>_K0 = sum_v a_v . (K0 b_v), K0 the (normalised, symmetrised) 9x9 reference stiffness
// of the calling context (device memory, staged in shared memory per block).
__device__ __forceinline__ void load_k0(const float* __restrict__ k0, float* s_k0) {
  for (int i = threadIdx.x; i < 81; i += blockDim.x) s_k0[i] = k0[i];
  __syncthreads();
}
__device__ __forceinline__ float k0_form(const float* s_k0, const float* a, const float* b) {
  float s = 0.f;
#pragma unroll
  for (int i = 0; i < 9; i++) {
    float t = 0.f;
#pragma unroll
    for (int j = 0; j < 9; j++) t += s_k0[9 * i + j] * b[j];
    s += a[i] * t;
  }
  return s;
}

// x += alpha p ; r -= alpha Ap ; partial <r, r>_K0 -- one voxel's 9 components per thread
// (component-major fields), four voxels at a time with 16-byte accesses when N3 % 4 == 0
__global__ void __launch_bounds__(RB) k_cg_xr_k0(float* __restrict__ x, float* __restrict__ r,
                                                 const float* __restrict__ p,
                                                 const float* __restrict__ Ap, long long N3,
                                                 const float* __restrict__ k0,
                                                 const double* __restrict__ sc,
                                                 double* __restrict__ part) {
  __shared__ float s_k0[81];
  load_k0(k0, s_k0);
  const float alpha = (float)sc[SC_ALPHA];
  const long long stride = (long long)gridDim.x * RB, t0 = (long long)blockIdx.x * RB + threadIdx.x;
  float s = 0.f;
  if ((N3 & 3) == 0) {
    const long long n4 = N3 >> 2;
    for (long long v = t0; v < n4; v += stride) {
      float rv[4][9];
#pragma unroll
      for (int i = 0; i < 9; i++) {
        const long long k = i * n4 + v;
        float4 xv = reinterpret_cast<float4*>(x)[k];
        const float4 pv = reinterpret_cast<const float4*>(p)[k];
        float4 qv = reinterpret_cast<float4*>(r)[k];
        const float4 av = reinterpret_cast<const float4*>(Ap)[k];
        xv.x += alpha * pv.x; xv.y += alpha * pv.y; xv.z += alpha * pv.z; xv.w += alpha * pv.w;
        qv.x -= alpha * av.x; qv.y -= alpha * av.y; qv.z -= alpha * av.z; qv.w -= alpha * av.w;
        reinterpret_cast<float4*>(x)[k] = xv;
        reinterpret_cast<float4*>(r)[k] = qv;
        rv[0][i] = qv.x; rv[1][i] = qv.y; rv[2][i] = qv.z; rv[3][i] = qv.w;
      }
#pragma unroll
      for (int u = 0; u < 4; u++) s += k0_form(s_k0, rv[u], rv[u]);
    }
  } else {
    for (long long v = t0; v < N3; v += stride) {
      float rv[9];
#pragma unroll
      for (int i = 0; i < 9; i++) {
        const long long k = i * N3 + v;
        x[k] += alpha * p[k];
        rv[i] = r[k] - alpha * Ap[k];
        r[k] = rv[i];
      }
      s += k0_form(s_k0, rv, rv);
    }
  }
  double sb = block_sum((double)s);
  if (threadIdx.x == 0) part[blockIdx.x] = sb;
}

// partial <a, b>_K0
__global__ void __launch_bounds__(RB) k_dot_k0(const float* __restrict__ a, const float* __restrict__ b,
                                               long long N3, const float* __restrict__ k0,
                                               double* __restrict__ part) {
  __shared__ float s_k0[81];
  load_k0(k0, s_k0);
  float s = 0.f;
  for (long long v = (long long)blockIdx.x * RB + threadIdx.x; v < N3; v += (long long)gridDim.x * RB) {
    float av[9], bv[9];
#pragma unroll
    for (int i = 0; i < 9; i++) { av[i] = a[i * N3 + v]; bv[i] = b[i * N3 + v]; }
    s += k0_form(s_k0, av, bv);
  }
  double sb = block_sum((double)s);
  if (threadIdx.x == 0) part[blockIdx.x] = sb;
}

// component sums of an (81, N3) FP32 field: part[m * gridDim.x + blockIdx.x]
__global__ void __launch_bounds__(RB) k_sum81(const float* __restrict__ K, long long N3,
                                              double* __restrict__ part) {
  const int m = blockIdx.y;
  double s = 0.0;
  for (long long v = (long long)blockIdx.x * RB + threadIdx.x; v < N3; v += (long long)gridDim.x * RB)
    s += (double)K[m * N3 + v];
  s = block_sum(s);
  if (threadIdx.x == 0) part[m * gridDim.x + blockIdx.x] = s;
}

// out[m] = sum of the np partials of row m (one block of 64 threads per row, np <= 64)
__global__ void __launch_bounds__(64) k_final_rows(const double* __restrict__ part, int np,
                                                   double* __restrict__ out) {
  __shared__ double ws[2];
  double v = threadIdx.x < np ? part[blockIdx.x * np + threadIdx.x] : 0.0;
  v = warp_sum(v);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) out[blockIdx.x] = ws[0] + ws[1];
}

__global__ void k_cg_cond(double* __restrict__ sc, cudaGraphConditionalHandle h, int use_handle) {
  const double rr = sc[SC_RRNEW];
  const double cnt = sc[SC_CNT] + 1.0;
  sc[SC_CNT] = cnt;
  int stop = STOP_NONE;
  if (!isfinite(rr)) {
    stop = STOP_NONFINITE;
  } else if (!(sc[SC_RR0] > 0.0)) {
    stop = STOP_TEST;  // nothing to reduce: let the caller's true residual decide
  } else {
    const double red = sqrt(fmax(rr, 0.0) / sc[SC_RR0]), est = sc[SC_RN] * red;
    if (red < sc[SC_DELTA] || est <= sc[SC_TOLB] || est <= sc[SC_TOL]) stop = STOP_TEST;
    else if (cnt >= sc[SC_MAXIT]) stop = STOP_MAXIT;
  }
  sc[SC_STOP] = (double)stop;
  if (use_handle) cudaGraphSetConditional(h, stop == STOP_NONE ? 1u : 0u);
}

// The iteration graph's first node: its WHILE loop runs only if the iterations are not
// already stopped (an eager first iteration may have met the stop test), so the host
// launches the graph without reading the stop flag first.
__global__ void k_cg_gate(const double* __restrict__ sc, cudaGraphConditionalHandle h) {
  cudaGraphSetConditional(h, sc[SC_STOP] == (double)STOP_NONE ? 1u : 0u);
}

int grid_for(long long n, int bs) {
  long long b = (n + bs - 1) / bs;
  return (int)(b < 1 ? 1 : (b > 2048 ? 2048 : b));
}

}  // namespace

static cudaError_t counted(int k) {
  g_kernel_launches += k;
  return cudaGetLastError();
}

cudaError_t dev_dot(const double* a, const double* b, long long n, double* part, double* sc,
                    int slot, int op, cudaStream_t st) {
  k_dot<double, double><<<NPART, RB, 0, st>>>(a, b, n, part);
  k_final<<<1, 1024, 0, st>>>(part, NPART, sc, slot, op);
  return counted(2);
}
cudaError_t dev_dot_f(const float* a, const float* b, long long n, double* part, double* sc,
                      int slot, int op, cudaStream_t st) {
  k_dot<float, float><<<NPART, RB, 0, st>>>(a, b, n, part);
  k_final<<<1, 1024, 0, st>>>(part, NPART, sc, slot, op);
  return counted(2);
}
template <typename T>
cudaError_t dev_cg_xr(T* x, T* r, const T* p, const T* Ap, long long n, double* part, double* sc,
                      cudaStream_t st) {
  if (sizeof(T) == 4)
    k_cg_xr4<<<NPART, RB, 0, st>>>((float*)x, (float*)r, (const float*)p, (const float*)Ap, n,
                                   sc, part);
  else
    k_cg_xr<T><<<NPART, RB, 0, st>>>(x, r, p, Ap, n, sc, part);
  k_final<<<1, 1024, 0, st>>>(part, NPART, sc, SC_RRNEW, OP_BETA);
  return counted(2);
}
template <typename T>
cudaError_t dev_cg_p(T* p, const T* r, long long n, double* sc, cudaStream_t st) {
  if (sizeof(T) == 4)
    k_cg_p4<<<grid_for(n / 4 + 1, 256), 256, 0, st>>>((float*)p, (const float*)r, n, sc);
  else
    k_cg_p<T><<<grid_for(n, 256), 256, 0, st>>>(p, r, n, sc);
  return counted(1);
}
cudaError_t dev_final(double* part, int np, double* sc, int slot, int op, cudaStream_t st) {
  k_final<<<1, 1024, 0, st>>>(part, np, sc, slot, op);
  return counted(1);
}
template cudaError_t dev_cg_xr<double>(double*, double*, const double*, const double*, long long,
                                       double*, double*, cudaStream_t);
template cudaError_t dev_cg_xr<float>(float*, float*, const float*, const float*, long long,
                                      double*, double*, cudaStream_t);
template cudaError_t dev_cg_p<double>(double*, const double*, long long, double*, cudaStream_t);
template cudaError_t dev_cg_p<float>(float*, const float*, long long, double*, cudaStream_t);

cudaError_t dev_axpy(double* y, const double* x, double a, long long n, cudaStream_t st) {
  k_axpy<<<grid_for(n, 256), 256, 0, st>>>(y, x, a, n);
  return counted(1);
}
cudaError_t dev_scale(double* y, double a, long long n, cudaStream_t st) {
  k_scale<<<grid_for(n, 256), 256, 0, st>>>(y, a, n);
  return counted(1);
}
cudaError_t dev_scale_f(float* y, float a, long long n, cudaStream_t st) {
  k_scale_f<<<grid_for(n, 256), 256, 0, st>>>(y, a, n);
  return counted(1);
}
cudaError_t dev_sub(double* y, const double* a, const double* b, long long n, cudaStream_t st) {
  k_sub<<<grid_for(n, 256), 256, 0, st>>>(y, a, b, n);
  return counted(1);
}
cudaError_t dev_fill9(double* y, long long N3, const double* v, cudaStream_t st) {
  k_fill9<<<grid_for(9 * N3, 256), 256, 0, st>>>(y, N3, v[0], v[1], v[2], v[3], v[4], v[5], v[6],
                                                  v[7], v[8]);
  return counted(1);
}
cudaError_t dev_add_const(double* y, double v, long long n, cudaStream_t st) {
  k_add_const<<<grid_for(n, 256), 256, 0, st>>>(y, v, n);
  return counted(1);
}
cudaError_t dev_to_f32(float* y, const double* x, double s, long long n, cudaStream_t st) {
  k_to_f32<<<grid_for(n, 256), 256, 0, st>>>(y, x, s, n);
  return counted(1);
}
cudaError_t dev_add_f32(double* y, const float* x, double s, long long n, cudaStream_t st) {
  k_add_f32<<<grid_for(n, 256), 256, 0, st>>>(y, x, s, n);
  return counted(1);
}
cudaError_t dev_sum9(const double* x, long long N3, double* part, double* sc, int slot0,
                     cudaStream_t st) {
  k_sum9<<<NPART, RB, 0, st>>>(x, N3, part);
  for (int c = 0; c < 9; c++)
    k_final<<<1, 1024, 0, st>>>(part + c * NPART, NPART, sc, slot0 + c, OP_STORE);
  return counted(10);
}

cudaError_t dev_cg_xr_k0(float* x, float* r, const float* p, const float* Ap, long long N3,
                         const float* k0, double* part, double* sc, cudaStream_t st) {
  k_cg_xr_k0<<<NPART, RB, 0, st>>>(x, r, p, Ap, N3, k0, sc, part);
  k_final<<<1, 1024, 0, st>>>(part, NPART, sc, SC_RRNEW, OP_BETA);
  return counted(2);
}
cudaError_t dev_dot_k0(const float* a, const float* b, long long N3, const float* k0,
                       double* part, double* sc, int slot, int op, cudaStream_t st) {
  k_dot_k0<<<NPART, RB, 0, st>>>(a, b, N3, k0, part);
  k_final<<<1, 1024, 0, st>>>(part, NPART, sc, slot, op);
  return counted(2);
}
cudaError_t dev_mean81(const float* K, long long N3, double* part, double* sc81, cudaStream_t st) {
  constexpr int NB = 64;
  k_sum81<<<dim3(NB, 81), RB, 0, st>>>(K, N3, part);
  k_final_rows<<<81, 64, 0, st>>>(part, NB, sc81);
  return counted(2);
}
cudaError_t dev_cg_cond(double* sc, cudaGraphConditionalHandle h, bool use_handle,
                        cudaStream_t st) {
  k_cg_cond<<<1, 1, 0, st>>>(sc, h, use_handle ? 1 : 0);
  return counted(1);
}

cudaError_t dev_cg_gate(const double* sc, cudaGraphConditionalHandle h, cudaStream_t st) {
  k_cg_gate<<<1, 1, 0, st>>>(sc, h);
  return counted(1);
}
