// mlp.cu -- training and batch inference of the learned initial guess (mlp.cuh) on the
// tcgen05 tensor cores: BF16 operands in shared memory, FP32 accumulators in TMEM.
//
// Training step on a minibatch of B tiles of 128 samples:
//   k_train_fwd  forward pass per tile; keeps the BF16 activations, SiLU'(z) and dL/dY
//   k_train_bwd  dA2 = dY W3, dW3^T = A2^T dY, dA1 = dZ2 W2, dW2 = dZ2^T A1, dW1 = dZ1^T X,
//                bias gradients; one partial gradient vector per tile
//   k_adam       sums the tile partials in a fixed order and applies Adam to the FP32
//                master weights
//   k_pack       BF16 operand copies of the weights (forward and transposed layouts)
// Loss: mean over samples and the NOUT outputs of the squared error in normalised units.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "common.cuh"
#include "mlp.cuh"

using namespace mlp;

namespace {

constexpr int BWD_SMEM = 2 * (TM * NO + NO * TM + NH * NO + NH * TM + TM * NH + NH * TM +
                              NH * NH + NH * TM + KIN * TM) + 64;

// per-tile intermediates of the forward pass kept for the backward pass
struct TileScratch {
  __nv_bfloat16 *A1, *A2;   // [tile][TM][NH] activations (BF16, as the MMAs saw them)
  float *S1, *S2;           // [tile][TM][NH] SiLU'(z)
  float* dY;                // [tile][TM][NO] dL/dY (normalised units), zero when masked
  __nv_bfloat16* X;         // [tile][TM][KIN] normalised inputs (BF16)
  float* loss;              // [tile] partial sums of squared errors
};

__global__ void k_pack(const float* __restrict__ p, __nv_bfloat16* __restrict__ q) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  auto put = [&](int base, int r, int k, int K, float v) {
    q[base + tc::kmaj_off(r, k, K) / 2] = __float2bfloat16_rn(v);
  };
  if (i < NH * KIN) {  // W1 [h][i]
    int h = i / KIN, k = i % KIN;
    put(K_W1, h, k, KIN, p[P_W1 + i]);
  }
  if (i < NH * NH) {  // W2 [j][h] and W2^T [h][j]
    int j = i / NH, h = i % NH;
    float v = p[P_W2 + i];
    put(K_W2, j, h, NH, v);
    put(K_W2T, h, j, NH, v);
  }
  if (i < NO * NH) {  // W3 [o][j] and W3^T [j][o]
    int o = i / NH, j = i % NH;
    float v = p[P_W3 + i];
    put(K_W3, o, j, NH, v);
    put(K_W3T, j, o, NO, v);
  }
}

// batch inference: raw features X[n][NIN] -> raw outputs Y[n][NOUT]
__global__ void __launch_bounds__(TM) k_forward(Weights w, const float* __restrict__ X,
                                                float* __restrict__ Y, int n, int* err) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tslot;
  if (threadIdx.x == 0) {
    tc::mbar_init(&bar, 1);
    tc::fence_mbar_init();
  }
  const uint32_t tmem = tmem_block_alloc(&tslot, 256);
  uint32_t phase = 0;
  const long long s = (long long)blockIdx.x * TM + threadIdx.x;
  float f[NIN], o[NOUT];
  for (int i = 0; i < NIN; i++) f[i] = s < n ? X[s * NIN + i] : 0.0f;
  if (!forward_tile(w, smem, tmem, &bar, &phase, f, o)) atomicExch(err, 1);
  if (s < n)
    for (int i = 0; i < NOUT; i++) Y[s * NOUT + i] = o[i];
  tmem_block_free(tmem, 256);
}

// forward pass of one training tile (samples idx[tile * TM + r], masked past n)
__global__ void __launch_bounds__(TM) k_train_fwd(Weights w, const float* __restrict__ X,
                                                  const float* __restrict__ T,
                                                  const int* __restrict__ idx, long long first,
                                                  long long n, float inv_count, TileScratch sc,
                                                  int* err) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tslot;
  __shared__ float red[TM / 32];
  unsigned char* sW1 = smem;
  unsigned char* sW2 = sW1 + 2 * NH * KIN;
  unsigned char* sW3 = sW2 + 2 * NH * NH;
  unsigned char* sX = sW3 + 2 * NO * NH;
  unsigned char* sA = sX + 2 * TM * KIN;
  float* sb = reinterpret_cast<float*>(sA + 2 * TM * NH);
  if (threadIdx.x == 0) {
    tc::mbar_init(&bar, 1);
    tc::fence_mbar_init();
  }
  const uint32_t tmem = tmem_block_alloc(&tslot, 256);
  uint32_t phase = 0;
  const int r = threadIdx.x, wq = r >> 5, tile = blockIdx.x;
  const long long pos = first + (long long)tile * TM + r;
  const bool valid = pos < n;
  const long long s = valid ? idx[pos] : 0;
  copy16(sW1, w.packed + K_W1, NH * KIN / 8);
  copy16(sW2, w.packed + K_W2, NH * NH / 8);
  copy16(sW3, w.packed + K_W3, NO * NH / 8);
  for (int i = threadIdx.x; i < NH; i += blockDim.x) {
    sb[i] = w.params[P_B1 + i];
    sb[NH + i] = w.params[P_B2 + i];
  }
  if (threadIdx.x < NO) sb[2 * NH + threadIdx.x] = w.params[P_B3 + threadIdx.x];
  const size_t row = (size_t)tile * TM + r;
  {
    float x[KIN];
    for (int i = 0; i < KIN; i++)
      x[i] = (valid && i < NIN) ? (X[s * NIN + i] - w.norm[i]) * w.norm[NIN + i] : 0.0f;
    for (int k = 0; k < KIN; k += 8) {
      st_row8(sX, r, k, KIN, x + k);
      *reinterpret_cast<uint4*>(sc.X + row * KIN + k) = pack8(x + k);
    }
  }
  operands_ready();
  bool ok = true;
  if (r == 0) gemm_issue(tmem, sX, sW1, KIN, TM, NH, &bar);
  ok &= gemm_wait(&bar, &phase);
  for (int c = 0; c < NH; c += 16) {
    float v[16];
    tc::tmem_ld16(tc::taddr(tmem, 32 * wq, c), v);
    for (int i = 0; i < 16; i++) {
      float z = v[i] + sb[c + i];
      sc.S1[row * NH + c + i] = dsilu(z);
      v[i] = silu(z);
    }
    uint4 q0 = pack8(v), q1 = pack8(v + 8);
    *reinterpret_cast<uint4*>(sA + tc::kmaj_off(r, c, NH)) = q0;
    *reinterpret_cast<uint4*>(sA + tc::kmaj_off(r, c + 8, NH)) = q1;
    *reinterpret_cast<uint4*>(sc.A1 + row * NH + c) = q0;
    *reinterpret_cast<uint4*>(sc.A1 + row * NH + c + 8) = q1;
  }
  operands_ready();
  if (r == 0) gemm_issue(tmem + NH, sA, sW2, NH, TM, NH, &bar);
  ok &= gemm_wait(&bar, &phase);
  for (int c = 0; c < NH; c += 16) {
    float v[16];
    tc::tmem_ld16(tc::taddr(tmem, 32 * wq, NH + c), v);
    for (int i = 0; i < 16; i++) {
      float z = v[i] + sb[NH + c + i];
      sc.S2[row * NH + c + i] = dsilu(z);
      v[i] = silu(z);
    }
    uint4 q0 = pack8(v), q1 = pack8(v + 8);
    *reinterpret_cast<uint4*>(sA + tc::kmaj_off(r, c, NH)) = q0;
    *reinterpret_cast<uint4*>(sA + tc::kmaj_off(r, c + 8, NH)) = q1;
    *reinterpret_cast<uint4*>(sc.A2 + row * NH + c) = q0;
    *reinterpret_cast<uint4*>(sc.A2 + row * NH + c + 8) = q1;
  }
  operands_ready();
  if (r == 0) gemm_issue(tmem, sA, sW3, NH, TM, NO, &bar);
  ok &= gemm_wait(&bar, &phase);
  float se = 0.0f;
  {
    float v[16];
    tc::tmem_ld16(tc::taddr(tmem, 32 * wq, 0), v);
    for (int o = 0; o < NO; o++) {
      float d = 0.0f;
      if (valid && o < NOUT) {
        float t = (T[s * NOUT + o] - w.norm[2 * NIN + o]) / w.norm[2 * NIN + NOUT + o];
        d = v[o] + sb[2 * NH + o] - t;
        se += d * d;
      }
      sc.dY[row * NO + o] = 2.0f * d * inv_count;
    }
  }
  for (int off = 16; off > 0; off >>= 1) se += __shfl_down_sync(0xffffffffu, se, off);
  if ((r & 31) == 0) red[r >> 5] = se;
  tmem_block_free(tmem, 256);
  if (r == 0) {
    sc.loss[tile] = red[0] + red[1] + red[2] + red[3];
    if (!ok) atomicExch(err, 1);
  }
}

// column sums over the 128 rows of the block (thread r holds row r): fixed-order tree
__device__ void colsum16(const float* v, float* red /*[4][16]*/, float* out /*16*/) {
  float s[16];
  for (int i = 0; i < 16; i++) {
    float x = v[i];
    for (int off = 16; off > 0; off >>= 1) x += __shfl_down_sync(0xffffffffu, x, off);
    s[i] = x;
  }
  if ((threadIdx.x & 31) == 0)
    for (int i = 0; i < 16; i++) red[(threadIdx.x >> 5) * 16 + i] = s[i];
  __syncthreads();
  if (threadIdx.x < 16)
    out[threadIdx.x] = red[threadIdx.x] + red[16 + threadIdx.x] + red[32 + threadIdx.x] +
                       red[48 + threadIdx.x];
  __syncthreads();
}

__global__ void __launch_bounds__(TM) k_train_bwd(Weights w, TileScratch sc, float* __restrict__ gpart,
                                                  int* err) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tslot;
  __shared__ float red[64];
  __shared__ float colout[16];
  unsigned char* sdYn = smem;                  // [b][o]  K = NO
  unsigned char* sdYt = sdYn + 2 * TM * NO;    // [o][b]  K = TM
  unsigned char* sW3t = sdYt + 2 * NO * TM;    // [j][o]  K = NO
  unsigned char* sA2t = sW3t + 2 * NH * NO;    // [j][b]  K = TM
  unsigned char* sZn = sA2t + 2 * NH * TM;     // [b][j]  K = NH   (dZ2, later dZ1^T)
  unsigned char* sZt = sZn + 2 * TM * NH;      // [j][b]  K = TM   (dZ2^T)
  unsigned char* sW2t = sZt + 2 * NH * TM;     // [h][j]  K = NH
  unsigned char* sA1t = sW2t + 2 * NH * NH;    // [h][b]  K = TM
  unsigned char* sXt = sA1t + 2 * NH * TM;     // [i][b]  K = TM
  if (threadIdx.x == 0) {
    tc::mbar_init(&bar, 1);
    tc::fence_mbar_init();
  }
  const uint32_t tmem = tmem_block_alloc(&tslot, 512);
  uint32_t phase = 0;
  const int r = threadIdx.x, wq = r >> 5, tile = blockIdx.x;
  const size_t row = (size_t)tile * TM + r;
  float* g = gpart + (size_t)tile * P_TOTAL;
  copy16(sW3t, w.packed + K_W3T, NH * NO / 8);
  copy16(sW2t, w.packed + K_W2T, NH * NH / 8);
  {
    float dy[NO];
    for (int o = 0; o < NO; o++) dy[o] = sc.dY[row * NO + o];
    st_row8(sdYn, r, 0, NO, dy);
    st_row8(sdYn, r, 8, NO, dy + 8);
    for (int o = 0; o < NO; o++) st_el(sdYt, o, r, TM, dy[o]);
    colsum16(dy, red, colout);  // db3
    if (r < NO) g[P_B3 + r] = colout[r];
    for (int j = 0; j < NH; j++) {
      st_el(sA2t, j, r, TM, __bfloat162float(sc.A2[row * NH + j]));
      st_el(sA1t, j, r, TM, __bfloat162float(sc.A1[row * NH + j]));
    }
    for (int i = 0; i < KIN; i++) st_el(sXt, i, r, TM, __bfloat162float(sc.X[row * KIN + i]));
  }
  operands_ready();
  bool ok = true;
  // dA2 = dY W3 -> cols [0,128); dW3^T = A2^T dY -> cols [128,144)
  if (r == 0) {
    gemm_mma(tmem, sdYn, sW3t, NO, TM, NH);
    gemm_issue(tmem + NH, sA2t, sdYt, TM, NH, NO, &bar);  // one commit covers both
  }
  ok &= gemm_wait(&bar, &phase);
  {
    float v[16];
    tc::tmem_ld16(tc::taddr(tmem, 32 * wq, NH), v);  // dW3^T row j = r
    for (int o = 0; o < NO; o++) g[P_W3 + o * NH + r] = v[o];
  }
  for (int c = 0; c < NH; c += 16) {
    float v[16];
    tc::tmem_ld16(tc::taddr(tmem, 32 * wq, c), v);
    for (int i = 0; i < 16; i++) v[i] *= sc.S2[row * NH + c + i];  // dZ2
    st_row8(sZn, r, c, NH, v);
    st_row8(sZn, r, c + 8, NH, v + 8);
    for (int i = 0; i < 16; i++) st_el(sZt, c + i, r, TM, v[i]);
    colsum16(v, red, colout);  // db2
    if (r < 16) g[P_B2 + c + r] = colout[r];
  }
  operands_ready();
  // dA1 = dZ2 W2 -> cols [0,128); dW2 = dZ2^T A1 -> cols [128,256)
  if (r == 0) {
    gemm_mma(tmem, sZn, sW2t, NH, TM, NH);
    gemm_issue(tmem + NH, sZt, sA1t, TM, NH, NH, &bar);
  }
  ok &= gemm_wait(&bar, &phase);
  for (int c = 0; c < NH; c += 16) {
    float v[16];
    tc::tmem_ld16(tc::taddr(tmem, 32 * wq, NH + c), v);  // dW2 row j = r
    for (int i = 0; i < 16; i++) g[P_W2 + r * NH + c + i] = v[i];
  }
  for (int c = 0; c < NH; c += 16) {
    float v[16];
    tc::tmem_ld16(tc::taddr(tmem, 32 * wq, c), v);
    for (int i = 0; i < 16; i++) v[i] *= sc.S1[row * NH + c + i];  // dZ1
    for (int i = 0; i < 16; i++) st_el(sZn, c + i, r, TM, v[i]);  // dZ1^T [h][b]
    colsum16(v, red, colout);  // db1
    if (r < 16) g[P_B1 + c + r] = colout[r];
  }
  operands_ready();
  // dW1 = dZ1^T X -> cols [256, 288)
  if (r == 0) gemm_issue(tmem + 2 * NH, sZn, sXt, TM, NH, KIN, &bar);
  ok &= gemm_wait(&bar, &phase);
  for (int c = 0; c < KIN; c += 16) {
    float v[16];
    tc::tmem_ld16(tc::taddr(tmem, 32 * wq, 2 * NH + c), v);  // dW1 row h = r
    for (int i = 0; i < 16; i++) g[P_W1 + r * KIN + c + i] = v[i];
  }
  tmem_block_free(tmem, 512);
  if (r == 0 && !ok) atomicExch(err, 1);
}

__global__ void k_adam(float* __restrict__ p, float* __restrict__ m, float* __restrict__ v,
                       const float* __restrict__ gpart, int ntiles, float lr, float b1, float b2,
                       float c1, float c2, float* __restrict__ gout) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P_TOTAL) return;
  float gsum = 0.0f;
  for (int t = 0; t < ntiles; t++) gsum += gpart[(size_t)t * P_TOTAL + i];
  if (gout) gout[i] = gsum;
  if (lr == 0.0f) return;
  const float mi = b1 * m[i] + (1.0f - b1) * gsum;
  const float vi = b2 * v[i] + (1.0f - b2) * gsum * gsum;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + 1e-8f);
}

}  // namespace

// ------------------------------------------------------------------ host side
namespace {

struct MlpCtx {
  float *params = nullptr, *m = nullptr, *v = nullptr, *norm = nullptr, *gpart = nullptr;
  float *X = nullptr, *T = nullptr;
  int* idx = nullptr;
  __nv_bfloat16* packed = nullptr;
  TileScratch sc{};
  int* err = nullptr;
  int max_tiles = 0;
  long long cap = 0;  // samples the X / T buffers hold
  long long adam_t = 0;
  bool ready = false;
};
MlpCtx g_mlp;

int ck(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    cpfft_set_error("%s: %s", what, cudaGetErrorString(e));
    return CPFFT_ERR_CUDA;
  }
  return 0;
}
#define CKM(x) do { int _r = ck((x), #x); if (_r) return _r; } while (0)
#define TRY(expr) do { int _rc = (expr); if (_rc) return _rc; } while (0)

template <typename P>
int dalloc_m(P*& p, size_t bytes) {
  if (p) cudaFree(p);
  p = nullptr;
  return ck(cudaMalloc((void**)&p, bytes), "cudaMalloc (mlp)");
}

int ensure_tiles(int tiles) {
  MlpCtx& c = g_mlp;
  if (tiles <= c.max_tiles) return 0;
  const size_t rows = (size_t)tiles * TM;
  int rc;
  if ((rc = dalloc_m(c.sc.A1, rows * NH * 2)) || (rc = dalloc_m(c.sc.A2, rows * NH * 2)) ||
      (rc = dalloc_m(c.sc.S1, rows * NH * 4)) || (rc = dalloc_m(c.sc.S2, rows * NH * 4)) ||
      (rc = dalloc_m(c.sc.dY, rows * NO * 4)) || (rc = dalloc_m(c.sc.X, rows * KIN * 2)) ||
      (rc = dalloc_m(c.sc.loss, tiles * 4)) ||
      (rc = dalloc_m(c.gpart, (size_t)tiles * P_TOTAL * 4)))
    return rc;
  c.max_tiles = tiles;
  return 0;
}

int ensure_data(long long n) {
  MlpCtx& c = g_mlp;
  if (n <= c.cap) return 0;
  int rc;
  if ((rc = dalloc_m(c.X, (size_t)n * NIN * 4)) || (rc = dalloc_m(c.T, (size_t)n * NOUT * 4)) ||
      (rc = dalloc_m(c.idx, (size_t)n * 4)))
    return rc;
  c.cap = n;
  return 0;
}

Weights weights() { return Weights{g_mlp.packed, g_mlp.params, g_mlp.norm}; }

int pack() {
  k_pack<<<(NH * NH + 255) / 256, 256>>>(g_mlp.params, g_mlp.packed);
  g_kernel_launches++;
  return ck(cudaGetLastError(), "k_pack");
}

int check_err() {
  int e = 0;
  CKM(cudaMemcpy(&e, g_mlp.err, sizeof(int), cudaMemcpyDeviceToHost));
  if (e) {
    cpfft_set_error("MLP: a tensor-core wait gave up");
    return CPFFT_ERR_CUDA;
  }
  return 0;
}

int set_attrs() {
  CKM(cudaFuncSetAttribute(k_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, FWD_SMEM));
  CKM(cudaFuncSetAttribute(k_train_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, FWD_SMEM));
  CKM(cudaFuncSetAttribute(k_train_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize, BWD_SMEM));
  return 0;
}

// one forward + backward over tiles [0, ntiles) of the permutation starting at `first`;
// lr > 0 also applies Adam; gout (device) receives the summed gradient when given
int step(long long first, long long n, int ntiles, float lr, float* gout, float* loss_out) {
  MlpCtx& c = g_mlp;
  long long cnt = std::min<long long>((long long)ntiles * TM, n - first);
  const float inv_count = 1.0f / (float)(cnt * NOUT);
  k_train_fwd<<<ntiles, TM, FWD_SMEM>>>(weights(), c.X, c.T, c.idx, first, n, inv_count, c.sc,
                                        c.err);
  k_train_bwd<<<ntiles, TM, BWD_SMEM>>>(weights(), c.sc, c.gpart, c.err);
  float b1 = 0.9f, b2 = 0.999f, c1 = 1.0f, c2 = 1.0f;
  if (lr > 0.0f) {
    c.adam_t++;
    c1 = 1.0f / (1.0f - std::pow(b1, (float)c.adam_t));
    c2 = 1.0f / (1.0f - std::pow(b2, (float)c.adam_t));
  }
  k_adam<<<(P_TOTAL + 255) / 256, 256>>>(c.params, c.m, c.v, c.gpart, ntiles, lr, b1, b2, c1, c2,
                                         gout);
  g_kernel_launches += 3;
  CKM(cudaGetLastError());
  if (lr > 0.0f) TRY(pack());
  if (loss_out) {
    std::vector<float> l(ntiles);
    CKM(cudaMemcpy(l.data(), c.sc.loss, ntiles * sizeof(float), cudaMemcpyDeviceToHost));
    double s = 0;
    for (float x : l) s += x;
    *loss_out = (float)(s / (double)(cnt * NOUT));
  }
  return 0;
}

}  // namespace

// the device weights of the learned initial guess and the tensor-core error flag, for
// the stress-update kernel
bool mlp_device_weights(Weights* w, int** err) {
  if (!g_mlp.ready) return false;
  *w = weights();
  *err = g_mlp.err;
  return true;
}
int mlp_check_error() { return g_mlp.ready ? check_err() : 0; }

extern "C" {

int cpfft_mlp_init(int seed) {
  MlpCtx& c = g_mlp;
  int rc;
  if (!c.params) {
    if ((rc = dalloc_m(c.params, P_TOTAL * 4)) || (rc = dalloc_m(c.m, P_TOTAL * 4)) ||
        (rc = dalloc_m(c.v, P_TOTAL * 4)) || (rc = dalloc_m(c.norm, N_NORM * 4)) ||
        (rc = dalloc_m(c.packed, K_TOTAL * 2)) || (rc = dalloc_m(c.err, sizeof(int))))
      return rc;
    TRY(set_attrs());
  }
  // Glorot-uniform weights (padded rows / columns zero), zero biases, identity scaling
  std::vector<float> p(P_TOTAL, 0.0f), nrm(N_NORM, 0.0f);
  std::mt19937 gen((unsigned)seed);
  auto fill = [&](int off, int rows, int cols, int fan_in, int fan_out, int rmax, int cmax) {
    std::uniform_real_distribution<float> u(-1.0f, 1.0f);
    float a = std::sqrt(6.0f / (float)(fan_in + fan_out));
    for (int i = 0; i < rows; i++)
      for (int j = 0; j < cols; j++) p[off + i * cols + j] = (i < rmax && j < cmax) ? a * u(gen) : 0.0f;
  };
  fill(P_W1, NH, KIN, NIN, NH, NH, NIN);
  fill(P_W2, NH, NH, NH, NH, NH, NH);
  fill(P_W3, NO, NH, NH, NOUT, NOUT, NH);
  for (int i = 0; i < NIN; i++) nrm[NIN + i] = 1.0f;
  for (int i = 0; i < NOUT; i++) nrm[2 * NIN + NOUT + i] = 1.0f;
  CKM(cudaMemcpy(c.params, p.data(), P_TOTAL * 4, cudaMemcpyHostToDevice));
  CKM(cudaMemcpy(c.norm, nrm.data(), N_NORM * 4, cudaMemcpyHostToDevice));
  CKM(cudaMemset(c.m, 0, P_TOTAL * 4));
  CKM(cudaMemset(c.v, 0, P_TOTAL * 4));
  CKM(cudaMemset(c.err, 0, sizeof(int)));
  c.adam_t = 0;
  TRY(pack());
  CKM(cudaDeviceSynchronize());
  c.ready = true;
  return 0;
}

int cpfft_mlp_set_params(const float* params, const float* norm) {
  if (!g_mlp.ready) {
    cpfft_set_error("cpfft_mlp_set_params: cpfft_mlp_init first");
    return CPFFT_ERR_NOT_INIT;
  }
  if (params) CKM(cudaMemcpy(g_mlp.params, params, P_TOTAL * 4, cudaMemcpyHostToDevice));
  if (norm) CKM(cudaMemcpy(g_mlp.norm, norm, N_NORM * 4, cudaMemcpyHostToDevice));
  TRY(pack());
  return ck(cudaDeviceSynchronize(), "mlp set params");
}

int cpfft_mlp_get_params(float* params, float* norm) {
  if (!g_mlp.ready) {
    cpfft_set_error("cpfft_mlp_get_params: cpfft_mlp_init first");
    return CPFFT_ERR_NOT_INIT;
  }
  if (params) CKM(cudaMemcpy(params, g_mlp.params, P_TOTAL * 4, cudaMemcpyDeviceToHost));
  if (norm) CKM(cudaMemcpy(norm, g_mlp.norm, N_NORM * 4, cudaMemcpyDeviceToHost));
  return 0;
}

int cpfft_mlp_forward(const float* X, long long n, float* Y) {
  if (!g_mlp.ready) {
    cpfft_set_error("cpfft_mlp_forward: cpfft_mlp_init first");
    return CPFFT_ERR_NOT_INIT;
  }
  if (n < 0 || (n > 0 && (!X || !Y))) {
    cpfft_set_error("cpfft_mlp_forward: bad arguments");
    return CPFFT_ERR_BAD_ARG;
  }
  if (n == 0) return 0;
  float *dX = nullptr, *dY = nullptr;
  int rc;
  if ((rc = dalloc_m(dX, (size_t)n * NIN * 4)) || (rc = dalloc_m(dY, (size_t)n * NOUT * 4))) {
    if (dX) cudaFree(dX);
    return rc;
  }
  cudaMemcpy(dX, X, (size_t)n * NIN * 4, cudaMemcpyHostToDevice);
  k_forward<<<(unsigned)((n + TM - 1) / TM), TM, FWD_SMEM>>>(weights(), dX, dY, (int)n, g_mlp.err);
  g_kernel_launches++;
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpy(Y, dY, (size_t)n * NOUT * 4, cudaMemcpyDeviceToHost);
  cudaFree(dX);
  cudaFree(dY);
  CKM(e);
  return check_err();
}

// loss and gradient (summed over the batch, normalised units) of one batch, no update
int cpfft_mlp_loss_grad(const float* X, const float* T, long long n, float* grad, float* loss) {
  if (!g_mlp.ready) {
    cpfft_set_error("cpfft_mlp_loss_grad: cpfft_mlp_init first");
    return CPFFT_ERR_NOT_INIT;
  }
  if (n <= 0 || !X || !T) {
    cpfft_set_error("cpfft_mlp_loss_grad: bad arguments");
    return CPFFT_ERR_BAD_ARG;
  }
  const int tiles = (int)((n + TM - 1) / TM);
  TRY(ensure_tiles(tiles));
  TRY(ensure_data(n));
  CKM(cudaMemcpy(g_mlp.X, X, (size_t)n * NIN * 4, cudaMemcpyHostToDevice));
  CKM(cudaMemcpy(g_mlp.T, T, (size_t)n * NOUT * 4, cudaMemcpyHostToDevice));
  std::vector<int> id(n);
  for (long long i = 0; i < n; i++) id[i] = (int)i;
  CKM(cudaMemcpy(g_mlp.idx, id.data(), (size_t)n * 4, cudaMemcpyHostToDevice));
  float* dg = nullptr;
  TRY(dalloc_m(dg, P_TOTAL * 4));
  int rc = step(0, n, tiles, 0.0f, dg, loss);
  if (!rc && grad) rc = ck(cudaMemcpy(grad, dg, P_TOTAL * 4, cudaMemcpyDeviceToHost), "grad copy");
  cudaFree(dg);
  if (rc) return rc;
  return check_err();
}

// Adam on (X, T) pairs held on the host: `epochs` passes over a fresh permutation each,
// minibatches of batch_tiles x 128 samples.  The normalisation is set from the data.
int cpfft_mlp_train(const float* X, const float* T, long long n, int epochs, int batch_tiles,
                    float lr, int seed, float* loss_out) {
  if (!g_mlp.ready) {
    cpfft_set_error("cpfft_mlp_train: cpfft_mlp_init first");
    return CPFFT_ERR_NOT_INIT;
  }
  if (n <= 0 || !X || !T || epochs < 0 || batch_tiles < 1 || !(lr > 0.0f)) {
    cpfft_set_error("cpfft_mlp_train: bad arguments");
    return CPFFT_ERR_BAD_ARG;
  }
  // normalisation from the data (FP64 sums on the host)
  std::vector<float> nrm(N_NORM);
  for (int i = 0; i < NIN; i++) {
    double s = 0, q = 0;
    for (long long k = 0; k < n; k++) { double x = X[k * NIN + i]; s += x; q += x * x; }
    double mu = s / n, var = q / n - mu * mu;
    nrm[i] = (float)mu;
    nrm[NIN + i] = var > 1e-24 ? (float)(1.0 / std::sqrt(var)) : 1.0f;
  }
  for (int o = 0; o < NOUT; o++) {
    double s = 0, q = 0;
    for (long long k = 0; k < n; k++) { double x = T[k * NOUT + o]; s += x; q += x * x; }
    double mu = s / n, var = q / n - mu * mu;
    nrm[2 * NIN + o] = (float)mu;
    nrm[2 * NIN + NOUT + o] = var > 1e-24 ? (float)std::sqrt(var) : 1.0f;
  }
  CKM(cudaMemcpy(g_mlp.norm, nrm.data(), N_NORM * 4, cudaMemcpyHostToDevice));
  TRY(ensure_tiles(batch_tiles));
  TRY(ensure_data(n));
  CKM(cudaMemcpy(g_mlp.X, X, (size_t)n * NIN * 4, cudaMemcpyHostToDevice));
  CKM(cudaMemcpy(g_mlp.T, T, (size_t)n * NOUT * 4, cudaMemcpyHostToDevice));
  std::mt19937_64 gen((unsigned long long)seed);
  std::vector<int> id(n);
  float last = 0.0f;
  for (int e = 0; e < epochs; e++) {
    for (long long i = 0; i < n; i++) id[i] = (int)i;
    std::shuffle(id.begin(), id.end(), gen);
    CKM(cudaMemcpy(g_mlp.idx, id.data(), (size_t)n * 4, cudaMemcpyHostToDevice));
    double esum = 0.0;
    long long ecount = 0;
    const long long per = (long long)batch_tiles * TM;
    for (long long first = 0; first < n; first += per) {
      int tiles = (int)std::min<long long>(batch_tiles, (n - first + TM - 1) / TM);
      float l = 0.0f;
      TRY(step(first, n, tiles, lr, nullptr, &l));
      long long cnt = std::min<long long>(per, n - first);
      esum += (double)l * cnt;
      ecount += cnt;
    }
    last = (float)(esum / (double)ecount);
  }
  TRY(ck(cudaDeviceSynchronize(), "mlp train"));
  if (loss_out) *loss_out = last;
  return check_err();
}

}  // extern "C"
