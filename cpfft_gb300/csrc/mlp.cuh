// mlp.cuh -- the learned initial guess of the local mm10 Newton solve: a 20-128-128-7
// multilayer perceptron with SiLU activations, BF16 weights and FP32 accumulation,
// evaluated and trained on the tcgen05 tensor cores (mlp.cu).
#pragma once
#include <cuda_bf16.h>
#include <cstdint>

#include "tc.cuh"

namespace mlp {

constexpr int NIN = 20;    // features: lattice quaternion 4, D 6, return-mapped trial stress 6,
                           // tau_n, extrapolated tau, cos(D, D_n), |D|
constexpr int NOUT = 7;    // targets: sigma - sigma_trial (6), tau - tau_extrapolated
constexpr int KIN = 32;    // NIN padded to the MMA K granularity
constexpr int NH = 128;    // hidden width
constexpr int NO = 16;     // NOUT padded to the smallest MMA N
constexpr int TM = 128;    // samples per tile = MMA M = threads per block

// FP32 master parameters, PyTorch Linear layout (out x in), padded rows/columns zero
constexpr int P_W1 = 0;                   // [NH][KIN]
constexpr int P_B1 = P_W1 + NH * KIN;     // [NH]
constexpr int P_W2 = P_B1 + NH;           // [NH][NH]
constexpr int P_B2 = P_W2 + NH * NH;      // [NH]
constexpr int P_W3 = P_B2 + NH;           // [NO][NH]
constexpr int P_B3 = P_W3 + NO * NH;      // [NO]
constexpr int P_TOTAL = P_B3 + NO;        // 22800

// BF16 copies in the tensor-core operand layout (tc::kmaj_off), element offsets
constexpr int K_W1 = 0;                   // W1  rows h, K = input    (forward layer 1)
constexpr int K_W2 = K_W1 + NH * KIN;     // W2  rows j, K = h        (forward layer 2)
constexpr int K_W3 = K_W2 + NH * NH;      // W3  rows o, K = j        (forward layer 3)
constexpr int K_W2T = K_W3 + NO * NH;     // W2^T rows h, K = j       (backward dA1)
constexpr int K_W3T = K_W2T + NH * NH;    // W3^T rows j, K = o       (backward dA2)
constexpr int K_TOTAL = K_W3T + NH * NO;

// feature / target normalisation: mu_in[NIN], inv_sd_in[NIN], mu_out[NOUT], sd_out[NOUT]
constexpr int N_NORM = 2 * NIN + 2 * NOUT;

// forward tile in shared memory: weights + input tile + activation tile + biases
constexpr int FWD_SMEM = 2 * (NH * KIN + NH * NH + NO * NH + TM * KIN + TM * NH) +
                         4 * (NH + NH + NO) + 64;

struct Weights {
  const __nv_bfloat16* packed;  // K_TOTAL
  const float* params;          // P_TOTAL (biases are read from here)
  const float* norm;            // N_NORM
};

}  // namespace mlp

// ---- device helpers shared by the MLP kernels and the stress-update kernel ----------
namespace mlp {

constexpr int MAX_POLLS = 1 << 24;  // mbarrier polls before a wait gives up

__device__ __forceinline__ float silu(float z) { return z / (1.0f + __expf(-z)); }
__device__ __forceinline__ float dsilu(float z) {
  const float s = 1.0f / (1.0f + __expf(-z));
  return s * (1.0f + z * (1.0f - s));
}

// 8 floats -> 8 bf16 (round to nearest even) as one 16-byte word
__device__ __forceinline__ uint4 pack8(const float* v) {
  uint4 q;
  uint32_t* u = reinterpret_cast<uint32_t*>(&q);
#pragma unroll
  for (int i = 0; i < 4; i++) {
    __nv_bfloat162 h = __floats2bfloat162_rn(v[2 * i], v[2 * i + 1]);
    u[i] = *reinterpret_cast<uint32_t*>(&h);
  }
  return q;
}
// row r, columns [k0, k0 + 8) of a K-major tile with K columns
__device__ __forceinline__ void st_row8(unsigned char* tile, int r, int k0, int K, const float* v) {
  *reinterpret_cast<uint4*>(tile + tc::kmaj_off(r, k0, K)) = pack8(v);
}
// element (r, k) of a K-major tile (transposed writes: one value per row)
__device__ __forceinline__ void st_el(unsigned char* tile, int r, int k, int K, float v) {
  *reinterpret_cast<__nv_bfloat16*>(tile + tc::kmaj_off(r, k, K)) = __float2bfloat16_rn(v);
}
// copy n16 16-byte words global -> shared with the whole block
__device__ __forceinline__ void copy16(unsigned char* dst, const void* src, int n16) {
  const uint4* s = reinterpret_cast<const uint4*>(src);
  uint4* d = reinterpret_cast<uint4*>(dst);
  for (int i = threadIdx.x; i < n16; i += blockDim.x) d[i] = s[i];
}

// D = A x B^T over K (K / 16 MMAs) issued by one thread, no commit
__device__ __forceinline__ void gemm_mma(uint32_t d, const unsigned char* A, const unsigned char* B,
                                         int K, int M, int N) {
  tc::fence_after_sync();
  const uint32_t id = tc::idesc_bf16(M, N);
  for (int kk = 0; kk < K / 16; kk++)
    tc::mma_bf16(d, tc::sdesc(A, K, kk), tc::sdesc(B, K, kk), id, kk > 0);
}
// the same followed by a commit: bar completes one phase when every MMA this thread
// issued so far has finished (one commit per wait, so a waiter never falls two phases
// behind)
__device__ __forceinline__ void gemm_issue(uint32_t d, const unsigned char* A, const unsigned char* B,
                                           int K, int M, int N, uint64_t* bar) {
  gemm_mma(d, A, B, K, M, N);
  tc::mma_commit(bar);
}

// every thread: wait for the next completion of bar, then order TMEM reads after it
__device__ __forceinline__ bool gemm_wait(uint64_t* bar, uint32_t* phase) {
  const bool ok = tc::mbar_wait(bar, *phase, MAX_POLLS);
  *phase ^= 1u;
  tc::fence_after_sync();
  return ok;
}

// all threads: make shared-memory operand writes visible to the tensor core, order prior
// TMEM loads before the barrier, synchronise
__device__ __forceinline__ void operands_ready() {
  tc::fence_async_smem();
  tc::fence_before_sync();
  __syncthreads();
}

// Block-level inference on one tile of TM samples (blockDim.x == TM; every thread calls,
// with a dummy sample where it has none): thread r passes its NIN raw features and
// receives NOUT raw outputs.  smem: FWD_SMEM bytes, 16-byte aligned; tmem: base of >= 256
// allocated columns; bar: an initialised mbarrier whose next phase parity is *phase.
// Returns false when a tensor-core wait gave up (out is then undefined).
__device__ __forceinline__ bool forward_tile(const Weights& w, unsigned char* smem, uint32_t tmem,
                                             uint64_t* bar, uint32_t* phase, const float* feat,
                                             float* out) {
  unsigned char* sW1 = smem;
  unsigned char* sW2 = sW1 + 2 * NH * KIN;
  unsigned char* sW3 = sW2 + 2 * NH * NH;
  unsigned char* sX = sW3 + 2 * NO * NH;
  unsigned char* sA = sX + 2 * TM * KIN;
  float* sb = reinterpret_cast<float*>(sA + 2 * TM * NH);  // b1 | b2 | b3
  const int r = threadIdx.x, wq = (threadIdx.x >> 5) & 3;
  copy16(sW1, w.packed + K_W1, NH * KIN / 8);
  copy16(sW2, w.packed + K_W2, NH * NH / 8);
  copy16(sW3, w.packed + K_W3, NO * NH / 8);
  for (int i = threadIdx.x; i < NH; i += blockDim.x) {
    sb[i] = w.params[P_B1 + i];
    sb[NH + i] = w.params[P_B2 + i];
  }
  if (threadIdx.x < NO) sb[2 * NH + threadIdx.x] = w.params[P_B3 + threadIdx.x];
  {  // normalised input row, zero padded to KIN
    float x[KIN];
#pragma unroll
    for (int i = 0; i < KIN; i++) x[i] = i < NIN ? (feat[i] - w.norm[i]) * w.norm[NIN + i] : 0.0f;
#pragma unroll
    for (int k = 0; k < KIN; k += 8) st_row8(sX, r, k, KIN, x + k);
  }
  operands_ready();
  bool ok = true;
  // layer 1: TMEM columns [0, 128)
  if (threadIdx.x == 0) gemm_issue(tmem, sX, sW1, KIN, TM, NH, bar);
  ok &= gemm_wait(bar, phase);
  for (int c = 0; c < NH; c += 16) {
    float v[16];
    tc::tmem_ld16(tc::taddr(tmem, 32 * wq, c), v);
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = silu(v[i] + sb[c + i]);
    st_row8(sA, r, c, NH, v);
    st_row8(sA, r, c + 8, NH, v + 8);
  }
  operands_ready();
  // layer 2: TMEM columns [128, 256)
  if (threadIdx.x == 0) gemm_issue(tmem + NH, sA, sW2, NH, TM, NH, bar);
  ok &= gemm_wait(bar, phase);
  for (int c = 0; c < NH; c += 16) {
    float v[16];
    tc::tmem_ld16(tc::taddr(tmem, 32 * wq, NH + c), v);
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = silu(v[i] + sb[NH + c + i]);
    st_row8(sA, r, c, NH, v);
    st_row8(sA, r, c + 8, NH, v + 8);
  }
  operands_ready();
  // layer 3: TMEM columns [0, 16)
  if (threadIdx.x == 0) gemm_issue(tmem, sA, sW3, NH, TM, NO, bar);
  ok &= gemm_wait(bar, phase);
  {
    float v[16];
    tc::tmem_ld16(tc::taddr(tmem, 32 * wq, 0), v);
#pragma unroll
    for (int o = 0; o < NOUT; o++)
      out[o] = (v[o] + sb[2 * NH + o]) * w.norm[2 * NIN + NOUT + o] + w.norm[2 * NIN + o];
  }
  tc::fence_before_sync();
  __syncthreads();  // the block's smem and TMEM may be reused after this
  return ok;
}

// TMEM allocation of a block: warp 0 allocates ncols, every thread gets the base
__device__ __forceinline__ uint32_t tmem_block_alloc(uint32_t* slot, uint32_t ncols) {
  if ((threadIdx.x >> 5) == 0) {
    tc::tmem_alloc(slot, ncols);
    tc::tmem_relinquish();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  return *slot;
}
__device__ __forceinline__ void tmem_block_free(uint32_t base, uint32_t ncols) {
  tc::fence_before_sync();
  __syncthreads();
  if ((threadIdx.x >> 5) == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(base, ncols);
  }
}

}  // namespace mlp
