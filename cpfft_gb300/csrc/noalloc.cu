// noalloc.cu -- G(K4 : x) for callers that cannot allocate device memory.
//
// Some host programs cannot call cudaMalloc once they are running: applications that
// hand all device memory to their own pool allocator at start-up, or that run under a
// fixed device-memory budget after initialisation.  cpfft_green_apply needs the
// library context (cpfft_init allocates the fields and the spectral scratch).  This
// entry point instead takes the caller's device buffers for its inputs and output and
// keeps its scratch -- the half spectrum of the 9 components and the twiddle table --
// in one file-scope __device__ array below, so the call itself allocates nothing.
//
// Limits and rules:
//  * grids up to NOALLOC_MAX_N = 32 points per axis (the array holds 2.5 MB, which
//    every GPU that loads the library keeps until the process exits);
//  * the first call on a device looks up the array's device address for that device
//    (cudaGetSymbolAddress with that device current); make that first call before any
//    stream capture;
//  * every call shares the one array, so calls that overlap on the GPU (different
//    streams, or different host threads on the same device) race; serialise them;
//  * nothing in the array has to start at zero: each call rewrites the twiddles for its
//    N and writes every spectral entry before reading it.
#include <atomic>

#include "fft_green.cuh"

namespace {

constexpr int NOALLOC_MAX_N = 32;
constexpr size_t NOALLOC_SPEC = (size_t)9 * NOALLOC_MAX_N * NOALLOC_MAX_N * (NOALLOC_MAX_N / 2 + 1);
constexpr size_t NOALLOC_WORDS = NOALLOC_SPEC + NOALLOC_MAX_N;  // spectrum + twiddles

// In host code this name is only a stand-in: the device address comes from
// cudaGetSymbolAddress in scratch_for_current_device().
static __device__ __align__(256) double2 g_noalloc_scratch[NOALLOC_WORDS];

// the array's device address per device, looked up once; host threads may race on the
// first lookup, and each stores the same value
constexpr int MAX_DEVICES = 64;
std::atomic<double2*> g_scratch_addr[MAX_DEVICES];

__global__ void k_twiddles(double2* tw, int N) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < N) {
    double s, c;
    sincospi(-2.0 * (double)k / (double)N, &s, &c);
    tw[k] = make_double2(c, s);
  }
}

int scratch_for_current_device(double2** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) {
    cpfft_set_error("green_apply_noalloc: no usable current device (%s)",
                    e != cudaSuccess ? cudaGetErrorString(e) : "device index out of range");
    return CPFFT_ERR_CUDA;
  }
  double2* addr = g_scratch_addr[dev].load(std::memory_order_acquire);
  if (!addr) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      cpfft_set_error("green_apply_noalloc: cudaGetSymbolAddress failed on device %d: %s", dev,
                      cudaGetErrorString(e));
      return CPFFT_ERR_CUDA;
    }
    addr = static_cast<double2*>(p);
    g_scratch_addr[dev].store(addr, std::memory_order_release);
  }
  *out = addr;
  return 0;
}

}  // namespace

extern "C" int cpfft_green_apply_noalloc(int N, int g_mapping, const double* x,
                                         const double* K4, int flgK, double* y,
                                         void* stream) {
  if (N < 2 || N > NOALLOC_MAX_N) {
    cpfft_set_error("green_apply_noalloc: N = %d outside [2, %d] (the static scratch holds "
                    "grids up to %d^3)", N, NOALLOC_MAX_N, NOALLOC_MAX_N);
    return CPFFT_ERR_BAD_ARG;
  }
  if (!x || !y || (flgK && !K4) ||
      (g_mapping != CPFFT_G_REF_SHIFT && g_mapping != CPFFT_G_CENTERED)) {
    cpfft_set_error("green_apply_noalloc: null pointer or unknown mapping");
    return CPFFT_ERR_BAD_ARG;
  }
  double2* scratch = nullptr;
  int rc = scratch_for_current_device(&scratch);
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  GridDesc g;
  g.N = N;
  g.H = N / 2 + 1;
  g.N3 = (long long)N * N * N;
  g.Nhalf = (N % 2 == 1) ? (N + 1) / 2 : N / 2 + 1;
  g.gmap = g_mapping;
  g.inv_n3 = 1.0 / (double)g.N3;
  g.tkb = 16;
  g.tkc = 2;
  g.plan = make_plan(N);
  double2* S = scratch;
  double2* tw = scratch + NOALLOC_SPEC;
  k_twiddles<<<1, NOALLOC_MAX_N, 0, st>>>(tw, N);
  g_kernel_launches += 1;
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = green_apply<double>(x, K4, flgK ? 1 : 0, y, S, tw, g, st);
  if (e != cudaSuccess) {
    cpfft_set_error("green_apply_noalloc: %s", cudaGetErrorString(e));
    return CPFFT_ERR_CUDA;
  }
  return 0;
}
