// fft_green.cuh -- declarations of the fused FFT + Green-operator passes.
#pragma once
#include "common.cuh"
#include "dfloat.cuh"

template <typename T> struct Vec2;
template <> struct Vec2<double> { typedef double2 t; };
template <> struct Vec2<float> { typedef float2 t; };
template <> struct Vec2<dfl> { typedef dfl2 t; };

// Mixed-radix factorisation N = prod R[s]; Ns[s] = prod of the radices before stage s.
struct FftPlan {
  int n, nst;
  int R[16];
  int Ns[16];
};

struct GridDesc {
  int N, H;          // points per axis, half-spectrum length N/2+1
  long long N3;
  int Nhalf, gmap;   // reference Nhalf (src/FFT_init.f:146-147) and the q mapping
  double inv_n3;     // backward scale 1/N^3
  int tkb, tkc;      // columns per block in passes B and C
  int pre = 0;       // FP32 passes: 1 = reference-medium operator with coefficients acoef
  const float* acoef = nullptr;  // (36, device) acoustic-tensor coefficients of the medium
  int wtb = 16, wtc = 0;  // warp passes: columns per block of passes B/D and of pass C (0: 4 for
                          // FP32, 2 for double-float)
  int wc2 = 0;            // FP32 warp passes: pass C in registers (wpass_c2) with this many
                          // columns per block (0: the shared-memory pass C)
  FftPlan plan;
};

FftPlan make_plan(int N);

// Shared-memory columns are padded: element k of a column sits at pidx(k) = k + k/8 and
// columns are padlen(N) apart.  The transforms access columns with power-of-two strides;
// the padding spreads those strides across the 32 banks.
__host__ __device__ __forceinline__ int pidx(int k) { return k + (k >> 3); }
__host__ __device__ __forceinline__ int padlen(int N) { return N + (N >> 3) + 1; }

// y = G(K4 : x) (flgK = 1) or y = G(x); S is the spectral scratch (9 * N * N * H complex),
// tw the length-N forward twiddle table.  All on stream st.
template <typename T>
cudaError_t green_apply(const T* x, const T* K4, int flgK, T* y, typename Vec2<T>::t* S,
                        const typename Vec2<T>::t* tw, GridDesc g, cudaStream_t st);
// the same, and with part != nullptr also the partial sums of x . y: *nparts partials
// in part (the warp-FFT sizes), or *nparts = 0 when this size does not fuse the product
// (the caller then reduces x . y itself).  rfuse != nullptr (FP32 warp-FFT sizes only,
// else cudaErrorNotSupported): x is the CG direction p, first updated in place to
// r + beta p (r = rfuse, beta = scf[SC_BETA]; scf[SC_RR] takes scf[SC_RRNEW])
template <typename T>
cudaError_t green_apply_dot(const T* x, const T* K4, int flgK, T* y, typename Vec2<T>::t* S,
                            const typename Vec2<T>::t* tw, GridDesc g, cudaStream_t st,
                            double* part, int* nparts, const T* rfuse = nullptr,
                            double* scf = nullptr);
template <typename T>
cudaError_t green_setup(int N);

// Reference medium of the preconditioned FP32 operator (GridDesc::pre = 1, acoef): the 36
// coefficients of the acoustic tensor A0(q)_ik = sum_jl K0_ijkl q_j q_l, six unique
// (i <= k) rows over the six products q_0q_0, q_1q_1, q_2q_2, q_0q_1, q_1q_2, q_0q_2.
// With pre = 1 pass C applies Ghat0(q) X = (A0(q)^-1 X q) (x) q in place of
// (X q) (x) q / |q|^2, and the fused product of green_apply_dot is <K : x, x>, summed in
// pass A, in place of <x, y>.

// FP64-accurate y = G(K : x) (flgK = 1) or G(x) in double-float arithmetic on the FP32
// pipes, for the power-of-two grids 32..256 of the warp-FFT passes (green_df_supported).
// x, y are FP64 fields; K is given as the float pair K4hi + K4lo (the FP64 tangent to 48
// bits); S is the FP64 spectral scratch (double-float complex values are 16 bytes too);
// tw the double-float twiddle table.  Relative error about 1e-13 against the FP64
// operator, from about a fifth of its time.
// One preconditioned FP32 CG iteration on the register-FFT grids (32..256), g.pre set:
// p = r + beta p, y = G0(K : p) with alpha = rr / <K : p, p>, x += alpha p,
// r -= alpha y, part_e = the (N/2) N block partials of <r, r>_K0 (k0: the 9 x 9 weights);
// y never reaches memory.  The caller finishes rr_new / beta and the stop test.
cudaError_t green_cg_iteration(float* x, float* r, float* p, const float* K4, float2* S,
                               const float2* tw, const GridDesc& g, cudaStream_t st,
                               double* part_a, double* part_e, const float* k0, double* sc);

bool green_df_supported(int N);
cudaError_t green_setup_df(int N);
cudaError_t green_apply_df(const double* x, const float* K4hi, const float* K4lo, int flgK,
                           double* y, dfl2* S, const dfl2* tw, GridDesc g, cudaStream_t st);

// Autotuner of the warp passes' tile shapes: times every candidate (columns per block of
// passes B/D in {8, 16, 32} x of pass C in {2, 4}) on the given buffers with CUDA events
// and stores the fastest in g->wtb / g->wtc (best_ms: its time per apply).  The buffers'
// contents are overwritten (y, S).  No-op for sizes without warp passes.
cudaError_t green_autotune_f32(const float* x, const float* K4, float* y, float2* S,
                               const float2* tw, GridDesc* g, cudaStream_t st, float* best_ms);
cudaError_t green_autotune_df(const double* x, const float* K4hi, const float* K4lo, double* y,
                              dfl2* S, const dfl2* tw, GridDesc* g, cudaStream_t st, float* best_ms);
