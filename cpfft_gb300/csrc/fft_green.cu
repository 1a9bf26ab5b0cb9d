// fft_green.cu -- y = G(K : x) or y = G(x) on the GPU: a hand-written real-to-complex
// 3-D FFT of the 9 tensor components fused with the spectral Green operator.
//
// Replaces G_K_dF / fftfem3d / ifftfem3d / ddot42n (src/G_K_dF.f:11-268), which run 18
// complex 3-D MKL transforms per call on real data and read an 81-wide stored Green
// table (src/FFT_init.f:272-340).  Here:
//   pass A  K:x fused into a real-to-complex transform along the fastest axis (two real
//           lines packed into one complex transform);
//   pass B  complex transform along the middle axis, tiles of columns in shared memory;
//   pass C  transform along the slowest axis, Green contraction evaluated from q on the
//           fly for all 9 components while they sit in shared memory, inverse transform
//           along the same axis -- the spectrum never round-trips HBM between the
//           transform and the contraction;
//   pass D  inverse along the middle axis;
//   pass E  complex-to-real inverse along the fastest axis, unpacking the line pairs.
// The reference's result is Re(IDFT(Ghat(q(f)) X(f))); for real input that equals
// IDFT(Hs(f) X(f)) with Hs(f) = (Ghat(q(f)) + Ghat(q(-f)))/2, which keeps the half
// spectrum Hermitian and is what pass C applies, for both frequency mappings.
#include "green_passes.cuh"


FftPlan make_plan(int N) {
  FftPlan p;
  p.n = N;
  p.nst = 0;
  int m = N, Ns = 1;
  auto push = [&](int r) {
    p.R[p.nst] = r;
    p.Ns[p.nst] = Ns;
    Ns *= r;
    p.nst++;
    m /= r;
  };
  while (m % 8 == 0) push(8);
  while (m % 4 == 0) push(4);
  while (m % 2 == 0) push(2);
  for (int f = 3; m > 1; f += 2)
    while (m % f == 0) push(f);
  return p;
}

template <typename T>
cudaError_t green_setup(int N) {
  cudaError_t e;
  // power-of-two grids take the register-FFT passes (FP64 too: 3.72 against 3.98 ms for
  // the shared-memory Stockham passes at 128^3, measured on a GB300)
  {
    switch (N) {
      case 32: return wgreen_setup<1, T>();
      case 64: return wgreen_setup<2, T>();
      case 128: return wgreen_setup<4, T>();
      case 256: return wgreen_setup<8, T>();
      default: break;
    }
  }
  size_t a = smem_a<T>(N), b = smem_b<T>(N, 16), c = smem_c<T>(N, tile_c<T>());
  // the shared-memory passes serve every N: the attribute only ever grows, so contexts of
  // different grids (concurrent ones included) never lower it under each other
  if ((e = raise_max_dynamic_smem((const void*)pass_a<T, T>, a))) return e;
  if ((e = raise_max_dynamic_smem((const void*)pass_b<T>, b))) return e;
  if ((e = raise_max_dynamic_smem((const void*)pass_c<T>, c))) return e;
  if ((e = raise_max_dynamic_smem((const void*)pass_e<T>, a))) return e;
  return cudaSuccess;
}

template <typename T>
cudaError_t green_apply_dot(const T* x, const T* K4, int flgK, T* y, typename Vec2<T>::t* S,
                            const typename Vec2<T>::t* tw, GridDesc g, cudaStream_t st,
                            double* part, int* nparts, const T* rfuse, double* scf) {
  const int N = g.N, H = g.H;
  bool warp_path = false;
  if (nparts) *nparts = 0;
  if (rfuse && !flgK) return cudaErrorInvalidValue;  // the fused update serves G(K : p) only
  {
    warp_path = true;
    switch (N) {
      case 32: wgreen_apply<1, T>(x, K4, nullptr, flgK, y, S, tw, g, st, part, rfuse, scf); break;
      case 64: wgreen_apply<2, T>(x, K4, nullptr, flgK, y, S, tw, g, st, part, rfuse, scf); break;
      case 128: wgreen_apply<4, T>(x, K4, nullptr, flgK, y, S, tw, g, st, part, rfuse, scf); break;
      case 256: wgreen_apply<8, T>(x, K4, nullptr, flgK, y, S, tw, g, st, part, rfuse, scf); break;
      default: warp_path = false;
    }
  }
  if (rfuse && !warp_path) return cudaErrorNotSupported;  // the fused update needs the warp passes
  if (warp_path) {
    if (part && nparts) *nparts = (N / 2) * N;
    g_kernel_launches += 5;
    return cudaGetLastError();
  }
  g.tkb = 16;
  g.tkc = tile_c<T>();
  const int npair = (N + 1) / 2;
  // the reference-medium operator's product <K : x, x> is summed in pass A; the plain
  // operator's <x, y> is left to the caller on this path
  double* part_a = (g.pre && part && flgK) ? part : nullptr;
  if (part_a && nparts) *nparts = npair * N;
  pass_a<T, T><<<npair * N, 256, smem_a<T>(N), st>>>(x, K4, flgK, S, g, tw, part_a);
  dim3 gb((H + g.tkb - 1) / g.tkb, N, 9);
  pass_b<T><<<gb, 256, smem_b<T>(N, g.tkb), st>>>(S, g, tw, 0);
  dim3 gc((H + g.tkc - 1) / g.tkc, N);
  pass_c<T><<<gc, 256, smem_c<T>(N, g.tkc), st>>>(S, g, tw);
  pass_b<T><<<gb, 256, smem_b<T>(N, g.tkb), st>>>(S, g, tw, 1);
  pass_e<T><<<npair * N, 256, smem_a<T>(N), st>>>(S, y, g, tw);
  g_kernel_launches += 5;
  return cudaGetLastError();
}

template <typename T>
cudaError_t green_apply(const T* x, const T* K4, int flgK, T* y, typename Vec2<T>::t* S,
                        const typename Vec2<T>::t* tw, GridDesc g, cudaStream_t st) {
  return green_apply_dot<T>(x, K4, flgK, y, S, tw, g, st, nullptr, nullptr, nullptr, nullptr);
}

cudaError_t green_cg_iteration(float* x, float* r, float* p, const float* K4, float2* S,
                               const float2* tw, const GridDesc& g, cudaStream_t st,
                               double* part_a, double* part_e, const float* k0, double* sc) {
  switch (g.N) {
    case 32: wcg_iteration<1>(x, r, p, K4, S, tw, g, st, part_a, part_e, k0, sc); break;
    case 64: wcg_iteration<2>(x, r, p, K4, S, tw, g, st, part_a, part_e, k0, sc); break;
    case 128: wcg_iteration<4>(x, r, p, K4, S, tw, g, st, part_a, part_e, k0, sc); break;
    case 256: wcg_iteration<8>(x, r, p, K4, S, tw, g, st, part_a, part_e, k0, sc); break;
    default: return cudaErrorNotSupported;
  }
  g_kernel_launches += 5;  // the transform passes (dev_final counts its own launch)
  return cudaGetLastError();
}

cudaError_t green_autotune_f32(const float* x, const float* K4, float* y, float2* S,
                               const float2* tw, GridDesc* g, cudaStream_t st, float* best_ms) {
  if (!green_df_supported(g->N)) return cudaSuccess;
  GridDesc t = *g;
  cudaError_t e = tune_tiles(t, [&](const GridDesc& gg) {
    green_apply_dot<float>(x, K4, 1, y, S, tw, gg, st, nullptr, nullptr, nullptr, nullptr);
  }, st, best_ms, true);
  if (e == cudaSuccess) { g->wtb = t.wtb; g->wtc = t.wtc; g->wc2 = t.wc2; }
  return e;
}


template cudaError_t green_setup<double>(int);
template cudaError_t green_setup<float>(int);
template cudaError_t green_apply<double>(const double*, const double*, int, double*, double2*,
                                         const double2*, GridDesc, cudaStream_t);
template cudaError_t green_apply<float>(const float*, const float*, int, float*, float2*,
                                        const float2*, GridDesc, cudaStream_t);
template cudaError_t green_apply_dot<float>(const float*, const float*, int, float*, float2*,
                                            const float2*, GridDesc, cudaStream_t, double*, int*,
                                            const float*, double*);
