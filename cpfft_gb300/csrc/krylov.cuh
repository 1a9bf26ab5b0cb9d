// krylov.cuh -- device vector operations for the Newton-Krylov loop.
#pragma once
#include "common.cuh"

constexpr int NPART = 1024;  // partial sums per reduction (blocks of the first pass)

// device scalar slots
enum {
  SC_RR = 0, SC_PAP = 1, SC_RRNEW = 2, SC_ALPHA = 3, SC_BETA = 4, SC_TMP = 5,
  SC_T1 = 6, SC_T2 = 7,  // scratch read back with others in one transfer
  SC_SUM9 = 8,     // 9 slots: component sums
  // stop test of a device-driven CG segment (k_cg_cond): <r,r> at the segment start,
  // the true residual norm there, the reference's absolute thresholds, the segment's
  // reduction target, the iteration counter and cap, and the reason the segment ended
  SC_RR0 = 17, SC_RN = 18, SC_TOLB = 19, SC_TOL = 20, SC_DELTA = 21,
  SC_CNT = 22, SC_MAXIT = 23, SC_STOP = 24,
  SC_COUNT = 32
};
// SC_STOP values
enum { STOP_NONE = 0, STOP_TEST = 1, STOP_MAXIT = 2, STOP_NONFINITE = 3 };
enum { OP_STORE = 0, OP_ALPHA = 1, OP_BETA = 2 };

cudaError_t dev_dot(const double* a, const double* b, long long n, double* part, double* sc,
                    int slot, int op, cudaStream_t st);
cudaError_t dev_dot_f(const float* a, const float* b, long long n, double* part, double* sc,
                      int slot, int op, cudaStream_t st);
template <typename T>
cudaError_t dev_cg_xr(T* x, T* r, const T* p, const T* Ap, long long n, double* part, double* sc,
                      cudaStream_t st);
template <typename T>
cudaError_t dev_cg_p(T* p, const T* r, long long n, double* sc, cudaStream_t st);
// sc[slot] = sum of np partials (with the op's CG follow-up)
cudaError_t dev_final(double* part, int np, double* sc, int slot, int op, cudaStream_t st);
cudaError_t dev_axpy(double* y, const double* x, double a, long long n, cudaStream_t st);
cudaError_t dev_scale(double* y, double a, long long n, cudaStream_t st);
cudaError_t dev_sub(double* y, const double* a, const double* b, long long n, cudaStream_t st);
cudaError_t dev_scale_f(float* y, float a, long long n, cudaStream_t st);
cudaError_t dev_fill9(double* y, long long N3, const double* v, cudaStream_t st);
cudaError_t dev_add_const(double* y, double v, long long n, cudaStream_t st);
cudaError_t dev_to_f32(float* y, const double* x, double s, long long n, cudaStream_t st);
cudaError_t dev_add_f32(double* y, const float* x, double s, long long n, cudaStream_t st);
cudaError_t dev_sum9(const double* x, long long N3, double* part, double* sc, int slot0,
                     cudaStream_t st);

// Reference-medium preconditioned FP32 CG: the inner product <a, b>_K0 uses the 9x9
// matrix k0 (device memory, row-major, (ij) index 3i+j).
// x += alpha p, r -= alpha Ap, sc[SC_RRNEW] = <r, r>_K0 and beta (fields (9, N3) FP32)
cudaError_t dev_cg_xr_k0(float* x, float* r, const float* p, const float* Ap, long long N3,
                         const float* k0, double* part, double* sc, cudaStream_t st);
cudaError_t dev_dot_k0(const float* a, const float* b, long long N3, const float* k0,
                       double* part, double* sc, int slot, int op, cudaStream_t st);
// sc81[m] = sum over voxels of component m of an (81, N3) FP32 field (part: 81 x 64)
cudaError_t dev_mean81(const float* K, long long N3, double* part, double* sc81, cudaStream_t st);

// End-of-iteration test of a preconditioned FP32 CG segment (one thread): counts the
// iteration and stops when the K0 norm of the residual has dropped by SC_DELTA since the
// segment began, when the true residual it predicts meets the reference's test, at the
// cap SC_MAXIT, or on a non-finite value.  With use_handle it drives the WHILE node of
// the captured iteration graph (cudaGraphSetConditional); the counter bounds that loop.
cudaError_t dev_cg_cond(double* sc, cudaGraphConditionalHandle h, bool use_handle,
                        cudaStream_t st);
// the graph's gate: its WHILE node runs while sc[SC_STOP] is STOP_NONE
cudaError_t dev_cg_gate(const double* sc, cudaGraphConditionalHandle h, cudaStream_t st);
