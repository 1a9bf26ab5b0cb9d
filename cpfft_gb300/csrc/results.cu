// results.cu -- the element result files of ouresult (src/ouresult.f:140-330) formatted on
// the GPU: one text line per voxel, every value in the Fortran edit descriptor E15.6 of
// `write(fid, '(30e15.6)')` (oupestr, src/ouresult.f:271-300), e.g. "   0.123456E+03".
//
// Each line has a fixed width (values x 15 + newline), so a line's place in the file is
// known from its voxel index and every field is written by its own thread.  A value's
// six digits are the decimal value rounded to nearest, ties to even, computed exactly
// with 128-bit integer arithmetic: v = M 2^E (M the 53-bit significand) times 10^k, with
// the remainder deciding the rounding.  The few values whose exact product does not fit
// 128 bits (magnitudes below about 1e-17) are flagged and formatted on the host.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "common.cuh"

namespace {

constexpr int FW = 15;  // field width of E15.6

__device__ __forceinline__ unsigned __int128 pow10_u128(int k) {  // k <= 38
  unsigned __int128 p = 1;
  for (int i = 0; i < k; i++) p *= 10u;
  return p;
}

// round_half_even(a * 10^k) for a = M 2^E2 > 0; false when it does not fit the exact path
__device__ bool scaled_round(unsigned long long M, int E2, int k, unsigned long long* m) {
  typedef unsigned __int128 u128;
  if (k >= 0) {
    if (k > 22 || E2 >= 0) return false;  // M 10^k must fit 128 bits; a >= 2^52 never gets here
    const u128 num = (u128)M * pow10_u128(k);
    const int sh = -E2;
    if (sh >= 128) return false;
    const u128 q = num >> sh;
    const u128 r = num - (q << sh);
    const u128 half = (u128)1 << (sh - 1);
    u128 qq = q;
    if (r > half || (r == half && (q & 1))) qq += 1;
    if (qq >> 64) return false;
    *m = (unsigned long long)qq;
    return true;
  }
  const int kk = -k;
  if (kk > 38) return false;
  const u128 den10 = pow10_u128(kk);
  u128 num, den;
  if (E2 >= 0) {
    if (E2 > 74) return false;
    num = (u128)M << E2;
    den = den10;
  } else {
    if (-E2 >= 127) return false;
    const u128 d2 = (u128)1 << (-E2);
    if (den10 > (~(u128)0) / d2) return false;
    num = (u128)M;
    den = den10 * d2;
  }
  const u128 q = num / den, r = num - q * den;
  u128 qq = q;
  const u128 twice = r << 1;  // r < den < 2^127
  if (twice > den || (twice == den && (q & 1))) qq += 1;
  if (qq >> 64) return false;
  *m = (unsigned long long)qq;
  return true;
}

// Fortran E15.6 of v into out[0..14]; false: format this value on the host instead
__device__ bool fmt_e15(double v, char* out) {
  for (int i = 0; i < FW; i++) out[i] = ' ';
  if (v == 0.0) {
    const char z[] = "0.000000E+00";
    for (int i = 0; i < 12; i++) out[3 + i] = z[i];
    return true;
  }
  if (!isfinite(v)) return false;
  const bool neg = v < 0.0;
  const double a = fabs(v);
  int ex2;
  const double fr = frexp(a, &ex2);                        // a = fr 2^ex2, fr in [0.5, 1)
  const unsigned long long M = (unsigned long long)ldexp(fr, 53);  // exact
  const int E2 = ex2 - 53;
  int e = (int)floor(log10(a)) + 1;                        // a = 0.d1d2... 10^e (estimate)
  unsigned long long m = 0;
  bool ok = false;
  for (int t = 0; t < 3; t++) {
    if (!scaled_round(M, E2, 6 - e, &m)) return false;
    if (m >= 1000000ull) { e++; continue; }
    if (m < 100000ull) { e--; continue; }
    ok = true;
    break;
  }
  if (!ok) return false;
  const int ae = e < 0 ? -e : e;
  if (ae > 999) return false;
  char s[FW];
  int n = 0;
  if (neg) s[n++] = '-';
  s[n++] = '0';
  s[n++] = '.';
  for (int i = 5; i >= 0; i--) {
    s[n + i] = (char)('0' + (int)(m % 10ull));
    m /= 10ull;
  }
  n += 6;
  if (ae <= 99) {  // E+dd
    s[n++] = 'E';
    s[n++] = e < 0 ? '-' : '+';
    s[n++] = (char)('0' + ae / 10);
    s[n++] = (char)('0' + ae % 10);
  } else {         // +ddd (the Fortran form for three-digit exponents)
    s[n++] = e < 0 ? '-' : '+';
    s[n++] = (char)('0' + ae / 100);
    s[n++] = (char)('0' + (ae / 10) % 10);
    s[n++] = (char)('0' + ae % 10);
  }
  for (int i = 0; i < n; i++) out[FW - n + i] = s[i];
  return true;
}

// one thread per field of the element lines: quantity 2 = stresses (the unrotated Cauchy
// stress, 26 values a line), 1 = strains (the unrotated strain, 22 values a line); the
// values past the six components are the reference's zero-initialised columns
__global__ void k_format_flat(const double* __restrict__ hist, long long N3, int word0,
                              int nvals, char* __restrict__ text,
                              unsigned char* __restrict__ flags) {
  const long long L = (long long)nvals * FW + 1;
  const long long total = N3 * nvals;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const long long v = t / nvals;
    const int j = (int)(t - v * nvals);
    double x = 0.0;
    if (j < 6) {
      x = hist[(word0 + j) * N3 + v];
      if (fabs(x) < 1.0e-30) x = 0.0;  // oupestr's small_tol
    }
    char* f = text + v * L + (long long)j * FW;
    const bool ok = fmt_e15(x, f);
    if (j < 6) flags[v * 6 + j] = ok ? 0 : 1;
    if (j == nvals - 1) f[FW] = '\n';
  }
}

__global__ void k_format_values(const double* __restrict__ x, long long n, char* __restrict__ out,
                                unsigned char* __restrict__ flags) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    flags[i] = fmt_e15(x[i], out + i * FW) ? 0 : 1;
}

}  // namespace

// Host formatting of one E15.6 field (the values the device path flags): the C library's
// correctly rounded "%.5e" digits moved into the Fortran 0.dddddd form.
void host_e15(double v, char* out) {
  char buf[40];
  memset(out, ' ', FW);
  if (v == 0.0) {
    memcpy(out + 3, "0.000000E+00", 12);
    return;
  }
  snprintf(buf, sizeof(buf), "%.5e", fabs(v));  // d.ddddde[+-]XX[X]
  const int e = atoi(buf + 8) + 1;
  const int ae = e < 0 ? -e : e;
  char s[24];
  int n = 0;
  if (v < 0) s[n++] = '-';
  s[n++] = '0';
  s[n++] = '.';
  s[n++] = buf[0];
  for (int i = 2; i < 7; i++) s[n++] = buf[i];
  if (ae <= 99) n += snprintf(s + n, sizeof(s) - n, "E%c%02d", e < 0 ? '-' : '+', ae);
  else n += snprintf(s + n, sizeof(s) - n, "%c%03d", e < 0 ? '-' : '+', ae);
  if (n > FW) n = FW;
  memcpy(out + FW - n, s, n);
}

cudaError_t launch_format_flat(const double* hist, long long N3, int word0, int nvals, char* text,
                               unsigned char* flags, cudaStream_t st) {
  const long long total = N3 * nvals;
  const int blocks = (int)std::min<long long>((total + 255) / 256, 65535);
  k_format_flat<<<blocks, 256, 0, st>>>(hist, N3, word0, nvals, text, flags);
  g_kernel_launches += 1;
  return cudaGetLastError();
}

cudaError_t launch_format_values(const double* x, long long n, char* out, unsigned char* flags,
                                 cudaStream_t st) {
  const int blocks = (int)std::min<long long>((n + 255) / 256, 65535);
  k_format_values<<<blocks, 256, 0, st>>>(x, n, out, flags);
  g_kernel_launches += 1;
  return cudaGetLastError();
}
