// disp.cu -- nodal displacements from the deformation gradient field: replaces f2disp
// (src/f2disp.f:16-135) with form_BTB (:136-400) and its PARDISO solve.
//
// The reference fits nodal positions x on the (N+1)^3 node mesh of the voxel grid (the
// hexahedral elements of oumodel's blkgen, src/oumodel.f:178-330) to F in the least-squares
// sense: (sum_e int B^T B) x = sum_e B^T F_e, B the gradient of the trilinear shape
// functions, the left side integrated with 2x2x2 Gauss points, the right side with one,
// node 1 held at the origin; u = x - X.  On the regular grid the left-side operator is the
// tensor product K(x)M(x)M + M(x)K(x)M + M(x)M(x)K of the 1-D linear-element stiffness K
// and consistent mass M (2-point Gauss integrates them exactly), which the DCT-I
// diagonalises: K v_k = lambda_K(k) W v_k, M v_k = lambda_M(k) W v_k with v_k(i) =
// cos(pi k i / N), W = diag(1/2, 1, .., 1, 1/2), lambda_K = (2/h)(1 - cos(pi k/N)),
// lambda_M = (h/3)(2 + cos(pi k/N)).  The pinned problem is the pure-Neumann one with node
// 1's equation replaced by the reaction that makes it compatible, shifted so that node 1
// stays at the origin.  So the solve is exact and direct: three separable DCT-I passes,
// a diagonal scaling, three more passes -- no sparse factorisation.
//
// Layouts: voxel v = a + N b + N^2 c with c along X (direction 1), b along Y, a along Z
// (the reference's element order, z fastest, src/oumodel.f:612-700); node n = i + (N+1) j
// + (N+1)^2 k with i along X (src/oumodel.f:855-900).  Nodal fields are (3, nodes).
#include <algorithm>

#include "common.cuh"

namespace {

// b: sum over the elements around each node of vol grad N_a(centre) . F_e (one-point
// rule), with node 0's entry replaced by minus the sum of all others (compatibility)
__global__ void k_disp_rhs(const double* __restrict__ F, int N, double hx, double hy, double hz,
                           double* __restrict__ b) {
  const long long N1 = N + 1, nodes = N1 * N1 * N1, N3 = (long long)N * N * N;
  const double vol = hx * hy * hz;
  const double cx = vol / (4.0 * hx), cy = vol / (4.0 * hy), cz = vol / (4.0 * hz);
  for (long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x; n < nodes;
       n += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(n % N1), j = (int)((n / N1) % N1), k = (int)(n / (N1 * N1));
    double s[3] = {0.0, 0.0, 0.0};
    for (int di = -1; di <= 0; di++)
      for (int dj = -1; dj <= 0; dj++)
        for (int dk = -1; dk <= 0; dk++) {
          const int ei = i + di, ej = j + dj, ek = k + dk;  // element's lowest corner
          if (ei < 0 || ej < 0 || ek < 0 || ei >= N || ej >= N || ek >= N) continue;
          // this node's local coordinates in that element: -1 at its lower face, +1 upper
          const double xi = di == 0 ? -1.0 : 1.0, eta = dj == 0 ? -1.0 : 1.0,
                       zeta = dk == 0 ? -1.0 : 1.0;
          const long long v = ek + (long long)N * ej + (long long)N * N * ei;  // a=z, b=y, c=x
          for (int r = 0; r < 3; r++)  // component r of x: F_r1, F_r2, F_r3 at (3r..3r+2)
            s[r] += xi * cx * F[(3 * r + 0) * N3 + v] + eta * cy * F[(3 * r + 1) * N3 + v] +
                    zeta * cz * F[(3 * r + 2) * N3 + v];
        }
    for (int r = 0; r < 3; r++) b[r * nodes + n] = s[r];
  }
}

// DCT-I along one axis of a (3, N1, N1, N1) nodal field: out[.., k, ..] = sum_i
// cos(pi k i / N) in[.., i, ..]; stride of the axis in nodes
__global__ void k_dct1_axis(const double* __restrict__ in, double* __restrict__ out, int N,
                            long long stride, const double* __restrict__ ctab) {
  const long long N1 = N + 1, nodes = N1 * N1 * N1;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < 3 * nodes;
       t += (long long)gridDim.x * blockDim.x) {
    const long long r = t / nodes, n = t - r * nodes;
    const int k = (int)((n / stride) % N1);
    const long long base = r * nodes + n - (long long)k * stride;
    const double* row = ctab + (long long)k * N1;
    double s = 0.0;
    for (int i = 0; i <= N; i++) s += row[i] * in[base + i * stride];
    out[t] = s;
  }
}

// z_hat = (2/N)^3 W3 b_hat / Lambda, mode (0,0,0) set to zero
__global__ void k_disp_scale(double* __restrict__ z, int N, double hx, double hy, double hz) {
  const long long N1 = N + 1, nodes = N1 * N1 * N1;
  const double pi = 3.14159265358979323846;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < 3 * nodes;
       t += (long long)gridDim.x * blockDim.x) {
    const long long n = t % nodes;
    const int k1 = (int)(n % N1), k2 = (int)((n / N1) % N1), k3 = (int)(n / (N1 * N1));
    if (k1 == 0 && k2 == 0 && k3 == 0) { z[t] = 0.0; continue; }
    const double c1 = cos(pi * k1 / N), c2 = cos(pi * k2 / N), c3 = cos(pi * k3 / N);
    const double K1 = 2.0 / hx * (1.0 - c1), K2 = 2.0 / hy * (1.0 - c2), K3 = 2.0 / hz * (1.0 - c3);
    const double M1 = hx / 3.0 * (2.0 + c1), M2 = hy / 3.0 * (2.0 + c2), M3 = hz / 3.0 * (2.0 + c3);
    const double lam = K1 * M2 * M3 + M1 * K2 * M3 + M1 * M2 * K3;
    const double w = (k1 == 0 || k1 == N ? 0.5 : 1.0) * (k2 == 0 || k2 == N ? 0.5 : 1.0) *
                     (k3 == 0 || k3 == N ? 0.5 : 1.0);
    const double f = 2.0 / N;
    z[t] *= f * f * f * w / lam;
  }
}

// u[3 n + r] = z[r][n] - z[r][0] - X_r(n): positions relative to node 1, minus the
// reference coordinates (the reference's u array, node-major)
__global__ void k_disp_out(const double* __restrict__ z, int N, double hx, double hy, double hz,
                           double* __restrict__ u) {
  const long long N1 = N + 1, nodes = N1 * N1 * N1;
  for (long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x; n < nodes;
       n += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(n % N1), j = (int)((n / N1) % N1), k = (int)(n / (N1 * N1));
    const double X[3] = {i * hx, j * hy, k * hz};
    for (int r = 0; r < 3; r++) u[3 * n + r] = n == 0 ? 0.0 : z[r * nodes + n] - z[r * nodes] - X[r];
  }
}

// node 0's entry of b: minus the sum of the others (one block)
__global__ void k_disp_pin(double* __restrict__ b, long long nodes) {
  __shared__ double part[256];
  for (int r = 0; r < 3; r++) {
    double s = 0.0;
    for (long long n = 1 + threadIdx.x; n < nodes; n += blockDim.x) s += b[r * nodes + n];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
      if ((int)threadIdx.x < w) part[threadIdx.x] += part[threadIdx.x + w];
      __syncthreads();
    }
    if (threadIdx.x == 0) b[r * nodes] = -part[0];
    __syncthreads();
  }
}

int grid_of(long long n) { return (int)std::min<long long>((n + 255) / 256, 8192); }

}  // namespace

// u (device, 3 x nodes doubles, node-major) from the device field F (9, N^3); work: two
// nodal fields (2 x 3 x nodes doubles); ctab: the (N+1)^2 table cos(pi k i / N)
cudaError_t f2disp_device(const double* F, int N, double lx, double ly, double lz,
                          const double* ctab, double* work, double* u, cudaStream_t st) {
  const long long N1 = N + 1, nodes = N1 * N1 * N1;
  const double hx = lx / N, hy = ly / N, hz = lz / N;
  double* a = work;
  double* b = work + 3 * nodes;
  k_disp_rhs<<<grid_of(nodes), 256, 0, st>>>(F, N, hx, hy, hz, a);
  k_disp_pin<<<1, 256, 0, st>>>(a, nodes);
  // forward DCT-I along x, y, z (strides 1, N1, N1^2), scale, and back
  k_dct1_axis<<<grid_of(3 * nodes), 256, 0, st>>>(a, b, N, 1, ctab);
  k_dct1_axis<<<grid_of(3 * nodes), 256, 0, st>>>(b, a, N, N1, ctab);
  k_dct1_axis<<<grid_of(3 * nodes), 256, 0, st>>>(a, b, N, N1 * N1, ctab);
  k_disp_scale<<<grid_of(3 * nodes), 256, 0, st>>>(b, N, hx, hy, hz);
  k_dct1_axis<<<grid_of(3 * nodes), 256, 0, st>>>(b, a, N, 1, ctab);
  k_dct1_axis<<<grid_of(3 * nodes), 256, 0, st>>>(a, b, N, N1, ctab);
  k_dct1_axis<<<grid_of(3 * nodes), 256, 0, st>>>(b, a, N, N1 * N1, ctab);
  k_disp_out<<<grid_of(nodes), 256, 0, st>>>(a, N, hx, hy, hz, u);
  g_kernel_launches += 10;
  return cudaGetLastError();
}
