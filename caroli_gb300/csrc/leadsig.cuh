// Lead self-energies on the device for a Hermitian definite coupling H1 = s c 1 (square and cubic
// leads, and multi-orbital leads whose coupling is a multiple of the identity): the fast path of
// caroli-green/src/modes.rs:540-710. The eigenvectors Y of the cell Hamiltonian serve every
// energy; at energy E each transverse mode k has the roots λ of λ² - μ_k λ + 1 = 0 (classified on
// the host, O(n) scalar work), and
//   Σ_R = s c Y diag(λ_R) Y^†,   Σ_L = s c Y diag(1/λ_L) Y^†      (the products of modes.rs:696-713)
//   Γ = i (Σ - Σ^†),             W_R = Y[:, propagating] sqrt(-2 s c Im λ_R)   (W_R W_R^† = Γ_R)
// The O(n³) products run here, in FP64.
#pragma once
#include <cstdint>

namespace caroli {

constexpr int LS_TILE = 32;  // output tile (rows and columns)
constexpr int LS_K = 16;     // inner-dimension chunk

// S[i, j] = sc Σ_k Y[i, k] d_k conj(Y[j, k]); Y n x n column-major. grid (n/32, n/32), 256 threads,
// each thread a 2 x 2 block of outputs.
__global__ void __launch_bounds__(256) lead_sigma_kernel(const double2* __restrict__ Y, int n,
                                                         const double2* __restrict__ d, double sc,
                                                         double2* __restrict__ S) {
  __shared__ double2 a[LS_K][LS_TILE + 1];  // Y[i0 + r, k0 + kk] d_k
  __shared__ double2 b[LS_K][LS_TILE + 1];  // conj(Y[j0 + r, k0 + kk])
  const int i0 = blockIdx.x * LS_TILE, j0 = blockIdx.y * LS_TILE;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  double2 acc[2][2];
  for (int p = 0; p < 2; ++p)
    for (int q = 0; q < 2; ++q) acc[p][q] = make_double2(0.0, 0.0);
  for (int k0 = 0; k0 < n; k0 += LS_K) {
    for (int e = threadIdx.x; e < LS_K * LS_TILE; e += 256) {
      const int r = e % LS_TILE, kk = e / LS_TILE, k = k0 + kk;
      double2 va = make_double2(0.0, 0.0), vb = make_double2(0.0, 0.0);
      if (k < n) {
        if (i0 + r < n) {
          const double2 y = Y[(i0 + r) + (int64_t)k * n], dk = d[k];
          va = make_double2(y.x * dk.x - y.y * dk.y, y.x * dk.y + y.y * dk.x);
        }
        if (j0 + r < n) {
          const double2 y = Y[(j0 + r) + (int64_t)k * n];
          vb = make_double2(y.x, -y.y);
        }
      }
      a[kk][r] = va;
      b[kk][r] = vb;
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < LS_K; ++kk) {
      double2 av[2], bv[2];
      for (int p = 0; p < 2; ++p) av[p] = a[kk][ty + 16 * p];
      for (int q = 0; q < 2; ++q) bv[q] = b[kk][tx + 16 * q];
      for (int p = 0; p < 2; ++p)
        for (int q = 0; q < 2; ++q) {
          acc[p][q].x = fma(av[p].x, bv[q].x, fma(-av[p].y, bv[q].y, acc[p][q].x));
          acc[p][q].y = fma(av[p].x, bv[q].y, fma(av[p].y, bv[q].x, acc[p][q].y));
        }
    }
    __syncthreads();
  }
  for (int p = 0; p < 2; ++p)
    for (int q = 0; q < 2; ++q) {
      const int i = i0 + ty + 16 * p, j = j0 + tx + 16 * q;
      if (i < n && j < n) S[i + (int64_t)j * n] = make_double2(sc * acc[p][q].x, sc * acc[p][q].y);
    }
}

// Γ = i (S - S^†), n x n.
__global__ void lead_gamma_kernel(const double2* __restrict__ S, int n, double2* __restrict__ G) {
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (idx >= (int64_t)n * n) return;
  const int i = (int)(idx % n), j = (int)(idx / n);
  const double2 a = S[i + (int64_t)j * n], b = S[j + (int64_t)i * n];
  // i ((a.x - b.x) + i (a.y + b.y)) = -(a.y + b.y) + i (a.x - b.x)
  G[idx] = make_double2(-(a.y + b.y), a.x - b.x);
}

// W[:, c] = Y[:, cols[c]] w[c], n x nc.
__global__ void lead_channels_kernel(const double2* __restrict__ Y, int n, const int32_t* __restrict__ cols,
                                     const double* __restrict__ w, int nc, double2* __restrict__ W) {
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (idx >= (int64_t)n * nc) return;
  const int i = (int)(idx % n), c = (int)(idx / n);
  const double2 y = Y[i + (int64_t)cols[c] * n];
  W[idx] = make_double2(y.x * w[c], y.y * w[c]);
}

}  // namespace caroli
