// FP32 Cholesky preconditioner of a large normal matrix for the conjugate-gradient solve of the
// mixed method (the quadratic block of the QNML fit, the kernel block of KRR).
//
// The preconditioner only steers the conjugate-gradient iteration: the iterates solve the FP64
// normal equations whatever its accuracy, and the diagonal shift it carries (relative 1e-3 at
// D ~ 6000) is far above FP32 rounding.  So it is factorised in FP32 on the CUDA cores, which
// run FP32 at 64x the FP64 rate of this GPU:
//   s_i = 1 / sqrt(d_i),  d_i = G_ii + max(lambda, rel G_ii)            (Jacobi scaling)
//   A   = S (G + diag(d - G_ii)) S, unit diagonal                          (FP32)
//   A   = L L^T                       blocked right-looking Cholesky, 64-column panels
//   R   = L^-1                        diagonal 64-blocks, then recursive doubling with GEMMs:
//                                     R21 = -R22 (L21 R11)
//   M^-1 r = S R^T R S r              two dense triangular matvecs, double-FP32 arithmetic
// M^-1 is a fixed symmetric positive-definite operator (R and R^T hold the same FP32 numbers),
// so the standard conjugate-gradient recurrences stay valid.
#include <cuda_runtime.h>
#include <math.h>

#include "ds.cuh"
#include "mld_internal.h"

namespace mld {

constexpr int kNB = 64;  // panel width of the FP32 factorisation and size of the base inverse blocks

// s_i and the scaled, shifted matrix (full square; only the lower triangle is used later).
// A column whose shifted diagonal is not positive (an all-zero feature without ridge) gets
// s_i = 0 and a unit diagonal: the preconditioner then leaves that direction untouched.
__global__ void k_p32_scale_diag(const double* __restrict__ G, int D, double lam, double rel, double* __restrict__ s) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= D) return;
  const double g = G[(size_t)i * D + i];
  const double d = g + fmax(lam, rel * g);
  s[i] = d > 0.0 ? 1.0 / sqrt(d) : 0.0;
}

__global__ void k_p32_scale(const double* __restrict__ G, int D, const double* __restrict__ s, float* __restrict__ A) {
  const int j = blockIdx.x * 32 + threadIdx.x;
  for (int i = blockIdx.y * 32 + threadIdx.y; i < min(D, blockIdx.y * 32 + 32); i += blockDim.y) {
    if (j >= D) continue;
    const double v = (i == j) ? 1.0 : G[(size_t)i * D + j] * s[i] * s[j];
    A[(size_t)i * D + j] = (float)v;
  }
}

// Factor the diagonal block [k0, k0 + nb) in place (one CTA); info = first failing column + 1.
__global__ void __launch_bounds__(256) k_p32_potrf_diag(float* A, int D, int k0, int nb, int* info) {
  __shared__ float L[kNB][kNB + 1];
  const int tid = threadIdx.x;
  for (int e = tid; e < nb * nb; e += blockDim.x) {
    const int i = e / nb, j = e % nb;
    L[i][j] = A[(size_t)(k0 + i) * D + (k0 + j)];
  }
  __syncthreads();
  for (int j = 0; j < nb; ++j) {
    if (tid == 0) {
      float d = L[j][j];
      if (!(d > 0.0f)) {
        if (info[0] == 0) info[0] = k0 + j + 1;
        d = 1.0f;
      }
      L[j][j] = sqrtf(d);
    }
    __syncthreads();
    const float djj = L[j][j];
    for (int i = j + 1 + tid; i < nb; i += blockDim.x) L[i][j] /= djj;
    __syncthreads();
    const int m = nb - j - 1;
    for (int e = tid; e < m * m; e += blockDim.x) {
      const int i = j + 1 + e / m, c = j + 1 + e % m;
      if (c <= i) L[i][c] -= L[i][j] * L[c][j];
    }
    __syncthreads();
  }
  for (int e = tid; e < nb * nb; e += blockDim.x) {
    const int i = e / nb, j = e % nb;
    if (j <= i) A[(size_t)(k0 + i) * D + (k0 + j)] = L[i][j];
  }
}

// Panel below the diagonal block: rows r >= k0 + kNB, A[r][k0..k0+kNB) <- A[r][..] L11^-T.
// One thread per row; the block is full width here (nb == kNB: only the last panel is ragged
// and it has no rows below it).
__global__ void __launch_bounds__(128) k_p32_trsm(float* A, int D, int k0) {
  __shared__ float L[kNB][kNB + 1];
  for (int e = threadIdx.x; e < kNB * kNB; e += blockDim.x) {
    const int i = e / kNB, j = e % kNB;
    L[i][j] = (j <= i) ? A[(size_t)(k0 + i) * D + (k0 + j)] : 0.0f;
  }
  __syncthreads();
  const int r = k0 + kNB + blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= D) return;
  float x[kNB];
  float* row = A + (size_t)r * D + k0;
#pragma unroll
  for (int j = 0; j < kNB; ++j) x[j] = row[j];
#pragma unroll
  for (int j = 0; j < kNB; ++j) {
    float v = x[j];
#pragma unroll
    for (int c = 0; c < j; ++c) v = fmaf(-x[c], L[j][c], v);
    x[j] = v / L[j][j];
  }
#pragma unroll
  for (int j = 0; j < kNB; ++j) row[j] = x[j];
}

// Trailing update of the lower triangle: A[i][j] -= sum_c P[i][c] P[j][c] over the panel
// columns c in [k0, k0 + kNB), for i, j >= k1 = k0 + kNB, j <= i.  64 x 64 tiles over the
// lower-triangular tile pairs, 16 x 16 threads with 4 x 4 outputs each.
__global__ void __launch_bounds__(256) k_p32_syrk(float* A, int D, int k0) {
  const int k1 = k0 + kNB;
  int t = blockIdx.x, ti = 0;
  while (t >= ti + 1) {
    t -= ti + 1;
    ++ti;
  }
  const int tj = t;
  const int i0 = k1 + ti * 64, j0 = k1 + tj * 64;
  if (i0 >= D) return;
  __shared__ float Pi[64][kNB + 1], Pj[64][kNB + 1];
  for (int e = threadIdx.x; e < 64 * kNB; e += blockDim.x) {
    const int r = e / kNB, c = e % kNB;
    Pi[r][c] = (i0 + r < D) ? A[(size_t)(i0 + r) * D + k0 + c] : 0.0f;
    Pj[r][c] = (j0 + r < D) ? A[(size_t)(j0 + r) * D + k0 + c] : 0.0f;
  }
  __syncthreads();
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  float acc[4][4] = {};
#pragma unroll 4
  for (int c = 0; c < kNB; ++c) {
    float a[4], b[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      a[u] = Pi[ty + 16 * u][c];
      b[u] = Pj[tx + 16 * u][c];
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) acc[u][v] = fmaf(a[u], b[v], acc[u][v]);
  }
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int i = i0 + ty + 16 * u, j = j0 + tx + 16 * v;
      if (i < D && j <= i) A[(size_t)i * D + j] -= acc[u][v];
    }
}

// Inverse of each diagonal 64-block of L (one CTA per block, one thread per column).
__global__ void __launch_bounds__(kNB) k_p32_trinv_diag(const float* __restrict__ L, int D, float* __restrict__ R) {
  __shared__ float Ld[kNB][kNB + 1], X[kNB][kNB + 1];
  const int k0 = blockIdx.x * kNB, nb = min(kNB, D - k0), t = threadIdx.x;
  for (int e = t; e < nb * nb; e += blockDim.x) {
    const int i = e / nb, j = e % nb;
    Ld[i][j] = (j <= i) ? L[(size_t)(k0 + i) * D + k0 + j] : 0.0f;
  }
  __syncthreads();
  if (t < nb) {
    for (int i = 0; i < nb; ++i) {
      float v = (i == t) ? 1.0f : 0.0f;
      for (int c = t; c < i; ++c) v = fmaf(-Ld[i][c], X[c][t], v);
      X[i][t] = (i < t) ? 0.0f : v / Ld[i][i];
    }
  }
  __syncthreads();
  for (int e = t; e < nb * nb; e += blockDim.x) {
    const int i = e / nb, j = e % nb;
    R[(size_t)(k0 + i) * D + k0 + j] = X[i][j];
  }
}

// C (M x N, ldc) = alpha * A (M x K, lda) * B (K x N, ldb); 64 x 64 tiles, K in chunks of 32,
// 16 x 16 threads with 4 x 4 outputs each.
__global__ void __launch_bounds__(256) k_p32_gemm(int M, int N, int K, const float* __restrict__ A, int lda,
                                                  const float* __restrict__ B, int ldb, float* __restrict__ C,
                                                  int ldc, float alpha) {
  __shared__ float As[64][33], Bs[32][65];
  const int m0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += 32) {
    for (int e = threadIdx.x; e < 64 * 32; e += 256) {
      const int r = e >> 5, c = e & 31;
      As[r][c] = (m0 + r < M && k0 + c < K) ? A[(size_t)(m0 + r) * lda + k0 + c] : 0.0f;
      const int kr = e >> 6, nc = e & 63;
      Bs[kr][nc] = (k0 + kr < K && n0 + nc < N) ? B[(size_t)(k0 + kr) * ldb + n0 + nc] : 0.0f;
    }
    __syncthreads();
#pragma unroll 8
    for (int c = 0; c < 32; ++c) {
      float a[4], b[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        a[u] = As[ty + 16 * u][c];
        b[u] = Bs[c][tx + 16 * u];
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = fmaf(a[u], b[v], acc[u][v]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int i = m0 + ty + 16 * u, j = n0 + tx + 16 * v;
      if (i < M && j < N) C[(size_t)i * ldc + j] = alpha * acc[u][v];
    }
}

// Rt = R^T for the lower triangle of R (the upper part of Rt); everything else zero.
__global__ void k_p32_transpose(const float* __restrict__ R, int D, float* __restrict__ Rt) {
  __shared__ float tile[32][33];
  const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int r = by + y, c = bx + threadIdx.x;
    tile[y][threadIdx.x] = (r < D && c < D && c <= r) ? R[(size_t)r * D + c] : 0.0f;
  }
  __syncthreads();
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int r = bx + y, c = by + threadIdx.x;
    if (r < D && c < D) Rt[(size_t)r * D + c] = tile[threadIdx.x][y];
  }
}

// x2 = (si * x) as double-FP32 pairs (si may be null: unit)
__global__ void k_p32_split(const double* __restrict__ si, const double* __restrict__ x, int D,
                            float2* __restrict__ x2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= D) return;
  float h, l;
  ds_split(si ? si[i] * x[i] : x[i], h, l);
  x2[i] = make_float2(h, l);
}

// y_i = so_i * sum_c T[i][c] * x2_c over the triangle of row i (FP32 matrix, double-FP32
// arithmetic on the FP32 pipe); so may be null (unit).  Warp per row.
__global__ void __launch_bounds__(256) k_p32_trmv(const float* __restrict__ T, int D, int upper,
                                                 const float2* __restrict__ x2, const double* __restrict__ so,
                                                 double* __restrict__ y) {
  const int lane = threadIdx.x & 31;
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (i >= D) return;
  const int lo = upper ? i : 0, hi = upper ? D : i + 1;
  const float* row = T + (size_t)i * D;
  float sh = 0.f, sl = 0.f;
  for (int c = lo + lane; c < hi; c += 32) {
    const float2 v = x2[c];
    ds_fma(sh, sl, row[c], v.x, v.y);
  }
  for (int o = 16; o > 0; o >>= 1) {
    const float oh = __shfl_xor_sync(0xffffffffu, sh, o), ol = __shfl_xor_sync(0xffffffffu, sl, o);
    ds_add(sh, sl, oh, ol);
  }
  if (lane == 0) {
    const double a = (double)sh + (double)sl;
    y[i] = so ? so[i] * a : a;
  }
}

size_t precond32_workspace_bytes(int D) {
  const size_t d2 = (size_t)D * D;
  const size_t h = (size_t)(D + 1) / 2;
  return sizeof(float) * (3 * d2 + h * h) + sizeof(double) * (size_t)D + 256 + sizeof(float2) * (size_t)D + 256;
}

// Factorise: on return *info (device) is 0 on success, or the first failing column + 1.
// ws: precond32_workspace_bytes(D) bytes; layout [s (D doubles) | L | R | Rt | T].
cudaError_t launch_precond32_build(const double* G, int D, double lam, double rel, void* ws, int* info,
                                   cudaStream_t st, int* launches) {
  double* s = (double*)ws;
  float* L = (float*)((char*)ws + ((sizeof(double) * (size_t)D + 255) / 256) * 256);
  const size_t d2 = (size_t)D * D;
  float* R = L + d2;
  float* Rt = R + d2;
  float* T = Rt + d2;
  int n = 0;
  cudaError_t e = cudaMemsetAsync(info, 0, sizeof(int), st);
  if (e != cudaSuccess) return e;
  k_p32_scale_diag<<<(D + 255) / 256, 256, 0, st>>>(G, D, lam, rel, s);
  dim3 g32((D + 31) / 32, (D + 31) / 32);
  k_p32_scale<<<g32, dim3(32, 8), 0, st>>>(G, D, s, L);
  n += 2;
  for (int k0 = 0; k0 < D; k0 += kNB) {
    const int nb = min(kNB, D - k0);
    k_p32_potrf_diag<<<1, 256, 0, st>>>(L, D, k0, nb, info);
    ++n;
    const int rows = D - k0 - nb;
    if (rows > 0) {
      k_p32_trsm<<<(rows + 127) / 128, 128, 0, st>>>(L, D, k0);
      const int nt = (rows + 63) / 64;
      k_p32_syrk<<<nt * (nt + 1) / 2, 256, 0, st>>>(L, D, k0);
      n += 2;
    }
  }
  // R = L^-1: zero, invert the diagonal blocks, then merge pairs of blocks of doubling size
  e = cudaMemsetAsync(R, 0, sizeof(float) * d2, st);
  if (e != cudaSuccess) return e;
  k_p32_trinv_diag<<<(D + kNB - 1) / kNB, kNB, 0, st>>>(L, D, R);
  ++n;
  for (int b = 2 * kNB; b / 2 < D; b *= 2) {
    const int h = b / 2;
    for (int s0 = 0; s0 + h < D; s0 += b) {
      const int n1 = h, n2 = min(h, D - s0 - h);
      // T (n2 x n1) = L21 R11
      dim3 gt((n1 + 63) / 64, (n2 + 63) / 64);
      k_p32_gemm<<<gt, 256, 0, st>>>(n2, n1, n1, L + (size_t)(s0 + h) * D + s0, D, R + (size_t)s0 * D + s0, D, T, n1,
                                     1.0f);
      // R21 = -R22 T
      k_p32_gemm<<<gt, 256, 0, st>>>(n2, n1, n2, R + (size_t)(s0 + h) * D + s0 + h, D, T, n1,
                                     R + (size_t)(s0 + h) * D + s0, D, -1.0f);
      n += 2;
    }
  }
  k_p32_transpose<<<g32, dim3(32, 8), 0, st>>>(R, D, Rt);
  ++n;
  if (launches) *launches = n;
  return cudaGetLastError();
}

// z = S R^T R S r; tmp holds D doubles
cudaError_t launch_precond32_apply(const void* ws, int D, const double* r, double* z, double* tmp, cudaStream_t st) {
  const double* s = (const double*)ws;
  const float* L = (const float*)((const char*)ws + ((sizeof(double) * (size_t)D + 255) / 256) * 256);
  const size_t d2 = (size_t)D * D;
  const float* R = L + d2;
  const float* Rt = R + d2;
  const size_t h = (size_t)(D + 1) / 2;
  float2* x2 = (float2*)((char*)(Rt + d2 + h * h) + (256 - ((uintptr_t)(Rt + d2 + h * h) & 255)) % 256);
  const unsigned blocks = (unsigned)(((long long)D * 32 + 255) / 256);
  k_p32_split<<<(D + 255) / 256, 256, 0, st>>>(s, r, D, x2);
  k_p32_trmv<<<blocks, 256, 0, st>>>(R, D, 0, x2, nullptr, tmp);
  k_p32_split<<<(D + 255) / 256, 256, 0, st>>>(nullptr, tmp, D, x2);
  k_p32_trmv<<<blocks, 256, 0, st>>>(Rt, D, 1, x2, s, z);
  return cudaGetLastError();
}

}  // namespace mld
