// FP32 inverse of a preconditioner factor for the conjugate-gradient solve of the mixed method
// (the wide blocks: the quadratic block of the QNML fit, the kernel block of KRR).
//
// The factor L (FP64, lower) comes from the Cholesky factorisation of the sketched normal matrix
// (sketch.cu).  Its inverse only steers the iteration: the iterates solve the FP64 normal
// equations whatever its accuracy, and an FP32 inverse of a triangular factor has a relative
// error of about 2^-24 times its condition number (the square root of the normal matrix's), well
// inside what CG absorbs.  So it is inverted in FP32 on the CUDA cores, which run FP32 at 64x the
// FP64 rate of this GPU:
//   s_i = 1 / |L_i,:|                 (Jacobi scaling: (L L^T)_ii = |L_i,:|^2)
//   A   = S L                         FP32, unit-norm rows
//   R   = A^-1                        diagonal 64-blocks, then recursive doubling with GEMMs:
//                                     R21 = -R22 (A21 R11)
//   M^-1 r = S R^T R S r              two dense triangular matvecs, double-FP32 arithmetic
// M^-1 is a fixed symmetric positive-definite operator (R and R^T hold the same FP32 numbers),
// so the standard conjugate-gradient recurrences stay valid.
#include <cuda_runtime.h>
#include <math.h>

#include "ds.cuh"
#include "mld_internal.h"

namespace mld {

constexpr int kNB = 64;  // panel width of the FP32 factorisation and size of the base inverse blocks

// s_i = 1 / |L_i,:| and A = S L in FP32 (lower triangle, zero above); warp per row.  A zero row
// (an all-zero feature) gets s_i = 0 and a unit diagonal.
__global__ void __launch_bounds__(256) k_p32_from_factor(const double* __restrict__ Lf, int D,
                                                         double* __restrict__ s, float* __restrict__ A) {
  const int lane = threadIdx.x & 31;
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (i >= D) return;
  const double* row = Lf + (size_t)i * D;
  double n2 = 0.0;
  for (int c = lane; c <= i; c += 32) n2 = fma(row[c], row[c], n2);
  for (int o = 16; o > 0; o >>= 1) n2 += __shfl_xor_sync(0xffffffffu, n2, o);
  const double si = n2 > 0.0 ? 1.0 / sqrt(n2) : 0.0;
  float* out = A + (size_t)i * D;
  for (int c = lane; c < D; c += 32)
    out[c] = c > i ? 0.0f : (si > 0.0 ? (float)(row[c] * si) : (c == i ? 1.0f : 0.0f));
  if (lane == 0) s[i] = si;
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

// From the FP64 factor Lf (lower triangle read): S, A = S L and R = A^-1, R^T.
// ws: precond32_workspace_bytes(D) bytes; layout [s (D doubles) | A | R | Rt | T].
cudaError_t launch_precond32_from_factor(const double* Lf, int D, void* ws, cudaStream_t st, int* launches) {
  double* s = (double*)ws;
  float* L = (float*)((char*)ws + ((sizeof(double) * (size_t)D + 255) / 256) * 256);
  const size_t d2 = (size_t)D * D;
  float* R = L + d2;
  float* Rt = R + d2;
  float* T = Rt + d2;
  int n = 0;
  k_p32_from_factor<<<(unsigned)(((long long)D * 32 + 255) / 256), 256, 0, st>>>(Lf, D, s, L);
  ++n;
  dim3 g32((D + 31) / 32, (D + 31) / 32);
  // R = L^-1: zero, invert the diagonal blocks, then merge pairs of blocks of doubling size
  cudaError_t e = cudaMemsetAsync(R, 0, sizeof(float) * d2, st);
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
