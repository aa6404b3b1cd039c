// Blocked FP64 Cholesky factorisation and triangular solves for large normal matrices
// (D > kJacobiMax, e.g. the quadratic block of the QNML fit).
//
// The reference solves the regularised normal equations (A W A^T + lambda I) w = A W y with
// LAPACK dgelsd (parameters.F90:1018-1099, stats_tools.F90:1153-1213).  For a symmetric
// positive-definite normal matrix the Cholesky solution is the same solution; a rank-deficient
// matrix without ridge gets a relative diagonal shift `jitter * max(diag)` (the min-norm
// solution differs only in the null space, predictions agree).  Iterative refinement with FP64
// residuals (driven from api.cu) recovers FP64-level coefficients.
//
// Right-looking blocked algorithm, block size kCB, lower triangle, row-major D x D (lda):
//   for each block column k: factor the diagonal block (one CTA), solve the panel below it
//   (L21 = A21 L11^-T), update the trailing lower triangle A22 -= L21 L21^T.
#include <cuda_runtime.h>
#include <math.h>

#include "ds.cuh"
#include "mld_internal.h"

namespace mld {

constexpr int kCB = 32;

// Factor the diagonal block [k0, k0+nb) in place; info[0] = first failing column + 1.
__global__ void __launch_bounds__(256) k_potrf_diag(double* A, int lda, int k0, int nb, double shift, int* info) {
  __shared__ double L[kCB][kCB + 1];
  const int tid = threadIdx.x;
  for (int e = tid; e < nb * nb; e += blockDim.x) {
    const int i = e / nb, j = e % nb;
    double v = A[(size_t)(k0 + i) * lda + (k0 + j)];
    if (i == j) v += shift;
    L[i][j] = v;
  }
  __syncthreads();
  for (int j = 0; j < nb; ++j) {
    if (tid == 0) {
      double d = L[j][j];
      if (!(d > 0.0)) {
        if (info[0] == 0) info[0] = k0 + j + 1;
        d = 1e-300;
      }
      L[j][j] = sqrt(d);
    }
    __syncthreads();
    const double djj = L[j][j];
    for (int i = j + 1 + tid; i < nb; i += blockDim.x) L[i][j] /= djj;
    __syncthreads();
    for (int e = tid; e < (nb - j - 1) * (nb - j - 1); e += blockDim.x) {
      const int i = j + 1 + e / (nb - j - 1), c = j + 1 + e % (nb - j - 1);
      if (c <= i) L[i][c] -= L[i][j] * L[c][j];
    }
    __syncthreads();
  }
  for (int e = tid; e < nb * nb; e += blockDim.x) {
    const int i = e / nb, j = e % nb;
    if (j <= i) A[(size_t)(k0 + i) * lda + (k0 + j)] = L[i][j];
  }
}

// Panel: rows r in [k0+nb, D): A[r][k0..k0+nb) <- A[r][..] L11^-T  (one thread per row)
__global__ void __launch_bounds__(128) k_trsm_panel(double* A, int lda, int D, int k0, int nb) {
  __shared__ double L[kCB][kCB + 1];
  for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) {
    const int i = e / nb, j = e % nb;
    L[i][j] = (j <= i) ? A[(size_t)(k0 + i) * lda + (k0 + j)] : 0.0;
  }
  __syncthreads();
  const int r = k0 + nb + blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= D) return;
  double x[kCB];
  for (int j = 0; j < nb; ++j) x[j] = A[(size_t)r * lda + k0 + j];
  for (int j = 0; j < nb; ++j) {
    double v = x[j];
    for (int c = 0; c < j; ++c) v -= x[c] * L[j][c];
    x[j] = v / L[j][j];
  }
  for (int j = 0; j < nb; ++j) A[(size_t)r * lda + k0 + j] = x[j];
}

// Trailing update of the lower triangle: A[i][j] -= sum_c L[i][c] L[j][c], i, j >= k1, j <= i.
// 32x32 tiles, 16x16 threads with 2x2 outputs.
__global__ void __launch_bounds__(256) k_syrk_update(double* A, int lda, int D, int k0, int nb, int k1) {
  const int ntile = (D - k1 + 31) / 32;
  int t = blockIdx.x, ti = 0;
  while (t >= ti + 1) {  // lower-triangular tile pairs (tj <= ti)
    t -= ti + 1;
    ++ti;
  }
  const int tj = t;
  if (ti >= ntile) return;
  const int i0 = k1 + ti * 32, j0 = k1 + tj * 32;
  __shared__ double Li[32][kCB + 1], Lj[32][kCB + 1];
  for (int e = threadIdx.x; e < 32 * nb; e += blockDim.x) {
    const int r = e / nb, c = e % nb;
    Li[r][c] = (i0 + r < D) ? A[(size_t)(i0 + r) * lda + k0 + c] : 0.0;
    Lj[r][c] = (j0 + r < D) ? A[(size_t)(j0 + r) * lda + k0 + c] : 0.0;
  }
  __syncthreads();
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  double acc[2][2] = {{0, 0}, {0, 0}};
  for (int c = 0; c < nb; ++c) {
    const double a0 = Li[ty][c], a1 = Li[ty + 16][c];
    const double b0 = Lj[tx][c], b1 = Lj[tx + 16][c];
    acc[0][0] = fma(a0, b0, acc[0][0]);
    acc[0][1] = fma(a0, b1, acc[0][1]);
    acc[1][0] = fma(a1, b0, acc[1][0]);
    acc[1][1] = fma(a1, b1, acc[1][1]);
  }
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 2; ++b) {
      const int i = i0 + ty + 16 * a, j = j0 + tx + 16 * b;
      if (i < D && j < D && j <= i) A[(size_t)i * lda + j] -= acc[a][b];
    }
}

// k_syrk_update in double-FP32 arithmetic on the FP32 pipe (GB300 issues FP64 at 1/64 of its FP32
// rate): the panel entries as FP32 pairs hi + lo, each product formed as the exact hi hi (fmaf)
// plus hi lo + lo hi, the sum over the panel as an unevaluated pair, one FP64 subtraction per
// element and panel.  About 2^-44 relative to the magnitudes of the products: used for the
// preconditioner factor of the mixed method, not for the plain solve.
__global__ void __launch_bounds__(256) k_syrk_update_ds(double* A, int lda, int D, int k0, int nb, int k1) {
  const int ntile = (D - k1 + 31) / 32;
  int t = blockIdx.x, ti = 0;
  while (t >= ti + 1) {
    t -= ti + 1;
    ++ti;
  }
  const int tj = t;
  if (ti >= ntile) return;
  const int i0 = k1 + ti * 32, j0 = k1 + tj * 32;
  __shared__ float2 Li[kCB][33], Lj[kCB][33];  // [c][row]
  for (int e = threadIdx.x; e < 32 * nb; e += blockDim.x) {
    const int r = e / nb, c = e % nb;
    float h, l;
    ds_split((i0 + r < D) ? A[(size_t)(i0 + r) * lda + k0 + c] : 0.0, h, l);
    Li[c][r] = make_float2(h, l);
    ds_split((j0 + r < D) ? A[(size_t)(j0 + r) * lda + k0 + c] : 0.0, h, l);
    Lj[c][r] = make_float2(h, l);
  }
  __syncthreads();
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  float sh[2][2] = {{0.f, 0.f}, {0.f, 0.f}}, sl[2][2] = {{0.f, 0.f}, {0.f, 0.f}};
  for (int c = 0; c < nb; ++c) {
    const float2 a[2] = {Li[c][ty], Li[c][ty + 16]};
    const float2 b[2] = {Lj[c][tx], Lj[c][tx + 16]};
#pragma unroll
    for (int p = 0; p < 2; ++p)
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        const float pr = a[p].x * b[q].x;
        const float pe = fmaf(a[p].x, b[q].y, fmaf(a[p].y, b[q].x, fmaf(a[p].x, b[q].x, -pr)));
        float su, er;
        two_sum(sh[p][q], pr, su, er);
        sh[p][q] = su;
        sl[p][q] += er + pe;
      }
  }
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 2; ++b) {
      const int i = i0 + ty + 16 * a, j = j0 + tx + 16 * b;
      if (i < D && j < D && j <= i) A[(size_t)i * lda + j] -= (double)sh[a][b] + (double)sl[a][b];
    }
}

// Solve L L^T x = b in one CTA (forward then backward substitution, blocked by kCB rows).
__global__ void __launch_bounds__(1024) k_chol_solve(const double* L, int lda, int D, const double* b, double* x) {
  extern __shared__ double sx[];  // D
  const int tid = threadIdx.x, nth = blockDim.x;
  for (int i = tid; i < D; i += nth) sx[i] = b[i];
  __syncthreads();
  __shared__ double red[32];
  // forward: L y = b
  for (int i = 0; i < D; ++i) {
    double part = 0.0;
    for (int c = tid; c < i; c += nth) part = fma(L[(size_t)i * lda + c], sx[c], part);
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    if ((tid & 31) == 0) red[tid >> 5] = part;
    __syncthreads();
    if (tid == 0) {
      double s = 0.0;
      for (int w = 0; w < (nth + 31) / 32; ++w) s += red[w];
      sx[i] = (sx[i] - s) / L[(size_t)i * lda + i];
    }
    __syncthreads();
  }
  // backward: L^T x = y
  for (int i = D - 1; i >= 0; --i) {
    double part = 0.0;
    for (int c = i + 1 + tid; c < D; c += nth) part = fma(L[(size_t)c * lda + i], sx[c], part);
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    if ((tid & 31) == 0) red[tid >> 5] = part;
    __syncthreads();
    if (tid == 0) {
      double s = 0.0;
      for (int w = 0; w < (nth + 31) / 32; ++w) s += red[w];
      sx[i] = (sx[i] - s) / L[(size_t)i * lda + i];
    }
    __syncthreads();
  }
  for (int i = tid; i < D; i += nth) x[i] = sx[i];
}

// r = h - (G + lambda I) w (full symmetric G, row-major), FP64.
__global__ void k_residual(const double* G, int D, double lambda, const double* w, const double* h, double* r) {
  const int lane = threadIdx.x & 31;
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (i >= D) return;
  double acc = 0.0;
  for (int c = lane; c < D; c += 32) acc = fma(G[(size_t)i * D + c], w[c], acc);
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) r[i] = h[i] - acc - lambda * w[i];
}

__global__ void k_axpy(int n, double a, const double* x, double* y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] += a * x[i];
}

// ------------------------------------------------------------------------------------
// Blocked triangular solves with the Cholesky factor, one launch per 64-row block step.
// Every CTA of a step solves the 64 x 64 diagonal block itself (cheap), so the block's
// solution never has to be published between CTAs; the running right-hand side `r` is only
// written outside the block being solved.
// ------------------------------------------------------------------------------------
constexpr int kTB = 64;

// forward, L y = r: y[k0..k0+nb) from the diagonal block, r[i] -= L[i][blk] . y[blk] for i below
__global__ void __launch_bounds__(256) k_trsv_fwd(const double* __restrict__ L, int D, int k0, int nb,
                                                  double* __restrict__ r, double* __restrict__ y) {
  __shared__ double Ld[kTB][kTB + 1];
  __shared__ double xs[kTB];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) {
    const int i = e / nb, j = e % nb;
    Ld[i][j] = (j <= i) ? L[(size_t)(k0 + i) * D + k0 + j] : 0.0;
  }
  for (int i = threadIdx.x; i < nb; i += blockDim.x) xs[i] = r[k0 + i];
  __syncthreads();
  if (warp == 0) {
    for (int j = 0; j < nb; ++j) {
      const double xj = xs[j] / Ld[j][j];
      __syncwarp();
      for (int i = j + 1 + lane; i < nb; i += 32) xs[i] -= Ld[i][j] * xj;
      if (lane == 0) xs[j] = xj;
      __syncwarp();
    }
  }
  __syncthreads();
  if (blockIdx.x == 0)
    for (int i = threadIdx.x; i < nb; i += blockDim.x) y[k0 + i] = xs[i];
  for (int i = k0 + nb + blockIdx.x * nw + warp; i < D; i += gridDim.x * nw) {
    double acc = 0.0;
    for (int c = lane; c < nb; c += 32) acc = fma(L[(size_t)i * D + k0 + c], xs[c], acc);
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) r[i] -= acc;
  }
}

// backward, L^T x = r: x[k0..k0+nb) from the diagonal block, r[i] -= sum_c L[k0+c][i] x[k0+c] for i < k0
__global__ void __launch_bounds__(256) k_trsv_bwd(const double* __restrict__ L, int D, int k0, int nb,
                                                  double* __restrict__ r, double* __restrict__ x) {
  __shared__ double Ld[kTB][kTB + 1];
  __shared__ double xs[kTB];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) {
    const int i = e / nb, j = e % nb;
    Ld[i][j] = (j <= i) ? L[(size_t)(k0 + i) * D + k0 + j] : 0.0;
  }
  for (int i = threadIdx.x; i < nb; i += blockDim.x) xs[i] = r[k0 + i];
  __syncthreads();
  if (warp == 0) {
    for (int j = nb - 1; j >= 0; --j) {
      const double xj = xs[j] / Ld[j][j];
      __syncwarp();
      for (int i = lane; i < j; i += 32) xs[i] -= Ld[j][i] * xj;
      if (lane == 0) xs[j] = xj;
      __syncwarp();
    }
  }
  __syncthreads();
  if (blockIdx.x == 0)
    for (int i = threadIdx.x; i < nb; i += blockDim.x) x[k0 + i] = xs[i];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < k0; i += gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int c = 0; c < nb; ++c) acc = fma(L[(size_t)(k0 + c) * D + i], xs[c], acc);
    r[i] -= acc;
  }
}

// A[i][i] += max(lambda, rel * A[i][i]); an empty (zero) diagonal entry gets 1
__global__ void k_shift_diag_rel(double* A, int D, double lambda, double rel) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= D) return;
  double* d = A + (size_t)i * D + i;
  *d += (*d > 0.0) ? fmax(lambda, rel * *d) : 1.0;
}

// ------------------------------------------------------------------------------------
// Preconditioned conjugate gradients on the normal equations, vector updates in one CTA.
// scal[0] = r.z of the current iterate, scal[1] = r.z of the first iterate, scal[2] = alpha,
// scal[3] = alpha * r.z, the decrease of sum_r w_r (y_r - x_r.w)^2 + lambda |w|^2 in the step.
// ------------------------------------------------------------------------------------
__device__ double block_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
  return s;
}

// x += alpha p, r -= alpha q with alpha = (r.z) / (p.q)
__global__ void __launch_bounds__(1024) k_pcg_alpha(int D, const double* __restrict__ p, const double* __restrict__ q,
                                                    double* __restrict__ x, double* __restrict__ r,
                                                    double* __restrict__ scal) {
  __shared__ double red[32];
  double s = 0.0;
  for (int i = threadIdx.x; i < D; i += blockDim.x) s = fma(p[i], q[i], s);
  const double pq = block_sum(s, red);
  const double alpha = (pq > 0.0) ? scal[0] / pq : 0.0;
  for (int i = threadIdx.x; i < D; i += blockDim.x) {
    x[i] = fma(alpha, p[i], x[i]);
    r[i] = fma(-alpha, q[i], r[i]);
  }
  if (threadIdx.x == 0) {
    scal[2] = alpha;
    scal[3] = alpha * scal[0];  // decrease of the least-squares objective in this step
  }
}

// p = z + beta p with beta = (r.z)_new / (r.z)_old; first: p = z
__global__ void __launch_bounds__(1024) k_pcg_beta(int D, const double* __restrict__ z, const double* __restrict__ r,
                                                   double* __restrict__ p, double* __restrict__ scal, int first) {
  __shared__ double red[32];
  double s = 0.0;
  for (int i = threadIdx.x; i < D; i += blockDim.x) s = fma(r[i], z[i], s);
  const double rz = block_sum(s, red);
  const double beta = (first || !(scal[0] > 0.0)) ? 0.0 : rz / scal[0];
  for (int i = threadIdx.x; i < D; i += blockDim.x) p[i] = fma(beta, p[i], z[i]);
  __syncthreads();
  if (threadIdx.x == 0) {
    scal[0] = rz;
    if (first) scal[1] = rz;
  }
}

cudaError_t launch_shift_diag_rel(double* A, int D, double lambda, double rel, cudaStream_t st) {
  k_shift_diag_rel<<<(D + 255) / 256, 256, 0, st>>>(A, D, lambda, rel);
  return cudaGetLastError();
}

cudaError_t launch_pcg_alpha(int D, const double* p, const double* q, double* x, double* r, double* scal,
                             cudaStream_t st) {
  k_pcg_alpha<<<1, 1024, 0, st>>>(D, p, q, x, r, scal);
  return cudaGetLastError();
}

cudaError_t launch_pcg_beta(int D, const double* z, const double* r, double* p, double* scal, int first,
                            cudaStream_t st) {
  k_pcg_beta<<<1, 1024, 0, st>>>(D, z, r, p, scal, first);
  return cudaGetLastError();
}

// x = (L L^T)^-1 b; tmp holds 2*D doubles
cudaError_t launch_chol_solve_blocked(const double* L, int D, const double* b, double* x, double* tmp,
                                      cudaStream_t st) {
  double* r = tmp;
  double* y = tmp + D;
  cudaError_t e = cudaMemcpyAsync(r, b, sizeof(double) * (size_t)D, cudaMemcpyDeviceToDevice, st);
  if (e != cudaSuccess) return e;
  for (int k0 = 0; k0 < D; k0 += kTB) {
    const int nb = min(kTB, D - k0);
    const int below = D - k0 - nb;
    const int grid = max(1, min((below + 7) / 8, 296));
    k_trsv_fwd<<<grid, 256, 0, st>>>(L, D, k0, nb, r, y);
  }
  const int nblk = (D + kTB - 1) / kTB;
  for (int b0 = nblk - 1; b0 >= 0; --b0) {
    const int k0 = b0 * kTB, nb = min(kTB, D - k0);
    const int grid = max(1, min((k0 + 255) / 256, 296));
    k_trsv_bwd<<<grid, 256, 0, st>>>(L, D, k0, nb, y, x);
  }
  return cudaGetLastError();
}

// ------------------------------------------------------------------------------------
// Explicit inverse R = L^-1 of the Cholesky factor (lower, row-major D x D), so that the
// preconditioner of the conjugate-gradient solve is two dense triangular matvecs instead of
// two chains of block substitutions.  Blocked by kCB: the diagonal blocks are inverted
// independently, then block row i of R follows from the rows above it:
//   R_ij = -R_ii * sum_{k=j}^{i-1} L_ik R_kj   (j < i).
// ------------------------------------------------------------------------------------
__global__ void __launch_bounds__(kCB) k_trinv_diag(const double* __restrict__ L, int D, double* __restrict__ R) {
  __shared__ double Ld[kCB][kCB + 1], X[kCB][kCB + 1];
  const int k0 = blockIdx.x * kCB, nb = min(kCB, D - k0), t = threadIdx.x;
  for (int e = t; e < nb * nb; e += blockDim.x) {
    const int i = e / nb, j = e % nb;
    Ld[i][j] = (j <= i) ? L[(size_t)(k0 + i) * D + k0 + j] : 0.0;
  }
  __syncthreads();
  if (t < nb) {
    // column t of the inverse by forward substitution (rows below t)
    for (int i = 0; i < nb; ++i) {
      double v = (i == t) ? 1.0 : 0.0;
      for (int c = t; c < i; ++c) v -= Ld[i][c] * X[c][t];
      X[i][t] = (i < t) ? 0.0 : v / Ld[i][i];
    }
  }
  __syncthreads();
  for (int e = t; e < nb * nb; e += blockDim.x) {
    const int i = e / nb, j = e % nb;
    R[(size_t)(k0 + i) * D + k0 + j] = (j <= i) ? X[i][j] : 0.0;
  }
}

// block row bi of R, block column j = blockIdx.x < bi (16 x 16 threads, 2 x 2 outputs each)
__global__ void __launch_bounds__(256) k_trinv_row(const double* __restrict__ L, int D, int bi, double* __restrict__ R) {
  __shared__ double A[kCB][kCB + 1], B[kCB][kCB + 1];
  const int i0 = bi * kCB, ni = min(kCB, D - i0);
  const int bj = blockIdx.x, j0 = bj * kCB;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  double acc[2][2] = {{0, 0}, {0, 0}};
  for (int bk = bj; bk < bi; ++bk) {
    const int k0 = bk * kCB;
    for (int e = threadIdx.x; e < kCB * kCB; e += 256) {
      const int r = e / kCB, c = e % kCB;
      A[r][c] = (r < ni) ? L[(size_t)(i0 + r) * D + k0 + c] : 0.0;         // L_ik (k block full)
      B[r][c] = R[(size_t)(k0 + r) * D + j0 + c];                          // R_kj
    }
    __syncthreads();
#pragma unroll 8
    for (int c = 0; c < kCB; ++c) {
      const double a0 = A[ty][c], a1 = A[ty + 16][c], b0 = B[c][tx], b1 = B[c][tx + 16];
      acc[0][0] = fma(a0, b0, acc[0][0]);
      acc[0][1] = fma(a0, b1, acc[0][1]);
      acc[1][0] = fma(a1, b0, acc[1][0]);
      acc[1][1] = fma(a1, b1, acc[1][1]);
    }
    __syncthreads();
  }
  // T in B, R_ii in A; R_ij = -R_ii T
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 2; ++b) B[ty + 16 * a][tx + 16 * b] = acc[a][b];
  for (int e = threadIdx.x; e < kCB * kCB; e += 256) {
    const int r = e / kCB, c = e % kCB;
    A[r][c] = (r < ni && c < ni) ? R[(size_t)(i0 + r) * D + i0 + c] : 0.0;
  }
  __syncthreads();
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 2; ++b) {
      const int r = ty + 16 * a, c = tx + 16 * b;
      double v = 0.0;
      for (int k = 0; k <= r; ++k) v = fma(A[r][k], B[k][c], v);
      if (r < ni) R[(size_t)(i0 + r) * D + j0 + c] = -v;
    }
}

// Rt = R^T (upper part of Rt = lower part of R; the rest zero)
__global__ void k_transpose_lower(const double* __restrict__ R, int D, double* __restrict__ Rt) {
  __shared__ double tile[32][33];
  const int bx = blockIdx.x * 32, by = blockIdx.y * 32;  // source block (rows by, cols bx)
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int r = by + y, c = bx + threadIdx.x;
    tile[y][threadIdx.x] = (r < D && c < D && c <= r) ? R[(size_t)r * D + c] : 0.0;
  }
  __syncthreads();
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int r = bx + y, c = by + threadIdx.x;  // Rt[r][c] = R[c][r]
    if (r < D && c < D) Rt[(size_t)r * D + c] = tile[threadIdx.x][y];
  }
}

// y = T x for a triangular T stored densely (zeros outside the triangle): warp per row,
// columns [lo, hi) of row i with lo = upper ? i : 0, hi = upper ? D : i + 1
__global__ void __launch_bounds__(256) k_trmv(const double* __restrict__ T, int D, int upper,
                                             const double* __restrict__ x, double* __restrict__ y) {
  const int lane = threadIdx.x & 31;
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (i >= D) return;
  const int lo = upper ? i : 0, hi = upper ? D : i + 1;
  double a = 0.0;
  for (int c = lo + lane; c < hi; c += 32) a = fma(T[(size_t)i * D + c], x[c], a);
  for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
  if (lane == 0) y[i] = a;
}

// R = L^-1 and Rt = R^T (D x D each); returns the launches issued through *launches
cudaError_t launch_cholesky_inverse(const double* L, int D, double* R, double* Rt, cudaStream_t st, int* launches) {
  const int nb = (D + kCB - 1) / kCB;
  k_trinv_diag<<<nb, kCB, 0, st>>>(L, D, R);
  for (int bi = 1; bi < nb; ++bi) k_trinv_row<<<bi, 256, 0, st>>>(L, D, bi, R);
  dim3 g((D + 31) / 32, (D + 31) / 32);
  k_transpose_lower<<<g, dim3(32, 8), 0, st>>>(R, D, Rt);
  *launches = nb + 1;
  return cudaGetLastError();
}

// z = (L L^T)^-1 r = Rt (R r); tmp holds D doubles
cudaError_t launch_precond_apply(const double* R, const double* Rt, int D, const double* r, double* z, double* tmp,
                                 cudaStream_t st) {
  const unsigned blocks = (unsigned)(((long long)D * 32 + 255) / 256);
  k_trmv<<<blocks, 256, 0, st>>>(R, D, 0, r, tmp);
  k_trmv<<<blocks, 256, 0, st>>>(Rt, D, 1, tmp, z);
  return cudaGetLastError();
}

cudaError_t launch_cholesky(double* A, int D, double shift, int* info, cudaStream_t st, bool ds_update) {
  cudaError_t e = cudaMemsetAsync(info, 0, sizeof(int), st);
  if (e != cudaSuccess) return e;
  for (int k0 = 0; k0 < D; k0 += kCB) {
    const int nb = min(kCB, D - k0);
    k_potrf_diag<<<1, 256, 0, st>>>(A, D, k0, nb, shift, info);
    const int k1 = k0 + nb;
    if (k1 < D) {
      const int rows = D - k1;
      k_trsm_panel<<<(rows + 127) / 128, 128, 0, st>>>(A, D, D, k0, nb);
      const int nt = (rows + 31) / 32;
      if (ds_update)
        k_syrk_update_ds<<<nt * (nt + 1) / 2, 256, 0, st>>>(A, D, D, k0, nb, k1);
      else
        k_syrk_update<<<nt * (nt + 1) / 2, 256, 0, st>>>(A, D, D, k0, nb, k1);
    }
    // the shift applies to the diagonal blocks only once: later blocks still hold raw values
  }
  return cudaGetLastError();
}

cudaError_t launch_chol_solve(const double* L, int D, const double* b, double* x, cudaStream_t st) {
  const size_t smem = sizeof(double) * (size_t)D;
  cudaError_t e = cudaFuncSetAttribute(k_chol_solve, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k_chol_solve<<<1, 1024, smem, st>>>(L, D, D, b, x);
  return cudaGetLastError();
}

cudaError_t launch_residual(const double* G, int D, double lambda, const double* w, const double* h, double* r,
                            cudaStream_t st) {
  const long long threads = (long long)D * 32;
  k_residual<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(G, D, lambda, w, h, r);
  return cudaGetLastError();
}

cudaError_t launch_axpy(int n, double a, const double* x, double* y, cudaStream_t st) {
  k_axpy<<<(n + 255) / 256, 256, 0, st>>>(n, a, x, y);
  return cudaGetLastError();
}

}  // namespace mld
