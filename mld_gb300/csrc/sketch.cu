// Sketched preconditioner of the mixed method's wide column blocks.
//
// The normal equations (X^T W X + mu I) w = X^T W y of a wide block (the kernel block of kernel
// ridge regression, the quadratic block of QNML) are solved by conjugate gradients with matvecs
// over X itself (fit.cu).  Their preconditioner must be accurate in the directions of the small
// eigenvalues, and a Gram formed from X in low precision is not: its error is amplified by the
// square of X's condition number.  A sketch is: Y = S W^1/2 X (s x D, s = 3 D) with a sparse sign
// embedding S (zeta = 8 signed entries of 1/sqrt(zeta) per row of X) has Y^T Y = X^T W X up to a
// distortion of a few units, so the Cholesky factor R of Y^T Y + mu I makes X R^-1 well
// conditioned and CG converges in a few dozen steps.  Only the s x D sketch needs an accurate
// Gram, which is formed here in double-FP32 arithmetic on the FP32 pipe.
//
//   * the embedding: copy j of row r goes to sketch row (pi_j(r) mod s) with a hashed sign,
//     pi_j(r) = (a_j r + b_j) mod M an affine permutation; sketch row i therefore gathers rows
//     r = a_j^-1 (t - b_j) mod M for t = i, i + s, ... < M, in a fixed order (deterministic sums);
//   * k_sketch_gather: one CTA per (sketch row, 2048-column block), two rows in flight,
//     double-FP32 sums of the signed, weighted rows, the result rounded to FP32 (a relative
//     perturbation of 2^-24, far inside the preconditioner's tolerance);
//   * k_ds_gram: upper 64 x 64 tiles of Y^T Y with exact FP32 products (fmaf) and double-FP32
//     sums, written as FP64.
// With M <= s the "sketch" is W^1/2 X itself (zeta = 1, identity permutation, sign +1).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>

#include "ds.cuh"
#include "mld_internal.h"

namespace mld {

namespace {
constexpr int kGT = 64;  // Gram tile
constexpr int kGK = 16;  // sketch rows per shared-memory stage

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

long long gcd_ll(long long a, long long b) {
  while (b) {
    const long long t = a % b;
    a = b;
    b = t;
  }
  return a;
}
// a^-1 mod m (gcd(a, m) = 1)
long long inv_mod(long long a, long long m) {
  long long t = 0, nt = 1, r = m, nr = a % m;
  while (nr) {
    const long long q = r / nr;
    long long x = t - q * nt;
    t = nt;
    nt = x;
    x = r - q * nr;
    r = nr;
    nr = x;
  }
  return t < 0 ? t + m : t;
}
}  // namespace

// sqrt(w_r) / sqrt(zeta) in FP32
__global__ void k_sketch_scale(const double* __restrict__ w, long long M, double inv_zeta, float* __restrict__ sw) {
  const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (r < M) sw[r] = (float)sqrt(w[r] * inv_zeta);
}

// Y[i, cb : cb + 256 CPT] = sum over the rows r of sketch row i of sign(r, j) sw[r] X[r, c0 + cb ...],
// cb = 256 CPT blockIdx.y: a CTA per (sketch row, column block)
template <int CPT>
__global__ void __launch_bounds__(256) k_sketch_gather(const float* __restrict__ X, int ldx, int c0, int D,
                                                       const float* __restrict__ sw, SketchParams P,
                                                       float* __restrict__ Y) {
  const int i = blockIdx.x;
  const int cb = blockIdx.y * 256 * CPT;
  const int lane = threadIdx.x & 31;
  float sh[CPT], sl[CPT];
#pragma unroll
  for (int u = 0; u < CPT; ++u) sh[u] = sl[u] = 0.f;
  for (int j = 0; j < P.zeta; ++j) {
    const long long cnt = i < P.M ? (P.M - 1 - i) / P.s + 1 : 0;  // t = i + k s < M
    for (long long k0 = 0; k0 < cnt; k0 += 32) {
      // lane l resolves entry k0 + l: its row and signed scale
      long long r = 0;
      float sc = 0.f;
      if (k0 + lane < cnt) {
        const long long t = i + (k0 + lane) * P.s;
        long long d = t - P.b[j];
        d %= P.M;
        if (d < 0) d += P.M;
        r = (long long)(((unsigned long long)P.ainv[j] * (unsigned long long)d) % (unsigned long long)P.M);
        const uint64_t h = mix64(P.seed ^ ((uint64_t)r * 8u + (uint64_t)j));
        sc = (P.zeta == 1 || (h & 1u)) ? sw[r] : -sw[r];
      }
      const int ne = (int)min(32LL, cnt - k0);
      // two rows per step: both rows' loads are in flight before either is added (an odd last
      // entry pairs with a zero-scaled copy of itself)
      for (int e = 0; e < ne; e += 2) {
        const int e2 = min(e + 1, ne - 1);
        const long long ra = __shfl_sync(0xffffffffu, r, e), rb = __shfl_sync(0xffffffffu, r, e2);
        const float sa = __shfl_sync(0xffffffffu, sc, e);
        const float sb = e + 1 < ne ? __shfl_sync(0xffffffffu, sc, e2) : 0.f;
        const float* xa = X + ra * ldx + c0;
        const float* xb = X + rb * ldx + c0;
        float va[CPT], vb[CPT];
#pragma unroll
        for (int u = 0; u < CPT; ++u) {
          const int c = cb + threadIdx.x + 256 * u;
          va[u] = c < D ? xa[c] : 0.f;
          vb[u] = c < D ? xb[c] : 0.f;
        }
#pragma unroll
        for (int u = 0; u < CPT; ++u) {
          float t, er;
          two_sum(sh[u], va[u] * sa, t, er);
          sh[u] = t;
          sl[u] += er;
          two_sum(sh[u], vb[u] * sb, t, er);
          sh[u] = t;
          sl[u] += er;
        }
      }
    }
  }
#pragma unroll
  for (int u = 0; u < CPT; ++u) {
    const int c = cb + threadIdx.x + 256 * u;
    if (c < D) Y[(size_t)i * D + c] = sh[u] + sl[u];
  }
}

// G[i, j] (i <= j, 64 x 64 tiles of the upper triangle) = sum_k Y[k, i] Y[k, j] in double-FP32
__global__ void __launch_bounds__(256) k_ds_gram(const float* __restrict__ Y, int s, int D, int nt,
                                                 double* __restrict__ G) {
  __shared__ float As[kGK][kGT], Bs[kGK][kGT];
  int t = blockIdx.x, ti = 0;
  while (t >= nt - ti) {
    t -= nt - ti;
    ++ti;
  }
  const int tj = ti + t;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  float hi[4][4], lo[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) hi[a][b] = lo[a][b] = 0.f;
  for (int k0 = 0; k0 < s; k0 += kGK) {
    for (int e = threadIdx.x; e < kGK * kGT; e += 256) {
      const int kk = e / kGT, c = e - kk * kGT;
      const int k = k0 + kk, ci = ti * kGT + c, cj = tj * kGT + c;
      As[kk][c] = (k < s && ci < D) ? Y[(size_t)k * D + ci] : 0.f;
      Bs[kk][c] = (k < s && cj < D) ? Y[(size_t)k * D + cj] : 0.f;
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < kGK; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        a[q] = As[kk][ty + 16 * q];
        b[q] = Bs[kk][tx + 16 * q];
      }
#pragma unroll
      for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const float pr = a[p] * b[q];
          const float pe = fmaf(a[p], b[q], -pr);  // exact product pr + pe
          float sum, er;
          two_sum(hi[p][q], pr, sum, er);
          hi[p][q] = sum;
          lo[p][q] += er + pe;
        }
    }
    __syncthreads();
  }
#pragma unroll
  for (int p = 0; p < 4; ++p)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int i = ti * kGT + ty + 16 * p, j = tj * kGT + tx + 16 * q;
      if (i < D && j < D && j >= i) G[(size_t)i * D + j] = (double)hi[p][q] + (double)lo[p][q];
    }
}

SketchParams sketch_params(long long M, int D, uint64_t seed) {
  SketchParams P{};
  P.M = M;
  P.seed = seed;
  const long long s3 = 3LL * D;
  if (M <= s3) {
    P.zeta = 1;
    P.s = (int)M;
    P.a[0] = P.ainv[0] = 1;
    P.b[0] = 0;
    return P;
  }
  P.zeta = kSketchZeta;
  P.s = (int)s3;
  uint64_t st = seed;
  auto next = [&]() {
    st += 0x9E3779B97F4A7C15ull;
    uint64_t z = st;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  };
  for (int j = 0; j < P.zeta; ++j) {
    long long a = 0;
    do {
      a = (long long)(next() % (uint64_t)M);
    } while (a < 2 || gcd_ll(a, M) != 1);
    P.a[j] = a;
    P.ainv[j] = inv_mod(a, M);
    P.b[j] = (long long)(next() % (uint64_t)M);
  }
  return P;
}

size_t sketch_workspace_bytes(long long M, int D) {
  const long long s = std::min<long long>(M, 3LL * D);
  return sizeof(float) * ((size_t)M + (size_t)s * D) + 512;
}

cudaError_t launch_sketch_gram(const float* X, int ldx, int c0, int D, const double* w, long long M,
                               const SketchParams& P, void* ws, double* G, cudaStream_t st, int* launches) {
  float* sw = static_cast<float*>(ws);
  float* Y = sw + ((M + 63) / 64 * 64);
  k_sketch_scale<<<(unsigned)((M + 255) / 256), 256, 0, st>>>(w, M, 1.0 / P.zeta, sw);
  constexpr int kCPT = 8;  // columns per thread: 2048 per CTA
  const dim3 gg((unsigned)P.s, (unsigned)((D + 256 * kCPT - 1) / (256 * kCPT)));
  k_sketch_gather<kCPT><<<gg, 256, 0, st>>>(X, ldx, c0, D, sw, P, Y);
  const int nt = (D + kGT - 1) / kGT;
  const long long ntile = (long long)nt * (nt + 1) / 2;
  k_ds_gram<<<(unsigned)ntile, 256, 0, st>>>(Y, P.s, D, nt, G);
  *launches = 3;
  return launch_symmetrize(G, D, st);
}

}  // namespace mld
