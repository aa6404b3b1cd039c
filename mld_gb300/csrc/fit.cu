// Design-row labels, weighted Gram / right-hand side, ridge solve and predictions.
//
//   phi = X^T W X + lambda*I (lambda < 0 -> 0; the intercept column is penalised too),
//   rhs = X^T W y                        -- MILADY src/mld/parameters.F90:1018-1099
//   w   = minimum-norm solution of phi w = rhs with singular values <= rcond*s_max dropped
//         (rcond < 0 -> machine precision), the semantics of LAPACK dgelsd as called by
//         serial_lsystem_by_svd (src/mld/stats_tools.F90:1153-1213)
//   predictions  X w                     -- src/mld/mld.F90:40-86,944-1020
// The symmetric solve uses a parallel cyclic Jacobi eigen-decomposition in one CTA (FP64):
// for a symmetric positive semi-definite phi its eigenvalues are its singular values.
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>
#include <type_traits>

#include "ds.cuh"
#include "mld_internal.h"
#include "ptx.cuh"

namespace mld {

// ------------------------------------------------------------------------------------
// row labels / weights and the constant column of the energy rows
// ------------------------------------------------------------------------------------
template <typename T>
__global__ void k_rows_prep(int S, const int* __restrict__ atom_start, const long long* __restrict__ rowE,
                            const long long* __restrict__ rowF, const long long* __restrict__ rowS,
                            const double* __restrict__ E, const double* __restrict__ F, const double* __restrict__ Sv,
                            const double* __restrict__ wefs, int D, T* __restrict__ X, double* __restrict__ y,
                            double* __restrict__ wrow, int* __restrict__ kind) {
  const int s = blockIdx.x;
  if (s >= S) return;
  const int a0 = atom_start[s], nat = atom_start[s + 1] - a0;
  if (rowE[s] >= 0 && threadIdx.x == 0) {
    long long r = rowE[s];
    X[r * D] = (T)nat;
    y[r] = E[s];
    wrow[r] = wefs[3 * s];
    kind[r] = 0;
  }
  if (rowF[s] >= 0) {
    for (int i = threadIdx.x; i < 3 * nat; i += blockDim.x) {
      long long r = rowF[s] + i;
      y[r] = F[3 * (size_t)a0 + i];
      wrow[r] = wefs[3 * s + 1];
      kind[r] = 1;
    }
  }
  if (rowS[s] >= 0 && threadIdx.x < 6) {
    long long r = rowS[s] + threadIdx.x;
    y[r] = Sv[6 * s + threadIdx.x];
    wrow[r] = wefs[3 * s + 2];
    kind[r] = 2;
  }
}

// ------------------------------------------------------------------------------------
// Gram:  G += X^T diag(w) X over a chunk of rows, 32x32 output tiles, FP64 accumulation.
// ------------------------------------------------------------------------------------
constexpr int GT = 32;   // tile edge
constexpr int GR = 32;   // rows per smem stage

// part != nullptr: each CTA stores its 32 x 32 partial tile at part[(blockIdx.y * npairs +
// blockIdx.x) * 1024] for k_gram_reduce (fixed summation order); else atomics into G.
template <typename T>
__global__ void __launch_bounds__(256) k_gram(const T* __restrict__ X, int ldx, const double* __restrict__ w,
                                              long long M, int D, long long rows_per_block, double* __restrict__ G,
                                              double* __restrict__ part) {
  const int nt = (D + GT - 1) / GT;
  // decode upper-triangular tile pair from blockIdx.x
  int t = blockIdx.x, ti = 0;
  while (t >= nt - ti) {
    t -= nt - ti;
    ++ti;
  }
  const int tj = ti + t;
  const int i0 = ti * GT, j0 = tj * GT;
  const long long r0 = (long long)blockIdx.y * rows_per_block;
  const long long r1 = min(M, r0 + rows_per_block);
  __shared__ double sa[GR][GT + 1];
  __shared__ double sb[GR][GT + 1];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;  // 16x16 threads, 2x2 outputs each
  double acc[2][2] = {{0, 0}, {0, 0}};
  for (long long rb = r0; rb < r1; rb += GR) {
    for (int e = threadIdx.x; e < GR * GT; e += 256) {
      const int rr = e / GT, cc = e % GT;
      const long long r = rb + rr;
      double va = 0, vb = 0;
      if (r < r1) {
        const double wr = w[r];
        if (i0 + cc < D) va = (double)X[r * ldx + i0 + cc] * wr;
        if (j0 + cc < D) vb = (double)X[r * ldx + j0 + cc];
      }
      sa[rr][cc] = va;
      sb[rr][cc] = vb;
    }
    __syncthreads();
#pragma unroll 8
    for (int rr = 0; rr < GR; ++rr) {
      const double a0 = sa[rr][ty], a1 = sa[rr][ty + 16];
      const double b0 = sb[rr][tx], b1 = sb[rr][tx + 16];
      acc[0][0] = fma(a0, b0, acc[0][0]);
      acc[0][1] = fma(a0, b1, acc[0][1]);
      acc[1][0] = fma(a1, b0, acc[1][0]);
      acc[1][1] = fma(a1, b1, acc[1][1]);
    }
    __syncthreads();
  }
  if (part) {
    double* pt = part + ((size_t)blockIdx.y * gridDim.x + blockIdx.x) * (GT * GT);
    for (int a = 0; a < 2; ++a)
      for (int b = 0; b < 2; ++b) pt[(ty + 16 * a) * GT + tx + 16 * b] = acc[a][b];
    return;
  }
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 2; ++b) {
      const int i = i0 + ty + 16 * a, j = j0 + tx + 16 * b;
      if (i < D && j < D && (ti != tj || i <= j)) atomicAdd(&G[(size_t)i * D + j], acc[a][b]);
    }
}

// G (upper triangle of each tile pair) = sum over the row chunks of the partial tiles, in chunk
// order; one CTA per tile pair, one thread per element.
__global__ void __launch_bounds__(GT * GT) k_gram_reduce(const double* __restrict__ part, int npairs, int chunks, int D,
                                                         double* __restrict__ G) {
  const int nt = (D + GT - 1) / GT;
  int t = blockIdx.x, ti = 0;
  while (t >= nt - ti) {
    t -= nt - ti;
    ++ti;
  }
  const int tj = ti + t;
  const int e = threadIdx.x, i = ti * GT + e / GT, j = tj * GT + e % GT;
  if (i >= D || j >= D || (ti == tj && i > j)) return;
  double sum = 0.0;
  for (int c = 0; c < chunks; ++c) sum += part[((size_t)c * npairs + blockIdx.x) * (GT * GT) + e];
  G[(size_t)i * D + j] = sum;
}

// q[c] = sum over the row blocks of part[b * D + c] in a fixed order: one warp per column, lane
// l adds the blocks l, l + 32, l + 64, ... in turn, then a fixed xor tree over the lanes.
__global__ void k_colsum_reduce(const double* __restrict__ part, long long nrb, int D, double* __restrict__ q) {
  const int c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (c >= D) return;  // whole warps leave together
  double sum = 0.0;
  for (long long b = lane; b < nrb; b += 32) sum += part[(size_t)b * D + c];
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
  if (lane == 0) q[c] = sum;
}
constexpr int kColsumColsPerBlock = 8;  // warps (columns) per block of k_colsum_reduce

__global__ void k_symmetrize(double* G, int D) {
  const int i = blockIdx.x, j = threadIdx.x;
  for (int jj = j; jj < D; jj += blockDim.x)
    if (jj < i) G[(size_t)i * D + jj] = G[(size_t)jj * D + i];
}

namespace {
long long rows_per_cta(long long M, int ncb, int nsm);
// row chunks of the FP64 Gram: enough CTAs to fill the machine (~8 per SM overall)
void gram_chunks(long long M, int D, int nsm, int* npairs, long long* chunks, long long* rpb) {
  const int nt = (D + GT - 1) / GT;
  *npairs = nt * (nt + 1) / 2;
  long long c = (long long)nsm * 8 / *npairs;
  if (c < 1) c = 1;
  long long r = (std::max<long long>(M, 1) + c - 1) / c;
  r = ((r + GR - 1) / GR) * GR;
  c = (std::max<long long>(M, 1) + r - 1) / r;
  if (c > 65535) {
    c = 65535;
    r = (M + c - 1) / c;
  }
  *chunks = c;
  *rpb = r;
}
int device_sms() {
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  return nsm;
}
}  // namespace

size_t gram_workspace_doubles(long long M, int D) {
  const int nsm = device_sms();
  int npairs = 0;
  long long chunks = 0, rpb = 0;
  gram_chunks(M, D, nsm, &npairs, &chunks, &rpb);
  const int ncb = (D + 255) / 256;
  const long long nrb = (std::max<long long>(M, 1) + rows_per_cta(M, ncb, nsm) - 1) / rows_per_cta(M, ncb, nsm);
  return std::max<size_t>((size_t)chunks * npairs * GT * GT, (size_t)nrb * D);
}

template <typename T>
cudaError_t launch_gram(const T* X, int ldx, const double* w, const double* y, long long M, int D, double* G,
                        double* h, cudaStream_t st, double* ws) {
  cudaError_t e = cudaMemsetAsync(G, 0, sizeof(double) * (size_t)D * D, st);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(h, 0, sizeof(double) * (size_t)D, st);
  if (e != cudaSuccess) return e;
  if (M == 0) return cudaSuccess;
  const int nsm = device_sms();
  int npairs = 0;
  long long chunks = 0, rpb = 0;
  gram_chunks(M, D, nsm, &npairs, &chunks, &rpb);
  k_gram<T><<<dim3(npairs, (unsigned)chunks), 256, 0, st>>>(X, ldx, w, M, D, rpb, G, ws);
  if (ws) k_gram_reduce<<<npairs, GT * GT, 0, st>>>(ws, npairs, (int)chunks, D, G);
  e = launch_rhs<T>(X, ldx, w, y, M, D, h, nsm, st, nullptr, ws);
  if (e != cudaSuccess) return e;
  k_symmetrize<<<D, 128, 0, st>>>(G, D);
  return cudaGetLastError();
}

// q[c] = sum_r w[r] v[r] X[r][c] (FP64 accumulation).  Columns in blocks of 256 (8 per lane,
// blockIdx.y), design rows in chunks (blockIdx.x) walked by the 8 warps; per-CTA partial sums
// are reduced in shared memory and added to q with one atomic per column.
template <typename T>
__global__ void __launch_bounds__(256) k_xtv(const T* __restrict__ X, int ldx, int D, const double* __restrict__ w,
                                             const double* __restrict__ v, long long M, long long rpb,
                                             double* __restrict__ q, double* __restrict__ part) {
  __shared__ double red[8][256];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int cb = blockIdx.y * 256;
  const long long r0 = (long long)blockIdx.x * rpb, r1 = min(M, r0 + rpb);
  double acc[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) acc[k] = 0.0;
  for (long long r = r0 + warp; r < r1; r += 8) {
    const double s = w[r] * v[r];
    const T* xr = X + r * ldx + cb;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const int c = lane + 32 * k;
      if (cb + c < D) acc[k] = fma((double)xr[c], s, acc[k]);
    }
  }
#pragma unroll
  for (int k = 0; k < 8; ++k) red[warp][lane + 32 * k] = acc[k];
  __syncthreads();
  double sum = 0.0;
#pragma unroll
  for (int w8 = 0; w8 < 8; ++w8) sum += red[w8][threadIdx.x];
  if (cb + threadIdx.x < D) {
    if (part) part[(size_t)blockIdx.x * D + cb + threadIdx.x] = sum;
    else if (sum != 0.0) atomicAdd(&q[cb + threadIdx.x], sum);
  }
}

// Normal-equation matvec of a narrow block (D <= 32*NK <= 256) in one pass over X:
// q = sum_r w[r] (x_r . p) x_r, the row held in registers between the dot and the update.
template <int NK>
__global__ void __launch_bounds__(256) k_normal_matvec_narrow(const float* __restrict__ X, int ldx, int D,
                                                              const float2* __restrict__ wds,
                                                              const double* __restrict__ p, long long M, long long rpb,
                                                              double* __restrict__ q, double* __restrict__ part) {
  __shared__ double red[8][32 * NK];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float ph[NK], pl[NK], ah[NK], al[NK];
#pragma unroll
  for (int k = 0; k < NK; ++k) {
    const int c = lane + 32 * k;
    ds_split(c < D ? p[c] : 0.0, ph[k], pl[k]);
    ah[k] = al[k] = 0.f;
  }
  // four design rows per warp step keep four row loads in flight
  constexpr int RU = 4;
  const long long r0 = (long long)blockIdx.x * rpb, r1 = min(M, r0 + rpb);
  int step = 0;
  for (long long rb = r0 + RU * warp; rb < r1; rb += RU * 8, ++step) {
    float x[RU][NK];
    float dh[RU], dl[RU];
#pragma unroll
    for (int u = 0; u < RU; ++u) {
      const long long r = rb + u;
      const float* xr = X + min(r, r1 - 1) * ldx;
#pragma unroll
      for (int k = 0; k < NK; ++k) {
        const int c = lane + 32 * k;
        x[u][k] = (c < D && r < r1) ? xr[c] : 0.f;
      }
    }
#pragma unroll
    for (int u = 0; u < RU; ++u) {
      dh[u] = dl[u] = 0.f;
#pragma unroll
      for (int k = 0; k < NK; ++k) ds_fma(dh[u], dl[u], x[u][k], ph[k], pl[k]);
    }
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
      for (int u = 0; u < RU; ++u) {
        const float oh = __shfl_xor_sync(0xffffffffu, dh[u], o), ol = __shfl_xor_sync(0xffffffffu, dl[u], o);
        ds_add(dh[u], dl[u], oh, ol);
      }
    }
#pragma unroll
    for (int u = 0; u < RU; ++u) {
      const long long r = rb + u;
      // s = w_r * d as a pair (zero past the chunk)
      const float2 wv = r < r1 ? wds[r] : make_float2(0.f, 0.f);
      const float wh = wv.x, wl = wv.y;
      const float sp = dh[u] * wh;
      const float se = fmaf(dh[u], wl, fmaf(dl[u], wh, fmaf(dh[u], wh, -sp)));
      const float sh = sp + se;
      const float sl = se - (sh - sp);
#pragma unroll
      for (int k = 0; k < NK; ++k) ds_fma(ah[k], al[k], x[u][k], sh, sl);
    }
    if ((step & 63) == 63) {
#pragma unroll
      for (int k = 0; k < NK; ++k) ds_norm(ah[k], al[k]);
    }
  }
#pragma unroll
  for (int k = 0; k < NK; ++k) red[warp][lane + 32 * k] = (double)ah[k] + (double)al[k];
  __syncthreads();
  for (int c = threadIdx.x; c < 32 * NK; c += 256) {
    double sum = 0.0;
#pragma unroll
    for (int w8 = 0; w8 < 8; ++w8) sum += red[w8][c];
    if (c < D) {
      if (part) part[(size_t)blockIdx.x * D + c] = sum;  // reduced in block order
      else if (sum != 0.0) atomicAdd(&q[c], sum);
    }
  }
}

// sv[r] = w[r] * (x_r . p) as a double-FP32 pair (warp per design row)
__global__ void __launch_bounds__(256) k_xp_ds(const float* __restrict__ X, int ldx, int D,
                                               const double* __restrict__ w, const double* __restrict__ p, long long M,
                                               float2* __restrict__ sv) {
  extern __shared__ float pp[];  // [2][D]
  for (int c = threadIdx.x; c < D; c += blockDim.x) ds_split(p[c], pp[c], pp[D + c]);
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const long long nw = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long r = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < M; r += nw) {
    const float* xr = X + r * ldx;
    float dh = 0.f, dl = 0.f;
    for (int c = lane; c < D; c += 32) ds_fma(dh, dl, xr[c], pp[c], pp[D + c]);
    for (int o = 16; o > 0; o >>= 1) {
      const float oh = __shfl_xor_sync(0xffffffffu, dh, o), ol = __shfl_xor_sync(0xffffffffu, dl, o);
      ds_add(dh, dl, oh, ol);
    }
    if (lane == 0) {
      const double s = ((double)dh + (double)dl) * w[r];
      float h, l;
      ds_split(s, h, l);
      sv[r] = make_float2(h, l);
    }
  }
}

// wds[r] = w[r] as a double-FP32 pair
__global__ void k_w_ds(const double* __restrict__ w, long long M, float2* __restrict__ wds) {
  const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= M) return;
  float h, l;
  ds_split(w[r], h, l);
  wds[r] = make_float2(h, l);
}

// sv[r] = w[r] * y[r] as a double-FP32 pair
__global__ void k_wy_ds(const double* __restrict__ w, const double* __restrict__ y, long long M,
                        float2* __restrict__ sv) {
  const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= M) return;
  float h, l;
  ds_split(w[r] * y[r], h, l);
  sv[r] = make_float2(h, l);
}

// q[c] = sum_r sv[r] X[r][c] with double-FP32 accumulation; columns in blocks of 256
// (blockIdx.y), design rows in chunks (blockIdx.x) walked by the 8 warps.
__global__ void __launch_bounds__(256) k_xtv_ds(const float* __restrict__ X, int ldx, int D,
                                                const float2* __restrict__ sv, long long M, long long rpb,
                                                double* __restrict__ q, double* __restrict__ part) {
  __shared__ double red[8][256];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int cb = blockIdx.y * 256;
  const long long r0 = (long long)blockIdx.x * rpb, r1 = min(M, r0 + rpb);
  float ah[8], al[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) ah[k] = al[k] = 0.f;
  for (long long r = r0 + warp; r < r1; r += 8) {
    const float2 s = sv[r];
    const float* xr = X + r * ldx + cb;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const int c = lane + 32 * k;
      if (cb + c < D) ds_fma(ah[k], al[k], xr[c], s.x, s.y);
    }
    if (((r - r0) & 511) == 504) {
#pragma unroll
      for (int k = 0; k < 8; ++k) ds_norm(ah[k], al[k]);
    }
  }
#pragma unroll
  for (int k = 0; k < 8; ++k) red[warp][lane + 32 * k] = (double)ah[k] + (double)al[k];
  __syncthreads();
  double sum = 0.0;
#pragma unroll
  for (int w8 = 0; w8 < 8; ++w8) sum += red[w8][threadIdx.x];
  if (cb + threadIdx.x < D) {
    if (part) part[(size_t)blockIdx.x * D + cb + threadIdx.x] = sum;
    else if (sum != 0.0) atomicAdd(&q[cb + threadIdx.x], sum);
  }
}

// ------------------------------------------------------------------------------------
// Normal-equation matvec of a wide block (D > 256) in one pass over X.  Design rows stream
// through a ring of shared-memory stages by 1-D bulk copies issued from one producer thread.
// Sixteen consumer warps own the columns c = tid + 512 j (j < CPT).  Per step of kWRows rows:
//   * each thread forms FP32 partial dots of its columns with p (rounded to FP32);
//   * warps reduce them, one warp per row sums the sixteen warp partials and scales by w_r,
//     giving t_r = w_r (x_r . p);
//   * each thread adds x_rc t_r to FP32 column sums, which are moved into double-FP32 sums
//     (TwoSum) every kWFlushSteps steps.
// FP32 arithmetic on chunks (12 columns of a dot, 8 rows of a column sum) with double-FP32
// between chunks keeps the relative error near 1e-7 at about three FP32 operations per element
// and leaves the FP64 pipe, 1/64 of the FP32 rate on this GPU, out of the loop.  The
// blocks that take this path (quadratic and kernel columns) are so ill-conditioned that the
// iteration stops at relative residuals far above 1e-7; the narrow linear blocks keep
// double-FP32 (k_normal_matvec_narrow).  A stage is `stride` floats, at least 512 * CPT past
// the row's first column: the tail beyond the copied row stays zero, so the inner loops carry
// no bounds tests (p is zero there and those column sums are dropped).
// Every wait is bounded: on expiry the CTA sets *err and leaves the loop uniformly.
// ------------------------------------------------------------------------------------
constexpr int kWConsumers = 512;
constexpr int kWWarps = kWConsumers / 32;
constexpr int kWRows = 4;        // design rows per consumer step
constexpr int kWFlushSteps = 2;  // steps between FP32 -> FP64 moves of the column sums
constexpr int kWMaxStages = 16;
constexpr int kWChunks = 8;      // bulk copies per design row
constexpr int kWThreads = kWConsumers + 32;

template <int CPT>
__global__ void __launch_bounds__(kWThreads, 1)
    k_normal_matvec_wide(const float* __restrict__ X, long long ldx, int c0, int D, const float2* __restrict__ wds,
                         const double* __restrict__ p, long long M, long long rpb, int rowf, int stride, int stages,
                         double* __restrict__ q, double* __restrict__ qpart, int* __restrict__ err) {
  extern __shared__ __align__(128) unsigned char wsm[];
  float* rows = reinterpret_cast<float*>(wsm);                                 // stages * stride
  float* part = rows + (size_t)stages * stride;                                // stages * kWWarps
  float* tv = part + stages * kWWarps;                                         // stages
  uint64_t* full = reinterpret_cast<uint64_t*>(tv + stages + (stages & 1));
  uint64_t* empty = full + stages;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int a0 = c0 & ~3, off = c0 - a0;
  const uint32_t bytes = (uint32_t)rowf * 4u;
  const long long r0 = (long long)blockIdx.x * rpb;
  const long long nr = min(M, r0 + rpb) - r0;
  if (nr <= 0) return;
  for (int e = tid; e < stages * stride; e += blockDim.x) rows[e] = 0.f;
  if (tid == 0) {
    for (int s = 0; s < stages; ++s) {
      ptx::mbar_init(&full[s], 1);
      ptx::mbar_init(&empty[s], kWWarps);
    }
    ptx::mbar_init_fence();
  }
  // the zero tails must be visible to the async proxy before the first bulk copy lands
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  __syncthreads();
  if (warp == kWWarps) {
    // producer warp: each row goes in kWChunks bulk copies issued by as many lanes, so that
    // several copies per row are in flight at once
    const uint32_t cb = ((bytes / kWChunks) + 15u) & ~15u;
    long long issued = 0;
    for (long long k = 0; k < nr; ++k) {
      const int s = (int)(k % stages);
      int okw = 1;
      if (k >= stages && lane == 0) okw = ptx::mbar_wait(&empty[s], (uint32_t)(((k / stages) - 1) & 1)) ? 1 : 0;
      okw = __shfl_sync(0xffffffffu, okw, 0);
      if (!okw) {
        if (lane == 0) atomicExch(err, 1);
        break;
      }
      if (lane == 0) ptx::mbar_expect_tx(&full[s], bytes);
      __syncwarp();
      const uint32_t o = (uint32_t)lane * cb;
      if (lane < kWChunks && o < bytes)
        ptx::bulk_load(reinterpret_cast<char*>(rows + (size_t)s * stride) + o,
                       reinterpret_cast<const char*>(X + (r0 + k) * ldx + a0) + o, min(cb, bytes - o), &full[s]);
      issued = k + 1;
    }
    if (lane == 0)
      for (long long k = max(0LL, issued - stages); k < issued; ++k)
        ptx::mbar_wait(&full[k % stages], (uint32_t)((k / stages) & 1));
    return;
  }
  // consumers
  float pf[CPT], acc[CPT], sh[CPT], sl[CPT];
#pragma unroll
  for (int j = 0; j < CPT; ++j) {
    const int c = tid + kWConsumers * j;
    pf[j] = c < D ? (float)p[c] : 0.f;
    acc[j] = sh[j] = sl[j] = 0.f;
  }
  long long step = 0;
  for (long long k = 0; k < nr; k += kWRows, ++step) {
    const int nv = (int)min((long long)kWRows, nr - k);
    // the row weight this warp needs after the barrier, loaded before the dots
    const float2 wv = warp < nv ? wds[r0 + k + warp] : make_float2(0.f, 0.f);
    const float* rp[kWRows];
    bool ok = true;
#pragma unroll
    for (int r = 0; r < kWRows; ++r) {
      const int s = (int)((k + r) % stages);
      rp[r] = rows + s * stride + off + tid;
      if (r < nv) ok = ok && ptx::mbar_wait(&full[s], (uint32_t)(((k + r) / stages) & 1));
    }
    float d[kWRows];
#pragma unroll
    for (int r = 0; r < kWRows; ++r) d[r] = 0.f;
    if (ok) {
#pragma unroll
      for (int j = 0; j < CPT; ++j)
#pragma unroll
        for (int r = 0; r < kWRows; ++r) d[r] = fmaf(rp[r][kWConsumers * j], pf[j], d[r]);
    }
#pragma unroll
    for (int r = 0; r < kWRows; ++r)
      for (int o = 16; o > 0; o >>= 1) d[r] += __shfl_xor_sync(0xffffffffu, d[r], o);
    if (lane == 0) {
#pragma unroll
      for (int r = 0; r < kWRows; ++r) part[(int)((k + r) % stages) * kWWarps + warp] = d[r];
    }
    int any_fail;
    asm volatile(
        "{\n .reg .pred pf, pr;\n setp.eq.u32 pf, %1, 0;\n bar.red.or.pred pr, 1, %2, pf;\n selp.u32 %0, 1, 0, pr;\n}\n"
        : "=r"(any_fail)
        : "r"((unsigned)ok), "n"(kWConsumers));
    if (any_fail) {
      if (tid == 0) atomicExch(err, 1);
      break;
    }
    // warp r sums the sixteen slices of row r and scales by w_r
    if (warp < kWRows) {
      const int sw = (int)((k + warp) % stages);
      float v = (lane < kWWarps && warp < nv) ? part[sw * kWWarps + lane] : 0.f;
      for (int o = 8; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) tv[sw] = v * wv.x + v * wv.y;
    }
    asm volatile("bar.sync 2, %0;\n" ::"n"(kWConsumers));
    float th[kWRows];
#pragma unroll
    for (int r = 0; r < kWRows; ++r) th[r] = tv[(int)((k + r) % stages)];
#pragma unroll
    for (int j = 0; j < CPT; ++j)
#pragma unroll
      for (int r = 0; r < kWRows; ++r) acc[j] = fmaf(rp[r][kWConsumers * j], th[r], acc[j]);
    // every stage of this step is read: release them to the producer
    __syncwarp();
    if (lane == 0) {
#pragma unroll
      for (int r = 0; r < kWRows; ++r)
        if (r < nv) ptx::mbar_arrive(&empty[(int)((k + r) % stages)]);
    }
    if ((step % kWFlushSteps) == kWFlushSteps - 1) {
      // chunk sums into double-FP32 column sums (TwoSum on the FP32 pipe)
#pragma unroll
      for (int j = 0; j < CPT; ++j) {
        float t, e;
        two_sum(sh[j], acc[j], t, e);
        sh[j] = t;
        sl[j] += e;
        acc[j] = 0.f;
      }
    }
  }
#pragma unroll
  for (int j = 0; j < CPT; ++j) {
    const int c = tid + kWConsumers * j;
    // partial column sums of this block, reduced in block order by k_colsum_reduce
    if (c < D) qpart[(size_t)blockIdx.x * D + c] = (double)sh[j] + (double)sl[j] + (double)acc[j];
  }
}

namespace {
// design-row chunk per CTA so that about 8 CTAs per SM run over all column blocks
long long rows_per_cta(long long M, int ncb, int nsm) {
  long long ctas = std::max<long long>(1, (long long)nsm * 8 / std::max(1, ncb));
  long long rpb = (M + ctas - 1) / ctas;
  return std::max<long long>(64, rpb);
}
}  // namespace

// h = X^T diag(w) y: double-FP32 accumulation for an FP32 X when `sv` (M float2 of scratch) is
// given, FP64 accumulation otherwise
template <typename T>
cudaError_t launch_rhs(const T* X, int ldx, const double* w, const double* y, long long M, int D, double* h,
                       int nsm, cudaStream_t st, float2* sv, double* ws) {
  cudaError_t e = cudaMemsetAsync(h, 0, sizeof(double) * (size_t)D, st);
  if (e != cudaSuccess || M == 0) return e;
  const int ncb = (D + 255) / 256;
  const long long rpb = rows_per_cta(M, ncb, nsm);
  const long long nrb = (M + rpb - 1) / rpb;
  bool done = false;
  if constexpr (std::is_same<T, float>::value) {
    if (sv) {
      k_wy_ds<<<(unsigned)((M + 255) / 256), 256, 0, st>>>(w, y, M, sv);
      k_xtv_ds<<<dim3((unsigned)nrb, (unsigned)ncb), 256, 0, st>>>(X, ldx, D, sv, M, rpb, h, ws);
      done = true;
    }
  }
  if (!done) k_xtv<T><<<dim3((unsigned)nrb, (unsigned)ncb), 256, 0, st>>>(X, ldx, D, w, y, M, rpb, h, ws);
  if (ws)
    k_colsum_reduce<<<(D + kColsumColsPerBlock - 1) / kColsumColsPerBlock, 32 * kColsumColsPerBlock, 0, st>>>(
        ws, nrb, D, h);
  return cudaGetLastError();
}

// out = sum_r w[r] y[r]^2: block b writes its partial to part[b]; k_sum_reduce adds them in order
__global__ void __launch_bounds__(256) k_weighted_sumsq(const double* __restrict__ w, const double* __restrict__ y,
                                                        long long M, double* __restrict__ part) {
  __shared__ double red[8];
  double a = 0.0;
  for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < M; r += (long long)gridDim.x * blockDim.x)
    a = fma(w[r] * y[r], y[r], a);
  for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = a;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < 8; ++k) t += red[k];
    part[blockIdx.x] = t;
  }
}

constexpr int kSumsqBlocks = kSumsqBlocksMax;

__global__ void k_sum_reduce(const double* __restrict__ part, int n, double* __restrict__ out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double t = 0.0;
  for (int b = 0; b < n; ++b) t += part[b];
  *out = t;
}

cudaError_t launch_weighted_sumsq(const double* w, const double* y, long long M, double* out, double* ws,
                                  cudaStream_t st) {
  if (M == 0) return cudaMemsetAsync(out, 0, sizeof(double), st);
  const unsigned blocks = (unsigned)std::min<long long>((M + 255) / 256, kSumsqBlocks);
  k_weighted_sumsq<<<blocks, 256, 0, st>>>(w, y, M, ws);
  k_sum_reduce<<<1, 32, 0, st>>>(ws, (int)blocks, out);
  return cudaGetLastError();
}

cudaError_t launch_split_weights(const double* w, long long M, float2* wds, cudaStream_t st) {
  if (M > 0) k_w_ds<<<(unsigned)((M + 255) / 256), 256, 0, st>>>(w, M, wds);
  return cudaGetLastError();
}

// q = X^T W X p (+ lambda p) over columns [c0, c0 + D) of an FP32 X in double-FP32 arithmetic:
// one fused pass (D <= 256: rows in registers; wider: rows streamed through shared memory) with
// the weights as pairs in wds (launch_split_weights); when a wide row does not fit the shared
// memory ring, sv = W X p then X^T sv (sv: M float2 of scratch, overwriting wds).
// *launches: kernels issued; *err: set by a wait that expired.
cudaError_t launch_normal_matvec(const float* X, int ldx, int c0, int D, const double* w, const double* p, long long M,
                                 double lambda, float2* sv, double* q, double* ws, int nsm, cudaStream_t st,
                                 int* launches, int* err) {
  cudaError_t e = cudaMemsetAsync(q, 0, sizeof(double) * (size_t)D, st);
  if (e != cudaSuccess) return e;
  *launches = 0;
  long long nparts = 0;  // per-block partial column sums in ws, reduced in block order below
  const float* Xc = X + c0;
  // shared memory of the wide fused kernel: the row ring and the per-warp partials
  const int a0 = c0 & ~3;
  const int rowf = ((c0 + D + 3) & ~3) - a0;
  static int optin = 0;
  if (!optin) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  }
  // columns per consumer thread of the wide kernel (instances 1, 2, 4, 8, 12, 16) and its stage
  // stride: the copied row plus a zero tail up to the last column a thread reads
  const int cpt = (D + kWConsumers - 1) / kWConsumers;
  const int cpti = cpt <= 1 ? 1 : cpt <= 2 ? 2 : cpt <= 4 ? 4 : cpt <= 8 ? 8 : cpt <= 12 ? 12 : 16;
  const int stride = (std::max(rowf, (c0 - a0) + kWConsumers * cpti) + 3) & ~3;
  const size_t per_stage = sizeof(float) * stride + (kWWarps + 2) * sizeof(float) + 2 * sizeof(uint64_t);
  const int stages = (int)std::min<size_t>(kWMaxStages, ((size_t)optin - 256) / per_stage);
  if (M > 0 && D <= 256) {
    const long long rpb = rows_per_cta(M, 1, nsm);
    const unsigned nrb = (unsigned)((M + rpb - 1) / rpb);
    switch ((D + 31) / 32) {
      case 1: k_normal_matvec_narrow<1><<<nrb, 256, 0, st>>>(Xc, ldx, D, sv, p, M, rpb, q, ws); break;
      case 2: k_normal_matvec_narrow<2><<<nrb, 256, 0, st>>>(Xc, ldx, D, sv, p, M, rpb, q, ws); break;
      case 3: k_normal_matvec_narrow<3><<<nrb, 256, 0, st>>>(Xc, ldx, D, sv, p, M, rpb, q, ws); break;
      case 4: k_normal_matvec_narrow<4><<<nrb, 256, 0, st>>>(Xc, ldx, D, sv, p, M, rpb, q, ws); break;
      case 5: k_normal_matvec_narrow<5><<<nrb, 256, 0, st>>>(Xc, ldx, D, sv, p, M, rpb, q, ws); break;
      case 6: k_normal_matvec_narrow<6><<<nrb, 256, 0, st>>>(Xc, ldx, D, sv, p, M, rpb, q, ws); break;
      case 7: k_normal_matvec_narrow<7><<<nrb, 256, 0, st>>>(Xc, ldx, D, sv, p, M, rpb, q, ws); break;
      default: k_normal_matvec_narrow<8><<<nrb, 256, 0, st>>>(Xc, ldx, D, sv, p, M, rpb, q, ws); break;
    }
    nparts = nrb;
    *launches = 1;
  } else if (M > 0 && ws && stages >= kWRows && (ldx % 4) == 0 && cpt <= 16) {
    const size_t smem = 256 + (size_t)stages * per_stage;
    const long long rpb = (M + nsm - 1) / nsm;
    const unsigned grid = (unsigned)((M + rpb - 1) / rpb);
    auto kern = cpti == 1 ? k_normal_matvec_wide<1>
              : cpti == 2 ? k_normal_matvec_wide<2>
              : cpti == 4 ? k_normal_matvec_wide<4>
              : cpti == 8 ? k_normal_matvec_wide<8>
              : cpti == 12 ? k_normal_matvec_wide<12> : k_normal_matvec_wide<16>;
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<grid, kWThreads, smem, st>>>(X, ldx, c0, D, sv, p, M, rpb, rowf, stride, stages, q, ws, err);
    nparts = grid;
    *launches = 1;
  } else if (M > 0) {
    const size_t smem = sizeof(float) * 2 * (size_t)D;
    if (smem > 48 * 1024) {
      e = cudaFuncSetAttribute(k_xp_ds, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
    }
    k_xp_ds<<<(unsigned)(nsm * 8), 256, smem, st>>>(Xc, ldx, D, w, p, M, sv);
    const int ncb = (D + 255) / 256;
    const long long rpb = rows_per_cta(M, ncb, nsm);
    const long long nrb = (M + rpb - 1) / rpb;
    k_xtv_ds<<<dim3((unsigned)nrb, (unsigned)ncb), 256, 0, st>>>(Xc, ldx, D, sv, M, rpb, q, ws);
    nparts = nrb;
    *launches = 2;
  }
  if (nparts > 0 && ws) {
    k_colsum_reduce<<<(D + kColsumColsPerBlock - 1) / kColsumColsPerBlock, 32 * kColsumColsPerBlock, 0, st>>>(
        ws, nparts, D, q);
    *launches += 1;
  }
  if (lambda > 0) {
    e = launch_axpy(D, lambda, p, q, st);
    *launches += 1;
  }
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

// doubles of the partial column sums launch_normal_matvec needs for M rows of D columns
size_t normal_matvec_workspace_doubles(long long M, int D, int nsm) {
  if (M <= 0 || D <= 0) return 1;
  const long long narrow = (M + rows_per_cta(M, 1, nsm) - 1) / rows_per_cta(M, 1, nsm);
  const long long wide = (M + (M + nsm - 1) / nsm - 1) / ((M + nsm - 1) / nsm);
  const int ncb = (D + 255) / 256;
  const long long rpb = rows_per_cta(M, ncb, nsm);
  const long long xtv = (M + rpb - 1) / rpb;
  return (size_t)std::max(narrow, std::max(wide, xtv)) * (size_t)D;
}

template cudaError_t launch_rhs<double>(const double*, int, const double*, const double*, long long, int, double*, int,
                                        cudaStream_t, float2*, double*);
template cudaError_t launch_rhs<float>(const float*, int, const double*, const double*, long long, int, double*, int,
                                       cudaStream_t, float2*, double*);

// lower triangle <- upper triangle
cudaError_t launch_symmetrize(double* G, int D, cudaStream_t st) {
  k_symmetrize<<<D, 128, 0, st>>>(G, D);
  return cudaGetLastError();
}


// ------------------------------------------------------------------------------------
// Symmetric min-norm solve by parallel cyclic Jacobi (one CTA, D <= kJacobiMax).
// ------------------------------------------------------------------------------------
constexpr int kJacobiMax = 112;

__global__ void __launch_bounds__(1024) k_jacobi_solve(const double* __restrict__ Gin, const double* __restrict__ h,
                                                       int D, double lambda, double rcond, double* __restrict__ wout,
                                                       double* __restrict__ evals, int* __restrict__ info) {
  extern __shared__ double sm[];
  __shared__ double wred[64];  // per-warp partial sums of the convergence test
  const int n = (D + 1) & ~1;  // even
  double* A = sm;               // n*n
  double* V = A + n * n;        // n*n
  double* cs = V + n * n;       // n/2 * 2
  int* pp = reinterpret_cast<int*>(cs + n);  // n/2
  int* qq = pp + n / 2;
  int* perm = qq + n / 2;       // n
  double* red = reinterpret_cast<double*>(perm + n);  // 2 doubles + flag
  const int tid = threadIdx.x, nth = blockDim.x;
  for (int e = tid; e < n * n; e += nth) {
    int i = e / n, j = e % n;
    double v = 0;
    if (i < D && j < D) v = Gin[(size_t)i * D + j] + ((i == j && lambda > 0) ? lambda : 0.0);
    A[e] = v;
    V[e] = (i == j) ? 1.0 : 0.0;
  }
  for (int e = tid; e < n; e += nth) perm[e] = e;
  __syncthreads();
  const int npair = n / 2;
  int sweep = 0;
  for (; sweep < 40; ++sweep) {
    // convergence test: off-diagonal Frobenius vs diagonal
    if (tid == 0) {
      red[0] = 0;
      red[1] = 0;
    }
    __syncthreads();
    double off = 0, dia = 0;
    for (int e = tid; e < n * n; e += nth) {
      int i = e / n, j = e % n;
      double v = A[e] * A[e];
      if (i == j) dia += v;
      else off += v;
    }
    for (int o = 16; o > 0; o >>= 1) {
      off += __shfl_xor_sync(0xffffffffu, off, o);
      dia += __shfl_xor_sync(0xffffffffu, dia, o);
    }
    // warp sums added in warp order (a fixed sweep count for a given matrix)
    if ((tid & 31) == 0) {
      wred[2 * (tid >> 5)] = off;
      wred[2 * (tid >> 5) + 1] = dia;
    }
    __syncthreads();
    if (tid == 0) {
      double so = 0.0, sd = 0.0;
      for (int w = 0; w < nth / 32; ++w) {
        so += wred[2 * w];
        sd += wred[2 * w + 1];
      }
      red[0] = so;
      red[1] = sd;
    }
    __syncthreads();
    if (red[0] <= 1e-28 * red[1] || red[1] == 0.0) break;
    __syncthreads();
    for (int round = 0; round < n - 1; ++round) {
      // tournament pairing: perm[0] fixed, the rest rotate
      if (tid < npair) {
        int p = perm[tid], q = perm[n - 1 - tid];
        if (p > q) {
          int t = p;
          p = q;
          q = t;
        }
        pp[tid] = p;
        qq[tid] = q;
        double apq = A[p * n + q];
        double c = 1.0, s = 0.0;
        if (p < D && q < D && apq != 0.0) {
          double app = A[p * n + p], aqq = A[q * n + q];
          double tau = (aqq - app) / (2.0 * apq);
          double t = (tau >= 0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
          c = 1.0 / sqrt(1.0 + t * t);
          s = t * c;
        }
        cs[2 * tid] = c;
        cs[2 * tid + 1] = s;
      }
      __syncthreads();
      // columns: A <- A J, V <- V J
      for (int e = tid; e < n * npair; e += nth) {
        int i = e / npair, k = e % npair;
        int p = pp[k], q = qq[k];
        double c = cs[2 * k], s = cs[2 * k + 1];
        double aip = A[i * n + p], aiq = A[i * n + q];
        A[i * n + p] = c * aip - s * aiq;
        A[i * n + q] = s * aip + c * aiq;
        double vip = V[i * n + p], viq = V[i * n + q];
        V[i * n + p] = c * vip - s * viq;
        V[i * n + q] = s * vip + c * viq;
      }
      __syncthreads();
      // rows: A <- J^T A
      for (int e = tid; e < n * npair; e += nth) {
        int j = e / npair, k = e % npair;
        int p = pp[k], q = qq[k];
        double c = cs[2 * k], s = cs[2 * k + 1];
        double apj = A[p * n + j], aqj = A[q * n + j];
        A[p * n + j] = c * apj - s * aqj;
        A[q * n + j] = s * apj + c * aqj;
      }
      __syncthreads();
      if (tid == 0) {
        int last = perm[n - 1];
        for (int k = n - 1; k > 1; --k) perm[k] = perm[k - 1];
        perm[1] = last;
      }
      __syncthreads();
    }
  }
  // min-norm solution: w = sum_{|lambda_i| > thr} (v_i . h / lambda_i) v_i
  __syncthreads();
  if (tid == 0) {
    double mx = 0;
    for (int i = 0; i < D; ++i) mx = fmax(mx, fabs(A[i * n + i]));
    red[0] = mx;
    int rank = 0;
    double thr = (rcond < 0 ? 1.1102230246251565e-16 : rcond) * mx;
    for (int i = 0; i < D; ++i) rank += fabs(A[i * n + i]) > thr;
    info[0] = sweep;
    info[1] = rank;
  }
  __syncthreads();
  const double thr = (rcond < 0 ? 1.1102230246251565e-16 : rcond) * red[0];
  double* coef = cs;  // reuse (n entries)
  for (int i = tid; i < D; i += nth) {
    double lam = A[i * n + i];
    double d = 0;
    for (int r = 0; r < D; ++r) d = fma(V[r * n + i], h[r], d);
    if (evals) evals[i] = lam;
    coef[i] = (fabs(lam) > thr) ? d / lam : 0.0;
  }
  __syncthreads();
  for (int r = tid; r < D; r += nth) {
    double acc = 0;
    for (int i = 0; i < D; ++i) acc = fma(V[r * n + i], coef[i], acc);
    wout[r] = acc;
  }
}

cudaError_t launch_solve_sym(double* G, const double* h, int D, double lambda, double rcond, double* wout,
                             double* evals, int* info, cudaStream_t st) {
  if (D > kJacobiMax) return cudaErrorInvalidValue;
  const int n = (D + 1) & ~1;
  size_t smem = sizeof(double) * (2 * (size_t)n * n + n) + sizeof(int) * (2 * n) + 4 * sizeof(double);
  cudaError_t e = cudaFuncSetAttribute(k_jacobi_solve, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k_jacobi_solve<<<1, 1024, smem, st>>>(G, h, D, lambda, rcond, wout, evals, info);
  return cudaGetLastError();
}

// ------------------------------------------------------------------------------------
// predictions and squared-error sums per row kind (0 energy, 1 force, 2 stress)
// ------------------------------------------------------------------------------------
// Predictions X w (warp per design row, grid-stride) and per-kind squared errors: FP64 dot for
// an FP64 X, double-FP32 dot for an FP32 X (w split into FP32 pairs in shared memory).  The
// squared errors are reduced per block before six FP64 atomics.
constexpr int kSqPartials = 8;  // offset of the per-CTA partials in the squared-error buffer

template <typename T>
__global__ void __launch_bounds__(256) k_predict(const T* __restrict__ X, int ldx, const double* __restrict__ w,
                                                 long long M, int D, double* __restrict__ pred,
                                                 const double* __restrict__ y, const int* __restrict__ kind,
                                                 double* __restrict__ sq /*3 sums + 3 counts, then per-CTA partials*/) {
  extern __shared__ float wsp[];  // [2][D] for FP32 X
  __shared__ double red[8][6];
  constexpr bool kDs = std::is_same<T, float>::value;
  if (kDs) {
    for (int c = threadIdx.x; c < D; c += blockDim.x) ds_split(w[c], wsp[c], wsp[D + c]);
    __syncthreads();
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double acc6[6] = {0, 0, 0, 0, 0, 0};
  const long long nw = (long long)gridDim.x * 8;
  for (long long r = (long long)blockIdx.x * 8 + warp; r < M; r += nw) {
    const T* xr = X + r * ldx;
    double v;
    if constexpr (kDs) {
      float dh = 0.f, dl = 0.f;
      for (int c = lane; c < D; c += 32) ds_fma(dh, dl, xr[c], wsp[c], wsp[D + c]);
      for (int o = 16; o > 0; o >>= 1) {
        const float oh = __shfl_xor_sync(0xffffffffu, dh, o), ol = __shfl_xor_sync(0xffffffffu, dl, o);
        ds_add(dh, dl, oh, ol);
      }
      v = (double)dh + (double)dl;
    } else {
      double a = 0.0;
      for (int c = lane; c < D; c += 32) a = fma((double)xr[c], w[c], a);
      for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
      v = a;
    }
    if (lane == 0) {
      if (pred) pred[r] = v;
      if (sq) {
        const double d = v - y[r];
        const int k = kind[r];
        acc6[k] += d * d;
        acc6[3 + k] += 1.0;
      }
    }
  }
  if (!sq) return;
  if (lane == 0)
    for (int k = 0; k < 6; ++k) red[warp][k] = acc6[k];
  __syncthreads();
  if (threadIdx.x < 6) {
    double t = 0.0;
    for (int w8 = 0; w8 < 8; ++w8) t += red[w8][threadIdx.x];
    sq[kSqPartials + 6 * (size_t)blockIdx.x + threadIdx.x] = t;
  }
}

// sq[0..5] = the per-CTA partials summed in CTA order
__global__ void k_sq_reduce(double* __restrict__ sq, int blocks) {
  const int k = threadIdx.x;
  if (k >= 6) return;
  double t = 0.0;
  for (int b = 0; b < blocks; ++b) t += sq[kSqPartials + 6 * (size_t)b + k];
  sq[k] = t;
}

template <typename T>
cudaError_t launch_predict_sq(const T* X, int ldx, const double* w, long long M, int D, double* pred,
                              const double* y, const int* kind, double* sq, cudaStream_t st) {
  if (M == 0) return cudaSuccess;
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const long long want = (M + 7) / 8;
  const unsigned blocks = (unsigned)std::min<long long>(want, (long long)nsm * 8);
  size_t smem = 0;
  if (std::is_same<T, float>::value) {
    smem = sizeof(float) * 2 * (size_t)D;
    if (smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(k_predict<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
    }
  }
  k_predict<T><<<blocks, 256, smem, st>>>(X, ldx, w, M, D, pred, y, kind, sq);
  if (sq) k_sq_reduce<<<1, 32, 0, st>>>(sq, (int)blocks);
  return cudaGetLastError();
}

size_t predict_sq_doubles() {
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  return kSqPartials + 6 * (size_t)nsm * 8;
}

template <typename T>
cudaError_t launch_rows_prep(int S, const int* atom_start, const DevRows& rows, const double* E, const double* F,
                             const double* Sv, const double* wefs, T* X, double* y, double* wrow, int* kind,
                             cudaStream_t st) {
  if (S == 0) return cudaSuccess;
  k_rows_prep<T><<<S, 128, 0, st>>>(S, atom_start, rows.rowE, rows.rowF, rows.rowS, E, F, Sv, wefs, rows.ldx, X, y,
                                    wrow, kind);
  return cudaGetLastError();
}

template cudaError_t launch_gram<double>(const double*, int, const double*, const double*, long long, int, double*,
                                         double*, cudaStream_t, double*);
template cudaError_t launch_gram<float>(const float*, int, const double*, const double*, long long, int, double*,
                                        double*, cudaStream_t, double*);
template cudaError_t launch_predict_sq<double>(const double*, int, const double*, long long, int, double*,
                                               const double*, const int*, double*, cudaStream_t);
template cudaError_t launch_predict_sq<float>(const float*, int, const double*, long long, int, double*, const double*,
                                              const int*, double*, cudaStream_t);
template cudaError_t launch_rows_prep<double>(int, const int*, const DevRows&, const double*, const double*,
                                              const double*, const double*, double*, double*, double*, int*,
                                              cudaStream_t);
template cudaError_t launch_rows_prep<float>(int, const int*, const DevRows&, const double*, const double*,
                                             const double*, const double*, float*, double*, double*, int*,
                                             cudaStream_t);

}  // namespace mld

namespace mld {

// CUDA-core FMA throughput probe: 8 independent FMA chains per thread, all SMs busy.  Used as
// the measured denominator of the descriptor kernel's roofline (FP64 or FP32 pipe).
template <typename T>
__global__ void __launch_bounds__(256) k_fma_peak(int iters, T seed, T* out) {
  T a0 = seed + threadIdx.x, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6,
    a7 = a0 + 7;
  const T m = (T)0.999999, c = (T)1e-7;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      a0 = fma(a0, m, c);
      a1 = fma(a1, m, c);
      a2 = fma(a2, m, c);
      a3 = fma(a3, m, c);
      a4 = fma(a4, m, c);
      a5 = fma(a5, m, c);
      a6 = fma(a6, m, c);
      a7 = fma(a7, m, c);
    }
  }
  T s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
  if (s == (T)-1) out[0] = s;  // never true; keeps the chains alive
}

template <typename T>
cudaError_t measure_fma_peak(cudaStream_t st, double* tflops) {
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  T* out = nullptr;
  cudaError_t e = cudaMalloc(&out, sizeof(T));
  if (e != cudaSuccess) return e;
  const int blocks = nsm * 8, threads = 256;
  const int iters = sizeof(T) == 8 ? 64 : 2048;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  k_fma_peak<T><<<blocks, threads, 0, st>>>(iters, (T)1, out);  // warm-up
  cudaEventRecord(a, st);
  const int reps = 5;
  for (int r = 0; r < reps; ++r) k_fma_peak<T><<<blocks, threads, 0, st>>>(iters, (T)1, out);
  cudaEventRecord(b, st);
  e = cudaEventSynchronize(b);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(out);
  const double flops = 2.0 * 8 * 16 * (double)iters * threads * blocks * reps;
  *tflops = flops / (ms * 1e-3) / 1e12;
  return e == cudaSuccess ? cudaGetLastError() : e;
}

template cudaError_t measure_fma_peak<double>(cudaStream_t, double*);
template cudaError_t measure_fma_peak<float>(cudaStream_t, double*);

}  // namespace mld
