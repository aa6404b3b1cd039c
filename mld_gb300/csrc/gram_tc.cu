// Weighted Gram matrix G = X^T W X on the 5th-generation tensor cores (tcgen05) in BF16 split
// precision with FP32 accumulation: the mixed method's normal matrix (parameters.F90:1018-1099
// for the linear block, :404-421,476-1015 for the quadratic block of the QNML fit).
//
//   x' = sqrt(w_r) x_r,  x' = hi + lo  (hi = bf16(x'), lo = bf16(x' - hi)),
//   x'_i x'_j ~= hi_i hi_j + hi_i lo_j + lo_i hi_j      (three bf16 MMAs per K step)
//
// A row chunk of X is first transposed into K-major bf16 planes Xt_hi / Xt_lo (D x Mp, the design
// row index contiguous), so both MMA operands of an output tile (features i, features j) are
// 128 x 64 K-major slices of the same planes, fetched by TMA with 128-byte swizzle.  Feature rows
// beyond D and design rows beyond the chunk are zero-filled by TMA.
//
// Grid: (upper-triangle tile pairs) x (row splits), split-major so that the CTAs resident at one
// time read the same rows (L2 reuse).  Per CTA: warp 0 issues TMA loads into a 3-stage ring,
// warp 1 allocates two 128-column TMEM accumulators and issues tcgen05.mma from one thread,
// warps 2-17 drain the accumulators with tcgen05.ld into compensated FP32 sums.  With several
// row splits each split writes its tile to a partial buffer and k_gram_tc_reduce adds the splits
// into the FP64 Gram in split order (without that buffer: FP64 atomics, order not fixed); with
// one split the CTA adds its tile directly.  Every mbarrier wait
// is bounded: on expiry the CTA sets *err, waits (bounded) for its copies in flight and still
// frees its TMEM.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>

#include "mld_internal.h"
#include "ptx.cuh"
#include "tc.cuh"

namespace mld {

namespace {

using tc::kTK;
using tc::kTM;
using tc::kTileBytes;
constexpr int kStages = 3;
constexpr int kStageBytes = 4 * kTileBytes;    // A_hi, A_lo, B_hi, B_lo
constexpr int kFlush = 1;                      // K slices per TMEM accumulation (64 design rows)
constexpr int kEpiWarps = 16;                  // four per TMEM lane quarter, 32 columns each
constexpr int kGramThreads = 32 * (2 + kEpiWarps);
constexpr size_t kGramSmem = (size_t)kStages * kStageBytes + 1024 + 256;

using ptx::mbar_expect_tx;
using ptx::mbar_init;
using ptx::mbar_wait;
using ptx::smem_u32;
using ptx::tma_load_2d;
using tc::mma_bf16;
using tc::mma_commit;
using tc::sw128_desc;

}  // namespace

// Transpose rows [r0, r0 + rows) of X (row stride ldx, columns [c0, c0 + D)) into the K-major
// bf16 planes hi/lo (D x Mp), scaling row r by sqrt(w[r]); design rows [rows, Mp) are zeroed.
// grid.x: 32-row blocks of the chunk, grid.y: 32-column blocks.
template <typename T>
__global__ void __launch_bounds__(256) k_split_bf16(const T* __restrict__ X, int ldx, int c0, int D,
                                                    const double* __restrict__ w, long long r0, long long rows,
                                                    long long Mp, __nv_bfloat16* __restrict__ hi,
                                                    __nv_bfloat16* __restrict__ lo) {
  __shared__ float tile[32][33];
  __shared__ float sw[32];
  const long long rb = (long long)blockIdx.x * 32;
  const int cb = blockIdx.y * 32;
  const int tid = threadIdx.y * blockDim.x + threadIdx.x;
  // sqrt(w) and x' in FP32: the split keeps about 17 bits of x', and FP64 runs at 1/64 rate
  if (tid < 32) sw[tid] = (rb + tid < rows) ? (float)sqrt(w[r0 + rb + tid]) : 0.f;
  __syncthreads();
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const long long r = rb + y;
    const int c = cb + threadIdx.x;
    float v = 0.f;
    if (r < rows && c < D) v = (float)X[(r0 + r) * ldx + c0 + c] * sw[y];
    tile[y][threadIdx.x] = v;
  }
  __syncthreads();
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int c = cb + y;
    const long long r = rb + threadIdx.x;
    if (c < D && r < Mp) {
      const float v = tile[threadIdx.x][y];
      const __nv_bfloat16 h = __float2bfloat16_rn(v);
      hi[(size_t)c * Mp + r] = h;
      lo[(size_t)c * Mp + r] = __float2bfloat16_rn(v - __bfloat162float(h));
    }
  }
}

// blockIdx.x = tile + ntile * split; tile enumerates the upper-triangle pairs ti <= tj.
// Row split s covers K slices [s * kps, min(nk, (s + 1) * kps)) of 64 design rows.
//
// The FP32 accumulator lives in TMEM for `flush` K slices only (kFlush = 1: 64 design rows), because
// the tensor core rounds its FP32 accumulation toward zero (a bias that grows with the chain): the MMA issuer
// alternates between two 128-column TMEM buffers, and the epilogue warps drain the idle buffer
// into compensated (Kahan) FP32 register sums, so the error of the whole split stays at the
// level of one short FP32 accumulation.  Epilogue warp w reads TMEM lane quarter w % 4 and one
// quarter (32 columns) of the tile.
__global__ void __launch_bounds__(kGramThreads, 1)
    k_gram_tc(const __grid_constant__ CUtensorMap map_hi, const __grid_constant__ CUtensorMap map_lo, int nt,
              int ntile, int nk, int kps, int flush, int D, double* __restrict__ G, double* __restrict__ part,
              int* __restrict__ err, int skip_loads, long long wait_limit) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* tiles = reinterpret_cast<unsigned char*>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = reinterpret_cast<uint64_t*>(tiles + kStages * kStageBytes);
  uint64_t* empty = full + kStages;
  uint64_t* tfull = empty + kStages;  // [2] accumulator buffer ready for the epilogue
  uint64_t* tempty = tfull + 2;       // [2] accumulator buffer drained
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(tempty + 2);

  int t = blockIdx.x % ntile, ti = 0;
  const int split = blockIdx.x / ntile;
  while (t >= nt - ti) {
    t -= nt - ti;
    ++ti;
  }
  const int tj = ti + t;
  const int kb = split * kps;
  const int nkl = min(nk, kb + kps) - kb;  // >= 1 by construction of the grid
  const int ngrp = (nkl + flush - 1) / flush;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&tfull[b], 1);
      mbar_init(&tempty[b], kEpiWarps);
    }
    ptx::mbar_init_fence();
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(2 * kTM));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = *tmem_slot;
  bool ok = true;

  if (warp == 0 && lane == 0) {
    // producer: A = features of tile ti, B = features of tile tj
    int issued = 0;
    for (int k = 0; k < (skip_loads ? 0 : nkl); ++k) {
      const int s = k % kStages;
      if (k >= kStages && !mbar_wait(&empty[s], ((k / kStages) - 1) & 1, wait_limit)) {
        ok = false;
        break;
      }
      unsigned char* st = tiles + s * kStageBytes;
      const int x = (kb + k) * kTK;
      mbar_expect_tx(&full[s], kStageBytes);
      tma_load_2d(st, &map_hi, x, ti * kTM, &full[s]);
      tma_load_2d(st + kTileBytes, &map_lo, x, ti * kTM, &full[s]);
      tma_load_2d(st + 2 * kTileBytes, &map_hi, x, tj * kTM, &full[s]);
      tma_load_2d(st + 3 * kTileBytes, &map_lo, x, tj * kTM, &full[s]);
      issued = k + 1;
    }
    // the copies issued last may still be in flight: wait for them (bounded) before leaving
    for (int k = max(0, issued - kStages); k < issued; ++k) mbar_wait(&full[k % kStages], (k / kStages) & 1, wait_limit);
  } else if (warp == 1 && lane == 0) {
    // MMA issuer: K-slice group g accumulates into TMEM buffer g & 1
    for (int g = 0; g < ngrp && ok; ++g) {
      const int b = g & 1;
      if (g >= 2 && !mbar_wait(&tempty[b], ((g >> 1) - 1) & 1, wait_limit)) {
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint32_t acc = tmem + (uint32_t)(b * kTM);
      const int k1 = min(nkl, (g + 1) * flush);
      for (int k = g * flush; k < k1; ++k) {
        const int s = k % kStages;
        if (!mbar_wait(&full[s], (k / kStages) & 1, wait_limit)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint32_t st = smem_u32(tiles + s * kStageBytes);
#pragma unroll
        for (int kk = 0; kk < kTK / 16; ++kk) {
          const uint32_t off = kk * 32;  // 16 bf16 along K inside the 128-byte swizzle row
          const uint64_t ahi = sw128_desc(st + off), alo = sw128_desc(st + kTileBytes + off);
          const uint64_t bhi = sw128_desc(st + 2 * kTileBytes + off), blo = sw128_desc(st + 3 * kTileBytes + off);
          mma_bf16(acc, ahi, bhi, (k > g * flush || kk > 0) ? 1u : 0u);
          mma_bf16(acc, ahi, blo, 1u);
          mma_bf16(acc, alo, bhi, 1u);
        }
        mma_commit(&empty[s]);  // frees the stage once these MMAs have read it
      }
      mma_commit(&tfull[b]);
    }
  } else if (warp >= 2) {
    // epilogue: Kahan sums of 32 columns of one TMEM lane quarter
    const int q = warp & 3, cq = (warp - 2) >> 2;
    float sum[32], cmp[32];
#pragma unroll
    for (int c = 0; c < 32; ++c) sum[c] = cmp[c] = 0.f;
    bool got = true;
    for (int g = 0; g < ngrp; ++g) {
      const int b = g & 1;
      if (!mbar_wait(&tfull[b], (g >> 1) & 1, wait_limit)) {
        got = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;");
#pragma unroll
      for (int h2 = 0; h2 < 4; ++h2) {
        uint32_t v[8];
        const uint32_t taddr = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * kTM + cq * 32 + h2 * 8);
        asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                     : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7])
                     : "r"(taddr));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int c = 0; c < 8; ++c) {
          const int e = h2 * 8 + c;
          const float y = __uint_as_float(v[c]) - cmp[e];
          const float tt = sum[e] + y;
          cmp[e] = (tt - sum[e]) - y;
          sum[e] = tt;
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;");
      __syncwarp();
      if (lane == 0) ptx::mbar_arrive(&tempty[b]);
    }
    if (got && part) {
      // this split's tile, added to G in split order by k_gram_tc_reduce
      double* pt = part + ((size_t)split * ntile + blockIdx.x % ntile) * (kTM * kTM) + (size_t)(q * 32 + lane) * kTM +
                   cq * 32;
#pragma unroll
      for (int c = 0; c < 32; ++c) pt[c] = (double)sum[c] - (double)cmp[c];
    } else if (got) {
      // straight into G: with a single split the CTA is the only writer of these elements
      const int i = ti * kTM + q * 32 + lane;
      if (i < D) {
#pragma unroll
        for (int c = 0; c < 32; ++c) {
          const int j = tj * kTM + cq * 32 + c;
          if (j < D && j >= i) atomicAdd(&G[(size_t)i * D + j], (double)sum[c] - (double)cmp[c]);
        }
      }
    } else if (lane == 0) {
      atomicExch(err, 1);
    }
  }
  if (!ok) atomicExch(err, 1);
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * kTM));
  }
}

// ---------------------------------------------------------------------------------------
// Test hook of the timeout path: with skip_loads the producer issues no TMA loads, so the MMA
// and epilogue warps' bounded waits expire (after wait_limit clocks), the CTA reports *err = 1
// and frees its TMEM.  (0, 0) restores normal operation.
namespace {
int g_skip_loads = 0;
long long g_wait_limit = ptx::kWaitLimit;
}  // namespace
void gram_tc_test_timeout(int skip_loads, long long wait_limit) {
  g_skip_loads = skip_loads ? 1 : 0;
  g_wait_limit = wait_limit > 0 ? wait_limit : ptx::kWaitLimit;
}

size_t gram_tc_min_workspace(int D) { return (size_t)4 * D * kTK + 256; }

namespace {
// row splits of one chunk of nk 64-row slices: at least two waves of CTAs where the tile count
// alone does not give them, every split non-empty
int gram_tc_splits(int nk, int ntile, int nsm, int* kps) {
  const int ns = std::max(1, std::min(nk, (2 * nsm + ntile - 1) / ntile));
  *kps = (nk + ns - 1) / ns;
  return (nk + *kps - 1) / *kps;
}

// G[i][j] += sum over the splits of their tile partials, in split order (upper triangle).
__global__ void k_gram_tc_reduce(const double* __restrict__ part, int nt, int ntile, int nsplit, int D,
                                 double* __restrict__ G) {
  const int tile = blockIdx.y;
  int t = tile, ti = 0;
  while (t >= nt - ti) {
    t -= nt - ti;
    ++ti;
  }
  const int tj = ti + t;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;  // element of the kTM x kTM tile
  if (e >= kTM * kTM) return;
  const int i = ti * kTM + e / kTM, j = tj * kTM + e % kTM;
  if (i >= D || j >= D || j < i) return;
  double s = 0.0;
  for (int sp = 0; sp < nsplit; ++sp) s += part[((size_t)sp * ntile + tile) * (kTM * kTM) + e];
  G[(size_t)i * D + j] += s;
}
}  // namespace

size_t gram_tc_part_doubles(int D, int nsm) {
  const int nt = (D + kTM - 1) / kTM, ntile = nt * (nt + 1) / 2;
  if (ntile >= 2 * nsm) return 0;  // one split per chunk: no partials
  return (size_t)(2 * nsm + ntile) * kTM * kTM;
}

bool gram_tc_available() { return tc::encode_fn() != nullptr; }

// G (FP64, D x D, upper triangle) += sum over rows r of w_r x_r x_r^T for columns [c0, c0 + D)
// of X (M rows, stride ldx).  `ws` holds ws_bytes >= gram_tc_min_workspace(D) bytes; the rows
// are processed in chunks that fit it.  The caller zeroes G and *err and symmetrises G.
template <typename T>
cudaError_t launch_gram_tc(const T* X, int ldx, int c0, int D, const double* w, long long M, double* G, void* ws,
                           size_t ws_bytes, int* err, int nsm, cudaStream_t st, double* part, size_t part_doubles) {
  if (M <= 0 || D <= 0) return cudaSuccess;
  if (ws_bytes < gram_tc_min_workspace(D) || ((uintptr_t)ws & 15)) return cudaErrorInvalidValue;
  // chunk rows: a multiple of 64 whose two planes fit the workspace
  long long chunk = (long long)((ws_bytes - 256) / (4 * (size_t)D)) / kTK * kTK;
  chunk = std::min(chunk, (M + kTK - 1) / kTK * kTK);
  static bool attr_set = false;
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(k_gram_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGramSmem);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  const int nt = (D + kTM - 1) / kTM;
  const int ntile = nt * (nt + 1) / 2;
  __nv_bfloat16* hi = reinterpret_cast<__nv_bfloat16*>(ws);
  for (long long r0 = 0; r0 < M; r0 += chunk) {
    const long long rows = std::min(chunk, M - r0);
    const long long Mp = (rows + 7) / 8 * 8;  // 16-byte plane row stride
    __nv_bfloat16* lo = hi + (size_t)D * Mp;
    dim3 g1((unsigned)((Mp + 31) / 32), (unsigned)((D + 31) / 32));
    k_split_bf16<T><<<g1, dim3(32, 8), 0, st>>>(X, ldx, c0, D, w, r0, rows, Mp, hi, lo);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    CUtensorMap mh, ml;
    if (!tc::make_plane_map(&mh, hi, Mp, D, Mp) || !tc::make_plane_map(&ml, lo, Mp, D, Mp)) return cudaErrorInvalidValue;
    const int nk = (int)((rows + kTK - 1) / kTK);
    int kps = 1;
    const int nsplit = gram_tc_splits(nk, ntile, nsm, &kps);
    // several splits of a tile: per-split partials reduced in split order when the workspace
    // holds them (deterministic); otherwise FP64 atomics (order of the splits not fixed)
    const bool use_part = nsplit > 1 && part && part_doubles >= (size_t)nsplit * ntile * kTM * kTM;
    double* pt = use_part ? part : nullptr;
    k_gram_tc<<<(unsigned)(ntile * nsplit), kGramThreads, kGramSmem, st>>>(mh, ml, nt, ntile, nk, kps, kFlush, D, G,
                                                                           pt, err, g_skip_loads, g_wait_limit);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if (use_part) {
      k_gram_tc_reduce<<<dim3((kTM * kTM + 255) / 256, (unsigned)ntile), 256, 0, st>>>(part, nt, ntile, nsplit, D, G);
      e = cudaGetLastError();
      if (e != cudaSuccess) return e;
    }
  }
  return cudaSuccess;
}

template cudaError_t launch_gram_tc<float>(const float*, int, int, int, const double*, long long, double*, void*,
                                           size_t, int*, int, cudaStream_t, double*, size_t);
template cudaError_t launch_gram_tc<double>(const double*, int, int, int, const double*, long long, double*, void*,
                                            size_t, int*, int, cudaStream_t, double*, size_t);

}  // namespace mld
