// Force rows of the kernel model on the tensor cores (mixed method).
//
// The force row of atom a for reference point k (compute_kernel.F90:476-866, mld_forces.F90:
// 268-320) is a sum over the derivative vectors of a: its own pair sum (v = 0, centre a, sign +1)
// and the reversed pairs j -> a (v >= 1, centre j, sign -1):
//   row(a, alpha, k) = sum_v sign_v (c1(ce_v, k) (V_{v,alpha} . z_k) - c2(ce_v, k) (V_{v,alpha} . x_{ce_v}))
// The products z_k . V over all reference points and rows are one large GEMM, Z (nk x KK) times
// V^T (KK x rows), which this file runs on the 5th-generation tensor cores in BF16 split precision
// (v = hi + lo; hi hi + lo hi + hi lo, three MMAs per K step, FP32 accumulation of KK <= 192
// products in TMEM), with the coefficient transform and the sum over v in the epilogue:
//   * operands: Z and V as K-major bf16 hi/lo planes, K padded to a multiple of 64;
//   * the 128 reference points of a CTA are the MMA's M side (TMEM lanes) and the rows of one
//     atom tile its N side (TMEM columns): the tile's vectors alpha-major, nvp (a multiple of 8)
//     rows per alpha, N = 3 nvp rounded up to 16 <= 256; an atom with more vectors than a tile
//     holds is split over several tiles;
//   * an epilogue thread owns one reference point (a TMEM lane), so its coefficients come from
//     coalesced rows of the kernel features, the sum over v stays in registers, and the three
//     alpha columns of a vector share one coefficient pair;
//   * CTA = one 128-point tile of Z (resident in shared memory) and a strided set of atom tiles,
//     with a TMA producer warp, an MMA warp (two TMEM accumulators of 256 columns) and sixteen
//     epilogue warps (four per lane quarter, splitting the vectors in chunks of eight); the
//     quarter's partial sums meet in shared memory and are added to the force rows with FP32
//     atomics (an atom split over tiles sums there too).
// Every mbarrier wait is bounded: on expiry the CTA sets *err, waits (bounded) for its copies in
// flight and frees its TMEM.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "mld_internal.h"
#include "ptx.cuh"
#include "tc.cuh"

namespace mld {

namespace {
using tc::kTK;
using tc::kTM;
using tc::kTileBytes;
constexpr int kKEpiWarps = 16;
constexpr int kKThreads = 32 * (2 + kKEpiWarps);
constexpr int kBoxRows = 32;                   // rows per TMA box of a V tile
constexpr int kBoxBytes = kBoxRows * kTK * 2;  // 4 KB
constexpr int kChunks = 3;                      // vector chunks per epilogue warp and tile
constexpr int kTmemCols = 512;                 // two accumulators of up to 256 columns
constexpr int kMaxStages = 4;                  // V tile stages

// rows of a V tile: up to 256 for K <= 128 (two K blocks), 128 for three K blocks (shared memory)
__host__ __device__ constexpr int max_tile_rows(int nkb) { return nkb <= 2 ? 256 : 128; }
// vectors of a tile with R components per vector (3 force directions, 6 stress components):
// R nvp <= rows, nvp a multiple of 8
__host__ __device__ constexpr int max_tile_vectors(int nkb, int R = 3) { return max_tile_rows(nkb) / R / 8 * 8; }
static_assert(max_tile_vectors(1) / 8 <= 4 * kChunks, "chunks per epilogue warp");
// float4 records per vector: {centre, f1, f2, 0} and the R values g, four per float4
__host__ __device__ constexpr int recs_of(int R) { return 1 + (R + 3) / 4; }

struct TileMeta {
  int atom;  // target atom (batch index)
  int row0;  // first plane row of the tile within the chunk
  int N;     // plane rows of the tile (MMA N): 3 nvp rounded up to 16
  int nvp;   // rows per alpha (a multiple of 8)
  int vr0;   // first vector record of the tile within the chunk (nvp records)
  int v0;    // first derivative vector of the atom in this tile
  int nvt;   // derivative vectors in this tile
  int pad;
};
static_assert(sizeof(TileMeta) == 32, "tile records are 32 bytes");
}  // namespace

// Z (nk x KK, row-major) -> bf16 hi/lo planes (nk x KP), zero past KK.
__global__ void k_ktc_zplanes(const float* __restrict__ Z, int nk, int KK, int KP, __nv_bfloat16* __restrict__ hi,
                              __nv_bfloat16* __restrict__ lo) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long long)nk * KP) return;
  const int k = (int)(e / KP), c = (int)(e - (long long)k * KP);
  const float v = c < KK ? Z[(size_t)k * KK + c] : 0.f;
  const __nv_bfloat16 h = __float2bfloat16_rn(v);
  hi[e] = h;
  lo[e] = __float2bfloat16_rn(v - __bfloat162float(h));
}

// The derivative vectors of a chunk's atom tiles as bf16 hi/lo planes (KP per row; rows past
// 3 nvp of a tile are zero), the first force row of each tile (trow), and one 32-byte record per
// vector: {centre (int bits), sign / sqrt
// f(x,x), sign dker_xx / (2 f(x,x) sqrt f(x,x)), 0} and {g_x, g_y, g_z, 0} with g = V . x_centre.
// A padding vector has centre = the atom and zero factors; a centre without neighbours has zero
// factors (krr_c12 of kernel_rows with the point terms left out).  One CTA (4 warps) per tile;
// warp w builds rows w, w + 4, ... of the tile.
__global__ void __launch_bounds__(128) k_ktc_vplanes(const TileMeta* __restrict__ tmeta, int KK, int KP,
                                                     const int* __restrict__ nbr_off, const int* __restrict__ nbr_idx,
                                                     const int* __restrict__ rev, const float* __restrict__ B,
                                                     const float* __restrict__ dB, const float* __restrict__ at,
                                                     __nv_bfloat16* __restrict__ hi, __nv_bfloat16* __restrict__ lo,
                                                     float* __restrict__ vrec, const int* __restrict__ atom_struct,
                                                     const int* __restrict__ atom_start,
                                                     const long long* __restrict__ rowF, long long* __restrict__ trow) {
  const TileMeta m = tmeta[blockIdx.x];
  if (threadIdx.x == 0) {
    // the tile's first force row (alpha = 0), -1 for a structure without force rows
    const int sidx = atom_struct[m.atom];
    const long long rf = rowF[sidx];
    trow[blockIdx.x] = rf >= 0 ? rf + 3LL * (m.atom - atom_start[sidx]) : -1;
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int a = m.atom;
  const int p0 = nbr_off[a], nn = nbr_off[a + 1] - p0;
  for (int lr = warp; lr < m.N; lr += 4) {
    const long long row = (long long)m.row0 + lr;
    const int al = lr / m.nvp, vl = lr - al * m.nvp, v = m.v0 + vl;
    const bool valid = al < 3 && vl < m.nvt;
    int ce = a;
    const float* src = nullptr;  // pair row (v >= 1) or null for the self sum
    if (valid && v > 0) {
      ce = nbr_idx[p0 + v - 1];
      const int q = rev[p0 + v - 1];
      if (q >= 0) src = dB + ((size_t)q * 3 + al) * KK;
    }
    float g = 0.f;
    for (int c = lane; c < KP; c += 32) {
      float x = 0.f;
      if (valid && c < KK) {
        if (v == 0) {
          for (int q = 0; q < nn; ++q) x += dB[((size_t)(p0 + q) * 3 + al) * KK + c];
        } else if (src) {
          x = src[c];
        }
        g = fmaf(x, B[(size_t)ce * KK + c], g);
      }
      const __nv_bfloat16 h = __float2bfloat16_rn(x);
      hi[row * KP + c] = h;
      lo[row * KP + c] = __float2bfloat16_rn(x - __bfloat162float(h));
    }
    for (int o = 16; o > 0; o >>= 1) g += __shfl_xor_sync(0xffffffffu, g, o);
    if (lane == 0 && al < 3) {
      float* r = vrec + 8 * ((size_t)m.vr0 + vl);
      r[4 + al] = g;
      if (al == 0) {
        float f1 = 0.f, f2 = 0.f;
        if (valid) {
          const float4 a4 = *reinterpret_cast<const float4*>(at + 4 * (size_t)ce);
          const float sg = v == 0 ? 1.f : -1.f;
          if (a4.w != 0.f) {
            f1 = sg / a4.y;
            f2 = a4.z / (2.f * a4.x) * f1;
          }
        }
        r[0] = __int_as_float(ce);
        r[1] = f1;
        r[2] = f2;
        r[3] = 0.f;
        r[7] = 0.f;
      }
    }
  }
}

namespace {
// the R values g of a vector record
template <int R>
__device__ __forceinline__ void load_g(const float4* p, float* g) {
  static_assert(R == 3 || R == 6, "force (3) or stress (6) components");
  const float4 a = p[0];
  g[0] = a.x, g[1] = a.y, g[2] = a.z;
  if constexpr (R == 6) {
    const float4 b = p[1];
    g[3] = a.w, g[4] = b.x, g[5] = b.y;
  }
}
// 3 x 8 consecutive TMEM columns (at taddr, taddr + stride, taddr + 2 stride) of the warp's 32
// lanes into registers, waited for inside the same statement
__device__ __forceinline__ void tmem_ld3x8(uint32_t taddr, uint32_t stride, float* out) {
  uint32_t v[24];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%24];\n"
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%8,%9,%10,%11,%12,%13,%14,%15}, [%25];\n"
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%16,%17,%18,%19,%20,%21,%22,%23}, [%26];\n"
      "tcgen05.wait::ld.sync.aligned;\n"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
        "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]),
        "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23])
      : "r"(taddr), "r"(taddr + stride), "r"(taddr + 2 * stride)
      : "memory");
#pragma unroll
  for (int c = 0; c < 24; ++c) out[c] = __uint_as_float(v[c]);
}
}  // namespace

// CTA (blockIdx.x = 128-point tile of Z, blockIdx.y = g): atom tiles t = g, g + G, ... of the
// chunk.  Shared memory: the Z tile (nkb K blocks x hi, lo), `stages` V tile stages (nkb x hi, lo
// blocks of vrows rows, vrows >= the largest N of the chunk; the loads of the next tiles overlap
// the MMAs of the current one), the vector records of three tiles (the current one, the next one whose
// kernel features are being fetched, and the one after, being staged), and the quarters' partial
// sums of two tiles.  The epilogue fetches the kernel features of tile i + 1 into registers
// before it waits for the accumulator of tile i + 1.  P: the kernel power when it is a small
// integer (1-4), 0 for any other power (powf).
template <int P, int R>
__global__ void __launch_bounds__(kKThreads, 1)
    k_krr_force_tc(const __grid_constant__ CUtensorMap vhi, const __grid_constant__ CUtensorMap vlo,
                   const __grid_constant__ CUtensorMap zhi, const __grid_constant__ CUtensorMap zlo, int ntiles,
                   int nkb, int stages, int vrows, int nvr, int nk, const TileMeta* __restrict__ tmeta,
                   const float4* __restrict__ vrec,
                   const float* __restrict__ F, const float* __restrict__ szz, float s2, float l2, float pw,
                   const long long* __restrict__ trow, const int* __restrict__ gstart, int c0, int ldx,
                   float* __restrict__ X, int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* ztile = reinterpret_cast<unsigned char*>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  const uint32_t zbytes = (uint32_t)nkb * 2 * kTileBytes;
  const uint32_t vblk = (uint32_t)vrows * kTK * 2;  // one K block of one plane
  const uint32_t sbytes = (uint32_t)nkb * 2 * vblk;  // one stage
  const int nvmax = nvr;  // record rows per buffer: the chunk's largest nvp
  unsigned char* vtile = ztile + zbytes;
  constexpr int RECS = recs_of(R);
  constexpr int NCH = (max_tile_vectors(1, R) / 8 + 3) / 4;  // vector chunks per epilogue warp and tile
  float4* srec = reinterpret_cast<float4*>(vtile + (size_t)stages * sbytes);  // [3][RECS nvmax]
  float* red = reinterpret_cast<float*>(srec + 3 * RECS * nvmax);            // [2][4][R][4][32]
  int* sce = reinterpret_cast<int*>(red + 2 * 4 * R * 4 * 32);               // [3][nvmax] centres
  uint64_t* bfull = reinterpret_cast<uint64_t*>(sce + 3 * nvmax);
  uint64_t* full = bfull + 1;                 // [kMaxStages]
  uint64_t* empty = full + kMaxStages;        // [kMaxStages]
  uint64_t* tfull = empty + kMaxStages;       // [2] accumulator ready
  uint64_t* tempty = tfull + 2;               // [2] accumulator drained
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(tempty + 2);

  const int n0 = blockIdx.x * kTM;
  // the CTA's tiles: the contiguous range [gstart[g], gstart[g + 1]) of the chunk, so that the
  // tiles of one owner (atom or structure) are added to its rows by one CTA, in order
  const int g = blockIdx.y;
  const int t0 = gstart[g];
  const int nmine = gstart[g + 1] - t0;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    ptx::mbar_init(bfull, 1);
    for (int st = 0; st < stages; ++st) {
      ptx::mbar_init(&full[st], 1);
      ptx::mbar_init(&empty[st], 1);
    }
    for (int b = 0; b < 2; ++b) {
      ptx::mbar_init(&tfull[b], 1);
      ptx::mbar_init(&tempty[b], kKEpiWarps);
    }
    ptx::mbar_init_fence();
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(ptx::smem_u32(tmem_slot)),
                 "n"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = *tmem_slot;
  bool ok = true;

  if (warp == 0 && lane == 0) {
    // producer: the Z tile once, then the atom tiles in 32-row boxes (the rows past a tile's N
    // belong to the next tile or to the chunk's spare rows and feed unused accumulator columns)
    ptx::mbar_expect_tx(bfull, zbytes);
    for (int kb = 0; kb < nkb; ++kb) {
      ptx::tma_load_2d(ztile + (2 * kb) * kTileBytes, &zhi, kb * kTK, n0, bfull);
      ptx::tma_load_2d(ztile + (2 * kb + 1) * kTileBytes, &zlo, kb * kTK, n0, bfull);
    }
    int issued = 0;
    for (int i = 0; i < nmine; ++i) {
      const int st = i % stages;
      if (i >= stages && !ptx::mbar_wait_sleep(&empty[st], ((i / stages) - 1) & 1)) {
        ok = false;
        break;
      }
      const TileMeta m = tmeta[t0 + i];
      const int nbox = (m.N + kBoxRows - 1) / kBoxRows;
      unsigned char* vs = vtile + (size_t)st * sbytes;
      ptx::mbar_expect_tx(&full[st], (uint32_t)(nkb * 2 * nbox * kBoxBytes));
      for (int kb = 0; kb < nkb; ++kb)
        for (int j = 0; j < nbox; ++j) {
          ptx::tma_load_2d(vs + (2 * kb) * vblk + j * kBoxBytes, &vhi, kb * kTK, m.row0 + j * kBoxRows, &full[st]);
          ptx::tma_load_2d(vs + (2 * kb + 1) * vblk + j * kBoxBytes, &vlo, kb * kTK, m.row0 + j * kBoxRows,
                           &full[st]);
        }
      issued = i + 1;
    }
    // copies still in flight are waited for (bounded) before leaving
    for (int i = max(0, issued - stages); i < issued; ++i) ptx::mbar_wait(&full[i % stages], (i / stages) & 1);
    ptx::mbar_wait(bfull, 0);
  } else if (warp == 1 && lane == 0) {
    // MMA issuer: atom tile i into TMEM buffer i & 1 (columns 256 (i & 1) + [0, N))
    if (nmine > 0 && !ptx::mbar_wait(bfull, 0)) ok = false;
    const uint32_t sz = ptx::smem_u32(ztile), sv = ptx::smem_u32(vtile);
    for (int i = 0; i < nmine && ok; ++i) {
      const int b = i & 1;
      if (i >= 2 && !ptx::mbar_wait_sleep(&tempty[b], ((i >> 1) - 1) & 1)) {
        ok = false;
        break;
      }
      const int st = i % stages;
      if (!ptx::mbar_wait_sleep(&full[st], (i / stages) & 1)) {
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint32_t idesc = tc::idesc_m128(tmeta[t0 + i].N);
      const uint32_t acc = tmem + (uint32_t)(b * (kTmemCols / 2));
      const uint32_t svs = sv + (uint32_t)st * sbytes;
      for (int kb = 0; kb < nkb; ++kb) {
#pragma unroll
        for (int kk = 0; kk < kTK / 16; ++kk) {
          const uint32_t off = kk * 32;  // 16 bf16 along K inside the 128-byte swizzle row
          const uint64_t zh = tc::sw128_desc(sz + (2 * kb) * kTileBytes + off);
          const uint64_t zl = tc::sw128_desc(sz + (2 * kb + 1) * kTileBytes + off);
          const uint64_t vh = tc::sw128_desc(svs + (2 * kb) * vblk + off);
          const uint64_t vl = tc::sw128_desc(svs + (2 * kb + 1) * vblk + off);
          tc::mma_bf16_id(acc, zh, vh, idesc, (kb > 0 || kk > 0) ? 1u : 0u);
          tc::mma_bf16_id(acc, zl, vh, idesc, 1u);
          tc::mma_bf16_id(acc, zh, vl, idesc, 1u);
        }
      }
      tc::mma_commit(&empty[st]);  // frees the stage once these MMAs have read it
      tc::mma_commit(&tfull[b]);
    }
  } else if (warp >= 2) {
    // epilogue: lane quarter q (reference points n0 + 32 q + lane), vector chunks sub, sub + 4, ...
    const int q = warp & 3, sub = (warp - 2) >> 2;
    const int etid = threadIdx.x - 64;  // 0 .. 511 over the epilogue warps
    const int k = n0 + q * 32 + lane;
    const bool kv = k < nk;
    const float il2 = 1.f / l2;
    const float izk = kv ? 1.f / szz[k] : 0.f;  // zero past nk: every coefficient vanishes
    // per vector v: c1 = k1 f1_v b^(p-1), c2 = izk f2_v b^p with b = s2 + F[centre, k] / l2; the
    // sums over v keep the per-point factors k1, izk outside
    const float k1 = pw * il2 * izk;
    // the records of tile j into buffer j % 3 (two float4 per vector) and its centres: a tile
    // has at most 2 nvmax <= 160 float4, one per epilogue thread, loaded into registers a whole
    // iteration before they are stored
    static_assert(RECS * max_tile_vectors(1, R) <= kKEpiWarps * 32, "one record float4 per epilogue thread");
    float4 rv = make_float4(0.f, 0.f, 0.f, 0.f);
    auto stage_load = [&](int j) {
      if (j >= nmine) return;
      const TileMeta m = tmeta[t0 + j];
      if (etid < RECS * m.nvp) rv = vrec[RECS * (size_t)m.vr0 + etid];
    };
    auto stage_store = [&](int j) {
      if (j >= nmine) return;
      if (etid < RECS * tmeta[t0 + j].nvp) {
        srec[(j % 3) * RECS * nvmax + etid] = rv;
        if (etid % RECS == 0) sce[(j % 3) * nvmax + etid / RECS] = __float_as_int(rv.x);
      }
    };
    // the kernel features F[centre of v, k] of the warp's vectors of tile j (coalesced rows)
    float xf[NCH][8];
    auto fetch = [&](int j) {
      if (j >= nmine) return;
      const int nch = tmeta[t0 + j].nvp >> 3;
      const int* ce = sce + (j % 3) * nvmax;
#pragma unroll
      for (int cc = 0; cc < NCH; ++cc) {
        const int c = sub + 4 * cc;
        int cv[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        if (c < nch) {
          const int4 lo = *reinterpret_cast<const int4*>(ce + c * 8);
          const int4 hi = *reinterpret_cast<const int4*>(ce + c * 8 + 4);
          cv[0] = lo.x, cv[1] = lo.y, cv[2] = lo.z, cv[3] = lo.w;
          cv[4] = hi.x, cv[5] = hi.y, cv[6] = hi.z, cv[7] = hi.w;
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) xf[cc][u] = (c < nch && kv) ? __ldg(F + (size_t)cv[u] * nk + k) : 0.f;
      }
    };
    stage_load(0);
    stage_store(0);
    stage_load(1);
    stage_store(1);
    asm volatile("bar.sync 1, %0;" ::"n"(kKEpiWarps * 32));
    fetch(0);
    bool got = true;
    for (int i = 0; i < nmine; ++i) {
      const int b = i & 1;
      const TileMeta m = tmeta[t0 + i];
      const long long xr = trow[t0 + i];
      stage_load(i + 2);
      // the accumulator; the barrier also publishes the records staged one tile earlier, and a
      // timed-out wait in any epilogue warp ends the loop for all of them together
      const bool ready = ptx::mbar_wait(&tfull[b], (i >> 1) & 1);
      int any_fail;
      asm volatile(
          "{\n .reg .pred pf, pr;\n setp.eq.u32 pf, %1, 0;\n bar.red.or.pred pr, 2, %2, pf;\n selp.u32 %0, 1, 0, pr;\n}\n"
          : "=r"(any_fail)
          : "r"((unsigned)ready), "n"(kKEpiWarps * 32));
      if (any_fail) {
        got = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;");
      const float4* s = srec + (i % 3) * RECS * nvmax;
      const int nch = m.nvp >> 3;
      const uint32_t tq = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * (kTmemCols / 2));
      // sum_v f1 b^(p-1) (V.z) and sum_v f2 b^p (V.x_centre) per alpha
      float sq[R], tq2[R];
#pragma unroll
      for (int c = 0; c < R; ++c) sq[c] = tq2[c] = 0.f;
#pragma unroll
      for (int cc = 0; cc < NCH; ++cc) {
        const int c = sub + 4 * cc;
        if (c < nch) {
          // three components: the accumulator columns first, so that their load overlaps the
          // coefficients; six: coefficients first, then three columns at a time (registers)
          float d0[24];
          if constexpr (R == 3) tmem_ld3x8(tq + (uint32_t)(c * 8), (uint32_t)m.nvp, d0);
          // per vector: e1 = f1 b^(p-1), e2 = f2 b^p; the g sums need no accumulator values
          float e1[8];
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            const float4 r = s[RECS * (c * 8 + u)];
            float gv[R];
            load_g<R>(s + RECS * (c * 8 + u) + 1, gv);
            const float base = fmaf(xf[cc][u], il2, s2);
            float bp1;  // base^(p - 1)
            if constexpr (P == 0) {
              bp1 = powf(base, pw - 1.f);
            } else {
              bp1 = 1.f;
#pragma unroll
              for (int j = 1; j < P; ++j) bp1 *= base;
            }
            e1[u] = r.y * bp1;
            const float e2 = r.z * (bp1 * base);
#pragma unroll
            for (int q2 = 0; q2 < R; ++q2) tq2[q2] = fmaf(e2, gv[q2], tq2[q2]);
          }
          // the accumulator columns, three components at a time
#pragma unroll
          for (int h = 0; h < R / 3; ++h) {
            float d[24];
            if constexpr (R == 3) {
#pragma unroll
              for (int x = 0; x < 24; ++x) d[x] = d0[x];
            } else {
              tmem_ld3x8(tq + (uint32_t)(c * 8 + 3 * h * m.nvp), (uint32_t)m.nvp, d);
            }
#pragma unroll
            for (int u = 0; u < 8; ++u)
#pragma unroll
              for (int q2 = 0; q2 < 3; ++q2) sq[3 * h + q2] = fmaf(e1[u], d[8 * q2 + u], sq[3 * h + q2]);
          }
        }
      }
      float av[R];
#pragma unroll
      for (int q2 = 0; q2 < R; ++q2) av[q2] = fmaf(k1, sq[q2], -izk * tq2[q2]);
      asm volatile("tcgen05.fence::before_thread_sync;");
      __syncwarp();
      if (lane == 0) ptx::mbar_arrive(&tempty[b]);
      // the quarter's four partial sums per alpha, added in a fixed order
      float* rq = red + (size_t)((i & 1) * 4 + q) * R * 4 * 32;  // [component][sub][lane]
#pragma unroll
      for (int q2 = 0; q2 < R; ++q2) rq[(q2 * 4 + sub) * 32 + lane] = av[q2];
      asm volatile("bar.sync %0, %1;" ::"r"(4 + q), "n"(128));
      for (int q2 = sub; q2 < R; q2 += 4) {
        const float* ra = rq + q2 * 4 * 32 + lane;
        const float sum = ((ra[0] + ra[32]) + ra[64]) + ra[96];
        if (kv && xr >= 0 && sum != 0.f) atomicAdd(&X[(xr + q2) * ldx + c0 + k], sum);
      }
      stage_store(i + 2);
      fetch(i + 1);
    }
    if (!got && lane == 0) atomicExch(err, 1);
  }
  if (!ok) atomicExch(err, 1);
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "n"(kTmemCols));
  }
}

bool krr_force_tc_available() { return tc::encode_fn() != nullptr; }

// Stress tiles: tile = a run of <= max_tile_vectors(nkb, 6) atoms of one structure (TileMeta.atom
// holds the structure, v0 its first atom within the structure).  Rows: Ts[a][sigma] (the stress
// partials of k_krr_stress_atom, sigma-major, nvp rows per component); records {atom, sc / sqrt
// f(x,x), sc dker_xx / (2 f(x,x) sqrt f(x,x)), 0}, {tx[a][0..3]}, {tx[a][4..5], 0, 0} with
// sc = sign_stress * 3 / volume (the normalisation of k_krr_stress_tiled).
__global__ void __launch_bounds__(128) k_ktc_splanes(const TileMeta* __restrict__ tmeta, int KK, int KP,
                                                     const int* __restrict__ atom_start, const float* __restrict__ Ts,
                                                     const float* __restrict__ tx, const float* __restrict__ at,
                                                     const double* __restrict__ volume, double sign_stress,
                                                     const long long* __restrict__ rowS,
                                                     __nv_bfloat16* __restrict__ hi, __nv_bfloat16* __restrict__ lo,
                                                     float* __restrict__ vrec, long long* __restrict__ trow) {
  const TileMeta m = tmeta[blockIdx.x];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int sidx = m.atom, a0 = atom_start[sidx] + m.v0;
  if (threadIdx.x == 0) trow[blockIdx.x] = rowS[sidx];
  const float sc = (float)(sign_stress * 3.0 / volume[sidx]);
  for (int lr = warp; lr < m.N; lr += 4) {
    const long long row = (long long)m.row0 + lr;
    const int q = lr / m.nvp, vl = lr - q * m.nvp;
    const bool valid = q < 6 && vl < m.nvt;
    const int a = valid ? a0 + vl : a0;
    for (int c = lane; c < KP; c += 32) {
      const float x = (valid && c < KK) ? Ts[((size_t)a * 6 + q) * KK + c] : 0.f;
      const __nv_bfloat16 h = __float2bfloat16_rn(x);
      hi[row * KP + c] = h;
      lo[row * KP + c] = __float2bfloat16_rn(x - __bfloat162float(h));
    }
    if (lane == 0 && q < 6) {
      float* r = vrec + 12 * ((size_t)m.vr0 + vl);
      r[4 + q] = valid ? tx[6 * (size_t)a + q] : 0.f;
      if (q == 0) {
        float f1 = 0.f, f2 = 0.f;
        if (valid) {
          const float4 a4 = *reinterpret_cast<const float4*>(at + 4 * (size_t)a);
          if (a4.w != 0.f) {
            f1 = sc / a4.y;
            f2 = a4.z / (2.f * a4.x) * f1;
          }
        }
        r[0] = __int_as_float(a);
        r[1] = f1;
        r[2] = f2;
        r[3] = 0.f;
        r[10] = 0.f;
        r[11] = 0.f;
      }
    }
  }
}

namespace {
size_t al256(size_t x) { return (x + 255) / 256 * 256; }
// split of a group of nv vectors into tiles: count, and vectors of tile j
int tiles_of(int nv, int nvmax) { return (nv + nvmax - 1) / nvmax; }
int tile_vectors(int nv, int ns, int j) { return nv / ns + (j < nv % ns ? 1 : 0); }
int rows_of(int nvp, int R) { return (R * nvp + 15) / 16 * 16; }
// workspace of a chunk: planes (with a spare box of rows), vector records, tile records and rows
constexpr int kMaxGroups = 1024;  // CTAs per column tile (<= SMs)
size_t chunk_bytes(size_t rows, size_t vecs, size_t tiles, int KP, int R) {
  return 2 * al256((rows + kBoxRows) * (size_t)KP * 2) + al256(vecs * 16 * recs_of(R)) +
         al256(tiles * sizeof(TileMeta)) + al256(tiles * sizeof(long long)) + al256(sizeof(int) * (kMaxGroups + 1));
}
// the tiles of a group of nv vectors owned by `owner` (row0 and vr0 are set per chunk)
void push_tiles(std::vector<TileMeta>& tiles, int owner, int nv, int nvmax, int R) {
  const int ns = tiles_of(nv, nvmax);
  for (int j = 0, v0 = 0; j < ns; ++j) {
    const int nvt = tile_vectors(nv, ns, j), nvp = (nvt + 7) / 8 * 8;
    tiles.push_back(TileMeta{owner, 0, rows_of(nvp, R), nvp, 0, v0, nvt, 0});
    v0 += nvt;
  }
}
size_t fixed_smem(int nkb, int nvr, int R) {
  return 1024 + (size_t)nkb * 2 * kTileBytes + 3 * (size_t)recs_of(R) * nvr * 16 + 2 * 4 * (size_t)R * 4 * 32 * 4 +
         3 * (size_t)nvr * 4 + 8 * (1 + 2 * kMaxStages + 4) + 8;
}
constexpr size_t kSmemMax = 227 * 1024;

using ForceKernel = void (*)(CUtensorMap, CUtensorMap, CUtensorMap, CUtensorMap, int, int, int, int, int, int,
                             const TileMeta*, const float4*, const float*, const float*, float, float, float,
                             const long long*, const int*, int, int, float*, int*);
template <int R>
ForceKernel kernel_for(int P) {
  return P == 1 ? k_krr_force_tc<1, R> : P == 2 ? k_krr_force_tc<2, R> : P == 3 ? k_krr_force_tc<3, R>
       : P == 4 ? k_krr_force_tc<4, R> : k_krr_force_tc<0, R>;
}

// shared state of the force and stress passes
struct PassCtx {
  int nkb, KP, nk, NT, nsm;
  CUtensorMap mzh, mzl;
  unsigned char* chunk_ws;  // after the Z planes
  size_t room;
  const float* F;
  const float* szz;
  float s2, l2, pw;
  int P, c0, ldx;
  float* X;
  int* err;
  cudaStream_t st;
};

// Runs `tiles` in chunks that fit the workspace: `build` writes a chunk's planes, records and
// tile rows, then the tensor-core kernel adds the chunk's rows into X.
template <int R, typename Build>
cudaError_t run_tiles(const std::vector<TileMeta>& tiles, const PassCtx& c, Build build, int* launches) {
  ForceKernel kern = kernel_for<R>(c.P);
  static bool attr[5] = {false, false, false, false, false};
  if (!attr[c.P]) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemMax);
    if (e != cudaSuccess) return e;
    attr[c.P] = true;
  }
  std::vector<TileMeta> meta;
  for (size_t i0 = 0; i0 < tiles.size();) {
    meta.clear();
    size_t nrows = 0, nvecs = 0, i1 = i0;
    while (i1 < tiles.size()) {
      TileMeta m = tiles[i1];
      if (chunk_bytes(nrows + m.N, nvecs + m.nvp, meta.size() + 1, c.KP, R) > c.room) break;
      m.row0 = (int)nrows;
      m.vr0 = (int)nvecs;
      meta.push_back(m);
      nrows += m.N;
      nvecs += m.nvp;
      ++i1;
    }
    if (i1 == i0) return cudaErrorInvalidValue;  // one tile alone exceeds the workspace
    const size_t nt = meta.size();
    // shared memory: everything but the V stages, then as many stages of the chunk's largest
    // tile as fit (at least one stage of max_tile_rows rows does)
    int maxN = 0, nvr = 8;
    for (const TileMeta& m : meta) {
      maxN = std::max(maxN, m.N);
      nvr = std::max(nvr, m.nvp);
    }
    const int vrows = (maxN + kBoxRows - 1) / kBoxRows * kBoxRows;
    const size_t sbytes = (size_t)c.nkb * 2 * vrows * kTK * 2;
    const size_t fixed = fixed_smem(c.nkb, nvr, R);
    const int stages = (int)std::min<size_t>(kMaxStages, (kSmemMax - fixed) / sbytes);
    if (stages < 1) return cudaErrorInvalidValue;
    const size_t smem = fixed + (size_t)stages * sbytes;
    unsigned char* p = c.chunk_ws;
    __nv_bfloat16* vhi = reinterpret_cast<__nv_bfloat16*>(p);
    p += al256((nrows + kBoxRows) * c.KP * 2);
    __nv_bfloat16* vlo = reinterpret_cast<__nv_bfloat16*>(p);
    p += al256((nrows + kBoxRows) * c.KP * 2);
    float* vrec = reinterpret_cast<float*>(p);
    p += al256(nvecs * 16 * recs_of(R));
    TileMeta* dmeta = reinterpret_cast<TileMeta*>(p);
    p += al256(sizeof(TileMeta) * nt);
    long long* trow = reinterpret_cast<long long*>(p);
    p += al256(sizeof(long long) * nt);
    int* dgs = reinterpret_cast<int*>(p);
    // one CTA per SM: the column tiles times G row groups in a single wave; group g takes the
    // contiguous tiles [gs[g], gs[g + 1]), about 1/G of the rows each, cut only between owners
    const int G = std::max(1, std::min<int>({(int)nt, c.NT >= c.nsm ? 1 : c.nsm / c.NT, kMaxGroups}));
    std::vector<int> gs(G + 1, (int)nt);
    gs[0] = 0;
    {
      size_t acc = 0;
      int gi = 1;
      for (size_t t = 0; t < nt && gi < G; ++t) {
        acc += (size_t)meta[t].N;
        const bool boundary = t + 1 == nt || meta[t + 1].atom != meta[t].atom;
        while (gi < G && boundary && acc * (size_t)G >= (size_t)gi * nrows) gs[gi++] = (int)(t + 1);
      }
    }
    cudaError_t e = cudaMemcpyAsync(dmeta, meta.data(), sizeof(TileMeta) * nt, cudaMemcpyHostToDevice, c.st);
    if (e != cudaSuccess) return e;
    e = cudaMemcpyAsync(dgs, gs.data(), sizeof(int) * (G + 1), cudaMemcpyHostToDevice, c.st);
    if (e != cudaSuccess) return e;
    build(dmeta, (int)nt, vhi, vlo, vrec, trow);
    CUtensorMap mvh, mvl;
    if (!tc::make_plane_map(&mvh, vhi, c.KP, (long long)(nrows + kBoxRows), c.KP, kBoxRows) ||
        !tc::make_plane_map(&mvl, vlo, c.KP, (long long)(nrows + kBoxRows), c.KP, kBoxRows))
      return cudaErrorInvalidValue;
    kern<<<dim3((unsigned)c.NT, (unsigned)G), kKThreads, smem, c.st>>>(
        mvh, mvl, c.mzh, c.mzl, (int)nt, c.nkb, stages, vrows, nvr, c.nk, dmeta,
        reinterpret_cast<const float4*>(vrec), c.F, c.szz, c.s2, c.l2, c.pw, trow, dgs, c.c0, c.ldx, c.X, c.err);
    *launches += 2;
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    // the host records of the next chunk overwrite dmeta only after this chunk's kernels
    e = cudaStreamSynchronize(c.st);
    if (e != cudaSuccess) return e;
    i0 = i1;
  }
  return cudaSuccess;
}
}  // namespace

size_t krr_force_tc_workspace_bytes(long long atoms, int maxnv, int nk, int KK) {
  const int nkb = (KK + kTK - 1) / kTK, KP = nkb * kTK;
  const int nvmax = max_tile_vectors(std::min(nkb, 3));
  const int ns = tiles_of(std::max(maxnv, 1), nvmax);
  const int nvp = (tile_vectors(std::max(maxnv, 1), ns, 0) + 7) / 8 * 8;
  const size_t tiles = (size_t)atoms * ns;
  return 2 * al256((size_t)nk * KP * 2) + 8 * 256 +
         chunk_bytes(tiles * rows_of(nvp, 3), tiles * nvp, tiles, KP, 3);
}

// Force and stress rows of the kernel block (columns [c0, c0 + nk) of X), replacing
// k_krr_force_tiled and k_krr_stress_tiled for the FP32 rows.  ws (ws_bytes) holds the Z planes
// and, per chunk of tiles, the row planes and their vector and tile records; chunks are as large
// as ws allows.  F, at, szz: the kernel features, atom terms and point norms of launch_krr_rows;
// Ts, tx: the stress partials of k_krr_stress_atom.  X must hold zeros in these columns (the sums
// are added atomically).
cudaError_t launch_krr_force_tc(const DevBatch& b, const DevRows& rows, const int* rev, const float* Bq,
                                const float* dBq, const float* Z, const float* F, const float* at, const float* szz,
                                const float* Ts, const float* tx, double sign_stress, int nk, int KK, double power,
                                double length, double sigma, void* ws, size_t ws_bytes, float* X, int c0, int* err,
                                int nsm, cudaStream_t st, int* launches) {
  *launches = 0;
  if (b.A == 0 || nk == 0) return cudaSuccess;
  const int nkb = (KK + kTK - 1) / kTK;
  const int KP = nkb * kTK;
  if (KK > kKrrTcMaxK) return cudaErrorInvalidValue;  // K blocks beyond the shared-memory budget
  const int nvmax3 = max_tile_vectors(nkb, 3), nvmax6 = max_tile_vectors(nkb, 6);
  if (fixed_smem(nkb, nvmax3, 3) + (size_t)nkb * 2 * max_tile_rows(nkb) * kTK * 2 > kSmemMax ||
      fixed_smem(nkb, nvmax6, 6) + (size_t)nkb * 2 * max_tile_rows(nkb) * kTK * 2 > kSmemMax)
    return cudaErrorInvalidValue;
  // tiles: per atom its derivative vectors (force), per structure its atoms (stress)
  std::vector<int> off(b.A + 1), ast(b.S + 1);
  cudaError_t e = cudaMemcpyAsync(off.data(), b.nbr_off, sizeof(int) * (b.A + 1), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(ast.data(), b.atom_start, sizeof(int) * (b.S + 1), cudaMemcpyDeviceToHost, st);
  if (e != cudaSuccess) return e;
  e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return e;
  std::vector<TileMeta> ftiles, stiles;
  for (int a = 0; a < b.A; ++a) push_tiles(ftiles, a, off[a + 1] - off[a] + 1, nvmax3, 3);
  for (int s = 0; s < b.S; ++s)
    if (ast[s + 1] > ast[s]) push_tiles(stiles, s, ast[s + 1] - ast[s], nvmax6, 6);
  // workspace: Z planes, then the chunks
  PassCtx c{};
  unsigned char* w = static_cast<unsigned char*>(ws);
  const size_t zb = al256((size_t)nk * KP * 2);
  __nv_bfloat16* zhi = reinterpret_cast<__nv_bfloat16*>(w);
  __nv_bfloat16* zlo = reinterpret_cast<__nv_bfloat16*>(w + zb);
  if (ws_bytes < 2 * zb + 8 * 256) return cudaErrorInvalidValue;
  c.chunk_ws = w + 2 * zb;
  c.room = ws_bytes - 2 * zb - 8 * 256;
  {
    const long long n = (long long)nk * KP;
    k_ktc_zplanes<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(Z, nk, KK, KP, zhi, zlo);
    ++*launches;
  }
  if (!tc::make_plane_map(&c.mzh, zhi, KP, nk, KP) || !tc::make_plane_map(&c.mzl, zlo, KP, nk, KP))
    return cudaErrorInvalidValue;
  c.nkb = nkb;
  c.KP = KP;
  c.nk = nk;
  c.NT = (nk + kTM - 1) / kTM;
  c.nsm = nsm;
  c.F = F;
  c.szz = szz;
  c.s2 = (float)(sigma * sigma);
  c.l2 = (float)(2.0 * length * length);
  c.pw = (float)power;
  const int ip = (int)power;
  c.P = ((double)ip == power && ip >= 1 && ip <= 4) ? ip : 0;
  c.c0 = c0;
  c.ldx = rows.ldx;
  c.X = X;
  c.err = err;
  c.st = st;
  int nl = 0;
  e = run_tiles<3>(ftiles, c,
                   [&](const TileMeta* dm, int nt, __nv_bfloat16* vhi, __nv_bfloat16* vlo, float* vrec,
                       long long* trow) {
                     k_ktc_vplanes<<<(unsigned)nt, 128, 0, st>>>(dm, KK, KP, b.nbr_off, b.nbr_idx, rev, Bq, dBq, at,
                                                                 vhi, vlo, vrec, b.atom_struct, b.atom_start,
                                                                 rows.rowF, trow);
                   },
                   &nl);
  *launches += nl;
  if (e != cudaSuccess) return e;
  nl = 0;
  e = run_tiles<6>(stiles, c,
                   [&](const TileMeta* dm, int nt, __nv_bfloat16* vhi, __nv_bfloat16* vlo, float* vrec,
                       long long* trow) {
                     k_ktc_splanes<<<(unsigned)nt, 128, 0, st>>>(dm, KK, KP, b.atom_start, Ts, tx, at, b.volume,
                                                                 sign_stress, rows.rowS, vhi, vlo, vrec, trow);
                   },
                   &nl);
  *launches += nl;
  return e;
}

}  // namespace mld
