// Force rows of the kernel model on the tensor cores (mixed method).
//
// The force row of atom a for reference point k (compute_kernel.F90:476-866, mld_forces.F90:
// 268-320) is a sum over the derivative vectors of a: its own pair sum (v = 0, centre a, sign +1)
// and the reversed pairs j -> a (v >= 1, centre j, sign -1):
//   row(a, alpha, k) = sum_v sign_v (c1(ce_v, k) (V_{v,alpha} . z_k) - c2(ce_v, k) (V_{v,alpha} . x_{ce_v}))
// The products V . z_k over all rows and reference points are one large GEMM, V (rows x KK) times
// Z^T (KK x nk), which this file runs on the 5th-generation tensor cores in BF16 split precision
// (v = hi + lo; hi hi + hi lo + lo hi, three MMAs per K step, FP32 accumulation of KK <= 192
// products in TMEM), with the coefficient transform and the sum over v in the epilogue:
//   * operands: V and Z as K-major bf16 hi/lo planes, K padded to a multiple of 64;
//   * rows of an atom are laid out alpha-major, each alpha padded to a multiple of 32 rows, and
//     every atom starts on a 128-row tile: a 32-row TMEM lane quarter then holds one atom and
//     one alpha, and a warp's 32 x 32 block reduces over its rows with a shuffle butterfly;
//   * CTA = one 128-point tile of Z (resident in shared memory) and a strided set of row tiles,
//     with the Gram kernel's roles: TMA producer warp, MMA warp (two TMEM accumulators), sixteen
//     epilogue warps; the per-quarter sums are added to the force rows with FP32 atomics.
// Every mbarrier wait is bounded: on expiry the CTA sets *err, waits (bounded) for its copies in
// flight and frees its TMEM.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "krr.cuh"
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

struct TileMeta {
  int atom;  // target atom (batch index)
  int ti;    // tile index within the atom
  int nvp;   // rows per alpha of the atom (multiple of 32)
  int nv;    // derivative vectors of the atom (its neighbours + 1)
};
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

// Derivative vectors of atoms [a0, a1) as bf16 hi/lo planes (KP per row) plus per-row
// centre, sign and g = V . x_centre.  One CTA (4 warps) per atom; warp w builds rows w, w + 4, ...
// of the atom's tiles.  tile0[a - a0] is the atom's first tile within the chunk.
__global__ void __launch_bounds__(128) k_ktc_vplanes(int a0, int a1, int KK, int KP, const int* __restrict__ nbr_off,
                                                     const int* __restrict__ nbr_idx, const int* __restrict__ rev,
                                                     const float* __restrict__ B, const float* __restrict__ dB,
                                                     const int* __restrict__ tile0, __nv_bfloat16* __restrict__ hi,
                                                     __nv_bfloat16* __restrict__ lo, int* __restrict__ rce,
                                                     float* __restrict__ rsg, float* __restrict__ rg) {
  const int a = a0 + blockIdx.x;
  if (a >= a1) return;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int p0 = nbr_off[a], nn = nbr_off[a + 1] - p0, nv = nn + 1;
  const int nvp = (nv + 31) / 32 * 32;
  const int t0 = tile0[a - a0], nt = tile0[a - a0 + 1] - t0;
  for (int lr = warp; lr < nt * kTM; lr += 4) {
    const long long row = (long long)t0 * kTM + lr;
    const int al = lr / nvp, v = lr - al * nvp;
    const bool valid = al < 3 && v < nv;
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
    if (lane == 0) {
      rce[row] = ce;
      rsg[row] = valid ? (v == 0 ? 1.f : -1.f) : 0.f;
      rg[row] = g;
    }
  }
}

// CTA (blockIdx.x = 128-point tile of Z, blockIdx.y = g): row tiles t = g, g + G, ... of the
// chunk.  Shared memory: the Z tile (nkb K blocks x hi, lo), `stages` row-tile stages, and the
// coefficient table of the current tile's atom: (c1, c2) per (reference point, derivative
// vector), tab[k * (tabv + 1) + v], filled with coalesced loads of the kernel features while the
// MMAs of the tile run (an atom with more than tabv vectors reads them per element instead).
__global__ void __launch_bounds__(kKThreads, 1)
    k_krr_force_tc(const __grid_constant__ CUtensorMap vhi, const __grid_constant__ CUtensorMap vlo,
                   const __grid_constant__ CUtensorMap zhi, const __grid_constant__ CUtensorMap zlo, int ntiles,
                   int nkb, int stages, int nk, const TileMeta* __restrict__ tmeta, const int* __restrict__ rce,
                   const float* __restrict__ rsg, const float* __restrict__ rg, const float* __restrict__ F,
                   const float* __restrict__ at, const float* __restrict__ szz, float s2, float l2, float pw,
                   const int* __restrict__ atom_struct, const int* __restrict__ atom_start,
                   const long long* __restrict__ rowF, int c0, int ldx, float* __restrict__ X, int tabv,
                   int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* btile = reinterpret_cast<unsigned char*>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  const uint32_t opb = (uint32_t)nkb * 2 * kTileBytes;  // bytes of one operand tile set (hi and lo blocks)
  unsigned char* atile = btile + opb;
  float2* tab = reinterpret_cast<float2*>(atile + (size_t)stages * opb);  // kTM x (tabv + 1)
  float* iszz = reinterpret_cast<float*>(tab + (size_t)kTM * (tabv + 1));  // kTM: 1 / szz of the CTA's points
  float2* fac = reinterpret_cast<float2*>(iszz + kTM);                      // tabv: per-vector centre factors
  uint64_t* bfull = reinterpret_cast<uint64_t*>(fac + tabv + (tabv & 1));
  uint64_t* full = bfull + 1;
  uint64_t* empty = full + stages;
  uint64_t* tfull = empty + stages;  // [2] accumulator ready
  uint64_t* tempty = tfull + 2;      // [2] accumulator drained
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(tempty + 2);

  const int n0 = blockIdx.x * kTM;
  const int g = blockIdx.y, G = gridDim.y;
  const int nmine = g < ntiles ? (ntiles - g + G - 1) / G : 0;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    ptx::mbar_init(bfull, 1);
    for (int s = 0; s < stages; ++s) {
      ptx::mbar_init(&full[s], 1);
      ptx::mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      ptx::mbar_init(&tfull[b], 1);
      ptx::mbar_init(&tempty[b], kKEpiWarps);
    }
    ptx::mbar_init_fence();
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(ptx::smem_u32(tmem_slot)),
                 "r"(2 * kTM));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = *tmem_slot;
  bool ok = true;

  if (warp == 0 && lane == 0) {
    // producer: the Z tile once, then the row tiles
    ptx::mbar_expect_tx(bfull, opb);
    for (int kb = 0; kb < nkb; ++kb) {
      ptx::tma_load_2d(btile + (2 * kb) * kTileBytes, &zhi, kb * kTK, n0, bfull);
      ptx::tma_load_2d(btile + (2 * kb + 1) * kTileBytes, &zlo, kb * kTK, n0, bfull);
    }
    int issued = 0;
    for (int i = 0; i < nmine; ++i) {
      const int s = i % stages;
      if (i >= stages && !ptx::mbar_wait(&empty[s], ((i / stages) - 1) & 1)) {
        ok = false;
        break;
      }
      const int t = g + i * G;
      unsigned char* st = atile + (size_t)s * opb;
      ptx::mbar_expect_tx(&full[s], opb);
      for (int kb = 0; kb < nkb; ++kb) {
        ptx::tma_load_2d(st + (2 * kb) * kTileBytes, &vhi, kb * kTK, t * kTM, &full[s]);
        ptx::tma_load_2d(st + (2 * kb + 1) * kTileBytes, &vlo, kb * kTK, t * kTM, &full[s]);
      }
      issued = i + 1;
    }
    // copies still in flight are waited for (bounded) before leaving
    for (int i = max(0, issued - stages); i < issued; ++i) ptx::mbar_wait(&full[i % stages], (i / stages) & 1);
    ptx::mbar_wait(bfull, 0);
  } else if (warp == 1 && lane == 0) {
    // MMA issuer: row tile i into TMEM buffer i & 1
    if (nmine > 0 && !ptx::mbar_wait(bfull, 0)) ok = false;
    const uint32_t sb = ptx::smem_u32(btile);
    for (int i = 0; i < nmine && ok; ++i) {
      const int b = i & 1, s = i % stages;
      if (i >= 2 && !ptx::mbar_wait(&tempty[b], ((i >> 1) - 1) & 1)) {
        ok = false;
        break;
      }
      if (!ptx::mbar_wait(&full[s], (i / stages) & 1)) {
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint32_t acc = tmem + (uint32_t)(b * kTM);
      const uint32_t sa = ptx::smem_u32(atile + (size_t)s * opb);
      for (int kb = 0; kb < nkb; ++kb) {
#pragma unroll
        for (int kk = 0; kk < kTK / 16; ++kk) {
          const uint32_t off = kk * 32;  // 16 bf16 along K inside the 128-byte swizzle row
          const uint64_t ahi = tc::sw128_desc(sa + (2 * kb) * kTileBytes + off);
          const uint64_t alo = tc::sw128_desc(sa + (2 * kb + 1) * kTileBytes + off);
          const uint64_t bhi = tc::sw128_desc(sb + (2 * kb) * kTileBytes + off);
          const uint64_t blo = tc::sw128_desc(sb + (2 * kb + 1) * kTileBytes + off);
          tc::mma_bf16(acc, ahi, bhi, (kb > 0 || kk > 0) ? 1u : 0u);
          tc::mma_bf16(acc, ahi, blo, 1u);
          tc::mma_bf16(acc, alo, bhi, 1u);
        }
      }
      tc::mma_commit(&empty[s]);  // frees the stage once these MMAs have read it
      tc::mma_commit(&tfull[b]);
    }
  } else if (warp >= 2) {
    // epilogue: lane quarter q (32 rows of one atom and one alpha), 32 reference points
    const int q = warp & 3, cq = (warp - 2) >> 2;
    const int etid = threadIdx.x - 64;  // 0 .. 511 over the epilogue warps
    const float il2 = 1.f / l2;
    const int ipw = (int)pw;
    const bool int_pow = (float)ipw == pw && ipw >= 1 && ipw <= 8;
    if (etid < kTM) iszz[etid] = (n0 + etid < nk) ? 1.f / szz[n0 + etid] : 0.f;
    bool got = true;
    for (int i = 0; i < nmine; ++i) {
      const int b = i & 1;
      const int t = g + i * G;
      const TileMeta tm = tmeta[t];
      const bool use_tab = tm.nv <= tabv;
      // coefficient table of the tile's atom (the previous tile's reads are done at the barrier)
      asm volatile("bar.sync 1, %0;" ::"n"(kKEpiWarps * 32));
      if (use_tab) {
        // per vector: the centre's factors 1 / sqrt f(x,x) and dker_xx / (2 f(x,x) sqrt f(x,x)), zero
        // for a centre without neighbours (krr_c12 with the divisions taken out of the entries)
        const long long r0 = (long long)(t - tm.ti) * kTM;  // the atom's alpha = 0 rows: vector v = row
        if (etid < tm.nv) {
          const float4 a4 = *reinterpret_cast<const float4*>(at + 4 * (size_t)rce[r0 + etid]);
          const float f1 = a4.w == 0.f ? 0.f : 1.f / a4.y;
          fac[etid] = make_float2(f1, a4.z / (2.f * a4.x) * f1);
        }
        asm volatile("bar.sync 3, %0;" ::"n"(kKEpiWarps * 32));
        // four entries per thread and pass, their loads issued together (the kernel features of
        // the neighbour centres are scattered rows of F)
        const int nvk = tm.nv * kTM;
        constexpr int kU = 4, kStep = kKEpiWarps * 32;
        for (int e0 = etid; e0 < nvk; e0 += kU * kStep) {
          float xf[kU];
#pragma unroll
          for (int u = 0; u < kU; ++u) {
            const int e = e0 + u * kStep, k = n0 + (e & (kTM - 1));
            xf[u] = (e < nvk && k < nk) ? F[(size_t)rce[r0 + (e >> 7)] * nk + k] : 0.f;
          }
#pragma unroll
          for (int u = 0; u < kU; ++u) {
            const int e = e0 + u * kStep;
            if (e >= nvk) break;
            const int kl = e & (kTM - 1), v = e >> 7;
            const float base = s2 + xf[u] * il2;
            float bp1 = 1.f;  // base^(p - 1)
            if (int_pow) {
              for (int j = 1; j < ipw; ++j) bp1 *= base;
            } else {
              bp1 = powf(base, pw - 1.f);
            }
            const float2 f = fac[v];
            const float sc = iszz[kl];  // zero past nk
            tab[(size_t)kl * (tabv + 1) + v] = make_float2(pw * bp1 * il2 * sc * f.x, bp1 * base * sc * f.y);
          }
        }
      }
      // the accumulator; the barrier also publishes the table, and a timed-out wait in any
      // epilogue warp ends the loop for all of them together
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
      float v[32];
#pragma unroll
      for (int h = 0; h < 4; ++h)
        tc::tmem_ld8(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * kTM + cq * 32 + h * 8), v + h * 8);
      asm volatile("tcgen05.fence::before_thread_sync;");
      __syncwarp();
      if (lane == 0) ptx::mbar_arrive(&tempty[b]);
      const int lr0 = tm.ti * kTM + q * 32;
      const int al = lr0 / tm.nvp;  // the same for the whole quarter
      if (al >= 3) continue;        // padding quarter
      const long long row = (long long)t * kTM + q * 32 + lane;
      const int vi = lr0 + lane - al * tm.nvp;  // derivative vector of this row
      const float sg = rsg[row], gv = rg[row];
      const int ce = rce[row];
#pragma unroll
      for (int c = 0; c < 32; ++c) {
        const int kl = cq * 32 + c, k = n0 + kl;
        float val = 0.f;
        if (sg != 0.f && k < nk) {
          float c1, c2;
          if (use_tab) {
            const float2 cc = tab[(size_t)kl * (tabv + 1) + vi];
            c1 = cc.x;
            c2 = cc.y;
          } else {
            krr_c12<float>(F[(size_t)ce * nk + k], at + 4 * (size_t)ce, szz[k], s2, l2, pw, c1, c2);
          }
          val = sg * (c1 * v[c] - c2 * gv);
        }
        v[c] = val;
      }
      // sum over the quarter's 32 rows: transposing butterfly, lane c ends with column c
#pragma unroll
      for (int sh = 16; sh >= 1; sh >>= 1) {
#pragma unroll
        for (int j = 0; j < sh; ++j) {
          const bool up = (lane & sh) != 0;
          const float send = up ? v[j] : v[j + sh];
          const float keep = up ? v[j + sh] : v[j];
          v[j] = keep + __shfl_xor_sync(0xffffffffu, send, sh);
        }
      }
      const int k = n0 + cq * 32 + lane;
      const int a = tm.atom, sidx = atom_struct[a];
      const long long rf = rowF[sidx];
      if (k < nk && rf >= 0 && v[0] != 0.f)
        atomicAdd(&X[(rf + 3LL * (a - atom_start[sidx]) + al) * ldx + c0 + k], v[0]);
    }
    if (!got && lane == 0) atomicExch(err, 1);
  }
  if (!ok) atomicExch(err, 1);
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * kTM));
  }
}

bool krr_force_tc_available() { return tc::encode_fn() != nullptr; }

// Force rows of the kernel block (columns [c0, c0 + nk) of X) for every atom with force rows,
// replacing k_krr_force_tiled for the FP32 rows.  ws (ws_bytes) holds the Z planes and, per
// chunk of atoms, the derivative-vector planes and their row and tile records; chunks are as
// large as ws allows.  F, at, szz: the kernel features, atom terms and point norms of
// launch_krr_rows.  X must hold zeros in these columns (the sums are added atomically).
cudaError_t launch_krr_force_tc(const DevBatch& b, const DevRows& rows, const int* rev, const float* Bq,
                                const float* dBq, const float* Z, const float* F, const float* at, const float* szz,
                                int nk, int KK, double power, double length, double sigma, void* ws, size_t ws_bytes,
                                float* X, int c0, int* err, int nsm, cudaStream_t st, int* launches) {
  *launches = 0;
  if (b.A == 0 || nk == 0) return cudaSuccess;
  const int nkb = (KK + kTK - 1) / kTK;
  const int KP = nkb * kTK;
  if (nkb > 3) return cudaErrorInvalidValue;  // K blocks beyond the shared-memory budget
  // one row-tile stage: the epilogue (coefficients, reduction) bounds the tile rate, and the rest
  // of shared memory holds the coefficient table of up to tabv derivative vectors
  const int stages = 1;
  const size_t opb = (size_t)nkb * 2 * kTileBytes;
  const size_t kSmemMax = 227 * 1024;
  const size_t fixed = 1024 + (1 + (size_t)stages) * opb + 8 * (3 + 2 * (size_t)stages + 4) + 16 + 4 * kTM + 8 * 66;
  if (fixed + (size_t)kTM * 8 * 2 > kSmemMax) return cudaErrorInvalidValue;
  const int tabv = (int)std::min<size_t>(64, (kSmemMax - fixed) / ((size_t)kTM * 8) - 1);
  const size_t smem = fixed + (size_t)kTM * 8 * (tabv + 1);
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_krr_force_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  if (smem > kSmemMax) return cudaErrorInvalidValue;
  // per-atom tiles from the neighbour counts
  std::vector<int> off(b.A + 1);
  cudaError_t e = cudaMemcpyAsync(off.data(), b.nbr_off, sizeof(int) * (b.A + 1), cudaMemcpyDeviceToHost, st);
  if (e != cudaSuccess) return e;
  e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return e;
  std::vector<int> ntile(b.A), nvp(b.A);
  for (int a = 0; a < b.A; ++a) {
    const int nv = off[a + 1] - off[a] + 1;
    nvp[a] = (nv + 31) / 32 * 32;
    ntile[a] = (3 * nvp[a] + kTM - 1) / kTM;
  }
  // workspace: Z planes, then the chunk's planes (4 KP bytes per row), row records (12 bytes per
  // row), tile records and the atoms' first tiles
  auto al256 = [](size_t x) { return (x + 255) / 256 * 256; };
  unsigned char* w = static_cast<unsigned char*>(ws);
  const size_t zb = al256((size_t)nk * KP * 2);
  __nv_bfloat16* zhi = reinterpret_cast<__nv_bfloat16*>(w);
  __nv_bfloat16* zlo = reinterpret_cast<__nv_bfloat16*>(w + zb);
  const size_t per_tile = (size_t)kTM * (4 * (size_t)KP + 12) + sizeof(TileMeta) + 4;
  if (ws_bytes < 2 * zb + 8 * 256 + per_tile * 16 + 8) return cudaErrorInvalidValue;
  const size_t room = ws_bytes - 2 * zb - 8 * 256;
  const long long max_tiles = (long long)(room / per_tile) - 1;
  {
    const long long n = (long long)nk * KP;
    k_ktc_zplanes<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(Z, nk, KK, KP, zhi, zlo);
    ++*launches;
  }
  CUtensorMap mzh, mzl;
  if (!tc::make_plane_map(&mzh, zhi, KP, nk, KP) || !tc::make_plane_map(&mzl, zlo, KP, nk, KP))
    return cudaErrorInvalidValue;
  const float s2 = (float)(sigma * sigma), l2 = (float)(2.0 * length * length), pw = (float)power;
  const int NT = (nk + kTM - 1) / kTM;
  std::vector<int> tile0;
  std::vector<TileMeta> meta;
  for (int a0 = 0; a0 < b.A;) {
    // the largest run of atoms whose tiles fit the workspace
    long long nt = 0;
    int a1 = a0;
    while (a1 < b.A && nt + ntile[a1] <= max_tiles) nt += ntile[a1++];
    if (a1 == a0) return cudaErrorInvalidValue;  // one atom alone exceeds the workspace
    tile0.assign(a1 - a0 + 1, 0);
    meta.clear();
    for (int a = a0; a < a1; ++a) {
      tile0[a - a0 + 1] = tile0[a - a0] + ntile[a];
      for (int ti = 0; ti < ntile[a]; ++ti) meta.push_back(TileMeta{a, ti, nvp[a], off[a + 1] - off[a] + 1});
    }
    const size_t rows_c = (size_t)nt * kTM;
    unsigned char* p = w + 2 * zb;
    __nv_bfloat16* vhi = reinterpret_cast<__nv_bfloat16*>(p);
    p += al256(rows_c * KP * 2);
    __nv_bfloat16* vlo = reinterpret_cast<__nv_bfloat16*>(p);
    p += al256(rows_c * KP * 2);
    int* rce = reinterpret_cast<int*>(p);
    p += al256(rows_c * 4);
    float* rsg = reinterpret_cast<float*>(p);
    p += al256(rows_c * 4);
    float* rg = reinterpret_cast<float*>(p);
    p += al256(rows_c * 4);
    TileMeta* dmeta = reinterpret_cast<TileMeta*>(p);
    p += al256(sizeof(TileMeta) * meta.size());
    int* dtile0 = reinterpret_cast<int*>(p);
    e = cudaMemcpyAsync(dmeta, meta.data(), sizeof(TileMeta) * meta.size(), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(dtile0, tile0.data(), sizeof(int) * tile0.size(), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return e;
    k_ktc_vplanes<<<(unsigned)(a1 - a0), 128, 0, st>>>(a0, a1, KK, KP, b.nbr_off, b.nbr_idx, rev, Bq, dBq, dtile0,
                                                      vhi, vlo, rce, rsg, rg);
    CUtensorMap mvh, mvl;
    if (!tc::make_plane_map(&mvh, vhi, KP, (long long)rows_c, KP) ||
        !tc::make_plane_map(&mvl, vlo, KP, (long long)rows_c, KP))
      return cudaErrorInvalidValue;
    const int G = std::max(1, std::min<int>((int)nt, (2 * nsm + NT - 1) / NT));
    k_krr_force_tc<<<dim3((unsigned)NT, (unsigned)G), kKThreads, smem, st>>>(
        mvh, mvl, mzh, mzl, (int)nt, nkb, stages, nk, dmeta, rce, rsg, rg, F, at, szz, s2, l2, pw, b.atom_struct,
        b.atom_start, rows.rowF, c0, rows.ldx, X, tabv, err);
    *launches += 2;
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    // the host records of the next chunk overwrite dmeta / dtile0 only after this chunk's kernels
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return e;
    a0 = a1;
  }
  return cudaSuccess;
}

}  // namespace mld
