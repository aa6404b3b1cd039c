// tcgen05 / TMA helpers shared by the tensor-core kernels of the mixed method (gram_tc.cu,
// krr_tc.cu): 128 x 128 BF16 MMAs with FP32 accumulation in TMEM, operands as K-major tiles of
// 128 rows x 64 elements written by TMA with 128-byte swizzle.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "ptx.cuh"

namespace mld {
namespace tc {

constexpr int kTM = 128;                   // tile rows (M) = tile columns (N)
constexpr int kTK = 64;                    // K elements per operand tile: 128 bytes of bf16
constexpr int kTileBytes = kTM * kTK * 2;  // 16 KB

// Shared-memory matrix descriptor of a K-major tile written by TMA with 128-byte swizzle:
// rows of 128 bytes, 8-row core groups 1024 bytes apart (stride byte offset), version 1.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);  // start address, bits 0-13
  d |= (uint64_t)1 << 16;                    // leading byte offset (not used by swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;          // stride byte offset, bits 32-45
  d |= (uint64_t)1 << 46;                    // descriptor version
  d |= (uint64_t)2 << 61;                    // 128-byte swizzle
  return d;
}

// kind::f16 instruction descriptor: D FP32 (bits 4-5 = 1), A and B BF16 (bits 7-9, 10-12 = 1),
// both K-major, N >> 3 at bits 17-22, M >> 4 at bits 24-28; M = N = 128.
__host__ __device__ constexpr uint32_t idesc_m128(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(kTM >> 4) << 24);
}
constexpr uint32_t kIdesc = idesc_m128(kTM);

// D (TMEM) += A B^T with the given instruction descriptor (M = 128, N a multiple of 16, <= 256)
__device__ __forceinline__ void mma_bf16_id(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc,
                                            uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}
__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t accumulate) {
  mma_bf16_id(tmem_d, a, b, kIdesc, accumulate);
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   ptx::smem_u32(bar))
               : "memory");
}
// 32 lanes x 8 consecutive FP32 columns of TMEM into registers (and wait for them)
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float* out) {
  uint32_t v[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7])
               : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int c = 0; c < 8; ++c) out[c] = __uint_as_float(v[c]);
}

using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
inline EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  }
  return fn;
}
// bf16 plane of `outer` rows x `inner` K elements (row stride row_elems * 2 bytes, a multiple of
// 16 bytes); box 64 (K) x box_rows, 128-byte swizzle; rows past `outer` read as zero
inline bool make_plane_map(CUtensorMap* m, void* base, long long inner, long long outer, long long row_elems,
                           int box_rows = kTM) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) return false;
  cuuint64_t dims[2] = {(cuuint64_t)inner, (cuuint64_t)outer};
  cuuint64_t strides[1] = {(cuuint64_t)row_elems * 2};
  cuuint32_t box[2] = {(cuuint32_t)kTK, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace tc
}  // namespace mld
