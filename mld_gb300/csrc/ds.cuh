// Double-FP32 ("double-single") arithmetic, shared by the kernels of the mixed method.
// GB300 issues FP64 at 1/64 of its FP32 rate, so sums and products that need more than FP32
// are formed from FP32 error-free transformations instead: TwoSum (Knuth) and TwoProd via fmaf
// give sums and products as unevaluated pairs hi + lo, about 2^-44 relative to the sum of the
// magnitudes.  With an FP32 x, x * (p_hi + p_lo) is formed exactly up to the x * p_lo term.
#pragma once
#include <cuda_runtime.h>

namespace mld {

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}
// (sh, sl) += x * (ph + pl)
__device__ __forceinline__ void ds_fma(float& sh, float& sl, float x, float ph, float pl) {
  const float p = x * ph;
  const float pe = fmaf(x, pl, fmaf(x, ph, -p));
  float t, e;
  two_sum(sh, p, t, e);
  sh = t;
  sl += e + pe;
}
// (sh, sl) += (oh, ol)
__device__ __forceinline__ void ds_add(float& sh, float& sl, float oh, float ol) {
  float t, e;
  two_sum(sh, oh, t, e);
  sh = t;
  sl += e + ol;
}
__device__ __forceinline__ void ds_norm(float& sh, float& sl) {
  const float t = sh + sl;
  sl = sl - (t - sh);
  sh = t;
}
__device__ __forceinline__ void ds_split(double v, float& h, float& l) {
  h = (float)v;
  l = (float)(v - (double)h);
}

}  // namespace mld
