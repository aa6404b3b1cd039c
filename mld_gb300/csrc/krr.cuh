// Coefficients of the normalised polynomial kernel (kernel_type 4, compute_kernel.F90:91-150)
// shared by the kernel-model row kernels.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

namespace mld {

// kernel coefficients of centre atom (its [f(x,x), sqrt f(x,x), dker_xx, has neighbours]) and
// a reference point, in the kernel's precision: (c1, c2); zero for an atom without neighbours
template <typename T>
__device__ __forceinline__ void krr_c12(T xz, const T* atc, T szz, T s2, T l2, T p, T& c1, T& c2) {
  if (atc[3] == T(0)) {
    c1 = c2 = T(0);
    return;
  }
  const T base = s2 + xz / l2;
  T bp1 = T(1);  // base^(p-1)
  const int ip = (int)p;
  if ((T)ip == p && ip >= 1 && ip <= 8) {
    for (int i = 1; i < ip; ++i) bp1 *= base;
  } else {
    bp1 = (T)pow((double)base, (double)p - 1.0);
  }
  const T kt = bp1 * base;
  const T inv_aaa = T(1) / (szz * atc[1]);
  c1 = p * bp1 / l2 * inv_aaa;
  c2 = kt * atc[2] / (T(2) * atc[0]) * inv_aaa;
}

}  // namespace mld
