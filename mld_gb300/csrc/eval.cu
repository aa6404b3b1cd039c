// Per-atom effective weights of the quadratic model for evaluation without design rows.
//
// The quadratic energy of atom a is w0 + w_lin . B_a + B_a^T W B_a with W the K x K block of the
// weights in the reference's full layout (index K*(id1-1)+id2, mld_energy.F90:170-266).  Its
// gradient with respect to B_a is beta_a = w_lin + (W + W^T) B_a, and the quadratic force and
// stress rows dotted with the weights reduce to the linear contraction of dB with beta
// (mld_forces.F90:410-500: the centre's beta; mld_stress.F90:580-603: the neighbour's beta).
#include <cuda_runtime.h>

#include "mld_internal.h"

namespace mld {

// One CTA per atom: beta[k] = w_lin[k] + sum_j Wsym[j][k] B[j] (Wsym symmetric, read by rows j
// so that consecutive threads read consecutive k) and the atom's energy w0 + B . (beta + w_lin) / 2.
template <typename T>
__global__ void __launch_bounds__(128) k_eval_beta(const T* __restrict__ B, int nchK, const double* __restrict__ wlin,
                                                  const double* __restrict__ wsym, double w0, T* __restrict__ beta,
                                                  double* __restrict__ Eatom) {
  extern __shared__ double bsh[];  // nchK
  __shared__ double red[4];
  const int a = blockIdx.x, tid = threadIdx.x;
  for (int j = tid; j < nchK; j += blockDim.x) bsh[j] = (double)B[(size_t)a * nchK + j];
  __syncthreads();
  double e = 0.0;
  for (int k = tid; k < nchK; k += blockDim.x) {
    double v = wlin[k];
    for (int j = 0; j < nchK; ++j) v = fma(wsym[(size_t)j * nchK + k], bsh[j], v);
    beta[(size_t)a * nchK + k] = (T)v;
    e = fma(0.5 * bsh[k], v + wlin[k], e);
  }
  for (int o = 16; o > 0; o >>= 1) e += __shfl_xor_sync(0xffffffffu, e, o);
  if ((tid & 31) == 0) red[tid >> 5] = e;
  __syncthreads();
  if (tid == 0) Eatom[a] = w0 + red[0] + red[1] + red[2] + red[3];
}

template <typename T>
cudaError_t launch_eval_beta(const T* B, int A, int nchK, const double* wlin, const double* wsym, double w0, T* beta,
                             double* Eatom, cudaStream_t st) {
  if (A <= 0) return cudaSuccess;
  k_eval_beta<T><<<A, 128, sizeof(double) * nchK, st>>>(B, nchK, wlin, wsym, w0, beta, Eatom);
  return cudaGetLastError();
}

template cudaError_t launch_eval_beta<double>(const double*, int, int, const double*, const double*, double, double*,
                                              double*, cudaStream_t);
template cudaError_t launch_eval_beta<float>(const float*, int, int, const double*, const double*, double, float*,
                                             double*, cudaStream_t);

}  // namespace mld
