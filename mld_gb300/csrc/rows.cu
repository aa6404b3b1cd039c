// Linear design rows and evaluation sums gathered from per-atom and per-pair descriptor outputs,
// with a fixed summation order (no floating-point atomics), and the longest-first atom order of
// the descriptor kernel's work queue.
//
// The descriptor kernel exports B_i per atom and v_q = w_ch dB_i/du_q per pair q = (i -> n).
// The reference's linear rows (mld_energy.F90:91-117, mld_forces.F90:222-263,
// mld_stress.F90:272-756) are then
//   energy row  sum_{i in s} B_i
//   force rows  atom i, component a:  sum_{q in nbrs(i)} v_q[a] - v_{rev(q)}[a]
//               (the centre's own derivative minus every derivative of a neighbour's descriptor
//               with respect to i; rev(q) is the pair (n -> i) with the opposite displacement)
//   stress rows sign_stress * 3/V * sum_{i in s} sum_q v_q[aa] * lever_q[bb] / r_q for the
//               (aa, bb) of xx, yy, zz, yz, xz, xy; lever = u (small box) or sign_big * (-u)
//               (large box), as mld_stress.F90:443-490 and :540-669 differ.
// The force rows of an atom and its stress partials come from one CTA per atom; the energy and
// stress rows of a structure sum its atoms in order.
#include <cuda_runtime.h>

#include <algorithm>

#include "mld_internal.h"

namespace mld {

namespace {

constexpr int kRowThreads = 256;

template <typename T>
__global__ void __launch_bounds__(kRowThreads) k_lin_force_rows(
    int A, int KK, const int* __restrict__ atom_struct, const int* __restrict__ atom_start,
    const int* __restrict__ nbr_off, const double* __restrict__ nbr_u, const int* __restrict__ rev,
    const int* __restrict__ small, double sign_big, const T* __restrict__ dB, const long long* __restrict__ rowF,
    const long long* __restrict__ rowS, T* __restrict__ X, int ldx, T* __restrict__ Sp) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int i = blockIdx.x;
  if (i >= A) return;
  const int s = atom_struct[i];
  const int p0 = nbr_off[i], nn = nbr_off[i + 1] - p0;
  const long long rf = rowF ? rowF[s] : -1, rs = rowS ? rowS[s] : -1;
  int* qrev = reinterpret_cast<int*>(smem_raw);                              // nn
  T* fac = reinterpret_cast<T*>(smem_raw + sizeof(int) * ((nn + 3) & ~3));  // nn * 3
  const int tid = threadIdx.x;
  const double sg = small[s] ? 1.0 : -sign_big;
  for (int n = tid; n < nn; n += blockDim.x) {
    qrev[n] = rev[p0 + n];
    const double* u = nbr_u + 3 * (size_t)(p0 + n);
    const double f = sg / sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
    fac[3 * n + 0] = (T)(f * u[0]);
    fac[3 * n + 1] = (T)(f * u[1]);
    fac[3 * n + 2] = (T)(f * u[2]);
  }
  __syncthreads();
  // thread (a, k): the force row entry and the stress partials (aa = a, bb >= a) of column k,
  // each summed over the neighbours in order from one read of the atom's own derivatives
  const bool want_f = rf >= 0, want_s = rs >= 0 && Sp;
  if (!want_f && !want_s) return;
  for (int c = tid; c < 3 * KK; c += blockDim.x) {
    const int a = c / KK, k = c - a * KK;
    T sum = T(0), acc[3] = {T(0), T(0), T(0)};
#pragma unroll 4
    for (int n = 0; n < nn; ++n) {
      const T own = dB[((size_t)(p0 + n) * 3 + a) * KK + k];
      const int q = qrev[n];
      const T back = q >= 0 ? dB[((size_t)q * 3 + a) * KK + k] : T(0);
      sum += own - back;
#pragma unroll
      for (int bb = 0; bb < 3; ++bb)
        if (bb >= a) acc[bb] = fma(own, fac[3 * n + bb], acc[bb]);
    }
    if (want_f) X[(rf + 3LL * (i - atom_start[s]) + a) * ldx + 1 + k] = sum;
    if (want_s) {
      // (aa, bb) -> stress index: (0,0) xx 0, (1,1) yy 1, (2,2) zz 2, (1,2) yz 3, (0,2) xz 4, (0,1) xy 5
#pragma unroll
      for (int bb = 0; bb < 3; ++bb) {
        if (bb < a) continue;
        const int sidx = bb == a ? a : (a == 1 ? 3 : (bb == 2 ? 4 : 5));
        Sp[((size_t)i * 6 + sidx) * KK + k] = acc[bb];
      }
    }
  }
}

// grid (S, 7): r = 0 energy row sum_i B_i; r = 1..6 stress rows sign_stress*3/V sum_i Sp_i.
template <typename T>
__global__ void __launch_bounds__(kRowThreads) k_lin_struct_rows(int KK, const int* __restrict__ atom_start,
                                                                 const T* __restrict__ B, const T* __restrict__ Sp,
                                                                 const double* __restrict__ volume, double sign_stress,
                                                                 const long long* __restrict__ rowE,
                                                                 const long long* __restrict__ rowS,
                                                                 T* __restrict__ X, int ldx) {
  const int s = blockIdx.x, r = blockIdx.y;
  const long long row = (r == 0) ? rowE[s] : (rowS[s] >= 0 ? rowS[s] + (r - 1) : -1);
  if (row < 0) return;
  const int a0 = atom_start[s], a1 = atom_start[s + 1];
  const T sc = (r == 0) ? T(1) : (T)(sign_stress * 3.0 / volume[s]);
  for (int k = threadIdx.x; k < KK; k += kRowThreads) {
    T sum = T(0);
    if (r == 0)
      for (int a = a0; a < a1; ++a) sum += B[(size_t)a * KK + k];
    else
      for (int a = a0; a < a1; ++a) sum += Sp[((size_t)a * 6 + (r - 1)) * KK + k];
    X[row * ldx + 1 + k] = sc * sum;
  }
}

// Evaluation: F_i[a] = sum_q pair_q[a] - pair_rev(q)[a], one thread per (atom, component).
__global__ void k_eval_forces(int A, const int* __restrict__ nbr_off, const int* __restrict__ rev,
                              const double* __restrict__ pair, double* __restrict__ F) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 3LL * A) return;
  const int i = (int)(t / 3), a = (int)(t - 3LL * i);
  double sum = 0.0;
  for (int q = nbr_off[i]; q < nbr_off[i + 1]; ++q) {
    const int b = rev[q];
    sum += pair[(size_t)q * 9 + a] - (b >= 0 ? pair[(size_t)b * 9 + a] : 0.0);
  }
  F[t] = sum;
}

// Evaluation, one CTA per structure: E_s = sum_i Eatom_i (when given), S_s = sign_stress*3/V *
// sum_i sum_q pair_q[3 + c]; per-thread sums over a fixed atom stride, then a fixed tree.
__global__ void __launch_bounds__(kRowThreads) k_eval_struct(const int* __restrict__ atom_start,
                                                             const int* __restrict__ nbr_off,
                                                             const double* __restrict__ pair,
                                                             const double* __restrict__ Eatom,
                                                             const double* __restrict__ volume, double sign_stress,
                                                             double* __restrict__ E, double* __restrict__ S) {
  __shared__ double red[7][kRowThreads];
  const int s = blockIdx.x, tid = threadIdx.x;
  double v[7] = {0, 0, 0, 0, 0, 0, 0};
  for (int i = atom_start[s] + tid; i < atom_start[s + 1]; i += kRowThreads) {
    if (Eatom) v[0] += Eatom[i];
    for (int q = nbr_off[i]; q < nbr_off[i + 1]; ++q)
#pragma unroll
      for (int c = 0; c < 6; ++c) v[1 + c] += pair[(size_t)q * 9 + 3 + c];
  }
#pragma unroll
  for (int c = 0; c < 7; ++c) red[c][tid] = v[c];
  __syncthreads();
  for (int o = kRowThreads / 2; o > 0; o >>= 1) {
    if (tid < o)
#pragma unroll
      for (int c = 0; c < 7; ++c) red[c][tid] += red[c][tid + o];
    __syncthreads();
  }
  if (tid == 0) {
    if (Eatom) E[s] = red[0][0];
    const double sc = sign_stress * 3.0 / volume[s];
    for (int c = 0; c < 6; ++c) S[6 * (size_t)s + c] = sc * red[1 + c][0];
  }
}

// ---- longest-first atom order (counting sort on the neighbour count, descending) ----
constexpr int kOrdThreads = 1024;

__global__ void k_ord_hist(int A, const int* __restrict__ nn, int maxnn, int* __restrict__ hist) {
  extern __shared__ int h[];
  for (int b = threadIdx.x; b <= maxnn; b += blockDim.x) h[b] = 0;
  __syncthreads();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < A; i += gridDim.x * blockDim.x)
    atomicAdd(&h[maxnn - min(nn[i], maxnn)], 1);
  __syncthreads();
  for (int b = threadIdx.x; b <= maxnn; b += blockDim.x)
    if (h[b]) atomicAdd(&hist[b], h[b]);
}

__global__ void k_ord_scan(int nbins, int* __restrict__ hist) {
  // single thread: a few hundred bins
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    int run = 0;
    for (int b = 0; b < nbins; ++b) {
      const int c = hist[b];
      hist[b] = run;
      run += c;
    }
  }
}

__global__ void k_ord_scatter(int A, const int* __restrict__ nn, int maxnn, int* __restrict__ cursor,
                              int* __restrict__ order) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool ok = i < A;
  const int bin = ok ? maxnn - min(nn[i], maxnn) : -1;
  // lanes of a warp with the same bin take consecutive slots with one atomic
  const unsigned same = __match_any_sync(0xffffffffu, bin);
  const int leader = __ffs(same) - 1;
  const int rank = __popc(same & ((1u << (threadIdx.x & 31)) - 1u));
  int base = 0;
  if (ok && (threadIdx.x & 31) == leader) base = atomicAdd(&cursor[bin], __popc(same));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (ok) order[base + rank] = i;
}

}  // namespace

size_t atom_order_tmp_ints(int maxnn) { return (size_t)maxnn + 2; }

cudaError_t launch_atom_order(const int* nn, int A, int maxnn, int* order, int* tmp, cudaStream_t st) {
  if (A <= 0) return cudaSuccess;
  maxnn = std::max(maxnn, 0);
  cudaError_t e = cudaMemsetAsync(tmp, 0, sizeof(int) * (maxnn + 1), st);
  if (e != cudaSuccess) return e;
  const int blocks = std::min(256, (A + kOrdThreads - 1) / kOrdThreads);
  k_ord_hist<<<blocks, kOrdThreads, sizeof(int) * (maxnn + 1), st>>>(A, nn, maxnn, tmp);
  k_ord_scan<<<1, 32, 0, st>>>(maxnn + 1, tmp);
  k_ord_scatter<<<(A + 255) / 256, 256, 0, st>>>(A, nn, maxnn, tmp, order);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_lin_rows(const DevBatch& b, const DevRows& rows, const BsoParams& p, int KK, const int* rev,
                            const T* B, const T* dB, T* Sp, T* X, cudaStream_t st) {
  if (b.A == 0) return cudaSuccess;
  const size_t sm = sizeof(int) * (size_t)((std::max(b.maxnn, 1) + 3) & ~3) + sizeof(T) * 3 * (size_t)std::max(b.maxnn, 1);
  cudaError_t e = cudaSuccess;
  if (sm > 48 * 1024) {
    e = cudaFuncSetAttribute(k_lin_force_rows<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
  }
  // one thread per (component, column) of the atom's force rows, in whole warps (192 for K = 55)
  const int nthr = std::min(kRowThreads, (3 * KK + 31) / 32 * 32);
  k_lin_force_rows<T><<<b.A, nthr, sm, st>>>(b.A, KK, b.atom_struct, b.atom_start, b.nbr_off, b.nbr_u, rev, b.small,
                                             p.sign_big, dB, rows.rowF, rows.rowS, X, rows.ldx, Sp);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_lin_struct_rows<T><<<dim3(b.S, 7), kRowThreads, 0, st>>>(KK, b.atom_start, B, Sp, b.volume, p.sign_stress,
                                                             rows.rowE, rows.rowS, X, rows.ldx);
  return cudaGetLastError();
}

cudaError_t launch_eval_gather(const DevBatch& b, const BsoParams& p, const int* rev, const double* pair,
                               const double* Eatom, double* E, double* F, double* S, cudaStream_t st) {
  if (b.A == 0) return cudaSuccess;
  const long long n = 3LL * b.A;
  k_eval_forces<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(b.A, b.nbr_off, rev, pair, F);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_eval_struct<<<b.S, kRowThreads, 0, st>>>(b.atom_start, b.nbr_off, pair, Eatom, b.volume, p.sign_stress, E, S);
  return cudaGetLastError();
}

template cudaError_t launch_lin_rows<double>(const DevBatch&, const DevRows&, const BsoParams&, int, const int*,
                                             const double*, const double*, double*, double*, cudaStream_t);
template cudaError_t launch_lin_rows<float>(const DevBatch&, const DevRows&, const BsoParams&, int, const int*,
                                            const float*, const float*, float*, float*, cudaStream_t);

}  // namespace mld
