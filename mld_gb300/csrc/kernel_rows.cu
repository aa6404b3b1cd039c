// Kernel ridge regression design rows (ml_type = 1, polynomial kernel kernel_type = 4).
//
// Columns [c0, c0 + nk) of the design rows, c0 = 1 + KK (the linear part is written by the
// descriptor kernel): for atom x (raw descriptor) and reference point z_k (standardised over the
// reference set, compute_kernel.F90:1058-1256), inner_kernel_po (compute_kernel.F90:91-150):
//   f = (s2 + x.z/l2)^p,  k = f / sqrt(f(x,x) f(z,z)),  l2 = 2 length^2, s2 = sigma^2,
//   dk(g) = c1 (g.z) - c2 (g.x)  for a descriptor derivative g = force(:, centre, n, a), with
//   c1 = p (s2 + x.z/l2)^(p-1) / l2 / sqrt(f(x,x) f(z,z)),
//   c2 = f * dker_xx / (2 f(x,x)) / sqrt(f(x,x) f(z,z)),  dker_xx = 2 p (s2 + x.x/l2)^(p-1) / l2.
// Packing as the linear rows (mld_energy.F90:122-144, mld_forces.F90:268-320,
// mld_stress.F90:456,577): energy row sums k over atoms with neighbours; force row of atom a gets
// + sum over its own pairs (self term) and - the pairs (j -> a) of which it is the neighbour;
// stress rows sum dk * uu/r over pairs.  By linearity the self term uses the sum of a's pair
// derivatives and the stress rows use per-atom sums T_s = sum_n g_{n, sa(s)} uu_{sb(s)} / r.
#include <cuda_runtime.h>

#include <algorithm>

#include "mld_internal.h"

namespace mld {

namespace {
constexpr int kKT = 256;   // threads per CTA (one reference point each per pass)
constexpr int kVC = 8;     // derivative vectors per register pass
__constant__ int c_sa[6] = {0, 1, 2, 1, 0, 0};
__constant__ int c_sb[6] = {0, 1, 2, 2, 2, 1};
}  // namespace

// per atom: [0] f(x,x), [1] sqrt f(x,x), [2] dker_xx, [3] 1 if the atom has neighbours
template <typename T>
__global__ void k_krr_atom(int A, int KK, const T* __restrict__ B, const int* __restrict__ nbr_off, double s2,
                           double l2, double p, T* __restrict__ at) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= A) return;
  const T* x = B + (size_t)a * KK;
  double xx = 0.0;
  for (int c = 0; c < KK; ++c) xx += (double)x[c] * (double)x[c];
  const double base = s2 + xx / l2;
  const double kxx = pow(base, p);
  at[4 * (size_t)a] = (T)kxx;
  at[4 * (size_t)a + 1] = (T)sqrt(kxx);
  at[4 * (size_t)a + 2] = (T)(2.0 * p * pow(base, p - 1.0) / l2);
  at[4 * (size_t)a + 3] = (T)(nbr_off[a + 1] > nbr_off[a] ? 1 : 0);
}

// per reference point: sqrt f(z,z)
template <typename T>
__global__ void k_krr_points(int nk, int KK, const T* __restrict__ Z, double s2, double l2, double p,
                             T* __restrict__ szz) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nk) return;
  double zz = 0.0;
  for (int c = 0; c < KK; ++c) zz += (double)Z[(size_t)k * KK + c] * (double)Z[(size_t)k * KK + c];
  szz[k] = (T)sqrt(pow(s2 + zz / l2, p));
}

// F[a][k] = x_a . z_k (atoms x reference points), 64 x 64 tiles, 4 x 4 outputs per thread
template <typename T>
__global__ void __launch_bounds__(256) k_krr_xz(int A, int nk, int KK, const T* __restrict__ B,
                                                const T* __restrict__ Z, T* __restrict__ F) {
  __shared__ T sa[16][64 + 1], sb[16][64 + 1];
  const int a0 = blockIdx.y * 64, k0 = blockIdx.x * 64;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  T acc[4][4] = {};
  for (int c0 = 0; c0 < KK; c0 += 16) {
    for (int e = threadIdx.x; e < 16 * 64; e += 256) {
      const int r = e / 16, c = e % 16;
      sa[c][r] = (a0 + r < A && c0 + c < KK) ? B[(size_t)(a0 + r) * KK + c0 + c] : T(0);
      sb[c][r] = (k0 + r < nk && c0 + c < KK) ? Z[(size_t)(k0 + r) * KK + c0 + c] : T(0);
    }
    __syncthreads();
#pragma unroll
    for (int c = 0; c < 16; ++c) {
      T av[4], bv[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        av[i] = sa[c][ty + 16 * i];
        bv[i] = sb[c][tx + 16 * i];
      }
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(av[i], bv[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int a = a0 + ty + 16 * i, k = k0 + tx + 16 * j;
      if (a < A && k < nk) F[(size_t)a * nk + k] = acc[i][j];
    }
}

// kernel value and the two derivative coefficients of centre atom a and reference point k
template <typename T>
__device__ __forceinline__ void krr_coef(T xz, const T* at, T szz, double s2, double l2, double p, T& kv, T& c1,
                                         T& c2) {
  const double base = s2 + (double)xz / l2;
  const double kt = pow(base, p);
  const double aaa = (double)szz * (double)at[1];
  kv = (T)(kt / aaa);
  c1 = (T)(p * pow(base, p - 1.0) / l2 / aaa);
  c2 = (T)(kt * (double)at[2] / (2.0 * (double)at[0]) / aaa);
}

// energy rows: grid (S, ceil(nk / kKT))
template <typename T>
__global__ void __launch_bounds__(kKT) k_krr_energy(int nk, const int* __restrict__ atom_start,
                                                    const long long* __restrict__ rowE, const T* __restrict__ F,
                                                    const T* __restrict__ at, const T* __restrict__ szz, double s2,
                                                    double l2, double p, int c0, int ldx, T* __restrict__ X) {
  const int s = blockIdx.x;
  const int k = blockIdx.y * kKT + threadIdx.x;
  if (rowE[s] < 0 || k >= nk) return;
  double acc = 0.0;
  for (int a = atom_start[s]; a < atom_start[s + 1]; ++a) {
    if (at[4 * (size_t)a + 3] == T(0)) continue;  // atoms without neighbours contribute zero
    T kv, c1, c2;
    krr_coef<T>(F[(size_t)a * nk + k], at + 4 * (size_t)a, szz[k], s2, l2, p, kv, c1, c2);
    acc += (double)kv;
  }
  X[rowE[s] * ldx + c0 + k] = (T)acc;
}

// Derivative vectors of target atom a (staged by k_krr_force): vector 0 is the sum of a's own
// pair derivatives (self term, centre a, sign +1); vectors 1..n are the derivatives of the
// reversed pairs (j -> a) (centre j, sign -1).  Per vector and direction also g . x_centre.
// One CTA per atom; threads over reference points.
template <typename T>
__global__ void __launch_bounds__(kKT) k_krr_force(
    int KK, int nk, const int* __restrict__ atom_struct, const int* __restrict__ atom_start,
    const long long* __restrict__ rowF, const int* __restrict__ nbr_off, const int* __restrict__ nbr_idx,
    const int* __restrict__ rev, const T* __restrict__ B, const T* __restrict__ dB, const T* __restrict__ Zt,
    const T* __restrict__ F, const T* __restrict__ at, const T* __restrict__ szz, double s2, double l2, double p,
    int c0, int ldx, T* __restrict__ X) {
  extern __shared__ __align__(16) unsigned char ksm[];
  const int a = blockIdx.x;
  const int s = atom_struct[a];
  if (rowF[s] < 0) return;
  const int p0 = nbr_off[a], nn = nbr_off[a + 1] - p0;
  const int nv = nn + 1;
  T* V = reinterpret_cast<T*>(ksm);                 // nv * 3 * KK
  T* gx = V + (size_t)nv * 3 * KK;                   // nv * 3
  int* cen = reinterpret_cast<int*>(gx + nv * 3);    // nv
  const int tid = threadIdx.x;
  // stage the vectors
  for (int e = tid; e < 3 * KK; e += kKT) {
    T acc = T(0);
    for (int q = 0; q < nn; ++q) acc += dB[(size_t)(p0 + q) * 3 * KK + e];
    V[e] = acc;
  }
  for (int e = tid; e < nn * 3 * KK; e += kKT) {
    const int q = e / (3 * KK), r = e - q * 3 * KK;
    V[(size_t)(q + 1) * 3 * KK + r] = dB[(size_t)rev[p0 + q] * 3 * KK + r];
  }
  for (int v = tid; v < nv; v += kKT) cen[v] = v == 0 ? a : nbr_idx[p0 + v - 1];
  __syncthreads();
  for (int e = tid; e < nv * 3; e += kKT) {
    const int v = e / 3;
    const T* x = B + (size_t)cen[v] * KK;
    const T* g = V + (size_t)e * KK;
    T d = T(0);
    for (int c = 0; c < KK; ++c) d = fma(g[c], x[c], d);
    gx[e] = d;
  }
  __syncthreads();
  const long long row = rowF[s] + 3LL * (a - atom_start[s]);
  for (int k = tid; k < nk; k += kKT) {
    T out[3] = {T(0), T(0), T(0)};
    const T sz = szz[k];
    for (int v0 = 0; v0 < nv; v0 += kVC) {
      const int vn = min(kVC, nv - v0);
      T dot[kVC][3];
#pragma unroll
      for (int v = 0; v < kVC; ++v) dot[v][0] = dot[v][1] = dot[v][2] = T(0);
      for (int c = 0; c < KK; ++c) {
        const T zc = Zt[(size_t)c * nk + k];
#pragma unroll
        for (int v = 0; v < kVC; ++v) {
          if (v < vn) {
            const T* g = V + (size_t)(v0 + v) * 3 * KK + c;
            dot[v][0] = fma(g[0], zc, dot[v][0]);
            dot[v][1] = fma(g[KK], zc, dot[v][1]);
            dot[v][2] = fma(g[2 * KK], zc, dot[v][2]);
          }
        }
      }
#pragma unroll
      for (int v = 0; v < kVC; ++v) {
        if (v < vn) {
          const int vv = v0 + v, ce = cen[vv];
          const T* atc = at + 4 * (size_t)ce;
          if (atc[3] == T(0)) continue;  // a centre without neighbours has no kernel derivative
          T kv, c1, c2;
          krr_coef<T>(F[(size_t)ce * nk + k], atc, sz, s2, l2, p, kv, c1, c2);
          const T sg = vv == 0 ? T(1) : T(-1);
#pragma unroll
          for (int al = 0; al < 3; ++al) out[al] += sg * (c1 * dot[v][al] - c2 * gx[vv * 3 + al]);
        }
      }
    }
#pragma unroll
    for (int al = 0; al < 3; ++al) X[(row + al) * ldx + c0 + k] = out[al];
  }
}

// per atom: T_s = sum_n g_{n, sa(s)} uu_{sb(s)} / r (6 x KK) and T_s . x (6)
template <typename T>
__global__ void __launch_bounds__(128) k_krr_stress_atom(int KK, const int* __restrict__ atom_struct,
                                                         const int* __restrict__ small,
                                                         const int* __restrict__ nbr_off,
                                                         const double* __restrict__ nbr_u, const T* __restrict__ B,
                                                         const T* __restrict__ dB, double sign_big,
                                                         T* __restrict__ Ts, T* __restrict__ tx) {
  const int a = blockIdx.x;
  const int p0 = nbr_off[a], nn = nbr_off[a + 1] - p0;
  const bool sm = small[atom_struct[a]] != 0;
  __shared__ double red[6][4];
  double part[6] = {0, 0, 0, 0, 0, 0};
  for (int e = threadIdx.x; e < 6 * KK; e += blockDim.x) {
    const int sidx = e / KK, c = e - sidx * KK;
    double acc = 0.0;
    for (int q = 0; q < nn; ++q) {
      const double* u = nbr_u + 3 * (size_t)(p0 + q);
      const double r = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
      const double uu = sm ? u[c_sb[sidx]] : -sign_big * u[c_sb[sidx]];
      acc += (double)dB[((size_t)(p0 + q) * 3 + c_sa[sidx]) * KK + c] * uu / r;
    }
    Ts[((size_t)a * 6 + sidx) * KK + c] = (T)acc;
    part[sidx] += acc * (double)B[(size_t)a * KK + c];
  }
  for (int sidx = 0; sidx < 6; ++sidx) {
    double v = part[sidx];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[sidx][threadIdx.x >> 5] = v;
  }
  __syncthreads();
  if (threadIdx.x < 6) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[threadIdx.x][w];
    tx[6 * (size_t)a + threadIdx.x] = (T)t;
  }
}

// stress rows: grid (S, ceil(nk / kKT)); scale sign_stress * 3 / V
template <typename T>
__global__ void __launch_bounds__(kKT) k_krr_stress(int KK, int nk, const int* __restrict__ atom_start,
                                                    const long long* __restrict__ rowS,
                                                    const double* __restrict__ volume, double sign_stress,
                                                    const T* __restrict__ Ts, const T* __restrict__ tx,
                                                    const T* __restrict__ Zt, const T* __restrict__ F,
                                                    const T* __restrict__ at, const T* __restrict__ szz, double s2,
                                                    double l2, double p, int c0, int ldx, T* __restrict__ X) {
  const int s = blockIdx.x;
  const int k = blockIdx.y * kKT + threadIdx.x;
  if (rowS[s] < 0 || k >= nk) return;
  double acc[6] = {0, 0, 0, 0, 0, 0};
  const T sz = szz[k];
  for (int a = atom_start[s]; a < atom_start[s + 1]; ++a) {
    const T* atc = at + 4 * (size_t)a;
    if (atc[3] == T(0)) continue;
    T kv, c1, c2;
    krr_coef<T>(F[(size_t)a * nk + k], atc, sz, s2, l2, p, kv, c1, c2);
    const T* Ta = Ts + (size_t)a * 6 * KK;
    T d[6] = {T(0), T(0), T(0), T(0), T(0), T(0)};
    for (int c = 0; c < KK; ++c) {
      const T zc = Zt[(size_t)c * nk + k];
#pragma unroll
      for (int sidx = 0; sidx < 6; ++sidx) d[sidx] = fma(Ta[sidx * KK + c], zc, d[sidx]);
    }
#pragma unroll
    for (int sidx = 0; sidx < 6; ++sidx)
      acc[sidx] += (double)c1 * (double)d[sidx] - (double)c2 * (double)tx[6 * (size_t)a + sidx];
  }
  const double sc = sign_stress * 3.0 / volume[s];
#pragma unroll
  for (int sidx = 0; sidx < 6; ++sidx) X[(rowS[s] + sidx) * ldx + c0 + k] = (T)(sc * acc[sidx]);
}

// Zt[c][k] = Z[k][c]
template <typename T>
__global__ void k_krr_transpose(int nk, int KK, const T* __restrict__ Z, T* __restrict__ Zt) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nk * KK) return;
  const int k = e / KK, c = e - k * KK;
  Zt[(size_t)c * nk + k] = Z[e];
}

size_t krr_workspace_elems(int A, int nk, int KK) {
  // at (4A), szz (nk), Zt (nk KK), F (A nk), Ts (6 A KK), tx (6A)
  return 4 * (size_t)A + nk + (size_t)nk * KK + (size_t)A * nk + 6 * (size_t)A * KK + 6 * (size_t)A + 64;
}

template <typename T>
cudaError_t launch_krr_rows(const DevBatch& b, const DevRows& rows, const int* rev, const T* Bq, const T* dBq,
                            const T* Z, int nk, int KK, double power, double length, double sigma,
                            double sign_stress, double sign_big, T* ws, T* X, int c0, cudaStream_t st,
                            int* launches) {
  if (b.A == 0 || nk == 0) return cudaSuccess;
  const double l2 = 2.0 * length * length, s2 = sigma * sigma;
  T* at = ws;
  T* szz = at + 4 * (size_t)b.A;
  T* Zt = szz + nk;
  T* F = Zt + (size_t)nk * KK;
  T* Ts = F + (size_t)b.A * nk;
  T* tx = Ts + 6 * (size_t)b.A * KK;
  k_krr_atom<T><<<(b.A + 255) / 256, 256, 0, st>>>(b.A, KK, Bq, b.nbr_off, s2, l2, power, at);
  k_krr_points<T><<<(nk + 255) / 256, 256, 0, st>>>(nk, KK, Z, s2, l2, power, szz);
  k_krr_transpose<T><<<(nk * KK + 255) / 256, 256, 0, st>>>(nk, KK, Z, Zt);
  dim3 gx((nk + 63) / 64, (b.A + 63) / 64);
  k_krr_xz<T><<<gx, 256, 0, st>>>(b.A, nk, KK, Bq, Z, F);
  dim3 gs(b.S, (nk + kKT - 1) / kKT);
  k_krr_energy<T><<<gs, kKT, 0, st>>>(nk, b.atom_start, rows.rowE, F, at, szz, s2, l2, power, c0, rows.ldx, X);
  // force rows: shared memory for the largest neighbour count
  const int maxnn = b.maxnn;
  const size_t smem = sizeof(T) * ((size_t)(maxnn + 1) * 3 * KK + 3 * (size_t)(maxnn + 1)) + sizeof(int) * (maxnn + 1) + 16;
  cudaError_t e = cudaFuncSetAttribute(k_krr_force<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k_krr_force<T><<<b.A, kKT, smem, st>>>(KK, nk, b.atom_struct, b.atom_start, rows.rowF, b.nbr_off, b.nbr_idx, rev,
                                         Bq, dBq, Zt, F, at, szz, s2, l2, power, c0, rows.ldx, X);
  k_krr_stress_atom<T><<<b.A, 128, 0, st>>>(KK, b.atom_struct, b.small, b.nbr_off, b.nbr_u, Bq, dBq, sign_big, Ts,
                                            tx);
  k_krr_stress<T><<<gs, kKT, 0, st>>>(KK, nk, b.atom_start, rows.rowS, b.volume, sign_stress, Ts, tx, Zt, F, at,
                                      szz, s2, l2, power, c0, rows.ldx, X);
  *launches = 8;
  return cudaGetLastError();
}

template cudaError_t launch_krr_rows<float>(const DevBatch&, const DevRows&, const int*, const float*, const float*,
                                            const float*, int, int, double, double, double, double, double, float*,
                                            float*, int, cudaStream_t, int*);
template cudaError_t launch_krr_rows<double>(const DevBatch&, const DevRows&, const int*, const double*,
                                             const double*, const double*, int, int, double, double, double, double,
                                             double, double*, double*, int, cudaStream_t, int*);

}  // namespace mld
