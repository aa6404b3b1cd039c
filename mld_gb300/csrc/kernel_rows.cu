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

#include "ds.cuh"
#include "krr.cuh"
#include "mld_internal.h"

namespace mld {

namespace {
constexpr int kKT = 256;   // threads per CTA (one reference point each per pass)
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


// energy rows: grid (S, ceil(nk / kKT))
template <typename T>
__global__ void __launch_bounds__(kKT) k_krr_energy(int nk, const int* __restrict__ atom_start,
                                                    const long long* __restrict__ rowE, const T* __restrict__ F,
                                                    const T* __restrict__ at, const T* __restrict__ szz, double s2,
                                                    double l2, double p, int c0, int ldx, T* __restrict__ X) {
  const int s = blockIdx.x;
  const int k = blockIdx.y * kKT + threadIdx.x;
  if (rowE[s] < 0 || k >= nk) return;
  // kernel values in the kernel's precision (FP64 runs at 1/64 rate), summed in double-FP32
  const T s2t = (T)s2, l2t = (T)l2, pt = (T)p;
  const int ip = (int)p;
  const bool ipow = (double)ip == p && ip >= 0 && ip <= 8;
  float sh = 0.f, sl = 0.f;
  double acc = 0.0;  // FP64 method
  for (int a = atom_start[s]; a < atom_start[s + 1]; ++a) {
    const T* ata = at + 4 * (size_t)a;
    if (ata[3] == T(0)) continue;  // atoms without neighbours contribute zero
    const T base = s2t + F[(size_t)a * nk + k] / l2t;
    T kt = T(1);
    if (ipow) {
      for (int i = 0; i < ip; ++i) kt *= base;
    } else {
      kt = (T)pow((double)base, (double)pt);
    }
    const T kv = kt / (szz[k] * ata[1]);
    if constexpr (sizeof(T) == 8) {
      acc += kv;
    } else {
      float t, e;
      two_sum(sh, kv, t, e);
      sh = t;
      sl += e;
    }
  }
  X[rowE[s] * ldx + c0 + k] = sizeof(T) == 8 ? (T)acc : (T)((double)sh + (double)sl);
}

// Force rows as a register-tiled product: CTA = (tile of NZ reference points, range of target
// atoms).  The tile of standardised reference points Zs[c][k] stays in shared memory; for each
// target atom a its derivative vectors are staged as rows r = 3 v + alpha (vector 0: sum of a's
// own pair derivatives, centre a, sign +1; vectors 1..n: the reversed pairs (j -> a), centre j,
// sign -1), the dots (row . z_k) are formed in 6 x (NZ/16) register tiles, and the epilogue
// forms sign * (c1(centre, k) dot - c2(centre, k) (row . x_centre)) and sums the rows of each
// alpha into the atom's three force rows.
template <int NZ_>
struct KrrTile {
  static constexpr int NZ = NZ_;      // reference points per tile
  static constexpr int CJ = NZ / 16;  // columns per thread
  static constexpr int RI = 6;        // rows per thread per pass (96 rows per pass)
};

// Sum the per-thread partials part[q][j] (column tx + 16 j of output row q) of the 16 thread rows
// ty of a 256-thread CTA into red[q * NZ + k] in a fixed order: the two rows of a warp through a
// shuffle (a + b is exact-symmetric), then the 8 warps in warp order through red8 (8 * Q * NZ).
template <typename T, int Q, int CJ, int NZ>
__device__ __forceinline__ void reduce_rows16(T (&part)[Q][CJ], T* red8, T* red) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, tx = tid & 15;
#pragma unroll
  for (int q = 0; q < Q; ++q)
#pragma unroll
    for (int j = 0; j < CJ; ++j) part[q][j] += __shfl_xor_sync(0xffffffffu, part[q][j], 16);
  if (lane < 16)
#pragma unroll
    for (int q = 0; q < Q; ++q)
#pragma unroll
      for (int j = 0; j < CJ; ++j) red8[((size_t)warp * Q + q) * NZ + tx + 16 * j] = part[q][j];
  __syncthreads();
  for (int e = tid; e < Q * NZ; e += 256) {
    T sum = T(0);
    for (int w = 0; w < 8; ++w) sum += red8[(size_t)w * Q * NZ + e];
    red[e] = sum;
  }
}

template <typename T, int NZ_>
__global__ void __launch_bounds__(256) k_krr_force_tiled(
    int KK, int nk, int A, int atoms_per_cta, int vc, const int* __restrict__ atom_struct,
    const int* __restrict__ atom_start, const long long* __restrict__ rowF, const int* __restrict__ nbr_off,
    const int* __restrict__ nbr_idx, const int* __restrict__ rev, const T* __restrict__ B, const T* __restrict__ dB,
    const T* __restrict__ Z, const T* __restrict__ F, const T* __restrict__ at, const T* __restrict__ szz, double s2,
    double l2, double p, int c0, int ldx, T* __restrict__ X) {
  using Tl = KrrTile<NZ_>;
  constexpr int NZ = Tl::NZ, CJ = Tl::CJ, RI = Tl::RI;
  extern __shared__ __align__(16) unsigned char ksm[];
  T* Zs = reinterpret_cast<T*>(ksm);                   // KK * NZ   [c][k]
  T* Vt = Zs + (size_t)KK * NZ;                        // KK * (3 vc)  [c][r]
  T* gx = Vt + (size_t)KK * 3 * vc;                    // 3 vc
  T* red = gx + 3 * vc;                                // 3 * NZ
  T* cf = red + 3 * NZ;                                // vc * NZ * 2 (c1, c2 per centre)
  T* red8 = cf + (size_t)2 * vc * NZ;                  // 8 * 3 * NZ (fixed-order reduction)
  int* cen = reinterpret_cast<int*>(red8 + (size_t)8 * 3 * NZ);  // vc
  const T s2t = (T)s2, l2t = (T)l2, pt = (T)p;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int k0 = blockIdx.x * NZ;
  const int nkt = min(NZ, nk - k0);
  for (int e = tid; e < KK * NZ; e += 256) {
    const int c = e / NZ, k = e - c * NZ;
    Zs[e] = (k < nkt) ? Z[(size_t)(k0 + k) * KK + c] : T(0);
  }
  const int a_begin = blockIdx.y * atoms_per_cta, a_end = min(A, a_begin + atoms_per_cta);
  for (int a = a_begin; a < a_end; ++a) {
    const int s = atom_struct[a];
    if (rowF[s] < 0) continue;  // uniform over the CTA
    const int p0 = nbr_off[a], nn = nbr_off[a + 1] - p0;
    const int nv = nn + 1;
    T part[3][CJ];
#pragma unroll
    for (int al = 0; al < 3; ++al)
#pragma unroll
      for (int j = 0; j < CJ; ++j) part[al][j] = T(0);
    // derivative vectors in chunks of vc (the atom's neighbour count may exceed what shared
    // memory holds next to the reference-point tile)
    for (int vb = 0; vb < nv; vb += vc) {
    const int nvc = min(vc, nv - vb), R = 3 * nvc;
    __syncthreads();  // previous chunk's (or atom's) epilogue is done with Vt / cf / red
    // stage the rows: Vt[c][3 v + alpha] for the chunk's vectors v = vb + (0 .. nvc - 1)
    if (vb == 0)
      for (int e = tid; e < 3 * KK; e += 256) {
        const int al = e / KK, c = e - al * KK;
        T acc = T(0);
        for (int q = 0; q < nn; ++q) acc += dB[((size_t)(p0 + q) * 3 + al) * KK + c];
        Vt[(size_t)c * R + al] = acc;
      }
    const int q0 = vb == 0 ? 0 : vb - 1, nq = vb + nvc - 1 - q0;  // pairs of the chunk
    for (int e = tid; e < nq * 3 * KK; e += 256) {
      const int qq = e / (3 * KK), r = e - qq * 3 * KK, al = r / KK, c = r - al * KK;
      const int q = q0 + qq, rq = rev[p0 + q];
      Vt[(size_t)c * R + 3 * (q + 1 - vb) + al] = rq >= 0 ? dB[(size_t)rq * 3 * KK + r] : T(0);
    }
    for (int v = tid; v < nvc; v += 256) cen[v] = vb + v == 0 ? a : nbr_idx[p0 + vb + v - 1];
    if (vb == 0)
      for (int e = tid; e < 3 * NZ; e += 256) red[e] = T(0);
    __syncthreads();
    for (int r = tid; r < R; r += 256) {
      const T* x = B + (size_t)cen[r / 3] * KK;
      T d = T(0);
      for (int c = 0; c < KK; ++c) d = fma(Vt[(size_t)c * R + r], x[c], d);
      gx[r] = d;
    }
    // coefficient table of the centres for this tile of reference points
    for (int e = tid; e < nvc * NZ; e += 256) {
      const int v = e / NZ, k = e - v * NZ;
      T c1 = T(0), c2 = T(0);
      if (k < nkt) {
        const int ce = cen[v];
        krr_c12<T>(F[(size_t)ce * nk + k0 + k], at + 4 * (size_t)ce, szz[k0 + k], s2t, l2t, pt, c1, c2);
      }
      cf[2 * (size_t)e] = c1;
      cf[2 * (size_t)e + 1] = c2;
    }
    __syncthreads();
    for (int rb = 0; rb < R; rb += 16 * RI) {
      T acc[RI][CJ];
#pragma unroll
      for (int i = 0; i < RI; ++i)
#pragma unroll
        for (int j = 0; j < CJ; ++j) acc[i][j] = T(0);
      for (int c = 0; c < KK; ++c) {
        T vr[RI], zc[CJ];
#pragma unroll
        for (int i = 0; i < RI; ++i) {
          const int r = rb + ty + 16 * i;
          vr[i] = r < R ? Vt[(size_t)c * R + r] : T(0);
        }
#pragma unroll
        for (int j = 0; j < CJ; ++j) zc[j] = Zs[(size_t)c * NZ + tx + 16 * j];
#pragma unroll
        for (int i = 0; i < RI; ++i)
#pragma unroll
          for (int j = 0; j < CJ; ++j) acc[i][j] = fma(vr[i], zc[j], acc[i][j]);
      }
      // epilogue of this row block
#pragma unroll
      for (int i = 0; i < RI; ++i) {
        const int r = rb + ty + 16 * i;
        if (r >= R) continue;
        const int v = r / 3, al = r - 3 * v;
        const T sg = vb + v == 0 ? T(1) : T(-1);
        const T g = gx[r];
        const T* cv = cf + (size_t)2 * v * NZ;
#pragma unroll
        for (int j = 0; j < CJ; ++j) {
          const int k = tx + 16 * j;
          const T val = sg * (cv[2 * k] * acc[i][j] - cv[2 * k + 1] * g);
          if (al == 0) part[0][j] += val;
          else if (al == 1) part[1][j] += val;
          else part[2][j] += val;
        }
      }
    }
    }  // vector chunks
    reduce_rows16<T, 3, CJ, NZ>(part, red8, red);
    __syncthreads();
    const long long row = rowF[s] + 3LL * (a - atom_start[s]);
    for (int e = tid; e < 3 * nkt; e += 256) {
      const int al = e / nkt, k = e - al * nkt;
      X[(row + al) * ldx + c0 + k0 + k] = red[al * NZ + k];
    }
  }
}

// per atom: T_s = sum_n g_{n, sa(s)} uu_{sb(s)} / r (6 x KK) and T_s . x (6); the pair factors
// uu_b / r are formed once per pair
template <typename T>
__global__ void __launch_bounds__(128) k_krr_stress_atom(int KK, int maxnn, const int* __restrict__ atom_struct,
                                                         const int* __restrict__ small,
                                                         const int* __restrict__ nbr_off,
                                                         const double* __restrict__ nbr_u, const T* __restrict__ B,
                                                         const T* __restrict__ dB, double sign_big,
                                                         T* __restrict__ Ts, T* __restrict__ tx) {
  extern __shared__ __align__(16) unsigned char ssm[];
  T* fac = reinterpret_cast<T*>(ssm);  // maxnn * 3: uu_b / r
  __shared__ double red[6][4];
  const int a = blockIdx.x;
  const int p0 = nbr_off[a], nn = nbr_off[a + 1] - p0;
  const bool sm = small[atom_struct[a]] != 0;
  for (int q = threadIdx.x; q < nn; q += blockDim.x) {
    const double* u = nbr_u + 3 * (size_t)(p0 + q);
    const double r = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
    const double sg = sm ? 1.0 : -sign_big;
    for (int b = 0; b < 3; ++b) fac[3 * q + b] = (T)(sg * u[b] / r);
  }
  __syncthreads();
  double part[6] = {0, 0, 0, 0, 0, 0};
  for (int e = threadIdx.x; e < 6 * KK; e += blockDim.x) {
    const int sidx = e / KK, c = e - sidx * KK;
    const int sa = c_sa[sidx], sb = c_sb[sidx];
    T acc = T(0);
    for (int q = 0; q < nn; ++q) acc = fma(dB[((size_t)(p0 + q) * 3 + sa) * KK + c], fac[3 * q + sb], acc);
    Ts[((size_t)a * 6 + sidx) * KK + c] = acc;
    part[sidx] += (double)acc * (double)B[(size_t)a * KK + c];
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

// Stress rows as a register-tiled product: CTA = (tile of NZ reference points, range of
// structures); per structure its atoms' stress vectors T_{a,s} (6 per atom, centre a) are
// staged 16 atoms (96 rows) at a time, dotted with the tile, turned into
// c1(a, k) dot - c2(a, k) (T_{a,s} . x_a) and summed into the six stress rows.
template <typename T, int NZ_>
__global__ void __launch_bounds__(256) k_krr_stress_tiled(
    int KK, int nk, int S, int structs_per_cta, const int* __restrict__ atom_start,
    const long long* __restrict__ rowS, const double* __restrict__ volume, double sign_stress,
    const T* __restrict__ Ts, const T* __restrict__ tx, const T* __restrict__ Z, const T* __restrict__ F,
    const T* __restrict__ at, const T* __restrict__ szz, double s2, double l2, double p, int c0, int ldx,
    T* __restrict__ X) {
  using Tl = KrrTile<NZ_>;
  constexpr int NZ = Tl::NZ, CJ = Tl::CJ, RI = Tl::RI;
  constexpr int RB = 16 * RI;  // 96 rows = 16 atoms
  extern __shared__ __align__(16) unsigned char ksm[];
  T* Zs = reinterpret_cast<T*>(ksm);  // KK * NZ
  T* Vt = Zs + (size_t)KK * NZ;       // KK * RB  [c][r]
  T* red = Vt + (size_t)KK * RB;      // 6 * NZ
  T* cf = red + 6 * NZ;               // 16 atoms * NZ * 2
  T* red8 = cf + (size_t)2 * 16 * NZ; // 8 * 6 * NZ (fixed-order reduction)
  const T s2t = (T)s2, l2t = (T)l2, pt = (T)p;
  const int tid = threadIdx.x, txi = tid & 15, ty = tid >> 4;
  const int k0 = blockIdx.x * NZ;
  const int nkt = min(NZ, nk - k0);
  for (int e = tid; e < KK * NZ; e += 256) {
    const int c = e / NZ, k = e - c * NZ;
    Zs[e] = (k < nkt) ? Z[(size_t)(k0 + k) * KK + c] : T(0);
  }
  const int s_begin = blockIdx.y * structs_per_cta, s_end = min(S, s_begin + structs_per_cta);
  for (int s = s_begin; s < s_end; ++s) {
    if (rowS[s] < 0) continue;
    const int a0 = atom_start[s], na = atom_start[s + 1] - a0;
    __syncthreads();
    for (int e = tid; e < 6 * NZ; e += 256) red[e] = T(0);
    T part[6][CJ];
#pragma unroll
    for (int q = 0; q < 6; ++q)
#pragma unroll
      for (int j = 0; j < CJ; ++j) part[q][j] = T(0);
    for (int ab = 0; ab < na; ab += 16) {
      const int nrow = 6 * min(16, na - ab);
      __syncthreads();
      for (int e = tid; e < nrow * KK; e += 256) {
        const int r = e / KK, c = e - r * KK;
        Vt[(size_t)c * RB + r] = Ts[(size_t)(a0 + ab) * 6 * KK + e];
      }
      for (int e = tid; e < (nrow / 6) * NZ; e += 256) {
        const int ai = e / NZ, k = e - ai * NZ;
        T c1 = T(0), c2 = T(0);
        if (k < nkt) {
          const int a = a0 + ab + ai;
          krr_c12<T>(F[(size_t)a * nk + k0 + k], at + 4 * (size_t)a, szz[k0 + k], s2t, l2t, pt, c1, c2);
        }
        cf[2 * (size_t)e] = c1;
        cf[2 * (size_t)e + 1] = c2;
      }
      __syncthreads();
      T acc[RI][CJ];
#pragma unroll
      for (int i = 0; i < RI; ++i)
#pragma unroll
        for (int j = 0; j < CJ; ++j) acc[i][j] = T(0);
      for (int c = 0; c < KK; ++c) {
        T vr[RI], zc[CJ];
#pragma unroll
        for (int i = 0; i < RI; ++i) {
          const int r = ty + 16 * i;
          vr[i] = r < nrow ? Vt[(size_t)c * RB + r] : T(0);
        }
#pragma unroll
        for (int j = 0; j < CJ; ++j) zc[j] = Zs[(size_t)c * NZ + txi + 16 * j];
#pragma unroll
        for (int i = 0; i < RI; ++i)
#pragma unroll
          for (int j = 0; j < CJ; ++j) acc[i][j] = fma(vr[i], zc[j], acc[i][j]);
      }
#pragma unroll
      for (int i = 0; i < RI; ++i) {
        const int r = ty + 16 * i;
        if (r >= nrow) continue;
        const int ai = r / 6, a = a0 + ab + ai, sidx = r % 6;
        const T tv = tx[6 * (size_t)a + sidx];
        const T* cv = cf + (size_t)2 * ai * NZ;
#pragma unroll
        for (int j = 0; j < CJ; ++j) {
          const int k = txi + 16 * j;
          const T val = cv[2 * k] * acc[i][j] - cv[2 * k + 1] * tv;
#pragma unroll
          for (int q = 0; q < 6; ++q)
            if (q == sidx) part[q][j] += val;
        }
      }
    }
    reduce_rows16<T, 6, CJ, NZ>(part, red8, red);
    __syncthreads();
    const double sc = sign_stress * 3.0 / volume[s];
    for (int e = tid; e < 6 * nkt; e += 256) {
      const int q = e / nkt, k = e - q * nkt;
      X[(rowS[s] + q) * ldx + c0 + k0 + k] = (T)(sc * (double)red[q * NZ + k]);
    }
  }
}

size_t krr_workspace_elems(int A, int nk, int KK) {
  // at (4A), szz (nk), F (A nk), Ts (6 A KK), tx (6A)
  return 4 * (size_t)A + nk + (size_t)A * nk + 6 * (size_t)A * KK + 6 * (size_t)A + 64;
}

template <typename T>
cudaError_t launch_krr_rows(const DevBatch& b, const DevRows& rows, const int* rev, const T* Bq, const T* dBq,
                            const T* Z, int nk, int KK, double power, double length, double sigma,
                            double sign_stress, double sign_big, T* ws, T* X, int c0, cudaStream_t st,
                            int* launches, void* tcws, size_t tcws_bytes, int* err, int nsm) {
  if (b.A == 0 || nk == 0) return cudaSuccess;
  *launches = 4;
  const double l2 = 2.0 * length * length, s2 = sigma * sigma;
  T* at = ws;
  T* szz = at + 4 * (size_t)b.A;
  T* F = szz + nk;
  T* Ts = F + (size_t)b.A * nk;
  T* tx = Ts + 6 * (size_t)b.A * KK;
  k_krr_atom<T><<<(b.A + 255) / 256, 256, 0, st>>>(b.A, KK, Bq, b.nbr_off, s2, l2, power, at);
  k_krr_points<T><<<(nk + 255) / 256, 256, 0, st>>>(nk, KK, Z, s2, l2, power, szz);
  dim3 gx((nk + 63) / 64, (b.A + 63) / 64);
  k_krr_xz<T><<<gx, 256, 0, st>>>(b.A, nk, KK, Bq, Z, F);
  dim3 gs(b.S, (nk + kKT - 1) / kKT);
  k_krr_energy<T><<<gs, kKT, 0, st>>>(nk, b.atom_start, rows.rowE, F, at, szz, s2, l2, power, c0, rows.ldx, X);
  // stress partials T_s, T_s . x per atom (both paths)
  k_krr_stress_atom<T><<<b.A, 128, sizeof(T) * 3 * (size_t)std::max(1, b.maxnn), st>>>(
      KK, b.maxnn, b.atom_struct, b.small, b.nbr_off, b.nbr_u, Bq, dBq, sign_big, Ts, tx);
  // force and stress rows: on the tensor cores for FP32 rows (krr_tc.cu) when a workspace is
  // given; otherwise register-tiled, reference-point tiles of NZ in shared memory (the widest
  // tile whose working set fits)
  bool force_done = false;
  if constexpr (sizeof(T) == 4) {
    if (tcws && krr_force_tc_available() && KK <= kKrrTcMaxK) {
      int nl = 0;
      cudaError_t e = launch_krr_force_tc(b, rows, rev, Bq, dBq, Z, F, at, szz, Ts, tx, sign_stress, nk, KK, power,
                                          length, sigma, tcws, tcws_bytes, X, c0, err, nsm, st, &nl);
      if (e != cudaSuccess) return e;
      *launches += nl + 1;
      force_done = true;
    }
  }
  if (!force_done) {
    static int optin = 0;
    if (!optin) {
      int dev = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    }
    const int maxnv = b.maxnn + 1;
    auto smem_for = [&](int nz, int vc) {
      return sizeof(T) * ((size_t)KK * nz + (size_t)KK * 3 * vc + 3 * (size_t)vc + 3 * (size_t)nz +
                          (size_t)2 * vc * nz + (size_t)8 * 3 * nz) +
             sizeof(int) * vc + 16;
    };
    // FP32 tiles up to 256 reference points, FP64 up to 64 (register budget of the 6 x NZ/16 tile),
    // all of an atom's derivative vectors at once where they fit, else in chunks of vc
    int nz = 0, vc = maxnv;
    for (int cand : {256, 128, 64, 32})
      if ((sizeof(T) == 4 || cand <= 64) && smem_for(cand, maxnv) <= (size_t)optin) {
        nz = cand;
        break;
      }
    if (!nz) {
      nz = 32;
      while (vc > 1 && smem_for(nz, vc) > (size_t)optin) vc = (vc + 1) / 2;
      if (smem_for(nz, vc) > (size_t)optin) return cudaErrorInvalidConfiguration;  // K too large for the tile
    }
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int ntiles = (nk + nz - 1) / nz;
    const int ranges = std::max(1, std::min(b.A, (2 * nsm + ntiles - 1) / ntiles * 4));
    const int apc = (b.A + ranges - 1) / ranges;
    dim3 g(ntiles, (b.A + apc - 1) / apc);
    const size_t smem = smem_for(nz, vc);
    auto kern = nz == 64 ? k_krr_force_tiled<T, 64> : k_krr_force_tiled<T, 32>;
    if constexpr (sizeof(T) == 4) {
      if (nz == 256) kern = k_krr_force_tiled<T, 256>;
      if (nz == 128) kern = k_krr_force_tiled<T, 128>;
    }
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<g, 256, smem, st>>>(KK, nk, b.A, apc, vc, b.atom_struct, b.atom_start, rows.rowF, b.nbr_off,
                               b.nbr_idx, rev, Bq, dBq, Z, F, at, szz, s2, l2, power, c0, rows.ldx, X);
    *launches += 1;
  }
  if (force_done) return cudaGetLastError();
  {
    static int optin2 = 0;
    if (!optin2) {
      int dev = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&optin2, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    }
    auto smem_for = [&](int nz) {
      return sizeof(T) * ((size_t)KK * nz + (size_t)KK * 96 + 6 * (size_t)nz + (size_t)2 * 16 * nz + (size_t)8 * 6 * nz) +
             16;
    };
    int nz = 0;
    for (int cand : {256, 128, 64, 32})
      if ((sizeof(T) == 4 || cand <= 64) && smem_for(cand) <= (size_t)optin2) {
        nz = cand;
        break;
      }
    if (!nz) return cudaErrorInvalidConfiguration;
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int ntiles = (nk + nz - 1) / nz;
    const int ranges = std::max(1, std::min(b.S, (2 * nsm + ntiles - 1) / ntiles * 4));
    const int spc = (b.S + ranges - 1) / ranges;
    dim3 g(ntiles, (b.S + spc - 1) / spc);
    const size_t smem = smem_for(nz);
    auto kern = nz == 64 ? k_krr_stress_tiled<T, 64> : k_krr_stress_tiled<T, 32>;
    if constexpr (sizeof(T) == 4) {
      if (nz == 256) kern = k_krr_stress_tiled<T, 256>;
      if (nz == 128) kern = k_krr_stress_tiled<T, 128>;
    }
    cudaError_t e2 = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e2 != cudaSuccess) return e2;
    kern<<<g, 256, smem, st>>>(KK, nk, b.S, spc, b.atom_start, rows.rowS, b.volume, sign_stress, Ts, tx, Z, F, at,
                               szz, s2, l2, power, c0, rows.ldx, X);
  }
  *launches += 2;  // stress partials and stress rows
  return cudaGetLastError();
}

template cudaError_t launch_krr_rows<float>(const DevBatch&, const DevRows&, const int*, const float*, const float*,
                                            const float*, int, int, double, double, double, double, double, float*,
                                            float*, int, cudaStream_t, int*, void*, size_t, int*, int);
template cudaError_t launch_krr_rows<double>(const DevBatch&, const DevRows&, const int*, const double*,
                                             const double*, const double*, int, int, double, double, double, double,
                                             double, double*, double*, int, cudaStream_t, int*, void*, size_t, int*,
                                             int);

}  // namespace mld
