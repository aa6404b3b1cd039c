// Quadratic design rows (mld_order = 2) from per-atom B and per-pair dB.
//
// The reference's quadratic rows (QML full layout, index K*(id1-1)+id2) are
//   energy  sum_i B_i(id1) B_i(id2)                                     (mld_energy.F90:170-266)
//   force   row(a) -= sum over centres c of [f_c(id1) B_c(id2) + f_c(id2) B_c(id1)], f_c the
//           post-flip derivative of centre c's descriptor w.r.t. atom a  (mld_forces.F90:410-500)
//   stress  sign*3/V sum_{i,n} [f(id1) B_nb(id2) + f(id2) B_nb(id1)] uu/r, B_nb the NEIGHBOUR's B
//           (mld_stress.F90:340-356, :580-603: ik = kind_neigh(ia, ia_n))
// Every quadratic feature is symmetric in (id1, id2), so this build stores the upper triangle
// once: column q(i,j) (i <= j, row-major triangle) holds sqrt(2)*F(i,j) off the diagonal and
// F(i,i) on it.  Least-squares predictions and the ridge penalty are then identical to the full
// layout (w_full(i,j) = w_full(j,i) = w(i,j)/sqrt(2)).
//
// Force rows of atom a gather their contributors through the reverse pair of each neighbour
// pair (b -> a), so no atomics are needed: contributor set {self: g = sum_n dB(a,n), B_a} and
// {neighbour b: g = -dB(b -> a), B_b}.  Row(a, alpha)(i,j) = sum_c g_i B_j + g_j B_i, i.e. a
// (K x C) x (C x K) product per component.  Stress rows group the pairs by their neighbour atom:
// H_s[b] = sum_{pairs q -> b} w_s(q) dB(q, alpha_s), S_s = sum_b H_s[b] (x) B_b + B_b (x) H_s[b].
#include <cuda_runtime.h>

#include "mld_internal.h"

namespace mld {

__device__ __forceinline__ int tri_index(int i, int j, int K) {  // i <= j
  return i * K - (i * (i - 1)) / 2 + (j - i);
}

// rev[p]: index of the pair (nbr(p) -> centre(p)) with the opposite displacement.
__global__ void k_reverse_pairs(int A, const int* __restrict__ nbr_off, const int* __restrict__ nbr_idx,
                                const double* __restrict__ nbr_u, int* __restrict__ rev) {
  const int lane = threadIdx.x & 31;
  const int a = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (a >= A) return;
  for (int p = nbr_off[a] + lane; p < nbr_off[a + 1]; p += 32) {
    const int b = nbr_idx[p];
    const double u0 = nbr_u[3 * (size_t)p], u1 = nbr_u[3 * (size_t)p + 1], u2 = nbr_u[3 * (size_t)p + 2];
    // the lists are in ascending neighbour order (images of one neighbour adjacent): binary
    // search for a's first entry in b's list, then its images in order; a full scan only if
    // that finds nothing, so the result is the first match in list order either way
    auto matches = [&](int q) {
      const double d = fabs(nbr_u[3 * (size_t)q] + u0) + fabs(nbr_u[3 * (size_t)q + 1] + u1) +
                       fabs(nbr_u[3 * (size_t)q + 2] + u2);
      return d < 1e-8;
    };
    const int q0 = nbr_off[b], q1 = nbr_off[b + 1];
    int lo = q0, hi = q1;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (nbr_idx[mid] < a) lo = mid + 1;
      else hi = mid;
    }
    int found = -1;
    for (int q = lo; q < q1 && nbr_idx[q] == a; ++q)
      if (matches(q)) {
        found = q;
        break;
      }
    if (found < 0)
      for (int q = q0; q < q1; ++q)
        if (nbr_idx[q] == a && matches(q)) {
          found = q;
          break;
        }
    rev[p] = found;
  }
}

constexpr int kQT = 4;    // 4x4 output tiles of the triangle
constexpr int kQC = 16;   // contributors staged per pass when they do not all fit

// One CTA per atom: its 3 quadratic force rows (dedup layout, written at column offset qoff)
// and its stress partials H[a][s][k].  The contributors (the atom itself, then each neighbour)
// are staged qc at a time: all at once when 1 + nn <= qc, so that every triangle block reads
// them without restaging.  FP32: three resident CTAs per SM (registers capped at 80).
template <typename T>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 3 : 1) k_quad_force(
    int A, int KK, const int* __restrict__ atom_struct, const int* __restrict__ atom_start,
    const int* __restrict__ nbr_off, const int* __restrict__ nbr_idx, const double* __restrict__ nbr_u,
    const int* __restrict__ rev, const int* __restrict__ small, double sign_big, const T* __restrict__ B,
    const T* __restrict__ dB, const long long* __restrict__ rowF, T* __restrict__ X, int ldx, int qoff,
    T* __restrict__ H, int maxnn, int qc) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int a = blockIdx.x;
  if (a >= A) return;
  const int s = atom_struct[a];
  const int a0 = atom_start[s];
  const int p0 = nbr_off[a], nn = nbr_off[a + 1] - p0;
  const int KP = (KK + kQT - 1) / kQT * kQT;
  T* G = reinterpret_cast<T*>(smem_raw);        // qc * 3 * KP
  T* Bc = G + (size_t)qc * 3 * KP;               // qc * KP
  T* fac = Bc + (size_t)qc * KP;                 // maxnn * 3: lever-arm factors of the reverse pairs
  int* qrev = reinterpret_cast<int*>(fac + 3 * (size_t)maxnn);  // maxnn
  const int tid = threadIdx.x, nth = blockDim.x;

  // stress partials of atom a (as the neighbour of its neighbours' pairs); the FP64 geometry of
  // each reverse pair is reduced to three factors once
  if (H) {
    const double sg = small[s] ? 1.0 : -sign_big;
    for (int n = tid; n < nn; n += nth) {
      const int q = rev[p0 + n];
      qrev[n] = q;
      if (q >= 0) {
        const double* u = nbr_u + 3 * (size_t)q;
        const double f = sg / sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
        fac[3 * n + 0] = (T)(f * u[0]);
        fac[3 * n + 1] = (T)(f * u[1]);
        fac[3 * n + 2] = (T)(f * u[2]);
      }
    }
    __syncthreads();
    for (int e = tid; e < 6 * KK; e += nth) {
      const int sidx = e / KK, k = e - sidx * KK;
      const int aa = sidx < 3 ? sidx : (sidx == 3 ? 1 : 0);
      const int bb = sidx < 3 ? sidx : (sidx == 5 ? 1 : 2);
      T acc = T(0);
      for (int n = 0; n < nn; ++n) {
        const int q = qrev[n];
        if (q < 0) continue;
        acc = fma(dB[((size_t)q * 3 + aa) * KK + k], fac[3 * n + bb], acc);
      }
      H[((size_t)a * 6 + sidx) * KK + k] = acc;
    }
  }
  if (!rowF || rowF[s] < 0) return;

  const int nblk = KP / kQT;
  const int ntri = nblk * (nblk + 1) / 2;
  const int ncontrib = 1 + nn;
  // contributors c0 .. c0 + cn - 1 into G (gradient rows, items (c, alpha, k)) and Bc: the atom
  // itself (c = 0: its pairs' derivatives summed in pair order) or neighbour c - 1 (minus the
  // derivative of its descriptor with respect to this atom)
  auto stage = [&](int c0, int cn) {
    for (int e = tid; e < cn * 3 * KP; e += nth) {
      const int c = e / (3 * KP), r = e - c * 3 * KP, al = r / KP, k = r - al * KP;
      const int cc = c0 + c;
      T g = T(0);
      if (k < KK) {
        if (cc == 0) {
          for (int n = 0; n < nn; ++n) g += dB[((size_t)(p0 + n) * 3 + al) * KK + k];
        } else {
          const int q = rev[p0 + cc - 1];
          if (q >= 0) g = -dB[((size_t)q * 3 + al) * KK + k];
        }
      }
      G[(c * 3 + al) * KP + k] = g;
    }
    for (int e = tid; e < cn * KP; e += nth) {
      const int c = e / KP, k = e - c * KP;
      const int cc = c0 + c;
      const int src = cc == 0 ? a : nbr_idx[p0 + cc - 1];
      Bc[c * KP + k] = k < KK ? B[(size_t)src * KK + k] : T(0);
    }
  };
  const bool once = ncontrib <= qc;
  if (once) {
    __syncthreads();
    stage(0, ncontrib);
    __syncthreads();
  }
  for (int tb = tid; tb < ((ntri + nth - 1) / nth) * nth; tb += nth) {
    // decode triangle block (bi <= bj)
    int bi = 0, t = tb;
    while (bi < nblk && t >= nblk - bi) {
      t -= nblk - bi;
      ++bi;
    }
    const int bj = bi + t;
    const bool valid = tb < ntri;
    T acc[3][kQT][kQT];
#pragma unroll
    for (int al = 0; al < 3; ++al)
#pragma unroll
      for (int x = 0; x < kQT; ++x)
#pragma unroll
        for (int y = 0; y < kQT; ++y) acc[al][x][y] = T(0);
    for (int c0 = 0; c0 < ncontrib; c0 += qc) {
      const int cn = min(qc, ncontrib - c0);
      if (!once) {
        __syncthreads();
        stage(c0, cn);
        __syncthreads();
      }
      if (valid) {
        for (int c = 0; c < cn; ++c) {
          T bi4[kQT], bj4[kQT];
#pragma unroll
          for (int x = 0; x < kQT; ++x) {
            bi4[x] = Bc[c * KP + bi * kQT + x];
            bj4[x] = Bc[c * KP + bj * kQT + x];
          }
#pragma unroll
          for (int al = 0; al < 3; ++al) {
            T gi[kQT], gj[kQT];
#pragma unroll
            for (int x = 0; x < kQT; ++x) {
              gi[x] = G[(c * 3 + al) * KP + bi * kQT + x];
              gj[x] = G[(c * 3 + al) * KP + bj * kQT + x];
            }
#pragma unroll
            for (int x = 0; x < kQT; ++x)
#pragma unroll
              for (int y = 0; y < kQT; ++y) acc[al][x][y] = fma(gi[x], bj4[y], fma(gj[y], bi4[x], acc[al][x][y]));
          }
        }
      }
    }
    if (valid) {
      const T r2 = (T)1.4142135623730951;
      const long long row0 = rowF[s] + 3LL * (a - a0);
#pragma unroll
      for (int x = 0; x < kQT; ++x)
#pragma unroll
        for (int y = 0; y < kQT; ++y) {
          const int i = bi * kQT + x, j = bj * kQT + y;
          if (i >= KK || j >= KK || i > j) continue;
          const T sc = (i == j) ? T(1) : r2;
          const int col = qoff + tri_index(i, j, KK);
#pragma unroll
          for (int al = 0; al < 3; ++al) X[(row0 + al) * ldx + col] = sc * acc[al][x][y];
        }
    }
  }
}

// grid (S, 7): r = 0 energy row (B (x) B), r = 1..6 stress rows (H_s (x) B + B (x) H_s) * 3/V.
template <typename T>
__global__ void __launch_bounds__(256) k_quad_struct(int KK, const int* __restrict__ atom_start,
                                                     const T* __restrict__ B, const T* __restrict__ H,
                                                     const double* __restrict__ volume, double sign_stress,
                                                     const long long* __restrict__ rowE,
                                                     const long long* __restrict__ rowS, T* __restrict__ X, int ldx,
                                                     int qoff) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int s = blockIdx.x, r = blockIdx.y;
  const long long row = (r == 0) ? rowE[s] : (rowS[s] >= 0 ? rowS[s] + (r - 1) : -1);
  if (row < 0) return;
  const int a0 = atom_start[s], nat = atom_start[s + 1] - a0;
  const int KP = (KK + kQT - 1) / kQT * kQT;
  constexpr int CH = 32;  // atoms per staged chunk
  T* Bs = reinterpret_cast<T*>(smem_raw);  // CH * KP
  T* Hs = Bs + CH * KP;                    // CH * KP
  const int tid = threadIdx.x, nth = blockDim.x;
  const int nblk = KP / kQT;
  const int ntri = nblk * (nblk + 1) / 2;
  for (int tb = tid; tb < ((ntri + nth - 1) / nth) * nth; tb += nth) {
    int bi = 0, t = tb;
    while (bi < nblk && t >= nblk - bi) {
      t -= nblk - bi;
      ++bi;
    }
    const int bj = bi + t;
    const bool valid = tb < ntri;
    T acc[kQT][kQT];
#pragma unroll
    for (int x = 0; x < kQT; ++x)
#pragma unroll
      for (int y = 0; y < kQT; ++y) acc[x][y] = T(0);
    for (int c0 = 0; c0 < nat; c0 += CH) {
      const int cn = min(CH, nat - c0);
      __syncthreads();
      for (int e = tid; e < cn * KP; e += nth) {
        const int c = e / KP, k = e - c * KP;
        const size_t at = (size_t)(a0 + c0 + c);
        Bs[c * KP + k] = (k < KK) ? B[at * KK + k] : T(0);
        Hs[c * KP + k] = (k < KK && r > 0) ? H[(at * 6 + (r - 1)) * KK + k] : T(0);
      }
      __syncthreads();
      if (!valid) continue;
      for (int c = 0; c < cn; ++c) {
        T bi4[kQT], bj4[kQT], hi4[kQT], hj4[kQT];
#pragma unroll
        for (int x = 0; x < kQT; ++x) {
          bi4[x] = Bs[c * KP + bi * kQT + x];
          bj4[x] = Bs[c * KP + bj * kQT + x];
          hi4[x] = Hs[c * KP + bi * kQT + x];
          hj4[x] = Hs[c * KP + bj * kQT + x];
        }
        if (r == 0) {
#pragma unroll
          for (int x = 0; x < kQT; ++x)
#pragma unroll
            for (int y = 0; y < kQT; ++y) acc[x][y] = fma(bi4[x], bj4[y], acc[x][y]);
        } else {
#pragma unroll
          for (int x = 0; x < kQT; ++x)
#pragma unroll
            for (int y = 0; y < kQT; ++y) acc[x][y] = fma(hi4[x], bj4[y], fma(bi4[x], hj4[y], acc[x][y]));
        }
      }
    }
    if (valid) {
      const T r2 = (T)1.4142135623730951;
      const T sc0 = (r == 0) ? T(1) : (T)(sign_stress * 3.0 / volume[s]);
#pragma unroll
      for (int x = 0; x < kQT; ++x)
#pragma unroll
        for (int y = 0; y < kQT; ++y) {
          const int i = bi * kQT + x, j = bj * kQT + y;
          if (i >= KK || j >= KK || i > j) continue;
          const T sc = ((i == j) ? T(1) : r2) * sc0;
          X[row * ldx + qoff + tri_index(i, j, KK)] = sc * acc[x][y];
        }
    }
  }
}

cudaError_t launch_reverse_pairs(const DevBatch& b, int* rev, cudaStream_t st) {
  if (b.A == 0) return cudaSuccess;
  const long long threads = (long long)b.A * 32;
  k_reverse_pairs<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(b.A, b.nbr_off, b.nbr_idx, b.nbr_u, rev);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_quad_rows(const DevBatch& b, const DevRows& rows, const BsoParams& p, int KK, const int* rev,
                             const T* B, const T* dB, T* H, T* X, int qoff, cudaStream_t st) {
  if (b.A == 0) return cudaSuccess;
  const int KP = (KK + kQT - 1) / kQT * kQT;
  const int mnn = std::max(1, b.maxnn);
  // every contributor staged once when they fit in 96 KB (two CTAs per SM), else kQC at a time
  auto smem_for = [&](int qc) {
    return sizeof(T) * ((size_t)qc * 4 * KP + 3 * (size_t)mnn) + sizeof(int) * (size_t)mnn + 16;
  };
  const int qc = smem_for(1 + mnn) <= 96 * 1024 ? 1 + mnn : kQC;
  const size_t sm1 = smem_for(qc);
  cudaError_t e = cudaFuncSetAttribute(k_quad_force<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm1);
  if (e != cudaSuccess) return e;
  k_quad_force<T><<<b.A, 256, sm1, st>>>(b.A, KK, b.atom_struct, b.atom_start, b.nbr_off, b.nbr_idx, b.nbr_u, rev,
                                         b.small, p.sign_big, B, dB, rows.rowF, X, rows.ldx, qoff, H, mnn, qc);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  size_t sm2 = sizeof(T) * (size_t)2 * 32 * KP;
  e = cudaFuncSetAttribute(k_quad_struct<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm2);
  if (e != cudaSuccess) return e;
  k_quad_struct<T><<<dim3(b.S, 7), 256, sm2, st>>>(KK, b.atom_start, B, H, b.volume, p.sign_stress, rows.rowE,
                                                    rows.rowS, X, rows.ldx, qoff);
  return cudaGetLastError();
}

template cudaError_t launch_quad_rows<double>(const DevBatch&, const DevRows&, const BsoParams&, int, const int*,
                                              const double*, const double*, double*, double*, int, cudaStream_t);
template cudaError_t launch_quad_rows<float>(const DevBatch&, const DevRows&, const BsoParams&, int, const int*,
                                             const float*, const float*, float*, float*, int, cudaStream_t);

}  // namespace mld
