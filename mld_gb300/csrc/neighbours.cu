// Neighbour lists within r < r_cut for a batch of periodic structures (one warp per atom).
//
// Large boxes with at least three cells of width r_cut along some lattice direction use linked
// cells: atoms are binned by their fractional coordinates into nc_1 x nc_2 x nc_3 cells (each at
// least r_cut + 1e-3 A wide, so every neighbour lies in one of the 27 cells around an atom's
// own, or fewer where a direction has one or two cells), the warp of an atom scans those cells,
// and each list is then sorted by neighbour index, the order of the all-atom scan.  This is the
// cell decomposition of the reference's large-box search (neighbours.F90:1091-1139,
// ondm_caltabt.F90, ondm_caltabi.F90), with the list order of its per-atom tables.
//
// Small box (some perpendicular cell width below 2*r_cut): every atom j and periodic image
// n in [-nsize, nsize]^3 is a candidate, u = x_j + n.cell - x_i, kept when 1e-15 <= |u|^2 and
// |u| < r_cut -- MILADY src/mld/neighbours.F90:1147-1328 followed by the strict filter of
// build_local_neighbours_ja (:330).  Large box: minimum image through the fractional
// coordinates, wrapping components with |ds| > 0.5 by nint (neighbours.F90:315-324).
// Candidates are scanned in (j, n1, n2, n3) order and compacted with a warp ballot, so the
// neighbour order (and hence every floating-point sum over neighbours) is deterministic.
// The counting pass (pass 0) also writes the FP32 copies of positions and fractional
// coordinates that both passes use for their pre-filter.
#include <cuda_runtime.h>

#include "mld_internal.h"

namespace mld {

// FP32 positions and fractional coordinates of every atom for the pre-filter.  Positions are
// taken relative to the structure's first atom and fractional coordinates are wrapped into [0, 1)
// in FP64 before the FP32 rounding, so that their FP32 error stays of order 1e-7 of the cell
// size even for unwrapped coordinates far from the origin (the pre-filter's band is 1e-3 A).
__global__ void k_nbr_prep(int A, const int* __restrict__ atom_struct, const int* __restrict__ atom_start,
                           const double* __restrict__ pos, const double* __restrict__ recip,
                           float4* __restrict__ pos32, float4* __restrict__ frac32) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= A) return;
  const int s = atom_struct[i];
  const double* bg = recip + 9 * (size_t)s;
  const double* o = pos + 3 * (size_t)atom_start[s];
  const double x0 = pos[3 * (size_t)i], x1 = pos[3 * (size_t)i + 1], x2 = pos[3 * (size_t)i + 2];
  pos32[i] = make_float4((float)(x0 - o[0]), (float)(x1 - o[1]), (float)(x2 - o[2]), 0.f);
  const double f0 = x0 * bg[0] + x1 * bg[1] + x2 * bg[2];
  const double f1 = x0 * bg[3] + x1 * bg[4] + x2 * bg[5];
  const double f2 = x0 * bg[6] + x1 * bg[7] + x2 * bg[8];
  frac32[i] = make_float4((float)(f0 - floor(f0)), (float)(f1 - floor(f1)), (float)(f2 - floor(f2)), 0.f);
}

// periodic image (n1, n2, n3), |n| < 128, packed in one int
__device__ __forceinline__ int pack_image(int n1, int n2, int n3) {
  return ((n1 + 128) << 16) | ((n2 + 128) << 8) | (n3 + 128);
}
// large box: u = x_j - x_i through the fractional coordinates, components with |ds| > 0.5
// wrapped by nint (neighbours.F90:315-324), in FP64
__device__ __forceinline__ void min_image_u(const double* __restrict__ pos, int j, double xi0, double xi1,
                                            double xi2, const double* cl, const double* bg, double* u) {
  const double* xj = pos + 3 * (size_t)j;
  const double e0 = xj[0] - xi0, e1 = xj[1] - xi1, e2 = xj[2] - xi2;
  double ds[3];
  for (int k = 0; k < 3; ++k) {
    double v = e0 * bg[3 * k] + e1 * bg[3 * k + 1] + e2 * bg[3 * k + 2];
    if (v > 0.5 || v < -0.5) v -= round(v);
    ds[k] = v;
  }
  u[0] = cl[0] * ds[0] + cl[3] * ds[1] + cl[6] * ds[2];
  u[1] = cl[1] * ds[0] + cl[4] * ds[1] + cl[7] * ds[2];
  u[2] = cl[2] * ds[0] + cl[5] * ds[1] + cl[8] * ds[2];
}

// One warp per centre atom; lanes take candidates (j, image) in order.  Candidates clearly
// inside or outside r_cut are classified in FP32 from the prepared copies (position error of
// order 1e-6 A against a band of 1e-3 A); only candidates within the band around r_cut (and the
// zero-distance self image) take the exact FP64 test of the reference, so the list is the FP64
// list.  GB300 issues FP64 at 1/64 of the FP32 rate: the counting pass does no FP64 work for the
// clear cases, and the filling pass forms the FP64 displacement only for accepted neighbours.
__global__ void __launch_bounds__(256) k_neighbours(
    int A, const int* __restrict__ atom_struct, const int* __restrict__ atom_start, const double* __restrict__ pos,
    const float4* __restrict__ pos32, const float4* __restrict__ frac32, const double* __restrict__ cell,
    const double* __restrict__ recip, const int* __restrict__ small, const int* __restrict__ nsize, double rcut,
    int pass, int* __restrict__ counts, int* __restrict__ maxcount, const int* __restrict__ offsets,
    int* __restrict__ nbr_idx, double* __restrict__ nbr_u, const int* __restrict__ cnc,
    const int* __restrict__ cell_off, const int* __restrict__ cell_of, const int* __restrict__ cell_start,
    const int* __restrict__ cell_atoms, int cap, int2* __restrict__ tmp) {
  constexpr float kBand = 1e-3f;
  const int lane = threadIdx.x & 31;
  const int g = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (g >= A) return;
  const int s = atom_struct[g];
  const int a0 = atom_start[s], nat = atom_start[s + 1] - a0;
  const double* cl = cell + 9 * (size_t)s;
  const double* bg = recip + 9 * (size_t)s;
  float c32[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) c32[k] = (float)cl[k];
  const float4 pi = pos32[g], fi = frac32[g];
  const double xi0 = pos[3 * (size_t)g], xi1 = pos[3 * (size_t)g + 1], xi2 = pos[3 * (size_t)g + 2];
  const double rc2 = rcut * rcut;
  const float rcb = (float)rcut + kBand, rcb2 = rcb * rcb;
  const float rci = (float)rcut - kBand, rci2 = rci > 0.f ? rci * rci : 0.f;
  constexpr float kSelf2 = 1e-8f;  // FP32 squared distances below this take the exact test (self image)
  const int sm = small[s];
  int n1s = 0, n2s = 0, n3s = 0, nimg = 1;
  if (sm) {
    n1s = nsize[3 * s];
    n2s = nsize[3 * s + 1];
    n3s = nsize[3 * s + 2];
    nimg = (2 * n1s + 1) * (2 * n2s + 1) * (2 * n3s + 1);
  }
  int count = 0;
  const int wbase = (pass == 1) ? offsets[g] : 0;
  if (!sm && cnc && cnc[3 * s] > 0) {
    // linked cells: the unique cells within one cell of the atom's own, in a fixed order
    const int n0 = cnc[3 * s], n1 = cnc[3 * s + 1], n2 = cnc[3 * s + 2];
    const int own = cell_of[g] - cell_off[s];
    const int c0 = own / (n1 * n2), c1 = (own / n2) % n1, c2 = own % n2;
    const int lo0 = n0 >= 3 ? -1 : 0, hi0 = n0 >= 3 ? 1 : n0 - 1;
    const int lo1 = n1 >= 3 ? -1 : 0, hi1 = n1 >= 3 ? 1 : n1 - 1;
    const int lo2 = n2 >= 3 ? -1 : 0, hi2 = n2 >= 3 ? 1 : n2 - 1;
    for (int d0 = lo0; d0 <= hi0; ++d0)
      for (int d1 = lo1; d1 <= hi1; ++d1)
        for (int d2 = lo2; d2 <= hi2; ++d2) {
          const int cell = cell_off[s] + (((c0 + d0 + n0) % n0) * n1 + (c1 + d1 + n1) % n1) * n2 + (c2 + d2 + n2) % n2;
          const int e0 = cell_start[cell], e1 = cell_start[cell + 1];
          for (int base = e0; base < e1; base += 32) {
            const int e = base + lane;
            bool ok = false;
            int jg = 0;
            if (e < e1) {
              jg = cell_atoms[e];
              if (jg != g) {
                const float4 fj = frac32[jg];
                float d0f = fj.x - fi.x, d1f = fj.y - fi.y, d2f = fj.z - fi.z;
                d0f -= rintf(d0f);
                d1f -= rintf(d1f);
                d2f -= rintf(d2f);
                const float g0 = c32[0] * d0f + c32[3] * d1f + c32[6] * d2f;
                const float g1 = c32[1] * d0f + c32[4] * d1f + c32[7] * d2f;
                const float g2 = c32[2] * d0f + c32[5] * d1f + c32[8] * d2f;
                const float r2f = g0 * g0 + g1 * g1 + g2 * g2;
                if (r2f < rci2) {
                  ok = true;
                } else if (r2f < rcb2) {
                  double u[3];
                  min_image_u(pos, jg, xi0, xi1, xi2, cl, bg, u);
                  ok = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]) < rcut;
                }
              }
            }
            const unsigned m = __ballot_sync(0xffffffffu, ok);
            if (pass == 1 && ok) {
              const int slot = wbase + count + __popc(m & ((1u << lane) - 1u));
              nbr_idx[slot] = jg;
              nbr_u[3 * (size_t)slot] = (double)g;
              nbr_u[3 * (size_t)slot + 1] = (double)pack_image(0, 0, 0);
            } else if (pass == 2 && ok) {
              const int k = count + __popc(m & ((1u << lane) - 1u));
              if (k < cap) tmp[(size_t)g * cap + k] = make_int2(jg, pack_image(0, 0, 0));
            }
            count += __popc(m);
          }
        }
    if (pass != 1 && lane == 0) {
      counts[g] = count;
      atomicMax(maxcount, count);
    }
    return;
  }
  const long long ncand = (long long)nat * nimg;
  for (long long base = 0; base < ncand; base += 32) {
    const long long cidx = base + lane;
    bool ok = false;
    int jj = 0, img = 0;
    if (cidx < ncand) {
      if (sm) {
        // 32-bit division when the candidate count fits (the 64-bit one is emulated)
        int im;
        if (ncand < 0x7fffffffLL) {
          const int ci = (int)cidx;
          jj = ci / nimg;
          im = ci - jj * nimg;
        } else {
          jj = (int)(cidx / nimg);
          im = (int)(cidx - (long long)jj * nimg);
        }
        const int n3 = im % (2 * n3s + 1) - n3s;
        im /= (2 * n3s + 1);
        const int n2 = im % (2 * n2s + 1) - n2s;
        const int n1 = im / (2 * n2s + 1) - n1s;
        const float4 pj = pos32[a0 + jj];
        const float f0 = (pi.x - pj.x) - (c32[0] * n1 + c32[3] * n2 + c32[6] * n3);
        const float f1 = (pi.y - pj.y) - (c32[1] * n1 + c32[4] * n2 + c32[7] * n3);
        const float f2 = (pi.z - pj.z) - (c32[2] * n1 + c32[5] * n2 + c32[8] * n3);
        const float r2f = f0 * f0 + f1 * f1 + f2 * f2;
        if (r2f < rci2 && r2f > kSelf2) {
          ok = true;
        } else if (r2f < rcb2) {
          const double* xj = pos + 3 * (size_t)(a0 + jj);
          const double t0 = xi0 - (xj[0] + cl[0] * n1 + cl[3] * n2 + cl[6] * n3);
          const double t1 = xi1 - (xj[1] + cl[1] * n1 + cl[4] * n2 + cl[7] * n3);
          const double t2 = xi2 - (xj[2] + cl[2] * n1 + cl[5] * n2 + cl[8] * n3);
          const double r2 = t0 * t0 + t1 * t1 + t2 * t2;
          ok = (r2 >= 1e-15) && (r2 <= rc2) && (sqrt(r2) < rcut);
        }
        img = pack_image(n1, n2, n3);
      } else {
        jj = (int)cidx;
        if (a0 + jj != g) {
          const float4 fj = frac32[a0 + jj];
          float d0 = fj.x - fi.x, d1 = fj.y - fi.y, d2 = fj.z - fi.z;
          d0 -= rintf(d0);
          d1 -= rintf(d1);
          d2 -= rintf(d2);
          const float g0 = c32[0] * d0 + c32[3] * d1 + c32[6] * d2;
          const float g1 = c32[1] * d0 + c32[4] * d1 + c32[7] * d2;
          const float g2 = c32[2] * d0 + c32[5] * d1 + c32[8] * d2;
          // the FP32 image can differ from the reference's only when a component sits at +-0.5,
          // i.e. at half a cell width (> r_cut for a large box), so its distance is a lower bound
          const float r2f = g0 * g0 + g1 * g1 + g2 * g2;
          // clearly inside: the FP32 image is the reference's (no component near +-0.5)
          if (r2f < rci2) {
            ok = true;
          } else if (r2f < rcb2) {
            double u[3];
            min_image_u(pos, a0 + jj, xi0, xi1, xi2, cl, bg, u);
            ok = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]) < rcut;
          }
        }
      }
    }
    const unsigned m = __ballot_sync(0xffffffffu, ok);
    if (pass == 1 && ok) {
      // the pair and its image; k_nbr_u forms the FP64 displacement, one thread per pair
      const int slot = wbase + count + __popc(m & ((1u << lane) - 1u));
      nbr_idx[slot] = a0 + jj;
      nbr_u[3 * (size_t)slot] = (double)g;
      nbr_u[3 * (size_t)slot + 1] = (double)img;
    } else if (pass == 2 && ok) {
      // single pass: the pair into the atom's fixed-capacity row (compacted after the scan)
      const int k = count + __popc(m & ((1u << lane) - 1u));
      if (k < cap) tmp[(size_t)g * cap + k] = make_int2(a0 + jj, img);
    }
    count += __popc(m);
  }
  if (pass != 1 && lane == 0) {
    counts[g] = count;
    atomicMax(maxcount, count);
  }
}

// Single-pass lists: atom g's pairs from its fixed-capacity row into the CSR (offsets from the
// scan of the counts), in their order; one warp per atom.
__global__ void k_nbr_compact(int A, int cap, const int* __restrict__ counts, const int* __restrict__ offsets,
                              const int2* __restrict__ tmp, int* __restrict__ nbr_idx, double* __restrict__ nbr_u) {
  const int lane = threadIdx.x & 31;
  const int g = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (g >= A) return;
  const int n = min(counts[g], cap), p0 = offsets[g];
  for (int k = lane; k < n; k += 32) {
    const int2 t = tmp[(size_t)g * cap + k];
    nbr_idx[p0 + k] = t.x;
    nbr_u[3 * (size_t)(p0 + k)] = (double)g;
    nbr_u[3 * (size_t)(p0 + k) + 1] = (double)t.y;
  }
}

// FP64 displacement u = x_j + image - x_i of every pair (the reference's arithmetic), from the
// centre and image recorded by the filling pass; one thread per pair.  u32 (optional) receives
// (u, 1/|u|) rounded to FP32 for the FP32 descriptor kernel, so that it runs no FP64 arithmetic.
__global__ void k_nbr_u(long long P, const int* __restrict__ atom_struct, const double* __restrict__ pos,
                        const double* __restrict__ cell, const double* __restrict__ recip,
                        const int* __restrict__ small, const int* __restrict__ nbr_idx, double* __restrict__ nbr_u,
                        float4* __restrict__ u32) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  const int i = (int)nbr_u[3 * p], img = (int)nbr_u[3 * p + 1], j = nbr_idx[p];
  const int s = atom_struct[i];
  const double* cl = cell + 9 * (size_t)s;
  const double xi0 = pos[3 * (size_t)i], xi1 = pos[3 * (size_t)i + 1], xi2 = pos[3 * (size_t)i + 2];
  double u[3];
  if (small[s]) {
    const int n1 = ((img >> 16) & 255) - 128, n2 = ((img >> 8) & 255) - 128, n3 = (img & 255) - 128;
    const double* xj = pos + 3 * (size_t)j;
    u[0] = -(xi0 - (xj[0] + cl[0] * n1 + cl[3] * n2 + cl[6] * n3));
    u[1] = -(xi1 - (xj[1] + cl[1] * n1 + cl[4] * n2 + cl[7] * n3));
    u[2] = -(xi2 - (xj[2] + cl[2] * n1 + cl[5] * n2 + cl[8] * n3));
  } else {
    min_image_u(pos, j, xi0, xi1, xi2, cl, recip + 9 * (size_t)s, u);
  }
  nbr_u[3 * p] = u[0];
  nbr_u[3 * p + 1] = u[1];
  nbr_u[3 * p + 2] = u[2];
  if (u32)
    u32[p] = make_float4((float)u[0], (float)u[1], (float)u[2],
                         (float)(1.0 / sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2])));
}

// Three-phase exclusive scan of n ints: out[0..n], out[n] = total.
constexpr int kScanBlock = 1024;

__global__ void k_scan_blocks(const int* __restrict__ in, int* __restrict__ out, int n, int* __restrict__ bsum) {
  __shared__ int sh[kScanBlock];
  const int i = blockIdx.x * kScanBlock + threadIdx.x;
  int v = (i < n) ? in[i] : 0;
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int o = 1; o < kScanBlock; o <<= 1) {
    int t = (threadIdx.x >= o) ? sh[threadIdx.x - o] : 0;
    __syncthreads();
    sh[threadIdx.x] += t;
    __syncthreads();
  }
  if (i < n) out[i] = sh[threadIdx.x] - v;  // exclusive
  if (threadIdx.x == kScanBlock - 1) bsum[blockIdx.x] = sh[threadIdx.x];
}

__global__ void k_scan_sums(int* __restrict__ bsum, int nb, int* __restrict__ total_out) {
  // single block: sequential chunks of kScanBlock
  __shared__ int sh[kScanBlock];
  int carry = 0;
  for (int base = 0; base < nb; base += kScanBlock) {
    const int i = base + threadIdx.x;
    int v = (i < nb) ? bsum[i] : 0;
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < kScanBlock; o <<= 1) {
      int t = (threadIdx.x >= o) ? sh[threadIdx.x - o] : 0;
      __syncthreads();
      sh[threadIdx.x] += t;
      __syncthreads();
    }
    if (i < nb) bsum[i] = carry + sh[threadIdx.x] - v;
    const int tot = sh[kScanBlock - 1];
    __syncthreads();
    carry += tot;
  }
  if (threadIdx.x == 0) *total_out = carry;
}

__global__ void k_scan_add(int* __restrict__ out, int n, const int* __restrict__ bsum, const int* total) {
  const int i = blockIdx.x * kScanBlock + threadIdx.x;
  if (i < n) out[i] += bsum[blockIdx.x];
  if (i == 0) out[n] = *total;
}

cudaError_t launch_scan(const int* in, int* out, int n, int* d_tmp, cudaStream_t st) {
  // d_tmp must hold ceil(n/1024) + 1 ints
  if (n <= 0) {
    return cudaMemsetAsync(out, 0, sizeof(int), st);
  }
  const int nb = (n + kScanBlock - 1) / kScanBlock;
  k_scan_blocks<<<nb, kScanBlock, 0, st>>>(in, out, n, d_tmp);
  k_scan_sums<<<1, kScanBlock, 0, st>>>(d_tmp, nb, d_tmp + nb);
  k_scan_add<<<nb, kScanBlock, 0, st>>>(out, n, d_tmp, d_tmp + nb);
  return cudaGetLastError();
}

// Cell of every atom of a celled structure from its fractional coordinates wrapped into [0, 1)
// in FP64; cell_start[cell] counts the cell's atoms (the scan turns the counts into offsets).
__global__ void k_cell_bin(int A, const int* __restrict__ atom_struct, const double* __restrict__ pos,
                           const double* __restrict__ recip, const int* __restrict__ cnc,
                           const int* __restrict__ cell_off, int* __restrict__ cell_of, int* __restrict__ count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= A) return;
  const int s = atom_struct[i];
  const int n[3] = {cnc[3 * s], cnc[3 * s + 1], cnc[3 * s + 2]};
  if (n[0] == 0) {
    cell_of[i] = -1;
    return;
  }
  const double* bg = recip + 9 * (size_t)s;
  const double x0 = pos[3 * (size_t)i], x1 = pos[3 * (size_t)i + 1], x2 = pos[3 * (size_t)i + 2];
  int c[3];
  for (int k = 0; k < 3; ++k) {
    double f = x0 * bg[3 * k] + x1 * bg[3 * k + 1] + x2 * bg[3 * k + 2];
    f -= floor(f);
    c[k] = min(n[k] - 1, max(0, (int)(f * n[k])));
  }
  const int cell = cell_off[s] + (c[0] * n[1] + c[1]) * n[2] + c[2];
  cell_of[i] = cell;
  atomicAdd(&count[cell], 1);
}

// atoms into their cells (order within a cell arbitrary: the lists are sorted afterwards)
__global__ void k_cell_fill(int A, const int* __restrict__ cell_of, const int* __restrict__ cell_start,
                            int* __restrict__ cursor, int* __restrict__ cell_atoms) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= A) return;
  const int cell = cell_of[i];
  if (cell < 0) return;
  cell_atoms[cell_start[cell] + atomicAdd(&cursor[cell], 1)] = i;
}

// the list of an atom of a celled structure, sorted by neighbour index (ranks of distinct
// values; one warp per atom); other atoms' lists are copied as they are
__global__ void k_sort_lists(int A, const int* __restrict__ cell_of, const int* __restrict__ nbr_off,
                             const int* __restrict__ idx, int* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int g = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (g >= A) return;
  const int p0 = nbr_off[g], n = nbr_off[g + 1] - p0;
  const bool sort = cell_of[g] >= 0;
  for (int e = lane; e < n; e += 32) {
    const int x = idx[p0 + e];
    int rank = e;
    if (sort) {
      rank = 0;
      for (int f = 0; f < n; ++f) rank += idx[p0 + f] < x;
    }
    out[p0 + rank] = x;
  }
}

cudaError_t launch_cells(const DevBatch& b, int* scan_tmp, cudaStream_t st) {
  if (b.A == 0 || b.ncells == 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(b.cell_start + b.ncells + 1, 0, sizeof(int) * b.ncells, st);
  if (e != cudaSuccess) return e;
  int* count = b.cell_start + b.ncells + 1;  // counts, then the fill cursor
  k_cell_bin<<<(b.A + 255) / 256, 256, 0, st>>>(b.A, b.atom_struct, b.pos, b.recip, b.cnc, b.cell_off, b.cell_of,
                                               count);
  e = launch_scan(count, b.cell_start, b.ncells, scan_tmp, st);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(count, 0, sizeof(int) * b.ncells, st);
  if (e != cudaSuccess) return e;
  k_cell_fill<<<(b.A + 255) / 256, 256, 0, st>>>(b.A, b.cell_of, b.cell_start, count, b.cell_atoms);
  return cudaGetLastError();
}

cudaError_t launch_sort_lists(const DevBatch& b, cudaStream_t st) {
  if (b.A == 0 || b.ncells == 0 || b.P == 0) return cudaSuccess;
  const long long threads = (long long)b.A * 32;
  k_sort_lists<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(b.A, b.cell_of, b.nbr_off, b.nbr_idx, b.sort_tmp);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return cudaMemcpyAsync(b.nbr_idx, b.sort_tmp, sizeof(int) * (size_t)b.P, cudaMemcpyDeviceToDevice, st);
}

cudaError_t launch_neighbours(const DevBatch& b, double rcut, int* counts, int* maxcount, cudaStream_t st, int pass) {
  if (b.A == 0) return cudaSuccess;
  const int threads = 256;
  const long long warps = b.A;
  const int blocks = (int)((warps * 32 + threads - 1) / threads);
  if (!b.pos32 || !b.frac32) return cudaErrorInvalidValue;
  if (pass == 0 || pass == 2)
    k_nbr_prep<<<(b.A + 255) / 256, 256, 0, st>>>(b.A, b.atom_struct, b.atom_start, b.pos, b.recip, b.pos32, b.frac32);
  if (pass == 2 && (!b.nbr_tmp || b.nbr_cap < 1)) return cudaErrorInvalidValue;
  if (pass != 3)
    k_neighbours<<<blocks, threads, 0, st>>>(b.A, b.atom_struct, b.atom_start, b.pos, b.pos32, b.frac32, b.cell,
                                             b.recip, b.small, b.nsize, rcut, pass, counts, maxcount,
                                             b.nbr_off, b.nbr_idx, b.nbr_u, b.ncells > 0 ? b.cnc : nullptr,
                                             b.cell_off, b.cell_of, b.cell_start, b.cell_atoms, b.nbr_cap, b.nbr_tmp);
  if (pass == 2) return cudaGetLastError();
  if (pass == 3 && b.P > 0)
    k_nbr_compact<<<blocks, threads, 0, st>>>(b.A, b.nbr_cap, counts, b.nbr_off, b.nbr_tmp, b.nbr_idx, b.nbr_u);
  if (pass >= 1 && b.P > 0 && b.ncells > 0) {
    // ascending neighbour order of the celled structures' lists, before their displacements
    if (!b.sort_tmp) return cudaErrorInvalidValue;
    cudaError_t e = launch_sort_lists(b, st);
    if (e != cudaSuccess) return e;
  }
  if (pass >= 1 && b.P > 0)
    k_nbr_u<<<(unsigned)((b.P + 255) / 256), 256, 0, st>>>(b.P, b.atom_struct, b.pos, b.cell, b.recip, b.small,
                                                           b.nbr_idx, b.nbr_u, b.nbr_u32);
  return cudaGetLastError();
}

}  // namespace mld
