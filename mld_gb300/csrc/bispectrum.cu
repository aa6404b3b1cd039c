// Bispectrum-SO(4) descriptors and their derivatives: persistent CTAs, one centre atom at a time.
//
// Per atom i with neighbours n (u_n = x_n - x_i, r_n < r_cut):
//   phase 1  c^j(p,q) = delta_pq + sum_n w_ch(type_n) f_c(r_n) U^j_pq(u_n)           (compute_bispectrum_so4.F90:288-439)
//   phase 2  Z blocks ZA/ZB/ZC by Clebsch-Gordan contraction of c, merged per (k, layer) into Y,
//            B_k = Re sum conj(c^l) ZA_k                                               (:1014-1143, :469-560)
//   phase 3  per chunk of neighbours: U/dU recursion -> vecall V = conj(d(f_c U)/du)  (angular_functions.f90:41-273),
//            dB_k/du_n = w_ch(type_n) Re sum Y V (register-tiled per layer)           (:469-717, descriptors.F90:298-302)
// Outputs: B per atom and w_ch * dB per pair (the design rows are gathered from them by
// rows.cu), or, for evaluation with fitted weights, per-pair force and stress contributions.
// Only half of every layer is computed (X(-p,-q) = (-1)^((p-q)/2) conj X(p,q) for U, c, Z, V);
// full-layer sums fold into weighted sums over the half.  The recursions run on lane groups:
// in phase 1 of 16, 8, 6 or 4 lanes per neighbour (the widest that covers the atom's neighbours
// in the fewest passes), each group writing its neighbour's U to a store that is summed in
// group order; in phase 3 of 16 lanes (a warp for a last chunk of at most 8 neighbours);
// phase 2 follows a host-balanced schedule of rounds of 32 terms of one inner extent per warp,
// each distinct Z computation evaluated once.
//
// Every floating-point sum has a fixed order: c is summed over the groups' U in group order,
// pass after pass, Z terms land in a term buffer from which the Y slots and B are summed, and the
// dB contraction writes each layer row into the buffer of its rank (a triple's distinct layers
// in ascending order), where every triple has at most one row, so dB = (rank 0 + rank 1) +
// rank 2.  Results are therefore bitwise reproducible and do not depend on which CTA takes which
// atom.
//
// CTAs are persistent: they stage the recursion records and the small tables in shared memory
// once, then pull atoms from a queue (ordered by descending neighbour count, or in index order,
// whichever the launch-shape autotuner found faster).  Each atom's phase-1 geometry records are
// kept for phase 3.
// T = double (plain FP64 method) or float (mixed method: FP32 descriptors).
#include <cuda_runtime.h>

#include <algorithm>

#include "mld_internal.h"

namespace mld {

template <typename T>
struct cx {
  T x, y;
};

template <typename T>
__device__ __forceinline__ cx<T> cmul(cx<T> a, cx<T> b) {
  return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
template <typename T>
__device__ __forceinline__ cx<T> cfma(cx<T> a, cx<T> b, cx<T> c) {  // a*b + c
  return {fma(a.x, b.x, fma(-a.y, b.y, c.x)), fma(a.x, b.y, fma(a.y, b.x, c.y))};
}
// decode an encoded half-layer reference: (idx << 2) | (conj << 1) | neg
template <typename T>
__device__ __forceinline__ cx<T> fetch(const cx<T>* base, int code) {
  const cx<T> v = base[code >> 2];
  const T sy = (code & 2) ? T(-1) : T(1);
  const T sn = (code & 1) ? T(-1) : T(1);
  return {sn * v.x, sn * sy * v.y};
}

// One Z term: sum_a c1_a sum_b c2_b c[i1 + a s1 + b] c[i2 - a s2 - b] with NB = nb known at compile
// time, so that the b loop unrolls and the term's NB coefficients c2 stay in registers.
template <int NB, typename T>
__device__ __forceinline__ cx<T> zterm(const cx<T>* __restrict__ cc, const T* __restrict__ cgs, uint4 zi) {
  // the item's 16 bytes: x = i1 | i2 << 16, y = cg1 | cg2 << 16, z = na | nb << 8 | s1 << 16 | s2 << 24
  const int cg1 = zi.y & 0xFFFF, cg2 = zi.y >> 16, na = zi.z & 0xFF, s1 = (zi.z >> 16) & 0xFF, s2 = zi.z >> 24;
  T c2[NB];
#pragma unroll
  for (int b = 0; b < NB; ++b) c2[b] = cgs[cg2 + b];
  cx<T> zs = {T(0), T(0)};
  int i1a = zi.x & 0xFFFF, i2a = zi.x >> 16;
#pragma unroll (NB <= 2 ? 4 : (NB <= 5 ? 2 : 1))
  for (int a = 0; a < na; ++a) {
    const T c1 = cgs[cg1 + a];
    cx<T> part = {T(0), T(0)};
#pragma unroll
    for (int b = 0; b < NB; ++b) {
      const cx<T> pr = cmul(cc[i1a + b], cc[i2a - b]);
      part.x = fma(c2[b], pr.x, part.x);
      part.y = fma(c2[b], pr.y, part.y);
    }
    zs.x = fma(c1, part.x, zs.x);
    zs.y = fma(c1, part.y, zs.y);
    i1a += s1;
    i2a -= s2;
  }
  return zs;
}

template <typename T>
struct RecEntry;
template <>
struct RecEntry<float> {
  using type = RecEntry32;
};
template <>
struct RecEntry<double> {
  using type = RecEntry64;
};

// The q < 0 variants are the conjugates: zm = conj(zp), xm = conj(xp), and their derivatives
// likewise, so only the q >= 0 set is kept.
template <typename T>
struct NbrGeom {
  cx<T> zp, xp;
  cx<T> dzp[3], dxp[3];
  T fc, dfr[3];  // fc and dfc * u_a / r
};

// angular_functions.f90:66-107 (the geometric set-up of spherical_4d) and the cutoff of
// compute_bispectrum_so4.F90:337-377 (type-2 cosine outer cut times (1 - inner type-3 cut)).
template <typename T>
__device__ __forceinline__ void nbr_geometry(T x0, T x1, T x2, T rcut, T inv_r0, T rin, T rin_w, NbrGeom<T>* g) {
  const T PI = (T)3.14159265358979323846;
  T rr = sqrt(x0 * x0 + x1 * x1 + x2 * x2);
  T r0 = rcut / inv_r0;
  T th0 = rr / r0;
  T s, c;
  if constexpr (sizeof(T) == 8) sincos(th0, &s, &c);
  else sincosf(th0, &s, &c);
  T sin_i = T(1) / s, tan_i = c / s;
  T l0 = rr * sin_i, l0i = T(1) / l0, z0 = rr * tan_i;
  g->zp = {z0 * l0i, x2 * l0i};
  g->xp = {x0 * l0i, x1 * l0i};
  T rinv = T(1) / rr;
  T drr[3] = {x0 * rinv, x1 * rinv, x2 * rinv};
  T dz = tan_i - th0 * sin_i * sin_i;
  T dil0 = (c / r0 - l0i) * rinv;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    T base = dz * l0i * drr[a];
    g->dzp[a] = {z0 * dil0 * drr[a] + base, x2 * dil0 * drr[a]};
    g->dxp[a] = {x0 * dil0 * drr[a], x1 * dil0 * drr[a]};
  }
  g->dzp[2].y += l0i;
  g->dxp[0].x += l0i;
  g->dxp[1].y += l0i;
  // cutoff (neighbours.F90:598-645, types 2 and 3)
  T fo = 0, dfo = 0;
  if (rr <= rcut) {
    T xx = rr / rcut;
    T sp, cp;
    if constexpr (sizeof(T) == 8) sincos(PI * xx, &sp, &cp);
    else sincosf(PI * xx, &sp, &cp);
    fo = T(0.5) * (cp + T(1));
    dfo = -T(0.5) * PI * sp / rcut;
  }
  T fi = 0, dfi = 0;
  if (rin > T(0)) {
    T rc2 = rin + rin_w, w = rin_w;
    if (rr <= rc2) {
      if (rr < rc2 - w) {
        fi = 1;
        dfi = 0;
      } else {
        T xx = PI * (rr - rc2 + w) / w;
        fi = T(0.5) * (cos(xx) + T(1));
        dfi = -T(0.5) * sin(xx) * PI / w;
      }
    }
  }
  g->fc = (T(1) - fi) * fo;
  T dfc = -dfi * fo + (T(1) - fi) * dfo;
#pragma unroll
  for (int a = 0; a < 3; ++a) g->dfr[a] = dfc * drr[a];
}

// Record of a neighbour in shared memory, written in phase 1 and read back in phase 3: zp, xp,
// dzp[3], dxp[3] as (x, y) pairs, then fc and dfr[3]; at kGeoIdx the neighbour's index and type
// (two ints), at kGeoU its displacement and 1/r (kGeo values, a multiple of 4 so that records
// stay 16-byte aligned).
constexpr int kGeo = 28;
constexpr int kGeoIdx = 20;
constexpr int kGeoU = 22;

template <typename T>
__device__ __forceinline__ void put_geo(const NbrGeom<T>& g, T* r) {
  r[0] = g.zp.x;
  r[1] = g.zp.y;
  r[2] = g.xp.x;
  r[3] = g.xp.y;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    r[4 + 2 * a] = g.dzp[a].x;
    r[5 + 2 * a] = g.dzp[a].y;
    r[10 + 2 * a] = g.dxp[a].x;
    r[11 + 2 * a] = g.dxp[a].y;
    r[17 + a] = g.dfr[a];
  }
  r[16] = g.fc;
}

template <typename T>
__device__ __forceinline__ void get_geo(const T* r, NbrGeom<T>* g) {
  g->zp = {r[0], r[1]};
  g->xp = {r[2], r[3]};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    g->dzp[a] = {r[4 + 2 * a], r[5 + 2 * a]};
    g->dxp[a] = {r[10 + 2 * a], r[11 + 2 * a]};
    g->dfr[a] = r[17 + a];
  }
  g->fc = r[16];
}

// U/dU layer recursion of one neighbour by a group of G lanes (sl = lane within the group) on
// half layers (phase 3); rec and hoff live in shared memory.  vecall is written to V[a*HU + h]:
// dU of layer j-1 stays raw in V until layer j is formed, then is converted.  Every group of the
// warp calls this with the same J so that the warp-wide __syncwarp calls line up; inactive
// groups pass active = false.
template <typename T, int G>
__device__ __forceinline__ void group_recursion(const NbrGeom<T>& g, const typename RecEntry<T>::type* __restrict__ rec,
                                                int J, const int* __restrict__ hoff, cx<T>* ubuf, int LH, cx<T>* V,
                                                int HU, int sl, bool active) {
  cx<T>* prev = ubuf;
  cx<T>* cur = ubuf + LH;
  if (active && sl == 0) {
    prev[0] = {T(1), T(0)};
#pragma unroll
    for (int a = 0; a < 3; ++a) V[a * HU] = {T(0), T(0)};
  }
  __syncwarp();
  for (int j = 1; j <= J; ++j) {
    const int h0 = hoff[j], ne = hoff[j + 1] - h0;
    const int pbase = hoff[j - 1];
    if (active) {
      for (int e = sl; e < ne; e += G) {
        const int idx = h0 + e;
        const auto r = rec[idx];
        const T tzq = (T)r.tz, txq = (T)r.tx;  // tz, tx signed by q: Z = zp or conj(zp), X = conj(xp) or xp
        const T tz = fabs(tzq), tx = fabs(txq);
        const int sz = r.sz, sx = r.sx;
        const cx<T> A = {tz * g.zp.x, tzq * g.zp.y};
        const cx<T> Bc = {-txq * g.xp.y, -tx * g.xp.x};  // -i*tx*X
        cx<T> u = {T(0), T(0)};
        cx<T> du[3] = {{T(0), T(0)}, {T(0), T(0)}, {T(0), T(0)}};
        if (sz >= 0) {
          const cx<T> Uz = fetch(prev, sz);
          u = cmul(A, Uz);
#pragma unroll
          for (int a = 0; a < 3; ++a) {
            du[a] = cfma(A, fetch(V + a * HU + pbase, sz), cmul(cx<T>{tz * g.dzp[a].x, tzq * g.dzp[a].y}, Uz));
          }
        }
        if (sx >= 0) {
          const cx<T> Ux = fetch(prev, sx);
          u = cfma(Bc, Ux, u);
#pragma unroll
          for (int a = 0; a < 3; ++a) {
            du[a] = cfma(Bc, fetch(V + a * HU + pbase, sx), cfma(cx<T>{-txq * g.dxp[a].y, -tx * g.dxp[a].x}, Ux, du[a]));
          }
        }
#pragma unroll
        for (int a = 0; a < 3; ++a) V[a * HU + idx] = du[a];
        cur[e] = u;
      }
    }
    __syncwarp();
    if (active) {
      const int np = h0 - pbase;
      for (int e = sl; e < np; e += G) {
        const cx<T> U = prev[e];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          const cx<T> d = V[a * HU + pbase + e];
          V[a * HU + pbase + e] = {fma(U.x, g.dfr[a], g.fc * d.x), fma(-U.y, g.dfr[a], -g.fc * d.y)};
        }
      }
    }
    __syncwarp();
    cx<T>* t = prev;
    prev = cur;
    cur = t;
  }
  if (active) {
    const int np = hoff[J + 1] - hoff[J];
    for (int e = sl; e < np; e += G) {
      const cx<T> U = prev[e];
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        const cx<T> d = V[a * HU + hoff[J] + e];
        V[a * HU + hoff[J] + e] = {fma(U.x, g.dfr[a], g.fc * d.x), fma(-U.y, g.dfr[a], -g.fc * d.y)};
      }
    }
  }
  __syncwarp();
}

template <typename T>
struct KernelArgs {
  DevTables tb;
  const typename RecEntry<T>::type* rec;
  const T* cg;
  // batch
  const int* atom_struct;
  const int* types;
  const int* small;
  const int* nbr_off;
  const int* nbr_idx;
  const double* nbr_u;
  const float4* u32;  // (u, 1/r) in FP32 for T = float (null: converted from nbr_u)
  // channel weights and inner cutoffs per type pair in T, converted once at launch
  T chw[kMaxCh * kMaxTypes];
  T rin[kMaxTypes * kMaxTypes];
  T rin_w;
  // work queue: atoms in the order given (nullptr: 0..A-1), taken through a global counter
  const int* order;
  int* counter;
  BsoParams p;
  // Y (the contracted Z blocks, nch * NYP complex per atom) in global memory, one slice per CTA,
  // when it does not fit in shared memory next to the rest (FP64 with several channels) or would
  // cost a resident CTA per SM (FP32 with several channels)
  void* yglobal;
  int g1;  // narrowest lane groups per neighbour in phase 1 (4, 6, 8 or 16) the U store allows
  int geo_cap;  // neighbours whose phase-1 geometry records are kept for phase 3 (the rest recompute)
  // outputs: B (A x nch*K) and w_ch * dB (P x 3 x nch*K); or evaluation (ev.pair != nullptr)
  T* Bout;
  T* dBout;
  DevEval<T> ev;
};

constexpr int kNW = 8;                  // warps per CTA (== kZWarps)
constexpr int kG = 16;                  // lanes per neighbour in the U/dU recursion (phase 3; a last
                                        // chunk of at most kNW neighbours takes a warp each)
constexpr int kNG = kNW * 32 / kG;      // lane groups per CTA in phase 3
constexpr int kNB = kNG;                // neighbours per phase-3 chunk (one per group)
// lanes per neighbour in the U recursion of phase 1: 16, 8, 6 or 4 per atom (16 to 64
// neighbours per pass), no narrower than the U store in shared memory allows (KernelArgs::g1)
static_assert(kNW == kZWarps, "phase-2 schedule is built for the CTA's warps");

// Shared-memory carve-up, in order (every region 16-byte aligned):
//   rec[HU]  hoff[kMaxJ+2]  rowk[NROWS]  tiles[NTILE]  rank_slot[2K]  cfull[nch*NU]
//   Y[nch*NYP] (shared Y)
//   V region (phase 1: U store of the lane groups, their f_c w_ch, c on half layers; phase 2:
//   term buffer; phase 3: vecall of a chunk)
//   W region (phase 2: CG coefficients; phase 3: recursion buffers, then the chunk's dB by rank:
//   rank 0 [cols][K], rank 1 [cols][nrank1], rank 2 [cols][nrank2])
//   Bk[nch*K]  nwt[nch*NB]  nuu[NB*4]  nidx[NB]  pacc[NB*9] (FP64)  next atom
//   sc[256] (Y-slot scales)  expand[NU]  half_diag[HU]  bk_off[K+1] (tables staged once per CTA)
//   geo[geo_cap*kGeo] (geometry records of the atom's first geo_cap neighbours)
struct SmemPlan {
  size_t rec, hoff, rowk, tiles, rslot, cfull, Y, V, W, Bk, nwt, nuu, nidx, pacc, next, sc, exp, hd, bko, geo, total;
};

__host__ __device__ inline size_t al16(size_t x) { return (x + 15) & ~(size_t)15; }

// lane groups per CTA in phase 1 for g1 lanes per neighbour (whole groups per warp)
__host__ __device__ constexpr int phase1_groups(int g1) { return kNW * (32 / g1); }

__host__ __device__ inline SmemPlan smem_plan(const DevTables& tb, int nch, int eb, bool y_in_smem, int g1 = 16,
                                              int geo_cap = 0) {
  const int ng1 = phase1_groups(g1);
  const size_t LH = tb.hoff[tb.J + 1] - tb.hoff[tb.J];
  const size_t cxb = 2 * (size_t)eb;
  const size_t recb = eb == 8 ? sizeof(RecEntry64) : sizeof(RecEntry32);
  // phase 1: U of every group's neighbour (all half layers), the groups' f_c w_ch, c so far
  const size_t v1 = (size_t)ng1 * (tb.HU + 15) + ((size_t)ng1 * nch + 1) / 2 + (size_t)nch * tb.HU;
  const size_t v2 = (size_t)tb.NZT;                                      // phase 2
  const size_t v3 = (size_t)kNB * 3 * tb.HU;                             // phase 3
  const size_t vblock = v1 > v2 ? (v1 > v3 ? v1 : v3) : (v2 > v3 ? v2 : v3);
  const size_t wrec = (size_t)kNG * 2 * LH * cxb;
  const size_t wdb = (size_t)3 * kNB * (tb.nrank[0] + tb.nrank[1] + tb.nrank[2]) * eb;
  const size_t wcg = al16((size_t)eb * tb.NCG) + (size_t)eb * 4 * tb.K;
  const size_t wblock = wrec > wdb ? (wrec > wcg ? wrec : wcg) : (wdb > wcg ? wdb : wcg);
  SmemPlan s;
  size_t o = 0;
  s.rec = o;   o = al16(o + recb * tb.HU);
  s.hoff = o;  o = al16(o + sizeof(int) * (kMaxJ + 2));
  s.rowk = o;  o = al16(o + sizeof(int16_t) * tb.NROWS);
  s.tiles = o; o = al16(o + sizeof(int) * tb.NTILE);
  s.rslot = o; o = al16(o + sizeof(int16_t) * (kRounds - 1) * tb.K);
  s.cfull = o; o = al16(o + cxb * nch * tb.NU);
  s.Y = o;     o = al16(o + (y_in_smem ? cxb * nch * tb.NYP : 0));
  s.V = o;     o = al16(o + cxb * vblock);
  s.W = o;     o = al16(o + wblock);
  s.Bk = o;    o = al16(o + (size_t)eb * nch * tb.K);
  s.nwt = o;   o = al16(o + (size_t)eb * nch * kNB);
  s.nuu = o;   o = al16(o + (size_t)eb * kNB * 4);
  s.nidx = o;  o = al16(o + sizeof(int) * kNB);
  s.pacc = o;  o = al16(o + sizeof(double) * kNB * 9);
  s.next = o;  o = al16(o + sizeof(int) * (4 + 3 * kMaxJ + 4 + kRounds));
  s.sc = o;    o = al16(o + (size_t)eb * 256);
  s.exp = o;   o = al16(o + sizeof(int16_t) * tb.NU);
  s.hd = o;    o = al16(o + tb.HU);
  s.bko = o;   o = al16(o + sizeof(int) * (tb.K + 1));
  s.geo = o;   o = al16(o + (size_t)eb * kGeo * geo_cap);
  s.total = o;
  return s;
}

// Displacement of pair q and 1/r in T (the values phase 3 uses for the stress lever arm).
template <typename T>
__device__ __forceinline__ void pair_u_rinv(const KernelArgs<T>& args, size_t q, T* x, T* rinv) {
  if constexpr (sizeof(T) == 4) {
    if (args.u32) {
      const float4 v = args.u32[q];
      x[0] = v.x;
      x[1] = v.y;
      x[2] = v.z;
      *rinv = v.w;
      return;
    }
  }
  const double* u3 = args.nbr_u + 3 * q;
  x[0] = (T)u3[0];
  x[1] = (T)u3[1];
  x[2] = (T)u3[2];
  *rinv = (T)(1.0 / sqrt(u3[0] * u3[0] + u3[1] * u3[1] + u3[2] * u3[2]));
}

// Phase 1 of one atom: c on half layers.  Lane groups of G lanes take one neighbour each
// (whole groups per warp; neighbour = pass start + group index) and write its U, all half
// layers, into the group's slot of the store Ust[group][HU], and f_c w_ch into fcw; after each
// pass chalf += sum over the groups in group order of fcw * U (the diagonal's +1 after the
// last pass).
template <typename T, int G>
__device__ __forceinline__ void phase1_c(const KernelArgs<T>& args, const typename RecEntry<T>::type* __restrict__ srec,
                                         const int* __restrict__ shoff, cx<T>* Ust, T* fcw, cx<T>* chalf,
                                         const int8_t* __restrict__ half_diag, T* sgeo, int nn, int p0, int ti, T rcut,
                                         T inv_r0, int J, int HU, int nch, int warp, int lane, int tid) {
  constexpr int NGW = 32 / G, NG = kNW * NGW;
  const int gw = lane / G, sl = lane - (lane / G) * G;
  const int grp = warp * NGW + gw;
  // group stride HS = G (mod 16): the 2G words of the groups of a warp fall on distinct banks
  const int HS = HU + ((G - HU % 16) + 16) % 16;
  cx<T>* ug = Ust + (size_t)(gw < NGW ? grp : 0) * HS;
  const int npass = (nn + NG - 1) / NG;
  for (int pass = 0; pass < npass; ++pass) {
    const int n = pass * NG + grp;
    const bool active = gw < NGW && n < nn;
    NbrGeom<T> g;
    if (active) {
      const int nb = args.nbr_idx[p0 + n];
      const int tn = args.types[nb];
      const T rin = args.p.has_rin ? args.rin[ti * args.p.ntypes + tn] : T(0);
      T x[3], rinv;
      pair_u_rinv<T>(args, (size_t)(p0 + n), x, &rinv);
      nbr_geometry<T>(x[0], x[1], x[2], rcut, inv_r0, rin, args.rin_w, &g);
      if (sl == 0) {
        ug[0] = {T(1), T(0)};
#pragma unroll
        for (int ch = 0; ch < kMaxCh; ++ch)
          if (ch < nch) fcw[grp * nch + ch] = g.fc * args.chw[ch * args.p.ntypes + tn];
        if (n < args.geo_cap) {
          T* r = sgeo + (size_t)n * kGeo;
          put_geo(g, r);
          reinterpret_cast<int*>(r + kGeoIdx)[0] = nb;
          reinterpret_cast<int*>(r + kGeoIdx)[1] = tn;
          r[kGeoU + 0] = x[0];
          r[kGeoU + 1] = x[1];
          r[kGeoU + 2] = x[2];
          r[kGeoU + 3] = rinv;
        }
      }
    }
    __syncwarp();
    for (int j = 1; j <= J; ++j) {
      const int h0 = shoff[j], ne = shoff[j + 1] - h0;
      const cx<T>* prev = ug + shoff[j - 1];
      if (active) {
        for (int e = sl; e < ne; e += G) {
          const auto r = srec[h0 + e];
          const T tzq = (T)r.tz, txq = (T)r.tx;  // tz, tx signed by q: Z = zp or conj(zp), X = conj(xp) or xp
          const T tz = fabs(tzq), tx = fabs(txq);
          const cx<T> A = {tz * g.zp.x, tzq * g.zp.y};
          const cx<T> Bc = {-txq * g.xp.y, -tx * g.xp.x};  // -i*tx*X
          cx<T> u = {T(0), T(0)};
          if (r.sz >= 0) u = cmul(A, fetch(prev, r.sz));
          if (r.sx >= 0) u = cfma(Bc, fetch(prev, r.sx), u);
          ug[h0 + e] = u;
        }
      }
      __syncwarp();
    }
    __syncthreads();  // the pass's U store complete
    const int ngact = min(NG, nn - pass * NG);
    const bool last = pass == npass - 1;
    for (int e = tid; e < nch * HU; e += kNW * 32) {
      const int ch = e / HU, h = e - ch * HU;
      cx<T> acc = pass == 0 ? cx<T>{T(0), T(0)} : chalf[e];
#pragma unroll 4
      for (int q = 0; q < ngact; ++q) {
        const T w = fcw[q * nch + ch];
        const cx<T> u = Ust[(size_t)q * HS + h];
        acc.x = fma(w, u.x, acc.x);
        acc.y = fma(w, u.y, acc.y);
      }
      if (last && half_diag[h]) acc.x += T(1);
      chalf[e] = acc;
    }
    __syncthreads();  // chalf of this pass complete; the store may be overwritten
  }
  if (npass == 0) {  // no neighbours: c is the identity
    for (int e = tid; e < nch * HU; e += kNW * 32) chalf[e] = {half_diag[e % HU] ? T(1) : T(0), T(0)};
    __syncthreads();
  }
}

// kYShared: Y lives in shared memory (one channel); otherwise in the per-CTA global slice
// args.yglobal (several channels), a separate instantiation so that the shared-memory
// variant keeps shared-memory addressing.
// kCT: columns (neighbour, component) per register tile of the dB contraction (autotuned).
template <typename T, bool kYShared, int kCT>
__global__ void __launch_bounds__(kNW * 32, sizeof(T) == 4 ? 2 : 1) k_bso4(KernelArgs<T> args, int A) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  using Rec = typename RecEntry<T>::type;
  const DevTables& tb = args.tb;
  const int J = tb.J, NU = tb.NU, HU = tb.HU, K = tb.K, NYP = tb.NYP;
  const int nch = args.p.nch;
  const int nchK = nch * K;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  constexpr int nth = kNW * 32;
  const int LH = tb.hoff[J + 1] - tb.hoff[J];  // largest half layer
  const SmemPlan sp = smem_plan(tb, nch, (int)sizeof(T), kYShared, args.g1, args.geo_cap);

  Rec* srec = reinterpret_cast<Rec*>(smem_raw + sp.rec);
  int* shoff = reinterpret_cast<int*>(smem_raw + sp.hoff);
  int16_t* srowk = reinterpret_cast<int16_t*>(smem_raw + sp.rowk);
  int* stile = reinterpret_cast<int*>(smem_raw + sp.tiles);
  int16_t* srslot = reinterpret_cast<int16_t*>(smem_raw + sp.rslot);
  cx<T>* cfull = reinterpret_cast<cx<T>*>(smem_raw + sp.cfull);
  cx<T>* Y = kYShared ? reinterpret_cast<cx<T>*>(smem_raw + sp.Y)
                      : reinterpret_cast<cx<T>*>(args.yglobal) + (size_t)blockIdx.x * nch * NYP;
  cx<T>* V = reinterpret_cast<cx<T>*>(smem_raw + sp.V);
  // phase 1 in V: the U store of the groups (as many as args.g1 gives), their f_c w_ch, c
  cx<T>* p1u = V;
  T* p1w = reinterpret_cast<T*>(V + (size_t)phase1_groups(args.g1) * (HU + 15));
  cx<T>* p1c = V + (size_t)phase1_groups(args.g1) * (HU + 15) + ((size_t)phase1_groups(args.g1) * nch + 1) / 2;
  unsigned char* W = smem_raw + sp.W;
  T* scg = reinterpret_cast<T*>(W);  // phase 2 only (restaged per atom)
  T* Bk = reinterpret_cast<T*>(smem_raw + sp.Bk);
  T* nwt = reinterpret_cast<T*>(smem_raw + sp.nwt);
  T* nuu = reinterpret_cast<T*>(smem_raw + sp.nuu);
  int* nidx = reinterpret_cast<int*>(smem_raw + sp.nidx);
  double* pacc = reinterpret_cast<double*>(smem_raw + sp.pacc);
  int* snext = reinterpret_cast<int*>(smem_raw + sp.next);
  T* sgeo = reinterpret_cast<T*>(smem_raw + sp.geo);
  T* ssc = reinterpret_cast<T*>(smem_raw + sp.sc);  // ssc[16 n + d] = n / d, the Y-slot scales

  // tables, once per CTA; Y zeroed once (its padding rows are never written)
  for (int e = tid; e < HU; e += nth) srec[e] = args.rec[e];
  for (int e = tid; e < kMaxJ + 2; e += nth) shoff[e] = tb.hoff[e];
  int* sMp = snext + 4;
  int* syoff = sMp + (kMaxJ + 1);
  int* srko = syoff + (kMaxJ + 1);
  int* snr = srko + (kMaxJ + 2);
  for (int e = tid; e < kMaxJ + 1; e += nth) { sMp[e] = tb.Mp[e]; syoff[e] = tb.yoff[e]; }
  for (int e = tid; e < kMaxJ + 2; e += nth) srko[e] = tb.rowk_off[e];
  for (int e = tid; e < kRounds; e += nth) snr[e] = tb.nrank[e];
  for (int e = tid; e < tb.NROWS; e += nth) srowk[e] = tb.rowk[e];
  for (int e = tid; e < tb.NTILE; e += nth) stile[e] = tb.tiles[e];
  for (int e = tid; e < (kRounds - 1) * K; e += nth) srslot[e] = tb.rank_slot[e];
  for (int e = tid; e < nch * NYP; e += nth) Y[e] = {T(0), T(0)};
  for (int e = tid; e < 256; e += nth) ssc[e] = (e & 15) ? (T)(e >> 4) / (T)(e & 15) : T(0);
  int16_t* sexp = reinterpret_cast<int16_t*>(smem_raw + sp.exp);
  int8_t* shd = reinterpret_cast<int8_t*>(smem_raw + sp.hd);
  int* sbko = reinterpret_cast<int*>(smem_raw + sp.bko);
  for (int e = tid; e < NU; e += nth) sexp[e] = tb.expand[e];
  for (int e = tid; e < HU; e += nth) shd[e] = tb.half_diag[e];
  for (int e = tid; e <= K; e += nth) sbko[e] = tb.bk_off[e];
  const int zr0 = tb.zitem_off[warp], zr1 = tb.zitem_off[warp + 1];  // this warp's Z rounds

  const T rcut = (T)args.p.rcut, inv_r0 = (T)args.p.inv_r0;
  const bool eval = args.ev.pair != nullptr;
  const bool need_d = eval || args.dBout != nullptr;

  // thread 0 takes the next queue position while the current atom runs; it publishes it at the
  // top of the loop, after at least one barrier that follows every thread's read of the last one
  int nxt = 0;
  if (tid == 0) nxt = atomicAdd(args.counter, 1);
  for (;;) {
    if (tid == 0) snext[0] = nxt;
    __syncthreads();  // also orders the table staging and the previous atom's last reads
    const int qi = snext[0];
    if (qi >= A) break;
    if (tid == 0) nxt = atomicAdd(args.counter, 1);
    const int atom = args.order ? args.order[qi] : qi;
    const int s = args.atom_struct[atom];
    const int ti = args.types[atom];
    const int p0 = args.nbr_off[atom];
    const int nn = args.nbr_off[atom + 1] - p0;

    // ---------------- phase 1: c^j on half layers, one lane group per neighbour ------------
    // (the CG coefficients of phase 2 are copied into W meanwhile by 16-byte asynchronous
    // copies, the device table being padded to whole chunks; W held the previous atom's dB)
    {
      const int n16 = (tb.NCG * (int)sizeof(T) + 15) >> 4;
      const char* src = reinterpret_cast<const char*>(args.cg);
      const unsigned dst = (unsigned)__cvta_generic_to_shared(scg);
      for (int e = tid; e < n16; e += nth)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(dst + 16u * e), "l"(src + 16 * (size_t)e) : "memory");
      asm volatile("cp.async.commit_group;\n" ::: "memory");
    }
    {
      // lanes per neighbour: the widest group that needs no more passes than the narrowest
      // allowed one (args.g1)
      const int npmin = (nn + phase1_groups(args.g1) - 1) / phase1_groups(args.g1);
      int g1 = args.g1;
      for (int cand : {16, 8, 6})
        if (cand > g1 && (nn + phase1_groups(cand) - 1) / phase1_groups(cand) <= npmin) {
          g1 = cand;
          break;
        }
      switch (g1) {
        case 16: phase1_c<T, 16>(args, srec, shoff, p1u, p1w, p1c, shd, sgeo, nn, p0, ti, rcut, inv_r0, J, HU, nch, warp, lane, tid); break;
        case 8: phase1_c<T, 8>(args, srec, shoff, p1u, p1w, p1c, shd, sgeo, nn, p0, ti, rcut, inv_r0, J, HU, nch, warp, lane, tid); break;
        case 6: phase1_c<T, 6>(args, srec, shoff, p1u, p1w, p1c, shd, sgeo, nn, p0, ti, rcut, inv_r0, J, HU, nch, warp, lane, tid); break;
        default: phase1_c<T, 4>(args, srec, shoff, p1u, p1w, p1c, shd, sgeo, nn, p0, ti, rcut, inv_r0, J, HU, nch, warp, lane, tid); break;
      }
    }
    // expansion to full layers
    for (int e = tid; e < nch * NU; e += nth) {
      const int ch = e / NU, f = e - ch * NU;
      cfull[e] = fetch(p1c + ch * HU, sexp[f]);
    }
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    __syncthreads();

    // ---------------- phase 2: Z terms -> term buffer -> Y slots and B ----------------------
    // lane l of a round computes one Z term; the 32 terms of a round share their inner extent nb
    // and have outer extents na in descending order, so the warp diverges only at the end of
    // the a loop.  Entries are prefetched two rounds ahead.
    cx<T>* tbuf = V;
    for (int ch = 0; ch < nch; ++ch) {
      const cx<T>* cc = cfull + ch * NU;
      {
        const int r0 = zr0, r1 = zr1;
        const uint4* zit = reinterpret_cast<const uint4*>(tb.zitems);
        uint4 n1 = make_uint4(0u, 0u, 0u, 0u), n2 = n1;
        if (r0 < r1) n1 = __ldg(zit + (size_t)r0 * 32 + lane);
        if (r0 + 1 < r1) n2 = __ldg(zit + (size_t)(r0 + 1) * 32 + lane);
        for (int r = r0; r < r1; ++r) {
          const uint4 zi = n1;
          n1 = n2;
          if (r + 2 < r1) n2 = __ldg(zit + (size_t)(r + 2) * 32 + lane);
          cx<T> zs;
          switch ((zi.z >> 8) & 0xFF) {  // nb, uniform over the round
            case 1: zs = zterm<1, T>(cc, scg, zi); break;
            case 2: zs = zterm<2, T>(cc, scg, zi); break;
            case 3: zs = zterm<3, T>(cc, scg, zi); break;
            case 4: zs = zterm<4, T>(cc, scg, zi); break;
            case 5: zs = zterm<5, T>(cc, scg, zi); break;
            case 6: zs = zterm<6, T>(cc, scg, zi); break;
            case 7: zs = zterm<7, T>(cc, scg, zi); break;
            case 8: zs = zterm<8, T>(cc, scg, zi); break;
            case 9: zs = zterm<9, T>(cc, scg, zi); break;
            case 10: zs = zterm<10, T>(cc, scg, zi); break;
            default: zs = zterm<11, T>(cc, scg, zi); break;
          }
          if ((zi.w & 0xFFFF) != kNoTerm) tbuf[zi.w & 0xFFFF] = zs;
        }
      }
      __syncthreads();
      cx<T>* Yc = Y + (size_t)ch * NYP;
      // slot entries (16 bytes) prefetched one iteration ahead
      uint4 nse = make_uint4(0u, 0u, 0u, 0u);
      if (tid < tb.NS) nse = __ldg(reinterpret_cast<const uint4*>(tb.slots) + tid);
      for (int e = tid; e < tb.NS; e += nth) {
        // the slot's 16 bytes: x = term0 | term1 << 16, y = term2 | ypos << 16,
        // z = nterm | wgt << 8 | snum0 << 16 | snum1 << 24, w = snum2 | sden0 << 8 | sden1 << 16 | sden2 << 24
        const uint4 se = nse;
        if (e + nth < tb.NS) nse = __ldg(reinterpret_cast<const uint4*>(tb.slots) + e + nth);
        const int nterm = se.z & 0xFF;
        const int terms[3] = {(int)(se.x & 0xFFFF), (int)(se.x >> 16), (int)(se.y & 0xFFFF)};
        const int snum[3] = {(int)((se.z >> 16) & 0xFF), (int)(se.z >> 24), (int)(se.w & 0xFF)};
        const int sden[3] = {(int)((se.w >> 8) & 0xFF), (int)((se.w >> 16) & 0xFF), (int)(se.w >> 24)};
        cx<T> v = {T(0), T(0)};
#pragma unroll
        for (int t = 0; t < 3; ++t) {  // nterm <= 3
          if (t < nterm) {
            const T sc = ssc[snum[t] * 16 + sden[t]];
            const cx<T> z = tbuf[terms[t]];
            v.x = fma(sc, z.x, v.x);
            v.y = fma(sc, z.y, v.y);
          }
        }
        const T wgt = (T)((se.z >> 8) & 0xFF);
        Yc[se.y >> 16] = {wgt * v.x, wgt * v.y};
      }
      // B_k in four fixed quarters of its items (threads from the top, which have fewer Y slots),
      // then ((q0 + q1) + q2) + q3
      T* bpart = reinterpret_cast<T*>(W + al16((size_t)tb.NCG * sizeof(T)));  // [4][K]
      for (int t2 = nth - 1 - tid; t2 < 4 * K; t2 += nth) {
        const int k = t2 >> 2, sub = t2 & 3;
        const int i0 = sbko[k], i1 = sbko[k + 1];
        const int per = (i1 - i0 + 3) >> 2;
        const int a0 = i0 + sub * per, a1 = min(i1, a0 + per);
        T b = T(0);
        for (int i0 = a0; i0 < a1; i0 += 4) {  // items loaded four at a time
          uint2 q[4];
#pragma unroll
          for (int u = 0; u < 4; ++u)
            q[u] = i0 + u < a1 ? __ldg(reinterpret_cast<const uint2*>(tb.bk_items) + i0 + u) : make_uint2(0u, 0u);
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            if (i0 + u < a1) {
              // x = term | ufull << 16, y = wgt | pad << 8
              const cx<T> cv = cc[q[u].x >> 16];
              const cx<T> z = tbuf[q[u].x & 0xFFFF];
              b = fma((T)(q[u].y & 0xFF), cv.x * z.x + cv.y * z.y, b);  // w * Re(conj(c) ZA)
            }
          }
        }
        bpart[sub * K + k] = b;
      }
      __syncthreads();
      for (int k = tid; k < K; k += nth)
        Bk[ch * K + k] = (nn == 0) ? T(0) : ((bpart[k] + bpart[K + k]) + bpart[2 * K + k]) + bpart[3 * K + k];
      __syncthreads();
    }
    if (args.Bout)
      for (int e = tid; e < nchK; e += nth) args.Bout[(size_t)atom * nchK + e] = Bk[e];
    if (args.ev.Eatom && warp == 0) {
      // linear model: energy of the atom, w0 + w_lin . B_a (FP64, fixed lane order)
      double e = 0.0;
      if (nn > 0)
        for (int k = lane; k < nchK; k += 32) e += args.ev.wlin[k] * (double)Bk[k];
      for (int o = 16; o > 0; o >>= 1) e += __shfl_xor_sync(0xffffffffu, e, o);
      if (lane == 0) args.ev.Eatom[atom] = e + args.ev.w0;
    }
    if (!need_d || nn == 0) continue;

    // ---------------- phase 3: dB per neighbour chunk (kNB neighbours, the last one the rest) -
    cx<T>* ubuf3 = reinterpret_cast<cx<T>*>(W);
    T* dBs = reinterpret_cast<T*>(W);  // 3*kNB*K [col][k], after the recursion of the chunk
    for (int base = 0; base < nn; base += kNB) {
      const int nb_here = min(kNB, nn - base);
      // lanes per neighbour in the recursion: a whole warp when the chunk (the last one) has no
      // more neighbours than warps, else kG
      const bool wide = nb_here <= kNW;
      const int grp = wide ? warp : tid / kG, sl = wide ? lane : tid % kG;
      {
        const int n = grp;  // one neighbour per group
        const bool active = n < nb_here;
        NbrGeom<T> g;
        if (active) {
          const size_t q = (size_t)(p0 + base + n);
          // neighbour index, type, displacement and 1/r: from phase 1's record (no global loads
          // in front of the recursion), else from the lists
          int nbi, tn;
          T x[3], rinv;
          if (base + n < args.geo_cap) {
            const T* r = sgeo + (size_t)(base + n) * kGeo;
            get_geo(r, &g);
            nbi = reinterpret_cast<const int*>(r + kGeoIdx)[0];
            tn = reinterpret_cast<const int*>(r + kGeoIdx)[1];
            x[0] = r[kGeoU + 0];
            x[1] = r[kGeoU + 1];
            x[2] = r[kGeoU + 2];
            rinv = r[kGeoU + 3];
          } else {
            nbi = args.nbr_idx[q];
            tn = args.types[nbi];
            const T rin = args.p.has_rin ? args.rin[ti * args.p.ntypes + tn] : T(0);
            pair_u_rinv<T>(args, q, x, &rinv);
            nbr_geometry<T>(x[0], x[1], x[2], rcut, inv_r0, rin, args.rin_w, &g);
          }
          if (sl == 0) {
            for (int ch = 0; ch < nch; ++ch) nwt[ch * kNB + n] = args.chw[ch * args.p.ntypes + tn];
            nidx[n] = nbi;
            // stress lever arm: x_n - x_i (small box) or sign_big*(x_i - x_n) (large box)
            const T sgn = args.small[s] ? T(1) : (T)(-args.p.sign_big);
            nuu[n * 4 + 0] = sgn * x[0];
            nuu[n * 4 + 1] = sgn * x[1];
            nuu[n * 4 + 2] = sgn * x[2];
            nuu[n * 4 + 3] = rinv;
          }
        }
        if (eval && sl < 9) pacc[min(n, kNB - 1) * 9 + sl] = 0.0;
        if (wide)
          group_recursion<T, 32>(g, srec, J, shoff, ubuf3 + (size_t)grp * 2 * LH, LH,
                                 V + (size_t)min(n, kNB - 1) * 3 * HU, HU, sl, active);
        else
          group_recursion<T, kG>(g, srec, J, shoff, ubuf3 + (size_t)grp * 2 * LH, LH,
                                 V + (size_t)min(n, kNB - 1) * 3 * HU, HU, sl, active);
      }
      __syncthreads();  // V of the chunk complete; the recursion buffers become dBs
      const int ncols = 3 * nb_here;
      const int ncolt = (ncols + kCT - 1) / kCT;
      for (int ch = 0; ch < nch; ++ch) {
        const cx<T>* Yc = Y + (size_t)ch * NYP;
        // register-tiled contraction, item = (row tile of layer j, column tile), heaviest
        // layers first; each row's result goes to the buffer of its rank, where it is the
        // triple's only row, so no two items write the same element
        T* dB1 = dBs + (size_t)3 * kNB * K;
        T* dB2 = dB1 + (size_t)3 * kNB * tb.nrank[1];
        const int nitem = tb.NTILE * ncolt;
        for (int k = 0; k * nth < nitem; ++k) {
          // rounds alternate direction, so the threads with the heaviest items of one round take
          // the lightest of the next (items are ordered heaviest layers first)
          const int it = (k & 1) ? (k + 1) * nth - 1 - tid : k * nth + tid;
          if (it >= nitem) continue;
          const int tix = it / ncolt;
          const int tile = stile[tix];
          const int ct = it - tix * ncolt;
          const int j = tile >> 8, rt = tile & 255;
          const int Mp = sMp[j], H = shoff[j + 1] - shoff[j];
          const cx<T>* Yp = Yc + syoff[j] + rt * kRowTile;
          // columns ct, ct + ncolt, ...: lanes of a warp read consecutive columns of V, whose
          // odd stride HU spreads them over distinct shared-memory banks
          const cx<T>* Vp[kCT];
#pragma unroll
          for (int c = 0; c < kCT; ++c) {
            const int col = min(ct + c * ncolt, ncols - 1);
            Vp[c] = V + (size_t)col * HU + shoff[j];  // col = n*3 + a -> V[n][a][.]
          }
          T acc[kRowTile][kCT];
#pragma unroll
          for (int r = 0; r < kRowTile; ++r)
#pragma unroll
            for (int c = 0; c < kCT; ++c) acc[r][c] = T(0);
#pragma unroll 4
          for (int e = 0; e < H; ++e) {
            cx<T> y[kRowTile], v[kCT];
#pragma unroll
            for (int r = 0; r < kRowTile; ++r) y[r] = Yp[e * Mp + r];
#pragma unroll
            for (int c = 0; c < kCT; ++c) v[c] = Vp[c][e];
#pragma unroll
            for (int r = 0; r < kRowTile; ++r)
#pragma unroll
              for (int c = 0; c < kCT; ++c) acc[r][c] = fma(y[r].x, v[c].x, fma(-y[r].y, v[c].y, acc[r][c]));
          }
#pragma unroll
          for (int r = 0; r < kRowTile; ++r) {
            const int code = srowk[srko[j] + rt * kRowTile + r];
            if (code < 0) continue;
            const int rank = code >> kRankShift, idx = code & ((1 << kRankShift) - 1);
            T* base = rank == 0 ? dBs : (rank == 1 ? dB1 : dB2);
            const int ld = snr[rank];
#pragma unroll
            for (int c = 0; c < kCT; ++c) {
              const int col = ct + c * ncolt;
              if (col < ncols) base[(size_t)col * ld + idx] = acc[r][c];
            }
          }
        }
        __syncthreads();
        // dB = (rank 0 + rank 1) + rank 2 of element e = col * K + k
        // element (col, k): lanes take the components k, warps the columns, so each lane looks
        // up its k's rank slots once and a warp's stores are contiguous
        const int nr1 = tb.nrank[1], nr2 = tb.nrank[2];
        if (eval) {
          for (int k = lane; k < K; k += 32) {
            const int s1 = srslot[k * (kRounds - 1)], s2 = srslot[k * (kRounds - 1) + 1];
            for (int col = warp; col < ncols; col += kNW) {
              T v = dBs[col * K + k];
              if (s1 >= 0) v += dB1[col * nr1 + s1];
              if (s2 >= 0) v += dB2[col * nr2 + s2];
              dBs[col * K + k] = v;  // in place: own element
            }
          }
          __syncthreads();
          // forces and stress with the effective weights: the centre's for the forces, the
          // neighbour's for the stress (the neighbour's B in the quadratic stress rows,
          // mld_stress.F90:580-603); sums per (neighbour, component) in T, per-pair totals in
          // FP64 accumulated over the channels in channel order
          const T* bc = args.ev.beta + (args.ev.beta_per_atom ? (size_t)atom * nchK : 0) + ch * K;
          for (int it = tid; it < 3 * nb_here; it += nth) {
            const int n = it / 3, a = it - 3 * n;
            const T* d = dBs + (size_t)(n * 3 + a) * K;
            T f = T(0);
            for (int k = 0; k < K; ++k) f = fma(d[k], bc[k], f);
            const T wn = nwt[ch * kNB + n];
            double* pa = pacc + n * 9;
            pa[a] += (double)(f * wn);
            T gsum = f;
            if (args.ev.beta_per_atom) {
              const T* bn = args.ev.beta + (size_t)nidx[n] * nchK + ch * K;
              gsum = T(0);
              for (int k = 0; k < K; ++k) gsum = fma(d[k], bn[k], gsum);
            }
            const double gv = (double)(gsum * wn) * (double)nuu[n * 4 + 3];
            const double ux = nuu[n * 4 + 0], uy = nuu[n * 4 + 1], uz = nuu[n * 4 + 2];
            if (a == 0) {  // xx, xz, xy
              pa[3] += gv * ux;
              pa[7] += gv * uz;
              pa[8] += gv * uy;
            } else if (a == 1) {  // yy, yz
              pa[4] += gv * uy;
              pa[6] += gv * uz;
            } else {  // zz
              pa[5] += gv * uz;
            }
          }
        } else {
          // w_ch * dB of every pair of the chunk; one channel's columns per pass
          T* out = args.dBout + (size_t)(p0 + base) * 3 * nchK + ch * K;
          for (int k = lane; k < K; k += 32) {
            const int s1 = srslot[k * (kRounds - 1)], s2 = srslot[k * (kRounds - 1) + 1];
            for (int col = warp; col < ncols; col += kNW) {  // col = n*3 + a
              T v = dBs[col * K + k];
              if (s1 >= 0) v += dB1[col * nr1 + s1];
              if (s2 >= 0) v += dB2[col * nr2 + s2];
              out[(size_t)col * nchK + k] = v * nwt[ch * kNB + col / 3];
            }
          }
        }
        __syncthreads();
      }
      if (eval) {
        for (int e = tid; e < nb_here * 9; e += nth) args.ev.pair[(size_t)(p0 + base) * 9 + e] = pacc[e];
        __syncthreads();
      }
    }
  }
}

static int max_optin_smem() {
  static int v = 0;
  if (!v) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  }
  return v;
}

// Y in shared memory unless it does not fit or costs a resident CTA per SM (several channels)
static bool y_shared(const DevTables& tb, int nch, int eb) {
  const size_t ss = smem_plan(tb, nch, eb, true).total, sg = smem_plan(tb, nch, eb, false).total;
  const size_t per_sm = 228 * 1024;
  return ss <= (size_t)max_optin_smem() && per_sm / (ss + 1024) >= per_sm / (sg + 1024);
}

size_t bso4_y_scratch_bytes(const DevTables& tb, int nch, int eb, int max_ctas, bool only_if_required) {
  const bool fits = smem_plan(tb, nch, eb, true).total <= (size_t)max_optin_smem();
  if (fits && (only_if_required || y_shared(tb, nch, eb))) return 0;
  return (size_t)max_ctas * nch * tb.NYP * 2 * eb;
}

template <typename T>
cudaError_t launch_bso4(const DevTables& tb, const DevBatch& b, const BsoParams& p, T* Bout, T* dBout,
                        const DevEval<T>* ev, const int* order, int* counter, cudaStream_t st, void* yscratch,
                        size_t yscratch_bytes, const Bso4Launch* shape) {
  const Bso4Launch sh = shape ? *shape : Bso4Launch{};
  if (b.A == 0) return cudaSuccess;
  if (!counter) return cudaErrorInvalidValue;
  KernelArgs<T> a{};
  a.tb = tb;
  if constexpr (sizeof(T) == 8) {
    a.rec = reinterpret_cast<const RecEntry64*>(tb.rec64);
    a.cg = reinterpret_cast<const T*>(tb.cg64);
  } else {
    a.rec = reinterpret_cast<const RecEntry32*>(tb.rec32);
    a.cg = reinterpret_cast<const T*>(tb.cg32);
  }
  a.atom_struct = b.atom_struct;
  a.types = b.types;
  a.small = b.small;
  a.nbr_off = b.nbr_off;
  a.nbr_idx = b.nbr_idx;
  a.nbr_u = b.nbr_u;
  a.u32 = sizeof(T) == 4 ? b.nbr_u32 : nullptr;
  for (int e = 0; e < kMaxCh * kMaxTypes; ++e) a.chw[e] = (T)p.chw[e];
  for (int e = 0; e < kMaxTypes * kMaxTypes; ++e) a.rin[e] = (T)p.rin[e];
  a.rin_w = (T)p.rin_width;
  a.order = sh.sorted_queue ? order : nullptr;
  a.counter = counter;
  a.p = p;
  a.Bout = Bout;
  a.dBout = dBout;
  if (ev) a.ev = *ev;
  if (a.ev.pair && dBout) return cudaErrorInvalidValue;
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const size_t per_sm = 228 * 1024;
  // Y in shared memory when it fits, unless it costs a resident CTA per SM and the scratch holds
  // a global slice for every CTA of the shape without it (several channels in FP32)
  bool y_in_smem = smem_plan(tb, p.nch, sizeof(T), true).total <= (size_t)max_optin_smem();
  if (y_in_smem && yscratch && !y_shared(tb, p.nch, (int)sizeof(T))) {
    const size_t sg = smem_plan(tb, p.nch, sizeof(T), false).total;
    const long long ctas = std::min<long long>((long long)b.A, (long long)nsm * (long long)(per_sm / (sg + 1024)));
    if ((long long)(yscratch_bytes / ((size_t)p.nch * tb.NYP * 2 * sizeof(T))) >= ctas) y_in_smem = false;
  }
  // the narrowest phase-1 groups (most neighbours per pass) whose U store fits without costing
  // a resident CTA per SM; each atom then takes the widest groups that need no more passes
  const size_t s16 = smem_plan(tb, p.nch, sizeof(T), y_in_smem, 16).total;
  a.g1 = 16;
  size_t smem = s16;
  for (int g1 : {4, 6, 8}) {
    const size_t sg = smem_plan(tb, p.nch, sizeof(T), y_in_smem, g1).total;
    if (sg <= (size_t)max_optin_smem() && per_sm / (sg + 1024) >= per_sm / (s16 + 1024)) {
      a.g1 = g1;
      smem = sg;
      break;
    }
  }
  if (smem > (size_t)max_optin_smem()) return cudaErrorInvalidConfiguration;
  // geometry records for the first geo_cap neighbours of an atom (at most 128), as many as keep
  // the resident CTAs per SM as they are.  The count depends on the configuration only, not on
  // the batch, so that an atom's results do not depend on the batch it is evaluated in.
  a.geo_cap = 0;
  for (int cap = 128; cap > 0; cap -= 8) {
    const size_t sc = smem_plan(tb, p.nch, sizeof(T), y_in_smem, a.g1, cap).total;
    if (sc <= (size_t)max_optin_smem() && per_sm / (sc + 1024) >= per_sm / (smem + 1024)) {
      a.geo_cap = cap;
      smem = sc;
      break;
    }
  }
  a.yglobal = nullptr;
  auto kern = sh.col_tile == 2 ? (y_in_smem ? k_bso4<T, true, 2> : k_bso4<T, false, 2>)
                               : (y_in_smem ? k_bso4<T, true, 4> : k_bso4<T, false, 4>);
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int occ = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, kNW * 32, smem);
  if (e != cudaSuccess) return e;
  if (occ < 1) return cudaErrorInvalidConfiguration;
  if (sh.ctas_per_sm > 0) occ = std::min(occ, sh.ctas_per_sm);
  long long grid = std::min<long long>((long long)b.A, (long long)nsm * occ);
  if (!y_in_smem) {
    // one Y slice per persistent CTA
    const size_t per_cta = (size_t)p.nch * tb.NYP * 2 * sizeof(T);
    const long long fit = yscratch ? (long long)(yscratch_bytes / per_cta) : 0;
    grid = std::min(grid, fit);
    if (grid < 1) return cudaErrorInvalidValue;  // Y scratch required and not given
    a.yglobal = yscratch;
  }
  e = cudaMemsetAsync(counter, 0, sizeof(int), st);
  if (e != cudaSuccess) return e;
  kern<<<(unsigned)grid, kNW * 32, smem, st>>>(a, b.A);
  return cudaGetLastError();
}

template cudaError_t launch_bso4<double>(const DevTables&, const DevBatch&, const BsoParams&, double*, double*,
                                         const DevEval<double>*, const int*, int*, cudaStream_t, void*, size_t,
                                         const Bso4Launch*);
template cudaError_t launch_bso4<float>(const DevTables&, const DevBatch&, const BsoParams&, float*, float*,
                                        const DevEval<float>*, const int*, int*, cudaStream_t, void*, size_t,
                                        const Bso4Launch*);

}  // namespace mld
