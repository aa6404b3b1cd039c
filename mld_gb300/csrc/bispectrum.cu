// Fused bispectrum-SO(4) descriptor + design-row kernel (one CTA per centre atom).
//
// Per atom i with neighbours n (u_n = x_n - x_i, r_n < r_cut):
//   phase 1  c^j(p,q) = delta_pq + sum_n w_ch(type_n) f_c(r_n) U^j_pq(u_n)           (compute_bispectrum_so4.F90:288-439)
//   phase 2  Z blocks ZA/ZB/ZC by Clebsch-Gordan contraction of c, merged per (k, layer) into Y,
//            B_k = Re sum conj(c^l) ZA_k                                               (:1014-1143, :469-560)
//   phase 3  per chunk of neighbours: U/dU recursion -> vecall V = conj(d(f_c U)/du)  (angular_functions.f90:41-273),
//            dB_k/du_n = w_ch(type_n) Re sum Y V (register-tiled per layer)           (:469-717, descriptors.F90:298-302)
//            scattered straight into the energy / force / stress design rows           (mld_energy.F90:91-117,
//            mld_forces.F90:222-263, mld_stress.F90:272-756)
// Only half of every layer is computed (X(-p,-q) = (-1)^((p-q)/2) conj X(p,q) for U, c, Z, V);
// full-layer sums fold into weighted sums over the half.  The layer recursions run on lane
// groups (8 lanes per neighbour for c, 16 for U+dU), phase 2 follows a host-balanced per-thread
// schedule.  T = double (plain FP64 method) or float (mixed method: FP32 descriptors).
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
__device__ __forceinline__ cx<T> zterm(const cx<T>* __restrict__ cc, const T* __restrict__ cgs, const ZItem& zi) {
  T c2[NB];
#pragma unroll
  for (int b = 0; b < NB; ++b) c2[b] = cgs[zi.cg2 + b];
  cx<T> zs = {T(0), T(0)};
  int i1a = zi.i1, i2a = zi.i2;
  for (int a = 0; a < zi.na; ++a) {
    const T c1 = cgs[zi.cg1 + a];
    cx<T> part = {T(0), T(0)};
#pragma unroll
    for (int b = 0; b < NB; ++b) {
      const cx<T> pr = cmul(cc[i1a + b], cc[i2a - b]);
      part.x = fma(c2[b], pr.x, part.x);
      part.y = fma(c2[b], pr.y, part.y);
    }
    zs.x = fma(c1, part.x, zs.x);
    zs.y = fma(c1, part.y, zs.y);
    i1a += zi.s1;
    i2a -= zi.s2;
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

template <typename T>
struct NbrGeom {
  cx<T> zp, zm, xp, xm;
  cx<T> dzp[3], dzm[3], dxp[3], dxm[3];
  T fc, dfr[3];  // fc and dfc * u_a / r
};

// angular_functions.f90:66-107 (the geometric set-up of spherical_4d) and the cutoff of
// compute_bispectrum_so4.F90:337-377 (type-2 cosine outer cut times (1 - inner type-3 cut)).
template <typename T>
__device__ void nbr_geometry(const double* u3, T rcut, T inv_r0, double rin, double rin_w, NbrGeom<T>* g) {
  const T PI = (T)3.14159265358979323846;
  T x0 = (T)u3[0], x1 = (T)u3[1], x2 = (T)u3[2];
  T rr = sqrt(x0 * x0 + x1 * x1 + x2 * x2);
  T r0 = rcut / inv_r0;
  T th0 = rr / r0;
  T s, c;
  if constexpr (sizeof(T) == 8) sincos(th0, &s, &c);
  else sincosf(th0, &s, &c);
  T sin_i = T(1) / s, tan_i = c / s;
  T l0 = rr * sin_i, l0i = T(1) / l0, z0 = rr * tan_i;
  g->zp = {z0 * l0i, x2 * l0i};
  g->zm = {z0 * l0i, -x2 * l0i};
  g->xp = {x0 * l0i, x1 * l0i};
  g->xm = {x0 * l0i, -x1 * l0i};
  T rinv = T(1) / rr;
  T drr[3] = {x0 * rinv, x1 * rinv, x2 * rinv};
  T dz = tan_i - th0 * sin_i * sin_i;
  T dil0 = (c / r0 - l0i) * rinv;
  for (int a = 0; a < 3; ++a) {
    T base = dz * l0i * drr[a];
    g->dzp[a] = {z0 * dil0 * drr[a] + base, x2 * dil0 * drr[a]};
    g->dzm[a] = {z0 * dil0 * drr[a] + base, -x2 * dil0 * drr[a]};
    g->dxp[a] = {x0 * dil0 * drr[a], x1 * dil0 * drr[a]};
    g->dxm[a] = {x0 * dil0 * drr[a], -x1 * dil0 * drr[a]};
  }
  g->dzp[2].y += l0i;
  g->dzm[2].y -= l0i;
  g->dxp[0].x += l0i;
  g->dxp[1].y += l0i;
  g->dxm[0].x += l0i;
  g->dxm[1].y -= l0i;
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
  if (rin > 0.0) {
    T rc2 = (T)(rin + rin_w), w = (T)rin_w;
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
  for (int a = 0; a < 3; ++a) g->dfr[a] = dfc * drr[a];
}

// Layer recursion of one neighbour by a group of G lanes (sl = lane within the group) on half
// layers.  WITH_DU: U and dU, vecall written to V[a*HU + h] (dU of layer j-1 stays raw in V
// until layer j is formed, then is converted).  Otherwise U only, f_c*w_ch*U added atomically to
// cpart[ch*HU + h] (the groups of a warp share cpart).  Every group of the warp calls this with
// the same J so the warp-wide __syncwarp calls line up; inactive groups pass active = false.
template <typename T, int G, bool WITH_DU>
__device__ void group_recursion(const NbrGeom<T>& g, const typename RecEntry<T>::type* __restrict__ rec, int J,
                                const int* hoff, cx<T>* ubuf, int LH, cx<T>* V, cx<T>* cpart, const T* wch, int nch,
                                int HU, int sl, bool active, bool private_part = false) {
  cx<T>* prev = ubuf;
  cx<T>* cur = ubuf + LH;
  if (active && sl == 0) {
    prev[0] = {T(1), T(0)};
    if constexpr (WITH_DU) {
      for (int a = 0; a < 3; ++a) V[a * HU] = {T(0), T(0)};
    } else {
      for (int ch = 0; ch < nch; ++ch) {
        if (private_part) cpart[ch * HU].x += g.fc * wch[ch];
        else atomicAdd(&cpart[ch * HU].x, g.fc * wch[ch]);
      }
    }
  }
  __syncwarp();
  for (int j = 1; j <= J; ++j) {
    const int h0 = hoff[j], ne = hoff[j + 1] - h0;
    const int pbase = hoff[j - 1];
    if (active) {
      for (int e = sl; e < ne; e += G) {
        const int idx = h0 + e;
        const auto r = rec[idx];
        const T tz = (T)r.tz, tx = (T)r.tx;
        const int sz = r.sz, sx = r.sx;
        const bool qn = r.qneg != 0;
        const cx<T> Z = qn ? g.zp : g.zm;
        const cx<T> X = qn ? g.xm : g.xp;
        const cx<T> A = {tz * Z.x, tz * Z.y};
        const cx<T> Bc = {tx * X.y, -tx * X.x};  // -i*tx*X
        cx<T> u = {T(0), T(0)};
        if constexpr (WITH_DU) {
          cx<T> du[3] = {{T(0), T(0)}, {T(0), T(0)}, {T(0), T(0)}};
          if (sz >= 0) {
            const cx<T> Uz = fetch(prev, sz);
            u = cmul(A, Uz);
#pragma unroll
            for (int a = 0; a < 3; ++a) {
              const cx<T> dZ = qn ? g.dzp[a] : g.dzm[a];
              du[a] = cfma(A, fetch(V + a * HU + pbase, sz), cmul(cx<T>{tz * dZ.x, tz * dZ.y}, Uz));
            }
          }
          if (sx >= 0) {
            const cx<T> Ux = fetch(prev, sx);
            u = cfma(Bc, Ux, u);
#pragma unroll
            for (int a = 0; a < 3; ++a) {
              const cx<T> dX = qn ? g.dxm[a] : g.dxp[a];
              du[a] = cfma(Bc, fetch(V + a * HU + pbase, sx), cfma(cx<T>{tx * dX.y, -tx * dX.x}, Ux, du[a]));
            }
          }
#pragma unroll
          for (int a = 0; a < 3; ++a) V[a * HU + idx] = du[a];
        } else {
          if (sz >= 0) u = cmul(A, fetch(prev, sz));
          if (sx >= 0) u = cfma(Bc, fetch(prev, sx), u);
          for (int ch = 0; ch < nch; ++ch) {
            const T f = g.fc * wch[ch];
            if (private_part) {
              cx<T> v = cpart[ch * HU + idx];
              cpart[ch * HU + idx] = {fma(f, u.x, v.x), fma(f, u.y, v.y)};
            } else {
              atomicAdd(&cpart[ch * HU + idx].x, f * u.x);
              atomicAdd(&cpart[ch * HU + idx].y, f * u.y);
            }
          }
        }
        cur[e] = u;
      }
    }
    __syncwarp();
    if constexpr (WITH_DU) {
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
    }
    cx<T>* t = prev;
    prev = cur;
    cur = t;
  }
  if constexpr (WITH_DU) {
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
}

template <typename T>
struct KernelArgs {
  DevTables tb;
  const typename RecEntry<T>::type* rec;
  const T* cg;
  // batch
  const int* atom_struct;
  const int* atom_start;
  const int* types;
  const int* small;
  const double* volume;
  const int* nbr_off;
  const int* nbr_idx;
  const double* nbr_u;
  // rows
  const long long* rowE;
  const long long* rowF;
  const long long* rowS;
  int D, ldx;
  int want_rows;
  int NB;  // neighbours per phase-3 chunk (2 per warp)
  BsoParams p;
  // Y (the contracted Z blocks, nch * NYP complex per atom) in global memory, one slice per CTA,
  // when it does not fit in shared memory next to the rest (FP64 with several channels)
  void* yglobal;
  // evaluation with fitted weights (eF != nullptr): no design rows
  DevEval<T> ev;
};

constexpr int kNW = 8;           // warps per CTA (== kZWarps)
constexpr int kG1 = 8;           // lanes per neighbour in phase 1
constexpr int kG3 = 16;          // lanes per neighbour in phase 3

// kYShared: Y lives in shared memory (the common case); otherwise in the per-CTA global slice
// args.yglobal (FP64 with several channels), a separate instantiation so that the shared-memory
// variant keeps shared-memory addressing.
template <typename T, bool kYShared>
__global__ void __launch_bounds__(kNW * 32, 2) k_bso4(KernelArgs<T> args, T* __restrict__ X, T* __restrict__ Bout,
                                                    T* __restrict__ dBout, int A) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const DevTables& tb = args.tb;
  const int J = tb.J, NU = tb.NU, HU = tb.HU, K = tb.K, NYP = tb.NYP;
  const int nch = args.p.nch;
  const int NB = args.NB;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  constexpr int nth = kNW * 32;
  const int LH = tb.hoff[J + 1] - tb.hoff[J];  // largest half layer

  // shared-memory carve-up
  cx<T>* cfull = reinterpret_cast<cx<T>*>(smem_raw);              // nch*NU
  cx<T>* Y = kYShared ? cfull + nch * NU
                      : reinterpret_cast<cx<T>*>(args.yglobal) + (size_t)blockIdx.x * nch * NYP;  // nch*NYP
  cx<T>* V = kYShared ? Y + (size_t)nch * NYP : cfull + nch * NU;  // max(NB*3, kNW*nch)*HU
  // V also holds the CG table during phase 2
  const size_t vblock = max((size_t)max(NB * 3, kNW * nch) * HU, (size_t)(tb.NCG + 1) / 2);
  cx<T>* ubuf = V + vblock;                                         // (32/kG1)*kNW*2*LH
  T* dBs = reinterpret_cast<T*>(ubuf + (size_t)(32 / kG1) * kNW * 2 * LH);  // 3*NB*K  [col][k]
  T* Bk = dBs + (size_t)3 * NB * K;                                 // nch*K
  T* selfacc = Bk + nch * K;                                        // nch*3*K
  T* stacc = selfacc + nch * 3 * K;                                 // nch*6*K
  T* nwt = stacc + nch * 6 * K;                                     // nch*NB neighbour weights
  T* nuu = nwt + nch * NB;                                          // NB*4 (uu[3] for stress, 1/r)
  int* nidx = reinterpret_cast<int*>(nuu + NB * 4);                 // NB neighbour atom index

  const T rcut = (T)args.p.rcut, inv_r0 = (T)args.p.inv_r0;
  const int ntile = tb.NTILE;

  for (int atom = blockIdx.x; atom < A; atom += gridDim.x) {
    const int s = args.atom_struct[atom];
    const int ti = args.types[atom];
    const int p0 = args.nbr_off[atom];
    const int nn = args.nbr_off[atom + 1] - p0;
    const long long rE = args.want_rows ? args.rowE[s] : -1;
    const long long rF = args.want_rows ? args.rowF[s] : -1;
    const long long rS = args.want_rows ? args.rowS[s] : -1;
    const bool eval = args.ev.F != nullptr;
    const bool need_d = (dBout != nullptr) || rF >= 0 || rS >= 0 || eval;
    const int a0 = args.atom_start[s];
    const int ldx = args.ldx;

    // ---------------- phase 1: c^j on half layers, 8 lanes per neighbour --------------
    // each lane group accumulates privately when the V block holds one partial per group
    const bool gpriv = (size_t)32 * nch * HU <= vblock;
    const int nparts = gpriv ? kNW * (32 / kG1) : kNW;
    for (int e = tid; e < nparts * nch * HU; e += nth) V[e] = {T(0), T(0)};
    for (int e = tid; e < nch * K * 10; e += nth) Bk[e] = T(0);  // Bk, selfacc, stacc
    for (int e = tid; e < nch * NYP; e += nth) Y[e] = {T(0), T(0)};
    __syncthreads();
    {
      constexpr int GPW = 32 / kG1;  // groups per warp
      const int grp = lane / kG1, sl = lane % kG1;
      cx<T>* cpart = V + (size_t)(gpriv ? warp * GPW + grp : warp) * nch * HU;
      cx<T>* ub = ubuf + (size_t)(warp * GPW + grp) * 2 * LH;
      for (int nb0 = warp * GPW; nb0 < nn; nb0 += kNW * GPW) {
        const int n = nb0 + grp;
        const bool active = n < nn;
        NbrGeom<T> g;
        T wch[kMaxCh] = {T(0), T(0), T(0)};
        if (active) {
          const int nb = args.nbr_idx[p0 + n];
          const int tn = args.types[nb];
          const double rin = args.p.has_rin ? args.p.rin[ti * args.p.ntypes + tn] : 0.0;
          nbr_geometry<T>(args.nbr_u + 3 * (size_t)(p0 + n), rcut, inv_r0, rin, args.p.rin_width, &g);
          for (int ch = 0; ch < nch; ++ch) wch[ch] = (T)args.p.chw[ch * args.p.ntypes + tn];
        }
        group_recursion<T, kG1, false>(g, args.rec, J, tb.hoff, ub, LH, nullptr, cpart, wch, nch, HU, sl, active,
                                       gpriv);
      }
    }
    __syncthreads();
    // reduce the warp partials into warp 0's block (thread-owned elements), expand to full layers
    for (int e = tid; e < nch * HU; e += nth) {
      cx<T> v = {T(0), T(0)};
      for (int w = 0; w < nparts; ++w) {
        const cx<T> q = V[(size_t)w * nch * HU + e];
        v.x += q.x;
        v.y += q.y;
      }
      if (tb.half_diag[e % HU]) v.x += T(1);
      V[e] = v;
    }
    __syncthreads();
    for (int e = tid; e < nch * NU; e += nth) {
      const int ch = e / NU, f = e - ch * NU;
      cfull[e] = fetch(V + ch * HU, tb.expand[f]);
    }
    __syncthreads();

    // ---------------- phase 2: folded Z -> Y, B in rounds of equal-shape terms ---------------
    // lane l of a round computes one Z term; the 32 terms of a round share their loop extents,
    // so the warp runs without divergence.  Terms add into Y (zeroed above) and B atomically.
    // The CG coefficients (a few thousand) are staged in V, free until phase 3, so that the
    // per-term coefficient loads come from shared memory.
    T* cgs = reinterpret_cast<T*>(V);
    for (int e = tid; e < tb.NCG; e += nth) cgs[e] = args.cg[e];
    __syncthreads();
    {
      const int r0 = tb.zitem_off[warp], r1 = tb.zitem_off[warp + 1];
      for (int ch = 0; ch < nch; ++ch) {
        const cx<T>* cc = cfull + ch * NU;
        cx<T>* Yc = Y + (size_t)ch * NYP;
        // each lane's entry of the next round is loaded while the current one is computed
        ZItem nx{};
        if (r0 < r1) nx = tb.zitems[(size_t)r0 * 32 + lane];
        for (int r = r0; r < r1; ++r) {
          const ZItem zi = nx;
          if (r + 1 < r1) nx = tb.zitems[(size_t)(r + 1) * 32 + lane];
          cx<T> zs;
          switch (zi.nb) {  // uniform over the round
            case 1: zs = zterm<1, T>(cc, cgs, zi); break;
            case 2: zs = zterm<2, T>(cc, cgs, zi); break;
            case 3: zs = zterm<3, T>(cc, cgs, zi); break;
            case 4: zs = zterm<4, T>(cc, cgs, zi); break;
            case 5: zs = zterm<5, T>(cc, cgs, zi); break;
            case 6: zs = zterm<6, T>(cc, cgs, zi); break;
            case 7: zs = zterm<7, T>(cc, cgs, zi); break;
            case 8: zs = zterm<8, T>(cc, cgs, zi); break;
            case 9: zs = zterm<9, T>(cc, cgs, zi); break;
            case 10: zs = zterm<10, T>(cc, cgs, zi); break;
            default: zs = zterm<11, T>(cc, cgs, zi); break;
          }
          if (zi.is_a) {
            const cx<T> cv = cc[zi.ufull];
            atomicAdd(&Bk[ch * K + zi.k], (T)zi.wgt * (cv.x * zs.x + cv.y * zs.y));  // w * Re(conj(c) ZA)
          }
          if (zi.wgt) {
            const T sc = (T)zi.snum / (T)zi.sden * (T)zi.wgt;
            atomicAdd(&Yc[zi.ypos].x, sc * zs.x);
            atomicAdd(&Yc[zi.ypos].y, sc * zs.y);
          }
        }
      }
    }
    __syncthreads();
    for (int e = tid; e < nch * K; e += nth) {
      const T b = (nn == 0) ? T(0) : Bk[e];
      if (Bout) Bout[(size_t)atom * nch * K + e] = b;
      if (rE >= 0) atomicAdd(&X[rE * ldx + 1 + e], b);
    }
    if (args.ev.E && args.ev.wlin && warp == 0) {
      // linear model: E_s += w0 + w_lin . B_a (FP64)
      double e = 0.0;
      if (nn > 0)
        for (int k = lane; k < nch * K; k += 32) e += args.ev.wlin[k] * (double)Bk[k];
      for (int o = 16; o > 0; o >>= 1) e += __shfl_xor_sync(0xffffffffu, e, o);
      if (lane == 0) atomicAdd(&args.ev.E[s], e + args.ev.w0);
    }
    if (!need_d || nn == 0) {
      __syncthreads();
      continue;
    }

    // ---------------- phase 3: dB per neighbour chunk, scattered into rows -----------
    const int nchunk = (nn + NB - 1) / NB;
    const int csz = (nn + nchunk - 1) / nchunk;  // balanced chunk size <= NB
    for (int base = 0; base < nn; base += csz) {
      const int nb_here = min(csz, nn - base);
      {
        constexpr int GPW = 32 / kG3;
        const int grp = lane / kG3, sl = lane % kG3;
        const int n = warp * GPW + grp;  // NB = kNW*GPW
        const bool active = n < nb_here;
        NbrGeom<T> g;
        const double* u3 = args.nbr_u + 3 * (size_t)(p0 + base + min(n, nb_here - 1));
        if (active) {
          const int nbi = args.nbr_idx[p0 + base + n];
          const int tn = args.types[nbi];
          const double rin = args.p.has_rin ? args.p.rin[ti * args.p.ntypes + tn] : 0.0;
          nbr_geometry<T>(u3, rcut, inv_r0, rin, args.p.rin_width, &g);
          if (sl == 0) {
            for (int ch = 0; ch < nch; ++ch) nwt[ch * NB + n] = (T)args.p.chw[ch * args.p.ntypes + tn];
            nidx[n] = nbi;
            const double r = sqrt(u3[0] * u3[0] + u3[1] * u3[1] + u3[2] * u3[2]);
            // stress lever arm: x_n - x_i (small box) or sign_big*(x_i - x_n) (large box)
            const double sg = args.small[s] ? 1.0 : -args.p.sign_big;
            nuu[n * 4 + 0] = (T)(sg * u3[0]);
            nuu[n * 4 + 1] = (T)(sg * u3[1]);
            nuu[n * 4 + 2] = (T)(sg * u3[2]);
            nuu[n * 4 + 3] = (T)(1.0 / r);
          }
        }
        group_recursion<T, kG3, true>(g, args.rec, J, tb.hoff, ubuf + (size_t)(warp * GPW + grp) * 2 * LH, LH,
                                      V + (size_t)min(n, NB - 1) * 3 * HU, nullptr, nullptr, nch, HU, sl, active);
      }
      const int ncols = 3 * nb_here;
      const int ncolt = (ncols + kColTile - 1) / kColTile;
      for (int ch = 0; ch < nch; ++ch) {
        for (int e = tid; e < 3 * NB * K; e += nth) dBs[e] = T(0);
        __syncthreads();
        // register-tiled contraction: item = (row tile of layer j, column tile)
        const cx<T>* Yc = Y + (size_t)ch * NYP;
        for (int it = tid; it < ntile * ncolt; it += nth) {
          const int tix = it / ncolt;
          const int tile = tb.tiles[tix];
          const int ct = it - tix * ncolt;
          const int j = tile >> 8, rt = tile & 255;
          const int Mp = tb.Mp[j], H = tb.hoff[j + 1] - tb.hoff[j];
          const cx<T>* Yp = Yc + tb.yoff[j] + rt * kRowTile;
          // columns ct, ct + ncolt, ...: lanes of a warp read consecutive columns of V, whose odd
          // stride HU spreads them over distinct shared-memory banks
          const cx<T>* Vp[kColTile];
#pragma unroll
          for (int c = 0; c < kColTile; ++c) {
            const int col = min(ct + c * ncolt, ncols - 1);
            Vp[c] = V + (size_t)col * HU + tb.hoff[j];  // col = n*3 + a -> V[n][a][.]
          }
          T acc[kRowTile][kColTile];
#pragma unroll
          for (int r = 0; r < kRowTile; ++r)
#pragma unroll
            for (int c = 0; c < kColTile; ++c) acc[r][c] = T(0);
#pragma unroll 2
          for (int e = 0; e < H; ++e) {
            cx<T> y[kRowTile], v[kColTile];
#pragma unroll
            for (int r = 0; r < kRowTile; ++r) y[r] = Yp[e * Mp + r];
#pragma unroll
            for (int c = 0; c < kColTile; ++c) v[c] = Vp[c][e];
#pragma unroll
            for (int r = 0; r < kRowTile; ++r)
#pragma unroll
              for (int c = 0; c < kColTile; ++c) acc[r][c] = fma(y[r].x, v[c].x, fma(-y[r].y, v[c].y, acc[r][c]));
          }
#pragma unroll
          for (int r = 0; r < kRowTile; ++r) {
            const int k = tb.rowk[tb.rowk_off[j] + rt * kRowTile + r];
            if (k < 0) continue;
#pragma unroll
            for (int c = 0; c < kColTile; ++c)
              if (ct + c * ncolt < ncols) atomicAdd(&dBs[(ct + c * ncolt) * K + k], acc[r][c]);
          }
        }
        __syncthreads();
        if (eval) {
          // forces and stress with the effective weights: the centre's for the forces, the
          // neighbour's for the stress (the neighbour's B in the quadratic stress rows,
          // mld_stress.F90:580-603); sums per (neighbour, component) in T, totals in FP64
          double* acc = reinterpret_cast<double*>(stacc);  // [0..2] self force, [3..8] stress
          const T* bc = args.ev.beta + (args.ev.beta_per_atom ? (size_t)atom * nch * K : 0) + ch * K;
          for (int it = tid; it < 3 * nb_here; it += nth) {
            const int n = it / 3, a = it - 3 * n;
            const T* d = dBs + (size_t)(n * 3 + a) * K;
            T f = T(0);
            for (int k = 0; k < K; ++k) f = fma(d[k], bc[k], f);
            const T wn = nwt[ch * NB + n];
            const double fv = (double)(f * wn);
            atomicAdd(&args.ev.F[3 * (size_t)nidx[n] + a], -fv);
            atomicAdd(&acc[a], fv);
            if (args.ev.S) {
              T g = f;
              if (args.ev.beta_per_atom) {
                const T* bn = args.ev.beta + (size_t)nidx[n] * nch * K + ch * K;
                g = T(0);
                for (int k = 0; k < K; ++k) g = fma(d[k], bn[k], g);
              }
              const double gv = (double)(g * wn) * (double)nuu[n * 4 + 3];
              const double ux = nuu[n * 4 + 0], uy = nuu[n * 4 + 1], uz = nuu[n * 4 + 2];
              if (a == 0) {  // xx, xz, xy
                atomicAdd(&acc[3], gv * ux);
                atomicAdd(&acc[7], gv * uz);
                atomicAdd(&acc[8], gv * uy);
              } else if (a == 1) {  // yy, yz
                atomicAdd(&acc[4], gv * uy);
                atomicAdd(&acc[6], gv * uz);
              } else {  // zz
                atomicAdd(&acc[5], gv * uz);
              }
            }
          }
          __syncthreads();
          continue;
        }
        // scatter: neighbour force rows (atomic), self force and stress accumulators
        for (int it = tid; it < 3 * K; it += nth) {
          const int a = it / K, k = it - a * K;
          T self = selfacc[ch * 3 * K + it];
          for (int n = 0; n < nb_here; ++n) {
            const T v = dBs[(n * 3 + a) * K + k] * nwt[ch * NB + n];
            self += v;
            if (rF >= 0) {
              const long long row = rF + 3LL * (nidx[n] - a0) + a;
              atomicAdd(&X[row * ldx + 1 + ch * K + k], -v);
            }
            if (dBout) dBout[((size_t)(p0 + base + n) * 3 + a) * nch * K + ch * K + k] = v;
          }
          selfacc[ch * 3 * K + it] = self;
        }
        if (rS >= 0) {
          for (int it = tid; it < 6 * K; it += nth) {
            const int sidx = it / K, k = it - sidx * K;
            const int aa = sidx < 3 ? sidx : (sidx == 3 ? 1 : 0);
            const int bb = sidx < 3 ? sidx : (sidx == 5 ? 1 : 2);
            T acc = stacc[ch * 6 * K + it];
            for (int n = 0; n < nb_here; ++n)
              acc += dBs[(n * 3 + aa) * K + k] * nwt[ch * NB + n] * nuu[n * 4 + bb] * nuu[n * 4 + 3];
            stacc[ch * 6 * K + it] = acc;
          }
        }
        __syncthreads();
      }
    }
    if (eval) {
      const double* acc = reinterpret_cast<const double*>(stacc);
      if (tid < 3) atomicAdd(&args.ev.F[3 * (size_t)atom + tid], acc[tid]);
      if (args.ev.S && tid >= 32 && tid < 38) {
        const double sc = args.p.sign_stress * 3.0 / args.volume[s];
        atomicAdd(&args.ev.S[6 * (size_t)s + tid - 32], sc * acc[3 + tid - 32]);
      }
      __syncthreads();
      continue;
    }
    // flush self force row and stress rows
    for (int ch = 0; ch < nch; ++ch) {
      if (rF >= 0) {
        for (int it = tid; it < 3 * K; it += nth) {
          const int a = it / K, k = it - a * K;
          const long long row = rF + 3LL * (atom - a0) + a;
          atomicAdd(&X[row * ldx + 1 + ch * K + k], selfacc[ch * 3 * K + it]);
        }
      }
      if (rS >= 0) {
        const T sc = (T)(args.p.sign_stress * 3.0 / args.volume[s]);
        for (int it = tid; it < 6 * K; it += nth) {
          const int sidx = it / K, k = it - sidx * K;
          atomicAdd(&X[(rS + sidx) * ldx + 1 + ch * K + k], sc * stacc[ch * 6 * K + it]);
        }
      }
    }
    __syncthreads();
  }
}

static size_t smem_bytes(const DevTables& tb, int nch, int eb, int NB, bool y_in_smem) {
  const size_t LH = tb.hoff[tb.J + 1] - tb.hoff[tb.J];
  const size_t cxb = 2 * (size_t)eb;
  const size_t vblock = std::max((size_t)std::max(NB * 3, kNW * nch) * tb.HU, (size_t)(tb.NCG + 1) / 2);
  size_t b = cxb * ((size_t)nch * tb.NU + (y_in_smem ? (size_t)nch * tb.NYP : 0) + vblock +
                    (size_t)(32 / kG1) * kNW * 2 * LH);
  b += (size_t)eb * ((size_t)3 * NB * tb.K + (size_t)nch * 10 * tb.K + (size_t)nch * NB + (size_t)NB * 4);
  b += sizeof(int) * NB;
  return b;
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

size_t bso4_y_scratch_bytes(const DevTables& tb, int nch, int eb, int max_ctas) {
  const int NB = kNW * (32 / kG3);
  if (smem_bytes(tb, nch, eb, NB, true) <= (size_t)max_optin_smem()) return 0;
  return (size_t)max_ctas * nch * tb.NYP * 2 * eb;
}

template <typename T>
cudaError_t launch_bso4_rows(const DevTables& tb, const DevBatch& b, const DevRows& rows, const BsoParams& p, T* X,
                             T* Bout, T* dBout, int want_rows, cudaStream_t st, void* yscratch, size_t yscratch_bytes,
                             const DevEval<T>* ev) {
  const int NB = kNW * (32 / kG3);
  if (b.A == 0) return cudaSuccess;
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
  a.atom_start = b.atom_start;
  a.types = b.types;
  a.small = b.small;
  a.volume = b.volume;
  a.nbr_off = b.nbr_off;
  a.nbr_idx = b.nbr_idx;
  a.nbr_u = b.nbr_u;
  a.rowE = rows.rowE;
  a.rowF = rows.rowF;
  a.rowS = rows.rowS;
  a.D = rows.D;
  a.ldx = rows.ldx;
  a.want_rows = want_rows;
  a.NB = NB;
  a.p = p;
  if (ev) a.ev = *ev;
  const bool y_in_smem = smem_bytes(tb, p.nch, sizeof(T), NB, true) <= (size_t)max_optin_smem();
  size_t smem = smem_bytes(tb, p.nch, sizeof(T), NB, y_in_smem);
  a.yglobal = nullptr;
  auto kern = y_in_smem ? k_bso4<T, true> : k_bso4<T, false>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int occ = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, kNW * 32, smem);
  if (occ < 1) return cudaErrorInvalidConfiguration;
  int grid = b.A;
  if (!y_in_smem) {
    // persistent CTAs (the kernel strides over atoms), one Y slice each
    const size_t per_cta = (size_t)p.nch * tb.NYP * 2 * sizeof(T);
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const long long fit = yscratch ? (long long)(yscratch_bytes / per_cta) : 0;
    grid = (int)std::min<long long>({(long long)b.A, (long long)nsm * occ, fit});
    if (grid < 1) return cudaErrorInvalidValue;  // Y scratch required and not given
    a.yglobal = yscratch;
  }
  kern<<<grid, kNW * 32, smem, st>>>(a, X, Bout, dBout, b.A);
  return cudaGetLastError();
}

template cudaError_t launch_bso4_rows<double>(const DevTables&, const DevBatch&, const DevRows&, const BsoParams&,
                                              double*, double*, double*, int, cudaStream_t, void*, size_t,
                                              const DevEval<double>*);
template cudaError_t launch_bso4_rows<float>(const DevTables&, const DevBatch&, const DevRows&, const BsoParams&,
                                             float*, float*, float*, int, cudaStream_t, void*, size_t,
                                             const DevEval<float>*);

}  // namespace mld
