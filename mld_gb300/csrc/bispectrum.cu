// Fused bispectrum-SO(4) descriptor + design-row kernel (one CTA per centre atom).
//
// Per atom i with neighbours n (u_n = x_n - x_i, r_n < r_cut):
//   phase 1  c^j(p,q) = delta_pq + sum_n w_ch(type_n) f_c(r_n) U^j_pq(u_n)          (compute_bispectrum_so4.F90:288-439)
//   phase 2  Z blocks ZA/ZB/ZC by Clebsch-Gordan contraction of c, merged per (k, layer) into Y,
//            B_k = Re sum conj(c^l) ZA_k                                              (:1014-1143, :469-560)
//   phase 3  per chunk of neighbours: dU recursion -> vecall V = conj(d(f_c U)/du) (angular_functions.f90:41-273),
//            dB_k/du_n = w_ch(type_n) Re sum_slots Y V                               (:469-717, descriptors.F90:298-302)
//            scattered straight into the energy / force / stress design rows          (mld_energy.F90:91-117,
//            mld_forces.F90:222-263, mld_stress.F90:272-756)
// T = double (plain FP64 method) or float (mixed method: FP32 descriptors).
#include <cuda_runtime.h>

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

// Per-flattened-index recursion coefficients: U = tz*Zsel*U[sz] + tx*(-i)*Xsel*U[sx]
// where (Zsel, Xsel) = (z-, x+) for q > -j and (z+, x-) for q == -j.
template <typename T>
struct RecTab {
  const T* tz;
  const T* tx;
  const int16_t* sz;   // index within layer j-1 (local), -1 if absent
  const int16_t* sx;
  const int8_t* qneg;
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
__device__ void nbr_geometry(const double* u3, double rcut, double inv_r0, double rin, double rin_w,
                             NbrGeom<T>* g) {
  const double PI = 3.14159265358979323846;
  T x0 = (T)u3[0], x1 = (T)u3[1], x2 = (T)u3[2];
  T rr = sqrt(x0 * x0 + x1 * x1 + x2 * x2);
  T r0 = (T)rcut / (T)inv_r0;
  T th0 = rr / r0;
  T s = sin(th0), c = cos(th0);
  T sin_i = T(1) / s, tan_i = c / s;
  T l0 = rr * sin_i, l0i = T(1) / l0, z0 = rr * tan_i;
  g->zp = {z0 * l0i, x2 * l0i};
  g->zm = {z0 * l0i, -x2 * l0i};
  g->xp = {x0 * l0i, x1 * l0i};
  g->xm = {x0 * l0i, -x1 * l0i};
  T drr[3] = {x0 / rr, x1 / rr, x2 / rr};
  T dz = tan_i - th0 * sin_i * sin_i;
  T dil0 = (c / r0 - l0i) / rr;
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
  if (rr <= (T)rcut) {
    T xx = rr / (T)rcut;
    fo = T(0.5) * (cos((T)PI * xx) + T(1));
    dfo = -T(0.5) * (T)PI * sin((T)PI * xx) / (T)rcut;
  }
  T fi = 0, dfi = 0;
  if (rin > 0.0) {
    T rc2 = (T)(rin + rin_w), w = (T)rin_w;
    if (rr <= rc2) {
      if (rr < rc2 - w) {
        fi = 1;
        dfi = 0;
      } else {
        T xx = (T)PI * (rr - rc2 + w) / w;
        fi = T(0.5) * (cos(xx) + T(1));
        dfi = -T(0.5) * sin(xx) * (T)PI / w;
      }
    }
  }
  g->fc = (T(1) - fi) * fo;
  T dfc = -dfi * fo + (T(1) - fi) * dfo;
  for (int a = 0; a < 3; ++a) g->dfr[a] = dfc * drr[a];
}

template <typename T>
__device__ __forceinline__ T tabval(const T* p, int i) {
  return __ldg(p + i);
}

// Phase-1 recursion of one neighbour by one warp, U only; accumulates f_c*w_ch*U into cpart.
template <typename T>
__device__ void warp_u_accumulate(const NbrGeom<T>& g, const RecTab<T>& rt, int J, const int* off, T* wch, int nch,
                                  cx<T>* ubuf /*2*(J+1)^2*/, cx<T>* cpart /*nch*NU*/, int NU, int lane) {
  cx<T>* prev = ubuf;
  cx<T>* cur = ubuf + (J + 1) * (J + 1);
  if (lane == 0) {
    prev[0] = {T(1), T(0)};
    for (int ch = 0; ch < nch; ++ch) {
      cx<T> v = cpart[ch * NU];
      cpart[ch * NU] = {v.x + g.fc * wch[ch], v.y};
    }
  }
  __syncwarp();
  for (int j = 1; j <= J; ++j) {
    int ne = (j + 1) * (j + 1);
    for (int e = lane; e < ne; e += 32) {
      int idx = off[j] + e;
      T tz = tabval<T>(rt.tz, idx), tx = tabval<T>(rt.tx, idx);
      int sz = rt.sz[idx], sx = rt.sx[idx];
      bool qn = rt.qneg[idx] != 0;
      cx<T> Z = qn ? g.zp : g.zm;
      cx<T> X = qn ? g.xm : g.xp;
      cx<T> u = {T(0), T(0)};
      if (sz >= 0) u = cmul(cx<T>{tz * Z.x, tz * Z.y}, prev[sz]);
      if (sx >= 0) u = cfma(cx<T>{tx * X.y, -tx * X.x}, prev[sx], u);  // (-i*tx*X)*U
      cur[e] = u;
      for (int ch = 0; ch < nch; ++ch) {
        T f = g.fc * wch[ch];
        cx<T> v = cpart[ch * NU + idx];
        cpart[ch * NU + idx] = {fma(f, u.x, v.x), fma(f, u.y, v.y)};
      }
    }
    __syncwarp();
    cx<T>* t = prev;
    prev = cur;
    cur = t;
  }
}

// Phase-3 recursion of one neighbour by one warp: U and dU, writing vecall into V[3][NU].
// dU of layer j-1 is kept in V until layer j has been formed, then converted in place.
template <typename T>
__device__ void warp_u_du_vecall(const NbrGeom<T>& g, const RecTab<T>& rt, int J, const int* off, cx<T>* ubuf,
                                 cx<T>* V, int NU, int lane) {
  cx<T>* prev = ubuf;
  cx<T>* cur = ubuf + (J + 1) * (J + 1);
  if (lane == 0) {
    prev[0] = {T(1), T(0)};
    for (int a = 0; a < 3; ++a) V[a * NU] = {T(0), T(0)};
  }
  __syncwarp();
  for (int j = 1; j <= J; ++j) {
    int ne = (j + 1) * (j + 1);
    for (int e = lane; e < ne; e += 32) {
      int idx = off[j] + e;
      T tz = tabval<T>(rt.tz, idx), tx = tabval<T>(rt.tx, idx);
      int sz = rt.sz[idx], sx = rt.sx[idx];
      bool qn = rt.qneg[idx] != 0;
      const cx<T> Z = qn ? g.zp : g.zm;
      const cx<T> X = qn ? g.xm : g.xp;
      cx<T> A = {tz * Z.x, tz * Z.y};
      cx<T> Bc = {tx * X.y, -tx * X.x};
      cx<T> u = {T(0), T(0)};
      cx<T> du[3] = {{T(0), T(0)}, {T(0), T(0)}, {T(0), T(0)}};
      int pz = off[j - 1] + sz, px = off[j - 1] + sx;
      if (sz >= 0) {
        cx<T> Uz = prev[sz];
        u = cmul(A, Uz);
        for (int a = 0; a < 3; ++a) {
          cx<T> dZ = qn ? g.dzp[a] : g.dzm[a];
          cx<T> dA = {tz * dZ.x, tz * dZ.y};
          du[a] = cfma(A, V[a * NU + pz], cmul(dA, Uz));
        }
      }
      if (sx >= 0) {
        cx<T> Ux = prev[sx];
        u = cfma(Bc, Ux, u);
        for (int a = 0; a < 3; ++a) {
          cx<T> dX = qn ? g.dxm[a] : g.dxp[a];
          cx<T> dB = {tx * dX.y, -tx * dX.x};
          du[a] = cfma(Bc, V[a * NU + px], cfma(dB, Ux, du[a]));
        }
      }
      cur[e] = u;
      for (int a = 0; a < 3; ++a) V[a * NU + idx] = du[a];
    }
    __syncwarp();
    // convert layer j-1 (raw dU) into vecall = conj(U)*dfc*u_a/r + fc*conj(dU)
    int np = j * j;
    for (int e = lane; e < np; e += 32) {
      int idx = off[j - 1] + e;
      cx<T> U = prev[e];
      for (int a = 0; a < 3; ++a) {
        cx<T> d = V[a * NU + idx];
        V[a * NU + idx] = {fma(U.x, g.dfr[a], g.fc * d.x), fma(-U.y, g.dfr[a], -g.fc * d.y)};
      }
    }
    __syncwarp();
    cx<T>* t = prev;
    prev = cur;
    cur = t;
  }
  {
    int np = (J + 1) * (J + 1);
    for (int e = lane; e < np; e += 32) {
      int idx = off[J] + e;
      cx<T> U = prev[e];
      for (int a = 0; a < 3; ++a) {
        cx<T> d = V[a * NU + idx];
        V[a * NU + idx] = {fma(U.x, g.dfr[a], g.fc * d.x), fma(-U.y, g.dfr[a], -g.fc * d.y)};
      }
    }
  }
  __syncwarp();
}

template <typename T>
struct KernelArgs {
  DevTables tb;
  RecTab<T> rt;
  const T* cg;
  int off[kMaxJ + 2];
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
  int D;
  int want_rows;
  BsoParams p;
};

template <typename T, int NW>
__global__ void __launch_bounds__(NW * 32) k_bso4(KernelArgs<T> args, T* __restrict__ X, T* __restrict__ Bout,
                                                   T* __restrict__ dBout, int A) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int J = args.tb.J, NU = args.tb.NU, K = args.tb.K, NY = args.tb.NY;
  const int nch = args.p.nch;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nth = NW * 32;
  const int LMAX = (J + 1) * (J + 1);

  // shared-memory carve-up
  cx<T>* c = reinterpret_cast<cx<T>*>(smem_raw);                 // nch*NU
  cx<T>* Y = c + nch * NU;                                          // NY
  cx<T>* V = Y + NY;                                                // NW*3*NU (phase 1: NW*nch*NU partial c)
  cx<T>* ubuf = V + (size_t)NW * 3 * NU;                            // NW*2*LMAX
  T* Bk = reinterpret_cast<T*>(ubuf + (size_t)NW * 2 * LMAX);       // K
  T* dBc = Bk + K;                                                  // NW*3*K
  T* selfacc = dBc + NW * 3 * K;                                    // 3*K
  T* stacc = selfacc + 3 * K;                                       // 6*K
  T* nw = stacc + 6 * K;                                            // NW (neighbour weight this channel)
  T* nuu = nw + NW;                                                 // NW*4 (uu[3] for stress, 1/r)
  int* nidx = reinterpret_cast<int*>(nuu + NW * 4);                 // NW neighbour atom index
  int* ntyp = nidx + NW;                                            // NW neighbour type

  for (int atom = blockIdx.x; atom < A; atom += gridDim.x) {
    const int s = args.atom_struct[atom];
    const int ti = args.types[atom];
    const int p0 = args.nbr_off[atom];
    const int nn = args.nbr_off[atom + 1] - p0;
    const long long rE = args.want_rows ? args.rowE[s] : -1;
    const long long rF = args.want_rows ? args.rowF[s] : -1;
    const long long rS = args.want_rows ? args.rowS[s] : -1;
    const bool need_d = (dBout != nullptr) || rF >= 0 || rS >= 0;
    const int a0 = args.atom_start[s];
    const int D = args.D;

    // ---------------- phase 1: c^j --------------------------------------------------
    for (int e = tid; e < NW * nch * NU; e += nth) V[e] = {T(0), T(0)};
    __syncthreads();
    {
      cx<T>* cpart = V + (size_t)warp * nch * NU;
      cx<T>* ub = ubuf + (size_t)warp * 2 * LMAX;
      for (int n = warp; n < nn; n += NW) {
        NbrGeom<T> g;
        int nb = args.nbr_idx[p0 + n];
        int tn = args.types[nb];
        double rin = args.p.has_rin ? args.p.rin[ti * args.p.ntypes + tn] : 0.0;
        nbr_geometry<T>(args.nbr_u + 3 * (size_t)(p0 + n), args.p.rcut, args.p.inv_r0, rin, args.p.rin_width, &g);
        T wch[kMaxCh];
        for (int ch = 0; ch < nch; ++ch) wch[ch] = (T)args.p.chw[ch * args.p.ntypes + tn];
        warp_u_accumulate<T>(g, args.rt, J, args.off, wch, nch, ub, cpart, NU, lane);
      }
    }
    __syncthreads();
    for (int e = tid; e < nch * NU; e += nth) {
      cx<T> v = {T(0), T(0)};
      for (int w = 0; w < NW; ++w) {
        cx<T> q = V[(size_t)w * nch * NU + e];
        v.x += q.x;
        v.y += q.y;
      }
      int idx = e % NU;
      if (args.tb.up[idx] == args.tb.uq[idx]) v.x += T(1);
      c[e] = v;
    }
    __syncthreads();

    for (int ch = 0; ch < nch; ++ch) {
      const cx<T>* cc = c + ch * NU;
      // ---------------- phase 2: Z -> Y, B ------------------------------------------
      for (int k = tid; k < K; k += nth) Bk[k] = T(0);
      for (int e = tid; e < 9 * K; e += nth) selfacc[e] = T(0);  // selfacc + stacc contiguous
      __syncthreads();
      for (int t = tid; t < NY; t += nth) {
        const int sidx = args.tb.yorder[t];
        const YSlot sl = args.tb.yslots[sidx];
        cx<T> acc = {T(0), T(0)};
        for (int tt = 0; tt < sl.nterm; ++tt) {
          const ZTerm z = args.tb.zterms[sl.term[tt]];
          cx<T> zs = {T(0), T(0)};
          int i1a = z.i1, i2a = z.i2;
          for (int a = 0; a < z.na; ++a) {
            T c1 = tabval<T>(args.cg, z.cg1 + a);
            cx<T> part = {T(0), T(0)};
            int i1 = i1a, i2 = i2a;
            for (int b = 0; b < z.nb; ++b) {
              T c2 = tabval<T>(args.cg, z.cg2 + b);
              cx<T> pr = cmul(cc[i1], cc[i2]);
              part.x = fma(c2, pr.x, part.x);
              part.y = fma(c2, pr.y, part.y);
              ++i1;
              --i2;
            }
            zs.x = fma(c1, part.x, zs.x);
            zs.y = fma(c1, part.y, zs.y);
            i1a += z.s1;
            i2a -= z.s2;
          }
          if (tt == 0 && sl.is_a) {
            cx<T> cv = cc[sl.uidx];
            atomicAdd(&Bk[sl.k], cv.x * zs.x + cv.y * zs.y);  // Re(conj(c) * ZA)
          }
          const T sc = (T)z.snum / (T)z.sden;
          acc.x = fma(sc, zs.x, acc.x);
          acc.y = fma(sc, zs.y, acc.y);
        }
        Y[sidx] = acc;
      }
      __syncthreads();
      if (nn == 0) {
        for (int k = tid; k < K; k += nth) Bk[k] = T(0);
        __syncthreads();
      }
      for (int k = tid; k < K; k += nth) {
        if (Bout) Bout[(size_t)atom * nch * K + ch * K + k] = Bk[k];
        if (rE >= 0) atomicAdd(&X[rE * D + 1 + ch * K + k], Bk[k]);
      }
      if (!need_d || nn == 0) {
        __syncthreads();
        continue;
      }

      // ---------------- phase 3: dB per neighbour chunk, scattered into rows ----------
      for (int base = 0; base < nn; base += NW) {
        const int nb_here = min(NW, nn - base);
        if (warp < nb_here) {
          const int n = base + warp;
          NbrGeom<T> g;
          int nb = args.nbr_idx[p0 + n];
          int tn = args.types[nb];
          double rin = args.p.has_rin ? args.p.rin[ti * args.p.ntypes + tn] : 0.0;
          const double* u3 = args.nbr_u + 3 * (size_t)(p0 + n);
          nbr_geometry<T>(u3, args.p.rcut, args.p.inv_r0, rin, args.p.rin_width, &g);
          warp_u_du_vecall<T>(g, args.rt, J, args.off, ubuf + (size_t)warp * 2 * LMAX, V + (size_t)warp * 3 * NU,
                              NU, lane);
          if (lane == 0) {
            nw[warp] = (T)args.p.chw[ch * args.p.ntypes + tn];
            nidx[warp] = nb;
            ntyp[warp] = tn;
            double r = sqrt(u3[0] * u3[0] + u3[1] * u3[1] + u3[2] * u3[2]);
            // stress lever arm: x_n - x_i (small box) or sign_big*(x_i - x_n) (large box)
            double sg = args.small[s] ? 1.0 : -args.p.sign_big;
            nuu[warp * 4 + 0] = (T)(sg * u3[0]);
            nuu[warp * 4 + 1] = (T)(sg * u3[1]);
            nuu[warp * 4 + 2] = (T)(sg * u3[2]);
            nuu[warp * 4 + 3] = (T)(1.0 / r);
          }
        }
        __syncthreads();
        // dB GEMM: item = (k, w); 3 outputs each
        for (int it = tid; it < K * nb_here; it += nth) {
          const int k = it / nb_here, w = it - k * nb_here;
          const cx<T>* Vw = V + (size_t)w * 3 * NU;
          T acc0 = 0, acc1 = 0, acc2 = 0;
          const int sb = args.tb.kslot_begin[k], se = args.tb.kslot_begin[k + 1];
          for (int si = sb; si < se; ++si) {
            const cx<T> y = Y[si];
            const int ui = args.tb.yslots[si].uidx;
            cx<T> v0 = Vw[ui], v1 = Vw[NU + ui], v2 = Vw[2 * NU + ui];
            acc0 = fma(y.x, v0.x, fma(-y.y, v0.y, acc0));
            acc1 = fma(y.x, v1.x, fma(-y.y, v1.y, acc1));
            acc2 = fma(y.x, v2.x, fma(-y.y, v2.y, acc2));
          }
          const T wt = nw[w];
          dBc[(w * 3 + 0) * K + k] = wt * acc0;
          dBc[(w * 3 + 1) * K + k] = wt * acc1;
          dBc[(w * 3 + 2) * K + k] = wt * acc2;
        }
        __syncthreads();
        // scatter: neighbour force rows (atomic), self force and stress accumulators
        for (int it = tid; it < 3 * K; it += nth) {
          const int a = it / K, k = it - a * K;
          T self = selfacc[it];
          for (int w = 0; w < nb_here; ++w) {
            T v = dBc[(w * 3 + a) * K + k];
            self += v;
            if (rF >= 0) {
              long long row = rF + 3LL * (nidx[w] - a0) + a;
              atomicAdd(&X[row * D + 1 + ch * K + k], -v);
            }
            if (dBout) dBout[((size_t)(p0 + base + w) * 3 + a) * nch * K + ch * K + k] = v;
          }
          selfacc[it] = self;
        }
        if (rS >= 0) {
          for (int it = tid; it < 6 * K; it += nth) {
            const int sidx = it / K, k = it - sidx * K;
            const int aa = sidx < 3 ? sidx : (sidx == 3 ? 1 : 0);
            const int bb = sidx < 3 ? sidx : (sidx == 5 ? 1 : 2);
            T acc = stacc[it];
            for (int w = 0; w < nb_here; ++w) acc += dBc[(w * 3 + aa) * K + k] * nuu[w * 4 + bb] * nuu[w * 4 + 3];
            stacc[it] = acc;
          }
        }
        __syncthreads();
      }
      // flush self force row and stress rows
      if (rF >= 0) {
        for (int it = tid; it < 3 * K; it += nth) {
          const int a = it / K, k = it - a * K;
          long long row = rF + 3LL * (atom - a0) + a;
          atomicAdd(&X[row * D + 1 + ch * K + k], selfacc[it]);
        }
      }
      if (rS >= 0) {
        const T sc = (T)(args.p.sign_stress * 3.0 / args.volume[s]);
        for (int it = tid; it < 6 * K; it += nth) {
          const int sidx = it / K, k = it - sidx * K;
          atomicAdd(&X[(rS + sidx) * D + 1 + ch * K + k], sc * stacc[it]);
        }
      }
      __syncthreads();
    }
  }
}

size_t bso4_smem_bytes(int NU, int NY, int K, int nch, int eb, int NW) {
  // mirrors the carve-up at the top of k_bso4
  int J = 0;
  while ((J + 1) * (J + 2) * (2 * J + 3) / 6 < NU) ++J;  // sum_{j<=J}(j+1)^2 == NU
  size_t LMAX = (size_t)(J + 1) * (J + 1);
  size_t cxb = 2 * (size_t)eb;
  size_t b = cxb * ((size_t)nch * NU + NY + (size_t)NW * 3 * NU + (size_t)NW * 2 * LMAX);
  b += (size_t)eb * (K + (size_t)NW * 3 * K + 9 * (size_t)K + NW + NW * 4);
  b += sizeof(int) * 2 * NW;
  return b;
}

template <typename T>
cudaError_t launch_bso4_rows(const DevTables& tb, const DevBatch& b, const DevRows& rows, const BsoParams& p, T* X,
                             T* Bout, T* dBout, int want_rows, cudaStream_t st) {
  constexpr int NW = sizeof(T) == 8 ? 4 : 8;
  if (b.A == 0) return cudaSuccess;
  KernelArgs<T> a{};
  a.tb = tb;
  if constexpr (sizeof(T) == 8) {
    a.rt.tz = reinterpret_cast<const T*>(tb.rec_tz64);
    a.rt.tx = reinterpret_cast<const T*>(tb.rec_tx64);
    a.cg = reinterpret_cast<const T*>(tb.cg64);
  } else {
    a.rt.tz = reinterpret_cast<const T*>(tb.rec_tz32);
    a.rt.tx = reinterpret_cast<const T*>(tb.rec_tx32);
    a.cg = reinterpret_cast<const T*>(tb.cg32);
  }
  a.rt.sz = tb.rec_sz;
  a.rt.sx = tb.rec_sx;
  a.rt.qneg = tb.rec_qneg;
  int J = tb.J;
  int o = 0;
  for (int j = 0; j <= J + 1; ++j) {
    a.off[j] = o;
    o += (j + 1) * (j + 1);
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
  a.want_rows = want_rows;
  a.p = p;
  size_t smem = bso4_smem_bytes(tb.NU, tb.NY, tb.K, p.nch, sizeof(T), NW);
  cudaError_t e = cudaFuncSetAttribute(k_bso4<T, NW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int dev = 0, nsm = 0, occ = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_bso4<T, NW>, NW * 32, smem);
  if (occ < 1) return cudaErrorInvalidConfiguration;
  int grid = b.A;
  k_bso4<T, NW><<<grid, NW * 32, smem, st>>>(a, X, Bout, dBout, b.A);
  return cudaGetLastError();
}

template cudaError_t launch_bso4_rows<double>(const DevTables&, const DevBatch&, const DevRows&, const BsoParams&,
                                              double*, double*, double*, int, cudaStream_t);
template cudaError_t launch_bso4_rows<float>(const DevTables&, const DevBatch&, const DevRows&, const BsoParams&,
                                             float*, float*, float*, int, cudaStream_t);

}  // namespace mld
