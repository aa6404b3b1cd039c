// Host-side precompute of the SO(4) bispectrum contraction tables.
//
// Triple enumeration and the Clebsch-Gordan products follow MILADY
// src/mld/compute/compute_bispectrum_so4.F90:740-918 (l1 = 0..J, l2 = 0..l1,
// l = |l1-l2|..min(J,l1+l2), l1+l2+l even, l >= l1) and the coefficient formula of
// src/mld/angular_functions.f90:432-483 (cg / wigner3j with doubled indices).
// Instead of one flattened list of CG products per term (the reference's cg_A/cg_B/cg_C),
// each Z output stores its two 1-D coefficient lists and the strided c indices, so the GPU
// derives the 34 946 products per block from a table of a few thousand entries.
#include <algorithm>
#include <cmath>
#include <map>
#include <tuple>

#include "mld_internal.h"

namespace mld {

static double factorial(int n) {
  double r = 1.0;
  for (int i = 2; i <= n; ++i) r *= (double)i;
  return r;
}

static double sgn(int e) { return (e % 2 == 0) ? 1.0 : -1.0; }

static double wigner3j(int j1, int m1, int j2, int m2, int j, int m) {
  const int nt = 2;
  double coef = sgn((j1 - j2 - m) / nt) *
                std::sqrt(factorial((j1 + m1) / nt) * factorial((j1 - m1) / nt) * factorial((j2 + m2) / nt) *
                          factorial((j2 - m2) / nt) * factorial((j + m) / nt) * factorial((j - m) / nt));
  double tri = std::sqrt(factorial((j1 + j2 - j) / nt) * factorial((j1 - j2 + j) / nt) *
                         factorial((-j1 + j2 + j) / nt) / factorial((j1 + j2 + j) / nt + 1));
  int tmin = std::max(std::max((j2 - j - m1) / nt, (j1 + m2 - j) / nt), 0);
  int tmax = std::min(std::min((j1 + j2 - j) / nt, (j1 - m1) / nt), (j2 + m2) / nt);
  double s = 0.0;
  for (int t = tmin; t <= tmax; ++t)
    s += sgn(t) / (factorial(t) * factorial((j1 + j2 - j) / nt - t) * factorial((j1 - m1) / nt - t) *
                   factorial((j2 + m2) / nt - t) * factorial((j - j2 + m1) / nt + t) * factorial((j - j1 - m2) / nt + t));
  return coef * tri * s;
}

double cg_coefficient(int j1, int m1, int j2, int m2, int j, int m) {
  if (m - m1 - m2 != 0) return 0.0;
  if (j1 + j2 - j < 0 || j - j1 + j2 < 0 || j - j2 + j1 < 0) return 0.0;
  if ((j + j1 + j2) % 2 == 1) return 0.0;
  if (m1 < -j1 || m1 > j1 || m2 < -j2 || m2 > j2 || m < -j || m > j) return 0.0;
  return sgn((j1 - j2 + m) / 2) * std::sqrt((double)j + 1.0) * wigner3j(j1, m1, j2, m2, j, -m);
}

bool build_bso4_tables(double j_max, Bso4Tables* t, std::string* err) {
  const int J = (int)(2.0 * j_max);
  if (J < 0 || J > kMaxJ) {
    *err = "j_max out of range (0 <= 2*j_max <= " + std::to_string(kMaxJ) + ")";
    return false;
  }
  *t = Bso4Tables();
  t->J = J;
  int NU = 0;
  for (int j = 0; j <= J; ++j) {
    t->off[j] = NU;
    NU += (j + 1) * (j + 1);
  }
  t->off[J + 1] = NU;
  t->NU = NU;
  auto uidx = [&](int j, int p, int q) { return t->off[j] + ((p + j) / 2) * (j + 1) + (q + j) / 2; };

  for (int l1 = 0; l1 <= J; ++l1)
    for (int l2 = 0; l2 <= l1; ++l2)
      for (int l = l1 - l2; l <= std::min(J, l1 + l2); ++l) {
        if ((l1 + l2 + l) % 2 == 1) continue;
        if (l < l1) continue;
        t->l1.push_back(l1);
        t->l2.push_back(l2);
        t->l.push_back(l);
      }
  t->K = (int)t->l.size();

  std::map<std::tuple<int, int, int, int>, int> cgoff;  // (jA,jB,jOut,m) -> offset
  auto cglist = [&](int jA, int jB, int jO, int m) -> int {
    auto key = std::make_tuple(jA, jB, jO, m);
    auto it = cgoff.find(key);
    if (it != cgoff.end()) return it->second;
    int o = (int)t->cg.size();
    for (int ma = std::max(-jA, m - jB); ma <= std::min(jA, m + jB); ma += 2)
      t->cg.push_back(cg_coefficient(jA, ma, jB, m - ma, jO, m));
    cgoff[key] = o;
    return o;
  };

  // ZTerm list per (k, block) and per (m1,m2)
  struct Block { int jA, jB, jO, snum, sden; int first; };
  std::vector<std::vector<Block>> kblocks(t->K);
  for (int k = 0; k < t->K; ++k) {
    int l1 = t->l1[k], l2 = t->l2[k], l = t->l[k];
    Block bl[3] = {{l1, l2, l, 1, 1, 0}, {l, l2, l1, l + 1, l1 + 1, 0}, {l1, l, l2, l + 1, l2 + 1, 0}};
    for (int b = 0; b < 3; ++b) {
      Block& B = bl[b];
      B.first = (int)t->zterms.size();
      for (int m1 = -B.jO; m1 <= B.jO; m1 += 2)
        for (int m2 = -B.jO; m2 <= B.jO; m2 += 2) {
          int malo = std::max(-B.jA, m1 - B.jB), mahi = std::min(B.jA, m1 + B.jB);
          int mblo = std::max(-B.jA, m2 - B.jB), mbhi = std::min(B.jA, m2 + B.jB);
          ZTerm z;
          z.na = (uint8_t)((mahi - malo) / 2 + 1);
          z.nb = (uint8_t)((mbhi - mblo) / 2 + 1);
          z.s1 = (uint8_t)(B.jA + 1);
          z.s2 = (uint8_t)(B.jB + 1);
          z.i1 = (uint16_t)uidx(B.jA, malo, mblo);
          z.i2 = (uint16_t)uidx(B.jB, m1 - malo, m2 - mblo);
          z.cg1 = (uint16_t)cglist(B.jA, B.jB, B.jO, m1);
          z.cg2 = (uint16_t)cglist(B.jA, B.jB, B.jO, m2);
          z.snum = (uint8_t)B.snum;
          z.sden = (uint8_t)B.sden;
          z.pad = 0;
          long long nt = (long long)z.na * z.nb;
          (b == 0 ? t->cg_terms_A : b == 1 ? t->cg_terms_B : t->cg_terms_C) += nt;
          t->zterms.push_back(z);
        }
      kblocks[k].push_back(B);
    }
  }
  if (t->cg.size() >= 65535 || t->zterms.size() >= 65535) {
    *err = "contraction tables exceed 16-bit offsets";
    return false;
  }

  // merged Y slots: per k, per distinct layer
  t->kslot_begin.assign(t->K + 1, 0);
  std::vector<long long> cost;
  for (int k = 0; k < t->K; ++k) {
    t->kslot_begin[k] = (int)t->yslots.size();
    const auto& bl = kblocks[k];
    std::vector<int> layers;
    for (int b = 0; b < 3; ++b)
      if (std::find(layers.begin(), layers.end(), bl[b].jO) == layers.end()) layers.push_back(bl[b].jO);
    for (int j : layers) {
      int pos = 0;
      for (int p = -j; p <= j; p += 2)
        for (int q = -j; q <= j; q += 2, ++pos) {
          YSlot s{};
          s.nterm = 0;
          s.is_a = 0;
          long long c = 0;
          for (int b = 0; b < 3; ++b) {
            if (bl[b].jO != j) continue;
            if (b == 0) s.is_a = 1;
            int zi = bl[b].first + pos;
            s.term[s.nterm++] = (uint16_t)zi;
            c += (long long)t->zterms[zi].na * t->zterms[zi].nb;
          }
          s.uidx = (uint16_t)uidx(j, p, q);
          s.k = (uint16_t)k;
          t->yslots.push_back(s);
          cost.push_back(c);
        }
    }
  }
  t->kslot_begin[t->K] = (int)t->yslots.size();
  t->yorder.resize(t->yslots.size());
  for (size_t i = 0; i < t->yorder.size(); ++i) t->yorder[i] = (int)i;
  std::stable_sort(t->yorder.begin(), t->yorder.end(), [&](int a, int b) { return cost[a] > cost[b]; });
  return true;
}

}  // namespace mld
