// Host-side precompute of the SO(4) bispectrum contraction tables.
//
// Triple enumeration and the Clebsch-Gordan products follow MILADY
// src/mld/compute/compute_bispectrum_so4.F90:740-918 (l1 = 0..J, l2 = 0..l1,
// l = |l1-l2|..min(J,l1+l2), l1+l2+l even, l >= l1); the coefficients themselves are the
// standard Clebsch-Gordan coefficients with doubled indices (the reference evaluates them
// through Wigner 3j symbols, src/mld/angular_functions.f90:432-483; here Racah's formula).
// Instead of one flattened list of CG products per term (the reference's cg_A/cg_B/cg_C),
// each Z output stores its two 1-D coefficient lists and the strided c indices, so the GPU
// derives the products from a table of a few thousand entries.  Only half of every layer is
// evaluated: U, c, Z and vecall all satisfy X(-p,-q) = (-1)^((p-q)/2) conj(X(p,q)), so the
// other half follows by conjugation and the sums over a full layer fold into 2*Re over the half
// (plus the self-symmetric centre of even layers).
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <map>
#include <tuple>

#include "mld_internal.h"

namespace mld {

static double factorial(int n) {
  double r = 1.0;
  for (int i = 2; i <= n; ++i) r *= (double)i;
  return r;
}

// Clebsch-Gordan coefficient <j1 m1 j2 m2 | j m> in the Condon-Shortley phase convention, from
// Racah's closed formula (G. Racah, Phys. Rev. 62, 438 (1942); D. A. Varshalovich et al.,
// "Quantum Theory of Angular Momentum", sec. 8.2.1):
//   C = delta(m, m1 + m2) sqrt((2j+1) (j1+j2-j)! (j1-j2+j)! (j2-j1+j)! / (j1+j2+j+1)!)
//       * sqrt((j1+m1)! (j1-m1)! (j2+m2)! (j2-m2)! (j+m)! (j-m)!)
//       * sum_k (-1)^k / [k! (j1+j2-j-k)! (j1-m1-k)! (j2+m2-k)! (j-j2+m1+k)! (j-j1-m2+k)!]
// with k over the integers that keep every factorial argument non-negative.  All arguments are
// doubled (2j, 2m), so the half-integer momenta of SO(4) are exact integers here.
double cg_coefficient(int j1, int m1, int j2, int m2, int j, int m) {
  if (m != m1 + m2) return 0.0;
  if (j1 + j2 < j || j1 + j < j2 || j2 + j < j1) return 0.0;  // triangle
  if ((j1 + j2 + j) % 2 != 0) return 0.0;
  if (std::abs(m1) > j1 || std::abs(m2) > j2 || std::abs(m) > j) return 0.0;
  if ((j1 + m1) % 2 || (j2 + m2) % 2 || (j + m) % 2) return 0.0;
  // undoubled integer combinations
  const int a = (j1 + j2 - j) / 2, b = (j1 - m1) / 2, c = (j2 + m2) / 2;
  const int d = (j - j2 + m1) / 2, e = (j - j1 - m2) / 2;
  const double norm = std::sqrt((double)(j + 1) * factorial(a) * factorial((j1 - j2 + j) / 2) *
                                factorial((j2 - j1 + j) / 2) / factorial((j1 + j2 + j) / 2 + 1)) *
                      std::sqrt(factorial((j1 + m1) / 2) * factorial(b) * factorial(c) * factorial((j2 - m2) / 2) *
                                factorial((j + m) / 2) * factorial((j - m) / 2));
  const int kmin = std::max(0, std::max(-d, -e));
  const int kmax = std::min(a, std::min(b, c));
  double sum = 0.0;
  for (int k = kmin; k <= kmax; ++k) {
    const double term = 1.0 / (factorial(k) * factorial(a - k) * factorial(b - k) * factorial(c - k) *
                               factorial(d + k) * factorial(e + k));
    sum += (k % 2 == 0) ? term : -term;
  }
  return norm * sum;
}

bool build_bso4_tables(double j_max, Bso4Tables* t, std::string* err) {
  const int J = (int)(2.0 * j_max);
  if (J < 0 || J > kMaxJ) {
    *err = "j_max out of range (0 <= 2*j_max <= " + std::to_string(kMaxJ) + ")";
    return false;
  }
  *t = Bso4Tables();
  t->J = J;
  int NU = 0, HU = 0;
  for (int j = 0; j <= J; ++j) {
    t->off[j] = NU;
    t->hoff[j] = HU;
    NU += (j + 1) * (j + 1);
    HU += ((j + 1) * (j + 1) + 1) / 2;
  }
  t->off[J + 1] = NU;
  t->hoff[J + 1] = HU;
  t->NU = NU;
  t->HU = HU;
  auto H = [&](int j) { return ((j + 1) * (j + 1) + 1) / 2; };
  auto loc = [&](int j, int p, int q) { return ((p + j) / 2) * (j + 1) + (q + j) / 2; };  // row-major in layer
  auto uidx = [&](int j, int p, int q) { return t->off[j] + loc(j, p, q); };
  // encoded reference to entry (p,q) of layer j through its stored half
  auto enc = [&](int j, int p, int q) -> int16_t {
    int e = loc(j, p, q);
    if (e < H(j)) return (int16_t)(e << 2);
    int partner = (j + 1) * (j + 1) - 1 - e;  // (-p,-q)
    int neg = (((p - q) / 2) % 2 != 0) ? 1 : 0;
    return (int16_t)((partner << 2) | 2 | neg);
  };

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

  // recursion and expansion tables on half layers (angular_functions.f90:108-272)
  t->rec_tz.assign(HU, 0.0);
  t->rec_tx.assign(HU, 0.0);
  t->rec_sz.assign(HU, -1);
  t->rec_sx.assign(HU, -1);
  t->rec_qneg.assign(HU, 0);
  t->half_diag.assign(HU, 0);
  t->expand.assign(NU, 0);
  for (int j = 0; j <= J; ++j) {
    for (int p = -j; p <= j; p += 2)
      for (int q = -j; q <= j; q += 2) {
        int e = loc(j, p, q);
        {
          // expansion reads the concatenated half layers: shift the local index by hoff[j]
          const int16_t code = enc(j, p, q);
          t->expand[t->off[j] + e] = (int16_t)((((code >> 2) + t->hoff[j]) << 2) | (code & 3));
        }
        if (e >= H(j)) continue;
        int hi = t->hoff[j] + e;
        if (p == q) t->half_diag[hi] = 1;
        if (j == 0) continue;
        int nterm = 0;
        if (q != -j) {
          double den = (double)(j + q);
          if (p != -j) {
            t->rec_tz[hi] = std::sqrt((double)(j + p) / den);
            t->rec_sz[hi] = enc(j - 1, p - 1, q - 1);
            ++nterm;
          }
          if (p != j) {
            t->rec_tx[hi] = std::sqrt((double)(j - p) / den);
            t->rec_sx[hi] = enc(j - 1, p + 1, q - 1);
            ++nterm;
          }
        } else {
          t->rec_qneg[hi] = 1;
          double den = (double)(j - q);
          if (p != j) {
            t->rec_tz[hi] = std::sqrt((double)(j - p) / den);
            t->rec_sz[hi] = enc(j - 1, p + 1, q + 1);
            ++nterm;
          }
          if (p != -j) {
            t->rec_tx[hi] = std::sqrt((double)(j + p) / den);
            t->rec_sx[hi] = enc(j - 1, p - 1, q + 1);
            ++nterm;
          }
        }
        (nterm == 1 ? t->u_one : t->u_two) += 1;
      }
  }

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

  // Z outputs on half layers; per (k, block) the index of its first half output
  struct Block { int jA, jB, jO, snum, sden, first; };
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
          long long nt = (long long)((mahi - malo) / 2 + 1) * ((mbhi - mblo) / 2 + 1);
          t->cg_terms_full += nt;
          if (loc(B.jO, m1, m2) >= H(B.jO)) continue;
          ZTerm z{};
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
          t->cg_terms += nt;
          t->zterms.push_back(z);
        }
      kblocks[k].push_back(B);
    }
  }
  if (t->cg.size() >= 65535 || t->zterms.size() >= 65535) {
    *err = "contraction tables exceed 16-bit offsets";
    return false;
  }
  // Z outputs with identical operands (the same c entries, CG lists and extents, e.g. the ZA
  // block of one triple and the ZB block of another) are one computation: each is evaluated
  // once, into the term buffer at its computation index, and every slot reads it there with its
  // own scale
  std::vector<int> zu(t->zterms.size());
  std::vector<int> zrep;  // representative output of each computation
  {
    std::map<std::tuple<int, int, int, int, int, int, int, int>, int> ids;
    for (size_t zi = 0; zi < t->zterms.size(); ++zi) {
      const ZTerm& z = t->zterms[zi];
      const auto key = std::make_tuple((int)z.i1, (int)z.i2, (int)z.cg1, (int)z.cg2, (int)z.na, (int)z.nb, (int)z.s1,
                                       (int)z.s2);
      auto it = ids.find(key);
      if (it == ids.end()) {
        it = ids.emplace(key, (int)zrep.size()).first;
        zrep.push_back((int)zi);
      }
      zu[zi] = it->second;
    }
    t->nzu = (int)zrep.size();
  }

  // layer-blocked Y: rows of layer j are the triples using layer j (any of l, l1, l2).  A
  // triple's distinct layers in ascending order have ranks 0, 1, 2; within a layer the rows are
  // grouped by rank, the layer padded to whole row tiles.  The dB contraction writes a row's
  // result into the buffer of its rank, where every triple has at most one row, so all tiles run
  // in one pass without atomics, and dB = (rank 0 + rank 1) + rank 2 in a fixed order.
  std::vector<std::vector<int>> rows(J + 1);  // row position -> triple (-1 padding)
  std::vector<std::vector<int>> rowrank(J + 1);  // row position -> rank
  std::vector<std::map<int, int>> rowpos(J + 1);  // triple -> row position
  t->rank_slot.assign((size_t)t->K * (kRounds - 1), -1);
  {
    std::vector<std::vector<std::vector<int>>> byrank(J + 1, std::vector<std::vector<int>>(kRounds));
    for (int k = 0; k < t->K; ++k) {
      int js[3] = {t->l[k], t->l1[k], t->l2[k]};
      std::sort(js, js + 3);
      int rank = 0;
      for (int b = 0; b < 3; ++b) {
        if (b > 0 && js[b] == js[b - 1]) continue;
        byrank[js[b]][rank++].push_back(k);
      }
    }
    for (int j = 0; j <= J; ++j)
      for (int r = 0; r < kRounds; ++r) {
        const std::vector<int>& v = byrank[j][r];
        if (v.empty()) continue;
        for (int k : v) {
          rowpos[j][k] = (int)rows[j].size();
          rows[j].push_back(k);
          rowrank[j].push_back(r);
          if (r > 0) t->rank_slot[(size_t)k * (kRounds - 1) + r - 1] = (int16_t)t->nrank[r]++;
        }
      }
    for (int j = 0; j <= J; ++j)
      while (rows[j].size() % kRowTile) {
        rows[j].push_back(-1);
        rowrank[j].push_back(0);
      }
    t->nrank[0] = t->K;
  }
  int ypos = 0, rk = 0;
  for (int j = 0; j <= J; ++j) {
    t->Mp[j] = (int)rows[j].size();
    t->yoff[j] = ypos;
    ypos += t->Mp[j] * H(j);
    t->rowk_off[j] = rk;
    for (int r = 0; r < t->Mp[j]; ++r) {
      const int k = rows[j][r], rank = rowrank[j][r];
      int16_t code = -1;
      if (k >= 0) code = (int16_t)((rank << kRankShift) | (rank == 0 ? k : t->rank_slot[(size_t)k * (kRounds - 1) + rank - 1]));
      t->rowk.push_back(code);
    }
    rk += t->Mp[j];
  }
  t->rowk_off[J + 1] = rk;
  t->NYP = ypos;
  if (ypos >= 65535) {
    *err = "Y table exceeds 16-bit offsets";
    return false;
  }
  if (t->K >= (1 << kRankShift)) {
    *err = "too many triples for the row destination code";
    return false;
  }
  // row tiles of the dB contraction, heaviest layers first
  for (int j = J; j >= 0; --j)
    for (int rt = 0; rt < t->Mp[j] / kRowTile; ++rt) t->tiles.push_back((j << 8) | rt);

  // folded slots; the kernel's slot entries; the ZA entries of every triple for B
  std::vector<std::vector<BkItem>> bk(t->K);
  for (int j = 0; j <= J; ++j) {
    for (const auto& kr : rowpos[j]) {
      const int k = kr.first, r = kr.second;
      const auto& bl = kblocks[k];
      for (int e = 0; e < H(j); ++e) {
        int p = -j + 2 * (e / (j + 1)), q = -j + 2 * (e % (j + 1));
        YSlot s{};
        SlotEntry se{};
        for (int b = 0; b < 3; ++b) {
          if (bl[b].jO != j) continue;
          if (b == 0) s.is_a = 1;
          int zi = bl[b].first + e;  // half outputs are stored in row-major order of the layer
          se.snum[s.nterm] = (uint8_t)t->zterms[zi].snum;
          se.sden[s.nterm] = (uint8_t)t->zterms[zi].sden;
          se.term[s.nterm] = (uint16_t)zu[zi];
          s.term[s.nterm++] = (uint16_t)zi;
        }
        s.ufull = (uint16_t)uidx(j, p, q);
        s.k = (uint16_t)k;
        s.ypos = (uint16_t)(t->yoff[j] + e * t->Mp[j] + r);
        s.wgt = (uint8_t)((p == 0 && q == 0) ? 1 : 2);
        se.ypos = s.ypos;
        se.nterm = s.nterm;
        se.wgt = s.wgt;
        t->yslots.push_back(s);
        t->slots.push_back(se);
        if (s.is_a) bk[k].push_back(BkItem{se.term[0], s.ufull, s.wgt, {0, 0, 0}});
      }
    }
  }
  t->bk_off.assign(t->K + 1, 0);
  for (int k = 0; k < t->K; ++k) {
    t->bk_off[k] = (int)t->bk_items.size();
    t->bk_items.insert(t->bk_items.end(), bk[k].begin(), bk[k].end());
  }
  t->bk_off[t->K] = (int)t->bk_items.size();

  // phase-2 schedule: every distinct Z computation is one work entry.  Entries of equal inner
  // extent nb (the kernel unrolls the b loop for it) form rounds of 32, one per lane: sorted by
  // descending na, so that a round's lanes run a-loops of nearly equal length (the round costs
  // its first lane's na * nb), the last round of each nb padded with entries of na = 0 that write
  // nothing.  Rounds go to the kZWarps warps longest-first (LPT) by that cost.  A term stores
  // its Z value at its own index of the term buffer; the slots and B are summed from there in a
  // fixed order.
  {
    std::map<int, std::vector<ZItem>> bynb;
    for (size_t u = 0; u < zrep.size(); ++u) {
      const ZTerm& z = t->zterms[zrep[u]];
      ZItem it{};
      it.i1 = z.i1;
      it.i2 = z.i2;
      it.cg1 = z.cg1;
      it.cg2 = z.cg2;
      it.na = z.na;
      it.nb = z.nb;
      it.s1 = z.s1;
      it.s2 = z.s2;
      it.term = (uint16_t)u;
      bynb[z.nb].push_back(it);
    }
    struct Round { long long cost; std::vector<ZItem> lanes; };
    std::vector<Round> rounds;
    for (auto& kv : bynb) {
      std::vector<ZItem>& v = kv.second;
      std::stable_sort(v.begin(), v.end(), [](const ZItem& x, const ZItem& y) { return x.na > y.na; });
      for (size_t i = 0; i < v.size(); i += 32) {
        Round r{(long long)v[i].na * kv.first, {}};
        for (size_t l = i; l < std::min(v.size(), i + 32); ++l) r.lanes.push_back(v[l]);
        while (r.lanes.size() < 32) {
          ZItem pad = v[i];  // valid offsets (the kernel loads its nb CG coefficients)
          pad.na = 0;
          pad.term = kNoTerm;
          r.lanes.push_back(pad);
        }
        rounds.push_back(std::move(r));
      }
    }
    std::stable_sort(rounds.begin(), rounds.end(), [](const Round& x, const Round& y) { return x.cost > y.cost; });
    std::vector<long long> load(kZWarps, 0);
    std::vector<std::vector<const Round*>> per(kZWarps);
    for (const Round& r : rounds) {
      int best = 0;
      for (int w = 1; w < kZWarps; ++w)
        if (load[w] < load[best]) best = w;
      load[best] += r.cost;
      per[best].push_back(&r);
    }
    t->zitem_off.assign(kZWarps + 1, 0);
    for (int w = 0; w < kZWarps; ++w) {
      t->zitem_off[w] = (int)(t->zitems.size() / 32);
      for (const Round* r : per[w]) t->zitems.insert(t->zitems.end(), r->lanes.begin(), r->lanes.end());
    }
    t->zitem_off[kZWarps] = (int)(t->zitems.size() / 32);
  }
  return true;
}

}  // namespace mld
