// Invariants of the host-built bispectrum tables that the descriptor kernel relies on without
// checking them itself: every Z term computed exactly once, rounds of one inner extent with
// outer extents in descending order, loop indices inside c and the CG table, slot and row codes
// in range and unique, recursion references inside the previous layer.  Built and run by
// tests/test_tables.py (host code only; no GPU).  Prints "ok <j_max>" per case, or the first
// failure and exits 1.
#include <cstdio>
#include <cstdlib>
#include <set>
#include <string>
#include <vector>

#include "../mld_gb300/csrc/mld_internal.h"

using namespace mld;

static int fail(double jm, const std::string& what) {
  std::printf("FAIL j_max=%.1f: %s\n", jm, what.c_str());
  return 1;
}

static int check(double jm) {
  Bso4Tables t;
  std::string err;
  if (!build_bso4_tables(jm, &t, &err)) return fail(jm, "build: " + err);
  const int NCG = (int)t.cg.size();
  // --- phase-2 rounds
  if (t.zitems.size() % 32) return fail(jm, "zitems not whole rounds");
  const int nrounds = (int)t.zitems.size() / 32;
  if ((int)t.zitem_off.size() != kZWarps + 1 || t.zitem_off[0] != 0 || t.zitem_off[kZWarps] != nrounds)
    return fail(jm, "zitem_off");
  for (int w = 0; w < kZWarps; ++w)
    if (t.zitem_off[w] > t.zitem_off[w + 1]) return fail(jm, "zitem_off not monotone");
  std::vector<int> seen(t.nzu, 0);
  for (int r = 0; r < nrounds; ++r) {
    const ZItem* z = &t.zitems[(size_t)r * 32];
    bool pads = false;
    for (int l = 0; l < 32; ++l) {
      if (z[l].nb != z[0].nb) return fail(jm, "round mixes inner extents");
      if (l > 0 && z[l].na > z[l - 1].na) return fail(jm, "outer extents not descending in a round");
      if (z[l].term == kNoTerm) {
        if (z[l].na != 0) return fail(jm, "padding lane with work");
        pads = true;
      } else {
        if (pads) return fail(jm, "real lane after padding");
        if (z[l].term >= t.nzu) return fail(jm, "term index out of range");
        seen[z[l].term]++;
      }
      if (z[l].nb < 1 || z[l].nb > 11) return fail(jm, "inner extent outside the kernel's cases");
      if (z[l].cg2 + z[l].nb > NCG) return fail(jm, "CG offset (inner) out of range");
      if (z[l].na > 0) {
        const int last1 = z[l].i1 + (z[l].na - 1) * z[l].s1 + (z[l].nb - 1);
        const int last2 = z[l].i2 - (z[l].na - 1) * z[l].s2 - (z[l].nb - 1);
        if (last1 >= t.NU || last2 < 0) return fail(jm, "c index out of range");
        if (z[l].cg1 + z[l].na > NCG) return fail(jm, "CG offset (outer) out of range");
      }
    }
  }
  for (int u = 0; u < t.nzu; ++u)
    if (seen[u] != 1) return fail(jm, "term not computed exactly once");
  // --- Y slots
  std::set<int> ypos;
  for (const SlotEntry& s : t.slots) {
    if (s.nterm < 1 || s.nterm > 3) return fail(jm, "slot term count");
    for (int q = 0; q < s.nterm; ++q) {
      if (s.term[q] >= t.nzu) return fail(jm, "slot term out of range");
      if (s.snum[q] < 1 || s.snum[q] > 15 || s.sden[q] < 1 || s.sden[q] > 15) return fail(jm, "slot scale outside the table");
    }
    if (s.ypos >= t.NYP || !ypos.insert(s.ypos).second) return fail(jm, "slot position out of range or repeated");
  }
  // --- contraction rows
  std::set<std::pair<int, int>> dst;
  int nrows = 0, ntiles = 0;
  for (int j = 0; j <= t.J; ++j) {
    if (t.Mp[j] % kRowTile) return fail(jm, "layer rows not whole tiles");
    nrows += t.Mp[j];
    ntiles += t.Mp[j] / kRowTile;
  }
  if (nrows != (int)t.rowk.size() || ntiles != (int)t.tiles.size()) return fail(jm, "row or tile count");
  for (int16_t c : t.rowk) {
    if (c < 0) continue;
    const int rank = c >> kRankShift, idx = c & ((1 << kRankShift) - 1);
    if (rank >= kRounds || idx >= t.nrank[rank]) return fail(jm, "row code out of range");
    if (!dst.insert({rank, idx}).second) return fail(jm, "two rows write one destination");
  }
  for (int k = 0; k < t.K; ++k)
    if (!dst.count({0, k})) return fail(jm, "triple without a rank-0 row");
  // --- B items
  for (size_t k = 0; k + 1 < t.bk_off.size(); ++k)
    if (t.bk_off[k] > t.bk_off[k + 1]) return fail(jm, "bk_off not monotone");
  for (const BkItem& b : t.bk_items)
    if (b.term >= t.nzu || b.ufull >= t.NU) return fail(jm, "B item out of range");
  // --- recursion records: non-negative coefficients (their sign carries q on the device) and
  // references inside the previous half layer
  for (int j = 1; j <= t.J; ++j) {
    const int nprev = t.hoff[j] - t.hoff[j - 1];
    for (int h = t.hoff[j]; h < t.hoff[j + 1]; ++h) {
      if (t.rec_tz[h] < 0.0 || t.rec_tx[h] < 0.0) return fail(jm, "negative recursion coefficient");
      if (t.rec_sz[h] >= 0 && (t.rec_sz[h] >> 2) >= nprev) return fail(jm, "z reference outside the previous layer");
      if (t.rec_sx[h] >= 0 && (t.rec_sx[h] >> 2) >= nprev) return fail(jm, "x reference outside the previous layer");
    }
  }
  for (int f = 0; f < t.NU; ++f)
    if ((t.expand[f] >> 2) >= t.HU) return fail(jm, "expansion reference out of range");
  std::printf("ok %.1f K=%d rounds=%d rows=%d\n", jm, t.K, nrounds, nrows);
  return 0;
}

int main(int argc, char** argv) {
  int bad = 0;
  for (int i = 1; i < argc; ++i) bad |= check(std::atof(argv[i]));
  return bad;
}
