// grand_solo.h -- the solo-column table of a code (host side, built with the code tables).
//
// A solo column is a nonzero column of H that contains no other nonzero column
// (no c' != c whose set rows all lie in c's).  A syndrome equal to a solo column
// c has exactly one nonzero column contained in it, c itself: its first
// threshold iteration has the active set {c} (a column's flagged-check count,
// with the irregular offset, reaches the first threshold exactly when the
// column lies inside the syndrome), and that set's one candidate, c, matches.
// The classification step settles such shots with one lookup of the syndrome's
// sketch in this table (open addressing, linear probing, keys = the column
// sketches, an empty slot holds column -1) instead of walking the columns.
#pragma once

#include <stdint.h>

#include <vector>

namespace grand {

struct SoloTable {
  std::vector<uint32_t> keys;  // column sketch per slot
  std::vector<int> cols;       // column per slot, -1 when empty
  uint32_t mask = 0;           // slots - 1 (a power of two minus one)
};

// cols: m columns of nwp words (nw meaningful); hcol: their sketches.
inline SoloTable build_solo_table(const std::vector<uint32_t> &cols, int nwp, int nw, int m,
                                  const std::vector<uint32_t> &hcol) {
  // nonzero columns grouped by their lowest set row: a column c' inside c has
  // its lowest row among c's rows, so only those groups need checking
  const int R = nw * 32;
  std::vector<int> lowrow(m, -1);
  for (int c = 0; c < m; ++c)
    for (int q = 0; q < nw && lowrow[c] < 0; ++q) {
      const uint32_t w = cols[(size_t)c * nwp + q];
      if (w) lowrow[c] = q * 32 + __builtin_ctz(w);
    }
  std::vector<int> start(R + 1, 0), group;
  for (int c = 0; c < m; ++c)
    if (lowrow[c] >= 0) ++start[lowrow[c] + 1];
  for (int r = 0; r < R; ++r) start[r + 1] += start[r];
  group.assign(start[R] > 0 ? start[R] : 1, 0);
  {
    std::vector<int> fill(start.begin(), start.end() - 1);
    for (int c = 0; c < m; ++c)
      if (lowrow[c] >= 0) group[fill[lowrow[c]]++] = c;
  }
  std::vector<int> solo;
  for (int c = 0; c < m; ++c) {
    if (lowrow[c] < 0) continue;
    bool alone = true;
    for (int q = 0; q < nw && alone; ++q)
      for (uint32_t w = cols[(size_t)c * nwp + q]; w && alone; w &= w - 1u) {
        const int r = q * 32 + __builtin_ctz(w);
        for (int i = start[r]; i < start[r + 1] && alone; ++i) {
          const int o = group[i];
          if (o == c) continue;
          bool inside = true;
          for (int k = 0; k < nw && inside; ++k)
            inside = (cols[(size_t)o * nwp + k] & ~cols[(size_t)c * nwp + k]) == 0u;
          if (inside) alone = false;
        }
      }
    if (alone) solo.push_back(c);
  }
  SoloTable t;
  size_t slots = 2;
  while (slots < 2 * solo.size()) slots <<= 1;
  t.keys.assign(slots, 0u);
  t.cols.assign(slots, -1);
  t.mask = (uint32_t)(slots - 1);
  for (int c : solo) {
    uint32_t i = hcol[c] & t.mask;
    while (t.cols[i] >= 0) i = (i + 1) & t.mask;
    t.keys[i] = hcol[c];
    t.cols[i] = c;
  }
  return t;
}

}  // namespace grand
