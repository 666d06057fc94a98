// lj_schedule.cpp -- stream-K split of the all-pairs work (see lj_schedule.h).
#include "lj_schedule.h"

#include <algorithm>
#include <cstdint>

namespace ljgb {

bool build_schedule(const int* n, int nsys, int BI, int TILE, int G, int tile_overhead, Schedule* out) {
  if (!n || nsys < 1 || BI < 1 || TILE < 1 || G < 1 || !out || tile_overhead < 0) return false;
  Schedule s;
  s.BI = BI;
  s.TILE = TILE;
  s.sys_block_first.push_back(0);
  int64_t p0 = 0;
  for (int k = 0; k < nsys; ++k) {
    if (n[k] < 1) return false;
    const int nb = (n[k] + BI - 1) / BI;
    const int njt = (n[k] + TILE - 1) / TILE;
    for (int b = 0; b < nb; ++b) {
      BlockInfo bi{};
      bi.sys = k;
      bi.i0 = b * BI;
      bi.n_i = std::min(BI, n[k] - b * BI);
      bi.p0 = (int)p0;
      bi.n_sys = n[k];
      bi.njt = njt;
      s.blocks.push_back(bi);
    }
    p0 += n[k];
    if (p0 > INT32_MAX) return false;
    s.sys_block_first.push_back((int)s.blocks.size());
  }
  const int nblocks = (int)s.blocks.size();

  // Flattened tile sequence: block-major, j-tile minor.  Cost of a tile = its
  // j count + a fixed overhead (every thread of the CTA runs each j).
  std::vector<int64_t> tile_first(nblocks + 1, 0);
  for (int b = 0; b < nblocks; ++b) tile_first[b + 1] = tile_first[b] + s.blocks[b].njt;
  if (tile_first[nblocks] > INT32_MAX) return false;
  const int ntiles = (int)tile_first[nblocks];
  s.ntiles = ntiles;
  std::vector<int64_t> block_cost_first(nblocks + 1, 0);
  for (int b = 0; b < nblocks; ++b)
    block_cost_first[b + 1] =
        block_cost_first[b] + (int64_t)s.blocks[b].n_sys + (int64_t)s.blocks[b].njt * tile_overhead;
  const int64_t total = block_cost_first[nblocks];
  auto cost_before = [&](int b, int jt) -> int64_t {
    const int64_t j = std::min<int64_t>((int64_t)jt * TILE, s.blocks[b].n_sys);
    return block_cost_first[b] + j + (int64_t)jt * tile_overhead;
  };

  // At most one CTA per tile, so that every CTA owns at least one tile.
  G = std::min(G, ntiles);
  s.G = G;
  std::vector<int> tb(G + 1, 0);
  {
    int b = 0, jt = 0;
    for (int g = 0; g < G; ++g) {
      const int64_t target = (int64_t)((__int128)total * g / G);
      while (b < nblocks && cost_before(b, jt) < target) {
        if (++jt == s.blocks[b].njt) {
          ++b;
          jt = 0;
        }
      }
      tb[g] = (b < nblocks) ? (int)tile_first[b] + jt : ntiles;
    }
  }
  tb[0] = 0;
  for (int g = 1; g < G; ++g) tb[g] = std::max(tb[g], tb[g - 1] + 1);
  for (int g = 1; g < G; ++g) tb[g] = std::min(tb[g], ntiles - (G - g));
  tb[G] = ntiles;
  s.cta_tile_begin = tb;

  // (block, jt) of each CTA's first tile.
  s.cta_block.assign(G, 0);
  s.cta_jt.assign(G, 0);
  {
    int b = 0;
    for (int g = 0; g < G; ++g) {
      while (tile_first[b + 1] <= tb[g]) ++b;
      s.cta_block[g] = b;
      s.cta_jt[g] = tb[g] - (int)tile_first[b];
    }
  }

  // Segments of block b: the CTAs g whose [tb[g], tb[g+1]) meets the block's
  // tiles; they are consecutive and non-empty, so the segment of (g, b) is
  // seg_first[b] + g - g_first[b].
  int seg = 0;
  int g = 0;
  for (int b = 0; b < nblocks; ++b) {
    const int t0 = (int)tile_first[b], t1 = (int)tile_first[b + 1];
    while (g + 1 < G && tb[g + 1] <= t0) ++g;  // last CTA starting at or before t0
    int gh = g;
    while (gh + 1 < G && tb[gh + 1] < t1) ++gh;  // last CTA starting before t1
    s.blocks[b].g_first = g;
    s.blocks[b].seg_first = seg;
    s.blocks[b].seg_count = gh - g + 1;
    seg += gh - g + 1;
  }
  s.nseg = seg;
  *out = std::move(s);
  return true;
}

}  // namespace ljgb
