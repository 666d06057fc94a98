// lj_schedule.cpp -- stream-K split of the all-pairs work (see lj_schedule.h).
#include "lj_schedule.h"

#include <algorithm>
#include <cstdint>

namespace ljgb {

bool build_schedule(const int* n, int nsys, int BI, int TILE, int G, int tile_overhead, Schedule* out, int grain) {
  if (!n || nsys < 1 || BI < 1 || TILE < 1 || G < 1 || !out || tile_overhead < 0) return false;
  if (grain < 1 || TILE % grain != 0) return false;
  Schedule s;
  s.BI = BI;
  s.TILE = TILE;
  s.grain = grain;
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

  // Work units: the j-chunks of `grain` records of every block, block-major.
  // Chunk c of a block covers j in [c*grain, min((c+1)*grain, n_sys)); its
  // tile is c*grain / TILE (TILE is a multiple of grain).  Cost of a chunk =
  // its j count, plus a fixed overhead for each tile a CTA starts.
  std::vector<int64_t> tile_first(nblocks + 1, 0), chunk_first(nblocks + 1, 0), cost_first(nblocks + 1, 0);
  for (int b = 0; b < nblocks; ++b) {
    const BlockInfo& bi = s.blocks[b];
    tile_first[b + 1] = tile_first[b] + bi.njt;
    chunk_first[b + 1] = chunk_first[b] + (bi.n_sys + grain - 1) / grain;
    cost_first[b + 1] = cost_first[b] + (int64_t)bi.n_sys + (int64_t)bi.njt * tile_overhead;
  }
  if (tile_first[nblocks] > INT32_MAX || chunk_first[nblocks] > INT32_MAX) return false;
  const int ntiles = (int)tile_first[nblocks];
  const int64_t nchunks = chunk_first[nblocks];
  s.ntiles = ntiles;
  const int64_t total = cost_first[nblocks];
  // Cost of the work before chunk c of block b.
  auto cost_before = [&](int b, int64_t c) -> int64_t {
    const int64_t j = std::min<int64_t>(c * grain, s.blocks[b].n_sys);
    return cost_first[b] + j + (c * grain + TILE - 1) / TILE * tile_overhead;
  };

  // CTA g starts at the first chunk whose preceding cost reaches g/G of the
  // total; at most one CTA per chunk, so that every CTA owns some work.
  G = (int)std::min<int64_t>(G, nchunks);
  s.G = G;
  std::vector<int64_t> cb(G + 1, 0);
  for (int g = 1; g < G; ++g) {
    const int64_t target = (int64_t)((__int128)total * g / G);
    int b = (int)(std::upper_bound(cost_first.begin(), cost_first.end(), target) - cost_first.begin()) - 1;
    b = std::max(0, std::min(b, nblocks - 1));
    int64_t lo = 0, hi = chunk_first[b + 1] - chunk_first[b];  // smallest c in [lo, hi] with cost >= target
    while (lo < hi) {
      const int64_t mid = (lo + hi) / 2;
      if (cost_before(b, mid) >= target) hi = mid;
      else lo = mid + 1;
    }
    cb[g] = chunk_first[b] + lo;
  }
  cb[0] = 0;
  for (int g = 1; g < G; ++g) cb[g] = std::max(cb[g], cb[g - 1] + 1);
  for (int g = G - 1; g >= 1; --g) cb[g] = std::min(cb[g], nchunks - (G - g));
  cb[G] = nchunks;

  // Start of each CTA as (flattened tile, block, tile in block, offset).
  s.cta_tile_begin.assign(G + 1, ntiles);
  s.cta_lo.assign(G + 1, 0);
  s.cta_block.assign(G, 0);
  s.cta_jt.assign(G, 0);
  {
    int b = 0;
    for (int g = 0; g < G; ++g) {
      while (chunk_first[b + 1] <= cb[g]) ++b;
      const int64_t j = (cb[g] - chunk_first[b]) * grain;
      s.cta_block[g] = b;
      s.cta_jt[g] = (int)(j / TILE);
      s.cta_lo[g] = (int)(j % TILE);
      s.cta_tile_begin[g] = (int)tile_first[b] + (int)(j / TILE);
    }
  }

  // Segments of block b: the CTAs whose chunk ranges meet the block's; they
  // are consecutive, so the segment of (g, b) is seg_first[b] + g - g_first[b].
  int seg = 0;
  int g = 0;
  for (int b = 0; b < nblocks; ++b) {
    const int64_t c0 = chunk_first[b], c1 = chunk_first[b + 1];
    while (g + 1 < G && cb[g + 1] <= c0) ++g;  // last CTA starting at or before c0
    int gh = g;
    while (gh + 1 < G && cb[gh + 1] < c1) ++gh;  // last CTA starting before c1
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
