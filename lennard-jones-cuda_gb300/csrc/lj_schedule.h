// lj_schedule.h -- stream-K work split of the all-pairs loop (host side).
//
// The (i-block, j-chunk) pairs of every box are laid out in one sequence
// (box-major, then i-block, then j) and cut into G contiguous ranges of
// equal cost, one per persistent CTA.  Cuts fall on j-chunks of `grain`
// records, not only on whole j-tiles: the persistent grid holds every CTA at
// once, the hardware spreads consecutive CTAs over the SMs, and whole-tile
// ranges (some CTAs one tile more than others) leave SMs with up to one tile
// per resident CTA more work than others.  A CTA emits one partial segment
// per i-block it touches; the integrator sums each block's segments in CTA
// order.
#pragma once

#include <vector>

#include "lj_internal.h"

namespace ljgb {

struct Schedule {
  int G = 0;         // CTAs (persistent grid)
  int BI = 0;        // i-block length (= CTA threads of the pair kernel)
  int TILE = 0;      // j-tile length
  int ntiles = 0;    // total tiles
  int nseg = 0;      // partial segments
  std::vector<BlockInfo> blocks;
  int grain = 0;     // j records per work chunk (cut granularity)
  std::vector<int> cta_tile_begin;  // G + 1: flattened tile holding each CTA's first j
  std::vector<int> cta_lo;          // G + 1: offset of that j within its tile (entry G: 0)
  std::vector<int> cta_block;       // G
  std::vector<int> cta_jt;          // G
  std::vector<int> sys_block_first; // nsys + 1
};

// Builds the schedule for boxes of sizes n[0..nsys).  `tile_overhead` is the
// fixed cost of a tile in units of one j-record (barrier, compensation).
// CTA g covers j from (cta_tile_begin[g], cta_lo[g]) up to, not including,
// (cta_tile_begin[g+1], cta_lo[g+1]): cta_tile_begin[g+1] - cta_tile_begin[g]
// tiles, plus the head of tile cta_tile_begin[g+1] when cta_lo[g+1] > 0.
// Returns false on invalid input (n < 1, BI/TILE < 1, G < 1, TILE not a
// multiple of grain).
constexpr int kSplitGrain = 32;
bool build_schedule(const int* n, int nsys, int BI, int TILE, int G, int tile_overhead, Schedule* out,
                    int grain = kSplitGrain);

}  // namespace ljgb
