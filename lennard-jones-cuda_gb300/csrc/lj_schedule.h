// lj_schedule.h -- stream-K work split of the all-pairs loop (host side).
//
// The (i-block, j-tile) pairs of every box are laid out in one sequence
// (box-major, then i-block, then j-tile) and cut into G contiguous ranges of
// equal cost, one per persistent CTA.  A CTA emits one partial segment per
// i-block it touches; the integrator sums each block's segments in CTA order.
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
  std::vector<int> cta_tile_begin;  // G + 1
  std::vector<int> cta_block;       // G
  std::vector<int> cta_jt;          // G
  std::vector<int> sys_block_first; // nsys + 1
};

// Builds the schedule for boxes of sizes n[0..nsys).  `tile_overhead` is the
// fixed cost of a tile in units of one j-record (barrier, compensation).
// Returns false on invalid input (n < 1, BI/TILE < 1, G < 1).
bool build_schedule(const int* n, int nsys, int BI, int TILE, int G, int tile_overhead, Schedule* out);

}  // namespace ljgb
