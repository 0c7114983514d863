// C entry point around the reference's sequential A*
// (artifacts/astar/seq_astar.hpp: SeqAstarSearch), compiled for the host
// from the reference tree.
//
// TEST INFRASTRUCTURE ONLY (builds into oracle/_ref/, never shipped).
//   ra_seq_astar(map, h, w)  SeqAstarSearch on a bitmap of h x w cells
#include <cstdint>
#include <queue>
#include <vector>

using std::priority_queue;
using std::vector;

#include "seq_astar.hpp"

extern "C" uint32_t ra_seq_astar(uint32_t* map, uint32_t h, uint32_t w) { return seq_astar::SeqAstarSearch(map, h, w); }
