// The search kernel for the top-down layout (both block sizes, both
// merge widths), compiled in a unit of its own so that the two layouts
// build in parallel.
#include "search_kernels.cuh"

namespace gh {
namespace search {

cudaError_t search_launch_topdown(const SearchConfig& c, const SearchArgs& a, int grid, cudaStream_t s) {
    return launch_layout<gh::kTopDown>(c, a, grid, s);
}

int search_blocks_per_sm_topdown(const SearchConfig& c) { return blocks_per_sm_layout<gh::kTopDown>(c); }

}  // namespace search
}  // namespace gh
