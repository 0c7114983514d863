// Kernel instantiations for uint64_t keys (see heap_launch.cuh).
#include <type_traits>
#define GH_INSTANTIATE 1
#include "heap_launch.cuh"

namespace gh {
namespace impl {
GH_INSTANTIATE_KEY(uint64_t)
}  // namespace impl
}  // namespace gh
