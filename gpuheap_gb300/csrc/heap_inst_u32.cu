// Kernel instantiations for uint32_t keys (see heap_launch.cuh).
#include <type_traits>
#define GH_INSTANTIATE 1
#include "heap_launch.cuh"

namespace gh {
namespace impl {
GH_INSTANTIATE_KEY(uint32_t)
}  // namespace impl
}  // namespace gh
