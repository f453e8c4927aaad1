// The reference-order BCP kernel with a 256-entry window (8 warps per
// trail block, 2 blocks per SM).
#define GPSAT_BCP_WARPS 8
#define GPSAT_BCP_MIN_BLOCKS 2
#define GPSAT_BCP_NS w8
#include "bcp_window.cuh"

namespace gpsat {
namespace bcp {
extern const Variant variant_w8 = {8, w8::launch, w8::occupancy};
}  // namespace bcp
}  // namespace gpsat
