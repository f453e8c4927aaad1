// The reference-order BCP kernel with a 64-entry window (2 warps per
// trail block, 8 blocks per SM).
#define GPSAT_BCP_WARPS 2
#define GPSAT_BCP_MIN_BLOCKS 8
#define GPSAT_BCP_NS w2
#include "bcp_window.cuh"

namespace gpsat {
namespace bcp {
extern const Variant variant_w2 = {2, w2::launch, w2::occupancy};
}  // namespace bcp
}  // namespace gpsat
