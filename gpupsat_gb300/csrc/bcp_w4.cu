// The reference-order BCP kernel with a 128-entry window (4 warps per
// trail block, 4 blocks per SM).
#define GPSAT_BCP_WARPS 4
#define GPSAT_BCP_MIN_BLOCKS 4
#define GPSAT_BCP_NS w4
#include "bcp_window.cuh"

namespace gpsat {
namespace bcp {
extern const Variant variant_w4 = {4, w4::launch, w4::occupancy};
}  // namespace bcp
}  // namespace gpsat
