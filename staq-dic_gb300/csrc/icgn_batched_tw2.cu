// The batched IC-GN kernel for teams of 2 warps without the staged g
// footprint (the set-up, the iterations and the fused 2-DOF form), in a
// translation unit of its own so that the instantiations compile in parallel.
#include "icgn_batched.cuh"

namespace stdic {

STDIC_BATCHED_UNIT(2, false, u)

}  // namespace stdic
