// The batched IC-GN kernel for teams of 4 warps with the staged g footprint
// (the iterations and the fused 2-DOF form), in a translation unit of its
// own so that the instantiations compile in parallel.
#include "icgn_batched.cuh"

namespace stdic {

STDIC_BATCHED_UNIT(4, true, s)

}  // namespace stdic
