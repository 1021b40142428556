// The batched IC-GN kernel for teams of 4 warps (set-up, iterations and the
// fused 2-DOF form), in a translation unit of its own so that the team
// widths compile in parallel.
#include "icgn_batched.cuh"

namespace stdic {

STDIC_BATCHED_TEAM_WIDTH(4)

}  // namespace stdic
