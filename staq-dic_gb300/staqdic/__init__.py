"""GB300-native (sm_103a) STAQ-DIC augmented-Lagrangian hot path.

The compute lives in libstaqdic.so (hand-written CUDA behind the C ABI of
include/staqdic.h); this package is the host-side mirror of the reference's
MATLAB interface (``staqdic.api``), plus seeded synthetic workloads.
"""
from ._lib import Context, StdicError, default_context, load  # noqa: F401
from .api import (  # noqa: F401
    GenerateQuadtreeMesh, LocalICGNQuadtree, funPOR_GPR, Subpb1Quadtree, Subpb2Quadtree, ba_interp2, funICGNQuadtree,
    admm, fill_nans, funImgGradient, funIntegerSearch, funIntegerSearchMg, icgn_adjoint, icgn_subsets, icgn_subsets_frames,
    nodal_strain, subpb1_subsets,
)
