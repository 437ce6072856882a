"""GB300-native exchange-correlation build for OCC's Kohn-Sham method.

Python mirror of the reference's XC call surface (occpy's Molecule, AOBasis,
DFT; src/python/dft_bindings.cpp:79-118), implemented over the C ABI in
include/occ_xc.h.  Every compute call runs the CUDA library; there is no CPU
path.
"""
from .xc import (  # noqa: F401
    FP64,
    MIXED,
    AOBasis,
    Atom,
    Batch,
    BuildSettings,
    DFT,
    Graph,
    GridSettings,
    Molecule,
    SemiNumericalExchange,
    Server,
    Shell,
    XCError,
    capture_scf_graph,
    library,
    library_path,
    molecular_grid,
    set_persistent_ctas,
)
