"""topopt.jl_gb300 -- GB300 (sm_103a) drop-in for TopOpt.jl's SIMP compliance loop.

The compute path is libtopopt_gb300.so (hand-written CUDA behind a C ABI,
include/topopt_gb300.h).  This package is its host-side mirror of the
reference's Julia API; the Julia binding lives in julia/TopOptGB300.jl.
Import it as ``topopt_gb300`` (see ``load()`` in the repository's
__graft_entry__.py; the directory name carries a dot).
"""
from ._lib import TopOptError, NotConverged, lib  # noqa: F401
from .vtk import save_mesh  # noqa: F401
from .inp import InpContent, InpStiffness, parse_inp, write_inp  # noqa: F401
from .topopt_api import (  # noqa: F401
    BatchedSIMP,
    BlockComplianceFun,
    ComplianceFun,
    DefaultCriteria,
    DensityFilterFun,
    EnergyCriteria,
    FEASolver,
    FixedElementProjectorFun,
    GB300FEASolver,
    GB300Solver,
    HalfMBB,
    HeavisideProjectionFun,
    LoadedCantilever,
    MeanComplianceFun,
    MultiLoad,
    PointLoadCantilever,
    PowerPenaltyFun,
    ProjectedDensityFilterFun,
    PseudoDensities,
    SensFilterFun,
    SigmoidProjectionFun,
    SIMPLoop,
    VolumeFun,
    WarmStartNet,
    cell_dofs,
    element_stiffness,
    find_nearest_dofs,
    generate_scenarios,
    hadamard,
    hutch_rand,
    get_fixed_element_projector,
    get_free_variable_count,
    get_free_variables,
    grid_counts,
    node_dofs,
    mma_reset,
    mma_update,
    oc_update,
    uneven_cantilever_set,
)
