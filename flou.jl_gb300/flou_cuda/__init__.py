"""flou_cuda: Flou.jl's DGSEM residual and explicit Runge-Kutta stepping on GB300 (sm_103a, FP64).

The Python side mirrors Flou's set-up API (CartesianMesh, apply_periodicBCs!, LagrangeBasis,
DGSEMrec, StdSegment/StdQuad/StdHex, equations, fluxes, operators, MultielementDisc,
EquationConfig, rhs!, timeintegrate, get_max_dt); all arithmetic runs in libflou_cuda.
"""
from ._lib import DomainError, FlouError, load
from .disc import Context, DofHandler, EquationConfig, MultielementDisc, get_max_dt, rhs_
from .equations import (BurgersEquation, ChandrasekharAverage, DirichletBC, EulerEquation, EulerInflowBC,
                        EulerOutflowBC, EulerSlipBC, GenericBC, HLL, HLLC, HybridDivOperator, KennedyGruberAverage, LinearAdvection, LxF,
                        MatrixDissipation, OutflowBC, ScalarDissipation, SplitDivOperator, StdAverage,
                        StrongDivOperator)
from .mesh import CartesianMesh, apply_periodicBCs
from .unstructured import UnstructuredMesh, perturbed_box, read_gmsh, write_gmsh22
from .std import DGSEMrec, LagrangeBasis, StdHex, StdQuad, StdSegment, VCJHrec
from .timeint import (ORK256, SSPRK33, CarpenterKennedy2N54, LowStorageRK2N, get_cfl_callback, get_limiter_callback,
                      get_monitor_callback, get_save_callback, make_callback_list, timeintegrate)
from . import initial
from .io import load_restart, save_restart, variablenames, write_vtkhdf, write_vtu
from .batch import Batch, adjoint_solve_batch

rhs = rhs_
