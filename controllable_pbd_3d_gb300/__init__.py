"""GB300 (sm_103a) implementation of the MGPBD global XPBD step of
JamesYang-7/Controllable_PBD_3D, behind the reference's Python interface,
with the comparison solvers of its convergence experiments (local XPBD
`Deform3D`, `VBDSolver`) and the greedy colourings they run on, and a
learned coarse correction for its multigrid PCG (`CoarseNet`).

The compute runs in libmgpbd.so (hand-written CUDA + C++); this package
is the ctypes binding and the Python mirrors of the reference classes.
"""

from .adaptive import AdaptiveZone, MGPBDAdaptiveSolver  # noqa: F401
from .batch import Body, BodyBatch  # noqa: F401
from .deform3d import Deform3D  # noqa: F401
from .framework import MGPBDConstraint, PbdFramework  # noqa: F401
from .learned import CoarseGraph, CoarseNet  # noqa: F401
from .graph_coloring import ColoringResult, color_edges, color_elements, color_vertices  # noqa: F401
from .mgpbd_gpu import MGPBDSolverGPU  # noqa: F401
from .solver_benchmark import SolverBenchmark  # noqa: F401
from .tet_data import TetData, load_tets  # noqa: F401
from .vbd import VBDSolver  # noqa: F401

__all__ = ['MGPBDSolverGPU', 'SolverBenchmark', 'MGPBDConstraint', 'PbdFramework', 'Body',
           'BodyBatch', 'AdaptiveZone', 'MGPBDAdaptiveSolver', 'Deform3D', 'VBDSolver',
           'ColoringResult', 'color_edges', 'color_elements', 'color_vertices', 'CoarseNet',
           'CoarseGraph', 'TetData', 'load_tets']
