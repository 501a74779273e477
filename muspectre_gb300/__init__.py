"""GB300-native µSpectre Newton-CG homogenization (sm_103a CUDA behind µSpectre's API).

Drop-in for the reference ``muSpectre`` Python package on its Newton-CG path::

    import muspectre_gb300 as µ
    rve = µ.SystemFactory([51, 51], [7., 5.], µ.Formulation.small_strain)
    hard = µ.material.MaterialLinearElastic1_2d.make(rve, "hard", 10e9, .33)
    ...
    solver = µ.solvers.SolverCG(rve, 1e-8, 401)
    r = µ.solvers.newton_cg(rve, Del0, solver, 1e-5, 2)

Everything runs on the GPU through ``libmusg.so`` (C ABI in ``include/musg.h``);
there is no CPU fallback.
"""
from . import batch, fft, material, solvers  # noqa: F401
from ._lib import ConvergenceError, CudaError, ProjectionError, SolverError, device_count, selftest_wait_timeout  # noqa: F401
from .cell import (Cell, CellBase, CellBase2d, CellBase3d, CellFactory, Communicator, FFT_PlanFlags, Formulation,  # noqa: F401
                   SystemFactory, get_domain_ccoord, get_domain_index, get_hermitian_sizes)

__version__ = '0.1.0'
