"""GB300 (sm_103a) backend `b200` of the sosfuse2 successive-orders-of-scattering source iteration.

`Kernel` and `Solver` (sosfuse2_gb300.solver) mirror the reference's `source_solver.Kernel` and
`source_iteration.Solver` over the C ABI of libsosb (include/sosb.h); `PackedState` (sosfuse2_gb300.state) carries
one state's constants and ray bundles.
"""

__version__ = '0.1.0'

from .state import PackedState  # noqa: F401


def Solver(*args, **kwargs):
    from .solver import Solver as _Solver

    return _Solver(*args, **kwargs)


def Kernel(*args, **kwargs):
    from .solver import Kernel as _Kernel

    return _Kernel(*args, **kwargs)
