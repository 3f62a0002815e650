"""gaugefields.jl_gb300 -- GB300 (sm_103a) backend for the SU(3) gauge-link hot
path of Gaugefields.jl: staples and plaquettes, the quenched-HMC force and
link/momentum updates, stout smearing (forward and adjoint) and the RK3
Wilson flow, behind the C-ABI library libgfgb300.so.

The directory name is not a Python identifier; load it by path, e.g.
``__graft_entry__.load_package()``, which registers it as ``gaugefields_gb300``.
"""
from . import _lib
from .api import *  # noqa: F401,F403
from .api import Gaugefields4D, TAGaugefields4D, MDDriver, MDResult, HMCResult  # noqa: F401


def build(force=False, verbose=False):
    from . import _nvcc_build as _build
    return _build.build(force=force, verbose=verbose)


def library():
    """The loaded libgfgb300.so (raises when absent: there is no CPU path)."""
    return _lib.load()
