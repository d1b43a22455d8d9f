"""GB300 (sm_103a) implementation of the pairwise-interaction hot path of
raven91/spssLangevinIntegration, behind its ParticleSystem / Stepper /
Observer interface.

The compute lives in ``libspss_gpu.so`` (C ABI in ``include/spss_gpu.h``);
``Context`` is the Python handle on one context, ``Batch`` on a batch of
independent systems stepped together.  There is no CPU fallback.
"""
from . import _native
from ._native import (ALL_PAIRS, GLOBAL_FIELD, LINKED_LIST, LINKED_LIST_VERLET, PRECISION_F32, PRECISION_F64, RK4,
                      STOCHASTIC_EULER, STOCHASTIC_RUNGE_KUTTA, VARIANT_DISPATCH, VERLET, SpssError)
from .context import Batch, Context, PinnedArray, make_params

__all__ = [
    "Context", "Batch", "PinnedArray", "make_params", "SpssError", "VARIANT_DISPATCH", "ALL_PAIRS", "LINKED_LIST", "VERLET", "LINKED_LIST_VERLET",
    "GLOBAL_FIELD", "PRECISION_F64", "PRECISION_F32", "RK4", "STOCHASTIC_EULER", "STOCHASTIC_RUNGE_KUTTA",
]
