"""exponax_gb300 -- the ETDRK pseudo-spectral stepping path of exponax,
rebuilt for NVIDIA GB300 (sm_103a).

Drop-in surface for the reference's hot path: ``stepper.*`` (``__call__``,
``step``, ``step_fourier``), ``etdrk.ETDRK0..4``, ``nonlin_fun.*``,
``rollout``, ``repeat``, ``RepeatedStepper``, ``spectral.fft/ifft`` and
``map_between_resolutions``.  All stepping runs in libexgb.so (hand-written
CUDA, C ABI in include/exgb.h); there is no CPU fallback.
"""

from . import etdrk, graphs, ic, metrics, nonlin_fun, poisson, spectral, stepper
from ._lib import ExgbError
from ._utils import (ForcedStepper, RepeatedStepper, make_grid, repeat, rollout, stack_sub_trajectories, vmap,
                     wrap_bc)
from .ic import build_ic_set
from .interpolation import FourierInterpolator, map_between_resolutions
from .metrics import get_spectrum
from .spectral import derivative, fft, ifft
from .stepper import BaseStepper

__version__ = "0.1.0"

__all__ = [
    "BaseStepper",
    "ExgbError",
    "ForcedStepper",
    "FourierInterpolator",
    "RepeatedStepper",
    "build_ic_set",
    "derivative",
    "etdrk",
    "fft",
    "get_spectrum",
    "graphs",
    "ic",
    "ifft",
    "make_grid",
    "map_between_resolutions",
    "metrics",
    "nonlin_fun",
    "poisson",
    "repeat",
    "rollout",
    "spectral",
    "stack_sub_trajectories",
    "stepper",
    "vmap",
    "wrap_bc",
]
