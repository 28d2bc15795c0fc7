"""pyshocks_gb300: the 1D conservation-law hot path of pyshocks on GB300.

The public names mirror ``pyshocks`` (``src/pyshocks/__init__.py``) for the
path that runs here: grids, the scheme/boundary generics, the WENO-JS53 and
ES-WENO32 reconstructions, the Rusanov / Lax-Friedrichs / ES-WENO schemes,
SSPRK33 stepping and the adjoint. Compute runs in ``libshocks.so``
(hand-written sm_103a kernels, C ABI in ``include/shocks.h``); there is no CPU
fallback.
"""

from pyshocks_gb300.grid import (
    Grid,
    Quadrature,
    UniformGrid,
    cell_average,
    make_leggauss_quadrature,
    make_uniform_cell_grid,
    norm,
    rnorm,
)
from pyshocks_gb300.schemes import (
    Boundary,
    BoundaryType,
    ConservationLawScheme,
    FiniteVolumeSchemeBase,
    SchemeBase,
    SchemeT,
    apply_boundary,
    apply_operator,
    bind,
    evaluate_boundary,
    flux,
    numerical_flux,
    predict_timestep,
)
from pyshocks_gb300 import burgers, reconstruction, scalar, timestepping  # noqa: E402

__version__ = "0.1.0"

__all__ = (
    "Boundary",
    "BoundaryType",
    "ConservationLawScheme",
    "FiniteVolumeSchemeBase",
    "Grid",
    "Quadrature",
    "SchemeBase",
    "SchemeT",
    "UniformGrid",
    "apply_boundary",
    "apply_operator",
    "bind",
    "burgers",
    "cell_average",
    "evaluate_boundary",
    "flux",
    "make_leggauss_quadrature",
    "make_uniform_cell_grid",
    "norm",
    "numerical_flux",
    "predict_timestep",
    "reconstruction",
    "rnorm",
    "scalar",
    "timestepping",
)
