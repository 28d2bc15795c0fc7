"""``jax.scipy`` stand-in (NumPy/SciPy backed); see ``jax/__init__.py``."""

import scipy.special as special  # noqa: F401
