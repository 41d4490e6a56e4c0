"""piquasso_gb300 — a GB300-native (sm_103a) engine for piquasso's permanent hot path.

Public API (drop-in for ``piquasso._math.permanent``):
    permanent(matrix, rows, cols)
    permanent_laplace(matrix, rows, cols)
plus the additive ``permanent_batch``, ``permanent_grad`` and the connector in
``piquasso_gb300.connector``; the samplers (exact, lossy, partially
distinguishable, postselected through ``piquasso_gb300.postselect``) in
``piquasso_gb300.sampling``, batched detection
probabilities and LXEB scoring in ``piquasso_gb300.probabilities``, and the
learned-proposal Metropolis sampler in ``piquasso_gb300.metropolis``.
"""

from .permanent import (  # noqa: F401
    PermanentInputError,
    PermanentTooLarge,
    measure_vector_peaks,
    permanent,
    permanent_batch,
    permanent_dd,
    permanent_grad,
    permanent_laplace,
    permanent_laplace_batch,
    sampler_step_batch,
)
from .plan import PermanentPlan  # noqa: F401
from .postselect import InvalidSimulation  # noqa: F401
from ._lib import EngineUnavailable, get_tuning, kernel_launches, last_timing, set_tuning  # noqa: F401

__version__ = "0.1.0"
