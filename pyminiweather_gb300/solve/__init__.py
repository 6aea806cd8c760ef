from .interpolate import (  # noqa: F401
    compute_flux_x,
    compute_flux_z,
    compute_tend_x,
    compute_tend_z,
    interpolate_x,
    interpolate_z,
)
from .source import add_source_terms  # noqa: F401
from .step import discrete_step, evolve, evolve_host, reset_direction  # noqa: F401
