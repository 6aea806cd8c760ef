from .stats import compute_solution_variables, compute_stats, compute_stats_device  # noqa: F401
