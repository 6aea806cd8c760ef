from .stats import compute_solution_variables, compute_stats, compute_stats_device, count_nonfinite  # noqa: F401
