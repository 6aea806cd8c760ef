"""CPU oracle for the PyMiniWeather time step (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may use
this package; the product path in pyminiweather_gb300 never imports it.
"""
