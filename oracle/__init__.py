"""CPU oracle for the batched TR-BDF2 box-model time advance (test infrastructure only).

Only the tests, the smoke check and bench.py's CPU-baseline leg use this package; the engine
never does.
"""
from .binding import AerosolOracle, E3smOracle, Oracle, load, lu_factor_blocked  # noqa: F401
