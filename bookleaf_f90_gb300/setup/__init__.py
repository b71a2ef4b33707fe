"""Host-side set-up: control-file reader, mesh generator, initial conditions.

Everything here runs once before the hot path, on the host, exactly as the
reference's own set-up does (src/packages/setup, src/packages/init).
"""
from .problem import Problem  # noqa: F401
from . import configs  # noqa: F401
