"""FP64 CPU oracle (test infrastructure only; see oracle/oracle.py)."""
from .oracle import *  # noqa: F401,F403
from . import oracle as _impl  # noqa: F401
