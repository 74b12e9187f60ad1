"""Solvers of the Warp emulation (test infrastructure)."""

from . import linear  # noqa: F401
