"""GB300-native (sm_103a) reionization grid step of Meraxes.

find_HII_bubbles, ComputeTs and the 21 cm brightness-temperature box behind the
reference's entry points and grid layouts; see include/mx_reion.h for the C ABI.
"""
from .params import ReionParams, Workload, workload  # noqa: F401

__all__ = ["ReionParams", "Workload", "workload", "ReionGridStep"]


def __getattr__(name):
    if name == "ReionGridStep":
        from .api import ReionGridStep

        return ReionGridStep
    raise AttributeError(name)
