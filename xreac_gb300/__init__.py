"""GB300-native ReaxFF evaluator with xreac's ForceField / Calculator / Evaluation API.

Energies, fixed-charge forces and QEq charges are computed by hand-written sm_103a CUDA kernels
(FP64) behind the C ABI of include/xreac_gb300.h. ``ForceField`` parsing is host-side.
"""

from .forcefield import ForceField

__all__ = ["Calculator", "Evaluation", "ForceField"]


def __getattr__(name):
    # The calculator loads the CUDA library; importing it lazily keeps the parser usable on hosts
    # without the built library (the build step and the CPU test suite).
    if name in ("Calculator", "Evaluation"):
        from . import calculator

        return getattr(calculator, name)
    raise AttributeError(name)
