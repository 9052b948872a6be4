"""GB300-native radar-sounder raypath engine (drop-in for the reference's
facet raypath -> phasor binning -> chirp range-compression path).

Python entry points mirror the reference's ``param_gen``, ``simple_surfaces``
and ``output_handling``; ``Scene`` / ``simulate`` run the hand-written sm_103a
kernels of ``libraypath.so`` through its C ABI (``include/raypath.h``).
"""
from . import param_gen, simple_surfaces, output_handling, scenes, traces  # noqa: F401

__all__ = ["param_gen", "simple_surfaces", "output_handling", "scenes", "traces",
           "Scene", "simulate"]


def __getattr__(name):
    if name in ("Scene", "simulate"):
        from . import simulator
        return getattr(simulator, name)
    raise AttributeError(name)
