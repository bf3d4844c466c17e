"""GB300 (sm_103a) HII-bubble filter bank of SimFast21's get_HIIbubbles stage.

The compute lives in libsf21hii.so (C-ABI: include/sf21_hii.h); this package
holds its build recipe, a Python mirror of the stage's host interface over
that ABI (``hii.FilterBank``), the reference's parameter semantics
(``params``) and the seeded synthetic input generator (``synth``).
"""
from . import params, synth  # noqa: F401

__all__ = ["params", "synth", "hii", "build"]
