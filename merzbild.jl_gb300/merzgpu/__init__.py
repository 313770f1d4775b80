"""merzgpu: GB300-native implementation of Merzbild.jl's per-step DSMC hot path.

The compute path is libmerzgpu.so (hand-written sm_103a CUDA behind a C ABI,
include/merzgpu.h); this package is the host-side mirror of the reference's
interface.  There is no CPU fallback: every operation runs in the library.
"""
from ._lib import MerzError, exported_symbols, lib  # noqa: F401
from .api import *  # noqa: F401,F403
from .gas import AR_MASS, HE_MASS, PSEUDO_MAXWELL, VHS  # noqa: F401
from .ncio import *  # noqa: F401,F403

__all__ = [n for n in dir() if not n.startswith("_")]
