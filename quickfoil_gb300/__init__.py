"""GB300-native engine for QuickFOIL's candidate-literal evaluation.

The work runs in ``libqfgpu.so`` (hand-written sm_103a CUDA kernels behind the
C ABI of ``include/qfgpu.h``); this package is the host-side mirror of the
reference's operator interface plus data generators for the benchmark
workloads.
"""
from ._capi import QfgError, load as load_library, library_path  # noqa: F401
from .engine import (BindingSet, CandidateLiteralEvaluator, CandidateLiteralInfo, Engine,  # noqa: F401
                     Literal, join_key)


def build(force: bool = False) -> str:
    """Compiles libqfgpu.so in-tree for sm_103a."""
    from . import _build
    return _build.build(force=force)
