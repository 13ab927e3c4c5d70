"""GB300-native (sm_103a) frame registration + stacking for SerStacker.

The product is ``libsst_gb300.so`` (C ABI, ``include/serstacker_gb300.h``)
built from ``csrc/``; ``capi`` binds it for Python callers and tests.
"""
from . import build  # noqa: F401

__all__ = ["build", "capi", "synth"]
