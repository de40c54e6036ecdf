"""GB300-native KillingFusion registration loop.

The hot path of saurabheights/KillingFusion -- projective TSDF integration,
the gradient-descent update of the displacement field psi (data, level-set and
Killing energies), warped weighted fusion and marching cubes -- as hand-written
sm_103a CUDA behind a C ABI (``include/killingfusion.h``), with C++ host
classes that keep the reference's names and call shapes
(``killingfusion_gb300/csrc/host``).

This Python package is a thin binding of the C ABI (``capi``), a frame loop
that keeps two frames in flight on CUDA streams (``pipeline``) and the
synthetic workload generators (``synth``).  The CUDA library must be built
first (``__graft_entry__.build()``); nothing here falls back to CPU code.
"""
from . import synth  # noqa: F401

__all__ = ["capi", "pipeline", "synth"]
