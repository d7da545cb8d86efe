"""GB300-native Bio-CFD hot path: Python harness over the C ABI.

``biocfd.solver.Solver`` drives ``libbiocfd_gb300.so`` (CUDA, sm_103a) with the
reference driver's set-up and per-step routine sequence; ``biocfd.synth``
builds the seeded synthetic workloads.
"""
from . import synth  # noqa: F401

__all__ = ["synth"]
