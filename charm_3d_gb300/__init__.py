"""GB300-native DG time step of CHARM_3D (Euler / multicomponent NS, p1 Taylor basis).

The compute path is libcharm_gpu.so (hand-written sm_103a CUDA behind the
C ABI in include/charm_gpu.h).  This package only loads it and mirrors the
reference's host interface: cases, the CPU octree, and the solver handle.
"""
from .case import Boundary, Case, Component, Reaction, synthetic  # noqa: F401

__all__ = ["Boundary", "Case", "Component", "synthetic"]
