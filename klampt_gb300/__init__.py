"""klampt_gb300 — GB300-native batched configuration-validity and proximity
engine for Klamp't robots (forward kinematics, environment/self collision,
planner edge checks, signed distance and its gradient).

The compute path is libkgpu.so (hand-written CUDA for sm_103a behind the C
ABI of include/kgpu.h).  Nothing here falls back to a CPU implementation: a
missing library raises on first use.
"""

__version__ = "0.1.0"

__all__ = ["build", "scenes", "engine", "klampt"]
