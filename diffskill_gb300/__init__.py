"""GB300-native (sm_103a) differentiable MLS-MPM substep of DiffSkill's plb/engine.

Public modules:
  config        SimulatorConfig / PrimitiveConfig (the reference's yacs fields)
  engine        MpmEngine (C-ABI handle, batched scenes) and Horizon (checkpointed fwd/bwd)
  scenes        seeded synthetic workloads
The CUDA library is diffskill_gb300/libmpm_gb300.so (C ABI: include/mpm_gb300.h).
"""
__version__ = "0.1.0"
