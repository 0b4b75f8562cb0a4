"""CPU oracle of the particle-mesh hot path -- test infrastructure only.

Imported by tests/, __graft_entry__.smoke() and bench.py's CPU baseline / reference
arm.  The product (the CUDA library and pmgpu/) never imports it.
"""
