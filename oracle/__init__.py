"""CPU oracle of the voxel cone tracing path -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this package.  The CUDA product library (vk_voxel_cone_tracing_gb300) never
imports, links or executes it.
"""
