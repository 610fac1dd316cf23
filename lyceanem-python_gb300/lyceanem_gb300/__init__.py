"""GB300-native raycasting + frequency-domain propagation (LyceanEM hot path).

Subpackages mirror the reference's interface:
  lyceanem_gb300.em                                  drop-in for lyceanem.em
  lyceanem_gb300.models.acceleration_structures      Tile / Brute_Force structures
  lyceanem_gb300.models.frequency_domain             calculate_scattering / calculate_farfield
  lyceanem_gb300.propagation                         torch-level device API
All compute runs in liblyem_gpu.so (hand-written sm_103a CUDA); importing the
compute modules fails if the library is not built.
"""
__version__ = "0.1.0"
