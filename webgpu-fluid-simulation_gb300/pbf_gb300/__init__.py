"""GB300-native Position Based Fluids substep (Python side of the C ABI).

`PBF` mirrors the reference simulator's interface; `FilteredParticleFluid`
produces the screen-space depth / thickness buffers of the reference's fluid
renderer; `scenes` builds the reference presets and the benchmark workloads.  All compute runs in
libpbf_gb300.so (CUDA, sm_103a).
"""
from . import _lib
from .simulator import PBF, PBFBatch, NeighborSearch, exclusive_scan, voxelize_mesh_points
from .simulator import mlp_init, mlp_params, mlp_fit_normalization, mlp_forward, mlp_gradient, mlp_train
from .render import FilteredParticleFluid
from . import scenes

__all__ = ["PBF", "PBFBatch", "NeighborSearch", "FilteredParticleFluid", "exclusive_scan", "scenes", "_lib"]
