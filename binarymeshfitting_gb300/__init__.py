"""GB300-native (sm_103a) chunk extraction for BinaryMeshFitting.

The compute path is libbmf_gb300.so (C ABI in include/bmf.h); this package is
the Python host layer over it: ``engine`` (tensors in, tensors out) and
``reference_api`` (the reference's Sampler / DMCChunk / MeshProcessor /
ChunkGenerator call surface).
"""
from ._lib import (BmfError, ChunkDesc, Field, FIELD_GRID, FIELD_SPHERE_WAVE, FIELD_TERRAIN_FBM, FIELD_TERRAIN_2D,
                   FIELD_TORUS_Z,
                   FIELD_SPHERE, FIELD_CUBOID, FIELD_PLANE_Y, MODE_R, MODE_Q, PLACE_CENTER, PLACE_MASSPOINT,
                   PLACE_QEF)

__all__ = ["BmfError", "ChunkDesc", "Field", "FIELD_GRID", "FIELD_SPHERE_WAVE", "FIELD_TERRAIN_FBM", "FIELD_TERRAIN_2D",
           "FIELD_TORUS_Z", "FIELD_SPHERE", "FIELD_CUBOID", "FIELD_PLANE_Y", "MODE_R", "MODE_Q", "PLACE_CENTER",
           "PLACE_MASSPOINT", "PLACE_QEF"]
