"""GB300-native spatial-query path of Thea: closest point on a mesh, first ray hit, k nearest neighbours, the LBVH
build and area-weighted mesh sampling, as hand-written sm_103a CUDA behind a C ABI (include/thea_gpu.h), with the
callers next to it (occlusion, Visibility, ShapeDiameter, the sample graph, closest pairs between BVHs) and the OFF,
OBJ and PLY mesh readers."""

from .bvh import (MeshBvh, PointBvh, MeshForest, PointForest, Graph, autotune_batch_closest,  # noqa: F401
                  sample_evenly_by_area, launch_count, profiling, profiling_reset,  # noqa: F401
                  profiling_read, point_gram_tile, random_sphere, sample_graph, write_sample_graph,  # noqa: F401
                  MeshData, read_mesh, triangulate_face, best_fit_sphere, shape_diameter_scale)
from .serve import Server  # noqa: F401
from ._native import TheaError, LIB_PATH  # noqa: F401
