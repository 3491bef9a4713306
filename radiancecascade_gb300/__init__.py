"""GB300-native radiance-cascade global illumination.

The compute path is librc.so (hand-written sm_103a CUDA behind the C ABI of
include/rc.h); this package is its Python host side.  Importing it loads the
library and raises ImportError when it has not been built -- there is no CPU
fallback.
"""
from ._ffi import lib as _load_lib, RCError, VOXEL_DT, BOX_DT, SPHERE_DT  # noqa: F401
from .engine import (Engine, Batch, GiStage, GiState, make_params, level_info, scene_spec, generate_scene,  # noqa: F401
                     advance_spheres, voxelise_host, directions, solid_angles, WORKLOADS, workload_scene,
                     batch_workload, BATCH_EDGES, BATCH_CASCADES, load_obj, mesh_to_grid, mesh_materials,
                     room_mesh, camera_view_proj, shade_vertices, shade_material, mesh_tbn,
                     frames, FrameLog)

_load_lib()
