"""gbsdf -- GB300-native mesh-to-signed-distance-field engine.

Drop-in for the "Fast SDF" path of golemid/rhizome_v24.15
(``CudaRasterizer::compute_mesh_sdf`` / ``build_from_mesh``), implemented as
hand-written sm_103a CUDA kernels behind a C ABI (include/gbsdf.h).
"""
from . import meshgen
from ._lib import LIB_PATH, load
from .api import (MODE_EXACT, MODE_EXACT_SIGNS, MODE_LEARNED, MODE_REFERENCE, PATH_AUTO, PATH_FAST, PATH_LEGACY, Batch,
                  CudaRasterizer, CudaVolumeGrid, GbsdfError, Result, build_from_mesh, compute_mesh_sdf,
                  compute_mesh_sdf_batch, extract_iso_surface, find_default_seed, interior_volume, mesh_lattice, orient_mesh, parse_ascii_stl, parse_binary_stl, parse_obj,
                  parse_stl)

__all__ = ["meshgen", "LIB_PATH", "load", "MODE_EXACT", "MODE_EXACT_SIGNS", "MODE_LEARNED", "MODE_REFERENCE",
           "PATH_AUTO", "PATH_FAST", "PATH_LEGACY", "Batch", "CudaRasterizer", "CudaVolumeGrid", "GbsdfError", "Result",
           "build_from_mesh", "compute_mesh_sdf", "compute_mesh_sdf_batch", "extract_iso_surface", "find_default_seed", "interior_volume", "mesh_lattice", "orient_mesh",
           "parse_ascii_stl", "parse_binary_stl", "parse_obj", "parse_stl"]
