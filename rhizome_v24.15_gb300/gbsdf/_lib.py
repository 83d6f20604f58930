"""ctypes binding of libgbsdf.so (the C ABI declared in include/gbsdf.h).

Loading fails loudly when the CUDA library has not been built: there is no CPU
fallback anywhere in this package.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libgbsdf.so"

# gbsdf_status
OK, EINVAL, EGUARD, ECSR, EVERIFY, ENOMEM, ECUDA, ENODEV = range(8)
STATUS_NAMES = {OK: "OK", EINVAL: "EINVAL", EGUARD: "EGUARD", ECSR: "ECSR", EVERIFY: "EVERIFY",
                ENOMEM: "ENOMEM", ECUDA: "ECUDA", ENODEV: "ENODEV"}
# gbsdf_mode / gbsdf_path
MODE_REFERENCE, MODE_EXACT, MODE_EXACT_SIGNS, MODE_LEARNED = 0, 1, 2, 3
PATH_AUTO, PATH_FAST, PATH_LEGACY = 0, 1, 2


class Options(C.Structure):
    _fields_ = [("mode", C.c_int32), ("path", C.c_int32), ("device", C.c_int32), ("tris_on_device", C.c_int32),
                ("max_rounds", C.c_int32), ("mlp_budget", C.c_int32), ("mlp_threshold", C.c_float),
                ("wait_poll_limit", C.c_int32), ("mlp_params", C.c_void_p), ("brick_scores", C.c_void_p),
                ("sweep_schedule", C.c_int32), ("host_output", C.c_int32),
                ("winding_eval", C.c_int32), ("splat_dense_cut", C.c_int32)]


MLP_PARAMS, MLP_FEATURES = 6337, 32


class Stats(C.Structure):
    _fields_ = [("status", C.c_int32), ("path_taken", C.c_int32), ("ms_total", C.c_float),
                ("ms_h2d", C.c_float), ("ms_prep", C.c_float), ("ms_splat", C.c_float), ("ms_parity", C.c_float),
                ("ms_fixup", C.c_float), ("ms_eikonal", C.c_float), ("ms_verify", C.c_float),
                ("ms_apply", C.c_float), ("ms_d2h", C.c_float),
                ("eikonal_rounds", C.c_int32), ("extra_rounds", C.c_int32), ("probes", C.c_int32),
                ("sites", C.c_int32), ("patch_rounds", C.c_int32), ("splat_dense_cut", C.c_int32),
                ("unknown_columns", C.c_int64), ("fixup_voxels", C.c_int64), ("far_residual", C.c_int64),
                ("safe_clamped", C.c_int64), ("patched_voxels", C.c_int64), ("fp64_rechecks", C.c_int64),
                ("band_voxels", C.c_int64), ("splat_evals", C.c_int64), ("gwn_pairs", C.c_int64),
                ("brick_pairs", C.c_int64), ("csr_entries", C.c_int64), ("kernel_launches", C.c_int64),
                ("proposed", C.c_int64), ("sweep_schedule", C.c_int64), ("winding_certified", C.c_int64),
                ("winding_summed", C.c_int64), ("escalated", C.c_int64), ("band_err_fp64", C.c_double),
                ("band_err_samples", C.c_int64), ("ms_sweeps", C.c_float), ("sweep_schedule_first", C.c_int32)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class MeshDesc(C.Structure):
    _fields_ = [("tris", C.c_void_p), ("n_tris", C.c_int64), ("voxel_size", C.c_float),
                ("min_coord", C.c_int32 * 3), ("max_coord", C.c_int32 * 3), ("out", C.c_void_p),
                ("status", C.c_int32), ("pad", C.c_int32)]


# every exported symbol of include/gbsdf.h
EXPORTS = ("gbsdf_default_options", "gbsdf_compute_mesh_sdf", "gbsdf_compute_mesh_sdf_batch",
           "gbsdf_mesh_lattice", "gbsdf_build_from_mesh",
           "gbsdf_brick_features", "gbsdf_mlp_forward", "gbsdf_mlp_backward", "gbsdf_mlp_adam",
           "gbsdf_batch_create", "gbsdf_batch_run", "gbsdf_batch_destroy", "gbsdf_parse_binary_stl", "gbsdf_parse_obj",
           "gbsdf_ascii_stl_capacity", "gbsdf_parse_ascii_stl", "gbsdf_orient_mesh",
           "gbsdf_extract_iso_surface", "gbsdf_extract_iso_surface_device", "gbsdf_iso_surface_table",
           "gbsdf_interior_volume", "gbsdf_find_default_seed",
           "gbsdf_release_workspace", "gbsdf_legacy_sdf_noalloc", "gbsdf_selftest", "gbsdf_version")

_lib = None


def load(path: Path | None = None):
    """Load libgbsdf.so (raises if it is missing: build it with __graft_entry__.build())."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise ImportError(f"{p} is missing: the CUDA engine has not been built (run __graft_entry__.build())")
    L = C.CDLL(str(p))
    i32p = C.POINTER(C.c_int32)
    L.gbsdf_default_options.argtypes = [C.POINTER(Options)]
    L.gbsdf_default_options.restype = None
    L.gbsdf_compute_mesh_sdf.argtypes = [C.c_void_p, C.c_int64, C.c_float, i32p, i32p, C.c_void_p, C.c_int32,
                                         C.POINTER(Options), C.POINTER(Stats), C.c_char_p, C.c_size_t]
    L.gbsdf_compute_mesh_sdf.restype = C.c_int
    L.gbsdf_compute_mesh_sdf_batch.argtypes = [C.POINTER(MeshDesc), C.c_int32, C.c_int32, C.POINTER(Options),
                                               C.POINTER(Stats), C.c_char_p, C.c_size_t]
    L.gbsdf_compute_mesh_sdf_batch.restype = C.c_int
    L.gbsdf_mesh_lattice.argtypes = [C.c_void_p, C.c_int64, C.c_float, i32p, i32p, C.c_char_p, C.c_size_t]
    L.gbsdf_mesh_lattice.restype = C.c_int
    L.gbsdf_build_from_mesh.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_float, i32p, i32p,
                                        C.c_void_p, C.c_int32, C.POINTER(Options), C.POINTER(Stats), C.c_char_p,
                                        C.c_size_t]
    L.gbsdf_build_from_mesh.restype = C.c_int
    L.gbsdf_brick_features.argtypes = [C.c_void_p, C.c_int64, C.c_float, i32p, i32p, C.c_int32, C.c_void_p,
                                       C.c_int64, i32p, C.c_char_p, C.c_size_t]
    L.gbsdf_brick_features.restype = C.c_int
    L.gbsdf_mlp_forward.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_int32, C.c_char_p,
                                    C.c_size_t]
    L.gbsdf_mlp_forward.restype = C.c_int
    L.gbsdf_mlp_backward.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p,
                                     C.c_void_p, C.c_int32, C.c_char_p, C.c_size_t]
    L.gbsdf_mlp_backward.restype = C.c_int
    L.gbsdf_mlp_adam.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_float, C.c_float, C.c_float,
                                 C.c_float, C.c_float, C.c_int32, C.c_int32, C.c_char_p, C.c_size_t]
    L.gbsdf_mlp_adam.restype = C.c_int
    L.gbsdf_batch_create.argtypes = [C.POINTER(MeshDesc), C.c_int32, C.c_int32, C.POINTER(Options),
                                     C.POINTER(C.c_void_p), C.c_char_p, C.c_size_t]
    L.gbsdf_batch_create.restype = C.c_int
    L.gbsdf_batch_run.argtypes = [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(Stats), C.c_char_p, C.c_size_t]
    L.gbsdf_batch_run.restype = C.c_int
    L.gbsdf_batch_destroy.argtypes = [C.c_void_p]
    L.gbsdf_batch_destroy.restype = None
    i64p = C.POINTER(C.c_int64)
    L.gbsdf_parse_binary_stl.argtypes = [C.c_void_p, C.c_size_t, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64,
                                         C.c_void_p, i64p, i64p, C.c_int32, C.c_char_p, C.c_size_t]
    L.gbsdf_parse_binary_stl.restype = C.c_int
    L.gbsdf_parse_obj.argtypes = [C.c_void_p, C.c_size_t, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, i64p, i64p,
                                  C.c_int32, C.c_char_p, C.c_size_t]
    L.gbsdf_parse_obj.restype = C.c_int
    L.gbsdf_ascii_stl_capacity.argtypes = [C.c_size_t, i64p]
    L.gbsdf_ascii_stl_capacity.restype = C.c_int
    L.gbsdf_parse_ascii_stl.argtypes = [C.c_void_p, C.c_size_t, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, i64p,
                                        i64p, C.c_int32, C.c_char_p, C.c_size_t]
    L.gbsdf_parse_ascii_stl.restype = C.c_int
    L.gbsdf_orient_mesh.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, i32p, i32p, i32p,
                                    C.POINTER(C.c_double), C.c_int32, C.c_char_p, C.c_size_t]
    L.gbsdf_orient_mesh.restype = C.c_int
    L.gbsdf_extract_iso_surface.argtypes = [C.c_void_p, C.c_int32, i32p, C.c_float, C.POINTER(C.c_float), C.c_float,
                                            C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_int32, i64p, i64p,
                                            C.c_int32, C.c_char_p, C.c_size_t]
    L.gbsdf_extract_iso_surface.restype = C.c_int
    L.gbsdf_extract_iso_surface_device.argtypes = [C.c_void_p, C.c_int32, i32p, C.c_float, C.POINTER(C.c_float),
                                                   C.c_float, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), i64p, i64p,
                                                   C.c_int32, C.c_char_p, C.c_size_t]
    L.gbsdf_extract_iso_surface_device.restype = C.c_int
    f3p = C.POINTER(C.c_float)
    L.gbsdf_interior_volume.argtypes = [C.c_void_p, C.c_int32, C.c_int64, C.c_float, f3p, i64p, C.c_int32,
                                        C.c_char_p, C.c_size_t]
    L.gbsdf_interior_volume.restype = C.c_int
    L.gbsdf_find_default_seed.argtypes = [C.c_void_p, C.c_int32, i32p, i32p, C.c_float, f3p, f3p, C.c_float, f3p,
                                          C.c_int32, C.c_char_p, C.c_size_t]
    L.gbsdf_find_default_seed.restype = C.c_int
    L.gbsdf_iso_surface_table.argtypes = [C.c_void_p]
    L.gbsdf_iso_surface_table.restype = C.c_int
    L.gbsdf_release_workspace.argtypes = [C.c_int32]
    L.gbsdf_release_workspace.restype = None
    L.gbsdf_legacy_sdf_noalloc.argtypes = [C.c_void_p, C.c_int64, C.c_float, i32p, i32p, C.c_void_p, C.c_int32,
                                           C.c_void_p, C.POINTER(Stats), C.c_char_p, C.c_size_t]
    L.gbsdf_legacy_sdf_noalloc.restype = C.c_int
    L.gbsdf_selftest.argtypes = [C.c_int32, C.c_int32, C.POINTER(C.c_uint64), C.c_char_p, C.c_size_t]
    L.gbsdf_selftest.restype = C.c_int
    L.gbsdf_version.argtypes = []
    L.gbsdf_version.restype = C.c_char_p
    if path is None:
        _lib = L
    return L
