"""Host-side mirror of the reference's CudaRasterizer mesh-to-SDF interface.

Reference (golemid/rhizome_v24.15):
  * ``CudaRasterizer::compute_mesh_sdf`` -- native/src/engine/sdf/cuda_rasterizer.hpp:21-28,
    cuda_rasterizer.cu:1163-1265: ``(triangles, voxel_size, min_coord, max_coord) ->
    bool``, ``out_distances`` resized to N and filled, ``out_time_ms`` set; on failure
    the output is left untouched and ``False`` is returned.
  * ``CudaRasterizer::build_from_mesh`` -- cuda_rasterizer.hpp:31-35,
    cuda_rasterizer.cu:1340-1435: ``(mesh, voxel_size) -> CudaVolumeGrid | nullptr``.
  * ``CudaVolumeGrid`` -- native/src/engine/sdf/cuda_types.hpp:155-175.

Everything runs through the C ABI (include/gbsdf.h) of libgbsdf.so; there is no CPU
path. Triangles are ``(T, 12)`` float32 arrays in the reference's ``CudaTriangle``
layout (v0, v1, v2, normal).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import (MODE_EXACT, MODE_EXACT_SIGNS, MODE_LEARNED, MODE_REFERENCE, PATH_AUTO, PATH_FAST, PATH_LEGACY,
                   STATUS_NAMES)

__all__ = ["GbsdfError", "Result", "Batch", "compute_mesh_sdf", "compute_mesh_sdf_batch", "parse_binary_stl",
           "parse_obj", "orient_mesh", "mesh_lattice", "build_from_mesh", "CudaRasterizer",
           "CudaVolumeGrid", "MODE_REFERENCE", "MODE_EXACT", "MODE_EXACT_SIGNS", "MODE_LEARNED", "PATH_AUTO", "PATH_FAST",
           "PATH_LEGACY"]


class GbsdfError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"gbsdf {STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


@dataclass
class Result:
    status: int
    stats: dict
    message: str = ""

    @property
    def ok(self) -> bool:
        return self.status == _lib.OK


def _i3(v):
    a = (C.c_int32 * 3)(*[int(x) for x in np.asarray(v).reshape(3)])
    return a


def _ptr_of(buf):
    """(address, on_device) of a numpy array or a torch tensor."""
    if isinstance(buf, np.ndarray):
        if not buf.flags["C_CONTIGUOUS"]:
            raise ValueError("buffer must be C-contiguous")
        return buf.ctypes.data, False
    # torch tensor (duck-typed: data_ptr / is_cuda)
    if hasattr(buf, "data_ptr"):
        if not buf.is_contiguous():
            raise ValueError("tensor must be contiguous")
        return buf.data_ptr(), bool(buf.is_cuda)
    raise TypeError(f"unsupported buffer type {type(buf)}")


def _mlp_device_params(mlp_params, device):
    """Device pointer (and the owning tensor) of the learned model's parameters: a CUDA
    tensor is used as is, a host array is copied to ``device``, None loads the model
    shipped with the package."""
    import torch

    if mlp_params is None:
        from .learn import MODEL_PATH
        mlp_params = np.load(MODEL_PATH)["params"]
    if not isinstance(mlp_params, torch.Tensor):
        mlp_params = torch.from_numpy(np.ascontiguousarray(mlp_params, np.float32)).to(f"cuda:{device}")
    if not mlp_params.is_cuda or mlp_params.dtype != torch.float32 or mlp_params.numel() != _lib.MLP_PARAMS:
        raise ValueError(f"mlp_params must be {_lib.MLP_PARAMS} float32 values")
    mlp_params = mlp_params.contiguous()
    return mlp_params.data_ptr(), mlp_params


def _set_learned(o, mode, device, mlp_params, mlp_budget, mlp_threshold, brick_scores=None):
    if int(mode) != MODE_LEARNED:
        return None
    if brick_scores is not None:
        import torch

        if not isinstance(brick_scores, torch.Tensor):
            brick_scores = torch.from_numpy(np.ascontiguousarray(brick_scores, np.float32)).to(f"cuda:{device}")
        if not brick_scores.is_cuda or brick_scores.dtype != torch.float32:
            raise ValueError("brick_scores must be float32")
        keep = brick_scores.contiguous()
        o.brick_scores = keep.data_ptr()
    else:
        ptr, keep = _mlp_device_params(mlp_params, device)
        o.mlp_params = ptr
    if mlp_budget is not None:
        o.mlp_budget = int(mlp_budget)
    if mlp_threshold is not None:
        o.mlp_threshold = float(mlp_threshold)
    return keep


def compute_mesh_sdf(tris, voxel_size, min_coord, max_coord, out=None, mode=MODE_REFERENCE, path=PATH_AUTO,
                     device=0, max_rounds=0, raise_on_error=True, mlp_params=None, mlp_budget=None,
                     mlp_threshold=None, brick_scores=None, sweep_schedule=0, host_output=0, winding_eval=0,
                     wait_poll_limit=0, splat_dense_cut=0):
    """Run the engine. ``tris``: (T,12) float32 numpy array (host) or CUDA tensor.
    ``out``: float32 buffer of N voxels (numpy = host, CUDA tensor = device); allocated
    on the host when None. ``MODE_LEARNED`` takes the sign-risk model's parameters
    (``mlp_params``; the shipped model when None), the most bricks it may propose and the
    probability threshold; ``brick_scores`` (one logit per 8^3 brick, x fastest) replaces
    the network's scores. ``sweep_schedule``: x + 10 w, x (1-5) a fixed x-sweep schedule and
    w (1-4) a fixed y / z walk schedule, a 0 digit autotuned (identical results).
    ``host_output``: 0 lets a page-locked host output be written directly by the sign-apply
    kernel, 1 stages it in device memory and copies.
    ``winding_eval``: 0 clustered exact winding decisions, 1 triangle-by-triangle sums.
    ``splat_dense_cut``: binned triangles per brick above which the splat uses its sub-brick
    kernel (0 = autotuned per lattice class; identical results at every cut).
    ``wait_poll_limit``: the eikonal's staged-tile waits (0 default; < 0 gives up at once,
    which exercises the failure path). Returns ``(out, Result)``."""
    mn = np.asarray(min_coord, np.int64).reshape(3)
    mx = np.asarray(max_coord, np.int64).reshape(3)
    dims = mx - mn + 1
    N = int(np.prod(dims)) if (dims > 0).all() else 0
    if isinstance(tris, np.ndarray):
        tris = np.ascontiguousarray(tris, np.float32).reshape(-1, 12)
    T = int(tris.shape[0])
    tp, tdev = _ptr_of(tris)
    if out is None:
        out = np.empty(max(N, 1), np.float32)
    op, odev = _ptr_of(out)
    o = _lib.Options()
    L = _lib.load()
    L.gbsdf_default_options(C.byref(o))
    o.mode, o.path, o.device, o.tris_on_device, o.max_rounds = int(mode), int(path), int(device), int(tdev), int(max_rounds)
    o.sweep_schedule = int(sweep_schedule)
    o.host_output = int(host_output)
    o.winding_eval = int(winding_eval)
    o.splat_dense_cut = int(splat_dense_cut)
    o.wait_poll_limit = int(wait_poll_limit)
    keep = _set_learned(o, mode, device, mlp_params, mlp_budget, mlp_threshold, brick_scores)  # noqa: F841
    st = _lib.Stats()
    err = C.create_string_buffer(512)
    rc = L.gbsdf_compute_mesh_sdf(tp, T, float(voxel_size), _i3(mn), _i3(mx), op, int(odev), C.byref(o),
                                  C.byref(st), err, len(err))
    res = Result(rc, st.as_dict(), err.value.decode(errors="replace"))
    if rc != _lib.OK and raise_on_error:
        raise GbsdfError(rc, res.message)
    return out, res


def compute_mesh_sdf_batch(meshes, outs=None, mode=MODE_REFERENCE, path=PATH_FAST, device=0,
                           raise_on_error=True, mlp_params=None, mlp_budget=None, mlp_threshold=None):
    """Batched build. ``meshes``: list of (tris, voxel_size, min_coord, max_coord); all
    triangles host arrays or all CUDA tensors; ``outs``: matching output buffers (host
    arrays allocated when None). Returns (outs, statuses, stats list, message)."""
    n = len(meshes)
    descs = (_lib.MeshDesc * n)()
    keep = []
    tdev = None
    if outs is None:
        outs = []
        for _, _, mn, mx in meshes:
            d = np.asarray(mx, np.int64) - np.asarray(mn, np.int64) + 1
            outs.append(np.empty(int(np.prod(d)), np.float32))
    odev = None
    for i, ((tris, h, mn, mx), out) in enumerate(zip(meshes, outs)):
        if isinstance(tris, np.ndarray):
            tris = np.ascontiguousarray(tris, np.float32).reshape(-1, 12)
        keep.append(tris)
        tp, td = _ptr_of(tris)
        op, od = _ptr_of(out)
        if tdev is None:
            tdev, odev = td, od
        if td != tdev or od != odev:
            raise ValueError("all triangles (and all outputs) must be on the same side")
        descs[i].tris, descs[i].n_tris, descs[i].voxel_size = tp, int(tris.shape[0]), float(h)
        for k in range(3):
            descs[i].min_coord[k] = int(np.asarray(mn).reshape(3)[k])
            descs[i].max_coord[k] = int(np.asarray(mx).reshape(3)[k])
        descs[i].out = op
    L = _lib.load()
    o = _lib.Options()
    L.gbsdf_default_options(C.byref(o))
    o.mode, o.path, o.device, o.tris_on_device = int(mode), int(path), int(device), int(bool(tdev))
    keep_p = _set_learned(o, mode, device, mlp_params, mlp_budget, mlp_threshold)  # noqa: F841
    stats = (_lib.Stats * n)()
    err = C.create_string_buffer(512)
    rc = L.gbsdf_compute_mesh_sdf_batch(descs, n, int(bool(odev)), C.byref(o), stats, err, len(err))
    statuses = [descs[i].status for i in range(n)]
    if rc != _lib.OK and raise_on_error:
        raise GbsdfError(rc, err.value.decode(errors="replace"))
    return outs, statuses, [s.as_dict() for s in stats], err.value.decode(errors="replace")


class Batch:
    """A planned batch (gbsdf_batch_create): the meshes' buffers are sized once and the
    whole build of every mesh is one CUDA graph; ``run()`` replays it. ``meshes``: list
    of (tris, voxel_size, min_coord, max_coord) with all triangles host arrays or all
    CUDA tensors; ``outs``: matching float32 outputs (host arrays allocated when None).
    The arrays are referenced, not copied: their contents may change between runs, their
    sizes may not."""

    def __init__(self, meshes, outs=None, mode=MODE_REFERENCE, device=0, sweep_schedule=0, mlp_params=None,
                 mlp_budget=None, mlp_threshold=None):
        n = len(meshes)
        self.n = n
        self._descs = (_lib.MeshDesc * n)()
        self._keep = []
        if outs is None:
            outs = [np.empty(int(np.prod(np.asarray(mx, np.int64) - np.asarray(mn, np.int64) + 1)), np.float32)
                    for _, _, mn, mx in meshes]
        self.outs = outs
        tdev = odev = None
        for i, ((tris, h, mn, mx), out) in enumerate(zip(meshes, outs)):
            tp, td = _ptr_of(tris)
            op, od = _ptr_of(out)
            if tdev is None:
                tdev, odev = td, od
            if td != tdev or od != odev:
                raise ValueError("all triangles (and all outputs) must be on the same side")
            self._keep.append((tris, out))
            d = self._descs[i]
            d.tris, d.n_tris, d.voxel_size, d.out = tp, int(tris.shape[0]), float(h), op
            for k in range(3):
                d.min_coord[k] = int(np.asarray(mn).reshape(3)[k])
                d.max_coord[k] = int(np.asarray(mx).reshape(3)[k])
        L = _lib.load()
        o = _lib.Options()
        L.gbsdf_default_options(C.byref(o))
        o.mode, o.path, o.device, o.tris_on_device = int(mode), int(PATH_FAST), int(device), int(bool(tdev))
        o.sweep_schedule = int(sweep_schedule)
        # learned mode: the network's parameters stay referenced for the batch's lifetime
        self._mlp = _set_learned(o, mode, device, mlp_params, mlp_budget, mlp_threshold)
        self._h = C.c_void_p()
        err = C.create_string_buffer(512)
        rc = L.gbsdf_batch_create(self._descs, n, int(bool(odev)), C.byref(o), C.byref(self._h), err, len(err))
        if rc != _lib.OK:
            raise GbsdfError(rc, err.value.decode(errors="replace"))

    def run(self, raise_on_error=False):
        """Replays the batch: returns (statuses, per-mesh stats dicts)."""
        st = (C.c_int32 * self.n)()
        stats = (_lib.Stats * self.n)()
        err = C.create_string_buffer(512)
        rc = _lib.load().gbsdf_batch_run(self._h, st, stats, err, len(err))
        if rc != _lib.OK and raise_on_error:
            raise GbsdfError(rc, err.value.decode(errors="replace"))
        return list(st), [s.as_dict() for s in stats]

    def close(self):
        if self._h:
            _lib.load().gbsdf_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def parse_binary_stl(data: bytes, device=0, normals=False):
    """GPU decode + weld of a binary STL (gbsdf_parse_binary_stl). Returns (vertices (V,3)
    float32, indices (I,) uint32) and, with ``normals``, the (T,3) record normals."""
    b = np.frombuffer(data, np.uint8)
    T = int(np.frombuffer(data[80:84], np.uint32)[0]) if len(data) >= 84 else 0
    verts = np.empty((max(3 * T, 1), 3), np.float32)
    idx = np.empty(max(3 * T, 1), np.uint32)
    nrm = np.empty((max(T, 1), 3), np.float32)
    nv, ni = C.c_int64(0), C.c_int64(0)
    err = C.create_string_buffer(512)
    rc = _lib.load().gbsdf_parse_binary_stl(b.ctypes.data, len(data), verts.ctypes.data, 3 * T, idx.ctypes.data, 3 * T,
                                            nrm.ctypes.data, C.byref(nv), C.byref(ni), int(device), err, len(err))
    if rc != _lib.OK:
        raise GbsdfError(rc, err.value.decode(errors="replace"))
    out = (verts[:nv.value], idx[:ni.value])
    return out + (nrm[:T],) if normals else out


def parse_obj(text: bytes, device=0):
    """GPU decode of OBJ text (gbsdf_parse_obj). Returns (vertices (V,3) float32, indices (I,) uint32)."""
    data = bytes(text)
    cap = len(data) // 10 + 1024
    b = np.frombuffer(data, np.uint8)
    verts = np.empty((cap, 3), np.float32)
    idx = np.empty(6 * cap, np.uint32)
    nv, ni = C.c_int64(0), C.c_int64(0)
    err = C.create_string_buffer(512)
    rc = _lib.load().gbsdf_parse_obj(b.ctypes.data, len(data), verts.ctypes.data, cap, idx.ctypes.data, 6 * cap,
                                     C.byref(nv), C.byref(ni), int(device), err, len(err))
    if rc != _lib.OK:
        raise GbsdfError(rc, err.value.decode(errors="replace"))
    return verts[:nv.value], idx[:ni.value]


def parse_ascii_stl(text: bytes, device=0):
    """GPU decode + weld of ASCII STL text (gbsdf_parse_ascii_stl). Returns (vertices (V,3)
    float32, indices (I,) uint32)."""
    data = bytes(text)
    L = _lib.load()
    cap = C.c_int64(0)
    L.gbsdf_ascii_stl_capacity(C.c_size_t(len(data)), C.byref(cap))
    b = np.frombuffer(data, np.uint8) if data else np.zeros(1, np.uint8)
    verts = np.empty((cap.value, 3), np.float32)
    idx = np.empty(cap.value, np.uint32)
    nv, ni = C.c_int64(0), C.c_int64(0)
    err = C.create_string_buffer(512)
    rc = L.gbsdf_parse_ascii_stl(b.ctypes.data, len(data), verts.ctypes.data, cap.value, idx.ctypes.data, cap.value,
                                 C.byref(nv), C.byref(ni), int(device), err, len(err))
    if rc != _lib.OK:
        raise GbsdfError(rc, err.value.decode(errors="replace"))
    return verts[:nv.value], idx[:ni.value]


def parse_stl(data: bytes, device=0):
    """StlParser::parse (stl_parser.cpp:9-66): a file of at least 84 bytes whose header
    count T > 0 fits (84 + 50 T bytes) is binary, anything else ASCII; decoded on the GPU,
    then oriented (orient_mesh). Returns (vertices, indices, orientable); raises GbsdfError
    where the reference returns false (too small, undecodable, no triangle)."""
    data = bytes(data)
    if len(data) < 84:
        raise GbsdfError(_lib.EINVAL, "STL file too small to be valid")
    T = int(np.frombuffer(data[80:84], np.uint32)[0])
    if T > 0 and len(data) >= 84 + 50 * T:
        verts, idx = parse_binary_stl(data, device=device)
    else:
        verts, idx = parse_ascii_stl(data, device=device)
    if len(idx) == 0:
        raise GbsdfError(_lib.EINVAL, "STL contains no valid non-degenerate triangles")
    idx, orientable, _, _, _ = orient_mesh(verts, idx, device=device)
    return verts, idx, orientable


class _DeviceArray:
    """A device buffer described by __cuda_array_interface__ (for torch.as_tensor)."""

    def __init__(self, ptr, shape, typestr):
        self.__cuda_array_interface__ = {"data": (int(ptr), False), "shape": tuple(shape), "typestr": typestr,
                                         "version": 2}


def extract_iso_surface(grid, dims, voxel_size, origin, iso_value=0.0, device=0, outputs_on_device=False):
    """Marching cubes of a grid (gbsdf_extract_iso_surface). ``grid``: N floats, x fastest --
    a numpy array (uploaded, as the reference does) or a CUDA tensor read in place (e.g. the
    ``out`` of compute_mesh_sdf). Returns (vertices (V,3) float32, indices (I,) uint32), numpy
    arrays, or CUDA tensors (indices int32) with ``outputs_on_device`` (one call through
    gbsdf_extract_iso_surface_device)."""
    d = _i3(dims)
    o = (C.c_float * 3)(*[float(x) for x in np.asarray(origin, np.float64).reshape(3)])
    on_dev = bool(getattr(grid, "is_cuda", False))
    if on_dev:
        import torch

        if grid.dtype != torch.float32 or not grid.is_contiguous():
            raise GbsdfError(_lib.EINVAL, "the device grid must be a contiguous float32 tensor")
        gptr = grid.data_ptr()
    else:
        grid = np.ascontiguousarray(grid, np.float32).ravel()
        gptr = grid.ctypes.data
    if int(np.prod(np.asarray(dims, np.int64))) > (grid.numel() if on_dev else grid.size):
        raise GbsdfError(_lib.EINVAL, "the grid holds fewer voxels than dims")
    L = _lib.load()
    nv, ni = C.c_int64(0), C.c_int64(0)
    err = C.create_string_buffer(512)
    if outputs_on_device:  # one call; copies of the library-owned device mesh
        import torch

        pv, pi = C.c_void_p(0), C.c_void_p(0)
        rc = L.gbsdf_extract_iso_surface_device(gptr, int(on_dev), d, float(voxel_size), o, float(iso_value),
                                                C.byref(pv), C.byref(pi), C.byref(nv), C.byref(ni), int(device), err,
                                                len(err))
        if rc != _lib.OK:
            raise GbsdfError(rc, err.value.decode(errors="replace"))
        dev = torch.device("cuda", int(device))
        if nv.value == 0:
            return torch.empty((0, 3), dtype=torch.float32, device=dev), torch.empty(0, dtype=torch.int32, device=dev)
        return (torch.as_tensor(_DeviceArray(pv.value, (nv.value, 3), "<f4"), device=dev).clone(),
                torch.as_tensor(_DeviceArray(pi.value, (ni.value,), "<i4"), device=dev).clone())
    rc = L.gbsdf_extract_iso_surface(gptr, int(on_dev), d, float(voxel_size), o, float(iso_value), None, 0, None, 0,
                                     0, C.byref(nv), C.byref(ni), int(device), err, len(err))
    if rc != _lib.OK and (nv.value == 0 and ni.value == 0 or rc != _lib.EINVAL):
        raise GbsdfError(rc, err.value.decode(errors="replace"))
    V, I = nv.value, ni.value
    verts = np.empty((max(V, 1), 3), np.float32)
    idx = np.empty(max(I, 1), np.uint32)
    vp, ip = verts.ctypes.data, idx.ctypes.data
    if V and I:
        rc = L.gbsdf_extract_iso_surface(gptr, int(on_dev), d, float(voxel_size), o, float(iso_value), vp, V, ip, I,
                                         0, C.byref(nv), C.byref(ni), int(device), err, len(err))
        if rc != _lib.OK:
            raise GbsdfError(rc, err.value.decode(errors="replace"))
    return verts[:nv.value], idx[:ni.value]


def _grid_ptr(grid):
    if bool(getattr(grid, "is_cuda", False)):
        import torch

        if grid.dtype != torch.float32 or not grid.is_contiguous():
            raise GbsdfError(_lib.EINVAL, "the device grid must be a contiguous float32 tensor")
        return grid.data_ptr(), 1, grid, int(grid.numel())
    g = np.ascontiguousarray(grid, np.float32).ravel()
    return g.ctypes.data, 0, g, int(g.size)


def interior_volume(grid, voxel_size, device=0):
    """Interior volume (gbsdf_interior_volume): (volume mm^3 as float32, inside voxels).
    ``grid``: numpy array (uploaded) or CUDA tensor (read in place)."""
    ptr, on_dev, keep, n = _grid_ptr(grid)
    vol, cnt = C.c_float(0.0), C.c_int64(0)
    err = C.create_string_buffer(256)
    rc = _lib.load().gbsdf_interior_volume(ptr, on_dev, n, float(voxel_size), C.byref(vol), C.byref(cnt), int(device),
                                           err, len(err))
    if rc != _lib.OK:
        raise GbsdfError(rc, err.value.decode(errors="replace"))
    return np.float32(vol.value), cnt.value


def find_default_seed(grid, dims, min_coord, voxel_size, min_p, max_p, desired_margin, device=0):
    """Default growth seed (gbsdf_find_default_seed): a float32 (3,) point."""
    ptr, on_dev, keep, n = _grid_ptr(grid)
    f3 = lambda v: (C.c_float * 3)(*[float(x) for x in np.asarray(v, np.float32).reshape(3)])
    out = (C.c_float * 3)()
    err = C.create_string_buffer(256)
    rc = _lib.load().gbsdf_find_default_seed(ptr, on_dev, _i3(dims), _i3(min_coord), float(voxel_size), f3(min_p),
                                             f3(max_p), float(desired_margin), out, int(device), err, len(err))
    if rc != _lib.OK:
        raise GbsdfError(rc, err.value.decode(errors="replace"))
    return np.array(list(out), np.float32)


def orient_mesh(vertices, indices, device=0):
    """GPU orientation pre-pass (gbsdf_orient_mesh). Returns (indices oriented (I,) uint32,
    orientable, had_inconsistent_winding, was_inverted, signed volume)."""
    v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
    idx = np.ascontiguousarray(indices, np.uint32).ravel().copy()
    o, i, w = C.c_int32(0), C.c_int32(0), C.c_int32(0)
    vol = C.c_double(0.0)
    err = C.create_string_buffer(512)
    rc = _lib.load().gbsdf_orient_mesh(v.ctypes.data, len(v), idx.ctypes.data, len(idx), C.byref(o), C.byref(i),
                                       C.byref(w), C.byref(vol), int(device), err, len(err))
    if rc != _lib.OK:
        raise GbsdfError(rc, err.value.decode(errors="replace"))
    return idx, bool(o.value), bool(i.value), bool(w.value), vol.value


def mesh_lattice(vertices, voxel_size):
    """Lattice of build_from_mesh (cuda_rasterizer.cu:1354-1372): returns (min, max)."""
    v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
    mn = (C.c_int32 * 3)()
    mx = (C.c_int32 * 3)()
    err = C.create_string_buffer(256)
    rc = _lib.load().gbsdf_mesh_lattice(v.ctypes.data, len(v), float(voxel_size), mn, mx, err, len(err))
    if rc != _lib.OK:
        raise GbsdfError(rc, err.value.decode())
    return np.array(list(mn), np.int32), np.array(list(mx), np.int32)


def build_from_mesh(vertices, indices, voxel_size, mode=MODE_REFERENCE, path=PATH_AUTO, device=0, out=None,
                    raise_on_error=True):
    """Indexed mesh -> SDF on the build_from_mesh lattice. Returns (out, min, max, Result)."""
    v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
    idx = np.ascontiguousarray(indices, np.uint32).reshape(-1)
    mn, mx = mesh_lattice(v, voxel_size)
    N = int(np.prod(mx.astype(np.int64) - mn + 1))
    if out is None:
        out = np.empty(N, np.float32)
    op, odev = _ptr_of(out)
    L = _lib.load()
    o = _lib.Options()
    L.gbsdf_default_options(C.byref(o))
    o.mode, o.path, o.device = int(mode), int(path), int(device)
    st = _lib.Stats()
    err = C.create_string_buffer(512)
    rc = L.gbsdf_build_from_mesh(v.ctypes.data, len(v), idx.ctypes.data, len(idx), float(voxel_size), _i3(mn),
                                 _i3(mx), op, int(odev), C.byref(o), C.byref(st), err, len(err))
    res = Result(rc, st.as_dict(), err.value.decode(errors="replace"))
    if rc != _lib.OK and raise_on_error:
        raise GbsdfError(rc, res.message)
    return out, mn, mx, res


@dataclass
class CudaVolumeGrid:
    """cuda_types.hpp:155-175: dense grid, x fastest, value at lattice point (min+i) h."""
    data: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))
    min_coord: np.ndarray = field(default_factory=lambda: np.zeros(3, np.int32))
    max_coord: np.ndarray = field(default_factory=lambda: np.zeros(3, np.int32))
    dims: np.ndarray = field(default_factory=lambda: np.zeros(3, np.int32))
    voxel_size: float = 0.5
    version: int = 1

    def is_valid(self) -> bool:
        return self.data.size > 0 and bool((self.dims > 0).all())


class CudaRasterizer:
    """Static entry points with the reference's names, argument meaning and
    error behaviour (bool / None on failure, output untouched)."""

    _next_version = 2

    @staticmethod
    def compute_mesh_sdf(triangles, voxel_size, min_coord, max_coord, out_distances: list | None = None):
        """Returns (ok, out_distances ndarray, out_time_ms). On failure returns
        (False, out_distances unchanged, time)."""
        mn = np.asarray(min_coord, np.int64)
        mx = np.asarray(max_coord, np.int64)
        dims = mx - mn + 1
        if (dims <= 0).any():
            return False, out_distances, 0.0
        N = int(np.prod(dims))
        buf = np.full(N, 1e6, np.float32)  # cuda_rasterizer.cu:1180
        _, res = compute_mesh_sdf(triangles, voxel_size, mn, mx, out=buf, raise_on_error=False)
        if not res.ok:
            return False, out_distances, res.stats.get("ms_total", 0.0)
        return True, buf, res.stats["ms_total"]

    @staticmethod
    def extract_iso_surface(grid, dims=None, voxel_size=None, origin=None, iso_value=0.0):
        """cuda_marching_cubes.cu:829-962: (distance_grid, dims, voxel_size, origin, iso) or
        (CudaVolumeGrid, iso) -> (ok, (vertices, indices), out_time_ms); dims < 2 gives an
        empty mesh."""
        import time as _time

        if isinstance(grid, CudaVolumeGrid):
            vol = grid
            iso_value = 0.0 if dims is None else float(dims)
            grid, dims, voxel_size = vol.data, vol.dims, vol.voxel_size
            origin = np.asarray(vol.min_coord, np.float32) * np.float32(vol.voxel_size)
        t0 = _time.perf_counter()
        try:
            mesh = extract_iso_surface(grid, dims, voxel_size, origin, iso_value)
        except GbsdfError:
            return False, (np.zeros((0, 3), np.float32), np.zeros(0, np.uint32)), 0.0
        return True, mesh, (_time.perf_counter() - t0) * 1e3

    @staticmethod
    def build_from_mesh(vertices, indices, voxel_size):
        """Returns (CudaVolumeGrid | None, out_time_ms)."""
        if len(vertices) == 0 or len(indices) == 0:
            return None, 0.0
        out, mn, mx, res = build_from_mesh(vertices, indices, voxel_size, raise_on_error=False)
        if not res.ok:
            return None, res.stats.get("ms_total", 0.0)
        CudaRasterizer._next_version += 1
        g = CudaVolumeGrid(out, mn, mx, (mx - mn + 1).astype(np.int32), float(voxel_size), CudaRasterizer._next_version)
        return g, res.stats["ms_total"]
