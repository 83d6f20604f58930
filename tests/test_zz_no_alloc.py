"""The entry point that allocates nothing: gbsdf_legacy_sdf_noalloc.

Some callers cannot call cudaMalloc -- a plugin whose host application owns every
device allocation, a step that runs under a device-memory budget fixed at start-up, or
a latency-critical loop that cannot take cudaMalloc's implicit synchronisation. For them
the library keeps the exact SDF build's scratch in a fixed array of its own, and the
caller passes only device buffers for the triangles and the output grid.

These tests call the entry point through the C ABI, twice in a row (the second call
reuses the array the first one left behind), and compare each result with the
allocating entry point (gbsdf_compute_mesh_sdf on the legacy path) within the tolerances
used by every parity test: identical signs, band distances within 1e-5 voxel, the rest
within 1e-4 voxel.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _check(got, ref, h):
    nz = ref != 0
    assert np.count_nonzero(np.signbit(got[nz]) != np.signbit(ref[nz])) == 0
    err = np.abs(got.astype(np.float64) - ref.astype(np.float64)) / h
    band = np.abs(ref) <= 8 * h
    assert err[band].max(initial=0) <= 1e-5
    assert err[~band].max(initial=0) <= 1e-4


def _mesh():
    from gbsdf import meshgen

    v, f = meshgen.mug(segments=64, n_bottom=3, n_wall=6, n_rim=1, handle_path=16, handle_around=12)
    vf, mn, mx = meshgen.fit_to_lattice(v, (40, 40, 44), 2.4)
    return meshgen.to_triangles(vf, f), mn, mx, 2.4


def _i3(v):
    return (C.c_int32 * 3)(*[int(a) for a in v])


def test_noalloc_matches_allocating_entry_point_twice(engine):
    import torch

    from gbsdf import _lib

    L = _lib.load()
    tris, mn, mx, h = _mesh()
    n = int(np.prod(mx.astype(np.int64) - mn + 1))
    ref, res = engine.compute_mesh_sdf(tris, h, mn, mx, path=engine.PATH_LEGACY)
    assert res.ok
    tris_dev = torch.from_numpy(tris).cuda()
    for _ in range(2):
        out = torch.full((n,), 7.0, dtype=torch.float32, device="cuda")
        st = _lib.Stats()
        err = C.create_string_buffer(256)
        rc = L.gbsdf_legacy_sdf_noalloc(tris_dev.data_ptr(), len(tris), h, _i3(mn), _i3(mx), out.data_ptr(), 0,
                                        None, C.byref(st), err, len(err))
        assert rc == _lib.OK, err.value
        torch.cuda.synchronize()
        _check(out.cpu().numpy(), ref, h)


def test_noalloc_rejects_lattice_above_its_limit(engine):
    import torch

    from gbsdf import _lib

    L = _lib.load()
    tris, _, _, h = _mesh()
    tris_dev = torch.from_numpy(tris).cuda()
    out = torch.zeros(16, dtype=torch.float32, device="cuda")
    err = C.create_string_buffer(256)
    rc = L.gbsdf_legacy_sdf_noalloc(tris_dev.data_ptr(), len(tris), h, _i3((0, 0, 0)), _i3((299, 299, 299)),
                                    out.data_ptr(), 0, None, None, err, len(err))
    assert rc == _lib.EINVAL and b"limit" in err.value
    assert torch.count_nonzero(out).item() == 0
