"""The entry point that allocates nothing: gbsdf_legacy_sdf_noalloc.

Some callers cannot call cudaMalloc -- a plugin whose host application owns every
device allocation, a step that runs under a device-memory budget fixed at start-up, or
a latency-critical loop that cannot take cudaMalloc's implicit synchronisation. For them
the library keeps the exact SDF build's scratch in a fixed array of its own, and the
caller passes only device buffers for the triangles and the output grid.

These tests call the entry point through the C ABI, several times in a row (each call
reuses the array the previous one left behind; the second lattice is smaller than the
first, so sign words left over from the larger one would show), and compare each result
with the allocating entry point (gbsdf_compute_mesh_sdf on the legacy path, winding
numbers summed triangle by triangle). Both run the same arithmetic (minimum squared
distance, one square root, exact winding decisions with the same FP64 re-checks), so the
grids must be bit-identical and the FP64 re-check counts equal.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _check(got, ref):
    assert got.shape == ref.shape
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), (
        f"{np.count_nonzero(got.view(np.uint32) != ref.view(np.uint32))} voxels differ from the allocating path")


def _mesh(dims=(40, 40, 44), h=2.4):
    from gbsdf import meshgen

    v, f = meshgen.mug(segments=64, n_bottom=3, n_wall=6, n_rim=1, handle_path=16, handle_around=12)
    vf, mn, mx = meshgen.fit_to_lattice(v, dims, h)
    return meshgen.to_triangles(vf, f), mn, mx, h


def _i3(v):
    return (C.c_int32 * 3)(*[int(a) for a in v])


def test_noalloc_matches_allocating_entry_point_twice(engine):
    import torch

    from gbsdf import _lib

    L = _lib.load()
    # a larger lattice, then a smaller one, then the larger one again
    cases = [_mesh((40, 40, 44), 2.4), _mesh((20, 22, 24), 4.8), _mesh((40, 40, 44), 2.4)]
    for tris, mn, mx, h in cases:
        n = int(np.prod(mx.astype(np.int64) - mn + 1))
        ref, res = engine.compute_mesh_sdf(tris, h, mn, mx, path=engine.PATH_LEGACY, winding_eval=1)
        assert res.ok
        tris_dev = torch.from_numpy(tris).cuda()
        out = torch.full((n,), 7.0, dtype=torch.float32, device="cuda")
        st = _lib.Stats()
        err = C.create_string_buffer(256)
        rc = L.gbsdf_legacy_sdf_noalloc(tris_dev.data_ptr(), len(tris), h, _i3(mn), _i3(mx), out.data_ptr(), 0,
                                        None, C.byref(st), err, len(err))
        assert rc == _lib.OK, err.value
        torch.cuda.synchronize()
        sd = st.as_dict()
        assert sd["status"] == _lib.OK and sd["path_taken"] == engine.PATH_LEGACY
        assert sd["fp64_rechecks"] == res.stats["fp64_rechecks"], (sd["fp64_rechecks"], res.stats["fp64_rechecks"])
        _check(out.cpu().numpy(), np.asarray(ref, np.float32))


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
