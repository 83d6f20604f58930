"""The band splat's tile cut (binned triangles per 8^3 brick above which a brick goes to the
sub-brick kernel instead of one whole-brick CTA) changes no result: a dense mesh of the
64-mesh workload (261k triangles on a 95^3 lattice, thousands of triangles per brick) built
with every brick on either kernel and at the autotuned cut gives the same grid, equal to the
oracle, and the autotuner reports one of its candidate cuts."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_splat_cut_changes_nothing(engine, oracle):
    from gbsdf import meshgen

    meshes = meshgen.batch_workload()
    tris, h, mn, mx = max(meshes, key=lambda m: len(m[0]) / np.prod(m[3].astype(np.int64) - m[2] + 1))
    outs = {}
    for cut in (1, 64, 256, 1 << 30):  # 1: (nearly) every brick dense; 1 << 30: every brick sparse
        out, res = engine.compute_mesh_sdf(tris, h, mn, mx, mode=engine.MODE_EXACT_SIGNS, path=engine.PATH_FAST,
                                           splat_dense_cut=cut)
        assert res.ok and res.stats["splat_dense_cut"] == cut
        outs[cut] = out
    for cut in (1, 64, 256):
        assert np.array_equal(outs[cut].view(np.uint32), outs[1 << 30].view(np.uint32)), cut
    out, res = engine.compute_mesh_sdf(tris, h, mn, mx, mode=engine.MODE_EXACT_SIGNS, path=engine.PATH_FAST)
    assert res.stats["splat_dense_cut"] in (128, 256, 512, 1024)
    assert np.array_equal(out.view(np.uint32), outs[1 << 30].view(np.uint32))
    st, ref, _, _ = oracle.fast_sdf(tris, h, mn, mx, fsm_mode=0, gwn_mode=1, signed_parity=True)
    assert st == oracle.OK
    assert np.array_equal(out.view(np.uint32), ref.view(np.uint32))
