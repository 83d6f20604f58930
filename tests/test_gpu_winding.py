"""The clustered winding evaluation (far clusters by a dipole with a rigorous error bound,
undecided voxels summed triangle by triangle) decides every voxel as the plain per-triangle
sum does: fixup of columns through holes, stratified probes, patch boxes, the legacy exact
path and learned proposals, on meshes with holes, jitter and overlapping shells."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cases():
    from gbsdf import meshgen

    out = []
    v, f = meshgen.vessel_tree(seed=3, levels=3, around=20, n_len=8, n_cap=2, hole_frac=0.02, n_jitter=30,
                               dup_frac=0.01)
    vf, mn, mx = meshgen.fit_to_lattice(v, (96, 90, 100), 1.0)
    out.append(("vessel", meshgen.to_triangles(vf, f), 1.0, mn, mx))
    v, f = meshgen.sh_blob(seed=4, n_lat=48, n_lon=96, degree=6, coeff_scale=4.0, vertex_noise=0.2, hole_frac=0.03)
    vf, mn, mx = meshgen.fit_to_lattice(v, (80, 84, 76), 0.7)
    out.append(("blob", meshgen.to_triangles(vf, f), 0.7, mn, mx))
    return out


@pytest.mark.parametrize("case", range(2))
def test_clustered_equals_per_triangle(engine, case):
    name, tris, h, mn, mx = _cases()[case]
    for mode, path in ((engine.MODE_REFERENCE, engine.PATH_FAST), (engine.MODE_EXACT_SIGNS, engine.PATH_FAST),
                       (engine.MODE_REFERENCE, engine.PATH_LEGACY)):
        a, ra = engine.compute_mesh_sdf(tris, h, mn, mx, mode=mode, path=path, winding_eval=0, raise_on_error=False)
        b, rb = engine.compute_mesh_sdf(tris, h, mn, mx, mode=mode, path=path, winding_eval=1, raise_on_error=False)
        assert ra.status == rb.status, (name, mode, path)
        if ra.ok:
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), (name, mode, path)
        assert ra.stats["winding_certified"] > 0, (name, mode, path)
        assert rb.stats["winding_certified"] == 0


def test_clustered_learned_proposals(engine):
    from gbsdf import MODE_LEARNED, PATH_FAST, learn

    # a defective mesh whose stratified probes find no mismatch: learned mode proposes
    for tris, h, mn, mx in learn.training_meshes(12, seed=31, grid=80):
        _, r = engine.compute_mesh_sdf(tris, h, mn, mx, mode=engine.MODE_REFERENCE, path=PATH_FAST,
                                       raise_on_error=False)
        if r.ok and r.stats["sites"] == 0:
            break
    else:
        pytest.fail("no training mesh without probe mismatches")
    trained = np.load(learn.MODEL_PATH)["params"]
    a, ra = engine.compute_mesh_sdf(tris, h, mn, mx, mode=MODE_LEARNED, path=PATH_FAST, mlp_params=trained,
                                    mlp_budget=200, winding_eval=0)
    b, rb = engine.compute_mesh_sdf(tris, h, mn, mx, mode=MODE_LEARNED, path=PATH_FAST, mlp_params=trained,
                                    mlp_budget=200, winding_eval=1)
    assert ra.stats["proposed"] == rb.stats["proposed"] > 0
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
