"""The oracle's shortcuts for the full-size parity tests leave its statuses, statistics and
decided signs unchanged: ``skip_eikonal`` (stage [D] changes no voxel the surface tolerance
reads) and ``lazy_winding`` (voxels of columns through holes and of patch boxes marked for
the winding number instead of summed). Cases: a self-overlap lens whose probes find 5 sites
(one patch round), a large overlap that declines, and a vessel tree with holes."""
import numpy as np
import pytest

KEYS = ("unknown_columns", "fixup_voxels", "probes", "sites", "patch_rounds", "patched_voxels", "band_voxels")


def _case(name):
    from gbsdf import meshgen

    if name == "lens":
        v, f = meshgen.overlapping_spheres(30.0, 56.0)
        dims, h = (64, 36, 36), 1.0
    elif name == "overlap":
        v, f = meshgen.overlapping_spheres(30.0, 36.0)
        dims, h = (96, 64, 64), 1.0
    else:
        v, f = meshgen.vessel_tree(seed=7, levels=3, around=16, n_len=8, n_cap=2, hole_frac=0.01, n_jitter=20,
                                   dup_frac=0.01)
        dims, h = (56, 56, 56), 1.0
    vf, mn, mx = meshgen.fit_to_lattice(v, dims, h)
    return meshgen.to_triangles(vf, f), h, mn, mx


@pytest.mark.parametrize("name,signed", [("lens", False), ("overlap", False), ("vessel", False), ("vessel", True)])
def test_lazy_oracle_equals_full(oracle, name, signed):
    tris, h, mn, mx = _case(name)
    a = oracle.fast_sdf(tris, h, mn, mx, fsm_mode=0, signed_parity=signed)
    b = oracle.fast_sdf(tris, h, mn, mx, fsm_mode=0, signed_parity=signed, skip_eikonal=True, lazy_winding=True)
    assert a[0] == b[0]
    for k in KEYS:
        assert a[3][k] == b[3][k], k
    if name == "lens":
        assert a[3]["patch_rounds"] == 1 and a[3]["sites"] > 0
    if name == "overlap":
        assert a[0] == 4
    if name == "vessel":
        assert a[3]["fixup_voxels"] > 0
    if a[0] == oracle.OK:
        lazy = b[2] == 3
        assert lazy.sum() == a[3]["fixup_voxels"] + a[3]["patched_voxels"] or a[3]["patch_rounds"] > 0
        assert np.array_equal(a[2][~lazy], b[2][~lazy])
        assert np.array_equal(np.signbit(a[1])[~lazy], np.signbit(b[1])[~lazy])
