"""Known answers from the reference's verification harness, on the engine: the eikonal
property of a sphere's field (harness_eikonal_cuda_tests.cpp, case (a): at least 85% of
55,000 shell samples within 0.02 of |grad f| = 1), in reference and exact-signs modes, the
reference-mode grid equal to the oracle's bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_eikonal_property_sphere(engine, oracle):
    from gbsdf import meshgen
    from test_oracle_golden import eikonal_fraction, sphere_case

    v, f = sphere_case()
    idx = f.astype(np.uint32).ravel()
    for mode in (engine.MODE_REFERENCE, engine.MODE_EXACT_SIGNS):
        out, mn, mx, res = engine.build_from_mesh(v, idx, 0.35, mode=mode, path=engine.PATH_FAST)
        assert res.ok
        frac = eikonal_fraction(out, mx - mn + 1, mn, 0.35, 20.0)
        assert frac >= 0.85, (mode, frac)
        if mode == engine.MODE_REFERENCE:
            st, ref, _, _ = oracle.fast_sdf(meshgen.to_triangles(v, f), 0.35, mn, mx, fsm_mode=0, gwn_mode=1)
            assert st == 0 and np.array_equal(out.view(np.uint32), ref.view(np.uint32))
