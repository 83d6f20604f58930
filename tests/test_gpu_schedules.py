"""The x-sweep schedules (cp.async-staged, TMA tiles on a CTA-barrier ring, TMA tiles on a
warp-specialised mbarrier pipeline) and the autotuner's pick give bit-identical grids,
equal to the oracle, on lattices whose rows do and do not admit a TMA descriptor."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _case(dims):
    from gbsdf import meshgen

    tris, mn, mx, h = meshgen.workload("mug_c1_128", dims=dims, h=1.0)
    return tris, mn, mx, h


@pytest.mark.parametrize("dims", [(96, 88, 92), (97, 83, 90), (44, 260, 30)])
def test_schedules_identical(engine, oracle, dims):
    tris, mn, mx, h = _case(dims)
    outs = {}
    for sched in (0, 1, 2, 3):
        out, res = engine.compute_mesh_sdf(tris, h, mn, mx, mode=engine.MODE_EXACT_SIGNS, path=engine.PATH_FAST,
                                           sweep_schedule=sched)
        assert res.ok
        outs[sched] = out
        expect = sched if sched else res.stats["sweep_schedule"]
        if dims[0] % 4:
            expect = 1  # no TMA descriptor: the cp.async schedule runs
        assert res.stats["sweep_schedule"] == expect
    for sched in (1, 2, 3):
        assert np.array_equal(outs[0].view(np.uint32), outs[sched].view(np.uint32)), sched
    st, ref, _, _ = oracle.fast_sdf(tris, h, mn, mx, fsm_mode=0, gwn_mode=1, signed_parity=True)
    assert st == oracle.OK
    assert np.array_equal(outs[0].view(np.uint32), ref.view(np.uint32))
