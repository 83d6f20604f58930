"""The eikonal sweep schedules -- x sweep staged by cp.async, by TMA tiles on a CTA-barrier
ring or on a warp-specialised mbarrier pipeline (one or two lines per thread, or wide 16-voxel
chunks); y / z walks staged by cp.async or by TMA
batches on a pipeline (one or four lines per thread, the four lines' updates scalar or in
packed FP32 pairs) -- and the autotuner's pick give
bit-identical grids, equal to the oracle, on lattices whose rows are and are not a multiple
of 8 floats (the latter swept in padded copies: 44-voxel rows padded by the first x sweep
itself, which reads the band field through a descriptor of its dense rows, except under the
cp.async x schedule; 97-voxel rows, whose dense pitch no descriptor takes, copied first)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _case(dims):
    from gbsdf import meshgen

    tris, mn, mx, h = meshgen.workload("mug_c1_128", dims=dims, h=1.0)
    return tris, mn, mx, h


# one voxel thick along y or z: both cross neighbours of a line lie outside the lattice
@pytest.mark.parametrize("dims", [(96, 88, 92), (97, 83, 90), (44, 260, 30), (200, 36, 70), (96, 1, 44), (96, 40, 1)])
def test_schedules_identical(engine, oracle, dims):
    tris, mn, mx, h = _case(dims)
    outs = {}
    scheds = (0, 1, 2, 3, 4, 5, 13, 23, 33, 43, 44, 45, 11, 21, 31, 41, 15)
    for sched in scheds:
        out, res = engine.compute_mesh_sdf(tris, h, mn, mx, mode=engine.MODE_EXACT_SIGNS, path=engine.PATH_FAST,
                                           sweep_schedule=sched)
        assert res.ok
        outs[sched] = out
        ran = res.stats["sweep_schedule"]
        x, w = ran % 10, ran // 10
        # every lattice has TMA descriptors (rows not a multiple of 8 floats are swept in
        # padded copies), so a forced schedule runs as asked
        if sched % 10:
            assert x == sched % 10
        if sched // 10:
            assert w == sched // 10
    for sched in scheds[1:]:
        assert np.array_equal(outs[0].view(np.uint32), outs[sched].view(np.uint32)), sched
    st, ref, _, _ = oracle.fast_sdf(tris, h, mn, mx, fsm_mode=0, gwn_mode=1, signed_parity=True)
    assert st == oracle.OK
    assert np.array_equal(outs[0].view(np.uint32), ref.view(np.uint32))
