"""Failure detection on the GPU without a fault: the eikonal's staged-tile waits are
bounded, and a build whose waits give up reports GBSDF_ECUDA, leaves the caller's output
untouched and leaves the device usable. The test sets the wait limit to no polling at
all (gbsdf_options.wait_poll_limit < 0), so every consumer's first wait gives up, the
producers let the copies already in flight land, and the state records the timeouts --
for every TMA sweep schedule."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _mug():
    from gbsdf import meshgen

    v, f = meshgen.mug(segments=96, n_bottom=4, n_wall=8, n_rim=2, handle_path=20, handle_around=16)
    vf, mn, mx = meshgen.fit_to_lattice(v, (48, 48, 52), 2.0)
    return meshgen.to_triangles(vf, f), mn, mx, 2.0


@pytest.mark.parametrize("sched", [22, 33, 43, 44, 45])
def test_tile_wait_timeout_reports_error_and_leaves_output(engine, oracle, sched):
    from gbsdf import _lib

    tris, mn, mx, h = _mug()
    n = int(np.prod(mx.astype(np.int64) - mn + 1))
    buf = np.full(n, 7.0, np.float32)
    _, res = engine.compute_mesh_sdf(tris, h, mn, mx, out=buf, mode=engine.MODE_REFERENCE, path=engine.PATH_FAST,
                                     sweep_schedule=sched, wait_poll_limit=-1, raise_on_error=False)
    assert res.status == _lib.ECUDA, (res.status, res.message)
    assert "timed out" in res.message
    assert np.all(buf == 7.0), "output must stay untouched on failure"
    # the context is still usable: the same build with the default limit matches the oracle
    out, res = engine.compute_mesh_sdf(tris, h, mn, mx, mode=engine.MODE_REFERENCE, path=engine.PATH_FAST,
                                       sweep_schedule=sched)
    assert res.ok
    st, ref, _, _ = oracle.fast_sdf(tris, h, mn, mx, fsm_mode=0, gwn_mode=1)
    assert st == oracle.OK and np.array_equal(out.view(np.uint32), ref.view(np.uint32))
