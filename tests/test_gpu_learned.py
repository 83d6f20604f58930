"""GPU checks of the learned sign-risk part (csrc/k_learn.cu) through the C ABI:
forward and gradient against the FP64 oracle restatement (oracle/mlp_oracle.py), Adam
against its FP64 formula, training on the GPU, deterministic proposals, and the
ablation on held-out meshes (plain fast path vs plain + network proposals vs random band
bricks at the same budget), scored against the exact winding number at every voxel."""
import numpy as np
import pytest

from oracle import mlp_oracle as M

pytestmark = pytest.mark.gpu


def _data(n, seed):
    rng = np.random.default_rng(seed)
    X = np.abs(rng.normal(0, 1.5, (n, M.F))).astype(np.float32)
    y = ((X[:, 0] - X[:, 3] + 0.5 * X[:, 10]) > 1.0).astype(np.float32)
    w = np.where(y > 0, 2.0, 1.0).astype(np.float32)
    return X, y, w


def test_forward_matches_oracle(engine):
    import torch

    from gbsdf.learn import SignRiskMLP, init_params

    P = init_params(3)
    X, _, _ = _data(5000, 4)
    mlp = SignRiskMLP(P)
    z = mlp.logits(torch.from_numpy(X).cuda()).cpu().numpy().astype(np.float64)
    zr, _ = M.forward(P, X)
    d = np.abs(z - zr)
    # FP32 accumulation vs FP64: tiny, except where an activation sits on a BF16
    # rounding boundary and rounds the other way (one BF16 ulp of one unit)
    assert np.median(d) <= 1e-5 * (1 + np.median(np.abs(zr)))
    assert np.mean(d > 1e-4 * (1 + np.abs(zr))) < 0.02
    assert np.all(d <= 0.05 * (1 + np.abs(zr)))


def test_gradient_matches_oracle(engine):
    import torch

    from gbsdf.learn import SignRiskMLP, init_params

    P = init_params(5)
    P[M.ob3] = 0.0
    X, y, w = _data(3000, 6)
    mlp = SignRiskMLP(P)
    g, loss = mlp.grad(torch.from_numpy(X).cuda(), torch.from_numpy(y).cuda(), torch.from_numpy(w).cuda())
    g = g.cpu().numpy().astype(np.float64)
    lr, gr = M.loss_and_grad(P, X, y, w)
    assert abs(loss - lr) <= 1e-4 * abs(lr)
    rel = np.linalg.norm(g - gr) / np.linalg.norm(gr)
    assert rel < 2e-3, rel
    # every parameter block on its own
    for a, b in ((M.oW1, M.ob1), (M.ob1, M.oW2), (M.oW2, M.ob2), (M.ob2, M.ow3), (M.ow3, M.ob3), (M.ob3, M.N_PARAMS)):
        n = np.linalg.norm(gr[a:b])
        assert np.linalg.norm(g[a:b] - gr[a:b]) <= 5e-3 * n + 1e-6, (a, b)


def test_gradient_is_deterministic(engine):
    import torch

    from gbsdf.learn import SignRiskMLP, init_params

    X, y, w = _data(2000, 7)
    Xd, yd, wd = (torch.from_numpy(a).cuda() for a in (X, y, w))
    mlp = SignRiskMLP(init_params(8))
    g1, l1 = mlp.grad(Xd, yd, wd)
    g2, l2 = mlp.grad(Xd, yd, wd)
    assert torch.equal(g1, g2) and l1 == l2


def test_adam_matches_formula(engine):
    import torch

    from gbsdf.learn import SignRiskMLP, init_params

    P = init_params(9).astype(np.float64)
    mlp = SignRiskMLP(P)
    m = np.zeros(M.N_PARAMS)
    v = np.zeros(M.N_PARAMS)
    rng = np.random.default_rng(10)
    for step in range(1, 4):
        g = rng.normal(0, 1, M.N_PARAMS).astype(np.float32)
        mlp.adam(torch.from_numpy(g).cuda(), lr=1e-2, scale=0.5)
        P, m, v = M.adam(P, g, m, v, step, 1e-2, scale=0.5)
    got = mlp.params().astype(np.float64)
    assert np.max(np.abs(got - P)) < 1e-5


def test_training_reduces_loss(engine):
    import torch

    from gbsdf.learn import SignRiskMLP

    X, y, _ = _data(20000, 11)
    mlp = SignRiskMLP(seed=12)
    hist = mlp.fit(torch.from_numpy(X).cuda(), torch.from_numpy(y).cuda(), epochs=8, batch=2048, lr=3e-3)
    assert hist[-1] < 0.5 * hist[0], hist
    z = mlp.logits(torch.from_numpy(X).cuda()).cpu().numpy()
    assert np.mean((z > 0) == (y > 0.5)) > 0.9


def _mesh(seed, grid=64):
    from gbsdf import learn

    return learn.training_meshes(1, seed=seed, grid=grid)[0]


def _quiet_mesh(seed, grid=64):
    """A defective training mesh whose stratified probes find no mismatch, so learned mode
    proposes bricks rather than escalating."""
    from gbsdf import MODE_REFERENCE, PATH_FAST, compute_mesh_sdf, learn

    for tris, h, mn, mx in learn.training_meshes(32, seed=seed, grid=grid):
        _, r = compute_mesh_sdf(tris, h, mn, mx, mode=MODE_REFERENCE, path=PATH_FAST, raise_on_error=False)
        if r.ok and r.stats["sites"] == 0:
            return tris, h, mn, mx
    pytest.fail("no training mesh without probe mismatches")


def test_brick_features(engine):
    import torch

    from gbsdf import learn

    tris, h, mn, mx = _mesh(77)
    X = learn.brick_features(tris, h, mn, mx)
    nb = learn.brick_grid(mn, mx)
    assert X.shape == (nb[0] * nb[1] * nb[2], 32)
    Xh = X.cpu().numpy()
    assert np.isfinite(Xh).all() and (Xh >= 0).all()
    # bricks holding voxels within h/2 of the surface (feature 7) have triangles binned to
    # them (feature 0); band bricks (feature 4) include them
    assert (Xh[:, 7] > 0).any() and np.all(Xh[Xh[:, 7] > 0, 0] > 0) and np.all(Xh[Xh[:, 7] > 0, 4] > 0)
    X2 = learn.brick_features(tris, h, mn, mx)
    assert torch.equal(X, X2)


def test_learned_mode_is_deterministic_and_within_budget(engine):
    from gbsdf import MODE_LEARNED, PATH_FAST, compute_mesh_sdf
    from gbsdf.learn import brick_grid, init_params

    tris, h, mn, mx = _quiet_mesh(78)
    P = init_params(13)
    P[M.ob3] = 5.0  # untrained network, biased to propose many bricks
    nb = brick_grid(mn, mx)
    budget = max(1, nb[0] * nb[1] * nb[2] // 20)
    a, r1 = compute_mesh_sdf(tris, h, mn, mx, mode=MODE_LEARNED, path=PATH_FAST, mlp_params=P, mlp_budget=budget,
                             mlp_threshold=0.5)
    b, r2 = compute_mesh_sdf(tris, h, mn, mx, mode=MODE_LEARNED, path=PATH_FAST, mlp_params=P, mlp_budget=budget,
                             mlp_threshold=0.5)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert 0 < r1.stats["proposed"] <= budget and r1.stats["proposed"] == r2.stats["proposed"]


def test_learned_mode_needs_params(engine):
    import ctypes as C

    from gbsdf import _lib

    tris, h, mn, mx = _mesh(79, grid=40)
    o = _lib.Options()
    L = _lib.load()
    L.gbsdf_default_options(C.byref(o))
    o.mode, o.path = _lib.MODE_LEARNED, _lib.PATH_FAST
    out = np.empty(int(np.prod(np.asarray(mx) - mn + 1)), np.float32)
    err = C.create_string_buffer(256)
    rc = L.gbsdf_compute_mesh_sdf(tris.ctypes.data, len(tris), h, (C.c_int32 * 3)(*mn), (C.c_int32 * 3)(*mx),
                                  out.ctypes.data, 0, C.byref(o), None, err, len(err))
    assert rc == _lib.EINVAL and b"mlp_params" in err.value


def _mismatch(out, exact, h):
    far = np.abs(exact) > 1e-5 * h
    return int(np.count_nonzero((np.signbit(out) != np.signbit(exact)) & far))


def test_ablation_learned_vs_plain_vs_random(engine):
    """Held-out meshes (seeds disjoint from the training set) whose stratified probes
    found no mismatch (so learned mode proposes instead of escalating), at most 3% of the
    bricks re-decided by the exact winding number: the shipped network's picks remove most
    of the plain fast path's sign errors, far more than the same number of random band
    bricks. The single best hand feature (the count of voxels where the sign and the
    signed crossings disagree) is printed beside them."""
    from gbsdf import MODE_LEARNED, MODE_REFERENCE, PATH_FAST, PATH_LEGACY, compute_mesh_sdf, learn

    trained = np.load(learn.MODEL_PATH)["params"]
    rng = np.random.default_rng(5)
    tot = {"plain": 0, "learned": 0, "random": 0, "disagreement": 0}
    proposed = bricks = 0
    for tris, h, mn, mx in learn.training_meshes(24, seed=424242):
        exact, _ = compute_mesh_sdf(tris, h, mn, mx, path=PATH_LEGACY)
        plain, rp = compute_mesh_sdf(tris, h, mn, mx, mode=MODE_REFERENCE, path=PATH_FAST, raise_on_error=False)
        if not rp.ok:
            continue
        X = learn.brick_features(tris, h, mn, mx).cpu().numpy()
        nb = X.shape[0]
        budget = max(1, nb * 3 // 100)
        lo, rl = compute_mesh_sdf(tris, h, mn, mx, mode=MODE_LEARNED, path=PATH_FAST, mlp_params=trained,
                                  mlp_budget=budget, mlp_threshold=0.01)
        if rl.stats["escalated"]:
            continue  # a probe found a mismatch: the signs were re-decided, nothing was proposed
        k = max(1, int(rl.stats["proposed"]))
        rand = np.where(X[:, 4] > 0, rng.uniform(0.0, 10.0, nb), -100.0).astype(np.float32)
        ra, rr = compute_mesh_sdf(tris, h, mn, mx, mode=MODE_LEARNED, path=PATH_FAST, brick_scores=rand,
                                  mlp_budget=k, mlp_threshold=1e-6)
        di, _ = compute_mesh_sdf(tris, h, mn, mx, mode=MODE_LEARNED, path=PATH_FAST,
                                 brick_scores=np.ascontiguousarray(X[:, 3] * 4.0 - 0.5), mlp_budget=k,
                                 mlp_threshold=1e-6)
        assert rr.stats["proposed"] <= k
        proposed += int(rl.stats["proposed"])
        bricks += nb
        tot["plain"] += _mismatch(plain, exact, h)
        tot["learned"] += _mismatch(lo, exact, h)
        tot["random"] += _mismatch(ra, exact, h)
        tot["disagreement"] += _mismatch(di, exact, h)
    print("ablation mismatched voxels:", tot, f"proposed bricks: {proposed} of {bricks}")
    assert tot["plain"] > 0, "held-out set has no sign errors to fix"
    assert tot["learned"] <= tot["random"] <= tot["plain"]
    assert tot["learned"] < 0.5 * tot["plain"], tot
    assert tot["plain"] - tot["learned"] > 3 * (tot["plain"] - tot["random"]), tot


def test_learned_mode_matches_oracle_with_given_proposals(engine, oracle):
    """Learned mode with caller-supplied brick scores (the proposals known exactly) against
    the oracle composed stage by stage: the reference fast path, then every voxel of the
    proposed bricks re-decided by the exact winding number (on-surface voxels inside), then
    the signs applied to the same unsigned field. Bit for bit."""
    from gbsdf import MODE_LEARNED, PATH_FAST, compute_mesh_sdf, learn

    tris, h, mn, mx = _quiet_mesh(81, grid=64)
    dims = mx.astype(np.int64) - mn + 1
    nb = learn.brick_grid(mn, mx)
    n_b = int(np.prod(nb))
    rng = np.random.default_rng(9)
    pick = rng.choice(n_b, size=max(1, n_b // 10), replace=False)
    scores = np.full(n_b, -10.0, np.float32)
    scores[pick] = 10.0
    out, res = compute_mesh_sdf(tris, h, mn, mx, mode=MODE_LEARNED, path=PATH_FAST, brick_scores=scores,
                                mlp_budget=len(pick), mlp_threshold=0.5)
    assert res.ok and res.stats["proposed"] == len(pick) and res.stats["escalated"] == 0
    st, ref, sign, _ = oracle.fast_sdf(tris, h, mn, mx, fsm_mode=0, gwn_mode=1)
    assert st == oracle.OK
    unsigned = np.abs(ref)
    s2 = sign.copy()
    vox = s2.reshape(dims[2], dims[1], dims[0])
    for b in pick:
        bx, by, bz = b % nb[0], (b // nb[0]) % nb[1], b // (nb[0] * nb[1])
        vox[bz * 8:bz * 8 + 8, by * 8:by * 8 + 8, bx * 8:bx * 8 + 8] = 2
    oracle.fixup_unknown(tris, h, mn, dims, s2, dist=unsigned, gwn_mode=1)
    want = np.where(s2 == 1, -unsigned, unsigned).astype(np.float32)
    assert np.array_equal(out.view(np.uint32), want.view(np.uint32)), (
        f"{np.count_nonzero(out.view(np.uint32) != want.view(np.uint32))} voxels differ")


def test_learned_mode_escalates_where_plain_declines(engine, oracle):
    """A self-overlapping shell whose lens fills more of the lattice than the stratified
    probes tolerate: the plain fast path declines (the reference's fall-back case); learned
    mode re-decides the signs instead -- signed crossings, the exact winding number for rays
    through holes -- and every voxel off the surface gets the full winding number's side."""
    from gbsdf import MODE_LEARNED, MODE_REFERENCE, PATH_FAST, compute_mesh_sdf, meshgen

    v, f = meshgen.overlapping_spheres(30.0, 36.0)
    vf, mn, mx = meshgen.fit_to_lattice(v, (96, 64, 64), 1.0)
    tris = meshgen.to_triangles(vf, f)
    _, rp = compute_mesh_sdf(tris, 1.0, mn, mx, mode=MODE_REFERENCE, path=PATH_FAST, raise_on_error=False)
    assert rp.status == 4  # EVERIFY
    out, rl = compute_mesh_sdf(tris, 1.0, mn, mx, mode=MODE_LEARNED, path=PATH_FAST)
    assert rl.ok and rl.stats["escalated"] == 1
    dims = mx.astype(np.int64) - mn + 1
    vid = np.arange(0, out.size, 5, dtype=np.int64)
    w_in = oracle.gwn_sign_voxels(tris, 1.0, mn, dims, vid, mode=1)
    off = np.abs(out[vid]) > 1e-3
    assert np.count_nonzero(((out[vid] < 0) != (w_in == 1)) & off) == 0


def test_learned_batch_matches_single_calls(engine):
    """Learned mode in a planned batch (one CUDA graph, device-side proposal budget) gives
    each mesh's single-call grid bit for bit, with the same statuses, proposals and
    escalations -- a declining mesh included."""
    import torch

    from gbsdf import MODE_LEARNED, PATH_FAST, Batch, compute_mesh_sdf, learn, meshgen

    meshes = [(t, h, mn, mx) for t, h, mn, mx in learn.training_meshes(5, seed=777, grid=48)]
    v, f = meshgen.overlapping_spheres(30.0, 36.0)
    vf, mn, mx = meshgen.fit_to_lattice(v, (96, 64, 64), 1.0)
    meshes.append((meshgen.to_triangles(vf, f), 1.0, mn, mx))
    P = torch.from_numpy(np.load(learn.MODEL_PATH)["params"]).cuda()
    dm = [(torch.from_numpy(t).cuda(), h, a, b) for t, h, a, b in meshes]
    outs = [torch.empty(int(np.prod(b.astype(np.int64) - a + 1)), dtype=torch.float32, device="cuda")
            for _, _, a, b in meshes]
    with Batch(dm, outs=outs, mode=MODE_LEARNED, mlp_params=P) as bt:
        sts, stats = bt.run()
    assert all(s == 0 for s in sts), sts
    assert any(s["escalated"] for s in stats)
    for (t, h, a, b), o, s in zip(meshes, outs, stats):
        ref, r = compute_mesh_sdf(t, h, a, b, mode=MODE_LEARNED, path=PATH_FAST, mlp_params=P)
        assert r.ok
        assert r.stats["proposed"] == s["proposed"] and r.stats["escalated"] == s["escalated"]
        assert np.array_equal(o.cpu().numpy().view(np.uint32), ref.view(np.uint32))
