"""Parity at the full-size workload configurations, against the oracle (CPU restatement).

* 64-mesh batch (mug / vessel tree / perturbed sphere, 2k-300k triangles, cubic lattices of
  64-384, 0.97G voxels): in plain (reference) mode every status, probe, site, patch-round,
  patched-voxel and band count equals the oracle's, the 20 declines included, and every
  built grid's signs equal the oracle's; in exact-signs mode the same, plus the whole
  distance field bit for bit on every fourth mesh.
* 512^3 defective vessel tree (412k triangles, holes, jitter, duplicated vertices),
  exact-signs: statistics and every sign equal to the oracle's, the distance field bit
  for bit against the oracle's band splat + eikonal over the whole lattice, and 4,096
  sampled voxels (band voxels included) on the side of the FP64 winding number.
* 1024^3 spherical-harmonic blob (1.98M triangles, 1% holes), exact-signs: statistics and
  every sign equal to the oracle's, and the band distances of four 128^3 windows bit for
  bit against the oracle's splat + eikonal run on the window with a 16-voxel margin.

The oracle here skips what cannot change the compared quantities (see ``fast_sdf``'s
``skip_eikonal`` and ``lazy_winding``): voxels it leaves to the winding number (columns
through holes, patch boxes) are checked on samples against its exact winding decision.
"""
import numpy as np
import pytest

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

KEYS = ("unknown_columns", "fixup_voxels", "probes", "sites", "patch_rounds", "patched_voxels", "band_voxels")
TOL_PLAIN, TOL_EXACT = 1e-5, 1e-3  # surface tolerances (voxel): on-surface voxels count as inside


def _dims(mn, mx):
    return np.asarray(mx, np.int64) - np.asarray(mn, np.int64) + 1


def _check_signs(oracle, tris, h, mn, mx, out, osign, tol, n_lazy, seed):
    """Signs of the built grid ``out`` against the oracle's: identical on every voxel the
    oracle decided; on up to ``n_lazy`` sampled voxels it left to the winding number, its
    exact winding decision (on-surface voxels inside). Returns the count of left voxels."""
    neg = np.signbit(out)
    lz = osign == 3
    bad = np.count_nonzero(neg[~lz] != (osign[~lz] == 1))
    assert bad == 0, f"{bad} signs differ from the oracle's"
    li = np.nonzero(lz)[0]
    if len(li):
        rng = np.random.default_rng(seed)
        vid = np.sort(rng.choice(li, size=min(n_lazy, len(li)), replace=False))
        w = oracle.gwn_sign_voxels(tris, h, mn, _dims(mn, mx), vid, mode=1)
        want = (w == 1) | (np.abs(out[vid]) <= tol * h)
        assert np.array_equal(neg[vid], want), f"{np.count_nonzero(neg[vid] != want)} sampled winding signs differ"
    return len(li)


def _stats_equal(got, ost, tag):
    for k in KEYS:
        assert got[k] == ost[k], (tag, k, got[k], ost[k])


def test_batch64_matches_oracle(engine, oracle):
    import torch

    from gbsdf import Batch, meshgen

    meshes = meshgen.batch_workload()
    dm = [(torch.from_numpy(t).cuda(), h, a, b) for t, h, a, b in meshes]
    outs = [torch.empty(int(np.prod(_dims(a, b))), dtype=torch.float32, device="cuda") for _, _, a, b in meshes]
    full = lazy_e = 0
    with Batch(dm, outs=outs, mode=engine.MODE_EXACT_SIGNS) as bt:
        sts, stats = bt.run()
    assert all(s == 0 for s in sts), sts
    for i, ((t, h, a, b), o, sp) in enumerate(zip(meshes, outs, stats)):
        got = o.cpu().numpy()
        whole = i % 4 == 0
        st, ref, osign, ost = oracle.fast_sdf(t, h, a, b, fsm_mode=0, gwn_mode=1, signed_parity=True,
                                              skip_eikonal=not whole, lazy_winding=True)
        assert st == oracle.OK, i
        _stats_equal(sp, ost, ("exact", i))
        lazy_e += _check_signs(oracle, t, h, a, b, got, osign, TOL_EXACT, 256, seed=i)
        if whole:
            assert sp["eikonal_rounds"] == ost["eikonal_rounds"], i
            assert np.array_equal(np.abs(got).view(np.uint32), np.abs(ref).view(np.uint32)), (
                f"mesh {i}: {np.count_nonzero(np.abs(got) != np.abs(ref))} distances differ")
            full += 1
    with Batch(dm, outs=outs, mode=engine.MODE_REFERENCE) as bt:
        sts, stats = bt.run()
    declined = lazy_p = 0
    for i, ((t, h, a, b), o, s, sp) in enumerate(zip(meshes, outs, sts, stats)):
        st, _, osign, ost = oracle.fast_sdf(t, h, a, b, fsm_mode=0, gwn_mode=1, skip_eikonal=True,
                                            lazy_winding=True)
        assert s == st, (i, s, st)
        _stats_equal(sp, ost, ("plain", i))
        if s == 0:
            lazy_p += _check_signs(oracle, t, h, a, b, o.cpu().numpy(), osign, TOL_PLAIN, 256, seed=100 + i)
        else:
            declined += 1
    print(f"64-mesh batch: exact-signs statistics and signs equal to the oracle's for all 64 "
          f"({lazy_e} voxels left to the winding number, sampled), distances bit for bit on {full}; "
          f"plain mode statuses and statistics equal for all 64, {declined} declined in both, "
          f"{lazy_p} patched voxels sampled")
    assert declined > 0


def test_vessel_512_exact_signs_matches_oracle(engine, oracle):
    from gbsdf import meshgen

    tris, mn, mx, h = meshgen.workload("vessel_c3_512")
    dims = _dims(mn, mx)
    out, res = engine.compute_mesh_sdf(tris, h, mn, mx, mode=engine.MODE_EXACT_SIGNS, path=engine.PATH_FAST)
    assert res.ok and res.stats["unknown_columns"] > 0
    st, odist, osign, ost = oracle.fast_sdf(tris, h, mn, mx, fsm_mode=0, gwn_mode=1, signed_parity=True,
                                            skip_eikonal=True, lazy_winding=True)
    del odist
    assert st == oracle.OK
    _stats_equal(res.stats, ost, "vessel")
    n_lazy = _check_signs(oracle, tris, h, mn, mx, out, osign, TOL_EXACT, 4096, seed=3)
    del osign
    # the whole distance field: the oracle's band splat and eikonal (signs play no part)
    g, _ = oracle.splat_band(tris, h, mn, dims)
    eik = oracle.eikonal(g, np.zeros(g.size, np.uint8), dims, h, fsm_mode=0)
    assert eik["far_residual"] == 0 and eik["rounds"] == res.stats["eikonal_rounds"]
    g[g > 1e29] = 1e6
    assert np.array_equal(np.abs(out).view(np.uint32), g.view(np.uint32)), (
        f"{np.count_nonzero(np.abs(out) != g)} distances differ")
    del g
    # the FP64 winding number on sampled voxels, half of them band voxels
    rng = np.random.default_rng(4)
    band = np.nonzero(np.abs(out) <= 8 * h)[0]
    vid = np.concatenate([rng.choice(out.size, 2048, replace=False), rng.choice(band, 2048, replace=False)])
    vid = vid[np.abs(out[vid]) > TOL_EXACT * h]
    x, y, z = vid % dims[0], (vid // dims[0]) % dims[1], vid // (dims[0] * dims[1])
    pts = ((mn[None, :] + np.stack([x, y, z], 1)).astype(np.float32) * np.float32(h)).astype(np.float32)
    w = oracle.gwn_points_f64(tris, pts)
    bad = np.count_nonzero(np.signbit(out[vid]) != (np.abs(w) >= 0.5))
    print(f"512^3 vessel tree: {len(tris)} triangles, {res.stats['unknown_columns']} columns through holes "
          f"({n_lazy} voxels, 4,096 sampled against the exact winding decision); signs and statistics equal to "
          f"the oracle's, distances bit for bit; {bad} of {len(vid)} sampled voxels off the FP64 winding number")
    assert bad == 0 and len(vid) >= 4000


def test_blob_1024_exact_signs_matches_oracle(engine, oracle):
    from gbsdf import meshgen

    tris, mn, mx, h = meshgen.workload("blob_c5_1024")
    dims = _dims(mn, mx)
    out, res = engine.compute_mesh_sdf(tris, h, mn, mx, mode=engine.MODE_EXACT_SIGNS, path=engine.PATH_FAST)
    assert res.ok
    st, odist, osign, ost = oracle.fast_sdf(tris, h, mn, mx, fsm_mode=0, gwn_mode=1, signed_parity=True,
                                            skip_eikonal=True, lazy_winding=True)
    del odist
    assert st == oracle.OK
    _stats_equal(res.stats, ost, "blob")
    n_lazy = _check_signs(oracle, tris, h, mn, mx, out, osign, TOL_EXACT, 4096, seed=5)
    del osign
    # band distances on 128^3 windows: a band value (<= 8 voxels) is lowered only through
    # chains of smaller neighbours, each link at least h/sqrt(3) lower, so a window run with
    # a 16-voxel margin holds the whole lattice's band values
    rng = np.random.default_rng(6)
    band = np.nonzero(np.abs(out) <= 8 * h)[0]
    V = out.reshape(dims[2], dims[1], dims[0])
    W, M = 128, 16
    n_band = lowered = 0
    for k in range(4):
        v = band[rng.integers(len(band))]
        c = np.array([v % dims[0], (v // dims[0]) % dims[1], v // (dims[0] * dims[1])])
        lo = np.clip(c - W // 2, M, dims - W - M)  # window [lo, lo+W) inside the margin
        cmn = mn + lo - M
        cd = np.full(3, W + 2 * M, np.int64)
        cg, _ = oracle.splat_band(tris, h, cmn, cd)
        cs = cg.copy()
        oracle.eikonal(cg, np.zeros(cg.size, np.uint8), cd, h, fsm_mode=0)
        inner = (slice(M, M + W),) * 3
        cg = cg.reshape(W + 2 * M, W + 2 * M, W + 2 * M)[inner]
        cs = cs.reshape(W + 2 * M, W + 2 * M, W + 2 * M)[inner]
        got = np.abs(V[lo[2]:lo[2] + W, lo[1]:lo[1] + W, lo[0]:lo[0] + W])
        sel = cs < 1e29
        assert np.array_equal(got[sel].view(np.uint32), cg[sel].view(np.uint32)), (
            f"window {k}: {np.count_nonzero(got[sel] != cg[sel])} band distances differ")
        n_band += int(sel.sum())
        lowered += int(np.count_nonzero(cg[sel] < cs[sel]))
    print(f"1024^3 blob: {len(tris)} triangles, signs and statistics equal to the oracle's ({n_lazy} voxels left "
          f"to the winding number, 4,096 sampled); {n_band} band voxels in four windows bit for bit "
          f"({lowered} lowered by the eikonal); stated band error {res.stats['band_err_fp64']:.2e} voxel "
          f"({res.stats['band_err_samples']} samples)")
    assert n_band > 0
    # coordinates reach 512 voxels from the origin: one FP32 ulp of a coordinate is 3.8e-5 voxel
    assert res.stats["band_err_samples"] > 100 and 0.0 <= res.stats["band_err_fp64"] <= 1e-4
