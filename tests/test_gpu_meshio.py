"""GPU mesh decoders (csrc/k_io.cu) through the C ABI against the oracle's restatement of
the reference's decoders: binary STL (decode, normals, GPU weld) and OBJ text, bit for bit
(OBJ numbers written with exponents within one ulp: the exponent scale is powf on both
sides, CUDA's and the C library's)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _stl_cases():
    from gbsdf import meshgen

    rng = np.random.default_rng(1)
    v, f = meshgen.vessel_tree(seed=5, levels=3, around=16, n_len=6, n_cap=2, hole_frac=0.01, n_jitter=20,
                               dup_frac=0.05)
    f = np.concatenate([f, f[:9][:, [0, 1, 1]]])
    n = rng.normal(0, 1, (len(f), 3)).astype(np.float32)
    n[::5] = 0.0
    yield meshgen.to_binary_stl(v, f, normals=n)
    v2, f2 = meshgen.mug(segments=96, n_bottom=4, n_wall=8, n_rim=1, handle_path=20, handle_around=16)
    v2 = np.concatenate([v2, v2[:80] + np.float32(1e-5), v2[:80] + np.float32(5e-4)])
    f2 = np.concatenate([f2, f2[:60] % 80 + len(v2) - 160, f2[:60] % 80 + len(v2) - 80])
    yield meshgen.to_binary_stl(v2, f2)
    v3, f3 = meshgen.perturbed_sphere(seed=3, n_lat=200, n_lon=400)  # ~160k triangles
    yield meshgen.to_binary_stl(v3, f3)


def test_binary_stl_matches_oracle(engine, oracle):
    for data in _stl_cases():
        v, i, n = engine.parse_binary_stl(data, normals=True)
        st, ov, oi, on = oracle.parse_binary_stl(data)
        assert st == 0
        assert np.array_equal(v.view(np.uint32), ov.view(np.uint32))
        assert np.array_equal(i, oi)
        assert np.array_equal(n.view(np.uint32), on.view(np.uint32))


def test_binary_stl_errors(engine):
    head = b" " * 80
    with pytest.raises(engine.GbsdfError):
        engine.parse_binary_stl(head + np.uint32(4).tobytes() + b"\0" * 120)
    v, i = engine.parse_binary_stl(head + np.uint32(0).tobytes())
    assert len(v) == 0 and len(i) == 0


def _ulps(a, b):
    ia = a.view(np.int32).astype(np.int64)
    ib = b.view(np.int32).astype(np.int64)
    return np.abs(ia - ib)


def test_obj_matches_oracle(engine, oracle):
    from gbsdf import meshgen

    v, f = meshgen.mug(segments=128, n_bottom=5, n_wall=10, n_rim=2, handle_path=24, handle_around=20)
    plain = meshgen.to_obj_text(v, f, fancy=False)
    gv, gi = engine.parse_obj(plain)
    st, ov, oi = oracle.parse_obj(plain)
    assert st == 0
    assert np.array_equal(gv.view(np.uint32), ov.view(np.uint32)) and np.array_equal(gi, oi)
    for seed in range(4):
        text = meshgen.to_obj_text(v, f, seed=seed)
        gv, gi = engine.parse_obj(text)
        st, ov, oi = oracle.parse_obj(text)
        assert st == 0
        assert np.array_equal(gi, oi)
        assert _ulps(gv, ov).max() <= 1
    edge = b"v 0 0 0\r\nv 1 0 0\nv 0 1 0\nv 0 0 1\nv 1 1 1\nf 1 2 3 4 5\nf 1 9 2\nf 0 1 2\nf -1 -2 -3"
    gv, gi = engine.parse_obj(edge)
    st, ov, oi = oracle.parse_obj(edge)
    assert st == 0 and np.array_equal(gi, oi) and np.array_equal(gv, ov)
    with pytest.raises(engine.GbsdfError):
        engine.parse_obj(b"# no geometry\nvn 0 0 1\n")


def test_decoded_mesh_builds_the_same_sdf(engine):
    """The decoded STL feeds build_from_mesh: same grid as the source indexed mesh."""
    from gbsdf import meshgen

    v, f = meshgen.mug(segments=64, n_bottom=3, n_wall=6, n_rim=1, handle_path=16, handle_around=12)
    v = v.astype(np.float32)
    dv, di = engine.parse_binary_stl(meshgen.to_binary_stl(v, f))
    a, mn, mx, _ = engine.build_from_mesh(v, f.astype(np.uint32).ravel(), 2.0)
    b, mn2, mx2, _ = engine.build_from_mesh(dv, di, 2.0)
    assert np.array_equal(mn, mn2) and np.array_equal(mx, mx2)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_orientation_matches_oracle(engine, oracle):
    from test_meshio_oracle import orient_cases

    for name, v, f, _ in orient_cases():
        gi, go, gc, gw, gv = engine.orient_mesh(v, f)
        oi, oo, oc, ow, ov = oracle.orient_mesh(v, f)
        assert (go, gc) == (oo, oc), name
        if oo:  # orientable: the orientation, hence the volume and the inversion, is unique
            assert gw == ow and np.array_equal(gi, oi), name
            assert abs(gv - ov) <= 1e-9 * max(1.0, abs(ov)), name


def test_orientation_large_component(engine, oracle):
    """A component whose diameter is far beyond 256 links converges (the reference's loop
    stops after 256 steps)."""
    from gbsdf import meshgen

    v, f = meshgen.perturbed_sphere(seed=5, n_lat=400, n_lon=800)
    rng = np.random.default_rng(3)
    g = f.copy()
    fl = rng.random(len(g)) < 0.5
    g[fl] = g[fl][:, [0, 2, 1]]
    gi, go, gc, gw, gv = engine.orient_mesh(v.astype(np.float32), g)
    assert go and gc and gv > 0
    assert np.array_equal(gi.reshape(-1, 3), f)


def test_ascii_stl_matches_oracle(engine, oracle):
    """ASCII STL: token finding, numbers and the 64-bit-key weld against the oracle (numbers
    written with exponents within one ulp: powf on both sides), on the oracle's edge cases
    and a ~160k-triangle sphere."""
    from gbsdf import meshgen
    from test_meshio_oracle import ascii_stl_cases

    v3, f3 = meshgen.perturbed_sphere(seed=3, n_lat=200, n_lon=400)
    cases = list(ascii_stl_cases()) + [meshgen.to_ascii_stl(v3, f3, seed=4)]
    for k, text in enumerate(cases):
        gv, gi = engine.parse_ascii_stl(text)
        st, ov, oi = oracle.parse_ascii_stl(text)
        assert st == 0
        assert np.array_equal(gi, oi), k
        assert _ulps(gv, ov).max() <= (0 if k == 0 else 1), k
    with pytest.raises(engine.GbsdfError):
        engine.parse_ascii_stl(b"vertex 1 2 3")
    with pytest.raises(engine.GbsdfError):
        engine.parse_ascii_stl(b"solid x\nvertex 1 2 3\nvertex 4 5 6\nendsolid x\n")


def test_parse_stl_front_end(engine):
    """StlParser::parse: binary when the header count fits the file, else ASCII; both
    oriented; the two encodings of one mesh give the same triangles."""
    from gbsdf import meshgen

    v, f = meshgen.mug(segments=64, n_bottom=3, n_wall=6, n_rim=1, handle_path=16, handle_around=12)
    v = v.astype(np.float32)
    rng = np.random.default_rng(7)
    g = f.copy()
    fl = rng.random(len(g)) < 0.3
    g[fl] = g[fl][:, [0, 2, 1]]  # scrambled winding: the front end orients it back
    bv, bi, bo = engine.parse_stl(meshgen.to_binary_stl(v, g))
    av, ai, ao = engine.parse_stl(meshgen.to_ascii_stl(v, g, fancy=False))
    assert bo and ao
    assert np.array_equal(bi, ai)  # same welding and orientation
    assert np.allclose(bv, av, rtol=0, atol=2e-5)
    assert np.array_equal(bv[bi.reshape(-1, 3)], v[f])  # the source's outward winding restored
    with pytest.raises(engine.GbsdfError):
        engine.parse_stl(b"solid tiny\n")
