"""CPU checks of the mesh-decoder oracle (oracle/meshio_oracle.cpp): the binary STL weld
against an independent numpy restatement, the OBJ decode against the source mesh, and --
where the reference tree is present -- the reference's own mug specimen against the facts
its documentation states (1,553 vertices, 3,106 triangles, 100.0 x 76.5 x 85.0 mm)."""
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as O


def _weld_numpy(data):
    """First-occurrence weld on round(coordinate * 10000) keys, as a numpy program."""
    T = int(np.frombuffer(data[80:84], np.uint32)[0])
    rec = np.frombuffer(data[84:84 + 50 * T], dtype=[("n", "<f4", 3), ("v", "<f4", (3, 3)), ("a", "<u2")])
    corners = rec["v"].reshape(-1, 3)
    x = (corners * np.float32(10000.0)).astype(np.float32).astype(np.float64)
    keys = (np.sign(x) * np.floor(np.abs(x) + 0.5)).astype(np.int64)  # round half away from zero
    _, first, inverse = np.unique(keys, axis=0, return_index=True, return_inverse=True)
    order = np.argsort(first, kind="stable")  # unique keys in first-occurrence order
    rank = np.empty_like(order)
    rank[order] = np.arange(len(order))
    vid = rank[inverse.ravel()].reshape(-1, 3)
    keep = (vid[:, 0] != vid[:, 1]) & (vid[:, 1] != vid[:, 2]) & (vid[:, 2] != vid[:, 0])
    return corners[np.sort(first)], vid[keep].ravel().astype(np.uint32)


def _stl_cases():
    from gbsdf import meshgen

    rng = np.random.default_rng(0)
    v, f = meshgen.vessel_tree(seed=2, levels=2, around=12, n_len=5, n_cap=2, hole_frac=0.02, n_jitter=10,
                               dup_frac=0.05)
    f = np.concatenate([f, f[:5][:, [0, 0, 1]]])  # degenerate records (repeated corner)
    n = rng.normal(0, 1, (len(f), 3)).astype(np.float32)
    n[::7] = 0.0  # zero normals: geometric fallback
    yield meshgen.to_binary_stl(v, f, normals=n)
    # near-duplicates inside one quantisation step, and across one
    v2 = np.concatenate([v, v[:50] + np.float32(2e-5), v[:50] + np.float32(3e-4)])
    f2 = np.concatenate([f, f[:30] % 50 + len(v), f[:30] % 50 + len(v) + 50])
    yield meshgen.to_binary_stl(v2, f2)


def test_stl_weld_matches_numpy_restatement():
    for data in _stl_cases():
        st, verts, idx, normals = O.parse_binary_stl(data)
        assert st == 0
        wv, wi = _weld_numpy(data)
        assert np.array_equal(verts, wv) and np.array_equal(idx, wi)
        assert np.allclose(np.linalg.norm(normals, axis=1), 1.0, atol=1e-5)


def test_stl_malformed_and_empty():
    assert O.parse_binary_stl(b"x" * 50)[0] == 1
    head = b" " * 80
    assert O.parse_binary_stl(head + np.uint32(3).tobytes() + b"\0" * 100)[0] == 1  # truncated
    st, v, i, _ = O.parse_binary_stl(head + np.uint32(0).tobytes())
    assert st == 0 and len(v) == 0 and len(i) == 0


def test_obj_decode_matches_source_mesh():
    from gbsdf import meshgen

    v, f = meshgen.mug(segments=48, n_bottom=3, n_wall=5, n_rim=1, handle_path=12, handle_around=10)
    for seed in range(3):
        st, ov, oi = O.parse_obj(meshgen.to_obj_text(v, f, seed=seed))
        assert st == 0
        assert np.allclose(ov, v.astype(np.float32), rtol=0, atol=2e-5)
        assert np.array_equal(oi.reshape(-1, 3), f)  # quads split back into the source pairs
    assert O.parse_obj(b"# nothing\nvn 0 0 1\n")[0] == 1
    st, ov, oi = O.parse_obj(b"v 0 0 0\nv 1 0 0\nv 0 1 0\nv 0 0 1\nv 1 1 1\nf 1 2 3 4 5\nf 1 9 2\nf 0 1 2\n")
    # a pentagon keeps its first four corners (split in two); an index past the vertices is
    # kept as written; index 0 is skipped, leaving a two-corner face that is dropped
    assert st == 0 and oi.tolist() == [0, 1, 2, 0, 2, 3, 0, 8, 1]


# the reference's own specimen, staged by oracle/build_ref.sh from the reference tree
REF_MUG = Path(__file__).resolve().parent.parent / "oracle" / "_ref" / "assets" / "mug.obj"


@pytest.mark.skipif(not REF_MUG.exists(), reason="the reference's specimen is not staged")
def test_reference_mug_specimen():
    st, v, i = O.parse_obj(REF_MUG.read_bytes())
    assert st == 0 and len(v) == 1553 and len(i) == 3 * 3106
    ext = v.max(0) - v.min(0)
    assert np.allclose(ext, [100.0, 76.5, 85.0], atol=0.05)


def _mobius(n=24):
    th = 2 * np.pi * np.arange(n) / n
    v = []
    for t in th:
        for w in (-0.3, 0.3):
            r = 1 + w * np.cos(t / 2)
            v.append([r * np.cos(t), r * np.sin(t), w * np.sin(t / 2)])
    f = []
    for i in range(n):
        a, b = 2 * i, 2 * i + 1
        if i + 1 < n:
            c, d = 2 * (i + 1), 2 * (i + 1) + 1
        else:
            c, d = 1, 0  # the twist: the strip's sides swap where it closes
        f += [[a, b, d], [a, d, c]]
    return np.asarray(v, np.float32), np.asarray(f, np.int64)


def orient_cases():
    """(name, vertices, faces, expected source faces or None) cases of the pre-pass."""
    from gbsdf import meshgen

    rng = np.random.default_rng(7)
    v, f = meshgen.perturbed_sphere(seed=2, n_lat=24, n_lon=48)
    v = v.astype(np.float32)
    g = f.copy()
    fl = rng.random(len(g)) < 0.35
    g[fl] = g[fl][:, [0, 2, 1]]
    out = [("flipped", v, g, f), ("inverted", v, f[:, [0, 2, 1]], f)]
    v2 = np.concatenate([v, v + np.float32(200.0)])
    f2 = np.concatenate([f, (f + len(v))[:, [0, 2, 1]]])  # second shell inside out
    out.append(("two_shells", v2, f2, None))
    mv, mf = _mobius()
    out.append(("mobius", mv, mf, None))
    extra = np.c_[f[:4, 0], f[:4, 1], f[4:8, 2]]  # third users of four edges: non-manifold
    out.append(("nonmanifold", v, np.concatenate([f, extra]), None))
    return out


def test_orientation_oracle():
    for name, v, f, expect in orient_cases():
        idx, orientable, inconsistent, inverted, vol = O.orient_mesh(v, f)
        if expect is not None:
            assert np.array_equal(idx.reshape(-1, 3), expect), name
            assert orientable and vol > 0, name
        if name == "flipped":
            assert inconsistent
        if name == "inverted":
            assert inverted and not inconsistent
        if name == "mobius":
            assert not orientable and inconsistent


# ---- ASCII STL ----------------------------------------------------------------------
F32 = np.float32


def _atof(b, p):
    """device_fast_atof (cuda_mesh_io.cu:810-843) in float32 steps, each rounded once."""
    while b[p] in (32, 9):
        p += 1
    sign = F32(1)
    if b[p] == 45:
        sign, p = F32(-1), p + 1
    elif b[p] == 43:
        p += 1
    val = F32(0)
    while 48 <= b[p] <= 57:
        val = F32(F32(val * F32(10)) + F32(b[p] - 48))
        p += 1
    if b[p] == 46:
        p += 1
        factor = F32(0.1)
        while 48 <= b[p] <= 57:
            val = F32(val + F32(F32(b[p] - 48) * factor))
            factor = F32(factor * F32(0.1))
            p += 1
    if b[p] in (101, 69):
        p += 1
        es = F32(1)
        if b[p] == 45:
            es, p = F32(-1), p + 1
        elif b[p] == 43:
            p += 1
        ev = 0
        while 48 <= b[p] <= 57:
            ev = ev * 10 + (b[p] - 48)
            p += 1
        val = F32(val * F32(10.0 ** float(F32(es * F32(ev)))))
    return F32(sign * val), p


def _ascii_stl_python(text):
    """The reference's ASCII STL rules as a plain Python program (tokens, numbers, 64-bit
    weld key, first-occurrence numbering)."""
    n = len(text)
    if n < 15:
        return None
    b = text + b"\0"
    cap = 1024
    while cap < n // 12 + 1024 and cap < (1 << 26):
        cap <<= 1
    offs = []
    i = text.find(b"vertex")
    while i != -1:
        if i + 7 < n and (i == 0 or b[i - 1] in b" \t\n\r") and b[i + 6] in b" \t" and len(offs) < cap:
            offs.append(i + 6)
        i = text.find(b"vertex", i + 1)
    m = len(offs) - len(offs) % 3
    if m == 0:
        return None
    raw = np.zeros((m, 3), np.float32)
    for k in range(m):
        p = offs[k]
        for c in range(3):
            raw[k, c], p = _atof(b, p)
    x = (raw * F32(10000.0)).astype(np.float64)
    q = (np.sign(x) * np.floor(np.abs(x) + 0.5)).astype(np.int64).astype(np.int32)
    u = q.view(np.uint32).astype(np.uint64)
    with np.errstate(over="ignore"):
        key = ((u[:, 0] * np.uint64(73856093)) ^ (u[:, 1] * np.uint64(19349663)) ^ (u[:, 2] * np.uint64(83492791)) ^
               ((u[:, 0] & np.uint64(0xFFFFF)) << np.uint64(42)) ^ ((u[:, 1] & np.uint64(0xFFFFF)) << np.uint64(21)) ^
               (u[:, 2] & np.uint64(0x1FFFFF)))
    key[key == 0] = 1
    ids, verts, idx = {}, [], []
    for k in range(m):
        kk = int(key[k])
        if kk not in ids:
            ids[kk] = len(verts)
            verts.append(raw[k])
        idx.append(ids[kk])
    return np.array(verts, np.float32).reshape(-1, 3), np.array(idx, np.uint32)


def ascii_stl_cases():
    from gbsdf import meshgen

    v, f = meshgen.mug(segments=24, n_bottom=2, n_wall=3, n_rim=1, handle_path=8, handle_around=6)
    yield meshgen.to_ascii_stl(v, f, fancy=False)
    yield meshgen.to_ascii_stl(v, f, seed=1)
    # near-duplicates inside one quantisation step (merged, first coordinates kept) and across one
    v2 = np.concatenate([v, v[:20] + F32(2e-5), v[:20] + F32(3e-4)])
    f2 = np.concatenate([f, f[:12] % 20 + len(v), f[:12] % 20 + len(v) + 20])
    yield meshgen.to_ascii_stl(v2, f2, seed=2)
    # token edge cases: a token at the text start, "endvertex" / "vertexx" / "xvertex" (not
    # tokens), tab after the keyword, a dangling eighth corner (cut to whole facets), and a
    # token in the last 7 bytes (ignored)
    yield (b"vertex 1 2 3\nvertex\t4 5 6 endvertex 7 7 7\n vertexx 9 9 9 xvertex 8 8 8\r\nvertex -1e1 .5 +2\n"
           b"\tvertex 1 2 3\n vertex 0 0 0\nvertex 3 2 1\nvertex 5 5 5\nvertex 6")
    # a solid named "vertex ..." (the reference's rule reads it as a vertex token, its
    # numbers as zeros), CR-only line ends, numbers with no digits and exponents (one underflowing to 0)
    yield (b"solid vertex model\rfacet normal 0 0 1\r outer loop\r  vertex 1 2 3\r  vertex - + .\r"
           b"  vertex 1e3 -2.5e-3 5e-324\r endloop\rendfacet\rendsolid vertex model\r")


def test_ascii_stl_oracle_matches_python_restatement():
    for text in ascii_stl_cases():
        st, ov, oi = O.parse_ascii_stl(text)
        want = _ascii_stl_python(text)
        assert st == 0 and want is not None
        assert np.array_equal(ov.view(np.uint32), want[0].view(np.uint32))
        assert np.array_equal(oi, want[1])
    st, ov, oi = O.parse_ascii_stl(next(iter(ascii_stl_cases())))
    from gbsdf import meshgen

    v, f = meshgen.mug(segments=24, n_bottom=2, n_wall=3, n_rim=1, handle_path=8, handle_around=6)
    # every corner kept, one vertex per source vertex, positions as written (6 decimals)
    assert len(ov) == len(v) and len(oi) == 3 * len(f)
    assert np.allclose(ov[oi].reshape(-1, 3, 3), v.astype(np.float32)[f], rtol=0, atol=2e-5)
    assert O.parse_ascii_stl(b"vertex 1 2 3")[0] == 1  # shorter than 15 bytes
    assert O.parse_ascii_stl(b"solid x\nvertex 1 2 3\nvertex 4 5 6\nendsolid x\n")[0] == 1  # no whole facet
