"""Seeded synthetic triangle meshes for the mesh-to-SDF workloads.

The reference ships one real specimen (``native/assets/mug.obj``) and no
benchmark data set, so every workload here is generated from a seed:

* ``mug``          -- thick-walled surface-of-revolution cup plus a swept-torus
                      handle whose ends are buried in the wall (two closed shells
                      that overlap, as in a procedural union without a boolean
                      clean-up; the overlap is where scanline parity and the
                      winding number disagree).
* ``vessel_tree``  -- branching tubes (bifurcation levels, branching angles,
                      radius decay), each tube a closed shell with hemispherical
                      caps, plus seeded defects: deleted triangles (holes),
                      jittered triangles (self-intersections) and duplicated
                      vertices (topological seams).
* ``sh_blob``      -- a sphere whose radius is perturbed by real spherical
                      harmonics of degrees 1..L with N(0, a/l) coefficients, plus
                      vertex noise and deleted triangles.
* ``perturbed_sphere`` -- low-order version of the blob, watertight.

Meshes are returned as ``(verts float32 (V,3), faces int64 (F,3))`` in mm with
outward-facing counter-clockwise winding. ``fit_to_lattice`` scales and centres
a mesh into a named lattice with the reference's 10-voxel pad
(``build_from_mesh``, cuda_rasterizer.cu:1358-1372) and a sub-voxel offset so
that no vertex sits exactly on a lattice point.
"""
from __future__ import annotations

import math

import numpy as np

__all__ = [
    "mug",
    "vessel_tree",
    "sh_blob",
    "perturbed_sphere",
    "overlapping_spheres",
    "fit_to_lattice",
    "signed_volume",
    "to_triangles",
    "workload",
    "batch_workload",
    "to_ascii_stl",
    "to_binary_stl",
    "to_obj_text",
    "WORKLOADS",
]


# ----------------------------------------------------------------------------------
# helpers
# ----------------------------------------------------------------------------------
def signed_volume(verts: np.ndarray, faces: np.ndarray) -> float:
    v = verts.astype(np.float64)
    a, b, c = v[faces[:, 0]], v[faces[:, 1]], v[faces[:, 2]]
    return float(np.einsum("ij,ij->i", a, np.cross(b, c)).sum() / 6.0)


def _orient_outward(verts, faces):
    if signed_volume(verts, faces) < 0:
        faces = faces[:, [0, 2, 1]]
    return faces


def _revolve(profile_rz: np.ndarray, segments: int):
    """Revolve a polyline (r, z) about the z axis. Points with r == 0 are poles."""
    verts = []
    ring_index = []
    for r, z in profile_rz:
        if r == 0.0:
            ring_index.append(("pole", len(verts)))
            verts.append((0.0, 0.0, z))
        else:
            start = len(verts)
            th = np.arange(segments) * (2.0 * math.pi / segments)
            for t in th:
                verts.append((r * math.cos(t), r * math.sin(t), z))
            ring_index.append(("ring", start))
    faces = []
    S = segments
    for i in range(len(profile_rz) - 1):
        ka, ia = ring_index[i]
        kb, ib = ring_index[i + 1]
        for j in range(S):
            jn = (j + 1) % S
            if ka == "pole" and kb == "ring":
                faces.append((ia, ib + j, ib + jn))
            elif ka == "ring" and kb == "pole":
                faces.append((ia + j, ib, ia + jn))
            elif ka == "ring" and kb == "ring":
                faces.append((ia + j, ib + j, ib + jn))
                faces.append((ia + j, ib + jn, ia + jn))
    return np.asarray(verts, np.float64), np.asarray(faces, np.int64)


def _sweep_tube(path: np.ndarray, binormal: np.ndarray, radius, around: int, caps: bool = True):
    """Sweep a circle along a polyline. ``binormal`` (3,) or (P,3) is a unit vector
    perpendicular to the path; the circle spans (normal, binormal). ``radius`` is a
    scalar or (P,) array. Flat fan caps close both ends."""
    P = len(path)
    tang = np.gradient(path, axis=0)
    tang /= np.linalg.norm(tang, axis=1, keepdims=True)
    bn = np.broadcast_to(np.asarray(binormal, np.float64), (P, 3)).copy()
    bn -= (bn * tang).sum(1, keepdims=True) * tang
    bn /= np.linalg.norm(bn, axis=1, keepdims=True)
    nm = np.cross(bn, tang)
    rad = np.broadcast_to(np.asarray(radius, np.float64), (P,))
    ph = np.arange(around) * (2.0 * math.pi / around)
    ring = (np.cos(ph)[None, :, None] * nm[:, None, :] + np.sin(ph)[None, :, None] * bn[:, None, :])
    verts = (path[:, None, :] + rad[:, None, None] * ring).reshape(-1, 3)
    faces = []
    A = around
    for i in range(P - 1):
        for j in range(A):
            jn = (j + 1) % A
            a, b, c, d = i * A + j, i * A + jn, (i + 1) * A + jn, (i + 1) * A + j
            faces.append((a, b, c))
            faces.append((a, c, d))
    faces = np.asarray(faces, np.int64)
    if caps:
        c0 = len(verts)
        c1 = c0 + 1
        verts = np.vstack([verts, path[0], path[-1]])
        f0 = [(c0, (j + 1) % A, j) for j in range(A)]
        f1 = [(c1, (P - 1) * A + j, (P - 1) * A + (j + 1) % A) for j in range(A)]
        faces = np.vstack([faces, np.asarray(f0 + f1, np.int64)])
    return verts, faces


def _concat(parts):
    vs, fs, off = [], [], 0
    for v, f in parts:
        vs.append(v)
        fs.append(f + off)
        off += len(v)
    return np.vstack(vs), np.vstack(fs)


def _subdiv(a, b, n):
    t = np.linspace(0.0, 1.0, n + 1)
    return a[None, :] * (1 - t[:, None]) + b[None, :] * t[:, None]


# ----------------------------------------------------------------------------------
# mug
# ----------------------------------------------------------------------------------
def mug(segments: int = 256, n_bottom: int = 6, n_wall: int = 14, n_rim: int = 2,
        handle_path: int = 28, handle_around: int = 32, r_out: float = 40.0,
        height: float = 95.0, wall: float = 3.0, floor: float = 4.0,
        handle_major: float = 22.0, handle_tube: float = 5.0):
    """Cup (surface of revolution) + swept-torus handle, two closed shells."""
    r_in = r_out - wall
    pts = [np.array([0.0, 0.0])]
    pts += list(_subdiv(np.array([0.0, 0.0]), np.array([r_out, 0.0]), n_bottom)[1:])
    pts += list(_subdiv(np.array([r_out, 0.0]), np.array([r_out, height]), n_wall)[1:])
    pts += list(_subdiv(np.array([r_out, height]), np.array([r_in, height]), n_rim)[1:])
    pts += list(_subdiv(np.array([r_in, height]), np.array([r_in, floor]), n_wall)[1:])
    pts += list(_subdiv(np.array([r_in, floor]), np.array([0.0, floor]), n_bottom)[1:])
    prof = np.asarray(pts)
    prof[-1, 0] = 0.0
    cup_v, cup_f = _revolve(prof, segments)
    cup_f = _orient_outward(cup_v, cup_f)

    # handle: straight stub from inside the wall, semicircle outward, stub back.
    z_mid = 0.5 * (floor + height) + 0.025 * height
    x_w = r_out - 0.5 * wall
    x_c = r_out + handle_tube + 1.0
    n_straight = max(2, handle_path // 8)
    n_arc = max(4, handle_path - 2 * n_straight)
    top = _subdiv(np.array([x_w, 0.0, z_mid + handle_major]), np.array([x_c, 0.0, z_mid + handle_major]),
                  n_straight)
    th = np.linspace(0.0, math.pi, n_arc + 1)[1:-1]
    arc = np.stack([x_c + handle_major * np.sin(th), np.zeros_like(th), z_mid + handle_major * np.cos(th)], 1)
    bot = _subdiv(np.array([x_c, 0.0, z_mid - handle_major]), np.array([x_w, 0.0, z_mid - handle_major]),
                  n_straight)
    path = np.vstack([top, arc, bot])
    hv, hf = _sweep_tube(path, np.array([0.0, 1.0, 0.0]), handle_tube, handle_around, caps=True)
    hf = _orient_outward(hv, hf)
    v, f = _concat([(cup_v, cup_f), (hv, hf)])
    return v.astype(np.float64), f


# ----------------------------------------------------------------------------------
# vessel tree
# ----------------------------------------------------------------------------------
def _rot_about(axis, angle):
    axis = axis / np.linalg.norm(axis)
    x, y, z = axis
    c, s = math.cos(angle), math.sin(angle)
    C = 1 - c
    return np.array([[c + x * x * C, x * y * C - z * s, x * z * C + y * s],
                     [y * x * C + z * s, c + y * y * C, y * z * C - x * s],
                     [z * x * C - y * s, z * y * C + x * s, c + z * z * C]])


def _capsule(p0, p1, radius, around, n_len, n_cap):
    """Closed tube from p0 to p1 with hemispherical caps (pole vertices)."""
    d = p1 - p0
    L = np.linalg.norm(d)
    t = d / L
    helper = np.array([1.0, 0.0, 0.0]) if abs(t[0]) < 0.9 else np.array([0.0, 1.0, 0.0])
    u = np.cross(t, helper)
    u /= np.linalg.norm(u)
    w = np.cross(t, u)
    rings = []
    # cap at p0: angles from -90deg (pole) to 0
    for k in range(1, n_cap + 1):
        a = -0.5 * math.pi + 0.5 * math.pi * k / (n_cap + 1)
        rings.append((p0 + t * radius * math.sin(a), radius * math.cos(a)))
    for k in range(n_len + 1):
        rings.append((p0 + d * (k / n_len), radius))
    for k in range(1, n_cap + 1):
        a = 0.5 * math.pi * k / (n_cap + 1)
        rings.append((p1 + t * radius * math.sin(a), radius * math.cos(a)))
    ph = np.arange(around) * (2 * math.pi / around)
    circ = np.cos(ph)[:, None] * u[None, :] + np.sin(ph)[:, None] * w[None, :]
    verts = [c + r * circ for c, r in rings]
    verts = np.vstack(verts + [(p0 - t * radius)[None, :], (p1 + t * radius)[None, :]])
    R = len(rings)
    A = around
    faces = []
    for i in range(R - 1):
        for j in range(A):
            jn = (j + 1) % A
            a, b, c, dd = i * A + j, i * A + jn, (i + 1) * A + jn, (i + 1) * A + j
            faces.append((a, b, c))
            faces.append((a, c, dd))
    pole0, pole1 = R * A, R * A + 1
    for j in range(A):
        jn = (j + 1) % A
        faces.append((pole0, jn, j))
        faces.append((pole1, (R - 1) * A + j, (R - 1) * A + jn))
    faces = np.asarray(faces, np.int64)
    return verts, _orient_outward(verts, faces)


def vessel_tree(seed: int = 3, levels: int = 6, around: int = 48, n_len: int = 25, n_cap: int = 4,
                root_radius: float = 6.0, radius_decay: float = 0.75, root_length: float = 22.0,
                length_decay: float = 0.8, angle_lo: float = 25.0, angle_hi: float = 50.0,
                hole_frac: float = 0.005, n_jitter: int = 200, jitter_sigma: float = 0.3,
                dup_frac: float = 0.01, defects: bool = True):
    rng = np.random.default_rng(seed)
    parts = []
    stack = [(np.zeros(3), np.array([0.0, 0.0, 1.0]), root_radius, root_length, 0)]
    while stack:
        p0, direc, r, L, lev = stack.pop()
        p1 = p0 + direc * L
        parts.append(_capsule(p0, p1, r, around, n_len, n_cap))
        if lev < levels:
            helper = np.array([1.0, 0.0, 0.0]) if abs(direc[0]) < 0.9 else np.array([0.0, 1.0, 0.0])
            perp = np.cross(direc, helper)
            perp /= np.linalg.norm(perp)
            perp = _rot_about(direc, rng.uniform(0, 2 * math.pi)) @ perp
            for sgn in (+1.0, -1.0):
                ang = math.radians(rng.uniform(angle_lo, angle_hi))
                nd = _rot_about(perp, sgn * ang) @ direc
                stack.append((p1, nd / np.linalg.norm(nd), r * radius_decay, L * length_decay, lev + 1))
    v, f = _concat(parts)
    if defects:
        v, f = _defects(v, f, rng, hole_frac, n_jitter, jitter_sigma, dup_frac)
    return v, f


def _defects(v, f, rng, hole_frac, n_jitter, jitter_sigma, dup_frac):
    v = v.copy()
    F = len(f)
    # jitter: move the vertices of n_jitter random triangles (neighbours follow)
    if n_jitter > 0:
        tj = rng.choice(F, size=min(n_jitter, F), replace=False)
        vids = np.unique(f[tj].ravel())
        v[vids] += rng.normal(0.0, jitter_sigma, size=(len(vids), 3))
    # duplicated vertices: re-point half of the incident corners to a copy
    if dup_frac > 0:
        used = np.unique(f.ravel())
        nd = int(round(dup_frac * len(used)))
        pick = rng.choice(used, size=nd, replace=False)
        new_id = np.full(len(v), -1, np.int64)
        new_id[pick] = len(v) + np.arange(nd)
        v = np.vstack([v, v[pick]])
        f = f.copy()
        flat = f.ravel()
        cand = np.nonzero(new_id[flat] >= 0)[0]
        take = cand[rng.random(len(cand)) < 0.5]
        flat[take] = new_id[flat[take]]
        f = flat.reshape(-1, 3)
    # holes: delete triangles
    if hole_frac > 0:
        keep = np.ones(len(f), bool)
        keep[rng.choice(len(f), size=int(round(hole_frac * len(f))), replace=False)] = False
        f = f[keep]
    return v, f


# ----------------------------------------------------------------------------------
# spherical-harmonic blob / perturbed sphere
# ----------------------------------------------------------------------------------
def _real_sh_sum(theta, phi, coeffs):
    """sum_{l,m} c[l][m+l] * Y_lm(theta, phi), real orthonormal SH via the standard
    associated-Legendre recurrence (no Condon-Shortley phase)."""
    x = np.cos(theta)
    sx = np.sqrt(np.maximum(0.0, 1.0 - x * x))
    L = len(coeffs) - 1
    out = np.zeros_like(theta)
    # P[m][l] computed per m
    for m in range(0, L + 1):
        # P_m^m
        pmm = np.ones_like(x)
        fact = 1.0
        for _ in range(m):
            pmm = pmm * fact * sx
            fact += 2.0
        plm_prev, plm = None, pmm
        for l in range(m, L + 1):
            if l == m:
                plm = pmm
            elif l == m + 1:
                plm_prev, plm = plm, x * (2 * m + 1) * pmm
            else:
                plm_prev, plm = plm, ((2 * l - 1) * x * plm - (l + m - 1) * plm_prev) / (l - m)
            if l < 1:
                continue
            norm = math.sqrt((2 * l + 1) / (4 * math.pi) * math.factorial(l - m) / math.factorial(l + m))
            c = coeffs[l]
            if m == 0:
                out = out + c[l] * norm * plm
            else:
                out = out + math.sqrt(2.0) * norm * plm * (c[l + m] * np.cos(m * phi) + c[l - m] * np.sin(m * phi))
    return out


def _uv_sphere(n_lat: int, n_lon: int):
    th = np.linspace(0.0, math.pi, n_lat + 1)[1:-1]
    ph = np.arange(n_lon) * (2 * math.pi / n_lon)
    T, P = np.meshgrid(th, ph, indexing="ij")
    dirs = np.stack([np.sin(T) * np.cos(P), np.sin(T) * np.sin(P), np.cos(T)], -1).reshape(-1, 3)
    theta = np.concatenate([T.ravel(), [0.0, math.pi]])
    phi = np.concatenate([P.ravel(), [0.0, 0.0]])
    dirs = np.vstack([dirs, [[0, 0, 1.0], [0, 0, -1.0]]])
    R = n_lat - 1
    A = n_lon
    i = np.arange(R - 1)[:, None]
    j = np.arange(A)[None, :]
    jn = (j + 1) % A
    a, b, c, d = i * A + j, i * A + jn, (i + 1) * A + jn, (i + 1) * A + j
    quads = np.stack([np.stack([a, c, b], -1), np.stack([a, d, c], -1)], 2).reshape(-1, 3)
    npole, spole = R * A, R * A + 1
    jj = np.arange(A)
    top = np.stack([np.full(A, npole), jj, (jj + 1) % A], -1)
    botr = (R - 1) * A
    bot = np.stack([np.full(A, spole), botr + (jj + 1) % A, botr + jj], -1)
    faces = np.vstack([quads, top, bot]).astype(np.int64)
    return dirs, theta, phi, faces


def sh_blob(seed: int = 5, n_lat: int = 708, n_lon: int = 1414, base_radius: float = 50.0, degree: int = 12,
            coeff_scale: float = 2.0, vertex_noise: float = 0.05, hole_frac: float = 0.01):
    rng = np.random.default_rng(seed)
    dirs, theta, phi, faces = _uv_sphere(n_lat, n_lon)
    coeffs = [np.zeros(1)] + [rng.normal(0.0, coeff_scale / l, size=2 * l + 1) for l in range(1, degree + 1)]
    r = base_radius + _real_sh_sum(theta, phi, coeffs)
    v = dirs * r[:, None]
    if vertex_noise > 0:
        v = v + rng.normal(0.0, vertex_noise, size=v.shape)
    faces = _orient_outward(v, faces)
    if hole_frac > 0:
        keep = np.ones(len(faces), bool)
        keep[rng.choice(len(faces), size=int(round(hole_frac * len(faces))), replace=False)] = False
        faces = faces[keep]
    return v, faces


def perturbed_sphere(seed: int = 4, n_lat: int = 64, n_lon: int = 128, base_radius: float = 30.0,
                     degree: int = 4, coeff_scale: float = 3.0):
    rng = np.random.default_rng(seed)
    dirs, theta, phi, faces = _uv_sphere(n_lat, n_lon)
    coeffs = [np.zeros(1)] + [rng.normal(0.0, coeff_scale / l, size=2 * l + 1) for l in range(1, degree + 1)]
    r = base_radius + _real_sh_sum(theta, phi, coeffs)
    v = dirs * r[:, None]
    return v, _orient_outward(v, faces)


def overlapping_spheres(radius: float = 30.0, distance: float = 56.0, n_lat: int = 48, n_lon: int = 96):
    """Two closed spheres whose shells overlap in a lens (centres `distance` apart on x),
    not merged: every ray through the lens crosses four shells, so scanline parity calls
    the lens outside while its winding number is 2 -- the self-overlap divergence the
    reference's stratified probes and patch boxes exist for (cuda_rasterizer.cu:1067-1132).
    A small lens gives a few probe sites and one patch round; a large one more sites than
    the reference's give-up cap."""
    dirs, _, _, faces = _uv_sphere(n_lat, n_lon)
    v = dirs * radius
    off = np.array([distance / 2.0, 0.0, 0.0])
    verts = np.vstack([v - off, v + off])
    f = _orient_outward(v, faces)
    return verts, np.vstack([f, f + len(v)])


# ----------------------------------------------------------------------------------
# lattice placement / triangle soup
# ----------------------------------------------------------------------------------
def fit_to_lattice(verts, dims, h, pad_voxels: float = 10.0, span: float | None = None,
                   offset_frac=(0.1234567, 0.2345678, 0.3456789)):
    """Scale and centre ``verts`` into the lattice ``dims`` at voxel size ``h``.

    With ``span`` None the mesh plus ``pad_voxels`` on each side fills the tightest
    axis; otherwise the mesh's largest extent is ``span`` x the lattice extent.
    Returns ``(verts float32, min_coord (3,) int, max_coord (3,) int)``; the lattice
    point (i, j, k) is the world point ((min+i) h, (min+j) h, (min+k) h).
    """
    dims = np.asarray(dims, np.int64)
    v = np.asarray(verts, np.float64)
    lo, hi = v.min(0), v.max(0)
    ext = hi - lo
    if span is None:
        avail = (dims - 1 - 2 * pad_voxels) * h
        s = float(np.min(avail / np.maximum(ext, 1e-12)))
    else:
        s = float(span * (dims.min() - 1) * h / ext.max())
    mn = -(dims // 2)
    mx = mn + dims - 1
    center_world = (mn + (dims - 1) / 2.0) * h + np.asarray(offset_frac) * h
    v = (v - (lo + hi) / 2.0) * s + center_world
    return v.astype(np.float32), mn.astype(np.int32), mx.astype(np.int32)


def to_triangles(verts, faces):
    """(T, 12) float32 triangle soup in the reference's CudaTriangle layout
    (v0, v1, v2, unit normal), degenerate faces (|cross|^2 <= 1e-12) dropped in index
    order (the rule of dev_try_build_cuda_triangle, math_utils.cuh:484-514)."""
    v = np.asarray(verts, np.float32)
    f = np.asarray(faces, np.int64)
    a, b, c = v[f[:, 0]], v[f[:, 1]], v[f[:, 2]]
    n = np.cross(b - a, c - a).astype(np.float32)
    l2 = (n * n).sum(1, dtype=np.float32)
    keep = l2 > np.float32(1e-12)
    n = n[keep] / np.sqrt(l2[keep])[:, None]
    return np.concatenate([a[keep], b[keep], c[keep], n], 1).astype(np.float32)


# ----------------------------------------------------------------------------------
# named workloads (the five configurations of the benchmark plan)
# ----------------------------------------------------------------------------------
WORKLOADS = {
    # name: (generator kwargs, dims, voxel size)
    "mug_c1_128": (dict(kind="mug", segments=256, n_bottom=6, n_wall=14, n_rim=2, handle_path=28,
                        handle_around=32), (128, 128, 128), 0.8),
    "mug_c2_860": (dict(kind="mug", segments=768, n_bottom=16, n_wall=37, n_rim=4, handle_path=96,
                        handle_around=64), (860, 860, 880), 0.1),
    "vessel_c3_512": (dict(kind="vessel", seed=3), (512, 512, 512), 0.15),
    "blob_c5_1024": (dict(kind="blob", seed=5), (1024, 1024, 1024), 0.1),
}


def to_binary_stl(verts, faces, normals=None, header: bytes = b"gbsdf binary STL") -> bytes:
    """Binary STL bytes (80-byte header, uint32 count, 50-byte records) of an indexed mesh;
    ``normals`` (T,3) defaults to the unnormalised face normals."""
    v = np.asarray(verts, np.float32)
    f = np.asarray(faces, np.int64).reshape(-1, 3)
    tri = v[f]
    if normals is None:
        normals = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    rec = np.zeros(len(f), dtype=[("n", "<f4", 3), ("v", "<f4", (3, 3)), ("attr", "<u2")])
    rec["n"] = np.asarray(normals, np.float32)
    rec["v"] = tri
    return header[:80].ljust(80, b" ") + np.uint32(len(f)).tobytes() + rec.tobytes()


def to_ascii_stl(verts, faces, seed: int = 0, fancy: bool = True) -> bytes:
    """ASCII STL text of an indexed mesh (solid / facet normal / outer loop / vertex lines).
    With ``fancy`` the writer varies the spellings the decoder must accept: indentation by
    spaces or tabs, tabs between numbers, CRLF line ends, signs and exponents."""
    rng = np.random.default_rng(seed)
    v = np.asarray(verts, np.float32)
    f = np.asarray(faces, np.int64).reshape(-1, 3)
    tri = v[f]
    nrm = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    out = ["solid gbsdf\n"]
    for t in range(len(f)):
        eol = "\r\n" if fancy and rng.random() < 0.1 else "\n"
        out.append("  facet normal %.6e %.6e %.6e%s    outer loop%s" % (nrm[t, 0], nrm[t, 1], nrm[t, 2], eol, eol))
        for k in range(3):
            p = tri[t, k]
            r = rng.random() if fancy else 1.0
            if r < 0.1:
                out.append("\tvertex\t%+.6e\t%.7g %.9g%s" % (p[0], p[1], p[2], eol))
            elif r < 0.2:
                out.append("      vertex %.8e %.8e %.8e%s" % (p[0], p[1], p[2], eol))
            else:
                out.append("      vertex %.6f %.6f %.6f%s" % (p[0], p[1], p[2], eol))
        out.append("    endloop%s  endfacet%s" % (eol, eol))
    out.append("endsolid gbsdf\n")
    return "".join(out).encode()


def to_obj_text(verts, faces, seed: int = 0, fancy: bool = True) -> bytes:
    """OBJ text of an indexed mesh. With ``fancy`` the writer varies the spellings the
    decoders must accept: comments, normals / texture lines, v/vt/vn face tokens, negative
    (relative) indices, tabs between numbers, CRLF line ends, signs, exponents and quads
    ("v" and "f" are always followed by a space: the reference recognises only those)."""
    rng = np.random.default_rng(seed)
    v = np.asarray(verts, np.float32)
    f = np.asarray(faces, np.int64).reshape(-1, 3)
    out = ["# gbsdf OBJ writer\n", "o mesh\n"]
    for i, p in enumerate(v):
        if fancy and rng.random() < 0.1:
            out.append("vn 0 0 1\n")
        if fancy and rng.random() < 0.2:
            out.append("v %+.6e\t%.7g  %.9g\r\n" % (p[0], p[1], p[2]))
        else:
            out.append("v %.6f %.6f %.6f\n" % (p[0], p[1], p[2]))
    nv = len(v)
    k = 0
    while k < len(f):
        a, b, c = (int(x) for x in f[k])
        if fancy and k + 1 < len(f) and rng.random() < 0.1 and f[k + 1][0] == a and f[k + 1][1] == c:
            d = int(f[k + 1][2])  # (a, b, c) + (a, c, d) written as one quad
            out.append("f %d %d %d %d\n" % (a + 1, b + 1, c + 1, d + 1))
            k += 2
            continue
        r = rng.random() if fancy else 1.0
        if r < 0.15:
            out.append("f %d/%d/%d %d/%d/%d %d/%d/%d\n" % (a + 1, 1, 1, b + 1, 1, 1, c + 1, 1, 1))
        elif r < 0.25:
            out.append("f %d %d %d\n" % (a - nv, b - nv, c - nv))
        elif r < 0.3:
            out.append("f %d//1\t%d//1 %d//1\r\n" % (a + 1, b + 1, c + 1))
        else:
            out.append("f %d %d %d\n" % (a + 1, b + 1, c + 1))
        k += 1
    return "".join(out).encode()


def batch_workload(seed: int = 4, n: int = 64, t_lo: float = 2000.0, t_hi: float = 300000.0, g_lo: int = 64,
                   g_hi: int = 384):
    """Batched workload: ``n`` meshes cycling through the mug, vessel-tree and perturbed-
    sphere generators, triangle counts log-uniform in [t_lo, t_hi], cubic lattices with
    edges uniform in [g_lo, g_hi] and the mesh spanning 90% of its lattice (voxel size 1).
    Returns a list of (tris, voxel_size, min_coord, max_coord)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        t = float(np.exp(rng.uniform(math.log(t_lo), math.log(t_hi))))
        g = int(rng.integers(g_lo, g_hi + 1))
        s = int(rng.integers(1 << 30))
        kind = i % 3
        if kind == 0:
            f = math.sqrt(t / 23300.0)
            v, fc = mug(segments=max(16, round(256 * f)), n_bottom=max(1, round(6 * f)), n_wall=max(2, round(14 * f)),
                        n_rim=max(1, round(2 * f)), handle_path=max(8, round(28 * f)),
                        handle_around=max(8, round(32 * f)))
        elif kind == 1:
            levels = int(np.clip(round(math.log2(max(t, 1.0) / 3000.0)), 1, 6))
            per = t / (2 ** (levels + 1) - 1)
            k = max(1.0, math.sqrt(per / 40.0))
            v, fc = vessel_tree(seed=s, levels=levels, around=max(8, round(4 * k)), n_len=max(2, round(3 * k)),
                                n_cap=max(1, round(k)), defects=False)
        else:
            nl = max(8, round(math.sqrt(t / 4.0)))
            v, fc = perturbed_sphere(seed=s, n_lat=nl, n_lon=2 * nl)
        vf, mn, mx = fit_to_lattice(v, (g, g, g), 1.0, span=0.9)
        out.append((to_triangles(vf, fc), 1.0, mn, mx))
    return out


def _generate(kind, **kw):
    if kind == "mug":
        return mug(**kw)
    if kind == "vessel":
        return vessel_tree(**kw)
    if kind == "blob":
        return sh_blob(**kw)
    if kind == "sphere":
        return perturbed_sphere(**kw)
    raise ValueError(kind)


def workload(name: str, dims=None, h=None, **over):
    """Generate a named workload: returns (tris (T,12) f32, min_coord, max_coord, h)."""
    kw, d0, h0 = WORKLOADS[name]
    kw = dict(kw)
    kw.update(over)
    dims = d0 if dims is None else dims
    h = h0 if h is None else h
    v, f = _generate(**kw)
    vf, mn, mx = fit_to_lattice(v, dims, h)
    return to_triangles(vf, f), mn, mx, float(h)
