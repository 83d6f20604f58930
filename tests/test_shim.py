"""The C++ shim (rhizome_v24.15_gb300/shim/cuda_rasterizer_gbsdf.cpp): the reference's two
CudaRasterizer statics on the engine's C ABI, compiled against the reference's own
headers (native/src/engine/sdf/cuda_rasterizer.hpp and what it includes, staged by
oracle/build_ref.sh, with the project's glm stand-in) and driven by tests/shim_check.cpp
the way the reference application calls them. The CPU test compiles and links it; the GPU
test compares its outputs with the C ABI's and checks the reference's vector contract:
resize to the lattice (new entries 1e6) before the attempt, false for no triangles after
that resize, false with the vector untouched for an empty lattice, nullptr for an empty
mesh."""
import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
STAGE = ROOT / "oracle" / "_ref" / "src"
LIBDIR = ROOT / "rhizome_v24.15_gb300" / "gbsdf"
needs_headers = pytest.mark.skipif(not (STAGE / "engine/sdf/cuda_rasterizer.hpp").exists(),
                                   reason="the reference's headers are not staged")


def _compile(out_dir: Path) -> Path:
    exe = out_dir / "shim_check"
    cmd = ["g++", "-std=c++20", "-O1", "-I", str(ROOT / "oracle/ref_shim"), "-I", str(STAGE), "-I",
           str(ROOT / "include"), str(ROOT / "rhizome_v24.15_gb300/shim/cuda_rasterizer_gbsdf.cpp"),
           str(ROOT / "tests/shim_check.cpp"), "-L", str(LIBDIR), "-lgbsdf", f"-Wl,-rpath,{LIBDIR}", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


@needs_headers
def test_shim_compiles_against_reference_headers(tmp_path):
    if not (LIBDIR / "libgbsdf.so").exists():
        pytest.skip("libgbsdf.so not built")
    assert _compile(tmp_path).exists()


@needs_headers
@pytest.mark.gpu
def test_shim_matches_c_abi_and_reference_contract(engine, tmp_path):
    from gbsdf import meshgen

    v, f = meshgen.mug(segments=64, n_bottom=3, n_wall=6, n_rim=1, handle_path=16, handle_around=12)
    vf, mn, mx = meshgen.fit_to_lattice(v, (40, 40, 44), 2.4)
    tris = meshgen.to_triangles(vf, f)
    h = 2.4
    verts = vf.astype(np.float32)
    idx = f.astype(np.uint32).reshape(-1)
    tris.tofile(tmp_path / "tris.bin")
    verts.tofile(tmp_path / "verts.bin")
    idx.tofile(tmp_path / "idx.bin")
    exe = _compile(tmp_path)
    args = [str(exe), str(tmp_path / "tris.bin"), str(len(tris)), repr(h), *map(str, mn), *map(str, mx),
            str(tmp_path / "verts.bin"), str(len(verts)), str(tmp_path / "idx.bin"), str(len(idx)), str(tmp_path) + "/"]
    r = subprocess.run(args, capture_output=True, text=True, env=dict(os.environ))
    assert r.returncode == 0, r.stderr
    rep = {ln.split()[0]: ln.split()[1:] for ln in (tmp_path / "report.txt").read_text().splitlines()}
    n = int(np.prod(mx.astype(np.int64) - mn + 1))
    # compute_mesh_sdf: the C ABI's result (reference mode, the reference's dispatch)
    assert rep["compute"] == ["1", str(n)]
    got = np.fromfile(tmp_path / "compute.bin", np.float32)
    want, res = engine.compute_mesh_sdf(tris, h, mn, mx)
    assert res.ok and np.array_equal(got.view(np.uint32), want.view(np.uint32))
    # no triangles: false after the resize; the first 3 entries kept, the rest 1e6
    assert rep["empty"] == ["0", str(n), str(n - 3), "1"]
    # an empty lattice: false, vector untouched, no time
    assert rep["inverted"] == ["0", "7", "0"]
    # build_from_mesh: the engine's lattice and grid, a fresh version
    b = rep["build"]
    assert b[0] == "1"
    lmn, lmx = engine.mesh_lattice(verts, h)
    assert list(map(int, b[1:4])) == list(lmn) and list(map(int, b[4:7])) == list(lmx)
    grid = np.fromfile(tmp_path / "build.bin", np.float32)
    out, mn2, mx2, rb = engine.build_from_mesh(verts, idx.reshape(-1, 3), h)
    assert rb.ok and np.array_equal(grid.view(np.uint32), np.asarray(out, np.float32).view(np.uint32))
    assert int(b[7]) >= 3
    assert rep["build_empty"] == ["0"]
