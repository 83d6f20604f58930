"""Learned sign-risk proposals: data, training and use of the brick-risk network.

The network (32 brick features -> 64 -> 64 -> 1, BF16 weights, FP32 accumulation; the
kernels are in csrc/k_learn.cu) scores each 8^3 brick's risk that the fast path's sign
there differs from the exact generalized winding number. In ``MODE_LEARNED`` the riskiest
bricks are re-decided by the exact winding kernel after the stratified probes and patch
boxes (which therefore run exactly as in the plain path, so a proposal can only replace a
sign by the exact one); the network never supplies a sign.

Labels come from the method itself: on a training lattice the plain fast path
(reference mode) and the legacy exact path (exact winding number at every voxel) are
both run, and a brick is positive when any of its voxels (off the surface) differs.

Usage (on a GPU):  python -m gbsdf.learn train --out gbsdf/sign_risk_mlp.npz
"""
from __future__ import annotations

import argparse
import ctypes as C
import math
from pathlib import Path

import numpy as np

from . import _lib, meshgen
from .api import GbsdfError

N_PARAMS = 6337
N_FEATURES = 32
HIDDEN = 64
MODEL_PATH = Path(__file__).resolve().parent / "sign_risk_mlp.npz"
SURFACE_TOL_VOXELS = 1e-5


def _err():
    return C.create_string_buffer(512)


def _check(rc, err):
    if rc != _lib.OK:
        raise GbsdfError(rc, err.value.decode(errors="replace"))


def init_params(seed: int = 0) -> np.ndarray:
    """He-uniform weights, zero biases, in the kernels' flat layout."""
    rng = np.random.default_rng(seed)
    p = np.zeros(N_PARAMS, np.float32)
    o = 0
    for fan_in, fan_out in ((N_FEATURES, HIDDEN), (HIDDEN, HIDDEN), (HIDDEN, 1)):
        lim = math.sqrt(6.0 / fan_in)
        p[o:o + fan_in * fan_out] = rng.uniform(-lim, lim, fan_in * fan_out)
        o += fan_in * fan_out + fan_out
    p[-1] = -2.0  # prior: most bricks are safe
    return p


def brick_grid(mn, mx):
    d = np.asarray(mx, np.int64) - np.asarray(mn, np.int64) + 1
    return tuple(int((x + 7) // 8) for x in d)


def brick_features(tris, h, mn, mx):
    """(n_bricks, 32) float32 CUDA tensor of the lattice's brick features."""
    import torch

    nb = brick_grid(mn, mx)
    nbr = nb[0] * nb[1] * nb[2]
    X = torch.empty((nbr, N_FEATURES), dtype=torch.float32, device="cuda")
    t = np.ascontiguousarray(tris, np.float32).reshape(-1, 12)
    L = _lib.load()
    err = _err()
    out_nb = (C.c_int32 * 3)()
    rc = L.gbsdf_brick_features(t.ctypes.data, len(t), float(h), (C.c_int32 * 3)(*map(int, mn)),
                                (C.c_int32 * 3)(*map(int, mx)), 0, X.data_ptr(), nbr, out_nb, err, len(err))
    _check(rc, err)
    return X


def voxel_mismatch(tris, h, mn, mx):
    """Voxels (off the surface) where the plain fast path's sign differs from the exact
    winding number: (mismatch bool array, plain grid, exact grid)."""
    from .api import MODE_REFERENCE, PATH_FAST, PATH_LEGACY, compute_mesh_sdf

    plain, r1 = compute_mesh_sdf(tris, h, mn, mx, mode=MODE_REFERENCE, path=PATH_FAST, raise_on_error=False)
    exact, _ = compute_mesh_sdf(tris, h, mn, mx, path=PATH_LEGACY)
    if not r1.ok:  # verification diverged: the plain path gave no grid
        return None, None, exact
    far = np.abs(exact) > SURFACE_TOL_VOXELS * h
    return (np.signbit(plain) != np.signbit(exact)) & far, plain, exact


def brick_labels(mismatch, mn, mx):
    """Per brick (x fastest): (label 0/1 float32, mismatched voxel count int32)."""
    d = (np.asarray(mx, np.int64) - np.asarray(mn, np.int64) + 1)[::-1]
    nb = brick_grid(mn, mx)[::-1]
    m = mismatch.reshape(d)
    m = np.pad(m, [(0, nb[i] * 8 - d[i]) for i in range(3)])
    cnt = m.reshape(nb[0], 8, nb[1], 8, nb[2], 8).sum(axis=(1, 3, 5), dtype=np.int32).ravel()
    return (cnt > 0).astype(np.float32), cnt


def training_meshes(n: int = 200, seed: int = 1000, grid: int = 72):
    """Seeded defective vessel trees and spherical-harmonic blobs with holes on small
    lattices: (tris, h, mn, mx) tuples."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        s = int(rng.integers(1 << 30))
        if i % 2 == 0:
            v, f = meshgen.vessel_tree(seed=s, levels=int(rng.integers(2, 4)), around=int(rng.integers(12, 25)),
                                       n_len=int(rng.integers(5, 10)), n_cap=2,
                                       hole_frac=float(rng.uniform(0.0, 0.02)), n_jitter=int(rng.integers(0, 40)),
                                       jitter_sigma=float(rng.uniform(0.1, 0.5)), dup_frac=0.01)
        else:
            v, f = meshgen.sh_blob(seed=s, n_lat=int(rng.integers(24, 48)), n_lon=int(rng.integers(48, 96)),
                                   degree=int(rng.integers(3, 9)), coeff_scale=float(rng.uniform(1.0, 6.0)),
                                   vertex_noise=float(rng.uniform(0.0, 0.3)),
                                   hole_frac=float(rng.uniform(0.0, 0.03)))
        g = int(rng.integers(grid - 16, grid + 17))
        dims = (g, int(rng.integers(g - 8, g + 9)), int(rng.integers(g - 8, g + 9)))
        h = float(rng.uniform(0.5, 2.0))
        vf, mn, mx = meshgen.fit_to_lattice(v, dims, h, offset_frac=tuple(rng.uniform(0, 1, 3)))
        out.append((meshgen.to_triangles(vf, f), h, mn, mx))
    return out


def dataset(meshes):
    """Stacked (features, labels, mismatched-voxel counts) CUDA tensors of the meshes'
    bricks."""
    import torch

    Xs, ys, cs = [], [], []
    for tris, h, mn, mx in meshes:
        mism, _, _ = voxel_mismatch(tris, h, mn, mx)
        if mism is None:
            continue
        y, cnt = brick_labels(mism, mn, mx)
        Xs.append(brick_features(tris, h, mn, mx))
        ys.append(torch.from_numpy(y).cuda())
        cs.append(torch.from_numpy(cnt).cuda())
    return torch.cat(Xs), torch.cat(ys), torch.cat(cs)


class SignRiskMLP:
    """FP32 master parameters on the device; forward / backward / Adam through the C ABI."""

    def __init__(self, params=None, seed: int = 0):
        import torch

        p = init_params(seed) if params is None else np.asarray(params, np.float32)
        assert p.shape == (N_PARAMS,)
        self.P = torch.from_numpy(p.copy()).cuda()
        self.m = torch.zeros_like(self.P)
        self.v = torch.zeros_like(self.P)
        self.step = 0

    def logits(self, X):
        import torch

        out = torch.empty(X.shape[0], dtype=torch.float32, device="cuda")
        err = _err()
        _check(_lib.load().gbsdf_mlp_forward(self.P.data_ptr(), X.data_ptr(), X.shape[0], out.data_ptr(), 0, err,
                                             len(err)), err)
        return out

    def grad(self, X, y, w=None):
        import torch

        g = torch.empty(N_PARAMS, dtype=torch.float32, device="cuda")
        loss = torch.empty(1, dtype=torch.float32, device="cuda")
        err = _err()
        _check(_lib.load().gbsdf_mlp_backward(self.P.data_ptr(), X.data_ptr(), y.data_ptr(),
                                              w.data_ptr() if w is not None else None, X.shape[0], g.data_ptr(),
                                              loss.data_ptr(), 0, err, len(err)), err)
        return g, float(loss.item())

    def adam(self, g, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8, scale=1.0):
        self.step += 1
        err = _err()
        _check(_lib.load().gbsdf_mlp_adam(self.P.data_ptr(), g.data_ptr(), self.m.data_ptr(), self.v.data_ptr(),
                                          lr, beta1, beta2, eps, scale, self.step, 0, err, len(err)), err)

    def fit(self, X, y, epochs=30, batch=4096, lr=2e-3, counts=None, seed=0, log=None):
        """Adam on the weighted cross-entropy. With ``counts`` (mismatched voxels per
        brick) a positive brick weighs 1 + its count, so the ranking favours the bricks
        that hold the most sign errors; otherwise positives weigh sqrt(neg / pos)."""
        import torch

        n = X.shape[0]
        if counts is not None:
            w = torch.where(y > 0.5, 1.0 + counts.float(), torch.ones_like(y))
        else:
            pos = float(y.sum().item())
            pw = max(1.0, (n - pos) / max(pos, 1.0)) ** 0.5
            w = torch.where(y > 0.5, torch.full_like(y, pw), torch.ones_like(y))
        gen = torch.Generator(device="cuda")
        gen.manual_seed(seed)
        hist = []
        for ep in range(epochs):
            perm = torch.randperm(n, device="cuda", generator=gen)
            tot = 0.0
            for i in range(0, n, batch):
                idx = perm[i:i + batch]
                Xb, yb, wb = X[idx].contiguous(), y[idx].contiguous(), w[idx].contiguous()
                g, loss = self.grad(Xb, yb, wb)
                self.adam(g, lr=lr, scale=1.0 / float(wb.sum().item()))
                tot += loss
            hist.append(tot / float(w.sum().item()))
            if log:
                log(f"epoch {ep}: loss {hist[-1]:.4f}")
        return hist

    def params(self) -> np.ndarray:
        return self.P.detach().cpu().numpy()

    def save(self, path=MODEL_PATH):
        np.savez_compressed(path, params=self.params())

    @staticmethod
    def load(path=MODEL_PATH) -> "SignRiskMLP":
        return SignRiskMLP(np.load(path)["params"])


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("cmd", choices=["train"])
    ap.add_argument("--out", default=str(MODEL_PATH))
    ap.add_argument("--meshes", type=int, default=200)
    ap.add_argument("--epochs", type=int, default=60)
    a = ap.parse_args()
    import torch

    torch.manual_seed(0)
    X, y, cnt = dataset(training_meshes(a.meshes))
    print(f"{X.shape[0]} bricks, {int(y.sum().item())} positive, {int(cnt.sum().item())} mismatched voxels")
    mlp = SignRiskMLP(seed=0)
    mlp.fit(X, y, epochs=a.epochs, counts=cnt, log=print)
    mlp.save(a.out)
    print("saved", a.out)


if __name__ == "__main__":
    main()
