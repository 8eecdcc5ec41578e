"""Learned selectivity estimator: training data from the engine's own exact joins, and
training / evaluation through the rs_mlp_* kernels (csrc/rs_mlp.cu).

Dataset pairs follow the learned-estimator configuration: per side 1k..200k objects
(log-uniform; the default run uses a smaller range), a mix of level-1 icospheres and
boxes, radii log-uniform in [0.1, 50], centres from a Gaussian mixture of 1..32
components in a 1000^3 world.  For each pair the engine computes both 128^3 grids
(rs_grid_stats), the exact pair count (rs_overlap_join) and the grid estimator's count
(rs_estimate_grid + the reference's alpha correction).  The network learns the correction
log1p(pairs) - log1p(grid estimate) from the pooled grids (rs_mlp_set_prior makes
rs_estimate_mlp add the grid estimate back), with decoupled weight decay, early stopping
on a validation split and symmetry augmentation: the exact pair count of a dataset pair
does not change when the two sets swap roles or when the world cube is reflected or its
axes permuted (48 maps), and those maps carry the pooled 16^3 grids onto each other (16
blocks of 8 cells per axis; the four channels are scalars), so every minibatch draws one
of the 96 images of each sample.
"""
from __future__ import annotations

import ctypes
import dataclasses
from typing import List, Optional

import numpy as np
import torch

from . import _lib, api, gen

WORLD = 1000.0
RES = 128
N_FEAT = 32768


@dataclasses.dataclass
class Sample:
    features: torch.Tensor      # float32[32768] on the device
    pairs: int                  # exact pair count
    grid_estimate: int          # the grid estimator's count
    objects: tuple


def _cell_volume() -> float:
    f32 = np.float32
    c = f32(f32(WORLD) / f32(RES))
    return float(f32(f32(c * c) * c))


def grid_cells(dg: api.DeviceGeometry, n_obj: int, stream=None) -> torch.Tensor:
    cells = torch.empty(RES ** 3 * 16, dtype=torch.uint8, device=dg.V.device)
    api._check(_lib.load().rs_grid_stats(dg.V.data_ptr(), dg.nV, dg.I.data_ptr(), dg.nF, dg.T.data_ptr(), n_obj,
                                         RES, WORLD, cells.data_ptr(), None, api._stream(stream)), "rs_grid_stats")
    return cells


def dataset_side(seed: int, n_lo: int, n_hi: int, rng: np.random.Generator):
    n = int(np.exp(rng.uniform(np.log(n_lo), np.log(n_hi))))
    k = int(rng.integers(1, 33))
    centers = gen.mixture_centers(n, k, WORLD, seed)
    n_box = int(n * rng.uniform(0.0, 0.5))
    parts = []
    if n - n_box:
        parts.append(gen.instanced_set(n - n_box, 1, 0.1, 50.0, WORLD, seed=seed + 1, centers=centers[:n - n_box]))
    if n_box:
        parts.append(gen.instanced_set(n_box, 0, 0.1, 50.0, WORLD, seed=seed + 2, kind="box",
                                       centers=centers[n - n_box:]))
    return gen.concat(parts), n


def dataset_pair(seed: int, n_lo: int = 1000, n_hi: int = 200_000):
    """The two sets of dataset pair `seed`: (A, objects of A, B, objects of B)."""
    rng = np.random.default_rng(seed)
    A, na = dataset_side(4 * seed, n_lo, n_hi, rng)
    B, nb = dataset_side(4 * seed + 3, n_lo, n_hi, rng)
    return A, na, B, nb


def make_sample(seed: int, n_lo: int = 1000, n_hi: int = 200_000, stream=None) -> Sample:
    """One dataset pair: features, exact pair count, grid estimate."""
    A, na, B, nb = dataset_pair(seed, n_lo, n_hi)
    L = _lib.load()
    ca, cb = grid_cells(A, na, stream), grid_cells(B, nb, stream)
    cv = _cell_volume()
    raw, means = api.estimate_grid(ca, cb, RES ** 3, cv, stream=stream)
    est = int(L.rs_estimate_pairs_from_raw(raw, (ctypes.c_float * 4)(*means), cv, 1))
    ps = api.PairSet(api.hash_size_pow2(est), pow2=True, stream=stream)
    ba, bb = api.Bvh(A, stream=stream), api.Bvh(B, stream=stream)
    api.overlap_join(ba, bb, ps, stream=stream)
    _, pairs = ps.info(stream)
    feat = torch.empty(N_FEAT, dtype=torch.float32, device=A.V.device)
    api._check(L.rs_mlp_features(ca.data_ptr(), cb.data_ptr(), RES, feat.data_ptr(), api._stream(stream)),
               "rs_mlp_features")
    ba.close()
    bb.close()
    ps.close()
    return Sample(feat, int(pairs), est, (na, nb))


class Mlp:
    """Handle on the engine's MLP."""

    def __init__(self, seed: int = 0, prior: bool = False, weight_decay: float = 0.0):
        self.L = _lib.load()
        self.h = ctypes.c_void_p()
        api._check(self.L.rs_mlp_create(int(seed), ctypes.byref(self.h)), "rs_mlp_create")
        self.prior = bool(prior)
        api._check(self.L.rs_mlp_set_prior(self.h, int(prior), _cell_volume(), 0.001, 0.8, 1), "rs_mlp_set_prior")
        api._check(self.L.rs_mlp_set_weight_decay(self.h, float(weight_decay)), "rs_mlp_set_weight_decay")

    @property
    def n_params(self) -> int:
        return int(self.L.rs_mlp_num_params())

    def params(self, grads: bool = False):
        p = np.empty(self.n_params, np.float32)
        g = np.empty(self.n_params, np.float32) if grads else None
        api._check(self.L.rs_mlp_get_params(self.h, p.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                            g.ctypes.data_as(ctypes.POINTER(ctypes.c_float)) if grads else None),
                   "rs_mlp_get_params")
        return (p, g) if grads else p

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, np.float32)
        api._check(self.L.rs_mlp_set_params(self.h, p.ctypes.data_as(ctypes.POINTER(ctypes.c_float))),
                   "rs_mlp_set_params")

    def forward(self, X: torch.Tensor) -> torch.Tensor:
        y = torch.empty(X.shape[0], dtype=torch.float32, device=X.device)
        api._check(self.L.rs_mlp_forward(self.h, X.data_ptr(), int(X.shape[0]), y.data_ptr(), api._stream(None)),
                   "rs_mlp_forward")
        return y

    def gradients(self, X: torch.Tensor, t: torch.Tensor) -> float:
        loss = ctypes.c_float()
        api._check(self.L.rs_mlp_gradients(self.h, X.data_ptr(), t.data_ptr(), int(X.shape[0]), ctypes.byref(loss),
                                           api._stream(None)), "rs_mlp_gradients")
        return loss.value

    def step(self, X: torch.Tensor, t: torch.Tensor, lr: float) -> float:
        loss = ctypes.c_float()
        api._check(self.L.rs_mlp_train_step(self.h, X.data_ptr(), t.data_ptr(), int(X.shape[0]), float(lr),
                                            ctypes.byref(loss), api._stream(None)), "rs_mlp_train_step")
        return loss.value

    def close(self):
        if self.h:
            self.L.rs_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def symmetry(X: torch.Tensor, g: torch.Generator) -> torch.Tensor:
    """Each feature row (2 sides x 4 channels x 16^3 blocks, z-major) under a random one of
    the 96 maps that keep the exact pair count: a swap of the two sides, reflections of the
    three axes and a permutation of them."""
    B = X.shape[0]
    V = X.view(B, 2, 4, 16, 16, 16)
    out = torch.empty_like(V)
    codes = torch.randint(0, 96, (B,), generator=g).tolist()
    perms = [(3, 4, 5), (3, 5, 4), (4, 3, 5), (4, 5, 3), (5, 3, 4), (5, 4, 3)]
    for i, c in enumerate(codes):
        v = V[i:i + 1]
        if c & 1:
            v = v.flip(1)
        flips = [3 + a for a in range(3) if (c >> (1 + a)) & 1]
        if flips:
            v = v.flip(flips)
        p = perms[(c >> 4) % 6]
        out[i:i + 1] = v.permute(0, 1, 2, *p)
    return out.view(B, -1)


def targets(samples: List[Sample], prior: bool, device) -> torch.Tensor:
    """log1p(pairs), less log1p(grid estimate) when the network corrects the grid estimator."""
    t = [np.log1p(s.pairs) - (np.log1p(max(s.grid_estimate, 0)) if prior else 0.0) for s in samples]
    return torch.tensor(t, dtype=torch.float32, device=device)


def train(samples: List[Sample], epochs: int = 60, batch: int = 64, lr: float = 1e-3, seed: int = 0,
          mlp: Optional[Mlp] = None, prior: bool = True, weight_decay: float = 1e-2, val_frac: float = 0.0,
          augment: bool = True):
    """Adam (decoupled weight decay) on the MSE of the target (see targets); cosine
    learning-rate decay; symmetry augmentation.  With val_frac > 0 the last part of the
    samples is held back and the parameters of the epoch with the lowest validation loss
    are kept (early stopping).  Returns (model, losses)."""
    n_val = int(round(len(samples) * val_frac))
    fit, val = samples[:len(samples) - n_val], samples[len(samples) - n_val:]
    X = torch.stack([s.features for s in fit]).contiguous()
    m = mlp or Mlp(seed, prior=prior, weight_decay=weight_decay)
    t = targets(fit, m.prior, X.device)
    if val:
        Xv = torch.stack([s.features for s in val]).contiguous()
        tv = targets(val, m.prior, X.device)
    g = torch.Generator(device="cpu")
    g.manual_seed(seed)
    losses = []
    n = len(fit)
    steps = epochs * max(1, (n + batch - 1) // batch)
    k = 0
    best, best_p = float("inf"), None
    for ep in range(epochs):
        perm = torch.randperm(n, generator=g).to(X.device)
        tot = 0.0
        for b0 in range(0, n, batch):
            idx = perm[b0:b0 + batch]
            cur = lr * 0.5 * (1.0 + np.cos(np.pi * k / steps))
            xb = symmetry(X[idx], g) if augment else X[idx].contiguous()
            tot += m.step(xb, t[idx].contiguous(), cur) * len(idx)
            k += 1
        losses.append(tot / n)
        if val:
            vl = float(((m.forward(Xv) - tv) ** 2).mean().item())
            if vl < best:
                best, best_p = vl, m.params()
    if best_p is not None:
        m.set_params(best_p)
    return m, losses


def predict(m: Mlp, samples: List[Sample]) -> np.ndarray:
    """Estimated pair counts of the samples (the grid estimate times the network's
    correction when the model has the prior)."""
    X = torch.stack([s.features for s in samples]).contiguous()
    y = m.forward(X).cpu().numpy().astype(np.float64)
    if m.prior:
        y = y + np.log1p(np.maximum(np.array([s.grid_estimate for s in samples], np.float64), 0.0))
    return np.maximum(np.expm1(y), 0.0)


def evaluate(m: Mlp, samples: List[Sample]) -> dict:
    """Errors of the network and of the grid estimator on the same pairs: mean absolute
    log1p error, and how often each picks the pair-table size the true count would."""
    true = np.array([s.pairs for s in samples], np.float64)
    grid = np.array([s.grid_estimate for s in samples], np.float64)
    mlp = predict(m, samples)
    L = _lib.load()

    def size(v):
        return np.array([L.rs_hash_size_pow2(int(round(x))) for x in v], np.float64)

    st = size(true)
    return {
        "samples": len(samples),
        "mlp_abs_log1p_error": float(np.mean(np.abs(np.log1p(mlp) - np.log1p(true)))),
        "grid_abs_log1p_error": float(np.mean(np.abs(np.log1p(grid) - np.log1p(true)))),
        "mlp_table_size_match": float(np.mean(size(mlp) == st)),
        "grid_table_size_match": float(np.mean(size(grid) == st)),
        "mlp_abs_log2_table_ratio": float(np.mean(np.abs(np.log2(size(mlp) / st)))),
        "grid_abs_log2_table_ratio": float(np.mean(np.abs(np.log2(size(grid) / st)))),
    }


def join_seconds(seed: int, estimate: float, n_lo: int = 1000, n_hi: int = 200_000, reps: int = 3) -> float:
    """Device seconds of the exact join of dataset pair `seed` with its pair table sized from
    `estimate` as raytracer_overlap_estimated sizes it (rs_hash_size_pow2): creating and
    clearing the table, the join (which regrows the table from its overflow table when it
    fills, and reruns only when that fills too) and the sorted pair list; the BVHs are built beforehand.  Mean of reps after one warm-up."""
    A, _, B, _ = dataset_pair(seed, n_lo, n_hi)
    ba, bb = api.Bvh(A), api.Bvh(B)
    size = api.hash_size_pow2(int(round(estimate)))
    times = []
    for _ in range(reps + 1):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        ps = api.PairSet(size, pow2=True)
        api.overlap_join(ba, bb, ps)
        ps.finalize()
        e1.record()
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1) / 1e3)
        ps.close()
    ba.close()
    bb.close()
    return float(np.mean(times[1:]))
