"""Learned estimator (rs_mlp_*): pooled features, the tensor-core forward pass and gradients
against the float64 CPU restatement (oracle/mlp.py), training, and the gain over the
grid estimator."""
import ctypes

import numpy as np
import pytest
import torch

from oracle import mlp as omlp
from rayspace3d_gb300 import _lib, api, formats, learned, synth

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("R", [16, 40, 128])
def test_features_match_oracle(cuda, R):
    rng = np.random.default_rng(R)
    n = R ** 3
    cells = np.zeros(n, formats.GRID_CELL_DTYPE)
    live = rng.random(n) < 0.05
    cells["CenterCount"][live] = rng.integers(0, 5, live.sum())
    cells["TouchCount"][live] = rng.integers(1, 30, live.sum())
    cells["AvgSizeMean"][live] = rng.uniform(0.1, 50, live.sum()).astype(np.float32)
    cells["VolRatio"][live] = rng.uniform(0, 1, live.sum()).astype(np.float32)
    other = np.roll(cells, 7)
    da = torch.from_numpy(cells.view(np.uint8).copy()).cuda()
    db = torch.from_numpy(other.view(np.uint8).copy()).cuda()
    out = torch.empty(32768, dtype=torch.float32, device="cuda")
    assert _lib.load().rs_mlp_features(da.data_ptr(), db.data_ptr(), R, out.data_ptr(), None) == 0
    torch.cuda.synchronize()
    want = np.concatenate([omlp.pool(cells, R), omlp.pool(other, R)])
    np.testing.assert_allclose(out.cpu().numpy(), want, rtol=1e-6, atol=1e-7)


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def test_forward_and_gradients_match_oracle(cuda):
    """Tensor-core forward pass and every gradient block against the float64 restatement
    with the same BF16 rounding points.  Tolerance: relative Frobenius error <= 1e-3 for the
    outputs and <= 5e-3 per gradient block (FP32 accumulation in a different order, and
    BF16 re-rounding of hidden activations that land near a rounding boundary)."""
    m = learned.Mlp(seed=11)
    rng = np.random.default_rng(12)
    B = 24
    X = rng.uniform(0.0, 4.0, size=(B, 32768)).astype(np.float32)
    X[:, rng.random(32768) < 0.7] = 0.0  # sparse like pooled grids
    t = rng.uniform(0.0, 8.0, size=B).astype(np.float32)
    dX, dt = torch.from_numpy(X).cuda(), torch.from_numpy(t).cuda()
    p = m.params()
    y = m.forward(dX).cpu().numpy()
    want_y, _ = omlp.forward(p, X)
    assert _rel(y, want_y) < 1e-3
    loss = m.gradients(dX, dt)
    _, g = m.params(grads=True)
    want_loss, want_g = omlp.gradients(p, X, t.astype(np.float64))
    assert abs(loss - want_loss) <= 1e-3 * max(1.0, want_loss)
    blocks = {"W1": (omlp.O_W1, omlp.O_B1), "b1": (omlp.O_B1, omlp.O_W2), "W2": (omlp.O_W2, omlp.O_B2),
              "b2": (omlp.O_B2, omlp.O_W3), "W3": (omlp.O_W3, omlp.O_B3), "b3": (omlp.O_B3, omlp.N_PARAMS)}
    for name, (a, b) in blocks.items():
        err = _rel(g[a:b].astype(np.float64), want_g[a:b])
        assert err < 5e-3, f"{name}: relative error {err}"
    m.close()


def test_training_fits_and_estimate_entry_point(cuda):
    """A short training run of the plain network (no prior, no weight decay, no
    augmentation) on engine-labelled dataset pairs: the loss falls by 10x, and
    rs_estimate_mlp agrees with the forward pass."""
    samples = [learned.make_sample(500 + i, 500, 4000) for i in range(40)]
    assert all(s.pairs >= 0 for s in samples)
    m, losses = learned.train(samples, epochs=120, batch=16, lr=1e-3, seed=1, prior=False, weight_decay=0.0,
                              augment=False)
    assert losses[-1] < 0.1 * losses[0]
    L = _lib.load()
    s = samples[0]
    y = m.forward(s.features[None].contiguous()).item()
    est, lg = ctypes.c_int64(), ctypes.c_double()
    rng = np.random.default_rng(500)
    A, na = learned.dataset_side(4 * 500, 500, 4000, rng)
    B, nb = learned.dataset_side(4 * 500 + 3, 500, 4000, rng)
    ca, cb = learned.grid_cells(A, na), learned.grid_cells(B, nb)
    assert L.rs_estimate_mlp(m.h, ca.data_ptr(), cb.data_ptr(), learned.RES, ctypes.byref(est), ctypes.byref(lg),
                             None) == 0
    assert abs(lg.value - y) < 1e-4 * max(1.0, abs(y))
    assert est.value == max(0, int(round(np.expm1(lg.value))))
    m.close()


def test_held_out_gain_over_grid_estimator(cuda):
    """What the network gains on dataset pairs it never saw: trained (grid-estimate prior,
    weight decay, symmetry augmentation, early stopping on a validation split) on 160
    engine-labelled pairs, its mean |log1p error| on 40 held-out pairs is below the grid
    estimator's, and rs_estimate_mlp with the prior returns the grid estimate corrected by
    the network."""
    samples = [learned.make_sample(7000 + i, 500, 4000) for i in range(200)]
    train, test = samples[:160], samples[160:]
    m, _ = learned.train(train, epochs=60, batch=32, lr=1e-3, seed=2, prior=True, weight_decay=1e-2,
                         val_frac=0.15)
    ev = learned.evaluate(m, test)
    assert ev["mlp_abs_log1p_error"] < ev["grid_abs_log1p_error"], ev
    L = _lib.load()
    seed = 7000 + 160
    A, na, B, nb = learned.dataset_pair(seed, 500, 4000)
    ca, cb = learned.grid_cells(A, na), learned.grid_cells(B, nb)
    est, lg = ctypes.c_int64(), ctypes.c_double()
    assert L.rs_estimate_mlp(m.h, ca.data_ptr(), cb.data_ptr(), learned.RES, ctypes.byref(est), ctypes.byref(lg),
                             None) == 0
    want = learned.predict(m, [test[0]])[0]
    assert abs(lg.value - np.log1p(want)) < 1e-4 * max(1.0, abs(lg.value))
    m.close()
