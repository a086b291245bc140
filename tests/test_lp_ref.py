"""The CPU reference of the learned p' network: its analytic gradient against
central differences (FP64, no BF16 rounding), on a 4x4x4 grid."""
import numpy as np

from oracle import lp_ref


def test_reference_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    p = lp_ref.init_params(5).astype(np.float64)
    x = np.zeros((4, 4, 4, 16))
    x[..., 0] = rng.normal(size=(4, 4, 4))
    x[..., 1] = (rng.uniform(size=(4, 4, 4)) > 0.2).astype(float)
    t = rng.normal(size=(4, 4, 4))
    loss, g, _ = lp_ref.loss_and_grads(p, x, t, bf16=False)
    assert np.isfinite(loss) and g.shape == (lp_ref.num_params(),)
    # one weight of every layer's live part, and every bias block
    idx, off = [], 0
    for l, (ci, co) in enumerate(lp_ref.LAYERS):
        nw = 27 * ci * co
        idx += [off + 13 * ci * co + 0 * ci + 0, off + nw + 0]   # centre tap (co 0, ci 0), bias 0
        off += nw + co
    eps = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += eps
        pm[i] -= eps
        fd = (lp_ref.loss_and_grads(pp, x, t, bf16=False)[0] - lp_ref.loss_and_grads(pm, x, t, bf16=False)[0]) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-5 * max(1.0, abs(fd)), (i, fd, g[i])


def test_bf16_rounding_is_round_to_nearest_even():
    vals = np.array([1.0, 1.00390625, 1.005859375, -2.5, 3.0e-3], dtype=np.float32)
    r = lp_ref.to_bf16(vals)
    # bf16 keeps 8 significant bits
    assert r[0] == 1.0
    assert r[1] == 1.0            # 1 + 2^-8: tie -> even (1.0)
    assert r[2] == 1.0078125      # above the tie -> up
    assert r[3] == -2.5
    assert abs(r[4] - 3.0e-3) / 3.0e-3 < 2 ** -8
