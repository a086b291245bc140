"""The learned p' initial guess on the GPU: forward pass and gradients against
the CPU reference (oracle/lp_ref.py, BF16 storage emulated, FP64 sums),
training on samples from the solver, and the guess inside the iteration."""
import numpy as np
import pytest

from gfm_gb300 import Case, GpuSolver, abi, configs
from oracle import lp_ref

pytestmark = pytest.mark.gpu


def _sample(rng, dims, torch):
    nx, ny, nz = dims
    x = np.zeros((nz, ny, nx, 16), np.float32)
    x[..., 0] = rng.normal(size=(nz, ny, nx))
    x[..., 1] = (rng.uniform(size=(nz, ny, nx)) > 0.15).astype(np.float32)
    x[..., 0] *= x[..., 1]
    t = (rng.normal(size=(nz, ny, nx)) * x[..., 1]).astype(np.float32)
    xb = torch.from_numpy(x.reshape(-1, 16)).to(torch.bfloat16).cuda()
    tb = torch.from_numpy(t.reshape(-1)).cuda()
    return x, t, xb, tb


@pytest.fixture(scope="module")
def torch():
    return pytest.importorskip("torch")


def test_forward_matches_cpu_reference(torch):
    from gfm_gb300.lp import LearnedPressure
    dims = (8, 6, 4)
    rng = np.random.default_rng(11)
    p = lp_ref.init_params(2)
    lp = LearnedPressure(dims, seed=1)
    lp.set_params(p)
    x, t, xb, tb = _sample(rng, dims, torch)
    got = lp.forward(xb, dims).cpu().numpy().reshape(dims[2], dims[1], dims[0])
    want = lp_ref.forward(p, x)["out"][..., 0]
    err = np.linalg.norm(got - want) / np.linalg.norm(want)
    assert err < 1e-2, err
    lp.close()


@pytest.mark.parametrize("dims", [(8, 16, 2), (24, 20, 6)])
def test_tcgen05_forward_matches_mma_sync_and_reference(torch, dims):
    """The forward pass with its convolutions on tcgen05 (tensor memory
    accumulators) agrees with the mma.sync path and the CPU reference."""
    from gfm_gb300.lp import LearnedPressure
    rng = np.random.default_rng(9)
    p = lp_ref.init_params(6)
    lp = LearnedPressure(dims, seed=1)
    lp.set_params(p)
    x, t, xb, tb = _sample(rng, dims, torch)
    lp.set_tensor_path(False)
    a = lp.forward(xb, dims).cpu().numpy()
    lp.set_tensor_path(True)
    b = lp.forward(xb, dims).cpu().numpy()
    assert lp.tensor_status() == 0
    want = lp_ref.forward(p, x)["out"][..., 0].reshape(-1)
    assert np.linalg.norm(b - a) / np.linalg.norm(a) < 1e-2
    assert np.linalg.norm(b - want) / np.linalg.norm(want) < 1e-2
    lp.close()


def test_tcgen05_wait_expiry_is_reported_and_the_pass_completes(torch, monkeypatch):
    """The bounded wait of a tcgen05 tile for its MMAs: with the first wait cut
    to no poll at all (GFM_LP_WAIT1=0, read at creation) it runs out, the
    status says so (1), the tile waits again with the normal limit, and the
    output is the same as without the cut; the launch completes and frees its
    tensor memory (later launches still run)."""
    from gfm_gb300.lp import LearnedPressure
    dims = (24, 20, 6)
    rng = np.random.default_rng(4)
    p = lp_ref.init_params(6)
    x, t, xb, tb = _sample(rng, dims, torch)
    ref = LearnedPressure(dims, seed=1)
    ref.set_params(p)
    want = ref.forward(xb, dims).cpu().numpy()
    assert ref.tensor_status() == 0
    ref.close()
    monkeypatch.setenv("GFM_LP_WAIT1", "0")
    lp = LearnedPressure(dims, seed=1)
    lp.set_params(p)
    got = lp.forward(xb, dims).cpu().numpy()
    assert lp.tensor_status() == 1
    assert np.array_equal(got, want)
    again = lp.forward(xb, dims).cpu().numpy()
    assert np.array_equal(again, want)
    lp.close()


def test_gradients_match_cpu_reference(torch):
    from gfm_gb300.lp import LearnedPressure
    dims = (8, 8, 4)
    rng = np.random.default_rng(5)
    p = lp_ref.init_params(4)
    lp = LearnedPressure(dims, seed=1)
    lp.set_params(p)
    x, t, xb, tb = _sample(rng, dims, torch)
    loss = lp.train_step(xb, tb, dims, update=False)
    g = lp.grads()
    loss_ref, g_ref, _ = lp_ref.loss_and_grads(p, x, t)
    assert abs(loss - loss_ref) <= 1e-2 * loss_ref, (loss, loss_ref)
    off = 0
    for l, (ci, co) in enumerate(lp_ref.LAYERS):
        n = 27 * ci * co + co
        a, b = g[off:off + n], g_ref[off:off + n]
        err = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)
        assert err < 3e-2, (l, err)
        off += n
    lp.close()


def test_training_reduces_error_of_the_p_prime_guess(torch):
    """Trained on p' systems of the 48x24x16 furnace, the guess is closer to the
    converged p' of later, unseen iterations than the zero start is."""
    from gfm_gb300.lp import LearnedPressure, collect_samples
    cfg = configs.small_furnace()
    train = collect_samples([cfg], iters=60, every=3, nsweeps=60, start=3)
    test = collect_samples([cfg], iters=80, every=5, nsweeps=60, start=65)
    dims = train[0][2]
    lp = LearnedPressure(dims, seed=3)

    def rel_err():
        # error of the best multiple of the guess: the solver fixes the scale itself
        e = []
        for f, t, d in test:
            out = lp.forward(f, d).double()
            tt = t.double()
            a = float(torch.dot(out, tt) / max(float(torch.dot(out, out)), 1e-300))
            e.append(float(torch.linalg.norm(a * out - tt) / torch.linalg.norm(tt)))
        return float(np.mean(e))

    before = rel_err()
    hist = lp.fit(train, steps=400, lr=2e-3)
    after = rel_err()
    assert np.isfinite(hist).all()
    assert np.mean(hist[-40:]) < np.mean(hist[:40])
    assert after < 0.8, (before, after)   # the zero start has relative error 1
    lp.close()


def test_training_is_deterministic(torch):
    """Gradients are summed in a fixed order, so two trainings on the same
    samples give the same parameters bit for bit."""
    from gfm_gb300.lp import LearnedPressure, collect_samples
    train = collect_samples([configs.small_furnace()], iters=12, every=3, nsweeps=20, start=3)
    ps = []
    for _ in range(2):
        lp = LearnedPressure(train[0][2], seed=5)
        lp.fit(train, steps=30, lr=2e-3, seed=1)
        ps.append(lp.params())
        lp.close()
    assert np.array_equal(ps[0], ps[1])


def test_trained_guess_lowers_the_p_prime_residual_of_the_same_iteration(torch):
    """From the same state, the p' solve that starts from the trained guess ends
    with a lower residual than the one that starts from zero (same sweeps)."""
    from gfm_gb300.lp import LearnedPressure, collect_samples
    cfg = configs.small_furnace()
    train = collect_samples([cfg], iters=60, every=3, nsweeps=60, start=3)
    lp = LearnedPressure(train[0][2], seed=3)
    lp.fit(train, steps=400, lr=2e-3)
    case = Case(cfg)
    s = GpuSolver(case, adi_mode=abi.GFM_ADI_REDBLACK, precision=abi.GFM_PREC_MIXED)
    s.start()
    s.gflow(64)
    state = s.download()
    plain, _ = s.gflow(1)
    s.upload(state)
    s.set_lp(lp)
    learned, _ = s.gflow(1)
    assert learned["lp_used"] == 1 and learned["lp_ratio"] < 1.0
    assert learned["pcorr_resid"] < plain["pcorr_resid"], (learned["pcorr_resid"], plain["pcorr_resid"])
    s.close()
    lp.close()


def test_solver_uses_the_guess_with_fallback(torch):
    from gfm_gb300.lp import LearnedPressure
    case = Case(configs.small_furnace())
    s = GpuSolver(case, adi_mode=abi.GFM_ADI_REDBLACK, precision=abi.GFM_PREC_MIXED)
    s.start()
    dims = (case.mp // 2 - 2, case.np // 2 - 2, case.lp // 2 - 2)
    lp = LearnedPressure(dims, seed=1)      # untrained: its guess is usually rejected
    s.set_lp(lp)
    st, nd = s.gflow(3)
    assert nd == 3 and np.isfinite(st["res_mass"])
    assert st["lp_used"] in (0, 1) and np.isfinite(st["lp_ratio"])
    if st["lp_ratio"] >= 1.0:
        assert st["lp_used"] == 0
    s.set_lp(None)
    st2, _ = s.gflow(1)
    assert st2["lp_used"] == 0
    s.close()
    lp.close()
