"""Path-guiding network on the GPU against its FP64 oracle.

Forward pass and gradients are compared with the oracle evaluated on the
GPU's own encoded inputs and the same BF16-rounded weights; the product sums
in FP32 (tensor cores) where the oracle sums in FP64, and it feeds deltas to
the tensor cores as BF16 high + low parts, so the comparisons carry the
tolerances written below.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

CENTER = (1.0, -2.0, 0.5)
HALF = 40.0


def _unit(v):
    return (v / np.linalg.norm(v, axis=1, keepdims=True)).astype(np.float32)


def _batch(n, seed):
    rng = np.random.default_rng(seed)
    pos = (np.array(CENTER) + rng.uniform(-HALF, HALF, (n, 3))).astype(np.float32)
    nrm = _unit(rng.normal(size=(n, 3)))
    sdir = _unit(rng.normal(size=(n, 3)))
    w = rng.lognormal(0.0, 1.0, n).astype(np.float32)
    return pos, nrm, sdir, w


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _guide(native, ctx, seed=1, kernel=0):
    return native.Guide(ctx, seed=seed, center=CENTER, half_extent=HALF, infer_kernel=kernel)


def _random_params(oracle, seed, scale=1.0):
    rng = np.random.default_rng(seed)
    n = oracle.mlp_num_params()
    p = np.zeros(n, np.float32)
    off = 0
    for fi, fo in [(80, 64), (64, 64), (64, 64), (64, 64), (64, 48)]:
        b = np.sqrt(6.0 / fi) * scale
        p[off:off + fi * fo] = rng.uniform(-b, b, fi * fo)
        off += fi * fo
        p[off:off + fo] = rng.normal(0, 0.1, fo)
        off += fo
    return p


def test_encoding_matches_oracle(native, ctx, oracle):
    g = _guide(native, ctx)
    pos, nrm, _, _ = _batch(1000, 0)
    out = torch.zeros((1000, 80), dtype=torch.float32, device="cuda")
    g.encode(_dev(pos), _dev(nrm), 1000, out)
    torch.cuda.synchronize()
    want = oracle.guide_encode(pos, nrm, CENTER, HALF)
    # FP32 versus FP64 normalisation of the position, amplified by 2^11 pi at the top frequency
    assert np.abs(out.cpu().numpy() - want).max() < 1e-3


@pytest.mark.parametrize("n", [1, 17, 1000, 4099])
def test_forward_matches_oracle(native, ctx, oracle, n):
    g = _guide(native, ctx)
    p = _random_params(oracle, n)
    g.set_params(p)
    pos, nrm, _, _ = _batch(n, n)
    d_pos, d_nrm = _dev(pos), _dev(nrm)
    enc = torch.zeros((n, 80), dtype=torch.float32, device="cuda")
    g.encode(d_pos, d_nrm, n, enc)
    y = torch.full((n, 40), float("nan"), dtype=torch.float32, device="cuda")
    g.infer(d_pos, d_nrm, n, y)
    torch.cuda.synchronize()
    got = y.cpu().numpy()
    want = oracle.mlp_forward(p, enc.cpu().numpy())[:, :40]
    scale = np.abs(want).max() + 1e-3
    err = np.abs(got - want)
    # FP32 sums vs FP64 sums; a sum landing next to a BF16 rounding boundary of
    # an activation can round the other way
    assert err.max() <= 2e-2 * scale and np.median(err) <= 1e-3 * scale, (err.max(), scale)


@pytest.mark.parametrize("kernel,n", [(0, 777), (1, 777), (0, 1), (0, 128), (0, 129)])
def test_gradients_match_oracle(native, ctx, oracle, kernel, n):
    """kernel 0: tcgen05 training (k_guide_train_tc), 1: mma.sync (k_guide_train_fb)."""
    g = _guide(native, ctx, kernel=kernel)
    p = _random_params(oracle, 7, scale=0.7)
    g.set_params(p)
    pos, nrm, sdir, w = _batch(n, 9)
    d_pos, d_nrm, d_sdir, d_w = _dev(pos), _dev(nrm), _dev(sdir), _dev(w)
    enc = torch.zeros((n, 80), dtype=torch.float32, device="cuda")
    g.encode(d_pos, d_nrm, n, enc)
    loss, grad = g.gradients(d_pos, d_nrm, d_sdir, d_w, n)
    want_loss, want = oracle.mlp_loss_grad(p, enc.cpu().numpy(), sdir, w)
    assert abs(loss - want_loss) <= 1e-3 * abs(want_loss)
    ctx.check()
    off = 0
    for fi, fo in [(80, 64), (64, 64), (64, 64), (64, 64), (64, 48)]:
        for part in (fi * fo, fo):
            a, b = grad[off:off + part].astype(np.float64), want[off:off + part]
            off += part
            rel = np.linalg.norm(a - b) / (np.linalg.norm(b) + 1e-30)
            cos = a @ b / (np.linalg.norm(a) * np.linalg.norm(b) + 1e-30)
            assert rel <= 2e-2 and cos >= 0.9995, (off, rel, cos)


def test_adam_step_matches_oracle(native, ctx, oracle):
    g = _guide(native, ctx)
    p0 = _random_params(oracle, 3)
    g.set_params(p0)
    n = 512
    pos, nrm, sdir, w = _batch(n, 5)
    args = (_dev(pos), _dev(nrm), _dev(sdir), _dev(w))
    _, grad = g.gradients(*args, n)
    g.train_step(*args, n)
    p1 = g.params()
    want, _, _ = oracle.adam_step(p0, np.zeros_like(p0), np.zeros_like(p0), grad, t=1)
    assert np.allclose(p1, want, rtol=1e-5, atol=1e-7)


def test_mixture_sampling_and_density(native, ctx, oracle):
    rng = np.random.default_rng(11)
    y = rng.normal(size=40).astype(np.float32)
    y[1::5] = rng.uniform(-2, 4, 8)
    n = 1 << 20
    u = rng.random((n, 3)).astype(np.float32)
    d_y = _dev(np.tile(y, (n, 1)))
    dirs = torch.zeros((n, 3), dtype=torch.float32, device="cuda")
    pdf = torch.zeros(n, dtype=torch.float32, device="cuda")
    L = native.load()
    native.check(L.dr_guide_mixture_sample(d_y.data_ptr(), _dev(u).data_ptr(), n, dirs.data_ptr(), pdf.data_ptr(), None))
    pdf2 = torch.zeros(n, dtype=torch.float32, device="cuda")
    native.check(L.dr_guide_mixture_pdf(d_y.data_ptr(), 0, dirs.data_ptr(), n, pdf2.data_ptr(), None))
    torch.cuda.synchronize()
    dd, pp = dirs.cpu().numpy(), pdf.cpu().numpy()
    assert np.allclose(np.linalg.norm(dd, axis=1), 1.0, atol=1e-5)
    assert np.allclose(pp, pdf2.cpu().numpy(), rtol=1e-6)
    for k in range(0, n, n // 16):
        assert abs(np.log(pp[k]) - oracle.vmf_mixture_log_pdf(y, dd[k])) < 2e-4
    # the samples follow the density: E_q[d] from samples against the density
    # integrated with uniform directions
    v = rng.normal(size=(n, 3))
    ud = (v / np.linalg.norm(v, axis=1, keepdims=True)).astype(np.float32)
    qu = torch.zeros(n, dtype=torch.float32, device="cuda")
    native.check(L.dr_guide_mixture_pdf(d_y.data_ptr(), 0, _dev(ud).data_ptr(), n, qu.data_ptr(), None))
    torch.cuda.synchronize()
    q = qu.cpu().numpy().astype(np.float64)
    assert abs(q.mean() * 4 * np.pi - 1.0) < 0.01
    mean_mc = (ud * q[:, None]).mean(0) * 4 * np.pi
    assert np.abs(dd.mean(0) - mean_mc).max() < 0.01


def test_training_fits_a_direction_field(native, ctx):
    """Targets drawn around mu(x) = direction of x from the centre: the loss
    falls well below the initial value within a few hundred steps."""
    g = _guide(native, ctx, seed=3)
    rng = np.random.default_rng(0)
    n = 4096
    losses = []
    for step in range(300):
        pos = (np.array(CENTER) + rng.uniform(-HALF, HALF, (n, 3))).astype(np.float32)
        mu = _unit(pos - np.array(CENTER, np.float32))
        sdir = _unit(mu + rng.normal(0, 0.15, (n, 3)))
        nrm = _unit(rng.normal(size=(n, 3)))
        w = np.ones(n, np.float32)
        g.train_step(_dev(pos), _dev(nrm), _dev(sdir), _dev(w), n)
        if step % 50 == 0 or step == 299:
            losses.append(g.last_loss())
    assert losses[-1] < losses[0] - 1.5, losses


def test_state_checkpoint_resumes_training(native, ctx):
    """A network restored from a checkpoint (dr_guide_get_state / _set_state,
    into a network created with another seed and centre) trains on exactly as
    the saved one: same parameters after the same further Adam steps, up to
    the order of the gradient sums' atomics. Restarting from the parameters
    alone (dr_guide_set_params resets Adam) lands elsewhere.

    The atomics' order changes a gradient sum in its last bits. Adam divides
    by the root of the second moment, so a parameter whose gradient is near
    zero can take a visibly different step from that alone (up to the
    learning rate per step); the comparison therefore bounds the RMS of the
    difference and lets a few parameters move by a few percent of the
    largest step."""
    batches = [tuple(_dev(a) for a in _batch(4096, 50 + k)) for k in range(8)]
    g1 = _guide(native, ctx, seed=3)
    for b in batches[:4]:
        g1.train_step(*b, 4096)
    state = g1.get_state()
    params_at_save = g1.params()
    for b in batches[4:]:
        g1.train_step(*b, 4096)
    want = g1.params()
    g2 = native.Guide(ctx, seed=99, center=(0.0, 0.0, 0.0), half_extent=1.0)
    g2.set_state(state)
    assert np.array_equal(g2.get_state(), state)
    for b in batches[4:]:
        g2.train_step(*b, 4096)
    got = g2.params()
    g3 = _guide(native, ctx, seed=5)
    g3.set_params(params_at_save)
    for b in batches[4:]:
        g3.train_step(*b, 4096)
    moved = np.abs(want - params_at_save).max()
    rms = lambda a: float(np.sqrt(np.mean(np.square(a, dtype=np.float64))))
    assert moved > 1e-5
    assert rms(got - want) < 1e-3 * rms(want - params_at_save), (rms(got - want), rms(want - params_at_save))
    assert np.abs(got - want).max() < 0.05 * moved, (np.abs(got - want).max(), moved)
    assert rms(g3.params() - want) > 0.1 * rms(want - params_at_save)
    bad = state.copy()
    bad[0] ^= 0xff
    with pytest.raises(Exception):
        g2.set_state(bad)
    for g in (g1, g2, g3):
        g.close()
