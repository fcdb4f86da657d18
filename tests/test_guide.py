"""The learned vMF-mixture proposal: GPU (BF16 tensor cores, FP32 accumulation)
against the FP64 numpy restatement (oracle/guide_ref.py) and the reference's
own VonMisesFisherDistribution (oracle/_ref).

Tolerances: forward outputs within 2e-2 of the FP64 model evaluated on the same
BF16-rounded operands (the GPU accumulates in FP32, in a different order, and
rounds hidden activations to BF16); gradients within 5e-2 relative L2 of the
quantisation-matched FP64 backward and cosine > 0.99 against the unquantised one.
"""
import numpy as np
import pytest

from oracle import guide_ref as G

LO, HI = np.array([-1.0, -1.0, -1.0]), np.array([1.0, 1.0, 1.0])


def points(n, seed):
    rng = np.random.default_rng(seed)
    pos = rng.uniform(-1, 1, (n, 3))
    nrm = rng.normal(size=(n, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    wo = rng.normal(size=(n, 3))
    wo /= np.linalg.norm(wo, axis=1, keepdims=True)
    return pos.astype(np.float32), nrm.astype(np.float32), wo.astype(np.float32)


def test_numpy_gradient_matches_finite_differences():
    """The FP64 oracle's analytic backward against central differences."""
    rng = np.random.default_rng(0)
    params = rng.normal(scale=0.2, size=G.N_PARAMS)
    pos, nrm, wo = points(16, 1)
    X = G.features(pos, nrm, wo, LO, HI)
    wdir = rng.normal(size=(16, 3))
    wdir /= np.linalg.norm(wdir, axis=1, keepdims=True)
    weight = rng.uniform(0.1, 2.0, 16)

    def loss(p):
        Y, _ = G.forward(p, X, quant=False)
        return G.loss_and_output_grad(Y, wdir, weight)[0]

    Y, acts = G.forward(params, X, quant=False)
    _, dY = G.loss_and_output_grad(Y, wdir, weight)
    g = G.backward(params, acts, dY, quant=False)
    for idx in rng.choice(G.N_PARAMS, 40, replace=False):
        e = np.zeros(G.N_PARAMS)
        e[idx] = 1e-6
        fd = (loss(params + e) - loss(params - e)) / 2e-6
        assert abs(fd - g[idx]) <= 1e-5 + 1e-4 * abs(fd)


@pytest.fixture(scope="module")
def guide():
    import __graft_entry__ as g
    g.build()
    from xitils_gb300 import api
    ctx = api.Context(0)
    gd = api.Guide(ctx, seed=3)
    gd.set_bounds(LO, HI)
    rng = np.random.default_rng(5)
    p = gd.params().astype(np.float64)
    p += rng.normal(scale=0.05, size=p.size)  # move off the initial symmetric output layer
    gd.set_params(p.astype(np.float32))
    return ctx, gd


@pytest.mark.gpu
def test_forward_matches_fp64(guide):
    ctx, gd = guide
    pos, nrm, wo = points(3000, 2)
    Y = gd.infer(pos, nrm, wo)
    Yref, _ = G.forward(gd.params().astype(np.float64), G.features(pos, nrm, wo, LO, HI), quant=True)
    err = np.abs(Y - Yref).max() / (np.abs(Yref).max() + 1e-6)
    assert err < 2e-2, err


@pytest.mark.gpu
def test_gradients_match_fp64(guide):
    ctx, gd = guide
    rng = np.random.default_rng(7)
    n = 4096
    pos, nrm, wo = points(n, 3)
    wi = rng.normal(size=(n, 3))
    wi = (wi / np.linalg.norm(wi, axis=1, keepdims=True)).astype(np.float32)
    pdf = rng.uniform(0.05, 1.0, n).astype(np.float32)
    rad = rng.uniform(0.0, 3.0, n).astype(np.float32)
    params = gd.params().astype(np.float64)
    loss_gpu = gd.train_batch(pos, nrm, wo, wi, pdf, rad, lr=0.0)
    g_gpu = gd.grads().astype(np.float64)
    X = G.features(pos, nrm, wo, LO, HI)
    w = rad.astype(np.float64) / pdf
    Yq, acts_q = G.forward(params, X, quant=True)
    loss_q, dYq = G.loss_and_output_grad(Yq, wi, w)
    g_q = G.backward(params, acts_q, dYq, quant=True)
    Y, acts = G.forward(params, X, quant=False)
    _, dY = G.loss_and_output_grad(Y, wi, w)
    g_exact = G.backward(params, acts, dY, quant=False)
    rel = np.linalg.norm(g_gpu - g_q) / np.linalg.norm(g_q)
    cos = g_gpu @ g_exact / (np.linalg.norm(g_gpu) * np.linalg.norm(g_exact))
    assert abs(loss_gpu - loss_q) <= 2e-2 * abs(loss_q) + 1e-3
    assert rel < 5e-2, rel
    assert cos > 0.99, cos
    assert np.array_equal(gd.params().astype(np.float64), params)  # lr = 0 leaves parameters untouched


@pytest.mark.gpu
def test_sampling_matches_reference_vmf(guide):
    """Mixture pdf of the GPU against the reference's own VonMisesFisherDistribution<8>::eval,
    and the sampled directions distributed by that pdf."""
    from oracle.bindings import CpuChecker
    import ctypes as C
    ctx, gd = guide
    n = 512
    pos, nrm, wo = points(n, 9)
    dirs, pdf = gd.sample(pos, nrm, wo, seed=11)
    assert np.allclose(np.linalg.norm(dirs, axis=1), 1.0, atol=1e-4)
    Y = gd.infer(pos, nrm, wo)
    np.testing.assert_allclose(pdf, G.mixture_pdf(Y, dirs), rtol=2e-3, atol=1e-6)
    try:
        ref = CpuChecker("reference")
    except Exception:
        pytest.skip("reference checker not staged")
    mu, kappa, alpha = G.decode(Y)
    f = ref.lib.xref_vmf8_eval
    for r in range(0, n, 64):
        enc = np.zeros(40, np.float32)
        for j in range(8):
            enc[5 * j:5 * j + 3] = mu[r, j]
            enc[5 * j + 3] = kappa[r, j]
            if j < 7:
                enc[5 * j + 4] = alpha[r, j]
        d = dirs[r:r + 1].astype(np.float32)
        out = np.zeros(1, np.float32)
        f(enc.ctypes.data_as(C.POINTER(C.c_float)), C.c_int(1), d.ctypes.data_as(C.POINTER(C.c_float)),
          out.ctypes.data_as(C.POINTER(C.c_float)))
        assert abs(out[0] - pdf[r]) <= 2e-3 * out[0] + 1e-6


@pytest.mark.gpu
def test_sample_histogram_follows_pdf(guide):
    ctx, gd = guide
    n = 60000
    pos = np.tile(np.array([[0.2, -0.3, 0.5]], np.float32), (n, 1))
    nrm = np.tile(np.array([[0, 1, 0]], np.float32), (n, 1))
    wo = np.tile(np.array([[0.6, 0.8, 0.0]], np.float32), (n, 1))
    dirs, pdf = gd.sample(pos[:n // 2], nrm[:n // 2], wo[:n // 2], seed=1)
    dirs2, _ = gd.sample(pos[n // 2:], nrm[n // 2:], wo[n // 2:], seed=2)
    dirs = np.concatenate([dirs, dirs2]).astype(np.float64)
    Y = gd.infer(pos[:1], nrm[:1], wo[:1])
    # expected counts in 8 octant bins by Monte Carlo integration of the pdf
    rng = np.random.default_rng(0)
    u = rng.normal(size=(400000, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    mu, kappa, alpha = G.decode(Y)
    p = np.sum(alpha[0] * G.vmf_pdf(mu[0], kappa[0], u[:, None, :]), axis=1)
    octant = lambda v: (v[:, 0] > 0).astype(int) * 4 + (v[:, 1] > 0) * 2 + (v[:, 2] > 0)
    expected = np.bincount(octant(u), weights=p * 4 * np.pi / u.shape[0], minlength=8) * n
    observed = np.bincount(octant(dirs), minlength=8)
    mask = expected > 50
    chi2 = np.sum((observed[mask] - expected[mask]) ** 2 / expected[mask])
    assert chi2 < 40, (observed, expected)


@pytest.mark.gpu
def test_training_concentrates_on_the_target(guide):
    """Adam on samples from one vMF lobe (mu = +y, kappa = 20, uniform proposal
    pdf): the negative log-likelihood falls from the near-uniform start."""
    from xitils_gb300 import api
    ctx, _ = guide
    gd = api.Guide(ctx, seed=1)
    gd.set_bounds(LO, HI)
    rng = np.random.default_rng(4)
    n = 8192
    kappa = 20.0
    losses = []
    for step in range(300):
        pos, nrm, wo = points(n, 100 + step)
        u = rng.uniform(size=n)
        w = 1.0 + np.log(u + (1 - u) * np.exp(-2 * kappa)) / kappa
        phi = rng.uniform(0, 2 * np.pi, n)
        s = np.sqrt(np.maximum(0, 1 - w * w))
        wi = np.stack([s * np.cos(phi), w, s * np.sin(phi)], axis=1).astype(np.float32)
        losses.append(gd.train_batch(pos, nrm, wo, wi, np.full(n, 1 / (4 * np.pi), np.float32),
                                     np.ones(n, np.float32), lr=3e-3))
    assert np.isfinite(losses).all()
    assert np.mean(losses[-20:]) < losses[0] - 1.5, (losses[0], np.mean(losses[-20:]))


def _fixture_mixture():
    import os
    f = np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_aov_vmf.npz"))
    enc = f["vmf_encoded"].astype(np.float64)
    mu = np.stack([enc[5 * j:5 * j + 3] for j in range(8)])
    kappa = np.array([enc[5 * j + 3] for j in range(8)])
    alpha = np.array([enc[5 * j + 4] for j in range(7)] + [0.0])
    alpha[7] = 1.0 - alpha[:7].sum()
    return f, mu, kappa, alpha


def _mixture_pdf(mu, kappa, alpha, w):
    w = np.asarray(w, np.float64).reshape(-1, 1, 3)
    k = np.where(kappa > 0, kappa, 1.0)
    v = np.where(kappa > 0, G.vmf_pdf(mu, k, w), 1.0 / (4 * np.pi))
    return np.sum(alpha * v, axis=1)


def test_numpy_vmf_matches_reference_fit_fixture():
    """The FP64 restatement of the mixture pdf against the reference's own
    VonMisesFisherDistribution<8>::eval on its EM fit (tests/golden)."""
    f, mu, kappa, alpha = _fixture_mixture()
    assert np.all(kappa >= 0) and np.isclose(alpha.sum(), 1.0)
    np.testing.assert_allclose(_mixture_pdf(mu, kappa, alpha, f["vmf_dirs"]), f["vmf_pdf"], rtol=2e-5, atol=1e-7)
    # the fit describes its own samples better than a uniform hemisphere does
    assert np.mean(np.log(f["vmf_sample_pdf"])) > np.log(1 / (2 * np.pi))


@pytest.mark.gpu
def test_gpu_mixture_of_reference_fit(guide):
    """A network whose output layer is the reference's EM fit (zero weights,
    biases = the fit): the GPU decodes that mixture, its pdf matches the
    reference's eval, and its samples follow it."""
    from xitils_gb300 import api
    ctx, _ = guide
    f, mu, kappa, alpha = _fixture_mixture()
    assert np.all((kappa > np.exp(G.KMIN)) & (kappa < np.exp(G.KMAX)))
    gd = api.Guide(ctx, seed=2)
    gd.set_bounds(LO, HI)
    d = G.split(gd.params().astype(np.float64))
    d["W3"][:] = 0.0
    b3 = d["b3"].reshape(8, 5)
    b3[:, 0:3] = mu
    b3[:, 3] = np.log(kappa)
    b3[:, 4] = np.log(alpha)
    gd.set_params(G.join(d).astype(np.float32))
    n = 60000
    pos = np.tile(np.array([[0.1, 0.2, 0.3]], np.float32), (n, 1))
    nrm = np.tile(np.array([[0, 0, 1]], np.float32), (n, 1))
    wo = nrm.copy()
    Y = gd.infer(pos[:1], nrm[:1], wo[:1])
    gmu, gk, ga = G.decode(Y)
    np.testing.assert_allclose(gmu[0], mu / np.linalg.norm(mu, axis=1, keepdims=True), atol=1e-6)
    np.testing.assert_allclose(gk[0], kappa, rtol=1e-5)
    np.testing.assert_allclose(ga[0], alpha, rtol=1e-5, atol=1e-7)
    dirs, pdf = gd.sample(pos[:n // 2], nrm[:n // 2], wo[:n // 2], seed=5)
    dirs2, pdf2 = gd.sample(pos[n // 2:], nrm[n // 2:], wo[n // 2:], seed=6)
    dirs = np.concatenate([dirs, dirs2]).astype(np.float64)
    pdf = np.concatenate([pdf, pdf2])
    np.testing.assert_allclose(pdf, _mixture_pdf(mu, kappa, alpha, dirs), rtol=2e-3, atol=1e-6)
    # octant histogram against the reference's pdf integrated over each octant
    rng = np.random.default_rng(0)
    u = rng.normal(size=(400000, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    p = _mixture_pdf(mu, kappa, alpha, u)
    octant = lambda v: (v[:, 0] > 0).astype(int) * 4 + (v[:, 1] > 0) * 2 + (v[:, 2] > 0)
    expected = np.bincount(octant(u), weights=p * 4 * np.pi / u.shape[0], minlength=8) * n
    observed = np.bincount(octant(dirs), minlength=8)
    mask = expected > 50
    chi2 = np.sum((observed[mask] - expected[mask]) ** 2 / expected[mask])
    assert chi2 < 40, (observed, expected)
