"""The learned edge's CPU oracle pinned on its own: the backward pass against
central differences of the (unrounded) forward pass, bfloat16 rounding on
known values, and the Adam step written out by hand."""
import numpy as np

from oracle import edge_ref as R


def _random(seed, n=40, scale=0.3):
    rng = np.random.default_rng(seed)
    params = (rng.standard_normal(R.SETS * R.SET_PARAMS) * scale).astype(np.float32)
    sets = rng.integers(0, R.SETS, n).astype(np.int32)
    x = rng.standard_normal((n, R.IN)).astype(np.float32)
    t = rng.standard_normal((n, R.OUT)).astype(np.float32)
    return params, sets, x, t


def test_gradient_matches_central_differences():
    params, sets, x, t = _random(1, n=24, scale=0.15)
    p64 = params.astype(np.float64)
    grad, loss = R.gradients(p64, sets, x, t, exact=True)

    def loss_at(p):
        y = R.forward(p, sets, x, exact=True)
        return float(np.mean((y - t) ** 2))

    assert abs(loss - loss_at(p64)) < 1e-12
    rng = np.random.default_rng(2)
    used = np.unique(sets)
    for _ in range(60):
        s = int(rng.choice(used))
        k = s * R.SET_PARAMS + int(rng.integers(0, R.SET_PARAMS))
        h = 1e-6
        pp, pm = p64.copy(), p64.copy()
        pp[k] += h
        pm[k] -= h
        fd = (loss_at(pp) - loss_at(pm)) / (2 * h)
        assert abs(fd - grad[k]) <= 1e-6 + 1e-5 * abs(fd), (k, fd, grad[k])
    # sets with no sample have zero gradient
    for s in set(range(R.SETS)) - set(used.tolist()):
        assert not np.any(grad[s * R.SET_PARAMS:(s + 1) * R.SET_PARAMS])


def test_bf16_rounding():
    # bfloat16 keeps 8 significant bits: the spacing above 1 is 2^-7
    v = np.array([1.0, 1 + 2.0 ** -7, 1 + 2.0 ** -8, 1 + 3 * 2.0 ** -8, 1 + 2.0 ** -8 + 2.0 ** -10, -2.5, 0.0],
                 np.float32)
    r = R.bf16(v)
    assert r[0] == 1.0 and r[1] == np.float32(1 + 2.0 ** -7)      # representable
    assert r[2] == 1.0                                            # tie, to the even neighbour
    assert r[3] == np.float32(1 + 2.0 ** -6)                      # tie, to the even neighbour
    assert r[4] == np.float32(1 + 2.0 ** -7)                      # above the tie
    assert r[5] == -2.5 and r[6] == 0.0
    assert np.all(R.bf16(r) == r)


def test_adam_step():
    rng = np.random.default_rng(3)
    w0 = rng.standard_normal(50).astype(np.float32)
    g1, g2 = rng.standard_normal(50).astype(np.float32), rng.standard_normal(50).astype(np.float32)
    opt = R.Adam(w0)
    opt.step(g1, 0.01)
    w = opt.step(g2, 0.01)
    m = 0.9 * (0.1 * g1.astype(np.float64)) + 0.1 * g2
    v = 0.999 * (0.001 * g1.astype(np.float64) ** 2) + 0.001 * g2.astype(np.float64) ** 2
    w1 = w0 - 0.01 * (0.1 * g1 / 0.1) / (np.sqrt(0.001 * g1.astype(np.float64) ** 2 / 0.001) + 1e-8)
    want = w1 - 0.01 * (m / (1 - 0.9 ** 2)) / (np.sqrt(v / (1 - 0.999 ** 2)) + 1e-8)
    np.testing.assert_allclose(w, want, rtol=1e-5, atol=1e-6)
