"""CPU checks of the learned texture decoder's oracle: its analytic backward pass against central
finite differences (float64, no roundings), the BF16 rounding helper, and the latent taps."""
import numpy as np

from oracle import neural as N


def _random_params(rng):
    p = np.zeros(N.PARAMS)
    w1 = rng.normal(0, 0.4, (64, 16))
    w1[:, 11:] = 0.0
    p[N.PW1:N.PW2] = w1.reshape(-1)
    p[N.PW2:N.PB2] = rng.normal(0, 0.2, 4096)
    p[N.PB2:N.PW3] = rng.normal(0, 0.1, 64)
    p[N.PW3:N.PB3] = rng.normal(0, 0.2, 512)
    p[N.PB3:] = rng.normal(0.5, 0.1, 8)
    return p


def _loss(p, x0, lvl, t):
    y = N.forward(p, x0, lvl, exact=True)["y"]
    return float(((y - t) ** 2).sum())


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(3)
    p = _random_params(rng)
    x0 = rng.normal(0, 0.7, (128, 8))
    lvl = rng.integers(0, 6, 128)
    t = rng.uniform(0, 1, (128, 8))
    cache = N.forward(p, x0, lvl, exact=True)
    g, dx0, loss = N.backward(p, cache, t, exact=True)
    assert abs(loss - _loss(p, x0, lvl, t)) < 1e-9 * max(1.0, loss)
    # the backward pass is the gradient of loss * GRAD_SCALE / 2 (tile mean of squared error)
    k = N.GRAD_SCALE / 2.0
    eps = 1e-5
    w1_live = np.arange(N.PW1, N.PW2).reshape(64, 16)[:, :11].reshape(-1)
    idx = np.concatenate([rng.choice(w1_live, 40, replace=False), np.arange(N.PW1 + 9, N.PW2, 16)[:4],
                          np.arange(N.PW1 + 10, N.PW2, 16)[:4], rng.choice(np.arange(N.PW2, N.PARAMS), 80, replace=False)])
    for i in idx:
        e = np.zeros_like(p)
        e[i] = eps
        fd = (_loss(p + e, x0, lvl, t) - _loss(p - e, x0, lvl, t)) / (2 * eps) * k
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)) + 1e-9, (i, fd, g[i])
    for s in range(0, 128, 17):
        for c in range(8):
            e = np.zeros_like(x0)
            e[s, c] = eps
            fd = (_loss(p, x0 + e, lvl, t) - _loss(p, x0 - e, lvl, t)) / (2 * eps) * k
            assert abs(fd - dx0[s, c]) <= 1e-6 * max(1.0, abs(fd)) + 1e-9


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, 1.0078125, -3.14159265, 0.0, 1e-30], dtype=np.float32)
    got = N.bf16(x)
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: rounds to even (1); 1 + 1.5 * 2^-8 rounds up
    assert got[0] == 1.0 and got[1] == 1.0 and got[2] == 1.0078125 and got[3] == 1.0078125
    assert got[4] == np.float32(-3.140625) and got[5] == 0.0
    assert (got.view(np.uint32) & 0xFFFF).max() == 0


def test_latent_taps_levels_fractions_and_wrap():
    # latent level 0 is 4 x 4 (texture level 2), latent level 1 is 2 x 2 at offset 16
    lw, lh, off = [4, 2], [4, 2], [0, 16]
    z = np.zeros(16, np.int64)
    idx, fx, fy = N.latent_taps(z, np.arange(16), z, lw, lh, off)  # texture level 0: 4x magnified
    assert np.allclose(fx[:4], [5 / 8, 7 / 8, 1 / 8, 3 / 8]) and np.allclose(fy, 5 / 8)
    # texel 0 sits left of latent texel 0: its left tap wraps to the last column, its upper tap to the last row
    assert idx[0].tolist() == [3 * 4 + 3, 3 * 4 + 0, 0 * 4 + 3, 0]
    idx1, fx1, fy1 = N.latent_taps(np.array([1]), np.array([7]), np.array([7]), lw, lh, off)  # 2x magnified
    assert fx1[0] == 0.25 and fy1[0] == 0.25 and idx1[0].tolist() == [3 * 4 + 3, 3 * 4 + 0, 0 * 4 + 3, 0]
    idx2, fx2, fy2 = N.latent_taps(np.array([2, 3]), np.array([2, 1]), np.array([3, 0]), lw, lh, off)  # 1:1
    assert np.all(fx2 == 0) and np.all(fy2 == 0)
    assert idx2[0, 0] == 3 * 4 + 2 and idx2[1, 0] == 16 + 0 * 2 + 1
    lat = np.arange(20 * 8, dtype=np.float32).reshape(20, 8) / 64
    assert np.array_equal(N.latent_inputs(lat, idx2, fx2, fy2), N.f16(lat[idx2[:, 0]]))
