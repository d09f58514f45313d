"""CPU pins of the surrogate's oracle (oracle/mlp.py): its closed-form bond integral
against the C oracle's exact (clip + erf) and adaptive (QAG) modes of the Gaussian
kernel, and its reverse-mode gradient against central finite differences."""
import numpy as np
import pytest

from oracle import mlp as M


def _bond_w(oracle, mode, d, a, b):
    # the grid point at (0, d); the bond on the x axis from a to b (units of w = 1)
    cg = oracle.make_cg("gaussian", rcut=3.0, mode=mode, order=5, width=1.0, epsabs=1e-14, epsrel=1e-13)
    norm = oracle.delta(cg, 2, 0.0)
    return oracle.bond(cg, 2, [0.0, d, 0.0], [a, 0.0, 0.0], [b - a, 0.0, 0.0]) / norm


def test_label_closed_form_matches_oracle_modes(oracle):
    rng = np.random.default_rng(3)
    for _ in range(200):
        d = rng.uniform(0, 3)
        tc = np.sqrt(9 - d * d)
        a = rng.uniform(-tc, tc)
        b = a + rng.uniform(0.05, 2.5) * rng.choice([-1, 1])
        want = M.label(d, a, b)
        assert abs(_bond_w(oracle, "exact", d, a, b) - want) <= 1e-13
        # adaptive QAG on [0, 1] meets its tolerance where the integrand is smooth; across
        # the jump at the edge of the support it converges slowly (why labels clip first)
        crossing = (d * d + b * b >= 9.0) != (d * d + a * a >= 9.0)
        assert abs(_bond_w(oracle, "adaptive", d, a, b) - want) <= (1e-5 if crossing else 1e-10)
    # symmetric in the direction of the bond and under reflection
    assert M.label(1.0, -0.5, 2.9) == pytest.approx(M.label(1.0, 2.9, -0.5), abs=1e-15)
    assert M.label(1.0, -0.5, 2.9) == pytest.approx(M.label(1.0, 0.5, -2.9), abs=1e-15)
    # fully outside -> 0
    assert M.label(2.5, 2.0, 3.0) == 0.0


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(5)
    p = rng.normal(0, 0.3, M.NPAR)
    n = 16
    feats = np.stack([rng.uniform(0, 3, n), rng.uniform(-3, 3, n), rng.uniform(0, 4, n),
                      rng.choice([1.0, 2.0], n)], axis=1).astype(np.float32)
    y = rng.uniform(0, 1, n).astype(np.float32)
    loss, g = M.loss_and_grad(p, feats, y)
    assert loss == pytest.approx(np.mean((M.forward(p, feats) - y.astype(np.float64)) ** 2), rel=1e-12)
    idx = np.concatenate([rng.choice(np.arange(lo, hi), 6, replace=False) for lo, hi in
                          [(M.O_W1, M.O_B1), (M.O_B1, M.O_W2), (M.O_W2, M.O_B2), (M.O_B2, M.O_W3),
                           (M.O_W3, M.O_B3), (M.O_B3, M.O_W4), (M.O_W4, M.O_B4)]] + [[M.O_B4]])
    h = 1e-6
    for k in idx:
        pp, pm = p.copy(), p.copy()
        pp[k] += h
        pm[k] -= h
        fd = (M.loss_and_grad(pp, feats, y)[0] - M.loss_and_grad(pm, feats, y)[0]) / (2 * h)
        assert g[k] == pytest.approx(fd, rel=2e-6, abs=1e-10), k


def test_bf16_rounding():
    v = np.array([1.0, 1.00390625, 1.005859375, -3.14159, 0.0], dtype=np.float32)
    r = M.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0  # tie to even
    assert r[2] == 1.0078125
    assert abs(r[3] + 3.140625) < 1e-7 and r[4] == 0.0


def test_baseline_is_gl4_on_the_clipped_segment_and_close():
    """The surrogate's baseline (four-point Gauss-Legendre on the part of the bond inside
    the support) is within 1e-4 relative of the exact integral over the sampled domain,
    which bounds the scaled target y = (B / base - 1) * 1e4 to about one."""
    rng = np.random.default_rng(9)
    n = 200000
    d = rng.uniform(0, 3, n)
    tc = np.sqrt(9 - d * d)
    a = rng.uniform(-tc, tc)
    b = a + rng.uniform(0, 2.5, n)
    keep = (b >= tc) & (b <= 4)
    f = np.stack([d, a, b, np.ones(n)], axis=1)[keep].astype(np.float32)
    lab = M.label(f[:, 0], f[:, 1], f[:, 2])
    bs = M.base(f)
    rel = np.abs(bs / lab - 1.0)
    assert rel.max() < 1e-4
    y = M.targets(f, lab)
    assert np.max(np.abs(y)) < 1.0
    big = bs > M.BASE_MIN  # below it the target is 0 and B is the baseline's (error < 1e-10)
    np.testing.assert_allclose(M.value(f, y)[big], lab[big], rtol=1e-12, atol=0)
    assert np.max(np.abs(M.value(f, y)[~big] - lab[~big])) < 1e-10
    # the rule itself: four points integrate a cubic on [a, t_c] exactly
    x, w = np.polynomial.legendre.leggauss(4)
    assert abs(np.sum(w * x ** 6) - 2.0 / 7.0) < 1e-15 and abs(np.sum(w * x ** 8) - 2.0 / 9.0) > 1e-3
