"""The CPU restatement of the warm-start network is itself checked: with the bfloat16 rounding
switched off its analytic gradients match central finite differences (float64, 1e-6 relative)."""
import numpy as np

from oracle import mlp_oracle as MO


def test_oracle_gradients_match_finite_differences(monkeypatch):
    monkeypatch.setattr(MO, "bf16", lambda a: np.asarray(a, np.float64))
    rng = np.random.Generator(np.random.PCG64(0))
    p = MO.init_params(0).astype(np.float64)
    p[MO.F * MO.H:MO.F * MO.H + MO.H] = rng.normal(0, 0.1, MO.H)
    norm = MO.identity_norm()
    x = rng.normal(0, 1, (17, 12))
    t = rng.normal(0, 1, (17, 3))
    g, _ = MO.gradients(p, norm, x, t)
    idx = rng.choice(MO.N_PARAMS, 60, replace=False)
    h = 1e-5
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        lp = MO.gradients(pp, norm, x, t)[1]
        lm = MO.gradients(pm, norm, x, t)[1]
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])


def test_bf16_rounding_is_round_to_nearest_even():
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 1.0 + 2 ** -9, -2.5], np.float32)
    r = MO.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -6 and r[3] == 1.0 and r[4] == -2.5
