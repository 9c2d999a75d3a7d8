"""The learned proposal's CPU oracle (oracle/net_oracle.py) pinned without
the library: BF16 rounding against hand-checked values, the features against
their definition, the analytic gradient against central differences."""
import numpy as np

from oracle import net_oracle as no


def test_bf16_rounding_known_values():
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: even mantissa (1.0) wins;
    # 1 + 3*2^-8 ties between 1 + 2^-7 and 1 + 2^-6: even is 1 + 2^-6
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 1.0 + 2 ** -8 + 2 ** -20, -2.5, 3.0e38], dtype=np.float32)
    r = no.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -6 and r[3] == 1.0 + 2 ** -7
    assert r[4] == -2.5
    assert np.isfinite(r[5]) and abs(r[5] / 3.0e38 - 1) < 2 ** -8


def test_features_definition():
    u = np.array([[0.0, 0.25, 0.5], [0.125, 1.0, 0.3]])
    f = no.features(u)
    assert f.shape == (2, 48)
    # octave 0, axis 1 of the first point: sin(pi/4), cos(pi/4)
    assert np.isclose(f[0, 2], np.sqrt(0.5)) and np.isclose(f[0, 3], np.sqrt(0.5))
    # octave 3, axis 0 of the second point: angle pi * 8 * 0.125 = pi
    assert np.isclose(f[1, 2 * 9], 0.0, atol=1e-12) and np.isclose(f[1, 2 * 9 + 1], -1.0)


def test_gradient_matches_central_differences():
    rng = np.random.default_rng(3)
    p = no.init_params(5)
    p[no.OFF_B1:no.OFF_W2] = rng.standard_normal(64) * 0.1
    p[no.OFF_B2:no.OFF_W3] = rng.standard_normal(64) * 0.1
    u = rng.random((256, 3))
    t = rng.standard_normal(256)
    assert no.fd_check(p, u, t, n_probe=60) < 1e-6


def test_rounded_forward_close_to_exact():
    """The BF16 roundings move the output by far less than the spread of lambda."""
    rng = np.random.default_rng(4)
    p = no.init_params(6)
    u = rng.random((2048, 3))
    a, _ = no.forward(p, u, rounding=True)
    b, _ = no.forward(p, u, rounding=False)
    assert np.max(np.abs(a - b)) < 0.05 * (np.std(b) + 1e-3) * 10
