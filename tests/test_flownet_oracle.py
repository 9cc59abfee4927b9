"""The float64 network oracle (oracle/flownet.py) against finite differences of its own loss."""
import numpy as np

import oracle.flownet as OF


def test_oracle_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    offs, total = OF.offsets()
    p = np.zeros(total)
    for (taps, cin, cout, _), (wo, bo) in zip(OF.LAYERS, offs):
        p[wo:wo + taps * cin * cout] = rng.standard_normal(taps * cin * cout) * np.sqrt(2 / (taps * cin))
        p[bo:bo + cout] = rng.standard_normal(cout) * 0.1
    x = rng.standard_normal((1, 8, 16, 16))
    lab = rng.standard_normal((1, 8, 16, 4)) * 0.5
    lab[0, 0, 0, 1] = np.nan
    _, g, _ = OF.loss_and_grads(p, x, lab)
    eps = 1e-6
    for li, (wo, bo) in enumerate(offs):
        for i in (wo + 3, wo + 7, bo):
            pp, pm = p.copy(), p.copy()
            pp[i] += eps
            pm[i] -= eps
            fd = (OF.loss_and_grads(pp, x, lab)[0] - OF.loss_and_grads(pm, x, lab)[0]) / (2 * eps)
            assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (li, i, fd, g[i])


def test_bf16_rounding_is_nearest_even():
    vals = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, 0.0, 3.14159], np.float64)
    got = OF.bf16_round(vals)
    assert got[0] == 1.0 and got[1] == 1.0 and got[2] == 1.0 + 2 ** -6 and got[3] == -2.5 and got[4] == 0.0
    assert abs(got[5] - 3.140625) < 1e-12
