"""The closure oracle's own identities (CPU): the discrete curl and its
adjoint, div of the curl, finite-difference gradients of the net and the
loss, and the box filter's conservation of mass and of div B = 0."""
import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parents[1] / "oracle"))
import closure_oracle as co  # noqa: E402


def test_curl_adjoint_and_divergence():
    rng = np.random.default_rng(0)
    e = rng.normal(size=(2, 6, 6, 6, 3))
    r = rng.normal(size=(2, 6, 6, 6, 3))
    assert abs(np.sum(co.curl_faces(e) * r) - np.sum(e * co.curl_faces_adjoint(r))) < 1e-10
    d = co.curl_faces(e)
    div = ((np.roll(d[..., 0], -1, axis=-1) - d[..., 0]) + (np.roll(d[..., 1], -1, axis=-2) - d[..., 1]) +
           (np.roll(d[..., 2], -1, axis=-3) - d[..., 2]))
    assert np.abs(div).max() < 1e-12


def test_net_gradient_finite_differences():
    rng = np.random.default_rng(1)
    params = [(rng.normal(size=(4, 3, 3, 3, 3)) * 0.2, rng.normal(size=4) * 0.1),
              (rng.normal(size=(8, 1, 1, 1, 4)) * 0.3, rng.normal(size=8) * 0.1)]
    x = rng.normal(size=(1, 5, 5, 5, 3))
    tu, tb = rng.normal(size=(1, 5, 5, 5, 5)), rng.normal(size=(1, 5, 5, 5, 3))

    def loss(ps):
        out, _ = co.net_forward(ps, x)
        return co.loss_and_grad(out, tu, tb)[0]

    out, cache = co.net_forward(params, x)
    l0, d = co.loss_and_grad(out, tu, tb)
    grads = co.net_backward(params, cache, d)
    eps = 1e-6
    for li, idx in ((0, (1, 2, 0, 1, 2)), (0, (3, 0, 2, 2, 0)), (1, (5, 0, 0, 0, 2)), (1, (0, 0, 0, 0, 1))):
        w, b = params[li]
        w2 = w.copy()
        w2[idx] += eps
        ps = [(w2, b) if i == li else p for i, p in enumerate(params)]
        fd = (loss(ps) - l0) / eps
        assert abs(fd - grads[li][0][idx]) < 1e-5 * max(1.0, abs(fd)), (li, idx, fd, grads[li][0][idx])
    b2 = params[1][1].copy()
    b2[6] += eps
    fd = (loss([params[0], (params[1][0], b2)]) - l0) / eps
    assert abs(fd - grads[1][1][6]) < 1e-5


def test_box_filter_conserves(mhd):
    u, b = mhd.init_turbulence(32, seed=2)
    uc, bc = co.box_filter(u, b, 32, 4)
    U = u.reshape(-1, 5).astype(np.float64)
    Uc = uc.reshape(-1, 5)
    assert np.allclose(U.mean(0), Uc.mean(0), rtol=1e-12, atol=1e-12)
    assert mhd.host_divb_max(bc.astype(np.float32), 8, 8, 8) < 1e-5
