"""The warm-start network's CPU restatement: its backward pass is the gradient of its
forward pass (central finite differences in exact FP64), and the bf16 rounding helper
rounds to nearest-even."""
import numpy as np

from nn_oracle import OracleNet, bf16, col2im, im2col, kp_of, layer_specs


def _weights(c, seed):
    rng = np.random.default_rng(seed)
    out = {}
    for name, cin, cout, _ in layer_specs(c):
        w = np.zeros((cout, kp_of(cin)))
        w[:, :27 * cin] = rng.normal(0, np.sqrt(2.0 / (27 * cin)), size=(cout, 27 * cin))
        if name == "y":
            w[3:] = 0.0
        out[name] = (w, rng.normal(0, 0.1, size=cout))
    return out


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -3.14159265, 1e-30])
    r = bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0          # tie to even
    assert r[2] == 1.0 + 4 * 2 ** -8            # tie to even (up)
    assert abs(r[3] + 3.140625) < 1e-12


def test_im2col_adjoint():
    rng = np.random.default_rng(0)
    g, cin = 4, 3
    X = rng.normal(size=(g ** 3, cin))
    Y = rng.normal(size=(g ** 3, kp_of(cin)))
    Y[:, 27 * cin:] = 0
    # <im2col X, Y> == <X, col2im Y>
    assert abs((im2col(X, g, cin, kp_of(cin)) * Y).sum() - (X * col2im(Y, g, cin)).sum()) < 1e-9


def test_backward_matches_finite_differences():
    c = (2, 3, 3, 4)
    n = 8
    w = _weights(c, 1)
    rng = np.random.default_rng(2)
    x = rng.normal(size=(n ** 3, 2))
    t = rng.normal(size=(n ** 3, 3))
    m = (rng.random(n ** 3) > 0.3).astype(np.float64)
    net = OracleNet(n, c, w, rounding=False)
    net.forward(x)
    _, gy = net.loss_grad(t, m)
    dW, dB = net.backward(gy)

    def loss(ww):
        o = OracleNet(n, c, ww, rounding=False)
        o.forward(x)
        return o.loss_grad(t, m)[0]

    eps = 1e-6
    for name, idx in [("e1", (1, 5)), ("b", (2, 40)), ("d2", (0, 17)), ("y", (1, 3)), ("d1", (1, 60))]:
        wp = {k: (v[0].copy(), v[1].copy()) for k, v in w.items()}
        wm = {k: (v[0].copy(), v[1].copy()) for k, v in w.items()}
        wp[name][0][idx] += eps
        wm[name][0][idx] -= eps
        fd = (loss(wp) - loss(wm)) / (2 * eps)
        assert abs(fd - dW[name][idx]) <= 1e-6 * max(1.0, abs(fd)), (name, fd, dW[name][idx])
    wp = {k: (v[0].copy(), v[1].copy()) for k, v in w.items()}
    wm = {k: (v[0].copy(), v[1].copy()) for k, v in w.items()}
    wp["e2"][1][1] += eps
    wm["e2"][1][1] -= eps
    fd = (loss(wp) - loss(wm)) / (2 * eps)
    assert abs(fd - dB["e2"][1]) <= 1e-6 * max(1.0, abs(fd))
