"""CPU restatement of the warm-start network's forward and backward passes (test
infrastructure: the GPU kernels are checked against it; nothing in the product imports
this file).

FP64 arithmetic with bf16 rounding at exactly the points where the GPU path stores
bf16 (input, weights, activations, gradients fed to the tensor-core GEMMs), so the
remaining difference to the GPU is its FP32 accumulation order.  Layout, architecture
and periodic 3x3x3 stencils are those of mflbm.warmstart: channels-last [z][y][x][c],
col[v][tap*Cin + c] = X[v + d_tap][c] with tap = (dz+1)*9 + (dy+1)*3 + (dx+1).
"""
import numpy as np

NOUT = 16


def bf16(a):
    """Round to bfloat16 (nearest, ties to even) and return as float64."""
    x = np.ascontiguousarray(a, dtype=np.float32)
    b = x.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def kp_of(cin):
    return ((27 * cin + 63) // 64) * 64


def layer_specs(c):
    c1, c2, c3, c4 = c
    return [("e1", 2, c1, True), ("e2", c1, c2, True), ("e3", c2, c3, True), ("b", c3, c4, True),
            ("d3", c4 + c3, c3, True), ("d2", c3 + c2, c2, True), ("d1", c2 + c1, c1, True), ("y", c1, NOUT, False)]


def _taps():
    return [(dz, dy, dx) for dz in (-1, 0, 1) for dy in (-1, 0, 1) for dx in (-1, 0, 1)]


def im2col(X, g, cin, kp):
    V = X.reshape(g, g, g, cin)
    col = np.zeros((g ** 3, kp))
    for t, (dz, dy, dx) in enumerate(_taps()):
        # value at v + d: roll by -d
        sh = np.roll(V, shift=(-dz, -dy, -dx), axis=(0, 1, 2)).reshape(g ** 3, cin)
        col[:, t * cin:(t + 1) * cin] = sh
    return col


def col2im(dcol, g, cin):
    out = np.zeros((g, g, g, cin))
    for t, (dz, dy, dx) in enumerate(_taps()):
        part = dcol[:, t * cin:(t + 1) * cin].reshape(g, g, g, cin)
        out += np.roll(part, shift=(dz, dy, dx), axis=(0, 1, 2))
    return out.reshape(g ** 3, cin)


def pool(X, g, c):
    V = X.reshape(g // 2, 2, g // 2, 2, g // 2, 2, c)
    return V.mean(axis=(1, 3, 5)).reshape(-1, c)


def pool_back(dY, g, c):
    V = dY.reshape(g // 2, g // 2, g // 2, c) * 0.125
    return np.repeat(np.repeat(np.repeat(V, 2, axis=0), 2, axis=1), 2, axis=2).reshape(-1, c)


def up_concat(Xc, c1, S, c2, g):
    V = Xc.reshape(g // 2, g // 2, g // 2, c1)
    up = np.repeat(np.repeat(np.repeat(V, 2, axis=0), 2, axis=1), 2, axis=2).reshape(-1, c1)
    return np.concatenate([up, S], axis=1)


def up_concat_back(dY, c1, c2, g):
    d_up = dY[:, :c1].reshape(g // 2, 2, g // 2, 2, g // 2, 2, c1).sum(axis=(1, 3, 5)).reshape(-1, c1)
    return d_up, dY[:, c1:]


class OracleNet:
    """rounding=False drops the bf16 rounding (exact FP64 network, for finite differences)."""

    def __init__(self, n, c, weights, rounding=True):
        self.n, self.c = n, c
        self.r = bf16 if rounding else (lambda a: np.asarray(a, dtype=np.float64))
        self.specs = {s[0]: s for s in layer_specs(c)}
        self.grid = {"e1": n, "e2": n // 2, "e3": n // 4, "b": n // 8, "d3": n // 4, "d2": n // 2, "d1": n, "y": n}
        self.Wb = {k: self.r(w) for k, (w, _) in weights.items()}
        self.B = {k: b.astype(np.float64) for k, (_, b) in weights.items()}

    def conv(self, name, X):
        _, cin, cout, relu = self.specs[name]
        g = self.grid[name]
        col = im2col(X, g, cin, kp_of(cin))
        pre = col @ self.Wb[name].T + self.B[name]
        self.cache[name] = (col, pre)
        y = np.maximum(pre, 0.0) if relu else pre
        return self.r(y) if name != "y" else y

    def forward(self, x):
        self.cache = {}
        n = self.n
        c1, c2, c3, c4 = self.c
        x = self.r(x)
        e1 = self.conv("e1", x)
        e2 = self.conv("e2", self.r(pool(e1, n, c1)))
        e3 = self.conv("e3", self.r(pool(e2, n // 2, c2)))
        b = self.conv("b", self.r(pool(e3, n // 4, c3)))
        d3 = self.conv("d3", up_concat(b, c4, e3, c3, n // 4))
        d2 = self.conv("d2", up_concat(d3, c3, e2, c2, n // 2))
        d1 = self.conv("d1", up_concat(d2, c2, e1, c1, n))
        self.out = self.conv("y", d1)
        return self.out

    def loss_grad(self, target, mask):
        cnt = max(1.0, mask.sum() * 3.0)
        d = (self.out[:, :3] - target) * mask[:, None]
        g = np.zeros_like(self.out)
        g[:, :3] = 2.0 * d / cnt
        return (d * d).sum() / cnt, g

    def conv_back(self, name, g):
        _, cin, cout, relu = self.specs[name]
        col, pre = self.cache[name]
        if relu:
            g = g * (pre > 0)
        self.dB[name] = g.sum(axis=0)
        gb = self.r(g)
        self.dW[name] = gb.T @ col
        dcol = gb @ self.Wb[name]
        return col2im(dcol, self.grid[name], cin)

    def backward(self, gy):
        n = self.n
        c1, c2, c3, c4 = self.c
        self.dW, self.dB = {}, {}
        gd1 = self.conv_back("y", gy)
        gcat = self.conv_back("d1", gd1)
        gd2, gs1 = up_concat_back(gcat, c2, c1, n)
        gcat = self.conv_back("d2", gd2)
        gd3, gs2 = up_concat_back(gcat, c3, c2, n // 2)
        gcat = self.conv_back("d3", gd3)
        gb_, gs3 = up_concat_back(gcat, c4, c3, n // 4)
        gp3 = self.conv_back("b", gb_)
        ge3 = pool_back(gp3, n // 4, c3) + gs3
        gp2 = self.conv_back("e3", ge3)
        ge2 = pool_back(gp2, n // 2, c2) + gs2
        gp1 = self.conv_back("e2", ge2)
        ge1 = pool_back(gp1, n, c1) + gs1
        self.conv_back("e1", ge1)
        return self.dW, self.dB


class OracleAdam:
    """Adam (Kingma & Ba 2015) on the FP64 weights {name: [W, b]}, the update of the GPU's
    k_adam without its bf16 weight copy."""

    def __init__(self, weights, lr, b1=0.9, b2=0.999, eps=1e-8):
        self.w = {k: [np.array(v[0], dtype=np.float64), np.array(v[1], dtype=np.float64)] for k, v in weights.items()}
        self.m = {k: [np.zeros_like(v[0]), np.zeros_like(v[1])] for k, v in self.w.items()}
        self.v = {k: [np.zeros_like(v[0]), np.zeros_like(v[1])] for k, v in self.w.items()}
        self.lr, self.b1, self.b2, self.eps, self.t = lr, b1, b2, eps, 0

    def step(self, dW, dB):
        self.t += 1
        for k in self.w:
            for j, g in enumerate((dW[k], dB[k])):
                self.m[k][j] = self.b1 * self.m[k][j] + (1 - self.b1) * g
                self.v[k][j] = self.b2 * self.v[k][j] + (1 - self.b2) * g * g
                mh = self.m[k][j] / (1 - self.b1 ** self.t)
                vh = self.v[k][j] / (1 - self.b2 ** self.t)
                self.w[k][j] -= self.lr * mh / (np.sqrt(vh) + self.eps)

    def weights(self):
        return {k: (v[0], v[1]) for k, v in self.w.items()}
