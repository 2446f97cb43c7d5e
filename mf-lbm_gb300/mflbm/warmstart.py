"""Learned warm start for singlephase permeability runs.

A 4-level 3-D convolutional encoder-decoder maps a periodic sample, encoded as two
channels (solid mask, signed distance to the solid surface / 8), to the steady velocity
field scaled by nu / F_z / 10.  Every convolution is a 3x3x3 periodic stencil computed as
im2col + BF16 GEMM on the tcgen05 tensor cores with FP32 accumulation
(mflbm_nn_gemm_bf16); pooling, upsampling, loss and Adam are the project's own kernels.
PyTorch only allocates the device buffers.  The LBM initialised from the prediction
(equilibrium at rho = 1 and the predicted u) still runs to the same convergence
criterion, so the plain method is both the fallback and the arbiter of the result.

Architecture (channels c = (c1, c2, c3, c4), grid n divisible by 8):
    e1 = conv(x, 2 -> c1)            n      p1 = pool(e1)
    e2 = conv(p1, c1 -> c2)          n/2    p2 = pool(e2)
    e3 = conv(p2, c2 -> c3)          n/4    p3 = pool(e3)
    b  = conv(p3, c3 -> c4)          n/8
    d3 = conv([up(b), e3], c4+c3 -> c3)     n/4
    d2 = conv([up(d3), e2], c3+c2 -> c2)    n/2
    d1 = conv([up(d2), e1], c2+c1 -> c1)    n
    y  = conv(d1, c1 -> 16), no activation; channels 0..2 are (u, v, w), 3 the density
         deviation from the sample's mean density
ReLU after every convolution but the last.
"""
import ctypes as C
import math

import numpy as np

from . import _capi

NOUT = 16          # output channels of the last GEMM (N % 16); 0..2 velocity, 3 density
U_SCALE = 10.0     # target = u * nu / F_z / U_SCALE
RHO_SCALE = 1e4    # target channel 3 = (rho - mean_density) * RHO_SCALE
NTARGET = 4


def _kp(cin):
    return ((27 * cin + 63) // 64) * 64


def layer_specs(c=(16, 32, 64, 128)):
    c1, c2, c3, c4 = c
    return [("e1", 2, c1, True), ("e2", c1, c2, True), ("e3", c2, c3, True), ("b", c3, c4, True),
            ("d3", c4 + c3, c3, True), ("d2", c3 + c2, c2, True), ("d1", c2 + c1, c1, True), ("y", c1, NOUT, False)]


def init_weights(c=(16, 32, 64, 128), seed=0):
    """He-initialised fp32 weights [Cout][Kp] (zero in the K padding) and zero biases;
    output channels >= 3 of the last layer start (and stay) at zero."""
    rng = np.random.default_rng(seed)
    out = {}
    for name, cin, cout, _ in layer_specs(c):
        kp = _kp(cin)
        w = np.zeros((cout, kp), dtype=np.float32)
        std = math.sqrt(2.0 / (27 * cin))
        w[:, :27 * cin] = rng.normal(0.0, std, size=(cout, 27 * cin)).astype(np.float32)
        if name == "y":
            w[NTARGET:] = 0.0
            w[:NTARGET] *= 0.1
        out[name] = (w, np.zeros(cout, dtype=np.float32))
    return out


class Net:
    """The network on one GPU for a fixed grid n (n^3 voxels, n % 8 == 0)."""

    def __init__(self, n, c=(16, 32, 64, 128), weights=None, seed=0, device=0, lib=None):
        import torch
        self.torch = torch
        self.lib = lib or _capi.load()
        self.dev = torch.device("cuda", device)
        self.n = n
        self.c = c
        self.specs = layer_specs(c)
        self.grid = {"e1": n, "e2": n // 2, "e3": n // 4, "b": n // 8, "d3": n // 4, "d2": n // 2, "d1": n, "y": n}
        w0 = weights or init_weights(c, seed)
        f32, b16 = torch.float32, torch.bfloat16
        self.W = {k: torch.from_numpy(w).to(self.dev) for k, (w, _) in w0.items()}
        self.B = {k: torch.from_numpy(b).to(self.dev) for k, (_, b) in w0.items()}
        self.Wb = {k: v.to(b16) for k, v in self.W.items()}
        self.dW = {k: torch.zeros_like(v) for k, v in self.W.items()}
        self.dB = {k: torch.zeros_like(v) for k, v in self.B.items()}
        self.mW = {k: torch.zeros_like(v) for k, v in self.W.items()}
        self.vW = {k: torch.zeros_like(v) for k, v in self.W.items()}
        self.mB = {k: torch.zeros_like(v) for k, v in self.B.items()}
        self.vB = {k: torch.zeros_like(v) for k, v in self.B.items()}
        self.step_count = 0
        self.calls = 0       # C-ABI calls issued (each launches one kernel, split-K GEMMs two)
        nv = n ** 3
        maxk = max(_kp(cin) for _, cin, _, _ in self.specs)
        self.col = {}        # im2col of every layer (kept for the backward pass)
        self.pre = {}        # pre-activations (fp32)
        self.act = {}        # activations (bf16)
        for name, cin, cout, _ in self.specs:
            g = self.grid[name]
            self.col[name] = torch.empty(g ** 3, _kp(cin), dtype=b16, device=self.dev)
            self.pre[name] = torch.empty(g ** 3, cout, dtype=f32, device=self.dev)
            self.act[name] = torch.empty(g ** 3, cout, dtype=b16, device=self.dev)
        self.pool = {k: torch.empty((n // s) ** 3, ch, dtype=b16, device=self.dev)
                     for k, s, ch in (("p1", 2, c[0]), ("p2", 4, c[1]), ("p3", 8, c[2]))}
        self.cat = {"d3": torch.empty((n // 4) ** 3, c[3] + c[2], dtype=b16, device=self.dev),
                    "d2": torch.empty((n // 2) ** 3, c[2] + c[1], dtype=b16, device=self.dev),
                    "d1": torch.empty(nv, c[1] + c[0], dtype=b16, device=self.dev)}
        self.acc = torch.empty(nv * max(cout for _, _, cout, _ in self.specs), dtype=f32, device=self.dev)
        self.x = torch.empty(nv, 2, dtype=b16, device=self.dev)
        self.out = torch.empty(nv, NOUT, dtype=f32, device=self.dev)
        # backward scratch
        self.g = {name: torch.empty(self.grid[name] ** 3, cout, dtype=f32, device=self.dev)
                  for name, _, cout, _ in self.specs}
        self.gcat = {k: torch.empty_like(v, dtype=f32) for k, v in self.cat.items()}
        self.gpool = {k: torch.empty_like(v, dtype=f32) for k, v in self.pool.items()}
        self.gskip = {k: torch.empty(self.grid[k] ** 3, ch, dtype=f32, device=self.dev)
                      for k, ch in (("e1", c[0]), ("e2", c[1]), ("e3", c[2]))}
        def vpad(name):
            return ((self.grid[name] ** 3 + 7) // 8) * 8
        maxc = max(cout for _, _, cout, _ in self.specs)
        self.gT = torch.empty(max(cout * vpad(nm) for nm, _, cout, _ in self.specs), dtype=b16, device=self.dev)
        self.colT = torch.empty(max(_kp(cin) * vpad(nm) for nm, cin, _, _ in self.specs), dtype=b16, device=self.dev)
        self.gb = torch.empty(max(cout * self.grid[nm] ** 3 for nm, _, cout, _ in self.specs), dtype=b16,
                              device=self.dev)
        self.WT = torch.empty(maxk * maxc, dtype=b16, device=self.dev)
        self.dcol = torch.empty(max(_kp(cin) * self.grid[nm] ** 3 for nm, cin, _, _ in self.specs), dtype=f32,
                                device=self.dev)
        self.ksplit = 256
        self.work = torch.empty(self.ksplit * maxk * maxc, dtype=f32, device=self.dev)
        self.err = torch.zeros(1, dtype=torch.int32, device=self.dev)
        self.partial = torch.empty((nv * NTARGET + 255) // 256, dtype=torch.float64, device=self.dev)
        self.stream = C.c_void_p(torch.cuda.current_stream(self.dev).cuda_stream)

    # ---- helpers -----------------------------------------------------------------------
    def _ck(self, rc, what):
        self.calls += 1
        if rc:
            raise _capi.MflbmError(rc, what)

    @staticmethod
    def _p(t):
        return C.c_void_p(t.data_ptr())

    # ---- forward -----------------------------------------------------------------------
    def _conv(self, name, X):
        _, cin, cout, relu = next(s for s in self.specs if s[0] == name)
        g = self.grid[name]
        nv = g ** 3
        kp = _kp(cin)
        L, p, s = self.lib, self._p, self.stream
        col = self.col[name]
        self._ck(L.mflbm_nn_im2col(p(X), g, g, g, cin, kp, p(col), s), "im2col")
        self._ck(L.mflbm_nn_gemm_bf16(p(col), kp, p(self.Wb[name]), kp, p(self.acc), cout, nv, cout, kp, 0,
                                      p(self.err), s), "gemm")
        yf = p(self.out) if name == "y" else None
        self._ck(L.mflbm_nn_bias_act(p(self.acc), p(self.B[name]), p(self.pre[name]), p(self.act[name]), yf, nv, cout,
                                     cout, int(relu), s), "bias_act")
        return self.act[name]

    def forward(self, x_bf16=None):
        """x: (n^3, 2) bf16 input in self.x (or given); returns self.out (n^3, 16) fp32."""
        if x_bf16 is not None:
            self.x.copy_(x_bf16)
        L, p, s, n = self.lib, self._p, self.stream, self.n
        c1, c2, c3, c4 = self.c
        e1 = self._conv("e1", self.x)
        self._ck(L.mflbm_nn_avgpool2(p(e1), p(self.pool["p1"]), n, n, n, c1, s), "pool")
        e2 = self._conv("e2", self.pool["p1"])
        self._ck(L.mflbm_nn_avgpool2(p(e2), p(self.pool["p2"]), n // 2, n // 2, n // 2, c2, s), "pool")
        e3 = self._conv("e3", self.pool["p2"])
        self._ck(L.mflbm_nn_avgpool2(p(e3), p(self.pool["p3"]), n // 4, n // 4, n // 4, c3, s), "pool")
        b = self._conv("b", self.pool["p3"])
        self._ck(L.mflbm_nn_up2_concat(p(b), c4, p(e3), c3, p(self.cat["d3"]), n // 4, n // 4, n // 4, s), "up")
        d3 = self._conv("d3", self.cat["d3"])
        self._ck(L.mflbm_nn_up2_concat(p(d3), c3, p(e2), c2, p(self.cat["d2"]), n // 2, n // 2, n // 2, s), "up")
        d2 = self._conv("d2", self.cat["d2"])
        self._ck(L.mflbm_nn_up2_concat(p(d2), c2, p(e1), c1, p(self.cat["d1"]), n, n, n, s), "up")
        d1 = self._conv("d1", self.cat["d1"])
        self._conv("y", d1)
        return self.out

    # ---- backward ----------------------------------------------------------------------
    def _conv_back(self, name, gY, need_dx, dX=None):
        """gY: fp32 gradient w.r.t. the layer output (modified in place by the ReLU mask)."""
        _, cin, cout, relu = next(s for s in self.specs if s[0] == name)
        g = self.grid[name]
        nv = g ** 3
        kp = _kp(cin)
        vp = ((nv + 7) // 8) * 8
        L, p, s = self.lib, self._p, self.stream
        if relu:
            self._ck(L.mflbm_nn_relu_back(p(gY), p(self.pre[name]), nv * cout, s), "relu_back")
        self._ck(L.mflbm_nn_bias_grad(p(gY), p(self.dB[name]), nv, cout, s), "bias_grad")
        # dW[cout][kp] = g^T[cout][V] . col^T[kp][V]^T, reduced over every voxel (split K)
        self._ck(L.mflbm_nn_transpose_bf16(p(gY), 1, cout, cout, nv, p(self.gT), vp, cout, vp, s), "transpose g")
        self._ck(L.mflbm_nn_transpose_bf16(p(self.col[name]), 0, kp, kp, nv, p(self.colT), vp, kp, vp, s),
                 "transpose col")
        ks = max(1, min(self.ksplit, (vp + 63) // 64 // 4))
        self._ck(L.mflbm_nn_gemm_bf16_splitk(p(self.gT), vp, p(self.colT), vp, p(self.dW[name]), kp, cout, kp, vp, 0,
                                             ks, p(self.work), p(self.err), s), "gemm dW")
        if need_dx:
            # dcol[V][kp] = g[V][cout] . W^T[kp][cout]^T, then the adjoint of im2col
            self._ck(L.mflbm_nn_to_bf16(p(gY), p(self.gb), nv * cout, s), "to_bf16")
            self._ck(L.mflbm_nn_transpose_bf16(p(self.Wb[name]), 0, kp, kp, cout, p(self.WT), cout, kp, cout, s),
                     "transpose W")
            self._ck(L.mflbm_nn_gemm_bf16(p(self.gb), cout, p(self.WT), cout, p(self.dcol), kp, nv, kp, cout, 0,
                                          p(self.err), s), "gemm dcol")
            self._ck(L.mflbm_nn_col2im(p(self.dcol), g, g, g, cin, kp, p(dX), s), "col2im")

    def backward(self):
        """Gradients of the loss whose output gradient is in self.g['y']."""
        L, p, s, n = self.lib, self._p, self.stream, self.n
        c1, c2, c3, c4 = self.c
        self._conv_back("y", self.g["y"], True, self.g["d1"])
        self._conv_back("d1", self.g["d1"], True, self.gcat["d1"])
        self._ck(L.mflbm_nn_up2_concat_back(p(self.gcat["d1"]), p(self.g["d2"]), c2, p(self.gskip["e1"]), c1, n, n, n,
                                            s), "up back")
        self._conv_back("d2", self.g["d2"], True, self.gcat["d2"])
        self._ck(L.mflbm_nn_up2_concat_back(p(self.gcat["d2"]), p(self.g["d3"]), c3, p(self.gskip["e2"]), c2, n // 2,
                                            n // 2, n // 2, s), "up back")
        self._conv_back("d3", self.g["d3"], True, self.gcat["d3"])
        self._ck(L.mflbm_nn_up2_concat_back(p(self.gcat["d3"]), p(self.g["b"]), c4, p(self.gskip["e3"]), c3, n // 4,
                                            n // 4, n // 4, s), "up back")
        self._conv_back("b", self.g["b"], True, self.gpool["p3"])
        self._ck(L.mflbm_nn_avgpool2_back(p(self.gpool["p3"]), p(self.g["e3"]), n // 4, n // 4, n // 4, c3, s), "pool b")
        self._ck(L.mflbm_nn_add(p(self.g["e3"]), p(self.gskip["e3"]), self.g["e3"].numel(), s), "add")
        self._conv_back("e3", self.g["e3"], True, self.gpool["p2"])
        self._ck(L.mflbm_nn_avgpool2_back(p(self.gpool["p2"]), p(self.g["e2"]), n // 2, n // 2, n // 2, c2, s), "pool b")
        self._ck(L.mflbm_nn_add(p(self.g["e2"]), p(self.gskip["e2"]), self.g["e2"].numel(), s), "add")
        self._conv_back("e2", self.g["e2"], True, self.gpool["p1"])
        self._ck(L.mflbm_nn_avgpool2_back(p(self.gpool["p1"]), p(self.g["e1"]), n, n, n, c1, s), "pool b")
        self._ck(L.mflbm_nn_add(p(self.g["e1"]), p(self.gskip["e1"]), self.g["e1"].numel(), s), "add")
        self._conv_back("e1", self.g["e1"], False)

    def loss_grad(self, target, mask):
        """Masked MSE of the first target.shape[1] channels against target (n^3, C) fp32;
        sets self.g['y']; returns the loss as a device tensor."""
        nv = self.n ** 3
        L, p, s = self.lib, self._p, self.stream
        nc = int(target.shape[1])
        self.g["y"].zero_()
        cnt = max(1.0, float(mask.sum().item()) * nc)
        self._ck(L.mflbm_nn_mse(p(self.out), NOUT, p(target), p(mask), p(self.g["y"]), p(self.partial), nv, nc,
                                1.0 / cnt, s), "mse")
        return self.partial.sum() / cnt

    def adam(self, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
        self.step_count += 1
        L, p, s = self.lib, self._p, self.stream
        for k in self.W:
            self._ck(L.mflbm_nn_adam(p(self.W[k]), p(self.dW[k]), p(self.mW[k]), p(self.vW[k]), p(self.Wb[k]),
                                     self.W[k].numel(), lr, b1, b2, eps, self.step_count, s), "adam")
            self._ck(L.mflbm_nn_adam(p(self.B[k]), p(self.dB[k]), p(self.mB[k]), p(self.vB[k]), None,
                                     self.B[k].numel(), lr, b1, b2, eps, self.step_count, s), "adam")

    def check_err(self):
        if int(self.err.item()):
            raise _capi.MflbmError(_capi.MFLBM_ETIMEOUT, "a bounded wait in the tensor-core GEMM gave up")

    def weights(self):
        return {k: (self.W[k].cpu().numpy().copy(), self.B[k].cpu().numpy().copy()) for k in self.W}


# ---- features and targets --------------------------------------------------------------
def features(walls_global):
    """(n^3, 2) float32 input: solid mask and periodic signed distance / 8 (positive in
    the pore space), voxel order (z, y, x) as the network's channels-last layout."""
    from scipy import ndimage
    s = (walls_global != 0)
    n = s.shape
    pad = [(m // 2, m // 2) for m in n]
    sp = np.pad(s, pad, mode="wrap")
    d_in = ndimage.distance_transform_edt(~sp)       # distance to solid for pore voxels
    d_out = ndimage.distance_transform_edt(sp)       # distance to pore for solid voxels
    sl = tuple(slice(m // 2, m // 2 + k) for m, k in zip(n, n))
    sd = (d_in - d_out)[sl] / 8.0
    x = np.stack([s.astype(np.float32), sd.astype(np.float32)], axis=-1)
    return x.reshape(-1, 2)


def mean_density(walls_global):
    """Mean fluid density of the settled flow of a periodic sample started from the
    reference's equilibrium at rest.  The mass that takes part in the update is the fluid
    nodes' plus the bounce-back link slots'; it starts as N_fluid + sum over links of the
    BGK weight w_q and settles as rho (N_fluid + sum over links of the MRT rest weight W_q)."""
    fl = walls_global == 0
    ex, ey, ez = (np.array([0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0]),
                  np.array([0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1]),
                  np.array([0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1]))
    wb = [1 / 3] + [1 / 18] * 6 + [1 / 36] * 12
    wm = [4 / 21] + [13 / 126] * 6 + [1 / 63] * 12
    sb = sm = 0.0
    for q in range(1, 19):
        nfl = np.roll(fl, shift=(-ez[q], -ey[q], -ex[q]), axis=(0, 1, 2))
        c = float(np.count_nonzero(~fl & nfl))
        sb += c * wb[q]
        sm += c * wm[q]
    nf = float(fl.sum())
    return (nf + sb) / (nf + sm)


def target_from_macro(macro, nu, fz, rho_mean):
    """(n^3, 4) targets from Solver.macro() (halo-1 arrays) in voxel order: the scaled
    velocity and the scaled density deviation (zero in the solid)."""
    u = [macro[k][1:-1, 1:-1, 1:-1] for k in ("u", "v", "w")]
    rho = macro["rho"][1:-1, 1:-1, 1:-1]
    dr = np.where(rho != 0.0, rho - rho_mean, 0.0) * RHO_SCALE
    t = np.concatenate([np.stack(u, axis=-1) * (nu / fz / U_SCALE), dr[..., None]], axis=-1)
    return t.reshape(-1, NTARGET).astype(np.float32)


def velocity_from_output(out, n, nu, fz, walls_global):
    """Network output -> (u, v, w) arrays (nz, ny, nx), zero in the solid."""
    o = out[:, :3].reshape(n, n, n, 3) * (U_SCALE * fz / nu)
    fluid = (walls_global == 0)
    return [o[..., a] * fluid for a in range(3)]


def density_from_output(out, n, walls_global, rho_mean):
    """Network output -> density (nz, ny, nx): the sample's mean density plus the
    predicted deviation in the fluid, 1 in the solid."""
    fluid = (walls_global == 0)
    return np.where(fluid, rho_mean + out[:, 3].reshape(n, n, n) / RHO_SCALE, 1.0)


def equilibrium_state(u, v, w, nx, ny, nz):
    """f_q = w_q (1 + 3 e.u + 4.5 (e.u)^2 - 1.5 u^2) at rho = 1 on the halo-1 box, the
    reference's equilibrium (Initialization.F90:248-276) with the given velocity."""
    ex = np.array([0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0])
    ey = np.array([0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1])
    ez = np.array([0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1])
    wq = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)
    U = np.zeros((3, nz + 2, ny + 2, nx + 2))
    for a, comp in enumerate((u, v, w)):
        U[a, 1:-1, 1:-1, 1:-1] = comp
        # periodic ghosts
        U[a, 0], U[a, -1] = U[a, -2], U[a, 1]
        U[a, :, 0], U[a, :, -1] = U[a, :, -2], U[a, :, 1]
        U[a, :, :, 0], U[a, :, :, -1] = U[a, :, :, -2], U[a, :, :, 1]
    usq = (U ** 2).sum(axis=0)
    f = np.empty((19, nz + 2, ny + 2, nx + 2))
    for q in range(19):
        cu = ex[q] * U[0] + ey[q] * U[1] + ez[q] * U[2]
        f[q] = wq[q] * (1.0 + 3.0 * cu + 4.5 * cu * cu - 1.5 * usq)
    return f


# ---- study: data generation, training, A/B evaluation -----------------------------------
def _make_sample(args):
    n, por, seed = args
    from . import geometry
    wg = geometry.sphere_packing((n, n, n), float(por), mean_r=8.0, sd_r=2.0, seed=int(seed))
    return wg, features(wg)


def make_samples(n, count, seed, por_lo=0.15, por_hi=0.35, workers=0):
    """Seeded sphere packings (porosity uniform in [por_lo, por_hi]) and their features.
    workers > 1 uses a spawn-started process pool (call before any GPU work)."""
    rng = np.random.default_rng(seed)
    jobs = [(n, p, s) for p, s in zip(rng.uniform(por_lo, por_hi, count), rng.integers(0, 2**31 - 1, count))]
    if workers > 1:
        import multiprocessing as mp
        with mp.get_context("spawn").Pool(workers) as pool:
            return pool.map(_make_sample, jobs)
    return [_make_sample(j) for j in jobs]


def solve(wg, precision=1, tol=1e-7, init_u=None, init_rho=None, rest_base=False, max_steps=400000, nu=1.0 / 6.0,
          fz=1e-6, device=0):
    """Steady singlephase run of one periodic sample (fluid-list layout); returns the
    SteadyResult, the solver's macro fields and the set-up time.

    Without init_u and rest_base the run starts as the reference does (equilibrium at
    rest with the BGK weights).  Otherwise it starts from the rest state of the
    reference's MRT collision at density init_rho (default: the sample's mean_density),
    plus the equilibrium velocity terms of init_u = (u, v, w) (interior arrays, the steady
    velocity as compute_macro_vars reports it: F_z/2 is added to w in the fluid because
    the stored post-collision momentum leads it by half the body force), with the
    bounce-back link slots set consistently (mflbm_init_velocity)."""
    import time as _t
    from . import geometry
    from .permeability import run_to_steady
    from .solver import Solver, make_params
    n = wg.shape[0]
    p = make_params(multiphase=0, nx=n, ny=n, nz=n, iper=1, jper=1, kper=1, wall_x_min=0, wall_x_max=0,
                    wall_y_min=0, wall_y_max=0, mrt=1, la_nu1=nu, force_z=fz, precision=precision, device=device)
    walls, _, _ = geometry.set_walls(p, wg)
    with Solver(p) as sim:
        sim.set_geometry(walls)
        t0 = _t.perf_counter()
        if init_u is None and init_rho is None and not rest_base:
            sim.init_equilibrium()
        else:
            fluid = (wg == 0)
            rho = init_rho if init_rho is not None else np.where(fluid, mean_density(wg), 1.0)
            if init_u is None:
                init_u = (None, None, 0.5 * fz * fluid)
            else:
                init_u = (init_u[0], init_u[1], init_u[2] + 0.5 * fz * fluid)
            sim.init_velocity(*init_u, rho=rho, rest_base=True)
        setup = _t.perf_counter() - t0
        r = run_to_steady(sim, p, check_every=100, tol=tol, max_steps=max_steps)
        mac = sim.macro()
    return r, mac, setup


def train(net, xs, ys, ms, epochs=8, lr=1e-3, lr_end=2e-4, seed=0, log=None):
    """Adam over the samples (device tensors), one sample per step, cosine-free linear
    learning-rate decay; returns the per-epoch mean loss."""
    rng = np.random.default_rng(seed)
    total = epochs * len(xs)
    hist = []
    it = 0
    for ep in range(epochs):
        order = rng.permutation(len(xs))
        acc = []
        for i in order:
            frac = it / max(1, total - 1)
            net.forward(xs[i])
            acc.append(net.loss_grad(ys[i], ms[i]))
            net.backward()
            net.adam(lr=lr + (lr_end - lr) * frac)
            it += 1
        net.check_err()
        hist.append(float(net.torch.stack(acc).mean()))
        if log:
            log(f"epoch {ep}: loss {hist[-1]:.4e}")
    return hist
