"""Warm-start network on the GPU (tcgen05 GEMMs + the project's kernels) against its CPU
restatement, which rounds to bf16 at the same points, so only FP32 accumulation order
differs: forward output and every weight/bias gradient within 2e-2 relative (Frobenius
norm).  Training on one sample must reduce its loss."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from mflbm import warmstart
from nn_oracle import OracleNet

pytestmark = pytest.mark.gpu

C4 = (16, 16, 16, 32)


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def _data(n, seed):
    rng = np.random.default_rng(seed)
    x = rng.normal(size=(n ** 3, 2)).astype(np.float32)
    t = rng.normal(size=(n ** 3, 3)).astype(np.float32)
    m = (rng.random(n ** 3) > 0.3).astype(np.float32)
    return x, t, m


@pytest.mark.parametrize("n", [8, 16])
def test_forward_and_gradients_match_oracle(n):
    w = warmstart.init_weights(C4, seed=3)
    # non-zero output channels and biases so that every path carries gradient
    rng = np.random.default_rng(4)
    for k in w:
        w[k][1][:] = rng.normal(0, 0.05, size=w[k][1].shape)
    x, t, m = _data(n, 5)
    net = warmstart.Net(n, C4, weights=w)
    dev = net.dev
    net.forward(torch.from_numpy(x).to(dev).to(torch.bfloat16))
    loss = net.loss_grad(torch.from_numpy(t).to(dev), torch.from_numpy(m).to(dev))
    net.backward()
    torch.cuda.synchronize()
    net.check_err()
    ref = OracleNet(n, C4, w)
    out_ref = ref.forward(x.astype(np.float64))
    loss_ref, gy = ref.loss_grad(t.astype(np.float64), m.astype(np.float64))
    dW, dB = ref.backward(gy)
    out = net.out.cpu().numpy()
    print(f"n={n}: out rel {_rel(out, out_ref):.2e}  loss {float(loss):.6e} vs {loss_ref:.6e}")
    assert _rel(out, out_ref) <= 2e-2
    assert abs(float(loss) - loss_ref) <= 2e-2 * abs(loss_ref)
    for k in dW:
        ew, eb = _rel(net.dW[k].cpu().numpy(), dW[k]), _rel(net.dB[k].cpu().numpy(), dB[k])
        print(f"  {k}: dW rel {ew:.2e}  dB rel {eb:.2e}")
        assert ew <= 2e-2, k
        assert eb <= 2e-2, k


def test_training_follows_oracle_and_fits_a_constant_field():
    """GPU training (forward, backward, Adam) follows the oracle's FP64 Adam trajectory, and
    a constant target field is fitted (the loss falls at least fivefold in 120 steps;
    the oracle's own trajectory falls 9.6x)."""
    from nn_oracle import OracleAdam
    n = 16
    x, t, m = _data(n, 9)
    w0 = warmstart.init_weights(C4, seed=1)
    net = warmstart.Net(n, C4, weights=w0)
    dev = net.dev
    xb = torch.from_numpy(x).to(dev).to(torch.bfloat16)
    tt, mm = torch.from_numpy(0.3 * t).to(dev), torch.from_numpy(m).to(dev)
    opt = OracleAdam(w0, lr=3e-3)
    for it in range(12):
        net.forward(xb)
        lg = float(net.loss_grad(tt, mm))
        net.backward()
        net.adam(lr=3e-3)
        ref = OracleNet(n, C4, opt.weights())
        ref.forward(x.astype(np.float64))
        lr_, gy = ref.loss_grad(0.3 * t.astype(np.float64), m.astype(np.float64))
        opt.step(*ref.backward(gy))
        assert abs(lg - lr_) <= 1e-2 * lr_, (it, lg, lr_)
    net.check_err()
    # constant target: reachable through the biases
    const = np.broadcast_to(np.array([[0.3, -0.2, 0.1]], dtype=np.float32), (n ** 3, 3)).copy()
    net2 = warmstart.Net(n, C4, seed=2)
    tc = torch.from_numpy(const).to(dev)
    losses = []
    for it in range(120):
        net2.forward(xb)
        losses.append(float(net2.loss_grad(tc, mm)))
        net2.backward()
        net2.adam(lr=3e-3)
    net2.check_err()
    print("constant target loss", losses[0], "->", losses[-1])
    assert losses[-1] < 0.2 * losses[0]


@pytest.mark.parametrize("precision", [0, 1])
def test_restart_from_converged_fields(precision):
    """Runs restarted from the settled velocity (and density) of a previous run need fewer
    steps than the reference's start and reproduce k; the mean density of the settled flow
    matches the mass balance of mean_density."""
    from mflbm import geometry
    wg = geometry.sphere_packing((48, 48, 48), 0.3, mean_r=8.0, sd_r=2.0, seed=5)
    r0, mac, _ = warmstart.solve(wg, precision=precision, tol=1e-7)
    fl = wg == 0
    rho = mac["rho"][1:-1, 1:-1, 1:-1]
    assert abs(rho[fl].mean() - warmstart.mean_density(wg)) <= 2e-6
    u = [mac[k][1:-1, 1:-1, 1:-1] for k in ("u", "v", "w")]
    rb, _, _ = warmstart.solve(wg, precision=precision, tol=1e-7, rest_base=True)
    r1, _, _ = warmstart.solve(wg, precision=precision, tol=1e-7, init_u=u)
    r2, _, _ = warmstart.solve(wg, precision=precision, tol=1e-7, init_u=u, init_rho=np.where(fl, rho, 1.0))
    print(f"precision {precision}: reference start {r0.steps}, MRT rest {rb.steps}, settled u {r1.steps}, "
          f"settled u and rho {r2.steps} steps; k {r0.k:.8e} / {r2.k:.8e}")
    for r in (rb, r1, r2):
        assert r.converged
        assert abs(r.k - r0.k) / r0.k <= 1e-3
    assert r1.steps < r0.steps
    assert r2.steps < rb.steps


def test_init_velocity_matches_equilibrium_formula():
    from mflbm import Solver, geometry
    from mflbm.solver import make_params
    n = 20
    wg = geometry.sphere_packing((n, n, n), 0.35, mean_r=4.0, sd_r=1.0, seed=2)
    rng = np.random.default_rng(3)
    u = [1e-3 * rng.normal(size=(n, n, n)) for _ in range(3)]
    ex = np.array([0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0])
    ey = np.array([0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1])
    ez = np.array([0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1])
    wq = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)
    wr = np.array([4 / 21] + [13 / 126] * 6 + [1 / 63] * 12)
    for layout in (1, 2):
        p = make_params(multiphase=0, nx=n, ny=n, nz=n, iper=1, jper=1, kper=1, wall_x_min=0, wall_x_max=0,
                        wall_y_min=0, wall_y_max=0, mrt=1, la_nu1=1 / 6, force_z=1e-6, layout=layout)
        walls, _, _ = geometry.set_walls(p, wg)
        with Solver(p) as sim:
            sim.set_geometry(walls)
            sim.init_velocity(*u, rest_base=True)
            f = sim.download_state()["f"][:, 1:-1, 1:-1, 1:-1]
        fl = wg == 0
        cu = ex[:, None] * u[0][fl] + ey[:, None] * u[1][fl] + ez[:, None] * u[2][fl]
        usq = u[0][fl] ** 2 + u[1][fl] ** 2 + u[2][fl] ** 2
        ref = wr[:, None] + wq[:, None] * (3 * cu + 4.5 * cu * cu - 1.5 * usq)
        assert np.abs(f[:, fl] - ref).max() <= 1e-16, layout
