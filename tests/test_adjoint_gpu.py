"""The adjoint of T iterations (nb_sim_adjoint_forward/backward), wrapped in a
torch.autograd.Function, against FP64 torch autograd of the same map and FP64
central finite differences (N = 512, T = 32)."""
from __future__ import annotations

import numpy as np
import pytest

import nbody_gb300 as nb
from helpers import disk_case, params

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

N, T, EVERY = 512, 32, 8
G, DT, DAMP = 1.0, 1e-3, 0.999
EPS = float(np.float32(1e-3))


def step64(x, v, m):
    """One iteration of the reference's update in FP64 torch (src/simulator.cu:197-228)."""
    r = x[None, :, :] - x[:, None, :]                # r_ij = x_j - x_i
    d2 = (r * r).sum(-1) + EPS
    s = d2.pow(-1.5) * m[None, :]
    s = s * (1.0 - torch.eye(x.shape[0], dtype=x.dtype))
    a = G * (r * s[..., None]).sum(1)
    v = DAMP * v + DT * a
    return x + DT * v, v


def run64(x, v, m, steps):
    for _ in range(steps):
        x, v = step64(x, v, m)
    return x, v


class NBodyT(torch.autograd.Function):
    """x_T = F(x_0, v_0) through the library; backward through its adjoint."""

    @staticmethod
    def forward(ctx, x0, v0, sim, steps, every):
        sim.set_state([x0[:, 0], x0[:, 1], x0[:, 2]], [v0[:, 0], v0[:, 1], v0[:, 2]])
        sim.adjoint_forward(steps, every)
        st = sim.get_state()
        ctx.sim = sim
        return torch.from_numpy(np.stack(st[:3], 1).copy())

    @staticmethod
    def backward(ctx, gx):
        gx0, gv0 = ctx.sim.adjoint_backward(gx.contiguous().numpy().reshape(-1))
        return torch.from_numpy(gx0.copy()), torch.from_numpy(gv0.copy()), None, None, None


@pytest.fixture(scope="module")
def case():
    pos, vel, m = disk_case(N, seed=4)
    x0 = np.stack(pos, 1).astype(np.float32)
    v0 = np.stack(vel, 1).astype(np.float32)
    rng = np.random.default_rng(5)
    xt0 = x0 + rng.normal(0, 1e-3, x0.shape).astype(np.float32)
    m64 = torch.from_numpy(m.astype(np.float64))
    target, _ = run64(torch.from_numpy(xt0.astype(np.float64)),
                      torch.from_numpy(v0.astype(np.float64)), m64, T)
    return x0, v0, m, target


def loss_fn(xT, target):
    return ((xT - target) ** 2).sum(-1).mean()


def reference_grads(x0, v0, m, target):
    x = torch.from_numpy(x0.astype(np.float64)).requires_grad_(True)
    v = torch.from_numpy(v0.astype(np.float64)).requires_grad_(True)
    xT, _ = run64(x, v, torch.from_numpy(m.astype(np.float64)), T)
    loss_fn(xT, target).backward()
    return x.grad.numpy(), v.grad.numpy()


def test_adjoint_matches_fp64_autograd(case):
    x0, v0, m, target = case
    with nb.Simulation(params(N, G=G, dt=DT, damping=DAMP), [x0[:, 0], x0[:, 1], x0[:, 2]],
                       [v0[:, 0], v0[:, 1], v0[:, 2]], m) as sim:
        x = torch.from_numpy(x0.copy()).requires_grad_(True)
        v = torch.from_numpy(v0.copy()).requires_grad_(True)
        xT = NBodyT.apply(x, v, sim, T, EVERY)
        loss = loss_fn(xT.double(), target)
        loss.backward()
        gx, gv = x.grad.numpy(), v.grad.numpy()
    rx, rv = reference_grads(x0, v0, m, target)
    for g, r in ((gx, rx), (gv, rv)):
        rel = np.linalg.norm(g - r) / np.linalg.norm(r)
        assert rel <= 1e-4, rel


def test_fp64_autograd_matches_central_differences(case):
    # Validates the reference gradient itself: FP64 central differences along
    # random directions of (x0, v0).
    x0, v0, m, target = case
    rx, rv = reference_grads(x0, v0, m, target)
    m64 = torch.from_numpy(m.astype(np.float64))
    rng = np.random.default_rng(8)
    for _ in range(3):
        ux = rng.normal(size=x0.shape)
        uv = rng.normal(size=v0.shape)
        h = 1e-6

        def L(sign):
            x = torch.from_numpy(x0.astype(np.float64) + sign * h * ux)
            v = torch.from_numpy(v0.astype(np.float64) + sign * h * uv)
            xT, _ = run64(x, v, m64, T)
            return float(loss_fn(xT, target))

        fd = (L(1) - L(-1)) / (2 * h)
        an = float(np.sum(rx * ux) + np.sum(rv * uv))
        assert abs(fd - an) <= 1e-6 * abs(an), (fd, an)


def test_adjoint_checkpoint_interval_does_not_change_result(case):
    x0, v0, m, target = case
    gxT = np.random.default_rng(3).normal(size=(N, 3)).astype(np.float32)
    outs = []
    for every in (1, 5, 32):
        with nb.Simulation(params(N, G=G, dt=DT, damping=DAMP), [x0[:, 0], x0[:, 1], x0[:, 2]],
                           [v0[:, 0], v0[:, 1], v0[:, 2]], m) as sim:
            sim.adjoint_forward(T, every)
            outs.append(sim.adjoint_backward(gxT.reshape(-1)))
    for gx, gv in outs[1:]:
        assert np.array_equal(gx, outs[0][0]) and np.array_equal(gv, outs[0][1])


def test_adjoint_per_pair_masses():
    n, steps = 300, 6
    pos, vel, _ = disk_case(n, seed=13)
    m = (np.random.default_rng(2).uniform(0.5, 1.5, n) / n).astype(np.float32)
    x0 = np.stack(pos, 1)
    v0 = np.stack(vel, 1)
    gxT = np.random.default_rng(4).normal(size=(n, 3))
    gvT = np.random.default_rng(5).normal(size=(n, 3))
    with nb.Simulation(params(n, G=G, dt=DT, damping=DAMP), pos, vel, m) as sim:
        sim.adjoint_forward(steps, 4)
        gx, gv = sim.adjoint_backward(gxT.astype(np.float32).reshape(-1),
                                      gvT.astype(np.float32).reshape(-1))
    x = torch.from_numpy(x0.astype(np.float64)).requires_grad_(True)
    v = torch.from_numpy(v0.astype(np.float64)).requires_grad_(True)
    xT, vT = run64(x, v, torch.from_numpy(m.astype(np.float64)), steps)
    ((xT * torch.from_numpy(gxT)).sum() + (vT * torch.from_numpy(gvT)).sum()).backward()
    for g, r in ((gx, x.grad.numpy()), (gv, v.grad.numpy())):
        assert np.linalg.norm(g - r) / np.linalg.norm(r) <= 1e-4


def test_adjoint_device_entry_point_matches_host_entry_point():
    # nb_sim_adjoint_backward_device: the same sweep on device arrays, stream-ordered.
    n, steps = 1000, 12
    pos, vel, _ = disk_case(n, seed=17)
    m = (np.random.default_rng(6).uniform(0.5, 1.5, n) / n).astype(np.float32)
    rng = np.random.default_rng(7)
    gxT = rng.normal(size=3 * n).astype(np.float32)
    gvT = rng.normal(size=3 * n).astype(np.float32)
    with nb.Simulation(params(n, G=G, dt=DT, damping=DAMP), pos, vel, m) as sim:
        sim.adjoint_forward(steps, 5)
        host = sim.adjoint_backward(gxT, gvT)
        host_nov = sim.adjoint_backward(gxT)
        dev_in = [torch.from_numpy(a).cuda() for a in (gxT, gvT)]
        out = [torch.full((3 * n,), float("nan"), device="cuda") for _ in range(2)]
        torch.cuda.synchronize()
        sim.adjoint_backward_device(dev_in[0].data_ptr(), dev_in[1].data_ptr(),
                                    out[0].data_ptr(), out[1].data_ptr())
        sim.synchronize()
        dev = [o.cpu().numpy().reshape(n, 3) for o in out]
        sim.adjoint_backward_device(dev_in[0].data_ptr(), None, out[0].data_ptr(),
                                    out[1].data_ptr())
        sim.synchronize()
        dev_nov = [o.cpu().numpy().reshape(n, 3) for o in out]
    for a, b in zip(host + host_nov, dev + dev_nov):
        assert np.array_equal(a, b)
