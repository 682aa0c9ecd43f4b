"""Hand-written adjoint of the 18-DOF half-implicit step (Rollout18, lfdm_traj18_*): gradients of
the rollout loss with respect to per-step controls and to five parameters, checked against central
finite differences (h = 1e-6) of the GPU rollout and of the reference algorithm on the CPU (the
oracle restatement stepped with the same controls), through torch.autograd.

Tolerance: median relative error of directional derivatives <= 1e-6 and >= 90% of vehicles
<= 1e-5. The rest are vehicles where the +-h perturbation crosses a branch of the tire model or the
drivetrain (regime boundary of tmxy_combined, sineStep band, clamp, gear shift), which a finite
difference straddles and the adjoint, differentiating the branch taken, does not.
"""
import numpy as np
import pytest

import oracle_lib as O
from conftest import pkg_mod

pytestmark = pytest.mark.gpu

DT = 1e-3


def _setup(lfdm, n=64, T=300, seed=3, ckpt=100):
    torch = pytest.importorskip("torch")
    fleet = pkg_mod("fleet")
    rng = np.random.default_rng(seed)
    cls, base = fleet.suv18()
    params = fleet.jitter_params(base, n, rng)
    ref, v = fleet.clothoid_refs(n, T, DT, rng, speed=(8.0, 18.0))
    states = fleet.states_at_speed(cls, params, v)
    sol = lfdm.d18SolverHalfImplicitGPU(n)
    sol.construct_class(cls, params)
    sol.set_states(states)
    sol.SetTimeStep(DT)
    t = np.arange(T) * DT
    A = rng.uniform(-0.08, 0.08, n)
    f = rng.uniform(0.5, 2.0, n)
    ctl = np.zeros((T, 3, n))
    ctl[:, 0, :] = A[None, :] * np.sin(2 * np.pi * f[None, :] * t[:, None])
    ctl[:, 1, :] = rng.uniform(0.2, 0.5, n)[None, :]
    dev = torch.device("cuda", 0)
    return {"sol": sol, "cls": cls, "params": params, "states": states, "ctl": ctl, "ref": ref,
            "ctl_t": torch.tensor(ctl, dtype=torch.float64, device=dev),
            "ref_t": torch.tensor(ref, dtype=torch.float64, device=dev), "T": T, "n": n,
            "ro": lfdm.Rollout18(sol, T, ckpt_every=ckpt)}


def _rel(a, b, floor):
    return np.abs(a - b) / np.maximum(np.abs(b), floor)


def test_control_gradient_matches_finite_differences(built_lib):
    torch = pytest.importorskip("torch")
    S = _setup(built_lib)
    ro, n, T = S["ro"], S["n"], S["T"]
    c = S["ctl_t"].clone().requires_grad_(True)
    loss = ro.loss(c, S["ref_t"])
    loss.sum().backward()
    g = c.grad.detach().cpu().numpy()
    rng = np.random.default_rng(9)
    d = np.zeros((T, 3, n))
    d[:, 0, :] = rng.standard_normal((T, n)) * 0.05
    d[:, 1, :] = rng.standard_normal((T, n)) * 0.05
    h = 1e-6
    dt_ = torch.tensor(d, dtype=torch.float64, device=c.device)
    lp = torch.empty(n, dtype=torch.float64, device=c.device)
    lm = torch.empty_like(lp)
    ro.forward_raw((S["ctl_t"] + h * dt_).contiguous(), S["ref_t"], lp)
    ro.forward_raw((S["ctl_t"] - h * dt_).contiguous(), S["ref_t"], lm)
    fd = (lp - lm).cpu().numpy() / (2 * h)
    ad = np.einsum("tcn,tcn->n", g, d)
    e = _rel(ad, fd, 1e-8 * np.abs(loss.detach().cpu().numpy()).max())
    print(f"control gradient: median rel err {np.median(e):.2e}, p90 {np.quantile(e, 0.9):.2e}, max {e.max():.2e}")
    assert np.median(e) <= 1e-6
    assert (e <= 1e-5).mean() >= 0.9


def test_parameter_gradients_match_finite_differences(built_lib):
    torch = pytest.importorskip("torch")
    S = _setup(built_lib, seed=4)
    ro, n = S["ro"], S["n"]
    theta = torch.zeros(5, n, dtype=torch.float64, device="cuda", requires_grad=True)
    loss = ro.loss(S["ctl_t"], S["ref_t"], theta)
    loss.sum().backward()
    g = theta.grad.detach().cpu().numpy()
    base = S["params"]
    P = pkg_mod("_abi").P
    scales = [base[:, P["m"]], base[:, P["jz"]], base[:, P["a"]], np.ones(n), base[:, P["kt"]]]
    for j, name in enumerate(built_lib.ROLLOUT_PARAMS):
        h = 1e-6 * scales[j]
        out = []
        for sgn in (1.0, -1.0):
            th = torch.zeros(5, n, dtype=torch.float64, device="cuda")
            th[j] = torch.tensor(sgn * h, dtype=torch.float64, device="cuda")
            with torch.no_grad():
                out.append(ro.loss(S["ctl_t"], S["ref_t"], th).cpu().numpy())
        fd = (out[0] - out[1]) / (2 * h)
        e = _rel(g[j], fd, 1e-8 * np.abs(fd).max())
        print(f"{name}: median rel err {np.median(e):.2e}, max {e.max():.2e}")
        assert np.median(e) <= 1e-6, name
        assert (e <= 1e-5).mean() >= 0.9, name


def _oracle_loss(S, ctl, idx):
    """The rollout loss of vehicles idx with the reference algorithm on the CPU (the oracle stepped
    one step at a time with the step's controls)."""
    st = S["states"][idx].copy()
    cls = S["cls"]
    P = S["params"][idx]
    L = np.zeros(len(idx))
    for k in range(S["T"]):
        u = ctl[k][:, idx].T.copy()
        st, _ = O.run18([cls], np.zeros(len(idx), np.int32), P, st, ctl=u, t0=k * DT, dt=DT, ksim=DT, schedule=2)
        Sx = pkg_mod("_abi").S
        xr, yr, pr = S["ref"][k][:, idx]
        el = -(st[:, Sx["x"]] - xr) * np.sin(pr) + (st[:, Sx["y"]] - yr) * np.cos(pr)
        eh = st[:, Sx["psi"]] - pr
        L += el * el + eh * eh + 1e-3 * (u * u).sum(axis=1)
    return L


def test_gradient_against_reference_algorithm_on_cpu(built_lib):
    """The adjoint's directional derivative against a central difference of the reference
    algorithm itself (oracle), and the GPU loss against the oracle's loss."""
    torch = pytest.importorskip("torch")
    S = _setup(built_lib, n=16, T=200, seed=5)
    ro = S["ro"]
    c = S["ctl_t"].clone().requires_grad_(True)
    loss = ro.loss(c, S["ref_t"])
    loss.sum().backward()
    g = c.grad.detach().cpu().numpy()
    idx = np.arange(4)
    lo = _oracle_loss(S, S["ctl"], idx)
    assert np.allclose(loss.detach().cpu().numpy()[idx], lo, rtol=1e-10, atol=0)
    rng = np.random.default_rng(2)
    d = np.zeros_like(S["ctl"])
    d[:, 0, :] = rng.standard_normal(d[:, 0, :].shape) * 0.05
    h = 1e-6
    fd = (_oracle_loss(S, S["ctl"] + h * d, idx) - _oracle_loss(S, S["ctl"] - h * d, idx)) / (2 * h)
    ad = np.einsum("tcn,tcn->n", g[:, :, idx], d[:, :, idx])
    e = _rel(ad, fd, 1e-8 * np.abs(lo).max())
    print("adjoint vs oracle central difference:", e)
    assert np.median(e) <= 1e-6


def test_checkpoint_interval_does_not_change_gradients(built_lib):
    torch = pytest.importorskip("torch")
    grads = []
    for ck in (100, 37, 300):
        S = _setup(built_lib, n=32, T=300, seed=6, ckpt=ck)
        c = S["ctl_t"].clone().requires_grad_(True)
        S["ro"].loss(c, S["ref_t"]).sum().backward()
        grads.append(c.grad.detach().cpu().numpy())
        S["sol"].close()
    assert np.array_equal(grads[0], grads[1]) and np.array_equal(grads[0], grads[2])


def test_backward_forward_time_ratio(built_lib):
    torch = pytest.importorskip("torch")
    S = _setup(built_lib, n=8192, T=500, seed=7)
    ro = S["ro"]
    c = S["ctl_t"].clone().requires_grad_(True)
    loss = ro.loss(c, S["ref_t"])
    loss.sum().backward()
    fwd, bwd = ro.last_ms()
    print(f"forward {fwd:.2f} ms, backward {bwd:.2f} ms, ratio {bwd / fwd:.2f}")
    assert bwd / fwd < 6.0
