"""Hand-written adjoint of the 18-DOF half-implicit step (Rollout18, lfdm_traj18_*): gradients of
the rollout loss with respect to per-step controls and to five parameters, checked against central
finite differences (h = 1e-6) of the GPU rollout and of the reference algorithm on the CPU (the
oracle restatement stepped with the same controls), through torch.autograd, over the
differentiation config's 2 s horizon (2,000 steps, a checkpoint every 100).

A central difference straddles a kink of the loss where the +h and -h rollouts take different
branches somewhere along the 2,000 steps (a tmxy_combined regime boundary, a sineStep band, a clamp,
a map segment, a gear shift); the adjoint differentiates the branch taken. Such rollouts are
detected, not assumed: lfdm_traj18_branch_signature hashes every discrete decision of every step,
and a step is usable for a direction only when its +h and -h rollouts have the same signature.

The difference itself has an error that no choice of one step removes for every direction: its
rounding error grows as 1/h, its truncation error and the chance of straddling a branch grow with h.
The loss of a 2,000-step rollout carries rounding noise of about 1e-14 of its value (the GPU and
the reference algorithm on the CPU, two FP64 implementations of the same steps, give losses up to
7e-15 apart), so a central difference with step h is uncertain by about 1e-14 |L| / h. Measured on
these rollouts, each direction's disagreement with the adjoint falls as 1/h until the step
straddles a branch. So each direction is differenced at a ladder of steps, and it must match the
adjoint to 1e-6 relative at one step that straddles no branch and whose rounding uncertainty is
below 1e-6 of the derivative. A direction whose derivative is too small against its loss for any
branch-free step to be that quiet is checked to the difference's own uncertainty instead
(|adjoint - difference| <= 1e-6 |difference| + 3 x 1e-14 |L| / h at its quietest branch-free step),
and counted. A direction that straddles a branch at every step cannot be checked by a central
difference at all; those are excluded, counted and capped at 5 %.
"""
import numpy as np
import pytest

import oracle_lib as O
from conftest import pkg_mod

pytestmark = pytest.mark.gpu

DT = 1e-3


def _setup(lfdm, n=64, T=2000, seed=3, ckpt=100, copies=1, chaotic=False):
    """n seeded SUV vehicles on clothoid reference paths with sine steering and constant throttle
    U[0.5, 0.9]; each vehicle appears `copies` times in a row (so that one rollout carries several
    perturbation directions per vehicle).

    Two choices keep the rollouts where a derivative exists, unless `chaotic` is set:
      * the wheel inertia is HMMWV-class (fleet.CALM_JW): with the configured SUV's 1.5 kg m^2 the
        explicit wheel-speed update chatters at dt = 1e-3 and the 2 s rollouts are rounding-chaotic
        (the reference algorithm built with fused multiply-adds moves the loss of 14 of 64 such
        vehicles by up to 3e-4), so a central difference at h = 1e-6 measures no derivative;
      * the crank starts 20 % above the speed the wheels drive it at, so the torque converter runs
        in forward flow: started exactly at lock-up (speed ratio 1) it flips between forward and
        reverse flow every few steps, and the reference's converter torque jumps by 2 (omega_in /
        cf)^2 at each flip (computePowertrainRHS, 18dof-gpu/dof18_gpu.cu:683-716)."""
    torch = pytest.importorskip("torch")
    fleet = pkg_mod("fleet")
    abi = pkg_mod("_abi")
    rng = np.random.default_rng(seed)
    cls, base = fleet.suv18()
    if not chaotic:
        base = base.copy()
        base[abi.P["jw"]] = fleet.CALM_JW
    params = fleet.jitter_params(base, n, rng)
    ref, v = fleet.clothoid_refs(n, T, DT, rng, speed=(8.0, 18.0))
    states = fleet.states_at_speed(cls, params, v)
    states[:, abi.S["crankomega"]] *= 1.2
    t = np.arange(T) * DT
    A = rng.uniform(-0.08, 0.08, n)
    f = rng.uniform(0.5, 2.0, n)
    ctl = np.zeros((T, 3, n))
    ctl[:, 0, :] = A[None, :] * np.sin(2 * np.pi * f[None, :] * t[:, None])
    ctl[:, 1, :] = rng.uniform(0.5, 0.9, n)[None, :]
    if copies > 1:
        params = np.repeat(params, copies, axis=0)
        states = np.repeat(states, copies, axis=0)
        ctl = np.repeat(ctl, copies, axis=2)
        ref = np.repeat(ref, copies, axis=2)
    N = n * copies
    sol = lfdm.d18SolverHalfImplicitGPU(N)
    sol.construct_class(cls, params)
    sol.set_states(states)
    sol.SetTimeStep(DT)
    dev = torch.device("cuda", 0)
    return {"sol": sol, "cls": cls, "params": params, "states": states, "ctl": ctl, "ref": ref,
            "ctl_t": torch.tensor(ctl, dtype=torch.float64, device=dev),
            "ref_t": torch.tensor(ref, dtype=torch.float64, device=dev), "T": T, "n": N,
            "ro": lfdm.Rollout18(sol, T, ckpt_every=ckpt)}


def _rel(a, b, floor):
    return np.abs(a - b) / np.maximum(np.abs(b), floor)


def _signature(S, ctl_t):
    torch = pytest.importorskip("torch")
    sig = torch.empty(S["n"], dtype=torch.int64, device=ctl_t.device)
    S["ro"].branch_signature(ctl_t.contiguous(), sig)
    return sig.cpu().numpy()


NOISE = 1e-14  # rounding noise of a rollout's loss, relative to the loss


def _check(name, ad, fds, loss, floor, cap=0.05):
    """fds: [(h, central difference, +h/-h signatures equal)] per step (h a scalar or one step per
    direction). Each direction's error is the smallest over its quiet branch-free steps (rounding
    uncertainty NOISE |loss| / h below 1e-6 of the difference); directions without one are checked
    to the uncertainty of their quietest branch-free step."""
    n = len(ad)
    best = np.full(n, np.inf)
    usable_any = np.zeros(n, bool)
    noisy_ok = np.zeros(n, bool)          # within uncertainty at the quietest branch-free step
    quietest = np.full(n, np.inf)         # the uncertainty of that step, relative to 1e-6 |fd|
    for h, fd, same in fds:
        e = _rel(ad, fd, floor)
        unc = NOISE * np.abs(loss) / np.abs(h)
        quiet = unc <= 1e-6 * np.maximum(np.abs(fd), floor)
        ok = same & quiet
        best = np.where(ok, np.minimum(best, e), best)
        usable_any |= same
        ratio = unc / (1e-6 * np.maximum(np.abs(fd), floor))
        take = same & (ratio < quietest)
        quietest = np.where(take, ratio, quietest)
        within = np.abs(ad - fd) <= 1e-6 * np.abs(fd) + 3 * unc
        noisy_ok = np.where(take, within, noisy_ok)
        hs = np.atleast_1d(h)
        print(f"{name}, h = {hs.min():.3g}{'' if np.ndim(h) == 0 else '..' + format(hs.max(), '.3g')}: "
              f"{int((~same).sum())}/{n} straddle a branch, {int((same & ~quiet).sum())} too noisy; the quiet: "
              f"median {np.median(e[ok]) if ok.any() else 0:.2e}, max {e[ok].max() if ok.any() else 0:.2e}")
    checked = np.isfinite(best)
    noisy = usable_any & ~checked
    ex = ~usable_any
    kept = best[checked]
    print(f"{name}: {int(checked.sum())}/{n} checked to 1e-6 (median {np.median(kept) if kept.size else 0:.2e}, max "
          f"{kept.max() if kept.size else 0:.2e}); {int(noisy.sum())} too small a derivative for a quiet step, "
          f"checked to the difference's uncertainty; {int(ex.sum())} straddle a branch at every step (excluded)")
    assert ex.mean() <= cap, (name, int(ex.sum()))
    assert (kept <= 1e-6).all(), (name, float(kept.max()), int(np.argmax(np.where(checked, best, 0))))
    assert noisy_ok[noisy].all(), (name, np.nonzero(noisy & ~noisy_ok)[0].tolist())


def test_control_gradient_matches_finite_differences(built_lib):
    """64 vehicles x 16 random directions of the 2,000 x 3 control sequence (steering and throttle),
    each vehicle's 16 directions carried by 16 copies of it in one rollout."""
    torch = pytest.importorskip("torch")
    nd = 16
    S = _setup(built_lib, n=64, copies=nd)
    ro, n, T = S["ro"], S["n"], S["T"]
    c = S["ctl_t"].clone().requires_grad_(True)
    loss = ro.loss(c, S["ref_t"])
    loss.sum().backward()
    g = c.grad.detach().cpu().numpy()
    rng = np.random.default_rng(9)
    d = np.zeros((T, 3, n))
    d[:, 0, :] = rng.standard_normal((T, n)) * 0.05
    d[:, 1, :] = rng.standard_normal((T, n)) * 0.05
    dt_ = torch.tensor(d, dtype=torch.float64, device=c.device)
    fds = []
    for h in (1e-6, 3e-6, 1e-5, 3e-5, 1e-4):
        lp = torch.empty(n, dtype=torch.float64, device=c.device)
        lm = torch.empty_like(lp)
        cp = (S["ctl_t"] + h * dt_).contiguous()
        cm = (S["ctl_t"] - h * dt_).contiguous()
        ro.forward_raw(cp, S["ref_t"], lp)
        ro.forward_raw(cm, S["ref_t"], lm)
        fds.append((h, (lp - lm).cpu().numpy() / (2 * h), _signature(S, cp) == _signature(S, cm)))
    ad = np.einsum("tcn,tcn->n", g, d)
    L0 = loss.detach().cpu().numpy()
    _check("control gradient", ad, fds, L0, 1e-8 * np.abs(L0).max())


def test_parameter_gradients_match_finite_differences(built_lib):
    """64 vehicles x the 5 parameters (mass, Jz, CG-to-front distance, tire friction scale, tire
    vertical stiffness), central differences with steps of 1e-6 to 3e-4 of each parameter's scale."""
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
    L0 = loss.detach().cpu().numpy()
    for j, name in enumerate(built_lib.ROLLOUT_PARAMS):
        fds = []
        for rel in (1e-6, 3e-6, 1e-5, 3e-5, 1e-4, 3e-4):
            h = rel * scales[j]
            out, sigs = [], []
            for sgn in (1.0, -1.0):
                th = torch.zeros(5, n, dtype=torch.float64, device="cuda")
                th[j] = torch.tensor(sgn * h, dtype=torch.float64, device="cuda")
                with torch.no_grad():
                    out.append(ro.loss(S["ctl_t"], S["ref_t"], th).cpu().numpy())
                sigs.append(_signature(S, S["ctl_t"]))  # at the parameters the loss call applied
            fds.append((h, (out[0] - out[1]) / (2 * h), sigs[0] == sigs[1]))
        _check(name, g[j], fds, L0, 1e-8 * np.abs(fds[0][1]).max())


def _oracle_loss(S, ctl, idx, fma=False):
    """The rollout loss of vehicles idx with the reference algorithm on the CPU (the oracle stepped
    one step at a time with the step's controls; fma: its build with fused multiply-adds)."""
    st = S["states"][idx].copy()
    cls = S["cls"]
    P = S["params"][idx]
    L = np.zeros(len(idx))
    Sx = pkg_mod("_abi").S
    for k in range(S["T"]):
        u = ctl[k][:, idx].T.copy()
        st, _ = O.run18([cls], np.zeros(len(idx), np.int32), P, st, ctl=u, t0=k * DT, dt=DT, ksim=DT, schedule=2,
                        fma=fma)
        xr, yr, pr = S["ref"][k][:, idx]
        el = -(st[:, Sx["x"]] - xr) * np.sin(pr) + (st[:, Sx["y"]] - yr) * np.cos(pr)
        eh = st[:, Sx["psi"]] - pr
        L += el * el + eh * eh + 1e-3 * (u * u).sum(axis=1)
    return L


def test_gradient_against_reference_algorithm_on_cpu(built_lib):
    """64 vehicles over the 2,000 steps: the GPU loss against the loss of the reference algorithm
    (oracle), and the adjoint's directional derivative against a central difference of the
    reference algorithm itself where the GPU's +h and -h rollouts take the same branches."""
    torch = pytest.importorskip("torch")
    S = _setup(built_lib, n=64, seed=5)
    ro, n = S["ro"], S["n"]
    c = S["ctl_t"].clone().requires_grad_(True)
    loss = ro.loss(c, S["ref_t"])
    loss.sum().backward()
    g = c.grad.detach().cpu().numpy()
    idx = np.arange(n)
    lo = _oracle_loss(S, S["ctl"], idx)
    # the reference algorithm's own rounding sensitivity: its build with fused multiply-adds (a gear
    # shift that a rounding difference moves by one step changes the loss by more than 1e-9)
    env = _rel(_oracle_loss(S, S["ctl"], idx, fma=True), lo, 0.0)
    el = _rel(loss.detach().cpu().numpy(), lo, 0.0)
    print(f"GPU loss vs oracle: max rel {el.max():.2e} (oracle FMA build {env.max():.2e}); "
          f"{int((el > 1e-9).sum())} vehicles beyond 1e-9")
    assert (el <= np.maximum(1e-9, 100 * env)).all(), (float(el.max()), int(el.argmax()))
    rng = np.random.default_rng(2)
    d = np.zeros_like(S["ctl"])
    d[:, 0, :] = rng.standard_normal(d[:, 0, :].shape) * 0.05
    dt_ = torch.tensor(d, dtype=torch.float64, device=c.device)
    fds = []
    for h in (1e-6, 1e-5):
        fd = (_oracle_loss(S, S["ctl"] + h * d, idx) - _oracle_loss(S, S["ctl"] - h * d, idx)) / (2 * h)
        same = _signature(S, (S["ctl_t"] + h * dt_).contiguous()) == _signature(S, (S["ctl_t"] - h * dt_).contiguous())
        fds.append((h, fd, same))
    ad = np.einsum("tcn,tcn->n", g, d)
    _check("adjoint vs oracle central difference", ad, fds, lo, 1e-8 * np.abs(lo).max())


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
    """The differentiation config: the configured SUV (1.5 kg m^2 wheels), 65,536 vehicles x 2,000
    steps, a checkpoint every 100 steps. Target: the gradient costs at most 3x the forward rollout."""
    torch = pytest.importorskip("torch")
    S = _setup(built_lib, n=65536, T=2000, seed=7, chaotic=True)
    ro = S["ro"]
    c = S["ctl_t"].clone().requires_grad_(True)
    for _ in range(2):  # the first pass allocates the checkpoints and the tape
        c.grad = None
        loss = ro.loss(c, S["ref_t"])
        loss.sum().backward()
    fwd, bwd = ro.last_ms()
    print(f"forward {fwd:.2f} ms, backward {bwd:.2f} ms, ratio {bwd / fwd:.2f}")
    assert bwd / fwd < 3.0
