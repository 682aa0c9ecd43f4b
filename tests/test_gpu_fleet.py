"""Mixed-DOF fleet (lfdm_fleet_*): one persistent launch over 18- and 24-DOF vehicles of four mass
classes with their own end times must give every vehicle exactly what the per-model, per-class,
per-horizon solver runs give it (the reference's way: one solver per model and end time, with
m_tend = the vehicle's end time), bit for bit, for every launch configuration."""
import numpy as np
import pytest

from conftest import pkg_mod

pytestmark = pytest.mark.gpu

KSIM = 0.5
DTOUT = 0.1


def _small_fleet(n=600, seed=11):
    fleet = pkg_mod("fleet")
    return fleet.mixed_fleet(n, seed=seed, horizon_range=(0.2, 2.3), n_tables=64)


def _make(lfdm, mf, launch=None):
    f = lfdm.Fleet(dt=1e-3, kernel_sim_time=KSIM, output_dt=DTOUT)
    base = f.add_rows(mf["rows"])
    for g in mf["groups"]:
        f.add(g["model"], g["cls"], g["params"], g["states"], g["horizons"], None, base + g["row_off"], g["row_len"])
    if launch:
        f.set_launch(*launch)
    return f


def _windows(h):
    """Windows the reference's Solve runs for end time h (window starts accumulated in FP64)."""
    t, w = 0.0, 0
    while t < h:
        t = t + KSIM
        w += 1
    return w


def _per_group(lfdm, mf, precision=0):
    """Each (model, class, window count) group through the regular solver: states and responses in
    the fleet's add order per model."""
    out = {18: [], 24: []}
    resp = {18: [], 24: []}
    for g in mf["groups"]:
        m = g["model"]
        cls_ = lfdm.d18SolverHalfImplicitGPU if m == 18 else lfdm.d24SolverHalfImplicitGPU
        nch = lfdm.RESP18 if m == 18 else lfdm.RESP24
        wins = np.array([_windows(h) for h in g["horizons"]])
        st = g["states"].copy()
        rs = [None] * len(wins)
        for w in np.unique(wins):
            idx = np.nonzero(wins == w)[0]
            sol = cls_(len(idx))
            sol.construct_class(g["cls"], g["params"][idx])
            sol.set_precision(precision)
            tabs = np.stack([mf["rows"][g["row_off"][i]: g["row_off"][i] + g["row_len"][i]] for i in idx])
            sol.set_driver_tables(tabs)
            sol.set_states(g["states"][idx])
            sol.SetKernelSimTime(KSIM)
            sol.SetEndTime(w * KSIM - 1e-9 if w > 0 else 0.0)  # any end time in ((w-1)*ksim, w*ksim] runs w windows
            buf = np.zeros((int(w * KSIM / DTOUT + 0.5) + 8, nch, len(idx)))
            sol.set_response_buffer(buf, 1.0 / DTOUT)
            if w > 0:
                sol.Solve()
            st[idx] = sol.get_states()
            n_s = sol.response_samples() if w > 0 else 0
            for j, i in enumerate(idx):
                rs[i] = buf[:n_s, :, j]
            sol.close()
        out[m].append(st)
        resp[m].extend(rs)
    return {m: np.concatenate(out[m]) for m in out if out[m]}, resp


@pytest.fixture(scope="module")
def reference_runs(built_lib):
    mf = _small_fleet()
    return mf, _per_group(built_lib, mf)


def _check(lfdm, f, mf, ref):
    states, resp = ref
    for m in (18, 24):
        got = f.get_states(m)
        assert np.array_equal(got, states[m]), (m, int(np.argwhere(got != states[m])[0][0]))
        fr = f.get_response(m)
        for i, r in enumerate(resp[m]):
            k = r.shape[0]
            assert np.array_equal(fr[:k, :, i], r), (m, i)
            assert not fr[k:, :, i].any(), (m, i)  # no samples beyond the vehicle's horizon
        assert not f.status_words(m).any()


def test_fleet_matches_per_group_solves_bit_for_bit(built_lib, reference_runs):
    mf, ref = reference_runs
    f = _make(built_lib, mf)
    info = f.info()
    assert info["n18"] == 360 and info["n24"] == 240
    f.solve()
    ms, launches = f.last_ms()
    assert launches == 1 and ms > 0
    _check(built_lib, f, mf, ref)
    f.close()


@pytest.mark.parametrize("launch", [(32, 0, 0), (64, 1, 137), (128, 0, 500), (96, 2, 1)])
def test_fleet_launch_configurations_agree(built_lib, reference_runs, launch):
    """Threads per block, resident blocks per SM and steps per launch change nothing in the results
    (steps per launch 1 exercises per-step launches with the window-end write-back)."""
    mf, ref = reference_runs
    f = _make(built_lib, mf, launch)
    f.solve()
    _check(built_lib, f, mf, ref)
    f.close()


@pytest.mark.parametrize("on", [False, True])
def test_fleet_model_affinity_changes_nothing(built_lib, reference_runs, on):
    """Splitting the SMs between the 18-DOF and 24-DOF tile lists (or not) changes no result; the
    18-DOF share of the estimated work is reported after the solve."""
    mf, ref = reference_runs
    f = _make(built_lib, mf, (64, 0, 0))
    f.set_affinity(on)
    f.solve()
    got_on, frac18 = f.get_affinity()
    assert got_on == on and 0.0 < frac18 < 1.0
    _check(built_lib, f, mf, ref)
    f.close()


@pytest.mark.parametrize("model", [18, 24])
def test_fleet_of_one_model(built_lib, reference_runs, model):
    """A fleet of one model only (the other tile list empty, the SMs all on one list)."""
    mf, (states, resp) = reference_runs
    f = built_lib.Fleet(dt=1e-3, kernel_sim_time=KSIM, output_dt=DTOUT)
    base = f.add_rows(mf["rows"])
    for g in mf["groups"]:
        if g["model"] == model:
            f.add(g["model"], g["cls"], g["params"], g["states"], g["horizons"], None, base + g["row_off"],
                  g["row_len"])
    f.solve()
    assert f.get_affinity()[1] == (1.0 if model == 18 else 0.0)
    assert np.array_equal(f.get_states(model), states[model])
    fr = f.get_response(model)
    for i, r in enumerate(resp[model]):
        assert np.array_equal(fr[: r.shape[0], :, i], r), i
    f.close()


def test_fleet_mixed_tire_precision_matches_per_group_solves(built_lib):
    """With the FP32 tire core (LFDM_PREC_MIXED_TIRE) the fleet kernel gives every vehicle what the
    window kernels of that precision give it, bit for bit, with and without model affinity."""
    mf = _small_fleet(n=300, seed=12)
    ref = _per_group(built_lib, mf, precision=2)
    for on in (True, False):
        f = _make(built_lib, mf, (64, 0, 0))
        f.set_precision(2)
        f.set_affinity(on)
        f.solve()
        _check(built_lib, f, mf, ref)
        f.close()
    fp64 = _per_group(built_lib, mf)[0]
    assert not np.array_equal(fp64[18], ref[0][18])  # the FP32 core does round differently
    f = _make(built_lib, mf)
    with pytest.raises(built_lib.LfdmError):
        f.set_precision(1)  # the FP32 right-hand side form is built for the window kernels only
    f.close()


def test_fleet_autotune_then_solve(built_lib, reference_runs):
    mf, ref = reference_runs
    f = _make(built_lib, mf)
    ms = f.tune(200)
    assert ms > 0
    threads, bps, spl = f.get_launch()
    assert threads in (32, 64, 128)
    f.solve()
    _check(built_lib, f, mf, ref)
    f.close()


def test_fleet_graph_replay_continues_like_solve(built_lib):
    """A second solve continues from the first one's states, like a second Solve() of the regular
    solver (time restarts at 0), and replays the same captured graph."""
    mf = _small_fleet(200, seed=5)
    f = _make(built_lib, mf)
    f.solve()
    f.solve()
    twice = {m: f.get_states(m) for m in (18, 24)}
    f.close()
    g = _make(built_lib, mf)
    g.solve()
    for m in (18, 24):
        g.set_states(m, g.get_states(m))  # host round trip of the states
    g.solve()
    for m in (18, 24):
        assert np.array_equal(g.get_states(m), twice[m])
    g.close()


def test_fleet_rejects_bad_input(built_lib):
    fleet = pkg_mod("fleet")
    cls, p = fleet.suv18()
    f = built_lib.Fleet()
    rows = np.array([[0.0, 0, 0.5, 0], [1.0, 0, 0.5, 0]])
    with pytest.raises(built_lib.LfdmError):
        f.add(11, cls, p[None], np.zeros((1, built_lib.S_COUNT)), [1.0], rows, [0], [2])
    with pytest.raises(built_lib.LfdmError):  # rows outside the table
        f.add(18, cls, p[None], np.zeros((1, built_lib.S_COUNT)), [1.0], rows, [1], [2])
    with pytest.raises(built_lib.LfdmError):  # decreasing times inside a table
        f.add(18, cls, p[None], np.zeros((1, built_lib.S_COUNT)), [1.0], rows[::-1].copy(), [0], [2])
    with pytest.raises(built_lib.LfdmError):  # nothing to solve
        f.solve()
    f.close()
