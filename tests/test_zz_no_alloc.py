"""lfdm_step18_noalloc (the entry point that allocates nothing; its scratch is one static device
array) on the GPU: two calls in a row on device-resident vehicles, checked bit for bit against the
solver API's SolveStep with the same per-vehicle controls and against the oracle (1e-12, or the
reference algorithm's own sensitivity near branch points), and the capacity check. Named so that
pytest collects it last; it also passes alone in a fresh process.
"""
import numpy as np
import pytest

import oracle_lib as O
from conftest import pkg_mod, rel_err, state_floors

pytestmark = pytest.mark.gpu


def _fleet(n, seed):
    f = pkg_mod("fleet").fleet18(n, seed=seed, horizon=2.0)
    rng = np.random.default_rng(seed)
    ctl = np.stack([rng.uniform(-0.3, 0.3, n), rng.uniform(0.0, 1.0, n), np.where(rng.random(n) < 0.2, 0.5, 0.0)],
                   axis=1)
    return f, ctl


def test_two_calls_in_a_row_match_solver_and_oracle(built_lib):
    torch = pytest.importorskip("torch")
    n = 3000  # not a multiple of the block size
    f, ctl = _fleet(n, seed=11)
    cls = f["cls"][0]

    # the same two windows through the solver API
    sol = built_lib.d18SolverHalfImplicitGPU(n)
    sol.construct_class(cls, f["params"])
    sol.set_states(f["states"])
    sol.SetKernelSimTime(0.02)
    steps0 = len(sol.window_times(0.0))
    t1 = sol.SolveStep(0.0, ctl[:, 0], ctl[:, 1], ctl[:, 2])
    steps1 = len(sol.window_times(t1))
    sol.SolveStep(t1, ctl[:, 0], ctl[:, 1], ctl[:, 2])
    want = sol.get_states()
    sol.close()

    dev = torch.device("cuda", 0)
    params = torch.from_numpy(np.ascontiguousarray(f["params"])).to(dev)
    states = torch.from_numpy(np.ascontiguousarray(f["states"])).to(dev)
    c = [torch.from_numpy(np.ascontiguousarray(ctl[:, k])).to(dev) for k in range(3)]
    stream = torch.cuda.current_stream(dev)
    torch.cuda.synchronize(dev)
    args = (cls, params.data_ptr(), states.data_ptr(), c[0].data_ptr(), c[1].data_ptr(), c[2].data_ptr(), n)
    built_lib.step18_noalloc(*args, 0.0, 1e-3, steps0, stream.cuda_stream)
    built_lib.step18_noalloc(*args, t1, 1e-3, steps1, stream.cuda_stream)
    torch.cuda.synchronize(dev)
    got = states.cpu().numpy()
    assert np.array_equal(got, want)

    # oracle: rounding-level agreement, or within 100x the reference algorithm's sensitivity where a
    # vehicle sits near a branch point (the largest deviation among its FMA-contracted build and
    # runs from u scaled by 1 +- 1e-15)
    def two_windows(s0, **kw):
        st = s0
        for t0 in (0.0, t1):
            st, _ = O.run18(f["cls"], f["class_of"], f["params"], st, ctl=ctl, t0=t0, ksim=0.02, schedule=2,
                            nthreads=8, **kw)
        return st

    fl = state_floors()
    ref = two_windows(f["states"])
    runs = [two_windows(f["states"], fma=True)]
    U = pkg_mod("_abi").S["u"]
    for eps in (1e-15, -1e-15):
        s2 = f["states"].copy()
        s2[:, U] *= 1.0 + eps
        runs.append(two_windows(s2))
    env = np.max([rel_err(r, ref, fl).max(axis=1) for r in runs], axis=0)
    e = rel_err(got, ref, fl).max(axis=1)
    assert (e <= np.maximum(1e-12, 100 * env)).all(), (float(e.max()), int(e.argmax()))
    assert (e[env <= 1e-13] <= 1e-12).all()


def test_capacity_and_arguments_rejected(built_lib):
    torch = pytest.importorskip("torch")
    cls, p = pkg_mod("fleet").suv18()
    big = built_lib.NOALLOC_MAX_VEHICLES + 1
    with pytest.raises(built_lib.LfdmError, match="capacity"):
        built_lib.step18_noalloc(cls, 1, 1, 1, 1, 1, big, 0.0, 1e-3, 10)
    x = torch.zeros(8, dtype=torch.float64, device="cuda")
    with pytest.raises(built_lib.LfdmError, match="null"):
        built_lib.step18_noalloc(cls, 0, x.data_ptr(), x.data_ptr(), x.data_ptr(), x.data_ptr(), 1, 0.0, 1e-3, 10)
    with pytest.raises(built_lib.LfdmError, match="dt"):
        built_lib.step18_noalloc(cls, x.data_ptr(), x.data_ptr(), x.data_ptr(), x.data_ptr(), x.data_ptr(), 1, 0.0,
                                 -1.0, 10)
