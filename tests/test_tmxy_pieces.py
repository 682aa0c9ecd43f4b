"""The division-free transition regime of the combined-slip force curve (tmxy_joint and
tmxy_transition in include/lfdm/device/dof18_device.cuh) against the reference's own formulas
(tmxy_combined, 18dof-gpu/dof18_gpu.cu:261-279: the first parabola's coefficient
a = (fm/sm)^2 / (df0loc sm), the joint sstar = sm + (fm - fs) / (a (ss - sm)), the second parabola's
b = a (sstar - sm) / (ss - sstar), the cubic's sn = (s - sm) / (ss - sm)), evaluated in numpy over
random tire states that reach all three pieces: the piece chosen by products equals the piece
chosen by the quotients, and f = num / den agrees with the reference's f to a few ulps.

The device code chooses the piece with H <= (ss - sm) E and (s - sm) E <= H, where D = df0loc sm,
E = (fm/sm)^2 (ss - sm) and H = (fm - fs) D, and returns the force over the denominator of its piece
(D, G = (ss - sm) E - H, or (ss - sm)^3). This restates those expressions to pin the algebra; the
GPU parity tests check the compiled curve inside the stepper against the oracle."""
import numpy as np


def _reference(s, sm, ss, fm, fs, df0loc):
    a = (fm / sm) ** 2 / (df0loc * sm)
    sstar = sm + (fm - fs) / (a * (ss - sm))
    piece = np.where(sstar <= ss, np.where(s <= sstar, 0, 1), 2)
    with np.errstate(divide="ignore", invalid="ignore"):
        b = a * (sstar - sm) / (ss - sstar)
        sn = (s - sm) / (ss - sm)
    f = np.select([piece == 0, piece == 1],
                  [fm - a * (s - sm) * (s - sm), fs + b * (ss - s) * (ss - s)],
                  fm - (fm - fs) * sn * sn * (3.0 - 2.0 * sn))
    return piece, f


def _division_free(s, sm, ss, fm, fs, df0loc):
    ism = 1.0 / sm
    q = fm * ism
    q2 = q * q
    D = df0loc * sm
    dss = ss - sm
    E = q2 * dss
    H = (fm - fs) * D
    piece = np.where(H <= dss * E, np.where((s - sm) * E <= H, 0, 1), 2)
    ds = s - sm
    G = dss * E - H
    r = ss - s
    d3 = dss * dss * dss
    num = np.select([piece == 0, piece == 1],
                    [fm * D - q2 * ds * ds, fs * G + q2 * (fm - fs) * r * r],
                    fm * d3 - (fm - fs) * ds * ds * (3.0 * dss - 2.0 * ds))
    den = np.select([piece == 0, piece == 1], [D, G], d3)
    return piece, num / den


def _tire_states(n, seed):
    rng = np.random.default_rng(seed)
    sm = rng.uniform(0.05, 0.3, n)
    ss = sm + rng.uniform(0.01, 1.0, n)
    fm = rng.uniform(1e3, 1e4, n)
    fs = fm * rng.uniform(0.5, 1.0, n)
    df0loc = np.maximum(2.0 * fm / sm, rng.uniform(1e3, 2e5, n))
    s = sm + rng.uniform(0.0, 1.0, n) * (ss - sm)
    return s, sm, ss, fm, fs, df0loc


def test_pieces_and_force_match_the_reference_formulas():
    args = _tire_states(200_000, 1)
    want_piece, want_f = _reference(*args)
    got_piece, got_f = _division_free(*args)
    counts = np.bincount(got_piece, minlength=3)
    print(f"pieces {counts.tolist()}")
    assert (counts > 1000).all()  # every piece is exercised
    assert np.array_equal(got_piece, want_piece)
    rel = np.abs(got_f - want_f) / np.abs(want_f)
    print(f"max relative difference {rel.max():.2e}")
    assert rel.max() <= 1e-14


def test_pieces_at_the_regime_ends():
    """At s = sm the first parabola gives fm; at s = ss the second parabola and the cubic give fs."""
    s, sm, ss, fm, fs, df0loc = _tire_states(10_000, 2)
    p0, f0 = _division_free(sm, sm, ss, fm, fs, df0loc)
    assert (p0 != 1).all()
    assert np.allclose(f0, fm, rtol=1e-14, atol=0.0)
    p1, f1 = _division_free(ss, sm, ss, fm, fs, df0loc)
    assert (p1 != 0).all()
    assert np.allclose(f1, fs, rtol=1e-13, atol=0.0)
