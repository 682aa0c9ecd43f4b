"""Seeded synthetic fleets (parameter jitter, driver-input families, initial states).

These stand in for the reference's JSON/driver-file fixtures at fleet scale. The vehicle is a
mid-size SUV: mass 2,100 kg, Jz 3,500 kg m^2, CG 1.6 m behind the front axle and 1.7 m ahead of
the rear axle, track 1.8 m, CG height 0.7 m, wheel radius 0.47 m, wheel inertia 1.5 kg m^2, a
6-point engine torque map peaking at 500 N m near 300 rad/s, a torque converter with 10-point
capacity-factor and torque-ratio tables, and TMeasy tires with vertical stiffness 2e5 N/m whose
force curves peak at 1.0*Fz at slip 0.1 and slide at 0.8*Fz from slip 0.5. Fields the
description leaves open are chosen here and listed in SUV18_VEHICLE / SUV_TIRE.

Driver families (per vehicle, seeded): steering wheel angle A*sin(2*pi*f*t) with
A ~ U[0, 0.5] rad and f ~ U[0.2, 1] Hz, given to the model as the normalised input
A/maxSteer*sin(...); throttle ramping linearly from 0 to U[0.3, 1] over 2 s; optionally a brake
pulse of 0.6 for 1 s starting at U[4, 8] s, during which the throttle is released. Tables are
sampled every `table_dt` seconds (rows {t, steering, throttle, braking}).
"""
from __future__ import annotations

import math

import numpy as np

from ._abi import Class18, P, P_COUNT, S, S_COUNT, S_TIRE0, S_TIRE_STRIDE, T, TIRE_TMEASY
from .params import vehicle_from_json

SUV18_VEHICLE = {
    "a": 1.6, "b": 1.7, "m": 2100.0, "h": 0.7, "jz": 3500.0, "jx": 900.0, "jxz": 3.0,
    "cf": 1.8, "cr": 1.8, "muf": 100.0, "mur": 100.0, "hrcf": 0.35, "hrcr": 0.32,
    "krof": 40000.0, "kror": 40000.0, "brof": 3500.0, "bror": 3500.0,
    "nonLinearSteer": False, "maxSteer": 0.6, "crankInertia": 0.8,
    "upshiftRPM": 4000.0, "downshiftRPM": 1800.0,
    "gearRatios": [0.05, 0.09, 0.14, 0.2],
    # 6 points (RPM, N m): peak 500 N m at 2865 RPM = 300 rad/s
    "torqueMap": [[-100.0, 300.0], [1000.0, 420.0], [2000.0, 480.0], [2865.0, 500.0], [4000.0, 430.0],
                  [5000.0, -300.0]],
    "lossesMap": [[-50.0, 20.0], [0.0, 0.0], [50.0, -20.0], [1000.0, -35.0], [2000.0, -50.0], [3000.0, -65.0]],
    "tcBool": True,
    "capacityFactorMap": [[0.0, 15.0], [0.1, 15.0], [0.2, 15.0], [0.3, 15.2], [0.4, 15.5], [0.5, 16.0],
                          [0.6, 16.5], [0.7, 17.5], [0.85, 20.0], [1.0, 35.0]],
    "torqueRatioMap": [[0.0, 2.2], [0.1, 2.05], [0.2, 1.9], [0.3, 1.75], [0.4, 1.6], [0.5, 1.45],
                       [0.6, 1.3], [0.7, 1.15], [0.85, 1.05], [1.0, 1.0]],
    "maxBrakeTorque": 4000.0, "throttleMod": False, "4wd": True, "rearWheels": True,
}
_PN = 5150.0  # nominal tire load ~ m*g/4
SUV_TIRE = {
    "jw": 1.5, "rr": 0.015, "r0": 0.47, "pn": _PN, "pnmax": 3.0 * _PN, "cx": 185000.0, "cy": 165000.0,
    "kt": 2.0e5, "dx": 3700.0, "dy": 3500.0, "rdyncoPn": 0.375, "rdyncoP2n": 0.75, "fzRdynco": 0.0,
    "rdyncoCrit": 0.0,
    "dfx0Pn": 25.0 * _PN, "dfx0P2n": 45.0 * _PN, "fxmPn": 1.0 * _PN, "fxmP2n": 2.0 * _PN,
    "fxsPn": 0.8 * _PN, "fxsP2n": 1.6 * _PN, "sxmPn": 0.1, "sxmP2n": 0.1, "sxsPn": 0.5, "sxsP2n": 0.5,
    "dfy0Pn": 22.0 * _PN, "dfy0P2n": 40.0 * _PN, "fymPn": 1.0 * _PN, "fymP2n": 2.0 * _PN,
    "fysPn": 0.8 * _PN, "fysP2n": 1.6 * _PN, "symPn": 0.1, "symP2n": 0.1, "sysPn": 0.5, "sysP2n": 0.5,
}
FRICTION_FIELDS = ("fxmpn", "fxmp2n", "fxspn", "fxsp2n", "fympn", "fymp2n", "fyspn", "fysp2n")
WHEELBASE = SUV18_VEHICLE["a"] + SUV18_VEHICLE["b"]


def suv18() -> tuple[Class18, np.ndarray]:
    return vehicle_from_json(SUV18_VEHICLE, SUV_TIRE, TIRE_TMEASY)


# The same SUV for the 11-DOF (single-track) model: its JSON holds only the 11-DOF keys.
SUV11_VEHICLE = {k: v for k, v in SUV18_VEHICLE.items()
                 if k not in ("jx", "jxz", "cf", "cr", "hrcf", "hrcr", "krof", "kror", "brof", "bror")}


def suv11() -> tuple[Class18, np.ndarray]:
    return vehicle_from_json(SUV11_VEHICLE, SUV_TIRE, TIRE_TMEASY, model=11)


def fleet11(n: int, seed: int = 20261203, horizon: float = 10.0, table_dt: float = 0.01,
            u0_range=(0.0, 20.0)) -> dict:
    """The seeded 11-DOF SUV fleet: one shared parameter set, per-vehicle driver tables (sine steering,
    throttle ramp, no brake) and initial speeds U[0, 20] m/s with the wheels rolling (omega = u0/r0)
    and the gear/crank set as in initial_states. States follow the LFDM11_S_* layout."""
    from ._abi import C
    rng = np.random.default_rng(seed)
    cls, base = suv11()
    params = np.repeat(base[None, :], n, axis=0)
    tables = driver_tables(n, rng, horizon, table_dt, params[:, P["maxsteer"]], brake_pulse=False)
    s18 = initial_states(cls, params, rng, u0_range)
    s = np.zeros((n, C["LFDM11_S_COUNT"]))
    s[:, C["LFDM11_S_U"]] = s18[:, S["u"]]
    s[:, C["LFDM11_S_CRANKOMEGA"]] = s18[:, S["crankomega"]]
    s[:, C["LFDM11_S_CURRENT_GR"]] = s18[:, S["current_gr"]]
    for k in range(2):
        s[:, C["LFDM11_S_TIRE0"] + k * S_TIRE_STRIDE + T["omega"]] = s18[:, S_TIRE0 + T["omega"]]
    return {"cls": [cls], "class_of": np.zeros(n, dtype=np.int32), "params": params, "tables": tables,
            "states": s, "seed": seed, "horizon": horizon}


def jitter_params(base: np.ndarray, n: int, rng: np.random.Generator, frac: float = 0.1) -> np.ndarray:
    """Per-vehicle copies of `base` with mass, Jz, CG position (a; b = wheelbase - a), tire vertical
    stiffness and peak-friction scale drawn uniformly within +/-frac of the base values. The
    friction scale multiplies the TMeasy peak and sliding forces (fxm*, fym*, fxs*, fys*)."""
    p = np.repeat(base[None, :], n, axis=0)
    u = lambda: rng.uniform(1.0 - frac, 1.0 + frac, size=n)  # noqa: E731
    p[:, P["m"]] *= u()
    p[:, P["jz"]] *= u()
    wb = base[P["a"]] + base[P["b"]]
    p[:, P["a"]] *= u()
    p[:, P["b"]] = wb - p[:, P["a"]]
    p[:, P["kt"]] *= u()
    mu = u()
    for f in FRICTION_FIELDS:
        p[:, P[f]] *= mu
    return p


def driver_tables(n: int, rng: np.random.Generator, horizon: float, table_dt: float = 0.01,
                  max_steer: np.ndarray | float = 0.6, brake_pulse: bool = True,
                  dtype=np.float64, amplitude: float = 0.5) -> np.ndarray:
    """[n][rows][4] tables {t, steering, throttle, braking}, rows = horizon/table_dt + 1; the steering
    wheel-angle amplitude is drawn from U[0, amplitude] rad."""
    rows = int(round(horizon / table_dt)) + 1
    t = (np.arange(rows, dtype=np.float64) / round(1.0 / table_dt)) if abs(1.0 / table_dt - round(1.0 / table_dt)) < 1e-9 \
        else np.arange(rows, dtype=np.float64) * table_dt
    A = rng.uniform(0.0, amplitude, size=n)
    f = rng.uniform(0.2, 1.0, size=n)
    thr = rng.uniform(0.3, 1.0, size=n)
    out = np.empty((n, rows, 4), dtype=dtype)
    out[:, :, 0] = t[None, :]
    ms = np.broadcast_to(np.asarray(max_steer, dtype=np.float64), (n,))
    out[:, :, 1] = (A / ms)[:, None] * np.sin(2.0 * math.pi * f[:, None] * t[None, :])
    out[:, :, 2] = thr[:, None] * np.minimum(t[None, :] / 2.0, 1.0)
    out[:, :, 3] = 0.0
    if brake_pulse:
        tb = rng.uniform(4.0, 8.0, size=n)
        on = (t[None, :] >= tb[:, None]) & (t[None, :] < tb[:, None] + 1.0)
        out[:, :, 3] = np.where(on, 0.6, 0.0)
        out[:, :, 2] = np.where(on, 0.0, out[:, :, 2])
    return out


def initial_states(cls: Class18, params: np.ndarray, rng: np.random.Generator,
                   u0_range=(0.0, 20.0)) -> np.ndarray:
    """[n][S_COUNT] states at rest pose moving straight at u0 ~ U[u0_range]. Every wheel spins at
    omega = u0 / r0; the gear is the lowest one whose crank speed omega/ratio is below the upshift
    speed, and the crank spins at that speed (converter locked)."""
    n = params.shape[0]
    u0 = rng.uniform(u0_range[0], u0_range[1], size=n)
    return states_at_speed(cls, params, u0)


def states_at_speed(cls: Class18, params: np.ndarray, u0: np.ndarray) -> np.ndarray:
    """initial_states with the given initial speeds u0 [n]."""
    n = params.shape[0]
    s = np.zeros((n, S_COUNT), dtype=np.float64)
    s[:, S["u"]] = u0
    w = u0 / params[:, P["r0"]]
    for k in range(4):
        s[:, S_TIRE0 + k * S_TIRE_STRIDE + T["omega"]] = w
    gears = np.array([cls.gearRatios[i] for i in range(cls.noGears)])
    ups = np.array([cls.shiftMap[i][1] for i in range(cls.noGears)])
    crank = w[:, None] / gears[None, :]
    ok = crank < ups[None, :]
    gear = np.where(ok.any(axis=1), ok.argmax(axis=1), cls.noGears - 1)
    s[:, S["current_gr"]] = gear
    s[:, S["crankomega"]] = w / gears[gear]
    return s


def clothoid_refs(n: int, nsteps: int, dt: float, rng: np.random.Generator, curvature=(-0.05, 0.05),
                  speed=(5.0, 25.0)) -> tuple[np.ndarray, np.ndarray]:
    """Seeded reference paths for the differentiable rollout: per vehicle a clothoid segment from the
    origin along +x whose curvature grows linearly from 0 to kappa ~ U[curvature] 1/m over the
    horizon, traversed at speed v ~ U[speed] m/s. Returns (ref [nsteps][3][n] = {x, y, yaw} at the
    end of each step, v [n])."""
    kappa = rng.uniform(curvature[0], curvature[1], size=n)
    v = rng.uniform(speed[0], speed[1], size=n)
    sub = 8  # integration sub-steps per time step
    ts = np.arange(1, nsteps * sub + 1) * (dt / sub)
    S = v * nsteps * dt
    s = ts[:, None] * v[None, :]
    psi = kappa[None, :] * s * s / (2.0 * S[None, :])
    ds = v * dt / sub
    x = np.cumsum(np.cos(psi) * ds[None, :], axis=0)
    y = np.cumsum(np.sin(psi) * ds[None, :], axis=0)
    ref = np.stack([x[sub - 1::sub], y[sub - 1::sub], psi[sub - 1::sub]], axis=1)
    return np.ascontiguousarray(ref), v


def fleet18(n: int, seed: int = 20261203, horizon: float = 10.0, table_dt: float = 0.01,
            brake_pulse: bool = True, jitter: bool = True, u0_range=(0.0, 20.0)) -> dict:
    """The seeded 18-DOF SUV fleet: one class, jittered parameters, per-vehicle driver tables and
    initial states. Returns dict(cls=[Class18], class_of, params, tables, states)."""
    rng = np.random.default_rng(seed)
    cls, base = suv18()
    params = jitter_params(base, n, rng) if jitter else np.repeat(base[None, :], n, axis=0)
    tables = driver_tables(n, rng, horizon, table_dt, params[:, P["maxsteer"]], brake_pulse)
    states = initial_states(cls, params, rng, u0_range)
    return {"cls": [cls], "class_of": np.zeros(n, dtype=np.int32), "params": params, "tables": tables,
            "states": states, "seed": seed, "horizon": horizon}


# Wheel inertia and brake of the calm companion fleet: an HMMWV-class wheel (the reference's HMMWV
# tire files give jw = 6.5 kg m^2) and a 2,000 N m brake, which the 0.6 brake pulse cannot lock.
CALM_JW = 6.5
CALM_MAX_BRAKE_TORQUE = 2000.0
CALM_STEER_AMPLITUDE = 0.1


def fleet18_calm(n: int, seed: int = 20261204, horizon: float = 10.0, table_dt: float = 0.01) -> dict:
    """A seeded 18-DOF SUV fleet whose whole trajectories are insensitive to rounding.

    The parameter jitter (mass, Jz, CG position, tire stiffness, peak friction within +/-10 %), the
    driver families (sine steering, throttle ramp, 1 s brake pulse of 0.6 at U[4, 8] s) and the
    initial speeds U[0, 20] m/s are those of fleet18. Three things differ: the wheel inertia is
    CALM_JW instead of 1.5 kg m^2 (a light wheel chatters in the explicit wheel-speed update at
    dt = 1e-3), the brake torque is CALM_MAX_BRAKE_TORQUE (the brake pulse no longer locks the
    wheels, whose sgn(omega) brake torque then chatters around zero speed) and the steering
    amplitude is U[0, CALM_STEER_AMPLITUDE] rad (no vehicle spins out). On 4,096 such vehicles the
    reference algorithm compiled with and without fused multiply-add contraction agrees to 5.3e-12
    per state after 10 s, so any FP64 implementation must agree with it to rounding level over
    the whole horizon."""
    rng = np.random.default_rng(seed)
    cls, base = suv18()
    base = base.copy()
    base[P["jw"]] = CALM_JW
    base[P["maxbraketorque"]] = CALM_MAX_BRAKE_TORQUE
    params = jitter_params(base, n, rng)
    tables = driver_tables(n, rng, horizon, table_dt, params[:, P["maxsteer"]], True,
                           amplitude=CALM_STEER_AMPLITUDE)
    states = initial_states(cls, params, rng, (0.0, 20.0))
    return {"cls": [cls], "class_of": np.zeros(n, dtype=np.int32), "params": params, "tables": tables,
            "states": states, "seed": seed, "horizon": horizon}

# The same SUV for the 24-DOF model: its JSON holds the 24-DOF keys (pitch inertia instead of the
# roll-stiffness terms) and a suspension with ks = 4e4 N/m and bs = 4e3 N s/m at every corner.
SUV24_VEHICLE = {k: v for k, v in SUV18_VEHICLE.items() if k not in ("jxz", "krof", "kror", "brof", "bror")}
SUV24_VEHICLE["jy"] = 3400.0
SUV24_SUS = {"ks": 4.0e4, "bs": 4.0e3}
G = 9.81  # utils/utils_gpu.cuh


def suv24() -> tuple[Class18, np.ndarray]:
    return vehicle_from_json(SUV24_VEHICLE, SUV_TIRE, TIRE_TMEASY, model=24, sus=SUV24_SUS)


def init_tire_sus24(params: np.ndarray, states: np.ndarray) -> np.ndarray:
    """initializeTireSus (24dof-gpu/dof24_gpu.cu:34-90, applied by Initialize) on [n] flat 24-DOF
    states in place: static tire loads and compressions, spring preload and strut lengths, unsprung
    vertical speed = chassis w."""
    from ._abi import C
    p = np.atleast_2d(params)
    s = np.atleast_2d(states)
    a, b, m, ks = p[:, P["a"]], p[:, P["b"]], p[:, P["m"]], p[:, P["ks"]]
    fz_f = (m * G * b) / (2 * (a + b)) + p[:, P["muf"]] * G
    fz_r = (m * G * a) / (2 * (a + b)) + p[:, P["mur"]] * G
    xsi_f = (m * G * b) / (2 * (a + b) * ks)
    xsi_r = (m * G * a) / (2 * (a + b) * ks)
    T0, TN, S0, SN = C["LFDM24_S_TIRE0"], C["LFDM24_T_COUNT"], C["LFDM24_S_SUS0"], C["LFDM24_SUS_COUNT"]
    for k in range(4):
        fz = fz_f if k < 2 else fz_r
        xsi = xsi_f if k < 2 else xsi_r
        t0, s0 = T0 + k * TN, S0 + k * SN
        s[:, t0 + C["LFDM24_T_FZ"]] = fz
        xt = fz / p[:, P["kt"]]
        s[:, t0 + C["LFDM24_T_XT"]] = xt
        s[:, s0 + C["LFDM24_SUS_XSI"]] = xsi
        s[:, s0 + C["LFDM24_SUS_XS"]] = xsi
        lsi = p[:, P["h"]] - (p[:, P["r0"]] - xt)
        s[:, s0 + C["LFDM24_SUS_LSI"]] = lsi
        s[:, s0 + C["LFDM24_SUS_LS"]] = lsi
        s[:, s0 + C["LFDM24_SUS_WU"]] = s[:, C["LFDM24_S_W"]]
    return states


def initial_states24(cls: Class18, params: np.ndarray, rng: np.random.Generator, u0_range=(0.0, 20.0)) -> np.ndarray:
    """[n][LFDM24_S_COUNT] states: the 18-DOF initial_states' speed, wheel spin, gear and crank,
    followed by initializeTireSus."""
    from ._abi import C
    s18 = initial_states(cls, params, rng, u0_range)
    s = np.zeros((params.shape[0], C["LFDM24_S_COUNT"]))
    s[:, C["LFDM24_S_U"]] = s18[:, S["u"]]
    s[:, C["LFDM24_S_CRANKOMEGA"]] = s18[:, S["crankomega"]]
    s[:, C["LFDM24_S_CURRENT_GR"]] = s18[:, S["current_gr"]]
    for k in range(4):
        s[:, C["LFDM24_S_TIRE0"] + k * C["LFDM24_T_COUNT"] + C["LFDM24_T_OMEGA"]] = s18[:, S_TIRE0 + T["omega"]]
    return init_tire_sus24(params, s)


def fleet24(n: int, seed: int = 20261203, horizon: float = 10.0, table_dt: float = 0.01,
            brake_pulse: bool = True, jitter: bool = True, u0_range=(0.0, 20.0)) -> dict:
    """The seeded 24-DOF SUV fleet (same draws as fleet18: jittered parameters, driver tables, initial
    speeds), with states in the LFDM24_S_* layout after initializeTireSus."""
    rng = np.random.default_rng(seed)
    cls, base = suv24()
    params = jitter_params(base, n, rng) if jitter else np.repeat(base[None, :], n, axis=0)
    tables = driver_tables(n, rng, horizon, table_dt, params[:, P["maxsteer"]], brake_pulse)
    states = initial_states24(cls, params, rng, u0_range)
    return {"cls": [cls], "class_of": np.zeros(n, dtype=np.int32), "params": params, "tables": tables,
            "states": states, "seed": seed, "horizon": horizon}


# Mixed-DOF fleet: four parameter classes around the SUV (mass 1,300 / 1,700 / 2,100 / 2,800 kg;
# inertias and the tire's nominal load scaled with the mass so that the force curves keep their
# shape relative to the load), 18-DOF and 24-DOF vehicles, log-uniform end times.
CLASS_MASSES = (1300.0, 1700.0, 2100.0, 2800.0)


def suv_tire(pn: float) -> dict:
    """SUV_TIRE with the nominal load pn and the load-proportional entries scaled with it."""
    t = dict(SUV_TIRE)
    s = pn / _PN
    for k in ("pn", "pnmax", "dfx0Pn", "dfx0P2n", "fxmPn", "fxmP2n", "fxsPn", "fxsP2n", "dfy0Pn", "dfy0P2n", "fymPn",
              "fymP2n", "fysPn", "fysP2n"):
        t[k] = SUV_TIRE[k] * s
    return t


def class_vehicle(model: int, mass: float) -> tuple[Class18, np.ndarray]:
    """The SUV scaled to `mass` for the 18- or 24-DOF model."""
    s = mass / SUV18_VEHICLE["m"]
    base = SUV24_VEHICLE if model == 24 else SUV18_VEHICLE
    veh = dict(base, m=mass, jz=base["jz"] * s, jx=base["jx"] * s)
    if model == 24:
        veh["jy"] = base["jy"] * s
        return vehicle_from_json(veh, suv_tire(_PN * s), TIRE_TMEASY, model=24, sus=SUV24_SUS)
    return vehicle_from_json(veh, suv_tire(_PN * s), TIRE_TMEASY)


def mixed_fleet(n: int, seed: int = 20261203, frac24: float = 0.4, horizon_range=(2.0, 20.0), n_tables: int = 4096,
                table_dt: float = 0.01, u0_range=(0.0, 20.0)) -> dict:
    """The seeded mixed fleet: vehicles split 1 - frac24 : frac24 between the 18- and 24-DOF models,
    spread evenly over the four mass classes, jittered +/-10% (mass, Jz, CG position, tire vertical
    stiffness, peak friction), end times log-uniform in horizon_range, and driver tables drawn from
    n_tables shared seeded tables (the 18-DOF families with a brake pulse) covering the longest
    horizon. Returns dict(rows [nrows][4], groups=[dict(model, cls, params, states, horizons,
    row_off, row_len, mass)])."""
    rng = np.random.default_rng(seed)
    hmax = float(horizon_range[1])
    rows_per = int(round(hmax / table_dt)) + 1
    tables = driver_tables(n_tables, rng, hmax, table_dt, SUV18_VEHICLE["maxSteer"], brake_pulse=True)
    rows = tables.reshape(-1, 4)
    n24 = int(round(n * frac24))
    counts = {18: n - n24, 24: n24}
    groups = []
    lo, hi = np.log(horizon_range[0]), np.log(horizon_range[1])
    for model in (18, 24):
        m_total = counts[model]
        for ci, mass in enumerate(CLASS_MASSES):
            k = m_total // len(CLASS_MASSES) + (1 if ci < m_total % len(CLASS_MASSES) else 0)
            if k == 0:
                continue
            cls, base = class_vehicle(model, mass)
            params = jitter_params(base, k, rng)
            if model == 24:
                states = initial_states24(cls, params, rng, u0_range)
            else:
                states = initial_states(cls, params, rng, u0_range)
            horizons = np.exp(rng.uniform(lo, hi, size=k))
            tix = rng.integers(0, n_tables, size=k)
            groups.append({"model": model, "cls": cls, "params": params, "states": states, "horizons": horizons,
                           "row_off": (tix * rows_per).astype(np.int64),
                           "row_len": np.full(k, rows_per, dtype=np.int32), "mass": mass})
    return {"rows": rows, "groups": groups, "seed": seed}
