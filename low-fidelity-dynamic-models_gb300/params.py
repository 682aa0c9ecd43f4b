"""Vehicle/tire JSON files -> (lfdm_class18, flat parameter vector), in pure Python.

Mirrors the reference loaders setVehParamsJSON (18dof-gpu/dof18_gpu.cu:1075-1218) and
setTireParamsJSON for TMeasy (:1222-1266), including their defaults (the default constructors of
VehicleParam, dof18_gpu.cuh:506-531, and TMeasyParam, :29-64) and unit conversions (engine and
shift maps given in RPM are stored in rad/s). The C++ loader inside the library
(csrc/json_loader.cpp) implements the same rules; tests check the two agree.
"""
from __future__ import annotations

import json
import math

import numpy as np

from ._abi import Class18, P, P_COUNT, TIRE_TMEASY, TIRE_TMEASY_NR, MAX_GEARS

RPM2RAD = math.pi / 30  # utils/utils_gpu.cuh:13 (C_PI / 30)

VEH_DEFAULTS = {  # VehicleParam() defaults, dof18_gpu.cuh:506-531
    "a": 1.6889, "b": 1.6889, "h": 0.713, "m": 2097.85, "jz": 4519.0, "jx": 1289.0, "jxz": 3.265,
    "cf": 1.82, "cr": 1.82, "muf": 127.866, "mur": 129.98, "hrcf": 0.379, "hrcr": 0.327,
    "krof": 31000.0, "kror": 31000.0, "brof": 3300.0, "bror": 3300.0, "maxsteer": 0.6525249,
    "crankinertia": 1.1, "maxbraketorque": 4000.0,
    "jy": 3516.0,  # 24-DOF VehicleParam() default, 24dof-gpu/dof24_gpu.cuh
}
SUS_DEFAULTS = {"ks": 150062.0, "bs": 19068.0}  # SuspensionParam() defaults, 24dof-gpu/dof24_gpu.cuh
TM_DEFAULTS = {  # TMeasyParam() defaults, dof18_gpu.cuh:29-64
    "jw": 6.69, "rr": 0.015, "mu": 0.8, "r0": 0.4699, "pn": 8562.8266, "pnmax": 29969.893,
    "cx": 185004.42, "cy": 164448.37, "kt": 411121.0, "dx": 3700.0, "dy": 3488.0, "rdyncopn": 0.375,
    "rdyncop2n": 0.75, "fzrdynco": 0.0, "rdyncocrit": 0.0, "dfx0pn": 151447.29, "dfx0p2n": 236412.79,
    "fxmpn": 7575.3614, "fxmp2n": 12808.276, "fxspn": 4657.9208, "fxsp2n": 8625.3352, "sxmpn": 0.12,
    "sxmp2n": 0.15, "sxspn": 0.9, "sxsp2n": 0.95, "dfy0pn": 50931.693, "dfy0p2n": 94293.847,
    "fympn": 6615.0404, "fymp2n": 12509.947, "fyspn": 6091.5092, "fysp2n": 11443.875, "sympn": 0.38786,
    "symp2n": 0.38786, "syspn": 0.82534, "sysp2n": 0.91309,
}
NR_DEFAULTS = {  # TMeasyNrParam() extra defaults, dof18_gpu.cuh:267-307
    "width": 0.245, "rim_radius": 0.254, "vcoulomb": 1.0, "frblend_begin": 1.0, "frblend_end": 3.0,
    "bearingcapacity": 10000.0, "li": 90.0, "p_li": 1.0, "p_use": 1.0,
}

# JSON key -> flat parameter name (vehicle scalars read unconditionally by the loader)
_VEH_KEYS = ["a", "b", "m", "h", "jz", "jx", "jxz", "cf", "cr", "muf", "mur", "hrcf", "hrcr", "krof", "kror",
             "brof", "bror"]
_TM_KEYS = ["jw", "rr", "r0", "pn", "pnmax", "cx", "cy", "kt", "dx", "dy", "rdyncoPn", "rdyncoP2n", "fzRdynco",
            "rdyncoCrit", "dfx0Pn", "dfx0P2n", "fxmPn", "fxmP2n", "fxsPn", "fxsP2n", "sxmPn", "sxmP2n", "sxsPn",
            "sxsP2n", "dfy0Pn", "dfy0P2n", "fymPn", "fymP2n", "fysPn", "fysP2n", "symPn", "symP2n", "sysPn",
            "sysP2n"]


def _load(obj):
    if isinstance(obj, dict):
        return obj
    with open(obj, "r", encoding="utf-8") as f:
        return json.load(f)


def interp_l(fz, w1, w2, pn):
    """InterpL, utils/utils_gpu.cuh:86-88."""
    return w1 + (w2 - w1) * (fz / pn - 1.0)


def tire_init(p: np.ndarray) -> np.ndarray:
    """tireInit, dof18_gpu.cu:227-233, on one flat parameter vector (in place)."""
    pn, r1, r2 = p[P["pn"]], p[P["rdyncopn"]], p[P["rdyncop2n"]]
    p[P["fzrdynco"]] = (pn * (r2 - 2.0 * r1 + 1.0)) / (2.0 * (r2 - r1))
    p[P["rdyncocrit"]] = interp_l(p[P["fzrdynco"]], r1, r2, pn)
    return p


def default_params() -> np.ndarray:
    p = np.zeros(P_COUNT, dtype=np.float64)
    for k, v in {**VEH_DEFAULTS, **TM_DEFAULTS, **NR_DEFAULTS, **SUS_DEFAULTS}.items():
        p[P[k]] = v
    return p


_VEH_KEYS_11 = ["a", "b", "m", "h", "jz", "muf", "mur"]  # setVehParamsJSON, 11dof-gpu/dof11_gpu.cu:910-1044
_DOUBLED_11 = ["jw", "rr", "pn", "pnmax", "cx", "cy", "kt", "dx", "dy", "fzrdynco", "rdyncocrit", "dfx0pn", "dfx0p2n",
               "fxmpn", "fxmp2n", "fxspn", "fxsp2n", "dfy0pn", "dfy0p2n", "fympn", "fymp2n", "fyspn", "fysp2n"]
_KEY_OF = {k.lower(): k for k in _TM_KEYS}
# setVehParamsJSON, 24dof-gpu/dof24_gpu.cu (24dof/dof24.cpp:2217-2339)
_VEH_KEYS_24 = ["a", "b", "m", "h", "jz", "jx", "jy", "cf", "cr", "muf", "mur", "hrcf", "hrcr"]


def vehicle_from_json(veh, tire, tire_type: int = TIRE_TMEASY, model: int = 18, sus=None) -> tuple[Class18, np.ndarray]:
    """Parse a vehicle JSON and a tire JSON (paths or dicts) the way Construct does.

    Returns the class record and the flat parameter vector with tireInit applied
    (d18SolverHalfImplicitGPU::Construct calls tireInit after loading, dof18_halfImplicit_gpu.cu:78).
    model 11 reads the 11-DOF vehicle keys (11dof-gpu/dof11_gpu.cu:910-1044); model 24 the 24-DOF
    ones and the suspension JSON `sus` (setSuspensionParamsJSON, 24dof/dof24.cpp:2192-2212).
    """
    d = _load(veh)
    t = _load(tire)
    p = default_params()
    c = Class18()
    c.driveType, c.whichWheels = 1, 1
    if model == 24:
        if sus is None:
            raise ValueError("the 24-DOF model needs a suspension JSON")
        s = _load(sus)
        p[P["ks"]] = float(s["ks"])
        p[P["bs"]] = float(s["bs"])
    for k in {11: _VEH_KEYS_11, 24: _VEH_KEYS_24}.get(model, _VEH_KEYS):
        p[P[k]] = float(d[k])
    c.nonLinearSteer = int(bool(d["nonLinearSteer"]))
    if c.nonLinearSteer:
        c.set_map("steerMap", d["steerMap"])
    p[P["maxsteer"]] = float(d["maxSteer"])
    gears = [float(g) for g in d["gearRatios"]]
    if len(gears) > MAX_GEARS:
        raise ValueError(f"{len(gears)} gears > LFDM_MAX_GEARS={MAX_GEARS}")
    c.noGears = len(gears)
    for i, g in enumerate(gears):
        c.gearRatios[i] = g
    for i in range(len(gears)):
        if "upshiftRPM" in d and "downshiftRPM" in d:
            c.shiftMap[i][0] = float(d["downshiftRPM"]) * RPM2RAD
            c.shiftMap[i][1] = float(d["upshiftRPM"]) * RPM2RAD
        else:
            c.shiftMap[i][0] = float(d["shiftMap"][i][0]) * RPM2RAD
            c.shiftMap[i][1] = float(d["shiftMap"][i][1]) * RPM2RAD
    c.tcbool = int(bool(d["tcBool"]))
    p[P["maxbraketorque"]] = float(d["maxBrakeTorque"])
    c.throttleMod = int(bool(d["throttleMod"]))
    c.set_map("powertrainMap", [(float(x) * RPM2RAD, float(y)) for x, y in d["torqueMap"]])
    c.set_map("lossesMap", [(float(x) * RPM2RAD, float(y)) for x, y in d["lossesMap"]])
    if c.tcbool:
        p[P["crankinertia"]] = float(d["crankInertia"])
        c.set_map("CFmap", d["capacityFactorMap"])
        c.set_map("TRmap", d["torqueRatioMap"])
    if "4wd" in d:
        c.driveType = int(bool(d["4wd"]))
        c.whichWheels = int(bool(d["rearWheels"]))
    if tire_type == TIRE_TMEASY:
        for k in _TM_KEYS:
            p[P[k.lower()]] = float(t[k])
        if model == 11:
            # the single-track tire stands for both wheels of an axle: setTireParamsJSON
            # (11dof-gpu/dof11_gpu.cu:1046-1099) doubles the inertia, resistance, loads,
            # stiffnesses, dampings, slopes and forces, and keeps r0, rdynco weights and slips
            for k in _DOUBLED_11:
                p[P[k]] = float(t[_KEY_OF[k]]) * 2.0
    elif tire_type == TIRE_TMEASY_NR:
        if t.get("highLevelParams", False):
            raise NotImplementedError("TMeasyNr high-level parameter guessing is not supported")
        for k in _TM_KEYS:
            if k in ("cx", "cy", "dx", "dy"):
                continue
            p[P[k.lower()]] = float(t[k])
    else:
        raise ValueError("unknown tire type")
    tire_init(p)
    return c, p


def load_driver_table(path_or_text, is_text: bool = False) -> np.ndarray:
    """LoadDriverData, utils/utils_gpu.cu:7-31: whitespace rows `t steering throttle braking`;
    parsing stops at the first line that does not hold four numbers."""
    if is_text:
        lines = path_or_text.splitlines()
    else:
        with open(path_or_text, "r", encoding="utf-8") as f:
            lines = f.read().splitlines()
    rows = []
    for line in lines:
        parts = line.split()
        try:
            vals = [float(x) for x in parts[:4]]
        except ValueError:
            break
        if len(vals) < 4:
            break
        rows.append(vals)
    return np.asarray(rows, dtype=np.float64).reshape(-1, 4)
