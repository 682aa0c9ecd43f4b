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
        _tmeasy_nr_params(t, p, model)
    else:
        raise ValueError("unknown tire type")
    tire_init(p)
    return c, p


# Maximum tire load [kg] by load index 0..279, the table of GetTireMaxLoad
# (18dof-gpu/dof18_gpu.cu:1470-1503; the 11- and 24-DOF models hold the same numbers). Indices past
# the end take the last entry.
_LOAD_INDEX_KG = (
    45, 46.5, 47.5, 48.7, 50, 51.5, 53, 54.5, 56, 58,  # LI 0-9
    60, 61.5, 63, 65, 67, 69, 71, 73, 75, 77.5,  # LI 10-19
    80.0, 82.5, 85.0, 87.5, 90.0, 92.5, 95.0, 97.5, 100.0, 103,  # LI 20-29
    106, 109, 112, 115, 118, 121, 125, 128, 132, 136,  # LI 30-39
    140, 145, 150, 155, 160, 165, 170, 175, 180, 185,  # LI 40-49
    190, 195, 200, 206, 212, 218, 224, 230, 236, 243,  # LI 50-59
    250, 257, 265, 272, 280, 290, 300, 307, 315, 325,  # LI 60-69
    335, 345, 355, 365, 375, 387, 400, 412, 425, 437,  # LI 70-79
    450, 462, 475, 487, 500, 515, 530, 545, 560, 580,  # LI 80-89
    600, 615, 630, 650, 670, 690, 710, 730, 750, 775,  # LI 90-99
    800, 825, 850, 875, 900, 925, 950, 975, 1000, 1030,  # LI 100-109
    1060, 1090, 1120, 1150, 1180, 1215, 1250, 1285, 1320, 1360,  # LI 110-119
    1400, 1450, 1500, 1550, 1600, 1650, 1700, 1750, 1800, 1850,  # LI 120-129
    1900, 1950, 2000, 2060, 2120, 2180, 2240, 2300, 2360, 2430,  # LI 130-139
    2500, 2575, 2650, 2725, 2800, 2900, 3000, 3075, 3150, 3250,  # LI 140-149
    3350, 3450, 3550, 3650, 3750, 3875, 4000, 4125, 4250, 4375,  # LI 150-159
    4500, 4625, 4750, 4875, 5000, 5150, 5300, 5450, 5600, 5850,  # LI 160-169
    6000, 6150, 6300, 6500, 6700, 6900, 7100, 7300, 7500, 7750,  # LI 170-179
    8000, 8250, 8500, 8750, 9000, 9250, 9500, 9750, 10000, 10300,  # LI 180-189
    10600, 10900, 11200, 11500, 11800, 12150, 12500, 12850, 13200, 13600,  # LI 190-199
    14000, 14500, 15000, 15550, 16000, 16500, 17000, 17500, 18000, 18500,  # LI 200-209
    19000, 19500, 20000, 20600, 21200, 21800, 22400, 23000, 23600, 24300,  # LI 210-219
    25000, 25750, 26500, 27250, 28000, 29000, 30000, 30750, 31500, 32500,  # LI 220-229
    33500, 34500, 35500, 36500, 37500, 38750, 40000, 41250, 42500, 43750,  # LI 230-239
    45000, 46250, 47500, 48750, 50000, 51500, 53000, 54500, 56000, 58000,  # LI 240-249
    60000, 61500, 63000, 65000, 67000, 69000, 71000, 73000, 75000, 77500,  # LI 250-259
    80000, 82500, 85000, 87500, 90000, 92500, 95000, 97500, 100000, 103000,  # LI 260-269
    106000, 109000, 112000, 115000, 118000, 121000, 125000, 128500, 132000, 136000,  # LI 270-279
)

# Load-normalised TMeasy curve parameters of GuessPassCar70Par and GuessTruck80Par
# (18dof-gpu/dof18_gpu.cu:1516-1615), data of the TMeasy model: (dfx0Pn, dfx0P2n, fxmPn, fxmP2n,
# fxsPn, fxsP2n, dfy0Pn, dfy0P2n, fymPn, fymP2n, fysPn, fysP2n) as multiples of pn (the P2n entries
# of 2 pn), then the slips (sxmPn, sxmP2n, sxsPn, sxsP2n, symPn, symP2n, sysPn, sysP2n).
_GUESS = {
    "Passenger": ((18.3741, 19.4669, 1.1292, 1.0896, 0.80149, 0.76917, 15.9826, 12.8509, 1.0009, 0.91367, 0.8336,
                   0.77336), (0.13913, 0.13913, 0.66667, 0.66667, 0.14852, 0.18504, 0.96524, 1.0714)),
    "Truck": ((17.7764, 14.5301, 0.89965, 0.77751, 0.46183, 0.42349, 7.4013, 6.8505, 0.75876, 0.72628, 0.68276,
               0.65319), (0.10811, 0.12389, 0.66667, 0.66667, 0.33167, 0.33216, 1.0296, 1.0296)),
}
_GUESS_FORCE_KEYS = ("dfx0pn", "dfx0p2n", "fxmpn", "fxmp2n", "fxspn", "fxsp2n", "dfy0pn", "dfy0p2n", "fympn",
                     "fymp2n", "fyspn", "fysp2n")
_GUESS_SLIP_KEYS = ("sxmpn", "sxmp2n", "sxspn", "sxsp2n", "sympn", "symp2n", "syspn", "sysp2n")


def _tmeasy_nr_params(t: dict, p: np.ndarray, model: int) -> None:
    """setTireParamsJSON for a TMeasyNr tire (18dof-gpu/dof18_gpu.cu:1278-1466; the 24-DOF loader is
    the same, 24dof-gpu/dof24_gpu.cu:1847-2070; the 11-DOF one, 11dof-gpu/dof11_gpu.cu:1101-1290,
    doubles the axle quantities). Low-level files give the curve parameters; with
    "highLevelParams": true they are guessed from the tire's size and load capacity (load index or
    maximum bearing capacity) for a passenger car or a truck tire."""
    two = 2.0 if model == 11 else 1.0
    if bool(t.get("highLevelParams", False)):
        p[P["jw"]] = float(t["jw"]) * two
        p[P["rr"]] = float(t["rr"]) * two
        p[P["mu"]] = float(t["mu"]) * two
        p[P["r0"]] = float(t["r0"])
        p[P["rdyncopn"]] = float(t["rdyncoPn"])
        p[P["rdyncop2n"]] = float(t["rdyncoP2n"])
        p[P["fzrdynco"]] = float(t["fzRdynco"]) * two
        p[P["rdyncocrit"]] = float(t["rdyncoCrit"]) * two
        p[P["vcoulomb"]] = float(t["vCoulomb"]) if "vCoulomb" in t else 1.0
        p[P["frblend_begin"]] = float(t["frblendBegin"]) if "frblendBegin" in t else 1.0
        p[P["frblend_end"]] = float(t["frblendEnd"]) if "frblendEnd" in t else 3.0
        width = float(t["width"])
        rim_radius = float(t["rimRadius"])
        p_li = float(t["inflationPressureDesign"]) if "inflationPressureDesign" in t else 0.0
        p_use = float(t["inflationPressureUse"]) if "inflationPressureUse" in t else 0.0
        if not (p_use > 0.0 and p_li > 0.0):
            p_li = p_use = 1.0
        p[P["p_li"]], p[P["p_use"]] = p_li, p_use
        if "loadIndex" in t:
            li = int(t["loadIndex"])
            p[P["li"]] = li
            load = _LOAD_INDEX_KG[min(li, len(_LOAD_INDEX_KG) - 1)] * 9.81
        else:
            load = float(t["maximumBearingCapacity"])
            p[P["bearingcapacity"]] = load
        kind = "Truck" if t["vehicleType"] == "Truck" else "Passenger"
        forces, slips = _GUESS[kind]
        # GuessPassCar70Par / GuessTruck80Par with ratio = (r0 - rim radius) / width and rim diameter
        # 2 rim radius: section height width * ratio, deflection at the rated load 0.16 of it
        ratio = (p[P["r0"]] - rim_radius) / width
        defl_max = 0.16 * (width * ratio)
        pn = 0.5 * load * (p_use / p_li) ** 0.8
        p[P["pn"]] = pn
        p[P["pnmax"]] = 3.5 * pn
        p[P["kt"]] = load / defl_max
        p[P["rim_radius"]] = 0.5 * (2 * rim_radius)
        p[P["width"]] = width
        for i, (k, c) in enumerate(zip(_GUESS_FORCE_KEYS, forces)):
            # the P2n entries are c * 2 * pn, evaluated as (c * 2.0) * pn
            p[P[k]] = ((c * 2.0) * pn if i % 2 else c * pn) * two
        for k, c in zip(_GUESS_SLIP_KEYS, slips):
            p[P[k]] = c
    else:
        for k in _TM_KEYS:
            if k in ("cx", "cy", "dx", "dy"):
                continue
            p[P[k.lower()]] = float(t[k])
        if model == 11:
            for k in _DOUBLED_11:
                if k not in ("cx", "cy", "dx", "dy"):
                    p[P[k]] = float(t[_KEY_OF[k]]) * 2.0


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
