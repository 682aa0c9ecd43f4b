"""ctypes mirror of include/lfdm.h (layouts, enums, the lfdm_class18 struct).

The numeric constants are parsed from the header itself so that the Python side cannot drift
from the C ABI; `tests/test_abi.py` checks the struct layout against the header's sizes.
"""
from __future__ import annotations

import ctypes
import os
import re

_HERE = os.path.dirname(os.path.abspath(__file__))
HEADER = os.path.join(os.path.dirname(_HERE), "include", "lfdm.h")


def _parse_enums(text: str) -> dict[str, int]:
    """Evaluate the `enum { A = 0, B, ... }` blocks and `#define NAME <int>` lines of the header."""
    out: dict[str, int] = {}
    for m in re.finditer(r"#define\s+(LFDM\w*)\s+(\d+)\b", text):
        out[m.group(1)] = int(m.group(2))
    for body in re.findall(r"enum\s*\w*\s*\{(.*?)\}", text, flags=re.S):
        body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
        nxt = 0
        for item in body.split(","):
            item = item.strip()
            if not item:
                continue
            if "=" in item:
                name, expr = (s.strip() for s in item.split("=", 1))
                val = eval(expr, {}, dict(out))  # expressions are sums of earlier names / ints
            else:
                name, val = item, nxt
            out[name] = int(val)
            nxt = int(val) + 1
    return out


with open(HEADER, "r", encoding="utf-8") as _f:
    C = _parse_enums(_f.read())

P_COUNT = C["LFDM_P_COUNT"]
S_COUNT = C["LFDM_S_COUNT"]
MAX_MAP = C["LFDM_MAX_MAP"]
MAX_GEARS = C["LFDM_MAX_GEARS"]
RESP18 = C["LFDM18_RESP_CHANNELS"]
S_TIRE0 = C["LFDM_S_TIRE0"]
S_TIRE_STRIDE = C["LFDM_S_TIRE_STRIDE"]
S11_COUNT = C["LFDM11_S_COUNT"]
S11_TIRE0 = C["LFDM11_S_TIRE0"]
RESP11 = C["LFDM11_RESP_CHANNELS"]
S24_COUNT = C["LFDM24_S_COUNT"]
RESP24 = C["LFDM24_RESP_CHANNELS"]

# name -> index maps, e.g. P["m"] == LFDM_P_M, S["x"] == LFDM_S_X, T["omega"] == LFDM_T_OMEGA
P = {k[len("LFDM_P_"):].lower(): v for k, v in C.items() if k.startswith("LFDM_P_") and k != "LFDM_P_COUNT"}
S = {k[len("LFDM_S_"):].lower(): v for k, v in C.items() if k.startswith("LFDM_S_") and k not in (
    "LFDM_S_COUNT", "LFDM_S_TIRE0", "LFDM_S_TIRE_STRIDE")}
T = {k[len("LFDM_T_"):].lower(): v for k, v in C.items() if k.startswith("LFDM_T_")}
S11 = {k[len("LFDM11_S_"):].lower(): v for k, v in C.items() if k.startswith("LFDM11_S_") and k not in (
    "LFDM11_S_COUNT", "LFDM11_S_TIRE0")}
S24 = {k[len("LFDM24_S_"):].lower(): v for k, v in C.items() if k.startswith("LFDM24_S_") and k not in (
    "LFDM24_S_COUNT", "LFDM24_S_TIRE0", "LFDM24_S_SUS0")}

TIRE_TMEASY = C["LFDM_TIRE_TMEASY"]
TIRE_TMEASY_NR = C["LFDM_TIRE_TMEASY_NR"]
PREC_FP64 = C["LFDM_PREC_FP64"]
PREC_MIXED = C["LFDM_PREC_MIXED"]
PREC_MIXED_TIRE = C["LFDM_PREC_MIXED_TIRE"]

STATUS = {v: k for k, v in C.items() if k.startswith("LFDM_OK") or k.startswith("LFDM_ERR_")}

_map = ctypes.c_double * 2 * MAX_MAP


class Class18(ctypes.Structure):
    """lfdm_class18: flags, gear ratios and maps shared by the vehicles of one class."""

    _fields_ = [
        ("nonLinearSteer", ctypes.c_int32),
        ("tcbool", ctypes.c_int32),
        ("throttleMod", ctypes.c_int32),
        ("driveType", ctypes.c_int32),
        ("whichWheels", ctypes.c_int32),
        ("noGears", ctypes.c_int32),
        ("steerMapSize", ctypes.c_int32),
        ("powertrainMapSize", ctypes.c_int32),
        ("lossesMapSize", ctypes.c_int32),
        ("CFmapSize", ctypes.c_int32),
        ("TRmapSize", ctypes.c_int32),
        ("pad_", ctypes.c_int32),
        ("gearRatios", ctypes.c_double * MAX_GEARS),
        ("shiftMap", ctypes.c_double * 2 * MAX_GEARS),
        ("steerMap", _map),
        ("powertrainMap", _map),
        ("lossesMap", _map),
        ("CFmap", _map),
        ("TRmap", _map),
    ]

    def set_map(self, name: str, points) -> None:
        pts = [(float(x), float(y)) for x, y in points]
        if len(pts) > MAX_MAP:
            raise ValueError(f"{name}: {len(pts)} points > LFDM_MAX_MAP={MAX_MAP}")
        arr = getattr(self, name)
        for i, (x, y) in enumerate(pts):
            arr[i][0] = x
            arr[i][1] = y
        size_field = {"steerMap": "steerMapSize", "powertrainMap": "powertrainMapSize",
                      "lossesMap": "lossesMapSize", "CFmap": "CFmapSize", "TRmap": "TRmapSize"}[name]
        setattr(self, size_field, len(pts))

    def get_map(self, name: str):
        size_field = {"steerMap": "steerMapSize", "powertrainMap": "powertrainMapSize",
                      "lossesMap": "lossesMapSize", "CFmap": "CFmapSize", "TRmap": "TRmapSize"}[name]
        arr = getattr(self, name)
        return [(arr[i][0], arr[i][1]) for i in range(getattr(self, size_field))]


def copy_class(c: Class18) -> Class18:
    out = Class18()
    ctypes.memmove(ctypes.byref(out), ctypes.byref(c), ctypes.sizeof(Class18))
    return out
