"""C ABI checks that need no GPU: exported symbols, struct layout, the library's JSON and driver-file
loaders against the pure-Python loaders, and loud failure without a device."""
import ctypes
import json
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import ROOT, TESTS, case_inputs, pkg_mod

HEADER = os.path.join(ROOT, "include", "lfdm.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(lfdm_\w+)\s*\(", text)))


def test_every_declared_symbol_is_exported(built_lib):
    lib = built_lib.lib()
    names = declared_functions()
    assert len(names) >= 35
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_struct_layout_matches_header(tmp_path):
    abi = pkg_mod("_abi")
    src = tmp_path / "sz.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "%s"\nint main(void){printf("%%zu %%zu %%zu\\n",'
                   'sizeof(lfdm_class18), offsetof(lfdm_class18, gearRatios), offsetof(lfdm_class18, TRmap));'
                   'return 0;}\n' % HEADER)
    exe = tmp_path / "sz"
    subprocess.run(["gcc", "-o", str(exe), str(src)], check=True)
    size, off_g, off_tr = map(int, subprocess.run([str(exe)], capture_output=True, text=True).stdout.split())
    assert ctypes.sizeof(abi.Class18) == size
    assert abi.Class18.gearRatios.offset == off_g
    assert abi.Class18.TRmap.offset == off_tr
    assert abi.P_COUNT == 67 and abi.S_COUNT == 75 and abi.RESP18 == 13


def _write(tmp, name, obj):
    p = os.path.join(tmp, name)
    with open(p, "w") as f:
        if isinstance(obj, str):
            f.write(obj)
        else:
            json.dump(obj, f)
    return p


def test_cpp_loader_matches_python_loader(built_lib, golden18):
    params = pkg_mod("params")
    seen = set()
    with tempfile.TemporaryDirectory() as tmp:
        for case in golden18["cases"]:
            key = case["source"].split(",")[0]
            if key in seen:
                continue
            seen.add(key)
            vj = _write(tmp, "v.json", case["vehicle"])
            tj = _write(tmp, "t.json", case["tire"])
            c_cls, c_p = built_lib.parse_vehicle18(vj, tj, case["tire_type"])
            py_cls, py_p = params.vehicle_from_json(case["vehicle"], case["tire"], case["tire_type"])
            assert np.array_equal(c_p, py_p)
            assert bytes(c_cls) == bytes(py_cls)
    assert len(seen) >= 2


@pytest.mark.parametrize("model", [11, 24])
def test_cpp_loader_matches_python_loader_11_24(built_lib, model):
    """The library's 11- and 24-DOF loaders (tire doubling, jy, suspension file, TMeasyNr high-level
    parameters) against the Python loader, on every distinct vehicle of the model's golden fixtures."""
    params = pkg_mod("params")
    with open(os.path.join(TESTS, "golden", f"golden{model}.json")) as f:
        cases = json.load(f)["cases"]
    seen = set()
    with tempfile.TemporaryDirectory() as tmp:
        for case in cases:
            key = json.dumps([case["vehicle"], case["tire"], case.get("sus")], sort_keys=True)
            if key in seen:
                continue
            seen.add(key)
            vj = _write(tmp, "v.json", case["vehicle"])
            tj = _write(tmp, "t.json", case["tire"])
            sj = _write(tmp, "s.json", case["sus"]) if model == 24 else None
            c_cls, c_p = built_lib.parse_vehicle(model, vj, tj, sj, case["tire_type"])
            py_cls, py_p = params.vehicle_from_json(case["vehicle"], case["tire"], case["tire_type"], model=model,
                                                    sus=case.get("sus"))
            assert np.array_equal(c_p, py_p), np.nonzero(c_p != py_p)
            assert bytes(c_cls) == bytes(py_cls)
    assert len(seen) >= 2


def test_loader_errors(built_lib):
    with tempfile.TemporaryDirectory() as tmp:
        good_v = pkg_mod("fleet").SUV18_VEHICLE
        good_t = pkg_mod("fleet").SUV_TIRE
        vj = _write(tmp, "v.json", good_v)
        tj = _write(tmp, "t.json", good_t)
        with pytest.raises(built_lib.LfdmError) as e:
            built_lib.parse_vehicle18(os.path.join(tmp, "missing.json"), tj)
        assert e.value.code == 2  # LFDM_ERR_IO
        bad = _write(tmp, "bad.json", '{"a": 1.0, ')
        with pytest.raises(built_lib.LfdmError) as e:
            built_lib.parse_vehicle18(bad, tj)
        assert e.value.code == 3  # LFDM_ERR_PARSE
        v2 = dict(good_v)
        del v2["jz"]
        with pytest.raises(built_lib.LfdmError) as e:
            built_lib.parse_vehicle18(_write(tmp, "v2.json", v2), tj)
        assert "jz" in str(e.value)
        long_map = dict(good_v, torqueMap=[[float(i), 1.0] for i in range(40)])
        with pytest.raises(built_lib.LfdmError):
            built_lib.parse_vehicle18(_write(tmp, "v3.json", long_map), tj)


def test_driver_file_parse_stop(built_lib):
    params = pkg_mod("params")
    text = "0 0 0 0\n0.5\t0 0.2 0\n1.0 0.1 0.4 0   extra\n\n2.0 0 0 0\n"
    with tempfile.TemporaryDirectory() as tmp:
        p = _write(tmp, "d.txt", text)
        rows = built_lib.load_driver_file(p)
        ref = params.load_driver_table(text, is_text=True)
        assert rows.shape == (3, 4)  # parsing stops at the empty line (utils_gpu.cu:17-25)
        assert np.array_equal(rows, ref)
        with pytest.raises(built_lib.LfdmError):
            built_lib.load_driver_file(_write(tmp, "e.txt", "time steering\n"))


def test_create_without_device_fails_loudly(built_lib):
    """No silent CPU fallback: on a machine without a CUDA device the solver refuses to exist."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    with pytest.raises(built_lib.LfdmError) as e:
        built_lib.d18SolverHalfImplicitGPU(4)
    assert e.value.code == 8  # LFDM_ERR_NODEVICE


def test_fleet_generator_is_seeded():
    fleet = pkg_mod("fleet")
    a = fleet.fleet18(16, seed=3, horizon=2.0)
    b = fleet.fleet18(16, seed=3, horizon=2.0)
    for k in ("params", "tables", "states"):
        assert np.array_equal(a[k], b[k])
    P = pkg_mod("_abi").P
    base = fleet.suv18()[1]
    r = a["params"][:, P["m"]] / base[P["m"]]
    assert (r >= 0.9).all() and (r <= 1.1).all()
    assert np.allclose(a["params"][:, P["a"]] + a["params"][:, P["b"]], base[P["a"]] + base[P["b"]])
    assert a["tables"].shape == (16, 201, 4)
