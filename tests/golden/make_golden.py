"""Generate tests/golden/golden18.json from the reference's own CPU 18-DOF solver.

Run where the reference checkout exists (it reads vehicle/tire JSON and driver tables from it):
    make -C oracle ref REF=<reference>/wheeled_vehicle_models
    python tests/golden/make_golden.py [<reference>/wheeled_vehicle_models]

Each case stores its complete inputs (vehicle and tire parameters re-serialised from the
reference's data files or from the seeded synthetic SUV fleet, the driver table rows, the
schedule and initial state) and the reference's outputs: sampled trajectories and the full final
state, printed with 17 significant digits. The oracle and the CUDA path are checked against these
values on machines that have no reference checkout.
"""
from __future__ import annotations

import importlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
lfdm = importlib.import_module("low-fidelity-dynamic-models_gb300")
from importlib import import_module  # noqa: E402

fleet = import_module("low-fidelity-dynamic-models_gb300.fleet")
abi = import_module("low-fidelity-dynamic-models_gb300._abi")

REFRUN = os.path.join(ROOT, "oracle", "_ref", "refrun18")
SEED = 20261203
# cases that also record the reference's IntegrateStepWithJacobian output at their final state (the
# first two vehicles of each synthetic fleet as well)
JAC_CASES = {"hmmwv_dl4_gpu", "sedan_nr_acc05_gpu", "hmmwv11_dl4_gpu", "sedan11_nr_acc05_gpu", "hmmwv24_dl4_gpu22",
             "sedan24_nr_acc05_gpu"}


def _fmt(x: float) -> str:
    return repr(float(x))


def parse_ref(stdout: str) -> list[dict]:
    """Rows of refrun{11,18,24}: S (samples), F (final state), with jac 1 also C (the controls of
    the Jacobian), JS and JC (the reference's state and control Jacobians, row-major); E ends a job."""
    results, cur = [], {"samples": []}
    for line in stdout.splitlines():
        tok = line.split()
        if not tok:
            continue
        if tok[0] == "S":
            cur["samples"].append([int(tok[1])] + [float(v) for v in tok[2:]])
        elif tok[0] == "F":
            cur["final"] = [float(v) for v in tok[1:]]
        elif tok[0] in ("C", "JS", "JC"):
            cur[tok[0]] = [float(v) for v in tok[1:]]
        elif tok[0] == "E":
            results.append(cur)
            cur = {"samples": []}
    return results


def run_ref(job_lines: list[str]) -> list[dict]:
    out = subprocess.run([REFRUN], input="\n".join(job_lines) + "\n", capture_output=True, text=True, check=True)
    return parse_ref(out.stdout)


def add_jacobian(case: dict, r: dict) -> None:
    """The reference's IntegrateStepWithJacobian output at the case's final state, if requested."""
    if "JS" not in r:
        return
    ny = int(round(len(r["JS"]) ** 0.5))
    assert ny * ny == len(r["JS"]) and len(r["JC"]) == 2 * ny
    case["jacobian"] = {"controls": r["C"], "state": r["JS"], "ny": ny, "control": r["JC"]}


def final_to_state(final: list[float]) -> list[float]:
    """refrun18 'F' row -> flat state vector (include/lfdm.h order)."""
    s = [0.0] * abi.S_COUNT
    s[:15] = final[:15]
    s[15:75] = final[15:75]
    return s


def _steer_map_for(max_steer: float) -> list:
    """The ART vehicle's steering map (18dof-gpu/data/json/ART/vehicle.json) rescaled so that full
    input gives the vehicle's own maximum wheel angle: a non-linear map for vehicles that ship
    without one. The angles are rounded to 9 significant digits: the reference's JSON reader
    (rapidjson without its full-precision flag) can round a 17-digit decimal to a neighbouring
    double, which the reference data files, written with few digits, never meet."""
    art = [(-1, -0.383972), (-0.8, -0.301942), (-0.6, -0.2199115), (-0.4, -0.151844), (-0.2, -0.0314159), (0, 0),
           (0.2, 0.0314159), (0.4, 0.151844), (0.6, 0.2199115), (0.8, 0.301942), (1, 0.383972)]
    return [[x, float(f"{y * max_steer / 0.383972:.9g}")] for x, y in art]


def fixture_cases(data: str, model: int) -> list:
    """Branch fixtures of one model from the reference's data files under `data` (<model>dof-gpu/data):
    (name, vehicle, tire, tire type, driver file, ksim, tend, source). They cover the steering map
    (vehToTireTransform's getMapY branch), throttleMod (driveTorque's scaled map), the 2WD torque split
    to the rear or the front axle in computePowertrainRHS, and vehicles without a torque converter."""
    j = lambda *p: json.load(open(os.path.join(data, "json", *p)))  # noqa: E731
    out = []
    pre = {18: "", 11: "11", 24: "24"}[model]
    if model in (18, 11):
        art_v, art_t = j("ART", "vehicle.json"), j("ART", "tmeasy.json")
        out += [(f"art{pre}_ls5_gpu", art_v, art_t, 0, "long_sine5", 2.0, 20.0, "ART vehicle.json + tmeasy.json"),
                (f"art{pre}_dl4_cpu", art_v, art_t, 0, "double_lane4", 0.0, None, "ART vehicle.json + tmeasy.json")]
        audi_v, audi_rwd, audi_t = j("audi", "vehicle.json"), j("audi", "vehicle_RWD.json"), j("audi", "tmeasy.json")
        audi_fwd = dict(audi_rwd, rearWheels=False)
        out += [(f"audi{pre}_dl4_gpu", audi_v, audi_t, 0, "double_lane4", 2.0, 22.0, "audi vehicle.json + tmeasy.json"),
                (f"audi{pre}_rwd_ls5_gpu", audi_rwd, audi_t, 0, "long_sine5", 1.0, 20.0,
                 "audi vehicle_RWD.json + tmeasy.json"),
                (f"audi{pre}_rwd_st3_cpu", audi_rwd, audi_t, 0, "st3_right", 0.0, None,
                 "audi vehicle_RWD.json + tmeasy.json"),
                (f"audi{pre}_fwd_ls5_gpu", audi_fwd, audi_t, 0, "long_sine5", 2.0, 20.0,
                 "audi vehicle_RWD.json with rearWheels false (front-wheel drive) + tmeasy.json")]
    sedan_v = j("Sedan", "vehicle.json")
    # 24dof-gpu/data/json/Sedan/vehicle_RWD.json is an 18-DOF file (no "jy"; the reference's 24-DOF
    # loader reads d["jy"] unconditionally, 24dof-gpu/dof24_gpu.cu:2237), so the 24-DOF rear-wheel-drive
    # Sedan is the 24-DOF vehicle.json with "4wd" false
    sedan_rwd = j("Sedan", "vehicle_RWD.json") if model != 24 else dict(sedan_v, **{"4wd": False})
    sedan_t, sedan_nr = j("Sedan", "tmeasy.json"), j("Sedan", "tmeasyNr.json")
    out += [(f"sedan{pre}_rwd_ls5_gpu", sedan_rwd, sedan_t, 0, "long_sine5", 2.0, 20.0,
             "Sedan vehicle_RWD.json + tmeasy.json"),
            (f"sedan{pre}_rwd_nr_acc05_gpu", sedan_rwd, sedan_nr, 1, "acc05", 2.0, 10.0,
             "Sedan vehicle_RWD.json + tmeasyNr.json")]
    hm = j("HMMWV", "vehicle.json")
    hm_mod = dict(hm, throttleMod=True, nonLinearSteer=True, steerMap=_steer_map_for(hm["maxSteer"]))
    out += [(f"hmmwv{pre}_tmod_nls_ls5_gpu", hm_mod, j("HMMWV", "tmeasy.json"), 0, "long_sine5", 2.0, 20.0,
             "HMMWV vehicle.json with throttleMod and a steering map + tmeasy.json")]
    sedan_mod = dict(sedan_v, throttleMod=True, nonLinearSteer=True, steerMap=_steer_map_for(sedan_v["maxSteer"]))
    out += [(f"sedan{pre}_tmod_nls_nr_dl4_gpu", sedan_mod, sedan_nr, 1, "double_lane4", 2.0, 22.0,
             "Sedan vehicle.json with throttleMod and a steering map + tmeasyNr.json")]
    if model == 24:
        out += [("sedan24_tm_dl4_gpu", sedan_v, sedan_t, 0, "double_lane4", 2.0, 22.0, "Sedan vehicle.json + tmeasy.json"),
                ("sedan24_rwd_st3_cpu", sedan_rwd, sedan_t, 0, "st3_right", 0.0, None,
                 "Sedan vehicle.json with 4wd false + tmeasy.json"),
                ("sedan24_fwd_ls5_gpu", dict(sedan_rwd, rearWheels=False), sedan_t, 0, "long_sine5", 2.0, 20.0,
                 "Sedan vehicle.json with 4wd and rearWheels false (front-wheel drive) + tmeasy.json")]
    return out


def main(ref: str) -> None:
    d18 = os.path.join(ref, "18dof-gpu", "data")
    veh_hmmwv = json.load(open(os.path.join(d18, "json", "HMMWV", "vehicle.json")))
    tire_hmmwv = json.load(open(os.path.join(d18, "json", "HMMWV", "tmeasy.json")))
    cases = []
    with tempfile.TemporaryDirectory() as tmp:
        def write_json(name, obj):
            p = os.path.join(tmp, name)
            with open(p, "w") as f:
                json.dump(obj, f)
            return p

        def write_table(name, rows):
            p = os.path.join(tmp, name)
            with open(p, "w") as f:
                for r in rows:
                    f.write(" ".join(_fmt(v) for v in r) + "\n")
            return p

        vj, tj = write_json("hmmwv_vehicle.json", veh_hmmwv), write_json("hmmwv_tmeasy.json", tire_hmmwv)
        named = [
            ("hmmwv_acc3_cpu", "acc3", 0.0, None, 100),
            ("hmmwv_acc3_gpu", "acc3", 2.0, 10.0, 100),
            ("hmmwv_dl4_gpu", "double_lane4", 2.0, 22.0, 100),
            ("hmmwv_st3_gpu", "st3_right", 2.0, None, 100),
        ]
        jobs, meta = [], []
        for name, drv, ksim, tend, sample in named:
            rows = lfdm.params.load_driver_table(os.path.join(d18, "input", drv + ".txt")).tolist()
            tp = write_table(f"{name}.txt", rows)
            tend_v = tend if tend is not None else rows[-1][0]
            jobs += [f"veh {vj}", f"tire {tj}", "tiretype 0", f"driver {tp}", "dt 0.001", f"tend {_fmt(tend_v)}",
                     f"ksim {_fmt(ksim)}", f"sample {sample}", f"jac {int(name in JAC_CASES)}", "run"]
            meta.append({"name": name, "vehicle": veh_hmmwv, "tire": tire_hmmwv, "tire_type": 0, "driver": rows,
                         "dt": 0.001, "tend": tend_v, "ksim": ksim, "sample": sample, "vp": {}, "tp": {},
                         "state": [0.0] * abi.S_COUNT, "source": f"HMMWV vehicle.json + tmeasy.json, {drv}.txt"})
        # TMeasyNr: the reference's Sedan files (high-level tire parameters, load index 97) on acc05,
        # the case of the reference test dof18HiNr (tests/18dof.cpp), under both schedules
        veh_sedan = json.load(open(os.path.join(d18, "json", "Sedan", "vehicle.json")))
        tire_sedan = json.load(open(os.path.join(d18, "json", "Sedan", "tmeasyNr.json")))
        vsj, tsj = write_json("sedan_vehicle.json", veh_sedan), write_json("sedan_tmeasyNr.json", tire_sedan)
        for name, ksim, tend in (("sedan_nr_acc05_cpu", 0.0, None), ("sedan_nr_acc05_gpu", 2.0, 10.0)):
            rows = lfdm.params.load_driver_table(os.path.join(d18, "input", "acc05.txt")).tolist()
            tp = write_table(f"{name}.txt", rows)
            tend_v = tend if tend is not None else rows[-1][0]
            jobs += [f"veh {vsj}", f"tire {tsj}", "tiretype 1", f"driver {tp}", "dt 0.001", f"tend {_fmt(tend_v)}",
                     f"ksim {_fmt(ksim)}", "sample 100", f"jac {int(name in JAC_CASES)}", "run"]
            meta.append({"name": name, "vehicle": veh_sedan, "tire": tire_sedan, "tire_type": 1, "driver": rows,
                         "dt": 0.001, "tend": tend_v, "ksim": ksim, "sample": 100, "vp": {}, "tp": {},
                         "state": [0.0] * abi.S_COUNT, "source": "Sedan vehicle.json + tmeasyNr.json, acc05.txt"})
        P = abi.P
        vfields = ["m", "jz", "a", "b"]
        tfields = ["kt"] + list(fleet.FRICTION_FIELDS)
        key = {"fxmpn": "fxmPn", "fxmp2n": "fxmP2n", "fxspn": "fxsPn", "fxsp2n": "fxsP2n", "fympn": "fymPn",
               "fymp2n": "fymP2n", "fyspn": "fysPn", "fysp2n": "fysP2n", "kt": "kt"}
        # Branch fixtures: the reference's ART (steering map, throttleMod, no converter, one gear),
        # Sedan and audi rear-wheel-drive files (2WD torque split) and audi 4WD files, plus the HMMWV
        # with throttleMod and a steering map switched on (the branches with a torque converter).
        for name, veh, tire, tt, drv, ksim, tend, src in fixture_cases(d18, 18):
            rows = lfdm.params.load_driver_table(os.path.join(d18, "input", drv + ".txt")).tolist()
            tp = write_table(f"{name}.txt", rows)
            vjx, tjx = write_json(f"{name}_v.json", veh), write_json(f"{name}_t.json", tire)
            tend_v = tend if tend is not None else rows[-1][0]
            jobs += [f"veh {vjx}", f"tire {tjx}", f"tiretype {tt}", f"driver {tp}", "dt 0.001",
                     f"tend {_fmt(tend_v)}", f"ksim {_fmt(ksim)}", "sample 100", "jac 0", "run"]
            meta.append({"name": name, "vehicle": veh, "tire": tire, "tire_type": tt, "driver": rows, "dt": 0.001,
                         "tend": tend_v, "ksim": ksim, "sample": 100, "vp": {}, "tp": {},
                         "state": [0.0] * abi.S_COUNT, "source": src + f", {drv}.txt"})
        # the calm companion fleet (rounding-insensitive over the whole horizon)
        n_calm = 6
        fc = fleet.fleet18_calm(n_calm, horizon=10.0)
        cvj = write_json("calm_vehicle.json", fleet.SUV18_VEHICLE)
        calm_tire = dict(fleet.SUV_TIRE, jw=fleet.CALM_JW)
        ctj = write_json("calm_tire.json", calm_tire)
        for i in range(n_calm):
            rows = fc["tables"][i].tolist()
            tp = write_table(f"calm_{i}.txt", rows)
            vp = {k: float(fc["params"][i, P[k]]) for k in vfields}
            vp["maxBrakeTorque"] = float(fc["params"][i, P["maxbraketorque"]])
            tpv = {key[k]: float(fc["params"][i, P[k]]) for k in tfields}
            st = fc["states"][i]
            lines = [f"veh {cvj}", f"tire {ctj}", "tiretype 0", f"driver {tp}", "dt 0.001", "tend 10",
                     "ksim 1", "sample 250"]
            lines += [f"vp {k} {_fmt(v)}" for k, v in vp.items()] + [f"tp {k} {_fmt(v)}" for k, v in tpv.items()]
            lines += [f"vs u {_fmt(st[abi.S['u']])}", f"vs crankOmega {_fmt(st[abi.S['crankomega']])}",
                      f"gear {int(st[abi.S['current_gr']])}"]
            lines += [f"ts {k} omega {_fmt(st[abi.S_TIRE0 + abi.T['omega']])}" for k in range(4)] + ["jac 0", "run"]
            jobs += lines
            meta.append({"name": f"calm_fleet_{i}", "vehicle": fleet.SUV18_VEHICLE, "tire": calm_tire,
                         "tire_type": 0, "driver": rows, "dt": 0.001, "tend": 10.0, "ksim": 1.0, "sample": 250,
                         "vp": vp, "tp": tpv, "state": st.tolist(),
                         "source": f"calm synthetic SUV fleet seed {fc['seed']} vehicle {i}"})
        # seeded synthetic SUV fleet (GPU schedule, 1 s windows)
        n_syn = 12
        fl = fleet.fleet18(n_syn, seed=SEED, horizon=10.0)
        sj, stj = write_json("suv_vehicle.json", fleet.SUV18_VEHICLE), write_json("suv_tire.json", fleet.SUV_TIRE)
        for i in range(n_syn):
            rows = fl["tables"][i].tolist()
            tp = write_table(f"suv_{i}.txt", rows)
            vp = {k: float(fl["params"][i, P[k]]) for k in vfields}
            tpv = {key[k]: float(fl["params"][i, P[k]]) for k in tfields}
            st = fl["states"][i]
            u0 = float(st[abi.S["u"]])
            w0 = float(st[abi.S_TIRE0 + abi.T["omega"]])
            crank = float(st[abi.S["crankomega"]])
            gear = int(st[abi.S["current_gr"]])
            lines = [f"veh {sj}", f"tire {stj}", "tiretype 0", f"driver {tp}", "dt 0.001", "tend 10",
                     "ksim 1", "sample 250"]
            lines += [f"vp {k} {_fmt(v)}" for k, v in vp.items()] + [f"tp {k} {_fmt(v)}" for k, v in tpv.items()]
            lines += [f"vs u {_fmt(u0)}", f"vs crankOmega {_fmt(crank)}", f"gear {gear}"]
            lines += [f"ts {k} omega {_fmt(w0)}" for k in range(4)] + [f"jac {int(i < 2)}", "run"]
            jobs += lines
            meta.append({"name": f"suv_fleet_{i}", "vehicle": fleet.SUV18_VEHICLE, "tire": fleet.SUV_TIRE,
                         "tire_type": 0, "driver": rows, "dt": 0.001, "tend": 10.0, "ksim": 1.0, "sample": 250,
                         "vp": vp, "tp": tpv, "state": st.tolist(),
                         "source": f"synthetic SUV fleet seed {SEED} vehicle {i}"})
        results = run_ref(jobs)
    assert len(results) == len(meta)
    for m, r in zip(meta, results):
        m["expected_samples"] = r["samples"]
        m["expected_final"] = final_to_state(r["final"])
        add_jacobian(m, r)
        cases.append(m)
    out = {"generator": "tests/golden/make_golden.py", "reference_solver": "d18SolverHalfImplicit (CPU), "
           "replayed step by step through IntegrateStep; ksim>0 uses the GPU solver's window schedule",
           "cases": cases}
    with open(os.path.join(HERE, "golden18.json"), "w") as f:
        json.dump(out, f, separators=(",", ":"))
    print(f"wrote {len(cases)} cases; e.g. {cases[0]['name']} x={cases[0]['expected_final'][0]!r}")


def main11(ref: str) -> None:
    """golden11.json: the reference's 11-DOF CPU solver (oracle/refrun11.cpp) on HMMWV fixtures and on
    seeded 11-DOF SUV vehicles (one shared parameter set, as in the 11-DOF fleet)."""
    refrun = os.path.join(ROOT, "oracle", "_ref", "refrun11")
    d11 = os.path.join(ref, "11dof-gpu", "data")
    veh = json.load(open(os.path.join(d11, "json", "HMMWV", "vehicle.json")))
    tire = json.load(open(os.path.join(d11, "json", "HMMWV", "tmeasy.json")))
    cases, jobs = [], []
    S11 = {k: abi.C[f"LFDM11_S_{k.upper()}"] for k in ("u", "crankomega", "current_gr")}
    with tempfile.TemporaryDirectory() as tmp:
        def write(name, text):
            p = os.path.join(tmp, name)
            with open(p, "w") as f:
                f.write(text)
            return p

        vj, tj = write("v.json", json.dumps(veh)), write("t.json", json.dumps(tire))
        for name, drv, ksim, tend in (("hmmwv11_acc3_cpu", "acc3", 0.0, None), ("hmmwv11_acc3_gpu22", "acc3", 2.0, 22.0),
                                      ("hmmwv11_dl4_gpu", "double_lane4", 2.0, 22.0)):
            rows = lfdm.params.load_driver_table(os.path.join(d11, "input", drv + ".txt")).tolist()
            tp = write(f"{name}.txt", "".join(" ".join(_fmt(v) for v in r) + "\n" for r in rows))
            tend_v = tend if tend is not None else rows[-1][0]
            jobs += [f"veh {vj}", f"tire {tj}", "tiretype 0", f"driver {tp}", "dt 0.001", f"tend {_fmt(tend_v)}",
                     f"ksim {_fmt(ksim)}", "sample 100", f"jac {int(name in JAC_CASES)}", "run"]
            cases.append({"name": name, "vehicle": veh, "tire": tire, "tire_type": 0, "driver": rows, "dt": 0.001,
                          "tend": tend_v, "ksim": ksim, "sample": 100, "vp": {}, "tp": {},
                          "state": [0.0] * abi.C["LFDM11_S_COUNT"], "source": f"HMMWV 11-DOF json, {drv}.txt"})
        # TMeasyNr: Sedan files on acc05 (reference test dof11HiNr, tests/11dof.cpp)
        veh_s = json.load(open(os.path.join(d11, "json", "Sedan", "vehicle.json")))
        tire_s = json.load(open(os.path.join(d11, "json", "Sedan", "tmeasyNr.json")))
        vsj, tsj = write("sv_sedan.json", json.dumps(veh_s)), write("st_sedan.json", json.dumps(tire_s))
        for name, ksim, tend in (("sedan11_nr_acc05_cpu", 0.0, None), ("sedan11_nr_acc05_gpu", 2.0, 10.0)):
            rows = lfdm.params.load_driver_table(os.path.join(d11, "input", "acc05.txt")).tolist()
            tp = write(f"{name}.txt", "".join(" ".join(_fmt(v) for v in r) + "\n" for r in rows))
            tend_v = tend if tend is not None else rows[-1][0]
            jobs += [f"veh {vsj}", f"tire {tsj}", "tiretype 1", f"driver {tp}", "dt 0.001", f"tend {_fmt(tend_v)}",
                     f"ksim {_fmt(ksim)}", "sample 100", f"jac {int(name in JAC_CASES)}", "run"]
            cases.append({"name": name, "vehicle": veh_s, "tire": tire_s, "tire_type": 1, "driver": rows, "dt": 0.001,
                          "tend": tend_v, "ksim": ksim, "sample": 100, "vp": {}, "tp": {},
                          "state": [0.0] * abi.C["LFDM11_S_COUNT"], "source": "Sedan 11-DOF json, tmeasyNr, acc05.txt"})
        for name, v, t, tt, drv, ksim, tend, src in fixture_cases(d11, 11):
            rows = lfdm.params.load_driver_table(os.path.join(d11, "input", drv + ".txt")).tolist()
            tp = write(f"{name}.txt", "".join(" ".join(_fmt(x) for x in r) + "\n" for r in rows))
            vjx, tjx = write(f"{name}_v.json", json.dumps(v)), write(f"{name}_t.json", json.dumps(t))
            tend_v = tend if tend is not None else rows[-1][0]
            jobs += [f"veh {vjx}", f"tire {tjx}", f"tiretype {tt}", f"driver {tp}", "dt 0.001", f"tend {_fmt(tend_v)}",
                     f"ksim {_fmt(ksim)}", "sample 100", "jac 0", "run"]
            cases.append({"name": name, "vehicle": v, "tire": t, "tire_type": tt, "driver": rows, "dt": 0.001,
                          "tend": tend_v, "ksim": ksim, "sample": 100, "vp": {}, "tp": {},
                          "state": [0.0] * abi.C["LFDM11_S_COUNT"], "source": f"{src} (11-DOF files), {drv}.txt"})
        fl = fleet.fleet11(8, seed=SEED, horizon=10.0)
        sj, stj = write("sv.json", json.dumps(fleet.SUV11_VEHICLE)), write("st.json", json.dumps(fleet.SUV_TIRE))
        for i in range(8):
            rows = fl["tables"][i].tolist()
            tp = write(f"s{i}.txt", "".join(" ".join(_fmt(v) for v in r) + "\n" for r in rows))
            st = fl["states"][i]
            w0 = float(st[abi.C["LFDM11_S_TIRE0"] + abi.T["omega"]])
            jobs += [f"veh {sj}", f"tire {stj}", "tiretype 0", f"driver {tp}", "dt 0.001", "tend 10", "ksim 1",
                     "sample 250", f"vs u {_fmt(st[S11['u']])}", f"vs crankOmega {_fmt(st[S11['crankomega']])}",
                     f"gear {int(st[S11['current_gr']])}", f"ts 0 omega {_fmt(w0)}", f"ts 1 omega {_fmt(w0)}",
                     f"jac {int(i < 2)}", "run"]
            cases.append({"name": f"suv11_{i}", "vehicle": fleet.SUV11_VEHICLE, "tire": fleet.SUV_TIRE, "tire_type": 0,
                          "driver": rows, "dt": 0.001, "tend": 10.0, "ksim": 1.0, "sample": 250, "vp": {}, "tp": {},
                          "state": st.tolist(), "source": f"synthetic 11-DOF SUV fleet seed {SEED} vehicle {i}"})
        out = subprocess.run([refrun], input="\n".join(jobs) + "\n", capture_output=True, text=True, check=True)
    results = parse_ref(out.stdout)
    assert len(results) == len(cases)
    for c, r in zip(cases, results):
        c["expected_samples"] = r["samples"]
        c["expected_final"] = r["final"]
        add_jacobian(c, r)
    with open(os.path.join(HERE, "golden11.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py", "model": 11, "cases": cases}, f, separators=(",", ":"))
    print(f"wrote {len(cases)} 11-DOF cases; {cases[0]['name']} x={cases[0]['expected_final'][0]!r}")


def main24(ref: str) -> None:
    """golden24.json: the reference's 24-DOF CPU solver (oracle/refrun24.cpp) on HMMWV fixtures and on
    seeded 24-DOF SUV vehicles. Case states are the states after Initialize (initializeTireSus)."""
    refrun = os.path.join(ROOT, "oracle", "_ref", "refrun24")
    d24 = os.path.join(ref, "24dof-gpu", "data")
    veh = json.load(open(os.path.join(d24, "json", "HMMWV", "vehicle.json")))
    tire = json.load(open(os.path.join(d24, "json", "HMMWV", "tmeasy.json")))
    sus = json.load(open(os.path.join(d24, "json", "HMMWV", "suspension.json")))
    C = abi.C
    cases, jobs = [], []
    with tempfile.TemporaryDirectory() as tmp:
        def write(name, text):
            p = os.path.join(tmp, name)
            with open(p, "w") as f:
                f.write(text)
            return p

        vj, tj, sj = write("v.json", json.dumps(veh)), write("t.json", json.dumps(tire)), write("s.json", json.dumps(sus))
        _, p_h = lfdm.params.vehicle_from_json(veh, tire, 0, model=24, sus=sus)
        s_h = fleet.init_tire_sus24(p_h[None], np.zeros((1, C["LFDM24_S_COUNT"])))[0]
        for name, drv, ksim, tend in (("hmmwv24_acc3_cpu", "acc3", 0.0, None), ("hmmwv24_acc3_gpu22", "acc3", 2.0, 22.0),
                                      ("hmmwv24_dl4_gpu22", "double_lane4", 2.0, 22.0)):
            rows = lfdm.params.load_driver_table(os.path.join(d24, "input", drv + ".txt")).tolist()
            tp = write(f"{name}.txt", "".join(" ".join(_fmt(v) for v in r) + "\n" for r in rows))
            tend_v = tend if tend is not None else rows[-1][0]
            jobs += [f"veh {vj}", f"tire {tj}", f"sus {sj}", f"driver {tp}", "dt 0.001", f"tend {_fmt(tend_v)}",
                     f"ksim {_fmt(ksim)}", "sample 100", f"jac {int(name in JAC_CASES)}", "run"]
            cases.append({"name": name, "vehicle": veh, "tire": tire, "sus": sus, "tire_type": 0, "driver": rows,
                          "dt": 0.001, "tend": tend_v, "ksim": ksim, "sample": 100, "vp": {}, "tp": {},
                          "state": s_h.tolist(), "source": f"HMMWV 24-DOF json, {drv}.txt"})
        # TMeasyNr: Sedan vehicle and tire with the HMMWV suspension on acc05 (reference test dof24HiNr,
        # tests/24dof.cpp)
        veh_s = json.load(open(os.path.join(d24, "json", "Sedan", "vehicle.json")))
        tire_s = json.load(open(os.path.join(d24, "json", "Sedan", "tmeasyNr.json")))
        vsj, tsj = write("v_sedan.json", json.dumps(veh_s)), write("t_sedan.json", json.dumps(tire_s))
        _, p_s = lfdm.params.vehicle_from_json(veh_s, tire_s, 1, model=24, sus=sus)
        s_s = fleet.init_tire_sus24(p_s[None], np.zeros((1, C["LFDM24_S_COUNT"])))[0]
        for name, ksim, tend in (("sedan24_nr_acc05_cpu", 0.0, None), ("sedan24_nr_acc05_gpu", 2.0, 10.0)):
            rows = lfdm.params.load_driver_table(os.path.join(d24, "input", "acc05.txt")).tolist()
            tp = write(f"{name}.txt", "".join(" ".join(_fmt(v) for v in r) + "\n" for r in rows))
            tend_v = tend if tend is not None else rows[-1][0]
            jobs += [f"veh {vsj}", f"tire {tsj}", f"sus {sj}", "tiretype 1", f"driver {tp}", "dt 0.001",
                     f"tend {_fmt(tend_v)}", f"ksim {_fmt(ksim)}", "sample 100", f"jac {int(name in JAC_CASES)}", "run"]
            cases.append({"name": name, "vehicle": veh_s, "tire": tire_s, "sus": sus, "tire_type": 1, "driver": rows,
                          "dt": 0.001, "tend": tend_v, "ksim": ksim, "sample": 100, "vp": {}, "tp": {},
                          "state": s_s.tolist(), "source": "Sedan 24-DOF json, tmeasyNr, HMMWV suspension, acc05.txt"})
        sus_sedan = json.load(open(os.path.join(d24, "json", "Sedan", "suspension.json")))
        ssj_sedan = write("s_sedan.json", json.dumps(sus_sedan))
        for name, v, t, tt, drv, ksim, tend, src in fixture_cases(d24, 24):
            su, suj = (sus, sj) if name.startswith("hmmwv") else (sus_sedan, ssj_sedan)
            rows = lfdm.params.load_driver_table(os.path.join(d24, "input", drv + ".txt")).tolist()
            tp = write(f"{name}.txt", "".join(" ".join(_fmt(x) for x in r) + "\n" for r in rows))
            vjx, tjx = write(f"{name}_v.json", json.dumps(v)), write(f"{name}_t.json", json.dumps(t))
            _, p_c = lfdm.params.vehicle_from_json(v, t, tt, model=24, sus=su)
            s_c = fleet.init_tire_sus24(p_c[None], np.zeros((1, C["LFDM24_S_COUNT"])))[0]
            tend_v = tend if tend is not None else rows[-1][0]
            jobs += [f"veh {vjx}", f"tire {tjx}", f"sus {suj}", f"tiretype {tt}", f"driver {tp}", "dt 0.001",
                     f"tend {_fmt(tend_v)}", f"ksim {_fmt(ksim)}", "sample 100", "jac 0", "run"]
            cases.append({"name": name, "vehicle": v, "tire": t, "sus": su, "tire_type": tt, "driver": rows,
                          "dt": 0.001, "tend": tend_v, "ksim": ksim, "sample": 100, "vp": {}, "tp": {},
                          "state": s_c.tolist(),
                          "source": f"{src} (24-DOF files), {'HMMWV' if su is sus else 'Sedan'} suspension.json, {drv}.txt"})
        fl = fleet.fleet24(8, seed=SEED, horizon=10.0)
        svj, stj, ssj = (write("sv.json", json.dumps(fleet.SUV24_VEHICLE)), write("st.json", json.dumps(fleet.SUV_TIRE)),
                         write("ss.json", json.dumps(fleet.SUV24_SUS)))
        P = abi.P
        key = {"fxmpn": "fxmPn", "fxmp2n": "fxmP2n", "fxspn": "fxsPn", "fxsp2n": "fxsP2n", "fympn": "fymPn",
               "fymp2n": "fymP2n", "fyspn": "fysPn", "fysp2n": "fysP2n", "kt": "kt"}
        for i in range(8):
            rows = fl["tables"][i].tolist()
            tp = write(f"s{i}.txt", "".join(" ".join(_fmt(v) for v in r) + "\n" for r in rows))
            st = fl["states"][i]
            vp = {k: float(fl["params"][i, P[k]]) for k in ("m", "jz", "a", "b")}
            tpv = {key[k]: float(fl["params"][i, P[k]]) for k in ["kt"] + list(fleet.FRICTION_FIELDS)}
            w0 = float(st[C["LFDM24_S_TIRE0"] + C["LFDM24_T_OMEGA"]])
            jobs += [f"veh {svj}", f"tire {stj}", f"sus {ssj}", f"driver {tp}", "dt 0.001", "tend 10", "ksim 1",
                     "sample 250"]
            jobs += [f"vp {k} {_fmt(v)}" for k, v in vp.items()] + [f"tp {k} {_fmt(v)}" for k, v in tpv.items()]
            jobs += [f"vs u {_fmt(st[C['LFDM24_S_U']])}", f"vs crankOmega {_fmt(st[C['LFDM24_S_CRANKOMEGA']])}",
                     f"gear {int(st[C['LFDM24_S_CURRENT_GR']])}"] + [f"ts {k} omega {_fmt(w0)}" for k in range(4)]
            jobs += [f"jac {int(i < 2)}", "run"]
            cases.append({"name": f"suv24_{i}", "vehicle": fleet.SUV24_VEHICLE, "tire": fleet.SUV_TIRE,
                          "sus": fleet.SUV24_SUS, "tire_type": 0, "driver": rows, "dt": 0.001, "tend": 10.0,
                          "ksim": 1.0, "sample": 250, "vp": vp, "tp": tpv, "state": st.tolist(),
                          "source": f"synthetic 24-DOF SUV fleet seed {SEED} vehicle {i}"})
        out = subprocess.run([refrun], input="\n".join(jobs) + "\n", capture_output=True, text=True, check=True)
    results = parse_ref(out.stdout)
    assert len(results) == len(cases)
    for c, r in zip(cases, results):
        assert len(r["final"]) == C["LFDM24_S_COUNT"]
        c["expected_samples"] = r["samples"]
        c["expected_final"] = r["final"]
        add_jacobian(c, r)
    with open(os.path.join(HERE, "golden24.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py", "model": 24, "cases": cases}, f, separators=(",", ":"))
    print(f"wrote {len(cases)} 24-DOF cases; {cases[0]['name']} x={cases[0]['expected_final'][0]!r}")


if __name__ == "__main__":
    # the reference checkout's wheeled_vehicle_models directory: argument, else $LFDM_REFERENCE, else
    # the default checkout location
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("LFDM_REFERENCE",
                                                                "/root/reference/wheeled_vehicle_models")
    main(ref)
    main11(ref)
    main24(ref)
