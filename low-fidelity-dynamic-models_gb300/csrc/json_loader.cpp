// Minimal JSON reader and the vehicle/tire/driver-file loaders of the library.
//
// The loaders follow the reference's setVehParamsJSON (18dof-gpu/dof18_gpu.cu:1075-1218),
// setTireParamsJSON for TMeasy (:1222-1266) and TMeasyNr low-level parameters (:1268-1330), and
// LoadDriverData (utils/utils_gpu.cu:7-31): same keys, defaults, unit conversions and parse-stop
// rule. Unlike the reference (which dereferences missing keys), a missing required key is
// reported as LFDM_ERR_PARSE.
#include "json_loader.h"

#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>

namespace lfdm {

namespace {

struct Parser {
    const char* p;
    const char* end;
    std::string err;

    void ws() {
        while (p < end && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r')) ++p;
    }
    bool fail(const std::string& m) {
        if (err.empty()) err = m;
        return false;
    }
    bool lit(const char* s, JVal& out, JVal::Kind k, bool b) {
        size_t n = std::strlen(s);
        if ((size_t)(end - p) < n || std::strncmp(p, s, n) != 0) return fail("bad literal");
        p += n;
        out.kind = k;
        out.b = b;
        return true;
    }
    bool str(std::string& s) {
        if (p >= end || *p != '"') return fail("expected string");
        ++p;
        while (p < end && *p != '"') {
            if (*p == '\\') {
                ++p;
                if (p >= end) return fail("bad escape");
                char c = *p;
                s.push_back(c == 'n' ? '\n' : c == 't' ? '\t' : c);
            } else {
                s.push_back(*p);
            }
            ++p;
        }
        if (p >= end) return fail("unterminated string");
        ++p;
        return true;
    }
    bool value(JVal& out, int depth) {
        if (depth > 64) return fail("nesting too deep");
        ws();
        if (p >= end) return fail("unexpected end");
        const char c = *p;
        if (c == '{') {
            ++p;
            out.kind = JVal::Obj;
            ws();
            if (p < end && *p == '}') {
                ++p;
                return true;
            }
            for (;;) {
                ws();
                std::string key;
                if (!str(key)) return false;
                ws();
                if (p >= end || *p != ':') return fail("expected ':'");
                ++p;
                JVal v;
                if (!value(v, depth + 1)) return false;
                out.obj.emplace_back(std::move(key), std::move(v));
                ws();
                if (p < end && *p == ',') {
                    ++p;
                    continue;
                }
                if (p < end && *p == '}') {
                    ++p;
                    return true;
                }
                return fail("expected ',' or '}'");
            }
        }
        if (c == '[') {
            ++p;
            out.kind = JVal::Arr;
            ws();
            if (p < end && *p == ']') {
                ++p;
                return true;
            }
            for (;;) {
                JVal v;
                if (!value(v, depth + 1)) return false;
                out.arr.push_back(std::move(v));
                ws();
                if (p < end && *p == ',') {
                    ++p;
                    continue;
                }
                if (p < end && *p == ']') {
                    ++p;
                    return true;
                }
                return fail("expected ',' or ']'");
            }
        }
        if (c == '"') {
            out.kind = JVal::Str;
            return str(out.s);
        }
        if (c == 't') return lit("true", out, JVal::Bool, true);
        if (c == 'f') return lit("false", out, JVal::Bool, false);
        if (c == 'n') return lit("null", out, JVal::Null, false);
        // number: strtod is correctly rounded, as the reference's parser is for these inputs
        char* e = nullptr;
        std::string tok;
        const char* q = p;
        while (q < end && (std::isdigit((unsigned char)*q) || *q == '-' || *q == '+' || *q == '.' || *q == 'e' ||
                           *q == 'E'))
            ++q;
        tok.assign(p, q);
        if (tok.empty()) return fail(std::string("unexpected character '") + c + "'");
        errno = 0;
        double d = std::strtod(tok.c_str(), &e);
        if (e != tok.c_str() + tok.size()) return fail("bad number '" + tok + "'");
        out.kind = JVal::Num;
        out.d = d;
        p = q;
        return true;
    }
};

}  // namespace

const JVal* JVal::get(const std::string& k) const {
    if (kind != Obj) return nullptr;
    for (auto& kv : obj)
        if (kv.first == k) return &kv.second;
    return nullptr;
}

bool json_parse(const std::string& text, JVal& out, std::string& err) {
    Parser ps{text.data(), text.data() + text.size(), {}};
    if (!ps.value(out, 0)) {
        err = ps.err;
        return false;
    }
    ps.ws();
    if (ps.p != ps.end) {
        err = "trailing characters";
        return false;
    }
    return true;
}

bool read_file(const std::string& path, std::string& out) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    std::ostringstream ss;
    ss << f.rdbuf();
    out = ss.str();
    return true;
}

namespace {

struct Ctx {
    const JVal* d;
    std::string file;
    std::string err;
    bool num(const char* k, double& v) {
        const JVal* x = d->get(k);
        if (!x || x->kind != JVal::Num) {
            if (err.empty()) err = file + ": missing or non-numeric key \"" + k + "\"";
            return false;
        }
        v = x->d;
        return true;
    }
    bool boolean(const char* k, bool& v) {
        const JVal* x = d->get(k);
        if (!x || (x->kind != JVal::Bool && x->kind != JVal::Num)) {
            if (err.empty()) err = file + ": missing or non-boolean key \"" + k + "\"";
            return false;
        }
        v = x->kind == JVal::Bool ? x->b : x->d != 0;
        return true;
    }
    bool map(const char* k, double (*dst)[2], int32_t& size, double xscale) {
        const JVal* x = d->get(k);
        if (!x || x->kind != JVal::Arr) {
            if (err.empty()) err = file + ": missing map \"" + k + "\"";
            return false;
        }
        if (x->arr.size() > LFDM_MAX_MAP) {
            if (err.empty()) err = file + ": map \"" + k + "\" has more than LFDM_MAX_MAP points";
            return false;
        }
        for (size_t i = 0; i < x->arr.size(); ++i) {
            const JVal& e = x->arr[i];
            if (e.kind != JVal::Arr || e.arr.size() < 2 || e.arr[0].kind != JVal::Num || e.arr[1].kind != JVal::Num) {
                if (err.empty()) err = file + ": bad entry in map \"" + k + "\"";
                return false;
            }
            dst[i][0] = e.arr[0].d * xscale;
            dst[i][1] = e.arr[1].d;
        }
        size = (int32_t)x->arr.size();
        return true;
    }
};

bool load_json(const std::string& path, JVal& v, std::string& err) {
    std::string text;
    if (!read_file(path, text)) {
        err = "cannot open " + path;
        return false;
    }
    std::string perr;
    if (!json_parse(text, v, perr)) {
        err = path + ": JSON parse error: " + perr;
        return false;
    }
    if (v.kind != JVal::Obj) {
        err = path + ": top level is not an object";
        return false;
    }
    return true;
}

}  // namespace

void default_vehicle(lfdm_class18& c, double* p) {
    std::memset(&c, 0, sizeof(c));
    c.driveType = 1;
    c.whichWheels = 1;
    // VehicleParam() defaults (dof18_gpu.cuh:506-531)
    p[LFDM_P_A] = 1.6889; p[LFDM_P_B] = 1.6889; p[LFDM_P_H] = 0.713; p[LFDM_P_M] = 2097.85;
    p[LFDM_P_JZ] = 4519.; p[LFDM_P_JX] = 1289.; p[LFDM_P_JXZ] = 3.265; p[LFDM_P_CF] = 1.82; p[LFDM_P_CR] = 1.82;
    p[LFDM_P_MUF] = 127.866; p[LFDM_P_MUR] = 129.98; p[LFDM_P_HRCF] = 0.379; p[LFDM_P_HRCR] = 0.327;
    p[LFDM_P_KROF] = 31000; p[LFDM_P_KROR] = 31000; p[LFDM_P_BROF] = 3300; p[LFDM_P_BROR] = 3300;
    p[LFDM_P_MAXSTEER] = 0.6525249; p[LFDM_P_CRANKINERTIA] = 1.1; p[LFDM_P_MAXBRAKETORQUE] = 4000.;
    // TMeasyParam() defaults (dof18_gpu.cuh:29-64)
    p[LFDM_P_JW] = 6.69; p[LFDM_P_RR] = 0.015; p[LFDM_P_MU] = 0.8; p[LFDM_P_R0] = 0.4699; p[LFDM_P_PN] = 8562.8266;
    p[LFDM_P_PNMAX] = 29969.893; p[LFDM_P_CX] = 185004.42; p[LFDM_P_CY] = 164448.37; p[LFDM_P_KT] = 411121.0;
    p[LFDM_P_DX] = 3700.; p[LFDM_P_DY] = 3488.; p[LFDM_P_RDYNCOPN] = 0.375; p[LFDM_P_RDYNCOP2N] = 0.75;
    p[LFDM_P_FZRDYNCO] = 0; p[LFDM_P_RDYNCOCRIT] = 0; p[LFDM_P_DFX0PN] = 151447.29; p[LFDM_P_DFX0P2N] = 236412.79;
    p[LFDM_P_FXMPN] = 7575.3614; p[LFDM_P_FXMP2N] = 12808.276; p[LFDM_P_FXSPN] = 4657.9208;
    p[LFDM_P_FXSP2N] = 8625.3352; p[LFDM_P_SXMPN] = 0.12; p[LFDM_P_SXMP2N] = 0.15; p[LFDM_P_SXSPN] = 0.9;
    p[LFDM_P_SXSP2N] = 0.95; p[LFDM_P_DFY0PN] = 50931.693; p[LFDM_P_DFY0P2N] = 94293.847;
    p[LFDM_P_FYMPN] = 6615.0404; p[LFDM_P_FYMP2N] = 12509.947; p[LFDM_P_FYSPN] = 6091.5092;
    p[LFDM_P_FYSP2N] = 11443.875; p[LFDM_P_SYMPN] = 0.38786; p[LFDM_P_SYMP2N] = 0.38786; p[LFDM_P_SYSPN] = 0.82534;
    p[LFDM_P_SYSP2N] = 0.91309;
    // TMeasyNrParam() extra defaults (dof18_gpu.cuh:267-307)
    p[LFDM_P_WIDTH] = 0.245; p[LFDM_P_RIM_RADIUS] = 0.254; p[LFDM_P_VCOULOMB] = 1.0; p[LFDM_P_FRBLEND_BEGIN] = 1.;
    p[LFDM_P_FRBLEND_END] = 3.; p[LFDM_P_BEARINGCAPACITY] = 10000; p[LFDM_P_LI] = 90; p[LFDM_P_P_LI] = 1.;
    p[LFDM_P_P_USE] = 1.;
    // 24-DOF: VehicleParam()::_jy and SuspensionParam() defaults (24dof-gpu/dof24_gpu.cuh)
    p[LFDM_P_JY] = 3516.; p[LFDM_P_KS] = 150062.; p[LFDM_P_BS] = 19068.;
}

void tire_init(double* p) {
    // tireInit (dof18_gpu.cu:227-233)
    const double pn = p[LFDM_P_PN], r1 = p[LFDM_P_RDYNCOPN], r2 = p[LFDM_P_RDYNCOP2N];
    p[LFDM_P_FZRDYNCO] = (pn * (r2 - 2.0 * r1 + 1.)) / (2. * (r2 - r1));
    const double fz = p[LFDM_P_FZRDYNCO];
    p[LFDM_P_RDYNCOCRIT] = r1 + (r2 - r1) * (fz / pn - 1.);
}

bool load_vehicle(int model, const std::string& veh_path, const std::string& tire_path, const std::string& sus_path,
                  int tire_type, lfdm_class18& c, double* p, std::string& err) {
    default_vehicle(c, p);
    JVal vd, td;
    if (!load_json(veh_path, vd, err)) return false;
    if (!load_json(tire_path, td, err)) return false;
    if (model == LFDM_MODEL_24) {
        // setSuspensionParamsJSON (24dof-gpu/dof24_gpu.cu; CPU 24dof/dof24.cpp:2192-2212)
        JVal sd;
        if (sus_path.empty()) {
            err = "the 24-DOF model needs a suspension JSON";
            return false;
        }
        if (!load_json(sus_path, sd, err)) return false;
        Ctx sc{&sd, sus_path, {}};
        if (!(sc.num("ks", p[LFDM_P_KS]) && sc.num("bs", p[LFDM_P_BS]))) {
            err = sc.err;
            return false;
        }
    }
    const double rpm2rad = 3.141592653589793238462643383279 / 30;  // utils_gpu.cuh:13
    Ctx v{&vd, veh_path, {}};
    static const struct {
        const char* k;
        int i;
    } vk[] = {{"a", LFDM_P_A},       {"b", LFDM_P_B},       {"m", LFDM_P_M},       {"h", LFDM_P_H},
              {"jz", LFDM_P_JZ},     {"jx", LFDM_P_JX},     {"jxz", LFDM_P_JXZ},   {"cf", LFDM_P_CF},
              {"cr", LFDM_P_CR},     {"muf", LFDM_P_MUF},   {"mur", LFDM_P_MUR},   {"hrcf", LFDM_P_HRCF},
              {"hrcr", LFDM_P_HRCR}, {"krof", LFDM_P_KROF}, {"kror", LFDM_P_KROR}, {"brof", LFDM_P_BROF},
              {"bror", LFDM_P_BROR}, {"jy", LFDM_P_JY}};
    bool ok = true;
    for (auto& e : vk) {
        // the 11-DOF vehicle file holds only a, b, m, h, jz, muf, mur (11dof-gpu/dof11_gpu.cu:910-1044);
        // the 24-DOF one adds jy and has no jxz or roll stiffness/damping (24dof/dof24.cpp:2217-2339)
        if (model == LFDM_MODEL_11 && !(e.i == LFDM_P_A || e.i == LFDM_P_B || e.i == LFDM_P_M || e.i == LFDM_P_H ||
                                        e.i == LFDM_P_JZ || e.i == LFDM_P_MUF || e.i == LFDM_P_MUR))
            continue;
        const bool only18 = e.i == LFDM_P_JXZ || e.i == LFDM_P_KROF || e.i == LFDM_P_KROR || e.i == LFDM_P_BROF ||
                            e.i == LFDM_P_BROR;
        if (model == LFDM_MODEL_24 && only18) continue;
        if (model == LFDM_MODEL_18 && e.i == LFDM_P_JY) continue;
        ok = ok && v.num(e.k, p[e.i]);
    }
    bool b = false;
    ok = ok && v.boolean("nonLinearSteer", b);
    c.nonLinearSteer = b;
    if (ok && c.nonLinearSteer) ok = v.map("steerMap", c.steerMap, c.steerMapSize, 1.0);
    ok = ok && v.num("maxSteer", p[LFDM_P_MAXSTEER]);
    const JVal* gears = vd.get("gearRatios");
    if (ok && (!gears || gears->kind != JVal::Arr || gears->arr.empty() || gears->arr.size() > LFDM_MAX_GEARS)) {
        err = veh_path + ": gearRatios missing, empty or longer than LFDM_MAX_GEARS";
        return false;
    }
    if (ok) {
        c.noGears = (int32_t)gears->arr.size();
        for (int i = 0; i < c.noGears; ++i) {
            if (gears->arr[i].kind != JVal::Num) {
                err = veh_path + ": bad gear ratio";
                return false;
            }
            c.gearRatios[i] = gears->arr[i].d;
        }
        const JVal* up = vd.get("upshiftRPM");
        const JVal* dn = vd.get("downshiftRPM");
        if (up && dn && up->kind == JVal::Num && dn->kind == JVal::Num) {
            for (int i = 0; i < c.noGears; ++i) {
                c.shiftMap[i][0] = dn->d * rpm2rad;
                c.shiftMap[i][1] = up->d * rpm2rad;
            }
        } else {
            const JVal* sm = vd.get("shiftMap");
            if (!sm || sm->kind != JVal::Arr || (int)sm->arr.size() < c.noGears) {
                err = veh_path + ": needs upshiftRPM/downshiftRPM or a shiftMap with one row per gear";
                return false;
            }
            for (int i = 0; i < c.noGears; ++i) {
                const JVal& r = sm->arr[i];
                if (r.kind != JVal::Arr || r.arr.size() < 2) {
                    err = veh_path + ": bad shiftMap row";
                    return false;
                }
                c.shiftMap[i][0] = r.arr[0].d * rpm2rad;
                c.shiftMap[i][1] = r.arr[1].d * rpm2rad;
            }
        }
    }
    ok = ok && v.boolean("tcBool", b);
    c.tcbool = b;
    ok = ok && v.num("maxBrakeTorque", p[LFDM_P_MAXBRAKETORQUE]);
    ok = ok && v.boolean("throttleMod", b);
    c.throttleMod = b;
    ok = ok && v.map("torqueMap", c.powertrainMap, c.powertrainMapSize, rpm2rad);
    ok = ok && v.map("lossesMap", c.lossesMap, c.lossesMapSize, rpm2rad);
    if (ok && c.tcbool) {
        ok = v.num("crankInertia", p[LFDM_P_CRANKINERTIA]) && v.map("capacityFactorMap", c.CFmap, c.CFmapSize, 1.0) &&
             v.map("torqueRatioMap", c.TRmap, c.TRmapSize, 1.0);
    }
    if (ok && vd.get("4wd")) {
        ok = v.boolean("4wd", b);
        c.driveType = b;
        ok = ok && v.boolean("rearWheels", b);
        c.whichWheels = b;
    }
    if (!ok) {
        err = v.err;
        return false;
    }
    Ctx t{&td, tire_path, {}};
    static const struct {
        const char* k;
        int i;
    } tk[] = {{"jw", LFDM_P_JW},          {"rr", LFDM_P_RR},          {"r0", LFDM_P_R0},
              {"pn", LFDM_P_PN},          {"pnmax", LFDM_P_PNMAX},    {"cx", LFDM_P_CX},
              {"cy", LFDM_P_CY},          {"kt", LFDM_P_KT},          {"dx", LFDM_P_DX},
              {"dy", LFDM_P_DY},          {"rdyncoPn", LFDM_P_RDYNCOPN}, {"rdyncoP2n", LFDM_P_RDYNCOP2N},
              {"fzRdynco", LFDM_P_FZRDYNCO}, {"rdyncoCrit", LFDM_P_RDYNCOCRIT}, {"dfx0Pn", LFDM_P_DFX0PN},
              {"dfx0P2n", LFDM_P_DFX0P2N}, {"fxmPn", LFDM_P_FXMPN},    {"fxmP2n", LFDM_P_FXMP2N},
              {"fxsPn", LFDM_P_FXSPN},    {"fxsP2n", LFDM_P_FXSP2N},  {"sxmPn", LFDM_P_SXMPN},
              {"sxmP2n", LFDM_P_SXMP2N},  {"sxsPn", LFDM_P_SXSPN},    {"sxsP2n", LFDM_P_SXSP2N},
              {"dfy0Pn", LFDM_P_DFY0PN},  {"dfy0P2n", LFDM_P_DFY0P2N}, {"fymPn", LFDM_P_FYMPN},
              {"fymP2n", LFDM_P_FYMP2N},  {"fysPn", LFDM_P_FYSPN},    {"fysP2n", LFDM_P_FYSP2N},
              {"symPn", LFDM_P_SYMPN},    {"symP2n", LFDM_P_SYMP2N},  {"sysPn", LFDM_P_SYSPN},
              {"sysP2n", LFDM_P_SYSP2N}};
    if (tire_type == LFDM_TIRE_TMEASY) {
        for (auto& e : tk) ok = ok && t.num(e.k, p[e.i]);
        if (ok && model == LFDM_MODEL_11) {
            // single-track tire = both wheels of an axle: setTireParamsJSON (11dof-gpu/dof11_gpu.cu:1046-1099)
            // doubles these fields and keeps r0, the rdynco weights and the slips
            static const int dbl[] = {LFDM_P_JW,     LFDM_P_RR,     LFDM_P_PN,       LFDM_P_PNMAX,      LFDM_P_CX,
                                      LFDM_P_CY,     LFDM_P_KT,     LFDM_P_DX,       LFDM_P_DY,         LFDM_P_FZRDYNCO,
                                      LFDM_P_RDYNCOCRIT, LFDM_P_DFX0PN, LFDM_P_DFX0P2N, LFDM_P_FXMPN, LFDM_P_FXMP2N,
                                      LFDM_P_FXSPN,  LFDM_P_FXSP2N, LFDM_P_DFY0PN,   LFDM_P_DFY0P2N,    LFDM_P_FYMPN,
                                      LFDM_P_FYMP2N, LFDM_P_FYSPN,  LFDM_P_FYSP2N};
            for (int i : dbl) p[i] *= 2.;
        }
    } else if (model != LFDM_MODEL_18) {
        err = tire_path + ": TMeasyNr tires are available for the 18-DOF model only";
        return false;
    } else {
        const JVal* hl = td.get("highLevelParams");
        if (hl && hl->kind == JVal::Bool && hl->b) {
            err = tire_path + ": TMeasyNr high-level parameters (load-index guessing) are not supported";
            return false;
        }
        for (auto& e : tk) {
            if (e.i == LFDM_P_CX || e.i == LFDM_P_CY || e.i == LFDM_P_DX || e.i == LFDM_P_DY) continue;
            ok = ok && t.num(e.k, p[e.i]);
        }
    }
    if (!ok) {
        err = t.err;
        return false;
    }
    tire_init(p);
    return true;
}

bool load_driver_file(const std::string& path, std::vector<double>& rows, std::string& err) {
    std::ifstream f(path);
    if (!f) {
        err = "cannot open driver file " + path;
        return false;
    }
    std::string line;
    rows.clear();
    while (std::getline(f, line)) {
        std::istringstream iss(line);
        double t, s, th, b;
        iss >> t >> s >> th >> b;
        if (iss.fail()) break;
        rows.insert(rows.end(), {t, s, th, b});
    }
    if (rows.empty()) {
        err = "driver file " + path + " holds no rows";
        return false;
    }
    return true;
}

}  // namespace lfdm
