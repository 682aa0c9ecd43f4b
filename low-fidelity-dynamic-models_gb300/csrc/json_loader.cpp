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

// Maximum tire load [kg] by load index 0..279, the table of GetTireMaxLoad
// (18dof-gpu/dof18_gpu.cu:1470-1503; the 11- and 24-DOF models hold the same numbers). Indices past
// the end take the last entry.
static const double kLoadIndexKg[] = {
    45, 46.5, 47.5, 48.7, 50, 51.5, 53, 54.5, 56, 58,  // LI 0-9
    60, 61.5, 63, 65, 67, 69, 71, 73, 75, 77.5,  // LI 10-19
    80.0, 82.5, 85.0, 87.5, 90.0, 92.5, 95.0, 97.5, 100.0, 103,  // LI 20-29
    106, 109, 112, 115, 118, 121, 125, 128, 132, 136,  // LI 30-39
    140, 145, 150, 155, 160, 165, 170, 175, 180, 185,  // LI 40-49
    190, 195, 200, 206, 212, 218, 224, 230, 236, 243,  // LI 50-59
    250, 257, 265, 272, 280, 290, 300, 307, 315, 325,  // LI 60-69
    335, 345, 355, 365, 375, 387, 400, 412, 425, 437,  // LI 70-79
    450, 462, 475, 487, 500, 515, 530, 545, 560, 580,  // LI 80-89
    600, 615, 630, 650, 670, 690, 710, 730, 750, 775,  // LI 90-99
    800, 825, 850, 875, 900, 925, 950, 975, 1000, 1030,  // LI 100-109
    1060, 1090, 1120, 1150, 1180, 1215, 1250, 1285, 1320, 1360,  // LI 110-119
    1400, 1450, 1500, 1550, 1600, 1650, 1700, 1750, 1800, 1850,  // LI 120-129
    1900, 1950, 2000, 2060, 2120, 2180, 2240, 2300, 2360, 2430,  // LI 130-139
    2500, 2575, 2650, 2725, 2800, 2900, 3000, 3075, 3150, 3250,  // LI 140-149
    3350, 3450, 3550, 3650, 3750, 3875, 4000, 4125, 4250, 4375,  // LI 150-159
    4500, 4625, 4750, 4875, 5000, 5150, 5300, 5450, 5600, 5850,  // LI 160-169
    6000, 6150, 6300, 6500, 6700, 6900, 7100, 7300, 7500, 7750,  // LI 170-179
    8000, 8250, 8500, 8750, 9000, 9250, 9500, 9750, 10000, 10300,  // LI 180-189
    10600, 10900, 11200, 11500, 11800, 12150, 12500, 12850, 13200, 13600,  // LI 190-199
    14000, 14500, 15000, 15550, 16000, 16500, 17000, 17500, 18000, 18500,  // LI 200-209
    19000, 19500, 20000, 20600, 21200, 21800, 22400, 23000, 23600, 24300,  // LI 210-219
    25000, 25750, 26500, 27250, 28000, 29000, 30000, 30750, 31500, 32500,  // LI 220-229
    33500, 34500, 35500, 36500, 37500, 38750, 40000, 41250, 42500, 43750,  // LI 230-239
    45000, 46250, 47500, 48750, 50000, 51500, 53000, 54500, 56000, 58000,  // LI 240-249
    60000, 61500, 63000, 65000, 67000, 69000, 71000, 73000, 75000, 77500,  // LI 250-259
    80000, 82500, 85000, 87500, 90000, 92500, 95000, 97500, 100000, 103000,  // LI 260-269
    106000, 109000, 112000, 115000, 118000, 121000, 125000, 128500, 132000, 136000,  // LI 270-279
};

// Load-normalised TMeasy curve parameters of GuessPassCar70Par and GuessTruck80Par
// (18dof-gpu/dof18_gpu.cu:1516-1615): force entries (dfx0, fxm, fxs, dfy0, fym, fys; Pn then P2n) as
// multiples of pn (of 2 pn for P2n), then the slips (sxm, sxs, sym, sys; Pn then P2n).
struct TireGuess {
    double force[12];
    double slip[8];
};
static const TireGuess kPassCar70 = {
    {18.3741, 19.4669, 1.1292, 1.0896, 0.80149, 0.76917, 15.9826, 12.8509, 1.0009, 0.91367, 0.8336, 0.77336},
    {0.13913, 0.13913, 0.66667, 0.66667, 0.14852, 0.18504, 0.96524, 1.0714}};
static const TireGuess kTruck80 = {
    {17.7764, 14.5301, 0.89965, 0.77751, 0.46183, 0.42349, 7.4013, 6.8505, 0.75876, 0.72628, 0.68276, 0.65319},
    {0.10811, 0.12389, 0.66667, 0.66667, 0.33167, 0.33216, 1.0296, 1.0296}};

// TMeasyNr "highLevelParams": design values from the file, curve parameters guessed from the tire's
// width, aspect ratio, rim and load capacity (load index or maximum bearing capacity). two = 2 for
// the single-track 11-DOF model, whose loader doubles the axle quantities.
static bool tmeasy_nr_high_level(Ctx& t, const JVal& td, double two, double* p) {
    bool ok = t.num("jw", p[LFDM_P_JW]) && t.num("rr", p[LFDM_P_RR]) && t.num("mu", p[LFDM_P_MU]) &&
              t.num("r0", p[LFDM_P_R0]) && t.num("rdyncoPn", p[LFDM_P_RDYNCOPN]) &&
              t.num("rdyncoP2n", p[LFDM_P_RDYNCOP2N]) && t.num("fzRdynco", p[LFDM_P_FZRDYNCO]) &&
              t.num("rdyncoCrit", p[LFDM_P_RDYNCOCRIT]);
    if (!ok) return false;
    for (int i : {LFDM_P_JW, LFDM_P_RR, LFDM_P_MU, LFDM_P_FZRDYNCO, LFDM_P_RDYNCOCRIT}) p[i] *= two;
    auto opt = [&](const char* k, double def) {
        const JVal* x = td.get(k);
        return (x && x->kind == JVal::Num) ? x->d : def;
    };
    p[LFDM_P_VCOULOMB] = opt("vCoulomb", 1.0);
    p[LFDM_P_FRBLEND_BEGIN] = opt("frblendBegin", 1.0);
    p[LFDM_P_FRBLEND_END] = opt("frblendEnd", 3.0);
    double width = 0, rim_radius = 0;
    if (!(t.num("width", width) && t.num("rimRadius", rim_radius))) return false;
    double p_li = opt("inflationPressureDesign", 0.0), p_use = opt("inflationPressureUse", 0.0);
    if (!(p_use > 0.0 && p_li > 0.0)) p_li = p_use = 1.0;
    p[LFDM_P_P_LI] = p_li;
    p[LFDM_P_P_USE] = p_use;
    double load = 0;
    const JVal* li = td.get("loadIndex");
    if (li && li->kind == JVal::Num) {
        const unsigned idx = (unsigned)li->d;
        p[LFDM_P_LI] = idx;
        const unsigned n = sizeof(kLoadIndexKg) / sizeof(kLoadIndexKg[0]);
        load = kLoadIndexKg[idx < n ? idx : n - 1] * 9.81;
    } else {
        if (!t.num("maximumBearingCapacity", load)) return false;
        p[LFDM_P_BEARINGCAPACITY] = load;
    }
    const JVal* vt = td.get("vehicleType");
    if (!vt || vt->kind != JVal::Str) {
        if (t.err.empty()) t.err = t.file + ": missing key \"vehicleType\"";
        return false;
    }
    const TireGuess& g = vt->s == "Truck" ? kTruck80 : kPassCar70;
    // GuessPassCar70Par / GuessTruck80Par with ratio = (r0 - rim radius) / width, rim diameter
    // 2 rim radius: section height width * ratio, deflection at the rated load 0.16 of it
    const double ratio = (p[LFDM_P_R0] - rim_radius) / width;
    const double defl_max = 0.16 * (width * ratio);
    const double pn = 0.5 * load * std::pow(p_use / p_li, 0.8);
    p[LFDM_P_PN] = pn;
    p[LFDM_P_PNMAX] = 3.5 * pn;
    p[LFDM_P_KT] = load / defl_max;
    p[LFDM_P_RIM_RADIUS] = 0.5 * (2 * rim_radius);
    p[LFDM_P_WIDTH] = width;
    static const int fk[12] = {LFDM_P_DFX0PN, LFDM_P_DFX0P2N, LFDM_P_FXMPN, LFDM_P_FXMP2N, LFDM_P_FXSPN, LFDM_P_FXSP2N,
                               LFDM_P_DFY0PN, LFDM_P_DFY0P2N, LFDM_P_FYMPN, LFDM_P_FYMP2N, LFDM_P_FYSPN, LFDM_P_FYSP2N};
    static const int sk[8] = {LFDM_P_SXMPN, LFDM_P_SXMP2N, LFDM_P_SXSPN, LFDM_P_SXSP2N,
                              LFDM_P_SYMPN, LFDM_P_SYMP2N, LFDM_P_SYSPN, LFDM_P_SYSP2N};
    for (int i = 0; i < 12; ++i) p[fk[i]] = ((i % 2) ? (g.force[i] * 2.0) * pn : g.force[i] * pn) * two;
    for (int i = 0; i < 8; ++i) p[sk[i]] = g.slip[i];
    return true;
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
    } else {
        // setTireParamsJSON for TMeasyNr (18dof-gpu/dof18_gpu.cu:1278-1466; 24-DOF the same,
        // 24dof-gpu/dof24_gpu.cu:1847-2070; 11-DOF doubling the axle quantities, 11dof-gpu/dof11_gpu.cu:1101-1290)
        const double two = model == LFDM_MODEL_11 ? 2.0 : 1.0;
        const JVal* hl = td.get("highLevelParams");
        if (hl && hl->kind == JVal::Bool && hl->b) {
            ok = tmeasy_nr_high_level(t, td, two, p);
        } else {
            for (auto& e : tk) {
                if (e.i == LFDM_P_CX || e.i == LFDM_P_CY || e.i == LFDM_P_DX || e.i == LFDM_P_DY) continue;
                ok = ok && t.num(e.k, p[e.i]);
            }
            if (ok && model == LFDM_MODEL_11) {
                static const int dbl[] = {LFDM_P_JW,     LFDM_P_RR,     LFDM_P_PN,      LFDM_P_PNMAX,  LFDM_P_KT,
                                          LFDM_P_FZRDYNCO, LFDM_P_RDYNCOCRIT, LFDM_P_DFX0PN, LFDM_P_DFX0P2N,
                                          LFDM_P_FXMPN,  LFDM_P_FXMP2N, LFDM_P_FXSPN,   LFDM_P_FXSP2N, LFDM_P_DFY0PN,
                                          LFDM_P_DFY0P2N, LFDM_P_FYMPN, LFDM_P_FYMP2N,  LFDM_P_FYSPN,  LFDM_P_FYSP2N};
                for (int i : dbl) p[i] *= 2.;
            }
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
