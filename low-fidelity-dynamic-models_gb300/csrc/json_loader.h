// JSON reader and input-file loaders of the library (see json_loader.cpp).
#pragma once

#include <string>
#include <utility>
#include <vector>

#include "../../include/lfdm.h"

namespace lfdm {

struct JVal {
    enum Kind { Null, Bool, Num, Str, Arr, Obj } kind = Null;
    bool b = false;
    double d = 0;
    std::string s;
    std::vector<JVal> arr;
    std::vector<std::pair<std::string, JVal>> obj;
    const JVal* get(const std::string& k) const;
};

bool json_parse(const std::string& text, JVal& out, std::string& err);
bool read_file(const std::string& path, std::string& out);

// Defaults of the reference's parameter structs, into a class record and a flat parameter vector.
void default_vehicle(lfdm_class18& c, double* p);
// tireInit (18dof-gpu/dof18_gpu.cu:227-233) on a flat parameter vector.
void tire_init(double* p);
// Vehicle JSON + tire JSON (+ suspension JSON for the 24-DOF model, else empty) -> class record +
// flat parameter vector (tireInit applied), for the 11-, 18- or 24-DOF model (the 11-DOF files hold
// fewer vehicle keys and its tire loader doubles most tire parameters; the 24-DOF vehicle file has
// jy instead of the roll-stiffness terms).
bool load_vehicle(int model, const std::string& veh_path, const std::string& tire_path, const std::string& sus_path,
                  int tire_type, lfdm_class18& c, double* p, std::string& err);
// LoadDriverData (utils/utils_gpu.cu:7-31): rows of {t, steering, throttle, braking}.
bool load_driver_file(const std::string& path, std::vector<double>& rows, std::string& err);

}  // namespace lfdm
