// input.toml reading for fvgb: a TOML subset (tables, dotted table headers,
// key = int | float | bool | "string", # comments) mapped onto fvgb_params the
// way TomlFileManager::treeToGlobalParameter does
// (FVMR/src/input/TomlFileManager.cpp:110-170), including the boundary-state
// input modes (200-265), mu0 <-> Re (47-104) and the defaults of
// FVMR/src/global/GlobalPara.cpp:4-90.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>

#include "internal.h"

namespace fvgb {

namespace {

struct Value {
    enum Kind { INT, FLOAT, BOOL, STR } kind;
    long long i = 0;
    double d = 0;
    bool b = false;
    std::string s;
};

using Table = std::map<std::string, Value>;

std::string trim(const std::string& x) {
    size_t a = x.find_first_not_of(" \t\r\n"), b = x.find_last_not_of(" \t\r\n");
    return a == std::string::npos ? std::string() : x.substr(a, b - a + 1);
}

int parse(const char* path, Table& t) {
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(FVGB_ERR_IO, std::string("cannot open ") + path);
    std::string prefix, line;
    char buf[4096];
    int lineno = 0;
    while (std::fgets(buf, sizeof buf, f)) {
        lineno++;
        line = buf;
        // strip a comment that is not inside a string
        bool inq = false;
        for (size_t k = 0; k < line.size(); k++) {
            if (line[k] == '"') inq = !inq;
            if (line[k] == '#' && !inq) {
                line.resize(k);
                break;
            }
        }
        line = trim(line);
        if (line.empty()) continue;
        if (line[0] == '[') {
            size_t e = line.find(']');
            if (e == std::string::npos) {
                std::fclose(f);
                return fail(FVGB_ERR_FORMAT, "input.toml line " + std::to_string(lineno) + ": bad table header");
            }
            prefix = trim(line.substr(1, e - 1)) + ".";
            continue;
        }
        size_t eq = line.find('=');
        if (eq == std::string::npos) {
            std::fclose(f);
            return fail(FVGB_ERR_FORMAT, "input.toml line " + std::to_string(lineno) + ": expected key = value");
        }
        std::string key = trim(line.substr(0, eq)), val = trim(line.substr(eq + 1));
        Value v;
        if (!val.empty() && val[0] == '"') {
            size_t e = val.find('"', 1);
            v.kind = Value::STR;
            v.s = val.substr(1, e == std::string::npos ? std::string::npos : e - 1);
        } else if (val == "true" || val == "false") {
            v.kind = Value::BOOL;
            v.b = (val == "true");
        } else {
            std::string num;
            for (char c : val)
                if (c != '_') num += c;
            char* endp = nullptr;
            bool is_float = num.find_first_of(".eE") != std::string::npos && num.find("0x") != 0;
            if (is_float || num == "inf" || num == "nan") {
                v.kind = Value::FLOAT;
                v.d = std::strtod(num.c_str(), &endp);
            } else {
                v.kind = Value::INT;
                v.i = std::strtoll(num.c_str(), &endp, 10);
                v.d = (double)v.i;
            }
            if (!endp || *endp != 0) {
                std::fclose(f);
                return fail(FVGB_ERR_FORMAT, "input.toml line " + std::to_string(lineno) + ": cannot read value of " + key);
            }
        }
        t[prefix + key] = v;
    }
    std::fclose(f);
    return 0;
}

struct Reader {
    const Table& t;
    std::string missing;
    bool has(const std::string& k) const { return t.count(k) != 0; }
    // cpptoml reads an integer as a double when asked for a double
    bool num(const std::string& k, double& out, bool required) {
        auto it = t.find(k);
        if (it == t.end()) {
            if (required) missing += " " + k;
            return false;
        }
        if (it->second.kind == Value::FLOAT || it->second.kind == Value::INT) {
            out = it->second.d;
            return true;
        }
        missing += " " + k + "(type)";
        return false;
    }
    bool integer(const std::string& k, int& out, bool required) {
        auto it = t.find(k);
        if (it == t.end()) {
            if (required) missing += " " + k;
            return false;
        }
        if (it->second.kind == Value::INT) {
            out = (int)it->second.i;
            return true;
        }
        missing += " " + k + "(type)";
        return false;
    }
    // TomlFileManager::getValueOrigin reads bools as bool or as int (TomlFileManager.h:60-78)
    bool boolean(const std::string& k, bool& out, bool required) {
        auto it = t.find(k);
        if (it == t.end()) {
            if (required) missing += " " + k;
            return false;
        }
        if (it->second.kind == Value::BOOL) out = it->second.b;
        else if (it->second.kind == Value::INT) out = it->second.i != 0;
        else {
            missing += " " + k + "(type)";
            return false;
        }
        return true;
    }
    bool str(const std::string& k, std::string& out) {
        auto it = t.find(k);
        if (it == t.end() || it->second.kind != Value::STR) return false;
        out = it->second.s;
        return true;
    }
};

// AirParameterConverter::get_ruvp_by_Ma_AoA_T0_p0_gamma_R, FVMR/src/input/AirParameterConverter.cpp:3-24
void ruvp_from_mach(double* ruvp, double Ma, double AoA, double T0, double p0, double gamma, double R) {
    const double PI = 3.1415926535897;
    double T = T0 / (1.0 + (gamma - 1.0) / 2.0 * Ma * Ma);
    double p = p0 * std::pow(T / T0, gamma / (gamma - 1.0));
    double c = std::sqrt(gamma * R * T);
    ruvp[0] = p / (R * T);
    ruvp[1] = c * Ma * std::cos(AoA / 180 * PI);
    ruvp[2] = c * Ma * std::sin(AoA / 180 * PI);
    ruvp[3] = p;
}

// TomlFileManager::getValue_boundaryCondition2D, TomlFileManager.cpp:200-265
int boundary_state(Reader& r, const std::string& parent, const fvgb_params& p, double* ruvp) {
    int mode = -1;
    if (!r.has(parent + ".input_mode")) return 0;  // keeps the default, as the reference does
    r.integer(parent + ".input_mode", mode, true);
    switch (mode) {
    case 0: {
        double Ma = 0, AoA = 0;
        if (r.has(parent + ".AOA")) r.num(parent + ".AOA", AoA, true);
        else r.num(parent + ".AoA", AoA, true);
        r.num(parent + ".Ma", Ma, true);
        ruvp_from_mach(ruvp, Ma, AoA, p.T0, 101325.0, p.gamma, p.R);
        return 0;
    }
    case 1:
        r.num(parent + ".rho", ruvp[0], true);
        r.num(parent + ".u", ruvp[1], true);
        r.num(parent + ".v", ruvp[2], true);
        r.num(parent + ".p", ruvp[3], true);
        return 0;
    case 2: {
        double U[4] = {0, 0, 0, 0}, g = 1.4;
        r.num(parent + ".rho", U[0], true);
        r.num(parent + ".rhou", U[1], true);
        r.num(parent + ".rhov", U[2], true);
        r.num(parent + ".rhoE", U[3], true);
        r.num("constant.gamma", g, false);
        ruvp[0] = U[0];
        ruvp[1] = U[1] / U[0];
        ruvp[2] = U[2] / U[0];
        ruvp[3] = ruvp[0] * (g - 1) * (U[3] / U[0] - (ruvp[1] * ruvp[1] + ruvp[2] * ruvp[2]) * 0.5);
        return 0;
    }
    case 3: {
        double u = 0, angle = 0;
        r.num(parent + ".rho", ruvp[0], true);
        r.num(parent + ".u", u, true);
        r.num(parent + ".angle_degree", angle, true);
        r.num(parent + ".p", ruvp[3], true);
        angle = angle * kPi / 180.0;
        ruvp[1] = u * std::cos(angle);
        ruvp[2] = u * std::sin(angle);
        return 0;
    }
    default:
        return fail(FVGB_ERR_FORMAT, "invalid input_mode at " + parent);
    }
}

}  // namespace

}  // namespace fvgb

using namespace fvgb;

extern "C" int fvgb_params_default(fvgb_params* p) {
    if (!p) return fail(FVGB_ERR_ARG, "null params");
    std::memset(p, 0, sizeof(*p));
    p->equation = 1;
    p->flux_scheme = 2002;
    p->reconstruct = 3001;
    p->gradient = 1;
    p->limiter = 2;  // _LIM_minmod: the reference default, which its limiter switch rejects
    p->time_advance = 3101;
    p->lsq_det_ref = 1;
    p->wall_bc_ref = 1;
    p->restrict_ref = 1;
    p->ic_type = 1;
    p->renumber = 1;
    p->device = 0;
    p->gamma = 1.4;
    p->R = 287.06;
    p->Pr = 0.73;
    p->mu0 = 17.9e-6;
    p->T0 = 288.16;
    p->CFL = 0.6;
    p->T_end = 20;
    p->Re = 1.0e8;
    p->vortex[2] = 1;
    p->shock[2] = 1.0;  // FieldInitializer.h:23-26: the shock normal points along +x
    p->dsr[2] = 60.0;   // CBoundaryDoubleShockReflect.h:14
    p->CFL_steady = 0.95;  // GlobalPara.cpp:38
    p->mesh_scale = 1.0;
    p->max_iteration = 5000;
    p->ref_area = 1.0;
    return 0;
}

extern "C" int fvgb_params_read_toml(const char* path, fvgb_params* p, char* mesh_name, int mesh_name_len) {
    if (!path || !p) return fail(FVGB_ERR_ARG, "null argument");
    Table t;
    int rc = parse(path, t);
    if (rc) return rc;
    fvgb_params_default(p);
    Reader r{t, ""};
    double p0 = 101325.0, refA = 1.0, scale = 1.0;
    r.num("constant.T0", p->T0, true);
    r.num("constant.p0", p0, true);
    r.num("constant.Pr", p->Pr, true);
    r.num("constant.gamma", p->gamma, true);
    r.num("constant.referenceArea", refA, true);
    r.num("constant.mesh_scale_factor", scale, false);
    p->mesh_scale = scale;
    refA *= scale;
    p->ref_area = refA;
    // boundary states (T0 and gamma already read, p0 of the config is used for Ma input)
    {
        fvgb_params tmp = *p;
        for (auto [name, dst] : {std::pair<const char*, double*>{"inf", p->inf}, {"inlet", p->inlet}, {"outlet", p->outlet}}) {
            std::string parent = std::string("boundaryCondition.2D.") + name;
            if (r.has(parent + ".input_mode")) {
                int mode = -1;
                r.integer(parent + ".input_mode", mode, true);
                if (mode == 0) {
                    double Ma = 0, AoA = 0;
                    if (r.has(parent + ".AOA")) r.num(parent + ".AOA", AoA, true);
                    else r.num(parent + ".AoA", AoA, true);
                    r.num(parent + ".Ma", Ma, true);
                    ruvp_from_mach(dst, Ma, AoA, tmp.T0, p0, tmp.gamma, tmp.R);
                    continue;
                }
            }
            if ((rc = boundary_state(r, parent, tmp, dst))) return rc;
        }
    }
    r.integer("initialCondition.type", p->ic_type, true);
    if (p->ic_type == 2) {
        r.num("initialCondition.isentropicVortex.vortex_x", p->vortex[0], true);
        r.num("initialCondition.isentropicVortex.vortex_y", p->vortex[1], true);
        r.num("initialCondition.isentropicVortex.vortex_strength", p->vortex[2], true);
    }
    if (p->ic_type == 3) {
        r.num("initialCondition.shockTube.shock_x", p->shock[0], false);
        r.num("initialCondition.shockTube.shock_y", p->shock[1], false);
        r.num("initialCondition.shockTube.shock_normal_x", p->shock[2], false);
        r.num("initialCondition.shockTube.shock_normal_y", p->shock[3], false);
    }
    if (p->ic_type == 4) {  // FieldInitializer::initialize_using_config, FieldInitializer.cpp:93-108
        r.num("initialCondition.doubleShockReflection.shock_x", p->dsr[0], true);
        r.num("initialCondition.doubleShockReflection.shock_y", p->dsr[1], true);
        r.num("initialCondition.doubleShockReflection.shock_angle_degree", p->dsr[2], true);
        if (p->dsr[2] > 90 || p->dsr[2] < 0)
            return fail(FVGB_ERR_FORMAT, "shock_angle_degree out of range [0,90]");
    }
    {  // read_mu0_Re_from_config, TomlFileManager.cpp:79-104
        double rho_ref, U_ref;
        if (p->ic_type == 3 || p->ic_type == 4) {
            double ui = std::sqrt(p->inlet[1] * p->inlet[1] + p->inlet[2] * p->inlet[2]);
            double uo = std::sqrt(p->outlet[1] * p->outlet[1] + p->outlet[2] * p->outlet[2]);
            if (ui > uo) { rho_ref = p->inlet[0]; U_ref = ui; }
            else { rho_ref = p->outlet[0]; U_ref = uo; }
        } else {
            rho_ref = p->inf[0];
            U_ref = std::sqrt(p->inf[1] * p->inf[1] + p->inf[2] * p->inf[2]);
        }
        bool by_re = false;
        r.boolean("constant.calculate_mu0_by_Re", by_re, false);
        if (by_re) {
            r.num("constant.Re", p->Re, true);
            p->mu0 = rho_ref * U_ref * refA / p->Re;
        } else {
            r.num("constant.mu0", p->mu0, true);
            p->Re = rho_ref * U_ref * refA / p->mu0;
        }
    }
    r.integer("output.maxIteration", p->max_iteration, false);
    r.integer("physicsModel.equation", p->equation, true);
    {  // CInput::readConfig accepts only 2D (CInput.cpp:55)
        int dim = 2;
        r.integer("basic.dimension", dim, false);
        if (dim != 2) return fail(FVGB_ERR_FORMAT, "input.toml: basic.dimension must be 2");
    }
    bool steady = false;
    r.boolean("time.is_steady", steady, false);
    p->steady = steady ? 1 : 0;
    // getValueOnCondition (TomlFileManager.h:113-130, .cpp:159-160): each is read where present
    // and required only in its own mode
    r.num("time.CFL_steady", p->CFL_steady, steady);
    r.num("time.CFL", p->CFL, !steady);
    r.num("time.max_physical_time", p->T_end, true);
    r.integer("time.time_advance", p->time_advance, true);
    r.integer("inviscid_flux_method.flag_reconstruct", p->reconstruct, true);
    r.integer("inviscid_flux_method.flag_gradient", p->gradient, true);
    r.integer("inviscid_flux_method.flux_conservation_scheme", p->flux_scheme, true);
    r.integer("inviscid_flux_method.flux_limiter", p->limiter, true);
    std::string s;
    if (r.str("gpu.lsq_det", s)) p->lsq_det_ref = (s == "ref");
    if (r.str("gpu.wall_bc", s)) p->wall_bc_ref = (s == "ref");
    if (r.str("gpu.restrict", s)) p->restrict_ref = (s == "ref");
    int ren = p->renumber;
    if (r.integer("gpu.renumber", ren, false)) p->renumber = ren;
    int colour = p->edge_colour;
    if (r.integer("gpu.edge_colour", colour, false)) p->edge_colour = colour;
    int dev = 0;
    if (r.integer("gpu.device", dev, false)) p->device = dev;
    if (mesh_name && mesh_name_len > 0) {
        std::string fn;
        r.str("basic.filename", fn);
        std::snprintf(mesh_name, (size_t)mesh_name_len, "%s", fn.c_str());
    }
    if (!r.missing.empty()) return fail(FVGB_ERR_FORMAT, "input.toml: missing or mistyped keys:" + r.missing);
    return 0;
}

// The driver's keys of input.toml (TomlFileManager.cpp:110-148; defaults of
// GlobalPara.cpp:26-29, 74-82): what CDriver::start reads besides the step's parameters.
extern "C" int fvgb_run_config_read_toml(const char* path, fvgb_run_config* c) {
    if (!path || !c) return fail(FVGB_ERR_ARG, "null argument");
    Table t;
    int rc = parse(path, t);
    if (rc) return rc;
    *c = fvgb_run_config{};
    c->continue_run = 1;
    c->step_per_print = 50;
    c->step_per_output_field = 50;
    c->step_per_output_hist = 50;
    c->start_output_field = 0;
    c->max_iteration = 5000;
    c->tolerance_residual = 1.0e-7;
    c->volume_preset = 2;    // FieldWriter.h:92-93: type_ruvp_Ma, type_ruvp_Cp
    c->boundary_preset = 1;
    std::snprintf(c->filename, sizeof c->filename, "%s", "default_project");
    std::snprintf(c->mesh_file_type, sizeof c->mesh_file_type, "%s", "inp");
    Reader r{t, ""};
    bool cont = true;
    if (r.boolean("basic.continue", cont, false)) c->continue_run = cont ? 1 : 0;
    std::string sv;
    if (r.str("basic.filename", sv)) std::snprintf(c->filename, sizeof c->filename, "%s", sv.c_str());
    if (r.str("basic.meshFileType", sv)) std::snprintf(c->mesh_file_type, sizeof c->mesh_file_type, "%s", sv.c_str());
    r.integer("output.step_per_print", c->step_per_print, false);
    r.integer("output.step_per_output_field", c->step_per_output_field, false);
    r.integer("output.step_per_output_hist", c->step_per_output_hist, false);
    r.integer("output.start_output_field", c->start_output_field, false);
    r.integer("output.maxIteration", c->max_iteration, false);
    r.num("output.tolerace_residual", c->tolerance_residual, false);
    r.integer("output.outputScheme_volume_preset", c->volume_preset, false);
    r.integer("output.outputScheme_boundary_preset", c->boundary_preset, false);
    c->time_strategy = 0;
    r.integer("time.strategy", c->time_strategy, false);  // TomlFileManager.cpp:154-156
    if (c->time_strategy != 0 && c->time_strategy != 1)   // CInput.cpp:53-54
        return fail(FVGB_ERR_FORMAT, "input.toml: time.strategy is 0 (none) or 1 (adaptive CFL)");
    if (c->volume_preset < 0 || c->volume_preset > 2 || c->boundary_preset < 0 || c->boundary_preset > 2)
        return fail(FVGB_ERR_FORMAT, "input.toml: output scheme presets are 0, 1 or 2");
    if (!r.missing.empty()) return fail(FVGB_ERR_FORMAT, "input.toml: wrong type for" + r.missing);
    if (c->step_per_print <= 0 || c->step_per_output_field <= 0 || c->step_per_output_hist <= 0)
        return fail(FVGB_ERR_FORMAT, "input.toml: output.step_per_* must be positive");
    return 0;
}
