// config_json.cpp -- LbmConfig as JSON, the format of IonSolver's
// file::read_config / file::write_config (src/file.rs:310-334), which
// serialise LbmConfig (src/lbm/mod.rs:45-101) with serde_json: an object with
// the struct's field names (including the reference's spelling
// "ext_equilibrium_boudaries"), unit enum variants as strings ("D3Q19",
// "Srt", "FP16S", propellant "H"), the nested Units (src/lbm/units.rs:14-27)
// and GraphicsConfig (src/lbm/graphics.rs:101-156).
//
// Reading takes every LbmConfig field it knows, maps
// graphics_config.graphics_active to update_fields (the reference defines
// UPDATE_FIELDS exactly when graphics are active, src/lbm/domain.rs:856) and
// ignores everything else, as serde ignores unknown fields.  Writing emits
// the reference's field order with GraphicsConfig::new()'s values
// (graphics_active = update_fields) and one extra key, "field_mode", which
// the reference ignores.
#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "ionsolver.h"

namespace ion {
int api_fail(int code, const char* msg);
}

namespace {

struct JVal {
    enum Kind { NUL, BOOL, NUM, STR, ARR, OBJ } kind = NUL;
    bool b = false;
    double num = 0.0;
    std::string str;
    std::vector<JVal> arr;
    std::map<std::string, JVal> obj;
};

struct JParser {
    const std::string& s;
    size_t i = 0;
    std::string err;
    explicit JParser(const std::string& src) : s(src) {}
    void ws() {
        while (i < s.size() && std::isspace((unsigned char)s[i])) i++;
    }
    bool fail(const char* m) {
        if (err.empty()) err = std::string(m) + " at byte " + std::to_string(i);
        return false;
    }
    bool lit(const char* w) {
        const size_t n = strlen(w);
        if (s.compare(i, n, w) != 0) return fail("unexpected token");
        i += n;
        return true;
    }
    bool string(std::string& out) {
        if (i >= s.size() || s[i] != '"') return fail("expected a string");
        i++;
        out.clear();
        while (i < s.size() && s[i] != '"') {
            char c = s[i++];
            if (c == '\\') {
                if (i >= s.size()) return fail("bad escape");
                const char e = s[i++];
                switch (e) {
                    case '"': c = '"'; break;
                    case '\\': c = '\\'; break;
                    case '/': c = '/'; break;
                    case 'b': c = '\b'; break;
                    case 'f': c = '\f'; break;
                    case 'n': c = '\n'; break;
                    case 'r': c = '\r'; break;
                    case 't': c = '\t'; break;
                    case 'u': {  // keep the code unit as '?' (no field name or value needs it)
                        if (i + 4 > s.size()) return fail("bad \\u escape");
                        i += 4;
                        c = '?';
                        break;
                    }
                    default: return fail("bad escape");
                }
            }
            out.push_back(c);
        }
        if (i >= s.size()) return fail("unterminated string");
        i++;
        return true;
    }
    bool value(JVal& v, int depth) {
        if (depth > 64) return fail("nesting too deep");
        ws();
        if (i >= s.size()) return fail("unexpected end");
        const char c = s[i];
        if (c == '{') {
            v.kind = JVal::OBJ;
            i++;
            ws();
            if (i < s.size() && s[i] == '}') { i++; return true; }
            for (;;) {
                ws();
                std::string k;
                if (!string(k)) return false;
                ws();
                if (i >= s.size() || s[i] != ':') return fail("expected ':'");
                i++;
                if (!value(v.obj[k], depth + 1)) return false;
                ws();
                if (i < s.size() && s[i] == ',') { i++; continue; }
                if (i < s.size() && s[i] == '}') { i++; return true; }
                return fail("expected ',' or '}'");
            }
        }
        if (c == '[') {
            v.kind = JVal::ARR;
            i++;
            ws();
            if (i < s.size() && s[i] == ']') { i++; return true; }
            for (;;) {
                v.arr.emplace_back();
                if (!value(v.arr.back(), depth + 1)) return false;
                ws();
                if (i < s.size() && s[i] == ',') { i++; continue; }
                if (i < s.size() && s[i] == ']') { i++; return true; }
                return fail("expected ',' or ']'");
            }
        }
        if (c == '"') { v.kind = JVal::STR; return string(v.str); }
        if (c == 't') { v.kind = JVal::BOOL; v.b = true; return lit("true"); }
        if (c == 'f') { v.kind = JVal::BOOL; v.b = false; return lit("false"); }
        if (c == 'n') { v.kind = JVal::NUL; return lit("null"); }
        // number
        const char* p = s.c_str() + i;
        char* end = nullptr;
        errno = 0;
        v.num = std::strtod(p, &end);
        if (end == p) return fail("expected a value");
        v.kind = JVal::NUM;
        i += (size_t)(end - p);
        return true;
    }
};

const char* const kVelocitySets[] = {"D2Q9", "D3Q15", "D3Q19", "D3Q27"};
const char* const kRelaxation[] = {"Srt", "Trt"};
const char* const kFloatTypes[] = {"FP16S", "FP16C", "FP32"};
const char* const kPropellants[] = {"H", "He", "Ne", "Ar", "Kr", "Xe"};

int enum_index(const JVal& v, const char* const* names, int count, const char* field, int& out) {
    if (v.kind == JVal::STR) {
        for (int k = 0; k < count; k++)
            if (v.str == names[k]) { out = k; return ION_OK; }
    } else if (v.kind == JVal::NUM && v.num >= 0 && v.num < count && v.num == std::floor(v.num)) {
        out = (int)v.num;
        return ION_OK;
    }
    char m[160];
    snprintf(m, sizeof m, "Could not parse file: unknown value of \"%s\"", field);
    return ion::api_fail(ION_E_FORMAT, m);
}

// shortest decimal that reads back to the same float (serde_json writes f32 that way)
std::string fmt_f32(float x) {
    if (!std::isfinite(x)) return "null";  // serde_json writes non-finite floats as null
    char b[48];
    for (int p = 1; p <= 9; p++) {
        snprintf(b, sizeof b, "%.*g", p, (double)x);
        if (std::strtof(b, nullptr) == x) break;
    }
    std::string s(b);
    const size_t ep = s.find('e');  // "1e-06" -> "1e-6", as serde_json writes exponents
    if (ep != std::string::npos) {
        size_t k = ep + 1;
        if (k < s.size() && (s[k] == '-' || s[k] == '+')) k++;
        while (k + 1 < s.size() && s[k] == '0') s.erase(k, 1);
        if (s[ep + 1] == '+') s.erase(ep + 1, 1);
    } else if (s.find('.') == std::string::npos) {
        s += ".0";  // serde_json always marks a float: "1.0"
    }
    return s;
}

}  // namespace

extern "C" {

int ion_config_write_json(const char* path, const ion_config* c) {
    if (!path || !c) return ion::api_fail(ION_E_INVALID, "null argument");
    if (c->velocity_set < 0 || c->velocity_set > 3 || c->relaxation_time < 0 || c->relaxation_time > 1 ||
        c->float_type < 0 || c->float_type > 2 || c->units.prop < 0 || c->units.prop > 5)
        return ion::api_fail(ION_E_INVALID, "enum value out of range");
    auto B = [](int v) { return v ? "true" : "false"; };
    std::ostringstream o;
    o << "{\"velocity_set\":\"" << kVelocitySets[c->velocity_set] << "\",\"relaxation_time\":\""
      << kRelaxation[c->relaxation_time] << "\",\"float_type\":\"" << kFloatTypes[c->float_type] << "\","
      << "\"units\":{\"m\":" << fmt_f32(c->units.m) << ",\"kg\":" << fmt_f32(c->units.kg)
      << ",\"s\":" << fmt_f32(c->units.s) << ",\"a\":" << fmt_f32(c->units.a) << ",\"k\":" << fmt_f32(c->units.k)
      << ",\"prop\":\"" << kPropellants[c->units.prop] << "\"},"
      << "\"n_x\":" << c->n_x << ",\"n_y\":" << c->n_y << ",\"n_z\":" << c->n_z << ",\"d_x\":" << c->d_x
      << ",\"d_y\":" << c->d_y << ",\"d_z\":" << c->d_z << ",\"nu\":" << fmt_f32(c->nu)
      << ",\"f_x\":" << fmt_f32(c->f_x) << ",\"f_y\":" << fmt_f32(c->f_y) << ",\"f_z\":" << fmt_f32(c->f_z)
      << ",\"ext_equilibrium_boudaries\":" << B(c->ext_equilibrium_boundaries)
      << ",\"ext_volume_force\":" << B(c->ext_volume_force) << ",\"ext_force_field\":" << B(c->ext_force_field)
      << ",\"ext_magneto_hydro\":" << B(c->ext_magneto_hydro) << ",\"ext_subgrid_ecr\":" << B(c->ext_subgrid_ecr)
      << ",\"mhd_lod_depth\":" << (unsigned)c->mhd_lod_depth << ",\"ecr_freq\":" << fmt_f32(c->ecr_freq)
      << ",\"ecr_field_strength\":" << fmt_f32(c->ecr_field_strength)
      // GraphicsConfig::new() (src/lbm/graphics.rs:158-192), graphics_active = update_fields
      << ",\"graphics_config\":{\"graphics_active\":" << B(c->update_fields)
      << ",\"background_color\":0,\"camera_width\":1920,\"camera_height\":1080,\"v_max\":0.25,\"q_min\":0.0001,"
         "\"f_max\":0.002,\"rho_delta\":0.5,\"streamline_every\":4,\"stream_line_lenght\":128,\"vec_vis_mode\":\"U\","
         "\"slice_mode\":\"Off\",\"slice_x\":0,\"slice_y\":0,\"slice_z\":0,\"max_slice_x\":0,\"max_slice_y\":0,"
         "\"max_slice_z\":0,\"field_vis\":\"Vector\",\"streamline_mode\":false,\"field_mode\":false,"
         "\"field_slice_mode\":false,\"q_mode\":false,\"q_field_mode\":false,\"flags_mode\":false,"
         "\"flags_surface_mode\":false,\"axes_mode\":false,\"ecrc_mode\":false,\"render_intervals\":false,"
         "\"keyframes\":[]}"
      << ",\"run_steps\":" << (unsigned long long)c->run_steps << ",\"field_mode\":" << (unsigned)c->field_mode << "}";
    std::ofstream f(path, std::ios::binary);
    if (!f) return ion::api_fail(ION_E_IO, "Could not create file.");
    const std::string s = o.str();
    f.write(s.data(), (std::streamsize)s.size());
    if (!f) return ion::api_fail(ION_E_IO, "Could not write file.");
    return ION_OK;
}

int ion_config_read_json(const char* path, ion_config* out) {
    if (!path || !out) return ion::api_fail(ION_E_INVALID, "null argument");
    std::ifstream f(path, std::ios::binary);
    if (!f) return ion::api_fail(ION_E_IO, "Could not find file.");
    const std::string text((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    JVal root;
    JParser p(text);
    if (!p.value(root, 0)) return ion::api_fail(ION_E_FORMAT, ("Could not parse file: " + p.err).c_str());
    p.ws();
    if (p.i != text.size()) return ion::api_fail(ION_E_FORMAT, "Could not parse file: trailing characters");
    if (root.kind != JVal::OBJ) return ion::api_fail(ION_E_FORMAT, "Could not parse file: not an object");
    ion_config c;
    ion_config_default(&c);
    const auto& o = root.obj;
    auto num = [&](const std::map<std::string, JVal>& m, const char* k, double& v) -> int {
        auto it = m.find(k);
        if (it == m.end()) return ION_E_FORMAT;
        if (it->second.kind != JVal::NUM) return ION_E_FORMAT;
        v = it->second.num;
        return ION_OK;
    };
    auto need = [&](const char* k) -> int {
        char m[160];
        snprintf(m, sizeof m, "Could not parse file: missing or invalid field `%s`", k);
        return ion::api_fail(ION_E_FORMAT, m);
    };
    double d = 0.0;
    int e = 0;
    auto it = o.find("velocity_set");
    if (it == o.end()) return need("velocity_set");
    if (int rc = enum_index(it->second, kVelocitySets, 4, "velocity_set", e)) return rc;
    c.velocity_set = e;
    it = o.find("relaxation_time");
    if (it == o.end()) return need("relaxation_time");
    if (int rc = enum_index(it->second, kRelaxation, 2, "relaxation_time", e)) return rc;
    c.relaxation_time = e;
    it = o.find("float_type");
    if (it == o.end()) return need("float_type");
    if (int rc = enum_index(it->second, kFloatTypes, 3, "float_type", e)) return rc;
    c.float_type = e;
    it = o.find("units");
    if (it == o.end() || it->second.kind != JVal::OBJ) return need("units");
    {
        const auto& u = it->second.obj;
        float* dst[5] = {&c.units.m, &c.units.kg, &c.units.s, &c.units.a, &c.units.k};
        const char* names[5] = {"m", "kg", "s", "a", "k"};
        for (int k = 0; k < 5; k++) {
            if (num(u, names[k], d)) return need(names[k]);
            *dst[k] = (float)d;
        }
        auto pi = u.find("prop");
        if (pi == u.end()) return need("prop");
        if (int rc = enum_index(pi->second, kPropellants, 6, "prop", e)) return rc;
        c.units.prop = e;
    }
    struct U32 { const char* k; uint32_t* v; } u32s[] = {{"n_x", &c.n_x}, {"n_y", &c.n_y}, {"n_z", &c.n_z},
                                                         {"d_x", &c.d_x}, {"d_y", &c.d_y}, {"d_z", &c.d_z}};
    for (auto& f32 : u32s) {
        if (num(o, f32.k, d) || d < 0 || d > 4294967295.0 || d != std::floor(d)) return need(f32.k);
        *f32.v = (uint32_t)d;
    }
    struct F32 { const char* k; float* v; } f32s[] = {{"nu", &c.nu}, {"f_x", &c.f_x}, {"f_y", &c.f_y}, {"f_z", &c.f_z},
                                                      {"ecr_freq", &c.ecr_freq},
                                                      {"ecr_field_strength", &c.ecr_field_strength}};
    for (auto& f : f32s) {
        if (num(o, f.k, d)) return need(f.k);
        *f.v = (float)d;
    }
    struct Bool { const char* k; uint8_t* v; } bools[] = {{"ext_equilibrium_boudaries", &c.ext_equilibrium_boundaries},
                                                          {"ext_volume_force", &c.ext_volume_force},
                                                          {"ext_force_field", &c.ext_force_field},
                                                          {"ext_magneto_hydro", &c.ext_magneto_hydro},
                                                          {"ext_subgrid_ecr", &c.ext_subgrid_ecr}};
    for (auto& b : bools) {
        auto bi = o.find(b.k);
        if (bi == o.end() || bi->second.kind != JVal::BOOL) return need(b.k);
        *b.v = bi->second.b ? 1 : 0;
    }
    if (num(o, "mhd_lod_depth", d) || d < 0 || d > 255 || d != std::floor(d)) return need("mhd_lod_depth");
    c.mhd_lod_depth = (uint8_t)d;
    if (num(o, "run_steps", d) || d < 0 || d != std::floor(d)) return need("run_steps");
    c.run_steps = (uint64_t)d;
    it = o.find("graphics_config");
    if (it == o.end() || it->second.kind != JVal::OBJ) return need("graphics_config");
    {
        auto gi = it->second.obj.find("graphics_active");
        if (gi == it->second.obj.end() || gi->second.kind != JVal::BOOL) return need("graphics_active");
        c.update_fields = gi->second.b ? 1 : 0;
    }
    it = o.find("field_mode");  // this library's key (absent in the reference's files)
    if (it != o.end() && it->second.kind == JVal::NUM && it->second.num >= 0 && it->second.num <= 2)
        c.field_mode = (uint8_t)it->second.num;
    *out = c;
    return ION_OK;
}

}  // extern "C"
