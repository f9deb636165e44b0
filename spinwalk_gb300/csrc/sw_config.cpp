// INI configuration reader with the semantics of SpinWalk's config_reader
// (src/sim/config_reader.cpp) on top of the mINI format it uses (include/ini.h, built with
// MINI_CASE_SENSITIVE, CMakeLists.txt:36). Project code: an INI tokenizer plus the key handling
// of config_reader::read / check / timing_scale.
//
//   * lines: split on '\n' ('\r' and NUL dropped, UTF-8 BOM skipped), trimmed; ';' at the start
//     is a comment; "[name]" (cut at the first ';', up to the last ']') opens a section;
//     otherwise the first '=' not written as "\=" separates key and value, both trimmed; values
//     keep any trailing text; later keys override earlier ones; keys outside a section are
//     ignored; keys and section names are case-sensitive.
//   * GENERAL.PARENT_CONFIG is read first (relative to the file), then this file's non-empty
//     values override. Vectors are read as floats and cast (str2vec, config_reader.cpp:16-23);
//     scalar times with std::stof, counts with std::stoi / std::stod, DIFFUSIVITY[i] with
//     std::stof into a double vector, P_XY rows as doubles into a float vector.
//   * FILES paths and OUTPUT_DIR are made absolute like the reference (OUTPUT_DIR against the
//     directory of the top-level file, config_reader.cpp:103-104).
#include <algorithm>
#include <cstdio>
#include <filesystem>
#include <fstream>
#include <iterator>
#include <map>
#include <sstream>
#include <string>
#include <unordered_map>
#include <vector>

#include "spinwalk_gpu.h"
#include "sw_config.h"

namespace fs = std::filesystem;

namespace sw {
namespace {

const char *kWs = " \t\n\r\f\v";

void trim(std::string &s) {
    s.erase(s.find_last_not_of(kWs) + 1);
    s.erase(0, s.find_first_not_of(kWs));
}

void replace_all(std::string &s, const std::string &a, const std::string &b) {
    if (a.empty()) return;
    size_t pos = 0;
    while ((pos = s.find(a, pos)) != std::string::npos) {
        s.replace(pos, a.size(), b);
        pos += b.size();
    }
}

using Section = std::unordered_map<std::string, std::string>;
using Ini = std::unordered_map<std::string, Section>;

bool parse_ini(const std::string &path, Ini &ini) {
    std::ifstream f(path, std::ios::in | std::ios::binary);
    if (!f.is_open()) return false;
    std::string text((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    if (text.size() >= 3 && (unsigned char)text[0] == 0xEF && (unsigned char)text[1] == 0xBB &&
        (unsigned char)text[2] == 0xBF)
        text.erase(0, 3);
    std::vector<std::string> lines;
    std::string buf;
    for (char c : text) {
        if (c == '\n') {
            lines.push_back(buf);
            buf.clear();
        } else if (c != '\0' && c != '\r') {
            buf += c;
        }
    }
    lines.push_back(buf);
    std::string section;
    bool in_section = false;
    for (std::string line : lines) {
        trim(line);
        if (line.empty() || line[0] == ';') continue;
        if (line[0] == '[') {
            std::string l = line;
            const size_t sc = l.find_first_of(';');
            if (sc != std::string::npos) l = l.substr(0, sc);
            const size_t cb = l.find_last_of(']');
            if (cb != std::string::npos) {
                section = l.substr(1, cb - 1);
                trim(section);
                ini[section];
                in_section = true;
                continue;
            }
        }
        std::string norm = line;
        replace_all(norm, "\\=", "  ");
        const size_t eq = norm.find_first_of('=');
        if (eq == std::string::npos || !in_section) continue;
        std::string key = line.substr(0, eq), value = line.substr(eq + 1);
        trim(key);
        replace_all(key, "\\=", "=");
        trim(value);
        ini[section][key] = value;
    }
    return true;
}

const std::string &get(const Ini &ini, const std::string &sec, const std::string &key) {
    static const std::string empty;
    auto s = ini.find(sec);
    if (s == ini.end()) return empty;
    auto k = s->second.find(key);
    return k == s->second.end() ? empty : k->second;
}

bool has(const Ini &ini, const std::string &sec, const std::string &key) {
    auto s = ini.find(sec);
    return s != ini.end() && s->second.count(key) == 1;
}

template <typename T>
std::vector<T> str2vec(const std::string &str) {        // config_reader.cpp:16-23
    std::istringstream ss(str);
    std::vector<T> v;
    for (std::istream_iterator<float> it(ss), end; it != end; ++it) v.push_back(static_cast<T>(*it));
    return v;
}

std::string indexed(const std::string &k, unsigned i) { return k + "[" + std::to_string(i) + "]"; }

struct Reader {
    Config &c;
    std::string top;          // the top-level file (output dir is resolved against it)
    std::string err;
    std::vector<std::string> chain;   // the files being read, outermost first

    bool read(const std::string &path) {
        if (!fs::exists(path)) {
            err = "config file does not exist: " + path;
            return false;
        }
        // a file that is its own ancestor would recurse forever (the reference's reader does);
        // here it is an error
        std::error_code ec;
        const std::string canon = fs::weakly_canonical(fs::absolute(path), ec).string();
        if (std::find(chain.begin(), chain.end(), canon) != chain.end()) {
            err = "PARENT_CONFIG cycle through " + path;
            return false;
        }
        chain.push_back(canon);
        const bool ok = read_one(path);
        chain.pop_back();
        return ok;
    }

    bool read_one(const std::string &path) {
        Ini ini;
        if (!parse_ini(path, ini)) {
            err = "failed to read config file: " + path;
            return false;
        }
        const std::string &parent = get(ini, "GENERAL", "PARENT_CONFIG");
        if (!parent.empty()) {
            fs::path pp(parent);
            if (pp.is_relative()) pp = fs::absolute(path).parent_path() / pp;
            if (!read(pp.string())) return false;
        }
        if (!get(ini, "GENERAL", "SEQ_NAME").empty()) c.seq_name = get(ini, "GENERAL", "SEQ_NAME");
        for (const char *name : {"PHANTOM", "XYZ0", "M0"}) {
            std::vector<std::string> &lst = c.files[name];
            if (has(ini, "FILES", indexed(name, 0))) lst.clear();
            for (unsigned i = 0; i < 65536 && !get(ini, "FILES", indexed(name, i)).empty(); i++)
                lst.push_back(get(ini, "FILES", indexed(name, i)));
            for (auto &p : lst)
                if (fs::path(p).is_relative())
                    p = fs::weakly_canonical(fs::absolute(path).parent_path() / p).string();
        }
        if (!get(ini, "FILES", "OUTPUT_DIR").empty()) c.output_dir = get(ini, "FILES", "OUTPUT_DIR");
        if (fs::path(c.output_dir).is_relative())
            c.output_dir = fs::weakly_canonical(fs::absolute(top).parent_path() / c.output_dir).string();

        const std::string S = "SCAN_PARAMETERS", P = "SIMULATION_PARAMETERS", T = "TISSUE_PARAMETERS";
        auto setf = [&](const std::string &sec, const char *key, auto &dst, auto conv) {
            const std::string &v = get(ini, sec, key);
            if (!v.empty()) dst = conv(v);
        };
        auto stof_ = [](const std::string &v) { return std::stof(v); };
        auto stoi_ = [](const std::string &v) { return std::stoi(v); };
        if (!get(ini, S, "TR").empty()) c.p.TR_us = (int32_t)std::stof(get(ini, S, "TR"));
        if (!get(ini, S, "TIME_STEP").empty())
            c.p.timestep_us = (int32_t)std::stof(get(ini, S, "TIME_STEP"));
        auto vec_i = [&](const char *key, std::vector<int32_t> &dst) {
            const std::string &v = get(ini, S, key);
            if (!v.empty()) dst = str2vec<int32_t>(v);
        };
        auto vec_f = [&](const char *key, std::vector<float> &dst) {
            const std::string &v = get(ini, S, key);
            if (!v.empty()) dst = str2vec<float>(v);
        };
        vec_i("TE", c.TE_us);
        vec_i("RF_T", c.RF_us);
        vec_f("RF_FA", c.RF_FA_deg);
        vec_f("RF_PH", c.RF_PH_deg);
        vec_i("DEPHASING_T", c.dephasing_us);
        vec_f("DEPHASING", c.dephasing_deg);
        vec_i("GRADIENT_T", c.gradient_us);
        vec_f("GRADIENT_X", c.gradientX_mTm);
        vec_f("GRADIENT_Y", c.gradientY_mTm);
        vec_f("GRADIENT_Z", c.gradientZ_mTm);
        setf(S, "DUMMY_SCAN", c.p.n_dummy_scan, stoi_);
        setf(S, "LINEAR_PHASE_CYCLING", c.p.linear_phase_cycling, stof_);
        setf(S, "QUADRATIC_PHASE_CYCLING", c.p.quadratic_phase_cycling, stof_);

        setf(P, "B0", c.p.B0, stof_);
        if (!get(ini, P, "SEED").empty()) c.p.seed = (uint64_t)(int64_t)std::stoi(get(ini, P, "SEED"));
        if (!get(ini, P, "NUMBER_OF_SPINS").empty())
            c.p.n_spins = (uint32_t)std::stod(get(ini, P, "NUMBER_OF_SPINS"));
        if (!get(ini, P, "CROSS_FOV").empty()) c.p.enCrossFOV = std::stoi(get(ini, P, "CROSS_FOV")) != 0;
        if (!get(ini, P, "RECORD_TRAJECTORY").empty())
            c.p.enRecordTrajectory = std::stoi(get(ini, P, "RECORD_TRAJECTORY")) != 0;
        if (!get(ini, P, "MAX_ITERATIONS").empty())
            c.p.max_iterations = (uint64_t)std::stod(get(ini, P, "MAX_ITERATIONS"));
        if (has(ini, P, "SCALE[0]")) c.scales.clear();
        for (unsigned i = 0; i < 65536 && !get(ini, P, indexed("SCALE", i)).empty(); i++)
            c.scales.push_back((float)std::stod(get(ini, P, indexed("SCALE", i))));
        c.p.n_scales = (uint32_t)c.scales.size();
        setf(P, "WHAT_TO_SCALE", c.scale_type, stoi_);

        std::vector<double> diff;
        for (unsigned i = 0; i < 65536 && !get(ini, T, indexed("DIFFUSIVITY", i)).empty(); i++)
            diff.push_back(std::stof(get(ini, T, indexed("DIFFUSIVITY", i))));
        if (!diff.empty()) c.diffusivity = diff;
        c.p.n_substrate = (uint32_t)c.diffusivity.size();
        std::vector<float> t1, t2, pxy;
        for (unsigned i = 0; i < 65536 && !get(ini, T, indexed("T1", i)).empty(); i++)
            t1.push_back(std::stof(get(ini, T, indexed("T1", i))));
        if (!t1.empty()) c.T1_ms = t1;
        for (unsigned i = 0; i < 65536 && !get(ini, T, indexed("T2", i)).empty(); i++)
            t2.push_back(std::stof(get(ini, T, indexed("T2", i))));
        if (!t2.empty()) c.T2_ms = t2;
        for (unsigned i = 0; i < 65536 && !get(ini, T, indexed("P_XY", i)).empty(); i++) {
            std::istringstream iss(get(ini, T, indexed("P_XY", i)));
            std::vector<double> row{std::istream_iterator<double>(iss), std::istream_iterator<double>()};
            pxy.insert(pxy.end(), row.begin(), row.end());
        }
        if (!pxy.empty()) c.pXY = pxy;
        return true;
    }

    // config_reader::check (config_reader.cpp:195-324)
    bool check() {
        auto bad = [&](const std::string &m) { err = m; return false; };
        if (c.RF_FA_deg.size() != c.RF_us.size() || c.RF_FA_deg.size() != c.RF_PH_deg.size())
            return bad("RF_FA, RF_PH and RF_T must have the same number of elements");
        if (c.dephasing_us.size() != c.dephasing_deg.size())
            return bad("DEPHASING and DEPHASING_T must have the same number of elements");
        if (c.gradientX_mTm.size() != c.gradientY_mTm.size() ||
            c.gradientX_mTm.size() != c.gradientZ_mTm.size())
            return bad("GRADIENTS must have the same number of elements");
        if (c.gradientX_mTm.size() != c.gradient_us.size())
            return bad("GRADIENT_XYZ and GRADIENT_T must have the same number of elements");
        if (c.T1_ms.size() != c.T2_ms.size()) return bad("T1 and T2 must have the same number of elements");
        if (c.T1_ms.size() != c.diffusivity.size())
            return bad("T1 and diffusivity must have the same number of elements");
        if (c.T1_ms.size() * c.T1_ms.size() != c.pXY.size())
            return bad("T1 and P_XY must have the same number of elements");
        if (c.scales.empty()) {
            c.scales.push_back(1.0f);
            c.p.n_scales = 1;
        }
        if (c.diffusivity.empty() || c.T1_ms.empty() || c.T2_ms.empty())
            return bad("Diffusivity, T1 and T2 must have at least one element");
        for (auto &kv : c.files)
            for (auto &p : kv.second)
                if (!fs::exists(p)) return bad("File does not exist: " + p);
        c.files["XYZ0"].resize(c.files["PHANTOM"].size(), "");
        c.files["M0"].resize(c.files["PHANTOM"].size(), "");
        try {
            fs::create_directories(fs::path(c.output_dir));
        } catch (const std::exception &e) {
            return bad("Creating directory " + c.output_dir + " failed. " + e.what());
        }
        c.outputs.clear();
        for (const auto &p : c.files["PHANTOM"]) {
            fs::path f = fs::path(c.output_dir) / (c.seq_name + "_" + fs::path(p).filename().string());
            c.outputs.push_back(f.replace_extension(".h5").string());
        }
        auto sorted_unique = [](const std::vector<int32_t> &v) {
            return std::is_sorted(v.begin(), v.end()) && std::adjacent_find(v.begin(), v.end()) == v.end();
        };
        if (c.TE_us.empty() || !sorted_unique(c.TE_us) || c.TE_us[0] < 0)
            return bad("TE must exist, be ascending, without duplicates or negative values");
        if (c.RF_us.empty() || !sorted_unique(c.RF_us) || c.RF_us[0] != 0)
            return bad("RF times must be ascending, start with 0 and have no duplicates");
        if (!sorted_unique(c.dephasing_us)) return bad("Dephasing times must be ascending without duplicates");
        if (!sorted_unique(c.gradient_us)) return bad("Gradient times must be ascending without duplicates");
        if (c.p.TR_us < 0 || c.p.timestep_us < 0) return bad("TR and timestep must be set");
        if (c.scale_type != 0 && c.scale_type != 1 && c.scale_type != 2)
            return bad("WHAT_TO_SCALE must be 0, 1, or 2");
        return true;
    }
};

void dump_vecf(FILE *f, const char *k, const std::vector<float> &v) {
    std::fprintf(f, "%s", k);
    for (float x : v) std::fprintf(f, " %.9g", x);
    std::fprintf(f, "\n");
}
void dump_veci(FILE *f, const char *k, const std::vector<int32_t> &v) {
    std::fprintf(f, "%s", k);
    for (int32_t x : v) std::fprintf(f, " %d", x);
    std::fprintf(f, "\n");
}

}  // namespace

Config::Config() {
    p = sw_params{};
    p.B0 = 9.4f;                    // defaults of struct parameters (simulation_parameters.cuh:178-201)
    p.TR_us = -1;
    p.timestep_us = -1;
    p.n_dummy_scan = 0;
    p.n_spins = 1000;
    p.n_scales = 1;
    p.seed = 0;
    p.max_iterations = 9999;
    p.enCrossFOV = 1;
    p.enRecordTrajectory = 0;
    p.fieldmap_exist = 1;
    files["PHANTOM"];
    files["XYZ0"];
    files["M0"];
}

// config_reader::prepare: read + check + timing_scale (config_reader.cpp:25-46).
int config_read(const std::string &path, Config &c, std::string &err) {
    c = Config();
    Reader r{c, path, ""};
    try {
        if (!r.read(path) || !r.check()) {
            err = r.err;
            return SW_ERR_CONFIG;
        }
    } catch (const std::exception &e) {
        err = std::string("config parse error: ") + e.what();
        return SW_ERR_CONFIG;
    }
    for (auto *v : {&c.TE_us, &c.RF_us, &c.dephasing_us, &c.gradient_us})
        for (auto &x : *v) x = x / c.p.timestep_us;
    return SW_OK;
}

// Same text layout as the test harness around the reference's config_reader.
int config_dump(const Config &c, const std::string &out) {
    FILE *f = std::fopen(out.c_str(), "w");
    if (!f) return SW_ERR_IO;
    std::fprintf(f, "ok 1\n");
    std::fprintf(f, "TR_us %d\ntimestep_us %d\nn_dummy_scan %d\n", c.p.TR_us, c.p.timestep_us,
                 c.p.n_dummy_scan);
    std::fprintf(f, "linear_phase_cycling %.9g\nquadratic_phase_cycling %.9g\n",
                 c.p.linear_phase_cycling, c.p.quadratic_phase_cycling);
    std::fprintf(f, "B0 %.9g\nseed %llu\nn_spins %u\nenCrossFOV %d\n", c.p.B0,
                 (unsigned long long)c.p.seed, c.p.n_spins, (int)(c.p.enCrossFOV != 0));
    std::fprintf(f, "enRecordTrajectory %d\nmax_iterations %llu\nn_substrate %u\n",
                 (int)(c.p.enRecordTrajectory != 0), (unsigned long long)c.p.max_iterations,
                 c.p.n_substrate);
    std::fprintf(f, "n_scales %u\nscale_type %d\n", c.p.n_scales, c.scale_type);
    std::fprintf(f, "diffusivity");
    for (double x : c.diffusivity) std::fprintf(f, " %.17g", x);
    std::fprintf(f, "\n");
    dump_vecf(f, "scales", c.scales);
    dump_vecf(f, "T1_ms", c.T1_ms);
    dump_vecf(f, "T2_ms", c.T2_ms);
    dump_vecf(f, "pXY", c.pXY);
    dump_vecf(f, "RF_FA_deg", c.RF_FA_deg);
    dump_vecf(f, "RF_PH_deg", c.RF_PH_deg);
    dump_veci(f, "RF_us", c.RF_us);
    dump_veci(f, "TE_us", c.TE_us);
    dump_vecf(f, "dephasing_deg", c.dephasing_deg);
    dump_veci(f, "dephasing_us", c.dephasing_us);
    dump_vecf(f, "gradientX_mTm", c.gradientX_mTm);
    dump_vecf(f, "gradientY_mTm", c.gradientY_mTm);
    dump_vecf(f, "gradientZ_mTm", c.gradientZ_mTm);
    dump_veci(f, "gradient_us", c.gradient_us);
    for (const char *key : {"PHANTOM", "XYZ0", "M0"}) {
        auto it = c.files.find(key);
        const size_t n = it == c.files.end() ? 0 : it->second.size();
        std::fprintf(f, "%s %zu\n", key, n);
        if (n)
            for (auto &s : it->second) std::fprintf(f, "  %s\n", s.c_str());
    }
    for (auto &o : c.outputs) std::fprintf(f, "output %s\n", o.c_str());
    std::fclose(f);
    return SW_OK;
}

}  // namespace sw

namespace sw {
namespace api {
int fail(int code, const std::string &msg);   // sets sw_last_error() (sw_api.cu)
}  // namespace api
}  // namespace sw

extern "C" int sw_config_dump(const char *ini_path, const char *out_path) {
    if (!ini_path || !out_path) return sw::api::fail(SW_ERR_INVALID, "sw_config_dump: null path");
    sw::Config c;
    std::string err;
    const int rc = sw::config_read(ini_path, c, err);
    if (rc != SW_OK) {
        FILE *f = std::fopen(out_path, "w");
        if (f) {
            std::fprintf(f, "ok 0\n");
            std::fclose(f);
        }
        return sw::api::fail(rc, err);
    }
    const int wrc = sw::config_dump(c, out_path);
    return wrc ? sw::api::fail(wrc, std::string("cannot write ") + out_path) : SW_OK;
}
