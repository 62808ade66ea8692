// host_io.cpp -- host side of libpms: config.txt parsing, parameter and grid
// derivation, legacy-VTK particle frames in, PLY meshes and diffuse VTK out,
// and the VisGPU frame loop.
//
//   config:  Params.cpp:24-152 with inih's rules (ini.c:60-181, INIReader.cpp)
//   grid:    FileData.cpp:240-279 (NOBOUND)
//   VTK in:  FileData.cpp:177-305 (vtkPolyDataReader, arrays "Vel" and "Rhop")
//   PLY out: FileData.cpp:1277-1332 (tinyply 2.3, ASCII)
//   diffuse: FileData.cpp:945-1036 (vtkPolyDataWriter, binary)
//   loop:    GPUPOST.cpp:34-91
#include "pms_internal.h"

#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdlib>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <thread>
#include <vector>
#include <algorithm>

// ---------------------------------------------------------------------------
// INI parsing
// ---------------------------------------------------------------------------
namespace {

std::string lower(std::string s) {
    for (char& ch : s) ch = (char)std::tolower((unsigned char)ch);
    return s;
}

std::string rstrip(const std::string& s) {
    size_t e = s.size();
    while (e > 0 && std::isspace((unsigned char)s[e - 1])) --e;
    return s.substr(0, e);
}

size_t lskip(const std::string& s, size_t i) {
    while (i < s.size() && std::isspace((unsigned char)s[i])) ++i;
    return i;
}

// first occurrence of c, or of a ';' preceded by whitespace (an inline comment)
size_t find_char_or_comment(const std::string& s, size_t i, char c) {
    bool was_ws = false;
    for (; i < s.size(); ++i) {
        if (s[i] == c || (was_ws && s[i] == ';')) return i;
        was_ws = std::isspace((unsigned char)s[i]) != 0;
    }
    return s.size();
}

struct Ini {
    std::map<std::string, std::string> values;   // "section.name" (lower case) -> value
    bool load(const char* path) {
        std::ifstream f(path);
        if (!f) return false;
        std::string line, section, prev_name;
        int lineno = 0;
        while (std::getline(f, line)) {
            ++lineno;
            if (lineno == 1 && line.size() >= 3 && (unsigned char)line[0] == 0xEF && (unsigned char)line[1] == 0xBB &&
                (unsigned char)line[2] == 0xBF)
                line = line.substr(3);
            if (!line.empty() && line.back() == '\r') line.pop_back();
            std::string r = rstrip(line);
            size_t st = lskip(r, 0);
            std::string s = r.substr(st);
            if (s.empty()) continue;
            if (s[0] == ';' || s[0] == '#') continue;
            if (!prev_name.empty() && st > 0) {         // continuation line
                add(section, prev_name, s);
                continue;
            }
            if (s[0] == '[') {
                size_t e = find_char_or_comment(s, 1, ']');
                if (e < s.size() && s[e] == ']') { section = s.substr(1, e - 1); prev_name.clear(); }
                continue;
            }
            size_t e = find_char_or_comment(s, 0, '=');
            if (e >= s.size() || s[e] != '=') e = find_char_or_comment(s, 0, ':');
            if (e < s.size() && (s[e] == '=' || s[e] == ':')) {
                std::string name = rstrip(s.substr(0, e));
                std::string value = s.substr(lskip(s, e + 1));
                size_t ce = find_char_or_comment(value, 0, '\0');
                if (ce < value.size() && value[ce] == ';') value = value.substr(0, ce);
                value = rstrip(value);
                prev_name = name;
                add(section, name, value);
            }
            // lines without '=' or ':' are parse errors that inih records and skips
        }
        return true;
    }
    void add(const std::string& sec, const std::string& name, const std::string& v) {
        std::string k = lower(sec + "." + name);
        auto it = values.find(k);
        if (it != values.end() && !it->second.empty()) it->second += "\n" + v;
        else values[k] = v;
    }
    std::string get(const char* sec, const char* name, const std::string& def) const {
        auto it = values.find(lower(std::string(sec) + "." + name));
        return it == values.end() ? def : it->second;
    }
    double real(const char* sec, const char* name, double def) const {
        std::string v = get(sec, name, "");
        const char* p = v.c_str();
        char* end = nullptr;
        double d = std::strtod(p, &end);
        return end > p ? d : def;
    }
    long integer(const char* sec, const char* name, long def) const {
        std::string v = get(sec, name, "");
        const char* p = v.c_str();
        char* end = nullptr;
        long d = std::strtol(p, &end, 0);
        return end > p ? d : def;
    }
    bool boolean(const char* sec, const char* name, bool def) const {
        std::string v = lower(get(sec, name, ""));
        if (v == "true" || v == "yes" || v == "on" || v == "1") return true;
        if (v == "false" || v == "no" || v == "off" || v == "0") return false;
        return def;
    }
};

void copy_str(char* dst, size_t cap, const std::string& s) {
    size_t n = std::min(cap - 1, s.size());
    memcpy(dst, s.data(), n);
    dst[n] = 0;
}

}  // namespace

extern "C" pms_status pms_config_default(pms_config* c) {
    if (!c) return PMS_ERR_INVALID_ARGUMENT;
    memset(c, 0, sizeof(*c));
    // Params.cpp:31-125 defaults
    c->gpu_id = 0;
    c->frame_start = 0; c->frame_end = 10; c->frame_step = 1; c->num_zeros = 4;
    copy_str(c->fluid_path, sizeof(c->fluid_path), "../flow/particles/");
    copy_str(c->fluid_prefix, sizeof(c->fluid_prefix), "PartFluid_");
    copy_str(c->surface_path, sizeof(c->surface_path), "../flow/particles/");
    copy_str(c->surface_prefix, sizeof(c->surface_prefix), "PartSurfaceTest_");
    copy_str(c->diffuse_path, sizeof(c->diffuse_path), "../flow/particles/");
    copy_str(c->diffuse_prefix, sizeof(c->diffuse_prefix), "PartDiffuse_");
    c->is_diffuse = 1; c->is_surface = 0;
    c->mass = 0; c->particle_spacing = 0.01;
    c->smoothing_radius_ratio = 4;
    c->min_num_neighbors = 8; c->isolate_num_neighbors = 4;
    c->lambda_for_smoothed = 0.5; c->iso_value = 0.5;
    c->min_wave_crests = 0; c->max_wave_crests = 100;
    c->min_trapped_air = 0; c->max_trapped_air = 100;
    c->min_kinetic_energy = 0; c->max_kinetic_energy = 100;
    c->trapped_air_multiplier = 800; c->wave_crests_multiplier = 4000;
    c->time_step = 0.01; c->life_time = 10; c->buoyancy_control = 0.8; c->drag_control = 0.5;
    c->sp_scale = 2; c->sc_scale = 2;
    for (int k = 0; k < 3; ++k) { c->domain_min[k] = 0; c->domain_max[k] = 3; }
    c->fp64_svd_cond = 1e6;
    c->rng_seed = 4;
    return PMS_OK;
}

extern "C" pms_status pms_config_load(const char* path, pms_config* c) {
    if (!path || !c) return PMS_ERR_INVALID_ARGUMENT;
    pms_config_default(c);
    Ini ini;
    if (!ini.load(path)) return PMS_ERR_CONFIG;
    // Params.cpp:31-106; integer fields read with GetReal are truncated
    c->gpu_id = (int)ini.real("Config", "GpuId", 0);
    c->frame_start = (int)ini.real("Config", "Framefrom", 0);
    c->frame_end = (int)ini.real("Config", "Frameto", 10);
    c->frame_step = (int)ini.real("Config", "FrameStep", 1);
    c->num_zeros = (int)ini.real("Config", "NumZeros", 4);
    copy_str(c->fluid_path, sizeof(c->fluid_path), ini.get("Config", "FluidPath", "../flow/particles/"));
    copy_str(c->fluid_prefix, sizeof(c->fluid_prefix), ini.get("Config", "FluidPrefix", "PartFluid_"));
    copy_str(c->surface_path, sizeof(c->surface_path), ini.get("Config", "SurfacePath", "../flow/particles/"));
    copy_str(c->surface_prefix, sizeof(c->surface_prefix), ini.get("Config", "SurfacePrefix", "PartSurfaceTest_"));
    copy_str(c->diffuse_path, sizeof(c->diffuse_path), ini.get("Config", "DiffusePath", "../flow/particles/"));
    copy_str(c->diffuse_prefix, sizeof(c->diffuse_prefix), ini.get("Config", "DiffusePrefix", "PartDiffuse_"));
    c->is_diffuse = ini.boolean("Config", "IsDiffuseGeneration", true);
    c->is_surface = ini.boolean("Config", "IsSurfaceReconstruct", false);
    c->mass = ini.real("Sim", "Mass", 0);
    c->particle_spacing = ini.real("Sim", "ParticleSpacing", 0.01);
    c->smoothing_radius_ratio = ini.real("Surface", "SmoothingRadiusRatio", 4);
    c->min_num_neighbors = ini.integer("Surface", "MinNumNeighbors", 8);
    c->isolate_num_neighbors = ini.integer("Surface", "IsolateNumNeighbors", 4);
    c->lambda_for_smoothed = ini.real("Surface", "LambdaForSmoothed", 0.5);
    c->iso_value = ini.real("Surface", "IsoValue", 0.5);
    c->min_wave_crests = ini.real("Diffuse", "MinWaveCrestsThreshold", 0);
    c->max_wave_crests = ini.real("Diffuse", "MaxWaveCrestsThreshold", 100);
    c->min_trapped_air = ini.real("Diffuse", "MinTrappedAirThreshold", 0);
    c->max_trapped_air = ini.real("Diffuse", "MaxTrappedAirThreshold", 100);
    c->min_kinetic_energy = ini.real("Diffuse", "MinKineticEnergyThreshold", 0);
    c->max_kinetic_energy = ini.real("Diffuse", "MaxKineticEnergyThreshold", 100);
    c->trapped_air_multiplier = ini.real("Diffuse", "DiffuseTrappedAirMultiplier", 800);
    c->wave_crests_multiplier = ini.real("Diffuse", "DiffuseWaveCrestsMultiplier", 4000);
    c->time_step = ini.real("Diffuse", "TimeStep", 0.01);
    c->life_time = ini.real("Diffuse", "LifefimeMultiplier", 10);
    c->buoyancy_control = ini.real("Diffuse", "BuoyancyControl", 0.8);
    c->drag_control = ini.real("Diffuse", "DragControl", 0.5);
    c->sp_scale = ini.real("Domain", "SpatialGridSizeScale", 2);
    c->sc_scale = ini.real("Domain", "SclarGridSizeScale", 2);
    const char* mins[3] = {"Min_x", "Min_y", "Min_z"};
    const char* maxs[3] = {"Max_x", "Max_y", "Max_z"};
    for (int k = 0; k < 3; ++k) { c->domain_min[k] = ini.real("Domain", mins[k], 0); c->domain_max[k] = ini.real("Domain", maxs[k], 3); }
    // additions of this build (not in the reference): [GB300] section
    c->fp64_svd_cond = ini.real("GB300", "Fp64SvdCondition", 1e6);
    c->rng_seed = (uint64_t)ini.real("GB300", "RandomSeed", 4);
    copy_str(c->band_model, sizeof(c->band_model), ini.get("GB300", "BandModel", ""));
    c->ply_binary = ini.boolean("GB300", "PlyBinary", false) ? 1 : 0;
    c->weld_mesh = ini.boolean("GB300", "WeldMesh", false) ? 1 : 0;
    return PMS_OK;
}

// ---------------------------------------------------------------------------
// Params.cpp:53-118, float32 as the reference's structs hold them
// ---------------------------------------------------------------------------
extern "C" pms_status pms_params_derive(const pms_config* c, pms_params* p) {
    if (!c || !p) return PMS_ERR_INVALID_ARGUMENT;
    memset(p, 0, sizeof(*p));
    p->mass = (float)c->mass;
    p->particle_spacing = (float)c->particle_spacing;
    p->smoothing_radius_ratio = (int)c->smoothing_radius_ratio;
    p->h = (float)p->smoothing_radius_ratio * p->particle_spacing;      // int * float
    p->h_inv = (float)(1.0 / (double)p->h);
    p->h_sq = p->h * p->h;
    p->aniso_radius = p->h * 2.0f;
    p->min_num_neighbors = (int)c->min_num_neighbors;
    p->isolate_num_neighbors = (int)c->isolate_num_neighbors;
    p->lambda_for_smoothed = (float)c->lambda_for_smoothed;
    p->iso_value = (float)c->iso_value;
    p->hd = (float)(1.732 * (double)p->particle_spacing);
    p->hd_inv = (float)(1.0 / (double)p->hd);
    p->hd_sq = p->hd * p->hd;
    p->hd_aniso = p->hd * 2.0f;
    {
        // (4 / 3) * PI * powf(spacing / 2, 3) * 315 / (64 * PI * powf(hd, 9)), float32,
        // left to right, with the integer division 4 / 3 == 1
        const float kPi = 3.14159265f;
        float num = 1.0f * kPi;
        num = num * powf(p->particle_spacing / 2.0f, 3.0f);
        num = num * 315.0f;
        float den = 64.0f * kPi;
        den = den * powf(p->hd, 9.0f);
        p->coefficient = num / den;
    }
    p->d_min_num_neighbors = (int)(signed char)c->min_num_neighbors;
    p->min_wc = (float)c->min_wave_crests; p->max_wc = (float)c->max_wave_crests;
    p->min_ta = (float)c->min_trapped_air; p->max_ta = (float)c->max_trapped_air;
    p->min_ke = (float)c->min_kinetic_energy; p->max_ke = (float)c->max_kinetic_energy;
    p->ta_mult = (int)c->trapped_air_multiplier;
    p->wc_mult = (int)c->wave_crests_multiplier;
    p->time_step = (float)c->time_step;
    p->life_time = (int)c->life_time;
    p->buoyancy = (float)c->buoyancy_control;
    p->drag = (float)c->drag_control;
    p->sp_scale = (int)c->sp_scale;
    p->sc_scale = (int)c->sc_scale;
    if (p->sc_scale == 0 || p->particle_spacing <= 0.f || p->smoothing_radius_ratio <= 0) return PMS_ERR_CONFIG;
    p->sp_grid_size = (float)((double)p->particle_spacing * 1.5);
    p->sc_grid_size = p->particle_spacing / (float)p->sc_scale;
    p->spexpand = (int)ceilf(p->h / p->sp_grid_size);
    p->scexpand = (int)ceilf(p->h / p->sc_grid_size);
    p->spexpand_diffuse = (int)ceilf(p->hd / p->sp_grid_size);
    return PMS_OK;
}

static uint32_t f2u_sat(float x) {
    if (!(x > 0.0f)) return 0u;
    if (x >= 4294967296.0f) return 0xffffffffu;
    return (uint32_t)x;
}

extern "C" pms_status pms_grid_from_bbox(const pms_params* p, const float bmin[3], const float bmax[3], pms_grid* g) {
    if (!p || !bmin || !bmax || !g) return PMS_ERR_INVALID_ARGUMENT;
    memset(g, 0, sizeof(*g));
    const float two_h = 2.0f * p->h, four_h = 4.0f * p->h;
    for (int k = 0; k < 3; ++k) {
        g->scmin_pos[k] = bmin[k] - two_h;
        g->scmax_pos[k] = bmax[k] + two_h;
        g->min_pos[k] = bmin[k] - four_h;
        g->max_pos[k] = bmax[k] + four_h;
    }
    g->sp_grid_size = p->sp_grid_size;
    g->sc_grid_size = p->sc_grid_size;
    uint64_t sp = 1, sc = 1;
    for (int k = 0; k < 3; ++k) {
        float a = (g->max_pos[k] - g->min_pos[k]) / g->sp_grid_size;
        g->spres[k] = f2u_sat(a);
        float b = (g->scmax_pos[k] - g->scmin_pos[k]) / g->sc_grid_size;
        double bd = (double)b + 0.5;
        g->scres[k] = bd >= 4294967295.0 ? 0xffffffffu : (uint32_t)bd;
        sp *= g->spres[k];
        sc *= g->scres[k];
    }
    g->spexpand = p->spexpand;
    g->scexpand = p->scexpand;
    g->spexpand_diffuse = p->spexpand_diffuse;
    g->sp_size = (uint32_t)sp;
    g->sc_size = (uint32_t)sc;
    if (sp >= (1ull << 32) || sc >= (1ull << 32)) return PMS_ERR_UNSUPPORTED;
    return PMS_OK;
}

// ---------------------------------------------------------------------------
// legacy VTK
// ---------------------------------------------------------------------------
namespace {

struct Reader {
    std::vector<char> buf;
    size_t pos = 0;
    bool binary = false;
    bool load(const char* path) {
        std::ifstream f(path, std::ios::binary);
        if (!f) return false;
        f.seekg(0, std::ios::end);
        std::streamoff sz = f.tellg();
        if (sz < 0) return false;
        f.seekg(0);
        buf.resize((size_t)sz);
        if (sz) f.read(buf.data(), sz);
        return (bool)f || f.eof();
    }
    bool eof() const { return pos >= buf.size(); }
    std::string line() {
        size_t s = pos;
        while (pos < buf.size() && buf[pos] != '\n') ++pos;
        std::string r(buf.data() + s, pos - s);
        if (pos < buf.size()) ++pos;
        if (!r.empty() && r.back() == '\r') r.pop_back();
        return r;
    }
    std::string token() {
        while (pos < buf.size() && std::isspace((unsigned char)buf[pos])) ++pos;
        size_t s = pos;
        while (pos < buf.size() && !std::isspace((unsigned char)buf[pos])) ++pos;
        return std::string(buf.data() + s, pos - s);
    }
    // binary payload starts after the newline that ends the header line
    void to_payload() {
        while (pos < buf.size() && buf[pos] != '\n') ++pos;
        if (pos < buf.size()) ++pos;
    }
};

size_t type_size(const std::string& t) {
    if (t == "float") return 4;
    if (t == "double") return 8;
    if (t == "int" || t == "unsigned_int") return 4;
    if (t == "short" || t == "unsigned_short") return 2;
    if (t == "char" || t == "unsigned_char" || t == "bit") return 1;
    if (t == "long" || t == "unsigned_long" || t == "vtktypeint64" || t == "vtktypeuint64") return 8;
    return 0;
}

double load_be(const char* p, const std::string& t) {
    unsigned char b[8];
    size_t n = type_size(t);
    for (size_t i = 0; i < n; ++i) b[i] = (unsigned char)p[n - 1 - i];
    if (t == "float") { float f; memcpy(&f, b, 4); return f; }
    if (t == "double") { double d; memcpy(&d, b, 8); return d; }
    if (t == "int") { int32_t v; memcpy(&v, b, 4); return v; }
    if (t == "unsigned_int") { uint32_t v; memcpy(&v, b, 4); return v; }
    if (t == "short") { int16_t v; memcpy(&v, b, 2); return v; }
    if (t == "unsigned_short") { uint16_t v; memcpy(&v, b, 2); return v; }
    if (t == "char") { return (double)(int8_t)b[0]; }
    if (t == "unsigned_char" || t == "bit") { return b[0]; }
    if (t == "long" || t == "vtktypeint64") { int64_t v; memcpy(&v, b, 8); return (double)v; }
    { uint64_t v; memcpy(&v, b, 8); return (double)v; }
}

// f(begin, end) over [0, n) split across the host's threads (one chunk when small)
template <class F>
void parallel_ranges(size_t n, F&& f) {
    const unsigned hw = std::thread::hardware_concurrency();
    const size_t T = std::max<size_t>(1, std::min<size_t>(hw ? hw : 1, n / 262144 + 1));
    if (T == 1) { f(0, n); return; }
    std::vector<std::thread> th;
    for (size_t c = 0; c < T; ++c) th.emplace_back([&, c]() { f(n * c / T, n * (c + 1) / T); });
    for (std::thread& t : th) t.join();
}

// reads count values of type t as doubles (ascii or big-endian binary); the binary
// decode and the ASCII number parsing run on all host threads
bool read_values(Reader& r, const std::string& t, size_t count, std::vector<double>* out) {
    if (out) out->resize(count);
    if (r.binary) {
        const size_t ts = type_size(t);
        if (!ts) return false;
        r.to_payload();
        if (r.pos + ts * count > r.buf.size()) return false;
        if (out) {
            const char* base = r.buf.data() + r.pos;
            double* o = out->data();
            if (t == "float")
                parallel_ranges(count, [&](size_t a, size_t b) {
                    for (size_t i = a; i < b; ++i) {
                        const unsigned char* q = reinterpret_cast<const unsigned char*>(base + 4 * i);
                        const uint32_t u = (uint32_t)q[0] << 24 | (uint32_t)q[1] << 16 | (uint32_t)q[2] << 8 | q[3];
                        float f;
                        memcpy(&f, &u, 4);
                        o[i] = f;
                    }
                });
            else if (t == "double")
                parallel_ranges(count, [&](size_t a, size_t b) {
                    for (size_t i = a; i < b; ++i) {
                        const unsigned char* q = reinterpret_cast<const unsigned char*>(base + 8 * i);
                        uint64_t u = 0;
                        for (int k = 0; k < 8; ++k) u = u << 8 | q[k];
                        double d;
                        memcpy(&d, &u, 8);
                        o[i] = d;
                    }
                });
            else
                parallel_ranges(count, [&](size_t a, size_t b) {
                    for (size_t i = a; i < b; ++i) o[i] = load_be(base + ts * i, t);
                });
        }
        r.pos += ts * count;
        return true;
    }
    // ASCII: the token starts in one pass, then the numbers in parallel
    std::vector<size_t> starts(count);
    for (size_t i = 0; i < count; ++i) {
        while (r.pos < r.buf.size() && std::isspace((unsigned char)r.buf[r.pos])) ++r.pos;
        if (r.pos >= r.buf.size()) return false;
        starts[i] = r.pos;
        while (r.pos < r.buf.size() && !std::isspace((unsigned char)r.buf[r.pos])) ++r.pos;
    }
    if (out) {
        double* o = out->data();
        parallel_ranges(count, [&](size_t a, size_t b) {
            std::string tok;
            for (size_t i = a; i < b; ++i) {
                size_t e = starts[i];
                while (e < r.buf.size() && !std::isspace((unsigned char)r.buf[e])) ++e;
                tok.assign(r.buf.data() + starts[i], e - starts[i]);
                o[i] = std::strtod(tok.c_str(), nullptr);
            }
        });
    }
    return true;
}

}  // namespace

extern "C" pms_status pms_read_vtk_particles(const char* path, float** pos_out, float** vel_out, float** rho_out,
                                             uint32_t* n_out) {
    if (!path || !pos_out || !n_out) return PMS_ERR_INVALID_ARGUMENT;
    *pos_out = nullptr;
    if (vel_out) *vel_out = nullptr;
    if (rho_out) *rho_out = nullptr;
    *n_out = 0;
    Reader r;
    if (!r.load(path)) return PMS_ERR_IO;
    std::string l0 = r.line();
    if (l0.find("vtk") == std::string::npos) return PMS_ERR_IO;
    r.line();                                        // title
    std::string fmt = lower(rstrip(r.line()));
    r.binary = fmt.find("binary") != std::string::npos;
    std::vector<double> pts, vel, rho;
    size_t npts = 0;
    while (!r.eof()) {
        std::string kw = r.token();
        if (kw.empty()) break;
        std::string KW = lower(kw);
        if (KW == "dataset") { r.token(); continue; }
        if (KW == "points") {
            npts = std::strtoull(r.token().c_str(), nullptr, 10);
            std::string t = r.token();
            if (!read_values(r, t, 3 * npts, &pts)) return PMS_ERR_IO;
        } else if (KW == "vertices" || KW == "lines" || KW == "polygons" || KW == "triangle_strips") {
            size_t a = std::strtoull(r.token().c_str(), nullptr, 10);
            size_t b = std::strtoull(r.token().c_str(), nullptr, 10);
            size_t save = r.pos;
            std::string next = lower(r.token());
            if (next == "offsets") {                   // VTK 5.1 cell layout
                std::string t = r.token();
                if (!read_values(r, t, a, nullptr)) return PMS_ERR_IO;
                std::string kc = lower(r.token());
                std::string t2 = r.token();
                if (kc != "connectivity" || !read_values(r, t2, b, nullptr)) return PMS_ERR_IO;
            } else {
                r.pos = save;
                if (!read_values(r, "int", b, nullptr)) return PMS_ERR_IO;
            }
        } else if (KW == "point_data" || KW == "cell_data") {
            r.token();
        } else if (KW == "scalars") {
            std::string name = r.token(), t = r.token();
            size_t save = r.pos;
            std::string maybe = r.token();
            size_t nc = 1;
            if (!maybe.empty() && std::isdigit((unsigned char)maybe[0])) nc = std::strtoul(maybe.c_str(), nullptr, 10);
            else r.pos = save;
            std::string lt = r.token();                // LOOKUP_TABLE
            r.token();                                  // table name
            (void)lt;
            std::vector<double> v;
            if (!read_values(r, t, nc * npts, &v)) return PMS_ERR_IO;
            if (name == "Rhop") rho.swap(v);
        } else if (KW == "vectors" || KW == "normals") {
            std::string name = r.token(), t = r.token();
            std::vector<double> v;
            if (!read_values(r, t, 3 * npts, &v)) return PMS_ERR_IO;
            if (name == "Vel") vel.swap(v);
        } else if (KW == "field") {
            r.token();
            int na = std::atoi(r.token().c_str());
            for (int a = 0; a < na; ++a) {
                std::string name = r.token();
                size_t nc = std::strtoull(r.token().c_str(), nullptr, 10);
                size_t nt = std::strtoull(r.token().c_str(), nullptr, 10);
                std::string t = r.token();
                std::vector<double> v;
                if (!read_values(r, t, nc * nt, &v)) return PMS_ERR_IO;
                if (name == "Vel" && nc == 3) vel.swap(v);
                if (name == "Rhop" && nc == 1) rho.swap(v);
            }
        } else if (KW == "metadata") {
            // VTK 9 writes an INFORMATION block terminated by an empty line
            while (!r.eof()) { std::string ln = r.line(); if (rstrip(ln).empty() && r.pos > 0) break; }
        } else if (KW == "lookup_table" || KW == "color_scalars" || KW == "texture_coordinates" || KW == "tensors") {
            return PMS_ERR_IO;
        }
    }
    if (npts == 0 || pts.size() != 3 * npts) {
        if (npts == 0) { *n_out = 0; return PMS_OK; }
        return PMS_ERR_IO;
    }
    if (npts >= (1ull << 32)) return PMS_ERR_UNSUPPORTED;
    float* P = (float*)malloc(12 * npts);
    float* V = (float*)malloc(12 * npts);
    float* R = (float*)malloc(4 * npts);
    if (!P || !V || !R) { free(P); free(V); free(R); return PMS_ERR_OUT_OF_MEMORY; }
    for (size_t i = 0; i < 3 * npts; ++i) P[i] = (float)pts[i];
    for (size_t i = 0; i < 3 * npts; ++i) V[i] = vel.size() == 3 * npts ? (float)vel[i] : 0.f;
    for (size_t i = 0; i < npts; ++i) R[i] = rho.size() == npts ? (float)rho[i] : 0.f;
    *pos_out = P;
    if (vel_out) *vel_out = V; else free(V);
    if (rho_out) *rho_out = R; else free(R);
    *n_out = (uint32_t)npts;
    return PMS_OK;
}

extern "C" void pms_free_host(void* p) { free(p); }

namespace {
void put_be32(std::string& s, const void* v) {
    const unsigned char* b = (const unsigned char*)v;
    s.push_back((char)b[3]); s.push_back((char)b[2]); s.push_back((char)b[1]); s.push_back((char)b[0]);
}
}  // namespace

extern "C" pms_status pms_write_vtk_particles(const char* path, const float* pos, const float* vel, const float* rho,
                                              uint32_t n) {
    if (!path || (n && !pos)) return PMS_ERR_INVALID_ARGUMENT;
    std::string s;
    s.reserve(40ull * n + 512);
    s += "# vtk DataFile Version 3.0\nparticles\nBINARY\nDATASET POLYDATA\n";
    s += "POINTS " + std::to_string(n) + " float\n";
    for (size_t i = 0; i < 3ull * n; ++i) put_be32(s, &pos[i]);
    s += "\nVERTICES " + std::to_string(n) + " " + std::to_string(2ull * n) + "\n";
    for (uint32_t i = 0; i < n; ++i) { int32_t one = 1, id = (int32_t)i; put_be32(s, &one); put_be32(s, &id); }
    s += "\nPOINT_DATA " + std::to_string(n) + "\nFIELD FieldData 2\n";
    s += "Vel 3 " + std::to_string(n) + " float\n";
    for (size_t i = 0; i < 3ull * n; ++i) { float v = vel ? vel[i] : 0.f; put_be32(s, &v); }
    s += "\nRhop 1 " + std::to_string(n) + " float\n";
    for (size_t i = 0; i < n; ++i) { float v = rho ? rho[i] : 0.f; put_be32(s, &v); }
    s += "\n";
    std::ofstream f(path, std::ios::binary);
    if (!f) return PMS_ERR_IO;
    f.write(s.data(), (std::streamsize)s.size());
    return f ? PMS_OK : PMS_ERR_IO;
}

// Surface mesh with the scalar values, legacy VTK polydata (the arrays of
// FileData::saveSurfaceVTKfile, FileData.cpp:677-773: points, triangles
// (i, i+1, i+2), Normal = -normal, Rhop, VelLength, Vel).  The reference writes
// it through VTK in ASCII; this writer is BINARY (big-endian), which VTK reads the same.
extern "C" pms_status pms_write_surface_vtk(const char* path, const float* pos, const float* nrm, const float* vel,
                                            const float* vel_len, const float* rhop, uint64_t nv) {
    if (!path || (nv && !pos) || nv >= (1ull << 31)) return PMS_ERR_INVALID_ARGUMENT;
    const uint64_t nt = nv / 3;
    std::string s;
    s.reserve(64ull * nv + 1024);
    s += "# vtk DataFile Version 3.0\nsurface\nBINARY\nDATASET POLYDATA\n";
    s += "POINTS " + std::to_string(nv) + " float\n";
    for (size_t i = 0; i < 3ull * nv; ++i) put_be32(s, &pos[i]);
    s += "\nPOLYGONS " + std::to_string(nt) + " " + std::to_string(4ull * nt) + "\n";
    for (uint64_t t = 0; t < nt; ++t) {
        const int32_t k = 3, a = (int32_t)(3 * t), b = a + 1, c = a + 2;
        put_be32(s, &k); put_be32(s, &a); put_be32(s, &b); put_be32(s, &c);
    }
    s += "\nPOINT_DATA " + std::to_string(nv) + "\nFIELD FieldData 4\n";
    s += "Normal 3 " + std::to_string(nv) + " float\n";
    for (size_t i = 0; i < 3ull * nv; ++i) { float v = nrm ? -nrm[i] : 0.f; put_be32(s, &v); }
    s += "\nRhop 1 " + std::to_string(nv) + " float\n";
    for (size_t i = 0; i < nv; ++i) { float v = rhop ? rhop[i] : 0.f; put_be32(s, &v); }
    s += "\nVelLength 1 " + std::to_string(nv) + " float\n";
    for (size_t i = 0; i < nv; ++i) { float v = vel_len ? vel_len[i] : 0.f; put_be32(s, &v); }
    s += "\nVel 3 " + std::to_string(nv) + " float\n";
    for (size_t i = 0; i < 3ull * nv; ++i) { float v = vel ? vel[i] : 0.f; put_be32(s, &v); }
    s += "\n";
    std::ofstream f(path, std::ios::binary);
    if (!f) return PMS_ERR_IO;
    f.write(s.data(), (std::streamsize)s.size());
    return f ? PMS_OK : PMS_ERR_IO;
}

// ---------------------------------------------------------------------------
// PLY, ASCII, in tinyply 2.3's layout: header, then "x y z \n" per vertex with
// the stream's default float formatting (printf %g), then "3 a b c \n" per face.
// ---------------------------------------------------------------------------
// Text of vertex lines [v0, v1) ("%g %g %g \n", tinyply's ASCII layout) and face
// lines [t0, t1) ("3 i i+1 i+2 \n") into out.
static void ply_lines(const float* pos, uint64_t v0, uint64_t v1, uint64_t t0, uint64_t t1, std::string& out) {
    char tmp[128];
    out.clear();
    out.reserve((size_t)((v1 - v0) * 36 + (t1 - t0) * 32));
    for (uint64_t i = v0; i < v1; ++i) {
        const int k = snprintf(tmp, sizeof(tmp), "%g %g %g \n", (double)pos[3 * i], (double)pos[3 * i + 1], (double)pos[3 * i + 2]);
        out.append(tmp, (size_t)k);
    }
    for (uint64_t t = t0; t < t1; ++t) {
        // decimal digits by hand: the same text as "3 %u %u %u \n"
        char* p = tmp;
        *p++ = '3';
        for (int c = 0; c < 3; ++c) {
            *p++ = ' ';
            uint32_t v = (uint32_t)(3 * t + c);
            char d[12];
            int nd = 0;
            do { d[nd++] = (char)('0' + v % 10); v /= 10; } while (v);
            while (nd) *p++ = d[--nd];
        }
        *p++ = ' ';
        *p++ = '\n';
        out.append(tmp, (size_t)(p - tmp));
    }
}

// The text is formatted in parallel chunks (one per hardware thread) and written in order, so
// the file is the same byte for byte as a serial writer's.
extern "C" pms_status pms_write_ply(const char* path, const float* pos, uint64_t nv) {
    if (!path || (nv && !pos)) return PMS_ERR_INVALID_ARGUMENT;
    FILE* f = fopen(path, "wb");
    if (!f) return PMS_ERR_IO;
    const uint64_t nf = nv / 3;
    fprintf(f, "ply\nformat ascii 1.0\ncomment generated by tinyply 2.3\n");
    fprintf(f, "element vertex %llu\nproperty float x\nproperty float y\nproperty float z\n", (unsigned long long)nv);
    fprintf(f, "element face %llu\nproperty list uchar uint vertex_indices\nend_header\n", (unsigned long long)nf);
    unsigned hw = std::thread::hardware_concurrency();
    const uint64_t T = std::max<uint64_t>(1, std::min<uint64_t>(hw ? hw : 1, (nv + nf) / 65536 + 1));
    // chunks: vertex lines first, then face lines, each split into T pieces; written in order
    std::vector<std::string> vtext(T), ftext(T);
    std::vector<std::thread> th;
    for (uint64_t c = 0; c < T; ++c)
        th.emplace_back([&, c]() {
            ply_lines(pos, nv * c / T, nv * (c + 1) / T, 0, 0, vtext[c]);
            ply_lines(pos, 0, 0, nf * c / T, nf * (c + 1) / T, ftext[c]);
        });
    for (std::thread& t : th) t.join();
    bool ok = true;
    for (const std::string& sv : vtext) ok = ok && fwrite(sv.data(), 1, sv.size(), f) == sv.size();
    for (const std::string& sf : ftext) ok = ok && fwrite(sf.data(), 1, sf.size(), f) == sf.size();
    ok = ferror(f) == 0 && ok;
    ok = fclose(f) == 0 && ok;
    return ok ? PMS_OK : PMS_ERR_IO;
}

extern "C" pms_status pms_write_ply_mesh(const char* path, const float* pos, uint64_t nv, const uint32_t* indices,
                                         uint64_t ni, int binary) {
    if (!path || (nv && !pos) || (indices && ni % 3)) return PMS_ERR_INVALID_ARGUMENT;
    if (!indices && !binary) return pms_write_ply(path, pos, nv);      // the reference's ASCII soup
    if (!indices) ni = nv - nv % 3;
    if (indices)
        for (uint64_t i = 0; i < ni; ++i)
            if (indices[i] >= nv) return PMS_ERR_INVALID_ARGUMENT;
    const uint64_t nf = ni / 3;
    FILE* f = fopen(path, "wb");
    if (!f) return PMS_ERR_IO;
    fprintf(f, "ply\nformat %s 1.0\ncomment generated by libpms\n", binary ? "binary_little_endian" : "ascii");
    fprintf(f, "element vertex %llu\nproperty float x\nproperty float y\nproperty float z\n", (unsigned long long)nv);
    fprintf(f, "element face %llu\nproperty list uchar uint vertex_indices\nend_header\n", (unsigned long long)nf);
    bool ok = true;
    if (binary) {
        // little-endian records: 12 bytes per vertex, 13 per face (count, then three uint32)
        std::vector<unsigned char> buf;
        buf.reserve(12 * nv);
        auto put32 = [&](uint32_t u) { for (int k = 0; k < 4; ++k) buf.push_back((unsigned char)(u >> (8 * k))); };
        for (uint64_t i = 0; i < 3 * nv; ++i) { uint32_t u; memcpy(&u, &pos[i], 4); put32(u); }
        ok = fwrite(buf.data(), 1, buf.size(), f) == buf.size();
        buf.clear();
        buf.reserve(13 * nf);
        for (uint64_t t = 0; t < nf; ++t) {
            buf.push_back(3);
            for (int k = 0; k < 3; ++k) put32(indices ? indices[3 * t + k] : (uint32_t)(3 * t + k));
        }
        ok = ok && fwrite(buf.data(), 1, buf.size(), f) == buf.size();
    } else {
        std::string out;
        char line[96];
        for (uint64_t i = 0; i < nv; ++i) {
            // 9 significant digits: the float32 values read back exactly
            const int k = snprintf(line, sizeof(line), "%.9g %.9g %.9g \n", pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
            out.append(line, (size_t)k);
        }
        for (uint64_t t = 0; t < nf; ++t) {
            const int k = snprintf(line, sizeof(line), "3 %u %u %u \n", indices[3 * t], indices[3 * t + 1], indices[3 * t + 2]);
            out.append(line, (size_t)k);
        }
        ok = fwrite(out.data(), 1, out.size(), f) == out.size();
    }
    ok = ferror(f) == 0 && ok;
    ok = fclose(f) == 0 && ok;
    return ok ? PMS_OK : PMS_ERR_IO;
}

extern "C" pms_status pms_write_diffuse_vtk(const char* path, const float* pos, const float* vel, const float* energy,
                                            const float* ita, const float* wave_crest, uint32_t n, float size) {
    if (!path || (n && !pos)) return PMS_ERR_INVALID_ARGUMENT;
    std::string s;
    s += "# vtk DataFile Version 3.0\ndiffuse particles\nBINARY\nDATASET POLYDATA\n";
    s += "POINTS " + std::to_string(n) + " float\n";
    for (size_t i = 0; i < 3ull * n; ++i) put_be32(s, &pos[i]);
    s += "\nVERTICES " + std::to_string(n) + " " + std::to_string(2ull * n) + "\n";
    for (uint32_t i = 0; i < n; ++i) { int32_t one = 1, id = (int32_t)i; put_be32(s, &one); put_be32(s, &id); }
    s += "\nPOINT_DATA " + std::to_string(n) + "\nFIELD FieldData 5\n";
    s += "Velocity 3 " + std::to_string(n) + " float\n";
    for (size_t i = 0; i < 3ull * n; ++i) { float v = vel ? vel[i] : 0.f; put_be32(s, &v); }
    s += "\nSize 1 " + std::to_string(n) + " float\n";
    for (size_t i = 0; i < n; ++i) put_be32(s, &size);
    const char* names[3] = {"energy", "Ita", "waveCrest"};
    const float* arrs[3] = {energy, ita, wave_crest};
    for (int a = 0; a < 3; ++a) {
        s += std::string("\n") + names[a] + " 1 " + std::to_string(n) + " float\n";
        for (size_t i = 0; i < n; ++i) { float v = arrs[a] ? arrs[a][i] : 0.f; put_be32(s, &v); }
    }
    s += "\n";
    std::ofstream f(path, std::ios::binary);
    if (!f) return PMS_ERR_IO;
    f.write(s.data(), (std::streamsize)s.size());
    return f ? PMS_OK : PMS_ERR_IO;
}

// ---------------------------------------------------------------------------
// the VisGPU frame loop (GPUPOST.cpp:34-91)
// ---------------------------------------------------------------------------
static std::string frame_name(const char* dir, const char* prefix, int nzeros, int frame, const char* ext) {
    char num[64];
    snprintf(num, sizeof(num), "%.*d", nzeros, frame);
    std::string d = dir;
    if (!d.empty() && d.back() != '/') d += "/";
    return d + prefix + num + ext;
}

// One frame's input, parsed on the reader thread.
struct FrameIn {
    float *pos = nullptr, *vel = nullptr, *rho = nullptr;
    uint32_t n = 0;
    pms_status st = PMS_OK;
    std::string path;
    void release() { pms_free_host(pos); pms_free_host(vel); pms_free_host(rho); pos = vel = rho = nullptr; }
};

// One frame's output, written on the writer thread.
struct FrameOut {
    std::string ply, dir;
    std::vector<float> pos;            // soup or welded vertices
    std::vector<uint32_t> idx;         // welded triangle indices (empty: soup)
    bool binary = false, surface = false;
    std::vector<std::vector<float>> dpos, dvel;   // diffuse spray, foam, bubble
    std::vector<std::string> dpaths;
    float dsize = 0.f;
};

static pms_status write_frame(const FrameOut& o) {
    pms_status st = PMS_OK;
    if (o.surface) {
        const uint64_t nv = o.pos.size() / 3;
        if (nv == 0) fprintf(stderr, "Nothing produced.\n");
        else if (o.idx.empty() && !o.binary) st = pms_write_ply(o.ply.c_str(), o.pos.data(), nv);
        else st = pms_write_ply_mesh(o.ply.c_str(), o.pos.data(), nv, o.idx.empty() ? nullptr : o.idx.data(),
                                     o.idx.size(), o.binary ? 1 : 0);
        if (st) { fprintf(stderr, "error: cannot write %s\n", o.ply.c_str()); return st; }
    }
    for (size_t k = 0; k < o.dpaths.size() && !st; ++k) {
        const uint32_t m = (uint32_t)(o.dpos[k].size() / 3);
        std::vector<float> zeros(m, 0.f);
        st = pms_write_diffuse_vtk(o.dpaths[k].c_str(), o.dpos[k].data(), o.dvel[k].data(), zeros.data(), zeros.data(),
                                   zeros.data(), m, o.dsize);
        if (st) fprintf(stderr, "error: cannot write %s\n", o.dpaths[k].c_str());
    }
    return st;
}

// The VisGPU frame loop as a pipeline: while the GPU reconstructs frame k, a reader
// thread parses frame k + 1 and a writer thread writes frame k - 1's files (the
// reference does the three one after another, GPUPOST.cpp:51-82).
extern "C" pms_status pms_run_config(const char* config_path, int verbose) {
    pms_config cfg;
    pms_status st = pms_config_load(config_path, &cfg);
    if (st) { fprintf(stderr, "error: cannot load %s\n", config_path ? config_path : "(null)"); return st; }
    pms_ctx* ctx = nullptr;
    if ((st = pms_create(&cfg, -1, &ctx))) { fprintf(stderr, "error: pms_create: %s\n", pms_status_string(st)); return st; }
    const int step = cfg.frame_step > 0 ? cfg.frame_step : 1;
    // parse a frame and stage it: pinned copy and host-to-device copy into the
    // context's second input buffers (on the reader thread, while the GPU runs the
    // frame before it)
    auto read = [&](int frame, FrameIn* in) {
        in->path = frame_name(cfg.fluid_path, cfg.fluid_prefix, cfg.num_zeros, frame, ".vtk");
        in->st = pms_read_vtk_particles(in->path.c_str(), &in->pos, &in->vel, &in->rho, &in->n);
        if (!in->st) in->st = pms_stage_particles(ctx, in->pos, in->vel, in->rho, in->n);
        in->release();
    };
    FrameIn cur, next;
    std::thread reader, writer;
    pms_status wst = PMS_OK;
    if (cfg.frame_start <= cfg.frame_end) read(cfg.frame_start, &cur);
    for (int frame = cfg.frame_start; frame <= cfg.frame_end; frame += step) {
        if (cur.st) {
            fprintf(stderr, "error: cannot read or stage %s: %s\n", cur.path.c_str(), pms_status_string(cur.st));
            st = cur.st;
            break;
        }
        const bool more = frame + step <= cfg.frame_end;
        if (verbose) printf("frame %d: %u particles from %s\n", frame, cur.n, cur.path.c_str());
        st = pms_upload_staged(ctx);
        // the next frame is staged only after this one took the staged buffers
        if (more) reader = std::thread(read, frame + step, &next);
        if (!st) st = pms_run_frame(ctx);
        FrameOut out;
        if (!st && cfg.is_surface) {
            out.surface = true;
            out.binary = cfg.ply_binary != 0;
            out.ply = frame_name(cfg.surface_path, cfg.surface_prefix, cfg.num_zeros, frame, ".ply");
            uint64_t nv = 0, ni = 0;
            if (cfg.weld_mesh) {
                if (!(st = pms_weld_mesh(ctx, 0)) && !(st = pms_download_welded_mesh(ctx, nullptr, nullptr, 0, nullptr, 0, &nv, &ni))) {
                    out.pos.resize(3 * (size_t)nv);
                    out.idx.resize((size_t)ni);
                    st = pms_download_welded_mesh(ctx, out.pos.data(), nullptr, nv, out.idx.data(), ni, &nv, &ni);
                }
            } else {
                pms_download_mesh(ctx, nullptr, nullptr, 0, &nv);
                out.pos.resize(3 * (size_t)nv);
                st = nv ? pms_download_mesh(ctx, out.pos.data(), nullptr, nv, &nv) : PMS_OK;
            }
            if (verbose && !st) printf("  %llu mesh vertices -> %s\n", (unsigned long long)(out.pos.size() / 3), out.ply.c_str());
        }
        if (!st && cfg.is_diffuse) st = pms::diffuse_frame_output(ctx, cfg, frame, out.dpos, out.dvel, out.dpaths, out.dsize);
        if (st) {
            fprintf(stderr, "error: frame %d: %s\n", frame, pms_last_error(ctx));
            if (reader.joinable()) reader.join();
            next.release();
            break;
        }
        if (writer.joinable()) writer.join();
        if (wst) { st = wst; if (reader.joinable()) reader.join(); next.release(); break; }
        writer = std::thread([o = std::move(out), &wst]() { wst = write_frame(o); });
        if (more) { reader.join(); cur = next; next = FrameIn(); }
    }
    if (writer.joinable()) writer.join();
    if (!st) st = wst;
    pms_destroy(ctx);
    return st;
}
