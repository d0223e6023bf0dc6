/*
 * lbm_host.cpp -- host side of the GB300 D3Q19 engine behind the C ABI of
 * include/lbm_gb300.h.
 *
 * It replaces the reference program's main() (LRTurbTest/LRMultiGPU7.cu,
 * "LR7", lines 2575-3029): the .inputs run record becomes the runtime
 * configuration (parsed here, written back byte-compatibly by WriteInputs'
 * format, LR7:2547-2573), ImageFcn/ImageFcnLR (LR7:68-127) build a one-byte
 * node mask per level on the host, and the time loop (LR7:2849-2950) becomes
 * a sequence of launches on one CUDA stream with no host synchronisation
 * between steps.  The reference's z-slab decomposition over GPUs with peer
 * copies of halo planes is replaced by one domain per level with periodic z.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/lbm_gb300.h"
#include "d3q19.cuh"
#include "lbm_kernels.cuh"
#include "sgs_infer.cuh"

using namespace lbm;

namespace {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

#define CUDA_TRY(call)                                                                      \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess) return fail(LBM_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

/* ------------------------------------------------------------------------ */
/* configuration: the .inputs record                                          */
/* ------------------------------------------------------------------------ */

struct Config {
    int nx = 0, ny = 0, nz = 0;
    int bs[3] = {64, 1, 1};
    float ob1[3] = {0, 0, 0}, r1 = 0;
    float ob2[3] = {0, 0, 0}, r2 = 0;
    float re = 100.f, umax = 0.05f;
    float omega_rec = 0;            /* the recorded omega line (informative) */
    bool has_dpdy = false;
    float dpdy = 0;
    int tmax = 1000, startf = 0, start_av = 100000, start_fluc = 250000;
    int refinement = 0;
    std::string model = "MRT";
    int les = 0;
    float cs = 0.02f;
    int lrx = 128, lry = 80, lrz = 8;
    float lrfactor = 0.5f;
    float lrx0 = 128.25f, lry0 = 64.25f, lrz0 = -0.75f;
    int lbs[3] = {64, 1, 1};
    float omega_lr_rec = 0;
    int gpus = 1;
    /* extension keys (not in the reference record) */
    std::string geometry = "channel_square";
    std::string precision = "fp32";
    /* "LAYOUT: soa | blocked | auto": population layout in HBM; auto stores
     * FP32, FP16 and BF16 in blocks of 32 nodes and keeps FP64 (the accuracy
     * twin) in the reference's structure-of-arrays layout */
    std::string pop_layout = "auto";
    float tau = 0;                  /* > 0: tau0 given directly instead of RE */
    float lid_u[3] = {0, 0, 0};
    bool lid_u_set = false;
    int lid_face = 5;               /* +z */
    float noise = 0;
    uint32_t seed = 12345u;
    int velav = 0;
    int init = -1;                  /* 0: MRT equilibrium, 1: BGK, 2: BGK incl. solids (CPU_3D); -1: by model */
    float init_u = -1e30f;          /* default: UMAX (channel), 0 (cavity / periodic) */
    int order = 2;
    int fc_zflip = 1;
    int pull_clamp = 0;             /* "EDGE PULL: clamp" (CPU_3D) or "wrap" */
    int halfway = 0;                /* "BOUNCEBACK: halfway" or "fullway" (the reference) */
    int lid_quirk = 0;              /* "LID BC: cpu3d" reproduces CPU_3D's lid as written */
    int sgs_mlp = 0;                /* "SGS: mlp": the learned closure replaces Smagorinsky */
    int sgs_every = 1;              /* "SGS every: k": the closure's eddy viscosity is evaluated on the
                                     * steps t with t % k == 0 and reused from a per-node buffer between */
    /* dynamic inlet (DI3): body force below DYNY1 (DI3:1358), P-control of
     * the mean velocity of the plane DYNY1 every DYN every steps after DYN
     * start (DI3:3150-3170), trip bodies (Obst2) until TRIP end (DI3:72-90) */
    int dyny1 = -1;
    int dyn_every = 100, dyn_start = 10000;
    int trip_end = 5000;
    std::string sgs_weights;        /* "SGS weights: <file>" of float32 parameters */
    /* "FACES: west east south north bottom top": a node type per box face
     * (x = 0, x = nx-1, y = 0, y = ny-1, z = 0, z = nz-1), "-" keeps the
     * geometry's own; y faces over z faces over x faces at edges */
    int faces[6] = {-1, -1, -1, -1, -1, -1};
    bool faces_set = false;
    /* "CF TIME: linear": the fine band gets coarse moments interpolated in
     * time before every fine sub-step after the first (the reference, "none",
     * fills it once per coarse step, LR7:2926) */
    int cf_time = 0;
    /* older records spell the LES line "Smagorinski LES: YES/NO"; DynInlet
     * records add "KP" (the inlet P-control gain, MRTtest/DynInlet3.cu:26) */
    bool les_yesno = false;
    float kp = 0;
    /* the parsed record's lines: label and separator as written, canonical key */
    struct Line {
        std::string label, sep, key;
    };
    std::vector<Line> layout;
};

std::string trim(const std::string& s) {
    size_t a = s.find_first_not_of(" \t\r\n"), b = s.find_last_not_of(" \t\r\n");
    return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
}

/* node type names, by code */
const char* const NODE_NAMES[NODE_TYPES] = {"FLUID",    "WALL",     "BODY",         "WEST_INLET", "EAST_OUTLET",
                                            "SOUTH_INLET", "NORTH_OUTLET", "LID",   "DIR_WEST",   "NEU_EAST",
                                            "NEU_EAST_REG", "XSYM_TOP", "XSYM_BOT", "YSYM_TOP",   "YSYM_BOT",
                                            "ZSYM_TOP", "ZSYM_BOT", "WEST_REG", "DIR_WEST_V", "DIR_NORTH",
                                            "DIR_SOUTH"};

bool parse_faces(const std::string& v, int out[6]) {
    std::istringstream in(v);
    std::string tok;
    int n = 0;
    while (in >> tok) {
        if (n == 6) return false;
        int code = -2;
        if (tok == "-") code = -1;
        for (int i = 0; i < NODE_TYPES; ++i)
            if (tok == NODE_NAMES[i]) code = i;
        if (code == -2) return false;
        out[n++] = code;
    }
    return n == 6;
}

bool parse_xyz_int(const std::string& v, int out[3]) {
    return sscanf(v.c_str(), "%dx%dx%d", &out[0], &out[1], &out[2]) == 3;
}
bool parse_xyz_float_x(const std::string& v, float out[3]) {
    return sscanf(v.c_str(), "%fx%fx%f", &out[0], &out[1], &out[2]) == 3;
}
bool parse_tuple(const std::string& v, float out[3]) {
    return sscanf(v.c_str(), " (%f , %f , %f )", &out[0], &out[1], &out[2]) == 3;
}

int parse_inputs(const char* text, Config& c) {
    std::istringstream in(text ? text : "");
    std::string line;
    int lineno = 0;
    bool have_dims = false;
    while (std::getline(in, line)) {
        ++lineno;
        if (trim(line).empty() || trim(line)[0] == '#') continue;
        size_t tab = line.find('\t');
        if (tab == std::string::npos) return fail(LBM_ERR_PARSE, ".inputs line %d has no TAB separator: '%s'", lineno, line.c_str());
        std::string key = trim(line.substr(0, tab));
        while (!key.empty() && key.back() == ':') key = trim(key.substr(0, key.size() - 1));
        std::string rest = line.substr(tab + 1);
        std::string val = trim(rest);
        std::string sep;
        if (!val.empty() && val[0] == ':') {
            sep = rest.substr(0, rest.find(':') + 1);
            size_t v0 = rest.find_first_not_of(' ', sep.size());
            sep = rest.substr(0, v0 == std::string::npos ? rest.size() : v0);
            val = trim(val.substr(1));
        }
        if (key == "Smagorinski LES") {
            c.les_yesno = true;
            val = (val == "YES" || val == "1") ? "1" : "0";
        }
        bool ok = true;
        auto F = [&](float& dst) { ok = sscanf(val.c_str(), "%f", &dst) == 1; };
        auto I = [&](int& dst) { ok = sscanf(val.c_str(), "%d", &dst) == 1; };
        if (key == "Base domain size") { int d[3]; ok = parse_xyz_int(val, d); c.nx = d[0]; c.ny = d[1]; c.nz = d[2]; have_dims = ok; }
        else if (key == "Base blocksize") ok = parse_xyz_int(val, c.bs);
        else if (key == "Obst1 location") ok = parse_tuple(val, c.ob1);
        else if (key == "Obst1 radius") F(c.r1);
        else if (key == "Obst2 location") ok = parse_tuple(val, c.ob2);
        else if (key == "Obst2 radius") F(c.r2);
        else if (key == "RE") F(c.re);
        else if (key == "UMAX") F(c.umax);
        else if (key == "omega") F(c.omega_rec);
        else if (key == "DPDY") { F(c.dpdy); c.has_dpdy = true; }
        else if (key == "TMAX") I(c.tmax);
        else if (key == "STARTF") I(c.startf);
        else if (key == "START_VELAV") I(c.start_av);
        else if (key == "START_VELFLUC") I(c.start_fluc);
        else if (key == "REFINEMENT") I(c.refinement);
        else if (key == "MODEL") c.model = val;
        else if (key == "Smagorinsky LES") I(c.les);
        else if (key == "CS") F(c.cs);
        else if (key == "LR domain size") { int d[3]; ok = parse_xyz_int(val, d); c.lrx = d[0]; c.lry = d[1]; c.lrz = d[2]; }
        else if (key == "LR factor") F(c.lrfactor);
        else if (key == "LR location") { float d[3]; ok = parse_xyz_float_x(val, d); c.lrx0 = d[0]; c.lry0 = d[1]; c.lrz0 = d[2]; }
        else if (key == "LR blocksize") ok = parse_xyz_int(val, c.lbs);
        else if (key == "omega in LR") F(c.omega_lr_rec);
        else if (key == "GPUs per node") I(c.gpus);
        else if (key == "Smagorinski LES") I(c.les);
        else if (key == "KP") F(c.kp);
        /* extension keys */
        else if (key == "GEOMETRY") c.geometry = val;
        else if (key == "PRECISION") {
            ok = (val == "fp32" || val == "fp16" || val == "bf16" || val == "fp64");
            c.precision = val;
        }
        else if (key == "LAYOUT") {
            ok = (val == "soa" || val == "blocked" || val == "auto");
            c.pop_layout = val;
        }
        else if (key == "TAU") F(c.tau);
        else if (key == "LID velocity") { ok = parse_tuple(val, c.lid_u); c.lid_u_set = true; }
        else if (key == "LID face") {
            static const char* faces[6] = {"-x", "+x", "-y", "+y", "-z", "+z"};
            ok = false;
            for (int i = 0; i < 6; ++i) if (val == faces[i]) { c.lid_face = i; ok = true; }
        }
        else if (key == "Inlet noise") F(c.noise);
        else if (key == "Seed") { unsigned long s = 0; ok = sscanf(val.c_str(), "%lu", &s) == 1; c.seed = uint32_t(s); }
        else if (key == "VELAV") I(c.velav);
        else if (key == "Init") I(c.init);
        else if (key == "Init velocity") F(c.init_u);
        else if (key == "ORDER") I(c.order);
        else if (key == "FC top zflip") I(c.fc_zflip);
        else if (key == "EDGE PULL") {
            ok = (val == "clamp" || val == "wrap");
            c.pull_clamp = val == "clamp";
        }
        else if (key == "BOUNCEBACK") {
            ok = (val == "halfway" || val == "fullway");
            c.halfway = val == "halfway";
        }
        else if (key == "SGS") {
            ok = (val == "mlp" || val == "smagorinsky");
            c.sgs_mlp = val == "mlp";
        }
        else if (key == "SGS weights") c.sgs_weights = val;
        else if (key == "SGS every") {
            I(c.sgs_every);
            ok = ok && c.sgs_every >= 1;
        }
        else if (key == "DYNY1") I(c.dyny1);
        else if (key == "DYN every") I(c.dyn_every);
        else if (key == "DYN start") I(c.dyn_start);
        else if (key == "TRIP end") I(c.trip_end);
        else if (key == "FACES") { ok = parse_faces(val, c.faces); c.faces_set = true; }
        else if (key == "CF TIME") {
            ok = (val == "linear" || val == "none");
            c.cf_time = val == "linear";
        }
        else if (key == "LID BC") {
            ok = (val == "cpu3d" || val == "regularized");
            c.lid_quirk = val == "cpu3d";
        }
        else return fail(LBM_ERR_PARSE, ".inputs line %d: unknown key '%s'", lineno, key.c_str());
        if (!ok) return fail(LBM_ERR_PARSE, ".inputs line %d: cannot read value '%s' of '%s'", lineno, val.c_str(), key.c_str());
        c.layout.push_back({line.substr(0, tab), sep, key});
    }
    if (!have_dims) return fail(LBM_ERR_PARSE, ".inputs record has no 'Base domain size' line");
    if (c.nx < 3 || c.ny < 3 || c.nz < 1) return fail(LBM_ERR_CONFIG, "domain %dx%dx%d is too small", c.nx, c.ny, c.nz);
    return LBM_OK;
}

int model_id(const std::string& m) {
    if (m == "MRT") return MRT;
    if (m == "MRT_DI3") return MRT_DI3;
    if (m == "BGK") return BGK;
    if (m == "MRT_CPU3D") return MRT_CPU3D;
    return -1;
}

int storage_id(const std::string& p) {
    if (p == "fp32") return STORE_F32;
    if (p == "fp16") return STORE_F16;
    if (p == "bf16") return STORE_BF16;
    if (p == "fp64") return STORE_F64;
    return -1;
}

size_t storage_bytes(int s) { return s == STORE_F64 ? 8 : (s == STORE_F32 ? 4 : 2); }

/* relaxation rates, LR7:2607-2619 */
void relaxation(const Config& c, float& omega, float& omegaLR, float& sf_cf, float& sf_fc) {
    if (c.tau > 0.f) omega = 1.0f / c.tau;
    else {
        float CharLength = c.r1 * 2.f;
        omega = 1.0f / (3.0f * (c.umax * CharLength / c.re) + 0.5f);
    }
    omegaLR = 2.0f / (1.0f + 2.0f * (2.0f / omega - 1.0f));
    if (c.lrfactor == 0.25f) omegaLR = 2.0f / (1.0f + 2.0f * (2.0f / omegaLR - 1.0f));
    if (c.lrfactor == 0.125f) {
        omegaLR = 2.0f / (1.0f + 2.0f * (2.0f / omegaLR - 1.0f));
        omegaLR = 2.0f / (1.0f + 2.0f * (2.0f / omegaLR - 1.0f));
    }
    sf_cf = omega * (1.0f - omegaLR) / ((1.0f - omega) * omegaLR / c.lrfactor);
    sf_fc = 1.f / sf_cf;
}

/* the record, in WriteInputs' order and format (LR7:2547-2573); extension
 * keys follow only when they differ from their defaults */
std::string value_of(const Config& c, const std::string& key, float omega, float omegaLR) {
    std::ostringstream o;
    static const char* faces[6] = {"-x", "+x", "-y", "+y", "-z", "+z"};
    if (key == "Base domain size") o << c.nx << "x" << c.ny << "x" << c.nz;
    else if (key == "Base blocksize") o << c.bs[0] << "x" << c.bs[1] << "x" << c.bs[2];
    else if (key == "Obst1 location") o << "(" << c.ob1[0] << "," << c.ob1[1] << "," << c.ob1[2] << ")";
    else if (key == "Obst1 radius") o << c.r1;
    else if (key == "Obst2 location") o << "(" << c.ob2[0] << "," << c.ob2[1] << "," << c.ob2[2] << ")";
    else if (key == "Obst2 radius") o << c.r2;
    else if (key == "RE") o << c.re;
    else if (key == "UMAX") o << c.umax;
    else if (key == "omega") o << omega;
    else if (key == "DPDY") o << c.dpdy;
    else if (key == "TMAX") o << c.tmax;
    else if (key == "STARTF") o << c.startf;
    else if (key == "START_VELAV") o << c.start_av;
    else if (key == "START_VELFLUC") o << c.start_fluc;
    else if (key == "REFINEMENT") o << c.refinement;
    else if (key == "MODEL") o << c.model;
    else if (key == "Smagorinsky LES") o << c.les;
    else if (key == "Smagorinski LES") o << (c.les ? "YES" : "NO");
    else if (key == "CS") o << c.cs;
    else if (key == "KP") o << c.kp;
    else if (key == "LR domain size") o << c.lrx << "x" << c.lry << "x" << c.lrz;
    else if (key == "LR factor") o << c.lrfactor;
    else if (key == "LR location") o << c.lrx0 << "x" << c.lry0 << "x" << c.lrz0;
    else if (key == "LR blocksize") o << c.lbs[0] << "x" << c.lbs[1] << "x" << c.lbs[2];
    else if (key == "omega in LR") o << omegaLR;
    else if (key == "GPUs per node") o << c.gpus;
    else if (key == "GEOMETRY") o << c.geometry;
    else if (key == "PRECISION") o << c.precision;
    else if (key == "LAYOUT") o << c.pop_layout;
    else if (key == "TAU") o << c.tau;
    else if (key == "LID velocity") o << "(" << c.lid_u[0] << "," << c.lid_u[1] << "," << c.lid_u[2] << ")";
    else if (key == "LID face") o << faces[c.lid_face];
    else if (key == "Inlet noise") o << c.noise;
    else if (key == "Seed") o << c.seed;
    else if (key == "VELAV") o << c.velav;
    else if (key == "Init") o << c.init;
    else if (key == "Init velocity") o << c.init_u;
    else if (key == "ORDER") o << c.order;
    else if (key == "FC top zflip") o << c.fc_zflip;
    else if (key == "EDGE PULL") o << (c.pull_clamp ? "clamp" : "wrap");
    else if (key == "LID BC") o << (c.lid_quirk ? "cpu3d" : "regularized");
    else if (key == "BOUNCEBACK") o << (c.halfway ? "halfway" : "fullway");
    else if (key == "SGS") o << (c.sgs_mlp ? "mlp" : "smagorinsky");
    else if (key == "SGS weights") o << c.sgs_weights;
    else if (key == "SGS every") o << c.sgs_every;
    else if (key == "DYNY1") o << c.dyny1;
    else if (key == "DYN every") o << c.dyn_every;
    else if (key == "DYN start") o << c.dyn_start;
    else if (key == "TRIP end") o << c.trip_end;
    else if (key == "CF TIME") o << (c.cf_time ? "linear" : "none");
    else if (key == "FACES")
        for (int i = 0; i < 6; ++i) o << (i ? " " : "") << (c.faces[i] < 0 ? "-" : NODE_NAMES[c.faces[i]]);
    return o.str();
}

/* The run record.  A parsed record is written back line by line with its own
 * labels (values from the configuration, the omega lines recomputed); a new
 * one follows WriteInputs (LR7:2547-2573), extension keys after it when they
 * differ from their defaults. */
std::string write_inputs(const Config& c, float omega, float omegaLR) {
    std::ostringstream o;
    if (!c.layout.empty()) {
        for (const auto& l : c.layout) o << l.label << "\t" << l.sep << value_of(c, l.key, omega, omegaLR) << std::endl;
        return o.str();
    }
    auto line = [&](const char* label, const char* key, const char* sep = "") {
        o << label << "\t" << sep << value_of(c, key, omega, omegaLR) << std::endl;
    };
    line("Base domain size ", "Base domain size");
    line("Base blocksize: ", "Base blocksize");
    line("Obst1 location: ", "Obst1 location");
    line("Obst1 radius: ", "Obst1 radius");
    line("Obst2 location: ", "Obst2 location");
    line("Obst2 radius: ", "Obst2 radius");
    line("RE: ", "RE");
    line("UMAX: ", "UMAX");
    line("omega ", "omega", ": ");
    if (c.has_dpdy) line("DPDY ", "DPDY", ": ");
    line("TMAX: ", "TMAX");
    line("STARTF: ", "STARTF");
    line("START_VELAV: ", "START_VELAV");
    line("START_VELFLUC: ", "START_VELFLUC");
    line("REFINEMENT: ", "REFINEMENT");
    line("MODEL: ", "MODEL");
    line("Smagorinsky LES: ", "Smagorinsky LES");
    line("CS: ", "CS");
    line("LR domain size ", "LR domain size");
    line("LR factor ", "LR factor");
    line("LR location ", "LR location");
    line("LR blocksize: ", "LR blocksize");
    line("omega in LR ", "omega in LR", ": ");
    line("GPUs per node ", "GPUs per node", ": ");
    Config d;
    if (c.geometry != d.geometry) line("GEOMETRY: ", "GEOMETRY");
    if (c.precision != d.precision) line("PRECISION: ", "PRECISION");
    if (c.pop_layout != d.pop_layout) line("LAYOUT: ", "LAYOUT");
    if (c.tau > 0.f) line("TAU: ", "TAU");
    if (c.lid_u_set) line("LID velocity: ", "LID velocity");
    if (c.lid_face != d.lid_face) line("LID face: ", "LID face");
    if (c.noise != 0.f) line("Inlet noise: ", "Inlet noise");
    if (c.seed != d.seed) line("Seed: ", "Seed");
    if (c.velav) line("VELAV: ", "VELAV");
    if (c.init >= 0) line("Init: ", "Init");
    if (c.init_u > -1e29f) line("Init velocity: ", "Init velocity");
    if (c.order != d.order) line("ORDER: ", "ORDER");
    if (c.fc_zflip != d.fc_zflip) line("FC top zflip: ", "FC top zflip");
    if (c.pull_clamp) line("EDGE PULL: ", "EDGE PULL");
    if (c.lid_quirk) line("LID BC: ", "LID BC");
    if (c.halfway) line("BOUNCEBACK: ", "BOUNCEBACK");
    if (c.sgs_mlp) line("SGS: ", "SGS");
    if (!c.sgs_weights.empty()) line("SGS weights: ", "SGS weights");
    if (c.sgs_every != 1) line("SGS every: ", "SGS every");
    if (c.dyny1 != d.dyny1) line("DYNY1: ", "DYNY1");
    if (c.dyn_every != d.dyn_every) line("DYN every: ", "DYN every");
    if (c.dyn_start != d.dyn_start) line("DYN start: ", "DYN start");
    if (c.trip_end != d.trip_end) line("TRIP end: ", "TRIP end");
    if (c.faces_set) line("FACES: ", "FACES");
    if (c.cf_time) line("CF TIME: ", "CF TIME");
    return o.str();
}

/* ------------------------------------------------------------------------ */
/* geometry: ImageFcn / ImageFcnLR                                            */
/* ------------------------------------------------------------------------ */

int body_shape(const std::string& g) {
    if (g == "channel_square") return 1;
    if (g == "channel_circle" || g == "duct") return 2;
    return 0;
}

/* the faces of a "duct" without a FACES line: CPU_3D's cylinder duct
 * (CPU:39-63, the variant with walls on the y and z faces), its Dirichlet
 * inlet and its outlet for rho = 1 */
constexpr int DUCT_FACES[6] = {DIR_WEST, NEU_EAST, WALL, WALL, WALL, WALL};

/* channel programs (LR7:88-127): body, then walls y = 0 / ny-1, inlet x = 0,
 * outlet x = nx-1 (walls override inlet/outlet, both override the body).
 * Then the FACES line, or a duct's default faces: x faces, then z, then y,
 * so that y faces hold the edges (the precedence of CPU_3D's ImageFcn). */
void mask_base(const Config& c, std::vector<uint8_t>& m, int t = 0) {
    const int nx = c.nx, ny = c.ny, nz = c.nz;
    m.assign(size_t(nx) * ny * nz, FLUID);
    const int shape = body_shape(c.geometry);
    const bool channel = c.geometry.rfind("channel", 0) == 0;
    const bool cavity = c.geometry == "cavity";
    const bool dyn = c.geometry == "dyninlet";
    const int* faces = c.faces_set ? c.faces : c.geometry == "duct" ? DUCT_FACES : nullptr;
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x) {
                uint8_t v = FLUID;
                if (shape == 1) {
                    if (std::fabs(float(x) - c.ob1[0]) < c.r1 && std::fabs(float(y) - c.ob1[1]) < c.r1) v = BODY;
                } else if (shape == 2) {
                    float dx = float(x) - c.ob1[0], dy = float(y) - c.ob1[1];
                    if (dx * dx + dy * dy < c.r1 * c.r1) v = BODY;
                }
                if (channel) {
                    if (y == 0 || y == ny - 1) v = WALL;
                    else if (x == 0) v = WEST_INLET;
                    else if (x == nx - 1) v = EAST_OUTLET;
                } else if (dyn) {
                    /* DI3's ImageFcn (DI3:72-90): trip blocks around Obst2
                     * (the second one only in the plane z = 10) until
                     * TRIP end, walls at x = 0 and nx - 1, periodic in y, z */
                    const float fx = float(x), fy = float(y);
                    if (t < c.trip_end) {
                        if (std::fabs(fx - c.ob2[0]) < c.r2 && std::fabs(fy - c.ob2[1]) < c.r2) v = BODY;
                        if (std::fabs(fx - c.ob2[0] - 3.f) < c.r2 && std::fabs(fy - c.ob2[1] - 3.f) < c.r2 && z == 10)
                            v = BODY;
                    }
                    if (x == 0 || x == nx - 1) v = WALL;
                } else if (cavity) {
                    int p[3] = {x, y, z}, n[3] = {nx, ny, nz};
                    int a = c.lid_face / 2;
                    bool on_lid = (c.lid_face % 2 == 0) ? p[a] == 0 : p[a] == n[a] - 1;
                    if (on_lid) v = LID;
                    else if (x == 0 || x == nx - 1 || y == 0 || y == ny - 1 || z == 0 || z == nz - 1) v = WALL;
                }
                if (faces) {
                    const int on[6] = {x == 0, x == nx - 1, z == 0, z == nz - 1, y == 0, y == ny - 1};
                    const int fi[6] = {0, 1, 4, 5, 2, 3};
                    for (int k = 0; k < 6; ++k)
                        if (on[k] && faces[fi[k]] >= 0) v = uint8_t(faces[fi[k]]);
                }
                m[(size_t(z) * ny + y) * nx + x] = v;
            }
}

/* ImageFcnLR (LR7:68-86) at fine-node coordinates */
void mask_fine(const Config& c, std::vector<uint8_t>& m) {
    const int nx = c.lrx, ny = c.lry, nz = c.lrz;
    m.assign(size_t(nx) * ny * nz, FLUID);
    const int shape = body_shape(c.geometry);
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x) {
                float xc = c.lrx0 + float(x) * c.lrfactor, yc = c.lry0 + float(y) * c.lrfactor;
                uint8_t v = FLUID;
                if (shape == 1) {
                    if (std::fabs(xc - c.ob1[0]) < c.r1 && std::fabs(yc - c.ob1[1]) < c.r1) v = BODY;
                } else if (shape == 2) {
                    float dx = xc - c.ob1[0], dy = yc - c.ob1[1];
                    if (dx * dx + dy * dy < c.r1 * c.r1) v = BODY;
                }
                m[(size_t(z) * ny + y) * nx + x] = v;
            }
}

/* ------------------------------------------------------------------------ */
/* handle                                                                     */
/* ------------------------------------------------------------------------ */

struct LevelState {
    Level L{};
    void* f[2] = {nullptr, nullptr};
    int cur = 0;
    uint8_t* mask = nullptr;        /* device, pitched */
    std::vector<uint8_t> hmask;     /* host, compact */
    float* stats = nullptr;         /* device, 4 x qstride */
    unsigned* body = nullptr;       /* device, pitched indices of BODY nodes */
    int nbody = 0;
    double* fpart = nullptr;        /* per-block force partials */
    unsigned* done = nullptr;       /* blocks finished in the force kernel (reset by its last block) */
    bool has_lid = false;           /* the mask has LID nodes */
    bool has_xbc = false;           /* the mask has alternate-boundary nodes */
    uint32_t* links = nullptr;      /* device, per node: bit q = pull source of q is solid */
    float* nu = nullptr;            /* device, per node: the learned closure's last eddy viscosity */
};

}  // namespace

int lbm::set_error(int code, const char* what, cudaError_t e) {
    if (e != cudaSuccess) return fail(code, "%s: %s", what, cudaGetErrorString(e));
    return fail(code, "%s", what);
}

struct lbm_handle {
    Config cfg;
    int storage = STORE_F32;
    int model = MRT;
    cudaStream_t stream = nullptr;
    LevelState lv[2];
    int nlevels = 1;
    float omega = 0, omegaLR = 0, sf_cf = 0, sf_fc = 0;
    int t = 0;
    double* force_hist = nullptr;   /* device, 3 doubles per recorded step */
    int force_cap = 0;
    float* mom = nullptr;           /* coarse moment export, [9][nz][eny][enx] */
    float* mom_prev = nullptr;      /* CF TIME linear: the previous coarse step's export */
    bool have_mom = false;          /* mom holds an export (CF TIME linear) */
    int enx = 0, eny = 0;
    double* audit_part = nullptr;
    double* audit_out = nullptr;
    RefineParams rp{};
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    /* the drag/lift reduction of a step reads the populations the step's
     * stream-collide reads, so it runs beside it on a high-priority side
     * stream: forked after the previous step, joined before the next */
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    /* refinement steps are launch-bound (a dozen small launches and events
     * each): lbm_step captures batches of steps into one CUDA graph, updated
     * in place from batch to batch (uniform runs too: it removes the gaps
     * between their launches) */
    cudaGraphExec_t gexec[17] = {}; /* by batch length (GRAPH_STEPS = 16) */
    long long launches = 0;         /* kernels this handle has launched */
    /* FP32 staging of the populations of a level for lbm_get/set_populations
     * (the stored layout or precision is not the caller's), allocated on
     * first use and kept */
    float* stage = nullptr;
    size_t stage_n = 0;
    /* learned subgrid closure: device weight blob and its error flag */
    unsigned char* mlp_blob = nullptr;
    int* mlp_err = nullptr;
    bool mlp_ready = false;
    bool mlp_warm = false;         /* a closure step ran directly: its launcher is set up */
    bool nu_valid = false;         /* lv[0].nu holds the closure's eddy viscosity of the current state's past */
    std::vector<float> mlp_params; /* host copy, for checkpoints */
    /* dynamic inlet: the body force on the device, the control history
     * (t, mean v, dpdy per control step) and whether the trip is in the mask */
    float* dpdy_dev = nullptr;
    float* dyn_hist = nullptr;
    int dyn_cap = 0, dyn_n = 0;
    bool trip_in_mask = false;
};

namespace {

void free_level(LevelState& s) {
    cudaFree(s.f[0]);
    cudaFree(s.f[1]);
    cudaFree(s.mask);
    cudaFree(s.stats);
    cudaFree(s.body);
    cudaFree(s.fpart);
    cudaFree(s.done);
    cudaFree(s.links);
    cudaFree(s.nu);
    s = LevelState();
}

/* FP16/BF16 offsets: the collision model's own equilibrium at rho = 1 and
 * the reference velocity u0 along x (the inlet velocity of a channel, rest
 * otherwise), so that the stored deviations f - off vanish in the free
 * stream.  It is the model's collision at omega = 1 of any state with that
 * density and momentum (every moment then takes its equilibrium value); for
 * LR7's MRT it differs from the lattice weights at rest (m2 has no density
 * term there, LR7:583-711), for BGK it is the BGK equilibrium. */
void set_offsets(Level& L, float u0, int model) {
    const bool reduced = L.storage == STORE_F16 || L.storage == STORE_BF16;
    double f[19];
    for (int q = 0; q < 19; ++q) {
        const double cu = double(cx(q)) * u0;
        f[q] = double(wq(q)) * (1.0 + 3.0 * cu + 4.5 * cu * cu - 1.5 * double(u0) * u0);
    }
    collide<double>(model, f, 1.0, false, 0.0, 0.0);
    for (int q = 0; q < 19; ++q) L.off[q] = reduced ? float(f[q]) : 0.f;
    L.u_ref = reduced ? u0 : 0.f;
}

int alloc_level(LevelState& s, int nx, int ny, int nz, int storage, int blocked, bool stats, float u_ref, int model) {
    Level& L = s.L;
    L.nx = nx;
    L.ny = ny;
    L.nz = nz;
    L.pitch = (nx + 31) / 32 * 32;
    L.plane = (long long)L.pitch * ny;
    L.qstride = L.plane * nz;
    L.storage = storage;
    L.blocked = blocked;
    set_offsets(L, u_ref, model);
    if (L.qstride * 19 >= (1LL << 31))
        return fail(LBM_ERR_CONFIG, "level %dx%dx%d too large: 19 populations must index below 2^31", nx, ny, nz);
    const size_t bytes = size_t(L.qstride) * 19 * storage_bytes(storage);
    for (int i = 0; i < 2; ++i) {
        CUDA_TRY(cudaMalloc(&s.f[i], bytes));
        CUDA_TRY(cudaMemset(s.f[i], 0, bytes));
    }
    CUDA_TRY(cudaMalloc(&s.mask, size_t(L.qstride)));
    CUDA_TRY(cudaMemset(s.mask, WALL, size_t(L.qstride)));
    if (stats) {
        CUDA_TRY(cudaMalloc(&s.stats, size_t(L.qstride) * 4 * sizeof(float)));
        CUDA_TRY(cudaMemset(s.stats, 0, size_t(L.qstride) * 4 * sizeof(float)));
    }
    CUDA_TRY(cudaMalloc(&s.fpart, size_t(force_partials()) * 3 * sizeof(double)));
    CUDA_TRY(cudaMalloc(&s.done, sizeof(unsigned)));
    CUDA_TRY(cudaMemset(s.done, 0, sizeof(unsigned)));
    return LBM_OK;
}

/* Upload a level's mask (pitched) with the NEAR_SOLID flag on non-solid nodes
 * that pull from a solid neighbour, and build the force list: BODY nodes for
 * full-way bounce-back, the fluid nodes next to BODY nodes for half-way. */
int upload_mask(lbm_handle* h, int level) {
    LevelState& s = h->lv[level];
    const Level& L = s.L;
    const bool clamp = h->cfg.pull_clamp, halfway = h->cfg.halfway;
    std::vector<uint8_t> pitched(size_t(L.qstride), WALL);
    auto type_at = [&](int x, int y, int z) { return s.hmask[(size_t(z) * L.ny + y) * L.nx + x]; };
    auto nb = [&](int i, int n) { return i < 0 ? (clamp ? 0 : i + n) : (i >= n ? (clamp ? n - 1 : i - n) : i); };
    static const int CX[19] = {0, 1, 0, -1, 0, 1, -1, -1, 1, 0, 1, 0, -1, 0, 0, 1, 0, -1, 0};
    static const int CY[19] = {0, 0, 1, 0, -1, 1, 1, -1, -1, 0, 0, 1, 0, -1, 0, 0, 1, 0, -1};
    static const int CZ[19] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 1, -1, -1, -1, -1, -1};
    std::vector<unsigned> list;
    std::vector<uint32_t> links(halfway ? size_t(L.qstride) : 0, 0u);
    s.has_lid = std::find(s.hmask.begin(), s.hmask.end(), uint8_t(LID)) != s.hmask.end();
    s.has_xbc = std::any_of(s.hmask.begin(), s.hmask.end(), [](uint8_t v) { return v >= DIR_WEST; });
    for (int z = 0; z < L.nz; ++z)
        for (int y = 0; y < L.ny; ++y)
            for (int x = 0; x < L.nx; ++x) {
                const uint8_t t = type_at(x, y, z);
                const size_t pc = size_t(z) * L.plane + size_t(y) * L.pitch + x;
                uint8_t m = t;
                bool near_solid = false, near_body = false;
                uint32_t lk = 0;
                if (t != WALL && t != BODY) {
                    for (int q = 1; q < 19; ++q) {
                        const uint8_t u = type_at(nb(x - CX[q], L.nx), nb(y - CY[q], L.ny), nb(z - CZ[q], L.nz));
                        near_solid |= (u == WALL || u == BODY);
                        near_body |= (u == BODY);
                        if (u == WALL || u == BODY) lk |= 1u << q;
                    }
                }
                if (halfway) links[pc] = lk;
                if (near_solid) m |= NEAR_SOLID;
                pitched[pc] = m;
                if (halfway ? near_body : (t == BODY)) list.push_back(unsigned(pc));
            }
    CUDA_TRY(cudaMemcpyAsync(s.mask, pitched.data(), pitched.size(), cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    cudaFree(s.links);
    s.links = nullptr;
    if (halfway) {
        CUDA_TRY(cudaMalloc(&s.links, links.size() * sizeof(uint32_t)));
        CUDA_TRY(cudaMemcpy(s.links, links.data(), links.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
    }
    cudaFree(s.body);
    s.body = nullptr;
    s.nbody = int(list.size());
    if (!list.empty()) {
        CUDA_TRY(cudaMalloc(&s.body, list.size() * sizeof(unsigned)));
        CUDA_TRY(cudaMemcpy(s.body, list.data(), list.size() * sizeof(unsigned), cudaMemcpyHostToDevice));
    }
    return LBM_OK;
}

int ensure_force_cap(lbm_handle* h, int n) {
    if (n <= h->force_cap) return LBM_OK;
    int cap = std::max(n, std::max(2 * h->force_cap, 1024));
    double* nh = nullptr;
    CUDA_TRY(cudaMalloc(&nh, size_t(cap) * 3 * sizeof(double)));
    CUDA_TRY(cudaMemsetAsync(nh, 0, size_t(cap) * 3 * sizeof(double), h->stream));
    if (h->force_hist) {
        CUDA_TRY(cudaMemcpyAsync(nh, h->force_hist, size_t(h->force_cap) * 3 * sizeof(double), cudaMemcpyDeviceToDevice,
                                 h->stream));
        CUDA_TRY(cudaStreamSynchronize(h->stream));
        cudaFree(h->force_hist);
    }
    h->force_hist = nh;
    h->force_cap = cap;
    return LBM_OK;
}

StepParams base_params(const lbm_handle* h, int level) {
    const Config& c = h->cfg;
    StepParams p{};
    p.model = h->model;
    p.les = c.les;
    p.omega = level == 0 ? h->omega : h->omegaLR;
    p.cs = c.cs;
    p.dpdy = c.dpdy;
    p.u_in = c.umax;          /* PoisProf3D returns UMAX (LR7:135-143) */
    p.rho_out = 1.0f;
    const bool lid_default = !c.lid_u_set;
    p.lid_u[0] = lid_default ? c.umax : c.lid_u[0];
    p.lid_u[1] = lid_default ? 0.f : c.lid_u[1];
    p.lid_u[2] = lid_default ? 0.f : c.lid_u[2];
    p.lid_face = c.lid_face;
    p.lid_quirk = c.lid_quirk;
    p.pull_clamp = c.pull_clamp;
    p.halfway = c.halfway;
    p.has_lid = h->lv[level].has_lid ? 1 : 0;
    p.has_xbc = h->lv[level].has_xbc ? 1 : 0;
    p.stats_on = c.velav;
    p.start_av = c.start_av;
    p.start_fluc = c.start_fluc;
    p.stats_weight = level == 0 ? 1.f : c.lrfactor;
    p.noise_amp = level == 0 ? c.noise : 0.f;
    p.noise_seed = c.seed;
    p.dpdy_dev = h->dpdy_dev;
    p.dyn_y1 = c.dyny1 >= 0 ? c.dyny1 : (1 << 30);
    return p;
}

int do_init(lbm_handle* h) {
    const Config& c = h->cfg;
    int kind = c.init >= 0 ? c.init : (h->model == BGK ? 1 : 0);
    float u0 = c.init_u > -1e29f ? c.init_u : (c.geometry == "cavity" || c.geometry == "periodic" ? 0.f : c.umax);
    /* the dynamic-inlet duct flows along y (DI3:1198-1209) */
    const int axis = c.geometry == "dyninlet" ? 1 : 0;
    if (c.geometry == "dyninlet" && !h->trip_in_mask && c.trip_end > 0) {
        mask_base(c, h->lv[0].hmask, 0);
        if (int rc = upload_mask(h, 0)) return rc;
        h->trip_in_mask = true;
    }
    if (h->dpdy_dev) CUDA_TRY(cudaMemcpyAsync(h->dpdy_dev, &c.dpdy, sizeof(float), cudaMemcpyHostToDevice, h->stream));
    h->dyn_n = 0;
    h->have_mom = false;
    h->nu_valid = false;
    for (int l = 0; l < h->nlevels; ++l) {
        LevelState& s = h->lv[l];
        for (int i = 0; i < 2; ++i) CUDA_TRY(launch_init(s.L, s.mask, s.f[i], kind, u0, h->stream, axis));
        h->launches += 2;
        s.cur = 0;
        if (s.stats) CUDA_TRY(cudaMemsetAsync(s.stats, 0, size_t(s.L.qstride) * 4 * sizeof(float), h->stream));
    }
    if (h->force_hist) CUDA_TRY(cudaMemsetAsync(h->force_hist, 0, size_t(h->force_cap) * 3 * sizeof(double), h->stream));
    h->t = 0;
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    return LBM_OK;
}

/* Launch the drag/lift reduction of level s's current populations on the
 * side stream, after everything queued so far on the main stream; the caller
 * joins (waits for ev_join) once the step's stream-collide is queued.  The
 * force kernel adds into `out` (3 doubles), which is zero or holds the other
 * level's sum of the same step. */
cudaError_t fork_force(lbm_handle* h, LevelState& s, double* out) {
    cudaError_t e = cudaEventRecord(h->ev_fork, h->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(h->side, h->ev_fork, 0);
    if (e == cudaSuccess)
        e = launch_force(s.L, s.f[s.cur], s.body, s.nbody, s.fpart, s.done, out, h->side, s.mask, h->cfg.halfway);
    if (e == cudaSuccess) e = cudaEventRecord(h->ev_join, h->side);
    ++h->launches;
    return e;
}

/* one base step and, with refinement, the patch sub-steps and the two
 * interpolations; the order of LR7:2849-2950 */
int one_step(lbm_handle* h) {
    const Config& c = h->cfg;
    const int t = h->t;
    LevelState& C = h->lv[0];
    StepParams p = base_params(h, 0);
    p.t = t;
    p.force_on = (!c.refinement && t > c.startf) ? 1 : 0;
    if (c.refinement) {
        p.exp_x0 = int(c.lrx0);
        p.exp_y0 = int(c.lry0);
        p.exp_nx = h->enx;
        p.exp_ny = h->eny;
    }
    const int fidx = t - c.startf;
    if (p.force_on) {
        int rc = ensure_force_cap(h, fidx + 1);
        if (rc) return rc;
    }
    if (h->trip_in_mask && t >= c.trip_end) {
        /* the trip blocks vanish (DI3's ImageFcn is false from TRIP end on) */
        CUDA_TRY(cudaStreamSynchronize(h->stream));
        mask_base(c, C.hmask, t);
        if (int rc = upload_mask(h, 0)) return rc;
        h->trip_in_mask = false;
        p.has_lid = C.has_lid ? 1 : 0;
    }
    if (c.sgs_mlp && !h->mlp_ready)
        return fail(LBM_ERR_STATE, "SGS mlp: no weights (SGS weights record line or lbm_set_sgs_mlp)");
    if (p.force_on) CUDA_TRY(fork_force(h, C, h->force_hist + 3LL * fidx));
    /* CF TIME linear: this step's export goes to the other buffer, the last
     * one is kept for the interpolation in time */
    bool blend = false;
    if (c.refinement && c.cf_time) {
        std::swap(h->mom, h->mom_prev);
        blend = h->have_mom;
        h->have_mom = true;
    }
    if (c.sgs_mlp) {
        /* the closure's eddy viscosity on the steps t % k == 0 (and the first
         * step after the state was set), kept per node for the steps between */
        p.nu = C.nu;
        if (!C.nu || !h->nu_valid || t % c.sgs_every == 0) {
            CUDA_TRY(launch_stream_collide_mlp(C.L, p, C.f[C.cur], C.f[1 - C.cur], C.mask, C.stats, C.links,
                                               h->mlp_blob, h->mlp_err, h->stream));
            h->mlp_warm = true;
            h->nu_valid = C.nu != nullptr;
        } else {
            p.nu_reuse = 1;
            p.les = 0;
            CUDA_TRY(launch_stream_collide(C.L, p, C.f[C.cur], C.f[1 - C.cur], C.mask, C.stats, h->mom, h->stream,
                                           C.links));
        }
    }
    else
        CUDA_TRY(launch_stream_collide(C.L, p, C.f[C.cur], C.f[1 - C.cur], C.mask, C.stats, h->mom, h->stream,
                                       C.links));
    ++h->launches;
    if (p.force_on) CUDA_TRY(cudaStreamWaitEvent(h->stream, h->ev_join, 0));
    C.cur = 1 - C.cur;
    if (h->dpdy_dev && c.dyny1 >= 0 && c.dyn_every > 0 && t % c.dyn_every == 0 && t > c.dyn_start &&
        h->dyn_n < h->dyn_cap) {
        /* the P-control on the state after step t (DI3:3150-3170) */
        CUDA_TRY(launch_dyn_control(C.L, C.f[C.cur], c.dyny1, c.umax, c.kp, std::fabs(c.dpdy), h->dpdy_dev,
                                    h->dyn_hist + 3LL * h->dyn_n, t, h->stream));
        ++h->launches;
        ++h->dyn_n;
    }
    if (c.refinement) {
        LevelState& Fn = h->lv[1];
        const int L = int(std::lround(1.0 / c.lrfactor));
        for (int i = 0; i < L; ++i) {
            if (blend && i > 0) {
                /* the band at fine time i / L of the coarse step */
                CUDA_TRY(launch_interp_cf(h->rp, Fn.L, h->mom, Fn.f[Fn.cur], Fn.mask, h->stream, h->mom_prev,
                                          float(i) / float(L)));
                ++h->launches;
            }
            StepParams pf = base_params(h, 1);
            pf.t = t;
            pf.force_on = (t > c.startf && i == 0) ? 1 : 0;
            if (pf.force_on) {
                int rc = ensure_force_cap(h, fidx + 1);
                if (rc) return rc;
            }
            if (pf.force_on) CUDA_TRY(fork_force(h, Fn, h->force_hist + 3LL * fidx));
            CUDA_TRY(launch_stream_collide(Fn.L, pf, Fn.f[Fn.cur], Fn.f[1 - Fn.cur], Fn.mask, Fn.stats, nullptr,
                                           h->stream, Fn.links));
            ++h->launches;
            if (pf.force_on) CUDA_TRY(cudaStreamWaitEvent(h->stream, h->ev_join, 0));
            Fn.cur = 1 - Fn.cur;
        }
        /* the band fill at the end of the coarse step and the restriction
         * touch disjoint nodes (band vs the coarse nodes over the interior
         * with its 2-node margin): one launch */
        CUDA_TRY(launch_interface(h->rp, C.L, Fn.L, h->mom, Fn.f[Fn.cur], Fn.mask, C.f[C.cur], C.mask, h->stream));
        ++h->launches;
    }
    h->t = t + 1;
    return LBM_OK;
}

constexpr int GRAPH_STEPS = 16; /* steps per captured graph */

/* k steps from h->t on can be captured: their steps call nothing that
 * synchronises (the trip leaving the mask does) or sets kernel attributes
 * and creates the tensor-memory lane on first use (the learned-closure
 * launcher does, in the direct step before the first batch) */
bool graph_ok(const lbm_handle* h, int k) {
    const Config& c = h->cfg;
    if (c.sgs_mlp && !h->mlp_warm) return false;
    if (h->trip_in_mask && h->t + k - 1 >= c.trip_end) return false;
    return true;
}

/* k steps captured from the main stream into one graph (the force and
 * band-fill stream forks from it and joins it again inside every step), then
 * launched.  The executable graph of the previous batch is updated in place
 * when the topology is the same (an update leaves launches already queued as
 * they were), else instantiated anew. */
int run_graph(lbm_handle* h, int k) {
    const Config& c = h->cfg;
    /* what could allocate or synchronise happens before the capture */
    const int last_fidx = h->t + k - 1 - c.startf;
    if (last_fidx >= 0)
        if (int rc = ensure_force_cap(h, last_fidx + 1)) return rc;
    /* the host-side step state the captured steps advance, put back when
     * the batch does not reach the GPU (its steps never ran) */
    const int t0 = h->t, cur0 = h->lv[0].cur, cur1 = h->lv[1].cur, dyn_n0 = h->dyn_n;
    const bool nu_valid0 = h->nu_valid;
    float* const mom0 = h->mom;
    float* const mom_prev0 = h->mom_prev;
    const bool have_mom0 = h->have_mom;
    const long long launches0 = h->launches;
    auto restore = [&] {
        h->t = t0, h->lv[0].cur = cur0, h->lv[1].cur = cur1, h->dyn_n = dyn_n0;
        h->mom = mom0, h->mom_prev = mom_prev0, h->have_mom = have_mom0, h->launches = launches0;
        h->nu_valid = nu_valid0;
    };
    CUDA_TRY(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    int rc = LBM_OK;
    for (int j = 0; j < k && rc == LBM_OK; ++j) rc = one_step(h);
    cudaGraph_t g = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(h->stream, &g);
    if (rc != LBM_OK || ec != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        restore();
        return rc != LBM_OK ? rc : fail(LBM_ERR_CUDA, "step capture: %s", cudaGetErrorString(ec));
    }
    cudaError_t e = cudaSuccess;
    cudaGraphExec_t& gx = h->gexec[k];
    if (gx) {
        cudaGraphExecUpdateResultInfo info{};
        if (cudaGraphExecUpdate(gx, g, &info) != cudaSuccess) {
            cudaGetLastError();
            cudaGraphExecDestroy(gx);
            gx = nullptr;
        }
    }
    if (!gx) e = cudaGraphInstantiate(&gx, g, 0);
    cudaGraphDestroy(g);
    if (e == cudaSuccess) e = cudaGraphLaunch(gx, h->stream);
    if (e != cudaSuccess) {
        restore();
        return fail(LBM_ERR_CUDA, "step graph: %s", cudaGetErrorString(e));
    }
    /* the graph's side-stream nodes replay on the main stream: later work
     * queued on the side stream (lbm_get_last_force_async) waits for it */
    e = cudaEventRecord(h->ev_fork, h->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(h->side, h->ev_fork, 0);
    if (e != cudaSuccess) return fail(LBM_ERR_CUDA, "step graph: %s", cudaGetErrorString(e));
    return LBM_OK;
}

int check_level(const lbm_handle* h, int level) {
    if (!h) return fail(LBM_ERR_ARG, "null handle");
    if (level < 0 || level >= h->nlevels) return fail(LBM_ERR_ARG, "level %d does not exist", level);
    return LBM_OK;
}

}  // namespace

/* ------------------------------------------------------------------------ */
/* C ABI                                                                       */
/* ------------------------------------------------------------------------ */

namespace {
const char CKPT_MAGIC[12] = {'L', 'B', 'M', 'G', 'B', '3', '0', '0', 'C', 'K', 'P', 'T'};
/* version 2: FP16 / BF16 levels store deviations from the collision model's
 * equilibrium (version 1 stored them from the BGK equilibrium) */
constexpr uint32_t CKPT_VERSION = 2;

template <class V> void put(std::ostream& o, const V& v) { o.write(reinterpret_cast<const char*>(&v), sizeof v); }
template <class V> bool get(std::istream& i, V& v) { return bool(i.read(reinterpret_cast<char*>(&v), sizeof v)); }
}  // namespace

extern "C" {

const char* lbm_last_error(void) { return g_err.c_str(); }
const char* lbm_version(void) { return "lbm_gb300 0.1 (sm_103a)"; }

int lbm_inputs_normalize(const char* inputs_text, char* buf, size_t cap, size_t* len) {
    Config c;
    if (int rc = parse_inputs(inputs_text, c)) return rc;
    float om, omlr, a, b;
    relaxation(c, om, omlr, a, b);
    std::string s = write_inputs(c, om, omlr);
    if (len) *len = s.size();
    if (buf && cap > 0) {
        size_t k = std::min(cap - 1, s.size());
        memcpy(buf, s.data(), k);
        buf[k] = 0;
        if (k < s.size()) return fail(LBM_ERR_ARG, "buffer of %zu bytes too small for %zu", cap, s.size() + 1);
    }
    return LBM_OK;
}

int lbm_inputs_mask(const char* inputs_text, int level, uint8_t* mask, size_t cap, size_t* n) {
    Config c;
    if (int rc = parse_inputs(inputs_text, c)) return rc;
    if (level < 0 || level > 1 || (level == 1 && !c.refinement)) return fail(LBM_ERR_ARG, "level %d does not exist", level);
    std::vector<uint8_t> m;
    if (level == 0) mask_base(c, m);
    else mask_fine(c, m);
    if (n) *n = m.size();
    if (mask) {
        if (cap < m.size()) return fail(LBM_ERR_ARG, "mask buffer of %zu bytes too small for %zu", cap, m.size());
        memcpy(mask, m.data(), m.size());
    }
    return LBM_OK;
}

static void write_level(std::ostream& out, std::ostream* slice, const Config& c, int level, const std::vector<float>& f,
                        const std::vector<float>& st, int nx, int ny, int nz);

/* WriteForces (LR7:2537-2545): "t, Fx/ref, Fy/ref, Fz/ref" with
 * ref = UMAX^2 ZDIM OBSTR1 (times LRLEVEL^2 with refinement), in FP32 as the
 * reference prints it */
static std::string format_forces(const Config& c, const double* F, int n) {
    std::ostringstream o;
    float ref = c.umax * c.umax * c.nz * c.r1;
    if (c.refinement) ref *= std::lround(1.0 / c.lrfactor) * std::lround(1.0 / c.lrfactor);
    for (int i = 0; i < n; ++i)
        o << i + c.startf << ", " << float(F[3 * i]) / ref << ", " << float(F[3 * i + 1]) / ref << ", "
          << float(F[3 * i + 2]) / ref << std::endl;
    return o.str();
}

static int copy_out(const std::string& s, char* buf, size_t cap, size_t* len) {
    if (len) *len = s.size();
    if (buf && cap > 0) {
        size_t k = std::min(cap - 1, s.size());
        memcpy(buf, s.data(), k);
        buf[k] = 0;
        if (k < s.size()) return fail(LBM_ERR_ARG, "buffer of %zu bytes too small for %zu", cap, s.size() + 1);
    }
    return LBM_OK;
}

int lbm_format_tecplot(const char* inputs_text, int level, const float* f, const float* stats4, char* buf, size_t cap,
                       size_t* len, char* slice, size_t slice_cap, size_t* slice_len) {
    Config c;
    if (int rc = parse_inputs(inputs_text, c)) return rc;
    if (!f) return fail(LBM_ERR_ARG, "f is null");
    if (level < 0 || level > 1 || (level == 1 && !c.refinement)) return fail(LBM_ERR_ARG, "level %d does not exist", level);
    const int nx = level ? c.lrx : c.nx, ny = level ? c.lry : c.ny, nz = level ? c.lrz : c.nz;
    const size_t N = size_t(nx) * ny * nz;
    std::vector<float> fv(f, f + 19 * N), st;
    if (stats4) st.assign(stats4, stats4 + 4 * N);
    std::ostringstream zone, sl;
    write_level(zone, &sl, c, level, fv, st, nx, ny, nz);
    if (int rc = copy_out(zone.str(), buf, cap, len)) return rc;
    return copy_out(sl.str(), slice, slice_cap, slice_len);
}

int lbm_create(const char* inputs_text, lbm_handle** out) {
    if (!out) return fail(LBM_ERR_ARG, "out is null");
    *out = nullptr;
    Config c;
    int rc = parse_inputs(inputs_text, c);
    if (rc) return rc;
    const int model = model_id(c.model);
    if (model < 0) return fail(LBM_ERR_CONFIG, "MODEL '%s' is not one of MRT, MRT_DI3, BGK, MRT_CPU3D", c.model.c_str());
    const int storage = storage_id(c.precision);
    if (storage < 0) return fail(LBM_ERR_CONFIG, "PRECISION '%s' is not one of fp32, fp16, bf16, fp64", c.precision.c_str());
    const int blocked = c.pop_layout == "blocked" || (c.pop_layout == "auto" && storage != STORE_F64) ? 1 : 0;
    if (blocked && storage == STORE_F64) return fail(LBM_ERR_CONFIG, "LAYOUT blocked is for FP32, FP16 and BF16 storage");
    static const char* geoms[] = {"channel_square", "channel_circle", "channel", "cavity", "periodic", "dyninlet", "duct"};
    if (std::find(std::begin(geoms), std::end(geoms), c.geometry) == std::end(geoms))
        return fail(LBM_ERR_CONFIG, "GEOMETRY '%s' is not supported", c.geometry.c_str());
    if (c.refinement) {
        /* LR7:2624-2627 */
        const int lev = int(std::lround(1.0 / c.lrfactor));
        if (std::fabs(c.lrfactor - 1.f / lev) > 0.001f || lev < 2)
            return fail(LBM_ERR_CONFIG, "LR factor %g is not 1/LRLEVEL", c.lrfactor);
        /* the reference's patch spans the periodic z extent from
         * z = -(1 - LRFACTOR/2); a patch bounded in z (an extension) sits in z
         * as in x and y */
        const bool full_z = c.lrz == lev * c.nz && std::fabs(c.lrz0 + (1.f - 0.5f * c.lrfactor)) <= 1e-6f;
        auto half_past = [&](float v) { return std::fabs((v - std::floor(v)) - 0.5f * c.lrfactor) <= 1e-6f; };
        if (!half_past(c.lrx0) || !half_past(c.lry0) || (!full_z && !half_past(c.lrz0)))
            return fail(LBM_ERR_CONFIG, "LR location must sit at half a fine spacing past a coarse node (or, spanning "
                                        "z, at z = %g)", -(1.f - 0.5f * c.lrfactor));
        if (!full_z) {
            const int ez = int(c.lrz * c.lrfactor) + 1;
            if (c.lrz0 < 0.f || int(c.lrz0) + ez > c.nz || c.lrz >= lev * c.nz)
                return fail(LBM_ERR_CONFIG, "a z-bounded refinement patch must lie inside the base grid's z extent");
            if (c.lrz < 2 * lev + 2) return fail(LBM_ERR_CONFIG, "refinement patch too small");
        }
        const int ex = int(c.lrx * c.lrfactor) + 1, ey = int(c.lry * c.lrfactor) + 1;
        if (int(c.lrx0) < 0 || int(c.lry0) < 0 || int(c.lrx0) + ex > c.nx || int(c.lry0) + ey > c.ny)
            return fail(LBM_ERR_CONFIG, "refinement patch does not fit in the base grid");
        if (c.lrx < 2 * lev + 2 || c.lry < 2 * lev + 2) return fail(LBM_ERR_CONFIG, "refinement patch too small");
    }
    /* the closure's collision carries no body force (the dynamic inlet's
     * DPDY drive) */
    if (c.sgs_mlp && (c.refinement || c.geometry == "cavity" || c.geometry == "duct" || c.geometry == "dyninlet" ||
                      c.faces_set || c.pull_clamp || c.dpdy != 0.f || storage == STORE_F64))
        return fail(LBM_ERR_CONFIG, "SGS mlp runs on channel and periodic levels without refinement, FACES or a "
                                    "body force (DPDY), FP32/FP16/BF16");
    std::vector<float> sgs_params;
    if (!c.sgs_weights.empty()) {
        std::ifstream in(c.sgs_weights, std::ios::binary);
        sgs_params.resize(sgs::NPARAM);
        if (!in.read(reinterpret_cast<char*>(sgs_params.data()), sgs::NPARAM * sizeof(float)))
            return fail(LBM_ERR_CONFIG, "SGS weights: cannot read %d float32 values from '%s'", sgs::NPARAM,
                        c.sgs_weights.c_str());
    }
    int dev = 0;
    CUDA_TRY(cudaGetDevice(&dev));
    lbm_handle* h = new lbm_handle();
    h->cfg = c;
    h->model = model;
    h->storage = storage;
    relaxation(c, h->omega, h->omegaLR, h->sf_cf, h->sf_fc);
    h->nlevels = c.refinement ? 2 : 1;
    auto bail = [&](int code) {
        lbm_destroy(h);
        return code;
    };
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess)
        return bail(fail(LBM_ERR_CUDA, "cannot create a CUDA stream"));
    cudaEventCreate(&h->ev0);
    cudaEventCreate(&h->ev1);
    {
        int lo = 0, hi = 0;
        cudaDeviceGetStreamPriorityRange(&lo, &hi);
        if (cudaStreamCreateWithPriority(&h->side, cudaStreamNonBlocking, hi) != cudaSuccess ||
            cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming) != cudaSuccess)
            return bail(fail(LBM_ERR_CUDA, "cannot create the force stream"));
    }
    /* reference velocity of the FP16/BF16 offsets: the inlet velocity of a channel */
    const float u_ref = c.geometry.rfind("channel", 0) == 0 || c.geometry == "duct" ? c.umax : 0.f;
    if ((rc = alloc_level(h->lv[0], c.nx, c.ny, c.nz, storage, blocked, c.velav != 0, u_ref, model))) return bail(rc);
    mask_base(c, h->lv[0].hmask);
    h->trip_in_mask = c.geometry == "dyninlet" && c.trip_end > 0;
    if (c.dyny1 >= 0) {
        if (c.dyny1 >= c.ny || c.dyn_every <= 0)
            return bail(fail(LBM_ERR_CONFIG, "DYNY1 %d must lie in 0..%d and DYN every be positive", c.dyny1, c.ny - 1));
        h->dyn_cap = std::max(1, c.tmax / c.dyn_every + 2);
        if (cudaMalloc(&h->dpdy_dev, sizeof(float)) != cudaSuccess ||
            cudaMalloc(&h->dyn_hist, size_t(h->dyn_cap) * 3 * sizeof(float)) != cudaSuccess)
            return bail(fail(LBM_ERR_NOMEM, "dynamic inlet buffers"));
        cudaMemcpy(h->dpdy_dev, &c.dpdy, sizeof(float), cudaMemcpyHostToDevice);
    }
    if ((rc = upload_mask(h, 0))) return bail(rc);
    if (c.refinement) {
        if ((rc = alloc_level(h->lv[1], c.lrx, c.lry, c.lrz, storage, blocked, c.velav != 0, u_ref, model)))
            return bail(rc);
        mask_fine(c, h->lv[1].hmask);
        if ((rc = upload_mask(h, 1))) return bail(rc);
        h->enx = int(c.lrx * c.lrfactor) + 1;
        h->eny = int(c.lry * c.lrfactor) + 1;
        if (c.cf_time) {
            if (cudaMalloc(&h->mom_prev, size_t(9) * h->enx * h->eny * c.nz * sizeof(float)) != cudaSuccess)
                return bail(fail(LBM_ERR_NOMEM, "cannot allocate the second moment export"));
            cudaMemset(h->mom_prev, 0, size_t(9) * h->enx * h->eny * c.nz * sizeof(float));
        }
        if (cudaMalloc(&h->mom, size_t(9) * h->enx * h->eny * c.nz * sizeof(float)) != cudaSuccess)
            return bail(fail(LBM_ERR_NOMEM, "cannot allocate the moment export"));
        cudaMemset(h->mom, 0, size_t(9) * h->enx * h->eny * c.nz * sizeof(float));
        RefineParams& r = h->rp;
        r.cnx = c.nx; r.cny = c.ny; r.cnz = c.nz;
        r.fnx = c.lrx; r.fny = c.lry; r.fnz = c.lrz;
        r.lrx0 = c.lrx0; r.lry0 = c.lry0; r.lrz0 = c.lrz0;
        r.lrfactor = c.lrfactor;
        r.lrlevel = int(std::lround(1.0 / c.lrfactor));
        r.order = c.order;
        r.cs = c.cs;
        r.omega_c = h->omega;
        r.omega_f = h->omegaLR;
        r.quirk_fc_top_zflip = c.fc_zflip;
        r.zbounded = c.lrz != r.lrlevel * c.nz || std::fabs(c.lrz0 + (1.f - 0.5f * c.lrfactor)) > 1e-6f;
        r.cz0 = r.zbounded ? int(c.lrz0) : 0;
        r.enx = h->enx;
        r.eny = h->eny;
    }
    if (cudaMalloc(&h->audit_part, size_t(audit_partials(h->lv[0].L)) * 4 * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&h->audit_out, 4 * sizeof(double)) != cudaSuccess)
        return bail(fail(LBM_ERR_NOMEM, "cannot allocate audit scratch"));
    if ((rc = ensure_force_cap(h, std::max(1, c.tmax - c.startf)))) return bail(rc);
    if (c.sgs_mlp && c.sgs_every > 1) {
        const size_t nb = size_t(h->lv[0].L.qstride) * sizeof(float);
        if (cudaMalloc(&h->lv[0].nu, nb) != cudaSuccess || cudaMemset(h->lv[0].nu, 0, nb) != cudaSuccess)
            return bail(fail(LBM_ERR_NOMEM, "cannot allocate the closure's eddy-viscosity buffer"));
    }
    if (!sgs_params.empty() && (rc = lbm_set_sgs_mlp(h, sgs_params.data(), sgs::NPARAM))) return bail(rc);
    if ((rc = do_init(h))) return bail(rc);
    *out = h;
    return LBM_OK;
}

int lbm_destroy(lbm_handle* h) {
    if (!h) return LBM_OK;
    if (h->stream) cudaStreamSynchronize(h->stream);
    for (auto& s : h->lv) free_level(s);
    cudaFree(h->force_hist);
    cudaFree(h->mom);
    cudaFree(h->mom_prev);
    cudaFree(h->audit_part);
    cudaFree(h->audit_out);
    if (h->ev0) cudaEventDestroy(h->ev0);
    if (h->ev1) cudaEventDestroy(h->ev1);
    cudaFree(h->mlp_blob);
    cudaFree(h->mlp_err);
    cudaFree(h->dpdy_dev);
    cudaFree(h->dyn_hist);
    if (h->ev_fork) cudaEventDestroy(h->ev_fork);
    if (h->ev_join) cudaEventDestroy(h->ev_join);
    for (cudaGraphExec_t& g : h->gexec)
        if (g) cudaGraphExecDestroy(g);
    cudaFree(h->stage);
    if (h->side) cudaStreamDestroy(h->side);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return LBM_OK;
}

int lbm_get_dims(const lbm_handle* h, int level, int* nx, int* ny, int* nz) {
    if (int rc = check_level(h, level)) return rc;
    const Level& L = h->lv[level].L;
    if (nx) *nx = L.nx;
    if (ny) *ny = L.ny;
    if (nz) *nz = L.nz;
    return LBM_OK;
}

int lbm_get_nlevels(const lbm_handle* h, int* n) {
    if (!h || !n) return fail(LBM_ERR_ARG, "null argument");
    *n = h->nlevels;
    return LBM_OK;
}

int lbm_get_params(const lbm_handle* h, float* o) {
    if (!h || !o) return fail(LBM_ERR_ARG, "null argument");
    o[0] = h->omega;
    o[1] = h->omegaLR;
    o[2] = h->sf_cf;
    o[3] = h->sf_fc;
    return LBM_OK;
}

int lbm_get_storage_offsets(const lbm_handle* h, int level, float* off19) {
    if (int rc = check_level(h, level)) return rc;
    if (!off19) return fail(LBM_ERR_ARG, "off19 is null");
    std::memcpy(off19, h->lv[level].L.off, sizeof(float) * 19);
    return LBM_OK;
}

int lbm_get_time(const lbm_handle* h, int* t) {
    if (!h || !t) return fail(LBM_ERR_ARG, "null argument");
    *t = h->t;
    return LBM_OK;
}

int lbm_get_mask(const lbm_handle* h, int level, uint8_t* mask) {
    if (int rc = check_level(h, level)) return rc;
    if (!mask) return fail(LBM_ERR_ARG, "mask is null");
    memcpy(mask, h->lv[level].hmask.data(), h->lv[level].hmask.size());
    return LBM_OK;
}

int lbm_set_mask(lbm_handle* h, int level, const uint8_t* mask) {
    if (int rc = check_level(h, level)) return rc;
    if (!mask) return fail(LBM_ERR_ARG, "mask is null");
    for (size_t i = 0; i < h->lv[level].hmask.size(); ++i)
        if (mask[i] >= NODE_TYPES) return fail(LBM_ERR_ARG, "mask value %d at %zu is not a node type", int(mask[i]), i);
    memcpy(h->lv[level].hmask.data(), mask, h->lv[level].hmask.size());
    return upload_mask(h, level);
}

int lbm_set_geometry(lbm_handle* h, const uint8_t* mask) {
    if (!h) return fail(LBM_ERR_ARG, "null handle");
    if (mask) return lbm_set_mask(h, 0, mask);
    /* the record's analytic geometry (ImageFcn / ImageFcnLR) at the handle's time */
    mask_base(h->cfg, h->lv[0].hmask, h->t);
    if (int rc = upload_mask(h, 0)) return rc;
    h->trip_in_mask = h->cfg.geometry == "dyninlet" && h->t < h->cfg.trip_end;
    if (h->nlevels > 1) {
        mask_fine(h->cfg, h->lv[1].hmask);
        if (int rc = upload_mask(h, 1)) return rc;
    }
    return LBM_OK;
}

int lbm_init_equilibrium(lbm_handle* h) {
    if (!h) return fail(LBM_ERR_ARG, "null handle");
    return do_init(h);
}

/* the handle's FP32 staging buffer, at least n floats */
static int staging(lbm_handle* h, size_t n, float** d) {
    if (h->stage_n < n) {
        CUDA_TRY(cudaStreamSynchronize(h->stream));
        cudaFree(h->stage);
        h->stage = nullptr;
        h->stage_n = 0;
        CUDA_TRY(cudaMalloc((void**)&h->stage, n * sizeof(float)));
        h->stage_n = n;
    }
    *d = h->stage;
    return LBM_OK;
}

/* the device's address of a caller buffer it can reach directly: page-locked
 * host memory mapped into the device's address space (cudaHostAlloc, or
 * cudaHostRegister with mapping, on a unified-addressing system); null for
 * pageable memory.  The layout kernels then read or write such a buffer over
 * the host link themselves: one pass, no copy engine and no staging copy */
static void* mapped_view(const void* p) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

int lbm_get_populations(lbm_handle* h, int level, float* f) {
    if (int rc = check_level(h, level)) return rc;
    if (!f) return fail(LBM_ERR_ARG, "f is null");
    LevelState& s = h->lv[level];
    const size_t n = size_t(s.L.nx) * s.L.ny * s.L.nz * 19;
    if (s.L.storage == STORE_F32 && s.L.pitch == s.L.nx && !s.L.blocked) {
        /* FP32 without row padding: the stored layout is the caller's */
        cudaError_t e = cudaMemcpyAsync(f, s.f[s.cur], n * sizeof(float), cudaMemcpyDeviceToHost, h->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
        if (e != cudaSuccess) return fail(LBM_ERR_CUDA, "get_populations: %s", cudaGetErrorString(e));
        return LBM_OK;
    }
    cudaError_t e;
    if (void* dv = mapped_view(f)) {
        e = launch_pack(s.L, s.f[s.cur], static_cast<float*>(dv), h->stream);
        ++h->launches;
    } else {
        float* d = nullptr;
        if (int rc = staging(h, n, &d)) return rc;
        e = launch_pack(s.L, s.f[s.cur], d, h->stream);
        ++h->launches;
        if (e == cudaSuccess) e = cudaMemcpyAsync(f, d, n * sizeof(float), cudaMemcpyDeviceToHost, h->stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return fail(LBM_ERR_CUDA, "get_populations: %s", cudaGetErrorString(e));
    return LBM_OK;
}

int lbm_set_populations(lbm_handle* h, int level, const float* f) {
    if (int rc = check_level(h, level)) return rc;
    if (!f) return fail(LBM_ERR_ARG, "f is null");
    LevelState& s = h->lv[level];
    h->nu_valid = false; /* the closure is evaluated again on the next step */
    const size_t n = size_t(s.L.nx) * s.L.ny * s.L.nz * 19;
    if (s.L.storage == STORE_F32 && s.L.pitch == s.L.nx && !s.L.blocked) {
        /* FP32 without row padding: straight into both buffers */
        cudaError_t e = cudaMemcpyAsync(s.f[0], f, n * sizeof(float), cudaMemcpyHostToDevice, h->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(s.f[1], s.f[0], n * sizeof(float), cudaMemcpyDeviceToDevice, h->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
        if (e != cudaSuccess) return fail(LBM_ERR_CUDA, "set_populations: %s", cudaGetErrorString(e));
        return LBM_OK;
    }
    cudaError_t e;
    if (const void* dv = mapped_view(f)) {
        /* one read of the host buffer into the current buffer, then a device
         * copy into the other */
        e = launch_unpack(s.L, static_cast<const float*>(dv), s.f[0], h->stream);
        ++h->launches;
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(s.f[1], s.f[0], size_t(s.L.qstride) * 19 * storage_bytes(s.L.storage),
                                cudaMemcpyDeviceToDevice, h->stream);
    } else {
        float* d = nullptr;
        if (int rc = staging(h, n, &d)) return rc;
        e = cudaMemcpyAsync(d, f, n * sizeof(float), cudaMemcpyHostToDevice, h->stream);
        for (int i = 0; i < 2 && e == cudaSuccess; ++i, ++h->launches) e = launch_unpack(s.L, d, s.f[i], h->stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return fail(LBM_ERR_CUDA, "set_populations: %s", cudaGetErrorString(e));
    return LBM_OK;
}

int lbm_step(lbm_handle* h, int nsteps) {
    if (!h) return fail(LBM_ERR_ARG, "null handle");
    if (nsteps < 0) return fail(LBM_ERR_ARG, "nsteps %d < 0", nsteps);
    /* the first step is launched directly and the batches grow 2, 4, 8, 16,
     * so that the host captures each batch while the GPU runs the one
     * before (one executable graph per batch length, updated in place) */
    int kb = 1;
    for (int i = 0; i < nsteps;) {
        const int k = std::min(kb, nsteps - i);
        kb = std::min(2 * kb, GRAPH_STEPS);
        int rc;
        if (k >= 2 && graph_ok(h, k)) {
            rc = run_graph(h, k);
            i += k;
        } else {
            rc = one_step(h);
            ++i;
        }
        if (rc) return rc;
    }
    return LBM_OK;
}

int lbm_step_timed(lbm_handle* h, int nsteps, float* ms) {
    if (!h || !ms) return fail(LBM_ERR_ARG, "null argument");
    CUDA_TRY(cudaEventRecord(h->ev0, h->stream));
    if (int rc = lbm_step(h, nsteps)) return rc;
    CUDA_TRY(cudaEventRecord(h->ev1, h->stream));
    CUDA_TRY(cudaEventSynchronize(h->ev1));
    CUDA_TRY(cudaEventElapsedTime(ms, h->ev0, h->ev1));
    return LBM_OK;
}

int lbm_synchronize(lbm_handle* h) {
    if (!h) return fail(LBM_ERR_ARG, "null handle");
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->side));
    if (h->mlp_err) {
        int e = 0;
        CUDA_TRY(cudaMemcpy(&e, h->mlp_err, sizeof(int), cudaMemcpyDeviceToHost));
        if (e) {
            cudaMemset(h->mlp_err, 0, sizeof(int));
            return fail(LBM_ERR_CUDA, "SGS mlp: a tensor-core completion wait ran out");
        }
    }
    return LBM_OK;
}

int lbm_set_sgs_mlp(lbm_handle* h, const float* params, int n) {
    if (!h || !params) return fail(LBM_ERR_ARG, "null argument");
    if (n != sgs::NPARAM) return fail(LBM_ERR_ARG, "SGS mlp: %d parameters, expected %d", n, sgs::NPARAM);
    if (!h->cfg.sgs_mlp) return fail(LBM_ERR_STATE, "SGS mlp: the record does not select 'SGS: mlp'");
    std::vector<unsigned char> blob(sgs::BLOB_BYTES);
    mlp_make_blob(params, blob.data());
    if (!h->mlp_blob) CUDA_TRY(cudaMalloc(&h->mlp_blob, sgs::BLOB_BYTES));
    if (!h->mlp_err) {
        CUDA_TRY(cudaMalloc(&h->mlp_err, sizeof(int)));
        CUDA_TRY(cudaMemset(h->mlp_err, 0, sizeof(int)));
    }
    CUDA_TRY(cudaMemcpyAsync(h->mlp_blob, blob.data(), blob.size(), cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    h->mlp_params.assign(params, params + n);
    h->mlp_ready = true;
    h->nu_valid = false;
    return LBM_OK;
}

/* ------------------------------------------------------------------------ */
/* checkpoint / restart (no counterpart in the reference)                     */
/* ------------------------------------------------------------------------ */

int lbm_save_state(lbm_handle* h, const char* path) {
    if (!h || !path) return fail(LBM_ERR_ARG, "null argument");
    if (int rc = lbm_synchronize(h)) return rc;
    std::ofstream o(path, std::ios::binary);
    if (!o) return fail(LBM_ERR_ARG, "checkpoint: cannot write '%s'", path);
    const std::string rec = write_inputs(h->cfg, h->omega, h->omegaLR);
    o.write(CKPT_MAGIC, sizeof CKPT_MAGIC);
    put(o, CKPT_VERSION);
    put(o, uint64_t(rec.size()));
    o.write(rec.data(), std::streamsize(rec.size()));
    put(o, int32_t(h->t));
    put(o, int32_t(h->nlevels));
    for (int l = 0; l < h->nlevels; ++l) {
        const LevelState& s = h->lv[l];
        const Level& L = s.L;
        /* storage code + 256 for the blocked layout: the raw populations are
         * only readable back into the same layout */
        const int32_t hdr[6] = {L.nx, L.ny, L.nz, L.pitch, h->storage + 256 * L.blocked, s.stats ? 1 : 0};
        for (int32_t v : hdr) put(o, v);
        /* the stored populations as they are (raw FP16 / BF16 / FP32 / FP64) */
        std::vector<char> raw(size_t(L.qstride) * 19 * storage_bytes(h->storage));
        CUDA_TRY(cudaMemcpy(raw.data(), s.f[s.cur], raw.size(), cudaMemcpyDeviceToHost));
        o.write(raw.data(), std::streamsize(raw.size()));
        if (s.stats) {
            std::vector<float> st(size_t(L.qstride) * 4);
            CUDA_TRY(cudaMemcpy(st.data(), s.stats, st.size() * sizeof(float), cudaMemcpyDeviceToHost));
            o.write(reinterpret_cast<const char*>(st.data()), std::streamsize(st.size() * sizeof(float)));
        }
    }
    const int32_t nf = std::max(0, std::min(h->t - h->cfg.startf, h->force_cap));
    put(o, nf);
    if (nf > 0) {
        std::vector<double> fh(size_t(nf) * 3);
        CUDA_TRY(cudaMemcpy(fh.data(), h->force_hist, fh.size() * sizeof(double), cudaMemcpyDeviceToHost));
        o.write(reinterpret_cast<const char*>(fh.data()), std::streamsize(fh.size() * sizeof(double)));
    }
    put(o, int32_t(h->mlp_params.size()));
    if (!h->mlp_params.empty())
        o.write(reinterpret_cast<const char*>(h->mlp_params.data()), std::streamsize(h->mlp_params.size() * 4));
    /* dynamic inlet: the controlled body force and the control history */
    float dp = h->cfg.dpdy;
    if (h->dpdy_dev) CUDA_TRY(cudaMemcpy(&dp, h->dpdy_dev, sizeof(float), cudaMemcpyDeviceToHost));
    put(o, dp);
    put(o, int32_t(h->dyn_n));
    if (h->dyn_n > 0) {
        std::vector<float> hh(size_t(h->dyn_n) * 3);
        CUDA_TRY(cudaMemcpy(hh.data(), h->dyn_hist, hh.size() * sizeof(float), cudaMemcpyDeviceToHost));
        o.write(reinterpret_cast<const char*>(hh.data()), std::streamsize(hh.size() * sizeof(float)));
    }
    /* CF TIME linear: the last coarse export, which the next step blends */
    if (h->cfg.refinement && h->cfg.cf_time) {
        put(o, int32_t(h->have_mom ? 1 : 0));
        if (h->have_mom) {
            std::vector<float> m(size_t(9) * h->enx * h->eny * h->cfg.nz);
            CUDA_TRY(cudaMemcpy(m.data(), h->mom, m.size() * sizeof(float), cudaMemcpyDeviceToHost));
            o.write(reinterpret_cast<const char*>(m.data()), std::streamsize(m.size() * sizeof(float)));
        }
    }
    if (!o) return fail(LBM_ERR_ARG, "checkpoint: write to '%s' failed", path);
    return LBM_OK;
}

static const char* layout_name(int b) { return b == 0 ? "soa" : b == 1 ? "blocked" : "unknown"; }

static int read_checkpoint_record(std::istream& in, std::string& rec) {
    char magic[sizeof CKPT_MAGIC];
    uint32_t ver = 0;
    uint64_t len = 0;
    if (!in.read(magic, sizeof magic) || std::memcmp(magic, CKPT_MAGIC, sizeof magic) != 0)
        return fail(LBM_ERR_PARSE, "checkpoint: not a checkpoint file");
    if (!get(in, ver) || ver != CKPT_VERSION) return fail(LBM_ERR_PARSE, "checkpoint: version %u not readable", ver);
    if (!get(in, len) || len > (1u << 24)) return fail(LBM_ERR_PARSE, "checkpoint: bad record length");
    rec.resize(len);
    if (!in.read(&rec[0], std::streamsize(len))) return fail(LBM_ERR_PARSE, "checkpoint: truncated record");
    return LBM_OK;
}

int lbm_restore_state(lbm_handle* h, const char* path) {
    if (!h || !path) return fail(LBM_ERR_ARG, "null argument");
    std::ifstream in(path, std::ios::binary);
    if (!in) return fail(LBM_ERR_ARG, "checkpoint: cannot read '%s'", path);
    std::string rec;
    if (int rc = read_checkpoint_record(in, rec)) return rc;
    int32_t t = 0, nl = 0;
    if (!get(in, t) || !get(in, nl) || nl != h->nlevels || t < 0)
        return fail(LBM_ERR_CONFIG, "checkpoint: %d levels, the handle has %d", nl, h->nlevels);
    if (int rc = lbm_synchronize(h)) return rc;
    for (int l = 0; l < nl; ++l) {
        LevelState& s = h->lv[l];
        const Level& L = s.L;
        int32_t hdr[6];
        for (int32_t& v : hdr)
            if (!get(in, v)) return fail(LBM_ERR_PARSE, "checkpoint: truncated level header");
        if (hdr[0] != L.nx || hdr[1] != L.ny || hdr[2] != L.nz || hdr[3] != L.pitch ||
            hdr[4] != h->storage + 256 * L.blocked)
            return fail(LBM_ERR_CONFIG, "checkpoint: level %d is %dx%dx%d (pitch %d, storage %d, layout %s), the "
                        "handle's %dx%dx%d (storage %d, layout %s)", l, hdr[0], hdr[1], hdr[2], hdr[3], hdr[4] & 255,
                        layout_name(hdr[4] >> 8), L.nx, L.ny, L.nz, h->storage, layout_name(L.blocked));
        std::vector<char> raw(size_t(L.qstride) * 19 * storage_bytes(h->storage));
        if (!in.read(raw.data(), std::streamsize(raw.size()))) return fail(LBM_ERR_PARSE, "checkpoint: truncated level");
        for (int b = 0; b < 2; ++b) CUDA_TRY(cudaMemcpy(s.f[b], raw.data(), raw.size(), cudaMemcpyHostToDevice));
        s.cur = 0;
        if (hdr[5]) {
            std::vector<float> st(size_t(L.qstride) * 4);
            if (!in.read(reinterpret_cast<char*>(st.data()), std::streamsize(st.size() * 4)))
                return fail(LBM_ERR_PARSE, "checkpoint: truncated statistics");
            if (s.stats) CUDA_TRY(cudaMemcpy(s.stats, st.data(), st.size() * 4, cudaMemcpyHostToDevice));
        }
    }
    int32_t nf = 0;
    if (!get(in, nf) || nf < 0) return fail(LBM_ERR_PARSE, "checkpoint: bad force history");
    if (nf > 0) {
        std::vector<double> fh(size_t(nf) * 3);
        if (!in.read(reinterpret_cast<char*>(fh.data()), std::streamsize(fh.size() * 8)))
            return fail(LBM_ERR_PARSE, "checkpoint: truncated force history");
        if (int rc = ensure_force_cap(h, nf)) return rc;
        CUDA_TRY(cudaMemcpy(h->force_hist, fh.data(), fh.size() * 8, cudaMemcpyHostToDevice));
    }
    int32_t np = 0;
    if (get(in, np) && np > 0) {
        std::vector<float> prm(np);
        if (!in.read(reinterpret_cast<char*>(prm.data()), std::streamsize(np) * 4))
            return fail(LBM_ERR_PARSE, "checkpoint: truncated closure weights");
        if (h->cfg.sgs_mlp)
            if (int rc = lbm_set_sgs_mlp(h, prm.data(), np)) return rc;
    }
    float dp = 0;
    int32_t nd = 0;
    if (get(in, dp) && get(in, nd) && nd >= 0) {
        std::vector<float> hh(size_t(nd) * 3);
        if (nd > 0 && !in.read(reinterpret_cast<char*>(hh.data()), std::streamsize(hh.size() * 4)))
            return fail(LBM_ERR_PARSE, "checkpoint: truncated control history");
        if (h->dpdy_dev) {
            CUDA_TRY(cudaMemcpy(h->dpdy_dev, &dp, sizeof(float), cudaMemcpyHostToDevice));
            const int k = std::min(int(nd), h->dyn_cap);
            if (k > 0) CUDA_TRY(cudaMemcpy(h->dyn_hist, hh.data(), size_t(k) * 3 * 4, cudaMemcpyHostToDevice));
            h->dyn_n = k;
        }
    }
    h->have_mom = false;
    if (h->cfg.refinement && h->cfg.cf_time) {
        int32_t hm = 0;
        if (get(in, hm) && hm) {
            std::vector<float> m(size_t(9) * h->enx * h->eny * h->cfg.nz);
            if (!in.read(reinterpret_cast<char*>(m.data()), std::streamsize(m.size() * sizeof(float))))
                return fail(LBM_ERR_PARSE, "checkpoint: truncated moment export");
            CUDA_TRY(cudaMemcpy(h->mom, m.data(), m.size() * sizeof(float), cudaMemcpyHostToDevice));
            h->have_mom = true;
        }
    }
    /* the trip blocks are in the mask only before TRIP end */
    if (h->cfg.geometry == "dyninlet" && h->trip_in_mask != (t < h->cfg.trip_end)) {
        mask_base(h->cfg, h->lv[0].hmask, t);
        if (int rc = upload_mask(h, 0)) return rc;
        h->trip_in_mask = t < h->cfg.trip_end;
    }
    h->t = t;
    h->nu_valid = false;
    return LBM_OK;
}

int lbm_create_from_state(const char* path, lbm_handle** out) {
    if (!path || !out) return fail(LBM_ERR_ARG, "null argument");
    *out = nullptr;
    std::string rec;
    {
        std::ifstream in(path, std::ios::binary);
        if (!in) return fail(LBM_ERR_ARG, "checkpoint: cannot read '%s'", path);
        if (int rc = read_checkpoint_record(in, rec)) return rc;
    }
    lbm_handle* h = nullptr;
    if (int rc = lbm_create(rec.c_str(), &h)) return rc;
    if (int rc = lbm_restore_state(h, path)) {
        const std::string msg = g_err;
        lbm_destroy(h);
        g_err = msg;
        return rc;
    }
    *out = h;
    return LBM_OK;
}

int lbm_get_fields(lbm_handle* h, int level, float* rho, float* u, float* v, float* w) {
    if (int rc = check_level(h, level)) return rc;
    LevelState& s = h->lv[level];
    const size_t n = size_t(s.L.nx) * s.L.ny * s.L.nz;
    float* d = nullptr;
    CUDA_TRY(cudaMallocAsync((void**)&d, 4 * n * sizeof(float), h->stream));
    cudaError_t e = launch_fields(s.L, s.f[s.cur], d, d + n, d + 2 * n, d + 3 * n, h->stream);
    ++h->launches;
    float* outs[4] = {rho, u, v, w};
    for (int i = 0; i < 4 && e == cudaSuccess; ++i)
        if (outs[i]) e = cudaMemcpyAsync(outs[i], d + i * n, n * sizeof(float), cudaMemcpyDeviceToHost, h->stream);
    cudaFreeAsync(d, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return fail(LBM_ERR_CUDA, "get_fields: %s", cudaGetErrorString(e));
    return LBM_OK;
}

int lbm_get_stats(lbm_handle* h, int level, float* stats4) {
    if (int rc = check_level(h, level)) return rc;
    LevelState& s = h->lv[level];
    if (!s.stats) return fail(LBM_ERR_STATE, "statistics are off (VELAV: 0)");
    const Level& L = s.L;
    const size_t n = size_t(L.nx) * L.ny * L.nz;
    std::vector<float> tmp(size_t(L.qstride) * 4);
    CUDA_TRY(cudaMemcpyAsync(tmp.data(), s.stats, tmp.size() * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    for (int k = 0; k < 4; ++k)
        for (int z = 0; z < L.nz; ++z)
            for (int y = 0; y < L.ny; ++y)
                memcpy(stats4 + k * n + (size_t(z) * L.ny + y) * L.nx,
                       tmp.data() + k * L.qstride + size_t(z) * L.plane + size_t(y) * L.pitch, L.nx * sizeof(float));
    return LBM_OK;
}

int lbm_get_forces(lbm_handle* h, double* fxyz, int max_steps, int* n) {
    if (!h || !fxyz || max_steps < 0) return fail(LBM_ERR_ARG, "bad argument");
    const int avail = std::max(0, std::min(h->t - h->cfg.startf, h->force_cap));
    const int k = std::min(avail, max_steps);
    if (k > 0) {
        CUDA_TRY(cudaMemcpyAsync(fxyz, h->force_hist, size_t(k) * 3 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
        CUDA_TRY(cudaStreamSynchronize(h->stream));
    }
    if (n) *n = k;
    return LBM_OK;
}

int lbm_get_dyn_history(lbm_handle* h, float* hist3, int max_entries, int* n) {
    if (!h || max_entries < 0 || (max_entries > 0 && !hist3)) return fail(LBM_ERR_ARG, "bad argument");
    const int k = std::min(h->dyn_n, max_entries);
    if (k > 0) {
        CUDA_TRY(cudaMemcpyAsync(hist3, h->dyn_hist, size_t(k) * 3 * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
        CUDA_TRY(cudaStreamSynchronize(h->stream));
    }
    if (n) *n = h->dyn_n;
    return LBM_OK;
}

int lbm_get_launch_count(const lbm_handle* h, long long* n) {
    if (!h || !n) return fail(LBM_ERR_ARG, "null argument");
    *n = h->launches;
    return LBM_OK;
}

int lbm_get_last_force(lbm_handle* h, double* f3) {
    if (!h || !f3) return fail(LBM_ERR_ARG, "null argument");
    const int i = h->t - 1 - h->cfg.startf;
    if (i < 0 || i >= h->force_cap) {
        f3[0] = f3[1] = f3[2] = 0.0;
        return LBM_OK;
    }
    CUDA_TRY(cudaMemcpyAsync(f3, h->force_hist + 3LL * i, 3 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    return LBM_OK;
}

int lbm_get_last_force_async(lbm_handle* h, double* f3) {
    if (!h || !f3) return fail(LBM_ERR_ARG, "null argument");
    const int i = h->t - 1 - h->cfg.startf;
    if (i < 0 || i >= h->force_cap) {
        f3[0] = f3[1] = f3[2] = 0.0;
        return LBM_OK;
    }
    /* on the force stream, behind the kernel that wrote the entry: the step
     * stream does not wait for the copy */
    CUDA_TRY(cudaMemcpyAsync(f3, h->force_hist + 3LL * i, 3 * sizeof(double), cudaMemcpyDeviceToHost, h->side));
    return LBM_OK;
}

int lbm_time_stream_collide(lbm_handle* h, int level, int n, float* ms) {
    if (int rc = check_level(h, level)) return rc;
    if (n < 1 || !ms) return fail(LBM_ERR_ARG, "bad argument");
    LevelState& s = h->lv[level];
    StepParams p = base_params(h, level);
    p.t = h->t;
    p.stats_on = 0;
    if (h->cfg.sgs_mlp && !h->mlp_ready) return fail(LBM_ERR_STATE, "SGS mlp: no weights");
    CUDA_TRY(cudaEventRecord(h->ev0, h->stream));
    for (int i = 0; i < n; ++i) {
        if (h->cfg.sgs_mlp)
            CUDA_TRY(launch_stream_collide_mlp(s.L, p, s.f[s.cur], s.f[1 - s.cur], s.mask, nullptr, s.links,
                                               h->mlp_blob, h->mlp_err, h->stream));
        else
            CUDA_TRY(launch_stream_collide(s.L, p, s.f[s.cur], s.f[1 - s.cur], s.mask, nullptr, nullptr, h->stream,
                                           s.links));
        ++h->launches;
        s.cur = 1 - s.cur;
    }
    CUDA_TRY(cudaEventRecord(h->ev1, h->stream));
    CUDA_TRY(cudaEventSynchronize(h->ev1));
    float t = 0;
    CUDA_TRY(cudaEventElapsedTime(&t, h->ev0, h->ev1));
    *ms = t / n;
    return LBM_OK;
}

int lbm_audit(lbm_handle* h, int level, double* out4) {
    if (int rc = check_level(h, level)) return rc;
    if (!out4) return fail(LBM_ERR_ARG, "out4 is null");
    LevelState& s = h->lv[level];
    CUDA_TRY(launch_audit(s.L, s.f[s.cur], s.mask, h->audit_part, audit_partials(s.L), h->audit_out, h->stream));
    h->launches += 2;
    CUDA_TRY(cudaMemcpyAsync(out4, h->audit_out, 4 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    return LBM_OK;
}

int lbm_write_inputs(const lbm_handle* h, char* buf, size_t cap, size_t* len) {
    if (!h) return fail(LBM_ERR_ARG, "null handle");
    std::string s = write_inputs(h->cfg, h->omega, h->omegaLR);
    if (len) *len = s.size();
    if (buf && cap > 0) {
        size_t k = std::min(cap - 1, s.size());
        memcpy(buf, s.data(), k);
        buf[k] = 0;
        if (k < s.size()) return fail(LBM_ERR_ARG, "buffer of %zu bytes too small for %zu", cap, s.size() + 1);
    }
    return LBM_OK;
}

/* tecplot POINT zones in WriteResults' layout (LR7:2350-2442, 2444-2535) */
static void write_level(std::ostream& out, std::ostream* slice, const Config& c, int level, const std::vector<float>& f,
                        const std::vector<float>& st, int nx, int ny, int nz) {
    const size_t N = size_t(nx) * ny * nz;
    out << "VARIABLES = \"X\",\"Y\",\"Z\",\"u\",\"v\",\"w\",\"rho\",\"velAv[0]\",\"velAv[1]\",\"ufluc\",\"vfluc\",\"Smag\"\n";
    out << "ZONE F=POINT, I=" << nx << ", J=" << ny << ", K=" << nz << "\n";
    if (slice) {
        *slice << "VARIABLES = \"X\",\"Y\",\"Z\",\"u\",\"v\",\"w\",\"rho\",\"velAv[0]\",\"velAv[1]\",\"ufluc\",\"vfluc\",\"Smag\"\n";
        *slice << "ZONE F=POINT, I=" << nx << ", J=" << ny << ", K=" << 1 << "\n";
    }
    const int slice_k = level == 0 ? 1 : 3;
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const size_t o = (size_t(k) * ny + j) * nx + i;
                float g[19];
                float rho = 0;
                for (int l = 0; l < 19; ++l) {
                    g[l] = f[l * N + o];
                    rho += g[l];
                }
                float u = g[1] - g[3] + g[5] - g[6] - g[7] + g[8] + g[10] - g[12] + g[15] - g[17];
                float v = g[2] - g[4] + g[5] + g[6] - g[7] - g[8] + g[11] - g[13] + g[16] - g[18];
                float w = g[9] + g[10] + g[11] + g[12] + g[13] - g[14] - g[15] - g[16] - g[17] - g[18];
                float smag = 0.f;
                const bool interior = k > 0 && k < nz - 1;
                if (interior) {
                    /* strain magnitude from the non-equilibrium stress moments
                     * (LR7:2386-2407; divided by LRFACTOR on the fine level) */
                    float m9 = 2.f * g[1] + -g[2] + 2.f * g[3] + -g[4] + g[5] + g[6] + g[7] + g[8] + -g[9] + g[10] +
                               -2.f * g[11] + g[12] + -2.f * g[13] + -g[14] + g[15] + -2.f * g[16] + g[17] + -2.f * g[18];
                    float m11 = g[2] + g[4] + g[5] + g[6] + g[7] + g[8] + -g[9] + -g[10] + -g[12] + -g[14] + -g[15] + -g[17];
                    float m13 = g[5] + -g[6] + g[7] + -g[8];
                    float m14 = g[11] + -g[13] + -g[16] + g[18];
                    float m15 = g[10] + -g[12] + -g[15] + g[17];
                    m9 -= 2.f * u * u - (v * v + w * w);
                    m11 -= v * v - w * w;
                    m13 -= u * v;
                    m14 -= v * w;
                    m15 -= u * w;
                    float P11 = -0.5f * (m9), P22 = -(-38.f * m9 - 3.0f * m11) / 76.f,
                          P33 = -(-38.f * m9 + 3.0f * m11) / 76.f;
                    float P12 = -1.5f * m13, P23 = -1.5f * m14, P13 = -1.5f * m15;
                    smag = std::sqrt(2.f * (P11 * P11 + P22 * P22 + P33 * P33 + 2.f * P12 * P12 + 2.f * P23 * P23 +
                                            2.f * P13 * P13));
                    if (level == 1) smag /= c.lrfactor;
                }
                float s0 = st.empty() ? 0.f : st[o], s1 = st.empty() ? 0.f : st[N + o];
                float s2 = st.empty() ? 0.f : st[2 * N + o], s3 = st.empty() ? 0.f : st[3 * N + o];
                std::ostringstream line;
                if (level == 0) line << i << ", " << j << ", " << k << ", ";
                else
                    line << (c.lrx0 + c.lrfactor * i) << ", " << (c.lry0 + c.lrfactor * j) << ", "
                         << (c.lrz0 + c.lrfactor * k) << ", ";
                line << u << "," << v << "," << w << "," << rho << "," << s0 << "," << s1 << ", " << s2 << "," << s3 << ",";
                if (interior) line << smag;
                else line << 0;
                out << line.str() << std::endl;
                if (slice && k == slice_k) *slice << line.str() << std::endl;
            }
}

/* WriteResults / WriteResultsLR: <base>_part<level>.dat and the slices of
 * every level appended to <base>_slice.dat */
static int write_tecplot_files(lbm_handle* h, const std::string& base) {
    const Config& c = h->cfg;
    std::ofstream slice(base + "_slice.dat");
    if (!slice) return fail(LBM_ERR_ARG, "cannot open '%s_slice.dat'", base.c_str());
    for (int l = 0; l < h->nlevels; ++l) {
        LevelState& s = h->lv[l];
        const size_t N = size_t(s.L.nx) * s.L.ny * s.L.nz;
        std::vector<float> f(N * 19), st;
        if (int rc = lbm_get_populations(h, l, f.data())) return rc;
        if (s.stats) {
            st.resize(4 * N);
            if (int rc = lbm_get_stats(h, l, st.data())) return rc;
        }
        /* WriteResults / WriteResultsLR append their slice to one file */
        std::ofstream part(base + "_part" + std::to_string(l) + ".dat");
        if (!part) return fail(LBM_ERR_ARG, "cannot open '%s_part%d.dat'", base.c_str(), l);
        write_level(part, &slice, c, l, f, st, s.L.nx, s.L.ny, s.L.nz);
        part << std::endl;
    }
    return LBM_OK;
}

int lbm_write_tecplot(lbm_handle* h, const char* casename) {
    if (!h || !casename) return fail(LBM_ERR_ARG, "null argument");
    return write_tecplot_files(h, casename);
}

int lbm_write_outputs(lbm_handle* h, const char* casename) {
    if (!h || !casename) return fail(LBM_ERR_ARG, "null argument");
    const Config& c = h->cfg;
    std::string base(casename);
    std::ofstream dat(base + ".dat"), force(base + ".force"), inputs(base + ".inputs");
    if (!dat || !force || !inputs) return fail(LBM_ERR_ARG, "cannot open output files for '%s'", casename);
    inputs << write_inputs(c, h->omega, h->omegaLR);
    if (int rc = write_tecplot_files(h, base)) return rc;
    const int nf = std::max(0, c.tmax - c.startf);
    std::vector<double> F(size_t(std::max(nf, 1)) * 3, 0.0);
    int got = 0;
    if (int rc = lbm_get_forces(h, F.data(), nf, &got)) return rc;
    force << format_forces(c, F.data(), nf);
    return LBM_OK;
}

int lbm_format_forces(const char* inputs_text, const double* fxyz, int n, char* buf, size_t cap, size_t* len) {
    Config c;
    if (int rc = parse_inputs(inputs_text, c)) return rc;
    if (!fxyz || n < 0) return fail(LBM_ERR_ARG, "bad force history");
    return copy_out(format_forces(c, fxyz, n), buf, cap, len);
}

/* ---- kernel-level API ---- */

static int kernel_level(Level& L, int nx, int ny, int nz, int pitch) {
    const int rc = f32_kernel_level(L, nx, ny, nz, pitch);
    if (rc == 1) return fail(LBM_ERR_ARG, "bad dimensions or pitch");
    if (rc == 2) return fail(LBM_ERR_ARG, "level too large: 19 populations must index below 2^31");
    return LBM_OK;
}

int lbm_stream_collide_f32(const float* fA, float* fB, const uint8_t* mask, int nx, int ny, int nz, int pitch, int model,
                           int les, float omega, float cs, float u_in, float rho_out, int t, void* cuda_stream) {
    if (!fA || !fB || !mask || fA == fB) return fail(LBM_ERR_ARG, "bad buffer pointers");
    if (model < 0 || model > 3) return fail(LBM_ERR_ARG, "model %d unknown", model);
    Level L;
    if (int rc = kernel_level(L, nx, ny, nz, pitch)) return rc;
    StepParams p{};
    p.model = model;
    p.les = les;
    p.omega = omega;
    p.cs = cs;
    p.u_in = u_in;
    p.rho_out = rho_out;
    p.t = t;
    p.stats_weight = 1.f;
    p.dyn_y1 = 1 << 30;
    p.has_lid = 1; /* the caller's mask may hold any node type */
    p.has_xbc = 1;
    CUDA_TRY(launch_stream_collide(L, p, fA, fB, mask, nullptr, nullptr, (cudaStream_t)cuda_stream));
    return LBM_OK;
}

size_t lbm_body_force_scratch_doubles(void) { return size_t(force_scan_partials()) * 3; }

int lbm_body_force_f32(const float* fA, const uint8_t* mask, int nx, int ny, int nz, int pitch, double* force_out,
                       double* scratch, void* cuda_stream) {
    if (!fA || !mask || !force_out || !scratch) return fail(LBM_ERR_ARG, "null device pointer");
    Level L;
    if (int rc = kernel_level(L, nx, ny, nz, pitch)) return rc;
    CUDA_TRY(launch_force_scan(L, fA, mask, scratch, force_out, (cudaStream_t)cuda_stream));
    return LBM_OK;
}

}  // extern "C"
