/*
 * lbm_run -- the reference programs' main() (LRTurbTest/LRMultiGPU7.cu:
 * 2575-3029) as a command over the C ABI:
 *
 *   lbm_run CASE.inputs [--out CASENAME] [--steps N]
 *
 * reads the run record the reference writes (WriteInputs, LR7:2547-2573),
 * runs TMAX steps (or N), prints the reference's timing line
 * ("Time taken for main kernel: <s> (<MLUPS>MLUPS)", LR7:2953-2961, fine
 * nodes counted LRLEVEL times) and writes CASENAME.inputs,
 * CASENAME_part0.dat (and _part1.dat with refinement), CASENAME_slice.dat
 * and CASENAME.force as the reference does (LR7:2963-3027).  CASENAME
 * defaults to the record's file name without its extension.
 */
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>

#include "../../include/lbm_gb300.h"

namespace {

/* the value of a record line "label<TAB>[: ]value" whose label, without a
 * trailing colon and spaces, is key */
std::string record_value(const std::string& text, const std::string& key) {
    std::istringstream in(text);
    std::string line;
    while (std::getline(in, line)) {
        const size_t tab = line.find('\t');
        if (tab == std::string::npos) continue;
        std::string label = line.substr(0, tab);
        while (!label.empty() && (label.back() == ' ' || label.back() == ':')) label.pop_back();
        if (label != key) continue;
        std::string val = line.substr(tab + 1);
        size_t a = val.find_first_not_of(" :\t\r");
        return a == std::string::npos ? std::string() : val.substr(a);
    }
    return std::string();
}

int usage() {
    std::fprintf(stderr, "usage: lbm_run CASE.inputs [--out CASENAME] [--steps N]\n");
    return 2;
}

int fail(const char* what) {
    std::fprintf(stderr, "lbm_run: %s: %s\n", what, lbm_last_error());
    return 1;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 2) return usage();
    std::string path = argv[1], casename;
    long steps = -1;
    for (int i = 2; i < argc; ++i) {
        if (!std::strcmp(argv[i], "--out") && i + 1 < argc) casename = argv[++i];
        else if (!std::strcmp(argv[i], "--steps") && i + 1 < argc) steps = std::atol(argv[++i]);
        else return usage();
    }
    std::ifstream f(path, std::ios::binary);
    if (!f) {
        std::fprintf(stderr, "lbm_run: cannot read %s\n", path.c_str());
        return 1;
    }
    std::stringstream ss;
    ss << f.rdbuf();
    const std::string text = ss.str();
    if (casename.empty()) {
        const size_t slash = path.find_last_of('/');
        casename = path.substr(slash == std::string::npos ? 0 : slash + 1);
        const size_t dot = casename.rfind('.');
        if (dot != std::string::npos && dot > 0) casename.erase(dot);
    }
    if (steps < 0) steps = std::atol(record_value(text, "TMAX").c_str());
    if (steps < 0) return usage();

    lbm_handle* h = nullptr;
    if (lbm_create(text.c_str(), &h)) return fail("create");
    int nlev = 1;
    lbm_get_nlevels(h, &nlev);
    double nodes = 0;
    for (int l = 0; l < nlev; ++l) {
        int nx = 0, ny = 0, nz = 0;
        lbm_get_dims(h, l, &nx, &ny, &nz);
        /* the fine patch updates LRLEVEL times per step (LR7:2959) */
        const double lrf = std::atof(record_value(text, "LR factor").c_str());
        const double factor = l == 0 || lrf <= 0 ? 1.0 : double(std::lround(1.0 / lrf));
        nodes += double(nx) * ny * nz * factor;
    }
    /* the loop in chunks, timed on the device */
    double ms_total = 0;
    for (long done = 0; done < steps;) {
        const int n = int(std::min<long>(steps - done, 1000));
        float ms = 0;
        if (lbm_step_timed(h, n, &ms)) {
            lbm_destroy(h);
            return fail("step");
        }
        ms_total += ms;
        done += n;
    }
    const double sec = ms_total * 1e-3;
    std::printf("Time taken for main kernel: %g (%gMLUPS)\n", sec, sec > 0 ? nodes * steps / 1e6 / sec : 0.0);
    if (lbm_write_outputs(h, casename.c_str())) {
        lbm_destroy(h);
        return fail("write outputs");
    }
    lbm_destroy(h);
    return 0;
}
