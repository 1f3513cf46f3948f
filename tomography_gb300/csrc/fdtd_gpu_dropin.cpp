// C++ drop-in  double FDTD_GPU(const std::vector<double>&)  (FDTD_GPU.cuh:8)
// over the C ABI; see include/tomography_fdtd.hpp for the contract.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/tomography.h"
#include "../../include/tomography_fdtd.hpp"

namespace {

std::mutex g_mu;
tomo_handle* g_handle = nullptr;
bool g_target_set = false;

void throw_status(int rc, const char* what) {
    throw std::runtime_error(std::string(what) + " failed (" + std::to_string(rc) + "): " + tomo_last_error());
}

std::vector<float> read_target_file(const char* path) {
    std::vector<float> v;
    FILE* fp = std::fopen(path, "rb");
    if (!fp) throw std::runtime_error(std::string("cannot open TOMO_MEASUREMENT_FILE ") + path);
    std::fseek(fp, 0, SEEK_END);
    long len = std::ftell(fp);
    std::fseek(fp, 0, SEEK_SET);
    std::vector<unsigned char> raw((size_t)std::max(len, 0L));
    size_t got = std::fread(raw.data(), 1, raw.size(), fp);
    std::fclose(fp);
    raw.resize(got);
    // text when every byte can be part of written numbers (raw float32 data
    // almost surely holds other bytes), else raw little-endian float32
    static const char kTextBytes[] = "0123456789+-.eEinfaINFA \t\r\n,";
    bool text = !raw.empty();
    for (unsigned char c : raw)
        if (c == 0 || !std::strchr(kTextBytes, c)) {
            text = false;
            break;
        }
    if (!text && raw.size() % 4 == 0) {
        v.resize(raw.size() / 4);
        std::memcpy(v.data(), raw.data(), raw.size());
        return v;
    }
    std::string s(raw.begin(), raw.end());
    for (char& c : s) if (c == ',') c = ' ';
    const char* p = s.c_str();
    char* end = nullptr;
    for (;;) {
        float f = std::strtof(p, &end);
        if (end == p) break;
        v.push_back(f);
        p = end;
    }
    return v;
}

tomo_handle* handle_locked() {
    if (g_handle) return g_handle;
    tomo_spec spec;
    int rc = tomo_spec_reference(&spec, 0);
    if (rc) throw_status(rc, "tomo_spec_reference");
    rc = tomo_create(&spec, &g_handle);
    if (rc) throw_status(rc, "tomo_create");
    return g_handle;
}

}  // namespace

double FDTD_GPU(const std::vector<double>& arguments) {
    std::lock_guard<std::mutex> lock(g_mu);
    tomo_handle* h = handle_locked();
    tomo_spec spec;
    tomo_spec_reference(&spec, 0);
    const size_t need = (size_t)tomo_num_params(&spec);
    if (arguments.size() < need) throw std::out_of_range("FDTD_GPU: expected 27 arguments");
    if (!g_target_set) {
        const char* path = std::getenv("TOMO_MEASUREMENT_FILE");
        if (!path) throw std::runtime_error("FDTD_GPU: no target; set TOMO_MEASUREMENT_FILE or call tomo_fdtd_gpu_set_target");
        std::vector<float> t = read_target_file(path);
        // the reference's misfit reads the first E*F*A = 4000 entries of its
        // target array (FDTD_GPU.cu:996-1008, an 8000-entry literal): a longer
        // file is used the same way
        const size_t n_target = (size_t)spec.n_excitations * spec.nfreq * spec.n_angles;
        if (t.size() > n_target) t.resize(n_target);
        int rc = tomo_set_target(h, t.data(), t.size());
        if (rc) throw_status(rc, "tomo_set_target");
        g_target_set = true;
    }
    double fit = 0;
    int rc = tomo_fitness(h, arguments.data(), need, &fit);
    if (rc) throw_status(rc, "tomo_fitness");
    return fit;
}

extern "C" int tomo_fdtd_gpu_set_target(const float* target, size_t n) {
    std::lock_guard<std::mutex> lock(g_mu);
    try {
        tomo_handle* h = handle_locked();
        int rc = tomo_set_target(h, target, n);
        if (rc == TOMO_OK) g_target_set = true;
        return rc;
    } catch (const std::exception&) {
        return TOMO_ECUDA;
    }
}

extern "C" void tomo_fdtd_gpu_release(void) {
    std::lock_guard<std::mutex> lock(g_mu);
    tomo_destroy(g_handle);
    g_handle = nullptr;
    g_target_set = false;
}
