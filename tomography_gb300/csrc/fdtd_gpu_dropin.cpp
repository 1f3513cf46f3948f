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
#include "engine.h"

namespace {

std::mutex g_mu;
tomo_handle* g_handle = nullptr;
bool g_target_set = false;

void throw_status(int rc, const char* what) {
    throw std::runtime_error(std::string(what) + " failed (" + std::to_string(rc) + "): " + tomo_last_error());
}

// Target values of a measurement file: raw little-endian float32, or text
// (numbers separated by spaces, commas or newlines; an optional UTF-8 byte
// order mark).  A NumPy .npy file, or text with anything else in it, is
// rejected rather than read as numbers it does not hold.
int read_target_file(const char* path, std::vector<float>& v, std::string& why) {
    v.clear();
    FILE* fp = std::fopen(path, "rb");
    if (!fp) {
        why = std::string("cannot open ") + path;
        return TOMO_EINVAL;
    }
    std::fseek(fp, 0, SEEK_END);
    long len = std::ftell(fp);
    std::fseek(fp, 0, SEEK_SET);
    std::vector<unsigned char> raw((size_t)std::max(len, 0L));
    size_t got = std::fread(raw.data(), 1, raw.size(), fp);
    std::fclose(fp);
    raw.resize(got);
    static const unsigned char kNpy[6] = {0x93, 'N', 'U', 'M', 'P', 'Y'};
    if (raw.size() >= 6 && std::memcmp(raw.data(), kNpy, 6) == 0) {
        why = std::string(path) + " is a NumPy .npy file; write the values as raw float32 or text";
        return TOMO_EINVAL;
    }
    size_t start = 0;
    if (raw.size() >= 3 && raw[0] == 0xEF && raw[1] == 0xBB && raw[2] == 0xBF) start = 3;   // UTF-8 BOM
    // text when every byte can be part of written numbers (raw float32 data
    // almost surely holds other bytes), else raw little-endian float32
    static const char kTextBytes[] = "0123456789+-.eEinfaINFA \t\r\n,";
    bool text = raw.size() > start;
    for (size_t i = start; i < raw.size(); ++i)
        if (raw[i] == 0 || !std::strchr(kTextBytes, raw[i])) {
            text = false;
            break;
        }
    if (!text && start == 0) {
        if (raw.size() % 4 != 0) {
            why = std::string(path) + " is neither text nor whole float32 values";
            return TOMO_EINVAL;
        }
        v.resize(raw.size() / 4);
        std::memcpy(v.data(), raw.data(), raw.size());
        return TOMO_OK;
    }
    if (!text) {
        why = std::string(path) + " holds characters that are not numbers, spaces, commas or newlines";
        return TOMO_EINVAL;
    }
    std::string s(raw.begin() + start, raw.end());
    for (char& c : s) if (c == ',') c = ' ';
    const char* p = s.c_str();
    for (;;) {
        while (*p == ' ' || *p == '\t' || *p == '\r' || *p == '\n') ++p;
        if (!*p) break;
        char* end = nullptr;
        float f = std::strtof(p, &end);
        if (end == p) {
            why = std::string(path) + ": not a number at byte " + std::to_string(start + (size_t)(p - s.c_str()));
            v.clear();
            return TOMO_EINVAL;
        }
        v.push_back(f);
        p = end;
    }
    return TOMO_OK;
}

// The reference's misfit reads the first E*F*A = 4000 entries of its target
// array (FDTD_GPU.cu:1004-1008), which holds 8000: the magnitudes, then the
// phases (FDTD_GPU.cu:996).  Both lengths are accepted, and only the first
// E*F*A values are used; any other length is an error.
int target_values(const float* t, size_t n, size_t n_target, std::vector<float>& out, std::string& why) {
    if (!t || (n != n_target && n != 2 * n_target)) {
        why = "the target needs " + std::to_string(n_target) + " values (or " + std::to_string(2 * n_target) +
              ": magnitudes then phases), got " + std::to_string(n);
        return TOMO_EINVAL;
    }
    out.assign(t, t + n_target);
    return TOMO_OK;
}

size_t reference_target_size() {
    tomo_spec spec;
    tomo_spec_reference(&spec, 0);
    return (size_t)spec.n_excitations * spec.nfreq * spec.n_angles;
}

// the process-wide handle, created on first use (caller holds g_mu)
int handle_locked(tomo_handle** h) {
    if (!g_handle) {
        tomo_spec spec;
        int rc = tomo_spec_reference(&spec, 0);
        if (rc == TOMO_OK) rc = tomo_create(&spec, &g_handle);
        if (rc) return rc;
    }
    *h = g_handle;
    return TOMO_OK;
}

}  // namespace

double FDTD_GPU(const std::vector<double>& arguments) {
    std::lock_guard<std::mutex> lock(g_mu);
    tomo_handle* h = nullptr;
    if (int rc = handle_locked(&h)) throw_status(rc, "tomo_create");
    tomo_spec spec;
    tomo_spec_reference(&spec, 0);
    const size_t need = (size_t)tomo_num_params(&spec);
    if (arguments.size() < need) throw std::out_of_range("FDTD_GPU: expected 27 arguments");
    if (!g_target_set) {
        const char* path = std::getenv("TOMO_MEASUREMENT_FILE");
        if (!path) throw std::runtime_error("FDTD_GPU: no target; set TOMO_MEASUREMENT_FILE or call tomo_fdtd_gpu_set_target");
        std::vector<float> raw, t;
        std::string why;
        if (read_target_file(path, raw, why) ||
            target_values(raw.data(), raw.size(), reference_target_size(), t, why))
            throw std::runtime_error("FDTD_GPU: TOMO_MEASUREMENT_FILE: " + why);
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
    return tomo::guarded([&]() -> int {
        std::lock_guard<std::mutex> lock(g_mu);
        std::vector<float> t;
        std::string why;
        if (target_values(target, n, reference_target_size(), t, why)) return tomo::fail(TOMO_EINVAL, why);
        tomo_handle* h = nullptr;
        int rc = handle_locked(&h);
        if (rc == TOMO_OK) rc = tomo_set_target(h, t.data(), t.size());
        if (rc == TOMO_OK) g_target_set = true;
        return rc;
    });
}

// Internal test hook (not part of the public ABI): the target the drop-in
// would take from the measurement file `path` (the same parsing and length
// rules as TOMO_MEASUREMENT_FILE), copied into out[0..cap).  Returns the
// number of values, or a negative status with the reason in tomo_last_error().
extern "C" int tomo_internal_read_target_file(const char* path, float* out, size_t cap) {
    return tomo::guarded([&]() -> int {
        std::vector<float> raw, t;
        std::string why;
        if (!path) return tomo::fail(TOMO_EINVAL, "NULL path");
        if (read_target_file(path, raw, why) || target_values(raw.data(), raw.size(), reference_target_size(), t, why))
            return tomo::fail(TOMO_EINVAL, why);
        if (!out || cap < t.size()) return tomo::fail(TOMO_EINVAL, "output buffer too small");
        std::copy(t.begin(), t.end(), out);
        return (int)t.size();
    });
}

extern "C" void tomo_fdtd_gpu_release(void) {
    std::lock_guard<std::mutex> lock(g_mu);
    tomo_destroy(g_handle);
    g_handle = nullptr;
    g_target_set = false;
}
