// Internal engine interface behind the C ABI.
#pragma once
#include <new>
#include <stdexcept>
#include <string>
#include "../../include/tomography.h"

namespace tomo {

class EngineBase {
   public:
    virtual ~EngineBase() = default;
    virtual int set_stream(void* s) = 0;
    virtual int set_budget(uint64_t bytes) = 0;
    virtual int set_target(const float* t, size_t n) = 0;
    virtual int forward(const double* args, size_t ncand, size_t nparam, const tomo_outputs* out) = 0;
    virtual int stats(tomo_stats* st) = 0;
    virtual int submit(const double* args, size_t ncand, size_t nparam, uint64_t* ticket) = 0;
    virtual int submit_spec(const tomo_spec* spec, const double* args, size_t ncand, size_t nparam, uint64_t* ticket) = 0;
    virtual int set_target_spec(const tomo_spec* spec, const float* t, size_t n) = 0;
    virtual int serve_step(int* n_active) = 0;
    virtual int request_bytes(const tomo_spec* spec, size_t ncand, uint64_t* bytes) = 0;
    virtual int poll(uint64_t ticket, double* fitness) = 0;
    virtual int cancel(uint64_t ticket) = 0;
    virtual int snapshot(size_t cand, int exc, int field, float* out, size_t n) = 0;
};

int fail(int code, const std::string& msg);
extern thread_local std::string g_last_error;

// The same as fail() without throwing: for the error paths of guarded().
inline int fail_noexcept(int code, const char* msg) noexcept {
    try {
        g_last_error = msg;
    } catch (...) {
        g_last_error.clear();
    }
    return code;
}

// Body of a C ABI entry point: no C++ exception crosses into a C (or ctypes)
// caller.  A host allocation failure is TOMO_ENOMEM_HOST, any other exception
// TOMO_EINVAL, with the reason in tomo_last_error().
template <class Body>
int guarded(Body&& body) noexcept {
    try {
        return body();
    } catch (const std::bad_alloc&) {
        return fail_noexcept(TOMO_ENOMEM_HOST, "host memory allocation failed");
    } catch (const std::length_error& e) {
        return fail_noexcept(TOMO_ENOMEM_HOST, e.what());
    } catch (const std::exception& e) {
        return fail_noexcept(TOMO_EINVAL, e.what());
    } catch (...) {
        return fail_noexcept(TOMO_EINVAL, "unexpected exception");
    }
}

int spec_reference(tomo_spec* s, int cpu_variant);
int spec_breast(tomo_spec* s, int config);
int spec_serving(tomo_spec* s, int edge, int n_antennas);
int num_params(const tomo_spec* s);
int num_excitations(const tomo_spec* s);
int create_engine(const tomo_spec* spec, EngineBase** out);

}  // namespace tomo
