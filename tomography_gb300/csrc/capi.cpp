// C ABI entry points (include/tomography.h) over the engine.
#include <chrono>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/tomography.h"
#include "engine.h"

struct tomo_handle {
    tomo::EngineBase* eng = nullptr;
    tomo_spec spec{};
};

using tomo::fail;

extern "C" {

int tomo_spec_reference(tomo_spec* spec, int cpu_variant) {
    return tomo::guarded([&]() -> int {
        return tomo::spec_reference(spec, cpu_variant);
    });
}
int tomo_spec_breast(tomo_spec* spec, int config) {
    return tomo::guarded([&]() -> int {
        return tomo::spec_breast(spec, config);
    });
}
int tomo_spec_serving(tomo_spec* spec, int edge, int n_antennas) {
    return tomo::guarded([&]() -> int {
        return tomo::spec_serving(spec, edge, n_antennas);
    });
}
int tomo_num_params(const tomo_spec* spec) { return tomo::num_params(spec); }
int tomo_num_excitations(const tomo_spec* spec) { return tomo::num_excitations(spec); }

int tomo_create(const tomo_spec* spec, tomo_handle** out) {
    return tomo::guarded([&]() -> int {
        if (!spec || !out) return fail(TOMO_EINVAL, "tomo_create: NULL argument");
        *out = nullptr;
        tomo::EngineBase* e = nullptr;
        int rc = tomo::create_engine(spec, &e);
        if (rc) return rc;
        tomo_handle* h = new (std::nothrow) tomo_handle;
        if (!h) {
            delete e;
            return fail(TOMO_ENOMEM_HOST, "host memory allocation failed");
        }
        h->eng = e;
        h->spec = *spec;
        *out = h;
        return TOMO_OK;
    });
}

void tomo_destroy(tomo_handle* h) {
    if (!h) return;
    delete h->eng;
    delete h;
}

int tomo_set_stream(tomo_handle* h, void* stream) {
    return tomo::guarded([&]() -> int {
        if (!h) return fail(TOMO_EINVAL, "NULL handle");
        return h->eng->set_stream(stream);
    });
}

int tomo_set_memory_budget(tomo_handle* h, uint64_t bytes) {
    return tomo::guarded([&]() -> int {
        if (!h) return fail(TOMO_EINVAL, "NULL handle");
        return h->eng->set_budget(bytes);
    });
}

int tomo_set_target(tomo_handle* h, const float* target, size_t n) {
    return tomo::guarded([&]() -> int {
        if (!h) return fail(TOMO_EINVAL, "NULL handle");
        return h->eng->set_target(target, n);
    });
}

int tomo_fitness(tomo_handle* h, const double* args, size_t n_args, double* fitness) {
    return tomo::guarded([&]() -> int {
        if (!h || !args || !fitness) return fail(TOMO_EINVAL, "tomo_fitness: NULL argument");
        tomo_outputs o{};
        o.fitness = fitness;
        return h->eng->forward(args, 1, n_args, &o);
    });
}

int tomo_fitness_batch(tomo_handle* h, const double* args, size_t n_cand, size_t n_param, double* fitness) {
    return tomo::guarded([&]() -> int {
        if (!h || !args || !fitness) return fail(TOMO_EINVAL, "tomo_fitness_batch: NULL argument");
        tomo_outputs o{};
        o.fitness = fitness;
        return h->eng->forward(args, n_cand, n_param, &o);
    });
}

int tomo_forward(tomo_handle* h, const double* args, size_t n_cand, size_t n_param, const tomo_outputs* out) {
    return tomo::guarded([&]() -> int {
        if (!h || !args) return fail(TOMO_EINVAL, "tomo_forward: NULL argument");
        tomo_outputs none{};
        return h->eng->forward(args, n_cand, n_param, out ? out : &none);
    });
}

int tomo_submit(tomo_handle* h, const double* args, size_t n_cand, size_t n_param, uint64_t* ticket) {
    return tomo::guarded([&]() -> int {
        if (!h || !args || !ticket) return fail(TOMO_EINVAL, "tomo_submit: NULL argument");
        return h->eng->submit(args, n_cand, n_param, ticket);
    });
}

int tomo_submit_spec(tomo_handle* h, const tomo_spec* spec, const double* args, size_t n_cand, size_t n_param,
                     uint64_t* ticket) {
    return tomo::guarded([&]() -> int {
        if (!h || !args || !ticket) return fail(TOMO_EINVAL, "tomo_submit_spec: NULL argument");
        return h->eng->submit_spec(spec, args, n_cand, n_param, ticket);
    });
}

int tomo_set_target_spec(tomo_handle* h, const tomo_spec* spec, const float* target, size_t n) {
    return tomo::guarded([&]() -> int {
        if (!h) return fail(TOMO_EINVAL, "NULL handle");
        return h->eng->set_target_spec(spec, target, n);
    });
}

int tomo_serve_step(tomo_handle* h, int* n_active) {
    return tomo::guarded([&]() -> int {
        if (!h) return fail(TOMO_EINVAL, "NULL handle");
        return h->eng->serve_step(n_active);
    });
}

int tomo_request_bytes(tomo_handle* h, const tomo_spec* spec, size_t n_cand, uint64_t* bytes) {
    return tomo::guarded([&]() -> int {
        if (!h || !bytes) return fail(TOMO_EINVAL, "tomo_request_bytes: NULL argument");
        return h->eng->request_bytes(spec, n_cand, bytes);
    });
}

int tomo_poll(tomo_handle* h, uint64_t ticket, double* fitness) {
    return tomo::guarded([&]() -> int {
        if (!h) return fail(TOMO_EINVAL, "NULL handle");
        return h->eng->poll(ticket, fitness);
    });
}

int tomo_wait(tomo_handle* h, uint64_t ticket, double timeout_ms, double* fitness) {
    return tomo::guarded([&]() -> int {
        if (!h) return fail(TOMO_EINVAL, "NULL handle");
        if (!(timeout_ms >= 0)) return fail(TOMO_EINVAL, "tomo_wait: timeout must be >= 0");
        const auto t0 = std::chrono::steady_clock::now();
        for (;;) {
            const int rc = h->eng->poll(ticket, fitness);
            if (rc != TOMO_ENOTREADY) return rc;
            const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
            if (ms >= timeout_ms)
                return fail(TOMO_ETIMEOUT, "ticket " + std::to_string(ticket) + " not finished after " +
                                               std::to_string(ms) + " ms");
            int active = 0;
            const int st = h->eng->serve_step(&active);
            if (st != TOMO_OK) return st;
        }
    });
}

// tomo_search_fitness: the search drivers of search.cpp with the handle's
// batch fitness (tomo_fitness_batch) as the generation evaluator.  A candidate
// whose solve diverges has a non-finite fitness (TOMO_ENUMERIC, every fitness
// written); the drivers rank it below every number and the search goes on, as
// the reference's search goes on past its clamped fields.
static int handle_fitness(void* user, const double* pop, size_t n, size_t np, double* fit) {
    const int rc = tomo_fitness_batch(static_cast<tomo_handle*>(user), pop, n, np, fit);
    return rc == TOMO_ENUMERIC ? TOMO_OK : rc;
}

int tomo_search_fitness(tomo_handle* h, const tomo_search_params* p, const double* min_bound,
                        const double* max_bound, tomo_generation_fn report, void* report_user, double* best_params,
                        double* best_fitness, double* history) {
    return tomo::guarded([&]() -> int {
        if (!h) return fail(TOMO_EINVAL, "NULL handle");
        const int np = tomo::num_params(&h->spec);
        if (np < 1) return fail(TOMO_EINVAL, "spec has no parameters");
        return tomo_search_run(p, min_bound, max_bound, (size_t)np, handle_fitness, h, report, report_user, best_params,
                               best_fitness, history, nullptr);
    });
}

int tomo_cancel(tomo_handle* h, uint64_t ticket) {
    return tomo::guarded([&]() -> int {
        if (!h) return fail(TOMO_EINVAL, "NULL handle");
        return h->eng->cancel(ticket);
    });
}

int tomo_get_stats(tomo_handle* h, tomo_stats* stats) {
    return tomo::guarded([&]() -> int {
        if (!h) return fail(TOMO_EINVAL, "NULL handle");
        return h->eng->stats(stats);
    });
}

int tomo_field_snapshot(tomo_handle* h, size_t candidate, int excitation, int field, float* out, size_t n) {
    return tomo::guarded([&]() -> int {
        if (!h) return fail(TOMO_EINVAL, "NULL handle");
        return h->eng->snapshot(candidate, excitation, field, out, n);
    });
}

const char* tomo_last_error(void) { return tomo::g_last_error.c_str(); }
const char* tomo_version(void) { return "tomography_gb300 0.1"; }

}  // extern "C"
