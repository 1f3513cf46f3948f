// C++ search drivers with the construction and go(f) call shape of tao's
// searches in the reference's driver (test.cxx:82-121):
//
//   ParticleSwarmMPI ps(min_bound, max_bound, arguments);  ps.go(FDTD_GPU);
//   DifferentialEvolutionMPI de(min_bound, max_bound, arguments);  de.go(FDTD_GPU);
//
// become
//
//   tomo::ParticleSwarm ps(min_bound, max_bound, arguments);  ps.go(FDTD_GPU);
//   tomo::DifferentialEvolution de(min_bound, max_bound, arguments);  de.go(batch_fitness);
//   tomo::NewtonMethod anm(min_bound, max_bound, radius, arguments);  anm.iterate(FDTD_GPU);
//
// go() takes either the reference's per-candidate fitness type
// (double (*)(const std::vector<double>&), one call per candidate) or a batch
// fitness that evaluates a whole generation in one call -- e.g. a lambda over
// tomo_fitness_batch, which advances every candidate x excitation solve of the
// generation together on the GPU.  The algorithms run in the library
// (tomo_search_run, include/tomography.h); fitness is maximised.  Arguments are
// tao's "--name value" pairs: --population_size, --maximum_iterations, --seed,
// --inertia, --local_best_weight, --global_best_weight (particle swarm),
// --crossover_rate, --differential_scale, --number_pairs, --parent_selection
// best|random (differential evolution), --regression_size, --line_search_size,
// --line_search_min, --line_search_max, --hessian_diagonal (Newton method).
// Errors throw std::runtime_error
// (std::invalid_argument for bad bounds or arguments).
#ifndef TOMOGRAPHY_SEARCH_HPP
#define TOMOGRAPHY_SEARCH_HPP

#include <cstdint>
#include <exception>
#include <functional>
#include <stdexcept>
#include <string>
#include <vector>

#include "tomography.h"

namespace tomo {

struct SearchResult {
    double best_fitness = 0;
    std::vector<double> best_params;
    std::vector<double> history;   // best fitness after the first and after every later generation
    int64_t evaluations = 0;
};

// fitness[i] of the n candidates population[i * n_param ...]
using BatchFitness = std::function<void(const double* population, size_t n, size_t n_param, double* fitness)>;

class Search {
   public:
    Search(int type, const std::vector<double>& min_bound, const std::vector<double>& max_bound,
           const std::vector<std::string>& arguments)
        : lo_(min_bound), hi_(max_bound) {
        if (lo_.size() != hi_.size() || lo_.empty())
            throw std::invalid_argument("min_bound and max_bound must be non-empty and of equal length");
        if (tomo_search_defaults(&p_, type) != TOMO_OK) throw std::runtime_error(tomo_last_error());
        std::vector<const char*> argv;
        for (const std::string& a : arguments) argv.push_back(a.c_str());
        if (tomo_search_parse_args(&p_, (int)argv.size(), argv.data()) != TOMO_OK)
            throw std::invalid_argument(tomo_last_error());
    }

    tomo_search_params& params() { return p_; }

    // a whole generation per call
    SearchResult go(const BatchFitness& f, const std::function<void(int, double, const double*)>& report = {}) {
        struct Ctx {
            const BatchFitness* f;
            const std::function<void(int, double, const double*)>* report;
            std::exception_ptr error;
        } ctx{&f, &report, nullptr};
        auto batch = [](void* u, const double* pop, size_t n, size_t np, double* fit) -> int {
            Ctx* c = static_cast<Ctx*>(u);
            try {
                (*c->f)(pop, n, np, fit);
                return TOMO_OK;
            } catch (...) {
                c->error = std::current_exception();
                return TOMO_EINVAL;
            }
        };
        auto rep = [](void* u, int gen, double best, const double* params) {
            Ctx* c = static_cast<Ctx*>(u);
            if (*c->report && !c->error) {
                try {
                    (*c->report)(gen, best, params);
                } catch (...) {
                    c->error = std::current_exception();
                }
            }
        };
        SearchResult r;
        r.best_params.resize(lo_.size());
        r.history.resize((size_t)p_.maximum_iterations + 1);
        const int rc = tomo_search_run(&p_, lo_.data(), hi_.data(), lo_.size(), batch, &ctx, rep, &ctx,
                                       r.best_params.data(), &r.best_fitness, r.history.data(), &r.evaluations);
        if (ctx.error) std::rethrow_exception(ctx.error);
        if (rc != TOMO_OK) throw std::runtime_error(tomo_last_error());
        return r;
    }

    // the reference's fitness type: one call per candidate
    SearchResult go(double (*f)(const std::vector<double>&)) {
        return go([f](const double* pop, size_t n, size_t np, double* fit) {
            std::vector<double> v(np);
            for (size_t i = 0; i < n; ++i) {
                v.assign(pop + i * np, pop + (i + 1) * np);
                fit[i] = f(v);
            }
        });
    }

   private:
    tomo_search_params p_{};
    std::vector<double> lo_, hi_;
};

class ParticleSwarm : public Search {
   public:
    ParticleSwarm(const std::vector<double>& min_bound, const std::vector<double>& max_bound,
                  const std::vector<std::string>& arguments = {})
        : Search(TOMO_SEARCH_PS, min_bound, max_bound, arguments) {}
};

class DifferentialEvolution : public Search {
   public:
    DifferentialEvolution(const std::vector<double>& min_bound, const std::vector<double>& max_bound,
                          const std::vector<std::string>& arguments = {})
        : Search(TOMO_SEARCH_DE, min_bound, max_bound, arguments) {}
};

// Regression Newton method with the construction of tao's
// AsynchronousNewtonMethod (min_bound, max_bound, radius, arguments) and its
// iterate(f) (test.cxx:116-121).  Arguments: --maximum_iterations,
// --regression_size, --line_search_size, --line_search_min,
// --line_search_max, --hessian_diagonal, --seed.
class NewtonMethod : public Search {
   public:
    NewtonMethod(const std::vector<double>& min_bound, const std::vector<double>& max_bound,
                 const std::vector<double>& radius, const std::vector<std::string>& arguments = {})
        : Search(TOMO_SEARCH_ANM, min_bound, max_bound, arguments), radius_(radius) {
        if (radius_.size() != min_bound.size())
            throw std::invalid_argument("radius must have one value per parameter");
    }
    SearchResult go(const BatchFitness& f, const std::function<void(int, double, const double*)>& report = {}) {
        params().radius = radius_.data();
        return Search::go(f, report);
    }
    SearchResult go(double (*f)(const std::vector<double>&)) {
        params().radius = radius_.data();
        return Search::go(f);
    }
    SearchResult iterate(const BatchFitness& f) { return go(f); }
    SearchResult iterate(double (*f)(const std::vector<double>&)) { return go(f); }

   private:
    std::vector<double> radius_;
};

}  // namespace tomo

#endif
