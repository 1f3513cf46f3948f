// Synchronous search drivers over whole generations: global-best particle
// swarm, differential evolution (DE/{best,random}/k/bin) and a regression
// Newton method.
//
// They take the place of tao's ParticleSwarmMPI / DifferentialEvolutionMPI /
// AsynchronousNewtonMethod in the reference's driver (test.cxx:82-121:
// `ps(min_bound, max_bound, arguments); ps.go(FDTD_GPU)`, `anm(min_bound,
// max_bound, radius, arguments); anm.iterate(FDTD_GPU)`).  tao farms one candidate per MPI rank and
// call; here a generation is ONE call of a batch fitness function, so every
// candidate x excitation solve of the generation advances together on the GPU
// (tomo_fitness_batch).  tao is an un-vendored submodule: the algorithms are
// the textbook synchronous forms with tao's parameter names
// (--population_size, --maximum_iterations, --inertia, --local_best_weight,
// --global_best_weight, --crossover_rate, --differential_scale,
// --number_pairs, --parent_selection, --seed; the Newton method's
// --regression_size, --line_search_size, --line_search_min,
// --line_search_max and --hessian_diagonal are this implementation's).  Fitness is maximised (the
// reference's fitness is a negative misfit).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#include "../../include/tomography.h"
#include "engine.h"

namespace {

using tomo::fail;

// xoshiro256** seeded through splitmix64 (public-domain generators by Blackman
// and Vigna): uniform doubles with 53 random bits.
struct Rng {
    uint64_t s[4];
    explicit Rng(uint64_t seed) {
        for (auto& w : s) {
            seed += 0x9e3779b97f4a7c15ULL;
            uint64_t z = seed;
            z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
            z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
            w = z ^ (z >> 31);
        }
    }
    static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    uint64_t next() {
        const uint64_t r = rotl(s[1] * 5, 7) * 9, t = s[1] << 17;
        s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl(s[3], 45);
        return r;
    }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
    // integer in [0, n)
    size_t below(size_t n) { return (size_t)(uniform() * (double)n) % n; }
};

struct Run {
    const tomo_search_params& p;
    const double* lo;
    const double* hi;
    size_t np;
    tomo_batch_fitness_fn f;
    void* user;
    tomo_generation_fn report;
    void* report_user;
    int64_t evals = 0;

    // a NaN fitness (a diverged or failed candidate) ranks below every number,
    // so that no comparison of the drivers can keep or prefer it
    int evaluate(const std::vector<double>& x, size_t n, std::vector<double>& fx) {
        fx.assign(n, 0.0);
        const int rc = f(user, x.data(), n, np, fx.data());
        if (rc != TOMO_OK) return rc;
        for (double& v : fx)
            if (std::isnan(v)) v = -HUGE_VAL;
        evals += (int64_t)n;
        return TOMO_OK;
    }
    double clip(size_t j, double v) const { return v < lo[j] ? lo[j] : (v > hi[j] ? hi[j] : v); }
};

size_t argmax(const std::vector<double>& v) {
    size_t b = 0;
    for (size_t i = 1; i < v.size(); ++i)
        if (v[i] > v[b]) b = i;
    return b;
}

int particle_swarm(Run& R, Rng& g, double* best_params, double* best_fitness, double* history) {
    const size_t n = (size_t)R.p.population_size, P = R.np;
    std::vector<double> x(n * P), v(n * P), fx, pbest, pfit, gbest(P);
    for (size_t i = 0; i < n; ++i)
        for (size_t j = 0; j < P; ++j) {
            const double span = R.hi[j] - R.lo[j];
            x[i * P + j] = R.lo[j] + g.uniform() * span;
            v[i * P + j] = (g.uniform() * 2.0 - 1.0) * span * 0.1;
        }
    if (int rc = R.evaluate(x, n, fx)) return rc;
    pbest = x;
    pfit = fx;
    size_t b = argmax(pfit);
    std::memcpy(gbest.data(), &pbest[b * P], sizeof(double) * P);
    double gfit = pfit[b];
    if (history) history[0] = gfit;
    for (int it = 0; it < R.p.maximum_iterations; ++it) {
        // v <- w v + c1 r1 (p_best - x) + c2 r2 (g_best - x);  x <- clip(x + v)
        for (size_t i = 0; i < n; ++i)
            for (size_t j = 0; j < P; ++j) {
                const size_t k = i * P + j;
                const double r1 = g.uniform(), r2 = g.uniform();
                v[k] = R.p.inertia * v[k] + R.p.local_best_weight * r1 * (pbest[k] - x[k]) +
                       R.p.global_best_weight * r2 * (gbest[j] - x[k]);
                x[k] = R.clip(j, x[k] + v[k]);
            }
        if (int rc = R.evaluate(x, n, fx)) return rc;
        for (size_t i = 0; i < n; ++i)
            if (fx[i] > pfit[i]) {
                pfit[i] = fx[i];
                std::memcpy(&pbest[i * P], &x[i * P], sizeof(double) * P);
            }
        b = argmax(pfit);
        if (pfit[b] > gfit) {
            gfit = pfit[b];
            std::memcpy(gbest.data(), &pbest[b * P], sizeof(double) * P);
        }
        if (history) history[it + 1] = gfit;
        if (R.report) R.report(R.report_user, it, gfit, gbest.data());
    }
    std::memcpy(best_params, gbest.data(), sizeof(double) * P);
    *best_fitness = gfit;
    return TOMO_OK;
}

int differential_evolution(Run& R, Rng& g, double* best_params, double* best_fitness, double* history) {
    const size_t n = (size_t)R.p.population_size, P = R.np;
    const size_t pairs = (size_t)R.p.number_pairs;
    std::vector<double> x(n * P), trial(n * P), fx, ft, donor(P);
    std::vector<size_t> others(n - 1);
    for (size_t i = 0; i < n; ++i)
        for (size_t j = 0; j < P; ++j) x[i * P + j] = R.lo[j] + g.uniform() * (R.hi[j] - R.lo[j]);
    if (int rc = R.evaluate(x, n, fx)) return rc;
    if (history) history[0] = fx[argmax(fx)];
    for (int it = 0; it < R.p.maximum_iterations; ++it) {
        const size_t best = argmax(fx);
        for (size_t i = 0; i < n; ++i) {
            // 2 * pairs distinct members other than i (partial Fisher-Yates)
            for (size_t a = 0, k = 0; a < n; ++a)
                if (a != i) others[k++] = a;
            for (size_t k = 0; k < 2 * pairs; ++k) std::swap(others[k], others[k + g.below(n - 1 - k)]);
            const size_t base = R.p.parent_best ? best : others[2 * pairs + g.below(n - 1 - 2 * pairs)];
            for (size_t j = 0; j < P; ++j) {
                double d = x[base * P + j];
                for (size_t k = 0; k < pairs; ++k)
                    d += R.p.differential_scale * (x[others[2 * k] * P + j] - x[others[2 * k + 1] * P + j]);
                donor[j] = d;
            }
            // binomial crossover with at least one donor gene
            const size_t forced = g.below(P);
            for (size_t j = 0; j < P; ++j) {
                const bool take = g.uniform() < R.p.crossover_rate || j == forced;
                trial[i * P + j] = R.clip(j, take ? donor[j] : x[i * P + j]);
            }
        }
        if (int rc = R.evaluate(trial, n, ft)) return rc;
        for (size_t i = 0; i < n; ++i)
            if (ft[i] >= fx[i]) {   // the trial replaces its target when it is not worse
                fx[i] = ft[i];
                std::memcpy(&x[i * P], &trial[i * P], sizeof(double) * P);
            }
        const size_t b = argmax(fx);
        if (history) history[it + 1] = fx[b];
        if (R.report) R.report(R.report_user, it, fx[b], &x[b * P]);
    }
    const size_t b = argmax(fx);
    std::memcpy(best_params, &x[b * P], sizeof(double) * P);
    *best_fitness = fx[b];
    return TOMO_OK;
}

// Solve A x = b (n x n, row-major, overwritten) by Gaussian elimination with
// partial pivoting; false when A is singular to working precision.
bool solve_dense(std::vector<double>& A, std::vector<double>& b, size_t n) {
    double scale = 0;
    for (double v : A) scale = std::max(scale, std::fabs(v));
    if (!(scale > 0)) return false;
    for (size_t c = 0; c < n; ++c) {
        size_t piv = c;
        for (size_t r = c + 1; r < n; ++r)
            if (std::fabs(A[r * n + c]) > std::fabs(A[piv * n + c])) piv = r;
        if (!(std::fabs(A[piv * n + c]) > 1e-13 * scale)) return false;
        if (piv != c) {
            for (size_t k = 0; k < n; ++k) std::swap(A[c * n + k], A[piv * n + k]);
            std::swap(b[c], b[piv]);
        }
        for (size_t r = c + 1; r < n; ++r) {
            const double f = A[r * n + c] / A[c * n + c];
            if (f == 0) continue;
            for (size_t k = c; k < n; ++k) A[r * n + k] -= f * A[c * n + k];
            b[r] -= f * b[c];
        }
    }
    for (size_t c = n; c-- > 0;) {
        double v = b[c];
        for (size_t k = c + 1; k < n; ++k) v -= A[c * n + k] * b[k];
        b[c] = v / A[c * n + c];
    }
    return true;
}

// Regression Newton method (the synchronous form of a Newton search driven by
// sampled fitness values).  The free parameters are those with max > min; the
// model is in scaled offsets z = (x - c) / radius from the best point c:
//   f ~ b0 + g.z + sum_a h_aa z_a^2 / 2 + sum_{a<b} h_ab z_a z_b   (full)
//   f ~ b0 + g.z + sum_a h_aa z_a^2 / 2                           (diagonal),
// fitted by least squares (normal equations with a small ridge).  The Newton
// step solves H s = -g (gradient step if H is singular); the line search
// evaluates c + a s for a evenly spaced in [line_search_min, line_search_max]
// (both directions, so a saddle of the model is not followed blindly).  The
// best point seen becomes the next centre.
int newton_method(Run& R, Rng& g, double* best_params, double* best_fitness, double* history) {
    const size_t P = R.np;
    std::vector<size_t> act;
    for (size_t j = 0; j < P; ++j)
        if (R.hi[j] > R.lo[j]) act.push_back(j);
    const size_t k = act.size();
    const bool diag = R.p.hessian_diagonal != 0;
    const size_t nq = diag ? k : k * (k + 1) / 2, nu = 1 + k + nq;
    // the normal equations hold nu^2 doubles and take O(nu^3) to solve
    constexpr size_t kMaxModelTerms = 8192;
    if (nu > kMaxModelTerms)
        return fail(TOMO_EINVAL, "the quadratic model of " + std::to_string(k) + " free parameters has " +
                                     std::to_string(nu) + " terms (at most " + std::to_string(kMaxModelTerms) +
                                     "); use --hessian_diagonal 1");
    const size_t m = R.p.regression_size > 0 ? (size_t)R.p.regression_size : std::max<size_t>(2 * nu, nu + 4);
    const size_t L = (size_t)R.p.line_search_size;
    std::vector<double> rad(P);
    for (size_t j = 0; j < P; ++j) rad[j] = R.p.radius ? std::fabs(R.p.radius[j]) : 0.1 * (R.hi[j] - R.lo[j]);
    for (size_t a = 0; a < k; ++a)
        if (!(rad[act[a]] > 0)) return fail(TOMO_EINVAL, "radius must be positive for every free parameter");
    // start: the midpoint of the bounds
    std::vector<double> c(P), fx;
    for (size_t j = 0; j < P; ++j) c[j] = 0.5 * (R.lo[j] + R.hi[j]);
    if (int rc = R.evaluate(c, 1, fx)) return rc;
    double fc = fx[0];
    if (history) history[0] = fc;
    std::vector<double> X(m * P), Y(L * P), z(k), phi(nu), A(nu * nu), rhs(nu), H(k * k), step(k);
    for (int it = 0; it < R.p.maximum_iterations; ++it) {
        // 1. regression sample around c
        for (size_t i = 0; i < m; ++i)
            for (size_t j = 0; j < P; ++j)
                X[i * P + j] = R.clip(j, c[j] + (R.hi[j] > R.lo[j] ? rad[j] * (2.0 * g.uniform() - 1.0) : 0.0));
        if (int rc = R.evaluate(X, m, fx)) return rc;
        // 2. least-squares quadratic model in z
        std::fill(A.begin(), A.end(), 0.0);
        std::fill(rhs.begin(), rhs.end(), 0.0);
        for (size_t i = 0; i < m; ++i) {
            if (!std::isfinite(fx[i])) continue;
            for (size_t a = 0; a < k; ++a) z[a] = (X[i * P + act[a]] - c[act[a]]) / rad[act[a]];
            size_t q = 0;
            phi[q++] = 1.0;
            for (size_t a = 0; a < k; ++a) phi[q++] = z[a];
            for (size_t a = 0; a < k; ++a) {
                if (diag) phi[q++] = 0.5 * z[a] * z[a];
                else
                    for (size_t b = a; b < k; ++b) phi[q++] = (a == b ? 0.5 : 1.0) * z[a] * z[b];
            }
            for (size_t u = 0; u < nu; ++u) {   // the upper triangle; mirrored below
                rhs[u] += phi[u] * fx[i];
                const double pu = phi[u];
                double* row = &A[u * nu];
                for (size_t v = u; v < nu; ++v) row[v] += pu * phi[v];
            }
        }
        for (size_t u = 0; u < nu; ++u)
            for (size_t v = 0; v < u; ++v) A[u * nu + v] = A[v * nu + u];
        double tr = 0;
        for (size_t u = 0; u < nu; ++u) tr += A[u * nu + u];
        for (size_t u = 0; u < nu; ++u) A[u * nu + u] += 1e-12 * tr / (double)nu;
        bool have = k > 0 && solve_dense(A, rhs, nu);
        // 3. Newton step (gradient step when the model's Hessian is singular)
        if (have) {
            std::fill(H.begin(), H.end(), 0.0);
            size_t q = 1 + k;
            for (size_t a = 0; a < k; ++a) {
                if (diag) H[a * k + a] = rhs[q++];
                else
                    for (size_t b = a; b < k; ++b) H[a * k + b] = H[b * k + a] = rhs[q++];
            }
            for (size_t a = 0; a < k; ++a) step[a] = -rhs[1 + a];
            std::vector<double> Hc = H;
            if (!solve_dense(Hc, step, k))
                for (size_t a = 0; a < k; ++a) step[a] = rhs[1 + a];
        }
        // 4. line search along the step (in parameter units)
        if (have)
            for (size_t l = 0; l < L; ++l) {
                const double al = R.p.line_search_min +
                                  (R.p.line_search_max - R.p.line_search_min) * (double)l / (double)(L - 1);
                for (size_t j = 0; j < P; ++j) Y[l * P + j] = c[j];
                for (size_t a = 0; a < k; ++a)
                    Y[l * P + act[a]] = R.clip(act[a], c[act[a]] + al * step[a] * rad[act[a]]);
            }
        std::vector<double> fy;
        if (have)
            if (int rc = R.evaluate(Y, L, fy)) return rc;
        // 5. the best point seen becomes the centre
        for (size_t i = 0; i < m; ++i)
            if (fx[i] > fc) { fc = fx[i]; std::memcpy(c.data(), &X[i * P], sizeof(double) * P); }
        for (size_t l = 0; l < fy.size(); ++l)
            if (fy[l] > fc) { fc = fy[l]; std::memcpy(c.data(), &Y[l * P], sizeof(double) * P); }
        if (history) history[it + 1] = fc;
        if (R.report) R.report(R.report_user, it, fc, c.data());
    }
    std::memcpy(best_params, c.data(), sizeof(double) * P);
    *best_fitness = fc;
    return TOMO_OK;
}

}  // namespace

extern "C" {

int tomo_search_defaults(tomo_search_params* p, int type) {
    return tomo::guarded([&]() -> int {
        if (!p) return fail(TOMO_EINVAL, "tomo_search_defaults: NULL params");
        if (type != TOMO_SEARCH_PS && type != TOMO_SEARCH_DE && type != TOMO_SEARCH_ANM)
            return fail(TOMO_EINVAL, "unknown search type");
        std::memset(p, 0, sizeof(*p));
        p->type = type;
        p->population_size = 50;
        p->maximum_iterations = 100;
        p->seed = 0x70F00001ULL;
        p->inertia = 0.75;
        p->local_best_weight = 1.5;
        p->global_best_weight = 1.5;
        p->crossover_rate = 0.5;
        p->differential_scale = 0.5;
        p->number_pairs = 1;
        p->parent_best = 1;
        p->radius = nullptr;
        p->regression_size = 0;
        p->line_search_size = 13;   // a step of 0.25 over [-1, 2]: the full Newton step a = 1 is one of them
        p->line_search_min = -1.0;
        p->line_search_max = 2.0;
        p->hessian_diagonal = 0;
        if (type == TOMO_SEARCH_ANM) p->maximum_iterations = 10;
        return TOMO_OK;
    });
}

int tomo_search_parse_args(tomo_search_params* p, int argc, const char* const* argv) {
    return tomo::guarded([&]() -> int {
        if (!p || argc < 0 || (argc > 0 && !argv)) return fail(TOMO_EINVAL, "tomo_search_parse_args: NULL argument");
        for (int i = 0; i + 1 < argc; ++i) {
            const std::string a = argv[i] ? argv[i] : "";
            const char* v = argv[i + 1];
            if (!v) continue;
            char* end = nullptr;
            if (a == "--population_size") p->population_size = (int32_t)std::strtol(v, &end, 10);
            else if (a == "--maximum_iterations") p->maximum_iterations = (int32_t)std::strtol(v, &end, 10);
            else if (a == "--seed") p->seed = (uint64_t)std::strtoull(v, &end, 0);
            else if (a == "--inertia") p->inertia = std::strtod(v, &end);
            else if (a == "--local_best_weight") p->local_best_weight = std::strtod(v, &end);
            else if (a == "--global_best_weight") p->global_best_weight = std::strtod(v, &end);
            else if (a == "--crossover_rate") p->crossover_rate = std::strtod(v, &end);
            else if (a == "--differential_scale") p->differential_scale = std::strtod(v, &end);
            else if (a == "--number_pairs") p->number_pairs = (int32_t)std::strtol(v, &end, 10);
            else if (a == "--regression_size") p->regression_size = (int32_t)std::strtol(v, &end, 10);
            else if (a == "--line_search_size") p->line_search_size = (int32_t)std::strtol(v, &end, 10);
            else if (a == "--line_search_min") p->line_search_min = std::strtod(v, &end);
            else if (a == "--line_search_max") p->line_search_max = std::strtod(v, &end);
            else if (a == "--hessian_diagonal") p->hessian_diagonal = (int32_t)std::strtol(v, &end, 10);
            else if (a == "--parent_selection") {
                const std::string s = v;
                if (s != "best" && s != "random") return fail(TOMO_EINVAL, "--parent_selection must be best or random");
                p->parent_best = s == "best";
                continue;
            } else continue;
            if (!end || *end != '\0') return fail(TOMO_EINVAL, "bad value for " + a + ": " + v);
        }
        return TOMO_OK;
    });
}

int tomo_search_run(const tomo_search_params* p, const double* min_bound, const double* max_bound, size_t n_param,
                    tomo_batch_fitness_fn f, void* user, tomo_generation_fn report, void* report_user,
                    double* best_params, double* best_fitness, double* history, int64_t* evaluations) {
    return tomo::guarded([&]() -> int {
        if (!p || !min_bound || !max_bound || !f || !best_params || !best_fitness)
            return fail(TOMO_EINVAL, "tomo_search_run: NULL argument");
        if (p->type != TOMO_SEARCH_PS && p->type != TOMO_SEARCH_DE && p->type != TOMO_SEARCH_ANM)
            return fail(TOMO_EINVAL, "unknown search type");
        if (n_param < 1) return fail(TOMO_EINVAL, "no parameters");
        for (size_t j = 0; j < n_param; ++j)
            if (!std::isfinite(min_bound[j]) || !std::isfinite(max_bound[j]) || max_bound[j] < min_bound[j])
                return fail(TOMO_EINVAL, "bounds must be finite with min <= max");
        if (p->type != TOMO_SEARCH_ANM && p->population_size < 4)
            return fail(TOMO_EINVAL, "population_size must be at least 4");
        if (p->type == TOMO_SEARCH_ANM &&
            (p->line_search_size < 2 || p->regression_size < 0 || !(p->line_search_max > p->line_search_min)))
            return fail(TOMO_EINVAL, "line_search_size must be >= 2 and line_search_max above line_search_min");
        if (p->maximum_iterations < 0) return fail(TOMO_EINVAL, "maximum_iterations must be >= 0");
        if (p->type == TOMO_SEARCH_DE && (p->number_pairs < 1 || p->population_size < 2 * p->number_pairs + 2))
            return fail(TOMO_EINVAL, "population too small for the number of difference pairs");
        Run R{*p, min_bound, max_bound, n_param, f, user, report, report_user};
        Rng g(p->seed);
        const int rc = p->type == TOMO_SEARCH_PS   ? particle_swarm(R, g, best_params, best_fitness, history)
                       : p->type == TOMO_SEARCH_DE ? differential_evolution(R, g, best_params, best_fitness, history)
                                                   : newton_method(R, g, best_params, best_fitness, history);
        if (evaluations) *evaluations = R.evals;
        return rc;
    });
}

}  // extern "C"
