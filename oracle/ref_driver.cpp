// Test-infrastructure driver around the reference's own CPU solver.
//
// This file is part of the oracle (checker) only: it is linked against the
// reference sources FDTD_CPU.cxx and FDTD_common.cxx, compiled unchanged from
// the reference sources by oracle/build.py, and is used to produce the golden
// vectors under tests/golden/.  Nothing in the product links or runs it.
//
// Modes
//   fitness <args.txt> <out.txt>
//       Calls the reference entry point  double FDTD_CPU(const vector<double>&)
//       (FDTD_CPU.cxx:669-892) on 162 arguments and writes the fitness
//       (%.17g).  The per-step stdout trace of FDTD_CPU.cxx:808 is discarded.
//   steps <args.txt> <nsteps> <out.bin>
//       Re-runs the body of FDTD_CPU (FDTD_CPU.cxx:746-840) through the
//       reference's own functions, but for <nsteps> time steps per excitation,
//       and dumps intermediate observables: Ez probe traces, the final fields
//       of excitation 0, the running-DFT surface currents, and the far-field
//       magnitudes D from N2FPostProcess (FDTD_CPU.cxx:538-614).
//   bench <args.txt> <nsteps> <nthreads>
//       Times the reference's own time loop (FDTD_CPU.cxx:803-813: H update,
//       E update, running DFT at every frequency) for <nsteps> steps of one
//       plane-wave excitation, in <nthreads> independent copies run at once
//       (one per host thread, as the reference farms one evaluation per MPI
//       rank).  Prints "seconds <wall> threads <n> steps <nsteps>".
//
// The reference's compile-time constants come from its own header
// FDTD_common.hxx (included from the reference tree).  That header defines
// short macros such as `d`, `dt`, `dx`, `nx`, `tau`: this file therefore uses
// no identifier with those spellings.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <vector>
#include <string>
#include <unistd.h>
#include <fcntl.h>
#include <chrono>
#include <thread>

#include "FDTD_common.hxx"

// Same memory layout as the reference's complex type (two floats); only
// pointers to it cross the boundary.
struct cpu_cuComplex { float r; float i; };

// Prototypes of the reference functions, as defined in FDTD_CPU.cxx.
void calculate_JandM(float* f, int* timestep, float* dev_Ez, float* dev_Hy, float* dev_Hx,
                     cpu_cuComplex* cjzxp, cpu_cuComplex* cjzyp, cpu_cuComplex* cjzxn, cpu_cuComplex* cjzyn,
                     cpu_cuComplex* cmxyp, cpu_cuComplex* cmyxp, cpu_cuComplex* cmxyn, cpu_cuComplex* cmyxn);
void cpu_H_field_update(float* dev_Hy, float* dev_Hx, float* dev_Ez, float* dev_bmx, float* dev_Psi_hyx,
                        float* dev_amx, float* dev_bmy, float* dev_amy, float* dev_Psi_hxy, float* kex);
void E_field_update(int* i, float* dev_Ez, float* dev_Hy, float* dev_Hx, float* dev_Psi_ezx, float* dev_aex,
                    float* dev_aey, float* dev_bex, float* dev_bey, float* dev_Psi_ezy, float* kex, float* Cezhy,
                    float* Cezhx, float* Ceze, float* Cezeip, float* Cezeic, float Phi);
void N2FPostProcess(float* D, float f, cpu_cuComplex* N, cpu_cuComplex* L, cpu_cuComplex* cjzxp,
                    cpu_cuComplex* cjzyp, cpu_cuComplex* cjzxn, cpu_cuComplex* cjzyn, cpu_cuComplex* cmxyp,
                    cpu_cuComplex* cmyxp, cpu_cuComplex* cmxyn, cpu_cuComplex* cmyxn);
void eps_r_z_init(float* eps_r_z, const std::vector<float>& argument);
void sigma_e_z_init(float* sigma_e_z, float* sigma_e_pml, const std::vector<float>& argument);
void Ceze_init(float* eps_r_z, float* sig_e_z, float* Ceze);
void Cezhy_init(float* eps_r_z, float* sigma_e_z, float* Cezhy, float* kex);
void k_e_init(float* k);
void k_m_init(float* k);
void sigma_e_pml_init(float* sigma_e_pml);
void sigma_m_pml_init(float* sigma_m_pml, float* sigma_e_pml);
void alpha_e_init(float* alpha_e);
void alpha_m_init(float* alpha_e, float* alpha_m);
void bex_init(float* bex, float* sigma_e_pml, float* kex, float* alpha_e_x);
void aex_init(float* aex, float* sigma_e_pml, float* kex, float* alpha_e_x, float* bex);
void bmx_init(float* bmx, float* sigma_m_pml, float* kmx, float* alpha_m_x);
void amx_init(float* amx, float* sigma_m_pml, float* kmx, float* alpha_m_x, float* bmx);
void cpu_scattered_parameter_init(float* eps_r_z, float* sigma_e_z, float* Cezeic, float* Cezeip);
double FDTD_CPU(const std::vector<double>& arguments);

static std::vector<double> read_args(const char* path) {
    std::vector<double> a;
    FILE* fp = std::fopen(path, "r");
    if (!fp) { std::perror(path); std::exit(2); }
    double v;
    while (std::fscanf(fp, "%lf", &v) == 1) a.push_back(v);
    std::fclose(fp);
    return a;
}

// Minimal self-describing dump: per record  u32 name_len, name, u32 ndim,
// u32 shape[ndim], float32 data.
static void put_record(FILE* fp, const char* name, const std::vector<unsigned>& shape, const float* data) {
    unsigned nl = (unsigned)std::strlen(name), nd = (unsigned)shape.size();
    size_t count = 1;
    for (unsigned s : shape) count *= s;
    std::fwrite(&nl, 4, 1, fp);
    std::fwrite(name, 1, nl, fp);
    std::fwrite(&nd, 4, 1, fp);
    std::fwrite(shape.data(), 4, nd, fp);
    std::fwrite(data, 4, count, fp);
}

static int run_fitness(const char* args_path, const char* out_path) {
    std::vector<double> args = read_args(args_path);
    std::fflush(stdout);
    int saved = dup(1);
    int devnull = open("/dev/null", O_WRONLY);
    dup2(devnull, 1);
    double fit = FDTD_CPU(args);
    std::fflush(stdout);
    dup2(saved, 1);
    close(devnull);
    close(saved);
    FILE* fp = std::fopen(out_path, "w");
    std::fprintf(fp, "%.17g\n", fit);
    std::fclose(fp);
    return 0;
}

static int run_steps(const char* args_path, int nsteps, const char* out_path) {
    std::vector<double> args = read_args(args_path);
    if (args.size() < 162) { std::fprintf(stderr, "need 162 arguments\n"); return 2; }
    std::vector<float> image(args.begin(), args.begin() + 162);

    const int NXg = nx, NYg = ny;            // 401 x 401 H grid, 402 x 402 Ez grid
    const int NEz = (NXg + 1) * (NYg + 1);
    const int NH = NXg * NYg;
    std::vector<float> Ceze(NEz), Cezhy(NEz), Cezeic(NEz), Cezeip(NEz), Ez(NEz), eps_r(NEz), sig(NEz);
    std::vector<float> Hy(NH), Hx(NH);
    std::vector<float> kex(16), kmx(16), aex(16), bex(16), amx(16), bmx(16), al_e(16), al_m(16), s_e(16), s_m(16);
    std::vector<float> psi_ezy(NXg * 20 + 64), psi_ezx(NXg * 20 + 64), psi_hyx(NYg * 20 + 64), psi_hxy(NXg * 20 + 64);
    const int ny_side = size_y_side, nx_side = size_x_side;     // per-frequency face lengths
    const int F = numberoffrequencies, A = numberofobservationangles, E = numberofexcitationangles;
    std::vector<cpu_cuComplex> cjzyp(ny_side * F), cjzyn(ny_side * F), cmxyp(ny_side * F), cmxyn(ny_side * F);
    std::vector<cpu_cuComplex> cjzxp(nx_side * F), cjzxn(nx_side * F), cmyxp(nx_side * F), cmyxn(nx_side * F);
    std::vector<cpu_cuComplex> Nn(size_NF2FF_total + 8), Ll(size_NF2FF_total + 8);
    std::vector<float> Dall((size_t)E * F * A, 0.f);

    eps_r_z_init(eps_r.data(), image);
    sigma_e_z_init(sig.data(), s_e.data(), image);
    Ceze_init(eps_r.data(), sig.data(), Ceze.data());
    k_e_init(kex.data());
    k_m_init(kmx.data());
    Cezhy_init(eps_r.data(), sig.data(), Cezhy.data(), kex.data());
    sigma_e_pml_init(s_e.data());
    sigma_m_pml_init(s_m.data(), s_e.data());
    alpha_e_init(al_e.data());
    alpha_m_init(al_e.data(), al_m.data());
    bex_init(bex.data(), s_e.data(), kex.data(), al_e.data());
    aex_init(aex.data(), s_e.data(), kex.data(), al_e.data(), bex.data());
    bmx_init(bmx.data(), s_m.data(), kmx.data(), al_m.data());
    amx_init(amx.data(), s_m.data(), kmx.data(), al_m.data(), bmx.data());
    cpu_scattered_parameter_init(eps_r.data(), sig.data(), Cezeic.data(), Cezeip.data());

    // probe cells (x, y) on the Ez grid
    const int probes[][2] = {{200, 200}, {215, 185}, {180, 210}, {230, 200}, {150, 200},
                             {5, 200},   {200, 395}, {100, 100}, {300, 250}};
    const int NP = (int)(sizeof(probes) / sizeof(probes[0]));
    std::vector<float> traces((size_t)E * nsteps * NP);

    FILE* fp = std::fopen(out_path, "wb");
    if (!fp) { std::perror(out_path); return 2; }
    std::vector<float> probe_xy;
    for (int p = 0; p < NP; ++p) { probe_xy.push_back((float)probes[p][0]); probe_xy.push_back((float)probes[p][1]); }
    put_record(fp, "probe_xy", {(unsigned)NP, 2u}, probe_xy.data());

    auto reset = [&]() {
        std::fill(Ez.begin(), Ez.end(), 0.f);
        std::fill(Hx.begin(), Hx.end(), 0.f);
        std::fill(Hy.begin(), Hy.end(), 0.f);
        std::fill(psi_ezx.begin(), psi_ezx.end(), 0.f);
        std::fill(psi_ezy.begin(), psi_ezy.end(), 0.f);
        std::fill(psi_hyx.begin(), psi_hyx.end(), 0.f);
        std::fill(psi_hxy.begin(), psi_hxy.end(), 0.f);
        for (auto* v : {&cjzyp, &cjzyn, &cmxyp, &cmxyn, &cjzxp, &cjzxn, &cmyxp, &cmyxn})
            std::fill(v->begin(), v->end(), cpu_cuComplex{0.f, 0.f});
    };
    reset();
    for (int pe = 0; pe < E; ++pe) {
        float Phi = (float)pe * 2 * PI / numberofexcitationangles;
        for (int it = 0; it < nsteps; ++it) {
            cpu_H_field_update(Hy.data(), Hx.data(), Ez.data(), bmx.data(), psi_hyx.data(), amx.data(), bmx.data(),
                               amx.data(), psi_hxy.data(), kmx.data());
            E_field_update(&it, Ez.data(), Hy.data(), Hx.data(), psi_ezx.data(), aex.data(), aex.data(), bex.data(),
                           bex.data(), psi_ezy.data(), kex.data(), Cezhy.data(), Cezhy.data(), Ceze.data(),
                           Cezeip.data(), Cezeic.data(), Phi);
            for (int p = 0; p < NP; ++p)
                traces[((size_t)pe * nsteps + it) * NP + p] = Ez[probes[p][0] + probes[p][1] * (NXg + 1)];
            for (int fi = 0; fi < F; ++fi) {
                float freq = startfrequency + deltafreq * fi;
                calculate_JandM(&freq, &it, Ez.data(), Hy.data(), Hx.data(), cjzxp.data() + fi * nx_side,
                                cjzyp.data() + fi * ny_side, cjzxn.data() + fi * nx_side, cjzyn.data() + fi * ny_side,
                                cmxyp.data() + fi * ny_side, cmyxp.data() + fi * nx_side, cmxyn.data() + fi * ny_side,
                                cmyxn.data() + fi * nx_side);
            }
        }
        for (int fi = 0; fi < F; ++fi) {
            float freq = startfrequency + deltafreq * fi;
            std::fill(Nn.begin(), Nn.end(), cpu_cuComplex{0.f, 0.f});
            std::fill(Ll.begin(), Ll.end(), cpu_cuComplex{0.f, 0.f});
            N2FPostProcess(Dall.data() + (size_t)pe * A * F + (size_t)fi * A, freq, Nn.data(), Ll.data(),
                           cjzxp.data() + nx_side * fi, cjzyp.data() + ny_side * fi, cjzxn.data() + nx_side * fi,
                           cjzyn.data() + ny_side * fi, cmxyp.data() + ny_side * fi, cmyxp.data() + nx_side * fi,
                           cmxyn.data() + ny_side * fi, cmyxn.data() + nx_side * fi);
        }
        if (pe == 0 || pe == 2) {
            // surface-current accumulators, complex interleaved, all frequencies
            char name[64];
            struct { const char* n; std::vector<cpu_cuComplex>* v; unsigned len; } acc[] = {
                {"cjzyn", &cjzyn, (unsigned)ny_side}, {"cjzxp", &cjzxp, (unsigned)nx_side},
                {"cjzyp", &cjzyp, (unsigned)ny_side}, {"cjzxn", &cjzxn, (unsigned)nx_side},
                {"cmxyn", &cmxyn, (unsigned)ny_side}, {"cmyxp", &cmyxp, (unsigned)nx_side},
                {"cmxyp", &cmxyp, (unsigned)ny_side}, {"cmyxn", &cmyxn, (unsigned)nx_side}};
            for (auto& a : acc) {
                std::snprintf(name, sizeof name, "%s_e%d", a.n, pe);
                put_record(fp, name, {(unsigned)F, a.len, 2u}, reinterpret_cast<const float*>(a.v->data()));
            }
        }
        if (pe == 0) {
            put_record(fp, "Ez_e0", {(unsigned)(NYg + 1), (unsigned)(NXg + 1)}, Ez.data());
            put_record(fp, "Hx_e0", {(unsigned)NYg, (unsigned)NXg}, Hx.data());
            put_record(fp, "Hy_e0", {(unsigned)NYg, (unsigned)NXg}, Hy.data());
        }
        reset();
    }
    put_record(fp, "traces", {(unsigned)E, (unsigned)nsteps, (unsigned)NP}, traces.data());
    put_record(fp, "D", {(unsigned)E, (unsigned)F, (unsigned)A}, Dall.data());
    std::fclose(fp);
    return 0;
}

// One independent copy of the reference time loop (FDTD_CPU.cxx:746-813 set-up
// and stepping) for nsteps steps of excitation 0; returns a checksum so the
// work cannot be optimised away.
static double bench_copy(const std::vector<float>& image, int nsteps) {
    const int NXg = nx, NYg = ny;
    const int NEz = (NXg + 1) * (NYg + 1), NH = NXg * NYg;
    std::vector<float> Ceze(NEz), Cezhy(NEz), Cezeic(NEz), Cezeip(NEz), Ez(NEz), eps_r(NEz), sig(NEz);
    std::vector<float> Hy(NH), Hx(NH);
    std::vector<float> kex(16), kmx(16), aex(16), bex(16), amx(16), bmx(16), al_e(16), al_m(16), s_e(16), s_m(16);
    std::vector<float> psi_ezy(NXg * 20 + 64), psi_ezx(NXg * 20 + 64), psi_hyx(NYg * 20 + 64), psi_hxy(NXg * 20 + 64);
    const int ny_side = size_y_side, nx_side = size_x_side, F = numberoffrequencies;
    std::vector<cpu_cuComplex> cjzyp(ny_side * F), cjzyn(ny_side * F), cmxyp(ny_side * F), cmxyn(ny_side * F);
    std::vector<cpu_cuComplex> cjzxp(nx_side * F), cjzxn(nx_side * F), cmyxp(nx_side * F), cmyxn(nx_side * F);
    eps_r_z_init(eps_r.data(), image);
    sigma_e_z_init(sig.data(), s_e.data(), image);
    Ceze_init(eps_r.data(), sig.data(), Ceze.data());
    k_e_init(kex.data());
    k_m_init(kmx.data());
    Cezhy_init(eps_r.data(), sig.data(), Cezhy.data(), kex.data());
    sigma_e_pml_init(s_e.data());
    sigma_m_pml_init(s_m.data(), s_e.data());
    alpha_e_init(al_e.data());
    alpha_m_init(al_e.data(), al_m.data());
    bex_init(bex.data(), s_e.data(), kex.data(), al_e.data());
    aex_init(aex.data(), s_e.data(), kex.data(), al_e.data(), bex.data());
    bmx_init(bmx.data(), s_m.data(), kmx.data(), al_m.data());
    amx_init(amx.data(), s_m.data(), kmx.data(), al_m.data(), bmx.data());
    cpu_scattered_parameter_init(eps_r.data(), sig.data(), Cezeic.data(), Cezeip.data());
    const float Phi = 0.f;
    for (int it = 0; it < nsteps; ++it) {
        cpu_H_field_update(Hy.data(), Hx.data(), Ez.data(), bmx.data(), psi_hyx.data(), amx.data(), bmx.data(),
                           amx.data(), psi_hxy.data(), kmx.data());
        E_field_update(&it, Ez.data(), Hy.data(), Hx.data(), psi_ezx.data(), aex.data(), aex.data(), bex.data(),
                       bex.data(), psi_ezy.data(), kex.data(), Cezhy.data(), Cezhy.data(), Ceze.data(), Cezeip.data(),
                       Cezeic.data(), Phi);
        for (int fi = 0; fi < F; ++fi) {
            float freq = startfrequency + deltafreq * fi;
            calculate_JandM(&freq, &it, Ez.data(), Hy.data(), Hx.data(), cjzxp.data() + fi * nx_side,
                            cjzyp.data() + fi * ny_side, cjzxn.data() + fi * nx_side, cjzyn.data() + fi * ny_side,
                            cmxyp.data() + fi * ny_side, cmyxp.data() + fi * nx_side, cmxyn.data() + fi * ny_side,
                            cmyxn.data() + fi * nx_side);
        }
    }
    double sum = 0;
    for (float v : Ez) sum += v;
    return sum + cjzyn[0].r;
}

static int run_bench(const char* args_path, int nsteps, int nthreads) {
    std::vector<double> args = read_args(args_path);
    if (args.size() < 162) { std::fprintf(stderr, "need 162 arguments\n"); return 2; }
    std::vector<float> image(args.begin(), args.begin() + 162);
    std::vector<double> sums(nthreads, 0.0);
    const auto tic = std::chrono::steady_clock::now();
    std::vector<std::thread> pool;
    for (int t = 0; t < nthreads; ++t) pool.emplace_back([&, t] { sums[t] = bench_copy(image, nsteps); });
    for (auto& th : pool) th.join();
    const auto toc = std::chrono::steady_clock::now();
    std::printf("seconds %.6f threads %d steps %d checksum %.9g\n", std::chrono::duration<double>(toc - tic).count(),
                nthreads, nsteps, sums[0]);
    return 0;
}

int main(int argc, char** argv) {
    if (argc >= 4 && std::strcmp(argv[1], "fitness") == 0) return run_fitness(argv[2], argv[3]);
    if (argc >= 5 && std::strcmp(argv[1], "steps") == 0) return run_steps(argv[2], std::atoi(argv[3]), argv[4]);
    if (argc >= 5 && std::strcmp(argv[1], "bench") == 0)
        return run_bench(argv[2], std::atoi(argv[3]), std::max(1, std::atoi(argv[4])));
    std::fprintf(stderr, "usage: %s fitness <args> <out> | steps <args> <nsteps> <out.bin> | bench <args> <nsteps> <threads>\n", argv[0]);
    return 2;
}
