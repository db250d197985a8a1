// A C++ consumer of the C ABI through include/fans_gb300_solver.hpp, as a FANS
// build would use it from createSolver (include/setup.h:76-85) and runSolver
// (src/main.cpp:10-46): build a SolverGPU<3,6> from Reader-like settings and a
// phase table, run load cases with solve() and extrapolateDisplacement(), and
// print get_homogenized_stress() and get_homogenized_tangent().
//
// Test infrastructure: tests/test_gpu_cpp_binding.py compiles it with g++,
// links it to libfans_gb300.so and compares its output with the oracle.
//
// Input (whitespace-separated text, argv[1]):
//   nx ny nz
//   FE_type precision method measure type TOL n_it
//   nphase, then per phase: law nparams params...
//   kapparef (36 values, row-major)
//   nload, then per load case 6 values of g0
//   the microstructure (nx*ny*nz phase ids, [x][y][z])
// Output lines: "iterations k n", "stress k s1..s6", "tangent c1..c36",
// "invalid_argument ok" (a bad FE_type is rejected as the reference rejects it).
#include "fans_gb300_solver.hpp"

#include <cstdio>
#include <fstream>
#include <iostream>

int main(int argc, char **argv)
{
    if (argc < 2) {
        std::fprintf(stderr, "usage: %s input.txt\n", argv[0]);
        return 2;
    }
    std::ifstream in(argv[1]);
    fansgpu::SolverGPUConfig cfg;
    in >> cfg.dims[0] >> cfg.dims[1] >> cfg.dims[2];
    in >> cfg.FE_type >> cfg.precision >> cfg.method >> cfg.measure >> cfg.type >> cfg.TOL >> cfg.n_it;
    int nph = 0;
    in >> nph;
    std::vector<fansgpu::PhaseMaterial> phases(nph);
    for (auto &p : phases) {
        int np = 0;
        in >> p.law >> np;
        p.params.resize(np);
        for (auto &v : p.params)
            in >> v;
    }
    std::vector<double> kref(36);
    for (auto &v : kref)
        in >> v;
    int nload = 0;
    in >> nload;
    std::vector<std::array<double, 6>> loads(nload);
    for (auto &g : loads)
        for (auto &v : g)
            in >> v;
    cfg.ms.resize((size_t)cfg.dims[0] * cfg.dims[1] * cfg.dims[2]);
    for (auto &m : cfg.ms) {
        int v = 0;
        in >> v;
        m = (uint16_t)v;
    }
    if (!in) {
        std::fprintf(stderr, "bad input\n");
        return 2;
    }
    try {
        fansgpu::SolverGPU<3, 6> solver(cfg, phases, kref);
        for (int k = 0; k < nload; ++k) {
            solver.set_gradient(loads[k]);
            solver.solve();
            const auto s = solver.get_homogenized_stress();
            std::printf("iterations %d %zu\n", k, solver.iter);
            std::printf("stress %d", k);
            for (double v : s)
                std::printf(" %.17g", v);
            std::printf("\n");
            solver.extrapolateDisplacement();
        }
        const auto C = solver.get_homogenized_tangent(1e-6);
        std::printf("tangent");
        for (double v : C)
            std::printf(" %.17g", v);
        std::printf("\n");
    } catch (const std::exception &e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    try {
        fansgpu::SolverGPUConfig bad = cfg;
        bad.FE_type                  = "HEX20";
        fansgpu::SolverGPU<3, 6> s(bad, phases, kref);
        std::printf("invalid_argument missing\n");
    } catch (const std::invalid_argument &) {
        std::printf("invalid_argument ok\n");
    }
    return 0;
}
