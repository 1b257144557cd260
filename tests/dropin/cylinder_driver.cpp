// A case driver written against the reference's header API, compiled here
// against the drop-in headers (lbm-2d_gb300/dropin) and run on the GPU by
// tests/test_dropin_gpu.py.  It follows the cylinder-wake driver pattern:
// set the globals, build LBMCapabilities, place the obstacle, write the
// initial populations through sys.f, loop execute_time_step and sum
// fx_body / fy_body every step, then write the final state.
//
// usage: cylinder_driver <nx> <ny> <steps> <tau> <u> <init.bin> <out.bin> [case] [les]
//   init.bin : nx*ny*9 FP64 populations; out.bin: f (nx*ny*9), then per-step
//   (fx_total, fy_total), all FP64 little-endian.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "lbm.hpp"

int main(int argc, char** argv) {
    if (argc < 8) {
        std::fprintf(stderr, "usage: %s nx ny steps tau u init.bin out.bin [case] [les]\n", argv[0]);
        return 2;
    }
    NX = std::atoi(argv[1]);
    NY = std::atoi(argv[2]);
    const int steps = std::atoi(argv[3]);
    const double tau = std::atof(argv[4]), u = std::atof(argv[5]);
    g_case = argc > 8 ? static_cast<CaseType>(std::atoi(argv[8])) : CaseType::CYLINDER;
    g_use_les = argc > 9 && std::atoi(argv[9]) != 0;
    LBMCapabilities system;
    if (g_case == CaseType::CAVITY)
        place_walls(system);
    else
        place_cylinder(system, NX / 4, NY / 2 + 1, NY / 10);
    std::vector<double> init(static_cast<size_t>(NX) * NY * 9);
    FILE* fi = std::fopen(argv[6], "rb");
    if (!fi || std::fread(init.data(), sizeof(double), init.size(), fi) != init.size()) return 3;
    std::fclose(fi);
    for (int n = 0; n < NX * NY; ++n) {
        double* f_node = &system.f[n * 9];
        for (int i = 0; i < 9; ++i) f_node[i] = init[static_cast<size_t>(n) * 9 + i];
    }
    std::vector<double> sums;
    for (int s = 0; s < steps; ++s) {
        execute_time_step(system, tau, u);
        double fx = 0.0, fy = 0.0;
        for (int n = 0; n < NX * NY; ++n) {
            fx += system.fx_body[n];
            fy += system.fy_body[n];
        }
        sums.push_back(fx);
        sums.push_back(fy);
    }
    FILE* fo = std::fopen(argv[7], "wb");
    if (!fo) return 4;
    const LBMCapabilities& cs = system;
    std::fwrite(cs.f.data(), sizeof(double), cs.f.size(), fo);
    std::fwrite(sums.data(), sizeof(double), sums.size(), fo);
    std::fclose(fo);
    // the output writers read the mirrors (downloaded lazily)
    save_json_frame(system, steps, "dropin_out");
    // the per-step drag/lift stream, read back once from the device history
    const int lines = save_forces_history_jsonl(system, "dropin_out", 0, NY / 5.0, u);
    return lines == (g_case == CaseType::CAVITY ? 0 : steps) ? 0 : 5;
}
