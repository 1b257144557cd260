// Frame-export driver for tests/test_frame_gpu.py, written against the
// reference's header API and compiled against the drop-in headers.  It steps
// a case, then writes the JSON frame (thermal frame for case 2) and the VTK
// frame twice: first while the device holds the newest state (the writers
// take their fields from lbm2d_frame_fields), then after a read of the f
// (and g) mirrors has brought the state to the host (the writers loop over
// the mirrors).  The two outputs must be byte-identical.
//
// usage: frame_driver <nx> <ny> <steps> <tau> <u> <case> <outdir>
//   case: 0 cylinder wake, 1 lid-driven cavity, 2 heated cavity (thermal DDF)
#include <cstdio>
#include <cstdlib>
#include <filesystem>
#include <string>

#include "lbm.hpp"

static int write_all(LBMCapabilities& system, int step, const std::string& dir, bool thermal) {
    std::filesystem::create_directories(dir);
    if (thermal)
        save_json_frame_thermal(system, step, dir, 1.25);
    else
        save_json_frame(system, step, dir);
    save_vtk_frame(system, step, dir);
    return 0;
}

int main(int argc, char** argv) {
    if (argc < 8) {
        std::fprintf(stderr, "usage: %s nx ny steps tau u case outdir\n", argv[0]);
        return 2;
    }
    NX = std::atoi(argv[1]);
    NY = std::atoi(argv[2]);
    const int steps = std::atoi(argv[3]);
    const double tau = std::atof(argv[4]), u = std::atof(argv[5]);
    const int kase = std::atoi(argv[6]);
    const std::string out = argv[7];
    const bool thermal = kase == 2;
    g_case = kase == 0 ? CaseType::CYLINDER : CaseType::CAVITY;
    LBMCapabilities system;
    if (kase == 0)
        place_cylinder(system, NX / 4, NY / 2 + 1, NY / 10);
    else
        place_walls(system);
    const double u0 = kase == 0 ? u : 0.0;
    for (int n = 0; n < NX * NY; ++n)
        for (int i = 0; i < 9; ++i) system.f[n * 9 + i] = compute_equilibrium(i, 1.0, u0, 0.0);
    if (thermal) {
        system.use_thermal = true;
        system.T_ref = 1.0;
        system.alpha = 0.02;
        system.omega_k = 1.0 / (0.5 + 3.0 * system.alpha);
        system.beta = 0.001;
        system.g_buoyancy = 0.5;
        // a hot left half and a cold right half
        for (int y = 0; y < NY; ++y)
            for (int x = 0; x < NX; ++x)
                for (int i = 0; i < 9; ++i)
                    system.g_thermal[node_index(x, y) * 9 + i] = thermal_weights[i] * (x < NX / 2 ? 1.5 : 0.5);
    }
    for (int s = 0; s < steps; ++s) execute_time_step(system, tau, kase == 2 ? 0.0 : u);
    const bool dev = system.device_state_current(thermal);
    write_all(system, steps, out + "/dev", thermal);
    const LBMCapabilities& cs = system;
    (void)cs.f.data();  // bring the state to the host mirrors
    if (thermal) (void)cs.g_thermal.data();
    const bool host = !system.device_state_current(thermal);
    write_all(system, steps, out + "/host", thermal);
    std::printf("device_path=%d host_path=%d\n", dev ? 1 : 0, host ? 1 : 0);
    return dev && host ? 0 : 6;
}
