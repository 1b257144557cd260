// Airfoil immersed-boundary driver for tests/test_ibm_gpu.py, written
// against the reference's header API and compiled against the drop-in
// headers.  The set-up is the airfoil driver's (NACA polygon at (NX/4, NY/2),
// chord NY/3, obstacle by point-in-polygon, uniform equilibrium at the
// inflow angle); the loop body is execute_time_step alone, with the
// immersed boundary's forcing attached to the device.
//
// usage: ibm_driver <nx> <ny> <steps> <tau> <u> <naca> <npts> <aoa> <spacing> <les> <out.bin>
//   out.bin: f (nx*ny*9), then U, V, FX, FY of the points, FP64.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "lbm.hpp"

int main(int argc, char** argv) {
    if (argc < 12) {
        std::fprintf(stderr, "usage: %s nx ny steps tau u naca npts aoa spacing les out.bin\n", argv[0]);
        return 2;
    }
    NX = std::atoi(argv[1]);
    NY = std::atoi(argv[2]);
    const int steps = std::atoi(argv[3]);
    const double tau = std::atof(argv[4]), u = std::atof(argv[5]);
    const int series = std::atoi(argv[6]), npts = std::atoi(argv[7]);
    const double aoa = std::atof(argv[8]), spacing = std::atof(argv[9]);
    g_use_les = std::atoi(argv[10]) != 0;
    LBMCapabilities system;
    auto poly = naca_coords(series, npts);
    transform_points(poly, static_cast<double>(NX) / 4, static_cast<double>(NY) / 2, static_cast<double>(NY) / 3.0,
                     aoa);
    for (int y = 0; y < NY; ++y)
        for (int x = 0; x < NX; ++x)
            if (point_in_polygon(static_cast<double>(x), static_cast<double>(y), poly))
                system.obstacle[node_index(x, y)] = true;
    const double a = aoa * M_PI / 180.0;
    for (int n = 0; n < NX * NY; ++n)
        for (int i = 0; i < 9; ++i) system.f[n * 9 + i] = compute_equilibrium(i, 1.0, u * std::cos(a), u * std::sin(a));
    ImmersedBoundary ib;
    ib.build_from_polygon(poly, spacing);
    lbm2d_dropin::attach_ibm(system, ib);
    for (int s = 0; s < steps; ++s) execute_time_step(system, tau, u);
    lbm2d_dropin::ibm_lagrangian(system, ib);
    FILE* fo = std::fopen(argv[11], "wb");
    if (!fo) return 4;
    const LBMCapabilities& cs = system;
    std::fwrite(cs.f.data(), sizeof(double), cs.f.size(), fo);
    for (int k = 0; k < 4; ++k)
        for (const auto& p : ib.points) {
            const double v = k == 0 ? p.U : k == 1 ? p.V : k == 2 ? p.FX : p.FY;
            std::fwrite(&v, sizeof(double), 1, fo);
        }
    std::fclose(fo);
    return 0;
}
