// Drives the drop-in's host-side node operators -- mrt_collide and
// apply_bouzidi_bb (lbm-2d_gb300/dropin/lbm.hpp) -- on inputs read from a
// file and writes their results, for a bit-for-bit comparison with the
// oracle.  No device call is made.
//
// input (little-endian): int32 nx, ny, use_mei, moving_wall, n_links, n_mrt;
//   double cx, cy, r, omega, rot_cx, rot_cy; uint8 mask[nx*ny];
//   double f[nx*ny*9]; int32 links[n_links][3] (x, y, i);
//   n_mrt x double[9 + 6] (f[9], rho, u, v, tau, cs_sq, y_plus)
// output: double f_next value per link, then 9 doubles per MRT case.
#include <cstdint>
#include <cstdio>
#include <vector>

#include "lbm.hpp"

template <class T>
static void rd(FILE* fp, T* p, size_t n) {
    if (fread(p, sizeof(T), n, fp) != n) throw std::runtime_error("short input");
}

int main(int argc, char** argv) {
    if (argc != 3) return 2;
    FILE* fp = std::fopen(argv[1], "rb");
    if (!fp) return 3;
    int32_t hdr[6];
    rd(fp, hdr, 6);
    double geo[6];
    rd(fp, geo, 6);
    NX = hdr[0];
    NY = hdr[1];
    LBMCapabilities sys;  // host mirrors only: no device solver is created here
    std::vector<uint8_t> mask((size_t)NX * NY);
    rd(fp, mask.data(), mask.size());
    for (size_t k = 0; k < mask.size(); ++k) sys.obstacle[k] = mask[k];
    std::vector<double> f((size_t)NX * NY * 9);
    rd(fp, f.data(), f.size());
    for (size_t k = 0; k < f.size(); ++k) sys.f[k] = f[k];
    sys.bb_geom.cx = geo[0];
    sys.bb_geom.cy = geo[1];
    sys.bb_geom.radius = geo[2];
    sys.bb_geom.use_mei_bb = hdr[2] != 0;
    sys.bb_geom.has_moving_wall = hdr[3] != 0;
    sys.bb_geom.omega = geo[3];
    sys.bb_geom.rot_cx = geo[4];
    sys.bb_geom.rot_cy = geo[5];
    std::vector<int32_t> links((size_t)hdr[4] * 3);
    rd(fp, links.data(), links.size());
    std::vector<double> out;
    for (int k = 0; k < hdr[4]; ++k) {
        const int x = links[3 * k], y = links[3 * k + 1], i = links[3 * k + 2];
        const int n = node_index(x, y);
        double fn[9];
        for (int j = 0; j < 9; ++j) fn[j] = f[(size_t)n * 9 + j];
        apply_bouzidi_bb(sys, x, y, i, fn, n);
        out.push_back(sys.f_next[(size_t)n * 9 + bounce_back[i]]);
    }
    for (int k = 0; k < hdr[5]; ++k) {
        double a[15];
        rd(fp, a, 15);
        mrt_collide(a, a[9], a[10], a[11], MRTParams::from_tau(a[12]), a[13], a[12], a[14]);
        out.insert(out.end(), a, a + 9);
    }
    std::fclose(fp);
    FILE* fo = std::fopen(argv[2], "wb");
    if (!fo) return 4;
    std::fwrite(out.data(), sizeof(double), out.size(), fo);
    std::fclose(fo);
    return 0;
}
