// lbm.hpp -- drop-in replacement of the reference's src/lbm.hpp.
//
// execute_time_step runs on the GPU (one fused sm_103a kernel per step, see
// lbm-2d_gb300/csrc/lbm2d_kernels.cu).  Everything else keeps the reference's
// names and host semantics: the boundary-condition helpers, the node-level
// MRT collision and interpolated bounce-back, the obstacle placement and the
// frame/force/metadata writers, which read the LBMCapabilities mirrors (so
// they download the device state on first use after a step).
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <filesystem>
#include <fstream>
#include <iostream>
#include <string>

#include "geometry.hpp"
#include "lbm_types.hpp"
#include "thermal.hpp"
#include "ibm.hpp"
#if __has_include("wall_functions.hpp")
#include "wall_functions.hpp"
#endif

// ---------------------------------------------------------------- boundary conditions (host)
// Zou/He velocity inlet at x = 0, src/lbm.hpp:21-34
inline void enforce_inflow(LBMCapabilities& sys, double u_inflow) {
    for (int y = 0; y < NY; ++y) {
        double* fn = &sys.f[static_cast<size_t>(node_index(0, y)) * 9];
        const double rho = (fn[0] + fn[2] + fn[4] + 2.0 * (fn[3] + fn[6] + fn[7])) / (1.0 - u_inflow);
        fn[1] = fn[3] + (2.0 / 3.0) * rho * u_inflow;
        fn[5] = fn[7] + (1.0 / 6.0) * rho * u_inflow;
        fn[8] = fn[6] + (1.0 / 6.0) * rho * u_inflow;
    }
}

// parabolic inlet, src/lbm.hpp:40-58
inline void enforce_step_inflow(LBMCapabilities& sys, int h_step, int h_inlet, double u_max) {
    for (int y = h_step; y < NY; ++y) {
        if (sys.obstacle[node_index(0, y)]) continue;
        double* fn = &sys.f[static_cast<size_t>(node_index(0, y)) * 9];
        const double yy = static_cast<double>(y - h_step), h = static_cast<double>(h_inlet);
        const double ul = u_max * 4.0 * yy * (h - yy) / (h * h);
        const double rho = (fn[0] + fn[2] + fn[4] + 2.0 * (fn[3] + fn[6] + fn[7])) / (1.0 - ul);
        fn[1] = fn[3] + (2.0 / 3.0) * rho * ul;
        fn[5] = fn[7] + (1.0 / 6.0) * rho * ul;
        fn[8] = fn[6] + (1.0 / 6.0) * rho * ul;
    }
}

// zero-gradient outlet, src/lbm.hpp:63-73
inline void enforce_outflow(LBMCapabilities& sys) {
    for (int y = 0; y < NY; ++y) {
        double* dst = &sys.f[static_cast<size_t>(node_index(NX - 1, y)) * 9];
        const double* src = &sys.f[static_cast<size_t>(node_index(NX - 2, y)) * 9];
        for (int i = 0; i < 9; ++i) dst[i] = src[i];
    }
}

// src/lbm.hpp:79-87
inline void place_walls(LBMCapabilities& sys) { lbm2d_mask_walls(NX, NY, sys.obstacle.data()); }

// src/lbm.hpp:93-104
inline bool check_convergence(const std::vector<double>& values, int window = 1000, double threshold = 1e-4) {
    const int n = static_cast<int>(values.size());
    if (n < 2 * window) return false;
    double recent = 0.0, earlier = 0.0;
    for (int i = n - window; i < n; ++i) recent += values[i];
    recent /= static_cast<double>(window);
    for (int i = n - 2 * window; i < n - window; ++i) earlier += values[i];
    earlier /= static_cast<double>(window);
    return std::abs(recent - earlier) < threshold;
}

// equilibrium lid at y = NY-1, src/lbm.hpp:110-120
inline void enforce_lid(LBMCapabilities& sys, double u_lid) {
    for (int x = 0; x < NX; ++x) {
        double* fn = &sys.f[static_cast<size_t>(node_index(x, NY - 1)) * 9];
        double rho, u, v;
        compute_macros(fn, rho, u, v);
        for (int i = 0; i < 9; ++i) fn[i] = compute_equilibrium(i, rho, u_lid, 0.0);
    }
}

// ---------------------------------------------------------------- node-level operators (host)
// d'Humieres MRT of one node with optional Smagorinsky / Van Driest,
// src/lbm.hpp:128-218.  The GPU kernel applies the same operator to every
// node.  This host form keeps the reference's operation order term by term
// (moments, the plain and then the damped LES rate, relaxation, the inverse
// transform as a sum over the moment vector), so with FP contraction off it
// gives the reference's bits.
inline void mrt_collide(double* f_node, double rho, double u, double v, const MRTParams& mrt, double cs_sq = 0.0,
                        double tau_base = 0.0, double y_plus = 0.0) {
    const double f0 = f_node[0], f1 = f_node[1], f2 = f_node[2], f3 = f_node[3], f4 = f_node[4];
    const double f5 = f_node[5], f6 = f_node[6], f7 = f_node[7], f8 = f_node[8];
    double e = -4 * f0 - f1 - f2 - f3 - f4 + 2 * (f5 + f6 + f7 + f8);
    double eps = 4 * f0 - 2 * (f1 + f2 + f3 + f4) + (f5 + f6 + f7 + f8);
    double qx = -2 * f1 + 2 * f3 + f5 - f6 - f7 + f8;
    double qy = -2 * f2 + 2 * f4 + f5 + f6 - f7 - f8;
    double pxx = f1 - f2 + f3 - f4;
    double pxy = f5 - f6 + f7 - f8;
    const double jx = rho * u, jy = rho * v, usq = u * u + v * v;
    const double e_eq = -2 * rho + 3 * rho * usq, eps_eq = rho - 3 * rho * usq;
    const double qx_eq = -jx, qy_eq = -jy;
    const double pxx_eq = rho * (u * u - v * v), pxy_eq = rho * u * v;
    auto clamp = [](double s) { return (s < 0.5) ? 0.5 : ((s > 1.99) ? 1.99 : s); };
    // LES relaxation rate for a Smagorinsky constant squared c2
    auto les_rate = [&](double c2) {
        const double a = pxx - pxx_eq, b = pxy - pxy_eq;
        const double Q = std::sqrt(2.0 * (a * a + b * b));
        const double A = 9.0 * c2 * Q / (2.0 * rho);
        const double t = (tau_base + std::sqrt(tau_base * tau_base + 4.0 * A)) / 2.0;
        return clamp(1.0 / t);
    };
    double s_eff = mrt.s_shear;
    if (cs_sq > 0.0 && tau_base > 0.0) s_eff = les_rate(cs_sq);
    if (cs_sq > 0.0 && tau_base > 0.0 && y_plus > 0.0) {  // Van Driest damping overrides
        const double cd = std::sqrt(cs_sq) * (1.0 - std::exp(-y_plus / 26.0));
        s_eff = les_rate(cd * cd);
    }
    e -= mrt.s_bulk * (e - e_eq);
    eps -= mrt.s_bulk * (eps - eps_eq);
    qx -= mrt.s_normal * (qx - qx_eq);
    qy -= mrt.s_normal * (qy - qy_eq);
    pxx -= s_eff * (pxx - pxx_eq);
    pxy -= s_eff * (pxy - pxy_eq);
    // inverse transform: row i of M^-1 dotted with (rho, e, eps, jx, qx, jy, qy, pxx, pxy)
    const double m[9] = {rho, e, eps, jx, qx, jy, qy, pxx, pxy};
    static constexpr double Minv[9][9] = {
        {1.0 / 9, -1.0 / 9, 1.0 / 9, 0, 0, 0, 0, 0, 0},
        {1.0 / 9, -1.0 / 36, -1.0 / 18, 1.0 / 6, -1.0 / 6, 0, 0, 1.0 / 4, 0},
        {1.0 / 9, -1.0 / 36, -1.0 / 18, 0, 0, 1.0 / 6, -1.0 / 6, -1.0 / 4, 0},
        {1.0 / 9, -1.0 / 36, -1.0 / 18, -1.0 / 6, 1.0 / 6, 0, 0, 1.0 / 4, 0},
        {1.0 / 9, -1.0 / 36, -1.0 / 18, 0, 0, -1.0 / 6, 1.0 / 6, -1.0 / 4, 0},
        {1.0 / 9, 1.0 / 18, 1.0 / 36, 1.0 / 6, 1.0 / 12, 1.0 / 6, 1.0 / 12, 0, 1.0 / 4},
        {1.0 / 9, 1.0 / 18, 1.0 / 36, -1.0 / 6, -1.0 / 12, 1.0 / 6, 1.0 / 12, 0, -1.0 / 4},
        {1.0 / 9, 1.0 / 18, 1.0 / 36, -1.0 / 6, -1.0 / 12, -1.0 / 6, -1.0 / 12, 0, 1.0 / 4},
        {1.0 / 9, 1.0 / 18, 1.0 / 36, 1.0 / 6, 1.0 / 12, -1.0 / 6, -1.0 / 12, 0, -1.0 / 4}};
    for (int i = 0; i < 9; ++i) {
        // left to right over the nonzero entries: the reference's sum order
        double acc = Minv[i][0] * m[0];
        for (int k = 1; k < 9; ++k)
            if (Minv[i][k] != 0.0) acc += Minv[i][k] * m[k];
        f_node[i] = acc;
    }
}

// Interpolated bounce-back of one link into sys.f_next (host), src/lbm.hpp:226-288:
// Mei / Filippova-Hanel by default; classic Bouzidi (the source node's value
// when q < 1/2, the node's own opposite value otherwise) with the Ladd wall
// term when use_mei_bb is off.  Same operation order as the reference.
inline void apply_bouzidi_bb(LBMCapabilities& sys, int x, int y, int i, const double* f_node, int node_idx) {
    if (sys.f_next.size() != sys.f.size()) sys.f_next.assign(sys.f.size(), 0.0);
    const BounceBackGeometry& g = sys.bb_geom;
    const double q = g.compute_q(static_cast<double>(x), static_cast<double>(y), i);
    const int bb = bounce_back[i];
    auto wall_velocity = [&](double& uwx, double& uwy) {
        g.compute_wall_velocity(static_cast<double>(x + cx[i]), static_cast<double>(y + cy[i]), uwx, uwy);
    };
    double fbb;
    if (g.use_mei_bb) {
        double rho, u, v;
        compute_macros(f_node, rho, u, v);
        double uwx = 0.0, uwy = 0.0;
        if (g.has_moving_wall) wall_velocity(uwx, uwy);
        const double feq_wall = compute_equilibrium(i, rho, uwx, uwy);
        const double ed = cx[i] * uwx + cy[i] * uwy;
        fbb = q * feq_wall + (1.0 - q) * f_node[i] + (2.0 * q - 1.0) * weights[i] * rho * ed * 3.0;
    } else if (q < 0.5) {
        const int sx = x - cx[i], sy = y - cy[i];
        if (sx >= 0 && sx < NX && sy >= 0 && sy < NY)
            fbb = 2.0 * q * f_node[i] + (1.0 - 2.0 * q) * sys.f[static_cast<size_t>(node_index(sx, sy)) * 9 + i];
        else
            fbb = f_node[i];
    } else {
        const double inv2q = 1.0 / (2.0 * q);
        fbb = inv2q * f_node[i] + (1.0 - inv2q) * sys.f[static_cast<size_t>(node_idx) * 9 + bb];
    }
    if (g.has_moving_wall && !g.use_mei_bb) {
        double uwx, uwy, rho, u, v;
        wall_velocity(uwx, uwy);
        compute_macros(f_node, rho, u, v);
        const double ed = cx[i] * uwx + cy[i] * uwy;
        fbb -= 2.0 * weights[i] * rho * ed * 3.0;
    }
    sys.f_next[static_cast<size_t>(node_idx) * 9 + bb] = fbb;
}

// ---------------------------------------------------------------- the time step (GPU)
// src/lbm.hpp:293-582: collision, streaming with (interpolated) bounce-back,
// boundary conditions and the momentum-exchange force, fused on the device.
inline void execute_time_step(LBMCapabilities& sys, double tau, double u_inflow) { sys.device_step(tau, u_inflow); }

// ---------------------------------------------------------------- obstacle placement
// src/lbm.hpp:931-944
inline void place_cylinder(LBMCapabilities& sys, int cx_cyl, int cy_cyl, int radius) {
    sys.bb_geom.cx = static_cast<double>(cx_cyl);
    sys.bb_geom.cy = static_cast<double>(cy_cyl);
    sys.bb_geom.radius = static_cast<double>(radius);
    lbm2d_mask_cylinder(NX, NY, sys.obstacle.data(), cx_cyl, cy_cyl, radius);
}

// src/lbm.hpp:951-964
inline void place_polygon(LBMCapabilities& sys, const std::vector<std::pair<double, double>>& poly) {
    sys.bb_geom.poly_vertices = poly;
    sys.bb_geom.is_polygon = true;
    std::vector<double> xy;
    xy.reserve(poly.size() * 2);
    for (auto& p : poly) {
        xy.push_back(p.first);
        xy.push_back(p.second);
    }
    lbm2d_mask_polygon(NX, NY, sys.obstacle.data(), xy.data(), static_cast<int>(poly.size()));
}

// ---------------------------------------------------------------- output writers (host)
namespace lbm2d_dropin {
// The frame fields from the host mirrors (used when the host has changed
// the state since the last step).
inline void host_frame_fields(const LBMCapabilities& sys, int ds, int nxd, int nyd, bool thermal, double T_wall,
                              std::vector<double>& vel, std::vector<double>& ua, std::vector<double>& va,
                              std::vector<double>& ra, std::vector<double>& om, std::vector<double>& ta,
                              std::vector<int>& ob) {
    const double* f = sys.f.data();
    const double* g = thermal ? sys.g_thermal.data() : nullptr;
    int k = 0;
    for (int y = 0; y < NY; y += ds) {
        for (int x = 0; x < NX; x += ds, ++k) {
            const int idx = node_index(x, y);
            if (sys.obstacle[idx]) {
                ob[k] = 1;
                if (thermal) ta[k] = T_wall;
                continue;
            }
            double rho, u, v;
            compute_macros(f + static_cast<size_t>(idx) * 9, rho, u, v);
            double T = 0.0;
            if (thermal) compute_temperature(g + static_cast<size_t>(idx) * 9, T);
            if (rho < 1e-12 || std::isnan(rho)) {
                rho = 1.0;
                u = 0.0;
                v = 0.0;
            }
            if (std::isnan(u)) u = 0.0;
            if (std::isnan(v)) v = 0.0;
            if (thermal && std::isnan(T)) T = 1.0;
            double s = std::sqrt(u * u + v * v);
            if (std::isnan(s)) s = 0.0;
            vel[k] = s;
            ua[k] = u;
            va[k] = v;
            ra[k] = rho;
            ta[k] = T;
        }
    }
    for (int j = 0; j < nyd; ++j)
        for (int i = 0; i < nxd; ++i) {
            const int idx = j * nxd + i;
            if (ob[idx]) continue;
            const int il = std::max(0, i - 1), ir = std::min(nxd - 1, i + 1);
            const int jd = std::max(0, j - 1), ju = std::min(nyd - 1, j + 1);
            const double dvdx = (va[j * nxd + ir] - va[j * nxd + il]) / (2.0 * static_cast<double>((ir - il) * ds));
            const double dudy = (ua[ju * nxd + i] - ua[jd * nxd + i]) / (2.0 * static_cast<double>((ju - jd) * ds));
            om[idx] = dvdx - dudy;
        }
}

// Downsampled macroscopic fields + vorticity, the frame format of
// src/lbm.hpp:588-701 (and :707-817 with a temperature channel).
inline void write_frame(const LBMCapabilities& sys, int step, const std::string& output_dir, bool thermal,
                        double T_wall) {
    const int ds = std::max(1, NX / 100);
    const int nxd = (NX + ds - 1) / ds, nyd = (NY + ds - 1) / ds, nd = nxd * nyd;
    const std::string dir = output_dir + "/frames";
    std::filesystem::create_directories(dir);
    std::ofstream out(dir + "/frame_" + std::to_string(step) + ".json");
    out.precision(6);
    out << std::fixed;
    std::vector<double> vel(nd, 0.0), ua(nd, 0.0), va(nd, 0.0), ra(nd, 0.0), om(nd, 0.0), ta(nd, 0.0);
    std::vector<int> ob(nd, 0);
    if (sys.device_state_current(thermal)) {
        // the same fields computed on the device; only the nd points cross
        std::vector<uint8_t> ob8(nd);
        lbm2d_solver* h = sys.device_handle();
        check(lbm2d_frame_fields(h, ds, 1, T_wall, ra.data(), ua.data(), va.data(), vel.data(), om.data(),
                                 thermal ? ta.data() : nullptr, ob8.data()),
              h, "frame fields");
        for (int i = 0; i < nd; ++i) ob[i] = ob8[i];
    } else {
        host_frame_fields(sys, ds, nxd, nyd, thermal, T_wall, vel, ua, va, ra, om, ta, ob);
    }
    auto arr = [&](const char* name, auto&& get, bool first) {
        out << (first ? "" : "],") << "\"" << name << "\":[";
        for (int i = 0; i < nd; ++i) {
            if (i > 0) out << ",";
            out << get(i);
        }
    };
    out << "{\"nx\":" << nxd << ",\"ny\":" << nyd << ",";
    arr("velocity", [&](int i) { return vel[i]; }, true);
    arr("u", [&](int i) { return ua[i]; }, false);
    arr("v", [&](int i) { return va[i]; }, false);
    arr("rho", [&](int i) { return ra[i]; }, false);
    arr("p", [&](int i) { return ra[i] / 3.0; }, false);
    arr("omega", [&](int i) { return om[i]; }, false);
    if (thermal) arr("temperature", [&](int i) { return ta[i]; }, false);
    arr("obstacle", [&](int i) { return ob[i]; }, false);
    out << "]}";
}
}  // namespace lbm2d_dropin

inline void save_json_frame(const LBMCapabilities& sys, int step, const std::string& output_dir) {
    lbm2d_dropin::write_frame(sys, step, output_dir, false, 0.0);
}

inline void save_json_frame_thermal(LBMCapabilities& sys, int step, const std::string& output_dir, double T_wall) {
    lbm2d_dropin::write_frame(sys, step, output_dir, true, T_wall);
}

// src/lbm.hpp:822-834 (one cached file handle per output directory)
inline void save_forces_jsonl(const std::string& output_dir, int step, double cd, double cl) {
    static std::string cached_dir;
    static std::ofstream out;
    if (cached_dir != output_dir) {
        if (out.is_open()) out.close();
        out.open(output_dir + "/forces.jsonl", std::ios::trunc);
        out.precision(6);
        out << std::fixed;
        cached_dir = output_dir;
    }
    out << "{\"step\":" << step << ",\"cd\":" << cd << ",\"cl\":" << cl << "}\n";
}

// Batched form of the per-step forces.jsonl stream (src/lbm.hpp:822-834 as
// called by src/main.cpp:106-122): the drag/lift sums of every step since the
// last upload are kept on the device; this reads them back once and writes
// the same lines the driver's per-step loop writes, with Cd, Cl =
// 2 F / (D u^2) (length_scale = 0 writes the raw sums, as the step, hills and
// canyon drivers do).  Returns the number of lines written.
inline int save_forces_history_jsonl(LBMCapabilities& sys, const std::string& output_dir, int first_step,
                                     double length_scale, double u_ref) {
    int n = 0;
    if (!sys.handle() || lbm2d_force_history(sys.handle(), nullptr, nullptr, 0, &n) != LBM2D_OK || n <= 0) return 0;
    std::vector<double> fx(n), fy(n);
    lbm2d_force_history(sys.handle(), fx.data(), fy.data(), n, &n);
    const double k = length_scale > 0.0 ? 2.0 / (length_scale * u_ref * u_ref) : 1.0;
    std::ofstream out(output_dir + "/forces.jsonl", std::ios::trunc);
    out.precision(6);
    out << std::fixed;
    for (int s = 0; s < n; ++s)
        out << "{\"step\":" << first_step + s << ",\"cd\":" << k * fx[s] << ",\"cl\":" << k * fy[s] << "}\n";
    return n;
}

// src/lbm.hpp:839-855
inline void save_meta_json(const std::string& output_dir, double re, double tau, double u_inflow,
                           double length_scale, const std::string& shape_type, int nx, int ny) {
    std::ofstream out(output_dir + "/meta.json");
    out.precision(6);
    out << std::fixed << "{\n"
        << "  \"nx\": " << nx << ",\n"
        << "  \"ny\": " << ny << ",\n"
        << "  \"re\": " << re << ",\n"
        << "  \"tau\": " << tau << ",\n"
        << "  \"u_inflow\": " << u_inflow << ",\n"
        << "  \"length_scale\": " << length_scale << ",\n"
        << "  \"shape_type\": \"" << shape_type << "\"\n"
        << "}\n";
}

// legacy VTK structured points, src/lbm.hpp:860-926
inline void save_vtk_frame(const LBMCapabilities& sys, int frame, const std::string& output_dir = "output") {
    std::ofstream out(output_dir + "/frame_" + std::to_string(frame) + ".vtk");
    out << "# vtk DataFile Version 3.0\nLBM Fluid Grid\nASCII\nDATASET STRUCTURED_POINTS\n";
    out << "DIMENSIONS " << NX << " " << NY << " 1\n";
    out << "ORIGIN 0 0 0\nSPACING 1 1 1\n";
    out << "POINT_DATA " << NX * NY << "\n";
    const size_t n = static_cast<size_t>(NX) * NY;
    std::vector<double> sp(n), ua(n), va(n), ra(n);
    std::vector<uint8_t> ob(n);
    if (sys.device_state_current(false)) {
        // full-resolution raw fields from the device (no NaN replacement)
        lbm2d_solver* h = sys.device_handle();
        lbm2d_dropin::check(lbm2d_frame_fields(h, 1, 0, 0.0, ra.data(), ua.data(), va.data(), sp.data(), nullptr,
                                               nullptr, ob.data()),
                            h, "frame fields");
    } else {
        const double* f = sys.f.data();
        for (size_t idx = 0; idx < n; ++idx) {
            ob[idx] = sys.obstacle[idx] ? 1 : 0;
            if (ob[idx]) continue;
            compute_macros(f + idx * 9, ra[idx], ua[idx], va[idx]);
            sp[idx] = std::sqrt(ua[idx] * ua[idx] + va[idx] * va[idx]);
        }
    }
    out << "SCALARS VelocityMagnitude double 1\nLOOKUP_TABLE default\n";
    for (size_t idx = 0; idx < n; ++idx) {
        if (ob[idx])
            out << "0.0\n";
        else
            out << sp[idx] << "\n";
    }
    out << "VECTORS Velocity double\n";
    for (size_t idx = 0; idx < n; ++idx) {
        if (ob[idx])
            out << "0 0 0\n";
        else
            out << ua[idx] << " " << va[idx] << " 0\n";
    }
    out << "SCALARS Density double 1\nLOOKUP_TABLE default\n";
    for (size_t idx = 0; idx < n; ++idx) {
        if (ob[idx])
            out << "0.0\n";
        else
            out << ra[idx] << "\n";
    }
    out << "SCALARS DragForce double 1\nLOOKUP_TABLE default\n";
    for (size_t idx = 0; idx < n; ++idx) {
        const double fx = sys.fx_body[idx], fy = sys.fy_body[idx];
        if (fx != 0.0 || fy != 0.0)
            out << fx << "\n";
        else
            out << "0.0\n";
    }
}
