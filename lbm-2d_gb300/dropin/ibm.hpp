// ibm.hpp -- drop-in replacement of the reference's src/ibm.hpp.
//
// The immersed-boundary helpers keep the reference's names and host
// semantics (Lagrangian points from a polygon, 4-point cosine delta, force
// spreading, velocity interpolation, no-slip direct forcing), so a driver
// that runs the reference's loop on the host mirrors compiles and behaves as
// before.  lbm2d_dropin::attach_ibm moves that loop to the device instead
// (lbm2d_set_ibm): the driver then calls execute_time_step alone.
#pragma once
#include <algorithm>
#include <cmath>
#include <utility>
#include <vector>

#include "lbm_types.hpp"

// src/ibm.hpp:16-19: 4-point smoothed delta, 0 for |r| >= 2
inline double ibm_delta(double r) {
    if (std::abs(r) >= 2.0) return 0.0;
    return 0.25 * (1.0 + std::cos(0.5 * M_PI * r));
}

// src/ibm.hpp:22-24: tensor-product kernel
inline double ibm_kernel(double dx, double dy) { return ibm_delta(dx) * ibm_delta(dy); }

// src/ibm.hpp:27-34
struct LagrangianPoint {
    double X;
    double Y;
    double FX = 0;
    double FY = 0;
    double U = 0;
    double V = 0;
};

// src/ibm.hpp:37-150
struct ImmersedBoundary {
    std::vector<LagrangianPoint> points;
    std::vector<std::pair<double, double>> surface;

    // max(8, perimeter / spacing) points, uniform in the vertex parameter
    // (the same arithmetic as lbm2d_ibm_points_from_polygon).
    void build_from_polygon(const std::vector<std::pair<double, double>>& poly, double spacing = 1.0) {
        surface = poly;
        points.clear();
        std::vector<double> xy;
        for (const auto& p : poly) {
            xy.push_back(p.first);
            xy.push_back(p.second);
        }
        const int n = static_cast<int>(poly.size());
        const int np = lbm2d_ibm_points_from_polygon(xy.data(), n, spacing, nullptr, nullptr, 0);
        std::vector<double> X(np), Y(np);
        lbm2d_ibm_points_from_polygon(xy.data(), n, spacing, X.data(), Y.data(), np);
        for (int k = 0; k < np; ++k) points.push_back({X[k], Y[k], 0, 0, 0, 0});
    }

    // Visit the 5x5 stencil of point p: in-grid nodes with a non-zero weight,
    // y-major, as the reference loops.
    template <class Fn>
    void for_stencil(size_t p, int nx, int ny, Fn&& fn) const {
        const double X = points[p].X, Y = points[p].Y;
        const int x0 = static_cast<int>(std::floor(X)) - 2, x1 = static_cast<int>(std::floor(X)) + 2;
        const int y0 = static_cast<int>(std::floor(Y)) - 2, y1 = static_cast<int>(std::floor(Y)) + 2;
        for (int y = std::max(y0, 0); y <= std::min(y1, ny - 1); ++y)
            for (int x = std::max(x0, 0); x <= std::min(x1, nx - 1); ++x) {
                const double k = ibm_kernel(x - X, y - Y);
                if (k != 0.0) fn(y * nx + x, k);
            }
    }

    // Adds fx_lag[p] * kernel to the grid force of every stencil node, points
    // in order.
    void spread_force(const std::vector<double>& fx_lag, const std::vector<double>& fy_lag,
                      std::vector<double>& fx_grid, std::vector<double>& fy_grid, int nx, int ny) const {
        for (size_t p = 0; p < points.size(); ++p)
            for_stencil(p, nx, ny, [&](int idx, double k) {
                fx_grid[idx] += fx_lag[p] * k;
                fy_grid[idx] += fy_lag[p] * k;
            });
    }

    // Kernel-weighted grid velocity at every point (all stencil nodes).
    void interpolate_velocity(const std::vector<double>& u_grid, const std::vector<double>& v_grid, int nx, int ny) {
        for (size_t p = 0; p < points.size(); ++p) {
            double u = 0, v = 0;
            for_stencil(p, nx, ny, [&](int idx, double k) {
                u += u_grid[idx] * k;
                v += v_grid[idx] * k;
            });
            points[p].U = u;
            points[p].V = v;
        }
    }

    // Direct forcing toward the wall velocity: (U_wall - U) / dt.
    void compute_no_slip_force(double dt, std::vector<double>& fx_lag, std::vector<double>& fy_lag,
                               double u_wall_x = 0.0, double u_wall_y = 0.0) const {
        fx_lag.resize(points.size());
        fy_lag.resize(points.size());
        for (size_t p = 0; p < points.size(); ++p) {
            fx_lag[p] = (u_wall_x - points[p].U) / dt;
            fy_lag[p] = (u_wall_y - points[p].V) / dt;
        }
    }
};

namespace lbm2d_dropin {
// Run the airfoil driver's immersed-boundary loop (src/airfoil_ibm.cpp:
// 121-176: interpolation from the fluid nodes, no-slip force, spreading, the
// step, explicit forcing) on the device around every execute_time_step of
// `sys`.  An empty boundary detaches it.
inline void attach_ibm(LBMCapabilities& sys, const ImmersedBoundary& ib, double dt = 1.0, double u_wall_x = 0.0,
                       double u_wall_y = 0.0) {
    std::vector<double> X, Y;
    for (const auto& p : ib.points) {
        X.push_back(p.X);
        Y.push_back(p.Y);
    }
    sys.set_ibm_points(std::move(X), std::move(Y), dt, u_wall_x, u_wall_y);
}

// Copy the device's Lagrangian velocities and forces (those that produced
// the forcing of the last step) into ib.points[].U, V, FX, FY.
inline void ibm_lagrangian(LBMCapabilities& sys, ImmersedBoundary& ib) {
    const size_t n = ib.points.size();
    std::vector<double> U(n), V(n), FX(n), FY(n);
    check(lbm2d_ibm_lagrangian(sys.handle(), U.data(), V.data(), FX.data(), FY.data()), sys.handle(),
          "immersed boundary");
    for (size_t p = 0; p < n; ++p) {
        ib.points[p].U = U[p];
        ib.points[p].V = V[p];
        ib.points[p].FX = FX[p];
        ib.points[p].FY = FY[p];
    }
}
}  // namespace lbm2d_dropin
