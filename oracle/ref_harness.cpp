// ref_harness.cpp -- drives the UNMODIFIED reference solver headers.
//
// TEST INFRASTRUCTURE ONLY.  Compiled by oracle/Makefile against the lbm-2d
// sources where they lie (include path to the reference's src/), into
// oracle/_ref/libref.so, never into the product.  It exposes the same call
// surface as oracle/lbm_oracle.c (prefix ref_ instead of or_) so the fixture
// generator can run one case on both and compare.
//
// The reference keeps its grid size and case selection in process globals
// (src/lbm_types.hpp:15-32), so this harness holds one solver at a time.
#include "lbm.hpp"

#include <cstring>
#include <random>
#include <vector>

static LBMCapabilities* g_sys = nullptr;

extern "C" {

int ref_create(int nx, int ny) {
    delete g_sys;
    NX = nx;
    NY = ny;
    g_case = CaseType::CYLINDER;
    g_collision = CollisionType::MRT;
    g_use_les = false;
    g_cs = 0.12;
    g_sys = new LBMCapabilities();
    return 0;
}

void ref_destroy() {
    delete g_sys;
    g_sys = nullptr;
}

void ref_set_case(int case_type, int collision, int use_les, double cs) {
    g_case = static_cast<CaseType>(case_type);
    g_collision = collision == 0 ? CollisionType::MRT : CollisionType::BGK;
    g_use_les = use_les != 0;
    g_cs = cs;
}

void ref_set_thermal(int use, double T_ref, double alpha, double omega_k, double beta, double g_buoyancy) {
    g_sys->use_thermal = use != 0;
    g_sys->T_ref = T_ref;
    g_sys->alpha = alpha;
    g_sys->omega_k = omega_k;
    g_sys->beta = beta;
    g_sys->g_buoyancy = g_buoyancy;
}

void ref_set_body_force(double fx) { g_sys->body_force_x = fx; }

void ref_set_moving_wall(int on, double omega, double rcx, double rcy) {
    g_sys->bb_geom.has_moving_wall = on != 0;
    g_sys->bb_geom.omega = omega;
    g_sys->bb_geom.rot_cx = rcx;
    g_sys->bb_geom.rot_cy = rcy;
}

void ref_set_mei(int on) { g_sys->bb_geom.use_mei_bb = on != 0; }

double* ref_f() { return g_sys->f.data(); }
double* ref_g() { return g_sys->g_thermal.data(); }
double* ref_fx() { return g_sys->fx_body.data(); }
double* ref_fy() { return g_sys->fy_body.data(); }
double* ref_wall_dist() { return g_sys->wall_dist.data(); }
uint8_t* ref_obstacle() { return g_sys->obstacle.data(); }

void ref_place_walls() { place_walls(*g_sys); }
void ref_place_cylinder(int cx_, int cy_, int r) { place_cylinder(*g_sys, cx_, cy_, r); }
void ref_place_polygon(const double* xy, int n) {
    std::vector<std::pair<double, double>> p(n);
    for (int k = 0; k < n; ++k) p[k] = {xy[2 * k], xy[2 * k + 1]};
    place_polygon(*g_sys, p);
}
void ref_compute_wall_distance() { compute_wall_distance(*g_sys); }
double ref_compute_q(double xf, double yf, int i) { return g_sys->bb_geom.compute_q(xf, yf, i); }

int ref_naca_coords(int series, int n, double* out) {
    auto p = naca_coords(series, n);
    for (size_t k = 0; k < p.size(); ++k) {
        out[2 * k] = p[k].first;
        out[2 * k + 1] = p[k].second;
    }
    return static_cast<int>(p.size());
}

void ref_transform_points(double* xy, int n, double cx_, double cy_, double scale, double angle_deg) {
    std::vector<std::pair<double, double>> p(n);
    for (int k = 0; k < n; ++k) p[k] = {xy[2 * k], xy[2 * k + 1]};
    transform_points(p, cx_, cy_, scale, angle_deg);
    for (int k = 0; k < n; ++k) {
        xy[2 * k] = p[k].first;
        xy[2 * k + 1] = p[k].second;
    }
}

int ref_point_in_polygon(double px, double py, const double* xy, int n) {
    std::vector<std::pair<double, double>> p(n);
    for (int k = 0; k < n; ++k) p[k] = {xy[2 * k], xy[2 * k + 1]};
    return point_in_polygon(px, py, p) ? 1 : 0;
}

double ref_equilibrium(int i, double rho, double u, double v) { return compute_equilibrium(i, rho, u, v); }

void ref_step(double tau, double u_in) { execute_time_step(*g_sys, tau, u_in); }

// Driver-side force sum in node order (as src/main.cpp:106-110).
void ref_force_sums(double* fx_total, double* fy_total) {
    double a = 0.0, b = 0.0;
    for (int n = 0; n < NX * NY; ++n) {
        a += g_sys->fx_body[n];
        b += g_sys->fy_body[n];
    }
    *fx_total = a;
    *fy_total = b;
}

// The drivers' post-step thermal passes, written out as the drivers do them.
// kind 1: src/thermal_cavity.cpp:168-204; kind 2: src/heated_cylinder.cpp:156-164.
void ref_thermal_hook(int kind, double Ta, double Tb) {
    LBMCapabilities& system = *g_sys;
    if (kind == 1) {
        for (int y = 1; y < NY - 1; ++y) {
            {
                int idx = node_index(1, y);
                double rho, u, v;
                compute_macros(&system.f[idx * 9], rho, u, v);
                for (int i = 0; i < 9; ++i) system.g_thermal[idx * 9 + i] = thermal_equilibrium(i, Ta, u, v);
            }
            {
                int idx = node_index(NX - 2, y);
                double rho, u, v;
                compute_macros(&system.f[idx * 9], rho, u, v);
                for (int i = 0; i < 9; ++i) system.g_thermal[idx * 9 + i] = thermal_equilibrium(i, Tb, u, v);
            }
        }
        for (int x = 1; x < NX - 1; ++x) {
            for (int yy : {1, NY - 2}) {
                int idx = node_index(x, yy);
                for (int i = 0; i < 9; ++i) system.g_thermal[idx * 9 + i] = system.g_thermal[idx * 9 + bounce_back[i]];
            }
        }
    } else if (kind == 2) {
        for (int n = 0; n < NX * NY; ++n)
            if (system.obstacle[n]) apply_thermal_isothermal(&system.g_thermal[n * 9], Ta);
    }
}

// Initial state of the cylinder-wake driver (src/main.cpp:60-83) with the
// standard library generator the driver uses.
void ref_init_cylinder_wake(double u_in, int cx_cyl, unsigned seed, double amp) {
    LBMCapabilities& system = *g_sys;
    for (int n = 0; n < NX * NY; ++n)
        for (int i = 0; i < 9; ++i) system.f[n * 9 + i] = compute_equilibrium(i, 1.0, u_in, 0.0);
    std::mt19937 rng(seed);
    std::uniform_real_distribution<double> pert(-amp, amp);
    for (int x = cx_cyl + 5; x < std::min(NX, cx_cyl + 60); ++x) {
        for (int y = 0; y < NY; ++y) {
            int n = node_index(x, y);
            if (system.obstacle[n]) continue;
            double* fn = &system.f[n * 9];
            double vp = pert(rng);
            double rho, u, v;
            compute_macros(fn, rho, u, v);
            for (int i = 0; i < 9; ++i) fn[i] = compute_equilibrium(i, rho, u, v + vp);
        }
    }
}

void ref_init_uniform(double rho, double u, double v) {
    for (int n = 0; n < NX * NY; ++n)
        for (int i = 0; i < 9; ++i) g_sys->f[n * 9 + i] = compute_equilibrium(i, rho, u, v);
}

void ref_init_thermal_uniform(double T, double u, double v) {
    for (int n = 0; n < NX * NY; ++n)
        for (int i = 0; i < 9; ++i) g_sys->g_thermal[n * 9 + i] = thermal_equilibrium(i, T, u, v);
}

// ---- immersed boundary (src/ibm.hpp) driven as src/airfoil_ibm.cpp:121-176 does
static ImmersedBoundary g_ibm;
static std::vector<double> g_fx_lag, g_fy_lag;
static double g_ibm_dt = 1.0;

int ref_ibm_from_polygon(const double* xy, int n, double spacing) {
    std::vector<std::pair<double, double>> p(n);
    for (int k = 0; k < n; ++k) p[k] = {xy[2 * k], xy[2 * k + 1]};
    g_ibm = ImmersedBoundary();
    g_ibm.build_from_polygon(p, spacing);
    g_fx_lag.assign(g_ibm.points.size(), 0.0);
    g_fy_lag.assign(g_ibm.points.size(), 0.0);
    return static_cast<int>(g_ibm.points.size());
}

void ref_ibm_points(double* X, double* Y) {
    for (size_t p = 0; p < g_ibm.points.size(); ++p) {
        X[p] = g_ibm.points[p].X;
        Y[p] = g_ibm.points[p].Y;
    }
}

void ref_ibm_set_dt(double dt) { g_ibm_dt = dt; }

double ref_ibm_kernel(double dx, double dy) { return ibm_kernel(dx, dy); }

// One iteration of the airfoil driver's loop: interpolate the velocity at the
// Lagrangian points (fluid nodes only), no-slip force, spread, step, then the
// explicit forcing of the fluid nodes.
void ref_ibm_step(double tau, double u_inflow) {
    LBMCapabilities& system = *g_sys;
    ImmersedBoundary& iboundary = g_ibm;
    for (size_t p = 0; p < iboundary.points.size(); ++p) {
        double X = iboundary.points[p].X;
        double Y = iboundary.points[p].Y;
        double u = 0, v = 0;
        int x0 = static_cast<int>(std::floor(X)) - 2;
        int x1 = static_cast<int>(std::floor(X)) + 2;
        int y0 = static_cast<int>(std::floor(Y)) - 2;
        int y1 = static_cast<int>(std::floor(Y)) + 2;
        for (int y = y0; y <= y1; ++y) {
            if (y < 0 || y >= NY) continue;
            for (int x = x0; x <= x1; ++x) {
                if (x < 0 || x >= NX) continue;
                double kernel = ibm_kernel(x - X, y - Y);
                if (kernel == 0.0) continue;
                int idx = node_index(x, y);
                if (system.obstacle[idx]) continue;
                double rho, uu, vv;
                compute_macros(&system.f[idx * 9], rho, uu, vv);
                u += uu * kernel;
                v += vv * kernel;
            }
        }
        iboundary.points[p].U = u;
        iboundary.points[p].V = v;
    }
    iboundary.compute_no_slip_force(g_ibm_dt, g_fx_lag, g_fy_lag);
    std::vector<double> fx_grid(NX * NY, 0.0), fy_grid(NX * NY, 0.0);
    iboundary.spread_force(g_fx_lag, g_fy_lag, fx_grid, fy_grid, NX, NY);
    execute_time_step(system, tau, u_inflow);
    for (int y = 0; y < NY; ++y) {
        for (int x = 0; x < NX; ++x) {
            int idx = node_index(x, y);
            if (system.obstacle[idx]) continue;
            double* f_node = &system.f[idx * 9];
            double fx = fx_grid[idx];
            double fy = fy_grid[idx];
            for (int i = 0; i < 9; ++i) {
                double edotu = cx[i] * 0 + cy[i] * 0;
                double Fdot = cx[i] * fx + cy[i] * fy;
                double correction = weights[i] * (3.0 * Fdot + 9.0 * edotu * (cx[i] * fx + cy[i] * fy));
                f_node[i] += correction;
            }
        }
    }
}

// Lagrangian velocities and forces of the last ref_ibm_step.
void ref_ibm_lagrangian(double* U, double* V, double* FX, double* FY) {
    for (size_t p = 0; p < g_ibm.points.size(); ++p) {
        U[p] = g_ibm.points[p].U;
        V[p] = g_ibm.points[p].V;
        FX[p] = g_fx_lag[p];
        FY[p] = g_fy_lag[p];
    }
}

}  // extern "C"
