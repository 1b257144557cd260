// lbm2d_host.cpp -- host services of the C-ABI: the reference's set-up
// arithmetic (masks, NACA profiles, point-in-polygon, wall distance, link
// list).  Compiled with -ffp-contract=off so every double expression rounds
// exactly as the reference's does; evaluation order follows the cited lines.
#include <cmath>
#include <vector>

#include "../../include/lbm2d.h"
#include "lbm2d_geometry.h"
#include "lbm2d_internal.h"

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

namespace {
constexpr int CX[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
constexpr int CY[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};
constexpr int BB[9] = {0, 3, 4, 1, 2, 7, 8, 5, 6};
constexpr double W[9] = {4.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0,
                         1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0};
}  // namespace

extern "C" {

double lbm2d_equilibrium(int i, double rho, double u, double v) {
    if (i < 0 || i > 8) return 0.0;
    const double ed = CX[i] * u + CY[i] * v;
    const double usq = u * u + v * v;
    return W[i] * rho * (1.0 + 3.0 * ed + 4.5 * ed * ed - 1.5 * usq);
}

int lbm2d_mask_walls(int nx, int ny, uint8_t* mask) {
    if (nx < 1 || ny < 1 || !mask) return LBM2D_ERR_INVALID;
    for (int x = 0; x < nx; ++x) mask[x] = 1;
    for (int y = 0; y < ny; ++y) {
        mask[(size_t)y * nx] = 1;
        mask[(size_t)y * nx + nx - 1] = 1;
    }
    return LBM2D_OK;
}

int lbm2d_mask_cylinder(int nx, int ny, uint8_t* mask, int cx, int cy, int radius) {
    if (nx < 1 || ny < 1 || !mask) return LBM2D_ERR_INVALID;
    for (int y = 0; y < ny; ++y)
        for (int x = 0; x < nx; ++x) {
            const double dx = static_cast<double>(x - cx), dy = static_cast<double>(y - cy);
            if (std::sqrt(dx * dx + dy * dy) < radius) mask[(size_t)y * nx + x] = 1;
        }
    return LBM2D_OK;
}

int lbm2d_point_in_polygon(double px, double py, const double* xy, int n) {
    if (!xy || n < 1) return 0;
    bool inside = false;
    for (int i = 0, j = n - 1; i < n; j = i++) {
        const double xi = xy[2 * i], yi = xy[2 * i + 1];
        const double xj = xy[2 * j], yj = xy[2 * j + 1];
        const bool hit = ((yi > py) != (yj > py)) && (px < (xj - xi) * (py - yi) / (yj - yi) + xi);
        if (hit) inside = !inside;
    }
    return inside ? 1 : 0;
}

int lbm2d_mask_polygon(int nx, int ny, uint8_t* mask, const double* xy, int n) {
    if (nx < 1 || ny < 1 || !mask || (n > 0 && !xy)) return LBM2D_ERR_INVALID;
    for (int y = 0; y < ny; ++y)
        for (int x = 0; x < nx; ++x)
            if (lbm2d_point_in_polygon(static_cast<double>(x), static_cast<double>(y), xy, n))
                mask[(size_t)y * nx + x] = 1;
    return LBM2D_OK;
}

int lbm2d_naca_coords(int series, int n, double* out) {
    if (n < 2 || !out) return 0;
    const int m_code = series / 1000, p_code = (series / 100) % 10, t_code = series % 100;
    const double m = static_cast<double>(m_code) / 100.0;
    const double p = static_cast<double>(p_code) / 10.0;
    const double t = static_cast<double>(t_code) / 100.0;
    std::vector<double> x(n), yt(n), yc(n, 0.0), dyc(n, 0.0);
    for (int i = 0; i < n; ++i) {
        const double beta = static_cast<double>(i) / (n - 1) * M_PI;
        x[i] = (1.0 - std::cos(beta)) / 2.0;
    }
    for (int i = 0; i < n; ++i)
        yt[i] = 5.0 * t *
                (0.2969 * std::sqrt(x[i]) - 0.1260 * x[i] - 0.3516 * x[i] * x[i] + 0.2843 * x[i] * x[i] * x[i] -
                 0.1015 * x[i] * x[i] * x[i] * x[i]);
    if (m > 1e-10 && p > 1e-10) {
        for (int i = 0; i < n; ++i) {
            if (x[i] < p) {
                yc[i] = (m / (p * p)) * (2.0 * p * x[i] - x[i] * x[i]);
                dyc[i] = (2.0 * m / (p * p)) * (p - x[i]);
            } else {
                yc[i] = (m / ((1.0 - p) * (1.0 - p))) * ((1.0 - 2.0 * p) + 2.0 * p * x[i] - x[i] * x[i]);
                dyc[i] = (2.0 * m / ((1.0 - p) * (1.0 - p))) * (p - x[i]);
            }
        }
    }
    int k = 0;
    for (int i = n - 1; i >= 0; --i) {  // upper surface, trailing edge -> leading edge
        const double th = std::atan(dyc[i]);
        out[2 * k] = x[i] - yt[i] * std::sin(th);
        out[2 * k + 1] = yc[i] + yt[i] * std::cos(th);
        ++k;
    }
    for (int i = 1; i < n; ++i) {  // lower surface, leading edge -> trailing edge
        const double th = std::atan(dyc[i]);
        out[2 * k] = x[i] + yt[i] * std::sin(th);
        out[2 * k + 1] = yc[i] - yt[i] * std::cos(th);
        ++k;
    }
    return k;
}

int lbm2d_transform_points(double* xy, int n, double cx, double cy, double scale, double angle_deg) {
    if (n < 0 || (n > 0 && !xy)) return LBM2D_ERR_INVALID;
    const double a = angle_deg * M_PI / 180.0;
    const double ca = std::cos(a), sa = std::sin(a);
    for (int k = 0; k < n; ++k) {
        const double xs = xy[2 * k] * scale, ys = xy[2 * k + 1] * scale;
        const double xr = xs * ca - ys * sa;
        const double yr = xs * sa + ys * ca;
        xy[2 * k] = xr + cx;
        xy[2 * k + 1] = yr + cy;
    }
    return LBM2D_OK;
}

int lbm2d_wall_distance(int nx, int ny, const uint8_t* mask, double* wd) {
    if (nx < 1 || ny < 1 || !mask || !wd) return LBM2D_ERR_INVALID;
    std::vector<double> d;
    lbm2d::wall_distance(nx, ny, mask, d);
    for (size_t k = 0; k < d.size(); ++k) wd[k] = d[k];
    return LBM2D_OK;
}

int lbm2d_force_stats(const double* v1, const double* v2, int n, double dt, lbm2d_force_stats_t* out) {
    if (!v1 || !v2 || !out || n < 0) return LBM2D_ERR_INVALID;
    int n_skip = static_cast<int>(n * 0.2);  // main(): skip the first 20% as transient
    if (n_skip < 10) n_skip = 0;
    double s1 = 0.0, s2 = 0.0;
    const int m = n - n_skip;
    for (int k = n_skip; k < n; ++k) {
        s1 += v1[k];
        s2 += v2[k];
    }
    out->mean_v1 = m > 0 ? s1 / m : NAN;
    out->mean_v2 = m > 0 ? s2 / m : NAN;
    double var = 0.0;
    for (int k = n_skip; k < n; ++k) var += (v2[k] - out->mean_v2) * (v2[k] - out->mean_v2);
    out->std_v2 = m > 0 ? std::sqrt(var / m) : NAN;
    out->n_skip = n_skip;
    // compute_strouhal: zero crossings of the mean after a 40% transient
    out->st = NAN;
    if (n >= 200) {
        int skip = static_cast<int>(n * 0.4);
        if (skip < 50) skip = 50;
        const int len = n - skip;
        if (len >= 100) {
            double mean = 0.0;
            for (int k = skip; k < n; ++k) mean += v2[k];
            mean /= len;
            int crossings = 0;
            for (int k = skip + 1; k < n; ++k)
                if (v2[k - 1] < mean && v2[k] >= mean) ++crossings;
            if (crossings >= 2) out->st = crossings / (2.0 * (len * dt));
        }
    }
    return LBM2D_OK;
}

int lbm2d_boundary_links(int nx, int ny, int case_type, const uint8_t* mask, const lbm2d_bb_geometry* geom,
                         int capacity, int32_t* node, int8_t* dir, int8_t* kind, double* q, double* uwx, double* uwy,
                         int8_t* counts_force, int* count) {
    if (nx < 3 || ny < 3 || !mask || !count) return LBM2D_ERR_INVALID;
    lbm2d::BBGeometry bb;
    if (geom) {
        bb.cx = geom->cx;
        bb.cy = geom->cy;
        bb.radius = geom->radius;
        if (geom->poly && geom->n_poly > 0) {
            bb.poly.assign(geom->poly, geom->poly + 2 * (size_t)geom->n_poly);
            bb.is_polygon = true;
        }
        bb.has_moving_wall = geom->has_moving_wall != 0;
        bb.omega = geom->omega;
        bb.rot_cx = geom->rot_cx;
        bb.rot_cy = geom->rot_cy;
    }
    lbm2d::GeometryInput in;
    in.nx = nx;
    in.ny = ny;
    in.case_type = case_type;
    in.mask = mask;
    in.bb = &bb;
    lbm2d::GeometryTables t;
    std::string err;
    if (!lbm2d::build_geometry(in, t, err)) return LBM2D_ERR_INVALID;
    int c = 0;
    for (size_t r = 0; r < t.rec_info.size(); ++r) {
        const uint32_t types = t.rec_info[r];
        for (int i = 1; i < 9; ++i) {  // reference link order per node
            const int j = BB[i];
            const uint32_t st = (types >> (2 * j)) & 3u;
            if (st == lbm2d::SLOT_REGULAR) continue;
            if (c < capacity) {
                if (node) node[c] = t.rec_node[r];
                if (dir) dir[c] = static_cast<int8_t>(i);
                if (kind) kind[c] = static_cast<int8_t>(st);
                if (q) q[c] = t.rec_q[r * 9 + j];
                if (uwx) uwx[c] = t.rec_uw[(r * 9 + j) * 2];
                if (uwy) uwy[c] = t.rec_uw[(r * 9 + j) * 2 + 1];
                if (counts_force) counts_force[c] = (t.rec_force[r] >> j) & 1u ? 1 : 0;
            }
            ++c;
        }
    }
    *count = c;
    return LBM2D_OK;
}

}  // extern "C"
