/*
 * lbm_oracle.c -- CPU restatement of the lbm-2d D2Q9 time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle and the timed CPU
 * baseline ("port").  It is never linked into the product library and the
 * product path never calls it.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py load it.
 *
 * It restates, in plain C, the arithmetic of the reference solver so that a
 * run here is bit-identical to the reference compiled from its own headers
 * (both built with -ffp-contract=off).  Parity of this restatement is pinned
 * against fixtures produced by the reference itself (tests/golden/).
 *
 * Every function cites the reference file:line it follows (paths are relative
 * to the lbm-2d project root).  Floating-point expressions keep the reference's
 * evaluation order on purpose: that order is what makes the results bit-exact.
 *
 * Layout follows the reference: populations are FP64, array-of-structures,
 * f[node*9 + i], node = y*nx + x (src/lbm_types.hpp:82-84, :188).
 */
#define _GNU_SOURCE
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* Case and collision enums: same numbering as src/lbm_types.hpp:20-27. */
enum {
    OR_CYLINDER = 0, OR_CAVITY = 1, OR_STEP = 2, OR_RIBS = 3, OR_URBAN_CANYON = 4,
    OR_DOWNWASH = 5, OR_SQUARE_CYLINDER = 6, OR_FLAT_PLATE = 7, OR_SPORTS_BALL = 8,
    OR_PERIODIC_HILLS = 9, OR_CYLINDER_NEAR_WALL = 10, OR_SIDE_BY_SIDE = 11,
    OR_ROTATING_CYLINDER = 12, OR_ORIFICE_PLATE = 13
};
enum { OR_MRT = 0, OR_BGK = 1 };

/* D2Q9 lattice: src/lbm_types.hpp:41-55.  Direction order 0..8 =
 * rest, E, N, W, S, NE, NW, SW, SE. */
static const int OR_CX[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
static const int OR_CY[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};
static const double OR_W[9] = {4.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0,
                               1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0};
static const int OR_BB[9] = {0, 3, 4, 1, 2, 7, 8, 5, 6};

/* Solver state: mirrors LBMCapabilities (src/lbm_types.hpp:187-224) plus the
 * process-global knobs of src/lbm_types.hpp:15-32, held per instance. */
typedef struct {
    int nx, ny;
    int case_type, collision, use_les;
    double cs;
    double *f, *f_next, *g, *g_next, *wall_dist, *fx, *fy;
    uint8_t *obstacle;
    int use_thermal;
    double T_ref, alpha, omega_k, beta, g_buoyancy;
    double body_force_x;
    /* BounceBackGeometry, src/lbm_types.hpp:90-182 */
    double bb_cx, bb_cy, bb_radius;
    double *poly; /* x0,y0,x1,y1,... */
    int npoly, is_polygon;
    int has_moving_wall;
    double omega, rot_cx, rot_cy;
    int use_mei_bb;
    /* immersed boundary (src/ibm.hpp:27-38), driven as src/airfoil_ibm.cpp */
    int ibm_n;
    double *ibm_X, *ibm_Y, *ibm_U, *ibm_V, *ibm_FX, *ibm_FY;
    double ibm_dt, ibm_uwx, ibm_uwy;
} or_state;

static inline int nidx(const or_state *s, int x, int y) { return y * s->nx + x; }

/* ---------------------------------------------------------------- lattice math */

/* compute_equilibrium, src/lbm_types.hpp:269-273 */
double or_equilibrium(int i, double rho, double u, double v) {
    double ed = OR_CX[i] * u + OR_CY[i] * v;
    double usq = u * u + v * v;
    return OR_W[i] * rho * (1.0 + 3.0 * ed + 4.5 * ed * ed - 1.5 * usq);
}

/* compute_macros, src/lbm_types.hpp:278-288 */
void or_macros(const double *fn, double *rho_out, double *u_out, double *v_out) {
    double rho = 0.0, mx = 0.0, my = 0.0;
    for (int i = 0; i < 9; ++i) {
        rho += fn[i];
        mx += fn[i] * OR_CX[i];
        my += fn[i] * OR_CY[i];
    }
    *rho_out = rho;
    *u_out = mx / rho;
    *v_out = my / rho;
}

static inline double or_clamp_rate(double x) { return (x < 0.5) ? 0.5 : ((x > 1.99) ? 1.99 : x); }

/* MRTParams::from_tau, src/lbm_types.hpp:72-76: s_shear, s_bulk, s_normal */
void or_mrt_params(double tau, double *s_shear, double *s_bulk, double *s_normal) {
    *s_shear = or_clamp_rate(1.0 / tau);
    *s_bulk = 1.2;
    *s_normal = 1.0;
}

/* mrt_collide, src/lbm.hpp:128-218 (moment transform, Smagorinsky :158-166,
 * Van Driest :171-182, relaxation :185-190, closed-form inverse :193-217). */
void or_mrt_collide(double *fn, double rho, double u, double v, double s_shear, double s_bulk,
                    double s_normal, double cs_sq, double tau_base, double y_plus) {
    const double f0 = fn[0], f1 = fn[1], f2 = fn[2], f3 = fn[3], f4 = fn[4];
    const double f5 = fn[5], f6 = fn[6], f7 = fn[7], f8 = fn[8];

    double m_e = -4 * f0 - f1 - f2 - f3 - f4 + 2 * (f5 + f6 + f7 + f8);
    double m_eps = 4 * f0 - 2 * (f1 + f2 + f3 + f4) + (f5 + f6 + f7 + f8);
    double m_qx = -2 * f1 + 2 * f3 + f5 - f6 - f7 + f8;
    double m_qy = -2 * f2 + 2 * f4 + f5 + f6 - f7 - f8;
    double m_pxx = f1 - f2 + f3 - f4;
    double m_pxy = f5 - f6 + f7 - f8;

    const double jx = rho * u, jy = rho * v;
    const double usq = u * u + v * v;
    const double e_eq = -2 * rho + 3 * rho * usq;
    const double eps_eq = rho - 3 * rho * usq;
    const double qx_eq = -jx, qy_eq = -jy;
    const double pxx_eq = rho * (u * u - v * v);
    const double pxy_eq = rho * u * v;

    double s_eff = s_shear;
    if (cs_sq > 0.0 && tau_base > 0.0) {
        double a = m_pxx - pxx_eq, b = m_pxy - pxy_eq;
        double Q = sqrt(2.0 * (a * a + b * b));
        double A = 9.0 * cs_sq * Q / (2.0 * rho);
        double tau_eff = (tau_base + sqrt(tau_base * tau_base + 4.0 * A)) / 2.0;
        s_eff = or_clamp_rate(1.0 / tau_eff);
    }
    if (cs_sq > 0.0 && tau_base > 0.0 && y_plus > 0.0) {
        double damp = 1.0 - exp(-y_plus / 26.0);
        double csd = sqrt(cs_sq) * damp;
        double csd_sq = csd * csd;
        double a = m_pxx - pxx_eq, b = m_pxy - pxy_eq;
        double Q = sqrt(2.0 * (a * a + b * b));
        double A = 9.0 * csd_sq * Q / (2.0 * rho);
        double tau_d = (tau_base + sqrt(tau_base * tau_base + 4.0 * A)) / 2.0;
        s_eff = or_clamp_rate(1.0 / tau_d);
    }

    m_e -= s_bulk * (m_e - e_eq);
    m_eps -= s_bulk * (m_eps - eps_eq);
    m_qx -= s_normal * (m_qx - qx_eq);
    m_qy -= s_normal * (m_qy - qy_eq);
    m_pxx -= s_eff * (m_pxx - pxx_eq);
    m_pxy -= s_eff * (m_pxy - pxy_eq);

    fn[0] = (1.0 / 9.0) * rho + (-1.0 / 9.0) * m_e + (1.0 / 9.0) * m_eps;
    fn[1] = (1.0 / 9.0) * rho + (-1.0 / 36.0) * m_e + (-1.0 / 18.0) * m_eps + (1.0 / 6.0) * jx +
            (-1.0 / 6.0) * m_qx + (1.0 / 4.0) * m_pxx;
    fn[2] = (1.0 / 9.0) * rho + (-1.0 / 36.0) * m_e + (-1.0 / 18.0) * m_eps + (1.0 / 6.0) * jy +
            (-1.0 / 6.0) * m_qy + (-1.0 / 4.0) * m_pxx;
    fn[3] = (1.0 / 9.0) * rho + (-1.0 / 36.0) * m_e + (-1.0 / 18.0) * m_eps + (-1.0 / 6.0) * jx +
            (1.0 / 6.0) * m_qx + (1.0 / 4.0) * m_pxx;
    fn[4] = (1.0 / 9.0) * rho + (-1.0 / 36.0) * m_e + (-1.0 / 18.0) * m_eps + (-1.0 / 6.0) * jy +
            (1.0 / 6.0) * m_qy + (-1.0 / 4.0) * m_pxx;
    fn[5] = (1.0 / 9.0) * rho + (1.0 / 18.0) * m_e + (1.0 / 36.0) * m_eps + (1.0 / 6.0) * jx +
            (1.0 / 12.0) * m_qx + (1.0 / 6.0) * jy + (1.0 / 12.0) * m_qy + (1.0 / 4.0) * m_pxy;
    fn[6] = (1.0 / 9.0) * rho + (1.0 / 18.0) * m_e + (1.0 / 36.0) * m_eps + (-1.0 / 6.0) * jx +
            (-1.0 / 12.0) * m_qx + (1.0 / 6.0) * jy + (1.0 / 12.0) * m_qy + (-1.0 / 4.0) * m_pxy;
    fn[7] = (1.0 / 9.0) * rho + (1.0 / 18.0) * m_e + (1.0 / 36.0) * m_eps + (-1.0 / 6.0) * jx +
            (-1.0 / 12.0) * m_qx + (-1.0 / 6.0) * jy + (-1.0 / 12.0) * m_qy + (1.0 / 4.0) * m_pxy;
    fn[8] = (1.0 / 9.0) * rho + (1.0 / 18.0) * m_e + (1.0 / 36.0) * m_eps + (1.0 / 6.0) * jx +
            (1.0 / 12.0) * m_qx + (-1.0 / 6.0) * jy + (-1.0 / 12.0) * m_qy + (-1.0 / 4.0) * m_pxy;
}

/* ---------------------------------------------------------------- thermal (src/thermal.hpp) */

/* thermal_equilibrium, src/thermal.hpp:25-30 (thermal weights = D2Q9 weights, :17-20) */
double or_thermal_equilibrium(int i, double T, double u, double v) {
    double ed = OR_CX[i] * u + OR_CY[i] * v;
    double usq = u * u + v * v;
    return OR_W[i] * T * (1.0 + 3.0 * ed + 4.5 * ed * ed - 1.5 * usq);
}

/* thermal_collide, src/thermal.hpp:35-41 */
static void or_thermal_collide(double *gn, double T, double u, double v, double omega_k) {
    for (int i = 0; i < 9; ++i) {
        double geq = or_thermal_equilibrium(i, T, u, v);
        gn[i] -= omega_k * (gn[i] - geq);
    }
}

/* compute_temperature, src/thermal.hpp:55-60 */
double or_temperature(const double *gn) {
    double T = 0.0;
    for (int i = 0; i < 9; ++i) T += gn[i];
    return T;
}

/* apply_thermal_isothermal, src/thermal.hpp:70-75 */
void or_thermal_isothermal(double *gn, double T_wall, double uw, double vw) {
    for (int i = 0; i < 9; ++i) gn[i] = or_thermal_equilibrium(i, T_wall, uw, vw);
}

/* apply_thermal_adiabatic, src/thermal.hpp:78-83 */
void or_thermal_adiabatic(double *gn, const double *g_opp) {
    for (int i = 0; i < 9; ++i) gn[i] = g_opp[OR_BB[i]];
}

/* compute_nusselt, src/thermal.hpp:88-91 */
double or_nusselt(double dTdr_wall, double D, double T_wall, double T_inf) {
    if (fabs(T_wall - T_inf) < 1e-12) return 0.0;
    return -2.0 * dTdr_wall * D / (T_wall - T_inf);
}

/* ---------------------------------------------------------------- geometry */

/* BounceBackGeometry::q_cylinder, src/lbm_types.hpp:118-138 */
static double or_q_cylinder(const or_state *s, double xf, double yf, int i) {
    double dx = xf - s->bb_cx, dy = yf - s->bb_cy;
    double ex = (double)OR_CX[i], ey = (double)OR_CY[i];
    double len2 = ex * ex + ey * ey;
    double b = 2.0 * (dx * ex + dy * ey);
    double c = dx * dx + dy * dy - s->bb_radius * s->bb_radius;
    double disc = b * b - 4.0 * len2 * c;
    if (disc < 0.0) return 1.0;
    double sd = sqrt(disc);
    double t1 = (-b - sd) / (2.0 * len2);
    double t2 = (-b + sd) / (2.0 * len2);
    if (t1 > 0.0 && t1 <= 1.0) return t1;
    if (t2 > 0.0 && t2 <= 1.0) return t2;
    return 1.0;
}

/* BounceBackGeometry::q_polygon, src/lbm_types.hpp:143-170 */
static double or_q_polygon(const or_state *s, double xf, double yf, int i) {
    double ex = (double)OR_CX[i], ey = (double)OR_CY[i];
    int n = s->npoly;
    if (n < 3) return 1.0;
    double best = 1.0;
    for (int k = 0; k < n; ++k) {
        int k2 = (k + 1) % n;
        double x1 = s->poly[2 * k], y1 = s->poly[2 * k + 1];
        double x2 = s->poly[2 * k2], y2 = s->poly[2 * k2 + 1];
        double ddx = x2 - x1, ddy = y2 - y1;
        double den = ex * ddy - ey * ddx;
        if (fabs(den) < 1e-15) continue;
        double t = ((x1 - xf) * ddy - (y1 - yf) * ddx) / den;
        double sp = ((x1 - xf) * ey - (y1 - yf) * ex) / den;
        if (t > 0.0 && t <= best && sp >= 0.0 && sp <= 1.0) best = t;
    }
    return best;
}

/* BounceBackGeometry::compute_q, src/lbm_types.hpp:173-176 */
double or_compute_q(const or_state *s, double xf, double yf, int i) {
    return s->is_polygon ? or_q_polygon(s, xf, yf, i) : or_q_cylinder(s, xf, yf, i);
}

/* BounceBackGeometry::compute_wall_velocity, src/lbm_types.hpp:106-114 */
static void or_wall_velocity(const or_state *s, double px, double py, double *uwx, double *uwy) {
    if (!s->has_moving_wall) { *uwx = 0.0; *uwy = 0.0; return; }
    double dx = px - s->rot_cx, dy = py - s->rot_cy;
    *uwx = -s->omega * dy;
    *uwy = s->omega * dx;
}

static int or_bb_valid(const or_state *s) { return s->bb_radius > 0.0 || s->is_polygon; }

/* point_in_polygon (ray casting), src/geometry.hpp:120-134; xy = x0,y0,x1,y1,... */
int or_point_in_polygon(double px, double py, const double *xy, int n) {
    int inside = 0;
    for (int i = 0, j = n - 1; i < n; j = i++) {
        double xi = xy[2 * i], yi = xy[2 * i + 1];
        double xj = xy[2 * j], yj = xy[2 * j + 1];
        int hit = ((yi > py) != (yj > py)) && (px < (xj - xi) * (py - yi) / (yj - yi) + xi);
        if (hit) inside = !inside;
    }
    return inside;
}

/* naca_coords, src/geometry.hpp:17-90.  Writes 2*n-1 points (x,y pairs) into
 * out (capacity 2*(2n-1) doubles); returns the point count. */
int or_naca_coords(int series, int n, double *out) {
    int m_code = series / 1000, p_code = (series / 100) % 10, t_code = series % 100;
    double m = (double)m_code / 100.0, p = (double)p_code / 10.0, t = (double)t_code / 100.0;
    double *x = malloc(sizeof(double) * n), *yt = malloc(sizeof(double) * n);
    double *yc = calloc(n, sizeof(double)), *dyc = calloc(n, sizeof(double));
    for (int i = 0; i < n; ++i) {
        double beta = (double)i / (n - 1) * M_PI;
        x[i] = (1.0 - cos(beta)) / 2.0;
    }
    for (int i = 0; i < n; ++i)
        yt[i] = 5.0 * t * (0.2969 * sqrt(x[i]) - 0.1260 * x[i] - 0.3516 * x[i] * x[i] +
                           0.2843 * x[i] * x[i] * x[i] - 0.1015 * x[i] * x[i] * x[i] * x[i]);
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
    /* upper surface trailing edge -> leading edge, then lower surface LE+1 -> TE */
    for (int i = n - 1; i >= 0; --i) {
        double th = atan(dyc[i]);
        out[2 * k] = x[i] - yt[i] * sin(th);
        out[2 * k + 1] = yc[i] + yt[i] * cos(th);
        ++k;
    }
    for (int i = 1; i < n; ++i) {
        double th = atan(dyc[i]);
        out[2 * k] = x[i] + yt[i] * sin(th);
        out[2 * k + 1] = yc[i] - yt[i] * cos(th);
        ++k;
    }
    free(x); free(yt); free(yc); free(dyc);
    return k;
}

/* transform_points, src/geometry.hpp:95-114 */
void or_transform_points(double *xy, int n, double cx, double cy, double scale, double angle_deg) {
    double a = angle_deg * M_PI / 180.0;
    double ca = cos(a), sa = sin(a);
    for (int k = 0; k < n; ++k) {
        double xs = xy[2 * k] * scale, ys = xy[2 * k + 1] * scale;
        double xr = xs * ca - ys * sa;
        double yr = xs * sa + ys * ca;
        xy[2 * k] = xr + cx;
        xy[2 * k + 1] = yr + cy;
    }
}

/* ---------------------------------------------------------------- state */

or_state *or_create(int nx, int ny) {
    or_state *s = calloc(1, sizeof(or_state));
    size_t n = (size_t)nx * ny;
    s->nx = nx; s->ny = ny;
    s->collision = OR_MRT;
    s->cs = 0.12;
    s->f = calloc(n * 9, sizeof(double));
    s->f_next = calloc(n * 9, sizeof(double));
    s->g = malloc(n * 9 * sizeof(double));
    s->g_next = malloc(n * 9 * sizeof(double));
    for (size_t k = 0; k < n * 9; ++k) { s->g[k] = 1.0; s->g_next[k] = 1.0; }
    s->wall_dist = calloc(n, sizeof(double));
    s->fx = calloc(n, sizeof(double));
    s->fy = calloc(n, sizeof(double));
    s->obstacle = calloc(n, 1);
    /* defaults of LBMCapabilities, src/lbm_types.hpp:196-207 */
    s->T_ref = 1.0; s->alpha = 0.1666666667; s->omega_k = 1.0;
    s->use_mei_bb = 1;
    return s;
}

void or_destroy(or_state *s) {
    if (!s) return;
    free(s->f); free(s->f_next); free(s->g); free(s->g_next); free(s->wall_dist);
    free(s->fx); free(s->fy); free(s->obstacle); free(s->poly);
    free(s->ibm_X); free(s->ibm_Y); free(s->ibm_U); free(s->ibm_V); free(s->ibm_FX); free(s->ibm_FY);
    free(s);
}

void or_set_case(or_state *s, int case_type, int collision, int use_les, double cs) {
    s->case_type = case_type; s->collision = collision; s->use_les = use_les; s->cs = cs;
}
void or_set_thermal(or_state *s, int use, double T_ref, double alpha, double omega_k, double beta,
                    double g_buoyancy) {
    s->use_thermal = use; s->T_ref = T_ref; s->alpha = alpha; s->omega_k = omega_k;
    s->beta = beta; s->g_buoyancy = g_buoyancy;
}
void or_set_body_force(or_state *s, double fx) { s->body_force_x = fx; }
void or_set_moving_wall(or_state *s, int on, double omega, double rcx, double rcy) {
    s->has_moving_wall = on; s->omega = omega; s->rot_cx = rcx; s->rot_cy = rcy;
}
void or_set_mei(or_state *s, int on) { s->use_mei_bb = on; }
double *or_f(or_state *s) { return s->f; }
double *or_g(or_state *s) { return s->g; }
double *or_fx(or_state *s) { return s->fx; }
double *or_fy(or_state *s) { return s->fy; }
double *or_wall_dist(or_state *s) { return s->wall_dist; }
uint8_t *or_obstacle(or_state *s) { return s->obstacle; }

/* place_walls, src/lbm.hpp:79-87 */
void or_place_walls(or_state *s) {
    for (int x = 0; x < s->nx; ++x) s->obstacle[nidx(s, x, 0)] = 1;
    for (int y = 0; y < s->ny; ++y) {
        s->obstacle[nidx(s, 0, y)] = 1;
        s->obstacle[nidx(s, s->nx - 1, y)] = 1;
    }
}

/* place_cylinder, src/lbm.hpp:931-944 (bb_geom keeps only the last circle) */
void or_place_cylinder(or_state *s, int cxc, int cyc, int r) {
    s->bb_cx = (double)cxc; s->bb_cy = (double)cyc; s->bb_radius = (double)r;
    for (int y = 0; y < s->ny; ++y)
        for (int x = 0; x < s->nx; ++x) {
            double dx = (double)(x - cxc), dy = (double)(y - cyc);
            if (sqrt(dx * dx + dy * dy) < r) s->obstacle[nidx(s, x, y)] = 1;
        }
}

/* place_polygon, src/lbm.hpp:951-964 */
void or_place_polygon(or_state *s, const double *xy, int n) {
    free(s->poly);
    s->poly = malloc(sizeof(double) * 2 * (n > 0 ? n : 1));
    memcpy(s->poly, xy, sizeof(double) * 2 * n);
    s->npoly = n; s->is_polygon = 1;
    for (int y = 0; y < s->ny; ++y)
        for (int x = 0; x < s->nx; ++x)
            if (or_point_in_polygon((double)x, (double)y, xy, n)) s->obstacle[nidx(s, x, y)] = 1;
}

/* compute_wall_distance (raster Gauss-Seidel sweeps until fixed point),
 * src/lbm_types.hpp:231-264 */
void or_compute_wall_distance(or_state *s) {
    int nx = s->nx, ny = s->ny;
    size_t n = (size_t)nx * ny;
    double *d = s->wall_dist;
    for (size_t k = 0; k < n; ++k) d[k] = s->obstacle[k] ? 0.0 : 1e9;
    int changed = 1;
    while (changed) {
        changed = 0;
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x) {
                int id = nidx(s, x, y);
                if (s->obstacle[id]) continue;
                double dd = d[id];
                const int ax[4] = {x - 1, x + 1, x, x};
                const int ay[4] = {y, y, y - 1, y + 1};
                for (int k = 0; k < 4; ++k) {
                    if (ax[k] < 0 || ax[k] >= nx || ay[k] < 0 || ay[k] >= ny) continue;
                    double nd = d[nidx(s, ax[k], ay[k])] + 1.0;
                    if (nd < dd) { dd = nd; changed = 1; }
                }
                d[id] = dd;
            }
    }
}

/* ---------------------------------------------------------------- boundary conditions */

/* enforce_inflow (Zou/He), src/lbm.hpp:21-34 */
static void or_enforce_inflow(or_state *s, double u) {
    for (int y = 0; y < s->ny; ++y) {
        double *fn = &s->f[(size_t)nidx(s, 0, y) * 9];
        double rho = (fn[0] + fn[2] + fn[4] + 2.0 * (fn[3] + fn[6] + fn[7])) / (1.0 - u);
        fn[1] = fn[3] + (2.0 / 3.0) * rho * u;
        fn[5] = fn[7] + (1.0 / 6.0) * rho * u;
        fn[8] = fn[6] + (1.0 / 6.0) * rho * u;
    }
}

/* enforce_step_inflow (parabolic), src/lbm.hpp:40-58 */
static void or_enforce_step_inflow(or_state *s, int h_step, int h_inlet, double u_max) {
    for (int y = h_step; y < s->ny; ++y) {
        if (s->obstacle[nidx(s, 0, y)]) continue;
        double *fn = &s->f[(size_t)nidx(s, 0, y) * 9];
        double yy = (double)(y - h_step), h = (double)h_inlet;
        double ul = u_max * 4.0 * yy * (h - yy) / (h * h);
        double rho = (fn[0] + fn[2] + fn[4] + 2.0 * (fn[3] + fn[6] + fn[7])) / (1.0 - ul);
        fn[1] = fn[3] + (2.0 / 3.0) * rho * ul;
        fn[5] = fn[7] + (1.0 / 6.0) * rho * ul;
        fn[8] = fn[6] + (1.0 / 6.0) * rho * ul;
    }
}

/* enforce_outflow (copy column NX-2 into NX-1), src/lbm.hpp:63-73 */
static void or_enforce_outflow(or_state *s) {
    for (int y = 0; y < s->ny; ++y) {
        double *dst = &s->f[(size_t)nidx(s, s->nx - 1, y) * 9];
        const double *src = &s->f[(size_t)nidx(s, s->nx - 2, y) * 9];
        for (int i = 0; i < 9; ++i) dst[i] = src[i];
    }
}

/* enforce_lid (equilibrium lid incl. corner nodes), src/lbm.hpp:110-120 */
static void or_enforce_lid(or_state *s, double u_lid) {
    for (int x = 0; x < s->nx; ++x) {
        double *fn = &s->f[(size_t)nidx(s, x, s->ny - 1) * 9];
        double rho, u, v;
        or_macros(fn, &rho, &u, &v);
        for (int i = 0; i < 9; ++i) fn[i] = or_equilibrium(i, rho, u_lid, 0.0);
    }
}

/* apply_bouzidi_bb (Mei/Filippova-Hanel by default; classic Bouzidi and the
 * Ladd correction when use_mei_bb is off), src/lbm.hpp:226-288 */
static void or_interp_bb(or_state *s, int x, int y, int i, const double *fn, int node) {
    double q = or_compute_q(s, (double)x, (double)y, i);
    int bb = OR_BB[i];
    double fbb;
    if (s->use_mei_bb) {
        double rho, u, v;
        or_macros(fn, &rho, &u, &v);
        double uwx = 0.0, uwy = 0.0;
        if (s->has_moving_wall)
            or_wall_velocity(s, (double)(x + OR_CX[i]), (double)(y + OR_CY[i]), &uwx, &uwy);
        double feqw = or_equilibrium(i, rho, uwx, uwy);
        double fpost = fn[i];
        double ed = OR_CX[i] * uwx + OR_CY[i] * uwy;
        fbb = q * feqw + (1.0 - q) * fpost + (2.0 * q - 1.0) * OR_W[i] * rho * ed * 3.0;
    } else {
        if (q < 0.5) {
            int sx = x - OR_CX[i], sy = y - OR_CY[i];
            if (sx >= 0 && sx < s->nx && sy >= 0 && sy < s->ny) {
                double fsrc = s->f[(size_t)nidx(s, sx, sy) * 9 + i];
                fbb = 2.0 * q * fn[i] + (1.0 - 2.0 * q) * fsrc;
            } else {
                fbb = fn[i];
            }
        } else {
            double inv2q = 1.0 / (2.0 * q);
            double fopp = s->f[(size_t)node * 9 + bb];
            fbb = inv2q * fn[i] + (1.0 - inv2q) * fopp;
        }
    }
    if (s->has_moving_wall && !s->use_mei_bb) {
        double uwx, uwy, rho, u, v;
        or_wall_velocity(s, (double)(x + OR_CX[i]), (double)(y + OR_CY[i]), &uwx, &uwy);
        or_macros(fn, &rho, &u, &v);
        double ed = OR_CX[i] * uwx + OR_CY[i] * uwy;
        fbb -= 2.0 * OR_W[i] * rho * ed * 3.0;
    }
    s->f_next[(size_t)node * 9 + bb] = fbb;
}

/* One interpolated bounce-back link of node (x, y), direction i, from the
 * current f (the pre-stream state the reference passes), as or_interp_bb
 * writes it into f_next; returns the written value.  Test hook for the C++
 * drop-in's host apply_bouzidi_bb. */
double or_interp_bb_link(or_state *s, int x, int y, int i) {
    const int node = nidx(s, x, y);
    or_interp_bb(s, x, y, i, &s->f[(size_t)node * 9], node);
    return s->f_next[(size_t)node * 9 + OR_BB[i]];
}

/* ---------------------------------------------------------------- the time step */

/* execute_time_step, src/lbm.hpp:293-582 */
void or_step(or_state *s, double tau, double u_in) {
    const int NXl = s->nx, NYl = s->ny;
    const size_t nn = (size_t)NXl * NYl;
    const int ct = s->case_type;
    const int periodic_xy = (ct == OR_RIBS || ct == OR_PERIODIC_HILLS);

    double Fscale = (s->body_force_x != 0.0) ? (1.0 - 1.0 / (2.0 * tau)) * 3.0 * s->body_force_x : 0.0;

    /* collision + fused body force + LES, src/lbm.hpp:300-354 */
    if (s->collision == OR_MRT) {
        double s_shear, s_bulk, s_normal;
        or_mrt_params(tau, &s_shear, &s_bulk, &s_normal);
        double cs_sq = s->use_les ? (s->cs * s->cs) : 0.0;
        if (cs_sq > 0.0) or_compute_wall_distance(s);
        double nu = (tau - 0.5) / 3.0;
#pragma omp parallel for collapse(2)
        for (int y = 0; y < NYl; ++y)
            for (int x = 0; x < NXl; ++x) {
                int id = nidx(s, x, y);
                if (s->obstacle[id]) continue;
                double *fn = &s->f[(size_t)id * 9];
                double rho, u, v;
                or_macros(fn, &rho, &u, &v);
                double y_plus = 0.0;
                if (cs_sq > 0.0 && nu > 0.0) {
                    double wd = s->wall_dist[id];
                    double speed = sqrt(u * u + v * v);
                    double u_tau = sqrt(speed * speed + 1e-12);
                    y_plus = wd * u_tau / nu;
                }
                or_mrt_collide(fn, rho, u, v, s_shear, s_bulk, s_normal, cs_sq, tau, y_plus);
                if (Fscale != 0.0)
                    for (int i = 0; i < 9; ++i) fn[i] += OR_W[i] * OR_CX[i] * Fscale;
            }
    } else {
#pragma omp parallel for collapse(2)
        for (int y = 0; y < NYl; ++y)
            for (int x = 0; x < NXl; ++x) {
                int id = nidx(s, x, y);
                if (s->obstacle[id]) continue;
                double *fn = &s->f[(size_t)id * 9];
                double rho, u, v;
                or_macros(fn, &rho, &u, &v);
                double inv_tau = 1.0 / tau;
                for (int i = 0; i < 9; ++i) {
                    double feq = or_equilibrium(i, rho, u, v);
                    fn[i] -= inv_tau * (fn[i] - feq);
                    if (Fscale != 0.0) fn[i] += OR_W[i] * OR_CX[i] * Fscale;
                }
            }
    }

    /* thermal collision + Boussinesq/Guo buoyancy on f, src/lbm.hpp:357-397 */
    if (s->use_thermal) {
        const double rho0 = 1.0;
#pragma omp parallel for collapse(2)
        for (int y = 0; y < NYl; ++y)
            for (int x = 0; x < NXl; ++x) {
                int id = nidx(s, x, y);
                if (s->obstacle[id]) continue;
                double *fn = &s->f[(size_t)id * 9];
                double *gn = &s->g[(size_t)id * 9];
                double rho, u, v;
                or_macros(fn, &rho, &u, &v);
                double T = or_temperature(gn);
                or_thermal_collide(gn, T, u, v, s->omega_k);
                if (s->beta > 0.0 && s->g_buoyancy != 0.0) {
                    /* boussinesq_force, src/thermal.hpp:46-52, with g = (0, g_buoyancy) */
                    double dT = T - s->T_ref;
                    double fxb = -rho0 * s->beta * dT * 0.0;
                    double fyb = -rho0 * s->beta * dT * s->g_buoyancy;
                    for (int i = 0; i < 9; ++i) {
                        double eu = OR_CX[i] * u + OR_CY[i] * v;
                        double Fd = OR_CX[i] * fxb + OR_CY[i] * fyb;
                        double corr = OR_W[i] * (3.0 * Fd + 9.0 * eu * (OR_CX[i] * fxb + OR_CY[i] * fyb));
                        fn[i] += corr;
                    }
                }
            }
    }

    /* zero the next buffers, src/lbm.hpp:400-403 */
    memset(s->f_next, 0, nn * 9 * sizeof(double));
    if (s->use_thermal) memset(s->g_next, 0, nn * 9 * sizeof(double));

    const int interp = or_bb_valid(s);
    /* push streaming, src/lbm.hpp:408-484 */
    if (ct == OR_CAVITY) {
#pragma omp parallel for collapse(2)
        for (int y = 0; y < NYl; ++y)
            for (int x = 0; x < NXl; ++x) {
                int id = nidx(s, x, y);
                if (s->obstacle[id]) continue;
                const double *fn = &s->f[(size_t)id * 9];
                for (int i = 0; i < 9; ++i) {
                    int tx = x + OR_CX[i], ty = y + OR_CY[i];
                    if (tx < 0 || tx >= NXl || ty < 0 || ty >= NYl) {
                        s->f_next[(size_t)id * 9 + OR_BB[i]] = fn[i];
                    } else {
                        int t = nidx(s, tx, ty);
                        if (s->obstacle[t]) {
                            if (interp) or_interp_bb(s, x, y, i, fn, id);
                            else s->f_next[(size_t)id * 9 + OR_BB[i]] = fn[i];
                        } else {
                            s->f_next[(size_t)t * 9 + i] = fn[i];
                        }
                    }
                }
            }
    } else if (periodic_xy) {
#pragma omp parallel for collapse(2)
        for (int y = 0; y < NYl; ++y)
            for (int x = 0; x < NXl; ++x) {
                int id = nidx(s, x, y);
                if (s->obstacle[id]) continue;
                const double *fn = &s->f[(size_t)id * 9];
                for (int i = 0; i < 9; ++i) {
                    int tx = x + OR_CX[i], ty = y + OR_CY[i];
                    if (tx < 0) tx += NXl;
                    if (tx >= NXl) tx -= NXl;
                    if (ty < 0) ty += NYl;
                    if (ty >= NYl) ty -= NYl;
                    int t = nidx(s, tx, ty);
                    if (s->obstacle[t]) s->f_next[(size_t)id * 9 + OR_BB[i]] = fn[i];
                    else s->f_next[(size_t)t * 9 + i] = fn[i];
                }
            }
    } else {
#pragma omp parallel for collapse(2)
        for (int y = 0; y < NYl; ++y)
            for (int x = 0; x < NXl; ++x) {
                int id = nidx(s, x, y);
                if (s->obstacle[id]) continue;
                const double *fn = &s->f[(size_t)id * 9];
                for (int i = 0; i < 9; ++i) {
                    int tx = x + OR_CX[i], ty = y + OR_CY[i];
                    if (ty < 0) ty += NYl;
                    if (ty >= NYl) ty -= NYl;
                    if (tx >= 0 && tx < NXl) {
                        int t = nidx(s, tx, ty);
                        if (s->obstacle[t]) {
                            if (interp) or_interp_bb(s, x, y, i, fn, id);
                            else s->f_next[(size_t)id * 9 + OR_BB[i]] = fn[i];
                        } else {
                            s->f_next[(size_t)t * 9 + i] = fn[i];
                        }
                    }
                }
            }
    }
    { double *t = s->f; s->f = s->f_next; s->f_next = t; }

    /* thermal streaming with adiabatic bounce-back, src/lbm.hpp:490-528 */
    if (s->use_thermal) {
#pragma omp parallel for collapse(2)
        for (int y = 0; y < NYl; ++y)
            for (int x = 0; x < NXl; ++x) {
                int id = nidx(s, x, y);
                if (s->obstacle[id]) continue;
                const double *gn = &s->g[(size_t)id * 9];
                for (int i = 0; i < 9; ++i) {
                    int tx = x + OR_CX[i], ty = y + OR_CY[i];
                    if (periodic_xy) {
                        if (tx < 0) tx += NXl;
                        if (tx >= NXl) tx -= NXl;
                        if (ty < 0) ty += NYl;
                        if (ty >= NYl) ty -= NYl;
                    } else {
                        if (ty < 0) ty += NYl;
                        if (ty >= NYl) ty -= NYl;
                    }
                    if (tx < 0 || tx >= NXl || ty < 0 || ty >= NYl) {
                        s->g_next[(size_t)id * 9 + OR_BB[i]] = gn[i];
                    } else {
                        int t = nidx(s, tx, ty);
                        if (s->obstacle[t]) s->g_next[(size_t)id * 9 + OR_BB[i]] = gn[i];
                        else s->g_next[(size_t)t * 9 + i] = gn[i];
                    }
                }
            }
        double *t = s->g; s->g = s->g_next; s->g_next = t;
    }

    /* boundary conditions, src/lbm.hpp:531-540 */
    if (ct == OR_CAVITY) {
        or_enforce_lid(s, u_in);
    } else if (ct == OR_STEP) {
        or_enforce_step_inflow(s, NYl / 3, NYl - 1 - NYl / 3, u_in);
        or_enforce_outflow(s);
    } else if (!periodic_xy) {
        or_enforce_inflow(s, u_in);
        or_enforce_outflow(s);
    }

    /* momentum-exchange force (serial), src/lbm.hpp:543-581 */
    if (ct != OR_CAVITY) {
        memset(s->fx, 0, nn * sizeof(double));
        memset(s->fy, 0, nn * sizeof(double));
        for (int y = 0; y < NYl; ++y)
            for (int x = 0; x < NXl; ++x) {
                int id = nidx(s, x, y);
                if (s->obstacle[id]) continue;
                for (int i = 0; i < 9; ++i) {
                    int tx = x + OR_CX[i], ty = y + OR_CY[i];
                    if (periodic_xy) {
                        if (ty < 0) ty += NYl;
                        if (ty >= NYl) ty -= NYl;
                        if (tx < 0) tx += NXl;
                        if (tx >= NXl) tx -= NXl;
                    } else {
                        if (ty < 0) ty += NYl;
                        if (ty >= NYl) ty -= NYl;
                        if (tx < 0 || tx >= NXl) continue;
                    }
                    int t = nidx(s, tx, ty);
                    if (s->obstacle[t]) {
                        if (ct == OR_CYLINDER_NEAR_WALL) {
                            double dx = (double)tx - s->bb_cx, dy = (double)ty - s->bb_cy;
                            if (sqrt(dx * dx + dy * dy) > s->bb_radius) continue;
                        }
                        double fb = s->f[(size_t)id * 9 + OR_BB[i]];
                        s->fx[id] += OR_CX[i] * 2.0 * fb;
                        s->fy[id] += OR_CY[i] * 2.0 * fb;
                    }
                }
            }
    }
}

/* Driver-side force sums in node order, src/main.cpp:106-110. */
void or_force_sums(const or_state *s, double *fx_total, double *fy_total) {
    double a = 0.0, b = 0.0;
    size_t nn = (size_t)s->nx * s->ny;
    for (size_t k = 0; k < nn; ++k) { a += s->fx[k]; b += s->fy[k]; }
    *fx_total = a; *fy_total = b;
}

/* Driver thermal boundary passes applied after each step.
 * kind 1: differentially heated cavity, src/thermal_cavity.cpp:168-204
 *         (Dirichlet at x=1 with Th and x=NX-2 with Tc, then the in-place
 *          adiabatic copy at y=1 and y=NY-2).
 * kind 2: heated cylinder, src/heated_cylinder.cpp:156-164 (isothermal
 *         equilibrium written into every solid node). */
void or_thermal_hook(or_state *s, int kind, double Ta, double Tb) {
    int nx = s->nx, ny = s->ny;
    if (kind == 1) {
        for (int y = 1; y < ny - 1; ++y) {
            int ids[2] = {nidx(s, 1, y), nidx(s, nx - 2, y)};
            double Tw[2] = {Ta, Tb};
            for (int k = 0; k < 2; ++k) {
                double rho, u, v;
                or_macros(&s->f[(size_t)ids[k] * 9], &rho, &u, &v);
                for (int i = 0; i < 9; ++i) s->g[(size_t)ids[k] * 9 + i] = or_thermal_equilibrium(i, Tw[k], u, v);
            }
        }
        for (int x = 1; x < nx - 1; ++x) {
            int ids[2] = {nidx(s, x, 1), nidx(s, x, ny - 2)};
            for (int k = 0; k < 2; ++k) {
                double *gn = &s->g[(size_t)ids[k] * 9];
                for (int i = 0; i < 9; ++i) gn[i] = gn[OR_BB[i]];
            }
        }
    } else if (kind == 2) {
        size_t nn = (size_t)nx * ny;
        for (size_t k = 0; k < nn; ++k)
            if (s->obstacle[k]) or_thermal_isothermal(&s->g[k * 9], Ta, 0.0, 0.0);
    }
}

/* ---------------------------------------------------------------- seeded initial states */

/* mt19937 (Matsumoto & Nishimura 1998), seeded as std::mt19937(seed). */
typedef struct { uint32_t mt[624]; int idx; } or_mt19937;
static void or_mt_seed(or_mt19937 *r, uint32_t seed) {
    r->mt[0] = seed;
    for (int i = 1; i < 624; ++i) r->mt[i] = 1812433253u * (r->mt[i - 1] ^ (r->mt[i - 1] >> 30)) + (uint32_t)i;
    r->idx = 624;
}
static uint32_t or_mt_next(or_mt19937 *r) {
    if (r->idx >= 624) {
        for (int i = 0; i < 624; ++i) {
            uint32_t yv = (r->mt[i] & 0x80000000u) | (r->mt[(i + 1) % 624] & 0x7fffffffu);
            uint32_t v = r->mt[(i + 397) % 624] ^ (yv >> 1);
            if (yv & 1u) v ^= 0x9908b0dfu;
            r->mt[i] = v;
        }
        r->idx = 0;
    }
    uint32_t yv = r->mt[r->idx++];
    yv ^= yv >> 11;
    yv ^= (yv << 7) & 0x9d2c5680u;
    yv ^= (yv << 15) & 0xefc60000u;
    yv ^= yv >> 18;
    return yv;
}
/* uniform real in [a,b) from two 32-bit draws, as the GNU C++ library's
 * generate_canonical<double,53> followed by a + (b-a)*u. */
static double or_mt_uniform(or_mt19937 *r, double a, double b) {
    const double two32 = 4294967296.0;
    double sum = (double)or_mt_next(r);
    sum += (double)or_mt_next(r) * two32;
    double u = sum / (two32 * two32);
    if (u >= 1.0) u = nextafter(1.0, 0.0);
    return u * (b - a) + a;
}

/* Equilibrium initial state with uniform (rho=1, u_in, 0) and the seeded
 * transverse perturbation of the cylinder-wake driver, src/main.cpp:60-83. */
void or_init_cylinder_wake(or_state *s, double u_in, int cx_cyl, unsigned seed, double amp) {
    size_t nn = (size_t)s->nx * s->ny;
    for (size_t k = 0; k < nn; ++k)
        for (int i = 0; i < 9; ++i) s->f[k * 9 + i] = or_equilibrium(i, 1.0, u_in, 0.0);
    or_mt19937 r;
    or_mt_seed(&r, seed);
    int xe = cx_cyl + 60 < s->nx ? cx_cyl + 60 : s->nx;
    for (int x = cx_cyl + 5; x < xe; ++x)
        for (int y = 0; y < s->ny; ++y) {
            int id = nidx(s, x, y);
            if (s->obstacle[id]) continue;
            double *fn = &s->f[(size_t)id * 9];
            double vp = or_mt_uniform(&r, -amp, amp);
            double rho, u, v;
            or_macros(fn, &rho, &u, &v);
            for (int i = 0; i < 9; ++i) fn[i] = or_equilibrium(i, rho, u, v + vp);
        }
}

/* Uniform equilibrium initial state, as every driver's init loop. */
void or_init_uniform(or_state *s, double rho, double u, double v) {
    size_t nn = (size_t)s->nx * s->ny;
    for (size_t k = 0; k < nn; ++k)
        for (int i = 0; i < 9; ++i) s->f[k * 9 + i] = or_equilibrium(i, rho, u, v);
}
void or_init_thermal_uniform(or_state *s, double T, double u, double v) {
    size_t nn = (size_t)s->nx * s->ny;
    for (size_t k = 0; k < nn; ++k)
        for (int i = 0; i < 9; ++i) s->g[k * 9 + i] = or_thermal_equilibrium(i, T, u, v);
}

/* ---------------------------------------------------------------- immersed boundary */

/* ibm_delta, src/ibm.hpp:16-19 (4-point cosine delta) */
double or_ibm_delta(double r) {
    if (fabs(r) >= 2.0) return 0.0;
    return 0.25 * (1.0 + cos(0.5 * M_PI * r));
}

/* ibm_kernel, src/ibm.hpp:22-24 */
double or_ibm_kernel(double dx, double dy) { return or_ibm_delta(dx) * or_ibm_delta(dy); }

/* ImmersedBoundary::build_from_polygon, src/ibm.hpp:42-69: points spaced
 * uniformly in the polygon's vertex parameter.  Writes at most cap points;
 * returns the point count. */
int or_ibm_points_from_polygon(const double *xy, int n, double spacing, double *X, double *Y, int cap) {
    if (n < 3) return 0;
    double total_len = 0.0;
    for (int i = 0; i < n; ++i) {
        int j = (i + 1) % n;
        double dx = xy[2 * j] - xy[2 * i];
        double dy = xy[2 * j + 1] - xy[2 * i + 1];
        total_len += sqrt(dx * dx + dy * dy);
    }
    int n_points = (int)(total_len / spacing);
    if (n_points < 8) n_points = 8;
    for (int k = 0; k < n_points && k < cap; ++k) {
        double t = (double)k / n_points;
        double seg = t * n;
        int i = (int)seg % n;
        int j = (i + 1) % n;
        double f = seg - floor(seg);
        X[k] = xy[2 * i] + f * (xy[2 * j] - xy[2 * i]);
        Y[k] = xy[2 * i + 1] + f * (xy[2 * j + 1] - xy[2 * i + 1]);
    }
    return n_points;
}

/* Install the Lagrangian points; the no-slip target velocity is (uwx, uwy)
 * (src/ibm.hpp:139-149).  n = 0 removes the boundary. */
void or_ibm_set(or_state *s, const double *X, const double *Y, int n, double dt, double uwx, double uwy) {
    free(s->ibm_X); free(s->ibm_Y); free(s->ibm_U); free(s->ibm_V); free(s->ibm_FX); free(s->ibm_FY);
    s->ibm_X = s->ibm_Y = s->ibm_U = s->ibm_V = s->ibm_FX = s->ibm_FY = NULL;
    s->ibm_n = n;
    s->ibm_dt = dt; s->ibm_uwx = uwx; s->ibm_uwy = uwy;
    if (n <= 0) return;
    s->ibm_X = malloc(n * sizeof(double)); s->ibm_Y = malloc(n * sizeof(double));
    s->ibm_U = calloc(n, sizeof(double)); s->ibm_V = calloc(n, sizeof(double));
    s->ibm_FX = calloc(n, sizeof(double)); s->ibm_FY = calloc(n, sizeof(double));
    memcpy(s->ibm_X, X, n * sizeof(double));
    memcpy(s->ibm_Y, Y, n * sizeof(double));
}

/* One iteration of the airfoil driver loop, src/airfoil_ibm.cpp:121-176:
 * 1. velocity at each Lagrangian point from the fluid nodes of its 5x5
 *    stencil (:124-147); 2. no-slip force (U_wall - U)/dt (src/ibm.hpp:
 *    139-149); 3. spread to the grid in point order (src/ibm.hpp:72-103);
 * 4. the time step; 5. explicit forcing of every fluid node,
 *    f_i += w_i (3 c_i.F + 9 (c_i.0)(c_i.F)) (:158-176). */
void or_ibm_step(or_state *s, double tau, double u_in) {
    const int nx = s->nx, ny = s->ny, np = s->ibm_n;
    size_t N = (size_t)nx * ny;
    for (int p = 0; p < np; ++p) {
        double X = s->ibm_X[p], Y = s->ibm_Y[p];
        double u = 0, v = 0;
        int x0 = (int)floor(X) - 2, x1 = (int)floor(X) + 2;
        int y0 = (int)floor(Y) - 2, y1 = (int)floor(Y) + 2;
        for (int y = y0; y <= y1; ++y) {
            if (y < 0 || y >= ny) continue;
            for (int x = x0; x <= x1; ++x) {
                if (x < 0 || x >= nx) continue;
                double kernel = or_ibm_kernel(x - X, y - Y);
                if (kernel == 0.0) continue;
                int idx = nidx(s, x, y);
                if (s->obstacle[idx]) continue;
                double rho, uu, vv;
                or_macros(&s->f[(size_t)idx * 9], &rho, &uu, &vv);
                u += uu * kernel;
                v += vv * kernel;
            }
        }
        s->ibm_U[p] = u;
        s->ibm_V[p] = v;
    }
    for (int p = 0; p < np; ++p) {
        s->ibm_FX[p] = (s->ibm_uwx - s->ibm_U[p]) / s->ibm_dt;
        s->ibm_FY[p] = (s->ibm_uwy - s->ibm_V[p]) / s->ibm_dt;
    }
    double *fxg = calloc(N, sizeof(double)), *fyg = calloc(N, sizeof(double));
    for (int p = 0; p < np; ++p) {
        double X = s->ibm_X[p], Y = s->ibm_Y[p];
        double fx = s->ibm_FX[p], fy = s->ibm_FY[p];
        int x0 = (int)floor(X) - 2, x1 = (int)floor(X) + 2;
        int y0 = (int)floor(Y) - 2, y1 = (int)floor(Y) + 2;
        for (int y = y0; y <= y1; ++y) {
            if (y < 0 || y >= ny) continue;
            for (int x = x0; x <= x1; ++x) {
                if (x < 0 || x >= nx) continue;
                double kernel = or_ibm_kernel(x - X, y - Y);
                if (kernel == 0.0) continue;
                int idx = y * nx + x;
                fxg[idx] += fx * kernel;
                fyg[idx] += fy * kernel;
            }
        }
    }
    or_step(s, tau, u_in);
    for (int y = 0; y < ny; ++y) {
        for (int x = 0; x < nx; ++x) {
            int idx = nidx(s, x, y);
            if (s->obstacle[idx]) continue;
            double *fn = &s->f[(size_t)idx * 9];
            double fx = fxg[idx], fy = fyg[idx];
            for (int i = 0; i < 9; ++i) {
                double edotu = OR_CX[i] * 0 + OR_CY[i] * 0;
                double Fdot = OR_CX[i] * fx + OR_CY[i] * fy;
                double correction = OR_W[i] * (3.0 * Fdot + 9.0 * edotu * (OR_CX[i] * fx + OR_CY[i] * fy));
                fn[i] += correction;
            }
        }
    }
    free(fxg);
    free(fyg);
}

/* Lagrangian velocities and forces of the last or_ibm_step. */
void or_ibm_lagrangian(const or_state *s, double *U, double *V, double *FX, double *FY) {
    for (int p = 0; p < s->ibm_n; ++p) {
        U[p] = s->ibm_U[p]; V[p] = s->ibm_V[p];
        FX[p] = s->ibm_FX[p]; FY[p] = s->ibm_FY[p];
    }
}
