// lbm_types.hpp -- drop-in replacement of the reference's src/lbm_types.hpp.
//
// Same names, same meaning: the process-global knobs (NX, NY, g_case,
// g_collision, g_use_les, g_cs), the D2Q9 constants, MRTParams,
// BounceBackGeometry, LBMCapabilities, compute_wall_distance,
// compute_equilibrium and compute_macros.  What changes is where the state
// lives: LBMCapabilities owns a GPU solver (include/lbm2d.h) and its vectors
// are host MIRRORS of the device state.  A mirror downloads lazily the first
// time it is touched after a step and remembers whether the host wrote it, so
// execute_time_step uploads only what a driver changed.  Drivers written for
// the reference (sys.f[n*9+i], &sys.f[idx*9], sys.obstacle[i] = true,
// sys.fx_body[n], std::count(sys.obstacle.begin(), ...)) compile and run
// unchanged.
//
// Environment: LBM2D_STORAGE = fp32 (default) | fp64 | fp16 | bf16,
//              LBM2D_DEVICE  = CUDA device ordinal (default 0).
#pragma once
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <functional>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "lbm2d.h"

// ---------------------------------------------------------------- globals (src/lbm_types.hpp:15-32)
inline int NX = 800;
inline int NY = 300;
constexpr int NUM_DIRECTIONS = 9;

enum class CaseType { CYLINDER, CAVITY, STEP, RIBS, URBAN_CANYON, DOWNWASH, SQUARE_CYLINDER, FLAT_PLATE,
                      SPORTS_BALL, PERIODIC_HILLS, CYLINDER_NEAR_WALL, SIDE_BY_SIDE, ROTATING_CYLINDER,
                      ORIFICE_PLATE };
enum class CollisionType { MRT, BGK };
inline CollisionType g_collision = CollisionType::MRT;
inline CaseType g_case = CaseType::CYLINDER;
inline bool g_use_les = false;
inline double g_cs = 0.12;

// ---------------------------------------------------------------- D2Q9 (src/lbm_types.hpp:41-55)
constexpr std::array<int, 9> cx = {0, 1, 0, -1, 0, 1, -1, -1, 1};
constexpr std::array<int, 9> cy = {0, 0, 1, 0, -1, 1, 1, -1, -1};
constexpr std::array<double, 9> weights = {4.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0,
                                           1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0};
constexpr std::array<int, 9> bounce_back = {0, 3, 4, 1, 2, 7, 8, 5, 6};

// MRTParams (src/lbm_types.hpp:60-77)
struct MRTParams {
    double s_shear;
    double s_bulk;
    double s_normal;
    static MRTParams from_tau(double tau) {
        const double s = 1.0 / tau;
        return {(s < 0.5) ? 0.5 : ((s > 1.99) ? 1.99 : s), 1.2, 1.0};
    }
};

inline int node_index(int x, int y) { return y * NX + x; }

// BounceBackGeometry (src/lbm_types.hpp:90-182): same fields and methods; the
// device solver receives circle/polygon/moving-wall parameters from it.
struct BounceBackGeometry {
    double cx = 0.0, cy = 0.0, radius = 0.0;
    std::vector<std::pair<double, double>> poly_vertices;
    bool is_polygon = false;
    bool has_moving_wall = false;
    double omega = 0.0;
    double rot_cx = 0.0, rot_cy = 0.0;
    bool use_mei_bb = true;

    bool is_valid() const { return radius > 0.0 || is_polygon; }

    void compute_wall_velocity(double px, double py, double& u_wall_x, double& u_wall_y) const {
        if (!has_moving_wall) {
            u_wall_x = 0.0;
            u_wall_y = 0.0;
            return;
        }
        const double dx = px - rot_cx, dy = py - rot_cy;
        u_wall_x = -omega * dy;
        u_wall_y = omega * dx;
    }

    double q_cylinder(double xf, double yf, int i) const {
        const double dx = xf - cx, dy = yf - cy;
        const double ex = static_cast<double>(::cx[i]), ey = static_cast<double>(::cy[i]);
        const double len2 = ex * ex + ey * ey;
        const double b = 2.0 * (dx * ex + dy * ey);
        const double c = dx * dx + dy * dy - radius * radius;
        const double disc = b * b - 4.0 * len2 * c;
        if (disc < 0.0) return 1.0;
        const double sd = std::sqrt(disc);
        const double t1 = (-b - sd) / (2.0 * len2);
        const double t2 = (-b + sd) / (2.0 * len2);
        if (t1 > 0.0 && t1 <= 1.0) return t1;
        if (t2 > 0.0 && t2 <= 1.0) return t2;
        return 1.0;
    }

    double q_polygon(double xf, double yf, int i) const {
        const double ex = static_cast<double>(::cx[i]), ey = static_cast<double>(::cy[i]);
        const int n = static_cast<int>(poly_vertices.size());
        if (n < 3) return 1.0;
        double best = 1.0;
        for (int v = 0; v < n; ++v) {
            const int v2 = (v + 1) % n;
            const double x1 = poly_vertices[v].first, y1 = poly_vertices[v].second;
            const double x2 = poly_vertices[v2].first, y2 = poly_vertices[v2].second;
            const double ddx = x2 - x1, ddy = y2 - y1;
            const double den = ex * ddy - ey * ddx;
            if (std::abs(den) < 1e-15) continue;
            const double t = ((x1 - xf) * ddy - (y1 - yf) * ddx) / den;
            const double s = ((x1 - xf) * ey - (y1 - yf) * ex) / den;
            if (t > 0.0 && t <= best && s >= 0.0 && s <= 1.0) best = t;
        }
        return best;
    }

    double compute_q(double xf, double yf, int i) const {
        return is_polygon ? q_polygon(xf, yf, i) : q_cylinder(xf, yf, i);
    }
};

namespace lbm2d_dropin {

// std::vector-like host mirror of one device array.
template <class T>
class Mirror {
   public:
    using value_type = T;
    using size_type = std::size_t;
    using iterator = T*;
    using const_iterator = const T*;
    using reference = T&;
    using const_reference = const T&;

    Mirror() = default;
    Mirror(const Mirror&) = delete;
    Mirror& operator=(const Mirror&) = delete;

    T& operator[](size_type i) {
        rw();
        return v_[i];
    }
    const T& operator[](size_type i) const {
        ro();
        return v_[i];
    }
    T& at(size_type i) {
        rw();
        return v_.at(i);
    }
    const T& at(size_type i) const {
        ro();
        return v_.at(i);
    }
    T* data() {
        rw();
        return v_.data();
    }
    const T* data() const {
        ro();
        return v_.data();
    }
    iterator begin() {
        rw();
        return v_.data();
    }
    iterator end() {
        rw();
        return v_.data() + v_.size();
    }
    const_iterator begin() const {
        ro();
        return v_.data();
    }
    const_iterator end() const {
        ro();
        return v_.data() + v_.size();
    }
    const_iterator cbegin() const { return begin(); }
    const_iterator cend() const { return end(); }
    size_type size() const { return v_.size(); }
    bool empty() const { return v_.empty(); }
    void resize(size_type n, const T& val = T()) {
        rw();
        v_.resize(n, val);
    }
    void assign(size_type n, const T& val) {
        v_.assign(n, val);
        stale_ = false;
        dirty_ = true;
    }

    // ---- synchronisation (used by LBMCapabilities)
    void mark_stale() { stale_ = true; }
    bool dirty() const { return dirty_; }
    void clear_dirty() { dirty_ = false; }
    bool stale() const { return stale_; }
    std::vector<T>& raw() { return v_; }
    void set_puller(std::function<void(std::vector<T>&)> fn) { pull_ = std::move(fn); }

   private:
    void ro() const {
        if (stale_) refresh();
    }
    void rw() {
        if (stale_) refresh();
        dirty_ = true;
    }
    void refresh() const {
        stale_ = false;
        if (pull_) pull_(v_);
    }
    mutable std::vector<T> v_;
    mutable bool stale_ = false;
    bool dirty_ = false;
    std::function<void(std::vector<T>&)> pull_;
};

inline void check(int rc, lbm2d_solver* h, const char* what) {
    if (rc != LBM2D_OK)
        throw std::runtime_error(std::string("lbm2d: ") + what + ": " +
                                 (h ? lbm2d_last_error(h) : lbm2d_global_error()));
}

inline int storage_from_env() {
    const char* s = std::getenv("LBM2D_STORAGE");
    if (!s) return LBM2D_STORE_FP32;
    const std::string v(s);
    if (v == "fp64") return LBM2D_STORE_FP64;
    if (v == "fp16") return LBM2D_STORE_FP16;
    if (v == "bf16") return LBM2D_STORE_BF16;
    return LBM2D_STORE_FP32;
}

inline int device_from_env() {
    const char* s = std::getenv("LBM2D_DEVICE");
    return s ? std::atoi(s) : 0;
}

}  // namespace lbm2d_dropin

// ---------------------------------------------------------------- state (src/lbm_types.hpp:187-224)
struct LBMCapabilities {
    lbm2d_dropin::Mirror<double> f;
    std::vector<double> f_next;  // kept for interface compatibility; the device owns the step buffers
    lbm2d_dropin::Mirror<uint8_t> obstacle;
    lbm2d_dropin::Mirror<double> wall_dist;

    lbm2d_dropin::Mirror<double> g_thermal;
    std::vector<double> g_thermal_next;
    bool use_thermal = false;
    double T_ref = 1.0;
    double alpha = 0.1666666667;
    double omega_k = 1.0;
    double beta = 0.0;
    double g_buoyancy = 0.0;

    lbm2d_dropin::Mirror<double> fx_body;
    lbm2d_dropin::Mirror<double> fy_body;

    BounceBackGeometry bb_geom;
    double body_force_x = 0.0;

    LBMCapabilities() {
        const int n_nodes = NX * NY;
        nx_ = NX;
        ny_ = NY;
        f.assign(static_cast<size_t>(n_nodes) * NUM_DIRECTIONS, 0.0);
        obstacle.assign(n_nodes, 0);
        wall_dist.assign(n_nodes, 0.0);
        g_thermal.assign(static_cast<size_t>(n_nodes) * NUM_DIRECTIONS, 1.0);
        g_thermal.clear_dirty();
        wall_dist.clear_dirty();
        reset_forces();
        f.set_puller([this](std::vector<double>& v) {
            lbm2d_dropin::check(lbm2d_download_f(h_, v.data()), h_, "download f");
        });
        g_thermal.set_puller([this](std::vector<double>& v) {
            lbm2d_dropin::check(lbm2d_download_g(h_, v.data()), h_, "download g");
        });
        fx_body.set_puller([this](std::vector<double>& v) { pull_forces(v, true); });
        fy_body.set_puller([this](std::vector<double>& v) { pull_forces(v, false); });
        wall_dist.set_puller([this](std::vector<double>& v) {
            lbm2d_dropin::check(lbm2d_download_wall_dist(h_, v.data()), h_, "wall distance");
        });
    }
    LBMCapabilities(const LBMCapabilities&) = delete;
    LBMCapabilities& operator=(const LBMCapabilities&) = delete;
    ~LBMCapabilities() {
        if (h_) lbm2d_destroy(h_);
    }

    void reset_forces() {
        fx_body.assign(static_cast<size_t>(NX) * NY, 0.0);
        fy_body.assign(static_cast<size_t>(NX) * NY, 0.0);
        fx_body.clear_dirty();
        fy_body.clear_dirty();
    }

    // One execute_time_step on the device (called by lbm.hpp).
    void device_step(double tau, double u_inflow);
    lbm2d_solver* handle() { return h_; }
    // True when the device holds the newest state and the host has changed
    // none of the mirrors the frame writers read since the last step, so the
    // writers can take their fields from the device (lbm2d_frame_fields).
    bool device_state_current(bool thermal) const {
        return h_ && step_version_ > 0 && f.stale() && !obstacle.dirty() &&
               (!thermal || (use_thermal && g_thermal.stale()));
    }
    lbm2d_solver* device_handle() const { return h_; }
    // Immersed-boundary points whose direct forcing the device applies
    // around every step (lbm2d_dropin::attach_ibm); sent with the next step.
    void set_ibm_points(std::vector<double> X, std::vector<double> Y, double dt, double uwx, double uwy) {
        ibm_X_ = std::move(X);
        ibm_Y_ = std::move(Y);
        ibm_dt_ = dt;
        ibm_uwx_ = uwx;
        ibm_uwy_ = uwy;
        ibm_dirty_ = true;
    }

   private:
    void ensure_handle();
    void push_settings();
    void pull_forces(std::vector<double>& v, bool want_x);

    lbm2d_solver* h_ = nullptr;
    int nx_ = 0, ny_ = 0;
    long long forces_version_ = -1, step_version_ = 0;
    std::vector<double> fx_cache_, fy_cache_;
    // last pushed bounce-back geometry
    double sent_cx_ = 0, sent_cy_ = 0, sent_r_ = 0;
    std::vector<std::pair<double, double>> sent_poly_;
    bool sent_is_poly_ = false, sent_moving_ = false, sent_mei_ = true;
    double sent_omega_ = 0, sent_rcx_ = 0, sent_rcy_ = 0;
    std::vector<double> ibm_X_, ibm_Y_;
    double ibm_dt_ = 1.0, ibm_uwx_ = 0.0, ibm_uwy_ = 0.0;
    bool ibm_dirty_ = false;
};

inline void LBMCapabilities::ensure_handle() {
    if (h_) return;
    lbm2d_config cfg{};
    cfg.nx = nx_;
    cfg.ny = ny_;
    cfg.case_type = static_cast<int>(g_case);
    cfg.collision = g_collision == CollisionType::MRT ? LBM2D_MRT : LBM2D_BGK;
    cfg.use_les = g_use_les ? 1 : 0;
    cfg.cs = g_cs;
    cfg.storage = lbm2d_dropin::storage_from_env();
    cfg.device = lbm2d_dropin::device_from_env();
    lbm2d_dropin::check(lbm2d_create(&cfg, &h_), nullptr, "create");
    obstacle.raw();  // the first push below sends the mask
    sent_mei_ = true;
}

inline void LBMCapabilities::push_settings() {
    using lbm2d_dropin::check;
    check(lbm2d_set_case(h_, static_cast<int>(g_case), g_collision == CollisionType::MRT ? 0 : 1, g_use_les ? 1 : 0,
                         g_cs),
          h_, "set case");
    if (obstacle.dirty() || step_version_ == 0) {
        check(lbm2d_set_mask(h_, obstacle.raw().data()), h_, "set mask");
        obstacle.clear_dirty();
    }
    const BounceBackGeometry& g = bb_geom;
    if (g.cx != sent_cx_ || g.cy != sent_cy_ || g.radius != sent_r_) {
        check(lbm2d_set_bb_cylinder(h_, g.cx, g.cy, g.radius), h_, "bb cylinder");
        sent_cx_ = g.cx;
        sent_cy_ = g.cy;
        sent_r_ = g.radius;
    }
    if (g.is_polygon != sent_is_poly_ || (g.is_polygon && g.poly_vertices != sent_poly_)) {
        std::vector<double> xy;
        if (g.is_polygon)
            for (auto& p : g.poly_vertices) {
                xy.push_back(p.first);
                xy.push_back(p.second);
            }
        check(lbm2d_set_bb_polygon(h_, xy.data(), g.is_polygon ? static_cast<int>(g.poly_vertices.size()) : 0), h_,
              "bb polygon");
        sent_is_poly_ = g.is_polygon;
        sent_poly_ = g.poly_vertices;
    }
    if (g.has_moving_wall != sent_moving_ || g.omega != sent_omega_ || g.rot_cx != sent_rcx_ || g.rot_cy != sent_rcy_) {
        check(lbm2d_set_moving_wall(h_, g.has_moving_wall ? 1 : 0, g.omega, g.rot_cx, g.rot_cy), h_, "moving wall");
        sent_moving_ = g.has_moving_wall;
        sent_omega_ = g.omega;
        sent_rcx_ = g.rot_cx;
        sent_rcy_ = g.rot_cy;
    }
    if (g.use_mei_bb != sent_mei_) {
        check(lbm2d_set_mei(h_, g.use_mei_bb ? 1 : 0), h_, "mei");
        sent_mei_ = g.use_mei_bb;
    }
    check(lbm2d_set_body_force(h_, body_force_x), h_, "body force");
    check(lbm2d_set_thermal(h_, use_thermal ? 1 : 0, T_ref, alpha, omega_k, beta, g_buoyancy), h_, "thermal");
    if (f.dirty() || step_version_ == 0) {
        check(lbm2d_upload_f(h_, f.raw().data()), h_, "upload f");
        f.clear_dirty();
    }
    if (g_thermal.dirty() || (step_version_ == 0 && use_thermal)) {
        check(lbm2d_upload_g(h_, g_thermal.raw().data()), h_, "upload g");
        g_thermal.clear_dirty();
    }
    if (ibm_dirty_) {
        check(lbm2d_set_ibm(h_, ibm_X_.data(), ibm_Y_.data(), static_cast<int>(ibm_X_.size()), ibm_dt_, ibm_uwx_,
                            ibm_uwy_),
              h_, "immersed boundary");
        ibm_dirty_ = false;
    }
}

inline void LBMCapabilities::device_step(double tau, double u_inflow) {
    ensure_handle();
    push_settings();
    lbm2d_dropin::check(lbm2d_step(h_, tau, u_inflow, 1), h_, "step");
    ++step_version_;
    f.mark_stale();
    if (use_thermal) g_thermal.mark_stale();
    if (g_case != CaseType::CAVITY) {  // the reference leaves the force fields alone for the cavity
        fx_body.mark_stale();
        fy_body.mark_stale();
    }
    if (g_use_les) wall_dist.mark_stale();
    fx_body.clear_dirty();
    fy_body.clear_dirty();
}

inline void LBMCapabilities::pull_forces(std::vector<double>& v, bool want_x) {
    if (forces_version_ != step_version_) {
        fx_cache_.resize(v.size());
        fy_cache_.resize(v.size());
        lbm2d_dropin::check(lbm2d_download_force_field(h_, fx_cache_.data(), fy_cache_.data()), h_, "forces");
        forces_version_ = step_version_;
    }
    v = want_x ? fx_cache_ : fy_cache_;
}

// ---------------------------------------------------------------- helpers (src/lbm_types.hpp:231-288)
inline void compute_wall_distance(LBMCapabilities& sys) {
    std::vector<uint8_t> m(sys.obstacle.size());
    for (size_t k = 0; k < m.size(); ++k) m[k] = sys.obstacle[k];
    std::vector<double> d(m.size());
    lbm2d_wall_distance(NX, NY, m.data(), d.data());
    for (size_t k = 0; k < d.size(); ++k) sys.wall_dist[k] = d[k];
}

inline double compute_equilibrium(int i, double rho, double u, double v) {
    const double ed = cx[i] * u + cy[i] * v;
    const double usq = u * u + v * v;
    return weights[i] * rho * (1.0 + 3.0 * ed + 4.5 * ed * ed - 1.5 * usq);
}

inline void compute_macros(const double* f_node, double& rho, double& u, double& v) {
    rho = 0.0;
    double mx = 0.0, my = 0.0;
    for (int i = 0; i < 9; ++i) {
        rho += f_node[i];
        mx += f_node[i] * cx[i];
        my += f_node[i] * cy[i];
    }
    u = mx / rho;
    v = my / rho;
}
