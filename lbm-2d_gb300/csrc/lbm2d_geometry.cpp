// lbm2d_geometry.cpp -- host set-up of flags and boundary records.
// Compiled with -ffp-contract=off: q and the wall velocity must reproduce the
// reference's double arithmetic bit for bit.
#include "lbm2d_geometry.h"

#include <cmath>
#include <cstring>
#include <deque>

#include "lbm2d_internal.h"

namespace lbm2d {
namespace {
constexpr int CX[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
constexpr int CY[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};
constexpr int BB[9] = {0, 3, 4, 1, 2, 7, 8, 5, 6};
constexpr int CASE_CAVITY = 1, CASE_RIBS = 3, CASE_HILLS = 9, CASE_NEAR_WALL = 10;
}  // namespace

// BounceBackGeometry::q_cylinder / q_polygon / compute_q, src/lbm_types.hpp:118-176
double BBGeometry::q(double xf, double yf, int i) const {
    const double ex = static_cast<double>(CX[i]), ey = static_cast<double>(CY[i]);
    if (is_polygon) {
        const int n = static_cast<int>(poly.size() / 2);
        if (n < 3) return 1.0;
        double best = 1.0;
        for (int k = 0; k < n; ++k) {
            const int k2 = (k + 1) % n;
            const double x1 = poly[2 * k], y1 = poly[2 * k + 1];
            const double x2 = poly[2 * k2], y2 = poly[2 * k2 + 1];
            const double ddx = x2 - x1, ddy = y2 - y1;
            const double den = ex * ddy - ey * ddx;
            if (std::abs(den) < 1e-15) continue;
            const double t = ((x1 - xf) * ddy - (y1 - yf) * ddx) / den;
            const double s = ((x1 - xf) * ey - (y1 - yf) * ex) / den;
            if (t > 0.0 && t <= best && s >= 0.0 && s <= 1.0) best = t;
        }
        return best;
    }
    const double dx = xf - cx, dy = yf - cy;
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

// BounceBackGeometry::compute_wall_velocity, src/lbm_types.hpp:106-114
void BBGeometry::wall_velocity(double px, double py, double& ux, double& uy) const {
    if (!has_moving_wall) {
        ux = 0.0;
        uy = 0.0;
        return;
    }
    const double dx = px - rot_cx, dy = py - rot_cy;
    ux = -omega * dy;
    uy = omega * dx;
}

void wall_distance(int nx, int ny, const uint8_t* mask, std::vector<double>& out) {
    const size_t n = static_cast<size_t>(nx) * ny;
    out.assign(n, 1e9);
    std::deque<int> qu;
    for (size_t k = 0; k < n; ++k)
        if (mask[k]) {
            out[k] = 0.0;
            qu.push_back(static_cast<int>(k));
        }
    while (!qu.empty()) {
        const int k = qu.front();
        qu.pop_front();
        const int x = k % nx, y = k / nx;
        const double d = out[k] + 1.0;
        const int ax[4] = {x - 1, x + 1, x, x}, ay[4] = {y, y, y - 1, y + 1};
        for (int t = 0; t < 4; ++t) {
            if (ax[t] < 0 || ax[t] >= nx || ay[t] < 0 || ay[t] >= ny) continue;
            const int m = ay[t] * nx + ax[t];
            if (mask[m]) continue;
            if (d < out[m]) {
                out[m] = d;
                qu.push_back(m);
            }
        }
    }
}

bool build_geometry(const GeometryInput& in, GeometryTables& t, std::string& err) {
    const int nx = in.nx, ny = in.ny;
    if (nx < 3 || ny < 3) {
        err = "grid must be at least 3x3";
        return false;
    }
    const size_t n = static_cast<size_t>(nx) * ny;
    const uint8_t* m = in.mask;
    const BBGeometry& g = *in.bb;
    const bool cavity = in.case_type == CASE_CAVITY;
    const bool periodic = in.case_type == CASE_RIBS || in.case_type == CASE_HILLS;
    // nodes a boundary condition may rewrite (src/lbm.hpp:531-540): the lid
    // row of the cavity, the inlet and outlet columns of the open cases.  They
    // get a record even without bounce-back links, so the step kernels find
    // every node that needs more than the plain pull from its flags alone.
    auto bc_node = [&](int x, int y) {
        if (cavity) return y == ny - 1;
        if (periodic) return false;
        return x == 0 || x == nx - 1;
    };
    const bool interp = g.valid();
    t = GeometryTables();
    t.flags.assign(n, 0u);
    if (in.les) wall_distance(nx, ny, m, t.wall_dist);
    auto solid = [&](int x, int y) { return m[static_cast<size_t>(y) * nx + x] != 0; };

    for (int y = 0; y < ny; ++y) {
        for (int x = 0; x < nx; ++x) {
            const size_t id = static_cast<size_t>(y) * nx + x;
            if (m[id]) {
                t.flags[id] = FLAG_SOLID;
                continue;
            }
            uint32_t ftypes = 0, gbb = 0, fmask = 0;
            double q[9] = {0}, uw[18] = {0};
            for (int j = 1; j < 9; ++j) {
                const int i = BB[j];  // link direction of the reference's push
                const int tx = x + CX[i], ty = y + CY[i];
                // momentum streaming, src/lbm.hpp:408-484
                uint32_t st = SLOT_REGULAR;
                if (cavity) {
                    if (tx < 0 || tx >= nx || ty < 0 || ty >= ny)
                        st = SLOT_SIMPLE_BB;
                    else if (solid(tx, ty))
                        st = interp ? SLOT_INTERP : SLOT_SIMPLE_BB;
                } else if (periodic) {
                    const int wx = (tx + nx) % nx, wy = (ty + ny) % ny;
                    if (solid(wx, wy)) st = SLOT_SIMPLE_BB;
                } else {
                    const int wy = (ty + ny) % ny;
                    if (tx < 0 || tx >= nx)
                        st = SLOT_ZERO;
                    else if (solid(tx, wy))
                        st = interp ? SLOT_INTERP : SLOT_SIMPLE_BB;
                }
                ftypes |= st << (2 * j);
                if (st == SLOT_INTERP) {
                    q[j] = g.q(static_cast<double>(x), static_cast<double>(y), i);
                    g.wall_velocity(static_cast<double>(x + CX[i]), static_cast<double>(y + CY[i]), uw[2 * j],
                                    uw[2 * j + 1]);
                    t.any_interp = true;
                }
                // thermal streaming, src/lbm.hpp:490-528 (y always wraps; x wraps
                // only in the periodic cases; outside or solid -> bounce-back)
                if (in.thermal) {
                    const int wy = (ty + ny) % ny;
                    const int wx = periodic ? (tx + nx) % nx : tx;
                    if (wx < 0 || wx >= nx || solid(wx, wy)) gbb |= 1u << j;
                }
                // momentum-exchange force, src/lbm.hpp:543-581
                if (!cavity) {
                    int fx = tx, fy = (ty + ny) % ny;
                    bool skip = false;
                    if (periodic)
                        fx = (tx + nx) % nx;
                    else if (tx < 0 || tx >= nx)
                        skip = true;
                    if (!skip && solid(fx, fy)) {
                        bool count = true;
                        if (in.case_type == CASE_NEAR_WALL) {
                            const double dx = static_cast<double>(fx) - g.cx;
                            const double dy = static_cast<double>(fy) - g.cy;
                            if (std::sqrt(dx * dx + dy * dy) > g.radius) count = false;
                        }
                        if (count) fmask |= 1u << j;
                    }
                }
            }
            if (ftypes == 0 && gbb == 0 && !bc_node(x, y)) {
                // the LES wall distance as an FP32 bit pattern: an integer
                // below 2^21 (or the reference's 1e9 for "no wall") has its
                // two lowest mantissa bits zero, so bits 0-1 stay free for the
                // solid / boundary flags and the kernels decode it with a mask
                uint32_t bits = 0;
                if (in.les) {
                    const double d = t.wall_dist[id];
                    if (d < 1e9 && d >= static_cast<double>(1u << 21)) {
                        err = "wall distance exceeds 2^21 nodes";
                        return false;
                    }
                    const float df = d >= 1e9 ? 1e9f : static_cast<float>(d);
                    std::memcpy(&bits, &df, sizeof(bits));
                }
                t.flags[id] = bits;
                continue;
            }
            const size_t r = t.rec_info.size();
            if (r >= MAX_RECORDS) {
                err = "too many boundary nodes";
                return false;
            }
            t.flags[id] = FLAG_BOUNDARY | (static_cast<uint32_t>(r) << 2);
            t.rec_info.push_back(ftypes | (gbb << REC_GBB_SHIFT));
            t.rec_force.push_back(fmask);
            t.rec_node.push_back(static_cast<int32_t>(id));
            t.rec_wd.push_back(in.les ? t.wall_dist[id] : 0.0);
            for (int j = 0; j < 9; ++j) t.rec_q.push_back(q[j]);
            for (int j = 0; j < 18; ++j) t.rec_uw.push_back(uw[j]);
            if (fmask) ++t.n_force_nodes;
        }
    }
    t.any_moving = g.has_moving_wall;
    return true;
}

int force_block_slots(const GeometryTables& t, int nx, int ny, int bx, int by, int threads, std::vector<int>& slots) {
    const int gx = (nx + bx - 1) / bx, gy = (ny + by - 1) / by;
    slots.assign(static_cast<size_t>(gx) * gy, -1);
    for (size_t r = 0; r < t.rec_force.size(); ++r) {
        if (!t.rec_force[r]) continue;
        const int id = t.rec_node[r];
        const int x = id % nx, y = id / nx;
        slots[static_cast<size_t>(y / by) * gx + x / bx] = 0;
    }
    const int warps = (threads + 31) / 32;  // each force block owns one slot per warp
    int k = 0;
    for (auto& s : slots)
        if (s == 0) {
            s = k;
            k += warps;
        }
    return k;
}

}  // namespace lbm2d
