// lbm2d_ibm.cpp -- immersed-boundary direct forcing on the device (host side).
//
// The reference's airfoil driver (src/airfoil_ibm.cpp:121-176, with the
// ImmersedBoundary of src/ibm.hpp) wraps every step in four host loops:
// velocity at the Lagrangian points from the fluid nodes of their 5x5 delta
// stencils, the no-slip force (U_wall - U) / dt, spreading to a full-size
// grid force, and after the step an explicit forcing of every fluid node.
// Here the points are static, so the stencils and their kernel weights are
// computed once on the host: every node in some stencil is a "band" node,
// with a per-node band index on the device, the band's spread lists (points
// in increasing order, as the reference accumulates) and the points'
// interpolation lists (stencil nodes in the driver's y-major order).  Each
// step then costs one small kernel over the band (see lbm2d_kernels.cu)
// instead of passes over the whole grid.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "lbm2d_runtime.h"

namespace lbm2d {
namespace rt {
namespace {

// ibm_delta, src/ibm.hpp:16-19: the 4-point cosine delta of Peskin.
double ibm_delta(double r) {
    if (std::fabs(r) >= 2.0) return 0.0;
    return 0.25 * (1.0 + std::cos(0.5 * M_PI * r));
}

// ibm_kernel, src/ibm.hpp:22-24
double ibm_kernel(double dx, double dy) { return ibm_delta(dx) * ibm_delta(dy); }

// Visit the stencil of point (X, Y) in the reference's loop order: y from
// floor(Y)-2 to floor(Y)+2, x likewise, nodes inside the grid with a
// non-zero kernel weight.
template <class Fn>
void for_stencil(int nx, int ny, double X, double Y, Fn&& fn) {
    const int x0 = static_cast<int>(std::floor(X)) - 2, x1 = static_cast<int>(std::floor(X)) + 2;
    const int y0 = static_cast<int>(std::floor(Y)) - 2, y1 = static_cast<int>(std::floor(Y)) + 2;
    for (int y = y0; y <= y1; ++y) {
        if (y < 0 || y >= ny) continue;
        for (int x = x0; x <= x1; ++x) {
            if (x < 0 || x >= nx) continue;
            const double w = ibm_kernel(x - X, y - Y);
            if (w == 0.0) continue;
            fn(static_cast<uint32_t>(y) * static_cast<uint32_t>(nx) + static_cast<uint32_t>(x), w);
        }
    }
}

size_t align_up(size_t v) { return (v + 255) & ~size_t(255); }

// Buffer block: uv[2nb] | F[2nb] | lag[2][4np].  lag slot ibm_next holds the
// point forces the next step applies, the other slot those the last step
// applied.
double* F_buf(const lbm2d_solver* h) { return h->d_ibm_buf + 2 * (size_t)h->ibm_nb; }
double* lag_slot(const lbm2d_solver* h, int slot) {
    return h->d_ibm_buf + 4 * (size_t)h->ibm_nb + 4 * (size_t)h->ibm_np * slot;
}

IbmParams launch_params(const lbm2d_solver* h, int in_slot) {
    IbmParams q = h->ibm_q;
    q.uv = h->d_ibm_buf;
    q.F = F_buf(h);
    q.lag_in = lag_slot(h, in_slot);
    q.lag_out = lag_slot(h, in_slot ^ 1);
    return q;
}

}  // namespace

void ibm_release(lbm2d_solver* h) {
    if (h->d_ibm_band) cudaFreeAsync(h->d_ibm_band, h->stream);
    if (h->d_ibm_tab) cudaFreeAsync(h->d_ibm_tab, h->stream);
    if (h->d_ibm_buf) cudaFreeAsync(h->d_ibm_buf, h->stream);
    h->d_ibm_band = nullptr;
    h->d_ibm_tab = nullptr;
    h->d_ibm_buf = nullptr;
    h->ibm_np = h->ibm_nb = 0;
    h->ibm_next = 0;
    h->ibm_q = IbmParams{};
}

// The forcing the current (rebuilt) state carries: the force of the last step.
void ibm_state_params(const lbm2d_solver* h, KParams& p) {
    if (!ibm_active(h)) return;
    p.ibm_band = h->d_ibm_band;
    p.ibm_F = F_buf(h);
}

int ibm_after_step(lbm2d_solver* h, const KParams& step) {
    if (!ibm_active(h)) return LBM2D_OK;
    const IbmParams q = launch_params(h, h->ibm_next);
    const int e = launch_ibm_after_step(h->storage, step, q, h->stream);
    h->launches += 2;
    if (e) return cuda_fail(h, (cudaError_t)e, "immersed boundary");
    return LBM2D_OK;
}

int ibm_from_stage(lbm2d_solver* h, const KParams& p) {
    if (!ibm_active(h)) return LBM2D_OK;
    IbmParams q = launch_params(h, h->ibm_next ^ 1);  // lag_out: what the next step applies
    const int e = launch_ibm_from_stage(h->storage, p, q, h->d_stage_f, h->stream);
    h->launches += 2;
    if (e) return cuda_fail(h, (cudaError_t)e, "immersed boundary");
    return LBM2D_OK;
}

}  // namespace rt
}  // namespace lbm2d

using namespace lbm2d::rt;

extern "C" {

int lbm2d_ibm_points_from_polygon(const double* xy, int n, double spacing, double* X, double* Y, int cap) {
    if (!xy || n < 3 || !(spacing > 0.0)) return 0;
    double total_len = 0.0;
    for (int i = 0; i < n; ++i) {
        const int j = (i + 1) % n;
        const double dx = xy[2 * j] - xy[2 * i];
        const double dy = xy[2 * j + 1] - xy[2 * i + 1];
        total_len += std::sqrt(dx * dx + dy * dy);
    }
    const int n_points = std::max(8, static_cast<int>(total_len / spacing));
    for (int k = 0; k < n_points && k < cap && X && Y; ++k) {
        const double t = static_cast<double>(k) / n_points;
        const double seg = t * n;
        const int i = static_cast<int>(seg) % n;
        const int j = (i + 1) % n;
        const double f = seg - std::floor(seg);
        X[k] = xy[2 * i] + f * (xy[2 * j] - xy[2 * i]);
        Y[k] = xy[2 * i + 1] + f * (xy[2 * j + 1] - xy[2 * i + 1]);
    }
    return n_points;
}

int lbm2d_set_ibm(lbm2d_solver* h, const double* X, const double* Y, int npts, double dt, double u_wall_x,
                  double u_wall_y) {
    int rc;
    if ((rc = check_handle(h))) return rc;
    if (npts < 0 || (npts > 0 && (!X || !Y)) || !(dt > 0.0))
        return fail(h, LBM2D_ERR_INVALID, "immersed boundary: points and dt > 0 required");
    for (int p = 0; p < npts; ++p)
        if (!std::isfinite(X[p]) || !std::isfinite(Y[p]) || std::fabs(X[p]) > 1e9 || std::fabs(Y[p]) > 1e9)
            return fail(h, LBM2D_ERR_INVALID, "immersed boundary: point coordinates must be finite");
    if (npts > 0 && h->thermal)
        return fail(h, LBM2D_ERR_INVALID, "immersed boundary: not available with the thermal DDF");
    if (npts > 0 && h->in_batch) return fail(h, LBM2D_ERR_INVALID, "immersed boundary: solver is in a batch");
    // the current state keeps the forcing it carries: rebuild it first
    if ((rc = before_setting_change(h))) return rc;
    ibm_release(h);
    if (npts == 0) return LBM2D_OK;
    const int nx = h->nx, ny = h->ny;
    // band nodes (sorted), per-node band index
    std::vector<uint32_t> nodes;
    for (int p = 0; p < npts; ++p)
        for_stencil(nx, ny, X[p], Y[p], [&](uint32_t n, double) { nodes.push_back(n); });
    std::sort(nodes.begin(), nodes.end());
    nodes.erase(std::unique(nodes.begin(), nodes.end()), nodes.end());
    const int nb = (int)nodes.size();
    std::vector<int> band(h->N, -1);
    for (int b = 0; b < nb; ++b) band[nodes[b]] = b;
    // interpolation lists (per point, stencil order) and spread lists (per
    // band node, points in increasing order)
    std::vector<int> ip_start(npts + 1, 0), ip_band;
    std::vector<double> ip_w;
    std::vector<std::vector<std::pair<int, double>>> per(nb);
    for (int p = 0; p < npts; ++p) {
        for_stencil(nx, ny, X[p], Y[p], [&](uint32_t n, double w) {
            ip_band.push_back(band[n]);
            ip_w.push_back(w);
            per[band[n]].push_back({p, w});
        });
        ip_start[p + 1] = (int)ip_band.size();
        if (ip_start[p + 1] - ip_start[p] > 25) return fail(h, LBM2D_ERR_INVALID, "internal: stencil over 5x5");
    }
    std::vector<int> sp_start(nb + 1, 0), sp_pt;
    std::vector<double> sp_w;
    for (int b = 0; b < nb; ++b) {
        for (const auto& e : per[b]) {
            sp_pt.push_back(e.first);
            sp_w.push_back(e.second);
        }
        sp_start[b + 1] = (int)sp_pt.size();
    }
    // one table block: [band_node | sp_start | sp_pt | sp_w | ip_start | ip_band | ip_w]
    const size_t o_bn = 0, o_ss = align_up(o_bn + nb * sizeof(uint32_t));
    const size_t o_sp = align_up(o_ss + (nb + 1) * sizeof(int));
    const size_t o_sw = align_up(o_sp + sp_pt.size() * sizeof(int));
    const size_t o_is = align_up(o_sw + sp_w.size() * sizeof(double));
    const size_t o_ib = align_up(o_is + (npts + 1) * sizeof(int));
    const size_t o_iw = align_up(o_ib + ip_band.size() * sizeof(int));
    const size_t tab_bytes = align_up(o_iw + ip_w.size() * sizeof(double));
    std::vector<char> tab(tab_bytes, 0);
    std::memcpy(tab.data() + o_bn, nodes.data(), nb * sizeof(uint32_t));
    std::memcpy(tab.data() + o_ss, sp_start.data(), (nb + 1) * sizeof(int));
    std::memcpy(tab.data() + o_sp, sp_pt.data(), sp_pt.size() * sizeof(int));
    std::memcpy(tab.data() + o_sw, sp_w.data(), sp_w.size() * sizeof(double));
    std::memcpy(tab.data() + o_is, ip_start.data(), (npts + 1) * sizeof(int));
    std::memcpy(tab.data() + o_ib, ip_band.data(), ip_band.size() * sizeof(int));
    std::memcpy(tab.data() + o_iw, ip_w.data(), ip_w.size() * sizeof(double));
    const size_t buf_doubles = 2 * (size_t)nb + 2 * (size_t)nb + 2 * 4 * (size_t)npts;
    void* d_band = nullptr;
    void* d_tab = nullptr;
    void* d_buf = nullptr;
    if (cudaMallocAsync(&d_band, h->N * sizeof(int), h->stream) != cudaSuccess ||
        cudaMallocAsync(&d_tab, tab_bytes, h->stream) != cudaSuccess ||
        cudaMallocAsync(&d_buf, buf_doubles * sizeof(double), h->stream) != cudaSuccess) {
        cudaGetLastError();
        if (d_band) cudaFreeAsync(d_band, h->stream);
        if (d_tab) cudaFreeAsync(d_tab, h->stream);
        if (d_buf) cudaFreeAsync(d_buf, h->stream);
        return fail(h, LBM2D_ERR_OOM, "immersed boundary tables");
    }
    h->d_ibm_band = static_cast<int*>(d_band);
    h->d_ibm_tab = static_cast<char*>(d_tab);
    h->d_ibm_buf = static_cast<double*>(d_buf);
    cudaError_t e = cudaMemcpyAsync(d_band, band.data(), h->N * sizeof(int), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_tab, tab.data(), tab_bytes, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_buf, 0, buf_doubles * sizeof(double), h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);  // host tables leave scope
    if (e != cudaSuccess) {
        ibm_release(h);
        return cuda_fail(h, e, "immersed boundary upload");
    }
    lbm2d::IbmParams& q = h->ibm_q;
    q = lbm2d::IbmParams{};
    q.nb = nb;
    q.np = npts;
    q.band_node = reinterpret_cast<const uint32_t*>(h->d_ibm_tab + o_bn);
    q.sp_start = reinterpret_cast<const int*>(h->d_ibm_tab + o_ss);
    q.sp_pt = reinterpret_cast<const int*>(h->d_ibm_tab + o_sp);
    q.sp_w = reinterpret_cast<const double*>(h->d_ibm_tab + o_sw);
    q.ip_start = reinterpret_cast<const int*>(h->d_ibm_tab + o_is);
    q.ip_band = reinterpret_cast<const int*>(h->d_ibm_tab + o_ib);
    q.ip_w = reinterpret_cast<const double*>(h->d_ibm_tab + o_iw);
    q.dt = dt;
    q.uwx = u_wall_x;
    q.uwy = u_wall_y;
    h->ibm_np = npts;
    h->ibm_nb = nb;
    h->ibm_next = 0;
    h->ibm_dt = dt;
    h->ibm_uwx = u_wall_x;
    h->ibm_uwy = u_wall_y;
    return LBM2D_OK;
}

int lbm2d_ibm_lagrangian(lbm2d_solver* h, double* U, double* V, double* FX, double* FY) {
    int rc;
    if ((rc = check_handle(h))) return rc;
    if (!ibm_active(h)) return fail(h, LBM2D_ERR_STATE, "no immersed boundary installed");
    if (h->staged || h->steps_since_collide == 0) return fail(h, LBM2D_ERR_STATE, "no step since the last upload");
    const size_t np = (size_t)h->ibm_np;
    // the points' values whose forces the last step applied
    const double* lag = lag_slot(h, h->ibm_next ^ 1);
    double* outs[4] = {U, V, FX, FY};
    for (int k = 0; k < 4; ++k) {
        if (!outs[k]) continue;
        const cudaError_t e =
            cudaMemcpyAsync(outs[k], lag + k * np, np * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
        if (e != cudaSuccess) return cuda_fail(h, e, "immersed boundary D2H");
    }
    const cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "immersed boundary D2H");
    return LBM2D_OK;
}

}  // extern "C"
