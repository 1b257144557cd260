// lbm2d_geometry.h -- host-side set-up of the boundary records (no device code).
//
// Given the solid mask, the case type and the interpolated-bounce-back
// geometry, classify every pull slot of every fluid node the way the
// reference's push streaming (src/lbm.hpp:408-484), thermal streaming
// (:490-528) and force pass (:543-581) treat the corresponding link, and
// compute q and the wall velocity of interpolated links with the reference's
// own double arithmetic (BounceBackGeometry, src/lbm_types.hpp:106-176), so the
// link list is bit-exact.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace lbm2d {

struct BBGeometry {
    double cx = 0.0, cy = 0.0, radius = 0.0;  // last placed circle
    std::vector<double> poly;                  // x0,y0,x1,y1,...
    bool is_polygon = false;
    bool has_moving_wall = false;
    double omega = 0.0, rot_cx = 0.0, rot_cy = 0.0;
    bool use_mei = true;
    bool valid() const { return radius > 0.0 || is_polygon; }
    double q(double xf, double yf, int i) const;
    void wall_velocity(double px, double py, double& ux, double& uy) const;
};

struct GeometryInput {
    int nx = 0, ny = 0;
    int case_type = 0;
    bool thermal = false;
    bool les = false;
    const uint8_t* mask = nullptr;
    const BBGeometry* bb = nullptr;
};

struct GeometryTables {
    std::vector<uint32_t> flags;      // per node
    std::vector<uint32_t> rec_info;   // per record
    std::vector<uint32_t> rec_force;  // per record
    std::vector<int32_t> rec_node;    // per record: node index
    std::vector<double> rec_wd;       // per record
    std::vector<double> rec_q;        // per record * 9
    std::vector<double> rec_uw;       // per record * 18
    std::vector<double> wall_dist;    // per node (only when les)
    bool any_interp = false;
    bool any_moving = false;
    int n_force_nodes = 0;
};

// Exact 4-neighbour distance to the nearest obstacle: the fixed point that
// compute_wall_distance (src/lbm_types.hpp:231-264) reaches, found by a
// multi-source breadth-first search.  Unreachable nodes get 1e9.
void wall_distance(int nx, int ny, const uint8_t* mask, std::vector<double>& out);

bool build_geometry(const GeometryInput& in, GeometryTables& out, std::string& err);

// Force-reduction slots for a launch shape (bx, by): every block holding a
// force node gets one slot per warp starting at slots[block] (-1 otherwise);
// returns the total slot count.
// (bx, by) is the node footprint of a block; threads its thread count.
int force_block_slots(const GeometryTables& t, int nx, int ny, int bx, int by, int threads, std::vector<int>& slots);

}  // namespace lbm2d
