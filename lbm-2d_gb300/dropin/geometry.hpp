// geometry.hpp -- drop-in replacement of the reference's src/geometry.hpp.
// The arithmetic lives in the library's host services (include/lbm2d.h), so
// polygons and masks are bit-exact with the reference.
#pragma once
#include <utility>
#include <vector>

#include "lbm2d.h"

// src/geometry.hpp:17-90
inline std::vector<std::pair<double, double>> naca_coords(int series, int n = 200) {
    std::vector<double> buf(static_cast<size_t>(4) * (n > 1 ? n : 2));
    const int k = lbm2d_naca_coords(series, n, buf.data());
    std::vector<std::pair<double, double>> out(k);
    for (int i = 0; i < k; ++i) out[i] = {buf[2 * i], buf[2 * i + 1]};
    return out;
}

// src/geometry.hpp:95-114
inline void transform_points(std::vector<std::pair<double, double>>& pts, double cx_, double cy_, double scale,
                             double angle_deg) {
    std::vector<double> xy;
    xy.reserve(pts.size() * 2);
    for (auto& p : pts) {
        xy.push_back(p.first);
        xy.push_back(p.second);
    }
    lbm2d_transform_points(xy.data(), static_cast<int>(pts.size()), cx_, cy_, scale, angle_deg);
    for (size_t i = 0; i < pts.size(); ++i) pts[i] = {xy[2 * i], xy[2 * i + 1]};
}

// src/geometry.hpp:120-134
inline bool point_in_polygon(double px, double py, const std::vector<std::pair<double, double>>& poly) {
    std::vector<double> xy;
    xy.reserve(poly.size() * 2);
    for (auto& p : poly) {
        xy.push_back(p.first);
        xy.push_back(p.second);
    }
    return lbm2d_point_in_polygon(px, py, xy.data(), static_cast<int>(poly.size())) != 0;
}
