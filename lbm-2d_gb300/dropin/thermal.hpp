// thermal.hpp -- drop-in replacement of the reference's src/thermal.hpp.
//
// The thermal double-distribution step itself runs on the GPU inside
// execute_time_step; these are the same host-side helpers the reference
// offers to drivers (equilibrium, node-level collision, Boussinesq force,
// temperature, wall conditions, Nusselt number), with the same formulas.
#pragma once
#include <array>
#include <cmath>

#include "lbm_types.hpp"

// src/thermal.hpp:17-20
constexpr std::array<double, 9> thermal_weights = {4.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0,
                                                   1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0};

// g_i^eq = w_i T (1 + 3 e.u + 4.5 (e.u)^2 - 1.5 u^2), src/thermal.hpp:25-30
inline double thermal_equilibrium(int i, double T, double u, double v) {
    const double ed = cx[i] * u + cy[i] * v;
    const double usq = u * u + v * v;
    return thermal_weights[i] * T * (1.0 + 3.0 * ed + 4.5 * ed * ed - 1.5 * usq);
}

// SRT relaxation of one node, src/thermal.hpp:35-41
inline void thermal_collide(double* g_node, double T, double u, double v, double omega_k) {
    for (int i = 0; i < 9; ++i) g_node[i] -= omega_k * (g_node[i] - thermal_equilibrium(i, T, u, v));
}

// F = -rho_0 beta (T - T_ref) g, src/thermal.hpp:46-52
inline void boussinesq_force(double T, double T_ref, double rho_0, double beta, double g_x, double g_y, double& fx,
                             double& fy) {
    const double dT = T - T_ref;
    fx = -rho_0 * beta * dT * g_x;
    fy = -rho_0 * beta * dT * g_y;
}

// src/thermal.hpp:55-60
inline void compute_temperature(const double* g_node, double& T) {
    T = 0.0;
    for (int i = 0; i < 9; ++i) T += g_node[i];
}

enum class ThermalBC { ISOTHERMAL, ADIABATIC, HEAT_FLUX };

// src/thermal.hpp:70-75
inline void apply_thermal_isothermal(double* g_node, double T_wall, double u_wall = 0.0, double v_wall = 0.0) {
    for (int i = 0; i < 9; ++i) g_node[i] = thermal_equilibrium(i, T_wall, u_wall, v_wall);
}

// src/thermal.hpp:78-83
inline void apply_thermal_adiabatic(double* g_node, const double* g_opp) {
    for (int i = 0; i < 9; ++i) g_node[i] = g_opp[bounce_back[i]];
}

// src/thermal.hpp:88-91
inline double compute_nusselt(double dTdr_wall, double D, double T_wall, double T_inf) {
    if (std::abs(T_wall - T_inf) < 1e-12) return 0.0;
    return -2.0 * dTdr_wall * D / (T_wall - T_inf);
}
