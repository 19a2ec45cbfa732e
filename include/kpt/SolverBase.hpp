// SolverBase (SolverBase.hpp:13-96): the state every library solver holds.
#pragma once

#include <cmath>
#include <stdexcept>

#include "Grid.hpp"
#include "ParticleSystem.hpp"

namespace kpt {

struct SolverBase {
    static constexpr int space_dim = 2;
    static constexpr int vec_dim = 3;

    ParticleSystem particles;
    CartesianGrid2D grid;
    VectorField B_vec, V_body;
    double dT{1.0};
    double courant_scale{0.3};
    double Omega0{0.0};

    SolverBase(CartesianGrid2D input_grid, VectorField input_B_vec, VectorField input_V_body)
        : grid(std::move(input_grid)), B_vec(std::move(input_B_vec)),
          V_body(std::move(input_V_body)) {}

    SolverBase(ParticleSystem input_particles, CartesianGrid2D input_grid,
               VectorField input_B_vec, VectorField input_V_body)
        : particles(std::move(input_particles)), grid(std::move(input_grid)),
          B_vec(std::move(input_B_vec)), V_body(std::move(input_V_body)) {}

    void set_dimensionless_time_step(double input_time_step) { dT = input_time_step; }
    void set_dimensionless_courant_scale(double input_courant_scale) {
        courant_scale = input_courant_scale;
    }
    void set_dimensionless_rotation_rate(double input_rotation_rate) {
        Omega0 = input_rotation_rate;
    }
    double time_step() const { return dT; }
    double courant_number() const { return courant_scale; }
    double rotation_rate() const { return Omega0; }
};

}  // namespace kpt
