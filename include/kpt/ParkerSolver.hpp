// ParkerSolver (ParkerSolver.hpp:69-301) over the C ABI: the lockstep
// Euler-Maruyama Parker step of the header library on the GPU, with the
// reference's constructors, step methods, error messages and return values.
// The packed coefficient basis is the only sampling path (the reference's
// unpacked path computes the same values); it lives on the device.
#pragma once

#include <cmath>
#include <memory>
#include <stdexcept>
#include <vector>

#include "Coefficients.hpp"
#include "RandomManager.hpp"
#include "SolverBase.hpp"

namespace kpt {

class ParkerSolver : public SolverBase {
public:
    using coefficient_field_set_type = ParkerCoefficient::TransportCoefficientFieldSet;
    static constexpr int packed_component_count = ParkerCoefficient::packed_component_count;

    coefficient_field_set_type coefficients;

    ParkerSolver(CartesianGrid2D input_grid, VectorField input_B_vec, VectorField input_V_body)
        : SolverBase(std::move(input_grid), std::move(input_B_vec), std::move(input_V_body)) {}

    ParkerSolver(CartesianGrid2D input_grid, VectorField input_B_vec, VectorField input_V_body,
                 coefficient_field_set_type input_coefficients)
        : SolverBase(std::move(input_grid), std::move(input_B_vec), std::move(input_V_body)),
          coefficients(std::move(input_coefficients)) {
        if (use_packed_ && coefficients.configured()) rebuild_packed_coefficient_basis();
    }

    ParkerSolver(ParticleSystem input_particles, CartesianGrid2D input_grid,
                 VectorField input_B_vec, VectorField input_V_body)
        : SolverBase(std::move(input_particles), std::move(input_grid), std::move(input_B_vec),
                     std::move(input_V_body)) {}

    ParkerSolver(ParticleSystem input_particles, CartesianGrid2D input_grid,
                 VectorField input_B_vec, VectorField input_V_body,
                 coefficient_field_set_type input_coefficients)
        : SolverBase(std::move(input_particles), std::move(input_grid), std::move(input_B_vec),
                     std::move(input_V_body)),
          coefficients(std::move(input_coefficients)) {
        if (use_packed_ && coefficients.configured()) rebuild_packed_coefficient_basis();
    }

    // set_coefficient_fields (ParkerSolver.hpp:157-163).
    void set_coefficient_fields(coefficient_field_set_type input_coefficients) {
        coefficients = std::move(input_coefficients);
        if (use_packed_ && coefficients.configured()) rebuild_packed_coefficient_basis();
    }
    void set_use_packed_coefficient_basis(bool enabled) {
        use_packed_ = enabled;
        if (use_packed_ && coefficients.configured()) rebuild_packed_coefficient_basis();
    }
    bool packed_coefficient_basis_enabled() const { return use_packed_; }

    // rebuild_packed_coefficient_basis (ParkerSolver.hpp:185-195): the basis
    // is copied to the device.
    void rebuild_packed_coefficient_basis() {
        if (!coefficients.configured()) {
            throw std::runtime_error("ParkerSolver: coefficient fields are not configured.");
        }
        if (coefficients.packed->size() != grid.point_count() * packed_component_count) {
            throw std::runtime_error(
                "ParkerSolver: packed coefficient basis point count does not match the grid.");
        }
        const int ratio = coefficients.constant_ratio ? 1 : 0;
        if (solver_) {
            check(kpt_parker_solver_set_basis(solver_.get(), coefficients.packed->data(), ratio));
            return;
        }
        kpt_parker_solver* raw = nullptr;
        check(kpt_parker_solver_create(grid.context().get(), grid.get(),
                                       coefficients.packed->data(), ratio, courant_scale, &raw));
        solver_ = std::shared_ptr<kpt_parker_solver>(
            raw, [](kpt_parker_solver* s) { kpt_parker_solver_destroy(s); });
    }

    // compute_adaptive_time_step (ParkerSolver.hpp:208-222).
    double compute_adaptive_time_step() const {
        prepare();
        double dt = 0.0;
        check(kpt_parker_compute_time_step(particles.ctx(), solver_.get(), particles.get(), &dt));
        return dt;
    }

    // advance_deterministic (ParkerSolver.hpp:229-259); returns the dt used.
    double advance_deterministic() {
        prepare();
        double dt = 0.0;
        check(kpt_parker_advance_deterministic(particles.ctx(), solver_.get(), particles.get(),
                                               &dt));
        dT = dt;
        return dt;
    }

    // advance_stochastic (ParkerSolver.hpp:265-294); returns the dt used.
    // The noise is the keyed stream of (random_manager.seed, particle index,
    // step), the step taken from the manager.
    double advance_stochastic(const RandomManager& random_manager) {
        prepare();
        double dt = 0.0;
        check(kpt_parker_advance_stochastic(particles.ctx(), solver_.get(), particles.get(),
                                            random_manager.seed, random_manager.next_step(),
                                            &dt));
        dT = dt;
        return dt;
    }
    double advance_sde(const RandomManager& random_manager) {
        return advance_stochastic(random_manager);
    }

    // Extension: `steps` stochastic steps recorded into one CUDA graph and
    // replayed, the dt staying on the device; returns each step's dt.  Same
    // results as `steps` advance_stochastic calls.
    std::vector<double> advance_stochastic_steps(const RandomManager& random_manager,
                                                 std::uint32_t steps) {
        prepare();
        std::vector<double> dts(steps);
        const std::uint32_t first = random_manager.step();
        check(kpt_parker_advance_stochastic_steps(particles.ctx(), solver_.get(),
                                                  particles.get(), random_manager.seed, first,
                                                  steps, dts.data()));
        random_manager.set_step(first + steps);
        if (steps > 0) dT = dts.back();
        return dts;
    }

    // Extension: one step with the caller's standard normals,
    // normals[k * count + i] (k = 0, 1, 2 spatial, 3 parallel).
    double advance_with_noise(const std::vector<double>& normals) {
        prepare();
        if (normals.size() != 4 * particles.particle_count()) {
            throw std::runtime_error("ParkerSolver: normals must hold 4 x particle_count values.");
        }
        double dt = 0.0;
        check(kpt_parker_advance_with_noise(particles.ctx(), solver_.get(), particles.get(),
                                            normals.data(), &dt));
        dT = dt;
        return dt;
    }

    // Extension: the arithmetic of the steps, KPT_PRECISION_F64 (the
    // reference's, the default) or KPT_PRECISION_MIXED (FP32 basis, terms and
    // noise with FP64 positions, momenta and dt; within a stated tolerance of
    // the FP64 steps).
    void set_precision(int precision) { precision_ = precision; }
    int precision() const { return precision_; }

private:
    int precision_{KPT_PRECISION_F64};
    bool use_packed_{true};
    std::shared_ptr<kpt_parker_solver> solver_;

    // validate_for_deterministic_step (ParkerSolver.hpp:312-342), the host part.
    void prepare() const {
        if (!coefficients.configured() || !solver_) {
            throw std::runtime_error("ParkerSolver: coefficient fields are not configured.");
        }
        if (!particles) {
            throw std::runtime_error("ParkerSolver: the solver has no particle system.");
        }
        check(kpt_parker_solver_set_courant(solver_.get(), courant_scale));
        check(kpt_parker_solver_set_precision(solver_.get(), precision_));
    }
};

}  // namespace kpt
