// FocusTransportSolver / FocusSolver (FocusSolver.hpp:79-303, :1889) over
// the C ABI: the lockstep focused-transport step of the header library on
// the GPU (streaming, drifts, three Picard iterations of the pitch-angle
// update with the slab-QLT closure), with the reference's constructors, step
// methods, error messages and return values.
#pragma once

#include <cmath>
#include <memory>
#include <stdexcept>
#include <vector>

#include "Coefficients.hpp"
#include "RandomManager.hpp"
#include "SolverBase.hpp"

namespace kpt {

class FocusTransportSolver : public SolverBase {
public:
    using coefficient_field_set_type = FocusCoefficient::TransportCoefficientFieldSet;
    static constexpr int packed_component_count = FocusCoefficient::packed_component_count;

    coefficient_field_set_type coefficients;
    double maximum_pitch_angle_cosine{1.0};

    FocusTransportSolver(CartesianGrid2D input_grid, VectorField input_B_vec,
                         VectorField input_V_body)
        : SolverBase(std::move(input_grid), std::move(input_B_vec), std::move(input_V_body)) {}

    FocusTransportSolver(CartesianGrid2D input_grid, VectorField input_B_vec,
                         VectorField input_V_body, coefficient_field_set_type input_coefficients)
        : SolverBase(std::move(input_grid), std::move(input_B_vec), std::move(input_V_body)),
          coefficients(std::move(input_coefficients)) {
        if (use_packed_ && coefficients.configured()) rebuild_packed_coefficient_basis();
    }

    FocusTransportSolver(ParticleSystem input_particles, CartesianGrid2D input_grid,
                         VectorField input_B_vec, VectorField input_V_body)
        : SolverBase(std::move(input_particles), std::move(input_grid), std::move(input_B_vec),
                     std::move(input_V_body)) {}

    FocusTransportSolver(ParticleSystem input_particles, CartesianGrid2D input_grid,
                         VectorField input_B_vec, VectorField input_V_body,
                         coefficient_field_set_type input_coefficients)
        : SolverBase(std::move(input_particles), std::move(input_grid), std::move(input_B_vec),
                     std::move(input_V_body)),
          coefficients(std::move(input_coefficients)) {
        if (use_packed_ && coefficients.configured()) rebuild_packed_coefficient_basis();
    }

    void set_coefficient_fields(coefficient_field_set_type input_coefficients) {
        coefficients = std::move(input_coefficients);
        solver_.reset();  // the scattering parameters travel with the coefficients
        if (use_packed_ && coefficients.configured()) rebuild_packed_coefficient_basis();
    }
    void set_use_packed_coefficient_basis(bool enabled) {
        use_packed_ = enabled;
        if (use_packed_ && coefficients.configured()) rebuild_packed_coefficient_basis();
    }
    bool packed_coefficient_basis_enabled() const { return use_packed_; }

    void rebuild_packed_coefficient_basis() {
        if (!coefficients.configured()) {
            throw std::runtime_error(
                "FocusTransportSolver: coefficient fields are not configured.");
        }
        if (coefficients.packed->size() != grid.point_count() * packed_component_count) {
            throw std::runtime_error(
                "FocusTransportSolver: packed coefficient basis point count does not match "
                "the grid.");
        }
        const int ratio = coefficients.constant_ratio ? 1 : 0;
        if (solver_) {
            check(kpt_focus_solver_set_basis(solver_.get(), coefficients.packed->data(), ratio));
            return;
        }
        const kpt_scattering_parameters scattering = coefficients.scattering.c_struct();
        kpt_focus_solver* raw = nullptr;
        check(kpt_focus_solver_create(grid.context().get(), grid.get(),
                                      coefficients.packed->data(), ratio, courant_scale,
                                      &scattering, &raw));
        solver_ = std::shared_ptr<kpt_focus_solver>(
            raw, [](kpt_focus_solver* s) { kpt_focus_solver_destroy(s); });
    }

    // set_maximum_pitch_angle_cosine (FocusSolver.hpp:219-226).
    void set_maximum_pitch_angle_cosine(double input_maximum_mu) {
        if (!std::isfinite(input_maximum_mu) || input_maximum_mu <= 0.0 ||
            input_maximum_mu > 1.0) {
            throw std::runtime_error(
                "FocusTransportSolver: maximum |mu| must satisfy 0 < value <= 1.");
        }
        maximum_pitch_angle_cosine = input_maximum_mu;
    }

    double compute_adaptive_time_step() const {
        prepare();
        double dt = 0.0;
        check(kpt_focus_compute_time_step(particles.ctx(), solver_.get(), particles.get(), &dt));
        return dt;
    }
    double advance_deterministic() {
        prepare();
        double dt = 0.0;
        check(kpt_focus_advance_deterministic(particles.ctx(), solver_.get(), particles.get(),
                                              &dt));
        dT = dt;
        return dt;
    }
    double advance_stochastic(const RandomManager& random_manager) {
        prepare();
        double dt = 0.0;
        check(kpt_focus_advance_stochastic(particles.ctx(), solver_.get(), particles.get(),
                                           random_manager.seed, random_manager.next_step(),
                                           &dt));
        dT = dt;
        return dt;
    }
    double advance_sde(const RandomManager& random_manager) {
        return advance_stochastic(random_manager);
    }
    std::vector<double> advance_stochastic_steps(const RandomManager& random_manager,
                                                 std::uint32_t steps) {
        prepare();
        std::vector<double> dts(steps);
        const std::uint32_t first = random_manager.step();
        check(kpt_focus_advance_stochastic_steps(particles.ctx(), solver_.get(), particles.get(),
                                                 random_manager.seed, first, steps, dts.data()));
        random_manager.set_step(first + steps);
        if (steps > 0) dT = dts.back();
        return dts;
    }
    double advance_with_noise(const std::vector<double>& normals) {
        prepare();
        if (normals.size() != 4 * particles.particle_count()) {
            throw std::runtime_error(
                "FocusTransportSolver: normals must hold 4 x particle_count values.");
        }
        double dt = 0.0;
        check(kpt_focus_advance_with_noise(particles.ctx(), solver_.get(), particles.get(),
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
    std::shared_ptr<kpt_focus_solver> solver_;

    void prepare() const {
        if (!coefficients.configured() || !solver_) {
            throw std::runtime_error(
                "FocusTransportSolver: coefficient fields are not configured.");
        }
        if (!particles) {
            throw std::runtime_error("FocusTransportSolver: the solver has no particle system.");
        }
        check(kpt_focus_solver_set_courant(solver_.get(), courant_scale));
        check(kpt_focus_solver_set_precision(solver_.get(), precision_));
        check(kpt_focus_solver_set_maximum_mu(solver_.get(), maximum_pitch_angle_cosine));
    }
};

// The reference's alias (FocusSolver.hpp:1889).
using FocusSolver = FocusTransportSolver;

}  // namespace kpt
