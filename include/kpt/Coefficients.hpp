// Coefficient models and builders of the header library over the C ABI:
// LegencyModel's parameter bundles (LegencyModel.hpp:33-117, :196-221),
// TurbulencePropertyModel::constant_code_units (TurbulenceProperties.hpp:76-91),
// and ParkerCoefficient / FocusCoefficient::make_legacy_transport_coefficient_
// fields (ParkerCoefficient.hpp:1102-1155, FocusCoefficient.hpp:852-1024).
//
// The reference's coefficient field sets are Fields on the device that the
// solver packs into its sampling basis (ParkerSolver.hpp:514-598,
// FocusSolver.hpp:106-136).  Here the builders compute the packed basis
// directly on the GPU (kpt_parker_coefficients / kpt_focus_coefficients) and
// the field set carries it; a caller that already has a packed basis can
// wrap it (packed_coefficient_basis).
#pragma once

#include <cmath>
#include <memory>
#include <stdexcept>
#include <vector>

#include "Grid.hpp"
#include "ParticleSystem.hpp"

namespace kpt {

// FieldGhostFillMode (Field.hpp:20-23).
enum class FieldGhostFillMode { PeriodicOrClamped = 0, PeriodicOnly = 1 };

namespace LegencyModel {

enum class PerpendicularDiffusionModelKind { ReadmeFormula = 0, ConstantParallelRatio = 1 };

// DiffusionModelParameters (LegencyModel.hpp:33-117).
struct DiffusionModelParameters {
    PerpendicularDiffusionModelKind perpendicular_model{
        PerpendicularDiffusionModelKind::ReadmeFormula};
    double parallel_prefactor{1.622};
    double perpendicular_prefactor{0.198};
    double perpendicular_parallel_ratio{0.0};
    double minimum_magnetic_field_magnitude{0.0};
    double minimum_solar_wind_speed{0.0};
    double minimum_sigma2{0.0};

    static DiffusionModelParameters with_constant_perpendicular_parallel_ratio(double ratio);
    static DiffusionModelParameters with_constant_perpendicular_parallel_ratio(
        double ratio, DiffusionModelParameters parameters) {
        parameters.perpendicular_model = PerpendicularDiffusionModelKind::ConstantParallelRatio;
        parameters.perpendicular_parallel_ratio = ratio;
        return parameters;
    }
    bool uses_constant_perpendicular_parallel_ratio() const {
        return perpendicular_model == PerpendicularDiffusionModelKind::ConstantParallelRatio;
    }
};

inline DiffusionModelParameters
DiffusionModelParameters::with_constant_perpendicular_parallel_ratio(double ratio) {
    return with_constant_perpendicular_parallel_ratio(ratio, DiffusionModelParameters{});
}

// PitchAngleScatteringParameters (LegencyModel.hpp:196-221).
struct PitchAngleScatteringParameters {
    double spectral_index{5.0 / 3.0};
    double resonance_regularization_h0{1.0e-6};
    double minimum_magnetic_field_magnitude{0.0};
    double minimum_sigma2{0.0};
    double minimum_correlation_length{0.0};
    double minimum_speed{0.0};

    kpt_scattering_parameters c_struct() const {
        return kpt_scattering_parameters{spectral_index, resonance_regularization_h0,
                                         minimum_magnetic_field_magnitude, minimum_sigma2,
                                         minimum_correlation_length, minimum_speed};
    }
};

}  // namespace LegencyModel

// Turbulence properties (TurbulenceProperties.hpp:294-484): the constant
// model's four lengths, or per-point fields on the grid.
struct TurbulenceProperties {
    bool constant{true};
    double sigma2{0.0}, l2d{0.0}, lslab{0.0}, lc{0.0};
    std::shared_ptr<const ScalarField> sigma2_field, l2d_field, lslab_field, lc_field;

    kpt_turbulence c_struct() const {
        kpt_turbulence t{};
        t.storage = constant ? 0 : 1;
        t.sigma2 = sigma2;
        t.l2d = l2d;
        t.lslab = lslab;
        t.lc = lc;
        if (!constant) {
            t.sigma2_field = sigma2_field ? sigma2_field->data() : nullptr;
            t.l2d_field = l2d_field ? l2d_field->data() : nullptr;
            t.lslab_field = lslab_field ? lslab_field->data() : nullptr;
            t.lc_field = lc_field ? lc_field->data() : nullptr;
        }
        return t;
    }

    static TurbulenceProperties from_fields(ScalarField sigma2_values, ScalarField l2d_values,
                                            ScalarField lc_values) {
        TurbulenceProperties t;
        t.constant = false;
        t.sigma2_field = std::make_shared<const ScalarField>(std::move(sigma2_values));
        t.l2d_field = std::make_shared<const ScalarField>(std::move(l2d_values));
        t.lc_field = std::make_shared<const ScalarField>(std::move(lc_values));
        return t;
    }
};

struct TurbulencePropertyModel {
    // constant_code_units(sigma2, l2d, lslab, lc) (TurbulenceProperties.hpp:76-91):
    // lc <= 0 takes the slab length.
    static TurbulenceProperties constant_code_units(double sigma2, double l2d, double lslab,
                                                    double lc = -1.0) {
        if (!std::isfinite(sigma2) || sigma2 < 0.0 || !std::isfinite(l2d) || l2d <= 0.0 ||
            !std::isfinite(lslab) || lslab <= 0.0) {
            throw std::runtime_error(
                "TurbulencePropertyModel: constant sigma2 must be non-negative and the "
                "correlation lengths positive.");
        }
        TurbulenceProperties t;
        t.sigma2 = sigma2;
        t.l2d = l2d;
        t.lslab = lslab;
        t.lc = lc > 0.0 ? lc : lslab;
        return t;
    }
};

namespace detail {
inline kpt_diffusion_parameters diffusion_c_struct(
    const LegencyModel::DiffusionModelParameters& p, double minimum_b2_for_drift,
    FieldGhostFillMode ghost_fill_mode) {
    kpt_diffusion_parameters d{};
    kpt_default_diffusion_parameters(&d);
    d.perpendicular_model = p.uses_constant_perpendicular_parallel_ratio() ? 1 : 0;
    d.ghost_fill_mode = ghost_fill_mode == FieldGhostFillMode::PeriodicOnly ? 1 : 0;
    d.parallel_prefactor = p.parallel_prefactor;
    d.perpendicular_prefactor = p.perpendicular_prefactor;
    d.perpendicular_parallel_ratio = p.perpendicular_parallel_ratio;
    d.minimum_magnetic_field_magnitude = p.minimum_magnetic_field_magnitude;
    d.minimum_solar_wind_speed = p.minimum_solar_wind_speed;
    d.minimum_sigma2 = p.minimum_sigma2;
    d.minimum_magnetic_field_squared_for_drift = minimum_b2_for_drift;
    return d;
}
}  // namespace detail

namespace ParkerCoefficient {

constexpr int packed_component_count = 18;

// TransportCoefficientFieldSet: here the packed basis (grid points x 18,
// ParkerSolver.hpp:96-116 order) and the diffusion branch.
struct TransportCoefficientFieldSet {
    std::shared_ptr<const std::vector<double>> packed;
    bool constant_ratio{false};
    bool configured() const { return static_cast<bool>(packed); }
};

// Wrap a packed basis the caller already has (extension).
inline TransportCoefficientFieldSet packed_coefficient_basis(std::vector<double> basis,
                                                             bool constant_ratio) {
    if (basis.size() % packed_component_count != 0) {
        throw std::runtime_error("ParkerCoefficient: a packed basis holds 18 values per point.");
    }
    return TransportCoefficientFieldSet{
        std::make_shared<const std::vector<double>>(std::move(basis)), constant_ratio};
}

// make_legacy_transport_coefficient_fields (ParkerCoefficient.hpp:1102-1155),
// computed on the GPU of the field's grid.
inline TransportCoefficientFieldSet make_legacy_transport_coefficient_fields(
    const VectorField& magnetic_field, const VectorField& solar_wind_velocity,
    const TurbulenceProperties& turbulence_properties,
    const ParticleProperties& particle_properties,
    const char* label = "parker_transport_coefficients",
    const LegencyModel::DiffusionModelParameters& parameters =
        LegencyModel::DiffusionModelParameters{},
    double minimum_magnetic_field_squared_for_drift = 0.0,
    FieldGhostFillMode ghost_fill_mode = FieldGhostFillMode::PeriodicOrClamped) {
    (void)label;
    const CartesianGrid2D& grid = magnetic_field.grid();
    if (solar_wind_velocity.point_count() != grid.point_count()) {
        throw std::runtime_error(
            "Parker transport coefficients require B and Vsw on the same grid.");
    }
    const kpt_turbulence turb = turbulence_properties.c_struct();
    const kpt_particle_properties props = particle_properties.c_struct();
    const kpt_diffusion_parameters diff = detail::diffusion_c_struct(
        parameters, minimum_magnetic_field_squared_for_drift, ghost_fill_mode);
    auto packed = std::make_shared<std::vector<double>>(grid.point_count() *
                                                        packed_component_count);
    check(kpt_parker_coefficients(grid.context().get(), grid.get(), magnetic_field.data(),
                                  solar_wind_velocity.data(), &turb, &props, &diff,
                                  packed->data()));
    return TransportCoefficientFieldSet{packed,
                                        parameters.uses_constant_perpendicular_parallel_ratio()};
}

}  // namespace ParkerCoefficient

namespace FocusCoefficient {

constexpr int packed_component_count = 27;

// The focused coefficient set: packed basis (grid points x 27,
// FocusSolver.hpp:106-136 order), diffusion branch and the pitch-angle
// scattering parameters the set was built with.
struct TransportCoefficientFieldSet {
    std::shared_ptr<const std::vector<double>> packed;
    bool constant_ratio{false};
    LegencyModel::PitchAngleScatteringParameters scattering{};
    bool configured() const { return static_cast<bool>(packed); }
};

inline TransportCoefficientFieldSet packed_coefficient_basis(
    std::vector<double> basis, bool constant_ratio,
    const LegencyModel::PitchAngleScatteringParameters& scattering =
        LegencyModel::PitchAngleScatteringParameters{}) {
    if (basis.size() % packed_component_count != 0) {
        throw std::runtime_error("FocusCoefficient: a packed basis holds 27 values per point.");
    }
    return TransportCoefficientFieldSet{
        std::make_shared<const std::vector<double>>(std::move(basis)), constant_ratio,
        scattering};
}

// make_legacy_transport_coefficient_fields_with_time_derivative
// (FocusCoefficient.hpp:852-993), on the GPU of the field's grid.
inline TransportCoefficientFieldSet make_legacy_transport_coefficient_fields_with_time_derivative(
    const VectorField& magnetic_field, const VectorField& solar_wind_velocity,
    const VectorField* solar_wind_time_derivative,
    const TurbulenceProperties& turbulence_properties,
    const ParticleProperties& particle_properties,
    const char* label = "focused_transport_coefficients",
    const LegencyModel::DiffusionModelParameters& diffusion_parameters =
        LegencyModel::DiffusionModelParameters{},
    const LegencyModel::PitchAngleScatteringParameters& scattering_parameters =
        LegencyModel::PitchAngleScatteringParameters{},
    double minimum_magnetic_field_magnitude = 0.0,
    FieldGhostFillMode ghost_fill_mode = FieldGhostFillMode::PeriodicOrClamped) {
    (void)label;
    const CartesianGrid2D& grid = magnetic_field.grid();
    if (solar_wind_velocity.point_count() != grid.point_count() ||
        (solar_wind_time_derivative != nullptr &&
         solar_wind_time_derivative->point_count() != grid.point_count())) {
        throw std::runtime_error(
            "Focused transport coefficients require B, Vsw and dVsw/dt on the same grid.");
    }
    const kpt_turbulence turb = turbulence_properties.c_struct();
    const kpt_particle_properties props = particle_properties.c_struct();
    const kpt_diffusion_parameters diff =
        detail::diffusion_c_struct(diffusion_parameters, 0.0, ghost_fill_mode);
    auto packed = std::make_shared<std::vector<double>>(grid.point_count() *
                                                        packed_component_count);
    check(kpt_focus_coefficients(
        grid.context().get(), grid.get(), magnetic_field.data(), solar_wind_velocity.data(),
        solar_wind_time_derivative != nullptr ? solar_wind_time_derivative->data() : nullptr,
        &turb, &props, &diff, minimum_magnetic_field_magnitude, packed->data()));
    return TransportCoefficientFieldSet{
        packed, diffusion_parameters.uses_constant_perpendicular_parallel_ratio(),
        scattering_parameters};
}

inline TransportCoefficientFieldSet make_legacy_transport_coefficient_fields_with_time_derivative(
    const VectorField& magnetic_field, const VectorField& solar_wind_velocity,
    const VectorField& solar_wind_time_derivative,
    const TurbulenceProperties& turbulence_properties,
    const ParticleProperties& particle_properties,
    const char* label = "focused_transport_coefficients",
    const LegencyModel::DiffusionModelParameters& diffusion_parameters =
        LegencyModel::DiffusionModelParameters{},
    const LegencyModel::PitchAngleScatteringParameters& scattering_parameters =
        LegencyModel::PitchAngleScatteringParameters{},
    double minimum_magnetic_field_magnitude = 0.0,
    FieldGhostFillMode ghost_fill_mode = FieldGhostFillMode::PeriodicOrClamped) {
    return make_legacy_transport_coefficient_fields_with_time_derivative(
        magnetic_field, solar_wind_velocity, &solar_wind_time_derivative,
        turbulence_properties, particle_properties, label, diffusion_parameters,
        scattering_parameters, minimum_magnetic_field_magnitude, ghost_fill_mode);
}

// make_legacy_transport_coefficient_fields (FocusCoefficient.hpp:998-1022):
// partial_t Vsw = 0.
inline TransportCoefficientFieldSet make_legacy_transport_coefficient_fields(
    const VectorField& magnetic_field, const VectorField& solar_wind_velocity,
    const TurbulenceProperties& turbulence_properties,
    const ParticleProperties& particle_properties,
    const char* label = "focused_transport_coefficients",
    const LegencyModel::DiffusionModelParameters& diffusion_parameters =
        LegencyModel::DiffusionModelParameters{},
    const LegencyModel::PitchAngleScatteringParameters& scattering_parameters =
        LegencyModel::PitchAngleScatteringParameters{},
    double minimum_magnetic_field_magnitude = 0.0,
    FieldGhostFillMode ghost_fill_mode = FieldGhostFillMode::PeriodicOrClamped) {
    return make_legacy_transport_coefficient_fields_with_time_derivative(
        magnetic_field, solar_wind_velocity, static_cast<const VectorField*>(nullptr),
        turbulence_properties, particle_properties, label, diffusion_parameters,
        scattering_parameters, minimum_magnetic_field_magnitude, ghost_fill_mode);
}

}  // namespace FocusCoefficient

}  // namespace kpt
