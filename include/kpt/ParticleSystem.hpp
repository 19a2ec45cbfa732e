// ParticleSystem<2> (ParticleSystem.hpp:312-1198) over the C ABI: the
// particle storage lives on the device (kpt_system); copies of a
// ParticleSystem share it, as copies of the reference's Kokkos Views do.
#pragma once

#include <cstdint>
#include <memory>
#include <vector>

#include "Grid.hpp"
#include "Runtime.hpp"

namespace kpt {

// ParticleStatus (ParticleSystem.hpp:35-39).
enum class ParticleStatus : int { Active = 0, Escaped = 1, Inactive = 2 };

// ParticleProperties (ParticleSystem.hpp:145-213), dimensionless.
struct ParticleProperties {
    double rest_mass{1.0};
    double charge{1.0};
    double speed_of_light{1.0};
    double energy_scale_erg{1.0};
    kpt_particle_properties c_struct() const {
        return kpt_particle_properties{rest_mass, charge, speed_of_light, energy_scale_erg};
    }
};

// ParticleSplittingPolicy (ParticleSystem.hpp:280-295).
struct ParticleSplittingPolicy {
    double energy_split_ratio{2.0};
    double minimum_child_weight{0.0};
};

// ParticleSplitStatistics (ParticleSystem.hpp:269-275).
struct ParticleSplitStatistics {
    std::uint64_t active_count{0};
    std::uint64_t split_count{0};
    std::uint64_t skipped_capacity_count{0};
    std::uint64_t skipped_invalid_baseline_count{0};
    std::uint64_t skipped_minimum_weight_count{0};
};

// Host copy of a particle system's storage (the reference's host mirrors of
// its Views), one entry per particle slot.
struct HostParticles {
    std::vector<std::uint64_t> particle_id;
    std::vector<double> x, y;                            // position
    std::vector<double> previous_x, previous_y;          // previous_position
    std::vector<double> previous_step_x, previous_step_y;  // previous_step_position
    std::vector<double> momentum, mu, weight, initial_kinetic_energy;
    std::vector<int32_t> status, split_level, sort_key;

    explicit HostParticles(std::size_t n = 0) { resize(n); }
    void resize(std::size_t n) {
        particle_id.resize(n);
        for (auto* v : {&x, &y, &previous_x, &previous_y, &previous_step_x, &previous_step_y,
                        &momentum, &mu, &weight, &initial_kinetic_energy}) {
            v->resize(n);
        }
        for (auto* v : {&status, &split_level, &sort_key}) v->resize(n);
    }
    std::size_t size() const { return x.size(); }
    kpt_system_arrays c_struct() {
        return kpt_system_arrays{particle_id.data(), x.data(), y.data(), previous_x.data(),
                                 previous_y.data(), previous_step_x.data(),
                                 previous_step_y.data(), momentum.data(), mu.data(),
                                 weight.data(), initial_kinetic_energy.data(), status.data(),
                                 split_level.data(), sort_key.data()};
    }
};

class ParticleSystem {
public:
    using size_type = std::uint64_t;
    static constexpr int space_dim = 2;

    ParticleSystem() = default;

    // ParticleSystem(count, properties) (ParticleSystem.hpp:360-364).
    ParticleSystem(size_type particle_count, const ParticleProperties& input_properties,
                   Context context = default_context())
        : ParticleSystem(particle_count, particle_count, input_properties,
                         ParticleSplittingPolicy{}, context) {}

    // ParticleSystem(count, capacity, properties) (ParticleSystem.hpp:369-375).
    ParticleSystem(size_type particle_count, size_type particle_capacity,
                   const ParticleProperties& input_properties,
                   Context context = default_context())
        : ParticleSystem(particle_count, particle_capacity, input_properties,
                         ParticleSplittingPolicy{}, context) {}

    // ParticleSystem(count, capacity, properties, policy)
    // (ParticleSystem.hpp:380-405): storage allocated, default state
    // initialised (initialize_default_state, ParticleSystem.hpp:1163-1198).
    ParticleSystem(size_type particle_count, size_type particle_capacity,
                   const ParticleProperties& input_properties,
                   const ParticleSplittingPolicy& policy, Context context = default_context())
        : properties(input_properties), context_(std::make_shared<Context>(context)),
          policy_(policy) {
        const kpt_particle_properties props = input_properties.c_struct();
        const kpt_split_policy split{policy.energy_split_ratio, policy.minimum_child_weight};
        kpt_system* raw = nullptr;
        check(kpt_system_create(context_->get(), particle_count, particle_capacity, &props,
                                &split, &raw));
        handle_ = std::shared_ptr<kpt_system>(raw, [](kpt_system* s) { kpt_system_destroy(s); });
    }

    ParticleProperties properties{};

    size_type particle_count() const {
        size_type count = 0;
        check(kpt_system_count(get(), &count, nullptr));
        return count;
    }
    size_type particle_capacity() const {
        size_type capacity = 0;
        check(kpt_system_count(get(), nullptr, &capacity));
        return capacity;
    }
    bool empty() const { return particle_count() == 0; }
    ParticleSplittingPolicy splitting_policy() const { return policy_; }
    void set_particle_count(size_type count) { check(kpt_system_set_count(get(), count)); }

    // Host mirrors: the first n slots (n = 0: the stored count).
    HostParticles copy_to_host(size_type n = 0) const {
        if (n == 0) n = particle_count();
        HostParticles host(n);
        kpt_system_arrays arrays = host.c_struct();
        check(kpt_system_download(get(), n, &arrays));
        return host;
    }
    void copy_from_host(HostParticles& host) {
        kpt_system_arrays arrays = host.c_struct();
        check(kpt_system_upload(get(), host.size(), &arrays));
    }

    // capture_previous_positions (ParticleSystem.hpp:623-629).
    void capture_previous_positions() {
        check(kpt_system_capture_previous_positions(ctx(), get()));
    }
    // reset_split_baselines (ParticleSystem.hpp:633-650).
    void reset_split_baselines() { check(kpt_system_reset_split_baselines(ctx(), get())); }
    // apply_grid_boundary_conditions(grid, PhysicalDomain) (ParticleSystem.hpp:661-706).
    void apply_grid_boundary_conditions(const CartesianGrid2D& grid,
                                        GridDomain domain = GridDomain::PhysicalDomain) {
        if (domain != GridDomain::PhysicalDomain) {
            throw std::runtime_error(
                "ParticleSystem: boundary conditions are applied on the physical domain.");
        }
        check(kpt_system_apply_boundary(ctx(), get(), grid.get()));
    }
    // sort_by_key(minimum_key, maximum_key) (ParticleSystem.hpp:727-760):
    // stable, equal keys keep index order.
    void sort_by_key(int minimum_key, int maximum_key) {
        check(kpt_system_sort_by_key(ctx(), get(), minimum_key, maximum_key));
    }
    // compact_active_particles (ParticleSystem.hpp:769-793).
    size_type compact_active_particles() {
        size_type active = 0;
        check(kpt_system_compact(ctx(), get(), &active));
        return active;
    }
    // split_particles_on_energy_growth (ParticleSystem.hpp:802-917):
    // children appended in parent-index order.
    ParticleSplitStatistics split_particles_on_energy_growth() {
        kpt_split_statistics s{};
        check(kpt_system_split_energy(ctx(), get(), &s));
        return ParticleSplitStatistics{s.active_count, s.split_count, s.skipped_capacity_count,
                                       s.skipped_invalid_baseline_count,
                                       s.skipped_minimum_weight_count};
    }

    kpt_system* get() const {
        if (!handle_) throw std::runtime_error("ParticleSystem: no storage allocated.");
        return handle_.get();
    }
    kpt_context* ctx() const { return context_->get(); }
    explicit operator bool() const { return static_cast<bool>(handle_); }

private:
    std::shared_ptr<Context> context_;
    ParticleSplittingPolicy policy_{};
    std::shared_ptr<kpt_system> handle_;
};

}  // namespace kpt
