// Random pool with the Kokkos Random_XorShift64_Pool interface whose states
// draw from the keyed Philox stream of oracle/kpt_philox.h instead of a
// per-thread XorShift64 state.  get_state() keys the stream by the running
// kernel (label -> tag), the loop index published by parallel_for, and the
// frame number the harness sets before each launch; this is the
// injected-noise hook that makes the reference's unmodified kernels consume
// the same increments as the GPU kernels.  Oracle-only shim.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#include "Kokkos_Core.hpp"
#include "../kpt_philox.h"

namespace Kokkos {

namespace ShimImpl {
inline std::uint32_t& current_frame() {
    static std::uint32_t frame = 0;
    return frame;
}
// When set, the frame key is auto_frame_base() + (launch ordinal - 1) of the
// running kernel: the driver launches inject and push once per frame.
inline int& auto_frame_enabled() {
    static int enabled = 0;
    return enabled;
}
inline std::uint32_t& auto_frame_base() {
    static std::uint32_t base = 0;
    return base;
}
inline std::uint32_t label_tag(const char* label) {
    if (label == nullptr) {
        return KPT_ORACLE_TAG_OTHER;
    }
    if (std::strstr(label, "inject_uniform_particles") != nullptr) {
        return KPT_ORACLE_TAG_INJECT;
    }
    if (std::strstr(label, "move_parker_particles_one_interval") != nullptr ||
        std::strstr(label, "move_particles_one_interval") != nullptr) {
        return KPT_ORACLE_TAG_PUSH;
    }
    if (std::strstr(label, "ParkerSolver::") != nullptr ||
        std::strstr(label, "FocusTransportSolver::") != nullptr ||
        std::strstr(label, "FocusSolver::") != nullptr) {
        return KPT_ORACLE_TAG_LIBRARY;
    }
    if (std::strstr(label, "ParticleGenerator::") != nullptr) {
        return KPT_ORACLE_TAG_GENERATOR;
    }
    return KPT_ORACLE_TAG_OTHER;
}
// Injected noise: when set, normal() returns external[k * count + index],
// k the number of normals the state has drawn (the library solvers'
// advance-with-noise parity mode).
inline const double*& external_normals() {
    static const double* normals = nullptr;
    return normals;
}
inline std::uint64_t& external_count() {
    static std::uint64_t count = 0;
    return count;
}
}  // namespace ShimImpl

template <class DeviceType>
class Random_XorShift64 {
public:
    kpt_oracle_stream stream{};
    bool has_spare = false;
    double spare = 0.0;
    int normals_drawn = 0;

    double drand() { return kpt_oracle_stream_u01(&stream); }
    double drand(const double range) { return range * drand(); }
    double drand(const double start, const double end) {
        return start + (end - start) * drand();
    }
    // Box-Muller transform on two stream draws, both of its normals used:
    // normal 2m is r cos(theta) and normal 2m+1 is r sin(theta) of draws 2m
    // and 2m+1 (u1 = 1 - draw 2m, u2 = draw 2m+1, theta = 2 pi u2).  Only
    // the header library's solvers draw normals; the driver path draws
    // uniforms alone.
    double normal() {
        if (const double* ext = ShimImpl::external_normals()) {
            const std::uint64_t k = static_cast<std::uint64_t>(normals_drawn++);
            return ext[k * ShimImpl::external_count() + stream.index];
        }
        if (has_spare) {
            has_spare = false;
            return spare;
        }
        const double u1 = 1.0 - drand();
        const double u2 = drand();
        const double r = std::sqrt(-2.0 * std::log(u1));
        const double theta = 6.283185307179586 * u2;
        spare = r * std::sin(theta);
        has_spare = true;
        return r * std::cos(theta);
    }
    double normal(const double mean, const double standard_deviation) {
        return mean + standard_deviation * normal();
    }
};

template <class DeviceType>
class Random_XorShift64_Pool {
public:
    using generator_type = Random_XorShift64<DeviceType>;
    using device_type = DeviceType;

    Random_XorShift64_Pool() = default;
    explicit Random_XorShift64_Pool(const std::uint64_t seed) : seed_(seed) {}

    generator_type get_state() const {
        const auto& context = ShimImpl::current_kernel();
        generator_type generator;
        const std::uint32_t frame =
            ShimImpl::auto_frame_enabled() != 0
                ? ShimImpl::auto_frame_base() + (context.ordinal - 1u)
                : ShimImpl::current_frame();
        kpt_oracle_stream_init(&generator.stream, seed_,
                               static_cast<std::uint32_t>(context.index), frame,
                               ShimImpl::label_tag(context.label));
        return generator;
    }
    void free_state(const generator_type&) const {}

private:
    std::uint64_t seed_ = 0;
};

}  // namespace Kokkos
