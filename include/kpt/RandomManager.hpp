// RandomManager (RandomManager.hpp:13-62) for the library solvers.
//
// The reference hands a Kokkos XorShift64 pool to advance_stochastic; its
// draws depend on which thread takes which pool state, so they do not repeat
// across thread counts.  Here each particle draws from a counter-based
// Philox4x32-10 stream keyed by (seed, particle index, step): the manager
// carries the seed and the step counter, and every stochastic step a solver
// takes with it uses the next step number.  Same seed and same sequence of
// steps give bit-identical results on any launch shape.
#pragma once

#include <cstdint>

namespace kpt {

class RandomManager {
public:
    static constexpr std::uint64_t default_seed = 114514u;

    explicit RandomManager(std::uint64_t input_seed = default_seed, std::uint32_t first_step = 0)
        : seed(input_seed), step_(first_step) {}

    std::uint64_t seed;

    // The step number the next stochastic step draws from.
    std::uint32_t step() const { return step_; }
    void set_step(std::uint32_t step) const { step_ = step; }
    // Take the current step number and advance (the solvers call this; the
    // reference's pool is likewise advanced through a const handle).
    std::uint32_t next_step() const { return step_++; }

private:
    mutable std::uint32_t step_;
};

}  // namespace kpt
