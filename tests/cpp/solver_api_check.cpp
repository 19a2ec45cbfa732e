// Drives the C++ drop-in headers (include/kpt/*.hpp) the way a user of the
// reference's header library drives ParkerSolver / FocusSolver /
// ParticleSystem, on inputs written by tests/test_gpu_cxx_api.py, and writes
// what the calls return and the particles they leave, for the test to
// compare with the reference's golden vectors.
//
// Usage: solver_api_check parker|focus|system IN OUT
// IN and OUT are sequences of records: name (32 bytes, NUL-padded), type
// ('d' f64, 'i' i32, 'u' u64), 7 pad bytes, count (u64), count values.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "kpt/kpt.hpp"

namespace {

struct Record {
    char type = 'd';
    std::vector<unsigned char> bytes;
    template <class T>
    std::vector<T> as() const {
        std::vector<T> out(bytes.size() / sizeof(T));
        std::memcpy(out.data(), bytes.data(), bytes.size());
        return out;
    }
};

std::map<std::string, Record> read_records(const std::string& path) {
    std::ifstream in(path, std::ios::binary);
    if (!in) throw std::runtime_error("cannot open " + path);
    std::map<std::string, Record> out;
    for (;;) {
        char name[32];
        if (!in.read(name, 32)) break;
        char head[8];
        std::uint64_t count = 0;
        in.read(head, 8);
        in.read(reinterpret_cast<char*>(&count), 8);
        Record r;
        r.type = head[0];
        const std::size_t width = r.type == 'i' ? 4 : 8;
        r.bytes.resize(count * width);
        in.read(reinterpret_cast<char*>(r.bytes.data()), static_cast<std::streamsize>(r.bytes.size()));
        out[std::string(name, strnlen(name, 32))] = std::move(r);
    }
    return out;
}

class Writer {
public:
    explicit Writer(const std::string& path) : out_(path, std::ios::binary) {
        if (!out_) throw std::runtime_error("cannot open " + path);
    }
    template <class T>
    void put(const std::string& name, char type, const std::vector<T>& values) {
        char head[32] = {};
        std::strncpy(head, name.c_str(), 31);
        out_.write(head, 32);
        char pad[8] = {type, 0, 0, 0, 0, 0, 0, 0};
        out_.write(pad, 8);
        const std::uint64_t count = values.size();
        out_.write(reinterpret_cast<const char*>(&count), 8);
        out_.write(reinterpret_cast<const char*>(values.data()),
                   static_cast<std::streamsize>(count * sizeof(T)));
    }
    void put_state(const std::string& prefix, const kpt::HostParticles& h) {
        put(prefix + "_id", 'u', h.particle_id);
        put(prefix + "_x", 'd', h.x);
        put(prefix + "_y", 'd', h.y);
        put(prefix + "_prev_x", 'd', h.previous_x);
        put(prefix + "_prev_y", 'd', h.previous_y);
        put(prefix + "_prevstep_x", 'd', h.previous_step_x);
        put(prefix + "_prevstep_y", 'd', h.previous_step_y);
        put(prefix + "_p", 'd', h.momentum);
        put(prefix + "_mu", 'd', h.mu);
        put(prefix + "_w", 'd', h.weight);
        put(prefix + "_e0", 'd', h.initial_kinetic_energy);
        put(prefix + "_status", 'i', h.status);
        put(prefix + "_level", 'i', h.split_level);
        put(prefix + "_key", 'i', h.sort_key);
    }

private:
    std::ofstream out_;
};

double scalar(const std::map<std::string, Record>& in, const std::string& name) {
    return in.at(name).as<double>().at(0);
}

kpt::HostParticles start_state(const std::map<std::string, Record>& in) {
    const auto x = in.at("start_x").as<double>();
    kpt::HostParticles h(x.size());
    h.particle_id = in.at("start_id").as<std::uint64_t>();
    h.x = x;
    h.y = in.at("start_y").as<double>();
    h.previous_x = in.at("start_prev_x").as<double>();
    h.previous_y = in.at("start_prev_y").as<double>();
    h.previous_step_x = in.at("start_prevstep_x").as<double>();
    h.previous_step_y = in.at("start_prevstep_y").as<double>();
    h.momentum = in.at("start_p").as<double>();
    h.mu = in.at("start_mu").as<double>();
    h.weight = in.at("start_w").as<double>();
    h.initial_kinetic_energy = in.at("start_e0").as<double>();
    h.status = in.at("start_status").as<int32_t>();
    h.split_level = in.at("start_level").as<int32_t>();
    h.sort_key = in.at("start_key").as<int32_t>();
    return h;
}

// The analytic grid on uniform edges, or a StoredCoordinateGrid2D when the
// input carries explicit faces.
kpt::CartesianGrid2D make_grid(const std::map<std::string, Record>& in) {
    const auto per = in.at("periodic").as<int32_t>();
    if (in.count("x_faces") != 0) {
        const auto xf = in.at("x_faces").as<double>();
        const auto yf = in.at("y_faces").as<double>();
        return kpt::StoredCoordinateGrid2D(static_cast<int>(xf.size()) - 5,
                                           static_cast<int>(yf.size()) - 5, xf, yf,
                                           {per.at(0) != 0, per.at(1) != 0});
    }
    const auto xe = in.at("x_edges").as<double>();
    const auto ye = in.at("y_edges").as<double>();
    return kpt::CartesianGrid2D(static_cast<int>(xe.size()) - 1, static_cast<int>(ye.size()) - 1,
                                xe, ye, {per.at(0) != 0, per.at(1) != 0});
}

// The message a call throws, or "" when it does not throw.
template <class F>
std::string message_of(F&& f) {
    try {
        f();
    } catch (const std::exception& e) {
        return e.what();
    }
    return "";
}

std::vector<double> as_codes(const std::string& s) {
    return std::vector<double>(s.begin(), s.end());
}

template <class Solver, bool FOCUSED, class Coefficients>
void run_solver(const std::map<std::string, Record>& in, Writer& out, Coefficients coefficients) {
    kpt::CartesianGrid2D grid = make_grid(in);
    kpt::HostParticles start = start_state(in);
    const auto count = static_cast<std::uint64_t>(scalar(in, "count"));
    kpt::ParticleSystem particles(count, start.size(), kpt::ParticleProperties{});
    particles.copy_from_host(start);
    kpt::VectorField B(grid), V(grid);

    // a solver without coefficients refuses to step, as the reference's does
    Solver bare(particles, grid, B, V);
    out.put("error_unconfigured", 'd',
            as_codes(message_of([&] { bare.compute_adaptive_time_step(); })));

    Solver solver(particles, grid, B, V, coefficients);
    solver.set_dimensionless_courant_scale(scalar(in, "courant"));
    if constexpr (FOCUSED) solver.set_maximum_pitch_angle_cosine(scalar(in, "max_mu"));
    const auto steps = static_cast<std::uint32_t>(scalar(in, "steps"));
    const bool stochastic = scalar(in, "stochastic") != 0.0;
    const kpt::RandomManager rng(static_cast<std::uint64_t>(scalar(in, "seed")),
                                 static_cast<std::uint32_t>(scalar(in, "first_step")));
    std::vector<double> dts{solver.compute_adaptive_time_step()};
    for (std::uint32_t k = 0; k < steps; ++k) {
        dts.push_back(stochastic ? solver.advance_stochastic(rng) : solver.advance_deterministic());
    }
    out.put("dts", 'd', dts);
    out.put("time_step_after", 'd', std::vector<double>{solver.time_step()});
    out.put_state("end", particles.copy_to_host(start.size()));

    // graph-replayed steps from the same start equal the single steps
    if (stochastic) {
        kpt::ParticleSystem again(count, start.size(), kpt::ParticleProperties{});
        again.copy_from_host(start);
        Solver replay(again, grid, B, V, coefficients);
        replay.set_dimensionless_courant_scale(scalar(in, "courant"));
        if constexpr (FOCUSED) replay.set_maximum_pitch_angle_cosine(scalar(in, "max_mu"));
        const kpt::RandomManager rng2(static_cast<std::uint64_t>(scalar(in, "seed")),
                                      static_cast<std::uint32_t>(scalar(in, "first_step")));
        out.put("graph_dts", 'd', replay.advance_stochastic_steps(rng2, steps));
        out.put_state("graph", again.copy_to_host(start.size()));
    }
    // the mixed-precision step (an extension): the same steps from the same
    // start, FP32 terms and noise with FP64 state
    {
        kpt::ParticleSystem mixed_particles(count, start.size(), kpt::ParticleProperties{});
        mixed_particles.copy_from_host(start);
        Solver mixed(mixed_particles, grid, B, V, coefficients);
        mixed.set_dimensionless_courant_scale(scalar(in, "courant"));
        if constexpr (FOCUSED) mixed.set_maximum_pitch_angle_cosine(scalar(in, "max_mu"));
        mixed.set_precision(KPT_PRECISION_MIXED);
        const kpt::RandomManager rng3(static_cast<std::uint64_t>(scalar(in, "seed")),
                                      static_cast<std::uint32_t>(scalar(in, "first_step")));
        std::vector<double> mixed_dts;
        for (std::uint32_t k = 0; k < steps; ++k) {
            mixed_dts.push_back(stochastic ? mixed.advance_stochastic(rng3)
                                           : mixed.advance_deterministic());
        }
        out.put("mixed_dts", 'd', mixed_dts);
        out.put_state("mixed", mixed_particles.copy_to_host(start.size()));
    }
    // a Courant scale of zero is refused with the reference's message
    solver.set_dimensionless_courant_scale(0.0);
    out.put("error_courant", 'd',
            as_codes(message_of([&] { solver.advance_stochastic(rng); })));
}

void run_system(const std::map<std::string, Record>& in, Writer& out) {
    kpt::CartesianGrid2D grid = make_grid(in);
    kpt::HostParticles start = start_state(in);
    const auto count = static_cast<std::uint64_t>(scalar(in, "count"));
    const kpt::ParticleSplittingPolicy policy{scalar(in, "split_ratio"),
                                              scalar(in, "min_child_weight")};
    for (const char* op : {"boundary", "sort", "compact", "split", "capture"}) {
        kpt::ParticleSystem system(count, start.size(), kpt::ParticleProperties{}, policy);
        system.copy_from_host(start);
        const std::string name(op);
        if (name == "boundary") {
            system.apply_grid_boundary_conditions(grid);
        } else if (name == "sort") {
            system.sort_by_key(-3, 40);
        } else if (name == "compact") {
            system.compact_active_particles();
        } else if (name == "split") {
            const kpt::ParticleSplitStatistics s = system.split_particles_on_energy_growth();
            out.put("split_stats", 'u',
                    std::vector<std::uint64_t>{s.active_count, s.split_count,
                                               s.skipped_capacity_count,
                                               s.skipped_invalid_baseline_count,
                                               s.skipped_minimum_weight_count});
        } else {
            system.capture_previous_positions();
        }
        out.put(name + "_count", 'u', std::vector<std::uint64_t>{system.particle_count()});
        out.put_state(name, system.copy_to_host(start.size()));
    }
}

}  // namespace

int main(int argc, char** argv) {
    if (argc != 4) {
        std::cerr << "usage: solver_api_check parker|focus|system IN OUT\n";
        return 2;
    }
    try {
        const std::string mode = argv[1];
        const auto in = read_records(argv[2]);
        Writer out(argv[3]);
        kpt::ScopeGuard guard(0);
        if (mode == "parker") {
            run_solver<kpt::ParkerSolver, false>(
                in, out,
                kpt::ParkerCoefficient::packed_coefficient_basis(
                    in.at("basis").as<double>(), scalar(in, "constant_ratio") != 0.0));
        } else if (mode == "focus") {
            kpt::LegencyModel::PitchAngleScatteringParameters scattering;
            scattering.spectral_index = scalar(in, "spectral_index");
            scattering.resonance_regularization_h0 = scalar(in, "h0");
            run_solver<kpt::FocusSolver, true>(
                in, out,
                kpt::FocusCoefficient::packed_coefficient_basis(
                    in.at("basis").as<double>(), scalar(in, "constant_ratio") != 0.0,
                    scattering));
        } else if (mode == "system") {
            run_system(in, out);
        } else {
            std::cerr << "unknown mode " << mode << "\n";
            return 2;
        }
    } catch (const std::exception& e) {
        std::cerr << "Error: " << e.what() << "\n";
        return 1;
    }
    return 0;
}
