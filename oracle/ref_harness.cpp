// Harness around the reference driver: it #includes the reference's own
// src/main.cpp (compiled unmodified against oracle/kokkos_shim, with main
// renamed to kpt_ref_main) and exposes its namespace functions through a flat
// C interface that Python (ctypes) calls to make golden vectors and to time
// the reference's CPU push.  Test infrastructure only; built into oracle/_ref
// by oracle/build_ref.sh.
//
// Functions driven (reference src/main.cpp):
//   load_parker_coefficient_frame / load_coefficient_frame   :932-962
//   inject_uniform_particles                                  :996-1048
//   move_parker_particles_one_interval                        :1084-1327
//   move_particles_one_interval                               :1334-1755
//   split_particles                                           :1761-1839
//   main (as kpt_ref_main)                                    :2692-2705
// and the header library's step API on a 2D Cartesian grid:
//   ParkerSolver::{advance_stochastic, advance_deterministic,
//                  compute_adaptive_time_step}           ParkerSolver.hpp:209-294
//   ParticleSystem::{apply_grid_boundary_conditions, sort_by_key,
//                    compact_active_particles,
//                    split_particles_on_energy_growth}    ParticleSystem.hpp:623-917
#include "src/main.cpp"

#include <type_traits>
#include <string>

#include "FocusSolver.hpp"
#include "ParticleGenerator.hpp"
#include "LegencyModel.hpp"
#include "ParkerSolver.hpp"

namespace {

thread_local std::string g_last_error;
// Seconds the last ref_push spent in the interval push alone (the driver's
// move_seconds: the push call between fences, src/main.cpp:2330-2341).
double g_last_move_seconds = 0.0;

// Parameter blocks passed from the host side.  Order is fixed and mirrored by
// tests/golden/make_golden.py and bench.py.
enum DoubleParam {
    DP_MHD_DT = 0,
    DP_P0,
    DP_PMIN,
    DP_PMAX,
    DP_GAMMA_TURB,
    DP_KPARA0,
    DP_KPERP_OVER_KPARA,
    DP_DT_MIN_REL,
    DP_DT_MAX_REL,
    DP_DRIFT1,
    DP_DRIFT2,
    DP_CHARGE,
    DP_PARTICLE_V0,
    DP_DUU0,
    DP_SPLIT_RATIO,
    DP_PMIN_SPLIT_OVER_P0,
    DP_MU_MAX,
    DP_COUNT
};
enum IntParam {
    IP_MAX_STEPS = 0,
    IP_MOMENTUM_DEPENDENCY,
    IP_MAGNETIC_DEPENDENCY,
    IP_TIME_INTERPOLATION,
    IP_SPLIT,
    IP_FOCUSED,
    IP_COUNT
};

using namespace Reconnection2DCalibration;

Reconnection2DSettings settings_from(const double* d, const int* i) {
    Reconnection2DSettings s;
    s.mhd_dt = d[DP_MHD_DT];
    s.p0 = d[DP_P0];
    s.pmin = d[DP_PMIN];
    s.pmax = d[DP_PMAX];
    s.gamma_turb = d[DP_GAMMA_TURB];
    s.kpara0 = d[DP_KPARA0];
    s.kperp_over_kpara = d[DP_KPERP_OVER_KPARA];
    s.dt_min_rel = d[DP_DT_MIN_REL];
    s.dt_max_rel = d[DP_DT_MAX_REL];
    s.drift_param1 = d[DP_DRIFT1];
    s.drift_param2 = d[DP_DRIFT2];
    s.charge = d[DP_CHARGE];
    s.particle_v0 = d[DP_PARTICLE_V0];
    s.duu0 = d[DP_DUU0];
    s.split_ratio = d[DP_SPLIT_RATIO];
    s.pmin_split_over_p0 = d[DP_PMIN_SPLIT_OVER_P0];
    s.mu_max = d[DP_MU_MAX];
    s.max_particle_steps_per_interval = i[IP_MAX_STEPS];
    s.momentum_dependency = i[IP_MOMENTUM_DEPENDENCY];
    s.magnetic_dependency = i[IP_MAGNETIC_DEPENDENCY];
    s.time_interpolation = i[IP_TIME_INTERPOLATION] != 0;
    s.split_particles = i[IP_SPLIT] != 0;
    s.transport_model = i[IP_FOCUSED] != 0 ? TransportModel::Focused : TransportModel::Parker;
    return s;
}

struct HostParticles {
    double* x;
    double* y;
    double* p;
    double* t;
    double* dt;
    double* w;
    double* mu;
    int* status;
    int* level;
};

template <typename Storage>
void load_storage(Storage& storage, const HostParticles& h, const std::uint64_t count) {
    for (std::uint64_t n = 0; n < count; ++n) {
        storage.position(n, 0) = h.x[n];
        storage.position(n, 1) = h.y[n];
        storage.momentum(n) = h.p[n];
        storage.time(n) = h.t[n];
        storage.step_dt(n) = h.dt[n];
        storage.weight(n) = h.w[n];
        storage.mu(n) = h.mu[n];
        storage.status(n) = h.status[n];
        storage.split_level(n) = h.level[n];
    }
    storage.count = count;
}

template <typename Storage>
void store_storage(const Storage& storage, const HostParticles& h, const std::uint64_t count) {
    for (std::uint64_t n = 0; n < count; ++n) {
        h.x[n] = storage.position(n, 0);
        h.y[n] = storage.position(n, 1);
        h.p[n] = storage.momentum(n);
        h.t[n] = storage.time(n);
        h.dt[n] = storage.step_dt(n);
        h.w[n] = storage.weight(n);
        h.mu[n] = storage.mu(n);
        h.status[n] = storage.status(n);
        h.level[n] = storage.split_level(n);
    }
}

template <typename Table>
auto device_settings_for(const Reconnection2DSettings& s, const Table& table) {
    return make_device_settings(s, table.grid);
}

// Background on explicit (possibly non-uniform) face edges: the reference's
// StoredCoordinateGrid (include/StoredCoordinateGrid.hpp) with the two ghost
// faces on each side continued periodically, B and V copied and ghost-filled
// exactly as the compact reader does (AthenaFieldReader.hpp:330-357).  The
// driver's coefficient builders and pushers are templates over the
// background/field type, so they run unchanged on it.
using StoredGrid = StoredCoordinateGrid<2, Device, typename DeviceTraits<Device>::array_layout, 3>;

struct StoredBackground {
    using grid_type = StoredGrid;
    using layout_type = typename DeviceTraits<Device>::array_layout;
    using vector_field_type = VectorField<grid_type, 3, layout_type>;
    grid_type grid;
    vector_field_type magnetic_field;
    vector_field_type velocity_field;
};

StoredBackground make_stored_background(int nx, int ny, const double* x_edges,
                                        const double* y_edges, const double* b,
                                        const double* v) {
    using metadata_type = Grid<2, Device, typename DeviceTraits<Device>::array_layout, 3>;
    typename metadata_type::index_array_type extents{};
    extents[0] = nx;
    extents[1] = ny;
    typename metadata_type::ghost_array_type ghosts{};
    typename metadata_type::periodic_array_type periodic{};
    for (int dim = 0; dim < 2; ++dim) {
        ghosts[dim][LowerBoundary] = 2;
        ghosts[dim][UpperBoundary] = 2;
        periodic[dim] = 1;
    }
    metadata_type metadata(extents, ghosts, periodic);
    const int max_faces = std::max(nx, ny) + 5;
    typename StoredGrid::coordinate_view_type faces("stored_faces", 2, max_faces);
    const double* edges[2] = {x_edges, y_edges};
    const int counts[2] = {nx, ny};
    for (int dim = 0; dim < 2; ++dim) {
        const int n = counts[dim];
        const double* e = edges[dim];
        const double w = e[n] - e[0];
        for (int storage = 0; storage < max_faces; ++storage) {
            const int k = storage - 2;
            double f = 0.0;
            if (k < 0) {
                f = e[n + k] - w;
            } else if (k > n) {
                f = (k - n <= n) ? e[k - n] + w : e[n] + w;
            } else {
                f = e[k];
            }
            faces(dim, storage) = f;
        }
    }
    StoredBackground result;
    result.grid = GridValidation::make_validated_stored_coordinate_grid<2, Device,
        typename DeviceTraits<Device>::array_layout, 3>(metadata, faces);
    result.magnetic_field = StoredBackground::vector_field_type(result.grid, "stored_b",
                                                                GridCentering::CellCentered);
    result.velocity_field = StoredBackground::vector_field_type(result.grid, "stored_v",
                                                                GridCentering::CellCentered);
    const std::size_t cells = static_cast<std::size_t>(nx) * static_cast<std::size_t>(ny);
    for (int comp = 0; comp < 3; ++comp) {
        for (int j = 0; j < ny; ++j) {
            for (int i = 0; i < nx; ++i) {
                typename StoredGrid::index_array_type idx{};
                idx[0] = i;
                idx[1] = j;
                const std::size_t src = static_cast<std::size_t>(comp) * cells +
                                        static_cast<std::size_t>(j) * nx + i;
                result.magnetic_field.data(result.magnetic_field.flatten(idx), comp) = b[src];
                result.velocity_field.data(result.velocity_field.flatten(idx), comp) = v[src];
            }
        }
    }
    result.magnetic_field.fill_ghost_cells(FieldGhostFillMode::PeriodicOrClamped, true);
    result.velocity_field.fill_ghost_cells(FieldGhostFillMode::PeriodicOrClamped, true);
    return result;
}

// ---- header library on a 2D Cartesian grid -------------------------------
using LibLayout = typename DeviceTraits<Device>::array_layout;
using LibMeta = Grid<2, Device, LibLayout, 3>;
using LibAnalyticGrid = AnalyticCoordinateGrid<2, Device, LibLayout, 3>;
using LibSystem = ParticleSystem<2, Device, LibLayout>;

// Uniform edges -> the analytic grid the field reader builds
// (AthenaFieldReader.hpp:195-227); periodic flags per axis.
LibAnalyticGrid make_lib_analytic_grid(int nx, int ny, const double* x_edges,
                                       const double* y_edges, const int* periodic) {
    typename LibMeta::index_array_type extents{};
    extents[0] = nx;
    extents[1] = ny;
    typename LibMeta::ghost_array_type ghosts{};
    typename LibMeta::periodic_array_type flags{};
    for (int dim = 0; dim < 2; ++dim) {
        ghosts[dim][LowerBoundary] = 2;
        ghosts[dim][UpperBoundary] = 2;
        flags[dim] = periodic[dim];
    }
    LibMeta metadata(extents, ghosts, flags);
    typename LibAnalyticGrid::discretization_array_type discretization{};
    typename LibAnalyticGrid::scalar_array_type start{};
    typename LibAnalyticGrid::scalar_array_type step{};
    const double* edges[2] = {x_edges, y_edges};
    const int counts[2] = {nx, ny};
    for (int dim = 0; dim < 2; ++dim) {
        discretization[dim] = AnalyticGridDiscretization::UniformSpacing;
        start[dim] = edges[dim][0];
        step[dim] = (edges[dim][counts[dim]] - edges[dim][0]) / counts[dim];
    }
    return GridValidation::make_validated_analytic_coordinate_grid<2, Device, LibLayout, 3>(
        metadata, discretization, start, step);
}

// Explicit faces (nx+5 / ny+5, face -2 first) -> the reference's validated
// StoredCoordinateGrid (StoredCoordinateGrid.hpp:53-66,
// GridValidation.hpp:773-784) with the same metadata as the analytic grid.
using LibStoredGrid = StoredCoordinateGrid<2, Device, LibLayout, 3>;
LibStoredGrid make_lib_stored_grid(int nx, int ny, const double* x_faces, const double* y_faces,
                                   const int* periodic) {
    typename LibMeta::index_array_type extents{};
    extents[0] = nx;
    extents[1] = ny;
    typename LibMeta::ghost_array_type ghosts{};
    typename LibMeta::periodic_array_type flags{};
    for (int dim = 0; dim < 2; ++dim) {
        ghosts[dim][LowerBoundary] = 2;
        ghosts[dim][UpperBoundary] = 2;
        flags[dim] = periodic[dim];
    }
    LibMeta metadata(extents, ghosts, flags);
    const int max_faces = std::max(nx, ny) + 5;
    typename LibStoredGrid::coordinate_view_type faces("lib_stored_faces", 2, max_faces);
    const double* f[2] = {x_faces, y_faces};
    const int counts[2] = {nx, ny};
    for (int dim = 0; dim < 2; ++dim) {
        for (int k = 0; k < max_faces; ++k) {
            // the shorter axis' unused tail continues its last spacing
            const int n = counts[dim] + 5;
            faces(dim, k) = k < n ? f[dim][k]
                                  : f[dim][n - 1] + (k - n + 1) * (f[dim][n - 1] - f[dim][n - 2]);
        }
    }
    return GridValidation::make_validated_stored_coordinate_grid<2, Device, LibLayout, 3>(
        metadata, faces);
}

// Faces of a stored grid for the library calls that follow (NULL: the
// analytic grid on the calls' uniform edges).
const double* g_lib_faces[2] = {nullptr, nullptr};

// Run body(grid) on the grid the next library call asks for; exceptions
// become the -1 return with the message kept.
template <typename Body>
long long on_lib_grid(int nx, int ny, const double* x_edges, const double* y_edges,
                      const int* periodic, Body&& body) {
    try {
        if (g_lib_faces[0] != nullptr) {
            const LibStoredGrid grid =
                make_lib_stored_grid(nx, ny, g_lib_faces[0], g_lib_faces[1], periodic);
            return body(grid);
        }
        const LibAnalyticGrid grid = make_lib_analytic_grid(nx, ny, x_edges, y_edges, periodic);
        return body(grid);
    } catch (const std::exception& error) {
        g_last_error = error.what();
        return -1;
    }
}

// Particle arrays of the host side: doubles [10][capacity] = x, y, prev x,
// prev y, prev-step x, prev-step y, momentum, mu, weight, E0; ints
// [3][capacity] = status, split level, sort key; ids [capacity].
struct LibHost {
    unsigned long long* id;
    double* d;
    int* i;
    long long capacity;
};

void lib_load(LibSystem& sys, const LibHost& h) {
    const long long c = h.capacity;
    for (long long n = 0; n < c; ++n) {
        sys.particle_id(n) = h.id[n];
        sys.position(n, 0) = h.d[0 * c + n];
        sys.position(n, 1) = h.d[1 * c + n];
        sys.previous_position(n, 0) = h.d[2 * c + n];
        sys.previous_position(n, 1) = h.d[3 * c + n];
        sys.previous_step_position(n, 0) = h.d[4 * c + n];
        sys.previous_step_position(n, 1) = h.d[5 * c + n];
        sys.momentum(n) = h.d[6 * c + n];
        sys.mu(n) = h.d[7 * c + n];
        sys.weight(n) = h.d[8 * c + n];
        sys.initial_kinetic_energy(n) = h.d[9 * c + n];
        sys.status(n) = h.i[0 * c + n];
        sys.split_level(n) = h.i[1 * c + n];
        sys.sort_key(n) = h.i[2 * c + n];
    }
}

void lib_store(const LibSystem& sys, const LibHost& h) {
    const long long c = h.capacity;
    for (long long n = 0; n < c; ++n) {
        h.id[n] = sys.particle_id(n);
        h.d[0 * c + n] = sys.position(n, 0);
        h.d[1 * c + n] = sys.position(n, 1);
        h.d[2 * c + n] = sys.previous_position(n, 0);
        h.d[3 * c + n] = sys.previous_position(n, 1);
        h.d[4 * c + n] = sys.previous_step_position(n, 0);
        h.d[5 * c + n] = sys.previous_step_position(n, 1);
        h.d[6 * c + n] = sys.momentum(n);
        h.d[7 * c + n] = sys.mu(n);
        h.d[8 * c + n] = sys.weight(n);
        h.d[9 * c + n] = sys.initial_kinetic_energy(n);
        h.i[0 * c + n] = sys.status(n);
        h.i[1 * c + n] = sys.split_level(n);
        h.i[2 * c + n] = sys.sort_key(n);
    }
}

ParticleProperties lib_properties(const double* props) {
    ParticleProperties p;
    p.species = ParticleSpecies::Custom;
    p.rest_mass = props[0];
    p.charge = props[1];
    p.speed_of_light = props[2];
    p.energy_scale_erg = props[3];
    return p;
}

}  // namespace

extern "C" {

const char* ref_last_error() { return g_last_error.c_str(); }
double ref_last_move_seconds() { return g_last_move_seconds; }

// Library calls after this one run on the stored grid of these faces
// (nx+5 / ny+5 each, face -2 first); NULL restores the analytic grid.
void ref_set_lib_stored_faces(const double* x_faces, const double* y_faces) {
    g_lib_faces[0] = x_faces;
    g_lib_faces[1] = y_faces;
}

// Build the driver's per-cell coefficient table (16 Parker or 21 focused
// components) for one compact field file.  out holds point_count * C doubles
// in the Field's flattened order (x fastest over nx+4, then ny+4).
long long ref_table(const char* path, int focused, double* out, long long out_len) {
    try {
        const std::string file(path);
        const auto slash = file.find_last_of('/');
        const std::string dir = file.substr(0, slash);
        const int frame = std::stoi(file.substr(slash + 6, 5));
        if (focused) {
            const auto table = load_coefficient_frame<>(dir, frame);
            const long long n = static_cast<long long>(table.point_count()) *
                                coefficient_component_count;
            if (out != nullptr && out_len >= n) {
                std::copy(table.data.data(), table.data.data() + n, out);
            }
            return n;
        }
        const auto table = load_parker_coefficient_frame<>(dir, frame);
        const long long n = static_cast<long long>(table.point_count()) *
                            parker_coefficient_component_count;
        if (out != nullptr && out_len >= n) {
            std::copy(table.data.data(), table.data.data() + n, out);
        }
        return n;
    } catch (const std::exception& error) {
        g_last_error = error.what();
        return -1;
    }
}

// inject_uniform_particles for one frame.  When band_lo < band_hi the y draw
// uses [band_lo, band_hi) instead of the whole domain (the injection band of
// the benchmark configuration; the rest of the kernel is unchanged).
long long ref_inject(const char* field_dir, const double* d, const int* ip,
                     unsigned long long seed, int frame, unsigned long long capacity,
                     unsigned long long count, unsigned long long requested,
                     double band_lo, double band_hi, double* x, double* y, double* p,
                     double* t, double* dt, double* w, double* mu, int* status,
                     int* level) {
    try {
        const auto s = settings_from(d, ip);
        const auto table = load_parker_coefficient_frame<>(field_dir, frame);
        auto ds = device_settings_for(s, table);
        if (band_lo < band_hi) {
            ds.y_lower = band_lo;
            ds.y_upper = band_hi;
        }
        ReconnectionParticleStorage<> storage(capacity);
        const HostParticles h{x, y, p, t, dt, w, mu, status, level};
        load_storage(storage, h, count);
        RandomManager<> rng(seed);
        Kokkos::ShimImpl::current_frame() = static_cast<std::uint32_t>(frame);
        const double interval_start = static_cast<double>(frame) * s.mhd_dt;
        inject_uniform_particles(storage, rng, ds, requested, interval_start);
        store_storage(storage, h, storage.count);
        return static_cast<long long>(storage.count);
    } catch (const std::exception& error) {
        g_last_error = error.what();
        return -1;
    }
}

// One interval push (Parker or focused per ip[IP_FOCUSED]) between
// fieldNNNNN.bin frames `frame` and `frame + 1` of field_dir.
long long ref_push(const char* field_dir, const double* d, const int* ip,
                   unsigned long long seed, int frame, unsigned long long capacity,
                   unsigned long long count, double* x, double* y, double* p, double* t,
                   double* dt, double* w, double* mu, int* status, int* level) {
    try {
        const auto s = settings_from(d, ip);
        ReconnectionParticleStorage<> storage(capacity);
        const HostParticles h{x, y, p, t, dt, w, mu, status, level};
        load_storage(storage, h, count);
        RandomManager<> rng(seed);
        Kokkos::ShimImpl::current_frame() = static_cast<std::uint32_t>(frame);
        const double interval_start = static_cast<double>(frame) * s.mhd_dt;
        if (ip[IP_FOCUSED]) {
            const auto lower = load_coefficient_frame<>(field_dir, frame);
            const auto upper = load_coefficient_frame<>(field_dir, frame + 1);
            const auto ds = device_settings_for(s, lower);
            Kokkos::fence();
            const auto t0 = std::chrono::steady_clock::now();
            move_particles_one_interval(storage, lower, upper, rng, ds, interval_start);
            Kokkos::fence();
            g_last_move_seconds = std::chrono::duration<double>(
                std::chrono::steady_clock::now() - t0).count();
        } else {
            const auto lower = load_parker_coefficient_frame<>(field_dir, frame);
            const auto upper = load_parker_coefficient_frame<>(field_dir, frame + 1);
            const auto ds = device_settings_for(s, lower);
            Kokkos::fence();
            const auto t0 = std::chrono::steady_clock::now();
            move_parker_particles_one_interval(storage, lower, upper, rng, ds,
                                               interval_start);
            Kokkos::fence();
            g_last_move_seconds = std::chrono::duration<double>(
                std::chrono::steady_clock::now() - t0).count();
        }
        store_storage(storage, h, count);
        return static_cast<long long>(count);
    } catch (const std::exception& error) {
        g_last_error = error.what();
        return -1;
    }
}

// split_particles; writes the split and skipped counters and returns the new
// stored count.  Run with one OpenMP thread for the serial child order.
long long ref_split(const char* field_dir, const double* d, const int* ip, int frame,
                    unsigned long long capacity, unsigned long long count, double* x,
                    double* y, double* p, double* t, double* dt, double* w, double* mu,
                    int* status, int* level, unsigned long long* split_out,
                    unsigned long long* skipped_out) {
    try {
        const auto s = settings_from(d, ip);
        const auto table = load_parker_coefficient_frame<>(field_dir, frame);
        const auto ds = device_settings_for(s, table);
        ReconnectionParticleStorage<> storage(capacity);
        const HostParticles h{x, y, p, t, dt, w, mu, status, level};
        load_storage(storage, h, count);
        const auto counts = split_particles(storage, ds);
        *split_out = counts.first;
        *skipped_out = counts.second;
        store_storage(storage, h, storage.count);
        return static_cast<long long>(storage.count);
    } catch (const std::exception& error) {
        g_last_error = error.what();
        return -1;
    }
}

// Coefficient table on explicit face edges (StoredCoordinateGrid path).
long long ref_table_stored(int nx, int ny, const double* x_edges, const double* y_edges,
                           const double* b, const double* v, int focused, double* out,
                           long long out_len) {
    try {
        const auto background = make_stored_background(nx, ny, x_edges, y_edges, b, v);
        if (focused) {
            const auto table = make_reconnection_coefficients(background, "stored_table");
            const long long n = static_cast<long long>(table.point_count()) *
                                coefficient_component_count;
            if (out != nullptr && out_len >= n) {
                std::copy(table.data.data(), table.data.data() + n, out);
            }
            return n;
        }
        const auto table = make_parker_reconnection_coefficients(background, "stored_table");
        const long long n = static_cast<long long>(table.point_count()) *
                            parker_coefficient_component_count;
        if (out != nullptr && out_len >= n) {
            std::copy(table.data.data(), table.data.data() + n, out);
        }
        return n;
    } catch (const std::exception& error) {
        g_last_error = error.what();
        return -1;
    }
}

// One interval push on explicit face edges: lower frame (b0, v0) and upper
// frame (b1, v1) share the edges.
long long ref_push_stored(int nx, int ny, const double* x_edges, const double* y_edges,
                          const double* b0, const double* v0, const double* b1,
                          const double* v1, const double* d, const int* ip,
                          unsigned long long seed, int frame, unsigned long long capacity,
                          unsigned long long count, double* x, double* y, double* p, double* t,
                          double* dt, double* w, double* mu, int* status, int* level) {
    try {
        const auto s = settings_from(d, ip);
        ReconnectionParticleStorage<> storage(capacity);
        const HostParticles h{x, y, p, t, dt, w, mu, status, level};
        load_storage(storage, h, count);
        RandomManager<> rng(seed);
        Kokkos::ShimImpl::current_frame() = static_cast<std::uint32_t>(frame);
        const double interval_start = static_cast<double>(frame) * s.mhd_dt;
        const auto lower_bg = make_stored_background(nx, ny, x_edges, y_edges, b0, v0);
        const auto upper_bg = make_stored_background(nx, ny, x_edges, y_edges, b1, v1);
        if (ip[IP_FOCUSED]) {
            const auto lower = make_reconnection_coefficients(lower_bg, "stored_lower");
            const auto upper = make_reconnection_coefficients(upper_bg, "stored_upper");
            const auto ds = device_settings_for(s, lower);
            move_particles_one_interval(storage, lower, upper, rng, ds, interval_start);
        } else {
            const auto lower = make_parker_reconnection_coefficients(lower_bg, "stored_lower");
            const auto upper = make_parker_reconnection_coefficients(upper_bg, "stored_upper");
            const auto ds = device_settings_for(s, lower);
            move_parker_particles_one_interval(storage, lower, upper, rng, ds,
                                               interval_start);
        }
        store_storage(storage, h, count);
        return static_cast<long long>(count);
    } catch (const std::exception& error) {
        g_last_error = error.what();
        return -1;
    }
}

// The reference's slab quasi-linear pitch-angle scattering closure
// (include/LegencyModel.hpp:557-645) on arrays of inputs.
long long ref_qlt(long long n, const double* mu, const double* omega, const double* speed,
                  const double* sigma2, const double* lc, const double* gk, const double* h0,
                  double* d_out, double* dd_out) {
    for (long long k = 0; k < n; ++k) {
        LegencyModel::PitchAngleScatteringParameters parameters;
        parameters.spectral_index = gk[k];
        parameters.resonance_regularization_h0 = h0[k];
        d_out[k] = LegencyModel::pitch_angle_diffusion_coefficient(mu[k], omega[k], speed[k],
                                                                   sigma2[k], lc[k], parameters);
        dd_out[k] = LegencyModel::pitch_angle_diffusion_derivative(mu[k], d_out[k], omega[k],
                                                                   speed[k], lc[k], parameters);
    }
    return n;
}

// ParkerSolver steps on a uniform 2D Cartesian grid.  basis holds the
// packed coefficient basis on every ghosted point (x fastest), 18 values per
// point in the solver's packed order: B(3) V(3) drift curl(3) primary(3)
// secondary(3) kappa_par kappa_perp divV (ParkerSolver.hpp:96-116); the
// fields handed to the solver are cut from it, so the solver rebuilds the
// same packed basis.  props = rest mass, charge, c, energy scale, courant.
// mode: 0 stochastic, 1 deterministic.  dts[steps] receives each step's dt;
// the noise frame of step s is first_step + s.  normals (NULL: the keyed
// stream) holds [steps][4][count] injected normals.
long long ref_lib_parker(int nx, int ny, const double* x_edges, const double* y_edges,
                         const int* periodic, const double* basis, int constant_ratio,
                         const double* props, unsigned long long seed, int first_step,
                         int steps, int mode, long long count, long long capacity,
                         unsigned long long* ids, double* d, int* ints, double* dts,
                         const double* normals) {
    return on_lib_grid(nx, ny, x_edges, y_edges, periodic,
                       [&](const auto& grid) -> long long {
        using G = std::decay_t<decltype(grid)>;
        using solver_type = ParkerSolver<G>;
        using vector_field = typename solver_type::vector_field_type;
        using scalar_field = typename solver_type::scalar_field_type;
        vector_field b(grid, "lib_b", GridCentering::CellCentered);
        vector_field v(grid, "lib_v", GridCentering::CellCentered);
        vector_field curl(grid, "lib_curl", GridCentering::CellCentered);
        vector_field primary(grid, "lib_primary", GridCentering::CellCentered);
        vector_field secondary(grid, "lib_secondary", GridCentering::CellCentered);
        scalar_field kpar(grid, "lib_kpar", GridCentering::CellCentered);
        scalar_field kperp(grid, "lib_kperp", GridCentering::CellCentered);
        scalar_field divv(grid, "lib_divv", GridCentering::CellCentered);
        const std::size_t points = b.point_count();
        for (std::size_t k = 0; k < points; ++k) {
            const double* row = basis + 18 * k;
            for (int c = 0; c < 3; ++c) {
                b.data(k, c) = row[c];
                v.data(k, c) = row[3 + c];
                curl.data(k, c) = row[6 + c];
                primary.data(k, c) = row[9 + c];
                secondary.data(k, c) = row[12 + c];
            }
            kpar.data(k, 0) = row[15];
            kperp.data(k, 0) = row[16];
            divv.data(k, 0) = row[17];
        }
        LegencyModel::DiffusionModelParameters parameters;
        ParkerCoefficient::DiffusionTensorDivergenceFieldSet<G> divergence;
        if (constant_ratio) {
            parameters.set_constant_perpendicular_parallel_ratio(1.0);
            divergence.perpendicular_model =
                LegencyModel::PerpendicularDiffusionModelKind::ConstantParallelRatio;
            divergence.constant_ratio_basis = primary;
        } else {
            divergence.parallel_basis = primary;
            divergence.perpendicular_basis = secondary;
        }
        typename solver_type::coefficient_field_set_type coefficients(
            curl, divergence, kpar, kperp, divv, parameters);
        LibSystem sys(static_cast<typename LibSystem::size_type>(count),
                      static_cast<typename LibSystem::size_type>(capacity),
                      lib_properties(props));
        const LibHost h{ids, d, ints, capacity};
        lib_load(sys, h);
        solver_type solver(sys, grid, b, v, coefficients);
        solver.set_dimensionless_courant_scale(Units::DimensionlessValue(props[4]));
        RandomManager<> random_manager(seed);
        Kokkos::ShimImpl::auto_frame_enabled() = 0;
        for (int s = 0; s < steps; ++s) {
            Kokkos::ShimImpl::current_frame() = static_cast<std::uint32_t>(first_step + s);
            Kokkos::ShimImpl::external_normals() =
                normals != nullptr ? normals + static_cast<std::size_t>(s) * 4 * count : nullptr;
            Kokkos::ShimImpl::external_count() = static_cast<std::uint64_t>(count);
            dts[s] = mode == 0 ? solver.advance_stochastic(random_manager)
                               : solver.advance_deterministic();
        }
        Kokkos::ShimImpl::external_normals() = nullptr;
        lib_store(solver.particles, h);
        return 0;
    });
}

// FocusTransportSolver steps on a uniform 2D Cartesian grid.  basis holds
// the 27-value packed basis per ghosted point (FocusSolver.hpp:106-136):
// B(3) b(3) V(3) gradient drift basis(3) curvature drift basis(3)
// perpendicular diffusion advection(3) |B| kappa_par kappa_perp divV
// focusing bb:gradV b.dV/dt sigma^2 Lc.  Fields the step does not read
// (ln B, grad ln B, curvature, dV/dt) are zero.  props = rest mass, charge,
// c, energy scale, courant; scat = spectral index, h0, floors (|B|, sigma^2,
// Lc, speed), maximum |mu|.
long long ref_lib_focus(int nx, int ny, const double* x_edges, const double* y_edges,
                        const int* periodic, const double* basis, int constant_ratio,
                        const double* props, const double* scat, unsigned long long seed,
                        int first_step, int steps, int mode, long long count, long long capacity,
                        unsigned long long* ids, double* d, int* ints, double* dts,
                        const double* normals) {
    return on_lib_grid(nx, ny, x_edges, y_edges, periodic,
                       [&](const auto& grid) -> long long {
        using G = std::decay_t<decltype(grid)>;
        using solver_type = FocusSolver<G>;
        using vector_field = typename solver_type::vector_field_type;
        using scalar_field = typename solver_type::scalar_field_type;
        auto vec = [&](const char* name) { return vector_field(grid, name, GridCentering::CellCentered); };
        auto sca = [&](const char* name) { return scalar_field(grid, name, GridCentering::CellCentered); };
        vector_field b = vec("f_b"), dir = vec("f_dir"), v = vec("f_v"), grad = vec("f_grad"),
                     curv = vec("f_curv"), perp = vec("f_perp"), glb = vec("f_glb"),
                     kcurv = vec("f_kcurv"), dvdt = vec("f_dvdt");
        scalar_field bmag = sca("f_bmag"), kpar = sca("f_kpar"), kperp = sca("f_kperp"),
                     divv = sca("f_divv"), focus = sca("f_focus"), bbgv = sca("f_bbgv"),
                     conv = sca("f_conv"), sig = sca("f_sig"), lc = sca("f_lc"),
                     logb = sca("f_logb");
        const std::size_t points = b.point_count();
        for (std::size_t k = 0; k < points; ++k) {
            const double* row = basis + 27 * k;
            for (int c = 0; c < 3; ++c) {
                b.data(k, c) = row[c];
                dir.data(k, c) = row[3 + c];
                v.data(k, c) = row[6 + c];
                grad.data(k, c) = row[9 + c];
                curv.data(k, c) = row[12 + c];
                perp.data(k, c) = row[15 + c];
                glb.data(k, c) = 0.0;
                kcurv.data(k, c) = 0.0;
                dvdt.data(k, c) = 0.0;
            }
            bmag.data(k, 0) = row[18];
            kpar.data(k, 0) = row[19];
            kperp.data(k, 0) = row[20];
            divv.data(k, 0) = row[21];
            focus.data(k, 0) = row[22];
            bbgv.data(k, 0) = row[23];
            conv.data(k, 0) = row[24];
            sig.data(k, 0) = row[25];
            lc.data(k, 0) = row[26];
            logb.data(k, 0) = 0.0;
        }
        LegencyModel::DiffusionModelParameters diffusion;
        if (constant_ratio) diffusion.set_constant_perpendicular_parallel_ratio(1.0);
        LegencyModel::PitchAngleScatteringParameters scattering;
        scattering.spectral_index = scat[0];
        scattering.resonance_regularization_h0 = scat[1];
        scattering.minimum_magnetic_field_magnitude = scat[2];
        scattering.minimum_sigma2 = scat[3];
        scattering.minimum_correlation_length = scat[4];
        scattering.minimum_speed = scat[5];
        typename solver_type::coefficient_field_set_type coefficients(
            dir, bmag, logb, glb, kcurv, grad, curv, perp, kpar, kperp, divv, focus, bbgv, dvdt,
            conv, sig, lc, diffusion, scattering);
        LibSystem sys(static_cast<typename LibSystem::size_type>(count),
                      static_cast<typename LibSystem::size_type>(capacity),
                      lib_properties(props));
        const LibHost h{ids, d, ints, capacity};
        lib_load(sys, h);
        solver_type solver(sys, grid, b, v, coefficients);
        solver.set_dimensionless_courant_scale(Units::DimensionlessValue(props[4]));
        solver.set_maximum_pitch_angle_cosine(scat[6]);
        RandomManager<> random_manager(seed);
        Kokkos::ShimImpl::auto_frame_enabled() = 0;
        for (int s = 0; s < steps; ++s) {
            Kokkos::ShimImpl::current_frame() = static_cast<std::uint32_t>(first_step + s);
            Kokkos::ShimImpl::external_normals() =
                normals != nullptr ? normals + static_cast<std::size_t>(s) * 4 * count : nullptr;
            Kokkos::ShimImpl::external_count() = static_cast<std::uint64_t>(count);
            dts[s] = mode == 0 ? solver.advance_stochastic(random_manager)
                               : solver.advance_deterministic();
        }
        Kokkos::ShimImpl::external_normals() = nullptr;
        lib_store(solver.particles, h);
        return 0;
    });
}

// ParticleSystem lifecycle on the same grid: op 0 boundary conditions,
// 1 sort_by_key(key_lo, key_hi), 2 compact_active_particles, 3
// split_particles_on_energy_growth (policy = split_ratio, min child weight),
// 4 capture_previous_positions.  stats[6]: count after, then the split
// statistics (active, split, skipped capacity, skipped invalid baseline,
// skipped minimum weight) for op 3.
long long ref_lib_system(int nx, int ny, const double* x_edges, const double* y_edges,
                         const int* periodic, const double* props, int op, int key_lo,
                         int key_hi, long long count, long long capacity,
                         unsigned long long* ids, double* d, int* ints,
                         unsigned long long* stats) {
    return on_lib_grid(nx, ny, x_edges, y_edges, periodic,
                       [&](const auto& grid) -> long long {
        using G = std::decay_t<decltype(grid)>;
        ParticleSplittingPolicy policy;
        policy.energy_split_ratio = props[5];
        policy.minimum_child_weight = props[6];
        LibSystem sys(static_cast<typename LibSystem::size_type>(count),
                      static_cast<typename LibSystem::size_type>(capacity),
                      lib_properties(props), policy);
        const LibHost h{ids, d, ints, capacity};
        lib_load(sys, h);
        for (int k = 0; k < 6; ++k) stats[k] = 0;
        if (op == 0) {
            sys.apply_grid_boundary_conditions(grid, GridDomain::PhysicalDomain);
        } else if (op == 1) {
            sys.sort_by_key(key_lo, key_hi);
        } else if (op == 2) {
            sys.compact_active_particles();
        } else if (op == 3) {
            const auto st = sys.split_particles_on_energy_growth();
            stats[1] = st.active_count;
            stats[2] = st.split_count;
            stats[3] = st.skipped_capacity_count;
            stats[4] = st.skipped_invalid_baseline_count;
            stats[5] = st.skipped_minimum_weight_count;
        } else if (op == 4) {
            sys.capture_previous_positions();
        }
        stats[0] = sys.particle_count();
        lib_store(sys, h);
        return 0;
    });
}

// The reference CLI entry point itself.  Noise frames are keyed as
// frame_base + launch ordinal, frame_base being the run's start frame.
int ref_main(int argc, char** argv, int frame_base) {
    Kokkos::ShimImpl::launch_ordinals() = Kokkos::ShimImpl::LaunchOrdinals{};
    Kokkos::ShimImpl::auto_frame_enabled() = 1;
    Kokkos::ShimImpl::auto_frame_base() = static_cast<std::uint32_t>(frame_base);
    const int rc = kpt_ref_main(argc, argv);
    Kokkos::ShimImpl::auto_frame_enabled() = 0;
    return rc;
}

}  // extern "C"

// ---- ParticleGenerator on the library grid ----------------------------------
namespace {

template <typename G, int C>
using LibGenField = Field<G, C>;

// field values: C doubles per stored point in the Field's flattened order
// (dim 0 fastest over the ghosted extent of its centering);
// centering[dim]: 0 cell, 1 face.
template <int C, typename G>
LibGenField<G, C> lib_gen_field(const G& grid, const int* centering, const double* values) {
    typename LibGenField<G, C>::centering_array_type c{};
    for (int dim = 0; dim < 2; ++dim) {
        c[dim] = centering[dim] == 0 ? GridCentering::CellCentered : GridCentering::FaceCentered;
    }
    LibGenField<G, C> field(grid, "lib_generator_field", c);
    const std::size_t points = field.point_count();
    for (std::size_t k = 0; k < points; ++k) {
        for (int comp = 0; comp < C; ++comp) field.data(k, comp) = values[k * C + comp];
    }
    return field;
}

AxisAlignedParticleRegion<2> lib_gen_region(const double* r) {
    Kokkos::Array<double, 2> lower{};
    Kokkos::Array<double, 2> upper{};
    lower[0] = r[0];
    lower[1] = r[1];
    upper[0] = r[2];
    upper[1] = r[3];
    return make_particle_region<2>(lower, upper);
}

template <int C, typename G>
void lib_generator_run(const G& grid, LibSystem& sys, int op, const int* centering,
                       const double* values, const double* region, const double* pred,
                       const double* kin, const unsigned long long* plan_in, int selection,
                       unsigned long long seed) {
    const auto field = lib_gen_field<C>(grid, centering, values);
    const double threshold = pred[0];
    const auto comparison = static_cast<FieldPredicateComparison>(static_cast<int>(pred[1]));
    const int component = static_cast<int>(pred[2]);
    const auto domain = static_cast<GridDomain>(static_cast<int>(pred[3]));
    ParticleInjectionKinematics<2> kinematics;
    kinematics.momentum_magnitude = kin[0];
    kinematics.mu = kin[1];
    kinematics.weight = kin[2];
    kinematics.status = static_cast<ParticleStatus>(static_cast<int>(kin[3]));
    ParticleInjectionPlan plan{plan_in[0], plan_in[1], plan_in[2], static_cast<int>(plan_in[3])};
    const auto select = static_cast<ParticleRecycleSelection>(selection);
    RandomManager<> random_manager(seed);
    switch (op) {
        case 0:
            inject_particles_uniform(sys, random_manager, lib_gen_region(region), plan, kinematics);
            break;
        case 1:
            inject_particles_uniform_if(
                sys, random_manager, lib_gen_region(region), plan, kinematics,
                make_field_threshold_particle_predicate(field, threshold, comparison, component,
                                                        domain));
            break;
        case 2:
            if (region != nullptr) {
                inject_particles_uniform_where_field(sys, random_manager, lib_gen_region(region),
                                                     plan, kinematics, field, threshold,
                                                     comparison, component, domain);
            } else {
                inject_particles_uniform_where_field(sys, random_manager, plan, kinematics, field,
                                                     threshold, comparison, component, domain);
            }
            break;
        case 3:
            inject_particles_uniform_in_grid(sys, random_manager, grid, plan, kinematics, domain);
            break;
        case 4:
            recycle_particles_uniform(sys, random_manager, lib_gen_region(region), kinematics,
                                      select);
            break;
        case 5:
            recycle_particles_uniform_if(
                sys, random_manager, lib_gen_region(region), kinematics,
                make_field_threshold_particle_predicate(field, threshold, comparison, component,
                                                        domain),
                select, static_cast<int>(plan_in[3]));
            break;
        case 6:
            if (region != nullptr) {
                recycle_particles_uniform_where_field(sys, random_manager, lib_gen_region(region),
                                                      kinematics, field, threshold, comparison,
                                                      component, domain, select);
            } else {
                recycle_particles_uniform_where_field(sys, random_manager, kinematics, field,
                                                      threshold, comparison, component, domain,
                                                      select);
            }
            break;
        case 7:
            recycle_particles_uniform_in_grid(sys, random_manager, grid, kinematics, select,
                                              domain);
            break;
        default:
            throw std::runtime_error("ref_lib_generator: unknown op");
    }
}

template <int C, typename G>
long long lib_candidates_run(const G& grid, int kind, const int* centering,
                             const double* values, const double* region, const double* pred,
                             unsigned long long* indices, double* cumulative, long long max_out,
                             double* total) {
    const auto domain = static_cast<GridDomain>(static_cast<int>(pred[3]));
    if (kind == 1) {
        const auto set = make_grid_particle_candidate_set(grid, domain);
        const long long n = static_cast<long long>(set.candidate_count());
        for (long long k = 0; k < n && k < max_out; ++k) {
            indices[k] = static_cast<unsigned long long>(k);
            cumulative[k] = set.cumulative_weights(k);
        }
        *total = set.total_weight_cache;
        return n;
    }
    const auto field = lib_gen_field<C>(grid, centering, values);
    const auto comparison = static_cast<FieldPredicateComparison>(static_cast<int>(pred[1]));
    const int component = static_cast<int>(pred[2]);
    const auto set = region != nullptr
                         ? make_field_particle_candidate_set_in_region(
                               field, lib_gen_region(region), pred[0], comparison, component,
                               domain)
                         : make_field_particle_candidate_set(field, pred[0], comparison,
                                                            component, domain);
    const long long n = static_cast<long long>(set.candidate_count());
    for (long long k = 0; k < n && k < max_out; ++k) {
        indices[k] = static_cast<unsigned long long>(set.point_indices(k));
        cumulative[k] = set.cumulative_weights(k);
    }
    *total = set.total_weight_cache;
    return n;
}

}  // namespace

extern "C" {

// ParticleGenerator (include/ParticleGenerator.hpp) on the library grid.
// components 1 or 3 of the field (centering[2]: 0 cell, 1 face); region[4]
// = lower x, lower y, upper x, upper y, or NULL for the grid-domain
// overloads of op 2 and 6; pred[4] = threshold, comparison, component,
// domain; kin[4] = momentum, mu, weight, status; plan[4] = first index,
// count, first id, max attempts (op 5 takes its max attempts from plan[3]).
// op: 0 inject_particles_uniform, 1 inject_particles_uniform_if with the
// field threshold predicate, 2 inject_particles_uniform_where_field, 3
// inject_particles_uniform_in_grid, 4 recycle_particles_uniform, 5
// recycle_particles_uniform_if, 6 recycle_particles_uniform_where_field, 7
// recycle_particles_uniform_in_grid.  The noise frame is `frame`.
// out_count receives the particle count afterwards.
long long ref_lib_generator(int nx, int ny, const double* x_edges, const double* y_edges,
                            const int* periodic, const double* props, int op, int components,
                            const int* centering, const double* values, const double* region,
                            const double* pred, const double* kin,
                            const unsigned long long* plan, int selection,
                            unsigned long long seed, unsigned frame, long long count,
                            long long capacity, unsigned long long* ids, double* d, int* ints,
                            unsigned long long* out_count) {
    return on_lib_grid(nx, ny, x_edges, y_edges, periodic,
                       [&](const auto& grid) -> long long {
        using G = std::decay_t<decltype(grid)>;
        LibSystem sys(static_cast<typename LibSystem::size_type>(count),
                      static_cast<typename LibSystem::size_type>(capacity),
                      lib_properties(props));
        const LibHost h{ids, d, ints, capacity};
        lib_load(sys, h);
        Kokkos::ShimImpl::auto_frame_enabled() = 0;
        Kokkos::ShimImpl::current_frame() = frame;
        if (components == 1) {
            lib_generator_run<1>(grid, sys, op, centering, values, region, pred, kin, plan,
                                 selection, seed);
        } else if (components == 3) {
            lib_generator_run<3>(grid, sys, op, centering, values, region, pred, kin, plan,
                                 selection, seed);
        } else {
            throw std::runtime_error("ref_lib_generator: components must be 1 or 3");
        }
        *out_count = sys.particle_count();
        lib_store(sys, h);
        return 0;
    });
}

// Candidate sets: kind 0 field points passing the predicate (region or NULL
// for the whole domain), kind 1 grid cells of the domain (pred[3]).  Writes
// up to max_out point indices (cell ordinals for kind 1) and cumulative
// weights; returns the candidate count (-1 on error) and the total weight.
long long ref_lib_candidates(int nx, int ny, const double* x_edges, const double* y_edges,
                             const int* periodic, int kind, int components,
                             const int* centering, const double* values, const double* region,
                             const double* pred, unsigned long long* indices, double* cumulative,
                             long long max_out, double* total) {
    return on_lib_grid(nx, ny, x_edges, y_edges, periodic,
                       [&](const auto& grid) -> long long {
        using G = std::decay_t<decltype(grid)>;
        if (components == 3) {
            return lib_candidates_run<3>(grid, kind, centering, values, region, pred, indices,
                                         cumulative, max_out, total);
        }
        return lib_candidates_run<1>(grid, kind, centering, values, region, pred, indices,
                                     cumulative, max_out, total);
    });
}

}  // extern "C"

// ---- Parker coefficient precompute on the library grid ---------------------
extern "C" {

// ParkerCoefficient::make_legacy_transport_coefficient_fields
// (include/ParkerCoefficient.hpp:1102-1155) from cell-centred B and V (3
// doubles per ghosted point, ghosts as given), then the solver's packed
// basis (ParkerSolver.hpp:514-598) copied to packed (18 doubles per point).
// turb_mode 0: constant state turb[4] = sigma2, l2d, lslab, lc (lc <= 0 =
// the slab length); 1: per-point fields turb_fields[4][points] = sigma2,
// l2d, lslab, lc.  props = rest mass, charge, c, energy scale; params =
// model (0 README, 1 constant ratio), parallel prefactor, perpendicular
// prefactor, ratio, minimum |B|, minimum Vsw, minimum sigma2; drift_floor =
// minimum B^2 of curl(B/B^2); ghost_mode 0 PeriodicOrClamped, 1 PeriodicOnly.
long long ref_lib_parker_coefficients(int nx, int ny, const double* x_edges,
                                      const double* y_edges, const int* periodic,
                                      const double* b_values, const double* v_values,
                                      int turb_mode, const double* turb,
                                      const double* turb_fields, const double* props,
                                      const double* params, double drift_floor, int ghost_mode,
                                      double* packed_out) {
    return on_lib_grid(nx, ny, x_edges, y_edges, periodic,
                       [&](const auto& grid) -> long long {
        using G = std::decay_t<decltype(grid)>;
        using solver_type = ParkerSolver<G>;
        using vector_field = typename solver_type::vector_field_type;
        vector_field b(grid, "coef_b", GridCentering::CellCentered);
        vector_field v(grid, "coef_v", GridCentering::CellCentered);
        const std::size_t points = b.point_count();
        for (std::size_t k = 0; k < points; ++k) {
            for (int c = 0; c < 3; ++c) {
                b.data(k, c) = b_values[3 * k + c];
                v.data(k, c) = v_values[3 * k + c];
            }
        }
        const auto model = TurbulencePropertyModel::constant_code_units(turb[0], turb[1],
                                                                        turb[2], turb[3]);
        TurbulenceProperties<G> turbulence(
            grid, model,
            turb_mode == 0 ? TurbulencePropertyStorageMode::ConstantOnly
                           : TurbulencePropertyStorageMode::Field);
        if (turb_mode != 0) {
            for (std::size_t k = 0; k < points; ++k) {
                turbulence.sigma2.data(k, 0) = turb_fields[0 * points + k];
                turbulence.l2d.data(k, 0) = turb_fields[1 * points + k];
                turbulence.lslab.data(k, 0) = turb_fields[2 * points + k];
                turbulence.lc.data(k, 0) = turb_fields[3 * points + k];
            }
        }
        LegencyModel::DiffusionModelParameters parameters;
        parameters.parallel_prefactor = params[1];
        parameters.perpendicular_prefactor = params[2];
        parameters.minimum_magnetic_field_magnitude = params[4];
        parameters.minimum_solar_wind_speed = params[5];
        parameters.minimum_sigma2 = params[6];
        if (static_cast<int>(params[0]) == 1) {
            parameters.set_constant_perpendicular_parallel_ratio(params[3]);
        } else {
            parameters.perpendicular_parallel_ratio = params[3];
            parameters.use_readme_perpendicular_formula();
        }
        const auto coefficients = ParkerCoefficient::make_legacy_transport_coefficient_fields(
            b, v, turbulence, lib_properties(props), "coef", parameters, drift_floor,
            ghost_mode == 0 ? FieldGhostFillMode::PeriodicOrClamped
                            : FieldGhostFillMode::PeriodicOnly);
        LibSystem sys(0, 1, lib_properties(props));
        solver_type solver(sys, grid, b, v, coefficients);
        for (std::size_t k = 0; k < points; ++k) {
            for (int c = 0; c < 18; ++c) {
                packed_out[18 * k + c] = solver.packed_coefficient_basis.data(k, c);
            }
        }
        return static_cast<long long>(points);
    });
}

}  // extern "C"

// ---- focused-transport coefficient precompute on the library grid ----------
extern "C" {

// FocusCoefficient::make_legacy_transport_coefficient_fields_with_time_
// derivative (include/FocusCoefficient.hpp:852-993) from cell-centred B, V
// and dV/dt (3 doubles per ghosted point; dvdt NULL = zero), then the
// solver's packed basis (FocusSolver.hpp:504-585) copied to packed (27
// doubles per point).  turbulence, props and params as
// ref_lib_parker_coefficients; builder_floor = the builder's minimum |B|.
long long ref_lib_focus_coefficients(int nx, int ny, const double* x_edges, const double* y_edges,
                                     const int* periodic, const double* b_values,
                                     const double* v_values, const double* dvdt_values,
                                     int turb_mode, const double* turb,
                                     const double* turb_fields, const double* props,
                                     const double* params, double builder_floor, int ghost_mode,
                                     double* packed_out) {
    return on_lib_grid(nx, ny, x_edges, y_edges, periodic,
                       [&](const auto& grid) -> long long {
        using G = std::decay_t<decltype(grid)>;
        using solver_type = FocusSolver<G>;
        using vector_field = typename solver_type::vector_field_type;
        vector_field b(grid, "fc_b", GridCentering::CellCentered);
        vector_field v(grid, "fc_v", GridCentering::CellCentered);
        vector_field dvdt(grid, "fc_dvdt", GridCentering::CellCentered);
        const std::size_t points = b.point_count();
        for (std::size_t k = 0; k < points; ++k) {
            for (int c = 0; c < 3; ++c) {
                b.data(k, c) = b_values[3 * k + c];
                v.data(k, c) = v_values[3 * k + c];
                dvdt.data(k, c) = dvdt_values != nullptr ? dvdt_values[3 * k + c] : 0.0;
            }
        }
        const auto model = TurbulencePropertyModel::constant_code_units(turb[0], turb[1],
                                                                        turb[2], turb[3]);
        TurbulenceProperties<G> turbulence(
            grid, model,
            turb_mode == 0 ? TurbulencePropertyStorageMode::ConstantOnly
                           : TurbulencePropertyStorageMode::Field);
        if (turb_mode != 0) {
            for (std::size_t k = 0; k < points; ++k) {
                turbulence.sigma2.data(k, 0) = turb_fields[0 * points + k];
                turbulence.l2d.data(k, 0) = turb_fields[1 * points + k];
                turbulence.lslab.data(k, 0) = turb_fields[2 * points + k];
                turbulence.lc.data(k, 0) = turb_fields[3 * points + k];
            }
        }
        LegencyModel::DiffusionModelParameters parameters;
        parameters.parallel_prefactor = params[1];
        parameters.perpendicular_prefactor = params[2];
        parameters.minimum_magnetic_field_magnitude = params[4];
        parameters.minimum_solar_wind_speed = params[5];
        parameters.minimum_sigma2 = params[6];
        if (static_cast<int>(params[0]) == 1) {
            parameters.set_constant_perpendicular_parallel_ratio(params[3]);
        } else {
            parameters.perpendicular_parallel_ratio = params[3];
            parameters.use_readme_perpendicular_formula();
        }
        const auto coefficients =
            FocusCoefficient::make_legacy_transport_coefficient_fields_with_time_derivative(
                b, v, dvdt, turbulence, lib_properties(props), "fcoef", parameters,
                LegencyModel::PitchAngleScatteringParameters{}, builder_floor,
                ghost_mode == 0 ? FieldGhostFillMode::PeriodicOrClamped
                                : FieldGhostFillMode::PeriodicOnly);
        LibSystem sys(0, 1, lib_properties(props));
        solver_type solver(sys, grid, b, v, coefficients);
        for (std::size_t k = 0; k < points; ++k) {
            for (int c = 0; c < 27; ++c) {
                packed_out[27 * k + c] = solver.packed_coefficient_basis.data(k, c);
            }
        }
        return static_cast<long long>(points);
    });
}

}  // extern "C"
