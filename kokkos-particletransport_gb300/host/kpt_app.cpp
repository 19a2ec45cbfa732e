// kokkos_particle_transport_app — the reference driver's command line, frame
// loop and output files, with every particle and field operation running on
// the GPU through the libkpt C ABI.
//
// Drop-in for the reference's src/main.cpp executable: same flags and
// profiles (src/main.cpp:528-590, 2466-2590), same inputs
// (FIELD_DIR/fieldNNNNN.bin, frame start+1 needed for time interpolation),
// same outputs (summary.csv with 22 columns, run.log, 128-bin
// momentum_histogram_NNNNN.csv, v4 particles_NNNNN.bin), same overwrite guard,
// restart and walltime behaviour, exit code 0, or 1 with "Error: <msg>".
// Extensions (stated in --help): --precision, --kperp-over-kpara,
// --inject-y-band, --histogram-bins, --device, --frame-prefetch, --sort-tile.
#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cctype>
#include <cstdint>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <future>
#include <iomanip>
#include <iostream>
#include <limits>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <string_view>
#include <vector>

#include "kpt.h"

namespace {

enum class Transport { Parker, Focused };

struct RunSettings {
    std::string profile_name{"particle-64000"};
    std::string field_dir{"cmake-build-debug/field_fortran_check"};
    std::string output_dir{"cmake-build-debug/reconnection_particle_64000"};
    std::string restart_path{};
    Transport transport{Transport::Parker};
    int start_frame{0};
    int end_frame{2};
    std::uint64_t particles_per_frame{64000};
    std::uint64_t rank_scale{1};
    std::uint64_t capacity{1000000};
    std::uint64_t seed{114514};
    int diagnostic_interval{1};
    int histogram_interval{1};
    int snapshot_interval{1};
    int max_steps{200000};
    bool split{true};
    bool time_interpolation{true};
    bool overwrite{false};
    double walltime_limit{0.0};
    double walltime_reserve{0.0};
    // physics block
    double mhd_dt{0.1};
    double p0{0.1};
    double pmin{1.0e-2};
    double pmax{1.0e1};
    double gamma_turb{1.6666667};
    double kpara0{0.00743592};
    double kperp_over_kpara{0.01};
    double dt_min_rel{1.0e-7};
    double dt_max_rel{1.0e-2};
    double drift1{850964.408};
    double drift2{13575468.975};
    double charge{-1.0};
    double particle_v0{17.20195};
    double duu0{5578.445};
    double split_ratio{2.0};
    double pmin_split_over_p0{2.0};
    double mu_max{0.99};
    // extensions
    int precision{KPT_PRECISION_F64};
    double band_lo{0.0};
    double band_hi{0.0};
    int histogram_bins{128};
    bool prefetch{true};  // read the next frame file while the GPU pushes
    int sort_tile{8};     // cell-sort tile before each push (cells), 0 = storage order
    int device{0};
    std::string push_stats_path{};  // per-frame push counters and diagnostic times
    int fp64_arithmetic{KPT_FP64_STRICT};

    int intervals() const { return end_frame - start_frame; }
    bool restart() const { return !restart_path.empty(); }
    bool walltime_enabled() const { return walltime_limit > 0.0; }
    double walltime_stop() const { return std::max(0.0, walltime_limit - walltime_reserve); }

    // Reconnection2DSettings::validate (src/main.cpp:187-240).
    void validate() const {
        if (end_frame <= start_frame) {
            throw std::runtime_error("Reconnection2DSettings: end frame must exceed start frame.");
        }
        if (start_frame < 0) {
            throw std::runtime_error("Reconnection2DSettings: start frame must be non-negative.");
        }
        if (restart() && !std::filesystem::exists(restart_path)) {
            throw std::runtime_error(
                "Reconnection2DSettings: restart particle snapshot does not exist.");
        }
        if (restart() && overwrite) {
            throw std::runtime_error(
                "Reconnection2DSettings: --overwrite-output cannot be combined with restart.");
        }
        if (particles_per_frame == 0 || rank_scale == 0 || capacity == 0) {
            throw std::runtime_error(
                "Reconnection2DSettings: particle counts and capacity must be positive.");
        }
        if (diagnostic_interval <= 0 || snapshot_interval < 0 || max_steps <= 0) {
            throw std::runtime_error(
                "Reconnection2DSettings: diagnostic interval and step guard must be "
                "positive, and particle snapshot interval must be non-negative.");
        }
        if (!std::isfinite(walltime_limit) || walltime_limit < 0.0 ||
            !std::isfinite(walltime_reserve) || walltime_reserve < 0.0 ||
            (walltime_limit <= 0.0 && walltime_reserve > 0.0)) {
            throw std::runtime_error(
                "Reconnection2DSettings: walltime limit must be non-negative, "
                "and reserve requires a positive walltime limit.");
        }
        kpt_settings s = physics();
        (void)s;
        const bool ok =
            std::isfinite(mhd_dt) && mhd_dt > 0.0 && std::isfinite(p0) && p0 > 0.0 &&
            std::isfinite(pmin) && pmin > 0.0 && std::isfinite(pmax) && pmax > pmin &&
            std::isfinite(gamma_turb) && std::isfinite(kpara0) && kpara0 > 0.0 &&
            std::isfinite(kperp_over_kpara) && kperp_over_kpara >= 0.0 &&
            std::isfinite(dt_min_rel) && dt_min_rel > 0.0 && std::isfinite(dt_max_rel) &&
            dt_max_rel >= dt_min_rel && std::isfinite(drift1) && std::isfinite(drift2) &&
            std::isfinite(charge) && charge != 0.0 && std::isfinite(particle_v0) &&
            particle_v0 > 0.0 && std::isfinite(duu0) && duu0 >= 0.0 &&
            std::isfinite(split_ratio) && split_ratio > 1.0 &&
            std::isfinite(pmin_split_over_p0) && pmin_split_over_p0 > 0.0 &&
            std::isfinite(mu_max) && mu_max > 0.0;
        if (!ok) {
            throw std::runtime_error("Reconnection2DSettings: invalid physical parameters.");
        }
        if (histogram_bins <= 0 || histogram_bins > 4096) {
            throw std::runtime_error("--histogram-bins must be in [1, 4096].");
        }
    }

    kpt_settings physics() const {
        kpt_settings s;
        kpt_default_settings(&s);
        s.mhd_dt = mhd_dt;
        s.p0 = p0;
        s.pmin = pmin;
        s.pmax = pmax;
        s.gamma_turb = gamma_turb;
        s.kpara0 = kpara0;
        s.kperp_over_kpara = kperp_over_kpara;
        s.dt_min_rel = dt_min_rel;
        s.dt_max_rel = dt_max_rel;
        s.drift_param1 = drift1;
        s.drift_param2 = drift2;
        s.charge = charge;
        s.particle_v0 = particle_v0;
        s.duu0 = duu0;
        s.split_ratio = split_ratio;
        s.pmin_split_over_p0 = pmin_split_over_p0;
        s.mu_max = mu_max;
        s.max_steps = max_steps;
        s.momentum_dependency = 1;
        s.magnetic_dependency = 1;
        s.time_interpolation = time_interpolation ? 1 : 0;
        s.split_particles = split ? 1 : 0;
        s.focused = transport == Transport::Focused ? 1 : 0;
        return s;
    }
};

void check(int rc) {
    if (rc != KPT_OK) {
        throw std::runtime_error(kpt_last_error());
    }
}

std::string frame_file(const std::string& dir, const char* prefix, int frame,
                       const char* suffix) {
    std::ostringstream path;
    path << dir << "/" << prefix << std::setw(5) << std::setfill('0') << frame << suffix;
    return path.str();
}

std::string field_path(const std::string& dir, int frame) {
    return frame_file(dir, "field", frame, ".bin");
}

std::string snapshot_path(const std::string& dir, int frame) {
    return frame_file(dir, "particles_", frame, ".bin");
}

bool ends_with(const std::string& s, std::string_view suffix) {
    return s.size() >= suffix.size() &&
           s.compare(s.size() - suffix.size(), suffix.size(), suffix) == 0;
}

bool starts_with(const std::string& s, std::string_view prefix) {
    return s.size() >= prefix.size() && s.compare(0, prefix.size(), prefix) == 0;
}

// Output artifacts guarded against overwrite (src/main.cpp:434-486).
bool is_output_artifact(const std::string& name) {
    if (name == "summary.csv" || name == "run.log") {
        return true;
    }
    return (name.size() > 14 && starts_with(name, "particles_") && ends_with(name, ".bin")) ||
           (name.size() > 23 && starts_with(name, "momentum_histogram_") &&
            ends_with(name, ".csv"));
}

void require_fresh_output(const RunSettings& s) {
    if (s.restart() || s.overwrite) {
        return;
    }
    const std::filesystem::path dir(s.output_dir);
    if (!std::filesystem::exists(dir)) {
        return;
    }
    if (!std::filesystem::is_directory(dir)) {
        throw std::runtime_error("Reconnection output path exists but is not a directory.");
    }
    for (const auto& entry : std::filesystem::directory_iterator(dir)) {
        if (is_output_artifact(entry.path().filename().string())) {
            throw std::runtime_error(
                "Output directory already contains reconnection solver outputs. "
                "Use --restart-particle-snapshot to continue a completed-frame "
                "snapshot, choose a new --output-dir, or pass --overwrite-output "
                "to replace the existing run.");
        }
    }
}

int infer_snapshot_frame(const std::string& path) {
    const std::string name = std::filesystem::path(path).filename().string();
    if (name.size() <= 14 || !starts_with(name, "particles_") || !ends_with(name, ".bin")) {
        return -1;
    }
    const std::string digits = name.substr(10, name.size() - 14);
    if (digits.empty() || !std::all_of(digits.begin(), digits.end(),
                                       [](unsigned char c) { return std::isdigit(c) != 0; })) {
        return -1;
    }
    return std::stoi(digits);
}

std::string default_field_dir() {
    const std::string check_dir{"cmake-build-debug/field_fortran_check"};
    if (std::filesystem::exists(field_path(check_dir, 0)) &&
        std::filesystem::exists(field_path(check_dir, 2))) {
        return check_dir;
    }
    return "cmake-build-debug/field";
}

// Named profiles (src/main.cpp:528-590).
void apply_profile(RunSettings& s, const std::string& name) {
    s = RunSettings{};
    s.profile_name = name;
    if (name == "particle-64000" || name == "particle-test") {
        s.field_dir = default_field_dir();
        s.output_dir = "cmake-build-debug/reconnection_particle_64000";
        s.start_frame = 0;
        s.end_frame = 2;
        s.particles_per_frame = 64000;
        s.capacity = 1000000;
        return;
    }
    if (name == "smoke") {
        s.field_dir = default_field_dir();
        s.output_dir = "cmake-build-debug/reconnection_smoke";
        s.start_frame = 0;
        s.end_frame = 1;
        s.particles_per_frame = 1024;
        s.capacity = 8192;
        return;
    }
    if (name == "fortran-rank") {
        s.field_dir = "cmake-build-debug/field";
        s.output_dir = "cmake-build-debug/reconnection_fortran_rank";
        s.end_frame = 200;
        s.particles_per_frame = 1600;
        s.capacity = 1000000;
        s.histogram_interval = 10;
        s.snapshot_interval = 10;
        return;
    }
    if (name == "fortran-global" || name == "full") {
        s.field_dir = "cmake-build-debug/field";
        s.output_dir = "cmake-build-debug/reconnection_fortran_global";
        s.end_frame = 200;
        s.particles_per_frame = 1600;
        s.rank_scale = 16;
        s.capacity = 16000000;
        s.histogram_interval = 10;
        s.snapshot_interval = 10;
        return;
    }
    throw std::runtime_error("Unknown run profile: " + name + ".");
}

Transport parse_transport(std::string name) {
    std::transform(name.begin(), name.end(), name.begin(),
                   [](unsigned char c) { return static_cast<char>(std::tolower(c)); });
    if (name == "parker" || name == "pte") {
        return Transport::Parker;
    }
    if (name == "focused" || name == "focus" || name == "fte") {
        return Transport::Focused;
    }
    throw std::runtime_error("Unknown transport model: " + name + ".");
}

void print_usage() {
    std::cout
        << "Usage: kokkos_particle_transport_app [options]\n"
        << "  --profile NAME                particle-64000(default), smoke, fortran-rank,\n"
        << "                                fortran-global, or full\n"
        << "  --transport MODEL             parker(default) or focused\n"
        << "  --focused-transport           shorthand for --transport focused\n"
        << "  --parker-transport            shorthand for --transport parker\n"
        << "  --restart-particle-snapshot PATH\n"
        << "                                load particles_XXXXX.bin and continue from frame XXXXX\n"
        << "  --overwrite-output           allow a fresh non-restart run to replace existing outputs\n"
        << "  --field-dir PATH              override profile field directory\n"
        << "  --output-dir PATH             override profile output directory\n"
        << "  --start-frame N               default 0\n"
        << "  --end-frame N                 reads through this frame\n"
        << "  --frames N                    sets end-frame = start-frame + N\n"
        << "  --particles-per-frame N       override profile particle injection count\n"
        << "  --rank-scale N                multiply particles per frame\n"
        << "  --capacity N                  override profile particle capacity\n"
        << "  --seed N                      default 114514\n"
        << "  --dt-out X                    default 0.1\n"
        << "  --diagnostic-interval N       profile default is usually 1\n"
        << "  --histogram-interval N        0 writes final histogram only\n"
        << "  --particle-snapshot-interval N\n"
        << "                                0 disables particle binary snapshots\n"
        << "  --max-steps-per-interval N    default 200000\n"
        << "  --walltime-hours X            stop after X hours, disabled at 0\n"
        << "  --walltime-seconds X          stop after X seconds, disabled at 0\n"
        << "  --walltime-reserve-minutes X  subtract X minutes from the stop limit\n"
        << "  --walltime-reserve-seconds X  subtract X seconds from the stop limit\n"
        << "  --particle-v0 X               focused initial speed at p0\n"
        << "  --duu0 X                      focused D_mumu normalization\n"
        << "  --split-ratio X               split threshold ratio between split levels\n"
        << "  --pmin-split-over-p0 X        first split threshold divided by p0\n"
        << "  --no-split                    disable Fortran-style particle splitting\n"
        << "  --no-time-interp              use the lower MHD frame only\n"
        << "GB300 extensions:\n"
        << "  --precision f64|mixed         push arithmetic (default f64)\n"
        << "  --kperp-over-kpara X          perpendicular/parallel diffusion ratio (default 0.01)\n"
        << "  --inject-y-band LO HI         inject y uniformly in [LO, HI) instead of the domain\n"
        << "  --frame-prefetch on|off       read the next field file during the push (default on)\n"
        << "  --histogram-bins N            momentum histogram bins (default 128)\n"
        << "  --sort-tile N                 visit particles by N x N-cell tiles in each push\n"
        << "                                (cache locality; results unchanged; default 8,\n"
        << "                                0 = storage order)\n"
        << "  --device N                    CUDA device (default 0)\n"
        << "  --push-stats PATH             write per-frame substep counts and diagnostic\n"
        << "                                times to PATH (CSV)\n"
        << "  --fp64-arithmetic strict|contracted\n"
        << "                                FP64 push rounding: as written, bit for bit with\n"
        << "                                the reference (default), or FMA-fused and faster\n";
}

std::string next_value(int argc, char** argv, int& i, const std::string& option) {
    if (i + 1 >= argc) {
        throw std::runtime_error("Missing value for " + option + ".");
    }
    return argv[++i];
}

// parse_settings (src/main.cpp:2448-2611).
RunSettings parse(int argc, char** argv) {
    RunSettings s;
    std::string profile = s.profile_name;
    bool start_set = false;
    int frame_count = -1;
    for (int i = 1; i < argc; ++i) {
        if (std::string(argv[i]) == "--profile") {
            if (i + 1 >= argc) {
                throw std::runtime_error("Missing value for --profile.");
            }
            profile = argv[++i];
        }
    }
    apply_profile(s, profile);
    for (int i = 1; i < argc; ++i) {
        const std::string arg(argv[i]);
        if (arg == "--help" || arg == "-h") {
            print_usage();
            std::exit(0);
        } else if (arg == "--profile") {
            (void)next_value(argc, argv, i, arg);
        } else if (arg == "--transport") {
            s.transport = parse_transport(next_value(argc, argv, i, arg));
        } else if (arg == "--focused-transport") {
            s.transport = Transport::Focused;
        } else if (arg == "--parker-transport") {
            s.transport = Transport::Parker;
        } else if (arg == "--restart-particle-snapshot") {
            s.restart_path = next_value(argc, argv, i, arg);
        } else if (arg == "--overwrite-output") {
            s.overwrite = true;
        } else if (arg == "--field-dir") {
            s.field_dir = next_value(argc, argv, i, arg);
        } else if (arg == "--output-dir") {
            s.output_dir = next_value(argc, argv, i, arg);
        } else if (arg == "--start-frame") {
            s.start_frame = std::stoi(next_value(argc, argv, i, arg));
            start_set = true;
            if (frame_count > 0) {
                s.end_frame = s.start_frame + frame_count;
            }
        } else if (arg == "--end-frame") {
            s.end_frame = std::stoi(next_value(argc, argv, i, arg));
        } else if (arg == "--frames") {
            frame_count = std::stoi(next_value(argc, argv, i, arg));
            s.end_frame = s.start_frame + frame_count;
        } else if (arg == "--particles-per-frame") {
            s.particles_per_frame = std::stoull(next_value(argc, argv, i, arg));
        } else if (arg == "--rank-scale") {
            s.rank_scale = std::stoull(next_value(argc, argv, i, arg));
        } else if (arg == "--capacity") {
            s.capacity = std::stoull(next_value(argc, argv, i, arg));
        } else if (arg == "--seed") {
            s.seed = std::stoull(next_value(argc, argv, i, arg));
        } else if (arg == "--dt-out") {
            s.mhd_dt = std::stod(next_value(argc, argv, i, arg));
        } else if (arg == "--diagnostic-interval") {
            s.diagnostic_interval = std::stoi(next_value(argc, argv, i, arg));
        } else if (arg == "--histogram-interval") {
            s.histogram_interval = std::stoi(next_value(argc, argv, i, arg));
        } else if (arg == "--particle-snapshot-interval") {
            s.snapshot_interval = std::stoi(next_value(argc, argv, i, arg));
        } else if (arg == "--max-steps-per-interval") {
            s.max_steps = std::stoi(next_value(argc, argv, i, arg));
        } else if (arg == "--walltime-hours") {
            s.walltime_limit = 3600.0 * std::stod(next_value(argc, argv, i, arg));
        } else if (arg == "--walltime-seconds") {
            s.walltime_limit = std::stod(next_value(argc, argv, i, arg));
        } else if (arg == "--walltime-reserve-minutes") {
            s.walltime_reserve = 60.0 * std::stod(next_value(argc, argv, i, arg));
        } else if (arg == "--walltime-reserve-seconds") {
            s.walltime_reserve = std::stod(next_value(argc, argv, i, arg));
        } else if (arg == "--particle-v0") {
            s.particle_v0 = std::stod(next_value(argc, argv, i, arg));
        } else if (arg == "--duu0") {
            s.duu0 = std::stod(next_value(argc, argv, i, arg));
        } else if (arg == "--split-ratio") {
            s.split_ratio = std::stod(next_value(argc, argv, i, arg));
        } else if (arg == "--pmin-split-over-p0") {
            s.pmin_split_over_p0 = std::stod(next_value(argc, argv, i, arg));
        } else if (arg == "--no-split") {
            s.split = false;
        } else if (arg == "--no-time-interp") {
            s.time_interpolation = false;
        } else if (arg == "--precision") {
            const std::string v = next_value(argc, argv, i, arg);
            if (v == "f64") {
                s.precision = KPT_PRECISION_F64;
            } else if (v == "mixed") {
                s.precision = KPT_PRECISION_MIXED;
            } else {
                throw std::runtime_error("Unknown precision: " + v + ".");
            }
        } else if (arg == "--kperp-over-kpara") {
            s.kperp_over_kpara = std::stod(next_value(argc, argv, i, arg));
        } else if (arg == "--inject-y-band") {
            s.band_lo = std::stod(next_value(argc, argv, i, arg));
            s.band_hi = std::stod(next_value(argc, argv, i, arg));
            if (!(s.band_lo < s.band_hi)) {
                throw std::runtime_error("--inject-y-band needs LO < HI.");
            }
        } else if (arg == "--histogram-bins") {
            s.histogram_bins = std::stoi(next_value(argc, argv, i, arg));
        } else if (arg == "--device") {
            s.device = std::stoi(next_value(argc, argv, i, arg));
        } else if (arg == "--frame-prefetch") {
            const std::string v = next_value(argc, argv, i, arg);
            if (v != "on" && v != "off") {
                throw std::runtime_error("--frame-prefetch needs on or off.");
            }
            s.prefetch = v == "on";
        } else if (arg == "--sort-tile") {
            s.sort_tile = std::stoi(next_value(argc, argv, i, arg));
            if (s.sort_tile < 0 || s.sort_tile > 4096) {
                throw std::runtime_error("--sort-tile must be in [0, 4096].");
            }
        } else if (arg == "--push-stats") {
            s.push_stats_path = next_value(argc, argv, i, arg);
        } else if (arg == "--fp64-arithmetic") {
            const std::string v = next_value(argc, argv, i, arg);
            if (v != "strict" && v != "contracted") {
                throw std::runtime_error("--fp64-arithmetic needs strict or contracted.");
            }
            s.fp64_arithmetic = v == "strict" ? KPT_FP64_STRICT : KPT_FP64_CONTRACTED;
        } else {
            throw std::runtime_error("Unknown option: " + arg);
        }
    }
    if (s.restart()) {
        const int frame = infer_snapshot_frame(s.restart_path);
        if (frame < 0) {
            throw std::runtime_error(
                "Cannot infer restart frame from particle snapshot name; expected "
                "particles_XXXXX.bin.");
        }
        if (start_set && s.start_frame != frame) {
            throw std::runtime_error(
                "Restart particle snapshot frame does not match --start-frame.");
        }
        if (!start_set) {
            s.start_frame = frame;
            if (frame_count > 0) {
                s.end_frame = s.start_frame + frame_count;
            }
        }
    }
    s.validate();
    return s;
}

using Clock = std::chrono::steady_clock;

double seconds_since(Clock::time_point start) {
    return std::chrono::duration<double>(Clock::now() - start).count();
}

void log_block(std::ofstream& log, const std::string& block) {
    std::cout << block;
    if (log) {
        log << block;
        log.flush();
    }
}

void log_line(std::ofstream& log, const std::string& line) { log_block(log, line + '\n'); }

struct HostParticles {
    std::vector<double> x, y, p, t, dt, w, mu;
    std::vector<int32_t> status, level;
    void resize(std::size_t n) {
        for (auto* v : {&x, &y, &p, &t, &dt, &w, &mu}) {
            v->assign(n, 0.0);
        }
        status.assign(n, 2);
        level.assign(n, 0);
    }
};

template <typename T>
void put(std::ofstream& stream, const T& value) {
    stream.write(reinterpret_cast<const char*>(&value), sizeof(T));
    if (!stream) {
        throw std::runtime_error("Failed to write particle binary scalar.");
    }
}

template <typename T>
T get(std::ifstream& stream) {
    T value{};
    stream.read(reinterpret_cast<char*>(&value), sizeof(T));
    if (!stream) {
        throw std::runtime_error("Failed to read particle binary scalar.");
    }
    return value;
}

bool metadata_matches(double actual, double expected) {
    if (!std::isfinite(actual) || !std::isfinite(expected)) {
        return false;
    }
    const double scale = std::max({1.0, std::abs(actual), std::abs(expected)});
    return std::abs(actual - expected) <= 1.0e-12 * scale;
}

// v4 snapshot reader for restart (src/main.cpp:2010-2126).
std::uint64_t load_snapshot(const RunSettings& s, int restart_frame, kpt_particles* parts) {
    std::ifstream stream(s.restart_path, std::ios::binary);
    if (!stream) {
        throw std::runtime_error("Failed to open restart particle snapshot.");
    }
    std::array<char, 8> magic{};
    stream.read(magic.data(), 8);
    const std::array<char, 8> expected{'K', 'P', 'T', 'P', 'R', 'T', '\0', '\0'};
    if (!stream || magic != expected) {
        throw std::runtime_error("Restart particle snapshot is not a repository KPTPRT file.");
    }
    const auto version = get<std::uint32_t>(stream);
    const auto endian = get<std::uint32_t>(stream);
    if (version != 4u) {
        throw std::runtime_error("Restart particle snapshot must use particle binary version 4.");
    }
    if (endian != 0x01020304u) {
        throw std::runtime_error("Restart particle snapshot endian does not match this host.");
    }
    const auto dim = get<std::int32_t>(stream);
    (void)get<std::int32_t>(stream);
    const auto count = get<std::uint64_t>(stream);
    const auto snap_capacity = get<std::uint64_t>(stream);
    (void)get<double>(stream);
    const double charge = get<double>(stream);
    (void)get<double>(stream);
    (void)get<double>(stream);
    const double split_ratio = get<double>(stream);
    (void)get<double>(stream);
    if (dim != 2) {
        throw std::runtime_error(
            "Restart particle snapshot dimensionality does not match reconnection storage.");
    }
    if (count > s.capacity) {
        std::ostringstream message;
        message << "Restart particle snapshot stores " << count
                << " particles, but configured capacity is " << s.capacity
                << ". Snapshot capacity was " << snap_capacity << '.';
        throw std::runtime_error(message.str());
    }
    if (!metadata_matches(charge, s.charge)) {
        throw std::runtime_error("Restart particle snapshot charge does not match current settings.");
    }
    if (!metadata_matches(split_ratio, s.split_ratio)) {
        throw std::runtime_error(
            "Restart particle snapshot split ratio does not match current settings.");
    }
    HostParticles h;
    h.resize(count);
    const double restart_time = static_cast<double>(restart_frame) * s.mhd_dt;
    for (std::uint64_t i = 0; i < count; ++i) {
        (void)get<std::uint64_t>(stream);
        h.status[i] = get<std::int32_t>(stream);
        h.level[i] = get<std::int32_t>(stream);
        (void)get<std::int32_t>(stream);
        h.x[i] = get<double>(stream);
        h.y[i] = get<double>(stream);
        for (int k = 0; k < 4; ++k) {
            (void)get<double>(stream);
        }
        h.p[i] = get<double>(stream);
        h.mu[i] = get<double>(stream);
        h.w[i] = get<double>(stream);
        (void)get<double>(stream);
        h.t[i] = restart_time;
        h.dt[i] = s.dt_min_rel * s.mhd_dt;
    }
    check(kpt_particles_upload(parts, count, h.x.data(), h.y.data(), h.p.data(), h.t.data(),
                               h.dt.data(), h.w.data(), h.mu.data(), h.status.data(),
                               h.level.data()));
    return count;
}

// v4 snapshot writer (src/main.cpp:2132-2202).
// Snapshot writer: the records are packed on the GPU into a page-locked
// buffer (one copy), and the file is written on a second host thread while
// the next frame is pushed.  The file is opened on the calling thread, so an
// unwritable path fails at once; a later write error is reported when the
// next snapshot starts or the run ends.
class SnapshotWriter {
public:
    ~SnapshotWriter() {
        if (pending_.valid()) pending_.wait();
        kpt_host_free(buffer_);
    }

    void finish() {
        if (pending_.valid()) pending_.get();
    }

    void write(const RunSettings& s, kpt_context* ctx, kpt_particles* parts, int frame) {
        finish();
        std::uint64_t count = 0, capacity = 0;
        check(kpt_particles_count(parts, &count, &capacity));
        const std::string path = snapshot_path(s.output_dir, frame);
        auto stream = std::make_shared<std::ofstream>(path, std::ios::binary);
        if (!*stream) {
            throw std::runtime_error("Failed to open particle snapshot output.");
        }
        std::vector<char> header;
        auto put_bytes = [&header](const auto& value) {
            const char* b = reinterpret_cast<const char*>(&value);
            header.insert(header.end(), b, b + sizeof(value));
        };
        const char magic[8] = {'K', 'P', 'T', 'P', 'R', 'T', '\0', '\0'};
        header.insert(header.end(), magic, magic + 8);
        put_bytes(std::uint32_t{4});
        put_bytes(std::uint32_t{0x01020304u});
        put_bytes(std::int32_t{2});
        put_bytes(std::int32_t{3});
        put_bytes(count);
        put_bytes(capacity);
        put_bytes(1.0);
        put_bytes(s.charge);
        put_bytes(1.0);
        put_bytes(1.0);
        put_bytes(s.split_ratio);
        put_bytes(0.0);
        const double e0 = std::sqrt(1.0 + s.p0 * s.p0) - 1.0;
        const std::uint64_t bytes = count * 100;
        if (bytes > size_) {
            kpt_host_free(buffer_);
            buffer_ = nullptr;
            size_ = 0;
            check(kpt_host_alloc(bytes, &buffer_));
            size_ = bytes;
        }
        if (bytes > 0) {
            check(kpt_particles_pack_records(ctx, parts, e0, buffer_, size_));
        }
        const char* records = static_cast<const char*>(buffer_);
        pending_ = std::async(std::launch::async, [stream, header, records, bytes]() {
            stream->write(header.data(), static_cast<std::streamsize>(header.size()));
            if (bytes > 0) {
                stream->write(records, static_cast<std::streamsize>(bytes));
            }
            stream->flush();
            if (!*stream) {
                throw std::runtime_error("Failed to write particle binary scalar.");
            }
        });
    }

private:
    void* buffer_ = nullptr;
    std::uint64_t size_ = 0;
    std::future<void> pending_;
};

// Histogram CSV (src/main.cpp:1942-1963).  Bin edges are formed as
// fma(bin, dlogp, log(pmin)), the contracted form the reference's optimised
// build produces (its tracked 128-bin example output matches it).
void write_histogram(const RunSettings& s, kpt_context* ctx, kpt_particles* parts, int frame) {
    std::vector<double> bins(static_cast<std::size_t>(s.histogram_bins), 0.0);
    check(kpt_histogram(ctx, parts, s.pmin, s.pmax, s.histogram_bins, bins.data()));
    std::ofstream stream(frame_file(s.output_dir, "momentum_histogram_", frame, ".csv"));
    if (!stream) {
        throw std::runtime_error("Failed to open momentum histogram output.");
    }
    stream << "bin,p_left,p_right,weight\n";
    const double log_pmin = std::log(s.pmin);
    const double dlogp = (std::log(s.pmax) - log_pmin) / static_cast<double>(s.histogram_bins);
    for (int b = 0; b < s.histogram_bins; ++b) {
        const double left = std::exp(std::fma(static_cast<double>(b), dlogp, log_pmin));
        const double right = std::exp(std::fma(static_cast<double>(b + 1), dlogp, log_pmin));
        stream << b << ',' << std::setprecision(16) << left << ',' << right << ','
               << bins[static_cast<std::size_t>(b)] << '\n';
    }
}

struct FrameTiming {
    double read_s{0.0}, inject_s{0.0}, move_s{0.0}, split_s{0.0};
    double summary_s{0.0}, histogram_s{0.0};
    std::uint64_t injected{0}, split{0}, skipped{0};
};

void write_summary_row(std::ofstream& stream, int frame, double time, const kpt_summary& sum,
                       const FrameTiming& timing, double frame_s, double elapsed_s) {
    stream << frame << ',' << std::setprecision(16) << time << ',' << sum.stored << ','
           << sum.active << ',' << sum.inactive << ',' << sum.weight_sum << ',' << sum.p_min
           << ',' << sum.p_max << ',' << sum.p_avg << ',' << sum.dt_min << ',' << sum.dt_max
           << ',' << sum.dt_avg << ',' << sum.max_split_level << ',' << timing.injected << ','
           << timing.split << ',' << timing.skipped << ',' << timing.read_s << ','
           << timing.inject_s << ',' << timing.move_s << ',' << timing.split_s << ','
           << frame_s << ',' << elapsed_s << '\n';
}

struct FieldDeleter {
    void operator()(kpt_field* f) const { kpt_field_destroy(f); }
};
using FieldPtr = std::unique_ptr<kpt_field, FieldDeleter>;

FieldPtr load_frame(kpt_context* ctx, const RunSettings& s, int frame) {
    kpt_field* f = nullptr;
    const int kind = s.transport == Transport::Focused ? KPT_TABLE_FOCUSED21 : KPT_TABLE_PARKER16;
    check(kpt_field_load(ctx, field_path(s.field_dir, frame).c_str(), kind, s.precision, &f));
    return FieldPtr(f);
}

struct FieldDataDeleter {
    void operator()(kpt_field_data* d) const { kpt_field_data_free(d); }
};
using FieldDataPtr = std::unique_ptr<kpt_field_data, FieldDataDeleter>;

// Frame prefetch: the compact file of a later frame is read into page-locked
// host memory on a second host thread while the GPU pushes the current
// frame; the table is built from it when the frame is needed.  A read error
// is reported when that frame is needed, as the serial reader would.
std::future<FieldDataPtr> prefetch_frame(const kpt_context* ctx, const RunSettings& s,
                                         int frame) {
    const std::string path = field_path(s.field_dir, frame);
    return std::async(std::launch::async, [ctx, path]() {
        kpt_field_data* d = nullptr;
        check(kpt_field_data_read(ctx, path.c_str(), &d));
        return FieldDataPtr(d);
    });
}

FieldPtr build_frame(kpt_context* ctx, const RunSettings& s, const FieldDataPtr& data) {
    kpt_field* f = nullptr;
    const int kind = s.transport == Transport::Focused ? KPT_TABLE_FOCUSED21 : KPT_TABLE_PARKER16;
    check(kpt_field_create_from_data(ctx, data.get(), kind, s.precision, &f));
    return FieldPtr(f);
}

// run + run_transport_loop (src/main.cpp:2255-2429, 2616-2688).
int run(const RunSettings& s) {
    require_fresh_output(s);
    std::filesystem::create_directories(s.output_dir);
    const std::string summary_path = s.output_dir + "/summary.csv";
    const std::string log_path = s.output_dir + "/run.log";
    const bool append = s.restart() && std::filesystem::exists(summary_path);
    const bool has_content = append && std::filesystem::file_size(summary_path) > 0;
    std::ofstream summary(summary_path, append ? (std::ios::out | std::ios::app) : std::ios::out);
    if (!summary) {
        throw std::runtime_error("Failed to open summary output.");
    }
    if (!has_content) {
        summary << "frame,time,stored,active,inactive,weight_sum,p_min,p_max,p_avg,"
                   "dt_min,dt_max,dt_avg,max_split_level,injected,split,"
                   "skipped_split_capacity,read_seconds,inject_seconds,move_seconds,"
                   "split_seconds,total_frame_seconds,total_elapsed_seconds\n";
    }
    std::ofstream log(log_path, s.restart() ? (std::ios::out | std::ios::app) : std::ios::out);
    if (!log) {
        throw std::runtime_error("Failed to open run log output.");
    }
    std::ofstream push_stats;
    if (!s.push_stats_path.empty()) {
        push_stats.open(s.push_stats_path, std::ios::out);
        if (!push_stats) {
            throw std::runtime_error("Failed to open push stats output.");
        }
        push_stats << "frame,stored,pushed,particle_steps,failed,max_steps,read_seconds,"
                      "inject_seconds,move_seconds,split_seconds,summary_seconds,"
                      "histogram_seconds\n";
    }
    const std::uint64_t seed =
        s.restart() ? s.seed + 0x9e3779b97f4a7c15ull * static_cast<std::uint64_t>(s.start_frame + 1)
                    : s.seed;
    kpt_context* raw_ctx = nullptr;
    check(kpt_context_create(s.device, &raw_ctx));
    std::unique_ptr<kpt_context, int (*)(kpt_context*)> ctx(raw_ctx, kpt_context_destroy);
    check(kpt_context_set_fp64_arithmetic(ctx.get(), s.fp64_arithmetic));
    kpt_particles* raw_parts = nullptr;
    check(kpt_particles_create(ctx.get(), s.capacity, &raw_parts));
    std::unique_ptr<kpt_particles, int (*)(kpt_particles*)> parts(raw_parts,
                                                                   kpt_particles_destroy);
    if (s.restart()) {
        const std::uint64_t loaded = load_snapshot(s, s.start_frame, parts.get());
        std::ostringstream msg;
        msg << "Restarted from particle snapshot " << s.restart_path << " at frame "
            << s.start_frame << " loaded_particles=" << loaded
            << " configured_capacity=" << s.capacity << " effective_seed=" << seed
            << " (RNG state is reseeded, not restored)";
        log_line(log, msg.str());
    }
    const kpt_settings physics = s.physics();
    auto read_start = Clock::now();
    FieldPtr lower = load_frame(ctx.get(), s, s.start_frame);
    FieldPtr upper = load_frame(ctx.get(), s, s.start_frame + 1);
    const double initial_read = seconds_since(read_start);

    std::ostringstream header;
    header << "Reconnection 2D calibration\n"
           << "  profile=" << s.profile_name << '\n'
           << "  transport=" << (s.transport == Transport::Focused ? "focused" : "parker") << '\n'
           << "  field_dir=" << s.field_dir << '\n'
           << "  output_dir=" << s.output_dir << '\n'
           << "  restart_particle_snapshot="
           << (s.restart() ? s.restart_path : std::string("disabled")) << '\n'
           << "  overwrite_output=" << (s.overwrite ? "enabled" : "disabled") << '\n'
           << "  frames=" << s.start_frame << ".." << s.end_frame << " (" << s.intervals()
           << " intervals)\n"
           << "  particles_per_frame=" << s.particles_per_frame * s.rank_scale << " ("
           << s.particles_per_frame << " * rank_scale " << s.rank_scale << ")\n"
           << "  capacity=" << s.capacity << '\n'
           << "  dt_out=" << s.mhd_dt << '\n'
           << "  histogram_interval=" << s.histogram_interval << '\n'
           << "  particle_snapshot_interval=" << s.snapshot_interval << '\n'
           << "  walltime_limit_s=";
    if (s.walltime_enabled()) {
        header << s.walltime_limit << " walltime_reserve_s=" << s.walltime_reserve
               << " walltime_stop_s=" << s.walltime_stop() << '\n';
    } else {
        header << "disabled\n";
    }
    header << "  kpara0=" << s.kpara0 << " kperp/kpara=" << s.kperp_over_kpara << '\n'
           << "  particle_v0=" << s.particle_v0 << " duu0=" << s.duu0 << '\n';
    log_block(log, header.str());

    const auto run_start = Clock::now();
    bool stopped = false;
    int last_frame = s.start_frame;
    std::future<FieldDataPtr> next_upper;
    SnapshotWriter snapshots;
    for (int frame = s.start_frame; frame < s.end_frame; ++frame) {
        const auto frame_start = Clock::now();
        FrameTiming timing;
        timing.read_s = frame == s.start_frame ? initial_read : 0.0;
        if (frame > s.start_frame) {
            lower = std::move(upper);
            const auto t0 = Clock::now();
            upper = s.prefetch ? build_frame(ctx.get(), s, next_upper.get())
                               : load_frame(ctx.get(), s, frame + 1);
            timing.read_s = seconds_since(t0);  // the part of the read not hidden by the push
        }
        if (s.prefetch && frame + 1 < s.end_frame) {
            next_upper = prefetch_frame(ctx.get(), s, frame + 2);
        }
        auto t0 = Clock::now();
        check(kpt_inject_uniform(ctx.get(), parts.get(), lower.get(), &physics,
                                 s.particles_per_frame * s.rank_scale,
                                 static_cast<std::uint32_t>(frame), seed, s.band_lo, s.band_hi,
                                 &timing.injected));
        check(kpt_context_synchronize(ctx.get()));
        timing.inject_s = seconds_since(t0);
        t0 = Clock::now();
        if (s.sort_tile > 0) {
            // work order by spatial tile; storage, ids and noise streams stay put
            check(kpt_particles_sort(ctx.get(), parts.get(), lower.get(), s.sort_tile,
                                     s.sort_tile));
        }
        kpt_push_stats push{};
        check(kpt_push_interval(ctx.get(), parts.get(), lower.get(), upper.get(), &physics,
                                static_cast<std::uint32_t>(frame), seed,
                                push_stats.is_open() ? &push : nullptr));
        check(kpt_context_synchronize(ctx.get()));
        timing.move_s = seconds_since(t0);
        t0 = Clock::now();
        check(kpt_split(ctx.get(), parts.get(), &physics, &timing.split, &timing.skipped));
        timing.split_s = seconds_since(t0);

        const double frame_s = seconds_since(frame_start);
        const double elapsed_s = seconds_since(run_start);
        const bool walltime_hit = s.walltime_enabled() && elapsed_s >= s.walltime_stop();
        const bool final_frame = frame + 1 == s.end_frame;
        const bool finishing = final_frame || walltime_hit;
        const int done = frame + 1 - s.start_frame;
        if (done % s.diagnostic_interval == 0 || finishing) {
            const auto summary_start = Clock::now();
            kpt_summary sum{};
            check(kpt_summarize(ctx.get(), parts.get(), &sum));
            timing.summary_s = seconds_since(summary_start);
            write_summary_row(summary, frame + 1, static_cast<double>(frame + 1) * s.mhd_dt, sum,
                              timing, frame_s, elapsed_s);
            summary.flush();
            std::ostringstream line;
            line << "frame " << frame + 1 << " active=" << sum.active << " stored=" << sum.stored
                 << " pmax=" << std::setprecision(6) << sum.p_max
                 << " read_s=" << timing.read_s << " inject_s=" << timing.inject_s
                 << " move_s=" << timing.move_s << " split_s=" << timing.split_s
                 << " frame_s=" << frame_s << " elapsed_s=" << elapsed_s;
            log_line(log, line.str());
        }
        if ((s.histogram_interval > 0 && done % s.histogram_interval == 0) || finishing) {
            const auto histogram_start = Clock::now();
            write_histogram(s, ctx.get(), parts.get(), frame + 1);
            timing.histogram_s = seconds_since(histogram_start);
        }
        if (push_stats.is_open()) {
            std::uint64_t stored = 0;
            check(kpt_particles_count(parts.get(), &stored, nullptr));
            push_stats << frame + 1 << ',' << stored << ',' << push.pushed << ','
                       << push.particle_steps << ',' << push.failed << ',' << push.max_steps
                       << ',' << std::setprecision(9) << timing.read_s << ',' << timing.inject_s
                       << ',' << timing.move_s << ',' << timing.split_s << ','
                       << timing.summary_s << ',' << timing.histogram_s << '\n';
            push_stats.flush();
        }
        if (s.snapshot_interval > 0 && (done % s.snapshot_interval == 0 || finishing)) {
            const auto snap_start = Clock::now();
            snapshots.write(s, ctx.get(), parts.get(), frame + 1);
            std::ostringstream line;
            line << "wrote particle snapshot " << snapshot_path(s.output_dir, frame + 1) << " in "
                 << seconds_since(snap_start) << " s";
            log_line(log, line.str());
        }
        last_frame = frame + 1;
        if (walltime_hit) {
            stopped = true;
            std::ostringstream line;
            line << "Reached walltime stop after frame " << last_frame << " elapsed_s="
                 << elapsed_s << " stop_s=" << s.walltime_stop()
                 << " limit_s=" << s.walltime_limit << " reserve_s=" << s.walltime_reserve;
            log_line(log, line.str());
            break;
        }
    }
    snapshots.finish();
    std::ostringstream footer;
    if (stopped) {
        footer << "Stopped by walltime after frame " << last_frame << " in "
               << seconds_since(run_start) << " s. Summary: " << s.output_dir << "/summary.csv\n";
    } else {
        footer << "Finished in " << seconds_since(run_start) << " s. Summary: " << s.output_dir
               << "/summary.csv\n";
    }
    log_block(log, footer.str());
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    try {
        return run(parse(argc, argv));
    } catch (const std::exception& error) {
        std::cerr << "Error: " << error.what() << '\n';
        return 1;
    }
}
