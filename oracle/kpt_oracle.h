/*
 * kpt_oracle — CPU restatement of the reference's driver push path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the CPU
 * baseline legs of bench.py may load this library, and only as the checker
 * or the timed CPU baseline; the product never links or calls it.
 *
 * Plain C99 + OpenMP, FP64, evaluation order transcribed from the reference
 * (file:line citations in kpt_oracle.c) so that, built with the same compiler
 * flags (-ffp-contract=off), its results are bit-identical to the reference's
 * own kernels compiled in oracle/_ref.
 */
#ifndef KPT_ORACLE_H
#define KPT_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Host-level run parameters (reference Reconnection2DSettings,
 * src/main.cpp:114-241).  Doubles first, then ints; mirrored by ctypes. */
typedef struct {
    double mhd_dt;
    double p0;
    double pmin;
    double pmax;
    double gamma_turb;
    double kpara0;
    double kperp_over_kpara;
    double dt_min_rel;
    double dt_max_rel;
    double drift_param1;
    double drift_param2;
    double charge;
    double particle_v0;
    double duu0;
    double split_ratio;
    double pmin_split_over_p0;
    double mu_max;
    int32_t max_steps;
    int32_t momentum_dependency;
    int32_t magnetic_dependency;
    int32_t time_interpolation;
    int32_t split_particles;
    int32_t focused;
    /* focused scattering closure: 0 driver (reference), 1 slab QLT
     * (LegencyModel.hpp:539-645) with Omega = qlt_omega0 |B| / sqrt(1+p^2),
     * v = particle_v0 p / p0 */
    int32_t closure;
    double qlt_sigma2;
    double qlt_spectral_index;
    double qlt_h0;
    double qlt_omega0;
    double qlt_lc;
} kpt_oracle_params;

/* 2D periodic grid with two ghost layers.  An axis whose edges are uniform
 * (reader tolerance, AthenaFieldReader.hpp:167-193) is analytic
 * (AnalyticCoordinateGrid.hpp:160-230); otherwise it stores its ghosted faces
 * and cell centres (StoredCoordinateGrid.hpp:130-174), ghost faces extended
 * periodically. */
typedef struct {
    int n[2];
    int stored[2];
    double start[2];
    double step[2];
    double* faces[2];   /* stored axes: n+5 faces, logical -2..n+2 */
    double* centers[2]; /* stored axes: n+4 centres, logical -2..n+1 */
    double lower[2];
    double upper[2];
    double width[2];
    double inv_width[2];
    double ghost_lower[2];
    double ghost_upper[2];
} kpt_oracle_grid;

typedef struct {
    uint64_t stored;
    uint64_t active;
    uint64_t inactive;
    double weight_sum;
    double p_min;
    double p_max;
    double p_avg;
    double dt_min;
    double dt_max;
    double dt_avg;
    int32_t max_split_level;
    int32_t pad;
} kpt_oracle_summary;

const char* kpt_oracle_last_error(void);

/* Returns 0, or -1 with kpt_oracle_last_error() set. force_stored=1 keeps
 * stored coordinates even for uniform edges. */
int kpt_oracle_grid_init(kpt_oracle_grid* grid, int nx, int ny, const double* x_edges,
                         const double* y_edges, int force_stored);
void kpt_oracle_grid_free(kpt_oracle_grid* grid);
size_t kpt_oracle_point_count(const kpt_oracle_grid* grid);

/* Copy cell data (3 x ny x nx, x fastest) into a ghosted point array
 * (points x 3) and fill ghosts periodically (Field.hpp:274-316). */
void kpt_oracle_load_vector_field(const kpt_oracle_grid* grid, const double* cells,
                                  double* ghosted);

/* Driver coefficient table: 16 Parker or 21 focused components per ghosted
 * point (src/main.cpp:840-957). */
void kpt_oracle_build_table(const kpt_oracle_grid* grid, const double* b_ghosted,
                            const double* v_ghosted, int focused, double* table);

/* Convenience: cells -> table for one frame. Returns 0 or -1. */
int kpt_oracle_table_from_cells(int nx, int ny, const double* x_edges, const double* y_edges,
                                const double* b_cells, const double* v_cells, int focused,
                                int force_stored, double* table);

/* One interval push of every active particle (src/main.cpp:1084-1327 Parker,
 * :1334-1755 focused).  steps (optional) receives each particle's executed
 * substep count.  threads <= 0 uses the OpenMP default. */
void kpt_oracle_push(const kpt_oracle_grid* grid, const double* lower_table,
                     const double* upper_table, const kpt_oracle_params* params,
                     double interval_start, uint32_t frame, uint64_t seed, size_t count,
                     double* x, double* y, double* p, double* t, double* step_dt, double* mu,
                     int32_t* status, uint32_t* steps, int threads);

/* inject_uniform_particles (src/main.cpp:996-1048).  band_lo < band_hi
 * narrows the y draw to that band.  Returns the new stored count. */
uint64_t kpt_oracle_inject(const kpt_oracle_grid* grid, const kpt_oracle_params* params,
                           double interval_start, uint32_t frame, uint64_t seed,
                           uint64_t capacity, uint64_t count, uint64_t requested,
                           double band_lo, double band_hi, double* x, double* y, double* p,
                           double* t, double* step_dt, double* weight, double* mu,
                           int32_t* status, int32_t* split_level);

/* split_particles in serial parent order (src/main.cpp:1761-1839). */
uint64_t kpt_oracle_split(const kpt_oracle_params* params, uint64_t capacity, uint64_t count,
                          double* x, double* y, double* p, double* t, double* step_dt,
                          double* weight, double* mu, int32_t* status, int32_t* split_level,
                          uint64_t* split_out, uint64_t* skipped_out);

/* write_momentum_histogram binning (src/main.cpp:1907-1964), nbins bins. */
void kpt_oracle_histogram(double pmin, double pmax, int nbins, uint64_t count, const double* p,
                          const double* weight, const int32_t* status, double* bins);

/* summarize_particles (src/main.cpp:1845-1901). */
void kpt_oracle_summarize(uint64_t count, const double* p, const double* step_dt,
                          const double* weight, const int32_t* status,
                          const int32_t* split_level, kpt_oracle_summary* out);

/* pitch_angle_diffusion_coefficient (LegencyModel.hpp:557-594). */
double kpt_oracle_qlt_dmumu(double mu, double omega, double speed, double sigma2, double lc,
                            double spectral_index, double h0);
/* pitch_angle_diffusion_derivative (LegencyModel.hpp:599-645). */
double kpt_oracle_qlt_dmumu_dmu(double mu, double dmumu, double omega, double speed, double lc,
                                double spectral_index, double h0);

/* wrap_periodic_coordinate (src/main.cpp:642-665). */
double kpt_oracle_wrap(double value, double lower, double upper, double width);

/* The project pow (kpt_pow.h) on the host, elementwise: out[i] = x[i]^y[i]. */
void kpt_oracle_pow_array(uint64_t n, const double* x, const double* y, double* out);

/* Sample a table (C components) at one particle position the way the push
 * does (src/main.cpp:1055-1077, 1142-1148). */
void kpt_oracle_sample(const kpt_oracle_grid* grid, const double* lower_table,
                       const double* upper_table, int ncomp, double x, double y, double rt,
                       int time_interpolation, double* out);

#ifdef __cplusplus
}
#endif

#endif
