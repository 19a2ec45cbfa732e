/*
 * kpt_oracle.c — CPU restatement of the reference driver's push path.
 *
 * TEST INFRASTRUCTURE ONLY (see kpt_oracle.h).  Every function cites the
 * reference file:line it restates.  Expressions keep the reference's
 * operand order so that, compiled with -ffp-contract=off, the results are
 * bit-identical to the reference kernels built in oracle/_ref.
 */
#include "kpt_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "kpt_philox.h"
/* the project pow, shared with the GPU push and the shim's Kokkos::pow */
#include "kpt_pow.h"

/* Powers: the project pow (kpt_pow.h, the one the GPU's strict FP64 push and
 * the reference build on the shim call), so the restatement's trajectories
 * equal theirs bit for bit.  Built with -DKPT_ORACLE_LIBM_POW the restatement
 * calls the C library's pow instead, as the reference's own Kokkos build
 * does: that build is the one timed as the CPU baseline (same algorithm,
 * powers within an ulp, at the C library's speed). */
#ifdef KPT_ORACLE_LIBM_POW
#define ORACLE_POW pow
#else
#define ORACLE_POW kpt_pow
#endif

static _Thread_local char g_error[256];

const char* kpt_oracle_last_error(void) { return g_error; }

static int fail(const char* message) {
    snprintf(g_error, sizeof(g_error), "%s", message);
    return -1;
}

/* ------------------------------------------------------------------ grid */

/* AthenaFieldReader.hpp:147-193: ascending, finite and (for the analytic
 * path) uniform within 1024 eps of the mean step. */
static int edges_ascending(const double* e, int n) {
    for (int i = 0; i <= n; ++i) {
        if (!isfinite(e[i])) {
            return 0;
        }
        if (i > 0 && !(e[i] > e[i - 1])) {
            return 0;
        }
    }
    return 1;
}

static int edges_uniform(const double* e, int n, double* step_out) {
    const double interval_count = (double)n;
    const double span = e[n] - e[0];
    const double step = span / interval_count;
    if (!isfinite(step) || step <= 0.0) {
        return 0;
    }
    for (int i = 1; i <= n; ++i) {
        const double current = e[i] - e[i - 1];
        double magnitude = fabs(span);
        if (fabs(step) > magnitude) magnitude = fabs(step);
        if (fabs(current) > magnitude) magnitude = fabs(current);
        if (1.0 > magnitude) magnitude = 1.0;
        const double tolerance = 1024.0 * 2.220446049250313080847e-16 * magnitude;
        if (fabs(current - step) > tolerance) {
            return 0;
        }
    }
    *step_out = step;
    return 1;
}

int kpt_oracle_grid_init(kpt_oracle_grid* g, int nx, int ny, const double* x_edges,
                         const double* y_edges, int force_stored) {
    memset(g, 0, sizeof(*g));
    if (nx <= 0 || ny <= 0) {
        return fail("grid: dimensions must be positive");
    }
    g->n[0] = nx;
    g->n[1] = ny;
    const double* edges[2] = {x_edges, y_edges};
    for (int d = 0; d < 2; ++d) {
        const int n = g->n[d];
        const double* e = edges[d];
        if (!edges_ascending(e, n)) {
            kpt_oracle_grid_free(g);
            return fail("grid: face coordinates must be finite and strictly ascending");
        }
        double step = 0.0;
        if (!force_stored && edges_uniform(e, n, &step)) {
            /* AnalyticCoordinateGrid.hpp:369-399 bounds cache. */
            const double x0 = e[0];
            g->stored[d] = 0;
            g->start[d] = x0;
            g->step[d] = step;
            g->lower[d] = x0 + 0.0 * step;
            g->upper[d] = x0 + (double)n * step;
            g->ghost_lower[d] = x0 + (double)(-2) * step;
            g->ghost_upper[d] = x0 + (double)(n + 2) * step;
        } else {
            /* StoredCoordinateGrid.hpp:75-99, 451-465 with ghost faces
             * continued periodically (stated extension). */
            const double w = e[n] - e[0];
            g->stored[d] = 1;
            g->faces[d] = (double*)malloc(sizeof(double) * (size_t)(n + 5));
            g->centers[d] = (double*)malloc(sizeof(double) * (size_t)(n + 4));
            for (int k = -2; k <= n + 2; ++k) {
                double f;
                if (k < 0) {
                    f = e[n + k] - w;
                } else if (k > n) {
                    f = e[k - n] + w;
                } else {
                    f = e[k];
                }
                g->faces[d][k + 2] = f;
            }
            for (int s = 0; s < n + 4; ++s) {
                g->centers[d][s] = 0.5 * (g->faces[d][s] + g->faces[d][s + 1]);
            }
            g->lower[d] = g->faces[d][2];
            g->upper[d] = g->faces[d][n + 2];
            g->ghost_lower[d] = g->faces[d][0];
            g->ghost_upper[d] = g->faces[d][n + 4];
        }
        g->width[d] = g->upper[d] - g->lower[d];
        g->inv_width[d] = g->width[d] != 0.0 ? 1.0 / g->width[d] : 0.0;
    }
    return 0;
}

void kpt_oracle_grid_free(kpt_oracle_grid* g) {
    for (int d = 0; d < 2; ++d) {
        free(g->faces[d]);
        free(g->centers[d]);
        g->faces[d] = NULL;
        g->centers[d] = NULL;
    }
}

size_t kpt_oracle_point_count(const kpt_oracle_grid* g) {
    return (size_t)(g->n[0] + 4) * (size_t)(g->n[1] + 4);
}

/* Cell-centre coordinate of logical cell `index`
 * (AnalyticCoordinateGrid.hpp:179-183 / StoredCoordinateGrid.hpp:104-109). */
static double cell_coordinate(const kpt_oracle_grid* g, int d, int index) {
    if (g->stored[d]) {
        return g->centers[d][index + 2];
    }
    const double ci = (double)index;
    const double f0 = g->start[d] + ci * g->step[d];
    const double f1 = g->start[d] + (ci + 1.0) * g->step[d];
    return 0.5 * (f0 + f1);
}

/* Continuous cell-centred logical index over the ghosted domain
 * (AnalyticCoordinateGrid.hpp:214-230; StoredCoordinateGrid.hpp:124-174). */
static double cell_grid_index(const kpt_oracle_grid* g, int d, double x) {
    if (!g->stored[d]) {
        return (x - g->start[d]) / g->step[d] - 0.5;
    }
    const double* c = g->centers[d];
    const int lower_index = -2;
    const int upper_index = g->n[d] + 1;
    const double lower_x = c[lower_index + 2];
    const double upper_x = c[upper_index + 2];
    int left, right;
    if (x <= lower_x) {
        left = lower_index;
    } else if (x >= upper_x) {
        left = upper_index - 1;
    } else {
        int lo = lower_index;
        int hi = upper_index - 1;
        left = lower_index;
        while (lo <= hi) {
            const int mid = lo + (hi - lo) / 2;
            const double x_left = c[mid + 2];
            const double x_right = c[mid + 3];
            if (x >= x_left && x < x_right) {
                left = mid;
                break;
            }
            if (x < x_left) {
                hi = mid - 1;
            } else {
                lo = mid + 1;
            }
        }
    }
    right = left + 1;
    const double x_left = c[left + 2];
    const double x_right = c[right + 2];
    return (double)left + (x - x_left) / (x_right - x_left);
}

/* MappedCoordinateGrid.hpp:284-306 / StoredCoordinateGrid.hpp:357-377. */
static double grid_wrap(const kpt_oracle_grid* g, int d, double x) {
    const double lower_x = g->lower[d];
    const double upper_x = g->upper[d];
    const double width = g->width[d];
    double wrapped = x - floor((x - lower_x) * g->inv_width[d]) * width;
    if (wrapped >= upper_x) {
        wrapped -= width;
    }
    if (wrapped < lower_x) {
        wrapped += width;
    }
    return wrapped;
}

/* src/main.cpp:642-665. */
double kpt_oracle_wrap(double value, double lower, double upper, double width) {
    double wrapped = value;
    if (wrapped >= upper) {
        wrapped -= width;
        if (wrapped >= upper) {
            wrapped -= floor((wrapped - lower) / width) * width;
        }
    } else if (wrapped < lower) {
        wrapped += width;
        if (wrapped < lower) {
            wrapped -= floor((wrapped - lower) / width) * width;
        }
    }
    if (wrapped >= upper) {
        wrapped -= width;
    }
    if (wrapped < lower) {
        wrapped += width;
    }
    return wrapped;
}

static size_t flatten(const kpt_oracle_grid* g, int i, int j) {
    return (size_t)(i + 2) + (size_t)(j + 2) * (size_t)(g->n[0] + 4);
}

/* ------------------------------------------------------------- fields */

/* AthenaFieldReader.hpp:195-240 copy plus Field.hpp:274-316 periodic ghost
 * fill (both axes periodic, src/main.cpp:965-968). */
void kpt_oracle_load_vector_field(const kpt_oracle_grid* g, const double* cells,
                                  double* ghosted) {
    const int nx = g->n[0], ny = g->n[1];
    const size_t cell_count = (size_t)nx * (size_t)ny;
    const size_t points = kpt_oracle_point_count(g);
    memset(ghosted, 0, sizeof(double) * points * 3);
    for (int comp = 0; comp < 3; ++comp) {
        for (int j = 0; j < ny; ++j) {
            for (int i = 0; i < nx; ++i) {
                ghosted[flatten(g, i, j) * 3 + (size_t)comp] =
                    cells[(size_t)comp * cell_count + (size_t)j * (size_t)nx + (size_t)i];
            }
        }
    }
    for (size_t pnt = 0; pnt < points; ++pnt) {
        const int i = (int)(pnt % (size_t)(nx + 4)) - 2;
        const int j = (int)(pnt / (size_t)(nx + 4)) - 2;
        int si = i, sj = j;
        int ghost = 0;
        if (i < 0 || i > nx - 1) {
            ghost = 1;
            si = i % nx;
            if (si < 0) si += nx;
        }
        if (j < 0 || j > ny - 1) {
            ghost = 1;
            sj = j % ny;
            if (sj < 0) sj += ny;
        }
        if (!ghost) {
            continue;
        }
        const size_t src = flatten(g, si, sj);
        for (int comp = 0; comp < 3; ++comp) {
            ghosted[pnt * 3 + (size_t)comp] = ghosted[src * 3 + (size_t)comp];
        }
    }
}

static double vec_at(const double* f, const kpt_oracle_grid* g, int i, int j, int comp) {
    return f[flatten(g, i, j) * 3 + (size_t)comp];
}

static double bmag_at(const double* b, const kpt_oracle_grid* g, int i, int j) {
    const double bx = vec_at(b, g, i, j, 0);
    const double by = vec_at(b, g, i, j, 1);
    const double bz = vec_at(b, g, i, j, 2);
    return sqrt(bx * bx + by * by + bz * bz);
}

/* derivative_component / derivative_magnetic_magnitude
 * (src/main.cpp:716-834); which < 0 selects |B|. */
static double derivative(const double* f, const kpt_oracle_grid* g, int i, int j, int dim,
                         int comp) {
    const int n = g->n[dim];
    if (n <= 1) {
        return 0.0;
    }
    const int lower = -2;
    const int upper = n + 1;
    const int idx = dim == 0 ? i : j;
#define KPT_AT(a, b) (comp < 0 ? bmag_at(f, g, (a), (b)) : vec_at(f, g, (a), (b), comp))
#define KPT_SHIFT(k) (dim == 0 ? KPT_AT((k), j) : KPT_AT(i, (k)))
    if (idx <= lower) {
        const double x0 = cell_coordinate(g, dim, lower);
        const double x2 = cell_coordinate(g, dim, lower + 2);
        return (-3.0 * KPT_SHIFT(lower) + 4.0 * KPT_SHIFT(lower + 1) - KPT_SHIFT(lower + 2)) /
               (x2 - x0);
    }
    if (idx >= upper) {
        const double x0 = cell_coordinate(g, dim, upper - 2);
        const double x2 = cell_coordinate(g, dim, upper);
        return (3.0 * KPT_SHIFT(upper) - 4.0 * KPT_SHIFT(upper - 1) + KPT_SHIFT(upper - 2)) /
               (x2 - x0);
    }
    const double xl = cell_coordinate(g, dim, idx - 1);
    const double xr = cell_coordinate(g, dim, idx + 1);
    return (KPT_SHIFT(idx + 1) - KPT_SHIFT(idx - 1)) / (xr - xl);
#undef KPT_SHIFT
#undef KPT_AT
}

/* make_parker_reconnection_coefficients (src/main.cpp:840-892) and
 * make_reconnection_coefficients (src/main.cpp:898-957); component order
 * src/main.cpp:38-79. */
void kpt_oracle_build_table(const kpt_oracle_grid* g, const double* b, const double* v,
                            int focused, double* table) {
    const size_t points = kpt_oracle_point_count(g);
    const int ncomp = focused ? 21 : 16;
#pragma omp parallel for schedule(static)
    for (long long pl = 0; pl < (long long)points; ++pl) {
        const size_t pnt = (size_t)pl;
        const int i = (int)(pnt % (size_t)(g->n[0] + 4)) - 2;
        const int j = (int)(pnt / (size_t)(g->n[0] + 4)) - 2;
        double* out = table + pnt * (size_t)ncomp;
        const double bx = vec_at(b, g, i, j, 0);
        const double by = vec_at(b, g, i, j, 1);
        const double bz = vec_at(b, g, i, j, 2);
        const double bm = sqrt(bx * bx + by * by + bz * bz);
        if (!focused) {
            out[0] = vec_at(v, g, i, j, 0);
            out[1] = vec_at(v, g, i, j, 1);
            out[2] = bx;
            out[3] = by;
            out[4] = bz;
            out[5] = bm;
            out[6] = derivative(v, g, i, j, 0, 0);
            out[7] = derivative(v, g, i, j, 1, 1);
            out[8] = derivative(b, g, i, j, 0, 0);
            out[9] = derivative(b, g, i, j, 1, 0);
            out[10] = derivative(b, g, i, j, 0, 1);
            out[11] = derivative(b, g, i, j, 1, 1);
            out[12] = derivative(b, g, i, j, 0, 2);
            out[13] = derivative(b, g, i, j, 1, 2);
            out[14] = derivative(b, g, i, j, 0, -1);
            out[15] = derivative(b, g, i, j, 1, -1);
        } else {
            out[0] = vec_at(v, g, i, j, 0);
            out[1] = vec_at(v, g, i, j, 1);
            out[2] = vec_at(v, g, i, j, 2);
            out[3] = bx;
            out[4] = by;
            out[5] = bz;
            out[6] = bm;
            out[7] = derivative(v, g, i, j, 0, 0);
            out[8] = derivative(v, g, i, j, 1, 0);
            out[9] = derivative(v, g, i, j, 0, 1);
            out[10] = derivative(v, g, i, j, 1, 1);
            out[11] = derivative(v, g, i, j, 0, 2);
            out[12] = derivative(v, g, i, j, 1, 2);
            out[13] = derivative(b, g, i, j, 0, 0);
            out[14] = derivative(b, g, i, j, 1, 0);
            out[15] = derivative(b, g, i, j, 0, 1);
            out[16] = derivative(b, g, i, j, 1, 1);
            out[17] = derivative(b, g, i, j, 0, 2);
            out[18] = derivative(b, g, i, j, 1, 2);
            out[19] = derivative(b, g, i, j, 0, -1);
            out[20] = derivative(b, g, i, j, 1, -1);
        }
    }
}

int kpt_oracle_table_from_cells(int nx, int ny, const double* x_edges, const double* y_edges,
                                const double* b_cells, const double* v_cells, int focused,
                                int force_stored, double* table) {
    kpt_oracle_grid g;
    if (kpt_oracle_grid_init(&g, nx, ny, x_edges, y_edges, force_stored) != 0) {
        return -1;
    }
    for (size_t k = 0; k < (size_t)nx * (size_t)ny * 3; ++k) {
        if (!isfinite(b_cells[k]) || !isfinite(v_cells[k])) {
            kpt_oracle_grid_free(&g);
            return fail("field: non-finite cell value");
        }
    }
    const size_t points = kpt_oracle_point_count(&g);
    double* b = (double*)malloc(sizeof(double) * points * 3);
    double* v = (double*)malloc(sizeof(double) * points * 3);
    kpt_oracle_load_vector_field(&g, b_cells, b);
    kpt_oracle_load_vector_field(&g, v_cells, v);
    kpt_oracle_build_table(&g, b, v, focused, table);
    free(b);
    free(v);
    kpt_oracle_grid_free(&g);
    return 0;
}

/* -------------------------------------------------------- interpolation */

/* LinearPositionInterpolator::compute_axis_stencil
 * (FieldInterpolator.hpp:509-559), cell-centred, ghosted domain. */
static void axis_stencil(const kpt_oracle_grid* g, int d, double coordinate, int* lo, int* hi,
                         double* w) {
    const int lower_bound = -2;
    const int upper_bound = g->n[d] + 1;
    const double logical = cell_grid_index(g, d, coordinate);
    if (logical <= (double)lower_bound) {
        *lo = lower_bound;
        *hi = lower_bound;
        *w = 0.0;
        return;
    }
    if (logical >= (double)upper_bound) {
        *lo = upper_bound;
        *hi = upper_bound;
        *w = 0.0;
        return;
    }
    const int candidate = (int)floor(logical);
    *lo = candidate;
    *hi = candidate + 1;
    *w = logical - (double)candidate;
    if (*lo < lower_bound) {
        *lo = lower_bound;
        *hi = lower_bound;
        *w = 0.0;
    } else if (*hi > upper_bound) {
        *lo = upper_bound;
        *hi = upper_bound;
        *w = 0.0;
    }
}

/* LinearPositionInterpolator::sample (FieldInterpolator.hpp:346-380) with
 * WrapPeriodic preparation (:482-503). */
static void sample_one(const kpt_oracle_grid* g, const double* table, int ncomp, double q0,
                       double q1, double* out) {
    const double c0 = grid_wrap(g, 0, q0);
    const double c1 = grid_wrap(g, 1, q1);
    int lo[2], hi[2];
    double w[2];
    axis_stencil(g, 0, c0, &lo[0], &hi[0], &w[0]);
    axis_stencil(g, 1, c1, &lo[1], &hi[1], &w[1]);
    for (int c = 0; c < ncomp; ++c) {
        out[c] = 0.0;
    }
    for (int corner = 0; corner < 4; ++corner) {
        const int ux = (corner & 1) != 0;
        const int uy = ((corner >> 1) & 1) != 0;
        double weight = 1.0;
        weight *= ux ? w[0] : (1.0 - w[0]);
        weight *= uy ? w[1] : (1.0 - w[1]);
        const double* cell = table + flatten(g, ux ? hi[0] : lo[0], uy ? hi[1] : lo[1]) *
                                         (size_t)ncomp;
        for (int c = 0; c < ncomp; ++c) {
            out[c] += weight * cell[c];
        }
    }
}

/* sample_time_interpolated_coefficients (src/main.cpp:1055-1077). */
static void sample_time(const kpt_oracle_grid* g, const double* lower, const double* upper,
                        int ncomp, double q0, double q1, double rt, int use_time, double* out) {
    double lv[21];
    sample_one(g, lower, ncomp, q0, q1, lv);
    if (use_time == 0) {
        for (int c = 0; c < ncomp; ++c) {
            out[c] = lv[c];
        }
        return;
    }
    double uv[21];
    sample_one(g, upper, ncomp, q0, q1, uv);
    const double upper_weight = rt < 0.0 ? 0.0 : (rt > 1.0 ? 1.0 : rt);
    const double lower_weight = 1.0 - upper_weight;
    for (int c = 0; c < ncomp; ++c) {
        out[c] = lower_weight * lv[c] + upper_weight * uv[c];
    }
}

void kpt_oracle_sample(const kpt_oracle_grid* g, const double* lower_table,
                       const double* upper_table, int ncomp, double x, double y, double rt,
                       int time_interpolation, double* out) {
    const double shift_x = 0.5 * ((g->upper[0] - g->lower[0]) / (double)g->n[0]);
    const double shift_y = 0.5 * ((g->upper[1] - g->lower[1]) / (double)g->n[1]);
    sample_time(g, lower_table, upper_table, ncomp, x + shift_x, y + shift_y, rt,
                time_interpolation, out);
}

/* ------------------------------------------------------------------ push */

typedef struct {
    double x_lower, x_upper, y_lower, y_upper, x_width, y_width, dx, dy;
    double shift_x, shift_y, pindex, dt_min, dt_max, pmin_split, h0;
} derived_settings;

/* make_device_settings (src/main.cpp:596-636). */
static derived_settings derive(const kpt_oracle_grid* g, const kpt_oracle_params* s) {
    derived_settings d;
    d.x_lower = g->lower[0];
    d.x_upper = g->upper[0];
    d.y_lower = g->lower[1];
    d.y_upper = g->upper[1];
    d.x_width = d.x_upper - d.x_lower;
    d.y_width = d.y_upper - d.y_lower;
    d.dx = d.x_width / (double)g->n[0];
    d.dy = d.y_width / (double)g->n[1];
    d.shift_x = 0.5 * d.dx;
    d.shift_y = 0.5 * d.dy;
    d.pindex = 3.0 - s->gamma_turb;
    d.dt_min = s->dt_min_rel * s->mhd_dt;
    d.dt_max = s->dt_max_rel * s->mhd_dt;
    d.pmin_split = s->pmin_split_over_p0 * s->p0;
    d.h0 = 0.2; /* Reconnection2DDeviceSettings default, src/main.cpp:279 */
    return d;
}

static double square(double v) { return v * v; }
static double min_positive(double a, double b) { return a < b ? a : b; }
static double clamp_mu(double v, double m) {
    if (v > m) return m;
    if (v < -m) return -m;
    return v;
}

static const double kSqrt3 = 1.7320508075688772935;
static const double kPi = 3.141592653589793238462643383279502884;

/* pitch_angle_spectrum_normalization (LegencyModel.hpp:539-552). */
static double qlt_normalization(double spectral_index) {
    const double sine_value = sin(kPi / spectral_index);
    return spectral_index * sine_value / kPi;
}

double kpt_oracle_qlt_dmumu(double mu, double omega, double speed, double sigma2, double lc,
                            double spectral_index, double h0) {
    const double one_minus_mu2 = 1.0 - mu * mu;
    if (one_minus_mu2 <= 0.0) {
        return 0.0;
    }
    const double regularized_abs_mu = (mu >= 0.0 ? mu : -mu) + h0;
    const double gamma_k = spectral_index;
    const double xi = omega * lc / speed;
    const double abs_mu_gamma = ORACLE_POW(regularized_abs_mu, gamma_k);
    const double xi_gamma = ORACLE_POW(xi, gamma_k);
    const double denominator = abs_mu_gamma + xi_gamma;
    const double prefactor = 0.25 * kPi * omega * sigma2 * qlt_normalization(gamma_k);
    return prefactor * one_minus_mu2 * xi * ORACLE_POW(regularized_abs_mu, gamma_k - 1.0) / denominator;
}

double kpt_oracle_qlt_dmumu_dmu(double mu, double dmumu, double omega, double speed, double lc,
                                double spectral_index, double h0) {
    if (dmumu == 0.0) {
        return 0.0;
    }
    const double sign_mu = mu > 0.0 ? 1.0 : (mu < 0.0 ? -1.0 : 0.0);
    if (sign_mu == 0.0) {
        return 0.0;
    }
    const double one_minus_mu2 = 1.0 - mu * mu;
    if (one_minus_mu2 <= 0.0) {
        return 0.0;
    }
    const double regularized_abs_mu = (mu >= 0.0 ? mu : -mu) + h0;
    const double gamma_k = spectral_index;
    const double xi = omega * lc / speed;
    const double abs_mu_gamma = ORACLE_POW(regularized_abs_mu, gamma_k);
    const double xi_gamma = ORACLE_POW(xi, gamma_k);
    const double denominator = abs_mu_gamma + xi_gamma;
    const double shape_derivative =
        sign_mu * ((gamma_k - 1.0) / regularized_abs_mu -
                   gamma_k * ORACLE_POW(regularized_abs_mu, gamma_k - 1.0) / denominator);
    const double endpoint_derivative = -2.0 * mu / one_minus_mu2;
    return dmumu * (endpoint_derivative + shape_derivative);
}

/* StochasticSampler::uniform_sqrt3 (RandomManager.hpp:111-114). */
static double uniform_sqrt3(kpt_oracle_stream* s) {
    return -kSqrt3 + (kSqrt3 - -kSqrt3) * kpt_oracle_stream_u01(s);
}

/* Per-particle body of move_parker_particles_one_interval
 * (src/main.cpp:1114-1324). */
static void push_parker_one(const kpt_oracle_grid* g, const double* lower_table,
                            const double* upper_table, const kpt_oracle_params* s,
                            const derived_settings* d, double interval_start,
                            double interval_end, uint32_t frame, uint64_t seed, size_t index,
                            double* X, double* Y, double* P, double* T, double* DT,
                            int32_t* status, uint32_t* steps) {
    if (status[index] != 0) {
        if (steps) steps[index] = 0;
        return;
    }
    kpt_oracle_stream gen;
    kpt_oracle_stream_init(&gen, seed, (uint32_t)index, frame, KPT_ORACLE_TAG_PUSH);
    double x = X[index];
    double y = Y[index];
    double p = P[index];
    double t = T[index];
    double dt = DT[index];
    double diagnostic_dt = dt;
    int step_guard = 0;
    int st = 0;
    double c[16];

    while (t < interval_end && step_guard < s->max_steps && st == 0) {
        ++step_guard;
        x = kpt_oracle_wrap(x, d->x_lower, d->x_upper, d->x_width);
        y = kpt_oracle_wrap(y, d->y_lower, d->y_upper, d->y_width);
        const double q0 = x + d->shift_x;
        const double q1 = y + d->shift_y;
        const double rt = (t - interval_start) / s->mhd_dt;
        sample_time(g, lower_table, upper_table, 16, q0, q1, rt, s->time_interpolation, c);

        const double vx = c[0], vy = c[1], bx = c[2], by = c[3], bz = c[4], b = c[5];
        const double dvx_dx = c[6], dvy_dy = c[7], dbx_dx = c[8], dbx_dy = c[9];
        const double dby_dx = c[10], dby_dy = c[11], dbz_dx = c[12], dbz_dy = c[13];
        const double db_dx = c[14], db_dy = c[15];

        if (!isfinite(p) || p <= 0.0 || !isfinite(b) || b <= 0.0) {
            st = 2;
            break;
        }
        const double ib = 1.0 / b;
        const double ib2 = ib * ib;
        const double ib3 = ib2 * ib;

        double knorm_para = 1.0;
        if (s->magnetic_dependency == 1) {
            knorm_para *= ORACLE_POW(b, s->gamma_turb - 2.0);
        }
        double knorm = knorm_para;
        if (s->momentum_dependency == 1) {
            knorm *= ORACLE_POW(p / s->p0, d->pindex);
        }
        const double kpara = s->kpara0 * knorm;
        const double kperp = kpara * s->kperp_over_kpara;
        if (!isfinite(kpara) || kpara <= 0.0 || !isfinite(kperp) || kperp < 0.0) {
            st = 2;
            break;
        }
        const double skpara = sqrt(2.0 * kpara);
        const double skperp = sqrt(2.0 * kperp);
        const double skpara_perp = sqrt(2.0 * (kpara - kperp));
        const double kpp = kpara - kperp;

        double dkdx = 0.0;
        double dkdy = 0.0;
        if (s->magnetic_dependency == 1) {
            const double magnetic_exponent = s->gamma_turb - 2.0;
            dkdx = db_dx * ib * magnetic_exponent;
            dkdy = db_dy * ib * magnetic_exponent;
        }
        const double dkxx_dx = kperp * dkdx + kpp * dkdx * bx * bx * ib2 +
                               2.0 * kpp * bx * (dbx_dx * b - bx * db_dx) * ib3;
        const double dkyy_dy = kperp * dkdy + kpp * dkdy * by * by * ib2 +
                               2.0 * kpp * by * (dby_dy * b - by * db_dy) * ib3;
        const double dkxy_dx = kpp * dkdx * bx * by * ib2 +
                               kpp * ((dbx_dx * by + bx * dby_dx) * ib2 -
                                      2.0 * bx * by * db_dx * ib3);
        const double dkxy_dy = kpp * dkdy * bx * by * ib2 +
                               kpp * ((dbx_dy * by + bx * dby_dy) * ib2 -
                                      2.0 * bx * by * db_dy * ib3);

        const double drift_denominator =
            sqrt(square(s->drift_param1 * s->p0 / p) +
                 square(s->drift_param2 * s->p0 * s->p0 / (p * p)));
        const double vdp = 1.0 / (3.0 * s->charge) / drift_denominator;
        const double vdx = vdp * (dbz_dy * ib2 - 2.0 * bz * db_dy * ib3);
        const double vdy = vdp * (-dbz_dx * ib2 + 2.0 * bz * db_dx * ib3);

        const double dx_dt = vx + vdx + dkxx_dx + dkxy_dy;
        const double dy_dt = vy + vdy + dkxy_dx + dkyy_dy;
        const double divv = dvx_dx + dvy_dy;
        const double dp_dt = -p * divv / 3.0;

        if (dx_dt != 0.0 && dy_dt != 0.0 && dp_dt != 0.0) {
            const double diffusion_dt_x = square(0.5 * d->dx / skpara);
            const double diffusion_dt_y = square(0.5 * d->dy / skpara);
            const double advection_scale = skperp > 0.0 ? skperp : skpara;
            const double advection_dt_x = square(advection_scale / dx_dt);
            const double advection_dt_y = square(advection_scale / dy_dt);
            const double momentum_dt = 0.1 * p / fabs(dp_dt);
            dt = min_positive(diffusion_dt_x, diffusion_dt_y);
            dt = min_positive(dt, advection_dt_x);
            dt = min_positive(dt, advection_dt_y);
            dt = min_positive(dt, momentum_dt);
        } else {
            dt = d->dt_min;
        }
        if (dt < d->dt_min) {
            dt = d->dt_min;
        }
        if (dt > d->dt_max) {
            dt = d->dt_max;
        }
        diagnostic_dt = dt;
        const double remaining = interval_end - t;
        if (dt > remaining) {
            dt = remaining;
        }
        if (!isfinite(dt) || dt <= 0.0) {
            st = 2;
            break;
        }

        const double sdt = sqrt(dt);
        const double ran1 = uniform_sqrt3(&gen);
        const double ran2 = uniform_sqrt3(&gen);
        const double ran3 = uniform_sqrt3(&gen);
        const double delta_x =
            dx_dt * dt + ran1 * skperp * sdt + ran3 * skpara_perp * sdt * bx * ib;
        const double delta_y =
            dy_dt * dt + ran2 * skperp * sdt + ran3 * skpara_perp * sdt * by * ib;
        (void)uniform_sqrt3(&gen);
        const double delta_p = dp_dt * dt;

        x += delta_x;
        y += delta_y;
        p += delta_p;
        t += dt;
        if (p < 0.25 * s->p0) {
            p = 0.25 * s->p0;
        }
        if (!isfinite(x) || !isfinite(y) || !isfinite(p) || !isfinite(t)) {
            st = 2;
            break;
        }
    }
    if (step_guard >= s->max_steps && t < interval_end) {
        st = 2;
    }
    status[index] = st;
    X[index] = kpt_oracle_wrap(x, d->x_lower, d->x_upper, d->x_width);
    Y[index] = kpt_oracle_wrap(y, d->y_lower, d->y_upper, d->y_width);
    P[index] = p;
    T[index] = t;
    DT[index] = diagnostic_dt;
    if (steps) steps[index] = (uint32_t)step_guard;
}

/* Per-particle body of move_particles_one_interval, focused branch
 * (src/main.cpp:1365-1752). */
static void push_focused_one(const kpt_oracle_grid* g, const double* lower_table,
                             const double* upper_table, const kpt_oracle_params* s,
                             const derived_settings* d, double interval_start,
                             double interval_end, uint32_t frame, uint64_t seed, size_t index,
                             double* X, double* Y, double* P, double* T, double* DT,
                             double* MU, int32_t* status, uint32_t* steps) {
    if (status[index] != 0) {
        if (steps) steps[index] = 0;
        return;
    }
    kpt_oracle_stream gen;
    kpt_oracle_stream_init(&gen, seed, (uint32_t)index, frame, KPT_ORACLE_TAG_PUSH);
    double x = X[index];
    double y = Y[index];
    double p = P[index];
    double pitch_mu = clamp_mu(MU[index], s->mu_max);
    double t = T[index];
    double dt = DT[index];
    double diagnostic_dt = dt;
    int step_guard = 0;
    int st = 0;
    double c[21];

    while (t < interval_end && step_guard < s->max_steps && st == 0) {
        ++step_guard;
        x = kpt_oracle_wrap(x, d->x_lower, d->x_upper, d->x_width);
        y = kpt_oracle_wrap(y, d->y_lower, d->y_upper, d->y_width);
        const double q0 = x + d->shift_x;
        const double q1 = y + d->shift_y;
        const double rt = (t - interval_start) / s->mhd_dt;
        sample_time(g, lower_table, upper_table, 21, q0, q1, rt, s->time_interpolation, c);

        const double vx = c[0], vy = c[1];
        const double bx = c[3], by = c[4], bz = c[5], b = c[6];
        const double dvx_dx = c[7], dvx_dy = c[8], dvy_dx = c[9], dvy_dy = c[10];
        const double dvz_dx = c[11], dvz_dy = c[12];
        const double dbx_dx = c[13], dbx_dy = c[14], dby_dx = c[15], dby_dy = c[16];
        const double dbz_dx = c[17], dbz_dy = c[18], db_dx = c[19], db_dy = c[20];

        if (!isfinite(p) || p <= 0.0 || !isfinite(b) || b <= 0.0) {
            st = 2;
            break;
        }
        const double ib = 1.0 / b;
        const double ib2 = ib * ib;
        const double ib3 = ib2 * ib;

        double knorm_para = 1.0;
        if (s->magnetic_dependency == 1) {
            knorm_para *= ORACLE_POW(b, s->gamma_turb - 2.0);
        }
        double knorm = knorm_para;
        if (s->momentum_dependency == 1) {
            knorm *= ORACLE_POW(p / s->p0, d->pindex);
        }
        const double kpara = s->kpara0 * knorm;
        const double kperp = kpara * s->kperp_over_kpara;
        if (!isfinite(kpara) || kpara <= 0.0 || !isfinite(kperp) || kperp < 0.0) {
            st = 2;
            break;
        }
        const double skpara = sqrt(2.0 * kpara);
        const double skperp = sqrt(2.0 * kperp);
        const double kpp = -kperp;

        double dkdx = 0.0;
        double dkdy = 0.0;
        if (s->magnetic_dependency == 1) {
            const double magnetic_exponent = s->gamma_turb - 2.0;
            dkdx = db_dx * ib * magnetic_exponent;
            dkdy = db_dy * ib * magnetic_exponent;
        }
        const double dkxx_dx = kperp * dkdx + kpp * dkdx * bx * bx * ib2 +
                               2.0 * kpp * bx * (dbx_dx * b - bx * db_dx) * ib3;
        const double dkyy_dy = kperp * dkdy + kpp * dkdy * by * by * ib2 +
                               2.0 * kpp * by * (dby_dy * b - by * db_dy) * ib3;
        const double dkxy_dx = kpp * dkdx * bx * by * ib2 +
                               kpp * ((dbx_dx * by + bx * dby_dx) * ib2 -
                                      2.0 * bx * by * db_dx * ib3);
        const double dkxy_dy = kpp * dkdy * bx * by * ib2 +
                               kpp * ((dbx_dy * by + bx * dby_dy) * ib2 -
                                      2.0 * bx * by * db_dy * ib3);

        const double drift_denominator =
            sqrt(square(s->drift_param1 * s->p0 / p) +
                 square(s->drift_param2 * s->p0 * s->p0 / (p * p)));

        pitch_mu = clamp_mu(pitch_mu, s->mu_max);
        const double mu2 = pitch_mu * pitch_mu;
        const double muf1 = 0.5 * (1.0 - mu2);
        const double muf2 = 0.5 * (3.0 * mu2 - 1.0);
        const double kx = bx * dbx_dx + by * dbx_dy;
        const double ky = bx * dby_dx + by * dby_dy;
        const double kz = bx * dbz_dx + by * dbz_dy;
        const double bdot_curvb = bx * dbz_dy - by * dbz_dx + bz * (dby_dx - dbx_dy);
        const double vdp = 1.0 / s->charge / drift_denominator;
        const double vdx = vdp * (muf1 * (-bz * db_dy) * ib2 + mu2 * (by * kz - bz * ky) * ib3 +
                                  muf1 * bx * bdot_curvb * ib3);
        const double vdy = vdp * (muf1 * (bz * db_dx) * ib2 + mu2 * (bz * kx - bx * kz) * ib3 +
                                  muf1 * by * bdot_curvb * ib3);
        const double speed = s->particle_v0 * p / s->p0;
        if (!isfinite(speed) || speed <= 0.0) {
            st = 2;
            break;
        }
        const double v_parallel_over_b = speed * pitch_mu * ib;
        const double vbx = v_parallel_over_b * bx;
        const double vby = v_parallel_over_b * by;
        const double dx_dt = vx + vdx + vbx + dkxx_dx + dkxy_dy;
        const double dy_dt = vy + vdy + vby + dkxy_dx + dkyy_dy;

        const double divv = dvx_dx + dvy_dy;
        const double bb_gradv = (bx * (bx * dvx_dx + by * dvx_dy) +
                                 by * (bx * dvy_dx + by * dvy_dy) +
                                 bz * (bx * dvz_dx + by * dvz_dy)) *
                                ib2;
        const double bv_gradv = (bx * (vx * dvx_dx + vy * dvx_dy) +
                                 by * (vx * dvy_dx + vy * dvy_dy) +
                                 bz * (vx * dvz_dx + vy * dvz_dy)) *
                                ib;
        const double acc_rate =
            -(muf1 * divv + muf2 * bb_gradv + pitch_mu * bv_gradv / speed);
        const double dp_dt = p * acc_rate;

        const double div_bnorm = -(bx * db_dx + by * db_dy) * ib2;
        double dmu_dt = speed * div_bnorm + pitch_mu * divv - 3.0 * pitch_mu * bb_gradv -
                        2.0 * bv_gradv / speed;
        dmu_dt *= 0.5 * (1.0 - mu2);
        double duu = 0.0;
        double duu_du = 0.0;
        if (s->closure == 1) {
            /* slab QLT closure (extension): LegencyModel's D_mumu, dD_mumu/dmu */
            const double lorentz = sqrt(1.0 + p * p);
            const double omega = s->qlt_omega0 * b / lorentz;
            duu = kpt_oracle_qlt_dmumu(pitch_mu, omega, speed, s->qlt_sigma2, s->qlt_lc,
                                       s->qlt_spectral_index, s->qlt_h0);
            duu_du = kpt_oracle_qlt_dmumu_dmu(pitch_mu, duu, omega, speed, s->qlt_lc,
                                              s->qlt_spectral_index, s->qlt_h0);
        } else {
            const double abs_mu = fabs(pitch_mu);
            const double dtmp = ORACLE_POW(abs_mu, s->gamma_turb - 1.0) + d->h0;
            duu = s->duu0 * (1.0 - mu2) * dtmp;
            if (pitch_mu > 0.0) {
                duu_du = s->duu0 * (-2.0 * pitch_mu * dtmp +
                                    (1.0 - mu2) * ORACLE_POW(abs_mu, s->gamma_turb - 2.0));
            } else if (pitch_mu < 0.0) {
                duu_du = s->duu0 * (-2.0 * pitch_mu * dtmp -
                                    (1.0 - mu2) * ORACLE_POW(abs_mu, s->gamma_turb - 2.0));
            }
            double duu_norm = 1.0;
            if (s->magnetic_dependency == 1) {
                duu_norm *= ORACLE_POW(b, 2.0 - s->gamma_turb);
            }
            if (s->momentum_dependency == 1) {
                duu_norm *= ORACLE_POW(p / s->p0, s->gamma_turb - 1.0);
            }
            duu *= duu_norm;
            duu_du *= duu_norm;
        }
        dmu_dt += duu_du;
        if (!isfinite(dmu_dt) || !isfinite(duu) || duu < 0.0) {
            st = 2;
            break;
        }

        const double diffusion_scale = skperp > 0.0 ? skperp : skpara;
        if (dx_dt != 0.0 && dy_dt != 0.0 && dp_dt != 0.0 && dmu_dt != 0.0 &&
            diffusion_scale > 0.0) {
            const double diffusion_dt_x = square(0.5 * d->dx / diffusion_scale);
            const double diffusion_dt_y = square(0.5 * d->dy / diffusion_scale);
            const double advection_dt_x = square(diffusion_scale / dx_dt);
            const double advection_dt_y = square(diffusion_scale / dy_dt);
            const double momentum_dt = 0.1 * p / fabs(dp_dt);
            const double pitch_advection_dt = 0.1 / fabs(dmu_dt);
            const double pitch_balance_dt = 2.0 * duu / square(dmu_dt);
            dt = min_positive(diffusion_dt_x, diffusion_dt_y);
            dt = min_positive(dt, advection_dt_x);
            dt = min_positive(dt, advection_dt_y);
            dt = min_positive(dt, momentum_dt);
            dt = min_positive(dt, pitch_advection_dt);
            dt = min_positive(dt, pitch_balance_dt);
        } else {
            dt = d->dt_min;
        }
        if (dt < d->dt_min) {
            dt = d->dt_min;
        }
        if (dt > d->dt_max) {
            dt = d->dt_max;
        }
        diagnostic_dt = dt;
        const double remaining = interval_end - t;
        if (dt > remaining) {
            dt = remaining;
        }
        if (!isfinite(dt) || dt <= 0.0) {
            st = 2;
            break;
        }

        const double sdt = sqrt(dt);
        const double delta_p = dp_dt * dt;
        const double ran1 = uniform_sqrt3(&gen);
        const double ran2 = uniform_sqrt3(&gen);
        const double bxn = bx * ib;
        const double byn = by * ib;
        const double bzn = bz * ib;
        const double bxy_norm = sqrt(bxn * bxn + byn * byn);
        double stochastic_x = 0.0;
        double stochastic_y = 0.0;
        if (bxy_norm > 0.0) {
            const double ibxy_norm = 1.0 / bxy_norm;
            stochastic_x = skperp * ibxy_norm * sdt * (-bxn * bzn * ran1 - by * ran2);
            stochastic_y = skperp * ibxy_norm * sdt * (-byn * bzn * ran1 + bx * ran2);
        }
        const double delta_x = dx_dt * dt + stochastic_x;
        const double delta_y = dy_dt * dt + stochastic_y;
        (void)uniform_sqrt3(&gen);
        const double pitch_random = uniform_sqrt3(&gen);
        pitch_mu = clamp_mu(pitch_mu + dmu_dt * dt + pitch_random * sqrt(2.0 * duu) * sdt,
                            s->mu_max);

        x += delta_x;
        y += delta_y;
        p += delta_p;
        t += dt;
        if (p < 0.25 * s->p0) {
            p = 0.25 * s->p0;
        }
        if (!isfinite(x) || !isfinite(y) || !isfinite(p) || !isfinite(t)) {
            st = 2;
            break;
        }
    }
    if (step_guard >= s->max_steps && t < interval_end) {
        st = 2;
    }
    status[index] = st;
    X[index] = kpt_oracle_wrap(x, d->x_lower, d->x_upper, d->x_width);
    Y[index] = kpt_oracle_wrap(y, d->y_lower, d->y_upper, d->y_width);
    P[index] = p;
    MU[index] = pitch_mu;
    T[index] = t;
    DT[index] = diagnostic_dt;
    if (steps) steps[index] = (uint32_t)step_guard;
}

void kpt_oracle_push(const kpt_oracle_grid* g, const double* lower_table,
                     const double* upper_table, const kpt_oracle_params* s,
                     double interval_start, uint32_t frame, uint64_t seed, size_t count,
                     double* x, double* y, double* p, double* t, double* step_dt, double* mu,
                     int32_t* status, uint32_t* steps, int threads) {
    const derived_settings d = derive(g, s);
    const double interval_end = interval_start + s->mhd_dt;
#ifdef _OPENMP
    const int nthreads = threads > 0 ? threads : omp_get_max_threads();
#else
    const int nthreads = 1;
    (void)threads;
#endif
    /* Dynamic chunks: substep counts differ per particle. */
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads)
    for (long long i = 0; i < (long long)count; ++i) {
        if (s->focused) {
            push_focused_one(g, lower_table, upper_table, s, &d, interval_start, interval_end,
                             frame, seed, (size_t)i, x, y, p, t, step_dt, mu, status, steps);
        } else {
            push_parker_one(g, lower_table, upper_table, s, &d, interval_start, interval_end,
                            frame, seed, (size_t)i, x, y, p, t, step_dt, status, steps);
        }
    }
}

/* ------------------------------------------------------------ lifecycle */

uint64_t kpt_oracle_inject(const kpt_oracle_grid* g, const kpt_oracle_params* s,
                           double interval_start, uint32_t frame, uint64_t seed,
                           uint64_t capacity, uint64_t count, uint64_t requested,
                           double band_lo, double band_hi, double* x, double* y, double* p,
                           double* t, double* step_dt, double* weight, double* mu,
                           int32_t* status, int32_t* split_level) {
    if (count >= capacity) {
        return count;
    }
    const uint64_t insert = requested < capacity - count ? requested : capacity - count;
    const derived_settings d = derive(g, s);
    const double y_lo = band_lo < band_hi ? band_lo : d.y_lower;
    const double y_hi = band_lo < band_hi ? band_hi : d.y_upper;
    for (uint64_t k = 0; k < insert; ++k) {
        kpt_oracle_stream gen;
        kpt_oracle_stream_init(&gen, seed, (uint32_t)k, frame, KPT_ORACLE_TAG_INJECT);
        const uint64_t n = count + k;
        x[n] = d.x_lower + (d.x_upper - d.x_lower) * kpt_oracle_stream_u01(&gen);
        y[n] = y_lo + (y_hi - y_lo) * kpt_oracle_stream_u01(&gen);
        p[n] = s->p0;
        t[n] = interval_start + (0.0 + (s->mhd_dt - 0.0) * kpt_oracle_stream_u01(&gen));
        step_dt[n] = d.dt_min;
        weight[n] = 1.0;
        mu[n] = s->mu_max * (2.0 * kpt_oracle_stream_u01(&gen) - 1.0);
        status[n] = 0;
        split_level[n] = 0;
    }
    return count + insert;
}

uint64_t kpt_oracle_split(const kpt_oracle_params* s, uint64_t capacity, uint64_t count,
                          double* x, double* y, double* p, double* t, double* step_dt,
                          double* weight, double* mu, int32_t* status, int32_t* split_level,
                          uint64_t* split_out, uint64_t* skipped_out) {
    *split_out = 0;
    *skipped_out = 0;
    if (count >= capacity || s->split_particles == 0) {
        return count;
    }
    const double pmin_split = s->pmin_split_over_p0 * s->p0;
    uint64_t next = count;
    for (uint64_t parent = 0; parent < count; ++parent) {
        if (status[parent] != 0) {
            continue;
        }
        const int old_level = split_level[parent];
        const double threshold = pmin_split * ORACLE_POW(s->split_ratio, (double)old_level);
        const double pp = p[parent];
        if (!(pp > threshold && pp <= s->pmax)) {
            continue;
        }
        const uint64_t child = next++;
        if (child >= capacity) {
            ++*skipped_out;
            continue;
        }
        const int new_level = old_level + 1;
        const double new_weight = ORACLE_POW(0.5, (double)new_level);
        x[child] = x[parent];
        y[child] = y[parent];
        p[child] = p[parent];
        t[child] = t[parent];
        step_dt[child] = step_dt[parent];
        weight[parent] = new_weight;
        weight[child] = new_weight;
        mu[child] = mu[parent];
        status[child] = 0;
        split_level[parent] = new_level;
        split_level[child] = new_level;
        ++*split_out;
    }
    return next < capacity ? next : capacity;
}

void kpt_oracle_histogram(double pmin, double pmax, int nbins, uint64_t count, const double* p,
                          const double* weight, const int32_t* status, double* bins) {
    for (int b = 0; b < nbins; ++b) {
        bins[b] = 0.0;
    }
    const double log_pmin = log(pmin);
    const double inv_dlogp = (double)nbins / (log(pmax) - log_pmin);
    for (uint64_t i = 0; i < count; ++i) {
        if (status[i] != 0) {
            continue;
        }
        const double pp = p[i];
        if (pp < pmin || pp > pmax) {
            continue;
        }
        int bin = (int)((log(pp) - log_pmin) * inv_dlogp);
        if (bin < 0) bin = 0;
        if (bin >= nbins) bin = nbins - 1;
        bins[bin] += weight[i];
    }
}

void kpt_oracle_summarize(uint64_t count, const double* p, const double* step_dt,
                          const double* weight, const int32_t* status,
                          const int32_t* split_level, kpt_oracle_summary* out) {
    memset(out, 0, sizeof(*out));
    out->stored = count;
    if (count == 0) {
        return;
    }
    double p_sum = 0.0, dt_sum = 0.0;
    out->p_min = INFINITY;
    out->dt_min = INFINITY;
    out->p_max = 0.0;
    out->dt_max = 0.0;
    for (uint64_t i = 0; i < count; ++i) {
        if (status[i] == 0) {
            ++out->active;
            const double pp = p[i];
            const double dt = step_dt[i];
            out->weight_sum += weight[i];
            p_sum += pp;
            dt_sum += dt;
            out->p_min = pp < out->p_min ? pp : out->p_min;
            out->p_max = out->p_max < pp ? pp : out->p_max;
            out->dt_min = dt < out->dt_min ? dt : out->dt_min;
            out->dt_max = out->dt_max < dt ? dt : out->dt_max;
            out->max_split_level =
                out->max_split_level < split_level[i] ? split_level[i] : out->max_split_level;
        } else {
            ++out->inactive;
        }
    }
    if (out->active > 0) {
        out->p_avg = p_sum / (double)out->active;
        out->dt_avg = dt_sum / (double)out->active;
    } else {
        out->p_min = 0.0;
        out->dt_min = 0.0;
    }
}

void kpt_oracle_pow_array(uint64_t n, const double* x, const double* y, double* out) {
    for (uint64_t i = 0; i < n; ++i) {
        out[i] = kpt_pow(x[i], y[i]);
    }
}
