// 2D Cartesian grids with two ghost layers per side (Grid.hpp:65) on the
// device, for the library solvers: uniform analytic axes
// (AnalyticCoordinateGrid.hpp) or explicit face coordinates
// (StoredCoordinateGrid.hpp).
#pragma once

#include <array>
#include <cstdint>
#include <memory>
#include <vector>

#include "Runtime.hpp"

namespace kpt {

// GridDomain (Grid.hpp): the physical cells or the cells plus ghosts.
enum class GridDomain { PhysicalDomain = KPT_PHYSICAL_DOMAIN, GhostedDomain = KPT_GHOSTED_DOMAIN };

class CartesianGrid2D {
public:
    static constexpr int space_dim = 2;
    static constexpr int ghost_layers = 2;

    // nx x ny cells between the given edges (nx + 1 and ny + 1 values,
    // uniform as the reference's compact-field reader requires,
    // AthenaFieldReader.hpp:167-193), periodic per axis.
    CartesianGrid2D(int nx, int ny, const std::vector<double>& x_edges,
                    const std::vector<double>& y_edges, std::array<bool, 2> periodic,
                    Context context = default_context())
        : context_(context), nx_(nx), ny_(ny), x_edges_(x_edges), y_edges_(y_edges),
          periodic_(periodic) {
        if (static_cast<int>(x_edges.size()) != nx + 1 ||
            static_cast<int>(y_edges.size()) != ny + 1) {
            throw std::runtime_error("CartesianGrid2D: edges must hold nx + 1 and ny + 1 values.");
        }
        const int32_t flags[2] = {periodic[0] ? 1 : 0, periodic[1] ? 1 : 0};
        kpt_grid* raw = nullptr;
        check(kpt_grid_create(context_.get(), nx, ny, x_edges.data(), y_edges.data(), flags,
                              &raw));
        handle_ = std::shared_ptr<kpt_grid>(raw, [](kpt_grid* g) { kpt_grid_destroy(g); });
    }

    int cell_count(int dim) const { return dim == 0 ? nx_ : ny_; }
    // Stored (ghosted) cells per axis and in total: the point count of a
    // cell-centred Field on this grid.
    int ghosted_count(int dim) const { return cell_count(dim) + 2 * ghost_layers; }
    std::size_t point_count() const {
        return static_cast<std::size_t>(ghosted_count(0)) * static_cast<std::size_t>(ghosted_count(1));
    }
    // Field::flatten (Field.hpp:185-192) for logical cell (i, j), -2 <= i < nx + 2.
    std::size_t flatten(int i, int j) const {
        return static_cast<std::size_t>(i + ghost_layers) +
               static_cast<std::size_t>(j + ghost_layers) * static_cast<std::size_t>(ghosted_count(0));
    }
    double lower(int dim) const { return dim == 0 ? x_edges_.front() : y_edges_.front(); }
    double upper(int dim) const { return dim == 0 ? x_edges_.back() : y_edges_.back(); }
    bool periodic(int dim) const { return periodic_[dim]; }
    const std::vector<double>& edges(int dim) const { return dim == 0 ? x_edges_ : y_edges_; }

    kpt_grid* get() const { return handle_.get(); }
    const Context& context() const { return context_; }

protected:
    struct StoredFaces {};
    // explicit faces: nx + 5 and ny + 5 values, face -2 first
    CartesianGrid2D(StoredFaces, int nx, int ny, const std::vector<double>& x_faces,
                    const std::vector<double>& y_faces, std::array<bool, 2> periodic,
                    Context context)
        : context_(context), nx_(nx), ny_(ny), periodic_(periodic) {
        if (static_cast<int>(x_faces.size()) != nx + 5 ||
            static_cast<int>(y_faces.size()) != ny + 5) {
            throw std::runtime_error(
                "StoredCoordinateGrid: face coordinate view is too short.");
        }
        x_edges_.assign(x_faces.begin() + ghost_layers, x_faces.end() - ghost_layers);
        y_edges_.assign(y_faces.begin() + ghost_layers, y_faces.end() - ghost_layers);
        const int32_t flags[2] = {periodic[0] ? 1 : 0, periodic[1] ? 1 : 0};
        kpt_grid* raw = nullptr;
        check(kpt_grid_create_stored(context_.get(), nx, ny, x_faces.data(), y_faces.data(),
                                     flags, &raw));
        handle_ = std::shared_ptr<kpt_grid>(raw, [](kpt_grid* g) { kpt_grid_destroy(g); });
    }

private:
    Context context_;
    int nx_, ny_;
    std::vector<double> x_edges_, y_edges_;
    std::array<bool, 2> periodic_;
    std::shared_ptr<kpt_grid> handle_;
};

// StoredCoordinateGrid (StoredCoordinateGrid.hpp:53-66, validated as
// GridValidation::make_validated_stored_coordinate_grid does): the same 2D
// Cartesian grid on explicit, possibly non-uniform face coordinates, nx + 5
// and ny + 5 of them in storage order, face -2 first (the two ghost faces
// on each side included).  It is a CartesianGrid2D: every field, solver and
// lifecycle call takes it; edges(dim) are its physical faces 0 .. n.
class StoredCoordinateGrid2D : public CartesianGrid2D {
public:
    StoredCoordinateGrid2D(int nx, int ny, const std::vector<double>& x_faces,
                           const std::vector<double>& y_faces, std::array<bool, 2> periodic,
                           Context context = default_context())
        : CartesianGrid2D(StoredFaces{}, nx, ny, x_faces, y_faces, periodic, context) {}
};

// Cell-centred field values on the host, C components per ghosted point of
// a grid, points in Field::flatten order (x fastest), components contiguous.
// The reference's Field<Grid, C> keeps these on the device; the coefficient
// builders and solvers here copy them to the device when they run.  Like the
// reference's Field, a HostField knows its grid.
template <int C>
class HostField {
public:
    static constexpr int components = C;
    explicit HostField(const CartesianGrid2D& grid)
        : grid_(grid), values_(grid.point_count() * C, 0.0) {}
    HostField(const CartesianGrid2D& grid, std::vector<double> values)
        : grid_(grid), values_(std::move(values)) {
        if (values_.size() != grid_.point_count() * C) {
            throw std::runtime_error("HostField: values must hold points x components doubles.");
        }
    }
    double& operator()(std::size_t point, int comp) { return values_[point * C + comp]; }
    double operator()(std::size_t point, int comp) const { return values_[point * C + comp]; }
    // value at logical cell (i, j), -2 <= i < nx + 2
    double& at(int i, int j, int comp) { return values_[grid_.flatten(i, j) * C + comp]; }
    std::size_t point_count() const { return grid_.point_count(); }
    const CartesianGrid2D& grid() const { return grid_; }
    const double* data() const { return values_.data(); }
    double* data() { return values_.data(); }

private:
    CartesianGrid2D grid_;
    std::vector<double> values_;
};

using VectorField = HostField<3>;
using ScalarField = HostField<1>;

}  // namespace kpt
