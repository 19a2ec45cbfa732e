// Host stand-ins for Kokkos::BinOp1D and Kokkos::BinSort as the reference's
// ParticleSystem uses them (integer keys, one bin per key value).  The sort
// is a stable counting sort, i.e. the serial order within each bin.
// Oracle-only shim.
#pragma once

#include <vector>

#include "Kokkos_Core.hpp"

namespace Kokkos {

template <class KeyView>
struct BinOp1D {
    int bins;
    long long min_key;
    BinOp1D(int max_bins, long long min_value, long long /*max_value*/)
        : bins(max_bins), min_key(min_value) {}
    int bin(long long key) const {
        long long b = key - min_key;
        return static_cast<int>(b < 0 ? 0 : (b >= bins ? bins - 1 : b));
    }
};

template <class KeyView, class BinOp>
class BinSort {
public:
    BinSort(const KeyView& keys, int begin, int end, const BinOp& op, bool /*sort_within_bins*/)
        : keys_(keys), begin_(begin), end_(end), op_(op) {}

    void create_permute_vector() {
        const int n = end_ - begin_;
        std::vector<int> counts(static_cast<std::size_t>(op_.bins) + 1, 0);
        for (int i = begin_; i < end_; ++i) {
            ++counts[static_cast<std::size_t>(op_.bin(keys_(i))) + 1];
        }
        for (std::size_t b = 1; b < counts.size(); ++b) {
            counts[b] += counts[b - 1];
        }
        permute_.assign(static_cast<std::size_t>(n), 0);
        for (int i = begin_; i < end_; ++i) {
            permute_[static_cast<std::size_t>(counts[static_cast<std::size_t>(op_.bin(keys_(i)))]++)] = i;
        }
    }

    template <class View>
    void sort(const View& view) const {
        const std::size_t width = View::rank == 2 ? view.extent(1) : 1;
        std::vector<typename View::non_const_value_type> copy(permute_.size() * width);
        for (std::size_t k = 0; k < permute_.size(); ++k) {
            for (std::size_t c = 0; c < width; ++c) {
                copy[k * width + c] = view.data()[static_cast<std::size_t>(permute_[k]) * width + c];
            }
        }
        for (std::size_t k = 0; k < permute_.size(); ++k) {
            for (std::size_t c = 0; c < width; ++c) {
                view.data()[(static_cast<std::size_t>(begin_) + k) * width + c] = copy[k * width + c];
            }
        }
    }

private:
    KeyView keys_;
    int begin_;
    int end_;
    BinOp op_;
    std::vector<int> permute_;
};

}  // namespace Kokkos
