// Minimal host-only stand-in for the subset of the Kokkos API that the
// reference driver (src/main.cpp) and its include chain use.  It exists so the
// reference's own, unmodified sources compile into the oracle in oracle/_ref;
// it is test infrastructure and never part of the product.
//
// Written from the documented semantics of the Kokkos API (Views are
// reference-counted handles; parallel_for over a RangePolicy calls the functor
// once per index; deep_copy / create_mirror_view copy between spaces; fences
// are no-ops for a synchronous host backend).  Everything lives in host memory
// with LayoutRight indexing.  parallel_for runs under OpenMP schedule(static)
// and publishes the kernel label and loop index in thread-local storage so the
// random pool (Kokkos_Random.hpp) can key its noise by particle index.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#define KOKKOS_INLINE_FUNCTION inline
#define KOKKOS_FUNCTION
#define KOKKOS_LAMBDA [=]

#include "Kokkos_MathematicalFunctions.hpp"

namespace Kokkos {

struct LayoutRight {};
struct LayoutLeft {};
struct HostSpace {
    using memory_space = HostSpace;
    using size_type = std::size_t;
};

template <class ExecSpace, class MemSpace>
struct Device {
    using execution_space = ExecSpace;
    using memory_space = MemSpace;
    using device_type = Device<ExecSpace, MemSpace>;
};

struct OpenMP {
    using execution_space = OpenMP;
    using memory_space = HostSpace;
    using array_layout = LayoutRight;
    using device_type = Device<OpenMP, HostSpace>;
    using size_type = std::size_t;
    // an execution-space instance: work is synchronous, so fencing is a no-op
    void fence(const char* = nullptr) const {}
};

using DefaultExecutionSpace = OpenMP;
using DefaultHostExecutionSpace = OpenMP;

template <unsigned Traits>
struct MemoryTraits {
    static constexpr unsigned value = Traits;
};
enum MemoryTraitsFlags : unsigned { Unmanaged = 1u, RandomAccess = 2u, Atomic = 4u };

namespace ShimImpl {

// Per-thread record of the running kernel, read by the random pool.
struct KernelContext {
    const char* label = nullptr;
    std::uint64_t index = 0;
    std::uint32_t ordinal = 0;  // 1-based launch count of this label
};
inline KernelContext& current_kernel() {
    static thread_local KernelContext context;
    return context;
}

// Launch count per kernel label (host thread only), used by the random pool
// to key noise by frame when the reference CLI drives the frame loop.
struct LaunchOrdinals {
    std::vector<std::string> labels;
    std::vector<std::uint32_t> counts;
};
inline LaunchOrdinals& launch_ordinals() {
    static LaunchOrdinals ordinals;
    return ordinals;
}
inline std::uint32_t count_launch(const std::string& label) {
    auto& o = launch_ordinals();
    for (std::size_t k = 0; k < o.labels.size(); ++k) {
        if (o.labels[k] == label) {
            return ++o.counts[k];
        }
    }
    o.labels.push_back(label);
    o.counts.push_back(1u);
    return 1u;
}

template <class T>
struct ViewDataTraits;

template <class T>
struct ViewDataTraits<T*> {
    using value_type = T;
    static constexpr int rank = 1;
    static constexpr std::size_t static_extent1 = 0;
};

template <class T, std::size_t N>
struct ViewDataTraits<T* [N]> {
    using value_type = T;
    static constexpr int rank = 2;
    static constexpr std::size_t static_extent1 = N;
};

template <class T>
struct ViewDataTraits<T**> {
    using value_type = T;
    static constexpr int rank = 2;
    static constexpr std::size_t static_extent1 = 0;
};

template <class T>
struct MutableDataType {
    using type = T;
};
template <class T>
struct MutableDataType<const T*> {
    using type = T*;
};
template <class T, std::size_t N>
struct MutableDataType<const T* [N]> {
    using type = T* [N];
};
template <class T>
struct MutableDataType<const T**> {
    using type = T**;
};

}  // namespace ShimImpl

template <class DataType, class... Properties>
class View {
public:
    using traits = ShimImpl::ViewDataTraits<DataType>;
    using value_type = typename traits::value_type;
    using non_const_value_type = std::remove_const_t<value_type>;
    using size_type = std::size_t;
    using memory_space = HostSpace;
    using execution_space = OpenMP;
    using HostMirror = View<typename ShimImpl::MutableDataType<DataType>::type, LayoutRight,
                            HostSpace>;
    static constexpr int rank = traits::rank;

    View() = default;

    explicit View(const std::string& label, std::size_t n0 = 0, std::size_t n1 = 0)
        : label_(label), n0_(n0) {
        n1_ = traits::static_extent1 != 0 ? traits::static_extent1 : (rank == 2 ? n1 : 1);
        storage_ = std::make_shared<std::vector<non_const_value_type>>(
            n0_ * (rank == 2 ? n1_ : 1));
        data_ = storage_->data();
    }

    // Shallow conversion between views of the same storage (e.g. to const).
    template <class OtherData, class... OtherProps>
    View(const View<OtherData, OtherProps...>& other)
        : label_(other.label_), n0_(other.n0_), n1_(other.n1_),
          storage_(other.storage_), data_(other.data_) {}

    value_type& operator()(const std::size_t i) const { return data_[i]; }
    value_type& operator()(const std::size_t i, const std::size_t j) const {
        return data_[i * n1_ + j];
    }

    std::size_t extent(const std::size_t dim) const {
        if (dim == 0) {
            return n0_;
        }
        if (dim == 1 && rank == 2) {
            return n1_;
        }
        return 1;
    }
    std::size_t size() const { return n0_ * (rank == 2 ? n1_ : 1); }
    std::size_t span() const { return size(); }
    value_type* data() const { return data_; }
    const std::string& label() const { return label_; }

    std::string label_;
    std::size_t n0_ = 0;
    std::size_t n1_ = 1;
    std::shared_ptr<std::vector<non_const_value_type>> storage_;
    non_const_value_type* data_ = nullptr;
};

template <class DataType, class... Props>
auto create_mirror_view(const View<DataType, Props...>& view) {
    using mirror_type = typename View<DataType, Props...>::HostMirror;
    mirror_type mirror(view.label(), view.extent(0), view.extent(1));
    return mirror;
}

template <class DataType, class... Props>
auto create_mirror_view_and_copy(const HostSpace&, const View<DataType, Props...>& view) {
    auto mirror = create_mirror_view(view);
    std::copy(view.data(), view.data() + view.size(), mirror.data());
    return mirror;
}

template <class D1, class... P1, class D2, class... P2>
void deep_copy(const View<D1, P1...>& dst, const View<D2, P2...>& src) {
    if (dst.size() != src.size()) {
        throw std::runtime_error("Kokkos shim: deep_copy extent mismatch.");
    }
    std::copy(src.data(), src.data() + src.size(), dst.data());
}

template <class Exec, class D1, class... P1, class D2, class... P2>
void deep_copy(const Exec&, const View<D1, P1...>& dst, const View<D2, P2...>& src) {
    deep_copy(dst, src);
}

template <class D1, class... P1, class Scalar,
          class = std::enable_if_t<std::is_arithmetic_v<Scalar>>>
void deep_copy(const View<D1, P1...>& dst, const Scalar value) {
    std::fill(dst.data(), dst.data() + dst.size(),
              static_cast<typename View<D1, P1...>::non_const_value_type>(value));
}

template <class ExecSpace = OpenMP>
struct RangePolicy {
    std::int64_t begin = 0;
    std::int64_t end = 0;
    template <class B, class E>
    RangePolicy(const B input_begin, const E input_end)
        : begin(static_cast<std::int64_t>(input_begin)),
          end(static_cast<std::int64_t>(input_end)) {}
};

template <class ExecSpace, class Functor>
void parallel_for(const std::string& label, const RangePolicy<ExecSpace>& policy,
                  const Functor& functor) {
    const char* label_text = label.c_str();
    const std::uint32_t ordinal = ShimImpl::count_launch(label);
#pragma omp parallel for schedule(static)
    for (std::int64_t i = policy.begin; i < policy.end; ++i) {
        auto& context = ShimImpl::current_kernel();
        context.label = label_text;
        context.index = static_cast<std::uint64_t>(i);
        context.ordinal = ordinal;
        functor(static_cast<std::size_t>(i));
    }
}

// Min reducer: identity is the largest value, join takes the minimum.
template <class T>
struct Min {
    T& result;
    explicit Min(T& target) : result(target) {}
};

// parallel_reduce with a Min reducer (functor(i, T& update)).
template <class ExecSpace, class Functor, class T>
void parallel_reduce(const std::string& label, const RangePolicy<ExecSpace>& policy,
                     const Functor& functor, const Min<T>& reducer) {
    (void)ShimImpl::count_launch(label);
    T value = std::numeric_limits<T>::max();
    for (std::int64_t i = policy.begin; i < policy.end; ++i) {
        auto& context = ShimImpl::current_kernel();
        context.label = label.c_str();
        context.index = static_cast<std::uint64_t>(i);
        T local = std::numeric_limits<T>::max();
        functor(static_cast<std::size_t>(i), local);
        value = local < value ? local : value;
    }
    reducer.result = value;
}

// parallel_reduce summing into a scalar (functor(i, T& update)), serial order.
template <class ExecSpace, class Functor, class T,
          class = std::enable_if_t<std::is_arithmetic_v<T>>>
void parallel_reduce(const std::string& label, const RangePolicy<ExecSpace>& policy,
                     const Functor& functor, T& result) {
    (void)ShimImpl::count_launch(label);
    T value = T(0);
    for (std::int64_t i = policy.begin; i < policy.end; ++i) {
        auto& context = ShimImpl::current_kernel();
        context.label = label.c_str();
        context.index = static_cast<std::uint64_t>(i);
        functor(static_cast<std::size_t>(i), value);
    }
    result = value;
}

// parallel_scan (functor(i, T& update, bool final_pass)) in serial order: a
// single final pass in which update holds the exclusive prefix on entry;
// result receives the total.
template <class ExecSpace, class Functor, class T>
void parallel_scan(const std::string& label, const RangePolicy<ExecSpace>& policy,
                   const Functor& functor, T& result) {
    (void)ShimImpl::count_launch(label);
    T value = T(0);
    for (std::int64_t i = policy.begin; i < policy.end; ++i) {
        auto& context = ShimImpl::current_kernel();
        context.label = label.c_str();
        context.index = static_cast<std::uint64_t>(i);
        functor(static_cast<std::size_t>(i), value, true);
    }
    result = value;
}

inline void fence() {}
inline void fence(const std::string&) {}

template <class T, std::size_t N>
struct Array {
    T values[N > 0 ? N : 1];
    T& operator[](const std::size_t i) { return values[i]; }
    const T& operator[](const std::size_t i) const { return values[i]; }
    static constexpr std::size_t size() { return N; }
    bool operator==(const Array& other) const {
        for (std::size_t i = 0; i < N; ++i) {
            if (!(values[i] == other.values[i])) {
                return false;
            }
        }
        return true;
    }
};

template <class T, class U>
T atomic_fetch_add(T* destination, const U value) {
    T previous;
#pragma omp atomic capture
    {
        previous = *destination;
        *destination += static_cast<T>(value);
    }
    return previous;
}

template <class T, class U>
void atomic_add(T* destination, const U value) {
#pragma omp atomic
    *destination += static_cast<T>(value);
}

inline void initialize(int&, char**) {}
inline void initialize() {}
inline void finalize() {}

[[noreturn]] inline void abort(const char* message) {
    std::fprintf(stderr, "Kokkos shim abort: %s\n", message);
    std::abort();
}

}  // namespace Kokkos
