// C++ drop-in for the reference's header library, over the C ABI (kpt.h):
// errors, the device context and the process-wide default context.
//
// The reference's classes are Kokkos templates whose storage lives in the
// default execution space after Kokkos::initialize.  Here the storage lives
// on one CUDA device behind a kpt_context; kpt::ScopeGuard (or
// kpt::initialize / kpt::finalize) plays the part of Kokkos::ScopeGuard and
// makes the default context every wrapper uses unless it is given another.
// Host-side validation errors throw std::runtime_error with the reference's
// messages, as the reference's host code does (kpt::Error derives from it).
#pragma once

#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>

#include "../kpt.h"

namespace kpt {

class Error : public std::runtime_error {
public:
    Error(int code, const std::string& message) : std::runtime_error(message), code_(code) {}
    int code() const { return code_; }

private:
    int code_;
};

inline void check(int rc) {
    if (rc != KPT_OK) {
        const char* msg = kpt_last_error();
        throw Error(rc, msg != nullptr ? std::string(msg) : std::string("kpt: error"));
    }
}

// One CUDA device and stream (kpt_context).  Copies share the context;
// objects made from it keep it alive.
class Context {
public:
    explicit Context(int device = 0) {
        kpt_context* raw = nullptr;
        check(kpt_context_create(device, &raw));
        handle_ = std::shared_ptr<kpt_context>(raw, [](kpt_context* c) {
            kpt_context_destroy(c);
        });
        device_ = device;
    }
    kpt_context* get() const { return handle_.get(); }
    int device() const { return device_; }
    void synchronize() const { check(kpt_context_synchronize(handle_.get())); }
    // Order later calls on an external cudaStream_t (nullptr: the context's own).
    void set_stream(void* cuda_stream) const {
        check(kpt_context_set_stream(handle_.get(), cuda_stream));
    }

private:
    std::shared_ptr<kpt_context> handle_;
    int device_ = 0;
};

namespace detail {
inline std::mutex& default_mutex() {
    static std::mutex m;
    return m;
}
inline std::shared_ptr<Context>& default_slot() {
    static std::shared_ptr<Context> slot;
    return slot;
}
}  // namespace detail

// Make the default context on `device` (Kokkos::initialize).  Calling it
// again with the default context alive is a no-op.
inline void initialize(int device = 0) {
    std::lock_guard<std::mutex> lock(detail::default_mutex());
    if (!detail::default_slot()) {
        detail::default_slot() = std::make_shared<Context>(device);
    }
}

// Drop the default context (Kokkos::finalize).  Objects made from it keep it
// alive until they are destroyed.
inline void finalize() {
    std::lock_guard<std::mutex> lock(detail::default_mutex());
    detail::default_slot().reset();
}

inline bool is_initialized() {
    std::lock_guard<std::mutex> lock(detail::default_mutex());
    return static_cast<bool>(detail::default_slot());
}

// The default context; made on device 0 on first use if initialize() was
// not called.
inline Context default_context() {
    std::lock_guard<std::mutex> lock(detail::default_mutex());
    if (!detail::default_slot()) {
        detail::default_slot() = std::make_shared<Context>(0);
    }
    return *detail::default_slot();
}

// RAII initialize/finalize (Kokkos::ScopeGuard).
class ScopeGuard {
public:
    explicit ScopeGuard(int device = 0) { initialize(device); }
    ~ScopeGuard() { finalize(); }
    ScopeGuard(const ScopeGuard&) = delete;
    ScopeGuard& operator=(const ScopeGuard&) = delete;
};

}  // namespace kpt
