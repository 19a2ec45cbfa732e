// Host math functions under the Kokkos names used by the reference.  Each
// one forwards to the C++ standard library (glibc), which is what Kokkos'
// host backends call, except pow: Kokkos::pow is the project pow
// (kokkos-particletransport_gb300/csrc/kpt_pow.h), the one the GPU's FP64 push
// and the C restatement call, so the reference's kernels round every power
// exactly as the GPU does (CUDA's pow and glibc's pow each err by up to about
// an ulp, and not alike).  Built with -DKPT_SHIM_LIBM_POW, Kokkos::pow is the
// C library's, as in a real Kokkos host build: that build is the one timed
// against the C restatement.  Oracle-only shim.
#pragma once

#include <cmath>
#include <type_traits>

#include "kpt_pow.h"

namespace Kokkos {
using std::abs;
using std::cos;
using std::exp;
using std::floor;
using std::isfinite;
using std::log;
using std::sin;
using std::sqrt;

#ifdef KPT_SHIM_LIBM_POW
inline double pow(double x, double y) { return std::pow(x, y); }
#else
inline double pow(double x, double y) { return kpt_pow(x, y); }
#endif

template <class X, class Y,
          class = std::enable_if_t<std::is_arithmetic_v<X> && std::is_arithmetic_v<Y>>>
inline double pow(X x, Y y) {
    return Kokkos::pow(static_cast<double>(x), static_cast<double>(y));
}
}  // namespace Kokkos
