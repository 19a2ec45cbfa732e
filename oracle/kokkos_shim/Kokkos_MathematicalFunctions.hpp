// Host math functions under the Kokkos names used by the reference; each one
// forwards to the C++ standard library (glibc), which is what Kokkos' host
// backends call.  Oracle-only shim.
#pragma once

#include <cmath>

namespace Kokkos {
using std::abs;
using std::cos;
using std::exp;
using std::floor;
using std::isfinite;
using std::log;
using std::pow;
using std::sin;
using std::sqrt;
}  // namespace Kokkos
