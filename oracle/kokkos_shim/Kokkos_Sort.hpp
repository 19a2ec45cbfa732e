// Placeholder so headers that include Kokkos_Sort.hpp parse; the driver path
// compiled into the oracle does not sort.  Oracle-only shim.
#pragma once
#include "Kokkos_Core.hpp"
