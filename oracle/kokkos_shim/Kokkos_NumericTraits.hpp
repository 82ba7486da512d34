// Kokkos_NumericTraits.hpp -- epsilon_v / finite_max_v / finite_min_v live in the shim's Kokkos_Core.hpp.
#pragma once
#include "Kokkos_Core.hpp"
