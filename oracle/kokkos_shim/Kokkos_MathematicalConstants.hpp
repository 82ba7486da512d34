// Kokkos_MathematicalConstants.hpp -- Kokkos::numbers::pi_v lives in the shim's Kokkos_Core.hpp.
#pragma once
#include "Kokkos_Core.hpp"
