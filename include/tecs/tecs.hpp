// tecs/tecs.hpp -- umbrella header of the C++20 drop-in layer over the GB300
// cell-step library (include/tecs_gpu.h); the counterpart of the reference's
// include/tecs.hpp for the per-timestep path.  Link with -ltecs_gb300.
#ifndef TECS_CXX_TECS_HPP
#define TECS_CXX_TECS_HPP

#include "components.hpp"
#include "config.hpp"
#include "grid.hpp"
#include "hdf5_reader.hpp"
#include "kokkos_compat.hpp"
#include "plane.hpp"
#include "random.hpp"
#include "simulation.hpp"
#include "vector.hpp"
#include "view.hpp"

#endif  // TECS_CXX_TECS_HPP
