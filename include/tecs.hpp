// tecs.hpp -- the drop-in layer's umbrella header at the path the reference's
// programs include (include/tecs.hpp, as "../include/tecs.hpp" from
// examples/).  A program compiled by g++ gets the simulation API with the
// built-in force laws; compiled by nvcc (-std=c++20 --extended-lambda) it
// also gets its own PAIRWISE_FORCE / GENERIC_FORCE / LINK_FORCE laws
// (tecs/pairwise.cuh).  Link with -ltecs_gb300.
#ifndef TECS_DROP_IN_TECS_HPP
#define TECS_DROP_IN_TECS_HPP

#include <iostream>  // the reference's umbrella brings the standard streams to its programs

#include "tecs/tecs.hpp"
#if defined(__CUDACC__)
#include "tecs/pairwise.cuh"
#endif

#endif  // TECS_DROP_IN_TECS_HPP
