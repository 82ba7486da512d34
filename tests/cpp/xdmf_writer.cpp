// xdmf_writer.cpp -- the write sequence of a TECS program through the
// drop-in layer's io::HDF5_Writer, without a simulation: write_static of a
// "cell_type" view, then writes of (position, polarity, links) at times
// 0, dt, 2 dt, ... in the argument order Simulation::write uses
// (simulation.hpp:607-611).  The test compares "<path>.xmf" with the
// reference writer's sidecar for the same counts.
//
//   xdmf_writer <path without extension> <cells> <links> <writes> <dt>
#include <cstdlib>
#include <string>

#include "tecs/tecs.hpp"

using namespace tecs;

int main(int argc, char** argv) {
  if (argc < 6) return 2;
  const std::string path = argv[1];
  const unsigned n = unsigned(std::atoi(argv[2]));
  const unsigned n_links = unsigned(std::atoi(argv[3]));
  const int writes = std::atoi(argv[4]);
  const double dt = std::atof(argv[5]);
  io::HDF5_Writer<DefaultSimulationConfig> w(path);
  View<VectorN<float, 3>> position("position", n);
  View<Polarity_<float>> polarity("polarity", n);
  for (unsigned i = 0; i < n; ++i) {
    position(i) = VectorN<float, 3>(float(i), 0.5f * i, -0.25f * i);
    polarity(i) = Polarity_<float>(0.01f * i, 0.02f * i);
  }
  View<Link> links("links", n_links);
  for (unsigned l = 0; l < n_links; ++l) links(l) = Link{l % n, (l + 1) % n};
  View<float> cell_type("cell_type", n);
  for (unsigned i = 0; i < n; ++i) cell_type(i) = float(i % 3);
  w.write_static(cell_type);
  for (int k = 0; k < writes; ++k) w.write(k * dt, unsigned(k), position, polarity, links);
  return 0;
}
