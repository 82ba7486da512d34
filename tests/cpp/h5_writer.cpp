// h5_writer.cpp -- writes a small snapshot file through the drop-in layer's
// io::HDF5_Writer (positions, polarity, links, a static view); the test reads
// it back and compares it byte for byte with tecs_gb300.h5's writer.
//
//   h5_writer <path without extension>
//   h5_writer <path without extension> <steps>   one write per step, t0 .. t<steps-1>, of a 2-cell position
//                                                view (a long run, as the reference's examples write)
#include <cstdio>
#include <string>

#include "tecs/tecs.hpp"

using namespace tecs;

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  io::HDF5_Writer<DefaultSimulationConfig> w(argv[1]);
  if (argc >= 3) {
    const unsigned steps = static_cast<unsigned>(std::stoul(argv[2]));
    View<VectorN<float, 3>> pos("position", 2);
    for (unsigned s = 0; s < steps; ++s) {
      pos(0) = VectorN<float, 3>(float(s), -float(s), 0.5f * float(s));
      pos(1) = VectorN<float, 3>(1.0f, float(s % 7), -2.0f);
      w.write(0.05 * s, s, pos);
    }
    return 0;
  }
  View<VectorN<float, 3>> pos0("position", 5);
  for (unsigned i = 0; i < 5; ++i) pos0(i) = VectorN<float, 3>(0.5f * i, -1.0f * i, 2.0f + i);
  View<Link> links("links", 3);
  for (unsigned l = 0; l < 3; ++l) links(l) = Link{l, 4 - l};
  w.write(0.0, 0, pos0, links);

  View<VectorN<float, 3>> pos1("position", 7);
  View<Polarity_<float>> pol1("polarity", 7);
  for (unsigned i = 0; i < 7; ++i) {
    pos1(i) = VectorN<float, 3>(1.0f + i, 0.25f * i, -0.5f * i);
    pol1(i) = Polarity_<float>(0.1f * i, -0.2f * i);
  }
  View<Link> no_links("links", 3);
  no_links.set_active_count(0);  // empty views are not written
  w.write(0.05, 1, pos1, pol1, no_links);

  View<float> type("cell_type", 4);
  for (unsigned i = 0; i < 4; ++i) type(i) = float(i % 2);
  w.write_static(type);
  try {
    w.write_static(type);
    return 3;  // a second static write must fail
  } catch (const std::runtime_error&) {
  }
  return 0;
}
