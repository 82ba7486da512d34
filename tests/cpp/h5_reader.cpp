// h5_reader.cpp -- io::HDF5_Reader of the drop-in layer: reads the named
// dataset of an HDF5 file into a view of the given kind and writes its
// values as raw float32 (vec3, polarity, float) or int32 (int) rows.
//
//   h5_reader <file.h5> <dataset> <vec3|polarity|float|int> <out.bin>
// prints the dataset's dimensions.
#include <cstdio>
#include <string>

#include "tecs/tecs.hpp"

using namespace tecs;

template <typename T>
static int dump(const io::HDF5_Reader& r, const std::string& name, const char* out) {
  const auto dims = r.get_dataset_dimensions(name);
  View<T> v("values", static_cast<unsigned>(dims.at(0)));
  r.read_dataset(name, v);
  FILE* f = std::fopen(out, "wb");
  if (!f) return 2;
  std::fwrite(v.data(), sizeof(T), dims[0], f);
  std::fclose(f);
  for (std::size_t d : dims) std::printf("%zu ", d);
  std::printf("\n");
  return 0;
}

int main(int argc, char** argv) {
  if (argc < 5) return 2;
  try {
    const io::HDF5_Reader r(argv[1]);
    const std::string kind = argv[3];
    if (kind == "vec3") return dump<VectorN<float, 3>>(r, argv[2], argv[4]);
    if (kind == "polarity") return dump<Polarity_<float>>(r, argv[2], argv[4]);
    if (kind == "float") return dump<float>(r, argv[2], argv[4]);
    if (kind == "int") return dump<int>(r, argv[2], argv[4]);
  } catch (const std::exception& e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 1;
  }
  return 2;
}
