// force_laws.cu -- the drop-in layer's predefined force functions
// (include/tecs/components.hpp, namespace tecs::forces) evaluated at a table
// of distances and displacements, with the parameters the reference-run
// fixture tests/golden/laws_predefined.npz used.  Built by g++ (as C++) the
// functions run on the host; built by nvcc they run in a kernel on the GPU.
//
//   force_laws <in.bin> <out.bin>
//   in:  uint32 m, float32 d[m], float32 disp[m*3]
//   out: float32 [m][28]: 7 magnitudes, then 7 vectors (x, y, z), in the order
//        Spring, PiecewiseLinear, PiecewiseQuadratic, Cubic, Morse,
//        LennardJones, HertzContact
#include <cstdio>
#include <vector>

#include "tecs/components.hpp"

using Vector = tecs::VectorN<float, 3>;

TECS_HD inline void evaluate(float r, const float* dv, float* o) {
  namespace F = tecs::forces;
  const Vector v{dv[0], dv[1], dv[2]};
  o[0] = F::SpringPotential(r, 1.0f, 0.5f);
  o[1] = F::PiecewiseLinearPotential(r, 0.8f, 1.5f, 0.3f);
  o[2] = F::PiecewiseQuadraticPotential(r, 1.0f, 1.4f, 1.8f, 2.0f, 0.7f);
  o[3] = F::CubicPotential(r, 1.0f, 1.6f, 3.0f);
  o[4] = F::MorsePotential(r, 1.0f, 2.0f, 0.25f);
  o[5] = F::LennardJonesPotential(r, 0.9f, 1.1f, 0.5f);
  o[6] = F::HertzContactPotential(r, 0.6f, 0.7f, 2.0f, 3.0f, 0.3f, 0.4f);
  const Vector w[7] = {F::Spring(v, r, 1.0f, 0.5f),
                       F::PiecewiseLinear(v, r, 0.8f, 1.5f, 0.3f),
                       F::PiecewiseQuadratic(v, r, 1.0f, 1.4f, 1.8f, 2.0f, 0.7f),
                       F::Cubic(v, r, 1.0f, 1.6f, 3.0f),
                       F::Morse(v, r, 1.0f, 2.0f, 0.25f),
                       F::LennardJones(v, r, 0.9f, 1.1f, 0.5f),
                       F::HertzContact(v, r, 0.6f, 0.7f, 2.0f, 3.0f, 0.3f, 0.4f)};
  for (int l = 0; l < 7; ++l)
    for (int c = 0; c < 3; ++c) o[7 + 3 * l + c] = w[l][c];
}

#if defined(__CUDACC__)
__global__ void k_laws(unsigned m, const float* d, const float* disp, float* out) {
  const unsigned k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < m) evaluate(d[k], disp + 3 * k, out + 28 * (size_t)k);
}
#endif

int main(int argc, char** argv) {
  if (argc < 3) return 2;
  FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 2;
  unsigned m = 0;
  if (std::fread(&m, 4, 1, f) != 1) return 2;
  std::vector<float> d(m), disp(3 * (size_t)m), out(28 * (size_t)m);
  if (std::fread(d.data(), 4, m, f) != m || std::fread(disp.data(), 4, disp.size(), f) != disp.size()) return 2;
  std::fclose(f);
#if defined(__CUDACC__)
  float *dd = nullptr, *ddisp = nullptr, *dout = nullptr;
  if (cudaMalloc(&dd, d.size() * 4) || cudaMalloc(&ddisp, disp.size() * 4) || cudaMalloc(&dout, out.size() * 4))
    return 3;
  cudaMemcpy(dd, d.data(), d.size() * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(ddisp, disp.data(), disp.size() * 4, cudaMemcpyHostToDevice);
  k_laws<<<(m + 127) / 128, 128>>>(m, dd, ddisp, dout);
  if (cudaMemcpy(out.data(), dout, out.size() * 4, cudaMemcpyDeviceToHost) != cudaSuccess) return 3;
  cudaFree(dd);
  cudaFree(ddisp);
  cudaFree(dout);
#else
  for (unsigned k = 0; k < m; ++k) evaluate(d[k], &disp[3 * (size_t)k], &out[28 * (size_t)k]);
#endif
  FILE* g = std::fopen(argv[2], "wb");
  if (!g) return 2;
  std::fwrite(out.data(), 4, out.size(), g);
  std::fclose(g);
  return 0;
}
