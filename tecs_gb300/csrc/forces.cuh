// forces.cuh -- built-in pairwise force laws evaluated inside the pass kernels.
//
// spring2r: include/forces/predefined.hpp:107-144 (PiecewiseLinear) with
//           separate repulsion / adhesion radii; displacement * F / distance.
// polarity: include/types/polarity.hpp:131-198 (dot, unidirectional and
//           bidirectional polarization force, bending_force), scaled by k_pol.
// Operation order mirrors the reference's VectorN expressions.
#pragma once

#include "common.cuh"

namespace tecs {

struct Acc {
  float x[3];
  float p[2];
};

__device__ __forceinline__ void pol_to_vec3(float th, float ph, float* v) {
  float st = sinf(th);
  v[0] = st * cosf(ph);
  v[1] = st * sinf(ph);
  v[2] = cosf(th);
}

// polarity.hpp:146-157
__device__ __forceinline__ void unidirectional(float th, float ph, float oth, float oph, float* r) {
  r[0] = cosf(th) * sinf(oth) * cosf(ph - oph) - sinf(th) * cosf(oth);
  r[1] = 0.0f;
  float s = sinf(th);
  if (fabsf(s) > kFltEpsilon) r[1] = -sinf(oth) * sinf(ph - oph) / s;
}

// Adds the pair (self, other) force to a; disp = x_self - x_other, dist = |disp| (dist > 0 not required).
template <int D, int FORCE>
__device__ __forceinline__ void pair_force(const ForceP& fp, const float* disp, float dist, float2 pi, float2 pj,
                                           Acc& a) {
  if (FORCE == 0) return;
  if (dist != 0.0f) {
    float F = fp.k_rep * fmaxf(fp.r_rep - dist, 0.0f) - fp.k_adh * fmaxf(dist - fp.r_adh, 0.0f);
#pragma unroll
    for (int d = 0; d < D; ++d) a.x[d] = a.x[d] + (disp[d] * F) / dist;
  }
  if (FORCE == 2 && D == 3) {
    const float k = fp.k_pol;
    float tv[3], ov[3];
    pol_to_vec3(pi.x, pi.y, tv);
    float prod_i = ((tv[0] * disp[0] + tv[1] * disp[1]) + tv[2] * disp[2]) / dist;
    pol_to_vec3(pj.x, pj.y, ov);
    float prod_j = ((ov[0] * disp[0] + ov[1] * disp[1]) + ov[2] * disp[2]) / dist;
    // Kokkos::pow(float, int) is evaluated in double; the quotient is narrowed on use.
    double dd = (double)dist * (double)dist;
    float si = -prod_i / dist;
    float qi = (float)(((double)prod_i * (double)prod_i) / dd);
    float sj = -prod_j / dist;
    float qj = (float)(((double)prod_j * (double)prod_j) / dd);
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      float t = si * tv[d];
      t = t + qi * disp[d];
      t = t + sj * ov[d];
      t = t + qj * disp[d];
      a.x[d] = a.x[d] + t * k;
    }
    // from_vector3(disp, dist), polarity.hpp:62-66
    float q = disp[2] / dist;
    float dth = acosf(fminf(1.0f, fmaxf(-1.0f, q)));
    float dph = atan2f(disp[1], disp[0]);
    float uni[2];
    unidirectional(pi.x, pi.y, dth, dph, uni);
    a.p[0] = a.p[0] + (-prod_i * uni[0]) * k;
    a.p[1] = a.p[1] + (-prod_i * uni[1]) * k;
    // bidirectional_polarization_force, polarity.hpp:165-168
    float dot = sinf(pi.x) * sinf(pj.x) * cosf(pi.y - pj.y) + cosf(pi.x) * cosf(pj.x);
    float u2[2];
    unidirectional(pi.x, pi.y, pj.x, pj.y, u2);
    a.p[0] = a.p[0] + (dot * u2[0]) * k;
    a.p[1] = a.p[1] + (dot * u2[1]) * k;
  }
}

}  // namespace tecs
