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

// unit vector of the angles (theta, phi): Polarity_::to_vector3, polarity.hpp:111-118
__device__ __forceinline__ void pol_to_vec3(float th, float ph, float* v) {
  const float st = sinf(th);
  v[0] = st * cosf(ph);
  v[1] = st * sinf(ph);
  v[2] = cosf(th);
}

// sin and cos of a polarity's two angles
struct PolTrig {
  float st, ct;  // sin, cos of theta
  float sp, cp;  // sin, cos of phi
};

__device__ __forceinline__ PolTrig pol_trig(float2 p) {
  PolTrig r;
  sincosf(p.x, &r.st, &r.ct);
  sincosf(p.y, &r.sp, &r.cp);
  return r;
}

// p^2 / d^2 rounded to float.  The reference evaluates Kokkos::pow(float, 2)
// in double, so both squares are exact there; here they are kept exact as
// float pairs (hi + lo, the low part from one fused multiply-add) and the
// quotient is corrected once -- double-precision division is slow on this
// part, and the result differs from the double path at most in the last bit.
__device__ __forceinline__ float sq_ratio(float p, float d) {
  const float ph = p * p, pl = fmaf(p, p, -ph);
  const float dh = d * d, dl = fmaf(d, d, -dh);
  const float q = ph / dh;
  const float r = (fmaf(-q, dh, ph) + pl) - q * dl;
  return q + r / dh;
}

// The polarity terms of the pair (self i, other j), each already times k_pol:
//   bv, bp  Polarity_::bending_force(disp, other, dist)   (polarity.hpp:181-198)
//   al      bidirectional_polarization_force(other)       (polarity.hpp:165-168)
// with unidirectional_polarization_force of polarity.hpp:146-157.
__device__ __forceinline__ void polarity_terms(const ForceP& fp, const float* disp, float dist, float2 pi,
                                               const PolTrig& ti, float2 pj, const PolTrig& tj, float* bv, float* bp,
                                               float* al) {
  const float k = fp.k_pol;
  const float tv[3] = {ti.st * ti.cp, ti.st * ti.sp, ti.ct};
  const float ov[3] = {tj.st * tj.cp, tj.st * tj.sp, tj.ct};
  const float prod_i = ((tv[0] * disp[0] + tv[1] * disp[1]) + tv[2] * disp[2]) / dist;
  const float prod_j = ((ov[0] * disp[0] + ov[1] * disp[1]) + ov[2] * disp[2]) / dist;
  const float si = -prod_i / dist, qi = sq_ratio(prod_i, dist);
  const float sj = -prod_j / dist, qj = sq_ratio(prod_j, dist);
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    float t = si * tv[d];
    t = t + qi * disp[d];
    t = t + sj * ov[d];
    t = t + qj * disp[d];
    bv[d] = t * k;
  }
  // the displacement as angles: from_vector3(disp, dist), polarity.hpp:62-66
  const float dth = acosf(fminf(1.0f, fmaxf(-1.0f, disp[2] / dist)));
  const float dph = atan2f(disp[1], disp[0]);
  float sdt, cdt, sdp, cdp;
  sincosf(dth, &sdt, &cdt);
  sincosf(pi.y - dph, &sdp, &cdp);
  const float u0 = ti.ct * sdt * cdp - ti.st * cdt;
  const float u1 = fabsf(ti.st) > kFltEpsilon ? -sdt * sdp / ti.st : 0.0f;
  bp[0] = (-prod_i * u0) * k;
  bp[1] = (-prod_i * u1) * k;
  float sij, cij;
  sincosf(pi.y - pj.y, &sij, &cij);
  const float dot = ti.st * tj.st * cij + ti.ct * tj.ct;
  const float w0 = ti.ct * tj.st * cij - ti.st * tj.ct;
  const float w1 = fabsf(ti.st) > kFltEpsilon ? -tj.st * sij / ti.st : 0.0f;
  al[0] = (dot * w0) * k;
  al[1] = (dot * w1) * k;
}

// spring2r: (displacement * F) / distance, zero at distance 0 (forces/predefined.hpp:134-143)
template <int D>
__device__ __forceinline__ void spring_term(const ForceP& fp, const float* disp, float dist, float* s) {
#pragma unroll
  for (int d = 0; d < D; ++d) s[d] = 0.0f;
  if (dist != 0.0f) {
    const float F = fp.k_rep * fmaxf(fp.r_rep - dist, 0.0f) - fp.k_adh * fmaxf(dist - fp.r_adh, 0.0f);
#pragma unroll
    for (int d = 0; d < D; ++d) s[d] = (disp[d] * F) / dist;
  }
}

// Adds the pair (self, other) force to a in the reference's order: the spring
// term, then the bending vector, then the bending and alignment polarity
// terms.  disp = x_self - x_other, dist = |disp|.
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
    float bv[3], bp[2], al[2];
    polarity_terms(fp, disp, dist, pi, pol_trig(pi), pj, pol_trig(pj), bv, bp, al);
#pragma unroll
    for (int d = 0; d < 3; ++d) a.x[d] = a.x[d] + bv[d];
    a.p[0] = a.p[0] + bp[0];
    a.p[1] = a.p[1] + bp[1];
    a.p[0] = a.p[0] + al[0];
    a.p[1] = a.p[1] + al[1];
  }
}

}  // namespace tecs
