// qsf_borders.h -- host-side border vectors of the flux observables.
//
// Restates the reference's outward border vectors (fluxes/borders_g.h:1-40,
// fluxes/borders_t.h:1-13, fluxes/borders.h:39-257) as plain functions of the
// centred node indices.  The library evaluates them once per grid and border set to
// build the sparse list of points where a border vector is non-zero; the GPU then
// only touches those points.  Node positions p_NS, p_SD, p_DT, p_CAP are the
// reference's mutable globals (borders.h:30-36), kept per grid here.
#pragma once
#include <cmath>
#include <cstdint>
#include <initializer_list>

namespace qsf {

struct BorderNodes {
  int64_t NS = 25, SD = 14, DT = 10, CAP = 40;
};

namespace bd {
inline double sgn(int64_t x) { return (double)((x > 0) - (x < 0)); }
inline bool rn(int64_t i, int64_t il, int64_t ir) { return i >= il && i < ir; }
inline bool rn2(int64_t i, int64_t il, int64_t ir) { return rn(i, il, ir) || rn(i, -ir, -il); }
inline double point_b(int64_t i, int64_t iat) { return i == iat - 1 ? sgn(i) : 0; }
inline double point_b2(int64_t i, int64_t iat) { return (i == iat - 1 || i == -iat) ? sgn(i) : 0; }
inline double seg_b(int64_t i, int64_t j, int64_t jat, int64_t il, int64_t ir) { return rn(i, il, ir) ? point_b(j, jat) : 0; }
inline double seg_i2j2(int64_t i, int64_t j, int64_t jat, int64_t il, int64_t ir) {
  return rn2(i, il, ir) ? point_b2(j, jat) : 0;
}
inline double patch_i2j2k2(int64_t i, int64_t j, int64_t k, int64_t kat, int64_t il, int64_t ir, int64_t jl, int64_t jr) {
  return rn2(i, il, ir) ? (rn2(j, jl, jr) ? point_b2(k, kat) : 0) : 0;
}
}  // namespace bd

// Normalised border vector of `type` (QSF_B_*) at centred indices ci[0..dim).
// Returns false when the type is not defined for this dimension.
inline bool border_vector(int type, int64_t box, int dim, const int64_t* ci, const BorderNodes& B, double* out) {
  using namespace bd;
  const int64_t i = ci[0], j = dim > 1 ? ci[1] : 0, k = dim > 2 ? ci[2] : 0;
  const int64_t NS = B.NS, SD = B.SD, DT = B.DT, CAP = B.CAP;
  out[0] = out[1] = out[2] = 0.0;
  auto sym3 = [&](int64_t kat, int64_t il, int64_t ir, int64_t jl, int64_t jr) {
    out[0] = patch_i2j2k2(j, k, i, kat, il, ir, jl, jr) + patch_i2j2k2(k, j, i, kat, il, ir, jl, jr);
    out[1] = patch_i2j2k2(k, i, j, kat, il, ir, jl, jr) + patch_i2j2k2(i, k, j, kat, il, ir, jl, jr);
    out[2] = patch_i2j2k2(i, j, k, kat, il, ir, jl, jr) + patch_i2j2k2(j, i, k, kat, il, ir, jl, jr);
  };
  auto plain3 = [&](int64_t kat, int64_t il, int64_t ir, int64_t jl, int64_t jr) {
    out[0] = patch_i2j2k2(j, k, i, kat, il, ir, jl, jr);
    out[1] = patch_i2j2k2(k, i, j, kat, il, ir, jl, jr);
    out[2] = patch_i2j2k2(i, j, k, kat, il, ir, jl, jr);
  };
  auto seg2 = [&](int64_t at, int64_t il, int64_t ir) {
    out[0] = seg_i2j2(j, i, at, il, ir);
    out[1] = seg_i2j2(i, j, at, il, ir);
  };
  switch (type) {
    case 0:  // BOX<size>
      if (dim == 1) out[0] = point_b2(i, box);
      else if (dim == 2) seg2(box, 0, box);
      else plain3(box, 0, box, 0, box);
      break;
    case 1:  // S2CAP
      if (dim == 2) seg2(CAP, 0, SD);
      else if (dim == 3) sym3(CAP, 0, DT, 0, SD);
      else return false;
      break;
    case 2:  // D2CAP
      if (dim == 2) seg2(CAP, SD, CAP);
      else if (dim == 3) sym3(CAP, SD, CAP, 0, DT);
      else return false;
      break;
    case 3:  // N2S
      if (dim == 2) seg2(NS, 0, SD);
      else if (dim == 3) sym3(NS, 0, SD, 0, DT - 1);
      else return false;
      break;
    case 4:  // N2D
      if (dim == 2) seg2(SD, SD, NS);
      else if (dim == 3) sym3(SD, SD, NS, 0, DT - 1);
      else return false;
      break;
    case 5:  // N2D_SYM (2e only)
      if (dim != 2) return false;
      out[0] = seg_b(j + 1, i, SD, SD, NS + 1) - seg_b(-j, -i - 1, SD, SD, NS + 1);
      out[1] = seg_b(i + 1, j, SD, SD, NS + 1) - seg_b(-i, -j - 1, SD, SD, NS + 1);
      break;
    case 6:  // N2D_ASYM
      if (dim != 2) return false;
      out[0] = -seg_b(j + 1, -i - 1, SD, SD, NS + 1) + seg_b(-j, i, SD, SD, NS + 1);
      out[1] = -seg_b(i + 1, -j - 1, SD, SD, NS + 1) + seg_b(-i, j, SD, SD, NS + 1);
      break;
    case 7:  // S2D
      if (dim == 2) seg2(SD, NS, CAP);
      else if (dim == 3) sym3(SD, NS, CAP, 0, DT);
      else return false;
      break;
    case 8:  // S2D_SYM
      if (dim != 2) return false;
      out[0] = seg_b(j, i, SD, NS, CAP) - seg_b(-j - 1, -i - 1, SD, NS, CAP);
      out[1] = seg_b(i, j, SD, NS, CAP) - seg_b(-i - 1, -j - 1, SD, NS, CAP);
      break;
    case 9:  // S2D_ASYM
      if (dim != 2) return false;
      out[0] = -seg_b(j, -i - 1, SD, NS, CAP) + seg_b(-j - 1, i, SD, NS, CAP);
      out[1] = -seg_b(i, -j - 1, SD, NS, CAP) + seg_b(-i - 1, j, SD, NS, CAP);
      break;
    case 10:  // N2T (3e only)
      if (dim != 3) return false;
      sym3(DT, DT - 1, NS, DT - 1, SD);
      break;
    case 11:  // S2T
      if (dim != 3) return false;
      sym3(DT, NS, CAP, DT, SD);
      break;
    case 12:  // D2T
      if (dim != 3) return false;
      plain3(DT, SD, CAP, SD, CAP);
      break;
    case 13:  // T2CAP
      if (dim != 3) return false;
      plain3(CAP, DT, CAP, DT, CAP);
      break;
    default:
      return false;
  }
  // borVec normalisation (borders_t.h:6-13)
  double s = 0.0;
  for (int d = 0; d < dim; ++d) s += out[d] * out[d];
  const double nrm = std::sqrt(s + 0.0);
  if (nrm > 0.001)
    for (int d = 0; d < dim; ++d) out[d] /= nrm;
  return true;
}

// Largest |centred index| at which a border of this set can be non-zero.
inline int64_t border_reach(const BorderNodes& B, int64_t box) {
  int64_t r = box;
  for (int64_t v : {B.NS, B.SD, B.DT, B.CAP}) r = v > r ? v : r;
  return r + 2;
}

}  // namespace qsf
