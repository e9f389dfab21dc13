// stencils.cuh -- per-node finite-difference rows of the field sources and recoveries.
//
// Each function evaluates one radial node i (1..nr) of one azimuthal mode m, reading its
// inputs through accessors `F(p, c, i)` (mode part p, component c, node i).  The per-mode
// CTA kernels (fields.cu) pass plain global-memory accessors; the cluster iteration
// kernel (iterate.cu) passes accessors that finish raw deposits on the fly.  Branch order
// follows the reference routines, which matters only for very small nr where the axis
// and edge rows coincide.
#pragma once

#include "qpad_internal.cuh"

namespace qpad {

// Slice field in the f1 layout.
struct GlobalF {
  const double* f;
  int ld, nc;
  __device__ __forceinline__ double operator()(int p, int c, int i) const { return f[fidx(ld, nc, p, c, i)]; }
};

// Deposit finishing (part2d_class.f03:914-1005): node 0 is zero, the axis node is
// multiplied by 8 for the one mode whose on-axis value survives (and zeroed otherwise),
// and node i >= 2 is divided by (i-1).  which: 0 = cu (J_r, J_phi survive for m = 1, J_z
// for m = 0), 1 = amu (m = 2), 2 = acu (m = 1).
__device__ __forceinline__ double finish_amj(const GridDev& G, int m, int which, int c, int i, double raw) {
  if (i == 0) return 0.0;
  if (i == 1) {
    double f;
    if (which == 0) f = c < 2 ? (m == 1 ? 8.0 : 0.0) : (m == 0 ? 8.0 : 0.0);
    else if (which == 1) f = m == 2 ? 8.0 : 0.0;
    else f = m == 1 ? 8.0 : 0.0;
    return f == 0.0 ? 0.0 : f * raw;
  }
  return raw * G.inv[(i) - G.toff];
}

// dJ_perp/dxi (field_src_class.f03:273-405).  m = 0: o[0..1] = dcu(0, 0..1, i);
// m >= 1: o = {dcu(re,0), dcu(re,1), dcu(im,0), dcu(im,1)}.
template <class AF, class UF>
__device__ __forceinline__ void row_djdxi(const GridDev& G, int m, int i, const AF& A_, const UF& U_, double o[4]) {
  const int nr = G.nr;
  const double idr = G.idr, idrh = idr * 0.5, dm = (double)m;
  if (m == 0) {
    if (i == 1) {
      o[0] = 0.0;
      o[1] = 0.0;
    } else if (i == nr) {
      const double ir = G.ir[(nr) - G.toff];
      o[0] = A_(0, 0, nr) + idrh * (4.0 * U_(0, 0, nr - 1) - U_(0, 0, nr - 2) - 3.0 * U_(0, 0, nr)) - ir * U_(0, 0, nr);
      o[1] = A_(0, 1, nr) + idrh * (4.0 * U_(0, 1, nr - 1) - U_(0, 1, nr - 2) - 3.0 * U_(0, 1, nr)) - ir * U_(0, 1, nr);
    } else {
      const double ir = G.ir[(i) - G.toff];
      o[0] = A_(0, 0, i) - idrh * (U_(0, 0, i + 1) - U_(0, 0, i - 1)) - ir * U_(0, 0, i);
      o[1] = A_(0, 1, i) - idrh * (U_(0, 1, i + 1) - U_(0, 1, i - 1)) - ir * U_(0, 1, i);
    }
    return;
  }
  const int r = part_re(m), s = part_im(m);
  if (i == 1) {
    if (m == 1) {
      o[0] = A_(r, 0, 1) - 2.0 * idr * U_(r, 0, 2) + dm * idr * U_(s, 1, 2);
      o[1] = A_(r, 1, 1) - 2.0 * idr * U_(r, 1, 2) + dm * idr * U_(s, 2, 2);
      o[2] = A_(s, 0, 1) - 2.0 * idr * U_(s, 0, 2) - dm * idr * U_(r, 1, 2);
      o[3] = A_(s, 1, 1) - 2.0 * idr * U_(s, 1, 2) - dm * idr * U_(r, 2, 2);
    } else {
      o[0] = o[1] = o[2] = o[3] = 0.0;
    }
  } else if (i == nr) {
    const double ir = G.ir[(nr) - G.toff];
    o[0] = A_(r, 0, nr) + idrh * (4.0 * U_(r, 0, nr - 1) - U_(r, 0, nr - 2) - 3.0 * U_(r, 0, nr)) - ir * U_(r, 0, nr) +
           dm * ir * U_(s, 1, nr);
    o[1] = A_(r, 1, nr) + idrh * (4.0 * U_(r, 1, nr - 1) - U_(r, 1, nr - 2) - 3.0 * U_(r, 1, nr)) - ir * U_(r, 1, nr) +
           dm * ir * U_(s, 2, nr);
    o[2] = A_(s, 0, nr) + idrh * (4.0 * U_(s, 0, nr - 1) - U_(s, 0, nr - 2) - 3.0 * U_(s, 0, nr)) - ir * U_(s, 0, nr) -
           dm * ir * U_(r, 1, nr);
    o[3] = A_(s, 1, nr) + idrh * (4.0 * U_(s, 1, nr - 1) - U_(s, 1, nr - 2) - 3.0 * U_(s, 1, nr)) - ir * U_(s, 1, nr) -
           dm * ir * U_(r, 2, nr);
  } else if (i == 2 && m == 2) {
    const double ir = idr;
    o[0] = A_(r, 0, 2) - idr * (U_(r, 0, 3) - U_(r, 0, 2)) - ir * U_(r, 0, 2) + dm * ir * U_(s, 1, 2);
    o[1] = A_(r, 1, 2) - idr * (U_(r, 1, 3) - U_(r, 1, 2)) - ir * U_(r, 1, 2) + dm * ir * U_(s, 2, 2);
    o[2] = A_(s, 0, 2) - idr * (U_(s, 0, 3) - U_(s, 0, 2)) - ir * U_(s, 0, 2) - dm * ir * U_(r, 1, 2);
    o[3] = A_(s, 1, 2) - idr * (U_(s, 1, 3) - U_(s, 1, 2)) - ir * U_(s, 1, 2) - dm * ir * U_(r, 2, 2);
  } else {
    const double ir = G.ir[(i) - G.toff];
    o[0] = A_(r, 0, i) - idrh * (U_(r, 0, i + 1) - U_(r, 0, i - 1)) - ir * U_(r, 0, i) + dm * ir * U_(s, 1, i);
    o[1] = A_(r, 1, i) - idrh * (U_(r, 1, i + 1) - U_(r, 1, i - 1)) - ir * U_(r, 1, i) + dm * ir * U_(s, 2, i);
    o[2] = A_(s, 0, i) - idrh * (U_(s, 0, i + 1) - U_(s, 0, i - 1)) - ir * U_(s, 0, i) - dm * ir * U_(r, 1, i);
    o[3] = A_(s, 1, i) - idrh * (U_(s, 1, i + 1) - U_(s, 1, i - 1)) - ir * U_(s, 1, i) - dm * ir * U_(r, 2, i);
  }
}

// Right-hand sides of the B-perp predictor-corrector (field_b_class.f03:360-506,
// 703-758): relaxation terms included.  m = 0: o[0..1] = (B+, B-) rows (real);
// m >= 1: o = {B+ re, B+ im, B- re, B- im}.  DC reads dcu, CU reads cu, BO the B_old.
template <class DF, class CF, class BF>
__device__ __forceinline__ void row_btiter_src(const GridDev& G, int m, int i, const DF& DC, const CF& CU,
                                               const BF& BO, double o[4]) {
  const int nr = G.nr;
  const double idr = G.idr, idrh = 0.5 * idr, rix = G.relax_fac * (idr * idr), dm = (double)m;
  if (m == 0) {
    if (i == 1) {
      o[0] = 0.0;
      o[1] = 0.0;
    } else if (i == nr) {
      o[0] = -DC(0, 1, nr) - BO(0, 0, nr) * rix;
      o[1] = DC(0, 0, nr) + idrh * (3.0 * CU(0, 2, nr) - 4.0 * CU(0, 2, nr - 1) + CU(0, 2, nr - 2)) - BO(0, 1, nr) * rix;
    } else if (i == 2) {
      o[0] = -DC(0, 1, 2) - BO(0, 0, 2) * rix;
      o[1] = DC(0, 0, 2) + idr * (CU(0, 2, 3) - CU(0, 2, 2)) - BO(0, 1, 2) * rix;
    } else {
      o[0] = -DC(0, 1, i) - BO(0, 0, i) * rix;
      o[1] = DC(0, 0, i) + idrh * (CU(0, 2, i + 1) - CU(0, 2, i - 1)) - BO(0, 1, i) * rix;
    }
    return;
  }
  const int pr = part_re(m), pi = part_im(m);
  double s1re, s1im, s2re, s2im;
  if (i == 1) {
    if (m == 1) {
      s1re = -DC(pr, 1, 1) + idr * dm * CU(pi, 2, 2);
      s1im = -DC(pi, 1, 1) - idr * dm * CU(pr, 2, 2);
      s2re = DC(pr, 0, 1) + idr * CU(pr, 2, 2);
      s2im = DC(pi, 0, 1) + idr * CU(pi, 2, 2);
    } else if (m % 2 == 0) {
      s1re = s1im = s2re = s2im = 0.0;
    } else {
      s1re = idr * dm * CU(pi, 2, 2);
      s1im = idr * dm * CU(pr, 2, 2);
      s2re = idr * CU(pr, 2, 2);
      s2im = idr * CU(pi, 2, 2);
    }
  } else if (i == nr) {
    const double ir = G.ir[(nr) - G.toff];
    s1re = -DC(pr, 1, nr) + dm * CU(pi, 2, nr) * ir;
    s1im = -DC(pi, 1, nr) - dm * CU(pr, 2, nr) * ir;
    s2re = DC(pr, 0, nr) + idrh * (3.0 * CU(pr, 2, nr) - 4.0 * CU(pr, 2, nr - 1) + CU(pr, 2, nr - 2));
    s2im = DC(pi, 0, nr) + idrh * (3.0 * CU(pi, 2, nr) - 4.0 * CU(pi, 2, nr - 1) + CU(pi, 2, nr - 2));
  } else {
    const double ir = G.ir[(i) - G.toff];
    s1re = -DC(pr, 1, i) + dm * CU(pi, 2, i) * ir;
    s1im = -DC(pi, 1, i) - dm * CU(pr, 2, i) * ir;
    s2re = DC(pr, 0, i) + idrh * (CU(pr, 2, i + 1) - CU(pr, 2, i - 1));
    s2im = DC(pi, 0, i) + idrh * (CU(pi, 2, i + 1) - CU(pi, 2, i - 1));
  }
  const double br0 = BO(pr, 0, i), bi0 = BO(pi, 0, i);
  const double br1 = BO(pr, 1, i), bi1 = BO(pi, 1, i);
  o[0] = s1re - s2im - (br0 - bi1) * rix;
  o[1] = s1im + s2re - (bi0 + br1) * rix;
  o[2] = s1re + s2im - (br0 + bi1) * rix;
  o[3] = s1im - s2re - (bi0 - br1) * rix;
}

// Bz right-hand side (field_b_class.f03:205-307); im = 0 for m = 0.
template <class CF>
__device__ __forceinline__ void row_bz_src(const GridDev& G, int m, int i, const CF& CU, double& re, double& im) {
  const int nr = G.nr;
  const double idr = G.idr, idrh = 0.5 * idr;
  if (m == 0) {
    if (i == 1) {
      re = -2.0 * idr * CU(0, 1, 2);
    } else if (i == nr) {
      const double ir = G.ir[(nr) - G.toff];
      re = -idrh * (3.0 * CU(0, 1, nr) - 4.0 * CU(0, 1, nr - 1) + CU(0, 1, nr - 2)) - ir * CU(0, 1, nr);
    } else {
      const double ir = G.ir[(i) - G.toff];
      re = -idrh * (CU(0, 1, i + 1) - CU(0, 1, i - 1)) - ir * CU(0, 1, i);
    }
    im = 0.0;
    return;
  }
  const int pr = part_re(m), pi = part_im(m);
  const double dm = (double)m;
  if (i == nr) {
    const double ir = G.ir[(nr) - G.toff];
    re = -idrh * (3.0 * CU(pr, 1, nr) - 4.0 * CU(pr, 1, nr - 1) + CU(pr, 1, nr - 2)) - ir * CU(pr, 1, nr) -
         dm * ir * CU(pi, 0, nr);
    im = -idrh * (3.0 * CU(pi, 1, nr) - 4.0 * CU(pi, 1, nr - 1) + CU(pi, 1, nr - 2)) - ir * CU(pi, 1, nr) +
         dm * ir * CU(pr, 0, nr);
  } else if (i == 1) {
    if (m % 2 == 0) {
      re = -2.0 * idr * CU(pr, 1, 2) - dm * idr * CU(pi, 0, 2);
      im = -2.0 * idr * CU(pi, 1, 2) + dm * idr * CU(pr, 0, 2);
    } else {
      re = 0.0;
      im = 0.0;
    }
  } else if (i == 2 && m == 1) {
    const double ir = idr;
    re = -idr * (CU(pr, 1, 3) - CU(pr, 1, 2)) - ir * CU(pr, 1, 2) - dm * ir * CU(pi, 0, 2);
    im = -idr * (CU(pi, 1, 3) - CU(pi, 1, 2)) - ir * CU(pi, 1, 2) + dm * ir * CU(pr, 0, 2);
  } else {
    const double ir = G.ir[(i) - G.toff];
    re = -idrh * (CU(pr, 1, i + 1) - CU(pr, 1, i - 1)) - ir * CU(pr, 1, i) - dm * ir * CU(pi, 0, i);
    im = -idrh * (CU(pi, 1, i + 1) - CU(pi, 1, i - 1)) - ir * CU(pi, 1, i) + dm * ir * CU(pr, 0, i);
  }
}

// Ez right-hand side (field_e_class.f03:148-259).  m = 0: re is the row value, the axis
// row (i = 1) is set afterwards from the weighted sum of the rows flagged `in_div`
// (the reference's MPI_REDUCE, :298-334); im = 0.
template <class CF>
__device__ __forceinline__ void row_ez_src(const GridDev& G, int m, int i, const CF& CU, double& re, double& im,
                                           bool& in_div) {
  const int nr = G.nr;
  const double idr = G.idr, idrh = 0.5 * idr, dm = (double)m;
  in_div = false;
  if (m == 0) {
    im = 0.0;
    if (i == 1) {
      re = 0.0;
    } else if (i == nr - 1) {
      const double ir = G.ir[(nr - 1) - G.toff];
      re = idrh * (CU(0, 0, nr) - CU(0, 0, nr - 2)) + ir * CU(0, 0, nr - 1);
    } else if (i == nr) {
      const double ir = G.ir[(nr) - G.toff];
      re = idr * (CU(0, 0, nr) - CU(0, 0, nr - 1)) + ir * CU(0, 0, nr);
    } else {
      const double ir = G.ir[(i) - G.toff];
      re = idrh * (CU(0, 0, i + 1) - CU(0, 0, i - 1)) + ir * CU(0, 0, i);
      in_div = true;
    }
    return;
  }
  const int pr = part_re(m), pi = part_im(m);
  if (i == nr) {
    const double ir = G.ir[(nr) - G.toff];
    re = idrh * (3.0 * CU(pr, 0, nr) - 4.0 * CU(pr, 0, nr - 1) + CU(pr, 0, nr - 2)) + ir * CU(pr, 0, nr) -
         dm * ir * CU(pi, 1, nr);
    im = idrh * (3.0 * CU(pi, 0, nr) - 4.0 * CU(pi, 0, nr - 1) + CU(pi, 0, nr - 2)) + ir * CU(pi, 0, nr) +
         dm * ir * CU(pr, 1, nr);
  } else if (i == 1) {
    if (m % 2 == 0) {
      re = 2.0 * idr * CU(pr, 0, 2) - dm * idr * CU(pi, 1, 2);
      im = 2.0 * idr * CU(pi, 0, 2) + dm * idr * CU(pr, 1, 2);
    } else {
      re = 0.0;
      im = 0.0;
    }
  } else if (i == 2 && m == 1) {
    const double ir = idr;
    re = idr * (CU(pr, 0, 3) - CU(pr, 0, 2)) + ir * CU(pr, 0, 2) - dm * ir * CU(pi, 1, 2);
    im = idr * (CU(pi, 0, 3) - CU(pi, 0, 2)) + ir * CU(pi, 0, 2) + dm * ir * CU(pr, 1, 2);
  } else {
    const double ir = G.ir[(i) - G.toff];
    re = idrh * (CU(pr, 0, i + 1) - CU(pr, 0, i - 1)) + ir * CU(pr, 0, i) - dm * ir * CU(pi, 1, i);
    im = idrh * (CU(pi, 0, i + 1) - CU(pi, 0, i - 1)) + ir * CU(pi, 0, i) + dm * ir * CU(pr, 1, i);
  }
}

// The m = 0 axis row of Ez from the sum of the flagged rows (field_e_class.f03:298-334).
template <class CF>
__device__ __forceinline__ double ez_axis_row(const GridDev& G, double div, const CF& CU) {
  const int nr = G.nr;
  div = div - 0.5 * G.idr * (CU(0, 0, nr - 2) + CU(0, 0, nr - 1)) * ((double)nr - 2.5);
  return -8.0 * div;
}

// E-perp from B and psi (field_e_class.f03:412-514).  m = 0: o[0..1] = (E_r, E_phi) of
// part 0; m >= 1: o = {E_r re, E_r im, E_phi re, E_phi im}.
template <class BF, class PF>
__device__ __forceinline__ void row_et(const GridDev& G, int m, int i, const BF& B, const PF& PS, double o[4]) {
  const int nr = G.nr;
  const double idr = G.idr, idrh = idr * 0.5, dm = (double)m;
  if (m == 0) {
    if (i == 1) {
      o[0] = 0.0;
      o[1] = 0.0;
    } else if (i == nr) {
      o[0] = B(0, 1, nr) + idrh * (4.0 * PS(0, 0, nr - 1) - PS(0, 0, nr - 2) - 3.0 * PS(0, 0, nr));
      o[1] = -B(0, 0, nr);
    } else {
      o[0] = B(0, 1, i) - idrh * (PS(0, 0, i + 1) - PS(0, 0, i - 1));
      o[1] = -B(0, 0, i);
    }
    return;
  }
  const int pr = part_re(m), pi = part_im(m);
  if (i == 1) {
    if (m == 1) {
      o[0] = B(pr, 1, 1) - idr * PS(pr, 0, 2);
      o[1] = B(pi, 1, 1) - idr * PS(pi, 0, 2);
      o[2] = -B(pr, 0, 1) + idr * PS(pi, 0, 2);
      o[3] = -B(pi, 0, 1) - idr * PS(pr, 0, 2);
    } else {
      o[0] = o[1] = o[2] = o[3] = 0.0;
    }
    return;
  }
  const double ir = G.ir[(i) - G.toff];
  if (i == nr) {
    o[0] = B(pr, 1, nr) + idrh * (4.0 * PS(pr, 0, nr - 1) - PS(pr, 0, nr - 2) - 3.0 * PS(pr, 0, nr));
    o[1] = B(pi, 1, nr) + idrh * (4.0 * PS(pi, 0, nr - 1) - PS(pi, 0, nr - 2) - 3.0 * PS(pi, 0, nr));
  } else {
    o[0] = B(pr, 1, i) - idrh * (PS(pr, 0, i + 1) - PS(pr, 0, i - 1));
    o[1] = B(pi, 1, i) - idrh * (PS(pi, 0, i + 1) - PS(pi, 0, i - 1));
  }
  o[2] = -B(pr, 0, i) + ir * dm * PS(pi, 0, i);
  o[3] = -B(pi, 0, i) - ir * dm * PS(pr, 0, i);
}

// convergence_tester (simulation_class.f03:522-606), one node i: the record is the
// per-node sum over modes of |b(comp)| for the Re and the Im parts; with `compare` the
// squared distance of the old record from the new one (accumulated by the same sequential
// subtraction) and the squared old record are folded into the running maxima.
template <class BF>
__device__ __forceinline__ void conv_node_v(const GridDev& G, const BF& B, int comp, int i, double ore, double oim,
                                            bool compare, double& nre, double& nim, double& mx_old, double& mx_new) {
  nre = 0.0;
  nim = 0.0;
  if (compare) mx_old = fmax(mx_old, ore * ore + oim * oim);
  for (int m = 0; m <= G.M; ++m) {
    const double vr = fabs(B(part_re(m), comp, i));
    nre = nre + vr;
    if (compare) ore = ore - vr;
    if (m == 0) continue;
    const double vi = fabs(B(part_im(m), comp, i));
    nim = nim + vi;
    if (compare) oim = oim - vi;
  }
  if (compare) mx_new = fmax(mx_new, ore * ore + oim * oim);
}

template <class BF>
__device__ __forceinline__ void conv_node(const GridDev& G, const BF& B, int comp, int i, double* s_re, double* s_im,
                                          bool compare, double& mx_old, double& mx_new) {
  double nre, nim;
  conv_node_v(G, B, comp, i, s_re[i - 1], s_im[i - 1], compare, nre, nim, mx_old, mx_new);
  s_re[i - 1] = nre;
  s_im[i - 1] = nim;
}

// ---- binomial smoothing of the species deposits (ufield::smooth_f1, ufield_class.f03:274-339)
// Deposit kinds: 0 rho (1 comp), 1 jay (cu and amu, 3 comps), 2 djdxi (the acu deposit, 2).
// Whether node 1 takes the axis form for mode m and component c (field_src_class.f03:114-118,
// 181-193, 256-266).
__host__ __device__ inline bool smooth_ax(int kind, int m, int c) {
  if (kind == 0) return m == 0;
  if (kind == 1) return m == 0 ? c == 2 : (m == 1 && c < 2);
  return m == 1;
}

// One pass at node i (1..nr) from the values at i-1, i, i+1 (single rank: node 1 the axis
// form or 0, node 2 the near-axis form, nodes >= 3 the r-weighted form with r = i - 1);
// kernel = (1, 2, 1) / 4.
__device__ __forceinline__ double smooth_node(const GridDev& G, int i, bool ax, double vm, double v0, double vp) {
  const double km = 0.25, k0 = 0.5, kp = 0.25;
  if (i == 1) return ax ? (k0 + kp) * v0 + 8.0 * kp * vp : 0.0;
  if (i == 2) return k0 * v0 + 0.125 * km * vm + 2.0 * kp * vp;
  const double ir = G.inv[(i) - G.toff];
  return k0 * v0 + (1.0 - ir) * km * vm + (1.0 + ir) * kp * vp;
}

// A deposit component after `order` (<= 2) smoothing passes, at node i, computed from an
// unsmoothed accessor F(p, c, i) (guard nodes 0 and nr + 1 are not smoothed).
template <class FF>
__device__ double smoothed_at(const GridDev& G, const FF& F, int kind, int m, int p, int c, int i, int order) {
  const bool ax = smooth_ax(kind, m, c);
  const auto s1 = [&](int k) {
    if (k < 1 || k > G.nr) return F(p, c, k);
    return smooth_node(G, k, ax, F(p, c, k - 1), F(p, c, k), F(p, c, k + 1));
  };
  if (order <= 0 || i < 1 || i > G.nr) return F(p, c, i);
  if (order == 1) return s1(i);
  return smooth_node(G, i, ax, s1(i - 1), s1(i), s1(i + 1));
}

// The decision from the maxima over nodes: relative and absolute residuals, convergence,
// and the loop state (iteration count, statistics, WHILE condition).  One thread.
__device__ inline void conv_decide_at(double mx_old, double mx_new, double reltol, double abstol, double* res,
                                      const ConvLoop& L, int it_prev, int jp) {
  const double old_norm = sqrt(mx_old), abs_res = sqrt(mx_new);
  const double rel = old_norm > 2.220446049250313e-16 ? abs_res / old_norm : 1.7976931348623157e308;
  const bool converged = rel < reltol || abs_res < abstol;
  res[0] = rel;
  res[1] = abs_res;
  res[2] = converged ? 1.0 : 0.0;
  if (L.iter_ctr) {
    const int it = it_prev + 1;
    *L.iter_ctr = it;
    if (L.stats && L.jp) {
      qpad_slice_stats s;
      s.iters = it;
      s.rel_res = rel;
      s.abs_res = abs_res;
      L.stats[jp - 1] = s;
    }
    const bool more = !converged && it < L.iter_max;
    if (L.use_h) cudaGraphSetConditional(L.h, more ? 1u : 0u);
    if (L.stop) *L.stop = more ? 0 : 1;
  }
}

__device__ inline void conv_decide(double mx_old, double mx_new, double reltol, double abstol, double* res,
                                   const ConvLoop& L) {
  conv_decide_at(mx_old, mx_new, reltol, abstol, res, L, L.iter_ctr ? *L.iter_ctr : 0,
                 (L.iter_ctr && L.stats && L.jp) ? *L.jp : 1);
}

}  // namespace qpad
