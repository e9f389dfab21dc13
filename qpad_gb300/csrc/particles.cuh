// particles.cuh -- device helpers shared by the plasma and beam particle kernels.
#pragma once

#include "qpad_internal.cuh"

namespace qpad {

// Radius with the reference's rounding (no FMA contraction): sqrt(x*x + y*y).  Cell
// indices and the edge test depend on it, so they are reproduced bit for bit.
__device__ __forceinline__ double radius_rn(double x, double y) {
  return __dsqrt_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)));
}

// gen_interp_info (interp_part2d.f03:28-65).  ok == false marks a particle whose
// normalised radius falls outside [0, nr): it gathers zero fields and deposits nothing
// (the reference would index past the upper guard cell there).
struct Interp {
  double w0, w1, pcos, psin;
  int idx;
  bool ok;
};

__device__ __forceinline__ Interp gen_interp(double x, double y, double idr, int nr) {
  Interp ii;
  double pos = radius_rn(x, y);
  ii.pcos = x / pos;
  ii.psin = y / pos;
  pos = __dmul_rn(pos, idr);
  if (!(pos >= 0.0 && pos < (double)nr)) {
    ii.ok = false;
    ii.idx = 1;
    ii.w0 = ii.w1 = 0.0;
    return ii;
  }
  const int ip = (int)pos;
  ii.idx = ip + 1;
  const double fr = __dsub_rn(pos, (double)ip);
  ii.w0 = 1.0 - fr;
  ii.w1 = fr;
  ii.ok = true;
  return ii;
}

// interp_field vector form (interp_part2d.f03:67-109) for a 3-component field.
__device__ __forceinline__ void gather3(const GridDev& G, const double* __restrict__ f, const Interp& ii,
                                        double fp[3]) {
  fp[0] = fp[1] = fp[2] = 0.0;
  if (!ii.ok) return;
  const int i0 = ii.idx;
  const size_t ld = G.ld;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const double* r = f + (size_t)c * ld + i0;
    fp[c] = fp[c] + __ldg(r) * ii.w0;
    fp[c] = fp[c] + __ldg(r + 1) * ii.w1;
  }
  double phr = 1.0, phi = 0.0;
  for (int m = 1; m <= G.M; ++m) {
    const double t = phr * ii.pcos - phi * ii.psin;
    phi = phr * ii.psin + phi * ii.pcos;
    phr = t;
    const double pre = 2.0 * phr, pim = 2.0 * phi;
    const double* fr = f + (size_t)(2 * m - 1) * 3 * ld + i0;
    const double* fi = f + (size_t)(2 * m) * 3 * ld + i0;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      fp[c] = fp[c] + (__ldg(fr + c * ld) * pre - __ldg(fi + c * ld) * pim) * ii.w0;
      fp[c] = fp[c] + (__ldg(fr + c * ld + 1) * pre - __ldg(fi + c * ld + 1) * pim) * ii.w1;
    }
  }
}

__device__ __forceinline__ double gather1(const GridDev& G, const double* __restrict__ f, const Interp& ii) {
  if (!ii.ok) return 0.0;
  const int i0 = ii.idx;
  const size_t ld = G.ld;
  double fp = 0.0;
  fp = fp + __ldg(f + i0) * ii.w0;
  fp = fp + __ldg(f + i0 + 1) * ii.w1;
  double phr = 1.0, phi = 0.0;
  for (int m = 1; m <= G.M; ++m) {
    const double t = phr * ii.pcos - phi * ii.psin;
    phi = phr * ii.psin + phi * ii.pcos;
    phr = t;
    const double pre = 2.0 * phr, pim = 2.0 * phi;
    const double* fr = f + (size_t)(2 * m - 1) * ld + i0;
    const double* fi = f + (size_t)(2 * m) * ld + i0;
    fp = fp + (__ldg(fr) * pre - __ldg(fi) * pim) * ii.w0;
    fp = fp + (__ldg(fr + 1) * pre - __ldg(fi + 1) * pim) * ii.w1;
  }
  return fp;
}

struct PArrays {
  double* a[8];
};

// ---- device-wide int32 exclusive scan (scan.cu) -------------------------------------
// out[i] = sum(in[0..i)), *total = sum(in); tmp needs scan_tmp_elems(n) int32.
int64_t scan_tmp_elems(int64_t n);
int scan_i32(qpad_ctx* ctx, const int32_t* in, int32_t* out, int64_t n, int32_t* tmp, int64_t* total);

}  // namespace qpad
