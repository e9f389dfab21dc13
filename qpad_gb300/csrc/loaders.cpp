// loaders.cpp -- host-side particle loaders with the project's own RNG.
//
// The reference samples with gfortran's random_number through rand_norm
// (math_module.f03:77-102), which is not reproducible outside gfortran.  The loaders here
// use a SplitMix64 stream (Steele, Lea & Flood, "Fast splittable pseudorandom number
// generators", OOPSLA 2014) feeding the same Box-Muller pairing (cosine first, the sine
// value kept for the next call), so a given seed gives the same particles on any host.
#include <cmath>
#include <cstdint>

#include "../../include/qpad_gpu.h"

namespace {
const double kPi = 3.141592653589793;  // 4*atan(1.0), param.f03:29

uint64_t splitmix64(uint64_t* s) {
  uint64_t z = (*s += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

double uniform(qpad_rng* r) { return ((double)(splitmix64(&r->s) >> 11) + 0.5) * (1.0 / 9007199254740992.0); }

double rand_norm(qpad_rng* r) {
  if (!r->have) {
    const double u1 = uniform(r), u2 = uniform(r);
    const double theta = 2.0 * kPi * u1;
    const double amp = std::sqrt(-2.0 * std::log(u2));
    r->next = amp * std::sin(theta);
    r->have = 1;
    return amp * std::cos(theta);
  }
  r->have = 0;
  const double v = r->next;
  r->next = 0.0;
  return v;
}
}  // namespace

extern "C" void qpad_rng_seed(qpad_rng* r, uint64_t seed) {
  r->s = seed;
  r->have = 0;
  r->next = 0.0;
}

// fdist2d::inject (fdist2d_class.f03:289-357) for uniform transverse and longitudinal
// profiles on one radial partition starting at the axis.
extern "C" int64_t qpad_load_plasma(int nr, double dr, qpad_rng* r, int ppc1, int ppc2, int num_theta, double qm,
                                    double density, const double uth[3], double* x, double* p, double* gamma,
                                    double* psi, double* q, int64_t cap) {
  if (nr < 1 || ppc1 < 1 || ppc2 < 1 || num_theta < 1 || !r || !x || !p || !gamma || !psi || !q || qm == 0.0)
    return -1;
  const double dtheta = 2.0 * kPi / num_theta;
  const int ppc_tot = ppc1 * ppc2;
  const double coef = (qm >= 0.0 ? 1.0 : -1.0) / ((double)ppc_tot * (double)num_theta);
  const double den_lon = 1.0, den_perp = 1.0, den_min = 1.0e-10;
  int64_t ip = 0;
  for (int j = 1; j <= num_theta; ++j)
    for (int i = 1; i <= nr; ++i)
      for (int i1 = 1; i1 <= ppc1; ++i1) {
        const double rn = (i1 - 0.5) / ppc1 + (double)(i - 1);
        for (int i2 = 1; i2 <= ppc2; ++i2) {
          const double theta = ((i2 - 0.5) / ppc2 + j - 1.0) * dtheta;
          const double xt = rn * dr * std::cos(theta), yt = rn * dr * std::sin(theta);
          if (den_lon * den_perp * density < den_min) continue;
          if (ip >= cap) return -1;
          x[2 * ip] = xt;
          x[2 * ip + 1] = yt;
          q[ip] = rn * den_perp * den_lon * density * coef;
          const double p1 = uth[0] * rand_norm(r);
          const double p2 = uth[1] * rand_norm(r);
          const double p3 = uth[2] * rand_norm(r);
          p[3 * ip] = p1;
          p[3 * ip + 1] = p2;
          p[3 * ip + 2] = p3;
          gamma[ip] = std::sqrt(1.0 + p1 * p1 + p2 * p2 + p3 * p3);
          psi[ip] = (1.0 - gamma[ip] + p3) / qm;
          ++ip;
        }
      }
  return ip;
}

// fdist3d_rnd::inject (fdist3d_rnd_class.f03:360-514) with Gaussian profiles in
// cartesian geometry; particles outside the box are dropped as the reference does.
extern "C" int64_t qpad_load_beam(int nr, int nz, double dr, double dxi, qpad_rng* r, const qpad_beam_load_desc* d,
                                  double* x, double* p, double* q, int64_t cap) {
  if (!r || !d || !x || !p || !q || d->tot_num < 0 || nr < 1 || nz < 1) return -1;
  // the rejection sampling below needs a non-empty range in every direction
  for (int k = 0; k < 3; ++k)
    if (!(d->range_lo[k] < d->range_hi[k]) || !(d->sigma[k] > 0.0)) return -1;
  const double er = (double)nr * dr, ez = (double)nz * dxi;
  const double q_per_part =
      (d->qm >= 0.0 ? 1.0 : -1.0) * d->tot_charge / (2.0 * kPi * (double)d->tot_num * (dr * dr) * dxi);
  int64_t n = 0;
  for (int64_t i = 0; i < d->tot_num; ++i) {
    double xt[3];
    for (;;) {
      xt[0] = rand_norm(r) * d->sigma[0] + d->center[0];
      if (xt[0] < d->range_lo[0] || xt[0] >= d->range_hi[0]) continue;
      xt[1] = rand_norm(r) * d->sigma[1] + d->center[1];
      if (xt[1] < d->range_lo[1] || xt[1] >= d->range_hi[1]) continue;
      xt[2] = rand_norm(r) * d->sigma[2] + d->center[2];
      if (xt[2] < d->range_lo[2] || xt[2] >= d->range_hi[2]) continue;
      break;
    }
    const double rt = std::sqrt(xt[0] * xt[0] + xt[1] * xt[1]);
    if (rt < 0.0 || rt >= er) continue;
    if (xt[2] < 0.0 || xt[2] >= ez) continue;
    if (n >= cap) return -1;
    x[3 * n] = xt[0];
    x[3 * n + 1] = xt[1];
    x[3 * n + 2] = xt[2];
    q[n] = q_per_part;
    const double p1 = d->uth[0] * rand_norm(r);
    const double p2 = d->uth[1] * rand_norm(r);
    double p3 = d->uth[2] * rand_norm(r) + d->gamma;
    p3 = std::sqrt(p3 * p3 - p1 * p1 - p2 * p2 - 1);
    p[3 * n] = p1;
    p[3 * n + 1] = p2;
    p[3 * n + 2] = p3;
    ++n;
  }
  if (d->quiet) {
    if (2 * n > cap) return -1;
    const int64_t ip = n;
    for (int64_t i = 0; i < ip; ++i) {
      x[3 * (ip + i)] = -x[3 * i];
      x[3 * (ip + i) + 1] = -x[3 * i + 1];
      x[3 * (ip + i) + 2] = x[3 * i + 2];
      p[3 * (ip + i)] = -p[3 * i];
      p[3 * (ip + i) + 1] = -p[3 * i + 1];
      p[3 * (ip + i) + 2] = p[3 * i + 2];
      q[i] = 0.5 * q[i];
      q[ip + i] = q[i];
    }
    n *= 2;
  }
  return n;
}
