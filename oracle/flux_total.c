/*
 * FP64 oracle of an insertion's total flux, summed per particle (test
 * infrastructure only: the parity tests and the bench's error fields call it
 * as the checker; the product never links it).
 *
 * The reference sums, for every pixel, w_p * S_p over the particles whose
 * footprint box holds the pixel (martini/martini.py:243-283) and reports the
 * total over the unpadded cube (martini/martini.py:367-375).  Summed over
 * pixels first, that total is
 *
 *     F = sum_p ( sum_{pixels of p's box in the unpadded cube} w_p(pixel) )
 *               * ( sum_c S_p(c) )
 *
 * which costs O(sum_p F_p + N * Nc) instead of O(N_pix * N), so it can be
 * evaluated at the full sizes of the benchmark configurations.  Everything
 * here is FP64 with C99 libm (erf, log, sqrt, asinh), restating the same
 * formulas as oracle/martini_oracle.py:
 *
 *   footprint box  |i - x| <= r            martini/martini.py:272-274
 *   WendlandC2     sph_kernels.py:400-441
 *   WendlandC6     sph_kernels.py:544-685  (the reference's rounded
 *                                           coefficients, :575-674)
 *   CubicSpline    sph_kernels.py:791-858
 *   QuarticSpline  sph_kernels.py:1486-1564
 *   Gaussian       sph_kernels.py:994-1044 (normalisation :931-954)
 *   DiracDelta     sph_kernels.py:1136-1165
 *   adaptive index -1 -> kernels[0]        sph_kernels.py:1330-1363
 *   spectra        spectral_models.py:63-200, Gaussian :386-425,
 *                  Dirac :544-570 (H(0) = 1 on both sides of an edge)
 *
 * Particles are split into contiguous ranges over threads and each range is
 * summed in order, so the result does not depend on scheduling.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>

enum { KT_WC2 = 0, KT_WC6 = 1, KT_CUBIC = 2, KT_QUARTIC = 3, KT_GAUSS = 4, KT_DIRAC = 5 };

static const double PI = 3.14159265358979323846;
/* sigma of the unit-FWHM Gaussian, 1 / (2 sqrt(2 ln 2)) (sph_kernels.py:931-954) */
static const double GAUSS_SIG = 0.42466090014400953;

static double ki_wc2(double dr2, double h) {
  const double R2 = dr2 / (h * h);
  double out;
  if (R2 == 0.0) {
    out = 2.0 / 3.0;
  } else if (R2 < 1.0) {
    const double A = sqrt(1.0 - R2);
    out = 5.0 * R2 * R2 * (0.5 * R2 + 3.0) * log((1.0 + A) / sqrt(R2)) +
          A * (-27.0 / 2.0 * R2 * R2 - 14.0 / 3.0 * R2 + 2.0 / 3.0);
  } else {
    return 0.0;
  }
  return out * (21.0 / 2.0 / PI) / (h * h);
}

static double c6_indef(double R, double z) {
  const double q = sqrt(R * R + z * z);
  const double L = log(q + z);
  const double R2 = R * R, R4 = R2 * R2, R6 = R4 * R2, R8 = R4 * R4, R10 = R8 * R2,
               R12 = R6 * R6;
  const double z2 = z * z, z3 = z2 * z, z5 = z3 * z2, z7 = z5 * z2, z9 = z7 * z2,
               z11 = z9 * z2;
  return -231 * R10 * z - 385 * R8 * z3 - 1155 * R8 * z - 462 * R6 * z5 - 1540 * R6 * z3 -
         462 * R6 * z - 330 * R4 * z7 - 1386 * R4 * z5 - 462 * R4 * z3 + 66 * R4 * z -
         (128 + 1.0 / 3.0) * R2 * z9 - 660 * R2 * z7 - 277.2 * R2 * z5 + 44 * R2 * z3 +
         8.0 / 3.0 * z11 * q + (16 + 4.0 / 15.0) * R2 * z9 * q + 70.4 * z9 * q +
         360.8 * R2 * z7 * q + 132 * z7 * q + 550 * R2 * z5 * q - 11 * R2 * z +
         7.21875 * R12 * L + 24.7813 * R10 * z * q + 173.25 * R10 * L +
         530.75 * R8 * z * q + 288.75 * R8 * L + 47.4792 * R8 * z3 * q +
         767.25 * R6 * z * q + 58.0167 * R6 * z5 * q + 819.5 * R6 * z3 * q +
         41.7 * R4 * z7 * q + 752.4 * R4 * z5 * q + 896.5 * R4 * z3 * q - 21 * z11 -
         (128 + 1.0 / 3.0) * z9 - 66 * z7 + 13.2 * z5 - 11.0 / 3.0 * z3 + z;
}

static double ki_wc6(double dr2, double h) {
  const double R = sqrt(dr2) / h;
  const double norm = 1365.0 / 64.0 / PI;
  double out;
  if (R == 0.0) {
    out = norm * 2.0 * (4.0 / 15.0);
  } else if (R < 1.0) {
    const double zmax = sqrt(1.0 - R * R);
    out = norm * 2.0 * (c6_indef(R, zmax) - c6_indef(R, 0.0));
  } else {
    return 0.0;
  }
  return out / (h * h);
}

static double ki_cubic(double dr2, double h) {
  /* offsets doubled (sph_kernels.py:791-858) */
  const double R2 = 4.0 * dr2 / (h * h);
  double out;
  if (R2 == 0.0) {
    out = 11.0 / 16.0 + 0.25 * 0.25;
  } else if (R2 <= 1.0) {
    const double A = sqrt(1.0 - R2), B = sqrt(4.0 - R2);
    const double I1 = A - 0.5 * A * A * A - 1.5 * R2 * A + 3.0 / 32.0 * A * (3 * R2 + 2) +
                      9.0 / 32.0 * R2 * R2 * (log(1 + A) - log(sqrt(R2)));
    const double I3 = -B * (3 * R2 + 56) / 4.0 + A * (4 * R2 + 50) / 8.0 -
                      3.0 / 8.0 * R2 * (R2 + 16) * log((2 + B) / (1 + A)) +
                      2 * (3 * R2 + 4) * (B - A) + 2 * (B * B * B - A * A * A);
    out = I1 + 0.25 * I3;
  } else if (R2 <= 4.0) {
    const double B = sqrt(4.0 - R2);
    const double I2 = -B * (3 * R2 + 56) / 4.0 -
                      3.0 / 8.0 * R2 * (R2 + 16) * log((2 + B) / sqrt(R2)) +
                      2 * (3 * R2 + 4) * B + 2 * B * B * B;
    out = 0.25 * I2;
  } else {
    return 0.0;
  }
  return out / 1.59689476201133 / (h * h) * 4.0;
}

static double quartic_IA(double R, double z, double A) {
  const double q = sqrt(z * z + R * R);
  const double R2 = R * R;
  return A * A * A * A * z - 2 * A * A * A * z * q + 2 * A * A * z * (3 * R2 + z * z) -
         A * R2 * (4 * A * A + 3 * R2) * asinh(z / R) / 2 -
         A * z * q * (5 * R2 + 2 * z * z) / 2 + R2 * R2 * z + 2 * R2 * z * z * z / 3 +
         z * z * z * z * z / 5;
}

static double ki_quartic(double dr2, double h) {
  const double R = sqrt(dr2) / h;
  double out = 0.0;
  if (R == 0.0) {
    out = 384.0 / 3125.0;
  } else {
    if (R < 0.2) out += 10 * quartic_IA(R, sqrt(0.04 - R * R), 0.2);
    if (R < 0.6) out -= 5 * quartic_IA(R, sqrt(0.36 - R * R), 0.6);
    if (R < 1.0) out += quartic_IA(R, sqrt(1.0 - R * R), 1.0);
  }
  out *= 2.0 * 15625.0 / 512.0 / PI;
  return out / (h * h);
}

static double gaussian_norm(double t) {
  return erf(t / sqrt(2.0)) - 2.0 * t / sqrt(2.0 * PI) * exp(-t * t / 2.0);
}

static double ki_gauss(double dx, double dy, double h, double t, double gnorm) {
  const double dr = sqrt(dx * dx + dy * dy);
  if ((dr - sqrt(0.5)) / h / GAUSS_SIG > t) return 0.0;
  const double q = dr / h / GAUSS_SIG;
  const double zmax = t > q ? sqrt(t * t - q * q) : 0.0;
  const double s = h * sqrt(2.0) * GAUSS_SIG;
  const double x0 = (dx - 0.5) / s, x1 = (dx + 0.5) / s;
  const double y0 = (dy - 0.5) / s, y1 = (dy + 0.5) / s;
  return 0.25 * erf(zmax / sqrt(2.0)) * (erf(x1) - erf(x0)) * (erf(y1) - erf(y0)) / gnorm;
}

/* integer range {i : |i - c| <= r} clipped to [lo_lim, hi_lim] (empty: lo > hi) */
static void box_range(double c, double r, long lo_lim, long hi_lim, long* lo, long* hi) {
  *lo = 1;
  *hi = 0;
  /* NaN or negative range, or a box wholly outside the limits: empty */
  if (!(r >= 0.0) || !(c + r >= (double)lo_lim - 1.0) || !(c - r <= (double)hi_lim + 1.0)) return;
  long a = (long)floor(c - r) - 1, b = (long)ceil(c + r) + 1;
  if (a < lo_lim) a = lo_lim;
  if (b > hi_lim) b = hi_lim;
  while (a <= b && !(fabs((double)a - c) <= r)) ++a;
  while (b >= a && !(fabs((double)b - c) <= r)) --b;
  *lo = a;
  *hi = b;
}

typedef struct {
  int64_t p0, p1;
  const double *x, *y, *r, *h;
  const int8_t* kidx;
  int n_kernels;
  const int* ktype;
  const double* trunc;
  double gnorm[4];
  const double* ssum;
  long ilo, ihi, jlo, jhi; /* unpadded region */
  double* wsum_out;        /* optional per-particle weight sums */
  double total;
} FluxJob;

static void* flux_job(void* arg) {
  FluxJob* J = (FluxJob*)arg;
  double acc = 0.0;
  for (int64_t p = J->p0; p < J->p1; ++p) {
    const double x = J->x[p], y = J->y[p], r = J->r[p], h = J->h[p];
    double wsum = 0.0;
    if (isfinite(x) && isfinite(y)) {
      int k = J->kidx ? J->kidx[p] : 0;
      if (k < 0 || k >= J->n_kernels) k = 0;
      const int t = J->ktype[k];
      long ilo, ihi, jlo, jhi;
      box_range(x, r, J->ilo, J->ihi, &ilo, &ihi);
      box_range(y, r, J->jlo, J->jhi, &jlo, &jhi);
      for (long i = ilo; i <= ihi; ++i) {
        const double dx = x - (double)i;
        for (long j = jlo; j <= jhi; ++j) {
          const double dy = y - (double)j;
          const double dr2 = dx * dx + dy * dy;
          double w = 0.0;
          switch (t) {
            case KT_WC2: w = ki_wc2(dr2, h); break;
            case KT_WC6: w = ki_wc6(dr2, h); break;
            case KT_CUBIC: w = ki_cubic(dr2, h); break;
            case KT_QUARTIC: w = ki_quartic(dr2, h); break;
            case KT_GAUSS: w = ki_gauss(dx, dy, h, J->trunc[k], J->gnorm[k]); break;
            case KT_DIRAC: w = (fabs(dx) < 0.5 && fabs(dy) < 0.5) ? 1.0 : 0.0; break;
            default: w = 0.0;
          }
          wsum += w;
        }
      }
    }
    if (J->wsum_out) J->wsum_out[p] = wsum;
    acc += wsum * J->ssum[p];
  }
  J->total = acc;
  return NULL;
}

/*
 * Total flux F (same units as the spectra) of particles inserted into an
 * nx x ny cube, counted over the unpadded pixels [padx, nx - padx) x
 * [pady, ny - pady).  ssum[p] = sum_c S_p(c).  wsum_out (optional, [n])
 * receives each particle's weight sum over its box in the unpadded cube.
 */
double mgo_flux_total(int64_t n, const double* x, const double* y, const double* r,
                      const double* h_eff, const int8_t* kidx, int n_kernels, const int* ktype,
                      const double* trunc, const double* ssum, int nx, int ny, int padx,
                      int pady, int nthreads, double* wsum_out) {
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  if (n < (int64_t)nthreads) nthreads = n > 0 ? (int)n : 1;
  FluxJob* jobs = (FluxJob*)calloc((size_t)nthreads, sizeof(FluxJob));
  pthread_t* th = (pthread_t*)calloc((size_t)nthreads, sizeof(pthread_t));
  if (!jobs || !th) {
    free(jobs);
    free(th);
    return NAN;
  }
  for (int t = 0; t < nthreads; ++t) {
    FluxJob* J = &jobs[t];
    J->p0 = n * t / nthreads;
    J->p1 = n * (t + 1) / nthreads;
    J->x = x; J->y = y; J->r = r; J->h = h_eff; J->kidx = kidx;
    J->n_kernels = n_kernels; J->ktype = ktype; J->trunc = trunc; J->ssum = ssum;
    for (int k = 0; k < n_kernels && k < 4; ++k)
      J->gnorm[k] = ktype[k] == KT_GAUSS ? gaussian_norm(trunc[k]) : 1.0;
    J->ilo = padx; J->ihi = nx - padx - 1; J->jlo = pady; J->jhi = ny - pady - 1;
    J->wsum_out = wsum_out;
  }
  char created[256] = {0};
  for (int t = 1; t < nthreads; ++t) {
    if (pthread_create(&th[t], NULL, flux_job, &jobs[t]) == 0)
      created[t] = 1;
    else
      flux_job(&jobs[t]);  /* no thread: run the range here */
  }
  flux_job(&jobs[0]);
  for (int t = 1; t < nthreads; ++t)
    if (created[t]) pthread_join(th[t], NULL);
  double total = 0.0;
  for (int t = 0; t < nthreads; ++t) total += jobs[t].total;
  free(jobs);
  free(th);
  return total;
}

typedef struct {
  int64_t p0, p1;
  const double *v, *sigma, *amp, *edges;
  double sigma_const;
  int model, nc;
  double* out;
} SpecJob;

static void* spec_job(void* arg) {
  SpecJob* J = (SpecJob*)arg;
  const int nc = J->nc;
  const int dec = J->edges[nc] < J->edges[0];
  for (int64_t p = J->p0; p < J->p1; ++p) {
    const double v = J->v[p];
    const double s = J->sigma ? J->sigma[p] : J->sigma_const;
    double acc = 0.0;
    for (int c = 0; c < nc; ++c) {
      const double a = dec ? J->edges[c + 1] : J->edges[c];
      const double b = dec ? J->edges[c] : J->edges[c + 1];
      double phi;
      if (J->model == 1) {
        phi = (v >= a && v <= b) ? 1.0 : 0.0;
      } else {
        const double k = 1.0 / (sqrt(2.0) * s);
        phi = 0.5 * (erf((b - v) * k) - erf((a - v) * k));
      }
      acc += phi / fabs(J->edges[c + 1] - J->edges[c]);
    }
    J->out[p] = J->amp[p] * acc;
  }
  return NULL;
}

/*
 * sum_c S_p(c) per particle (Jy): S_p(c) = amp_p * phi_p(c) / |dv_c|, model
 * 0 Gaussian (sigma[p], or sigma_const when sigma is NULL), 1 Dirac.
 */
void mgo_spectrum_sums(int64_t n, const double* v, const double* sigma, double sigma_const,
                       const double* amp, int model, int nc, const double* edges, int nthreads,
                       double* out) {
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  if (n < (int64_t)nthreads) nthreads = n > 0 ? (int)n : 1;
  SpecJob jobs[256];
  pthread_t th[256];
  for (int t = 0; t < nthreads; ++t) {
    SpecJob* J = &jobs[t];
    J->p0 = n * t / nthreads;
    J->p1 = n * (t + 1) / nthreads;
    J->v = v; J->sigma = sigma; J->amp = amp; J->edges = edges;
    J->sigma_const = sigma_const; J->model = model; J->nc = nc; J->out = out;
  }
  char created[256] = {0};
  for (int t = 1; t < nthreads; ++t) {
    if (pthread_create(&th[t], NULL, spec_job, &jobs[t]) == 0)
      created[t] = 1;
    else
      spec_job(&jobs[t]);
  }
  spec_job(&jobs[0]);
  for (int t = 1; t < nthreads; ++t)
    if (created[t]) pthread_join(th[t], NULL);
}
