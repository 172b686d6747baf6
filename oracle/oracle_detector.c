/*
 * TEST INFRASTRUCTURE (oracle) -- not part of the engine.
 *
 * FP64 CPU restatement of the reference detector response
 * (src/xmi_detector_f.F90):
 *   xmi_detector_convolute_spectrum  :339-580 (absorption, escape, pile-up,
 *                                      Gaussian + tail convolution, Poisson)
 *   xmi_detector_escape              :582-809 (sequential in-place loop)
 *   xmi_detector_sum_peaks           :56-217  (Gardner pulse train)
 * The pulse train draws each pulse group from the Philox stream
 * (seed, group, 0xD0000000) -- the group decomposition of the reference's
 * serial train -- so the GPU engine's parallel pile-up can be checked
 * exactly.  Inputs that need atomic data (channel absorption factors, escape
 * line energies and edges) are passed in by the caller.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "oracle_rng.h"

static int findpos(const double *a, int n, double x) {
  int i;
  if (fabs(x - a[0]) < 1e-10) return 0;
  for (i = 1; i < n; i++)
    if (x <= a[i]) return i - 1;
  return -1;
}

typedef struct {
  int n_el, nfe, nce, nco;
  const double *edge;     /* [n_el][4] K, L1, L2, L3 */
  const double *line_e;   /* [n_el][109] LineEnergy of lines 1..109 */
  const double *fluo;     /* Fortran (n_el, 109, nfe) */
  const double *fe;
  const double *comp;     /* Fortran (nce, nco) */
  const double *ce, *co;
} oracle_escape;

/* xmi_detector_escape, src/xmi_detector_f.F90:582-809 */
static void detector_escape(double *ch, int nch, double gain, double zero, const oracle_escape *er) {
  double channel_1e = (0.5) * gain + zero;
  double cod = er->co[1] - er->co[0];
  int i, j, k;
  static const int first[4] = {1, 32, 60, 86}, last[4] = {29, 58, 85, 109};
  for (i = 0; i <= nch - 1; i++) {
    double ce = ((double)(float)i + 0.5) * gain + zero, sum_ratio = 0.0;
    for (j = 0; j < er->n_el; j++) {
      int sh;
      for (sh = 0; sh < 4; sh++) {
        if (!(ce > er->edge[j * 4 + sh])) continue;
        for (k = first[sh]; k <= last[sh]; k++) {
          double le = er->line_e[j * 109 + (k - 1)];
          if ((ce - le) >= channel_1e && ce >= er->fe[0] && ce < er->fe[er->nfe - 1]) {
            int pos = findpos(er->fe, er->nfe, ce), ei;
            double a1, b1, a2, b2, ratio;
            if (pos < 0) continue;
            a1 = er->fe[pos];
            b1 = er->fe[pos + 1];
            a2 = er->fluo[j + er->n_el * ((k - 1) + 109 * pos)];
            b2 = er->fluo[j + er->n_el * ((k - 1) + 109 * (pos + 1))];
            ratio = a2 + ((b2 - a2) * (ce - a1) / (b1 - a1));
            sum_ratio = sum_ratio + ratio;
            ei = (int)((ce - le - zero) / gain);
            if (sh == 0 ? (ei >= 0 && ei < nch - 1) : (ei >= 0 && ei <= nch - 1))
              ch[ei] = ch[ei] + ratio * ch[i];
          }
        }
      }
    }
    for (j = 0; j <= i - 1; j++) {
      double cc = ((double)(float)j + 0.5) * gain + zero, cdiff = ce - cc;
      if (ce >= er->ce[0] && ce < er->ce[er->nce - 1] && cdiff >= er->co[0] && cdiff < er->co[er->nco - 1]) {
        int p1 = findpos(er->ce, er->nce, ce), p2 = findpos(er->co, er->nco, cdiff);
        double x0, x1, y0, y1, den, v, ratio;
        if (p1 < 0 || p2 < 0) continue;
        x0 = er->ce[p1]; x1 = er->ce[p1 + 1]; y0 = er->co[p2]; y1 = er->co[p2 + 1];
        den = (x1 - x0) * (y1 - y0);
        v = (x1 - ce) * (y1 - cdiff) / den * er->comp[p1 + er->nce * p2] +
            (ce - x0) * (y1 - cdiff) / den * er->comp[p1 + 1 + er->nce * p2] +
            (x1 - ce) * (cdiff - y0) / den * er->comp[p1 + er->nce * (p2 + 1)] +
            (ce - x0) * (cdiff - y0) / den * er->comp[p1 + 1 + er->nce * (p2 + 1)];
        ratio = v * gain / cod;
        ch[j] = ch[j] + ratio * ch[i];
        sum_ratio = sum_ratio + ratio;
      }
    }
    ch[i] = ch[i] * (1.0 - sum_ratio);
  }
}

/* xmi_detector_sum_peaks, src/xmi_detector_f.F90:56-217 */
static int sum_peaks(double *ch, int nch, double live_time, double pulse_width, double gain, double zero,
                     uint64_t seed) {
  double Nt = 0.0, lambda, mu, *cdf, acc = 0.0, *out;
  long long Nt_long, npulses_all = 0, grp = 0;
  int i;
  for (i = 0; i < nch; i++) Nt += ch[i];
  Nt_long = (long long)Nt;
  if (Nt_long <= 0) return 1;
  lambda = Nt / live_time;
  mu = 1.0 / lambda;
  cdf = (double *)malloc(sizeof(double) * nch);
  out = (double *)calloc(nch, sizeof(double));
  for (i = 0; i < nch; i++) {
    acc += ch[i] > 0.0 ? ch[i] : 0.0;
    cdf[i] = acc;
  }
  for (;;) {
    orng g;
    int n, first = -1;
    double esum = 0.0;
    orng_init(&g, seed, (uint64_t)grp, 0xD0000000u);
    for (n = 1;; n++) {
      double x = orng_uniform(&g) * cdf[nch - 1], dt;
      int lo = 0, hi = nch - 1;
      while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (x < cdf[mid]) hi = mid; else lo = mid + 1;
      }
      dt = -mu * log1p(-orng_uniform(&g));
      esum += (double)(lo + 1) * gain + zero;
      if (n == 1) first = lo;
      npulses_all++;
      if (n > 100) {
        free(cdf);
        free(out);
        return 0;
      }
      if (dt > pulse_width) {
        if (n == 1) out[first] += 1.0;
        else {
          unsigned long long ps = (unsigned long long)((esum - zero) / gain);
          if (ps > 0 && ps <= (unsigned long long)nch) out[ps - 1] += 1.0;
        }
        break;
      }
    }
    grp++;
    if (npulses_all >= Nt_long) break;
  }
  memcpy(ch, out, sizeof(double) * nch);
  free(cdf);
  free(out);
  return 1;
}

/* Gaussian + tail convolution, src/xmi_detector_f.F90:481-558 */
static void convolute(const double *temp, double *conv, int nch, double gain, double zero, double fano, double noise,
                      int det_type) {
  const double c = sqrt(2.0) / (2.0 * sqrt(2.0 * log(2.0)));
  const double a = noise * noise, b = (double)((float)(2.3548f * 2.3548f) * 3.85f) * fano / 1000.0;
  const double sqrtpi = 1.77245385090551602729816748334;
  double *R = (double *)malloc(sizeof(double) * (nch + 101));
  int I0, I;
  memset(conv, 0, sizeof(double) * nch);
  for (I0 = 0; I0 <= nch - 1; I0++) {
    double E0 = zero + gain * I0, FWHM, B0, A0, A3, A4, ALFA, my_sum = 0.0;
    if (E0 < 1.0) continue;
    FWHM = sqrt(a + b * E0);
    B0 = c * FWHM;
    A0 = 1.0 / (B0 * sqrtpi);
    A3 = 2.73E-3 * exp(-0.21 * E0) + 1.E-4;
    A4 = 0.000188 * exp(-0.00296 * pow(E0, 0.763)) + 1.355E-5 * exp(0.968 * pow(E0, 0.498));
    ALFA = 1.179 * exp(8.6E-4 * pow(E0, 1.877)) - 7.793 * exp(-3.81 * pow(E0, -0.0716));
    for (I = 0; I <= I0 + 100; I++) {
      double E, X, G, F;
      if (I >= nch) break;
      E = zero + gain * I;
      X = (E - E0) / B0;
      G = exp(-X * X);
      F = erfc(X);
      if (E0 > 50.0) R[I] = A0 * G;
      else if (det_type == 0) R[I] = A0 * G + 1.0 * (2.7 * A3 + 15.0 * A4 * exp(ALFA * (E - E0))) * F;
      else if (det_type == 2) R[I] = A0 * G + 1.0 * (0.63 * A3 + 15.0 * A4 * exp(ALFA * (E - E0))) * F;
      else R[I] = A0 * G + 1.0 * (2.7 * A3 + 15.0 * A4 * exp(ALFA * (E - E0))) * F;
      my_sum = my_sum + R[I];
    }
    for (I = 0; I <= I0 + 100; I++) {
      if (I >= nch) break;
      conv[I] = conv[I] + R[I] * temp[I0] / my_sum;
    }
  }
  free(R);
}

/* One interaction order: channel absorption (det_corr given), escape
 * (er != NULL), pile-up, convolution.  Returns 1 on success. */
int oracle_convolute_spectrum(const double *noconv, const double *det_corr, int nch, double gain, double zero,
                              double fano, double noise, int det_type, double live_time, double pulse_width,
                              const oracle_escape *er, int use_sum_peaks, uint64_t pile_seed, double *out) {
  double *temp = (double *)malloc(sizeof(double) * nch);
  int i, ok = 1;
  for (i = 0; i < nch; i++) temp[i] = noconv[i] * det_corr[i];
  if (er) detector_escape(temp, nch, gain, zero, er);
  if (use_sum_peaks) ok = sum_peaks(temp, nch, live_time, pulse_width, gain, zero, pile_seed);
  if (ok) convolute(temp, out, nch, gain, zero, fano, noise, det_type);
  free(temp);
  return ok;
}

/* exposes the escape step alone */
void oracle_detector_escape(double *ch, int nch, double gain, double zero, const oracle_escape *er) {
  detector_escape(ch, nch, gain, zero, er);
}

/* xmi_detector_poisson, src/xmi_detector_f.F90:862-905: every channel above
 * 1 count and below 2^32 - 1 becomes a Poisson variate of that mean.  The
 * reference draws from one serial MT19937 stream through GSL; here channel i
 * draws from the Philox stream (seed, i, 0xE0000000) so that the GPU engine
 * can be checked draw for draw.  The variate is exact: the multiplication
 * method below a mean of 10, above it the transformed rejection with squeeze
 * (PTRS) of W. Hormann, Insurance: Mathematics and Economics 12 (1993) 39-45. */
static double poisson_variate(double lam, orng *g) {
  if (lam < 10.0) {
    double L = exp(-lam), prod = orng_uniform(g);
    int n = 0;
    while (prod > L && n < 4096) {
      prod *= orng_uniform(g);
      n++;
    }
    return (double)n;
  } else {
    double slam = sqrt(lam), loglam = log(lam);
    double b = 0.931 + 2.53 * slam, a = -0.059 + 0.02483 * b;
    double inv_alpha = 1.1239 + 1.1328 / (b - 3.4), vr = 0.9277 - 3.6224 / (b - 2.0);
    int it;
    for (it = 0; it < 4096; it++) {
      double U = orng_uniform(g) - 0.5, V = orng_uniform(g);
      double us = 0.5 - fabs(U);
      double k = floor((2.0 * a / us + b) * U + lam + 0.43);
      if (us >= 0.07 && V <= vr) return k;
      if (k < 0.0 || (us < 0.013 && V > us)) continue;
      if (log(V) + log(inv_alpha) - log(a / (us * us) + b) <= -lam + k * loglam - lgamma(k + 1.0)) return k;
    }
    return floor(lam + 0.5);
  }
}

void oracle_poisson(double *ch, int nch, uint64_t seed) {
  const double limit = 4294967296.0 - 1.0;
  int i;
  for (i = 0; i < nch; i++) {
    orng g;
    if (!(ch[i] > 1.0) || ch[i] > limit) continue;
    orng_init(&g, seed, (uint64_t)i, 0xE0000000u);
    ch[i] = poisson_variate(ch[i], &g);
  }
}

/* the pile-up step alone (in place) */
int oracle_sum_peaks(double *ch, int nch, double live_time, double pulse_width, double gain, double zero,
                     uint64_t seed) {
  return sum_peaks(ch, nch, live_time, pulse_width, gain, zero, seed);
}
