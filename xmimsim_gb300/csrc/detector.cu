/*
 * Detector response on the GPU: xmi_detector_convolute_all/_spectrum/_history
 * (src/xmi_detector_f.F90:56-905) and the escape-ratio Monte Carlo
 * (src/xmi_main.F90:5473-5800, driven by src/xmi_detector.c:91-141).
 *
 * Per interaction order the unconvolved spectrum goes through
 *   1. detector window / crystal absorption per channel,
 *   2. escape peaks: each output channel gathers the Compton-escape
 *      contributions of every higher channel (O(nch^2) bilinear lookups, one
 *      thread per output channel) and receives the fluorescence-escape
 *      contributions scattered by its source channels,
 *   3. pulse pile-up: the reference's serial Gardner pulse train is a
 *      sequence of independent pulse groups (a group closes when the
 *      exponential gap exceeds the pulse width); groups are generated in
 *      parallel from Philox streams keyed by the group index, and a prefix
 *      sum over group sizes applies the reference's stopping rule,
 *   4. Gaussian + tail/step convolution over the I0..I0+100 window, as a
 *      normalisation pass per source channel and a gather per output channel,
 *   5. optional Poisson noise.
 * All kernels are FP64 (the convolution parity target is 1e-5 relative).
 */
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <atomic>
#include <vector>

#include "dev_bundle.cuh"
#include "transport.cuh"
#include "xmi_internal.h"
#include "xrlite.h"

namespace {

constexpr double kSqrtPi = 1.77245385090551602729816748334;

struct EscDev {
  int n_el, nfe, nce, nco;
  const int *lines_n;           /* [n_el] number of escape lines */
  const double *line_e;         /* [n_el][64] energies */
  const int *line_k;            /* [n_el][64] line index (1..109) */
  const double *edge;           /* [n_el][4] K, L1, L2, L3 edges */
  const double *fluo;           /* Fortran (n_el,109,nfe) */
  const double *fe;             /* [nfe] */
  const double *comp;           /* Fortran (nce, nco) */
  const double *ce, *co;
};

__device__ inline int findpos_lin(const double *a, int n, double x) {
  if (fabs(x - a[0]) < 1e-10) return 0;
  /* binary search for the first i >= 1 with x <= a[i] */
  if (x > a[n - 1]) return -1;
  int lo = 1, hi = n - 1;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (x <= a[mid]) hi = mid; else lo = mid + 1;
  }
  return lo - 1;
}

/* fluorescence-escape lines of escape element e that apply to channel energy ce */
__device__ void fluo_ratio(const EscDev &s, int e, int line_pos, double ce, double gain, double zero, double c1e,
                           double *ratio, int *target) {
  *ratio = 0.0;
  *target = -1;
  int k = s.line_k[e * 64 + line_pos];
  double le = s.line_e[e * 64 + line_pos];
  int shell = k <= 29 ? 0 : (k <= 58 ? 1 : (k <= 85 ? 2 : 3));
  if (!(ce > s.edge[e * 4 + shell])) return;
  if (!((ce - le) >= c1e && ce >= s.fe[0] && ce < s.fe[s.nfe - 1])) return;
  int pos = findpos_lin(s.fe, s.nfe, ce);
  if (pos < 0) return;
  double a1 = s.fe[pos], b1 = s.fe[pos + 1];
  double a2 = s.fluo[e + s.n_el * ((k - 1) + 109 * pos)], b2 = s.fluo[e + s.n_el * ((k - 1) + 109 * (pos + 1))];
  *ratio = a2 + ((b2 - a2) * (ce - a1) / (b1 - a1));
  *target = (int)((ce - le - zero) / gain);
}

/* per source channel: fluorescence escape scatter and the total escape ratio */
__global__ void escape_source_kernel(EscDev s, const double *in, int nch, double gain, double zero, double *add,
                                     double *sum_ratio) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nch) return;
  double ce = ((double)(float)i + 0.5) * gain + zero;
  double c1e = 0.5 * gain + zero;
  double sr = 0.0;
  for (int e = 0; e < s.n_el; e++)
    for (int l = 0; l < s.lines_n[e]; l++) {
      double r;
      int t;
      fluo_ratio(s, e, l, ce, gain, zero, c1e, &r, &t);
      if (t < 0) continue; /* conditions of the reference not met */
      sr += r;
      int k = s.line_k[e * 64 + l];
      /* the K-line branch of the reference stops one channel short */
      bool in_range = k <= 29 ? (t >= 0 && t < nch - 1) : (t >= 0 && t <= nch - 1);
      if (in_range) atomicAdd(&add[t], r * in[i]);
    }
  /* Compton escape into every lower channel */
  double cod = s.co[1] - s.co[0];
  if (ce >= s.ce[0] && ce < s.ce[s.nce - 1]) {
    int p1 = findpos_lin(s.ce, s.nce, ce);
    for (int j = 0; j < i; j++) {
      double cc = ((double)(float)j + 0.5) * gain + zero;
      double cdiff = ce - cc;
      if (!(cdiff >= s.co[0] && cdiff < s.co[s.nco - 1])) continue;
      int p2 = findpos_lin(s.co, s.nco, cdiff);
      if (p1 < 0 || p2 < 0) continue;
      double x0 = s.ce[p1], x1 = s.ce[p1 + 1], y0 = s.co[p2], y1 = s.co[p2 + 1];
      double den = (x1 - x0) * (y1 - y0);
      double v = (x1 - ce) * (y1 - cdiff) / den * s.comp[p1 + s.nce * p2] +
                 (ce - x0) * (y1 - cdiff) / den * s.comp[p1 + 1 + s.nce * p2] +
                 (x1 - ce) * (cdiff - y0) / den * s.comp[p1 + s.nce * (p2 + 1)] +
                 (ce - x0) * (cdiff - y0) / den * s.comp[p1 + 1 + s.nce * (p2 + 1)];
      sr += v * gain / cod;
    }
  }
  sum_ratio[i] = sr;
}

/* per output channel: Compton escape gathered from every higher channel */
__global__ void escape_gather_kernel(EscDev s, const double *in, int nch, double gain, double zero,
                                     const double *add, const double *sum_ratio, double *out) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nch) return;
  double cc = ((double)(float)j + 0.5) * gain + zero;
  double cod = s.co[1] - s.co[0];
  double acc = 0.0;
  for (int i = j + 1; i < nch; i++) {
    double ce = ((double)(float)i + 0.5) * gain + zero;
    double cdiff = ce - cc;
    if (!(ce >= s.ce[0] && ce < s.ce[s.nce - 1] && cdiff >= s.co[0] && cdiff < s.co[s.nco - 1])) continue;
    int p1 = findpos_lin(s.ce, s.nce, ce), p2 = findpos_lin(s.co, s.nco, cdiff);
    if (p1 < 0 || p2 < 0) continue;
    double x0 = s.ce[p1], x1 = s.ce[p1 + 1], y0 = s.co[p2], y1 = s.co[p2 + 1];
    double den = (x1 - x0) * (y1 - y0);
    double v = (x1 - ce) * (y1 - cdiff) / den * s.comp[p1 + s.nce * p2] +
               (ce - x0) * (y1 - cdiff) / den * s.comp[p1 + 1 + s.nce * p2] +
               (x1 - ce) * (cdiff - y0) / den * s.comp[p1 + s.nce * (p2 + 1)] +
               (ce - x0) * (cdiff - y0) / den * s.comp[p1 + 1 + s.nce * (p2 + 1)];
    acc += v * gain / cod * in[i];
  }
  out[j] = in[j] * (1.0 - sum_ratio[j]) + add[j] + acc;
}

struct ConvParams {
  int nch, det_type;
  double gain, zero, a, b, c;
};

/* Gaussian + tail line shape of src/xmi_detector_f.F90:481-545 */
__device__ __forceinline__ double line_shape(const ConvParams &p, int I0, int I, double &A0out) {
  double E0 = p.zero + p.gain * I0;
  double FWHM = sqrt(p.a + p.b * E0);
  double B0 = p.c * FWHM;
  double A0 = 1.0 / (B0 * kSqrtPi);
  double A3 = 2.73E-3 * exp(-0.21 * E0) + 1.E-4;
  double A4 = 0.000188 * exp(-0.00296 * pow(E0, 0.763)) + 1.355E-5 * exp(0.968 * pow(E0, 0.498));
  double ALFA = 1.179 * exp(8.6E-4 * pow(E0, 1.877)) - 7.793 * exp(-3.81 * pow(E0, -0.0716));
  double E = p.zero + p.gain * I;
  double X = (E - E0) / B0;
  double G = exp(-X * X);
  double F = erfc(X);
  A0out = A0;
  if (E0 > 50.0) return A0 * G;
  if (p.det_type == 2) return A0 * G + 1.0 * (0.63 * A3 + 15.0 * A4 * exp(ALFA * (E - E0))) * F;
  return A0 * G + 1.0 * (2.7 * A3 + 15.0 * A4 * exp(ALFA * (E - E0))) * F;
}

__global__ void conv_norm_kernel(ConvParams p, double *norm) {
  int I0 = blockIdx.x * blockDim.x + threadIdx.x;
  if (I0 >= p.nch) return;
  double E0 = p.zero + p.gain * I0;
  if (E0 < 1.0) { norm[I0] = 0.0; return; }
  double s = 0.0, a0;
  int hi = I0 + 100 < p.nch - 1 ? I0 + 100 : p.nch - 1;
  for (int I = 0; I <= hi; I++) s += line_shape(p, I0, I, a0);
  norm[I0] = s;
}

__global__ void conv_gather_kernel(ConvParams p, const double *in, const double *norm, double *out) {
  int I = blockIdx.x * blockDim.x + threadIdx.x;
  if (I >= p.nch) return;
  double acc = 0.0, a0;
  int lo = I - 100 > 0 ? I - 100 : 0;
  for (int I0 = lo; I0 < p.nch; I0++) {
    double E0 = p.zero + p.gain * I0;
    if (E0 < 1.0 || norm[I0] == 0.0) continue;
    acc += line_shape(p, I0, I, a0) * in[I0] / norm[I0];
  }
  out[I] = acc;
}

/* pile-up: group g draws pulses from stream (seed, g, 0xD0000000) */
struct PileParams {
  int nch;
  double mu, pulse_width, gain, zero;
  unsigned long long seed;
  long long n_groups;
};

__device__ int sample_channel(const double *cdf, int nch, double u) {
  double x = u * cdf[nch - 1];
  int lo = 0, hi = nch - 1;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (x < cdf[mid]) hi = mid; else lo = mid + 1;
  }
  return lo;
}

__device__ int pile_group(const PileParams &p, const double *cdf, long long g, int *chan_out, bool *overflow) {
  xmi_rng r;
  xmi_rng_init(&r, p.seed, (uint64_t)g, 0xD0000000u);
  double esum = 0.0;
  int first = -1;
  for (int n = 1; n <= 101; n++) {
    int c = sample_channel(cdf, p.nch, xmi_rng_uniform(&r));
    double dt = -p.mu * log1p(-xmi_rng_uniform(&r));
    esum += (double)(c + 1) * p.gain + p.zero;
    if (n == 1) first = c;
    if (n > 100) { *overflow = true; return n; }
    if (dt > p.pulse_width) {
      if (n == 1) *chan_out = first;
      else {
        unsigned long long ps = (unsigned long long)((esum - p.zero) / p.gain);
        *chan_out = (ps > 0 && ps <= (unsigned long long)p.nch) ? (int)ps - 1 : -1;
      }
      return n;
    }
  }
  *overflow = true;
  return 101;
}

__global__ void pile_sizes_kernel(PileParams p, const double *cdf, long long g0, int *sizes, int *flag) {
  long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= p.n_groups) return;
  int ch;
  bool ov = false;
  sizes[g] = pile_group(p, cdf, g0 + g, &ch, &ov);
  if (ov) atomicExch(flag, 1);
}

__global__ void pile_tally_kernel(PileParams p, const double *cdf, long long n_used, double *out) {
  long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n_used) return;
  int ch = -1;
  bool ov = false;
  pile_group(p, cdf, g, &ch, &ov);
  if (ch >= 0) atomicAdd(&out[ch], 1.0);
}

/* Exact Poisson variate of mean lam from stream r: the multiplication method
 * (count uniforms until their product drops below exp(-lam)) for lam < 10,
 * and for lam >= 10 the transformed rejection with squeeze of W. Hörmann,
 * "The transformed rejection method for generating Poisson random variables",
 * Insurance: Mathematics and Economics 12 (1993) 39-45 (PTRS).  Both loops
 * are bounded at 4096 rounds, far beyond what their acceptance rates ever
 * need (PTRS accepts most candidates at the first or second try). */
__device__ double poisson_draw(double lam, xmi_rng *r) {
  if (lam < 10.0) {
    const double L = exp(-lam);
    double prod = xmi_rng_uniform(r);
    int n = 0;
    while (prod > L && n < 4096) {
      prod *= xmi_rng_uniform(r);
      n++;
    }
    return (double)n;
  }
  const double slam = sqrt(lam), loglam = log(lam);
  const double b = 0.931 + 2.53 * slam, a = -0.059 + 0.02483 * b;
  const double inv_alpha = 1.1239 + 1.1328 / (b - 3.4), vr = 0.9277 - 3.6224 / (b - 2.0);
  for (int it = 0; it < 4096; it++) {
    const double U = xmi_rng_uniform(r) - 0.5, V = xmi_rng_uniform(r);
    const double us = 0.5 - fabs(U);
    const double k = floor((2.0 * a / us + b) * U + lam + 0.43);
    if (us >= 0.07 && V <= vr) return k;
    if (k < 0.0 || (us < 0.013 && V > us)) continue;
    if (log(V) + log(inv_alpha) - log(a / (us * us) + b) <= -lam + k * loglam - lgamma(k + 1.0)) return k;
  }
  return floor(lam + 0.5);
}

/* src/xmi_detector_f.F90:862-905: every channel above 1 count (and below
 * 2^32 - 1) is replaced by a Poisson variate of that mean; channel i draws
 * from stream (seed, i, 0xE0000000) */
__global__ void poisson_kernel(int nch, unsigned long long seed, double *ch) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nch) return;
  double lam = ch[i];
  const double limit = 4294967296.0 - 1.0;
  if (!(lam > 1.0) || lam > limit) return;
  xmi_rng r;
  xmi_rng_init(&r, seed, (uint64_t)i, 0xE0000000u);
  ch[i] = poisson_draw(lam, &r);
}

bool ck(cudaError_t e, const char *w) {
  if (e != cudaSuccess) {
    xmi_set_error("%s: %s", w, cudaGetErrorString(e));
    return false;
  }
  return true;
}

unsigned long long seed_for(xmi_inputFPtr in, xmi_main_options *o, unsigned long long salt) {
  if (in && in->gpu.seed) return in->gpu.seed ^ salt;
  if (o && o->use_default_seeds) return 0x5EED0001ull ^ salt;
  unsigned long long s = 0;
  FILE *f = fopen("/dev/urandom", "rb");
  if (f) {
    if (fread(&s, sizeof(s), 1, f) != 1) s = 0;
    fclose(f);
  }
  return s ? s : (0x5EED0001ull ^ salt);
}

/* detector absorption of the channel energies, src/xmi_detector_f.F90:437-454 */
std::vector<double> channel_det_corr(const xmi_input *in) {
  int nch = in->detector->nchannels;
  std::vector<double> c(nch, 1.0);
  for (int i = 0; i < nch; i++) {
    double E = i * in->detector->gain + in->detector->zero, dc = 1.0;
    for (int j = 0; j < in->absorbers->n_det_layers; j++) {
      const xmi_layer *l = &in->absorbers->det_layers[j];
      dc = dc * exp(-1.0 * l->density * l->thickness * xmi_layer_mu(l, E));
    }
    for (int j = 0; j < in->detector->n_crystal_layers; j++) {
      const xmi_layer *l = &in->detector->crystal_layers[j];
      dc = -1.0 * dc * expm1(-1.0 * l->density * l->thickness * xmi_layer_mu(l, E));
    }
    c[i] = dc;
  }
  return c;
}

}  // namespace

extern "C" {

/* reference src/xmi_detector_f.F90:339-580 */
void xmi_detector_convolute_spectrum(xmi_inputFPtr inputFPtr, double *channels_noconv, double **channels_conv,
                                     xmi_main_options *options, xmi_escape_ratios *er, int n_interactions) {
  *channels_conv = nullptr;
  if (!inputFPtr || !channels_noconv || !options) {
    xmi_set_error("xmi_detector_convolute_spectrum: NULL argument");
    return;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    xmi_set_error("no CUDA device available: the detector response has no CPU fallback");
    return;
  }
  const xmi_input *in = inputFPtr->input;
  const xmi_detector *det = in->detector;
  const int nch = det->nchannels;
  std::vector<double> temp(channels_noconv, channels_noconv + nch);
  std::vector<double> dc = channel_det_corr(in);
  for (int i = 0; i < nch; i++) temp[i] *= dc[i];

  double *d_in = nullptr, *d_out = nullptr, *d_add = nullptr, *d_sr = nullptr, *d_norm = nullptr;
  bool ok = ck(cudaMalloc(&d_in, sizeof(double) * nch), "cudaMalloc") &&
            ck(cudaMalloc(&d_out, sizeof(double) * nch), "cudaMalloc") &&
            ck(cudaMalloc(&d_add, sizeof(double) * nch), "cudaMalloc") &&
            ck(cudaMalloc(&d_sr, sizeof(double) * nch), "cudaMalloc") &&
            ck(cudaMalloc(&d_norm, sizeof(double) * nch), "cudaMalloc");
  std::vector<void *> extra;
  const int T = 128, B = (nch + T - 1) / T;
  if (ok) ok = ck(cudaMemcpy(d_in, temp.data(), sizeof(double) * nch, cudaMemcpyHostToDevice), "copy");

  /* escape peaks */
  if (ok && options->use_escape_peaks == 1 && er) {
    EscDev s;
    s.n_el = er->n_elements;
    s.nfe = er->n_fluo_input_energies;
    s.nce = er->n_compton_input_energies;
    s.nco = er->n_compton_output_energies;
    std::vector<int> ln(s.n_el, 0), lk(s.n_el * 64, 0);
    std::vector<double> le(s.n_el * 64, 0.0), edge(s.n_el * 4, 0.0);
    for (int e = 0; e < s.n_el; e++) {
      int Z = er->Z[e], n = 0;
      for (int sh = 0; sh < 4; sh++) edge[e * 4 + sh] = XD->EdgeEnergy(Z, sh);
      /* K: KL1..KP5, L1: L1M1..L1P5, L2: L2M1..L2Q1, L3: L3M1..L3P3 */
      const int ranges[4][2] = {{1, 29}, {32, 58}, {60, 85}, {86, 109}};
      for (int r = 0; r < 4; r++)
        for (int k = ranges[r][0]; k <= ranges[r][1] && n < 64; k++) {
          bool used = false;
          for (int ie = 0; ie < s.nfe && !used; ie++) used = er->fluo_escape_ratios[e + s.n_el * ((k - 1) + 109 * ie)] != 0.0;
          if (!used) continue;
          lk[e * 64 + n] = k;
          le[e * 64 + n] = XD->LineEnergy(Z, k);
          n++;
        }
      ln[e] = n;
    }
    auto up = [&](const void *src, size_t bytes) -> void * {
      void *p = nullptr;
      if (cudaMalloc(&p, bytes > 0 ? bytes : 8) != cudaSuccess) return nullptr;
      extra.push_back(p);
      if (bytes) cudaMemcpy(p, src, bytes, cudaMemcpyHostToDevice);
      return p;
    };
    s.lines_n = (const int *)up(ln.data(), sizeof(int) * ln.size());
    s.line_e = (const double *)up(le.data(), sizeof(double) * le.size());
    s.line_k = (const int *)up(lk.data(), sizeof(int) * lk.size());
    s.edge = (const double *)up(edge.data(), sizeof(double) * edge.size());
    s.fluo = (const double *)up(er->fluo_escape_ratios, sizeof(double) * (size_t)s.n_el * 109 * s.nfe);
    s.fe = (const double *)up(er->fluo_escape_input_energies, sizeof(double) * s.nfe);
    s.comp = (const double *)up(er->compton_escape_ratios, sizeof(double) * (size_t)s.nce * s.nco);
    s.ce = (const double *)up(er->compton_escape_input_energies, sizeof(double) * s.nce);
    s.co = (const double *)up(er->compton_escape_output_energies, sizeof(double) * s.nco);
    cudaMemset(d_add, 0, sizeof(double) * nch);
    escape_source_kernel<<<B, T>>>(s, d_in, nch, det->gain, det->zero, d_add, d_sr);
    escape_gather_kernel<<<B, T>>>(s, d_in, nch, det->gain, det->zero, d_add, d_sr, d_out);
    ok = ck(cudaGetLastError(), "escape kernels") && ck(cudaMemcpy(d_in, d_out, sizeof(double) * nch, cudaMemcpyDeviceToDevice), "copy");
  }

  /* pile-up */
  if (ok && options->use_sum_peaks == 1) {
    std::vector<double> h(nch), cdf(nch);
    cudaMemcpy(h.data(), d_in, sizeof(double) * nch, cudaMemcpyDeviceToHost);
    double Nt = 0.0, acc = 0.0;
    for (int i = 0; i < nch; i++) Nt += h[i];
    for (int i = 0; i < nch; i++) {
      acc += h[i] > 0.0 ? h[i] : 0.0;
      cdf[i] = acc;
    }
    long long Nt_long = (long long)Nt;
    if (Nt_long > 0 && acc > 0.0) {
      PileParams p;
      p.nch = nch;
      p.mu = 1.0 / (Nt / det->live_time);
      p.pulse_width = det->pulse_width;
      p.gain = det->gain;
      p.zero = det->zero;
      p.seed = seed_for(inputFPtr, options, 0x5055ull);
      double *d_cdf = nullptr;
      int *d_sizes = nullptr, *d_flag = nullptr;
      long long done = 0, g0 = 0, used = -1;
      const long long chunk = Nt_long < (1ll << 24) ? Nt_long : (1ll << 24);
      std::vector<int> sizes(chunk);
      ok = ck(cudaMalloc(&d_cdf, sizeof(double) * nch), "cudaMalloc") && ck(cudaMalloc(&d_flag, sizeof(int)), "cudaMalloc") &&
           ck(cudaMalloc(&d_sizes, sizeof(int) * chunk), "cudaMalloc");
      if (ok) {
        cudaMemcpy(d_cdf, cdf.data(), sizeof(double) * nch, cudaMemcpyHostToDevice);
        cudaMemset(d_flag, 0, sizeof(int));
      }
      /* every group holds at least one pulse, so Nt_long groups always reach the budget */
      while (ok && used < 0 && g0 < Nt_long) {
        long long n = Nt_long - g0 < chunk ? Nt_long - g0 : chunk;
        p.n_groups = n;
        pile_sizes_kernel<<<(unsigned)((n + 255) / 256), 256>>>(p, d_cdf, g0, d_sizes, d_flag);
        ok = ck(cudaGetLastError(), "pile sizes") &&
             ck(cudaMemcpy(sizes.data(), d_sizes, sizeof(int) * n, cudaMemcpyDeviceToHost), "pile sizes");
        for (long long g = 0; g < n && ok; g++) {
          done += sizes[g];
          if (done >= Nt_long) {
            used = g0 + g + 1;
            break;
          }
        }
        g0 += n;
      }
      int flag = 0;
      if (ok) cudaMemcpy(&flag, d_flag, sizeof(int), cudaMemcpyDeviceToHost);
      if (flag) {
        xmi_set_error("pulsetrain maximum reached: adjust the pulse width or disable pile-up");
        ok = false;
      }
      if (ok && used > 0) {
        cudaMemset(d_out, 0, sizeof(double) * nch);
        pile_tally_kernel<<<(unsigned)((used + 255) / 256), 256>>>(p, d_cdf, used, d_out);
        ok = ck(cudaGetLastError(), "pile-up") &&
             ck(cudaMemcpy(d_in, d_out, sizeof(double) * nch, cudaMemcpyDeviceToDevice), "copy");
      }
      cudaFree(d_cdf);
      cudaFree(d_sizes);
      cudaFree(d_flag);
    }
  }

  /* Gaussian convolution */
  if (ok) {
    ConvParams p;
    p.nch = nch;
    p.det_type = (int)det->detector_type;
    p.gain = det->gain;
    p.zero = det->zero;
    p.a = det->noise * det->noise;
    p.b = (double)((float)(2.3548f * 2.3548f) * 3.85f) * det->fano / 1000.0;
    p.c = sqrt(2.0) / (2.0 * sqrt(2.0 * log(2.0)));
    conv_norm_kernel<<<B, T>>>(p, d_norm);
    conv_gather_kernel<<<B, T>>>(p, d_in, d_norm, d_out);
    ok = ck(cudaGetLastError(), "convolution");
  }
  if (ok && options->use_poisson == 1) {
    poisson_kernel<<<B, T>>>(nch, seed_for(inputFPtr, options, 0x9015ull), d_out);
    ok = ck(cudaGetLastError(), "poisson");
  }
  double *res = nullptr;
  if (ok) {
    res = (double *)malloc(sizeof(double) * nch);
    ok = ck(cudaMemcpy(res, d_out, sizeof(double) * nch, cudaMemcpyDeviceToHost), "copy back");
  }
  for (void *p : extra) cudaFree(p);
  cudaFree(d_in);
  cudaFree(d_out);
  cudaFree(d_add);
  cudaFree(d_sr);
  cudaFree(d_norm);
  if (!ok) {
    free(res);
    return;
  }
  *channels_conv = res;
}

/* reference src/xmi_detector_f.F90:291-337 */
void xmi_detector_convolute_history(xmi_inputFPtr inputFPtr, double *history, xmi_main_options *options) {
  (void)options;
  if (!inputFPtr || !history) return;
  const xmi_input *in = inputFPtr->input;
  const int N = in->general->n_interactions_trajectory;
  for (int k = 1; k <= 100; k++)
    for (int j = 1; j <= 383; j++) {
      double line_energy = -1.0;
      for (int i = 1; i <= N; i++) {
        size_t idx = ((size_t)(k - 1) * 385 + (j - 1)) * N + (i - 1);
        double counts = history[idx];
        if (!(counts > 0.0)) continue;
        if (line_energy < 0.0) line_energy = XD->LineEnergy(k, j);
        if (!(line_energy > 0.0)) continue;
        double det_corr = 1.0;
        for (int l = 0; l < in->absorbers->n_det_layers; l++) {
          const xmi_layer *a = &in->absorbers->det_layers[l];
          det_corr = det_corr * exp(-1.0 * a->density * a->thickness * xmi_layer_mu(a, line_energy));
        }
        for (int l = 0; l < in->detector->n_crystal_layers; l++) {
          const xmi_layer *a = &in->detector->crystal_layers[l];
          det_corr = -1.0 * det_corr * expm1(-1.0 * a->density * a->thickness * xmi_layer_mu(a, line_energy));
        }
        history[idx] = counts * det_corr;
      }
    }
}

/* reference src/xmi_detector_f.F90:219-289 */
void xmi_detector_convolute_all(xmi_inputFPtr inputFPtr, double **channels_noconv, double **channels_conv,
                                double *brute_history, double *var_red_history, xmi_main_options *options,
                                xmi_escape_ratios *escape_ratios, int n_interactions_all, int zero_interaction) {
  int start = zero_interaction == 1 ? 0 : 1;
  for (int i = 0; i < start; i++) channels_conv[i] = nullptr;
  for (int i = start; i <= n_interactions_all; i++)
    xmi_detector_convolute_spectrum(inputFPtr, channels_noconv[i], &channels_conv[i], options, escape_ratios, i);
  if (options->use_variance_reduction == 1 && var_red_history)
    xmi_detector_convolute_history(inputFPtr, var_red_history, options);
  if (brute_history) xmi_detector_convolute_history(inputFPtr, brute_history, options);
}

void xmi_detector_convolute_all_custom(xmi_inputFPtr inputFPtr, double **channels_noconv, double **channels_conv,
                                       double *brute_history, double *var_red_history, xmi_main_options *options,
                                       xmi_escape_ratios *escape_ratios, int n_interactions_all,
                                       int zero_interaction) {
  xmi_detector_convolute_all(inputFPtr, channels_noconv, channels_conv, brute_history, var_red_history, options,
                             escape_ratios, n_interactions_all, zero_interaction);
}

/* ---------------------------------------------------------------- */
/* escape ratios                                                     */
/* ---------------------------------------------------------------- */
xmi_escape_ratios_options xmi_get_default_escape_ratios_options(void) {
  xmi_escape_ratios_options o;
  o.n_input_energies = 1990;
  o.n_compton_output_energies = 1999;
  o.n_photons = 500000;
  o.input_energy_min = 1.0;
  o.input_energy_delta = 0.1;
  o.compton_output_energy_min = 0.1;
  o.compton_output_energy_delta = 0.1;
  return o;
}

void xmi_free_escape_ratios(xmi_escape_ratios *e) {
  if (!e) return;
  free(e->Z);
  free(e->fluo_escape_ratios);
  free(e->fluo_escape_input_energies);
  free(e->compton_escape_ratios);
  free(e->compton_escape_output_energies);
  free(e->xmi_input_string);
  free(e);
}

}  // extern "C"

namespace {

struct EscTally {
  double *fluo;     /* [nE][n_el][109] */
  double *comp;     /* [nE][nco] */
  double *interacted; /* [nE] */
};

/* escape-mode histories: photon w of input energy iE (src/xmi_main.F90:5633-5755) */
template <typename R>
__global__ void __launch_bounds__(256) escape_kernel(xmi::DevBundle<R> b, xmi::DevTally t, EscTally et,
                                                     xmi_escape_ratios_options ero, long long n_total) {
  using namespace xmi;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long w = (long long)blockIdx.x * blockDim.x + threadIdx.x; w < n_total; w += stride) {
    const int iE = (int)(w / ero.n_photons);
    const double E = ero.input_energy_min + iE * ero.input_energy_delta;
    Photon<R> p;
    p.id = w;
    p.n_int = 0;
    p.last = XMI_NO_INTERACTION;
    p.hit = 0;
    p.h_type = XMI_NO_INTERACTION;
    p.h_elem = 0;
    p.h_slot = 0;
    p.elem = 0;
    p.E = (R)E;
    mu_calc(b, p.E, p.mus);
    xmi_rng g;
    xmi_rng_init(&g, b.seed, (uint64_t)w, 0u);
    /* xmi_coords_dir with a point source */
    double x1m = atan(b.slit_x / b.d_source_slit / 2.0), y1m = atan(b.slit_y / b.d_source_slit / 2.0);
    double u = xmi_rng_uniform(&g);
    double x1 = x1m * (-1.0 * (1.0 - u) + 1.0 * u);
    u = xmi_rng_uniform(&g);
    double y1 = y1m * (-1.0 * (1.0 - u) + 1.0 * u);
    p.c[0] = p.c[1] = p.c[2] = 0.0;
    double dx = tan(x1), dy = tan(y1), nn = sqrt(dx * dx + dy * dy + 1.0);
    p.d[0] = (R)(dx / nn);
    p.d[1] = (R)(dy / nn);
    p.d[2] = (R)(1.0 / nn);
    p.theta = acos(p.d[2]);
    p.phi = atan2(p.d[1], p.d[0]);
    p.w = (R)1;
    p.we = p.w;
    double te = xmi_rng_uniform(&g) * kPi * 2.0;
    p.el[0] = (R)cos(te);
    p.el[1] = (R)sin(te);
    p.el[2] = (R)0;
    R cosalfa = rdot(p.el, p.d);
    R c_alfa = acos(cosalfa);
    R c_ae = (R)1.0 / sin(c_alfa), c_be = -c_ae * cosalfa;
    for (int k = 0; k < 3; k++) p.el[k] = c_ae * p.el[k] + c_be * p.d[k];
    /* xmi_photon_shift_first_layer */
    p.layer = -1;
    if (p.c[2] >= b.zbeg[0]) {
      for (int i = 0; i < b.n_layers; i++)
        if (p.c[2] < b.zend[i]) { p.layer = i; break; }
      if (p.layer < 0) continue;
    } else {
      double ip[3], dd;
      if (!plane_step(p.c, p.d, b.n_sample, b.zbeg[0], ip, &dd)) continue;
      p.c[0] = ip[0]; p.c[1] = ip[1]; p.c[2] = ip[2];
      p.layer = 0;
    }
    if (!simulate_photon(b, p, t, xmi::VrQueue<R>{nullptr, nullptr, nullptr, 0}, 0)) continue;
    if (p.last != XMI_NO_INTERACTION) atomicAdd(&et.interacted[iE], (double)p.w);
    if (!p.inside && p.last != XMI_NO_INTERACTION) {
      if (p.last == XMI_COMPTON) {
        int ci = (int)(((double)p.E - ero.compton_output_energy_min) / ero.compton_output_energy_delta) + 1;
        if (ci >= 1 && ci <= ero.n_compton_output_energies)
          atomicAdd(&et.comp[(size_t)iE * ero.n_compton_output_energies + (ci - 1)], (double)p.w);
      } else if (p.last == XMI_PHOTOELECTRIC) {
        int line = -p.h_type;
        if (p.h_type <= -1 && p.h_type >= -109)
          atomicAdd(&et.fluo[((size_t)iE * b.n_elem + p.h_elem) * 109 + (line - 1)], (double)p.we);
      }
    }
  }
}

}  // namespace

/* The escape-mode input and tables of a detector: its crystal layers become
 * the sample (src/xmi_detector.c:91-141), run part prepared, seeded. */
static bool escape_handles(xmi_input *inputPtr, xmi_main_options *options, xmi_inputFPtr *h_out,
                           xmi_hdf5FPtr *t_out) {
  /* escape input: the detector crystal becomes the sample (src/xmi_detector.c:91-141) */
  xmi_input *esc = nullptr;
  xmi_input_copy(inputPtr, &esc);
  for (int i = 0; i < esc->composition->n_layers; i++) {
    free(esc->composition->layers[i].Z);
    free(esc->composition->layers[i].weight);
  }
  free(esc->composition->layers);
  esc->composition->n_layers = esc->detector->n_crystal_layers;
  esc->composition->layers = (xmi_layer *)calloc(esc->composition->n_layers, sizeof(xmi_layer));
  for (int i = 0; i < esc->composition->n_layers; i++) {
    const xmi_layer *a = &esc->detector->crystal_layers[i];
    xmi_layer *l = &esc->composition->layers[i];
    *l = *a;
    l->Z = (int *)malloc(sizeof(int) * a->n_elements);
    l->weight = (double *)malloc(sizeof(double) * a->n_elements);
    memcpy(l->Z, a->Z, sizeof(int) * a->n_elements);
    memcpy(l->weight, a->weight, sizeof(double) * a->n_elements);
  }
  esc->composition->reference_layer = 1;
  esc->geometry->d_sample_source = 1.0;
  esc->geometry->d_source_slit = 1.0;
  esc->geometry->slit_size_x = 0.0001;
  esc->geometry->slit_size_y = 0.0001;
  esc->geometry->n_sample_orientation[0] = 0.0;
  esc->geometry->n_sample_orientation[1] = 0.0;
  esc->geometry->n_sample_orientation[2] = 1.0;
  esc->general->n_interactions_trajectory = 1;
  esc->general->n_photons_line = 100000;

  xmi_inputFPtr h = nullptr;
  xmi_hdf5FPtr t = nullptr;
  xmi_main_options *eo = xmi_main_options_new();
  eo->use_M_lines = 0;
  eo->use_cascade_auger = 0;
  eo->use_cascade_radiative = 0;
  eo->use_variance_reduction = 0;
  eo->use_sum_peaks = 0;
  eo->escape_ratios_mode = 1;
  eo->use_advanced_compton = 0;
  eo->use_default_seeds = options ? options->use_default_seeds : 0;
  bool ok = xmi_input_C2F(esc, &h) && xmi_init_input_escape_ratios(&h);
  xmi_input_free(esc);
  if (ok) ok = xmi_init_from_hdf5(nullptr, h, &t, eo) == 1;
  if (ok) {
    xmi_bundle_set_run(h, t, eo, 1, 0, 1);
    t->b.seed = seed_for(nullptr, options, 0xE5Cull);
  }
  xmi_main_options_free(eo);
  if (!ok) {
    if (t) xmi_free_hdf5_F(&t);
    if (h) xmi_free_input_F(&h);
    return false;
  }
  *h_out = h;
  *t_out = t;
  return true;
}

extern "C" int xmi_gpu_escape_tables(xmi_input *inputPtr, xmi_main_options *options, xmi_inputFPtr *h,
                                     xmi_hdf5FPtr *t) {
  if (!inputPtr || !h || !t) {
    xmi_set_error("xmi_gpu_escape_tables: NULL argument");
    return 0;
  }
  return escape_handles(inputPtr, options, h, t) ? 1 : 0;
}

extern "C" void xmi_escape_ratios_calculation(xmi_input *inputPtr, xmi_escape_ratios **escape_ratios,
                                              char *input_string, char *hdf5_file, xmi_main_options *options,
                                              xmi_escape_ratios_options ero) {
  (void)hdf5_file;
  *escape_ratios = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    xmi_set_error("no CUDA device available: the escape-ratio Monte Carlo has no CPU fallback");
    return;
  }
  xmi_inputFPtr h = nullptr;
  xmi_hdf5FPtr t = nullptr;
  bool ok = escape_handles(inputPtr, options, &h, &t);
  xmi_escape_ratios *er = nullptr;
  if (ok) ok = xmi_dev_sync_tables(t, 0) == 1;

  if (ok) {
    const xmi_bundle &hb = t->b;
    const long nE = ero.n_input_energies, nco = ero.n_compton_output_energies;
    const int nel = hb.n_elem;
    double *d_f = nullptr, *d_c = nullptr, *d_i = nullptr, *d_tally = nullptr;
    unsigned long long *d_cnt = nullptr;
    size_t nf = (size_t)nE * nel * 109, ncp = (size_t)nE * nco;
    ok = ck(cudaMalloc(&d_f, sizeof(double) * nf), "cudaMalloc") && ck(cudaMalloc(&d_c, sizeof(double) * ncp), "cudaMalloc") &&
         ck(cudaMalloc(&d_i, sizeof(double) * nE), "cudaMalloc") && ck(cudaMalloc(&d_tally, sizeof(double) * 16), "cudaMalloc") &&
         ck(cudaMalloc(&d_cnt, sizeof(unsigned long long) * 8), "cudaMalloc");
    if (ok) {
      cudaMemset(d_f, 0, sizeof(double) * nf);
      cudaMemset(d_c, 0, sizeof(double) * ncp);
      cudaMemset(d_i, 0, sizeof(double) * nE);
      cudaMemset(d_cnt, 0, sizeof(unsigned long long) * 8);
      xmi::DevBundle<double> db;
      xmi_dev_bundle_copy64(t, &db);
      xmi::DevTally tl{d_tally, d_tally, d_tally, d_cnt};
      EscTally et{d_f, d_c, d_i};
      int dev = 0, sms = 1;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      long long n_total = (long long)nE * ero.n_photons;
      escape_kernel<double><<<sms * 4, 128>>>(db, tl, et, ero, n_total);
      ok = ck(cudaGetLastError(), "escape_kernel") && ck(cudaDeviceSynchronize(), "escape_kernel");
      unsigned long long cnt[8];
      cudaMemcpy(cnt, d_cnt, sizeof(cnt), cudaMemcpyDeviceToHost);
      if (ok && cnt[1] != 0) {
        xmi_set_error("escape kernel reported error code %llu", cnt[1]);
        ok = false;
      }
      if (ok) {
        std::vector<double> f(nf), c(ncp), it(nE);
        cudaMemcpy(f.data(), d_f, sizeof(double) * nf, cudaMemcpyDeviceToHost);
        cudaMemcpy(c.data(), d_c, sizeof(double) * ncp, cudaMemcpyDeviceToHost);
        cudaMemcpy(it.data(), d_i, sizeof(double) * nE, cudaMemcpyDeviceToHost);
        er = (xmi_escape_ratios *)calloc(1, sizeof(xmi_escape_ratios));
        er->n_elements = nel;
        er->n_fluo_input_energies = (int)nE;
        er->n_compton_input_energies = (int)nE;
        er->n_compton_output_energies = (int)nco;
        er->Z = (int *)malloc(sizeof(int) * nel);
        memcpy(er->Z, hb.elem_Z, sizeof(int) * nel);
        er->fluo_escape_input_energies = (double *)malloc(sizeof(double) * nE);
        er->compton_escape_input_energies = er->fluo_escape_input_energies;
        er->compton_escape_output_energies = (double *)malloc(sizeof(double) * nco);
        for (long i = 0; i < nE; i++) er->fluo_escape_input_energies[i] = ero.input_energy_min + i * ero.input_energy_delta;
        for (long i = 0; i < nco; i++)
          er->compton_escape_output_energies[i] = ero.compton_output_energy_min + i * ero.compton_output_energy_delta;
        er->fluo_escape_ratios = (double *)calloc(nf, sizeof(double));
        er->compton_escape_ratios = (double *)calloc(ncp, sizeof(double));
        for (long i = 0; i < nE; i++) {
          for (int e = 0; e < nel; e++)
            for (int l = 0; l < 109; l++)
              er->fluo_escape_ratios[e + (size_t)nel * (l + (size_t)109 * i)] = f[((size_t)i * nel + e) * 109 + l] / it[i];
          for (long o = 0; o < nco; o++) er->compton_escape_ratios[i + (size_t)nE * o] = c[(size_t)i * nco + o] / it[i];
        }
        er->xmi_input_string = input_string ? strdup(input_string) : nullptr;
      }
    }
    cudaFree(d_f);
    cudaFree(d_c);
    cudaFree(d_i);
    cudaFree(d_tally);
    cudaFree(d_cnt);
  }
  if (t) xmi_free_hdf5_F(&t);
  if (h) xmi_free_input_F(&h);
  *escape_ratios = er;
}

/* ---------------------------------------------------------------- */
/* Allocation-free detector convolution                               */
/* ---------------------------------------------------------------- */
/* Some callers cannot call cudaMalloc at the point where they need a
 * spectrum convolved: a real-time acquisition or spectrum-fitting loop that
 * runs under a fixed device-memory budget set up front, a host application
 * whose GPU memory is owned by another allocator (a framework's caching
 * allocator, a pool shared with other work) and must not be fragmented or
 * competed with, or code that must not block on the driver's allocator.
 * For them the convolution below uses a fixed scratch area that lives as long
 * as the library is loaded: XMI_NOALLOC_MAX_CHANNELS channels, three buffers
 * of doubles (384 KiB on every GPU that loads the library, until exit). */
#define XMI_NOALLOC_MAX_CHANNELS 16384

static __device__ __align__(256) double xmi_noalloc_scratch[3 * XMI_NOALLOC_MAX_CHANNELS];

namespace {
/* device address of the scratch array per device, looked up once per device
 * (on the first call made with that device current); the host-side symbol is
 * only a stand-in.  Threads that make their first calls at the same time may
 * each look it up; they find the same address and store it atomically.
 * The address belongs to the device's context at the time of that first
 * call: after a cudaDeviceReset() of the device the cached address is no
 * longer valid, so a process that resets a device must not call this entry
 * point on it again. */
std::atomic<double *> g_noalloc_ptr[64];

double *noalloc_scratch_for_current_device() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
    xmi_set_error("xmi_detector_convolute_spectrum_noalloc: no current CUDA device");
    return nullptr;
  }
  double *p = g_noalloc_ptr[dev].load(std::memory_order_acquire);
  if (!p) {
    cudaError_t rc = cudaGetSymbolAddress((void **)&p, xmi_noalloc_scratch);
    if (rc != cudaSuccess || !p) {
      xmi_set_error("xmi_detector_convolute_spectrum_noalloc: cudaGetSymbolAddress failed: %s",
                    cudaGetErrorString(rc));
      return nullptr;
    }
    g_noalloc_ptr[dev].store(p, std::memory_order_release);
  }
  return p;
}

/* host staging of the absorption-corrected input, per calling thread */
thread_local double g_noalloc_stage[XMI_NOALLOC_MAX_CHANNELS];
}  // namespace

extern "C" int xmi_detector_convolute_spectrum_noalloc(xmi_inputFPtr inputFPtr, const double *channels_noconv,
                                                      double *channels_conv, xmi_main_options *options) {
  if (!inputFPtr || !channels_noconv || !channels_conv || !options) {
    xmi_set_error("xmi_detector_convolute_spectrum_noalloc: NULL argument");
    return 0;
  }
  const xmi_input *in = inputFPtr->input;
  const xmi_detector *det = in->detector;
  const int nch = det->nchannels;
  if (nch < 1 || nch > XMI_NOALLOC_MAX_CHANNELS) {
    xmi_set_error("xmi_detector_convolute_spectrum_noalloc: %d channels exceed the fixed scratch of %d channels",
                  nch, XMI_NOALLOC_MAX_CHANNELS);
    return 0;
  }
  if (options->use_escape_peaks == 1 || options->use_sum_peaks == 1) {
    xmi_set_error("xmi_detector_convolute_spectrum_noalloc: escape peaks and pile-up need per-call device tables; "
                  "use xmi_detector_convolute_spectrum");
    return 0;
  }
  double *scratch = noalloc_scratch_for_current_device();
  if (!scratch) return 0;
  /* detector window / crystal absorption per channel, src/xmi_detector_f.F90:437-454 */
  for (int i = 0; i < nch; i++) {
    double E = i * det->gain + det->zero, dc = 1.0;
    for (int j = 0; j < in->absorbers->n_det_layers; j++) {
      const xmi_layer *l = &in->absorbers->det_layers[j];
      dc = dc * exp(-1.0 * l->density * l->thickness * xmi_layer_mu(l, E));
    }
    for (int j = 0; j < det->n_crystal_layers; j++) {
      const xmi_layer *l = &det->crystal_layers[j];
      dc = -1.0 * dc * expm1(-1.0 * l->density * l->thickness * xmi_layer_mu(l, E));
    }
    g_noalloc_stage[i] = channels_noconv[i] * dc;
  }
  double *d_in = scratch, *d_norm = scratch + XMI_NOALLOC_MAX_CHANNELS, *d_out = scratch + 2 * XMI_NOALLOC_MAX_CHANNELS;
  if (!ck(cudaMemcpy(d_in, g_noalloc_stage, sizeof(double) * nch, cudaMemcpyHostToDevice), "noalloc copy in"))
    return 0;
  ConvParams p;
  p.nch = nch;
  p.det_type = (int)det->detector_type;
  p.gain = det->gain;
  p.zero = det->zero;
  p.a = det->noise * det->noise;
  p.b = (double)((float)(2.3548f * 2.3548f) * 3.85f) * det->fano / 1000.0;
  p.c = sqrt(2.0) / (2.0 * sqrt(2.0 * log(2.0)));
  const int T = 128, B = (nch + T - 1) / T;
  conv_norm_kernel<<<B, T>>>(p, d_norm);
  conv_gather_kernel<<<B, T>>>(p, d_in, d_norm, d_out);
  if (!ck(cudaGetLastError(), "noalloc convolution")) return 0;
  if (options->use_poisson == 1) {
    poisson_kernel<<<B, T>>>(nch, seed_for(inputFPtr, options, 0x9015ull), d_out);
    if (!ck(cudaGetLastError(), "noalloc poisson")) return 0;
  }
  return ck(cudaMemcpy(channels_conv, d_out, sizeof(double) * nch, cudaMemcpyDeviceToHost), "noalloc copy out") ? 1
                                                                                                                : 0;
}
