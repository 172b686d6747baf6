/*
 * Host side of the engine: data-model helpers, the input handle
 * (xmi_input_C2F / xmi_init_input), and the tabulator that turns an input
 * plus the atomic data model into the table bundle the GPU kernels consume
 * (the role of xmi_init_from_hdf5, reference src/xmi_data_f.F90:164-848,
 * with the table semantics of xmi_db_Z_specific, src/xmi_data_f.F90:880-1481).
 */
#include "xmi_internal.h"
#include "xrlite.h"

#include <math.h>
#include <pthread.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------ */
/* errors and logging                                                  */
/* ------------------------------------------------------------------ */
static __thread char last_error[512];

void xmi_set_error(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(last_error, sizeof(last_error), fmt, ap);
  va_end(ap);
}

const char *xmi_gpu_last_error(void) { return last_error; }

void xmi_log(int verbose, const char *fmt, ...) {
  va_list ap;
  if (!verbose) return;
  va_start(ap, fmt);
  vfprintf(stdout, fmt, ap);
  va_end(ap);
  fflush(stdout);
}

void xmi_free(void *ptr) { free(ptr); }

/* ------------------------------------------------------------------ */
/* data model helpers                                                   */
/* ------------------------------------------------------------------ */
static char *dupstr(const char *s) {
  char *r;
  if (!s) s = "";
  r = (char *)malloc(strlen(s) + 1);
  strcpy(r, s);
  return r;
}

static void layer_copy(const xmi_layer *a, xmi_layer *b) {
  b->n_elements = a->n_elements;
  b->density = a->density;
  b->thickness = a->thickness;
  b->Z = (int *)malloc(sizeof(int) * (a->n_elements > 0 ? a->n_elements : 1));
  b->weight = (double *)malloc(sizeof(double) * (a->n_elements > 0 ? a->n_elements : 1));
  if (a->n_elements > 0) {
    memcpy(b->Z, a->Z, sizeof(int) * a->n_elements);
    memcpy(b->weight, a->weight, sizeof(double) * a->n_elements);
  }
}

static xmi_layer *layers_copy(const xmi_layer *a, int n) {
  xmi_layer *b;
  int i;
  if (n <= 0 || !a) return NULL;
  b = (xmi_layer *)calloc(n, sizeof(xmi_layer));
  for (i = 0; i < n; i++) layer_copy(&a[i], &b[i]);
  return b;
}

static void layers_free(xmi_layer *l, int n) {
  int i;
  if (!l) return;
  for (i = 0; i < n; i++) {
    free(l[i].Z);
    free(l[i].weight);
  }
  free(l);
}

static xmi_layer make_layer(int Z, double w, double rho, double t) {
  xmi_layer l;
  l.n_elements = 1;
  l.Z = (int *)malloc(sizeof(int));
  l.weight = (double *)malloc(sizeof(double));
  l.Z[0] = Z;
  l.weight[0] = w;
  l.density = rho;
  l.thickness = t;
  return l;
}

/* default input of the reference, src/xmi_data_structs.c:551-640 */
xmi_input *xmi_input_init_empty(void) {
  xmi_input *rv = (xmi_input *)calloc(1, sizeof(xmi_input));
  rv->general = (xmi_general *)calloc(1, sizeof(xmi_general));
  rv->general->version = 8.1f;
  rv->general->outputfile = dupstr("");
  rv->general->comments = dupstr("");
  rv->general->n_photons_interval = 10000;
  rv->general->n_photons_line = 100000;
  rv->general->n_interactions_trajectory = 4;

  rv->composition = (xmi_composition *)calloc(1, sizeof(xmi_composition));
  rv->composition->reference_layer = -1;

  rv->geometry = (xmi_geometry *)calloc(1, sizeof(xmi_geometry));
  rv->geometry->d_sample_source = 100.0;
  rv->geometry->n_sample_orientation[1] = -1.0 * sqrt(2.0) / 2.0;
  rv->geometry->n_sample_orientation[2] = sqrt(2.0) / 2.0;
  rv->geometry->p_detector_window[1] = 1.0;
  rv->geometry->p_detector_window[2] = 100.0;
  rv->geometry->n_detector_orientation[1] = -1.0;
  rv->geometry->area_detector = 0.3;
  rv->geometry->d_source_slit = 100.0;
  rv->geometry->slit_size_x = 0.001;
  rv->geometry->slit_size_y = 0.001;

  rv->excitation = (xmi_excitation *)calloc(1, sizeof(xmi_excitation));
  rv->excitation->n_discrete = 1;
  rv->excitation->discrete = (xmi_energy_discrete *)calloc(1, sizeof(xmi_energy_discrete));
  rv->excitation->discrete[0].energy = 28.0;
  rv->excitation->discrete[0].horizontal_intensity = 1e12;
  rv->excitation->discrete[0].vertical_intensity = 1e9;
  rv->excitation->discrete[0].distribution_type = XMI_ENERGY_DISCRETE_DISTRIBUTION_MONOCHROMATIC;

  rv->absorbers = (xmi_absorbers *)calloc(1, sizeof(xmi_absorbers));
  rv->absorbers->n_det_layers = 1;
  rv->absorbers->det_layers = (xmi_layer *)calloc(1, sizeof(xmi_layer));
  rv->absorbers->det_layers[0] = make_layer(4, 1.0, 1.85, 0.002);

  rv->detector = (xmi_detector *)calloc(1, sizeof(xmi_detector));
  rv->detector->detector_type = XMI_DETECTOR_CONVOLUTION_PROFILE_SILI;
  rv->detector->live_time = 1.0;
  rv->detector->pulse_width = 10e-6;
  rv->detector->gain = 20.0 / 1000.0;
  rv->detector->zero = 0.0;
  rv->detector->fano = 0.12;
  rv->detector->noise = 0.1;
  rv->detector->nchannels = 2048;
  rv->detector->n_crystal_layers = 1;
  rv->detector->crystal_layers = (xmi_layer *)calloc(1, sizeof(xmi_layer));
  rv->detector->crystal_layers[0] = make_layer(14, 1.0, 2.33, 0.5);
  return rv;
}

void xmi_input_free(xmi_input *in) {
  if (!in) return;
  if (in->general) {
    free(in->general->outputfile);
    free(in->general->comments);
    free(in->general);
  }
  if (in->composition) {
    layers_free(in->composition->layers, in->composition->n_layers);
    free(in->composition);
  }
  free(in->geometry);
  if (in->excitation) {
    free(in->excitation->discrete);
    free(in->excitation->continuous);
    free(in->excitation);
  }
  if (in->absorbers) {
    layers_free(in->absorbers->exc_layers, in->absorbers->n_exc_layers);
    layers_free(in->absorbers->det_layers, in->absorbers->n_det_layers);
    free(in->absorbers);
  }
  if (in->detector) {
    layers_free(in->detector->crystal_layers, in->detector->n_crystal_layers);
    free(in->detector);
  }
  free(in);
}

void xmi_input_copy(xmi_input *A, xmi_input **B) {
  xmi_input *b = (xmi_input *)calloc(1, sizeof(xmi_input));
  b->general = (xmi_general *)malloc(sizeof(xmi_general));
  *b->general = *A->general;
  b->general->outputfile = dupstr(A->general->outputfile);
  b->general->comments = dupstr(A->general->comments);
  b->composition = (xmi_composition *)malloc(sizeof(xmi_composition));
  *b->composition = *A->composition;
  b->composition->layers = layers_copy(A->composition->layers, A->composition->n_layers);
  b->geometry = (xmi_geometry *)malloc(sizeof(xmi_geometry));
  *b->geometry = *A->geometry;
  b->excitation = (xmi_excitation *)malloc(sizeof(xmi_excitation));
  *b->excitation = *A->excitation;
  b->excitation->discrete = NULL;
  b->excitation->continuous = NULL;
  if (A->excitation->n_discrete > 0) {
    b->excitation->discrete = (xmi_energy_discrete *)malloc(sizeof(xmi_energy_discrete) * A->excitation->n_discrete);
    memcpy(b->excitation->discrete, A->excitation->discrete, sizeof(xmi_energy_discrete) * A->excitation->n_discrete);
  }
  if (A->excitation->n_continuous > 0) {
    b->excitation->continuous = (xmi_energy_continuous *)malloc(sizeof(xmi_energy_continuous) * A->excitation->n_continuous);
    memcpy(b->excitation->continuous, A->excitation->continuous, sizeof(xmi_energy_continuous) * A->excitation->n_continuous);
  }
  b->absorbers = (xmi_absorbers *)malloc(sizeof(xmi_absorbers));
  *b->absorbers = *A->absorbers;
  b->absorbers->exc_layers = layers_copy(A->absorbers->exc_layers, A->absorbers->n_exc_layers);
  b->absorbers->det_layers = layers_copy(A->absorbers->det_layers, A->absorbers->n_det_layers);
  b->detector = (xmi_detector *)malloc(sizeof(xmi_detector));
  *b->detector = *A->detector;
  b->detector->crystal_layers = layers_copy(A->detector->crystal_layers, A->detector->n_crystal_layers);
  *B = b;
}

/* defaults of src/xmi_data_structs.c:2531-2547 */
xmi_main_options *xmi_main_options_new(void) {
  xmi_main_options *o = (xmi_main_options *)calloc(1, sizeof(xmi_main_options));
  o->use_M_lines = 1;
  o->use_cascade_auger = 1;
  o->use_cascade_radiative = 1;
  o->use_variance_reduction = 1;
  o->use_sum_peaks = 0;
  o->use_escape_peaks = 1;
  o->escape_ratios_mode = 0;
  o->verbose = 0;
  o->use_poisson = 0;
  o->use_gpu = 1;
  o->omp_num_threads = 1;
  o->extra_verbose = 0;
  o->custom_detector_response = NULL;
  o->use_advanced_compton = 0;
  o->use_default_seeds = 0;
  return o;
}

void xmi_main_options_free(xmi_main_options *o) {
  if (!o) return;
  free(o->custom_detector_response);
  free(o);
}

void xmi_gpu_default_options(xmi_gpu_options *g) {
  memset(g, 0, sizeof(*g));
  g->precision = 0;
  g->use_surrogate = 0;
  g->surrogate_tolerance = 1e-3;
}

/* ------------------------------------------------------------------ */
/* input handle and geometry (src/xmi_main.F90:1687-1918)              */
/* ------------------------------------------------------------------ */
static int validate_input(const xmi_input *in) {
  int i, j;
  if (!in || !in->general || !in->composition || !in->geometry || !in->excitation ||
      !in->absorbers || !in->detector) {
    xmi_set_error("incomplete xmi_input");
    return 0;
  }
  if (in->composition->n_layers < 1 || in->composition->n_layers > XMI_MAXL) {
    xmi_set_error("number of layers %d outside 1..%d", in->composition->n_layers, XMI_MAXL);
    return 0;
  }
  if (in->composition->reference_layer < 1 || in->composition->reference_layer > in->composition->n_layers) {
    xmi_set_error("invalid reference_layer %d", in->composition->reference_layer);
    return 0;
  }
  for (i = 0; i < in->composition->n_layers; i++) {
    const xmi_layer *l = &in->composition->layers[i];
    if (l->n_elements < 1) { xmi_set_error("layer %d has no elements", i + 1); return 0; }
    if (l->density <= 0.0 || l->thickness <= 0.0) { xmi_set_error("layer %d has non-positive density/thickness", i + 1); return 0; }
    for (j = 0; j < l->n_elements; j++)
      if (l->Z[j] < 1 || l->Z[j] > 94) { xmi_set_error("layer %d: Z=%d outside 1..94", i + 1, l->Z[j]); return 0; }
  }
  if (in->general->n_interactions_trajectory < 1 || in->general->n_interactions_trajectory > XMI_MAXN) {
    xmi_set_error("n_interactions_trajectory %d outside 1..%d", in->general->n_interactions_trajectory, XMI_MAXN);
    return 0;
  }
  if (in->detector->nchannels < 1 || in->detector->gain <= 0.0) {
    xmi_set_error("invalid detector channels/gain");
    return 0;
  }
  if (in->excitation->n_discrete + in->excitation->n_continuous < 1) {
    xmi_set_error("empty excitation spectrum");
    return 0;
  }
  return 1;
}

static void normalize_layers(xmi_layer *l, int n) {
  int i, j;
  for (i = 0; i < n; i++) {
    double s = 0.0;
    for (j = 0; j < l[i].n_elements; j++) s += l[i].weight[j];
    if (s > 0.0)
      for (j = 0; j < l[i].n_elements; j++) l[i].weight[j] = l[i].weight[j] / s;
  }
}

/* reference src/xmi_aux_f.F90:782-1026: copies the input and normalises the
 * weight fractions of every layer */
int xmi_input_C2F(xmi_input *input, xmi_inputFPtr *inputFPtr) {
  struct xmi_input_handle *h;
  if (!inputFPtr || !validate_input(input)) return 0;
  h = (struct xmi_input_handle *)calloc(1, sizeof(*h));
  xmi_input_copy(input, &h->input);
  normalize_layers(h->input->composition->layers, h->input->composition->n_layers);
  normalize_layers(h->input->absorbers->exc_layers, h->input->absorbers->n_exc_layers);
  normalize_layers(h->input->absorbers->det_layers, h->input->absorbers->n_det_layers);
  normalize_layers(h->input->detector->crystal_layers, h->input->detector->n_crystal_layers);
  xmi_gpu_default_options(&h->gpu);
  *inputFPtr = h;
  return 1;
}

void xmi_free_input_F(xmi_inputFPtr *p) {
  if (!p || !*p) return;
  xmi_input_free((*p)->input);
  xmi_surrogate_free((*p)->surrogate);
  free(*p);
  *p = NULL;
}

int xmi_gpu_set_options(xmi_inputFPtr h, const xmi_gpu_options *g) {
  if (!h || !g) return 0;
  if (g->precision != 0 && g->precision != 1) { xmi_set_error("precision must be 0 or 1"); return 0; }
  h->gpu = *g;
  return 1;
}

static double dot3(const double *a, const double *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static void normalize3(double *a) {
  double n = sqrt(dot3(a, a));
  a[0] /= n; a[1] /= n; a[2] /= n;
}
static void cross3(const double *a, const double *b, double *r) {
  r[0] = a[1] * b[2] - a[2] * b[1];
  r[1] = a[2] * b[0] - a[0] * b[2];
  r[2] = a[0] * b[1] - a[1] * b[0];
}

/* 3x3 inverse by cofactors (row-major) */
static int inverse3(const double *m, double *inv) {
  double det = m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) +
               m[2] * (m[3] * m[7] - m[4] * m[6]);
  if (det == 0.0) return 0;
  inv[0] = (m[4] * m[8] - m[5] * m[7]) / det;
  inv[1] = (m[2] * m[7] - m[1] * m[8]) / det;
  inv[2] = (m[1] * m[5] - m[2] * m[4]) / det;
  inv[3] = (m[5] * m[6] - m[3] * m[8]) / det;
  inv[4] = (m[0] * m[8] - m[2] * m[6]) / det;
  inv[5] = (m[2] * m[3] - m[0] * m[5]) / det;
  inv[6] = (m[3] * m[7] - m[4] * m[6]) / det;
  inv[7] = (m[1] * m[6] - m[0] * m[7]) / det;
  inv[8] = (m[0] * m[4] - m[1] * m[3]) / det;
  return 1;
}

static void layer_coordinates(struct xmi_input_handle *h) {
  const xmi_composition *c = h->input->composition;
  int ref = c->reference_layer - 1, j;
  for (j = 0; j < c->n_layers; j++) h->layer_thickz[j] = fabs(c->layers[j].thickness / h->n_sample[2]);
  h->layer_zbeg[ref] = 0.0 + h->input->geometry->d_sample_source;
  h->layer_zend[ref] = h->layer_thickz[ref] + h->input->geometry->d_sample_source;
  for (j = ref + 1; j < c->n_layers; j++) {
    h->layer_zbeg[j] = h->layer_zend[j - 1];
    h->layer_zend[j] = h->layer_zbeg[j] + h->layer_thickz[j];
  }
  for (j = ref - 1; j >= 0; j--) {
    h->layer_zend[j] = h->layer_zbeg[j + 1];
    h->layer_zbeg[j] = h->layer_zend[j] - h->layer_thickz[j];
  }
}

/* reference src/xmi_main.F90:1741-1918 */
int xmi_init_input(xmi_inputFPtr *p) {
  struct xmi_input_handle *h;
  xmi_geometry *g;
  double nx[3], ny[3], nz[3], ex[3] = {1.0, 0.0, 0.0}, ey[3] = {0.0, 1.0, 0.0}, d[3];
  double dist, half_apex;
  int r;
  if (!p || !*p) return 0;
  h = *p;
  g = h->input->geometry;
  memcpy(h->n_sample, g->n_sample_orientation, sizeof(h->n_sample));
  normalize3(h->n_sample);
  if (h->n_sample[2] < 0.0) {
    h->n_sample[0] = -h->n_sample[0]; h->n_sample[1] = -h->n_sample[1]; h->n_sample[2] = -h->n_sample[2];
  }
  memcpy(h->n_det, g->n_detector_orientation, sizeof(h->n_det));
  normalize3(h->n_det);
  memcpy(h->p_det, g->p_detector_window, sizeof(h->p_det));

  h->det_radius = sqrt(g->area_detector / M_PI);
  if (g->collimator_height > 0.0 && g->collimator_diameter > 0.0) {
    h->coll_present = 1;
    h->coll_radius = g->collimator_diameter / 2.0;
    h->coll_height = g->collimator_height;
    if (h->coll_radius >= h->det_radius) {
      xmi_set_error("Non conical collimator found");
      return 0;
    }
    h->coll_half_apex = atan((h->det_radius - h->coll_radius) / g->collimator_height);
    h->coll_vertex_x = h->det_radius / tan(h->coll_half_apex);
  } else {
    h->coll_present = 0;
    h->coll_radius = 0.0;
    h->coll_height = g->collimator_height;
  }
  memcpy(nx, h->n_det, sizeof(nx));
  /* the reference compares against the single-precision literal 1.0E-6 */
  if (fabs(dot3(nx, ex)) > (double)1.0e-6f) cross3(ey, nx, ny);
  else cross3(ex, nx, ny);
  normalize3(ny);
  cross3(nx, ny, nz);
  for (r = 0; r < 3; r++) {
    h->det_new[3 * r + 0] = nx[r];
    h->det_new[3 * r + 1] = ny[r];
    h->det_new[3 * r + 2] = nz[r];
  }
  if (!inverse3(h->det_new, h->det_inv)) {
    xmi_set_error("singular detector frame");
    return 0;
  }
  d[0] = g->p_detector_window[0];
  d[1] = g->p_detector_window[1];
  d[2] = g->p_detector_window[2] - g->d_sample_source;
  dist = sqrt(dot3(d, d));
  half_apex = atan(h->det_radius / dist);
  h->detector_solid_angle = 2 * M_PI * (1.0 - cos(half_apex));
  layer_coordinates(h);
  h->escape_geometry = 0;
  h->initialized = 1;
  return 1;
}

/* reference src/xmi_main.F90:1687-1738: only the layer coordinates */
int xmi_init_input_escape_ratios(xmi_inputFPtr *p) {
  struct xmi_input_handle *h;
  if (!p || !*p) return 0;
  h = *p;
  memcpy(h->n_sample, h->input->geometry->n_sample_orientation, sizeof(h->n_sample));
  memcpy(h->n_det, h->input->geometry->n_detector_orientation, sizeof(h->n_det));
  memcpy(h->p_det, h->input->geometry->p_detector_window, sizeof(h->p_det));
  layer_coordinates(h);
  h->escape_geometry = 1;
  h->initialized = 1;
  return 1;
}

double xmi_layer_mu(const xmi_layer *layer, double E) {
  double rv = 0.0;
  int i;
  for (i = 0; i < layer->n_elements; i++) rv += XD->CS_Total_Kissel(layer->Z[i], E) * layer->weight[i];
  return rv;
}

/* ------------------------------------------------------------------ */
/* tabulation                                                           */
/* ------------------------------------------------------------------ */
static int cmp_int(const void *a, const void *b) { return *(const int *)a - *(const int *)b; }
static int cmp_dbl(const void *a, const void *b) {
  double x = *(const double *)a, y = *(const double *)b;
  return x < y ? -1 : (x > y ? 1 : 0);
}

/* Vacancy-transfer coefficients of one element for a cascade type:
 * T[t][s] = expected new vacancies in shell s per vacancy in shell t (t < s),
 * from Coster-Kronig transitions (always), radiative lines (radiative and
 * full cascade) and non-radiative decays (Auger and full cascade).  The
 * cascade-corrected partials then follow P[s] = part[s] + sum_t T[t][s] P[t],
 * the structure of xraylib's P*_{pure,auger_cascade,rad_cascade,full_cascade}_kissel
 * called at src/xmi_variance_reduction.F90:392-571. */
static void cascade_coefficients(int Z, int cascade, double T[9][9]) {
  int aug = (cascade == XMI_CASCADE_NONRADIATIVE || cascade == XMI_CASCADE_FULL);
  int rad = (cascade == XMI_CASCADE_RADIATIVE || cascade == XMI_CASCADE_FULL);
  static const int ck_of[9][9] = {
      {-1, -1, -1, -1, -1, -1, -1, -1, -1},
      {-1, -1, XMI_FL12, XMI_FL13, -1, -1, -1, -1, -1},
      {-1, -1, -1, XMI_FL23, -1, -1, -1, -1, -1},
      {-1, -1, -1, -1, -1, -1, -1, -1, -1},
      {-1, -1, -1, -1, -1, XMI_FM12, XMI_FM13, XMI_FM14, XMI_FM15},
      {-1, -1, -1, -1, -1, -1, XMI_FM23, XMI_FM24, XMI_FM25},
      {-1, -1, -1, -1, -1, -1, -1, XMI_FM34, XMI_FM35},
      {-1, -1, -1, -1, -1, -1, -1, -1, XMI_FM45},
      {-1, -1, -1, -1, -1, -1, -1, -1, -1}};
  int s, t, l;
  memset(T, 0, sizeof(double) * 81);
  for (t = 0; t < 9; t++) {
    double w = XD->FluorYield(Z, t), a = XD->AugerYield(Z, t);
    for (s = t + 1; s < 9; s++) {
      int same_group = (t >= 1 && t <= 3 && s <= 3) || (t >= 4 && s >= 4);
      if (same_group) {
        if (ck_of[t][s] >= 0) T[t][s] = XD->CosKronTransProb(Z, ck_of[t][s]);
        continue;
      }
      if (rad)
        for (l = xrl_shell_first_line(t); l <= xrl_shell_last_line(t); l++)
          if (xrl_line_upper_shell(l) == s) T[t][s] += w * XD->RadRate(Z, l);
      if (aug) T[t][s] += a * XD->AugerVacancies(Z, t, s);
    }
  }
}

static void cascade_partials(double T[9][9], double edge_k, const double *part, double E, double *P) {
  int s, t;
  P[0] = (E >= edge_k) ? part[0] : 0.0;
  for (s = 1; s < 9; s++) {
    double v = part[s];
    for (t = 0; t < s; t++)
      if (P[t] > 0.0) v += T[t][s] * P[t];
    P[s] = v;
  }
}

/* corrected fluorescence yields, src/xmi_data_f.F90:1244-1304 */
static void yield_corr(int Z, double *y) {
  double w[9], c[XMI_NCK];
  int s;
  for (s = 0; s < 9; s++) w[s] = XD->FluorYield(Z, s);
  for (s = 0; s < XMI_NCK; s++) c[s] = XD->CosKronTransProb(Z, s);
  y[0] = w[0];
  y[1] = w[1] + c[XMI_FL12] * w[2] + (c[XMI_FL13] + c[XMI_FL12] * c[XMI_FL23]) * w[3];
  y[2] = w[2] + c[XMI_FL23] * w[3];
  y[3] = w[3];
  y[4] = w[4] + c[XMI_FM12] * w[5] + (c[XMI_FM13] + c[XMI_FM12] * c[XMI_FM23]) * w[6] +
         (c[XMI_FM14] + c[XMI_FM13] * c[XMI_FM34] + c[XMI_FM12] * c[XMI_FM24] +
          c[XMI_FM12] * c[XMI_FM23] * c[XMI_FM34]) * w[7] +
         (c[XMI_FM15] + c[XMI_FM14] * c[XMI_FM45] + c[XMI_FM13] * c[XMI_FM35] +
          c[XMI_FM12] * c[XMI_FM25] + c[XMI_FM13] * c[XMI_FM34] * c[XMI_FM45] +
          c[XMI_FM12] * c[XMI_FM24] * c[XMI_FM45] + c[XMI_FM12] * c[XMI_FM23] * c[XMI_FM35] +
          c[XMI_FM12] * c[XMI_FM23] * c[XMI_FM34] * c[XMI_FM45]) * w[8];
  y[5] = w[5] + c[XMI_FM23] * w[6] + (c[XMI_FM24] + c[XMI_FM23] * c[XMI_FM34]) * w[7] +
         (c[XMI_FM25] + c[XMI_FM24] * c[XMI_FM45] + c[XMI_FM23] * c[XMI_FM35] +
          c[XMI_FM23] * c[XMI_FM34] * c[XMI_FM45]) * w[8];
  y[6] = w[6] + c[XMI_FM34] * w[7] + (c[XMI_FM35] + c[XMI_FM34] * c[XMI_FM45]) * w[8];
  y[7] = w[7] + c[XMI_FM45] * w[8];
  y[8] = w[8];
}

/* theta inverse CDF of a differential cross section (semantics of
 * src/xmi_data_f.F90:987-1064: row over 2000 uniform r, first 0, last pi) */
static void theta_icdf(int Z, double E, int rayl, const double *rs, double *out) {
  enum { NT = 4001 };
  double cdf[NT], h = M_PI / (NT - 1), prev, sum = 0.0;
  int i, k;
  cdf[0] = 0.0;
  prev = 0.0;
  for (i = 1; i < NT; i++) {
    double th = i * h;
    double f = (rayl ? XD->DCS_Rayl(Z, E, th) : XD->DCS_Compt(Z, E, th)) * sin(th);
    sum += 0.5 * (prev + f) * h;
    cdf[i] = sum;
    prev = f;
  }
  for (i = 0; i < NT; i++) cdf[i] /= sum;
  k = 1;
  for (i = 0; i < XMI_ICDF_NR; i++) {
    double r = rs[i];
    while (k < NT - 1 && cdf[k] < r) k++;
    if (cdf[k] > cdf[k - 1])
      out[i] = (k - 1) * h + h * (r - cdf[k - 1]) / (cdf[k] - cdf[k - 1]);
    else
      out[i] = k * h;
  }
  out[0] = 0.0;
  out[XMI_ICDF_NR - 1] = M_PI;
}

/* Doppler momentum inverse CDF, src/xmi_data_f.F90:1188-1210 (pz in 0..100 a.u.);
 * the profile is the xrl_ComptonProfile shape, evaluated from per-shell
 * parameters computed once */
static void doppler_icdf(int Z, const double *rs, double *out) {
  enum { NP = 200001, NS = 29 };
  double *cdf = (double *)malloc(sizeof(double) * NP);
  double nel[NS], sig[NS];
  double h = 100.0 / (NP - 1), prev = 0.0, sum = 0.0;
  int i, k, s;
  for (s = 0; s < NS; s++) {
    double eb = XD->EdgeEnergy(Z, s);
    nel[s] = XD->ElectronConfig(Z, s);
    if (eb < 0.005) eb = 0.005;
    sig[s] = sqrt(2.0 * eb / 0.0272114);
  }
  for (i = 0; i < NP; i++) {
    double pz = i * h, f = 0.0;
    for (s = 0; s < NS; s++) {
      double x;
      if (nel[s] <= 0.0) continue;
      x = 1.0 + (pz / sig[s]) * (pz / sig[s]);
      f += nel[s] * 8.0 / (3.0 * M_PI * sig[s]) / (x * x * x);
    }
    if (i > 0) sum += 0.5 * (prev + f) * h;
    cdf[i] = sum;
    prev = f;
  }
  for (i = 0; i < NP; i++) cdf[i] /= sum;
  k = 1;
  for (i = 0; i < XMI_DOPPLER_N; i++) {
    double r = rs[i];
    while (k < NP - 1 && cdf[k] < r) k++;
    if (cdf[k] > cdf[k - 1])
      out[i] = (k - 1) * h + h * (r - cdf[k - 1]) / (cdf[k] - cdf[k - 1]);
    else
      out[i] = k * h;
  }
  out[0] = 0.0;
  out[XMI_DOPPLER_N - 1] = 100.0;
  free(cdf);
}

/* azimuthal inverse CDF, CDF(phi) = (phi - t sin(2 phi))/(2 pi), src/xmi_data_f.F90:1483-1550 */
static void phi_icdf_row(double t, const double *rs, double *out) {
  int j;
  for (j = 0; j < XMI_ICDF_NR; j++) {
    double r = rs[j], lo = 0.0, hi = 2.0 * M_PI, x = 2.0 * M_PI * r;
    int it;
    for (it = 0; it < 60; it++) {
      double f = (x - t * sin(2.0 * x)) / (2.0 * M_PI) - r;
      double d = (1.0 - 2.0 * t * cos(2.0 * x)) / (2.0 * M_PI);
      double xn;
      if (f > 0.0) hi = x; else lo = x;
      xn = (d > 1e-12) ? x - f / d : 0.5 * (lo + hi);
      if (xn <= lo || xn >= hi) xn = 0.5 * (lo + hi);
      if (fabs(xn - x) < 1e-15) { x = xn; break; }
      x = xn;
    }
    out[j] = x;
  }
  out[0] = 0.0;
  out[XMI_ICDF_NR - 1] = 2.0 * M_PI;
}

/* Tables that depend on Z alone (theta inverse CDFs on the fixed 400 x 2000
 * grid, the Doppler momentum inverse CDF, form factor and scattering
 * function): computed once per element per process and shared by every
 * bundle built afterwards -- the role of the per-Z records of the reference's
 * data file (src/xmi_data_f.F90:880-1481).  Filling is serialised; reads of
 * filled entries need no lock since entries are never modified once set. */
typedef struct {
  double *rayl, *compt, *dop, *ff2, *sf;
  int ready;
  /* per-shell Compton profiles, filled on demand (cp_ready) */
  int cp_n, cp_shell[XMI_CP_SH], cp_ready;
  double cp_occ[XMI_CP_SH], cp_edge[XMI_CP_SH], cp_sig[XMI_CP_SH];
  double *cp_cdf, *cp_qinv;
} z_tables;
static z_tables z_cache[XRL_MAXZ + 1];
static int z_cache_used = 0;

int xmi_host_tables_built(void) { return z_cache_used; }
static pthread_mutex_t z_cache_lock = PTHREAD_MUTEX_INITIALIZER;

static void z_tables_fill(const int *Zs, int n, const double *energies, const double *rs, const double *dop_rs) {
  int todo[XRL_MAXZ + 1], nt = 0, i, k;
  pthread_mutex_lock(&z_cache_lock);
  for (i = 0; i < n; i++) {
    int Z = Zs[i], seen = 0;
    if (Z < 1 || Z > XRL_MAXZ || z_cache[Z].ready) continue;
    for (k = 0; k < nt; k++) seen |= todo[k] == Z;
    if (!seen) todo[nt++] = Z;
  }
  for (k = 0; k < nt; k++) {
    z_tables *zt = &z_cache[todo[k]];
    zt->rayl = (double *)malloc(sizeof(double) * XMI_ICDF_NE * XMI_ICDF_NR);
    zt->compt = (double *)malloc(sizeof(double) * XMI_ICDF_NE * XMI_ICDF_NR);
    zt->dop = (double *)malloc(sizeof(double) * XMI_DOPPLER_N);
    zt->ff2 = (double *)malloc(sizeof(double) * XMI_NQ);
    zt->sf = (double *)malloc(sizeof(double) * XMI_NQ);
  }
#pragma omp parallel for schedule(dynamic, 4) collapse(2)
  for (k = 0; k < nt; k++)
    for (i = 0; i < XMI_ICDF_NE; i++) {
      z_tables *zt = &z_cache[todo[k]];
      theta_icdf(todo[k], energies[i], 1, rs, zt->rayl + (size_t)i * XMI_ICDF_NR);
      theta_icdf(todo[k], energies[i], 0, rs, zt->compt + (size_t)i * XMI_ICDF_NR);
    }
#pragma omp parallel for schedule(dynamic, 1)
  for (k = 0; k < nt; k++) doppler_icdf(todo[k], dop_rs, z_cache[todo[k]].dop);
  for (k = 0; k < nt; k++) {
    int Z = todo[k];
    z_tables *zt = &z_cache[Z];
    double scale = XRL_RE2 * XRL_AVOGNUM / XD->AtomicWeight(Z);
    for (i = 0; i < XMI_NQ; i++) {
      double q = XMI_QMAX * i / (XMI_NQ - 1.0);
      double ff = XD->FF_Rayl(Z, q);
      zt->ff2[i] = ff * ff * scale;
      zt->sf[i] = XD->SF_Compt(Z, q) * scale;
    }
    zt->ready = 1;
  }
  pthread_mutex_unlock(&z_cache_lock);
}

/* Per-shell Compton profile tables of the advanced Compton scattering,
 * src/xmi_data_f.F90:1124-1230.  Shells: K, then every shell L1.. with
 * electrons, each with its occupancy and binding energy.  Shell k's profile
 * is the stand-in atomic model's partial profile (the xrl_ComptonProfile
 * shape: n 8 / (3 pi s) / (1 + (pz/s)^2)^3, s from the binding energy).
 *  cdf[k][j]:  trapezoid integral of the profile over [0, Q_j] on the
 *              10001-point grid Q_j = 100 j / 10000, scaled to 0.5 at Q = 100
 *              (the reference's rule, src/xmi_data_f.F90:1189-1197);
 *  qinv[k][j]: the Q where the profile's integral, scaled the same way,
 *              reaches c_j = 0.5 j / 10000.  The reference inverts a 10^7-point
 *              trapezoid integral (src/xmi_data_f.F90:1198-1228), which
 *              converges to the exact inverse used here: the shape integrates
 *              in closed form, int_0^X (1+x^2)^-3 dx =
 *              X / (4 (1+X^2)^2) + 3 X / (8 (1+X^2)) + 3/8 atan X. */
static double cp_shape_integral(double X) {
  const double u = 1.0 + X * X;
  return X / (4.0 * u * u) + 3.0 * X / (8.0 * u) + 0.375 * atan(X);
}

static void cp_shell_tables(double sig, double *cdf, double *qinv) {
  const int N = XMI_CP_N;
  const double dq = 100.0 * 1.0 / (N - 1.0) - 100.0 * 0.0 / (N - 1.0);
  const double xm = 100.0 / sig, gm = cp_shape_integral(xm);
  double prev = 0.0, q0 = 0.0;
  int j;
  cdf[0] = 0.0;
  for (j = 0; j < N; j++) {
    const double q = 100.0 * j / (N - 1.0), x = q / sig, u = 1.0 + x * x;
    const double f = 1.0 / (u * u * u); /* the constant factor cancels in the scaling */
    if (j > 0) cdf[j] = cdf[j - 1] + dq * (f + prev) * 0.5;
    prev = f;
  }
  {
    const double last = cdf[N - 1];
    for (j = 1; j < N; j++) cdf[j] = cdf[j] * 0.5 / last;
  }
  /* inverse: G(X) / G(xm) = 2 c_j, Newton steps inside a shrinking bracket */
  qinv[0] = 0.0;
  for (j = 1; j < N - 1; j++) {
    const double target = (0.5 * j / (N - 1.0)) * 2.0 * gm;
    double lo = q0 / sig, hi = xm, x = lo;
    int it;
    for (it = 0; it < 200; it++) {
      const double g = cp_shape_integral(x) - target, u = 1.0 + x * x;
      double xn;
      if (g > 0.0) hi = x; else lo = x;
      xn = x - g * (u * u * u);
      if (!(xn > lo && xn < hi)) xn = 0.5 * (lo + hi);
      if (fabs(xn - x) <= 1e-15 * (1.0 + x)) { x = xn; break; }
      x = xn;
    }
    qinv[j] = x * sig;
    q0 = qinv[j];
  }
  qinv[N - 1] = 100.0;
}

static void cp_tables_fill(const int *Zs, int n) {
  int todo[XRL_MAXZ + 1], nt = 0, i, k, tasks = 0;
  int task_z[(XRL_MAXZ + 1) * XMI_CP_SH], task_k[(XRL_MAXZ + 1) * XMI_CP_SH];
  pthread_mutex_lock(&z_cache_lock);
  for (i = 0; i < n; i++) {
    int Z = Zs[i], seen = 0;
    if (Z < 1 || Z > XRL_MAXZ || z_cache[Z].cp_ready) continue;
    for (k = 0; k < nt; k++) seen |= todo[k] == Z;
    if (!seen) todo[nt++] = Z;
  }
  for (k = 0; k < nt; k++) {
    const int Z = todo[k];
    z_tables *zt = &z_cache[Z];
    int s, m = 0;
    for (s = 0; s < XRL_NSHELL_ALL && m < XMI_CP_SH; s++) {
      const double occ = XD->ElectronConfig(Z, s);
      double eb;
      if (s > 0 && !(occ > 0.0)) continue;
      eb = XD->EdgeEnergy(Z, s);
      zt->cp_shell[m] = s;
      zt->cp_occ[m] = occ;
      zt->cp_edge[m] = eb;
      if (eb < 0.005) eb = 0.005;
      zt->cp_sig[m] = sqrt(2.0 * eb / 0.0272114);
      task_z[tasks] = Z;
      task_k[tasks++] = m;
      m++;
    }
    zt->cp_n = m;
    zt->cp_cdf = (double *)malloc(sizeof(double) * (size_t)m * XMI_CP_N);
    zt->cp_qinv = (double *)malloc(sizeof(double) * (size_t)m * XMI_CP_N);
  }
#pragma omp parallel for schedule(dynamic, 1)
  for (i = 0; i < tasks; i++) {
    z_tables *zt = &z_cache[task_z[i]];
    const size_t o = (size_t)task_k[i] * XMI_CP_N;
    cp_shell_tables(zt->cp_sig[task_k[i]], zt->cp_cdf + o, zt->cp_qinv + o);
  }
  for (k = 0; k < nt; k++) z_cache[todo[k]].cp_ready = 1;
  pthread_mutex_unlock(&z_cache_lock);
}

int xmi_bundle_compton_profiles(xmi_bundle *b) {
  const size_t E = (size_t)(b->n_elem > 0 ? b->n_elem : 1);
  int e, k;
  if (b->cp_nshell) return 1;
  cp_tables_fill(b->elem_Z, b->n_elem);
  b->cp_nshell = (int *)calloc(E, sizeof(int));
  b->cp_shell = (int *)calloc(E * XMI_CP_SH, sizeof(int));
  b->cp_occ = (double *)calloc(E * XMI_CP_SH, sizeof(double));
  b->cp_edge = (double *)calloc(E * XMI_CP_SH, sizeof(double));
  b->cp_cdf = (const double **)calloc(E, sizeof(double *));
  b->cp_qinv = (const double **)calloc(E, sizeof(double *));
  if (!b->cp_nshell || !b->cp_shell || !b->cp_occ || !b->cp_edge || !b->cp_cdf || !b->cp_qinv) {
    xmi_set_error("out of host memory for the Compton profile tables");
    return 0;
  }
  for (e = 0; e < b->n_elem; e++) {
    const z_tables *zt = &z_cache[b->elem_Z[e]];
    b->cp_nshell[e] = zt->cp_n;
    for (k = 0; k < zt->cp_n; k++) {
      b->cp_shell[(size_t)e * XMI_CP_SH + k] = zt->cp_shell[k];
      b->cp_occ[(size_t)e * XMI_CP_SH + k] = zt->cp_occ[k];
      b->cp_edge[(size_t)e * XMI_CP_SH + k] = zt->cp_edge[k];
    }
    b->cp_cdf[e] = zt->cp_cdf;
    b->cp_qinv[e] = zt->cp_qinv;
  }
  return 1;
}

/* azimuth inverse CDFs of polarised scattering: independent of the element,
 * computed once per process and shared like the tables above */
static const double *phi_table(const double *thetas, const double *rs) {
  static double *table = NULL;
  int i;
  pthread_mutex_lock(&z_cache_lock);
  if (!table) {
    double *t = (double *)malloc(sizeof(double) * XMI_PHI_NT * XMI_ICDF_NR);
#pragma omp parallel for schedule(dynamic, 4)
    for (i = 0; i < XMI_PHI_NT; i++) phi_icdf_row(thetas[i], rs, t + (size_t)i * XMI_ICDF_NR);
    table = t;
  }
  pthread_mutex_unlock(&z_cache_lock);
  return table;
}

void xmi_bundle_free(xmi_bundle *b) {
  free(b->layer_el); free(b->layer_w); free(b->elem_Z); free(b->elem_yield_corr);
  free(b->elem_fluor_yield); free(b->elem_ck); free(b->elem_edge); free(b->elem_line_off);
  free(b->elem_shell_off); free(b->line_index); free(b->line_elem); free(b->line_shell);
  free(b->line_energy); free(b->line_rate); free(b->line_channel); free(b->precalc_mu);
  free(b->precalc_xrf); free(b->seg_lo); free(b->seg_lnlo); free(b->seg_invh); free(b->seg_lut); free(b->seg_off);
  free(b->seg_n); free(b->el_tab); free(b->mu_tab); free(b->exc_tab); free(b->icdf_energies);
  free(b->icdf_rs); free((void *)b->rayl_icdf); free((void *)b->compt_icdf); free(b->phi_thetas);
  free(b->doppler_rs); free((void *)b->doppler_icdf); free((void *)b->ff2); free((void *)b->sf);
  free(b->items);
  free(b->ent_off); free(b->ent_slot); free(b->ent_shell); free(b->ent_coef); free(b->ent_pmu);
  free(b->line_casc_shell); free(b->auger_rate);
  free(b->cp_nshell); free(b->cp_shell); free(b->cp_occ); free(b->cp_edge);
  free((void *)b->cp_cdf); free((void *)b->cp_qinv);
  memset(b, 0, sizeof(*b));
}

static double grid_eval(const xmi_bundle *b, const double *tab, int stride, int col, double E) {
  int i;
  double f;
  xmi_grid_locate(b, E, &i, &f);
  return tab[(size_t)i * stride + col] + f * (tab[(size_t)(i + 1) * stride + col] - tab[(size_t)i * stride + col]);
}

static double max_source_energy(const xmi_input *in, int *nonmono) {
  double e = 0.0;
  int i;
  *nonmono = 0;
  for (i = 0; i < in->excitation->n_discrete; i++) {
    if (in->excitation->discrete[i].energy > e) e = in->excitation->discrete[i].energy;
    if (in->excitation->discrete[i].distribution_type != XMI_ENERGY_DISCRETE_DISTRIBUTION_MONOCHROMATIC) *nonmono = 1;
  }
  for (i = 0; i < in->excitation->n_continuous; i++)
    if (in->excitation->continuous[i].energy > e) e = in->excitation->continuous[i].energy;
  return e;
}

/* builds everything that depends on the input and the cascade/M-line options */
int xmi_bundle_build(struct xmi_input_handle *in, struct xmi_tables_handle *t,
                     const xmi_main_options *options) {
  xmi_bundle *b = &t->b;
  const xmi_input *inp = in->input;
  const xmi_composition *comp = inp->composition;
  int cascade, i, j, e, s, n_pairs = 0, nonmono;
  z_cache_used = 1; /* the atomic data source is fixed from here on */
  int zs[XMI_MAXL * 128];
  int nz = 0;
  double e_lo = 0.1, e_hi, ln_span, h_target;
  double *brk;
  int n_brk;

  memset(b, 0, sizeof(*b));
  if (options->use_cascade_auger == 0 && options->use_cascade_radiative == 0) cascade = XMI_CASCADE_NONE;
  else if (options->use_cascade_auger == 1 && options->use_cascade_radiative == 0) cascade = XMI_CASCADE_NONRADIATIVE;
  else if (options->use_cascade_auger == 0 && options->use_cascade_radiative == 1) cascade = XMI_CASCADE_RADIATIVE;
  else cascade = XMI_CASCADE_FULL;
  t->cascade_type = cascade;
  t->use_M_lines = options->use_M_lines;
  b->cascade_type = cascade;
  b->use_M_lines = options->use_M_lines;
  b->line_last = options->use_M_lines ? 219 : 113;
  b->max_shell = options->use_M_lines ? 8 : 3;

  /* geometry */
  memcpy(b->n_sample, in->n_sample, sizeof(b->n_sample));
  memcpy(b->p_det, in->p_det, sizeof(b->p_det));
  memcpy(b->n_det, in->n_det, sizeof(b->n_det));
  memcpy(b->det_new, in->det_new, sizeof(b->det_new));
  memcpy(b->det_inv, in->det_inv, sizeof(b->det_inv));
  b->det_radius = in->det_radius;
  b->coll_radius = in->coll_radius;
  b->coll_height = in->coll_height;
  b->coll_present = in->coll_present;
  b->coll_half_apex = in->coll_half_apex;
  b->coll_vertex_x = in->coll_vertex_x;
  b->n_layers = comp->n_layers;
  b->reference_layer = comp->reference_layer - 1;
  b->d_source_slit = inp->geometry->d_source_slit;
  b->slit_x = inp->geometry->slit_size_x;
  b->slit_y = inp->geometry->slit_size_y;
  for (j = 0; j < comp->n_layers; j++) {
    b->layer_zbeg[j] = in->layer_zbeg[j];
    b->layer_zend[j] = in->layer_zend[j];
    b->layer_thickz[j] = in->layer_thickz[j];
    b->layer_rho[j] = comp->layers[j].density;
    b->layer_nel[j] = comp->layers[j].n_elements;
    b->layer_off[j] = n_pairs;
    n_pairs += comp->layers[j].n_elements;
    for (i = 0; i < comp->layers[j].n_elements; i++) zs[nz++] = comp->layers[j].Z[i];
  }

  /* distinct elements, sorted (hdf5F%uniqZ of the reference) */
  qsort(zs, nz, sizeof(int), cmp_int);
  b->elem_Z = (int *)malloc(sizeof(int) * nz);
  for (i = 0; i < nz; i++)
    if (b->n_elem == 0 || b->elem_Z[b->n_elem - 1] != zs[i]) b->elem_Z[b->n_elem++] = zs[i];
  for (e = 0; e < b->n_elem; e++) if (XD->prepare) XD->prepare(b->elem_Z[e]);
  for (j = 0; j < inp->absorbers->n_exc_layers; j++)
    for (i = 0; i < inp->absorbers->exc_layers[j].n_elements; i++) if (XD->prepare) XD->prepare(inp->absorbers->exc_layers[j].Z[i]);

  b->n_layer_el = n_pairs;
  b->layer_el = (int *)malloc(sizeof(int) * n_pairs);
  b->layer_w = (double *)malloc(sizeof(double) * n_pairs);
  for (j = 0; j < comp->n_layers; j++)
    for (i = 0; i < comp->layers[j].n_elements; i++) {
      int k, z = comp->layers[j].Z[i];
      for (k = 0; k < b->n_elem; k++)
        if (b->elem_Z[k] == z) break;
      b->layer_el[b->layer_off[j] + i] = k;
      b->layer_w[b->layer_off[j] + i] = comp->layers[j].weight[i];
    }

  /* per element atomic parameters */
  b->elem_yield_corr = (double *)malloc(sizeof(double) * 9 * b->n_elem);
  b->elem_fluor_yield = (double *)malloc(sizeof(double) * 9 * b->n_elem);
  b->elem_ck = (double *)malloc(sizeof(double) * XMI_NCK * b->n_elem);
  b->elem_edge = (double *)malloc(sizeof(double) * 9 * b->n_elem);
  b->elem_line_off = (int *)malloc(sizeof(int) * (b->n_elem + 1));
  b->elem_shell_off = (int *)malloc(sizeof(int) * 10 * b->n_elem);
  for (e = 0; e < b->n_elem; e++) {
    int Z = b->elem_Z[e];
    yield_corr(Z, &b->elem_yield_corr[9 * e]);
    for (s = 0; s < 9; s++) {
      b->elem_fluor_yield[9 * e + s] = XD->FluorYield(Z, s);
      b->elem_edge[9 * e + s] = XD->EdgeEnergy(Z, s);
    }
    for (s = 0; s < XMI_NCK; s++) b->elem_ck[XMI_NCK * e + s] = XD->CosKronTransProb(Z, s);
  }

  /* line slots */
  {
    int cap = 64 * b->n_elem + 16, n = 0;
    b->line_index = (int *)malloc(sizeof(int) * cap);
    b->line_elem = (int *)malloc(sizeof(int) * cap);
    b->line_shell = (int *)malloc(sizeof(int) * cap);
    b->line_energy = (double *)malloc(sizeof(double) * cap);
    b->line_rate = (double *)malloc(sizeof(double) * cap);
    b->line_channel = (int *)malloc(sizeof(int) * cap);
    for (e = 0; e < b->n_elem; e++) {
      int Z = b->elem_Z[e], l;
      b->elem_line_off[e] = n;
      for (s = 0; s <= 9; s++) b->elem_shell_off[10 * e + s] = -1;
      for (s = 0; s < 9; s++) {
        b->elem_shell_off[10 * e + s] = n;
        for (l = xrl_shell_first_line(s); l <= xrl_shell_last_line(s); l++) {
          double rr = XD->RadRate(Z, l);
          if (rr <= 0.0) continue;
          if (n >= cap) {
            cap *= 2;
            b->line_index = (int *)realloc(b->line_index, sizeof(int) * cap);
            b->line_elem = (int *)realloc(b->line_elem, sizeof(int) * cap);
            b->line_shell = (int *)realloc(b->line_shell, sizeof(int) * cap);
            b->line_energy = (double *)realloc(b->line_energy, sizeof(double) * cap);
            b->line_rate = (double *)realloc(b->line_rate, sizeof(double) * cap);
            b->line_channel = (int *)realloc(b->line_channel, sizeof(int) * cap);
          }
          b->line_index[n] = l;
          b->line_elem[n] = e;
          b->line_shell[n] = s;
          b->line_energy[n] = XD->LineEnergy(Z, l);
          b->line_rate[n] = rr;
          b->line_channel[n] = -1;
          n++;
        }
      }
      b->elem_shell_off[10 * e + 9] = n;
    }
    b->elem_line_off[b->n_elem] = n;
    b->n_lines = n;
  }
  b->n_slots = b->n_lines + 2 * b->n_elem;

  /* analog cascades: the shell a radiative cascade continues from
   * (src/xmi_main.F90:4606-4686) and the Auger transition probabilities
   * (src/xmi_main.F90:2433-2470) */
  b->line_casc_shell = (int *)malloc(sizeof(int) * (size_t)(b->n_lines > 0 ? b->n_lines : 1));
  for (i = 0; i < b->n_lines; i++) {
    const int lo = b->line_shell[i], up = xrl_line_upper_shell(b->line_index[i]);
    b->line_casc_shell[i] = -1;
    if (lo == 0 && up >= 1 && up <= 8) b->line_casc_shell[i] = up;
    if (lo >= 1 && lo <= 3 && up >= 4 && up <= 8) b->line_casc_shell[i] = up;
  }
  b->auger_rate = (double *)calloc((size_t)(b->n_elem > 0 ? b->n_elem : 1) * 4 * XMI_AUGER_K, sizeof(double));
  for (e = 0; e < b->n_elem; e++)
    for (s = 0; s < 4; s++) {
      const int nt = s == 0 ? XMI_AUGER_K : XMI_AUGER_L, t0 = s == 0 ? 0 : XMI_AUGER_K + (s - 1) * XMI_AUGER_L;
      int t;
      for (t = 0; t < nt; t++) b->auger_rate[((size_t)e * 4 + s) * XMI_AUGER_K + t] = XD->AugerRate(b->elem_Z[e], t0 + t);
    }

  /* energy grid with absorption edges as segment breakpoints */
  e_hi = max_source_energy(inp, &nonmono);
  if (nonmono) e_hi = 200.0;
  if (in->escape_geometry) e_hi = 200.0;
  e_hi = e_hi * 1.0001 + 1e-6;
  if (e_hi > 200.0) e_hi = 200.0 * 1.0001;
  brk = (double *)malloc(sizeof(double) * (9 * b->n_elem + 2));
  n_brk = 0;
  brk[n_brk++] = e_lo;
  brk[n_brk++] = e_hi;
  for (e = 0; e < b->n_elem; e++)
    for (s = 0; s < 9; s++) {
      double ed = b->elem_edge[9 * e + s];
      if (ed > e_lo && ed < e_hi) brk[n_brk++] = ed;
    }
  qsort(brk, n_brk, sizeof(double), cmp_dbl);
  {
    int m = 0;
    for (i = 0; i < n_brk; i++)
      if (m == 0 || brk[i] > brk[m - 1] * (1.0 + 1e-12)) brk[m++] = brk[i];
    n_brk = m;
  }
  if (n_brk - 1 > XMI_MAXSEG) {
    xmi_set_error("too many absorption edges in the energy range (%d)", n_brk);
    free(brk);
    return 0;
  }
  b->n_seg = n_brk - 1;
  b->seg_lo = (double *)malloc(sizeof(double) * n_brk);
  b->seg_lnlo = (double *)malloc(sizeof(double) * b->n_seg);
  b->seg_invh = (double *)malloc(sizeof(double) * b->n_seg);
  b->seg_off = (int *)malloc(sizeof(int) * b->n_seg);
  b->seg_n = (int *)malloc(sizeof(int) * b->n_seg);
  memcpy(b->seg_lo, brk, sizeof(double) * n_brk);
  ln_span = log(e_hi / e_lo);
  h_target = ln_span / 4000.0;
  b->n_nodes = 0;
  for (i = 0; i < b->n_seg; i++) {
    double len = log(brk[i + 1] / brk[i]);
    int n = (int)ceil(len / h_target) + 1;
    if (n < 2) n = 2;
    b->seg_n[i] = n;
    b->seg_off[i] = b->n_nodes;
    b->seg_lnlo[i] = log(brk[i]);
    b->seg_invh[i] = (double)(n - 1) / len;
    b->n_nodes += n;
  }
  free(brk);
  b->seg_lut = (int *)malloc(sizeof(int) * XMI_SEG_LUT);
  b->seg_lut_ln0 = log(b->seg_lo[0]);
  b->seg_lut_inv = XMI_SEG_LUT / (log(b->seg_lo[b->n_seg]) - b->seg_lut_ln0);
  {
    int lo = 0;
    for (i = 0; i < XMI_SEG_LUT; i++) {
      const double x = exp(b->seg_lut_ln0 + i / b->seg_lut_inv);
      while (lo < b->n_seg - 1 && x >= b->seg_lo[lo + 1]) lo++;
      b->seg_lut[i] = lo;
    }
  }

  /* per-node element records and layer mu */
  b->el_tab = (double *)calloc((size_t)b->n_elem * b->n_nodes * XMI_EL_REC, sizeof(double));
  b->mu_tab = (double *)calloc((size_t)b->n_nodes * XMI_MAXL, sizeof(double));
  b->exc_tab = (double *)calloc((size_t)b->n_nodes, sizeof(double));
  {
    double *node_e = (double *)malloc(sizeof(double) * b->n_nodes);
    for (i = 0; i < b->n_seg; i++) {
      int k;
      for (k = 0; k < b->seg_n[i]; k++) {
        double E = (k == b->seg_n[i] - 1) ? nextafter(b->seg_lo[i + 1], 0.0)
                                          : exp(b->seg_lnlo[i] + k / b->seg_invh[i]);
        node_e[b->seg_off[i] + k] = E;
      }
    }
    double (*T)[9][9] = (double (*)[9][9])malloc(sizeof(double) * 81 * b->n_elem);
    for (e = 0; e < b->n_elem; e++) cascade_coefficients(b->elem_Z[e], cascade, T[e]);
#pragma omp parallel for schedule(dynamic, 16) private(e, s)
    for (i = 0; i < b->n_nodes; i++) {
      double E = node_e[i];
      for (e = 0; e < b->n_elem; e++) {
        int Z = b->elem_Z[e];
        double *r = &b->el_tab[((size_t)e * b->n_nodes + i) * XMI_EL_REC];
        double cr = XD->CS_Rayl(Z, E), cc = XD->CS_Compt(Z, E), ph = XD->CS_Photo_Total(Z, E);
        double tot = cr + cc + ph, part[9], P[9];
        r[XMI_REC_TOT] = tot;
        r[XMI_REC_PR] = cr / tot;
        r[XMI_REC_PRC] = cc / tot + cr / tot;
        r[XMI_REC_PHOTO] = ph;
        for (s = 0; s < 9; s++) part[s] = r[XMI_REC_PART + s] = XD->CS_Photo_Partial(Z, s, E);
        cascade_partials(T[e], b->elem_edge[9 * e], part, E, P);
        for (s = 0; s < 9; s++) r[XMI_REC_XRF + s] = P[s];
      }
    }
    for (i = 0; i < b->n_nodes; i++) {
      double ex = 0.0;
      int k;
      for (j = 0; j < b->n_layers; j++) {
        double mu = 0.0;
        for (k = 0; k < b->layer_nel[j]; k++) {
          int p = b->layer_off[j] + k;
          mu += b->el_tab[((size_t)b->layer_el[p] * b->n_nodes + i) * XMI_EL_REC + XMI_REC_TOT] * b->layer_w[p];
        }
        b->mu_tab[(size_t)i * XMI_MAXL + j] = mu;
      }
      for (j = 0; j < inp->absorbers->n_exc_layers; j++) {
        const xmi_layer *l = &inp->absorbers->exc_layers[j];
        ex += l->density * l->thickness * xmi_layer_mu(l, node_e[i]);
      }
      b->exc_tab[i] = ex;
    }
    free(node_e);
    free(T);
  }

  /* line-energy tables derived from the grid (so that transport sees
   * mu(E_line) and P_shell(E_line) consistent with its own lookups) */
  b->precalc_mu = (double *)malloc(sizeof(double) * (size_t)(b->n_layers > 0 ? b->n_layers : 1) * (b->n_lines > 0 ? b->n_lines : 1));
  b->precalc_xrf = (double *)malloc(sizeof(double) * (size_t)b->n_elem * 9 * (b->n_lines > 0 ? b->n_lines : 1));
  for (i = 0; i < b->n_lines; i++) {
    double E = b->line_energy[i];
    for (j = 0; j < b->n_layers; j++) b->precalc_mu[(size_t)j * b->n_lines + i] = grid_eval(b, b->mu_tab, XMI_MAXL, j, E);
    for (e = 0; e < b->n_elem; e++)
      for (s = 0; s < 9; s++)
        b->precalc_xrf[((size_t)e * 9 + s) * b->n_lines + i] =
            grid_eval(b, b->el_tab + (size_t)e * b->n_nodes * XMI_EL_REC, XMI_EL_REC, XMI_REC_XRF + s, E);
  }

  /* estimator line lists per (layer, element) pair */
  {
    int k, sl, n = 0;
    b->ent_off = (int *)malloc(sizeof(int) * (size_t)(b->n_layer_el + 1));
    for (k = 0; k < b->n_layer_el; k++) {
      e = b->layer_el[k];
      b->ent_off[k] = n;
      for (sl = b->elem_line_off[e]; sl < b->elem_line_off[e + 1]; sl++) {
        int line = b->line_index[sl];
        if (line > b->line_last || b->line_energy[sl] < 1.0 || line == 30 || line == 31 || line == 59) continue;
        if (b->elem_fluor_yield[9 * e + b->line_shell[sl]] * b->line_rate[sl] == 0.0) continue;
        n++;
      }
    }
    b->ent_off[b->n_layer_el] = n;
    b->n_ent = n;
    b->ent_slot = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    b->ent_shell = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    b->ent_coef = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
    b->ent_pmu = (double *)calloc((size_t)(n > 0 ? n : 1) * XMI_MAXL, sizeof(double));
    n = 0;
    for (k = 0; k < b->n_layer_el; k++) {
      e = b->layer_el[k];
      for (sl = b->elem_line_off[e]; sl < b->elem_line_off[e + 1]; sl++) {
        int line = b->line_index[sl], sh = b->line_shell[sl];
        if (line > b->line_last || b->line_energy[sl] < 1.0 || line == 30 || line == 31 || line == 59) continue;
        if (b->elem_fluor_yield[9 * e + sh] * b->line_rate[sl] == 0.0) continue;
        b->ent_slot[n] = sl;
        b->ent_shell[n] = sh;
        b->ent_coef[n] = b->elem_fluor_yield[9 * e + sh] * b->line_rate[sl];
        for (j = 0; j < b->n_layers; j++) b->ent_pmu[(size_t)n * XMI_MAXL + j] = b->precalc_mu[(size_t)j * b->n_lines + sl];
        n++;
      }
    }
    b->stage_max = 1;
    for (j = 0; j < b->n_layers; j++) {
      int o = b->layer_off[j], ne = b->layer_nel[j];
      int m = b->ent_off[o + ne] - b->ent_off[o] + 2 * ne;
      if (m > b->stage_max) b->stage_max = m;
    }
  }

  /* angular tables */
  b->icdf_energies = (double *)malloc(sizeof(double) * XMI_ICDF_NE);
  b->icdf_rs = (double *)malloc(sizeof(double) * XMI_ICDF_NR);
  for (i = 0; i < XMI_ICDF_NE; i++) b->icdf_energies[i] = 0.1 + (200.0 - 0.1) * i / (XMI_ICDF_NE - 1.0);
  for (i = 0; i < XMI_ICDF_NR; i++) b->icdf_rs[i] = (double)i / (XMI_ICDF_NR - 1.0);
  b->doppler_rs = (double *)malloc(sizeof(double) * XMI_DOPPLER_N);
  for (i = 0; i < XMI_DOPPLER_N; i++) b->doppler_rs[i] = (double)i / (XMI_DOPPLER_N - 1.0);
  b->rayl_icdf = (const double **)malloc(sizeof(double *) * (size_t)(b->n_elem > 0 ? b->n_elem : 1));
  b->compt_icdf = (const double **)malloc(sizeof(double *) * (size_t)(b->n_elem > 0 ? b->n_elem : 1));
  b->doppler_icdf = (const double **)malloc(sizeof(double *) * (size_t)(b->n_elem > 0 ? b->n_elem : 1));
  b->ff2 = (const double **)malloc(sizeof(double *) * (size_t)(b->n_elem > 0 ? b->n_elem : 1));
  b->sf = (const double **)malloc(sizeof(double *) * (size_t)(b->n_elem > 0 ? b->n_elem : 1));
  z_tables_fill(b->elem_Z, b->n_elem, b->icdf_energies, b->icdf_rs, b->doppler_rs);
  for (e = 0; e < b->n_elem; e++) {
    const z_tables *zt = &z_cache[b->elem_Z[e]];
    b->rayl_icdf[e] = zt->rayl;
    b->compt_icdf[e] = zt->compt;
    b->doppler_icdf[e] = zt->dop;
    b->ff2[e] = zt->ff2;
    b->sf[e] = zt->sf;
  }
  b->phi_thetas = (double *)malloc(sizeof(double) * XMI_PHI_NT);
  for (i = 0; i < XMI_PHI_NT; i++) b->phi_thetas[i] = 0.5 * i / (XMI_PHI_NT - 1.0);
  b->phi_icdf = phi_table(b->phi_thetas, b->icdf_rs);
  return 1;
}

static uint64_t random_seed(void) {
  uint64_t s = 0;
  FILE *f = fopen("/dev/urandom", "rb");
  if (f) {
    if (fread(&s, sizeof(s), 1, f) != 1) s = 0;
    fclose(f);
  }
  if (s == 0) s = 0x9E3779B97F4A7C15ull ^ (uint64_t)(size_t)&s;
  return s;
}

/* run-dependent part: options, detector channel mapping and source items
 * (photon budget and weights of src/xmi_main.F90:240-858).  Replica r of R
 * simulates photons [r*n/R, (r+1)*n/R) of every item. */
void xmi_bundle_set_run(struct xmi_input_handle *in, struct xmi_tables_handle *t,
                        const xmi_main_options *options, int n_mpi_hosts,
                        int replica, int n_replicas) {
  xmi_bundle *b = &t->b;
  const xmi_input *inp = in->input;
  const xmi_excitation *exc = inp->excitation;
  int i, n = 0;
  int64_t first = 0;
  (void)n_mpi_hosts;
  b->n_interactions = inp->general->n_interactions_trajectory;
  b->use_vr = options->use_variance_reduction;
  b->escape_mode = options->escape_ratios_mode;
  b->use_advanced_compton = options->use_advanced_compton == 1;
  b->nchannels = inp->detector->nchannels;
  b->gain = inp->detector->gain;
  b->zero = inp->detector->zero;
  b->live_time = inp->detector->live_time;
  if (in->gpu.seed != 0) b->seed = in->gpu.seed;
  else if (options->use_default_seeds) b->seed = 0x5EED0001ull;
  else b->seed = random_seed();
  for (i = 0; i < b->n_lines; i++) {
    double E = b->line_energy[i];
    int ch = -1;
    if (E >= 1.0) ch = (int)((E - b->zero) / b->gain);
    b->line_channel[i] = (ch >= 0 && ch < b->nchannels) ? ch : -1;
  }

  free(b->items);
  b->items = (xmi_source_item *)calloc((size_t)(exc->n_continuous + exc->n_discrete + 1), sizeof(xmi_source_item));
  if (n_replicas < 1) n_replicas = 1;
  /* continuous intervals, src/xmi_main.F90:319-343 */
  for (i = 0; i + 1 < exc->n_continuous; i++) {
    const xmi_energy_continuous *c0 = &exc->continuous[i], *c1 = &exc->continuous[i + 1];
    xmi_source_item *it = &b->items[n];
    double i0 = c0->vertical_intensity + c0->horizontal_intensity;
    double i1 = c1->vertical_intensity + c1->horizontal_intensity;
    double total = (i0 + i1) * (c1->energy - c0->energy) / 2.0;
    int64_t np = inp->general->n_photons_interval;
    if (total == 0.0) continue;
    it->kind = 0;
    it->e0 = c0->energy;
    it->e1 = c1->energy;
    it->i0 = i0;
    it->i1 = i1;
    it->h0 = c0->horizontal_intensity;
    it->h1 = c1->horizontal_intensity;
    it->weight = total / (double)inp->general->n_photons_interval;
    it->trap[1] = (i1 - i0) / (c1->energy - c0->energy);
    it->trap[0] = (c1->energy - c0->energy) * (i0 - c0->energy * it->trap[1]) +
                  it->trap[1] * (c1->energy * c1->energy - c0->energy * c0->energy) / 2.0;
    it->trap[2] = c0->energy;
    it->trap[3] = c1->energy;
    it->trap[4] = i0;
    it->trap[5] = i1;
    it->sigma_x = c0->sigma_x;
    it->sigma_xp = c0->sigma_xp;
    it->sigma_y = c0->sigma_y;
    it->sigma_yp = c0->sigma_yp;
    it->first = first + np * replica / n_replicas;
    it->n_photons = np * (replica + 1) / n_replicas - np * replica / n_replicas;
    it->local0 = np * replica / n_replicas;
    first += np;
    n++;
  }
  /* discrete lines, src/xmi_main.F90:579-620 */
  for (i = 0; i < exc->n_discrete; i++) {
    const xmi_energy_discrete *d = &exc->discrete[i];
    xmi_source_item *it = &b->items[n];
    double total = d->vertical_intensity + d->horizontal_intensity, exc_corr = 1.0;
    int64_t np = inp->general->n_photons_line;
    int j;
    for (j = 0; j < inp->absorbers->n_exc_layers; j++) {
      const xmi_layer *l = &inp->absorbers->exc_layers[j];
      exc_corr *= exp(-1.0 * l->density * l->thickness * xmi_layer_mu(l, d->energy));
    }
    it->kind = 1;
    it->dist_type = (int)d->distribution_type;
    it->e0 = d->energy;
    it->scale = d->scale_parameter;
    it->hor_ver_ratio = d->horizontal_intensity * (double)np / total;
    it->weight = total * exc_corr / (double)np;
    it->sigma_x = d->sigma_x;
    it->sigma_xp = d->sigma_xp;
    it->sigma_y = d->sigma_y;
    it->sigma_yp = d->sigma_yp;
    it->first = first + np * replica / n_replicas;
    it->n_photons = np * (replica + 1) / n_replicas - np * replica / n_replicas;
    it->local0 = np * replica / n_replicas;
    first += np;
    n++;
  }
  b->n_items = n;
  b->n_photons_total = 0;
  for (i = 0; i < n; i++) b->n_photons_total += b->items[i].n_photons;
}

int xmi_update_input_from_hdf5(xmi_inputFPtr inputFPtr, xmi_hdf5FPtr hdf5FPtr) {
  return (inputFPtr && hdf5FPtr) ? 1 : 0;
}

int xmi_init_from_hdf5(char *hdf5_file, xmi_inputFPtr inputFPtr, xmi_hdf5FPtr *hdf5FPtr,
                       xmi_main_options *options) {
  struct xmi_tables_handle *t;
  xmi_main_options *def = NULL;
  (void)hdf5_file;
  if (!inputFPtr || !hdf5FPtr) {
    xmi_set_error("xmi_init_from_hdf5: NULL handle");
    return 0;
  }
  if (!inputFPtr->initialized) {
    xmi_set_error("xmi_init_from_hdf5: call xmi_init_input first");
    return 0;
  }
  if (!options) options = def = xmi_main_options_new();
  t = (struct xmi_tables_handle *)calloc(1, sizeof(*t));
  if (!xmi_bundle_build(inputFPtr, t, options)) {
    xmi_bundle_free(&t->b);
    free(t);
    xmi_main_options_free(def);
    return 0;
  }
  xmi_main_options_free(def);
  *hdf5FPtr = t;
  return 1;
}

const void *xmi_gpu_bundle(xmi_hdf5FPtr t) { return t ? (const void *)&t->b : NULL; }

int xmi_gpu_set_replica(xmi_hdf5FPtr t, int replica, int n_replicas) {
  if (!t || n_replicas < 1 || replica < 0 || replica >= n_replicas) {
    xmi_set_error("xmi_gpu_set_replica: invalid replica %d of %d", replica, n_replicas);
    return 0;
  }
  t->replica = replica;
  t->n_replicas = n_replicas;
  return 1;
}

/* grid axes of the solid-angle table, xmi_solid_angle_inputs_f
 * (src/xmi_solid_angle_f.F90:62-301): r from the detector distance of the
 * depths S1/S2 at which R1=1e-5 / R2=0.99999 of the beam is absorbed at the
 * lowest/highest excitation energy, theta in [1e-5, pi/2] */
static double s_depth(const struct xmi_input_handle *h, double energy, double R) {
  const xmi_composition *c = h->input->composition;
  double mu[XMI_MAXL], my_sum = 0.0, pabs, myln;
  int i, m = c->n_layers - 1;
  for (i = 0; i < c->n_layers; i++) {
    mu[i] = xmi_layer_mu(&c->layers[i], energy);
    my_sum = my_sum + mu[i] * c->layers[i].density * h->layer_thickz[i];
  }
  pabs = -1.0 * expm1(-1.0 * my_sum);
  myln = -1.0 * log1p(-1.0 * R * pabs);
  my_sum = 0.0;
  for (i = 0; i < c->n_layers; i++) {
    my_sum = my_sum + mu[i] * c->layers[i].density * h->layer_thickz[i];
    if (my_sum > myln) {
      m = i - 1;
      break;
    }
  }
  my_sum = 0.0;
  for (i = 0; i <= m; i++)
    my_sum = my_sum + (1.0 - (mu[i] * c->layers[i].density) / (mu[m + 1] * c->layers[m + 1].density)) * h->layer_thickz[i];
  return my_sum + myln / (mu[m + 1] * c->layers[m + 1].density) + h->layer_zbeg[0];
}

void xmi_solid_angle_axes(const struct xmi_input_handle *h, int nr, int nt, double *r_vals, double *t_vals) {
  const xmi_excitation *e = h->input->excitation;
  double emin, emax, s1, s2, d1, d2, r0, r1, t0 = 0.00001, t1 = M_PI / 2.0, p[3];
  int i;
  if (e->n_continuous > 1 && e->n_discrete > 0) {
    emin = fmin(e->continuous[0].energy, e->discrete[0].energy);
    emax = fmax(e->continuous[e->n_continuous - 1].energy, e->discrete[e->n_discrete - 1].energy);
  } else if (e->n_continuous > 1) {
    emin = e->continuous[0].energy;
    emax = e->continuous[e->n_continuous - 1].energy;
  } else {
    emin = e->discrete[0].energy;
    emax = e->discrete[e->n_discrete - 1].energy;
  }
  s1 = s_depth(h, emin, 0.00001);
  s2 = s_depth(h, emax, 0.99999);
  memcpy(p, h->input->geometry->p_detector_window, sizeof(p));
  d1 = sqrt(p[0] * p[0] + p[1] * p[1] + (s1 - p[2]) * (s1 - p[2]));
  d2 = sqrt(p[0] * p[0] + p[1] * p[1] + (s2 - p[2]) * (s2 - p[2]));
  r1 = fmax(d1, d2) * 1.25;
  r0 = r1 / nr;
  for (i = 0; i < nr; i++) r_vals[i] = r0 + (r1 - r0) * (double)i / (double)(nr - 1);
  for (i = 0; i < nt; i++) t_vals[i] = t0 + (t1 - t0) * (double)i / (double)(nt - 1);
}

#include "philox.h"
/* raw Philox4x32-10 block of the engine's generator (known-answer tests) */
void xmi_gpu_philox_block(const uint32_t *ctr, const uint32_t *key, uint32_t *out) {
  xmi_u32x4 c, r;
  int i;
  for (i = 0; i < 4; i++) c.v[i] = ctr[i];
  r = xmi_philox4x32_10(c, key[0], key[1]);
  for (i = 0; i < 4; i++) out[i] = r.v[i];
}

/* raw Threefry4x32-20 block of the engine's reference solid-angle stream */
void xmi_gpu_threefry_block(const uint32_t *ctr, const uint32_t *key, uint32_t *out) {
  xmi_u32x4 c, k, r;
  int i;
  for (i = 0; i < 4; i++) {
    c.v[i] = ctr[i];
    k.v[i] = key[i];
  }
  r = xmi_threefry4x32_20(c, k);
  for (i = 0; i < 4; i++) out[i] = r.v[i];
}

/* exported names of the atomic data model and the line table (used by the
 * host-side tube model and by tests) */
const char *xmi_gpu_line_name(int line) { return xrl_line_name(line); }
