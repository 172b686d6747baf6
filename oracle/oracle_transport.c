/*
 * TEST INFRASTRUCTURE (oracle) -- not part of the engine.
 *
 * FP64 CPU restatement of the reference photon transport:
 *   xmi_main_msim            src/xmi_main.F90:66-954
 *   xmi_coords_dir_*         src/xmi_main.F90:957-1136
 *   xmi_photon_shift_first_layer src/xmi_main.F90:1140-1186
 *   xmi_simulate_photon      src/xmi_main.F90:1188-1685
 *   xmi_check_photon_detector_hit src/xmi_main.F90:1920-1984
 *   xmi_simulate_photon_rayleigh/compton/fluorescence src/xmi_main.F90:1986-2411
 *   xmi_update_photon_energy_compton2 src/xmi_main.F90:4985-5067
 *   xmi_simulate_photon_cascade_auger/radiative src/xmi_main.F90:2413-4783
 *   xmi_update_photon_energy_compton (advanced) src/xmi_main.F90:4785-4983,
 *   xmi_compton_varred src/xmi_variance_reduction.F90:752-947,
 *   xmi_get_qimax / xmi_get_energy_from_q / xmi_get_q_from_energy
 *   src/xmi_aux_f.F90:1951-2074
 *   xmi_update_photon_dirv/elecv src/xmi_main.F90:5071-5182
 *   xmi_coster_kronig_check, xmi_fluorescence_yield_check,
 *   xmi_fluorescence_line_check src/xmi_main.F90:5184-5437
 *   xmi_variance_reduction, xmi_compton_varred2,
 *   xmi_update_photon_energy_compton_var_red src/xmi_variance_reduction.F90:29-1101
 *   xmi_get_solid_angle, xmi_single_solid_angle_calculation src/xmi_solid_angle_f.F90:432-801
 *   helpers (findpos, bilinear_interpolation, intersection, ran_trap,
 *   poly_solve_quadratic, check_detector_intersection) src/xmi_aux_f.F90:1109-1941
 * It reads the same table bundle as the GPU engine and draws its random
 * numbers from the same Philox streams (photon, phase, draw), so single
 * photons replay identically; it tallies straight into the reference
 * output layouts (channels cumulative per order, 100x385xN histories).
 *
 * Deliberate differences from the reference (same in the engine): Philox
 * streams instead of per-thread MT19937, Box-Muller instead of the ziggurat
 * Gaussian, tables from the bundle instead of xraylib calls.  The offspring
 * of an analog cascade draws from streams of its own (id | 2^62) instead of
 * continuing its parent's stream, and is walked after its parent.
 */
#include "../include/xmimsim_bundle.h"
#include "oracle_rng.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define O_ENERGY_THRESHOLD 1.0
#define O_ENERGY_MAX 200.0
#define O_NO_INTERSECTION 0
#define O_COLLIMATOR_INTERSECTION 1
#define O_DETECTOR_INTERSECTION 2
#define O_DETECTOR_BAD_INTERSECTION 3

/* physical constants of src/xmi_main.F90:47-57 */
static const double O_MEC2 = 9.10938188e-31 * 2.99792458e8 * 2.99792458e8 / 1.602176487e-19 / 1000.0;

/* algorithmic table words read per lookup (interpolation corners counted
 * once), accumulated per thread to define the roofline bytes per history */
static __thread long long o_words = 0, o_words_est = 0;
static long long o_words_total = 0, o_words_est_total = 0;

typedef struct {
  double coords[3], dirv[3], elecv[3];
  double theta, phi, energy, weight, weight_escape;
  double mus[XMI_MAXL];
  int cur_layer;          /* 0-based */
  int cur_elem;           /* element index (bundle) */
  int cur_elem_in_layer;  /* index within the layer */
  int n_int;
  int last_interaction;
  int inside;
  int detector_hit;
  int hist_type[XMI_MAXN + 2];   /* RAYLEIGH/COMPTON or -line for fluorescence */
  int hist_elem[XMI_MAXN + 2];   /* element index */
  int hist_slot[XMI_MAXN + 2];   /* line slot of the emitted line */
  int64_t id;
  long sa_not_found;
  int casc_used;          /* the photon's analog cascade has been simulated (its cascade options are off) */
} ophoton;

/* offspring photons of the analog cascades draw from the streams of this id */
#define O_OFFSPRING_ID (1ll << 62)

typedef struct {
  double *channels;  /* [(N+1)][nch] cumulative */
  double *var_red;   /* [100][385][N] */
  double *brute;     /* [100][385][N] */
  long not_found;
  int error;
} otally;

static double dot3(const double *a, const double *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static double norm3(const double *a) { return sqrt(dot3(a, a)); }
static void normalize3(double *a) {
  double n = norm3(a);
  a[0] /= n; a[1] /= n; a[2] /= n;
}
static void matvec(const double *m, const double *v, double *r) {
  r[0] = m[0] * v[0] + m[1] * v[1] + m[2] * v[2];
  r[1] = m[3] * v[0] + m[4] * v[1] + m[5] * v[2];
  r[2] = m[6] * v[0] + m[7] * v[1] + m[8] * v[2];
}
static void cross3(const double *a, const double *b, double *r) {
  r[0] = a[1] * b[2] - a[2] * b[1];
  r[1] = a[2] * b[0] - a[0] * b[2];
  r[2] = a[0] * b[1] - a[1] * b[0];
}
static double dist3(const double *a, const double *b) {
  return sqrt((a[0] - b[0]) * (a[0] - b[0]) + (a[1] - b[1]) * (a[1] - b[1]) + (a[2] - b[2]) * (a[2] - b[2]));
}

/* xmi_intersection_plane_line, src/xmi_aux_f.F90:1143-1170 */
static int intersect_plane(const double *ppoint, const double *pnorm, const double *lpoint,
                           const double *ldir, double *out) {
  double itn = dot3(ldir, pnorm), d, diff[3];
  if (itn == 0.0) return 0;
  diff[0] = ppoint[0] - lpoint[0];
  diff[1] = ppoint[1] - lpoint[1];
  diff[2] = ppoint[2] - lpoint[2];
  d = dot3(diff, pnorm) / itn;
  out[0] = d * ldir[0] + lpoint[0];
  out[1] = d * ldir[1] + lpoint[1];
  out[2] = d * ldir[2] + lpoint[2];
  return 1;
}

/* findpos, src/xmi_aux_f.F90:1305-1335 (0-based result, -1 when not found) */
static int findpos(const double *a, int n, double x) {
  int i;
  if (fabs(x - a[0]) < 1e-10) return 0;
  for (i = 1; i < n; i++)
    if (x <= a[i]) return i - 1;
  return -1;
}

/* bilinear_interpolation, src/xmi_aux_f.F90:1337-1428; array2d[i2*n1 + i1] */
static double bilinear(const double *a2, const double *a1, int n1, const double *b1, int n2,
                       double x1, double x2, int *err) {
  int p1 = findpos(a1, n1, x1), p2 = findpos(b1, n2, x2);
  double denom, c1, c2, c3, c4;
  o_words += 4;
  if (p1 < 0 || p2 < 0) {
    *err = 1;
    return 0.0;
  }
  denom = (a1[p1 + 1] - a1[p1]) * (b1[p2 + 1] - b1[p2]);
  c1 = (a1[p1 + 1] - x1) * (b1[p2 + 1] - x2) / denom;
  c2 = (x1 - a1[p1]) * (b1[p2 + 1] - x2) / denom;
  c3 = (a1[p1 + 1] - x1) * (x2 - b1[p2]) / denom;
  c4 = (x1 - a1[p1]) * (x2 - b1[p2]) / denom;
  return c1 * a2[(size_t)p2 * n1 + p1] + c2 * a2[(size_t)p2 * n1 + p1 + 1] +
         c3 * a2[(size_t)(p2 + 1) * n1 + p1] + c4 * a2[(size_t)(p2 + 1) * n1 + p1 + 1];
}

/* interpolate_simple, src/xmi_aux_f.F90:1267-1276 */
static double interp_simple(double ax, double ay, double bx, double by, double c) {
  return ay + ((by - ay) * (c - ax) / (bx - ax));
}

/* table evaluation on the bundle's energy grid */
static double grid_val(const xmi_bundle *b, const double *tab, int stride, int col, int node, double f) {
  o_words += 2;
  double v0 = tab[(size_t)node * stride + col], v1 = tab[(size_t)(node + 1) * stride + col];
  return v0 + f * (v1 - v0);
}
static void mu_calc(const xmi_bundle *b, double E, double *mus) {
  int node, j;
  double f;
  xmi_grid_locate(b, E, &node, &f);
  for (j = 0; j < b->n_layers; j++) mus[j] = grid_val(b, b->mu_tab, XMI_MAXL, j, node, f);
}
static double el_val(const xmi_bundle *b, int e, int col, int node, double f) {
  return grid_val(b, b->el_tab + (size_t)e * b->n_nodes * XMI_EL_REC, XMI_EL_REC, col, node, f);
}

/* linear interpolation on a uniform q grid */
static double qtab(const double *t, double q) {
  o_words += 2;
  double x = q * (XMI_NQ - 1) / XMI_QMAX, f;
  int i = (int)x;
  if (i < 0) i = 0;
  if (i > XMI_NQ - 2) i = XMI_NQ - 2;
  f = x - i;
  return t[i] + f * (t[i + 1] - t[i]);
}

/* DCSP_Rayl and DCSP_Compt (xraylib) from the bundle's form-factor tables */
static double dcsp_rayl(const xmi_bundle *b, int e, double E, double theta, double phi) {
  double q = E / 12.39852 * sin(theta / 2.0), st = sin(theta), cp = cos(phi);
  return (1.0 - st * st * cp * cp) * qtab(b->ff2[e], q);
}
static double dcsp_compt(const xmi_bundle *b, int e, double E, double theta, double phi) {
  double q = E / 12.39852 * sin(theta / 2.0), ct = cos(theta), st = sin(theta), cp = cos(phi);
  double k0k = 1.0 + (1.0 - ct) * E / 510.998928, kk0 = 1.0 / k0k;
  double kn = 0.25 * kk0 * kk0 * (kk0 + k0k - 2.0 * st * st * cp * cp);
  return kn * qtab(b->sf[e], q);
}

/* ------------------------------------------------------------------ */
/* solid angle                                                          */
/* ------------------------------------------------------------------ */
/* xmi_single_solid_angle_calculation, src/xmi_solid_angle_f.F90:432-710 */
typedef double (*ouniform_fn)(void *);
static double ouni_philox(void *g) { return orng_uniform((orng *)g); }
static double ouni_cl(void *g) { return oclrng_uniform((oclrng *)g); }

static double single_solid_angle(const xmi_bundle *b, double r1, double theta1, ouniform_fn uni, void *g,
                                 long hits_per_single) {
  double r, theta, fcbr, beta, alpha1, fca, cfca, fcsa, rot[9];
  double line_point[3];
  long hits = 0, i;
  int outside;
  const double detr = b->det_radius, collr = b->coll_radius, collh = b->coll_height;
  if (!b->coll_present) {
    r = r1;
    theta = theta1;
    fcbr = detr;
    outside = 0;
  } else if (fabs(collr - detr) < 0.000001) {
    if (r1 * cos(theta1) <= detr) {
      r = r1;
      theta = theta1;
      fcbr = detr;
    } else {
      r = sqrt(r1 * r1 - 2.0 * r1 * sin(theta1) * collh + collh * collh);
      theta = acos(r1 * cos(theta1) / r);
      fcbr = collr;
    }
    outside = (r1 * sin(theta1) > collh);
  } else {
    if (r1 * cos(theta1) <= detr && r1 * sin(theta1) <= collh * (r1 * cos(theta1) - detr) / (collr - detr)) {
      r = r1;
      theta = theta1;
      fcbr = detr;
    } else if (r1 * sin(theta1) <= collh) {
      return 0.0;
    } else {
      r = sqrt(r1 * r1 - 2.0 * r1 * sin(theta1) * collh + collh * collh);
      theta = acos(r1 * cos(theta1) / r);
      fcbr = collr;
    }
    outside = (r1 * sin(theta1) > collh);
  }
  beta = atan(fcbr / r);
  alpha1 = atan(fcbr * sin(theta) / (r - fcbr * cos(theta)));
  if (alpha1 <= 0.0) alpha1 = alpha1 + M_PI;
  fca = beta > alpha1 ? beta : alpha1;
  cfca = cos(fca);
  fcsa = 2 * M_PI * (1.0 - cfca);
  /* rows of the rotation matrix (columns of the Fortran one) */
  rot[0] = 1.0; rot[1] = 0.0; rot[2] = 0.0;
  rot[3] = 0.0; rot[4] = -1.0 * sin(theta); rot[5] = -1.0 * cos(theta);
  rot[6] = 0.0; rot[7] = cos(theta); rot[8] = -1.0 * sin(theta);
  line_point[0] = 0.0;
  line_point[1] = r1 * cos(theta1);
  line_point[2] = r1 * sin(theta1);
  for (i = 0; i < hits_per_single; i++) {
    double th = acos(1.0 - uni(g) * (1.0 - cfca));
    double ph = uni(g) * 2.0 * M_PI;
    double dc[3], dd[3], ip[3];
    static const double dn[3] = {0.0, 0.0, 1.0}, origin[3] = {0.0, 0.0, 0.0};
    dc[0] = sin(th) * cos(ph);
    dc[1] = sin(th) * sin(ph);
    dc[2] = cos(th);
    matvec(rot, dc, dd);
    if (dot3(dn, dd) >= 0.0) continue;
    if (outside) {
      double cp[3] = {0.0, 0.0, collh};
      if (!intersect_plane(cp, dn, line_point, dd, ip)) continue;
      ip[2] = 0.0;
      if (norm3(ip) > collr) continue;
    }
    if (!intersect_plane(origin, dn, line_point, dd, ip)) continue;
    if (norm3(ip) <= detr) hits++;
  }
  return fcsa * (double)hits / (double)hits_per_single;
}

double oracle_single_solid_angle(const xmi_bundle *b, double r1, double theta1, orng *g, long hits_per_single) {
  return single_solid_angle(b, r1, theta1, ouni_philox, g, hits_per_single);
}

/* grid points (ir[k], it[k]) with the OpenCL kernel's Threefry stream, for
 * the point-by-point comparison with that kernel */
void oracle_solid_angle_points_cl_stream(const xmi_bundle *b, const double *r_vals, const double *t_vals,
                                         const int *ir, const int *it, int n, long hits_per_single, double *out) {
  int k;
#pragma omp parallel for schedule(dynamic, 1)
  for (k = 0; k < n; k++) {
    oclrng g;
    oclrng_init(&g, (uint32_t)ir[k], (uint32_t)it[k]);
    out[k] = single_solid_angle(b, r_vals[ir[k]], t_vals[it[k]], ouni_cl, &g, hits_per_single);
  }
}

/* full grid (xmi_solid_angle_calculation_f, src/xmi_solid_angle_f.F90:303-429)
 * for the points [p0, p1) of the flattened [theta][r] grid */
void oracle_solid_angle_points(const xmi_bundle *b, const double *r_vals, int nr, const double *t_vals,
                               int64_t p0, int64_t p1, long hits_per_single, double *out) {
  int64_t p;
#pragma omp parallel for schedule(dynamic, 1)
  for (p = p0; p < p1; p++) {
    orng g;
    int it = (int)(p / nr), ir = (int)(p % nr);
    orng_init(&g, b->seed, (uint64_t)p, 0xF0000000u);
    out[p - p0] = oracle_single_solid_angle(b, r_vals[ir], t_vals[it], &g, hits_per_single);
  }
}

/* xmi_get_solid_angle, src/xmi_solid_angle_f.F90:712-801 */
static double get_solid_angle(const xmi_bundle *b, const double *coords, ophoton *ph, int *err) {
  double r = dist3(b->p_det, coords), dirv[3], tt, theta;
  int p1, p2;
  dirv[0] = coords[0] - b->p_det[0];
  dirv[1] = coords[1] - b->p_det[1];
  dirv[2] = coords[2] - b->p_det[2];
  normalize3(dirv);
  tt = acos(dot3(dirv, b->n_det));
  if (tt > M_PI / 2.0) tt = M_PI - tt;
  theta = (M_PI / 2.0) - tt;
  if (theta < b->sa_t[0]) return 0.0;
  p1 = findpos(b->sa_r, b->sa_nr, r);
  p2 = findpos(b->sa_t, b->sa_nt, theta);
  if (p1 == -1 || p2 == -1) {
    orng g;
    orng_init(&g, b->seed, (uint64_t)ph->id, 0x80000000u | (uint32_t)ph->n_int);
    ph->sa_not_found++;
    return oracle_single_solid_angle(b, r, theta, &g, b->sa_hits_per_single);
  }
  return bilinear(b->sa_grid, b->sa_r, b->sa_nr, b->sa_t, b->sa_nt, r, theta, err);
}

/* ------------------------------------------------------------------ */
/* tallies                                                              */
/* ------------------------------------------------------------------ */
static void tally_channel(const xmi_bundle *b, otally *t, int n, double E, double w) {
  int ch, k;
  if (E >= O_ENERGY_THRESHOLD) ch = (int)((E - b->zero) / b->gain);
  else ch = -1;
  if (ch >= 0 && ch <= b->nchannels - 1)
    for (k = n; k <= b->n_interactions; k++) t->channels[(size_t)k * b->nchannels + ch] += w;
}
/* thread tallies hold the history rows of the run's elements only: row of
 * atomic number Z (set per run by oracle_xmi_main_msim; all rows = Z - 1
 * outside a run) */
static int o_zrow[101];
static int o_zrow_set = 0;

static size_t hidx(const xmi_bundle *b, int Z, int line, int n) {
  const int row = o_zrow_set ? o_zrow[Z] : Z - 1;
  return ((size_t)row * 385 + (line - 1)) * b->n_interactions + (n - 1);
}

/* ------------------------------------------------------------------ */
/* photon helpers                                                       */
/* ------------------------------------------------------------------ */
/* xmi_update_photon_dirv, src/xmi_main.F90:5071-5148 */
static void update_dirv(ophoton *p, double theta_i, double phi_i) {
  double phn, cphi = cos(p->phi), sphi = sin(p->phi), cth = cos(p->theta), sth = sin(p->theta);
  double m[9], d[3], ts;
  if (phi_i > 2.0 * M_PI) phn = phi_i - 2.0 * M_PI;
  else if (phi_i < 0.0 * M_PI) phn = phi_i + 2.0 * M_PI;
  else phn = phi_i;
  m[0] = cth * cphi; m[1] = -sphi; m[2] = sth * cphi;
  m[3] = cth * sphi; m[4] = cphi;  m[5] = sth * sphi;
  m[6] = -sth;       m[7] = 0.0;   m[8] = cth;
  ts = sin(theta_i);
  d[0] = ts * cos(phn);
  d[1] = ts * sin(phn);
  d[2] = cos(theta_i);
  matvec(m, d, p->dirv);
  normalize3(p->dirv);
  p->theta = acos(p->dirv[2]);
  p->phi = atan2(p->dirv[1], p->dirv[0]);
  if (p->phi > 2.0 * M_PI) p->phi = p->phi - 2.0 * M_PI;
  else if (p->phi < 0.0 * M_PI) p->phi = p->phi + 2.0 * M_PI;
}

/* xmi_update_photon_elecv, src/xmi_main.F90:5150-5182 */
static void update_elecv(ophoton *p) {
  double cosalfa = dot3(p->dirv, p->elecv);
  double c_alfa = acos(cosalfa), sinalfa = sin(c_alfa);
  double c_ae = 1.0 / sinalfa, c_be = -c_ae * cosalfa;
  int k;
  for (k = 0; k < 3; k++) p->elecv[k] = c_ae * p->elecv[k] + c_be * p->dirv[k];
  normalize3(p->elecv);
}

/* phi0 of the polarisation frame, src/xmi_main.F90:2070-2079 */
static double polarisation_phi0(const ophoton *p) {
  double cphi = cos(p->phi), sphi = sin(p->phi), cth = cos(p->theta), sth = sin(p->theta);
  double a[3] = {cphi * cth, cth * sphi, -sth}, bvec[3] = {sphi, -cphi, 0.0};
  double cosphi0 = dot3(p->elecv, a), sinphi0 = dot3(p->elecv, bvec), phi0;
  if (fabs(cosphi0) > 1.0) cosphi0 = cosphi0 > 0.0 ? 1.0 : -1.0;
  phi0 = acos(cosphi0);
  if (sinphi0 > 0.0) phi0 = -phi0;
  return phi0;
}

/* Doppler-broadened Compton energy: compton2 (transport, src/xmi_main.F90:4985-5067)
 * and compton_var_red (VR, src/xmi_variance_reduction.F90:1010-1101) */
static double compton_energy(const xmi_bundle *b, int e, double E, double theta_i, orng *g,
                             int varred, int *err) {
  const double c = (double)1.2399e-6f, c0 = (double)4.85e-12f, c1 = (double)1.456e-2f;
  const double *rn = b->doppler_rs, *icdf = b->doppler_icdf[e];
  double energy = E * 1000.0, c_lamb0 = c / energy, sth2 = sin(theta_i / 2.0);
  int it = 0, tries = 0;
  for (;;) {
    double r = orng_uniform(g), pz, dlamb, c_lamb;
    int pos = (int)(r / (rn[1] - rn[0]));
    if (++tries > 100000) { *err = 2; return 0.0; }
    if (varred && pos == XMI_DOPPLER_N - 2) continue;
    if (pos > XMI_DOPPLER_N - 2) pos = XMI_DOPPLER_N - 2;
    o_words += 2;
    pz = interp_simple(rn[pos], icdf[pos], rn[pos + 1], icdf[pos + 1], r);
    if (orng_uniform(g) < 0.5) pz = -pz;
    dlamb = c0 * sth2 * sth2 - c1 * c_lamb0 * sth2 * pz;
    c_lamb = c_lamb0 + dlamb;
    energy = c / c_lamb / 1000.0;
    /* the reference accepts when energy <= E; dlamb >= 0 is the same test in
     * exact arithmetic and cannot be defeated by rounding when dlamb is tiny */
    if (dlamb >= 0.0) break;
    if (varred) {
      if (it == 100) { *err = 3; return 0.0; }
      it++;
    }
  }
  return energy;
}

/* ---- advanced Compton: per-shell impulse approximation ----
 * MEC2 of these functions is xraylib's constant (keV); the tolerances
 * 1E-8, 1E-4 and 1E-10 of the reference are default-real literals. */
#define O_XRL_MEC2 510.998928

/* xmi_get_qimax, src/xmi_aux_f.F90:1951-1977 (ctheta = cos theta) */
static double o_qimax(double energy, double Ii, double ctheta) {
  double emi, q;
  if (Ii != 0.0 && energy < Ii) return 0.0;
  emi = energy - Ii;
  q = 137.0 * (emi * energy * (1.0 - ctheta) / O_XRL_MEC2 - Ii);
  return q / sqrt(emi * emi + energy * energy - 2.0 * emi * energy * ctheta);
}

/* xmi_get_q_from_energy, src/xmi_aux_f.F90:2058-2074 */
static double o_q_from_energy(double old_e, double new_e, double c) {
  double q = 137.0 * (new_e - old_e + (1.0 - c) * old_e * new_e / O_XRL_MEC2);
  return q / sqrt(new_e * new_e + old_e * old_e - 2.0 * old_e * new_e * c);
}

/* xmi_get_energy_from_q, src/xmi_aux_f.F90:1979-2056; *err = 1 where the
 * reference stops the program (neither root has the sign of Q) */
static double o_energy_from_q(double a, double Q, double theta, int *err) {
  const double b = O_XRL_MEC2, c = cos(theta), k2 = 137.0 * 137.0;
  double d, aq, bq, cq, e1, e2, q1, q2, delta;
  if (fabs(c - 1.0) < (double)1e-8f) return 0.0;
  if (fabs(Q) < (double)1e-4f) return a / (1.0 + a * (1.0 - c) / b);
  d = 1.0 + a / b - a * c / b;
  aq = k2 * (d * d) - Q * Q;
  bq = -(2.0 * k2 * a * d) + 2.0 * a * c * (Q * Q);
  cq = k2 * (a * a) - (a * a) * (Q * Q);
  /* xmi_poly_solve_quadratic, src/xmi_aux_f.F90:1872-1905 */
  if (aq == 0.0) {
    if (bq == 0.0) return 0.0;
    e1 = e2 = -1.0 * cq / bq;
  } else {
    delta = bq * bq - 4.0 * aq * cq;
    if (delta < 0.0) return 0.0;
    if (delta == 0.0) {
      e1 = e2 = -bq / 2.0 / aq;
    } else {
      const double sd = sqrt(delta), r1 = (-bq + sd) / 2.0 / aq, r2 = (-bq - sd) / 2.0 / aq;
      e1 = r1 < r2 ? r1 : r2;
      e2 = r1 < r2 ? r2 : r1;
    }
  }
  q1 = o_q_from_energy(a, e1, c);
  q2 = o_q_from_energy(a, e2, c);
  if (Q * q1 > 0.0) return e1;
  if (Q * q2 > 0.0) return e2;
  if (fabs(e1 - e2) < (double)1e-10f || fabs(q1 - q2) < (double)1e-10f) return e1;
  *err = 1;
  return 0.0;
}

/* the cumulative profile of one shell up to qimax (the cdfs of
 * src/xmi_main.F90:4808-4856): row = the shell's cdf table */
static double o_shell_cdf(const double *row, double qimax) {
  const double dq = 100.0 * 1.0 / (XMI_CP_N - 1.0) - 100.0 * 0.0 / (XMI_CP_N - 1.0);
  double x, v;
  int pos;
  if (qimax != qimax) qimax = 0.0; /* 0/0 at theta = 0 with a zero binding energy: undefined in the reference */
  if (qimax < -100.0) return 0.0;
  if (qimax > 100.0) return 1.0;
  x = qimax < 0.0 ? -qimax : qimax;
  pos = (int)(x / dq);
  if (pos > XMI_CP_N - 2) pos = XMI_CP_N - 2; /* x = 100 exactly: the last interval */
  o_words += 2;
  v = interp_simple(100.0 * pos / (XMI_CP_N - 1.0), row[pos], 100.0 * (pos + 1) / (XMI_CP_N - 1.0), row[pos + 1], x);
  return qimax < 0.0 ? 1.0 - (0.5 + v) : 0.5 + v;
}

/* Q of a shell at cumulative value cdf (src/xmi_main.F90:4897-4958) */
static double o_shell_q(const double *row, double cdf) {
  const double dc = 0.5 * 1.0 / (XMI_CP_N - 1.0) - 0.5 * 0.0 / (XMI_CP_N - 1.0);
  const int neg = cdf < 0.5;
  const double cp = neg ? 0.5 - cdf : cdf - 0.5;
  double q;
  int pos = (int)(cp / dc);
  /* the reference stops the program at pos = N - 1 (cdf exactly 0 or 1) */
  if (pos > XMI_CP_N - 2) pos = XMI_CP_N - 2;
  o_words += 2;
  q = interp_simple(0.5 * pos / (XMI_CP_N - 1.0), row[pos], 0.5 * (pos + 1) / (XMI_CP_N - 1.0), row[pos + 1], cp);
  return neg ? -q : q;
}

/* cdfs of every shell of element e and their occupancy-weighted sum */
static double o_shell_cdfs(const xmi_bundle *b, int e, double energy, double theta, double *cdfs) {
  const int ns = b->cp_nshell[e];
  const double c = cos(theta);
  double sum = 0.0;
  int k;
  for (k = 0; k < ns; k++) {
    const double qi = o_qimax(energy, b->cp_edge[(size_t)e * XMI_CP_SH + k], c);
    cdfs[k] = o_shell_cdf(b->cp_cdf[e] + (size_t)k * XMI_CP_N, qi);
  }
  for (k = 0; k < ns; k++) sum = sum + b->cp_occ[(size_t)e * XMI_CP_SH + k] * cdfs[k];
  return sum;
}

/* xmi_update_photon_energy_compton, src/xmi_main.F90:4785-4983: the new
 * energy (0: photon absorbed) */
static double compton_energy_advanced(const xmi_bundle *b, int e, double energy, double theta_i, orng *g, int *err) {
  const int ns = b->cp_nshell[e];
  double cdfs[XMI_CP_SH], sum, r, tsum = 0.0, q;
  int k, sel = -1;
  sum = o_shell_cdfs(b, e, energy, theta_i, cdfs);
  if (sum == 0.0) return 0.0;
  r = orng_uniform(g);
  for (k = 0; k < ns; k++) {
    const double w = b->cp_occ[(size_t)e * XMI_CP_SH + k] * cdfs[k] / sum;
    if (w > 0.0) sel = k; /* rounding can leave the running sum below r: the last shell with weight */
    tsum = tsum + w;
    if (r <= tsum) { sel = k; break; }
  }
  if (sel < 0) { *err = 1; return 0.0; } /* not reached with finite tables */
  r = orng_uniform(g);
  q = o_shell_q(b->cp_qinv[e] + (size_t)sel * XMI_CP_N, r * cdfs[sel]);
  return o_energy_from_q(energy, q, theta_i, err);
}

/* xmi_check_detector_intersection, src/xmi_aux_f.F90:1622-1834, including
 * the reference's assignment of the scalar segment length to all three
 * direction components in the collimator-free branch */
static int check_detector_intersection(const xmi_bundle *b, const double *bc, const double *ec) {
  double bd[3], ed[3], t0[3], t1[3], ip[3];
  static const double origin[3] = {0.0, 0.0, 0.0}, nx[3] = {1.0, 0.0, 0.0};
  int k;
  for (k = 0; k < 3; k++) { t0[k] = bc[k] - b->p_det[k]; t1[k] = ec[k] - b->p_det[k]; }
  matvec(b->det_inv, t0, bd);
  matvec(b->det_inv, t1, ed);
  if (!b->coll_present) {
    double s, dirv[3];
    if (bd[0] * ed[0] > 0) return O_NO_INTERSECTION;
    for (k = 0; k < 3; k++) t0[k] = ed[k] - bd[k];
    s = norm3(t0);
    dirv[0] = dirv[1] = dirv[2] = s;
    if (!intersect_plane(origin, nx, ed, dirv, ip)) return O_DETECTOR_BAD_INTERSECTION;
    ip[0] = 0.0;
    if (norm3(ip) <= b->det_radius) {
      if (dot3(dirv, nx) >= 0.0) return O_DETECTOR_BAD_INTERSECTION;
      return O_DETECTOR_INTERSECTION;
    }
    return O_NO_INTERSECTION;
  } else {
    double dirv[3], delta[3], X1[3], X2[3], c0, c1, c2, cos2t, disc, tb, te, tt1, tt2;
    double vx = b->coll_vertex_x;
    int nvalid = 0;
    for (k = 0; k < 3; k++) dirv[k] = ed[k] - bd[k];
    tb = (bd[0] - ed[0]) / dirv[0];
    te = (ed[0] - ed[0]) / dirv[0];
    delta[0] = ed[0] - vx; delta[1] = ed[1]; delta[2] = ed[2];
    cos2t = cos(b->coll_half_apex) * cos(b->coll_half_apex);
    /* M = diag(1-cos2t, -cos2t, -cos2t) */
    c2 = dirv[0] * (1.0 - cos2t) * dirv[0] - dirv[1] * cos2t * dirv[1] - dirv[2] * cos2t * dirv[2];
    c1 = dirv[0] * (1.0 - cos2t) * delta[0] - dirv[1] * cos2t * delta[1] - dirv[2] * cos2t * delta[2];
    c0 = delta[0] * (1.0 - cos2t) * delta[0] - delta[1] * cos2t * delta[1] - delta[2] * cos2t * delta[2];
    disc = c1 * c1 - c0 * c2;
    if (disc < 0.0) return O_NO_INTERSECTION;
    tt1 = (-c1 + sqrt(disc)) / c2;
    for (k = 0; k < 3; k++) X1[k] = ed[k] + tt1 * dirv[k];
    if (-(X1[0] - vx) >= 0.0) nvalid = 1;
    tt2 = (-c1 - sqrt(disc)) / c2;
    for (k = 0; k < 3; k++) X2[k] = ed[k] + tt2 * dirv[k];
    if (-(X2[0] - vx) >= 0.0) nvalid = (nvalid == 1) ? 3 : 2;
    if (nvalid == 0) return O_NO_INTERSECTION;
    if (nvalid == 1 || nvalid == 2) {
      double tsel = nvalid == 1 ? tt1 : tt2, *Xs = nvalid == 1 ? X1 : X2;
      double tmax = tb > te ? tb : te, tmin = tb < te ? tb : te;
      if (tsel <= tmax && tsel >= tmin && Xs[0] <= b->coll_height) return O_COLLIMATOR_INTERSECTION;
      if (!intersect_plane(origin, nx, ed, dirv, ip)) return O_DETECTOR_BAD_INTERSECTION;
      ip[0] = 0.0;
      if (norm3(ip) <= b->det_radius && dist3(bd, ip) <= dist3(bd, ed)) {
        if (dot3(dirv, nx) >= 0.0) return O_DETECTOR_BAD_INTERSECTION;
        return O_DETECTOR_INTERSECTION;
      }
      return O_NO_INTERSECTION;
    } else {
      double tmax = tb > te ? tb : te, tmin = tb < te ? tb : te;
      if (tt1 <= tmax && tt1 >= tmin && X1[0] <= b->coll_height) return O_COLLIMATOR_INTERSECTION;
      if (tt2 <= tmax && tt2 >= tmin && X2[0] <= b->coll_height) return O_COLLIMATOR_INTERSECTION;
      return O_NO_INTERSECTION;
    }
  }
}

/* xmi_check_photon_detector_hit, src/xmi_main.F90:1920-1984 */
static int check_photon_detector_hit(const xmi_bundle *b, const ophoton *p) {
  double dd[3], cd[3], t[3], ip[3];
  static const double origin[3] = {0.0, 0.0, 0.0}, nx[3] = {1.0, 0.0, 0.0};
  int k;
  if (dot3(p->dirv, b->n_det) >= 0.0) return 0;
  matvec(b->det_inv, p->dirv, dd);
  for (k = 0; k < 3; k++) t[k] = p->coords[k] - b->p_det[k];
  matvec(b->det_inv, t, cd);
  if (!intersect_plane(origin, nx, cd, dd, ip)) return 0;
  if (norm3(ip) > b->det_radius) return 0;
  if (!b->coll_present) return 1;
  {
    double cp[3] = {b->coll_height, 0.0, 0.0};
    if (!intersect_plane(cp, nx, cd, dd, ip)) return 0;
  }
  ip[0] = 0.0;
  if (norm3(ip) > b->coll_radius) return 0;
  return 1;
}

/* ------------------------------------------------------------------ */
/* variance reduction, src/xmi_variance_reduction.F90:29-726            */
/* ------------------------------------------------------------------ */
/* The estimator's draws come from streams of their own (engine convention):
 * (photon, 0x40000000 | n << 8 | 0xFF) for the point on the detector and
 * (photon, 0x40000000 | n << 8 | i) for the Compton energy of the i-th element
 * of the layer; the reference draws them from the photon's single stream. */
static uint32_t vr_stream(int n, int sub) { return 0x40000000u | ((uint32_t)n << 8) | (uint32_t)sub; }

static void variance_reduction(const xmi_bundle *b, ophoton *p, otally *t) {
  orng gp, *g = &gp;
  double radius, theta, dp[3], lcp[3], dirv[3], lcd[3], tmp[3], total_distance, ndc[3];
  double dotprod, phi, proj[3], en[3], distances[XMI_MAXL], tc[3], murhod, pesc_rayl, omega, pdir_fluo;
  int step_max, step_dir, i, k, kk, n = p->n_int, layer = p->cur_layer, err = 0, node;
  double f;
  if (p->energy <= O_ENERGY_THRESHOLD) return;
  orng_init(g, b->seed, (uint64_t)p->id, vr_stream(n, 0xFF));
  radius = sqrt(orng_uniform(g)) * b->det_radius;
  theta = 2.0 * M_PI * orng_uniform(g);
  dp[0] = 0.0;
  dp[1] = cos(theta) * radius;
  dp[2] = sin(theta) * radius;
  for (k = 0; k < 3; k++) tmp[k] = p->coords[k] - b->p_det[k];
  matvec(b->det_inv, tmp, lcp);
  matvec(b->det_inv, p->dirv, dirv);
  for (k = 0; k < 3; k++) lcd[k] = dp[k] - lcp[k];
  if (lcd[0] >= 0.0) return;
  total_distance = dist3(dp, lcp);
  normalize3(dirv);
  normalize3(lcd);
  matvec(b->det_new, lcd, ndc);
  dotprod = dot3(dirv, lcd);
  if (dotprod > 1.0) dotprod = 1.0;
  else if (dotprod < -1.0) dotprod = -1.0;
  theta = acos(dotprod);
  {
    double d = dot3(ndc, p->dirv), ne;
    for (k = 0; k < 3; k++) proj[k] = ndc[k] - d * p->dirv[k];
    normalize3(proj);
    ne = norm3(p->elecv);
    for (k = 0; k < 3; k++) en[k] = p->elecv[k] / ne;
  }
  dotprod = dot3(proj, en);
  if (dotprod > 1.0) dotprod = 1.0;
  else if (dotprod < -1.0) dotprod = -1.0;
  phi = acos(dotprod);
  if (dot3(ndc, b->n_sample) > 0.0) {
    step_max = b->n_layers - 1;
    step_dir = 1;
  } else {
    step_max = 0;
    step_dir = -1;
  }
  for (i = 0; i < XMI_MAXL; i++) distances[i] = 0.0;
  memcpy(tc, p->coords, sizeof(tc));
  for (i = layer;; i += step_dir) {
    double pp[3] = {0.0, 0.0, step_dir == 1 ? b->layer_zend[i] : b->layer_zbeg[i]}, ip[3];
    if (!intersect_plane(pp, b->n_sample, tc, ndc, ip)) { t->error = 4; return; }
    distances[i] = dist3(tc, ip);
    if (distances[i] > total_distance) {
      distances[i] = total_distance;
      break;
    }
    memcpy(tc, ip, sizeof(tc));
    total_distance = total_distance - distances[i];
    if (i == step_max) break;
  }
  murhod = 0.0;
  for (i = layer;; i += step_dir) {
    murhod = murhod + p->mus[i] * b->layer_rho[i] * distances[i];
    if (i == step_max) break;
  }
  pesc_rayl = exp(-murhod);
  omega = get_solid_angle(b, p->coords, p, &err);
  if (err) { t->error = 5; return; }
  pdir_fluo = omega / 4.0 / M_PI;

  xmi_grid_locate(b, p->energy, &node, &f);
  const long long words_before = o_words;
  for (i = 0; i < b->layer_nel[layer]; i++) {
    int pair = b->layer_off[layer] + i, e = b->layer_el[pair], Z = b->elem_Z[e], s, sl;
    double w = b->layer_w[pair], pconv, pdir, tw, P[9], mus_c[XMI_MAXL], ec, pesc;
    /* Rayleigh */
    pconv = w / p->mus[layer];
    pdir = omega * dcsp_rayl(b, e, p->energy, theta, phi);
    tw = pconv * pdir * pesc_rayl * p->weight;
    t->var_red[hidx(b, Z, 384, n)] += tw;
    tally_channel(b, t, n, p->energy, tw);
    /* Compton */
    orng_init(g, b->seed, (uint64_t)p->id, vr_stream(n, i));
    if (b->use_advanced_compton) {
      /* xmi_compton_varred, src/xmi_variance_reduction.F90:752-947: one
       * energy per shell, weighted by the shell's share */
      double cdfs[XMI_CP_SH];
      const double sum = o_shell_cdfs(b, e, p->energy, theta, cdfs);
      int k;
      pdir = omega * dcsp_compt(b, e, p->energy, theta, phi);
      for (k = 0; sum != 0.0 && k < b->cp_nshell[e]; k++) {
        const double sw = b->cp_occ[(size_t)e * XMI_CP_SH + k] * cdfs[k] / sum;
        double q;
        if (sw == 0.0) continue;
        q = o_shell_q(b->cp_qinv[e] + (size_t)k * XMI_CP_N, orng_uniform(g) * cdfs[k]);
        ec = o_energy_from_q(p->energy, q, theta, &err);
        if (err) { t->error = 6; return; }
        if (ec == 0.0) continue;
        mu_calc(b, ec, mus_c);
        murhod = 0.0;
        for (kk = layer;; kk += step_dir) {
          murhod = murhod + mus_c[kk] * b->layer_rho[kk] * distances[kk];
          if (kk == step_max) break;
        }
        pesc = exp(-murhod);
        tw = pconv * pdir * pesc * p->weight * sw;
        t->var_red[hidx(b, Z, 385, n)] += tw;
        tally_channel(b, t, n, ec, tw);
      }
      goto fluorescence;
    }
    ec = compton_energy(b, e, p->energy, theta, g, 1, &err);
    if (err) { t->error = 6; return; }
    mu_calc(b, ec, mus_c);
    murhod = 0.0;
    for (k = layer;; k += step_dir) {
      murhod = murhod + mus_c[k] * b->layer_rho[k] * distances[k];
      if (k == step_max) break;
    }
    pesc = exp(-murhod);
    pdir = omega * dcsp_compt(b, e, p->energy, theta, phi);
    tw = pconv * pdir * pesc * p->weight / 1.0;
    t->var_red[hidx(b, Z, 385, n)] += tw;
    tally_channel(b, t, n, ec, tw);
  fluorescence:
    /* fluorescence */
    if (n > 1 && p->hist_type[n - 1] < 0) {
      for (s = 0; s < 9; s++) P[s] = b->precalc_xrf[((size_t)e * 9 + s) * b->n_lines + p->hist_slot[n - 1]];
      o_words += 9;
      if (!b->use_M_lines)
        for (s = 4; s < 9; s++) P[s] = 0.0;
    } else {
      for (s = 0; s < 9; s++) P[s] = el_val(b, e, XMI_REC_XRF + s, node, f);
      if (!b->use_M_lines)
        for (s = 4; s < 9; s++) P[s] = 0.0;
    }
    for (sl = b->elem_line_off[e]; sl < b->elem_line_off[e + 1]; sl++) {
      int line = b->line_index[sl], sh = b->line_shell[sl];
      double efl = b->line_energy[sl];
      if (line > b->line_last) continue;
      if (efl < O_ENERGY_THRESHOLD) continue;
      /* the reference skips L1L2, L1L3 and L2L3 in this loop */
      if (line == 30 || line == 31 || line == 59) continue;
      if (P[sh] == 0.0) continue;
      pconv = w * P[sh] * b->elem_fluor_yield[9 * e + sh] * b->line_rate[sl] / p->mus[layer];
      o_words += 4 + b->n_layers; /* line record + per-layer mu at the line energy */
      murhod = 0.0;
      for (k = layer;; k += step_dir) {
        murhod = murhod + b->precalc_mu[(size_t)k * b->n_lines + sl] * b->layer_rho[k] * distances[k];
        if (k == step_max) break;
      }
      pesc = exp(-murhod);
      tw = pconv * pdir_fluo * pesc * p->weight;
      if (tw == 0.0) continue;
      t->var_red[hidx(b, Z, line, n)] += tw;
      tally_channel(b, t, n, efl, tw);
    }
  }
  o_words_est += o_words - words_before;
}

/* ------------------------------------------------------------------ */
/* interactions                                                         */
/* ------------------------------------------------------------------ */
static int rayleigh(const xmi_bundle *b, ophoton *p, orng *g) {
  int e = p->cur_elem, err = 0;
  double theta_i, tt, phi_i, phi0, r;
  r = orng_uniform(g);
  theta_i = bilinear(b->rayl_icdf[e], b->icdf_rs, XMI_ICDF_NR,
                     b->icdf_energies, XMI_ICDF_NE, r, p->energy, &err);
  if (err) return 0;
  tt = sin(theta_i) * sin(theta_i);
  tt = tt / (4.0 - 2.0 * tt);
  r = orng_uniform(g);
  phi_i = bilinear(b->phi_icdf, b->icdf_rs, XMI_ICDF_NR, b->phi_thetas, XMI_PHI_NT, r, tt, &err);
  if (err) return 0;
  phi0 = polarisation_phi0(p);
  update_dirv(p, theta_i, phi0 + phi_i);
  update_elecv(p);
  p->hist_type[p->n_int] = XMI_RAYLEIGH;
  p->hist_elem[p->n_int] = e;
  return 1;
}

static int compton(const xmi_bundle *b, ophoton *p, orng *g) {
  int e = p->cur_elem, err = 0;
  double theta_i, k0k, tt, phi_i, phi0, r, pp, rat, rk, w_h;
  r = orng_uniform(g);
  theta_i = bilinear(b->compt_icdf[e], b->icdf_rs, XMI_ICDF_NR,
                     b->icdf_energies, XMI_ICDF_NE, r, p->energy, &err);
  if (err) return 0;
  k0k = 1.0 + p->energy * (1.0 - cos(theta_i)) / O_MEC2;
  tt = sin(theta_i) * sin(theta_i);
  tt = tt / (k0k + (1.0 / k0k) - tt) / 2.0;
  r = orng_uniform(g);
  phi_i = bilinear(b->phi_icdf, b->icdf_rs, XMI_ICDF_NR, b->phi_thetas, XMI_PHI_NT, r, tt, &err);
  if (err) return 0;
  phi0 = polarisation_phi0(p);
  if (b->use_advanced_compton) {
    p->energy = compton_energy_advanced(b, e, p->energy, theta_i, g, &err);
    if (err) return 0;
    if (p->energy == 0.0) return 1;
    mu_calc(b, p->energy, p->mus);
  } else {
    p->energy = compton_energy(b, e, p->energy, theta_i, g, 0, &err);
    if (err) return 0;
    mu_calc(b, p->energy, p->mus);
    if (p->energy == 0.0) return 1;
  }
  update_dirv(p, theta_i, phi_i + phi0);
  update_elecv(p);
  pp = 2.0 * ((cos(theta_i) * cos(phi_i)) * (cos(theta_i) * cos(phi_i)) + sin(phi_i) * sin(phi_i));
  rat = 1.0 / (1.0 + (1 - cos(theta_i)) * p->energy / (double)510.998910f);
  rk = rat - 2.0 + 1.0 / rat;
  pp = pp / (rk + pp);
  r = orng_uniform(g);
  w_h = (1.0 + pp) / 2.0;
  if (r > w_h) {
    double c[3];
    cross3(p->dirv, p->elecv, c);
    memcpy(p->elecv, c, sizeof(c));
  }
  p->hist_type[p->n_int] = XMI_COMPTON;
  p->hist_elem[p->n_int] = e;
  return 1;
}

/* xmi_coster_kronig_check, src/xmi_main.F90:5184-5323 */
static int coster_kronig(const double *ck, int shell, orng *g) {
  for (;;) {
    double r, sumz;
    if (shell == 2) {
      r = orng_uniform(g);
      if (r < ck[XMI_FL23]) shell = 3;
      return shell;
    } else if (shell == 1) {
      r = orng_uniform(g);
      sumz = ck[XMI_FL12];
      if (r < sumz) { shell = 2; continue; }
      sumz += ck[XMI_FL13];
      if (r < sumz) return 3;
      return shell;
    } else if (shell == 7) {
      r = orng_uniform(g);
      if (r < ck[XMI_FM45]) shell = 8;
      return shell;
    } else if (shell == 6) {
      r = orng_uniform(g);
      sumz = ck[XMI_FM34];
      if (r < sumz) { shell = 7; continue; }
      sumz += ck[XMI_FM35];
      if (r < sumz) return 8;
      return shell;
    } else if (shell == 5) {
      r = orng_uniform(g);
      sumz = ck[XMI_FM23];
      if (r < sumz) { shell = 6; continue; }
      sumz += ck[XMI_FM24];
      if (r < sumz) { shell = 7; continue; }
      sumz += ck[XMI_FM25];
      if (r < sumz) return 8;
      return shell;
    } else if (shell == 4) {
      r = orng_uniform(g);
      sumz = ck[XMI_FM12];
      if (r < sumz) { shell = 5; continue; }
      sumz += ck[XMI_FM13];
      if (r < sumz) { shell = 6; continue; }
      sumz += ck[XMI_FM14];
      if (r < sumz) { shell = 7; continue; }
      sumz += ck[XMI_FM15];
      if (r < sumz) return 8;
      return shell;
    }
    return shell;
  }
}

/* ---- analog cascades (VR off), src/xmi_main.F90:2413-4783 ---- */

/* The photon of a vacancy in shell s (1..8 = L1..M5) of element e, set up as
 * the cascade routines set up their photons: xmi_fluorescence_yield_check
 * with the cascade-corrected yield, xmi_coster_kronig_check,
 * xmi_fluorescence_line_check, an isotropic direction and a random E-vector
 * perpendicular to it (src/xmi_main.F90:4696-4760).  Returns 1 when a line
 * above the threshold is emitted; q's other fields are left to the caller.
 * Shells beyond M5 emit nothing: they have no lines in the tables, and the
 * reference reads past its 9-shell yield table for them. */
static int o_cascade_photon(const xmi_bundle *b, int e, int s, ophoton *q, orng *g) {
  double r, sumz = 0.0, cosalfa, c_alfa, c_ae, c_be, rr;
  int sl, slot = -1, k;
  if (s < 1 || s > 8) return 0;
  if (s >= 4 && !b->use_M_lines) return 0;
  r = orng_uniform(g);
  if (r > b->elem_yield_corr[9 * e + s]) return 0;
  s = coster_kronig(b->elem_ck + (size_t)e * XMI_NCK, s, g);
  r = orng_uniform(g);
  for (sl = b->elem_shell_off[10 * e + s]; sl < b->elem_shell_off[10 * e + s + 1]; sl++) {
    sumz = sumz + b->line_rate[sl];
    if (r < sumz) {
      slot = sl;
      break;
    }
  }
  if (slot < 0 || b->line_energy[slot] <= O_ENERGY_THRESHOLD) return 0;
  q->energy = b->line_energy[slot];
  for (k = 0; k < b->n_layers; k++) q->mus[k] = b->precalc_mu[(size_t)k * b->n_lines + slot];
  q->theta = acos(2.0 * orng_uniform(g) - 1.0);
  q->phi = 2.0 * M_PI * orng_uniform(g);
  q->dirv[0] = sin(q->theta) * cos(q->phi);
  q->dirv[1] = sin(q->theta) * sin(q->phi);
  q->dirv[2] = cos(q->theta);
  rr = 2.0 * M_PI * orng_uniform(g);
  q->elecv[0] = cos(rr);
  q->elecv[1] = sin(rr);
  q->elecv[2] = 0.0;
  cosalfa = dot3(q->elecv, q->dirv);
  if (fabs(cosalfa) > 1.0) return 0; /* the reference stops the program here */
  c_alfa = acos(cosalfa);
  c_ae = 1.0 / sin(c_alfa);
  c_be = -c_ae * cosalfa;
  for (k = 0; k < 3; k++) q->elecv[k] = c_ae * q->elecv[k] + c_be * q->dirv[k];
  q->hist_type[q->n_int] = -b->line_index[slot];
  q->hist_elem[q->n_int] = e;
  q->hist_slot[q->n_int] = slot;
  q->last_interaction = XMI_PHOTOELECTRIC;
  return 1;
}

static int o_casc_auger(const xmi_bundle *b) {
  return b->use_vr == 0 && b->escape_mode == 0 &&
         (b->cascade_type == XMI_CASCADE_NONRADIATIVE || b->cascade_type == XMI_CASCADE_FULL);
}
static int o_casc_radiative(const xmi_bundle *b) {
  return b->use_vr == 0 && b->escape_mode == 0 &&
         (b->cascade_type == XMI_CASCADE_RADIATIVE || b->cascade_type == XMI_CASCADE_FULL);
}

/* the offspring of photon p: its state at the interaction, its own id */
static void o_offspring_from(const ophoton *p, ophoton *q) {
  *q = *p;
  q->id = p->id | O_OFFSPRING_ID;
  q->detector_hit = 0;
  q->inside = 0;
  q->casc_used = 1; /* offspring simulate no cascade of their own */
  q->sa_not_found = 0;
}

/* xmi_simulate_photon_cascade_auger, src/xmi_main.F90:2413-4594: a K/L
 * vacancy of p's element decayed without a photon (p's energy is already 0).
 * The transition's first vacancy turns p into its fluorescence photon, the
 * second gives the offspring. */
static void o_cascade_auger(const xmi_bundle *b, ophoton *p, int shell, ophoton *child, int *spawned, orng *g) {
  const int e = p->cur_elem, nt = shell == 0 ? XMI_AUGER_K : XMI_AUGER_L, nb = shell == 0 ? 30 : 27;
  const int f0 = shell == 0 ? 1 : 4;
  const double *rate = b->auger_rate + ((size_t)e * 4 + shell) * XMI_AUGER_K;
  double r = orng_uniform(g), sumz = 0.0;
  int t = -1, k;
  ophoton q;
  for (k = 0; k < nt; k++) {
    sumz = sumz + rate[k];
    if (r < sumz) {
      t = k;
      break;
    }
  }
  if (t < 0) return;
  o_offspring_from(p, &q);
  if (o_cascade_photon(b, e, f0 + t / nb, p, g)) p->casc_used = 1;
  if (o_cascade_photon(b, e, f0 + t % nb, &q, g)) {
    *child = q;
    *spawned = 1;
  }
}

/* child: where an analog cascade puts its offspring (NULL: none allowed) */
static int fluorescence(const xmi_bundle *b, ophoton *p, orng *g, ophoton *child, int *spawned) {
  int e = p->cur_elem, shell, found = 0, sl, slot = -1, node, k;
  double f, photo_total, sumz, r;
  xmi_grid_locate(b, p->energy, &node, &f);
  photo_total = el_val(b, e, XMI_REC_PHOTO, node, f);
  sumz = 0.0;
  r = orng_uniform(g);
  for (shell = 0; shell <= b->max_shell; shell++) {
    sumz = sumz + el_val(b, e, XMI_REC_PART + shell, node, f) / photo_total;
    if (r < sumz) {
      found = 1;
      break;
    }
  }
  if (!found) {
    p->energy = 0.0;
    return 1;
  }
  if (b->use_vr == 0 && b->escape_mode == 0) {
    /* xmi_fluorescence_yield_check; a non-radiative decay may start the
     * Auger cascade */
    r = orng_uniform(g);
    if (r > b->elem_yield_corr[9 * e + shell]) {
      p->energy = 0.0;
      if (child && !p->casc_used && o_casc_auger(b) && shell <= 3) o_cascade_auger(b, p, shell, child, spawned, g);
      return 1;
    }
  } else {
    (void)orng_uniform(g); /* unused draw of xmi_fluorescence_yield_check_varred_optim */
    if (b->escape_mode) p->weight_escape = p->weight_escape * b->elem_yield_corr[9 * e + shell];
    else p->weight = p->weight * b->elem_yield_corr[9 * e + shell];
  }
  shell = coster_kronig(b->elem_ck + (size_t)e * XMI_NCK, shell, g);
  /* xmi_fluorescence_line_check, src/xmi_main.F90:5352-5437 */
  r = orng_uniform(g);
  sumz = 0.0;
  found = 0;
  for (sl = b->elem_shell_off[10 * e + shell]; sl < b->elem_shell_off[10 * e + shell + 1]; sl++) {
    sumz = sumz + b->line_rate[sl];
    if (r < sumz) {
      found = 1;
      slot = sl;
      break;
    }
  }
  if (!found) {
    p->energy = 0.0;
    return 1;
  }
  p->energy = b->line_energy[slot];
  for (k = 0; k < b->n_layers; k++) p->mus[k] = b->precalc_mu[(size_t)k * b->n_lines + slot];
  {
    double theta_i = acos(-2.0 * orng_uniform(g) + 1.0);
    double phi_i = 2.0 * M_PI * orng_uniform(g);
    update_dirv(p, theta_i, phi_i);
  }
  update_elecv(p);
  p->hist_type[p->n_int] = -b->line_index[slot];
  p->hist_elem[p->n_int] = e;
  p->hist_slot[p->n_int] = slot;
  /* xmi_simulate_photon_cascade_radiative, src/xmi_main.F90:4596-4783 */
  if (child && !p->casc_used && o_casc_radiative(b) && b->line_casc_shell[slot] >= 0) {
    ophoton q;
    o_offspring_from(p, &q);
    if (o_cascade_photon(b, e, b->line_casc_shell[slot], &q, g)) {
      *child = q;
      *spawned = 1;
      p->casc_used = 1;
    }
  }
  return 1;
}

/* xmi_simulate_photon, src/xmi_main.F90:1188-1685 */
static int simulate_photon(const xmi_bundle *b, ophoton *p, otally *t, ophoton *child, int *spawned) {
  for (;;) {
    orng g;
    double R;
    int step_max, step_dir, i, k;
    if (p->energy < O_ENERGY_THRESHOLD) break;
    p->inside = 0;
    orng_init(&g, b->seed, (uint64_t)p->id, (uint32_t)(p->n_int + 1));
    if (dot3(p->dirv, b->n_sample) > 0.0) {
      step_max = b->n_layers - 1;
      step_dir = 1;
    } else {
      step_max = 0;
      step_dir = -1;
    }
    R = orng_uniform(&g);
    if ((b->escape_mode == 1 && p->n_int == 1) || (b->use_vr == 0 && b->escape_mode == 0)) {
      /* analog step through the layers */
      double minr = 0.0, maxr = 0.0, blbs = 1.0, ip[3], tc[3];
      for (i = p->cur_layer;; i += step_dir) {
        double pp[3] = {0.0, 0.0, step_dir == 1 ? b->layer_zend[i] : b->layer_zbeg[i]}, dist, tempexp, tp;
        if (!intersect_plane(pp, b->n_sample, p->coords, p->dirv, ip)) return 0;
        dist = dist3(p->coords, ip);
        tp = -1.0 * dist * b->layer_rho[i] * p->mus[i];
        tempexp = exp(tp);
        minr = maxr;
        maxr = maxr - blbs * expm1(tp);
        if (R <= maxr) {
          dist = -1.0 * log1p(-1.0 * (R - minr) / blbs) / p->mus[i] / b->layer_rho[i];
          memcpy(tc, p->coords, sizeof(tc));
          for (k = 0; k < 3; k++) p->coords[k] = p->coords[k] + dist * p->dirv[k];
          if (b->escape_mode != 1) {
            int rc = check_detector_intersection(b, tc, p->coords);
            if (rc == O_COLLIMATOR_INTERSECTION || rc == O_DETECTOR_BAD_INTERSECTION) return 1;
            if (rc == O_DETECTOR_INTERSECTION) {
              p->detector_hit = 1;
              return 1;
            }
          }
          p->cur_layer = i;
          p->inside = 1;
          break;
        } else {
          if (b->escape_mode != 1) {
            int rc = check_detector_intersection(b, p->coords, ip);
            if (rc == O_COLLIMATOR_INTERSECTION || rc == O_DETECTOR_BAD_INTERSECTION) return 1;
            if (rc == O_DETECTOR_INTERSECTION) {
              p->detector_hit = 1;
              return 1;
            }
          }
          memcpy(p->coords, ip, sizeof(ip));
          blbs = blbs * tempexp;
        }
        if (i == step_max) break;
      }
    } else {
      /* forced interaction */
      double distances[XMI_MAXL], lp[3], ip[3], pabs, pabs2, negln, my_sum, temp_sum;
      int my_index;
      if (p->n_int == b->n_interactions) break;
      memcpy(lp, p->coords, sizeof(lp));
      for (i = p->cur_layer;; i += step_dir) {
        double pp[3] = {0.0, 0.0, step_dir == 1 ? b->layer_zend[i] : b->layer_zbeg[i]};
        if (!intersect_plane(pp, b->n_sample, lp, p->dirv, ip)) return 0;
        distances[i] = dist3(lp, ip);
        memcpy(lp, ip, sizeof(lp));
        if (i == step_max) break;
      }
      pabs = 0.0;
      for (i = p->cur_layer;; i += step_dir) {
        pabs = pabs + p->mus[i] * b->layer_rho[i] * distances[i];
        if (i == step_max) break;
      }
      pabs2 = -1.0 * expm1(-1.0 * pabs);
      p->weight = p->weight * pabs2;
      if (b->escape_mode == 1) p->weight_escape = p->weight;
      negln = -1.0 * log1p(-1.0 * R * pabs2);
      my_index = p->cur_layer;
      my_sum = 0.0;
      for (i = p->cur_layer;; i += step_dir) {
        my_sum = my_sum + p->mus[i] * b->layer_rho[i] * distances[i];
        if (my_sum > negln) {
          my_index = i;
          break;
        }
        if (i == step_max) break;
      }
      temp_sum = 0.0;
      for (i = p->cur_layer;; i += step_dir) {
        temp_sum = temp_sum + (1.0 - (p->mus[i] * b->layer_rho[i] / (p->mus[my_index] * b->layer_rho[my_index]))) * distances[i];
        if (i == my_index) break;
      }
      temp_sum = temp_sum - 1.0 * log1p(-1.0 * R * pabs2) / (p->mus[my_index] * b->layer_rho[my_index]);
      for (k = 0; k < 3; k++) p->coords[k] = p->coords[k] + temp_sum * p->dirv[k];
      p->inside = 1;
      p->cur_layer = my_index;
    }
    if (!p->inside) {
      if (b->escape_mode != 1) p->detector_hit = check_photon_detector_hit(b, p);
      break;
    }
    if (p->n_int == b->n_interactions) break;
    p->n_int = p->n_int + 1;
    if (b->use_vr == 1) {
      variance_reduction(b, p, t);
      if (t->error) return 0;
    }
    /* atom selection, src/xmi_main.F90:1556-1572 */
    {
      int node, L = p->cur_layer, sel = -1;
      double f, thr = 0.0, r;
      r = orng_uniform(&g);
      xmi_grid_locate(b, p->energy, &node, &f);
      for (i = 0; i < b->layer_nel[L]; i++) {
        int pair = b->layer_off[L] + i;
        thr = thr + b->layer_w[pair] * el_val(b, b->layer_el[pair], XMI_REC_TOT, node, f) / p->mus[L];
        if (r < thr) {
          sel = i;
          break;
        }
      }
      if (sel < 0) sel = b->layer_nel[L] - 1;
      p->cur_elem_in_layer = sel;
      p->cur_elem = b->layer_el[b->layer_off[L] + sel];
      /* interaction type, src/xmi_main.F90:1576-1652 */
      r = orng_uniform(&g);
      {
        double pr = el_val(b, p->cur_elem, XMI_REC_PR, node, f);
        double prc = el_val(b, p->cur_elem, XMI_REC_PRC, node, f);
        int ok;
        if (r < pr) {
          p->last_interaction = XMI_RAYLEIGH;
          ok = rayleigh(b, p, &g);
        } else if (r < prc) {
          p->last_interaction = XMI_COMPTON;
          ok = compton(b, p, &g);
        } else {
          p->last_interaction = XMI_PHOTOELECTRIC;
          ok = fluorescence(b, p, &g, child, spawned);
        }
        if (!ok) return 0;
      }
    }
  }
  return 1;
}

/* ------------------------------------------------------------------ */
/* source sampling, src/xmi_main.F90:319-858                            */
/* ------------------------------------------------------------------ */
static double ran_flat(orng *g, double a, double bb) {
  double u = orng_uniform(g);
  return a * (1.0 - u) + bb * u;
}
static double ran_gauss(orng *g, double sigma) {
  double u1 = orng_uniform(g), u2 = orng_uniform(g);
  if (u1 <= 0.0) u1 = 1.0 / 9007199254740992.0;
  return sigma * sqrt(-2.0 * log(u1)) * cos(2.0 * M_PI * u2);
}
static double ran_cauchy(orng *g, double a) {
  double u;
  do {
    u = orng_uniform(g);
  } while (u == 0.5);
  return a * tan(M_PI * u);
}

/* xmi_ran_trap + xmi_poly_solve_quadratic, src/xmi_aux_f.F90:1841-1941 */
int oracle_poly_solve_quadratic(double a, double bq, double c, double *r1, double *r2) {
  double delta, sd, t1, t2;
  if (a == 0.0) {
    if (bq == 0.0) return 0;
    *r1 = -1.0 * c / bq;
    return 1;
  }
  delta = bq * bq - 4.0 * a * c;
  if (delta < 0.0) return 0;
  if (delta == 0.0) {
    *r1 = -bq / 2.0 / a;
    *r2 = *r1;
    return 2;
  }
  sd = sqrt(delta);
  t1 = (-bq + sd) / 2.0 / a;
  t2 = (-bq - sd) / 2.0 / a;
  *r1 = t1 < t2 ? t1 : t2;
  *r2 = t1 > t2 ? t1 : t2;
  return 2;
}
static int ran_trap(const double *w, orng *g, double *out) {
  double denom = w[0], m = w[1], x1 = w[2], x2 = w[3], y1 = w[4];
  double a = m / 2.0, bq = y1 - x1 * m, c = -x1 * y1 + m * x1 * x1 / 2.0 - denom * orng_uniform(g);
  double r1 = 0.0, r2 = 0.0;
  if (oracle_poly_solve_quadratic(a, bq, c, &r1, &r2) == 0) return 0;
  if (x1 <= r1 && r1 <= x2) *out = r1;
  else if (x1 <= r2 && r2 <= x2) *out = r2;
  else return 0;
  return 1;
}

/* xmi_coords_dir + xmi_coords_point/gaussian */
static void coords_dir(const xmi_bundle *b, const xmi_source_item *it, ophoton *p, orng *g) {
  double x1, y1;
  if (fabs(it->sigma_x * it->sigma_y) < (double)1.0e-20f) {
    double x1m = atan(b->slit_x / b->d_source_slit / 2.0), y1m = atan(b->slit_y / b->d_source_slit / 2.0);
    x1 = x1m * ran_flat(g, -1.0, 1.0);
    y1 = y1m * ran_flat(g, -1.0, 1.0);
    p->coords[0] = p->coords[1] = p->coords[2] = 0.0;
  } else {
    x1 = ran_gauss(g, it->sigma_xp);
    y1 = ran_gauss(g, it->sigma_yp);
    p->coords[0] = ran_gauss(g, it->sigma_x) - b->d_source_slit * sin(x1);
    p->coords[1] = ran_gauss(g, it->sigma_y) - b->d_source_slit * sin(y1);
    p->coords[2] = 0.0;
  }
  p->dirv[0] = tan(x1);
  p->dirv[1] = tan(y1);
  p->dirv[2] = 1.0;
  normalize3(p->dirv);
  p->theta = acos(p->dirv[2]);
  p->phi = atan2(p->dirv[1], p->dirv[0]);
}

/* xmi_photon_shift_first_layer, src/xmi_main.F90:1140-1186 */
static int shift_first_layer(const xmi_bundle *b, ophoton *p) {
  int i;
  double pp[3] = {0.0, 0.0, b->layer_zbeg[0]}, ip[3];
  p->cur_layer = -1;
  if (p->coords[2] >= b->layer_zbeg[0]) {
    for (i = 0; i < b->n_layers; i++)
      if (p->coords[2] < b->layer_zend[i]) {
        p->cur_layer = i;
        return 1;
      }
    return 0;
  }
  if (!intersect_plane(pp, b->n_sample, p->coords, p->dirv, ip)) return 0;
  memcpy(p->coords, ip, sizeof(ip));
  p->cur_layer = 0;
  return 1;
}

/* Simulates photons [g0, g1) of the run (global ids counted over the items)
 * and accumulates the raw tallies (before live-time scaling). */

/* tallies of a photon leaving the system, src/xmi_main.F90:441-525 */
static void tally_exit(const xmi_bundle *b, otally *t, const ophoton *p) {
  t->not_found += p->sa_not_found;
  if (p->detector_hit) {
    if (b->use_vr == 0) tally_channel(b, t, p->n_int, p->energy, p->weight);
    if (p->n_int > 0) {
      int kk = p->n_int, Z = b->elem_Z[p->hist_elem[kk]];
      int ht = p->hist_type[kk];
      if (ht <= -1 && ht >= -383) t->brute[hidx(b, Z, -ht, kk)] += p->weight;
      else if (ht == XMI_RAYLEIGH) t->brute[hidx(b, Z, 384, kk)] += p->weight;
      else if (ht == XMI_COMPTON) t->brute[hidx(b, Z, 385, kk)] += p->weight;
    }
  }
}

static int run_photon(const xmi_bundle *b, const xmi_source_item *it, int64_t j, otally *t) {
  ophoton p;
  orng g;
  double hvr = 0.0, exc_corr = 1.0, cosalfa, c_alfa, c_ae, c_be;
  int k;
  memset(&p, 0, sizeof(p));
  p.id = it->first + j;
  orng_init(&g, b->seed, (uint64_t)p.id, 0u);
  if (it->kind == 0) {
    int node;
    double f;
    if (!ran_trap(it->trap, &g, &p.energy)) return 0;
    hvr = interp_simple(it->e0, it->h0, it->e1, it->h1, p.energy) /
          interp_simple(it->e0, it->i0, it->e1, it->i1, p.energy);
    xmi_grid_locate(b, p.energy, &node, &f);
    exc_corr = exp(-1.0 * (b->exc_tab[node] + f * (b->exc_tab[node + 1] - b->exc_tab[node])));
    mu_calc(b, p.energy, p.mus);
    p.weight = it->weight * exc_corr;
    coords_dir(b, it, &p, &g);
    if (orng_uniform(&g) <= hvr) {
      p.elecv[0] = 0.0; p.elecv[1] = 1.0; p.elecv[2] = 0.0;
    } else {
      p.elecv[0] = 1.0; p.elecv[1] = 0.0; p.elecv[2] = 0.0;
    }
  } else {
    int64_t jl = it->local0 + j;
    if (it->dist_type == 1) {
      p.energy = ran_gauss(&g, it->scale) + it->e0;
      if (p.energy <= O_ENERGY_THRESHOLD || p.energy > O_ENERGY_MAX) return 1;
    } else if (it->dist_type == 2) {
      p.energy = ran_cauchy(&g, it->scale) + it->e0;
      if (p.energy <= O_ENERGY_THRESHOLD || p.energy > O_ENERGY_MAX) return 1;
    } else {
      p.energy = it->e0;
    }
    mu_calc(b, p.energy, p.mus);
    p.weight = it->weight;
    coords_dir(b, it, &p, &g);
    if ((double)(jl + 1) <= it->hor_ver_ratio) {
      p.elecv[0] = 0.0; p.elecv[1] = 1.0; p.elecv[2] = 0.0;
    } else {
      p.elecv[0] = 1.0; p.elecv[1] = 0.0; p.elecv[2] = 0.0;
    }
  }
  p.weight_escape = p.weight;
  cosalfa = dot3(p.elecv, p.dirv);
  if (fabs(cosalfa) > 1.0) return 0;
  c_alfa = acos(cosalfa);
  c_ae = 1.0 / sin(c_alfa);
  c_be = -c_ae * cosalfa;
  for (k = 0; k < 3; k++) p.elecv[k] = c_ae * p.elecv[k] + c_be * p.dirv[k];
  if (!shift_first_layer(b, &p)) return 0;
  p.last_interaction = XMI_NO_INTERACTION;
  {
    ophoton child;
    int spawned = 0, none = 0;
    if (!simulate_photon(b, &p, t, &child, &spawned)) return 0;
    tally_exit(b, t, &p);
    /* the offspring of an analog cascade, walked after its parent as the
     * reference walks photon%offspring (src/xmi_main.F90:441-555) */
    if (spawned) {
      if (!simulate_photon(b, &child, t, NULL, &none)) return 0;
      tally_exit(b, t, &child);
    }
  }
  return 1;
}

/* Entry point: runs the photons of the bundle's items in [ph0, ph1) of each
 * item's local index range (all if ph1 < 0) with nthreads OpenMP threads and
 * writes the reference outputs: channels[(N+1)*nch] (cumulative, x live
 * time), brute/var_red[100*385*N] (x live time x n_mpi_hosts).
 * Returns 1 on success. */
int oracle_xmi_main_msim(const xmi_bundle *b, int n_mpi_hosts, int nthreads, int64_t max_photons_per_item,
                         double *channels, double *brute, double *var_red, long *not_found) {
  int N = b->n_interactions, nch = b->nchannels, ok = 1;
  size_t nc = (size_t)(N + 1) * nch, nh = (size_t)100 * 385 * N, i;
  memset(channels, 0, sizeof(double) * nc);
  memset(brute, 0, sizeof(double) * nh);
  memset(var_red, 0, sizeof(double) * nh);
  *not_found = 0;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
  {
    /* one loop over every (item, photon) pair, so that an item of few photons
     * costs no barrier; the thread tallies are summed in parallel afterwards */
    int64_t *first = (int64_t *)malloc(sizeof(int64_t) * (size_t)(b->n_items + 1)), total;
    int it_i, nt = 1;
    otally *tl;
    first[0] = 0;
    for (it_i = 0; it_i < b->n_items; it_i++) {
      int64_t n = b->items[it_i].n_photons;
      if (max_photons_per_item >= 0 && n > max_photons_per_item) n = max_photons_per_item;
      first[it_i + 1] = first[it_i] + n;
    }
    total = first[b->n_items];
#ifdef _OPENMP
    nt = omp_get_max_threads();
#endif
    tl = (otally *)calloc((size_t)nt, sizeof(otally));
    /* compact history rows: the thread tallies cover the run's elements only */
    size_t nhc;
    for (it_i = 0; it_i <= 100; it_i++) o_zrow[it_i] = 0;
    for (it_i = 0; it_i < b->n_elem; it_i++) o_zrow[b->elem_Z[it_i]] = it_i;
    o_zrow_set = 1;
    nhc = (size_t)(b->n_elem > 0 ? b->n_elem : 1) * 385 * N;
#pragma omp parallel
    {
      int tid = 0;
      int64_t g;
      otally *t;
#ifdef _OPENMP
      tid = omp_get_thread_num();
#endif
      t = &tl[tid];
      t->channels = (double *)calloc(nc, sizeof(double));
      t->brute = (double *)calloc(nhc, sizeof(double));
      t->var_red = (double *)calloc(nhc, sizeof(double));
#pragma omp for schedule(dynamic, 64)
      for (g = 0; g < total; g++) {
        int lo = 0, hi = b->n_items - 1;
        while (lo < hi) { /* the item holding photon g */
          int mid = (lo + hi + 1) >> 1;
          if (first[mid] <= g) lo = mid; else hi = mid - 1;
        }
        if (!t->error && !run_photon(b, &b->items[lo], g - first[lo], t) && !t->error) t->error = 1;
      }
#pragma omp critical
      {
        o_words_total += o_words;
        o_words_est_total += o_words_est;
        o_words = 0;
        o_words_est = 0;
      }
#pragma omp barrier
#pragma omp for schedule(static)
      for (i = 0; i < nhc; i++) {
        const size_t e = i / ((size_t)385 * N);
        size_t full;
        int k;
        if ((int)e >= b->n_elem) continue;
        full = ((size_t)(b->elem_Z[e] - 1) * 385 * N) + i % ((size_t)385 * N);
        for (k = 0; k < nt; k++) {
          if (!tl[k].brute) continue;
          brute[full] += tl[k].brute[i];
          var_red[full] += tl[k].var_red[i];
        }
      }
#pragma omp for schedule(static)
      for (i = 0; i < nc; i++) {
        int k;
        for (k = 0; k < nt; k++)
          if (tl[k].channels) channels[i] += tl[k].channels[i];
      }
    }
    o_zrow_set = 0;
    for (it_i = 0; it_i < nt; it_i++) {
      *not_found += tl[it_i].not_found;
      if (tl[it_i].error) ok = 0;
      free(tl[it_i].channels);
      free(tl[it_i].brute);
      free(tl[it_i].var_red);
    }
    free(tl);
    free(first);
  }
  for (i = 0; i < nc; i++) channels[i] *= b->live_time;
  for (i = 0; i < nh; i++) {
    brute[i] *= b->live_time * n_mpi_hosts;
    var_red[i] *= b->live_time * n_mpi_hosts;
  }
  return ok;
}

/* table words read since the last call (all threads); *estimator receives
 * the part read by the estimator's element and line loops */
long long oracle_words_counted(long long *estimator) {
  long long w = o_words_total;
  if (estimator) *estimator = o_words_est_total;
  o_words_total = 0;
  o_words_est_total = 0;
  return w;
}

/* known-answer helper: raw Philox block */
/* Escape-ratio Monte Carlo, src/xmi_main.F90:5473-5800 (the photon loop
 * 5645-5755): photon w of input energy iE = w / n_photons starts at the point
 * source with a slit direction (xmi_coords_dir, 957-1010) and a random
 * E-vector, is simulated in escape mode, and, when it leaves after at least
 * one interaction, is tallied by its last interaction: a Compton photon by
 * its energy bin, a fluorescence photon (lines KL1..L3P3) by element and line
 * with its escape weight.  Raw sums: fluo[nE][n_elem][109], comp[nE][nco],
 * interacted[nE] (the ratios are these over interacted).  Same Philox
 * streams as the engine's escape kernel: (photon w, stream 0) for the source,
 * (w, k) for step k. */
int oracle_escape_ratios(const xmi_bundle *b, long nE, double emin, double de, long n_photons, long nco,
                         double cmin, double cde, int nthreads, double *fluo, double *comp, double *interacted) {
  const long long n_total = (long long)nE * n_photons;
  size_t nf = (size_t)nE * b->n_elem * 109, i;
  int ok = 1;
  memset(fluo, 0, sizeof(double) * nf);
  memset(comp, 0, sizeof(double) * (size_t)nE * nco);
  memset(interacted, 0, sizeof(double) * nE);
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel
  {
    size_t nc = (size_t)(b->n_interactions + 1) * b->nchannels, nh = (size_t)100 * 385 * b->n_interactions;
    otally t;
    memset(&t, 0, sizeof(t));
    t.channels = (double *)calloc(nc > 0 ? nc : 1, sizeof(double));
    t.var_red = (double *)calloc(nh > 0 ? nh : 1, sizeof(double));
    t.brute = (double *)calloc(nh > 0 ? nh : 1, sizeof(double));
#pragma omp for schedule(dynamic, 256)
    for (long long w = 0; w < n_total; w++) {
      ophoton p;
      orng g;
      const long iE = (long)(w / n_photons);
      double x1m, y1m, x1, y1, te, cosalfa, c_alfa, c_ae, c_be;
      int k, spawned = 0;
      memset(&p, 0, sizeof(p));
      p.id = w;
      p.energy = emin + iE * de;
      mu_calc(b, p.energy, p.mus);
      orng_init(&g, b->seed, (uint64_t)w, 0u);
      x1m = atan(b->slit_x / b->d_source_slit / 2.0);
      y1m = atan(b->slit_y / b->d_source_slit / 2.0);
      x1 = x1m * ran_flat(&g, -1.0, 1.0);
      y1 = y1m * ran_flat(&g, -1.0, 1.0);
      p.dirv[0] = tan(x1);
      p.dirv[1] = tan(y1);
      p.dirv[2] = 1.0;
      normalize3(p.dirv);
      p.theta = acos(p.dirv[2]);
      p.phi = atan2(p.dirv[1], p.dirv[0]);
      p.weight = 1.0;
      p.weight_escape = p.weight;
      te = orng_uniform(&g) * M_PI * 2.0;
      p.elecv[0] = cos(te);
      p.elecv[1] = sin(te);
      p.elecv[2] = 0.0;
      cosalfa = dot3(p.elecv, p.dirv);
      c_alfa = acos(cosalfa);
      c_ae = 1.0 / sin(c_alfa);
      c_be = -c_ae * cosalfa;
      for (k = 0; k < 3; k++) p.elecv[k] = c_ae * p.elecv[k] + c_be * p.dirv[k];
      if (!shift_first_layer(b, &p)) continue;
      p.last_interaction = XMI_NO_INTERACTION;
      if (!simulate_photon(b, &p, &t, NULL, &spawned)) continue;
      if (p.last_interaction != XMI_NO_INTERACTION) {
#pragma omp atomic
        interacted[iE] += p.weight;
      }
      if (!p.inside && p.last_interaction != XMI_NO_INTERACTION) {
        if (p.last_interaction == XMI_COMPTON) {
          const int ci = (int)((p.energy - cmin) / cde) + 1;
          if (ci >= 1 && ci <= nco) {
#pragma omp atomic
            comp[(size_t)iE * nco + (ci - 1)] += p.weight;
          }
        } else if (p.last_interaction == XMI_PHOTOELECTRIC) {
          const int ht = p.hist_type[p.n_int];
          if (ht <= -1 && ht >= -109) {
#pragma omp atomic
            fluo[((size_t)iE * b->n_elem + p.hist_elem[p.n_int]) * 109 + (-ht - 1)] += p.weight_escape;
          }
        }
      }
    }
    if (t.error) {
#pragma omp atomic write
      ok = 0;
    }
    free(t.channels);
    free(t.var_red);
    free(t.brute);
  }
  (void)i;
  return ok;
}

void oracle_philox_block(const uint32_t *ctr, const uint32_t *key, uint32_t *out) { orng_block(ctr, key, out); }

void oracle_threefry_block(const uint32_t *ctr, const uint32_t *key, uint32_t *out) { othreefry4x32(ctr, key, out); }

/* test hooks of the advanced Compton kinematics and profile tables */
double oracle_compton_qimax(double energy, double Ii, double theta) { return o_qimax(energy, Ii, cos(theta)); }
double oracle_compton_q_from_energy(double old_e, double new_e, double theta) {
  return o_q_from_energy(old_e, new_e, cos(theta));
}
double oracle_compton_energy_from_q(double a, double Q, double theta, int *err) {
  *err = 0;
  return o_energy_from_q(a, Q, theta, err);
}
/* shells of element e (shell index, occupancy, binding energy); -1 before
 * the tables exist */
int oracle_compton_shells(const xmi_bundle *b, int e, int *shell, double *occ, double *edge) {
  int k;
  if (!b->cp_nshell || e < 0 || e >= b->n_elem) return -1;
  for (k = 0; k < b->cp_nshell[e]; k++) {
    shell[k] = b->cp_shell[(size_t)e * XMI_CP_SH + k];
    occ[k] = b->cp_occ[(size_t)e * XMI_CP_SH + k];
    edge[k] = b->cp_edge[(size_t)e * XMI_CP_SH + k];
  }
  return b->cp_nshell[e];
}
void oracle_compton_rows(const xmi_bundle *b, int e, int k, double *cdf, double *qinv) {
  memcpy(cdf, b->cp_cdf[e] + (size_t)k * XMI_CP_N, sizeof(double) * XMI_CP_N);
  memcpy(qinv, b->cp_qinv[e] + (size_t)k * XMI_CP_N, sizeof(double) * XMI_CP_N);
}
/* the shell cumulative values and the sampled scattered energy of the
 * transport for element e at (energy, theta) from Philox stream (id, stream) */
double oracle_compton_energy_advanced(const xmi_bundle *b, int e, double energy, double theta, uint64_t id,
                                      uint32_t stream, double *cdfs, int *err) {
  orng g;
  *err = 0;
  o_shell_cdfs(b, e, energy, theta, cdfs);
  orng_init(&g, b->seed, id, stream);
  return compton_energy_advanced(b, e, energy, theta, &g, err);
}
