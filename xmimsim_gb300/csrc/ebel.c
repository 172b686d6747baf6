/*
 * X-ray tube excitation spectra: Ebel's model (H. Ebel, X-Ray Spectrometry 28
 * (1999) 255-266) with the reference's extension to L lines and its
 * transmission-tube form, xmi_tube_ebel (src/xmi_ebel.F90:115-521), and the
 * transmission-efficiency file reader (src/xmi_transmission_efficiency.c:26-88)
 * with its natural cubic spline (src/xmi_spline.c).  Host code: the spectrum
 * is an input of the transport, computed once.
 *
 * Atomic data come from the engine's tabulator (xrlite): total cross
 * sections, edge and line energies, radiative rates, K fluorescence yields,
 * atomic weights.  The L-shell yields of the line intensities are the
 * published table of Hubbell et al. (J. Phys. Chem. Ref. Data 23 (1994) 339,
 * Table 8, with the 2004 erratum), the table the reference uses, kept
 * value for value (including its Z = 31 entry).
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "xmi_internal.h"
#include "xrlite.h"

#define TUBE_MINIMUM_ENERGY 1.0 /* keV, src/xmi_ebel.F90:16 */

static const double omega_l[100] = {
    0.0,     0.0,     0.0,     0.0,     0.0,     0.0,     0.0,     0.0,     0.0,     0.0,
    2.17E-4, 3.04E-4, 4.15E-4, 5.53E-4, 7.24E-4, 9.30E-4, 0.00118, 0.00147, 0.00181, 0.00221,
    0.00268, 0.00321, 0.00381, 0.00450, 0.00527, 0.00614, 0.00711, 0.00819, 0.00939, 0.0107,
    0.122,   0.0138,  0.0155,  0.0174,  0.0195,  0.0218,  0.0242,  0.0263,  0.0285,  0.0309,
    0.0335,  0.0363,  0.0393,  0.0425,  0.0459,  0.0495,  0.0534,  0.0575,  0.0618,  0.0655,
    0.0714,  0.0765,  0.0820,  0.0877,  0.0938,  0.100,   0.107,   0.114,   0.121,   0.129,
    0.137,   0.145,   0.153,   0.163,   0.172,   0.182,   0.192,   0.202,   0.212,   0.223,
    0.234,   0.245,   0.257,   0.269,   0.281,   0.293,   0.305,   0.318,   0.331,   0.343,
    0.356,   0.369,   0.382,   0.395,   0.409,   0.422,   0.435,   0.448,   0.461,   0.474,
    0.486,   0.499,   0.511,   0.524,   0.536,   0.548,   0.560,   0.572,   0.583,   0.595};

/* L-line intensity correction of light anodes (src/xmi_ebel.F90:99-111) */
static double fcorr(int Z) { return Z >= 80 ? 1.0 : -0.4814 + 0.03781 * Z - 2.413E-4 * Z * Z; }

/* ---- natural cubic spline (Burden & Faires, Numerical Analysis, alg. 3.4) ---- */
typedef struct {
  int n; /* intervals */
  double *x, *a, *b, *c, *d;
} spline;

static int spline_init(spline *s, const double *x, const double *y, int npts) {
  int n = npts - 1, i;
  double *h, *alpha, *l, *mu, *z;
  if (n < 1) return 0;
  s->n = n;
  s->x = (double *)malloc(sizeof(double) * npts);
  s->a = (double *)malloc(sizeof(double) * npts);
  s->b = (double *)malloc(sizeof(double) * n);
  s->c = (double *)malloc(sizeof(double) * npts);
  s->d = (double *)malloc(sizeof(double) * n);
  h = (double *)malloc(sizeof(double) * n);
  alpha = (double *)calloc(npts, sizeof(double));
  l = (double *)malloc(sizeof(double) * npts);
  mu = (double *)malloc(sizeof(double) * npts);
  z = (double *)malloc(sizeof(double) * npts);
  memcpy(s->x, x, sizeof(double) * npts);
  memcpy(s->a, y, sizeof(double) * npts);
  for (i = 0; i < n; i++) h[i] = x[i + 1] - x[i];
  for (i = 1; i < n; i++) alpha[i] = 3.0 * (y[i + 1] - y[i]) / h[i] - 3.0 * (y[i] - y[i - 1]) / h[i - 1];
  l[0] = 1.0;
  mu[0] = z[0] = 0.0;
  for (i = 1; i < n; i++) {
    l[i] = 2.0 * (x[i + 1] - x[i - 1]) - h[i - 1] * mu[i - 1];
    mu[i] = h[i] / l[i];
    z[i] = (alpha[i] - h[i - 1] * z[i - 1]) / l[i];
  }
  l[n] = 1.0;
  z[n] = s->c[n] = 0.0;
  for (i = n - 1; i >= 0; i--) {
    s->c[i] = z[i] - mu[i] * s->c[i + 1];
    s->b[i] = (y[i + 1] - y[i]) / h[i] - h[i] * (s->c[i + 1] + 2.0 * s->c[i]) / 3.0;
    s->d[i] = (s->c[i + 1] - s->c[i]) / (3.0 * h[i]);
  }
  free(h);
  free(alpha);
  free(l);
  free(mu);
  free(z);
  return 1;
}

static double spline_eval(const spline *s, double x) {
  int i = 0;
  double dx;
  /* the interval of x, clamped to the end intervals */
  while (i < s->n - 1 && x >= s->x[i + 1]) i++;
  dx = x - s->x[i];
  return s->a[i] + s->b[i] * dx + s->c[i] * dx * dx + s->d[i] * dx * dx * dx;
}

static void spline_free(spline *s) {
  free(s->x);
  free(s->a);
  free(s->b);
  free(s->c);
  free(s->d);
}

/* exp(-rho t mu(E)) of a single-element layer (window or filter) */
static double layer_transmission(const xmi_layer *l, double E) {
  if (!l) return 1.0;
  return exp(-1.0 * l->density * l->thickness * XD->CS_Total_Kissel(l->Z[0], E));
}

int xmi_tube_ebel(xmi_layer *tube_anode, xmi_layer *tube_window, xmi_layer *tube_filter, double tube_voltage,
                  double tube_current, double tube_angle_electron, double tube_angle_xray, double tube_delta_energy,
                  double tube_solid_angle, int tube_transmission, size_t tube_nefficiencies, double *tube_energies,
                  double *tube_efficiencies, xmi_excitation **ebel_spectrum) {
  int Z, ncont, ndisc = 0, i, line;
  double sinalphae, sinalphax, sinfactor, x, m, logz, eta, p3, rhozmax;
  const double const1 = 1.35E+09, const2_K = 5.0E+13, zk = 2.0, zl = 8.0, bk = 0.35, bl = 0.25;
  xmi_energy_continuous *cont;
  xmi_energy_discrete *disc;
  int *disc_line;
  double *disc_edge;
  if (!tube_anode || !ebel_spectrum || tube_anode->n_elements < 1 || tube_voltage <= TUBE_MINIMUM_ENERGY ||
      tube_delta_energy <= 0.0) {
    xmi_set_error("xmi_tube_ebel: invalid arguments");
    return 0;
  }
  *ebel_spectrum = NULL;
  Z = tube_anode->Z[0];
  if (Z < 1 || Z > 100) {
    xmi_set_error("xmi_tube_ebel: anode element %d outside 1..100", Z);
    return 0;
  }
  if (XD->prepare) XD->prepare(Z);
  if (tube_window) if (XD->prepare) XD->prepare(tube_window->Z[0]);
  if (tube_filter) if (XD->prepare) XD->prepare(tube_filter->Z[0]);

  /* angles (src/xmi_ebel.F90:221-224) */
  sinalphae = sin(M_PI / 180.0 * tube_angle_electron);
  sinalphax = sin(M_PI / 180.0 * tube_angle_xray);
  sinfactor = sinalphae / sinalphax;

  /* Bremsstrahlung intervals: 1 keV in steps of delta, the last at the tube
   * voltage (src/xmi_ebel.F90:229-244) */
  ncont = (int)floor((tube_voltage - TUBE_MINIMUM_ENERGY) / tube_delta_energy) + 1;
  if (tube_voltage / tube_delta_energy != (double)lround(tube_voltage / tube_delta_energy)) ncont++;
  cont = (xmi_energy_continuous *)calloc(ncont, sizeof(xmi_energy_continuous));
  for (i = 0; i < ncont - 1; i++) cont[i].energy = TUBE_MINIMUM_ENERGY + i * tube_delta_energy;
  cont[ncont - 1].energy = tube_voltage;

  /* depth of the generated photons (Ebel's eta, rho z_max, rho z) */
  x = 1.109 - 0.00435 * Z + 0.00175 * tube_voltage;
  m = 0.1382 - 0.9211 / sqrt((double)Z);
  logz = log((double)Z);
  eta = (0.1904 - 0.2236 * logz + 0.1292 * logz * logz - 0.0149 * logz * logz * logz) * pow(tube_voltage, m);
  p3 = 0.787E-05 * sqrt((double)Z * 0.0135) * pow(tube_voltage, 1.5) + 0.735E-06 * tube_voltage * tube_voltage;
  rhozmax = XD->AtomicWeight(Z) * p3 / Z;
  for (i = 0; i < ncont; i++) {
    const double Em = cont[i].energy + tube_delta_energy / 2.0;
    const double u0 = tube_voltage / Em, logu0 = log(u0);
    const double p1 = logu0 * (0.49269 - 1.09870 * eta + 0.78557 * eta * eta);
    const double p2 = 0.70256 - 1.09865 * eta + 1.00460 * eta * eta + logu0;
    const double rhoz = rhozmax * (p1 / p2);
    const double tau = XD->CS_Total_Kissel(Z, Em);
    const double rhelp = tau * 2.0 * rhoz * sinfactor;
    double I = 0.0;
    if (rhelp > 0.0) {
      if (tube_transmission == 0)
        I = const1 * Z * pow(u0 - 1.0, x) * (1.0 - exp(-1.0 * rhelp)) / rhelp;
      else
        I = const1 * Z * pow(u0 - 1.0, x) *
            (exp(-tau * (tube_anode->density * tube_anode->thickness - 2.0 * rhoz) / sinalphax) -
             exp(-tau * tube_anode->density * tube_anode->thickness / sinalphax)) /
            rhelp;
    }
    cont[i].horizontal_intensity = I;
  }

  /* characteristic K and L lines above 1 keV whose shell the voltage
   * ionises (src/xmi_ebel.F90:301-347) */
  disc = (xmi_energy_discrete *)calloc(xrl_shell_last_line(3) + 1, sizeof(xmi_energy_discrete));
  disc_line = (int *)calloc(xrl_shell_last_line(3) + 1, sizeof(int));
  disc_edge = (double *)calloc(xrl_shell_last_line(3) + 1, sizeof(double));
  for (line = xrl_shell_first_line(0); line <= xrl_shell_last_line(3); line++) {
    int shell;
    double edge;
    if (!(XD->RadRate(Z, line) > 0.0 && XD->LineEnergy(Z, line) > TUBE_MINIMUM_ENERGY)) continue;
    for (shell = 0; shell < 4; shell++)
      if (line >= xrl_shell_first_line(shell) && line <= xrl_shell_last_line(shell)) break;
    edge = XD->EdgeEnergy(Z, shell);
    if (edge == 0.0 || edge > tube_voltage) continue;
    disc_line[ndisc] = line;
    disc_edge[ndisc] = edge;
    disc[ndisc].energy = XD->LineEnergy(Z, line);
    ndisc++;
  }
  for (i = 0; i < ndisc; i++) {
    const int ln = disc_line[i];
    const int is_k = ln <= xrl_shell_last_line(0);
    const double u0 = tube_voltage / disc_edge[i], logu0 = log(u0), su0 = sqrt(u0);
    double oneovers = (su0 * logu0 + 2.0 * (1.0 - su0)) / (u0 * logu0 + 1.0 - u0);
    double r, p1, p2, rhoz, tau, rhelp, I;
    oneovers = 1.0 + 16.05 * sqrt(0.0135 * Z / disc_edge[i]) * oneovers;
    oneovers = (is_k ? zk * bk : zl * bl) / Z * (u0 * logu0 + 1.0 - u0) * oneovers;
    r = 1.0 - 0.0081517 * Z + 3.613e-05 * Z * Z + 0.009583 * Z * exp(-1.0 * u0) + tube_voltage * 0.001141;
    p1 = logu0 * (0.49269 - 1.09870 * eta + 0.78557 * eta * eta);
    p2 = 0.70256 - 1.09865 * eta + 1.00460 * eta * eta + logu0;
    rhoz = rhozmax * (p1 / p2);
    tau = XD->CS_Total_Kissel(Z, disc[i].energy);
    rhelp = tau * 2.0 * rhoz * sinfactor;
    if (rhelp > 0.0) {
      if (tube_transmission == 0)
        rhelp = (1.0 - exp(-1.0 * rhelp)) / rhelp;
      else
        rhelp = (exp(-tau * (tube_anode->density * tube_anode->thickness - 2.0 * rhoz) / sinalphax) -
                 exp(-tau * tube_anode->density * tube_anode->thickness / sinalphax)) /
                rhelp;
    }
    if (is_k)
      I = rhelp * const2_K * oneovers * r * XD->RadRate(Z, ln) * XD->FluorYield(Z, 0);
    else if (ln <= xrl_shell_last_line(1))
      I = rhelp * fcorr(Z) * 0.71E13 * oneovers * r * XD->RadRate(Z, ln) * omega_l[Z - 1];
    else if (ln <= xrl_shell_last_line(2))
      I = rhelp * fcorr(Z) * 2.70E13 * oneovers * r * XD->RadRate(Z, ln) * omega_l[Z - 1];
    else
      I = rhelp * 4.94E13 * oneovers * r * XD->RadRate(Z, ln) * omega_l[Z - 1];
    disc[i].horizontal_intensity = I;
    disc[i].distribution_type = XMI_ENERGY_DISCRETE_DISTRIBUTION_MONOCHROMATIC;
    disc[i].scale_parameter = 0.0;
  }
  free(disc_line);
  free(disc_edge);

  /* window and filter (src/xmi_ebel.F90:433-460): lines at their energy,
   * intervals at their middle for the window and at their start for the
   * filter, as the reference evaluates them */
  for (i = 0; i < ndisc; i++)
    disc[i].horizontal_intensity *=
        layer_transmission(tube_window, disc[i].energy) * layer_transmission(tube_filter, disc[i].energy);
  for (i = 0; i < ncont; i++)
    cont[i].horizontal_intensity *= layer_transmission(tube_window, cont[i].energy + tube_delta_energy / 2.0) *
                                    layer_transmission(tube_filter, cont[i].energy);

  /* current and solid angle; unpolarised (src/xmi_ebel.F90:463-483) */
  for (i = 0; i < ncont; i++) {
    cont[i].horizontal_intensity *= tube_solid_angle * tube_current / 2.0;
    cont[i].vertical_intensity = cont[i].horizontal_intensity;
  }
  for (i = 0; i < ndisc; i++) {
    disc[i].horizontal_intensity *= tube_solid_angle * tube_current / 2.0;
    disc[i].vertical_intensity = disc[i].horizontal_intensity;
  }

  /* transmission efficiency profile (src/xmi_ebel.F90:486-499) */
  if (tube_nefficiencies > 0 && tube_energies && tube_efficiencies) {
    spline s;
    if (!spline_init(&s, tube_energies, tube_efficiencies, (int)tube_nefficiencies)) {
      free(cont);
      free(disc);
      xmi_set_error("xmi_tube_ebel: at least two transmission efficiencies are needed");
      return 0;
    }
    for (i = 0; i < ncont; i++) {
      cont[i].horizontal_intensity *= spline_eval(&s, cont[i].energy);
      cont[i].vertical_intensity = cont[i].horizontal_intensity;
    }
    for (i = 0; i < ndisc; i++) {
      disc[i].horizontal_intensity *= spline_eval(&s, disc[i].energy);
      disc[i].vertical_intensity = disc[i].horizontal_intensity;
    }
    spline_free(&s);
  }

  *ebel_spectrum = (xmi_excitation *)calloc(1, sizeof(xmi_excitation));
  (*ebel_spectrum)->n_continuous = ncont;
  (*ebel_spectrum)->continuous = cont;
  (*ebel_spectrum)->n_discrete = ndisc;
  if (ndisc > 0) {
    (*ebel_spectrum)->discrete = disc;
  } else {
    free(disc);
    (*ebel_spectrum)->discrete = NULL;
  }
  return 1;
}

/* two columns (keV, efficiency in [0, 1]); energies increasing, the first
 * below 1 keV; at least 10 rows; blank lines ignored
 * (src/xmi_transmission_efficiency.c:26-88) */
int xmi_transmission_efficiency_read(const char *filename, size_t *nefficiencies, double **energies,
                                     double **efficiencies) {
  FILE *f;
  char buf[512];
  size_t n = 0, cap = 64;
  double *ex, *ey;
  if (!filename || !nefficiencies || !energies || !efficiencies) {
    xmi_set_error("xmi_transmission_efficiency_read: NULL argument");
    return 0;
  }
  f = fopen(filename, "r");
  if (!f) {
    xmi_set_error("xmi_transmission_efficiency_read: cannot open %s", filename);
    return 0;
  }
  ex = (double *)malloc(sizeof(double) * cap);
  ey = (double *)malloc(sizeof(double) * cap);
  while (fgets(buf, sizeof(buf), f)) {
    double e, v;
    char *p = buf;
    while (*p == ' ' || *p == '\t' || *p == '\r' || *p == '\n') p++;
    if (*p == '\0') continue;
    if (sscanf(p, "%lg %lg", &e, &v) != 2 || e < 0.0 || v < 0.0 || v > 1.0 || (n > 0 && e <= ex[n - 1]) ||
        (n == 0 && e >= 1.0)) {
      fclose(f);
      free(ex);
      free(ey);
      xmi_set_error("Error reading %s. The transmission efficiency file should contain two columns with energies "
                    "(keV) in the left column and the transmission efficiency (value between 0 and 1) in the second "
                    "column. Empty lines are ignored. First energy must be between 0 and 1 keV. At least 10 values "
                    "are required.",
                    filename);
      return 0;
    }
    if (n == cap) {
      cap *= 2;
      ex = (double *)realloc(ex, sizeof(double) * cap);
      ey = (double *)realloc(ey, sizeof(double) * cap);
    }
    ex[n] = e;
    ey[n] = v;
    n++;
  }
  fclose(f);
  if (n < 10) {
    free(ex);
    free(ey);
    xmi_set_error("Error reading %s: at least 10 transmission efficiencies are required", filename);
    return 0;
  }
  *nefficiencies = n;
  *energies = ex;
  *efficiencies = ey;
  return 1;
}
