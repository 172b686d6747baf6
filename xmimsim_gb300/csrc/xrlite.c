/*
 * Stand-in atomic data model; see xrlite.h for what it is and is not.
 * Every number below is either a public physical constant (K-edge
 * energies, standard atomic weights) or a smooth parametrisation chosen to
 * give plausible magnitudes and the right structure (edges, jumps, line
 * families, Z trends).
 */
#include "xrlite.h"
#include "../../include/xmimsim_bundle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

static const char *line_names[386] = {
#include "xrl_line_names.inc"
};

/* K-shell binding energies, keV, Z = 1..94 */
static const double k_edge[XRL_MAXZ + 1] = {0.0,
  0.0136, 0.0246, 0.0548, 0.1115, 0.1880, 0.2842, 0.4099, 0.5431, 0.6967, 0.8701,
  1.0721, 1.3050, 1.5596, 1.8389, 2.1455, 2.4720, 2.8224, 3.2029, 3.6074, 4.0381,
  4.4928, 4.9664, 5.4651, 5.9892, 6.5390, 7.1120, 7.7089, 8.3328, 8.9789, 9.6586,
  10.3671, 11.1031, 11.8667, 12.6578, 13.4737, 14.3256, 15.1997, 16.1046, 17.0384, 17.9976,
  18.9856, 19.9995, 21.0440, 22.1172, 23.2199, 24.3503, 25.5140, 26.7112, 27.9399, 29.2001,
  30.4912, 31.8138, 33.1694, 34.5614, 35.9846, 37.4406, 38.9246, 40.4430, 41.9906, 43.5689,
  45.1840, 46.8342, 48.5190, 50.2391, 51.9957, 53.7885, 55.6177, 57.4855, 59.3896, 61.3323,
  63.3138, 65.3508, 67.4164, 69.5250, 71.6764, 73.8708, 76.1110, 78.3948, 80.7249, 83.1023,
  85.5304, 88.0045, 90.5259, 93.1050, 95.7299, 98.4040, 101.137, 103.922, 106.755, 109.651,
  112.601, 115.606, 118.678, 121.791};

/* standard atomic weights, g/mol, Z = 1..94 */
static const double atomic_weight[XRL_MAXZ + 1] = {0.0,
  1.008, 4.0026, 6.94, 9.0122, 10.81, 12.011, 14.007, 15.999, 18.998, 20.180,
  22.990, 24.305, 26.982, 28.085, 30.974, 32.06, 35.45, 39.948, 39.098, 40.078,
  44.956, 47.867, 50.942, 51.996, 54.938, 55.845, 58.933, 58.693, 63.546, 65.38,
  69.723, 72.630, 74.922, 78.971, 79.904, 83.798, 85.468, 87.62, 88.906, 91.224,
  92.906, 95.95, 98.0, 101.07, 102.91, 106.42, 107.87, 112.41, 114.82, 118.71,
  121.76, 127.60, 126.90, 131.29, 132.91, 137.33, 138.91, 140.12, 140.91, 144.24,
  145.0, 150.36, 151.96, 157.25, 158.93, 162.50, 164.93, 167.26, 168.93, 173.05,
  174.97, 178.49, 180.95, 183.84, 186.21, 190.23, 192.22, 195.08, 196.97, 200.59,
  204.38, 207.2, 208.98, 209.0, 210.0, 222.0, 223.0, 226.0, 227.0, 232.04,
  231.04, 238.03, 237.0, 244.0};

/* first Z with electrons in shell (K..Q1, xraylib shell order) */
static const int shell_first_z[XRL_NSHELL_ALL] = {
  1,           /* K */
  3, 5, 5,     /* L1 L2 L3 */
  11, 13, 13, 21, 21,           /* M1..M5 */
  19, 31, 31, 39, 39, 58, 58,   /* N1..N7 */
  37, 49, 49, 57, 57, 90, 90,   /* O1..O7 */
  55, 81, 81, 89, 89,           /* P1..P5 */
  87};                          /* Q1 */

/* full occupancy of each subshell */
static const int shell_capacity[XRL_NSHELL_ALL] = {
  2, 2, 2, 4, 2, 2, 4, 4, 6, 2, 2, 4, 4, 6, 6, 8, 2, 2, 4, 4, 6, 6, 8,
  2, 2, 4, 4, 6, 2};

static const char *shell_names[XRL_NSHELL_ALL] = {
  "K", "L1", "L2", "L3", "M1", "M2", "M3", "M4", "M5",
  "N1", "N2", "N3", "N4", "N5", "N6", "N7",
  "O1", "O2", "O3", "O4", "O5", "O6", "O7",
  "P1", "P2", "P3", "P4", "P5", "Q1"};

static int zok(int Z) { return Z >= 1 && Z <= XRL_MAXZ; }

double xrl_AtomicWeight(int Z) { return zok(Z) ? atomic_weight[Z] : 0.0; }

/* ---------------------------------------------------------------------- */
/* electron configuration: Aufbau filling in the usual subshell order       */
/* ---------------------------------------------------------------------- */
static const int aufbau_order[] = {
  0,            /* 1s */
  1,            /* 2s */
  2, 3,         /* 2p1/2 2p3/2 */
  4,            /* 3s */
  5, 6,         /* 3p */
  9,            /* 4s */
  7, 8,         /* 3d */
  10, 11,       /* 4p */
  16,           /* 5s */
  12, 13,       /* 4d */
  17, 18,       /* 5p */
  23,           /* 6s */
  14, 15,       /* 4f */
  19, 20,       /* 5d */
  24, 25,       /* 6p */
  28,           /* 7s */
  21, 22,       /* 5f */
  26, 27        /* 6d */
};

double xrl_ElectronConfig(int Z, int shell) {
  int occ[XRL_NSHELL_ALL];
  int left, i;
  if (!zok(Z) || shell < 0 || shell >= XRL_NSHELL_ALL) return 0.0;
  memset(occ, 0, sizeof(occ));
  left = Z;
  for (i = 0; i < (int)(sizeof(aufbau_order) / sizeof(int)) && left > 0; i++) {
    int s = aufbau_order[i];
    int take = shell_capacity[s] < left ? shell_capacity[s] : left;
    occ[s] = take;
    left -= take;
  }
  /* a shell listed as occupied from shell_first_z keeps at least one electron
   * (simple treatment of the 4s/3d, 5d/4f irregularities) */
  if (occ[shell] == 0 && Z >= shell_first_z[shell]) return 1.0;
  return (double)occ[shell];
}

static int shell_occupied(int Z, int shell) {
  if (!zok(Z) || shell < 0 || shell >= XRL_NSHELL_ALL) return 0;
  return Z >= shell_first_z[shell];
}

/* ---------------------------------------------------------------------- */
/* binding energies                                                         */
/* ---------------------------------------------------------------------- */
static void binding_energies(int Z, double *eb /* [XRL_NSHELL_ALL] */) {
  double z = (double)Z;
  double ek = k_edge[Z];
  double rl3 = 0.150 - 0.16 * exp(-(z - 10.0) / 14.0);
  double el3, el2, el1, rm5, em5, em4, em3, em2, em1;
  int s;
  if (rl3 < 0.02) rl3 = 0.02;
  el3 = ek * rl3;
  el2 = el3 * (1.0 + 0.3 * pow(z / 100.0, 2.5));
  el1 = el2 * (1.03 + 0.5 * exp(-z / 18.0));
  rm5 = 0.22 - 0.30 * exp(-(z - 30.0) / 20.0);
  if (rm5 < 0.010) rm5 = 0.010;
  em5 = el3 * rm5;
  em4 = em5 * (1.0 + 0.05 * (z / 92.0) * (z / 92.0));
  em3 = em5 * (1.2 + 0.5 * exp(-(z - 40.0) / 12.0));
  if (em3 > 0.8 * el3) em3 = 0.8 * el3;
  em2 = em3 * (1.05 + 0.15 * (z / 92.0) * (z / 92.0));
  em1 = em2 * (1.07 + 0.6 * exp(-(z - 30.0) / 10.0));
  if (em1 > 0.9 * el3) em1 = 0.9 * el3;
  if (em2 > em1) em2 = 0.98 * em1;
  eb[0] = ek;
  eb[1] = el1; eb[2] = el2; eb[3] = el3;
  eb[4] = em1; eb[5] = em2; eb[6] = em3; eb[7] = em4; eb[8] = em5;
  eb[9] = 0.36 * em5;  eb[10] = 0.29 * em5; eb[11] = 0.245 * em5;
  eb[12] = 0.17 * em5; eb[13] = 0.16 * em5; eb[14] = 0.055 * em5; eb[15] = 0.053 * em5;
  eb[16] = 0.060 * em5; eb[17] = 0.040 * em5; eb[18] = 0.033 * em5;
  eb[19] = 0.009 * em5; eb[20] = 0.008 * em5; eb[21] = 0.003 * em5; eb[22] = 0.003 * em5;
  eb[23] = 0.002 * em5; eb[24] = 0.0015 * em5; eb[25] = 0.0012 * em5;
  eb[26] = 0.0010 * em5; eb[27] = 0.0009 * em5; eb[28] = 0.0008 * em5;
  for (s = 0; s < XRL_NSHELL_ALL; s++)
    if (!shell_occupied(Z, s)) eb[s] = 0.0;
}

double xrl_EdgeEnergy(int Z, int shell) {
  double eb[XRL_NSHELL_ALL];
  if (!zok(Z) || shell < 0 || shell >= XRL_NSHELL_ALL) return 0.0;
  binding_energies(Z, eb);
  return eb[shell];
}

/* ---------------------------------------------------------------------- */
/* line names, shells                                                       */
/* ---------------------------------------------------------------------- */
const char *xrl_line_name(int line) {
  if (line < 0 || line > 385) return "";
  return line_names[line];
}

int xrl_line_from_name(const char *name) {
  int i;
  for (i = 1; i < 386; i++)
    if (strcmp(line_names[i], name) == 0) return i;
  return 0;
}

static int parse_shell(const char *s, int *len) {
  int i, best = -1, bestlen = 0;
  for (i = 0; i < XRL_NSHELL_ALL; i++) {
    int l = (int)strlen(shell_names[i]);
    if (strncmp(s, shell_names[i], l) == 0 && l > bestlen) {
      best = i;
      bestlen = l;
    }
  }
  *len = bestlen;
  return best;
}

int xrl_line_lower_shell(int line) {
  int len;
  if (line < 1 || line > XRL_NLINES) return -1;
  return parse_shell(line_names[line], &len);
}

int xrl_line_upper_shell(int line) {
  int len, len2, up;
  const char *n;
  if (line < 1 || line > XRL_NLINES) return -1;
  n = line_names[line];
  if (parse_shell(n, &len) < 0) return -1;
  up = parse_shell(n + len, &len2);
  if (up < 0 || n[len + len2] != '\0') return -1; /* aggregate (KO, L1N67, ...) */
  return up;
}

/* transition ranges scanned by the line selection of the reference */
static const int shell_first[9] = {1, 30, 59, 86, 118, 140, 161, 182, 201};
static const int shell_last[9] = {29, 58, 85, 113, 136, 158, 180, 200, 219};

int xrl_shell_first_line(int shell) { return (shell >= 0 && shell < 9) ? shell_first[shell] : 0; }
int xrl_shell_last_line(int shell) { return (shell >= 0 && shell < 9) ? shell_last[shell] : -1; }

/* ---------------------------------------------------------------------- */
/* radiative transitions                                                    */
/* ---------------------------------------------------------------------- */
/* (line name, relative strength) of the modelled dipole lines; the Z factor
 * is applied in line_strength() */
typedef struct { const char *name; double w; } line_def;
static const line_def model_lines[] = {
  {"KL2", 0.51}, {"KL3", 1.0}, {"KM2", 0.51}, {"KM3", 1.0}, {"KN2", 0.5}, {"KN3", 1.0},
  {"L1M2", 0.6}, {"L1M3", 1.0}, {"L1M4", 0.01}, {"L1M5", 0.015}, {"L1N2", 0.15}, {"L1N3", 0.22},
  {"L2M1", 0.03}, {"L2M3", 0.005}, {"L2M4", 1.0}, {"L2N1", 0.01}, {"L2N4", 0.2},
  {"L3M1", 0.05}, {"L3M4", 0.11}, {"L3M5", 1.0}, {"L3N1", 0.012}, {"L3N4", 0.02}, {"L3N5", 0.18},
  {"M1N2", 0.5}, {"M1N3", 1.0},
  {"M2N1", 0.2}, {"M2N4", 1.0},
  {"M3N1", 0.1}, {"M3N4", 0.1}, {"M3N5", 1.0},
  {"M4N2", 0.05}, {"M4N6", 1.0},
  {"M5N3", 0.05}, {"M5N6", 0.06}, {"M5N7", 1.0}};
#define N_MODEL_LINES ((int)(sizeof(model_lines) / sizeof(model_lines[0])))

/* line index, lower and upper shell of each modelled line, resolved once */
static int model_idx[N_MODEL_LINES], model_lo[N_MODEL_LINES], model_up[N_MODEL_LINES];
static int model_ready = 0;

static void model_init(void) {
  int k;
  if (model_ready) return;
  for (k = 0; k < N_MODEL_LINES; k++) {
    model_idx[k] = xrl_line_from_name(model_lines[k].name);
    model_lo[k] = xrl_line_lower_shell(model_idx[k]);
    model_up[k] = xrl_line_upper_shell(model_idx[k]);
  }
  model_ready = 1;
}

static double line_strength(int Z, int k) {
  int lo = model_lo[k], up = model_up[k];
  double z = (double)Z, w = model_lines[k].w;
  if (lo < 0 || up < 0) return 0.0;
  if (!shell_occupied(Z, lo) || !shell_occupied(Z, up)) return 0.0;
  if (lo == 0 && (up == 5 || up == 6)) w *= 0.10 + 0.12 * (1.0 - exp(-(z - 13.0) / 25.0));
  if (lo == 0 && (up == 10 || up == 11)) w *= 0.02 + 0.05 * (1.0 - exp(-(z - 31.0) / 20.0));
  return w;
}

double xrl_RadRate(int Z, int line) {
  int k, lo, target = -1;
  double sum = 0.0;
  if (!zok(Z) || line < 1 || line > XRL_NLINES) return 0.0;
  model_init();
  lo = xrl_line_lower_shell(line);
  for (k = 0; k < N_MODEL_LINES; k++) {
    if (model_lo[k] != lo) continue;
    sum += line_strength(Z, k);
    if (model_idx[k] == line) target = k;
  }
  if (target < 0 || sum <= 0.0) return 0.0;
  return line_strength(Z, target) / sum;
}

double xrl_LineEnergy(int Z, int line) {
  double eb[XRL_NSHELL_ALL], e;
  int lo, up;
  if (!zok(Z) || line < 1 || line > XRL_NLINES) return 0.0;
  lo = xrl_line_lower_shell(line);
  up = xrl_line_upper_shell(line);
  if (lo < 0 || up < 0) return 0.0;
  binding_energies(Z, eb);
  if (eb[lo] <= 0.0 || eb[up] <= 0.0) return 0.0;
  e = eb[lo] - eb[up];
  return e > 0.0 ? e : 0.0;
}

/* ---------------------------------------------------------------------- */
/* yields and Coster-Kronig                                                  */
/* ---------------------------------------------------------------------- */
double xrl_FluorYield(int Z, int shell) {
  double z4;
  if (!zok(Z) || shell < 0 || shell > 8 || !shell_occupied(Z, shell)) return 0.0;
  z4 = pow((double)Z, 4.0);
  switch (shell) {
    case 0: return z4 / (8.5e5 + z4);
    case 1: return 0.35 * z4 / (1.0e8 + z4);
    case 2: return 1.1 * z4 / (1.0e8 + z4);
    case 3: return z4 / (1.0e8 + z4);
    case 4: case 5: case 6: return 0.5 * z4 / (1.5e9 + z4);
    default: return z4 / (1.5e9 + z4);
  }
}

double xrl_CosKronTransProb(int Z, int trans) {
  double z = (double)Z, sl, sm;
  if (!zok(Z)) return 0.0;
  sl = Z >= 12 ? 1.0 - exp(-(z - 12.0) / 20.0) : 0.0;
  sm = Z >= 40 ? 1.0 - exp(-(z - 40.0) / 20.0) : 0.0;
  switch (trans) {
    case XMI_FL12: return sl > 0.0 ? 0.05 + 0.12 * sl : 0.0;
    case XMI_FL13: return sl > 0.0 ? 0.20 + 0.40 * sl : 0.0;
    case XMI_FLP13: return 0.0;
    case XMI_FL23: return sl > 0.0 ? 0.08 + 0.08 * sl : 0.0;
    case XMI_FM12: return 0.05 * sm;
    case XMI_FM13: return 0.08 * sm;
    case XMI_FM14: return 0.03 * sm;
    case XMI_FM15: return 0.04 * sm;
    case XMI_FM23: return 0.08 * sm;
    case XMI_FM24: return 0.04 * sm;
    case XMI_FM25: return 0.04 * sm;
    case XMI_FM34: return 0.08 * sm;
    case XMI_FM35: return 0.08 * sm;
    case XMI_FM45: return 0.06 * sm;
    default: return 0.0;
  }
}

double xrl_AugerYield(int Z, int shell) {
  double a = 1.0 - xrl_FluorYield(Z, shell);
  if (!zok(Z) || shell < 0 || shell > 8 || !shell_occupied(Z, shell)) return 0.0;
  switch (shell) {
    case 1: a -= xrl_CosKronTransProb(Z, XMI_FL12) + xrl_CosKronTransProb(Z, XMI_FL13); break;
    case 2: a -= xrl_CosKronTransProb(Z, XMI_FL23); break;
    case 4: a -= xrl_CosKronTransProb(Z, XMI_FM12) + xrl_CosKronTransProb(Z, XMI_FM13) +
                 xrl_CosKronTransProb(Z, XMI_FM14) + xrl_CosKronTransProb(Z, XMI_FM15); break;
    case 5: a -= xrl_CosKronTransProb(Z, XMI_FM23) + xrl_CosKronTransProb(Z, XMI_FM24) +
                 xrl_CosKronTransProb(Z, XMI_FM25); break;
    case 6: a -= xrl_CosKronTransProb(Z, XMI_FM34) + xrl_CosKronTransProb(Z, XMI_FM35); break;
    case 7: a -= xrl_CosKronTransProb(Z, XMI_FM45); break;
    default: break;
  }
  return a > 0.0 ? a : 0.0;
}

double xrl_AugerVacancies(int Z, int s, int t) {
  static const double k_to[9] = {0.0, 0.40, 0.45, 0.85, 0.05, 0.05, 0.10, 0.02, 0.03};
  static const double l1_to[9] = {0, 0, 0, 0, 0.20, 0.20, 0.40, 0.40, 0.60};
  static const double l23_to[9] = {0, 0, 0, 0, 0.15, 0.15, 0.30, 0.50, 0.70};
  if (!zok(Z) || t < 0 || t > 8 || !shell_occupied(Z, t)) return 0.0;
  if (s == 0) return k_to[t];
  if (s == 1) return l1_to[t];
  if (s == 2 || s == 3) return l23_to[t];
  return 0.0;
}

/* Probability of Auger transition `trans` in xraylib's numbering (0..239 a
 * K vacancy, 240..374 L1, 375..509 L2, 510..644 L3) given a non-radiative
 * decay.  The transition of a K vacancy fills vacancies (a, b) with a in
 * L1..M5 and b in L1..Q3 (list positions 1..30: L1..L3, M1..M5, N1..N7,
 * O1..O7, P1..P5, Q1..Q3); of an L vacancy a in M1..M5, b in M1..Q3.  The
 * stand-in rate is p_a q_b: p follows the expected vacancies of
 * xrl_AugerVacancies over the first shell's range (normalised), q puts half of
 * them on the same shells and the rest on the occupied outer shells by
 * occupancy, so that the mean vacancies per decay stay close to
 * xrl_AugerVacancies. */
double xrl_AugerRate(int Z, int trans) {
  int s0, t, nb, first0, a, b, k;
  double p[31], q[31], sp = 0.0, sq = 0.0, outer = 0.0, vsum = 0.0;
  if (!zok(Z) || trans < 0 || trans > 644) return 0.0;
  if (trans < 240) { s0 = 0; t = trans; nb = 30; first0 = 1; }
  else { s0 = 1 + (trans - 240) / 135; t = (trans - 240) % 135; nb = 27; first0 = 4; }
  if (!shell_occupied(Z, s0)) return 0.0;
  a = first0 + t / nb;
  b = first0 + t % nb;
  for (k = 0; k <= 30; k++) p[k] = q[k] = 0.0;
  for (k = first0; k <= 8; k++) {
    const double v = xrl_AugerVacancies(Z, s0, k);
    p[k] = v;
    q[k] = 0.5 * v;
    sp += v;
    vsum += 0.5 * v;
  }
  for (k = 9; k <= 30; k++) {
    q[k] = k < XRL_NSHELL_ALL ? xrl_ElectronConfig(Z, k) : 0.0;
    outer += q[k];
  }
  for (k = 9; k <= 30; k++) q[k] = outer > 0.0 ? q[k] / outer * (vsum < 1.0 ? 1.0 - vsum : 0.0) : 0.0;
  for (k = first0; k <= 30; k++) sq += q[k];
  if (sp <= 0.0 || sq <= 0.0) return 0.0;
  return (p[a] / sp) * (q[b] / sq);
}

/* ---------------------------------------------------------------------- */
/* photo-absorption: jump-ratio partition of a power-law envelope           */
/* ---------------------------------------------------------------------- */
static double jump_ratio(int Z, int s) {
  double z = (double)Z;
  switch (s) {
    case 0: return 3.8 + 65.0 / pow(z, 0.9);
    case 1: return 1.16;
    case 2: return 1.40;
    case 3: return 3.0 - 0.006 * z;
    case 4: return 1.05;
    case 5: return 1.08;
    case 6: return 1.20;
    case 7: return 1.40;
    default: return 1.80;
  }
}

static double photo_envelope(int Z, double E) {
  return 43.7 * pow((double)Z, 3.7) / atomic_weight[Z] * pow(E, -2.75);
}

double xrl_CS_Photo_Partial(int Z, int shell, double E) {
  double eb[XRL_NSHELL_ALL], f;
  int t;
  if (!zok(Z) || shell < 0 || shell > 8 || E <= 0.0) return 0.0;
  binding_energies(Z, eb);
  if (eb[shell] <= 0.0 || E < eb[shell]) return 0.0;
  f = photo_envelope(Z, E) * (1.0 - 1.0 / jump_ratio(Z, shell));
  for (t = 0; t < shell; t++)
    if (eb[t] > 0.0) f /= jump_ratio(Z, t);
  return f;
}

double xrl_CS_Photo_Total(int Z, double E) {
  double eb[XRL_NSHELL_ALL], f, tot = 0.0, below = 1.0;
  int t;
  if (!zok(Z) || E <= 0.0) return 0.0;
  binding_energies(Z, eb);
  f = photo_envelope(Z, E);
  for (t = 0; t < 9; t++) {
    if (eb[t] <= 0.0) continue;
    if (E >= eb[t]) tot += f * below * (1.0 - 1.0 / jump_ratio(Z, t));
    below /= jump_ratio(Z, t);
  }
  return tot + f * below; /* remaining outer-shell absorption */
}

/* ---------------------------------------------------------------------- */
/* scattering                                                               */
/* ---------------------------------------------------------------------- */
double xrl_FF_Rayl(int Z, double q) {
  double q0, x;
  if (!zok(Z)) return 0.0;
  q0 = 0.55 * pow((double)Z, 0.45);
  x = 1.0 + (q / q0) * (q / q0);
  return (double)Z / (x * x);
}

double xrl_SF_Compt(int Z, double q) {
  double qs, x;
  if (!zok(Z)) return 0.0;
  qs = 0.45 * pow((double)Z, 0.35);
  x = 1.0 + (q / qs) * (q / qs);
  return (double)Z * (1.0 - 1.0 / (x * x));
}

static double moment_transfer(double E, double theta) {
  return E / XRL_KEV2ANGST * sin(theta / 2.0);
}

double xrl_DCS_Rayl(int Z, double E, double theta) {
  double ff, ct = cos(theta);
  if (!zok(Z)) return 0.0;
  ff = xrl_FF_Rayl(Z, moment_transfer(E, theta));
  return XRL_RE2 * (1.0 + ct * ct) / 2.0 * ff * ff * XRL_AVOGNUM / atomic_weight[Z];
}

double xrl_DCS_Compt(int Z, double E, double theta) {
  double ct = cos(theta), st = sin(theta);
  double k0k = 1.0 + (1.0 - ct) * E / XRL_MEC2, kk0 = 1.0 / k0k;
  double kn = XRL_RE2 / 2.0 * kk0 * kk0 * (kk0 + k0k - st * st);
  if (!zok(Z)) return 0.0;
  return kn * xrl_SF_Compt(Z, moment_transfer(E, theta)) * XRL_AVOGNUM / atomic_weight[Z];
}

double xrl_DCSP_Rayl(int Z, double E, double theta, double phi) {
  double ff, st = sin(theta), cp = cos(phi);
  if (!zok(Z)) return 0.0;
  ff = xrl_FF_Rayl(Z, moment_transfer(E, theta));
  return XRL_RE2 * (1.0 - st * st * cp * cp) * ff * ff * XRL_AVOGNUM / atomic_weight[Z];
}

double xrl_DCSP_Compt(int Z, double E, double theta, double phi) {
  double ct = cos(theta), st = sin(theta), cp = cos(phi);
  double k0k = 1.0 + (1.0 - ct) * E / XRL_MEC2, kk0 = 1.0 / k0k;
  double kn = XRL_RE2 / 4.0 * kk0 * kk0 * (kk0 + k0k - 2.0 * st * st * cp * cp);
  if (!zok(Z)) return 0.0;
  return kn * xrl_SF_Compt(Z, moment_transfer(E, theta)) * XRL_AVOGNUM / atomic_weight[Z];
}

/* integrated cross sections: Simpson rule over theta */
static double integrate_theta(int Z, double E, int rayl) {
  const int n = 1000; /* even */
  double h = M_PI / n, sum = 0.0;
  int i;
  for (i = 0; i <= n; i++) {
    double th = i * h;
    double f = (rayl ? xrl_DCS_Rayl(Z, E, th) : xrl_DCS_Compt(Z, E, th)) * sin(th);
    double c = (i == 0 || i == n) ? 1.0 : ((i & 1) ? 4.0 : 2.0);
    sum += c * f;
  }
  return 2.0 * M_PI * sum * h / 3.0;
}

/* The integrated scattering cross sections are defined as the log-log
 * interpolation of the Simpson integral on a fixed log grid (0.05-250 keV,
 * 601 points), built once per Z. */
#define XRL_CS_NG 601
#define XRL_CS_ELO 0.05
#define XRL_CS_EHI 250.0
static double *cs_cache[XRL_MAXZ + 1][2];

void xrl_prepare(int Z) {
  int k, i;
  model_init();
  if (!zok(Z)) return;
  for (k = 0; k < 2; k++) {
    double *t;
    if (cs_cache[Z][k]) continue;
    t = (double *)malloc(sizeof(double) * XRL_CS_NG);
    for (i = 0; i < XRL_CS_NG; i++) {
      double le = log(XRL_CS_ELO) + (log(XRL_CS_EHI) - log(XRL_CS_ELO)) * i / (XRL_CS_NG - 1);
      t[i] = log(integrate_theta(Z, exp(le), k == 0));
    }
    cs_cache[Z][k] = t;
  }
}

static double cs_interp(int Z, int k, double E) {
  double lo = log(XRL_CS_ELO), hi = log(XRL_CS_EHI);
  double x, f;
  int i;
  if (!cs_cache[Z][k]) xrl_prepare(Z);
  x = (log(E) - lo) / (hi - lo) * (XRL_CS_NG - 1);
  i = (int)floor(x);
  if (i < 0) i = 0;
  if (i > XRL_CS_NG - 2) i = XRL_CS_NG - 2;
  f = x - i;
  return exp(cs_cache[Z][k][i] + f * (cs_cache[Z][k][i + 1] - cs_cache[Z][k][i]));
}

double xrl_CS_Rayl(int Z, double E) { return (zok(Z) && E > 0.0) ? cs_interp(Z, 0, E) : 0.0; }
double xrl_CS_Compt(int Z, double E) { return (zok(Z) && E > 0.0) ? cs_interp(Z, 1, E) : 0.0; }

double xrl_CS_Total_Kissel(int Z, double E) {
  return xrl_CS_Photo_Total(Z, E) + xrl_CS_Rayl(Z, E) + xrl_CS_Compt(Z, E);
}

/* Compton profile: sum over occupied shells of hydrogenic-shaped profiles
 * J_s(pz) = n_s 8/(3 pi sigma) (1+(pz/sigma)^2)^-3, sigma from the binding energy */
double xrl_ComptonProfile(int Z, double pz) {
  double eb[XRL_NSHELL_ALL], j = 0.0;
  int s;
  if (!zok(Z)) return 0.0;
  binding_energies(Z, eb);
  for (s = 0; s < XRL_NSHELL_ALL; s++) {
    double n = xrl_ElectronConfig(Z, s), ebs, sig, x;
    if (n <= 0.0) continue;
    ebs = eb[s] > 0.005 ? eb[s] : 0.005;
    sig = sqrt(2.0 * ebs / 0.0272114);
    x = 1.0 + (pz / sig) * (pz / sig);
    j += n * 8.0 / (3.0 * M_PI * sig) / (x * x * x);
  }
  return j;
}
