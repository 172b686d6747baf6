/*
 * Table bundle: the host-side, plain-C description of one simulation
 * (geometry after initialisation, layers, source items, tabulated physics,
 * solid-angle grid and run options).  It plays the role of the reference's
 * `xmi_input` Fortran TYPE plus the `xmi_hdf5` tables
 * (src/xmi_aux_f.F90:89-117, 420-523) after xmi_init_input
 * (src/xmi_main.F90:1741-1918) and xmi_init_from_hdf5 (src/xmi_data_f.F90:164).
 *
 * The engine library fills it (host tabulation) and uploads a copy to the
 * GPU; the FP64 CPU oracle under oracle/ reads the very same host arrays so
 * that the GPU kernels and the oracle consume identical numbers.
 *
 * Indexing conventions (all 0-based in C):
 *  - shells: 0=K, 1=L1, 2=L2, 3=L3, 4=M1 .. 8=M5 (xraylib's K_SHELL..M5_SHELL)
 *  - lines: 1..383 = minus the xraylib line macro (KL1=1 .. P3P5=383),
 *           384 = Rayleigh, 385 = Compton (history layout of the reference)
 *  - element index e: position in the run's list of distinct sample elements
 *  - line slot: position in the run's concatenated per-element line lists
 */
#ifndef XMIMSIM_GB300_BUNDLE_H
#define XMIMSIM_GB300_BUNDLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define XMI_MAXL 8        /* maximum number of sample layers */
#define XMI_MAXN 10       /* maximum interactions per trajectory */
#define XMI_NSHELL 9      /* K..M5 */
#define XMI_NCK 14        /* Coster-Kronig transitions FL12..FM45 */
#define XMI_MAXSEG 2048   /* maximum energy-grid segments */

/* per-node record of element tables (el_tab) */
enum {
  XMI_REC_TOT = 0,    /* CS_Total_Kissel(Z,E) cm2/g */
  XMI_REC_PR = 1,     /* CS_Rayl/CS_Total (interaction_probs col 1) */
  XMI_REC_PRC = 2,    /* (CS_Rayl+CS_Compt)/CS_Total (col 2) */
  XMI_REC_PHOTO = 3,  /* CS_Photo_Total */
  XMI_REC_XRF = 4,    /* 4..12: cascade-corrected P_shell (PK..PM5), 16-byte aligned */
  XMI_REC_PART = 13,  /* 13..21: CS_Photo_Partial(Z,shell,E) */
  XMI_EL_REC = 24     /* 96-byte records (2 unused), so a record starts on 16 bytes */
};

/* Coster-Kronig transition indices (xraylib FL12_TRANS..FM45_TRANS order) */
enum {
  XMI_FL12 = 0, XMI_FL13, XMI_FLP13, XMI_FL23,
  XMI_FM12, XMI_FM13, XMI_FM14, XMI_FM15,
  XMI_FM23, XMI_FM24, XMI_FM25, XMI_FM34, XMI_FM35, XMI_FM45
};

/* cascade types (reference src/xmi_aux_f.F90:660-663) */
enum { XMI_CASCADE_NONE = 1, XMI_CASCADE_NONRADIATIVE = 2,
       XMI_CASCADE_RADIATIVE = 3, XMI_CASCADE_FULL = 4 };

/* interaction codes (reference src/xmi_aux_f.F90:653-656) */
enum { XMI_NO_INTERACTION = 0, XMI_RAYLEIGH = 1, XMI_COMPTON = 2,
       XMI_PHOTOELECTRIC = 3 };

/* theta ICDF grids (reference src/xmi_data.c:148-151) */
#define XMI_SEG_LUT 4096
#define XMI_ICDF_NE 400
#define XMI_ICDF_NR 2000
#define XMI_PHI_NT 200
#define XMI_DOPPLER_N 10001
#define XMI_NQ 4096
#define XMI_AUGER_K 240   /* Auger transitions of a K vacancy (xraylib K_L1L1..K_M5Q3) */
#define XMI_AUGER_L 135   /* of an L1, L2 or L3 vacancy (L*_M1M1..L*_M5Q3) */
#define XMI_CP_N 10001    /* Compton profile grids (reference src/xmi_data.c:152) */
#define XMI_CP_SH 32      /* room for every shell with electrons (29 in xraylib's K..Q1 order) */
#define XMI_QMAX 20.0

/* one source item: a valid continuous interval or a discrete line
 * (reference src/xmi_main.F90:319-858) */
typedef struct {
  int kind;          /* 0 continuous interval, 1 discrete line */
  int dist_type;     /* discrete: XmiEnergyDiscreteDistribution */
  int64_t first;     /* first global photon id of this item */
  int64_t n_photons; /* photons simulated for this item */
  double e0, e1;     /* interval ends (continuous) / e0 = line energy */
  double i0, i1;     /* total intensity density at e0,e1 (continuous) */
  double h0, h1;     /* horizontal intensity density at e0,e1 */
  double hor_ver_ratio; /* discrete: H*n/(H+V) threshold on the 1-based index */
  double weight;     /* initial photon weight */
  double trap[6];    /* trapezoid workspace: denom, m, x1, x2, y1, y2 */
  double sigma_x, sigma_xp, sigma_y, sigma_yp;
  double scale;      /* gaussian sigma / lorentzian scale */
  int64_t local0;    /* index of this replica's first photon within the item */
} xmi_source_item;

typedef struct {
  /* ---- run options ---- */
  int n_interactions;   /* n_interactions_trajectory */
  int use_vr;           /* use_variance_reduction */
  int use_M_lines;
  int cascade_type;     /* XMI_CASCADE_* */
  int escape_mode;      /* escape_ratios_mode (escape-ratio MC) */
  int use_advanced_compton; /* 1: per-shell impulse-approximation Compton (needs the cp_* tables) */
  int nchannels;
  double gain, zero, live_time;
  uint64_t seed;        /* Philox key */
  int line_last;        /* 219 (M5P5) with M lines, else 113 (L3Q1) */
  int max_shell;        /* 8 (M5) with M lines, else 3 (L3) */

  /* ---- geometry after xmi_init_input (src/xmi_main.F90:1741-1918) ---- */
  double n_sample[3];
  double p_det[3];
  double n_det[3];
  double det_new[9];    /* detector frame, row-major: det_new[3*r+c] */
  double det_inv[9];    /* inverse, row-major */
  double det_radius;
  double coll_radius, coll_height;
  double coll_half_apex, coll_vertex_x; /* conical collimator in the detector frame */
  int coll_present;
  int n_layers;
  int reference_layer;  /* 0-based */
  double d_source_slit, slit_x, slit_y;
  double layer_zbeg[XMI_MAXL], layer_zend[XMI_MAXL];
  double layer_rho[XMI_MAXL], layer_thickz[XMI_MAXL];
  int layer_nel[XMI_MAXL], layer_off[XMI_MAXL];
  int n_layer_el;       /* total (layer, element) pairs */
  int *layer_el;        /* element index per pair */
  double *layer_w;      /* weight fraction per pair */

  /* ---- elements ---- */
  int n_elem;
  int *elem_Z;              /* [n_elem] */
  double *elem_yield_corr;  /* [n_elem][9] FluorYieldsCorr (CK folded) */
  double *elem_fluor_yield; /* [n_elem][9] FluorYield */
  double *elem_ck;          /* [n_elem][14] CosKronTransProb */
  double *elem_edge;        /* [n_elem][9] EdgeEnergy */
  int *elem_line_off;       /* [n_elem+1] into the line slot arrays */
  int *elem_shell_off;      /* [n_elem][10] first slot of each shell, slot range of shell s = [off[s], off[s+1]) */

  /* ---- line slots (all lines with RadRate > 0, sorted by line index per element) ---- */
  int n_lines;
  int *line_index;      /* 1..383 */
  int *line_elem;       /* element of the slot */
  int *line_shell;      /* 0..8 */
  double *line_energy;  /* LineEnergy */
  double *line_rate;    /* RadRate */
  int *line_channel;    /* INT((E-zero)/gain) or -1 */
  double *precalc_mu;   /* [n_layers][n_lines] mu of each layer at each line energy */
  double *precalc_xrf;  /* [n_elem][9][n_lines] P_shell of element at line energy */

  /* ---- energy grid: segments between absorption edges, log-uniform inside ---- */
  int n_seg;
  double *seg_lo;       /* [n_seg+1] breakpoints (keV) */
  double *seg_lnlo;     /* [n_seg] log(seg_lo) */
  double *seg_invh;     /* [n_seg] 1/log-step */
  int *seg_off;         /* [n_seg] first node */
  int *seg_n;           /* [n_seg] nodes in segment (>= 2) */
  /* segment search table: bin i of XMI_SEG_LUT uniform bins in log E over
   * [seg_lo[0], seg_lo[n_seg]] holds the segment of its lower edge, so the
   * segment of an energy is found from its bin with a step or two */
  int *seg_lut;         /* [XMI_SEG_LUT] */
  double seg_lut_ln0, seg_lut_inv;
  int n_nodes;
  double *el_tab;       /* [n_elem][n_nodes][XMI_EL_REC] */
  double *mu_tab;       /* [n_nodes][XMI_MAXL] layer mu (xmi_mu_calc) */
  double *exc_tab;      /* [n_nodes] sum over excitation absorbers of rho*t*mu(E) */

  /* ---- angular tables ---- */
  double *icdf_energies;  /* [400] 0.1..200 keV */
  double *icdf_rs;        /* [2000] 0..1 */
  /* tables that depend on Z alone are shared by every bundle of the process:
   * per element a pointer into the cache, not owned by the bundle */
  const double **rayl_icdf;  /* [n_elem] -> [400][2000] theta */
  const double **compt_icdf; /* [n_elem] -> [400][2000] theta */
  double *phi_thetas;     /* [200] 0..0.5 */
  const double *phi_icdf; /* [200][2000], shared by every bundle of the process */
  double *doppler_rs;     /* [10001] */
  const double **doppler_icdf; /* [n_elem] -> [10001] pz */
  const double **ff2;      /* [n_elem] -> [XMI_NQ] Rayleigh form factor squared x N_A/A x r_e^2 */
  const double **sf;       /* [n_elem] -> [XMI_NQ] incoherent scattering function x N_A/A */

  /* ---- source ---- */
  int n_items;
  xmi_source_item *items;
  int64_t n_photons_total;

  /* ---- solid-angle grid (VR only) ---- */
  int sa_nr, sa_nt;
  double *sa_r, *sa_t;   /* [sa_nr], [sa_nt] */
  double *sa_grid;       /* [sa_nt][sa_nr] */
  int sa_hits_per_single;

  /* tally layout */
  int n_slots;           /* n_lines + 2*n_elem: Rayleigh at n_lines+2e, Compton +1 */

  /* ---- estimator line lists ----
   * Per (layer, element) pair, the line slots the variance-reduction
   * estimator visits (src/xmi_variance_reduction.F90:575-709): energy >= 1 keV,
   * line <= line_last, not L1L2/L1L3/L2L3, FluorYield x RadRate > 0.
   * Entries of pair k: [ent_off[k], ent_off[k+1]). */
  int n_ent;
  int *ent_off;          /* [n_layer_el+1] */
  int *ent_slot;         /* [n_ent] line slot */
  int *ent_shell;        /* [n_ent] 0..8 */
  double *ent_coef;      /* [n_ent] FluorYield(Z, shell) x RadRate(Z, line) */
  double *ent_pmu;       /* [n_ent][XMI_MAXL] precalc_mu of every layer at the line energy (0 beyond n_layers) */
  int stage_max;         /* max over layers of (line entries + 2 x elements): history slots one layer feeds */

  /* ---- analog cascades (VR off; reference src/xmi_main.F90:2413-4783) ----
   * Radiative: after a line from shell s, the vacancy moves to the line's
   * upper shell u and may emit again: line_casc_shell[slot] = u for K lines
   * to L1..M5 and L lines to M1..M5 (the latter only with M lines), else -1.
   * Auger: a K/L1/L2/L3 vacancy decaying without a photon picks transition t
   * with probability auger_rate[(e * 4 + s) * XMI_AUGER_K + t]; its two new
   * vacancies are (1 + t / 30, 1 + t % 30) for K and (4 + t / 27, 4 + t % 27)
   * for L, as positions of the list L1 L2 L3 M1..M5 N1..N7 O1..O7 P1..P5 Q1..Q3
   * (positions 1..8 are the shells L1..M5 of the line tables). */
  int *line_casc_shell;  /* [n_lines] */
  double *auger_rate;    /* [n_elem][4][XMI_AUGER_K] */

  /* ---- per-shell Compton profiles (advanced Compton; reference
   * src/xmi_data_f.F90:1124-1230), built on demand by
   * xmi_bundle_compton_profiles: NULL until then.  Shell k of element e is
   * the k-th shell with electrons, K first.  Q grid: Q_j = 100 j / (N - 1);
   * CDF grid: c_j = 0.5 j / (N - 1), N = XMI_CP_N. ---- */
  int *cp_nshell;          /* [n_elem] */
  int *cp_shell;           /* [n_elem][XMI_CP_SH] xraylib shell index */
  double *cp_occ;          /* [n_elem][XMI_CP_SH] electrons in the shell (ElectronConfig_Biggs) */
  double *cp_edge;         /* [n_elem][XMI_CP_SH] binding energy EdgeEnergy(Z, shell), keV */
  const double **cp_cdf;   /* [n_elem] -> [nshell][N] partial profile integral over [0, Q_j], scaled to 0.5 at Q = 100 */
  const double **cp_qinv;  /* [n_elem] -> [nshell][N] Q at which that integral reaches c_j */
} xmi_bundle;

/* Evaluation rule of every energy table of the bundle: E is located in the
 * segment [seg_lo[k], seg_lo[k+1]) and the value is interpolated linearly in
 * log(E) between the two nodes around it: v = tab[i] + f*(tab[i+1]-tab[i]).
 * Energies outside the grid are clamped to its ends. */
#include <math.h>
static inline void xmi_grid_locate(const xmi_bundle *b, double E, int *node, double *frac) {
  int lo = 0, hi = b->n_seg - 1, k, i;
  double t;
  if (E <= b->seg_lo[0]) { *node = 0; *frac = 0.0; return; }
  if (E >= b->seg_lo[b->n_seg]) { *node = b->n_nodes - 2; *frac = 1.0; return; }
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (E >= b->seg_lo[mid]) lo = mid; else hi = mid - 1;
  }
  k = lo;
  t = (log(E) - b->seg_lnlo[k]) * b->seg_invh[k];
  i = (int)t;
  if (i < 0) i = 0;
  if (i > b->seg_n[k] - 2) i = b->seg_n[k] - 2;
  *node = b->seg_off[k] + i;
  *frac = t - (double)i;
}

#ifdef __cplusplus
}
#endif
#endif
