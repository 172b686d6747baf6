/* Device view of the table bundle and small device helpers shared by the
 * transport, solid-angle and detector kernels. */
#ifndef XMIMSIM_GB300_DEV_BUNDLE_CUH
#define XMIMSIM_GB300_DEV_BUNDLE_CUH

#include <cstdint>
#include "../../include/xmimsim_bundle.h"
#include "philox.h"

namespace xmi {

constexpr double kEnergyThreshold = 1.0;  /* src/xmi_aux_f.F90:673 */
constexpr double kEnergyMax = 200.0;      /* src/xmi_aux_f.F90:674 */
constexpr double kPi = 3.14159265358979323846;
/* words per (element, line) record of the device copy of precalc_xrf: the 9
 * shell factors, padded to 12 so that a record is three 16-byte words (FP32) */
constexpr int kXrfRec = 12;

/* FP32 working copy of a source item, read by the FP32 transport's source
 * sampling instead of the FP64 fields.  Intensities are divided by
 * max(i0, i1): the trapezoid's inverse CDF and the horizontal share are
 * ratios, unchanged by a common scale, and the scaled values stay far from
 * FP32 overflow. */
struct __align__(16) ItemF {
  float e0, de, inv_de, y1;  /* interval start (line energy), width, 1 / width, intensity at e0 */
  float m, area, h0, dh;     /* slope, area, horizontal intensity at e0 and its change over the interval */
  float i0, di, weight, scale; /* total intensity at e0 and its change, photon weight, line width */
  int gauss, pad0, pad1, pad2; /* 1: Gaussian beam (sigma_x * sigma_y != 0) */
};

__host__ inline ItemF item_f_of(const xmi_source_item &it) {
  ItemF f = {};
  const double big = it.i0 > it.i1 ? it.i0 : it.i1, s = big > 0.0 ? 1.0 / big : 1.0;
  f.e0 = (float)it.e0;
  if (it.kind == 0) {
    f.de = (float)(it.e1 - it.e0);
    f.inv_de = (float)(1.0 / (it.e1 - it.e0));
    f.y1 = (float)(it.trap[4] * s);
    f.m = (float)(it.trap[1] * s);
    f.area = (float)(it.trap[0] * s);
    f.h0 = (float)(it.h0 * s);
    f.dh = (float)((it.h1 - it.h0) * s);
    f.i0 = (float)(it.i0 * s);
    f.di = (float)((it.i1 - it.i0) * s);
  }
  f.weight = (float)it.weight;
  f.scale = (float)it.scale;
  f.gauss = (it.sigma_x * it.sigma_y < 0.0 ? -(it.sigma_x * it.sigma_y) : it.sigma_x * it.sigma_y) < (double)1.0e-20f ? 0 : 1;
  return f;
}

/* Device copy of an xmi_bundle.  R is the precision of the physics tables
 * and of the per-photon arithmetic except positions, which are always FP64
 * (FP32 cannot resolve 10 nm layers at 10-100 cm from the origin). */
template <typename R>
struct DevBundle {
  int N, nch, use_vr, use_M_lines, line_last, max_shell, escape_mode;
  int n_layers, n_elem, n_lines, n_slots, n_nodes, n_seg, n_items, n_layer_el;
  int coll_present, sa_nr, sa_nt, sa_hits;
  int use_surrogate; /* solid angles of the estimator from the surrogate network */
  unsigned long long seed;
  long long n_photons_total;
  double gain, zero;
  double n_sample[3], p_det[3], n_det[3], det_new[9], det_inv[9];
  /* the same in the working precision (no FP64 -> FP32 conversions on the step) */
  R n_sample_r[3], n_det_r[3], det_new_r[9], det_inv_r[9], det_radius_r;
  R zero_r, inv_gain_r; /* channel = (E - zero) / gain as (E - zero_r) * inv_gain_r */
  double det_radius, coll_radius, coll_height, coll_half_apex, coll_vertex_x;
  double d_source_slit, slit_x, slit_y;
  double slit_ax, slit_ay; /* half-angles of the slit seen from the source, atan(slit / d / 2), from the host */
  R slit_ax_r, slit_ay_r, d_source_slit_r;
  double hbeg0; /* height of the first layer's entry plane along the sample normal, zbeg[0] n_z */
  double zbeg[XMI_MAXL], zend[XMI_MAXL];
  R thick_n[XMI_MAXL]; /* layer thickness along the sample normal, (zend - zbeg) n_z */
  R rho[XMI_MAXL];
  int nel[XMI_MAXL], off[XMI_MAXL];
  /* sa grid metadata (uniform axes) */
  double sa_r0, sa_rinv, sa_t0, sa_tinv;

  const int *layer_el;
  const R *layer_w;
  const int *elem_Z;
  const R *yield_corr, *fluor_yield, *ck;
  const int *line_off, *shell_off;
  const int *line_index, *line_shell;
  const R *line_energy, *line_rate;
  const R *precalc_mu;
  const R *precalc_xrf; /* [n_elem][n_lines][kXrfRec]: the host's [n_elem][9][n_lines] regrouped by line */
  const R *seg_lo, *seg_lnlo, *seg_invh;
  const int *seg_off, *seg_n, *seg_lut;
  /* FP32 copies of a segment's fields in one record, for the FP32 grid
   * location: {seg_lo[i], seg_lo[i + 1], seg_lnlo[i], seg_invh[i]} and
   * {seg_off[i], seg_n[i]} */
  const float4 *seg_rec;
  const int2 *seg_on;
  R seg_lut_ln0, seg_lut_inv;
  const R *el_tab, *mu_tab, *exc_tab;
  /* [n_nodes][n_layer_el]: per layer, the running sum over its elements of
   * weight x total cross section (the last term of a layer is its mu) */
  const R *layer_cs;
  const R *icdf_e, *icdf_r, *phi_t, *phi_icdf, *dop_r;
  /* per element: device copies of the tables that depend on Z alone, shared
   * by every bundle on the device */
  const R *const *rayl_icdf, *const *compt_icdf, *const *dop_icdf, *const *ff2, *const *sf;
  const xmi_source_item *items;
  const ItemF *items_f;        /* [n_items] FP32 working copies (FP32 transport) */
  const long long *item_first; /* [n_items] global id of the first photon */
  const double *sa_r, *sa_t;
  const R *sa_grid;
  /* estimator line lists per (layer, element) pair */
  int n_ent, stage_max;
  const int *ent_off, *ent_slot, *ent_shell;
  const R *ent_coef, *ent_pmu;
  /* analog cascades (VR off): flags, the radiative cascade's next shell per
   * line slot, Auger transition probabilities [n_elem][4][XMI_AUGER_K] */
  int casc_auger, casc_rad;
  const int *line_casc;
  const R *auger_rate;
  /* per-shell Compton profiles (advanced Compton; null unless in use) */
  int use_adv_compton;
  const int *cp_nshell;                 /* [n_elem] */
  const double *cp_occ, *cp_edge;       /* [n_elem][XMI_CP_SH] */
  const R *const *cp_cdf, *const *cp_qinv; /* [n_elem] -> [nshell][XMI_CP_N] */
};

/* Tally buffers of one run (device pointers). */
struct DevTally {
  double *hist_vr;    /* [N][n_slots] */
  double *hist_brute; /* [N][n_slots] */
  double *chan;       /* [N+1][nch] per order (non-cumulative) */
  unsigned long long *counters; /* [0] off-grid solid angles, [1] error code, [2] photons done */
};

__host__ __device__ inline double dot3(const double *a, const double *b) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

}  // namespace xmi
#endif
