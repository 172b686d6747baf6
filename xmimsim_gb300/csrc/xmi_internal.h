/* Internal declarations shared by the host (C) and device (CUDA) parts of
 * the engine library.  Not part of the public C-ABI. */
#ifndef XMIMSIM_GB300_INTERNAL_H
#define XMIMSIM_GB300_INTERNAL_H

#include "../../include/xmi_data_structs.h"
#include "../../include/xmimsim_bundle.h"
#include "../../include/xmimsim_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* opaque input handle behind xmi_inputFPtr: a deep copy of the caller's
 * xmi_input plus the derived geometry of xmi_init_input */
struct xmi_input_handle {
  xmi_input *input;
  int initialized;
  double n_sample[3], p_det[3], n_det[3];
  double det_new[9], det_inv[9];
  double det_radius, coll_radius, coll_height, detector_solid_angle;
  double coll_half_apex, coll_vertex_x;
  int coll_present;
  double layer_zbeg[XMI_MAXL], layer_zend[XMI_MAXL], layer_thickz[XMI_MAXL];
  int escape_geometry; /* built by xmi_init_input_escape_ratios */
  xmi_gpu_options gpu;
  void *surrogate; /* trained solid-angle network (owned by the CUDA side) */
};

/* opaque table handle behind xmi_hdf5FPtr */
struct xmi_tables_handle {
  xmi_bundle b;
  int cascade_type, use_M_lines;
  double *exc_tab;   /* [n_nodes] sum over excitation absorbers of rho*t*mu(E) */
  int replica, n_replicas; /* photon-range partition of this process (0 of 1 by default) */
  void *dev;         /* device mirror, owned by the CUDA side */
  const double *dev_sa_src; /* host grid pointer the device copy was made from */
};

/* host helpers (host.c) */
int xmi_bundle_build(struct xmi_input_handle *in, struct xmi_tables_handle *t,
                     const xmi_main_options *options);
void xmi_bundle_free(xmi_bundle *b);
int xmi_bundle_compton_profiles(xmi_bundle *b);
void xmi_bundle_set_run(struct xmi_input_handle *in, struct xmi_tables_handle *t,
                        const xmi_main_options *options, int n_mpi_hosts,
                        int replica, int n_replicas);
double xmi_layer_mu(const xmi_layer *layer, double E);
void xmi_solid_angle_axes(const struct xmi_input_handle *h, int nr, int nt, double *r_vals, double *t_vals);
void xmi_set_error(const char *fmt, ...);
/* 1 once the host tabulator has built a table of any element */
int xmi_host_tables_built(void);
/* the atomic data source in use (xmi_set_atomic_data) */
#define XD (xmi_get_atomic_data())
void xmi_log(int verbose, const char *fmt, ...);

/* device side (engine.cu) */
int xmi_dev_sync_tables(struct xmi_tables_handle *t, int precision);
void xmi_dev_free_tables(struct xmi_tables_handle *t);
/* copies the FP64 device view (xmi::DevBundle<double>) into out */
int xmi_dev_bundle_copy64(struct xmi_tables_handle *t, void *out);

/* surrogate network (mlp.cu) */
void xmi_surrogate_free(void *sg);
/* multiplies the solid-angle factors of the queued estimator events of the
 * configurations that use the network (dev_bundles[n_cfg] on the device,
 * indexed by the events' configuration) by its solid angle; events in
 * flagged cells go through fb_list (cap entries, *fb_count zeroed by the
 * caller) to the integrator; all on stream */
int xmi_surrogate_apply(const void *sg, int precision, const void *dev_bundles, int n_cfg, void *events,
                        const unsigned long long *count, long long cap, unsigned long long *fallbacks, int *fb_list,
                        unsigned long long *fb_count, int *err, void *stream);
/* The grid path's off-grid solid angles: the queued events that the step
 * kernel flagged (sa_pending) get the 5000-sample integral at their (r,
 * theta), one warp per event, draw for draw as the serial integral; fb_list
 * (cap entries, *fb_count zeroed by the caller); on stream */
int xmi_solid_angle_deferred(int precision, const void *dev_bundles, int n_cfg, void *events,
                             const unsigned long long *count, long long cap, int *fb_list,
                             unsigned long long *fb_count, void *stream);

#ifdef __cplusplus
}
#endif
#endif
