/*
 * C-ABI of the GB300 XRF Monte Carlo engine (libxmimsim_gb300.so).
 *
 * Drop-in for the simulation call of XMI-MSIM 8.1: the entry points keep the
 * reference's names, argument meaning, output layouts and ownership rules,
 * so a caller written against the reference (bin/xmimsim.c:249-669,
 * tests/libxmimsim-test.c:182-270) links against this library instead.
 * Each declaration cites the reference interface it replaces.
 *
 * Conventions kept from the reference:
 *  - int-returning calls return 1 on success and 0 on failure; the library
 *    never calls exit() -- the reason of the last failure is available from
 *    xmi_gpu_last_error();
 *  - output arrays are allocated by the callee and released with xmi_free();
 *  - channels[(N+1)*nchannels]: row i (i = 0..N) is the spectrum after at
 *    most i interactions (cumulative over orders), times live_time;
 *  - histories[100*385*N]: element (Z, line, k) at ((Z-1)*385 + line-1)*N + k-1,
 *    line = -xraylib macro (1..383), 384 Rayleigh, 385 Compton.
 */
#ifndef XMIMSIM_GB300_H
#define XMIMSIM_GB300_H

#include <stddef.h>

#include "xmi_data_structs.h"

#ifdef __cplusplus
extern "C" {
#endif

/* opaque handles (reference: void* to Fortran TYPEs, include/xmi_data.h:29
 * and include/xmi_aux.h) */
typedef struct xmi_input_handle *xmi_inputFPtr;
typedef struct xmi_tables_handle *xmi_hdf5FPtr;

/* GPU-specific settings, kept out of xmi_main_options so that struct stays
 * layout-identical to the reference */
typedef struct {
  int precision;            /* 0: FP64 transport; 1: FP32 transport, FP64 tallies */
  int use_surrogate;        /* 1: solid angle from the MLP surrogate (VR only) */
  double surrogate_tolerance; /* fall back to the grid where held-out error exceeds this */
  int threads_per_block;    /* 0: default */
  int blocks_per_sm;        /* 0: default */
  unsigned long long seed;  /* Philox key; 0: fixed default key (0x5EED0001) */
  int solid_angle_stream;   /* 0: Philox grid draws; 1: the OpenCL backend's Threefry
                               stream (src/xmi_kernels.cl:226-227), for point-by-point
                               comparison with that kernel */
  long long queue_events;   /* estimator events per chunk (device queue size); 0: default 2^25 */
  int grid_nr, grid_nt;     /* solid-angle grid points along r and theta; 0: the reference's 1024 */
  int overlap_chunks;       /* 1: the transport of the next chunk runs beside the sort, solid
                               angles and estimator of the current one (second stream, two
                               event queues); 0: the phases of consecutive chunks run one after
                               another (faster on GB300: both phases wait on table gathers
                               through the same caches) */
  int estimator_blocks_per_sm; /* estimator blocks resident per SM; 0: as many as fit */
} xmi_gpu_options;

/* ---- atomic data source of the host tabulator ----
 * Every cross section and atomic parameter the tabulator reads (the values
 * the reference takes from xraylib: src/xmi_aux_f.F90:22, src/xmi_data_f.F90
 * :880-1481, src/xmi_variance_reduction.F90:344-709, src/xmi_detector_f.F90,
 * src/xmi_ebel.F90) comes through this table; the entries have xraylib's
 * names and argument order.  Index conventions: shell 0 = K, 1..3 = L1..L3,
 * 4..8 = M1..M5 (xraylib's K_SHELL..M5_SHELL); line = the positive index
 * 1..383 of the history layout, i.e. minus xraylib's line macro (an xraylib
 * adapter calls LineEnergy(Z, -line)); CosKronTransProb trans 0..13 in
 * xraylib's order FL12, FL13, FLP13, FL23, FM12 .. FM45; AugerRate trans
 * 0..644 in xraylib's order (K_L1L1 = 0 .. L3_M5Q3 = 644); AugerVacancies(Z,
 * s, t) = expected new vacancies in shell t per non-radiative decay of shell
 * s (an xraylib adapter sums AugerRate over the transitions of s weighted by
 * the vacancies each leaves in t).  prepare(Z) may be NULL; it is called once
 * per element before the others, from one thread.  The default table is the
 * stand-in model compiled into the library (xrlite: xraylib and its data are
 * absent on the build and GPU machines).  No counterpart in the reference,
 * which links xraylib directly. */
typedef struct {
  const char *name;
  double (*AtomicWeight)(int Z);
  double (*EdgeEnergy)(int Z, int shell);
  double (*ElectronConfig)(int Z, int shell);
  double (*LineEnergy)(int Z, int line);
  double (*RadRate)(int Z, int line);
  double (*FluorYield)(int Z, int shell);
  double (*AugerYield)(int Z, int shell);
  double (*CosKronTransProb)(int Z, int trans);
  double (*AugerRate)(int Z, int trans);
  double (*AugerVacancies)(int Z, int shell, int to_shell);
  double (*CS_Total_Kissel)(int Z, double E);
  double (*CS_Photo_Total)(int Z, double E);
  double (*CS_Photo_Partial)(int Z, int shell, double E);
  double (*CS_Rayl)(int Z, double E);
  double (*CS_Compt)(int Z, double E);
  double (*FF_Rayl)(int Z, double q);
  double (*SF_Compt)(int Z, double q);
  double (*DCS_Rayl)(int Z, double E, double theta);
  double (*DCS_Compt)(int Z, double E, double theta);
  double (*ComptonProfile)(int Z, double pz);
  void (*prepare)(int Z);
} xmi_atomic_data;
/* Installs a data source (copied; NULL restores the default).  Only before
 * the first table of the process is built: returns 0 with an error once
 * tables (cached per element and shared by every bundle) exist, or when an
 * entry other than prepare is NULL. */
int xmi_set_atomic_data(const xmi_atomic_data *data);
/* the table in use */
const xmi_atomic_data *xmi_get_atomic_data(void);

/* ---- data model helpers (reference src/xmi_data_structs.c) ---- */
xmi_input *xmi_input_init_empty(void);                 /* src/xmi_data_structs.c:551 */
void xmi_input_free(xmi_input *input);                 /* include/xmi_data_structs.h:331 */
void xmi_input_copy(xmi_input *A, xmi_input **B);      /* include/xmi_data_structs.h:332 */
xmi_main_options *xmi_main_options_new(void);          /* include/xmi_data_structs.h:497 */
void xmi_main_options_free(xmi_main_options *options); /* include/xmi_data_structs.h:498 */
void xmi_free(void *ptr);                              /* src/xmi_aux.c (g_free wrapper) */
const char *xmi_gpu_last_error(void);
void xmi_gpu_default_options(xmi_gpu_options *gpu);

/* ---- initialisation chain (bin/xmimsim.c:275-294) ---- */
int xmi_input_C2F(xmi_input *input, xmi_inputFPtr *inputFPtr);   /* src/xmi_aux_f.F90:782 */
void xmi_free_input_F(xmi_inputFPtr *inputFPtr);                 /* src/xmi_aux_f.F90:1027 */
int xmi_init_input(xmi_inputFPtr *inputFPtr);                    /* src/xmi_main.F90:1741 */
int xmi_init_input_escape_ratios(xmi_inputFPtr *inputFPtr);      /* src/xmi_main.F90:1687 */
/* hdf5_file is accepted for signature compatibility; the tables come from the
 * host tabulator (there is no xraylib data file on the target machines) */
int xmi_init_from_hdf5(char *hdf5_file, xmi_inputFPtr inputFPtr,
                       xmi_hdf5FPtr *hdf5FPtr, xmi_main_options *options); /* include/xmi_data.h:45 */
int xmi_update_input_from_hdf5(xmi_inputFPtr inputFPtr, xmi_hdf5FPtr hdf5FPtr); /* include/xmi_data.h:50 */
void xmi_free_hdf5_F(xmi_hdf5FPtr *hdf5FPtr);                    /* include/xmi_data.h:48 */
int xmi_gpu_set_options(xmi_inputFPtr inputFPtr, const xmi_gpu_options *gpu);

/* ---- output: unpacking and .xmso files ---- */
/* GLib's error type, declared here only so that a caller's GError ** passes
 * through; the library never sets it (the reason of a failure is available
 * from xmi_gpu_last_error()) */
typedef struct _GError GError;
/* the raw outputs of xmi_main_msim (channels_unconv[(N+1)*nchannels],
 * histories [100*385*N]) and the convolved spectra per order unpacked into
 * an xmi_output: per element of the sample with counts, per line with
 * counts, per interaction number with counts (src/xmi_data_structs.c
 * :1371-1518).  The input is copied; free with xmi_output_free. */
xmi_output *xmi_output_raw2struct(xmi_input *input, double *brute_history, double *var_red_history,
                                  double **channels_conv, double *channels_unconv, char *inputfile,
                                  int use_zero_interactions); /* include/xmi_data_structs.h:574 */
void xmi_output_free(xmi_output *output);                   /* include/xmi_data_structs.h:406 */
/* writes the output as an .xmso document (xmimsim-1.0 DTD), numbers with 17
 * significant digits, without the GUI's SVG graphs (src/xmi_xml.c:1638) */
int xmi_output_write_to_xml_file(xmi_output *output, const char *xmsofile, GError **error);

/* ---- solid-angle grid (include/xmi_solid_angle.h:39) ---- */
extern long hits_per_single; /* samples per grid point, src/xmi_solid_angle_f.F90:43-44 */
void xmi_solid_angle_calculation(xmi_inputFPtr inputFPtr, xmi_solid_angle **solid_angle,
                                 char *input_string, xmi_main_options *options);
/* backend-plugin symbol with the XmiSolidAngleCalculation typedef of
 * src/xmi_solid_angle.c:50 (the slot the OpenCL/Metal plugins fill) */
int xmi_solid_angle_calculation_cuda(xmi_inputFPtr inputFPtr, xmi_solid_angle **solid_angle,
                                     char *input_string, xmi_main_options *options);
void xmi_free_solid_angle(xmi_solid_angle *solid_angle);          /* include/xmi_solid_angle.h:52 */

/* ---- transport (include/xmi_main.h:29) ---- */
int xmi_main_msim(xmi_inputFPtr inputFPtr, xmi_hdf5FPtr hdf5FPtr, int n_mpi_hosts,
                  double **channels, xmi_main_options *options, double **brute_history,
                  double **var_red_history, xmi_solid_angle *solid_angles);

/* ---- detector response (include/xmi_main.h:31-37) ---- */
void xmi_detector_convolute_spectrum(xmi_inputFPtr inputFPtr, double *channels_noconv,
                                     double **channels_conv, xmi_main_options *options,
                                     xmi_escape_ratios *escape_ratios, int n_interactions);
void xmi_detector_convolute_all(xmi_inputFPtr inputFPtr, double **channels_noconv,
                                double **channels_conv, double *brute_history,
                                double *var_red_history, xmi_main_options *options,
                                xmi_escape_ratios *escape_ratios, int n_interactions_all,
                                int zero_interaction);
void xmi_detector_convolute_history(xmi_inputFPtr inputFPtr, double *history,
                                    xmi_main_options *options);
/* custom-detector-response plugin symbol (typedef XmiDetectorConvoluteAll,
 * include/xmi_main.h:37; loaded by bin/xmimsim.c:505-526) */
void xmi_detector_convolute_all_custom(xmi_inputFPtr inputFPtr, double **channels_noconv,
                                       double **channels_conv, double *brute_history,
                                       double *var_red_history, xmi_main_options *options,
                                       xmi_escape_ratios *escape_ratios, int n_interactions_all,
                                       int zero_interaction);

/* Allocation-free detector convolution.  No counterpart in the reference.
 * For callers that cannot allocate device memory when they convolve (a
 * real-time acquisition or fitting loop under a device-memory budget fixed up
 * front, an application whose GPU memory belongs to another allocator): same
 * result as xmi_detector_convolute_spectrum with use_escape_peaks = 0 and
 * use_sum_peaks = 0 (channel absorption, Gaussian + tail convolution, optional
 * Poisson noise), written into the caller's channels_conv[nchannels].
 * It calls no cudaMalloc/cudaFree: the device scratch is a fixed array of
 * 3 x 16384 doubles (384 KiB) kept on every GPU that loads the library until
 * exit.  Returns 0 with an error for nchannels > 16384 or when escape peaks
 * or pile-up are requested.  The first call on a device looks up the
 * scratch address for that device; make it before any stream capture.  That
 * address is cached for the life of the process: after a cudaDeviceReset()
 * of the device it is stale, so do not call this entry point on a device
 * that has been reset.  All calls share the scratch, which keeps the last
 * call's contents; calls that overlap on the GPU (concurrent host threads)
 * race. */
int xmi_detector_convolute_spectrum_noalloc(xmi_inputFPtr inputFPtr, const double *channels_noconv,
                                            double *channels_conv, xmi_main_options *options);

/* Batched transport.  No counterpart in the reference, which simulates one
 * configuration per call (a quantification front-end such as
 * bin/xmimsim-pymca.c:597-620 loops over xmi_main_msim).  Runs n prepared
 * configurations (each handle built by the initialisation chain above, all
 * with the same xmi_gpu_options precision) in one chunked launch sequence,
 * captured as one CUDA graph: their photons share the transport, sort and
 * estimator kernels.  Configurations with xmi_gpu_options.use_surrogate = 1
 * and a trained surrogate take their solid angles from it (all such
 * configurations of one call must share one network, see
 * xmi_gpu_share_surrogate); the others from their grid.  Outputs per configuration as xmi_main_msim's, in
 * channels[c], brute_histories[c], var_red_histories[c] (n_mpi_hosts = 1).
 * Calls are serialised within a process. */
int xmi_main_msim_batch(int n, xmi_inputFPtr *inputFPtrs, xmi_hdf5FPtr *hdf5FPtrs, xmi_main_options **options,
                        xmi_solid_angle **solid_angles, double **channels, double **brute_histories,
                        double **var_red_histories);

/* Autotuner of the batched call (no counterpart in the reference): times
 * xmi_main_msim_batch on `share` of every configuration's photons (the
 * first 1/R of each source item, R = round(1 / share)) for the candidate
 * launch shapes of the wavefront kernels -- threads per block 64/128 x
 * blocks per SM 4/8/12/16 -- and then the estimator queue sizes 2^23/2^24/2^25
 * events, keeps the fastest by device time and writes it into every
 * configuration's xmi_gpu_options.  report[4]: threads per block, blocks
 * per SM, queue events, device ms of the best trial. */
int xmi_gpu_autotune_batch(int n, xmi_inputFPtr *inputFPtrs, xmi_hdf5FPtr *hdf5FPtrs, xmi_main_options **options,
                           xmi_solid_angle **solid_angles, double share, double *report);

/* ---- solid-angle surrogate network (no counterpart in the reference) ----
 * A 3 -> 4 x 128 (SiLU) -> 1 network, BF16 weights and FP32 accumulation on
 * the tensor cores, maps a point's (log r, axial distance, cos angle) to the
 * log of its collimated detector solid angle.  xmi_gpu_build_surrogate trains
 * it for an initialised input: n_train points uniform over the sample volume
 * (the slab of the layers within 2 cm of the beam axis), targets from the
 * engine's own integrator (hits_train cone samples each, FP32), Adam for
 * `epochs` passes; then checks it on 16 x 1024 further points against the
 * FP64 integrator (two independent integrations of hits_check / 2 samples
 * per point, whose difference measures the reference values' own noise) and
 * flags the cells of a 32 x 32 partition of the grid's (log r, theta) box
 * whose RMS relative error, less that noise, exceeds
 * xmi_gpu_options.surrogate_tolerance (and the cells no point reached):
 * there the integrator keeps serving.  report[6]: median relative error of
 * the checking points, largest error in an unflagged cell, share of checking
 * points in flagged cells (the expected fallback rate), final training loss,
 * seconds, number of cells.  With xmi_gpu_options.use_surrogate = 1, xmi_main_msim
 * then needs no solid-angle grid. */
int xmi_gpu_build_surrogate(xmi_inputFPtr inputFPtr, int n_train, int hits_train, int epochs, int hits_check,
                            double *report);
int xmi_gpu_surrogate_report(xmi_inputFPtr inputFPtr, double *report);
/* The solid angle the transport would take from the input's trained
 * surrogate at n points (r, theta of the grid's coordinates), as it serves
 * them: omega[i], and source[i] = 0 network, 1 tabulated integrator of a
 * flagged cell, 2 outside the checked region (the transport integrates such
 * a point itself; omega[i] is then set to -1), 3 below the grid's lowest
 * theta (omega 0).  No counterpart in the reference (it has no surrogate);
 * used to validate the network on held-out points. */
int xmi_gpu_surrogate_eval(xmi_inputFPtr inputFPtr, int n, const double *r, const double *theta, double *omega,
                           int *source);
/* The engine's solid-angle integrator (the grid's per-point Monte Carlo of
 * src/xmi_solid_angle_f.F90:432-710) at n arbitrary points with `hits`
 * samples each, FP64 (precision 0) or FP32 (1), Philox key `seed`: point i
 * draws from stream (seed, i, 0xF1000000).  No counterpart in the reference
 * as an entry point; the values the surrogate is checked against. */
int xmi_gpu_solid_angle_points(xmi_inputFPtr inputFPtr, int n, const double *r, const double *theta, int hits,
                               int precision, unsigned long long seed, double *omega);
/* the same training and check on caller-given points (r, theta) of the
 * solid-angle grid's frame -- typically the points where the estimator of a
 * pilot run queried solid angles (xmi_gpu_sample_event_points): the first
 * 16 x 1024 points (after a fixed shuffle) check, the rest train */
int xmi_gpu_build_surrogate_points(xmi_inputFPtr inputFPtr, int n_points, const double *r, const double *theta,
                                   int hits_train, int epochs, int hits_check, double *report);
/* Pilot run for surrogate training: runs the transport of a prepared
 * configuration on `share` of its photons (the first 1/R of each source item,
 * R = round(1 / share)) and returns the (r, theta) of about max_points of the
 * estimator's solid-angle queries, drawn uniformly over all of them (two
 * passes: count, then a hash-selected share).  Needs variance reduction; no
 * grid or network is used (the pilot's tallies are discarded). */
int xmi_gpu_sample_event_points(xmi_inputFPtr inputFPtr, xmi_hdf5FPtr hdf5FPtr, xmi_main_options *options,
                                double share, int max_points, double *r, double *theta, int *n_points);
/* lets input `to` use the network trained for input `from` (same detector
 * radius and collimator required; points outside the network's checked box
 * are served by the integrator) -- one training serves a batch of samples
 * measured with one detector */
int xmi_gpu_share_surrogate(xmi_inputFPtr from, xmi_inputFPtr to);
/* device time of the surrogate phase of the last xmi_main_msim and the
 * number of estimator events served by the integrator fallback */
int xmi_gpu_last_surrogate(double *surrogate_ms, long long *fallbacks);
/* bytes copied host -> device and device -> host by the last xmi_main_msim
 * or xmi_main_msim_batch call (source items, run descriptors, a changed
 * solid-angle grid; tallies and status words) */
int xmi_gpu_last_transfers(long long *h2d_bytes, long long *d2h_bytes);
/* the network alone, for tests of the tensor-core kernels: parameter count,
 * outputs, gradient of the mean squared error, Adam training */
int xmi_mlp_nparam(void);
int xmi_gpu_mlp_forward(const float *theta, int n, const float *features, float *out);
int xmi_gpu_mlp_grad(const float *theta, int n, const float *features, const float *targets, float *grad,
                     double *loss);
int xmi_gpu_mlp_train(float *theta, int n, const float *features, const float *targets, int epochs, float lr,
                      double *loss_per_epoch);

/* ---- X-ray tube spectra (include/xmi_ebel.h:26-33) ----
 * Ebel's model of the tube's continuum and K/L lines (src/xmi_ebel.F90:115-521),
 * window and filter attenuation, optional transmission-efficiency profile
 * (natural cubic spline through the given points).  Allocates
 * *ebel_spectrum (free with xmi_free on its arrays and itself). */
int xmi_tube_ebel(xmi_layer *tube_anode, xmi_layer *tube_window, xmi_layer *tube_filter, double tube_voltage,
                  double tube_current, double tube_angle_electron, double tube_angle_xray, double tube_delta_energy,
                  double tube_solid_angle, int tube_transmission, size_t tube_nefficiencies, double *tube_energies,
                  double *tube_efficiencies, xmi_excitation **ebel_spectrum);
/* include/xmi_transmission_efficiency.h:27; the reference's GError is the
 * 0 return with the reason in xmi_gpu_last_error() */
int xmi_transmission_efficiency_read(const char *filename, size_t *nefficiencies, double **energies,
                                     double **efficiencies);

/* ---- escape ratios (include/xmi_detector.h:55-57) ---- */
xmi_escape_ratios_options xmi_get_default_escape_ratios_options(void);
void xmi_escape_ratios_calculation(xmi_input *inputPtr, xmi_escape_ratios **escape_ratios,
                                   char *input_string, char *hdf5_file,
                                   xmi_main_options *options, xmi_escape_ratios_options ero);
void xmi_free_escape_ratios(xmi_escape_ratios *escape_ratios);   /* include/xmi_detector.h:71 */

/* ---- introspection used by the test-suite and benchmark ---- */
/* the escape-mode input and tables xmi_escape_ratios_calculation builds for
 * a detector (crystal layers as the sample, src/xmi_detector.c:91-141) */
int xmi_gpu_escape_tables(xmi_input *inputPtr, xmi_main_options *options, xmi_inputFPtr *inputFPtr,
                          xmi_hdf5FPtr *hdf5FPtr);
struct xmi_bundle_s; /* see xmimsim_bundle.h */
const void *xmi_gpu_bundle(xmi_hdf5FPtr hdf5FPtr);
/* prepares the run-dependent part of the bundle (source items, options)
 * exactly as xmi_main_msim would, without running it */
int xmi_gpu_prepare_run(xmi_inputFPtr inputFPtr, xmi_hdf5FPtr hdf5FPtr,
                        xmi_main_options *options, int n_mpi_hosts,
                        xmi_solid_angle *solid_angles);
/* Replicas: this process simulates photons [r*n/R, (r+1)*n/R) of every source
 * item (r = replica, R = n_replicas), with the weights of the full budget, so
 * the element-wise sum of the outputs of all R replicas is the single-process
 * result.  Replaces the reference's MPI photon split (src/xmi_main.F90:314,574;
 * bin/xmimsim.c:396-413). */
int xmi_gpu_set_replica(xmi_hdf5FPtr hdf5FPtr, int replica, int n_replicas);
/* device time (ms, CUDA events) and kernel launches of the last call */
int xmi_gpu_last_timing(double *transport_ms, double *total_ms, int *launches);
/* device time of the phases of the last xmi_main_msim (transport kernel,
 * sort of the estimator events, estimator kernel) and the number of
 * estimator events */
int xmi_gpu_last_phases(double *transport_kernel_ms, double *sort_ms, double *estimator_ms, long long *events);
/* how the last xmi_main_msim_batch ran its chunk sequence: -1 no graph, 0 a
 * graph instantiated for this call, 1 the previous call's executable graph
 * updated in place (same shape), 100 + the cudaGraphExecUpdateResult when the
 * previous graph could not take this call's sequence (a new one was
 * instantiated) */
int xmi_gpu_last_graph(int *updated);
/* the device functions of the per-shell Compton kinematics
 * (xmi_get_qimax / xmi_get_energy_from_q, src/xmi_aux_f.F90:1951-2074) in
 * their FP32 and FP64 forms on n points (energy, binding energy, theta, Q):
 * out[6 i ..] = qimax FP32, qimax FP64, scattered energy FP32, FP64, and the
 * FP32 / FP64 "no root" flags */
int xmi_gpu_compton_kinematics(int n, const double *energy, const double *binding, const double *theta,
                               const double *q, double *out);

#ifdef __cplusplus
}
#endif
#endif
