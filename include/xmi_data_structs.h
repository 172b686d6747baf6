/*
 * Input/option/output data model of the XRF Monte Carlo engine.
 *
 * The struct layouts are kept field-for-field identical to the reference's
 * C data model (include/xmi_data_structs.h:40-495 of XMI-MSIM 8.1) so that a
 * caller compiled against the reference headers can hand its xmi_input and
 * xmi_main_options to this library unchanged.  Only the layouts are shared;
 * every function behind them is this project's own.
 */
#ifndef XMIMSIM_GB300_DATA_STRUCTS_H
#define XMIMSIM_GB300_DATA_STRUCTS_H

#ifdef __cplusplus
extern "C" {
#endif

/* reference include/xmi_data_structs.h:40-47 */
typedef struct _xmi_general {
  float version;
  char *outputfile;
  long n_photons_interval;
  long n_photons_line;
  int n_interactions_trajectory;
  char *comments;
} xmi_general;

/* reference include/xmi_data_structs.h:64-70 */
typedef struct _xmi_layer {
  int n_elements;
  int *Z;
  double *weight;
  double density;   /* g/cm3 */
  double thickness; /* cm */
} xmi_layer;

/* reference include/xmi_data_structs.h:87-91 (reference_layer is 1-based) */
typedef struct _xmi_composition {
  int n_layers;
  xmi_layer *layers;
  int reference_layer;
} xmi_composition;

/* reference include/xmi_data_structs.h:117-128 */
typedef struct _xmi_geometry {
  double d_sample_source;
  double n_sample_orientation[3];
  double p_detector_window[3];
  double n_detector_orientation[3];
  double area_detector;
  double collimator_height;
  double collimator_diameter;
  double d_source_slit;
  double slit_size_x;
  double slit_size_y;
} xmi_geometry;

/* reference include/xmi_data_structs.h:144-148 */
typedef enum {
  XMI_ENERGY_DISCRETE_DISTRIBUTION_MONOCHROMATIC = 0,
  XMI_ENERGY_DISCRETE_DISTRIBUTION_GAUSSIAN = 1,
  XMI_ENERGY_DISCRETE_DISTRIBUTION_LORENTZIAN = 2
} XmiEnergyDiscreteDistribution;

/* reference include/xmi_data_structs.h:166-176 */
typedef struct _xmi_energy_discrete {
  double energy;
  double horizontal_intensity;
  double vertical_intensity;
  double sigma_x;
  double sigma_xp;
  double sigma_y;
  double sigma_yp;
  XmiEnergyDiscreteDistribution distribution_type;
  double scale_parameter;
} xmi_energy_discrete;

/* reference include/xmi_data_structs.h:197-205 */
typedef struct _xmi_energy_continuous {
  double energy;
  double horizontal_intensity; /* photons/s/keV */
  double vertical_intensity;
  double sigma_x;
  double sigma_xp;
  double sigma_y;
  double sigma_yp;
} xmi_energy_continuous;

/* reference include/xmi_data_structs.h:226-231 */
typedef struct _xmi_excitation {
  int n_discrete;
  xmi_energy_discrete *discrete;
  int n_continuous;
  xmi_energy_continuous *continuous;
} xmi_excitation;

/* reference include/xmi_data_structs.h:253-258 */
typedef struct _xmi_absorbers {
  int n_exc_layers;
  xmi_layer *exc_layers;
  int n_det_layers;
  xmi_layer *det_layers;
} xmi_absorbers;

/* reference include/xmi_data_structs.h:278-282 */
typedef enum {
  XMI_DETECTOR_CONVOLUTION_PROFILE_SILI = 0,
  XMI_DETECTOR_CONVOLUTION_PROFILE_GE = 1,
  XMI_DETECTOR_CONVOLUTION_PROFILE_SI_SDD = 2
} XmiDetectorConvolutionProfile;

/* reference include/xmi_data_structs.h:301-312 */
typedef struct _xmi_detector {
  XmiDetectorConvolutionProfile detector_type;
  double live_time;
  double pulse_width;
  double gain;
  double zero;
  double fano;
  double noise;
  int nchannels;
  int n_crystal_layers;
  xmi_layer *crystal_layers;
} xmi_detector;

/* reference include/xmi_data_structs.h:331-338 */
typedef struct _xmi_input {
  xmi_general *general;
  xmi_composition *composition;
  xmi_geometry *geometry;
  xmi_excitation *excitation;
  xmi_absorbers *absorbers;
  xmi_detector *detector;
} xmi_input;

/* reference include/xmi_data_structs.h:479-495; defaults of
 * src/xmi_data_structs.c:2531-2547 are returned by xmi_main_options_new() */
typedef struct _xmi_main_options {
  int use_M_lines;
  int use_cascade_auger;
  int use_cascade_radiative;
  int use_variance_reduction;
  int use_sum_peaks;
  int use_escape_peaks;
  int escape_ratios_mode;
  int verbose;
  int use_poisson;
  int use_gpu;
  int omp_num_threads;
  int extra_verbose;
  char *custom_detector_response;
  int use_advanced_compton;
  int use_default_seeds;
} xmi_main_options;

/* reference include/xmi_solid_angle.h:28-35; solid_angles is stored
 * [theta][r] (r fastest), i.e. the Fortran (r, theta) array */
typedef struct _xmi_solid_angle {
  double *solid_angles;
  long int grid_dims_r_n;
  long int grid_dims_theta_n;
  double *grid_dims_r_vals;
  double *grid_dims_theta_vals;
  char *xmi_input_string;
} xmi_solid_angle;

/* reference include/xmi_detector.h:27-39.  fluo_escape_ratios is the
 * Fortran (n_elements, 109, n_fluo_input_energies) array; compton_escape_ratios
 * the Fortran (n_compton_input_energies, n_compton_output_energies) array. */
typedef struct _xmi_escape_ratios {
  int n_elements;
  int n_fluo_input_energies;
  int n_compton_input_energies;
  int n_compton_output_energies;
  int *Z;
  double *fluo_escape_ratios;
  double *fluo_escape_input_energies;
  double *compton_escape_ratios;
  double *compton_escape_input_energies;
  double *compton_escape_output_energies;
  char *xmi_input_string;
} xmi_escape_ratios;

/* reference include/xmi_detector.h:41-50 */
typedef struct _xmi_escape_ratios_options {
  long n_input_energies;          /* default 1990 */
  long n_compton_output_energies; /* default 1999 */
  long n_photons;                 /* default 500000 */
  double input_energy_min;        /* default 1.0 keV */
  double input_energy_delta;      /* default 0.1 keV */
  double compton_output_energy_min;   /* default 0.1 keV */
  double compton_output_energy_delta; /* default 0.1 keV */
} xmi_escape_ratios_options;

/* reference include/xmi_data_structs.h:337-399: the unpacked output of one
 * simulation (xmi_output_raw2struct) -- spectra per interaction order and
 * the histories per element, line and interaction number */
typedef struct _xmi_counts {
  double counts;
  int interaction_number;
} xmi_counts;

typedef struct _xmi_fluorescence_line {
  char *line_type;
  double energy;
  double total_counts;
  int n_interactions;
  xmi_counts *interactions;
} xmi_fluorescence_line;

typedef struct _xmi_fluorescence_line_counts {
  int atomic_number;
  double total_counts;
  int n_lines;
  xmi_fluorescence_line *lines;
} xmi_fluorescence_line_counts;

typedef struct _xmi_output {
  float version;
  char *inputfile;
  char *outputfile;
  xmi_input *input;
  xmi_fluorescence_line_counts *brute_force_history;
  xmi_fluorescence_line_counts *var_red_history;
  int nbrute_force_history;
  int nvar_red_history;
  double **channels_conv;
  double **channels_unconv;
  int ninteractions;
  int use_zero_interactions;
} xmi_output;

#ifdef __cplusplus
}
#endif
#endif
