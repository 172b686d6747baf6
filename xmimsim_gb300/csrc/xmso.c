/*
 * The output side of the library surface: unpacking the raw outputs of
 * xmi_main_msim (and of the detector response) into an xmi_output
 * (xmi_output_raw2struct, src/xmi_data_structs.c:1371-1518) and writing it as
 * an .xmso file (xmi_output_write_to_xml_file, src/xmi_xml.c:1638-1675 with
 * the body of :1453-1628 and the input section of :1680-1850), without
 * libxml2 or GLib: the document is written with stdio in the element order,
 * names and attributes of the xmimsim-1.0 DTD that the reference writes.
 *
 * Kept from the reference because readers depend on them: the element and
 * attribute names and order; elements with a history, and within them lines,
 * listed only when their counts are non-zero (elements in ascending Z, lines
 * in index order, interaction numbers where counts > 0); spectra per order
 * from 1 (0 too with use_zero_interactions); channel energies gain * i +
 * zero; weight fractions in percent.  Different on purpose: numbers carry 17
 * significant digits (the reference prints "%g", 6 digits), so that a file
 * read back gives the same doubles; the SVG preview graphs of the GUI
 * (:1576-1625) are not written.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "xmi_internal.h"
#include "xrlite.h"

/* the version the files claim: the format of XMI-MSIM 8.1 */
#define XMSO_VERSION "8.1"

static const char *const kSymbols[] = {
    "H",  "He", "Li", "Be", "B",  "C",  "N",  "O",  "F",  "Ne", "Na", "Mg", "Al", "Si", "P",  "S",  "Cl",
    "Ar", "K",  "Ca", "Sc", "Ti", "V",  "Cr", "Mn", "Fe", "Co", "Ni", "Cu", "Zn", "Ga", "Ge", "As", "Se",
    "Br", "Kr", "Rb", "Sr", "Y",  "Zr", "Nb", "Mo", "Tc", "Ru", "Rh", "Pd", "Ag", "Cd", "In", "Sn", "Sb",
    "Te", "I",  "Xe", "Cs", "Ba", "La", "Ce", "Pr", "Nd", "Pm", "Sm", "Eu", "Gd", "Tb", "Dy", "Ho", "Er",
    "Tm", "Yb", "Lu", "Hf", "Ta", "W",  "Re", "Os", "Ir", "Pt", "Au", "Hg", "Tl", "Pb", "Bi", "Po", "At",
    "Rn", "Fr", "Ra", "Ac", "Th", "Pa", "U",  "Np", "Pu", "Am", "Cm", "Bk", "Cf", "Es", "Fm"};

static char *dup_str(const char *s) {
  char *d;
  size_t n;
  if (!s) return NULL;
  n = strlen(s) + 1;
  d = (char *)malloc(n);
  if (d) memcpy(d, s, n);
  return d;
}

static int cmp_int(const void *a, const void *b) { return *(const int *)a - *(const int *)b; }

/* index of history entry (Z, line, k) in the flat layout of xmi_main_msim */
static size_t hpos(int Z, int line, int k, int N) { return ((size_t)(Z - 1) * 385 + (line - 1)) * N + (k - 1); }

/* the per-element history of one raw table (src/xmi_data_structs.c:1422-1459) */
static xmi_fluorescence_line_counts *unpack_history(const double *h, const int *uniqZ, int nuniq, int N, int *n_out) {
  xmi_fluorescence_line_counts *out = NULL;
  int n = 0, i, j, k;
  for (i = 0; i < nuniq; i++) {
    const int Z = uniqZ[i];
    double zsum = 0.0;
    xmi_fluorescence_line_counts *fc;
    if (Z < 1 || Z > 100) continue;
    for (j = 1; j <= 383; j++)
      for (k = 1; k <= N; k++) zsum += h[hpos(Z, j, k, N)];
    if (zsum == 0.0) continue;
    out = (xmi_fluorescence_line_counts *)realloc(out, sizeof(*out) * (size_t)(n + 1));
    fc = &out[n++];
    fc->atomic_number = Z;
    fc->total_counts = zsum;
    fc->n_lines = 0;
    fc->lines = NULL;
    for (j = 1; j <= 383; j++) {
      double lsum = 0.0;
      xmi_fluorescence_line *fl;
      for (k = 1; k <= N; k++) lsum += h[hpos(Z, j, k, N)];
      if (lsum == 0.0) continue;
      fc->lines = (xmi_fluorescence_line *)realloc(fc->lines, sizeof(*fc->lines) * (size_t)(fc->n_lines + 1));
      fl = &fc->lines[fc->n_lines++];
      fl->line_type = dup_str(xrl_line_name(j));
      fl->energy = XD->LineEnergy(Z, j);
      fl->total_counts = lsum;
      fl->n_interactions = 0;
      fl->interactions = NULL;
      for (k = 1; k <= N; k++) {
        const double c = h[hpos(Z, j, k, N)];
        if (c <= 0.0) continue;
        fl->interactions = (xmi_counts *)realloc(fl->interactions, sizeof(xmi_counts) * (size_t)(fl->n_interactions + 1));
        fl->interactions[fl->n_interactions].counts = c;
        fl->interactions[fl->n_interactions].interaction_number = k;
        fl->n_interactions++;
      }
    }
  }
  *n_out = n;
  return out;
}

/* reference src/xmi_data_structs.c:1371-1518 */
xmi_output *xmi_output_raw2struct(xmi_input *input, double *brute_history, double *var_red_history,
                                  double **channels_conv, double *channels_unconv, char *inputfile,
                                  int use_zero_interactions) {
  xmi_output *out;
  int N, nch, i, j, k, nuniq = 0, cap;
  int *uniqZ;
  if (!input || !input->general || !input->detector || !input->composition || !brute_history || !channels_unconv) {
    xmi_set_error("xmi_output_raw2struct: NULL argument");
    return NULL;
  }
  N = input->general->n_interactions_trajectory;
  nch = input->detector->nchannels;
  out = (xmi_output *)calloc(1, sizeof(xmi_output));
  out->version = 8.1f;
  xmi_input_copy(input, &out->input);
  out->inputfile = dup_str(inputfile ? inputfile : "");
  out->outputfile = dup_str(input->general->outputfile ? input->general->outputfile : "");
  out->use_zero_interactions = use_zero_interactions;
  out->ninteractions = N;
  out->channels_conv = (double **)calloc((size_t)N + 1, sizeof(double *));
  out->channels_unconv = (double **)calloc((size_t)N + 1, sizeof(double *));
  for (i = 0; i <= N; i++) {
    out->channels_unconv[i] = (double *)calloc((size_t)nch, sizeof(double));
    out->channels_conv[i] = (double *)calloc((size_t)nch, sizeof(double));
    if (i == 0 && use_zero_interactions == 0) continue;
    for (j = 0; j < nch; j++) {
      out->channels_unconv[i][j] = channels_unconv[(size_t)nch * i + j];
      out->channels_conv[i][j] = channels_conv && channels_conv[i] ? channels_conv[i][j] : 0.0;
    }
  }
  /* the sample's distinct elements in ascending Z */
  cap = 0;
  for (i = 0; i < input->composition->n_layers; i++) cap += input->composition->layers[i].n_elements;
  uniqZ = (int *)malloc(sizeof(int) * (size_t)(cap > 0 ? cap : 1));
  for (i = 0; i < input->composition->n_layers; i++)
    for (j = 0; j < input->composition->layers[i].n_elements; j++) {
      const int Z = input->composition->layers[i].Z[j];
      int found = 0;
      for (k = 0; k < nuniq; k++) found |= uniqZ[k] == Z;
      if (!found) uniqZ[nuniq++] = Z;
    }
  qsort(uniqZ, (size_t)nuniq, sizeof(int), cmp_int);
  out->brute_force_history = unpack_history(brute_history, uniqZ, nuniq, N, &out->nbrute_force_history);
  if (var_red_history)
    out->var_red_history = unpack_history(var_red_history, uniqZ, nuniq, N, &out->nvar_red_history);
  free(uniqZ);
  return out;
}

static void free_history(xmi_fluorescence_line_counts *h, int n) {
  int i, j;
  if (!h) return;
  for (i = 0; i < n; i++) {
    for (j = 0; j < h[i].n_lines; j++) {
      free(h[i].lines[j].line_type);
      free(h[i].lines[j].interactions);
    }
    free(h[i].lines);
  }
  free(h);
}

/* reference include/xmi_data_structs.h:406 */
void xmi_output_free(xmi_output *o) {
  int i;
  if (!o) return;
  free(o->inputfile);
  free(o->outputfile);
  for (i = 0; i <= o->ninteractions; i++) {
    if (o->channels_conv) free(o->channels_conv[i]);
    if (o->channels_unconv) free(o->channels_unconv[i]);
  }
  free(o->channels_conv);
  free(o->channels_unconv);
  free_history(o->brute_force_history, o->nbrute_force_history);
  free_history(o->var_red_history, o->nvar_red_history);
  if (o->input) xmi_input_free(o->input);
  free(o);
}

/* ------------------------------------------------------------------ */
/* writer                                                              */
/* ------------------------------------------------------------------ */
static void put_text(FILE *f, const char *s) {
  for (; s && *s; s++) switch (*s) {
      case '&': fputs("&amp;", f); break;
      case '<': fputs("&lt;", f); break;
      case '>': fputs("&gt;", f); break;
      case '"': fputs("&quot;", f); break;
      default: fputc(*s, f);
    }
}

static void indent(FILE *f, int d) {
  while (d-- > 0) fputs("  ", f);
}

static void elem_s(FILE *f, int d, const char *tag, const char *v) {
  indent(f, d);
  if (!v || !*v) {
    fprintf(f, "<%s/>\n", tag);
    return;
  }
  fprintf(f, "<%s>", tag);
  put_text(f, v);
  fprintf(f, "</%s>\n", tag);
}

static void elem_g(FILE *f, int d, const char *tag, double v) {
  indent(f, d);
  fprintf(f, "<%s>%.17g</%s>\n", tag, v, tag);
}

static void elem_i(FILE *f, int d, const char *tag, long v) {
  indent(f, d);
  fprintf(f, "<%s>%ld</%s>\n", tag, v, tag);
}

static void write_layer(FILE *f, int d, const xmi_layer *l) {
  int i;
  indent(f, d);
  fputs("<layer>\n", f);
  for (i = 0; i < l->n_elements; i++) {
    indent(f, d + 1);
    fputs("<element>\n", f);
    elem_i(f, d + 2, "atomic_number", l->Z[i]);
    elem_g(f, d + 2, "weight_fraction", l->weight[i] * 100.0);
    indent(f, d + 1);
    fputs("</element>\n", f);
  }
  elem_g(f, d + 1, "density", l->density);
  elem_g(f, d + 1, "thickness", l->thickness);
  indent(f, d);
  fputs("</layer>\n", f);
}

static void write_xyz(FILE *f, int d, const char *tag, const double *v) {
  indent(f, d);
  fprintf(f, "<%s>\n", tag);
  elem_g(f, d + 1, "x", v[0]);
  elem_g(f, d + 1, "y", v[1]);
  elem_g(f, d + 1, "z", v[2]);
  indent(f, d);
  fprintf(f, "</%s>\n", tag);
}

static void write_source(FILE *f, int d, const char *tag, double E, double h, double v, double sx, double sxp,
                         double sy, double syp) {
  indent(f, d);
  fprintf(f, "<%s>\n", tag);
  elem_g(f, d + 1, "energy", E);
  elem_g(f, d + 1, "horizontal_intensity", h);
  elem_g(f, d + 1, "vertical_intensity", v);
  elem_g(f, d + 1, "sigma_x", sx);
  elem_g(f, d + 1, "sigma_xp", sxp);
  elem_g(f, d + 1, "sigma_y", sy);
  elem_g(f, d + 1, "sigma_yp", syp);
}

/* the input section, src/xmi_xml.c:1680-1850 */
static void write_input(FILE *f, int d, const xmi_input *in) {
  static const char *const dist_names[] = {"monochromatic", "gaussian", "lorentzian"};
  static const char *const det_names[] = {"SiLi", "Ge", "Si_SDD"};
  int i;
  indent(f, d);
  fputs("<general version=\"" XMSO_VERSION "\">\n", f);
  elem_s(f, d + 1, "outputfile", in->general->outputfile);
  elem_i(f, d + 1, "n_photons_interval", in->general->n_photons_interval);
  elem_i(f, d + 1, "n_photons_line", in->general->n_photons_line);
  elem_i(f, d + 1, "n_interactions_trajectory", in->general->n_interactions_trajectory);
  elem_s(f, d + 1, "comments", in->general->comments);
  indent(f, d);
  fputs("</general>\n", f);
  indent(f, d);
  fputs("<composition>\n", f);
  for (i = 0; i < in->composition->n_layers; i++) write_layer(f, d + 1, &in->composition->layers[i]);
  elem_i(f, d + 1, "reference_layer", in->composition->reference_layer);
  indent(f, d);
  fputs("</composition>\n", f);
  indent(f, d);
  fputs("<geometry>\n", f);
  elem_g(f, d + 1, "d_sample_source", in->geometry->d_sample_source);
  write_xyz(f, d + 1, "n_sample_orientation", in->geometry->n_sample_orientation);
  write_xyz(f, d + 1, "p_detector_window", in->geometry->p_detector_window);
  write_xyz(f, d + 1, "n_detector_orientation", in->geometry->n_detector_orientation);
  elem_g(f, d + 1, "area_detector", in->geometry->area_detector);
  elem_g(f, d + 1, "collimator_height", in->geometry->collimator_height);
  elem_g(f, d + 1, "collimator_diameter", in->geometry->collimator_diameter);
  elem_g(f, d + 1, "d_source_slit", in->geometry->d_source_slit);
  indent(f, d + 1);
  fputs("<slit_size>\n", f);
  elem_g(f, d + 2, "slit_size_x", in->geometry->slit_size_x);
  elem_g(f, d + 2, "slit_size_y", in->geometry->slit_size_y);
  indent(f, d + 1);
  fputs("</slit_size>\n", f);
  indent(f, d);
  fputs("</geometry>\n", f);
  indent(f, d);
  fputs("<excitation>\n", f);
  for (i = 0; i < in->excitation->n_discrete; i++) {
    const xmi_energy_discrete *x = &in->excitation->discrete[i];
    write_source(f, d + 1, "discrete", x->energy, x->horizontal_intensity, x->vertical_intensity, x->sigma_x,
                 x->sigma_xp, x->sigma_y, x->sigma_yp);
    if (x->distribution_type != XMI_ENERGY_DISCRETE_DISTRIBUTION_MONOCHROMATIC && (int)x->distribution_type >= 0 &&
        (int)x->distribution_type <= 2) {
      indent(f, d + 2);
      fprintf(f, "<scale_parameter distribution_type=\"%s\">%.17g</scale_parameter>\n",
              dist_names[(int)x->distribution_type], x->scale_parameter);
    }
    indent(f, d + 1);
    fputs("</discrete>\n", f);
  }
  for (i = 0; i < in->excitation->n_continuous; i++) {
    const xmi_energy_continuous *x = &in->excitation->continuous[i];
    write_source(f, d + 1, "continuous", x->energy, x->horizontal_intensity, x->vertical_intensity, x->sigma_x,
                 x->sigma_xp, x->sigma_y, x->sigma_yp);
    indent(f, d + 1);
    fputs("</continuous>\n", f);
  }
  indent(f, d);
  fputs("</excitation>\n", f);
  indent(f, d);
  fputs("<absorbers>\n", f);
  if (in->absorbers->n_exc_layers > 0) {
    indent(f, d + 1);
    fputs("<excitation_path>\n", f);
    for (i = 0; i < in->absorbers->n_exc_layers; i++) write_layer(f, d + 2, &in->absorbers->exc_layers[i]);
    indent(f, d + 1);
    fputs("</excitation_path>\n", f);
  }
  if (in->absorbers->n_det_layers > 0) {
    indent(f, d + 1);
    fputs("<detector_path>\n", f);
    for (i = 0; i < in->absorbers->n_det_layers; i++) write_layer(f, d + 2, &in->absorbers->det_layers[i]);
    indent(f, d + 1);
    fputs("</detector_path>\n", f);
  }
  indent(f, d);
  fputs("</absorbers>\n", f);
  indent(f, d);
  fputs("<detector>\n", f);
  elem_s(f, d + 1, "detector_type",
         (int)in->detector->detector_type >= 0 && (int)in->detector->detector_type <= 2
             ? det_names[(int)in->detector->detector_type]
             : "SiLi");
  elem_g(f, d + 1, "live_time", in->detector->live_time);
  elem_g(f, d + 1, "pulse_width", in->detector->pulse_width);
  elem_i(f, d + 1, "nchannels", in->detector->nchannels);
  elem_g(f, d + 1, "gain", in->detector->gain);
  elem_g(f, d + 1, "zero", in->detector->zero);
  elem_g(f, d + 1, "fano", in->detector->fano);
  elem_g(f, d + 1, "noise", in->detector->noise);
  indent(f, d + 1);
  fputs("<crystal>\n", f);
  for (i = 0; i < in->detector->n_crystal_layers; i++) write_layer(f, d + 2, &in->detector->crystal_layers[i]);
  indent(f, d + 1);
  fputs("</crystal>\n", f);
  indent(f, d);
  fputs("</detector>\n", f);
}

static void write_spectrum(FILE *f, const char *tag, const xmi_output *o, double *const *ch) {
  const xmi_detector *det = o->input->detector;
  int i, j;
  fprintf(f, "  <%s>\n", tag);
  for (j = 0; j < det->nchannels; j++) {
    fputs("    <channel>\n", f);
    fprintf(f, "      <channelnr>%d</channelnr>\n", j);
    fprintf(f, "      <energy>%.17g</energy>\n", det->gain * j + det->zero);
    for (i = o->use_zero_interactions == 1 ? 0 : 1; i <= o->input->general->n_interactions_trajectory; i++)
      fprintf(f, "      <counts interaction_number=\"%d\">%.17g</counts>\n", i, ch[i][j]);
    fputs("    </channel>\n", f);
  }
  fprintf(f, "  </%s>\n", tag);
}

static void write_history(FILE *f, const char *tag, const xmi_fluorescence_line_counts *h, int n) {
  int i, j, k;
  if (!h || n == 0) {
    fprintf(f, "  <%s/>\n", tag);
    return;
  }
  fprintf(f, "  <%s>\n", tag);
  for (i = 0; i < n; i++) {
    const int Z = h[i].atomic_number;
    fprintf(f, "    <fluorescence_line_counts atomic_number=\"%d\" symbol=\"%s\" total_counts=\"%.17g\">\n", Z,
            Z >= 1 && Z <= 100 ? kSymbols[Z - 1] : "", h[i].total_counts);
    for (j = 0; j < h[i].n_lines; j++) {
      const xmi_fluorescence_line *l = &h[i].lines[j];
      fputs("      <fluorescence_line type=\"", f);
      put_text(f, l->line_type);
      fprintf(f, "\" energy=\"%.17g\" total_counts=\"%.17g\">\n", l->energy, l->total_counts);
      for (k = 0; k < l->n_interactions; k++)
        fprintf(f, "        <counts interaction_number=\"%d\">%.17g</counts>\n", l->interactions[k].interaction_number,
                l->interactions[k].counts);
      fputs("      </fluorescence_line>\n", f);
    }
    fputs("    </fluorescence_line_counts>\n", f);
  }
  fprintf(f, "  </%s>\n", tag);
}

/* reference src/xmi_xml.c:1638-1675 */
int xmi_output_write_to_xml_file(xmi_output *output, const char *xmsofile, GError **error) {
  FILE *f;
  (void)error; /* the reason of a failure is available from xmi_gpu_last_error() */
  if (!output || !output->input || !xmsofile) {
    xmi_set_error("xmi_output_write_to_xml_file: NULL argument");
    return 0;
  }
  f = fopen(xmsofile, "w");
  if (!f) {
    xmi_set_error("xmi_output_write_to_xml_file: cannot open %s for writing", xmsofile);
    return 0;
  }
  fputs("<?xml version=\"1.0\" encoding=\"UTF-8\"?>\n", f);
  fputs("<!DOCTYPE xmimsim-results SYSTEM \"http://www.xmi.UGent.be/xml/xmimsim-1.0.dtd\">\n", f);
  fputs("<xmimsim-results version=\"" XMSO_VERSION "\">\n", f);
  elem_s(f, 1, "inputfile", output->inputfile);
  write_spectrum(f, "spectrum_conv", output, output->channels_conv);
  write_spectrum(f, "spectrum_unconv", output, output->channels_unconv);
  write_history(f, "brute_force_history", output->brute_force_history, output->nbrute_force_history);
  write_history(f, "variance_reduction_history", output->var_red_history, output->nvar_red_history);
  fputs("  <xmimsim-input>\n", f);
  write_input(f, 2, output->input);
  fputs("  </xmimsim-input>\n", f);
  fputs("</xmimsim-results>\n", f);
  if (fclose(f) != 0) {
    xmi_set_error("xmi_output_write_to_xml_file: write to %s failed", xmsofile);
    return 0;
  }
  return 1;
}
