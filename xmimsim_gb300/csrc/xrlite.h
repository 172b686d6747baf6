/*
 * Stand-in atomic data model ("xrlite").
 *
 * The reference takes every cross section and atomic parameter from
 * xraylib (src/xmi_aux_f.F90:22 `USE :: xraylib`; configure.ac:115-116
 * `libxrl >= 3.99.0`), which is not available on the build or GPU machines.
 * This module provides the same function surface (CS_Total_Kissel,
 * CS_Photo_Partial, DCSP_Rayl, RadRate, ...) from a compact parametrised
 * model: tabulated K-edge energies and atomic weights, screened-hydrogenic
 * ratios for the L/M/N edges, dipole line sets with smooth branching ratios,
 * Bambynek-style fluorescence yields, jump-ratio photo-absorption partials,
 * Thomson/Klein-Nishina scattering with analytic form factor and
 * incoherent scattering functions, and hydrogenic Compton profiles.
 *
 * It is a physically plausible stand-in for engine testing, not a
 * replacement for xraylib: absolute intensities differ from real materials.
 * The transport engine never calls this module; it only consumes the tables
 * the host tabulator builds from it.
 */
#ifndef XMIMSIM_GB300_XRLITE_H
#define XMIMSIM_GB300_XRLITE_H

#ifdef __cplusplus
extern "C" {
#endif

#define XRL_MAXZ 94
#define XRL_NSHELL_ALL 29  /* K..Q1 as in xraylib shell numbering */
#define XRL_NLINES 383

/* physical constants */
#define XRL_RE2 0.07940775      /* classical electron radius squared, barn */
#define XRL_AVOGNUM 0.602214129 /* Avogadro / 1e24 (barn -> cm2/g with A in g/mol) */
#define XRL_KEV2ANGST 12.39852
#define XRL_MEC2 510.998928

double xrl_AtomicWeight(int Z);
double xrl_EdgeEnergy(int Z, int shell);       /* keV, 0 if shell empty */
double xrl_ElectronConfig(int Z, int shell);   /* electrons in shell */
double xrl_LineEnergy(int Z, int line);        /* line 1..383, keV */
double xrl_RadRate(int Z, int line);
double xrl_FluorYield(int Z, int shell);
double xrl_CosKronTransProb(int Z, int trans); /* trans 0..13, XMI_FL12.. */
double xrl_AugerYield(int Z, int shell);
/* expected vacancies created in shell t per non-radiative decay of shell s */
double xrl_AugerVacancies(int Z, int s, int t);
/* probability of Auger transition trans (xraylib numbering K_L1L1 = 0 ..
 * L3_M5Q3 = 644) given a non-radiative decay of its initial shell */
double xrl_AugerRate(int Z, int trans);

/* builds the per-Z scattering cross-section cache; call once per Z from a
 * single thread before using the CS functions from several threads */
void xrl_prepare(int Z);

double xrl_CS_Photo_Partial(int Z, int shell, double E);
double xrl_CS_Photo_Total(int Z, double E);
double xrl_CS_Rayl(int Z, double E);
double xrl_CS_Compt(int Z, double E);
double xrl_CS_Total_Kissel(int Z, double E);

double xrl_FF_Rayl(int Z, double q);
double xrl_SF_Compt(int Z, double q);
double xrl_DCS_Rayl(int Z, double E, double theta);
double xrl_DCS_Compt(int Z, double E, double theta);
double xrl_DCSP_Rayl(int Z, double E, double theta, double phi);
double xrl_DCSP_Compt(int Z, double E, double theta, double phi);
double xrl_ComptonProfile(int Z, double pz);

/* line names (reference src/xmi_lines.c), index 0..385 */
const char *xrl_line_name(int line);
int xrl_line_from_name(const char *name);
/* first/last line index of each shell's transitions as scanned by the
 * reference (src/xmi_main.F90:5373-5400) */
int xrl_shell_first_line(int shell);
int xrl_shell_last_line(int shell);
/* lower (vacancy) shell and upper (donor) shell of a line; -1 if none */
int xrl_line_lower_shell(int line);
int xrl_line_upper_shell(int line);

#ifdef __cplusplus
}
#endif
#endif
