/*
 * TEST INFRASTRUCTURE (oracle/_ref) -- not part of the engine.
 *
 * Runs the reference's own OpenCL solid-angle kernel
 * (src/xmi_kernels.cl:219-453, XMI-MSIM) on the host: the kernel source and
 * the vendored Random123 headers are compiled from where they lie in the
 * reference tree (paths given by the build recipe, oracle/ref_cl/Makefile),
 * in the order the reference's OpenCL host code concatenates them.
 * Each work item (r index, theta index) is one call of the kernel body with
 * the ids set as the OpenCL runtime would for a 2-D range of
 * nr/RANGE_DIVIDER x nt/RANGE_DIVIDER items launched at the offsets of
 * src/xmi_solid_angle_cl.c:379-392.
 */
#include "cl_host_shim.h"

#include <vector>

#include REF_R123_OPENCLFEATURES
#include REF_R123_COMPILERFEATURES
#include REF_R123_SSE
#include REF_R123_ARRAY
#include REF_R123_THREEFRY
#include REF_KERNELS_CL

extern "C" {

/* Solid angles of the grid points (ir[k], it[k]) of an nr x nt grid whose
 * axes are r_vals / theta_vals (FP32, as the reference uploads them). */
void ref_cl_solid_angle_points(const float *r_vals, int nr, const float *theta_vals, int nt, const int *ir,
                               const int *it, int n, int collimator_present, float detector_radius,
                               float collimator_radius, float collimator_height, int hits_per_single,
                               float *out) {
  std::vector<float> grid((size_t)nr * nt, NAN);
#pragma omp parallel for schedule(dynamic, 4)
  for (int k = 0; k < n; k++) {
    cl_gid[0] = (size_t)ir[k];
    cl_gid[1] = (size_t)it[k];
    cl_gsize[0] = (size_t)nr / RANGE_DIVIDER;
    cl_gsize[1] = (size_t)nt / RANGE_DIVIDER;
    xmi_solid_angle_calculation(r_vals, theta_vals, grid.data(), collimator_present, detector_radius,
                                collimator_radius, collimator_height, hits_per_single);
  }
  for (int k = 0; k < n; k++) out[k] = grid[(size_t)it[k] * nr + ir[k]];
}

/* one Threefry4x32-20 block through the reference's Random123 header */
void ref_cl_threefry4x32(const uint32_t *ctr, const uint32_t *key, uint32_t *out) {
  threefry4x32_ctr_t c = {{ctr[0], ctr[1], ctr[2], ctr[3]}};
  threefry4x32_key_t k = {{key[0], key[1], key[2], key[3]}};
  threefry4x32_ctr_t r = threefry4x32(c, k);
  for (int i = 0; i < 4; i++) out[i] = r.v[i];
}
}
