/*
 * Solid-angle grid kernel: xmi_solid_angle_calculation_f
 * (src/xmi_solid_angle_f.F90:303-429) / the OpenCL kernel
 * (src/xmi_kernels.cl:219-453), one warp per (r, theta) grid point.
 *
 * Each cone sample i of a point draws its two uniforms from Philox block i
 * of the point's stream (seed, point, 0xF0000000), so the lanes of a warp
 * take samples i = lane, lane+32, ... independently and the hit count is
 * exactly that of the sequential oracle.  The FP32 variant uses the same
 * draws truncated to 24 bits.  The work is FP32/FP64 issue-bound (about 40 flops and 3-5
 * transcendental ops per sample, no memory traffic beyond the result).
 *
 * stream = 1 replaces the Philox draws by the OpenCL backend's own stream
 * (src/xmi_kernels.cl:226-227,393-404): Threefry4x32-20 with key
 * (r index, 0xdecafbad, 0xfacebead, theta index) and counter
 * (j, 0xf00dcafe, 0xdeadbeef, 0xbeeff00d) for the j-th pair of samples
 * (j = 1, 2, ...), each uniform a 32-bit word / 2^32 in single precision.
 * With it the grid can be checked point by point against the reference
 * kernel itself; lanes then take sample pairs j = lane + 1, lane + 33, ....
 */
#ifndef XMIMSIM_GB300_SOLID_ANGLE_CUH
#define XMIMSIM_GB300_SOLID_ANGLE_CUH

#include "transport.cuh"

namespace xmi {

struct SaGeom {
  double det_radius, coll_radius, coll_height;
  int coll_present;
};

template <typename R>
__device__ __forceinline__ bool sa_setup(const SaGeom &s, R r1, R theta1, R &cfca, R &fcsa, R &st, R &ct, R &py,
                                         R &pz, bool &outside) {
  R r, theta, fcbr;
  const R detr = (R)s.det_radius, collr = (R)s.coll_radius, collh = (R)s.coll_height;
  if (!s.coll_present) {
    r = r1; theta = theta1; fcbr = detr; outside = false;
  } else if (fabs(collr - detr) < (R)0.000001) {
    if (r1 * cos(theta1) <= detr) {
      r = r1; theta = theta1; fcbr = detr;
    } else {
      sa_opening<R>(r1, theta1, collh, r, theta);
      fcbr = collr;
    }
    outside = r1 * sin(theta1) > collh;
  } else {
    if (r1 * cos(theta1) <= detr && r1 * sin(theta1) <= collh * (r1 * cos(theta1) - detr) / (collr - detr)) {
      r = r1; theta = theta1; fcbr = detr;
    } else if (r1 * sin(theta1) <= collh) {
      return false;
    } else {
      sa_opening<R>(r1, theta1, collh, r, theta);
      fcbr = collr;
    }
    outside = r1 * sin(theta1) > collh;
  }
  R beta = atan(fcbr / r);
  R alpha1 = atan(fcbr * sin(theta) / (r - fcbr * cos(theta)));
  if (alpha1 <= (R)0) alpha1 = alpha1 + (R)kPi;
  R fca = beta > alpha1 ? beta : alpha1;
  cfca = cos(fca);
  fcsa = (R)(2 * kPi) * ((R)1 - cfca);
  st = sin(theta);
  ct = cos(theta);
  py = r1 * cos(theta1);
  pz = r1 * sin(theta1);
  return true;
}

template <typename R>
__device__ __forceinline__ int sa_sample(const SaGeom &s, R cfca, R st, R ct, R py, R pz, bool outside, R u1, R u2) {
  const R detr = (R)s.det_radius, collr = (R)s.coll_radius, collh = (R)s.coll_height;
  R th = acos((R)1 - u1 * ((R)1 - cfca));
  R ph = u2 * (R)2 * (R)kPi;
  R sth = sin(th);
  R dcx = sth * cos(ph), dcy = sth * sin(ph), dcz = cos(th);
  R dx = dcx, dy = -st * dcy - ct * dcz, dz = ct * dcy - st * dcz;
  if (dz >= (R)0) return 0;
  if (outside) {
    R q = (collh - pz) / dz;
    R ix = q * dx, iy = q * dy + py;
    if (sqrt(ix * ix + iy * iy) > collr) return 0;
  }
  R q = (-pz) / dz;
  R ix = q * dx, iy = q * dy + py, iz = q * dz + pz;
  return sqrt(ix * ix + iy * iy + iz * iz) <= detr ? 1 : 0;
}

/* the two uniforms of a cone sample from one Philox block: in FP64 the
 * 53-bit draws of the transport's generator; in FP32 the same draws
 * truncated to 24 bits (the transport's FP32 rule), with no FP64 arithmetic */
__device__ __forceinline__ void cone_draws(const xmi_u32x4 &o, double &u1, double &u2) {
  u1 = ((double)(o.v[0] >> 5) * 67108864.0 + (double)(o.v[1] >> 6)) * (1.0 / 9007199254740992.0);
  u2 = ((double)(o.v[2] >> 5) * 67108864.0 + (double)(o.v[3] >> 6)) * (1.0 / 9007199254740992.0);
}
__device__ __forceinline__ void cone_draws(const xmi_u32x4 &o, float &u1, float &u2) {
  u1 = (float)(o.v[0] >> 8) * 0x1p-24f;
  u2 = (float)(o.v[2] >> 8) * 0x1p-24f;
}

/* out[t*nr + r] = solid angle of grid point (r_vals[r], t_vals[t]) */
template <typename R>
__global__ void __launch_bounds__(256) solid_angle_grid_kernel(SaGeom s, const double *r_vals, int nr,
                                                                const double *t_vals, long long p0, long long p1,
                                                                int hits_per_single, unsigned long long seed,
                                                                int stream, double *out) {
  const int lane = threadIdx.x & 31;
  const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long p = p0 + (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); p < p1; p += warps) {
    const int it = (int)(p / nr), ir = (int)(p % nr);
    R cfca, fcsa, st, ct, py, pz;
    bool outside;
    int hits = 0;
    bool live = sa_setup<R>(s, (R)r_vals[ir], (R)t_vals[it], cfca, fcsa, st, ct, py, pz, outside);
    if (live && stream == 1) {
      xmi_u32x4 key, c;
      key.v[0] = (uint32_t)ir;
      key.v[1] = 0xdecafbadu;
      key.v[2] = 0xfacebeadu;
      key.v[3] = (uint32_t)it;
      c.v[1] = 0xf00dcafeu;
      c.v[2] = 0xdeadbeefu;
      c.v[3] = 0xbeeff00du;
      const int pairs = (hits_per_single + 1) / 2;
      for (int j = lane; j < pairs; j += 32) {
        c.v[0] = (uint32_t)(j + 1);
        xmi_u32x4 o = xmi_threefry4x32_20(c, key);
        const float inv = 4294967296.0f;
        hits += sa_sample<R>(s, cfca, st, ct, py, pz, outside, (R)((float)o.v[0] / inv), (R)((float)o.v[1] / inv));
        if (2 * j + 1 < hits_per_single)
          hits += sa_sample<R>(s, cfca, st, ct, py, pz, outside, (R)((float)o.v[2] / inv),
                               (R)((float)o.v[3] / inv));
      }
    } else if (live) {
      for (int i = lane; i < hits_per_single; i += 32) {
        xmi_u32x4 c;
        c.v[0] = (uint32_t)i;
        c.v[1] = 0xF0000000u;
        c.v[2] = (uint32_t)p;
        c.v[3] = (uint32_t)((unsigned long long)p >> 32);
        xmi_u32x4 o = xmi_philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
        R u1, u2;
        cone_draws(o, u1, u2);
        hits += sa_sample<R>(s, cfca, st, ct, py, pz, outside, u1, u2);
      }
    }
    hits = __reduce_add_sync(0xffffffffu, hits);
    if (lane == 0) out[p - p0] = live ? (double)(fcsa * (R)hits / (R)hits_per_single) : 0.0;
  }
}

/* solid angle at arbitrary points (r[i], t[i]), i < n: one warp per point,
 * Philox block k of stream (seed, point, 0xF1000000) for sample k (the
 * integrator behind the surrogate network's training targets and checks) */
template <typename R>
__global__ void __launch_bounds__(256) solid_angle_points_kernel(SaGeom s, const double *r, const double *t,
                                                                 long long n, int hits_per_single,
                                                                 unsigned long long seed, double *out) {
  const int lane = threadIdx.x & 31;
  const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long p = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); p < n; p += warps) {
    R cfca, fcsa, st, ct, py, pz;
    bool outside;
    int hits = 0;
    const bool live = sa_setup<R>(s, (R)r[p], (R)t[p], cfca, fcsa, st, ct, py, pz, outside);
    if (live) {
      for (int i = lane; i < hits_per_single; i += 32) {
        xmi_u32x4 c;
        c.v[0] = (uint32_t)i;
        c.v[1] = 0xF1000000u;
        c.v[2] = (uint32_t)p;
        c.v[3] = (uint32_t)((unsigned long long)p >> 32);
        xmi_u32x4 o = xmi_philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
        R u1, u2;
        cone_draws(o, u1, u2);
        hits += sa_sample<R>(s, cfca, st, ct, py, pz, outside, u1, u2);
      }
    }
    hits = __reduce_add_sync(0xffffffffu, hits);
    if (lane == 0) out[p] = live ? (double)fcsa * (double)hits / (double)hits_per_single : 0.0;
  }
}

}  // namespace xmi
#endif
