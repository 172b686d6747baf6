/*
 * GB300 engine: device mirror of the table bundle, the transport and
 * solid-angle launches behind the C-ABI, and the reshaping of the device
 * tallies into the reference's output layouts.
 */
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <chrono>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "estimator.cuh"
#include "solid_angle.cuh"
#include "transport.cuh"
#include "wavefront.cuh"
#include "xmi_internal.h"

long hits_per_single = 5000; /* src/xmi_solid_angle_f.F90:43-44 */

namespace {

struct Timing {
  double transport_ms = 0.0, total_ms = 0.0;
  int launches = 0;
  /* phases of the last xmi_main_msim: transport, event sort, surrogate solid angles, estimator */
  double phase_ms[4] = {0.0, 0.0, 0.0, 0.0};
  long long events = 0, surrogate_fallbacks = 0;
  /* host<->device bytes copied by the last xmi_main_msim / _batch call */
  long long h2d_bytes = 0, d2h_bytes = 0;
  /* the batched call's graph: -1 none, 0 instantiated, 1 updated in place */
  int graph_updated = -1;
};
thread_local Timing g_timing;

bool cuda_ok(cudaError_t e, const char *what) {
  if (e != cudaSuccess) {
    xmi_set_error("%s: %s", what, cudaGetErrorString(e));
    return false;
  }
  return true;
}

/* device allocations of one precision */
struct DevSide {
  std::vector<void *> allocs;
  bool valid = false;
  void *b = nullptr; /* DevBundle<R> (host copy of the device struct) */
  void release() {
    for (void *p : allocs) cudaFree(p);
    allocs.clear();
    valid = false;
  }
};

/* device buffers of the estimator event queue of one chunk */
struct QueueBufs {
  void *events = nullptr;
  int *key = nullptr, *order = nullptr;
  int *fb = nullptr;        /* events the surrogate leaves to the integrator */
  unsigned *hist = nullptr; /* [2][nkeys]: counts, then scatter cursors */
  unsigned long long *count = nullptr; /* [0] events queued, [1] estimator work counter, [2] fb entries */
  size_t bytes = 0;
  long long cap = 0;
  int nkeys = 0;
  void release() {
    cudaFree(events);
    cudaFree(key);
    cudaFree(order);
    cudaFree(fb);
    cudaFree(hist);
    cudaFree(count);
    *this = QueueBufs();
  }
};

/* The event queues of a chunk sequence: two, so that chunk k+1's transport
 * fills one while chunk k's sort, solid angles and estimator read the other
 * on a second stream. */
struct EventQueue {
  QueueBufs buf[2];
  cudaStream_t side = nullptr; /* stream of the sort / solid-angle / estimator phases */
  cudaEvent_t filled[2] = {nullptr, nullptr}, drained[2] = {nullptr, nullptr}, joined = nullptr;
  /* executable graph of the last captured chunk sequence on this queue: the
   * next capture of the same shape updates it in place (cudaGraphExecUpdate)
   * instead of instantiating a new one */
  cudaGraphExec_t exec = nullptr;
  /* timing events of the chunk sequence, kept across calls so that a
   * captured sequence of the same shape records the same events */
  std::vector<cudaEvent_t> marks;
  void drop_exec() {
    if (exec) cudaGraphExecDestroy(exec);
    exec = nullptr;
  }
  bool ensure_side() {
    if (side) return true;
    if (cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking) != cudaSuccess) return false;
    bool ok = cudaEventCreateWithFlags(&joined, cudaEventDisableTiming) == cudaSuccess;
    for (int i = 0; i < 2; i++)
      ok = ok && cudaEventCreateWithFlags(&filled[i], cudaEventDisableTiming) == cudaSuccess &&
           cudaEventCreateWithFlags(&drained[i], cudaEventDisableTiming) == cudaSuccess;
    return ok;
  }
  void release() {
    drop_exec();
    for (cudaEvent_t e : marks) cudaEventDestroy(e);
    marks.clear();
    buf[0].release();
    buf[1].release();
    if (side) {
      cudaStreamSynchronize(side);
      cudaStreamDestroy(side);
    }
    for (int i = 0; i < 2; i++) {
      if (filled[i]) cudaEventDestroy(filled[i]);
      if (drained[i]) cudaEventDestroy(drained[i]);
    }
    if (joined) cudaEventDestroy(joined);
    *this = EventQueue();
  }
};

/* photon states and lists of the wavefront transport of one chunk */
struct WfBuffers {
  void *st = nullptr;
  int *lists = nullptr; /* 5 lists of cap entries */
  unsigned *count = nullptr;
  unsigned char *casc = nullptr; /* [cap] cascade-used flags of the analog cascades */
  size_t st_bytes = 0;
  long long cap = 0;
  void release() {
    cudaFree(st);
    cudaFree(lists);
    cudaFree(count);
    cudaFree(casc);
    *this = WfBuffers();
  }
};

struct DevState {
  DevSide d64, d32;
  xmi::DevBundle<double> b64;
  xmi::DevBundle<float> b32;
  /* run buffers */
  xmi_source_item *items = nullptr;
  xmi::ItemF *items_f = nullptr;
  long long *item_first = nullptr;
  int items_cap = 0;
  double *sa_r = nullptr, *sa_t = nullptr, *sa_g64 = nullptr;
  float *sa_g32 = nullptr;
  int sa_n = 0;
  const double *sa_src = nullptr;
  double *tally = nullptr;
  size_t tally_cap = 0;
  unsigned long long *counters = nullptr;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  void *d_bundle = nullptr;      /* device copy of the run's DevBundle (estimator argument) */
  xmi::DevTally *d_tally = nullptr;
};

/* Event queue and wavefront state of a run (several GB at the default
 * queue size).  Runs borrow them from a per-device pool instead of owning
 * them per handle, so hundreds of handles run one after another in the
 * memory of one run; concurrent runs on different host threads each take
 * their own set. */
struct RunBuffers {
  int device = 0;
  EventQueue q;
  WfBuffers wf;
};
std::mutex g_pool_lock;
std::vector<RunBuffers *> g_pool;

RunBuffers *acquire_buffers() {
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(g_pool_lock);
  for (size_t i = 0; i < g_pool.size(); i++)
    if (g_pool[i]->device == dev) {
      RunBuffers *rb = g_pool[i];
      g_pool.erase(g_pool.begin() + (long)i);
      return rb;
    }
  RunBuffers *rb = new RunBuffers();
  rb->device = dev;
  return rb;
}

void release_buffers(RunBuffers *rb) {
  std::lock_guard<std::mutex> lk(g_pool_lock);
  g_pool.push_back(rb);
}

template <typename R>
const R *upload(DevSide &s, const double *src, size_t n) {
  if (n == 0) n = 1;
  std::vector<R> tmp(n);
  for (size_t i = 0; i < n; i++) tmp[i] = src ? (R)src[i] : (R)0;
  void *p = nullptr;
  if (cudaMalloc(&p, sizeof(R) * n) != cudaSuccess) return nullptr;
  s.allocs.push_back(p);
  cudaMemcpy(p, tmp.data(), sizeof(R) * n, cudaMemcpyHostToDevice);
  return (const R *)p;
}

/* Device copies of the tables that depend on Z alone, made once per device
 * and precision and shared by every bundle: keyed by the host table they
 * copy, which the host keeps for the life of the process.  A batch of
 * hundreds of configurations over the same elements then holds one copy of
 * each element's angular tables instead of one per configuration. */
std::mutex g_ztab_lock;
std::map<std::tuple<int, int, const double *>, void *> g_ztab;

template <typename R>
const R *shared_table(const double *src, size_t n) {
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(g_ztab_lock);
  const auto key = std::make_tuple(dev, (int)sizeof(R), src);
  auto it = g_ztab.find(key);
  if (it != g_ztab.end()) return (const R *)it->second;
  std::vector<R> tmp(n);
  for (size_t i = 0; i < n; i++) tmp[i] = (R)src[i];
  void *p = nullptr;
  if (cudaMalloc(&p, sizeof(R) * n) != cudaSuccess) return nullptr;
  if (cudaMemcpy(p, tmp.data(), sizeof(R) * n, cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaFree(p);
    return nullptr;
  }
  g_ztab[key] = p;
  return (const R *)p;
}

/* per-element array of device pointers to the shared tables */
template <typename R>
const R *const *upload_per_element(DevSide &s, const double *const *src, int E, size_t n) {
  std::vector<const R *> ptrs(E > 0 ? E : 1, nullptr);
  for (int e = 0; e < E; e++)
    if (!(ptrs[e] = shared_table<R>(src[e], n))) return nullptr;
  void *p = nullptr;
  if (cudaMalloc(&p, sizeof(const R *) * ptrs.size()) != cudaSuccess) return nullptr;
  s.allocs.push_back(p);
  cudaMemcpy(p, ptrs.data(), sizeof(const R *) * ptrs.size(), cudaMemcpyHostToDevice);
  return (const R *const *)p;
}

const void *upload_bytes(DevSide &s, const void *src, size_t bytes) {
  void *p = nullptr;
  if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
  s.allocs.push_back(p);
  cudaMemcpy(p, src, bytes, cudaMemcpyHostToDevice);
  return p;
}

const int *upload_int(DevSide &s, const int *src, size_t n) {
  if (n == 0) n = 1;
  void *p = nullptr;
  if (cudaMalloc(&p, sizeof(int) * n) != cudaSuccess) return nullptr;
  s.allocs.push_back(p);
  if (src) cudaMemcpy(p, src, sizeof(int) * n, cudaMemcpyHostToDevice);
  else cudaMemset(p, 0, sizeof(int) * n);
  return (const int *)p;
}

/* the Compton profile tables of the bundle's elements (advanced Compton):
 * added to a device copy on first use; false on a failed upload */
template <typename R>
bool upload_compton_profiles(const xmi_bundle &h, DevSide &s, xmi::DevBundle<R> &d) {
  if (d.cp_cdf || !h.cp_nshell) return true;
  const int E = h.n_elem;
  std::vector<const R *> pc(E > 0 ? E : 1, nullptr), pq(E > 0 ? E : 1, nullptr);
  for (int e = 0; e < E; e++) {
    const size_t n = (size_t)h.cp_nshell[e] * XMI_CP_N;
    if (!(pc[e] = shared_table<R>(h.cp_cdf[e], n)) || !(pq[e] = shared_table<R>(h.cp_qinv[e], n))) return false;
  }
  void *a = nullptr, *q = nullptr;
  if (cudaMalloc(&a, sizeof(const R *) * pc.size()) != cudaSuccess) return false;
  s.allocs.push_back(a);
  if (cudaMalloc(&q, sizeof(const R *) * pq.size()) != cudaSuccess) return false;
  s.allocs.push_back(q);
  cudaMemcpy(a, pc.data(), sizeof(const R *) * pc.size(), cudaMemcpyHostToDevice);
  cudaMemcpy(q, pq.data(), sizeof(const R *) * pq.size(), cudaMemcpyHostToDevice);
  d.cp_nshell = upload_int(s, h.cp_nshell, E);
  d.cp_occ = upload<double>(s, h.cp_occ, (size_t)E * XMI_CP_SH);
  d.cp_edge = upload<double>(s, h.cp_edge, (size_t)E * XMI_CP_SH);
  if (!d.cp_nshell || !d.cp_occ || !d.cp_edge || cudaGetLastError() != cudaSuccess) return false;
  d.cp_cdf = (const R *const *)a;
  d.cp_qinv = (const R *const *)q;
  return true;
}


const double *upload_d(DevSide &s, const double *src, size_t n) {
  if (n == 0) n = 1;
  void *p = nullptr;
  if (cudaMalloc(&p, sizeof(double) * n) != cudaSuccess) return nullptr;
  s.allocs.push_back(p);
  if (src) cudaMemcpy(p, src, sizeof(double) * n, cudaMemcpyHostToDevice);
  return (const double *)p;
}

/* fills the scalar part of a DevBundle from the host bundle */
template <typename R>
void fill_scalars(const xmi_bundle &h, xmi::DevBundle<R> &d) {
  d.N = h.n_interactions;
  d.nch = h.nchannels;
  d.use_vr = h.use_vr;
  d.use_M_lines = h.use_M_lines;
  d.use_adv_compton = h.use_advanced_compton && d.cp_cdf ? 1 : 0;
  {
    const bool analog = h.use_vr == 0 && h.escape_mode == 0;
    d.casc_auger = analog && (h.cascade_type == XMI_CASCADE_NONRADIATIVE || h.cascade_type == XMI_CASCADE_FULL);
    d.casc_rad = analog && (h.cascade_type == XMI_CASCADE_RADIATIVE || h.cascade_type == XMI_CASCADE_FULL);
  }
  d.line_last = h.line_last;
  d.max_shell = h.max_shell;
  d.escape_mode = h.escape_mode;
  d.n_layers = h.n_layers;
  d.n_elem = h.n_elem;
  d.n_lines = h.n_lines;
  d.n_slots = h.n_slots;
  d.n_nodes = h.n_nodes;
  d.n_seg = h.n_seg;
  d.n_items = h.n_items;
  d.n_layer_el = h.n_layer_el;
  d.n_ent = h.n_ent;
  d.stage_max = h.stage_max;
  d.coll_present = h.coll_present;
  d.seed = h.seed;
  d.n_photons_total = h.n_photons_total;
  d.gain = h.gain;
  d.zero = h.zero;
  for (int k = 0; k < 3; k++) {
    d.n_sample[k] = h.n_sample[k];
    d.p_det[k] = h.p_det[k];
    d.n_det[k] = h.n_det[k];
  }
  for (int k = 0; k < 9; k++) {
    d.det_new[k] = h.det_new[k];
    d.det_inv[k] = h.det_inv[k];
  }
  d.det_radius = h.det_radius;
  d.det_radius_r = (R)h.det_radius;
  d.zero_r = (R)h.zero;
  d.inv_gain_r = (R)(1.0 / h.gain);
  for (int k = 0; k < 3; k++) {
    d.n_sample_r[k] = (R)h.n_sample[k];
    d.n_det_r[k] = (R)h.n_det[k];
  }
  for (int k = 0; k < 9; k++) {
    d.det_new_r[k] = (R)h.det_new[k];
    d.det_inv_r[k] = (R)h.det_inv[k];
  }
  d.coll_radius = h.coll_radius;
  d.coll_height = h.coll_height;
  d.coll_half_apex = h.coll_half_apex;
  d.coll_vertex_x = h.coll_vertex_x;
  d.d_source_slit = h.d_source_slit;
  d.slit_x = h.slit_x;
  d.slit_y = h.slit_y;
  d.slit_ax = std::atan(h.slit_x / h.d_source_slit / 2.0);
  d.slit_ay = std::atan(h.slit_y / h.d_source_slit / 2.0);
  d.slit_ax_r = (R)d.slit_ax;
  d.slit_ay_r = (R)d.slit_ay;
  d.d_source_slit_r = (R)h.d_source_slit;
  d.hbeg0 = h.layer_zbeg[0] * h.n_sample[2];
  for (int j = 0; j < XMI_MAXL; j++) {
    d.zbeg[j] = h.layer_zbeg[j];
    d.zend[j] = h.layer_zend[j];
    d.thick_n[j] = (R)((h.layer_zend[j] - h.layer_zbeg[j]) * h.n_sample[2]);
    d.rho[j] = (R)h.layer_rho[j];
    d.nel[j] = h.layer_nel[j];
    d.off[j] = h.layer_off[j];
  }
}

template <typename R>
bool upload_tables(const xmi_bundle &h, DevSide &s, xmi::DevBundle<R> &d) {
  s.release();
  d.cp_nshell = nullptr;
  d.cp_occ = d.cp_edge = nullptr;
  d.cp_cdf = d.cp_qinv = nullptr;
  fill_scalars(h, d);
  const size_t E = h.n_elem, NL = h.n_lines;
  d.layer_el = upload_int(s, h.layer_el, h.n_layer_el);
  d.layer_w = upload<R>(s, h.layer_w, h.n_layer_el);
  d.elem_Z = upload_int(s, h.elem_Z, E);
  d.yield_corr = upload<R>(s, h.elem_yield_corr, 9 * E);
  d.fluor_yield = upload<R>(s, h.elem_fluor_yield, 9 * E);
  d.ck = upload<R>(s, h.elem_ck, XMI_NCK * E);
  d.line_off = upload_int(s, h.elem_line_off, E + 1);
  d.shell_off = upload_int(s, h.elem_shell_off, 10 * E);
  d.line_index = upload_int(s, h.line_index, NL);
  d.line_shell = upload_int(s, h.line_shell, NL);
  d.line_energy = upload<R>(s, h.line_energy, NL);
  d.line_rate = upload<R>(s, h.line_rate, NL);
  d.precalc_mu = upload<R>(s, h.precalc_mu, (size_t)h.n_layers * NL);
  {
    /* one record per (element, line): the shell factors of an event excited
     * by that line are one 48-byte read instead of nine words n_lines apart */
    std::vector<double> xr(E * (NL > 0 ? NL : 1) * xmi::kXrfRec, 0.0);
    for (size_t e = 0; e < E; e++)
      for (size_t i = 0; i < NL; i++)
        for (int sh = 0; sh < 9; sh++) xr[(e * NL + i) * xmi::kXrfRec + sh] = h.precalc_xrf[(e * 9 + sh) * NL + i];
    d.precalc_xrf = upload<R>(s, xr.data(), xr.size());
  }
  d.seg_lo = upload<R>(s, h.seg_lo, h.n_seg + 1);
  d.seg_lnlo = upload<R>(s, h.seg_lnlo, h.n_seg);
  d.seg_invh = upload<R>(s, h.seg_invh, h.n_seg);
  d.seg_lut = upload_int(s, h.seg_lut, XMI_SEG_LUT);
  d.seg_lut_ln0 = (R)h.seg_lut_ln0;
  d.seg_lut_inv = (R)h.seg_lut_inv;
  d.seg_off = upload_int(s, h.seg_off, h.n_seg);
  d.seg_n = upload_int(s, h.seg_n, h.n_seg);
  {
    const size_t ns = h.n_seg > 0 ? (size_t)h.n_seg : 1;
    std::vector<float4> rec(ns, make_float4(0.f, 0.f, 0.f, 0.f));
    std::vector<int2> on(ns, make_int2(0, 0));
    for (int i = 0; i < h.n_seg; i++) {
      rec[i] = make_float4((float)h.seg_lo[i], (float)h.seg_lo[i + 1], (float)h.seg_lnlo[i], (float)h.seg_invh[i]);
      on[i] = make_int2(h.seg_off[i], h.seg_n[i]);
    }
    d.seg_rec = (const float4 *)upload_bytes(s, rec.data(), sizeof(float4) * ns);
    d.seg_on = (const int2 *)upload_bytes(s, on.data(), sizeof(int2) * ns);
  }
  d.el_tab = upload<R>(s, h.el_tab, E * h.n_nodes * XMI_EL_REC);
  d.mu_tab = upload<R>(s, h.mu_tab, (size_t)h.n_nodes * XMI_MAXL);
  {
    /* running sums in the order and arithmetic of mu_tab's, so a layer's
     * last sum is its mu */
    std::vector<double> cs((size_t)h.n_nodes * (h.n_layer_el > 0 ? h.n_layer_el : 1), 0.0);
    for (int i = 0; i < h.n_nodes; i++)
      for (int j = 0; j < h.n_layers; j++) {
        double mu = 0.0;
        for (int k = 0; k < h.layer_nel[j]; k++) {
          const int p = h.layer_off[j] + k;
          mu += h.el_tab[((size_t)h.layer_el[p] * h.n_nodes + i) * XMI_EL_REC + XMI_REC_TOT] * h.layer_w[p];
          cs[(size_t)i * h.n_layer_el + p] = mu;
        }
      }
    d.layer_cs = upload<R>(s, cs.data(), cs.size());
  }
  d.exc_tab = upload<R>(s, h.exc_tab, h.n_nodes);
  d.icdf_e = upload<R>(s, h.icdf_energies, XMI_ICDF_NE);
  d.icdf_r = upload<R>(s, h.icdf_rs, XMI_ICDF_NR);
  d.rayl_icdf = upload_per_element<R>(s, h.rayl_icdf, (int)E, (size_t)XMI_ICDF_NE * XMI_ICDF_NR);
  d.compt_icdf = upload_per_element<R>(s, h.compt_icdf, (int)E, (size_t)XMI_ICDF_NE * XMI_ICDF_NR);
  d.phi_t = upload<R>(s, h.phi_thetas, XMI_PHI_NT);
  d.phi_icdf = shared_table<R>(h.phi_icdf, (size_t)XMI_PHI_NT * XMI_ICDF_NR);
  d.dop_r = upload<R>(s, h.doppler_rs, XMI_DOPPLER_N);
  d.dop_icdf = upload_per_element<R>(s, h.doppler_icdf, (int)E, XMI_DOPPLER_N);
  d.ff2 = upload_per_element<R>(s, h.ff2, (int)E, XMI_NQ);
  d.sf = upload_per_element<R>(s, h.sf, (int)E, XMI_NQ);
  d.ent_off = upload_int(s, h.ent_off, (size_t)h.n_layer_el + 1);
  d.ent_slot = upload_int(s, h.ent_slot, h.n_ent);
  d.ent_shell = upload_int(s, h.ent_shell, h.n_ent);
  d.ent_coef = upload<R>(s, h.ent_coef, h.n_ent);
  if (sizeof(R) == 4) {
    /* FP32: the line mu scaled by -log2(e), for exp2 in the estimator */
    std::vector<double> pmu2((size_t)h.n_ent * XMI_MAXL);
    for (size_t i = 0; i < pmu2.size(); i++) pmu2[i] = h.ent_pmu ? -1.4426950408889634 * h.ent_pmu[i] : 0.0;
    d.ent_pmu = upload<R>(s, pmu2.data(), pmu2.size());
  } else {
    d.ent_pmu = upload<R>(s, h.ent_pmu, (size_t)h.n_ent * XMI_MAXL);
  }
  d.line_casc = upload_int(s, h.line_casc_shell, NL);
  d.auger_rate = upload<R>(s, h.auger_rate, E * 4 * XMI_AUGER_K);
  if (cudaGetLastError() != cudaSuccess || !d.rayl_icdf || !d.compt_icdf || !d.dop_icdf || !d.ff2 || !d.sf ||
      !d.phi_icdf || !d.ent_pmu || !d.line_casc || !d.auger_rate || !d.layer_cs || !d.seg_rec || !d.seg_on) {
    xmi_set_error("device table upload failed");
    s.release();
    return false;
  }
  s.valid = true;
  return true;
}

DevState *state_of(struct xmi_tables_handle *t) {
  if (!t->dev) {
    DevState *s = new DevState();
    cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    cudaEventCreate(&s->ev0);
    cudaEventCreate(&s->ev1);
    t->dev = s;
  }
  return (DevState *)t->dev;
}

bool ensure_device() {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n < 1) {
    xmi_set_error("no CUDA device available: the engine has no CPU fallback");
    return false;
  }
  return true;
}

int num_sms() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms > 0 ? sms : 1;
}

}  // namespace

extern "C" {

int xmi_dev_sync_tables(struct xmi_tables_handle *t, int precision) {
  if (!ensure_device()) return 0;
  DevState *s = state_of(t);
  if (precision == 0) {
    if (!s->d64.valid && !upload_tables<double>(t->b, s->d64, s->b64)) return 0;
    if (!upload_compton_profiles<double>(t->b, s->d64, s->b64)) {
      xmi_set_error("device upload of the Compton profile tables failed");
      return 0;
    }
    fill_scalars(t->b, s->b64);
  } else {
    if (!s->d32.valid && !upload_tables<float>(t->b, s->d32, s->b32)) return 0;
    if (!upload_compton_profiles<float>(t->b, s->d32, s->b32)) {
      xmi_set_error("device upload of the Compton profile tables failed");
      return 0;
    }
    fill_scalars(t->b, s->b32);
  }
  return 1;
}

int xmi_dev_bundle_copy64(struct xmi_tables_handle *t, void *out) {
  DevState *s = state_of(t);
  if (!s->d64.valid) return 0;
  fill_scalars(t->b, s->b64);
  *(xmi::DevBundle<double> *)out = s->b64;
  return 1;
}

void xmi_dev_free_tables(struct xmi_tables_handle *t) {
  if (!t || !t->dev) return;
  DevState *s = (DevState *)t->dev;
  s->d64.release();
  s->d32.release();
  cudaFree(s->items);
  cudaFree(s->items_f);
  cudaFree(s->item_first);
  cudaFree(s->sa_r);
  cudaFree(s->sa_t);
  cudaFree(s->sa_g64);
  cudaFree(s->sa_g32);
  cudaFree(s->tally);
  cudaFree(s->counters);
  cudaFree(s->d_bundle);
  cudaFree(s->d_tally);
  if (s->ev0) cudaEventDestroy(s->ev0);
  if (s->ev1) cudaEventDestroy(s->ev1);
  if (s->stream) cudaStreamDestroy(s->stream);
  delete s;
  t->dev = nullptr;
}

void xmi_free_hdf5_F(xmi_hdf5FPtr *p) {
  if (!p || !*p) return;
  xmi_dev_free_tables(*p);
  xmi_bundle_free(&(*p)->b);
  free(*p);
  *p = nullptr;
}

#ifdef XMI_CHECKED
/* first bounds violation recorded by the diagnostic build: tag, index, limit, count */
int xmi_gpu_check_record(unsigned long long *out) {
  if (cudaMemcpyFromSymbol(out, xmi::xmi_check_record, sizeof(unsigned long long) * 4) != cudaSuccess) return 0;
  return 1;
}
#endif

int xmi_gpu_last_timing(double *transport_ms, double *total_ms, int *launches) {
  if (transport_ms) *transport_ms = g_timing.transport_ms;
  if (total_ms) *total_ms = g_timing.total_ms;
  if (launches) *launches = g_timing.launches;
  return 1;
}

int xmi_gpu_last_graph(int *updated) {
  if (updated) *updated = g_timing.graph_updated;
  return 1;
}

int xmi_gpu_last_phases(double *transport_kernel_ms, double *sort_ms, double *estimator_ms, long long *events) {
  if (transport_kernel_ms) *transport_kernel_ms = g_timing.phase_ms[0];
  if (sort_ms) *sort_ms = g_timing.phase_ms[1];
  if (estimator_ms) *estimator_ms = g_timing.phase_ms[3];
  if (events) *events = g_timing.events;
  return 1;
}

int xmi_gpu_last_transfers(long long *h2d_bytes, long long *d2h_bytes) {
  if (h2d_bytes) *h2d_bytes = g_timing.h2d_bytes;
  if (d2h_bytes) *d2h_bytes = g_timing.d2h_bytes;
  return 1;
}

int xmi_gpu_last_surrogate(double *surrogate_ms, long long *fallbacks) {
  if (surrogate_ms) *surrogate_ms = g_timing.phase_ms[2];
  if (fallbacks) *fallbacks = g_timing.surrogate_fallbacks;
  return 1;
}

/* ---------------------------------------------------------------- */
/* solid angle grid                                                  */
/* ---------------------------------------------------------------- */
static int solid_angle_impl(xmi_inputFPtr in, xmi_solid_angle **out, char *input_string, int precision,
                            unsigned long long seed) {
  if (!in || !out || !in->initialized) {
    xmi_set_error("xmi_solid_angle_calculation: input not initialised");
    return 0;
  }
  /* the reference's grid is 1024 x 1024 (src/xmi_solid_angle_f.F90:62-301) */
  const int nr = in->gpu.grid_nr > 0 ? in->gpu.grid_nr : 1024, nt = in->gpu.grid_nt > 0 ? in->gpu.grid_nt : 1024;
  if (nr < 2 || nt < 2 || (long long)nr * nt > (1ll << 28)) {
    xmi_set_error("xmi_solid_angle_calculation: grid of %d x %d points out of range", nr, nt);
    return 0;
  }
  if (!ensure_device()) return 0;
  xmi_solid_angle *sa = (xmi_solid_angle *)calloc(1, sizeof(xmi_solid_angle));
  sa->grid_dims_r_n = nr;
  sa->grid_dims_theta_n = nt;
  sa->grid_dims_r_vals = (double *)malloc(sizeof(double) * nr);
  sa->grid_dims_theta_vals = (double *)malloc(sizeof(double) * nt);
  sa->solid_angles = (double *)malloc(sizeof(double) * nr * nt);
  sa->xmi_input_string = input_string ? strdup(input_string) : nullptr;
  xmi_solid_angle_axes(in, nr, nt, sa->grid_dims_r_vals, sa->grid_dims_theta_vals);

  double *dr = nullptr, *dt = nullptr, *dout = nullptr;
  bool ok = cuda_ok(cudaMalloc(&dr, sizeof(double) * nr), "cudaMalloc") &&
            cuda_ok(cudaMalloc(&dt, sizeof(double) * nt), "cudaMalloc") &&
            cuda_ok(cudaMalloc(&dout, sizeof(double) * nr * nt), "cudaMalloc");
  if (ok) {
    cudaMemcpy(dr, sa->grid_dims_r_vals, sizeof(double) * nr, cudaMemcpyHostToDevice);
    cudaMemcpy(dt, sa->grid_dims_theta_vals, sizeof(double) * nt, cudaMemcpyHostToDevice);
    xmi::SaGeom g{in->det_radius, in->coll_radius, in->coll_height, in->coll_present};
    int blocks = num_sms() * 8;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0);
    if (precision == 0)
      xmi::solid_angle_grid_kernel<double><<<blocks, 256>>>(g, dr, nr, dt, 0, (long long)nr * nt,
                                                              (int)hits_per_single, seed, in->gpu.solid_angle_stream,
                                                              dout);
    else
      xmi::solid_angle_grid_kernel<float><<<blocks, 256>>>(g, dr, nr, dt, 0, (long long)nr * nt,
                                                             (int)hits_per_single, seed, in->gpu.solid_angle_stream,
                                                             dout);
    cudaEventRecord(e1);
    ok = cuda_ok(cudaGetLastError(), "solid_angle_grid_kernel") && cuda_ok(cudaEventSynchronize(e1), "sync");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    g_timing.transport_ms = ms;
    g_timing.total_ms = ms;
    g_timing.launches = 1;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (ok) ok = cuda_ok(cudaMemcpy(sa->solid_angles, dout, sizeof(double) * nr * nt, cudaMemcpyDeviceToHost), "copy");
  }
  cudaFree(dr);
  cudaFree(dt);
  cudaFree(dout);
  if (!ok) {
    xmi_free_solid_angle(sa);
    return 0;
  }
  *out = sa;
  return 1;
}

static unsigned long long sa_seed(xmi_inputFPtr in, xmi_main_options *options) {
  if (in && in->gpu.seed) return in->gpu.seed;
  if (options && options->use_default_seeds) return 0x5EED0001ull;
  unsigned long long s = 0;
  FILE *f = fopen("/dev/urandom", "rb");
  if (f) {
    if (fread(&s, sizeof(s), 1, f) != 1) s = 0;
    fclose(f);
  }
  return s ? s : 0x5EED0001ull;
}

int xmi_solid_angle_calculation_cuda(xmi_inputFPtr inputFPtr, xmi_solid_angle **solid_angle, char *input_string,
                                     xmi_main_options *options) {
  return solid_angle_impl(inputFPtr, solid_angle, input_string, inputFPtr ? inputFPtr->gpu.precision : 0,
                          sa_seed(inputFPtr, options));
}

void xmi_solid_angle_calculation(xmi_inputFPtr inputFPtr, xmi_solid_angle **solid_angle, char *input_string,
                                 xmi_main_options *options) {
  if (!xmi_solid_angle_calculation_cuda(inputFPtr, solid_angle, input_string, options)) *solid_angle = nullptr;
}

void xmi_free_solid_angle(xmi_solid_angle *sa) {
  if (!sa) return;
  free(sa->solid_angles);
  free(sa->grid_dims_r_vals);
  free(sa->grid_dims_theta_vals);
  free(sa->xmi_input_string);
  free(sa);
}

/* ---------------------------------------------------------------- */
/* transport                                                         */
/* ---------------------------------------------------------------- */
static int attach_solid_angles(struct xmi_tables_handle *t, xmi_solid_angle *sa) {
  xmi_bundle *b = &t->b;
  if (!sa || !sa->solid_angles) {
    b->sa_nr = b->sa_nt = 0;
    return 1;
  }
  b->sa_nr = (int)sa->grid_dims_r_n;
  b->sa_nt = (int)sa->grid_dims_theta_n;
  b->sa_r = sa->grid_dims_r_vals;
  b->sa_t = sa->grid_dims_theta_vals;
  b->sa_grid = sa->solid_angles;
  b->sa_hits_per_single = (int)hits_per_single;
  return 1;
}

static int prepare_run(xmi_inputFPtr in, xmi_hdf5FPtr t, xmi_main_options *options, int n_mpi_hosts,
                       xmi_solid_angle *sa, bool need_solid_angles);

int xmi_gpu_prepare_run(xmi_inputFPtr in, xmi_hdf5FPtr t, xmi_main_options *options, int n_mpi_hosts,
                        xmi_solid_angle *sa) {
  return prepare_run(in, t, options, n_mpi_hosts, sa, true);
}
}  // extern "C"

static int prepare_run(xmi_inputFPtr in, xmi_hdf5FPtr t, xmi_main_options *options, int n_mpi_hosts,
                       xmi_solid_angle *sa, bool need_solid_angles) {
  if (!in || !t || !options) {
    xmi_set_error("xmi_gpu_prepare_run: NULL argument");
    return 0;
  }
  int cascade;
  if (options->use_cascade_auger == 0 && options->use_cascade_radiative == 0) cascade = XMI_CASCADE_NONE;
  else if (options->use_cascade_auger == 1 && options->use_cascade_radiative == 0) cascade = XMI_CASCADE_NONRADIATIVE;
  else if (options->use_cascade_auger == 0 && options->use_cascade_radiative == 1) cascade = XMI_CASCADE_RADIATIVE;
  else cascade = XMI_CASCADE_FULL;
  if (cascade != t->cascade_type || options->use_M_lines != t->use_M_lines) {
    /* tables depend on the cascade type and M-line option: rebuild */
    xmi_dev_free_tables(t);
    xmi_bundle_free(&t->b);
    if (!xmi_bundle_build(in, t, options)) return 0;
  }
  {
    /* n_mpi_hosts > 1 keeps the reference's per-host share n/n_mpi_hosts */
    int R = t->n_replicas > 0 ? t->n_replicas : 1, r = t->replica;
    if (n_mpi_hosts > R) R = n_mpi_hosts;
    if (r >= R) r = R - 1;
    xmi_bundle_set_run(in, t, options, n_mpi_hosts, r, R);
  }
  /* per-shell Compton profiles of the advanced Compton scattering */
  if (options->use_advanced_compton == 1 && !xmi_bundle_compton_profiles(&t->b)) return 0;
  attach_solid_angles(t, sa);
  if (need_solid_angles && options->use_variance_reduction && (!sa || !sa->solid_angles) &&
      !(in->gpu.use_surrogate && in->surrogate)) {
    xmi_set_error("variance reduction requires a solid angle grid (or a trained surrogate with use_surrogate = 1)");
    return 0;
  }
  return 1;
}

/* the estimator's solid angles come from the input's trained surrogate */
static bool surrogate_in_use(xmi_inputFPtr in, const xmi_main_options *options) {
  return in && in->gpu.use_surrogate && in->surrogate && options && options->use_variance_reduction == 1;
}

/* events held on the device per chunk; a chunk is as many photons as can
 * each make N estimator events (one per interaction) within it */
constexpr long long kMaxQueuedEvents = 1ll << 25;
static long long queue_events_of(const xmi_gpu_options &g) {
  return g.queue_events >= (1ll << 16) && g.queue_events <= (1ll << 27) ? g.queue_events : kMaxQueuedEvents;
}
/* photons per chunk without variance reduction (wavefront state ~170 B each) */
constexpr long long kMaxChunkPhotons = 1ll << 23;

template <typename R>
static bool ensure_wf(WfBuffers &wb, long long cap) {
  const size_t bytes = (size_t)cap * sizeof(xmi::WfPhoton<R>);
  if (bytes <= wb.st_bytes && cap <= wb.cap) return true;
  wb.release();
  if (!cuda_ok(cudaMalloc(&wb.st, bytes), "cudaMalloc photon states") ||
      !cuda_ok(cudaMalloc(&wb.lists, sizeof(int) * 5 * cap), "cudaMalloc photon lists") ||
      !cuda_ok(cudaMalloc(&wb.count, sizeof(unsigned) * 5), "cudaMalloc") ||
      !cuda_ok(cudaMalloc(&wb.casc, (size_t)cap), "cudaMalloc cascade flags"))
    return false;
  wb.st_bytes = bytes;
  wb.cap = cap;
  return true;
}

/* the wavefront transport of work indices [w0, w1): start, then max_iter
 * rounds of step + the three interaction kernels; returns the launches */
template <typename R, bool Batched>
static int launch_wavefront(cudaStream_t st, WfBuffers &wb, const xmi::DevBundle<R> &b0, const xmi::DevTally &t0,
                            const xmi::DevBundle<R> *bundles, const xmi::DevTally *tallies, const long long *cfg_first,
                            int n_cfg, long long w0, long long w1, int max_iter, const xmi::VrQueue<R> &vq,
                            int threads, int blocks, bool adv, bool casc) {
  const long long cap = wb.cap;
  xmi::WfLists q;
  q.active[0] = wb.lists;
  q.active[1] = wb.lists + cap;
  for (int k = 0; k < 3; k++) q.inter[k] = wb.lists + (2 + k) * cap;
  q.count = wb.count;
  /* analog cascades: photons in [0, cap / 2), offspring in [cap / 2, cap) */
  q.casc = wb.casc;
  q.half = casc ? cap / 2 : cap;
  xmi::WfPhoton<R> *ps = (xmi::WfPhoton<R> *)wb.st;
  cudaMemsetAsync(wb.count, 0, sizeof(unsigned) * 5, st);
  if (casc) cudaMemsetAsync(wb.casc, 0, (size_t)q.half, st);
  xmi::wf_start<R, Batched><<<blocks, threads, 0, st>>>(b0, t0, bundles, tallies, cfg_first, n_cfg, w0, w1, ps, q);
  int launches = 1, cur = 0;
  for (int it = 0; it < max_iter; it++) {
    const int next = cur ^ 1;
    xmi::wf_reset<<<1, 32, 0, st>>>(q, next);
    xmi::wf_step<R, Batched><<<blocks, threads, 0, st>>>(b0, t0, bundles, tallies, ps, q, cur, cap, vq);
    for (int k = 0; k < 3; k++) {
      if (k == 1 && adv)
        xmi::wf_interact<R, Batched, true><<<blocks, threads, 0, st>>>(b0, t0, bundles, tallies, ps, q, k, next, cap);
      else if (k == 2 && casc)
        xmi::wf_interact<R, Batched, false, true><<<blocks, threads, 0, st>>>(b0, t0, bundles, tallies, ps, q, k, next,
                                                                             cap);
      else
        xmi::wf_interact<R, Batched><<<blocks, threads, 0, st>>>(b0, t0, bundles, tallies, ps, q, k, next, cap);
    }
    launches += 5;
    cur = next;
  }
  return launches;
}

/* rounds of the wavefront: with variance reduction every photon interacts at
 * most N times (N + 1 steps); analog histories end within the guard of the
 * history loop */
static int wavefront_rounds(const xmi_bundle &h) { return h.use_vr ? h.n_interactions + 1 : 4 * XMI_MAXN + 8; }

template <typename R>
static bool ensure_queue(EventQueue &eq, QueueBufs &q, long long cap, int nkeys) {
  const size_t bytes = (size_t)cap * sizeof(xmi::VrEvent<R>);
  if (bytes > q.bytes || cap > q.cap) {
    eq.drop_exec();
    cudaFree(q.events);
    cudaFree(q.key);
    cudaFree(q.order);
    cudaFree(q.fb);
    q.events = nullptr;
    q.key = q.order = q.fb = nullptr;
    q.bytes = 0;
    q.cap = 0;
    if (!cuda_ok(cudaMalloc(&q.events, bytes), "cudaMalloc event queue") ||
        !cuda_ok(cudaMalloc(&q.key, sizeof(int) * cap), "cudaMalloc event keys") ||
        !cuda_ok(cudaMalloc(&q.order, sizeof(int) * cap), "cudaMalloc event order") ||
        !cuda_ok(cudaMalloc(&q.fb, sizeof(int) * cap), "cudaMalloc fallback list"))
      return false;
    q.bytes = bytes;
    q.cap = cap;
  }
  if (nkeys > q.nkeys) {
    eq.drop_exec();
    cudaFree(q.hist);
    q.hist = nullptr;
    q.nkeys = 0;
    if (!cuda_ok(cudaMalloc(&q.hist, 2 * sizeof(unsigned) * nkeys), "cudaMalloc key histogram")) return false;
    q.nkeys = nkeys;
  }
  if (!q.count && !cuda_ok(cudaMalloc(&q.count, 3 * sizeof(unsigned long long)), "cudaMalloc")) return false;
  return true;
}

struct Phases {
  double ms[4] = {0.0, 0.0, 0.0, 0.0}; /* transport kernel, event sort, surrogate solid angles, estimator kernel */
  double total_ms = 0.0;
  int launches = 0;
};

/* Runs work indices [0, n) in chunks on stream st: per chunk the transport
 * launch (events into an event queue), the counting sort of the events by
 * key, the solid angles of the events and the estimator launch.  With
 * variance reduction and more than one chunk (and overlap set), two event
 * queues alternate: chunk k's sort, solid angles and estimator run on a
 * second stream while chunk k+1's transport fills the other queue on st;
 * a queue is refilled once the estimator that read it is done.  CUDA events
 * around each phase give its device time (with overlap, phases of different
 * chunks run at the same time, so their sum exceeds the total).
 * transport(stream, w0, w1, vq), surrogate(stream, vq, fb, fb_count) and
 * estimator(stream, vq, order, work) enqueue the phases. */
template <typename R, typename TF, typename SF, typename EF>
static bool run_chunks(cudaStream_t st, EventQueue &q, long long n, int N, int nkeys, bool vr, long long qev,
                       unsigned long long *total_events, TF &&transport, SF &&surrogate, EF &&estimator, Phases &ph,
                       bool graph = false, bool overlap = false) {
  const int sms = num_sms();
  long long chunk = n < kMaxChunkPhotons ? n : kMaxChunkPhotons;
  if (chunk < 1) chunk = 1;
  long long cap = 0;
  if (vr) {
    chunk = qev / (N > 0 ? N : 1);
    if (chunk > n) chunk = n;
    if (chunk < 1) chunk = 1;
    cap = chunk * N;
  }
  const bool two = vr && overlap && n > chunk;
  if (vr) {
    if (!ensure_queue<R>(q, q.buf[0], cap, nkeys)) return false;
    if (two && (!ensure_queue<R>(q, q.buf[1], cap, nkeys) || !q.ensure_side())) {
      xmi_set_error("second event queue or stream could not be created");
      return false;
    }
  }
  cudaStream_t as = two ? q.side : st; /* stream of the phases after transport */
  /* under stream capture an event record must be marked external to become a
   * real record when the graph runs (so that it can be timed and waited on) */
  size_t n_marks = 0;
  auto mark = [&](cudaStream_t s) {
    if (n_marks == q.marks.size()) {
      cudaEvent_t e;
      cudaEventCreate(&e);
      q.marks.push_back(e);
    }
    cudaEvent_t e = q.marks[n_marks++];
    if (graph) cudaEventRecordWithFlags(e, s, cudaEventRecordExternal);
    else cudaEventRecord(e, s);
  };
  int launches = 0;
  cudaGraph_t g = nullptr;
  if (graph && !cuda_ok(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "graph capture")) return false;
  mark(st);
  long long k = 0;
  for (long long w0 = 0; w0 < n; w0 += chunk, k++) {
    const long long w1 = w0 + chunk < n ? w0 + chunk : n;
    const int qi = two ? (int)(k & 1) : 0;
    QueueBufs &qb = q.buf[qi];
    xmi::VrQueue<R> vq{nullptr, nullptr, nullptr, 0};
    if (vr) {
      vq.ev = (xmi::VrEvent<R> *)qb.events;
      vq.key = qb.key;
      vq.count = qb.count;
      vq.cap = cap;
      /* the queue's previous chunk must be through its estimator */
      if (two && k >= 2) cudaStreamWaitEvent(st, q.drained[qi], 0);
      cudaMemsetAsync(qb.count, 0, sizeof(unsigned long long), st);
      cudaMemsetAsync(qb.hist, 0, sizeof(unsigned) * nkeys, st);
    }
    mark(st);
    launches += transport(st, w0, w1, vq);
    mark(st);
    if (vr) {
      if (two) {
        cudaEventRecord(q.filled[qi], st);
        cudaStreamWaitEvent(as, q.filled[qi], 0);
      }
      mark(as);
      /* positions of events whose key the sort would skip stay -1 and are refused by the estimator */
      cudaMemsetAsync(qb.order, 0xff, sizeof(int) * (w1 - w0) * N, as);
      xmi::event_key_histogram<<<sms * 8, 256, 0, as>>>(qb.key, qb.count, cap, nkeys, qb.hist);
      xmi::event_key_scan<<<1, xmi::kScanThreads, 0, as>>>(qb.hist, nkeys, qb.hist + nkeys, qb.count, total_events);
      xmi::event_key_scatter<<<sms * 8, 256, 0, as>>>(qb.key, qb.count, cap, nkeys, qb.hist + nkeys, qb.order);
      cudaMemsetAsync(qb.count + 1, 0, 2 * sizeof(unsigned long long), as);
      mark(as);
      launches += surrogate(as, vq, qb.fb, qb.count + 2);
      mark(as);
      estimator(as, vq, (const int *)qb.order, qb.count + 1);
      mark(as);
      launches += 4;
      if (two) cudaEventRecord(q.drained[qi], as);
    }
    if (!cuda_ok(cudaGetLastError(), "transport launch")) break;
  }
  if (two) {
    cudaEventRecord(q.joined, as);
    cudaStreamWaitEvent(st, q.joined, 0);
  }
  mark(st);
  bool ok = cuda_ok(cudaGetLastError(), "transport launch");
  if (graph) {
    /* the whole chunk sequence as one graph launch; the executable graph of
     * the previous call is updated with this capture's parameters (buffers,
     * counts, timing events) when the sequence has the same shape, and
     * instantiated anew otherwise */
    ok = cuda_ok(cudaStreamEndCapture(st, &g), "graph capture") && ok;
    if (ok) {
      bool updated = false;
      int status = 0;
      if (q.exec) {
        cudaGraphExecUpdateResultInfo info;
        updated = cudaGraphExecUpdate(q.exec, g, &info) == cudaSuccess;
        if (!updated) {
          (void)cudaGetLastError(); /* a different shape: not an error */
          q.drop_exec();
          status = 100 + (int)info.result;
        }
      }
      if (!updated) ok = cuda_ok(cudaGraphInstantiate(&q.exec, g, 0), "graph instantiate");
      if (ok) {
        g_timing.graph_updated = updated ? 1 : status;
        ok = cuda_ok(cudaGraphLaunch(q.exec, st), "graph launch");
      }
    }
  }
  std::vector<cudaEvent_t> marks(q.marks.begin(), q.marks.begin() + n_marks);
  ok = ok && cuda_ok(cudaEventSynchronize(marks.back()), "transport");
  if (g) cudaGraphDestroy(g);
  if (ok) {
    /* marks: start, per chunk (transport begin, end[, sort begin, sort end,
     * solid angles end, estimator end]), end */
    float total = 0.f;
    cudaEventElapsedTime(&total, marks.front(), marks.back());
    ph.total_ms = total;
    const size_t per = vr ? 6 : 2;
    for (size_t i = 1; i + per < marks.size(); i += per) {
      float f = 0.f;
      cudaEventElapsedTime(&f, marks[i], marks[i + 1]);
      ph.ms[0] += f;
      for (size_t k2 = 0; vr && k2 < 3; k2++) {
        cudaEventElapsedTime(&f, marks[i + 2 + k2], marks[i + 3 + k2]);
        ph.ms[1 + k2] += f;
      }
    }
    ph.launches = launches;
  }
  return ok;
}

/* Uploads what one run of a configuration needs besides its tables (source
 * items, solid-angle grid), clears its tallies and fills the run fields of
 * its device bundle and tally view.  Copies go to the handle's stream. */
template <typename R>
static bool stage_run(DevState *s, xmi::DevBundle<R> &d, const xmi_bundle &h, xmi::DevTally &tl, bool surrogate) {
  std::vector<long long> first(h.n_items > 0 ? h.n_items : 1, 0);
  for (int i = 1; i < h.n_items; i++) first[i] = first[i - 1] + h.items[i - 1].n_photons;
  if (h.n_items > s->items_cap) {
    cudaFree(s->items);
    cudaFree(s->items_f);
    cudaFree(s->item_first);
    s->items = nullptr;
    s->items_f = nullptr;
    s->item_first = nullptr;
    s->items_cap = 0;
    if (!cuda_ok(cudaMalloc(&s->items, sizeof(xmi_source_item) * h.n_items), "cudaMalloc items") ||
        !cuda_ok(cudaMalloc(&s->items_f, sizeof(xmi::ItemF) * h.n_items), "cudaMalloc items") ||
        !cuda_ok(cudaMalloc(&s->item_first, sizeof(long long) * h.n_items), "cudaMalloc items"))
      return false;
    s->items_cap = h.n_items;
  }
  if (h.n_items > 0) {
    std::vector<xmi::ItemF> items_f(h.n_items);
    for (int i = 0; i < h.n_items; i++) items_f[i] = xmi::item_f_of(h.items[i]);
    cudaMemcpyAsync(s->items, h.items, sizeof(xmi_source_item) * h.n_items, cudaMemcpyHostToDevice, s->stream);
    cudaMemcpyAsync(s->items_f, items_f.data(), sizeof(xmi::ItemF) * h.n_items, cudaMemcpyHostToDevice, s->stream);
    cudaMemcpyAsync(s->item_first, first.data(), sizeof(long long) * h.n_items, cudaMemcpyHostToDevice, s->stream);
    g_timing.h2d_bytes += (long long)(sizeof(xmi_source_item) + sizeof(xmi::ItemF) + sizeof(long long)) * h.n_items;
  }
  /* solid-angle grid (kept on the device while the caller's grid is the same) */
  if (h.sa_nr > 0 && (s->sa_src != h.sa_grid || s->sa_n != h.sa_nr * h.sa_nt)) {
    size_t n = (size_t)h.sa_nr * h.sa_nt;
    cudaFree(s->sa_r);
    cudaFree(s->sa_t);
    cudaFree(s->sa_g64);
    cudaFree(s->sa_g32);
    s->sa_r = s->sa_t = s->sa_g64 = nullptr;
    s->sa_g32 = nullptr;
    s->sa_src = nullptr;
    if (!cuda_ok(cudaMalloc(&s->sa_r, sizeof(double) * h.sa_nr), "cudaMalloc") ||
        !cuda_ok(cudaMalloc(&s->sa_t, sizeof(double) * h.sa_nt), "cudaMalloc") ||
        !cuda_ok(cudaMalloc(&s->sa_g64, sizeof(double) * n), "cudaMalloc") ||
        !cuda_ok(cudaMalloc(&s->sa_g32, sizeof(float) * n), "cudaMalloc"))
      return false;
    std::vector<float> g32(n);
    for (size_t i = 0; i < n; i++) g32[i] = (float)h.sa_grid[i];
    cudaMemcpy(s->sa_r, h.sa_r, sizeof(double) * h.sa_nr, cudaMemcpyHostToDevice);
    cudaMemcpy(s->sa_t, h.sa_t, sizeof(double) * h.sa_nt, cudaMemcpyHostToDevice);
    cudaMemcpy(s->sa_g64, h.sa_grid, sizeof(double) * n, cudaMemcpyHostToDevice);
    cudaMemcpy(s->sa_g32, g32.data(), sizeof(float) * n, cudaMemcpyHostToDevice);
    g_timing.h2d_bytes += (long long)(sizeof(double) * (h.sa_nr + h.sa_nt + n) + sizeof(float) * n);
    s->sa_src = h.sa_grid;
    s->sa_n = (int)n;
  }
  const size_t nh = (size_t)h.n_interactions * h.n_slots;
  const size_t nc = (size_t)(h.n_interactions + 1) * h.nchannels;
  const size_t need = 2 * nh + nc;
  if (need > s->tally_cap) {
    cudaFree(s->tally);
    s->tally = nullptr;
    s->tally_cap = 0;
    if (!cuda_ok(cudaMalloc(&s->tally, need * sizeof(double)), "cudaMalloc tally")) return false;
    s->tally_cap = need;
  }
  if (!s->counters && !cuda_ok(cudaMalloc(&s->counters, 8 * sizeof(unsigned long long)), "cudaMalloc")) return false;
  cudaMemsetAsync(s->tally, 0, need * sizeof(double), s->stream);
  cudaMemsetAsync(s->counters, 0, 8 * sizeof(unsigned long long), s->stream);
  tl.hist_vr = s->tally;
  tl.hist_brute = s->tally + nh;
  tl.chan = s->tally + 2 * nh;
  tl.counters = s->counters;
  d.items = s->items;
  d.items_f = s->items_f;
  d.item_first = s->item_first;
  d.sa_r = s->sa_r;
  d.sa_t = s->sa_t;
  d.sa_nr = h.sa_nr;
  d.sa_nt = h.sa_nt;
  d.sa_hits = h.sa_hits_per_single > 0 ? h.sa_hits_per_single : (int)hits_per_single;
  d.use_surrogate = surrogate ? 1 : 0;
  if (h.sa_nr > 1) {
    d.sa_r0 = h.sa_r[0];
    d.sa_rinv = (h.sa_nr - 1) / (h.sa_r[h.sa_nr - 1] - h.sa_r[0]);
    d.sa_t0 = h.sa_t[0];
    d.sa_tinv = (h.sa_nt - 1) / (h.sa_t[h.sa_nt - 1] - h.sa_t[0]);
  }
  if (sizeof(R) == 8) d.sa_grid = (const R *)s->sa_g64;
  else d.sa_grid = (const R *)s->sa_g32;
  return true;
}

/* stage rows of the estimator: values per warp row, capped so that the eight
 * rows of a CTA fit shared memory (layers that need more run per-lane) */
template <typename R>
static int stage_cap_for(int stage_max) {
  /* a multiple of 4 values, so that each warp's scratch (after its stage
   * row) starts on 16 bytes for the line loop's vector reads */
  const int limit = ((int)(200 * 1024 / (8 * sizeof(R))) - xmi::kScratchPerWarp) & ~3;
  const int cap = (stage_max + 3) & ~3;
  return cap < limit ? cap : limit;
}

template <typename R, bool Adv = false>
static int estimator_blocks(int stage_cap, size_t *smem, int cap_per_sm = 0) {
  *smem = (size_t)8 * (stage_cap + xmi::kScratchPerWarp) * sizeof(R);
  if (*smem > 48 * 1024)
    cudaFuncSetAttribute(xmi::estimator_kernel<R, Adv>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)*smem);
  int per_sm = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, xmi::estimator_kernel<R, Adv>, 256, *smem);
  if (cap_per_sm > 0 && per_sm > cap_per_sm) per_sm = cap_per_sm;
  if (per_sm < 1) per_sm = 1;
  return num_sms() * per_sm;
}

/* one configuration on its handle's stream */
/* Records the (r, theta) of a pseudo-random share p of the queued estimator
 * events (selected by a hash of photon id and order, so the selection does
 * not depend on the queue's order) -- the points a surrogate network will be
 * queried at. */
struct PointRecorder {
  double p = 0.0;
  float *r = nullptr, *t = nullptr;
  unsigned long long *n = nullptr;
  long long max = 0;
};

__device__ __forceinline__ double event_hash01(long long id, int n) {
  unsigned long long z = (unsigned long long)id * 0x9E3779B97F4A7C15ull + (unsigned long long)n * 0xD1B54A32D192ED03ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

template <typename R>
__global__ void record_points_kernel(const xmi::VrEvent<R> *ev, const unsigned long long *count, long long cap,
                                     double p, float *out_r, float *out_t, unsigned long long *out_n,
                                     long long max_out) {
  const long long n = (long long)*count < cap ? (long long)*count : cap;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    if (event_hash01(ev[i].id, ev[i].n) >= p) continue;
    const unsigned long long pos = atomicAdd(out_n, 1ull);
    if ((long long)pos < max_out) {
      out_r[pos] = (float)ev[i].sa_r;
      out_t[pos] = (float)ev[i].sa_t;
    }
  }
}

template <typename R>
static bool launch_single(DevState *s, xmi::DevBundle<R> &d, const xmi::DevTally &tl, const xmi_bundle &h,
                          int threads, int blocks_per_sm, const xmi_gpu_options &go, const void *sg, Phases &ph,
                          const PointRecorder *rec = nullptr) {
  const long long qev = queue_events_of(go);
  const int sms = num_sms();
  if (!s->d_bundle && !cuda_ok(cudaMalloc(&s->d_bundle, sizeof(xmi::DevBundle<double>)), "cudaMalloc")) return false;
  if (!s->d_tally && !cuda_ok(cudaMalloc(&s->d_tally, sizeof(xmi::DevTally)), "cudaMalloc")) return false;
  cudaMemcpyAsync(s->d_bundle, &d, sizeof(d), cudaMemcpyHostToDevice, s->stream);
  cudaMemcpyAsync(s->d_tally, &tl, sizeof(tl), cudaMemcpyHostToDevice, s->stream);
  g_timing.h2d_bytes += (long long)(sizeof(d) + sizeof(tl));
  const int stage_cap = stage_cap_for<R>(h.stage_max);
  size_t smem = 0;
  const bool adv = d.use_adv_compton != 0;
  const int est_blocks = adv ? estimator_blocks<R, true>(stage_cap, &smem, go.estimator_blocks_per_sm)
                             : estimator_blocks<R>(stage_cap, &smem, go.estimator_blocks_per_sm);
  const long long chunk_cap = h.use_vr ? qev / (h.n_interactions > 0 ? h.n_interactions : 1) : kMaxChunkPhotons;
  /* back to the pool once the run's stream is idle */
  struct Borrow {
    cudaStream_t st;
    RunBuffers *rb = acquire_buffers();
    ~Borrow() {
      cudaStreamSynchronize(st);
      release_buffers(rb);
    }
  } borrow{s->stream};
  EventQueue &q = borrow.rb->q;
  WfBuffers &wf = borrow.rb->wf;
  /* analog cascades: one offspring slot per photon slot */
  const bool casc = d.casc_auger || d.casc_rad;
  if (!ensure_wf<R>(wf, (casc ? 2 : 1) * (h.n_photons_total < chunk_cap ? (h.n_photons_total > 0 ? h.n_photons_total : 1)
                                                                         : chunk_cap)))
    return false;
  const int rounds = wavefront_rounds(h);
  auto transport = [&](cudaStream_t ts, long long w0, long long w1, const xmi::VrQueue<R> &vq) {
    return launch_wavefront<R, false>(ts, wf, d, tl, nullptr, nullptr, nullptr, 1, w0, w1, rounds, vq,
                                      threads, sms * blocks_per_sm, adv, casc);
  };
  auto estimator = [&](cudaStream_t es, const xmi::VrQueue<R> &vq, const int *order, unsigned long long *work) {
    if (adv)
      xmi::estimator_kernel<R, true><<<est_blocks, 256, smem, es>>>(
          (const xmi::DevBundle<R> *)s->d_bundle, s->d_tally, 1, vq.ev, order, vq.count, vq.cap, work, stage_cap,
          &s->counters[1]);
    else
      xmi::estimator_kernel<R><<<est_blocks, 256, smem, es>>>(
          (const xmi::DevBundle<R> *)s->d_bundle, s->d_tally, 1, vq.ev, order, vq.count, vq.cap, work, stage_cap,
          &s->counters[1]);
  };
  auto surrogate = [&](cudaStream_t ss, const xmi::VrQueue<R> &vq, int *fb, unsigned long long *fb_count) -> int {
    if (!d.use_surrogate) {
      /* the grid path: integrals of the events off the grid */
      xmi_solid_angle_deferred(sizeof(R) == 8 ? 0 : 1, s->d_bundle, 1, vq.ev, vq.count, vq.cap, fb, fb_count,
                               ss);
      return 2;
    }
    if (rec) {
      record_points_kernel<R><<<sms * 4, 256, 0, ss>>>(vq.ev, vq.count, vq.cap, rec->p, rec->r, rec->t, rec->n,
                                                               rec->max);
      return 1;
    }
    xmi_surrogate_apply(sg, sizeof(R) == 8 ? 0 : 1, s->d_bundle, 1, vq.ev, vq.count, vq.cap, &s->counters[4], fb,
                        fb_count, (int *)&s->counters[5], ss);
    return 2;
  };
  return run_chunks<R>(s->stream, q, h.n_photons_total, h.n_interactions, XMI_MAXL * XMI_MAXN, h.use_vr != 0,
                       qev, &s->counters[3], transport, surrogate, estimator, ph, false, go.overlap_chunks != 0);
}

/* device tallies -> the reference's output layouts (host) */
static int collect_outputs(DevState *s, const xmi_bundle &h, int n_mpi_hosts, double **channels_out,
                           double **brute_out, double **var_red_out, unsigned long long *events,
                           unsigned long long *fallbacks = nullptr) {
  const int N = h.n_interactions, nch = h.nchannels, S = h.n_slots;
  const size_t nh = (size_t)N * S, nc = (size_t)(N + 1) * nch;
  std::vector<double> tally(2 * nh + nc);
  unsigned long long counters[8];
  cudaMemcpyAsync(tally.data(), s->tally, sizeof(double) * tally.size(), cudaMemcpyDeviceToHost, s->stream);
  cudaMemcpyAsync(counters, s->counters, sizeof(counters), cudaMemcpyDeviceToHost, s->stream);
  g_timing.d2h_bytes += (long long)(sizeof(double) * tally.size() + sizeof(counters));
  if (!cuda_ok(cudaStreamSynchronize(s->stream), "copy back")) return 0;
  if (counters[1] != 0) {
    xmi_set_error("transport kernel reported error code %llu", counters[1]);
    return 0;
  }
  if (counters[5] != 0) {
    xmi_set_error("surrogate solid-angle kernel: tensor-core wait ran out");
    return 0;
  }
  if (events) *events = counters[3];
  if (fallbacks) *fallbacks = counters[4];
  const double *hv = tally.data(), *hb = tally.data() + nh, *chan = tally.data() + 2 * nh;

  /* channels: per-order scatter tallies plus the fluorescence lines derived
   * from the per-order line histories, then cumulative over orders */
  double *channels = (double *)calloc(nc, sizeof(double));
  std::vector<double> per(nc, 0.0);
  for (size_t i = 0; i < nc; i++) per[i] = chan[i];
  if (h.use_vr)
    for (int n = 1; n <= N; n++)
      for (int sl = 0; sl < h.n_lines; sl++) {
        int ch = h.line_channel[sl];
        if (ch >= 0) per[(size_t)n * nch + ch] += hv[(size_t)(n - 1) * S + sl];
      }
  for (int i = 0; i <= N; i++)
    for (int k = 0; k <= i; k++)
      for (int c = 0; c < nch; c++) channels[(size_t)i * nch + c] += per[(size_t)k * nch + c];
  for (size_t i = 0; i < nc; i++) channels[i] *= h.live_time;

  /* histories in the reference layout ((Z-1)*385 + line-1)*N + k-1 */
  const size_t hsz = (size_t)100 * 385 * N;
  double *brute = (double *)calloc(hsz, sizeof(double));
  double *var_red = h.use_vr ? (double *)calloc(hsz, sizeof(double)) : nullptr;
  const double scale = h.live_time * n_mpi_hosts;
  for (int n = 1; n <= N; n++)
    for (int sl = 0; sl < S; sl++) {
      int e, line;
      if (sl < h.n_lines) {
        e = h.line_elem[sl];
        line = h.line_index[sl];
      } else {
        e = (sl - h.n_lines) / 2;
        line = 384 + (sl - h.n_lines) % 2;
      }
      size_t idx = ((size_t)(h.elem_Z[e] - 1) * 385 + (line - 1)) * N + (n - 1);
      brute[idx] = hb[(size_t)(n - 1) * S + sl] * scale;
      if (var_red) var_red[idx] = hv[(size_t)(n - 1) * S + sl] * scale;
    }
  *channels_out = channels;
  *brute_out = brute;
  *var_red_out = var_red;
  return 1;
}

extern "C" int xmi_main_msim(xmi_inputFPtr in, xmi_hdf5FPtr t, int n_mpi_hosts, double **channels_out,
                  xmi_main_options *options, double **brute_out, double **var_red_out, xmi_solid_angle *sa) {
  cudaEvent_t all0, all1;
  if (!ensure_device()) return 0;
  if (!xmi_gpu_prepare_run(in, t, options, n_mpi_hosts, sa)) return 0;
  g_timing.h2d_bytes = g_timing.d2h_bytes = 0;
  g_timing.graph_updated = -1;
  const xmi_bundle &h = t->b;
  const int precision = in->gpu.precision;
  if (!xmi_dev_sync_tables(t, precision)) return 0;
  DevState *s = state_of(t);
  cudaEventCreate(&all0);
  cudaEventCreate(&all1);
  cudaEventRecord(all0, s->stream);
  xmi::DevTally tl;
  const int threads = in->gpu.threads_per_block > 0 ? in->gpu.threads_per_block : 128;
  if (threads > 128 || threads % 32) {
    xmi_set_error("threads_per_block must be a multiple of 32 up to 128 (got %d)", threads);
    return 0;
  }
  const int bps = in->gpu.blocks_per_sm > 0 ? in->gpu.blocks_per_sm : 8;
  Phases ph;
  const bool use_sg = surrogate_in_use(in, options);
  const void *sg = use_sg ? in->surrogate : nullptr;
  bool ok = precision == 0
                ? stage_run<double>(s, s->b64, h, tl, use_sg) &&
                      launch_single<double>(s, s->b64, tl, h, threads, bps, in->gpu, sg, ph)
                : stage_run<float>(s, s->b32, h, tl, use_sg) &&
                      launch_single<float>(s, s->b32, tl, h, threads, bps, in->gpu, sg, ph);
  if (!ok) return 0;
  unsigned long long events = 0, fallbacks = 0;
  if (!collect_outputs(s, h, n_mpi_hosts, channels_out, brute_out, var_red_out, &events, &fallbacks)) return 0;
  cudaEventRecord(all1, s->stream);
  cudaEventSynchronize(all1);
  float tot = 0.f;
  cudaEventElapsedTime(&tot, all0, all1);
  cudaEventDestroy(all0);
  cudaEventDestroy(all1);
  g_timing.transport_ms = ph.total_ms;
  g_timing.total_ms = tot;
  g_timing.launches = ph.launches;
  for (int k = 0; k < 4; k++) g_timing.phase_ms[k] = ph.ms[k];
  g_timing.events = (long long)events;
  g_timing.surrogate_fallbacks = (long long)fallbacks;
  return 1;
}

/* ---------------------------------------------------------------- */
/* batched runs                                                       */
/* ---------------------------------------------------------------- */
namespace {
template <typename R> xmi::DevBundle<R> &dev_bundle_of(DevState *s);
template <> xmi::DevBundle<double> &dev_bundle_of<double>(DevState *s) { return s->b64; }
template <> xmi::DevBundle<float> &dev_bundle_of<float>(DevState *s) { return s->b32; }

/* device arrays of the batched call, kept while large enough */
struct BatchState {
  void *bundles = nullptr;
  size_t bundles_bytes = 0;
  xmi::DevTally *tallies = nullptr;
  long long *cfg_first = nullptr;
  int cap = 0;
  unsigned long long *flags = nullptr; /* [0] estimator error, [1] events */
  EventQueue q;
  WfBuffers wf;
  cudaStream_t stream = nullptr;
};
BatchState g_batch;
std::mutex g_batch_lock;

template <typename R>
bool launch_batch(int n, DevState **st, xmi_hdf5FPtr *t, const xmi::DevTally *tl, int threads, int blocks_per_sm,
                  const xmi_gpu_options &go, const void *sg, bool graph, Phases &ph) {
  const long long qev = queue_events_of(go);
  BatchState &B = g_batch;
  std::vector<xmi::DevBundle<R>> bundles(n);
  std::vector<long long> first(n + 1, 0);
  int N = 1;
  bool vr = false;
  for (int c = 0; c < n; c++) {
    bundles[c] = dev_bundle_of<R>(st[c]);
    first[c + 1] = first[c] + t[c]->b.n_photons_total;
    if (t[c]->b.n_interactions > N) N = t[c]->b.n_interactions;
    vr = vr || t[c]->b.use_vr;
  }
  if (!B.stream) cudaStreamCreateWithFlags(&B.stream, cudaStreamNonBlocking);
  if (n > B.cap || sizeof(xmi::DevBundle<R>) * n > B.bundles_bytes) {
    cudaFree(B.bundles);
    cudaFree(B.tallies);
    cudaFree(B.cfg_first);
    B.bundles = nullptr;
    B.tallies = nullptr;
    B.cfg_first = nullptr;
    B.cap = 0;
    B.bundles_bytes = 0;
    if (!cuda_ok(cudaMalloc(&B.bundles, sizeof(xmi::DevBundle<double>) * n), "cudaMalloc bundles") ||
        !cuda_ok(cudaMalloc(&B.tallies, sizeof(xmi::DevTally) * n), "cudaMalloc tallies") ||
        !cuda_ok(cudaMalloc(&B.cfg_first, sizeof(long long) * (n + 1)), "cudaMalloc offsets"))
      return false;
    B.cap = n;
    B.bundles_bytes = sizeof(xmi::DevBundle<double>) * n;
  }
  if (!B.flags && !cuda_ok(cudaMalloc(&B.flags, 4 * sizeof(unsigned long long)), "cudaMalloc")) return false;
  cudaMemcpyAsync(B.bundles, bundles.data(), sizeof(xmi::DevBundle<R>) * n, cudaMemcpyHostToDevice, B.stream);
  cudaMemcpyAsync(B.tallies, tl, sizeof(xmi::DevTally) * n, cudaMemcpyHostToDevice, B.stream);
  cudaMemcpyAsync(B.cfg_first, first.data(), sizeof(long long) * (n + 1), cudaMemcpyHostToDevice, B.stream);
  g_timing.h2d_bytes += (long long)((sizeof(xmi::DevBundle<R>) + sizeof(xmi::DevTally)) * n + sizeof(long long) * (n + 1));
  cudaMemsetAsync(B.flags, 0, 4 * sizeof(unsigned long long), B.stream);
  const xmi::DevBundle<R> *db = (const xmi::DevBundle<R> *)B.bundles;
  const int sms = num_sms();
  int stage_max = 1;
  for (int c = 0; c < n; c++) stage_max = t[c]->b.stage_max > stage_max ? t[c]->b.stage_max : stage_max;
  bool adv = false; /* kernels with the advanced Compton scattering if any configuration uses it */
  for (int c = 0; c < n; c++) adv = adv || (t[c]->b.use_advanced_compton && t[c]->b.cp_nshell);
  const int stage_cap = stage_cap_for<R>(stage_max);
  size_t smem = 0;
  const int est_blocks = adv ? estimator_blocks<R, true>(stage_cap, &smem, go.estimator_blocks_per_sm)
                             : estimator_blocks<R>(stage_cap, &smem, go.estimator_blocks_per_sm);
  int rounds = 1;
  for (int c = 0; c < n; c++) rounds = wavefront_rounds(t[c]->b) > rounds ? wavefront_rounds(t[c]->b) : rounds;
  const long long chunk_cap = vr ? qev / N : kMaxChunkPhotons;
  bool casc = false; /* analog cascades in any configuration: one offspring slot per photon slot */
  for (int c = 0; c < n; c++) {
    const xmi_bundle &hb = t[c]->b;
    casc = casc || (hb.use_vr == 0 && hb.escape_mode == 0 && hb.cascade_type != XMI_CASCADE_NONE);
  }
  if (!ensure_wf<R>(B.wf, (casc ? 2 : 1) * (first[n] < chunk_cap ? (first[n] > 0 ? first[n] : 1) : chunk_cap)))
    return false;
  xmi::DevBundle<R> unused_b{};
  xmi::DevTally unused_t{};
  auto transport = [&](cudaStream_t ts, long long w0, long long w1, const xmi::VrQueue<R> &vq) {
    return launch_wavefront<R, true>(ts, B.wf, unused_b, unused_t, db, B.tallies, B.cfg_first, n, w0, w1,
                                     rounds, vq, threads, sms * blocks_per_sm, adv, casc);
  };
  auto estimator = [&](cudaStream_t es, const xmi::VrQueue<R> &vq, const int *order, unsigned long long *work) {
    if (adv)
      xmi::estimator_kernel<R, true><<<est_blocks, 256, smem, es>>>(db, B.tallies, n, vq.ev, order, vq.count,
                                                                          vq.cap, work, stage_cap, B.flags);
    else
      xmi::estimator_kernel<R><<<est_blocks, 256, smem, es>>>(db, B.tallies, n, vq.ev, order, vq.count, vq.cap,
                                                                    work, stage_cap, B.flags);
  };
  /* flags: [0] estimator error, [1] events, [2] integrator fallbacks of the
   * surrogate, [3] surrogate error */
  auto surrogate = [&](cudaStream_t ss, const xmi::VrQueue<R> &vq, int *fb, unsigned long long *fb_count) -> int {
    /* the integrals of the events off their configuration's grid first (a
     * configuration served by the network leaves none), then the network */
    xmi_solid_angle_deferred(sizeof(R) == 8 ? 0 : 1, db, n, vq.ev, vq.count, vq.cap, fb, fb_count, ss);
    if (!sg) return 2;
    cudaMemsetAsync(fb_count, 0, sizeof(unsigned long long), ss);
    xmi_surrogate_apply(sg, sizeof(R) == 8 ? 0 : 1, db, n, vq.ev, vq.count, vq.cap, &B.flags[2], fb, fb_count,
                        (int *)&B.flags[3], ss);
    return 4;
  };
  if (!run_chunks<R>(B.stream, B.q, first[n], N, n * XMI_MAXL * XMI_MAXN, vr, qev, &B.flags[1], transport,
                     surrogate, estimator, ph, graph, go.overlap_chunks != 0))
    return false;
  unsigned long long flags[4];
  cudaMemcpy(flags, B.flags, sizeof(flags), cudaMemcpyDeviceToHost);
  g_timing.d2h_bytes += (long long)sizeof(flags);
  if (flags[0] != 0) {
    xmi_set_error("estimator kernel reported error code %llu", flags[0]);
    return false;
  }
  if (flags[3] != 0) {
    xmi_set_error("surrogate solid-angle kernel reported error code %llu", flags[3]);
    return false;
  }
  g_timing.events = (long long)flags[1];
  g_timing.surrogate_fallbacks = (long long)flags[2];
  return true;
}
}  // namespace

extern "C" int xmi_main_msim_batch(int n, xmi_inputFPtr *inputFPtrs, xmi_hdf5FPtr *hdf5FPtrs,
                                   xmi_main_options **options, xmi_solid_angle **solid_angles, double **channels,
                                   double **brute_histories, double **var_red_histories) {
  if (n < 1 || !inputFPtrs || !hdf5FPtrs || !options || !channels || !brute_histories || !var_red_histories) {
    xmi_set_error("xmi_main_msim_batch: invalid arguments");
    return 0;
  }
  if (!ensure_device()) return 0;
  std::lock_guard<std::mutex> lock(g_batch_lock);
  const int precision = inputFPtrs[0]->gpu.precision;
  std::vector<DevState *> st(n);
  std::vector<xmi::DevTally> tl(n);
  const auto wall0 = std::chrono::steady_clock::now();
  g_timing.h2d_bytes = g_timing.d2h_bytes = 0;
  g_timing.graph_updated = -1;
  const void *sg = nullptr;
  for (int c = 0; c < n; c++) {
    channels[c] = brute_histories[c] = var_red_histories[c] = nullptr;
    if (inputFPtrs[c]->gpu.precision != precision) {
      xmi_set_error("xmi_main_msim_batch: configurations %d and 0 differ in precision", c);
      return 0;
    }
    xmi_solid_angle *sa = solid_angles ? solid_angles[c] : nullptr;
    if (!xmi_gpu_prepare_run(inputFPtrs[c], hdf5FPtrs[c], options[c], 1, sa)) return 0;
    if (!xmi_dev_sync_tables(hdf5FPtrs[c], precision)) return 0;
    st[c] = state_of(hdf5FPtrs[c]);
    const xmi_bundle &h = hdf5FPtrs[c]->b;
    const bool use_sg = surrogate_in_use(inputFPtrs[c], options[c]);
    if (use_sg && sg && inputFPtrs[c]->surrogate != sg) {
      xmi_set_error("xmi_main_msim_batch: configuration %d uses another surrogate than the ones before it", c);
      return 0;
    }
    if (use_sg) sg = inputFPtrs[c]->surrogate;
    bool ok = precision == 0 ? stage_run<double>(st[c], st[c]->b64, h, tl[c], use_sg)
                             : stage_run<float>(st[c], st[c]->b32, h, tl[c], use_sg);
    if (!ok) return 0;
  }
  for (int c = 0; c < n; c++)
    if (!cuda_ok(cudaStreamSynchronize(st[c]->stream), "staging")) return 0;
  const int threads = inputFPtrs[0]->gpu.threads_per_block > 0 ? inputFPtrs[0]->gpu.threads_per_block : 128;
  if (threads > 128 || threads % 32) {
    xmi_set_error("threads_per_block must be a multiple of 32 up to 128 (got %d)", threads);
    return 0;
  }
  const int bps = inputFPtrs[0]->gpu.blocks_per_sm > 0 ? inputFPtrs[0]->gpu.blocks_per_sm : 8;
  Phases ph;
  const xmi_gpu_options &go = inputFPtrs[0]->gpu;
  bool ok = precision == 0 ? launch_batch<double>(n, st.data(), hdf5FPtrs, tl.data(), threads, bps, go, sg, true, ph)
                           : launch_batch<float>(n, st.data(), hdf5FPtrs, tl.data(), threads, bps, go, sg, true, ph);
  if (!ok) return 0;
  for (int c = 0; c < n; c++)
    if (!collect_outputs(st[c], hdf5FPtrs[c]->b, 1, &channels[c], &brute_histories[c], &var_red_histories[c],
                         nullptr))
      return 0;
  g_timing.transport_ms = ph.total_ms;
  g_timing.total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - wall0).count();
  g_timing.launches = ph.launches;
  for (int k = 0; k < 4; k++) g_timing.phase_ms[k] = ph.ms[k];
  return 1;
}

/* ---------------------------------------------------------------- */
/* points where the estimator queries solid angles (surrogate training)  */
/* ---------------------------------------------------------------- */
extern "C" int xmi_gpu_sample_event_points(xmi_inputFPtr in, xmi_hdf5FPtr t, xmi_main_options *options,
                                           double share, int max_points, double *r_out, double *theta_out,
                                           int *n_out) {
  if (!in || !t || !options || !(share > 0.0 && share <= 1.0) || max_points < 1 || !r_out || !theta_out || !n_out) {
    xmi_set_error("xmi_gpu_sample_event_points: invalid arguments");
    return 0;
  }
  if (!options->use_variance_reduction) {
    xmi_set_error("xmi_gpu_sample_event_points: the estimator runs only with variance reduction");
    return 0;
  }
  if (!ensure_device()) return 0;
  const int rep0 = t->replica, nrep0 = t->n_replicas;
  t->replica = 0;
  t->n_replicas = std::max(1, (int)std::lround(1.0 / share));
  bool ok = prepare_run(in, t, options, 1, nullptr, false) != 0;
  const int precision = in->gpu.precision;
  ok = ok && xmi_dev_sync_tables(t, precision);
  DevState *s = ok ? state_of(t) : nullptr;
  float *pr = nullptr, *pt = nullptr;
  unsigned long long *pn = nullptr, n_rec = 0;
  ok = ok && cuda_ok(cudaMalloc(&pr, sizeof(float) * max_points), "cudaMalloc") &&
       cuda_ok(cudaMalloc(&pt, sizeof(float) * max_points), "cudaMalloc") &&
       cuda_ok(cudaMalloc(&pn, sizeof(unsigned long long)), "cudaMalloc");
  const int threads = in->gpu.threads_per_block > 0 ? in->gpu.threads_per_block : 128;
  const int bps = in->gpu.blocks_per_sm > 0 ? in->gpu.blocks_per_sm : 8;
  /* pass 1 counts the events (share 0 recorded), pass 2 records about
   * max_points of them */
  double p = 0.0;
  for (int pass = 0; pass < 2 && ok; pass++) {
    PointRecorder rec;
    rec.p = p;
    rec.r = pr;
    rec.t = pt;
    rec.n = pn;
    rec.max = max_points;
    cudaMemsetAsync(pn, 0, sizeof(unsigned long long), s->stream);
    xmi::DevTally tl;
    Phases ph;
    ok = precision == 0 ? stage_run<double>(s, s->b64, t->b, tl, true) &&
                              launch_single<double>(s, s->b64, tl, t->b, threads, bps, in->gpu,
                                                    nullptr, ph, &rec)
                        : stage_run<float>(s, s->b32, t->b, tl, true) &&
                              launch_single<float>(s, s->b32, tl, t->b, threads, bps, in->gpu,
                                                   nullptr, ph, &rec);
    unsigned long long counters[8];
    ok = ok && cuda_ok(cudaMemcpy(counters, s->counters, sizeof(counters), cudaMemcpyDeviceToHost), "copy") &&
         cuda_ok(cudaMemcpy(&n_rec, pn, sizeof(n_rec), cudaMemcpyDeviceToHost), "copy");
    if (ok && counters[1] != 0) {
      xmi_set_error("transport kernel reported error code %llu", counters[1]);
      ok = false;
    }
    if (ok && pass == 0) {
      const double events = (double)counters[3];
      p = events > 0.0 ? std::min(1.0, 0.98 * max_points / events) : 1.0;
    }
  }
  const long long n = std::min((long long)n_rec, (long long)max_points);
  if (ok) {
    std::vector<float> hr(n > 0 ? n : 1), ht(n > 0 ? n : 1);
    ok = cuda_ok(cudaMemcpy(hr.data(), pr, sizeof(float) * n, cudaMemcpyDeviceToHost), "copy") &&
         cuda_ok(cudaMemcpy(ht.data(), pt, sizeof(float) * n, cudaMemcpyDeviceToHost), "copy");
    for (long long i = 0; ok && i < n; i++) {
      r_out[i] = hr[i];
      theta_out[i] = ht[i];
    }
    *n_out = (int)n;
  }
  cudaFree(pr);
  cudaFree(pt);
  cudaFree(pn);
  t->replica = rep0;
  t->n_replicas = nrep0;
  return ok ? 1 : 0;
}

/* ---------------------------------------------------------------- */
/* autotuner of the batched call                                     */
/* ---------------------------------------------------------------- */
extern "C" int xmi_gpu_autotune_batch(int n, xmi_inputFPtr *inputFPtrs, xmi_hdf5FPtr *hdf5FPtrs,
                                      xmi_main_options **options, xmi_solid_angle **solid_angles, double share,
                                      double *report) {
  if (n < 1 || !inputFPtrs || !hdf5FPtrs || !options || !(share > 0.0 && share <= 1.0)) {
    xmi_set_error("xmi_gpu_autotune_batch: invalid arguments");
    return 0;
  }
  const int R = std::max(1, (int)std::lround(1.0 / share));
  std::vector<int> rep0(n), nrep0(n);
  for (int c = 0; c < n; c++) {
    rep0[c] = hdf5FPtrs[c]->replica;
    nrep0[c] = hdf5FPtrs[c]->n_replicas;
    hdf5FPtrs[c]->replica = 0;
    hdf5FPtrs[c]->n_replicas = R;
  }
  std::vector<double *> ch(n), br(n), vr(n);
  auto trial = [&](int tpb, int bps, long long qev, double &ms) -> bool {
    for (int c = 0; c < n; c++) {
      inputFPtrs[c]->gpu.threads_per_block = tpb;
      inputFPtrs[c]->gpu.blocks_per_sm = bps;
      inputFPtrs[c]->gpu.queue_events = qev;
    }
    if (!xmi_main_msim_batch(n, inputFPtrs, hdf5FPtrs, options, solid_angles, ch.data(), br.data(), vr.data()))
      return false;
    ms = g_timing.transport_ms;
    for (int c = 0; c < n; c++) {
      free(ch[c]);
      free(br[c]);
      free(vr[c]);
    }
    return true;
  };
  int best_tpb = 128, best_bps = 8;
  long long best_qev = kMaxQueuedEvents;
  double best_ms = 1e300, ms = 0.0;
  bool ok = trial(best_tpb, best_bps, best_qev, ms); /* warm-up: buffers and tables (not compared) */
  const int tpbs[] = {64, 128}, bpss[] = {4, 8, 12, 16};
  for (int tpb : tpbs)
    for (int bps : bpss) {
      if (!ok) break;
      ok = trial(tpb, bps, best_qev, ms);
      if (ok && ms < best_ms) best_ms = ms, best_tpb = tpb, best_bps = bps;
    }
  const long long qevs[] = {1ll << 23, 1ll << 24};
  for (long long qev : qevs) {
    if (!ok) break;
    ok = trial(best_tpb, best_bps, qev, ms);
    if (ok && ms < best_ms) best_ms = ms, best_qev = qev;
  }
  for (int c = 0; c < n; c++) {
    hdf5FPtrs[c]->replica = rep0[c];
    hdf5FPtrs[c]->n_replicas = nrep0[c];
    inputFPtrs[c]->gpu.threads_per_block = best_tpb;
    inputFPtrs[c]->gpu.blocks_per_sm = best_bps;
    inputFPtrs[c]->gpu.queue_events = best_qev;
  }
  if (!ok) return 0;
  if (report) {
    report[0] = best_tpb;
    report[1] = best_bps;
    report[2] = (double)best_qev;
    report[3] = best_ms;
  }
  return 1;
}

/* ---------------------------------------------------------------- */
/* Diagnostic: the momentum kinematics of the advanced Compton path    */
/* ---------------------------------------------------------------- */
namespace {
__global__ void compton_kinematics_kernel(int n, const double *energy, const double *binding, const double *theta,
                                          const double *q, double *out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double th = theta[i];
  const float thf = (float)th, shf = sinf(0.5f * thf);
  bool bad64 = false, bad32 = false;
  out[6 * i + 0] = (double)xmi::cp_qimax<float>((float)energy[i], (float)binding[i], cosf(thf), shf * shf);
  out[6 * i + 1] = xmi::cp_qimax<double>(energy[i], binding[i], cos(th), 0.0);
  out[6 * i + 2] = (double)xmi::cp_energy_from_q((float)energy[i], (float)q[i], cosf(thf), sinf(thf), bad32);
  out[6 * i + 3] = xmi::cp_energy_from_q(energy[i], q[i], cos(th), sin(th), bad64);
  out[6 * i + 4] = bad32 ? 1.0 : 0.0;
  out[6 * i + 5] = bad64 ? 1.0 : 0.0;
}
}  // namespace

/* Runs the device functions of the per-shell Compton kinematics (FP32 and
 * FP64 forms) on n points: out[6 i ..] = qimax FP32, qimax FP64, scattered
 * energy FP32, scattered energy FP64, and the two "no root" flags. */
extern "C" int xmi_gpu_compton_kinematics(int n, const double *energy, const double *binding, const double *theta,
                                          const double *q, double *out) {
  if (n < 0 || (n > 0 && (!energy || !binding || !theta || !q || !out))) {
    xmi_set_error("xmi_gpu_compton_kinematics: bad arguments");
    return 0;
  }
  if (n == 0) return 1;
  double *d = nullptr;
  const size_t in_bytes = sizeof(double) * (size_t)n;
  if (cudaMalloc(&d, in_bytes * 10) != cudaSuccess) {
    xmi_set_error("xmi_gpu_compton_kinematics: cudaMalloc failed");
    return 0;
  }
  bool ok = cudaMemcpy(d, energy, in_bytes, cudaMemcpyHostToDevice) == cudaSuccess &&
            cudaMemcpy(d + n, binding, in_bytes, cudaMemcpyHostToDevice) == cudaSuccess &&
            cudaMemcpy(d + 2 * (size_t)n, theta, in_bytes, cudaMemcpyHostToDevice) == cudaSuccess &&
            cudaMemcpy(d + 3 * (size_t)n, q, in_bytes, cudaMemcpyHostToDevice) == cudaSuccess;
  if (ok) {
    compton_kinematics_kernel<<<(n + 127) / 128, 128>>>(n, d, d + n, d + 2 * (size_t)n, d + 3 * (size_t)n,
                                                        d + 4 * (size_t)n);
    ok = cudaGetLastError() == cudaSuccess &&
         cudaMemcpy(out, d + 4 * (size_t)n, in_bytes * 6, cudaMemcpyDeviceToHost) == cudaSuccess;
  }
  cudaFree(d);
  if (!ok) xmi_set_error("xmi_gpu_compton_kinematics: CUDA error");
  return ok ? 1 : 0;
}
