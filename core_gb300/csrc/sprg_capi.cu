// C ABI of the estimate-and-mark library: context (flattened mesh on the
// device), buffer management and the orchestration of the kernels for each
// reference call.  See include/spr_gb300.h for the contract of every entry.
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <algorithm>
#include <vector>

#include "spr_gb300.h"
#include "sprg_fast.h"
#include "sprg_learned.h"
#include "sprg_internal.h"

using namespace sprg;

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
};

// Final element sets of the listed (grown or refit) patches; they depend
// on the mesh geometry only, so they are built on the first pass and reused.
struct PatchCache {
  bool valid = false;
  int count = 0;
  DevBuf v, n, el;
  // tets: per-mesh weights of the cached patches' fits (w_ready once built)
  bool w_ready = false;
  DevBuf woff, w, wn;
};

// events of one timed host call: 0 call start, 1 field uploaded, 2 pass done,
// 3 flags upload joined, 4 marks applied, 5 flags downloaded, 6 call end (main
// stream); 7 / 8 flags upload, 9 / 10 size conversion + download (copy stream)
constexpr int kE2EEvents = 11;
constexpr int kE2EStages = 8;
const char* const kE2EStageNames[kE2EStages] = {"upload_field", "pass", "wait_flags_upload", "mark_sweep",
                                                "download_flags", "tail", "upload_flags_overlapped",
                                                "size_download_overlapped"};
const int kE2EStagePairs[kE2EStages][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 4}, {4, 5}, {5, 6}, {7, 8}, {9, 10}};

struct sprg_ctx {
  int device = 0;
  cudaStream_t own = nullptr;
  cudaStream_t stream = nullptr;
  int precision = SPRG_FP64;
  DevMesh m{};
  // mesh
  DevBuf xyz, xyzq, ev, edv, poff, pel, aoff, ael, tmp;
  // fields
  DevBuf f, ip, rec, err, esize, size, L, flags, q, sizes3, frames9;
  int ip_nc = 0;
  bool ip_valid = false, size_valid = false, L_valid = false, q_valid = false;
  // scratch
  DevBuf partials, out3, status, count, xitems, xcount, slab, bits;
  DevBuf titems, tcountb;  // triangle patches above the thread-per-vertex size
  DevBuf Lx, pairs, red, eflags;  // MA sweeps: lengths, vertex pairs, reduction scratch, element flags
  DevBuf logm;                    // LogAnisoSizeField: per-vertex log-metrics (V x 9)
  // FP64 recovery on tets: per-mesh QR weights and the listed patches
  DevBuf qw, qwlisted, qwitems, qwcount;
  bool qw_ready = false;
  // mixed-precision anisotropic pass: triangle patch weights and their
  // listed vertices (per mesh), FP32 metric records, guarded edges
  DevBuf tw, twlisted, twitems, twcount, met32, qrec32, agitems, agcount, kidx, kval, klen, rec9, cj64, qties;
  bool tw_ready = false;
  int op_kc = 3;  // operator components per slot (2 on a mesh in the z = 0 plane)
  // FP32 path buffers
  DevBuf crec, vrec, rec32, q32, sz2, fcnt, guard, tetd, wts, w64, listed, geo, geo64, elen, fitems;
  DevBuf gstamp, gfit, grec;  // guard pipeline scratch
  DevBuf tnext;               // work counter of the tet kernel
  DevBuf edone;               // blocks of the error kernel done (zero between passes)
  // learned form
  DevBuf hess;  // nodal Hessian upload (sprg_hessian_metric)
  // batch of independent meshes (sprg_set_batch)
  int batch_n = 0, batch_nseg = 0;
  DevBuf bvoff, bseg, bsegoff, bratios;
  static constexpr int kSegTets = 2048;  // elements per error segment (8 per thread)
  // binned recover: patch-size bins, tiles, tuned configuration
  DevBuf pcls, bverts, btiles, bnext, bcnt, cent;
  DevBuf qmax;  // the mesh's largest |cof J|^2 / |det J| (FP64 bits)
  DevBuf soff, sel, sw;  // sliced copy of the patch lists (offsets, element ids, weights)
  BinSlices bslices{};
  bool sliced = false;  // the sliced copy is built (lanes 0 available)
  bool bins_ready = false, tuned = false, autotune = true;
  int bin_count[4] = {0, 0, 0, 0};
  int bin_lanes[4] = {4, 4, 4, 4};
  int tile_verts = 256, grid_per_sm = 8, n_tiles = 0, n_sms = 152;
  int tile_mode = -1;  // the lane mode every tile shares, or -1
  std::string tune_json;
  // CUDA graph of the resident pass (sprg_graph_capture / sprg_graph_replay)
  cudaGraphExec_t graph_exec = nullptr;
  // the host entry point's own graph of the resident pass: captured on the
  // third call in a row with the same adapt ratio, form, stream and size
  // download (per-mesh setup is done by then), replayed after that; any
  // setter or mesh change drops it, a failed capture turns it off
  cudaGraphExec_t e2e_exec = nullptr;
  int e2e_calls = 0;
  int64_t e2e_launches = 0;
  double e2e_ratio = 0;
  int e2e_prec = -1;
  cudaStream_t e2e_stream = nullptr;
  bool e2e_early = false, e2e_off = false;
  DevBuf vvoff, vv, vtile, vr16, rec16, ql, sizel, fbitems, fbcount, mlp_packed, mlp_err, mlp_tmp;
  DevBuf lrange, ldone, lsc;  // learned records: field range scratch, its counter, difference scales
  bool vv_ready = false, have_mlp = false;
  int max_degree = 0;
  int use_mlp = 1;
  float z_max = 8.f;
  int stall_polls = 0;      // test hook: network-kernel wait on a barrier nothing completes (0: off)
  int alloc_fail_in = -1;   // test hook: device allocations left before one fails (-1: off)
  // side stream for the FP64 fits of listed patches, forked from and joined
  // back into the pass's stream
  cudaStream_t side = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  // copy stream of the host entry point: the flags upload and (FP32) the size
  // download run beside the pass
  cudaStream_t copy = nullptr;
  cudaEvent_t copy_fork = nullptr, copy_join = nullptr;
  cudaEvent_t size_ready = nullptr, size_join = nullptr;
  bool size_hook = false;  // the FP32 pass records size_ready after the vertex average
  // stage timing of the host entry point (sprg_e2e_timing): events at the
  // stage boundaries of each call, summed per stage, plus the host's enqueue
  // and wait times
  bool e2e_timing = false;
  cudaEvent_t e2e_ev[kE2EEvents] = {};
  double e2e_sum[kE2EStages] = {};
  double e2e_host[3] = {};  // enqueue, wait, whole call (ms)
  int e2e_n = 0;
  std::string e2e_json;
  DevBuf mcount;           // split / collapse counts of the host entry point
  // pinned staging of the small results read back after a pass (status,
  // integrals, counters): enqueued on the stream, read after one synchronize
  struct HostStage {
    DevStatus st;
    int xc, fb, me;
    int fc[6];
    double o3[3];
    unsigned long long counts[2];
  };
  HostStage* stage = nullptr;
  bool vrec_ready = false;  // coordinate records and SPR weights (per mesh)
  bool crec_ready = false;  // coordinate records alone (the mixed anisotropic pass)
  double frame[4] = {0, 0, 0, 1};  // coordinate records: x' = (x - c) s + 1 in [1, 2]
  bool planar = false;             // every vertex has z = 0
  int n_listed = 0, n_refit = 0;
  PatchCache cache64, cache32, cache2d;
  static constexpr int kGuardCap = 1 << 20;
  static constexpr float kGuardRel = 2e-6f;
  std::string err_msg;
  int64_t launches = 0;
  sprg_size_info last_info{};
  // per-kernel CUDA-event timing (sprg_profile_*)
  bool prof = false;
  std::vector<cudaEvent_t> ev_pool;
  size_t ev_used = 0;
  std::vector<std::pair<std::string, size_t>> pending;  // name, index of start event
  std::map<std::string, std::pair<int64_t, double>> prof_acc;
  std::string prof_json;
};

namespace {

int fail(sprg_ctx* c, int code, const std::string& msg) {
  if (c) c->err_msg = msg;
  return code;
}

int cuda_fail(sprg_ctx* c, cudaError_t e, const char* where) {
  std::string msg = std::string(where) + ": " + cudaGetErrorString(e);
  int code = (e == cudaErrorMemoryAllocation) ? SPRG_ENOMEM : SPRG_ECUDA;
  return fail(c, code, msg);
}

#define CK(call)                                              \
  do {                                                        \
    cudaError_t e_ = (call);                                  \
    if (e_ != cudaSuccess) return cuda_fail(c, e_, #call);    \
  } while (0)

// grow-only device buffer
int ensure(sprg_ctx* c, DevBuf& b, size_t bytes) {
  if (bytes == 0) bytes = 16;
  if (b.bytes >= bytes) return SPRG_OK;
  if (c->alloc_fail_in == 0) return fail(c, SPRG_ENOMEM, "device allocation failed (injected)");
  if (c->alloc_fail_in > 0) --c->alloc_fail_in;
  if (b.p) cudaFree(b.p);
  b.p = nullptr;
  b.bytes = 0;
  cudaError_t e = cudaMalloc(&b.p, bytes);
  if (e != cudaSuccess) return cuda_fail(c, e, "cudaMalloc");
  b.bytes = bytes;
  return SPRG_OK;
}

void release(DevBuf& b) {
  if (b.p) cudaFree(b.p);
  b.p = nullptr;
  b.bytes = 0;
}

template <class T>
T* P(DevBuf& b) { return static_cast<T*>(b.p); }

#define ENSURE(buf, bytes)                     \
  do {                                         \
    int rc_ = ensure(c, (buf), (bytes));       \
    if (rc_) return rc_;                       \
  } while (0)

int check_launch(sprg_ctx* c, const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(c, e, what);
  return SPRG_OK;
}

int ensure_stage(sprg_ctx* c) {
  if (c->stage) return SPRG_OK;
  void* p = nullptr;
  cudaError_t e = cudaMallocHost(&p, sizeof(sprg_ctx::HostStage));
  if (e != cudaSuccess) return cuda_fail(c, e, "cudaMallocHost");
  c->stage = static_cast<sprg_ctx::HostStage*>(p);
  memset(c->stage, 0, sizeof(sprg_ctx::HostStage));
  return SPRG_OK;
}

// the device status word, read back with the stream's other results
int sync_and_status(sprg_ctx* c) {
  int rc = ensure_stage(c);
  if (rc) return rc;
  cudaError_t e = cudaMemcpyAsync(&c->stage->st, c->status.p, sizeof(DevStatus), cudaMemcpyDeviceToHost, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "status readback");
  e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "cudaStreamSynchronize");
  const DevStatus st = c->stage->st;
  if (st.code == SPRG_EPATCH)
    return fail(c, SPRG_EPATCH,
                st.where >= 0 ? "SPR: patch construction failed at vertex " + std::to_string(st.where)
                              : std::string("SPR: expansion list overflow"));
  if (st.code == SPRG_EFLAGS)
    return fail(c, SPRG_EFLAGS, "markEntities: entity " + std::to_string(st.where) + " already carries the true flag");
  if (st.code == SPRG_EEIGEN)
    return fail(c, SPRG_EEIGEN, "eigenQR of a log-metric did not converge (entity " + std::to_string(st.where) + ")");
  if (st.code) return fail(c, st.code, "device status " + std::to_string(st.code));
  return SPRG_OK;
}

int reset_status(sprg_ctx* c) {
  CK(cudaMemsetAsync(c->status.p, 0, sizeof(DevStatus), c->stream));
  return SPRG_OK;
}

int set_device(sprg_ctx* c) {
  CK(cudaSetDevice(c->device));
  return SPRG_OK;
}

// ---- per-kernel timing ----------------------------------------------------
// When profiling is on, every kernel launch of the pass is bracketed by two
// events from a preallocated pool, recorded on the launching stream.
void prof_begin(sprg_ctx* c, const char* name) {
  if (!c->prof) return;
  if (c->ev_used + 2 > c->ev_pool.size()) return;  // pool exhausted: stop recording
  cudaEventRecord(c->ev_pool[c->ev_used], c->stream);
  c->pending.emplace_back(name, c->ev_used);
  c->ev_used += 2;
}
void prof_end(sprg_ctx* c) {
  if (!c->prof || c->pending.empty()) return;
  size_t i = c->pending.back().second;
  if (i + 1 < c->ev_pool.size()) cudaEventRecord(c->ev_pool[i + 1], c->stream);
}
#define PB(name) prof_begin(c, name)
#define PE() prof_end(c)

// ---- pipeline steps on resident buffers -------------------------------

// Listed patches: grow them on the first pass (recording the final element
// sets), afterwards one QR fit per cached set.
// Tets: once a patch cache exists, the QR of each cached patch runs once
// (per mesh) into weights, and later passes take weighted sums.  Runs on
// the context stream (it reads the patch sizes back).
int ensure_cache_weights(sprg_ctx* c, PatchCache& pc) {
  if (!pc.valid || pc.w_ready || c->m.dim != 3 || pc.count <= 0) return SPRG_OK;
  std::vector<int> n((size_t)pc.count);
  CK(cudaMemcpyAsync(n.data(), pc.n.p, sizeof(int) * n.size(), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  std::vector<long long> off(n.size());
  long long total = 0;
  for (size_t i = 0; i < n.size(); ++i) {
    off[i] = total;
    total += n[i] > 0 ? n[i] : 0;
  }
  ENSURE(pc.woff, sizeof(long long) * off.size());
  ENSURE(pc.w, sizeof(double) * (size_t)(total > 0 ? total : 1));
  ENSURE(pc.wn, sizeof(int) * n.size());
  ENSURE(c->slab, sizeof(double) * (size_t)expand_grid() * expand_max_elems() * 8);
  CK(cudaMemcpyAsync(pc.woff.p, off.data(), sizeof(long long) * off.size(), cudaMemcpyHostToDevice, c->stream));
  PB("cached_weights_f64");
  launch_cached_weights_f64(c->m, pc.count, P<int>(pc.v), P<int>(pc.n), P<int>(pc.el), P<long long>(pc.woff),
                            P<double>(pc.w), P<int>(pc.wn), P<double>(c->slab), c->stream);
  PE();
  c->launches += 1;
  int rc = check_launch(c, "cached patch weights");
  if (rc) return rc;
  CK(cudaStreamSynchronize(c->stream));  // the host offsets stay alive until the copy is done
  pc.w_ready = true;
  return SPRG_OK;
}

int listed_fits(sprg_ctx* c, PatchCache& pc, const double* ip, const double* u, int nc, double* rec64, ExpandList xl,
                cudaStream_t on = nullptr) {
  DevMesh& m = c->m;
  if (pc.valid) {
    if (!on) {
      int rc = ensure_cache_weights(c, pc);
      if (rc) return rc;
    }
    cudaStream_t s = on ? on : c->stream;
    if (!on) PB("cached_fit_f64");
    if (pc.w_ready)
      launch_cached_wsum_f64(m, ip, u, nc, rec64, pc.count, P<int>(pc.v), P<int>(pc.el), P<long long>(pc.woff),
                             P<double>(pc.w), P<int>(pc.wn), P<DevStatus>(c->status), s);
    else
      launch_cached_fit_f64(m, ip, u, nc, rec64, pc.count, P<int>(pc.v), P<int>(pc.n), P<int>(pc.el),
                            P<double>(c->slab), P<DevStatus>(c->status), s);
    if (!on) PE();
    c->launches += 1;
    return check_launch(c, "cached fit");
  }
  int xc = 0;
  CK(cudaMemcpyAsync(&xc, xl.count, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  if (xc > xl.cap) xc = xl.cap;
  size_t slots = (size_t)(xc > 0 ? xc : 1);
  ENSURE(pc.v, sizeof(int) * slots);
  ENSURE(pc.n, sizeof(int) * slots);
  ENSURE(pc.el, sizeof(int) * slots * expand_max_elems());
  PB("expand_f64");
  launch_expand_f64(m, ip, u, nc, rec64, xl, P<double>(c->slab), P<DevStatus>(c->status), c->stream, P<int>(pc.v),
                    P<int>(pc.n), P<int>(pc.el));
  PE();
  c->launches += 1;
  int rc = check_launch(c, "expand");
  if (rc) return rc;
  pc.count = xc;
  pc.valid = true;
  if (m.dim != 3) return SPRG_OK;
  // tets: this pass already takes the weighted sums, so every pass gives the
  // same bits for the listed patches
  if ((rc = ensure_cache_weights(c, pc))) return rc;
  if (!pc.w_ready) return SPRG_OK;
  launch_cached_wsum_f64(m, ip, u, nc, rec64, pc.count, P<int>(pc.v), P<int>(pc.el), P<long long>(pc.woff),
                         P<double>(pc.w), P<int>(pc.wn), P<DevStatus>(c->status), c->stream);
  c->launches += 1;
  return check_launch(c, "cached fit");
}

int step_grad(sprg_ctx* c, int ncin) {
  DevMesh& m = c->m;
  ENSURE(c->ip, sizeof(double) * (size_t)m.T * 3 * ncin);
  PB("grad_ip_f64");
  launch_grad_ip_f64(m, P<double>(c->f), ncin, P<double>(c->ip), c->stream);
  PE();
  c->launches += 1;
  c->ip_nc = 3 * ncin;
  c->ip_valid = true;
  return check_launch(c, "grad_ip");
}

int step_recover(sprg_ctx* c) {
  DevMesh& m = c->m;
  int nc = c->ip_nc;
  ENSURE(c->rec, sizeof(double) * (size_t)m.V * nc);
  ENSURE(c->slab, sizeof(double) * (size_t)expand_grid() * expand_max_elems() * (4 + nc + 1));
  if (m.dim == 3) {
    // tets: the per-mesh FP64 QR weights, a weighted sum per vertex; the
    // listed patches (growth, size) through the slab fits
    ENSURE(c->qwitems, sizeof(int) * (size_t)(m.V > 0 ? m.V : 1));
    ENSURE(c->qwcount, sizeof(int));
    const ExpandList lst{P<int>(c->qwitems), P<int>(c->qwcount), m.V};
    if (!c->qw_ready) {
      ENSURE(c->qw, sizeof(double) * (size_t)m.T * m.nn);
      ENSURE(c->qwlisted, (size_t)(m.V > 0 ? m.V : 1));
      CK(cudaMemsetAsync(c->qwcount.p, 0, sizeof(int), c->stream));
      PB("qr_weights_f64");
      launch_qr_weights(m, P<double>(c->qw), P<unsigned char>(c->qwlisted), lst, c->stream);
      PE();
      c->launches += 1;
      int rc = check_launch(c, "QR weights");
      if (rc) return rc;
      c->qw_ready = true;
    }
    PB("recover_f64");
    launch_recover_w64(m, P<double>(c->ip), nc, P<double>(c->qw), P<unsigned char>(c->qwlisted), P<double>(c->rec),
                       c->stream);
    PE();
    c->launches += 1;
    int rc = check_launch(c, "recover");
    if (rc) return rc;
    return listed_fits(c, c->cache64, P<double>(c->ip), nullptr, nc, P<double>(c->rec), lst);
  }
  ENSURE(c->xitems, sizeof(int) * (size_t)(m.V > 0 ? m.V : 1));
  ENSURE(c->xcount, sizeof(int));
  ENSURE(c->titems, sizeof(int) * (size_t)(m.dim == 2 && m.V > 0 ? m.V : 1));
  ENSURE(c->tcountb, sizeof(int));
  CK(cudaMemsetAsync(c->xcount.p, 0, sizeof(int), c->stream));
  CK(cudaMemsetAsync(c->tcountb.p, 0, sizeof(int), c->stream));
  ExpandList xl{P<int>(c->xitems), P<int>(c->xcount), m.V};
  ExpandList big{P<int>(c->titems), P<int>(c->tcountb), m.dim == 2 ? m.V : 0};
  PB("recover_f64");
  launch_recover_f64(m, P<double>(c->ip), nc, P<double>(c->rec), xl, big, P<DevStatus>(c->status), c->stream);
  PE();
  c->launches += 1;
  int rc = check_launch(c, "recover");
  if (rc) return rc;
  // patches that need growth: the reference growth order, on the device
  return listed_fits(c, c->cache64, P<double>(c->ip), nullptr, nc, P<double>(c->rec), xl);
}

int step_size(sprg_ctx* c, int mode, double adapt_ratio, double target, double alpha, double beta) {
  DevMesh& m = c->m;
  int nc = c->ip_nc;
  int nb = error_blocks(m.T);
  ENSURE(c->err, sizeof(double) * (size_t)m.T);
  ENSURE(c->esize, sizeof(double) * (size_t)m.T);
  ENSURE(c->size, sizeof(double) * (size_t)m.V);
  ENSURE(c->partials, sizeof(double) * 2 * (size_t)(nb > 0 ? nb : 1));
  ENSURE(c->out3, sizeof(double) * 4);
  double p = 1, d = m.dim;
  double gexp = (2 * d) / (2 * p + d);
  PB("error_f64");
  launch_error_f64(m, P<double>(c->ip), nc, P<double>(c->rec), P<double>(c->err), P<double>(c->partials), nb, gexp,
                   c->stream);
  PE();
  PB("size_factor");
  launch_size_factor(P<double>(c->partials), nb, mode, adapt_ratio, target, m.dim, P<double>(c->out3), c->stream);
  PE();
  PB("esize_f64");
  launch_esize_f64(m, P<double>(c->err), P<double>(c->out3), mode, alpha, beta, P<double>(c->esize), c->stream);
  PE();
  PB("average_f64");
  launch_average(m, P<double>(c->esize), P<double>(c->size), c->stream);
  PE();
  c->launches += 4;
  c->size_valid = true;
  return check_launch(c, "size field");
}

int step_measure_iso(sprg_ctx* c) {
  DevMesh& m = c->m;
  ENSURE(c->L, sizeof(double) * (size_t)m.E);
  PB("measure_f64");
  launch_measure_iso_f64(m, P<double>(c->size), P<double>(c->L), c->stream);
  PE();
  c->launches += 1;
  c->L_valid = true;
  return check_launch(c, "measure");
}

// the pass's integrals and counters, copied into the staging block on the
// stream (read by info_from_stage after the stream is synchronized)
int enqueue_info(sprg_ctx* c) {
  int rc = ensure_stage(c);
  if (rc) return rc;
  sprg_ctx::HostStage* h = c->stage;
  CK(cudaMemcpyAsync(h->o3, c->out3.p, sizeof h->o3, cudaMemcpyDeviceToHost, c->stream));
  // listed patches of the last FP64 recovery (tets: the per-mesh list of
  // the QR weights; triangles: the pass's expansion list)
  h->xc = 0;
  const DevBuf& cnt = c->m.dim == 3 ? c->qwcount : c->xcount;
  if (cnt.p) CK(cudaMemcpyAsync(&h->xc, cnt.p, sizeof h->xc, cudaMemcpyDeviceToHost, c->stream));
  if (c->precision == SPRG_LEARNED && c->fbcount.p) {
    CK(cudaMemcpyAsync(&h->fb, c->fbcount.p, sizeof h->fb, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(&h->me, c->mlp_err.p, sizeof h->me, cudaMemcpyDeviceToHost, c->stream));
  }
  if (c->precision == SPRG_FP32 && c->fcnt.p)
    CK(cudaMemcpyAsync(h->fc, c->fcnt.p, sizeof h->fc, cudaMemcpyDeviceToHost, c->stream));
  return SPRG_OK;
}

int info_from_stage(sprg_ctx* c, sprg_size_info* info) {
  const sprg_ctx::HostStage* h = c->stage;
  c->last_info.eps_star_norm2 = h->o3[0];
  c->last_info.error_sum = h->o3[1];
  c->last_info.size_factor = h->o3[2];
  c->last_info.n_expanded = h->xc;
  c->last_info.n_fp64_refits = 0;
  c->last_info.n_guard_edges = 0;
  c->last_info.n_guard_unresolved = 0;
  c->last_info.n_learned_fallback = 0;
  c->last_info.n_rounding_dominated = 0;
  if (c->precision == SPRG_LEARNED && c->fbcount.p) {
    if (h->me) return fail(c, SPRG_ECUDA, "learned form: a tensor-core wait ran out of time");
    c->last_info.n_learned_fallback = h->fb;
    c->last_info.n_fp64_refits = c->n_refit;
    c->last_info.n_expanded = c->n_listed - c->n_refit;
  }
  if (c->precision == SPRG_FP32 && c->fcnt.p) {
    c->last_info.n_fp64_refits = c->n_refit;
    c->last_info.n_guard_edges = h->fc[1];
    c->last_info.n_guard_unresolved = h->fc[4];
    c->last_info.n_rounding_dominated = c->batch_n ? 0 : h->fc[5];
    c->last_info.n_expanded = c->n_listed - c->n_refit;
  }
  if (info) *info = c->last_info;
  return SPRG_OK;
}

int fill_info(sprg_ctx* c, sprg_size_info* info) {
  int rc = enqueue_info(c);
  if (rc) return rc;
  CK(cudaStreamSynchronize(c->stream));
  return info_from_stage(c, info);
}

int upload_ip(sprg_ctx* c, const double* ip, int ncomp) {
  if (ncomp != 3 && ncomp != 9) return fail(c, SPRG_EINVAL, "ip field must have 3 or 9 components");
  if (ip) {
    ENSURE(c->ip, sizeof(double) * (size_t)c->m.T * ncomp);
    CK(cudaMemcpyAsync(c->ip.p, ip, sizeof(double) * (size_t)c->m.T * ncomp, cudaMemcpyHostToDevice, c->stream));
    c->ip_nc = ncomp;
    c->ip_valid = true;
  } else {
    if (!c->ip_valid) return fail(c, SPRG_ESTATE, "no resident integration-point field");
    if (c->ip_nc != ncomp) return fail(c, SPRG_EINVAL, "component count differs from the resident ip field");
  }
  return SPRG_OK;
}

}  // namespace

// ======================================================================
// C ABI
// ======================================================================
extern "C" {

// the FP32 records' frame from the bounding box: shift to the lower corner
// and scale by a power of two so every coordinate lands in [1, 2]
static void set_frame(sprg_ctx* c, const double* lo, const double* hi) {
  double ext = 0;
  for (int k = 0; k < 3; ++k) ext = hi[k] - lo[k] > ext ? hi[k] - lo[k] : ext;
  double s = 1;
  while (s * ext > 1) s *= 0.5;
  while (ext > 0 && s * ext <= 0.5) s *= 2;
  c->frame[0] = lo[0];
  c->frame[1] = lo[1];
  c->frame[2] = lo[2];
  c->frame[3] = s;
  c->planar = lo[2] == 0.0 && hi[2] == 0.0;
}

// index arrays must stay inside the entity counts: a bad id would reach
// the kernels as an out-of-range gather
static bool ids_in_range(const int32_t* a, size_t n, int64_t limit) {
  for (size_t i = 0; i < n; ++i)
    if (a[i] < 0 || a[i] >= limit) return false;
  return true;
}

// a vertex -> element CSR: offsets from 0 to T nn, non-decreasing, entries
// element ids
static bool csr_valid(const int32_t* off, const int32_t* el, int64_t V, int64_t T, int nn) {
  if (off[0] != 0 || off[V] != T * nn) return false;
  for (int64_t v = 0; v < V; ++v)
    if (off[v + 1] < off[v]) return false;
  return ids_in_range(el, (size_t)(T * nn), T);
}

int sprg_create(const sprg_mesh_view* mv, int device, sprg_ctx** out) {
  if (!out) return SPRG_EINVAL;
  *out = nullptr;
  if (!mv || (mv->dim != 2 && mv->dim != 3) || mv->n_verts <= 0 || mv->n_elems <= 0 || mv->n_edges <= 0 ||
      !mv->coords || !mv->elem_verts || !mv->edge_verts)
    return SPRG_EINVAL;
  if (mv->n_verts > INT32_MAX || mv->n_edges > INT32_MAX || mv->n_elems * (mv->dim + 1) > INT32_MAX)
    return SPRG_EINVAL;
  if ((mv->vert_elem_offsets == nullptr) != (mv->vert_elems == nullptr)) return SPRG_EINVAL;
  if (!ids_in_range(mv->elem_verts, (size_t)(mv->n_elems * (mv->dim + 1)), mv->n_verts) ||
      !ids_in_range(mv->edge_verts, (size_t)(2 * mv->n_edges), mv->n_verts))
    return SPRG_EINVAL;
  if (mv->vert_elem_offsets &&
      !csr_valid(mv->vert_elem_offsets, mv->vert_elems, mv->n_verts, mv->n_elems, mv->dim + 1))
    return SPRG_EINVAL;
  sprg_ctx* c = new sprg_ctx();
  c->device = device;
  int rc = set_device(c);
  if (rc) { delete c; return rc; }
  if (cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking) != cudaSuccess) { delete c; return SPRG_ECUDA; }
  c->stream = c->own;
  DevMesh& m = c->m;
  m.dim = mv->dim;
  m.nn = mv->dim + 1;
  m.ne_el = mv->dim == 3 ? 6 : 3;
  m.V = (int)mv->n_verts;
  m.T = (int)mv->n_elems;
  m.E = (int)mv->n_edges;
  auto bail = [&](int code) { sprg_destroy(c); return code; };
#define CKC(call)                                                            \
  do {                                                                       \
    cudaError_t e_ = (call);                                                 \
    if (e_ != cudaSuccess) return bail(cuda_fail(c, e_, #call));             \
  } while (0)
#define ENSUREC(buf, bytes)                                                  \
  do {                                                                       \
    int rc_ = ensure(c, (buf), (bytes));                                     \
    if (rc_) return bail(rc_);                                               \
  } while (0)
  size_t nel = (size_t)m.T * m.nn;
  ENSUREC(c->xyz, sizeof(double) * 3 * (size_t)m.V);
  ENSUREC(c->xyzq, sizeof(int) * 4 * (size_t)m.V);
  ENSUREC(c->ev, sizeof(int) * nel);
  ENSUREC(c->edv, sizeof(int) * 2 * (size_t)m.E);
  ENSUREC(c->poff, sizeof(int) * ((size_t)m.V + 1));
  ENSUREC(c->pel, sizeof(int) * nel);
  ENSUREC(c->tmp, sizeof(int) * (size_t)m.V);
  ENSUREC(c->status, sizeof(DevStatus));
  ENSUREC(c->count, sizeof(unsigned long long));
  CKC(cudaMemsetAsync(c->status.p, 0, sizeof(DevStatus), c->stream));
  CKC(cudaMemcpyAsync(c->xyz.p, mv->coords, sizeof(double) * 3 * (size_t)m.V, cudaMemcpyHostToDevice, c->stream));
  CKC(cudaMemcpyAsync(c->ev.p, mv->elem_verts, sizeof(int) * nel, cudaMemcpyHostToDevice, c->stream));
  CKC(cudaMemcpyAsync(c->edv.p, mv->edge_verts, sizeof(int) * 2 * (size_t)m.E, cudaMemcpyHostToDevice, c->stream));
  {
    // bounding box -> the FP32 records' frame: shift to the lower corner and
    // scale by a power of two so every coordinate lands in [1, 2]
    double lo[3] = {mv->coords[0], mv->coords[1], mv->coords[2]}, hi[3] = {lo[0], lo[1], lo[2]};
    for (int64_t v = 1; v < mv->n_verts; ++v)
      for (int k = 0; k < 3; ++k) {
        const double x = mv->coords[3 * v + k];
        lo[k] = x < lo[k] ? x : lo[k];
        hi[k] = x > hi[k] ? x : hi[k];
      }
    set_frame(c, lo, hi);
  }
  m.xyz = P<double>(c->xyz);
  m.xyzq = P<int>(c->xyzq);
  m.ev = P<int>(c->ev);
  m.edv = P<int>(c->edv);
  if (mv->vert_elem_offsets) {
    // caller-supplied reference adjacency order for averaging; sorted copy for patches
    ENSUREC(c->aoff, sizeof(int) * ((size_t)m.V + 1));
    ENSUREC(c->ael, sizeof(int) * nel);
    CKC(cudaMemcpyAsync(c->aoff.p, mv->vert_elem_offsets, sizeof(int) * ((size_t)m.V + 1), cudaMemcpyHostToDevice,
                        c->stream));
    CKC(cudaMemcpyAsync(c->ael.p, mv->vert_elems, sizeof(int) * nel, cudaMemcpyHostToDevice, c->stream));
    CKC(cudaMemcpyAsync(c->poff.p, c->aoff.p, sizeof(int) * ((size_t)m.V + 1), cudaMemcpyDeviceToDevice, c->stream));
    CKC(cudaMemcpyAsync(c->pel.p, c->ael.p, sizeof(int) * nel, cudaMemcpyDeviceToDevice, c->stream));
    launch_sort_segments(m.V, P<int>(c->poff), P<int>(c->pel), c->stream);
    m.a_off = P<int>(c->aoff);
    m.a_el = P<int>(c->ael);
  } else {
    launch_build_v2e(m, P<int>(c->poff), P<int>(c->pel), P<int>(c->tmp), c->stream);
    launch_sort_segments(m.V, P<int>(c->poff), P<int>(c->pel), c->stream);
    m.a_off = P<int>(c->poff);
    m.a_el = P<int>(c->pel);
  }
  m.p_off = P<int>(c->poff);
  m.p_el = P<int>(c->pel);
  launch_xyz_to_fixed(m, c->frame, P<int>(c->xyzq), c->stream);
  CKC(cudaGetLastError());
  CKC(cudaStreamSynchronize(c->stream));
  // validate the adjacency: every offset array must end at T * nn
  int last = 0;
  CKC(cudaMemcpy(&last, P<int>(c->poff) + m.V, sizeof(int), cudaMemcpyDeviceToHost));
  if ((size_t)last != nel) {
    c->err_msg = "vertex-element adjacency does not cover every element vertex";
    return bail(SPRG_EINVAL);
  }
#undef CKC
#undef ENSUREC
  *out = c;
  return SPRG_OK;
}

// every per-mesh result, cache and derived structure, after the mesh changed
static void drop_e2e_graph(sprg_ctx* c) {
  if (c->e2e_exec) cudaGraphExecDestroy(c->e2e_exec);
  c->e2e_exec = nullptr;
  c->e2e_calls = 0;
}

static void invalidate_mesh_state(sprg_ctx* c) {
  drop_e2e_graph(c);
  c->ip_valid = c->size_valid = c->L_valid = c->q_valid = false;
  c->vrec_ready = false;
  c->crec_ready = false;
  c->bins_ready = false;
  // the tuned launch shape stays: every choice gives bitwise the same result,
  // and an adapt iteration changes the patch-size mix little
  c->tw_ready = false;
  c->qw_ready = false;
  c->vv_ready = false;
  c->cache64.valid = c->cache32.valid = c->cache2d.valid = false;
  c->cache64.w_ready = c->cache32.w_ready = c->cache2d.w_ready = false;
  c->batch_n = 0;
  c->batch_nseg = 0;
  // stamps are zeroed when (re)allocated at the next guard pass
  release(c->gstamp);
  if (c->graph_exec) {
    cudaGraphExecDestroy(c->graph_exec);
    c->graph_exec = nullptr;
  }
}

int sprg_update_mesh(sprg_ctx* c, const sprg_mesh_delta* d) {
  if (!c || !d) return SPRG_EINVAL;
  DevMesh& m = c->m;
  const int nn = m.nn;
  const int64_t V1 = d->n_verts, T1 = d->n_elems, E1 = d->n_edges;
  // ---- validation (nothing changes before it passes)
  if (V1 <= 0 || T1 <= 0 || E1 <= 0 || V1 > INT32_MAX || E1 > INT32_MAX || T1 * nn > INT32_MAX)
    return fail(c, SPRG_EINVAL, "counts must be positive and fit 32-bit ids");
  if (d->n_vert_rows < 0 || d->n_elem_rows < 0 || d->n_edge_rows < 0 ||
      (d->n_vert_rows && (!d->vert_ids || !d->coords)) || (d->n_elem_rows && (!d->elem_ids || !d->elem_verts)) ||
      (d->n_edge_rows && (!d->edge_ids || !d->edge_verts)))
    return fail(c, SPRG_EINVAL, "row lists need their ids and values");
  if ((d->vert_elem_offsets == nullptr) != (d->vert_elems == nullptr))
    return fail(c, SPRG_EINVAL, "averaging CSR: offsets and elements go together");
  auto rows_ok = [](int64_t n, const int32_t* ids, int64_t count, int64_t old) {
    std::vector<char> seen(count > old ? (size_t)(count - old) : 0, 0);
    for (int64_t r = 0; r < n; ++r) {
      if (ids[r] < 0 || ids[r] >= count) return false;
      if (ids[r] >= old) seen[(size_t)(ids[r] - old)] = 1;
    }
    for (char x : seen)
      if (!x) return false;
    return true;
  };
  if (!rows_ok(d->n_vert_rows, d->vert_ids, V1, m.V) || !rows_ok(d->n_elem_rows, d->elem_ids, T1, m.T) ||
      !rows_ok(d->n_edge_rows, d->edge_ids, E1, m.E))
    return fail(c, SPRG_EINVAL, "row ids out of range, or new rows not all listed");
  if (!ids_in_range(d->elem_verts, (size_t)(d->n_elem_rows * nn), V1) ||
      !ids_in_range(d->edge_verts, (size_t)(2 * d->n_edge_rows), V1))
    return fail(c, SPRG_EINVAL, "element or edge vertex id out of range");
  if (d->vert_elem_offsets && !csr_valid(d->vert_elem_offsets, d->vert_elems, V1, T1, nn))
    return fail(c, SPRG_EINVAL, "averaging CSR does not match the new counts");
  int rc = set_device(c);
  if (rc) return rc;
  c->launches = 0;
  CK(cudaStreamSynchronize(c->stream));
  // ---- the new arrays: kept rows copied, listed rows scattered
  DevBuf nxyz, nev, nedv, ids, vals, bad;
  auto cleanup = [&]() {
    release(nxyz); release(nev); release(nedv); release(ids); release(vals); release(bad);
  };
#define CKU(call)                                                  \
  do {                                                             \
    cudaError_t e_ = (call);                                       \
    if (e_ != cudaSuccess) { cleanup(); return cuda_fail(c, e_, #call); } \
  } while (0)
#define ENSUREU(buf, bytes)                                        \
  do {                                                             \
    int rc_ = ensure(c, (buf), (bytes));                           \
    if (rc_) { cleanup(); return rc_; }                            \
  } while (0)
  ENSUREU(nxyz, sizeof(double) * 3 * (size_t)V1);
  ENSUREU(nev, sizeof(int) * (size_t)(T1 * nn));
  ENSUREU(nedv, sizeof(int) * 2 * (size_t)E1);
  const int64_t kv = V1 < m.V ? V1 : m.V, kt = T1 < m.T ? T1 : m.T, ke = E1 < m.E ? E1 : m.E;
  CKU(cudaMemcpyAsync(nxyz.p, c->xyz.p, sizeof(double) * 3 * (size_t)kv, cudaMemcpyDeviceToDevice, c->stream));
  CKU(cudaMemcpyAsync(nev.p, c->ev.p, sizeof(int) * (size_t)(kt * nn), cudaMemcpyDeviceToDevice, c->stream));
  CKU(cudaMemcpyAsync(nedv.p, c->edv.p, sizeof(int) * 2 * (size_t)ke, cudaMemcpyDeviceToDevice, c->stream));
  const int64_t maxrows = std::max(d->n_vert_rows, std::max(d->n_elem_rows, d->n_edge_rows));
  ENSUREU(ids, sizeof(int) * (size_t)(maxrows > 0 ? maxrows : 1));
  ENSUREU(vals, sizeof(double) * 3 * (size_t)(maxrows > 0 ? maxrows : 1) + sizeof(int) * (size_t)(maxrows * nn));
  ENSUREU(bad, sizeof(unsigned long long));
  auto scatter_i32 = [&](int64_t n, const int32_t* hid, const int32_t* hval, int width, int* dst) -> int {
    if (!n) return SPRG_OK;
    CKU(cudaMemcpyAsync(ids.p, hid, sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, c->stream));
    CKU(cudaMemcpyAsync(vals.p, hval, sizeof(int) * (size_t)(n * width), cudaMemcpyHostToDevice, c->stream));
    launch_scatter_rows_i32(n, width, P<int>(ids), P<int>(vals), dst, c->stream);
    CKU(cudaStreamSynchronize(c->stream));  // the staging buffers are reused
    return SPRG_OK;
  };
  if (d->n_vert_rows) {
    CKU(cudaMemcpyAsync(ids.p, d->vert_ids, sizeof(int) * (size_t)d->n_vert_rows, cudaMemcpyHostToDevice, c->stream));
    CKU(cudaMemcpyAsync(vals.p, d->coords, sizeof(double) * 3 * (size_t)d->n_vert_rows, cudaMemcpyHostToDevice,
                        c->stream));
    launch_scatter_rows_f64(d->n_vert_rows, 3, P<int>(ids), P<double>(vals), P<double>(nxyz), c->stream);
    CKU(cudaStreamSynchronize(c->stream));
  }
  if ((rc = scatter_i32(d->n_elem_rows, d->elem_ids, d->elem_verts, nn, P<int>(nev)))) return rc;
  if ((rc = scatter_i32(d->n_edge_rows, d->edge_ids, d->edge_verts, 2, P<int>(nedv)))) return rc;
  // kept rows may name vertices beyond a smaller vertex count
  CKU(cudaMemsetAsync(bad.p, 0, sizeof(unsigned long long), c->stream));
  launch_count_out_of_range(T1 * nn, P<int>(nev), (int)V1, P<unsigned long long>(bad), c->stream);
  launch_count_out_of_range(2 * E1, P<int>(nedv), (int)V1, P<unsigned long long>(bad), c->stream);
  unsigned long long nbad = 0;
  CKU(cudaMemcpyAsync(&nbad, bad.p, sizeof nbad, cudaMemcpyDeviceToHost, c->stream));
  CKU(cudaStreamSynchronize(c->stream));
  if (nbad) {
    cleanup();
    return fail(c, SPRG_EINVAL, "kept elements or edges name vertices beyond the new vertex count");
  }
  // ---- swap in, rebuild what derives from the arrays
  release(c->xyz); release(c->ev); release(c->edv);
  c->xyz = nxyz; c->ev = nev; c->edv = nedv;
  nxyz = DevBuf{}; nev = DevBuf{}; nedv = DevBuf{};
  cleanup();
#undef CKU
#undef ENSUREU
  m.V = (int)V1;
  m.T = (int)T1;
  m.E = (int)E1;
  m.xyz = P<double>(c->xyz);
  m.ev = P<int>(c->ev);
  m.edv = P<int>(c->edv);
  const size_t nel = (size_t)m.T * nn;
  ENSURE(c->xyzq, sizeof(int) * 4 * (size_t)m.V);
  m.xyzq = P<int>(c->xyzq);
  ENSURE(c->red, sizeof(double) * (size_t)(sum_partials_count() + 4));
  launch_bbox(m.V, m.xyz, P<unsigned long long>(c->red), c->stream);
  unsigned long long keys[6];
  CK(cudaMemcpyAsync(keys, c->red.p, sizeof keys, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  double lo[3], hi[3];
  for (int k = 0; k < 3; ++k) {
    lo[k] = key_to_double(keys[k]);
    hi[k] = key_to_double(keys[3 + k]);
  }
  set_frame(c, lo, hi);
  launch_xyz_to_fixed(m, c->frame, P<int>(c->xyzq), c->stream);
  ENSURE(c->poff, sizeof(int) * ((size_t)m.V + 1));
  ENSURE(c->pel, sizeof(int) * nel);
  ENSURE(c->tmp, sizeof(int) * (size_t)m.V);
  if (d->vert_elem_offsets) {
    ENSURE(c->aoff, sizeof(int) * ((size_t)m.V + 1));
    ENSURE(c->ael, sizeof(int) * nel);
    CK(cudaMemcpyAsync(c->aoff.p, d->vert_elem_offsets, sizeof(int) * ((size_t)m.V + 1), cudaMemcpyHostToDevice,
                       c->stream));
    CK(cudaMemcpyAsync(c->ael.p, d->vert_elems, sizeof(int) * nel, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->poff.p, c->aoff.p, sizeof(int) * ((size_t)m.V + 1), cudaMemcpyDeviceToDevice, c->stream));
    CK(cudaMemcpyAsync(c->pel.p, c->ael.p, sizeof(int) * nel, cudaMemcpyDeviceToDevice, c->stream));
    launch_sort_segments(m.V, P<int>(c->poff), P<int>(c->pel), c->stream);
    m.a_off = P<int>(c->aoff);
    m.a_el = P<int>(c->ael);
  } else {
    launch_build_v2e(m, P<int>(c->poff), P<int>(c->pel), P<int>(c->tmp), c->stream);
    launch_sort_segments(m.V, P<int>(c->poff), P<int>(c->pel), c->stream);
    m.a_off = P<int>(c->poff);
    m.a_el = P<int>(c->pel);
  }
  m.p_off = P<int>(c->poff);
  m.p_el = P<int>(c->pel);
  c->launches += 5;
  if ((rc = check_launch(c, "mesh update"))) return rc;
  CK(cudaStreamSynchronize(c->stream));
  invalidate_mesh_state(c);
  return SPRG_OK;
}

int sprg_destroy(sprg_ctx* c) {
  if (!c) return SPRG_OK;
  cudaSetDevice(c->device);
  if (c->own) cudaStreamSynchronize(c->own);
  DevBuf* bufs[] = {&c->soff, &c->sel, &c->sw, &c->qmax, &c->bcnt, &c->cent, &c->xyz,   &c->xyzq,   &c->ev,   &c->edv,   &c->poff,    &c->pel,    &c->aoff,
                    &c->ael,   &c->tmp,     &c->f,    &c->ip,    &c->rec,     &c->err,    &c->esize,
                    &c->size,  &c->L,       &c->flags, &c->q,    &c->sizes3,  &c->frames9, &c->partials,
                    &c->out3,  &c->status,  &c->count, &c->mcount, &c->xitems, &c->xcount, &c->slab, &c->bits, &c->titems, &c->tcountb, &c->Lx, &c->pairs, &c->red, &c->eflags, &c->logm, &c->qw, &c->qwlisted, &c->qwitems, &c->qwcount, &c->tw, &c->twlisted, &c->twitems, &c->twcount, &c->met32, &c->qrec32, &c->cj64, &c->qties, &c->kidx, &c->kval, &c->klen, &c->rec9, &c->cache2d.v, &c->cache2d.n, &c->cache2d.el, &c->agitems, &c->agcount,
                    &c->crec,  &c->vrec,    &c->rec32, &c->q32, &c->sz2,  &c->fcnt,   &c->guard, &c->tetd,
                    &c->wts,   &c->w64,     &c->listed, &c->geo, &c->geo64, &c->elen, &c->fitems, &c->gstamp, &c->gfit, &c->grec, &c->tnext, &c->edone,
                    &c->hess, &c->pcls, &c->bverts, &c->btiles, &c->bnext, &c->bvoff, &c->bseg, &c->bsegoff, &c->bratios, &c->vvoff, &c->vv, &c->vtile, &c->vr16, &c->rec16,
                    &c->ql,    &c->sizel,   &c->fbitems, &c->fbcount, &c->mlp_packed, &c->mlp_err, &c->mlp_tmp, &c->lrange, &c->ldone, &c->lsc,
                    &c->cache64.v, &c->cache64.n, &c->cache64.el, &c->cache32.v, &c->cache32.n, &c->cache32.el,
                    &c->cache64.woff, &c->cache64.w, &c->cache64.wn, &c->cache32.woff, &c->cache32.w,
                    &c->cache32.wn};
  for (DevBuf* b : bufs) release(*b);
  for (auto& e : c->ev_pool) cudaEventDestroy(e);
  if (c->copy) {
    cudaStreamSynchronize(c->copy);
    cudaStreamDestroy(c->copy);
    cudaEventDestroy(c->copy_fork);
    cudaEventDestroy(c->copy_join);
    if (c->size_ready) cudaEventDestroy(c->size_ready);
    if (c->size_join) cudaEventDestroy(c->size_join);
  }
  for (auto& e : c->e2e_ev)
    if (e) cudaEventDestroy(e);
  if (c->stage) cudaFreeHost(c->stage);
  if (c->side) {
    cudaStreamSynchronize(c->side);
    cudaStreamDestroy(c->side);
  }
  if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
  if (c->e2e_exec) cudaGraphExecDestroy(c->e2e_exec);
  if (c->fork) cudaEventDestroy(c->fork);
  if (c->join) cudaEventDestroy(c->join);
  if (c->own) cudaStreamDestroy(c->own);
  delete c;
  return SPRG_OK;
}

const char* sprg_last_error(const sprg_ctx* c) { return c ? c->err_msg.c_str() : "null context"; }

int sprg_set_precision(sprg_ctx* c, int precision) {
  if (!c) return SPRG_EINVAL;
  if (precision != SPRG_FP64 && precision != SPRG_FP32 && precision != SPRG_LEARNED)
    return fail(c, SPRG_EINVAL, "unknown precision");
  if (precision == SPRG_LEARNED && c->m.dim != 3)
    return fail(c, SPRG_EINVAL, "the learned form covers tet meshes");
  c->precision = precision;
  drop_e2e_graph(c);
  return SPRG_OK;
}

int sprg_set_stream(sprg_ctx* c, void* stream) {
  if (!c) return SPRG_EINVAL;
  c->stream = stream ? static_cast<cudaStream_t>(stream) : c->own;
  drop_e2e_graph(c);
  return SPRG_OK;
}

int64_t sprg_last_launch_count(const sprg_ctx* c) { return c ? c->launches : 0; }

int sprg_get_grad_ip_field(sprg_ctx* c, const double* f, int ncomp_in, int order, double* ip_out) {
  if (!c || !f) return SPRG_EINVAL;
  if (order != 1) return fail(c, SPRG_EINVAL, "only integration order 1 is supported");
  if (ncomp_in != 1 && ncomp_in != 3) return fail(c, SPRG_EINVAL, "field must be SCALAR (1) or VECTOR (3)");
  int rc = set_device(c);
  if (rc) return rc;
  c->launches = 0;
  DevMesh& m = c->m;
  ENSURE(c->f, sizeof(double) * (size_t)m.V * ncomp_in);
  CK(cudaMemcpyAsync(c->f.p, f, sizeof(double) * (size_t)m.V * ncomp_in, cudaMemcpyHostToDevice, c->stream));
  int saved = c->precision;
  c->precision = SPRG_FP64;  // the explicit ip field is always the FP64 one
  rc = step_grad(c, ncomp_in);
  c->precision = saved;
  if (rc) return rc;
  if (ip_out)
    CK(cudaMemcpyAsync(ip_out, c->ip.p, sizeof(double) * (size_t)m.T * 3 * ncomp_in, cudaMemcpyDeviceToHost,
                       c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return SPRG_OK;
}

int sprg_recover_field(sprg_ctx* c, const double* ip, int ncomp, double* out) {
  if (!c) return SPRG_EINVAL;
  int rc = set_device(c);
  if (rc) return rc;
  c->launches = 0;
  int saved = c->precision;
  rc = upload_ip(c, ip, ncomp);
  if (rc) return rc;
  c->precision = SPRG_FP64;  // explicit ip fields take the FP64 path
  if ((rc = reset_status(c)) || (rc = step_recover(c))) { c->precision = saved; return rc; }
  c->precision = saved;
  if (out)
    CK(cudaMemcpyAsync(out, c->rec.p, sizeof(double) * (size_t)c->m.V * ncomp, cudaMemcpyDeviceToHost, c->stream));
  return sync_and_status(c);
}

static int size_field_common(sprg_ctx* c, const double* ip, int ncomp, int mode, double adapt_ratio, double target,
                             double alpha, double beta, double* size_out, sprg_size_info* info) {
  int rc = set_device(c);
  if (rc) return rc;
  c->launches = 0;
  rc = upload_ip(c, ip, ncomp);
  if (rc) return rc;
  int saved = c->precision;
  c->precision = SPRG_FP64;
  if ((rc = reset_status(c)) || (rc = step_recover(c)) ||
      (rc = step_size(c, mode, adapt_ratio, target, alpha, beta))) {
    c->precision = saved;
    return rc;
  }
  c->precision = saved;
  if (size_out)
    CK(cudaMemcpyAsync(size_out, c->size.p, sizeof(double) * (size_t)c->m.V, cudaMemcpyDeviceToHost, c->stream));
  rc = sync_and_status(c);
  if (rc) return rc;
  return fill_info(c, info);
}

int sprg_get_spr_size_field(sprg_ctx* c, const double* ip, int ncomp, double adapt_ratio, double* size_out,
                            sprg_size_info* info) {
  if (!c) return SPRG_EINVAL;
  if (!(adapt_ratio > 0)) return fail(c, SPRG_EINVAL, "adapt_ratio must be positive");
  return size_field_common(c, ip, ncomp, 0, adapt_ratio, 0, 0, 0, size_out, info);
}

int sprg_get_target_spr_size_field(sprg_ctx* c, const double* ip, int ncomp, size_t target, double alpha,
                                   double beta, double* size_out, sprg_size_info* info) {
  if (!c) return SPRG_EINVAL;
  if (target == 0) return fail(c, SPRG_EINVAL, "target must be > 0");   // spr/sprEstimateTargetError.cc:250
  if (!(alpha < beta)) return fail(c, SPRG_EINVAL, "alpha must be < beta");  // :251
  return size_field_common(c, ip, ncomp, 1, 0, (double)target, alpha, beta, size_out, info);
}

int sprg_measure_edges(sprg_ctx* c, const double* size, double* lengths) {
  if (!c) return SPRG_EINVAL;
  int rc = set_device(c);
  if (rc) return rc;
  c->launches = 0;
  if (size) {
    ENSURE(c->size, sizeof(double) * (size_t)c->m.V);
    CK(cudaMemcpyAsync(c->size.p, size, sizeof(double) * (size_t)c->m.V, cudaMemcpyHostToDevice, c->stream));
    c->size_valid = true;
  } else if (!c->size_valid) {
    return fail(c, SPRG_ESTATE, "no resident size field");
  }
  rc = step_measure_iso(c);
  if (rc) return rc;
  if (lengths)
    CK(cudaMemcpyAsync(lengths, c->L.p, sizeof(double) * (size_t)c->m.E, cudaMemcpyDeviceToHost, c->stream));
  return sync_and_status(c);
}

int sprg_measure_edges_aniso(sprg_ctx* c, const double* sizes, const double* frames, double* lengths) {
  if (!c || !sizes || !frames) return SPRG_EINVAL;
  int rc = set_device(c);
  if (rc) return rc;
  c->launches = 0;
  DevMesh& m = c->m;
  ENSURE(c->sizes3, sizeof(double) * 3 * (size_t)m.V);
  ENSURE(c->frames9, sizeof(double) * 9 * (size_t)m.V);
  ENSURE(c->L, sizeof(double) * (size_t)m.E);
  CK(cudaMemcpyAsync(c->sizes3.p, sizes, sizeof(double) * 3 * (size_t)m.V, cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(c->frames9.p, frames, sizeof(double) * 9 * (size_t)m.V, cudaMemcpyHostToDevice, c->stream));
  launch_measure_aniso_f64(m, P<double>(c->sizes3), P<double>(c->frames9), P<double>(c->L), c->stream);
  c->launches += 1;
  rc = check_launch(c, "measure aniso");
  if (rc) return rc;
  c->L_valid = true;
  if (lengths)
    CK(cudaMemcpyAsync(lengths, c->L.p, sizeof(double) * (size_t)m.E, cudaMemcpyDeviceToHost, c->stream));
  return sync_and_status(c);
}

static int apply_bits(sprg_ctx* c, int which, const uint32_t* bits, int* d_flags) {
  CK(cudaMemsetAsync(c->count.p, 0, sizeof(unsigned long long), c->stream));
  launch_apply_bits(c->m.E, bits, which, d_flags, P<unsigned long long>(c->count), P<DevStatus>(c->status),
                    c->stream);
  c->launches += 1;
  return check_launch(c, "apply marks");
}

static int mark_resident(sprg_ctx* c, int which, int* d_flags) {
  CK(cudaMemsetAsync(c->count.p, 0, sizeof(unsigned long long), c->stream));
  launch_mark(c->m.E, P<double>(c->L), which, d_flags, P<unsigned long long>(c->count), P<DevStatus>(c->status),
              c->stream);
  c->launches += 1;
  return check_launch(c, "mark");
}

int sprg_mark_edges(sprg_ctx* c, int which, int32_t* flags, long* count) {
  if (!c || !flags) return SPRG_EINVAL;
  if (which != SPRG_MARK_SPLIT && which != SPRG_MARK_COLLAPSE) return fail(c, SPRG_EINVAL, "unknown mark pass");
  if (!c->L_valid) return fail(c, SPRG_ESTATE, "no resident edge lengths (call sprg_measure_edges first)");
  int rc = set_device(c);
  if (rc) return rc;
  c->launches = 0;
  DevMesh& m = c->m;
  ENSURE(c->flags, sizeof(int) * (size_t)m.E);
  CK(cudaMemcpyAsync(c->flags.p, flags, sizeof(int) * (size_t)m.E, cudaMemcpyHostToDevice, c->stream));
  if ((rc = reset_status(c)) || (rc = mark_resident(c, which, P<int>(c->flags)))) return rc;
  unsigned long long n = 0;
  CK(cudaMemcpyAsync(&n, c->count.p, sizeof n, cudaMemcpyDeviceToHost, c->stream));
  rc = sync_and_status(c);
  if (rc) return rc;  // flags left untouched on the host on error
  CK(cudaMemcpy(flags, c->flags.p, sizeof(int) * (size_t)m.E, cudaMemcpyDeviceToHost));
  if (count) *count = (long)n;
  return SPRG_OK;
}

int sprg_measure_quality(sprg_ctx* c, const double* size, const double* sizes, const double* frames, double* q) {
  if (!c || !q) return SPRG_EINVAL;
  if ((sizes == nullptr) != (frames == nullptr)) return fail(c, SPRG_EINVAL, "sizes and frames go together");
  int rc = set_device(c);
  if (rc) return rc;
  c->launches = 0;
  DevMesh& m = c->m;
  ENSURE(c->q, sizeof(double) * (size_t)m.T);
  const double* dsize = nullptr;
  const double* dsizes = nullptr;
  const double* dframes = nullptr;
  if (sizes) {
    ENSURE(c->sizes3, sizeof(double) * 3 * (size_t)m.V);
    ENSURE(c->frames9, sizeof(double) * 9 * (size_t)m.V);
    CK(cudaMemcpyAsync(c->sizes3.p, sizes, sizeof(double) * 3 * (size_t)m.V, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->frames9.p, frames, sizeof(double) * 9 * (size_t)m.V, cudaMemcpyHostToDevice, c->stream));
    dsizes = P<double>(c->sizes3);
    dframes = P<double>(c->frames9);
  } else {
    if (size) {
      ENSURE(c->size, sizeof(double) * (size_t)m.V);
      CK(cudaMemcpyAsync(c->size.p, size, sizeof(double) * (size_t)m.V, cudaMemcpyHostToDevice, c->stream));
      c->size_valid = true;
    } else if (!c->size_valid) {
      return fail(c, SPRG_ESTATE, "no resident size field");
    }
    dsize = P<double>(c->size);
  }
  launch_quality_f64(m, dsize, dsizes, dframes, P<double>(c->q), c->stream);
  c->launches += 1;
  rc = check_launch(c, "quality");
  if (rc) return rc;
  c->q_valid = true;
  CK(cudaMemcpyAsync(q, c->q.p, sizeof(double) * (size_t)m.T, cudaMemcpyDeviceToHost, c->stream));
  return sync_and_status(c);
}

// ---- MA sweeps around the marks ----------------------------------------

// device inputs of a size field of the given kind (uploads host arrays;
// an isotropic field without `size` is the resident one; the log-
// interpolated field gets its per-vertex log-metrics in *dlm)
static int size_field_inputs(sprg_ctx* c, int kind, const double* size, const double* sizes, const double* frames,
                             const double** ds, const double** dss, const double** dff, const double** dlm) {
  DevMesh& m = c->m;
  *ds = *dss = *dff = *dlm = nullptr;
  if (kind == SPRG_SIZE_IDENTITY) return SPRG_OK;
  if (kind == SPRG_SIZE_ISO) {
    if (size) {
      ENSURE(c->size, sizeof(double) * (size_t)m.V);
      CK(cudaMemcpyAsync(c->size.p, size, sizeof(double) * (size_t)m.V, cudaMemcpyHostToDevice, c->stream));
      c->size_valid = true;
    } else if (!c->size_valid) {
      return fail(c, SPRG_ESTATE, "no resident size field");
    }
    *ds = P<double>(c->size);
    return SPRG_OK;
  }
  if (kind == SPRG_SIZE_ANISO || kind == SPRG_SIZE_LOG_ANISO) {
    if (!sizes || !frames) return fail(c, SPRG_EINVAL, "an anisotropic size field needs sizes and frames");
    ENSURE(c->sizes3, sizeof(double) * 3 * (size_t)m.V);
    ENSURE(c->frames9, sizeof(double) * 9 * (size_t)m.V);
    CK(cudaMemcpyAsync(c->sizes3.p, sizes, sizeof(double) * 3 * (size_t)m.V, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->frames9.p, frames, sizeof(double) * 9 * (size_t)m.V, cudaMemcpyHostToDevice, c->stream));
    *dss = P<double>(c->sizes3);
    *dff = P<double>(c->frames9);
    if (kind == SPRG_SIZE_LOG_ANISO) {
      ENSURE(c->logm, sizeof(double) * 9 * (size_t)(m.V > 0 ? m.V : 1));
      launch_log_metric(m.V, *dss, *dff, P<double>(c->logm), c->stream);
      c->launches += 1;
      *dlm = P<double>(c->logm);
    }
    return SPRG_OK;
  }
  return fail(c, SPRG_EINVAL, "unknown size field kind");
}

int sprg_measure_vertex_pairs(sprg_ctx* c, int kind, const double* size, const double* sizes, const double* frames,
                              int64_t n_pairs, const int32_t* pairs, double* lengths) {
  if (!c || n_pairs < 0 || (n_pairs > 0 && (!pairs || !lengths))) return SPRG_EINVAL;
  const int V = c->m.V;
  for (int64_t i = 0; i < 2 * n_pairs; ++i)
    if (pairs[i] < 0 || pairs[i] >= V) return fail(c, SPRG_EINVAL, "vertex id out of range");
  int rc = set_device(c);
  if (rc) return rc;
  c->launches = 0;
  const double *ds, *dss, *dff, *dlm;
  if ((rc = reset_status(c))) return rc;
  if ((rc = size_field_inputs(c, kind, size, sizes, frames, &ds, &dss, &dff, &dlm))) return rc;
  if (n_pairs == 0) return sync_and_status(c);
  ENSURE(c->pairs, sizeof(int) * 2 * (size_t)n_pairs);
  ENSURE(c->Lx, sizeof(double) * (size_t)n_pairs);
  CK(cudaMemcpyAsync(c->pairs.p, pairs, sizeof(int) * 2 * (size_t)n_pairs, cudaMemcpyHostToDevice, c->stream));
  launch_measure_pairs(c->m, kind, n_pairs, P<int>(c->pairs), ds, dss, dff, dlm, P<double>(c->Lx),
                       P<DevStatus>(c->status), c->stream);
  c->launches += 1;
  if ((rc = check_launch(c, "measure pairs"))) return rc;
  CK(cudaMemcpyAsync(lengths, c->Lx.p, sizeof(double) * (size_t)n_pairs, cudaMemcpyDeviceToHost, c->stream));
  return sync_and_status(c);
}

int sprg_get_maximum_edge_length(sprg_ctx* c, int kind, const double* size, const double* sizes,
                                 const double* frames, double* out) {
  if (!c || !out) return SPRG_EINVAL;
  int rc = set_device(c);
  if (rc) return rc;
  c->launches = 0;
  DevMesh& m = c->m;
  const double *ds, *dss, *dff, *dlm;
  if ((rc = reset_status(c))) return rc;
  if ((rc = size_field_inputs(c, kind, size, sizes, frames, &ds, &dss, &dff, &dlm))) return rc;
  ENSURE(c->Lx, sizeof(double) * (size_t)(m.E > 0 ? m.E : 1));
  ENSURE(c->red, sizeof(double) * (size_t)(sum_partials_count() + 4));
  launch_measure_pairs(m, kind, m.E, nullptr, ds, dss, dff, dlm, P<double>(c->Lx), P<DevStatus>(c->status),
                       c->stream);
  launch_max_positive(m.E, P<double>(c->Lx), P<unsigned long long>(c->red), c->stream);
  c->launches += 2;
  if ((rc = check_launch(c, "maximum edge length"))) return rc;
  unsigned long long bits = 0;
  CK(cudaMemcpyAsync(&bits, c->red.p, sizeof bits, cudaMemcpyDeviceToHost, c->stream));
  if ((rc = sync_and_status(c))) return rc;
  double v;
  std::memcpy(&v, &bits, sizeof v);
  *out = v;
  return SPRG_OK;
}

int sprg_get_average_edge_length(sprg_ctx* c, double* out) {
  if (!c || !out) return SPRG_EINVAL;
  int rc = set_device(c);
  if (rc) return rc;
  c->launches = 0;
  DevMesh& m = c->m;
  ENSURE(c->Lx, sizeof(double) * (size_t)(m.E > 0 ? m.E : 1));
  ENSURE(c->red, sizeof(double) * (size_t)(sum_partials_count() + 4));
  launch_measure_pairs(m, SPRG_SIZE_IDENTITY, m.E, nullptr, nullptr, nullptr, nullptr, nullptr, P<double>(c->Lx),
                       nullptr, c->stream);
  double* partials = P<double>(c->red) + 4;
  launch_sum(m.E, P<double>(c->Lx), partials, P<double>(c->red), c->stream);
  c->launches += 3;
  if ((rc = check_launch(c, "average edge length"))) return rc;
  double sum = 0;
  CK(cudaMemcpyAsync(&sum, c->red.p, sizeof sum, cudaMemcpyDeviceToHost, c->stream));
  if ((rc = sync_and_status(c))) return rc;
  *out = sum / (double)m.E;
  return SPRG_OK;
}

int sprg_measure_edges_log_aniso(sprg_ctx* c, const double* sizes, const double* frames, double* lengths) {
  if (!c || !sizes || !frames) return SPRG_EINVAL;
  int rc = set_device(c);
  if (rc) return rc;
  c->launches = 0;
  DevMesh& m = c->m;
  const double *ds, *dss, *dff, *dlm;
  if ((rc = reset_status(c))) return rc;
  if ((rc = size_field_inputs(c, SPRG_SIZE_LOG_ANISO, nullptr, sizes, frames, &ds, &dss, &dff, &dlm))) return rc;
  ENSURE(c->L, sizeof(double) * (size_t)(m.E > 0 ? m.E : 1));
  launch_measure_pairs(m, SPRG_SIZE_LOG_ANISO, m.E, nullptr, nullptr, nullptr, nullptr, dlm, P<double>(c->L),
                       P<DevStatus>(c->status), c->stream);
  c->launches += 1;
  if ((rc = check_launch(c, "measure log-aniso"))) return rc;
  if ((rc = sync_and_status(c))) return rc;
  c->L_valid = true;
  if (lengths) CK(cudaMemcpy(lengths, c->L.p, sizeof(double) * (size_t)m.E, cudaMemcpyDeviceToHost));
  return SPRG_OK;
}

int sprg_measure_quality_log_aniso(sprg_ctx* c, const double* sizes, const double* frames, double* q) {
  if (!c || !sizes || !frames || !q) return SPRG_EINVAL;
  int rc = set_device(c);
  if (rc) return rc;
  c->launches = 0;
  DevMesh& m = c->m;
  const double *ds, *dss, *dff, *dlm;
  if ((rc = reset_status(c))) return rc;
  if ((rc = size_field_inputs(c, SPRG_SIZE_LOG_ANISO, nullptr, sizes, frames, &ds, &dss, &dff, &dlm))) return rc;
  ENSURE(c->q, sizeof(double) * (size_t)(m.T > 0 ? m.T : 1));
  launch_quality_f64(m, nullptr, nullptr, nullptr, P<double>(c->q), c->stream, dlm, P<DevStatus>(c->status));
  c->launches += 1;
  if ((rc = check_launch(c, "quality log-aniso"))) return rc;
  if ((rc = sync_and_status(c))) return rc;
  c->q_valid = true;
  CK(cudaMemcpy(q, c->q.p, sizeof(double) * (size_t)m.T, cudaMemcpyDeviceToHost));
  return SPRG_OK;
}

int sprg_max_iterations_for_length(double max_metric_length) {
  const int iter = (int)std::ceil(std::log2(max_metric_length));
  return iter >= 10 ? 10 : iter + 1;
}

int sprg_mark_bad_quality(sprg_ctx* c, double good_quality, int32_t* flags, long* count) {
  if (!c || !flags) return SPRG_EINVAL;
  if (!c->q_valid) return fail(c, SPRG_ESTATE, "no resident element qualities (call sprg_measure_quality first)");
  int rc = set_device(c);
  if (rc) return rc;
  c->launches = 0;
  DevMesh& m = c->m;
  ENSURE(c->eflags, sizeof(int) * (size_t)(m.T > 0 ? m.T : 1));
  CK(cudaMemcpyAsync(c->eflags.p, flags, sizeof(int) * (size_t)m.T, cudaMemcpyHostToDevice, c->stream));
  if ((rc = reset_status(c))) return rc;
  CK(cudaMemsetAsync(c->count.p, 0, sizeof(unsigned long long), c->stream));
  launch_mark_quality(m.T, P<double>(c->q), good_quality, P<int>(c->eflags), P<unsigned long long>(c->count),
                      P<DevStatus>(c->status), c->stream);
  c->launches += 1;
  if ((rc = check_launch(c, "mark bad quality"))) return rc;
  unsigned long long n = 0;
  CK(cudaMemcpyAsync(&n, c->count.p, sizeof n, cudaMemcpyDeviceToHost, c->stream));
  if ((rc = sync_and_status(c))) return rc;  // flags left untouched on the host on error
  CK(cudaMemcpy(flags, c->eflags.p, sizeof(int) * (size_t)m.T, cudaMemcpyDeviceToHost));
  if (count) *count = (long)n;
  return SPRG_OK;
}

int sprg_get_min_quality(sprg_ctx* c, double* out) {
  if (!c || !out) return SPRG_EINVAL;
  if (!c->q_valid) return fail(c, SPRG_ESTATE, "no resident element qualities (call sprg_measure_quality first)");
  int rc = set_device(c);
  if (rc) return rc;
  c->launches = 0;
  DevMesh& m = c->m;
  ENSURE(c->red, sizeof(double) * (size_t)(sum_partials_count() + 4));
  unsigned long long* key = P<unsigned long long>(c->red);
  launch_first_min_below(m.T, P<double>(c->q), 1.0, key, key + 1, c->stream);
  c->launches += 2;
  if ((rc = check_launch(c, "minimum quality"))) return rc;
  unsigned long long first = 0;
  CK(cudaMemcpyAsync(&first, key + 1, sizeof first, cudaMemcpyDeviceToHost, c->stream));
  if ((rc = sync_and_status(c))) return rc;
  if (first == ~0ull) {
    *out = 1.0;  // no element below the reference's starting value
    return SPRG_OK;
  }
  CK(cudaMemcpy(out, P<double>(c->q) + first, sizeof(double), cudaMemcpyDeviceToHost));
  return SPRG_OK;
}

static SlicedPatches sliced_view(sprg_ctx* c) {
  return SlicedPatches{P<int>(c->soff), P<int>(c->sel), P<float>(c->sw)};
}

static BatchView batch_view(sprg_ctx* c) {
  if (!c->batch_n) return BatchView{0, nullptr, nullptr, nullptr, nullptr};
  return BatchView{c->batch_n, P<int>(c->bvoff), P<int2>(c->bseg), P<int>(c->bsegoff), P<double>(c->bratios)};
}

// per mesh (FP32 and learned forms): coordinate records, element and edge
// geometry, SPR weights and the listed patches
static int fast_setup(sprg_ctx* c, ExpandList xl) {
  if (c->vrec_ready) return SPRG_OK;
  DevMesh& m = c->m;
  int rc;
  const size_t nel = (size_t)m.T * m.nn;
  ENSURE(c->crec, 32 * (size_t)m.V);
  ENSURE(c->wts, sizeof(float) * nel);
  ENSURE(c->w64, sizeof(double) * nel);
  ENSURE(c->listed, (size_t)m.V);
  ENSURE(c->geo, 8 * (size_t)m.T);
  ENSURE(c->geo64, 16 * (size_t)m.T);
  ENSURE(c->cent, 24 * (size_t)m.T);
  ENSURE(c->qmax, sizeof(unsigned long long));
  ENSURE(c->elen, 4 * (size_t)m.E);
  CK(cudaMemsetAsync(c->fcnt.p, 0, 8 * sizeof(int), c->stream));
  PB("setup_coords");
  fast_prep_coords(m, c->frame, P<float4>(c->crec), c->stream);
  PE();
  c->crec_ready = true;
  PB("setup_geometry");
  fast_geometry(m, P<float2>(c->geo), P<double2>(c->geo64), P<double>(c->cent), P<unsigned long long>(c->qmax),
                P<float>(c->elen), c->stream);
  PE();
  PB("setup_weights");
  fast_weights(m, P<double>(c->cent), P<float>(c->wts), P<double>(c->w64), xl, P<int>(c->fcnt),
               P<unsigned char>(c->listed), c->stream);
  PE();
  int h[2] = {0, 0};
  CK(cudaMemcpyAsync(&h[0], P<int>(c->fcnt) + 3, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaMemcpyAsync(&h[1], c->fcnt.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  if ((rc = check_launch(c, "fast setup"))) return rc;
  c->n_listed = h[0] < m.V ? h[0] : m.V;
  c->n_refit = h[1];
  c->vrec_ready = true;
  return SPRG_OK;
}

// the listed patches' FP64 fits: the first pass grows the patches (and
// caches them) in order; later passes run the cached fits on the side
// stream, joined by the caller before the results are used
static int listed_fork(sprg_ctx* c, ExpandList xl, bool* forked) {
  *forked = false;
  if (!c->cache32.valid) return SPRG_OK;
  int wrc = ensure_cache_weights(c, c->cache32);
  if (wrc) return wrc;
  if (!c->side) {
    CK(cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&c->fork, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&c->join, cudaEventDisableTiming));
  }
  CK(cudaEventRecord(c->fork, c->stream));
  CK(cudaStreamWaitEvent(c->side, c->fork, 0));
  int rc = listed_fits(c, c->cache32, nullptr, P<double>(c->f), 3, P<double>(c->rec), xl, c->side);
  if (rc) return rc;
  CK(cudaEventRecord(c->join, c->side));
  *forked = true;
  return SPRG_OK;
}

static int listed_join(sprg_ctx* c, ExpandList xl, bool forked) {
  if (forked) {
    CK(cudaStreamWaitEvent(c->stream, c->join, 0));
    return SPRG_OK;
  }
  return listed_fits(c, c->cache32, nullptr, P<double>(c->f), 3, P<double>(c->rec), xl);
}

// patch-size bins of the non-listed vertices (stable: ascending ids within a
// bin), once per mesh
// the sliced copy of the patch lists over the bins (after the bins and the
// weights): widths on the device, their exclusive sums x 32 on the host
static int build_slices(sprg_ctx* c) {
  DevMesh& m = c->m;
  BinSlices& bs = c->bslices;
  int start = 0, slices = 0;
  for (int b = 0; b < 4; ++b) {
    bs.start[b] = start;
    bs.slice0[b] = slices;
    start += c->bin_count[b];
    slices += (c->bin_count[b] + 31) / 32;
  }
  bs.start[4] = start;
  bs.slice0[4] = slices;
  c->sliced = false;
  ENSURE(c->soff, sizeof(int) * ((size_t)slices + 1));
  fast_slice_width(m, bs, P<int>(c->bverts), P<int>(c->soff), c->stream);
  std::vector<int> off((size_t)slices + 1);
  if (slices) CK(cudaMemcpyAsync(off.data(), c->soff.p, sizeof(int) * slices, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  long long run = 0;
  for (int k = 0; k < slices; ++k) {
    const long long wdt = off[k];
    off[k] = (int)run;
    run += 32 * wdt;
    if (run > INT32_MAX) return SPRG_OK;  // too large for int offsets: the CSR lane modes only
  }
  off[slices] = (int)run;
  CK(cudaMemcpyAsync(c->soff.p, off.data(), sizeof(int) * off.size(), cudaMemcpyHostToDevice, c->stream));
  ENSURE(c->sel, sizeof(int) * (size_t)(run > 0 ? run : 1));
  ENSURE(c->sw, sizeof(float) * (size_t)(run > 0 ? run : 1));
  CK(cudaMemsetAsync(c->sel.p, 0, sizeof(int) * (size_t)(run > 0 ? run : 1), c->stream));
  CK(cudaMemsetAsync(c->sw.p, 0, sizeof(float) * (size_t)(run > 0 ? run : 1), c->stream));
  fast_slice_fill(m, bs, P<int>(c->bverts), P<float>(c->wts), P<int>(c->soff), P<int>(c->sel), P<float>(c->sw),
                  c->stream);
  CK(cudaStreamSynchronize(c->stream));  // off lives on this frame
  int rc = check_launch(c, "sliced patch lists");
  if (rc) return rc;
  c->sliced = true;
  return SPRG_OK;
}

static int build_bins(sprg_ctx* c) {
  if (c->bins_ready) return SPRG_OK;
  DevMesh& m = c->m;
  int rc;
  ENSURE(c->pcls, (size_t)m.V);
  ENSURE(c->bverts, sizeof(int) * (size_t)m.V);
  ENSURE(c->bnext, sizeof(int));
  fast_patch_class(m, P<unsigned char>(c->listed), P<unsigned char>(c->pcls), c->stream);
  // per-block class counts -> per-class exclusive offsets of every block
  // (host scan of 4 ints per 1024 vertices) -> device scatter
  const int nb = fast_bin_blocks(m.V);
  ENSURE(c->bcnt, sizeof(int) * 8 * (size_t)nb);
  fast_bin_count(m.V, P<unsigned char>(c->pcls), P<int>(c->bcnt), c->stream);
  std::vector<int> cnt(4 * (size_t)nb), offs(4 * (size_t)nb);
  CK(cudaMemcpyAsync(cnt.data(), c->bcnt.p, sizeof(int) * cnt.size(), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  long long base = 0;
  for (int b = 0; b < 4; ++b) {
    long long run = base;
    for (int k = 0; k < nb; ++k) {
      offs[4 * (size_t)k + b] = (int)run;
      run += cnt[4 * (size_t)k + b];
    }
    c->bin_count[b] = (int)(run - base);
    base = run;
  }
  CK(cudaMemcpyAsync(P<int>(c->bcnt) + 4 * (size_t)nb, offs.data(), sizeof(int) * offs.size(),
                     cudaMemcpyHostToDevice, c->stream));
  fast_bin_scatter(m.V, P<unsigned char>(c->pcls), P<int>(c->bcnt) + 4 * (size_t)nb, P<int>(c->bverts), c->stream);
  CK(cudaStreamSynchronize(c->stream));  // offs lives on this frame
  if ((rc = check_launch(c, "patch-size bins"))) return rc;
  if ((rc = build_slices(c))) return rc;
  int dev = 0;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&c->n_sms, cudaDevAttrMultiProcessorCount, dev));
  c->bins_ready = true;
  return SPRG_OK;
}

// tiles (first, count, lanes, slice of first) of the current configuration;
// `only` >= 0 keeps one bin (autotuning).  A bin in the sliced mode without
// the sliced copy, or with tiles that do not start on a slice, takes 1 lane.
static int build_tiles(sprg_ctx* c, int only = -1) {
  std::vector<int4> tiles;
  int first = 0;
  c->tile_mode = -2;  // no tile yet
  for (int b = 0; b < 4; ++b) {
    int lanes = c->bin_lanes[b];
    if (lanes == 0 && (!c->sliced || c->tile_verts % 32)) lanes = 1;
    for (int i = 0; i < c->bin_count[b]; i += c->tile_verts) {
      const int n = std::min(c->tile_verts, c->bin_count[b] - i);
      if (only < 0 || only == b) {
        tiles.push_back(make_int4(first + i, n, lanes, c->bslices.slice0[b] + i / 32));
        c->tile_mode = c->tile_mode == -2 || c->tile_mode == lanes ? lanes : -1;
      }
    }
    first += c->bin_count[b];
  }
  ENSURE(c->btiles, sizeof(int4) * (tiles.empty() ? 1 : tiles.size()));
  if (!tiles.empty())
    CK(cudaMemcpy(c->btiles.p, tiles.data(), sizeof(int4) * tiles.size(), cudaMemcpyHostToDevice));
  c->n_tiles = (int)tiles.size();
  return SPRG_OK;
}

static void run_tiles(sprg_ctx* c, float4* rec32) {
  fast_recover_tiles(c->m, P<float>(c->wts), sliced_view(c), P<uint4>(c->tetd), rec32, P<int>(c->bverts),
                     P<int4>(c->btiles), c->n_tiles, c->tile_mode < 0 ? -1 : c->tile_mode, P<int>(c->bnext),
                     c->n_sms * c->grid_per_sm, c->stream);
}

// CUDA-event time of the binned recover under the current configuration
static float time_tiles(sprg_ctx* c, float4* rec32, int only) {
  if (build_tiles(c, only)) return 1e30f;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int r = 0; r < 3; ++r) {
    cudaEventRecord(e0, c->stream);
    run_tiles(c, rec32);
    cudaEventRecord(e1, c->stream);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return best;
}

// Autotuner (first pass, element gradients in place): coordinate descent
// over lanes per bin {1, 2, 4, 0 = sliced}, then that per-bin choice against
// one lane mode for every bin (a kernel specialised to it), tile size {64,
// 256, 1024} vertices and blocks per SM {4, 8, 16}; every configuration gives bitwise the same
// result, so the choice only changes time.  The choice and the timings are
// kept for sprg_tuning_report.
static int autotune(sprg_ctx* c, float4* rec32) {
  std::string log = "[";
  auto note = [&](const char* what, int val, float ms) {
    if (log.size() > 1) log += ",";
    log += "{\"" + std::string(what) + "\":" + std::to_string(val) + ",\"ms\":" + std::to_string(ms) + "}";
  };
  for (int b = 0; b < 4; ++b) {
    if (!c->bin_count[b]) continue;
    int best_l = c->bin_lanes[b];
    float best = 1e30f;
    for (int l : {1, 2, 4, 0}) {
      if (l == 0 && !c->sliced) continue;
      c->bin_lanes[b] = l;
      const float ms = time_tiles(c, rec32, b);
      note(("lanes_bin" + std::to_string(b)).c_str(), l, ms);
      if (ms < best) {
        best = ms;
        best_l = l;
      }
    }
    c->bin_lanes[b] = best_l;
  }
  {
    // one lane mode for every bin runs a kernel specialised to that mode
    // (fewer registers, more resident warps): the per-bin choice against
    // each uniform one, over the whole launch
    int chosen[4];
    for (int b = 0; b < 4; ++b) chosen[b] = c->bin_lanes[b];
    float best = time_tiles(c, rec32, -1);
    note("per_bin_lanes", 1, best);
    for (int l : {2, 4, 1, 0}) {
      if (l == 0 && !c->sliced) continue;
      for (int b = 0; b < 4; ++b) c->bin_lanes[b] = l;
      const float ms = time_tiles(c, rec32, -1);
      note("uniform_lanes", l, ms);
      if (ms < best) {
        best = ms;
        for (int b = 0; b < 4; ++b) chosen[b] = l;
      }
    }
    for (int b = 0; b < 4; ++b) c->bin_lanes[b] = chosen[b];
  }
  {
    int best_t = c->tile_verts;
    float best = 1e30f;
    for (int t : {64, 256, 1024}) {
      c->tile_verts = t;
      const float ms = time_tiles(c, rec32, -1);
      note("tile_verts", t, ms);
      if (ms < best) {
        best = ms;
        best_t = t;
      }
    }
    c->tile_verts = best_t;
  }
  {
    int best_g = c->grid_per_sm;
    float best = 1e30f;
    for (int g : {4, 8, 16}) {
      c->grid_per_sm = g;
      const float ms = time_tiles(c, rec32, -1);
      note("blocks_per_sm", g, ms);
      if (ms < best) {
        best = ms;
        best_g = g;
      }
    }
    c->grid_per_sm = best_g;
  }
  log += "]";
  int rc = build_tiles(c);
  if (rc) return rc;
  c->tune_json = "{\"bins\":[" + std::to_string(c->bin_count[0]) + "," + std::to_string(c->bin_count[1]) + "," +
                 std::to_string(c->bin_count[2]) + "," + std::to_string(c->bin_count[3]) + "],\"lanes\":[" +
                 std::to_string(c->bin_lanes[0]) + "," + std::to_string(c->bin_lanes[1]) + "," +
                 std::to_string(c->bin_lanes[2]) + "," + std::to_string(c->bin_lanes[3]) +
                 "],\"tile_verts\":" + std::to_string(c->tile_verts) +
                 ",\"blocks_per_sm\":" + std::to_string(c->grid_per_sm) + ",\"timings\":" + log + "}";
  c->tuned = true;
  return check_launch(c, "autotune");
}

// FP32 pass: packed double-float records, FP32 fits and sweeps, FP64
// reference path for ill-conditioned or growing patches (sprg_kernels_f32.cu).
static int pass_fast(sprg_ctx* c, double adapt_ratio, uint32_t* d_split, uint32_t* d_collapse) {
  DevMesh& m = c->m;
  int rc;
  if (m.dim != 3)
    return fail(c, SPRG_EINVAL, "the FP32 isotropic pass covers tet meshes (on triangles SPRG_FP32 is the mixed anisotropic pass)");
  const BatchView bv = batch_view(c);
  const int nb = bv.n ? c->batch_nseg : fast_error_blocks(m.T);
  const size_t nel = (size_t)m.T * m.nn;
  ENSURE(c->vrec, 32 * (size_t)m.V);
  ENSURE(c->rec32, 32 * (size_t)m.V);
  ENSURE(c->tetd, 16 * (size_t)m.T);
  ENSURE(c->tnext, sizeof(int));
  if (!c->edone.p) {
    ENSURE(c->edone, sizeof(unsigned));
    CK(cudaMemsetAsync(c->edone.p, 0, sizeof(unsigned), c->stream));
  }
  ENSURE(c->q32, 8 * (size_t)m.T);
  ENSURE(c->sz2, 8 * (size_t)m.V);
  ENSURE(c->rec, 24 * (size_t)m.V);
  ENSURE(c->fitems, sizeof(int) * (size_t)m.V);
  ENSURE(c->xcount, sizeof(int));
  ENSURE(c->slab, sizeof(double) * (size_t)expand_grid() * expand_max_elems() * (4 + 3 + 1));
  ENSURE(c->fcnt, 8 * sizeof(int));
  ENSURE(c->guard, sizeof(int) * (size_t)sprg_ctx::kGuardCap);
  ENSURE(c->partials, sizeof(double) * 2 * (size_t)(nb > 0 ? nb : 1));
  ENSURE(c->out3, sizeof(double) * 4 * (size_t)(bv.n > 0 ? bv.n : 1));
  if ((rc = reset_status(c))) return rc;
  // fcnt: [0] refit patches, [1] guard edges, [3] listed patches,
  // [4] unresolved guard edges, [5] rounding dominance (max |u| as float
  // bits from the prep kernel, then 0 / 1 from the error kernel's last
  // block) (0, 3 per mesh; 1, 4, 5 per pass)
  ExpandList xl{P<int>(c->fitems), P<int>(c->fcnt) + 3, m.V};
  float4* vrec = P<float4>(c->vrec);
  float4* rec32 = P<float4>(c->rec32);
  if ((rc = fast_setup(c, xl))) return rc;
  // the FP64 fits of the listed patches depend on the field only: once their
  // patches are cached they run on the side stream, beside the FP32 phases
  bool fork = false;
  if ((rc = listed_fork(c, xl, &fork))) return rc;
  CK(cudaMemsetAsync(P<int>(c->fcnt) + 1, 0, sizeof(int), c->stream));
  CK(cudaMemsetAsync(P<int>(c->fcnt) + 4, 0, 2 * sizeof(int), c->stream));
  PB("prep_f32");
  fast_prep(m, P<double>(c->f), P<float4>(c->crec), vrec, P<int>(c->fcnt) + 5, c->stream);
  PE();
  PB("tet_f32");
  fast_tet(m, vrec, P<double>(c->f), (float)c->frame[3], P<uint4>(c->tetd), P<int>(c->tnext), c->stream);
  PE();
  if (!c->bins_ready) {
    PB("setup_bins");
    if ((rc = build_bins(c))) return rc;
    if ((rc = build_tiles(c))) return rc;
    PE();
  }
  if (c->autotune && !c->tuned && (rc = autotune(c, rec32))) return rc;
  PB("recover_f32");
  run_tiles(c, rec32);
  PE();
  if ((rc = listed_join(c, xl, fork))) return rc;
  PB("merge_f64");
  fast_merge_ref(xl, P<double>(c->rec), rec32, c->stream);
  PE();
  // one mesh: the error kernel's last block also computes the size factor
  PB("error_f32");
  fast_error(m, P<uint4>(c->tetd), P<float2>(c->geo), rec32, P<float2>(c->q32), P<double>(c->partials), nb,
             bv.n ? P<int2>(c->bseg) : nullptr, bv.n ? nullptr : P<unsigned>(c->edone), adapt_ratio,
             P<double>(c->out3), P<int>(c->fcnt) + 5, P<unsigned long long>(c->qmax), c->stream);
  PE();
  if (bv.n) {
    PB("size_factor");
    launch_size_factor_batch(P<double>(c->partials), bv, m.dim, P<double>(c->out3), c->stream);
    PE();
  }
  PB("average_f32");
  fast_average(m, P<float2>(c->q32), P<double>(c->out3), P<float2>(c->sz2), bv, c->stream);
  PE();
  // while the pass is being captured into a graph, an external record (the
  // graph then records the event at this point on every replay)
  if (c->size_hook) {
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    CK(cudaStreamIsCapturing(c->stream, &cap));
    if (cap == cudaStreamCaptureStatusActive)
      CK(cudaEventRecordWithFlags(c->size_ready, c->stream, cudaEventRecordExternal));
    else
      CK(cudaEventRecord(c->size_ready, c->stream));
  }
  PB("measure_f32");
  fast_measure(m, P<float>(c->elen), P<float2>(c->sz2), d_split, d_collapse, P<int>(c->guard), P<int>(c->fcnt) + 1,
               sprg_ctx::kGuardCap, sprg_ctx::kGuardRel, c->stream);
  PE();
  if (!c->gstamp.p) {  // V stamps (zero) and the stamp-id counter (one)
    ENSURE(c->gstamp, sizeof(int) * ((size_t)m.V + 1));
    CK(cudaMemsetAsync(c->gstamp.p, 0, sizeof(int) * (size_t)m.V, c->stream));
    const int one = 1;
    CK(cudaMemcpyAsync(P<int>(c->gstamp) + m.V, &one, sizeof(int), cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
  }
  ENSURE(c->gfit, sizeof(int) * ((size_t)m.V + 1));
  ENSURE(c->grec, 3 * sizeof(double) * (size_t)m.V);
  GuardScratch gs{P<int>(c->gstamp), P<int>(c->gstamp) + m.V, P<int>(c->gfit) + 1,   P<int>(c->gfit),
                  m.V,               P<double>(c->grec), P<double>(c->w64),           P<unsigned char>(c->listed),
                  P<double>(c->rec), P<double2>(c->geo64)};
  static const char* const kGuardNames[kGuardStages] = {"guard_collect", "guard_fit", "guard_decide"};
  for (int stage = 0; stage < kGuardStages; ++stage) {
    PB(kGuardNames[stage]);
    launch_guard_stage(stage, m, P<double>(c->f), P<double>(c->out3), P<int>(c->guard), P<int>(c->fcnt) + 1,
                       sprg_ctx::kGuardCap, d_split, d_collapse, P<int>(c->fcnt) + 4, gs, bv, c->stream);
    PE();
  }
  c->launches += (bv.n ? 8 : 7) + kGuardStages;  // FP32-path and guard kernels (listed_fits counts its own)
  c->size_valid = false;  // the FP64 size buffer is filled on demand
  c->L_valid = false;
  return check_launch(c, "fast pass");
}

// the learned records' scratch: the field range's block partials, the
// last-block counter (zeroed when allocated; every pass leaves it zero) and
// the two difference scales
static int learned_scratch(sprg_ctx* c) {
  ENSURE(c->lrange, learned_range_bytes());
  if (!c->ldone.p) {
    ENSURE(c->ldone, sizeof(unsigned));
    CK(cudaMemsetAsync(c->ldone.p, 0, sizeof(unsigned), c->stream));
  }
  ENSURE(c->lsc, 2 * sizeof(float));
  return SPRG_OK;
}

// 2^-30 / s: the coordinate records' difference scale
static float learned_cs(const sprg_ctx* c) { return (float)(std::ldexp(1.0, -30) / c->frame[3]); }

static void learned_records(sprg_ctx* c, const double* d_u) {
  learned_prep(c->m, d_u, learned_cs(c), P<double>(c->lrange), P<unsigned>(c->ldone), P<float>(c->lsc),
               P<float4>(c->vr16), c->stream);
}

// Learned pass: network recovery with plain-SPR fallback, FP32 sweeps
// (sprg_learned.cu).
static int pass_learned(sprg_ctx* c, double adapt_ratio, uint32_t* d_split, uint32_t* d_collapse) {
  DevMesh& m = c->m;
  int rc;
  if (!c->have_mlp) return fail(c, SPRG_ESTATE, "learned form: no network parameters (sprg_set_mlp_params)");
  const int nb = learned_error_blocks(m.T);
  ENSURE(c->rec, 24 * (size_t)m.V);
  ENSURE(c->fitems, sizeof(int) * (size_t)m.V);
  ENSURE(c->xcount, sizeof(int));
  ENSURE(c->slab, sizeof(double) * (size_t)expand_grid() * expand_max_elems() * (4 + 3 + 1));
  ENSURE(c->fcnt, 8 * sizeof(int));
  ENSURE(c->partials, sizeof(double) * 2 * (size_t)(nb > 0 ? nb : 1));
  ENSURE(c->out3, sizeof(double) * 4);
  ENSURE(c->vr16, 16 * (size_t)m.V);
  ENSURE(c->rec16, 32 * (size_t)m.V);
  ENSURE(c->ql, 4 * (size_t)m.T);
  ENSURE(c->sizel, 4 * (size_t)m.V);
  ENSURE(c->fbitems, sizeof(int) * (size_t)m.V);
  ENSURE(c->fbcount, sizeof(int));
  ENSURE(c->mlp_err, sizeof(int));
  if ((rc = learned_scratch(c))) return rc;
  if ((rc = reset_status(c))) return rc;
  ExpandList xl{P<int>(c->fitems), P<int>(c->fcnt) + 3, m.V};
  if ((rc = fast_setup(c, xl))) return rc;
  if (!c->vv_ready) {
    ENSURE(c->vvoff, sizeof(int) * ((size_t)m.V + 1));
    ENSURE(c->vv, sizeof(int) * 2 * (size_t)m.E);
    ENSURE(c->tmp, sizeof(int) * (size_t)m.V);
    ENSURE(c->vtile, ((size_t)m.V + 127) / 128);
    learned_build_v2v(m, P<int>(c->vvoff), P<int>(c->vv), P<int>(c->tmp), P<unsigned char>(c->vtile),
                      P<int>(c->fcnt) + 6, c->stream);
    CK(cudaMemcpyAsync(&c->max_degree, P<int>(c->fcnt) + 6, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaMemsetAsync(c->mlp_err.p, 0, sizeof(int), c->stream));
    if ((rc = check_launch(c, "vertex adjacency"))) return rc;
    c->vv_ready = true;
  }
  bool fork = false;
  if ((rc = listed_fork(c, xl, &fork))) return rc;
  LearnMesh lm{P<int>(c->vvoff), P<int>(c->vv), P<unsigned char>(c->listed), P<unsigned char>(c->vtile)};
  float4* vr = P<float4>(c->vr16);
  float4* rec = P<float4>(c->rec16);
  CK(cudaMemsetAsync(c->fbcount.p, 0, sizeof(int), c->stream));
  PB("prep_l");
  learned_records(c, P<double>(c->f));
  PE();
  PB("mlp_l");
  CK(cudaMemsetAsync(c->mlp_err.p, 0, sizeof(int), c->stream));  // a wait that ran out is reported once
  learned_infer(m, lm, vr, P<float>(c->lsc), c->mlp_packed.p, rec, P<int>(c->fbitems), P<int>(c->fbcount), c->z_max,
                c->use_mlp, c->max_degree, c->stall_polls, P<int>(c->mlp_err), c->stream);
  PE();
  if ((rc = listed_join(c, xl, fork))) return rc;
  PB("fallback_l");
  learned_fallback(m, lm, vr, P<float>(c->lsc), P<float>(c->wts), P<double>(c->rec), P<int>(c->fbitems),
                   P<int>(c->fbcount), m.V, rec, c->stream);
  PE();
  PB("error_l");
  learned_error(m, rec, P<float>(c->lsc), P<float2>(c->geo), P<float>(c->ql), P<double>(c->partials), nb, c->stream);
  PE();
  PB("size_factor");
  launch_size_factor(P<double>(c->partials), nb, 0, adapt_ratio, 0, m.dim, P<double>(c->out3), c->stream);
  PE();
  PB("average_l");
  learned_average(m, P<float>(c->ql), P<double>(c->out3), P<float>(c->sizel), c->stream);
  PE();
  PB("measure_l");
  learned_measure(m, P<float>(c->elen), P<float>(c->sizel), d_split, d_collapse, c->stream);
  PE();
  c->launches += 8;  // range, prep, network, fallback, error, size factor, average, measure
  c->size_valid = false;
  c->L_valid = false;
  return check_launch(c, "learned pass");
}

static int pass_resident(sprg_ctx* c, double adapt_ratio, uint32_t* d_split, uint32_t* d_collapse) {
  int rc;
  if (c->batch_n && c->precision != SPRG_FP32)
    return fail(c, SPRG_EINVAL, "a batch of meshes runs in SPRG_FP32 (per-mesh size factors)");
  if (c->precision == SPRG_FP32) return pass_fast(c, adapt_ratio, d_split, d_collapse);
  if (c->precision == SPRG_LEARNED) return pass_learned(c, adapt_ratio, d_split, d_collapse);
  if ((rc = reset_status(c)) || (rc = step_grad(c, 1)) || (rc = step_recover(c)) ||
      (rc = step_size(c, 0, adapt_ratio, 0, 0, 0)) || (rc = step_measure_iso(c)))
    return rc;
  PB("mark_bits");
  launch_mark_bits(c->m.E, P<double>(c->L), d_split, d_collapse, c->stream);
  PE();
  c->launches += 1;
  return check_launch(c, "mark bits");
}

int sprg_estimate_and_mark_resident(sprg_ctx* c, const double* d_u, double adapt_ratio, uint32_t* d_split_bits,
                                    uint32_t* d_collapse_bits) {
  if (!c || !d_u || !d_split_bits || !d_collapse_bits) return SPRG_EINVAL;
  if (!(adapt_ratio > 0)) return fail(c, SPRG_EINVAL, "adapt_ratio must be positive");
  int rc = set_device(c);
  if (rc) return rc;
  c->launches = 0;
  ENSURE(c->f, sizeof(double) * (size_t)c->m.V);
  CK(cudaMemcpyAsync(c->f.p, d_u, sizeof(double) * (size_t)c->m.V, cudaMemcpyDeviceToDevice, c->stream));
  return pass_resident(c, adapt_ratio, d_split_bits, d_collapse_bits);
}

int sprg_rounding_dominated(sprg_ctx* c, int* out) {
  if (!c || !out) return SPRG_EINVAL;
  *out = 0;
  if (c->precision != SPRG_FP32 || c->batch_n || !c->fcnt.p) return SPRG_OK;
  int rc = set_device(c);
  if (rc) return rc;
  int v = 0;
  CK(cudaMemcpyAsync(&v, P<int>(c->fcnt) + 5, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  *out = v ? 1 : 0;
  return SPRG_OK;
}

// the resident pass of the host entry point: direct launches for the first
// two calls with a key, a captured graph from the third on
static int e2e_pass(sprg_ctx* c, double adapt_ratio, uint32_t* d_split, uint32_t* d_collapse) {
  const int call = c->e2e_calls++;
  if (c->prof || c->e2e_off) return pass_resident(c, adapt_ratio, d_split, d_collapse);
  if (c->e2e_exec) {
    CK(cudaGraphLaunch(c->e2e_exec, c->stream));
    c->launches += c->e2e_launches;
    return SPRG_OK;
  }
  if (call < 2) return pass_resident(c, adapt_ratio, d_split, d_collapse);
  const int64_t before = c->launches;
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal);
  int rc = SPRG_OK;
  if (e == cudaSuccess) {
    rc = pass_resident(c, adapt_ratio, d_split, d_collapse);
    e = cudaStreamEndCapture(c->stream, &graph);
    if (rc == SPRG_OK && e == cudaSuccess && graph) e = cudaGraphInstantiate(&c->e2e_exec, graph, 0);
  }
  if (graph) cudaGraphDestroy(graph);
  if (rc == SPRG_OK && e == cudaSuccess && c->e2e_exec) {
    c->e2e_launches = c->launches - before;
    CK(cudaGraphLaunch(c->e2e_exec, c->stream));
    return SPRG_OK;
  }
  // the pass did not capture: direct launches from now on
  cudaGetLastError();
  if (c->e2e_exec) cudaGraphExecDestroy(c->e2e_exec);
  c->e2e_exec = nullptr;
  c->e2e_off = true;
  c->launches = before;
  return pass_resident(c, adapt_ratio, d_split, d_collapse);
}

int sprg_estimate_and_mark(sprg_ctx* c, const double* u, double adapt_ratio, double* size_out, int32_t* flags,
                           long* n_split, long* n_collapse, sprg_size_info* info) {
  if (!c || !u) return SPRG_EINVAL;
  if (!(adapt_ratio > 0)) return fail(c, SPRG_EINVAL, "adapt_ratio must be positive");
  int rc = set_device(c);
  if (rc) return rc;
  c->launches = 0;
  DevMesh& m = c->m;
  ENSURE(c->f, sizeof(double) * (size_t)m.V);
  ENSURE(c->flags, sizeof(int) * (size_t)m.E);
  ENSURE(c->mcount, 2 * sizeof(unsigned long long));
  if ((rc = ensure_stage(c))) return rc;
  if (!c->copy) {
    CK(cudaStreamCreateWithFlags(&c->copy, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&c->copy_fork, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&c->copy_join, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&c->size_ready, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&c->size_join, cudaEventDisableTiming));
  }
  const auto t_call = std::chrono::steady_clock::now();
  if (c->e2e_timing && !c->e2e_ev[0])
    for (auto& e : c->e2e_ev) CK(cudaEventCreate(&e));
  auto mark = [&](int i, cudaStream_t s) { return c->e2e_timing ? cudaEventRecord(c->e2e_ev[i], s) : cudaSuccess; };
  CK(mark(0, c->stream));
  PB("upload_field");
  CK(cudaMemcpyAsync(c->f.p, u, sizeof(double) * (size_t)m.V, cudaMemcpyHostToDevice, c->stream));
  PE();
  CK(mark(1, c->stream));
  // the flag words are needed only by the write-back at the end: their
  // upload runs on the copy stream beside the pass, after the field's upload
  // (which then has the link to itself) and this stream's earlier work
  // (which may still read the buffer)
  if (flags) {
    CK(cudaEventRecord(c->copy_fork, c->stream));
    CK(cudaStreamWaitEvent(c->copy, c->copy_fork, 0));
    CK(mark(7, c->copy));
    CK(cudaMemcpyAsync(c->flags.p, flags, sizeof(int) * (size_t)m.E, cudaMemcpyHostToDevice, c->copy));
    CK(mark(8, c->copy));
    CK(cudaEventRecord(c->copy_join, c->copy));
  } else {
    CK(mark(7, c->stream));
    CK(mark(8, c->stream));
    CK(cudaMemsetAsync(c->flags.p, 0, sizeof(int) * (size_t)m.E, c->stream));
  }
  size_t nw = ((size_t)m.E + 31) / 32;
  ENSURE(c->bits, sizeof(uint32_t) * 2 * nw);
  uint32_t* sb = P<uint32_t>(c->bits);
  // FP32: the size field is final after the vertex average, so its FP64
  // conversion and download run on the copy stream beside the measure and
  // the guard
  const bool early_size = size_out && c->precision == SPRG_FP32;
  if (early_size) ENSURE(c->size, sizeof(double) * (size_t)m.V);
  if (c->e2e_prec != c->precision || c->e2e_ratio != adapt_ratio || c->e2e_stream != c->stream ||
      c->e2e_early != early_size) {
    drop_e2e_graph(c);
    c->e2e_prec = c->precision;
    c->e2e_ratio = adapt_ratio;
    c->e2e_stream = c->stream;
    c->e2e_early = early_size;
  }
  c->size_hook = early_size;
  rc = e2e_pass(c, adapt_ratio, sb, sb + nw);
  c->size_hook = false;
  if (rc) return rc;
  CK(mark(2, c->stream));
  if (early_size) {
    CK(cudaStreamWaitEvent(c->copy, c->size_ready, 0));
    CK(mark(9, c->copy));
    fast_size_to_f64(m.V, P<float2>(c->sz2), P<double>(c->size), c->copy);
    c->launches += 1;
    CK(cudaMemcpyAsync(size_out, c->size.p, sizeof(double) * (size_t)m.V, cudaMemcpyDeviceToHost, c->copy));
    CK(mark(10, c->copy));
    CK(cudaEventRecord(c->size_join, c->copy));
    c->size_valid = true;
  }
  if (flags) CK(cudaStreamWaitEvent(c->stream, c->copy_join, 0));
  CK(mark(3, c->stream));
  PB("apply_marks");
  CK(cudaMemsetAsync(c->mcount.p, 0, 2 * sizeof(unsigned long long), c->stream));
  // FP32 on one mesh: a rounding-dominated pass leaves the flags unchanged,
  // and runs again in FP64 below
  const int* skip = c->precision == SPRG_FP32 && !c->batch_n ? P<int>(c->fcnt) + 5 : nullptr;
  launch_apply_marks(m.E, sb, sb + nw, P<int>(c->flags), P<unsigned long long>(c->mcount), P<DevStatus>(c->status), skip,
                     c->stream);
  PE();
  c->launches += 1;
  if ((rc = check_launch(c, "apply marks"))) return rc;
  CK(mark(4, c->stream));
  if (flags) {
    PB("download_flags");
    CK(cudaMemcpyAsync(flags, c->flags.p, sizeof(int) * (size_t)m.E, cudaMemcpyDeviceToHost, c->stream));
    PE();
  }
  CK(mark(5, c->stream));
  if (!early_size) {
    CK(mark(9, c->stream));
    if (c->precision == SPRG_FP32) {
      ENSURE(c->size, sizeof(double) * (size_t)m.V);
      fast_size_to_f64(m.V, P<float2>(c->sz2), P<double>(c->size), c->stream);
      c->launches += 1;
      c->size_valid = true;
    } else if (c->precision == SPRG_LEARNED) {
      ENSURE(c->size, sizeof(double) * (size_t)m.V);
      learned_size_to_f64(m.V, P<float>(c->sizel), P<double>(c->size), c->stream);
      c->launches += 1;
      c->size_valid = true;
    }
    if (size_out)
      CK(cudaMemcpyAsync(size_out, c->size.p, sizeof(double) * (size_t)m.V, cudaMemcpyDeviceToHost, c->stream));
    CK(mark(10, c->stream));
  } else {
    CK(cudaStreamWaitEvent(c->stream, c->size_join, 0));
  }
  PB("readback");
  CK(cudaMemcpyAsync(c->stage->counts, c->mcount.p, sizeof c->stage->counts, cudaMemcpyDeviceToHost, c->stream));
  if ((rc = enqueue_info(c))) return rc;
  PE();
  CK(mark(6, c->stream));
  const auto t_enq = std::chrono::steady_clock::now();
  if ((rc = sync_and_status(c))) return rc;
  if (c->e2e_timing) {
    const auto t_end = std::chrono::steady_clock::now();
    for (int k = 0; k < kE2EStages; ++k) {
      float ms = 0.f;
      CK(cudaEventElapsedTime(&ms, c->e2e_ev[kE2EStagePairs[k][0]], c->e2e_ev[kE2EStagePairs[k][1]]));
      c->e2e_sum[k] += ms;
    }
    c->e2e_host[0] += std::chrono::duration<double, std::milli>(t_enq - t_call).count();
    c->e2e_host[1] += std::chrono::duration<double, std::milli>(t_end - t_enq).count();
    c->e2e_host[2] += std::chrono::duration<double, std::milli>(t_end - t_call).count();
    c->e2e_n += 1;
  }
  if (n_split) *n_split = (long)c->stage->counts[0];
  if (n_collapse) *n_collapse = (long)c->stage->counts[1];
  rc = info_from_stage(c, info);
  if (rc || c->precision != SPRG_FP32 || c->batch_n || c->last_info.n_rounding_dominated == 0) return rc;
  // Rounding-dominated pass: the reference's size factor, and with it its
  // sizes, follow its own FP64 rounding, which the FP32 arithmetic (and its
  // error bounds) does not model.  The flags came back unchanged; the FP64
  // pass (the reference's operation order) decides them.
  const int64_t nr = c->last_info.n_rounding_dominated;
  c->precision = SPRG_FP64;
  rc = sprg_estimate_and_mark(c, u, adapt_ratio, size_out, flags, n_split, n_collapse, info);
  c->precision = SPRG_FP32;
  c->last_info.n_rounding_dominated = nr;
  if (info) info->n_rounding_dominated = nr;
  return rc;
}

int sprg_debug_read(sprg_ctx* c, const char* name, void* host, size_t bytes) {
  if (!c || !name || !host) return SPRG_EINVAL;
  int rc = set_device(c);
  if (rc) return rc;
  struct { const char* n; DevBuf* b; } table[] = {
      {"ip", &c->ip},       {"rec", &c->rec},     {"err", &c->err},       {"esize", &c->esize},
      {"size", &c->size},   {"L", &c->L},         {"vrec", &c->vrec},     {"rec32", &c->rec32},
      {"q32", &c->q32},     {"sz2", &c->sz2},     {"tetd", &c->tetd},     {"out3", &c->out3},
      {"fcnt", &c->fcnt},   {"guard", &c->guard}, {"xitems", &c->xitems}, {"xcount", &c->xcount}, {"agcount", &c->agcount}, {"sizes3", &c->sizes3}, {"frames9", &c->frames9}, {"twcount", &c->twcount}, {"met32", &c->met32}, {"rec9", &c->rec9},
      {"wts", &c->wts},     {"geo", &c->geo},     {"elen", &c->elen},     {"rec16", &c->rec16},
      {"sizel", &c->sizel}, {"ql", &c->ql},       {"vr16", &c->vr16},     {"fbitems", &c->fbitems},
      {"fbcount", &c->fbcount}, {"listed", &c->listed}, {"bverts", &c->bverts}, {"pcls", &c->pcls}};
  for (auto& e : table) {
    if (strcmp(e.n, name) != 0) continue;
    if (!e.b->p) return fail(c, SPRG_ESTATE, std::string("buffer not allocated: ") + name);
    if (bytes > e.b->bytes) bytes = e.b->bytes;
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaMemcpy(host, e.b->p, bytes, cudaMemcpyDeviceToHost));
    return SPRG_OK;
  }
  return fail(c, SPRG_EINVAL, std::string("unknown buffer: ") + name);
}

int sprg_profile_enable(sprg_ctx* c, int on) {
  if (!c) return SPRG_EINVAL;
  int rc = set_device(c);
  if (rc) return rc;
  if (on && c->ev_pool.empty()) {
    c->ev_pool.resize(8192);
    for (auto& e : c->ev_pool) CK(cudaEventCreate(&e));
  }
  c->prof = on != 0;
  return SPRG_OK;
}

int sprg_profile_flush(sprg_ctx* c) {
  if (!c) return SPRG_EINVAL;
  int rc = set_device(c);
  if (rc) return rc;
  CK(cudaStreamSynchronize(c->stream));
  for (auto& p : c->pending) {
    float ms = 0;
    if (p.second + 1 < c->ev_pool.size() &&
        cudaEventElapsedTime(&ms, c->ev_pool[p.second], c->ev_pool[p.second + 1]) == cudaSuccess) {
      auto& a = c->prof_acc[p.first];
      a.first += 1;
      a.second += ms;
    }
  }
  c->pending.clear();
  c->ev_used = 0;
  return SPRG_OK;
}

const char* sprg_profile_report(sprg_ctx* c, int reset) {
  if (!c) return "{}";
  sprg_profile_flush(c);
  std::string j = "{";
  bool first = true;
  for (auto& kv : c->prof_acc) {
    char buf[160];
    snprintf(buf, sizeof buf, "%s\"%s\": [%lld, %.6f]", first ? "" : ", ", kv.first.c_str(),
             (long long)kv.second.first, kv.second.second);
    j += buf;
    first = false;
  }
  j += "}";
  c->prof_json = j;
  if (reset) c->prof_acc.clear();
  return c->prof_json.c_str();
}

int sprg_e2e_timing(sprg_ctx* c, int on) {
  if (!c) return SPRG_EINVAL;
  c->e2e_timing = on != 0;
  for (double& x : c->e2e_sum) x = 0;
  for (double& x : c->e2e_host) x = 0;
  c->e2e_n = 0;
  return SPRG_OK;
}

const char* sprg_e2e_timing_report(sprg_ctx* c) {
  if (!c) return "{}";
  const double n = c->e2e_n > 0 ? c->e2e_n : 1;
  std::string j = "{\"calls\": " + std::to_string(c->e2e_n);
  char buf[128];
  for (int k = 0; k < kE2EStages; ++k) {
    snprintf(buf, sizeof buf, ", \"%s_ms\": %.6f", kE2EStageNames[k], c->e2e_sum[k] / n);
    j += buf;
  }
  snprintf(buf, sizeof buf, ", \"host_enqueue_ms\": %.6f, \"host_wait_ms\": %.6f, \"call_ms\": %.6f}",
           c->e2e_host[0] / n, c->e2e_host[1] / n, c->e2e_host[2] / n);
  j += buf;
  c->e2e_json = j;
  return c->e2e_json.c_str();
}

int sprg_apply_marks(int64_t n_edges, const uint32_t* split_bits, const uint32_t* collapse_bits, int32_t* flags,
                     long* n_split, long* n_collapse) {
  if (n_edges < 0 || !flags) return SPRG_EINVAL;
  const int SPLIT_PASS[3] = {SPRG_SPLIT, SPRG_NEED_NOT_SPLIT, SPRG_DONT_SPLIT | SPRG_NEED_NOT_SPLIT};
  const int COLL_PASS[3] = {SPRG_COLLAPSE, SPRG_NEED_NOT_COLLAPSE, SPRG_DONT_COLLAPSE | SPRG_NEED_NOT_COLLAPSE};
  // the true flag must be clear on every edge before either pass (ma/maAdapt.cc:304)
  for (int64_t e = 0; e < n_edges; ++e) {
    if (collapse_bits && (flags[e] & COLL_PASS[0])) return SPRG_EFLAGS;
    if (split_bits && (flags[e] & SPLIT_PASS[0])) return SPRG_EFLAGS;
  }
  long counts[2] = {0, 0};
  const uint32_t* bits[2] = {collapse_bits, split_bits};
  const int* pass[2] = {COLL_PASS, SPLIT_PASS};
  for (int k = 0; k < 2; ++k) {
    if (!bits[k]) continue;
    for (int64_t e = 0; e < n_edges; ++e) {
      int f = flags[e];
      if (pass[k][2] & f) continue;
      if ((bits[k][e >> 5] >> (e & 31)) & 1u) { f |= pass[k][0]; ++counts[k]; }
      else f |= pass[k][1];
      flags[e] = f;
    }
  }
  if (n_collapse) *n_collapse = counts[0];
  if (n_split) *n_split = counts[1];
  return SPRG_OK;
}

int sprg_set_mlp_params(sprg_ctx* c, const float* params, int n_params) {
  if (!c || !params || n_params != kMlpParams) return SPRG_EINVAL;
  int rc = set_device(c);
  if (rc) return rc;
  ENSURE(c->mlp_tmp, sizeof(float) * kMlpParams);
  ENSURE(c->mlp_packed, kMlpPackedBytes);
  CK(cudaMemcpyAsync(c->mlp_tmp.p, params, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice, c->stream));
  learned_pack(P<float>(c->mlp_tmp), c->mlp_packed.p, c->stream);
  CK(cudaStreamSynchronize(c->stream));
  if ((rc = check_launch(c, "pack network parameters"))) return rc;
  c->have_mlp = true;
  drop_e2e_graph(c);
  return SPRG_OK;
}

int sprg_test_hooks(sprg_ctx* c, int wait_polls, int alloc_fail_after) {
  if (!c || wait_polls < 0 || alloc_fail_after < -1) return SPRG_EINVAL;
  c->stall_polls = wait_polls;
  c->alloc_fail_in = alloc_fail_after;
  drop_e2e_graph(c);
  return SPRG_OK;
}

int sprg_set_learned_options(sprg_ctx* c, int use_mlp, double z_max) {
  if (!c || !(z_max > 0)) return SPRG_EINVAL;
  c->use_mlp = use_mlp ? 1 : 0;
  c->z_max = (float)z_max;
  drop_e2e_graph(c);
  return SPRG_OK;
}

int sprg_learned_features(sprg_ctx* c, const double* d_u, uint16_t* d_x, float* d_aux) {
  if (!c || !d_u || !d_x || !d_aux) return SPRG_EINVAL;
  if (c->m.dim != 3) return fail(c, SPRG_EINVAL, "the learned form covers tet meshes");
  int rc = set_device(c);
  if (rc) return rc;
  DevMesh& m = c->m;
  ENSURE(c->fitems, sizeof(int) * (size_t)m.V);
  ENSURE(c->fcnt, 8 * sizeof(int));
  ENSURE(c->vr16, 16 * (size_t)m.V);
  if ((rc = learned_scratch(c))) return rc;
  ExpandList xl{P<int>(c->fitems), P<int>(c->fcnt) + 3, m.V};
  if ((rc = fast_setup(c, xl))) return rc;
  if (!c->vv_ready) {
    ENSURE(c->vvoff, sizeof(int) * ((size_t)m.V + 1));
    ENSURE(c->vv, sizeof(int) * 2 * (size_t)m.E);
    ENSURE(c->tmp, sizeof(int) * (size_t)m.V);
    ENSURE(c->mlp_err, sizeof(int));
    ENSURE(c->vtile, ((size_t)m.V + 127) / 128);
    learned_build_v2v(m, P<int>(c->vvoff), P<int>(c->vv), P<int>(c->tmp), P<unsigned char>(c->vtile),
                      P<int>(c->fcnt) + 6, c->stream);
    CK(cudaMemcpyAsync(&c->max_degree, P<int>(c->fcnt) + 6, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaMemsetAsync(c->mlp_err.p, 0, sizeof(int), c->stream));
    c->vv_ready = true;
  }
  LearnMesh lm{P<int>(c->vvoff), P<int>(c->vv), P<unsigned char>(c->listed), P<unsigned char>(c->vtile)};
  learned_records(c, d_u);
  learned_features(m, lm, P<float4>(c->vr16), P<float>(c->lsc), d_x, d_aux, c->stream);
  CK(cudaStreamSynchronize(c->stream));
  return check_launch(c, "learned features");
}

size_t sprg_mlp_scratch_bytes(int n) { return n > 0 ? mlp_scratch_bytes(n) : 0; }

int sprg_mlp_forward(const float* d_params, const uint16_t* d_x, int n, float* d_out, void* d_scratch, void* stream) {
  if (!d_params || !d_x || !d_out || n <= 0 || !d_scratch) return SPRG_EINVAL;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  mlp_run(0, d_params, d_x, nullptr, n, d_out, nullptr, nullptr, d_scratch, s);
  return cudaGetLastError() == cudaSuccess ? SPRG_OK : SPRG_ECUDA;
}

int sprg_mlp_grad(const float* d_params, const uint16_t* d_x, const float* d_y, int n, float* d_grad, float* d_loss,
                  void* d_scratch, void* stream) {
  if (!d_params || !d_x || !d_y || !d_grad || n <= 0 || !d_scratch) return SPRG_EINVAL;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  mlp_run(1, d_params, d_x, d_y, n, nullptr, d_grad, d_loss, d_scratch, s);
  return cudaGetLastError() == cudaSuccess ? SPRG_OK : SPRG_ECUDA;
}

int sprg_mlp_adam(float* d_params, float* d_m1, float* d_m2, const float* d_grad, float lr, float beta1, float beta2,
                  float eps, int step, void* stream) {
  if (!d_params || !d_m1 || !d_m2 || !d_grad || step < 1) return SPRG_EINVAL;
  mlp_adam(d_params, d_m1, d_m2, d_grad, lr, beta1, beta2, eps, step, static_cast<cudaStream_t>(stream));
  return cudaGetLastError() == cudaSuccess ? SPRG_OK : SPRG_ECUDA;
}

int sprg_hessian_metric(sprg_ctx* c, const double* hessian, double eps, double h_min, double h_max,
                        double* sizes_out, double* frames_out) {
  if (!c || !hessian || !sizes_out || !frames_out) return SPRG_EINVAL;
  if (!(eps > 0) || !(h_min > 0) || !(h_max >= h_min)) return fail(c, SPRG_EINVAL, "need eps > 0, 0 < h_min <= h_max");
  int rc = set_device(c);
  if (rc) return rc;
  c->launches = 0;
  DevMesh& m = c->m;
  ENSURE(c->hess, sizeof(double) * 9 * (size_t)m.V);
  ENSURE(c->sizes3, sizeof(double) * 3 * (size_t)m.V);
  ENSURE(c->frames9, sizeof(double) * 9 * (size_t)m.V);
  CK(cudaMemcpyAsync(c->hess.p, hessian, sizeof(double) * 9 * (size_t)m.V, cudaMemcpyHostToDevice, c->stream));
  launch_hessian_metric(m, P<double>(c->hess), eps, h_min, h_max, P<double>(c->sizes3), P<double>(c->frames9),
                        c->stream);
  c->launches += 1;
  if ((rc = check_launch(c, "hessian metric"))) return rc;
  CK(cudaMemcpyAsync(sizes_out, c->sizes3.p, sizeof(double) * 3 * (size_t)m.V, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaMemcpyAsync(frames_out, c->frames9.p, sizeof(double) * 9 * (size_t)m.V, cudaMemcpyDeviceToHost, c->stream));
  return sync_and_status(c);
}

// The mixed-precision pass's nodal Hessian on triangles: per mesh, the
// patch weights and the recovery-of-gradient operator K (FP64); per pass
// rec1 = K u and H = K rec1, the listed patches (growth or more than the
// weights' patch size) by the FP64 slab fits with in-place gradients.
static int hessian_operator_2d(sprg_ctx* c) {
  DevMesh& m = c->m;
  int rc;
  const int ks = tri_operator_slots();
  // the list buffers exist before any kernel or list view refers to them
  ENSURE(c->twitems, sizeof(int) * (size_t)(m.V > 0 ? m.V : 1));
  ENSURE(c->twcount, sizeof(int));
  const ExpandList lst{P<int>(c->twitems), P<int>(c->twcount), m.V};
  if (!c->tw_ready) {
    ENSURE(c->tw, sizeof(double) * (size_t)m.T * m.nn);
    ENSURE(c->twlisted, (size_t)(m.V > 0 ? m.V : 1));
    ENSURE(c->kidx, sizeof(int) * (size_t)m.V * ks);
    c->op_kc = c->planar ? 2 : 3;
    ENSURE(c->kval, sizeof(double) * c->op_kc * (size_t)m.V * ks);
    ENSURE(c->klen, sizeof(int) * (size_t)(m.V > 0 ? m.V : 1));
    CK(cudaMemsetAsync(c->twcount.p, 0, sizeof(int), c->stream));
    PB("tri_weights_f64");
    launch_tri_weights(m, P<double>(c->tw), P<unsigned char>(c->twlisted), lst, c->stream);
    PE();
    PB("tri_operator_f64");
    launch_tri_operator(m, c->op_kc, P<double>(c->tw), P<unsigned char>(c->twlisted), lst, P<int>(c->kidx),
                        P<double>(c->kval), P<int>(c->klen), c->stream);
    PE();
    c->launches += 2;
    if ((rc = check_launch(c, "triangle operator"))) return rc;
    c->tw_ready = true;
  }
  ENSURE(c->rec, sizeof(double) * 3 * (size_t)m.V);
  ENSURE(c->rec9, sizeof(double) * 9 * (size_t)m.V);
  ENSURE(c->slab, sizeof(double) * (size_t)expand_grid() * expand_max_elems() * (4 + 9 + 1));
  PB("recover_grad_op_f64");
  launch_apply_operator(m.V, 1, c->op_kc, P<unsigned char>(c->twlisted), P<int>(c->kidx), P<double>(c->kval),
                        P<int>(c->klen), P<double>(c->f), P<double>(c->rec), c->stream);
  PE();
  c->launches += 1;
  if ((rc = listed_fits(c, c->cache2d, nullptr, P<double>(c->f), 3, P<double>(c->rec), lst))) return rc;
  PB("recover_grad_op_f64");
  launch_apply_operator(m.V, 3, c->op_kc, P<unsigned char>(c->twlisted), P<int>(c->kidx), P<double>(c->kval),
                        P<int>(c->klen), P<double>(c->rec), P<double>(c->rec9), c->stream);
  PE();
  c->launches += 1;
  return listed_fits(c, c->cache2d, nullptr, P<double>(c->rec), 9, P<double>(c->rec9), lst);
}

// the mixed-precision anisotropic pass (SPRG_FP32): FP64 nodal Hessian
// (on triangles through the per-mesh operator) and metric; FP32 edge measure
// with the FP64 guard band; FP32 qualities
static int aniso_pass_mixed(sprg_ctx* c, double eps, double h_min, double h_max, uint32_t* d_split_bits,
                            uint32_t* d_collapse_bits, double* d_quality) {
  DevMesh& m = c->m;
  int rc;
  const double* H;
  if (m.dim == 2) {
    if ((rc = hessian_operator_2d(c))) return rc;
    H = P<double>(c->rec9);
  } else {  // tets: the FP64 gradients and recoveries
    if ((rc = step_grad(c, 1)) || (rc = step_recover(c))) return rc;
    CK(cudaMemcpyAsync(c->f.p, c->rec.p, sizeof(double) * 3 * (size_t)m.V, cudaMemcpyDeviceToDevice, c->stream));
    if ((rc = step_grad(c, 3)) || (rc = step_recover(c))) return rc;
    H = P<double>(c->rec);
  }
  ENSURE(c->met32, sizeof(float) * 12 * (size_t)(m.V > 0 ? m.V : 1));
  ENSURE(c->qrec32, (size_t)quality_rec_bytes() * (size_t)(m.V > 0 ? m.V : 1));
  if (!c->crec_ready) {  // the coordinate records of the edge and element Jacobians (per mesh)
    ENSURE(c->crec, 32 * (size_t)(m.V > 0 ? m.V : 1));
    fast_prep_coords(m, c->frame, P<float4>(c->crec), c->stream);
    c->launches += 1;
    c->crec_ready = true;
  }
  ENSURE(c->agitems, sizeof(int) * (size_t)(m.E > 0 ? m.E : 1));
  ENSURE(c->agcount, sizeof(int));
  CK(cudaMemsetAsync(c->agcount.p, 0, sizeof(int), c->stream));
  // triangles: the FP32 records straight from the Hessian, and the FP64
  // metric rebuilt only where the guard and the quality's tie-breaks need
  // it; tets: the FP64 metric, then its FP32 records
  const double* sizes64 = nullptr;
  const double* frames64 = nullptr;
  if (m.dim == 2) {
    PB("metric_f32");
    launch_metric_mixed2d(m.V, H, eps, h_min, h_max, P<float>(c->met32), c->qrec32.p, c->stream);
    PE();
  } else {
    PB("hessian_metric");
    launch_hessian_metric(m, H, eps, h_min, h_max, P<double>(c->sizes3), P<double>(c->frames9), c->stream);
    PE();
    PB("metric_f32");
    launch_metric_f32(m.V, m.dim, P<double>(c->sizes3), P<double>(c->frames9), P<float>(c->met32), c->qrec32.p,
                      c->stream);
    PE();
    sizes64 = P<double>(c->sizes3);
    frames64 = P<double>(c->frames9);
  }
  PB("measure_aniso_f32");
  launch_measure_aniso_f32(m, P<float>(c->met32), P<float4>(c->crec), c->frame[3], d_split_bits, d_collapse_bits,
                           P<int>(c->agitems), P<int>(c->agcount), m.E, c->stream);
  PE();
  PB("guard_measure_f64");
  launch_measure_guard_f64(m, sizes64, frames64, H, eps, h_min, h_max, P<int>(c->agitems), P<int>(c->agcount), m.E,
                           d_split_bits, d_collapse_bits, c->stream);
  PE();
  c->launches += 4;
  if (d_quality) {
    PB("quality_f32");
    ENSURE(c->cj64, sizeof(double) * (size_t)(m.V > 0 ? m.V : 1));
    ENSURE(c->qties, sizeof(int) * ((size_t)m.T + 1));
    launch_quality_aniso_f32(m, c->qrec32.p, P<float4>(c->crec), c->frame[3], sizes64, frames64, H, eps, h_min,
                             h_max, P<double>(c->cj64), P<int>(c->qties) + 1, P<int>(c->qties), d_quality, c->stream);
    PE();
    c->launches += 2;
  }
  c->L_valid = false;  // no FP64 length array in this form
  c->size_valid = false;
  return check_launch(c, "mixed aniso pass");
}

int sprg_aniso_estimate_and_mark_resident(sprg_ctx* c, const double* d_u, double eps, double h_min, double h_max,
                                          uint32_t* d_split_bits, uint32_t* d_collapse_bits, double* d_quality) {
  if (!c || !d_u || !d_split_bits || !d_collapse_bits) return SPRG_EINVAL;
  if (!(eps > 0) || !(h_min > 0) || !(h_max >= h_min)) return fail(c, SPRG_EINVAL, "need eps > 0, 0 < h_min <= h_max");
  int rc = set_device(c);
  if (rc) return rc;
  c->launches = 0;
  DevMesh& m = c->m;
  ENSURE(c->f, sizeof(double) * 3 * (size_t)m.V);
  ENSURE(c->sizes3, sizeof(double) * 3 * (size_t)m.V);
  ENSURE(c->frames9, sizeof(double) * 9 * (size_t)m.V);
  ENSURE(c->L, sizeof(double) * (size_t)m.E);
  if ((rc = reset_status(c))) return rc;
  CK(cudaMemcpyAsync(c->f.p, d_u, sizeof(double) * (size_t)m.V, cudaMemcpyDeviceToDevice, c->stream));
  if (c->precision == SPRG_FP32) return aniso_pass_mixed(c, eps, h_min, h_max, d_split_bits, d_collapse_bits, d_quality);
  // recovered gradient, then the recovered gradient of it (nodal Hessian)
  if ((rc = step_grad(c, 1)) || (rc = step_recover(c))) return rc;
  CK(cudaMemcpyAsync(c->f.p, c->rec.p, sizeof(double) * 3 * (size_t)m.V, cudaMemcpyDeviceToDevice, c->stream));
  if ((rc = step_grad(c, 3)) || (rc = step_recover(c))) return rc;
  PB("hessian_metric");
  launch_hessian_metric(m, P<double>(c->rec), eps, h_min, h_max, P<double>(c->sizes3), P<double>(c->frames9),
                        c->stream);
  PE();
  PB("measure_aniso_f64");
  launch_measure_aniso_f64(m, P<double>(c->sizes3), P<double>(c->frames9), P<double>(c->L), c->stream);
  PE();
  PB("mark_bits");
  launch_mark_bits(m.E, P<double>(c->L), d_split_bits, d_collapse_bits, c->stream);
  PE();
  c->launches += 3;
  if (d_quality) {
    PB("quality_f64");
    launch_quality_f64(m, nullptr, P<double>(c->sizes3), P<double>(c->frames9), d_quality, c->stream);
    PE();
    c->launches += 1;
  }
  c->L_valid = true;
  c->size_valid = false;
  return check_launch(c, "aniso pass");
}

int sprg_set_batch(sprg_ctx* c, int n_meshes, const int64_t* vert_offsets, const int64_t* elem_offsets,
                   const double* adapt_ratios) {
  if (!c) return SPRG_EINVAL;
  int rc = set_device(c);
  if (rc) return rc;
  drop_e2e_graph(c);
  if (n_meshes == 0) {
    c->batch_n = 0;
    return SPRG_OK;
  }
  if (n_meshes < 0 || !vert_offsets || !elem_offsets || !adapt_ratios) return SPRG_EINVAL;
  const DevMesh& m = c->m;
  if (vert_offsets[0] != 0 || elem_offsets[0] != 0 || vert_offsets[n_meshes] != m.V || elem_offsets[n_meshes] != m.T)
    return fail(c, SPRG_EINVAL, "batch offsets must start at 0 and end at the vertex / element counts");
  std::vector<int> voff(n_meshes + 1), segoff(n_meshes + 1);
  std::vector<int2> seg;
  for (int k = 0; k < n_meshes; ++k) {
    if (vert_offsets[k + 1] <= vert_offsets[k] || elem_offsets[k + 1] <= elem_offsets[k])
      return fail(c, SPRG_EINVAL, "batch offsets must increase");
    if (!(adapt_ratios[k] > 0)) return fail(c, SPRG_EINVAL, "adapt ratios must be positive");
    voff[k] = (int)vert_offsets[k];
    segoff[k] = (int)seg.size();
    for (int64_t t = elem_offsets[k]; t < elem_offsets[k + 1]; t += sprg_ctx::kSegTets) {
      int64_t e = t + sprg_ctx::kSegTets;
      if (e > elem_offsets[k + 1]) e = elem_offsets[k + 1];
      seg.push_back(make_int2((int)t, (int)e));
    }
  }
  voff[n_meshes] = m.V;
  segoff[n_meshes] = (int)seg.size();
  ENSURE(c->bvoff, sizeof(int) * voff.size());
  ENSURE(c->bsegoff, sizeof(int) * segoff.size());
  ENSURE(c->bseg, sizeof(int2) * seg.size());
  ENSURE(c->bratios, sizeof(double) * n_meshes);
  CK(cudaMemcpy(c->bvoff.p, voff.data(), sizeof(int) * voff.size(), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(c->bsegoff.p, segoff.data(), sizeof(int) * segoff.size(), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(c->bseg.p, seg.data(), sizeof(int2) * seg.size(), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(c->bratios.p, adapt_ratios, sizeof(double) * n_meshes, cudaMemcpyHostToDevice));
  c->batch_n = n_meshes;
  c->batch_nseg = (int)seg.size();
  return SPRG_OK;
}

int sprg_batch_info(sprg_ctx* c, double* out) {
  if (!c || !out || !c->batch_n || !c->out3.p) return SPRG_EINVAL;
  int rc = set_device(c);
  if (rc) return rc;
  std::vector<double> o4(4 * (size_t)c->batch_n);
  CK(cudaStreamSynchronize(c->stream));
  CK(cudaMemcpy(o4.data(), c->out3.p, sizeof(double) * o4.size(), cudaMemcpyDeviceToHost));
  for (int k = 0; k < c->batch_n; ++k)
    for (int j = 0; j < 3; ++j) out[3 * (size_t)k + j] = o4[4 * (size_t)k + j];
  return SPRG_OK;
}

int sprg_set_autotune(sprg_ctx* c, int on) {
  if (!c) return SPRG_EINVAL;
  c->autotune = on != 0;
  c->tuned = false;  // on: tune again at the next pass
  drop_e2e_graph(c);
  return SPRG_OK;
}

const char* sprg_tuning_report(sprg_ctx* c) {
  if (!c) return "";
  if (c->tune_json.empty()) {
    c->tune_json = "{\"bins\":[" + std::to_string(c->bin_count[0]) + "," + std::to_string(c->bin_count[1]) + "," +
                   std::to_string(c->bin_count[2]) + "," + std::to_string(c->bin_count[3]) + "],\"lanes\":[" +
                   std::to_string(c->bin_lanes[0]) + "," + std::to_string(c->bin_lanes[1]) + "," +
                   std::to_string(c->bin_lanes[2]) + "," + std::to_string(c->bin_lanes[3]) +
                   "],\"tile_verts\":" + std::to_string(c->tile_verts) +
                   ",\"blocks_per_sm\":" + std::to_string(c->grid_per_sm) + ",\"tuned\":false}";
  }
  return c->tune_json.c_str();
}

int sprg_graph_capture(sprg_ctx* c, const double* d_u, double adapt_ratio, uint32_t* d_split_bits,
                       uint32_t* d_collapse_bits) {
  if (!c || !d_u || !d_split_bits || !d_collapse_bits) return SPRG_EINVAL;
  int rc = set_device(c);
  if (rc) return rc;
  if (c->stream == c->own || c->stream == nullptr)
    return fail(c, SPRG_ESTATE, "graph capture needs a caller stream (sprg_set_stream)");
  // one ordinary pass first: buffers, per-mesh setup, patch cache and tuning
  if ((rc = sprg_estimate_and_mark_resident(c, d_u, adapt_ratio, d_split_bits, d_collapse_bits))) return rc;
  CK(cudaStreamSynchronize(c->stream));
  const bool prof = c->prof;
  c->prof = false;
  if (c->graph_exec) {
    cudaGraphExecDestroy(c->graph_exec);
    c->graph_exec = nullptr;
  }
  CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  rc = sprg_estimate_and_mark_resident(c, d_u, adapt_ratio, d_split_bits, d_collapse_bits);
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamEndCapture(c->stream, &graph);
  c->prof = prof;
  if (rc) {
    if (graph) cudaGraphDestroy(graph);
    return rc;
  }
  if (e != cudaSuccess) return cuda_fail(c, e, "cudaStreamEndCapture");
  e = cudaGraphInstantiate(&c->graph_exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return cuda_fail(c, e, "cudaGraphInstantiate");
  return SPRG_OK;
}

int sprg_graph_replay(sprg_ctx* c) {
  if (!c) return SPRG_EINVAL;
  if (!c->graph_exec) return fail(c, SPRG_ESTATE, "no captured graph (sprg_graph_capture)");
  int rc = set_device(c);
  if (rc) return rc;
  CK(cudaGraphLaunch(c->graph_exec, c->stream));
  return SPRG_OK;
}

int sprg_set_tiling(sprg_ctx* c, const int* lanes, int tile_verts, int blocks_per_sm) {
  if (!c || !lanes || tile_verts <= 0 || blocks_per_sm <= 0) return SPRG_EINVAL;
  for (int b = 0; b < 4; ++b) {
    if (lanes[b] != 0 && lanes[b] != 1 && lanes[b] != 2 && lanes[b] != 4)
      return fail(c, SPRG_EINVAL, "lanes per vertex: 1, 2 or 4, or 0 (sliced)");
    if (lanes[b] == 0 && tile_verts % 32)
      return fail(c, SPRG_EINVAL, "the sliced mode needs tiles of a multiple of 32 vertices");
  }
  int rc = set_device(c);
  if (rc) return rc;
  for (int b = 0; b < 4; ++b) c->bin_lanes[b] = lanes[b];
  c->tile_verts = tile_verts;
  c->grid_per_sm = blocks_per_sm;
  c->autotune = false;
  c->tuned = true;
  c->tune_json.clear();
  drop_e2e_graph(c);
  return c->bins_ready ? build_tiles(c) : SPRG_OK;
}

}  // extern "C"
