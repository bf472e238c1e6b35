// C ABI of the batched rigid-body step (declared in include/cubez_gpu.h).
//
// A batch owns every device buffer it uses (allocated once in
// cz_batch_create), one non-blocking CUDA stream, and a cache of captured
// CUDA graphs for multi-step rollouts.  Calls on one batch are serialised by
// the caller (the reference is single-threaded, contact.go has no locking).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <numeric>
#include <string>
#include <utility>
#include <vector>

#include "../../include/cubez_gpu.h"
#include "cz_forms.h"
#include "cz_layout.cuh"

// Worlds of more bodies than this are resolved by k_resolve_big (bodies and
// contacts in global memory, 32 or 16 lanes per world).
constexpr int kBigWorld = 64;

namespace {

thread_local std::string g_last_error;
std::atomic<long long> g_launches{0};

int fail(int status, const std::string& msg) {
  g_last_error = msg;
  return status;
}

#define CZ_CUDA(call)                                                                                   \
  do {                                                                                                  \
    cudaError_t e_ = (call);                                                                            \
    if (e_ != cudaSuccess)                                                                              \
      return fail(CZ_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));                    \
  } while (0)

long long round_up(long long x, long long m) { return (x + m - 1) / m * m; }

}  // namespace

int cz::set_error(int status, const char* what, cudaError_t e) {
  g_last_error = std::string(what) + (e != cudaSuccess ? std::string(": ") + cudaGetErrorString(e) : "");
  return status;
}

struct cz_batch {
  const cz::FormOps* ops = nullptr;
  int form = 0;
  int device = 0;
  int sm_count = 0;
  size_t smem_optin = 0;
  cudaStream_t stream = nullptr;

  int num_worlds = 0;
  long long nb = 0, nb_pad = 0, nc_total = 0;
  std::vector<int> counts, bstart, ccap, h2p;
  std::vector<long long> cstart;
  int max_n = 0, nbs = 4, max_cap = 1;
  // worlds of more than kBigWorld bodies are resolved by k_resolve_big; the
  // others by k_resolve with a shared-memory slot of rs_nbs bodies
  int rs_nbs = 4, nsmall = 0;
  std::vector<int> big_ids;
  int* d_big = nullptr;
  int* d_units = nullptr;  // cz_collide's unit list
  long long units_cap = 0;
  void* big_bw = nullptr;
  void* big_br = nullptr;
  uint8_t* big_aw = nullptr;
  int *big_off = nullptr, *big_cnt = nullptr, *big_adj = nullptr;

  // device buffers
  void* body = nullptr;
  uint8_t* awake = nullptr;
  uint8_t* can_sleep = nullptr;
  int* shape = nullptr;
  int *d_bstart = nullptr, *d_bcount = nullptr, *d_ccap = nullptr, *d_ccount = nullptr;
  long long* d_cstart = nullptr;
  uint32_t* d_wstatus = nullptr;
  int *d_piters = nullptr, *d_viters = nullptr;
  void* contact = nullptr;
  int* cbodies = nullptr;
  void* work = nullptr;
  int* wbodies = nullptr;
  void* kmat = nullptr;  // per contact: friction K and response row, 16 reals
  int* d_order = nullptr;
  int* d_order_rs = nullptr;
  unsigned* d_queue = nullptr;
  uint32_t* d_status = nullptr;
  unsigned long long* d_counters = nullptr;
  int* d_h2p = nullptr;
  double* d_stage = nullptr;
  uint8_t* d_stage_u8 = nullptr;
  int* d_stage_i32 = nullptr;
  double* d_cstage = nullptr;
  int* d_cstage_b = nullptr;
  double* d_pow = nullptr;
  // collider Offsets (allocated by the first upload that carries them)
  void* d_offset = nullptr;       // [12][nb_pad] rows in the form's real type
  double* d_off_stage = nullptr;  // [n][12]
  double* h_off_stage = nullptr;  // pinned [n][12]
  bool has_offset = false;        // the last upload carried Offsets
  // pinned host staging
  double* h_stage = nullptr;
  uint8_t* h_stage_u8 = nullptr;
  int* h_stage_i32 = nullptr;
  double* h_cstage = nullptr;
  int* h_cstage_b = nullptr;
  double* h_pow = nullptr;
  uint32_t* h_status = nullptr;

  std::vector<double> lin_damp, ang_damp;
  double pow_dt = std::nan("");
  double plane[4] = {0, 1, 0, 0};
  int iter_mult = 4;
  int max_iterations = -1;

  // tuning
  int np_threads = 128, np_grid = 1, rs_cs = 128, rs_grid = 1, rs_ctas_per_sm = 0, int_threads = 256;
  int rs_lanes = 8;  // lanes per world in the resolver (32 / rs_lanes worlds per warp)
  int big_lanes = 32; // lanes per world in the large-world resolver (16: two worlds per warp)
  int wait_limit = 1 << 22;  // polls of the narrowphase's bounded wait
  int wait_extra_tx = 0;     // test hook: bytes that wait expects beyond its copies
  int grid_min_bodies = 128; // narrowphase grid for worlds of at least this many bodies (0: never)
  int fused = 0;             // one launch per frame (the fused frame) where the batch allows it
  size_t fr_smem = 0;        // the fused frame's shared memory per CTA (0: it does not fit)
  int fr_grid = 1;           // the fused frame's CTAs
  int mode = 0;      // resolver mode: 0 plain, 1 harvest, 2 learned warm start
  cz::MlpDev mlp{};  // device copy of the warm-start network
  void* mlp_mem = nullptr;
  float* hv_features = nullptr;
  float* hv_labels = nullptr;
  unsigned long long* hv_count = nullptr;
  long long hv_cap = 0;
  void* ws_rows = nullptr;  // per-body warm-start / harvest scratch (allocated on first use)
  int* ws_int = nullptr;
  uint8_t* ws_u8 = nullptr;
  uint8_t* ws_world = nullptr;
  float* ws_feat = nullptr;  // harvest features, allocated by the first cz_harvest
  int wf_grid = 1;           // k_warm_features CTAs
  int warm_shift = 2;        // warm-start worlds whose last solve used <= max_it >> warm_shift
  size_t np_smem = 0, rs_smem = 0;

  // graph cache: (nsteps, dt) -> executable graph
  std::map<std::pair<int, double>, cudaGraphExec_t> graphs;
  // rollouts with event-record nodes between the phases (cz_step_timed)
  struct Timed {
    cudaGraphExec_t exec = nullptr;
    std::vector<cudaEvent_t> ev;  // 3 * nsteps + 1
  };
  std::map<std::pair<int, double>, Timed> timed;
  // on-device copy of the body state (cz_snapshot / cz_restore)
  void* snap_body = nullptr;
  uint8_t* snap_u8 = nullptr;  // awake, can_sleep
  double snap_pow_dt = std::nan("");

  cz::HostView view() const {
    cz::HostView v;
    v.body = body;
    v.awake = awake;
    v.can_sleep = can_sleep;
    v.shape = shape;
    v.offset = has_offset ? d_offset : nullptr;
    v.nb_pad = nb_pad;
    v.num_worlds = num_worlds;
    v.max_bodies = max_n;
    v.body_start = d_bstart;
    v.body_count = d_bcount;
    v.contact_start = d_cstart;
    v.contact_cap = d_ccap;
    v.contact_count = d_ccount;
    v.world_status = d_wstatus;
    v.pos_iters = d_piters;
    v.vel_iters = d_viters;
    v.contact = contact;
    v.contact_bodies = cbodies;
    v.work = work;
    v.kmat = kmat;
    v.work_bodies = wbodies;
    v.nc_total = nc_total;
    v.order = d_order;
    v.order_rs = d_order_rs;
    v.queue = d_queue;
    v.status = d_status;
    v.counters = d_counters;
    for (int i = 0; i < 4; ++i) v.plane[i] = plane[i];
    v.iter_mult = iter_mult;
    v.max_iterations = max_iterations;
    v.contact_writeback = 0;
    v.uniform_material = 1;
    v.mode = mode;
    v.mlp = mlp;
    v.hv_features = hv_features;
    v.hv_labels = hv_labels;
    v.hv_count = hv_count;
    v.hv_cap = hv_cap;
    v.ws_rows = ws_rows;
    v.ws_int = ws_int;
    v.ws_u8 = ws_u8;
    v.ws_world = ws_world;
    v.ws_feat = ws_feat;
    v.warm_shift = warm_shift;
    v.big_list = d_big;
    v.big_count = (int)big_ids.size();
    v.big_bw = big_bw;
    v.big_br = big_br;
    v.big_aw = big_aw;
    v.big_off = big_off;
    v.big_cnt = big_cnt;
    v.big_adj = big_adj;
    v.wait_limit = wait_limit;
    v.wait_extra_tx = wait_extra_tx;
    v.grid_min_bodies = grid_min_bodies;
    return v;
  }
};

namespace {

// Resolver queue for the next frame: worlds in decreasing adjustPositions +
// adjustVelocities iterations of this frame (a counting sort in one CTA), so
// that the worlds sharing a warp in lockstep have similar work.  The order of
// independent worlds does not change any result.
constexpr int kReorderBuckets = 2048;
__global__ void __launch_bounds__(1024) k_reorder(const int* __restrict__ pos_it, const int* __restrict__ vel_it,
                                                  int W, int* __restrict__ order,
                                                  const uint8_t* __restrict__ plain_next = nullptr) {
  __shared__ int hist[kReorderBuckets];
  __shared__ int wsum[32];
  const int tid = threadIdx.x;
  for (int i = tid; i < kReorderBuckets; i += blockDim.x) hist[i] = 0;
  __syncthreads();
  // with the warm start on, the worlds it will serve (plain_next[w] == 0)
  // go first: their solve is usually short, but one that falls back solves
  // twice, and late in the queue that would be the frame's tail
  auto key_of_world = [&](int w) {
    if (plain_next && !plain_next[w]) return kReorderBuckets - 1;
    return min(pos_it[w] + vel_it[w], kReorderBuckets - 1);
  };
  for (int w = tid; w < W; w += blockDim.x) atomicAdd(&hist[kReorderBuckets - 1 - key_of_world(w)], 1);
  __syncthreads();
  // exclusive scan of 2048 buckets, two per thread
  const int a = hist[2 * tid], c = hist[2 * tid + 1];
  int x = a + c;
  const int lane = tid & 31, wid = tid >> 5;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, d);
    if (lane >= d) x += y;
  }
  if (lane == 31) wsum[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int t = wsum[lane];
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, t, d);
      if (lane >= d) t += y;
    }
    wsum[lane] = t;
  }
  __syncthreads();
  const int excl = x - (a + c) + (wid > 0 ? wsum[wid - 1] : 0);
  __syncthreads();
  hist[2 * tid] = excl;
  hist[2 * tid + 1] = excl + a;
  __syncthreads();
  for (int w = tid; w < W; w += blockDim.x) order[atomicAdd(&hist[kReorderBuckets - 1 - key_of_world(w)], 1)] = w;
}

void free_batch(cz_batch* b) {
  if (!b) return;
  cudaSetDevice(b->device);
  for (auto& kv : b->graphs) cudaGraphExecDestroy(kv.second);
  for (auto& kv : b->timed) {
    cudaGraphExecDestroy(kv.second.exec);
    for (cudaEvent_t e : kv.second.ev) cudaEventDestroy(e);
  }
  void* dev[] = {
      b->d_offset,  b->d_off_stage, b->ws_feat,   b->d_units,     b->d_big,      b->big_bw,      b->big_br,
      b->big_aw,    b->big_off,     b->big_cnt,   b->big_adj,     b->ws_rows,    b->ws_int,      b->ws_u8,
      b->ws_world,  b->mlp_mem,     b->hv_features, b->hv_labels, b->hv_count,   b->snap_body,   b->snap_u8,
      b->body,      b->awake,       b->can_sleep, b->shape,       b->d_bstart,   b->d_bcount,    b->d_ccap,
      b->d_ccount,  b->d_cstart,    b->d_wstatus, b->d_piters,    b->d_viters,   b->contact,     b->cbodies,
      b->work,      b->wbodies,     b->kmat,      b->d_order,    b->d_order_rs,  b->d_queue,
      b->d_status,  b->d_counters,  b->d_h2p,     b->d_stage,     b->d_stage_u8, b->d_stage_i32, b->d_cstage,
      b->d_cstage_b, b->d_pow};
  for (void* p : dev)
    if (p) cudaFree(p);
  void* host[] = {b->h_off_stage, b->h_stage,    b->h_stage_u8, b->h_stage_i32,
                  b->h_cstage,     b->h_cstage_b, b->h_pow,      b->h_status};
  for (void* p : host)
    if (p) cudaFreeHost(p);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

// Synchronise the batch stream and turn the device status word into a cz_status.
int finish(cz_batch* b) {
  CZ_CUDA(cudaMemcpyAsync(b->h_status, b->d_status, sizeof(uint32_t), cudaMemcpyDeviceToHost, b->stream));
  CZ_CUDA(cudaStreamSynchronize(b->stream));
  const uint32_t bits = *b->h_status;
  const int st = cz::status_from_bits(bits);
  if (st != CZ_OK) {
    char buf[96];
    std::snprintf(buf, sizeof buf, "device status bits 0x%x", bits);
    g_last_error = buf;
  }
  return st;
}

int reset_status(cz_batch* b) {
  CZ_CUDA(cudaMemsetAsync(b->d_status, 0, sizeof(uint32_t), b->stream));
  return CZ_OK;
}

// pow(LinearDamping, dt) and pow(AngularDamping, dt) per body, computed on the
// host (math.Pow in the reference, rigidbody.go:233-234).
int ensure_pows(cz_batch* b, double dt) {
  if (b->pow_dt == dt) return CZ_OK;
  const long long P = b->nb_pad;
  for (long long i = 0; i < 2 * P; ++i) b->h_pow[i] = 1.0;
  for (long long h = 0; h < b->nb; ++h) {
    const long long p = b->h2p[h];
    b->h_pow[p] = std::pow(b->lin_damp[h], dt);
    b->h_pow[P + p] = std::pow(b->ang_damp[h], dt);
  }
  CZ_CUDA(cudaMemcpyAsync(b->d_pow, b->h_pow, sizeof(double) * 2 * P, cudaMemcpyHostToDevice, b->stream));
  CZ_CUDA(b->ops->set_rows(b->view(), cz::B_LINPOW, 2, b->d_pow, b->stream));
  g_launches++;
  CZ_CUDA(cudaStreamSynchronize(b->stream));
  b->pow_dt = dt;
  return CZ_OK;
}

// Whether stepping runs the fused frame: one world per warp, plain resolver,
// every world within the shared-memory slot.
bool uses_frame(const cz_batch* b) {
  return b->fused && b->fr_smem > 0 && b->big_ids.empty() && b->rs_lanes == 32 && b->mode == 0 && b->nsmall > 0;
}

int launches_per_step(const cz_batch* b) {
  if (uses_frame(b)) return 1 + (b->nsmall > 1 ? 1 : 0);
  return 2 + (b->nsmall > 0 ? 1 + (b->nsmall > 32 / b->rs_lanes ? 1 : 0) + (b->mode != 0 ? 1 : 0) : 0) +
         (b->big_ids.empty() ? 0 : 1);
}

int launch_integrate(cz_batch* b, double dt) {
  CZ_CUDA(b->ops->integrate(b->view(), dt, std::pow(0.5, dt), b->int_threads, b->stream));
  g_launches++;
  return CZ_OK;
}
int launch_narrowphase(cz_batch* b) {
  CZ_CUDA(cudaMemsetAsync(b->d_queue, 0, sizeof(unsigned), b->stream));
  CZ_CUDA(b->ops->narrowphase(b->view(), b->nbs, b->np_threads, b->np_grid, b->np_smem, b->stream));
  g_launches++;
  return CZ_OK;
}
// The resolver launches of one frame: k_resolve over the worlds that fit its
// slot (then the re-queue of those worlds by cost), k_resolve_big over the
// others.
int launch_resolve_with(cz_batch* b, double dt, const cz::HostView& v, int cs, size_t smem) {
  if (b->nsmall > 0) {
    if (v.mode != 0) {  // features (and, warm-starting, predictions) ahead of the resolver
      CZ_CUDA(cudaMemsetAsync(b->d_queue + 2, 0, sizeof(unsigned), b->stream));
      CZ_CUDA(b->ops->warm_features(v, b->rs_nbs, b->wf_grid, dt, b->stream));
      g_launches++;
    }
    CZ_CUDA(cudaMemsetAsync(b->d_queue + 1, 0, sizeof(unsigned), b->stream));
    CZ_CUDA(b->ops->resolve(v, b->rs_nbs, cs, b->rs_lanes, b->rs_grid, smem, dt, b->stream));
    g_launches++;
    if (b->nsmall > 32 / b->rs_lanes) {
      k_reorder<<<1, 1024, 0, b->stream>>>(b->d_piters, b->d_viters, b->num_worlds, b->d_order_rs,
                                           v.mode == 2 ? v.ws_world : nullptr);
      CZ_CUDA(cudaGetLastError());
      g_launches++;
    }
  }
  if (!b->big_ids.empty()) {
    CZ_CUDA(b->ops->resolve_big(v, (int)b->big_ids.size(), b->big_lanes, dt, b->stream));
    g_launches++;
  }
  return CZ_OK;
}
int launch_resolve(cz_batch* b, double dt, const cz::HostView* override_view = nullptr) {
  return launch_resolve_with(b, dt, override_view ? *override_view : b->view(), b->rs_cs, b->rs_smem);
}
// The fused frame: integrate, narrowphase and resolve of every world in one
// launch (then the re-queue by cost).
int launch_frame(cz_batch* b, double dt) {
  CZ_CUDA(cudaMemsetAsync(b->d_queue + 1, 0, sizeof(unsigned), b->stream));
  CZ_CUDA(b->ops->frame(b->view(), b->rs_nbs, b->rs_cs, b->fr_grid, b->fr_smem, dt, std::pow(0.5, dt), b->stream));
  g_launches++;
  if (b->nsmall > 1) {
    k_reorder<<<1, 1024, 0, b->stream>>>(b->d_piters, b->d_viters, b->num_worlds, b->d_order_rs);
    CZ_CUDA(cudaGetLastError());
    g_launches++;
  }
  return CZ_OK;
}

// The captured graphs hold the kernels' parameters (the batch view); drop them
// whenever those change.
void drop_graphs(cz_batch* b) {
  for (auto& kv : b->graphs) cudaGraphExecDestroy(kv.second);
  b->graphs.clear();
  for (auto& kv : b->timed) {
    cudaGraphExecDestroy(kv.second.exec);
    for (cudaEvent_t e : kv.second.ev) cudaEventDestroy(e);
  }
  b->timed.clear();
}

int configure(cz_batch* b) {
  // resolver shared-memory tile: shrink the contact capacity until it fits
  int cs = std::min<long long>(b->rs_cs, round_up(b->max_cap, 32));
  cs = std::max(cs, 32);
  while (cs > 32 && b->ops->rs_smem(b->rs_nbs, cs, b->rs_lanes, b->mode) > b->smem_optin) cs -= 32;
  b->rs_cs = cs;
  b->rs_smem = b->ops->rs_smem(b->rs_nbs, cs, b->rs_lanes, b->mode);
  b->np_smem = b->ops->np_smem(b->nbs);
  if (b->np_smem > b->smem_optin || b->rs_smem > b->smem_optin)
    return fail(CZ_ERR_BODY_LIMIT, "world too large for the shared-memory tiles");
  CZ_CUDA(b->ops->prepare(b->np_smem, b->rs_smem, b->rs_lanes));
  int npb = 0, rsb = 0;
  CZ_CUDA(b->ops->occupancy(&npb, b->np_threads, b->np_smem, &rsb, b->rs_smem, b->rs_lanes, b->mode,
                            b->grid_min_bodies > 0 && b->max_n >= b->grid_min_bodies));
  npb = std::max(npb, 1);
  rsb = std::max(rsb, 1);
  if (b->rs_ctas_per_sm > 0) rsb = std::min(rsb, b->rs_ctas_per_sm);
  b->np_grid = (int)std::min<long long>(b->num_worlds, (long long)npb * b->sm_count);
  const long long groups = (std::max(b->nsmall, 1) + 32 / b->rs_lanes - 1) / (32 / b->rs_lanes);
  const int wpc = b->ops->rs_wpc(b->rs_lanes);
  b->rs_grid = (int)std::min<long long>((groups + wpc - 1) / wpc, (long long)rsb * b->sm_count);
  b->np_grid = std::max(b->np_grid, 1);
  b->rs_grid = std::max(b->rs_grid, 1);
  b->wf_grid = (int)std::min<long long>(std::max(b->nsmall, 1),
                                        (long long)b->ops->warm_features_blocks(b->rs_nbs) * b->sm_count);
  // the fused frame's slot holds the resolver's tile and the narrowphase's
  b->fr_smem = b->ops->frame_smem(b->rs_nbs, b->rs_cs);
  if (b->fr_smem > b->smem_optin) {
    b->fr_smem = 0;
  } else {
    int frb = 0;
    CZ_CUDA(b->ops->frame_occupancy(&frb, b->fr_smem));
    frb = std::max(frb, 1);
    if (b->rs_ctas_per_sm > 0) frb = std::min(frb, b->rs_ctas_per_sm);
    b->fr_grid = (int)std::max<long long>(1, std::min<long long>(std::max(b->nsmall, 1), (long long)frb * b->sm_count));
  }
  drop_graphs(b);
  return CZ_OK;
}

}  // namespace

extern "C" {

const char* cz_status_string(int status) {
  switch (status) {
    case CZ_OK: return "ok";
    case CZ_ERR_BAD_ARG: return "bad argument";
    case CZ_ERR_CUDA: return "CUDA error";
    case CZ_ERR_NO_DEVICE: return "no CUDA device";
    case CZ_ERR_NONFINITE: return "non-finite box transform in the box-box test";
    case CZ_ERR_CAPACITY: return "contact capacity exceeded";
    case CZ_ERR_TIMEOUT: return "device wait timed out";
    case CZ_ERR_FRICTIONLESS: return "frictionless impulse on a single-body contact";
    case CZ_ERR_BODY_LIMIT: return "world too large for the kernel tiles";
    default: return "unknown status";
  }
}

const char* cz_last_error(void) { return g_last_error.c_str(); }

int64_t cz_kernel_launches(void) { return g_launches.load(); }

int cz_batch_create(const cz_batch_desc* d, cz_batch** out) {
  if (!d || !out || d->num_worlds <= 0 || !d->body_counts || (d->form != CZ_FORM_FP64 && d->form != CZ_FORM_FP32))
    return fail(CZ_ERR_BAD_ARG, "cz_batch_create: bad descriptor");
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) return fail(CZ_ERR_NO_DEVICE, "no CUDA device");
  if (d->device < 0 || d->device >= ndev) return fail(CZ_ERR_BAD_ARG, "cz_batch_create: bad device ordinal");
  for (int w = 0; w < d->num_worlds; ++w)
    if (d->body_counts[w] < 0 || d->body_counts[w] >= 65535)
      return fail(CZ_ERR_BAD_ARG, "cz_batch_create: body count out of range");
  cz_batch* b = new cz_batch();
  b->form = d->form;
  b->ops = d->form == CZ_FORM_FP64 ? &cz::kFormFP64 : &cz::kFormFP32;
  b->device = d->device;
  int st = CZ_OK;
  auto bail = [&](int s) {
    free_batch(b);
    return s;
  };
  if (cudaSetDevice(b->device) != cudaSuccess) return bail(fail(CZ_ERR_CUDA, "cudaSetDevice failed"));
  cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, b->device);
  int optin = 0;
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, b->device);
  b->smem_optin = (size_t)optin;
  b->num_worlds = d->num_worlds;
  b->counts.assign(d->body_counts, d->body_counts + d->num_worlds);
  for (int i = 0; i < 3; ++i) b->plane[i] = d->plane[i];
  b->plane[3] = d->plane[3];
  if (d->plane[0] == 0 && d->plane[1] == 0 && d->plane[2] == 0) {
    b->plane[0] = 0; b->plane[1] = 1; b->plane[2] = 0;
  }
  b->iter_mult = d->iteration_multiplier > 0 ? d->iteration_multiplier : 4;
  b->max_iterations = d->max_iterations > 0 ? d->max_iterations : -1;
  // layout
  long long nb = 0, np = 0, nc = 0;
  for (int w = 0; w < b->num_worlds; ++w) {
    const int n = b->counts[w];
    b->bstart.push_back((int)np);
    for (int i = 0; i < n; ++i) b->h2p.push_back((int)(np + i));
    np = round_up(np + n, 4);
    nb += n;
    b->max_n = std::max(b->max_n, n);
    const long long worst = 8LL * n + (long long)n * (n - 1);
    long long cap = std::min<long long>(worst, std::max<long long>(64LL * n, 4608));
    if (d->contact_capacity > 0) cap = std::min<long long>(worst, d->contact_capacity);
    cap = std::max<long long>(cap, 1);
    b->ccap.push_back((int)cap);
    b->cstart.push_back(nc);
    nc += round_up(cap, 4);
    b->max_cap = std::max<int>(b->max_cap, (int)cap);
  }
  b->nb = nb;
  b->nb_pad = std::max<long long>(np, 4);
  b->nc_total = std::max<long long>(nc, 4);
  b->nbs = (int)std::max<long long>(round_up(b->max_n, 4), 4);
  int max_small = 0;
  for (int w = 0; w < b->num_worlds; ++w) {
    if (b->counts[w] > kBigWorld)
      b->big_ids.push_back(w);
    else
      max_small = std::max(max_small, b->counts[w]);
  }
  b->nsmall = b->num_worlds - (int)b->big_ids.size();
  b->rs_nbs = (int)std::max<long long>(round_up(max_small, 4), 4);
  b->np_threads = b->max_n >= 256 ? 256 : 128;
  // defaults from the tuned precision workload: a world per warp in float32;
  // two per warp in float64, which shares their float64 chains (the tuner
  // may change both)
  b->rs_cs = 96;
  b->rs_lanes = d->form == CZ_FORM_FP64 ? 16 : 32;
  // world queue: decreasing body count (pair work grows as n^2)
  std::vector<int> order(b->num_worlds);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int c) { return b->counts[a] > b->counts[c]; });

  const size_t R = b->ops->real_size;
  const long long P = b->nb_pad, C = b->nc_total, W = b->num_worlds;
  auto dmalloc = [&](void** p, size_t bytes) -> bool {
    if (cudaMalloc(p, std::max<size_t>(bytes, 16)) != cudaSuccess) return false;
    return true;
  };
  bool ok = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) == cudaSuccess;
  ok = ok && dmalloc(&b->body, R * cz::B_NROWS * P);
  ok = ok && dmalloc((void**)&b->awake, P) && dmalloc((void**)&b->can_sleep, P) &&
       dmalloc((void**)&b->shape, sizeof(int) * P);
  ok = ok && dmalloc((void**)&b->d_bstart, sizeof(int) * W) && dmalloc((void**)&b->d_bcount, sizeof(int) * W) &&
       dmalloc((void**)&b->d_ccap, sizeof(int) * W) && dmalloc((void**)&b->d_ccount, sizeof(int) * W) &&
       dmalloc((void**)&b->d_cstart, sizeof(long long) * W) && dmalloc((void**)&b->d_wstatus, sizeof(uint32_t) * W) &&
       dmalloc((void**)&b->d_piters, sizeof(int) * W) && dmalloc((void**)&b->d_viters, sizeof(int) * W) &&
       dmalloc((void**)&b->d_order, sizeof(int) * W) && dmalloc((void**)&b->d_order_rs, sizeof(int) * W);
  ok = ok && dmalloc(&b->contact, R * cz::C_NROWS * C) && dmalloc((void**)&b->cbodies, sizeof(int) * C);
  ok = ok && dmalloc(&b->work, R * cz::W_NROWS * C) && dmalloc((void**)&b->wbodies, sizeof(int) * C);
  ok = ok && dmalloc(&b->kmat, R * cz::K_ROW * C);
  ok = ok && dmalloc((void**)&b->d_queue, 4 * sizeof(unsigned)) && dmalloc((void**)&b->d_status, sizeof(uint32_t)) &&
       dmalloc((void**)&b->d_counters, 8 * sizeof(unsigned long long));
  ok = ok && dmalloc((void**)&b->d_h2p, sizeof(int) * std::max<long long>(nb, 1));
  ok = ok && dmalloc((void**)&b->d_stage, sizeof(double) * cz::SG_NDOUBLES * std::max<long long>(nb, 1)) &&
       dmalloc((void**)&b->d_stage_u8, 2 * std::max<long long>(nb, 1)) &&
       dmalloc((void**)&b->d_stage_i32, sizeof(int) * std::max<long long>(nb, 1));
  ok = ok && dmalloc((void**)&b->d_cstage, sizeof(double) * cz::C_NROWS * b->max_cap) &&
       dmalloc((void**)&b->d_cstage_b, sizeof(int) * b->max_cap);
  ok = ok && dmalloc((void**)&b->d_pow, sizeof(double) * 2 * P);
  ok = ok && dmalloc(&b->snap_body, R * cz::B_NROWS * P) && dmalloc((void**)&b->snap_u8, 2 * P);
  if (!b->big_ids.empty()) {
    ok = ok && dmalloc((void**)&b->d_big, sizeof(int) * b->big_ids.size()) &&
         dmalloc(&b->big_bw, sizeof(double) * 7 * P) && dmalloc(&b->big_br, R * 20 * P) &&
         dmalloc((void**)&b->big_aw, P) && dmalloc((void**)&b->big_off, sizeof(int) * P) &&
         dmalloc((void**)&b->big_cnt, sizeof(int) * P) && dmalloc((void**)&b->big_adj, sizeof(int) * 2 * C);
  }
  if (!ok) return bail(fail(CZ_ERR_CUDA, "device allocation failed"));
  ok = cudaMallocHost((void**)&b->h_stage, sizeof(double) * cz::SG_NDOUBLES * std::max<long long>(nb, 1)) ==
           cudaSuccess &&
       cudaMallocHost((void**)&b->h_stage_u8, 2 * std::max<long long>(nb, 1)) == cudaSuccess &&
       cudaMallocHost((void**)&b->h_stage_i32, sizeof(int) * std::max<long long>(nb, 1)) == cudaSuccess &&
       cudaMallocHost((void**)&b->h_cstage, sizeof(double) * cz::C_NROWS * b->max_cap) == cudaSuccess &&
       cudaMallocHost((void**)&b->h_cstage_b, sizeof(int) * b->max_cap) == cudaSuccess &&
       cudaMallocHost((void**)&b->h_pow, sizeof(double) * 2 * P) == cudaSuccess &&
       cudaMallocHost((void**)&b->h_status, sizeof(uint32_t)) == cudaSuccess;
  if (!ok) return bail(fail(CZ_ERR_CUDA, "pinned host allocation failed"));
  cudaStream_t s = b->stream;
  std::vector<int> bcount(b->counts);
  if (cudaMemsetAsync(b->body, 0, R * cz::B_NROWS * P, s) != cudaSuccess ||
      cudaMemsetAsync(b->awake, 0, P, s) != cudaSuccess || cudaMemsetAsync(b->can_sleep, 0, P, s) != cudaSuccess ||
      cudaMemsetAsync(b->shape, 0xFF, sizeof(int) * P, s) != cudaSuccess ||
      cudaMemsetAsync(b->d_ccount, 0, sizeof(int) * W, s) != cudaSuccess ||
      cudaMemsetAsync(b->d_wstatus, 0, sizeof(uint32_t) * W, s) != cudaSuccess ||
      cudaMemsetAsync(b->d_piters, 0, sizeof(int) * W, s) != cudaSuccess ||
      cudaMemsetAsync(b->d_viters, 0, sizeof(int) * W, s) != cudaSuccess ||
      cudaMemsetAsync(b->d_queue, 0, 4 * sizeof(unsigned), s) != cudaSuccess ||
      cudaMemsetAsync(b->d_status, 0, sizeof(uint32_t), s) != cudaSuccess ||
      cudaMemsetAsync(b->d_counters, 0, 8 * sizeof(unsigned long long), s) != cudaSuccess ||
      cudaMemsetAsync(b->cbodies, 0xFF, sizeof(int) * C, s) != cudaSuccess ||
      cudaMemcpyAsync(b->d_bstart, b->bstart.data(), sizeof(int) * W, cudaMemcpyHostToDevice, s) != cudaSuccess ||
      cudaMemcpyAsync(b->d_bcount, bcount.data(), sizeof(int) * W, cudaMemcpyHostToDevice, s) != cudaSuccess ||
      cudaMemcpyAsync(b->d_ccap, b->ccap.data(), sizeof(int) * W, cudaMemcpyHostToDevice, s) != cudaSuccess ||
      cudaMemcpyAsync(b->d_cstart, b->cstart.data(), sizeof(long long) * W, cudaMemcpyHostToDevice, s) !=
          cudaSuccess ||
      cudaMemcpyAsync(b->d_order, order.data(), sizeof(int) * W, cudaMemcpyHostToDevice, s) != cudaSuccess ||
      cudaMemcpyAsync(b->d_order_rs, order.data(), sizeof(int) * W, cudaMemcpyHostToDevice, s) != cudaSuccess ||
      (!b->big_ids.empty() && cudaMemcpyAsync(b->d_big, b->big_ids.data(), sizeof(int) * b->big_ids.size(),
                                              cudaMemcpyHostToDevice, s) != cudaSuccess) ||
      (nb > 0 &&
       cudaMemcpyAsync(b->d_h2p, b->h2p.data(), sizeof(int) * nb, cudaMemcpyHostToDevice, s) != cudaSuccess) ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return bail(fail(CZ_ERR_CUDA, "device initialisation failed"));
  b->lin_damp.assign(nb, 0.95);
  b->ang_damp.assign(nb, 0.95);
  st = configure(b);
  if (st != CZ_OK) return bail(st);
  *out = b;
  return CZ_OK;
}

int cz_batch_destroy(cz_batch* b) {
  if (!b) return fail(CZ_ERR_BAD_ARG, "cz_batch_destroy: null batch");
  free_batch(b);
  return CZ_OK;
}

int cz_set_tuning(cz_batch* b, const cz_tuning* t) {
  if (!b || !t) return fail(CZ_ERR_BAD_ARG, "cz_set_tuning: null argument");
  CZ_CUDA(cudaSetDevice(b->device));
  if (t->narrowphase_threads > 0) {
    if (t->narrowphase_threads % 32 != 0 || t->narrowphase_threads > 256)
      return fail(CZ_ERR_BAD_ARG, "narrowphase_threads must be a multiple of 32, at most 256");
    b->np_threads = t->narrowphase_threads;
  }
  if (t->resolver_contacts > 0) b->rs_cs = (int)round_up(t->resolver_contacts, 32);
  if (t->resolver_lanes > 0) {
    if (t->resolver_lanes != 4 && t->resolver_lanes != 8 && t->resolver_lanes != 16 && t->resolver_lanes != 32)
      return fail(CZ_ERR_BAD_ARG, "resolver_lanes must be 4, 8, 16 or 32");
    b->rs_lanes = t->resolver_lanes;
  }
  if (t->resolver_ctas_per_sm > 0) b->rs_ctas_per_sm = t->resolver_ctas_per_sm;
  if (t->integrate_threads > 0) {
    if (t->integrate_threads % 32 != 0 || t->integrate_threads > 256)
      return fail(CZ_ERR_BAD_ARG, "integrate_threads must be a multiple of 32, at most 256");
    b->int_threads = t->integrate_threads;
  }
  if (t->large_world_lanes > 0) {
    if (t->large_world_lanes != 16 && t->large_world_lanes != 32)
      return fail(CZ_ERR_BAD_ARG, "large_world_lanes must be 16 or 32");
    b->big_lanes = t->large_world_lanes;
  }
  if (t->warm_start_budget_shift > 0) {
    if (t->warm_start_budget_shift > 8) return fail(CZ_ERR_BAD_ARG, "warm_start_budget_shift must be 1 to 8");
    b->warm_shift = t->warm_start_budget_shift;
  }
  if (t->fused_frame != 0) b->fused = t->fused_frame > 0 ? 1 : 0;
  if (t->broadphase_min_bodies != 0) {
    if (t->broadphase_min_bodies < -1) return fail(CZ_ERR_BAD_ARG, "broadphase_min_bodies must be -1 or positive");
    b->grid_min_bodies = t->broadphase_min_bodies < 0 ? 0 : t->broadphase_min_bodies;
  }
  return configure(b);
}

int cz_set_wait_test(cz_batch* b, int32_t extra_bytes, int32_t wait_limit) {
  if (!b || extra_bytes < 0 || extra_bytes > 4096 || wait_limit < 0) return CZ_ERR_BAD_ARG;
  b->wait_extra_tx = extra_bytes;
  b->wait_limit = wait_limit > 0 ? wait_limit : (1 << 22);
  drop_graphs(b);
  return CZ_OK;
}

int cz_get_tuning(cz_batch* b, cz_tuning* t) {
  if (!b || !t) return fail(CZ_ERR_BAD_ARG, "cz_get_tuning: null argument");
  t->narrowphase_threads = b->np_threads;
  t->resolver_contacts = b->rs_cs;
  t->resolver_ctas_per_sm = b->rs_grid / std::max(b->sm_count, 1);
  t->integrate_threads = b->int_threads;
  t->resolver_lanes = b->rs_lanes;
  t->warm_start_budget_shift = b->warm_shift;
  t->broadphase_min_bodies = b->grid_min_bodies > 0 ? b->grid_min_bodies : -1;
  t->fused_frame = b->fused ? 1 : -1;
  t->large_world_lanes = b->big_lanes;
  return CZ_OK;
}

int cz_upload_bodies(cz_batch* b, const cz_bodies* in) {
  if (!b || !in) return fail(CZ_ERR_BAD_ARG, "cz_upload_bodies: null argument");
  if (!in->position || !in->orientation || !in->velocity || !in->rotation || !in->acceleration ||
      !in->inverse_inertia || !in->inverse_mass || !in->linear_damping || !in->angular_damping || !in->is_awake ||
      !in->can_sleep || !in->shape || !in->half_size || !in->radius)
    return fail(CZ_ERR_BAD_ARG, "cz_upload_bodies: missing body field");
  CZ_CUDA(cudaSetDevice(b->device));
  const long long n = b->nb;
  if (n == 0) return CZ_OK;
  for (long long h = 0; h < n; ++h)
    if (in->shape[h] != CZ_SHAPE_SPHERE && in->shape[h] != CZ_SHAPE_CUBE)
      return fail(CZ_ERR_BAD_ARG, "cz_upload_bodies: unknown shape");
  double* sg = b->h_stage;
  std::memcpy(sg + cz::SG_POS * n, in->position, sizeof(double) * 3 * n);
  std::memcpy(sg + cz::SG_Q * n, in->orientation, sizeof(double) * 4 * n);
  std::memcpy(sg + cz::SG_VEL * n, in->velocity, sizeof(double) * 3 * n);
  std::memcpy(sg + cz::SG_ROT * n, in->rotation, sizeof(double) * 3 * n);
  std::memcpy(sg + cz::SG_ACC * n, in->acceleration, sizeof(double) * 3 * n);
  std::memcpy(sg + cz::SG_IB * n, in->inverse_inertia, sizeof(double) * 9 * n);
  std::memcpy(sg + cz::SG_INVM * n, in->inverse_mass, sizeof(double) * n);
  if (in->motion) std::memcpy(sg + cz::SG_MOTION * n, in->motion, sizeof(double) * n);
  else for (long long h = 0; h < n; ++h) sg[cz::SG_MOTION * n + h] = 0.3 * 2.0;
  std::memcpy(sg + cz::SG_HALF * n, in->half_size, sizeof(double) * 3 * n);
  std::memcpy(sg + cz::SG_RAD * n, in->radius, sizeof(double) * n);
  const int has_iw = in->inverse_inertia_world != nullptr;
  const int has_lfa = in->last_frame_acceleration != nullptr;
  if (has_iw) std::memcpy(sg + cz::SG_IW * n, in->inverse_inertia_world, sizeof(double) * 9 * n);
  if (has_lfa) std::memcpy(sg + cz::SG_LFA * n, in->last_frame_acceleration, sizeof(double) * 3 * n);
  std::memcpy(b->h_stage_u8, in->is_awake, n);
  std::memcpy(b->h_stage_u8 + n, in->can_sleep, n);
  std::memcpy(b->h_stage_i32, in->shape, sizeof(int) * n);
  const bool has_off = in->collider_offset != nullptr;
  if (has_off && !b->d_offset) {
    const size_t rows = b->ops->real_size * 12 * std::max<long long>(b->nb_pad, 1);
    void* rows_d = nullptr;
    double *stage_d = nullptr, *stage_h = nullptr;
    if (cudaMalloc(&rows_d, rows) != cudaSuccess ||
        cudaMalloc((void**)&stage_d, sizeof(double) * 12 * n) != cudaSuccess ||
        cudaMallocHost((void**)&stage_h, sizeof(double) * 12 * n) != cudaSuccess) {
      if (rows_d) cudaFree(rows_d);
      if (stage_d) cudaFree(stage_d);
      return fail(CZ_ERR_CUDA, "cz_upload_bodies: Offset allocation failed");
    }
    b->d_offset = rows_d;
    b->d_off_stage = stage_d;
    b->h_off_stage = stage_h;
    CZ_CUDA(cudaMemsetAsync(b->d_offset, 0, rows, b->stream));
  }
  if (has_off != b->has_offset) {
    drop_graphs(b);  // the narrowphase's view changes
    b->has_offset = has_off;
  }
  if (has_off) {
    std::memcpy(b->h_off_stage, in->collider_offset, sizeof(double) * 12 * n);
    CZ_CUDA(cudaMemcpyAsync(b->d_off_stage, b->h_off_stage, sizeof(double) * 12 * n, cudaMemcpyHostToDevice,
                            b->stream));
  }
  b->lin_damp.assign(in->linear_damping, in->linear_damping + n);
  b->ang_damp.assign(in->angular_damping, in->angular_damping + n);
  b->pow_dt = std::nan("");
  CZ_CUDA(cudaMemcpyAsync(b->d_stage, sg, sizeof(double) * cz::SG_NDOUBLES * n, cudaMemcpyHostToDevice, b->stream));
  CZ_CUDA(cudaMemcpyAsync(b->d_stage_u8, b->h_stage_u8, 2 * n, cudaMemcpyHostToDevice, b->stream));
  CZ_CUDA(cudaMemcpyAsync(b->d_stage_i32, b->h_stage_i32, sizeof(int) * n, cudaMemcpyHostToDevice, b->stream));
  CZ_CUDA(b->ops->upload(b->view(), b->d_stage, b->d_stage_u8, b->d_stage_i32, b->d_h2p, (int)n, has_iw, has_lfa,
                         has_off ? b->d_off_stage : nullptr, b->stream));
  g_launches++;
  CZ_CUDA(cudaStreamSynchronize(b->stream));
  return CZ_OK;
}

int cz_download_bodies(cz_batch* b, cz_bodies* out) {
  if (!b || !out) return fail(CZ_ERR_BAD_ARG, "cz_download_bodies: null argument");
  CZ_CUDA(cudaSetDevice(b->device));
  const long long n = b->nb;
  if (n == 0) return CZ_OK;
  const bool want_off = out->collider_offset && b->has_offset;
  CZ_CUDA(b->ops->download(b->view(), b->d_stage, b->d_stage_u8, b->d_stage_i32, b->d_h2p, (int)n,
                           want_off ? b->d_off_stage : nullptr, b->stream));
  g_launches++;
  if (want_off)
    CZ_CUDA(cudaMemcpyAsync(b->h_off_stage, b->d_off_stage, sizeof(double) * 12 * n, cudaMemcpyDeviceToHost,
                            b->stream));
  CZ_CUDA(cudaMemcpyAsync(b->h_stage, b->d_stage, sizeof(double) * cz::SG_NDOUBLES * n, cudaMemcpyDeviceToHost,
                          b->stream));
  CZ_CUDA(cudaMemcpyAsync(b->h_stage_u8, b->d_stage_u8, 2 * n, cudaMemcpyDeviceToHost, b->stream));
  CZ_CUDA(cudaMemcpyAsync(b->h_stage_i32, b->d_stage_i32, sizeof(int) * n, cudaMemcpyDeviceToHost, b->stream));
  CZ_CUDA(cudaStreamSynchronize(b->stream));
  const double* sg = b->h_stage;
  auto cp = [&](double* dst, int blk, int width) {
    if (dst) std::memcpy(dst, sg + (long long)blk * n, sizeof(double) * width * n);
  };
  cp(out->position, cz::SG_POS, 3);
  cp(out->orientation, cz::SG_Q, 4);
  cp(out->velocity, cz::SG_VEL, 3);
  cp(out->rotation, cz::SG_ROT, 3);
  cp(out->acceleration, cz::SG_ACC, 3);
  cp(out->inverse_inertia, cz::SG_IB, 9);
  cp(out->inverse_mass, cz::SG_INVM, 1);
  cp(out->motion, cz::SG_MOTION, 1);
  cp(out->half_size, cz::SG_HALF, 3);
  cp(out->radius, cz::SG_RAD, 1);
  cp(out->inverse_inertia_world, cz::SG_IW, 9);
  cp(out->last_frame_acceleration, cz::SG_LFA, 3);
  if (out->linear_damping) std::memcpy(out->linear_damping, b->lin_damp.data(), sizeof(double) * n);
  if (out->angular_damping) std::memcpy(out->angular_damping, b->ang_damp.data(), sizeof(double) * n);
  if (out->is_awake) std::memcpy(out->is_awake, b->h_stage_u8, n);
  if (out->can_sleep) std::memcpy(out->can_sleep, b->h_stage_u8 + n, n);
  if (want_off) {
    std::memcpy(out->collider_offset, b->h_off_stage, sizeof(double) * 12 * n);
  } else if (out->collider_offset) {
    static const double id[12] = {1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0};
    for (long long h = 0; h < n; ++h) std::memcpy(out->collider_offset + 12 * h, id, sizeof id);
  }
  if (out->shape) std::memcpy(out->shape, b->h_stage_i32, sizeof(int) * n);
  return CZ_OK;
}

int cz_integrate(cz_batch* b, double dt) {
  if (!b) return fail(CZ_ERR_BAD_ARG, "cz_integrate: null batch");
  CZ_CUDA(cudaSetDevice(b->device));
  int st = ensure_pows(b, dt);
  if (st) return st;
  if ((st = reset_status(b))) return st;
  if ((st = launch_integrate(b, dt))) return st;
  return finish(b);
}

int cz_narrowphase(cz_batch* b) {
  if (!b) return fail(CZ_ERR_BAD_ARG, "cz_narrowphase: null batch");
  CZ_CUDA(cudaSetDevice(b->device));
  int st = reset_status(b);
  if (st) return st;
  if ((st = launch_narrowphase(b))) return st;
  return finish(b);
}

int cz_resolve(cz_batch* b, double dt) {
  if (!b) return fail(CZ_ERR_BAD_ARG, "cz_resolve: null batch");
  CZ_CUDA(cudaSetDevice(b->device));
  int st = reset_status(b);
  if (st) return st;
  if ((st = launch_resolve(b, dt))) return st;
  return finish(b);
}

// Capture (once per (nsteps, dt)) the plain rollout graph.
static int get_graph(cz_batch* b, int nsteps, double dt, cudaGraphExec_t* out) {
  auto key = std::make_pair(nsteps, dt);
  auto it = b->graphs.find(key);
  if (it != b->graphs.end()) {
    *out = it->second;
    return CZ_OK;
  }
  CZ_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  const long long before = g_launches.load();
  int cst = CZ_OK;
  const bool fused = uses_frame(b);
  for (int s = 0; s < nsteps && cst == CZ_OK; ++s) {
    if (fused) {
      cst = launch_frame(b, dt);
      continue;
    }
    cst = launch_integrate(b, dt);
    if (!cst) cst = launch_narrowphase(b);
    if (!cst) cst = launch_resolve(b, dt);
  }
  g_launches.store(before);  // captured launches are counted when the graph runs
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamEndCapture(b->stream, &graph);
  if (cst != CZ_OK) {
    if (graph) cudaGraphDestroy(graph);
    return cst;
  }
  if (e != cudaSuccess) return fail(CZ_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
  cudaGraphExec_t exec = nullptr;
  e = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return fail(CZ_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
  b->graphs.emplace(key, exec);
  *out = exec;
  return CZ_OK;
}

// Capture the rollout with event-record nodes around every phase.
static int get_timed(cz_batch* b, int nsteps, double dt, cz_batch::Timed** out) {
  auto key = std::make_pair(nsteps, dt);
  auto it = b->timed.find(key);
  if (it != b->timed.end()) {
    *out = &it->second;
    return CZ_OK;
  }
  cz_batch::Timed t;
  t.ev.resize(3 * (size_t)nsteps + 1);
  for (auto& e : t.ev) CZ_CUDA(cudaEventCreate(&e));
  CZ_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  const long long before = g_launches.load();
  auto record = [&](int k) {
    return cudaEventRecordWithFlags(t.ev[k], b->stream, cudaEventRecordExternal) == cudaSuccess ? CZ_OK
                                                                                                : CZ_ERR_CUDA;
  };
  int cst = record(0);
  const bool fused = uses_frame(b);
  for (int s = 0; s < nsteps && cst == CZ_OK; ++s) {
    if (fused) {  // one launch: its time is reported as the resolve phase
      cst = record(3 * s + 1);
      if (!cst) cst = record(3 * s + 2);
      if (!cst) cst = launch_frame(b, dt);
      if (!cst) cst = record(3 * s + 3);
      continue;
    }
    cst = launch_integrate(b, dt);
    if (!cst) cst = record(3 * s + 1);
    if (!cst) cst = launch_narrowphase(b);
    if (!cst) cst = record(3 * s + 2);
    if (!cst) cst = launch_resolve(b, dt);
    if (!cst) cst = record(3 * s + 3);
  }
  g_launches.store(before);
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamEndCapture(b->stream, &graph);
  if (cst != CZ_OK || e != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    for (auto& ev : t.ev) cudaEventDestroy(ev);
    return fail(CZ_ERR_CUDA, "timed graph capture failed");
  }
  e = cudaGraphInstantiate(&t.exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) {
    for (auto& ev : t.ev) cudaEventDestroy(ev);
    return fail(CZ_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
  }
  *out = &b->timed.emplace(key, std::move(t)).first->second;
  return CZ_OK;
}

int cz_step(cz_batch* b, int32_t nsteps, double dt) {
  if (!b || nsteps < 0) return fail(CZ_ERR_BAD_ARG, "cz_step: bad argument");
  if (nsteps == 0) return CZ_OK;
  CZ_CUDA(cudaSetDevice(b->device));
  int st = ensure_pows(b, dt);
  if (st) return st;
  if ((st = reset_status(b))) return st;
  cudaGraphExec_t exec = nullptr;
  if ((st = get_graph(b, nsteps, dt, &exec))) return st;
  CZ_CUDA(cudaGraphLaunch(exec, b->stream));
  g_launches += (long long)launches_per_step(b) * nsteps;
  return finish(b);
}

int cz_prepare_rollout(cz_batch* b, int32_t nsteps, double dt) {
  if (!b || nsteps <= 0) return fail(CZ_ERR_BAD_ARG, "cz_prepare_rollout: bad argument");
  CZ_CUDA(cudaSetDevice(b->device));
  int st = ensure_pows(b, dt);
  if (st) return st;
  cudaGraphExec_t exec = nullptr;
  if ((st = get_graph(b, nsteps, dt, &exec))) return st;
  cz_batch::Timed* t = nullptr;
  return get_timed(b, nsteps, dt, &t);
}

int cz_contact_counts(cz_batch* b, int32_t* counts) {
  if (!b || !counts) return fail(CZ_ERR_BAD_ARG, "cz_contact_counts: null argument");
  CZ_CUDA(cudaSetDevice(b->device));
  CZ_CUDA(cudaMemcpyAsync(counts, b->d_ccount, sizeof(int) * b->num_worlds, cudaMemcpyDeviceToHost, b->stream));
  CZ_CUDA(cudaStreamSynchronize(b->stream));
  return CZ_OK;
}

int cz_download_contacts(cz_batch* b, int32_t world, cz_contact* out, int32_t capacity, int32_t* count) {
  if (!b || world < 0 || world >= b->num_worlds || (capacity > 0 && !out))
    return fail(CZ_ERR_BAD_ARG, "cz_download_contacts: bad argument");
  CZ_CUDA(cudaSetDevice(b->device));
  int n = 0;
  CZ_CUDA(cudaMemcpyAsync(&n, b->d_ccount + world, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
  CZ_CUDA(cudaStreamSynchronize(b->stream));
  if (count) *count = n;
  int m = std::min(n, b->ccap[world]);
  m = std::min(m, std::max(capacity, 0));
  if (m <= 0) return n > b->ccap[world] ? fail(CZ_ERR_CAPACITY, "world exceeded its contact capacity") : CZ_OK;
  CZ_CUDA(b->ops->contacts_out(b->view(), b->cstart[world], m, b->d_cstage, b->d_cstage_b, b->stream));
  g_launches++;
  CZ_CUDA(cudaMemcpyAsync(b->h_cstage, b->d_cstage, sizeof(double) * cz::C_NROWS * m, cudaMemcpyDeviceToHost,
                          b->stream));
  CZ_CUDA(cudaMemcpyAsync(b->h_cstage_b, b->d_cstage_b, sizeof(int) * m, cudaMemcpyDeviceToHost, b->stream));
  CZ_CUDA(cudaStreamSynchronize(b->stream));
  for (int k = 0; k < m; ++k) {
    const double* c = b->h_cstage + (long long)k * cz::C_NROWS;
    cz_contact& o = out[k];
    o.body[0] = cz::body0_of(b->h_cstage_b[k]);
    o.body[1] = cz::body1_of(b->h_cstage_b[k]);
    o.point[0] = c[cz::C_PX]; o.point[1] = c[cz::C_PY]; o.point[2] = c[cz::C_PZ];
    o.normal[0] = c[cz::C_NX]; o.normal[1] = c[cz::C_NY]; o.normal[2] = c[cz::C_NZ];
    o.penetration = c[cz::C_PEN];
    o.friction = c[cz::C_FRIC];
    o.restitution = c[cz::C_REST];
  }
  if (n > b->ccap[world]) return fail(CZ_ERR_CAPACITY, "world exceeded its contact capacity");
  return CZ_OK;
}

int cz_world_stats(cz_batch* b, int32_t* pos_it, int32_t* vel_it, uint32_t* status) {
  if (!b) return fail(CZ_ERR_BAD_ARG, "cz_world_stats: null batch");
  CZ_CUDA(cudaSetDevice(b->device));
  const size_t W = b->num_worlds;
  if (pos_it) CZ_CUDA(cudaMemcpyAsync(pos_it, b->d_piters, sizeof(int) * W, cudaMemcpyDeviceToHost, b->stream));
  if (vel_it) CZ_CUDA(cudaMemcpyAsync(vel_it, b->d_viters, sizeof(int) * W, cudaMemcpyDeviceToHost, b->stream));
  if (status) CZ_CUDA(cudaMemcpyAsync(status, b->d_wstatus, sizeof(uint32_t) * W, cudaMemcpyDeviceToHost, b->stream));
  CZ_CUDA(cudaStreamSynchronize(b->stream));
  return CZ_OK;
}

int cz_resolve_contacts(cz_batch* b, int32_t max_iterations, cz_contact* contacts, int32_t ncontacts,
                        double duration, cz_bodies* bodies) {
  if (!b || !bodies || ncontacts < 0 || (ncontacts > 0 && !contacts))
    return fail(CZ_ERR_BAD_ARG, "cz_resolve_contacts: bad argument");
  if (b->num_worlds != 1) return fail(CZ_ERR_BAD_ARG, "cz_resolve_contacts: the batch must hold one world");
  if (ncontacts > b->ccap[0]) return fail(CZ_ERR_CAPACITY, "cz_resolve_contacts: more contacts than capacity");
  // ResolveContacts' own guards (contact.go:210-212): nothing changes
  if (duration <= 0.0 || ncontacts == 0) return CZ_OK;
  const int n = b->counts[0];
  for (int k = 0; k < ncontacts; ++k) {
    const int b0 = contacts[k].body[0], b1 = contacts[k].body[1];
    if (b0 < -1 || b0 >= n || b1 < -1 || b1 >= n || (b0 < 0 && b1 < 0))
      return fail(CZ_ERR_BAD_ARG, "cz_resolve_contacts: contact body index out of range");
  }
  int st = cz_upload_bodies(b, bodies);
  if (st) return st;
  CZ_CUDA(cudaSetDevice(b->device));
  for (int k = 0; k < ncontacts; ++k) {
    double* c = b->h_cstage + (long long)k * cz::C_NROWS;
    const cz_contact& s = contacts[k];
    c[cz::C_PX] = s.point[0]; c[cz::C_PY] = s.point[1]; c[cz::C_PZ] = s.point[2];
    c[cz::C_NX] = s.normal[0]; c[cz::C_NY] = s.normal[1]; c[cz::C_NZ] = s.normal[2];
    c[cz::C_PEN] = s.penetration;
    c[cz::C_FRIC] = s.friction;
    c[cz::C_REST] = s.restitution;
    b->h_cstage_b[k] = cz::pack_bodies(s.body[0], s.body[1]);
  }
  CZ_CUDA(cudaMemcpyAsync(b->d_cstage, b->h_cstage, sizeof(double) * cz::C_NROWS * ncontacts, cudaMemcpyHostToDevice,
                          b->stream));
  CZ_CUDA(cudaMemcpyAsync(b->d_cstage_b, b->h_cstage_b, sizeof(int) * ncontacts, cudaMemcpyHostToDevice, b->stream));
  CZ_CUDA(b->ops->contacts_in(b->view(), b->cstart[0], ncontacts, b->d_cstage, b->d_cstage_b, b->stream));
  g_launches++;
  CZ_CUDA(cudaMemcpyAsync(b->d_ccount, &ncontacts, sizeof(int), cudaMemcpyHostToDevice, b->stream));
  if ((st = reset_status(b))) return st;
  cz::HostView v = b->view();
  v.max_iterations = std::max(max_iterations, 0);
  v.contact_writeback = 1;
  v.uniform_material = 0;
  if ((st = launch_resolve(b, duration, &v))) return st;
  st = finish(b);
  if (st != CZ_OK && st != CZ_ERR_FRICTIONLESS) return st;
  const int st2 = cz_download_bodies(b, bodies);
  if (st2) return st2;
  // write the resolved contacts back (penetration, swapped bodies/normal)
  CZ_CUDA(b->ops->contacts_out(b->view(), b->cstart[0], ncontacts, b->d_cstage, b->d_cstage_b, b->stream));
  g_launches++;
  CZ_CUDA(cudaMemcpyAsync(b->h_cstage, b->d_cstage, sizeof(double) * cz::C_NROWS * ncontacts, cudaMemcpyDeviceToHost,
                          b->stream));
  CZ_CUDA(cudaMemcpyAsync(b->h_cstage_b, b->d_cstage_b, sizeof(int) * ncontacts, cudaMemcpyDeviceToHost, b->stream));
  CZ_CUDA(cudaStreamSynchronize(b->stream));
  for (int k = 0; k < ncontacts; ++k) {
    const double* c = b->h_cstage + (long long)k * cz::C_NROWS;
    contacts[k].body[0] = cz::body0_of(b->h_cstage_b[k]);
    contacts[k].body[1] = cz::body1_of(b->h_cstage_b[k]);
    contacts[k].normal[0] = c[cz::C_NX];
    contacts[k].normal[1] = c[cz::C_NY];
    contacts[k].normal[2] = c[cz::C_NZ];
    contacts[k].penetration = c[cz::C_PEN];
  }
  return st;
}

int cz_snapshot(cz_batch* b) {
  if (!b) return fail(CZ_ERR_BAD_ARG, "cz_snapshot: null batch");
  CZ_CUDA(cudaSetDevice(b->device));
  const size_t bytes = b->ops->real_size * cz::B_NROWS * b->nb_pad;
  CZ_CUDA(cudaMemcpyAsync(b->snap_body, b->body, bytes, cudaMemcpyDeviceToDevice, b->stream));
  CZ_CUDA(cudaMemcpyAsync(b->snap_u8, b->awake, b->nb_pad, cudaMemcpyDeviceToDevice, b->stream));
  CZ_CUDA(cudaMemcpyAsync(b->snap_u8 + b->nb_pad, b->can_sleep, b->nb_pad, cudaMemcpyDeviceToDevice, b->stream));
  CZ_CUDA(cudaStreamSynchronize(b->stream));
  b->snap_pow_dt = b->pow_dt;
  return CZ_OK;
}

int cz_restore(cz_batch* b) {
  if (!b) return fail(CZ_ERR_BAD_ARG, "cz_restore: null batch");
  CZ_CUDA(cudaSetDevice(b->device));
  const size_t bytes = b->ops->real_size * cz::B_NROWS * b->nb_pad;
  CZ_CUDA(cudaMemcpyAsync(b->body, b->snap_body, bytes, cudaMemcpyDeviceToDevice, b->stream));
  CZ_CUDA(cudaMemcpyAsync(b->awake, b->snap_u8, b->nb_pad, cudaMemcpyDeviceToDevice, b->stream));
  CZ_CUDA(cudaMemcpyAsync(b->can_sleep, b->snap_u8 + b->nb_pad, b->nb_pad, cudaMemcpyDeviceToDevice, b->stream));
  CZ_CUDA(cudaStreamSynchronize(b->stream));
  b->pow_dt = b->snap_pow_dt;  // the snapshot holds the damping factors of its own dt
  return CZ_OK;
}

int cz_step_timed(cz_batch* b, int32_t nsteps, double dt, double* total_ms, double* phase_ms) {
  if (!b || nsteps <= 0) return fail(CZ_ERR_BAD_ARG, "cz_step_timed: bad argument");
  CZ_CUDA(cudaSetDevice(b->device));
  int st = ensure_pows(b, dt);
  if (st) return st;
  if ((st = reset_status(b))) return st;
  cz_batch::Timed* t = nullptr;
  if ((st = get_timed(b, nsteps, dt, &t))) return st;
  CZ_CUDA(cudaGraphLaunch(t->exec, b->stream));
  g_launches += (long long)launches_per_step(b) * nsteps;
  st = finish(b);
  double ph[3] = {0, 0, 0};
  const bool fused = uses_frame(b);
  for (int s = 0; s < nsteps; ++s)
    if (fused) {  // the whole frame (with the gaps between its event nodes) is the resolve phase
      float ms = 0.f;
      CZ_CUDA(cudaEventElapsedTime(&ms, t->ev[3 * s], t->ev[3 * s + 3]));
      ph[2] += ms;
    } else
      for (int k = 0; k < 3; ++k) {
        float ms = 0.f;
        CZ_CUDA(cudaEventElapsedTime(&ms, t->ev[3 * s + k], t->ev[3 * s + k + 1]));
        ph[k] += ms;
      }
  float tot = 0.f;
  CZ_CUDA(cudaEventElapsedTime(&tot, t->ev[0], t->ev[3 * (size_t)nsteps]));
  if (total_ms) *total_ms = tot;
  if (phase_ms)
    for (int k = 0; k < 3; ++k) phase_ms[k] = ph[k];
  return st;
}

// The per-body scratch of the warm start and the harvest.
static int ensure_ws(cz_batch* b) {
  if (b->ws_rows) return CZ_OK;
  const size_t P = (size_t)b->nb_pad;
  CZ_CUDA(cudaMalloc(&b->ws_rows, b->ops->real_size * 13 * P));
  CZ_CUDA(cudaMalloc((void**)&b->ws_int, sizeof(int) * cz::WS_NINT * P));
  CZ_CUDA(cudaMalloc((void**)&b->ws_u8, 2 * P));
  CZ_CUDA(cudaMalloc((void**)&b->ws_world, (size_t)b->num_worlds));
  CZ_CUDA(cudaMemset(b->ws_world, 0, (size_t)b->num_worlds));
  return CZ_OK;
}

int cz_collide(cz_batch* b, int32_t world, const double* plane, const int32_t* units, int32_t nunits) {
  if (!b || world < 0 || world >= b->num_worlds || nunits < 0 || (nunits > 0 && !units))
    return fail(CZ_ERR_BAD_ARG, "cz_collide: bad argument");
  const int n = b->counts[world];
  for (int u = 0; u < nunits; ++u) {
    const int i = units[2 * u], j = units[2 * u + 1];
    if (i < 0 || i >= n || j < -1 || j >= n || j == i)
      return fail(CZ_ERR_BAD_ARG, "cz_collide: unit " + std::to_string(u) + " is not (body, other body or -1)");
  }
  CZ_CUDA(cudaSetDevice(b->device));
  if (nunits > b->units_cap) {
    cudaFree(b->d_units);
    b->d_units = nullptr;
    b->units_cap = 0;
    CZ_CUDA(cudaMalloc((void**)&b->d_units, sizeof(int) * 2 * (size_t)nunits));
    b->units_cap = nunits;
  }
  if (nunits > 0)
    CZ_CUDA(cudaMemcpyAsync(b->d_units, units, sizeof(int) * 2 * (size_t)nunits, cudaMemcpyHostToDevice, b->stream));
  int st = reset_status(b);
  if (st) return st;
  cz::HostView v = b->view();
  if (plane)
    for (int k = 0; k < 4; ++k) v.plane[k] = plane[k];
  CZ_CUDA(b->ops->collide(v, world, b->d_units, nunits, b->nbs, b->np_smem, b->stream));
  g_launches++;
  return finish(b);
}

int cz_set_warm_start(cz_batch* b, const float* blob) {
  if (!b) return fail(CZ_ERR_BAD_ARG, "cz_set_warm_start: null batch");
  CZ_CUDA(cudaSetDevice(b->device));
  if (!blob) {
    b->mode = 0;
    return configure(b);
  }
  if (int st = ensure_ws(b)) return st;
  const size_t blob_bytes = sizeof(float) * cz::MLP_BLOB;
  const size_t off = (blob_bytes + 255) & ~(size_t)255;
  if (!b->mlp_mem) CZ_CUDA(cudaMalloc(&b->mlp_mem, off + cz::mlp_packed_bytes()));
  unsigned char* mem = static_cast<unsigned char*>(b->mlp_mem);
  CZ_CUDA(cudaMemcpyAsync(mem, blob, blob_bytes, cudaMemcpyHostToDevice, b->stream));
  CZ_CUDA(cz::mlp_pack(reinterpret_cast<const float*>(mem), mem + off, b->stream));
  CZ_CUDA(cudaStreamSynchronize(b->stream));
  b->mlp = cz::mlp_view(mem + off);
  b->mode = 2;
  return configure(b);
}

int cz_harvest(cz_batch* b, int32_t nsteps, double dt, int32_t every, float* features, float* labels,
               int64_t capacity, int64_t* count) {
  if (!b || nsteps < 0 || every <= 0 || capacity < 0 || (capacity > 0 && (!features || !labels)))
    return fail(CZ_ERR_BAD_ARG, "cz_harvest: bad argument");
  CZ_CUDA(cudaSetDevice(b->device));
  if (capacity > b->hv_cap) {
    cudaFree(b->hv_features);
    cudaFree(b->hv_labels);
    b->hv_features = b->hv_labels = nullptr;
    b->hv_cap = 0;
    CZ_CUDA(cudaMalloc((void**)&b->hv_features, sizeof(float) * cz::MLP_IN * std::max<int64_t>(capacity, 1)));
    CZ_CUDA(cudaMalloc((void**)&b->hv_labels, sizeof(float) * cz::MLP_OUT * std::max<int64_t>(capacity, 1)));
    b->hv_cap = capacity;
  }
  if (!b->hv_count) CZ_CUDA(cudaMalloc((void**)&b->hv_count, sizeof(unsigned long long)));
  if (int st0 = ensure_ws(b)) return st0;
  if (!b->ws_feat) CZ_CUDA(cudaMalloc((void**)&b->ws_feat, sizeof(float) * cz::MLP_IN * (size_t)b->nc_total));
  CZ_CUDA(cudaMemsetAsync(b->hv_count, 0, sizeof(unsigned long long), b->stream));
  int st = ensure_pows(b, dt);
  if (st) return st;
  if ((st = reset_status(b))) return st;
  // the plain resolver, writing features and applied impulses every `every` frames
  const int saved_mode = b->mode;
  int cs = b->rs_cs;
  while (cs > 32 && b->ops->rs_smem(b->rs_nbs, cs, b->rs_lanes, 1) > b->smem_optin) cs -= 32;
  const size_t smem1 = b->ops->rs_smem(b->rs_nbs, cs, b->rs_lanes, 1);
  CZ_CUDA(b->ops->prepare(b->np_smem, smem1, b->rs_lanes));
  for (int s = 0; s < nsteps && st == CZ_OK; ++s) {
    st = launch_integrate(b, dt);
    if (!st) st = launch_narrowphase(b);
    if (!st) {
      const bool h = (s % every) == every - 1;
      cz::HostView v = b->view();
      v.mode = h ? 1 : 0;
      v.hv_cap = b->hv_cap;
      st = launch_resolve_with(b, dt, v, h ? cs : b->rs_cs, h ? smem1 : b->rs_smem);
    }
  }
  b->mode = saved_mode;
  if (st) return st;
  st = finish(b);
  unsigned long long n = 0;
  CZ_CUDA(cudaMemcpy(&n, b->hv_count, sizeof n, cudaMemcpyDeviceToHost));
  const int64_t m = std::min<int64_t>((int64_t)n, capacity);
  if (m > 0) {
    CZ_CUDA(cudaMemcpy(features, b->hv_features, sizeof(float) * cz::MLP_IN * m, cudaMemcpyDeviceToHost));
    CZ_CUDA(cudaMemcpy(labels, b->hv_labels, sizeof(float) * cz::MLP_OUT * m, cudaMemcpyDeviceToHost));
  }
  if (count) *count = m;
  return st;
}

int cz_counters(cz_batch* b, int64_t* out, int32_t reset) {
  if (!b) return fail(CZ_ERR_BAD_ARG, "cz_counters: null batch");
  CZ_CUDA(cudaSetDevice(b->device));
  unsigned long long c[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  CZ_CUDA(cudaMemcpyAsync(c, b->d_counters, sizeof c, cudaMemcpyDeviceToHost, b->stream));
  if (reset) CZ_CUDA(cudaMemsetAsync(b->d_counters, 0, sizeof c, b->stream));
  CZ_CUDA(cudaStreamSynchronize(b->stream));
  if (out)
    for (int i = 0; i < 8; ++i) out[i] = (int64_t)c[i];
  return CZ_OK;
}

int cz_batch_info(cz_batch* b, int64_t* info) {
  if (!b || !info) return fail(CZ_ERR_BAD_ARG, "cz_batch_info: null argument");
  info[0] = b->nb;
  info[1] = b->nb_pad;
  info[2] = b->nc_total;
  info[3] = (int64_t)b->ops->real_size;
  info[4] = b->sm_count;
  info[5] = b->np_grid;
  info[6] = b->rs_grid;
  info[7] = (int64_t)b->np_smem;
  info[8] = (int64_t)b->rs_smem;
  return CZ_OK;
}

}  // extern "C"
