// Kernel instantiation and launch wrappers for one form; included by
// cz_fp64.cu / cz_fp32.cu with CZ_R, CZ_W and CZ_FORM_NAME defined.
#pragma once
#include "cz_forms.h"
#include "cz_kernels.cuh"

namespace cz {
namespace CZ_FORM_NS {

using R = CZ_R;
using W = CZ_W;

static BatchView<R> view_of(const HostView& h) {
  BatchView<R> v;
  v.body = static_cast<R*>(h.body);
  v.awake = h.awake;
  v.can_sleep = h.can_sleep;
  v.shape = h.shape;
  v.offset = static_cast<const R*>(h.offset);
  v.nb_pad = h.nb_pad;
  v.num_worlds = h.num_worlds;
  v.max_bodies = h.max_bodies;
  v.body_start = h.body_start;
  v.body_count = h.body_count;
  v.contact_start = h.contact_start;
  v.contact_cap = h.contact_cap;
  v.contact_count = h.contact_count;
  v.world_status = h.world_status;
  v.pos_iters = h.pos_iters;
  v.vel_iters = h.vel_iters;
  v.contact = static_cast<R*>(h.contact);
  v.contact_bodies = h.contact_bodies;
  v.work = static_cast<R*>(h.work);
  v.kmat = static_cast<R*>(h.kmat);
  v.work_bodies = h.work_bodies;
  v.nc_total = h.nc_total;
  v.order = h.order;
  v.order_rs = h.order_rs;
  v.queue = h.queue;
  v.status = h.status;
  v.counters = h.counters;
  v.plane_nx = (R)h.plane[0];
  v.plane_ny = (R)h.plane[1];
  v.plane_nz = (R)h.plane[2];
  v.plane_offset = (R)h.plane[3];
  v.iter_mult = h.iter_mult;
  v.max_iterations = h.max_iterations;
  v.contact_writeback = h.contact_writeback;
  v.uniform_material = h.uniform_material;
  v.mode = h.mode;
  v.mlp = h.mlp;
  v.hv_features = h.hv_features;
  v.hv_labels = h.hv_labels;
  v.hv_count = h.hv_count;
  v.hv_cap = h.hv_cap;
  v.ws_rows = static_cast<R*>(h.ws_rows);
  v.ws_int = h.ws_int;
  v.ws_u8 = h.ws_u8;
  v.ws_world = h.ws_world;
  v.ws_feat = h.ws_feat;
  v.warm_shift = h.warm_shift;
  v.big_list = h.big_list;
  v.big_count = h.big_count;
  v.big_bw = h.big_bw;
  v.big_br = static_cast<R*>(h.big_br);
  v.big_aw = h.big_aw;
  v.big_off = h.big_off;
  v.big_cnt = h.big_cnt;
  v.big_adj = h.big_adj;
  v.wait_limit = h.wait_limit;
  v.wait_extra_tx = h.wait_extra_tx;
  v.grid_min_bodies = h.grid_min_bodies;
  return v;
}

// Host body data (staged AoS doubles) -> device rows, then
// CalculateDerivedData where no world inertia was given.
__global__ void k_upload(BatchView<R> v, const double* __restrict__ sg, const uint8_t* __restrict__ u8,
                         const int* __restrict__ i32, const int* __restrict__ h2p, int nb, int has_iw, int has_lfa,
                         const double* __restrict__ off) {
  const int h = blockIdx.x * blockDim.x + threadIdx.x;
  if (h >= nb) return;
  const long long p = h2p[h];
  const long long S = v.nb_pad;
  const long long n = nb;
  R* b = v.body + p;
  for (int k = 0; k < 3; ++k) {
    b[(B_PX + k) * S] = (R)sg[SG_POS * n + 3 * h + k];
    b[(B_VX + k) * S] = (R)sg[SG_VEL * n + 3 * h + k];
    b[(B_RX + k) * S] = (R)sg[SG_ROT * n + 3 * h + k];
    b[(B_AX + k) * S] = (R)sg[SG_ACC * n + 3 * h + k];
    b[(B_HX + k) * S] = (R)sg[SG_HALF * n + 3 * h + k];
    b[(B_LX + k) * S] = has_lfa ? (R)sg[SG_LFA * n + 3 * h + k] : (R)0;
  }
  q4<R> q{(R)sg[SG_Q * n + 4 * h], (R)sg[SG_Q * n + 4 * h + 1], (R)sg[SG_Q * n + 4 * h + 2],
          (R)sg[SG_Q * n + 4 * h + 3]};
  m3<R> ib;
  for (int k = 0; k < 9; ++k) ib.m[k] = (R)sg[SG_IB * n + 9 * h + k];
  m3<R> iw;
  if (has_iw) {
    for (int k = 0; k < 9; ++k) iw.m[k] = (R)sg[SG_IW * n + 9 * h + k];
  } else {
    // RigidBody.CalculateDerivedData, rigidbody.go:268-272
    q4<W> qw = cvtq<W>(q);
    qnormalize_island<R, W>(qw);
    q = cvtq<R>(qw);
    R rm[9];
    rotation_of(q, rm);
    iw = world_inertia(rm, ib);
  }
  b[B_QW * S] = q.w; b[B_QX * S] = q.x; b[B_QY * S] = q.y; b[B_QZ * S] = q.z;
  for (int k = 0; k < 9; ++k) {
    b[(B_IB0 + k) * S] = ib.m[k];
    b[(B_IW0 + k) * S] = iw.m[k];
  }
  b[B_INVM * S] = (R)sg[SG_INVM * n + h];
  b[B_MOTION * S] = (R)sg[SG_MOTION * n + h];
  b[B_RAD * S] = (R)sg[SG_RAD * n + h];
  v.awake[p] = u8[h];
  v.can_sleep[p] = u8[n + h];
  v.shape[p] = i32[h];
  if (off && v.offset) {
    R* o = const_cast<R*>(v.offset) + p;
    for (int k = 0; k < 12; ++k) o[k * S] = (R)off[12 * h + k];
  }
}

__global__ void k_download(BatchView<R> v, double* __restrict__ sg, uint8_t* __restrict__ u8, int* __restrict__ i32,
                           const int* __restrict__ h2p, int nb, double* __restrict__ off) {
  const int h = blockIdx.x * blockDim.x + threadIdx.x;
  if (h >= nb) return;
  const long long p = h2p[h];
  const long long S = v.nb_pad;
  const long long n = nb;
  const R* b = v.body + p;
  for (int k = 0; k < 3; ++k) {
    sg[SG_POS * n + 3 * h + k] = (double)b[(B_PX + k) * S];
    sg[SG_VEL * n + 3 * h + k] = (double)b[(B_VX + k) * S];
    sg[SG_ROT * n + 3 * h + k] = (double)b[(B_RX + k) * S];
    sg[SG_ACC * n + 3 * h + k] = (double)b[(B_AX + k) * S];
    sg[SG_HALF * n + 3 * h + k] = (double)b[(B_HX + k) * S];
    sg[SG_LFA * n + 3 * h + k] = (double)b[(B_LX + k) * S];
  }
  sg[SG_Q * n + 4 * h + 0] = (double)b[B_QW * S];
  sg[SG_Q * n + 4 * h + 1] = (double)b[B_QX * S];
  sg[SG_Q * n + 4 * h + 2] = (double)b[B_QY * S];
  sg[SG_Q * n + 4 * h + 3] = (double)b[B_QZ * S];
  for (int k = 0; k < 9; ++k) {
    sg[SG_IB * n + 9 * h + k] = (double)b[(B_IB0 + k) * S];
    sg[SG_IW * n + 9 * h + k] = (double)b[(B_IW0 + k) * S];
  }
  sg[SG_INVM * n + h] = (double)b[B_INVM * S];
  sg[SG_MOTION * n + h] = (double)b[B_MOTION * S];
  sg[SG_RAD * n + h] = (double)b[B_RAD * S];
  u8[h] = v.awake[p];
  u8[n + h] = v.can_sleep[p];
  i32[h] = v.shape[p];
  if (off && v.offset)
    for (int k = 0; k < 12; ++k) off[12 * h + k] = (double)v.offset[k * S + p];
}

__global__ void k_contacts_out(BatchView<R> v, long long start, int count, double* __restrict__ sg,
                               int* __restrict__ bodies) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  const long long S = v.nc_total;
  const R* c = v.contact + start + k;
  for (int f = 0; f < C_NROWS; ++f) sg[(long long)k * C_NROWS + f] = (double)c[f * S];
  bodies[k] = v.contact_bodies[start + k];
}

__global__ void k_contacts_in(BatchView<R> v, long long start, int count, const double* __restrict__ sg,
                              const int* __restrict__ bodies) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  const long long S = v.nc_total;
  R* c = v.contact + start + k;
  for (int f = 0; f < C_NROWS; ++f) c[f * S] = (R)sg[(long long)k * C_NROWS + f];
  v.contact_bodies[start + k] = bodies[k];
}

__global__ void k_set_rows(BatchView<R> v, int row, int nrows, const double* __restrict__ src) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long total = (long long)nrows * v.nb_pad;
  if (i >= total) return;
  v.body[(long long)row * v.nb_pad + i] = (R)src[i];
}

static size_t np_smem(int nbs) { return np_smem_bytes<R>(nbs); }
// warps per resolver CTA for G lanes per world (rs_wpc)
static int rs_wpc_of(int lanes) { return lanes == 32 ? rs_wpc<R, 32, false>() : 1; }
static size_t rs_smem(int nbs, int cs, int lanes, int mode) {
  (void)mode;  // the learned paths keep their scratch in global memory and registers
  return (size_t)rs_wpc_of(lanes) * (32 / lanes) * rs_slot_bytes<R, W>(nbs, cs);
}

// the resolver instantiation for G lanes per world, plain or with the
// learned paths (harvest, warm start)
static const void* resolve_fn_mode(int lanes, int mode) {
  const bool learn = mode != 0;
  switch (lanes) {
    case 4: return learn ? (const void*)k_resolve<R, W, 4, true> : (const void*)k_resolve<R, W, 4, false>;
    case 8: return learn ? (const void*)k_resolve<R, W, 8, true> : (const void*)k_resolve<R, W, 8, false>;
    case 16: return learn ? (const void*)k_resolve<R, W, 16, true> : (const void*)k_resolve<R, W, 16, false>;
    case 32: return learn ? (const void*)k_resolve<R, W, 32, true> : (const void*)k_resolve<R, W, 32, false>;
    default: return nullptr;
  }
}
static const void* resolve_fn(int lanes) { return resolve_fn_mode(lanes, 0); }

// Raise a kernel's dynamic shared-memory limit to `bytes` if it is lower.  The
// limit is per function and process-wide, so it is never lowered: another
// batch may launch the same kernel with a larger tile.
static cudaError_t raise_smem_limit(const void* f, size_t bytes) {
  cudaFuncAttributes a;
  cudaError_t e = cudaFuncGetAttributes(&a, f);
  if (e != cudaSuccess) return e;
  if ((size_t)a.maxDynamicSharedSizeBytes >= bytes) return cudaSuccess;
  return cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

// The narrowphase instantiation a batch runs: with the grid only when one of
// its worlds is large enough for it.
static bool uses_grid(const HostView& h) { return h.grid_min_bodies > 0 && h.max_bodies >= h.grid_min_bodies; }
static const void* narrowphase_fn(bool grid) {
  return grid ? (const void*)k_narrowphase<R, true> : (const void*)k_narrowphase<R, false>;
}

static cudaError_t prepare(size_t np, size_t rs, int lanes) {
  cudaError_t e = raise_smem_limit(narrowphase_fn(false), np);
  if (e != cudaSuccess) return e;
  if ((e = raise_smem_limit(narrowphase_fn(true), np)) != cudaSuccess) return e;
  for (int mode = 0; mode <= 1; ++mode) {
    const void* f = resolve_fn_mode(lanes, mode);
    if (!f) return cudaErrorInvalidValue;
    if ((e = raise_smem_limit(f, rs)) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

static cudaError_t integrate(const HostView& h, double dt, double bias, int threads, cudaStream_t s) {
  const long long nb = h.nb_pad;
  const int grid = (int)((nb + threads - 1) / threads);
  k_integrate<R, W><<<grid, threads, 0, s>>>(view_of(h), (R)dt, (R)bias);
  return cudaGetLastError();
}

static cudaError_t narrowphase(const HostView& h, int nbs, int threads, int grid, size_t smem, cudaStream_t s) {
  if (uses_grid(h))
    k_narrowphase<R, true><<<grid, threads, smem, s>>>(view_of(h), nbs);
  else
    k_narrowphase<R, false><<<grid, threads, smem, s>>>(view_of(h), nbs);
  return cudaGetLastError();
}

static cudaError_t resolve(const HostView& h, int nbs, int cs, int lanes, int grid, size_t smem, double dt,
                           cudaStream_t s) {
  const BatchView<R> v = view_of(h);
  const bool learn = h.mode != 0;
#define CZ_LAUNCH_RS(G)                                                                              \
  if (learn)                                                                                        \
    k_resolve<R, W, G, true><<<grid, 32 * rs_wpc<R, G, false>(), smem, s>>>(v, nbs, cs, (R)dt);      \
  else                                                                                              \
    k_resolve<R, W, G, false><<<grid, 32 * rs_wpc<R, G, false>(), smem, s>>>(v, nbs, cs, (R)dt);
  switch (lanes) {
    case 4: CZ_LAUNCH_RS(4) break;
    case 8: CZ_LAUNCH_RS(8) break;
    case 16: CZ_LAUNCH_RS(16) break;
    case 32: CZ_LAUNCH_RS(32) break;
    default: return cudaErrorInvalidValue;
  }
#undef CZ_LAUNCH_RS
  return cudaGetLastError();
}

static size_t frame_smem(int nbs, int cs) { return frame_slot_bytes<R, W>(nbs, cs); }

static cudaError_t frame_occupancy(int* blocks, size_t smem) {
  cudaError_t e = raise_smem_limit((const void*)k_resolve<R, W, 32, false, true>, smem);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, k_resolve<R, W, 32, false, true>, 32, smem);
}

static cudaError_t frame(const HostView& h, int nbs, int cs, int grid, size_t smem, double dt, double sleep_bias,
                         cudaStream_t s) {
  k_resolve<R, W, 32, false, true><<<grid, 32, smem, s>>>(view_of(h), nbs, cs, (R)dt, (R)sleep_bias);
  return cudaGetLastError();
}

static cudaError_t collide(const HostView& h, int world, const void* units, int nunits, int nbs, size_t smem,
                           cudaStream_t s) {
  const void* f = (const void*)k_collide<R>;
  cudaFuncAttributes a;
  cudaError_t e = cudaFuncGetAttributes(&a, f);
  if (e != cudaSuccess) return e;
  if ((size_t)a.maxDynamicSharedSizeBytes < smem &&
      (e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) != cudaSuccess)
    return e;
  k_collide<R><<<1, 256, smem, s>>>(view_of(h), world, static_cast<const int2*>(units), nunits, nbs);
  return cudaGetLastError();
}

static cudaError_t warm_features(const HostView& h, int nbs, int grid, double dt, cudaStream_t s) {
  const size_t smem = wf_smem_bytes<R, W>(nbs);
  {
    const void* f = (const void*)k_warm_features<R, W>;
    cudaFuncAttributes a;
    cudaError_t e = cudaFuncGetAttributes(&a, f);
    if (e != cudaSuccess) return e;
    if ((size_t)a.maxDynamicSharedSizeBytes < smem &&
        (e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) != cudaSuccess)
      return e;
  }
  k_warm_features<R, W><<<grid, 32 * kWfWarps, smem, s>>>(view_of(h), nbs, (R)dt);
  return cudaGetLastError();
}

static int warm_features_blocks(int nbs) {
  const size_t smem = wf_smem_bytes<R, W>(nbs);
  const void* f = (const void*)k_warm_features<R, W>;
  cudaFuncAttributes a;
  if (cudaFuncGetAttributes(&a, f) != cudaSuccess) return 1;
  if ((size_t)a.maxDynamicSharedSizeBytes < smem &&
      cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return 1;
  int blocks = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_warm_features<R, W>, 32 * kWfWarps, smem) !=
      cudaSuccess)
    return 1;
  return blocks > 0 ? blocks : 1;
}

static cudaError_t resolve_big(const HostView& h, int nbig, int lanes, double dt, cudaStream_t s) {
  if (nbig <= 0) return cudaSuccess;
  if (lanes == 16)
    k_resolve_big<R, W, 16><<<(nbig + 1) / 2, 32, 0, s>>>(view_of(h), (R)dt);
  else
    k_resolve_big<R, W, 32><<<nbig, 32, 0, s>>>(view_of(h), (R)dt);
  return cudaGetLastError();
}

static cudaError_t upload(const HostView& h, const double* sg, const uint8_t* u8, const int* i32, const int* h2p,
                          int nb, int has_iw, int has_lfa, const double* off, cudaStream_t s) {
  if (nb <= 0) return cudaSuccess;
  k_upload<<<(nb + 255) / 256, 256, 0, s>>>(view_of(h), sg, u8, i32, h2p, nb, has_iw, has_lfa, off);
  return cudaGetLastError();
}

static cudaError_t download(const HostView& h, double* sg, uint8_t* u8, int* i32, const int* h2p, int nb,
                            double* off, cudaStream_t s) {
  if (nb <= 0) return cudaSuccess;
  k_download<<<(nb + 255) / 256, 256, 0, s>>>(view_of(h), sg, u8, i32, h2p, nb, off);
  return cudaGetLastError();
}

static cudaError_t occupancy(int* npb, int np_threads, size_t nps, int* rsb, size_t rss, int lanes, int mode,
                             int grid) {
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(npb, narrowphase_fn(grid != 0), np_threads, nps);
  if (e != cudaSuccess) return e;
  const void* f = resolve_fn_mode(lanes, mode);  // the instantiation that runs (registers differ)
  if (!f) return cudaErrorInvalidValue;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(rsb, f, 32 * rs_wpc_of(lanes), rss);
}

static cudaError_t contacts_out(const HostView& h, long long start, int count, double* sg, int* bodies,
                                cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  k_contacts_out<<<(count + 127) / 128, 128, 0, s>>>(view_of(h), start, count, sg, bodies);
  return cudaGetLastError();
}

static cudaError_t contacts_in(const HostView& h, long long start, int count, const double* sg, const int* bodies,
                               cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  k_contacts_in<<<(count + 127) / 128, 128, 0, s>>>(view_of(h), start, count, sg, bodies);
  return cudaGetLastError();
}

static cudaError_t set_rows(const HostView& h, int row, int nrows, const double* src, cudaStream_t s) {
  const long long total = (long long)nrows * h.nb_pad;
  k_set_rows<<<(int)((total + 255) / 256), 256, 0, s>>>(view_of(h), row, nrows, src);
  return cudaGetLastError();
}

}  // namespace CZ_FORM_NS

const FormOps CZ_FORM_OBJ = {sizeof(CZ_R),
                             CZ_FORM_NS::np_smem,
                             CZ_FORM_NS::rs_smem,
                             CZ_FORM_NS::rs_wpc_of,
                             CZ_FORM_NS::prepare,
                             CZ_FORM_NS::integrate,
                             CZ_FORM_NS::narrowphase,
                             CZ_FORM_NS::collide,
                             CZ_FORM_NS::warm_features,
                             CZ_FORM_NS::warm_features_blocks,
                             CZ_FORM_NS::resolve_big,
                             CZ_FORM_NS::resolve,
                             CZ_FORM_NS::upload,
                             CZ_FORM_NS::download,
                             CZ_FORM_NS::occupancy,
                             CZ_FORM_NS::contacts_out,
                             CZ_FORM_NS::contacts_in,
                             CZ_FORM_NS::set_rows,
                             CZ_FORM_NS::resolve_fn,
                             CZ_FORM_NS::frame_smem,
                             CZ_FORM_NS::frame,
                             CZ_FORM_NS::frame_occupancy};

}  // namespace cz
