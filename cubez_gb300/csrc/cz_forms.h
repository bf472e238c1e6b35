// Host-side interface between the C ABI (cz_api.cu) and the per-form kernel
// instantiations (cz_fp64.cu, cz_fp32.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

#include "../../include/cubez_gpu.h"
#include "cz_layout.cuh"
#include "cz_mlp.cuh"

namespace cz {

// Type-erased device view; each form turns it into BatchView<R>.
struct HostView {
  void* body;
  uint8_t* awake;
  uint8_t* can_sleep;
  int32_t* shape;
  const void* offset;  // [12][nb_pad] collider Offset rows, or null (identity)
  long long nb_pad;
  int num_worlds;
  int max_bodies;
  const int* body_start;
  const int* body_count;
  const long long* contact_start;
  const int* contact_cap;
  int* contact_count;
  uint32_t* world_status;
  int* pos_iters;
  int* vel_iters;
  void* contact;
  int* contact_bodies;
  void* work;
  int* work_bodies;
  void* kmat;  // [nc_total][16] reals
  long long nc_total;
  const int* order;
  const int* order_rs;
  unsigned* queue;
  uint32_t* status;
  unsigned long long* counters;
  double plane[4];
  int iter_mult;
  int max_iterations;
  int contact_writeback;
  int uniform_material;
  int mode;
  MlpDev mlp;
  float* hv_features;
  float* hv_labels;
  unsigned long long* hv_count;
  long long hv_cap;
  void* ws_rows;
  int* ws_int;
  uint8_t* ws_u8;
  uint8_t* ws_world;
  float* ws_feat;
  int warm_shift;
  const int* big_list;
  int big_count;
  void* big_bw;
  void* big_br;
  uint8_t* big_aw;
  int* big_off;
  int* big_cnt;
  int* big_adj;
  int wait_limit;
  int wait_extra_tx;
  int grid_min_bodies;
};

// Staging layout of host body data on the device (doubles, field blocks of n):
enum StageBlock : int {
  SG_POS = 0, SG_Q = 3, SG_VEL = 7, SG_ROT = 10, SG_ACC = 13, SG_IB = 16, SG_INVM = 25, SG_MOTION = 26,
  SG_HALF = 27, SG_RAD = 30, SG_IW = 31, SG_LFA = 40, SG_NDOUBLES = 43
};

struct FormOps {
  size_t real_size;
  size_t (*np_smem)(int nbs);
  size_t (*rs_smem)(int nbs, int cs, int lanes, int mode);  // per CTA (rs_wpc warps, 32 / lanes worlds each)
  int (*rs_wpc)(int lanes);                                   // warps per resolver CTA
  cudaError_t (*prepare)(size_t np_smem, size_t rs_smem, int lanes);  // function attributes
  cudaError_t (*integrate)(const HostView& v, double dt, double sleep_bias, int threads, cudaStream_t s);
  cudaError_t (*narrowphase)(const HostView& v, int nbs, int threads, int grid, size_t smem, cudaStream_t s);
  // the narrowphase over a list of units (int2: body, other body or -1 = half-space) of one world
  cudaError_t (*collide)(const HostView& v, int world, const void* units, int nunits, int nbs, size_t smem,
                         cudaStream_t s);
  // the learned paths' features / predictions ahead of the resolver (k_warm_features)
  cudaError_t (*warm_features)(const HostView& v, int nbs, int grid, double dt, cudaStream_t s);
  int (*warm_features_blocks)(int nbs);  // resident CTAs per SM
  // worlds above the shared-memory slot; `lanes` per world: 32, or 16 (two worlds per warp)
  cudaError_t (*resolve_big)(const HostView& v, int nbig, int lanes, double dt, cudaStream_t s);
  cudaError_t (*resolve)(const HostView& v, int nbs, int cs, int lanes, int grid, size_t smem, double dt,
                         cudaStream_t s);
  // `off` ([n][12] doubles, the collider Offsets) may be null; the upload
  // writes the Offset rows only when both it and v.offset are set
  cudaError_t (*upload)(const HostView& v, const double* stage, const uint8_t* u8, const int* i32, const int* h2p,
                        int nb, int has_iw, int has_lfa, const double* off, cudaStream_t s);
  cudaError_t (*download)(const HostView& v, double* stage, uint8_t* u8, int* i32, const int* h2p, int nb,
                          double* off, cudaStream_t s);
  cudaError_t (*occupancy)(int* np_blocks, int np_threads, size_t np_smem, int* rs_blocks, size_t rs_smem,
                           int lanes, int mode, int grid);
  // contacts: device rows <-> AoS doubles staging (10 doubles + 2 ints per contact)
  cudaError_t (*contacts_out)(const HostView& v, long long start, int count, double* stage, int* bodies,
                              cudaStream_t s);
  cudaError_t (*contacts_in)(const HostView& v, long long start, int count, const double* stage, const int* bodies,
                             cudaStream_t s);
  cudaError_t (*set_rows)(const HostView& v, int row, int nrows, const double* src, cudaStream_t s);
  const void* (*resolve_kernel)(int lanes);  // the resolver instantiation for `lanes` lanes per world
  // the fused frame (k_frame): integrate, narrowphase and resolver per world, one warp each
  size_t (*frame_smem)(int nbs, int cs);
  cudaError_t (*frame)(const HostView& v, int nbs, int cs, int grid, size_t smem, double dt, double sleep_bias,
                       cudaStream_t s);
  cudaError_t (*frame_occupancy)(int* blocks, size_t smem);  // also raises its shared-memory limit
};

extern const FormOps kFormFP64;
extern const FormOps kFormFP32;

// Warm-start network: packed device copy of a float32 parameter blob.
size_t mlp_packed_bytes();
MlpDev mlp_view(unsigned char* packed);
cudaError_t mlp_pack(const float* dev_blob, unsigned char* dev_packed, cudaStream_t s);

// Records the message cz_last_error() returns; returns status.
int set_error(int status, const char* what, cudaError_t e);

// Device status bits (ST_*) -> the cz_status a call returns, most severe first.
inline int status_from_bits(uint32_t bits) {
  if (bits & ST_TIMEOUT) return CZ_ERR_TIMEOUT;
  if (bits & ST_NONFINITE) return CZ_ERR_NONFINITE;
  if (bits & ST_CAPACITY) return CZ_ERR_CAPACITY;
  if (bits & ST_BODY_LIMIT) return CZ_ERR_BODY_LIMIT;
  if (bits & ST_FRICTIONLESS_NIL) return CZ_ERR_FRICTIONLESS;
  return CZ_OK;
}

}  // namespace cz
