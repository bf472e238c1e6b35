// Device layout of a batch of independent worlds (structure of arrays).
//
// Bodies: one row per field, each row `nb_pad` long; world w owns rows
// [body_start[w], body_start[w] + body_count[w]) with body_start a multiple of
// 4, so that every world's slice of a row starts on a 16-byte (float) or
// 32-byte (double) boundary and can be staged with a bulk copy.
// Contacts: one row per field, each `nc_total` long; world w owns
// [contact_start[w], contact_start[w] + contact_cap[w]).
#pragma once
#include <cstdint>

#include "cz_mlp.cuh"

namespace cz {

// integer rows of the per-body warm-start scratch
enum WsInt : int {
  WS_DEG = 0,   // contacts touching the body
  WS_NBB,       // contacts between the body and other bodies
  WS_LOAD,      // sum of their positive desired delta velocities, fixed point 2^-16
  WS_FIRST,     // first and last index of the body's half-space contacts
  WS_LAST,
  WS_SCALE,     // warm-start scale (float bits)
  WS_NINT
};
constexpr float kLoadScale = 65536.f;

enum BodyRow : int {
  B_PX, B_PY, B_PZ,                                      // RigidBody.Position
  B_QW, B_QX, B_QY, B_QZ,                                // RigidBody.Orientation
  B_HX, B_HY, B_HZ, B_RAD,                               // CollisionCube.HalfSize / CollisionSphere.Radius
  B_VX, B_VY, B_VZ,                                      // Velocity
  B_RX, B_RY, B_RZ,                                      // Rotation (angular velocity)
  B_AX, B_AY, B_AZ,                                      // Acceleration
  B_LX, B_LY, B_LZ,                                      // lastFrameAccelleration
  B_IB0, B_IB1, B_IB2, B_IB3, B_IB4, B_IB5, B_IB6, B_IB7, B_IB8,  // InverseInertiaTensor (body)
  B_IW0, B_IW1, B_IW2, B_IW3, B_IW4, B_IW5, B_IW6, B_IW7, B_IW8,  // inverseInertiaTensorWorld
  B_INVM,                                                // inverseMass
  B_LINPOW, B_ANGPOW,                                    // pow(LinearDamping, dt), pow(AngularDamping, dt)
  B_MOTION,                                              // motion
  B_NROWS
};

// Narrowphase output (Contact fields set by the colliders).
enum ContactRow : int { C_PX, C_PY, C_PZ, C_NX, C_NY, C_NZ, C_PEN, C_FRIC, C_REST, C_NROWS };

// Resolver working set (Contact's private fields, contact.go:38-50).  The
// third basis column is never stored: calculateContactBasis (contact.go:
// 118-156) derives it from the normal and the second column by the same
// formulas.  The second column (W_TY*) is a function of the normal alone and
// is stored: recomputing it where the basis is used freed three rows of the
// resolver's shared-memory tile (10 instead of 9 CTAs per SM for the
// precision form) but cost more on the update path than the occupancy gained
// (measured: resolve +2.4 %).
enum WorkRow : int {
  W_PEN, W_DDV,
  W_NX, W_NY, W_NZ,
  W_R0X, W_R0Y, W_R0Z,
  W_R1X, W_R1Y, W_R1Z,
  W_CVX, W_CVY, W_CVZ,
  W_TYX, W_TYY, W_TYZ,
  W_J0, W_J1, W_J2,  // contact-frame impulse: predicted (warm start) or applied in total (harvest)
  W_NROWS
};
// reals per contact of the friction solve's matrices (K: 9, the response's
// first row: 3, padding: 4), contact-major, so the resolved contact's are one
// aligned 64- (float32) or 128-byte (float64) block
constexpr int K_ROW = 16;
// whether the form stores the basis tangent row
template <class R> __host__ __device__ constexpr bool stores_tangent() { return true; }
// rows the resolver keeps per contact in its shared-memory tile
template <class R> __host__ __device__ constexpr int w_rows_kept() { return stores_tangent<R>() ? W_J0 : W_TYX; }

// World status bits (also OR-ed into the batch status word).
enum : uint32_t {
  ST_NONFINITE = 1u,        // box-box test reached with no accepted axis (non-finite state)
  ST_FRICTIONLESS_NIL = 2u, // frictionless impulse on a single-body contact (the reference panics)
  ST_CAPACITY = 4u,         // more contacts than the world's capacity
  ST_TIMEOUT = 8u,          // a bounded wait gave up
  ST_BODY_LIMIT = 16u,      // world larger than the kernel's shared-memory tile
};

// packed body pair of a contact: low 16 bits body 0, high 16 bits body 1
// (0xFFFF = nil).  World-local indices, so a world holds at most 65535 bodies.
__host__ __device__ __forceinline__ int pack_bodies(int b0, int b1) {
  return (int)(((unsigned)(b0 & 0xFFFF)) | ((unsigned)(b1 & 0xFFFF) << 16));
}
__host__ __device__ __forceinline__ int body0_of(int p) {
  int b = p & 0xFFFF;
  return b == 0xFFFF ? -1 : b;
}
__host__ __device__ __forceinline__ int body1_of(int p) {
  int b = (int)(((unsigned)p) >> 16);
  return b == 0xFFFF ? -1 : b;
}

template <class R> struct BatchView {
  R* body;              // [B_NROWS][nb_pad]
  uint8_t* awake;       // [nb_pad]
  uint8_t* can_sleep;   // [nb_pad]
  int32_t* shape;       // [nb_pad] 0 sphere, 1 cube, -1 padding
  const R* offset;      // [12][nb_pad] collider Offset (column-major 3x4), null = identity for every body
  long long nb_pad;
  int num_worlds;
  int max_bodies;       // largest world
  const int* body_start;
  const int* body_count;
  const long long* contact_start;
  const int* contact_cap;
  int* contact_count;   // [num_worlds] narrowphase output
  uint32_t* world_status;
  int* pos_iters;
  int* vel_iters;
  R* contact;           // [C_NROWS][nc_total]
  int* contact_bodies;  // [nc_total]
  R* work;              // [W_NROWS][nc_total]
  R* kmat;              // [nc_total][16] reals per contact: K of its friction solve (9, inverted in the
                        // island type), the friction response's first row (3), padding (4)
  int* work_bodies;     // [nc_total]
  long long nc_total;
  const int* order;     // narrowphase queue: worlds in decreasing body count
  const int* order_rs;  // resolver queue: worlds in decreasing iterations of the previous frame
  unsigned* queue;      // [0] narrowphase, [1] resolver, [2..3] spare
  uint32_t* status;     // batch status word
  unsigned long long* counters;  // [0] contacts generated, [1] adjustPositions iterations,
                                 // [2] adjustVelocities iterations, [3] contacts resolved,
                                 // [4] warm-started worlds re-solved plainly, [5] warm-started worlds
  R plane_nx, plane_ny, plane_nz, plane_offset;
  int iter_mult;        // ResolveContacts(len(contacts) * iter_mult)
  int max_iterations;   // >= 0 overrides len(contacts) * iter_mult
  int contact_writeback; // copy the resolved contacts back to the contact rows
  int uniform_material;  // every contact has the colliders' friction 0.9 / restitution 0.1
  int mode;              // resolver: 0 plain, 1 harvest, 2 learned warm start
  MlpDev mlp;            // warm-start network (mode 2)
  float* hv_features;    // harvest output [hv_cap][18]
  float* hv_labels;      // harvest output [hv_cap][3]
  unsigned long long* hv_count;
  long long hv_cap;
  // per-body scratch of the warm start and the harvest (modes 1, 2), indexed
  // like the body rows (row stride nb_pad)
  R* ws_rows;            // [13]: saved velocity 0-2, rotation 3-5, motion 6; warm-start change 7-12
  int* ws_int;           // [WS_NINT]
  uint8_t* ws_u8;        // [2]: awake flags at the start of adjustVelocities, at prepareContacts
  uint8_t* ws_world;     // [num_worlds]: the world's last velocity solve used more than max_it >> warm_shift
  float* ws_feat;        // [nc_total][18] harvest features (k_warm_features, mode 1)
  int warm_shift;        // warm-start a world when its last solve used <= max_it >> warm_shift
  // worlds above the shared-memory slot of k_resolve, resolved by k_resolve_big
  const int* big_list;   // [big_count] world ids
  int big_count;
  void* big_bw;          // [7][nb_pad] positions / orientations in the island type
  R* big_br;             // [20][nb_pad] velocity, rotation, lfa, iitWorld, inverse mass, motion
  uint8_t* big_aw;       // [nb_pad] awake flags
  int* big_off;          // [nb_pad] start of each body's contact list in its world's segment
  int* big_cnt;          // [nb_pad] end of each body's contact list
  int* big_adj;          // [2 * nc_total] contact lists, a world's segment at 2 * contact_start
  // the narrowphase's bounded wait on its staging copies: polls before it
  // gives up, and extra bytes expected beyond those copied (0; a test raises
  // it so that the wait runs out with every real copy landed)
  int wait_limit;
  int wait_extra_tx;
  int grid_min_bodies;  // narrowphase: worlds of at least this many bodies use the grid (0: none)
};

}  // namespace cz
