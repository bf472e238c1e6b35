/*
 * cubez_gpu.h - C ABI of the GB300 (sm_103a) rigid-body step.
 *
 * This is the boundary a cgo binding of cubez binds: plain pointers, sizes and
 * int status codes, no CUDA or C++ types.  Bodies and contacts live on the
 * device in structure-of-arrays form inside a batch handle; the host passes
 * and receives array-of-structures doubles laid out like cubez's value types
 * (m.Vector3 = 3 doubles, m.Quat = (w,x,y,z), m.Matrix3 = 9 doubles
 * column-major).  Worlds in a batch are independent: contacts of one world
 * never touch bodies of another (contact.go:204-207 recommends exactly this
 * split for ResolveContacts).
 *
 * Reference interfaces replaced (tbogdala/cubez):
 *   RigidBody fields/methods ........ rigidbody.go:23-272
 *   RigidBody.Integrate ............. rigidbody.go:213-259  -> cz_integrate / cz_step
 *   RigidBody.CalculateDerivedData .. rigidbody.go:268-272  -> cz_upload_bodies
 *   Collider.CheckAgainst{HalfSpace,Sphere,Cube}, CheckForCollisions
 *                                     colliders.go:15-23, 178-710, 720-747
 *                                                           -> cz_narrowphase / cz_step,
 *                                                              cz_collide (a caller's order)
 *   CollisionCube/Sphere.Offset ..... colliders.go:44,62    -> cz_bodies.collider_offset
 *   the per-frame loop of examples/cubedrop.go:29-75      -> cz_step
 *   ResolveContacts ................. contact.go:208-222    -> cz_resolve / cz_resolve_contacts
 *   Contact (exported fields) ....... contact.go:17-36      -> cz_contact
 *
 * Every function returns a cz_status.  Nothing traps on the device: conditions
 * under which the Go reference panics (non-finite box transforms, a
 * frictionless single-body contact) are reported as status bits.
 */
#ifndef CUBEZ_GPU_H
#define CUBEZ_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum cz_status {
  CZ_OK = 0,
  CZ_ERR_BAD_ARG = 1,      /* invalid handle, size or pointer */
  CZ_ERR_CUDA = 2,         /* a CUDA call failed; see cz_last_error() */
  CZ_ERR_NO_DEVICE = 3,    /* no CUDA device */
  CZ_ERR_NONFINITE = 4,    /* non-finite box transform met in the box-box test (the reference panics) */
  CZ_ERR_CAPACITY = 5,     /* a world produced more contacts than its capacity */
  CZ_ERR_TIMEOUT = 6,      /* a bounded device wait gave up */
  CZ_ERR_FRICTIONLESS = 7, /* frictionless impulse on a single-body contact (contact.go:512 dereferences nil) */
  CZ_ERR_BODY_LIMIT = 8,   /* a world has more bodies than the kernels' tile; raise max_bodies */
} cz_status;

typedef enum cz_form {
  CZ_FORM_FP64 = 0, /* plain form: every operation in float64, as the reference */
  CZ_FORM_FP32 = 1, /* precision form: float32, with float64 for quaternion renormalisation,
                       the positions/orientations accumulated across adjustPositions and the
                       contact-frame 3x3 inversion of the friction impulse */
} cz_form;

typedef enum cz_shape { CZ_SHAPE_SPHERE = 0, CZ_SHAPE_CUBE = 1 } cz_shape;

typedef struct cz_batch cz_batch; /* opaque */

/* Batch description (cz_batch_create). */
typedef struct cz_batch_desc {
  int32_t form;                 /* cz_form */
  int32_t num_worlds;
  const int32_t* body_counts;   /* [num_worlds] bodies per world (world-local index < 65535) */
  int32_t contact_capacity;     /* per world; 0 = worst case 8n + n(n-1) capped at max(64n, 4608) */
  double plane[4];              /* the ground CollisionPlane: normal xyz, offset (colliders.go:29-35) */
  int32_t iteration_multiplier; /* ResolveContacts(len(contacts) * k, ...) as examples/cubedrop.go:73; 0 = 4 */
  int32_t max_iterations;       /* > 0: a fixed maxIterations instead of len(contacts) * k */
  int32_t device;               /* CUDA device ordinal */
} cz_batch_desc;

/* Host array-of-structures body data, world-major (bodies of world 0 first).
 * Fields mirror RigidBody (rigidbody.go:23-101) and the collider shapes
 * (colliders.go:37-71).  On download, NULL pointers are skipped. */
typedef struct cz_bodies {
  double* position;                /* [n][3]  RigidBody.Position */
  double* orientation;             /* [n][4]  RigidBody.Orientation (w,x,y,z) */
  double* velocity;                /* [n][3]  RigidBody.Velocity */
  double* rotation;                /* [n][3]  RigidBody.Rotation (angular velocity) */
  double* acceleration;            /* [n][3]  RigidBody.Acceleration */
  double* inverse_inertia;         /* [n][9]  RigidBody.InverseInertiaTensor (body space) */
  double* inverse_mass;            /* [n]     1/mass (SetMass) or 0 (SetInfiniteMass) */
  double* linear_damping;          /* [n]     RigidBody.LinearDamping */
  double* angular_damping;         /* [n]     RigidBody.AngularDamping */
  double* motion;                  /* [n]     sleep motion average */
  uint8_t* is_awake;               /* [n]     RigidBody.IsAwake */
  uint8_t* can_sleep;              /* [n]     RigidBody.CanSleep */
  int32_t* shape;                  /* [n]     cz_shape */
  double* half_size;               /* [n][3]  CollisionCube.HalfSize */
  double* radius;                  /* [n]     CollisionSphere.Radius */
  double* inverse_inertia_world;   /* [n][9]  derived; upload: NULL = CalculateDerivedData */
  double* last_frame_acceleration; /* [n][3]  derived; upload: NULL = zero */
  double* collider_offset;         /* [n][12] CollisionCube/CollisionSphere.Offset (colliders.go:44,62), a
                                    *          column-major Matrix3x4; upload: NULL = the identity that
                                    *          NewCollisionCube/Sphere set (colliders.go:138,267) */
} cz_bodies;

/* One contact, the exported fields of Contact (contact.go:17-36).  Bodies are
 * world-local indices, -1 for nil. */
typedef struct cz_contact {
  int32_t body[2];
  double friction;
  double restitution;
  double point[3];
  double normal[3];
  double penetration;
} cz_contact;

/* Create / destroy a batch of worlds on one GPU.  All device buffers of the
 * batch are allocated here. */
int cz_batch_create(const cz_batch_desc* desc, cz_batch** out);
int cz_batch_destroy(cz_batch* batch);

/* Copy bodies in (and run RigidBody.CalculateDerivedData + the colliders'
 * CalculateDerivedData, rigidbody.go:268-272, colliders.go:173-176/302-304),
 * or copy the current state out.  Blocking. */
int cz_upload_bodies(cz_batch* batch, const cz_bodies* in);
int cz_download_bodies(cz_batch* batch, cz_bodies* out);

/* One frame in the order of examples/cubedrop.go:69-75, nsteps times:
 * Integrate + collider derived data for every body, the ordered all-pairs
 * narrowphase (plane first, then every other body), and ResolveContacts per
 * world.  The sequence is captured once as a CUDA graph per (nsteps, dt) and
 * replayed.  Blocking; returns the first error status seen. */
int cz_step(cz_batch* batch, int32_t nsteps, double dt);

/* Compute the damping factors for dt and capture the rollout graphs of
 * cz_step / cz_step_timed for nsteps without running them. */
int cz_prepare_rollout(cz_batch* batch, int32_t nsteps, double dt);

/* The three phases separately (blocking).  The narrowphase derives each
 * collider's transform from its body's current position and orientation:
 * what the reference's collider holds right after Integrate, the frame loop's
 * order.  (After a resolve with no Integrate in between, the reference would
 * still test the transforms of the last Integrate.) */
int cz_integrate(cz_batch* batch, double dt);                   /* rigidbody.go:213-259 */
int cz_narrowphase(cz_batch* batch);                            /* examples/cubedrop.go:41-67 */
int cz_resolve(cz_batch* batch, double dt);                     /* contact.go:208-222 */

/* Contacts produced by the last narrowphase, in the reference's order. */
int cz_contact_counts(cz_batch* batch, int32_t* counts /* [num_worlds] */);
int cz_download_contacts(cz_batch* batch, int32_t world, cz_contact* out, int32_t capacity, int32_t* count);

/* Per-world statistics of the last resolve: adjustPositions and
 * adjustVelocities iterations used, and status bits. */
int cz_world_stats(cz_batch* batch, int32_t* pos_iterations, int32_t* vel_iterations, uint32_t* status);

/* ResolveContacts(maxIterations, contacts, duration) for one caller-supplied
 * contact list (contact.go:208-222): bodies and contacts are read, resolved on
 * the device and written back in place.  A contact with body[0] == -1 is
 * swapped as calculateInternals does (contact.go:61-65).  Uses the batch's
 * form; the batch must have been created with one world holding nbodies
 * bodies and capacity >= ncontacts. */
int cz_resolve_contacts(cz_batch* batch, int32_t max_iterations, cz_contact* contacts, int32_t ncontacts,
                        double duration, cz_bodies* bodies);

/* Save the whole device body state / put it back (device-to-device copies;
 * the rollout benchmark restarts every timed rollout from the same state). */
int cz_snapshot(cz_batch* batch);
int cz_restore(cz_batch* batch);

/* cz_step with CUDA events recorded on the batch stream around every phase
 * inside the captured rollout: total_ms = whole rollout, phase_ms[0..2] =
 * integrate, narrowphase, resolve summed over the steps. */
int cz_step_timed(cz_batch* batch, int32_t nsteps, double dt, double* total_ms, double* phase_ms);

/* Running totals since creation or the last reset: [0] contacts generated,
 * [1] adjustPositions iterations, [2] adjustVelocities iterations (with the
 * warm start: both solves of a re-solved world), [3] contacts resolved,
 * [4] warm-started worlds re-solved by the plain path, [5] warm-started
 * worlds, [6] sum over warm-started bodies of the scale their line search
 * picked, in millionths, [7] warm-started bodies.  reset != 0 zeroes them
 * after reading. */
int cz_counters(cz_batch* batch, int64_t* out /* [8] */, int32_t reset);

/* Sizes: [0] bodies, [1] padded bodies, [2] contact slots, [3] bytes per real,
 * [4] SMs, [5] narrowphase CTAs, [6] resolver CTAs, [7] narrowphase shared
 * bytes, [8] resolver shared bytes. */
int cz_batch_info(cz_batch* batch, int64_t* info /* [9] */);

/* ResolveContacts for one world without allocating any memory.  This entry
 * point has no counterpart in the reference; it serves callers that cannot
 * call cudaMalloc (a frame loop that must not allocate once it runs, or a host
 * that only hands the library pointers into device memory it already owns).
 * Same semantics as cz_resolve_contacts, but every array is in DEVICE memory
 * owned by the caller: `contacts` is a device array of cz_contact, and
 * `bodies` is a host struct whose pointers point to device arrays (position,
 * orientation, velocity, rotation, inverse_inertia, inverse_mass, is_awake
 * are required; inverse_inertia_world, last_frame_acceleration and motion are
 * optional as in cz_upload_bodies).  Results are written back into those
 * arrays, and the call synchronises `stream` (a cudaStream_t; NULL = the
 * legacy default stream) before it returns.
 *   Scratch: a statically reserved device array of about 2.8 MB that every
 *   GPU loading the library holds until exit; hence the limits of at most 64
 *   bodies and 8192 contacts (CZ_ERR_BAD_ARG beyond).  The first call on a
 *   device also looks up the array's device address.  All calls share the
 *   array, so calls whose GPU work overlaps race on it: serialise them. */
int cz_resolve_contacts_static(int32_t form, int32_t max_iterations, cz_contact* contacts, int32_t ncontacts,
                               double duration, const cz_bodies* bodies, int32_t nbodies, void* stream);

/* The narrowphase for a caller's list of tests in one world, in the list's
 * order: units[2u], units[2u+1] = (i, j) runs CheckForCollisions(collider i,
 * collider j) (colliders.go:720-747), and (i, -1) runs collider i's
 * CheckAgainstHalfSpace against the plane (colliders.go:180-207, 308-366).
 * Indices are world-local.  `plane` = {nx, ny, nz, offset}, or NULL for the
 * batch's plane.  The world's contact list is replaced by the contacts of the
 * tests in order (read them with cz_contact_counts / cz_download_contacts);
 * the bodies are the uploaded ones.  This is what a caller with its own pair
 * list (a broadphase, or per-pair calls of the Go API) binds. */
int cz_collide(cz_batch* batch, int32_t world, const double* plane, const int32_t* units, int32_t nunits);

/* ---- Learned warm start of adjustVelocities (no counterpart in the
 * reference; the precision form's third variant).  A parameter blob is
 * CZ_MLP_BLOB floats: W1[64][18] b1[64] W2[64][64] b2[64] W3[64][64] b3[64]
 * W4[3][64] b4[3] (trainable), then the feature mean[18], 1/std[18] and the
 * output scale[3].  The network maps 18 contact features (in the contact
 * basis: the contacts between body 0 and other bodies, a half-space flag,
 * contact velocity, penetration, desired delta velocity, the 6 entries of
 * the symmetric velocity-per-impulse matrix, the impulse resolving the
 * contact alone, and per body the contacts touching it and their summed
 * positive desired delta velocities) to the contact-frame impulse the plain
 * resolver applies in total.  Bodies whose contacts are all with the
 * half-space are warm-started: their predicted impulses are projected onto
 * the friction cone, scaled by a per-body line search so that no contact is
 * pushed past its resolved velocity, and applied before adjustVelocities,
 * which then runs to the reference's epsilons; a world that uses all its
 * iterations is re-solved by the plain path. */
#define CZ_MLP_IN 18
#define CZ_MLP_OUT 3
#define CZ_MLP_NPARAM 9539
#define CZ_MLP_BLOB 9578

/* Enable the warm start with a parameter blob (host floats), or disable it
 * (blob = NULL).  Affects cz_step / cz_step_timed / cz_resolve. */
int cz_set_warm_start(cz_batch* batch, const float* blob);

/* Run nsteps frames with the plain resolver and, every `every` frames, write
 * each contact's features and the contact-frame impulse adjustVelocities
 * applied to it in total (the training labels) to host arrays
 * features[capacity][18], labels[capacity][3]; *count = rows written. */
int cz_harvest(cz_batch* batch, int32_t nsteps, double dt, int32_t every, float* features, float* labels,
               int64_t capacity, int64_t* count);

/* Trainer of the warm-start network: hand-written BF16 tensor-core forward,
 * backward and weight-gradient kernels with FP32 accumulation, Adam on FP32
 * master weights, mean squared error on normalised outputs. */
typedef struct cz_mlp cz_mlp;
int cz_mlp_create(int32_t device, uint64_t seed, cz_mlp** out);
int cz_mlp_destroy(cz_mlp* mlp);
int cz_mlp_get_params(cz_mlp* mlp, float* blob /* [CZ_MLP_BLOB] */);
int cz_mlp_set_params(cz_mlp* mlp, const float* blob);
/* Training data (host arrays, copied); set_normalization != 0 also sets the
 * feature mean / std and output scale from the data. */
int cz_mlp_set_data(cz_mlp* mlp, const float* features, const float* labels, int64_t n, int32_t set_normalization);
int cz_mlp_train(cz_mlp* mlp, int32_t epochs, int32_t batch, float lr, uint64_t seed, float* epoch_loss);
/* Mean loss and gradient over the first n data rows, without an update. */
int cz_mlp_loss_and_grad(cz_mlp* mlp, int64_t n, float* loss, float* grad /* [CZ_MLP_NPARAM] */);
int cz_mlp_predict(cz_mlp* mlp, const float* features, int64_t n, float* impulses /* [n][3] */);

/* Tuning knobs picked by the autotuner (0 keeps the current value). */
typedef struct cz_tuning {
  int32_t narrowphase_threads; /* CTA size of the narrowphase */
  int32_t resolver_contacts;   /* contacts kept in shared memory per world */
  int32_t resolver_ctas_per_sm;/* resident resolver CTAs per SM (a CTA is 4 independent warps in the
                                  float32 form with 32 lanes per world, else 1 warp) */
  int32_t integrate_threads;
  int32_t resolver_lanes;      /* lanes per world in the resolver: 4, 8, 16 or 32 */
  int32_t warm_start_budget_shift; /* learned warm start: a world is warm-started when its last
                                      solve used at most max_iterations >> shift iterations
                                      (1 to 8; default 2) */
  int32_t large_world_lanes;   /* lanes per world of more than 64 bodies: 32 (the default) or
                                  16 (two worlds per warp in lockstep) */
  int32_t broadphase_min_bodies; /* the narrowphase bins the bodies of worlds of at least this many
                                    bodies in a uniform grid and tests only pairs of neighbouring
                                    cells (default 128; -1 = never).  The grid drops only pairs the
                                    float32 culls reject and keeps the reference's pair order, so
                                    contact lists are the same bit for bit (an ordered all-pairs
                                    loop, examples/cubedrop.go:41-67, that the reference marks as
                                    O(n^2) at examples/cubedrop.go:54 and README.md:98-99) */
  int32_t fused_frame;         /* 1: cz_step runs each frame as one launch in which a warp integrates,
                                  tests and resolves one world after another from a device queue;
                                  -1: three launches per frame (the default).  Taken where the batch
                                  runs one world per warp (resolver_lanes 32), the plain resolver
                                  and no world above 64 bodies; same results either way */
} cz_tuning;
int cz_set_tuning(cz_batch* batch, const cz_tuning* tuning);
int cz_get_tuning(cz_batch* batch, cz_tuning* tuning);

/* Test hook for the failure path of the narrowphase's one device wait (no
 * counterpart in the reference).  The narrowphase stages each world's bodies
 * with bulk copies and waits, bounded, for their bytes; with extra_bytes > 0
 * it expects that many bytes more than it copies, so the wait runs out after
 * wait_limit polls (0 = the default limit) with every real copy landed, and
 * the call reports CZ_ERR_TIMEOUT.  cz_set_wait_test(batch, 0, 0) restores
 * the normal wait; the batch then steps on as before. */
int cz_set_wait_test(cz_batch* batch, int32_t extra_bytes, int32_t wait_limit);

/* Error reporting. */
const char* cz_status_string(int status);
const char* cz_last_error(void);

/* Library information: number of kernel launches issued so far by this
 * process (all batches), for launch accounting. */
int64_t cz_kernel_launches(void);

#ifdef __cplusplus
}
#endif

#endif /* CUBEZ_GPU_H */
