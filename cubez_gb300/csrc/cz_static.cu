// Allocation-free ResolveContacts for one world: cz_resolve_contacts_static.
//
// Some callers of this library cannot call cudaMalloc.  A game or simulation
// frame loop may be forbidden to allocate once it runs (an allocation can
// block on the device and costs an unbounded time); a host may only hand the
// library pointers into device memory it already owns (a Go program passing
// buffers from its own pool through cgo, an engine with one fixed arena).
// For them this entry point resolves one world's contact list with no
// allocation at all: its scratch is the file-scope array below, reserved with
// the library's code, of a fixed size stated by kStaticMaxBodies and
// kStaticMaxContacts (about 2.8 MB).  Every GPU that loads the library holds
// that array until the process exits.
//
// The array holds the world in the resolver's own layout: body rows, contact
// rows, the resolver's working rows and a few counters.  All calls share it
// and it keeps the last call's contents (each call first resets what must
// start at zero), so calls whose GPU work overlaps -- on two streams, or from
// two host threads -- race on it; the caller must serialise them.
//
// The host code names the array only through cudaGetSymbolAddress: the
// array's host-side name is a stand-in, not a device address.  The address is
// looked up once per device, with that device current, by the first call on
// that device (the set-up); that first call should therefore come before any
// stream capture.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <mutex>

#include "../../include/cubez_gpu.h"
#include "cz_forms.h"
#include "cz_layout.cuh"
#include "cz_math.cuh"

namespace {

constexpr int kStaticMaxBodies = 64;
constexpr int kStaticMaxContacts = 8192;
constexpr int kStaticContactTile = 128;  // contacts kept in shared memory; the rest use the working rows below

constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }
// section offsets in bytes, sized for float64 (float32 uses the same offsets)
constexpr size_t kOffBody = 0;
constexpr size_t kOffAwake = align256(kOffBody + sizeof(double) * cz::B_NROWS * kStaticMaxBodies);
constexpr size_t kOffContact = align256(kOffAwake + kStaticMaxBodies);
constexpr size_t kOffCBodies = align256(kOffContact + sizeof(double) * cz::C_NROWS * kStaticMaxContacts);
constexpr size_t kOffWork = align256(kOffCBodies + sizeof(int) * kStaticMaxContacts);
constexpr size_t kOffWBodies = align256(kOffWork + sizeof(double) * cz::W_NROWS * kStaticMaxContacts);
constexpr size_t kOffKmat = align256(kOffWBodies + sizeof(int) * kStaticMaxContacts);
constexpr size_t kOffMeta = align256(kOffKmat + sizeof(double) * cz::K_ROW * kStaticMaxContacts);
constexpr size_t kScratchBytes = align256(kOffMeta + 256);

static __device__ __align__(256) unsigned char g_static_scratch[kScratchBytes];

// counters and per-world metadata of the single world, inside the scratch
struct Meta {
  long long contact_start;
  unsigned long long counters[8];
  int body_start, body_count, contact_cap, contact_count;
  uint32_t world_status, status;
  int pos_iters, vel_iters, order, order_rs;
  unsigned queue[4];
};
static_assert(sizeof(Meta) <= 256, "metadata section");

// Caller's arrays -> scratch rows (RigidBody.CalculateDerivedData where no
// world inertia is given, as cz_upload_bodies does); contacts -> contact rows,
// with their body indices checked.
template <class R, class W>
__global__ void k_static_in(unsigned char* scratch, cz_bodies in, const cz_contact* __restrict__ cs, int n, int nc) {
  R* body = reinterpret_cast<R*>(scratch + kOffBody);
  uint8_t* awake = scratch + kOffAwake;
  R* crow = reinterpret_cast<R*>(scratch + kOffContact);
  int* cb = reinterpret_cast<int*>(scratch + kOffCBodies);
  Meta* m = reinterpret_cast<Meta*>(scratch + kOffMeta);
  const long long S = kStaticMaxBodies, CS = kStaticMaxContacts;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int nthreads = gridDim.x * blockDim.x;
  for (int i = tid; i < n; i += nthreads) {
    R* b = body + i;
    for (int k = 0; k < 3; ++k) {
      b[(cz::B_PX + k) * S] = (R)in.position[3 * i + k];
      b[(cz::B_VX + k) * S] = (R)in.velocity[3 * i + k];
      b[(cz::B_RX + k) * S] = (R)in.rotation[3 * i + k];
      b[(cz::B_LX + k) * S] = in.last_frame_acceleration ? (R)in.last_frame_acceleration[3 * i + k] : (R)0;
    }
    cz::q4<R> q{(R)in.orientation[4 * i], (R)in.orientation[4 * i + 1], (R)in.orientation[4 * i + 2],
                (R)in.orientation[4 * i + 3]};
    cz::m3<R> ib, iw;
    for (int k = 0; k < 9; ++k) ib.m[k] = (R)in.inverse_inertia[9 * i + k];
    if (in.inverse_inertia_world) {
      for (int k = 0; k < 9; ++k) iw.m[k] = (R)in.inverse_inertia_world[9 * i + k];
    } else {
      cz::q4<W> qw = cz::cvtq<W>(q);
      cz::qnormalize_island<R, W>(qw);
      q = cz::cvtq<R>(qw);
      R rm[9];
      cz::rotation_of(q, rm);
      iw = cz::world_inertia(rm, ib);
    }
    b[cz::B_QW * S] = q.w; b[cz::B_QX * S] = q.x; b[cz::B_QY * S] = q.y; b[cz::B_QZ * S] = q.z;
    for (int k = 0; k < 9; ++k) {
      b[(cz::B_IB0 + k) * S] = ib.m[k];
      b[(cz::B_IW0 + k) * S] = iw.m[k];
    }
    b[cz::B_INVM * S] = (R)in.inverse_mass[i];
    b[cz::B_MOTION * S] = in.motion ? (R)in.motion[i] : (R)(0.3 * 2.0);
    awake[i] = in.is_awake[i];
  }
  for (int k = tid; k < nc; k += nthreads) {
    const cz_contact c = cs[k];
    R* o = crow + k;
    o[cz::C_PX * CS] = (R)c.point[0]; o[cz::C_PY * CS] = (R)c.point[1]; o[cz::C_PZ * CS] = (R)c.point[2];
    o[cz::C_NX * CS] = (R)c.normal[0]; o[cz::C_NY * CS] = (R)c.normal[1]; o[cz::C_NZ * CS] = (R)c.normal[2];
    o[cz::C_PEN * CS] = (R)c.penetration;
    o[cz::C_FRIC * CS] = (R)c.friction;
    o[cz::C_REST * CS] = (R)c.restitution;
    const int b0 = c.body[0], b1 = c.body[1];
    if (b0 < -1 || b0 >= n || b1 < -1 || b1 >= n || (b0 < 0 && b1 < 0)) atomicOr(&m->status, 0x80000000u);
    cb[k] = cz::pack_bodies(b0, b1);
  }
}

// Reset what must start at zero (the scratch keeps the previous call's values).
__global__ void k_static_reset(unsigned char* scratch, int n, int nc) {
  Meta* m = reinterpret_cast<Meta*>(scratch + kOffMeta);
  m->contact_start = 0;
  for (int i = 0; i < 8; ++i) m->counters[i] = 0;
  for (int i = 0; i < 4; ++i) m->queue[i] = 0;
  m->body_start = 0;
  m->body_count = n;
  m->contact_cap = nc;
  m->contact_count = 0;
  m->world_status = 0;
  m->pos_iters = 0;
  m->vel_iters = 0;
  m->order = 0;
  m->order_rs = 0;
  m->status = 0;
}

// After the inputs are checked: an invalid contact list resolves nothing.
__global__ void k_static_count(unsigned char* scratch, int nc) {
  Meta* m = reinterpret_cast<Meta*>(scratch + kOffMeta);
  m->contact_count = (m->status & 0x80000000u) ? 0 : nc;
}

// Scratch rows -> the caller's arrays; resolved contacts written back in place.
template <class R>
__global__ void k_static_out(unsigned char* scratch, cz_bodies out, cz_contact* __restrict__ cs, int n, int nc) {
  const R* body = reinterpret_cast<const R*>(scratch + kOffBody);
  const uint8_t* awake = scratch + kOffAwake;
  const R* crow = reinterpret_cast<const R*>(scratch + kOffContact);
  const int* cb = reinterpret_cast<const int*>(scratch + kOffCBodies);
  const long long S = kStaticMaxBodies, CS = kStaticMaxContacts;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int nthreads = gridDim.x * blockDim.x;
  if (reinterpret_cast<const Meta*>(scratch + kOffMeta)->status & 0x80000000u) return;  // invalid input: untouched
  for (int i = tid; i < n; i += nthreads) {
    const R* b = body + i;
    for (int k = 0; k < 3; ++k) {
      out.position[3 * i + k] = (double)b[(cz::B_PX + k) * S];
      out.velocity[3 * i + k] = (double)b[(cz::B_VX + k) * S];
      out.rotation[3 * i + k] = (double)b[(cz::B_RX + k) * S];
    }
    for (int k = 0; k < 4; ++k) out.orientation[4 * i + k] = (double)b[(cz::B_QW + k) * S];
    if (out.inverse_inertia_world)
      for (int k = 0; k < 9; ++k) out.inverse_inertia_world[9 * i + k] = (double)b[(cz::B_IW0 + k) * S];
    if (out.motion) out.motion[i] = (double)b[cz::B_MOTION * S];
    out.is_awake[i] = awake[i];
  }
  for (int k = tid; k < nc; k += nthreads) {
    const R* o = crow + k;
    cs[k].normal[0] = (double)o[cz::C_NX * CS];
    cs[k].normal[1] = (double)o[cz::C_NY * CS];
    cs[k].normal[2] = (double)o[cz::C_NZ * CS];
    cs[k].penetration = (double)o[cz::C_PEN * CS];
    cs[k].body[0] = cz::body0_of(cb[k]);
    cs[k].body[1] = cz::body1_of(cb[k]);
  }
}

std::mutex g_static_mutex;
void* g_static_ptr[64] = {};

// Set-up, once per device with that device current: the device address of the array.
int static_scratch(int dev, unsigned char** out) {
  if (dev < 0 || dev >= 64) return CZ_ERR_BAD_ARG;
  std::lock_guard<std::mutex> lock(g_static_mutex);
  if (!g_static_ptr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_static_scratch) != cudaSuccess || !p) return CZ_ERR_CUDA;
    g_static_ptr[dev] = p;
  }
  *out = static_cast<unsigned char*>(g_static_ptr[dev]);
  return CZ_OK;
}

template <class R>
cz::HostView static_view(unsigned char* scratch, int n) {
  Meta* m = reinterpret_cast<Meta*>(scratch + kOffMeta);
  cz::HostView v{};
  v.body = scratch + kOffBody;
  v.awake = scratch + kOffAwake;
  v.can_sleep = nullptr;
  v.shape = nullptr;
  v.nb_pad = kStaticMaxBodies;
  v.num_worlds = 1;
  v.max_bodies = n;
  v.body_start = &m->body_start;
  v.body_count = &m->body_count;
  v.contact_start = &m->contact_start;
  v.contact_cap = &m->contact_cap;
  v.contact_count = &m->contact_count;
  v.world_status = &m->world_status;
  v.pos_iters = &m->pos_iters;
  v.vel_iters = &m->vel_iters;
  v.contact = scratch + kOffContact;
  v.contact_bodies = reinterpret_cast<int*>(scratch + kOffCBodies);
  v.work = scratch + kOffWork;
  v.work_bodies = reinterpret_cast<int*>(scratch + kOffWBodies);
  v.kmat = scratch + kOffKmat;
  v.nc_total = kStaticMaxContacts;
  v.order = &m->order;
  v.order_rs = &m->order_rs;
  v.queue = m->queue;
  v.status = &m->status;
  v.counters = m->counters;
  v.plane[0] = 0; v.plane[1] = 1; v.plane[2] = 0; v.plane[3] = 0;
  v.iter_mult = 0;
  v.max_iterations = 0;
  v.contact_writeback = 1;
  v.uniform_material = 0;
  v.mode = 0;
  v.wait_limit = 1 << 22;
  v.wait_extra_tx = 0;
  v.grid_min_bodies = 0;
  return v;
}

template <class R, class W>
int resolve_static(const cz::FormOps& ops, int32_t max_iterations, cz_contact* contacts, int32_t nc, double duration,
                   const cz_bodies* bodies, int32_t n, cudaStream_t s) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cz::set_error(CZ_ERR_NO_DEVICE, "cz_resolve_contacts_static: cudaGetDevice", e);
  unsigned char* scratch = nullptr;
  int st = static_scratch(dev, &scratch);
  if (st != CZ_OK) return cz::set_error(st, "cz_resolve_contacts_static: cudaGetSymbolAddress", cudaGetLastError());
  (void)cudaGetLastError();  // start from a clear error state
  const int threads = 256;
  const int blocks = (nc > n ? nc : n) / threads + 1;
  k_static_reset<<<1, 1, 0, s>>>(scratch, n, nc);
  k_static_in<R, W><<<blocks, threads, 0, s>>>(scratch, *bodies, contacts, n, nc);
  k_static_count<<<1, 1, 0, s>>>(scratch, nc);
  if ((e = cudaGetLastError()) != cudaSuccess)
    return cz::set_error(CZ_ERR_CUDA, "cz_resolve_contacts_static: input kernels", e);
  cz::HostView v = static_view<R>(scratch, n);
  v.max_iterations = max_iterations < 0 ? 0 : max_iterations;
  const size_t smem = ops.rs_smem(kStaticMaxBodies, kStaticContactTile, 32, 0);
  // the kernel's dynamic shared-memory limit may have been set by a batch:
  // raise it when this launch needs more, never lower it
  const void* fn = ops.resolve_kernel(32);
  cudaFuncAttributes attr;
  if ((e = cudaFuncGetAttributes(&attr, fn)) != cudaSuccess)
    return cz::set_error(CZ_ERR_CUDA, "cz_resolve_contacts_static: resolver attributes", e);
  if ((size_t)attr.maxDynamicSharedSizeBytes < smem &&
      (e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) != cudaSuccess)
    return cz::set_error(CZ_ERR_CUDA, "cz_resolve_contacts_static: resolver shared-memory limit", e);
  if ((e = ops.resolve(v, kStaticMaxBodies, kStaticContactTile, 32, 1, smem, duration, s)) != cudaSuccess)
    return cz::set_error(CZ_ERR_CUDA, "cz_resolve_contacts_static: resolver launch", e);
  k_static_out<R><<<blocks, threads, 0, s>>>(scratch, *bodies, contacts, n, nc);
  if ((e = cudaGetLastError()) != cudaSuccess)
    return cz::set_error(CZ_ERR_CUDA, "cz_resolve_contacts_static: output kernel", e);
  uint32_t bits = 0;  // read back into host stack memory
  Meta* m = reinterpret_cast<Meta*>(scratch + kOffMeta);
  if ((e = cudaMemcpyAsync(&bits, &m->status, sizeof bits, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
      (e = cudaStreamSynchronize(s)) != cudaSuccess)
    return cz::set_error(CZ_ERR_CUDA, "cz_resolve_contacts_static: status read-back", e);
  if (bits & 0x80000000u)
    return cz::set_error(CZ_ERR_BAD_ARG, "cz_resolve_contacts_static: a contact's body index is out of range",
                         cudaSuccess);
  const int st_bits = cz::status_from_bits(bits);
  if (st_bits != CZ_OK) {
    char buf[96];
    std::snprintf(buf, sizeof buf, "cz_resolve_contacts_static: device status bits 0x%x", bits);
    return cz::set_error(st_bits, buf, cudaSuccess);
  }
  return CZ_OK;
}

}  // namespace

extern "C" int cz_resolve_contacts_static(int32_t form, int32_t max_iterations, cz_contact* contacts,
                                          int32_t ncontacts, double duration, const cz_bodies* bodies,
                                          int32_t nbodies, void* stream) {
  if (!bodies || nbodies < 0 || ncontacts < 0 || (ncontacts > 0 && !contacts) ||
      (form != CZ_FORM_FP64 && form != CZ_FORM_FP32))
    return CZ_ERR_BAD_ARG;
  if (nbodies > kStaticMaxBodies || ncontacts > kStaticMaxContacts) return CZ_ERR_BAD_ARG;  // the stated maximum
  // ResolveContacts' own guards (contact.go:210-212): nothing changes
  if (duration <= 0.0 || ncontacts == 0 || nbodies == 0) return CZ_OK;
  if (!bodies->position || !bodies->orientation || !bodies->velocity || !bodies->rotation ||
      !bodies->inverse_inertia || !bodies->inverse_mass || !bodies->is_awake)
    return CZ_ERR_BAD_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (form == CZ_FORM_FP64)
    return resolve_static<double, double>(cz::kFormFP64, max_iterations, contacts, ncontacts, duration, bodies,
                                          nbodies, s);
  return resolve_static<float, double>(cz::kFormFP32, max_iterations, contacts, ncontacts, duration, bodies,
                                       nbodies, s);
}
