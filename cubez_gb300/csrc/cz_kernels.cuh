// Kernels of the batched rigid-body step, templated on the bulk type R and the
// island type W (plain form: double/double; precision form: float/double).
//
//   k_integrate    one thread per body: RigidBody.Integrate +
//                  CalculateDerivedData (rigidbody.go:213-299)
//   k_narrowphase  one CTA per world, worlds pulled from a device queue; body
//                  rows staged in shared memory with bulk async copies; the
//                  plane test and all ordered pairs in the reference's loop
//                  order (examples/cubedrop.go:41-67), compacted with warp
//                  prefix sums so the contact list order is the reference's
//   k_resolve      (cz_resolve.cuh) G lanes per world, 32/G worlds per warp,
//                  worlds pulled from a device queue: prepareContacts,
//                  adjustPositions, adjustVelocities (contact.go:204-445)
#pragma once
#include <cuda_runtime.h>

#include "cz_layout.cuh"
#include "cz_math.cuh"

namespace cz {

constexpr unsigned FULL = 0xffffffffu;

// ============================================================== integrate

template <class R, class W>
__global__ void __launch_bounds__(256) k_integrate(BatchView<R> v, R dt, R sleep_bias) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= v.nb_pad) return;
  if (!v.awake[i]) return;  // rigidbody.go:214-216
  const long long S = v.nb_pad;
  R* b = v.body + i;
#define F(r) b[(long long)(r) * S]
  const R zero = (R)0;
  const R invm = F(B_INVM);
  // lastFrameAccelleration = Acceleration + forceAccum * inverseMass (forceAccum is 0)
  v3<R> lfa = V<R>(F(B_AX), F(B_AY), F(B_AZ));
  add_scaled(lfa, V<R>(zero, zero, zero), invm);
  m3<R> iw;
#pragma unroll
  for (int k = 0; k < 9; ++k) iw.m[k] = F(B_IW0 + k);
  // angularAcceleration = iitWorld * torqueAccum (torqueAccum is 0)
  v3<R> ang = mulv(iw, V<R>(zero, zero, zero));
  v3<R> vel = V<R>(F(B_VX), F(B_VY), F(B_VZ));
  v3<R> rot = V<R>(F(B_RX), F(B_RY), F(B_RZ));
  add_scaled(vel, lfa, dt);
  add_scaled(rot, ang, dt);
  mul_with(vel, F(B_LINPOW));
  mul_with(rot, F(B_ANGPOW));
  v3<R> pos = V<R>(F(B_PX), F(B_PY), F(B_PZ));
  add_scaled(pos, vel, dt);
  q4<R> q{F(B_QW), F(B_QX), F(B_QY), F(B_QZ)};
  add_scaled_vector(q, rot, dt);
  // CalculateDerivedData: renormalise (island type), transform, world inertia
  q4<W> qw = cvtq<W>(q);
  qnormalize(qw);
  q = cvtq<R>(qw);
  R rm[9];
  rotation_of(q, rm);
  m3<R> ib;
#pragma unroll
  for (int k = 0; k < 9; ++k) ib.m[k] = F(B_IB0 + k);
  iw = world_inertia(rm, ib);
  // sleep bookkeeping, rigidbody.go:248-258
  if (v.can_sleep[i]) {
    R cm = dot(vel, vel) + dot(rot, rot);
    R motion = sleep_bias * F(B_MOTION) + ((R)1 - sleep_bias) * cm;
    if (motion < (R)0.3) {
      v.awake[i] = 0;
      vel = V<R>(zero, zero, zero);
      rot = V<R>(zero, zero, zero);
    } else if (motion > (R)3.0) {
      motion = (R)3.0;
    }
    F(B_MOTION) = motion;
  }
  F(B_PX) = pos.x; F(B_PY) = pos.y; F(B_PZ) = pos.z;
  F(B_QW) = q.w; F(B_QX) = q.x; F(B_QY) = q.y; F(B_QZ) = q.z;
  F(B_VX) = vel.x; F(B_VY) = vel.y; F(B_VZ) = vel.z;
  F(B_RX) = rot.x; F(B_RY) = rot.y; F(B_RZ) = rot.z;
  F(B_LX) = lfa.x; F(B_LY) = lfa.y; F(B_LZ) = lfa.z;
#pragma unroll
  for (int k = 0; k < 9; ++k) F(B_IW0 + k) = iw.m[k];
#undef F
}

// ============================================================== narrowphase

template <class R> struct NPContact {
  R px, py, pz, nx, ny, nz, pen;
  int b0, b1;
};

// Shared-memory tile of one world for the narrowphase.
template <class R> struct NPTile {
  R* stage;      // [11][nbs]: PX PY PZ QW QX QY QZ HX HY HZ RAD (bulk-copied)
  R* T;          // [12][nbs]: collider transforms
  int* shape;    // [nbs] (bulk-copied)
  float* cull;   // [5][nbs]: centre xyz, bounding radius |h|_2 (or r), |h|_1 (or r)
  int nbs;
  __device__ __forceinline__ R s(int r, int i) const { return stage[r * nbs + i]; }
  __device__ __forceinline__ xf<R> xform(int i) const {
    xf<R> t;
#pragma unroll
    for (int r = 0; r < 12; ++r) t.m[r] = T[r * nbs + i];
    return t;
  }
  __device__ __forceinline__ v3<R> half(int i) const { return V<R>(s(7, i), s(8, i), s(9, i)); }
  __device__ __forceinline__ R radius(int i) const { return s(10, i); }
};

template <class R>
__device__ __forceinline__ R transform_to_axis(const xf<R>& t, const v3<R>& h, const v3<R>& axis) {
  // colliders.go:762-770
  return h.x * fabs_<R>(dot(axis, t.axis(0))) + h.y * fabs_<R>(dot(axis, t.axis(1))) +
         h.z * fabs_<R>(dot(axis, t.axis(2)));
}

// tryAxis, colliders.go:458-477 (false = separating axis found)
template <class R>
__device__ __forceinline__ bool try_axis(const xf<R>& t1, const v3<R>& h1, const xf<R>& t2, const v3<R>& h2,
                                         v3<R> axis, const v3<R>& tc, int index, R& smallest, int& best) {
  if (sqmag(axis) < Lim<R>::eps()) return true;
  normalize(axis);
  R one = transform_to_axis(t1, h1, axis);
  R two = transform_to_axis(t2, h2, axis);
  R dist = fabs_<R>(dot(tc, axis));
  R p = one + two - dist;  // penetrationOnAxis, colliders.go:445-456
  if (p < (R)0) return false;
  if (p < smallest) {
    smallest = p;
    best = index;
  }
  return true;
}

// fillPointFaceBoxBox, colliders.go:479-517
template <class R>
__device__ __forceinline__ void fill_point_face(const xf<R>& one, const xf<R>& two, const v3<R>& h2, const v3<R>& tc,
                                                int best, R pen, int b0, int b1, NPContact<R>& c) {
  v3<R> nrm = one.axis(best);
  if (dot(nrm, tc) > (R)0) mul_with(nrm, (R)-1);
  v3<R> vv = h2;
  if (dot(two.axis(0), nrm) < (R)0) vv.x = -vv.x;
  if (dot(two.axis(1), nrm) < (R)0) vv.y = -vv.y;
  if (dot(two.axis(2), nrm) < (R)0) vv.z = -vv.z;
  v3<R> p = xf_mul(two, vv);
  c.px = p.x; c.py = p.y; c.pz = p.z;
  c.nx = nrm.x; c.ny = nrm.y; c.nz = nrm.z;
  c.pen = pen;
  c.b0 = b0;
  c.b1 = b1;
}

// contactPoint, colliders.go:519-573
template <class R>
__device__ __forceinline__ v3<R> edge_contact_point(const v3<R>& p1, const v3<R>& d1, R s1, const v3<R>& p2,
                                                    const v3<R>& d2, R s2, bool use_one) {
  R sm1 = sqmag(d1);
  R sm2 = sqmag(d2);
  R d12 = dot(d2, d1);
  v3<R> to = p1;
  sub(to, p2);
  R ds1 = dot(d1, to);
  R ds2 = dot(d2, to);
  R denom = sm1 * sm2 - d12 * d12;
  if (fabs_<R>(denom) < Lim<R>::eps()) return use_one ? p1 : p2;
  R mua = (d12 * ds2 - sm2 * ds1) / denom;
  R mub = (sm1 * ds2 - d12 * ds1) / denom;
  if (mua > s1 || mua < -s1 || mub > s2 || mub < -s2) return use_one ? p1 : p2;
  v3<R> c1 = d1;
  mul_with(c1, mua);
  add(c1, p1);
  v3<R> c2 = d2;
  mul_with(c2, mub);
  add(c2, p2);
  mul_with(c1, (R)0.5);
  mul_with(c2, (R)0.5);
  add(c1, c2);
  return c1;
}

// CollisionCube.CheckAgainstCube, colliders.go:575-710
template <class R>
__device__ int cube_cube(const xf<R>& t1, const v3<R>& h1, int i1, const xf<R>& t2, const v3<R>& h2, int i2,
                         NPContact<R>& c, uint32_t& err) {
  v3<R> tc = t2.axis(3);
  sub(tc, t1.axis(3));
  R pen = Lim<R>::max_value();
  int best = 0xffffff;
#pragma unroll 1
  for (int i = 0; i < 3; ++i)
    if (!try_axis(t1, h1, t2, h2, t1.axis(i), tc, i, pen, best)) return 0;
#pragma unroll 1
  for (int i = 0; i < 3; ++i)
    if (!try_axis(t1, h1, t2, h2, t2.axis(i), tc, i + 3, pen, best)) return 0;
  const int best_single = best;
#pragma unroll 1
  for (int i = 0; i < 3; ++i) {
#pragma unroll 1
    for (int j = 0; j < 3; ++j) {
      if (!try_axis(t1, h1, t2, h2, cross(t1.axis(i), t2.axis(j)), tc, i * 3 + j + 6, pen, best)) return 0;
    }
  }
  if (best < 3) {
    fill_point_face(t1, t2, h2, tc, best, pen, i1, i2, c);
    return 1;
  }
  if (best < 6) {
    v3<R> nc = tc;
    mul_with(nc, (R)-1);
    fill_point_face(t2, t1, h1, nc, best - 3, pen, i2, i1, c);
    return 1;
  }
  if (best == 0xffffff) {  // only with non-finite transforms; the reference panics here
    err |= ST_NONFINITE;
    return 0;
  }
  best -= 6;
  const int ai = best / 3, bi = best % 3;
  v3<R> oa = t1.axis(ai);
  v3<R> ob = t2.axis(bi);
  v3<R> axis = cross(oa, ob);
  normalize(axis);
  if (dot(axis, tc) > (R)0) mul_with(axis, (R)-1);
  R e1[3] = {h1.x, h1.y, h1.z};
  R e2[3] = {h2.x, h2.y, h2.z};
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    if (i == ai) e1[i] = (R)0;
    else if (dot(t1.axis(i), axis) > (R)0) e1[i] = -e1[i];
    if (i == bi) e2[i] = (R)0;
    else if (dot(t2.axis(i), axis) < (R)0) e2[i] = -e2[i];
  }
  v3<R> p1 = xf_mul(t1, V<R>(e1[0], e1[1], e1[2]));
  v3<R> p2 = xf_mul(t2, V<R>(e2[0], e2[1], e2[2]));
  const R s1 = ai == 0 ? h1.x : (ai == 1 ? h1.y : h1.z);
  const R s2 = bi == 0 ? h2.x : (bi == 1 ? h2.y : h2.z);
  v3<R> vtx = edge_contact_point(p1, oa, s1, p2, ob, s2, best_single > 2);
  c.px = vtx.x; c.py = vtx.y; c.pz = vtx.z;
  c.nx = axis.x; c.ny = axis.y; c.nz = axis.z;
  c.pen = pen;
  c.b0 = i1;
  c.b1 = i2;
  return 1;
}

// CollisionCube.CheckAgainstSphere, colliders.go:368-441.  `svel` is the
// sphere body's velocity, read only for the zero-normal fallback.
template <class R>
__device__ int cube_sphere(const xf<R>& tc, const v3<R>& h, int ic, const xf<R>& ts, R r, int is,
                           const R* svel_rows, long long svel_stride, NPContact<R>& c) {
  v3<R> pos = ts.axis(3);
  v3<R> rel = xf_inv(tc, pos);
  if (fabs_<R>(rel.x) - r > h.x || fabs_<R>(rel.y) - r > h.y || fabs_<R>(rel.z) - r > h.z) return 0;
  R hh[3] = {h.x, h.y, h.z};
  R rc[3] = {rel.x, rel.y, rel.z};
  R cl[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    R d = rc[i];
    if (d > hh[i]) d = hh[i];
    else if (d < -hh[i]) d = -hh[i];
    cl[i] = d;
  }
  v3<R> dc = V<R>(cl[0], cl[1], cl[2]);
  sub(dc, rel);
  R dist = sqmag(dc);
  if (dist > r * r) return 0;
  v3<R> cw = xf_mul(tc, V<R>(cl[0], cl[1], cl[2]));
  v3<R> nrm = cw;
  sub(nrm, pos);
  if (real_equal<R>(mag(nrm), (R)0)) {
    nrm = V<R>(svel_rows[0], svel_rows[svel_stride], svel_rows[2 * svel_stride]);
  }
  normalize(nrm);
  R pen = r;
  if (!real_equal<R>(dist, (R)0)) pen -= sqrt_<R>(dist);
  else pen = (R)0;
  c.px = cw.x; c.py = cw.y; c.pz = cw.z;
  c.nx = nrm.x; c.ny = nrm.y; c.nz = nrm.z;
  c.pen = pen;
  c.b0 = ic;
  c.b1 = is;
  return 1;
}

// CollisionSphere.CheckAgainstSphere, colliders.go:215-254
template <class R>
__device__ __forceinline__ int sphere_sphere(const v3<R>& p1, R r1, int i1, const v3<R>& p2, R r2, int i2,
                                             NPContact<R>& c) {
  v3<R> mid = p1;
  sub(mid, p2);
  R size = mag(mid);
  if (size <= (R)0 || size >= r1 + r2) return 0;
  v3<R> pt = mid;
  mul_with(pt, (R)0.5);
  add(pt, p1);
  v3<R> nrm = mid;
  mul_with(nrm, (R)1 / size);
  c.px = pt.x; c.py = pt.y; c.pz = pt.z;
  c.nx = nrm.x; c.ny = nrm.y; c.nz = nrm.z;
  c.pen = r1 + r2 - size;
  c.b0 = i1;
  c.b1 = i2;
  return 1;
}

// Vertex sign table, colliders.go:319-327 (bit k set = negative component k)
__device__ __forceinline__ v3<float> vsign(int k) {
  return V<float>((k & 1) ? -1.f : 1.f, (k & 2) ? -1.f : 1.f, (k & 4) ? -1.f : 1.f);
}

// Plane tests: CollisionSphere/CollisionCube.CheckAgainstHalfSpace
// (colliders.go:178-207, 306-366, 750-760).  Returns the number of contacts;
// with `out` non-null it also writes them (in vertex order) at out[0..].
template <class R>
__device__ int plane_contacts(const NPTile<R>& tl, int i, const BatchView<R>& v, R* out, int* outb, long long stride,
                              int room) {
  const v3<R> pn = V<R>(v.plane_nx, v.plane_ny, v.plane_nz);
  const R off = v.plane_offset;
  const xf<R> t = tl.xform(i);
  const v3<R> pos = t.axis(3);
  if (tl.shape[i] == 0) {
    const R r = tl.radius(i);
    R d = dot(pn, pos) - r;
    if (!(d <= off)) return 0;
    if (out && room > 0) {
      v3<R> p = pn;
      mul_with(p, d + r * (R)-1);
      add(p, pos);
      out[C_PX * stride] = p.x; out[C_PY * stride] = p.y; out[C_PZ * stride] = p.z;
      out[C_NX * stride] = pn.x; out[C_NY * stride] = pn.y; out[C_NZ * stride] = pn.z;
      out[C_PEN * stride] = -d;
      out[C_FRIC * stride] = (R)0.9;
      out[C_REST * stride] = (R)0.1;
      outb[0] = pack_bodies(i, -1);
    }
    return 1;
  }
  const v3<R> h = tl.half(i);
  R proj = transform_to_axis(t, h, pn);
  R cd = dot(pn, pos) - proj;
  if (!(cd <= off)) return 0;
  int cnt = 0;
#pragma unroll 1
  for (int k = 0; k < 8; ++k) {
    v3<float> sg = vsign(k);
    v3<R> vv = V<R>((R)sg.x * h.x, (R)sg.y * h.y, (R)sg.z * h.z);
    v3<R> vp = xf_mul(t, vv);
    R vd = dot(vp, pn);
    if (vd <= off) {
      if (out && cnt < room) {
        v3<R> p = pn;
        mul_with(p, vd - off);
        add(p, vp);
        R* o = out + cnt;
        o[C_PX * stride] = p.x; o[C_PY * stride] = p.y; o[C_PZ * stride] = p.z;
        o[C_NX * stride] = pn.x; o[C_NY * stride] = pn.y; o[C_NZ * stride] = pn.z;
        o[C_PEN * stride] = off - vd;
        o[C_FRIC * stride] = (R)0.9;
        o[C_REST * stride] = (R)0.1;
        outb[cnt] = pack_bodies(i, -1);
      }
      ++cnt;
    }
  }
  return cnt;
}

// Conservative float32 rejection tests.  Each returns true only when the
// reference's own test is certain to report no contact, so skipping the full
// test changes no result:
//   box-box      bounding spheres apart by 10% of the radii + 1 mm: the boxes
//                are disjoint by more than the separating-axis test's rounding
//                and more than its skipping of near-parallel edge axes
//                (|a x b|^2 < 1e-7, colliders.go:461) can hide;
//   sphere-sphere  centres farther than r1 + r2 + 1 mm (colliders.go:227);
//   box-sphere   centre distance above |h|_1 + 3r + 1 mm, so some axis has
//                |rel_i| - r > h_i (the early exit of colliders.go:374-378).
// The margins dwarf the float32 rounding of positions (1e-5 relative is
// added); non-finite centres never reject.
struct Cull {
  const float* c;
  int nbs;
  __device__ __forceinline__ float d2_scale(int i, int j, float& scale) const {
    float dx = c[j] - c[i];
    float dy = c[nbs + j] - c[nbs + i];
    float dz = c[2 * nbs + j] - c[2 * nbs + i];
    scale = 1.f + fabsf(c[i]) + fabsf(c[nbs + i]) + fabsf(c[2 * nbs + i]) + fabsf(c[j]) + fabsf(c[nbs + j]) +
            fabsf(c[2 * nbs + j]);
    return dx * dx + dy * dy + dz * dz;
  }
  __device__ __forceinline__ float rb(int i) const { return c[3 * nbs + i]; }  // |h|_2 or r
  __device__ __forceinline__ float rl(int i) const { return c[4 * nbs + i]; }  // |h|_1 or r
  __device__ __forceinline__ bool boxes(int i, int j) const {
    float sc, d2 = d2_scale(i, j, sc);
    float t = (rb(i) + rb(j)) * 1.1f + 1e-3f + 1e-5f * sc;
    return d2 > t * t;
  }
  __device__ __forceinline__ bool spheres(int i, int j) const {
    float sc, d2 = d2_scale(i, j, sc);
    float t = rb(i) + rb(j) + 1e-3f + 1e-5f * sc;
    return d2 > t * t;
  }
  __device__ __forceinline__ bool box_sphere(int box, int sph) const {
    float sc, d2 = d2_scale(box, sph, sc);
    float t = rl(box) + 3.f * rb(sph) + 1e-3f + 1e-5f * sc;
    return d2 > t * t;
  }
};

// One ordered pair (i, j): CheckForCollisions(collider i, collider j)
// (colliders.go:718-747 with the forwarding of colliders.go:209-213).
template <class R>
__device__ int pair_test(const NPTile<R>& tl, int i, int j, const BatchView<R>& v, int bstart, NPContact<R>& c,
                         uint32_t& err) {
  const int si = tl.shape[i], sj = tl.shape[j];
  const Cull cl{tl.cull, tl.nbs};
  if (sj == 0) {
    if (si == 0) {
      if (cl.spheres(i, j)) return 0;
      return sphere_sphere(V<R>(tl.T[9 * tl.nbs + i], tl.T[10 * tl.nbs + i], tl.T[11 * tl.nbs + i]), tl.radius(i), i,
                           V<R>(tl.T[9 * tl.nbs + j], tl.T[10 * tl.nbs + j], tl.T[11 * tl.nbs + j]), tl.radius(j), j,
                           c);
    }
    if (cl.box_sphere(i, j)) return 0;
    return cube_sphere(tl.xform(i), tl.half(i), i, tl.xform(j), tl.radius(j), j,
                       v.body + (long long)B_VX * v.nb_pad + bstart + j, v.nb_pad, c);
  }
  if (si == 0) {
    if (cl.box_sphere(j, i)) return 0;
    return cube_sphere(tl.xform(j), tl.half(j), j, tl.xform(i), tl.radius(i), i,
                       v.body + (long long)B_VX * v.nb_pad + bstart + i, v.nb_pad, c);
  }
  if (cl.boxes(i, j)) return 0;
  return cube_cube(tl.xform(i), tl.half(i), i, tl.xform(j), tl.half(j), j, c, err);
}

// ---- bulk async copy (TMA engine) helpers
__device__ __forceinline__ unsigned smem_addr(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}
// Bounded wait on an mbarrier phase; false if it gave up.
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity, int limit) {
  unsigned a = smem_addr(bar);
  for (int it = 0; it < limit; ++it) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

template <class R> __host__ __device__ inline size_t np_smem_bytes(int nbs) {
  size_t b = 16;                                  // mbarrier + pad
  b += (size_t)(11 + 12) * nbs * sizeof(R);       // staged rows + transforms
  b += (size_t)nbs * sizeof(int);                 // shape
  b += (size_t)5 * nbs * sizeof(float);           // cull data
  b += 2 * 33 * sizeof(int);                      // scan scratch (double-buffered) + world id
  return b;
}

// Whether a collider Offset's rotation part is orthonormal to within 1e-5
// (a reflection included): then the collider transform is an isometry up to
// rounding and the cube's bounding radii hold.  NaN fails.
template <class R> __device__ __forceinline__ bool offset_is_rigid(const R (&o)[12]) {
  bool ok = true;
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = a; b < 3; ++b) {
      const float d = (float)o[3 * a] * (float)o[3 * b] + (float)o[3 * a + 1] * (float)o[3 * b + 1] +
                      (float)o[3 * a + 2] * (float)o[3 * b + 2];
      ok = ok && fabsf(d - (a == b ? 1.f : 0.f)) <= 1e-5f;
    }
  return ok;
}

// Collider transforms (SetAsTransform x Offset) and the float32 cull data of
// the staged bodies of one world, by the whole CTA.  `off` is the world's
// first body in the Offset rows (row stride `so`), or null for the identity.
// A cube whose Offset is not rigid gets infinite bounding radii: its pairs are
// never culled.
template <class R>
__device__ __forceinline__ void np_build_tile(const NPTile<R>& tl, int n, const R* __restrict__ off, long long so) {
  const int nbs = tl.nbs;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    v3<R> p = V<R>(tl.s(0, i), tl.s(1, i), tl.s(2, i));
    q4<R> q{tl.s(3, i), tl.s(4, i), tl.s(5, i), tl.s(6, i)};
    xf<R> t;
    bool rigid = true;
    if (off) {
      R o[12];
#pragma unroll
      for (int r = 0; r < 12; ++r) o[r] = off[r * so + i];
      t = collider_transform(p, q, o);
      rigid = offset_is_rigid(o);
    } else {
      t = collider_transform(p, q);
    }
#pragma unroll
    for (int r = 0; r < 12; ++r) tl.T[r * nbs + i] = t.m[r];
    float rb, rl;
    if (tl.shape[i] == 0) {
      rb = rl = (float)tl.s(10, i);
    } else if (!rigid) {
      rb = rl = __int_as_float(0x7f800000);
    } else {
      float hx = (float)tl.s(7, i), hy = (float)tl.s(8, i), hz = (float)tl.s(9, i);
      rb = sqrtf(hx * hx + hy * hy + hz * hz) * 1.0001f;
      rl = (hx + hy + hz) * 1.0001f;
    }
    tl.cull[i] = (float)t.m[9];
    tl.cull[nbs + i] = (float)t.m[10];
    tl.cull[2 * nbs + i] = (float)t.m[11];
    tl.cull[3 * nbs + i] = rb;
    tl.cull[4 * nbs + i] = rl;
  }
}

// Block-wide scan of one chunk's per-unit contact counts in unit order: the
// thread's exclusive offset and the chunk total.  The warp totals are
// double-buffered (scan[32 * parity]), so a chunk needs two barriers.
__device__ __forceinline__ void np_chunk_scan(int cnt, int* scan, int parity, int* excl, int* total) {
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nwarps = (blockDim.x + 31) >> 5;
  int x = cnt;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    int y = __shfl_up_sync(FULL, x, d);
    if (lane >= d) x += y;
  }
  int* wt = scan + 32 * parity;
  if (lane == 31) wt[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int t = lane < nwarps ? wt[lane] : 0;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      int y = __shfl_up_sync(FULL, t, d);
      if (lane >= d) t += y;
    }
    if (lane < nwarps) wt[lane] = t;
  }
  __syncthreads();
  *excl = (wid > 0 ? wt[wid - 1] : 0) + x - cnt;
  *total = wt[nwarps - 1];
}

// Write one unit's contacts (a pair's single contact or a half-space test's
// 0..8) at slot `off` of the world's contact slab, within its capacity.
template <class R>
__device__ __forceinline__ void np_emit(const NPTile<R>& tl, const BatchView<R>& v, long long cs, int cap, int off,
                                        int cnt, int i, bool plane, const NPContact<R>& c) {
  if (cnt <= 0) return;
  const int room = cap - off;
  if (room <= 0) return;
  R* o = v.contact + cs + off;
  int* ob = v.contact_bodies + cs + off;
  if (plane) {
    plane_contacts<R>(tl, i, v, o, ob, v.nc_total, room);
  } else {
    const long long S = v.nc_total;
    o[C_PX * S] = c.px; o[C_PY * S] = c.py; o[C_PZ * S] = c.pz;
    o[C_NX * S] = c.nx; o[C_NY * S] = c.ny; o[C_NZ * S] = c.nz;
    o[C_PEN * S] = c.pen;
    o[C_FRIC * S] = (R)0.9;
    o[C_REST * S] = (R)0.1;
    ob[0] = pack_bodies(c.b0, c.b1);
  }
}

template <class R>
__global__ void __launch_bounds__(256) k_narrowphase(BatchView<R> v, int nbs) {
  extern __shared__ __align__(128) unsigned char smem[];
  unsigned long long* bar = reinterpret_cast<unsigned long long*>(smem);
  NPTile<R> tl;
  tl.nbs = nbs;
  tl.stage = reinterpret_cast<R*>(smem + 16);
  tl.T = tl.stage + 11 * nbs;
  tl.shape = reinterpret_cast<int*>(tl.T + 12 * nbs);
  tl.cull = reinterpret_cast<float*>(tl.shape + nbs);
  int* scan = reinterpret_cast<int*>(tl.cull + 5 * nbs);  // [2][32] + [64] world id
  const int tid = threadIdx.x;
  if (tid == 0) mbar_init(bar, 1);
  __syncthreads();
  unsigned phase = 0;
  int chunk_parity = 0;
  for (;;) {
    if (tid == 0) {
      unsigned q = atomicAdd(&v.queue[0], 1u);
      scan[64] = q < (unsigned)v.num_worlds ? v.order[q] : -1;
    }
    __syncthreads();
    const int w = scan[64];
    if (w < 0) break;
    const int n = v.body_count[w];
    const int bstart = v.body_start[w];
    if (n > nbs) {
      if (tid == 0) {
        v.world_status[w] |= ST_BODY_LIMIT;
        atomicOr(v.status, ST_BODY_LIMIT);
        v.contact_count[w] = 0;
      }
      __syncthreads();
      continue;
    }
    const int n4 = (n + 3) & ~3;
    if (tid == 0 && n4 > 0) {
      // order smem accesses of the previous world before the async-proxy writes
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      const unsigned rb = (unsigned)(n4 * sizeof(R));
      mbar_expect_tx(bar, rb * 11u + (unsigned)(n4 * sizeof(int)));
#pragma unroll 1
      for (int r = 0; r < 11; ++r) bulk_g2s(tl.stage + r * nbs, v.body + (long long)r * v.nb_pad + bstart, rb, bar);
      bulk_g2s(tl.shape, v.shape + bstart, (unsigned)(n4 * sizeof(int)), bar);
    }
    if (n4 > 0) {
      bool ok = mbar_wait(bar, phase, 1 << 22);
      phase ^= 1u;
      if (!ok) {  // give up on the whole launch; the copies are bounded and tiny, so this is a fault signal
        if (tid == 0) {
          v.world_status[w] |= ST_TIMEOUT;
          atomicOr(v.status, ST_TIMEOUT);
        }
        return;
      }
    }
    np_build_tile(tl, n, v.offset ? v.offset + bstart : nullptr, v.nb_pad);
    __syncthreads();
    const long long cs = v.contact_start[w];
    const int cap = v.contact_cap[w];
    const long long U = (long long)n * n;
    int out = 0;
    uint32_t err = 0;
    for (long long base = 0; base < U; base += blockDim.x) {
      const long long u = base + tid;
      int cnt = 0, i = 0, k = 0;
      NPContact<R> c;
      if (u < U) {
        i = (int)(u / n);
        k = (int)(u - (long long)i * n);
        if (k == 0) {
          cnt = plane_contacts<R>(tl, i, v, nullptr, nullptr, 0, 0);
        } else {
          int j = k - 1;
          if (j >= i) ++j;
          cnt = pair_test<R>(tl, i, j, v, bstart, c, err);
        }
      }
      int excl, total;
      np_chunk_scan(cnt, scan, chunk_parity, &excl, &total);
      chunk_parity ^= 1;
      np_emit<R>(tl, v, cs, cap, out + excl, cnt, i, k == 0, c);
      out += total;
    }
    if (err) {
      atomicOr(&v.world_status[w], err);
      atomicOr(v.status, err);
    }
    if (tid == 0) {
      v.contact_count[w] = out;
      atomicAdd(&v.counters[0], (unsigned long long)out);
      if (out > cap) {
        atomicOr(&v.world_status[w], ST_CAPACITY);
        atomicOr(v.status, ST_CAPACITY);
      }
    }
    __syncthreads();
  }
}

// The narrowphase for a caller's list of units of one world (colliders.go:
// CheckAgainstHalfSpace when j < 0, else CheckForCollisions(i, j)), in the
// list's order, replacing the world's contact list: one CTA, bodies staged by
// plain loads, the same tests, scan and emission as k_narrowphase.  Indices
// are validated by the host.
template <class R>
__global__ void __launch_bounds__(256) k_collide(BatchView<R> v, int w, const int2* __restrict__ units, int nunits,
                                                 int nbs) {
  extern __shared__ __align__(128) unsigned char smem[];
  NPTile<R> tl;
  tl.nbs = nbs;
  tl.stage = reinterpret_cast<R*>(smem + 16);
  tl.T = tl.stage + 11 * nbs;
  tl.shape = reinterpret_cast<int*>(tl.T + 12 * nbs);
  tl.cull = reinterpret_cast<float*>(tl.shape + nbs);
  int* scan = reinterpret_cast<int*>(tl.cull + 5 * nbs);
  const int tid = threadIdx.x;
  const int n = v.body_count[w];
  const int bstart = v.body_start[w];
  for (int i = tid; i < n; i += blockDim.x) {
#pragma unroll
    for (int r = 0; r < 11; ++r) tl.stage[r * nbs + i] = v.body[(long long)r * v.nb_pad + bstart + i];
    tl.shape[i] = v.shape[bstart + i];
  }
  __syncthreads();
  np_build_tile(tl, n, v.offset ? v.offset + bstart : nullptr, v.nb_pad);
  __syncthreads();
  const long long cs = v.contact_start[w];
  const int cap = v.contact_cap[w];
  int out = 0, parity = 0;
  uint32_t err = 0;
  for (int base = 0; base < nunits; base += blockDim.x) {
    const int u = base + tid;
    int cnt = 0, i = 0;
    bool plane = false;
    NPContact<R> c;
    if (u < nunits) {
      const int2 un = units[u];
      i = un.x;
      plane = un.y < 0;
      cnt = plane ? plane_contacts<R>(tl, i, v, nullptr, nullptr, 0, 0) : pair_test<R>(tl, i, un.y, v, bstart, c, err);
    }
    int excl, total;
    np_chunk_scan(cnt, scan, parity, &excl, &total);
    parity ^= 1;
    np_emit<R>(tl, v, cs, cap, out + excl, cnt, i, plane, c);
    out += total;
  }
  if (err) {
    atomicOr(&v.world_status[w], err);
    atomicOr(v.status, err);
  }
  if (tid == 0) {
    v.contact_count[w] = out;
    atomicAdd(&v.counters[0], (unsigned long long)out);
    if (out > cap) {
      atomicOr(&v.world_status[w], ST_CAPACITY);
      atomicOr(v.status, ST_CAPACITY);
    }
  }
}

}  // namespace cz

#include "cz_resolve.cuh"
#include "cz_resolve_big.cuh"
