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
//   k_resolve      one warp per world, worlds pulled from a device queue:
//                  prepareContacts, adjustPositions, adjustVelocities
//                  (contact.go:204-445) with a warp argmax whose tie-break is
//                  the reference's first-maximum rule
#pragma once
#include <cuda_runtime.h>

#include "cz_layout.cuh"
#include "cz_math.cuh"

namespace cz {

constexpr unsigned FULL = 0xffffffffu;

// ============================================================== bit keys
// Order-preserving keys for the argmax.  A value v gets key(v) > 0 exactly
// when v > eps and v is not NaN; for such values key order is value order
// (IEEE bit patterns of non-negative numbers sort like the numbers).
__device__ __forceinline__ unsigned long long key_of(double v, double eps) {
  long long b = __double_as_longlong(v);
  long long e = __double_as_longlong(eps);
  return (b > e && b <= 0x7FF0000000000000LL) ? (unsigned long long)b : 0ull;
}
__device__ __forceinline__ unsigned key_of(float v, float eps) {
  int b = __float_as_int(v);
  int e = __float_as_int(eps);
  return (b > e && b <= 0x7F800000) ? (unsigned)b : 0u;
}

// First maximum over the warp: returns the smallest contact index holding the
// largest key, or -1 when no key is positive (no value above the epsilon).
__device__ __forceinline__ int warp_first_max(unsigned long long key, int idx) {
  unsigned hi = (unsigned)(key >> 32);
  unsigned mhi = __reduce_max_sync(FULL, hi);
  unsigned lo = (hi == mhi) ? (unsigned)key : 0u;
  unsigned mlo = __reduce_max_sync(FULL, lo);
  if (mhi == 0u && mlo == 0u) return -1;
  int cand = (hi == mhi && (unsigned)key == mlo) ? idx : 0x7fffffff;
  return __reduce_min_sync(FULL, cand);
}
__device__ __forceinline__ int warp_first_max(unsigned key, int idx) {
  unsigned m = __reduce_max_sync(FULL, key);
  if (m == 0u) return -1;
  return __reduce_min_sync(FULL, key == m ? idx : 0x7fffffff);
}

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
  float* cull;   // [4][nbs]: centre xyz, bounding radius
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

// Conservative bounding-sphere rejection for a box pair.  Two boxes whose
// bounding spheres are apart by more than the margin are disjoint by a gap
// larger than any rounding error of the separating-axis test and larger than
// what the test's skipping of near-parallel edge axes (|a x b|^2 < 1e-7) can
// hide, so the full test would report no contact; the margin is generous on
// both counts.  Non-finite centres never reject.
__device__ __forceinline__ bool boxes_far_apart(const float* cull, int nbs, int i, int j) {
  float dx = cull[j] - cull[i];
  float dy = cull[nbs + j] - cull[nbs + i];
  float dz = cull[2 * nbs + j] - cull[2 * nbs + i];
  float ri = cull[3 * nbs + i], rj = cull[3 * nbs + j];
  float scale = 1.f + fabsf(cull[i]) + fabsf(cull[nbs + i]) + fabsf(cull[2 * nbs + i]) + fabsf(cull[j]) +
                fabsf(cull[nbs + j]) + fabsf(cull[2 * nbs + j]);
  float thr = (ri + rj) * 1.1f + 1e-3f + 1e-5f * scale;
  return dx * dx + dy * dy + dz * dz > thr * thr;
}

// One ordered pair (i, j): CheckForCollisions(collider i, collider j)
// (colliders.go:718-747 with the forwarding of colliders.go:209-213).
template <class R>
__device__ int pair_test(const NPTile<R>& tl, int i, int j, const BatchView<R>& v, int bstart, NPContact<R>& c,
                         uint32_t& err) {
  const int si = tl.shape[i], sj = tl.shape[j];
  if (sj == 0) {
    if (si == 0)
      return sphere_sphere(V<R>(tl.T[9 * tl.nbs + i], tl.T[10 * tl.nbs + i], tl.T[11 * tl.nbs + i]), tl.radius(i), i,
                           V<R>(tl.T[9 * tl.nbs + j], tl.T[10 * tl.nbs + j], tl.T[11 * tl.nbs + j]), tl.radius(j), j,
                           c);
    return cube_sphere(tl.xform(i), tl.half(i), i, tl.xform(j), tl.radius(j), j,
                       v.body + (long long)B_VX * v.nb_pad + bstart + j, v.nb_pad, c);
  }
  if (si == 0)
    return cube_sphere(tl.xform(j), tl.half(j), j, tl.xform(i), tl.radius(i), i,
                       v.body + (long long)B_VX * v.nb_pad + bstart + i, v.nb_pad, c);
  if (boxes_far_apart(tl.cull, tl.nbs, i, j)) return 0;
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
  b += (size_t)4 * nbs * sizeof(float);           // cull data
  b += 2 * 33 * sizeof(int);                      // scan scratch (double-buffered) + world id
  return b;
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
  int* scan = reinterpret_cast<int*>(tl.cull + 4 * nbs);  // [2][32] + [64] world id
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nwarps = (blockDim.x + 31) >> 5;
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
    // collider transforms + bounding data
    for (int i = tid; i < n; i += blockDim.x) {
      v3<R> p = V<R>(tl.s(0, i), tl.s(1, i), tl.s(2, i));
      q4<R> q{tl.s(3, i), tl.s(4, i), tl.s(5, i), tl.s(6, i)};
      xf<R> t = collider_transform(p, q);
#pragma unroll
      for (int r = 0; r < 12; ++r) tl.T[r * nbs + i] = t.m[r];
      float rb;
      if (tl.shape[i] == 0) {
        rb = (float)tl.s(10, i);
      } else {
        float hx = (float)tl.s(7, i), hy = (float)tl.s(8, i), hz = (float)tl.s(9, i);
        rb = sqrtf(hx * hx + hy * hy + hz * hz) * 1.0001f;
      }
      tl.cull[i] = (float)t.m[9];
      tl.cull[nbs + i] = (float)t.m[10];
      tl.cull[2 * nbs + i] = (float)t.m[11];
      tl.cull[3 * nbs + i] = rb;
    }
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
      // block-wide inclusive scan of the counts in unit order
      int x = cnt;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        int y = __shfl_up_sync(FULL, x, d);
        if (lane >= d) x += y;
      }
      int* wt = scan + 32 * chunk_parity;
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
      const int prefix = wid > 0 ? wt[wid - 1] : 0;
      const int total = wt[nwarps - 1];
      const int off = out + prefix + x - cnt;
      chunk_parity ^= 1;
      if (cnt > 0) {
        const int room = cap - off;
        if (room > 0) {
          R* o = v.contact + cs + off;
          int* ob = v.contact_bodies + cs + off;
          if (k == 0) {
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
      }
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

// ============================================================== resolver

template <class R, class W> struct RCtx {
  W* bw;          // [7][nbs]: position xyz, orientation wxyz (island type)
  R* br;          // [20][nbs]: vel 0-2, rot 3-5, lfa 6-8, iitWorld 9-17, invMass 18, motion 19
  uint8_t* aw;    // [nbs] awake
  int nbs;
  R* cw;          // working rows of this world's contacts
  int* cb;        // packed bodies of this world's contacts
  long long cst;  // row stride of cw
  R* bc;          // broadcast scratch [12]
  R dt;
  __device__ __forceinline__ W& P(int c, int i) const { return bw[c * nbs + i]; }
  __device__ __forceinline__ R& Bf(int r, int i) const { return br[r * nbs + i]; }
  __device__ __forceinline__ R& Cf(int f, int k) const { return cw[(long long)f * cst + k]; }
  __device__ __forceinline__ v3<R> Bv(int r, int i) const { return V<R>(Bf(r, i), Bf(r + 1, i), Bf(r + 2, i)); }
  __device__ __forceinline__ v3<R> Cv(int f, int k) const { return V<R>(Cf(f, k), Cf(f + 1, k), Cf(f + 2, k)); }
  __device__ __forceinline__ void setCv(int f, int k, const v3<R>& a) const {
    Cf(f, k) = a.x; Cf(f + 1, k) = a.y; Cf(f + 2, k) = a.z;
  }
  __device__ __forceinline__ m3<R> iit(int i) const {
    m3<R> m;
#pragma unroll
    for (int k = 0; k < 9; ++k) m.m[k] = Bf(9 + k, i);
    return m;
  }
  // contactToWorld columns
  __device__ __forceinline__ m3<R> basis(int k) const {
    m3<R> m;
#pragma unroll
    for (int q = 0; q < 9; ++q) m.m[q] = Cf(W_NX + q, k);
    return m;
  }
};

// calculateDesiredDeltaVelocity, contact.go:87-112
template <class R, class W> __device__ __forceinline__ R desired_dv(const RCtx<R, W>& x, int k) {
  const int bb = x.cb[k];
  const int b0 = body0_of(bb), b1 = body1_of(bb);
  const v3<R> n = x.Cv(W_NX, k);
  R vfa = (R)0;
  if (x.aw[b0]) {
    v3<R> t = x.Bv(6, b0);
    mul_with(t, x.dt);
    vfa += dot(t, n);
  }
  if (b1 >= 0 && x.aw[b1]) {
    v3<R> t = x.Bv(6, b1);
    mul_with(t, x.dt);
    vfa -= dot(t, n);
  }
  R rest = x.Cf(W_REST, k);
  const R cvx = x.Cf(W_CVX, k);
  if (fabs_<R>(cvx) < (R)0.25) rest = (R)0;
  return -cvx - rest * (cvx - vfa);
}

// calculateLocalVelocity, contact.go:158-182
template <class R, class W>
__device__ __forceinline__ v3<R> local_velocity(const RCtx<R, W>& x, int body, const v3<R>& rp, const m3<R>& C) {
  v3<R> vel = cross(x.Bv(3, body), rp);
  add(vel, x.Bv(0, body));
  v3<R> cv = mulv_t(C, vel);
  v3<R> acc = x.Bv(6, body);
  mul_with(acc, x.dt);
  acc = mulv_t(C, acc);
  acc.x = (R)0;
  add(cv, acc);
  return cv;
}

// calculateInternals, contact.go:59-85, from the narrowphase rows.
template <class R, class W>
__device__ void prepare_contact(const RCtx<R, W>& x, const BatchView<R>& v, long long src, int k) {
  const long long S = v.nc_total;
  const R* g = v.contact + src;
  v3<R> n = V<R>(g[C_NX * S], g[C_NY * S], g[C_NZ * S]);
  const v3<R> p = V<R>(g[C_PX * S], g[C_PY * S], g[C_PZ * S]);
  int bb = v.contact_bodies[src];
  int b0 = body0_of(bb), b1 = body1_of(bb);
  if (b0 < 0) {
    mul_with(n, (R)-1);
    b0 = b1;
    b1 = -1;
    bb = pack_bodies(b0, b1);
  }
  // calculateContactBasis, contact.go:114-156
  v3<R> ty, tz;
  if (fabs_<R>(n.x) > fabs_<R>(n.y)) {
    R s = (R)1 / sqrt_<R>(n.z * n.z + n.x * n.x);
    ty = V<R>(n.z * s, (R)0, n.x * -s);
    tz = V<R>(n.y * ty.x, n.z * ty.x - n.x * ty.z, -n.y * ty.x);
  } else {
    R s = (R)1 / sqrt_<R>(n.z * n.z + n.y * n.y);
    ty = V<R>((R)0, -n.z * s, n.y * s);
    tz = V<R>(n.y * ty.z - n.z * ty.y, -n.x * ty.z, n.x * ty.y);
  }
  m3<R> C;
  C.m[0] = n.x; C.m[1] = n.y; C.m[2] = n.z;
  C.m[3] = ty.x; C.m[4] = ty.y; C.m[5] = ty.z;
  C.m[6] = tz.x; C.m[7] = tz.y; C.m[8] = tz.z;
  v3<R> rp0 = p;
  sub(rp0, V<R>((R)x.P(0, b0), (R)x.P(1, b0), (R)x.P(2, b0)));
  v3<R> cv = local_velocity(x, b0, rp0, C);
  v3<R> rp1 = V<R>((R)0, (R)0, (R)0);
  if (b1 >= 0) {
    rp1 = p;
    sub(rp1, V<R>((R)x.P(0, b1), (R)x.P(1, b1), (R)x.P(2, b1)));
    v3<R> cv1 = local_velocity(x, b1, rp1, C);
    sub(cv, cv1);
  }
  x.cb[k] = bb;
  x.Cf(W_PEN, k) = g[C_PEN * S];
  x.setCv(W_NX, k, n);
  x.setCv(W_TYX, k, ty);
  x.setCv(W_TZX, k, tz);
  x.setCv(W_R0X, k, rp0);
  x.setCv(W_R1X, k, rp1);
  x.setCv(W_CVX, k, cv);
  x.Cf(W_FRIC, k) = g[C_FRIC * S];
  x.Cf(W_REST, k) = g[C_REST * S];
  x.Cf(W_DDV, k) = desired_dv(x, k);
}

// SetAwake(true) (rigidbody.go:182-187) through matchAwakeState (contact.go:184-202)
template <class R, class W> __device__ __forceinline__ void match_awake(const RCtx<R, W>& x, int bb) {
  const int b0 = body0_of(bb), b1 = body1_of(bb);
  if (b1 < 0) return;
  const bool a0 = x.aw[b0] != 0, a1 = x.aw[b1] != 0;
  if ((a0 || a1) && !(a0 && a1)) {
    const int t = a0 ? b1 : b0;
    x.aw[t] = 1;
    x.Bf(19, t) = (R)(0.3 * 2.0);
  }
}

// CalculateDerivedData for a body that is asleep during adjustPositions
// (contact.go:380-382): renormalise, refresh the world inverse inertia.
template <class R, class W>
__device__ void derive_asleep(const RCtx<R, W>& x, const BatchView<R>& v, int bstart, int body) {
  q4<R> q{(R)x.P(3, body), (R)x.P(4, body), (R)x.P(5, body), (R)x.P(6, body)};
  q4<W> qw = cvtq<W>(q);
  qnormalize(qw);
  q = cvtq<R>(qw);
  R rm[9];
  rotation_of(q, rm);
  m3<R> ib;
#pragma unroll
  for (int k = 0; k < 9; ++k) ib.m[k] = v.body[(long long)(B_IB0 + k) * v.nb_pad + bstart + body];
  m3<R> iw = world_inertia(rm, ib);
#pragma unroll
  for (int k = 0; k < 9; ++k) x.Bf(9 + k, body) = iw.m[k];
  x.P(3, body) = (W)q.w; x.P(4, body) = (W)q.x; x.P(5, body) = (W)q.y; x.P(6, body) = (W)q.z;
}

// applyPositionChange, contact.go:285-386 (single lane); the linear and
// angular changes of both bodies go to x.bc[0..11].
template <class R, class W>
__device__ void apply_position_change(const RCtx<R, W>& x, const BatchView<R>& v, int bstart, int k, R penetration) {
  const int bb = x.cb[k];
  const int body[2] = {body0_of(bb), body1_of(bb)};
  const v3<R> n = x.Cv(W_NX, k);
  const v3<R> rp[2] = {x.Cv(W_R0X, k), x.Cv(W_R1X, k)};
  R angI[2] = {(R)0, (R)0}, linI[2] = {(R)0, (R)0};
  R total = (R)0;
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    if (body[i] < 0) continue;
    v3<R> a = cross(rp[i], n);
    a = mulv(x.iit(body[i]), a);
    a = cross(a, rp[i]);
    angI[i] = dot(a, n);
    linI[i] = x.Bf(18, body[i]);
    total += linI[i] + angI[i];
  }
  v3<R> lin[2], ang[2];
  const R z = (R)0;
  lin[0] = lin[1] = ang[0] = ang[1] = V<R>(z, z, z);
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    if (body[i] < 0) continue;
    const int b = body[i];
    const R sign = i != 0 ? (R)-1 : (R)1;
    R am = sign * penetration * (angI[i] / total);
    R lm = sign * penetration * (linI[i] / total);
    v3<R> proj = rp[i];
    add_scaled(proj, n, -dot(rp[i], n));
    const R maxm = (R)0.2 * mag(proj);
    if (am < -maxm) {
      R tm = am + lm;
      am = -maxm;
      lm = tm - am;
    } else if (am > maxm) {
      R tm = am + lm;
      am = maxm;
      lm = tm - am;
    }
    if (am == (R)0) {
      ang[i] = V<R>(z, z, z);
    } else {
      ang[i] = mulv(x.iit(b), cross(rp[i], n));
      mul_with(ang[i], am / angI[i]);
    }
    lin[i] = n;
    mul_with(lin[i], lm);
    // Position.AddScaled(normal, linearMove): product in R, accumulated in W
    x.P(0, b) += (W)(n.x * lm);
    x.P(1, b) += (W)(n.y * lm);
    x.P(2, b) += (W)(n.z * lm);
    q4<W> q{x.P(3, b), x.P(4, b), x.P(5, b), x.P(6, b)};
    add_scaled_vector(q, cvt<W>(ang[i]), (W)1);
    qnormalize(q);
    x.P(3, b) = q.w; x.P(4, b) = q.x; x.P(5, b) = q.y; x.P(6, b) = q.z;
    if (!x.aw[b]) {
      // the stored orientation is the R-rounded one before CalculateDerivedData
      x.P(3, b) = (W)(R)q.w; x.P(4, b) = (W)(R)q.x; x.P(5, b) = (W)(R)q.y; x.P(6, b) = (W)(R)q.z;
      derive_asleep(x, v, bstart, b);
    }
  }
  x.bc[0] = lin[0].x; x.bc[1] = lin[0].y; x.bc[2] = lin[0].z;
  x.bc[3] = lin[1].x; x.bc[4] = lin[1].y; x.bc[5] = lin[1].z;
  x.bc[6] = ang[0].x; x.bc[7] = ang[0].y; x.bc[8] = ang[0].z;
  x.bc[9] = ang[1].x; x.bc[10] = ang[1].y; x.bc[11] = ang[1].z;
}

template <class R> __device__ __forceinline__ m3<R> skew(const v3<R>& v) {  // contact.go:612-616
  m3<R> m;
  m.m[0] = (R)0; m.m[3] = -v.z; m.m[6] = v.y;
  m.m[1] = v.z; m.m[4] = (R)0; m.m[7] = -v.x;
  m.m[2] = -v.y; m.m[5] = v.x; m.m[8] = (R)0;
  return m;
}

// calculateFrictionImpulse, contact.go:533-606 (3x3 inversion and solve in W)
template <class R, class W>
__device__ v3<R> friction_impulse(const RCtx<R, W>& x, int k, int b0, int b1, const m3<R>& C) {
  R inv_mass = x.Bf(18, b0);
  m3<R> itt = skew(x.Cv(W_R0X, k));
  m3<R> dvw = mulm(itt, x.iit(b0));
  dvw = mulm(dvw, itt);
  mulm_with(dvw, (R)-1);
  if (b1 >= 0) {
    itt = skew(x.Cv(W_R1X, k));
    m3<R> d2 = mulm(itt, x.iit(b1));
    d2 = mulm(d2, itt);
    mulm_with(d2, (R)-1);
#pragma unroll
    for (int q = 0; q < 9; ++q) dvw.m[q] += d2.m[q];
    inv_mass += x.Bf(18, b1);
  }
  m3<R> dv = transpose(C);
  dv = mulm(dv, dvw);
  dv = mulm(dv, C);
  dv.m[0] += inv_mass;
  dv.m[4] += inv_mass;
  dv.m[8] += inv_mass;
  m3<W> dvw64;
#pragma unroll
  for (int q = 0; q < 9; ++q) dvw64.m[q] = (W)dv.m[q];
  const m3<W> K = invert(dvw64);
  const R ddv = x.Cf(W_DDV, k);
  const v3<W> kill = V<W>((W)ddv, (W)-x.Cf(W_CVY, k), (W)-x.Cf(W_CVZ, k));
  v3<R> ic = cvt<R>(mulv(K, kill));
  const R fr = x.Cf(W_FRIC, k);
  R planar = sqrt_<R>(ic.y * ic.y + ic.z * ic.z);
  if (planar > ic.x * fr) {
    ic.y /= planar;
    ic.z /= planar;
    ic.x = dv.m[0] + dv.m[3] * fr * ic.y + dv.m[6] * fr * ic.z;
    ic.x = ddv / ic.x;
    ic.y *= fr * ic.x;
    ic.z *= fr * ic.x;
  }
  return ic;
}

// applyVelocityChange, contact.go:447-494 (single lane); velocity and
// rotation changes of both bodies go to x.bc[0..11].
template <class R, class W>
__device__ void apply_velocity_change(const RCtx<R, W>& x, const BatchView<R>& v, int w, int k) {
  const int bb = x.cb[k];
  const int b0 = body0_of(bb), b1 = body1_of(bb);
  const m3<R> C = x.basis(k);
  v3<R> ic;
  if (x.Cf(W_FRIC, k) == (R)0) {
    // calculateFrictionlessImpulse, contact.go:496-531
    v3<R> d = cross(x.Cv(W_R0X, k), x.Cv(W_NX, k));
    d = mulv(x.iit(b0), d);
    d = cross(d, x.Cv(W_R0X, k));
    R dvel = dot(d, x.Cv(W_NX, k));
    dvel += x.Bf(18, b0);
    if (b1 < 0) {
      atomicOr(&v.world_status[w], ST_FRICTIONLESS_NIL);
      atomicOr(v.status, ST_FRICTIONLESS_NIL);
    }
    ic = V<R>(x.Cf(W_DDV, k) / dvel, (R)0, (R)0);
  } else {
    ic = friction_impulse(x, k, b0, b1, C);
  }
  const v3<R> imp = mulv(C, ic);
  const R z = (R)0;
  v3<R> vc0 = V<R>(z, z, z), vc1 = V<R>(z, z, z), rc1 = V<R>(z, z, z);
  v3<R> rc0 = mulv(x.iit(b0), cross(x.Cv(W_R0X, k), imp));
  add_scaled(vc0, imp, x.Bf(18, b0));
  x.Bf(0, b0) += vc0.x; x.Bf(1, b0) += vc0.y; x.Bf(2, b0) += vc0.z;
  x.Bf(3, b0) += rc0.x; x.Bf(4, b0) += rc0.y; x.Bf(5, b0) += rc0.z;
  if (b1 >= 0) {
    rc1 = mulv(x.iit(b1), cross(imp, x.Cv(W_R1X, k)));
    add_scaled(vc1, imp, -x.Bf(18, b1));
    x.Bf(0, b1) += vc1.x; x.Bf(1, b1) += vc1.y; x.Bf(2, b1) += vc1.z;
    x.Bf(3, b1) += rc1.x; x.Bf(4, b1) += rc1.y; x.Bf(5, b1) += rc1.z;
  }
  x.bc[0] = vc0.x; x.bc[1] = vc0.y; x.bc[2] = vc0.z;
  x.bc[3] = vc1.x; x.bc[4] = vc1.y; x.bc[5] = vc1.z;
  x.bc[6] = rc0.x; x.bc[7] = rc0.y; x.bc[8] = rc0.z;
  x.bc[9] = rc1.x; x.bc[10] = rc1.y; x.bc[11] = rc1.z;
}

template <class R, class W> __host__ __device__ inline size_t rs_smem_bytes(int nbs, int cs) {
  size_t b = (size_t)7 * nbs * sizeof(W);
  b += (size_t)20 * nbs * sizeof(R);
  b += (size_t)W_NROWS * cs * sizeof(R);
  b += 16 * sizeof(R);
  b += (size_t)cs * sizeof(int);
  b += (size_t)((nbs + 15) & ~15);
  return b;
}

// One warp per world (one warp per CTA), worlds pulled from queue[1].
template <class R, class W>
__global__ void __launch_bounds__(32) k_resolve(BatchView<R> v, int nbs, int cs, R dt) {
  extern __shared__ __align__(128) unsigned char smem[];
  RCtx<R, W> x;
  x.nbs = nbs;
  x.dt = dt;
  x.bw = reinterpret_cast<W*>(smem);
  x.br = reinterpret_cast<R*>(x.bw + 7 * nbs);
  R* cw_s = x.br + 20 * nbs;
  x.bc = cw_s + (size_t)W_NROWS * cs;
  int* cb_s = reinterpret_cast<int*>(x.bc + 16);
  x.aw = reinterpret_cast<uint8_t*>(cb_s + cs);
  const int lane = threadIdx.x;
  const long long S = v.nb_pad;
  for (;;) {
    unsigned qi = 0;
    if (lane == 0) qi = atomicAdd(&v.queue[1], 1u);
    qi = __shfl_sync(FULL, qi, 0);
    if (qi >= (unsigned)v.num_worlds) break;
    const int w = v.order[qi];
    const int n = v.body_count[w];
    const int bstart = v.body_start[w];
    int C = v.contact_count[w];
    const int cap = v.contact_cap[w];
    if (C > cap) C = cap;  // the world is already flagged ST_CAPACITY
    if (lane == 0) {
      v.pos_iters[w] = 0;
      v.vel_iters[w] = 0;
    }
    if (C == 0 || !(dt > (R)0)) continue;  // ResolveContacts guards, contact.go:210-212
    if (n > nbs) {
      if (lane == 0) {
        v.world_status[w] |= ST_BODY_LIMIT;
        atomicOr(v.status, ST_BODY_LIMIT);
      }
      continue;
    }
    // bodies -> shared memory
    for (int i = lane; i < n; i += 32) {
      const long long g = bstart + i;
      x.P(0, i) = (W)v.body[B_PX * S + g];
      x.P(1, i) = (W)v.body[B_PY * S + g];
      x.P(2, i) = (W)v.body[B_PZ * S + g];
      x.P(3, i) = (W)v.body[B_QW * S + g];
      x.P(4, i) = (W)v.body[B_QX * S + g];
      x.P(5, i) = (W)v.body[B_QY * S + g];
      x.P(6, i) = (W)v.body[B_QZ * S + g];
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        x.Bf(r, i) = v.body[(B_VX + r) * S + g];
        x.Bf(3 + r, i) = v.body[(B_RX + r) * S + g];
        x.Bf(6 + r, i) = v.body[(B_LX + r) * S + g];
      }
#pragma unroll
      for (int r = 0; r < 9; ++r) x.Bf(9 + r, i) = v.body[(B_IW0 + r) * S + g];
      x.Bf(18, i) = v.body[B_INVM * S + g];
      x.Bf(19, i) = v.body[B_MOTION * S + g];
      x.aw[i] = v.awake[g];
    }
    const long long cst = v.contact_start[w];
    if (C <= cs) {
      x.cw = cw_s;
      x.cb = cb_s;
      x.cst = cs;
    } else {
      x.cw = v.work + cst;
      x.cb = v.work_bodies + cst;
      x.cst = v.nc_total;
    }
    __syncwarp();
    for (int k = lane; k < C; k += 32) prepare_contact(x, v, cst + k, k);
    __syncwarp();
    const int max_it = v.max_iterations >= 0 ? v.max_iterations : C * v.iter_mult;
    // ---------------- adjustPositions, contact.go:231-283
    int used = 0;
    const R peps = (R)0.01;
    while (used < max_it) {
      auto best = key_of(peps, peps);
      int bidx = 0x7fffffff;
      for (int k = lane; k < C; k += 32) {
        auto key = key_of(x.Cf(W_PEN, k), peps);
        if (key > best) {
          best = key;
          bidx = k;
        }
      }
      const int idx = warp_first_max(best, bidx);
      if (idx < 0) break;
      if (lane == 0) {
        match_awake(x, x.cb[idx]);
        apply_position_change(x, v, bstart, idx, x.Cf(W_PEN, idx));
      }
      __syncwarp();
      const int rb = x.cb[idx];
      const int d0 = body0_of(rb), d1 = body1_of(rb);
      for (int k = lane; k < C; k += 32) {
        const int bb = x.cb[k];
        const int kb[2] = {body0_of(bb), body1_of(bb)};
        if (kb[0] != d0 && kb[0] != d1 && kb[1] != d0 && kb[1] != d1) continue;
        const v3<R> n = x.Cv(W_NX, k);
        R pen = x.Cf(W_PEN, k);
#pragma unroll
        for (int b = 0; b < 2; ++b) {
          if (kb[b] < 0) continue;
          const v3<R> r = b == 0 ? x.Cv(W_R0X, k) : x.Cv(W_R1X, k);
#pragma unroll
          for (int d = 0; d < 2; ++d) {
            if (kb[b] == (d == 0 ? d0 : d1)) {
              v3<R> dp = cross(V<R>(x.bc[6 + 3 * d], x.bc[7 + 3 * d], x.bc[8 + 3 * d]), r);
              add(dp, V<R>(x.bc[3 * d], x.bc[3 * d + 1], x.bc[3 * d + 2]));
              const R sign = b == 0 ? (R)-1 : (R)1;
              pen += dot(dp, n) * sign;
            }
          }
        }
        x.Cf(W_PEN, k) = pen;
      }
      __syncwarp();
      ++used;
    }
    const int pos_used = used;
    // ---------------- adjustVelocities, contact.go:388-445
    used = 0;
    const R veps = (R)0.01;
    while (used < max_it) {
      auto best = key_of(veps, veps);
      int bidx = 0x7fffffff;
      for (int k = lane; k < C; k += 32) {
        auto key = key_of(x.Cf(W_DDV, k), veps);
        if (key > best) {
          best = key;
          bidx = k;
        }
      }
      const int idx = warp_first_max(best, bidx);
      if (idx < 0) break;
      if (lane == 0) {
        match_awake(x, x.cb[idx]);
        apply_velocity_change(x, v, w, idx);
      }
      __syncwarp();
      const int rb = x.cb[idx];
      const int d0 = body0_of(rb), d1 = body1_of(rb);
      for (int k = lane; k < C; k += 32) {
        const int bb = x.cb[k];
        const int kb[2] = {body0_of(bb), body1_of(bb)};
        if (kb[0] != d0 && kb[0] != d1 && kb[1] != d0 && kb[1] != d1) continue;
        bool touched = false;
        m3<R> Ck = x.basis(k);
        v3<R> cv = x.Cv(W_CVX, k);
#pragma unroll
        for (int b = 0; b < 2; ++b) {
          if (kb[b] < 0) continue;
          const v3<R> r = b == 0 ? x.Cv(W_R0X, k) : x.Cv(W_R1X, k);
#pragma unroll
          for (int d = 0; d < 2; ++d) {
            if (kb[b] == (d == 0 ? d0 : d1)) {
              v3<R> dv = cross(V<R>(x.bc[6 + 3 * d], x.bc[7 + 3 * d], x.bc[8 + 3 * d]), r);
              add(dv, V<R>(x.bc[3 * d], x.bc[3 * d + 1], x.bc[3 * d + 2]));
              const R sign = b == 1 ? (R)-1 : (R)1;
              v3<R> t = mulv_t(Ck, dv);
              mul_with(t, sign);
              add(cv, t);
              touched = true;
            }
          }
        }
        if (touched) {
          x.setCv(W_CVX, k, cv);
          x.Cf(W_DDV, k) = desired_dv(x, k);
        }
      }
      __syncwarp();
      ++used;
    }
    if (lane == 0) {
      v.pos_iters[w] = pos_used;
      v.vel_iters[w] = used;
      atomicAdd(&v.counters[1], (unsigned long long)pos_used);
      atomicAdd(&v.counters[2], (unsigned long long)used);
      atomicAdd(&v.counters[3], (unsigned long long)C);
    }
    if (v.contact_writeback) {
      // the caller's Contact values after ResolveContacts (penetration,
      // swapped bodies and normal of calculateInternals)
      const long long CS = v.nc_total;
      for (int k = lane; k < C; k += 32) {
        R* o = v.contact + cst + k;
        o[C_NX * CS] = x.Cf(W_NX, k);
        o[C_NY * CS] = x.Cf(W_NY, k);
        o[C_NZ * CS] = x.Cf(W_NZ, k);
        o[C_PEN * CS] = x.Cf(W_PEN, k);
        v.contact_bodies[cst + k] = x.cb[k];
      }
    }
    // bodies -> global
    for (int i = lane; i < n; i += 32) {
      const long long g = bstart + i;
      v.body[B_PX * S + g] = (R)x.P(0, i);
      v.body[B_PY * S + g] = (R)x.P(1, i);
      v.body[B_PZ * S + g] = (R)x.P(2, i);
      v.body[B_QW * S + g] = (R)x.P(3, i);
      v.body[B_QX * S + g] = (R)x.P(4, i);
      v.body[B_QY * S + g] = (R)x.P(5, i);
      v.body[B_QZ * S + g] = (R)x.P(6, i);
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        v.body[(B_VX + r) * S + g] = x.Bf(r, i);
        v.body[(B_RX + r) * S + g] = x.Bf(3 + r, i);
      }
#pragma unroll
      for (int r = 0; r < 9; ++r) v.body[(B_IW0 + r) * S + g] = x.Bf(9 + r, i);
      v.body[B_MOTION * S + g] = x.Bf(19, i);
      v.awake[g] = x.aw[i];
    }
    __syncwarp();
  }
}

}  // namespace cz
