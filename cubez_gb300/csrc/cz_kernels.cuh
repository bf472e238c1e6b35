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

// RigidBody.Integrate + CalculateDerivedData of body row i
// (rigidbody.go:213-299), in place in the batch rows.
template <class R, class W>
__device__ __forceinline__ void integrate_body(const BatchView<R>& v, long long i, R dt, R sleep_bias) {
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
  qnormalize_island<R, W>(qw);
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

template <class R, class W>
__global__ void __launch_bounds__(256, sizeof(R) == 4 ? 4 : 0) k_integrate(BatchView<R> v, R dt, R sleep_bias) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= v.nb_pad) return;
  integrate_body<R, W>(v, i, dt, sleep_bias);
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
  // colliders.go:417-421; the precision form also takes the fallback when the
  // centre needed no clamping (float32 rounding of the round trip exceeds the
  // reference's absolute 1e-14)
  if (real_equal<R>(mag(nrm), (R)0) || (sizeof(R) < sizeof(double) && dist == (R)0)) {
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

// Whether the float32 culls rule out any contact of the ordered pair (i, j).
template <class R> __device__ __forceinline__ bool pair_culled(const NPTile<R>& tl, int i, int j) {
  const int si = tl.shape[i], sj = tl.shape[j];
  const Cull cl{tl.cull, tl.nbs};
  if (sj == 0) return si == 0 ? cl.spheres(i, j) : cl.box_sphere(i, j);
  return si == 0 ? cl.box_sphere(j, i) : cl.boxes(i, j);
}

// One ordered pair (i, j) past the culls: CheckForCollisions(collider i,
// collider j) (colliders.go:718-747 with the forwarding of colliders.go:209-213).
template <class R>
__device__ int pair_full(const NPTile<R>& tl, int i, int j, const BatchView<R>& v, int bstart, NPContact<R>& c,
                         uint32_t& err) {
  const int si = tl.shape[i], sj = tl.shape[j];
  if (si == 0 && sj == 0)
    return sphere_sphere(V<R>(tl.T[9 * tl.nbs + i], tl.T[10 * tl.nbs + i], tl.T[11 * tl.nbs + i]), tl.radius(i), i,
                         V<R>(tl.T[9 * tl.nbs + j], tl.T[10 * tl.nbs + j], tl.T[11 * tl.nbs + j]), tl.radius(j), j, c);
  if (si != 0 && sj != 0) return cube_cube(tl.xform(i), tl.half(i), i, tl.xform(j), tl.half(j), j, c, err);
  // a cube and a sphere, in either order: one call site
  const int bx = si != 0 ? i : j, sp = si != 0 ? j : i;
  return cube_sphere(tl.xform(bx), tl.half(bx), bx, tl.xform(sp), tl.radius(sp), sp,
                     v.body + (long long)B_VX * v.nb_pad + bstart + sp, v.nb_pad, c);
}

template <class R>
__device__ __forceinline__ int pair_test(const NPTile<R>& tl, int i, int j, const BatchView<R>& v, int bstart,
                                         NPContact<R>& c, uint32_t& err) {
  return pair_culled(tl, i, j) ? 0 : pair_full(tl, i, j, v, bstart, c, err);
}

// Whether a float32 cull rules out any contact of body i with the half-space
// n.x <= offset: a sphere's d = n.c - r (colliders.go:190-192), a cube's
// n.c - (projected half-size) with the projection at most |n| |h|_2
// (colliders.go:750-770); the margin is the pair culls' (1 mm + 1e-5 of the
// magnitudes).  A cube with a non-rigid Offset has an infinite radius.
template <class R> __device__ __forceinline__ bool plane_culled(const NPTile<R>& tl, int i, const BatchView<R>& v) {
  const float nx = (float)v.plane_nx, ny = (float)v.plane_ny, nz = (float)v.plane_nz, off = (float)v.plane_offset;
  const float cx = tl.cull[i], cy = tl.cull[tl.nbs + i], cz = tl.cull[2 * tl.nbs + i];
  const float d = nx * cx + ny * cy + nz * cz;
  const float nlen = sqrtf(nx * nx + ny * ny + nz * nz) * 1.0001f;
  const float r = tl.shape[i] == 0 ? tl.cull[3 * tl.nbs + i] : tl.cull[3 * tl.nbs + i] * nlen;
  const float scale = 1.f + (fabsf(cx) + fabsf(cy) + fabsf(cz)) * nlen + fabsf(off);
  return d - r > off + 1e-3f + 1e-5f * scale;  // false for NaN and infinite radii
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

// Units past the culls held for their full tests: room for a round of culls
// (up to 1024 units) on top of a partly filled list, and at least one body's
// units (the grid path lists a body's units together).
constexpr int kSurvivors = 1280;
// np_flush's scratch for a CTA of bd threads: the chunk's order by kind of
// test, its counts, and per-kind counts of each warp (6 kinds x 8 warps)
__host__ __device__ constexpr int np_sort_ints(int bd) { return 2 * bd + 64; }
__host__ __device__ inline int np_surv_cap(int nbs) { return nbs + 1 > kSurvivors ? ((nbs + 32) & ~31) : kSurvivors; }

template <class R> __host__ __device__ inline size_t np_smem_bytes(int nbs) {
  size_t b = 16;                                  // mbarrier + pad
  b += (size_t)(11 + 12) * nbs * sizeof(R);       // staged rows + transforms
  b += (size_t)nbs * sizeof(int);                 // shape
  b += (size_t)5 * nbs * sizeof(float);           // cull data
  b += 2 * 33 * sizeof(int);                      // scan scratch (double-buffered) + world id + wait outcome
  b += (size_t)np_surv_cap(nbs) * sizeof(int);    // units past the culls, awaiting their full tests
  b += (size_t)np_sort_ints(256) * sizeof(int);   // np_flush's sort of a chunk by kind of test
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

// The full tests of the listed units (unit u = i * n + k: k = 0 the
// half-space, else the pair with j = k - 1, skipping i), in chunks of the
// CTA's size, emitting their contacts in list order at out onwards.  Within a
// chunk the units are taken in order of their kind of test (half-space with
// a sphere, with a cube; sphere-sphere, sphere-cube, cube-cube), stably, so
// the lanes of a warp mostly run one test's code; the counts are then
// scanned in list order, so every contact lands where the list order puts
// it (the reference's contact order).  sortw: np_sort_ints(blockDim.x) ints.
template <class R>
__device__ void np_flush(const NPTile<R>& tl, const BatchView<R>& v, int bstart, int n, long long cs, int cap,
                         const int* surv, int nsurv, int* scan, int& parity, int& out, uint32_t& err, int* sortw) {
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, bd = blockDim.x, nwarps = (bd + 31) >> 5;
  int* perm = sortw;
  int* cntb = sortw + bd;
  int* wcnt = sortw + 2 * bd;  // [kind * 8 + warp]
  for (int sb = 0; sb < nsurv; sb += bd) {
    const int m = nsurv - sb < bd ? nsurv - sb : bd;
    int key = 5;  // no unit
    if (tid < m) {
      const int uu = surv[sb + tid];
      const int i = uu / n, k = uu - i * n;
      if (k == 0) {
        key = tl.shape[i] != 0 ? 1 : 0;
      } else {
        int j = k - 1;
        if (j >= i) ++j;
        key = 2 + (tl.shape[i] != 0 ? 1 : 0) + (tl.shape[j] != 0 ? 1 : 0);
      }
    }
    int rank = 0;
#pragma unroll
    for (int q = 0; q < 6; ++q) {
      const unsigned bal = __ballot_sync(FULL, key == q);
      if (key == q) rank = __popc(bal & ((1u << lane) - 1u));
      if (lane == 0) wcnt[q * 8 + wid] = __popc(bal);
    }
    __syncthreads();
    int dst = rank;
    for (int q = 0; q < key; ++q)
      for (int w2 = 0; w2 < nwarps; ++w2) dst += wcnt[q * 8 + w2];
    for (int w2 = 0; w2 < wid; ++w2) dst += wcnt[key * 8 + w2];
    perm[dst] = tid;
    __syncthreads();
    const int src = perm[tid];  // this thread tests the chunk's unit src
    int cnt = 0, i = 0, k = 0;
    NPContact<R> c;
    if (src < m) {
      const int uu = surv[sb + src];
      i = uu / n;
      k = uu - i * n;
      if (k == 0) {
        cnt = plane_contacts<R>(tl, i, v, nullptr, nullptr, 0, 0);
      } else {
        int j = k - 1;
        if (j >= i) ++j;
        cnt = pair_full<R>(tl, i, j, v, bstart, c, err);
      }
    }
    cntb[src] = cnt;
    __syncthreads();
    int excl, total;
    np_chunk_scan(cntb[tid], scan, parity, &excl, &total);  // list order
    parity ^= 1;
    cntb[tid] = excl;
    __syncthreads();
    np_emit<R>(tl, v, cs, cap, out + cntb[src], cnt, i, k == 0, c);
    out += total;
    __syncthreads();  // perm and cntb are reused by the next chunk
  }
}

// ---- broadphase: a uniform grid over a large world's bodies
//
// A pair (i, j) passes the float32 culls only if its centres are within
// reach_i + reach_j + 1 mm + 1e-5 (1 + |c_i|_1 + |c_j|_1), with reach = the
// larger of 1.1 |h|_2 and |h|_1 for a box, 3 r for a sphere (the thresholds
// of Cull).  With cells at least that wide for every pair of the world, the
// pairs the culls keep are all between neighbouring cells: the grid drops
// only pairs the culls reject.  Each body's kept units are listed in
// ascending unit order and bodies in index order, so the contact list is the
// all-pairs path's, bit for bit.

// Grid scratch inside the staged position / orientation rows, which are
// dead once the collider transforms are built.
struct NPGrid {
  float* red;   // [8 warps][8] block reductions
  int* info;    // [8]: ok, gx, gy, gz, ncells, last list length
  float* finfo; // [4]: origin xyz, cell size
  int* cell;    // [cells_cap + 1] counts, then cursor / end of each cell
  int* sorted;  // [n] bodies ordered by cell
  int* cellof;  // [n] linear cell of each body
  int cells_cap;
};

template <class R> __device__ __forceinline__ NPGrid np_grid_scratch(const NPTile<R>& tl) {
  NPGrid g;
  unsigned char* base = reinterpret_cast<unsigned char*>(tl.stage);
  const int words = (int)((size_t)7 * tl.nbs * sizeof(R) / 4);
  g.red = reinterpret_cast<float*>(base);
  g.info = reinterpret_cast<int*>(base) + 64;
  g.finfo = reinterpret_cast<float*>(g.info + 8);
  g.sorted = g.info + 12;
  g.cellof = g.sorted + tl.nbs;
  g.cell = g.cellof + tl.nbs;
  g.cells_cap = words - 76 - 2 * tl.nbs - 1;
  return g;
}

// Block-wide max of 8 floats (NaN in any input gives NaN through the
// comparison trick below: a value that is not >= itself is kept).
__device__ __forceinline__ void np_block_max8(float (&x)[8], float* red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int q = 0; q < 8; ++q)
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
      const float y = __shfl_xor_sync(FULL, x[q], d);
      x[q] = (y > x[q] || y != y) ? y : x[q];
    }
  if (lane == 0)
#pragma unroll
    for (int q = 0; q < 8; ++q) red[wid * 8 + q] = x[q];
  __syncthreads();
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    float m = red[q];
    for (int k = 1; k < nw; ++k) {
      const float y = red[k * 8 + q];
      m = (y > m || y != y) ? y : m;
    }
    x[q] = m;
  }
  __syncthreads();
}

// Builds the grid of one world; false (uniform over the CTA) when it would
// not help or cannot be sized: non-finite centres or radii (a non-rigid
// Offset's infinite radius included), or more cells than the scratch holds.
template <class R> __device__ bool np_grid_build(const NPTile<R>& tl, int n, const NPGrid& g, int* scan, int& parity) {
  const int nbs = tl.nbs;
  float x[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) x[q] = -__int_as_float(0x7f800000);
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const float cx = tl.cull[i], cy = tl.cull[nbs + i], cz = tl.cull[2 * nbs + i];
    const float rb = tl.cull[3 * nbs + i], rl = tl.cull[4 * nbs + i];
    const float reach = tl.shape[i] == 0 ? 3.f * rb : fmaxf(1.1f * rb, rl);
    const float fin = (isfinite(cx) && isfinite(cy) && isfinite(cz) && isfinite(reach)) ? 0.f : 1.f;
    // max of: the centres (the box's upper corner), their negations (the
    // lower corner), the reach, non-finite flag
    const float v8[8] = {cx, cy, cz, -cx, -cy, -cz, reach, fin};
#pragma unroll
    for (int q = 0; q < 8; ++q) x[q] = (v8[q] > x[q] || v8[q] != v8[q]) ? v8[q] : x[q];
  }
  np_block_max8(x, g.red);
  if (threadIdx.x == 0) {
    int ok = x[7] == 0.f && x[6] == x[6];
    // |c|_1 of every centre is at most the larger corner's per axis
    const float m1 = fmaxf(fabsf(x[0]), fabsf(x[3])) + fmaxf(fabsf(x[1]), fabsf(x[4])) +
                     fmaxf(fabsf(x[2]), fabsf(x[5]));
    // cell size: every kept pair is within 2 * max reach + the culls' margin
    const float L = (2.f * x[6] + 1e-3f + 1e-5f * (1.f + 2.f * m1)) * 1.001f + 1e-6f;
    const float ox = -x[3], oy = -x[4], oz = -x[5];
    int gx = 0, gy = 0, gz = 0;
    if (ok && L > 0.f) {
      const float ex = (x[0] - ox) / L, ey = (x[1] - oy) / L, ez = (x[2] - oz) / L;
      ok = ex < 1e6f && ey < 1e6f && ez < 1e6f;
      if (ok) {
        gx = (int)ex + 1;
        gy = (int)ey + 1;
        gz = (int)ez + 1;
        ok = (long long)gx * gy * gz <= g.cells_cap;
      }
    } else {
      ok = 0;
    }
    g.info[0] = ok;
    g.info[1] = gx;
    g.info[2] = gy;
    g.info[3] = gz;
    g.info[4] = gx * gy * gz;
    g.finfo[0] = ox;
    g.finfo[1] = oy;
    g.finfo[2] = oz;
    g.finfo[3] = L;
  }
  __syncthreads();
  if (!g.info[0]) return false;
  const int gx = g.info[1], gy = g.info[2], gz = g.info[3], nc = g.info[4];
  const float ox = g.finfo[0], oy = g.finfo[1], oz = g.finfo[2], L = g.finfo[3];
  for (int c = threadIdx.x; c <= nc; c += blockDim.x) g.cell[c] = 0;
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int cx = min((int)((tl.cull[i] - ox) / L), gx - 1);
    const int cy = min((int)((tl.cull[nbs + i] - oy) / L), gy - 1);
    const int cz = min((int)((tl.cull[2 * nbs + i] - oz) / L), gz - 1);
    const int c = (cz * gy + cy) * gx + cx;
    g.cellof[i] = c;
    atomicAdd(&g.cell[c], 1);
  }
  __syncthreads();
  // exclusive scan of the counts: cell[c] = first slot of cell c
  int run = 0;
  for (int b0 = 0; b0 < nc; b0 += blockDim.x) {
    const int c = b0 + threadIdx.x;
    const int cnt = c < nc ? g.cell[c] : 0;
    int excl, total;
    np_chunk_scan(cnt, scan, parity, &excl, &total);
    parity ^= 1;
    if (c < nc) g.cell[c] = run + excl;
    run += total;
  }
  __syncthreads();
  // scatter; afterwards cell[c] is the end of cell c (the start of c + 1)
  for (int i = threadIdx.x; i < n; i += blockDim.x) g.sorted[atomicAdd(&g.cell[g.cellof[i]], 1)] = i;
  __syncthreads();
  return true;
}

// Body i's units past the culls from its 27 neighbouring cells: counted, or
// written at dst (plane unit, then the pairs, unsorted).
template <class R>
__device__ int np_grid_units(const NPTile<R>& tl, const BatchView<R>& v, const NPGrid& g, int n, int i, int* dst) {
  int cnt = 0;
  if (!plane_culled(tl, i, v)) {
    if (dst) dst[cnt] = i * n;
    ++cnt;
  }
  const int gx = g.info[1], gy = g.info[2], gz = g.info[3];
  const int c = g.cellof[i];
  const int cx = c % gx, cy = (c / gx) % gy, cz = c / (gx * gy);
  for (int dz = -1; dz <= 1; ++dz) {
    if (cz + dz < 0 || cz + dz >= gz) continue;
    for (int dy = -1; dy <= 1; ++dy) {
      if (cy + dy < 0 || cy + dy >= gy) continue;
      for (int dx = -1; dx <= 1; ++dx) {
        if (cx + dx < 0 || cx + dx >= gx) continue;
        const int nc = ((cz + dz) * gy + cy + dy) * gx + cx + dx;
        const int s0 = nc == 0 ? 0 : g.cell[nc - 1], s1 = g.cell[nc];
        for (int s = s0; s < s1; ++s) {
          const int j = g.sorted[s];
          if (j == i || pair_culled(tl, i, j)) continue;
          if (dst) dst[cnt] = i * n + (j < i ? j + 1 : j);
          ++cnt;
        }
      }
    }
  }
  return cnt;
}

// The narrowphase of world w, its bodies' tile built: the ordered units
// culled, the kept ones listed (scap of them at a time) and tested, the
// contacts emitted in the reference's order; sets the world's contact count.
// Every thread of the CTA calls it.
template <class R, bool GRID>
__device__ void np_world(const NPTile<R>& tl, const BatchView<R>& v, int w, int n, int bstart, int* scan,
                         int& chunk_parity, int* surv, int scap) {
  const int tid = threadIdx.x;
  const long long cs = v.contact_start[w];
  const int cap = v.contact_cap[w];
  const int U = n * n;  // ordered units: for body i, the half-space (k = 0), then k - 1 = j skipping i
  int out = 0, nsurv = 0;
  uint32_t err = 0;
  const NPGrid g = np_grid_scratch(tl);
  if (GRID && v.grid_min_bodies > 0 && n >= v.grid_min_bodies && np_grid_build(tl, n, g, scan, chunk_parity)) {
    // Grid: each body's kept units (counted, then listed and sorted), as
    // many bodies at a time as the list holds, then their full tests.
    for (int ib = 0; ib < n;) {
      const int i = ib + tid;
      const int cnt = i < n ? np_grid_units(tl, v, g, n, i, nullptr) : 0;
      int excl, total;
      np_chunk_scan(cnt, scan, chunk_parity, &excl, &total);
      chunk_parity ^= 1;
      const bool fits = i < n && excl + cnt <= scap;  // a prefix of the bodies: at least body ib
      const int m = __syncthreads_count(fits);
      if (fits) {
        int* d = surv + excl;
        np_grid_units(tl, v, g, n, i, d);
        for (int a = 1; a < cnt; ++a) {  // ascending unit order (the plane unit, k = 0, first)
          const int key = d[a];
          int b = a - 1;
          while (b >= 0 && d[b] > key) {
            d[b + 1] = d[b];
            --b;
          }
          d[b + 1] = key;
        }
        if (tid == m - 1) g.info[5] = excl + cnt;
      }
      __syncthreads();
      nsurv = g.info[5];
      np_flush(tl, v, bstart, n, cs, cap, surv, nsurv, scan, chunk_parity, out, err, surv + scap);
      __syncthreads();
      ib += m;
    }
  } else {
    // All pairs: the culls run over every unit, upt consecutive units per
    // thread and one scan per round; the units they keep are listed in unit
    // order and get their full tests in chunks of the CTA's size, so the
    // lanes of a warp run the costly tests together.  Counting, scanning and
    // emitting in list order keeps the reference's contact order.
    const int bd = blockDim.x;
    int upt = (scap - bd) / bd;
    upt = upt < 1 ? 1 : (upt > 8 ? 8 : upt);
    const int round = bd * upt;  // at most scap - bd: the list never overflows
    for (int base = 0; base < U; base += round) {
      const int u0 = base + tid * upt;
      unsigned keep = 0;
      if (u0 < U) {
        int i = u0 / n, k = u0 - i * n;
        for (int q = 0; q < upt && u0 + q < U; ++q) {
          int j = k - 1;
          if (j >= i) ++j;
          if (k == 0 ? !plane_culled(tl, i, v) : !pair_culled(tl, i, j)) keep |= 1u << q;
          if (++k == n) {
            k = 0;
            ++i;
          }
        }
      }
      int excl, total;
      np_chunk_scan(__popc(keep), scan, chunk_parity, &excl, &total);
      chunk_parity ^= 1;
      for (int o = nsurv + excl; keep; keep &= keep - 1) surv[o++] = u0 + __ffs(keep) - 1;
      nsurv += total;
      if (nsurv <= scap - round && base + round < U) continue;
      __syncthreads();
      np_flush(tl, v, bstart, n, cs, cap, surv, nsurv, scan, chunk_parity, out, err, surv + scap);
      nsurv = 0;
      __syncthreads();
    }
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

// GRID = false compiles the all-pairs path alone (worlds too small for the
// grid), so its registers and occupancy stay those of that path; in float32
// it is bounded to 64 registers (8 CTAs of 128 threads per SM instead of 6;
// a few registers spill), which hides more of its barrier waits.
template <class R, bool GRID>
__global__ void __launch_bounds__(256, sizeof(R) == 4 && !GRID ? 4 : 0) k_narrowphase(BatchView<R> v, int nbs) {
  extern __shared__ __align__(128) unsigned char smem[];
  unsigned long long* bar = reinterpret_cast<unsigned long long*>(smem);
  NPTile<R> tl;
  tl.nbs = nbs;
  tl.stage = reinterpret_cast<R*>(smem + 16);
  tl.T = tl.stage + 11 * nbs;
  tl.shape = reinterpret_cast<int*>(tl.T + 12 * nbs);
  tl.cull = reinterpret_cast<float*>(tl.shape + nbs);
  int* scan = reinterpret_cast<int*>(tl.cull + 5 * nbs);  // [2][32] + [64] world id + [65] wait outcome
  int* surv = scan + 66;                                   // [kSurvivors] units past the culls
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
      mbar_expect_tx(bar, rb * 11u + (unsigned)(n4 * sizeof(int)) + (unsigned)v.wait_extra_tx);
#pragma unroll 1
      for (int r = 0; r < 11; ++r) bulk_g2s(tl.stage + r * nbs, v.body + (long long)r * v.nb_pad + bstart, rb, bar);
      bulk_g2s(tl.shape, v.shape + bstart, (unsigned)(n4 * sizeof(int)), bar);
    }
    if (n4 > 0) {
      // Thread 0 waits, bounded, and decides for the CTA; the others then
      // observe the completed phase themselves (their acquire of the copies).
      if (tid == 0) scan[65] = mbar_wait(bar, phase, v.wait_limit) ? 1 : 0;
      __syncthreads();
      const bool ok = scan[65] != 0;
      if (!ok) {
        // Give up on this CTA's worlds (the copies are a few KB, so this
        // signals a fault) and report it.  The copies issued may still be
        // landing in this CTA's shared memory: one more bounded wait for
        // them before the CTA ends.
        if (tid == 0) {
          v.world_status[w] |= ST_TIMEOUT;
          atomicOr(v.status, ST_TIMEOUT);
          mbar_wait(bar, phase, v.wait_limit);
        }
        __syncthreads();
        return;
      }
      if (tid != 0) mbar_wait(bar, phase, v.wait_limit);
      phase ^= 1u;
    }
    np_build_tile(tl, n, v.offset ? v.offset + bstart : nullptr, v.nb_pad);
    __syncthreads();
    np_world<R, GRID>(tl, v, w, n, bstart, scan, chunk_parity, surv, np_surv_cap(nbs));
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
