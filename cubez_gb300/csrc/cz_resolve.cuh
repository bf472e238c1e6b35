// ResolveContacts (contact.go:204-445) for batches of worlds.
//
// One warp holds 32 / G worlds; the G lanes of a group own one world.  Within
// a group the contacts are lane-strided: the argmax is a G-lane butterfly
// (warp reductions for G = 32) whose tie-break is the reference's
// first-maximum rule, and the per-iteration update of every contact touching
// the two resolved bodies is lane-parallel (gathered to those contacts in the
// float64 form).  The sequential part of an iteration (applyPositionChange
// on lanes 0 and 1, one body each; applyVelocityChange on the group leader,
// or on six lanes in the float64 form) runs for all groups at once, so each
// instruction of that chain serves 32 / G worlds: on GB300 a float64 warp
// instruction costs the same pipe time whatever its active mask, so packing
// worlds into a warp divides the float64 cost of the plain form and of the
// precision form's islands by 32 / G; with 16 or 32 lanes per world the
// position and orientation updates are spread over 14 lanes of the group as
// well (apply_position_change).  The friction solve's matrices do not change
// during adjustVelocities and are computed once per contact, off the chain
// (friction_prepare).  With one world per warp in float32 a CTA runs four
// independent warps (rs_wpc).
//
// Groups of a warp advance in lockstep rounds; a group whose world is done
// idles until the warp's last world finishes its phase.  Worlds are queued in
// decreasing cost, so the worlds sharing a warp have similar iteration counts.
//
// Also here: k_warm_features (the learned warm start's features, tensor-core
// inference and plan, launched before k_resolve) and the shared pieces of
// k_resolve_big (cz_resolve_big.cuh).
#pragma once
#include "cz_layout.cuh"
#include "cz_math.cuh"
#include "cz_mlp.cuh"

namespace cz {

// calculateContactBasis's second column, contact.go:114-156: a function of
// the normal alone.
template <class R> __device__ __forceinline__ v3<R> contact_tangent(const v3<R>& n) {
  if (fabs_<R>(n.x) > fabs_<R>(n.y)) {
    const R s = (R)1 / sqrt_<R>(n.z * n.z + n.x * n.x);
    return V<R>(n.z * s, (R)0, n.x * -s);
  }
  const R s = (R)1 / sqrt_<R>(n.z * n.z + n.y * n.y);
  return V<R>((R)0, -n.z * s, n.y * s);
}

template <class R, class W> struct RCtx {
  W* bw;          // [7][nbs]: position xyz, orientation wxyz (island type)
  R* br;          // [20][nbs]: vel 0-2, rot 3-5, lfa * dt 6-8, iitWorld 9-17, invMass 18, motion 19
  uint8_t* aw;    // [nbs] awake
  int nbs;
  R* cw;          // working rows of this world's contacts
  int* cb;        // packed bodies of this world's contacts
  long long cst;  // row stride of cw
  R* bc;          // broadcast scratch [12]
  // warm start / harvest (modes 1, 2): this world's per-body scratch in
  // global memory (row stride wst) and its contacts' impulse rows
  R* save;        // [7]: velocity 0-2, rotation 3-5, motion 6 at the start of adjustVelocities
  R* delta;       // [6]: warm-start velocity and rotation change
  int* wi;        // [WS_NINT] integer rows (WsInt)
  long long wst;
  R* jw;          // impulse rows J0..J2 (row stride jst)
  long long jst;
  R* kw;          // per contact, K_ROW reals: K of the friction solve (inverted in W, kept in R), 9,
                  // then the response matrix's first row, 3
  const R* gmat;  // friction / restitution rows of the contact list (null: 0.9 / 0.1)
  long long gst;
  R dt;
  __device__ __forceinline__ W& P(int c, int i) const { return bw[c * nbs + i]; }
  __device__ __forceinline__ R& Bf(int r, int i) const { return br[r * nbs + i]; }
  __device__ __forceinline__ R& Cf(int f, int k) const { return cw[(long long)f * cst + k]; }
  __device__ __forceinline__ R& J(int c, int k) const { return jw[(long long)c * jst + k]; }
  __device__ __forceinline__ R& K(int q, int k) const { return kw[(long long)k * K_ROW + q]; }
  __device__ __forceinline__ R& KD(int q, int k) const { return kw[(long long)k * K_ROW + 9 + q]; }
  __device__ __forceinline__ int& WI(int r, int i) const { return wi[(long long)r * wst + i]; }
  __device__ __forceinline__ R& Save(int r, int i) const { return save[(long long)r * wst + i]; }
  __device__ __forceinline__ R& Delta(int r, int i) const { return delta[(long long)r * wst + i]; }
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
  __device__ __forceinline__ R friction(int k) const { return gmat ? gmat[k] : (R)0.9; }
  __device__ __forceinline__ R restitution(int k) const { return gmat ? gmat[gst + k] : (R)0.1; }
  // contactToWorld: columns normal, tangent y, tangent z; the last is the
  // reference's formula of the first two (contact.go:136-138, 149-151)
  __device__ __forceinline__ m3<R> basis(int k) const {
    const v3<R> n = Cv(W_NX, k);
    const v3<R> ty = stores_tangent<R>() ? Cv(W_TYX, k) : contact_tangent(n);
    m3<R> m;
    m.m[0] = n.x; m.m[1] = n.y; m.m[2] = n.z;
    m.m[3] = ty.x; m.m[4] = ty.y; m.m[5] = ty.z;
    if (fabs_<R>(n.x) > fabs_<R>(n.y)) {
      m.m[6] = n.y * ty.x;
      m.m[7] = n.z * ty.x - n.x * ty.z;
      m.m[8] = -n.y * ty.x;
    } else {
      m.m[6] = n.y * ty.z - n.z * ty.y;
      m.m[7] = -n.x * ty.z;
      m.m[8] = n.x * ty.y;
    }
    return m;
  }
};

// ---------------------------------------------------------------- argmax keys
// Order-preserving keys: key(v) > 0 exactly when v > eps and v is not NaN;
// for such values key order is value order (IEEE bit patterns of positive
// numbers sort like the numbers).
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

// The first maximum over a whole warp by warp reductions (redux.sync): the
// largest key, then the smallest index among the lanes holding it; a 64-bit
// key is reduced by its high half, then its low half.
__device__ __forceinline__ void warp_first_max(unsigned& key, int& idx) {
  const unsigned m = __reduce_max_sync(0xffffffffu, key);
  idx = (int)__reduce_min_sync(0xffffffffu, key == m ? (unsigned)idx : 0xffffffffu);
  key = m;
}
__device__ __forceinline__ void warp_first_max(unsigned long long& key, int& idx) {
  const unsigned hi = (unsigned)(key >> 32), lo = (unsigned)key;
  const unsigned mh = __reduce_max_sync(0xffffffffu, hi);
  const unsigned ml = __reduce_max_sync(0xffffffffu, hi == mh ? lo : 0u);
  idx = (int)__reduce_min_sync(0xffffffffu, (hi == mh && lo == ml) ? (unsigned)idx : 0xffffffffu);
  key = ((unsigned long long)mh << 32) | ml;
}

// Largest key over the G lanes of a group, smallest index among equal keys
// (the first maximum of the reference's scan, contact.go:238-245, 394-402).
template <int G, class K> __device__ __forceinline__ void group_first_max(K& key, int& idx) {
  if constexpr (G == 32) {
    warp_first_max(key, idx);
    return;
  }
#pragma unroll
  for (int off = G / 2; off > 0; off >>= 1) {
    const K ok = __shfl_xor_sync(0xffffffffu, key, off);
    const int oi = __shfl_xor_sync(0xffffffffu, idx, off);
    if (ok > key || (ok == key && oi < idx)) {
      key = ok;
      idx = oi;
    }
  }
}

// calculateDesiredDeltaVelocity, contact.go:87-112, of contact k between
// bodies b0, b1 with normal n and contact velocity x component cvx (the
// callers pass what they hold in registers).
template <class R, class W>
__device__ __forceinline__ R desired_dv_of(const RCtx<R, W>& x, int k, int b0, int b1, const v3<R>& n, R cvx) {
  R vfa = (R)0;
  // rows 6-8 hold LastFrameAcceleration * duration, formed when the body is
  // loaded (the reference's product, once instead of at every use)
  if (x.aw[b0]) vfa += dot(x.Bv(6, b0), n);
  if (b1 >= 0 && x.aw[b1]) vfa -= dot(x.Bv(6, b1), n);
  R rest = x.restitution(k);
  if (fabs_<R>(cvx) < (R)0.25) rest = (R)0;
  return -cvx - rest * (cvx - vfa);
}
template <class R, class W> __device__ __forceinline__ R desired_dv(const RCtx<R, W>& x, int k) {
  const int bb = x.cb[k];
  return desired_dv_of(x, k, body0_of(bb), body1_of(bb), x.Cv(W_NX, k), x.Cf(W_CVX, k));
}

// calculateLocalVelocity, contact.go:158-182
template <class R, class W>
__device__ __forceinline__ v3<R> local_velocity(const RCtx<R, W>& x, int body, const v3<R>& rp, const m3<R>& C) {
  v3<R> vel = cross(x.Bv(3, body), rp);
  add(vel, x.Bv(0, body));
  v3<R> cv = mulv_t(C, vel);
  v3<R> acc = x.Bv(6, body);  // LastFrameAcceleration * duration
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
  x.cb[k] = bb;
  x.setCv(W_NX, k, n);
  if (stores_tangent<R>()) x.setCv(W_TYX, k, contact_tangent(n));  // calculateContactBasis
  const m3<R> C = x.basis(k);
  v3<R> rp0 = p;
  sub(rp0, V<R>((R)(x.P(0, b0)), (R)(x.P(1, b0)), (R)(x.P(2, b0))));
  v3<R> cv = local_velocity(x, b0, rp0, C);
  v3<R> rp1 = V<R>((R)0, (R)0, (R)0);
  if (b1 >= 0) {
    rp1 = p;
    sub(rp1, V<R>((R)(x.P(0, b1)), (R)(x.P(1, b1)), (R)(x.P(2, b1))));
    v3<R> cv1 = local_velocity(x, b1, rp1, C);
    sub(cv, cv1);
  }
  x.Cf(W_PEN, k) = g[C_PEN * S];
  x.setCv(W_R0X, k, rp0);
  x.setCv(W_R1X, k, rp1);
  x.setCv(W_CVX, k, cv);
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
  qnormalize_island<R, W>(qw);
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

// applyPositionChange, contact.go:285-386, by lanes 0 and 1 of a group with
// `on` (every lane of the warp calls it): lane i moves body i, so the two
// bodies' float64 position / quaternion updates run side by side; their
// inertias meet through a shuffle and the total is summed in the reference's
// order (body 0, then body 1).  Each body's operations are the one-lane
// formula's, so results are identical.  Lane i leaves body i's linear and
// angular change in x.bc[3i..3i+2] and x.bc[6+3i..8+3i].
//
// With at least 16 lanes per world, the updates of position and orientation
// are spread over the group: lanes 2-7 add one position component each (body
// (gl-2)/3), lanes 8-15 one quaternion component each (body (gl-8)/4) and
// square it; the quaternion's first lane sums the squares in the reference's
// order and decides the renormalisation (the precision form's island, or
// Normalize in the float64 form), which every component lane applies.  A
// float64 warp instruction costs the pipe the same whatever its active
// lanes, so this takes one float64 add for all fourteen components (seven
// per body on one lane before) and one multiply for the squares, and in the
// precision form each lane converts one value.  The operations on every
// value are the one-lane formula's.
template <class R, class W, int G>
__device__ void apply_position_change(const RCtx<R, W>& x, const BatchView<R>& v, int bstart, int k, bool on, int gl) {
  constexpr bool kSpread = G >= 16;
  const bool mine = on && gl < 2;
  const R z = (R)0;
  int b = -1;
  v3<R> n = V<R>(z, z, z), rp = V<R>(z, z, z);
  R angI = z, linI = z, penetration = z;
  if (mine) {
    const int bb = x.cb[k];
    b = gl == 0 ? body0_of(bb) : body1_of(bb);
    n = x.Cv(W_NX, k);
    rp = gl == 0 ? x.Cv(W_R0X, k) : x.Cv(W_R1X, k);
    penetration = x.Cf(W_PEN, k);
    if (b >= 0) {
      v3<R> a = cross(rp, n);
      a = mulv(x.iit(b), a);
      a = cross(a, rp);
      angI = dot(a, n);
      linI = x.Bf(18, b);
    }
  }
  const R angO = __shfl_sync(0xffffffffu, angI, gl ^ 1, G);
  const R linO = __shfl_sync(0xffffffffu, linI, gl ^ 1, G);
  const int bO = __shfl_sync(0xffffffffu, b, gl ^ 1, G);
  if (!kSpread && !mine) return;
  v3<R> lin = V<R>(z, z, z), ang = V<R>(z, z, z);
  if (mine) {
    const int b0 = gl == 0 ? b : bO, b1 = gl == 0 ? bO : b;
    R total = z;
    if (b0 >= 0) total += (gl == 0 ? linI : linO) + (gl == 0 ? angI : angO);
    if (b1 >= 0) total += (gl == 0 ? linO : linI) + (gl == 0 ? angO : angI);
    if (b >= 0) {
      const R sign = gl != 0 ? (R)-1 : (R)1;
      R am = sign * penetration * (angI / total);
      R lm = sign * penetration * (linI / total);
      v3<R> proj = rp;
      add_scaled(proj, n, -dot(rp, n));
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
      if (am != (R)0) {
        ang = mulv(x.iit(b), cross(rp, n));
        mul_with(ang, am / angI);
      }
      lin = n;
      mul_with(lin, lm);
      if constexpr (!kSpread) {
        // Position.AddScaled(normal, linearMove): product in R, accumulated in W
        x.P(0, b) += cvt_fast<W>(n.x * lm);
        x.P(1, b) += cvt_fast<W>(n.y * lm);
        x.P(2, b) += cvt_fast<W>(n.z * lm);
        q4<W> q{x.P(3, b), x.P(4, b), x.P(5, b), x.P(6, b)};
        add_scaled_vector_island<R, W>(q, ang);
        qnormalize_island<R, W>(q);
        x.P(3, b) = q.w; x.P(4, b) = q.x; x.P(5, b) = q.y; x.P(6, b) = q.z;
        if (!x.aw[b]) {
          // CalculateDerivedData reads the stored (R-rounded) orientation
          x.P(3, b) = (W)(R)q.w; x.P(4, b) = (W)(R)q.x; x.P(5, b) = (W)(R)q.y; x.P(6, b) = (W)(R)q.z;
          derive_asleep(x, v, bstart, b);
        }
      }
    }
    x.bc[3 * gl] = lin.x; x.bc[3 * gl + 1] = lin.y; x.bc[3 * gl + 2] = lin.z;
    x.bc[6 + 3 * gl] = ang.x; x.bc[7 + 3 * gl] = ang.y; x.bc[8 + 3 * gl] = ang.z;
  }
  if constexpr (kSpread) {
    const bool plane = gl >= 2 && gl < 8, qlane = gl >= 8 && gl < 16;
    const int pc = (gl - 2) % 3, qc = (gl - 8) & 3;
    const int src = plane ? (gl - 2) / 3 : (qlane ? (gl - 8) >> 2 : 0);  // the body's lane
    const int bs = __shfl_sync(0xffffffffu, mine ? b : -1, src, G);
    const bool act = (plane || qlane) && bs >= 0;
    // the quaternion, narrowed by its component lanes for the increment
    // (add_scaled_vector_island's first step)
    W acc = (W)0;
    R qr = z;
    if (act && qlane) {
      acc = x.P(3 + qc, bs);
      qr = cvt_fast<R>(acc);
    }
    const int qsrc = 8 + 4 * (gl & 1);
    const R r0 = __shfl_sync(0xffffffffu, qr, qsrc, G), r1 = __shfl_sync(0xffffffffu, qr, qsrc + 1, G);
    const R r2 = __shfl_sync(0xffffffffu, qr, qsrc + 2, G), r3 = __shfl_sync(0xffffffffu, qr, qsrc + 3, G);
    R h0 = z, h1 = z, h2 = z, h3 = z;
    if (mine && b >= 0) {
      const q4<R> qq{r0, r1, r2, r3};
      q4<R> t{(R)0, ang.x * (R)1, ang.y * (R)1, ang.z * (R)1};
      t = qmul(t, qq);
      h0 = t.w * (R)0.5; h1 = t.x * (R)0.5; h2 = t.y * (R)0.5; h3 = t.z * (R)0.5;
    }
    const R H0 = __shfl_sync(0xffffffffu, h0, src, G), H1 = __shfl_sync(0xffffffffu, h1, src, G);
    const R H2 = __shfl_sync(0xffffffffu, h2, src, G), H3 = __shfl_sync(0xffffffffu, h3, src, G);
    const R L0 = __shfl_sync(0xffffffffu, lin.x, src, G), L1 = __shfl_sync(0xffffffffu, lin.y, src, G);
    const R L2 = __shfl_sync(0xffffffffu, lin.z, src, G);
    // one float64 add: lanes 2-7 Position.AddScaled(normal, linearMove),
    // lanes 8-15 the quaternion increment
    if (act) {
      R val;
      if (plane) {
        acc = x.P(pc, bs);
        val = pc == 0 ? L0 : (pc == 1 ? L1 : L2);
      } else {
        val = qc == 0 ? H0 : (qc == 1 ? H1 : (qc == 2 ? H2 : H3));
      }
      acc += cvt_fast<W>(val);
      if (plane) x.P(pc, bs) = acc;
    }
    // qnormalize_island: the squares on the component lanes, the sum in
    // order and the decision on the quaternion's first lane
    const W sq = act && qlane ? acc * acc : (W)0;
    const W s1 = __shfl_sync(0xffffffffu, sq, gl + 1, G), s2 = __shfl_sync(0xffffffffu, sq, gl + 2, G);
    const W s3 = __shfl_sync(0xffffffffu, sq, gl + 3, G);
    int mode = 0;  // 0: leave, 1: scale by inv, 2: the identity (a zero quaternion)
    W inv = (W)0;
    if (act && qlane && qc == 0) {
      const W s = sq + s1 + s2 + s3;
      const W e = s - (W)1;
      const W ae = fabs(e);
      if (sizeof(R) != sizeof(W) && ae < (W)4e-7) {
      } else if (sizeof(R) != sizeof(W) && ae < (W)0x1p-11) {
        inv = (W)1 + e * ((W)-0.5 + e * ((W)0.375 + e * ((W)-0.3125 + e * (W)0.2734375)));
        mode = 1;
      } else {  // Normalize, quaternion.go:77-99, on the same sum
        W len = sqrt_<W>(s);
        if (real_equal<W>((W)1, len)) {
        } else if (len == (W)0) {
          mode = 2;
        } else {
          if (len == Lim<W>::inf()) len = Lim<W>::max_value();
          inv = (W)1 / len;
          mode = 1;
        }
      }
    }
    const int lead = qlane ? gl - qc : 0;
    mode = __shfl_sync(0xffffffffu, mode, lead, G);
    inv = __shfl_sync(0xffffffffu, inv, lead, G);
    if (act && qlane) {
      if (mode == 1) acc *= inv;
      else if (mode == 2) acc = qc == 0 ? (W)1 : (W)0;
      x.P(3 + qc, bs) = acc;
    }
    __syncwarp();
    if (mine && b >= 0 && !x.aw[b]) {
      // CalculateDerivedData reads the stored (R-rounded) orientation
#pragma unroll
      for (int c = 3; c < 7; ++c) x.P(c, b) = (W)(R)x.P(c, b);
      derive_asleep(x, v, bstart, b);
    }
  }
}

template <class R> __device__ __forceinline__ m3<R> skew(const v3<R>& v) {  // contact.go:612-616
  m3<R> m;
  m.m[0] = (R)0; m.m[3] = -v.z; m.m[6] = v.y;
  m.m[1] = v.z; m.m[4] = (R)0; m.m[7] = -v.x;
  m.m[2] = -v.y; m.m[5] = v.x; m.m[8] = (R)0;
  return m;
}

// The response matrix of calculateFrictionImpulse (contact.go:540-575): the
// contact-frame velocity change per unit impulse of both bodies, in R.
template <class R, class W>
__device__ __forceinline__ m3<R> friction_response(const RCtx<R, W>& x, int k, int b0, int b1, const m3<R>& C) {
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
  return dv;
}

// The matrices of contact k's friction solve for the whole of
// adjustVelocities: K = Invert(response) in W (contact.go:577-580,
// matrix.go:125-153), kept in R for the solve, and the response's first row
// (R).  They depend on the
// relative positions, the basis, the inverse masses and the bodies' world
// inverse inertia, none of which adjustVelocities changes, so computing them
// once, lane-parallel, at the start of the phase gives exactly the values the
// reference recomputes at every iteration; the sequential chain then only
// forms K * (desired delta velocity, -vy, -vz).
template <class R, class W> __device__ __forceinline__ void friction_prepare(const RCtx<R, W>& x, int k) {
  if (x.friction(k) == (R)0) return;  // calculateFrictionlessImpulse needs neither
  const int bb = x.cb[k];
  const m3<R> dv = friction_response(x, k, body0_of(bb), body1_of(bb), x.basis(k));
  m3<W> dv_w;
#pragma unroll
  for (int q = 0; q < 9; ++q) dv_w.m[q] = (W)(dv.m[q]);
  const m3<W> K = invert(dv_w);
#pragma unroll
  for (int q = 0; q < 9; ++q) x.K(q, k) = (R)(K.m[q]);
  x.KD(0, k) = dv.m[0];
  x.KD(1, k) = dv.m[3];
  x.KD(2, k) = dv.m[6];
}

// calculateFrictionImpulse, contact.go:533-606, from the matrices of
// friction_prepare: the solve K * (desired delta velocity, -vy, -vz) in R,
// then the dynamic-friction correction.
// A contact's K (the first 9 reals of its K_ROW block) by 16-byte loads, and
// the response's first row (reals 9-11), which only the dynamic-friction
// branch reads.
__device__ __forceinline__ void load_k(const float* p, float (&o)[9]) {
  const float4* q = reinterpret_cast<const float4*>(p);
  const float4 a = q[0], b = q[1];
  o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = a.w;
  o[4] = b.x; o[5] = b.y; o[6] = b.z; o[7] = b.w;
  o[8] = p[8];
}
__device__ __forceinline__ void load_k(const double* p, double (&o)[9]) {
  const double2* q = reinterpret_cast<const double2*>(p);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const double2 t = q[i];
    o[2 * i] = t.x; o[2 * i + 1] = t.y;
  }
  o[8] = p[8];
}

template <class R, class W> __device__ v3<R> friction_impulse(const RCtx<R, W>& x, int k) {
  const R* row = x.kw + (long long)k * K_ROW;
  m3<R> K;
  load_k(row, K.m);
  const R ddv = x.Cf(W_DDV, k);
  const v3<R> kill = V<R>(ddv, -x.Cf(W_CVY, k), -x.Cf(W_CVZ, k));
  v3<R> ic = mulv(K, kill);
  const R fr = x.friction(k);
  R planar = sqrt_<R>(ic.y * ic.y + ic.z * ic.z);
  if (planar > ic.x * fr) {
    ic.y /= planar;
    ic.z /= planar;
    ic.x = row[9] + row[10] * fr * ic.y + row[11] * fr * ic.z;
    ic.x = ddv / ic.x;
    ic.y *= fr * ic.x;
    ic.z *= fr * ic.x;
  }
  return ic;
}

// applyVelocityChange, contact.go:447-494 (group leader); velocity and
// rotation changes of both bodies go to x.bc[0..11].
template <class R, class W, bool LEARN>
__device__ void apply_velocity_change(const RCtx<R, W>& x, const BatchView<R>& v, int w, int k) {
  const int bb = x.cb[k];
  const int b0 = body0_of(bb), b1 = body1_of(bb);
  const m3<R> C = x.basis(k);
  v3<R> ic;
  if (x.friction(k) == (R)0) {
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
    ic = friction_impulse(x, k);
  }
  if (LEARN && v.mode == 1) {  // harvest: total impulse applied at this contact
    x.J(0, k) += ic.x;
    x.J(1, k) += ic.y;
    x.J(2, k) += ic.z;
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


// applyVelocityChange (contact.go:447-494) spread over lanes 0-5 of a group
// with `on` (every lane of the warp calls it), for the float64 form, whose
// chain runs on the float64 pipe: a float64 warp instruction costs the pipe
// the same whatever its active lanes, so lane c (c = gl % 3) forms component
// c of the friction solve's product and of the impulse, and lane 3i + c
// forms component c of body i's velocity and rotation changes, where one
// lane formed them all before.  Every component is the one-lane formula's
// (mulv's row, cross's component, add_scaled), so the results are identical.
// Lane 3i + c leaves body i's changes in x.bc[3i + c] and x.bc[6 + 3i + c].
template <class R, class W, int G, bool LEARN>
__device__ void apply_velocity_change_spread(const RCtx<R, W>& x, const BatchView<R>& v, int w, int k, bool on,
                                             int gl) {
  const int g0 = (threadIdx.x & 31) - gl;  // the group's first lane
  const int c = gl % 3, i = gl / 3;
  const int p = c == 2 ? 0 : c + 1, q = c == 0 ? 2 : c - 1;  // cross component c = a_p b_q - a_q b_p
  const bool mine = on && gl < 6;
  const R z = (R)0;
  int b0 = 0, b1 = -1;
  m3<R> C;
  v3<R> ic = V<R>(z, z, z);
  R icc = z;
  bool frictionless = false;
  if (on) {
    const int bb = x.cb[k];
    b0 = body0_of(bb);
    b1 = body1_of(bb);
    C = x.basis(k);
    frictionless = x.friction(k) == (R)0;
    if (frictionless) {
      // calculateFrictionlessImpulse, contact.go:496-531 (rare: every lane)
      v3<R> d = cross(x.Cv(W_R0X, k), x.Cv(W_NX, k));
      d = mulv(x.iit(b0), d);
      d = cross(d, x.Cv(W_R0X, k));
      R dvel = dot(d, x.Cv(W_NX, k));
      dvel += x.Bf(18, b0);
      if (b1 < 0 && gl == 0) {
        atomicOr(&v.world_status[w], ST_FRICTIONLESS_NIL);
        atomicOr(v.status, ST_FRICTIONLESS_NIL);
      }
      ic = V<R>(x.Cf(W_DDV, k) / dvel, z, z);
    } else {
      // component c of K * (desired delta velocity, -vy, -vz) (mulv's row c)
      const R* row = x.kw + (long long)k * K_ROW;
      const R kx = x.Cf(W_DDV, k), ky = -x.Cf(W_CVY, k), kz = -x.Cf(W_CVZ, k);
      icc = row[c] * kx + row[3 + c] * ky + row[6 + c] * kz;
    }
  }
  {
    const R i0 = __shfl_sync(FULL, icc, g0, 32), i1 = __shfl_sync(FULL, icc, g0 + 1, 32);
    const R i2 = __shfl_sync(FULL, icc, g0 + 2, 32);
    if (on && !frictionless) {
      ic = V<R>(i0, i1, i2);
      // calculateFrictionImpulse's dynamic friction, contact.go:586-604 (every lane)
      const R* row = x.kw + (long long)k * K_ROW;
      const R fr = x.friction(k);
      const R ddv = x.Cf(W_DDV, k);
      R planar = sqrt_<R>(ic.y * ic.y + ic.z * ic.z);
      if (planar > ic.x * fr) {
        ic.y /= planar;
        ic.z /= planar;
        ic.x = row[9] + row[10] * fr * ic.y + row[11] * fr * ic.z;
        ic.x = ddv / ic.x;
        ic.y *= fr * ic.x;
        ic.z *= fr * ic.x;
      }
    }
  }
  if (LEARN && on && v.mode == 1 && gl == 0) {  // harvest: total impulse applied at this contact
    x.J(0, k) += ic.x;
    x.J(1, k) += ic.y;
    x.J(2, k) += ic.z;
  }
  // component c of the impulse C * ic (mulv's row c)
  R impc = z;
  if (on) {
    const R m0 = c == 0 ? C.m[0] : (c == 1 ? C.m[1] : C.m[2]);
    const R m3 = c == 0 ? C.m[3] : (c == 1 ? C.m[4] : C.m[5]);
    const R m6 = c == 0 ? C.m[6] : (c == 1 ? C.m[7] : C.m[8]);
    impc = m0 * ic.x + m3 * ic.y + m6 * ic.z;
  }
  const R ix = __shfl_sync(FULL, impc, g0, 32), iy = __shfl_sync(FULL, impc, g0 + 1, 32);
  const R iz = __shfl_sync(FULL, impc, g0 + 2, 32);
  const v3<R> imp = V<R>(ix, iy, iz);
  const int b = i == 0 ? b0 : b1;
  const bool act = mine && b >= 0;
  // component c of cross(r0, imp) (body 0) or cross(imp, r1) (body 1)
  R crc = z;
  v3<R> r = V<R>(z, z, z);
  if (act) {
    r = i == 0 ? x.Cv(W_R0X, k) : x.Cv(W_R1X, k);
    const v3<R> a = i == 0 ? r : imp, bv = i == 0 ? imp : r;
    const R ap = p == 0 ? a.x : (p == 1 ? a.y : a.z), aq = q == 0 ? a.x : (q == 1 ? a.y : a.z);
    const R bp = p == 0 ? bv.x : (p == 1 ? bv.y : bv.z), bq = q == 0 ? bv.x : (q == 1 ? bv.y : bv.z);
    crc = ap * bq - aq * bp;
  }
  const int t0 = g0 + 3 * (gl < 6 ? i : 0);
  const R cx = __shfl_sync(FULL, crc, t0, 32), cy = __shfl_sync(FULL, crc, t0 + 1, 32);
  const R cz = __shfl_sync(FULL, crc, t0 + 2, 32);
  R vc = z, rc = z;
  if (act) {
    // rc = iitWorld * cross (mulv's row c); vc = 0 + imp * (+-inverse mass)
    rc = x.Bf(9 + c, b) * cx + x.Bf(12 + c, b) * cy + x.Bf(15 + c, b) * cz;
    const R im = i == 0 ? x.Bf(18, b) : -x.Bf(18, b);
    const R impc_own = c == 0 ? imp.x : (c == 1 ? imp.y : imp.z);
    vc += impc_own * im;
    x.Bf(c, b) += vc;
    x.Bf(3 + c, b) += rc;
  }
  if (mine) {
    x.bc[3 * i + c] = vc;
    x.bc[6 + 3 * i + c] = rc;
  }
}


// A world's body rows from the batch rows into the working rows of x, by the
// `step` lanes of a group (lane index `first`).
template <class R, class W>
__device__ __forceinline__ void load_bodies(const RCtx<R, W>& x, const BatchView<R>& v, long long bstart, int n,
                                            int first, int step) {
  const long long S = v.nb_pad;
  for (int i = first; i < n; i += step) {
    const long long g = bstart + i;
    x.P(0, i) = (W)(v.body[B_PX * S + g]);
    x.P(1, i) = (W)(v.body[B_PY * S + g]);
    x.P(2, i) = (W)(v.body[B_PZ * S + g]);
    x.P(3, i) = (W)(v.body[B_QW * S + g]);
    x.P(4, i) = (W)(v.body[B_QX * S + g]);
    x.P(5, i) = (W)(v.body[B_QY * S + g]);
    x.P(6, i) = (W)(v.body[B_QZ * S + g]);
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      x.Bf(r, i) = v.body[(B_VX + r) * S + g];
      x.Bf(3 + r, i) = v.body[(B_RX + r) * S + g];
      x.Bf(6 + r, i) = v.body[(B_LX + r) * S + g] * x.dt;
    }
#pragma unroll
    for (int r = 0; r < 9; ++r) x.Bf(9 + r, i) = v.body[(B_IW0 + r) * S + g];
    x.Bf(18, i) = v.body[B_INVM * S + g];
    x.Bf(19, i) = v.body[B_MOTION * S + g];
    x.aw[i] = v.awake[g];
  }
}

// ---------------------------------------------------------------- world slots
// Shared memory of one world: body rows (W and R), contact working rows,
// broadcast scratch, packed bodies, awake flags.  The learned paths keep
// their per-body scratch and the impulse rows in global memory, so they use
// the same slot (and reach the same occupancy) as the plain resolver.
// The float64 form (8 or more lanes per world) gathers the contacts touching
// the two resolved bodies before updating them (see position_loop_g); room
// for one gather.
constexpr int kTouchList = 64;
template <class R> __host__ __device__ constexpr bool gathers_updates() { return sizeof(R) == 8; }

template <class R, class W> __host__ __device__ inline size_t rs_slot_bytes(int nbs, int cs) {
  const size_t nb16 = (size_t)((nbs + 15) & ~15);
  size_t b = (size_t)7 * nbs * sizeof(W);
  b += (size_t)20 * nbs * sizeof(R);
  b += (size_t)w_rows_kept<R>() * cs * sizeof(R);
  b += 16 * sizeof(R);
  b += (size_t)cs * sizeof(int);
  b += nb16;
  if (gathers_updates<R>()) b += (size_t)kTouchList * sizeof(int);
  return (b + 15) & ~(size_t)15;
}

template <class R, class W> struct Slot {
  RCtx<R, W> x;
  int* ml;          // [kTouchList] contacts touching the two bodies just resolved (float64 form)
  R* cw_s;
  int* cb_s;
  uint8_t* aw_pos;  // awake flags at the start of adjustVelocities (global)
  uint8_t* aw_pre;  // awake flags at prepareContacts (global)
};

template <class R, class W>
__device__ __forceinline__ Slot<R, W> make_slot(unsigned char* base, int nbs, int cs, R dt) {
  Slot<R, W> s;
  RCtx<R, W>& x = s.x;
  x.nbs = nbs;
  x.dt = dt;
  x.bw = reinterpret_cast<W*>(base);
  x.br = reinterpret_cast<R*>(x.bw + 7 * nbs);
  s.cw_s = x.br + 20 * nbs;
  x.bc = s.cw_s + (size_t)w_rows_kept<R>() * cs;
  s.cb_s = reinterpret_cast<int*>(x.bc + 16);
  x.aw = reinterpret_cast<uint8_t*>(s.cb_s + cs);
  s.ml = reinterpret_cast<int*>(x.aw + ((nbs + 15) & ~15));
  x.save = x.delta = x.jw = nullptr;
  x.wi = nullptr;
  x.wst = x.jst = 0;
  s.aw_pos = s.aw_pre = nullptr;
  return s;
}

template <class R, class W>
__device__ __forceinline__ void bind_contacts(Slot<R, W>& s, const BatchView<R>& v, int C, int cs, long long cst) {
  RCtx<R, W>& x = s.x;
  if (C <= cs) {
    x.cw = s.cw_s;
    x.cb = s.cb_s;
    x.cst = cs;
  } else {
    x.cw = v.work + cst;
    x.cb = v.work_bodies + cst;
    x.cst = v.nc_total;
  }
  x.gmat = v.uniform_material ? nullptr : v.contact + (long long)C_FRIC * v.nc_total + cst;
  x.gst = (long long)(C_REST - C_FRIC) * v.nc_total;
  x.kw = v.kmat + cst * K_ROW;
}

// the learned paths' global scratch of the world whose bodies start at bstart
template <class R, class W>
__device__ __forceinline__ void bind_ws(Slot<R, W>& s, const BatchView<R>& v, long long bstart, long long cst) {
  RCtx<R, W>& x = s.x;
  x.wst = v.nb_pad;
  x.save = v.ws_rows + bstart;
  x.delta = v.ws_rows + 7 * v.nb_pad + bstart;
  x.wi = v.ws_int + bstart;
  x.jw = v.work + (long long)W_J0 * v.nc_total + cst;
  x.jst = v.nc_total;
  s.aw_pos = v.ws_u8 + bstart;
  s.aw_pre = v.ws_u8 + v.nb_pad + bstart;
}

// The 18 features of a contact at the start of adjustVelocities, all in the
// contact basis where they are vectors: the number of contacts between body 0
// and other bodies, a half-space flag, the contact velocity (3), penetration, desired delta
// velocity, the response matrix (6: nn, tt, ss, nt, ns, ts), the impulse that
// would resolve the contact alone along its normal (desired delta velocity /
// response nn), and per body the contacts touching it and their summed
// positive desired delta velocities (2 + 2).
template <class R, class W> __device__ void contact_features(const RCtx<R, W>& x, int k, float* f) {
  const int bb = x.cb[k];
  const int b0 = body0_of(bb), b1 = body1_of(bb);
  const v3<R> cv = x.Cv(W_CVX, k);
  const R ddv = x.Cf(W_DDV, k);
  f[0] = (float)x.WI(WS_NBB, b0);
  f[1] = b1 < 0 ? 1.f : 0.f;
  f[2] = (float)cv.x; f[3] = (float)cv.y; f[4] = (float)cv.z;
  f[5] = (float)x.Cf(W_PEN, k);
  f[6] = (float)ddv;
  const m3<R> K = friction_response(x, k, b0, b1, x.basis(k));
  f[7] = (float)K.m[0]; f[8] = (float)K.m[4]; f[9] = (float)K.m[8];
  f[10] = (float)K.m[3]; f[11] = (float)K.m[6]; f[12] = (float)K.m[7];
  f[13] = K.m[0] > (R)0 ? (float)(ddv / K.m[0]) : 0.f;
  f[14] = (float)x.WI(WS_DEG, b0);
  f[15] = b1 >= 0 ? (float)x.WI(WS_DEG, b1) : 0.f;
  f[16] = (float)(unsigned)x.WI(WS_LOAD, b0) * (1.f / kLoadScale);
  f[17] = b1 >= 0 ? (float)(unsigned)x.WI(WS_LOAD, b1) * (1.f / kLoadScale) : 0.f;
}

template <int G> __device__ __forceinline__ int group_sum(int v) {
#pragma unroll
  for (int off = G / 2; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  return v;
}

// The warm start of one world, planned by k_warm_features for its bodies
// whose contacts are all with the half-space ("grounded" bodies), at the state
// adjustVelocities starts from (adjustPositions changes no velocity).  A
// grounded body's contacts depend on that body's velocity alone, so each one
// is warm-started independently:
//  1. Predictions of its contacts are projected: normal impulse >= 0,
//     friction inside the cone |J_t| <= friction * J_n.  Contacts of other
//     bodies get none.
//  2. The body's velocity and rotation change of all those impulses,
//     accumulated in contact order (deterministic); the half-space contacts
//     of a body are one run of the contact list when the narrowphase made
//     them, else the whole list is scanned.
//  3. A line search picks the body's scale s in [0, 1]: none of its contacts
//     may be pushed past what resolving it would do (normal velocity at most
//     velocity + max(desired delta, 0) + the velocity epsilon), and no
//     tangential speed may grow beyond max(current, epsilon).  The resolver
//     only removes approaching velocity, so it could not undo an overshoot.
//  4. The plan: the body's change times s in the delta rows, each contact's
//     velocity change times its body's s in the impulse rows (zeros where the
//     warm start does nothing); warm_start_apply adds them.
// The 32 lanes of a warp plan one world.  Adds this lane's warm-started bodies
// and the sum of their scales to *nw and *ssum.
template <class R, class W>
__device__ void warm_start_plan(const RCtx<R, W>& x, int n, int C, int lane, int* nw, float* ssum) {
  const R z = (R)0, eps = (R)0.01;
  for (int k = lane; k < C; k += 32) {
    const int bb = x.cb[k];
    v3<R> J = V<R>(x.J(0, k), x.J(1, k), x.J(2, k));
    if (body1_of(bb) >= 0 || x.WI(WS_NBB, body0_of(bb)) != 0 || !(J.x > z)) J = V<R>(z, z, z);  // also NaN
    const R lim = x.friction(k) * J.x;
    const R planar = sqrt_<R>(J.y * J.y + J.z * J.z);
    if (planar > lim) {
      const R f = planar > z ? lim / planar : z;
      J.y *= f;
      J.z *= f;
    }
    if (!(planar == planar)) J = V<R>(z, z, z);
    x.J(0, k) = J.x;
    x.J(1, k) = J.y;
    x.J(2, k) = J.z;
  }
  __syncwarp();
  for (int i = lane; i < n; i += 32) {
    v3<R> dvel = V<R>(z, z, z), drot = V<R>(z, z, z);
    const int deg = x.WI(WS_DEG, i);
    if (x.WI(WS_NBB, i) == 0 && deg > 0) {
      const m3<R> I = x.iit(i);
      const R invm = x.Bf(18, i);
      const int first = x.WI(WS_FIRST, i), last = x.WI(WS_LAST, i);
      const bool run = last - first + 1 == deg;
      for (int k = run ? first : 0; k <= (run ? last : C - 1); ++k) {
        if (!run && body0_of(x.cb[k]) != i) continue;
        const v3<R> J = V<R>(x.J(0, k), x.J(1, k), x.J(2, k));
        if (J.x == z) continue;
        const v3<R> imp = mulv(x.basis(k), J);
        add(drot, mulv(I, cross(x.Cv(W_R0X, k), imp)));
        add_scaled(dvel, imp, invm);
      }
    }
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      x.Delta(r, i) = (&dvel.x)[r];
      x.Delta(3 + r, i) = (&drot.x)[r];
    }
    x.WI(WS_SCALE, i) = __float_as_int(1.f);
  }
  __syncwarp();
  // contact velocity change at s = 1 (into the impulse rows) and the largest
  // scale each contact allows; a body's scale is the smallest of its contacts'
  for (int k = lane; k < C; k += 32) {
    const int bb = x.cb[k];
    const int b0 = body0_of(bb);
    if (body1_of(bb) >= 0 || x.WI(WS_NBB, b0) != 0) {
      x.J(0, k) = z;
      x.J(1, k) = z;
      x.J(2, k) = z;
      continue;
    }
    const m3<R> Ck = x.basis(k);
    const v3<R> dr = V<R>(x.Delta(3, b0), x.Delta(4, b0), x.Delta(5, b0));
    const v3<R> dl = V<R>(x.Delta(0, b0), x.Delta(1, b0), x.Delta(2, b0));
    v3<R> dv = cross(dr, x.Cv(W_R0X, k));
    add(dv, dl);
    const v3<R> dcv = mulv_t(Ck, dv);
    x.J(0, k) = dcv.x;
    x.J(1, k) = dcv.y;
    x.J(2, k) = dcv.z;
    R sk = (R)1;
    const R ddv = x.Cf(W_DDV, k);
    if (dcv.x > z) {
      const R q = ((ddv > z ? ddv : z) + eps) / dcv.x;
      if (q < sk) sk = q;
    }
    const R ty = x.Cf(W_CVY, k), tz = x.Cf(W_CVZ, k);
    const R a = dcv.y * dcv.y + dcv.z * dcv.z;
    if (a > z) {
      const R t2 = ty * ty + tz * tz;
      const R bound2 = t2 > eps * eps ? t2 : eps * eps;
      const R hb = ty * dcv.y + tz * dcv.z;
      // largest s with |t + s dt|^2 <= bound^2: root of a s^2 + 2 hb s + (t2 - bound2)
      const R disc = hb * hb - a * (t2 - bound2);
      const R q = (-hb + sqrt_<R>(disc > z ? disc : z)) / a;
      if (q < sk) sk = q;
    }
    float sf = (float)sk;
    if (!(sf >= 0.f)) sf = 0.f;  // NaN or negative: no warm start
    if (sf < 1.f) atomicMin(&x.WI(WS_SCALE, b0), __float_as_int(sf));  // non-negative floats order as ints
  }
  __syncwarp();
  for (int i = lane; i < n; i += 32) {
    bool moved = false;
#pragma unroll
    for (int r = 0; r < 6; ++r) moved |= x.Delta(r, i) != z;
    const R sb = (R)__int_as_float(x.WI(WS_SCALE, i));
    if (moved) {
      ++*nw;
      *ssum += (float)sb;
    }
#pragma unroll
    for (int r = 0; r < 6; ++r) x.Delta(r, i) = moved && sb != z ? sb * x.Delta(r, i) : z;
  }
  __syncwarp();
  for (int k = lane; k < C; k += 32) {
    const int bb = x.cb[k];
    const int b0 = body0_of(bb);
    if (body1_of(bb) >= 0 || x.WI(WS_NBB, b0) != 0) continue;
    const R sb = (R)__int_as_float(x.WI(WS_SCALE, b0));
#pragma unroll
    for (int c = 0; c < 3; ++c) x.J(c, k) = x.J(c, k) != z ? sb * x.J(c, k) : z;
  }
}

// The planned warm start, applied at the start of adjustVelocities: each body
// takes its scaled change, each contact its scaled velocity change and a
// recomputed desired delta velocity, as adjustVelocities does after an
// impulse (contact.go:416-445).  A body or contact with nothing planned keeps
// its values bit for bit.  Every lane of the warp calls it (it synchronises
// the warp); `on` selects the groups warm-starting.  Returns the bodies this
// lane moved.
template <class R, class W, int G>
__device__ int warm_start_apply(const RCtx<R, W>& x, int n, int C, int gl, bool on) {
  const R z = (R)0;
  int moved = 0;
  for (int i = gl; on && i < n; i += G) {
    bool any = false;
#pragma unroll
    for (int r = 0; r < 6; ++r) any |= x.Delta(r, i) != z;
    if (!any) continue;
    ++moved;
#pragma unroll
    for (int r = 0; r < 6; ++r) x.Bf(r, i) += x.Delta(r, i);
  }
  __syncwarp();
  for (int k = gl; on && k < C; k += G) {
    const v3<R> dcv = V<R>(x.J(0, k), x.J(1, k), x.J(2, k));
    if (dcv.x == z && dcv.y == z && dcv.z == z) continue;
    v3<R> cv = x.Cv(W_CVX, k);
    add(cv, dcv);
    x.setCv(W_CVX, k, cv);
    x.Cf(W_DDV, k) = desired_dv(x, k);
  }
  return moved;
}

// Which resolved body each body of contact k is: e[b] = d when contact body
// b is resolved body d (d1 < 0: there is none), else -1.  A contact body is
// at most one of the two, so a contact takes at most two changes: body 0's
// first, then body 1's, which is the order of the reference's (b, d) loops
// (contact.go:254-280, 412-440).  The updates below run one code block per
// contact body, with d taken from e, instead of one per (b, d) pair: a warp
// runs a block whenever any of its lanes needs it.
__device__ __forceinline__ int2 touching(int bb, int d0, int d1) {
  const int kb0 = body0_of(bb), kb1 = body1_of(bb);
  int2 e;
  e.x = kb0 == d0 ? 0 : (d1 >= 0 && kb0 == d1 ? 1 : -1);
  e.y = kb1 < 0 ? -1 : (kb1 == d0 ? 0 : (d1 >= 0 && kb1 == d1 ? 1 : -1));
  return e;
}

// adjustPositions' update of contact k after resolving a contact between
// bodies d0, d1 (d1 < 0: none) whose linear / angular changes are in x.bc
// (contact.go:254-280); a contact touching neither is left alone.
template <class R, class W>
__device__ __forceinline__ void penetration_update(const RCtx<R, W>& x, int k, int d0, int d1) {
  const int2 e = touching(x.cb[k], d0, d1);
  if (e.x < 0 && e.y < 0) return;
  const v3<R> nk = x.Cv(W_NX, k);
  R pen = x.Cf(W_PEN, k);
#pragma unroll
  for (int b = 0; b < 2; ++b) {
    const int d = b == 0 ? e.x : e.y;
    if (d >= 0) {
      const v3<R> r = b == 0 ? x.Cv(W_R0X, k) : x.Cv(W_R1X, k);
      v3<R> dp = cross(d == 0 ? V<R>(x.bc[6], x.bc[7], x.bc[8]) : V<R>(x.bc[9], x.bc[10], x.bc[11]), r);
      add(dp, d == 0 ? V<R>(x.bc[0], x.bc[1], x.bc[2]) : V<R>(x.bc[3], x.bc[4], x.bc[5]));
      const R sign = b == 0 ? (R)-1 : (R)1;
      pen += dot(dp, nk) * sign;
    }
  }
  x.Cf(W_PEN, k) = pen;
}

// adjustVelocities' update of contact k (contact.go:412-440), as above.
template <class R, class W>
__device__ __forceinline__ void velocity_update(const RCtx<R, W>& x, int k, int d0, int d1) {
  const int bb = x.cb[k];
  const int2 e = touching(bb, d0, d1);
  if (e.x < 0 && e.y < 0) return;
  const m3<R> Ck = x.basis(k);
  v3<R> cv = x.Cv(W_CVX, k);
#pragma unroll
  for (int b = 0; b < 2; ++b) {
    const int d = b == 0 ? e.x : e.y;
    if (d >= 0) {
      const v3<R> r = b == 0 ? x.Cv(W_R0X, k) : x.Cv(W_R1X, k);
      v3<R> dv = cross(d == 0 ? V<R>(x.bc[6], x.bc[7], x.bc[8]) : V<R>(x.bc[9], x.bc[10], x.bc[11]), r);
      add(dv, d == 0 ? V<R>(x.bc[0], x.bc[1], x.bc[2]) : V<R>(x.bc[3], x.bc[4], x.bc[5]));
      const R sign = b == 1 ? (R)-1 : (R)1;
      v3<R> t = mulv_t(Ck, dv);
      mul_with(t, sign);
      add(cv, t);
    }
  }
  x.setCv(W_CVX, k, cv);
  x.Cf(W_DDV, k) = desired_dv_of(x, k, body0_of(bb), body1_of(bb), V<R>(Ck.m[0], Ck.m[1], Ck.m[2]), cv.x);
}

// adjustVelocities, contact.go:388-445, for the groups with run set; returns
// the iterations used.
template <class R, class W, int G, bool LEARN>
__device__ int velocity_loop(const RCtx<R, W>& x, const BatchView<R>& v, int w, int C, int gl, int max_it, bool run) {
  int used = 0;
  // the lane's best key over its contacts (k = gl mod G): scanned once here,
  // then by the update pass of each iteration, which visits the same contacts
  // in the same order right after changing them (a contact's desired delta
  // velocity changes only in its own lane), so the argmax is the same
  auto best = key_of((R)0, (R)0);
  int bidx = 0x7fffffff;
  if (run)
    for (int k = gl; k < C; k += G) {
      const auto key = key_of(x.Cf(W_DDV, k), (R)0.01);
      if (key > best) {
        best = key;
        bidx = k;
      }
    }
  while (__any_sync(FULL, run)) {
    group_first_max<G>(best, bidx);
    if (best == 0) run = false;
    if (run && gl == 0) {
      match_awake(x, x.cb[bidx]);
      apply_velocity_change<R, W, LEARN>(x, v, w, bidx);
    }
    __syncwarp();
    auto nbest = key_of((R)0, (R)0);
    int nidx = 0x7fffffff;
    if (run) {
      const int rb = x.cb[bidx];
      const int d0 = body0_of(rb), d1 = body1_of(rb);
      for (int k = gl; k < C; k += G) {
        velocity_update(x, k, d0, d1);
        const auto key = key_of(x.Cf(W_DDV, k), (R)0.01);
        if (key > nbest) {
          nbest = key;
          nidx = k;
        }
      }
    }
    __syncwarp();
    if (run && ++used >= max_it) run = false;
    best = nbest;
    bidx = nidx;
  }
  return used;
}

// ---------------------------------------------------------------- gathered updates
// The float64 form updates, after a resolved contact, only the contacts
// touching its two bodies: gathered in contact order (a ballot per G
// contacts of each world) and updated one per lane of the world's group,
// instead of every lane walking all its contacts, where a matching contact's
// float64 update ran once per loop position with a match anywhere in the
// warp, at the cost of a whole warp instruction on the float64 pipe for
// each.  The reference's loop visits every contact but changes only these,
// and each update touches only its own contact (contact.go:254-280,
// 412-440), so the result is the same bit for bit.  The next argmax is then
// a separate scan of the world's keys.  With G < 32 the worlds of a warp do
// this side by side (lockstep, as the other loops).  (In float32 the gather
// did not pay: the same number of instructions, and more registers.)

// Applies upd(k) to every contact k of the group's world touching body d0 or
// d1 (nothing where `on` is false).  Every lane of the warp calls it.
template <int G, class R, class W, class F>
__device__ __forceinline__ void update_touching(const RCtx<R, W>& x, int C, int gl, int d0, int d1, int* ml, bool on,
                                                F&& upd) {
  const int lane = threadIdx.x & 31;
  const unsigned gmask = G == 32 ? FULL : (((1u << G) - 1u) << (lane - gl));
  const int Cg = on ? C : 0;
  int Cmax = Cg;  // the warp's trip count: the largest of its worlds'
#pragma unroll
  for (int off = G; off < 32; off <<= 1) Cmax = max(Cmax, __shfl_xor_sync(FULL, Cmax, off));
  int m = 0;
  for (int base = 0; base < Cmax; base += G) {
    const int k = base + gl;
    bool hit = false;
    if (k < Cg) {
      const int bb = x.cb[k];
      const int kb0 = body0_of(bb), kb1 = body1_of(bb);
      hit = kb0 == d0 || (d1 >= 0 && kb0 == d1) || (kb1 >= 0 && (kb1 == d0 || kb1 == d1));
    }
    const unsigned bal = __ballot_sync(FULL, hit) & gmask;
    if (hit) ml[m + __popc(bal & ((1u << lane) - 1u))] = k;
    m += __popc(bal);
    if (__any_sync(FULL, m > kTouchList - G) || base + G >= Cmax) {
      __syncwarp();
      for (int j = gl; j < m; j += G) upd(ml[j]);
      __syncwarp();
      m = 0;
    }
  }
}

// The group's first maximum of a row's keys (W_PEN or W_DDV) over its
// world's contacts (key 0 where `on` is false).
template <int G, class R, class W>
__device__ __forceinline__ void group_row_first_max(const RCtx<R, W>& x, int row, int C, int gl, bool on,
                                                    decltype(key_of((R)0, (R)0))& best, int& bidx) {
  best = key_of((R)0, (R)0);
  bidx = 0x7fffffff;
  for (int k = gl; on && k < C; k += G) {
    const auto key = key_of(x.Cf(row, k), (R)0.01);
    if (key > best) {
      best = key;
      bidx = k;
    }
  }
  group_first_max<G>(best, bidx);
}

// adjustPositions (contact.go:231-283) with gathered updates, G lanes per
// world; returns the iterations used.
template <class R, class W, int G>
__device__ int position_loop_g(const RCtx<R, W>& x, const BatchView<R>& v, int bstart, int C, int gl, int max_it,
                               bool run, int* ml) {
  int used = 0;
  while (__any_sync(FULL, run)) {
    decltype(key_of((R)0, (R)0)) best;
    int bidx;
    group_row_first_max<G>(x, W_PEN, C, gl, run, best, bidx);
    if (best == 0) run = false;
    if (run && gl == 0) match_awake(x, x.cb[bidx]);
    __syncwarp();
    apply_position_change<R, W, G>(x, v, bstart, bidx, run, gl);
    __syncwarp();
    int d0 = -2, d1 = -2;
    if (run) {
      const int rb = x.cb[bidx];
      d0 = body0_of(rb);
      d1 = body1_of(rb);
    }
    update_touching<G>(x, C, gl, d0, d1, ml, run, [&](int k) { penetration_update(x, k, d0, d1); });
    if (run && ++used >= max_it) run = false;
  }
  return used;
}

// adjustVelocities (contact.go:388-445) with gathered updates, G lanes per
// world; returns the iterations used.
template <class R, class W, int G, bool LEARN>
__device__ int velocity_loop_g(const RCtx<R, W>& x, const BatchView<R>& v, int w, int C, int gl, int max_it,
                               bool run, int* ml) {
  int used = 0;
  while (__any_sync(FULL, run)) {
    decltype(key_of((R)0, (R)0)) best;
    int bidx;
    group_row_first_max<G>(x, W_DDV, C, gl, run, best, bidx);
    if (best == 0) run = false;
    if constexpr (sizeof(R) == 8) {
      if (run && gl == 0) match_awake(x, x.cb[bidx]);
      __syncwarp();
      apply_velocity_change_spread<R, W, G, LEARN>(x, v, w, bidx, run, gl);
    } else if (run && gl == 0) {
      match_awake(x, x.cb[bidx]);
      apply_velocity_change<R, W, LEARN>(x, v, w, bidx);
    }
    __syncwarp();
    int d0 = -2, d1 = -2;
    if (run) {
      const int rb = x.cb[bidx];
      d0 = body0_of(rb);
      d1 = body1_of(rb);
    }
    update_touching<G>(x, C, gl, d0, d1, ml, run, [&](int k) { velocity_update(x, k, d0, d1); });
    if (run && ++used >= max_it) run = false;
  }
  return used;
}

// v.mode: 0 plain, 1 harvest (plain, copying k_warm_features' features and
// writing the applied impulses), 2 learned warm start (applying
// k_warm_features' plan) with fallback to the plain solve.  LEARN = false
// compiles the plain resolver alone (v.mode is ignored), so the learned paths
// cost the plain kernel no registers.
// ---------------------------------------------------------------- one frame per world
// Survivor list of the narrowphase inside the fused frame (one warp per CTA).
constexpr int kFrameSurvivors = 128;

// Bytes of the narrowphase tile of one world in the fused frame: staged rows
// and collider transforms, shapes, cull data, scan scratch, survivor list.
template <class R> __host__ __device__ inline size_t frame_tile_bytes(int nbs) {
  size_t b = (size_t)(11 + 12) * nbs * sizeof(R) + (size_t)nbs * sizeof(int) + (size_t)5 * nbs * sizeof(float);
  b += (66 + kFrameSurvivors + np_sort_ints(32)) * sizeof(int);
  return (b + 15) & ~(size_t)15;
}
// The fused frame's slot: the resolver's, large enough for the narrowphase
// tile too (the narrowphase runs first, in the same bytes).
template <class R, class W> __host__ __device__ inline size_t frame_slot_bytes(int nbs, int cs) {
  const size_t a = rs_slot_bytes<R, W>(nbs, cs), b = frame_tile_bytes<R>(nbs);
  return a > b ? a : b;
}

// Integrate + the colliders' derived data of world w's bodies, then its
// narrowphase, by the calling warp, the tile in the shared memory at base:
// the first two steps of the frame of examples/cubedrop.go:69-75, as
// k_integrate and k_narrowphase run them.
template <class R, class W>
__device__ void frame_front(const BatchView<R>& v, int w, int n, int bstart, int nbs, R dt, R sleep_bias,
                            unsigned char* base) {
  const int lane = threadIdx.x;
  for (int i = lane; i < n; i += 32) integrate_body<R, W>(v, (long long)bstart + i, dt, sleep_bias);
  __syncwarp();
  NPTile<R> tl;
  tl.nbs = nbs;
  tl.stage = reinterpret_cast<R*>(base);
  tl.T = tl.stage + 11 * nbs;
  tl.shape = reinterpret_cast<int*>(tl.T + 12 * nbs);
  tl.cull = reinterpret_cast<float*>(tl.shape + nbs);
  int* scan = reinterpret_cast<int*>(tl.cull + 5 * nbs);
  int* surv = scan + 66;
  for (int i = lane; i < n; i += 32) {
#pragma unroll
    for (int r = 0; r < 11; ++r) tl.stage[r * nbs + i] = v.body[(long long)r * v.nb_pad + bstart + i];
    tl.shape[i] = v.shape[bstart + i];
  }
  __syncwarp();
  np_build_tile(tl, n, v.offset ? v.offset + bstart : nullptr, v.nb_pad);
  __syncwarp();
  int parity = 0;
  np_world<R, false>(tl, v, w, n, bstart, scan, parity, surv, kFrameSurvivors);
  __syncwarp();
}

// The resolver: G lanes per world, worlds from the device queue.  FRAME (the
// fused frame): each world's integrate and narrowphase first
// (frame_front), so one launch runs a whole frame (one world per warp, plain
// resolver).
// Warps per CTA: one world per warp in float32 runs four independent warps
// per CTA (each its own slot and its own worlds from the queue), so the SM's
// per-CTA shared-memory reserve is paid once per four slots: 5 CTAs of 4
// warps (20 warps) fit where 18 one-warp CTAs did.
template <class R, int G, bool FRAME> __host__ __device__ constexpr int rs_wpc() {
  return sizeof(R) == 4 && G == 32 && !FRAME ? 4 : 1;
}
// Registers: one world per warp in float32 is bounded to 20 warps per SM (96
// registers, a few spilled), the count its shared-memory slots allow.
template <class R, class W, int G, bool LEARN, bool FRAME = false>
__global__ void __launch_bounds__(32 * rs_wpc<R, G, FRAME>(),
                                  FRAME ? (sizeof(R) == 4 ? 18 : 8)
                                        : (G == 32 && sizeof(R) == 4 ? 5 : (LEARN ? 16 : 0)))
    k_resolve(BatchView<R> v, int nbs, int cs, R dt, R sleep_bias = (R)0) {
  static_assert(!FRAME || (G == 32 && !LEARN), "the fused frame runs one world per warp, plain");
  extern __shared__ __align__(128) unsigned char smem[];
  constexpr int NG = 32 / G;
  const int lane = threadIdx.x & 31;
  const int grp = lane / G, gl = lane % G;
  const int mode = LEARN ? v.mode : 0;
  const size_t slot_bytes = FRAME ? frame_slot_bytes<R, W>(nbs, cs) : rs_slot_bytes<R, W>(nbs, cs);
  Slot<R, W> sl = make_slot<R, W>(smem + (size_t)((threadIdx.x >> 5) * NG + grp) * slot_bytes, nbs, cs, dt);
  RCtx<R, W>& x = sl.x;
  const long long S = v.nb_pad;
  for (;;) {
    unsigned q0 = 0;
    if (lane == 0) q0 = atomicAdd(&v.queue[1], (unsigned)NG);
    q0 = __shfl_sync(FULL, q0, 0);
    if (q0 >= (unsigned)v.num_worlds) break;
    const unsigned qi = q0 + grp;
    bool has = qi < (unsigned)v.num_worlds;
    const int w = has ? v.order_rs[qi] : 0;
    if (has && v.big_count > 0 && v.body_count[w] > nbs) has = false;  // a world of k_resolve_big
    const int n = has ? v.body_count[w] : 0;
    const int bstart = has ? v.body_start[w] : 0;
    if constexpr (FRAME) {
      if (has && n <= nbs) frame_front<R, W>(v, w, n, bstart, nbs, dt, sleep_bias, smem);
      __syncwarp();
    }
    int C = has ? v.contact_count[w] : 0;
    if (has) {
      const int cap = v.contact_cap[w];
      if (C > cap) C = cap;  // the world is already flagged ST_CAPACITY
      if (gl == 0) {
        v.pos_iters[w] = 0;
        v.vel_iters[w] = 0;
      }
    }
    bool active = has && C > 0 && dt > (R)0;  // ResolveContacts guards, contact.go:210-212
    if (active && n > nbs) {
      if (gl == 0) {
        atomicOr(&v.world_status[w], ST_BODY_LIMIT);
        atomicOr(v.status, ST_BODY_LIMIT);
      }
      active = false;
    }
    const long long cst = has ? v.contact_start[w] : 0;
    bind_contacts(sl, v, C, cs, cst);
    if (LEARN && mode) bind_ws(sl, v, bstart, cst);
    if (active) {
      load_bodies(x, v, bstart, n, gl, G);
      if (mode)
        for (int i = gl; i < n; i += G) sl.aw_pre[i] = x.aw[i];
    }
    __syncwarp();
    if (active)
      for (int k = gl; k < C; k += G) prepare_contact(x, v, cst + k, k);
    __syncwarp();
    const int max_it = v.max_iterations >= 0 ? v.max_iterations : C * v.iter_mult;
    constexpr bool kGather = G >= 8 && gathers_updates<R>();
    // ---------------- adjustPositions, contact.go:231-283
    int used = 0;
    if constexpr (kGather) {
      used = position_loop_g<R, W, G>(x, v, bstart, C, gl, max_it, active && max_it > 0, sl.ml);
    } else {
    bool run = active && max_it > 0;
    // as in velocity_loop: the update pass also finds the next argmax
    auto best = key_of((R)0, (R)0);
    int bidx = 0x7fffffff;
    if (run)
      for (int k = gl; k < C; k += G) {
        const auto key = key_of(x.Cf(W_PEN, k), (R)0.01);
        if (key > best) {
          best = key;
          bidx = k;
        }
      }
    while (__any_sync(FULL, run)) {
      group_first_max<G>(best, bidx);
      if (best == 0) run = false;
      if (run && gl == 0) match_awake(x, x.cb[bidx]);
      __syncwarp();
      apply_position_change<R, W, G>(x, v, bstart, bidx, run, gl);
      __syncwarp();
      auto nbest = key_of((R)0, (R)0);
      int nidx = 0x7fffffff;
      if (run) {
        const int rb = x.cb[bidx];
        const int d0 = body0_of(rb), d1 = body1_of(rb);
        for (int k = gl; k < C; k += G) {
          penetration_update(x, k, d0, d1);
          const auto key = key_of(x.Cf(W_PEN, k), (R)0.01);
          if (key > nbest) {
            nbest = key;
            nidx = k;
          }
        }
      }
      __syncwarp();
      if (run && ++used >= max_it) run = false;
      best = nbest;
      bidx = nidx;
    }
    }
    const int pos_used = used;
    const bool solve = active && max_it > 0;
    if (solve)
      for (int k = gl; k < C; k += G) friction_prepare(x, k);
    __syncwarp();
    // ---------------- learned warm start / harvest set-up
    long long hv_base = -1;
    if (LEARN && mode) {
      // the state before adjustVelocities, for the fallback; the per-body
      // aggregates and the predicted impulses come from k_warm_features
      for (int i = gl; solve && i < n; i += G) {
        sl.aw_pos[i] = x.aw[i];
#pragma unroll
        for (int r = 0; r < 6; ++r) x.Save(r, i) = x.Bf(r, i);
        x.Save(6, i) = x.Bf(19, i);
      }
      if (mode == 1)  // harvest: the impulse totals start at zero
        for (int k = gl; solve && k < C; k += G) {
          x.J(0, k) = (R)0;
          x.J(1, k) = (R)0;
          x.J(2, k) = (R)0;
        }
    }
    __syncwarp();
    if (LEARN && mode == 1) {
      // every lane takes part in the shuffle; only solving groups reserve rows
      unsigned long long b0 = 0;
      if (solve && gl == 0) b0 = atomicAdd(v.hv_count, (unsigned long long)C);
      b0 = __shfl_sync(FULL, b0, grp * G);
      if (solve && (long long)(b0 + C) <= v.hv_cap) {
        hv_base = (long long)b0;
        for (int k = gl; k < C; k += G) {
          const float* f = v.ws_feat + (cst + k) * MLP_IN;  // written by k_warm_features
          float* o = v.hv_features + (hv_base + k) * MLP_IN;
#pragma unroll
          for (int c = 0; c < MLP_IN; ++c) o[c] = f[c];
        }
      }
    }
    bool warmed = false;  // this world had a warm-started body
    // a world whose last solve used more than max_it >> warm_shift iterations
    // (a quarter by default) is solved plainly: hard worlds are the ones that
    // exhaust the budget and are then re-solved (a re-solve costs a whole
    // solve in lockstep)
    const bool warm_ok = LEARN && mode == 2 && solve && !v.ws_world[w];
    if (LEARN && mode == 2) {
      const int nw = warm_start_apply<R, W, G>(x, n, C, gl, warm_ok);
      __syncwarp();
      warmed = group_sum<G>(nw) > 0;
    }
    // ---------------- adjustVelocities, contact.go:388-445
    if constexpr (kGather)
      used = velocity_loop_g<R, W, G, LEARN>(x, v, w, C, gl, max_it, solve, sl.ml);
    else
      used = velocity_loop<R, W, G, LEARN>(x, v, w, C, gl, max_it, solve);
    int vel_used = used;
    if (LEARN && mode == 2) {
      // the plain resolver has the last word: a warm-started world that used
      // all its iterations is solved again by the plain path from the saved
      // state (a world without a warm-started body was solved plainly)
      const bool fb = solve && warmed && used >= max_it;
      if (solve && gl == 0) v.ws_world[w] = ((long long)used << v.warm_shift) > max_it;
      if (__any_sync(FULL, fb)) {
        if (fb) {
          for (int i = gl; i < n; i += G) {
#pragma unroll
            for (int r = 0; r < 6; ++r) x.Bf(r, i) = x.Save(r, i);
            x.Bf(19, i) = x.Save(6, i);
            x.aw[i] = sl.aw_pos[i];
          }
        }
        __syncwarp();
        if (fb) {
          // contact velocities as prepareContacts left them (same velocities,
          // relative positions and basis), desired delta velocity with the
          // awake flags of that moment
          uint8_t* aw_now = x.aw;
          x.aw = sl.aw_pre;
          for (int k = gl; k < C; k += G) {
            const int bb = x.cb[k];
            const int b0 = body0_of(bb), b1 = body1_of(bb);
            const m3<R> Ck = x.basis(k);
            v3<R> cv = local_velocity(x, b0, x.Cv(W_R0X, k), Ck);
            if (b1 >= 0) sub(cv, local_velocity(x, b1, x.Cv(W_R1X, k), Ck));
            x.setCv(W_CVX, k, cv);
            x.Cf(W_DDV, k) = desired_dv(x, k);
          }
          x.aw = aw_now;
        }
        __syncwarp();
        int used2;
        if constexpr (kGather)
          used2 = velocity_loop_g<R, W, G, LEARN>(x, v, w, C, gl, max_it, fb, sl.ml);
        else
          used2 = velocity_loop<R, W, G, LEARN>(x, v, w, C, gl, max_it, fb);
        if (fb) vel_used += used2;
        if (fb && gl == 0) atomicAdd(&v.counters[4], 1ull);
      }
      if (warm_ok && gl == 0) atomicAdd(&v.counters[5], 1ull);
    }
    if (LEARN && mode == 1 && hv_base >= 0) {
      for (int k = gl; k < C; k += G) {
        float* lab = v.hv_labels + (hv_base + k) * MLP_OUT;
        lab[0] = (float)x.J(0, k);
        lab[1] = (float)x.J(1, k);
        lab[2] = (float)x.J(2, k);
      }
    }
    if (has && gl == 0) {
      v.pos_iters[w] = pos_used;
      v.vel_iters[w] = vel_used;
      atomicAdd(&v.counters[1], (unsigned long long)pos_used);
      atomicAdd(&v.counters[2], (unsigned long long)vel_used);
      atomicAdd(&v.counters[3], (unsigned long long)C);
    }
    if (active && v.contact_writeback) {
      // the caller's Contact values after ResolveContacts (penetration,
      // swapped bodies and normal of calculateInternals)
      const long long CS = v.nc_total;
      for (int k = gl; k < C; k += G) {
        R* o = v.contact + cst + k;
        o[C_NX * CS] = x.Cf(W_NX, k);
        o[C_NY * CS] = x.Cf(W_NY, k);
        o[C_NZ * CS] = x.Cf(W_NZ, k);
        o[C_PEN * CS] = x.Cf(W_PEN, k);
        v.contact_bodies[cst + k] = x.cb[k];
      }
    }
    if (active) {
      for (int i = gl; i < n; i += G) {
        const long long g = bstart + i;
        v.body[B_PX * S + g] = (R)(x.P(0, i));
        v.body[B_PY * S + g] = (R)(x.P(1, i));
        v.body[B_PZ * S + g] = (R)(x.P(2, i));
        v.body[B_QW * S + g] = (R)(x.P(3, i));
        v.body[B_QX * S + g] = (R)(x.P(4, i));
        v.body[B_QY * S + g] = (R)(x.P(5, i));
        v.body[B_QZ * S + g] = (R)(x.P(6, i));
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
    }
    __syncwarp();
  }
}


// ---------------------------------------------------------------- k_warm_features
// Shared-memory copy of the inference weights (fragment layouts of MlpDev).
constexpr size_t WF_W1 = 0;                       // [64][32] bf16
constexpr size_t WF_W2 = WF_W1 + 64 * 32 * 2;     // [64][64]
constexpr size_t WF_W3 = WF_W2 + 64 * 64 * 2;     // [64][64]
constexpr size_t WF_W4 = WF_W3 + 64 * 64 * 2;     // [8][64]
constexpr size_t WF_B1 = WF_W4 + 8 * 64 * 2;      // f32 [64]
constexpr size_t WF_B2 = WF_B1 + 64 * 4;
constexpr size_t WF_B3 = WF_B2 + 64 * 4;
constexpr size_t WF_B4 = WF_B3 + 64 * 4;          // [8]
constexpr size_t WF_MU = WF_B4 + 8 * 4;           // [32]
constexpr size_t WF_IS = WF_MU + 32 * 4;          // [32]
constexpr size_t WF_OS = WF_IS + 32 * 4;          // [4]
constexpr size_t WF_BYTES = WF_OS + 16;
constexpr int kWfWarps = 4;                       // worlds in flight per CTA

// bytes of one warp's body rows, and of a CTA
template <class R, class W> __host__ __device__ inline size_t wf_slot_bytes(int nbs) {
  return ((size_t)7 * nbs * sizeof(W) + (size_t)20 * nbs * sizeof(R) + (size_t)((nbs + 15) & ~15) + 15) & ~(size_t)15;
}
template <class R, class W> __host__ __device__ inline size_t wf_smem_bytes(int nbs) {
  return WF_BYTES + kWfWarps * wf_slot_bytes<R, W>(nbs);
}

// The learned warm start's features and predictions, ahead of k_resolve and
// off its sequential path: one warp per world, kWfWarps worlds per CTA, the
// network's weights staged once per CTA in shared memory.  A warp takes the
// worlds k_resolve will warm-start (in harvest mode, v.mode == 1: every world
// it solves), stages the bodies, runs calculateInternals (prepare_contact) into
// the world's global working rows, accumulates the per-body aggregates
// (integer atomics: order-free, deterministic) and computes each contact's
// features; mode 2 predicts the impulses in 16-contact BF16 tensor-core tiles
// into the impulse rows, mode 1 writes the features to ws_feat for the harvest.
// Same bodies, contacts and arithmetic as k_resolve's own prepareContacts, so
// the features describe the state adjustVelocities starts from.
template <class R, class W>
__global__ void __launch_bounds__(32 * kWfWarps) k_warm_features(BatchView<R> v, int nbs, R dt) {
  extern __shared__ __align__(128) unsigned char smem[];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  // weights: global (v.mlp) -> shared
  {
    auto copy = [&](size_t off, const void* src, size_t bytes) {
      const uint4* s4 = reinterpret_cast<const uint4*>(src);
      uint4* d4 = reinterpret_cast<uint4*>(smem + off);
      for (size_t i = tid; i < bytes / 16; i += blockDim.x) d4[i] = s4[i];
    };
    if (v.mode == 2) {
      copy(WF_W1, v.mlp.W1, 64 * 32 * 2);
      copy(WF_W2, v.mlp.W2, 64 * 64 * 2);
      copy(WF_W3, v.mlp.W3, 64 * 64 * 2);
      copy(WF_W4, v.mlp.W4, 8 * 64 * 2);
      copy(WF_B1, v.mlp.b1, 64 * 4);
      copy(WF_B2, v.mlp.b2, 64 * 4);
      copy(WF_B3, v.mlp.b3, 64 * 4);
      copy(WF_B4, v.mlp.b4, 8 * 4);
      float* mu = reinterpret_cast<float*>(smem + WF_MU);
      float* is = reinterpret_cast<float*>(smem + WF_IS);
      float* os = reinterpret_cast<float*>(smem + WF_OS);
      for (int c = tid; c < 32; c += blockDim.x) {
        mu[c] = c < MLP_IN ? v.mlp.mu[c] : 0.f;
        is[c] = c < MLP_IN ? v.mlp.inv_sigma[c] : 0.f;
      }
      for (int c = tid; c < 4; c += blockDim.x) os[c] = c < MLP_OUT ? v.mlp.out_scale[c] : 0.f;
    }
  }
  __syncthreads();
  MlpDev m;
  m.W1 = reinterpret_cast<const __nv_bfloat16*>(smem + WF_W1);
  m.W2 = reinterpret_cast<const __nv_bfloat16*>(smem + WF_W2);
  m.W3 = reinterpret_cast<const __nv_bfloat16*>(smem + WF_W3);
  m.W4 = reinterpret_cast<const __nv_bfloat16*>(smem + WF_W4);
  m.b1 = reinterpret_cast<const float*>(smem + WF_B1);
  m.b2 = reinterpret_cast<const float*>(smem + WF_B2);
  m.b3 = reinterpret_cast<const float*>(smem + WF_B3);
  m.b4 = reinterpret_cast<const float*>(smem + WF_B4);
  const float* mu = reinterpret_cast<const float*>(smem + WF_MU);
  const float* isg = reinterpret_cast<const float*>(smem + WF_IS);
  const float* osc = reinterpret_cast<const float*>(smem + WF_OS);
  unsigned char* slot = smem + WF_BYTES + (size_t)wid * wf_slot_bytes<R, W>(nbs);
  RCtx<R, W> x;
  x.nbs = nbs;
  x.dt = dt;
  x.bw = reinterpret_cast<W*>(slot);
  x.br = reinterpret_cast<R*>(x.bw + 7 * nbs);
  x.aw = reinterpret_cast<uint8_t*>(x.br + 20 * nbs);
  x.bc = nullptr;
  x.save = x.delta = nullptr;
  x.kw = nullptr;
  const bool harvest = v.mode == 1;
  for (;;) {
    unsigned q = 0;
    if (lane == 0) q = atomicAdd(&v.queue[2], 1u);
    q = __shfl_sync(FULL, q, 0);
    if (q >= (unsigned)v.num_worlds) break;
    const int w = (int)q;
    const int n = v.body_count[w];
    int C = v.contact_count[w];
    const int cap = v.contact_cap[w];
    if (C > cap) C = cap;
    const int max_it = v.max_iterations >= 0 ? v.max_iterations : C * v.iter_mult;
    // the worlds k_resolve solves, and warm-starts unless solving plainly
    if (C <= 0 || dt <= (R)0 || n > nbs || max_it <= 0 || (!harvest && v.ws_world[w])) continue;
    const long long bstart = v.body_start[w];
    const long long cst = v.contact_start[w];
    x.cw = v.work + cst;
    x.cb = v.work_bodies + cst;
    x.cst = v.nc_total;
    x.gmat = v.uniform_material ? nullptr : v.contact + (long long)C_FRIC * v.nc_total + cst;
    x.gst = (long long)(C_REST - C_FRIC) * v.nc_total;
    x.wi = v.ws_int + bstart;
    x.wst = v.nb_pad;
    x.jw = v.work + (long long)W_J0 * v.nc_total + cst;
    x.jst = v.nc_total;
    x.delta = v.ws_rows + 7 * v.nb_pad + bstart;
    load_bodies(x, v, bstart, n, lane, 32);
    for (int i = lane; i < n; i += 32) {
      x.WI(WS_DEG, i) = 0;
      x.WI(WS_NBB, i) = 0;
      x.WI(WS_LOAD, i) = 0;
      x.WI(WS_FIRST, i) = 0x7fffffff;
      x.WI(WS_LAST, i) = -1;
    }
    __syncwarp();
    for (int k = lane; k < C; k += 32) {
      prepare_contact(x, v, cst + k, k);
      const int bb = x.cb[k];
      const int b0 = body0_of(bb), b1 = body1_of(bb);
      const float dd = (float)x.Cf(W_DDV, k);
      const int fx = dd > 0.f ? (int)(fminf(dd, 100.f) * kLoadScale + 0.5f) : 0;
      atomicAdd(&x.WI(WS_DEG, b0), 1);
      atomicAdd(&x.WI(WS_LOAD, b0), fx);
      if (b1 >= 0) {
        atomicAdd(&x.WI(WS_DEG, b1), 1);
        atomicAdd(&x.WI(WS_LOAD, b1), fx);
        atomicAdd(&x.WI(WS_NBB, b0), 1);
        atomicAdd(&x.WI(WS_NBB, b1), 1);
      } else {
        atomicMin(&x.WI(WS_FIRST, b0), k);
        atomicMax(&x.WI(WS_LAST, b0), k);
      }
    }
    __syncwarp();
    if (harvest) {
      for (int k = lane; k < C; k += 32) contact_features(x, k, v.ws_feat + (cst + k) * MLP_IN);
      __syncwarp();
      continue;
    }
    for (int t0 = 0; t0 < C; t0 += 16) {
      // lanes 0..15 compute one contact's normalised features each; the tile
      // reaches the MMA fragments and back by shuffles alone
      unsigned row[16];
      const int k = t0 + lane;
      const bool mine = lane < 16 && k < C;
      float f[MLP_IN];
      if (mine) contact_features(x, k, f);
#pragma unroll
      for (int c = 0; c < MLP_K1; c += 2) {
        float lo = 0.f, hi = 0.f;
        if (mine && c < MLP_IN) lo = (f[c] - mu[c]) * isg[c];
        if (mine && c + 1 < MLP_IN) hi = (f[c + 1] - mu[c + 1]) * isg[c + 1];
        row[c / 2] = pack_bf16(lo, hi);
      }
      unsigned a[2][4];
      rows_to_a(row, a);
      float o[4], y[3];
      mlp_forward_tile(m, a, o);
      out_to_rows(o, y);
      if (mine) {
#pragma unroll
        for (int c = 0; c < 3; ++c) x.J(c, k) = (R)(y[c] * osc[c]);
      }
    }
    __syncwarp();
    int nw = 0;
    float ssum = 0.f;
    warm_start_plan(x, n, C, lane, &nw, &ssum);
    if (nw) {
      atomicAdd(&v.counters[6], (unsigned long long)((double)ssum * 1e6 + 0.5));
      atomicAdd(&v.counters[7], (unsigned long long)nw);
    }
    __syncwarp();
  }
}

}  // namespace cz

