// Oracle: a CPU restatement of cubez's rigid-body step (TEST INFRASTRUCTURE).
//
// This file is the checker for the GPU kernels, not part of the product.  Only
// the tests, the smoke check and the CPU-baseline leg of the benchmark load it.
//
// It restates, operation for operation and in Go's left-to-right evaluation
// order, the reference files
//   math/math.go, math/vector.go, math/quaternion.go, math/matrix.go,
//   rigidbody.go, colliders.go, contact.go
// and the per-frame driver order of examples/cubedrop.go:29-75.  Every function
// cites the reference file:line it follows.  It must be compiled with
// -ffp-contract=off (no FMA contraction) and without -ffast-math.
//
// Two type parameters:
//   R  the bulk arithmetic type (double in the plain form, float in the
//      precision form);
//   W  the "island" type used where the precision form keeps FP64: quaternion
//      renormalisation, the per-body position/orientation accumulated across
//      adjustPositions, and the contact-frame 3x3 inversion of the friction
//      impulse.  In the plain form W == R == double, so the islands vanish.
//
// Parity status: the reference's own tests pin only the math layer
// (math/*_test.go); those known answers are re-asserted against this file by
// tests/test_oracle_math.py.  No reference test pins Integrate, the colliders
// or the resolver, and no Go toolchain is available to run the reference, so
// step-level parity is anchored on this restatement plus hand-built
// known-answer cases for every narrowphase branch.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>

namespace orc {

// ---------------------------------------------------------------- math.go

// math/math.go:27-33
template <class R> struct K {
  static constexpr R Epsilon = (R)1e-7;
  static constexpr R MinNormal = (R)1.1754943508222875e-38;
  static constexpr R MaxValue = std::numeric_limits<R>::max();
};

template <class R> inline R Abs(R a) { return std::fabs(a); }
template <class R> inline R Sqrt(R a) { return std::sqrt(a); }

// RealEqual, math/math.go:64-78
template <class R> inline bool RealEqual(R a, R b) {
  if (a == b) return true;
  R diff = Abs<R>(a - b);
  if (a * b == 0 || diff < K<R>::MinNormal) return diff < K<R>::Epsilon * K<R>::Epsilon;
  return diff / (Abs<R>(a) + Abs<R>(b)) < K<R>::Epsilon;
}

// ---------------------------------------------------------------- vector.go

template <class R> struct V3 {
  R v[3];
  R& operator[](int i) { return v[i]; }
  const R& operator[](int i) const { return v[i]; }
};
template <class R> struct Q4 {  // (w, x, y, z), math/math.go:58-59
  R v[4];
  R& operator[](int i) { return v[i]; }
  const R& operator[](int i) const { return v[i]; }
};
template <class R> struct M3 {  // column-major, math/math.go:41-42
  R m[9];
  R& operator[](int i) { return m[i]; }
  const R& operator[](int i) const { return m[i]; }
};
template <class R> struct M34 {  // column-major 3x4, math/math.go:44-47
  R m[12];
  R& operator[](int i) { return m[i]; }
  const R& operator[](int i) const { return m[i]; }
};

template <class R> inline V3<R> mk3(R a, R b, R c) { V3<R> r; r[0] = a; r[1] = b; r[2] = c; return r; }

// vector.go:14-19 Add
template <class R> inline void Add(V3<R>& v, const V3<R>& o) { v[0] += o[0]; v[1] += o[1]; v[2] += o[2]; }
// vector.go:21-26 AddScaled
template <class R> inline void AddScaled(V3<R>& v, const V3<R>& o, R s) {
  v[0] += o[0] * s; v[1] += o[1] * s; v[2] += o[2] * s;
}
// vector.go:28-31 Clear
template <class R> inline void Clear(V3<R>& v) { v[0] = 0; v[1] = 0; v[2] = 0; }
// vector.go:33-38 ComponentProduct
template <class R> inline void ComponentProduct(V3<R>& v, const V3<R>& o) { v[0] *= o[0]; v[1] *= o[1]; v[2] *= o[2]; }
// vector.go:40-47 Cross
template <class R> inline V3<R> Cross(const V3<R>& v, const V3<R>& o) {
  return mk3<R>(v[1] * o[2] - v[2] * o[1], v[2] * o[0] - v[0] * o[2], v[0] * o[1] - v[1] * o[0]);
}
// vector.go:49-52 Dot
template <class R> inline R Dot(const V3<R>& v, const V3<R>& o) { return v[0] * o[0] + v[1] * o[1] + v[2] * o[2]; }
// vector.go:54-57 Magnitude
template <class R> inline R Magnitude(const V3<R>& v) { return Sqrt<R>(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); }
// vector.go:59-62 SquareMagnitude
template <class R> inline R SquareMagnitude(const V3<R>& v) { return v[0] * v[0] + v[1] * v[1] + v[2] * v[2]; }
// vector.go:64-69 MulWith
template <class R> inline void MulWith(V3<R>& v, R r) { v[0] *= r; v[1] *= r; v[2] *= r; }
// vector.go:71-80 Normalize
template <class R> inline void Normalize(V3<R>& v) {
  R m = Magnitude(v);
  if (!RealEqual<R>(m, (R)0.0)) {
    R l = (R)1.0 / m;
    v[0] *= l; v[1] *= l; v[2] *= l;
  }
}
// vector.go:89-94 Sub
template <class R> inline void Sub(V3<R>& v, const V3<R>& o) { v[0] -= o[0]; v[1] -= o[1]; v[2] -= o[2]; }

// ---------------------------------------------------------------- quaternion.go

// quaternion.go:35-38 SetIdentity
template <class R> inline void SetIdentity(Q4<R>& q) { q[0] = 1; q[1] = 0; q[2] = 0; q[3] = 0; }
// quaternion.go:40-43 Len
template <class R> inline R Len(const Q4<R>& q) { return Sqrt<R>(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]); }
// quaternion.go:45-53 Mul (q = q * q2)
template <class R> inline void Mul(Q4<R>& q, const Q4<R>& q2) {
  R w = q[0] * q2[0] - q[1] * q2[1] - q[2] * q2[2] - q[3] * q2[3];
  R x = q[0] * q2[1] + q[1] * q2[0] + q[2] * q2[3] - q[3] * q2[2];
  R y = q[0] * q2[2] + q[2] * q2[0] + q[3] * q2[1] - q[1] * q2[3];
  R z = q[0] * q2[3] + q[3] * q2[0] + q[1] * q2[2] - q[2] * q2[1];
  q[0] = w; q[1] = x; q[2] = y; q[3] = z;
}
// quaternion.go:18-33 AddScaledVector
template <class R> inline void AddScaledVector(Q4<R>& q, const V3<R>& v, R scale) {
  Q4<R> t;
  t[0] = 0.0;
  t[1] = v[0] * scale;
  t[2] = v[1] * scale;
  t[3] = v[2] * scale;
  Mul(t, q);
  q[0] += t[0] * (R)0.5;
  q[1] += t[1] * (R)0.5;
  q[2] += t[2] * (R)0.5;
  q[3] += t[3] * (R)0.5;
}
// quaternion.go:77-99 Normalize
template <class R> inline void Normalize(Q4<R>& q) {
  R length = Len(q);
  if (RealEqual<R>((R)1.0, length)) return;
  if (length == (R)0.0) { SetIdentity(q); return; }
  if (length == std::numeric_limits<R>::infinity()) length = K<R>::MaxValue;
  R inv = (R)1.0 / length;
  q[0] *= inv; q[1] *= inv; q[2] *= inv; q[3] *= inv;
}
// quaternion.go:55-70 Rotate (used only by the math known-answer tests)
template <class R> inline V3<R> Rotate(const Q4<R>& q, const V3<R>& v) {
  V3<R> qvec = mk3<R>(q[1], q[2], q[3]);
  V3<R> cross = Cross(qvec, v);
  V3<R> result = v;
  MulWith<R>(qvec, (R)2.0);
  V3<R> c2 = Cross(qvec, cross);
  Add(result, c2);
  MulWith<R>(cross, (R)2.0 * q[0]);
  Add(result, cross);
  return result;
}

// ---------------------------------------------------------------- matrix.go

// matrix.go:14-19 SetIdentity (Matrix3)
template <class R> inline void SetIdentity(M3<R>& m) {
  for (int i = 0; i < 9; ++i) m[i] = 0;
  m[0] = 1; m[4] = 1; m[8] = 1;
}
// matrix.go:21-26 SetIdentity (Matrix3x4)
template <class R> inline void SetIdentity(M34<R>& m) {
  for (int i = 0; i < 12; ++i) m[i] = 0;
  m[0] = 1; m[4] = 1; m[8] = 1;
}
// matrix.go:36-47 Add
template <class R> inline void Add(M3<R>& m, const M3<R>& o) { for (int i = 0; i < 9; ++i) m[i] += o[i]; }
// matrix.go:52-56 SetComponents
template <class R> inline void SetComponents(M3<R>& m, const V3<R>& a, const V3<R>& b, const V3<R>& c) {
  m[0] = a[0]; m[3] = b[0]; m[6] = c[0];
  m[1] = a[1]; m[4] = b[1]; m[7] = c[1];
  m[2] = a[2]; m[5] = b[2]; m[8] = c[2];
}
// matrix.go:59-63 SetInertiaTensorCoeffs
template <class R> inline void SetInertiaTensorCoeffs(M3<R>& m, R ix, R iy, R iz, R ixy, R ixz, R iyz) {
  m[0] = ix; m[3] = -ixy; m[6] = -ixz;
  m[1] = -ixy; m[4] = iy; m[7] = -iyz;
  m[2] = -ixz; m[5] = -iyz; m[8] = iz;
}
// matrix.go:68-77 SetBlockInertiaTensor
template <class R> inline void SetBlockInertiaTensor(M3<R>& m, const V3<R>& half, R mass) {
  V3<R> sq = half;
  ComponentProduct(sq, half);
  SetInertiaTensorCoeffs<R>(m, (R)0.3 * mass * (sq[1] + sq[2]), (R)0.3 * mass * (sq[0] + sq[2]),
                            (R)0.3 * mass * (sq[0] + sq[1]), 0, 0, 0);
}
// matrix.go:79-86 MulVector3 (Matrix3)
template <class R> inline V3<R> MulVector3(const M3<R>& m, const V3<R>& v) {
  return mk3<R>(m[0] * v[0] + m[3] * v[1] + m[6] * v[2], m[1] * v[0] + m[4] * v[1] + m[7] * v[2],
                m[2] * v[0] + m[5] * v[1] + m[8] * v[2]);
}
// matrix.go:88-101 MulMatrix3
template <class R> inline M3<R> MulMatrix3(const M3<R>& a, const M3<R>& b) {
  M3<R> r;
  r[0] = a[0] * b[0] + a[3] * b[1] + a[6] * b[2];
  r[1] = a[1] * b[0] + a[4] * b[1] + a[7] * b[2];
  r[2] = a[2] * b[0] + a[5] * b[1] + a[8] * b[2];
  r[3] = a[0] * b[3] + a[3] * b[4] + a[6] * b[5];
  r[4] = a[1] * b[3] + a[4] * b[4] + a[7] * b[5];
  r[5] = a[2] * b[3] + a[5] * b[4] + a[8] * b[5];
  r[6] = a[0] * b[6] + a[3] * b[7] + a[6] * b[8];
  r[7] = a[1] * b[6] + a[4] * b[7] + a[7] * b[8];
  r[8] = a[2] * b[6] + a[5] * b[7] + a[8] * b[8];
  return r;
}
// matrix.go:103-114 MulWith (Matrix3)
template <class R> inline void MulWith(M3<R>& m, R s) { for (int i = 0; i < 9; ++i) m[i] *= s; }
// matrix.go:116-123 Transpose
template <class R> inline M3<R> Transpose(const M3<R>& m) {
  M3<R> r;
  r[0] = m[0]; r[1] = m[3]; r[2] = m[6];
  r[3] = m[1]; r[4] = m[4]; r[5] = m[7];
  r[6] = m[2]; r[7] = m[5]; r[8] = m[8];
  return r;
}
// matrix.go:125-129 Determinant
template <class R> inline R Determinant(const M3<R>& m) {
  return m[0] * m[4] * m[8] + m[3] * m[7] * m[2] + m[6] * m[1] * m[5] - m[6] * m[4] * m[2] - m[3] * m[1] * m[8] -
         m[0] * m[7] * m[5];
}
// matrix.go:131-153 Invert (returns the zero matrix when RealEqual(det, 0))
template <class R> inline M3<R> Invert(const M3<R>& m) {
  R det = Determinant(m);
  M3<R> r;
  if (RealEqual<R>(det, (R)0.0)) {
    for (int i = 0; i < 9; ++i) r[i] = 0;
    return r;
  }
  r[0] = m[4] * m[8] - m[5] * m[7];
  r[1] = m[2] * m[7] - m[1] * m[8];
  r[2] = m[1] * m[5] - m[2] * m[4];
  r[3] = m[5] * m[6] - m[3] * m[8];
  r[4] = m[0] * m[8] - m[2] * m[6];
  r[5] = m[2] * m[3] - m[0] * m[5];
  r[6] = m[3] * m[7] - m[4] * m[6];
  r[7] = m[1] * m[6] - m[0] * m[7];
  r[8] = m[0] * m[4] - m[1] * m[3];
  MulWith<R>(r, (R)1 / det);
  return r;
}
// matrix.go:155-163 TransformTranspose
template <class R> inline V3<R> TransformTranspose(const M3<R>& m, const V3<R>& v) {
  return mk3<R>(v[0] * m[0] + v[1] * m[1] + v[2] * m[2], v[0] * m[3] + v[1] * m[4] + v[2] * m[5],
                v[0] * m[6] + v[1] * m[7] + v[2] * m[8]);
}
// matrix.go:165-185 SetAsTransform
template <class R> inline void SetAsTransform(M34<R>& m, const V3<R>& pos, const Q4<R>& rot) {
  R w = rot[0], x = rot[1], y = rot[2], z = rot[3];
  m[0] = (R)1 - (R)2 * y * y - (R)2 * z * z;
  m[1] = (R)2 * x * y + (R)2 * w * z;
  m[2] = (R)2 * x * z - (R)2 * w * y;
  m[3] = (R)2 * x * y - (R)2 * w * z;
  m[4] = (R)1 - (R)2 * x * x - (R)2 * z * z;
  m[5] = (R)2 * y * z + (R)2 * w * x;
  m[6] = (R)2 * x * z + (R)2 * w * y;
  m[7] = (R)2 * y * z - (R)2 * w * x;
  m[8] = (R)1 - (R)2 * x * x - (R)2 * y * y;
  m[9] = pos[0];
  m[10] = pos[1];
  m[11] = pos[2];
}
// matrix.go:187-194 MulVector3 (Matrix3x4)
template <class R> inline V3<R> MulVector3(const M34<R>& m, const V3<R>& v) {
  return mk3<R>(v[0] * m[0] + v[1] * m[3] + v[2] * m[6] + m[9], v[0] * m[1] + v[1] * m[4] + v[2] * m[7] + m[10],
                v[0] * m[2] + v[1] * m[5] + v[2] * m[8] + m[11]);
}
// matrix.go:196-217 MulMatrix3x4
template <class R> inline M34<R> MulMatrix3x4(const M34<R>& m, const M34<R>& o) {
  M34<R> r;
  r[0] = m[0] * o[0] + m[3] * o[1] + m[6] * o[2];
  r[1] = m[1] * o[0] + m[4] * o[1] + m[7] * o[2];
  r[2] = m[2] * o[0] + m[5] * o[1] + m[8] * o[2];
  r[3] = m[0] * o[3] + m[3] * o[4] + m[6] * o[5];
  r[4] = m[1] * o[3] + m[4] * o[4] + m[7] * o[5];
  r[5] = m[2] * o[3] + m[5] * o[4] + m[8] * o[5];
  r[6] = m[0] * o[6] + m[3] * o[7] + m[6] * o[8];
  r[7] = m[1] * o[6] + m[4] * o[7] + m[7] * o[8];
  r[8] = m[2] * o[6] + m[5] * o[7] + m[8] * o[8];
  r[9] = m[0] * o[9] + m[3] * o[10] + m[6] * o[11] + m[9];
  r[10] = m[1] * o[9] + m[4] * o[10] + m[7] * o[11] + m[10];
  r[11] = m[2] * o[9] + m[5] * o[10] + m[8] * o[11] + m[11];
  return r;
}
// matrix.go:219-233 TransformInverse
template <class R> inline V3<R> TransformInverse(const M34<R>& m, const V3<R>& v) {
  V3<R> t = v;
  t[0] -= m[9];
  t[1] -= m[10];
  t[2] -= m[11];
  return mk3<R>(t[0] * m[0] + t[1] * m[1] + t[2] * m[2], t[0] * m[3] + t[1] * m[4] + t[2] * m[5],
                t[0] * m[6] + t[1] * m[7] + t[2] * m[8]);
}
// matrix.go:235-247 GetAxis
template <class R> inline V3<R> GetAxis(const M34<R>& m, int col) {
  int i = col > 3 ? 3 : col;
  return mk3<R>(m[i * 3 + 0], m[i * 3 + 1], m[i * 3 + 2]);
}

// conversions between the bulk and island types
template <class A, class B> inline V3<A> cv3(const V3<B>& v) { return mk3<A>((A)v[0], (A)v[1], (A)v[2]); }
template <class A, class B> inline Q4<A> cq4(const Q4<B>& q) {
  Q4<A> r; r[0] = (A)q[0]; r[1] = (A)q[1]; r[2] = (A)q[2]; r[3] = (A)q[3]; return r;
}
template <class A, class B> inline M3<A> cm3(const M3<B>& m) { M3<A> r; for (int i = 0; i < 9; ++i) r[i] = (A)m[i]; return r; }

// Orientation.AddScaledVector(v, 1.0) of an orientation held in W across
// adjustPositions (contact.go:374-375): the increment t = (0, v) * q and
// t * 0.5 in R, from q rounded to R, added to q in W.  With R == W this is
// AddScaledVector (quaternion.go:18-33) itself.
template <class R, class W> inline void AddScaledVectorIsland(Q4<W>& q, const V3<R>& v) {
  Q4<R> qr = cq4<R>(q);
  Q4<R> t;
  t[0] = 0.0;
  t[1] = v[0] * (R)1.0;
  t[2] = v[1] * (R)1.0;
  t[3] = v[2] * (R)1.0;
  Mul(t, qr);
  q[0] += (W)(t[0] * (R)0.5);
  q[1] += (W)(t[1] * (R)0.5);
  q[2] += (W)(t[2] * (R)0.5);
  q[3] += (W)(t[3] * (R)0.5);
}

// ---------------------------------------------------------------- rigidbody.go

enum Shape : int32_t { kSphere = 0, kCube = 1 };

// RigidBody (rigidbody.go:23-101) merged with its collider (colliders.go:37-71);
// the collider Offset defaults to the identity set by NewCollisionSphere/Cube
// (colliders.go:138,267).  Orientation is kept in the island type W so the
// precision form can accumulate adjustPositions corrections in FP64.
template <class R, class W> struct Body {
  R linearDamping, angularDamping;
  V3<R> position;
  Q4<R> orientation;
  V3<R> velocity, acceleration, rotation;
  M3<R> inverseInertiaTensor;
  bool isAwake, canSleep;
  M3<R> iitWorld;
  R inverseMass;
  M34<R> transform;
  V3<R> forceAccum, torqueAccum, lastFrameAccel;
  R motion;
  // collider
  int32_t shape;
  V3<R> halfSize;
  R radius;
  M34<R> offset;
  M34<R> ctransform;  // collider transform = body transform x Offset
};

constexpr double kSleepEpsilon = 0.3;  // rigidbody.go:14

// transformInertiaTensor, rigidbody.go:274-299
template <class R> inline void transformInertiaTensor(M3<R>& w, const M3<R>& b, const M34<R>& r) {
  R t4 = r[0] * b[0] + r[3] * b[1] + r[6] * b[2];
  R t9 = r[0] * b[3] + r[3] * b[4] + r[6] * b[5];
  R t14 = r[0] * b[6] + r[3] * b[7] + r[6] * b[8];
  R t28 = r[1] * b[0] + r[4] * b[1] + r[7] * b[2];
  R t33 = r[1] * b[3] + r[4] * b[4] + r[7] * b[5];
  R t38 = r[1] * b[6] + r[4] * b[7] + r[7] * b[8];
  R t52 = r[2] * b[0] + r[5] * b[1] + r[8] * b[2];
  R t57 = r[2] * b[3] + r[5] * b[4] + r[8] * b[5];
  R t62 = r[2] * b[6] + r[5] * b[7] + r[8] * b[8];
  w[0] = t4 * r[0] + t9 * r[3] + t14 * r[6];
  w[3] = t4 * r[1] + t9 * r[4] + t14 * r[7];
  w[6] = t4 * r[2] + t9 * r[5] + t14 * r[8];
  w[1] = t28 * r[0] + t33 * r[3] + t38 * r[6];
  w[4] = t28 * r[1] + t33 * r[4] + t38 * r[7];
  w[7] = t28 * r[2] + t33 * r[5] + t38 * r[8];
  w[2] = t52 * r[0] + t57 * r[3] + t62 * r[6];
  w[5] = t52 * r[1] + t57 * r[4] + t62 * r[7];
  w[8] = t52 * r[2] + t57 * r[5] + t62 * r[8];
}

// Quaternion renormalisation of an orientation held in W (quaternion.go:
// 77-99).  The plain form (R == W) is Normalize.  The precision form's
// float64 island: with s = |q|^2 and e = s - 1, nothing when |e| < 4e-7
// (where RealEqual(1, |q|) holds), q * 1/sqrt(s) from its five-term Taylor
// series in e when |e| < 2^-11 (IEEE multiplies and adds only), else
// Normalize.
template <class R, class W> inline void NormalizeW(Q4<W>& q) {
  if (sizeof(R) == sizeof(W)) {
    Normalize(q);
    return;
  }
  const W s = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
  const W e = s - (W)1;
  const W ae = e < (W)0 ? -e : e;
  if (ae < (W)4e-7) return;
  if (ae < (W)0x1p-11) {
    const W inv = (W)1 + e * ((W)-0.5 + e * ((W)0.375 + e * ((W)-0.3125 + e * (W)0.2734375)));
    q[0] *= inv; q[1] *= inv; q[2] *= inv; q[3] *= inv;
    return;
  }
  Normalize(q);
}

// Quaternion renormalisation, in W (rigidbody.go:269 -> quaternion.go:78-99)
template <class R, class W> inline void NormalizeIsland(Q4<R>& q) {
  Q4<W> qw = cq4<W>(q);
  NormalizeW<R, W>(qw);
  q = cq4<R>(qw);
}

// CalculateDerivedData, rigidbody.go:268-272
template <class R, class W> inline void CalculateDerivedData(Body<R, W>& b) {
  NormalizeIsland<R, W>(b.orientation);
  SetAsTransform(b.transform, b.position, b.orientation);
  transformInertiaTensor(b.iitWorld, b.inverseInertiaTensor, b.transform);
}
// Collider CalculateDerivedData, colliders.go:173-176 / 302-304
template <class R, class W> inline void ColliderDerivedData(Body<R, W>& b) {
  b.ctransform = MulMatrix3x4(b.transform, b.offset);
}
// SetAwake, rigidbody.go:182-192
template <class R, class W> inline void SetAwake(Body<R, W>& b, bool awake) {
  if (awake) {
    b.isAwake = true;
    b.motion = (R)(kSleepEpsilon * 2.0);
  } else {
    b.isAwake = false;
    Clear(b.velocity);
    Clear(b.rotation);
  }
}

// Integrate, rigidbody.go:213-259.  The two damping factors
// pow(LinearDamping, dt), pow(AngularDamping, dt) and the sleep bias
// pow(0.5, dt) are computed once on the host and passed in.
template <class R, class W>
inline void Integrate(Body<R, W>& b, R duration, R linPow, R angPow, R sleepBias) {
  if (b.isAwake == false) return;
  b.lastFrameAccel = b.acceleration;
  AddScaled(b.lastFrameAccel, b.forceAccum, b.inverseMass);
  V3<R> angAcc = MulVector3(b.iitWorld, b.torqueAccum);
  AddScaled(b.velocity, b.lastFrameAccel, duration);
  AddScaled(b.rotation, angAcc, duration);
  MulWith(b.velocity, linPow);
  MulWith(b.rotation, angPow);
  AddScaled(b.position, b.velocity, duration);
  AddScaledVector(b.orientation, b.rotation, duration);
  CalculateDerivedData(b);
  Clear(b.forceAccum);
  Clear(b.torqueAccum);
  if (b.canSleep) {
    R currentMotion = Dot(b.velocity, b.velocity) + Dot(b.rotation, b.rotation);
    R bias = sleepBias;
    b.motion = bias * b.motion + ((R)1.0 - bias) * currentMotion;
    if (b.motion < (R)kSleepEpsilon) {
      SetAwake(b, false);
    } else if (b.motion > (R)(10 * kSleepEpsilon)) {
      b.motion = (R)(10 * kSleepEpsilon);
    }
  }
}

// ---------------------------------------------------------------- contact.go (struct)

// Contact, contact.go:17-51.  Bodies are world-local indices, -1 for nil.
template <class R> struct Contact {
  int32_t body[2];
  R friction, restitution;
  V3<R> point, normal;
  R penetration;
  M3<R> contactToWorld;
  V3<R> relPos[2];
  V3<R> contactVelocity;
  R desiredDeltaVelocity;
};

template <class R> inline Contact<R> NewContact() {  // contact.go:53-57
  Contact<R> c;
  std::memset(&c, 0, sizeof(c));
  c.body[0] = -1;
  c.body[1] = -1;
  return c;
}

// Status bits raised where the Go reference would panic.
enum : uint32_t {
  kErrNonFinite = 1u,         // CheckAgainstCube reached with no tried axis (NaN state)
  kErrFrictionlessNil = 2u,   // calculateFrictionlessImpulse with Bodies[1]==nil (contact.go:512)
  kErrCapacity = 4u,
  kErrBadBody = 8u,
};

// ---------------------------------------------------------------- colliders.go

// Plane, colliders.go:29-35
template <class R> struct Plane {
  V3<R> normal;
  R offset;
};

// CollisionSphere.CheckAgainstHalfSpace, colliders.go:178-207
template <class R, class W>
inline bool SphereHalfSpace(const Body<R, W>& s, int si, const Plane<R>& p, std::vector<Contact<R>>& out) {
  V3<R> positionAxis = GetAxis(s.ctransform, 3);
  R distance = Dot(p.normal, positionAxis) - s.radius;
  if ((distance <= p.offset) == false) return false;
  Contact<R> c = NewContact<R>();
  c.point = p.normal;
  MulWith(c.point, distance + s.radius * (R)-1.0);
  Add(c.point, positionAxis);
  c.normal = p.normal;
  c.penetration = -distance;
  c.body[0] = si;
  c.body[1] = -1;
  c.friction = (R)0.9;
  c.restitution = (R)0.1;
  out.push_back(c);
  return true;
}

// CollisionSphere.CheckAgainstSphere, colliders.go:215-254
template <class R, class W>
inline bool SphereSphere(const Body<R, W>& s, int si, const Body<R, W>& t, int ti, std::vector<Contact<R>>& out) {
  V3<R> positionOne = GetAxis(s.ctransform, 3);
  V3<R> positionTwo = GetAxis(t.ctransform, 3);
  V3<R> midline = positionOne;
  Sub(midline, positionTwo);
  R size = Magnitude(midline);
  if (size <= (R)0.0 || size >= s.radius + t.radius) return false;
  Contact<R> c = NewContact<R>();
  c.point = midline;
  MulWith(c.point, (R)0.5);
  Add(c.point, positionOne);
  c.normal = midline;
  MulWith(c.normal, (R)1.0 / size);
  c.penetration = s.radius + t.radius - size;
  c.body[0] = si;
  c.body[1] = ti;
  c.friction = (R)0.9;
  c.restitution = (R)0.1;
  out.push_back(c);
  return true;
}

// transformToAxis, colliders.go:762-770
template <class R, class W> inline R transformToAxis(const Body<R, W>& cube, const V3<R>& axis) {
  V3<R> x = GetAxis(cube.ctransform, 0);
  V3<R> y = GetAxis(cube.ctransform, 1);
  V3<R> z = GetAxis(cube.ctransform, 2);
  return cube.halfSize[0] * Abs<R>(Dot(axis, x)) + cube.halfSize[1] * Abs<R>(Dot(axis, y)) +
         cube.halfSize[2] * Abs<R>(Dot(axis, z));
}

// intersectCubeAndHalfSpace, colliders.go:750-760
template <class R, class W> inline bool intersectCubeAndHalfSpace(const Body<R, W>& cube, const Plane<R>& p) {
  R projectedRadius = transformToAxis(cube, p.normal);
  V3<R> axis = GetAxis(cube.ctransform, 3);
  R cubeDistance = Dot(p.normal, axis) - projectedRadius;
  return cubeDistance <= p.offset;
}

// Vertex sign table, colliders.go:319-327
static const double kMults[8][3] = {{1, 1, 1}, {-1, 1, 1}, {1, -1, 1}, {-1, -1, 1},
                                    {1, 1, -1}, {-1, 1, -1}, {1, -1, -1}, {-1, -1, -1}};

// CollisionCube.CheckAgainstHalfSpace, colliders.go:306-366
template <class R, class W>
inline bool CubeHalfSpace(const Body<R, W>& cube, int ci, const Plane<R>& p, std::vector<Contact<R>>& out) {
  if (!intersectCubeAndHalfSpace(cube, p)) return false;
  bool detected = false;
  for (int k = 0; k < 8; ++k) {
    V3<R> v = mk3<R>((R)kMults[k][0], (R)kMults[k][1], (R)kMults[k][2]);
    ComponentProduct(v, cube.halfSize);
    V3<R> vertexPos = MulVector3(cube.ctransform, v);
    R vertexDistance = Dot(vertexPos, p.normal);
    if (vertexDistance <= p.offset) {
      Contact<R> c = NewContact<R>();
      c.point = p.normal;
      MulWith(c.point, vertexDistance - p.offset);
      Add(c.point, vertexPos);
      c.normal = p.normal;
      c.penetration = p.offset - vertexDistance;
      c.body[0] = ci;
      c.body[1] = -1;
      c.friction = (R)0.9;
      c.restitution = (R)0.1;
      out.push_back(c);
      detected = true;
    }
  }
  return detected;
}

// CollisionCube.CheckAgainstSphere, colliders.go:368-441
template <class R, class W>
inline bool CubeSphere(const Body<R, W>& cube, int ci, const Body<R, W>& sphere, int si, std::vector<Contact<R>>& out) {
  V3<R> position = GetAxis(sphere.ctransform, 3);
  V3<R> relCenter = TransformInverse(cube.ctransform, position);
  if (Abs<R>(relCenter[0]) - sphere.radius > cube.halfSize[0] ||
      Abs<R>(relCenter[1]) - sphere.radius > cube.halfSize[1] ||
      Abs<R>(relCenter[2]) - sphere.radius > cube.halfSize[2])
    return false;
  V3<R> closest;
  for (int i = 0; i < 3; ++i) {
    R dist = relCenter[i];
    if (dist > cube.halfSize[i]) {
      dist = cube.halfSize[i];
    } else if (dist < -cube.halfSize[i]) {
      dist = -cube.halfSize[i];
    }
    closest[i] = dist;
  }
  V3<R> distCheck = closest;
  Sub(distCheck, relCenter);
  R dist = SquareMagnitude(distCheck);
  if (dist > sphere.radius * sphere.radius) return false;
  V3<R> closestWorld = MulVector3(cube.ctransform, closest);
  Contact<R> c = NewContact<R>();
  c.point = closestWorld;
  c.normal = closestWorld;
  Sub(c.normal, position);
  // colliders.go:417-421.  The reference tests the world-space round trip
  // against RealEqual's absolute 1e-14, which float32 rounding exceeds, so
  // the precision form (R = float) also takes the fallback when the centre
  // needed no clamping (it lies in the box: the box-space distance is zero).
  if (RealEqual<R>(Magnitude(c.normal), (R)0.0) || (sizeof(R) < sizeof(double) && dist == (R)0)) {
    c.normal = sphere.velocity;
  }
  Normalize(c.normal);
  c.penetration = sphere.radius;
  if (!RealEqual<R>(dist, (R)0.0)) {
    c.penetration -= Sqrt<R>(dist);
  } else {
    c.penetration = 0.0;
  }
  c.body[0] = ci;
  c.body[1] = si;
  c.friction = (R)0.9;
  c.restitution = (R)0.1;
  out.push_back(c);
  return true;
}

// penetrationOnAxis, colliders.go:443-456
template <class R, class W>
inline R penetrationOnAxis(const Body<R, W>& one, const Body<R, W>& two, const V3<R>& axis, const V3<R>& toCenter) {
  R oneProject = transformToAxis(one, axis);
  R twoProject = transformToAxis(two, axis);
  R distance = Abs<R>(Dot(toCenter, axis));
  return oneProject + twoProject - distance;
}

// tryAxis, colliders.go:458-477.  Returns false on a separating axis.
template <class R, class W>
inline bool tryAxis(const Body<R, W>& one, const Body<R, W>& two, V3<R> axis, const V3<R>& toCenter, int index,
                    R& smallestPenetration, int& smallestCase) {
  if (SquareMagnitude(axis) < K<R>::Epsilon) return true;
  Normalize(axis);
  R penetration = penetrationOnAxis(one, two, axis, toCenter);
  if (penetration < (R)0) return false;
  if (penetration < smallestPenetration) {
    smallestPenetration = penetration;
    smallestCase = index;
  }
  return true;
}

// fillPointFaceBoxBox, colliders.go:479-517
template <class R, class W>
inline void fillPointFaceBoxBox(const Body<R, W>& one, int oi, const Body<R, W>& two, int ti, const V3<R>& toCenter,
                                int best, R pen, std::vector<Contact<R>>& out) {
  V3<R> normal = GetAxis(one.ctransform, best);
  if (Dot(normal, toCenter) > (R)0) MulWith(normal, (R)-1.0);
  V3<R> v = two.halfSize;
  if (Dot(GetAxis(two.ctransform, 0), normal) < (R)0) v[0] = -v[0];
  if (Dot(GetAxis(two.ctransform, 1), normal) < (R)0) v[1] = -v[1];
  if (Dot(GetAxis(two.ctransform, 2), normal) < (R)0) v[2] = -v[2];
  Contact<R> c = NewContact<R>();
  c.normal = normal;
  c.penetration = pen;
  c.point = MulVector3(two.ctransform, v);
  c.body[0] = oi;
  c.body[1] = ti;
  c.friction = (R)0.9;
  c.restitution = (R)0.1;
  out.push_back(c);
}

// contactPoint, colliders.go:519-573
template <class R>
inline V3<R> contactPoint(const V3<R>& pOne, const V3<R>& dOne, R oneSize, const V3<R>& pTwo, const V3<R>& dTwo,
                          R twoSize, bool useOne) {
  R smOne = SquareMagnitude(dOne);
  R smTwo = SquareMagnitude(dTwo);
  R dpOneTwo = Dot(dTwo, dOne);
  V3<R> toSt = pOne;
  Sub(toSt, pTwo);
  R dpStaOne = Dot(dOne, toSt);
  R dpStaTwo = Dot(dTwo, toSt);
  R denom = smOne * smTwo - dpOneTwo * dpOneTwo;
  if (Abs<R>(denom) < K<R>::Epsilon) return useOne ? pOne : pTwo;
  R mua = (dpOneTwo * dpStaTwo - smTwo * dpStaOne) / denom;
  R mub = (smOne * dpStaTwo - dpOneTwo * dpStaOne) / denom;
  if (mua > oneSize || mua < -oneSize || mub > twoSize || mub < -twoSize) return useOne ? pOne : pTwo;
  V3<R> cOne = dOne;
  MulWith(cOne, mua);
  Add(cOne, pOne);
  V3<R> cTwo = dTwo;
  MulWith(cTwo, mub);
  Add(cTwo, pTwo);
  MulWith(cOne, (R)0.5);
  MulWith(cTwo, (R)0.5);
  Add(cOne, cTwo);
  return cOne;
}

// CollisionCube.CheckAgainstCube, colliders.go:575-710
template <class R, class W>
inline bool CubeCube(const Body<R, W>& one, int oi, const Body<R, W>& two, int ti, std::vector<Contact<R>>& out,
                     uint32_t& err) {
  V3<R> toCenter = GetAxis(two.ctransform, 3);
  V3<R> oneAxis3 = GetAxis(one.ctransform, 3);
  Sub(toCenter, oneAxis3);
  R pen = K<R>::MaxValue;
  int best = 0xffffff;
  for (int i = 0; i <= 2; ++i)
    if (!tryAxis(one, two, GetAxis(one.ctransform, i), toCenter, i, pen, best)) return false;
  for (int i = 0; i <= 2; ++i)
    if (!tryAxis(one, two, GetAxis(two.ctransform, i), toCenter, i + 3, pen, best)) return false;
  int bestSingleAxis = best;
  for (int i = 0; i <= 2; ++i) {
    for (int j = 0; j <= 2; ++j) {
      V3<R> cross = Cross(GetAxis(one.ctransform, i), GetAxis(two.ctransform, j));
      if (!tryAxis(one, two, cross, toCenter, i * 3 + j + 6, pen, best)) return false;
    }
  }
  if (best < 3) {
    fillPointFaceBoxBox(one, oi, two, ti, toCenter, best, pen, out);
    return true;
  } else if (best < 6) {
    V3<R> newCenter = toCenter;
    MulWith(newCenter, (R)-1.0);
    fillPointFaceBoxBox(two, ti, one, oi, newCenter, best - 3, pen, out);
    return true;
  }
  if (best == 0xffffff) {
    // No axis was ever accepted: only reachable with non-finite transforms.
    // The Go code indexes HalfSize[5592403] here and panics.
    err |= kErrNonFinite;
    return false;
  }
  best -= 6;
  int oneAxisIndex = best / 3;
  int twoAxisIndex = best % 3;
  V3<R> oneAxis = GetAxis(one.ctransform, oneAxisIndex);
  V3<R> twoAxis = GetAxis(two.ctransform, twoAxisIndex);
  V3<R> axis = Cross(oneAxis, twoAxis);
  Normalize(axis);
  if (Dot(axis, toCenter) > (R)0) MulWith(axis, (R)-1.0);
  V3<R> ptOnOneEdge = one.halfSize;
  V3<R> ptOnTwoEdge = two.halfSize;
  for (int i = 0; i < 3; ++i) {
    if (i == oneAxisIndex) {
      ptOnOneEdge[i] = 0;
    } else if (Dot(GetAxis(one.ctransform, i), axis) > (R)0) {
      ptOnOneEdge[i] = -ptOnOneEdge[i];
    }
    if (i == twoAxisIndex) {
      ptOnTwoEdge[i] = 0;
    } else if (Dot(GetAxis(two.ctransform, i), axis) < (R)0) {
      ptOnTwoEdge[i] = -ptOnTwoEdge[i];
    }
  }
  ptOnOneEdge = MulVector3(one.ctransform, ptOnOneEdge);
  ptOnTwoEdge = MulVector3(two.ctransform, ptOnTwoEdge);
  bool useOne = bestSingleAxis > 2;
  V3<R> vertex = contactPoint(ptOnOneEdge, oneAxis, one.halfSize[oneAxisIndex], ptOnTwoEdge, twoAxis,
                              two.halfSize[twoAxisIndex], useOne);
  Contact<R> c = NewContact<R>();
  c.normal = axis;
  c.penetration = pen;
  c.point = vertex;
  c.body[0] = oi;
  c.body[1] = ti;
  c.friction = (R)0.9;
  c.restitution = (R)0.1;
  out.push_back(c);
  return true;
}

// CheckForCollisions, colliders.go:718-747, with the sphere->cube forwarding of
// colliders.go:209-213 and the plane forwarding of colliders.go:115-125.
template <class R, class W>
inline bool CheckForCollisions(const Body<R, W>& one, int oi, const Body<R, W>& two, int ti,
                               std::vector<Contact<R>>& out, uint32_t& err) {
  if (two.shape == kSphere) {
    if (one.shape == kSphere) return SphereSphere(one, oi, two, ti, out);
    return CubeSphere(one, oi, two, ti, out);
  }
  // two is a cube
  if (one.shape == kSphere) return CubeSphere(two, ti, one, oi, out);
  return CubeCube(one, oi, two, ti, out, err);
}

// Collider.CheckAgainstHalfSpace dispatch
template <class R, class W>
inline bool CheckAgainstHalfSpace(const Body<R, W>& b, int bi, const Plane<R>& p, std::vector<Contact<R>>& out) {
  if (b.shape == kSphere) return SphereHalfSpace(b, bi, p, out);
  return CubeHalfSpace(b, bi, p, out);
}

// generateContacts, examples/cubedrop.go:41-67: for each body the plane test,
// then every other body in list order (both (i,j) and (j,i) are tested).
template <class R, class W>
inline void GenerateContacts(const Body<R, W>* bodies, int n, const Plane<R>& p, std::vector<Contact<R>>& out,
                             uint32_t& err) {
  out.clear();
  for (int i = 0; i < n; ++i) {
    CheckAgainstHalfSpace(bodies[i], i, p, out);
    for (int j = 0; j < n; ++j) {
      if (j == i) continue;
      CheckForCollisions(bodies[i], i, bodies[j], j, out, err);
    }
  }
}

// ---------------------------------------------------------------- contact.go (resolver)

template <class R, class W> struct Resolver {
  Body<R, W>* bodies;  // world-local body array
  // Position/orientation held in W across adjustPositions (the precision
  // form's FP64 accumulators); identical to the body fields when W == R.
  std::vector<V3<W>> posW;
  std::vector<Q4<W>> oriW;
  uint32_t err = 0;
  int posIterations = 0, velIterations = 0;

  Body<R, W>& B(int i) { return bodies[i]; }

  // calculateContactBasis, contact.go:114-156
  static void calculateContactBasis(Contact<R>& c) {
    V3<R> ty, tz;
    R ax = Abs<R>(c.normal[0]);
    R ay = Abs<R>(c.normal[1]);
    if (ax > ay) {
      R s = (R)1.0 / Sqrt<R>(c.normal[2] * c.normal[2] + c.normal[0] * c.normal[0]);
      ty[0] = c.normal[2] * s;
      ty[1] = 0;
      ty[2] = c.normal[0] * -s;
      tz[0] = c.normal[1] * ty[0];
      tz[1] = c.normal[2] * ty[0] - c.normal[0] * ty[2];
      tz[2] = -c.normal[1] * ty[0];
    } else {
      R s = (R)1.0 / Sqrt<R>(c.normal[2] * c.normal[2] + c.normal[1] * c.normal[1]);
      ty[0] = 0;
      ty[1] = -c.normal[2] * s;
      ty[2] = c.normal[1] * s;
      tz[0] = c.normal[1] * ty[2] - c.normal[2] * ty[1];
      tz[1] = -c.normal[0] * ty[2];
      tz[2] = c.normal[0] * ty[1];
    }
    SetComponents(c.contactToWorld, c.normal, ty, tz);
  }

  // calculateLocalVelocity, contact.go:158-182
  V3<R> calculateLocalVelocity(Contact<R>& c, int bi, R duration) {
    Body<R, W>& body = B(c.body[bi]);
    V3<R> velocity = Cross(body.rotation, c.relPos[bi]);
    Add(velocity, body.velocity);
    V3<R> cvel = TransformTranspose(c.contactToWorld, velocity);
    V3<R> acc = body.lastFrameAccel;
    MulWith(acc, duration);
    acc = TransformTranspose(c.contactToWorld, acc);
    acc[0] = 0.0;
    Add(cvel, acc);
    return cvel;
  }

  // calculateDesiredDeltaVelocity, contact.go:87-112
  void calculateDesiredDeltaVelocity(Contact<R>& c, R duration) {
    const R velocityLimit = (R)0.25;
    R velocityFromAcc = 0;
    V3<R> tmp;
    if (B(c.body[0]).isAwake) {
      tmp = B(c.body[0]).lastFrameAccel;
      MulWith(tmp, duration);
      velocityFromAcc += Dot(tmp, c.normal);
    }
    if (c.body[1] >= 0 && B(c.body[1]).isAwake) {
      tmp = B(c.body[1]).lastFrameAccel;
      MulWith(tmp, duration);
      velocityFromAcc -= Dot(tmp, c.normal);
    }
    R restitution = c.restitution;
    if (Abs<R>(c.contactVelocity[0]) < velocityLimit) restitution = 0.0;
    c.desiredDeltaVelocity = -c.contactVelocity[0] - restitution * (c.contactVelocity[0] - velocityFromAcc);
  }

  // calculateInternals, contact.go:59-85
  void calculateInternals(Contact<R>& c, R duration) {
    if (c.body[0] < 0) {
      MulWith(c.normal, (R)-1.0);
      c.body[0] = c.body[1];
      c.body[1] = -1;
    }
    calculateContactBasis(c);
    c.relPos[0] = c.point;
    Sub(c.relPos[0], B(c.body[0]).position);
    c.contactVelocity = calculateLocalVelocity(c, 0, duration);
    if (c.body[1] >= 0) {
      c.relPos[1] = c.point;
      Sub(c.relPos[1], B(c.body[1]).position);
      V3<R> cv1 = calculateLocalVelocity(c, 1, duration);
      Sub(c.contactVelocity, cv1);
    }
    calculateDesiredDeltaVelocity(c, duration);
  }

  // matchAwakeState, contact.go:184-202
  void matchAwakeState(Contact<R>& c) {
    if (c.body[1] < 0) return;
    bool a0 = B(c.body[0]).isAwake, a1 = B(c.body[1]).isAwake;
    if ((a0 || a1) && !(a0 && a1)) {
      if (a0) SetAwake(B(c.body[1]), true);
      else SetAwake(B(c.body[0]), true);
    }
  }

  // applyPositionChange, contact.go:285-386
  void applyPositionChange(Contact<R>& c, R penetration, V3<R> linearChange[2], V3<R> angularChange[2]) {
    const R angularLimit = (R)0.2;
    R angularInertia[2] = {0, 0}, linearInertia[2] = {0, 0}, angularMove[2] = {0, 0}, linearMove[2] = {0, 0};
    R totalInertia = 0;
    Clear(linearChange[0]); Clear(linearChange[1]);
    Clear(angularChange[0]); Clear(angularChange[1]);
    for (int i = 0; i < 2; ++i) {
      if (c.body[i] < 0) continue;
      Body<R, W>& body = B(c.body[i]);
      M3<R> iit = body.iitWorld;
      V3<R> aiw = Cross(c.relPos[i], c.normal);
      aiw = MulVector3(iit, aiw);
      aiw = Cross(aiw, c.relPos[i]);
      angularInertia[i] = Dot(aiw, c.normal);
      linearInertia[i] = body.inverseMass;
      totalInertia += linearInertia[i] + angularInertia[i];
    }
    for (int i = 0; i < 2; ++i) {
      if (c.body[i] < 0) continue;
      Body<R, W>& body = B(c.body[i]);
      R sign = (i != 0) ? (R)-1.0 : (R)1.0;
      angularMove[i] = sign * penetration * (angularInertia[i] / totalInertia);
      linearMove[i] = sign * penetration * (linearInertia[i] / totalInertia);
      V3<R> projection = c.relPos[i];
      AddScaled(projection, c.normal, -Dot(c.relPos[i], c.normal));
      R maxMagnitude = angularLimit * Magnitude(projection);
      if (angularMove[i] < -maxMagnitude) {
        R totalMove = angularMove[i] + linearMove[i];
        angularMove[i] = -maxMagnitude;
        linearMove[i] = totalMove - angularMove[i];
      } else if (angularMove[i] > maxMagnitude) {
        R totalMove = angularMove[i] + linearMove[i];
        angularMove[i] = maxMagnitude;
        linearMove[i] = totalMove - angularMove[i];
      }
      if (angularMove[i] == (R)0.0) {
        Clear(angularChange[i]);
      } else {
        V3<R> tad = Cross(c.relPos[i], c.normal);
        M3<R> iit = body.iitWorld;
        angularChange[i] = MulVector3(iit, tad);
        MulWith(angularChange[i], angularMove[i] / angularInertia[i]);
      }
      linearChange[i] = c.normal;
      MulWith(linearChange[i], linearMove[i]);
      // Position.AddScaled(normal, linearMove): the product in R, accumulated in W.
      V3<W>& pw = posW[c.body[i]];
      pw[0] += (W)(c.normal[0] * linearMove[i]);
      pw[1] += (W)(c.normal[1] * linearMove[i]);
      pw[2] += (W)(c.normal[2] * linearMove[i]);
      // Orientation.AddScaledVector(angularChange, 1.0); Orientation.Normalize()
      // the increment in R from the orientation rounded to R, accumulated in W
      Q4<W>& qw = oriW[c.body[i]];
      AddScaledVectorIsland<R, W>(qw, angularChange[i]);
      NormalizeW<R, W>(qw);
      body.position = cv3<R>(pw);
      body.orientation = cq4<R>(qw);
      if (body.isAwake == false) {
        CalculateDerivedData(body);
        qw = cq4<W>(body.orientation);
      }
    }
  }

  // adjustPositions, contact.go:231-283
  void adjustPositions(int maxIterations, std::vector<Contact<R>>& cs, R duration) {
    (void)duration;
    int used = 0;
    const int n = (int)cs.size();
    while (used < maxIterations) {
      R max = (R)0.01;  // positionEpsilon, contact.go:13
      int index = n;
      for (int i = 0; i < n; ++i) {
        if (cs[i].penetration > max) {
          max = cs[i].penetration;
          index = i;
        }
      }
      if (index == n) break;
      Contact<R>& contact = cs[index];
      matchAwakeState(contact);
      V3<R> lin[2], ang[2];
      applyPositionChange(contact, max, lin, ang);
      for (int k = 0; k < n; ++k) {
        Contact<R>& c = cs[k];
        for (int b = 0; b < 2; ++b) {
          if (c.body[b] < 0) continue;
          for (int d = 0; d < 2; ++d) {
            if (c.body[b] == contact.body[d]) {
              V3<R> dp = Cross(ang[d], c.relPos[b]);
              Add(dp, lin[d]);
              R sign = (b == 0) ? (R)-1.0 : (R)1.0;
              c.penetration += Dot(dp, c.normal) * sign;
            }
          }
        }
      }
      ++used;
    }
    posIterations = used;
  }

  // calculateFrictionImpulse, contact.go:533-606; the 3x3 inversion and the
  // impulse solve run in W.
  V3<R> calculateFrictionImpulse(Contact<R>& c, const M3<R> iit[2]) {
    R inverseMass = B(c.body[0]).inverseMass;
    M3<R> itt;
    setSkewSymmetric(itt, c.relPos[0]);
    M3<R> dvw = MulMatrix3(itt, iit[0]);
    dvw = MulMatrix3(dvw, itt);
    MulWith(dvw, (R)-1.0);
    if (c.body[1] >= 0) {
      setSkewSymmetric(itt, c.relPos[1]);
      M3<R> dvw2 = MulMatrix3(itt, iit[1]);
      dvw2 = MulMatrix3(dvw2, itt);
      MulWith(dvw2, (R)-1.0);
      Add(dvw, dvw2);
      inverseMass += B(c.body[1]).inverseMass;
    }
    M3<R> dv = Transpose(c.contactToWorld);
    dv = MulMatrix3(dv, dvw);
    dv = MulMatrix3(dv, c.contactToWorld);
    dv[0] += inverseMass;
    dv[4] += inverseMass;
    dv[8] += inverseMass;
    // the inversion in W; the solve in R
    M3<R> impulseMatrix = cm3<R>(Invert(cm3<W>(dv)));
    V3<R> velKill = mk3<R>(c.desiredDeltaVelocity, -c.contactVelocity[1], -c.contactVelocity[2]);
    V3<R> ic = MulVector3(impulseMatrix, velKill);
    R planar = Sqrt<R>(ic[1] * ic[1] + ic[2] * ic[2]);
    if (planar > ic[0] * c.friction) {
      ic[1] /= planar;
      ic[2] /= planar;
      ic[0] = dv[0] + dv[3] * c.friction * ic[1] + dv[6] * c.friction * ic[2];
      ic[0] = c.desiredDeltaVelocity / ic[0];
      ic[1] *= c.friction * ic[0];
      ic[2] *= c.friction * ic[0];
    }
    return ic;
  }

  // calculateFrictionlessImpulse, contact.go:496-531 (only reached when
  // Friction == 0; the Go code dereferences a nil body when Bodies[1] is nil).
  V3<R> calculateFrictionlessImpulse(Contact<R>& c, const M3<R> iit[2]) {
    V3<R> dvw = Cross(c.relPos[0], c.normal);
    dvw = MulVector3(iit[0], dvw);
    dvw = Cross(dvw, c.relPos[0]);
    R deltaVelocity = Dot(dvw, c.normal);
    deltaVelocity += B(c.body[0]).inverseMass;
    if (c.body[1] < 0) {
      err |= kErrFrictionlessNil;
    }
    return mk3<R>(c.desiredDeltaVelocity / deltaVelocity, 0, 0);
  }

  static void setSkewSymmetric(M3<R>& m, const V3<R>& v) {  // contact.go:612-616
    m[0] = 0.0; m[3] = -v[2]; m[6] = v[1];
    m[1] = v[2]; m[4] = 0.0; m[7] = -v[0];
    m[2] = -v[1]; m[5] = v[0]; m[8] = 0.0;
  }

  // applyVelocityChange, contact.go:447-494
  void applyVelocityChange(Contact<R>& c, V3<R> velocityChange[2], V3<R> rotationChange[2]) {
    M3<R> iit[2];
    iit[0] = B(c.body[0]).iitWorld;
    for (int i = 0; i < 9; ++i) iit[1][i] = 0;
    if (c.body[1] >= 0) iit[1] = B(c.body[1]).iitWorld;
    V3<R> ic;
    if (c.friction == (R)0.0) ic = calculateFrictionlessImpulse(c, iit);
    else ic = calculateFrictionImpulse(c, iit);
    V3<R> impulse = MulVector3(c.contactToWorld, ic);
    V3<R> torque = Cross(c.relPos[0], impulse);
    rotationChange[0] = MulVector3(iit[0], torque);
    Clear(velocityChange[0]);
    AddScaled(velocityChange[0], impulse, B(c.body[0]).inverseMass);
    Add(B(c.body[0]).velocity, velocityChange[0]);
    Add(B(c.body[0]).rotation, rotationChange[0]);
    Clear(velocityChange[1]);
    Clear(rotationChange[1]);
    if (c.body[1] >= 0) {
      torque = Cross(impulse, c.relPos[1]);
      rotationChange[1] = MulVector3(iit[1], torque);
      Clear(velocityChange[1]);
      AddScaled(velocityChange[1], impulse, -B(c.body[1]).inverseMass);
      Add(B(c.body[1]).velocity, velocityChange[1]);
      Add(B(c.body[1]).rotation, rotationChange[1]);
    }
  }

  // adjustVelocities, contact.go:388-445
  void adjustVelocities(int maxIterations, std::vector<Contact<R>>& cs, R duration) {
    int used = 0;
    const int n = (int)cs.size();
    while (used < maxIterations) {
      R max = (R)0.01;  // velocityEpsilon, contact.go:12
      int index = n;
      for (int i = 0; i < n; ++i) {
        if (cs[i].desiredDeltaVelocity > max) {
          max = cs[i].desiredDeltaVelocity;
          index = i;
        }
      }
      if (index == n) break;
      Contact<R>& contact = cs[index];
      matchAwakeState(contact);
      V3<R> vel[2], rot[2];
      applyVelocityChange(contact, vel, rot);
      for (int k = 0; k < n; ++k) {
        Contact<R>& c2 = cs[k];
        for (int b = 0; b < 2; ++b) {
          if (c2.body[b] < 0) continue;
          for (int d = 0; d < 2; ++d) {
            if (c2.body[b] == contact.body[d]) {
              V3<R> dv = Cross(rot[d], c2.relPos[b]);
              Add(dv, vel[d]);
              R sign = (b == 1) ? (R)-1.0 : (R)1.0;
              V3<R> t = TransformTranspose(c2.contactToWorld, dv);
              MulWith(t, sign);
              Add(c2.contactVelocity, t);
              calculateDesiredDeltaVelocity(c2, duration);
            }
          }
        }
      }
      ++used;
    }
    velIterations = used;
  }

  // ResolveContacts, contact.go:204-222
  void ResolveContacts(int maxIterations, std::vector<Contact<R>>& cs, R duration, int nbodies) {
    posIterations = velIterations = 0;
    if (duration <= (R)0.0 || cs.empty()) return;
    posW.resize(nbodies);
    oriW.resize(nbodies);
    for (int i = 0; i < nbodies; ++i) {
      posW[i] = cv3<W>(bodies[i].position);
      oriW[i] = cq4<W>(bodies[i].orientation);
    }
    for (auto& c : cs) calculateInternals(c, duration);  // prepareContacts, contact.go:224-229
    adjustPositions(maxIterations, cs, duration);
    adjustVelocities(maxIterations, cs, duration);
  }
};

// One world's frame in the order of examples/cubedrop.go:69-75:
// integrate + collider derived data for every body, ordered all-pairs
// narrowphase, then ResolveContacts(len(contacts) * iterMult).
template <class R, class W> struct StepStats {
  int contacts = 0, posIterations = 0, velIterations = 0;
  uint32_t err = 0;
};

template <class R, class W>
inline StepStats<R, W> StepWorld(Body<R, W>* bodies, int n, const Plane<R>& plane, R dt, const R* linPow,
                                 const R* angPow, R sleepBias, int iterMult, std::vector<Contact<R>>& contacts,
                                 std::vector<Contact<R>>* generated) {
  StepStats<R, W> st;
  for (int i = 0; i < n; ++i) {
    Integrate(bodies[i], dt, linPow[i], angPow[i], sleepBias);
    ColliderDerivedData(bodies[i]);
  }
  uint32_t err = 0;
  GenerateContacts(bodies, n, plane, contacts, err);
  if (generated) *generated = contacts;
  st.contacts = (int)contacts.size();
  if (!contacts.empty()) {
    Resolver<R, W> rs;
    rs.bodies = bodies;
    rs.ResolveContacts((int)contacts.size() * iterMult, contacts, dt, n);
    st.posIterations = rs.posIterations;
    st.velIterations = rs.velIterations;
    err |= rs.err;
  }
  st.err = err;
  return st;
}

}  // namespace orc
