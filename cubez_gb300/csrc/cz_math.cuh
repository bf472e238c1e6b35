// Device vector / quaternion / matrix operations of the rigid-body step.
//
// Each function evaluates in the same order as the reference's math package
// (Go evaluates left to right, no fused multiply-add), so that the plain FP64
// form produces the same bits as a correctly rounded CPU evaluation.  The
// translation units that include this header are compiled with --fmad=false;
// division and square root are IEEE round-to-nearest (no fast-math).
//
//   math/math.go:64-78        RealEqual
//   math/vector.go            Add/AddScaled/Cross/Dot/Magnitude/Normalize/...
//   math/quaternion.go:20-99  AddScaledVector, Mul, Normalize
//   math/matrix.go            Matrix3 / Matrix3x4 (column-major)
#pragma once
#include <cstdint>

namespace cz {

template <class R> struct Lim;
template <> struct Lim<double> {
  static __device__ __forceinline__ double eps() { return 1e-7; }
  static __device__ __forceinline__ double min_normal() { return 1.1754943508222875e-38; }
  static __device__ __forceinline__ double max_value() { return 1.7976931348623157e308; }
  static __device__ __forceinline__ double inf() { return __longlong_as_double(0x7FF0000000000000LL); }
};
template <> struct Lim<float> {
  static __device__ __forceinline__ float eps() { return 1e-7f; }
  static __device__ __forceinline__ float min_normal() { return 1.17549435e-38f; }
  static __device__ __forceinline__ float max_value() { return 3.40282347e38f; }
  static __device__ __forceinline__ float inf() { return __int_as_float(0x7F800000); }
};

template <class R> __device__ __forceinline__ R fabs_(R a) { return a < (R)0 ? -a : (a == (R)0 ? (R)0 : a); }
template <> __device__ __forceinline__ double fabs_<double>(double a) { return fabs(a); }
template <> __device__ __forceinline__ float fabs_<float>(float a) { return fabsf(a); }
template <class R> __device__ __forceinline__ R sqrt_(R a);
template <> __device__ __forceinline__ double sqrt_<double>(double a) { return sqrt(a); }
template <> __device__ __forceinline__ float sqrt_<float>(float a) { return sqrtf(a); }

// math/math.go:64-78
template <class R> __device__ __forceinline__ bool real_equal(R a, R b) {
  if (a == b) return true;
  R diff = fabs_<R>(a - b);
  if (a * b == (R)0 || diff < Lim<R>::min_normal()) return diff < Lim<R>::eps() * Lim<R>::eps();
  return diff / (fabs_<R>(a) + fabs_<R>(b)) < Lim<R>::eps();
}

template <class R> struct v3 {
  R x, y, z;
};
template <class R> struct q4 {
  R w, x, y, z;
};
// column-major 3x3 (m[col*3 + row])
template <class R> struct m3 {
  R m[9];
};

// float <-> double conversions by integer operations for the common cases
// (normal values and zeros; exact widening, round-to-nearest-even
// narrowing, as the conversion instructions), the conversion instruction
// for the rest.  On GB300 a conversion instruction has the latency of a
// float64 operation (about 80 cycles) and shares its slow pipe; these run on
// the integer pipe.  Same bits either way.
__device__ __forceinline__ double widen(float f) {
  const unsigned b = __float_as_uint(f);
  const unsigned e = (b >> 23) & 0xffu, m = b & 0x7fffffu, sign = b & 0x80000000u;
  if (e - 1u < 254u) return __hiloint2double((int)(sign | ((e + 896u) << 20) | (m >> 3)), (int)(m << 29));
  if ((b << 1) == 0u) return __hiloint2double((int)sign, 0);
  return (double)f;  // subnormal, infinite or NaN
}
__device__ __forceinline__ float narrow(double d) {
  const unsigned hi = (unsigned)__double2hiint(d), lo = (unsigned)__double2loint(d);
  const unsigned e = (hi >> 20) & 0x7ffu, sign = hi & 0x80000000u;
  if (e - 897u < 254u) {  // a normal float (or, rounding up from the top binade, infinity)
    unsigned r = ((e - 896u) << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29);
    const unsigned rest = lo & 0x1fffffffu;
    r += (rest > 0x10000000u || (rest == 0x10000000u && (r & 1u))) ? 1u : 0u;
    return __uint_as_float(sign | r);
  }
  if (((hi << 1) | lo) == 0u) return __uint_as_float(sign);
  return __double2float_rn(d);  // subnormal or out of range, infinite or NaN
}
// The integer-pipe conversion, for the sequential chain of adjustPositions
// (elsewhere the instruction: inlined everywhere, these cost registers).
template <class A, class B> __device__ __forceinline__ A cvt_fast(B x) {
  if constexpr (sizeof(A) == 8 && sizeof(B) == 4)
    return widen(x);
  else if constexpr (sizeof(A) == 4 && sizeof(B) == 8)
    return narrow(x);
  else
    return (A)x;
}

template <class R> __device__ __forceinline__ v3<R> V(R x, R y, R z) { return v3<R>{x, y, z}; }
template <class A, class B> __device__ __forceinline__ v3<A> cvt(const v3<B>& v) {
  return v3<A>{(A)(v.x), (A)(v.y), (A)(v.z)};
}
template <class A, class B> __device__ __forceinline__ q4<A> cvtq(const q4<B>& q) {
  return q4<A>{(A)(q.w), (A)(q.x), (A)(q.y), (A)(q.z)};
}

// vector.go:40-47
template <class R> __device__ __forceinline__ v3<R> cross(const v3<R>& a, const v3<R>& b) {
  return v3<R>{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
// vector.go:49-52
template <class R> __device__ __forceinline__ R dot(const v3<R>& a, const v3<R>& b) {
  return a.x * b.x + a.y * b.y + a.z * b.z;
}
// vector.go:59-62 / 54-57
template <class R> __device__ __forceinline__ R sqmag(const v3<R>& a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
template <class R> __device__ __forceinline__ R mag(const v3<R>& a) { return sqrt_<R>(a.x * a.x + a.y * a.y + a.z * a.z); }
// vector.go:14-19, 21-26, 64-69, 89-94
template <class R> __device__ __forceinline__ void add(v3<R>& a, const v3<R>& b) { a.x += b.x; a.y += b.y; a.z += b.z; }
template <class R> __device__ __forceinline__ void add_scaled(v3<R>& a, const v3<R>& b, R s) {
  a.x += b.x * s; a.y += b.y * s; a.z += b.z * s;
}
template <class R> __device__ __forceinline__ void mul_with(v3<R>& a, R s) { a.x *= s; a.y *= s; a.z *= s; }
template <class R> __device__ __forceinline__ void sub(v3<R>& a, const v3<R>& b) { a.x -= b.x; a.y -= b.y; a.z -= b.z; }
// vector.go:71-80
template <class R> __device__ __forceinline__ void normalize(v3<R>& a) {
  R m = mag(a);
  if (!real_equal<R>(m, (R)0)) {
    R l = (R)1 / m;
    a.x *= l; a.y *= l; a.z *= l;
  }
}

// quaternion.go:45-53 (q = q * p)
template <class R> __device__ __forceinline__ q4<R> qmul(const q4<R>& q, const q4<R>& p) {
  return q4<R>{q.w * p.w - q.x * p.x - q.y * p.y - q.z * p.z, q.w * p.x + q.x * p.w + q.y * p.z - q.z * p.y,
               q.w * p.y + q.y * p.w + q.z * p.x - q.x * p.z, q.w * p.z + q.z * p.w + q.x * p.y - q.y * p.x};
}
// quaternion.go:18-33
template <class R> __device__ __forceinline__ void add_scaled_vector(q4<R>& q, const v3<R>& v, R s) {
  q4<R> t{(R)0, v.x * s, v.y * s, v.z * s};
  t = qmul(t, q);
  q.w += t.w * (R)0.5;
  q.x += t.x * (R)0.5;
  q.y += t.y * (R)0.5;
  q.z += t.z * (R)0.5;
}
// AddScaledVector(v, 1) of an orientation held in the island type W
// (applyPositionChange, contact.go:374-375): the increment 0.5 * (v q) in R
// from q rounded to R, accumulated in W.  With R == W it is AddScaledVector.
template <class R, class W> __device__ __forceinline__ void add_scaled_vector_island(q4<W>& q, const v3<R>& v) {
  const q4<R> qr{cvt_fast<R>(q.w), cvt_fast<R>(q.x), cvt_fast<R>(q.y), cvt_fast<R>(q.z)};
  q4<R> t{(R)0, v.x * (R)1, v.y * (R)1, v.z * (R)1};
  t = qmul(t, qr);
  q.w += cvt_fast<W>(t.w * (R)0.5);
  q.x += cvt_fast<W>(t.x * (R)0.5);
  q.y += cvt_fast<W>(t.y * (R)0.5);
  q.z += cvt_fast<W>(t.z * (R)0.5);
}
// quaternion.go:77-99
template <class R> __device__ __forceinline__ void qnormalize(q4<R>& q) {
  R len = sqrt_<R>(q.w * q.w + q.x * q.x + q.y * q.y + q.z * q.z);
  if (real_equal<R>((R)1, len)) return;
  if (len == (R)0) {
    q = q4<R>{(R)1, (R)0, (R)0, (R)0};
    return;
  }
  if (len == Lim<R>::inf()) len = Lim<R>::max_value();
  R inv = (R)1 / len;
  q.w *= inv; q.x *= inv; q.y *= inv; q.z *= inv;
}

// Quaternion renormalisation in the precision form's float64 island (W =
// double, R = float).  A frame or a position change moves a unit quaternion
// a little, so s = |q|^2 is near 1; with e = s - 1:
//   |e| < 4e-7       nothing, where the reference's RealEqual(1, |q|) holds
//                    (|1 - |q|| < 1e-7 (1 + |q|), and |q| - 1 is e/2 to first
//                    order);
//   |e| < 2^-11      q times 1/sqrt(s) from its Taylor series in e, five
//                    terms by Horner (truncation below 1e-17): IEEE multiplies
//                    and adds only, eight dependent float64 operations instead
//                    of a square root and two divisions (about 30 dependent
//                    ones at ~100 cycles each on GB300);
//   otherwise        Normalize (quaternion.go:77-99) as the reference does.
// The oracle's island evaluates the same operations.  With R == W (the plain
// form) it is Normalize.
template <class R, class W> __device__ __forceinline__ void qnormalize_island(q4<W>& q) {
  if constexpr (sizeof(R) == sizeof(W)) {
    qnormalize(q);
  } else {
    const W s = q.w * q.w + q.x * q.x + q.y * q.y + q.z * q.z;
    const W e = s - (W)1;
    const W ae = fabs(e);
    if (ae < (W)4e-7) return;
    if (ae < (W)0x1p-11) {
      const W inv = (W)1 + e * ((W)-0.5 + e * ((W)0.375 + e * ((W)-0.3125 + e * (W)0.2734375)));
      q.w *= inv; q.x *= inv; q.y *= inv; q.z *= inv;
      return;
    }
    qnormalize(q);
  }
}

// matrix.go:79-86
template <class R> __device__ __forceinline__ v3<R> mulv(const m3<R>& a, const v3<R>& v) {
  return v3<R>{a.m[0] * v.x + a.m[3] * v.y + a.m[6] * v.z, a.m[1] * v.x + a.m[4] * v.y + a.m[7] * v.z,
               a.m[2] * v.x + a.m[5] * v.y + a.m[8] * v.z};
}
// matrix.go:155-163
template <class R> __device__ __forceinline__ v3<R> mulv_t(const m3<R>& a, const v3<R>& v) {
  return v3<R>{v.x * a.m[0] + v.y * a.m[1] + v.z * a.m[2], v.x * a.m[3] + v.y * a.m[4] + v.z * a.m[5],
               v.x * a.m[6] + v.y * a.m[7] + v.z * a.m[8]};
}
// matrix.go:88-101
template <class R> __device__ __forceinline__ m3<R> mulm(const m3<R>& a, const m3<R>& b) {
  m3<R> r;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
#pragma unroll
    for (int w = 0; w < 3; ++w)
      r.m[c * 3 + w] = a.m[w] * b.m[c * 3 + 0] + a.m[3 + w] * b.m[c * 3 + 1] + a.m[6 + w] * b.m[c * 3 + 2];
  }
  return r;
}
// matrix.go:103-114
template <class R> __device__ __forceinline__ void mulm_with(m3<R>& a, R s) {
#pragma unroll
  for (int i = 0; i < 9; ++i) a.m[i] *= s;
}
// matrix.go:116-123
template <class R> __device__ __forceinline__ m3<R> transpose(const m3<R>& a) {
  m3<R> r;
  r.m[0] = a.m[0]; r.m[1] = a.m[3]; r.m[2] = a.m[6];
  r.m[3] = a.m[1]; r.m[4] = a.m[4]; r.m[5] = a.m[7];
  r.m[6] = a.m[2]; r.m[7] = a.m[5]; r.m[8] = a.m[8];
  return r;
}
// matrix.go:125-153 (zero matrix when RealEqual(det, 0))
template <class R> __device__ __forceinline__ m3<R> invert(const m3<R>& a) {
  const R* m = a.m;
  R det = m[0] * m[4] * m[8] + m[3] * m[7] * m[2] + m[6] * m[1] * m[5] - m[6] * m[4] * m[2] - m[3] * m[1] * m[8] -
          m[0] * m[7] * m[5];
  m3<R> r;
  if (real_equal<R>(det, (R)0)) {
#pragma unroll
    for (int i = 0; i < 9; ++i) r.m[i] = (R)0;
    return r;
  }
  r.m[0] = m[4] * m[8] - m[5] * m[7];
  r.m[1] = m[2] * m[7] - m[1] * m[8];
  r.m[2] = m[1] * m[5] - m[2] * m[4];
  r.m[3] = m[5] * m[6] - m[3] * m[8];
  r.m[4] = m[0] * m[8] - m[2] * m[6];
  r.m[5] = m[2] * m[3] - m[0] * m[5];
  r.m[6] = m[3] * m[7] - m[4] * m[6];
  r.m[7] = m[1] * m[6] - m[0] * m[7];
  r.m[8] = m[0] * m[4] - m[1] * m[3];
  mulm_with<R>(r, (R)1 / det);
  return r;
}

// Collider transform: 3x4 column-major, cols 0..2 rotation axes, col 3 position.
template <class R> struct xf {
  R m[12];
  __device__ __forceinline__ v3<R> axis(int c) const { return v3<R>{m[c * 3], m[c * 3 + 1], m[c * 3 + 2]}; }
};

// matrix.go:165-185 SetAsTransform followed by MulMatrix3x4 (matrix.go:
// 198-217) with the collider's Offset o (column-major 3x4; colliders.go:
// 173-176, 302-304).  The products are all evaluated, as the reference does,
// so with the identity Offset signed zeros and non-finite values propagate
// alike.
template <class R>
__device__ __forceinline__ xf<R> collider_transform(const v3<R>& p, const q4<R>& q, const R (&o)[12]) {
  R w = q.w, x = q.x, y = q.y, z = q.z;
  R b[12];
  b[0] = (R)1 - (R)2 * y * y - (R)2 * z * z;
  b[1] = (R)2 * x * y + (R)2 * w * z;
  b[2] = (R)2 * x * z - (R)2 * w * y;
  b[3] = (R)2 * x * y - (R)2 * w * z;
  b[4] = (R)1 - (R)2 * x * x - (R)2 * z * z;
  b[5] = (R)2 * y * z + (R)2 * w * x;
  b[6] = (R)2 * x * z + (R)2 * w * y;
  b[7] = (R)2 * y * z - (R)2 * w * x;
  b[8] = (R)1 - (R)2 * x * x - (R)2 * y * y;
  b[9] = p.x;
  b[10] = p.y;
  b[11] = p.z;
  xf<R> t;
#pragma unroll
  for (int w2 = 0; w2 < 3; ++w2) {
    t.m[w2] = b[w2] * o[0] + b[3 + w2] * o[1] + b[6 + w2] * o[2];
    t.m[3 + w2] = b[w2] * o[3] + b[3 + w2] * o[4] + b[6 + w2] * o[5];
    t.m[6 + w2] = b[w2] * o[6] + b[3 + w2] * o[7] + b[6 + w2] * o[8];
    t.m[9 + w2] = b[w2] * o[9] + b[3 + w2] * o[10] + b[6 + w2] * o[11] + b[9 + w2];
  }
  return t;
}
// the identity Offset set by NewCollisionCube / NewCollisionSphere
// (colliders.go:138, 267)
template <class R> __device__ __forceinline__ xf<R> collider_transform(const v3<R>& p, const q4<R>& q) {
  const R id[12] = {(R)1, (R)0, (R)0, (R)0, (R)1, (R)0, (R)0, (R)0, (R)1, (R)0, (R)0, (R)0};
  return collider_transform(p, q, id);
}

// matrix.go:187-194
template <class R> __device__ __forceinline__ v3<R> xf_mul(const xf<R>& t, const v3<R>& v) {
  return v3<R>{v.x * t.m[0] + v.y * t.m[3] + v.z * t.m[6] + t.m[9], v.x * t.m[1] + v.y * t.m[4] + v.z * t.m[7] + t.m[10],
               v.x * t.m[2] + v.y * t.m[5] + v.z * t.m[8] + t.m[11]};
}
// matrix.go:219-233
template <class R> __device__ __forceinline__ v3<R> xf_inv(const xf<R>& t, const v3<R>& v) {
  R a = v.x - t.m[9], b = v.y - t.m[10], c = v.z - t.m[11];
  return v3<R>{a * t.m[0] + b * t.m[1] + c * t.m[2], a * t.m[3] + b * t.m[4] + c * t.m[5],
               a * t.m[6] + b * t.m[7] + c * t.m[8]};
}

// rigidbody.go:274-299 (iitWorld = R * iitBody * R^T in the reference's order);
// r is the body transform's rotation part (column-major).
template <class R> __device__ __forceinline__ m3<R> world_inertia(const R* r, const m3<R>& b) {
  const R* i = b.m;
  R t4 = r[0] * i[0] + r[3] * i[1] + r[6] * i[2];
  R t9 = r[0] * i[3] + r[3] * i[4] + r[6] * i[5];
  R t14 = r[0] * i[6] + r[3] * i[7] + r[6] * i[8];
  R t28 = r[1] * i[0] + r[4] * i[1] + r[7] * i[2];
  R t33 = r[1] * i[3] + r[4] * i[4] + r[7] * i[5];
  R t38 = r[1] * i[6] + r[4] * i[7] + r[7] * i[8];
  R t52 = r[2] * i[0] + r[5] * i[1] + r[8] * i[2];
  R t57 = r[2] * i[3] + r[5] * i[4] + r[8] * i[5];
  R t62 = r[2] * i[6] + r[5] * i[7] + r[8] * i[8];
  m3<R> w;
  w.m[0] = t4 * r[0] + t9 * r[3] + t14 * r[6];
  w.m[3] = t4 * r[1] + t9 * r[4] + t14 * r[7];
  w.m[6] = t4 * r[2] + t9 * r[5] + t14 * r[8];
  w.m[1] = t28 * r[0] + t33 * r[3] + t38 * r[6];
  w.m[4] = t28 * r[1] + t33 * r[4] + t38 * r[7];
  w.m[7] = t28 * r[2] + t33 * r[5] + t38 * r[8];
  w.m[2] = t52 * r[0] + t57 * r[3] + t62 * r[6];
  w.m[5] = t52 * r[1] + t57 * r[4] + t62 * r[7];
  w.m[8] = t52 * r[2] + t57 * r[5] + t62 * r[8];
  return w;
}

// SetAsTransform rotation part only (matrix.go:165-177)
template <class R> __device__ __forceinline__ void rotation_of(const q4<R>& q, R* b) {
  R w = q.w, x = q.x, y = q.y, z = q.z;
  b[0] = (R)1 - (R)2 * y * y - (R)2 * z * z;
  b[1] = (R)2 * x * y + (R)2 * w * z;
  b[2] = (R)2 * x * z - (R)2 * w * y;
  b[3] = (R)2 * x * y - (R)2 * w * z;
  b[4] = (R)1 - (R)2 * x * x - (R)2 * z * z;
  b[5] = (R)2 * y * z + (R)2 * w * x;
  b[6] = (R)2 * x * z + (R)2 * w * y;
  b[7] = (R)2 * y * z - (R)2 * w * x;
  b[8] = (R)1 - (R)2 * x * x - (R)2 * y * y;
}

}  // namespace cz
