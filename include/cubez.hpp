/* cubez.hpp — the cubez rigid-body API (rigidbody.go, colliders.go,
 * contact.go of tbogdala/cubez) for C++ callers, over the C ABI of
 * cubez_gpu.h.
 *
 * Same type and member names, argument meanings and call order as the Go
 * package, so a port of a cubez program (the frame loop of
 * examples/cubedrop.go:29-75) reads like the original:
 *
 *   cubez::RigidBody body;                    // NewRigidBody()
 *   cubez::CollisionCube cube(&body, half);   // NewCollisionCube(body, half)
 *   body.Integrate(dt);
 *   cube.CheckAgainstHalfSpace(ground, contacts);
 *   cubez::CheckForCollisions(cube, other, contacts);
 *   cubez::ResolveContacts(int(contacts.size()) * 4, contacts, dt);
 *
 * Every step of the path runs on the GPU, in the plain float64 form, which is
 * bit-identical to the reference's arithmetic: Integrate and
 * CalculateDerivedData through cz_integrate / cz_upload_bodies,
 * CheckAgainst* / CheckForCollisions through cz_collide, ResolveContacts
 * through cz_resolve_contacts.  Each call is one small GPU round trip; a
 * program that steps many bodies or worlds per frame batches them with
 * cz_step instead (the numbers are the same).
 *
 * Differences from Go, all forced by C++:
 *  - []*Contact becomes std::vector<Contact> (values; contacts point at
 *    bodies, not the other way round), and (bool, []*Contact) returns become
 *    a bool plus the vector appended in place;
 *  - where the reference panics (a nil body dereference in the frictionless
 *    impulse, a box-box test reaching no axis), a cubez::Error carrying the
 *    cz_status is thrown;
 *  - a collider's transform (body transform x Offset) is derived where it is
 *    used, so CalculateDerivedData on a collider has nothing to store;
 *  - the constructor functions (NewRigidBody, NewCollisionPlane/Sphere/Cube)
 *    return std::unique_ptr where Go returns a pointer, and NewContact a
 *    value.
 *
 * Host-side setup helpers (SetBlockInertiaTensor, Invert, SetAsTransform)
 * compute what the Go setup code computes once per body; they are not on the
 * per-frame path.
 */
#pragma once
#include <array>
#include <cmath>
#include <cstdint>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "cubez_gpu.h"

namespace cubez {

using Real = double;                    // m.Real (math/math.go)
using Vector3 = std::array<Real, 3>;    // m.Vector3
using Quat = std::array<Real, 4>;       // m.Quat: w, x, y, z
using Matrix3 = std::array<Real, 9>;    // m.Matrix3, column-major
using Matrix3x4 = std::array<Real, 12>; // m.Matrix3x4, column-major, column 3 = translation

constexpr Real kMaxValue = std::numeric_limits<Real>::max();  // m.MaxValue
constexpr Real kEpsilon = 1e-7;                               // m.Epsilon

class Error : public std::runtime_error {
 public:
  Error(int code, const std::string& what) : std::runtime_error(what), status(code) {}
  int status;
};

namespace detail {
inline void check(int st, const char* call) {
  if (st != CZ_OK) throw Error(st, std::string(call) + ": " + cz_status_string(st) + ": " + cz_last_error());
}
// RealEqual, math/math.go:64-78
inline bool RealEqual(Real a, Real b) {
  if (a == b) return true;
  const Real diff = std::fabs(a - b);
  if (a * b == 0 || diff < std::numeric_limits<Real>::min()) return diff < kEpsilon * kEpsilon;
  return diff / (std::fabs(a) + std::fabs(b)) < kEpsilon;
}
}  // namespace detail

// ---------------------------------------------------------------- setup math
inline Matrix3 Identity3() { return Matrix3{1, 0, 0, 0, 1, 0, 0, 0, 1}; }
inline Matrix3x4 Identity3x4() { return Matrix3x4{1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0}; }

// Matrix3.SetInertiaTensorCoeffs, math/matrix.go:59-66
inline Matrix3 InertiaTensorCoeffs(Real ix, Real iy, Real iz, Real ixy = 0, Real ixz = 0, Real iyz = 0) {
  return Matrix3{ix, -ixy, -ixz, -ixy, iy, -iyz, -ixz, -iyz, iz};
}
// Matrix3.SetBlockInertiaTensor, math/matrix.go:68-77 (the reference's 0.3 factor)
inline Matrix3 BlockInertiaTensor(const Vector3& halfSize, Real mass) {
  const Real x2 = halfSize[0] * halfSize[0], y2 = halfSize[1] * halfSize[1], z2 = halfSize[2] * halfSize[2];
  return InertiaTensorCoeffs(0.3 * mass * (y2 + z2), 0.3 * mass * (x2 + z2), 0.3 * mass * (x2 + y2));
}
// Matrix3.Invert, math/matrix.go:125-153 (zero matrix when RealEqual(det, 0))
inline Matrix3 Invert(const Matrix3& m) {
  const Real det = m[0] * m[4] * m[8] + m[3] * m[7] * m[2] + m[6] * m[1] * m[5] - m[6] * m[4] * m[2] -
                   m[3] * m[1] * m[8] - m[0] * m[7] * m[5];
  if (detail::RealEqual(det, 0)) return Matrix3{};
  Matrix3 r{m[4] * m[8] - m[5] * m[7], m[2] * m[7] - m[1] * m[8], m[1] * m[5] - m[2] * m[4],
            m[5] * m[6] - m[3] * m[8], m[0] * m[8] - m[2] * m[6], m[2] * m[3] - m[0] * m[5],
            m[3] * m[7] - m[4] * m[6], m[1] * m[6] - m[0] * m[7], m[0] * m[4] - m[1] * m[3]};
  const Real s = 1 / det;
  for (Real& x : r) x *= s;
  return r;
}
// Matrix3x4.SetAsTransform, math/matrix.go:165-185
inline Matrix3x4 AsTransform(const Vector3& p, const Quat& q) {
  const Real w = q[0], x = q[1], y = q[2], z = q[3];
  return Matrix3x4{1 - 2 * y * y - 2 * z * z, 2 * x * y + 2 * w * z,     2 * x * z - 2 * w * y,
                   2 * x * y - 2 * w * z,     1 - 2 * x * x - 2 * z * z, 2 * y * z + 2 * w * x,
                   2 * x * z + 2 * w * y,     2 * y * z - 2 * w * x,     1 - 2 * x * x - 2 * y * y,
                   p[0],                      p[1],                      p[2]};
}

// Matrix3x4.MulMatrix3x4, math/matrix.go:196-217
inline Matrix3x4 MulMatrix3x4(const Matrix3x4& m, const Matrix3x4& o) {
  Matrix3x4 r;
  for (int c = 0; c < 3; ++c)
    for (int i = 0; i < 3; ++i) r[3 * c + i] = m[i] * o[3 * c] + m[3 + i] * o[3 * c + 1] + m[6 + i] * o[3 * c + 2];
  for (int i = 0; i < 3; ++i) r[9 + i] = m[i] * o[9] + m[3 + i] * o[10] + m[6 + i] * o[11] + m[9 + i];
  return r;
}

class RigidBody;
class CollisionPlane;
class CollisionSphere;
class CollisionCube;

// ---------------------------------------------------------------- GPU runtime
namespace gpu {
// Batches of one world, cached by body count: the per-object calls of this
// API upload their bodies into one, run one C-ABI call and read the result
// back.  One runtime per process, serialised by a mutex.
class Runtime {
 public:
  static Runtime& get() {
    static Runtime r;
    return r;
  }
  ~Runtime() {
    for (auto& kv : batches_) cz_batch_destroy(kv.second);
  }
  std::mutex& mutex() { return mu_; }
  // a single-world float64 batch of n bodies holding at least `contacts` contacts
  cz_batch* batch(int n, int contacts) {
    const int worst = 8 * n + n * (n - 1);
    auto it = batches_.find(n);
    if (it != batches_.end() && caps_[n] >= contacts) return it->second;
    if (it != batches_.end()) {
      cz_batch_destroy(it->second);
      batches_.erase(it);
    }
    const int cap = std::max(std::min(worst, std::max(contacts, 64 * n)), std::max(contacts, 1));
    int32_t counts[1] = {n};
    cz_batch_desc d{};
    d.form = CZ_FORM_FP64;
    d.num_worlds = 1;
    d.body_counts = counts;
    d.contact_capacity = cap;
    d.plane[1] = 1;
    d.iteration_multiplier = 4;
    cz_batch* b = nullptr;
    detail::check(cz_batch_create(&d, &b), "cz_batch_create");
    batches_[n] = b;
    caps_[n] = std::min(cap, worst);
    return b;
  }

 private:
  Runtime() = default;
  std::mutex mu_;
  std::map<int, cz_batch*> batches_;
  std::map<int, int> caps_;
};

// Structure-of-arrays staging of a list of bodies for cz_bodies.
struct Staging {
  std::vector<double> position, orientation, velocity, rotation, acceleration, inverse_inertia, inverse_mass,
      linear_damping, angular_damping, motion, half_size, radius, iit_world, lfa, offset;
  bool has_offset = false;  // some collider's Offset is not the identity
  std::vector<uint8_t> is_awake, can_sleep;
  std::vector<int32_t> shape;
  cz_bodies view() {
    cz_bodies b{};
    b.position = position.data();
    b.orientation = orientation.data();
    b.velocity = velocity.data();
    b.rotation = rotation.data();
    b.acceleration = acceleration.data();
    b.inverse_inertia = inverse_inertia.data();
    b.inverse_mass = inverse_mass.data();
    b.linear_damping = linear_damping.data();
    b.angular_damping = angular_damping.data();
    b.motion = motion.data();
    b.is_awake = is_awake.data();
    b.can_sleep = can_sleep.data();
    b.shape = shape.data();
    b.half_size = half_size.data();
    b.radius = radius.data();
    b.inverse_inertia_world = iit_world.data();
    b.last_frame_acceleration = lfa.data();
    b.collider_offset = has_offset ? offset.data() : nullptr;
    return b;
  }
};
}  // namespace gpu

// ---------------------------------------------------------------- RigidBody
// rigidbody.go:23-101
class RigidBody {
 public:
  Real LinearDamping = 0.95;   // defaultLinearDamping (NewRigidBody sets both dampings to it)
  Real AngularDamping = 0.95;
  Vector3 Position{};
  Quat Orientation{1, 0, 0, 0};
  Vector3 Velocity{};
  Vector3 Acceleration{0, -9.78, 0};  // defaultAcceleration
  Vector3 Rotation{};
  Matrix3 InverseInertiaTensor{};
  bool IsAwake = true;
  bool CanSleep = true;

  // NewRigidBody, rigidbody.go:104-114
  RigidBody() { SetAwake(true); }
  RigidBody Clone() const { return *this; }

  // rigidbody.go:124-178
  void SetMass(Real mass) {
    mass_ = mass;
    inverseMass_ = 1.0 / mass;
  }
  void SetInfiniteMass() {
    mass_ = 0;
    inverseMass_ = 0;
  }
  bool HasFiniteMass() const { return inverseMass_ > 0.0; }
  Real GetMass() const { return inverseMass_ == 0.0 ? kMaxValue : mass_; }
  Real GetInverseMass() const { return inverseMass_; }
  Matrix3x4 GetTransform() const { return transform_; }
  Vector3 GetLastFrameAccelleration() const { return lastFrameAccelleration_; }
  Matrix3 GetInverseInertiaTensorWorld() const { return iitWorld_; }
  void SetInertiaTensor(const Matrix3& m) { InverseInertiaTensor = Invert(m); }
  // rigidbody.go:182-192 (does not respect CanSleep)
  void SetAwake(bool awake) {
    if (awake) {
      IsAwake = true;
      motion_ = 0.3 * 2.0;
    } else {
      IsAwake = false;
      Velocity = Vector3{};
      Rotation = Vector3{};
    }
  }
  void AddVelocity(const Vector3& v) {
    for (int i = 0; i < 3; ++i) Velocity[i] += v[i];
  }
  void AddRotation(const Vector3& v) {
    for (int i = 0; i < 3; ++i) Rotation[i] += v[i];
  }
  // the reference keeps force and torque accumulators that nothing on the
  // path adds to; they stay zero here
  void ClearAccumulators() {}

  // rigidbody.go:213-259, on the GPU
  void Integrate(Real duration);
  // rigidbody.go:268-272, on the GPU
  void CalculateDerivedData();

 private:
  friend struct Marshal;
  Real mass_ = 0, inverseMass_ = 0;
  Matrix3 iitWorld_ = Identity3();
  Matrix3x4 transform_ = Identity3x4();
  Vector3 lastFrameAccelleration_{};
  Real motion_ = 0;
};

// ---------------------------------------------------------------- Contact
// contact.go:17-51 (the private working fields live on the device)
struct Contact {
  std::array<RigidBody*, 2> Bodies{{nullptr, nullptr}};
  Real Friction = 0;
  Real Restitution = 0;
  Vector3 ContactPoint{};
  Vector3 ContactNormal{};
  Real Penetration = 0;
};

// ---------------------------------------------------------------- colliders
// colliders.go:15-23
class Collider {
 public:
  virtual ~Collider() = default;
  virtual RigidBody* GetBody() const = 0;
  virtual Matrix3x4 GetTransform() const = 0;
  // the collider transform is the body transform times the Offset
  // (colliders.go:173-176, 302-304); the GPU derives it where it needs it
  virtual void CalculateDerivedData() {}
  virtual bool CheckAgainstHalfSpace(const CollisionPlane& plane, std::vector<Contact>& contacts) = 0;
  virtual bool CheckAgainstSphere(CollisionSphere& sphere, std::vector<Contact>& contacts) = 0;
  virtual bool CheckAgainstCube(CollisionCube& cube, std::vector<Contact>& contacts) = 0;
};

// colliders.go:29-35, 81-125
class CollisionPlane : public Collider {
 public:
  Vector3 Normal;
  Real Offset;
  CollisionPlane(const Vector3& n, Real o) : Normal(n), Offset(o) {}
  RigidBody* GetBody() const override { return nullptr; }
  Matrix3x4 GetTransform() const override { return Identity3x4(); }
  bool CheckAgainstHalfSpace(const CollisionPlane&, std::vector<Contact>&) override { return false; }
  bool CheckAgainstSphere(CollisionSphere& sphere, std::vector<Contact>& contacts) override;
  bool CheckAgainstCube(CollisionCube& cube, std::vector<Contact>& contacts) override;
};

// colliders.go:57-71, 136-254
class CollisionSphere : public Collider {
 public:
  RigidBody* Body;
  Matrix3x4 Offset = Identity3x4();
  Real Radius;
  // NewCollisionSphere: a null body gets a new RigidBody owned by the collider
  CollisionSphere(RigidBody* optBody, Real radius) : Body(optBody), Radius(radius) {
    if (!Body) {
      own_ = std::make_unique<RigidBody>();
      Body = own_.get();
    }
  }
  RigidBody* GetBody() const override { return Body; }
  Matrix3x4 GetTransform() const override;
  bool CheckAgainstHalfSpace(const CollisionPlane& plane, std::vector<Contact>& contacts) override;
  bool CheckAgainstSphere(CollisionSphere& sphere, std::vector<Contact>& contacts) override;
  bool CheckAgainstCube(CollisionCube& cube, std::vector<Contact>& contacts) override;

 private:
  std::unique_ptr<RigidBody> own_;
};

// colliders.go:39-52, 265-710
class CollisionCube : public Collider {
 public:
  RigidBody* Body;
  Matrix3x4 Offset = Identity3x4();
  Vector3 HalfSize;
  CollisionCube(RigidBody* optBody, const Vector3& halfSize) : Body(optBody), HalfSize(halfSize) {
    if (!Body) {
      own_ = std::make_unique<RigidBody>();
      Body = own_.get();
    }
  }
  RigidBody* GetBody() const override { return Body; }
  Matrix3x4 GetTransform() const override;
  bool CheckAgainstHalfSpace(const CollisionPlane& plane, std::vector<Contact>& contacts) override;
  bool CheckAgainstSphere(CollisionSphere& sphere, std::vector<Contact>& contacts) override;
  bool CheckAgainstCube(CollisionCube& cube, std::vector<Contact>& contacts) override;

 private:
  std::unique_ptr<RigidBody> own_;
};

// ---------------------------------------------------------------- marshalling
struct Marshal {
  // one body (with its collider's shape) into slot k of the staging arrays
  static void put(gpu::Staging& s, int k, const RigidBody& b, int shape, const Vector3& half, Real radius,
                  const Matrix3x4& offset = Identity3x4()) {
    auto set = [&](std::vector<double>& v, int w, const Real* src) {
      for (int i = 0; i < w; ++i) v[(size_t)k * w + i] = src[i];
    };
    set(s.position, 3, b.Position.data());
    set(s.orientation, 4, b.Orientation.data());
    set(s.velocity, 3, b.Velocity.data());
    set(s.rotation, 3, b.Rotation.data());
    set(s.acceleration, 3, b.Acceleration.data());
    set(s.inverse_inertia, 9, b.InverseInertiaTensor.data());
    set(s.iit_world, 9, b.iitWorld_.data());
    set(s.lfa, 3, b.lastFrameAccelleration_.data());
    set(s.half_size, 3, half.data());
    set(s.offset, 12, offset.data());
    if (offset != Identity3x4()) s.has_offset = true;
    s.inverse_mass[k] = b.inverseMass_;
    s.linear_damping[k] = b.LinearDamping;
    s.angular_damping[k] = b.AngularDamping;
    s.motion[k] = b.motion_;
    s.radius[k] = radius;
    s.is_awake[k] = b.IsAwake ? 1 : 0;
    s.can_sleep[k] = b.CanSleep ? 1 : 0;
    s.shape[k] = shape;
  }
  // the device's results for slot k back into the body; `derived`: the call
  // ran CalculateDerivedData on it, so its transform is refreshed (the
  // reference leaves an awake body's transform stale through ResolveContacts)
  static void get(const gpu::Staging& s, int k, RigidBody& b, bool derived) {
    auto cp = [&](const std::vector<double>& v, int w, Real* dst) {
      for (int i = 0; i < w; ++i) dst[i] = v[(size_t)k * w + i];
    };
    cp(s.position, 3, b.Position.data());
    cp(s.orientation, 4, b.Orientation.data());
    cp(s.velocity, 3, b.Velocity.data());
    cp(s.rotation, 3, b.Rotation.data());
    cp(s.iit_world, 9, b.iitWorld_.data());
    cp(s.lfa, 3, b.lastFrameAccelleration_.data());
    b.motion_ = s.motion[k];
    b.IsAwake = s.is_awake[k] != 0;
    if (derived) b.transform_ = AsTransform(b.Position, b.Orientation);
  }
  static gpu::Staging staging(int n) {
    gpu::Staging s;
    for (auto* v : {&s.position, &s.velocity, &s.rotation, &s.acceleration, &s.half_size, &s.lfa}) v->assign(3 * n, 0);
    s.orientation.assign(4 * n, 0);
    s.inverse_inertia.assign(9 * n, 0);
    s.iit_world.assign(9 * n, 0);
    s.offset.clear();
    for (int k = 0; k < n; ++k) {
      const Matrix3x4 id = Identity3x4();
      s.offset.insert(s.offset.end(), id.begin(), id.end());
    }
    for (auto* v : {&s.inverse_mass, &s.linear_damping, &s.angular_damping, &s.motion, &s.radius}) v->assign(n, 0);
    s.is_awake.assign(n, 0);
    s.can_sleep.assign(n, 0);
    s.shape.assign(n, CZ_SHAPE_SPHERE);
    return s;
  }
};

namespace detail {
struct Shape {
  RigidBody* body;
  int shape;
  Vector3 half;
  Real radius;
  Matrix3x4 offset;
};
inline Shape shape_of(const CollisionSphere& s) { return Shape{s.Body, CZ_SHAPE_SPHERE, Vector3{}, s.Radius, s.Offset}; }
inline Shape shape_of(const CollisionCube& c) { return Shape{c.Body, CZ_SHAPE_CUBE, c.HalfSize, 0, c.Offset}; }

// Run one narrowphase test on the GPU and append its contacts: (a, b) is
// CheckForCollisions(a, b); b == nullptr is a's CheckAgainstHalfSpace(plane).
inline bool collide(const Shape& a, const Shape* b, const CollisionPlane* plane, std::vector<Contact>& contacts) {
  gpu::Runtime& rt = gpu::Runtime::get();
  std::lock_guard<std::mutex> lock(rt.mutex());
  const int n = b ? 2 : 1;
  cz_batch* batch = rt.batch(n, 8);
  gpu::Staging s = Marshal::staging(n);
  Marshal::put(s, 0, *a.body, a.shape, a.half, a.radius, a.offset);
  if (b) Marshal::put(s, 1, *b->body, b->shape, b->half, b->radius, b->offset);
  cz_bodies v = s.view();
  check(cz_upload_bodies(batch, &v), "cz_upload_bodies");
  const int32_t unit[2] = {0, b ? 1 : -1};
  double pl[4] = {0, 1, 0, 0};
  if (plane) pl[0] = plane->Normal[0], pl[1] = plane->Normal[1], pl[2] = plane->Normal[2], pl[3] = plane->Offset;
  check(cz_collide(batch, 0, pl, unit, 1), "cz_collide");
  cz_contact out[8];
  int32_t count = 0;
  check(cz_download_contacts(batch, 0, out, 8, &count), "cz_download_contacts");
  RigidBody* bodies[2] = {a.body, b ? b->body : nullptr};
  for (int k = 0; k < count; ++k) {
    Contact c;
    c.Bodies[0] = out[k].body[0] >= 0 ? bodies[out[k].body[0]] : nullptr;
    c.Bodies[1] = out[k].body[1] >= 0 ? bodies[out[k].body[1]] : nullptr;
    c.Friction = out[k].friction;
    c.Restitution = out[k].restitution;
    for (int i = 0; i < 3; ++i) {
      c.ContactPoint[i] = out[k].point[i];
      c.ContactNormal[i] = out[k].normal[i];
    }
    c.Penetration = out[k].penetration;
    contacts.push_back(c);
  }
  return count > 0;
}

// Integrate (integrate = true) or CalculateDerivedData of one body.
inline void body_step(RigidBody& body, Real dt, bool integrate) {
  gpu::Runtime& rt = gpu::Runtime::get();
  std::lock_guard<std::mutex> lock(rt.mutex());
  cz_batch* batch = rt.batch(1, 1);
  gpu::Staging s = Marshal::staging(1);
  Marshal::put(s, 0, body, CZ_SHAPE_SPHERE, Vector3{}, 0);
  cz_bodies v = s.view();
  if (!integrate) v.inverse_inertia_world = nullptr;  // the upload derives it (CalculateDerivedData)
  check(cz_upload_bodies(batch, &v), "cz_upload_bodies");
  if (integrate) check(cz_integrate(batch, dt), "cz_integrate");
  v = s.view();
  check(cz_download_bodies(batch, &v), "cz_download_bodies");
  Marshal::get(s, 0, body, true);
}
}  // namespace detail

inline void RigidBody::Integrate(Real duration) {
  if (!IsAwake) return;  // rigidbody.go:214-216
  detail::body_step(*this, duration, true);
}
inline void RigidBody::CalculateDerivedData() { detail::body_step(*this, 0, false); }

inline bool CollisionPlane::CheckAgainstSphere(CollisionSphere& sphere, std::vector<Contact>& contacts) {
  return sphere.CheckAgainstHalfSpace(*this, contacts);  // colliders.go:116-119
}
inline bool CollisionPlane::CheckAgainstCube(CollisionCube& cube, std::vector<Contact>& contacts) {
  return cube.CheckAgainstHalfSpace(*this, contacts);  // colliders.go:122-125
}
inline Matrix3x4 CollisionSphere::GetTransform() const { return MulMatrix3x4(Body->GetTransform(), Offset); }
inline Matrix3x4 CollisionCube::GetTransform() const { return MulMatrix3x4(Body->GetTransform(), Offset); }
inline bool CollisionSphere::CheckAgainstHalfSpace(const CollisionPlane& plane, std::vector<Contact>& contacts) {
  return detail::collide(detail::shape_of(*this), nullptr, &plane, contacts);
}
inline bool CollisionSphere::CheckAgainstSphere(CollisionSphere& sphere, std::vector<Contact>& contacts) {
  const detail::Shape other = detail::shape_of(sphere);
  return detail::collide(detail::shape_of(*this), &other, nullptr, contacts);
}
inline bool CollisionSphere::CheckAgainstCube(CollisionCube& cube, std::vector<Contact>& contacts) {
  const detail::Shape other = detail::shape_of(cube);
  return detail::collide(detail::shape_of(*this), &other, nullptr, contacts);
}
inline bool CollisionCube::CheckAgainstHalfSpace(const CollisionPlane& plane, std::vector<Contact>& contacts) {
  return detail::collide(detail::shape_of(*this), nullptr, &plane, contacts);
}
inline bool CollisionCube::CheckAgainstSphere(CollisionSphere& sphere, std::vector<Contact>& contacts) {
  const detail::Shape other = detail::shape_of(sphere);
  return detail::collide(detail::shape_of(*this), &other, nullptr, contacts);
}
inline bool CollisionCube::CheckAgainstCube(CollisionCube& cube, std::vector<Contact>& contacts) {
  const detail::Shape other = detail::shape_of(cube);
  return detail::collide(detail::shape_of(*this), &other, nullptr, contacts);
}

// The Go package's constructor functions, returning owned objects where Go
// returns pointers (rigidbody.go:104-114, colliders.go:81-86, 136-141,
// 265-270, contact.go:54-57).  A collider given no body owns a new one.
inline std::unique_ptr<RigidBody> NewRigidBody() { return std::make_unique<RigidBody>(); }
inline std::unique_ptr<CollisionPlane> NewCollisionPlane(const Vector3& n, Real o) {
  return std::make_unique<CollisionPlane>(n, o);
}
inline std::unique_ptr<CollisionSphere> NewCollisionSphere(RigidBody* optBody, Real radius) {
  return std::make_unique<CollisionSphere>(optBody, radius);
}
inline std::unique_ptr<CollisionCube> NewCollisionCube(RigidBody* optBody, const Vector3& halfSize) {
  return std::make_unique<CollisionCube>(optBody, halfSize);
}
inline Contact NewContact() { return Contact{}; }

// CheckForCollisions, colliders.go:720-747: dispatch on the second collider's type
inline bool CheckForCollisions(Collider& one, Collider& two, std::vector<Contact>& contacts) {
  if (auto* s = dynamic_cast<CollisionSphere*>(&two)) return one.CheckAgainstSphere(*s, contacts);
  if (auto* c = dynamic_cast<CollisionCube*>(&two)) return one.CheckAgainstCube(*c, contacts);
  if (auto* p = dynamic_cast<CollisionPlane*>(&two)) return one.CheckAgainstHalfSpace(*p, contacts);
  return false;
}

// ResolveContacts, contact.go:208-222, on the GPU: the bodies the contacts
// touch are uploaded, resolved and written back; the contacts are written
// back as the reference leaves them (penetration, swapped bodies and normal).
inline void ResolveContacts(int maxIterations, std::vector<Contact>& contacts, Real duration) {
  if (contacts.empty() || duration <= 0) return;  // contact.go:210-212
  std::vector<RigidBody*> bodies;
  std::map<RigidBody*, int> index;
  auto idx = [&](RigidBody* b) -> int {
    if (!b) return -1;
    auto it = index.find(b);
    if (it != index.end()) return it->second;
    const int k = (int)bodies.size();
    index[b] = k;
    bodies.push_back(b);
    return k;
  };
  std::vector<cz_contact> cs(contacts.size());
  for (size_t k = 0; k < contacts.size(); ++k) {
    const Contact& c = contacts[k];
    cz_contact& o = cs[k];
    o.body[0] = idx(c.Bodies[0]);
    o.body[1] = idx(c.Bodies[1]);
    o.friction = c.Friction;
    o.restitution = c.Restitution;
    for (int i = 0; i < 3; ++i) {
      o.point[i] = c.ContactPoint[i];
      o.normal[i] = c.ContactNormal[i];
    }
    o.penetration = c.Penetration;
  }
  if (bodies.empty()) return;
  gpu::Runtime& rt = gpu::Runtime::get();
  std::lock_guard<std::mutex> lock(rt.mutex());
  const int n = (int)bodies.size();
  cz_batch* batch = rt.batch(n, (int)cs.size());
  gpu::Staging s = Marshal::staging(n);
  for (int k = 0; k < n; ++k) Marshal::put(s, k, *bodies[k], CZ_SHAPE_SPHERE, Vector3{}, 0);
  cz_bodies v = s.view();
  detail::check(cz_resolve_contacts(batch, maxIterations, cs.data(), (int32_t)cs.size(), duration, &v),
                "cz_resolve_contacts");
  // an asleep body moved by applyPositionChange had its derived data refreshed
  for (int k = 0; k < n; ++k) Marshal::get(s, k, *bodies[k], !bodies[k]->IsAwake);
  for (size_t k = 0; k < contacts.size(); ++k) {
    Contact& c = contacts[k];
    const cz_contact& o = cs[k];
    c.Bodies[0] = o.body[0] >= 0 ? bodies[o.body[0]] : nullptr;
    c.Bodies[1] = o.body[1] >= 0 ? bodies[o.body[1]] : nullptr;
    for (int i = 0; i < 3; ++i) c.ContactNormal[i] = o.normal[i];
    c.Penetration = o.penetration;
  }
}

}  // namespace cubez
