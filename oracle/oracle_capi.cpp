// C entry points of the oracle (TEST INFRASTRUCTURE: loaded by the tests, the
// smoke check and the CPU-baseline leg of the benchmark through ctypes; never by
// the product path).  Built with -O2 -ffp-contract=off by oracle/build.py.
//
// A batch holds many independent worlds.  Bodies arrive as host arrays of
// doubles in world-major order; the precision form rounds them to float.
#include <atomic>
#include <cstdio>
#include <memory>
#include <thread>

#include "cubez_ref.hpp"

using namespace orc;

extern "C" {

struct orc_bodies {
  double* position;         // [n][3]
  double* orientation;      // [n][4] (w,x,y,z)
  double* velocity;         // [n][3]
  double* rotation;         // [n][3]
  double* acceleration;     // [n][3]
  double* inverse_inertia;  // [n][9] body space, column-major
  double* inverse_mass;     // [n]
  double* linear_damping;   // [n]
  double* angular_damping;  // [n]
  double* motion;           // [n]
  uint8_t* is_awake;        // [n]
  uint8_t* can_sleep;       // [n]
  int32_t* shape;           // [n] 0 sphere, 1 cube
  double* half_size;        // [n][3]
  double* radius;           // [n]
  double* collider_offset;  // [n][12] collider Offset (column-major 3x4), null = identity
  double* last_frame_acceleration;  // [n][3] lastFrameAccelleration at setup, null = zero (as NewRigidBody)
};
}

namespace {

struct BatchBase {
  virtual ~BatchBase() {}
  virtual uint32_t step(int nsteps, double dt, int iterMult, int nthreads) = 0;
  virtual void integrate(double dt) = 0;
  virtual uint32_t narrowphase() = 0;
  virtual uint32_t collide(int w, const int32_t* units, int nunits) = 0;
  virtual uint32_t resolve(double dt, int iterMult) = 0;
  virtual void get(orc_bodies* out) = 0;
  virtual int contactCount(int w) = 0;
  virtual int contacts(int w, int32_t* b2, double* p3, double* n3, double* pen, int cap) = 0;
  virtual void stats(int32_t* c, int32_t* pit, int32_t* vit) = 0;
  virtual void setContacts(int w, const int32_t* b2, const double* p3, const double* n3, const double* pen,
                           const double* fric, const double* rest, int n) = 0;
  virtual uint32_t resolveFixed(double dt, int maxIter) = 0;
  virtual int resolved(int w, int32_t* b2, double* n3, double* pen, int cap) = 0;
};

template <class R, class W> struct Batch : BatchBase {
  int nworlds;
  std::vector<int> start, count;
  std::vector<Body<R, W>> bodies;
  std::vector<double> linD, angD;  // damping coefficients as uploaded
  Plane<R> plane;
  std::vector<std::vector<Contact<R>>> work, generated;
  std::vector<StepStats<R, W>> st;

  Batch(int nw, const int32_t* counts, const orc_bodies* in, const double* plane4) : nworlds(nw) {
    int total = 0;
    for (int w = 0; w < nw; ++w) {
      start.push_back(total);
      count.push_back(counts[w]);
      total += counts[w];
    }
    bodies.resize(total);
    linD.resize(total);
    angD.resize(total);
    for (int i = 0; i < total; ++i) {
      Body<R, W>& b = bodies[i];
      std::memset(&b, 0, sizeof(b));
      for (int k = 0; k < 3; ++k) {
        b.position[k] = (R)in->position[3 * i + k];
        b.velocity[k] = (R)in->velocity[3 * i + k];
        b.rotation[k] = (R)in->rotation[3 * i + k];
        b.acceleration[k] = (R)in->acceleration[3 * i + k];
        b.halfSize[k] = (R)in->half_size[3 * i + k];
      }
      for (int k = 0; k < 4; ++k) b.orientation[k] = (R)in->orientation[4 * i + k];
      for (int k = 0; k < 9; ++k) b.inverseInertiaTensor[k] = (R)in->inverse_inertia[9 * i + k];
      b.inverseMass = (R)in->inverse_mass[i];
      linD[i] = in->linear_damping[i];
      angD[i] = in->angular_damping[i];
      b.linearDamping = (R)linD[i];
      b.angularDamping = (R)angD[i];
      b.motion = (R)in->motion[i];
      b.isAwake = in->is_awake[i] != 0;
      b.canSleep = in->can_sleep[i] != 0;
      b.shape = in->shape[i];
      b.radius = (R)in->radius[i];
      if (in->collider_offset) {
        for (int k = 0; k < 12; ++k) b.offset[k] = (R)in->collider_offset[12 * i + k];
      } else {
        SetIdentity(b.offset);
      }
      // Body.CalculateDerivedData + Collider.CalculateDerivedData at setup
      // (examples/cubedrop.go:171-172).
      CalculateDerivedData(b);
      ColliderDerivedData(b);
      if (in->last_frame_acceleration)
        for (int k = 0; k < 3; ++k) b.lastFrameAccel[k] = (R)in->last_frame_acceleration[3 * i + k];
    }
    for (int k = 0; k < 3; ++k) plane.normal[k] = (R)plane4[k];
    plane.offset = (R)plane4[3];
    work.resize(nw);
    generated.resize(nw);
    st.resize(nw);
  }

  void pows(double dt, std::vector<R>& lp, std::vector<R>& ap, R& bias) {
    lp.resize(bodies.size());
    ap.resize(bodies.size());
    for (size_t i = 0; i < bodies.size(); ++i) {
      lp[i] = (R)std::pow(linD[i], dt);
      ap[i] = (R)std::pow(angD[i], dt);
    }
    bias = (R)std::pow(0.5, dt);
  }

  uint32_t step(int nsteps, double dt, int iterMult, int nthreads) override {
    std::vector<R> lp, ap;
    R bias;
    pows(dt, lp, ap, bias);
    std::atomic<int> next(0);
    std::atomic<uint32_t> err(0);
    auto worker = [&]() {
      for (;;) {
        int w = next.fetch_add(1);
        if (w >= nworlds) break;
        uint32_t e = 0;
        for (int s = 0; s < nsteps; ++s) {
          const bool last = (s == nsteps - 1);
          st[w] = StepWorld<R, W>(&bodies[start[w]], count[w], plane, (R)dt, &lp[start[w]], &ap[start[w]], bias,
                                  iterMult, work[w], last ? &generated[w] : nullptr);
          e |= st[w].err;
        }
        err.fetch_or(e);
      }
    };
    if (nthreads <= 1) {
      worker();
    } else {
      std::vector<std::thread> th;
      for (int t = 0; t < nthreads; ++t) th.emplace_back(worker);
      for (auto& t : th) t.join();
    }
    return err.load();
  }

  void integrate(double dt) override {
    std::vector<R> lp, ap;
    R bias;
    pows(dt, lp, ap, bias);
    for (size_t i = 0; i < bodies.size(); ++i) {
      Integrate(bodies[i], (R)dt, lp[i], ap[i], bias);
      ColliderDerivedData(bodies[i]);
    }
  }

  uint32_t narrowphase() override {
    uint32_t err = 0;
    for (int w = 0; w < nworlds; ++w) {
      GenerateContacts(&bodies[start[w]], count[w], plane, work[w], err);
      generated[w] = work[w];
      st[w].contacts = (int)work[w].size();
    }
    return err;
  }

  // A caller's list of tests of world w in the caller's order: (i, -1) is
  // body i's CheckAgainstHalfSpace(plane), (i, j) CheckForCollisions(i, j)
  // (colliders.go:720-747); the world's contact list is replaced.
  uint32_t collide(int w, const int32_t* units, int nunits) override {
    uint32_t err = 0;
    Body<R, W>* b = &bodies[start[w]];
    work[w].clear();
    for (int u = 0; u < nunits; ++u) {
      const int i = units[2 * u], j = units[2 * u + 1];
      if (j < 0)
        CheckAgainstHalfSpace(b[i], i, plane, work[w]);
      else
        CheckForCollisions(b[i], i, b[j], j, work[w], err);
    }
    generated[w] = work[w];
    st[w].contacts = (int)work[w].size();
    return err;
  }

  uint32_t resolve(double dt, int iterMult) override {
    uint32_t err = 0;
    for (int w = 0; w < nworlds; ++w) {
      Resolver<R, W> rs;
      rs.bodies = &bodies[start[w]];
      rs.ResolveContacts((int)work[w].size() * iterMult, work[w], (R)dt, count[w]);
      st[w].posIterations = rs.posIterations;
      st[w].velIterations = rs.velIterations;
      err |= rs.err;
    }
    return err;
  }

  void get(orc_bodies* o) override {
    for (size_t i = 0; i < bodies.size(); ++i) {
      const Body<R, W>& b = bodies[i];
      for (int k = 0; k < 3; ++k) {
        if (o->position) o->position[3 * i + k] = (double)b.position[k];
        if (o->velocity) o->velocity[3 * i + k] = (double)b.velocity[k];
        if (o->rotation) o->rotation[3 * i + k] = (double)b.rotation[k];
        if (o->acceleration) o->acceleration[3 * i + k] = (double)b.acceleration[k];
        if (o->half_size) o->half_size[3 * i + k] = (double)b.halfSize[k];
      }
      for (int k = 0; k < 4; ++k)
        if (o->orientation) o->orientation[4 * i + k] = (double)b.orientation[k];
      for (int k = 0; k < 9; ++k)
        if (o->inverse_inertia) o->inverse_inertia[9 * i + k] = (double)b.iitWorld[k];
      if (o->inverse_mass) o->inverse_mass[i] = (double)b.inverseMass;
      if (o->motion) o->motion[i] = (double)b.motion;
      if (o->is_awake) o->is_awake[i] = b.isAwake ? 1 : 0;
      if (o->can_sleep) o->can_sleep[i] = b.canSleep ? 1 : 0;
      if (o->shape) o->shape[i] = b.shape;
      if (o->radius) o->radius[i] = (double)b.radius;
    }
  }

  void setContacts(int w, const int32_t* b2, const double* p3, const double* n3, const double* pen,
                   const double* fric, const double* rest, int n) override {
    work[w].clear();
    for (int i = 0; i < n; ++i) {
      Contact<R> c = NewContact<R>();
      c.body[0] = b2[2 * i];
      c.body[1] = b2[2 * i + 1];
      for (int k = 0; k < 3; ++k) {
        c.point[k] = (R)p3[3 * i + k];
        c.normal[k] = (R)n3[3 * i + k];
      }
      c.penetration = (R)pen[i];
      c.friction = (R)fric[i];
      c.restitution = (R)rest[i];
      work[w].push_back(c);
    }
    generated[w] = work[w];
  }

  // ResolveContacts(maxIter, contacts, dt) on the contact lists set above
  uint32_t resolveFixed(double dt, int maxIter) override {
    uint32_t err = 0;
    for (int w = 0; w < nworlds; ++w) {
      Resolver<R, W> rs;
      rs.bodies = &bodies[start[w]];
      rs.ResolveContacts(maxIter, work[w], (R)dt, count[w]);
      st[w].posIterations = rs.posIterations;
      st[w].velIterations = rs.velIterations;
      err |= rs.err;
    }
    return err;
  }

  int resolved(int w, int32_t* b2, double* n3, double* pen, int cap) override {
    const auto& cs = work[w];
    int n = (int)cs.size();
    for (int i = 0; i < n && i < cap; ++i) {
      b2[2 * i] = cs[i].body[0];
      b2[2 * i + 1] = cs[i].body[1];
      for (int k = 0; k < 3; ++k) n3[3 * i + k] = (double)cs[i].normal[k];
      pen[i] = (double)cs[i].penetration;
    }
    return n;
  }

  int contactCount(int w) override { return (int)generated[w].size(); }

  int contacts(int w, int32_t* b2, double* p3, double* n3, double* pen, int cap) override {
    const auto& cs = generated[w];
    int n = (int)cs.size();
    for (int i = 0; i < n && i < cap; ++i) {
      b2[2 * i] = cs[i].body[0];
      b2[2 * i + 1] = cs[i].body[1];
      for (int k = 0; k < 3; ++k) {
        p3[3 * i + k] = (double)cs[i].point[k];
        n3[3 * i + k] = (double)cs[i].normal[k];
      }
      pen[i] = (double)cs[i].penetration;
    }
    return n;
  }

  void stats(int32_t* c, int32_t* pit, int32_t* vit) override {
    for (int w = 0; w < nworlds; ++w) {
      if (c) c[w] = st[w].contacts;
      if (pit) pit[w] = st[w].posIterations;
      if (vit) vit[w] = st[w].velIterations;
    }
  }
};

}  // namespace

extern "C" {

// form: 0 = plain FP64, 1 = precision form (FP32 bulk, FP64 islands)
void* orc_create(int form, int nworlds, const int32_t* counts, const orc_bodies* in, const double* plane4) {
  if (form == 0) return new Batch<double, double>(nworlds, counts, in, plane4);
  return new Batch<float, double>(nworlds, counts, in, plane4);
}
void orc_destroy(void* h) { delete static_cast<BatchBase*>(h); }
int orc_step(void* h, int nsteps, double dt, int iterMult, int nthreads) {
  return (int)static_cast<BatchBase*>(h)->step(nsteps, dt, iterMult, nthreads);
}
void orc_integrate(void* h, double dt) { static_cast<BatchBase*>(h)->integrate(dt); }
int orc_narrowphase(void* h) { return (int)static_cast<BatchBase*>(h)->narrowphase(); }
int orc_collide(void* h, int w, const int32_t* units, int nunits) {
  return (int)static_cast<BatchBase*>(h)->collide(w, units, nunits);
}
int orc_resolve(void* h, double dt, int iterMult) { return (int)static_cast<BatchBase*>(h)->resolve(dt, iterMult); }
void orc_get_bodies(void* h, orc_bodies* out) { static_cast<BatchBase*>(h)->get(out); }
int orc_contact_count(void* h, int w) { return static_cast<BatchBase*>(h)->contactCount(w); }
int orc_get_contacts(void* h, int w, int32_t* b2, double* p3, double* n3, double* pen, int cap) {
  return static_cast<BatchBase*>(h)->contacts(w, b2, p3, n3, pen, cap);
}
void orc_get_stats(void* h, int32_t* c, int32_t* pit, int32_t* vit) { static_cast<BatchBase*>(h)->stats(c, pit, vit); }
void orc_set_contacts(void* h, int w, const int32_t* b2, const double* p3, const double* n3, const double* pen,
                      const double* fric, const double* rest, int n) {
  static_cast<BatchBase*>(h)->setContacts(w, b2, p3, n3, pen, fric, rest, n);
}
int orc_resolve_fixed(void* h, double dt, int maxIter) {
  return (int)static_cast<BatchBase*>(h)->resolveFixed(dt, maxIter);
}
int orc_get_resolved(void* h, int w, int32_t* b2, double* n3, double* pen, int cap) {
  return static_cast<BatchBase*>(h)->resolved(w, b2, n3, pen, cap);
}
int orc_hardware_threads() { return (int)std::thread::hardware_concurrency(); }

// ---- math layer entry points for the known-answer tests (math/*_test.go)
int orc_real_equal(double a, double b) { return RealEqual<double>(a, b) ? 1 : 0; }
double orc_quat_len(const double* q) {
  Q4<double> a; for (int i = 0; i < 4; ++i) a[i] = q[i];
  return Len(a);
}
void orc_quat_normalize(double* q) {
  Q4<double> a; for (int i = 0; i < 4; ++i) a[i] = q[i];
  Normalize(a);
  for (int i = 0; i < 4; ++i) q[i] = a[i];
}
void orc_quat_mul(double* q, const double* q2) {
  Q4<double> a, b;
  for (int i = 0; i < 4; ++i) { a[i] = q[i]; b[i] = q2[i]; }
  Mul(a, b);
  for (int i = 0; i < 4; ++i) q[i] = a[i];
}
// QuatFromAxis, quaternion.go:8-16
void orc_quat_from_axis(double angle, double x, double y, double z, double* q) {
  double s = std::sin(angle / 2.0), c = std::cos(angle / 2.0);
  Q4<double> r; r[0] = c; r[1] = x * s; r[2] = y * s; r[3] = z * s;
  Normalize(r);
  for (int i = 0; i < 4; ++i) q[i] = r[i];
}
void orc_quat_rotate(const double* q, const double* v, double* out) {
  Q4<double> a; for (int i = 0; i < 4; ++i) a[i] = q[i];
  V3<double> r = Rotate(a, mk3(v[0], v[1], v[2]));
  for (int i = 0; i < 3; ++i) out[i] = r[i];
}
void orc_quat_add_scaled_vector(double* q, const double* v, double scale) {
  Q4<double> a; for (int i = 0; i < 4; ++i) a[i] = q[i];
  AddScaledVector(a, mk3(v[0], v[1], v[2]), scale);
  for (int i = 0; i < 4; ++i) q[i] = a[i];
}
void orc_m3_mul(const double* a, const double* b, double* out) {
  M3<double> x, y; for (int i = 0; i < 9; ++i) { x[i] = a[i]; y[i] = b[i]; }
  M3<double> r = MulMatrix3(x, y);
  for (int i = 0; i < 9; ++i) out[i] = r[i];
}
void orc_m3_invert(const double* a, double* out) {
  M3<double> x; for (int i = 0; i < 9; ++i) x[i] = a[i];
  M3<double> r = Invert(x);
  for (int i = 0; i < 9; ++i) out[i] = r[i];
}
void orc_m34_mul(const double* a, const double* b, double* out) {
  M34<double> x, y; for (int i = 0; i < 12; ++i) { x[i] = a[i]; y[i] = b[i]; }
  M34<double> r = MulMatrix3x4(x, y);
  for (int i = 0; i < 12; ++i) out[i] = r[i];
}
// Matrix3x4.SetAsTransform, matrix.go:165-185
void orc_set_as_transform(const double* pos, const double* q, double* out) {
  M34<double> m;
  SetAsTransform(m, mk3(pos[0], pos[1], pos[2]), Q4<double>{{q[0], q[1], q[2], q[3]}});
  for (int i = 0; i < 12; ++i) out[i] = m[i];
}
// op: 0 Add, 1 AddScaled(s), 2 ComponentProduct, 3 Cross, 4 Sub, 5 MulWith(s), 6 Normalize
void orc_v3_op(int op, double* v, const double* o, double s) {
  V3<double> a = mk3(v[0], v[1], v[2]), b = mk3(o[0], o[1], o[2]);
  switch (op) {
    case 0: Add(a, b); break;
    case 1: AddScaled(a, b, s); break;
    case 2: ComponentProduct(a, b); break;
    case 3: a = Cross(a, b); break;
    case 4: Sub(a, b); break;
    case 5: MulWith(a, s); break;
    case 6: Normalize(a); break;
  }
  for (int i = 0; i < 3; ++i) v[i] = a[i];
}
double orc_v3_dot(const double* a, const double* b) { return Dot(mk3(a[0], a[1], a[2]), mk3(b[0], b[1], b[2])); }
double orc_v3_magnitude(const double* a) { return Magnitude(mk3(a[0], a[1], a[2])); }
double orc_v3_square_magnitude(const double* a) { return SquareMagnitude(mk3(a[0], a[1], a[2])); }
// SetBlockInertiaTensor + Invert, matrix.go:68-77 and rigidbody.go:176-178
void orc_block_inverse_inertia(const double* half, double mass, double* out) {
  M3<double> m;
  SetBlockInertiaTensor(m, mk3(half[0], half[1], half[2]), mass);
  M3<double> r = Invert(m);
  for (int i = 0; i < 9; ++i) out[i] = r[i];
}
}
