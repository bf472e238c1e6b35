// The frame loops of the reference's examples written against the C++ mirror
// of the cubez API (include/cubez.hpp): one body at a time, one pair at a
// time, exactly as the Go examples call the package.
//
//   mirror_loops cubedrop|ballistic <in.bin> <out.bin> <frames>
//
// cubedrop  (examples/cubedrop.go:29-75): every body is integrated; for each
//           body the half-space test, then every other body;
//           ResolveContacts(len(contacts) * 4), the benchmark configurations'
//           budget (the example itself passes 8).
// ballistic (examples/ballistic.go:27-105): body 0 is the cube, body 1 the
//           backboard (never integrated), bodies 2.. the bullets; the
//           example's test order; ResolveContacts(len(contacts) * 8).
//
// in.bin: plane (4 doubles), n (1 double), then per body 49 doubles:
//   shape, mass (0 = SetInfiniteMass), half_size[3], radius, position[3],
//   orientation[4], velocity[3], rotation[3], acceleration[3],
//   inverse_inertia[9], linear_damping, angular_damping, can_sleep,
//   (3 spare), collider Offset[12].
// out.bin: per frame the contact count (1 double), then per body
//   position[3], orientation[4], velocity[3], rotation[3].
#include <cstdio>
#include <cstring>
#include <memory>
#include <vector>

#include "cubez.hpp"

using namespace cubez;

namespace {
constexpr int kRow = 49;

struct World {
  std::vector<std::unique_ptr<RigidBody>> bodies;
  std::vector<std::unique_ptr<Collider>> colliders;
};

void build(const std::vector<double>& in, int n, World& wd) {
  for (int i = 0; i < n; ++i) {
    const double* p = &in[5 + kRow * (size_t)i];
    auto body = std::make_unique<RigidBody>();
    if (p[1] == 0)
      body->SetInfiniteMass();
    else
      body->SetMass(p[1]);
    body->Position = Vector3{p[6], p[7], p[8]};
    body->Orientation = Quat{p[9], p[10], p[11], p[12]};
    body->Velocity = Vector3{p[13], p[14], p[15]};
    body->Rotation = Vector3{p[16], p[17], p[18]};
    body->Acceleration = Vector3{p[19], p[20], p[21]};
    for (int k = 0; k < 9; ++k) body->InverseInertiaTensor[k] = p[22 + k];
    body->LinearDamping = p[31];
    body->AngularDamping = p[32];
    body->CanSleep = p[33] != 0;
    body->CalculateDerivedData();
    Matrix3x4 offset;
    for (int k = 0; k < 12; ++k) offset[k] = p[37 + k];
    if (p[0] == CZ_SHAPE_CUBE) {
      auto c = std::make_unique<CollisionCube>(body.get(), Vector3{p[2], p[3], p[4]});
      c->Offset = offset;
      wd.colliders.push_back(std::move(c));
    } else {
      auto s = std::make_unique<CollisionSphere>(body.get(), p[5]);
      s->Offset = offset;
      wd.colliders.push_back(std::move(s));
    }
    wd.colliders.back()->CalculateDerivedData();
    wd.bodies.push_back(std::move(body));
  }
}

void write_frame(std::FILE* o, size_t contacts, const World& wd) {
  const double count = (double)contacts;
  std::fwrite(&count, sizeof count, 1, o);
  for (auto& b : wd.bodies) {
    std::fwrite(b->Position.data(), sizeof(double), 3, o);
    std::fwrite(b->Orientation.data(), sizeof(double), 4, o);
    std::fwrite(b->Velocity.data(), sizeof(double), 3, o);
    std::fwrite(b->Rotation.data(), sizeof(double), 3, o);
  }
}

// examples/cubedrop.go:29-75
void cubedrop_frame(World& wd, const CollisionPlane& ground, double dt, std::vector<Contact>& contacts) {
  const int n = (int)wd.bodies.size();
  for (int i = 0; i < n; ++i) {
    wd.bodies[i]->Integrate(dt);
    wd.colliders[i]->CalculateDerivedData();
  }
  contacts.clear();
  for (int i = 0; i < n; ++i) {
    wd.colliders[i]->CheckAgainstHalfSpace(ground, contacts);
    for (int j = 0; j < n; ++j)
      if (j != i) CheckForCollisions(*wd.colliders[i], *wd.colliders[j], contacts);
  }
  ResolveContacts((int)contacts.size() * 4, contacts, dt);
}

// examples/ballistic.go:27-105 (updateObjects, generateContacts, updateCallback)
void ballistic_frame(World& wd, CollisionPlane& ground, double dt, std::vector<Contact>& contacts) {
  const int n = (int)wd.bodies.size();
  Collider& cube = *wd.colliders[0];
  Collider& backboard = *wd.colliders[1];
  wd.bodies[0]->Integrate(dt);
  cube.CalculateDerivedData();
  for (int k = 2; k < n; ++k) {
    wd.bodies[k]->Integrate(dt);
    wd.colliders[k]->CalculateDerivedData();
  }
  contacts.clear();
  bool found = CheckForCollisions(cube, ground, contacts);
  found = CheckForCollisions(cube, backboard, contacts) || found;
  for (int k = 2; k < n; ++k) {
    Collider& bullet = *wd.colliders[k];
    found = CheckForCollisions(bullet, ground, contacts) || found;
    found = CheckForCollisions(cube, bullet, contacts) || found;
    found = CheckForCollisions(backboard, bullet, contacts) || found;
    for (int k2 = 2; k2 < n; ++k2)
      if (k2 != k) found = CheckForCollisions(*wd.colliders[k2], bullet, contacts) || found;
  }
  if (found) ResolveContacts((int)contacts.size() * 8, contacts, dt);
}
}  // namespace

int main(int argc, char** argv) {
  if (argc != 5 || (std::strcmp(argv[1], "cubedrop") != 0 && std::strcmp(argv[1], "ballistic") != 0)) {
    std::fprintf(stderr, "usage: %s cubedrop|ballistic in.bin out.bin frames\n", argv[0]);
    return 2;
  }
  const bool ballistic = std::strcmp(argv[1], "ballistic") == 0;
  std::FILE* f = std::fopen(argv[2], "rb");
  if (!f) return 2;
  std::vector<double> in;
  double x;
  while (std::fread(&x, sizeof x, 1, f) == 1) in.push_back(x);
  std::fclose(f);
  const int frames = std::atoi(argv[4]);
  const double dt = 1.0 / 60.0;
  if (in.size() < 5) return 2;
  const int n = (int)in[4];
  if (in.size() != 5 + (size_t)kRow * n || (ballistic && n < 2)) return 2;

  CollisionPlane ground(Vector3{in[0], in[1], in[2]}, in[3]);
  World wd;
  build(in, n, wd);
  std::FILE* o = std::fopen(argv[3], "wb");
  if (!o) return 2;
  try {
    std::vector<Contact> contacts;
    for (int frame = 0; frame < frames; ++frame) {
      if (ballistic)
        ballistic_frame(wd, ground, dt, contacts);
      else
        cubedrop_frame(wd, ground, dt, contacts);
      write_frame(o, contacts.size(), wd);
    }
  } catch (const Error& e) {
    std::fprintf(stderr, "cubez error %d: %s\n", e.status, e.what());
    std::fclose(o);
    return 1;
  }
  std::fclose(o);
  return 0;
}
