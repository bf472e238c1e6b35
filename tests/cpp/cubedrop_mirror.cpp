// The cubedrop frame loop (examples/cubedrop.go:29-75) written against the
// C++ mirror of the cubez API (include/cubez.hpp): one body at a time, one
// pair at a time, exactly as the Go example calls the package.
//
//   cubedrop_mirror <in.bin> <out.bin> <frames>
//
// in.bin: plane (4 doubles), n (1 double), then per body 37 doubles:
//   shape, mass, half_size[3], radius, position[3], orientation[4],
//   velocity[3], rotation[3], acceleration[3], inverse_inertia[9],
//   linear_damping, angular_damping, can_sleep, (3 spare)
// out.bin: per frame the contact count (1 double), then per body
//   position[3], orientation[4], velocity[3], rotation[3].
#include <cstdio>
#include <memory>
#include <vector>

#include "cubez.hpp"

using namespace cubez;

int main(int argc, char** argv) {
  if (argc != 4) {
    std::fprintf(stderr, "usage: %s in.bin out.bin frames\n", argv[0]);
    return 2;
  }
  std::FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 2;
  std::vector<double> in;
  double x;
  while (std::fread(&x, sizeof x, 1, f) == 1) in.push_back(x);
  std::fclose(f);
  const int frames = std::atoi(argv[3]);
  const double dt = 1.0 / 60.0;

  CollisionPlane ground(Vector3{in[0], in[1], in[2]}, in[3]);
  const int n = (int)in[4];
  std::vector<std::unique_ptr<RigidBody>> bodies;
  std::vector<std::unique_ptr<Collider>> colliders;
  for (int i = 0; i < n; ++i) {
    const double* p = &in[5 + 37 * (size_t)i];
    auto body = std::make_unique<RigidBody>();
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
    if (p[0] == CZ_SHAPE_CUBE)
      colliders.push_back(std::make_unique<CollisionCube>(body.get(), Vector3{p[2], p[3], p[4]}));
    else
      colliders.push_back(std::make_unique<CollisionSphere>(body.get(), p[5]));
    bodies.push_back(std::move(body));
  }

  std::FILE* o = std::fopen(argv[2], "wb");
  if (!o) return 2;
  try {
    std::vector<Contact> contacts;
    for (int frame = 0; frame < frames; ++frame) {
      for (auto& b : bodies) b->Integrate(dt);
      contacts.clear();
      for (int i = 0; i < n; ++i) {
        colliders[i]->CheckAgainstHalfSpace(ground, contacts);
        for (int j = 0; j < n; ++j)
          if (j != i) CheckForCollisions(*colliders[i], *colliders[j], contacts);
      }
      ResolveContacts((int)contacts.size() * 4, contacts, dt);
      const double count = (double)contacts.size();
      std::fwrite(&count, sizeof count, 1, o);
      for (auto& b : bodies) {
        std::fwrite(b->Position.data(), sizeof(double), 3, o);
        std::fwrite(b->Orientation.data(), sizeof(double), 4, o);
        std::fwrite(b->Velocity.data(), sizeof(double), 3, o);
        std::fwrite(b->Rotation.data(), sizeof(double), 3, o);
      }
    }
  } catch (const Error& e) {
    std::fprintf(stderr, "cubez error %d: %s\n", e.status, e.what());
    std::fclose(o);
    return 1;
  }
  std::fclose(o);
  return 0;
}
