// The C++ mirror's host-side setup math (include/cubez.hpp: MulMatrix3x4,
// Invert, BlockInertiaTensor, AsTransform, RealEqual), run on records read
// from a file, for comparison with the oracle bit for bit, after a check of
// the Go constructor functions' defaults (exit 3 if one is wrong).  Uses no
// GPU.
//
//   host_math <in.bin> <out.bin>
//
// in.bin, per record (doubles): a[12], b[12], m[9], half[3], mass, x, y,
//   position[3], quaternion[4].
// out.bin, per record (doubles): MulMatrix3x4(a, b)[12], Invert(m)[9],
//   Invert(BlockInertiaTensor(half, mass))[9], RealEqual(x, y) (0 or 1),
//   AsTransform(position, quaternion)[12].
#include <cstdio>
#include <vector>

#include "cubez.hpp"

using namespace cubez;

// The Go constructor functions give the Go defaults (rigidbody.go:104-114,
// colliders.go:81-86, 136-141, 265-270, contact.go:54-57).
static bool constructors_ok() {
  auto body = NewRigidBody();
  auto plane = NewCollisionPlane(Vector3{0, 1, 0}, 2.5);
  auto cube = NewCollisionCube(nullptr, Vector3{0.5, 0.25, 1});
  auto sphere = NewCollisionSphere(body.get(), 0.75);
  const Contact c = NewContact();
  return body->LinearDamping == 0.95 && body->AngularDamping == 0.95 && body->Acceleration[1] == -9.78 &&
         body->Orientation == Quat{1, 0, 0, 0} && body->IsAwake && body->CanSleep && !body->HasFiniteMass() &&
         plane->Offset == 2.5 && cube->GetBody() != nullptr && cube->Offset == Identity3x4() &&
         sphere->GetBody() == body.get() && sphere->Radius == 0.75 && c.Bodies[0] == nullptr &&
         c.Penetration == 0 && c.Friction == 0;
}

int main(int argc, char** argv) {
  if (argc != 3) return 2;
  if (!constructors_ok()) return 3;
  std::FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 2;
  std::vector<double> in;
  double x;
  while (std::fread(&x, sizeof x, 1, f) == 1) in.push_back(x);
  std::fclose(f);
  const size_t rec = 12 + 12 + 9 + 3 + 1 + 2 + 3 + 4;
  if (in.size() % rec != 0) return 2;
  std::FILE* o = std::fopen(argv[2], "wb");
  if (!o) return 2;
  for (size_t r = 0; r < in.size() / rec; ++r) {
    const double* p = &in[r * rec];
    Matrix3x4 a, b;
    Matrix3 m;
    for (int k = 0; k < 12; ++k) a[k] = p[k], b[k] = p[12 + k];
    for (int k = 0; k < 9; ++k) m[k] = p[24 + k];
    const Vector3 half{p[33], p[34], p[35]};
    const double mass = p[36], rx = p[37], ry = p[38];
    const Vector3 pos{p[39], p[40], p[41]};
    const Quat q{p[42], p[43], p[44], p[45]};
    const Matrix3x4 ab = MulMatrix3x4(a, b);
    const Matrix3 mi = Invert(m);
    const Matrix3 bi = Invert(BlockInertiaTensor(half, mass));
    const double eq = detail::RealEqual(rx, ry) ? 1.0 : 0.0;
    const Matrix3x4 t = AsTransform(pos, q);
    std::fwrite(ab.data(), sizeof(double), 12, o);
    std::fwrite(mi.data(), sizeof(double), 9, o);
    std::fwrite(bi.data(), sizeof(double), 9, o);
    std::fwrite(&eq, sizeof eq, 1, o);
    std::fwrite(t.data(), sizeof(double), 12, o);
  }
  std::fclose(o);
  return 0;
}
