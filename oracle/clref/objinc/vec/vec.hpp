// vec/vec.hpp stand-in — TEST INFRASTRUCTURE ONLY.  The reference includes
// the author's separate header-only "vec" library (<vec/vec.hpp>), which its
// checkout does not vendor.  Its OBJ loader uses only a 3- and 4-float vector
// with x()/y()/z()/w() accessors, brace initialisation and multiplication by
// a scalar (obj_load.cpp:83-116, 482-484); that much is restated here.
#pragma once

template <int N>
struct vecf {
  float v[N];
  float& x() { return v[0]; }
  float& y() { return v[1]; }
  float& z() { return v[2]; }
  float& w() { return v[3]; }
  float x() const { return v[0]; }
  float y() const { return v[1]; }
  float z() const { return v[2]; }
  float w() const { return v[3]; }
  vecf operator*(float s) const {
    vecf r;
    for (int i = 0; i < N; i++) r.v[i] = v[i] * s;
    return r;
  }
};

typedef vecf<3> vec3f;
typedef vecf<4> vec4f;
