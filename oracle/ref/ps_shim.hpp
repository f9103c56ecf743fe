// Minimal stand-in for the parts of FDPS v5.0c (namespace PS) that the
// reference's physics headers name.  FDPS itself is not vendored with the
// reference (it is cloned at build time by CloneFDPS.sh:2-7), so this shim
// supplies only the scalar typedefs, a 3-vector with FDPS's operator meaning
// (`*` = dot product, `^` = cross product), an indexable particle container,
// an empty domain object, single-process Comm reductions and the monopole
// superparticle type used by CalcGravityForce<PS::SPJMonopole>
// (main.cpp:100-101).  It is test infrastructure for the oracle only.
#pragma once

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

namespace PS {
typedef double F64;
typedef float F32;
typedef int S32;
typedef long long S64;
typedef unsigned int U32;
typedef unsigned long long U64;

struct F64vec {
    F64 x, y, z;
    F64vec() : x(0), y(0), z(0) {}
    F64vec(const F64 s) : x(s), y(s), z(s) {}
    F64vec(const F64 a, const F64 b, const F64 c) : x(a), y(b), z(c) {}
    F64vec &operator=(const F64 s) { x = y = z = s; return *this; }
    F64vec operator+(const F64vec &o) const { return F64vec(x + o.x, y + o.y, z + o.z); }
    F64vec operator-(const F64vec &o) const { return F64vec(x - o.x, y - o.y, z - o.z); }
    F64vec operator-() const { return F64vec(-x, -y, -z); }
    F64 operator*(const F64vec &o) const { return x * o.x + y * o.y + z * o.z; }
    F64vec operator^(const F64vec &o) const {
        return F64vec(y * o.z - z * o.y, z * o.x - x * o.z, x * o.y - y * o.x);
    }
    F64vec operator*(const F64 s) const { return F64vec(x * s, y * s, z * s); }
    F64vec operator/(const F64 s) const { return F64vec(x / s, y / s, z / s); }
    F64vec &operator+=(const F64vec &o) { x += o.x; y += o.y; z += o.z; return *this; }
    F64vec &operator-=(const F64vec &o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
    F64vec &operator*=(const F64 s) { x *= s; y *= s; z *= s; return *this; }
    F64vec &operator/=(const F64 s) { x /= s; y /= s; z /= s; return *this; }
};
inline F64vec operator*(const F64 s, const F64vec &v) { return F64vec(s * v.x, s * v.y, s * v.z); }

template <class T>
class ParticleSystem {
public:
    std::vector<T> ptcl;
    T &operator[](const S32 i) { return ptcl[i]; }
    const T &operator[](const S32 i) const { return ptcl[i]; }
    S32 getNumberOfParticleLocal() const { return (S32)ptcl.size(); }
    void setNumberOfParticleLocal(const S32 n) { ptcl.resize(n); }
};

struct DomainInfo {};

namespace Comm {
template <class T> inline T getMinValue(const T v) { return v; }
template <class T> inline T getMaxValue(const T v) { return v; }
template <class T> inline T getSum(const T v) { return v; }
inline S32 getRank() { return 0; }
inline S32 getNumberOfProc() { return 1; }
}  // namespace Comm

// FDPS monopole superparticle: total mass and centre of mass.
struct SPJMonopole {
    F64 mass;
    F64vec pos;
    F64vec getPos() const { return pos; }
    F64 getCharge() const { return mass; }
};
}  // namespace PS
