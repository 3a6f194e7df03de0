// shim.h -- the small part of the GMTL 0.6.1 interface that the reference's
// ray-tracing sources (src/Scene.cpp, Mesh.cpp, Triangle.cpp, Material.cpp,
// the recorders, Datatype.cpp, SoundFile.cpp) call, written for this
// project so that those sources compile where they lie.  GMTL itself is not
// vendored and not installed; this is not its code.
//
// TEST INFRASTRUCTURE ONLY (oracle/build_ref.py builds oracle/_ref with
// it).  The arithmetic follows the oracle's restatement exactly, so a
// difference between the reference-built render and the oracle is a
// difference in the reference's own code:
//   * dot / lengthSquared = (x*x' + y*y') + z*z'; length = sqrtf of it;
//   * normalize divides each component by the length when it is non-zero;
//   * cross in the usual component order; reflect(v, n) = v - 2 (v.n) n;
//   * the triangle normal normalizes cross(v1 - v0, v2 - v0);
//   * intersectDoubleSided is Moller & Trumbore (1997), non-culling,
//     epsilon 1e-6, in the paper's order of operations;
//   * Math::unitRandom replays a tape of uniforms (ref_tape_*), so the
//     reference consumes the oracle's counter-based draws in its own call
//     order.  A call past the end of the tape sets a flag and returns 0.5.
#pragma once

#include <cmath>
#include <ostream>

namespace gmtl {

template <typename T, unsigned N>
struct VecBase {
  T mData[N];
  VecBase() {
    for (unsigned i = 0; i < N; ++i) mData[i] = T(0);
  }
  VecBase(T x, T y, T z) {
    mData[0] = x;
    mData[1] = y;
    mData[2] = z;
  }
  T& operator[](unsigned i) { return mData[i]; }
  const T& operator[](unsigned i) const { return mData[i]; }
  T* getData() { return mData; }
  const T* getData() const { return mData; }
};

template <typename T, unsigned N>
struct Vec : VecBase<T, N> {
  Vec() {}
  Vec(T x, T y, T z) : VecBase<T, N>(x, y, z) {}
  Vec(const VecBase<T, N>& o) : VecBase<T, N>(o) {}
};

template <typename T, unsigned N>
struct Point : VecBase<T, N> {
  Point() {}
  Point(T x, T y, T z) : VecBase<T, N>(x, y, z) {}
  Point(const VecBase<T, N>& o) : VecBase<T, N>(o) {}
};

typedef Vec<float, 3> Vec3f;
typedef Point<float, 3> Point3f;

template <typename T, unsigned N>
VecBase<T, N> operator+(const VecBase<T, N>& a, const VecBase<T, N>& b) {
  VecBase<T, N> r;
  for (unsigned i = 0; i < N; ++i) r[i] = a[i] + b[i];
  return r;
}
template <typename T, unsigned N>
VecBase<T, N> operator-(const VecBase<T, N>& a, const VecBase<T, N>& b) {
  VecBase<T, N> r;
  for (unsigned i = 0; i < N; ++i) r[i] = a[i] - b[i];
  return r;
}
template <typename T, unsigned N>
VecBase<T, N> operator-(const VecBase<T, N>& a) {
  VecBase<T, N> r;
  for (unsigned i = 0; i < N; ++i) r[i] = -a[i];
  return r;
}
template <typename T, unsigned N>
VecBase<T, N> operator*(const VecBase<T, N>& a, T s) {
  VecBase<T, N> r;
  for (unsigned i = 0; i < N; ++i) r[i] = a[i] * s;
  return r;
}
template <typename T, unsigned N>
VecBase<T, N> operator*(T s, const VecBase<T, N>& a) {
  VecBase<T, N> r;
  for (unsigned i = 0; i < N; ++i) r[i] = s * a[i];
  return r;
}
template <typename T, unsigned N>
VecBase<T, N> operator/(const VecBase<T, N>& a, T s) {
  VecBase<T, N> r;
  for (unsigned i = 0; i < N; ++i) r[i] = a[i] / s;
  return r;
}
template <typename T, unsigned N>
VecBase<T, N>& operator+=(VecBase<T, N>& a, const VecBase<T, N>& b) {
  for (unsigned i = 0; i < N; ++i) a[i] += b[i];
  return a;
}
template <typename T, unsigned N>
VecBase<T, N>& operator-=(VecBase<T, N>& a, const VecBase<T, N>& b) {
  for (unsigned i = 0; i < N; ++i) a[i] -= b[i];
  return a;
}
template <typename T, unsigned N>
VecBase<T, N>& operator*=(VecBase<T, N>& a, T s) {
  for (unsigned i = 0; i < N; ++i) a[i] *= s;
  return a;
}
template <typename T, unsigned N>
VecBase<T, N>& operator/=(VecBase<T, N>& a, T s) {
  for (unsigned i = 0; i < N; ++i) a[i] /= s;
  return a;
}
template <typename T, unsigned N>
bool operator==(const VecBase<T, N>& a, const VecBase<T, N>& b) {
  for (unsigned i = 0; i < N; ++i)
    if (a[i] != b[i]) return false;
  return true;
}
template <typename T, unsigned N>
std::ostream& operator<<(std::ostream& os, const VecBase<T, N>& v) {
  os << "(";
  for (unsigned i = 0; i < N; ++i) os << (i ? ", " : "") << v[i];
  return os << ")";
}

template <typename T, unsigned N>
T dot(const VecBase<T, N>& a, const VecBase<T, N>& b) {
  return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2];
}
template <typename T, unsigned N>
T lengthSquared(const VecBase<T, N>& a) {
  return dot(a, a);
}
template <typename T, unsigned N>
T length(const VecBase<T, N>& a) {
  return std::sqrt(lengthSquared(a));
}
template <typename T, unsigned N>
T normalize(VecBase<T, N>& a) {
  const T l = length(a);
  if (l != T(0))
    for (unsigned i = 0; i < N; ++i) a[i] /= l;
  return l;
}
template <typename T, unsigned N>
Vec<T, N> makeNormal(const VecBase<T, N>& a) {
  Vec<T, N> r(a);
  normalize(r);
  return r;
}
template <typename T>
VecBase<T, 3>& cross(VecBase<T, 3>& r, const VecBase<T, 3>& a, const VecBase<T, 3>& b) {
  const T x = a[1] * b[2] - a[2] * b[1];
  const T y = a[2] * b[0] - a[0] * b[2];
  const T z = a[0] * b[1] - a[1] * b[0];
  r[0] = x;
  r[1] = y;
  r[2] = z;
  return r;
}
template <typename T>
Vec<T, 3> makeCross(const VecBase<T, 3>& a, const VecBase<T, 3>& b) {
  Vec<T, 3> r;
  cross(r, a, b);
  return r;
}
template <typename T, unsigned N>
VecBase<T, N>& reflect(VecBase<T, N>& r, const VecBase<T, N>& v, const VecBase<T, N>& n) {
  const T d = dot(v, n);
  VecBase<T, N> out;
  for (unsigned i = 0; i < N; ++i) out[i] = v[i] - T(2) * (d * n[i]);
  r = out;
  return r;
}

template <typename T>
struct Ray {
  Point<T, 3> mOrigin;
  Vec<T, 3> mDir;
  Ray() {}
  Ray(const Point<T, 3>& o, const Vec<T, 3>& d) : mOrigin(o), mDir(d) {}
  const Point<T, 3>& getOrigin() const { return mOrigin; }
  const Vec<T, 3>& getDir() const { return mDir; }
};
typedef Ray<float> Rayf;

template <typename T>
struct LineSeg : Ray<T> {
  LineSeg() {}
  LineSeg(const Point<T, 3>& a, const Point<T, 3>& b) : Ray<T>(a, Vec<T, 3>(b - a)) {}
  T getLength() const { return length(this->mDir); }
};
typedef LineSeg<float> LineSegf;

template <typename T>
struct Tri {
  Point<T, 3> mVerts[3];
  Tri() {}
  Tri(const Point<T, 3>& a, const Point<T, 3>& b, const Point<T, 3>& c) {
    mVerts[0] = a;
    mVerts[1] = b;
    mVerts[2] = c;
  }
  Point<T, 3>& operator[](unsigned i) { return mVerts[i]; }
  const Point<T, 3>& operator[](unsigned i) const { return mVerts[i]; }
  Vec<T, 3> edge(int i) const { return Vec<T, 3>(mVerts[(i + 1) % 3] - mVerts[i]); }
};
typedef Tri<float> Trif;

template <typename T>
Vec<T, 3> normal(const Tri<T>& t) {
  Vec<T, 3> n = makeCross(Vec<T, 3>(t[1] - t[0]), Vec<T, 3>(t[2] - t[0]));
  normalize(n);
  return n;
}

template <typename T>
bool intersectDoubleSided(const Tri<T>& tri, const Ray<T>& ray, T& u, T& v, T& t) {
  const Vec<T, 3> e1(tri[1] - tri[0]), e2(tri[2] - tri[0]);
  const Vec<T, 3> pvec = makeCross(ray.mDir, e2);
  const T det = dot(e1, pvec);
  if (det > T(-1e-6) && det < T(1e-6)) return false;
  const T inv_det = T(1) / det;
  const Vec<T, 3> tvec(ray.mOrigin - tri[0]);
  u = dot(tvec, pvec) * inv_det;
  if (u < T(0) || u > T(1)) return false;
  const Vec<T, 3> qvec = makeCross(tvec, e1);
  v = dot(ray.mDir, qvec) * inv_det;
  if (v < T(0) || u + v > T(1)) return false;
  t = dot(e2, qvec) * inv_det;
  return true;
}

namespace Math {
float unitRandom();
inline void seedRandom(unsigned) {}
inline float rangeRandom(float a, float b) { return (b - a) * unitRandom() + a; }
inline float sqrt(float x) { return std::sqrt(x); }
}  // namespace Math

}  // namespace gmtl
