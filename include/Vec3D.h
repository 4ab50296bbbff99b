// Vec3D<T>: the 3-vector type of the drop-in API (same name, members and operator semantics as the
// reference's include/Vec3D.h:29-109, so user code compiles unchanged).  Mixed float/double
// expressions promote exactly as in the reference: a template operator takes the other type and
// multiplies in the wider one.
#ifndef VX_GB300_VEC3D_H
#define VX_GB300_VEC3D_H

#include <cfloat>
#include <cmath>

#define vec3_X 0
#define vec3_Y 1
#define vec3_Z 2

template <typename T = double>
class Vec3D {
 public:
  T x, y, z;

  Vec3D() : x(0), y(0), z(0) {}
  Vec3D(const T dx, const T dy, const T dz) : x(dx), y(dy), z(dz) {}
  Vec3D(const Vec3D& s) : x(s.x), y(s.y), z(s.z) {}
  template <typename U>
  Vec3D(const Vec3D<U>& s) : x((T)s.x), y((T)s.y), z((T)s.z) {}
  template <typename U>
  operator Vec3D<U>() const { return Vec3D<U>((U)x, (U)y, (U)z); }

  bool IsValid() const { return std::isfinite((double)x) && std::isfinite((double)y) && std::isfinite((double)z); }

  Vec3D& operator=(const Vec3D& s) { x = s.x; y = s.y; z = s.z; return *this; }
  template <typename U>
  Vec3D<T> operator=(const Vec3D<U>& s) { x = (T)s.x; y = (T)s.y; z = (T)s.z; return *this; }

  template <typename U>
  const Vec3D<T> operator+(const Vec3D<U>& s) { return Vec3D<T>(x + s.x, y + s.y, z + s.z); }
  template <typename U>
  const Vec3D<T> operator-(const Vec3D<U>& s) { return Vec3D<T>(x - s.x, y - s.y, z - s.z); }
  template <typename U>
  const Vec3D<T> operator*(const U& f) const { return Vec3D<T>(f * x, f * y, f * z); }
  template <typename U>
  const friend Vec3D<T> operator*(const U f, const Vec3D<T>& v) { return v * f; }
  template <typename U>
  const Vec3D<T>& operator+=(const Vec3D<U>& s) { x += s.x; y += s.y; z += s.z; return *this; }
  template <typename U>
  const Vec3D<T>& operator-=(const Vec3D<U>& s) { x -= s.x; y -= s.y; z -= s.z; return *this; }

  const Vec3D operator+(const Vec3D& v) const { return Vec3D(x + v.x, y + v.y, z + v.z); }
  const Vec3D operator-(const Vec3D& v) const { return Vec3D(x - v.x, y - v.y, z - v.z); }
  const Vec3D operator-() const { return Vec3D(-x, -y, -z); }
  const Vec3D operator*(const T& f) const { return Vec3D(f * x, f * y, f * z); }
  const friend Vec3D operator*(const T f, const Vec3D& v) { return v * f; }
  const Vec3D operator/(const T& f) const { T inv = (T)1.0 / f; return Vec3D(inv * x, inv * y, inv * z); }
  bool operator==(const Vec3D& v) const { return x == v.x && y == v.y && z == v.z; }
  bool operator!=(const Vec3D& v) const { return !(*this == v); }
  const Vec3D& operator+=(const Vec3D& s) { x += s.x; y += s.y; z += s.z; return *this; }
  const Vec3D& operator-=(const Vec3D& s) { x -= s.x; y -= s.y; z -= s.z; return *this; }
  const Vec3D& operator*=(const T f) { x *= f; y *= f; z *= f; return *this; }
  const Vec3D& operator/=(const T f) { T inv = (T)1.0 / f; x *= inv; y *= inv; z *= inv; return *this; }
  const T& operator[](int i) const { int k = i % 3; return k == 0 ? x : (k == 1 ? y : z); }
  T& operator[](int i) { int k = i % 3; return k == 0 ? x : (k == 1 ? y : z); }

  T getX() const { return x; }
  T getY() const { return y; }
  T getZ() const { return z; }
  void setX(const T v) { x = v; }
  void setY(const T v) { y = v; }
  void setZ(const T v) { z = v; }

  T Normalize() { T l = std::sqrt(x * x + y * y + z * z); if (l > 0) { x /= l; y /= l; z /= l; } return l; }
  void NormalizeFast() { T l = std::sqrt(x * x + y * y + z * z); if (l > 0) { T li = 1.0 / l; x *= li; y *= li; z *= li; } }
  Vec3D Rot(const Vec3D u, const T a) {
    T ca = std::cos(a), sa = std::sin(a), t = 1 - ca;
    return Vec3D((u.x * u.x * t + ca) * x + (u.x * u.y * t - u.z * sa) * y + (u.z * u.x * t + u.y * sa) * z,
                 (u.x * u.y * t + u.z * sa) * x + (u.y * u.y * t + ca) * y + (u.y * u.z * t - u.x * sa) * z,
                 (u.z * u.x * t - u.y * sa) * x + (u.y * u.z * t + u.x * sa) * y + (u.z * u.z * t + ca) * z);
  }
  void RotZ(const T a) { T xt = x * std::cos(a) - y * std::sin(a); T yt = x * std::sin(a) + y * std::cos(a); x = xt; y = yt; }
  void RotY(const T a) { T xt = x * std::cos(a) + z * std::sin(a); T zt = -x * std::sin(a) + z * std::cos(a); x = xt; z = zt; }
  void RotX(const T a) { T yt = y * std::cos(a) + z * std::sin(a); T zt = -y * std::sin(a) + z * std::cos(a); y = yt; z = zt; }

  Vec3D Cross(const Vec3D& v) const { return Vec3D(y * v.z - z * v.y, z * v.x - x * v.z, x * v.y - y * v.x); }
  T Dot(const Vec3D& v) const { return x * v.x + y * v.y + z * v.z; }
  Vec3D Abs() const { return Vec3D(x >= 0 ? x : -x, y >= 0 ? y : -y, z >= 0 ? z : -z); }
  Vec3D Normalized() const { T l = std::sqrt(x * x + y * y + z * z); return l > 0 ? (*this) / l : (*this); }
  bool IsNear(const Vec3D& s, const T thresh) { return Dist2(s) < thresh * thresh; }
  T Length() const { return std::sqrt(x * x + y * y + z * z); }
  T Length2() const { return x * x + y * y + z * z; }
  Vec3D Min(const Vec3D& s) const { return Vec3D(x < s.x ? x : s.x, y < s.y ? y : s.y, z < s.z ? z : s.z); }
  Vec3D Max(const Vec3D& s) const { return Vec3D(x > s.x ? x : s.x, y > s.y ? y : s.y, z > s.z ? z : s.z); }
  T Min() const { T m = x < y ? x : y; return z < m ? z : m; }
  T Max() const { T m = x > y ? x : y; return z > m ? z : m; }
  Vec3D Scale(const Vec3D& v) const { return Vec3D(x * v.x, y * v.y, z * v.z); }
  Vec3D ScaleInv(const Vec3D& v) const { return Vec3D(x / v.x, y / v.y, z / v.z); }
  T Dist(const Vec3D& v) const { return std::sqrt(Dist2(v)); }
  T Dist2(const Vec3D& v) const { return (v.x - x) * (v.x - x) + (v.y - y) * (v.y - y) + (v.z - z) * (v.z - z); }
  T AlignWith(const Vec3D target, Vec3D& rotax) const {
    Vec3D a = Normalized(), b = target.Normalized(), ax = a.Cross(b);
    if (ax.Length2() == 0) ax = target.ArbitraryNormal();
    rotax = ax.Normalized();
    return std::acos(a.Dot(b));
  }
  Vec3D ArbitraryNormal() const {
    Vec3D n = Normalized();
    if (std::fabs(n.x) <= std::fabs(n.y) && std::fabs(n.x) <= std::fabs(n.z)) n.x = 1;
    else if (std::fabs(n.y) <= std::fabs(n.x) && std::fabs(n.y) <= std::fabs(n.z)) n.y = 1;
    else n.z = 1;
    return Cross(n).Normalized();
  }
};

#endif
