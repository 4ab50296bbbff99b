// Quat3D<T>: the quaternion type of the drop-in API (same name, members and semantics as the
// reference's include/Quat3D.h:42-204).  Host-side evaluation uses the C library, like the
// reference; the GPU path evaluates the same formulas with correctly rounded functions.
#ifndef VX_GB300_QUAT3D_H
#define VX_GB300_QUAT3D_H

#include <cmath>

#include "Vec3D.h"

#ifndef PI
#define PI 3.14159265358979
#endif
#define DBL_EPSILONx24 5.328e-15
#define DISCARD_ANGLE_RAD 1e-7
#define SMALL_ANGLE_RAD 1.732e-2
#define SMALL_ANGLE_W 0.9999625
#define W_THRESH_ACOS2SQRT 0.9988
#define SLTHRESH_ACOS2SQRT 2.4e-3

template <typename T = double>
class Quat3D {
 public:
  T w, x, y, z;

  Quat3D() : w(1), x(0), y(0), z(0) {}
  Quat3D(const T dw, const T dx, const T dy, const T dz) : w(dw), x(dx), y(dy), z(dz) {}
  Quat3D(const Quat3D& q) : w(q.w), x(q.x), y(q.y), z(q.z) {}
  Quat3D(const Vec3D<T>& rotationVector) { FromRotationVector(rotationVector); }
  Quat3D(const T angle, const Vec3D<T>& axis) {
    const T a = angle * (T)0.5;
    const T s = std::sin(a);
    w = std::cos(a);
    x = axis.x * s; y = axis.y * s; z = axis.z * s;
  }
  Quat3D(const Vec3D<T>& from, const Vec3D<T>& to) {
    T theta = std::acos(from.Dot(to) / std::sqrt(from.Length2() * to.Length2()));
    if (theta <= 0) { *this = Quat3D(1, 0, 0, 0); return; }
    Vec3D<T> axis = from.Cross(to);
    axis.NormalizeFast();
    if (theta > PI - DISCARD_ANGLE_RAD) { *this = Quat3D(axis); return; }
    *this = Quat3D(theta, axis);
  }
  template <typename U>
  Quat3D(const Quat3D<U>& q) : w(q.w), x(q.x), y(q.y), z(q.z) {}
  template <typename U>
  Quat3D(const Vec3D<U>& v) : w(0), x(v.x), y(v.y), z(v.z) {}
  template <typename U>
  operator Quat3D<U>() const { return Quat3D<U>(w, x, y, z); }

  Quat3D& operator=(const Quat3D& s) { w = s.w; x = s.x; y = s.y; z = s.z; return *this; }
  const Quat3D operator+(const Quat3D& s) const { return Quat3D(w + s.w, x + s.x, y + s.y, z + s.z); }
  const Quat3D operator-(const Quat3D& s) const { return Quat3D(w - s.w, x - s.x, y - s.y, z - s.z); }
  const Quat3D operator*(const T f) const { return Quat3D(w * f, x * f, y * f, z * f); }
  const friend Quat3D operator*(const T f, const Quat3D v) { return Quat3D(v.w * f, v.x * f, v.y * f, v.z * f); }
  const Quat3D operator*(const Quat3D& f) const {
    return Quat3D(w * f.w - x * f.x - y * f.y - z * f.z, w * f.x + x * f.w + y * f.z - z * f.y,
                  w * f.y - x * f.z + y * f.w + z * f.x, w * f.z + x * f.y - y * f.x + z * f.w);
  }
  bool operator==(const Quat3D& s) const { return w == s.w && x == s.x && y == s.y && z == s.z; }
  bool operator!=(const Quat3D& s) const { return !(*this == s); }
  const Quat3D& operator+=(const Quat3D& s) { w += s.w; x += s.x; y += s.y; z += s.z; return *this; }
  const Quat3D& operator-=(const Quat3D& s) { w -= s.w; x -= s.x; y -= s.y; z -= s.z; return *this; }
  const Vec3D<T> ToVec() const { return Vec3D<T>(x, y, z); }

  const T Length() const { return std::sqrt(Length2()); }
  const T Length2() const { return w * w + x * x + y * y + z * z; }
  const T Normalize() {
    T l = Length();
    if (l == 0) { w = 1; x = y = z = 0; }
    else if (l > 0) { T li = 1.0 / l; w *= li; x *= li; y *= li; z *= li; }
    return l;
  }
  void NormalizeFast() {
    T l = std::sqrt(x * x + y * y + z * z + w * w);
    if (l != 0) { T li = 1.0 / l; w *= li; x *= li; y *= li; z *= li; }
    if (w >= 1.0) { w = 1.0; x = y = z = 0; }
  }
  const Quat3D Inverse() const { T n = w * w + x * x + y * y + z * z; return Quat3D(w / n, -x / n, -y / n, -z / n); }
  const Quat3D Conjugate() const { return Quat3D(w, -x, -y, -z); }

  const T Angle() const { return 2.0 * std::acos(w > 1 ? 1 : w); }
  const T AngleDegrees() const { return Angle() * 57.29577951308232; }
  bool IsNegligibleAngle() const { return 2.0 * std::acos(w) < DISCARD_ANGLE_RAD; }
  bool IsSmallAngle() const { return w > SMALL_ANGLE_W; }
  Vec3D<T> Axis() const {
    T sl = 1.0 - w * w;
    if (sl <= 0) return Vec3D<T>(1, 0, 0);
    return Vec3D<T>(x, y, z) / std::sqrt(sl);
  }
  Vec3D<T> AxisUnNormalized() const { return Vec3D<T>(x, y, z); }
  void AngleAxis(T& angle, Vec3D<T>& axis) const { AngleAxisUnNormalized(angle, axis); axis.NormalizeFast(); }
  void AngleAxisUnNormalized(T& angle, Vec3D<T>& axis) const {
    if (w >= 1.0) { angle = 0; axis = Vec3D<T>(1, 0, 0); return; }
    angle = 2.0 * std::acos(w > 1 ? 1 : w);
    axis = Vec3D<T>(x, y, z);
  }

  // rotation vector (axis * angle) of this rotation; near zero angle acos(w) ~ sqrt(2-2w)
  const Vec3D<T> ToRotationVector() const {
    if (w >= 1.0 || w <= -1.0) return Vec3D<T>(0, 0, 0);
    T sl = 1.0 - w * w;
    if (sl < SLTHRESH_ACOS2SQRT) return Vec3D<T>(x, y, z) * 2.0 * std::sqrt((2 - 2 * w) / sl);
    return Vec3D<T>(x, y, z) * 2.0 * std::acos(w) / std::sqrt(sl);
  }
  void FromRotationVector(const Vec3D<T>& v) {
    Vec3D<T> th = v / 2;
    T s, m2 = th.Length2();
    if (m2 * m2 < DBL_EPSILONx24) {
      w = 1.0 - 0.5 * m2;
      s = 1.0 - m2 / 6.0;
    } else {
      T m = std::sqrt(m2);
      w = std::cos(m);
      s = std::sin(m) / m;
    }
    x = th.x * s; y = th.y * s; z = th.z * s;
  }
  // rotation that takes `from` onto +X
  void FromAngleToPosX(const Vec3D<T>& from) {
    if (Vec3D<T>(0, 0, 0) == from) return;
    T yx = from.y / from.x, zx = from.z / from.x;
    if (yx < SMALL_ANGLE_RAD && yx > -SMALL_ANGLE_RAD && zx < SMALL_ANGLE_RAD && zx > -SMALL_ANGLE_RAD) {
      x = 0; y = 0.5 * zx; z = -0.5 * yx;
      w = 1 + 0.5 * (-y * y - z * z);
      return;
    }
    Vec3D<double> n = from;
    n.NormalizeFast();
    T theta = std::acos(n.x);
    if (theta > PI - DISCARD_ANGLE_RAD) { w = 0; x = 0; y = 1; z = 0; return; }
    const T ami = 1.0 / std::sqrt(n.z * n.z + n.y * n.y);
    const T a = 0.5 * theta;
    const T s = std::sin(a);
    w = std::cos(a); x = 0; y = n.z * ami * s; z = -n.y * ami * s;
  }
  const Vec3D<T> RotateVec3D(const Vec3D<T>& f) const {
    T tw = f.x * x + f.y * y + f.z * z, tx = f.x * w - f.y * z + f.z * y;
    T ty = f.x * z + f.y * w - f.z * x, tz = -f.x * y + f.y * x + f.z * w;
    return Vec3D<T>(w * tx + x * tw + y * tz - z * ty, w * ty - x * tz + y * tw + z * tx, w * tz + x * ty - y * tx + z * tw);
  }
  template <typename U>
  const Vec3D<U> RotateVec3D(const Vec3D<U>& f) const {
    U fx = (U)f.x, fy = (U)f.y, fz = (U)f.z;
    U tw = (U)(fx * x + fy * y + fz * z), tx = (U)(fx * w - fy * z + fz * y);
    U ty = (U)(fx * z + fy * w - fz * x), tz = (U)(-fx * y + fy * x + fz * w);
    return Vec3D<U>((U)(w * tx + x * tw + y * tz - z * ty), (U)(w * ty - x * tz + y * tw + z * tx),
                    (U)(w * tz + x * ty - y * tx + z * tw));
  }
  const Vec3D<T> RotateVec3DInv(const Vec3D<T>& f) const {
    T tw = x * f.x + y * f.y + z * f.z, tx = w * f.x - y * f.z + z * f.y;
    T ty = w * f.y + x * f.z - z * f.x, tz = w * f.z - x * f.y + y * f.x;
    return Vec3D<T>(tw * x + tx * w + ty * z - tz * y, tw * y - tx * z + ty * w + tz * x, tw * z + tx * y - ty * x + tz * w);
  }
  template <typename U>
  const Vec3D<U> RotateVec3DInv(const Vec3D<U>& f) const {
    T tw = x * f.x + y * f.y + z * f.z, tx = w * f.x - y * f.z + z * f.y;
    T ty = w * f.y + x * f.z - z * f.x, tz = w * f.z - x * f.y + y * f.x;
    return Vec3D<U>(tw * x + tx * w + ty * z - tz * y, tw * y - tx * z + ty * w + tz * x, tw * z + tx * y - ty * x + tz * w);
  }
};

#endif
