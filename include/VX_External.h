// CVX_External: fixed degrees of freedom, prescribed displacements, external force and moment of a
// voxel.  Same API as the reference (include/VX_External.h:18-100).  Setters tell the owning
// CVoxelyze that the device copy of the externals table is stale.
#ifndef VX_GB300_EXTERNAL_H
#define VX_GB300_EXTERNAL_H

#include "Quat3D.h"
#include "Vec3D.h"

typedef unsigned char dofObject;
enum dofComponent {
  X_TRANSLATE = 1 << 0,
  Y_TRANSLATE = 1 << 1,
  Z_TRANSLATE = 1 << 2,
  X_ROTATE = 1 << 3,
  Y_ROTATE = 1 << 4,
  Z_ROTATE = 1 << 5
};
inline void dofSet(dofObject& obj, dofComponent dof, bool set) { set ? obj |= dof : obj &= ~dof; }
inline void dofSetAll(dofObject& obj, bool set) { set ? obj |= 0x3F : obj &= ~0x3F; }
inline bool dofIsSet(dofObject obj, dofComponent dof) { return (dof & obj) ? true : false; }
inline bool dofIsAllSet(dofObject obj) { return (obj & 0x3F) == 0x3F; }
inline bool dofIsNoneSet(dofObject obj) { return !(obj & 0x3F); }
inline dofObject dof(bool tx, bool ty, bool tz, bool rx, bool ry, bool rz) {
  dofObject r = 0;
  dofSet(r, X_TRANSLATE, tx); dofSet(r, Y_TRANSLATE, ty); dofSet(r, Z_TRANSLATE, tz);
  dofSet(r, X_ROTATE, rx); dofSet(r, Y_ROTATE, ry); dofSet(r, Z_ROTATE, rz);
  return r;
}

class CVoxelyze;

class CVX_External {
 public:
  CVX_External();
  ~CVX_External() {}
  CVX_External(const CVX_External& e) { *this = e; }
  CVX_External& operator=(const CVX_External& e);
  bool operator==(const CVX_External& b) {
    return dofFixed == b.dofFixed && extForce == b.extForce && extMoment == b.extMoment &&
           extTranslation == b.extTranslation && extRotation == b.extRotation;
  }

  void reset();
  bool isEmpty() { return dofFixed == 0 && extForce == Vec3D<float>() && extMoment == Vec3D<float>(); }

  bool isFixed(dofComponent d) const { return dofIsSet(dofFixed, d); }
  bool isFixedAll() const { return dofIsAllSet(dofFixed); }
  bool isFixedAllTranslation() const { return isFixed(X_TRANSLATE) && isFixed(Y_TRANSLATE) && isFixed(Z_TRANSLATE); }
  bool isFixedAllRotation() const { return isFixed(X_ROTATE) && isFixed(Y_ROTATE) && isFixed(Z_ROTATE); }
  bool isFixedAny() const { return dofFixed != 0; }
  bool isFixedAnyTranslation() const { return isFixed(X_TRANSLATE) || isFixed(Y_TRANSLATE) || isFixed(Z_TRANSLATE); }
  bool isFixedAnyRotation() const { return isFixed(X_ROTATE) || isFixed(Y_ROTATE) || isFixed(Z_ROTATE); }

  Vec3D<double> translation() const { return extTranslation; }
  Vec3D<double> rotation() const { return extRotation; }
  Quat3D<double> rotationQuat() const { return hasRotQ ? extRotationQ : Quat3D<double>(); }

  void setFixed(bool xTranslate, bool yTranslate, bool zTranslate, bool xRotate, bool yRotate, bool zRotate);
  void setFixed(dofComponent d, bool fixed = true) { fixed ? setDisplacement(d) : clearDisplacement(d); }
  void setFixedAll(bool fixed = true) { fixed ? setDisplacementAll() : clearDisplacementAll(); }
  void setDisplacement(dofComponent d, double displacement = 0.0);
  void setDisplacementAll(const Vec3D<double>& translation = Vec3D<double>(0, 0, 0),
                          const Vec3D<double>& rotation = Vec3D<double>(0, 0, 0));
  void clearDisplacement(dofComponent d);
  void clearDisplacementAll();

  Vec3D<float> force() const { return extForce; }
  Vec3D<float> moment() const { return extMoment; }
  void setForce(const float fx, const float fy, const float fz) { extForce = Vec3D<float>(fx, fy, fz); touch(); }
  void setForce(const Vec3D<float>& f) { extForce = f; touch(); }
  void setMoment(const float mx, const float my, const float mz) { extMoment = Vec3D<float>(mx, my, mz); touch(); }
  void setMoment(const Vec3D<float>& m) { extMoment = m; touch(); }
  void addForce(const float fx, const float fy, const float fz) { extForce += Vec3D<float>(fx, fy, fz); touch(); }
  void addForce(const Vec3D<float>& f) { extForce += f; touch(); }
  void addMoment(const float mx, const float my, const float mz) { extMoment += Vec3D<float>(mx, my, mz); touch(); }
  void addMoment(const Vec3D<float>& m) { extMoment += m; touch(); }
  void clearForce() { extForce = Vec3D<float>(); touch(); }
  void clearMoment() { extMoment = Vec3D<float>(); touch(); }

 private:
  dofObject dofFixed;
  Vec3D<float> extForce, extMoment;
  Vec3D<double> extTranslation, extRotation;
  Quat3D<double> extRotationQ;  // cached like the reference's _extRotationQ
  bool hasRotQ;
  CVoxelyze* owner = nullptr;
  void rotationChanged();
  void touch();
  friend class CVoxelyze;
  friend class CVX_Voxel;
};

#endif
