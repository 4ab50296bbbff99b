// CVX_MaterialVoxel: a material at a given voxel size, with mass, inertia and damping constants
// (same interface as the reference's include/VX_MaterialVoxel.h:22-72).
#ifndef VX_GB300_MATERIALVOXEL_H
#define VX_GB300_MATERIALVOXEL_H

#include "VX_Material.h"

class CVX_MaterialVoxel : public CVX_Material {
 public:
  CVX_MaterialVoxel(float youngsModulus = 1e6f, float density = 1e3f, double nominalSize = 0.001);
  CVX_MaterialVoxel(const CVX_Material& mat, double nominalSize = 0.001);
  CVX_MaterialVoxel(const CVX_MaterialVoxel& vIn) { *this = vIn; }
  virtual CVX_MaterialVoxel& operator=(const CVX_MaterialVoxel& vIn);

  bool setNominalSize(double size);
  double nominalSize() { return nomSize; }
  Vec3D<double> size() { return nomSize * extScale; }

  float mass() { return _mass; }
  float momentInertia() { return _momentInertia; }

  float internalDampingTranslateC() const { return zetaInternal * _2xSqMxExS; }
  float internalDampingRotateC() const { return zetaInternal * _2xSqIxExSxSxS; }
  float globalDampingTranslateC() const { return zetaGlobal * _2xSqMxExS; }
  float globalDampingRotateC() const { return zetaGlobal * _2xSqIxExSxSxS; }
  float collisionDampingTranslateC() const { return zetaCollision * _2xSqMxExS; }
  float collisionDampingRotateC() const { return zetaCollision * _2xSqIxExSxSxS; }

  float penetrationStiffness() const { return (float)(2 * E * nomSize); }

 protected:
  void initialize(double nominalSize);
  void setGravityMultiplier(float gravityMultiplier) { gravMult = gravityMultiplier; }
  float gravityMuliplier() { return gravMult; }
  float gravityForce() { return -_mass * 9.80665f * gravMult; }

  virtual bool updateAll() { return false; }
  virtual bool updateDerived();

  double nomSize;
  float gravMult;
  float _mass, _massInverse, _sqrtMass, _firstMoment, _momentInertia, _momentInertiaInverse;
  float _2xSqMxExS, _2xSqIxExSxSxS;

  friend class CVoxelyze;
  friend class CVX_Voxel;
  friend class CVX_MaterialLink;
};

#endif
