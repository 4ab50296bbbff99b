// CVX_Voxel: one voxel of a CVoxelyze (same public interface as the reference's
// include/VX_Voxel.h:35-137).  Dynamic state (position, momenta, orientation, temperature...) lives
// on the GPU; accessors read the owning CVoxelyze's host mirror, which is refreshed from the device
// on the first read after a time step.
#ifndef VX_GB300_VOXEL_H
#define VX_GB300_VOXEL_H

#include "Quat3D.h"
#include "VX_External.h"
#include "VX_Link.h"
#include "VX_MaterialVoxel.h"
#include "Vec3D.h"

class CVoxelyze;

class CVX_Voxel {
 public:
  enum linkDirection { X_POS = 0, X_NEG = 1, Y_POS = 2, Y_NEG = 3, Z_POS = 4, Z_NEG = 5 };
  enum voxelCorner { NNN = 0, NNP = 1, NPN = 2, NPP = 3, PNN = 4, PNP = 5, PPN = 6, PPP = 7 };

  CVX_Link* link(linkDirection direction) const { return links[direction]; }
  int linkCount() const { int n = 0; for (int i = 0; i < 6; i++) if (links[i]) n++; return n; }
  CVX_Voxel* adjacentVoxel(linkDirection direction) const;
  short indexX() { return ix; }
  short indexY() { return iy; }
  short indexZ() { return iz; }

  CVX_MaterialVoxel* material() { return mat; }
  bool externalExists() { return ext ? true : false; }
  CVX_External* external();

  Vec3D<double> position() const;
  Vec3D<double> originalPosition() const { double s = mat->nominalSize(); return Vec3D<double>(ix * s, iy * s, iz * s); }
  Vec3D<double> displacement() const { return position() - originalPosition(); }
  Vec3D<float> size() const { return cornerOffset(PPP) - cornerOffset(NNN); }
  Vec3D<float> cornerPosition(voxelCorner corner) const;
  Vec3D<float> cornerOffset(voxelCorner corner) const;
  bool isInterior() const;
  bool isSurface() const { return !isInterior(); }

  Vec3D<double> baseSize() const;
  double baseSize(CVX_Link::linkAxis axis) const;
  double baseSizeAverage() const { Vec3D<double> b = baseSize(); return (b.x + b.y + b.z) / 3.0f; }

  Quat3D<double> orientation() const;
  float orientationAngle() const { return (float)orientation().Angle(); }
  Vec3D<double> orientationAxis() const { return orientation().Axis(); }

  float displacementMagnitude() const { return (float)displacement().Length(); }
  float angularDisplacementMagnitude() const { return (float)orientation().Angle(); }
  Vec3D<double> velocity() const;
  float velocityMagnitude() const;
  Vec3D<double> angularVelocity() const;
  float angularVelocityMagnitude() const;
  float kineticEnergy() const;
  float volumetricStrain() const;
  float pressure() const;

  bool isYielded() const;
  bool isFailed() const;

  float temperature();
  void setTemperature(float temperature);

  Vec3D<float> externalForce();
  Vec3D<float> externalMoment();
  void haltMotion();

  void enableFloor(bool enabled);
  bool isFloorEnabled() const;
  bool isFloorStaticFriction() const;
  float floorPenetration() const;

  Vec3D<double> force();
  Vec3D<double> moment();

  float transverseArea(CVX_Link::linkAxis axis);
  float transverseStrainSum(CVX_Link::linkAxis axis);
  float dampingMultiplier();

  static inline CVX_Link::linkAxis toAxis(linkDirection d) { return (CVX_Link::linkAxis)((int)d / 2); }
  static inline linkDirection toDirection(CVX_Link::linkAxis axis, bool positiveDirection) {
    return (linkDirection)(2 * ((int)axis) + (positiveDirection ? 0 : 1));
  }
  static inline bool isNegative(linkDirection d) { return d % 2 == 1; }
  static inline bool isPositive(linkDirection d) { return d % 2 == 0; }
  static inline linkDirection toOpposite(linkDirection d) { return (linkDirection)(d - d % 2 + (d + 1) % 2); }

  int index() const { return idx; }

 private:
  CVX_Voxel(CVoxelyze* owner, CVX_MaterialVoxel* material, short indexX, short indexY, short indexZ);
  ~CVX_Voxel();

  CVoxelyze* vx;
  int idx;
  CVX_MaterialVoxel* mat;
  short ix, iy, iz;
  CVX_External* ext;
  CVX_Link* links[6];

  Vec3D<float> strain(bool poissonsStrain) const;
  Vec3D<float> poissonsStrain();  // cached Poisson strain, filled on first use after a step

  friend class CVoxelyze;
  friend class CVX_Link;
};

#endif
