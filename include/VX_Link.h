// CVX_Link: a beam element between two adjacent voxels (same public interface as the reference's
// include/VX_Link.h:33-107).  The link's state lives on the GPU; accessors read the owning
// CVoxelyze's host mirror, refreshed from the device on demand.
#ifndef VX_GB300_LINK_H
#define VX_GB300_LINK_H

#include "Quat3D.h"
#include "Vec3D.h"

class CVX_Voxel;
class CVX_MaterialLink;
class CVoxelyze;

class CVX_Link {
 public:
  enum linkAxis { X_AXIS = 0, Y_AXIS = 1, Z_AXIS = 2 };

  CVX_Voxel* voxel(bool positiveEnd) const { return positiveEnd ? pVPos : pVNeg; }
  Vec3D<> force(bool positiveEnd) const;
  Vec3D<> moment(bool positiveEnd) const;

  float axialStrain() const;
  float axialStrain(bool positiveEnd) const;
  float axialStress() const;

  bool isSmallAngle() const;
  bool isYielded() const;
  bool isFailed() const;

  float strainEnergy() const;
  float axialStiffness();

  void updateRestLength();
  void updateTransverseInfo();

  linkAxis axis() const { return ax; }
  int index() const { return idx; }

 private:
  CVX_Link(CVoxelyze* owner, CVX_Voxel* voxel1, CVX_Voxel* voxel2, CVX_MaterialLink* material);
  ~CVX_Link() {}
  void reset();

  CVoxelyze* vx;
  int idx;
  CVX_Voxel* pVNeg;
  CVX_Voxel* pVPos;
  linkAxis ax;
  CVX_MaterialLink* mat;

  friend class CVoxelyze;
  friend class CVX_Voxel;
};

#endif
