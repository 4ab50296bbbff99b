// CVX_Collision: a watched voxel pair (same interface as the reference's include/VX_Collision.h:25-45).
// Pairs and contact forces live on the GPU; CVoxelyze::collisionList() materialises these objects
// from the device pair list on demand.
#ifndef VX_GB300_COLLISION_H
#define VX_GB300_COLLISION_H

#include "Vec3D.h"

class CVX_Voxel;

class CVX_Collision {
 public:
  CVX_Collision(CVX_Voxel* v1, CVX_Voxel* v2) : pV1(v1), pV2(v2) {}
  Vec3D<float> const contactForce(CVX_Voxel* pVoxel) {
    if (pVoxel == pV1) return force;
    if (pVoxel == pV2) return -force;
    return Vec3D<float>(0, 0, 0);
  }
  CVX_Voxel* voxel1() const { return pV1; }
  CVX_Voxel* voxel2() const { return pV2; }
  static float envelopeRadius;

 private:
  CVX_Voxel *pV1, *pV2;
  Vec3D<float> force;
  friend class CVoxelyze;
};

#endif
