// CVX_MaterialLink: the series combination of two voxel materials and its beam constants (same
// interface as the reference's include/VX_MaterialLink.h:20-47).
#ifndef VX_GB300_MATERIALLINK_H
#define VX_GB300_MATERIALLINK_H

#include "VX_MaterialVoxel.h"

class CVX_MaterialLink : public CVX_MaterialVoxel {
 public:
  CVX_MaterialLink(CVX_MaterialVoxel* mat1, CVX_MaterialVoxel* mat2);
  CVX_MaterialLink(const CVX_MaterialLink& VIn) : CVX_MaterialVoxel() { *this = VIn; }
  virtual CVX_MaterialLink& operator=(const CVX_MaterialLink& VIn);

 protected:
  virtual bool updateAll();
  virtual bool updateDerived();

  CVX_MaterialVoxel* vox1Mat;
  CVX_MaterialVoxel* vox2Mat;
  float _a1, _a2, _b1, _b2, _b3;
  float _sqA1, _sqA2xIp, _sqB1, _sqB2xFMp, _sqB3xIp;

  friend class CVoxelyze;
  friend class CVX_Link;
};

#endif
