// CVoxelyze: the drop-in simulation object (same public interface as the reference's
// include/Voxelyze.h:45-134).  Scene building runs on the host in the reference's voxel and link
// order; doTimeStep runs on the GPU through the vxg engine (include/vxg.h).  Not thread-safe, like
// the reference.  *.vxl.json scene files are read and written in the reference's format (without
// its rapidjson dependency); the PARDISO linear solve of the reference is not provided.
#ifndef VX_GB300_VOXELYZE_H
#define VX_GB300_VOXELYZE_H

#include <list>
#include <string>
#include <vector>

#include "VX_Collision.h"
#include "VX_External.h"
#include "VX_Link.h"
#include "VX_Material.h"
#include "VX_MaterialLink.h"
#include "VX_MaterialVoxel.h"
#include "VX_Voxel.h"

#define DEFAULT_VOXEL_SIZE 0.001

struct VxImpl;

class CVoxelyze {
 public:
  enum stateInfoType { DISPLACEMENT, VELOCITY, KINETIC_ENERGY, ANGULAR_DISPLACEMENT, ANGULAR_VELOCITY,
                       ENG_STRESS, ENG_STRAIN, STRAIN_ENERGY, PRESSURE, MASS };
  enum valueType { MIN, MAX, TOTAL, AVERAGE };
  // GPU arithmetic of the time step (extension of the reference API)
  enum precisionMode { PRECISION_FP64 = 0, PRECISION_FP32C = 1 };

  CVoxelyze(double voxelSize = DEFAULT_VOXEL_SIZE);
  CVoxelyze(const char* jsonFilePath);  // Voxelyze.h:70
  ~CVoxelyze();
  CVoxelyze(CVoxelyze& VIn);
  CVoxelyze& operator=(CVoxelyze& VIn);

  void clear();
  // *.vxl.json scene files (Voxelyze.cpp:61-241): the scene's voxel size, materials, voxels and
  // externals; the state is not saved
  bool loadJSON(const char* jsonFilePath);
  bool saveJSON(const char* jsonFilePath);

  bool doTimeStep(float dt = -1.0f);
  float recommendedTimeStep() const;
  void resetTime();

  CVX_Material* addMaterial(float youngsModulus = 1e6f, float density = 1e3f);
  CVX_Material* addMaterial(const CVX_Material& mat);
  bool removeMaterial(CVX_Material* toRemove);
  bool replaceMaterial(CVX_Material* replaceMe, CVX_Material* replaceWith);
  int materialCount() { return (int)voxelMats.size(); }
  CVX_Material* material(int materialIndex) { return (CVX_Material*)voxelMats[materialIndex]; }

  CVX_Voxel* setVoxel(CVX_Material* material, int xIndex, int yIndex, int zIndex);
  CVX_Voxel* voxel(int xIndex, int yIndex, int zIndex) const;
  int voxelCount() const { return (int)voxelsList.size(); }
  CVX_Voxel* voxel(int voxelIndex) const { return voxelsList[voxelIndex]; }
  const std::vector<CVX_Voxel*>* voxelList() const { return &voxelsList; }

  int indexMinX() const;
  int indexMaxX() const;
  int indexMinY() const;
  int indexMaxY() const;
  int indexMinZ() const;
  int indexMaxZ() const;

  CVX_Link* link(int xIndex, int yIndex, int zIndex, CVX_Voxel::linkDirection direction) const;
  int linkCount() const { return (int)linksList.size(); }
  CVX_Link* link(int linkIndex) { return linksList[linkIndex]; }
  const std::vector<CVX_Link*>* linkList() const { return &linksList; }

  const std::vector<CVX_Collision*>* collisionList() const;

  void setVoxelSize(double voxelSize);
  double voxelSize() const { return voxSize; }

  void setAmbientTemperature(float relativeTemperature, bool allVoxels = false);
  float ambientTemperature(void) const { return ambientTemp; }
  void setGravity(float g = 1.0f);
  float gravity(void) const { return grav; }
  void enableFloor(bool enabled = true);
  bool isFloorEnabled(void) const { return floor; }
  void enableCollisions(bool enabled = true);
  bool isCollisionsEnabled(void) const { return collisions; }

  float stateInfo(stateInfoType info, valueType type);

  // ---- extensions of the reference API -------------------------------------------------
  float currentTime() const;
  // FP64 (bit-faithful, default) or FP32C; takes effect at the next doTimeStep
  void setPrecision(precisionMode mode);
  precisionMode precision() const;
  // runs n steps in one GPU batch; returns the number completed (< n only on divergence)
  int doTimeSteps(int n, float dt = -1.0f);
  // bulk host<->device transfers of the GPU state (component-major, see include/vxg.h)
  bool readField(int vxgField, void* host, long long count);
  // per-voxel temperatures for every voxel at once (setTemperature on each voxel)
  bool setTemperatures(const float* temperatures);
  // stateInfo computed by a GPU reduction (MIN/MAX exact, TOTAL/AVERAGE accumulated in double)
  float stateInfoDevice(stateInfoType info, valueType type);
  const char* lastError() const;
  // creates the GPU engine if needed and uploads every pending host-side change now
  bool upload();
  VxImpl* impl() { return pimpl; }

 private:
  double voxSize;
  float ambientTemp;
  float grav;
  bool floor, collisions;
  float boundingRadius, watchDistance;

  std::vector<CVX_MaterialVoxel*> voxelMats;
  std::list<CVX_MaterialLink*> linkMats;
  std::vector<CVX_Voxel*> voxelsList;
  std::vector<CVX_Link*> linksList;
  mutable std::vector<CVX_Collision*> collisionsList;
  VxImpl* pimpl;

  bool exists(const CVX_MaterialVoxel* m);
  CVX_MaterialLink* combinedMaterial(CVX_MaterialVoxel* mat1, CVX_MaterialVoxel* mat2);
  CVX_Voxel* addVoxel(CVX_MaterialVoxel* m, int x, int y, int z);
  void removeVoxel(int x, int y, int z);
  void replaceVoxel(CVX_MaterialVoxel* m, int x, int y, int z);
  CVX_Link* addLink(int x, int y, int z, CVX_Voxel::linkDirection d);
  void removeLink(int x, int y, int z, CVX_Voxel::linkDirection d);
  bool readJSON(const void* documentRoot);  // a parsed vxjson::Value (vx_json.h)
  std::string writeJSON();

  // host mirror synchronisation
  void syncDown() const;       // device -> host mirror if the device is ahead
  void markState() const;      // host mirror edited: upload before the next step
  void markTables();           // materials or externals changed
  void markExternals();        // an existing external changed
  bool pushPending() const;    // queued per-voxel temperatures -> device
  void markTopology();         // voxel or link added/removed
  bool flush();                // upload whatever is stale

  friend class CVX_Voxel;
  friend class CVX_Link;
  friend class CVX_External;
  friend class CVX_Material;
  friend struct VxImpl;
};

#endif
