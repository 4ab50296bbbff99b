// CVX_Material: material model of the drop-in API (same public interface as the reference's
// include/VX_Material.h:32-160).  Derived constants are computed on the host with the reference's
// float/double promotions (src/VX_Material.cpp) and uploaded to the GPU as a small table.
// The JSON read/write members of the reference are not part of this library.
#ifndef VX_GB300_MATERIAL_H
#define VX_GB300_MATERIAL_H

#include <string>
#include <vector>

#include "Vec3D.h"

class CVoxelyze;

class CVX_Material {
 public:
  CVX_Material(float youngsModulus = 1e6f, float density = 1e3f);
  virtual ~CVX_Material() {}
  CVX_Material(const CVX_Material& vIn) { *this = vIn; }
  virtual CVX_Material& operator=(const CVX_Material& vIn);

  void clear();
  const char* lastError() const { return error.c_str(); }
  void setName(const char* name) { myName = std::string(name); }
  const char* name() const { return myName.c_str(); }

  float stress(float strain, float transverseStrainSum = 0.0f, bool forceLinear = false);
  float modulus(float strain);
  bool isYielded(float strain) { return epsilonYield != -1.0f && strain > epsilonYield; }
  bool isFailed(float strain) { return epsilonFail != -1.0f && strain > epsilonFail; }

  void setColor(int red, int green, int blue, int alpha = 255);
  void setRed(int red);
  void setGreen(int green);
  void setBlue(int blue);
  void setAlpha(int alpha);
  int red() const { return r; }
  int green() const { return g; }
  int blue() const { return b; }
  int alpha() const { return a; }

  bool setModel(int dataPointCount, float* pStrainValues, float* pStressValues);
  bool setModelLinear(float youngsModulus, float failureStress = -1);
  bool setModelBilinear(float youngsModulus, float plasticModulus, float yieldStress, float failureStress = -1);
  bool isModelLinear() const { return linear; }

  float youngsModulus() const { return E; }
  float yieldStress() const { return sigmaYield; }
  float failureStress() const { return sigmaFail; }
  int modelDataPoints() const { return (int)strainData.size(); }
  const float* modelDataStrain() const { return &strainData[0]; }
  const float* modelDataStress() const { return &stressData[0]; }

  void setPoissonsRatio(float poissonsRatio);
  float poissonsRatio() const { return nu; }
  float bulkModulus() const { return E / (3 * (1 - 2 * nu)); }
  float lamesFirstParameter() const { return (E * nu) / ((1 + nu) * (1 - 2 * nu)); }
  float shearModulus() const { return E / (2 * (1 + nu)); }
  bool isXyzIndependent() const { return nu == 0.0f; }

  void setDensity(float density);
  float density() const { return rho; }
  void setStaticFriction(float staticFrictionCoefficient);
  float staticFriction() const { return muStatic; }
  void setKineticFriction(float kineticFrictionCoefficient);
  float kineticFriction() const { return muKinetic; }

  void setInternalDamping(float zeta);
  float internalDamping() const { return zetaInternal; }
  void setGlobalDamping(float zeta);
  float globalDamping() const { return zetaGlobal; }
  void setCollisionDamping(float zeta);
  float collisionDamping() const { return zetaCollision; }

  void setExternalScaleFactor(Vec3D<double> factor);
  void setExternalScaleFactor(double factor) { setExternalScaleFactor(Vec3D<double>(factor, factor, factor)); }
  Vec3D<double> externalScaleFactor() { return extScale; }

  void setCte(float cte) { alphaCTE = cte; touch(); }
  float cte() const { return alphaCTE; }

 protected:
  std::string error;
  std::string myName;
  int r, g, b, a;
  bool linear;
  float E, sigmaYield, sigmaFail, epsilonYield, epsilonFail;
  std::vector<float> strainData, stressData;
  float nu, rho, alphaCTE, muStatic, muKinetic, zetaInternal, zetaGlobal, zetaCollision;
  Vec3D<double> extScale;

  virtual bool updateAll() { return false; }
  virtual bool updateDerived();
  float _eHat;

  bool setYieldFromData(float percentStrainOffset = 0.2);
  float strain(float stress);
  std::vector<CVX_Material*> dependentMaterials;

  CVoxelyze* owner = nullptr;  // set while the material belongs to a CVoxelyze
  void touch();

  friend class CVoxelyze;
  friend class CVX_Voxel;
  friend class CVX_Link;
};

#endif
