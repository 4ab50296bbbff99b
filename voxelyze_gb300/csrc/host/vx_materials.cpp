// Materials and externals of the drop-in API: CVX_Material, CVX_MaterialVoxel, CVX_MaterialLink
// and CVX_External.  Every derived constant is computed with the reference's float/double
// promotions, expression by expression, because the GPU path is bit-faithful to them:
//   CVX_Material       src/VX_Material.cpp:15-532
//   CVX_MaterialVoxel  src/VX_MaterialVoxel.cpp:16-86
//   CVX_MaterialLink   src/VX_MaterialLink.cpp:16-141
//   CVX_External       src/VX_External.cpp:14-109
#include <cfloat>
#include <cmath>

#include "Voxelyze.h"
#include "vx_host.h"

// ---------------------------------------------------------------------------------------------
CVX_Material::CVX_Material(float youngsModulus, float density) {
  clear();
  rho = density;
  setModelLinear(youngsModulus);
  updateDerived();
}

CVX_Material& CVX_Material::operator=(const CVX_Material& v) {
  error = v.error;
  myName = v.myName;
  r = v.r; g = v.g; b = v.b; a = v.a;
  linear = v.linear;
  E = v.E;
  sigmaYield = v.sigmaYield;
  sigmaFail = v.sigmaFail;
  epsilonYield = v.epsilonYield;
  epsilonFail = v.epsilonFail;
  strainData = v.strainData;
  stressData = v.stressData;
  nu = v.nu;
  rho = v.rho;
  alphaCTE = v.alphaCTE;
  muStatic = v.muStatic;
  muKinetic = v.muKinetic;
  zetaInternal = v.zetaInternal;
  zetaGlobal = v.zetaGlobal;
  zetaCollision = v.zetaCollision;
  _eHat = v._eHat;
  touch();
  return *this;
}

void CVX_Material::clear() {
  r = g = b = a = -1;
  nu = 0.0f;
  rho = 1.0f;
  alphaCTE = 0.0f;
  muStatic = muKinetic = 0.0f;
  zetaInternal = 1.0f;
  zetaGlobal = 0.0f;
  zetaCollision = 0.0f;
  extScale = Vec3D<>(1.0, 1.0, 1.0);
  setModelLinear(1.0);
  updateDerived();
}

void CVX_Material::touch() {
  if (owner) owner->markTables();
}

float CVX_Material::stress(float strain, float tss, bool forceLinear) {
  if (isFailed(strain)) return 0.0f;
  if (strain <= strainData[1] || linear || forceLinear) {
    if (nu == 0.0f) return E * strain;
    return _eHat * ((1 - nu) * strain + nu * tss);
  }
  int n = modelDataPoints();
  for (int i = 2; i < n; i++) {
    if (strain <= strainData[i] || i == n - 1) {
      float perc = (strain - strainData[i - 1]) / (strainData[i] - strainData[i - 1]);
      float basic = stressData[i - 1] + perc * (stressData[i] - stressData[i - 1]);
      if (nu == 0.0f) return basic;
      float mod = (stressData[i] - stressData[i - 1]) / (strainData[i] - strainData[i - 1]);
      float modHat = mod / ((1 - 2 * nu) * (1 + nu));
      float effStrain = basic / mod;
      float effTss = tss * (effStrain / strain);
      return modHat * ((1 - nu) * effStrain + nu * effTss);
    }
  }
  return 0.0f;
}

float CVX_Material::strain(float s) {
  if (s <= stressData[1] || linear) return s / E;
  int n = modelDataPoints();
  for (int i = 2; i < n; i++)
    if (s <= stressData[i] || i == n - 1) {
      float perc = (s - stressData[i - 1]) / (stressData[i] - stressData[i - 1]);
      return strainData[i - 1] + perc * (strainData[i] - strainData[i - 1]);
    }
  return 0.0f;
}

float CVX_Material::modulus(float s) {
  if (isFailed(s)) return 0.0f;
  if (s <= strainData[1] || linear) return E;
  int n = modelDataPoints();
  for (int i = 2; i < n; i++)
    if (s <= strainData[i] || i == n - 1) return (stressData[i] - stressData[i - 1]) / (strainData[i] - strainData[i - 1]);
  return 0.0f;
}

static int clamp255(int v) { return v > 255 ? 255 : (v < 0 ? 0 : v); }
void CVX_Material::setColor(int red, int green, int blue, int alpha) {
  setRed(red); setGreen(green); setBlue(blue); setAlpha(alpha);
}
void CVX_Material::setRed(int v) { r = clamp255(v); }
void CVX_Material::setGreen(int v) { g = clamp255(v); }
void CVX_Material::setBlue(int v) { b = clamp255(v); }
void CVX_Material::setAlpha(int v) { a = clamp255(v); }

bool CVX_Material::setModel(int n, float* strainV, float* stressV) {
  if (*strainV == 0 && *stressV == 0) { strainV++; stressV++; n--; }
  if (n <= 0) { error = "Not enough data points"; return false; }
  if (*strainV <= 0 || *stressV <= 0) { error = "First stress and strain data points negative or zero"; return false; }
  std::vector<float> ts{0.0f}, tt{0.0f};
  float sw = 0.0f, ss = 0.0f;
  for (int i = 0; i < n; i++) {
    float a1 = strainV[i], b1 = stressV[i];
    if (a1 <= sw) { error = "Out of order strain data"; return false; }
    if (b1 <= ss) error = "Stress data is not monotonically increasing";
    if (i > 0 && (b1 - ss) / (a1 - sw) > tt[0] / ts[0]) {
      error = "Slope of stress/strain curve should never exceed that of the first line segment (youngs modulus)";
      return false;
    }
    sw = a1;
    ss = b1;
    ts.push_back(a1);
    tt.push_back(b1);
  }
  strainData = ts;
  stressData = tt;
  E = stressData[1] / strainData[1];
  sigmaFail = stressData.back();
  epsilonFail = strainData.back();
  linear = (n == 1);
  if (n == 1 || n == 2) {
    sigmaYield = stressData[1];
    epsilonYield = strainData[1];
  } else {
    setYieldFromData();
  }
  return updateDerived();
}

bool CVX_Material::setModelLinear(float youngs, float fail) {
  if (youngs <= 0) { error = "Young's modulus must be positive"; return false; }
  if (fail != -1.0f && fail <= 0) { error = "Failure stress must be positive"; return false; }
  float tf = fail;
  if (tf == -1) tf = 1000000;
  float tfs = tf / youngs;
  strainData.assign({0.0f, tfs});
  stressData.assign({0.0f, tf});
  linear = true;
  E = youngs;
  sigmaYield = fail;
  sigmaFail = fail;
  epsilonYield = (fail == -1) ? -1 : tfs;
  epsilonFail = (fail == -1) ? -1 : tfs;
  return updateDerived();
}

bool CVX_Material::setModelBilinear(float youngs, float plastic, float yieldS, float fail) {
  if (youngs <= 0) { error = "Young's modulus must be positive"; return false; }
  if (plastic <= 0 || plastic >= youngs) { error = "Plastic modulus must be positive but less than Young's modulus"; return false; }
  if (yieldS <= 0) { error = "Yield stress must be positive"; return false; }
  if (fail != -1.0f && fail <= yieldS) { error = "Failure stress must be positive and greater than the yield stress"; return false; }
  float ys = yieldS / youngs;
  float tf = fail;
  if (tf == -1) tf = 3 * yieldS;
  float tM = plastic;
  float tB = yieldS - tM * ys;
  float tfs = (tf - tB) / tM;
  strainData.assign({0.0f, ys, tfs});
  stressData.assign({0.0f, yieldS, tf});
  linear = false;
  E = youngs;
  sigmaYield = yieldS;
  sigmaFail = fail;
  epsilonYield = ys;
  epsilonFail = fail == -1.0f ? -1.0f : tfs;
  return updateDerived();
}

bool CVX_Material::setYieldFromData(float pct) {
  sigmaYield = -1.0f;
  epsilonYield = -1.0f;
  float oM = E;
  float oB = (-pct / 100 * oM);
  int pts = (int)strainData.size() - 1;
  for (int i = 1; i < pts - 1; i++) {
    float x1 = strainData[i], x2 = strainData[i + 1], y1 = stressData[i], y2 = stressData[i + 1];
    float tM = (y2 - y1) / (x2 - x1);
    float tB = y1 - tM * x1;
    if (oM != tM) {
      float xi = (tB - oB) / (oM - tM);
      if (xi > x1 && xi < x2) {
        float p = (xi - x1) / (x2 - x1);
        sigmaYield = y1 + p * (y2 - y1);
        epsilonYield = xi;
        return true;
      }
    }
  }
  sigmaYield = sigmaFail;
  epsilonYield = epsilonFail;
  return false;
}

void CVX_Material::setPoissonsRatio(float v) {
  if (v < 0) v = 0;
  if (v >= 0.5) v = 0.5 - FLT_EPSILON * 2;
  nu = v;
  updateDerived();
}
void CVX_Material::setDensity(float d) {
  if (d <= 0) d = FLT_MIN;
  rho = d;
  updateDerived();
}
void CVX_Material::setStaticFriction(float v) { muStatic = v <= 0 ? 0 : v; touch(); }
void CVX_Material::setKineticFriction(float v) { muKinetic = v <= 0 ? 0 : v; touch(); }
void CVX_Material::setInternalDamping(float v) { zetaInternal = v <= 0 ? 0 : v; touch(); }
void CVX_Material::setGlobalDamping(float v) { zetaGlobal = v <= 0 ? 0 : v; touch(); }
void CVX_Material::setCollisionDamping(float v) { zetaCollision = v <= 0 ? 0 : v; touch(); }
void CVX_Material::setExternalScaleFactor(Vec3D<double> f) {
  if (f.x <= 0) f.x = FLT_MIN;
  if (f.y <= 0) f.y = FLT_MIN;
  if (f.z <= 0) f.z = FLT_MIN;
  extScale = f;
  touch();
}

bool CVX_Material::updateDerived() {
  _eHat = E / ((1 - 2 * nu) * (1 + nu));
  for (CVX_Material* d : dependentMaterials) d->updateAll();
  touch();
  return true;
}

// ---------------------------------------------------------------------------------------------
CVX_MaterialVoxel::CVX_MaterialVoxel(float youngs, float density, double nominalSize) : CVX_Material(youngs, density) {
  initialize(nominalSize);
}
CVX_MaterialVoxel::CVX_MaterialVoxel(const CVX_Material& m, double nominalSize) : CVX_Material(m) {
  initialize(nominalSize);
}
void CVX_MaterialVoxel::initialize(double nominalSize) {
  nomSize = nominalSize;
  gravMult = 0.0f;
  updateDerived();
}
CVX_MaterialVoxel& CVX_MaterialVoxel::operator=(const CVX_MaterialVoxel& v) {
  CVX_Material::operator=(v);
  nomSize = v.nomSize;
  gravMult = v.gravMult;
  _eHat = v._eHat;
  _mass = v._mass;
  _massInverse = v._massInverse;
  _sqrtMass = v._sqrtMass;
  _firstMoment = v._firstMoment;
  _momentInertia = v._momentInertia;
  _momentInertiaInverse = v._momentInertiaInverse;
  _2xSqMxExS = v._2xSqMxExS;
  _2xSqIxExSxSxS = v._2xSqIxExSxSxS;
  return *this;
}
bool CVX_MaterialVoxel::updateDerived() {
  CVX_Material::updateDerived();
  double volume = nomSize * nomSize * nomSize;
  _mass = (float)(volume * rho);
  _momentInertia = (float)(_mass * nomSize * nomSize / 6.0f);
  _firstMoment = (float)(_mass * nomSize / 2.0f);
  if (volume == 0 || _mass == 0 || _momentInertia == 0) {
    _massInverse = _sqrtMass = _momentInertiaInverse = _2xSqMxExS = _2xSqIxExSxSxS = 0.0f;
    return false;
  }
  _massInverse = 1.0f / _mass;
  _sqrtMass = std::sqrt(_mass);
  _momentInertiaInverse = 1.0f / _momentInertia;
  _2xSqMxExS = (float)(2.0f * std::sqrt(_mass * E * nomSize));
  _2xSqIxExSxSxS = (float)(2.0f * std::sqrt(_momentInertia * E * nomSize * nomSize * nomSize));
  return true;
}
bool CVX_MaterialVoxel::setNominalSize(double size) {
  if (size <= 0) size = FLT_MIN;
  nomSize = size;
  return updateDerived();
}

// ---------------------------------------------------------------------------------------------
CVX_MaterialLink::CVX_MaterialLink(CVX_MaterialVoxel* m1, CVX_MaterialVoxel* m2) {
  vox1Mat = m1;
  vox2Mat = m2;
  updateAll();
}
CVX_MaterialLink& CVX_MaterialLink::operator=(const CVX_MaterialLink& v) {
  CVX_MaterialVoxel::operator=(v);
  vox1Mat = v.vox1Mat;
  vox2Mat = v.vox2Mat;
  _a1 = v._a1; _a2 = v._a2; _b1 = v._b1; _b2 = v._b2; _b3 = v._b3;
  _sqA1 = v._sqA1; _sqA2xIp = v._sqA2xIp; _sqB1 = v._sqB1; _sqB2xFMp = v._sqB2xFMp; _sqB3xIp = v._sqB3xIp;
  return *this;
}
bool CVX_MaterialLink::updateAll() {
  const CVX_MaterialVoxel& A = *vox1Mat;
  const CVX_MaterialVoxel& B = *vox2Mat;
  nomSize = 0.5 * (A.nomSize + B.nomSize);
  r = (int)(0.5 * (A.r + B.r));
  g = (int)(0.5 * (A.g + B.g));
  b = (int)(0.5 * (A.b + B.b));
  a = (int)(0.5 * (A.a + B.a));
  rho = 0.5f * (A.rho + B.rho);
  alphaCTE = 0.5f * (A.alphaCTE + B.alphaCTE);
  muStatic = 0.5f * (A.muStatic + B.muStatic);
  muKinetic = 0.5f * (A.muKinetic + B.muKinetic);
  zetaInternal = 0.5f * (A.zetaInternal + B.zetaInternal);
  zetaGlobal = 0.5f * (A.zetaGlobal + B.zetaGlobal);
  zetaCollision = 0.5f * (A.zetaCollision + B.zetaCollision);
  extScale = Vec3D<>(1.0, 1.0, 1.0);
  float f1 = A.sigmaFail, f2 = B.sigmaFail, sf;
  if (f1 == -1.0f) sf = f2;
  else if (f2 == -1.0f) sf = f1;
  else sf = f1 < f2 ? f1 : f2;
  if (A.linear && B.linear) {
    setModelLinear(2.0f * A.E * B.E / (A.E + B.E), sf);
  } else {
    // springs in series over the union of both models' strain points
    CVX_MaterialVoxel& AA = *vox1Mat;
    CVX_MaterialVoxel& BB = *vox2Mat;
    std::vector<float> ns{0.0f}, nt{0.0f};
    size_t i1 = 1, i2 = 1;
    while (i1 < A.strainData.size() && i2 < B.strainData.size()) {
      float s = FLT_MAX;
      if (i1 < A.strainData.size()) s = A.strainData[i1];
      if (i2 < B.strainData.size() && B.strainData[i2] < s) s = B.strainData[i2];
      if (s == A.strainData[i1]) i1++;
      if (s == B.strainData[i2]) i2++;
      float mA = AA.modulus(s - FLT_EPSILON);
      float mB = BB.modulus(s - FLT_EPSILON);
      float mod = 2.0f * mA * mB / (mA + mB);
      size_t last = ns.size() - 1;
      ns.push_back(s);
      nt.push_back(nt[last] + mod * (s - ns[last]));
    }
    setModel((int)ns.size(), ns.data(), nt.data());
    sigmaFail = sf;
    epsilonFail = sf == -1.0f ? -1.0f : strain(sf);
  }
  if (A.nu == 0 && B.nu == 0) {
    nu = 0;
  } else {
    float th = 2 * A._eHat * B._eHat / (A._eHat + B._eHat);
    float te = youngsModulus();
    float c2 = (th - te) / (2 * th) + 0.0625;
    nu = std::sqrt(c2) - 0.25;
  }
  return updateDerived();
}
bool CVX_MaterialLink::updateDerived() {
  CVX_MaterialVoxel::updateDerived();
  float L = (float)nomSize;
  _a1 = E * L;
  _a2 = E * L * L * L / (12.0f * (1 + nu));
  _b1 = E * L;
  _b2 = E * L * L / 2.0f;
  _b3 = E * L * L * L / 6.0f;
  _sqA1 = std::sqrt(_a1);
  _sqA2xIp = std::sqrt(_a2 * L * L / 6.0f);
  _sqB1 = std::sqrt(_b1);
  _sqB2xFMp = std::sqrt(_b2 * L / 2.0f);
  _sqB3xIp = std::sqrt(_b3 * L * L / 6.0f);
  return true;
}

// ---------------------------------------------------------------------------------------------
CVX_External::CVX_External() : hasRotQ(false) { reset(); }
CVX_External& CVX_External::operator=(const CVX_External& e) {
  dofFixed = e.dofFixed;
  extForce = e.extForce;
  extMoment = e.extMoment;
  extTranslation = e.extTranslation;
  extRotation = e.extRotation;
  rotationChanged();
  touch();
  return *this;
}
void CVX_External::touch() {
  if (owner) owner->markExternals();
}
void CVX_External::reset() {
  dofFixed = 0;
  extForce = extMoment = Vec3D<float>();
  extTranslation = Vec3D<double>();
  extRotation = Vec3D<double>();
  rotationChanged();
  touch();
}
void CVX_External::setFixed(bool tx, bool ty, bool tz, bool rx, bool ry, bool rz) {
  dofFixed = dof(tx, ty, tz, rx, ry, rz);
  extTranslation = extRotation = Vec3D<double>();  // the cached quaternion is left as it was
  touch();
}
void CVX_External::setDisplacement(dofComponent d, double v) {
  dofSet(dofFixed, d, true);
  if (v != 0.0f) {
    if (d & X_TRANSLATE) extTranslation.x = v;
    if (d & Y_TRANSLATE) extTranslation.y = v;
    if (d & Z_TRANSLATE) extTranslation.z = v;
    if (d & X_ROTATE) extRotation.x = v;
    if (d & Y_ROTATE) extRotation.y = v;
    if (d & Z_ROTATE) extRotation.z = v;
  }
  rotationChanged();
  touch();
}
void CVX_External::setDisplacementAll(const Vec3D<double>& t, const Vec3D<double>& rr) {
  dofSetAll(dofFixed, true);
  extTranslation = t;
  extRotation = rr;
  rotationChanged();
  touch();
}
void CVX_External::clearDisplacement(dofComponent d) {
  dofSet(dofFixed, d, false);
  if (d & X_TRANSLATE) extTranslation.x = 0.0;
  if (d & Y_TRANSLATE) extTranslation.y = 0.0;
  if (d & Z_TRANSLATE) extTranslation.z = 0.0;
  if (d & X_ROTATE) extRotation.x = 0.0;
  if (d & Y_ROTATE) extRotation.y = 0.0;
  if (d & Z_ROTATE) extRotation.z = 0.0;
  rotationChanged();
  touch();
}
void CVX_External::clearDisplacementAll() {
  dofSetAll(dofFixed, false);
  extTranslation = Vec3D<double>();
  extRotation = Vec3D<double>();
  rotationChanged();
  touch();
}
void CVX_External::rotationChanged() {
  if (extRotation != Vec3D<double>()) {
    extRotationQ = Quat3D<double>(extRotation);
    hasRotQ = true;
  } else if (hasRotQ) {
    extRotationQ = Quat3D<double>();
  }
}

float CVX_Collision::envelopeRadius = 0.625f;
