// ORACLE — test infrastructure, not product code.
//
// A CPU restatement of the reference's time-step path (CVoxelyze::doTimeStep and everything it
// calls), used only as the checker for the GPU path: by tests/, by __graft_entry__.smoke() and by
// bench.py's CPU-baseline leg.  It exposes the vxo_* facade (oracle/facade.h).
//
// Parity pin: its results are compared bit for bit with the reference library compiled from its own
// sources (oracle/_ref, tests/test_oracle_reference.py) and with committed golden vectors
// generated from that build (tests/golden/, tests/golden/make_golden.py).
//
// Every routine cites the reference file:line it restates.  Float/double promotions follow the
// reference expression by expression, because the parity bar is bit-exactness.  Build with
// -ffp-contract=off.  The link and voxel loops can run under OpenMP (the reference's USE_OMP
// parallelisation, Voxelyze.cpp:260-277); the Poisson strain cache is filled by a serial-equivalent
// pre-pass first, so the threaded run gives the same bits as the serial one.
#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <list>
#include <unordered_map>
#include <vector>

#include "facade.h"
// Correctly rounded sin/cos/acos, selectable with vxo_set_math(1).  The GPU path evaluates these
// functions correctly rounded; the C library the reference links is not correctly rounded in about
// 0.1% of calls.  In mode 1 the oracle uses the same correctly rounded values (validated on their
// own against 256-bit arithmetic in tests/test_crmath.py), so GPU parity can be checked bit for bit;
// mode 0 (default) is the faithful restatement of the reference with the C library.
#include "vx_crmath.h"

namespace vxo {

static int g_math_mode = 0;
static inline double m_sin(double x) {
  if (g_math_mode) { int f = 0; return vxm::cr_sin(x, &f); }
  return std::sin(x);
}
static inline double m_cos(double x) {
  if (g_math_mode) { int f = 0; return vxm::cr_cos(x, &f); }
  return std::cos(x);
}
static inline double m_acos(double x) {
  if (g_math_mode) { int f = 0; return vxm::cr_acos(x, &f); }
  return std::acos(x);
}

// ---------------------------------------------------------------------------------------------
// small vector / quaternion helpers (Vec3D.h, Quat3D.h semantics)
struct V3 {
  double x = 0, y = 0, z = 0;
};
struct F3 {
  float x = 0, y = 0, z = 0;
};
struct Q4 {
  double w = 1, x = 0, y = 0, z = 0;
};
static inline V3 v3(double a, double b, double c) { V3 r; r.x = a; r.y = b; r.z = c; return r; }
static inline Q4 q4(double w, double x, double y, double z) { Q4 q; q.w = w; q.x = x; q.y = y; q.z = z; return q; }
static inline double comp(const V3& v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }
static inline float compf(const F3& v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }

// Quat3D::RotateVec3D  Quat3D.h:170-177
static inline V3 rotate(const Q4& q, const V3& f) {
  double tw = f.x * q.x + f.y * q.y + f.z * q.z;
  double tx = f.x * q.w - f.y * q.z + f.z * q.y;
  double ty = f.x * q.z + f.y * q.w - f.z * q.x;
  double tz = -f.x * q.y + f.y * q.x + f.z * q.w;
  return v3(q.w * tx + q.x * tw + q.y * tz - q.z * ty, q.w * ty - q.x * tz + q.y * tw + q.z * tx,
            q.w * tz + q.x * ty - q.y * tx + q.z * tw);
}
// Quat3D::RotateVec3DInv  Quat3D.h:188-195
static inline V3 rotate_inv(const Q4& q, const V3& f) {
  double tw = q.x * f.x + q.y * f.y + q.z * f.z;
  double tx = q.w * f.x - q.y * f.z + q.z * f.y;
  double ty = q.w * f.y + q.x * f.z - q.z * f.x;
  double tz = q.w * f.z - q.x * f.y + q.y * f.x;
  return v3(tw * q.x + tx * q.w + ty * q.z - tz * q.y, tw * q.y - tx * q.z + ty * q.w + tz * q.x,
            tw * q.z + tx * q.y - ty * q.x + tz * q.w);
}
// Quat3D::operator*  Quat3D.h:83
static inline Q4 qmul(const Q4& a, const Q4& f) {
  return q4(a.w * f.w - a.x * f.x - a.y * f.y - a.z * f.z, a.w * f.x + a.x * f.w + a.y * f.z - a.z * f.y,
            a.w * f.y - a.x * f.z + a.y * f.w + a.z * f.x, a.w * f.z + a.x * f.y - a.y * f.x + a.z * f.w);
}
// Quat3D::ToRotationVector  Quat3D.h:117-122
static inline V3 to_rotation_vector(const Q4& q) {
  if (q.w >= 1.0 || q.w <= -1.0) return V3();
  double sl = 1.0 - q.w * q.w;
  if (sl < 2.4e-3) {
    double s = std::sqrt((2 - 2 * q.w) / sl);
    return v3(s * (2.0 * q.x), s * (2.0 * q.y), s * (2.0 * q.z));
  }
  double a = m_acos(q.w);
  double inv = 1.0 / std::sqrt(sl);
  return v3(inv * (a * (2.0 * q.x)), inv * (a * (2.0 * q.y)), inv * (a * (2.0 * q.z)));
}
// Quat3D::FromRotationVector  Quat3D.h:124-139
static inline Q4 from_rotation_vector(const V3& in) {
  V3 th = v3(0.5 * in.x, 0.5 * in.y, 0.5 * in.z);
  double m2 = th.x * th.x + th.y * th.y + th.z * th.z;
  double w, s;
  if (m2 * m2 < 5.328e-15) {
    w = 1.0 - 0.5 * m2;
    s = 1.0 - m2 / 6.0;
  } else {
    double m = std::sqrt(m2);
    w = m_cos(m);
    s = m_sin(m) / m;
  }
  return q4(w, th.x * s, th.y * s, th.z * s);
}
// Quat3D::FromAngleToPosX  Quat3D.h:141-166 (q is left untouched for a zero vector)
static inline void from_angle_to_pos_x(Q4& q, const V3& r) {
  if (r.x == 0 && r.y == 0 && r.z == 0) return;
  double yx = r.y / r.x, zx = r.z / r.x;
  if (yx < 1.732e-2 && yx > -1.732e-2 && zx < 1.732e-2 && zx > -1.732e-2) {
    q.x = 0;
    q.y = 0.5 * zx;
    q.z = -0.5 * yx;
    q.w = 1 + 0.5 * (-q.y * q.y - q.z * q.z);
    return;
  }
  V3 n = r;
  double l = std::sqrt(n.x * n.x + n.y * n.y + n.z * n.z);
  if (l > 0) {
    double li = 1.0 / l;
    n.x *= li; n.y *= li; n.z *= li;
  }
  double theta = m_acos(n.x);
  if (theta > 3.14159265358979 - 1e-7) {
    q = q4(0, 0, 1, 0);
    return;
  }
  double ami = 1.0 / std::sqrt(n.z * n.z + n.y * n.y);
  double a = 0.5 * theta;
  double s = m_sin(a);
  q.w = m_cos(a);
  q.x = 0;
  q.y = n.z * ami * s;
  q.z = -n.y * ami * s;
}

// ---------------------------------------------------------------------------------------------
// materials (VX_Material.cpp, VX_MaterialVoxel.cpp, VX_MaterialLink.cpp)
struct Material {
  bool linear = true;
  float E = 1, sigmaYield = -1, sigmaFail = -1, epsilonYield = -1, epsilonFail = -1;
  std::vector<float> strainData, stressData;
  float nu = 0, rho = 1, alphaCTE = 0, muStatic = 0, muKinetic = 0;
  float zetaInternal = 1, zetaGlobal = 0, zetaCollision = 0;
  float eHat = 1;
  double nomSize = 0.001;
  float gravMult = 0;
  float mass = 0, massInv = 0, sqrtMass = 0, firstMoment = 0, inertia = 0, inertiaInv = 0;
  float c2xSqMxExS = 0, c2xSqIxExSxSxS = 0;
  // link-only constants (VX_MaterialLink.h:29-38)
  float a1 = 0, a2 = 0, b1 = 0, b2 = 0, b3 = 0, sqA1 = 0, sqA2xIp = 0, sqB1 = 0, sqB2xFMp = 0, sqB3xIp = 0;
  bool is_link = false;
  int m1 = -1, m2 = -1;  // constituent voxel materials of a link material

  bool isFailed(float s) const { return epsilonFail != -1.0f && s > epsilonFail; }  // VX_Material.h:49
  bool isYielded(float s) const { return epsilonYield != -1.0f && s > epsilonYield; }

  // CVX_Material::stress  VX_Material.cpp:165-195
  float stress(float strain, float tss = 0.0f, bool forceLinear = false) const {
    if (isFailed(strain)) return 0.0f;
    if (strain <= strainData[1] || linear || forceLinear) {
      if (nu == 0.0f) return E * strain;
      return eHat * ((1 - nu) * strain + nu * tss);
    }
    int n = (int)strainData.size();
    for (int i = 2; i < n; ++i) {
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
  // CVX_Material::strain(stress)  VX_Material.cpp:197-211
  float strain_of(float s) const {
    if (s <= stressData[1] || linear) return s / E;
    int n = (int)stressData.size();
    for (int i = 2; i < n; ++i)
      if (s <= stressData[i] || i == n - 1) {
        float perc = (s - stressData[i - 1]) / (stressData[i] - stressData[i - 1]);
        return strainData[i - 1] + perc * (strainData[i] - strainData[i - 1]);
      }
    return 0.0f;
  }
  // CVX_Material::modulus  VX_Material.cpp:214-226
  float modulus(float s) const {
    if (isFailed(s)) return 0.0f;
    if (s <= strainData[1] || linear) return E;
    int n = (int)strainData.size();
    for (int i = 2; i < n; ++i)
      if (s <= strainData[i] || i == n - 1)
        return (stressData[i] - stressData[i - 1]) / (strainData[i] - strainData[i - 1]);
    return 0.0f;
  }
  // CVX_MaterialVoxel::updateDerived  VX_MaterialVoxel.cpp:57-79 (+ CVX_Material part :525-532)
  void derive_voxel() {
    eHat = E / ((1 - 2 * nu) * (1 + nu));
    double volume = nomSize * nomSize * nomSize;
    mass = (float)(volume * rho);
    inertia = (float)(mass * nomSize * nomSize / 6.0f);
    firstMoment = (float)(mass * nomSize / 2.0f);
    if (volume == 0 || mass == 0 || inertia == 0) {
      massInv = sqrtMass = inertiaInv = c2xSqMxExS = c2xSqIxExSxSxS = 0.0f;
      return;
    }
    massInv = 1.0f / mass;
    sqrtMass = std::sqrt(mass);
    inertiaInv = 1.0f / inertia;
    c2xSqMxExS = (float)(2.0f * std::sqrt(mass * E * nomSize));
    c2xSqIxExSxSxS = (float)(2.0f * std::sqrt(inertia * E * nomSize * nomSize * nomSize));
  }
  // CVX_MaterialLink::updateDerived  VX_MaterialLink.cpp:121-141
  void derive_link() {
    derive_voxel();
    float L = (float)nomSize;
    a1 = E * L;
    a2 = E * L * L * L / (12.0f * (1 + nu));
    b1 = E * L;
    b2 = E * L * L / 2.0f;
    b3 = E * L * L * L / 6.0f;
    sqA1 = std::sqrt(a1);
    sqA2xIp = std::sqrt(a2 * L * L / 6.0f);
    sqB1 = std::sqrt(b1);
    sqB2xFMp = std::sqrt(b2 * L / 2.0f);
    sqB3xIp = std::sqrt(b3 * L * L / 6.0f);
  }
  void derive() {
    if (is_link) derive_link(); else derive_voxel();
  }
  // CVX_Material::setModelLinear  VX_Material.cpp:355-384
  bool set_linear(float youngs, float fail) {
    if (youngs <= 0) return false;
    if (fail != -1.0f && fail <= 0) return false;
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
    derive();
    return true;
  }
  // CVX_Material::setModelBilinear  VX_Material.cpp:389-434
  bool set_bilinear(float youngs, float plastic, float yieldS, float fail) {
    if (youngs <= 0) return false;
    if (plastic <= 0 || plastic >= youngs) return false;
    if (yieldS <= 0) return false;
    if (fail != -1.0f && fail <= yieldS) return false;
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
    derive();
    return true;
  }
  // CVX_Material::setYieldFromData  VX_Material.cpp:437-470
  bool yield_from_data(float pct = 0.2f) {
    sigmaYield = -1.0f;
    epsilonYield = -1.0f;
    float oM = E;
    float oB = (-pct / 100 * oM);
    int pts = (int)strainData.size() - 1;
    for (int i = 1; i < pts - 1; ++i) {
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
  // CVX_Material::setModel  VX_Material.cpp:283-350
  bool set_model(int n, const float* strain, const float* stress) {
    if (*strain == 0 && *stress == 0) { ++strain; ++stress; --n; }
    if (n <= 0) return false;
    if (*strain <= 0 || *stress <= 0) return false;
    std::vector<float> a{0.0f}, b{0.0f};
    float sw = 0.0f, ss = 0.0f;
    for (int i = 0; i < n; ++i) {
      float ts = strain[i], tt = stress[i];
      if (ts <= sw) return false;
      if (i > 0 && (tt - ss) / (ts - sw) > b[0] / a[0]) return false;
      sw = ts;
      ss = tt;
      a.push_back(ts);
      b.push_back(tt);
    }
    strainData = a;
    stressData = b;
    E = stressData[1] / strainData[1];
    sigmaFail = stressData.back();
    epsilonFail = strainData.back();
    linear = (n == 1);
    if (n == 1 || n == 2) {
      sigmaYield = stressData[1];
      epsilonYield = strainData[1];
    } else {
      yield_from_data();
    }
    derive();
    return true;
  }
};

// ---------------------------------------------------------------------------------------------
struct External {
  uint8_t dof = 0;
  F3 force, moment;
  V3 translation, rotation;
  Q4 rotQ;  // cached quaternion: refreshed only where the reference calls rotationChanged()
  bool fixedAll() const { return (dof & 0x3F) == 0x3F; }
  bool fixed(int d) const { return (dof & d) != 0; }
  bool fixedAllRot() const { return fixed(8) && fixed(16) && fixed(32); }
  bool fixedAnyRot() const { return fixed(8) || fixed(16) || fixed(32); }
  // CVX_External::rotationChanged  VX_External.cpp:100-109
  void rotation_changed() {
    if (rotation.x != 0 || rotation.y != 0 || rotation.z != 0) rotQ = from_rotation_vector(rotation);
    else rotQ = Q4();
  }
};

struct Voxel {
  int mat;
  short ix, iy, iz;
  int ext = -1;
  int links[6] = {-1, -1, -1, -1, -1, -1};
  V3 pos, linMom, angMom;
  Q4 orient;
  bool interior = false, floorEnabled = false, staticFriction = true, collisionsEnabled = false;
  float temp = 0, previousDt = 0;
  F3 pStrain;
  bool pStrainInvalid = true;
  // collisions
  F3 lastColWatch;
  std::vector<int> colWatch, nearby;
};

struct Link {
  int vneg, vpos, axis, mat;
  V3 forceNeg, forcePos, momentNeg, momentPos;
  float strain = 0, maxStrain = 0, strainOffset = 0, strainRatio = 1;
  bool localVelValid = false, smallAngle = true;
  V3 pos2, angle1v, angle2v;
  double restLength = 0;
  float transArea = 0, transStrainSum = 0;
  float stress = 0;
};

struct Collision {
  int v1, v2;
  float stiff, dampC;
  F3 force;
};

struct Key {
  int x, y, z;
  bool operator==(const Key& o) const { return x == o.x && y == o.y && z == o.z; }
};
struct KeyHash {
  size_t operator()(const Key& k) const {
    return ((size_t)(uint32_t)k.x * 73856093u) ^ ((size_t)(uint32_t)k.y * 19349663u) ^ ((size_t)(uint32_t)k.z * 83492791u);
  }
};

struct Sim {
  double voxSize;
  float currentTime = 0, ambientTemp = 0, grav = 0;
  bool floor = false, collisions = false, collisionsStale = true, nearbyStale = true;
  float boundingRadius = 0.75f, watchDistance = 1.0f;
  std::vector<Material> vmats;   // voxel materials
  std::vector<Material> lmats;   // link materials, creation order
  std::vector<Voxel> voxels;
  std::vector<Link> links;
  std::vector<External> exts;
  std::vector<Collision> cols;
  std::unordered_map<Key, int, KeyHash> vmap;      // lattice index -> voxel index
  std::unordered_map<Key, int, KeyHash> lmap[3];   // link lattice index per axis -> link index
  int nthreads = 1;

  explicit Sim(double s) : voxSize(s <= 0 ? 0.001 : s) {}

  External& ext_of(int v) {
    Voxel& vx = voxels[v];
    if (vx.ext < 0) {
      vx.ext = (int)exts.size();
      exts.emplace_back();
    }
    return exts[vx.ext];
  }

  // ---- voxel helpers (VX_Voxel.h / VX_Voxel.cpp) ---------------------------------------
  double base_size(const Voxel& v, int) const {  // VX_Voxel.h:89 (extScale is 1)
    const Material& m = vmats[v.mat];
    return m.nomSize * (1 + v.temp * m.alphaCTE);
  }
  double base_size_avg(const Voxel& v) const {  // VX_Voxel.h:90
    const Material& m = vmats[v.mat];
    float f = 1 + v.temp * m.alphaCTE;
    double b = (double)f * m.nomSize;
    return (b + b + b) / 3.0f;
  }
  float floor_penetration(const Voxel& v) const {  // VX_Voxel.h:122
    return (float)(base_size_avg(v) / 2 - vmats[v.mat].nomSize / 2 - v.pos.z);
  }
  float damping_multiplier(const Voxel& v) const {  // VX_Voxel.h:130
    const Material& m = vmats[v.mat];
    return 2 * m.sqrtMass * m.zetaInternal / v.previousDt;
  }
  // CVX_Link::axialStrain(bool)  VX_Link.cpp:121-124
  static float link_axial_strain(const Link& l, bool positiveEnd) {
    return positiveEnd ? 2.0f * l.strain * l.strainRatio / (1.0f + l.strainRatio)
                       : 2.0f * l.strain / (1.0f + l.strainRatio);
  }
  // CVX_Voxel::strain  VX_Voxel.cpp:300-334
  F3 voxel_strain(const Voxel& v, bool poissons) const {
    float s[3] = {0, 0, 0};
    int nb[3] = {0, 0, 0};
    bool tension[3] = {false, false, false};
    for (int i = 0; i < 6; ++i) {
      if (v.links[i] >= 0) {
        int ax = i / 2;
        s[ax] += link_axial_strain(links[v.links[i]], i % 2 == 1);
        nb[ax]++;
      }
    }
    for (int i = 0; i < 3; ++i) {
      if (nb[i] == 2) s[i] *= 0.5f;
      if (poissons) {
        bool t = nb[i] == 2;
        if (!t && v.ext >= 0 && nb[i] == 1) {
          const External& e = exts[v.ext];
          t = e.fixed(1 << i) || compf(e.force, i) != 0;
        }
        tension[i] = t;
      }
    }
    if (poissons && !(tension[0] && tension[1] && tension[2])) {
      float add = 0;
      for (int i = 0; i < 3; ++i)
        if (tension[i]) add += s[i];
      float value = std::pow(1.0f + add, -vmats[v.mat].nu) - 1.0f;
      for (int i = 0; i < 3; ++i)
        if (!tension[i]) s[i] = value;
    }
    F3 r;
    r.x = s[0]; r.y = s[1]; r.z = s[2];
    return r;
  }
  // CVX_Voxel::poissonsStrain  VX_Voxel.cpp:336-343
  F3 poissons_strain(Voxel& v) {
    if (v.pStrainInvalid) {
      v.pStrain = voxel_strain(v, true);
      v.pStrainInvalid = false;
    }
    return v.pStrain;
  }
  // CVX_Voxel::transverseStrainSum  VX_Voxel.cpp:346-359
  float transverse_strain_sum(Voxel& v, int axis) {
    if (vmats[v.mat].nu == 0) return 0;
    F3 p = poissons_strain(v);
    switch (axis) {
      case 0: return p.y + p.z;
      case 1: return p.x + p.z;
      default: return p.x + p.y;
    }
  }
  // CVX_Voxel::transverseArea  VX_Voxel.cpp:361-374
  float transverse_area(Voxel& v, int axis) {
    float size = (float)vmats[v.mat].nomSize;
    if (vmats[v.mat].nu == 0) return size * size;
    F3 p = poissons_strain(v);
    double px = p.x, py = p.y, pz = p.z;
    switch (axis) {
      case 0: return (float)(size * size * (1 + py) * (1 + pz));
      case 1: return (float)(size * size * (1 + px) * (1 + pz));
      default: return (float)(size * size * (1 + px) * (1 + py));
    }
  }

  // ---- link helpers (VX_Link.cpp) --------------------------------------------------------
  void update_rest_length(Link& l) {  // VX_Link.cpp:137-140
    l.restLength = 0.5 * (base_size(voxels[l.vneg], l.axis) + base_size(voxels[l.vpos], l.axis));
  }
  void update_transverse_info(Link& l) {  // VX_Link.cpp:142-147
    l.transArea = 0.5f * (transverse_area(voxels[l.vneg], l.axis) + transverse_area(voxels[l.vpos], l.axis));
    l.transStrainSum =
        0.5f * (transverse_strain_sum(voxels[l.vneg], l.axis) + transverse_strain_sum(voxels[l.vpos], l.axis));
  }
  void reset_link(Link& l) {  // VX_Link.cpp:61-75
    l.pos2 = l.angle1v = l.angle2v = V3();
    l.forceNeg = l.forcePos = l.momentNeg = l.momentPos = V3();
    l.strain = l.maxStrain = l.strainOffset = l.stress = 0.0f;
    l.strainRatio = vmats[voxels[l.vpos].mat].E / vmats[voxels[l.vneg].mat].E;
    l.smallAngle = true;
    l.localVelValid = false;
    update_rest_length(l);
    update_transverse_info(l);
  }
  // CVX_Link::updateStrain  VX_Link.cpp:220-249
  float update_strain(Link& l, float axial) {
    const Material& m = lmats[l.mat];
    l.strain = axial;
    if (m.linear) {
      if (axial > l.maxStrain) l.maxStrain = axial;
      return m.stress(axial, l.transStrainSum);
    }
    float ret;
    if (axial > l.maxStrain) {
      l.maxStrain = axial;
      ret = m.stress(axial, l.transStrainSum);
      if (m.nu != 0.0f) l.strainOffset = l.maxStrain - m.stress(axial) / (m.eHat * (1 - m.nu));
      else l.strainOffset = l.maxStrain - ret / m.E;
    } else {
      float rel = axial - l.strainOffset;
      if (m.nu != 0.0f) ret = m.stress(rel, l.transStrainSum, true);
      else ret = m.E * rel;
    }
    return ret;
  }
  static V3 to_axis_x(int axis, const V3& v) {  // VX_Link.h:114
    switch (axis) {
      case 1: return v3(v.y, -v.x, v.z);
      case 2: return v3(v.z, v.y, -v.x);
      default: return v;
    }
  }
  static Q4 to_axis_x(int axis, const Q4& q) {  // VX_Link.h:115
    switch (axis) {
      case 1: return q4(q.w, q.y, -q.x, q.z);
      case 2: return q4(q.w, q.z, q.y, -q.x);
      default: return q;
    }
  }
  static void to_axis_original(int axis, V3& v) {  // VX_Link.h:116
    if (axis == 1) { double t = v.y; v.y = v.x; v.x = -t; }
    else if (axis == 2) { double t = v.z; v.z = v.x; v.x = -t; }
  }

  // CVX_Link::updateForces + orientLink  VX_Link.cpp:77-119, 149-217
  void update_forces(Link& l) {
    const Voxel& vn = voxels[l.vneg];
    const Voxel& vp = voxels[l.vpos];
    V3 oldPos2 = l.pos2, oldA1 = l.angle1v, oldA2 = l.angle2v;
    // orientLink
    V3 pos2 = to_axis_x(l.axis, v3(vp.pos.x - vn.pos.x, vp.pos.y - vn.pos.y, vp.pos.z - vn.pos.z));
    Q4 angle1 = to_axis_x(l.axis, vn.orient);
    Q4 angle2 = to_axis_x(l.axis, vp.orient);
    Q4 totalRot = q4(angle1.w, -angle1.x, -angle1.y, -angle1.z);
    pos2 = rotate(totalRot, pos2);
    angle2 = qmul(totalRot, angle2);
    angle1 = Q4();
    float smallTurn = (float)((std::fabs(pos2.z) + std::fabs(pos2.y)) / pos2.x);
    float extendPerc = (float)(std::fabs(1 - pos2.x / l.restLength));
    const float HF = 1.2f, BEND = 0.05f, EXT = 0.50f;  // VX_Link.cpp:21-23
    if (!l.smallAngle && smallTurn < BEND && extendPerc < EXT) {
      l.smallAngle = true;
      l.localVelValid = false;
    } else if (l.smallAngle && (smallTurn > HF * BEND || extendPerc > HF * EXT)) {
      l.smallAngle = false;
      l.localVelValid = false;
    }
    if (l.smallAngle) {
      pos2.x -= l.restLength;
    } else {
      from_angle_to_pos_x(angle1, pos2);
      angle2 = qmul(angle1, angle2);
      pos2 = v3(std::sqrt(pos2.x * pos2.x + pos2.y * pos2.y + pos2.z * pos2.z) - l.restLength, 0, 0);
    }
    V3 a1v = to_rotation_vector(angle1);
    V3 a2v = to_rotation_vector(angle2);
    l.pos2 = pos2;
    l.angle1v = a1v;
    l.angle2v = a2v;

    V3 dPos2 = v3(0.5 * (pos2.x - oldPos2.x), 0.5 * (pos2.y - oldPos2.y), 0.5 * (pos2.z - oldPos2.z));
    V3 dA1 = v3(0.5 * (a1v.x - oldA1.x), 0.5 * (a1v.y - oldA1.y), 0.5 * (a1v.z - oldA1.z));
    V3 dA2 = v3(0.5 * (a2v.x - oldA2.x), 0.5 * (a2v.y - oldA2.y), 0.5 * (a2v.z - oldA2.z));

    const Material& m = lmats[l.mat];
    if (!(m.nu == 0.0f) || l.transStrainSum != 0) update_transverse_info(l);

    l.stress = update_strain(l, (float)(pos2.x / l.restLength));
    if (m.isFailed(l.maxStrain)) {
      l.forceNeg = l.forcePos = l.momentNeg = l.momentPos = V3();
      return;
    }
    float b1 = m.b1, b2 = m.b2, b3 = m.b3, a2 = m.a2;
    V3 fN = v3((double)(l.stress * l.transArea), b1 * pos2.y - b2 * (a1v.z + a2v.z),
               b1 * pos2.z + b2 * (a1v.y + a2v.y));
    V3 fP = v3(-fN.x, -fN.y, -fN.z);
    V3 mN = v3(a2 * (a2v.x - a1v.x), -b2 * pos2.z - b3 * (2 * a1v.y + a2v.y),
               b2 * pos2.y - b3 * (2 * a1v.z + a2v.z));
    V3 mP = v3(a2 * (a1v.x - a2v.x), -b2 * pos2.z - b3 * (a1v.y + 2 * a2v.y),
               b2 * pos2.y - b3 * (a1v.z + 2 * a2v.z));
    if (l.localVelValid) {
      float sqA1 = m.sqA1, sqA2xIp = m.sqA2xIp, sqB1 = m.sqB1, sqB2xFMp = m.sqB2xFMp, sqB3xIp = m.sqB3xIp;
      V3 pc = v3(sqA1 * dPos2.x, sqB1 * dPos2.y - sqB2xFMp * (dA1.z + dA2.z),
                 sqB1 * dPos2.z + sqB2xFMp * (dA1.y + dA2.y));
      float dmN = damping_multiplier(vn), dmP = damping_multiplier(vp);
      fN.x += dmN * pc.x; fN.y += dmN * pc.y; fN.z += dmN * pc.z;
      fP.x -= dmP * pc.x; fP.y -= dmP * pc.y; fP.z -= dmP * pc.z;
      double hN = 0.5 * dmN, hP = 0.5 * dmP;
      V3 tN = v3(-sqA2xIp * (dA2.x - dA1.x), sqB2xFMp * dPos2.z + sqB3xIp * (2 * dA1.y + dA2.y),
                 -sqB2xFMp * dPos2.y + sqB3xIp * (2 * dA1.z + dA2.z));
      V3 tP = v3(sqA2xIp * (dA2.x - dA1.x), sqB2xFMp * dPos2.z + sqB3xIp * (dA1.y + 2 * dA2.y),
                 -sqB2xFMp * dPos2.y + sqB3xIp * (dA1.z + 2 * dA2.z));
      mN.x -= hN * tN.x; mN.y -= hN * tN.y; mN.z -= hN * tN.z;
      mP.x -= hP * tP.x; mP.y -= hP * tP.y; mP.z -= hP * tP.z;
    } else {
      l.localVelValid = true;
    }
    if (!l.smallAngle) {
      fN = rotate_inv(angle1, fN);
      mN = rotate_inv(angle1, mN);
    }
    fP = rotate_inv(angle2, fP);
    mP = rotate_inv(angle2, mP);
    to_axis_original(l.axis, fN);
    to_axis_original(l.axis, fP);
    to_axis_original(l.axis, mN);
    to_axis_original(l.axis, mP);
    l.forceNeg = fN;
    l.forcePos = fP;
    l.momentNeg = mN;
    l.momentPos = mP;
  }

  // CVX_Voxel::force  VX_Voxel.cpp:234-256
  V3 voxel_force(const Voxel& v) const {
    V3 t;
    for (int i = 0; i < 6; ++i) {
      if (v.links[i] < 0) continue;
      const Link& l = links[v.links[i]];
      const V3& f = (i % 2 == 1) ? l.forcePos : l.forceNeg;
      t.x += f.x; t.y += f.y; t.z += f.z;
    }
    t = rotate(v.orient, t);
    const Material& m = vmats[v.mat];
    if (v.ext >= 0) {
      const External& e = exts[v.ext];
      t.x += e.force.x; t.y += e.force.y; t.z += e.force.z;
    }
    float c = m.zetaGlobal * m.c2xSqMxExS;
    t.x -= c * (m.massInv * v.linMom.x);
    t.y -= c * (m.massInv * v.linMom.y);
    t.z -= c * (m.massInv * v.linMom.z);
    t.z += -m.mass * 9.80665f * m.gravMult;
    if (v.collisionsEnabled) {
      for (int ci : v.colWatch) {
        const Collision& c2 = cols[ci];
        F3 f = c2.force;
        if (c2.v2 == (int)(&v - voxels.data())) { f.x = -f.x; f.y = -f.y; f.z = -f.z; }
        t.x -= f.x; t.y -= f.y; t.z -= f.z;
      }
    }
    return t;
  }
  // CVX_Voxel::moment  VX_Voxel.cpp:258-271
  V3 voxel_moment(const Voxel& v) const {
    V3 t;
    for (int i = 0; i < 6; ++i) {
      if (v.links[i] < 0) continue;
      const Link& l = links[v.links[i]];
      const V3& f = (i % 2 == 1) ? l.momentPos : l.momentNeg;
      t.x += f.x; t.y += f.y; t.z += f.z;
    }
    t = rotate(v.orient, t);
    const Material& m = vmats[v.mat];
    if (v.ext >= 0) {
      const External& e = exts[v.ext];
      t.x += e.moment.x; t.y += e.moment.y; t.z += e.moment.z;
    }
    float c = m.zetaGlobal * m.c2xSqIxExSxSxS;
    t.x -= c * (m.inertiaInv * v.angMom.x);
    t.y -= c * (m.inertiaInv * v.angMom.y);
    t.z -= c * (m.inertiaInv * v.angMom.z);
    return t;
  }
  // CVX_Voxel::floorForce  VX_Voxel.cpp:274-298
  void floor_force(Voxel& v, V3& F) const {
    float pen = floor_penetration(v);
    const Material& m = vmats[v.mat];
    if (pen >= 0) {
      V3 vel = v3(m.massInv * v.linMom.x, m.massInv * v.linMom.y, m.massInv * v.linMom.z);
      float normal = (float)(2 * m.E * m.nomSize) * pen;
      F.z += normal - (m.zetaCollision * m.c2xSqMxExS) * vel.z;
      if (v.staticFriction) {
        float surf = (float)(F.x * F.x + F.y * F.y);
        float fric = (m.muStatic * normal) * (m.muStatic * normal);
        if (surf > fric) v.staticFriction = false;
      } else {
        float k = m.muKinetic * normal;
        V3 h = v3(vel.x, vel.y, 0);
        double len = std::sqrt(h.x * h.x + h.y * h.y + h.z * h.z);
        if (len > 0) {
          double inv = 1.0 / len;
          h = v3(inv * h.x, inv * h.y, inv * h.z);
        }
        F.x -= k * h.x; F.y -= k * h.y; F.z -= k * h.z;
      }
    } else {
      v.staticFriction = false;
    }
  }
  // CVX_Voxel::timeStep  VX_Voxel.cpp:162-232
  void voxel_step(Voxel& v, float dt) {
    v.previousDt = dt;
    if (dt == 0.0f) return;
    const Material& m = vmats[v.mat];
    if (v.ext >= 0 && exts[v.ext].fixedAll()) {
      const External& e = exts[v.ext];
      double s = m.nomSize;
      v.pos = v3(v.ix * s + e.translation.x, v.iy * s + e.translation.y, v.iz * s + e.translation.z);
      v.orient = e.rotQ;
      v.linMom = v.angMom = V3();
      return;
    }
    V3 F = voxel_force(v);
    V3 fric = F;
    if (v.floorEnabled) floor_force(v, F);
    fric = v3(F.x - fric.x, F.y - fric.y, F.z - fric.z);
    v.linMom.x += dt * F.x; v.linMom.y += dt * F.y; v.linMom.z += dt * F.z;
    float dtm = dt * m.massInv;
    V3 tr = v3(dtm * v.linMom.x, dtm * v.linMom.y, dtm * v.linMom.z);
    if (v.floorEnabled && floor_penetration(v) >= 0) {
      double work = fric.x * tr.x + fric.y * tr.y;
      double hKe = 0.5 * m.massInv * (v.linMom.x * v.linMom.x + v.linMom.y * v.linMom.y);
      if (hKe + work <= 0) v.staticFriction = true;
      if (v.staticFriction) {
        v.linMom.x = v.linMom.y = 0;
        tr.x = tr.y = 0;
      }
    } else {
      v.staticFriction = false;
    }
    v.pos.x += tr.x; v.pos.y += tr.y; v.pos.z += tr.z;
    V3 M = voxel_moment(v);
    v.angMom.x += dt * M.x; v.angMom.y += dt * M.y; v.angMom.z += dt * M.z;
    float dti = dt * m.inertiaInv;
    Q4 dq = from_rotation_vector(v3(dti * v.angMom.x, dti * v.angMom.y, dti * v.angMom.z));
    v.orient = qmul(dq, v.orient);
    if (v.ext >= 0) {
      const External& e = exts[v.ext];
      double s = m.nomSize;
      if (e.fixed(1)) { v.pos.x = v.ix * s + e.translation.x; v.linMom.x = 0; }
      if (e.fixed(2)) { v.pos.y = v.iy * s + e.translation.y; v.linMom.y = 0; }
      if (e.fixed(4)) { v.pos.z = v.iz * s + e.translation.z; v.linMom.z = 0; }
      if (e.fixedAnyRot()) {
        if (e.fixedAllRot()) {
          v.orient = e.rotQ;
          v.angMom = V3();
        } else {
          V3 r = to_rotation_vector(v.orient);
          if (e.fixed(8)) { r.x = 0; v.angMom.x = 0; }
          if (e.fixed(16)) { r.y = 0; v.angMom.y = 0; }
          if (e.fixed(32)) { r.z = 0; v.angMom.z = 0; }
          v.orient = from_rotation_vector(r);
        }
      }
    }
    v.pStrainInvalid = true;
  }

  // ---- collisions (Voxelyze.cpp:670-750, VX_Collision.cpp, VX_Voxel.cpp:395-418) -----------
  int adjacent(int v, int dir) const {
    int li = voxels[v].links[dir];
    if (li < 0) return -1;
    const Link& l = links[li];
    return l.vpos == v ? l.vneg : l.vpos;
  }
  void generate_nearby(int v, int depth) {
    std::vector<int> all{v};
    std::unordered_map<int, char> seen{{v, 1}};
    size_t cur = 0;
    for (int k = 0; k < depth; ++k) {
      size_t end = all.size();
      while (cur != end) {
        int p = all[cur++];
        for (int d = 0; d < 6; ++d) {
          int q = adjacent(p, d);
          if (q >= 0 && !seen.count(q)) { seen[q] = 1; all.push_back(q); }
        }
      }
    }
    Voxel& vx = voxels[v];
    vx.nearby.clear();
    for (int q : all)
      if (!voxels[q].interior && q != v) vx.nearby.push_back(q);
    std::sort(vx.nearby.begin(), vx.nearby.end());
  }
  void clear_collisions() {
    cols.clear();
    for (Voxel& v : voxels) v.colWatch.clear();
  }
  // CVoxelyze::regenerateCollisions  Voxelyze.cpp:725-750.  The reference tests every later voxel
  // j > i for each surface voxel i (O(N^2)); the same pairs come from a grid of cells slightly
  // wider than the watch radius, so that every j within the radius lies in one of the 27 cells
  // around i's, each candidate then passing the reference's exact double-precision distance test
  // and nearby exclusion.  Pairs are listed in (i, j) order as the reference's loops produce them,
  // and each voxel's watch list in that list order, so the result is the reference's.
  void regenerate_collisions(float thr) {
    clear_collisions();
    const int n = (int)voxels.size();
    const double h = std::sqrt((double)thr) * 1.001 + 1e-300;
    std::unordered_map<Key, std::vector<int>, KeyHash> cell;
    auto key_of = [&](const V3& p) {
      Key k;
      k.x = (int)std::floor(p.x / h); k.y = (int)std::floor(p.y / h); k.z = (int)std::floor(p.z / h);
      return k;
    };
    std::vector<int> surf;
    for (int i = 0; i < n; ++i) {
      Voxel& a = voxels[i];
      if (a.interior) continue;
      a.lastColWatch.x = (float)a.pos.x; a.lastColWatch.y = (float)a.pos.y; a.lastColWatch.z = (float)a.pos.z;
      cell[key_of(a.pos)].push_back(i);  // ascending i within each cell
      surf.push_back(i);
    }
    std::vector<std::vector<int>> partners(surf.size());
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 64)
    for (long long si = 0; si < (long long)surf.size(); ++si) {
      const int i = surf[si];
      const Voxel& a = voxels[i];
      const Key c = key_of(a.pos);
      std::vector<int>& out = partners[si];
      for (int dz = -1; dz <= 1; ++dz)
        for (int dy = -1; dy <= 1; ++dy)
          for (int dx = -1; dx <= 1; ++dx) {
            Key k;
            k.x = c.x + dx; k.y = c.y + dy; k.z = c.z + dz;
            auto it = cell.find(k);
            if (it == cell.end()) continue;
            for (int j : it->second) {
              if (j <= i) continue;
              const Voxel& b = voxels[j];
              double ex = a.pos.x - b.pos.x, ey = a.pos.y - b.pos.y, ez = a.pos.z - b.pos.z;
              if (ex * ex + ey * ey + ez * ez > thr) continue;
              if (std::binary_search(a.nearby.begin(), a.nearby.end(), j)) continue;
              out.push_back(j);
            }
          }
      std::sort(out.begin(), out.end());
    }
    for (size_t si = 0; si < surf.size(); ++si) {
      const int i = surf[si];
      for (int j : partners[si]) {
        Voxel& a = voxels[i];
        Voxel& b = voxels[j];
        const Material& m1 = vmats[a.mat];
        const Material& m2 = vmats[b.mat];
        Collision c;
        c.v1 = i;
        c.v2 = j;
        c.stiff = 2.0f / (1.0f / (float)(2 * m1.E * m1.nomSize) + 1.0f / (float)(2 * m2.E * m2.nomSize));
        c.dampC = 0.5f * (m1.zetaCollision * m1.c2xSqMxExS + m2.zetaCollision * m2.c2xSqMxExS);
        cols.push_back(c);
        a.colWatch.push_back((int)cols.size() - 1);
        b.colWatch.push_back((int)cols.size() - 1);
      }
    }
    collisionsStale = false;
  }
  void update_contact(Collision& c) {  // VX_Collision.cpp:42-56
    const Voxel& a = voxels[c.v1];
    const Voxel& b = voxels[c.v2];
    float ox = (float)(b.pos.x - a.pos.x), oy = (float)(b.pos.y - a.pos.y), oz = (float)(b.pos.z - a.pos.z);
    float nom = (float)((base_size_avg(a) + base_size_avg(b)) * 0.625f);
    float rel = nom - std::sqrt(ox * ox + oy * oy + oz * oz);
    if (rel > 0) {
      float l = std::sqrt(ox * ox + oy * oy + oz * oz);
      float ux = ox, uy = oy, uz = oz;
      if (l > 0) {
        float inv = (float)1.0 / l;
        ux = inv * ox; uy = inv * oy; uz = inv * oz;
      }
      const Material& m1 = vmats[a.mat];
      const Material& m2 = vmats[b.mat];
      double v1x = m1.massInv * a.linMom.x, v1y = m1.massInv * a.linMom.y, v1z = m1.massInv * a.linMom.z;
      double v2x = m2.massInv * b.linMom.x, v2y = m2.massInv * b.linMom.y, v2z = m2.massInv * b.linMom.z;
      float relVel = (float)((v1x * (double)ux + v1y * (double)uy + v1z * (double)uz) -
                             (v2x * (double)ux + v2y * (double)uy + v2z * (double)uz));
      float k = c.stiff * rel + c.dampC * relVel;
      c.force.x = ux * k; c.force.y = uy * k; c.force.z = uz * k;
    } else {
      c.force = F3();
    }
  }
  void update_collisions() {
    float watchVx = 2 * boundingRadius + watchDistance;
    float watchMm = (float)(voxSize * watchVx);
    float recalc = (float)(voxSize * watchDistance / 2);
    if (nearbyStale) {
      // each voxel's list depends on the lattice only
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 256)
      for (int v = 0; v < (int)voxels.size(); ++v) generate_nearby(v, (int)(watchVx * 2));
      nearbyStale = false;
      collisionsStale = true;
    }
    for (const Voxel& v : voxels) {
      if (v.interior) continue;
      double dx = v.pos.x - v.lastColWatch.x, dy = v.pos.y - v.lastColWatch.y, dz = v.pos.z - v.lastColWatch.z;
      if (dx * dx + dy * dy + dz * dz > recalc * recalc) collisionsStale = true;
    }
    if (collisionsStale) regenerate_collisions(watchMm * watchMm);
#pragma omp parallel for num_threads(nthreads) schedule(static)
    for (long long k = 0; k < (long long)cols.size(); ++k) update_contact(cols[k]);
  }

  // ---- scene building (Voxelyze.cpp:357-640) ---------------------------------------------
  int combined_material(int a, int b) {  // Voxelyze.cpp:626-640
    for (size_t i = 0; i < lmats.size(); ++i)
      if ((lmats[i].m1 == a && lmats[i].m2 == b) || (lmats[i].m1 == b && lmats[i].m2 == a)) return (int)i;
    Material m;
    m.is_link = true;
    m.m1 = a;
    m.m2 = b;
    lmats.push_back(m);
    link_material_update((int)lmats.size() - 1);
    return (int)lmats.size() - 1;
  }
  // CVX_MaterialLink::updateAll  VX_MaterialLink.cpp:45-119
  void link_material_update(int li) {
    Material& L = lmats[li];
    const Material& A = vmats[L.m1];
    const Material& B = vmats[L.m2];
    L.nomSize = 0.5 * (A.nomSize + B.nomSize);
    L.rho = 0.5f * (A.rho + B.rho);
    L.alphaCTE = 0.5f * (A.alphaCTE + B.alphaCTE);
    L.muStatic = 0.5f * (A.muStatic + B.muStatic);
    L.muKinetic = 0.5f * (A.muKinetic + B.muKinetic);
    L.zetaInternal = 0.5f * (A.zetaInternal + B.zetaInternal);
    L.zetaGlobal = 0.5f * (A.zetaGlobal + B.zetaGlobal);
    L.zetaCollision = 0.5f * (A.zetaCollision + B.zetaCollision);
    float f1 = A.sigmaFail, f2 = B.sigmaFail, sf;
    if (f1 == -1.0f) sf = f2;
    else if (f2 == -1.0f) sf = f1;
    else sf = f1 < f2 ? f1 : f2;
    if (A.linear && B.linear) {
      L.set_linear(2.0f * A.E * B.E / (A.E + B.E), sf);
    } else {
      std::vector<float> ns{0.0f}, nt{0.0f};
      size_t i1 = 1, i2 = 1;
      while (i1 < A.strainData.size() && i2 < B.strainData.size()) {
        float s = FLT_MAX;
        if (i1 < A.strainData.size()) s = A.strainData[i1];
        if (i2 < B.strainData.size() && B.strainData[i2] < s) s = B.strainData[i2];
        if (s == A.strainData[i1]) i1++;
        if (s == B.strainData[i2]) i2++;
        float mA = A.modulus(s - FLT_EPSILON);
        float mB = B.modulus(s - FLT_EPSILON);
        float mod = 2.0f * mA * mB / (mA + mB);
        size_t last = ns.size() - 1;
        ns.push_back(s);
        nt.push_back(nt[last] + mod * (s - ns[last]));
      }
      L.set_model((int)ns.size(), ns.data(), nt.data());
      L.sigmaFail = sf;
      L.epsilonFail = sf == -1.0f ? -1.0f : L.strain_of(sf);
    }
    if (A.nu == 0 && B.nu == 0) {
      L.nu = 0;
    } else {
      float th = 2 * A.eHat * B.eHat / (A.eHat + B.eHat);
      float te = L.E;
      float c2 = (th - te) / (2 * th) + 0.0625;
      L.nu = std::sqrt(c2) - 0.25;
    }
    L.derive_link();
  }
  void voxel_material_changed(int m) {  // CVX_Material::updateDerived -> dependents updateAll
    vmats[m].derive_voxel();
    for (size_t i = 0; i < lmats.size(); ++i)
      if (lmats[i].m1 == m || lmats[i].m2 == m) link_material_update((int)i);
  }
  void update_surface(Voxel& v) {  // VX_Voxel.cpp:376-381
    bool in = true;
    for (int i = 0; i < 6; ++i)
      if (v.links[i] < 0) in = false;
    v.interior = in;
  }
  static const int* dir_off(int d) {
    static const int off[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
    return off[d];
  }
  int voxel_at(int x, int y, int z) const {
    auto it = vmap.find(Key{x, y, z});
    return it == vmap.end() ? -1 : it->second;
  }
  // CVoxelyze::addLink  Voxelyze.cpp:508-539
  void add_link(int x, int y, int z, int dir) {
    int ax = dir / 2;
    Key lk{x - (dir == 1), y - (dir == 3), z - (dir == 5)};
    if (lmap[ax].count(lk)) return;
    const int* o = dir_off(dir);
    int v1 = voxel_at(x, y, z), v2 = voxel_at(x + o[0], y + o[1], z + o[2]);
    if (v1 < 0 || v2 < 0) return;
    int lm = combined_material(voxels[v1].mat, voxels[v2].mat);
    Link l;
    bool reverse = (dir % 2 == 1);  // voxel1 sits on the positive side for a negative direction
    l.vneg = reverse ? v2 : v1;
    l.vpos = reverse ? v1 : v2;
    l.axis = ax;
    l.mat = lm;
    links.push_back(l);
    int li = (int)links.size() - 1;
    reset_link(links[li]);
    lmap[ax][lk] = li;
    voxels[v1].links[dir] = li;
    update_surface(voxels[v1]);
    int opp = dir - dir % 2 + (dir + 1) % 2;
    voxels[v2].links[opp] = li;
    update_surface(voxels[v2]);
  }
  void set_temperature(int v, float t) {  // VX_Voxel.cpp:108-114
    voxels[v].temp = t;
    for (int i = 0; i < 6; ++i)
      if (voxels[v].links[i] >= 0) update_rest_length(links[voxels[v].links[i]]);
  }
  // CVoxelyze::addVoxel  Voxelyze.cpp:439-461
  int add_voxel(int mat, int x, int y, int z) {
    nearbyStale = collisionsStale = true;
    Voxel v;
    v.mat = mat;
    v.ix = (short)x; v.iy = (short)y; v.iz = (short)z;
    double s = vmats[mat].nomSize;
    v.pos = v3(v.ix * s, v.iy * s, v.iz * s);  // reset()
    voxels.push_back(v);
    int idx = (int)voxels.size() - 1;
    vmap[Key{x, y, z}] = idx;
    voxels[idx].pos = v3(x * voxSize, y * voxSize, z * voxSize);
    voxels[idx].floorEnabled = floor;
    set_temperature(idx, ambientTemp);
    voxels[idx].collisionsEnabled = collisions;
    for (int d = 0; d < 6; ++d) add_link(x, y, z, d);
    return idx;
  }

  // ---- topology edits (Voxelyze.cpp:384-498, 541-575, 643-668) ---------------------------
  // CVoxelyze::removeLink: the link leaves the list (later links move down one index) and both end
  // voxels lose it (surface flags updated)
  void remove_link(int x, int y, int z, int dir) {
    int ax = dir / 2;
    auto it = lmap[ax].find(Key{x - (dir == 1), y - (dir == 3), z - (dir == 5)});
    if (it == lmap[ax].end()) return;
    const int li = it->second;
    lmap[ax].erase(it);
    links.erase(links.begin() + li);
    for (auto& m : lmap)
      for (auto& kv : m)
        if (kv.second > li) kv.second--;
    for (Voxel& v : voxels)
      for (int& sl : v.links) {
        if (sl == li) sl = -1;
        else if (sl > li) sl--;
      }
    int v1 = voxel_at(x, y, z);
    if (v1 >= 0) update_surface(voxels[v1]);
    const int* o = dir_off(dir);
    int v2 = voxel_at(x + o[0], y + o[1], z + o[2]);
    if (v2 >= 0) update_surface(voxels[v2]);
  }
  // CVoxelyze::removeVoxel: the voxel leaves the list (later voxels move down one index) with its
  // links
  void remove_voxel(int x, int y, int z) {
    nearbyStale = collisionsStale = true;
    const int v = voxel_at(x, y, z);
    if (v < 0) return;
    vmap.erase(Key{x, y, z});
    for (int d = 0; d < 6; ++d) remove_link(x, y, z, d);
    voxels.erase(voxels.begin() + v);
    for (auto& kv : vmap)
      if (kv.second > v) kv.second--;
    for (Link& l : links) {
      if (l.vneg > v) l.vneg--;
      if (l.vpos > v) l.vpos--;
    }
  }
  // CVoxelyze::replaceVoxel with CVX_Voxel::replaceMaterial (VX_Voxel.cpp:78-90): momenta scaled to
  // keep the velocities, static friction cleared, Poisson cache invalid, links rebuilt (they move
  // to the end of the list)
  void replace_voxel(int mat, int x, int y, int z) {
    collisionsStale = true;
    const int v = voxel_at(x, y, z);
    Voxel& vx = voxels[v];
    const float fm = vmats[mat].mass / vmats[vx.mat].mass;
    const float fi = vmats[mat].inertia / vmats[vx.mat].inertia;
    vx.linMom = v3(vx.linMom.x * fm, vx.linMom.y * fm, vx.linMom.z * fm);
    vx.angMom = v3(vx.angMom.x * fi, vx.angMom.y * fi, vx.angMom.z * fi);
    vx.staticFriction = false;
    vx.pStrainInvalid = true;
    vx.mat = mat;
    for (int d = 0; d < 6; ++d) {
      remove_link(x, y, z, d);
      add_link(x, y, z, d);
    }
  }
  // CVoxelyze::setVoxel (Voxelyze.cpp:422-437)
  int set_voxel(int mat, int x, int y, int z) {
    if (mat < 0) {
      remove_voxel(x, y, z);
      return -1;
    }
    int v = voxel_at(x, y, z);
    if (v >= 0) {
      replace_voxel(mat, x, y, z);
      return v;
    }
    return add_voxel(mat, x, y, z);
  }
  // CVoxelyze::replaceMaterial: the lattice is visited z, then y, then x (the reference walks its
  // bounding box in that order; an empty cell there dereferences a null voxel, so only occupied
  // cells are visited here)
  void replace_material(int a, int b) {
    std::vector<Key> cells;
    for (const Voxel& v : voxels)
      if (v.mat == a) cells.push_back(Key{v.ix, v.iy, v.iz});
    std::sort(cells.begin(), cells.end(), [](const Key& p, const Key& q) {
      if (p.z != q.z) return p.z < q.z;
      if (p.y != q.y) return p.y < q.y;
      return p.x < q.x;
    });
    for (const Key& k : cells) set_voxel(b, k.x, k.y, k.z);
  }
  // CVoxelyze::removeMaterial: its voxels, then the material; the link materials built from it go
  // too (the reference leaves them in its list, unused)
  void remove_material(int m) {
    std::vector<Key> cells;
    for (const Voxel& v : voxels)
      if (v.mat == m) cells.push_back(Key{v.ix, v.iy, v.iz});
    for (const Key& k : cells) remove_voxel(k.x, k.y, k.z);
    std::vector<int> lnew(lmats.size(), -1);
    std::vector<Material> keep;
    for (size_t i = 0; i < lmats.size(); ++i)
      if (lmats[i].m1 != m && lmats[i].m2 != m) {
        lnew[i] = (int)keep.size();
        keep.push_back(lmats[i]);
      }
    lmats.swap(keep);
    for (Material& L : lmats) {
      if (L.m1 > m) L.m1--;
      if (L.m2 > m) L.m2--;
    }
    for (Link& l : links) l.mat = lnew[l.mat];
    vmats.erase(vmats.begin() + m);
    for (Voxel& v : voxels)
      if (v.mat > m) v.mat--;
  }
  // CVoxelyze::setVoxelSize: voxel materials take the new nominal size (CVX_MaterialVoxel::
  // setNominalSize, whose derived update also refreshes the link materials built from it),
  // positions scale, motion stops, static friction clears, links reset
  void set_voxel_size(double s) {
    double f = s / voxSize;
    voxSize = s;
    for (size_t k = 0; k < vmats.size(); ++k) {
      vmats[k].nomSize = s <= 0 ? FLT_MIN : s;
      voxel_material_changed((int)k);
    }
    for (Voxel& v : voxels) {
      v.pos = v3(v.pos.x * f, v.pos.y * f, v.pos.z * f);
      v.linMom = v.angMom = V3();
      v.staticFriction = false;
    }
    for (Link& l : links) reset_link(l);
    collisionsStale = true;
  }

  // ---- time step (Voxelyze.cpp:251-311) --------------------------------------------------
  float recommended_dt() {
    float mx = 0.0f;
    for (Link& l : links) {
      float m1 = vmats[voxels[l.vneg].mat].mass, m2 = vmats[voxels[l.vpos].mat].mass;
      const Material& m = lmats[l.mat];
      float k;
      if (m.nu == 0.0f) {
        k = m.a1;
      } else {
        update_rest_length(l);
        update_transverse_info(l);
        k = (float)(m.eHat * l.transArea / ((l.strain + 1) * l.restLength));
      }
      float f = k / (m1 < m2 ? m1 : m2);
      if (f > mx) mx = f;
    }
    if (mx <= 0.0f) {
      for (const Voxel& v : voxels) {
        const Material& m = vmats[v.mat];
        float f = m.E * m.nomSize / m.mass;
        if (f > mx) mx = f;
      }
    }
    if (mx <= 0.0f) return 0.0f;
    return 1.0f / (6.283185f * std::sqrt(mx));
  }

  // Serial-equivalent Poisson strain pre-pass: the first link of each nu != 0 voxel would fill the
  // cache from the previous step's link strains (VX_Voxel.cpp:336-343, VX_Link.cpp:160).
  void poisson_prepass() {
    // each voxel's cache reads only the previous step's link strains and writes only itself
    const int nv = (int)voxels.size();
#pragma omp parallel for num_threads(nthreads) schedule(static)
    for (int k = 0; k < nv; ++k) {
      Voxel& v = voxels[k];
      if (!v.pStrainInvalid || vmats[v.mat].nu == 0) continue;
      bool any = false;
      for (int i = 0; i < 6; ++i) any |= v.links[i] >= 0;
      if (any) poissons_strain(v);
    }
  }

  bool do_time_step(float dt) {
    if (dt == 0) return true;
    if (dt < 0) dt = recommended_dt();
    poisson_prepass();
    int nl = (int)links.size();
    int diverged = 0;
#pragma omp parallel for num_threads(nthreads) schedule(static) reduction(| : diverged)
    for (int i = 0; i < nl; ++i) {
      update_forces(links[i]);
      if (links[i].strain > 100) diverged |= 1;
    }
    if (diverged) return false;
    if (collisions) update_collisions();
    int nv = (int)voxels.size();
#pragma omp parallel for num_threads(nthreads) schedule(static)
    for (int i = 0; i < nv; ++i) voxel_step(voxels[i], dt);
    currentTime += dt;
    return true;
  }

  // CVoxelyze::resetTime  Voxelyze.cpp:313-321 + CVX_Voxel::reset VX_Voxel.cpp:47-56
  void reset_time() {
    currentTime = 0.0f;
    collisionsStale = true;
    nearbyStale = true;
    for (Voxel& v : voxels) {
      double s = vmats[v.mat].nomSize;
      v.pos = v3(v.ix * s, v.iy * s, v.iz * s);
      v.orient = Q4();
      v.linMom = v.angMom = V3();
      v.staticFriction = true;
      v.temp = 0.0f;
      v.previousDt = 0.0f;
      v.pStrainInvalid = true;
    }
    for (Link& l : links) reset_link(l);
  }

  // ---- per-voxel and per-link queries (VX_Voxel.h:79-130, VX_Voxel.cpp:100-159, VX_Link.cpp:127-135,
  // 251-257) ----------------------------------------------------------------------------------
  bool link_failed(int li) const { return li >= 0 && lmats[links[li].mat].isFailed(links[li].maxStrain); }
  bool link_yielded(int li) const { return li >= 0 && lmats[links[li].mat].isYielded(links[li].maxStrain); }
  // CVX_Voxel::isYielded / isFailed  VX_Voxel.cpp:92-106: any of its links
  bool voxel_yielded(const Voxel& v) const {
    for (int i = 0; i < 6; ++i)
      if (link_yielded(v.links[i])) return true;
    return false;
  }
  bool voxel_failed(const Voxel& v) const {
    for (int i = 0; i < 6; ++i)
      if (link_failed(v.links[i])) return true;
    return false;
  }
  // CVX_Voxel::externalForce  VX_Voxel.cpp:117-127: the applied force, with each fixed translation
  // replaced by the reaction -force() (computed in double, taken as float)
  F3 external_force(const Voxel& v) const {
    const External& e = exts[v.ext];
    F3 r = e.force;
    if (e.fixed(1) || e.fixed(2) || e.fixed(4)) {
      V3 f = voxel_force(v);
      F3 t;
      t.x = (float)-f.x; t.y = (float)-f.y; t.z = (float)-f.z;
      if (e.fixed(1)) r.x = t.x;
      if (e.fixed(2)) r.y = t.y;
      if (e.fixed(4)) r.z = t.z;
    }
    return r;
  }
  // CVX_Voxel::externalMoment  VX_Voxel.cpp:129-139
  F3 external_moment(const Voxel& v) const {
    const External& e = exts[v.ext];
    F3 r = e.moment;
    if (e.fixed(8) || e.fixed(16) || e.fixed(32)) {
      V3 m = voxel_moment(v);
      F3 t;
      t.x = (float)-m.x; t.y = (float)-m.y; t.z = (float)-m.z;
      if (e.fixed(8)) r.x = t.x;
      if (e.fixed(16)) r.y = t.y;
      if (e.fixed(32)) r.z = t.z;
    }
    return r;
  }
  // CVX_Voxel::cornerOffset  VX_Voxel.cpp:146-159: per axis the half-link strain of the link on the
  // corner's side (1 without a link or with a failed one), signed, scaling half the base size
  F3 corner_offset(const Voxel& v, int corner) const {
    double half = 0.5 * base_size(v, 0);
    double st[3];
    for (int i = 0; i < 3; ++i) {
      const bool posLink = (corner & (1 << (2 - i))) != 0;
      const int li = v.links[2 * i + (posLink ? 0 : 1)];
      if (li >= 0 && !link_failed(li)) st[i] = (1 + link_axial_strain(links[li], posLink)) * (posLink ? 1 : -1);
      else st[i] = posLink ? 1.0 : -1.0;
    }
    F3 r;
    r.x = (float)(half * st[0]); r.y = (float)(half * st[1]); r.z = (float)(half * st[2]);
    return r;
  }
  // CVX_Voxel::cornerPosition  VX_Voxel.cpp:141-144: float position plus the offset rotated by the
  // double orientation in the mixed-type form of Quat3D::RotateVec3D (Quat3D.h:179-186)
  F3 corner_position(const Voxel& v, int corner) const {
    const F3 f = corner_offset(v, corner);
    const Q4& q = v.orient;
    const float tw = (float)(f.x * q.x + f.y * q.y + f.z * q.z);
    const float tx = (float)(f.x * q.w - f.y * q.z + f.z * q.y);
    const float ty = (float)(f.x * q.z + f.y * q.w - f.z * q.x);
    const float tz = (float)(-f.x * q.y + f.y * q.x + f.z * q.w);
    const float rx = (float)(q.w * tx + q.x * tw + q.y * tz - q.z * ty);
    const float ry = (float)(q.w * ty - q.x * tz + q.y * tw + q.z * tx);
    const float rz = (float)(q.w * tz + q.x * ty - q.y * tx + q.z * tw);
    F3 r;
    r.x = (float)v.pos.x + rx; r.y = (float)v.pos.y + ry; r.z = (float)v.pos.z + rz;
    return r;
  }
  // CVX_Voxel::pressure  VX_Voxel.h:103-104
  float pressure(const Voxel& v) const {
    const Material& m = vmats[v.mat];
    F3 st = voxel_strain(v, false);
    float vol = (float)(st.x + st.y + st.z);
    return -m.E * vol / (3 * (1 - 2 * m.nu));
  }
  // CVX_Link::strainEnergy  VX_Link.cpp:251-257
  float strain_energy(const Link& l) const {
    const Material& m = lmats[l.mat];
    return l.forceNeg.x * l.forceNeg.x / (2.0f * m.a1) + l.momentNeg.x * l.momentNeg.x / (2.0 * m.a2) +
           (l.momentNeg.z * l.momentNeg.z - l.momentNeg.z * l.momentPos.z + l.momentPos.z * l.momentPos.z) / (3.0 * m.b3) +
           (l.momentNeg.y * l.momentNeg.y - l.momentNeg.y * l.momentPos.y + l.momentPos.y * l.momentPos.y) / (3.0 * m.b3);
  }

  float state_info(int info, int type) {  // Voxelyze.cpp:752-800
    float r = 0;
    if (type == 1) r = -FLT_MAX;
    else if (type == 0) r = FLT_MAX;
    auto acc = [&](float t) {
      switch (type) {
        case 0: if (t < r) r = t; break;
        case 1: if (t > r) r = t; break;
        default: r += t;
      }
    };
    if (info == 7 || info == 5 || info == 6) {
      if (links.empty()) return 0.0f;
      for (const Link& l : links) {
        float t = 0;
        const Material& m = lmats[l.mat];
        (void)m;
        if (info == 7) {
          t = strain_energy(l);
        } else if (info == 5) {
          t = l.stress;
        } else {
          t = l.strain;
        }
        acc(t);
      }
      if (type == 3) r /= links.size();
    } else {
      if (voxels.empty()) return 0.0f;
      for (const Voxel& v : voxels) {
        const Material& m = vmats[v.mat];
        float t = 0;
        double s = m.nomSize;
        switch (info) {
          case 0: {
            double dx = v.pos.x - v.ix * s, dy = v.pos.y - v.iy * s, dz = v.pos.z - v.iz * s;
            t = (float)std::sqrt(dx * dx + dy * dy + dz * dz);
            break;
          }
          case 1:
            t = (float)(std::sqrt(v.linMom.x * v.linMom.x + v.linMom.y * v.linMom.y + v.linMom.z * v.linMom.z) *
                        m.massInv);
            break;
          case 2:
            t = (float)(0.5 * (m.massInv * (v.linMom.x * v.linMom.x + v.linMom.y * v.linMom.y + v.linMom.z * v.linMom.z) +
                               m.inertiaInv * (v.angMom.x * v.angMom.x + v.angMom.y * v.angMom.y + v.angMom.z * v.angMom.z)));
            break;
          case 3:
          case 4: {
            if (info == 3) {
              double w = v.orient.w > 1 ? 1 : v.orient.w;
              t = (float)(2.0 * std::acos(w));
            } else {
              t = (float)(std::sqrt(v.angMom.x * v.angMom.x + v.angMom.y * v.angMom.y + v.angMom.z * v.angMom.z) *
                          m.inertiaInv);
            }
            break;
          }
          case 8: t = pressure(v); break;
          case 9: t = m.mass; break;
          default: t = 0;
        }
        acc(t);
      }
      if (type == 3) r /= voxels.size();
    }
    return r;
  }
};

}  // namespace vxo

using vxo::Sim;
static Sim* S(void* s) { return static_cast<Sim*>(s); }

extern "C" {

void* vxo_create(double voxel_size) { return new Sim(voxel_size); }
void vxo_destroy(void* s) { delete S(s); }

// CPU threads for the link and voxel loops (the reference's USE_OMP build); 1 = serial.
void vxo_set_threads(void* s, int n) { S(s)->nthreads = n < 1 ? 1 : n; }

// 0: sin/cos/acos from the C library (the reference's arithmetic); 1: correctly rounded.
void vxo_set_math(int mode) { vxo::g_math_mode = mode ? 1 : 0; }

// Evaluates the correctly rounded functions of vx_crmath.h on the host (fn 0 sin, 1 cos, 2 acos)
// so tests can check them against high-precision arithmetic.
void vxo_crmath_eval(int fn, int n, const double* x, double* y, int* flags) {
  for (int i = 0; i < n; ++i) {
    int f = 0;
    y[i] = fn == 0 ? vxm::cr_sin(x[i], &f) : (fn == 1 ? vxm::cr_cos(x[i], &f) : vxm::cr_acos(x[i], &f));
    if (flags) flags[i] = f;
  }
}

int vxo_add_material(void* s, float E, float rho) {  // Voxelyze.cpp:357-366
  Sim* r = S(s);
  vxo::Material m;
  m.rho = 1.0f;
  m.set_linear(1.0f, -1.0f);
  m.rho = rho;
  m.set_linear(E, -1.0f);
  m.nomSize = r->voxSize;
  m.gravMult = 0.0f;
  m.derive_voxel();
  m.gravMult = r->grav;
  r->vmats.push_back(m);
  return (int)r->vmats.size() - 1;
}

int vxo_material_set(void* s, int mat, int prop, float value) {
  Sim* r = S(s);
  if (mat < 0 || mat >= (int)r->vmats.size()) return -1;
  vxo::Material& m = r->vmats[mat];
  switch (prop) {
    case VXF_PROP_POISSON:  // VX_Material.cpp:472-478
      if (value < 0) value = 0;
      if (value >= 0.5) value = 0.5 - FLT_EPSILON * 2;
      m.nu = value;
      r->voxel_material_changed(mat);
      break;
    case VXF_PROP_CTE: m.alphaCTE = value; break;
    case VXF_PROP_MU_STATIC: m.muStatic = value <= 0 ? 0 : value; break;
    case VXF_PROP_MU_KINETIC: m.muKinetic = value <= 0 ? 0 : value; break;
    case VXF_PROP_ZETA_INTERNAL: m.zetaInternal = value <= 0 ? 0 : value; break;
    case VXF_PROP_ZETA_GLOBAL: m.zetaGlobal = value <= 0 ? 0 : value; break;
    case VXF_PROP_ZETA_COLLISION: m.zetaCollision = value <= 0 ? 0 : value; break;
    case VXF_PROP_DENSITY:
      if (value <= 0) value = FLT_MIN;
      m.rho = value;
      r->voxel_material_changed(mat);
      break;
    default: return -1;
  }
  return 0;
}
int vxo_material_set_model_linear(void* s, int mat, float E, float fail) {
  Sim* r = S(s);
  bool ok = r->vmats[mat].set_linear(E, fail);
  if (ok) r->voxel_material_changed(mat);
  return ok ? 0 : -1;
}
int vxo_material_set_model_bilinear(void* s, int mat, float E, float Ep, float ys, float fs) {
  Sim* r = S(s);
  bool ok = r->vmats[mat].set_bilinear(E, Ep, ys, fs);
  if (ok) r->voxel_material_changed(mat);
  return ok ? 0 : -1;
}
int vxo_material_set_model(void* s, int mat, int n, const float* strain, const float* stress) {
  Sim* r = S(s);
  bool ok = r->vmats[mat].set_model(n, strain, stress);
  if (ok) r->voxel_material_changed(mat);
  return ok ? 0 : -1;
}

float vxo_material_stress(void* s, int mat, float strain, float tss, int force_linear) {
  return S(s)->vmats[mat].stress(strain, tss, force_linear != 0);
}
float vxo_material_modulus(void* s, int mat, float strain) { return S(s)->vmats[mat].modulus(strain); }

int vxo_set_voxel(void* s, int mat, int x, int y, int z) {
  Sim* r = S(s);
  if (mat < 0 || mat >= (int)r->vmats.size()) return -1;
  return r->set_voxel(mat, x, y, z);
}
int vxo_remove_voxel(void* s, int x, int y, int z) {
  S(s)->set_voxel(-1, x, y, z);
  return 0;
}
int vxo_replace_material(void* s, int a, int b) {
  Sim* r = S(s);
  if (a < 0 || b < 0 || a >= (int)r->vmats.size() || b >= (int)r->vmats.size()) return -1;
  r->replace_material(a, b);
  return 0;
}
int vxo_remove_material(void* s, int m) {
  Sim* r = S(s);
  if (m < 0 || m >= (int)r->vmats.size()) return -1;
  r->remove_material(m);
  return 0;
}
void vxo_set_voxel_size(void* s, double size) { S(s)->set_voxel_size(size); }
int vxo_set_voxels(void* s, int n, const int* mat, const int* xyz) {
  for (int i = 0; i < n; ++i) vxo_set_voxel(s, mat[i], xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
  return 0;
}
int vxo_voxel_count(void* s) { return (int)S(s)->voxels.size(); }
int vxo_link_count(void* s) { return (int)S(s)->links.size(); }
int vxo_voxel_index(void* s, int x, int y, int z) { return S(s)->voxel_at(x, y, z); }

static bool valid(void* s, int v) { return v >= 0 && v < (int)S(s)->voxels.size(); }

int vxo_external_set_fixed(void* s, int v, int m) {  // VX_External.cpp:47-51 (no rotationChanged)
  if (!valid(s, v)) return -1;
  vxo::External& e = S(s)->ext_of(v);
  e.dof = (uint8_t)(m & 0x3F);
  e.translation = e.rotation = vxo::V3();
  return 0;
}
int vxo_external_set_displacement(void* s, int v, int dof, double d) {  // VX_External.cpp:53-66
  if (!valid(s, v)) return -1;
  vxo::External& e = S(s)->ext_of(v);
  e.dof |= (uint8_t)dof;
  if (d != 0.0f) {
    if (dof & 1) e.translation.x = d;
    if (dof & 2) e.translation.y = d;
    if (dof & 4) e.translation.z = d;
    if (dof & 8) e.rotation.x = d;
    if (dof & 16) e.rotation.y = d;
    if (dof & 32) e.rotation.z = d;
  }
  e.rotation_changed();
  return 0;
}
int vxo_external_clear_displacement(void* s, int v, int dof) {  // VX_External.cpp:77-89
  if (!valid(s, v)) return -1;
  vxo::External& e = S(s)->ext_of(v);
  e.dof &= (uint8_t)~dof;
  if (dof & 1) e.translation.x = 0.0;
  if (dof & 2) e.translation.y = 0.0;
  if (dof & 4) e.translation.z = 0.0;
  if (dof & 8) e.rotation.x = 0.0;
  if (dof & 16) e.rotation.y = 0.0;
  if (dof & 32) e.rotation.z = 0.0;
  e.rotation_changed();
  return 0;
}
int vxo_external_set_displacement_all(void* s, int v, const double* t, const double* rr) {  // :68-75
  if (!valid(s, v)) return -1;
  vxo::External& e = S(s)->ext_of(v);
  e.dof |= 0x3F;
  e.translation = vxo::v3(t[0], t[1], t[2]);
  e.rotation = vxo::v3(rr[0], rr[1], rr[2]);
  e.rotation_changed();
  return 0;
}
int vxo_external_set_fixed_all(void* s, int v, int fixed) {  // VX_External.h:60
  if (!valid(s, v)) return -1;
  if (fixed) {
    double z[3] = {0, 0, 0};
    return vxo_external_set_displacement_all(s, v, z, z);
  }
  vxo::External& e = S(s)->ext_of(v);  // clearDisplacementAll  VX_External.cpp:91-98
  e.dof &= (uint8_t)~0x3F;
  e.translation = e.rotation = vxo::V3();
  e.rotation_changed();
  return 0;
}
int vxo_external_set_force(void* s, int v, float fx, float fy, float fz) {
  if (!valid(s, v)) return -1;
  vxo::External& e = S(s)->ext_of(v);
  e.force.x = fx; e.force.y = fy; e.force.z = fz;
  return 0;
}
int vxo_external_set_moment(void* s, int v, float mx, float my, float mz) {
  if (!valid(s, v)) return -1;
  vxo::External& e = S(s)->ext_of(v);
  e.moment.x = mx; e.moment.y = my; e.moment.z = mz;
  return 0;
}

void vxo_set_gravity(void* s, float g) {  // Voxelyze.cpp:596-602
  S(s)->grav = g;
  for (auto& m : S(s)->vmats) m.gravMult = g;
}
void vxo_enable_floor(void* s, int e) {  // Voxelyze.cpp:604-610
  S(s)->floor = e != 0;
  for (auto& v : S(s)->voxels) v.floorEnabled = e != 0;
}
void vxo_enable_collisions(void* s, int e) {  // Voxelyze.cpp:612-622
  Sim* r = S(s);
  if (r->collisions == (e != 0)) return;
  r->collisions = e != 0;
  for (auto& v : r->voxels) v.collisionsEnabled = e != 0;
  if (!r->collisions) r->clear_collisions();
  r->collisionsStale = true;
}
void vxo_set_ambient_temperature(void* s, float t, int all) {  // Voxelyze.cpp:585-594
  S(s)->ambientTemp = t;
  if (all)
    for (int v = 0; v < (int)S(s)->voxels.size(); ++v) S(s)->set_temperature(v, t);
}
int vxo_voxel_set_temperature(void* s, int v, float t) {
  if (!valid(s, v)) return -1;
  S(s)->set_temperature(v, t);
  return 0;
}

int vxo_do_time_step(void* s, float dt) { return S(s)->do_time_step(dt) ? 1 : 0; }
int vxo_do_time_steps(void* s, int n, float dt) {
  for (int i = 0; i < n; ++i)
    if (!S(s)->do_time_step(dt)) return i;
  return n;
}
float vxo_recommended_time_step(void* s) { return S(s)->recommended_dt(); }
void vxo_reset_time(void* s) { S(s)->reset_time(); }
float vxo_current_time(void* s) { return S(s)->currentTime; }

int vxo_get_voxel_state(void* s, double* d, float* f, int* i) {
  Sim* r = S(s);
  for (size_t k = 0; k < r->voxels.size(); ++k) {
    const vxo::Voxel& p = r->voxels[k];
    if (d) {
      double* o = d + 13 * k;
      o[0] = p.pos.x; o[1] = p.pos.y; o[2] = p.pos.z;
      o[3] = p.linMom.x; o[4] = p.linMom.y; o[5] = p.linMom.z;
      o[6] = p.orient.w; o[7] = p.orient.x; o[8] = p.orient.y; o[9] = p.orient.z;
      o[10] = p.angMom.x; o[11] = p.angMom.y; o[12] = p.angMom.z;
    }
    if (f) {
      float* o = f + 5 * k;
      o[0] = p.temp; o[1] = p.previousDt; o[2] = p.pStrain.x; o[3] = p.pStrain.y; o[4] = p.pStrain.z;
    }
    if (i) {
      i[2 * k] = p.staticFriction ? 1 : 0;
      i[2 * k + 1] = p.pStrainInvalid ? 1 : 0;
    }
  }
  return (int)r->voxels.size();
}

int vxo_get_link_state(void* s, double* d, float* f, int* i) {
  Sim* r = S(s);
  for (size_t k = 0; k < r->links.size(); ++k) {
    const vxo::Link& p = r->links[k];
    if (d) {
      double* o = d + 22 * k;
      const vxo::V3* v[7] = {&p.pos2, &p.angle1v, &p.angle2v, &p.forceNeg, &p.forcePos, &p.momentNeg, &p.momentPos};
      for (int j = 0; j < 7; ++j) { o[3 * j] = v[j]->x; o[3 * j + 1] = v[j]->y; o[3 * j + 2] = v[j]->z; }
      o[21] = p.restLength;
    }
    if (f) {
      float* o = f + 6 * k;
      o[0] = p.strain; o[1] = p.maxStrain; o[2] = p.strainOffset; o[3] = p.stress;
      o[4] = p.transArea; o[5] = p.transStrainSum;
    }
    if (i) {
      int* o = i + 6 * k;
      o[0] = p.smallAngle; o[1] = p.localVelValid; o[2] = p.axis; o[3] = p.vneg; o[4] = p.vpos; o[5] = p.mat;
    }
  }
  return (int)r->links.size();
}

// ---- per-voxel and per-link queries ---------------------------------------------------------
static int put3(const vxo::F3& f, float* out) {
  out[0] = f.x; out[1] = f.y; out[2] = f.z;
  return 0;
}
static bool valid_link(void* s, int l) { return l >= 0 && l < (int)S(s)->links.size(); }
int vxo_voxel_external_force(void* s, int v, float* out3) {
  if (!valid(s, v)) return -1;
  const vxo::Voxel& x = S(s)->voxels[v];
  if (x.ext < 0) { out3[0] = out3[1] = out3[2] = 0.0f; return 0; }
  return put3(S(s)->external_force(x), out3);
}
int vxo_voxel_external_moment(void* s, int v, float* out3) {
  if (!valid(s, v)) return -1;
  const vxo::Voxel& x = S(s)->voxels[v];
  if (x.ext < 0) { out3[0] = out3[1] = out3[2] = 0.0f; return 0; }
  return put3(S(s)->external_moment(x), out3);
}
int vxo_voxel_corner_offset(void* s, int v, int corner, float* out3) {
  if (!valid(s, v) || corner < 0 || corner > 7) return -1;
  return put3(S(s)->corner_offset(S(s)->voxels[v], corner), out3);
}
int vxo_voxel_corner_position(void* s, int v, int corner, float* out3) {
  if (!valid(s, v) || corner < 0 || corner > 7) return -1;
  return put3(S(s)->corner_position(S(s)->voxels[v], corner), out3);
}
int vxo_voxel_force(void* s, int v, double* out3) {
  if (!valid(s, v)) return -1;
  vxo::V3 f = S(s)->voxel_force(S(s)->voxels[v]);
  out3[0] = f.x; out3[1] = f.y; out3[2] = f.z;
  return 0;
}
int vxo_voxel_moment(void* s, int v, double* out3) {
  if (!valid(s, v)) return -1;
  vxo::V3 f = S(s)->voxel_moment(S(s)->voxels[v]);
  out3[0] = f.x; out3[1] = f.y; out3[2] = f.z;
  return 0;
}
int vxo_voxel_is_yielded(void* s, int v) { return valid(s, v) ? (S(s)->voxel_yielded(S(s)->voxels[v]) ? 1 : 0) : -1; }
int vxo_voxel_is_failed(void* s, int v) { return valid(s, v) ? (S(s)->voxel_failed(S(s)->voxels[v]) ? 1 : 0) : -1; }
float vxo_voxel_pressure(void* s, int v) { return valid(s, v) ? S(s)->pressure(S(s)->voxels[v]) : 0.0f; }
float vxo_link_strain_energy(void* s, int l) { return valid_link(s, l) ? S(s)->strain_energy(S(s)->links[l]) : 0.0f; }
int vxo_link_is_yielded(void* s, int l) { return valid_link(s, l) ? (S(s)->link_yielded(l) ? 1 : 0) : -1; }
int vxo_link_is_failed(void* s, int l) { return valid_link(s, l) ? (S(s)->link_failed(l) ? 1 : 0) : -1; }

int vxo_get_collisions(void* s, int* pairs, int cap) {
  Sim* r = S(s);
  int n = (int)r->cols.size();
  for (int k = 0; k < n && k < cap; ++k) {
    pairs[2 * k] = r->cols[k].v1;
    pairs[2 * k + 1] = r->cols[k].v2;
  }
  return n;
}

float vxo_state_info(void* s, int info, int type) { return S(s)->state_info(info, type); }

}  // extern "C"
