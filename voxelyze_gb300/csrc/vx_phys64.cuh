// FP64 time-step physics for sm_103a, one thread per link / per voxel, structure-of-arrays state.
//
// Every function restates one routine of the reference with the same float/double promotions and
// the same operation order (the FP64 path is bit-faithful; build with -fmad=false so no a*b+c is
// contracted).  Transcendental functions are the correctly rounded ones of vx_crmath.h; powf for
// the Poisson term is read from a table the host filled with the C library's powf.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

#include "vx_crmath.h"
#include "vxg.h"

#if defined(__CUDACC__)
#define VX_HD __host__ __device__ __forceinline__
#define VX_HDN __host__ __device__
#else
#define VX_HD inline
#define VX_HDN inline
#endif

namespace vx64 {

VX_HD void atomic_add_u64(unsigned long long* p, unsigned long long v) {
#if defined(__CUDA_ARCH__)
  atomicAdd(p, v);
#else
  *p += v;
#endif
}
VX_HD unsigned float_bits(float x) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(x);
#else
  unsigned u;
  std::memcpy(&u, &x, 4);
  return u;
#endif
}

struct d3 {
  double x, y, z;
};
struct q4 {
  double w, x, y, z;
};
VX_HD d3 D3(double a, double b, double c) { d3 r; r.x = a; r.y = b; r.z = c; return r; }
VX_HD q4 Q4(double w, double x, double y, double z) { q4 q; q.w = w; q.x = x; q.y = y; q.z = z; return q; }

// device control block
struct Ctl {
  int diverged;         // set by the link pass of the current step when some strain > 100
  int halt;             // set by the voxel pass once a step diverged: later passes do nothing
  int steps;            // completed steps in this batch
  int status;           // device error bits
  unsigned maxf[2];     // recommendedTimeStep maximum (float bits), double-buffered by step parity
  int n_large;          // FP32C split link pass: links deferred to the general kernel this step
  int pad_;
  float time;           // CVoxelyze::currentTime
  float last_dt;
  float inv_last_dt;    // 1 / last_dt (IEEE division), for the FP32C link pass's local damping
  int pad2_;
  unsigned long long counters[VXG_C_COUNT];
};

// Structure-of-arrays view of the whole scene; multi-component arrays are component-major.
struct View {
  int nv, nl;
  const int* vmat;
  const int* vidx;     // 3 nv
  const int* vlinks;   // 6 nv
  const int* vext;
  uint32_t* vflags;
  double* pos;         // 3 nv
  double* linMom;      // 3 nv
  double* orient;      // 4 nv
  double* angMom;      // 3 nv
  float* temp;
  float* prevDt;
  float* pStrain;      // 3 nv
  const int* lvox;     // 2 nl
  const int* lmat;
  uint32_t* lflags;
  double* pos2;        // 3 nl
  double* a1v;         // 3 nl
  double* a2v;         // 3 nl
  double* fN;          // 3 nl
  double* fP;
  double* mN;
  double* mP;
  double* rest;        // nl
  float* strain;
  float* maxStrain;
  float* strainOffset;
  float* stress;
  float* strainRatio;
  float* tArea;
  float* tSS;
  const vxg_voxel_material* vm;
  const vxg_link_material* lm;
  const vxg_external* ext;
  const float* powtab; // slots of 2^24 floats
  // collisions: per voxel CSR of (collision index, sign) in ascending partner order
  const int* colOff;   // nv + 1
  const int* colItem;  // collision index * 2 + (voxel is the second of the pair)
  const float* colForce; // 3 per collision
  // collisions on: the voxel pass votes whether any surface voxel moved past the rebuild distance
  // from its position at the last rebuild (colLast), for the next step's collision stage (colVote
  // is null when collisions are off)
  int* colVote;
  const float* colLast;  // 3 nv
  double colRecalc2;     // rebuild distance squared
  double colS;           // voxel size (FP32C positions: lattice index * colS + displacement)
  Ctl* ctl;
};

VX_HD void count(const View& S, int which, int flags) {
  atomic_add_u64(&S.ctl->counters[VXG_C_TRANSCENDENTAL], 1ull);
  if (flags & vxm::VXM_AMBIGUOUS) atomic_add_u64(&S.ctl->counters[VXG_C_AMBIGUOUS], 1ull);
  if (flags & vxm::VXM_LIBM_BAND) atomic_add_u64(&S.ctl->counters[VXG_C_LIBM_BAND], 1ull);
  (void)which;
}
VX_HD double c_sin(const View& S, double x) { int f = 0; double r = vxm::cr_sin(x, &f); count(S, 0, f); return r; }
VX_HD double c_cos(const View& S, double x) { int f = 0; double r = vxm::cr_cos(x, &f); count(S, 1, f); return r; }
VX_HD double c_acos(const View& S, double x) { int f = 0; double r = vxm::cr_acos(x, &f); count(S, 2, f); return r; }

// Quat3D::RotateVec3D  Quat3D.h:170-177
VX_HD d3 rotate(const q4& q, const d3& f) {
  double tw = f.x * q.x + f.y * q.y + f.z * q.z;
  double tx = f.x * q.w - f.y * q.z + f.z * q.y;
  double ty = f.x * q.z + f.y * q.w - f.z * q.x;
  double tz = -f.x * q.y + f.y * q.x + f.z * q.w;
  return D3(q.w * tx + q.x * tw + q.y * tz - q.z * ty, q.w * ty - q.x * tz + q.y * tw + q.z * tx,
            q.w * tz + q.x * ty - q.y * tx + q.z * tw);
}
// Quat3D::RotateVec3DInv  Quat3D.h:188-195
VX_HD d3 rotate_inv(const q4& q, const d3& f) {
  double tw = q.x * f.x + q.y * f.y + q.z * f.z;
  double tx = q.w * f.x - q.y * f.z + q.z * f.y;
  double ty = q.w * f.y + q.x * f.z - q.z * f.x;
  double tz = q.w * f.z - q.x * f.y + q.y * f.x;
  return D3(tw * q.x + tx * q.w + ty * q.z - tz * q.y, tw * q.y - tx * q.z + ty * q.w + tz * q.x,
            tw * q.z + tx * q.y - ty * q.x + tz * q.w);
}
// Quat3D::operator*  Quat3D.h:83
VX_HD q4 qmul(const q4& a, const q4& f) {
  return Q4(a.w * f.w - a.x * f.x - a.y * f.y - a.z * f.z, a.w * f.x + a.x * f.w + a.y * f.z - a.z * f.y,
            a.w * f.y - a.x * f.z + a.y * f.w + a.z * f.x, a.w * f.z + a.x * f.y - a.y * f.x + a.z * f.w);
}
// Quat3D::ToRotationVector  Quat3D.h:117-122
VX_HD d3 to_rotation_vector(const View& S, const q4& q) {
  if (q.w >= 1.0 || q.w <= -1.0) return D3(0, 0, 0);
  double sl = 1.0 - q.w * q.w;
  if (sl < 2.4e-3) {
    double s = sqrt((2 - 2 * q.w) / sl);
    return D3(s * (2.0 * q.x), s * (2.0 * q.y), s * (2.0 * q.z));
  }
  double a = c_acos(S, q.w);
  double inv = 1.0 / sqrt(sl);
  return D3(inv * (a * (2.0 * q.x)), inv * (a * (2.0 * q.y)), inv * (a * (2.0 * q.z)));
}
// Quat3D::FromRotationVector  Quat3D.h:124-139
VX_HD q4 from_rotation_vector(const View& S, const d3& in) {
  d3 th = D3(0.5 * in.x, 0.5 * in.y, 0.5 * in.z);
  double m2 = th.x * th.x + th.y * th.y + th.z * th.z;
  double w, s;
  if (m2 * m2 < 5.328e-15) {
    w = 1.0 - 0.5 * m2;
    s = 1.0 - m2 / 6.0;
  } else {
    double m = sqrt(m2);
    w = c_cos(S, m);
    s = c_sin(S, m) / m;
  }
  return Q4(w, th.x * s, th.y * s, th.z * s);
}
// Quat3D::FromAngleToPosX  Quat3D.h:141-166 (q untouched for a zero vector)
VX_HD void from_angle_to_pos_x(const View& S, q4& q, const d3& r) {
  if (r.x == 0 && r.y == 0 && r.z == 0) return;
  double yx = r.y / r.x, zx = r.z / r.x;
  if (yx < 1.732e-2 && yx > -1.732e-2 && zx < 1.732e-2 && zx > -1.732e-2) {
    q.x = 0;
    q.y = 0.5 * zx;
    q.z = -0.5 * yx;
    q.w = 1 + 0.5 * (-q.y * q.y - q.z * q.z);
    return;
  }
  d3 n = r;
  double l = sqrt(n.x * n.x + n.y * n.y + n.z * n.z);
  if (l > 0) {
    double li = 1.0 / l;
    n.x *= li; n.y *= li; n.z *= li;
  }
  double theta = c_acos(S, n.x);
  if (theta > 3.14159265358979 - 1e-7) {
    q = Q4(0, 0, 1, 0);
    return;
  }
  double ami = 1.0 / sqrt(n.z * n.z + n.y * n.y);
  double a = 0.5 * theta;
  double s = c_sin(S, a);
  q.w = c_cos(S, a);
  q.x = 0;
  q.y = n.z * ami * s;
  q.z = -n.y * ami * s;
}

VX_HD d3 ld3(const double* p, int n, int i) { return D3(p[i], p[n + i], p[2 * n + i]); }
VX_HD void st3(double* p, int n, int i, const d3& v) { p[i] = v.x; p[n + i] = v.y; p[2 * n + i] = v.z; }
VX_HD q4 ldq(const double* p, int n, int i) { return Q4(p[i], p[n + i], p[2 * n + i], p[3 * n + i]); }
VX_HD void stq(double* p, int n, int i, const q4& q) { p[i] = q.w; p[n + i] = q.x; p[2 * n + i] = q.y; p[3 * n + i] = q.z; }

// CVX_Material::stress  VX_Material.cpp:165-195
VX_HD float mat_stress(const vxg_link_material& m, float strain, float tss, bool forceLinear) {
  if (m.epsilonFail != -1.0f && strain > m.epsilonFail) return 0.0f;
  if (strain <= m.strain[1] || m.linear || forceLinear) {
    if (m.nu == 0.0f) return m.E * strain;
    return m.eHat * ((1 - m.nu) * strain + m.nu * tss);
  }
  int n = m.ndata;
  for (int i = 2; i < n; ++i) {
    if (strain <= m.strain[i] || i == n - 1) {
      float perc = (strain - m.strain[i - 1]) / (m.strain[i] - m.strain[i - 1]);
      float basic = m.stress[i - 1] + perc * (m.stress[i] - m.stress[i - 1]);
      if (m.nu == 0.0f) return basic;
      float mod = (m.stress[i] - m.stress[i - 1]) / (m.strain[i] - m.strain[i - 1]);
      float modHat = mod / ((1 - 2 * m.nu) * (1 + m.nu));
      float effStrain = basic / mod;
      float effTss = tss * (effStrain / strain);
      return modHat * ((1 - m.nu) * effStrain + m.nu * effTss);
    }
  }
  return 0.0f;
}

// powf(x, e) as the host C library computes it: tabulated over [0.5, 2); outside that range the
// value is evaluated in double and rounded once (counted as a table miss).
VX_HD float lib_powf(const View& S, int slot, float x, float e) {
  unsigned b = float_bits(x);
  unsigned lo = 0x3F000000u;  // 0.5f
  if (slot >= 0 && b >= lo && b < 0x40000000u) return S.powtab[(size_t)slot * (1u << 24) + (b - lo)];
  atomic_add_u64(&S.ctl->counters[VXG_C_POWF_MISS], 1ull);
  return (float)exp((double)e * log((double)x));
}

// CVX_Link::axialStrain(bool)  VX_Link.cpp:121-124
VX_HD float link_axial_strain(const View& S, int l, bool positiveEnd) {
  float s = S.strain[l], r = S.strainRatio[l];
  return positiveEnd ? 2.0f * s * r / (1.0f + r) : 2.0f * s / (1.0f + r);
}

// CVX_Voxel::strain(true)  VX_Voxel.cpp:300-334
// (the voxel's six link slots `lk`, in direction order, already loaded by the caller)
VX_HDN void poisson_strain_links(const View& S, int v, const int lk[6], float out[3]) {
  float s[3] = {0, 0, 0};
  int nb[3] = {0, 0, 0};
  for (int i = 0; i < 6; ++i) {
    int li = lk[i];
    if (li >= 0) {
      s[i / 2] += link_axial_strain(S, li, i % 2 == 1);
      nb[i / 2]++;
    }
  }
  bool tension[3];
  int ei = S.vext[v];
  for (int i = 0; i < 3; ++i) {
    if (nb[i] == 2) s[i] *= 0.5f;
    bool t = nb[i] == 2;
    if (!t && ei >= 0 && nb[i] == 1) {
      const vxg_external& e = S.ext[ei];
      t = (e.dof & (1 << i)) != 0 || e.force[i] != 0;
    }
    tension[i] = t;
  }
  if (!(tension[0] && tension[1] && tension[2])) {
    float add = 0;
    for (int i = 0; i < 3; ++i)
      if (tension[i]) add += s[i];
    const vxg_voxel_material& m = S.vm[S.vmat[v]];
    float value = lib_powf(S, m.powf_slot, 1.0f + add, -m.nu) - 1.0f;
    for (int i = 0; i < 3; ++i)
      if (!tension[i]) s[i] = value;
  }
  out[0] = s[0]; out[1] = s[1]; out[2] = s[2];
}
VX_HDN void poisson_strain(const View& S, int v, float out[3]) {
  int lk[6];
  for (int i = 0; i < 6; ++i) lk[i] = S.vlinks[i * S.nv + v];
  poisson_strain_links(S, v, lk, out);
}

// CVX_Voxel::baseSize(axis)  VX_Voxel.h:89
VX_HD double base_size(const View& S, int v, int axis) {
  const vxg_voxel_material& m = S.vm[S.vmat[v]];
  return m.size[axis] * (1 + S.temp[v] * m.alphaCTE);
}
// CVX_Voxel::baseSizeAverage  VX_Voxel.h:90
VX_HD double base_size_avg(const View& S, int v) {
  const vxg_voxel_material& m = S.vm[S.vmat[v]];
  float f = 1 + S.temp[v] * m.alphaCTE;
  return ((double)f * m.size[0] + (double)f * m.size[1] + (double)f * m.size[2]) / 3.0f;
}
// CVX_Voxel::transverseArea / transverseStrainSum  VX_Voxel.cpp:346-374 (cache already filled)
VX_HD float transverse_area(const View& S, int v, int axis) {
  const vxg_voxel_material& m = S.vm[S.vmat[v]];
  float size = (float)m.nomSize;
  if (m.nu == 0) return size * size;
  double px = S.pStrain[v], py = S.pStrain[S.nv + v], pz = S.pStrain[2 * S.nv + v];
  switch (axis) {
    case 0: return (float)(size * size * (1 + py) * (1 + pz));
    case 1: return (float)(size * size * (1 + px) * (1 + pz));
    default: return (float)(size * size * (1 + px) * (1 + py));
  }
}
VX_HD float transverse_strain_sum(const View& S, int v, int axis) {
  if (S.vm[S.vmat[v]].nu == 0) return 0;
  float px = S.pStrain[v], py = S.pStrain[S.nv + v], pz = S.pStrain[2 * S.nv + v];
  switch (axis) {
    case 0: return py + pz;
    case 1: return px + pz;
    default: return px + py;
  }
}

VX_HD d3 to_axis_x(int axis, const d3& v) {  // VX_Link.h:114
  return axis == 1 ? D3(v.y, -v.x, v.z) : (axis == 2 ? D3(v.z, v.y, -v.x) : v);
}
VX_HD q4 to_axis_x(int axis, const q4& q) {  // VX_Link.h:115
  return axis == 1 ? Q4(q.w, q.y, -q.x, q.z) : (axis == 2 ? Q4(q.w, q.z, q.y, -q.x) : q);
}
VX_HD d3 to_axis_original(int axis, const d3& v) {  // VX_Link.h:116
  return axis == 1 ? D3(-v.y, v.x, v.z) : (axis == 2 ? D3(-v.z, v.y, v.x) : v);
}

// CVX_Voxel::dampingMultiplier  VX_Voxel.h:130
VX_HD float damping_multiplier(const View& S, int v) {
  const vxg_voxel_material& m = S.vm[S.vmat[v]];
  return 2 * m.sqrtMass * m.zetaInternal / S.prevDt[v];
}

// CVX_Link::axialStiffness with its side effects  VX_Link.cpp:259-267, Voxelyze.cpp:291-297
VX_HD float link_freq2(const View& S, int l, int vn, int vp, int axis,
                                            const vxg_link_material& m) {
  float k;
  if (m.nu == 0.0f) {
    k = m.a1;
  } else {
    double rest = 0.5 * (base_size(S, vn, axis) + base_size(S, vp, axis));
    float ta = 0.5f * (transverse_area(S, vn, axis) + transverse_area(S, vp, axis));
    float ts = 0.5f * (transverse_strain_sum(S, vn, axis) + transverse_strain_sum(S, vp, axis));
    S.rest[l] = rest;
    S.tArea[l] = ta;
    S.tSS[l] = ts;
    k = (float)(m.eHat * ta / ((S.strain[l] + 1) * rest));
  }
  float m1 = S.vm[S.vmat[vn]].mass, m2 = S.vm[S.vmat[vp]].mass;
  return k / (m1 < m2 ? m1 : m2);
}

// CVX_Link::updateForces + orientLink + updateStrain  VX_Link.cpp:77-119, 149-249
VX_HDN void link_update(const View& S, int l) {
  const int nl = S.nl;
  uint32_t lf = S.lflags[l];
  int axis = (lf >> 8) & 3;
  bool smallAngle = lf & VXG_LF_SMALL_ANGLE;
  bool lvv = lf & VXG_LF_LOCAL_VEL_VALID;
  int vn = S.lvox[l], vp = S.lvox[nl + l];
  const vxg_link_material& m = S.lm[S.lmat[l]];
  double rest = S.rest[l];

  d3 oldPos2 = ld3(S.pos2, nl, l), oldA1 = ld3(S.a1v, nl, l), oldA2 = ld3(S.a2v, nl, l);
  d3 pn = ld3(S.pos, S.nv, vn), pp = ld3(S.pos, S.nv, vp);
  d3 pos2 = to_axis_x(axis, D3(pp.x - pn.x, pp.y - pn.y, pp.z - pn.z));
  q4 angle1 = to_axis_x(axis, ldq(S.orient, S.nv, vn));
  q4 angle2 = to_axis_x(axis, ldq(S.orient, S.nv, vp));
  q4 totalRot = Q4(angle1.w, -angle1.x, -angle1.y, -angle1.z);
  pos2 = rotate(totalRot, pos2);
  angle2 = qmul(totalRot, angle2);
  angle1 = Q4(1, 0, 0, 0);
  float smallTurn = (float)((fabs(pos2.z) + fabs(pos2.y)) / pos2.x);
  float extendPerc = (float)(fabs(1 - pos2.x / rest));
  const float HF = 1.2f, BEND = 0.05f, EXT = 0.50f;  // VX_Link.cpp:21-23
  if (!smallAngle && smallTurn < BEND && extendPerc < EXT) {
    smallAngle = true;
    lvv = false;
  } else if (smallAngle && (smallTurn > HF * BEND || extendPerc > HF * EXT)) {
    smallAngle = false;
    lvv = false;
  }
  if (smallAngle) {
    pos2.x -= rest;
  } else {
    from_angle_to_pos_x(S, angle1, pos2);
    angle2 = qmul(angle1, angle2);
    pos2 = D3(sqrt(pos2.x * pos2.x + pos2.y * pos2.y + pos2.z * pos2.z) - rest, 0, 0);
  }
  d3 a1v = to_rotation_vector(S, angle1);
  d3 a2v = to_rotation_vector(S, angle2);
  st3(S.pos2, nl, l, pos2);
  st3(S.a1v, nl, l, a1v);
  st3(S.a2v, nl, l, a2v);

  d3 dPos2 = D3(0.5 * (pos2.x - oldPos2.x), 0.5 * (pos2.y - oldPos2.y), 0.5 * (pos2.z - oldPos2.z));
  d3 dA1 = D3(0.5 * (a1v.x - oldA1.x), 0.5 * (a1v.y - oldA1.y), 0.5 * (a1v.z - oldA1.z));
  d3 dA2 = D3(0.5 * (a2v.x - oldA2.x), 0.5 * (a2v.y - oldA2.y), 0.5 * (a2v.z - oldA2.z));

  float tArea = S.tArea[l], tSS = S.tSS[l];
  if (!(m.nu == 0.0f) || tSS != 0) {
    tArea = 0.5f * (transverse_area(S, vn, axis) + transverse_area(S, vp, axis));
    tSS = 0.5f * (transverse_strain_sum(S, vn, axis) + transverse_strain_sum(S, vp, axis));
    S.tArea[l] = tArea;
    S.tSS[l] = tSS;
  }

  // updateStrain  VX_Link.cpp:220-249
  float axial = (float)(pos2.x / rest);
  float maxStrain = S.maxStrain[l], strainOffset = S.strainOffset[l], stress;
  if (m.linear) {
    if (axial > maxStrain) maxStrain = axial;
    stress = mat_stress(m, axial, tSS, false);
  } else if (axial > maxStrain) {
    maxStrain = axial;
    stress = mat_stress(m, axial, tSS, false);
    if (m.nu != 0.0f) strainOffset = maxStrain - mat_stress(m, axial, 0.0f, false) / (m.eHat * (1 - m.nu));
    else strainOffset = maxStrain - stress / m.E;
  } else {
    float rel = axial - strainOffset;
    if (m.nu != 0.0f) stress = mat_stress(m, rel, tSS, true);
    else stress = m.E * rel;
  }
  S.strain[l] = axial;
  S.maxStrain[l] = maxStrain;
  S.strainOffset[l] = strainOffset;
  S.stress[l] = stress;

  d3 fN, fP, mN, mP;
  if (m.epsilonFail != -1.0f && maxStrain > m.epsilonFail) {
    fN = fP = mN = mP = D3(0, 0, 0);
  } else {
    float b1 = m.b1, b2 = m.b2, b3 = m.b3, a2 = m.a2;
    fN = D3((double)(stress * tArea), b1 * pos2.y - b2 * (a1v.z + a2v.z), b1 * pos2.z + b2 * (a1v.y + a2v.y));
    fP = D3(-fN.x, -fN.y, -fN.z);
    mN = D3(a2 * (a2v.x - a1v.x), -b2 * pos2.z - b3 * (2 * a1v.y + a2v.y), b2 * pos2.y - b3 * (2 * a1v.z + a2v.z));
    mP = D3(a2 * (a1v.x - a2v.x), -b2 * pos2.z - b3 * (a1v.y + 2 * a2v.y), b2 * pos2.y - b3 * (a1v.z + 2 * a2v.z));
    if (lvv) {
      float sqA1 = m.sqA1, sqA2xIp = m.sqA2xIp, sqB1 = m.sqB1, sqB2xFMp = m.sqB2xFMp, sqB3xIp = m.sqB3xIp;
      d3 pc = D3(sqA1 * dPos2.x, sqB1 * dPos2.y - sqB2xFMp * (dA1.z + dA2.z), sqB1 * dPos2.z + sqB2xFMp * (dA1.y + dA2.y));
      float dmN = damping_multiplier(S, vn), dmP = damping_multiplier(S, vp);
      fN.x += dmN * pc.x; fN.y += dmN * pc.y; fN.z += dmN * pc.z;
      fP.x -= dmP * pc.x; fP.y -= dmP * pc.y; fP.z -= dmP * pc.z;
      double hN = 0.5 * dmN, hP = 0.5 * dmP;
      d3 tN = D3(-sqA2xIp * (dA2.x - dA1.x), sqB2xFMp * dPos2.z + sqB3xIp * (2 * dA1.y + dA2.y),
                 -sqB2xFMp * dPos2.y + sqB3xIp * (2 * dA1.z + dA2.z));
      d3 tP = D3(sqA2xIp * (dA2.x - dA1.x), sqB2xFMp * dPos2.z + sqB3xIp * (dA1.y + 2 * dA2.y),
                 -sqB2xFMp * dPos2.y + sqB3xIp * (dA1.z + 2 * dA2.z));
      mN.x -= hN * tN.x; mN.y -= hN * tN.y; mN.z -= hN * tN.z;
      mP.x -= hP * tP.x; mP.y -= hP * tP.y; mP.z -= hP * tP.z;
    } else {
      lvv = true;
    }
    if (!smallAngle) {
      fN = rotate_inv(angle1, fN);
      mN = rotate_inv(angle1, mN);
    }
    fP = rotate_inv(angle2, fP);
    mP = rotate_inv(angle2, mP);
    fN = to_axis_original(axis, fN);
    fP = to_axis_original(axis, fP);
    mN = to_axis_original(axis, mN);
    mP = to_axis_original(axis, mP);
  }
  st3(S.fN, nl, l, fN);
  st3(S.fP, nl, l, fP);
  st3(S.mN, nl, l, mN);
  st3(S.mP, nl, l, mP);
  uint32_t nf = (lf & ~3u) | (smallAngle ? VXG_LF_SMALL_ANGLE : 0u) | (lvv ? VXG_LF_LOCAL_VEL_VALID : 0u);
  S.lflags[l] = nf;
}

// CVX_Voxel::timeStep + force + moment + floorForce  VX_Voxel.cpp:162-298
// DEC 0 takes the floor-contact and static-friction decisions as the reference does.  DEC 1 also
// records them in *dec: bit 0 the voxel touches the floor (penetration >= 0), bit 1 static friction
// holds at the end of the step.  DEC 2 replays them from *dec instead of comparing, so a perturbed
// run follows the recorded run's branches (finite differences of the branch an adjoint
// differentiates); the forces are still evaluated from the perturbed state.
template <int DEC = 0>
VX_HDN void voxel_update(const View& S, int v, float dt, uint8_t* dec = nullptr) {
  const int nv = S.nv;
  S.prevDt[v] = dt;
  if (dt == 0.0f) return;
  const vxg_voxel_material& m = S.vm[S.vmat[v]];
  int ei = S.vext[v];
  const vxg_external* e = ei >= 0 ? &S.ext[ei] : nullptr;
  int ix = S.vidx[v], iy = S.vidx[nv + v], iz = S.vidx[2 * nv + v];
  if (e && (e->dof & 0x3F) == 0x3F) {
    double s = m.nomSize;
    st3(S.pos, nv, v, D3(ix * s + e->translation[0], iy * s + e->translation[1], iz * s + e->translation[2]));
    stq(S.orient, nv, v, Q4(e->rotq[0], e->rotq[1], e->rotq[2], e->rotq[3]));
    st3(S.linMom, nv, v, D3(0, 0, 0));
    st3(S.angMom, nv, v, D3(0, 0, 0));
    return;
  }
  uint32_t flags = S.vflags[v];
  d3 pos = ld3(S.pos, nv, v), lin = ld3(S.linMom, nv, v), ang = ld3(S.angMom, nv, v);
  q4 orient = ldq(S.orient, nv, v);
  int lk[6];
#pragma unroll
  for (int i = 0; i < 6; ++i) lk[i] = S.vlinks[i * nv + v];

  // force()  VX_Voxel.cpp:234-256
  d3 F = D3(0, 0, 0);
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    if (lk[i] < 0) continue;
    const double* src = (i & 1) ? S.fP : S.fN;
    F.x += src[lk[i]]; F.y += src[S.nl + lk[i]]; F.z += src[2 * S.nl + lk[i]];
  }
  F = rotate(orient, F);
  if (e) { F.x += e->force[0]; F.y += e->force[1]; F.z += e->force[2]; }
  {
    float c = m.zetaGlobal * m.c2xSqMxExS;
    F.x -= c * (m.massInv * lin.x);
    F.y -= c * (m.massInv * lin.y);
    F.z -= c * (m.massInv * lin.z);
  }
  F.z += -m.mass * 9.80665f * m.gravMult;
  if (flags & VXG_VF_COLLISIONS) {
    int b = S.colOff[v], en = S.colOff[v + 1];
    for (int k = b; k < en; ++k) {
      int it = S.colItem[k];
      int c = it >> 1;
      float fx = S.colForce[3 * c], fy = S.colForce[3 * c + 1], fz = S.colForce[3 * c + 2];
      if (it & 1) { fx = -fx; fy = -fy; fz = -fz; }
      F.x -= fx; F.y -= fy; F.z -= fz;
    }
  }
  d3 fric = F;
  bool floorOn = flags & VXG_VF_FLOOR;
  bool staticF = flags & VXG_VF_STATIC_FRICTION;
  // floorForce  VX_Voxel.cpp:274-298
  double bsa = base_size_avg(S, v);
  if (floorOn) {
    float pen = (float)(bsa / 2 - m.nomSize / 2 - pos.z);
    if (DEC == 2 ? (*dec & 1) != 0 : pen >= 0) {
      d3 vel = D3(m.massInv * lin.x, m.massInv * lin.y, m.massInv * lin.z);
      float normal = m.penetrationStiffness * pen;
      F.z += normal - (m.zetaCollision * m.c2xSqMxExS) * vel.z;
      if (staticF) {
        float surf = (float)(F.x * F.x + F.y * F.y);
        float fr = (m.muStatic * normal) * (m.muStatic * normal);
        if (DEC != 2 && surf > fr) staticF = false;
      } else {
        float k = m.muKinetic * normal;
        d3 h = D3(vel.x, vel.y, 0);
        double len = sqrt(h.x * h.x + h.y * h.y + h.z * h.z);
        if (len > 0) {
          double inv = 1.0 / len;
          h = D3(inv * h.x, inv * h.y, inv * h.z);
        }
        F.x -= k * h.x; F.y -= k * h.y; F.z -= k * h.z;
      }
    } else {
      staticF = false;
    }
  }
  fric = D3(F.x - fric.x, F.y - fric.y, F.z - fric.z);
  lin.x += dt * F.x; lin.y += dt * F.y; lin.z += dt * F.z;
  float dtm = dt * m.massInv;
  d3 tr = D3(dtm * lin.x, dtm * lin.y, dtm * lin.z);
  const bool contact = floorOn && (DEC == 2 ? (*dec & 1) != 0 : (float)(bsa / 2 - m.nomSize / 2 - pos.z) >= 0);
  if (contact) {
    double work = fric.x * tr.x + fric.y * tr.y;
    double hKe = 0.5 * m.massInv * (lin.x * lin.x + lin.y * lin.y);
    if (DEC == 2) staticF = (*dec & 2) != 0;
    else if (hKe + work <= 0) staticF = true;
    if (staticF) {
      lin.x = lin.y = 0;
      tr.x = tr.y = 0;
    }
  } else {
    staticF = false;
  }
  if (DEC == 1) *dec = (uint8_t)((contact ? 1 : 0) | (staticF ? 2 : 0));
  pos.x += tr.x; pos.y += tr.y; pos.z += tr.z;

  // moment()  VX_Voxel.cpp:258-271
  d3 M = D3(0, 0, 0);
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    if (lk[i] < 0) continue;
    const double* src = (i & 1) ? S.mP : S.mN;
    M.x += src[lk[i]]; M.y += src[S.nl + lk[i]]; M.z += src[2 * S.nl + lk[i]];
  }
  M = rotate(orient, M);
  if (e) { M.x += e->moment[0]; M.y += e->moment[1]; M.z += e->moment[2]; }
  {
    float c = m.zetaGlobal * m.c2xSqIxExSxSxS;
    M.x -= c * (m.inertiaInv * ang.x);
    M.y -= c * (m.inertiaInv * ang.y);
    M.z -= c * (m.inertiaInv * ang.z);
  }
  ang.x += dt * M.x; ang.y += dt * M.y; ang.z += dt * M.z;
  float dti = dt * m.inertiaInv;
  q4 dq = from_rotation_vector(S, D3(dti * ang.x, dti * ang.y, dti * ang.z));
  orient = qmul(dq, orient);
  if (e) {
    double s = m.nomSize;
    if (e->dof & 1) { pos.x = ix * s + e->translation[0]; lin.x = 0; }
    if (e->dof & 2) { pos.y = iy * s + e->translation[1]; lin.y = 0; }
    if (e->dof & 4) { pos.z = iz * s + e->translation[2]; lin.z = 0; }
    if (e->dof & 56) {
      if ((e->dof & 56) == 56) {
        orient = Q4(e->rotq[0], e->rotq[1], e->rotq[2], e->rotq[3]);
        ang = D3(0, 0, 0);
      } else {
        d3 r = to_rotation_vector(S, orient);
        if (e->dof & 8) { r.x = 0; ang.x = 0; }
        if (e->dof & 16) { r.y = 0; ang.y = 0; }
        if (e->dof & 32) { r.z = 0; ang.z = 0; }
        orient = from_rotation_vector(S, r);
      }
    }
  }
  st3(S.pos, nv, v, pos);
  st3(S.linMom, nv, v, lin);
  st3(S.angMom, nv, v, ang);
  stq(S.orient, nv, v, orient);
  S.vflags[v] = (flags & ~(uint32_t)VXG_VF_STATIC_FRICTION) | (staticF ? VXG_VF_STATIC_FRICTION : 0u) |
                VXG_VF_PSTRAIN_INVALID;
}

}  // namespace vx64
