// FP32-compensated time step (precision mode VXG_FP32C).
//
// Same algorithm and branch structure as the FP64 path (vx_phys64.cuh, which cites the reference
// routine by routine), with the bulk arithmetic in FP32 and accuracy won back where FP32 alone
// would lose it:
//   * position = exact lattice origin (ix, iy, iz) * voxel size + FP32 displacement d, updated each
//     step with Kahan compensation (true displacement = d - c);
//   * the link's relative pose is formed from displacement differences, never from absolute
//     positions; its axial extension is written so that no two nearly equal numbers are
//     subtracted: pos2.x - L = -2 s (y^2 + z^2) + (R d).x - (L - s) in the small-angle branch and
//     (|pos2|^2 - s^2) / (|pos2| + s) - (L - s) in the large-angle one, with the rest length held
//     as its offset from the nominal size (L - s, exactly 0 at zero temperature);
//   * link pose and rotation vectors are small quantities stored as such (extension, not length).
// Transcendental functions are the CUDA single-precision ones.  Errors against the FP64 path are
// measured, not bounded: tests/test_gpu_fp32c.py reports them per workload.
#pragma once
#include <cmath>
#include <cstdint>

#include "vx_phys64.cuh"

namespace vx32 {

struct f3 {
  float x, y, z;
};
struct q4 {
  float w, x, y, z;
};
VX_HD f3 F3(float a, float b, float c) { f3 r; r.x = a; r.y = b; r.z = c; return r; }
VX_HD q4 Q4(float w, float x, float y, float z) { q4 q; q.w = w; q.x = x; q.y = y; q.z = z; return q; }

// FP32 working state; everything else (topology, flags, float strain/temperature fields,
// materials, externals, control block) is the FP64 View's.
struct View {
  vx64::View B;     // shared arrays
  float4* P;        // nv records (d.x, d.y, d.z, 0): displacement d from the lattice origin
  float4* Q;        // nv records (w, x, y, z): orientation
  float* c;         // 3 nv Kahan compensation of d (true displacement = d - c)
  float* qc;        // 4 nv Kahan compensation of the orientation (true orientation = q - qc)
  float* lin;       // 3 nv linear momentum
  float* ang;       // 3 nv angular momentum
  float* pos2;      // 3 nl (x holds the extension pos2.x - L, as in the reference's state)
  float* a1v;       // 3 nl
  float* a2v;       // 3 nl
  float* fN;        // 3 nl
  float* fP;
  float* mN;
  float* mP;
  float* restDelta; // nl: rest length - nominal size
  int* large;       // nl: links the small-angle link pass deferred to the general one this step
  float s;          // nominal voxel size
};

VX_HD f3 ld3(const float* p, int n, int i) { return F3(p[i], p[n + i], p[2 * n + i]); }
VX_HD void st3(float* p, int n, int i, const f3& v) { p[i] = v.x; p[n + i] = v.y; p[2 * n + i] = v.z; }
VX_HD q4 ldq(const float* p, int n, int i) { return Q4(p[i], p[n + i], p[2 * n + i], p[3 * n + i]); }
VX_HD void stq(float* p, int n, int i, const q4& q) { p[i] = q.w; p[n + i] = q.x; p[2 * n + i] = q.y; p[3 * n + i] = q.z; }

VX_HD f3 rotate(const q4& q, const f3& f) {
  float tw = f.x * q.x + f.y * q.y + f.z * q.z;
  float tx = f.x * q.w - f.y * q.z + f.z * q.y;
  float ty = f.x * q.z + f.y * q.w - f.z * q.x;
  float tz = -f.x * q.y + f.y * q.x + f.z * q.w;
  return F3(q.w * tx + q.x * tw + q.y * tz - q.z * ty, q.w * ty - q.x * tz + q.y * tw + q.z * tx,
            q.w * tz + q.x * ty - q.y * tx + q.z * tw);
}
VX_HD f3 rotate_inv(const q4& q, const f3& f) {
  float tw = q.x * f.x + q.y * f.y + q.z * f.z;
  float tx = q.w * f.x - q.y * f.z + q.z * f.y;
  float ty = q.w * f.y + q.x * f.z - q.z * f.x;
  float tz = q.w * f.z - q.x * f.y + q.y * f.x;
  return F3(tw * q.x + tx * q.w + ty * q.z - tz * q.y, tw * q.y - tx * q.z + ty * q.w + tz * q.x,
            tw * q.z + tx * q.y - ty * q.x + tz * q.w);
}
VX_HD q4 qmul(const q4& a, const q4& f) {
  return Q4(a.w * f.w - a.x * f.x - a.y * f.y - a.z * f.z, a.w * f.x + a.x * f.w + a.y * f.z - a.z * f.y,
            a.w * f.y - a.x * f.z + a.y * f.w + a.z * f.x, a.w * f.z + a.x * f.y - a.y * f.x + a.z * f.w);
}
VX_HD f3 to_rotation_vector(const q4& q) {
  // In FP32, w = cos(angle/2) rounds to exactly 1 for angles below ~5e-4 rad, so the FP64 test
  // "w >= 1 means no rotation" would drop every small relative rotation; the vector part decides.
  // |v| = sin(angle/2) comes from the vector part: no cancellation for w close to 1.
  float sl = q.x * q.x + q.y * q.y + q.z * q.z;
  if (sl <= 0.0f) return F3(0, 0, 0);
  if (q.w > 0.0f) {
    // small rotations (all but a few links): with r = |v| / w, angle / |v| = 2 atan(r) / (r w)
    // = (2 / w)(1 - r^2/3 + r^4/5 - ...); for r^2 < 1e-4 the next term is below 2e-13
    const float iw = 1.0f / q.w, r2 = sl * iw * iw;
    if (r2 < 1e-4f) {
      const float k = 2.0f * iw * (1.0f - r2 * (1.0f / 3.0f) + r2 * r2 * 0.2f);
      return F3(k * q.x, k * q.y, k * q.z);
    }
  }
  float vl = sqrtf(sl);
  float ang = 2.0f * atan2f(vl, q.w);  // same angle as 2 acos(w) on a unit quaternion
  float k = ang / vl;
  return F3(k * q.x, k * q.y, k * q.z);
}
VX_HD q4 from_rotation_vector(const f3& in) {
  f3 th = F3(0.5f * in.x, 0.5f * in.y, 0.5f * in.z);
  float m2 = th.x * th.x + th.y * th.y + th.z * th.z;
  float w, s;
  if (m2 < 1e-6f) {  // Taylor terms beyond m^4 are below FP32 resolution here
    w = 1.0f - 0.5f * m2 + m2 * m2 * (1.0f / 24.0f);
    s = 1.0f - m2 * (1.0f / 6.0f) + m2 * m2 * (1.0f / 120.0f);
  } else {
    float m = sqrtf(m2);
    w = cosf(m);
    s = sinf(m) / m;
  }
  return Q4(w, th.x * s, th.y * s, th.z * s);
}
// The same rotation as from_rotation_vector, returned as its difference from the identity quaternion
// (w - 1, x, y, z): the orientation update q' = dq q is then q + (dq - 1) q, a small increment that
// is added with compensation.  w - 1 is formed without cancellation.
VX_HD q4 rotation_increment(const f3& in) {
  f3 th = F3(0.5f * in.x, 0.5f * in.y, 0.5f * in.z);
  float m2 = th.x * th.x + th.y * th.y + th.z * th.z;
  float wm1, s;
  if (m2 < 1e-6f) {
    wm1 = -0.5f * m2 + m2 * m2 * (1.0f / 24.0f);
    s = 1.0f - m2 * (1.0f / 6.0f) + m2 * m2 * (1.0f / 120.0f);
  } else {
    float m = sqrtf(m2);
    float h = sinf(0.5f * m);
    wm1 = -2.0f * h * h;  // cos m - 1
    s = sinf(m) / m;
  }
  return Q4(wm1, th.x * s, th.y * s, th.z * s);
}
VX_HD void from_angle_to_pos_x(q4& q, const f3& r) {
  if (r.x == 0 && r.y == 0 && r.z == 0) return;
  float yx = r.y / r.x, zx = r.z / r.x;
  if (yx < 1.732e-2f && yx > -1.732e-2f && zx < 1.732e-2f && zx > -1.732e-2f) {
    q.x = 0;
    q.y = 0.5f * zx;
    q.z = -0.5f * yx;
    q.w = 1 + 0.5f * (-q.y * q.y - q.z * q.z);
    return;
  }
  float l = sqrtf(r.x * r.x + r.y * r.y + r.z * r.z);
  f3 n = F3(r.x / l, r.y / l, r.z / l);
  float t = sqrtf(n.z * n.z + n.y * n.y);
  float theta = atan2f(t, n.x);
  if (theta > 3.14159265358979f - 1e-7f) {
    q = Q4(0, 0, 1, 0);
    return;
  }
  float a = 0.5f * theta;
  float s = sinf(a) / t;
  q.w = cosf(a);
  q.x = 0;
  q.y = n.z * s;
  q.z = -n.y * s;
}
VX_HD f3 to_axis_x(int axis, const f3& v) { return axis == 1 ? F3(v.y, -v.x, v.z) : (axis == 2 ? F3(v.z, v.y, -v.x) : v); }
VX_HD q4 to_axis_x(int axis, const q4& q) { return axis == 1 ? Q4(q.w, q.y, -q.x, q.z) : (axis == 2 ? Q4(q.w, q.z, q.y, -q.x) : q); }
VX_HD f3 to_axis_original(int axis, const f3& v) { return axis == 1 ? F3(-v.y, v.x, v.z) : (axis == 2 ? F3(-v.z, v.y, v.x) : v); }

// rest length offset L - s of a link from the two voxels' temperatures (CTE expansion)
VX_HD float rest_delta(const View& S, int vn, int vp, int axis) {
  const vxg_voxel_material& a = S.B.vm[S.B.vmat[vn]];
  const vxg_voxel_material& b = S.B.vm[S.B.vmat[vp]];
  float ea = a.sizeF[axis] * (S.B.temp[vn] * a.alphaCTE) + (a.sizeF[axis] - S.s);
  float eb = b.sizeF[axis] * (S.B.temp[vp] * b.alphaCTE) + (b.sizeF[axis] - S.s);
  return 0.5f * (ea + eb);
}
// CVX_Voxel::transverseArea in FP32 (the FP64 path's promotions would put double operations on
// GB300's slow FP64 pipe for every link)
VX_HD float transverse_area32(const vx64::View& B, int v, int axis) {
  const vxg_voxel_material& m = B.vm[B.vmat[v]];
  float size = m.nomSizeF;
  if (m.nu == 0) return size * size;
  float px = B.pStrain[v], py = B.pStrain[B.nv + v], pz = B.pStrain[2 * B.nv + v];
  switch (axis) {
    case 0: return size * size * (1 + py) * (1 + pz);
    case 1: return size * size * (1 + px) * (1 + pz);
    default: return size * size * (1 + px) * (1 + py);
  }
}

VX_HD float link_freq2(const View& S, int l, int vn, int vp, int axis, const vxg_link_material& m) {
  float k;
  if (m.nu == 0.0f) {
    k = m.a1;
  } else {
    float rd = rest_delta(S, vn, vp, axis);
    float ta = 0.5f * (transverse_area32(S.B, vn, axis) + transverse_area32(S.B, vp, axis));
    float ts = 0.5f * (vx64::transverse_strain_sum(S.B, vn, axis) + vx64::transverse_strain_sum(S.B, vp, axis));
    S.restDelta[l] = rd;
    S.B.tArea[l] = ta;
    S.B.tSS[l] = ts;
    k = m.eHat * ta / ((S.B.strain[l] + 1) * (S.s + rd));
  }
  float m1 = S.B.vm[S.B.vmat[vn]].mass, m2 = S.B.vm[S.B.vmat[vp]].mass;
  return k / (m1 < m2 ? m1 : m2);
}

// Everything the link pass reads for one link, gathered before any arithmetic: the link's own
// state, its endpoints' poses and materials and, where a material has Poisson's ratio != 0, their
// cached Poisson strains.  The one-thread-per-link kernel fills it straight from global memory;
// the pipelined kernel fills it from shared memory that cp.async staged one tile ahead.  Both then
// run link_compute, so their results are identical bit for bit.
struct LinkIn {
  uint32_t lf;           // link flags (axis, small angle, local velocity valid)
  int lmat;              // link material
  float rd;              // rest length - nominal size
  f3 oldPos2, oldA1, oldA2;
  float tArea, tSS, maxStrain, strainOffset;
  f3 dn, dp;             // endpoint displacements
  q4 qn, qp;             // endpoint orientations
  int vmn, vmp;          // endpoint voxel materials
  f3 psn, psp;           // endpoint Poisson strains (read only for materials with nu != 0)
};

VX_HD f3 f3_of(const float4& a) { return F3(a.x, a.y, a.z); }
VX_HD q4 q4_of(const float4& a) { return Q4(a.x, a.y, a.z, a.w); }

// CVX_Voxel::transverseArea / transverseStrainSum from a voxel's material and Poisson strain
VX_HD float transverse_area_of(const vxg_voxel_material& m, const f3& ps, int axis) {
  float size = m.nomSizeF;
  if (m.nu == 0) return size * size;
  switch (axis) {
    case 0: return size * size * (1 + ps.y) * (1 + ps.z);
    case 1: return size * size * (1 + ps.x) * (1 + ps.z);
    default: return size * size * (1 + ps.x) * (1 + ps.y);
  }
}
VX_HD float transverse_strain_sum_of(const vxg_voxel_material& m, const f3& ps, int axis) {
  if (m.nu == 0) return 0;
  switch (axis) {
    case 0: return ps.y + ps.z;
    case 1: return ps.x + ps.z;
    default: return ps.x + ps.y;
  }
}

// POIS: some voxel material has nu != 0 (otherwise no Poisson strain is ever read).
// link_gather_own loads the link's own state and endpoint ids, link_gather_ends the rest (rest
// length, endpoint poses, materials and Poisson caches).
template <bool POIS>
VX_HD void link_gather_own(const View& S, int l, LinkIn& in, int& vn, int& vp) {
  const vx64::View& B = S.B;
  const int nl = B.nl;
  in.lf = B.lflags[l];
  in.lmat = B.lmat[l];
  in.oldPos2 = ld3(S.pos2, nl, l);
  // a small-angle link's angle1 is the identity, so its stored rotation vector is zero
  // (CVX_Link::orientLink, src/VX_Link.cpp:101-111; a new link starts small-angle with zeros, :63-68)
  in.oldA1 = (in.lf & VXG_LF_SMALL_ANGLE) ? F3(0, 0, 0) : ld3(S.a1v, nl, l);
  in.oldA2 = ld3(S.a2v, nl, l);
  // the stored transverse terms are used only where the link material has nu == 0; otherwise
  // updateForces recomputes both before any use (src/VX_Link.cpp:160)
  if (!POIS || B.lm[in.lmat].nu == 0.0f) {
    in.tArea = B.tArea[l];
    in.tSS = B.tSS[l];
  } else {
    in.tArea = in.tSS = 0.0f;
  }
  in.maxStrain = B.maxStrain[l];
  in.strainOffset = B.strainOffset[l];
  vn = B.lvox[l];
  vp = B.lvox[nl + l];
}
// ACT: the voxels' temperatures were set for this step (in-step actuation): the rest length offset
// is recomputed from them here, as CVX_Link::updateRestLength does after setTemperature
// (src/VX_Link.cpp:137-140), instead of in a separate pass; the caller stores it.
template <bool POIS, bool ACT = false>
VX_HD void link_gather_ends(const View& S, int l, LinkIn& in, int vn, int vp) {
  const vx64::View& B = S.B;
  const int nv = B.nv;
  in.rd = ACT ? rest_delta(S, vn, vp, (in.lf >> 8) & 3) : S.restDelta[l];
  in.dn = f3_of(S.P[vn]);
  in.dp = f3_of(S.P[vp]);
  in.qn = q4_of(S.Q[vn]);
  in.qp = q4_of(S.Q[vp]);
  in.vmn = B.vmat[vn];
  in.vmp = B.vmat[vp];
  if (POIS) {
    in.psn = ld3(B.pStrain, nv, vn);
    in.psp = ld3(B.pStrain, nv, vp);
  } else {
    in.psn = in.psp = F3(0, 0, 0);
  }
}
template <bool POIS, bool ACT = false>
VX_HD LinkIn link_gather(const View& S, int l) {
  LinkIn in;
  int vn, vp;
  link_gather_own<POIS>(S, l, in, vn, vp);
  link_gather_ends<POIS, ACT>(S, l, in, vn, vp);
  return in;
}

// CVX_Link::updateForces + orientLink + updateStrain in FP32C for link l from its gathered inputs;
// writes the link's new state and returns the axial strain (the divergence test's value).
// ipdt is the reciprocal of every voxel's previous time step (the local damping divides by it).
// SMALL: the caller has seen the small-angle flag set.  The link's angle1 is then the identity and
// its rotation vector zero for the whole step, unless the hysteresis test below moves it to the
// large-angle branch: in that case nothing is written, *deferred is set, and the general form
// (SMALL = false) must process the link from the same inputs.  For a link that stays small-angle
// both forms evaluate the same expressions in the same order, so their results are bit-identical.
template <bool SMALL>
VX_HDN float link_compute_t(const View& S, int l, const LinkIn& in, float ipdt, bool* deferred) {
  const vx64::View& B = S.B;
  const int nl = B.nl;
  uint32_t lf = in.lf;
  int axis = (lf >> 8) & 3;
  bool smallAngle = SMALL || (lf & VXG_LF_SMALL_ANGLE);
  bool lvv = lf & VXG_LF_LOCAL_VEL_VALID;
  const vxg_link_material& m = B.lm[in.lmat];
  const float s = S.s;
  float rd = in.rd;
  float L = s + rd;

  const f3 oldPos2 = in.oldPos2, oldA1 = in.oldA1, oldA2 = in.oldA2;
  const f3 dn = in.dn, dp = in.dp;
  f3 del = to_axis_x(axis, F3(dp.x - dn.x, dp.y - dn.y, dp.z - dn.z));
  q4 a1 = to_axis_x(axis, in.qn);
  q4 a2 = to_axis_x(axis, in.qp);
  q4 tr = Q4(a1.w, -a1.x, -a1.y, -a1.z);
  f3 r = rotate(tr, del);
  // pos2 = s * R e_x + R del, R = rotation by tr; the x part is split off to avoid s - s
  float ex = -2.0f * s * (tr.y * tr.y + tr.z * tr.z) + r.x;  // pos2.x - s
  float py = 2.0f * s * (tr.x * tr.y + tr.w * tr.z) + r.y;
  float pz = 2.0f * s * (tr.x * tr.z - tr.w * tr.y) + r.z;
  q4 angle2 = qmul(tr, a2);
  q4 angle1 = Q4(1, 0, 0, 0);
  float px = s + ex;
  const float iL = 1.0f / L;  // one division for the two uses of the current length
  float extendPerc = fabsf((ex - rd) * iL);
  const float HF = 1.2f, BEND = 0.05f, EXT = 0.50f;
  // the bend (|pz| + |py|) / px against its two thresholds, compared as products where px > 0
  // (every link short of folding over); the quotient itself otherwise
  const float turn = fabsf(pz) + fabsf(py);
  bool bentBelow, bentAbove;
  if (px > 0.0f) {
    bentBelow = turn < BEND * px;
    bentAbove = turn > (HF * BEND) * px;
  } else {
    const float smallTurn = turn / px;
    bentBelow = smallTurn < BEND;
    bentAbove = smallTurn > HF * BEND;
  }
  if (SMALL) {
    if (bentAbove || extendPerc > HF * EXT) {
      *deferred = true;
      return 0.0f;
    }
  } else if (!smallAngle && bentBelow && extendPerc < EXT) {
    smallAngle = true;
    lvv = false;
  } else if (smallAngle && (bentAbove || extendPerc > HF * EXT)) {
    smallAngle = false;
    lvv = false;
  }
  f3 pos2;
  if (SMALL || smallAngle) {
    pos2 = F3(ex - rd, py, pz);
  } else {
    from_angle_to_pos_x(angle1, F3(px, py, pz));
    angle2 = qmul(angle1, angle2);
    float len = sqrtf(px * px + py * py + pz * pz);
    float lms = (ex * (2.0f * s + ex) + py * py + pz * pz) / (len + s);  // |pos2| - s
    pos2 = F3(lms - rd, 0, 0);
  }
  const f3 a1v = SMALL ? F3(0, 0, 0) : to_rotation_vector(angle1);  // the identity's rotation vector is +0
  f3 a2v = to_rotation_vector(angle2);
  st3(S.pos2, nl, l, pos2);
  if (!SMALL && !(smallAngle && (lf & VXG_LF_SMALL_ANGLE))) st3(S.a1v, nl, l, a1v);  // else zeros, already stored
  st3(S.a2v, nl, l, a2v);
  f3 dPos2 = F3(0.5f * (pos2.x - oldPos2.x), 0.5f * (pos2.y - oldPos2.y), 0.5f * (pos2.z - oldPos2.z));
  f3 dA1 = F3(0.5f * (a1v.x - oldA1.x), 0.5f * (a1v.y - oldA1.y), 0.5f * (a1v.z - oldA1.z));
  f3 dA2 = F3(0.5f * (a2v.x - oldA2.x), 0.5f * (a2v.y - oldA2.y), 0.5f * (a2v.z - oldA2.z));

  float tArea = in.tArea, tSS = in.tSS;
  const vxg_voxel_material& mn = B.vm[in.vmn];
  const vxg_voxel_material& mp = B.vm[in.vmp];
  if (!(m.nu == 0.0f) || tSS != 0) {
    tArea = 0.5f * (transverse_area_of(mn, in.psn, axis) + transverse_area_of(mp, in.psp, axis));
    tSS = 0.5f * (transverse_strain_sum_of(mn, in.psn, axis) + transverse_strain_sum_of(mp, in.psp, axis));
    B.tArea[l] = tArea;
    B.tSS[l] = tSS;
  }
  float axial = pos2.x * iL;
  float maxStrain = in.maxStrain, strainOffset = in.strainOffset, stress;
  if (m.linear) {
    if (axial > maxStrain) maxStrain = axial;
    stress = vx64::mat_stress(m, axial, tSS, false);
  } else if (axial > maxStrain) {
    maxStrain = axial;
    stress = vx64::mat_stress(m, axial, tSS, false);
    if (m.nu != 0.0f) strainOffset = maxStrain - vx64::mat_stress(m, axial, 0.0f, false) / (m.eHat * (1 - m.nu));
    else strainOffset = maxStrain - stress / m.E;
  } else {
    float rel = axial - strainOffset;
    if (m.nu != 0.0f) stress = vx64::mat_stress(m, rel, tSS, true);
    else stress = m.E * rel;
  }
  B.strain[l] = axial;
  // the plastic history and the flags change rarely: stored only when their bits change
  if (vx64::float_bits(maxStrain) != vx64::float_bits(in.maxStrain)) B.maxStrain[l] = maxStrain;
  if (vx64::float_bits(strainOffset) != vx64::float_bits(in.strainOffset)) B.strainOffset[l] = strainOffset;
  B.stress[l] = stress;

  f3 fN, fP, mN, mP;
  if (m.epsilonFail != -1.0f && maxStrain > m.epsilonFail) {
    fN = fP = mN = mP = F3(0, 0, 0);
  } else {
    float b1 = m.b1, b2 = m.b2, b3 = m.b3, a2c = m.a2;
    fN = F3(stress * tArea, b1 * pos2.y - b2 * (a1v.z + a2v.z), b1 * pos2.z + b2 * (a1v.y + a2v.y));
    fP = F3(-fN.x, -fN.y, -fN.z);
    mN = F3(a2c * (a2v.x - a1v.x), -b2 * pos2.z - b3 * (2 * a1v.y + a2v.y), b2 * pos2.y - b3 * (2 * a1v.z + a2v.z));
    mP = F3(a2c * (a1v.x - a2v.x), -b2 * pos2.z - b3 * (a1v.y + 2 * a2v.y), b2 * pos2.y - b3 * (a1v.z + 2 * a2v.z));
    if (lvv) {
      f3 pc = F3(m.sqA1 * dPos2.x, m.sqB1 * dPos2.y - m.sqB2xFMp * (dA1.z + dA2.z), m.sqB1 * dPos2.z + m.sqB2xFMp * (dA1.y + dA2.y));
      float dmN = 2 * mn.sqrtMass * mn.zetaInternal * ipdt, dmP = 2 * mp.sqrtMass * mp.zetaInternal * ipdt;
      fN.x += dmN * pc.x; fN.y += dmN * pc.y; fN.z += dmN * pc.z;
      fP.x -= dmP * pc.x; fP.y -= dmP * pc.y; fP.z -= dmP * pc.z;
      float hN = 0.5f * dmN, hP = 0.5f * dmP;
      f3 tN = F3(-m.sqA2xIp * (dA2.x - dA1.x), m.sqB2xFMp * dPos2.z + m.sqB3xIp * (2 * dA1.y + dA2.y),
                 -m.sqB2xFMp * dPos2.y + m.sqB3xIp * (2 * dA1.z + dA2.z));
      f3 tP = F3(m.sqA2xIp * (dA2.x - dA1.x), m.sqB2xFMp * dPos2.z + m.sqB3xIp * (dA1.y + 2 * dA2.y),
                 -m.sqB2xFMp * dPos2.y + m.sqB3xIp * (dA1.z + 2 * dA2.z));
      mN.x -= hN * tN.x; mN.y -= hN * tN.y; mN.z -= hN * tN.z;
      mP.x -= hP * tP.x; mP.y -= hP * tP.y; mP.z -= hP * tP.z;
    } else {
      lvv = true;
    }
    if (!SMALL && !smallAngle) {
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
  const uint32_t nf = (lf & ~3u) | (smallAngle ? VXG_LF_SMALL_ANGLE : 0u) | (lvv ? VXG_LF_LOCAL_VEL_VALID : 0u);
  if (nf != lf) B.lflags[l] = nf;
  return axial;
}
VX_HDN float link_compute(const View& S, int l, const LinkIn& in, float ipdt) {
  return link_compute_t<false>(S, l, in, ipdt, nullptr);
}

// ipdt: 1 / the dt every voxel stepped with last
template <bool POIS, bool ACT = false>
VX_HDN float link_update_ip(const View& S, int l, float ipdt) {
  const LinkIn in = link_gather<POIS, ACT>(S, l);
  if (ACT) S.restDelta[l] = in.rd;
  return link_compute(S, l, in, ipdt);
}
template <bool POIS, bool ACT = false>
VX_HDN float link_update(const View& S, int l) {
  return link_update_ip<POIS, ACT>(S, l, S.B.ctl->inv_last_dt);
}

// The small-angle form for link l whose flags lf the caller has read and found small-angle:
// gathers the rest of the link's inputs (its angle1v is zero and is not read) and computes it.
// Returns the axial strain, or sets *deferred (nothing written) if the link leaves the branch.
template <bool POIS>
VX_HDN float link_update_small(const View& S, int l, uint32_t lf, bool* deferred) {
  const vx64::View& B = S.B;
  const int nl = B.nl;
  LinkIn in;
  in.lf = lf;
  in.lmat = B.lmat[l];
  in.oldPos2 = ld3(S.pos2, nl, l);
  in.oldA1 = F3(0, 0, 0);
  in.oldA2 = ld3(S.a2v, nl, l);
  if (!POIS || B.lm[in.lmat].nu == 0.0f) {
    in.tArea = B.tArea[l];
    in.tSS = B.tSS[l];
  } else {
    in.tArea = in.tSS = 0.0f;
  }
  in.maxStrain = B.maxStrain[l];
  in.strainOffset = B.strainOffset[l];
  const int vn = B.lvox[l], vp = B.lvox[nl + l];
  link_gather_ends<POIS>(S, l, in, vn, vp);
  return link_compute_t<true>(S, l, in, B.ctl->inv_last_dt, deferred);
}


VX_HD void kahan_add(float& sum, float& comp, float x) {
  float y = x - comp;
  float t = sum + y;
  comp = (t - sum) - y;
  sum = t;
}

// What the voxel pass reads of the voxel itself: written only by voxel passes and host uploads,
// never by the link pass or the collision stage of the same step.
struct VoxIn {
  int vmat, ei;
  uint32_t flags;
  f3 d, c, lin, ang;
  q4 q, qc;
  int lk[6];
  float temp;
  int iz;
};
VX_HD void voxel_gather_own(const View& S, int v, VoxIn& in) {
  const vx64::View& B = S.B;
  const int nv = B.nv;
  in.vmat = B.vmat[v];
  in.ei = B.vext[v];
  in.flags = B.vflags[v];
  in.d = f3_of(S.P[v]);
  in.c = ld3(S.c, nv, v);
  in.lin = ld3(S.lin, nv, v);
  in.ang = ld3(S.ang, nv, v);
  in.q = q4_of(S.Q[v]);
  in.qc = ldq(S.qc, nv, v);
#pragma unroll
  for (int i = 0; i < 6; ++i) in.lk[i] = B.vlinks[i * nv + v];
  in.temp = B.temp[v];
  in.iz = B.vidx[2 * nv + v];
}

// FUSE_POIS: fill the Poisson-strain cache for the next step's link pass here, from this step's
// link strains (which no later kernel of the step changes), instead of in a separate pre-pass
// dOut / cOut (optional): the voxel's displacement and its compensation after the step.
template <bool FUSE_POIS>
VX_HDN void voxel_step(const View& S, int v, float dt, const VoxIn& in, f3* dOut = nullptr, f3* cOut = nullptr) {
  const vx64::View& B = S.B;
  const int nv = B.nv, nl = B.nl;
  if (dOut) { *dOut = in.d; *cOut = in.c; }
  if (dt == 0.0f) return;
  const vxg_voxel_material& m = B.vm[in.vmat];
  int ei = in.ei;
  const vxg_external* e = ei >= 0 ? &B.ext[ei] : nullptr;
  if (e && (e->dof & 0x3F) == 0x3F) {
    S.P[v] = make_float4((float)e->translation[0], (float)e->translation[1], (float)e->translation[2], 0.0f);
    st3(S.c, nv, v, F3(0, 0, 0));
    if (dOut) { *dOut = F3((float)e->translation[0], (float)e->translation[1], (float)e->translation[2]); *cOut = F3(0, 0, 0); }
    S.Q[v] = make_float4((float)e->rotq[0], (float)e->rotq[1], (float)e->rotq[2], (float)e->rotq[3]);
    stq(S.qc, nv, v, Q4(0, 0, 0, 0));
    st3(S.lin, nv, v, F3(0, 0, 0));
    st3(S.ang, nv, v, F3(0, 0, 0));
    return;
  }
  const uint32_t flags = in.flags;
  f3 d = in.d, c = in.c, lin = in.lin, ang = in.ang;
  q4 q = in.q, qc = in.qc;
  int lk[6];
#pragma unroll
  for (int i = 0; i < 6; ++i) lk[i] = in.lk[i];
  f3 F = F3(0, 0, 0);
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    if (lk[i] < 0) continue;
    const float* src = (i & 1) ? S.fP : S.fN;
    F.x += src[lk[i]]; F.y += src[nl + lk[i]]; F.z += src[2 * nl + lk[i]];
  }
  F = rotate(q, F);
  if (e) { F.x += e->force[0]; F.y += e->force[1]; F.z += e->force[2]; }
  {
    float cg = m.zetaGlobal * m.c2xSqMxExS;
    F.x -= cg * (m.massInv * lin.x);
    F.y -= cg * (m.massInv * lin.y);
    F.z -= cg * (m.massInv * lin.z);
  }
  F.z += -m.mass * 9.80665f * m.gravMult;
  if (flags & VXG_VF_COLLISIONS) {  // contact forces in the partner order of the contact list
    int b = B.colOff[v], en = B.colOff[v + 1];
    for (int k = b; k < en; ++k) {
      int it = B.colItem[k];
      int c = it >> 1;
      float fx = B.colForce[3 * c], fy = B.colForce[3 * c + 1], fz = B.colForce[3 * c + 2];
      if (it & 1) { fx = -fx; fy = -fy; fz = -fz; }
      F.x -= fx; F.y -= fy; F.z -= fz;
    }
  }
  f3 fric = F;
  bool floorOn = flags & VXG_VF_FLOOR;
  bool staticF = flags & VXG_VF_STATIC_FRICTION;
  // floor penetration: (base size - nominal)/2 - z, with z = iz s + d.z
  float expand = m.sizeAvgF * (1 + in.temp * m.alphaCTE) - m.nomSizeF;
  float zorg = (float)in.iz * S.s;
  float pen = (0.5f * expand - zorg) - (d.z - c.z);
  if (floorOn) {
    if (pen >= 0) {
      f3 vel = F3(m.massInv * lin.x, m.massInv * lin.y, m.massInv * lin.z);
      float normal = m.penetrationStiffness * pen;
      F.z += normal - (m.zetaCollision * m.c2xSqMxExS) * vel.z;
      if (staticF) {
        float surf = F.x * F.x + F.y * F.y;
        float fr = (m.muStatic * normal) * (m.muStatic * normal);
        if (surf > fr) staticF = false;
      } else {
        float k = m.muKinetic * normal;
        float len = sqrtf(vel.x * vel.x + vel.y * vel.y);
        if (len > 0) {
          F.x -= k * (vel.x / len);
          F.y -= k * (vel.y / len);
        }
      }
    } else {
      staticF = false;
    }
  }
  fric = F3(F.x - fric.x, F.y - fric.y, F.z - fric.z);
  lin.x += dt * F.x; lin.y += dt * F.y; lin.z += dt * F.z;
  float dtm = dt * m.massInv;
  f3 tr = F3(dtm * lin.x, dtm * lin.y, dtm * lin.z);
  if (floorOn && pen >= 0) {
    float work = fric.x * tr.x + fric.y * tr.y;
    float hKe = 0.5f * m.massInv * (lin.x * lin.x + lin.y * lin.y);
    if (hKe + work <= 0) staticF = true;
    if (staticF) {
      lin.x = lin.y = 0;
      tr.x = tr.y = 0;
    }
  } else {
    staticF = false;
  }
  kahan_add(d.x, c.x, tr.x);
  kahan_add(d.y, c.y, tr.y);
  kahan_add(d.z, c.z, tr.z);
  f3 M = F3(0, 0, 0);
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    if (lk[i] < 0) continue;
    const float* src = (i & 1) ? S.mP : S.mN;
    M.x += src[lk[i]]; M.y += src[nl + lk[i]]; M.z += src[2 * nl + lk[i]];
  }
  M = rotate(q, M);
  if (e) { M.x += e->moment[0]; M.y += e->moment[1]; M.z += e->moment[2]; }
  {
    float cg = m.zetaGlobal * m.c2xSqIxExSxSxS;
    M.x -= cg * (m.inertiaInv * ang.x);
    M.y -= cg * (m.inertiaInv * ang.y);
    M.z -= cg * (m.inertiaInv * ang.z);
  }
  ang.x += dt * M.x; ang.y += dt * M.y; ang.z += dt * M.z;
  float dti = dt * m.inertiaInv;
  {
    q4 dq = qmul(rotation_increment(F3(dti * ang.x, dti * ang.y, dti * ang.z)), q);
    kahan_add(q.w, qc.w, dq.w);
    kahan_add(q.x, qc.x, dq.x);
    kahan_add(q.y, qc.y, dq.y);
    kahan_add(q.z, qc.z, dq.z);
  }
  if (e) {
    if (e->dof & 1) { d.x = (float)e->translation[0]; c.x = 0; lin.x = 0; }
    if (e->dof & 2) { d.y = (float)e->translation[1]; c.y = 0; lin.y = 0; }
    if (e->dof & 4) { d.z = (float)e->translation[2]; c.z = 0; lin.z = 0; }
    if (e->dof & 56) {
      if ((e->dof & 56) == 56) {
        q = Q4((float)e->rotq[0], (float)e->rotq[1], (float)e->rotq[2], (float)e->rotq[3]);
        qc = Q4(0, 0, 0, 0);
        ang = F3(0, 0, 0);
      } else {
        f3 r = to_rotation_vector(q);
        if (e->dof & 8) { r.x = 0; ang.x = 0; }
        if (e->dof & 16) { r.y = 0; ang.y = 0; }
        if (e->dof & 32) { r.z = 0; ang.z = 0; }
        q = from_rotation_vector(r);
        qc = Q4(0, 0, 0, 0);
      }
    }
  }
  S.P[v] = make_float4(d.x, d.y, d.z, 0.0f);
  st3(S.c, nv, v, c);
  if (dOut) { *dOut = d; *cOut = c; }
  st3(S.lin, nv, v, lin);
  st3(S.ang, nv, v, ang);
  S.Q[v] = make_float4(q.w, q.x, q.y, q.z);
  stq(S.qc, nv, v, qc);
  uint32_t nf = (flags & ~(uint32_t)(VXG_VF_STATIC_FRICTION | VXG_VF_PSTRAIN_EAGER)) |
                (staticF ? VXG_VF_STATIC_FRICTION : 0u) | VXG_VF_PSTRAIN_INVALID;
  if (FUSE_POIS && m.nu != 0) {
    bool any = false;
#pragma unroll
    for (int i = 0; i < 6; ++i) any |= lk[i] >= 0;
    if (any) {
      float p[3];
      vx64::poisson_strain_links(B, v, lk, p);
      st3(B.pStrain, nv, v, F3(p[0], p[1], p[2]));
      nf = (nf & ~(uint32_t)VXG_VF_PSTRAIN_INVALID) | VXG_VF_PSTRAIN_EAGER;
    }
  }
  if (nf != flags) B.vflags[v] = nf;  // the flags change rarely (friction latch, Poisson cache state)
}
template <bool FUSE_POIS>
VX_HDN void voxel_update(const View& S, int v, float dt) {
  VoxIn in;
  voxel_gather_own(S, v, in);
  voxel_step<FUSE_POIS>(S, v, dt, in);
}

}  // namespace vx32
