// Reverse-mode derivatives of one FP64 time step (link pass + voxel pass), hand-written.
//
// Scope of the differentiated step: linear link materials with Poisson's ratio 0 and no failure
// strain, no voxel-voxel collisions; links in either branch of orientLink (VX_Link.cpp:77-119, the
// branch and its hysteresis taken as the forward pass took them); externals add forces and moments
// and fix any of the six degrees of freedom; floor contact and
// static/kinetic friction are differentiated along the branch the forward pass took
// (VX_Voxel.cpp:274-298 and the latch at :194-205).  Every forward quantity is recomputed here with
// the arithmetic of vx_phys64.cuh from the state recorded at the start of the step; the derivative
// of a float rounding is taken as 1.
//
// Conventions: g<name> is the adjoint (dJ/d<name>) of a forward quantity; *_adj functions ADD the
// adjoints of their inputs into the g arguments.
#pragma once
#include "vx_phys64.cuh"

namespace vxa {
using vx64::D3;
using vx64::d3;
using vx64::Q4;
using vx64::q4;

VX_HD void add(d3& a, const d3& b) { a.x += b.x; a.y += b.y; a.z += b.z; }
VX_HD void add(q4& a, const q4& b) { a.w += b.w; a.x += b.x; a.y += b.y; a.z += b.z; }
VX_HD double dot(const d3& a, const d3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
VX_HD d3 scale(double s, const d3& a) { return D3(s * a.x, s * a.y, s * a.z); }

// adjoint of vx64::rotate(q, f) (Quat3D::RotateVec3D, a quadratic form in q, linear in f)
VX_HD void rotate_adj(const q4& q, const d3& f, const d3& go, q4& gq, d3& gf) {
  double tw = f.x * q.x + f.y * q.y + f.z * q.z;
  double tx = f.x * q.w - f.y * q.z + f.z * q.y;
  double ty = f.x * q.z + f.y * q.w - f.z * q.x;
  double tz = -f.x * q.y + f.y * q.x + f.z * q.w;
  double gtw = q.x * go.x + q.y * go.y + q.z * go.z;
  double gtx = q.w * go.x + q.z * go.y - q.y * go.z;
  double gty = -q.z * go.x + q.w * go.y + q.x * go.z;
  double gtz = q.y * go.x - q.x * go.y + q.w * go.z;
  gq.w += tx * go.x + ty * go.y + tz * go.z;
  gq.x += tw * go.x - tz * go.y + ty * go.z;
  gq.y += tz * go.x + tw * go.y - tx * go.z;
  gq.z += -ty * go.x + tx * go.y + tw * go.z;
  gf.x += q.x * gtw + q.w * gtx + q.z * gty - q.y * gtz;
  gf.y += q.y * gtw - q.z * gtx + q.w * gty + q.x * gtz;
  gf.z += q.z * gtw + q.y * gtx - q.x * gty + q.w * gtz;
  gq.x += f.x * gtw - f.z * gty + f.y * gtz;
  gq.y += f.y * gtw + f.z * gtx - f.x * gtz;
  gq.z += f.z * gtw - f.y * gtx + f.x * gty;
  gq.w += f.x * gtx + f.y * gty + f.z * gtz;
}

// adjoint of vx64::rotate_inv(q, f) (Quat3D::RotateVec3DInv)
VX_HD void rotate_inv_adj(const q4& q, const d3& f, const d3& go, q4& gq, d3& gf) {
  double tw = q.x * f.x + q.y * f.y + q.z * f.z;
  double tx = q.w * f.x - q.y * f.z + q.z * f.y;
  double ty = q.w * f.y + q.x * f.z - q.z * f.x;
  double tz = q.w * f.z - q.x * f.y + q.y * f.x;
  double gtw = q.x * go.x + q.y * go.y + q.z * go.z;
  double gtx = q.w * go.x - q.z * go.y + q.y * go.z;
  double gty = q.z * go.x + q.w * go.y - q.x * go.z;
  double gtz = -q.y * go.x + q.x * go.y + q.w * go.z;
  gq.x += tw * go.x + tz * go.y - ty * go.z;
  gq.y += -tz * go.x + tw * go.y + tx * go.z;
  gq.z += ty * go.x - tx * go.y + tw * go.z;
  gq.w += tx * go.x + ty * go.y + tz * go.z;
  gq.x += f.x * gtw + f.z * gty - f.y * gtz;
  gq.y += f.y * gtw - f.z * gtx + f.x * gtz;
  gq.z += f.z * gtw + f.y * gtx - f.x * gty;
  gq.w += f.x * gtx + f.y * gty + f.z * gtz;
  gf.x += q.x * gtw + q.w * gtx - q.z * gty + q.y * gtz;
  gf.y += q.y * gtw + q.z * gtx + q.w * gty - q.x * gtz;
  gf.z += q.z * gtw - q.y * gtx + q.x * gty + q.w * gtz;
}

// adjoint of vx64::qmul(a, f) = a * f (Quat3D::operator*)
VX_HD void qmul_adj(const q4& a, const q4& f, const q4& gc, q4& ga, q4& gf) {
  ga.w += gc.w * f.w + gc.x * f.x + gc.y * f.y + gc.z * f.z;
  ga.x += -gc.w * f.x + gc.x * f.w - gc.y * f.z + gc.z * f.y;
  ga.y += -gc.w * f.y + gc.x * f.z + gc.y * f.w - gc.z * f.x;
  ga.z += -gc.w * f.z - gc.x * f.y + gc.y * f.x + gc.z * f.w;
  gf.w += gc.w * a.w + gc.x * a.x + gc.y * a.y + gc.z * a.z;
  gf.x += -gc.w * a.x + gc.x * a.w + gc.y * a.z - gc.z * a.y;
  gf.y += -gc.w * a.y - gc.x * a.z + gc.y * a.w + gc.z * a.x;
  gf.z += -gc.w * a.z + gc.x * a.y - gc.y * a.x + gc.z * a.w;
}

// Quat3D::ToRotationVector (Quat3D.h:117-122) without the transcendental counters; same values as
// vx64::to_rotation_vector.
VX_HD d3 rotation_vector(const q4& q) {
  if (q.w >= 1.0 || q.w <= -1.0) return D3(0, 0, 0);
  double sl = 1.0 - q.w * q.w;
  if (sl < 2.4e-3) {
    double s = sqrt((2 - 2 * q.w) / sl);
    return D3(s * (2.0 * q.x), s * (2.0 * q.y), s * (2.0 * q.z));
  }
  int f = 0;
  double a = vxm::cr_acos(q.w, &f);
  double inv = 1.0 / sqrt(sl);
  return D3(inv * (a * (2.0 * q.x)), inv * (a * (2.0 * q.y)), inv * (a * (2.0 * q.z)));
}
// Its adjoint.  r = k(w) (x, y, z): k = 2 sqrt((2 - 2w) / (1 - w^2)) = 2 sqrt(2 / (1 + w)) on the
// near-identity branch, k = 2 acos(w) / sqrt(1 - w^2) otherwise; k' is taken from the closed forms.
VX_HD void rotation_vector_adj(const q4& q, const d3& gr, q4& gq) {
  if (q.w >= 1.0 || q.w <= -1.0) return;
  double sl = 1.0 - q.w * q.w;
  double k, dk;
  if (sl < 2.4e-3) {
    k = 2.0 * sqrt((2 - 2 * q.w) / sl);
    dk = -k / (2.0 * (1.0 + q.w));
  } else {
    int f = 0;
    double a = vxm::cr_acos(q.w, &f);
    double inv = 1.0 / sqrt(sl);
    k = 2.0 * a * inv;
    dk = 2.0 * (q.w * a * inv - 1.0) / sl;
  }
  gq.x += k * gr.x;
  gq.y += k * gr.y;
  gq.z += k * gr.z;
  gq.w += dk * (q.x * gr.x + q.y * gr.y + q.z * gr.z);
}

// Quat3D::FromRotationVector (Quat3D.h:124-139) and its adjoint
VX_HD q4 from_rotation_vector(const d3& in) {
  d3 th = D3(0.5 * in.x, 0.5 * in.y, 0.5 * in.z);
  double m2 = th.x * th.x + th.y * th.y + th.z * th.z;
  double w, s;
  if (m2 * m2 < 5.328e-15) {
    w = 1.0 - 0.5 * m2;
    s = 1.0 - m2 / 6.0;
  } else {
    double m = sqrt(m2);
    int f = 0;
    w = vxm::cr_cos(m, &f);
    s = vxm::cr_sin(m, &f) / m;
  }
  return Q4(w, th.x * s, th.y * s, th.z * s);
}
VX_HD void from_rotation_vector_adj(const d3& in, const q4& gq, d3& gin) {
  d3 th = D3(0.5 * in.x, 0.5 * in.y, 0.5 * in.z);
  double m2 = th.x * th.x + th.y * th.y + th.z * th.z;
  double s, gm2;
  if (m2 * m2 < 5.328e-15) {
    s = 1.0 - m2 / 6.0;
    double gs = th.x * gq.x + th.y * gq.y + th.z * gq.z;
    gm2 = -0.5 * gq.w - gs / 6.0;
  } else {
    double m = sqrt(m2);
    double sn = sin(m), cs = cos(m);
    s = sn / m;
    double gs = th.x * gq.x + th.y * gq.y + th.z * gq.z;
    double gm = -sn * gq.w + (m * cs - sn) / m2 * gs;
    gm2 = gm / (2.0 * m);
  }
  d3 gth = D3(s * gq.x + 2.0 * th.x * gm2, s * gq.y + 2.0 * th.y * gm2, s * gq.z + 2.0 * th.z * gm2);
  gin.x += 0.5 * gth.x;
  gin.y += 0.5 * gth.y;
  gin.z += 0.5 * gth.z;
}

// to_axis_x / to_axis_original are signed permutations: each one's adjoint is the other.
VX_HD void to_axis_x_q_adj(int axis, const q4& g, q4& gq) {  // q' = to_axis_x(axis, q)
  gq.w += g.w;
  if (axis == 1) {         // q' = (w, y, -x, z)
    gq.y += g.x; gq.x -= g.y; gq.z += g.z;
  } else if (axis == 2) {  // q' = (w, z, y, -x)
    gq.z += g.x; gq.y += g.y; gq.x -= g.z;
  } else {
    gq.x += g.x; gq.y += g.y; gq.z += g.z;
  }
}

// ---- link ------------------------------------------------------------------------------------
// Inputs of one link's update: the two voxels' pose at the start of the step, the link's pose from
// the previous step, its rest length and flags, and the float material constants it reads.
struct LinkIn {
  d3 pn, pp;
  q4 qn, qp;
  d3 oldPos2, oldA1, oldA2;
  double rest;
  int axis;
  bool smallAngle, lvv;  // flags at the start of the step
  float E, a2, b1, b2, b3, sqA1, sqA2xIp, sqB1, sqB2xFMp, sqB3xIp, tArea;
  float dmN, dmP;        // damping multipliers 2 sqrt(m) zeta / previous dt of the two voxels
  float maxStrain;       // the largest axial strain so far (CVX_Link::maxStrain) at the step's start
  float epsilonFail;     // the material's failure strain, -1: none
  // Poisson's ratio of the link material and its eHat (nu = 0: the stored transverse area tArea is
  // used), and each end voxel's transverse data: its material's nominal size, whether that
  // material has nu != 0, and its Poisson strains this step (CVX_Voxel::poissonsStrain)
  float nu, eHat;
  float sizeN, sizeP;
  bool nuN, nuP;
  d3 psn, psp;
};
// CVX_Voxel::transverseArea / transverseStrainSum across the link's axis (vx64::transverse_area's
// and vx64::transverse_strain_sum's arithmetic) and their adjoints with respect to the Poisson strains
VX_HD float transverse_area_of(float size, bool hasNu, const d3& ps, int axis) {
  if (!hasNu) return size * size;
  switch (axis) {
    case 0: return (float)(size * size * (1 + ps.y) * (1 + ps.z));
    case 1: return (float)(size * size * (1 + ps.x) * (1 + ps.z));
    default: return (float)(size * size * (1 + ps.x) * (1 + ps.y));
  }
}
VX_HD float transverse_strain_sum_of(bool hasNu, const d3& ps, int axis) {
  if (!hasNu) return 0;
  const float px = (float)ps.x, py = (float)ps.y, pz = (float)ps.z;
  switch (axis) {
    case 0: return py + pz;
    case 1: return px + pz;
    default: return px + py;
  }
}
VX_HD void transverse_adj(float size, bool hasNu, const d3& ps, int axis, double gTA, double gTS, d3& gps) {
  if (!hasNu) return;
  const double s2 = (double)(size * size);
  switch (axis) {
    case 0: gps.y += gTA * s2 * (1 + ps.z) + gTS; gps.z += gTA * s2 * (1 + ps.y) + gTS; break;
    case 1: gps.x += gTA * s2 * (1 + ps.z) + gTS; gps.z += gTA * s2 * (1 + ps.x) + gTS; break;
    default: gps.x += gTA * s2 * (1 + ps.y) + gTS; gps.y += gTA * s2 * (1 + ps.x) + gTS;
  }
}
// the link's transverse area and strain sum this step (CVX_Link::updateTransverseInfo,
// VX_Link.cpp:142-147, for nu != 0; the stored area otherwise)
VX_HD void link_transverse(const LinkIn& in, float* tArea, float* tSS) {
  *tArea = in.tArea;
  *tSS = 0.0f;
  if (in.nu != 0.0f) {
    *tArea = 0.5f * (transverse_area_of(in.sizeN, in.nuN, in.psn, in.axis) +
                     transverse_area_of(in.sizeP, in.nuP, in.psp, in.axis));
    *tSS = 0.5f * (transverse_strain_sum_of(in.nuN, in.psn, in.axis) + transverse_strain_sum_of(in.nuP, in.psp, in.axis));
  }
}
// CVX_Material::stress for a linear material (vx64::mat_stress)
VX_HD float link_stress(const LinkIn& in, float strain, float tss) {
  if (in.epsilonFail != -1.0f && strain > in.epsilonFail) return 0.0f;
  if (in.nu == 0.0f) return in.E * strain;
  return in.eHat * ((1 - in.nu) * strain + in.nu * tss);
}
struct LinkOut {
  d3 fN, fP, mN, mP;     // in the voxels' frames, original axes (what the voxel pass gathers)
  d3 pos2, a1v, a2v;
  bool smallAngle, lvv, failed;
  float axial, stress, maxStrain;
};
// CVX_Link::updateStrain's history for a linear material and CVX_Link::isFailed
// (VX_Link.cpp:220-249, 149-217): the largest strain so far, and whether it passed the failure strain
VX_HD bool link_failed(const LinkIn& in, float axial, float* maxStrain) {
  float ms = in.maxStrain;
  if (axial > ms) ms = axial;
  *maxStrain = ms;
  return in.epsilonFail != -1.0f && ms > in.epsilonFail;
}

// CVX_Link::orientLink's large-angle frame (vx64::from_angle_to_pos_x, Quat3D::FromAngleToPosX,
// include/Quat3D.h:163-204): the rotation q that takes the link direction r onto +x
VX_HD void from_angle_to_pos_x(q4& q, const d3& r) {
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
  int f = 0;
  double theta = vxm::cr_acos(n.x, &f);
  if (theta > 3.14159265358979 - 1e-7) {
    q = Q4(0, 0, 1, 0);
    return;
  }
  double ami = 1.0 / sqrt(n.z * n.z + n.y * n.y);
  double a = 0.5 * theta;
  double s = vxm::cr_sin(a, &f);
  q.w = vxm::cr_cos(a, &f);
  q.x = 0;
  q.y = n.z * ami * s;
  q.z = -n.y * ami * s;
}
// Its adjoint with respect to r (the starting q is the identity), along the branch r takes; the
// antiparallel branch is a constant.
VX_HD void from_angle_to_pos_x_adj(const d3& r, const q4& gq, d3& gr) {
  if (r.x == 0 && r.y == 0 && r.z == 0) return;
  double yx = r.y / r.x, zx = r.z / r.x;
  if (yx < 1.732e-2 && yx > -1.732e-2 && zx < 1.732e-2 && zx > -1.732e-2) {
    const double qy = 0.5 * zx, qz = -0.5 * yx;
    const double gqy = gq.y - qy * gq.w, gqz = gq.z - qz * gq.w;  // w = 1 - (qy^2 + qz^2) / 2
    const double gzx = 0.5 * gqy, gyx = -0.5 * gqz;
    gr.y += gyx / r.x;
    gr.z += gzx / r.x;
    gr.x -= (gyx * r.y + gzx * r.z) / (r.x * r.x);
    return;
  }
  const double l = sqrt(r.x * r.x + r.y * r.y + r.z * r.z);
  const d3 n = D3(r.x / l, r.y / l, r.z / l);
  int f = 0;
  const double theta = vxm::cr_acos(n.x, &f);
  if (theta > 3.14159265358979 - 1e-7) return;
  const double ami = 1.0 / sqrt(n.z * n.z + n.y * n.y);
  const double a = 0.5 * theta, s = sin(a), c = cos(a);
  // q = (cos a, 0, u sin a, w sin a) with (u, w) = (n.z, -n.y) ami
  const double u = n.z * ami, w = -n.y * ami;
  const double gs = u * gq.y + w * gq.z;
  const double ga = -s * gq.w + c * gs;
  const double gu = s * gq.y, gw = s * gq.z;
  const double gtheta = 0.5 * ga;
  d3 gn = D3(-gtheta / sqrt(1.0 - n.x * n.x), 0, 0);
  const double gami = n.z * gu - n.y * gw;
  const double ami3 = ami * ami * ami;
  gn.z += ami * gu - n.z * ami3 * gami;
  gn.y += -ami * gw - n.y * ami3 * gami;
  // n = r / |r|
  const double ng = n.x * gn.x + n.y * gn.y + n.z * gn.z;
  gr.x += (gn.x - n.x * ng) / l;
  gr.y += (gn.y - n.y * ng) / l;
  gr.z += (gn.z - n.z * ng) / l;
}

// CVX_Link::updateForces for a linear, nu = 0, non-failing material (vx64::link_update's arithmetic)
VX_HD LinkOut link_forward(const LinkIn& in) {
  LinkOut o;
  d3 pos2 = vx64::to_axis_x(in.axis, D3(in.pp.x - in.pn.x, in.pp.y - in.pn.y, in.pp.z - in.pn.z));
  q4 angle1 = vx64::to_axis_x(in.axis, in.qn);
  q4 angle2 = vx64::to_axis_x(in.axis, in.qp);
  q4 totalRot = Q4(angle1.w, -angle1.x, -angle1.y, -angle1.z);
  pos2 = vx64::rotate(totalRot, pos2);
  angle2 = vx64::qmul(totalRot, angle2);
  angle1 = Q4(1, 0, 0, 0);
  bool smallAngle = in.smallAngle, lvv = in.lvv;
  float smallTurn = (float)((fabs(pos2.z) + fabs(pos2.y)) / pos2.x);
  float extendPerc = (float)(fabs(1 - pos2.x / in.rest));
  const float HF = 1.2f, BEND = 0.05f, EXT = 0.50f;
  if (!smallAngle && smallTurn < BEND && extendPerc < EXT) {
    smallAngle = true;
    lvv = false;
  } else if (smallAngle && (smallTurn > HF * BEND || extendPerc > HF * EXT)) {
    smallAngle = false;
    lvv = false;
  }
  o.smallAngle = smallAngle;
  const bool lvvBranch = lvv;  // the flag after the branch test, before the force terms set it
  if (smallAngle) {
    pos2.x -= in.rest;
  } else {
    from_angle_to_pos_x(angle1, pos2);
    angle2 = vx64::qmul(angle1, angle2);
    pos2 = D3(sqrt(pos2.x * pos2.x + pos2.y * pos2.y + pos2.z * pos2.z) - in.rest, 0, 0);
  }
  d3 a1v = rotation_vector(angle1);
  d3 a2v = rotation_vector(angle2);
  d3 dPos2 = D3(0.5 * (pos2.x - in.oldPos2.x), 0.5 * (pos2.y - in.oldPos2.y), 0.5 * (pos2.z - in.oldPos2.z));
  d3 dA1 = D3(0.5 * (a1v.x - in.oldA1.x), 0.5 * (a1v.y - in.oldA1.y), 0.5 * (a1v.z - in.oldA1.z));
  d3 dA2 = D3(0.5 * (a2v.x - in.oldA2.x), 0.5 * (a2v.y - in.oldA2.y), 0.5 * (a2v.z - in.oldA2.z));
  float tArea, tSS;
  link_transverse(in, &tArea, &tSS);
  float axial = (float)(pos2.x / in.rest);
  float stress = link_stress(in, axial, tSS);
  o.failed = link_failed(in, axial, &o.maxStrain);
  float b1 = in.b1, b2 = in.b2, b3 = in.b3, a2 = in.a2;
  d3 fN = D3((double)(stress * tArea), b1 * pos2.y - b2 * (a1v.z + a2v.z), b1 * pos2.z + b2 * (a1v.y + a2v.y));
  d3 fP = D3(-fN.x, -fN.y, -fN.z);
  d3 mN = D3(a2 * (a2v.x - a1v.x), -b2 * pos2.z - b3 * (2 * a1v.y + a2v.y), b2 * pos2.y - b3 * (2 * a1v.z + a2v.z));
  d3 mP = D3(a2 * (a1v.x - a2v.x), -b2 * pos2.z - b3 * (a1v.y + 2 * a2v.y), b2 * pos2.y - b3 * (a1v.z + 2 * a2v.z));
  if (lvv) {
    float sqA1 = in.sqA1, sqA2xIp = in.sqA2xIp, sqB1 = in.sqB1, sqB2xFMp = in.sqB2xFMp, sqB3xIp = in.sqB3xIp;
    d3 pc = D3(sqA1 * dPos2.x, sqB1 * dPos2.y - sqB2xFMp * (dA1.z + dA2.z), sqB1 * dPos2.z + sqB2xFMp * (dA1.y + dA2.y));
    float dmN = in.dmN, dmP = in.dmP;
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
    fN = vx64::rotate_inv(angle1, fN);
    mN = vx64::rotate_inv(angle1, mN);
  }
  fP = vx64::rotate_inv(angle2, fP);
  mP = vx64::rotate_inv(angle2, mP);
  o.fN = vx64::to_axis_original(in.axis, fN);
  o.fP = vx64::to_axis_original(in.axis, fP);
  o.mN = vx64::to_axis_original(in.axis, mN);
  o.mP = vx64::to_axis_original(in.axis, mP);
  if (o.failed) {  // a failed link applies nothing; the force terms that set the flag do not run
    o.fN = o.fP = o.mN = o.mP = D3(0, 0, 0);
    lvv = lvvBranch;
  }
  o.pos2 = pos2;
  o.a1v = a1v;
  o.a2v = a2v;
  o.lvv = lvv;
  o.axial = axial;
  o.stress = stress;
  return o;
}

struct LinkGrad {
  d3 gpn, gpp;
  q4 gqn, gqp;
  d3 gOldPos2, gOldA1, gOldA2;
  double gRest, gE, gDmN, gDmP;  // gE: with respect to the link material's E (all constants scale with it)
  d3 gpsn, gpsp;                 // with respect to the end voxels' Poisson strains this step
};

// Adjoint of link_forward, in both branches of orientLink, along the branch the step takes.
// gfN..gmP: adjoints of the four force/moment outputs; gPos2, gA1v, gA2v: of the new link pose
// (read by the next step's damping terms); gAxial: of the new axial strain (read by the next
// step's Poisson strains).
VX_HD bool link_adjoint(const LinkIn& in, const d3& gfN_o, const d3& gfP_o, const d3& gmN_o, const d3& gmP_o,
                        const d3& gPos2_in, const d3& gA1v_in, const d3& gA2v_in, double gAxial_in, LinkGrad& g) {
  // ---- forward recomputation ----
  d3 D = vx64::to_axis_x(in.axis, D3(in.pp.x - in.pn.x, in.pp.y - in.pn.y, in.pp.z - in.pn.z));
  q4 A1 = vx64::to_axis_x(in.axis, in.qn);
  q4 A2 = vx64::to_axis_x(in.axis, in.qp);
  q4 T = Q4(A1.w, -A1.x, -A1.y, -A1.z);
  d3 R = vx64::rotate(T, D);
  q4 G0 = vx64::qmul(T, A2);
  bool smallAngle = in.smallAngle, lvv = in.lvv;
  float smallTurn = (float)((fabs(R.z) + fabs(R.y)) / R.x);
  float extendPerc = (float)(fabs(1 - R.x / in.rest));
  const float HF = 1.2f, BEND = 0.05f, EXT = 0.50f;
  if (!smallAngle && smallTurn < BEND && extendPerc < EXT) {
    smallAngle = true;
    lvv = false;
  } else if (smallAngle && (smallTurn > HF * BEND || extendPerc > HF * EXT)) {
    smallAngle = false;
    lvv = false;
  }
  q4 Q1 = Q4(1, 0, 0, 0), G = G0;
  d3 p;
  double Rlen = 0;
  if (smallAngle) {
    p = D3(R.x - in.rest, R.y, R.z);
  } else {
    from_angle_to_pos_x(Q1, R);
    G = vx64::qmul(Q1, G0);
    Rlen = sqrt(R.x * R.x + R.y * R.y + R.z * R.z);
    p = D3(Rlen - in.rest, 0, 0);
  }
  d3 a1 = rotation_vector(Q1);
  d3 a2v = rotation_vector(G);
  d3 dP = D3(0.5 * (p.x - in.oldPos2.x), 0.5 * (p.y - in.oldPos2.y), 0.5 * (p.z - in.oldPos2.z));
  d3 dA1 = D3(0.5 * (a1.x - in.oldA1.x), 0.5 * (a1.y - in.oldA1.y), 0.5 * (a1.z - in.oldA1.z));
  d3 dA2 = D3(0.5 * (a2v.x - in.oldA2.x), 0.5 * (a2v.y - in.oldA2.y), 0.5 * (a2v.z - in.oldA2.z));
  float tArea, tSS;
  link_transverse(in, &tArea, &tSS);
  double axial = (double)(float)(p.x / in.rest);
  float stress = link_stress(in, (float)axial, tSS);
  const double b1 = in.b1, b2 = in.b2, b3 = in.b3, a2c = in.a2;
  d3 fN0 = D3((double)(stress * tArea), b1 * p.y - b2 * (a1.z + a2v.z), b1 * p.z + b2 * (a1.y + a2v.y));
  d3 mN0 = D3(a2c * (a2v.x - a1.x), -b2 * p.z - b3 * (2 * a1.y + a2v.y), b2 * p.y - b3 * (2 * a1.z + a2v.z));
  d3 mP0 = D3(a2c * (a1.x - a2v.x), -b2 * p.z - b3 * (a1.y + 2 * a2v.y), b2 * p.y - b3 * (a1.z + 2 * a2v.z));
  d3 fN = fN0, mN = mN0;
  d3 fP = D3(-fN0.x, -fN0.y, -fN0.z);
  d3 mP = mP0;
  d3 pc = D3(0, 0, 0), tN = D3(0, 0, 0), tP = D3(0, 0, 0);
  const double sqA1 = in.sqA1, sqA2 = in.sqA2xIp, sqB1 = in.sqB1, sqB2 = in.sqB2xFMp, sqB3 = in.sqB3xIp;
  const double dmN = in.dmN, dmP = in.dmP;
  if (lvv) {
    pc = D3(sqA1 * dP.x, sqB1 * dP.y - sqB2 * (dA1.z + dA2.z), sqB1 * dP.z + sqB2 * (dA1.y + dA2.y));
    fN.x += dmN * pc.x; fN.y += dmN * pc.y; fN.z += dmN * pc.z;
    fP.x -= dmP * pc.x; fP.y -= dmP * pc.y; fP.z -= dmP * pc.z;
    tN = D3(-sqA2 * (dA2.x - dA1.x), sqB2 * dP.z + sqB3 * (2 * dA1.y + dA2.y), -sqB2 * dP.y + sqB3 * (2 * dA1.z + dA2.z));
    tP = D3(sqA2 * (dA2.x - dA1.x), sqB2 * dP.z + sqB3 * (dA1.y + 2 * dA2.y), -sqB2 * dP.y + sqB3 * (dA1.z + 2 * dA2.z));
    double hN = 0.5 * dmN, hP = 0.5 * dmP;
    mN.x -= hN * tN.x; mN.y -= hN * tN.y; mN.z -= hN * tN.z;
    mP.x -= hP * tP.x; mP.y -= hP * tP.y; mP.z -= hP * tP.z;
  }

  // ---- reverse ----
  const int ax = in.axis;
  float msNew;
  const bool failed = link_failed(in, (float)axial, &msNew);  // its forces depend on nothing
  const d3 zero = D3(0, 0, 0);
  d3 gfNr = vx64::to_axis_x(ax, failed ? zero : gfN_o), gfPr = vx64::to_axis_x(ax, failed ? zero : gfP_o);
  d3 gmNr = vx64::to_axis_x(ax, failed ? zero : gmN_o), gmPr = vx64::to_axis_x(ax, failed ? zero : gmP_o);
  q4 gG = Q4(0, 0, 0, 0), gQ1 = Q4(0, 0, 0, 0);
  d3 gfN = D3(0, 0, 0), gmN = D3(0, 0, 0), gfP = D3(0, 0, 0), gmP = D3(0, 0, 0);
  if (smallAngle) {
    gfN = gfNr;
    gmN = gmNr;
  } else {  // fN = rotate_inv(Q1, fN'), mN likewise
    rotate_inv_adj(Q1, fN, gfNr, gQ1, gfN);
    rotate_inv_adj(Q1, mN, gmNr, gQ1, gmN);
  }
  rotate_inv_adj(G, fP, gfPr, gG, gfP);
  rotate_inv_adj(G, mP, gmPr, gG, gmP);
  d3 gp = gPos2_in, ga2 = gA2v_in, ga1 = gA1v_in, gdP = D3(0, 0, 0), gdA1 = D3(0, 0, 0), gdA2 = D3(0, 0, 0);
  double gb1 = 0, gb2 = 0, gb3 = 0, ga2c = 0, gsqA1 = 0, gsqA2 = 0, gsqB1 = 0, gsqB2 = 0, gsqB3 = 0;
  g.gDmN = 0;
  g.gDmP = 0;
  d3 gfN0 = gfN, gfP0 = gfP, gmN0 = gmN, gmP0 = gmP;
  if (lvv) {
    // mP = mP0 - dmP/2 tP ; mN = mN0 - dmN/2 tN ; fP = fP0 - dmP pc ; fN = fN0 + dmN pc
    d3 gtP = scale(-0.5 * dmP, gmP), gtN = scale(-0.5 * dmN, gmN);
    g.gDmP += -0.5 * dot(tP, gmP) - dot(pc, gfP);
    g.gDmN += -0.5 * dot(tN, gmN) + dot(pc, gfN);
    d3 gpc = D3(dmN * gfN.x - dmP * gfP.x, dmN * gfN.y - dmP * gfP.y, dmN * gfN.z - dmP * gfP.z);
    // tN
    gdA2.x += -sqA2 * gtN.x; gdA1.x += sqA2 * gtN.x; gsqA2 += -(dA2.x - dA1.x) * gtN.x;
    gdP.z += sqB2 * gtN.y; gdA1.y += 2 * sqB3 * gtN.y; gdA2.y += sqB3 * gtN.y;
    gsqB2 += dP.z * gtN.y; gsqB3 += (2 * dA1.y + dA2.y) * gtN.y;
    gdP.y -= sqB2 * gtN.z; gdA1.z += 2 * sqB3 * gtN.z; gdA2.z += sqB3 * gtN.z;
    gsqB2 -= dP.y * gtN.z; gsqB3 += (2 * dA1.z + dA2.z) * gtN.z;
    // tP
    gdA2.x += sqA2 * gtP.x; gdA1.x -= sqA2 * gtP.x; gsqA2 += (dA2.x - dA1.x) * gtP.x;
    gdP.z += sqB2 * gtP.y; gdA1.y += sqB3 * gtP.y; gdA2.y += 2 * sqB3 * gtP.y;
    gsqB2 += dP.z * gtP.y; gsqB3 += (dA1.y + 2 * dA2.y) * gtP.y;
    gdP.y -= sqB2 * gtP.z; gdA1.z += sqB3 * gtP.z; gdA2.z += 2 * sqB3 * gtP.z;
    gsqB2 -= dP.y * gtP.z; gsqB3 += (dA1.z + 2 * dA2.z) * gtP.z;
    // pc
    gdP.x += sqA1 * gpc.x; gsqA1 += dP.x * gpc.x;
    gdP.y += sqB1 * gpc.y; gdA1.z -= sqB2 * gpc.y; gdA2.z -= sqB2 * gpc.y;
    gsqB1 += dP.y * gpc.y; gsqB2 -= (dA1.z + dA2.z) * gpc.y;
    gdP.z += sqB1 * gpc.z; gdA1.y += sqB2 * gpc.z; gdA2.y += sqB2 * gpc.z;
    gsqB1 += dP.z * gpc.z; gsqB2 += (dA1.y + dA2.y) * gpc.z;
  }
  // fP0 = -fN0
  gfN0.x -= gfP0.x; gfN0.y -= gfP0.y; gfN0.z -= gfP0.z;
  // fN0
  double gstress = (double)tArea * gfN0.x;
  const double gtArea = (double)stress * gfN0.x;
  gp.y += b1 * gfN0.y; ga1.z -= b2 * gfN0.y; ga2.z -= b2 * gfN0.y;
  gb1 += p.y * gfN0.y; gb2 -= (a1.z + a2v.z) * gfN0.y;
  gp.z += b1 * gfN0.z; ga1.y += b2 * gfN0.z; ga2.y += b2 * gfN0.z;
  gb1 += p.z * gfN0.z; gb2 += (a1.y + a2v.y) * gfN0.z;
  // mN0
  ga2.x += a2c * gmN0.x; ga1.x -= a2c * gmN0.x; ga2c += (a2v.x - a1.x) * gmN0.x;
  gp.z -= b2 * gmN0.y; ga1.y -= 2 * b3 * gmN0.y; ga2.y -= b3 * gmN0.y;
  gb2 -= p.z * gmN0.y; gb3 -= (2 * a1.y + a2v.y) * gmN0.y;
  gp.y += b2 * gmN0.z; ga1.z -= 2 * b3 * gmN0.z; ga2.z -= b3 * gmN0.z;
  gb2 += p.y * gmN0.z; gb3 -= (2 * a1.z + a2v.z) * gmN0.z;
  // mP0
  ga1.x += a2c * gmP0.x; ga2.x -= a2c * gmP0.x; ga2c += (a1.x - a2v.x) * gmP0.x;
  gp.z -= b2 * gmP0.y; ga1.y -= b3 * gmP0.y; ga2.y -= 2 * b3 * gmP0.y;
  gb2 -= p.z * gmP0.y; gb3 -= (a1.y + 2 * a2v.y) * gmP0.y;
  gp.y += b2 * gmP0.z; ga1.z -= b3 * gmP0.z; ga2.z -= 2 * b3 * gmP0.z;
  gb2 += p.y * gmP0.z; gb3 -= (a1.z + 2 * a2v.z) * gmP0.z;
  // stress = E axial (nu = 0) or eHat ((1 - nu) axial + nu tSS), zero past the failure strain;
  // axial = p.x / rest, whose adjoint also comes from the next step's Poisson strains (gAxial_in)
  double E = in.E;
  double gaxial = gAxial_in, gtSS = 0, gE = 0;
  if (!(in.epsilonFail != -1.0f && (float)axial > in.epsilonFail)) {
    if (in.nu == 0.0f) {
      gaxial += E * gstress;
    } else {
      gaxial += (double)in.eHat * (1 - in.nu) * gstress;
      gtSS = (double)in.eHat * in.nu * gstress;
    }
    gE = (E != 0 ? (double)stress / E : 0.0) * gstress;  // eHat is proportional to E
  }
  g.gpsn = D3(0, 0, 0);
  g.gpsp = D3(0, 0, 0);
  if (in.nu != 0.0f) {  // tArea, tSS: the means of the two ends' transverse terms
    transverse_adj(in.sizeN, in.nuN, in.psn, in.axis, 0.5 * gtArea, 0.5 * gtSS, g.gpsn);
    transverse_adj(in.sizeP, in.nuP, in.psp, in.axis, 0.5 * gtArea, 0.5 * gtSS, g.gpsp);
  }
  gp.x += gaxial / in.rest;
  double grest = -p.x / (in.rest * in.rest) * gaxial;
  // dP, dA1, dA2
  gp.x += 0.5 * gdP.x; gp.y += 0.5 * gdP.y; gp.z += 0.5 * gdP.z;
  g.gOldPos2 = scale(-0.5, gdP);
  ga1.x += 0.5 * gdA1.x; ga1.y += 0.5 * gdA1.y; ga1.z += 0.5 * gdA1.z;
  g.gOldA1 = scale(-0.5, gdA1);
  ga2.x += 0.5 * gdA2.x; ga2.y += 0.5 * gdA2.y; ga2.z += 0.5 * gdA2.z;
  g.gOldA2 = scale(-0.5, gdA2);
  // a2v = rotation_vector(G), a1 = rotation_vector(Q1)
  rotation_vector_adj(G, ga2, gG);
  q4 gG0 = Q4(0, 0, 0, 0);
  d3 gR = D3(0, 0, 0);
  if (smallAngle) {  // p = R - (rest, 0, 0), G = G0, a1 = 0
    gG0 = gG;
    gR = gp;
    grest -= gp.x;
  } else {  // p = (|R| - rest, 0, 0), G = Q1 G0, Q1 = from_angle_to_pos_x(R)
    rotation_vector_adj(Q1, ga1, gQ1);
    qmul_adj(Q1, G0, gG, gQ1, gG0);
    gR = scale(gp.x / Rlen, R);
    grest -= gp.x;
    from_angle_to_pos_x_adj(R, gQ1, gR);
  }
  // G0 = T * A2 ; R = rotate(T, D) ; T = conj(A1)
  q4 gT = Q4(0, 0, 0, 0), gA2 = Q4(0, 0, 0, 0);
  qmul_adj(T, A2, gG0, gT, gA2);
  d3 gD = D3(0, 0, 0);
  rotate_adj(T, D, gR, gT, gD);
  q4 gA1 = Q4(gT.w, -gT.x, -gT.y, -gT.z);
  g.gqn = Q4(0, 0, 0, 0);
  g.gqp = Q4(0, 0, 0, 0);
  to_axis_x_q_adj(ax, gA1, g.gqn);
  to_axis_x_q_adj(ax, gA2, g.gqp);
  d3 gD0 = vx64::to_axis_original(ax, gD);
  g.gpp = gD0;
  g.gpn = D3(-gD0.x, -gD0.y, -gD0.z);
  g.gRest = grest;
  // every material constant is proportional to E (a1, a2, b1, b2, b3) or to sqrt(E) (the sq* terms)
  double Ed = E != 0 ? E : 1.0;
  g.gE = gE + (gb1 * b1 + gb2 * b2 + gb3 * b3 + ga2c * a2c) / Ed +
         0.5 * (gsqA1 * sqA1 + gsqA2 * sqA2 + gsqB1 * sqB1 + gsqB2 * sqB2 + gsqB3 * sqB3) / Ed;
  return true;
}

// CVX_Voxel::strain(true) (vx64::poisson_strain_links, VX_Voxel.cpp:300-334) differentiated with
// respect to the axial strains its links' ends see: e[i] for slot i where has[i]; extT[i]: an
// external fixes or loads axis i (which makes an axis with one link count as in tension); gP: the
// adjoint of the three Poisson strains; adds into ge.
VX_HD void poisson_adjoint(const float e[6], const bool has[6], const bool extT[3], float nu, const double gP[3],
                           double ge[6]) {
  float s[3] = {0, 0, 0};
  int nb[3] = {0, 0, 0};
  for (int i = 0; i < 6; ++i)
    if (has[i]) {
      s[i / 2] += e[i];
      nb[i / 2]++;
    }
  bool tension[3];
  for (int i = 0; i < 3; ++i) {
    if (nb[i] == 2) s[i] *= 0.5f;
    tension[i] = nb[i] == 2 || (nb[i] == 1 && extT[i]);
  }
  double gs[3] = {0, 0, 0};
  for (int i = 0; i < 3; ++i)
    if (tension[i]) gs[i] += gP[i];
  if (!(tension[0] && tension[1] && tension[2])) {  // the other axes: powf(1 + sum, -nu) - 1
    float add = 0;
    for (int i = 0; i < 3; ++i)
      if (tension[i]) add += s[i];
    double gval = 0;
    for (int i = 0; i < 3; ++i)
      if (!tension[i]) gval += gP[i];
    const double gadd = gval * (-(double)nu * pow(1.0 + (double)add, -(double)nu - 1.0));
    for (int i = 0; i < 3; ++i)
      if (tension[i]) gs[i] += gadd;
  }
  for (int i = 0; i < 3; ++i)
    if (nb[i] == 2) gs[i] *= 0.5;
  for (int i = 0; i < 6; ++i)
    if (has[i]) ge[i] += gs[i / 2];
}

// ---- voxel -----------------------------------------------------------------------------------
struct VoxelIn {
  d3 pos, lin, ang;
  q4 orient;
  d3 Fl, Ml;           // sum of the link forces / moments in the voxel frame (gathered in slot order)
  bool floorOn, staticF;
  float dt;
  float mass, massInv, inertiaInv, c2xSqMxExS, c2xSqIxExSxSxS, zetaGlobal, zetaCollision, gravMult,
      penetrationStiffness, muStatic, muKinetic;
  double halfPenOffset;  // base size average / 2 - nominal size / 2 (temperature dependent)
  d3 extF, extM;
  int dof;               // the external's fixed degrees of freedom (bits 0-2 translation, 3-5 rotation)
  d3 fixPos;             // the prescribed position and orientation of those degrees of freedom
  q4 fixOrient;
};
struct VoxelOut {
  d3 pos, lin, ang;
  q4 orient;
  bool staticF;
};

// the external's fixes at the end of CVX_Voxel::timeStep (VX_Voxel.cpp:215-229, vx64::voxel_update)
VX_HD void apply_fixes(const VoxelIn& in, d3& pos, d3& lin, q4& orient, d3& ang) {
  if (in.dof & 1) { pos.x = in.fixPos.x; lin.x = 0; }
  if (in.dof & 2) { pos.y = in.fixPos.y; lin.y = 0; }
  if (in.dof & 4) { pos.z = in.fixPos.z; lin.z = 0; }
  if (in.dof & 56) {
    if ((in.dof & 56) == 56) {
      orient = in.fixOrient;
      ang = D3(0, 0, 0);
    } else {
      d3 r = rotation_vector(orient);
      if (in.dof & 8) { r.x = 0; ang.x = 0; }
      if (in.dof & 16) { r.y = 0; ang.y = 0; }
      if (in.dof & 32) { r.z = 0; ang.z = 0; }
      orient = from_rotation_vector(r);
    }
  }
}
// Its adjoint: the adjoints of the state before the fixes from those after (q: the orientation
// before them).  A fixed component's value does not depend on anything.
VX_HD void apply_fixes_adj(const VoxelIn& in, const q4& q, d3& gpos, d3& glin, q4& gq, d3& gang) {
  if (in.dof & 1) { gpos.x = 0; glin.x = 0; }
  if (in.dof & 2) { gpos.y = 0; glin.y = 0; }
  if (in.dof & 4) { gpos.z = 0; glin.z = 0; }
  if (in.dof & 56) {
    if ((in.dof & 56) == 56) {
      gq = Q4(0, 0, 0, 0);
      gang = D3(0, 0, 0);
    } else {
      d3 r = rotation_vector(q);
      if (in.dof & 8) { r.x = 0; gang.x = 0; }
      if (in.dof & 16) { r.y = 0; gang.y = 0; }
      if (in.dof & 32) { r.z = 0; gang.z = 0; }
      d3 gr = D3(0, 0, 0);
      from_rotation_vector_adj(r, gq, gr);
      if (in.dof & 8) gr.x = 0;
      if (in.dof & 16) gr.y = 0;
      if (in.dof & 32) gr.z = 0;
      gq = Q4(0, 0, 0, 0);
      rotation_vector_adj(q, gr, gq);
    }
  }
}

// CVX_Voxel::timeStep without collisions (vx64::voxel_update's arithmetic)
VX_HD VoxelOut voxel_forward(const VoxelIn& in) {
  VoxelOut o;
  d3 lin = in.lin, ang = in.ang, pos = in.pos;
  d3 F = vx64::rotate(in.orient, in.Fl);
  F.x += in.extF.x; F.y += in.extF.y; F.z += in.extF.z;
  {
    float c = in.zetaGlobal * in.c2xSqMxExS;
    F.x -= c * (in.massInv * lin.x);
    F.y -= c * (in.massInv * lin.y);
    F.z -= c * (in.massInv * lin.z);
  }
  F.z += -in.mass * 9.80665f * in.gravMult;
  d3 fric = F;
  bool staticF = in.staticF;
  float pen = (float)(in.halfPenOffset - pos.z);
  if (in.floorOn) {
    if (pen >= 0) {
      d3 vel = D3(in.massInv * lin.x, in.massInv * lin.y, in.massInv * lin.z);
      float normal = in.penetrationStiffness * pen;
      F.z += normal - (in.zetaCollision * in.c2xSqMxExS) * vel.z;
      if (staticF) {
        float surf = (float)(F.x * F.x + F.y * F.y);
        float fr = (in.muStatic * normal) * (in.muStatic * normal);
        if (surf > fr) staticF = false;
      } else {
        float k = in.muKinetic * normal;
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
  float dt = in.dt;
  lin.x += dt * F.x; lin.y += dt * F.y; lin.z += dt * F.z;
  float dtm = dt * in.massInv;
  d3 tr = D3(dtm * lin.x, dtm * lin.y, dtm * lin.z);
  if (in.floorOn && pen >= 0) {
    double work = fric.x * tr.x + fric.y * tr.y;
    double hKe = 0.5 * in.massInv * (lin.x * lin.x + lin.y * lin.y);
    if (hKe + work <= 0) staticF = true;
    if (staticF) {
      lin.x = lin.y = 0;
      tr.x = tr.y = 0;
    }
  } else {
    staticF = false;
  }
  pos.x += tr.x; pos.y += tr.y; pos.z += tr.z;
  d3 M = vx64::rotate(in.orient, in.Ml);
  M.x += in.extM.x; M.y += in.extM.y; M.z += in.extM.z;
  {
    float c = in.zetaGlobal * in.c2xSqIxExSxSxS;
    M.x -= c * (in.inertiaInv * ang.x);
    M.y -= c * (in.inertiaInv * ang.y);
    M.z -= c * (in.inertiaInv * ang.z);
  }
  ang.x += dt * M.x; ang.y += dt * M.y; ang.z += dt * M.z;
  float dti = dt * in.inertiaInv;
  q4 dq = from_rotation_vector(D3(dti * ang.x, dti * ang.y, dti * ang.z));
  q4 orient = vx64::qmul(dq, in.orient);
  apply_fixes(in, pos, lin, orient, ang);
  o.orient = orient;
  o.pos = pos;
  o.lin = lin;
  o.ang = ang;
  o.staticF = staticF;
  return o;
}

struct VoxelGrad {
  d3 gpos, glin, gang;
  q4 gorient;
  d3 gFl, gMl;
  double gMass, gMassInv, gInertiaInv, gC2x, gC2xI, gPenStiff, gHalfPenOffset;
};

// Adjoint of voxel_forward given the adjoints of the new state.
VX_HD void voxel_adjoint(const VoxelIn& in, const d3& gpos_f, const d3& glin_f, const q4& gq_f, const d3& gang_f,
                         VoxelGrad& g) {
  // ---- forward recomputation ----
  const d3 lin0 = in.lin;
  d3 F0 = vx64::rotate(in.orient, in.Fl);
  d3 F = F0;
  F.x += in.extF.x; F.y += in.extF.y; F.z += in.extF.z;
  const double c = (float)(in.zetaGlobal * in.c2xSqMxExS);
  F.x -= c * (in.massInv * lin0.x);
  F.y -= c * (in.massInv * lin0.y);
  F.z -= c * (in.massInv * lin0.z);
  F.z += -in.mass * 9.80665f * in.gravMult;
  d3 fric = F;
  bool staticF = in.staticF;
  float pen = (float)(in.halfPenOffset - in.pos.z);
  bool contact = in.floorOn && pen >= 0;
  bool kinetic = false;
  d3 vel = D3(in.massInv * lin0.x, in.massInv * lin0.y, in.massInv * lin0.z);
  float normal = 0.0f, k = 0.0f;
  d3 h = D3(0, 0, 0);
  double len = 0;
  const double cc = (float)(in.zetaCollision * in.c2xSqMxExS);
  if (in.floorOn) {
    if (pen >= 0) {
      normal = in.penetrationStiffness * pen;
      F.z += normal - cc * vel.z;
      if (staticF) {
        float surf = (float)(F.x * F.x + F.y * F.y);
        float fr = (in.muStatic * normal) * (in.muStatic * normal);
        if (surf > fr) staticF = false;
      } else {
        kinetic = true;
        k = in.muKinetic * normal;
        h = D3(vel.x, vel.y, 0);
        len = sqrt(h.x * h.x + h.y * h.y);
        if (len > 0) h = D3(h.x / len, h.y / len, 0);
        F.x -= k * h.x; F.y -= k * h.y;
      }
    } else {
      staticF = false;
    }
  }
  fric = D3(F.x - fric.x, F.y - fric.y, F.z - fric.z);
  const double dt = in.dt;
  d3 lin = D3(lin0.x + dt * F.x, lin0.y + dt * F.y, lin0.z + dt * F.z);
  const double dtm = (float)(in.dt * in.massInv);
  d3 tr = D3(dtm * lin.x, dtm * lin.y, dtm * lin.z);
  bool latched = false;
  if (contact) {
    double work = fric.x * tr.x + fric.y * tr.y;
    double hKe = 0.5 * in.massInv * (lin.x * lin.x + lin.y * lin.y);
    if (hKe + work <= 0) staticF = true;
    latched = staticF;
  }
  d3 M0 = vx64::rotate(in.orient, in.Ml);
  d3 M = M0;
  M.x += in.extM.x; M.y += in.extM.y; M.z += in.extM.z;
  const double cI = (float)(in.zetaGlobal * in.c2xSqIxExSxSxS);
  M.x -= cI * (in.inertiaInv * in.ang.x);
  M.y -= cI * (in.inertiaInv * in.ang.y);
  M.z -= cI * (in.inertiaInv * in.ang.z);
  d3 ang = D3(in.ang.x + dt * M.x, in.ang.y + dt * M.y, in.ang.z + dt * M.z);
  const double dti = (float)(in.dt * in.inertiaInv);
  d3 rv = D3(dti * ang.x, dti * ang.y, dti * ang.z);
  q4 dq = from_rotation_vector(rv);

  // ---- reverse ----
  // the external's fixes, last in the forward step, first here
  d3 gpos_n = gpos_f, glin_n = glin_f, gang_n = gang_f;
  q4 gq_n = gq_f;
  if (in.dof) apply_fixes_adj(in, vx64::qmul(dq, in.orient), gpos_n, glin_n, gq_n, gang_n);
  g.gMass = g.gMassInv = g.gInertiaInv = g.gC2x = g.gC2xI = g.gPenStiff = g.gHalfPenOffset = 0;
  // orient' = dq * orient
  q4 gdq = Q4(0, 0, 0, 0);
  g.gorient = Q4(0, 0, 0, 0);
  qmul_adj(dq, in.orient, gq_n, gdq, g.gorient);
  d3 grv = D3(0, 0, 0);
  from_rotation_vector_adj(rv, gdq, grv);
  d3 gang = gang_n;
  add(gang, scale(dti, grv));
  g.gInertiaInv += dt * dot(ang, grv);
  // ang' = ang + dt M ; M = rotate(q, Ml) + ext - cI IInv ang
  d3 gM = scale(dt, gang);
  g.gang = gang;
  g.gang.x -= cI * in.inertiaInv * gM.x;
  g.gang.y -= cI * in.inertiaInv * gM.y;
  g.gang.z -= cI * in.inertiaInv * gM.z;
  double gcI = -in.inertiaInv * dot(in.ang, gM);
  g.gInertiaInv += -cI * dot(in.ang, gM);
  g.gC2xI += in.zetaGlobal * gcI;
  g.gMl = D3(0, 0, 0);
  rotate_adj(in.orient, in.Ml, gM, g.gorient, g.gMl);
  // pos' = pos + tr ; tr = dtm lin' (x, y zero when latched)
  g.gpos = gpos_n;
  d3 gtr = gpos_n;
  d3 glin = glin_n;
  if (latched) { gtr.x = gtr.y = 0; glin.x = glin.y = 0; }
  glin.x += dtm * gtr.x; glin.y += dtm * gtr.y; glin.z += dtm * gtr.z;
  g.gMassInv += dt * dot(lin, gtr);
  // lin' = lin + dt F
  g.glin = glin;
  d3 gF = scale(dt, glin);
  // floor
  if (contact) {
    double gnormal = 0;
    d3 gvel = D3(0, 0, 0);
    if (kinetic) {
      double gk = -(h.x * gF.x + h.y * gF.y);
      d3 gh = D3(-k * gF.x, -k * gF.y, 0);
      if (len > 0) {
        double hg = h.x * gh.x + h.y * gh.y;
        gvel.x += (gh.x - h.x * hg) / len;
        gvel.y += (gh.y - h.y * hg) / len;
      }
      gnormal += in.muKinetic * gk;
    }
    gnormal += gF.z;
    gvel.z -= cc * gF.z;
    g.gC2x += -in.zetaCollision * vel.z * gF.z;
    g.glin.x += in.massInv * gvel.x;
    g.glin.y += in.massInv * gvel.y;
    g.glin.z += in.massInv * gvel.z;
    g.gMassInv += dot(lin0, gvel);
    g.gPenStiff += (double)pen * gnormal;
    double gpen = in.penetrationStiffness * gnormal;
    g.gpos.z -= gpen;
    g.gHalfPenOffset += gpen;
  }
  // gravity
  g.gMass += -9.80665 * (double)in.gravMult * gF.z;
  // global damping
  g.glin.x -= c * in.massInv * gF.x;
  g.glin.y -= c * in.massInv * gF.y;
  g.glin.z -= c * in.massInv * gF.z;
  double gc = -in.massInv * dot(lin0, gF);
  g.gMassInv += -c * dot(lin0, gF);
  g.gC2x += in.zetaGlobal * gc;
  g.gFl = D3(0, 0, 0);
  rotate_adj(in.orient, in.Fl, gF, g.gorient, g.gFl);
}

}  // namespace vxa
