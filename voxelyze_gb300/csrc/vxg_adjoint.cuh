// Adjoint kernels of the FP64 time step (included by vxg_engine.cu).
//
// A differentiated run records, for every step of one checkpoint segment, the state the step starts
// from (the tape); the reverse sweep walks the segment backwards, one step at a time:
//   k_adj_link_forces  recompute the link forces of the step from the tape,
//   k_adj_voxel        voxel pass adjoint: adjoint of the voxel state one step earlier (partial),
//                      adjoints of the summed link forces/moments, material and temperature terms,
//   k_adj_link         link pass adjoint: per-link contributions to both voxels' pose adjoints, the
//                      adjoint of the link's previous pose, and its material/rest-length terms,
//   k_adj_gather       per voxel, in slot order: add the link contributions (no atomics) and fold
//                      the parameter terms into dJ/dE, dJ/drho and dJ/dphase.
// Per-step arithmetic is vx_adjoint.cuh.
#pragma once
#include "vx_adjoint.cuh"

namespace {

// Per-step actuation parameters (the engine's vxg_set_actuation state)
struct ActParams {
  int mode;
  double amp, freq;
  const float* phase;
};

struct AdjBuf {
  int K;                // tape slots
  double* tv;           // K x 13 nv: pos 3, linMom 3, orient 4, angMom 3 (component-major)
  uint32_t* tvf;        // K x nv voxel flags
  float* tpd;           // K x nv previous dt
  double* tl;           // K x 9 nl: pos2 3, angle1v 3, angle2v 3
  uint32_t* tlf;        // K x nl link flags
  float* tms;           // K x nl largest axial strain so far (failure)
  float* tstrain;       // K x nl axial strain at the step's start (the previous step's, nu != 0)
  float* tps;           // K x 3 nv Poisson strains the step's links used (nu != 0)
  double* lps;          // 6 nl: adjoints of the negative and positive voxels' Poisson strains
  double* gS;           // 6 nv: adjoint of the axial strain each voxel's slot-i link shows it, from
                        // the Poisson strains of the step after (read by the link adjoint)
  float* ttime;         // K step start times
  float* ttemp;         // K x nv temperatures each step used (after its actuation)
  double* tforce;       // K x 12 nl link forces and moments of each step (null: recomputed)
  double* lam;          // 13 nv adjoint of the voxel state
  double* gFM;          // 6 nv adjoint of the summed link force (3) and moment (3), voxel frame
  double* mu;           // 9 nl adjoint of the link pose (pos2, angle1v, angle2v)
  double* lcon;         // 14 nl: gpn 3, gqn 4, gpp 3, gqp 4
  double* lpar;         // 4 nl: gRest, gE (link material), gDmN, gDmP
  double* lforce;       // 12 nl: fN, fP, mN, mP recomputed for the step
  double* gTempV;       // nv: temperature adjoint from the voxel pass (floor penetration)
  double* accE;         // nv: dJ/dE of each voxel's material
  double* accRho;       // nv: dJ/drho
  double* accPhase;     // nv: dJ/dphase
  int* err;             // bit 0: a link's adjoint could not be taken
};

__device__ __forceinline__ double act_dtemp_dphase(const ActParams& A, int v, float time) {
  double arg = 2.0 * 3.141592653589793 * A.freq * (double)time + (A.phase ? (double)A.phase[v] : 0.0);
  return A.amp * cos(arg);
}

// what step `slot` computed and the reverse sweep reads: the temperatures it used and, when the
// tape has room, its link forces and moments (the layout k_adj_link_forces writes); launched right
// after the step, before the next actuation or link pass
__global__ void k_tape_step(View S, AdjBuf T, int slot) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int nv = S.nv, nl = S.nl;
  if (i < nv) {
    T.ttemp[(size_t)slot * nv + i] = S.temp[i];
    for (int c = 0; c < 3; ++c) T.tps[((size_t)slot * 3 + c) * nv + i] = S.pStrain[(size_t)c * nv + i];
  }
  if (T.tforce && i < nl) {
    double* tf = T.tforce + (size_t)slot * 12 * nl;
    for (int c = 0; c < 3; ++c) {
      tf[(size_t)c * nl + i] = S.fN[(size_t)c * nl + i];
      tf[(size_t)(3 + c) * nl + i] = S.fP[(size_t)c * nl + i];
      tf[(size_t)(6 + c) * nl + i] = S.mN[(size_t)c * nl + i];
      tf[(size_t)(9 + c) * nl + i] = S.mP[(size_t)c * nl + i];
    }
  }
}

__global__ void k_tape_save(View S, AdjBuf T, int slot) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int nv = S.nv, nl = S.nl;
  if (i < nv) {
    double* tv = T.tv + (size_t)slot * 13 * nv;
    for (int c = 0; c < 3; ++c) {
      tv[c * nv + i] = S.pos[c * nv + i];
      tv[(3 + c) * nv + i] = S.linMom[c * nv + i];
      tv[(10 + c) * nv + i] = S.angMom[c * nv + i];
    }
    for (int c = 0; c < 4; ++c) tv[(6 + c) * nv + i] = S.orient[c * nv + i];
    T.tvf[(size_t)slot * nv + i] = S.vflags[i];
    T.tpd[(size_t)slot * nv + i] = S.prevDt[i];
  }
  if (i < nl) {
    double* tl = T.tl + (size_t)slot * 9 * nl;
    for (int c = 0; c < 3; ++c) {
      tl[c * nl + i] = S.pos2[c * nl + i];
      tl[(3 + c) * nl + i] = S.a1v[c * nl + i];
      tl[(6 + c) * nl + i] = S.a2v[c * nl + i];
    }
    T.tlf[(size_t)slot * nl + i] = S.lflags[i];
    T.tms[(size_t)slot * nl + i] = S.maxStrain[i];
    T.tstrain[(size_t)slot * nl + i] = S.strain[i];
  }
  if (i == 0) T.ttime[slot] = S.ctl->time;
}

__device__ vxa::LinkIn tape_link_in(const View& S, const AdjBuf& T, const ActParams& A, int slot, int l) {
  const int nv = S.nv, nl = S.nl;
  const double* tv = T.tv + (size_t)slot * 13 * nv;
  const double* tl = T.tl + (size_t)slot * 9 * nl;
  uint32_t lf = T.tlf[(size_t)slot * nl + l];
  int vn = S.lvox[l], vp = S.lvox[nl + l];
  vxa::LinkIn in;
  in.axis = (lf >> 8) & 3;
  in.smallAngle = lf & VXG_LF_SMALL_ANGLE;
  in.lvv = lf & VXG_LF_LOCAL_VEL_VALID;
  in.pn = vx64::D3(tv[vn], tv[nv + vn], tv[2 * nv + vn]);
  in.pp = vx64::D3(tv[vp], tv[nv + vp], tv[2 * nv + vp]);
  in.qn = vx64::Q4(tv[6 * nv + vn], tv[7 * nv + vn], tv[8 * nv + vn], tv[9 * nv + vn]);
  in.qp = vx64::Q4(tv[6 * nv + vp], tv[7 * nv + vp], tv[8 * nv + vp], tv[9 * nv + vp]);
  in.oldPos2 = vx64::D3(tl[l], tl[nl + l], tl[2 * nl + l]);
  in.oldA1 = vx64::D3(tl[3 * nl + l], tl[4 * nl + l], tl[5 * nl + l]);
  in.oldA2 = vx64::D3(tl[6 * nl + l], tl[7 * nl + l], tl[8 * nl + l]);
  const vxg_voxel_material& mn = S.vm[S.vmat[vn]];
  const vxg_voxel_material& mp = S.vm[S.vmat[vp]];
  if (A.mode) {  // CVX_Link::updateRestLength after the step's setTemperature (VX_Link.cpp:137-140)
    const float* tt = T.ttemp + (size_t)slot * nv;
    float tn = tt[vn], tp = tt[vp];
    in.rest = 0.5 * (mn.size[in.axis] * (1 + tn * mn.alphaCTE) + mp.size[in.axis] * (1 + tp * mp.alphaCTE));
  } else {
    in.rest = S.rest[l];
  }
  const vxg_link_material& m = S.lm[S.lmat[l]];
  in.E = m.E; in.a2 = m.a2; in.b1 = m.b1; in.b2 = m.b2; in.b3 = m.b3;
  in.sqA1 = m.sqA1; in.sqA2xIp = m.sqA2xIp; in.sqB1 = m.sqB1; in.sqB2xFMp = m.sqB2xFMp; in.sqB3xIp = m.sqB3xIp;
  in.tArea = S.tArea[l];
  in.maxStrain = T.tms[(size_t)slot * nl + l];
  in.epsilonFail = m.epsilonFail;
  in.nu = m.nu;
  in.eHat = m.eHat;
  in.sizeN = (float)mn.nomSize;
  in.sizeP = (float)mp.nomSize;
  in.nuN = mn.nu != 0.0f;
  in.nuP = mp.nu != 0.0f;
  const float* ps = T.tps + (size_t)slot * 3 * nv;
  in.psn = vx64::D3(ps[vn], ps[nv + vn], ps[2 * nv + vn]);
  in.psp = vx64::D3(ps[vp], ps[nv + vp], ps[2 * nv + vp]);
  // CVX_Voxel::dampingMultiplier with the previous dt the step saw (VX_Voxel.h:130)
  in.dmN = 2 * mn.sqrtMass * mn.zetaInternal / T.tpd[(size_t)slot * nv + vn];
  in.dmP = 2 * mp.sqrtMass * mp.zetaInternal / T.tpd[(size_t)slot * nv + vp];
  return in;
}

__global__ void k_adj_link_forces(View S, AdjBuf T, ActParams A, int slot) {
  int l = blockIdx.x * blockDim.x + threadIdx.x;
  const int nl = S.nl;
  if (l >= nl) return;
  vxa::LinkIn in = tape_link_in(S, T, A, slot, l);
  vxa::LinkOut o = vxa::link_forward(in);
  const vx64::d3 F[4] = {o.fN, o.fP, o.mN, o.mP};
  for (int k = 0; k < 4; ++k) {
    T.lforce[(3 * k) * (size_t)nl + l] = F[k].x;
    T.lforce[(3 * k + 1) * (size_t)nl + l] = F[k].y;
    T.lforce[(3 * k + 2) * (size_t)nl + l] = F[k].z;
  }
}

__device__ __forceinline__ bool fixed_all(const View& S, int v) {
  int ei = S.vext[v];
  return ei >= 0 && (S.ext[ei].dof & 0x3F) == 0x3F;
}

__global__ void k_adj_voxel(View S, AdjBuf T, ActParams A, int slot, float dt) {
  int v = blockIdx.x * blockDim.x + threadIdx.x;
  const int nv = S.nv, nl = S.nl;
  if (v >= nv) return;
  if (fixed_all(S, v)) {  // the new state is the prescribed one: nothing flows back
    for (int c = 0; c < 13; ++c) T.lam[(size_t)c * nv + v] = 0.0;
    for (int c = 0; c < 6; ++c) T.gFM[(size_t)c * nv + v] = 0.0;
    T.gTempV[v] = 0.0;
    return;
  }
  const double* tv = T.tv + (size_t)slot * 13 * nv;
  uint32_t flags = T.tvf[(size_t)slot * nv + v];
  const vxg_voxel_material& m = S.vm[S.vmat[v]];
  vxa::VoxelIn in;
  in.pos = vx64::D3(tv[v], tv[nv + v], tv[2 * nv + v]);
  in.lin = vx64::D3(tv[3 * nv + v], tv[4 * nv + v], tv[5 * nv + v]);
  in.orient = vx64::Q4(tv[6 * nv + v], tv[7 * nv + v], tv[8 * nv + v], tv[9 * nv + v]);
  in.ang = vx64::D3(tv[10 * nv + v], tv[11 * nv + v], tv[12 * nv + v]);
  vx64::d3 F = vx64::D3(0, 0, 0), M = vx64::D3(0, 0, 0);
  for (int i = 0; i < 6; ++i) {  // CVX_Voxel::force / moment gather order (VX_Voxel.cpp:234-271)
    int l = S.vlinks[i * nv + v];
    if (l < 0) continue;
    int fo = (i & 1) ? 3 : 0, mo = (i & 1) ? 9 : 6;
    F.x += T.lforce[(size_t)fo * nl + l]; F.y += T.lforce[(size_t)(fo + 1) * nl + l]; F.z += T.lforce[(size_t)(fo + 2) * nl + l];
    M.x += T.lforce[(size_t)mo * nl + l]; M.y += T.lforce[(size_t)(mo + 1) * nl + l]; M.z += T.lforce[(size_t)(mo + 2) * nl + l];
  }
  in.Fl = F;
  in.Ml = M;
  in.floorOn = flags & VXG_VF_FLOOR;
  in.staticF = flags & VXG_VF_STATIC_FRICTION;
  in.dt = dt;
  in.mass = m.mass; in.massInv = m.massInv; in.inertiaInv = m.inertiaInv;
  in.c2xSqMxExS = m.c2xSqMxExS; in.c2xSqIxExSxSxS = m.c2xSqIxExSxSxS;
  in.zetaGlobal = m.zetaGlobal; in.zetaCollision = m.zetaCollision; in.gravMult = m.gravMult;
  in.penetrationStiffness = m.penetrationStiffness; in.muStatic = m.muStatic; in.muKinetic = m.muKinetic;
  float temp = T.ttemp[(size_t)slot * nv + v];
  {  // CVX_Voxel::baseSizeAverage (VX_Voxel.h:90) at this step's temperature
    float f = 1 + temp * m.alphaCTE;
    double bsa = ((double)f * m.size[0] + (double)f * m.size[1] + (double)f * m.size[2]) / 3.0f;
    in.halfPenOffset = bsa / 2 - m.nomSize / 2;
  }
  int ei = S.vext[v];
  in.dof = 0;
  in.fixPos = vx64::D3(0, 0, 0);
  in.fixOrient = vx64::Q4(1, 0, 0, 0);
  if (ei >= 0) {
    const vxg_external& e = S.ext[ei];
    in.extF = vx64::D3(e.force[0], e.force[1], e.force[2]);
    in.extM = vx64::D3(e.moment[0], e.moment[1], e.moment[2]);
    in.dof = e.dof & 0x3F;
    const double s = m.nomSize;
    in.fixPos = vx64::D3(S.vidx[v] * s + e.translation[0], S.vidx[nv + v] * s + e.translation[1],
                         S.vidx[2 * nv + v] * s + e.translation[2]);
    in.fixOrient = vx64::Q4(e.rotq[0], e.rotq[1], e.rotq[2], e.rotq[3]);
  } else {
    in.extF = in.extM = vx64::D3(0, 0, 0);
  }
  vx64::d3 gpos = vx64::D3(T.lam[v], T.lam[nv + v], T.lam[2 * nv + v]);
  vx64::d3 glin = vx64::D3(T.lam[3 * nv + v], T.lam[4 * nv + v], T.lam[5 * nv + v]);
  vx64::q4 gq = vx64::Q4(T.lam[6 * nv + v], T.lam[7 * nv + v], T.lam[8 * nv + v], T.lam[9 * nv + v]);
  vx64::d3 gang = vx64::D3(T.lam[10 * nv + v], T.lam[11 * nv + v], T.lam[12 * nv + v]);
  vxa::VoxelGrad g;
  vxa::voxel_adjoint(in, gpos, glin, gq, gang, g);
  const double st[13] = {g.gpos.x, g.gpos.y, g.gpos.z, g.glin.x, g.glin.y, g.glin.z, g.gorient.w, g.gorient.x,
                         g.gorient.y, g.gorient.z, g.gang.x, g.gang.y, g.gang.z};
  for (int c = 0; c < 13; ++c) T.lam[(size_t)c * nv + v] = st[c];
  const double fm[6] = {g.gFl.x, g.gFl.y, g.gFl.z, g.gMl.x, g.gMl.y, g.gMl.z};
  for (int c = 0; c < 6; ++c) T.gFM[(size_t)c * nv + v] = fm[c];
  // material terms: mass = volume rho, I = m L^2 / 6, 2 sqrt(m E L), 2 sqrt(I E L^3), 2 E L
  double mass = m.mass, E = m.E;
  double gm = g.gMass - g.gMassInv * (double)m.massInv * m.massInv - g.gInertiaInv * (double)m.inertiaInv / mass +
              (g.gC2x * m.c2xSqMxExS + g.gC2xI * m.c2xSqIxExSxSxS) / (2.0 * mass);
  double volume = m.nomSize * m.nomSize * m.nomSize;
  T.accRho[v] += gm * volume;
  T.accE[v] += (g.gC2x * m.c2xSqMxExS + g.gC2xI * m.c2xSqIxExSxSxS) / (2.0 * E) +
               g.gPenStiff * m.penetrationStiffness / E;
  // d(halfPenOffset)/d(temperature) = alphaCTE (size.x + size.y + size.z) / 6
  T.gTempV[v] = g.gHalfPenOffset * (double)m.alphaCTE * (m.size[0] + m.size[1] + m.size[2]) / 6.0;
}

__global__ void k_adj_link(View S, AdjBuf T, ActParams A, int slot) {
  int l = blockIdx.x * blockDim.x + threadIdx.x;
  const int nv = S.nv, nl = S.nl;
  if (l >= nl) return;
  vxa::LinkIn in = tape_link_in(S, T, A, slot, l);
  int vn = S.lvox[l], vp = S.lvox[nl + l];
  auto g3 = [&](int base, int v) { return vx64::D3(T.gFM[(size_t)base * nv + v], T.gFM[(size_t)(base + 1) * nv + v], T.gFM[(size_t)(base + 2) * nv + v]); };
  vx64::d3 gfN = g3(0, vn), gfP = g3(0, vp), gmN = g3(3, vn), gmP = g3(3, vp);
  vx64::d3 gPos2 = vx64::D3(T.mu[l], T.mu[nl + l], T.mu[2 * nl + l]);
  vx64::d3 gA1v = vx64::D3(T.mu[3 * nl + l], T.mu[4 * nl + l], T.mu[5 * nl + l]);
  vx64::d3 gA2v = vx64::D3(T.mu[6 * nl + l], T.mu[7 * nl + l], T.mu[8 * nl + l]);
  // the axial strain's adjoint from the next step's Poisson strains: this link is the negative
  // voxel's slot 2 axis and the positive voxel's slot 2 axis + 1 (vx64::link_axial_strain's ends)
  double gAxial = 0;
  if (in.nu != 0.0f) {
    const double r = S.strainRatio[l];
    gAxial = T.gS[(size_t)(2 * in.axis) * nv + vn] * (2.0 / (1.0 + r)) +
             T.gS[(size_t)(2 * in.axis + 1) * nv + vp] * (2.0 * r / (1.0 + r));
  }
  vxa::LinkGrad g;
  if (!vxa::link_adjoint(in, gfN, gfP, gmN, gmP, gPos2, gA1v, gA2v, gAxial, g)) {
    atomicOr(T.err, 1);
    for (int c = 0; c < 9; ++c) T.mu[(size_t)c * nl + l] = 0.0;
    for (int c = 0; c < 14; ++c) T.lcon[(size_t)c * nl + l] = 0.0;
    for (int c = 0; c < 4; ++c) T.lpar[(size_t)c * nl + l] = 0.0;
    for (int c = 0; c < 6; ++c) T.lps[(size_t)c * nl + l] = 0.0;
    return;
  }
  const double mu[9] = {g.gOldPos2.x, g.gOldPos2.y, g.gOldPos2.z, g.gOldA1.x, g.gOldA1.y, g.gOldA1.z,
                        g.gOldA2.x, g.gOldA2.y, g.gOldA2.z};
  for (int c = 0; c < 9; ++c) T.mu[(size_t)c * nl + l] = mu[c];
  const double con[14] = {g.gpn.x, g.gpn.y, g.gpn.z, g.gqn.w, g.gqn.x, g.gqn.y, g.gqn.z,
                          g.gpp.x, g.gpp.y, g.gpp.z, g.gqp.w, g.gqp.x, g.gqp.y, g.gqp.z};
  for (int c = 0; c < 14; ++c) T.lcon[(size_t)c * nl + l] = con[c];
  const double par[4] = {g.gRest, g.gE, g.gDmN, g.gDmP};
  for (int c = 0; c < 4; ++c) T.lpar[(size_t)c * nl + l] = par[c];
  const double lps[6] = {g.gpsn.x, g.gpsn.y, g.gpsn.z, g.gpsp.x, g.gpsp.y, g.gpsp.z};
  for (int c = 0; c < 6; ++c) T.lps[(size_t)c * nl + l] = lps[c];
}

__global__ void k_adj_gather(View S, AdjBuf T, ActParams A, int slot) {
  int v = blockIdx.x * blockDim.x + threadIdx.x;
  const int nv = S.nv, nl = S.nl;
  if (v >= nv) return;
  const vxg_voxel_material& m = S.vm[S.vmat[v]];
  double lam[7] = {0, 0, 0, 0, 0, 0, 0};  // pos 3, orient 4
  double gE = 0, gSqrtMass = 0, gTemp = T.gTempV[v], gP[3] = {0, 0, 0};
  float pdt = T.tpd[(size_t)slot * nv + v];
  for (int i = 0; i < 6; ++i) {
    int l = S.vlinks[i * nv + v];
    if (l < 0) continue;
    bool neg = (i & 1) == 0;  // even slots (X+, Y+, Z+): this voxel is the link's negative end
    int o = neg ? 0 : 7;
    for (int c = 0; c < 7; ++c) lam[c] += T.lcon[(size_t)(o + c) * nl + l];
    for (int c = 0; c < 3; ++c) gP[c] += T.lps[(size_t)((neg ? 0 : 3) + c) * nl + l];
    double gDm = T.lpar[(size_t)(neg ? 2 : 3) * nl + l];
    if (gDm != 0.0) gSqrtMass += gDm * (2.0 * (double)m.zetaInternal / (double)pdt);
    int other = neg ? S.lvox[nl + l] : S.lvox[l];
    double Ea = m.E, Eb = S.vm[S.vmat[other]].E;
    gE += T.lpar[(size_t)nl + l] * (2.0 * Eb * Eb / ((Ea + Eb) * (Ea + Eb)));  // d(2 Ea Eb / (Ea + Eb)) / dEa
    if (A.mode) {
      int axis = (S.lflags[l] >> 8) & 3;
      gTemp += T.lpar[l] * 0.5 * m.size[axis] * (double)m.alphaCTE;
    }
  }
  const int idx[7] = {0, 1, 2, 6, 7, 8, 9};
  for (int c = 0; c < 7; ++c) T.lam[(size_t)idx[c] * nv + v] += lam[c];
  T.accE[v] += gE;
  if (gSqrtMass != 0.0) {
    double volume = m.nomSize * m.nomSize * m.nomSize;
    T.accRho[v] += gSqrtMass * 0.5 / (double)m.sqrtMass * volume;
  }
  if (A.mode == 2) T.accPhase[v] += gTemp * act_dtemp_dphase(A, v, T.ttime[slot]);
  // the Poisson strains this step's links used, where the pre-pass recomputed them (the cache was
  // invalid at the step's start), from the previous step's axial strains: their adjoints, per slot,
  // for that step's link adjoint (elsewhere the cache is a constant: nothing flows back)
  double ge[6] = {0, 0, 0, 0, 0, 0};
  if (m.nu != 0.0f && (T.tvf[(size_t)slot * nv + v] & VXG_VF_PSTRAIN_INVALID) && (gP[0] != 0 || gP[1] != 0 || gP[2] != 0)) {
    float e[6];
    bool has[6], extT[3] = {false, false, false};
    for (int i = 0; i < 6; ++i) {
      const int l = S.vlinks[i * nv + v];
      has[i] = l >= 0;
      e[i] = 0.0f;
      if (has[i]) {  // vx64::link_axial_strain at this voxel's end
        const float s = T.tstrain[(size_t)slot * nl + l], r = S.strainRatio[l];
        e[i] = (i & 1) ? 2.0f * s * r / (1.0f + r) : 2.0f * s / (1.0f + r);
      }
    }
    const int ei = S.vext[v];
    if (ei >= 0)
      for (int i = 0; i < 3; ++i) extT[i] = (S.ext[ei].dof & (1 << i)) != 0 || S.ext[ei].force[i] != 0;
    vxa::poisson_adjoint(e, has, extT, m.nu, gP, ge);
  }
  for (int c = 0; c < 6; ++c) T.gS[(size_t)c * nv + v] = ge[c];
}

// After k_adj_gather, where some Poisson's ratio is not 0: the end strains a voxel's Poisson strains
// read are 2 s / (1 + r) and 2 s r / (1 + r) with the link's strain ratio r = E(positive voxel) /
// E(negative voxel) (CVX_Link::axialStrain): their adjoints (gS, this step) reach both voxels'
// Young's moduli through r.  One thread per voxel over its links, so no atomics.
__global__ void k_adj_ratio(View S, AdjBuf T, int slot) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  const int nv = S.nv, nl = S.nl;
  if (v >= nv) return;
  const double Ev = S.vm[S.vmat[v]].E;
  double g = 0;
  for (int i = 0; i < 6; ++i) {
    const int l = S.vlinks[i * nv + v];
    if (l < 0) continue;
    const int a = i / 2, vn = S.lvox[l], vp = S.lvox[nl + l];
    const double s = T.tstrain[(size_t)slot * nl + l], r = S.strainRatio[l];
    const double d = 2.0 * s / ((1.0 + r) * (1.0 + r));  // -d(2 s / (1 + r))/dr = d(2 s r / (1 + r))/dr
    const double gr = -T.gS[(size_t)(2 * a) * nv + vn] * d + T.gS[(size_t)(2 * a + 1) * nv + vp] * d;
    g += (v == vp ? 1.0 : -1.0) * gr * r / Ev;
  }
  T.accE[v] += g;
}

// Objective: sum over bodies of the mass-weighted centre-of-mass x.  One block per body (contiguous
// voxel range); sets the final-state adjoint (d/dx = m / M) and the density term of the weights.
__global__ void k_adj_objective(View S, AdjBuf T, const int* off, double* obj) {
  int b = blockIdx.x;
  int lo = off[b], hi = off[b + 1];
  __shared__ double sh[2][32];
  double msum = 0, mx = 0;
  for (int v = lo + threadIdx.x; v < hi; v += blockDim.x) {
    double mv = S.vm[S.vmat[v]].mass;
    msum += mv;
    mx += mv * S.pos[v];
  }
  for (int o = 16; o > 0; o >>= 1) {
    msum += __shfl_xor_sync(0xffffffffu, msum, o);
    mx += __shfl_xor_sync(0xffffffffu, mx, o);
  }
  int w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  if ((threadIdx.x & 31) == 0) { sh[0][w] = msum; sh[1][w] = mx; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 1; k < nw; ++k) { msum += sh[0][k]; mx += sh[1][k]; }
    sh[0][0] = msum;
    sh[1][0] = mx;
  }
  __syncthreads();
  msum = sh[0][0];
  mx = sh[1][0];
  double com = msum > 0 ? mx / msum : 0.0;
  if (threadIdx.x == 0) obj[b] = com;
  if (msum <= 0) return;
  const int nv = S.nv;
  for (int v = lo + threadIdx.x; v < hi; v += blockDim.x) {
    const vxg_voxel_material& m = S.vm[S.vmat[v]];
    T.lam[v] = (double)m.mass / msum;
    double volume = m.nomSize * m.nomSize * m.nomSize;
    T.accRho[v] += (S.pos[v] - com) / msum * volume;
  }
  (void)nv;
}

}  // namespace
