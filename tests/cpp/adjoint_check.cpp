// Host-side checks of the hand-written step adjoint (voxelyze_gb300/csrc/vx_adjoint.cuh):
//  1. link_forward / voxel_forward reproduce vx64::link_update / vx64::voxel_update bit for bit
//     (links small- and large-angle, with and without Poisson's ratio or a failure strain; voxels
//     with and without partial fixes);
//  2. link_adjoint / voxel_adjoint agree with central finite differences of those forwards, output
//     by output, input by input (the large-angle links in a check of their own, "link_large");
//  3. poisson_adjoint agrees with differences of vx64::poisson_strain_links over its links' strains.
// Prints one line per check: "<name> <worst relative error> <entries> <cases>"; exits 1 on a
// forward mismatch.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <vector>

#include "vx_adjoint.cuh"

using namespace vxa;

static std::mt19937_64 rng(12345);
static double U(double a, double b) { return std::uniform_real_distribution<double>(a, b)(rng); }

static q4 small_rotation(double mag) {
  d3 r = D3(U(-mag, mag), U(-mag, mag), U(-mag, mag));
  return vxa::from_rotation_vector(r);
}

struct LinkConsts {
  float E, a2, b1, b2, b3, sqA1, sqA2xIp, sqB1, sqB2xFMp, sqB3xIp;
};
// CVX_MaterialLink::updateDerived for nu = 0 (float arithmetic, as the host derives it)
static LinkConsts link_consts(float E, float L) {
  LinkConsts c;
  c.E = E;
  float a1 = E * L;
  c.a2 = E * L * L * L / (12.0f * (1 + 0.0f));
  c.b1 = E * L;
  c.b2 = E * L * L / 2.0f;
  c.b3 = E * L * L * L / 6.0f;
  c.sqA1 = std::sqrt(a1);
  c.sqA2xIp = std::sqrt(c.a2 * L * L / 6.0f);
  c.sqB1 = std::sqrt(c.b1);
  c.sqB2xFMp = std::sqrt(c.b2 * L / 2.0f);
  c.sqB3xIp = std::sqrt(c.b3 * L * L / 6.0f);
  return c;
}
static void set_consts(LinkIn& in, const LinkConsts& c) {
  in.E = c.E; in.a2 = c.a2; in.b1 = c.b1; in.b2 = c.b2; in.b3 = c.b3;
  in.sqA1 = c.sqA1; in.sqA2xIp = c.sqA2xIp; in.sqB1 = c.sqB1; in.sqB2xFMp = c.sqB2xFMp; in.sqB3xIp = c.sqB3xIp;
}

static const double L0 = 0.01;

// kind 0: small-angle; 1: large-angle, bent so that orientLink's frame comes from its near-x
// formula; 2: large-angle, bent further (its general formula)
static LinkIn random_link(int kind = 0) {
  LinkIn in;
  in.axis = (int)(rng() % 3);
  d3 e = D3(in.axis == 0, in.axis == 1, in.axis == 2);
  in.pn = D3(U(-0.05, 0.05), U(-0.05, 0.05), U(0.0, 0.05));
  double ext = L0 * (1 + U(-2e-3, 2e-3));
  q4 base = small_rotation(0.3);
  d3 d = vx64::rotate(base, D3(ext * e.x + U(-2e-5, 2e-5), ext * e.y + U(-2e-5, 2e-5), ext * e.z + U(-2e-5, 2e-5)));
  in.pp = D3(in.pn.x + d.x, in.pn.y + d.y, in.pn.z + d.z);
  // relative rotation of the two ends ~0.05 rad: 1 - w of it stays well above the difference steps
  in.qn = vx64::qmul(small_rotation(0.01), base);
  in.qp = vx64::qmul(small_rotation(0.06), base);
  in.oldPos2 = D3(U(-2e-5, 2e-5), U(-2e-5, 2e-5), U(-2e-5, 2e-5));
  in.oldA1 = D3(0, 0, 0);
  if (rng() % 4 == 0) in.oldA1 = D3(U(-1e-3, 1e-3), U(-1e-3, 1e-3), U(-1e-3, 1e-3));
  in.oldA2 = D3(U(-1e-2, 1e-2), U(-1e-2, 1e-2), U(-1e-2, 1e-2));
  in.rest = L0 * (1 + U(-1e-3, 1e-3));
  in.smallAngle = true;
  // one link in four has a failure strain: half of them failed already (largest strain so far
  // 2e-3 against 1e-3), half far from failing
  in.maxStrain = 0.0f;
  in.epsilonFail = -1.0f;
  // one link in three (with either kind) has Poisson's ratio 0.3 with its ends' Poisson strains
  in.nu = 0.0f;
  in.eHat = 0.0f;
  in.sizeN = in.sizeP = (float)L0;
  in.nuN = in.nuP = false;
  in.psn = in.psp = D3(0, 0, 0);
  if (rng() % 3 == 0) {
    in.nu = 0.3f;
    in.nuN = in.nuP = true;
    in.psn = D3((float)U(-1e-3, 1e-3), (float)U(-1e-3, 1e-3), (float)U(-1e-3, 1e-3));
    in.psp = D3((float)U(-1e-3, 1e-3), (float)U(-1e-3, 1e-3), (float)U(-1e-3, 1e-3));
  }
  if (rng() % 4 == 0) {
    const bool failed = rng() % 2;
    in.maxStrain = failed ? 2e-3f : 0.0f;
    in.epsilonFail = failed ? 1e-3f : 0.9f;
  }
  if (kind) {
    // kind 2: bent, the positive end displaced sideways by 0.2-0.5 of the length (the bend far past
    // the hysteresis bound 1.2 x 0.05); kind 1: stretched by 60 % (past the extension bound 0.5)
    // and barely bent, |y| and |z| below 1.732e-2 of x in the link frame (the near-x frame formula)
    const double side = U(0.2, 0.5);
    d3 off = D3(U(-1, 1), U(-1, 1), U(-1, 1));
    d3 loc = D3(ext, side * ext * (off.y > 0 ? 1 : -1), side * ext * off.z);
    if (kind == 1) {
      const double x = 1.6 * ext;
      loc = D3(x, 5e-3 * x * (off.y > 0 ? 1 : -1), 4e-3 * x * (off.z > 0 ? 1 : -1));
      in.qn = base;
    }
    // loc in the link frame (x along the axis) to world axes
    d3 w = in.axis == 0 ? loc : in.axis == 1 ? D3(loc.z, loc.x, loc.y) : D3(loc.y, loc.z, loc.x);
    d3 dw = vx64::rotate(base, w);
    in.pp = D3(in.pn.x + dw.x, in.pn.y + dw.y, in.pn.z + dw.z);
    in.qp = vx64::qmul(small_rotation(0.3), base);
    in.smallAngle = false;
    in.oldA1 = D3(U(-0.2, 0.2), U(-0.2, 0.2), U(-0.2, 0.2));
    in.oldA2 = D3(U(-0.2, 0.2), U(-0.2, 0.2), U(-0.2, 0.2));
    in.oldPos2 = D3(U(-1e-4, 1e-4), 0, 0);
  }
  in.lvv = rng() % 4 != 0;
  set_consts(in, link_consts((float)std::exp(U(std::log(3e5), std::log(3e6))), (float)L0));
  in.eHat = in.E / ((1 - 2 * in.nu) * (1 + in.nu));
  in.tArea = (float)(L0 * L0);
  double m = 1000.0 * L0 * L0 * L0;
  float dt = 2e-5f;
  in.dmN = 2 * (float)std::sqrt(m) * 1.0f / dt;
  in.dmP = 2 * (float)std::sqrt(m * 1.7) * 0.8f / dt;
  return in;
}

// vx64::link_update on a one-link host View built from a LinkIn
static LinkOut engine_link(const LinkIn& in) {
  double pos[6] = {in.pn.x, in.pp.x, in.pn.y, in.pp.y, in.pn.z, in.pp.z};
  double orient[8] = {in.qn.w, in.qp.w, in.qn.x, in.qp.x, in.qn.y, in.qp.y, in.qn.z, in.qp.z};
  double pos2[3] = {in.oldPos2.x, in.oldPos2.y, in.oldPos2.z}, a1v[3] = {in.oldA1.x, in.oldA1.y, in.oldA1.z},
         a2v[3] = {in.oldA2.x, in.oldA2.y, in.oldA2.z};
  double fN[3], fP[3], mN[3], mP[3], rest[1] = {in.rest};
  float strain[1] = {0}, maxStrain[1] = {in.maxStrain}, strainOffset[1] = {0}, stress[1] = {0}, ratio[1] = {1},
        tArea[1] = {in.tArea}, tSS[1] = {0}, temp[2] = {0, 0}, prevDt[2];
  float pStrain[6] = {(float)in.psn.x, (float)in.psp.x, (float)in.psn.y, (float)in.psp.y, (float)in.psn.z,
                      (float)in.psp.z};
  uint32_t lflags[1] = {(uint32_t)(in.axis << 8) | (in.smallAngle ? VXG_LF_SMALL_ANGLE : 0u) |
                        (in.lvv ? VXG_LF_LOCAL_VEL_VALID : 0u)};
  int lvox[2] = {0, 1}, lmat[1] = {0}, vmat[2] = {0, 1};
  vxg_link_material lm;
  std::memset(&lm, 0, sizeof(lm));
  lm.linear = 1; lm.ndata = 2; lm.E = in.E; lm.nu = in.nu; lm.eHat = in.eHat; lm.epsilonFail = in.epsilonFail;
  lm.a2 = in.a2; lm.b1 = in.b1; lm.b2 = in.b2; lm.b3 = in.b3;
  lm.sqA1 = in.sqA1; lm.sqA2xIp = in.sqA2xIp; lm.sqB1 = in.sqB1; lm.sqB2xFMp = in.sqB2xFMp; lm.sqB3xIp = in.sqB3xIp;
  lm.strain[1] = 1e30f;
  vxg_voxel_material vm[2];
  std::memset(vm, 0, sizeof(vm));
  // damping_multiplier = 2 sqrtMass zetaInternal / prevDt: choose values that reproduce dmN, dmP
  vm[0].sqrtMass = in.dmN / 2.0f; vm[0].zetaInternal = 1.0f; prevDt[0] = 1.0f;
  vm[1].sqrtMass = in.dmP / 2.0f; vm[1].zetaInternal = 1.0f; prevDt[1] = 1.0f;
  vm[0].nu = in.nuN ? 0.3f : 0.0f; vm[0].nomSize = in.sizeN;
  vm[1].nu = in.nuP ? 0.3f : 0.0f; vm[1].nomSize = in.sizeP;
  vx64::Ctl ctl;
  std::memset(&ctl, 0, sizeof(ctl));
  vx64::View S;
  std::memset(&S, 0, sizeof(S));
  S.nv = 2; S.nl = 1; S.vmat = vmat; S.pos = pos; S.orient = orient; S.temp = temp; S.prevDt = prevDt;
  S.pStrain = pStrain; S.lvox = lvox; S.lmat = lmat; S.lflags = lflags; S.pos2 = pos2; S.a1v = a1v; S.a2v = a2v;
  S.fN = fN; S.fP = fP; S.mN = mN; S.mP = mP; S.rest = rest; S.strain = strain; S.maxStrain = maxStrain;
  S.strainOffset = strainOffset; S.stress = stress; S.strainRatio = ratio; S.tArea = tArea; S.tSS = tSS;
  S.vm = vm; S.lm = &lm; S.ctl = &ctl;
  vx64::link_update(S, 0);
  LinkOut o;
  o.fN = D3(fN[0], fN[1], fN[2]); o.fP = D3(fP[0], fP[1], fP[2]);
  o.mN = D3(mN[0], mN[1], mN[2]); o.mP = D3(mP[0], mP[1], mP[2]);
  o.pos2 = D3(pos2[0], pos2[1], pos2[2]); o.a1v = D3(a1v[0], a1v[1], a1v[2]); o.a2v = D3(a2v[0], a2v[1], a2v[2]);
  o.smallAngle = lflags[0] & VXG_LF_SMALL_ANGLE;
  o.lvv = lflags[0] & VXG_LF_LOCAL_VEL_VALID;
  return o;
}

static bool same(const d3& a, const d3& b) { return a.x == b.x && a.y == b.y && a.z == b.z; }

// Worst relative error of adjoint against central differences with one-hot output seeds: for
// output k, the adjoint's gradient over all inputs is compared with differences of output k alone;
// the floor is 1e-4 of that output's largest gradient component (float roundings inside the
// forward make differences of smaller components noisy).
struct Check {
  const char* name;
  double err = 0;
  int n = 0;
  int tag = 0;
  double floor_frac = 1e-4;
  void row(const std::vector<double>& fd, const std::vector<double>& ad) {
    double big = 0;
    for (double x : ad) big = std::max(big, std::fabs(x));
    for (double x : fd) big = std::max(big, std::fabs(x));
    if (big == 0) return;
    for (size_t i = 0; i < fd.size(); ++i) {
      double e = std::fabs(fd[i] - ad[i]) / std::max(std::max(std::fabs(fd[i]), std::fabs(ad[i])), floor_frac * big);
      if (e > err) {
        err = e;
        if (std::getenv("ADJ_VERBOSE")) printf("  %s worst so far: output %d input %zu fd %.9e ad %.9e\n", name, tag, i, fd[i], ad[i]);
      }
      n++;
    }
  }
};

static double link_out(const LinkOut& o, int k) {
  if (k == 21) return o.axial;
  const d3 O[7] = {o.fN, o.fP, o.mN, o.mP, o.pos2, o.a1v, o.a2v};
  const double v[3] = {O[k / 3].x, O[k / 3].y, O[k / 3].z};
  return v[k % 3];
}
static double voxel_out(const VoxelOut& o, int k) {
  const double v[13] = {o.pos.x, o.pos.y, o.pos.z, o.lin.x, o.lin.y, o.lin.z, o.ang.x, o.ang.y, o.ang.z,
                        o.orient.w, o.orient.x, o.orient.y, o.orient.z};
  return v[k];
}

int main() {
  int bad_forward = 0, link_cases = 0;
  Check cl{"link"};
  // large-angle links: strains of 0.1-0.6 and damping forces ~1e3 N make the differences of the
  // smallest gradient components noisy, so their floor is 1e-3 of each output's largest component
  Check cll{"link_large"};
  cll.floor_frac = 1e-3;
  int large_cases = 0;
  for (int c = 0; c < 300; ++c) {
    const int kind = c % 3;  // small-angle, large-angle near-x frame, large-angle general frame
    LinkIn in = random_link(kind);
    LinkOut a = link_forward(in), b = engine_link(in);
    if (!(same(a.fN, b.fN) && same(a.fP, b.fP) && same(a.mN, b.mN) && same(a.mP, b.mP) && same(a.pos2, b.pos2) &&
          same(a.a1v, b.a1v) && same(a.a2v, b.a2v) && a.smallAngle == b.smallAngle && a.lvv == b.lvv))
      bad_forward++;
    if (a.smallAngle != (kind == 0)) continue;  // stayed in the branch its kind aims at
    if (c % 4 && kind == 0) continue;  // derivative checks on every fourth small-angle case, every large one
    link_cases++;
    if (kind) large_cases++;
    for (int k = 0; k < 22; ++k) {  // the 21 pose, force and moment components, then the axial strain
      d3 s[7] = {D3(0, 0, 0), D3(0, 0, 0), D3(0, 0, 0), D3(0, 0, 0), D3(0, 0, 0), D3(0, 0, 0), D3(0, 0, 0)};
      if (k < 21) (k % 3 == 0 ? s[k / 3].x : k % 3 == 1 ? s[k / 3].y : s[k / 3].z) = 1.0;
      LinkGrad g;
      if (!link_adjoint(in, s[0], s[1], s[2], s[3], s[4], s[5], s[6], k == 21 ? 1.0 : 0.0, g)) continue;
      // steps large enough that the float-rounded axial strain and stress change by many ulps (a
      // large-angle link carries a strain of ~0.1-0.6, so its steps are larger; its rotation vectors
      // and frame formulas have kinks within 1e-4 of a quaternion component)
      const double hs = kind ? 100.0 : 1.0, hq = kind ? 3.0 : 1.0;
      std::vector<double> fd, ad;
      auto J = [&](const LinkIn& x) { return link_out(link_forward(x), k); };
      // a large-angle link's difference is taken at six steps (10 h down to h / 30) and the one
      // nearest the adjoint kept: rounding noise grows as the step shrinks, and the kinks of the
      // frame and rotation-vector formulas sit within the larger steps of some inputs
      auto dd = [&](double* x, double h, double grad) {
        double x0 = *x, best = 0;
        const double scales[6] = {1.0, 10.0, 3.0, 1.0 / 3, 0.1, 1.0 / 30};
        for (int t = 0; t < (kind ? 6 : 1); ++t) {
          const double hh = h * scales[t];
          *x = x0 + hh; double jp = J(in);
          *x = x0 - hh; double jm = J(in);
          *x = x0;
          const double d = (jp - jm) / (2 * hh);
          if (t == 0 || std::fabs(d - grad) < std::fabs(best - grad)) best = d;
        }
        fd.push_back(best);
        ad.push_back(grad);
      };
      dd(&in.pn.x, 1e-7 * hs, g.gpn.x); dd(&in.pn.y, 1e-7 * hs, g.gpn.y); dd(&in.pn.z, 1e-7 * hs, g.gpn.z);
      dd(&in.pp.x, 1e-7 * hs, g.gpp.x); dd(&in.pp.y, 1e-7 * hs, g.gpp.y); dd(&in.pp.z, 1e-7 * hs, g.gpp.z);
      dd(&in.qn.w, 1e-5 * hq, g.gqn.w); dd(&in.qn.x, 1e-5 * hq, g.gqn.x); dd(&in.qn.y, 1e-5 * hq, g.gqn.y);
      dd(&in.qn.z, 1e-5 * hq, g.gqn.z);
      dd(&in.qp.w, 1e-5 * hq, g.gqp.w); dd(&in.qp.x, 1e-5 * hq, g.gqp.x); dd(&in.qp.y, 1e-5 * hq, g.gqp.y);
      dd(&in.qp.z, 1e-5 * hq, g.gqp.z);
      dd(&in.oldPos2.x, 1e-8 * hs, g.gOldPos2.x); dd(&in.oldPos2.y, 1e-8 * hs, g.gOldPos2.y);
      dd(&in.oldPos2.z, 1e-8 * hs, g.gOldPos2.z);
      dd(&in.oldA1.x, 1e-6 * hq, g.gOldA1.x); dd(&in.oldA1.y, 1e-6 * hq, g.gOldA1.y); dd(&in.oldA1.z, 1e-6 * hq, g.gOldA1.z);
      dd(&in.oldA2.x, 1e-6 * hq, g.gOldA2.x); dd(&in.oldA2.y, 1e-6 * hq, g.gOldA2.y); dd(&in.oldA2.z, 1e-6 * hq, g.gOldA2.z);
      dd(&in.rest, 1e-7 * hs, g.gRest);
      if (in.nu != 0.0f) {  // the ends' Poisson strains (floats, so steps of many ulps)
        dd(&in.psn.x, 1e-4, g.gpsn.x); dd(&in.psn.y, 1e-4, g.gpsn.y); dd(&in.psn.z, 1e-4, g.gpsn.z);
        dd(&in.psp.x, 1e-4, g.gpsp.x); dd(&in.psp.y, 1e-4, g.gpsp.y); dd(&in.psp.z, 1e-4, g.gpsp.z);
      }
      {
        float E0 = in.E;
        double h = 1e-3;
        set_consts(in, link_consts((float)(E0 * (1 + h)), (float)L0)); double jp = J(in);
        set_consts(in, link_consts((float)(E0 * (1 - h)), (float)L0)); double jm = J(in);
        set_consts(in, link_consts(E0, (float)L0));
        fd.push_back((jp - jm) / (2 * h * E0));
        ad.push_back(g.gE);
      }
      for (int side = 0; side < 2; ++side) {
        float* d = side ? &in.dmP : &in.dmN;
        float d0 = *d;
        *d = d0 * 1.001f; double hp = *d - d0; double jp = J(in);
        *d = d0 * 0.999f; double hm = d0 - *d; double jm = J(in);
        *d = d0;
        fd.push_back((jp - jm) / (hp + hm));
        ad.push_back(side ? g.gDmP : g.gDmN);
      }
      Check& ck = kind ? cll : cl;
      ck.tag = k;
      ck.row(fd, ad);
    }
  }
  printf("link_forward_mismatch %d 300\n", bad_forward);
  printf("%s %.3e %d %d\n", cl.name, cl.err, cl.n, link_cases);
  printf("%s %.3e %d %d\n", cll.name, cll.err, cll.n, large_cases);

  int bad_vforward = 0, vcases = 0;
  Check cv{"voxel"};
  for (int c = 0; c < 400; ++c) {
    VoxelIn in;
    double m = 1000.0 * L0 * L0 * L0 * U(0.5, 2.0);
    double E = std::exp(U(std::log(3e5), std::log(3e6)));
    float mass = (float)m, inertia = (float)(mass * L0 * L0 / 6.0f);
    in.mass = mass; in.massInv = 1.0f / mass; in.inertiaInv = 1.0f / inertia;
    in.c2xSqMxExS = (float)(2.0f * std::sqrt(mass * (float)E * (float)L0));
    in.c2xSqIxExSxSxS = (float)(2.0f * std::sqrt(inertia * (float)E * (float)(L0 * L0 * L0)));
    in.zetaGlobal = (rng() % 2) ? 0.1f : 0.0f;
    in.zetaCollision = (rng() % 2) ? 0.5f : 0.0f;
    in.gravMult = 1.0f;
    in.penetrationStiffness = (float)(2 * E * L0);
    in.muStatic = 1.0f; in.muKinetic = 0.5f;
    in.dt = 2e-5f;
    in.floorOn = rng() % 4 != 0;
    in.staticF = rng() % 2;
    double off = U(-1e-5, 1e-5);
    in.lin = D3(U(-1e-4, 1e-4), U(-1e-4, 1e-4), U(-1e-4, 1e-4));
    in.ang = D3(U(-1e-8, 1e-8), U(-1e-8, 1e-8), U(-1e-8, 1e-8));
    if (rng() % 3 == 0) in.ang = D3(U(-1e-5, 1e-5), U(-1e-5, 1e-5), U(-1e-5, 1e-5));
    in.orient = small_rotation(0.5);
    in.Fl = D3(U(-0.02, 0.02), U(-0.02, 0.02), U(-0.02, 0.02));
    in.Ml = D3(U(-1e-4, 1e-4), U(-1e-4, 1e-4), U(-1e-4, 1e-4));
    in.extF = D3(0, 0, 0);
    in.extM = D3(0, 0, 0);
    // every third case an external that fixes some degrees of freedom (all but all six)
    vxg_external ext;
    std::memset(&ext, 0, sizeof(ext));
    in.dof = 0;
    in.fixPos = D3(0, 0, 0);
    in.fixOrient = Q4(1, 0, 0, 0);
    if (c % 3 == 1) {
      static const int dofs[16] = {1, 2, 4, 3, 5, 6, 8, 16, 32, 24, 40, 48, 56, 7 | 8, 4 | 56, 1 | 32};
      in.dof = dofs[rng() % 16];
      ext.dof = in.dof;
      for (int k = 0; k < 3; ++k) ext.translation[k] = U(-1e-4, 1e-4);
      q4 r = small_rotation(0.3);
      ext.rotq[0] = r.w; ext.rotq[1] = r.x; ext.rotq[2] = r.y; ext.rotq[3] = r.z;
      in.fixPos = D3(ext.translation[0], ext.translation[1], ext.translation[2]);  // at lattice index 0
      in.fixOrient = r;
    }
    {  // the engine forward on a one-voxel View whose single link slot carries Fl, Ml
      vxg_voxel_material vm;
      std::memset(&vm, 0, sizeof(vm));
      vm.mass = in.mass; vm.massInv = in.massInv; vm.inertiaInv = in.inertiaInv; vm.c2xSqMxExS = in.c2xSqMxExS;
      vm.c2xSqIxExSxSxS = in.c2xSqIxExSxSxS; vm.zetaGlobal = in.zetaGlobal; vm.zetaCollision = in.zetaCollision;
      vm.gravMult = in.gravMult; vm.penetrationStiffness = in.penetrationStiffness; vm.muStatic = in.muStatic;
      vm.muKinetic = in.muKinetic;
      vm.nomSize = L0;
      vm.size[0] = vm.size[1] = vm.size[2] = L0 + 2 * off;
      int vlinks[6] = {0, -1, -1, -1, -1, -1}, vmat[1] = {0}, vidx[3] = {0, 0, 0}, vext[1] = {in.dof ? 0 : -1};
      float temp[1] = {0}, prevDt[1] = {0};
      vx64::Ctl ctl;
      std::memset(&ctl, 0, sizeof(ctl));
      vx64::View S;
      std::memset(&S, 0, sizeof(S));
      S.nv = 1; S.nl = 1; S.vmat = vmat; S.vidx = vidx; S.vlinks = vlinks; S.vext = vext; S.temp = temp;
      S.prevDt = prevDt; S.vm = &vm; S.ctl = &ctl; S.ext = &ext;
      in.halfPenOffset = vx64::base_size_avg(S, 0) / 2 - vm.nomSize / 2;
      in.pos = D3(U(-0.1, 0.1), U(-0.1, 0.1), in.halfPenOffset + U(-3e-5, 3e-5));
      double pos[3] = {in.pos.x, in.pos.y, in.pos.z}, lin[3] = {in.lin.x, in.lin.y, in.lin.z},
             ang[3] = {in.ang.x, in.ang.y, in.ang.z}, orient[4] = {in.orient.w, in.orient.x, in.orient.y, in.orient.z};
      double fN[3] = {in.Fl.x, in.Fl.y, in.Fl.z}, mN[3] = {in.Ml.x, in.Ml.y, in.Ml.z}, fP[3] = {0, 0, 0}, mP[3] = {0, 0, 0};
      uint32_t vflags[1] = {(in.floorOn ? VXG_VF_FLOOR : 0u) | (in.staticF ? VXG_VF_STATIC_FRICTION : 0u)};
      S.vflags = vflags; S.pos = pos; S.linMom = lin; S.orient = orient; S.angMom = ang;
      S.fN = fN; S.fP = fP; S.mN = mN; S.mP = mP;
      vx64::voxel_update(S, 0, in.dt);
      VoxelOut a = voxel_forward(in);
      if (!(same(a.pos, D3(pos[0], pos[1], pos[2])) && same(a.lin, D3(lin[0], lin[1], lin[2])) &&
            same(a.ang, D3(ang[0], ang[1], ang[2])) && a.orient.w == orient[0] && a.orient.x == orient[1] &&
            a.orient.y == orient[2] && a.orient.z == orient[3] &&
            a.staticF == ((vflags[0] & VXG_VF_STATIC_FRICTION) != 0)))
        bad_vforward++;
    }
    double pen = in.halfPenOffset - in.pos.z;
    if (std::fabs(pen) < 1e-7 || c % 4) continue;  // finite differences stay on one side of the contact test
    bool sf0 = voxel_forward(in).staticF;
    bool flipped = false;
    std::vector<std::vector<double>> FD(13), AD(13);
    for (int k = 0; k < 13; ++k) {
      d3 gp = D3(0, 0, 0), gl = D3(0, 0, 0), ga = D3(0, 0, 0);
      q4 gq = Q4(0, 0, 0, 0);
      double* seed[13] = {&gp.x, &gp.y, &gp.z, &gl.x, &gl.y, &gl.z, &ga.x, &ga.y, &ga.z, &gq.w, &gq.x, &gq.y, &gq.z};
      *seed[k] = 1.0;
      VoxelGrad g;
      voxel_adjoint(in, gp, gl, gq, ga, g);
      auto J = [&](bool* sf) { VoxelOut o = voxel_forward(in); *sf = o.staticF; return voxel_out(o, k); };
      auto dd = [&](double* x, double h, double grad) {
        double x0 = *x;
        bool s1, s2;
        *x = x0 + h; double jp = J(&s1);
        *x = x0 - h; double jm = J(&s2);
        *x = x0;
        if (s1 != sf0 || s2 != sf0) flipped = true;
        FD[k].push_back((jp - jm) / (2 * h));
        AD[k].push_back(grad);
      };
      auto df = [&](float* x, double grad) {
        float x0 = *x;
        bool s1, s2;
        *x = x0 * 1.001f; double hp = (double)*x - x0; double jp = J(&s1);
        *x = x0 * 0.999f; double hm = x0 - (double)*x; double jm = J(&s2);
        *x = x0;
        if (s1 != sf0 || s2 != sf0) flipped = true;
        FD[k].push_back((jp - jm) / (hp + hm));
        AD[k].push_back(grad);
      };
      dd(&in.pos.x, 1e-8, g.gpos.x); dd(&in.pos.y, 1e-8, g.gpos.y); dd(&in.pos.z, 1e-8, g.gpos.z);
      dd(&in.lin.x, 1e-9, g.glin.x); dd(&in.lin.y, 1e-9, g.glin.y); dd(&in.lin.z, 1e-9, g.glin.z);
      dd(&in.ang.x, 1e-11, g.gang.x); dd(&in.ang.y, 1e-11, g.gang.y); dd(&in.ang.z, 1e-11, g.gang.z);
      dd(&in.orient.w, 1e-7, g.gorient.w); dd(&in.orient.x, 1e-7, g.gorient.x);
      dd(&in.orient.y, 1e-7, g.gorient.y); dd(&in.orient.z, 1e-7, g.gorient.z);
      dd(&in.Fl.x, 1e-6, g.gFl.x); dd(&in.Fl.y, 1e-6, g.gFl.y); dd(&in.Fl.z, 1e-6, g.gFl.z);
      dd(&in.Ml.x, 1e-8, g.gMl.x); dd(&in.Ml.y, 1e-8, g.gMl.y); dd(&in.Ml.z, 1e-8, g.gMl.z);
      df(&in.mass, g.gMass); df(&in.massInv, g.gMassInv); df(&in.inertiaInv, g.gInertiaInv);
      df(&in.c2xSqMxExS, g.gC2x); df(&in.c2xSqIxExSxSxS, g.gC2xI); df(&in.penetrationStiffness, g.gPenStiff);
      dd(&in.halfPenOffset, 1e-8, g.gHalfPenOffset);
    }
    if (flipped) continue;
    vcases++;
    for (int k = 0; k < 13; ++k) cv.row(FD[k], AD[k]);
  }
  printf("voxel_forward_mismatch %d 400\n", bad_vforward);
  printf("%s %.3e %d %d\n", cv.name, cv.err, cv.n, vcases);

  // the Poisson strains of a voxel (vx64::poisson_strain_links on a one-voxel View whose six slots
  // hold links 0..5, some absent) against poisson_adjoint, per slot strain
  Check cp{"poisson"};
  int pcases = 0;
  for (int c = 0; c < 300; ++c) {
    float strain[6], ratio[6];
    int lk[6];
    bool has[6], extT[3];
    for (int i = 0; i < 6; ++i) {
      has[i] = rng() % 5 != 0;
      lk[i] = has[i] ? i : -1;
      strain[i] = (float)U(-2e-3, 2e-3);
      ratio[i] = (float)std::exp(U(std::log(0.5), std::log(2.0)));
    }
    vxg_external ext;
    std::memset(&ext, 0, sizeof(ext));
    int vext[1] = {-1};
    if (rng() % 2) {
      vext[0] = 0;
      ext.dof = (int)(rng() % 8);
      ext.force[rng() % 3] = 0.01f;
    }
    for (int i = 0; i < 3; ++i) extT[i] = vext[0] >= 0 && ((ext.dof & (1 << i)) != 0 || ext.force[i] != 0);
    vxg_voxel_material vm;
    std::memset(&vm, 0, sizeof(vm));
    vm.nu = 0.3f;
    vm.powf_slot = -1;
    int vmat[1] = {0};
    vx64::Ctl ctl;
    std::memset(&ctl, 0, sizeof(ctl));
    vx64::View S;
    std::memset(&S, 0, sizeof(S));
    S.nv = 1; S.nl = 6; S.vmat = vmat; S.vext = vext; S.ext = &ext; S.vm = &vm; S.ctl = &ctl;
    S.strain = strain; S.strainRatio = ratio;
    auto P = [&](int k) { float out[3]; vx64::poisson_strain_links(S, 0, lk, out); return (double)out[k]; };
    for (int k = 0; k < 3; ++k) {
      double gP[3] = {0, 0, 0};
      gP[k] = 1.0;
      float e[6];
      for (int i = 0; i < 6; ++i) e[i] = (i & 1) ? 2.0f * strain[i] * ratio[i] / (1.0f + ratio[i]) : 2.0f * strain[i] / (1.0f + ratio[i]);
      double ge[6] = {0, 0, 0, 0, 0, 0};
      poisson_adjoint(e, has, extT, vm.nu, gP, ge);
      std::vector<double> fd, ad;
      for (int i = 0; i < 6; ++i) {
        if (!has[i]) continue;
        const double r = ratio[i];
        const double de = (i & 1) ? 2.0 * r / (1.0 + r) : 2.0 / (1.0 + r);  // d(end strain)/d(strain)
        float s0 = strain[i];  // a wide step: the result is powf(1 + sum, -nu) - 1 rounded to float
        strain[i] = s0 + 4e-4f; double hp = (double)strain[i] - s0; double jp = P(k);
        strain[i] = s0 - 4e-4f; double hm = s0 - (double)strain[i]; double jm = P(k);
        strain[i] = s0;
        fd.push_back((jp - jm) / (hp + hm));
        ad.push_back(ge[i] * de);
      }
      cp.tag = k;
      cp.row(fd, ad);
    }
    pcases++;
  }
  printf("%s %.3e %d %d\n", cp.name, cp.err, cp.n, pcases);
  return (bad_forward || bad_vforward) ? 1 : 0;
}
