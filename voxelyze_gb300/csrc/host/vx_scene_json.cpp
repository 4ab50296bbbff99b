// *.vxl.json scene files for the drop-in CVoxelyze: loadJSON / saveJSON and the JSON constructor
// (src/Voxelyze.cpp:61-241, src/VX_Material.cpp:75-160, include/Voxelyze.h:70-78).
//
// The format, the keys, which of them are read back and the order in which they are written follow
// the reference, so the same scene saves to the same bytes (see vx_json.h for the number layout).
// Reading follows the reference's rules for value kinds: a key is used only when its value has the
// kind the reference tests for (youngsModulus, density, ... must be written as doubles, colours as
// integers), otherwise it is skipped.  Deliberate differences:
//   * strainData / stressData are read element by element (the reference calls GetDouble on the
//     whole array, so a data-model material never loads there);
//   * the top-level object is always closed (the reference closes it only inside its externals
//     block, so a scene without externals saves as truncated JSON);
//   * voxels listed twice at one lattice site replace each other (setVoxel semantics) instead of
//     stacking two voxels at one site.
// As in the reference, gravity, floor, collisions and ambient temperature are written but not read
// back, and the simulation state is not saved.
#include <fstream>
#include <sstream>
#include <unordered_map>

#include "Voxelyze.h"
#include "vx_json.h"

namespace {

using vxjson::Value;

// the model part of CVX_Material::readJSON (VX_Material.cpp:122-140) for one entry of "materials";
// false when the entry holds no valid model (the reference then stops reading that entry)
bool read_material_model(CVX_Material& m, const Value& v) {
  const Value* E = v.member("youngsModulus");
  const Value* sd = v.member("strainData");
  const Value* st = v.member("stressData");
  if (E && E->is_double()) {
    float failStress = -1.0f;
    const Value* ef = v.member("epsilonFail");
    if (ef && ef->is_double()) failStress = (float)(ef->get_double() * E->get_double());
    m.setModelLinear((float)E->get_double(), failStress);
  } else if (sd && sd->is_array() && st && st->is_array() && sd->size() == st->size()) {
    std::vector<float> strain, stress;
    for (size_t i = 0; i < sd->size(); ++i) {
      strain.push_back((float)sd->a[i].get_double());
      stress.push_back((float)st->a[i].get_double());
    }
    if (!strain.empty()) m.setModel((int)strain.size(), strain.data(), stress.data());
  } else {
    return false;  // no valid model
  }
  return true;
}

const Value* member_of(const Value& v, const char* key, Value::Kind kind) {
  const Value* m = v.member(key);
  return (m && m->kind == kind) ? m : nullptr;
}

}  // namespace

CVoxelyze::CVoxelyze(const char* jsonFilePath) : CVoxelyze(DEFAULT_VOXEL_SIZE) { loadJSON(jsonFilePath); }

bool CVoxelyze::loadJSON(const char* jsonFilePath) {  // Voxelyze.cpp:61-77
  std::ifstream t(jsonFilePath, std::ios::binary);
  if (!t) return false;
  std::stringstream buffer;
  buffer << t.rdbuf();
  Value doc;
  std::string err;
  if (!vxjson::parse(buffer.str(), doc, &err)) doc = Value();  // the reference reads an empty document then
  readJSON(&doc);
  return true;  // as the reference: true whenever the file opened
}

bool CVoxelyze::saveJSON(const char* jsonFilePath) {  // Voxelyze.cpp:79-93
  std::ofstream t(jsonFilePath, std::ios::binary);
  if (!t) return false;
  t << writeJSON();
  return (bool)t;
}

bool CVoxelyze::readJSON(const void* root) {  // Voxelyze.cpp:95-162
  const Value& vxl = *static_cast<const Value*>(root);
  clear();
  if (!vxl.is_object()) return false;
  const Value* vs = member_of(vxl, "voxelSize", Value::DOUBLE);
  if (!vs) return false;
  setVoxelSize(vs->get_double());
  const Value* mats = member_of(vxl, "materials", Value::ARRAY);
  if (!mats) return false;
  for (const Value& mv : mats->a) {
    // CVX_MaterialVoxel(rapidjson::Value&, voxSize): CVX_Material::readJSON, then the voxel
    // derivation at this scene's voxel size.  (Not through addMaterial(const CVX_Material&): the
    // reference's material copy leaves the external scale factor out, VX_Material.cpp:29-57.)
    CVX_Material& m = *addMaterial(1.0f, 1.0f);
    m.clear();
    if (read_material_model(m, mv)) {
      auto dbl = [&](const char* k, float& dst) {
        const Value* x = member_of(mv, k, Value::DOUBLE);
        if (x) dst = (float)x->get_double();
      };
      auto integer = [&](const char* k, int& dst) {
        const Value* x = mv.member(k);
        if (x && x->is_int()) dst = x->get_int();
      };
      dbl("density", m.rho);
      if (const Value* x = member_of(mv, "name", Value::STRING)) m.myName = x->s;
      integer("red", m.r);
      integer("green", m.g);
      integer("blue", m.b);
      integer("alpha", m.a);
      dbl("poissonsRatio", m.nu);
      dbl("CTE", m.alphaCTE);
      dbl("staticFriction", m.muStatic);
      dbl("kineticFriction", m.muKinetic);
      dbl("internalDamping", m.zetaInternal);
      dbl("globalDamping", m.zetaGlobal);
      dbl("collisionDamping", m.zetaCollision);
      const Value* es = member_of(mv, "externalScaleFactor", Value::ARRAY);
      if (es && es->size() == 3)
        for (int i = 0; i < 3; i++) m.extScale[i] = es->a[i].get_double();
    }
    m.updateDerived();
    m.touch();
  }
  const Value* vox = member_of(vxl, "voxels", Value::ARRAY);
  if (vox && vox->size() % 4 == 0) {
    const int n = (int)vox->size() / 4;
    for (int i = 0; i < n; i++) {
      int mi = vox->a[4 * i + 3].get_int();
      if (mi < 0 || mi >= materialCount()) continue;  // the reference indexes past its list here
      setVoxel(material(mi), vox->a[4 * i].get_int(), vox->a[4 * i + 1].get_int(), vox->a[4 * i + 2].get_int());
    }
  }
  const Value* exts = member_of(vxl, "externals", Value::ARRAY);
  if (exts) {
    for (const Value& ext : exts->a) {
      const Value* idx = member_of(ext, "voxelIndices", Value::ARRAY);
      if (!idx) continue;  // invalid external
      bool dofs[6] = {false, false, false, false, false, false};
      double disp[6] = {0, 0, 0, 0, 0, 0};
      Vec3D<float> force, moment;
      const Value* f = member_of(ext, "fixed", Value::ARRAY);
      if (f && f->size() == 6)
        for (int j = 0; j < 6; j++) dofs[j] = f->a[j].get_bool();
      const Value* tr = member_of(ext, "translate", Value::ARRAY);
      if (tr && tr->size() == 3)
        for (int j = 0; j < 3; j++) disp[j] = tr->a[j].get_double();
      const Value* ro = member_of(ext, "rotate", Value::ARRAY);
      if (ro && ro->size() == 3)
        for (int j = 0; j < 3; j++) disp[3 + j] = ro->a[j].get_double();
      const Value* fo = member_of(ext, "force", Value::ARRAY);
      if (fo && fo->size() == 3)
        for (int j = 0; j < 3; j++) force[j] = (float)fo->a[j].get_double();
      const Value* mo = member_of(ext, "moment", Value::ARRAY);
      if (mo && mo->size() == 3)
        for (int j = 0; j < 3; j++) moment[j] = (float)mo->a[j].get_double();
      for (const Value& vi : idx->a) {
        int k = vi.get_int();
        if (k < 0 || k >= voxelCount()) continue;
        CVX_External* pE = voxel(k)->external();
        for (int d = 0; d < 6; d++)
          if (dofs[d]) pE->setDisplacement((dofComponent)(1 << d), disp[d]);
        pE->addForce(force);
        pE->addMoment(moment);
      }
    }
  }
  return true;
}

std::string CVoxelyze::writeJSON() {  // Voxelyze.cpp:164-241, VX_Material.cpp:75-120
  vxjson::Writer w;
  w.start_object();
  w.key("voxelSize");
  w.value_double(voxSize);
  if (ambientTemp != 0) { w.key("relativeAmbientTemperature"); w.value_double((double)ambientTemp); }
  if (grav != 0) { w.key("gravityAcceleration"); w.value_double((double)grav); }
  if (floor) { w.key("floorEnabled"); w.value_bool(floor); }
  if (collisions) { w.key("collisionsEnabled"); w.value_bool(collisions); }

  std::unordered_map<const CVX_Material*, int> m2i;
  w.key("materials");
  w.start_array();
  for (int i = 0; i < materialCount(); i++) {
    const CVX_Material& m = *material(i);
    m2i[&m] = i;
    w.start_object();
    if (m.linear) {
      w.key("youngsModulus"); w.value_double((double)m.E);
      if (m.epsilonFail != -1) { w.key("epsilonFail"); w.value_double((double)m.epsilonFail); }
    } else {
      w.key("strainData");
      w.start_array();
      for (float x : m.strainData) w.value_double((double)x);
      w.end_array();
      w.key("stressData");
      w.start_array();
      for (float x : m.stressData) w.value_double((double)x);
      w.end_array();
    }
    if (m.rho != 1.0f) { w.key("density"); w.value_double(m.rho); }
    if (m.myName != "") { w.key("name"); w.value_string(m.myName); }
    if (m.r != -1) { w.key("red"); w.value_int(m.r); }
    if (m.g != -1) { w.key("green"); w.value_int(m.g); }
    if (m.b != -1) { w.key("blue"); w.value_int(m.b); }
    if (m.a != -1) { w.key("alpha"); w.value_int(m.a); }
    if (m.nu != 0) { w.key("poissonsRatio"); w.value_double(m.nu); }
    if (m.alphaCTE != 0) { w.key("CTE"); w.value_double(m.alphaCTE); }
    if (m.muStatic != 0) { w.key("staticFriction"); w.value_double(m.muStatic); }
    if (m.muKinetic != 0) { w.key("kineticFriction"); w.value_double(m.muKinetic); }
    if (m.zetaInternal != 1) { w.key("internalDamping"); w.value_double(m.zetaInternal); }
    if (m.zetaGlobal != 0) { w.key("globalDamping"); w.value_double(m.zetaGlobal); }
    if (m.zetaCollision != 1) { w.key("collisionDamping"); w.value_double(m.zetaCollision); }
    if (m.extScale.x != 1 || m.extScale.y != 1 || m.extScale.z != 1) {
      w.key("externalScaleFactor");
      w.start_array();
      for (int i = 0; i < 3; i++) w.value_double(m.extScale[i]);
      w.end_array();
    }
    w.end_object();
  }
  w.end_array();

  std::vector<CVX_External*> exts;          // distinct externals, in first-use order
  std::vector<std::vector<int>> extVoxels;  // voxels of each
  w.key("voxels");
  w.start_array();
  for (int i = 0; i < voxelCount(); i++) {  // x0, y0, z0, material0, x1, ...
    CVX_Voxel* v = voxel(i);
    w.value_int(v->indexX());
    w.value_int(v->indexY());
    w.value_int(v->indexZ());
    w.value_int(m2i[v->material()]);
    if (v->externalExists() && !v->external()->isEmpty()) {
      bool match = false;
      for (size_t j = 0; j < exts.size(); j++) {
        if (*v->external() == *exts[j]) {
          extVoxels[j].push_back(i);
          match = true;
          break;
        }
      }
      if (!match) {
        exts.push_back(v->external());
        extVoxels.push_back(std::vector<int>(1, i));
      }
    }
  }
  w.end_array();

  if (!exts.empty()) {
    w.key("externals");
    w.start_array();
    for (size_t i = 0; i < exts.size(); i++) {
      CVX_External* e = exts[i];
      w.start_object();
      if (e->isFixedAny()) {
        w.key("fixed");
        w.start_array();
        w.value_bool(e->isFixed(X_TRANSLATE)); w.value_bool(e->isFixed(Y_TRANSLATE));
        w.value_bool(e->isFixed(Z_TRANSLATE)); w.value_bool(e->isFixed(X_ROTATE));
        w.value_bool(e->isFixed(Y_ROTATE)); w.value_bool(e->isFixed(Z_ROTATE));
        w.end_array();
      }
      if (e->isFixedAnyTranslation() && e->translation() != Vec3D<double>()) {
        w.key("translate");
        w.start_array();
        for (int j = 0; j < 3; j++) w.value_double(e->translation()[j]);
        w.end_array();
      }
      if (e->isFixedAnyRotation() && e->rotation() != Vec3D<double>()) {
        w.key("rotate");
        w.start_array();
        for (int j = 0; j < 3; j++) w.value_double(e->rotation()[j]);
        w.end_array();
      }
      if (!e->isFixedAllTranslation() && e->force() != Vec3D<float>()) {
        w.key("force");
        w.start_array();
        for (int j = 0; j < 3; j++) w.value_double(e->force()[j]);
        w.end_array();
      }
      if (!e->isFixedAllRotation() && e->moment() != Vec3D<float>()) {
        w.key("moment");
        w.start_array();
        for (int j = 0; j < 3; j++) w.value_double(e->moment()[j]);
        w.end_array();
      }
      w.key("voxelIndices");
      w.start_array();
      for (int k : extVoxels[i]) w.value_int(k);
      w.end_array();
      w.end_object();
    }
    w.end_array();
  }
  w.end_object();
  return w.str();
}
