// Test-infrastructure driver for the REFERENCE library compiled from its own sources.
//
// oracle/build_ref.sh compiles this file together with the reference's src/*.cpp (read in place,
// never copied) into oracle/_ref/libvxref.so.  It exposes the vxr_* facade (oracle/facade.h) so the
// Python tests can push a scene into the reference exactly as into the oracle or the product and
// read back the full state.  It only calls the reference's public API; the state dump needs the
// private members, which is why the access specifiers are opened for this translation unit.
#include <algorithm>
#include <cstring>
#include <map>
#include <vector>

#define private public
#define protected public
#include "Voxelyze.h"
#include "VX_Collision.h"
#include "VX_Link.h"
#include "VX_Material.h"
#include "VX_MaterialLink.h"
#include "VX_MaterialVoxel.h"
#include "VX_Voxel.h"
#include "VX_MeshRender.h"
#undef private
#undef protected

#include "facade.h"

namespace {
struct RefSim {
  CVoxelyze vx;
  std::vector<CVX_Material*> mats;
  CVX_MeshRender* mesh = nullptr;
  explicit RefSim(double s) : vx(s) {}
  ~RefSim() { delete mesh; }
};
RefSim* S(void* s) { return static_cast<RefSim*>(s); }
int index_of(RefSim* r, CVX_Voxel* p) {
  if (!p) return -1;
  const std::vector<CVX_Voxel*>& l = *r->vx.voxelList();
  for (int i = (int)l.size() - 1; i >= 0; --i)
    if (l[i] == p) return i;
  return -1;
}
CVX_Voxel* V(void* s, int v) {
  RefSim* r = S(s);
  if (v < 0 || v >= r->vx.voxelCount()) return nullptr;
  return r->vx.voxel(v);
}
}  // namespace

extern "C" {

void* vxr_create(double voxel_size) { return new RefSim(voxel_size); }
void vxr_destroy(void* s) { delete S(s); }

int vxr_add_material(void* s, float E, float rho) {
  RefSim* r = S(s);
  CVX_Material* m = r->vx.addMaterial(E, rho);
  if (!m) return -1;
  r->mats.push_back(m);
  return (int)r->mats.size() - 1;
}

int vxr_material_set(void* s, int mat, int prop, float value) {
  RefSim* r = S(s);
  if (mat < 0 || mat >= (int)r->mats.size()) return -1;
  CVX_Material* m = r->mats[mat];
  switch (prop) {
    case VXF_PROP_POISSON: m->setPoissonsRatio(value); break;
    case VXF_PROP_CTE: m->setCte(value); break;
    case VXF_PROP_MU_STATIC: m->setStaticFriction(value); break;
    case VXF_PROP_MU_KINETIC: m->setKineticFriction(value); break;
    case VXF_PROP_ZETA_INTERNAL: m->setInternalDamping(value); break;
    case VXF_PROP_ZETA_GLOBAL: m->setGlobalDamping(value); break;
    case VXF_PROP_ZETA_COLLISION: m->setCollisionDamping(value); break;
    case VXF_PROP_DENSITY: m->setDensity(value); break;
    default: return -1;
  }
  return 0;
}

int vxr_material_set_model_linear(void* s, int mat, float E, float fail) {
  RefSim* r = S(s);
  return r->mats[mat]->setModelLinear(E, fail) ? 0 : -1;
}
int vxr_material_set_model_bilinear(void* s, int mat, float E, float Ep, float ys, float fs) {
  RefSim* r = S(s);
  return r->mats[mat]->setModelBilinear(E, Ep, ys, fs) ? 0 : -1;
}
int vxr_material_set_model(void* s, int mat, int n, const float* strain, const float* stress) {
  RefSim* r = S(s);
  std::vector<float> a(strain, strain + n), b(stress, stress + n);
  return r->mats[mat]->setModel(n, a.data(), b.data()) ? 0 : -1;
}

float vxr_material_stress(void* s, int mat, float strain, float tss, int force_linear) {
  RefSim* r = S(s);
  return r->mats[mat]->stress(strain, tss, force_linear != 0);
}
float vxr_material_modulus(void* s, int mat, float strain) {
  RefSim* r = S(s);
  return r->mats[mat]->modulus(strain);
}

int vxr_set_voxel(void* s, int mat, int x, int y, int z) {
  RefSim* r = S(s);
  CVX_Material* m = (mat >= 0 && mat < (int)r->mats.size()) ? r->mats[mat] : nullptr;
  return index_of(r, r->vx.setVoxel(m, x, y, z));
}
int vxr_remove_voxel(void* s, int x, int y, int z) {
  S(s)->vx.setVoxel(nullptr, x, y, z);
  return 0;
}
int vxr_replace_material(void* s, int a, int b) {
  RefSim* r = S(s);
  if (a < 0 || b < 0 || a >= (int)r->mats.size() || b >= (int)r->mats.size()) return -1;
  return r->vx.replaceMaterial(r->mats[a], r->mats[b]) ? 0 : -1;
}
int vxr_remove_material(void* s, int m) {
  RefSim* r = S(s);
  if (m < 0 || m >= (int)r->mats.size()) return -1;
  if (!r->vx.removeMaterial(r->mats[m])) return -1;
  r->mats.erase(r->mats.begin() + m);
  return 0;
}
void vxr_set_voxel_size(void* s, double size) { S(s)->vx.setVoxelSize(size); }
int vxr_set_voxels(void* s, int n, const int* mat, const int* xyz) {
  RefSim* r = S(s);
  for (int i = 0; i < n; ++i) {
    CVX_Material* m = (mat[i] >= 0 && mat[i] < (int)r->mats.size()) ? r->mats[mat[i]] : nullptr;
    r->vx.setVoxel(m, xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
  }
  return 0;
}
int vxr_voxel_count(void* s) { return S(s)->vx.voxelCount(); }
int vxr_link_count(void* s) { return S(s)->vx.linkCount(); }
int vxr_voxel_index(void* s, int x, int y, int z) {
  RefSim* r = S(s);
  return index_of(r, r->vx.voxel(x, y, z));
}

int vxr_external_set_fixed(void* s, int v, int m) {
  CVX_Voxel* p = V(s, v);
  if (!p) return -1;
  p->external()->setFixed(m & 1, m & 2, m & 4, m & 8, m & 16, m & 32);
  return 0;
}
int vxr_external_set_fixed_all(void* s, int v, int fixed) {
  CVX_Voxel* p = V(s, v);
  if (!p) return -1;
  p->external()->setFixedAll(fixed != 0);
  return 0;
}
int vxr_external_set_displacement(void* s, int v, int dof, double value) {
  CVX_Voxel* p = V(s, v);
  if (!p) return -1;
  p->external()->setDisplacement((dofComponent)dof, value);
  return 0;
}
int vxr_external_set_displacement_all(void* s, int v, const double* t3, const double* r3) {
  CVX_Voxel* p = V(s, v);
  if (!p) return -1;
  p->external()->setDisplacementAll(Vec3D<double>(t3[0], t3[1], t3[2]),
                                    Vec3D<double>(r3[0], r3[1], r3[2]));
  return 0;
}
int vxr_external_clear_displacement(void* s, int v, int dof) {
  CVX_Voxel* p = V(s, v);
  if (!p) return -1;
  p->external()->clearDisplacement((dofComponent)dof);
  return 0;
}
int vxr_external_set_force(void* s, int v, float fx, float fy, float fz) {
  CVX_Voxel* p = V(s, v);
  if (!p) return -1;
  p->external()->setForce(fx, fy, fz);
  return 0;
}
int vxr_external_set_moment(void* s, int v, float mx, float my, float mz) {
  CVX_Voxel* p = V(s, v);
  if (!p) return -1;
  p->external()->setMoment(mx, my, mz);
  return 0;
}

void vxr_set_gravity(void* s, float g) { S(s)->vx.setGravity(g); }
void vxr_enable_floor(void* s, int e) { S(s)->vx.enableFloor(e != 0); }
void vxr_enable_collisions(void* s, int e) { S(s)->vx.enableCollisions(e != 0); }
void vxr_set_ambient_temperature(void* s, float t, int all) {
  S(s)->vx.setAmbientTemperature(t, all != 0);
}
int vxr_voxel_set_temperature(void* s, int v, float t) {
  CVX_Voxel* p = V(s, v);
  if (!p) return -1;
  p->setTemperature(t);
  return 0;
}

int vxr_do_time_step(void* s, float dt) { return S(s)->vx.doTimeStep(dt) ? 1 : 0; }
int vxr_load_json(void* s, const char* path) {
  RefSim* r = S(s);
  delete r->mesh;
  r->mesh = nullptr;
  bool ok = r->vx.loadJSON(path);
  r->mats.clear();
  for (int i = 0; i < r->vx.materialCount(); ++i) r->mats.push_back(r->vx.material(i));
  return ok ? 1 : 0;
}
// the reference's CVX_MeshRender (src/VX_MeshRender.cpp), same entry points as the product's vx_mesh_*
int vxr_mesh_generate(void* s) {
  RefSim* r = S(s);
  if (!r->mesh) r->mesh = new CVX_MeshRender(&r->vx);
  else r->mesh->generateMesh();
  return 0;
}
int vxr_mesh_update(void* s, int coloring, int state_info) {
  RefSim* r = S(s);
  if (!r->mesh) return -1;
  r->mesh->updateMesh((CVX_MeshRender::viewColoring)coloring, (CVoxelyze::stateInfoType)state_info);
  return 0;
}
int vxr_mesh_counts(void* s, int* out3) {
  RefSim* r = S(s);
  if (!r->mesh) return -1;
  out3[0] = (int)r->mesh->vertices.size() / 3;
  out3[1] = (int)r->mesh->quads.size() / 4;
  out3[2] = (int)r->mesh->lines.size() / 2;
  return 0;
}
int vxr_mesh_read(void* s, float* vertices, int* quads, float* normals, float* colors, int* lines) {
  RefSim* r = S(s);
  if (!r->mesh) return -1;
  CVX_MeshRender& m = *r->mesh;
  if (vertices) std::copy(m.vertices.begin(), m.vertices.end(), vertices);
  if (quads) std::copy(m.quads.begin(), m.quads.end(), quads);
  if (normals) std::copy(m.quadNormals.begin(), m.quadNormals.end(), normals);
  if (colors) std::copy(m.quadColors.begin(), m.quadColors.end(), colors);
  if (lines) std::copy(m.lines.begin(), m.lines.end(), lines);
  return 0;
}
int vxr_mesh_save_obj(void* s, const char* path) {
  RefSim* r = S(s);
  if (!r->mesh) return -1;
  r->mesh->saveObj(path);
  return 0;
}
int vxr_save_json(void* s, const char* path) { return S(s)->vx.saveJSON(path) ? 1 : 0; }
int vxr_do_time_steps(void* s, int n, float dt) {
  for (int i = 0; i < n; ++i)
    if (!S(s)->vx.doTimeStep(dt)) return i;
  return n;
}
float vxr_recommended_time_step(void* s) { return S(s)->vx.recommendedTimeStep(); }
void vxr_reset_time(void* s) { S(s)->vx.resetTime(); }
float vxr_current_time(void* s) { return S(s)->vx.currentTime; }

int vxr_get_voxel_state(void* s, double* d, float* f, int* i) {
  RefSim* r = S(s);
  const std::vector<CVX_Voxel*>& l = *r->vx.voxelList();
  for (size_t k = 0; k < l.size(); ++k) {
    CVX_Voxel* p = l[k];
    if (d) {
      double* o = d + 13 * k;
      o[0] = p->pos.x; o[1] = p->pos.y; o[2] = p->pos.z;
      o[3] = p->linMom.x; o[4] = p->linMom.y; o[5] = p->linMom.z;
      o[6] = p->orient.w; o[7] = p->orient.x; o[8] = p->orient.y; o[9] = p->orient.z;
      o[10] = p->angMom.x; o[11] = p->angMom.y; o[12] = p->angMom.z;
    }
    if (f) {
      float* o = f + 5 * k;
      o[0] = p->temp; o[1] = p->previousDt;
      o[2] = p->pStrain.x; o[3] = p->pStrain.y; o[4] = p->pStrain.z;
    }
    if (i) {
      i[2 * k] = p->isFloorStaticFriction() ? 1 : 0;
      i[2 * k + 1] = p->poissonsStrainInvalid ? 1 : 0;
    }
  }
  return (int)l.size();
}

int vxr_get_link_state(void* s, double* d, float* f, int* i) {
  RefSim* r = S(s);
  const std::vector<CVX_Link*>& l = *r->vx.linkList();
  std::map<const void*, int> mat_id;
  int next = 0;
  for (std::list<CVX_MaterialLink*>::iterator it = r->vx.linkMats.begin(); it != r->vx.linkMats.end(); ++it)
    mat_id[*it] = next++;
  std::map<const void*, int> vid;
  for (int k = 0; k < r->vx.voxelCount(); ++k) vid[r->vx.voxel(k)] = k;
  for (size_t k = 0; k < l.size(); ++k) {
    CVX_Link* p = l[k];
    if (d) {
      double* o = d + 22 * k;
      const Vec3D<double>* v[7] = {&p->pos2, &p->angle1v, &p->angle2v, &p->forceNeg, &p->forcePos,
                                   &p->momentNeg, &p->momentPos};
      for (int j = 0; j < 7; ++j) { o[3 * j] = v[j]->x; o[3 * j + 1] = v[j]->y; o[3 * j + 2] = v[j]->z; }
      o[21] = p->currentRestLength;
    }
    if (f) {
      float* o = f + 6 * k;
      o[0] = p->strain; o[1] = p->maxStrain; o[2] = p->strainOffset; o[3] = p->_stress;
      o[4] = p->currentTransverseArea; o[5] = p->currentTransverseStrainSum;
    }
    if (i) {
      int* o = i + 6 * k;
      o[0] = p->smallAngle ? 1 : 0;
      o[1] = p->isLocalVelocityValid() ? 1 : 0;
      o[2] = (int)p->axis;
      o[3] = vid[p->pVNeg];
      o[4] = vid[p->pVPos];
      o[5] = mat_id[p->mat];
    }
  }
  return (int)l.size();
}

int vxr_get_collisions(void* s, int* pairs, int cap) {
  RefSim* r = S(s);
  const std::vector<CVX_Collision*>& c = *r->vx.collisionList();
  std::map<const void*, int> vid;
  for (int k = 0; k < r->vx.voxelCount(); ++k) vid[r->vx.voxel(k)] = k;
  int n = (int)c.size();
  for (int k = 0; k < n && k < cap; ++k) {
    pairs[2 * k] = vid[c[k]->pV1];
    pairs[2 * k + 1] = vid[c[k]->pV2];
  }
  return n;
}

// per-voxel and per-link queries through the reference's own methods (VX_Voxel.h:79-130,
// VX_Link.h:47-66).  externalForce/externalMoment dereference the external, so voxels without one
// answer zero here without calling them.
static int put3f(const Vec3D<float>& f, float* out) {
  out[0] = f.x; out[1] = f.y; out[2] = f.z;
  return 0;
}
static CVX_Link* L(void* s, int l) {
  const std::vector<CVX_Link*>& v = *S(s)->vx.linkList();
  return l >= 0 && l < (int)v.size() ? v[l] : nullptr;
}
int vxr_voxel_external_force(void* s, int v, float* out3) {
  CVX_Voxel* p = V(s, v);
  if (!p) return -1;
  if (!p->externalExists()) { out3[0] = out3[1] = out3[2] = 0.0f; return 0; }
  return put3f(p->externalForce(), out3);
}
int vxr_voxel_external_moment(void* s, int v, float* out3) {
  CVX_Voxel* p = V(s, v);
  if (!p) return -1;
  if (!p->externalExists()) { out3[0] = out3[1] = out3[2] = 0.0f; return 0; }
  return put3f(p->externalMoment(), out3);
}
int vxr_voxel_corner_offset(void* s, int v, int corner, float* out3) {
  CVX_Voxel* p = V(s, v);
  if (!p || corner < 0 || corner > 7) return -1;
  return put3f(p->cornerOffset((CVX_Voxel::voxelCorner)corner), out3);
}
int vxr_voxel_corner_position(void* s, int v, int corner, float* out3) {
  CVX_Voxel* p = V(s, v);
  if (!p || corner < 0 || corner > 7) return -1;
  return put3f(p->cornerPosition((CVX_Voxel::voxelCorner)corner), out3);
}
int vxr_voxel_force(void* s, int v, double* out3) {
  CVX_Voxel* p = V(s, v);
  if (!p) return -1;
  Vec3D<double> f = p->force();
  out3[0] = f.x; out3[1] = f.y; out3[2] = f.z;
  return 0;
}
int vxr_voxel_moment(void* s, int v, double* out3) {
  CVX_Voxel* p = V(s, v);
  if (!p) return -1;
  Vec3D<double> f = p->moment();
  out3[0] = f.x; out3[1] = f.y; out3[2] = f.z;
  return 0;
}
int vxr_voxel_is_yielded(void* s, int v) { CVX_Voxel* p = V(s, v); return p ? (p->isYielded() ? 1 : 0) : -1; }
int vxr_voxel_is_failed(void* s, int v) { CVX_Voxel* p = V(s, v); return p ? (p->isFailed() ? 1 : 0) : -1; }
float vxr_voxel_pressure(void* s, int v) { CVX_Voxel* p = V(s, v); return p ? p->pressure() : 0.0f; }
float vxr_link_strain_energy(void* s, int l) { CVX_Link* p = L(s, l); return p ? p->strainEnergy() : 0.0f; }
int vxr_link_is_yielded(void* s, int l) { CVX_Link* p = L(s, l); return p ? (p->isYielded() ? 1 : 0) : -1; }
int vxr_link_is_failed(void* s, int l) { CVX_Link* p = L(s, l); return p ? (p->isFailed() ? 1 : 0) : -1; }

float vxr_state_info(void* s, int info, int type) {
  return S(s)->vx.stateInfo((CVoxelyze::stateInfoType)info, (CVoxelyze::valueType)type);
}

}  // extern "C"
