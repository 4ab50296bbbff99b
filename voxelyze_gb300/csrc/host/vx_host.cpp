// Drop-in CVoxelyze / CVX_Voxel / CVX_Link on the host, driving the GPU engine (include/vxg.h).
//
// Scene building follows the reference exactly, because it fixes the voxel and link order the
// GPU arrays use: voxels in insertion order (src/Voxelyze.cpp:439-461), links in creation order with
// the six directions tried X+,X-,Y+,Y-,Z+,Z- (src/Voxelyze.cpp:508-539), link materials created on
// first use (src/Voxelyze.cpp:626-640).  The dynamic state lives on the GPU; this file keeps a
// structure-of-arrays mirror that is downloaded on the first host read after a step (syncDown) and
// uploaded before the next step when the host edited it (flush).  Rare host-side operations
// (resetTime, setTemperature on one voxel, topology edits) run on the mirror with the reference's
// semantics; the time step itself never runs on the host.
#include <algorithm>
#include <memory>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstring>
#include <thread>
#include <unordered_set>

#include "VX_MeshRender.h"
#include "Voxelyze.h"
#include "vx_host.h"
#include "vxg.h"

namespace {
const int kDirOff[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};

// powf(x, e) for every float x in [0.5, 2), with the C library the reference links
void fill_powf_table(float e, std::vector<float>& tab) {
  const uint32_t lo = 0x3F000000u, n = 1u << 24;
  tab.resize(n);
  unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  std::vector<std::thread> th;
  for (unsigned t = 0; t < nt; ++t)
    th.emplace_back([&, t]() {
      for (uint32_t i = t; i < n; i += nt) {
        uint32_t b = lo + i;
        float x;
        std::memcpy(&x, &b, 4);
        tab[i] = std::pow(x, e);
      }
    });
  for (auto& x : th) x.join();
}
}  // namespace

// =============================================================================================
// CVoxelyze
CVoxelyze::CVoxelyze(double voxelSize) : pimpl(new VxImpl()) {
  clear();
  voxSize = voxelSize <= 0 ? DEFAULT_VOXEL_SIZE : voxelSize;
}

CVoxelyze::~CVoxelyze() {
  clear();
  if (pimpl->eng) vxg_destroy(pimpl->eng);
  delete pimpl;
}

CVoxelyze::CVoxelyze(CVoxelyze& VIn) : pimpl(new VxImpl()) {
  clear();
  voxSize = VIn.voxSize;
  *this = VIn;
}

CVoxelyze& CVoxelyze::operator=(CVoxelyze& VIn) {  // Voxelyze.cpp:39-58
  setVoxelSize(VIn.voxSize);
  setAmbientTemperature(VIn.ambientTemperature(), true);
  setGravity(VIn.gravity());
  enableFloor(VIn.isFloorEnabled());
  enableCollisions(VIn.isCollisionsEnabled());
  std::unordered_map<CVX_Material*, CVX_Material*> mm;
  for (int i = 0; i < VIn.materialCount(); i++) mm[VIn.material(i)] = addMaterial(*(VIn.material(i)));
  for (int i = 0; i < VIn.voxelCount(); i++) {
    CVX_Voxel* a = VIn.voxel(i);
    CVX_Voxel* b = setVoxel(mm[a->material()], a->indexX(), a->indexY(), a->indexZ());
    *b->external() = *a->external();
  }
  return *this;
}

void CVoxelyze::clear() {  // Voxelyze.cpp:323-355
  for (CVX_Link* l : linksList) delete l;
  linksList.clear();
  for (CVX_Voxel* v : voxelsList) delete v;
  voxelsList.clear();
  for (CVX_MaterialVoxel* m : voxelMats) delete m;
  voxelMats.clear();
  for (CVX_MaterialLink* m : linkMats) delete m;
  linkMats.clear();
  pimpl->link_mat_of.clear();
  for (CVX_Collision* c : collisionsList) delete c;
  collisionsList.clear();
  ambientTemp = 0.0f;
  grav = 0.0f;
  floor = false;
  collisions = false;
  boundingRadius = 0.75f;
  watchDistance = 1.0f;
  pimpl->clear_mirror();
  pimpl->time = 0.0f;
  pimpl->device_ahead = false;
  markTopology();
}

void CVoxelyze::markState() const {
  pimpl->state_dirty = true;
}
void CVoxelyze::markTables() {
  pimpl->tables_dirty = true;
  pimpl->eager_stale = true;
}
void CVoxelyze::markExternals() {
  pimpl->ext_dirty = true;
  pimpl->eager_stale = true;
}
bool CVoxelyze::pushPending() const {
  VxImpl& I = *pimpl;
  if (I.pend_voxel.empty()) return true;
  int rc = I.eng ? vxg_set_temperatures_sparse(I.eng, (int)I.pend_voxel.size(), I.pend_voxel.data(), I.pend_temp.data())
                 : VXG_E_STATE;
  for (int v : I.pend_voxel) I.pend_slot[v] = -1;
  I.pend_voxel.clear();
  I.pend_temp.clear();
  if (rc) { I.err = I.eng ? vxg_last_error(I.eng) : "no engine"; return false; }
  return true;
}
void CVoxelyze::markTopology() {
  pimpl->topo_dirty = true;
  pimpl->tables_dirty = true;
  pimpl->state_dirty = true;
  pimpl->nearby_dirty = true;
}

CVX_Material* CVoxelyze::addMaterial(float E, float rho) {  // Voxelyze.cpp:357-366
  CVX_MaterialVoxel* m = new CVX_MaterialVoxel(E, rho, voxSize);
  m->setGravityMultiplier(grav);
  m->owner = this;
  voxelMats.push_back(m);
  markTables();
  return m;
}
CVX_Material* CVoxelyze::addMaterial(const CVX_Material& mat) {  // Voxelyze.cpp:376-382
  CVX_MaterialVoxel* m = new CVX_MaterialVoxel(mat, voxSize);
  m->setGravityMultiplier(grav);
  m->owner = this;
  m->dependentMaterials.clear();
  voxelMats.push_back(m);
  markTables();
  return m;
}

bool CVoxelyze::exists(const CVX_MaterialVoxel* m) {
  return std::find(voxelMats.begin(), voxelMats.end(), m) != voxelMats.end();
}

bool CVoxelyze::removeMaterial(CVX_Material* toRemove) {  // Voxelyze.cpp:384-404
  CVX_MaterialVoxel* m = (CVX_MaterialVoxel*)toRemove;
  if (!exists(m)) return false;
  std::vector<CVX_Voxel*> doomed;
  for (CVX_Voxel* v : voxelsList)
    if (v->mat == m) doomed.push_back(v);
  for (CVX_Voxel* v : doomed) removeVoxel(v->ix, v->iy, v->iz);
  for (auto it = linkMats.begin(); it != linkMats.end();) {
    if ((*it)->vox1Mat == m || (*it)->vox2Mat == m) {
      for (CVX_MaterialVoxel* o : voxelMats) {
        auto& d = o->dependentMaterials;
        d.erase(std::remove(d.begin(), d.end(), (CVX_Material*)*it), d.end());
      }
      pimpl->link_mat_of.erase(VxImpl::mat_pair((*it)->vox1Mat, (*it)->vox2Mat));
      delete *it;
      it = linkMats.erase(it);
    } else {
      ++it;
    }
  }
  voxelMats.erase(std::find(voxelMats.begin(), voxelMats.end(), m));
  delete m;
  markTopology();
  return true;
}

bool CVoxelyze::replaceMaterial(CVX_Material* a, CVX_Material* b) {  // Voxelyze.cpp:406-420
  if (!exists((CVX_MaterialVoxel*)a) || !exists((CVX_MaterialVoxel*)b)) return false;
  // the reference walks its bounding box z, then y, then x (each replacement moves the voxel's
  // links to the end of the link list, so the order fixes the link order); occupied cells only
  std::vector<CVX_Voxel*> hit;
  for (CVX_Voxel* v : voxelsList)
    if (v->mat == (CVX_MaterialVoxel*)a) hit.push_back(v);
  std::sort(hit.begin(), hit.end(), [](const CVX_Voxel* p, const CVX_Voxel* q) {
    if (p->iz != q->iz) return p->iz < q->iz;
    if (p->iy != q->iy) return p->iy < q->iy;
    return p->ix < q->ix;
  });
  for (CVX_Voxel* v : hit) setVoxel(b, v->ix, v->iy, v->iz);
  return true;
}

CVX_MaterialLink* CVoxelyze::combinedMaterial(CVX_MaterialVoxel* m1, CVX_MaterialVoxel* m2) {
  // Voxelyze.cpp:628-640: the first existing link material of this pair, else a new one
  auto key = VxImpl::mat_pair(m1, m2);
  auto it = pimpl->link_mat_of.find(key);
  if (it != pimpl->link_mat_of.end()) return it->second;
  CVX_MaterialLink* n = new CVX_MaterialLink(m1, m2);
  pimpl->link_mat_of.emplace(key, n);
  n->owner = this;
  linkMats.push_back(n);
  m1->dependentMaterials.push_back(n);
  m2->dependentMaterials.push_back(n);
  markTables();
  return n;
}

CVX_Voxel* CVoxelyze::voxel(int x, int y, int z) const {
  auto it = pimpl->vmap.find(VxImpl::key(x, y, z));
  return it == pimpl->vmap.end() ? nullptr : it->second;
}

static int idx_bound(const std::vector<CVX_Voxel*>& l, int which, bool mx) {
  if (l.empty()) return mx ? INT_MIN : INT_MAX;
  int r = mx ? INT_MIN : INT_MAX;
  for (CVX_Voxel* v : l) {
    int c = which == 0 ? v->indexX() : (which == 1 ? v->indexY() : v->indexZ());
    r = mx ? std::max(r, c) : std::min(r, c);
  }
  return r;
}
int CVoxelyze::indexMinX() const { return idx_bound(voxelsList, 0, false); }
int CVoxelyze::indexMaxX() const { return idx_bound(voxelsList, 0, true); }
int CVoxelyze::indexMinY() const { return idx_bound(voxelsList, 1, false); }
int CVoxelyze::indexMaxY() const { return idx_bound(voxelsList, 1, true); }
int CVoxelyze::indexMinZ() const { return idx_bound(voxelsList, 2, false); }
int CVoxelyze::indexMaxZ() const { return idx_bound(voxelsList, 2, true); }

CVX_Voxel* CVoxelyze::setVoxel(CVX_Material* material, int x, int y, int z) {  // Voxelyze.cpp:422-437
  if (!material) {
    removeVoxel(x, y, z);
    return nullptr;
  }
  CVX_Voxel* v = voxel(x, y, z);
  if (v) {
    replaceVoxel((CVX_MaterialVoxel*)material, x, y, z);
    return v;
  }
  return addVoxel((CVX_MaterialVoxel*)material, x, y, z);
}

CVX_Voxel* CVoxelyze::addVoxel(CVX_MaterialVoxel* m, int x, int y, int z) {  // Voxelyze.cpp:439-461
  syncDown();
  VxImpl& I = *pimpl;
  CVX_Voxel* v = new CVX_Voxel(this, m, (short)x, (short)y, (short)z);
  v->idx = (int)voxelsList.size();
  I.push_voxel();
  int i = v->idx;
  // CVX_Voxel::reset  VX_Voxel.cpp:47-56 (originalPosition), then the addVoxel overrides
  double s = m->nominalSize();
  I.vd[VD_PX][i] = v->ix * s; I.vd[VD_PY][i] = v->iy * s; I.vd[VD_PZ][i] = v->iz * s;
  I.vd[VD_OW][i] = 1.0;
  I.vflags[i] = VXG_VF_STATIC_FRICTION | VXG_VF_PSTRAIN_INVALID;
  I.vmap[VxImpl::key(x, y, z)] = v;
  voxelsList.push_back(v);
  I.vd[VD_PX][i] = x * voxSize; I.vd[VD_PY][i] = y * voxSize; I.vd[VD_PZ][i] = z * voxSize;
  if (floor) I.vflags[i] |= VXG_VF_FLOOR;
  I.vf[VF_TEMP][i] = ambientTemp;  // setTemperature before any link exists
  if (collisions) I.vflags[i] |= VXG_VF_COLLISIONS;
  for (int d = 0; d < 6; d++) addLink(x, y, z, (CVX_Voxel::linkDirection)d);
  markTopology();
  return v;
}

static void update_surface(VxImpl& I, CVX_Voxel* v, CVX_Link* const* links, int idx) {
  bool in = true;
  for (int i = 0; i < 6; i++)
    if (!links[i]) in = false;
  if (in) I.vflags[idx] |= VXG_VF_INTERIOR;
  else I.vflags[idx] &= ~(uint32_t)VXG_VF_INTERIOR;
  (void)v;
}

CVX_Link* CVoxelyze::link(int x, int y, int z, CVX_Voxel::linkDirection d) const {
  int ax = d / 2;
  auto it = pimpl->lmap[ax].find(VxImpl::key(x - (d == CVX_Voxel::X_NEG), y - (d == CVX_Voxel::Y_NEG), z - (d == CVX_Voxel::Z_NEG)));
  return it == pimpl->lmap[ax].end() ? nullptr : it->second;
}

CVX_Link* CVoxelyze::addLink(int x, int y, int z, CVX_Voxel::linkDirection d) {  // Voxelyze.cpp:508-539
  CVX_Link* pL = link(x, y, z, d);
  if (pL) return pL;
  CVX_Voxel* v1 = voxel(x, y, z);
  CVX_Voxel* v2 = voxel(x + kDirOff[d][0], y + kDirOff[d][1], z + kDirOff[d][2]);
  if (!v1 || !v2) return nullptr;
  CVX_MaterialLink* m = combinedMaterial(v1->mat, v2->mat);
  pL = new CVX_Link(this, v1, v2, m);
  pL->idx = (int)linksList.size();
  pimpl->push_link();
  linksList.push_back(pL);
  pL->reset();
  int ax = d / 2;
  pimpl->lmap[ax][VxImpl::key(x - (d == CVX_Voxel::X_NEG), y - (d == CVX_Voxel::Y_NEG), z - (d == CVX_Voxel::Z_NEG))] = pL;
  v1->links[d] = pL;
  update_surface(*pimpl, v1, v1->links, v1->idx);
  CVX_Voxel::linkDirection o = CVX_Voxel::toOpposite(d);
  v2->links[o] = pL;
  update_surface(*pimpl, v2, v2->links, v2->idx);
  return pL;
}

void CVoxelyze::removeLink(int x, int y, int z, CVX_Voxel::linkDirection d) {  // Voxelyze.cpp:541-575
  CVX_Link* pL = link(x, y, z, d);
  if (!pL) return;
  syncDown();
  int ax = d / 2;
  pimpl->lmap[ax].erase(VxImpl::key(x - (d == CVX_Voxel::X_NEG), y - (d == CVX_Voxel::Y_NEG), z - (d == CVX_Voxel::Z_NEG)));
  int li = pL->idx;
  linksList.erase(linksList.begin() + li);
  pimpl->erase_link(li);
  for (size_t k = li; k < linksList.size(); ++k) linksList[k]->idx = (int)k;
  CVX_Voxel* v1 = voxel(x, y, z);
  if (v1) { v1->links[d] = nullptr; update_surface(*pimpl, v1, v1->links, v1->idx); }
  CVX_Voxel* v2 = voxel(x + kDirOff[d][0], y + kDirOff[d][1], z + kDirOff[d][2]);
  if (v2) {
    CVX_Voxel::linkDirection o = CVX_Voxel::toOpposite(d);
    v2->links[o] = nullptr;
    update_surface(*pimpl, v2, v2->links, v2->idx);
  }
  delete pL;
  markTopology();
}

void CVoxelyze::removeVoxel(int x, int y, int z) {  // Voxelyze.cpp:464-483 (removed once, links first)
  CVX_Voxel* v = voxel(x, y, z);
  if (!v) return;
  syncDown();
  for (int d = 0; d < 6; d++) removeLink(x, y, z, (CVX_Voxel::linkDirection)d);
  pimpl->vmap.erase(VxImpl::key(x, y, z));
  int vi = v->idx;
  voxelsList.erase(voxelsList.begin() + vi);
  pimpl->erase_voxel(vi);
  for (size_t k = vi; k < voxelsList.size(); ++k) voxelsList[k]->idx = (int)k;
  delete v;
  markTopology();
}

void CVoxelyze::replaceVoxel(CVX_MaterialVoxel* m, int x, int y, int z) {  // Voxelyze.cpp:485-498
  syncDown();
  CVX_Voxel* v = voxel(x, y, z);
  VxImpl& I = *pimpl;
  int i = v->idx;
  // CVX_Voxel::replaceMaterial  VX_Voxel.cpp:78-90
  double fm = m->_mass / v->mat->_mass, fi = m->_momentInertia / v->mat->_momentInertia;
  for (int c = 0; c < 3; ++c) {
    I.vd[VD_LX + c][i] *= fm;
    I.vd[VD_AX + c][i] *= fi;
  }
  I.vflags[i] &= ~(uint32_t)VXG_VF_STATIC_FRICTION;
  I.vflags[i] |= VXG_VF_PSTRAIN_INVALID;
  v->mat = m;
  for (int d = 0; d < 6; d++) {
    removeLink(x, y, z, (CVX_Voxel::linkDirection)d);
    addLink(x, y, z, (CVX_Voxel::linkDirection)d);
  }
  markTopology();
}

void CVoxelyze::setVoxelSize(double s) {  // Voxelyze.cpp:643-668
  syncDown();
  double f = s / voxSize;
  voxSize = s;
  for (CVX_MaterialVoxel* m : voxelMats) m->setNominalSize(s);
  VxImpl& I = *pimpl;
  for (CVX_Voxel* v : voxelsList) {
    int i = v->idx;
    for (int c = 0; c < 3; ++c) {
      I.vd[VD_PX + c][i] *= f;
      I.vd[VD_LX + c][i] = 0;
      I.vd[VD_AX + c][i] = 0;
    }
    I.vflags[i] &= ~(uint32_t)VXG_VF_STATIC_FRICTION;
  }
  for (CVX_Link* l : linksList) l->reset();
  markTopology();
}

void CVoxelyze::setAmbientTemperature(float t, bool all) {  // Voxelyze.cpp:585-594
  ambientTemp = t;
  if (!all) return;
  if (pimpl->device_ahead && !pimpl->state_dirty && !pimpl->topo_dirty && pimpl->eng) {
    flush();
    vxg_set_all_temperatures(pimpl->eng, t);
    return;  // mirror stays stale; read back on demand
  }
  syncDown();
  for (CVX_Voxel* v : voxelsList) {
    pimpl->vf[VF_TEMP][v->idx] = t;
  }
  for (CVX_Link* l : linksList) l->updateRestLength();
  markState();
}

bool CVoxelyze::setTemperatures(const float* t) {
  if (!flush()) return false;
  int rc = vxg_set_temperatures(pimpl->eng, t);
  if (rc) { pimpl->err = vxg_last_error(pimpl->eng); return false; }
  pimpl->device_ahead = true;
  return true;
}

void CVoxelyze::setGravity(float g) {  // Voxelyze.cpp:596-602
  grav = g;
  for (CVX_MaterialVoxel* m : voxelMats) m->setGravityMultiplier(g);
  markTables();
}

void CVoxelyze::enableFloor(bool on) {  // Voxelyze.cpp:604-610
  syncDown();
  floor = on;
  for (CVX_Voxel* v : voxelsList) {
    if (on) pimpl->vflags[v->idx] |= VXG_VF_FLOOR;
    else pimpl->vflags[v->idx] &= ~(uint32_t)VXG_VF_FLOOR;
  }
  markState();
}

void CVoxelyze::enableCollisions(bool on) {  // Voxelyze.cpp:612-622
  if (collisions == on) return;
  syncDown();
  collisions = on;
  for (CVX_Voxel* v : voxelsList) {
    if (on) pimpl->vflags[v->idx] |= VXG_VF_COLLISIONS;
    else pimpl->vflags[v->idx] &= ~(uint32_t)VXG_VF_COLLISIONS;
  }
  pimpl->nearby_dirty = true;
  markState();
  markTables();
}

// ---- synchronisation --------------------------------------------------------------------------
struct FieldMap {
  int field;
  bool link;
  int kind;   // 0 double, 1 float, 2 uint32 flags
  int first;  // first mirror component
  int comps;
};
static const FieldMap kState[] = {
    {VXG_F_POS, false, 0, VD_PX, 3},           {VXG_F_LINMOM, false, 0, VD_LX, 3},
    {VXG_F_ORIENT, false, 0, VD_OW, 4},        {VXG_F_ANGMOM, false, 0, VD_AX, 3},
    {VXG_F_TEMP, false, 1, VF_TEMP, 1},        {VXG_F_PREV_DT, false, 1, VF_PDT, 1},
    {VXG_F_PSTRAIN, false, 1, VF_PSX, 3},      {VXG_F_VOXEL_FLAGS, false, 2, 0, 1},
    {VXG_F_LINK_FLAGS, true, 2, 0, 1},         {VXG_F_POS2, true, 0, LD_P2X, 3},
    {VXG_F_ANGLE1V, true, 0, LD_A1X, 3},       {VXG_F_ANGLE2V, true, 0, LD_A2X, 3},
    {VXG_F_FORCE_NEG, true, 0, LD_FNX, 3},     {VXG_F_FORCE_POS, true, 0, LD_FPX, 3},
    {VXG_F_MOMENT_NEG, true, 0, LD_MNX, 3},    {VXG_F_MOMENT_POS, true, 0, LD_MPX, 3},
    {VXG_F_REST_LENGTH, true, 0, LD_REST, 1},  {VXG_F_STRAIN, true, 1, LF_STRAIN, 1},
    {VXG_F_MAX_STRAIN, true, 1, LF_MAXS, 1},   {VXG_F_STRAIN_OFFSET, true, 1, LF_SOFF, 1},
    {VXG_F_STRESS, true, 1, LF_STRESS, 1},     {VXG_F_STRAIN_RATIO, true, 1, LF_RATIO, 1},
    {VXG_F_TRANSVERSE_AREA, true, 1, LF_TAREA, 1}, {VXG_F_TRANSVERSE_STRAIN_SUM, true, 1, LF_TSS, 1},
};

static bool transfer(VxImpl& I, const FieldMap& f, bool up) {
  size_t n = f.link ? I.lflags.size() : I.vflags.size();
  long long cnt = (long long)n * f.comps;
  if (n == 0) return true;
  int rc = 0;
  if (f.kind == 2) {
    std::vector<uint32_t>& src = f.link ? I.lflags : I.vflags;
    rc = up ? vxg_set_field(I.eng, f.field, src.data(), cnt) : vxg_get_field(I.eng, f.field, src.data(), cnt);
  } else if (f.kind == 0) {
    std::vector<double> st((size_t)cnt);
    std::vector<double>* comp = f.link ? I.ld : I.vd;
    if (up) {
      for (int c = 0; c < f.comps; ++c) std::memcpy(st.data() + c * n, comp[f.first + c].data(), n * 8);
      rc = vxg_set_field(I.eng, f.field, st.data(), cnt);
    } else {
      rc = vxg_get_field(I.eng, f.field, st.data(), cnt);
      for (int c = 0; c < f.comps && !rc; ++c) std::memcpy(comp[f.first + c].data(), st.data() + c * n, n * 8);
    }
  } else {
    std::vector<float> st((size_t)cnt);
    std::vector<float>* comp = f.link ? I.lf : I.vf;
    if (up) {
      for (int c = 0; c < f.comps; ++c) std::memcpy(st.data() + c * n, comp[f.first + c].data(), n * 4);
      rc = vxg_set_field(I.eng, f.field, st.data(), cnt);
    } else {
      rc = vxg_get_field(I.eng, f.field, st.data(), cnt);
      for (int c = 0; c < f.comps && !rc; ++c) std::memcpy(comp[f.first + c].data(), st.data() + c * n, n * 4);
    }
  }
  if (rc) I.err = vxg_last_error(I.eng);
  return rc == 0;
}

void CVoxelyze::syncDown() const {
  VxImpl& I = *pimpl;
  if (!I.device_ahead || !I.eng) return;
  pushPending();
  for (const FieldMap& f : kState) transfer(I, f, false);
  vxg_get_field(I.eng, VXG_F_TIME, &I.time, 1);
  I.device_ahead = false;
}

// one voxel's externals as the engine table holds them (include/VX_External.h:92-97)
static vxg_external external_entry(const CVX_External& e) {
  vxg_external d;
  std::memset(&d, 0, sizeof(d));
  for (int k = 0; k < 6; ++k)
    if (e.isFixed((dofComponent)(1 << k))) d.dof |= 1 << k;
  Vec3D<float> f = e.force(), m = e.moment();
  Vec3D<double> t = e.translation();
  d.force[0] = f.x; d.force[1] = f.y; d.force[2] = f.z;
  d.moment[0] = m.x; d.moment[1] = m.y; d.moment[2] = m.z;
  d.translation[0] = t.x; d.translation[1] = t.y; d.translation[2] = t.z;
  Quat3D<double> q = e.rotationQuat();
  d.rotq[0] = q.w; d.rotq[1] = q.x; d.rotq[2] = q.y; d.rotq[3] = q.z;
  return d;
}

bool CVoxelyze::flush() {
  VxImpl& I = *pimpl;
  if (!I.eng) {
    if (vxg_create(&I.eng, I.device, I.precision) != VXG_OK) {
      I.err = "vxg_create failed (no CUDA device?)";
      I.eng = nullptr;
      return false;
    }
    I.topo_dirty = I.tables_dirty = I.state_dirty = I.nearby_dirty = true;
    I.powf_slots.clear();
  }
  if (I.topo_dirty && I.act_mode) I.act_dirty = true;
  const int nv = (int)voxelsList.size(), nl = (int)linksList.size();
  if (I.topo_dirty) {
    std::unordered_map<const CVX_MaterialVoxel*, int> vmi;
    for (size_t k = 0; k < voxelMats.size(); ++k) vmi[voxelMats[k]] = (int)k;
    if (vxg_resize(I.eng, nv, nl)) { I.err = vxg_last_error(I.eng); return false; }
    std::vector<int> a((size_t)nv), idx3((size_t)3 * nv), lk((size_t)6 * nv);
    for (int i = 0; i < nv; ++i) {
      CVX_Voxel* v = voxelsList[i];
      a[i] = vmi[v->mat];
      idx3[i] = v->ix; idx3[nv + i] = v->iy; idx3[2 * nv + i] = v->iz;
      for (int d = 0; d < 6; ++d) lk[(size_t)d * nv + i] = v->links[d] ? v->links[d]->idx : -1;
    }
    std::unordered_map<const CVX_MaterialLink*, int> lmi;
    int k = 0;
    for (CVX_MaterialLink* m : linkMats) lmi[m] = k++;
    std::vector<int> lv((size_t)2 * nl), lm((size_t)nl);
    for (int i = 0; i < nl; ++i) {
      lv[i] = linksList[i]->pVNeg->idx;
      lv[nl + i] = linksList[i]->pVPos->idx;
      lm[i] = lmi[linksList[i]->mat];
    }
    int rc = 0;
    if (nv) {
      rc |= vxg_set_field(I.eng, VXG_F_VOXEL_MATERIAL, a.data(), nv);
      rc |= vxg_set_field(I.eng, VXG_F_VOXEL_INDEX, idx3.data(), 3ll * nv);
      rc |= vxg_set_field(I.eng, VXG_F_VOXEL_LINKS, lk.data(), 6ll * nv);
    }
    if (nl) {
      rc |= vxg_set_field(I.eng, VXG_F_LINK_VOXELS, lv.data(), 2ll * nl);
      rc |= vxg_set_field(I.eng, VXG_F_LINK_MATERIAL, lm.data(), nl);
    }
    if (rc) { I.err = vxg_last_error(I.eng); return false; }
    I.topo_dirty = false;
    I.tables_dirty = I.state_dirty = I.nearby_dirty = true;
  }
  if (I.tables_dirty) {
    bool any_poisson = false;
    float fallback = 0.0f;
    std::vector<vxg_voxel_material> vm(voxelMats.size());
    for (size_t k = 0; k < voxelMats.size(); ++k) {
      CVX_MaterialVoxel* m = voxelMats[k];
      vxg_voxel_material& d = vm[k];
      std::memset(&d, 0, sizeof(d));
      d.E = m->E; d.nu = m->nu; d.rho = m->rho; d.alphaCTE = m->alphaCTE;
      d.muStatic = m->muStatic; d.muKinetic = m->muKinetic;
      d.zetaInternal = m->zetaInternal; d.zetaGlobal = m->zetaGlobal; d.zetaCollision = m->zetaCollision;
      d.mass = m->_mass; d.massInv = m->_massInverse; d.sqrtMass = m->_sqrtMass;
      d.inertia = m->_momentInertia; d.inertiaInv = m->_momentInertiaInverse;
      d.c2xSqMxExS = m->_2xSqMxExS; d.c2xSqIxExSxSxS = m->_2xSqIxExSxSxS;
      d.gravMult = m->gravMult; d.penetrationStiffness = m->penetrationStiffness(); d.eHat = m->_eHat;
      d.nomSize = m->nomSize;
      Vec3D<double> sz = m->size();
      d.size[0] = sz.x; d.size[1] = sz.y; d.size[2] = sz.z;
      d.nomSizeF = (float)m->nomSize;
      d.sizeF[0] = (float)sz.x; d.sizeF[1] = (float)sz.y; d.sizeF[2] = (float)sz.z;
      d.sizeAvgF = (float)((sz.x + sz.y + sz.z) / 3.0);
      d.powf_slot = -1;
      if (m->nu != 0.0f) {
        any_poisson = true;
        float e = -m->nu;
        auto it = I.powf_slots.find(e);
        if (it == I.powf_slots.end()) {
          int slot = (int)I.powf_slots.size();
          std::vector<float> tab;
          fill_powf_table(e, tab);
          if (vxg_set_powf_table(I.eng, slot, e, tab.data())) { I.err = vxg_last_error(I.eng); return false; }
          it = I.powf_slots.emplace(e, slot).first;
        }
        d.powf_slot = it->second;
      }
    }
    for (CVX_Voxel* v : voxelsList) {  // recommendedTimeStep fallback  Voxelyze.cpp:302-307
      float f = v->mat->youngsModulus() * v->mat->nomSize / v->mat->mass();
      if (f > fallback) fallback = f;
    }
    std::vector<vxg_link_material> lm;
    for (CVX_MaterialLink* m : linkMats) {
      vxg_link_material d;
      std::memset(&d, 0, sizeof(d));
      if ((int)m->strainData.size() > VXG_MAX_MODEL_POINTS) { I.err = "material model has too many data points"; return false; }
      d.linear = m->linear ? 1 : 0;
      d.ndata = (int)m->strainData.size();
      for (int i = 0; i < d.ndata; ++i) { d.strain[i] = m->strainData[i]; d.stress[i] = m->stressData[i]; }
      d.E = m->E; d.nu = m->nu; d.eHat = m->_eHat; d.epsilonFail = m->epsilonFail;
      d.a1 = m->_a1; d.a2 = m->_a2; d.b1 = m->_b1; d.b2 = m->_b2; d.b3 = m->_b3;
      d.sqA1 = m->_sqA1; d.sqA2xIp = m->_sqA2xIp; d.sqB1 = m->_sqB1; d.sqB2xFMp = m->_sqB2xFMp; d.sqB3xIp = m->_sqB3xIp;
      lm.push_back(d);
    }
    std::vector<vxg_external> ex;
    std::vector<int> vext((size_t)nv, -1);
    I.ext_voxels.clear();
    for (int i = 0; i < nv; ++i) {
      CVX_External* e = voxelsList[i]->ext;
      if (!e) continue;
      vext[i] = (int)ex.size();
      ex.push_back(external_entry(*e));
      I.ext_voxels.push_back(i);
    }
    if (vxg_set_tables(I.eng, vm.data(), (int)vm.size(), lm.data(), (int)lm.size(), ex.data(), (int)ex.size())) {
      I.err = vxg_last_error(I.eng);
      return false;
    }
    if (nv && vxg_set_field(I.eng, VXG_F_VOXEL_EXTERNAL, vext.data(), nv)) { I.err = vxg_last_error(I.eng); return false; }
    vxg_globals g;
    std::memset(&g, 0, sizeof(g));
    g.collisions = collisions ? 1 : 0;
    g.any_poisson = any_poisson ? 1 : 0;
    g.boundingRadius = boundingRadius;
    g.watchDistance = watchDistance;
    g.voxSize = voxSize;
    g.fallback_freq2 = fallback;
    vxg_set_globals(I.eng, &g);
    I.tables_dirty = false;
    I.ext_dirty = false;
  }
  if (I.ext_dirty) {  // externals edited, none added: their table only
    std::vector<vxg_external> ex;
    ex.reserve(I.ext_voxels.size());
    for (int i : I.ext_voxels) ex.push_back(external_entry(*voxelsList[i]->ext));
    if (vxg_set_externals(I.eng, ex.data(), (int)ex.size())) { I.err = vxg_last_error(I.eng); return false; }
    I.ext_dirty = false;
  }
  if (!pushPending()) return false;
  if (I.state_dirty) {
    for (const FieldMap& f : kState)
      if (!transfer(I, f, true)) return false;
    vxg_set_field(I.eng, VXG_F_TIME, &I.time, 1);
    I.state_dirty = false;
  }
  if (collisions && I.nearby_dirty) {
    // CVX_Voxel::generateNearby with linkDepth int(2*(2*boundingRadius+watchDistance))
    // (VX_Voxel.cpp:395-418, Voxelyze.cpp:677-683): surface voxels within that many link hops
    int depth = (int)((2 * boundingRadius + watchDistance) * 2);
    std::vector<int> off((size_t)nv + 1, 0), items;
    std::vector<int> stamp((size_t)nv, -1), frontier, nextf, found;
    for (int v = 0; v < nv; ++v) {
      found.clear();
      frontier.assign(1, v);
      stamp[v] = v;
      for (int k = 0; k < depth; ++k) {
        nextf.clear();
        for (int p : frontier)
          for (int d = 0; d < 6; ++d) {
            CVX_Link* l = voxelsList[p]->links[d];
            if (!l) continue;
            int q = l->pVPos->idx == p ? l->pVNeg->idx : l->pVPos->idx;
            if (stamp[q] != v) { stamp[q] = v; nextf.push_back(q); found.push_back(q); }
          }
        frontier.swap(nextf);
      }
      std::vector<int> keep;
      for (int q : found)
        if (!(I.vflags[q] & VXG_VF_INTERIOR)) keep.push_back(q);
      std::sort(keep.begin(), keep.end());
      off[v + 1] = off[v] + (int)keep.size();
      items.insert(items.end(), keep.begin(), keep.end());
    }
    if (vxg_set_nearby(I.eng, off.data(), items.data(), (long long)items.size())) { I.err = vxg_last_error(I.eng); return false; }
    I.nearby_dirty = false;
  }
  if (I.act_dirty) {
    if (I.act_mode == 2 && I.act_phase.size() != (size_t)nv) { I.err = "actuation phases do not match the voxel count"; return false; }
    if (vxg_set_actuation(I.eng, I.act_mode, I.act_amp, I.act_freq, I.act_mode == 2 ? I.act_phase.data() : nullptr)) {
      I.err = vxg_last_error(I.eng);
      return false;
    }
    I.act_dirty = false;
  }
  return true;
}

bool CVoxelyze::doTimeStep(float dt) {  // Voxelyze.cpp:251-284
  if (dt == 0) return true;
  return doTimeSteps(1, dt) == 1;
}

int CVoxelyze::doTimeSteps(int n, float dt) {
  if (n <= 0) return 0;
  if (dt == 0) return n;
  if (!flush()) return -1;
  int done = 0, div = 0;
  int rc = vxg_step(pimpl->eng, n, dt, &done, &div);
  pimpl->device_ahead = true;
  if (rc) { pimpl->err = vxg_last_error(pimpl->eng); return -1; }
  if (done > 0) pimpl->eager_stale = false;
  return done;
}

float CVoxelyze::recommendedTimeStep() const {  // Voxelyze.cpp:286-311 (on the GPU)
  CVoxelyze* self = const_cast<CVoxelyze*>(this);
  if (!self->flush()) return 0.0f;
  float dt = 0.0f;
  if (vxg_recommended_dt(pimpl->eng, &dt)) { pimpl->err = vxg_last_error(pimpl->eng); return 0.0f; }
  pimpl->device_ahead = true;  // nu != 0 updates link rest lengths and transverse terms
  return dt;
}

void CVoxelyze::resetTime() {  // Voxelyze.cpp:313-321
  syncDown();
  VxImpl& I = *pimpl;
  I.time = 0.0f;
  for (CVX_Voxel* v : voxelsList) {  // CVX_Voxel::reset  VX_Voxel.cpp:47-56
    int i = v->idx;
    double s = v->mat->nominalSize();
    I.vd[VD_PX][i] = v->ix * s; I.vd[VD_PY][i] = v->iy * s; I.vd[VD_PZ][i] = v->iz * s;
    I.vd[VD_OW][i] = 1.0; I.vd[VD_OX][i] = 0.0; I.vd[VD_OY][i] = 0.0; I.vd[VD_OZ][i] = 0.0;
    for (int c = 0; c < 3; ++c) { I.vd[VD_LX + c][i] = 0.0; I.vd[VD_AX + c][i] = 0.0; }
    I.vflags[i] |= VXG_VF_STATIC_FRICTION | VXG_VF_PSTRAIN_INVALID;
    I.vf[VF_TEMP][i] = 0.0f;
    I.vf[VF_PDT][i] = 0.0f;
  }
  for (CVX_Link* l : linksList) l->reset();
  I.nearby_dirty = true;  // collisions and nearby lists go stale
  markState();
}

float CVoxelyze::currentTime() const {
  syncDown();
  return pimpl->time;
}

void CVoxelyze::setPrecision(precisionMode m) {
  syncDown();
  if (pimpl->eng) {
    vxg_destroy(pimpl->eng);
    pimpl->eng = nullptr;
  }
  pimpl->precision = (int)m;
  markTopology();
}
CVoxelyze::precisionMode CVoxelyze::precision() const { return (precisionMode)pimpl->precision; }

bool CVoxelyze::readField(int field, void* host, long long count) {
  if (!flush()) return false;
  int rc = vxg_get_field(pimpl->eng, field, host, count);
  if (rc) pimpl->err = vxg_last_error(pimpl->eng);
  return rc == 0;
}

const char* CVoxelyze::lastError() const { return pimpl->err.c_str(); }
bool CVoxelyze::upload() { return flush(); }

const std::vector<CVX_Collision*>* CVoxelyze::collisionList() const {
  for (CVX_Collision* c : collisionsList) delete c;
  collisionsList.clear();
  if (!collisions || !pimpl->eng) return &collisionsList;
  int n = 0;
  vxg_get_collisions(pimpl->eng, nullptr, 0, &n);
  std::vector<int> p((size_t)2 * std::max(n, 1));
  vxg_get_collisions(pimpl->eng, p.data(), n, &n);
  for (int k = 0; k < n; ++k) collisionsList.push_back(new CVX_Collision(voxelsList[p[2 * k]], voxelsList[p[2 * k + 1]]));
  return &collisionsList;
}

float CVoxelyze::stateInfo(stateInfoType info, valueType type) {  // Voxelyze.cpp:752-800
  syncDown();
  float r = 0;
  if (type == MAX) r = -FLT_MAX;
  else if (type == MIN) r = FLT_MAX;
  auto acc = [&](float t) {
    switch (type) {
      case MIN: if (t < r) r = t; break;
      case MAX: if (t > r) r = t; break;
      default: r += t;
    }
  };
  if (info == STRAIN_ENERGY || info == ENG_STRESS || info == ENG_STRAIN) {
    if (linksList.empty()) return 0.0f;
    for (CVX_Link* l : linksList) {
      float t = 0;
      switch (info) {
        case STRAIN_ENERGY: t = l->strainEnergy(); break;
        case ENG_STRESS: t = l->axialStress(); break;
        default: t = l->axialStrain();
      }
      acc(t);
    }
    if (type == AVERAGE) r /= linkCount();
  } else {
    if (voxelsList.empty()) return 0.0f;
    for (CVX_Voxel* v : voxelsList) {
      float t = 0;
      switch (info) {
        case DISPLACEMENT: t = v->displacementMagnitude(); break;
        case VELOCITY: t = v->velocityMagnitude(); break;
        case KINETIC_ENERGY: t = v->kineticEnergy(); break;
        case ANGULAR_DISPLACEMENT: t = v->angularDisplacementMagnitude(); break;
        case ANGULAR_VELOCITY: t = v->angularVelocityMagnitude(); break;
        case PRESSURE: t = v->pressure(); break;
        case MASS: t = v->material()->mass(); break;
        default: t = 0;
      }
      acc(t);
    }
    if (type == AVERAGE) r /= voxelCount();
  }
  return r;
}

float CVoxelyze::stateInfoDevice(stateInfoType info, valueType type) {
  if (info == PRESSURE) return stateInfo(info, type);
  if (!flush()) return 0.0f;
  float out = 0.0f;
  if (vxg_reduce(pimpl->eng, (int)info, (int)type, &out)) pimpl->err = vxg_last_error(pimpl->eng);
  return out;
}

// =============================================================================================
// CVX_Voxel
CVX_Voxel::CVX_Voxel(CVoxelyze* owner, CVX_MaterialVoxel* m, short x, short y, short z)
    : vx(owner), idx(-1), mat(m), ix(x), iy(y), iz(z), ext(nullptr) {
  for (int i = 0; i < 6; ++i) links[i] = nullptr;
}
CVX_Voxel::~CVX_Voxel() { delete ext; }

CVX_External* CVX_Voxel::external() {
  if (!ext) {
    ext = new CVX_External();
    ext->owner = vx;
    vx->markTables();
  }
  return ext;
}

CVX_Voxel* CVX_Voxel::adjacentVoxel(linkDirection d) const {
  CVX_Link* l = links[(int)d];
  if (!l) return nullptr;
  return l->voxel(true) == this ? l->voxel(false) : l->voxel(true);
}

#define VXI (*vx->pimpl)
Vec3D<double> CVX_Voxel::position() const {
  vx->syncDown();
  return Vec3D<double>(VXI.vd[VD_PX][idx], VXI.vd[VD_PY][idx], VXI.vd[VD_PZ][idx]);
}
Quat3D<double> CVX_Voxel::orientation() const {
  vx->syncDown();
  return Quat3D<double>(VXI.vd[VD_OW][idx], VXI.vd[VD_OX][idx], VXI.vd[VD_OY][idx], VXI.vd[VD_OZ][idx]);
}
bool CVX_Voxel::isInterior() const { return (VXI.vflags[idx] & VXG_VF_INTERIOR) != 0; }
Vec3D<double> CVX_Voxel::baseSize() const {
  vx->syncDown();
  return mat->size() * (1 + VXI.vf[VF_TEMP][idx] * mat->alphaCTE);
}
double CVX_Voxel::baseSize(CVX_Link::linkAxis axis) const {
  vx->syncDown();
  return mat->size()[axis] * (1 + VXI.vf[VF_TEMP][idx] * mat->alphaCTE);
}
Vec3D<double> CVX_Voxel::velocity() const {
  vx->syncDown();
  return Vec3D<double>(VXI.vd[VD_LX][idx], VXI.vd[VD_LY][idx], VXI.vd[VD_LZ][idx]) * mat->_massInverse;
}
float CVX_Voxel::velocityMagnitude() const {
  vx->syncDown();
  return (float)(Vec3D<double>(VXI.vd[VD_LX][idx], VXI.vd[VD_LY][idx], VXI.vd[VD_LZ][idx]).Length() * mat->_massInverse);
}
Vec3D<double> CVX_Voxel::angularVelocity() const {
  vx->syncDown();
  return Vec3D<double>(VXI.vd[VD_AX][idx], VXI.vd[VD_AY][idx], VXI.vd[VD_AZ][idx]) * mat->_momentInertiaInverse;
}
float CVX_Voxel::angularVelocityMagnitude() const {
  vx->syncDown();
  return (float)(Vec3D<double>(VXI.vd[VD_AX][idx], VXI.vd[VD_AY][idx], VXI.vd[VD_AZ][idx]).Length() * mat->_momentInertiaInverse);
}
float CVX_Voxel::kineticEnergy() const {
  vx->syncDown();
  Vec3D<double> l(VXI.vd[VD_LX][idx], VXI.vd[VD_LY][idx], VXI.vd[VD_LZ][idx]);
  Vec3D<double> a(VXI.vd[VD_AX][idx], VXI.vd[VD_AY][idx], VXI.vd[VD_AZ][idx]);
  return (float)(0.5 * (mat->_massInverse * l.Length2() + mat->_momentInertiaInverse * a.Length2()));
}
// CVX_Voxel::strain  VX_Voxel.cpp:300-334, on the mirror
Vec3D<float> CVX_Voxel::strain(bool poissons) const {
  vx->syncDown();
  Vec3D<float> s(0, 0, 0);
  int nb[3] = {0, 0, 0};
  bool tension[3] = {false, false, false};
  for (int i = 0; i < 6; i++)
    if (links[i]) {
      int ax = i / 2;
      s[ax] += links[i]->axialStrain(isNegative((linkDirection)i));
      nb[ax]++;
    }
  for (int i = 0; i < 3; i++) {
    if (nb[i] == 2) s[i] *= 0.5f;
    if (poissons)
      tension[i] = (nb[i] == 2) || (ext && (nb[i] == 1 && (ext->isFixed((dofComponent)(1 << i)) || ext->force()[i] != 0)));
  }
  if (poissons && !(tension[0] && tension[1] && tension[2])) {
    float add = 0;
    for (int i = 0; i < 3; i++)
      if (tension[i]) add += s[i];
    float value = std::pow(1.0f + add, -mat->poissonsRatio()) - 1.0f;
    for (int i = 0; i < 3; i++)
      if (!tension[i]) s[i] = value;
  }
  return s;
}
float CVX_Voxel::volumetricStrain() const {
  Vec3D<float> s = strain(false);
  return (float)(s.x + s.y + s.z);
}
float CVX_Voxel::pressure() const {
  return -mat->youngsModulus() * volumetricStrain() / (3 * (1 - 2 * mat->poissonsRatio()));
}
bool CVX_Voxel::isYielded() const {
  for (int i = 0; i < 6; i++)
    if (links[i] && links[i]->isYielded()) return true;
  return false;
}
bool CVX_Voxel::isFailed() const {
  for (int i = 0; i < 6; i++)
    if (links[i] && links[i]->isFailed()) return true;
  return false;
}
float CVX_Voxel::temperature() {
  vx->syncDown();
  return VXI.vf[VF_TEMP][idx];
}
void CVX_Voxel::setTemperature(float t) {  // VX_Voxel.cpp:108-114
  VxImpl& I = *vx->pimpl;
  if (I.device_ahead && I.eng && !I.state_dirty && !I.topo_dirty) {
    // the device holds the newer state: queue the change instead of a full round trip
    if (I.pend_slot.size() < vx->voxelsList.size()) I.pend_slot.resize(vx->voxelsList.size(), -1);
    int& slot = I.pend_slot[idx];
    if (slot < 0) {
      slot = (int)I.pend_voxel.size();
      I.pend_voxel.push_back(idx);
      I.pend_temp.push_back(t);
    } else {
      I.pend_temp[slot] = t;
    }
    return;
  }
  vx->syncDown();
  VXI.vf[VF_TEMP][idx] = t;
  for (int i = 0; i < 6; i++)
    if (links[i]) links[i]->updateRestLength();
  vx->markState();
}
void CVX_Voxel::haltMotion() {
  vx->syncDown();
  for (int c = 0; c < 3; ++c) { VXI.vd[VD_LX + c][idx] = 0; VXI.vd[VD_AX + c][idx] = 0; }
  vx->markState();
}
void CVX_Voxel::enableFloor(bool on) {
  vx->syncDown();
  if (on) VXI.vflags[idx] |= VXG_VF_FLOOR;
  else VXI.vflags[idx] &= ~(uint32_t)VXG_VF_FLOOR;
  vx->markState();
}
bool CVX_Voxel::isFloorEnabled() const { return (VXI.vflags[idx] & VXG_VF_FLOOR) != 0; }
bool CVX_Voxel::isFloorStaticFriction() const {
  vx->syncDown();
  return (VXI.vflags[idx] & VXG_VF_STATIC_FRICTION) != 0;
}
float CVX_Voxel::floorPenetration() const {
  return (float)(baseSizeAverage() / 2 - mat->nominalSize() / 2 - position().z);
}
// CVX_Voxel::force / moment  VX_Voxel.cpp:234-271 (contact forces are not included here)
Vec3D<double> CVX_Voxel::force() {
  vx->syncDown();
  Vec3D<double> t(0, 0, 0);
  for (int i = 0; i < 6; i++)
    if (links[i]) t += links[i]->force(isNegative((linkDirection)i));
  t = orientation().RotateVec3D(t);
  if (ext) t += ext->force();
  t -= velocity() * mat->globalDampingTranslateC();
  t.z += mat->gravityForce();
  return t;
}
Vec3D<double> CVX_Voxel::moment() {
  vx->syncDown();
  Vec3D<double> t(0, 0, 0);
  for (int i = 0; i < 6; i++)
    if (links[i]) t += links[i]->moment(isNegative((linkDirection)i));
  t = orientation().RotateVec3D(t);
  if (ext) t += ext->moment();
  t -= angularVelocity() * mat->globalDampingRotateC();
  return t;
}
Vec3D<float> CVX_Voxel::externalForce() {  // VX_Voxel.cpp:117-127
  Vec3D<float> r(external()->force());
  if (ext->isFixed(X_TRANSLATE) || ext->isFixed(Y_TRANSLATE) || ext->isFixed(Z_TRANSLATE)) {
    Vec3D<float> f = (Vec3D<float>)-force();
    if (ext->isFixed(X_TRANSLATE)) r.x = f.x;
    if (ext->isFixed(Y_TRANSLATE)) r.y = f.y;
    if (ext->isFixed(Z_TRANSLATE)) r.z = f.z;
  }
  return r;
}
Vec3D<float> CVX_Voxel::externalMoment() {  // VX_Voxel.cpp:129-139
  Vec3D<float> r(external()->moment());
  if (ext->isFixed(X_ROTATE) || ext->isFixed(Y_ROTATE) || ext->isFixed(Z_ROTATE)) {
    Vec3D<float> m = (Vec3D<float>)-moment();
    if (ext->isFixed(X_ROTATE)) r.x = m.x;
    if (ext->isFixed(Y_ROTATE)) r.y = m.y;
    if (ext->isFixed(Z_ROTATE)) r.z = m.z;
  }
  return r;
}
Vec3D<float> CVX_Voxel::cornerOffset(voxelCorner corner) const {  // VX_Voxel.cpp:146-159
  Vec3D<> s;
  for (int i = 0; i < 3; i++) {
    bool posLink = corner & (1 << (2 - i)) ? true : false;
    CVX_Link* l = links[2 * i + (posLink ? 0 : 1)];
    if (l && !l->isFailed()) s[i] = (1 + l->axialStrain(posLink)) * (posLink ? 1 : -1);
    else s[i] = posLink ? 1.0 : -1.0;
  }
  return (0.5 * baseSize()).Scale(s);
}
Vec3D<float> CVX_Voxel::cornerPosition(voxelCorner corner) const {  // VX_Voxel.cpp:141-144
  return (Vec3D<float>)position() + orientation().RotateVec3D(cornerOffset(corner));
}
// CVX_Voxel::transverseArea / transverseStrainSum with the lazily filled Poisson cache
// (VX_Voxel.cpp:336-374), on the mirror
Vec3D<float> CVX_Voxel::poissonsStrain() {
  VxImpl& I = *vx->pimpl;
  if ((I.vflags[idx] & VXG_VF_PSTRAIN_INVALID) || ((I.vflags[idx] & VXG_VF_PSTRAIN_EAGER) && I.eager_stale)) {
    Vec3D<float> p = strain(true);
    I.vf[VF_PSX][idx] = p.x; I.vf[VF_PSY][idx] = p.y; I.vf[VF_PSZ][idx] = p.z;
    I.vflags[idx] &= ~(uint32_t)(VXG_VF_PSTRAIN_INVALID | VXG_VF_PSTRAIN_EAGER);
  }
  return Vec3D<float>(I.vf[VF_PSX][idx], I.vf[VF_PSY][idx], I.vf[VF_PSZ][idx]);
}
float CVX_Voxel::transverseStrainSum(CVX_Link::linkAxis axis) {
  vx->syncDown();
  if (mat->poissonsRatio() == 0) return 0;
  Vec3D<float> p = poissonsStrain();
  switch (axis) {
    case CVX_Link::X_AXIS: return p.y + p.z;
    case CVX_Link::Y_AXIS: return p.x + p.z;
    default: return p.x + p.y;
  }
}
float CVX_Voxel::transverseArea(CVX_Link::linkAxis axis) {
  vx->syncDown();
  float size = (float)mat->nominalSize();
  if (mat->poissonsRatio() == 0) return size * size;
  Vec3D<> p = poissonsStrain();
  switch (axis) {
    case CVX_Link::X_AXIS: return (float)(size * size * (1 + p.y) * (1 + p.z));
    case CVX_Link::Y_AXIS: return (float)(size * size * (1 + p.x) * (1 + p.z));
    default: return (float)(size * size * (1 + p.x) * (1 + p.y));
  }
}
float CVX_Voxel::dampingMultiplier() {
  vx->syncDown();
  return 2 * mat->_sqrtMass * mat->zetaInternal / VXI.vf[VF_PDT][idx];
}
#undef VXI

// =============================================================================================
// CVX_Link
CVX_Link::CVX_Link(CVoxelyze* owner, CVX_Voxel* v1, CVX_Voxel* v2, CVX_MaterialLink* m)
    : vx(owner), idx(-1), mat(m) {  // VX_Link.cpp:26-59
  bool reverse = false;
  if (v1->ix == v2->ix && v1->iy == v2->iy) {
    reverse = v1->iz == v2->iz + 1;
    ax = Z_AXIS;
  } else if (v1->ix == v2->ix && v1->iz == v2->iz) {
    reverse = v1->iy == v2->iy + 1;
    ax = Y_AXIS;
  } else {
    reverse = v1->ix == v2->ix + 1;
    ax = X_AXIS;
  }
  pVNeg = reverse ? v2 : v1;
  pVPos = reverse ? v1 : v2;
}

#define LXI (*vx->pimpl)
void CVX_Link::reset() {  // VX_Link.cpp:61-75
  VxImpl& I = LXI;
  for (int c = 0; c < LD_REST; ++c) I.ld[c][idx] = 0.0;
  I.lf[LF_STRAIN][idx] = I.lf[LF_MAXS][idx] = I.lf[LF_SOFF][idx] = I.lf[LF_STRESS][idx] = 0.0f;
  I.lf[LF_RATIO][idx] = pVPos->material()->youngsModulus() / pVNeg->material()->youngsModulus();
  I.lflags[idx] = VXG_LF_SMALL_ANGLE | ((uint32_t)ax << 8);
  updateRestLength();
  updateTransverseInfo();
}
void CVX_Link::updateRestLength() {  // VX_Link.cpp:137-140
  LXI.ld[LD_REST][idx] = 0.5 * (pVNeg->baseSize(ax) + pVPos->baseSize(ax));
  vx->markState();
}
void CVX_Link::updateTransverseInfo() {  // VX_Link.cpp:142-147
  float a = 0.5f * (pVNeg->transverseArea(ax) + pVPos->transverseArea(ax));
  float s = 0.5f * (pVNeg->transverseStrainSum(ax) + pVPos->transverseStrainSum(ax));
  LXI.lf[LF_TAREA][idx] = a;
  LXI.lf[LF_TSS][idx] = s;
  vx->markState();
}
Vec3D<> CVX_Link::force(bool positiveEnd) const {
  vx->syncDown();
  int b = positiveEnd ? LD_FPX : LD_FNX;
  return Vec3D<>(LXI.ld[b][idx], LXI.ld[b + 1][idx], LXI.ld[b + 2][idx]);
}
Vec3D<> CVX_Link::moment(bool positiveEnd) const {
  vx->syncDown();
  int b = positiveEnd ? LD_MPX : LD_MNX;
  return Vec3D<>(LXI.ld[b][idx], LXI.ld[b + 1][idx], LXI.ld[b + 2][idx]);
}
float CVX_Link::axialStrain() const {
  vx->syncDown();
  return LXI.lf[LF_STRAIN][idx];
}
float CVX_Link::axialStrain(bool positiveEnd) const {  // VX_Link.cpp:121-124
  vx->syncDown();
  float s = LXI.lf[LF_STRAIN][idx], r = LXI.lf[LF_RATIO][idx];
  return positiveEnd ? 2.0f * s * r / (1.0f + r) : 2.0f * s / (1.0f + r);
}
float CVX_Link::axialStress() const {
  vx->syncDown();
  return LXI.lf[LF_STRESS][idx];
}
bool CVX_Link::isSmallAngle() const {
  vx->syncDown();
  return (LXI.lflags[idx] & VXG_LF_SMALL_ANGLE) != 0;
}
bool CVX_Link::isYielded() const {
  vx->syncDown();
  return mat->isYielded(LXI.lf[LF_MAXS][idx]);
}
bool CVX_Link::isFailed() const {
  vx->syncDown();
  return mat->isFailed(LXI.lf[LF_MAXS][idx]);
}
float CVX_Link::strainEnergy() const {  // VX_Link.cpp:251-257
  Vec3D<> fN = force(false), mN = moment(false), mP = moment(true);
  return fN.x * fN.x / (2.0f * mat->_a1) + mN.x * mN.x / (2.0 * mat->_a2) +
         (mN.z * mN.z - mN.z * mP.z + mP.z * mP.z) / (3.0 * mat->_b3) +
         (mN.y * mN.y - mN.y * mP.y + mP.y * mP.y) / (3.0 * mat->_b3);
}
float CVX_Link::axialStiffness() {  // VX_Link.cpp:259-267
  if (mat->isXyzIndependent()) return mat->_a1;
  vx->syncDown();
  updateRestLength();
  updateTransverseInfo();
  return (float)(mat->_eHat * LXI.lf[LF_TAREA][idx] / ((LXI.lf[LF_STRAIN][idx] + 1) * LXI.ld[LD_REST][idx]));
}
#undef LXI

// =============================================================================================
// vx_* C facade (include/vx_capi.h)
namespace {
struct Handle {
  CVoxelyze vx;
  std::vector<CVX_Material*> mats;
  std::unique_ptr<CVX_MeshRender> mesh;
  explicit Handle(double s) : vx(s) {}
};
Handle* H(void* s) { return static_cast<Handle*>(s); }
CVX_Voxel* Vx(void* s, int v) {
  Handle* h = H(s);
  if (v < 0 || v >= h->vx.voxelCount()) return nullptr;
  return h->vx.voxel(v);
}
}  // namespace

extern "C" {

void* vx_create(double voxel_size) { return new Handle(voxel_size); }
void vx_destroy(void* s) { delete H(s); }
int vx_add_material(void* s, float E, float rho) {
  Handle* h = H(s);
  CVX_Material* m = h->vx.addMaterial(E, rho);
  if (!m) return -1;
  h->mats.push_back(m);
  return (int)h->mats.size() - 1;
}
int vx_material_set(void* s, int mat, int prop, float v) {
  Handle* h = H(s);
  if (mat < 0 || mat >= (int)h->mats.size()) return -1;
  CVX_Material* m = h->mats[mat];
  switch (prop) {
    case 0: m->setPoissonsRatio(v); break;
    case 1: m->setCte(v); break;
    case 2: m->setStaticFriction(v); break;
    case 3: m->setKineticFriction(v); break;
    case 4: m->setInternalDamping(v); break;
    case 5: m->setGlobalDamping(v); break;
    case 6: m->setCollisionDamping(v); break;
    case 7: m->setDensity(v); break;
    default: return -1;
  }
  return 0;
}
int vx_material_set_model_linear(void* s, int mat, float E, float f) {
  Handle* h = H(s);
  if (mat < 0 || mat >= (int)h->mats.size()) return -1;
  return h->mats[mat]->setModelLinear(E, f) ? 0 : -1;
}
int vx_material_set_model_bilinear(void* s, int mat, float E, float Ep, float ys, float fs) {
  Handle* h = H(s);
  if (mat < 0 || mat >= (int)h->mats.size()) return -1;
  return h->mats[mat]->setModelBilinear(E, Ep, ys, fs) ? 0 : -1;
}
int vx_material_set_model(void* s, int mat, int n, const float* strain, const float* stress) {
  Handle* h = H(s);
  if (mat < 0 || mat >= (int)h->mats.size() || n <= 0) return -1;
  std::vector<float> a(strain, strain + n), b(stress, stress + n);
  return h->mats[mat]->setModel(n, a.data(), b.data()) ? 0 : -1;
}
float vx_material_stress(void* s, int mat, float strain, float tss, int force_linear) {
  Handle* h = H(s);
  if (mat < 0 || mat >= (int)h->mats.size()) return 0.0f;
  return h->mats[mat]->stress(strain, tss, force_linear != 0);
}
float vx_material_modulus(void* s, int mat, float strain) {
  Handle* h = H(s);
  if (mat < 0 || mat >= (int)h->mats.size()) return 0.0f;
  return h->mats[mat]->modulus(strain);
}
int vx_set_voxel(void* s, int mat, int x, int y, int z) {
  Handle* h = H(s);
  CVX_Material* m = (mat >= 0 && mat < (int)h->mats.size()) ? h->mats[mat] : nullptr;
  CVX_Voxel* v = h->vx.setVoxel(m, x, y, z);
  return v ? v->index() : -1;
}
int vx_remove_voxel(void* s, int x, int y, int z) {
  H(s)->vx.setVoxel(nullptr, x, y, z);
  return 0;
}
int vx_replace_material(void* s, int a, int b) {
  Handle* h = H(s);
  if (a < 0 || b < 0 || a >= (int)h->mats.size() || b >= (int)h->mats.size()) return -1;
  return h->vx.replaceMaterial(h->mats[a], h->mats[b]) ? 0 : -1;
}
int vx_remove_material(void* s, int m) {
  Handle* h = H(s);
  if (m < 0 || m >= (int)h->mats.size()) return -1;
  if (!h->vx.removeMaterial(h->mats[m])) return -1;
  h->mats.erase(h->mats.begin() + m);
  return 0;
}
void vx_set_voxel_size(void* s, double size) { H(s)->vx.setVoxelSize(size); }
int vx_set_voxels(void* s, int n, const int* mat, const int* xyz) {
  for (int i = 0; i < n; ++i) vx_set_voxel(s, mat[i], xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
  return 0;
}
int vx_voxel_count(void* s) { return H(s)->vx.voxelCount(); }
int vx_link_count(void* s) { return H(s)->vx.linkCount(); }
int vx_voxel_index(void* s, int x, int y, int z) {
  CVX_Voxel* v = H(s)->vx.voxel(x, y, z);
  return v ? v->index() : -1;
}
int vx_external_set_fixed(void* s, int v, int m) {
  CVX_Voxel* p = Vx(s, v);
  if (!p) return -1;
  p->external()->setFixed(m & 1, m & 2, m & 4, m & 8, m & 16, m & 32);
  return 0;
}
int vx_external_set_fixed_all(void* s, int v, int fixed) {
  CVX_Voxel* p = Vx(s, v);
  if (!p) return -1;
  p->external()->setFixedAll(fixed != 0);
  return 0;
}
int vx_external_set_displacement(void* s, int v, int dof, double value) {
  CVX_Voxel* p = Vx(s, v);
  if (!p) return -1;
  p->external()->setDisplacement((dofComponent)dof, value);
  return 0;
}
int vx_external_set_displacement_all(void* s, int v, const double* t, const double* r) {
  CVX_Voxel* p = Vx(s, v);
  if (!p) return -1;
  p->external()->setDisplacementAll(Vec3D<double>(t[0], t[1], t[2]), Vec3D<double>(r[0], r[1], r[2]));
  return 0;
}
int vx_external_clear_displacement(void* s, int v, int dof) {
  CVX_Voxel* p = Vx(s, v);
  if (!p) return -1;
  p->external()->clearDisplacement((dofComponent)dof);
  return 0;
}
int vx_external_set_force(void* s, int v, float fx, float fy, float fz) {
  CVX_Voxel* p = Vx(s, v);
  if (!p) return -1;
  p->external()->setForce(fx, fy, fz);
  return 0;
}
int vx_external_set_moment(void* s, int v, float mx, float my, float mz) {
  CVX_Voxel* p = Vx(s, v);
  if (!p) return -1;
  p->external()->setMoment(mx, my, mz);
  return 0;
}
void vx_set_gravity(void* s, float g) { H(s)->vx.setGravity(g); }
void vx_enable_floor(void* s, int e) { H(s)->vx.enableFloor(e != 0); }
void vx_enable_collisions(void* s, int e) { H(s)->vx.enableCollisions(e != 0); }
void vx_set_ambient_temperature(void* s, float t, int all) { H(s)->vx.setAmbientTemperature(t, all != 0); }
int vx_voxel_set_temperature(void* s, int v, float t) {
  CVX_Voxel* p = Vx(s, v);
  if (!p) return -1;
  p->setTemperature(t);
  return 0;
}
int vx_do_time_step(void* s, float dt) {
  int n = H(s)->vx.doTimeSteps(1, dt);
  return n < 0 ? -1 : (n == 1 ? 1 : 0);
}
int vx_do_time_steps(void* s, int n, float dt) { return H(s)->vx.doTimeSteps(n, dt); }
float vx_recommended_time_step(void* s) { return H(s)->vx.recommendedTimeStep(); }
void vx_reset_time(void* s) { H(s)->vx.resetTime(); }
int vx_load_json(void* s, const char* path) {
  Handle* h = H(s);
  h->mesh.reset();
  bool ok = h->vx.loadJSON(path);
  h->mats.clear();  // material handles index the scene's materials
  for (int i = 0; i < h->vx.materialCount(); ++i) h->mats.push_back(h->vx.material(i));
  return ok ? 1 : 0;
}
int vx_mesh_generate(void* s) {
  Handle* h = H(s);
  if (!h->mesh) h->mesh.reset(new CVX_MeshRender(&h->vx));
  else h->mesh->generateMesh();
  return h->mesh->ok() ? 0 : -1;
}
int vx_mesh_update(void* s, int coloring, int state_info) {
  Handle* h = H(s);
  if (!h->mesh || coloring < 0 || coloring > 2 || state_info < 0 || state_info > 9) return -1;
  h->mesh->updateMesh((CVX_MeshRender::viewColoring)coloring, (CVoxelyze::stateInfoType)state_info);
  return h->mesh->ok() ? 0 : -1;
}
int vx_mesh_counts(void* s, int* out3) {
  Handle* h = H(s);
  if (!h->mesh || !out3) return -1;
  out3[0] = (int)h->mesh->vertexPositions().size() / 3;
  out3[1] = (int)h->mesh->quadVertices().size() / 4;
  out3[2] = (int)h->mesh->lineVertices().size() / 2;
  return 0;
}
int vx_mesh_read(void* s, float* vertices, int* quads, float* normals, float* colors, int* lines) {
  Handle* h = H(s);
  if (!h->mesh) return -1;
  const CVX_MeshRender& m = *h->mesh;
  if (vertices) std::copy(m.vertexPositions().begin(), m.vertexPositions().end(), vertices);
  if (quads) std::copy(m.quadVertices().begin(), m.quadVertices().end(), quads);
  if (normals) std::copy(m.quadNormalValues().begin(), m.quadNormalValues().end(), normals);
  if (colors) std::copy(m.quadColorValues().begin(), m.quadColorValues().end(), colors);
  if (lines) std::copy(m.lineVertices().begin(), m.lineVertices().end(), lines);
  return 0;
}
int vx_mesh_save_obj(void* s, const char* path) {
  Handle* h = H(s);
  if (!h->mesh) return -1;
  h->mesh->saveObj(path);
  return 0;
}
int vx_save_json(void* s, const char* path) { return H(s)->vx.saveJSON(path) ? 1 : 0; }
float vx_current_time(void* s) { return H(s)->vx.currentTime(); }

int vx_get_voxel_state(void* s, double* d, float* f, int* i) {
  CVoxelyze& vx = H(s)->vx;
  VxImpl& I = *vx.impl();
  int n = vx.voxelCount();
  if (n) vx.voxel(0)->position();  // refresh the mirror
  for (int k = 0; k < n; ++k) {
    if (d) {
      double* o = d + 13 * (size_t)k;
      for (int c = 0; c < VD_N; ++c) o[c] = I.vd[c][k];
    }
    if (f) {
      float* o = f + 5 * (size_t)k;
      for (int c = 0; c < VF_N; ++c) o[c] = I.vf[c][k];
    }
    if (i) {
      i[2 * k] = (I.vflags[k] & VXG_VF_STATIC_FRICTION) ? 1 : 0;
      i[2 * k + 1] = (I.vflags[k] & VXG_VF_PSTRAIN_INVALID) ? 1 : 0;
    }
  }
  return n;
}
int vx_get_link_state(void* s, double* d, float* f, int* i) {
  CVoxelyze& vx = H(s)->vx;
  VxImpl& I = *vx.impl();
  int n = vx.linkCount();
  if (n) vx.link(0)->axialStrain();  // refresh the mirror
  for (int k = 0; k < n; ++k) {
    CVX_Link* l = vx.link(k);
    if (d) {
      double* o = d + 22 * (size_t)k;
      for (int c = 0; c < LD_N; ++c) o[c] = I.ld[c][k];
    }
    if (f) {
      float* o = f + 6 * (size_t)k;
      o[0] = I.lf[LF_STRAIN][k]; o[1] = I.lf[LF_MAXS][k]; o[2] = I.lf[LF_SOFF][k]; o[3] = I.lf[LF_STRESS][k];
      o[4] = I.lf[LF_TAREA][k]; o[5] = I.lf[LF_TSS][k];
    }
    if (i) {
      int* o = i + 6 * (size_t)k;
      o[0] = (I.lflags[k] & VXG_LF_SMALL_ANGLE) ? 1 : 0;
      o[1] = (I.lflags[k] & VXG_LF_LOCAL_VEL_VALID) ? 1 : 0;
      o[2] = (int)l->axis();
      o[3] = l->voxel(false)->index();
      o[4] = l->voxel(true)->index();
      o[5] = -1;
    }
  }
  return n;
}
int vx_get_collisions(void* s, int* pairs, int cap) {
  const std::vector<CVX_Collision*>* c = H(s)->vx.collisionList();
  int n = (int)c->size();
  for (int k = 0; k < n && k < cap; ++k) {
    pairs[2 * k] = (*c)[k]->voxel1()->index();
    pairs[2 * k + 1] = (*c)[k]->voxel2()->index();
  }
  return n;
}
float vx_state_info(void* s, int info, int type) {
  return H(s)->vx.stateInfo((CVoxelyze::stateInfoType)info, (CVoxelyze::valueType)type);
}
int vx_set_precision(void* s, int mode) {
  if (mode != 0 && mode != 1) return -1;
  H(s)->vx.setPrecision((CVoxelyze::precisionMode)mode);
  return 0;
}
int vx_read_positions(void* s, double* xyz) {
  CVoxelyze& vx = H(s)->vx;
  return vx.readField(VXG_F_POS, xyz, 3ll * vx.voxelCount()) ? 0 : -1;
}
int vx_read_positions_async(void* s, double* xyz) {
  CVoxelyze& vx = H(s)->vx;
  if (!vx.upload()) return -1;
  return vxg_read_positions_async(vx.impl()->eng, xyz) ? -1 : 0;
}
int vx_read_wait(void* s) {
  CVoxelyze& vx = H(s)->vx;
  if (!vx.impl()->eng) return 0;
  return vxg_read_wait(vx.impl()->eng) ? -1 : 0;
}
int vx_set_temperatures(void* s, const float* t) { return H(s)->vx.setTemperatures(t) ? 0 : -1; }
float vx_state_info_device(void* s, int info, int type) {
  return H(s)->vx.stateInfoDevice((CVoxelyze::stateInfoType)info, (CVoxelyze::valueType)type);
}
int vx_state_info_into(void* s, int info, int type, float* d_out, const char** why) {
  // No flush here: uploading pending host edits may allocate, so they are refused instead.
  VxImpl& I = *H(s)->vx.impl();
  if (!I.eng || I.topo_dirty || I.tables_dirty || I.state_dirty || I.act_dirty) {
    if (why) *why = "vx_state_info_into: host edits are not on the device yet (step or upload first)";
    return VXG_E_STATE;
  }
  return vxg_reduce_fixed(I.eng, info, type, d_out, why);
}
// per-voxel and per-link queries (VX_Voxel.h:79-130, VX_Link.h:47-66) on the host mirror, which
// the first read after a step downloads.  A voxel without an external answers zero for its
// external force and moment (the reference dereferences the missing external there).
static int put3f(const Vec3D<float>& f, float* out) {
  out[0] = f.x; out[1] = f.y; out[2] = f.z;
  return 0;
}
static CVX_Link* Lk(void* s, int l) {
  CVoxelyze& vx = H(s)->vx;
  return l >= 0 && l < vx.linkCount() ? vx.link(l) : nullptr;
}
int vx_voxel_external_force(void* s, int v, float* out3) {
  CVX_Voxel* p = Vx(s, v);
  if (!p || !out3) return -1;
  if (!p->externalExists()) { out3[0] = out3[1] = out3[2] = 0.0f; return 0; }
  return put3f(p->externalForce(), out3);
}
int vx_voxel_external_moment(void* s, int v, float* out3) {
  CVX_Voxel* p = Vx(s, v);
  if (!p || !out3) return -1;
  if (!p->externalExists()) { out3[0] = out3[1] = out3[2] = 0.0f; return 0; }
  return put3f(p->externalMoment(), out3);
}
int vx_voxel_corner_offset(void* s, int v, int corner, float* out3) {
  CVX_Voxel* p = Vx(s, v);
  if (!p || !out3 || corner < 0 || corner > 7) return -1;
  return put3f(p->cornerOffset((CVX_Voxel::voxelCorner)corner), out3);
}
int vx_voxel_corner_position(void* s, int v, int corner, float* out3) {
  CVX_Voxel* p = Vx(s, v);
  if (!p || !out3 || corner < 0 || corner > 7) return -1;
  return put3f(p->cornerPosition((CVX_Voxel::voxelCorner)corner), out3);
}
int vx_voxel_force(void* s, int v, double* out3) {
  CVX_Voxel* p = Vx(s, v);
  if (!p || !out3) return -1;
  Vec3D<double> f = p->force();
  out3[0] = f.x; out3[1] = f.y; out3[2] = f.z;
  return 0;
}
int vx_voxel_moment(void* s, int v, double* out3) {
  CVX_Voxel* p = Vx(s, v);
  if (!p || !out3) return -1;
  Vec3D<double> f = p->moment();
  out3[0] = f.x; out3[1] = f.y; out3[2] = f.z;
  return 0;
}
int vx_voxel_is_yielded(void* s, int v) { CVX_Voxel* p = Vx(s, v); return p ? (p->isYielded() ? 1 : 0) : -1; }
int vx_voxel_is_failed(void* s, int v) { CVX_Voxel* p = Vx(s, v); return p ? (p->isFailed() ? 1 : 0) : -1; }
float vx_voxel_pressure(void* s, int v) { CVX_Voxel* p = Vx(s, v); return p ? p->pressure() : 0.0f; }
float vx_link_strain_energy(void* s, int l) { CVX_Link* p = Lk(s, l); return p ? p->strainEnergy() : 0.0f; }
int vx_link_is_yielded(void* s, int l) { CVX_Link* p = Lk(s, l); return p ? (p->isYielded() ? 1 : 0) : -1; }
int vx_link_is_failed(void* s, int l) { CVX_Link* p = Lk(s, l); return p ? (p->isFailed() ? 1 : 0) : -1; }

int vx_counters(void* s, long long* out, int n) {
  CVoxelyze& vx = H(s)->vx;
  if (!vx.impl()->eng) return -1;
  return vxg_counters(vx.impl()->eng, out, n);
}
int vx_enable_timing(void* s, int on) {
  CVoxelyze& vx = H(s)->vx;
  if (!vx.upload()) return -1;
  return vxg_enable_timing(vx.impl()->eng, on);
}
int vx_step_timing(void* s, float* out4) {
  vxg_engine* e = H(s)->vx.impl()->eng;
  if (!e || !out4) return -1;
  vxg_last_batch_ms(e, &out4[0]);
  return vxg_last_step_timing(e, &out4[1], &out4[2], &out4[3]);
}
const char* vx_last_error(void* s) { return H(s)->vx.lastError(); }
int vx_set_actuation(void* s, int mode, double amplitude, double frequency, const float* phase) {
  CVoxelyze& vx = H(s)->vx;
  VxImpl& I = *vx.impl();
  if (mode < 0 || mode > 2 || (mode == 2 && !phase && vx.voxelCount())) return -1;
  vx.upload();
  I.act_mode = mode;
  I.act_amp = amplitude;
  I.act_freq = frequency;
  if (mode == 2) I.act_phase.assign(phase, phase + vx.voxelCount());
  else I.act_phase.clear();
  I.act_dirty = true;
  return vx.upload() ? 0 : -1;
}
int vx_body_com(void* s, const int* offsets, int n_bodies, double* out) {
  CVoxelyze& vx = H(s)->vx;
  if (!vx.upload()) return -1;
  int rc = vxg_body_com(vx.impl()->eng, offsets, n_bodies, out);
  if (rc) vx.impl()->err = vxg_last_error(vx.impl()->eng);
  return rc ? -1 : 0;
}
int vx_snapshot(void* s, int slot) {
  CVoxelyze& vx = H(s)->vx;
  if (!vx.upload()) return -1;
  int rc = vxg_snapshot(vx.impl()->eng, slot);
  if (rc) vx.impl()->err = vxg_last_error(vx.impl()->eng);
  return rc ? -1 : 0;
}
int vx_restore(void* s, int slot) {
  CVoxelyze& vx = H(s)->vx;
  if (!vx.upload()) return -1;
  int rc = vxg_restore(vx.impl()->eng, slot);
  if (rc) { vx.impl()->err = vxg_last_error(vx.impl()->eng); return -1; }
  vx.impl()->device_ahead = true;
  return 0;
}
int vx_adjoint_com_x(void* s, int nsteps, float dt, int checkpoint_every, const int* body_offsets, int n_bodies,
                     double* objective, double* dE, double* drho, double* dphase) {
  CVoxelyze& vx = H(s)->vx;
  if (!vx.upload()) return -1;
  int rc = vxg_adjoint_com_x(vx.impl()->eng, nsteps, dt, checkpoint_every, body_offsets, n_bodies, objective, dE, drho,
                             dphase);
  vx.impl()->device_ahead = true;
  if (rc) { vx.impl()->err = vxg_last_error(vx.impl()->eng); return -1; }
  return 0;
}
int vx_set_launch(void* s, int block_link, int block_voxel, int graph_chunk) {
  CVoxelyze& vx = H(s)->vx;
  if (!vx.upload()) return -1;
  return vxg_set_launch(vx.impl()->eng, block_link, block_voxel, graph_chunk) ? -1 : 0;
}
int vx_get_launch(void* s, int* block_link, int* block_voxel, int* graph_chunk) {
  CVoxelyze& vx = H(s)->vx;
  if (!vx.upload()) return -1;
  return vxg_get_launch(vx.impl()->eng, block_link, block_voxel, graph_chunk) ? -1 : 0;
}
int vx_set_link_pipeline(void* s, int blocks_per_sm) {
  CVoxelyze& vx = H(s)->vx;
  if (!vx.upload()) return -1;
  return vxg_set_link_pipeline(vx.impl()->eng, blocks_per_sm) ? -1 : 0;
}
int vx_set_link_split(void* s, int on) {
  CVoxelyze& vx = H(s)->vx;
  if (!vx.upload()) return -1;
  return vxg_set_link_split(vx.impl()->eng, on) ? -1 : 0;
}
int vx_get_link_split(void* s, int* on) {
  CVoxelyze& vx = H(s)->vx;
  if (!vx.upload()) return -1;
  return vxg_get_link_split(vx.impl()->eng, on) ? -1 : 0;
}
int vx_set_body_batches(void* s, int voxels_per_group) {
  CVoxelyze& vx = H(s)->vx;
  if (!vx.upload()) return -1;
  return vxg_set_body_batches(vx.impl()->eng, voxels_per_group) ? -1 : 0;
}
int vx_get_body_batches(void* s, int* voxels_per_group, int* groups) {
  CVoxelyze& vx = H(s)->vx;
  if (!vx.upload()) return -1;
  return vxg_get_body_batches(vx.impl()->eng, voxels_per_group, groups) ? -1 : 0;
}
int vx_set_poisson_fusion(void* s, int on) {
  CVoxelyze& vx = H(s)->vx;
  if (!vx.upload()) return -1;
  return vxg_set_poisson_fusion(vx.impl()->eng, on) ? -1 : 0;
}
void* vx_engine(void* s) {
  CVoxelyze& vx = H(s)->vx;
  return vx.upload() ? (void*)vx.impl()->eng : nullptr;
}
int vx_set_decisions(void* s, int mode, long long steps) {
  CVoxelyze& vx = H(s)->vx;
  if (!vx.upload()) return -1;
  return vxg_set_decisions(vx.impl()->eng, mode, steps) ? -1 : 0;
}
int vx_get_decisions(void* s, unsigned char* out, long long steps) {
  vxg_engine* e = H(s)->vx.impl()->eng;
  return e && vxg_get_decisions(e, out, steps) == 0 ? 0 : -1;
}
int vx_put_decisions(void* s, const unsigned char* in, long long steps) {
  vxg_engine* e = H(s)->vx.impl()->eng;
  return e && vxg_put_decisions(e, in, steps) == 0 ? 0 : -1;
}
int vx_get_link_pipeline(void* s, int* blocks_per_sm) {
  CVoxelyze& vx = H(s)->vx;
  if (!vx.upload()) return -1;
  return vxg_get_link_pipeline(vx.impl()->eng, blocks_per_sm) ? -1 : 0;
}
int vx_autotune(void* s, int trial_steps, float dt, int* out3) {
  CVoxelyze& vx = H(s)->vx;
  if (!vx.upload() || !out3) return -1;
  int rc = vxg_autotune(vx.impl()->eng, trial_steps, dt, &out3[0], &out3[1], &out3[2]);
  if (rc) vx.impl()->err = vxg_last_error(vx.impl()->eng);
  return rc ? -1 : 0;
}

}  // extern "C"
