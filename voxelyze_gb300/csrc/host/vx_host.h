// Private host-side state of a CVoxelyze: the structure-of-arrays mirror of the GPU state (in the
// reference's voxel-list and link-list order), the dirty flags that decide what to upload before
// the next step, and the engine handle.
#pragma once
#include <cstdint>
#include <map>
#include <string>
#include <unordered_map>
#include <vector>

#include "vxg.h"

// vxg_engine.cu: stateInfo reduction into caller device memory through fixed device scratch
// (library-internal; exposed as vx_state_info_into)
__attribute__((visibility("hidden"))) int vxg_reduce_fixed(vxg_engine* e, int info, int type, float* d_out,
                                                          const char** why);

class CVoxelyze;
class CVX_Voxel;
class CVX_Link;

// voxel doubles / floats and link doubles / floats of the mirror
enum { VD_PX, VD_PY, VD_PZ, VD_LX, VD_LY, VD_LZ, VD_OW, VD_OX, VD_OY, VD_OZ, VD_AX, VD_AY, VD_AZ, VD_N };
enum { VF_TEMP, VF_PDT, VF_PSX, VF_PSY, VF_PSZ, VF_N };
enum { LD_P2X, LD_P2Y, LD_P2Z, LD_A1X, LD_A1Y, LD_A1Z, LD_A2X, LD_A2Y, LD_A2Z, LD_FNX, LD_FNY, LD_FNZ,
       LD_FPX, LD_FPY, LD_FPZ, LD_MNX, LD_MNY, LD_MNZ, LD_MPX, LD_MPY, LD_MPZ, LD_REST, LD_N };
enum { LF_STRAIN, LF_MAXS, LF_SOFF, LF_STRESS, LF_RATIO, LF_TAREA, LF_TSS, LF_N };

struct VxImpl {
  // mirror
  std::vector<double> vd[VD_N];
  std::vector<float> vf[VF_N];
  std::vector<uint32_t> vflags;
  std::vector<double> ld[LD_N];
  std::vector<float> lf[LF_N];
  std::vector<uint32_t> lflags;  // small angle, local velocity valid, axis << 8
  float time = 0.0f;

  // lattice lookups
  std::unordered_map<uint64_t, CVX_Voxel*> vmap;
  std::unordered_map<uint64_t, CVX_Link*> lmap[3];

  // engine and synchronisation state
  vxg_engine* eng = nullptr;
  int device = 0;
  int precision = VXG_FP64;
  bool topo_dirty = true;    // counts or connectivity changed: full re-upload
  bool tables_dirty = true;  // materials / externals changed
  bool state_dirty = true;   // host mirror edited
  bool device_ahead = false; // device state newer than the mirror
  bool nearby_dirty = true;  // collision lattice lists need regeneration
  // materials or externals edited since the last step: Poisson caches the FP32C voxel pass filled
  // ahead of time (VXG_VF_PSTRAIN_EAGER) may differ from what the lazy fill would give now
  bool eager_stale = false;
  // per-voxel setTemperature calls while the device holds the newer state: applied on the device
  // (vxg_set_temperatures_sparse) before the next step or host read, the last call per voxel wins
  std::vector<int> pend_voxel;
  std::vector<float> pend_temp;
  std::vector<int> pend_slot;  // per voxel: its entry in pend_voxel, or -1
  // externals edited, none added: only the externals table is uploaded (vxg_set_externals)
  bool ext_dirty = false;
  std::vector<int> ext_voxels;  // voxels holding an external, in slot order
  // per-step actuation handed to the engine (vxg_set_actuation); re-sent after topology changes
  int act_mode = 0;
  double act_amp = 0, act_freq = 0;
  std::vector<float> act_phase;
  bool act_dirty = false;
  std::map<float, int> powf_slots;  // exponent -> table slot already on the device
  // combined link material of an (unordered) pair of voxel materials: the reference searches the
  // link-material list linearly, which is quadratic when every voxel has its own material
  struct PairHash {
    size_t operator()(const std::pair<const void*, const void*>& p) const {
      size_t a = reinterpret_cast<size_t>(p.first), b = reinterpret_cast<size_t>(p.second);
      return a * 0x9E3779B97F4A7C15ull ^ (b + 0x7F4A7C159E3779B9ull + (a << 6) + (a >> 2));
    }
  };
  std::unordered_map<std::pair<const void*, const void*>, CVX_MaterialLink*, PairHash> link_mat_of;
  static std::pair<const void*, const void*> mat_pair(const void* a, const void* b) {
    return a < b ? std::make_pair(a, b) : std::make_pair(b, a);
  }
  std::string err;

  static uint64_t key(int x, int y, int z) {
    const uint64_t B = 1u << 20;
    return ((uint64_t)(x + B) << 42) | ((uint64_t)(y + B) << 21) | (uint64_t)(z + B);
  }
  void push_voxel() {
    for (auto& a : vd) a.push_back(0.0);
    for (auto& a : vf) a.push_back(0.0f);
    vflags.push_back(0);
  }
  void push_link() {
    for (auto& a : ld) a.push_back(0.0);
    for (auto& a : lf) a.push_back(0.0f);
    lflags.push_back(0);
  }
  void erase_voxel(int i) {
    for (auto& a : vd) a.erase(a.begin() + i);
    for (auto& a : vf) a.erase(a.begin() + i);
    vflags.erase(vflags.begin() + i);
  }
  void erase_link(int i) {
    for (auto& a : ld) a.erase(a.begin() + i);
    for (auto& a : lf) a.erase(a.begin() + i);
    lflags.erase(lflags.begin() + i);
  }
  void clear_mirror() {
    for (auto& a : vd) a.clear();
    for (auto& a : vf) a.clear();
    vflags.clear();
    for (auto& a : ld) a.clear();
    for (auto& a : lf) a.clear();
    lflags.clear();
    vmap.clear();
    for (auto& m : lmap) m.clear();
  }
};
