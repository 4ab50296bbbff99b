/* Scene / stepping facade shared by the three CPU-side simulators used in tests:
 *   vxr_*  the reference library compiled from its own sources (oracle/_ref, test infrastructure)
 *   vxo_*  the oracle: a CPU restatement of the reference time step (oracle/vx_oracle.cpp)
 * The product exposes the same function list with the vx_* prefix (include/vx_capi.h), so one
 * Python driver can push an identical scene into any of them and compare the results.
 *
 * Every entry point mirrors one call of the reference's public C++ API (Voxelyze.h, VX_Material.h,
 * VX_External.h, VX_Voxel.h); the citation is on the product declaration in include/vx_capi.h.
 *
 * This header is test infrastructure. Nothing in the product includes it.
 */
#ifndef VX_ORACLE_FACADE_H
#define VX_ORACLE_FACADE_H

#ifdef __cplusplus
extern "C" {
#endif

#define VXF_DECLARE(P)                                                                              \
  void* P##_create(double voxel_size);                                                              \
  void P##_destroy(void* s);                                                                        \
  int P##_add_material(void* s, float E, float rho);                                                \
  int P##_material_set(void* s, int mat, int prop, float value);                                    \
  int P##_material_set_model_linear(void* s, int mat, float E, float fail_stress);                  \
  int P##_material_set_model_bilinear(void* s, int mat, float E, float plastic_E, float yield_stress, \
                                      float fail_stress);                                           \
  int P##_material_set_model(void* s, int mat, int n, const float* strain, const float* stress);    \
  float P##_material_stress(void* s, int mat, float strain, float tss, int force_linear);           \
  float P##_material_modulus(void* s, int mat, float strain);                                       \
  int P##_set_voxel(void* s, int mat, int x, int y, int z);                                         \
  int P##_set_voxels(void* s, int n, const int* mat, const int* xyz);                               \
  int P##_remove_voxel(void* s, int x, int y, int z);                                               \
  int P##_replace_material(void* s, int a, int b);                                                  \
  int P##_remove_material(void* s, int m);                                                          \
  void P##_set_voxel_size(void* s, double size);                                                    \
  int P##_voxel_count(void* s);                                                                     \
  int P##_link_count(void* s);                                                                      \
  int P##_voxel_index(void* s, int x, int y, int z);                                                \
  int P##_external_set_fixed(void* s, int v, int dof_mask);                                         \
  int P##_external_set_fixed_all(void* s, int v, int fixed);                                        \
  int P##_external_set_displacement(void* s, int v, int dof, double value);                         \
  int P##_external_set_displacement_all(void* s, int v, const double* t3, const double* r3);        \
  int P##_external_clear_displacement(void* s, int v, int dof);                                     \
  int P##_external_set_force(void* s, int v, float fx, float fy, float fz);                         \
  int P##_external_set_moment(void* s, int v, float mx, float my, float mz);                        \
  void P##_set_gravity(void* s, float g);                                                           \
  void P##_enable_floor(void* s, int enabled);                                                      \
  void P##_enable_collisions(void* s, int enabled);                                                 \
  void P##_set_ambient_temperature(void* s, float t, int all_voxels);                               \
  int P##_voxel_set_temperature(void* s, int v, float t);                                           \
  int P##_do_time_step(void* s, float dt);                                                          \
  int P##_do_time_steps(void* s, int n, float dt);                                                  \
  float P##_recommended_time_step(void* s);                                                         \
  void P##_reset_time(void* s);                                                                     \
  float P##_current_time(void* s);                                                                  \
  int P##_get_voxel_state(void* s, double* d13, float* f5, int* i2);                                \
  int P##_get_link_state(void* s, double* d22, float* f6, int* i6);                                 \
  int P##_get_collisions(void* s, int* pairs, int cap);                                             \
  float P##_state_info(void* s, int info, int type);                                               \
  int P##_voxel_external_force(void* s, int v, float* out3);                                        \
  int P##_voxel_external_moment(void* s, int v, float* out3);                                       \
  int P##_voxel_corner_offset(void* s, int v, int corner, float* out3);                             \
  int P##_voxel_corner_position(void* s, int v, int corner, float* out3);                           \
  int P##_voxel_force(void* s, int v, double* out3);                                                \
  int P##_voxel_moment(void* s, int v, double* out3);                                               \
  int P##_voxel_is_yielded(void* s, int v);                                                         \
  int P##_voxel_is_failed(void* s, int v);                                                          \
  float P##_voxel_pressure(void* s, int v);                                                         \
  float P##_link_strain_energy(void* s, int l);                                                     \
  int P##_link_is_yielded(void* s, int l);                                                          \
  int P##_link_is_failed(void* s, int l);

/* material property ids for *_material_set (VX_Material.h:75-107) */
enum {
  VXF_PROP_POISSON = 0,      /* setPoissonsRatio   VX_Material.cpp:472 */
  VXF_PROP_CTE = 1,          /* setCte             VX_Material.h:106 */
  VXF_PROP_MU_STATIC = 2,    /* setStaticFriction  VX_Material.cpp:487 */
  VXF_PROP_MU_KINETIC = 3,   /* setKineticFriction VX_Material.cpp:493 */
  VXF_PROP_ZETA_INTERNAL = 4,/* setInternalDamping VX_Material.cpp:499 */
  VXF_PROP_ZETA_GLOBAL = 5,  /* setGlobalDamping   VX_Material.cpp:505 */
  VXF_PROP_ZETA_COLLISION = 6,/* setCollisionDamping VX_Material.cpp:511 */
  VXF_PROP_DENSITY = 7       /* setDensity         VX_Material.cpp:480 */
};

/* Layout of the per-voxel state dump (*_get_voxel_state), voxel-list order:
 *   d13: pos.xyz, linMom.xyz, orient.wxyz, angMom.xyz          (VX_Voxel.h:163-166)
 *   f5 : temp, previousDt, pStrain.xyz                          (VX_Voxel.h:171,179,183)
 *   i2 : FLOOR_STATIC_FRICTION flag, poissonsStrainInvalid       (VX_Voxel.h:146,180)
 * Layout of the per-link state dump (*_get_link_state), link-list order:
 *   d22: pos2, angle1v, angle2v, forceNeg, forcePos, momentNeg, momentPos, currentRestLength
 *   f6 : strain, maxStrain, strainOffset, _stress, currentTransverseArea, currentTransverseStrainSum
 *   i6 : smallAngle, LOCAL_VELOCITY_VALID, axis, neg voxel index, pos voxel index, link material id
 * (VX_Link.h:70-107)
 */

#ifdef __cplusplus
}
#endif
#endif
