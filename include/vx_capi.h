/* vx_capi — C facade of the drop-in CVoxelyze API, for callers that bind C symbols (ctypes, cgo,
 * JNI, N-API).  Each call wraps one call of the C++ API with the same argument meaning and error
 * behaviour; the reference interface it mirrors is cited beside it (file:line in the reference
 * tree).  Objects are addressed by index: materials in creation order, voxels in voxel-list order.
 * Calls returning int give 0 (or an index / count) on success and -1 on a bad argument.
 */
#ifndef VX_CAPI_H
#define VX_CAPI_H

#ifdef __cplusplus
extern "C" {
#endif

void* vx_create(double voxel_size);                         /* CVoxelyze(double)        src/Voxelyze.cpp:28-32 */
void vx_destroy(void* s);                                   /* ~CVoxelyze               src/Voxelyze.cpp:34-37 */
int vx_add_material(void* s, float E, float rho);           /* addMaterial(float,float) src/Voxelyze.cpp:357-366 */
int vx_material_set(void* s, int mat, int prop, float value); /* CVX_Material::set*     src/VX_Material.cpp:472-515 */
int vx_material_set_model_linear(void* s, int mat, float E, float fail_stress);   /* src/VX_Material.cpp:355-384 */
int vx_material_set_model_bilinear(void* s, int mat, float E, float plastic_E, float yield_stress,
                                   float fail_stress);                            /* src/VX_Material.cpp:389-434 */
int vx_material_set_model(void* s, int mat, int n, const float* strain, const float* stress); /* :283-350 */
float vx_material_stress(void* s, int mat, float strain, float tss, int force_linear); /* CVX_Material::stress :165-195 */
float vx_material_modulus(void* s, int mat, float strain);                            /* CVX_Material::modulus :214-226 */
int vx_set_voxel(void* s, int mat, int x, int y, int z);    /* setVoxel                 src/Voxelyze.cpp:422-437 */
int vx_remove_voxel(void* s, int x, int y, int z);          /* setVoxel(NULL, ...)      src/Voxelyze.cpp:424-427, 464-483 */
int vx_replace_material(void* s, int a, int b);             /* replaceMaterial          src/Voxelyze.cpp:406-420 */
int vx_remove_material(void* s, int m);                     /* removeMaterial           src/Voxelyze.cpp:384-404 */
void vx_set_voxel_size(void* s, double size);               /* setVoxelSize             src/Voxelyze.cpp:643-668 */
int vx_set_voxels(void* s, int n, const int* mat, const int* xyz); /* n setVoxel calls in order */
int vx_voxel_count(void* s);                                /* voxelCount               include/Voxelyze.h:98 */
int vx_link_count(void* s);                                 /* linkCount                include/Voxelyze.h:111 */
int vx_voxel_index(void* s, int x, int y, int z);           /* voxel(x,y,z) -> index or -1 */
int vx_external_set_fixed(void* s, int v, int dof_mask);    /* CVX_External::setFixed(6 bools) src/VX_External.cpp:47-51 */
int vx_external_set_fixed_all(void* s, int v, int fixed);   /* setFixedAll              include/VX_External.h:60 */
int vx_external_set_displacement(void* s, int v, int dof, double value); /* src/VX_External.cpp:53-66 */
int vx_external_set_displacement_all(void* s, int v, const double* t3, const double* r3); /* :68-75 */
int vx_external_clear_displacement(void* s, int v, int dof); /* src/VX_External.cpp:77-89 */
int vx_external_set_force(void* s, int v, float fx, float fy, float fz);  /* include/VX_External.h:69 */
int vx_external_set_moment(void* s, int v, float mx, float my, float mz); /* include/VX_External.h:71 */
void vx_set_gravity(void* s, float g);                      /* src/Voxelyze.cpp:596-602 */
void vx_enable_floor(void* s, int enabled);                 /* src/Voxelyze.cpp:604-610 */
void vx_enable_collisions(void* s, int enabled);            /* src/Voxelyze.cpp:612-622 */
void vx_set_ambient_temperature(void* s, float t, int all_voxels); /* src/Voxelyze.cpp:585-594 */
int vx_voxel_set_temperature(void* s, int v, float t);      /* CVX_Voxel::setTemperature src/VX_Voxel.cpp:108-114 */
int vx_do_time_step(void* s, float dt);                     /* doTimeStep: 1 ok, 0 diverged, -1 error  src/Voxelyze.cpp:251-284 */
int vx_do_time_steps(void* s, int n, float dt);             /* n doTimeStep calls in one GPU batch; steps completed */
float vx_recommended_time_step(void* s);                    /* src/Voxelyze.cpp:286-311 */
void vx_reset_time(void* s);                                /* src/Voxelyze.cpp:313-321 */
int vx_load_json(void* s, const char* path);                /* CVoxelyze::loadJSON  src/Voxelyze.cpp:61-77, 95-162 */
int vx_save_json(void* s, const char* path);                /* CVoxelyze::saveJSON  src/Voxelyze.cpp:79-93, 164-241 */
/* deformed mesh of the scene (one CVX_MeshRender per simulator): */
int vx_mesh_generate(void* s);                              /* CVX_MeshRender(CVoxelyze*) / generateMesh  src/VX_MeshRender.cpp:43-138 */
int vx_mesh_update(void* s, int coloring, int state_info);  /* updateMesh  src/VX_MeshRender.cpp:141-218 */
int vx_mesh_counts(void* s, int* out3);                     /* vertices, quads, edges */
int vx_mesh_read(void* s, float* vertices, int* quads, float* normals, float* colors, int* lines);
int vx_mesh_save_obj(void* s, const char* path);            /* saveObj  src/VX_MeshRender.cpp:238-252 */
float vx_current_time(void* s);                             /* CVoxelyze::currentTime   include/Voxelyze.h:138 */
/* full state dumps, layouts as in oracle/facade.h: voxels d13/f5/i2, links d22/f6/i6 */
int vx_get_voxel_state(void* s, double* d13, float* f5, int* i2);
int vx_get_link_state(void* s, double* d22, float* f6, int* i6);
int vx_get_collisions(void* s, int* pairs, int cap);        /* collisionList() as index pairs */
float vx_state_info(void* s, int info, int type);           /* stateInfo                src/Voxelyze.cpp:752-800 */
/* per-voxel and per-link queries, read from the state after the last step (the first read after a
 * step downloads it from the GPU).  Voxels by voxel-list index, links by link-list index, corners
 * as CVX_Voxel::voxelCorner (bit 2 = +x, bit 1 = +y, bit 0 = +z).  A voxel without an external
 * gives zero external force and moment (the reference dereferences its missing external there).
 * force/moment leave out collision contact forces, which stay on the GPU. */
int vx_voxel_external_force(void* s, int v, float* out3);   /* CVX_Voxel::externalForce   src/VX_Voxel.cpp:117-127 */
int vx_voxel_external_moment(void* s, int v, float* out3);  /* CVX_Voxel::externalMoment  src/VX_Voxel.cpp:129-139 */
int vx_voxel_corner_offset(void* s, int v, int corner, float* out3);   /* cornerOffset   src/VX_Voxel.cpp:146-159 */
int vx_voxel_corner_position(void* s, int v, int corner, float* out3); /* cornerPosition src/VX_Voxel.cpp:141-144 */
int vx_voxel_force(void* s, int v, double* out3);           /* CVX_Voxel::force           src/VX_Voxel.cpp:234-256 */
int vx_voxel_moment(void* s, int v, double* out3);          /* CVX_Voxel::moment          src/VX_Voxel.cpp:258-271 */
int vx_voxel_is_yielded(void* s, int v);                    /* CVX_Voxel::isYielded: 1/0  src/VX_Voxel.cpp:92-98 */
int vx_voxel_is_failed(void* s, int v);                     /* CVX_Voxel::isFailed: 1/0   src/VX_Voxel.cpp:100-106 */
float vx_voxel_pressure(void* s, int v);                    /* CVX_Voxel::pressure        include/VX_Voxel.h:103-104 */
float vx_link_strain_energy(void* s, int l);                /* CVX_Link::strainEnergy     src/VX_Link.cpp:251-257 */
int vx_link_is_yielded(void* s, int l);                     /* CVX_Link::isYielded: 1/0   src/VX_Link.cpp:127-130 */
int vx_link_is_failed(void* s, int l);                      /* CVX_Link::isFailed: 1/0    src/VX_Link.cpp:132-135 */

/* extensions for throughput users */
int vx_set_precision(void* s, int mode);                    /* 0 = FP64 (default), 1 = FP32C */
int vx_read_positions(void* s, double* xyz);                /* 3 n_voxels doubles, component-major, straight from the GPU */
int vx_read_positions_async(void* s, double* xyz);          /* the same, copied while later steps run: vxg_read_positions_async */
int vx_read_wait(void* s);                                  /* every vx_read_positions_async has landed: vxg_read_wait */
int vx_set_temperatures(void* s, const float* t);           /* n_voxels floats: every voxel's setTemperature */
float vx_state_info_device(void* s, int info, int type);    /* GPU reduction, see vxg_reduce */
/* stateInfo (info, type as vx_state_info; not PRESSURE) reduced on the GPU and written as one float
 * to d_out, a pointer into device memory of the simulation's device; no counterpart in the
 * reference, whose stateInfo (src/Voxelyze.cpp:752-800) is a host loop.  For callers that may not
 * allocate: a control loop reading the state every step, which must not stall on an allocation's
 * implicit synchronisation, or a process whose device memory is held by another allocator.  This
 * call allocates no device or host memory and does not synchronise: the value is ready once the
 * simulation's stream (vxg_stream) reaches it.  Partial results live in a fixed scratch array in
 * the library (24 KB per device), so at most 4,194,304 voxels or links are reduced; larger counts
 * return VXG_E_SIZE.  Its completion counter starts at zero when the library loads and each call
 * leaves it at zero.  The first call on a device looks the scratch up and may make the CUDA runtime
 * load this library's device code: make it before any stream capture.  Calls that overlap in time
 * on one device (several threads, streams or simulations) share the scratch and race: serialise
 * them.  Host edits not yet on the device are refused (VXG_E_STATE), not uploaded, and so is a
 * scene whose indices no step has checked yet.  In FP32C only the state fields the quantity reads
 * are converted to FP64 first (none for MASS, ENG_STRESS, ENG_STRAIN).  The simulation's device is
 * current during the call; the caller's current device is restored before it returns.  Returns 0,
 * or a VXG_E_* code with a static message in *why (why may be NULL); nothing is written to d_out
 * then. */
int vx_state_info_into(void* s, int info, int type, float* d_out, const char** why);
int vx_counters(void* s, long long* out, int n);            /* vxg_counters of the engine */
int vx_enable_timing(void* s, int on);                      /* vxg_enable_timing */
int vx_step_timing(void* s, float* out4);                   /* batch ms, link/collide/voxel ms per step */
const char* vx_last_error(void* s);
/* per-step temperature actuation inside the GPU step, see vxg_set_actuation (mode 0 off, 1 one
 * phase, 2 per-voxel phase[n_voxels]); kept across topology edits */
int vx_set_actuation(void* s, int mode, double amplitude, double frequency, const float* phase);
int vx_body_com(void* s, const int* offsets, int n_bodies, double* out);   /* vxg_body_com */
int vx_snapshot(void* s, int slot);                         /* vxg_snapshot: device checkpoint */
int vx_restore(void* s, int slot);                          /* vxg_restore (same scene only) */
/* gradient of the per-body centre-of-mass x after nsteps with respect to every voxel's E, density
 * and actuation phase: vxg_adjoint_com_x (no counterpart in the reference) */
int vx_adjoint_com_x(void* s, int nsteps, float dt, int checkpoint_every, const int* body_offsets, int n_bodies,
                     double* objective, double* dE, double* drho, double* dphase);
int vx_set_launch(void* s, int block_link, int block_voxel, int graph_chunk); /* vxg_set_launch */
int vx_get_launch(void* s, int* block_link, int* block_voxel, int* graph_chunk); /* vxg_get_launch */
int vx_autotune(void* s, int trial_steps, float dt, int* out3);            /* vxg_autotune: link, voxel, chunk */
int vx_set_link_pipeline(void* s, int blocks_per_sm);                      /* vxg_set_link_pipeline */
int vx_get_link_pipeline(void* s, int* blocks_per_sm);                     /* vxg_get_link_pipeline */
int vx_set_link_split(void* s, int on);                                    /* vxg_set_link_split */
int vx_get_link_split(void* s, int* on);                                   /* vxg_get_link_split */
int vx_set_body_batches(void* s, int voxels_per_group);                    /* vxg_set_body_batches */
int vx_get_body_batches(void* s, int* voxels_per_group, int* groups);      /* vxg_get_body_batches */
int vx_set_poisson_fusion(void* s, int on);                                /* vxg_set_poisson_fusion */
/* the engine behind a handle (include/vxg.h), pending host edits uploaded first; NULL on failure.
 * No counterpart in the reference: for callers that mix the engine ABI with this facade. */
void* vx_engine(void* s);
int vx_set_decisions(void* s, int mode, long long steps);                  /* vxg_set_decisions */
int vx_get_decisions(void* s, unsigned char* out, long long steps);        /* vxg_get_decisions */
int vx_put_decisions(void* s, const unsigned char* in, long long steps);   /* vxg_put_decisions */

#ifdef __cplusplus
}
#endif
#endif
