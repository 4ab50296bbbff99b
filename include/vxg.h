/* vxg — C ABI of the GB300 time-step engine (sm_103a).
 *
 * The drop-in C++ API (Voxelyze.h and friends) builds the scene on the host in the reference's
 * voxel and link order and drives the engine through these calls only.  Everything crossing the
 * boundary is a plain pointer plus a count; device memory never leaves the engine.  All calls
 * return 0 on success and a negative VXG_E* code otherwise; they never abort.  One engine is
 * driven by one host thread (the reference is not thread-safe either, Voxelyze.h:134).
 *
 * Reference interfaces these calls replace (file:line in the reference tree):
 *   vxg_step            CVoxelyze::doTimeStep                      src/Voxelyze.cpp:251-284
 *                         link pass  CVX_Link::updateForces         src/VX_Link.cpp:149-217
 *                         collisions CVoxelyze::updateCollisions    src/Voxelyze.cpp:670-710
 *                         voxel pass CVX_Voxel::timeStep            src/VX_Voxel.cpp:162-232
 *   vxg_recommended_dt  CVoxelyze::recommendedTimeStep             src/Voxelyze.cpp:286-311
 *   vxg_set_all_temperatures  CVoxelyze::setAmbientTemperature(t, true)  src/Voxelyze.cpp:585-594
 *   vxg_reduce          CVoxelyze::stateInfo                       src/Voxelyze.cpp:752-800
 *   vxg_set_field / vxg_get_field  the voxel and link state members  include/VX_Voxel.h:150-192,
 *                                                                    include/VX_Link.h:70-107
 */
#ifndef VXG_H
#define VXG_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct vxg_engine vxg_engine;

/* precision modes */
enum { VXG_FP64 = 0,   /* bit-faithful to the reference's double-precision arithmetic */
       VXG_FP32C = 1   /* FP32 bulk arithmetic, lattice origin + compensated FP32 displacement */ };

/* error codes */
enum { VXG_OK = 0, VXG_E_ARG = -1, VXG_E_CUDA = -2, VXG_E_STATE = -3, VXG_E_SIZE = -4,
       VXG_E_DEVICE_STATUS = -5 };

#define VXG_MAX_MODEL_POINTS 32

/* voxel flag bits (per voxel, uint32) */
enum { VXG_VF_FLOOR = 1, VXG_VF_STATIC_FRICTION = 2, VXG_VF_COLLISIONS = 4, VXG_VF_INTERIOR = 8,
       VXG_VF_PSTRAIN_INVALID = 16,
       /* FP32C: the Poisson-strain cache was filled by the voxel pass from that step's link strains,
        * ahead of the next link pass that the reference fills it in (src/VX_Voxel.cpp:336-343).  It
        * equals the lazy value unless externals, materials or link state were edited since; after
        * such an edit the next step recomputes it first. */
       VXG_VF_PSTRAIN_EAGER = 32 };
/* link flag bits (per link, uint32); bits 8..9 hold the axis */
enum { VXG_LF_SMALL_ANGLE = 1, VXG_LF_LOCAL_VEL_VALID = 2 };

/* Voxel material constants, all derived on the host exactly as CVX_MaterialVoxel::updateDerived
 * (src/VX_MaterialVoxel.cpp:57-79) and CVX_Material (include/VX_Material.h:117-140). */
typedef struct {
  float E, nu, rho, alphaCTE, muStatic, muKinetic, zetaInternal, zetaGlobal, zetaCollision;
  float mass, massInv, sqrtMass, inertia, inertiaInv, c2xSqMxExS, c2xSqIxExSxSxS;
  float gravMult, penetrationStiffness, eHat;
  float nomSizeF;  /* FP32 copies for the FP32C path, which runs no FP64 arithmetic */
  float sizeF[3];
  float sizeAvgF;  /* (size.x + size.y + size.z) / 3 */
  double nomSize;
  double size[3];  /* nomSize * external scale factor per axis (CVX_MaterialVoxel::size) */
  int powf_slot;   /* powf table slot for exponent -nu, -1 when nu == 0 */
  int pad1;
} vxg_voxel_material;

/* Link material constants (src/VX_MaterialLink.cpp:45-141) with its stress-strain model data. */
typedef struct {
  int linear, ndata;
  float E, nu, eHat, epsilonFail;
  float a1, a2, b1, b2, b3, sqA1, sqA2xIp, sqB1, sqB2xFMp, sqB3xIp;
  float strain[VXG_MAX_MODEL_POINTS], stress[VXG_MAX_MODEL_POINTS];
} vxg_link_material;

/* One voxel's externals (include/VX_External.h:92-97).  rotq is the cached quaternion the
 * reference keeps in _extRotationQ (identity unless a rotation was prescribed). */
typedef struct {
  int dof; /* dofComponent bits */
  float force[3], moment[3];
  int pad;
  double translation[3];
  double rotq[4];
} vxg_external;

typedef struct {
  int collisions;          /* CVoxelyze collisions flag */
  int any_poisson;         /* some voxel material has nu != 0 */
  float boundingRadius;    /* Voxelyze.cpp:353 */
  float watchDistance;     /* Voxelyze.cpp:354 */
  double voxSize;
  float fallback_freq2;    /* recommendedTimeStep's per-voxel E*L/m maximum, used when no link has one */
  int pad;
} vxg_globals;

/* State and topology fields for vxg_set_field / vxg_get_field.  Multi-component fields are
 * component-major: all x, then all y, ...  Counts are in elements. */
enum {
  /* voxel topology */
  VXG_F_VOXEL_MATERIAL = 0, /* int32  [n_voxels] */
  VXG_F_VOXEL_INDEX,        /* int32  [3 n_voxels] lattice ix, iy, iz */
  VXG_F_VOXEL_LINKS,        /* int32  [6 n_voxels] link per direction X+,X-,Y+,Y-,Z+,Z- or -1 */
  VXG_F_VOXEL_EXTERNAL,     /* int32  [n_voxels] external slot or -1 */
  /* voxel state */
  VXG_F_POS,                /* double [3 n_voxels] */
  VXG_F_LINMOM,             /* double [3 n_voxels] */
  VXG_F_ORIENT,             /* double [4 n_voxels] w, x, y, z */
  VXG_F_ANGMOM,             /* double [3 n_voxels] */
  VXG_F_TEMP,               /* float  [n_voxels] */
  VXG_F_PREV_DT,            /* float  [n_voxels] */
  VXG_F_PSTRAIN,            /* float  [3 n_voxels] cached Poisson strain */
  VXG_F_VOXEL_FLAGS,        /* uint32 [n_voxels] VXG_VF_* */
  /* link topology */
  VXG_F_LINK_VOXELS,        /* int32  [2 n_links] negative end, positive end */
  VXG_F_LINK_MATERIAL,      /* int32  [n_links] */
  /* link state */
  VXG_F_LINK_FLAGS,         /* uint32 [n_links] VXG_LF_* | axis << 8 */
  VXG_F_POS2,               /* double [3 n_links] */
  VXG_F_ANGLE1V,            /* double [3 n_links] */
  VXG_F_ANGLE2V,            /* double [3 n_links] */
  VXG_F_FORCE_NEG,          /* double [3 n_links] */
  VXG_F_FORCE_POS,          /* double [3 n_links] */
  VXG_F_MOMENT_NEG,         /* double [3 n_links] */
  VXG_F_MOMENT_POS,         /* double [3 n_links] */
  VXG_F_REST_LENGTH,        /* double [n_links] */
  VXG_F_STRAIN,             /* float  [n_links] */
  VXG_F_MAX_STRAIN,         /* float  [n_links] */
  VXG_F_STRAIN_OFFSET,      /* float  [n_links] */
  VXG_F_STRESS,             /* float  [n_links] */
  VXG_F_STRAIN_RATIO,       /* float  [n_links] */
  VXG_F_TRANSVERSE_AREA,    /* float  [n_links] */
  VXG_F_TRANSVERSE_STRAIN_SUM, /* float [n_links] */
  /* scalars */
  VXG_F_TIME,               /* float  [1] CVoxelyze::currentTime */
  VXG_F_COUNT
};

/* counters returned by vxg_counters */
enum { VXG_C_TRANSCENDENTAL = 0, /* correctly rounded sin/cos/acos evaluations */
       VXG_C_AMBIGUOUS = 1,      /* evaluations whose rounding could not be certified */
       VXG_C_LIBM_BAND = 2,      /* evaluations within 1/64 ulp of a rounding midpoint */
       VXG_C_POWF_MISS = 3,      /* powf arguments outside the tabulated range */
       VXG_C_REBUILDS = 4,       /* collision pair-list rebuilds */
       VXG_C_PAIRS = 5,          /* current number of collision pairs */
       VXG_C_LAUNCHES = 6,       /* kernels the time step launched (graph replays count their kernels) */
       VXG_C_COUNT = 8 };

int vxg_create(vxg_engine** out, int device, int precision);
int vxg_destroy(vxg_engine* e);
int vxg_precision(const vxg_engine* e);
/* (Re)allocates every device array for the given counts.  State is undefined until set. */
int vxg_resize(vxg_engine* e, int n_voxels, int n_links);
/* Index fields (voxel materials, externals and links, link voxels and materials) are checked on
 * the device before the first kernel that dereferences them after an upload (vxg_step,
 * vxg_recommended_dt, vxg_reduce, ...): an index out of range makes that call return VXG_E_ARG,
 * naming the field and element, and nothing runs. */
int vxg_set_field(vxg_engine* e, int field, const void* host, long long count);
int vxg_get_field(vxg_engine* e, int field, void* host, long long count);
/* Every voxel's position (VXG_F_POS: 3 n_voxels doubles, component-major) read without waiting:
 * the positions as of this call are converted into one of two device staging buffers on the
 * engine's stream and copied to `host` on a second stream, so the copy runs while later steps
 * compute.  `host` is written once vxg_read_wait returns (pinned host memory for the copy to
 * overlap; pageable memory makes the call wait for it).  A third read reuses the first staging
 * buffer once its copy has left.  No counterpart in the reference, whose positions are host
 * memory (CVX_Voxel::position, include/VX_Voxel.h:131). */
int vxg_read_positions_async(vxg_engine* e, double* host);
int vxg_read_wait(vxg_engine* e);
int vxg_set_tables(vxg_engine* e, const vxg_voxel_material* vm, int n_vm, const vxg_link_material* lm,
                   int n_lm, const vxg_external* ext, int n_ext);
/* Uploads only the externals table (the layout and slot numbering of vxg_set_tables), after
 * setForce / setMoment / setDisplacement on voxels that already have externals
 * (include/VX_External.h:39-90); captured graphs stay valid while the table keeps its size. */
int vxg_set_externals(vxg_engine* e, const vxg_external* ext, int n_ext);
/* CVX_Voxel::setTemperature (src/VX_Voxel.cpp:108-114) for n voxels at once, on the device: their
 * temperatures, then the rest lengths of their links.  Indices must be distinct. */
int vxg_set_temperatures_sparse(vxg_engine* e, int n, const int* voxels, const float* temps);
/* Deformed mesh of CVX_MeshRender (src/VX_MeshRender.cpp:49-218).  vxg_mesh_topology uploads the
 * mesh: for each vertex the 8 voxels whose corner j it is (vertex_voxels[8 i + j], -1 for none, at
 * least one per vertex) and 4 vertex indices per quad.  vxg_mesh_update computes on the device, from
 * the current state, each vertex as the average of those voxels' corner positions
 * (CVX_Voxel::cornerPosition, src/VX_Voxel.cpp:141-159) and each quad's unit normal, and copies
 * them to vertices (3 floats per vertex) and normals (3 per quad) when those are not NULL.  The
 * device copies stay readable through vxg_mesh_device_buffers (valid until the next topology). */
int vxg_mesh_topology(vxg_engine* e, int n_vertices, const int* vertex_voxels, int n_quads, const int* quads);
int vxg_mesh_update(vxg_engine* e, float* vertices, float* normals);
int vxg_mesh_device_buffers(vxg_engine* e, const float** vertices, const float** normals);
/* Tabulated powf(x, exponent) for every float x in [0.5, 2): 2^24 entries indexed by
 * (bits(x) - bits(0.5f)), computed on the host by the C library the reference links. */
int vxg_set_powf_table(vxg_engine* e, int slot, float exponent, const float* table);
int vxg_set_globals(vxg_engine* e, const vxg_globals* g);
/* Collision lattice data: per voxel, the sorted list of surface voxels within 5 link hops
 * (CVX_Voxel::generateNearby, src/VX_Voxel.cpp:395-418), CSR form. */
int vxg_set_nearby(vxg_engine* e, const int* offsets /* n_voxels+1 */, const int* items, long long n_items);
/* Runs nsteps of doTimeStep(dt); dt < 0 recomputes recommendedTimeStep every step.  Stops at the
 * first divergent step like the reference (links advanced, voxels not).  *steps_done receives the
 * number of completed steps, *diverged 1 if the run stopped on divergence. */
int vxg_step(vxg_engine* e, int nsteps, float dt, int* steps_done, int* diverged);
/* recommendedTimeStep() with its side effects on link state when nu != 0. */
int vxg_recommended_dt(vxg_engine* e, float* dt);
int vxg_set_all_temperatures(vxg_engine* e, float t);
/* Every voxel's CVX_Voxel::setTemperature at once (n_voxels floats), then every rest length. */
int vxg_set_temperatures(vxg_engine* e, const float* t);
/* stateInfo(info, type).  MIN/MAX are exact; TOTAL/AVERAGE accumulate in double. */
int vxg_reduce(vxg_engine* e, int info, int type, float* out);
/* Collision pairs in the reference's order (i < j, voxel-list order), 2 ints per pair.
 * Returns the pair count through *n (pairs beyond cap are not written). */
int vxg_get_collisions(vxg_engine* e, int* pairs, int cap, int* n);
int vxg_counters(vxg_engine* e, long long* out, int n);
/* Per-step actuation inside the step (and inside captured graphs): before every step's link pass
 * each voxel's temperature becomes amplitude * sin(2 pi frequency t + phase) with t the current
 * time, and every rest length follows - the reference's setAmbientTemperature(T, true) (mode 1)
 * or per-voxel setTemperature (mode 2, phase[n_voxels]) called before each doTimeStep
 * (src/Voxelyze.cpp:585-594, src/VX_Voxel.cpp:108-114).  Mode 0 turns it off. */
int vxg_set_actuation(vxg_engine* e, int mode, double amplitude, double frequency, const float* phase);
/* Mass-weighted centre of mass of each body, bodies being contiguous voxel ranges
 * [offsets[b], offsets[b+1]); out receives 3 doubles per body. */
int vxg_body_com(vxg_engine* e, const int* offsets, int n_bodies, double* out);
/* Launch shapes: threads per block of the link and voxel passes (64..512, 0 keeps the current) and
 * the number of steps per captured CUDA graph replayed for long runs (even; 0 keeps). */
int vxg_set_launch(vxg_engine* e, int block_link, int block_voxel, int graph_chunk);
int vxg_get_launch(vxg_engine* e, int* block_link, int* block_voxel, int* graph_chunk);
/* FP32C link pass (CVX_Link::updateForces, src/VX_Link.cpp:149-217) at a fixed dt: blocks_per_sm
 * > 0 runs the pipelined kernel (a resident grid of that many blocks per SM, clamped to what fits;
 * each tile's link state and endpoint gathers are copied into shared memory while the previous
 * tile is computed), -1 as many blocks as fit, 0 (the default) the one-thread-per-link kernel.
 * Both give identical results. */
int vxg_set_link_pipeline(vxg_engine* e, int blocks_per_sm);
int vxg_get_link_pipeline(vxg_engine* e, int* blocks_per_sm);
/* FP32C link pass at a fixed dt, one thread per link: on (1) a small-angle kernel runs every link
 * that stays in CVX_Link::orientLink's small-angle branch (src/VX_Link.cpp:92-110) and a general
 * kernel the links it deferred (large-angle, or leaving the branch this step); off (0, the default)
 * the general kernel runs every link.  Results are bit-identical either way.  vxg_autotune compares
 * both. */
int vxg_set_link_split(vxg_engine* e, int on);
int vxg_get_link_split(vxg_engine* e, int* on);
/* Body batches (no counterpart in the reference, which steps one scene per CVoxelyze): for a scene
 * of many bodies that no link joins, FP32C at a fixed dt without collisions.  The voxel order is cut
 * wherever no link spans the cut; consecutive pieces are packed into groups of up to
 * voxels_per_group voxels (1: every piece its own group; 0, the default: off), and each vxg_step
 * batch runs in one persistent launch whose CTAs take the groups largest first and run each
 * through every step of the batch (in-step actuation, links, voxels, with block barriers), so a
 * group's state stays in L2 across the steps.  Needs the links in the order of their pieces (a scene
 * built body after body) and at least one group per SM; otherwise batches run as passes.  Results
 * are bit-identical either way: each CTA first copies its group's slice of every array a step
 * writes, and a batch in which a group diverges is put back and run again as passes.
 * vxg_autotune compares group sizes with the passes.  `groups` (optional): the groups of the
 * current scene. */
int vxg_set_body_batches(vxg_engine* e, int voxels_per_group);
int vxg_get_body_batches(vxg_engine* e, int* voxels_per_group, int* groups);
/* Branch decisions of the FP64 voxel pass (no counterpart in the reference), for finite differences
 * that follow one run's branches: mode 1 records, for each of the next `steps` steps, every voxel's
 * floor-contact and static-friction decisions (CVX_Voxel::floorForce and the static-friction latch
 * of CVX_Voxel::timeStep, src/VX_Voxel.cpp:188-199, 274-298; one byte per voxel per step); mode 2
 * replays them (the run takes the recorded branches instead of comparing); 0 stops.  Setting a mode
 * restarts at the first row; a batch longer than the rows left fails with VXG_E_SIZE; steps run
 * one launch at a time meanwhile.  vxg_get_decisions / vxg_put_decisions copy the first `steps` rows
 * (steps * n_voxels bytes) out of or into the engine. */
int vxg_set_decisions(vxg_engine* e, int mode, long long steps);
int vxg_get_decisions(vxg_engine* e, unsigned char* host, long long steps);
int vxg_put_decisions(vxg_engine* e, const unsigned char* host, long long steps);
/* FP32C with Poisson's ratio != 0: on (the default), the voxel pass fills each voxel's Poisson-
 * strain cache for the next step's link pass from that step's link strains (CVX_Voxel::strain,
 * src/VX_Voxel.cpp:300-343, which the reference evaluates lazily in the next link pass); off, a
 * pre-pass fills it before every link pass.  Both give identical positions, momenta and link
 * state; the cached values read between steps are the ones the next step will use. */
int vxg_set_poisson_fusion(vxg_engine* e, int on);
/* Times short runs of the current scene for every block-size pair, (FP32C at a fixed dt) the
 * pipelined link pass at several residencies, and several graph lengths, and keeps the fastest
 * (the link-pass choice is read back with vxg_get_link_pipeline); the state is restored afterwards. */
int vxg_autotune(vxg_engine* e, int trial_steps, float dt, int* best_link, int* best_voxel, int* best_chunk);
/* Differentiated run of the FP64 path (no counterpart in the reference).  Runs nsteps steps of
 * length dt from the current state (the engine ends in the same state as after vxg_step) and
 * returns, per body (voxel ranges [body_offsets[b], body_offsets[b+1])), the mass-weighted centre
 * of mass x after the last step, and the gradient of the sum of those objectives with respect to
 * every voxel's material Young's modulus (dE), density (drho) and per-voxel actuation phase
 * (dphase, actuation mode 2), each n_voxels doubles (NULL to skip).  Gradients are taken per voxel:
 * with one material per voxel they are the derivatives with respect to that material's E and rho.
 * Reverse mode with hand-written adjoint kernels; the state is checkpointed every checkpoint_every
 * steps and each segment is recomputed once, so device memory grows with checkpoint_every.
 * Scope: linear materials (with or without a failure strain), one Poisson's ratio for every
 * voxel material (0 or not), no collisions; links in either branch of CVX_Link::orientLink;
 * externals may fix any of the degrees of freedom (a partial rotation fix is differentiated through
 * the rotation vector it zeroes); floor contact, friction, each link's branch and its failure are
 * differentiated along the branch the forward run took. */
int vxg_adjoint_com_x(vxg_engine* e, int nsteps, float dt, int checkpoint_every, const int* body_offsets,
                      int n_bodies, double* objective, double* dE, double* drho, double* dphase);
/* Full device-side copies of the simulation state (checkpoint / restart). */
int vxg_snapshot(vxg_engine* e, int slot);
int vxg_restore(vxg_engine* e, int slot);
/* Timing mode 1: vxg_step records CUDA events on the engine stream around the link pass (with the
 * Poisson pre-pass), the collision stage and the voxel pass of every step (no graph replay);
 * vxg_last_step_timing gives the per-step averages of the last batch in milliseconds and
 * vxg_last_batch_ms the device time from its first to its last kernel.  Mode 2: one event pair
 * around the whole batch as it normally runs (graph replay included); vxg_last_batch_ms gives
 * its device time.  Mode 0: off. */
int vxg_enable_timing(vxg_engine* e, int on);
int vxg_last_step_timing(vxg_engine* e, float* ms_link, float* ms_collide, float* ms_voxel);
int vxg_last_batch_ms(vxg_engine* e, float* ms);
const char* vxg_last_error(const vxg_engine* e);
void* vxg_stream(vxg_engine* e); /* cudaStream_t the engine launches on */
int vxg_synchronize(vxg_engine* e);
/* FP64 fused multiply-adds per second that `device` sustains (independent fma.rn.f64 chains on
 * every SM, best of five event-timed launches of `iters` iterations): the measured denominator of
 * the FP64 path's compute roofline.  No counterpart in the reference.  *ms = the best launch. */
int vxg_probe_fp64_rate(int device, int iters, double* fma_per_s, float* ms);

#ifdef __cplusplus
}
#endif
#endif
