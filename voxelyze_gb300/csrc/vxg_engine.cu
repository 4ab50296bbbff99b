// GB300 time-step engine: device state, sm_103a kernels and the vxg_* C ABI (include/vxg.h).
//
// One step of CVoxelyze::doTimeStep (src/Voxelyze.cpp:251-284) is, on one CUDA stream:
//   k_poisson   Poisson-strain cache pre-pass (only when some material has nu != 0); fills the
//               cache the reference fills lazily from the previous step's link strains
//               (src/VX_Voxel.cpp:336-343, first touched in the link pass at src/VX_Link.cpp:160)
//   k_link      one thread per link: CVX_Link::updateForces; with dt < 0 it first evaluates
//               recommendedTimeStep's per-link term (with its side effects) and reduces the maximum
//               with warp shuffles and one atomic per block; flags divergence (strain > 100)
//   collisions  when enabled (vxg_collide.cuh)
//   k_voxel     one thread per voxel: CVX_Voxel::timeStep; gathers its 6 link slots in direction
//               order, no atomics; skips the step when the link pass diverged
// Batches of steps are enqueued back to back and, for repeated batch shapes, replayed from a
// captured CUDA graph.  Nothing is synchronised inside a batch; the host reads the control block
// once per batch.
#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <cfloat>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "vx_phys32.cuh"
#include "vx_phys64.cuh"
#include "vxg.h"

using vx64::Ctl;
using vx64::View;

namespace {

constexpr int kBlock = 256;

// ---------------------------------------------------------------------------------------------
// kernels
// REDO: also refill caches the FP32C voxel pass filled ahead of time (VXG_VF_PSTRAIN_EAGER), after
// a host edit of what they depend on (externals, materials, link state)
template <bool REDO>
__global__ void k_poisson(View S) {
  int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= S.nv) return;
  if (S.ctl->halt) return;
  uint32_t f = S.vflags[v];
  if (!(f & (REDO ? (VXG_VF_PSTRAIN_INVALID | VXG_VF_PSTRAIN_EAGER) : VXG_VF_PSTRAIN_INVALID))) return;
  if (S.vm[S.vmat[v]].nu == 0) return;
  bool any = false;
#pragma unroll
  for (int i = 0; i < 6; ++i) any |= S.vlinks[i * S.nv + v] >= 0;
  if (!any) return;
  float p[3];
  vx64::poisson_strain(S, v, p);
  S.pStrain[v] = p[0];
  S.pStrain[S.nv + v] = p[1];
  S.pStrain[2 * S.nv + v] = p[2];
  S.vflags[v] = f & ~(uint32_t)(VXG_VF_PSTRAIN_INVALID | VXG_VF_PSTRAIN_EAGER);
}

__device__ __forceinline__ void block_max_to(unsigned* dst, float f) {
  // warp max then one atomic per warp; NaN never wins (the reference's `>` test), negatives lose to 0
  unsigned u = (f > 0.0f) ? __float_as_uint(f) : 0u;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) u = max(u, __shfl_xor_sync(0xffffffffu, u, o));
  if ((threadIdx.x & 31) == 0 && u) atomicMax(dst, u);
}

template <bool RECOMMEND, bool FORCES>
__global__ void __launch_bounds__(512) k_link(View S, int parity) {
  int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (S.ctl->halt) return;
  float f2 = 0.0f;
  bool live = l < S.nl;
  if (RECOMMEND && live) {
    uint32_t lf = S.lflags[l];
    int vn = S.lvox[l], vp = S.lvox[S.nl + l];
    f2 = vx64::link_freq2(S, l, vn, vp, (lf >> 8) & 3, S.lm[S.lmat[l]]);
  }
  if (RECOMMEND) block_max_to(&S.ctl->maxf[parity], f2);
  if (!FORCES || !live) return;
  vx64::link_update(S, l);
  if (S.strain[l] > 100) S.ctl->diverged = 1;
}

// dt of this step: fixed, or 1/(2 pi sqrt(max)) from the link pass (Voxelyze.cpp:302-310)
__device__ __forceinline__ float step_dt(const View& S, bool recommend, float dt_fixed, int parity,
                                         float fallback) {
  if (!recommend) return dt_fixed;
  float mx = __uint_as_float(S.ctl->maxf[parity]);
  if (mx <= 0.0f) mx = fallback;
  if (mx <= 0.0f) return 0.0f;
  return 1.0f / (6.283185f * sqrtf(mx));
}

// The collision stale vote (CVoxelyze::updateCollisions, src/Voxelyze.cpp:686-694) for the next
// step, from this step's new positions: one warp ballot, one store per warp that saw a surface
// voxel move past the rebuild distance.  Lanes past the scene's end vote false.
__device__ __forceinline__ void col_vote(const View& S, bool moved) {
  const unsigned any = __ballot_sync(0xffffffffu, moved);
  if (any && (threadIdx.x & 31) == __ffs(any) - 1) *S.colVote = 1;
}
__device__ __forceinline__ bool col_moved(const View& S, int v, double px, double py, double pz) {
  const int nv = S.nv;
  const double dx = px - S.colLast[v], dy = py - S.colLast[nv + v], dz = pz - S.colLast[2 * nv + v];
  return dx * dx + dy * dy + dz * dz > S.colRecalc2;
}

template <bool RECOMMEND, int DEC = 0>
__global__ void __launch_bounds__(512) k_voxel(View S, float dt_fixed, int parity, float fallback,
                                               uint8_t* dec = nullptr) {
  int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (S.ctl->halt) return;
  if (S.ctl->diverged) {
    if (v == 0) S.ctl->halt = 1;
    return;
  }
  float dt = step_dt(S, RECOMMEND, dt_fixed, parity, fallback);
  if (v == 0) {
    S.ctl->steps += 1;
    S.ctl->time += dt;
    S.ctl->last_dt = dt;
    S.ctl->inv_last_dt = 1.0f / dt;
    if (RECOMMEND) S.ctl->maxf[parity ^ 1] = 0u;  // next step's slot; nobody reads it in this pass
  }
  const bool live = v < S.nv;
  if (live) vx64::voxel_update<DEC>(S, v, dt, DEC ? dec + v : nullptr);
  if (S.colVote) {  // uniform for the launch
    bool moved = false;
    if (live && !(S.vflags[v] & VXG_VF_INTERIOR))
      moved = col_moved(S, v, S.pos[v], S.pos[S.nv + v], S.pos[2 * S.nv + v]);
    col_vote(S, moved);
  }
}

// setAmbientTemperature(t, true): every voxel's temperature, then every link's rest length
// (src/Voxelyze.cpp:585-594, src/VX_Voxel.cpp:108-114, src/VX_Link.cpp:137-140)
__global__ void k_set_temp(View S, float t) {
  int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v < S.nv) S.temp[v] = t;
}
// every voxel's temperature read straight from host memory the device can address (pinned),
// 16 bytes a thread where both ends allow it
__global__ void k_temp_in(View S, const float* src) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int nv = S.nv;
  const bool vec = ((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(S.temp)) & 15) == 0;
  if (vec) {
    if (4 * i + 3 < nv) {
      reinterpret_cast<float4*>(S.temp)[i] = reinterpret_cast<const float4*>(src)[i];
    } else {
      for (int v = 4 * i; v < nv; ++v) S.temp[v] = src[v];
    }
  } else if (i < nv) {
    S.temp[i] = src[i];
  }
}
__global__ void k_rest_length(View S) {
  int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= S.nl) return;
  int axis = (S.lflags[l] >> 8) & 3;
  S.rest[l] = 0.5 * (vx64::base_size(S, S.lvox[l], axis) + vx64::base_size(S, S.lvox[S.nl + l], axis));
}

// CVX_Voxel::setTemperature on a list of voxels (src/VX_Voxel.cpp:108-114): temperatures, then
// the rest lengths of their links (a link shared by two listed voxels is written twice with the
// same value, computed from both final temperatures)
__global__ void k_temp_sparse(View S, int n, const int* idx, const float* t) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) S.temp[idx[i]] = t[i];
}
template <bool FP32>
__global__ void k_rest_sparse(vx32::View V, int n, const int* idx) {
  const View& S = V.B;
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= 6 * n) return;
  int l = S.vlinks[(k % 6) * S.nv + idx[k / 6]];
  if (l < 0) return;
  int axis = (S.lflags[l] >> 8) & 3;
  int vn = S.lvox[l], vp = S.lvox[S.nl + l];
  if (FP32) V.restDelta[l] = vx32::rest_delta(V, vn, vp, axis);
  else S.rest[l] = 0.5 * (vx64::base_size(S, vn, axis) + vx64::base_size(S, vp, axis));
}

// ---- deformed mesh: CVX_MeshRender::updateMesh geometry (src/VX_MeshRender.cpp:141-180) -------
// Position and orientation of voxel v in double: the FP64 state, or the FP32C state converted as a
// host read converts it.
__device__ __forceinline__ void mesh_pose(const View& S, const vx32::View& V, bool fp32, double s, int v,
                                          double p[3], double q[4]) {
  const int nv = S.nv;
  if (!fp32) {
    for (int k = 0; k < 3; ++k) p[k] = S.pos[k * nv + v];
    for (int k = 0; k < 4; ++k) q[k] = S.orient[k * nv + v];
    return;
  }
  const float4 d = V.P[v], o = V.Q[v];
  const float dd[3] = {d.x, d.y, d.z}, oo[4] = {o.x, o.y, o.z, o.w};
  for (int k = 0; k < 3; ++k) p[k] = S.vidx[k * nv + v] * s + ((double)dd[k] - (double)V.c[k * nv + v]);
  for (int k = 0; k < 4; ++k) q[k] = (double)oo[k] - (double)V.qc[k * nv + v];
}
// CVX_Voxel::cornerPosition (src/VX_Voxel.cpp:141-159): the corner offset from the half base size
// scaled by each axis' half-link strain (double, returned as float), rotated by the orientation
// with the float-vector quaternion rotation (Quat3D.h:179-186), added to the float position
__device__ void mesh_corner(const View& S, int v, int corner, const double p[3], const double q[4], float out[3]) {
  const int nv = S.nv;
  const vxg_voxel_material& m = S.vm[S.vmat[v]];
  const float f = 1 + S.temp[v] * m.alphaCTE;
  float off[3];
  for (int i = 0; i < 3; ++i) {
    const bool pos = corner & (1 << (2 - i));
    const int l = S.vlinks[(2 * i + (pos ? 0 : 1)) * nv + v];
    double st = pos ? 1.0 : -1.0;
    if (l >= 0) {
      const vxg_link_material& lm = S.lm[S.lmat[l]];
      const bool failed = lm.epsilonFail != -1.0f && S.maxStrain[l] > lm.epsilonFail;
      if (!failed) {
        const float s0 = S.strain[l], r = S.strainRatio[l];
        const float half = pos ? 2.0f * s0 * r / (1.0f + r) : 2.0f * s0 / (1.0f + r);  // CVX_Link::axialStrain(bool)
        st = (double)((1 + half) * (float)(pos ? 1 : -1));
      }
    }
    off[i] = (float)((0.5 * ((double)f * m.size[i])) * st);
  }
  const double w = q[0], x = q[1], y = q[2], z = q[3];
  const float fx = off[0], fy = off[1], fz = off[2];
  const float tw = (float)(fx * x + fy * y + fz * z);
  const float tx = (float)(fx * w - fy * z + fz * y);
  const float ty = (float)(fx * z + fy * w - fz * x);
  const float tz = (float)(-fx * y + fy * x + fz * w);
  out[0] = (float)p[0] + (float)(w * tx + x * tw + y * tz - z * ty);
  out[1] = (float)p[1] + (float)(w * ty - x * tz + y * tw + z * tx);
  out[2] = (float)p[2] + (float)(w * tz + x * ty - y * tx + z * tw);
}
// one mesh vertex: the average of the corner positions of the up to 8 voxels sharing it
// (vertex_voxels[8 i + j] is the voxel whose corner j the vertex is, or -1)
__global__ void k_mesh_vertices(View S, vx32::View V, int fp32, double s, int nvert, const int* vertex_voxels,
                                float* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nvert) return;
  float a[3] = {0.0f, 0.0f, 0.0f};
  int n = 0;
  for (int j = 0; j < 8; ++j) {
    const int v = vertex_voxels[8 * i + j];
    if (v < 0) continue;
    double p[3], q[4];
    mesh_pose(S, V, fp32 != 0, s, v, p, q);
    float c[3];
    mesh_corner(S, v, j, p, q, c);
    a[0] += c[0]; a[1] += c[1]; a[2] += c[2];
    ++n;
  }
  const float inv = 1.0f / (float)n;  // Vec3D::operator/= multiplies by the reciprocal
  out[3 * i] = a[0] * inv;
  out[3 * i + 1] = a[1] * inv;
  out[3 * i + 2] = a[2] * inv;
}
// quad normals: (v1 - v0) x (v3 - v0), normalised (float)
__global__ void k_mesh_normals(int nquad, const int* quads, const float* vert, float* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nquad) return;
  float v[4][3];
  for (int j = 0; j < 4; ++j)
    for (int k = 0; k < 3; ++k) v[j][k] = vert[3 * quads[4 * i + j] + k];
  const float a0 = v[1][0] - v[0][0], a1 = v[1][1] - v[0][1], a2 = v[1][2] - v[0][2];
  const float b0 = v[3][0] - v[0][0], b1 = v[3][1] - v[0][1], b2 = v[3][2] - v[0][2];
  float n0 = a1 * b2 - a2 * b1, n1 = a2 * b0 - a0 * b2, n2 = a0 * b1 - a1 * b0;
  const float l = sqrtf(n0 * n0 + n1 * n1 + n2 * n2);
  if (l > 0) {  // Vec3D::Normalize divides each component
    n0 /= l; n1 /= l; n2 /= l;
  }
  out[3 * i] = n0;
  out[3 * i + 1] = n1;
  out[3 * i + 2] = n2;
}

// stateInfo reductions (Voxelyze.cpp:752-800): per element value, block partials in double
__device__ float info_value(const View& S, int info, int i) {
  if (info == 5) return S.stress[i];
  if (info == 6) return S.strain[i];
  if (info == 7) {
    const vxg_link_material& m = S.lm[S.lmat[i]];
    int nl = S.nl;
    double fnx = S.fN[i], mnx = S.mN[i], mny = S.mN[nl + i], mnz = S.mN[2 * nl + i];
    double mpy = S.mP[nl + i], mpz = S.mP[2 * nl + i];
    return (float)(fnx * fnx / (2.0f * m.a1) + mnx * mnx / (2.0 * m.a2) + (mnz * mnz - mnz * mpz + mpz * mpz) / (3.0 * m.b3) +
                   (mny * mny - mny * mpy + mpy * mpy) / (3.0 * m.b3));
  }
  const vxg_voxel_material& m = S.vm[S.vmat[i]];
  int nv = S.nv;
  double s = m.nomSize;
  switch (info) {
    case 0: {
      double dx = S.pos[i] - S.vidx[i] * s, dy = S.pos[nv + i] - S.vidx[nv + i] * s, dz = S.pos[2 * nv + i] - S.vidx[2 * nv + i] * s;
      return (float)sqrt(dx * dx + dy * dy + dz * dz);
    }
    case 1: {
      double x = S.linMom[i], y = S.linMom[nv + i], z = S.linMom[2 * nv + i];
      return (float)(sqrt(x * x + y * y + z * z) * m.massInv);
    }
    case 2: {
      double x = S.linMom[i], y = S.linMom[nv + i], z = S.linMom[2 * nv + i];
      double a = S.angMom[i], b = S.angMom[nv + i], c = S.angMom[2 * nv + i];
      return (float)(0.5 * (m.massInv * (x * x + y * y + z * z) + m.inertiaInv * (a * a + b * b + c * c)));
    }
    case 3: {
      double w = S.orient[i];
      int f = 0;
      return (float)(2.0 * vxm::cr_acos(w > 1 ? 1 : w, &f));
    }
    case 4: {
      double a = S.angMom[i], b = S.angMom[nv + i], c = S.angMom[2 * nv + i];
      return (float)(sqrt(a * a + b * b + c * c) * m.inertiaInv);
    }
    case 9: return m.mass;
    default: return 0.0f;
  }
}
// MIN starts at FLT_MAX and MAX at -FLT_MAX, as CVoxelyze::stateInfo does (src/Voxelyze.cpp:755-756):
// an all-infinite or all-NaN field then gives the reference's answer
constexpr double kInfoMin0 = (double)FLT_MAX, kInfoMax0 = -(double)FLT_MAX;
__global__ void k_reduce(View S, int info, int n, double* out /* 3 per block: min, max, sum */) {
  __shared__ double smin[kBlock / 32], smax[kBlock / 32], ssum[kBlock / 32];
  double mn = kInfoMin0, mx = kInfoMax0, sm = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    float t = info_value(S, info, i);
    mn = t < mn ? t : mn;
    mx = t > mx ? t : mx;
    sm += t;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, o));
    mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    sm += __shfl_xor_sync(0xffffffffu, sm, o);
  }
  int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) { smin[w] = mn; smax[w] = mx; ssum[w] = sm; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 1; k < kBlock / 32; ++k) { mn = fmin(mn, smin[k]); mx = fmax(mx, smax[k]); sm += ssum[k]; }
    out[3 * blockIdx.x] = mn;
    out[3 * blockIdx.x + 1] = mx;
    out[3 * blockIdx.x + 2] = sm;
  }
}

// ---- the same reduction into caller memory with a fixed scratch array -------------------------
// Block b reduces elements [b * kFixedSpan, (b + 1) * kFixedSpan); its min, max and sum go to
// slots 3b..3b+2 of the scratch; the block that finishes last (the completion counter after the
// partials) folds the partials in block order, writes the result and sets the counter back to 0.
constexpr int kFixedBlocks = 1024;                // partial slots
constexpr int kFixedItems = 16;                   // elements per thread
constexpr int kFixedSpan = kBlock * kFixedItems;  // elements per block
constexpr long long kFixedMaxElements = (long long)kFixedBlocks * kFixedSpan;  // 4,194,304
// 24 KB + the counter.  Zero when the module loads, and zero again at the end of every call.
static __device__ __align__(256) double g_fixed_scratch[3 * kFixedBlocks + 2];

__global__ void k_reduce_fixed(View S, int info, int n, int type, double* scratch, float* out) {
  __shared__ double smin[kBlock / 32], smax[kBlock / 32], ssum[kBlock / 32];
  __shared__ int last;
  double mn = kInfoMin0, mx = kInfoMax0, sm = 0.0;
  const int base = blockIdx.x * kFixedSpan;
  for (int k = 0; k < kFixedItems; ++k) {
    int i = base + k * kBlock + threadIdx.x;
    if (i < n) {
      float t = info_value(S, info, i);
      mn = t < mn ? t : mn;
      mx = t > mx ? t : mx;
      sm += t;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, o));
    mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    sm += __shfl_xor_sync(0xffffffffu, sm, o);
  }
  int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) { smin[w] = mn; smax[w] = mx; ssum[w] = sm; }
  __syncthreads();
  unsigned* done = reinterpret_cast<unsigned*>(scratch + 3 * kFixedBlocks);
  if (threadIdx.x == 0) {
    for (int k = 1; k < kBlock / 32; ++k) { mn = fmin(mn, smin[k]); mx = fmax(mx, smax[k]); sm += ssum[k]; }
    scratch[3 * blockIdx.x] = mn;
    scratch[3 * blockIdx.x + 1] = mx;
    scratch[3 * blockIdx.x + 2] = sm;
    __threadfence();
    last = atomicAdd(done, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last || threadIdx.x != 0) return;
  __threadfence();
  const volatile double* part = scratch;
  double a = part[0], b = part[1], c = 0.0;
  for (unsigned k = 0; k < gridDim.x; ++k) {
    a = fmin(a, part[3 * k]);
    b = fmax(b, part[3 * k + 1]);
    c += part[3 * k + 2];
  }
  *out = type == 0 ? (float)a : type == 1 ? (float)b : type == 2 ? (float)c : (float)(c / n);
  *done = 0u;
  __threadfence();
}

// Every index the step kernels dereference, checked on the device once per upload of topology or
// tables: a bad value becomes an error return instead of an out-of-bounds access.  Records the
// smallest (field << 32 | element) found; reads only the index arrays themselves, in bounds.
enum { VAL_VMAT = 1, VAL_VEXT, VAL_VLINKS, VAL_LVOX, VAL_LMAT, VAL_POWSLOT };
__global__ void k_validate(View S, int n_vm, int n_lm, int n_ext, int n_powslots, unsigned long long* bad) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int nv = S.nv, nl = S.nl;
  auto flag = [&](int field, long long el) { atomicMin(bad, ((unsigned long long)field << 32) | (unsigned long long)el); };
  if (i < nv) {
    const int m = S.vmat[i], x = S.vext[i];
    if (m < 0 || m >= n_vm) flag(VAL_VMAT, i);
    if (x < -1 || x >= n_ext) flag(VAL_VEXT, i);
    for (int k = 0; k < 6; ++k) {
      const int l = S.vlinks[(size_t)k * nv + i];
      if (l < -1 || l >= nl) flag(VAL_VLINKS, (long long)k * nv + i);
    }
  }
  if (i < nl) {
    const int a = S.lvox[i], b = S.lvox[(size_t)nl + i], m = S.lmat[i];
    if (a < 0 || a >= nv) flag(VAL_LVOX, i);
    if (b < 0 || b >= nv) flag(VAL_LVOX, (long long)nl + i);
    if (m < 0 || m >= n_lm) flag(VAL_LMAT, i);
  }
  if (i < n_vm) {
    const int ps = S.vm[i].powf_slot;
    if (ps < -1 || ps >= n_powslots) flag(VAL_POWSLOT, i);
  }
}

int grid_for(int n) { return std::max(1, (n + kBlock - 1) / kBlock); }
int grid_of(int n, int b) { return std::max(1, (n + b - 1) / b); }

// ---- FP32C kernels ------------------------------------------------------------------------
// Programmatic dependent launch between the passes of a step: a pass launched with
// cudaLaunchAttributeProgrammaticStreamSerialization may start its blocks while the previous
// kernel is still running.  Before pdl_wait a block reads only state that the previous kernel does
// not write; pdl_wait returns once the previous kernel has finished and its writes are visible.  A
// block lets the next pass launch (pdl_trigger) only after its own wait, so at most two kernels
// overlap and everything before the previous kernel is complete.  Launched normally, the wait
// returns at once.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory"); }

// ACT: in-step actuation set the temperatures just before: the rest length offsets are recomputed
// here from them (no separate rest-length pass)
template <bool RECOMMEND, bool FORCES, bool POIS, bool ACT = false>
__global__ void __launch_bounds__(512) k_link32(vx32::View S, int parity) {
  int l = blockIdx.x * blockDim.x + threadIdx.x;
  // nothing is read before the wait (loading the link's own state ahead of it measured slower)
  pdl_wait();
  pdl_trigger();
  if (S.B.ctl->halt) return;
  float f2 = 0.0f;
  bool live = l < S.B.nl;
  if (RECOMMEND && live) {
    uint32_t lf = S.B.lflags[l];
    int vn = S.B.lvox[l], vp = S.B.lvox[S.B.nl + l];
    f2 = vx32::link_freq2(S, l, vn, vp, (lf >> 8) & 3, S.B.lm[S.B.lmat[l]]);
  }
  if (RECOMMEND) block_max_to(&S.B.ctl->maxf[parity], f2);
  if (!FORCES || !live) return;
  if (vx32::link_update<POIS, ACT>(S, l) > 100) S.B.ctl->diverged = 1;
}

// ---- split FP32C link pass ----------------------------------------------------------------------
// Nearly every link of a lattice stays in the small-angle branch (CVX_Link::orientLink,
// src/VX_Link.cpp:92-110), whose code needs no angle1 quaternion, rotation vector or large-angle
// pose.  k_link32s runs only that branch, with the registers it needs.  A link that is large-angle
// or leaves the small-angle branch this step is left untouched and appended to a list (one atomic
// per warp: ballot, population count, prefix in the warp); k_link32L then runs the general form on
// the listed links.  Each link writes only its own state, so the list's order does not matter and
// the results are bit-identical to the one-kernel pass.  The count is zeroed at the start of every
// batch and by every voxel pass, and each link is listed at most once per step, so the list (nl
// entries) cannot overflow.
template <bool POIS>
__global__ void __launch_bounds__(512) k_link32s(vx32::View S) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  pdl_wait();
  pdl_trigger();
  if (S.B.ctl->halt) return;
  bool defer = false;
  float axial = 0.0f;
  if (l < S.B.nl) {
    const uint32_t lf = S.B.lflags[l];
    if (lf & VXG_LF_SMALL_ANGLE) axial = vx32::link_update_small<POIS>(S, l, lf, &defer);
    else defer = true;
  }
  const unsigned m = __ballot_sync(0xffffffffu, defer);
  if (m) {
    const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(&S.B.ctl->n_large, __popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (defer) S.large[base + __popc(m & ((1u << lane) - 1u))] = l;
  }
  if (axial > 100) S.B.ctl->diverged = 1;
}
template <bool POIS>
__global__ void __launch_bounds__(256) k_link32L(vx32::View S) {
  pdl_wait();
  pdl_trigger();
  if (S.B.ctl->halt) return;
  const int n = S.B.ctl->n_large;
  bool diverged = false;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    diverged |= vx32::link_update<POIS>(S, S.large[i]) > 100;
  if (diverged) S.B.ctl->diverged = 1;
}

// ---- pipelined FP32C link pass ----------------------------------------------------------------
// The one-thread-per-link pass is latency bound: each link's work waits on a chain of dependent
// loads (link -> endpoint ids -> endpoint poses and materials), and the registers of its arithmetic
// leave too few warps resident to cover that chain.  Here a resident grid walks tiles of kLpT
// links (one link per thread, tiles handed out round robin); while a tile is computed, the next
// tile's link state and endpoint gathers are already in flight as cp.async copies into the other
// half of a double-buffered shared-memory stage, and the endpoint ids of the tile after that are
// in flight as plain loads.  Each thread copies and later reads only its own link's slots, so no
// block barrier is needed: cp.async.wait_group makes a thread's own copies visible to it.
constexpr int kLpT = 128;                                 // links per tile = threads per block
constexpr int kLpF4 = 4;                                  // float4 slots per link: P, Q of both ends
constexpr int kLpW = 24;                                  // 4-byte slots per link
constexpr int kLpStage = kLpT * (16 * kLpF4 + 4 * kLpW);  // bytes per stage (20 KB)
constexpr int kLpSmem = 2 * kLpStage;
// 4-byte slot indices
enum { LW_FLAGS, LW_MAT, LW_RD, LW_POS2, LW_A1 = LW_POS2 + 3, LW_A2 = LW_A1 + 3, LW_TAREA = LW_A2 + 3, LW_TSS,
       LW_MAXS, LW_SOFF, LW_VMN, LW_VMP, LW_PSN, LW_PSP = LW_PSN + 3, LW_END = LW_PSP + 3 };
static_assert(LW_END == kLpW, "slot count");

__device__ __forceinline__ void cp_async4(void* sdst, const void* gsrc) {
  unsigned a = (unsigned)__cvta_generic_to_shared(sdst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(a), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async16(void* sdst, const void* gsrc) {
  unsigned a = (unsigned)__cvta_generic_to_shared(sdst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(a), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

// stage layout: float4 slots [kLpF4][kLpT], then 4-byte slots [kLpW][kLpT]
template <bool POIS>
__device__ __forceinline__ void lp_issue(const vx32::View& S, char* stage, int t, int l, int vn, int vp) {
  const vx64::View& B = S.B;
  const int nl = B.nl, nv = B.nv;
  float4* f4 = reinterpret_cast<float4*>(stage);
  uint32_t* w = reinterpret_cast<uint32_t*>(stage + 16 * kLpF4 * kLpT);
  cp_async16(&f4[0 * kLpT + t], &S.P[vn]);
  cp_async16(&f4[1 * kLpT + t], &S.Q[vn]);
  cp_async16(&f4[2 * kLpT + t], &S.P[vp]);
  cp_async16(&f4[3 * kLpT + t], &S.Q[vp]);
  cp_async4(&w[LW_VMN * kLpT + t], &B.vmat[vn]);
  cp_async4(&w[LW_VMP * kLpT + t], &B.vmat[vp]);
  cp_async4(&w[LW_FLAGS * kLpT + t], &B.lflags[l]);
  cp_async4(&w[LW_MAT * kLpT + t], &B.lmat[l]);
  cp_async4(&w[LW_RD * kLpT + t], &S.restDelta[l]);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    cp_async4(&w[(LW_POS2 + k) * kLpT + t], &S.pos2[k * nl + l]);
    cp_async4(&w[(LW_A1 + k) * kLpT + t], &S.a1v[k * nl + l]);
    cp_async4(&w[(LW_A2 + k) * kLpT + t], &S.a2v[k * nl + l]);
  }
  cp_async4(&w[LW_TAREA * kLpT + t], &B.tArea[l]);
  cp_async4(&w[LW_TSS * kLpT + t], &B.tSS[l]);
  cp_async4(&w[LW_MAXS * kLpT + t], &B.maxStrain[l]);
  cp_async4(&w[LW_SOFF * kLpT + t], &B.strainOffset[l]);
  if (POIS) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      cp_async4(&w[(LW_PSN + k) * kLpT + t], &B.pStrain[k * nv + vn]);
      cp_async4(&w[(LW_PSP + k) * kLpT + t], &B.pStrain[k * nv + vp]);
    }
  }
}

template <bool POIS>
__device__ __forceinline__ vx32::LinkIn lp_read(const char* stage, int t) {
  const float4* f4 = reinterpret_cast<const float4*>(stage);
  const uint32_t* w = reinterpret_cast<const uint32_t*>(stage + 16 * kLpF4 * kLpT);
  auto F = [&](int k) { return __uint_as_float(w[k * kLpT + t]); };
  vx32::LinkIn in;
  in.dn = vx32::f3_of(f4[0 * kLpT + t]);
  in.qn = vx32::q4_of(f4[1 * kLpT + t]);
  in.dp = vx32::f3_of(f4[2 * kLpT + t]);
  in.qp = vx32::q4_of(f4[3 * kLpT + t]);
  in.vmn = (int)w[LW_VMN * kLpT + t];
  in.vmp = (int)w[LW_VMP * kLpT + t];
  in.lf = w[LW_FLAGS * kLpT + t];
  in.lmat = (int)w[LW_MAT * kLpT + t];
  in.rd = F(LW_RD);
  in.oldPos2 = vx32::F3(F(LW_POS2), F(LW_POS2 + 1), F(LW_POS2 + 2));
  in.oldA1 = vx32::F3(F(LW_A1), F(LW_A1 + 1), F(LW_A1 + 2));
  in.oldA2 = vx32::F3(F(LW_A2), F(LW_A2 + 1), F(LW_A2 + 2));
  in.tArea = F(LW_TAREA);
  in.tSS = F(LW_TSS);
  in.maxStrain = F(LW_MAXS);
  in.strainOffset = F(LW_SOFF);
  if (POIS) {
    in.psn = vx32::F3(F(LW_PSN), F(LW_PSN + 1), F(LW_PSN + 2));
    in.psp = vx32::F3(F(LW_PSP), F(LW_PSP + 1), F(LW_PSP + 2));
  } else {
    in.psn = in.psp = vx32::F3(0, 0, 0);
  }
  return in;
}

template <bool POIS>
__global__ void __launch_bounds__(kLpT) k_link32p(vx32::View S, int ntiles) {
  extern __shared__ __align__(16) char lp_smem[];
  const vx64::View& B = S.B;
  if (B.ctl->halt) return;
  const int t = threadIdx.x, nl = B.nl, G = gridDim.x;
  const float ipdt = B.ctl->inv_last_dt;  // every voxel stepped with the same dt last step
  int tile = blockIdx.x;
  if (tile >= ntiles) return;
  // prologue: ids of the first two tiles, copies of the first
  int l = tile * kLpT + t;
  if (l < nl) lp_issue<POIS>(S, lp_smem, t, l, B.lvox[l], B.lvox[nl + l]);
  cp_async_commit();
  int nt = tile + G;
  int l1 = nt * kLpT + t;
  bool ok1 = nt < ntiles && l1 < nl;
  int vn1 = 0, vp1 = 0;
  if (ok1) { vn1 = B.lvox[l1]; vp1 = B.lvox[nl + l1]; }
  bool diverged = false;
  for (int k = 0; tile < ntiles; ++k) {
    char* cur = lp_smem + (k & 1) * kLpStage;
    char* nxt = lp_smem + ((k & 1) ^ 1) * kLpStage;
    const int t2 = nt + G;
    const int l2 = t2 * kLpT + t;
    const bool ok2 = t2 < ntiles && l2 < nl;
    int vn2 = 0, vp2 = 0;
    if (ok2) { vn2 = B.lvox[l2]; vp2 = B.lvox[nl + l2]; }
    if (ok1) lp_issue<POIS>(S, nxt, t, l1, vn1, vp1);
    cp_async_commit();
    cp_async_wait1();  // this tile's copies (all but the group just committed) have landed
    l = tile * kLpT + t;
    if (l < nl) diverged |= vx32::link_compute(S, l, lp_read<POIS>(cur, t), ipdt) > 100;
    tile = nt;
    nt = t2;
    l1 = l2;
    ok1 = ok2;
    vn1 = vn2;
    vp1 = vp2;
  }
  if (diverged) B.ctl->diverged = 1;
}

template <bool RECOMMEND, bool FUSE_POIS>
__global__ void __launch_bounds__(512) k_voxel32(vx32::View S, float dt_fixed, int parity, float fallback) {
  int v = blockIdx.x * blockDim.x + threadIdx.x;
  const bool live = v < S.B.nv;
  vx32::VoxIn in;
  // the voxel's own state: neither the link pass nor the collision stage writes it
  if (live) vx32::voxel_gather_own(S, v, in);
  pdl_wait();
  pdl_trigger();
  if (v == 0) S.B.ctl->n_large = 0;  // every link pass of this step has finished with the list
  if (S.B.ctl->halt) return;
  if (S.B.ctl->diverged) {
    if (v == 0) S.B.ctl->halt = 1;
    return;
  }
  float dt = step_dt(S.B, RECOMMEND, dt_fixed, parity, fallback);
  if (v == 0) {
    S.B.ctl->steps += 1;
    S.B.ctl->time += dt;
    S.B.ctl->last_dt = dt;  // the next step's link pass reads it as every voxel's previous dt
    S.B.ctl->inv_last_dt = 1.0f / dt;
    if (RECOMMEND) S.B.ctl->maxf[parity ^ 1] = 0u;
  }
  if (!S.B.colVote) {  // uniform for the launch
    if (live) vx32::voxel_step<FUSE_POIS>(S, v, dt, in);
    return;
  }
  bool moved = false;
  if (live) {
    vx32::f3 d, c;
    vx32::voxel_step<FUSE_POIS>(S, v, dt, in, &d, &c);
    if (!(in.flags & VXG_VF_INTERIOR)) {  // the position as a host read converts it
      const int nv = S.B.nv;
      const double s = S.B.colS;
      moved = col_moved(S.B, v, S.B.vidx[v] * s + ((double)d.x - (double)c.x),
                        S.B.vidx[nv + v] * s + ((double)d.y - (double)c.y), in.iz * s + ((double)d.z - (double)c.z));
    }
  }
  col_vote(S.B, moved);
}
// ---- body batches (FP32C) ---------------------------------------------------------------------
// A scene of many bodies that no link joins (a population): the voxels split into segments that
// no link crosses, consecutive segments are packed into groups, and each CTA of one persistent
// launch takes a group (largest first, from a shared counter) and runs it through every step of the
// batch before it takes the next: per step the group's actuation temperatures, a block barrier,
// its links, a barrier, its voxels, a barrier.  A group's state is touched by one CTA only, so a
// block barrier orders a step's phases, and the group's working set stays in L2 across the steps
// instead of streaming from HBM once per pass.  The same link and voxel functions and the same
// float time arithmetic as the passes, so the same results bit for bit.  A group whose links
// diverge stops at that step and records it; the host then puts back the state the batch started
// from and runs the batch as passes, which stop where the reference stops (src/Voxelyze.cpp:263-269).
// That state is the copy each CTA makes of its group's slice of every array a step writes (the
// BodyCol list) before the group's first step; the slice's first read also brings it into L2 for
// that step.
// threads per CTA, one CTA per SM (64 registers a thread, a few spilled): 32 warps per SM measured
// 12 % faster than 512 threads with 92 registers on 4,096 bodies of 4..24 cells a side
constexpr int kBodyCta = 1024;
struct BodyCol {
  uint32_t* src;  // an array a step writes
  uint32_t* dst;  // its copy from the start of the batch
  int words;      // 32-bit words per element
  int per_link;   // indexed by link (1) or by voxel (0)
};
template <bool POIS, bool FUSE_POIS, bool ACT>
__global__ void __launch_bounds__(kBodyCta, 1)
    k_bodies32(vx32::View S, float dt, int nsteps, const int4* groups, int ngroups, int* next, float amp32, float w32,
               const float* phase, int* first_div, const BodyCol* cols, int ncols) {
  __shared__ int g_sh;
  const vx64::Ctl* ctl = S.B.ctl;
  if (ctl->halt) return;  // written before this launch
  const float time0 = ctl->time, ipdt0 = ctl->inv_last_dt, ipdt1 = 1.0f / dt;
  for (;;) {
    if (threadIdx.x == 0) g_sh = atomicAdd(next, 1);
    __syncthreads();
    const int g = g_sh;
    __syncthreads();  // every thread has read g_sh before thread 0 writes the next
    if (g >= ngroups) return;
    const int4 G = groups[g];  // voxels [x, y), links [z, w)
    for (int c = 0; c < ncols; ++c) {
      const BodyCol C = cols[c];
      const size_t e0 = (size_t)(C.per_link ? G.z : G.x) * C.words, e1 = (size_t)(C.per_link ? G.w : G.y) * C.words;
      for (size_t i = e0 + threadIdx.x; i < e1; i += kBodyCta) C.dst[i] = C.src[i];
    }
    __syncthreads();
    float time = time0, ipdt = ipdt0;
    for (int st = 0; st < nsteps; ++st) {
      if (ACT) {  // k_actuate's expression, at the group's own copy of the time
        for (int v = G.x + threadIdx.x; v < G.y; v += kBodyCta)
          S.B.temp[v] = amp32 * sinf(w32 * time + (phase ? phase[v] : 0.0f));
        __syncthreads();
      }
      bool div = false;
      for (int l = G.z + threadIdx.x; l < G.w; l += kBodyCta) div |= vx32::link_update_ip<POIS, ACT>(S, l, ipdt) > 100;
      if (__syncthreads_or(div)) {
        if (threadIdx.x == 0) atomicMin(first_div, st);
        break;
      }
      for (int v = G.x + threadIdx.x; v < G.y; v += kBodyCta) vx32::voxel_update<FUSE_POIS>(S, v, dt);
      __syncthreads();
      time += dt;  // k_voxel32's accumulation
      ipdt = ipdt1;
    }
  }
}
// the batch's first four control words (diverged, halt, steps, status) into mapped host memory
__global__ void k_ctl_out(const vx64::Ctl* ctl, int* out) {
  const int* w = reinterpret_cast<const int*>(ctl);
  if (threadIdx.x < 4) out[threadIdx.x] = w[threadIdx.x];
}
// after k_bodies32: the control words of a batch that ran to its end (the voxel pass's updates,
// step by step); a batch some group diverged in is flagged (diverged without halt) for the host,
// which runs it again as passes.  Leaves the counter and the first diverged step for the next batch.
__global__ void k_bodies_done(vx64::Ctl* ctl, float dt, int nsteps, int* bctl) {
  if (threadIdx.x != 0) return;
  const int fd = bctl[1];
  bctl[0] = 0;
  bctl[1] = INT_MAX;
  if (ctl->halt) return;
  if (fd < nsteps) {
    ctl->diverged = 1;
    return;
  }
  float t = ctl->time;
  for (int k = 0; k < nsteps; ++k) t += dt;
  ctl->time = t;
  ctl->steps += nsteps;
  ctl->last_dt = dt;
  ctl->inv_last_dt = 1.0f / dt;
}

// FP64 interchange fields <-> FP32C working state, one field per launch (only the fields the host
// writes are converted on upload, only the fields it reads on download)
__global__ void k_conv(vx32::View S, double s, int field, int to32) {
  const vx64::View& B = S.B;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int nv = B.nv, nl = B.nl;
  auto cv = [&](double* d64, float* d32, int comps, int n) {
    if (i >= n) return;
    for (int k = 0; k < comps; ++k) {
      if (to32) d32[k * n + i] = (float)d64[k * n + i];
      else d64[k * n + i] = d32[k * n + i];
    }
  };
  switch (field) {
    case VXG_F_POS:
      if (i < nv)
        for (int k = 0; k < 3; ++k) {
          if (to32) {
            double dd = B.pos[k * nv + i] - B.vidx[k * nv + i] * s;
            float d = (float)dd;
            reinterpret_cast<float*>(&S.P[i])[k] = d;
            S.c[k * nv + i] = (float)((double)d - dd);  // true displacement = d - c
          } else {
            B.pos[k * nv + i] = B.vidx[k * nv + i] * s +
                                ((double)reinterpret_cast<const float*>(&S.P[i])[k] - (double)S.c[k * nv + i]);
          }
        }
      break;
    case VXG_F_LINMOM: cv(B.linMom, S.lin, 3, nv); break;
    case VXG_F_ORIENT:
      if (i < nv)
        for (int k = 0; k < 4; ++k) {
          if (to32) {
            double q64 = B.orient[k * nv + i];
            float q = (float)q64;
            reinterpret_cast<float*>(&S.Q[i])[k] = q;
            S.qc[k * nv + i] = (float)((double)q - q64);  // true orientation = q - qc
          } else {
            B.orient[k * nv + i] = (double)reinterpret_cast<const float*>(&S.Q[i])[k] - (double)S.qc[k * nv + i];
          }
        }
      break;
    case VXG_F_ANGMOM: cv(B.angMom, S.ang, 3, nv); break;
    case VXG_F_PREV_DT:
      if (to32) {
        if (i == 0 && nv) {
          B.ctl->last_dt = B.prevDt[0];
          B.ctl->inv_last_dt = 1.0f / B.prevDt[0];
        }
      }
      else if (i < nv) B.prevDt[i] = B.ctl->last_dt;
      break;
    case VXG_F_POS2: cv(B.pos2, S.pos2, 3, nl); break;
    case VXG_F_ANGLE1V: cv(B.a1v, S.a1v, 3, nl); break;
    case VXG_F_ANGLE2V: cv(B.a2v, S.a2v, 3, nl); break;
    case VXG_F_FORCE_NEG: cv(B.fN, S.fN, 3, nl); break;
    case VXG_F_FORCE_POS: cv(B.fP, S.fP, 3, nl); break;
    case VXG_F_MOMENT_NEG: cv(B.mN, S.mN, 3, nl); break;
    case VXG_F_MOMENT_POS: cv(B.mP, S.mP, 3, nl); break;
    case VXG_F_REST_LENGTH:
      if (i < nl) {
        if (to32) S.restDelta[i] = (float)(B.rest[i] - s);
        else B.rest[i] = s + (double)S.restDelta[i];
      }
      break;
    default: break;
  }
}
// FP32C positions converted straight into a destination the device can write (pinned host memory
// reached over the host link, or device memory): the same conversion as k_conv, no staging copy
__global__ void k_pos_out(vx32::View S, double s, double* dst) {
  const vx64::View& B = S.B;
  const int nv = B.nv;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nv) return;
  const float4 d = S.P[i];
  const float dd[3] = {d.x, d.y, d.z};
#pragma unroll
  for (int k = 0; k < 3; ++k) dst[k * nv + i] = B.vidx[k * nv + i] * s + ((double)dd[k] - (double)S.c[k * nv + i]);
}

// Per-step actuation: before each step's link pass every voxel's temperature is set to
//   amplitude * sin(2 pi frequency t + phase)      (t = CVoxelyze::currentTime at the step start)
// and every rest length follows, i.e. the reference's setAmbientTemperature(T, true) (mode 1, one
// phase) or CVX_Voxel::setTemperature per voxel (mode 2, per-voxel phase) before doTimeStep
// (src/Voxelyze.cpp:585-594, src/VX_Voxel.cpp:108-114).  Evaluated in double with the correctly
// rounded sine on the FP64 path, in float on the FP32C path; the result is rounded to float like
// the reference's float temperature argument.
// The actuation temperature amp * sin(2 pi freq t + phase[v]) of every voxel at the step's start
// time t.  FP64: the argument and the sine in double, rounded once to the float temperature as the
// reference's driver would compute it.  FP32C (fp32 != 0): in float (w32 = 2 pi freq and amp32 as
// floats), which keeps the FP64 pipe out of the pass.  Launched to overlap the previous voxel
// pass's tail where that pass is the kernel before it: nothing is read before the wait.
__global__ void k_actuate(View S, double amp, double freq, const float* phase, int fp32, float amp32, float w32) {
  pdl_wait();
  pdl_trigger();
  int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= S.nv || S.ctl->halt) return;
  float t;
  if (fp32) {
    t = amp32 * sinf(w32 * S.ctl->time + (phase ? phase[v] : 0.0f));
  } else {
    const double arg = 2.0 * 3.141592653589793 * freq * (double)S.ctl->time + (phase ? (double)phase[v] : 0.0);
    // Ziv's rounding test: only the float result is kept.  The library sine is within a few ulp of
    // sin(arg), so amp * sin(arg) lies within 2^-45 (relative) of y; when that whole interval
    // rounds to one float, it is the float the correctly rounded sine gives.  Otherwise (about one
    // value in four million), and for y == 0, evaluate the correctly rounded sine.
    const double y = amp * sin(arg);
    const double d = fabs(y) * 0x1p-45;
    const float lo = __double2float_rn(y - d), hi = __double2float_rn(y + d);
    if (y != 0.0 && lo == hi) {
      t = lo;
    } else {
      int f = 0;
      t = (float)(amp * vxm::cr_sin(arg, &f));
    }
  }
  S.temp[v] = t;
}

// mass-weighted centre of mass of contiguous voxel ranges (one block per body), double accumulation
__global__ void k_body_com(View S, const float4* d32, const float* c32, double s, const int* off, double* out) {
  int b = blockIdx.x;
  int lo = off[b], hi = off[b + 1];
  double m = 0, x = 0, y = 0, z = 0;
  for (int v = lo + threadIdx.x; v < hi; v += blockDim.x) {
    double mv = S.vm[S.vmat[v]].mass, px, py, pz;
    if (d32) {
      float4 d = d32[v];
      px = S.vidx[v] * s + ((double)d.x - (double)c32[v]);
      py = S.vidx[S.nv + v] * s + ((double)d.y - (double)c32[S.nv + v]);
      pz = S.vidx[2 * S.nv + v] * s + ((double)d.z - (double)c32[2 * S.nv + v]);
    } else {
      px = S.pos[v]; py = S.pos[S.nv + v]; pz = S.pos[2 * S.nv + v];
    }
    m += mv; x += mv * px; y += mv * py; z += mv * pz;
  }
  __shared__ double sh[4][32];
  for (int o = 16; o > 0; o >>= 1) {
    m += __shfl_xor_sync(0xffffffffu, m, o);
    x += __shfl_xor_sync(0xffffffffu, x, o);
    y += __shfl_xor_sync(0xffffffffu, y, o);
    z += __shfl_xor_sync(0xffffffffu, z, o);
  }
  int w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  if ((threadIdx.x & 31) == 0) { sh[0][w] = m; sh[1][w] = x; sh[2][w] = y; sh[3][w] = z; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 1; k < nw; ++k) { m += sh[0][k]; x += sh[1][k]; y += sh[2][k]; z += sh[3][k]; }
    out[3 * b] = m > 0 ? x / m : 0.0;
    out[3 * b + 1] = m > 0 ? y / m : 0.0;
    out[3 * b + 2] = m > 0 ? z / m : 0.0;
  }
}

__global__ void k_rest32(vx32::View S) {
  int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= S.B.nl) return;
  int axis = (S.B.lflags[l] >> 8) & 3;
  S.restDelta[l] = vx32::rest_delta(S, S.B.lvox[l], S.B.lvox[S.B.nl + l], axis);
}

}  // namespace

// ---------------------------------------------------------------------------------------------
struct FieldDesc {
  size_t elem;  // bytes per element
  int comps;    // elements per voxel or link
  bool per_link;
};

static FieldDesc field_desc(int f) {
  switch (f) {
    case VXG_F_VOXEL_MATERIAL: return {4, 1, false};
    case VXG_F_VOXEL_INDEX: return {4, 3, false};
    case VXG_F_VOXEL_LINKS: return {4, 6, false};
    case VXG_F_VOXEL_EXTERNAL: return {4, 1, false};
    case VXG_F_POS: return {8, 3, false};
    case VXG_F_LINMOM: return {8, 3, false};
    case VXG_F_ORIENT: return {8, 4, false};
    case VXG_F_ANGMOM: return {8, 3, false};
    case VXG_F_TEMP: return {4, 1, false};
    case VXG_F_PREV_DT: return {4, 1, false};
    case VXG_F_PSTRAIN: return {4, 3, false};
    case VXG_F_VOXEL_FLAGS: return {4, 1, false};
    case VXG_F_LINK_VOXELS: return {4, 2, true};
    case VXG_F_LINK_MATERIAL: return {4, 1, true};
    case VXG_F_LINK_FLAGS: return {4, 1, true};
    case VXG_F_POS2: case VXG_F_ANGLE1V: case VXG_F_ANGLE2V: case VXG_F_FORCE_NEG: case VXG_F_FORCE_POS:
    case VXG_F_MOMENT_NEG: case VXG_F_MOMENT_POS: return {8, 3, true};
    case VXG_F_REST_LENGTH: return {8, 1, true};
    case VXG_F_STRAIN: case VXG_F_MAX_STRAIN: case VXG_F_STRAIN_OFFSET: case VXG_F_STRESS:
    case VXG_F_STRAIN_RATIO: case VXG_F_TRANSVERSE_AREA: case VXG_F_TRANSVERSE_STRAIN_SUM: return {4, 1, true};
    default: return {0, 0, false};
  }
}

#include "vxg_collide.cuh"
#include "vxg_adjoint.cuh"

struct vxg_engine {
  int device = 0;
  int precision = VXG_FP64;
  int nv = 0, nl = 0;
  cudaStream_t stream = nullptr;
  // vxg_read_positions_async: two device staging buffers (3 nv doubles each), copied to the host on
  // their own stream while later steps run; a buffer is reused only after its last copy has left
  cudaStream_t cstream = nullptr;
  double* d_stage[2] = {nullptr, nullptr};
  size_t stage_bytes = 0;
  cudaEvent_t ev_staged[2] = {nullptr, nullptr}, ev_copied[2] = {nullptr, nullptr};
  bool stage_used[2] = {false, false};
  int stage_next = 0;
  char* arena = nullptr;
  size_t arena_bytes = 0;
  void* field_ptr[VXG_F_COUNT] = {};
  View S{};
  vx32::View V{};          // FP32C working state (precision == VXG_FP32C)
  char* arena32 = nullptr;
  size_t arena32_bytes = 0;
  uint32_t dirty64 = 0;    // FP32C: state fields the host wrote, not yet converted to FP32
  uint32_t stale64 = 0;    // FP32C: state fields whose FP64 copy is older than the FP32 state
  Ctl* ctl = nullptr;
  vxg_voxel_material* d_vm = nullptr;
  vxg_link_material* d_lm = nullptr;
  vxg_external* d_ext = nullptr;
  int n_vm = 0, n_lm = 0, n_ext = 0;        // live entries
  int cap_vm = 0, cap_lm = 0, cap_ext = 0;  // allocated entries
  float* d_powtab = nullptr;
  int n_powslots = 0;
  double* d_partials = nullptr;
  vxg_globals g{};
  bool have_globals = false;
  Collide col;
  // whether the scene is inside the differentiated scope (set with the tables)
  const char* adj_scope = "no tables";
  int timing = 0;                 // 0 off, 1 per-pass events every step, 2 one event pair per batch
  cudaEvent_t bev[2] = {nullptr, nullptr};
  cudaEvent_t ev[4] = {};
  std::vector<cudaEvent_t> tev;  // timing mode: 4 events per step of the last batch
  int tev_used = 0;
  float t_link = 0, t_col = 0, t_vox = 0, t_batch = 0;
  std::string err;
  // captured batches: a graph of `graph_chunk` steps replayed for long runs, and one for short ones
  cudaGraphExec_t graph = nullptr;
  int graph_n = -1;
  float graph_dt = 0;
  bool graph_valid = false;
  cudaGraphExec_t cgraph = nullptr;
  float cgraph_dt = 0;
  int cgraph_n = -1;
  // single steps (a control loop calling one step at a time): the step captured as well, with and
  // without the rest-length update of host-set temperatures in its link pass
  cudaGraphExec_t g1[2] = {nullptr, nullptr};
  float g1_dt[2] = {0, 0};
  long long g1_kernels[2] = {0, 0};
  int graph_chunk = 64;
  // launch shapes (vxg_set_launch / vxg_autotune)
  int blk_link = 256, blk_voxel = 256;
  // FP32C link pass: resident blocks per SM of the pipelined kernel (-1: as many as fit; 0, the
  // default: the one-thread-per-link kernel instead), and the occupancy limits found for it
  int lp_bps = 0;
  int lp_fit[2] = {0, 0};
  // FP32C at a fixed dt with the one-thread-per-link kernels: the small-angle pass plus the general
  // pass over the links it deferred (1), or the general pass over every link (0, the default: the
  // small-angle kernel needs as many registers as the general one, and the second launch made the
  // step slower, 0.150 against 0.144 ms on the 128x128x64 lattice)
  int link_split = 0;
  // FP32C: temperatures the host set (vxg_set_temperatures, vxg_set_all_temperatures) whose links'
  // rest lengths are not recomputed yet; the next step's link pass or a rest-length pass does it
  bool rest_pending = false;
  // body batches (k_bodies32; vxg_set_body_batches, vxg_autotune): voxels per group (0: off), the
  // groups of the current topology (built for groups_target), and the device words [next group,
  // first diverged step]
  int body_target = 0;
  bool groups_valid = false;
  int groups_target = 0, n_groups = 0, n_groups_cap = 0;
  int4* d_groups = nullptr;
  int* d_bctl = nullptr;
  int body_fit = -1;  // k_bodies32 CTAs resident per SM (-1: not yet asked)
  bool body_rerun = false;  // running a diverged body batch again as passes
  BodyCol* d_body_cols = nullptr;
  uint32_t* d_body_bak = nullptr;
  std::vector<BodyCol> body_cols;
  int lL_grid = 0;  // grid of the general pass over deferred links (resident blocks on every SM)
  int n_sm = 0;
  bool tab_poisson = false;  // some voxel material has nu != 0
  // FP32C with nu != 0: the voxel pass fills the Poisson cache for the next step; a host edit since
  // the last step makes the next batch refill those caches first (k_poisson<true>)
  bool poisson_redo = true;
  bool poisson_fuse = true;  // vxg_set_poisson_fusion
  bool pdl = true;           // FP32C passes launched to overlap the previous kernel's tail
  bool topo_ok = false;      // k_validate passed for the current index fields and tables
  unsigned long long* d_bad = nullptr;
  // the batch's control words in mapped pinned memory, written there by a kernel (k_ctl_out) so that
  // reading them never queues behind a large copy on a copy engine (vxg_read_positions_async)
  int* h_ctl = nullptr;
  int* h_ctl_dev = nullptr;
  // kernels launched by the time step (a graph replay counts the kernels it holds)
  long long n_launch = 0, graph_kernels = 0, cgraph_kernels = 0;
  // FP64 branch decisions (vxg_set_decisions): 0 off, 1 record, 2 replay; one byte per voxel per
  // step for dec_cap steps; dec_step is the next step's row
  int dec_mode = 0;
  uint8_t* d_dec = nullptr;
  long long dec_cap = 0, dec_step = 0;
  // per-step actuation (vxg_set_actuation)
  int act_mode = 0;
  double act_amp = 0, act_freq = 0;
  float* d_phase = nullptr;
  int n_phase = 0;
  // deformed mesh (vxg_mesh_topology / vxg_mesh_update)
  int* d_mesh_vv = nullptr;     // 8 voxels per vertex
  int* d_mesh_quads = nullptr;  // 4 vertices per quad
  float* d_mesh_vert = nullptr;
  float* d_mesh_norm = nullptr;
  int n_mesh_vert = 0, n_mesh_quad = 0;
  // sparse temperature edits (vxg_set_temperatures_sparse)
  int* d_sp_idx = nullptr;
  float* d_sp_t = nullptr;
  int n_sp_cap = 0;
  // scratch of the body centre-of-mass reduction
  int* d_body_off = nullptr;
  double* d_body_out = nullptr;
  int n_body_cap = 0;
  // device snapshots of the full state
  struct Snap {
    char* p[4] = {nullptr, nullptr, nullptr, nullptr};
    size_t n[4] = {0, 0, 0, 0};
    int nv = -1, nl = -1, precision = -1;
  };
  std::vector<Snap> snaps;
};

static int fail(vxg_engine* e, int code, const char* what, cudaError_t ce = cudaSuccess) {
  if (e) {
    e->err = what;
    if (ce != cudaSuccess) {
      e->err += ": ";
      e->err += cudaGetErrorString(ce);
    }
  }
  return code;
}
#define VXG_CK(call)                                                     \
  do {                                                                   \
    cudaError_t _c = (call);                                             \
    if (_c != cudaSuccess) return fail(e, VXG_E_CUDA, #call, _c);        \
  } while (0)

static void release_arena(vxg_engine* e) {
  if (e->d_body_cols) cudaFree(e->d_body_cols);
  if (e->d_body_bak) cudaFree(e->d_body_bak);
  e->d_body_cols = nullptr;
  e->d_body_bak = nullptr;
  e->body_cols.clear();
  if (e->arena) cudaFree(e->arena);
  if (e->arena32) cudaFree(e->arena32);
  e->arena32 = nullptr;
  e->arena = nullptr;
  e->arena_bytes = 0;
  std::memset(e->field_ptr, 0, sizeof(e->field_ptr));
}

static void rebuild_view(vxg_engine* e) {
  View& S = e->S;
  S.nv = e->nv;
  S.nl = e->nl;
  auto P = [&](int f) { return e->field_ptr[f]; };
  S.vmat = (const int*)P(VXG_F_VOXEL_MATERIAL);
  S.vidx = (const int*)P(VXG_F_VOXEL_INDEX);
  S.vlinks = (const int*)P(VXG_F_VOXEL_LINKS);
  S.vext = (const int*)P(VXG_F_VOXEL_EXTERNAL);
  S.vflags = (uint32_t*)P(VXG_F_VOXEL_FLAGS);
  S.pos = (double*)P(VXG_F_POS);
  S.linMom = (double*)P(VXG_F_LINMOM);
  S.orient = (double*)P(VXG_F_ORIENT);
  S.angMom = (double*)P(VXG_F_ANGMOM);
  S.temp = (float*)P(VXG_F_TEMP);
  S.prevDt = (float*)P(VXG_F_PREV_DT);
  S.pStrain = (float*)P(VXG_F_PSTRAIN);
  S.lvox = (const int*)P(VXG_F_LINK_VOXELS);
  S.lmat = (const int*)P(VXG_F_LINK_MATERIAL);
  S.lflags = (uint32_t*)P(VXG_F_LINK_FLAGS);
  S.pos2 = (double*)P(VXG_F_POS2);
  S.a1v = (double*)P(VXG_F_ANGLE1V);
  S.a2v = (double*)P(VXG_F_ANGLE2V);
  S.fN = (double*)P(VXG_F_FORCE_NEG);
  S.fP = (double*)P(VXG_F_FORCE_POS);
  S.mN = (double*)P(VXG_F_MOMENT_NEG);
  S.mP = (double*)P(VXG_F_MOMENT_POS);
  S.rest = (double*)P(VXG_F_REST_LENGTH);
  S.strain = (float*)P(VXG_F_STRAIN);
  S.maxStrain = (float*)P(VXG_F_MAX_STRAIN);
  S.strainOffset = (float*)P(VXG_F_STRAIN_OFFSET);
  S.stress = (float*)P(VXG_F_STRESS);
  S.strainRatio = (float*)P(VXG_F_STRAIN_RATIO);
  S.tArea = (float*)P(VXG_F_TRANSVERSE_AREA);
  S.tSS = (float*)P(VXG_F_TRANSVERSE_STRAIN_SUM);
  S.vm = e->d_vm;
  S.lm = e->d_lm;
  S.ext = e->d_ext;
  S.powtab = e->d_powtab;
  S.ctl = e->ctl;
  e->col.bind(S);
  e->V.B = S;
  e->V.s = (float)e->g.voxSize;
  if (e->precision == VXG_FP32C) e->col.bind32(e->V);
  e->graph_valid = false;
  e->topo_ok = false;
  e->groups_valid = false;
}

static bool is_state_field(int f) {
  return f == VXG_F_POS || f == VXG_F_LINMOM || f == VXG_F_ORIENT || f == VXG_F_ANGMOM || f == VXG_F_PREV_DT ||
         f == VXG_F_POS2 || f == VXG_F_ANGLE1V || f == VXG_F_ANGLE2V || f == VXG_F_FORCE_NEG ||
         f == VXG_F_FORCE_POS || f == VXG_F_MOMENT_NEG || f == VXG_F_MOMENT_POS || f == VXG_F_REST_LENGTH;
}
static uint32_t all_state_bits() {
  uint32_t m = 0;
  for (int f = 0; f < VXG_F_COUNT; ++f)
    if (is_state_field(f)) m |= 1u << f;
  return m;
}
static void conv(vxg_engine* e, int f, int to32) {
  int n = std::max(e->nv, e->nl);
  if (n) k_conv<<<grid_for(n), kBlock, 0, e->stream>>>(e->V, e->g.voxSize, f, to32);
}
// FP32C: convert the fields the host wrote before the FP32 state is used
static void ensure32(vxg_engine* e) {
  if (e->precision != VXG_FP32C) return;
  for (int f = 0; f < VXG_F_COUNT; ++f)
    if (e->dirty64 & (1u << f)) conv(e, f, 1);
  e->dirty64 = 0;
}
// FP32C: the rest lengths of temperatures the host set, before anything reads or copies them
static void flush_rest(vxg_engine* e) {
  if (!e->rest_pending) return;
  if (e->nl) k_rest32<<<grid_for(e->nl), kBlock, 0, e->stream>>>(e->V);
  e->rest_pending = false;
}
// FP32C: refresh the FP64 copy of one field (or all with f < 0) before it is read
static void ensure64(vxg_engine* e, int f = -1) {
  if (e->precision != VXG_FP32C) return;
  uint32_t want = f < 0 ? e->stale64 : (e->stale64 & (1u << f));
  if (want & (1u << VXG_F_REST_LENGTH)) flush_rest(e);
  for (int k = 0; k < VXG_F_COUNT; ++k)
    if (want & (1u << k)) conv(e, k, 0);
  e->stale64 &= ~want;
}

// *cap is the allocated capacity, *live the entries in use (what k_validate checks indices against)
// FP32C: refresh only the FP64 fields that info_value reads for stateInfo quantity `info`
// (stress and strain are shared by both precisions; MASS reads the material table only)
static void ensure64_info(vxg_engine* e, int info) {
  switch (info) {
    case 0: ensure64(e, VXG_F_POS); break;
    case 1: ensure64(e, VXG_F_LINMOM); break;
    case 2: ensure64(e, VXG_F_LINMOM); ensure64(e, VXG_F_ANGMOM); break;
    case 3: ensure64(e, VXG_F_ORIENT); break;
    case 4: ensure64(e, VXG_F_ANGMOM); break;
    case 7: ensure64(e, VXG_F_FORCE_NEG); ensure64(e, VXG_F_MOMENT_NEG); ensure64(e, VXG_F_MOMENT_POS); break;
    default: break;
  }
}

template <class T>
static int upload_table(vxg_engine* e, T** dptr, int* cap, int* live, const T* src, int n) {
  if (n > *cap || !*dptr) {
    if (*dptr) cudaFree(*dptr);
    *dptr = nullptr;
    *cap = 0;
    cudaError_t c = cudaMalloc(dptr, sizeof(T) * (size_t)std::max(n, 1));
    if (c != cudaSuccess) return fail(e, VXG_E_CUDA, "table alloc", c);
    *cap = std::max(n, 1);
  }
  if (*live != n) e->topo_ok = false;  // indices must be checked against the new count
  *live = n;
  if (n) {
    cudaError_t c = cudaMemcpyAsync(*dptr, src, sizeof(T) * (size_t)n, cudaMemcpyHostToDevice, e->stream);
    if (c != cudaSuccess) return fail(e, VXG_E_CUDA, "table copy", c);
  }
  return VXG_OK;
}

// ---- fixed-scratch set-up: one device address per device, looked up once -------------------
namespace {
std::mutex g_fixed_mu;
constexpr int kFixedMaxDevices = 64;
double* g_fixed_addr[kFixedMaxDevices] = {};
}  // namespace

// Same quantity as vxg_reduce, written to d_out (device memory) on the engine's stream, through
// the fixed scratch above: no device or host memory is allocated, nothing is synchronised.  The
// first call on a device looks the scratch up with cudaGetSymbolAddress, which may load this
// library's device code and so allocate inside the CUDA runtime: make that first call before any
// stream capture.  All calls on one device share the scratch: calls that overlap in time (several
// host threads or streams, several engines on one device) race and must be serialised by the
// caller.  Errors return a code and a static message in *why; nothing is written to d_out then.
__attribute__((visibility("hidden"))) int vxg_reduce_fixed(vxg_engine* e, int info, int type, float* d_out,
                                                          const char** why) {
  const char* dummy = nullptr;
  if (!why) why = &dummy;
  *why = nullptr;
  if (!e || !d_out || info < 0 || info > 9 || type < 0 || type > 3) {
    *why = "vx_state_info_into: bad engine, output pointer, info or type";
    return VXG_E_ARG;
  }
  if (info == 8) {
    *why = "vx_state_info_into: PRESSURE is reduced on the host";
    return VXG_E_ARG;
  }
  if (!e->topo_ok) {  // checking the index fields would allocate: a step checks them
    *why = "vx_state_info_into: the scene's indices are not checked yet (step first)";
    return VXG_E_STATE;
  }
  const bool link = info == 5 || info == 6 || info == 7;
  const long long n = link ? e->nl : e->nv;
  if (n > kFixedMaxElements) {
    *why = "vx_state_info_into: more elements than the fixed scratch covers (at most 4,194,304 voxels or links)";
    return VXG_E_SIZE;
  }
  if (e->device < 0 || e->device >= kFixedMaxDevices) {
    *why = "vx_state_info_into: the engine's device number is beyond the fixed scratch's device table";
    return VXG_E_ARG;
  }
  // the engine's device is made current for the call and the caller's device is put back after it
  int prev = -1;
  if (cudaGetDevice(&prev) != cudaSuccess || cudaSetDevice(e->device) != cudaSuccess) {
    *why = "vx_state_info_into: cannot make the engine's device current";
    return VXG_E_CUDA;
  }
  struct RestoreDevice {
    int d;
    ~RestoreDevice() { if (d >= 0) cudaSetDevice(d); }
  } restore{prev};
  double* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_fixed_mu);
    if (!g_fixed_addr[e->device]) {
      void* p = nullptr;
      cudaError_t c = cudaGetSymbolAddress(&p, g_fixed_scratch);  // with e->device current
      if (c != cudaSuccess || !p) {
        *why = "vx_state_info_into: cudaGetSymbolAddress of the fixed scratch failed";
        return VXG_E_CUDA;
      }
      g_fixed_addr[e->device] = static_cast<double*>(p);
    }
    scratch = g_fixed_addr[e->device];
  }
  if (n == 0) {
    if (cudaMemsetAsync(d_out, 0, sizeof(float), e->stream) != cudaSuccess) {
      *why = "vx_state_info_into: cudaMemsetAsync failed";
      return VXG_E_CUDA;
    }
    return VXG_OK;
  }
  ensure64_info(e, info);  // FP32C: kernels that convert only the fields this quantity reads
  // cudaLaunchKernel reports this launch's own error; an error left pending by an unrelated earlier
  // call is neither returned nor cleared
  View S = e->S;
  int n_arg = (int)n;
  void* args[] = {&S, &info, &n_arg, &type, &scratch, &d_out};
  const int blocks = (int)((n + kFixedSpan - 1) / kFixedSpan);
  if (cudaLaunchKernel((const void*)k_reduce_fixed, dim3(blocks), dim3(kBlock), args, 0, e->stream) != cudaSuccess) {
    *why = "vx_state_info_into: kernel launch failed";
    return VXG_E_CUDA;
  }
  return VXG_OK;
}

extern "C" {

int vxg_create(vxg_engine** out, int device, int precision) {
  if (!out) return VXG_E_ARG;
  *out = nullptr;
  if (precision != VXG_FP64 && precision != VXG_FP32C) return VXG_E_ARG;
  vxg_engine* e = new vxg_engine();
  e->device = device;
  e->precision = precision;
  // FP32C link pass: 128-thread blocks measured ~2 % faster than 256 on GB300 (vxg_autotune
  // compares all shapes)
  if (precision == VXG_FP32C) e->blk_link = 128;
  cudaError_t c = cudaSetDevice(device);
  if (c != cudaSuccess) { delete e; return VXG_E_CUDA; }
  c = cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking);
  if (c == cudaSuccess) c = cudaMalloc(&e->ctl, sizeof(Ctl));
  if (c == cudaSuccess) c = cudaMemset(e->ctl, 0, sizeof(Ctl));
  if (c == cudaSuccess) c = cudaMalloc(&e->d_partials, sizeof(double) * 3 * 4096);
  for (int i = 0; i < 4 && c == cudaSuccess; ++i) c = cudaEventCreate(&e->ev[i]);
  if (c != cudaSuccess) { vxg_destroy(e); return VXG_E_CUDA; }
  *out = e;
  return VXG_OK;
}

int vxg_destroy(vxg_engine* e) {
  if (!e) return VXG_OK;
  cudaSetDevice(e->device);
  if (e->stream) cudaStreamSynchronize(e->stream);
  if (e->graph) cudaGraphExecDestroy(e->graph);
  if (e->cgraph) cudaGraphExecDestroy(e->cgraph);
  for (cudaGraphExec_t g : e->g1)
    if (g) cudaGraphExecDestroy(g);
  if (e->d_phase) cudaFree(e->d_phase);
  if (e->d_body_off) cudaFree(e->d_body_off);
  if (e->d_body_out) cudaFree(e->d_body_out);
  if (e->d_groups) cudaFree(e->d_groups);
  if (e->d_bctl) cudaFree(e->d_bctl);
  for (auto& sl : e->snaps)
    for (char* p : sl.p) if (p) cudaFree(p);
  release_arena(e);
  e->col.release();
  if (e->ctl) cudaFree(e->ctl);
  if (e->d_vm) cudaFree(e->d_vm);
  if (e->d_lm) cudaFree(e->d_lm);
  if (e->d_ext) cudaFree(e->d_ext);
  if (e->d_powtab) cudaFree(e->d_powtab);
  if (e->d_sp_idx) cudaFree(e->d_sp_idx);
  if (e->d_sp_t) cudaFree(e->d_sp_t);
  if (e->d_dec) cudaFree(e->d_dec);
  if (e->d_bad) cudaFree(e->d_bad);
  for (void* p : {(void*)e->d_mesh_vv, (void*)e->d_mesh_quads, (void*)e->d_mesh_vert, (void*)e->d_mesh_norm})
    if (p) cudaFree(p);
  if (e->d_partials) cudaFree(e->d_partials);
  for (int i = 0; i < 4; ++i)
    if (e->ev[i]) cudaEventDestroy(e->ev[i]);
  for (cudaEvent_t x : e->tev) cudaEventDestroy(x);
  for (cudaEvent_t x : e->bev) if (x) cudaEventDestroy(x);
  if (e->h_ctl) cudaFreeHost(e->h_ctl);
  if (e->cstream) {
    cudaStreamSynchronize(e->cstream);
    cudaStreamDestroy(e->cstream);
  }
  for (int k = 0; k < 2; ++k) {
    if (e->d_stage[k]) cudaFree(e->d_stage[k]);
    if (e->ev_staged[k]) cudaEventDestroy(e->ev_staged[k]);
    if (e->ev_copied[k]) cudaEventDestroy(e->ev_copied[k]);
  }
  if (e->stream) cudaStreamDestroy(e->stream);
  delete e;
  return VXG_OK;
}

int vxg_precision(const vxg_engine* e) { return e ? e->precision : VXG_E_ARG; }

int vxg_resize(vxg_engine* e, int nv, int nl) {
  if (!e || nv < 0 || nl < 0) return VXG_E_ARG;
  VXG_CK(cudaSetDevice(e->device));
  VXG_CK(cudaStreamSynchronize(e->stream));
  release_arena(e);
  e->rest_pending = false;
  // decision rows are sized by the voxel count: a new scene starts without them
  if (e->d_dec) cudaFree(e->d_dec);
  e->d_dec = nullptr;
  e->dec_cap = e->dec_step = 0;
  e->dec_mode = 0;
  e->nv = nv;
  e->nl = nl;
  size_t off[VXG_F_COUNT] = {};
  size_t total = 0;
  for (int f = 0; f < VXG_F_TIME; ++f) {
    FieldDesc d = field_desc(f);
    size_t n = (size_t)d.comps * (d.per_link ? nl : nv);
    off[f] = total;
    total += ((n * d.elem + 255) / 256) * 256;
  }
  if (total == 0) total = 256;
  VXG_CK(cudaMalloc(&e->arena, total));
  VXG_CK(cudaMemsetAsync(e->arena, 0, total, e->stream));
  e->arena_bytes = total;
  for (int f = 0; f < VXG_F_TIME; ++f) e->field_ptr[f] = e->arena + off[f];
  if (e->precision == VXG_FP32C) {
    size_t vb = ((sizeof(float) * 21 * (size_t)nv + 255) / 256) * 256;
    size_t lb = ((sizeof(float) * 23 * (size_t)nl + 255) / 256) * 256;
    e->arena32_bytes = std::max<size_t>(vb + lb, 256);
    VXG_CK(cudaMalloc(&e->arena32, e->arena32_bytes));
    VXG_CK(cudaMemsetAsync(e->arena32, 0, vb + lb, e->stream));
    float* p = (float*)e->arena32;
    // float4 records first (16-byte aligned), then the per-component arrays
    e->V.P = (float4*)p; e->V.Q = (float4*)(p + 4 * (size_t)nv); e->V.c = p + 8 * (size_t)nv;
    e->V.qc = p + 11 * (size_t)nv; e->V.lin = p + 15 * (size_t)nv; e->V.ang = p + 18 * (size_t)nv;
    float* L = (float*)(e->arena32 + vb);
    e->V.pos2 = L; e->V.a1v = L + 3 * (size_t)nl; e->V.a2v = L + 6 * (size_t)nl; e->V.fN = L + 9 * (size_t)nl;
    e->V.fP = L + 12 * (size_t)nl; e->V.mN = L + 15 * (size_t)nl; e->V.mP = L + 18 * (size_t)nl;
    e->V.restDelta = L + 21 * (size_t)nl;
    e->V.large = (int*)(L + 22 * (size_t)nl);
  }
  int rc = e->col.resize(nv);
  if (rc) return fail(e, rc, "collision buffers");
  VXG_CK(cudaMemsetAsync(e->ctl, 0, sizeof(Ctl), e->stream));
  rebuild_view(e);
  VXG_CK(cudaStreamSynchronize(e->stream));
  return VXG_OK;
}

int vxg_set_field(vxg_engine* e, int f, const void* host, long long count) {
  if (!e || !host || f < 0 || f >= VXG_F_COUNT) return VXG_E_ARG;
  VXG_CK(cudaSetDevice(e->device));
  if (f == VXG_F_TIME) {
    if (count != 1) return VXG_E_SIZE;
    VXG_CK(cudaMemcpyAsync(&e->ctl->time, host, 4, cudaMemcpyHostToDevice, e->stream));
    VXG_CK(cudaStreamSynchronize(e->stream));
    return VXG_OK;
  }
  FieldDesc d = field_desc(f);
  long long n = (long long)d.comps * (d.per_link ? e->nl : e->nv);
  if (count != n) return fail(e, VXG_E_SIZE, "vxg_set_field: element count mismatch");
  if (n == 0) return VXG_OK;
  if (f == VXG_F_REST_LENGTH) e->rest_pending = false;  // the host's rest lengths win
  else flush_rest(e);  // from the temperatures as they were set, before any field changes
  e->poisson_redo = true;
  if (f == VXG_F_VOXEL_MATERIAL || f == VXG_F_VOXEL_LINKS || f == VXG_F_VOXEL_EXTERNAL ||
      f == VXG_F_LINK_VOXELS || f == VXG_F_LINK_MATERIAL)
    e->topo_ok = e->groups_valid = false;
  if (e->precision == VXG_FP32C && is_state_field(f)) {
    e->dirty64 |= 1u << f;   // the FP64 copy is now the newer one
    e->stale64 &= ~(1u << f);
  }
  VXG_CK(cudaMemcpyAsync(e->field_ptr[f], host, (size_t)n * d.elem, cudaMemcpyHostToDevice, e->stream));
  VXG_CK(cudaStreamSynchronize(e->stream));
  return VXG_OK;
}

int vxg_get_field(vxg_engine* e, int f, void* host, long long count) {
  if (!e || !host || f < 0 || f >= VXG_F_COUNT) return VXG_E_ARG;
  VXG_CK(cudaSetDevice(e->device));
  if (f == VXG_F_TIME) {
    if (count != 1) return VXG_E_SIZE;
    VXG_CK(cudaMemcpyAsync(host, &e->ctl->time, 4, cudaMemcpyDeviceToHost, e->stream));
    VXG_CK(cudaStreamSynchronize(e->stream));
    return VXG_OK;
  }
  FieldDesc d = field_desc(f);
  long long n = (long long)d.comps * (d.per_link ? e->nl : e->nv);
  if (count != n) return fail(e, VXG_E_SIZE, "vxg_get_field: element count mismatch");
  if (n == 0) return VXG_OK;
  if (f == VXG_F_POS && e->precision == VXG_FP32C && (e->stale64 & (1u << VXG_F_POS))) {
    // positions the device can write directly (pinned host memory): convert into them in one pass
    cudaPointerAttributes pa;
    if (cudaPointerGetAttributes(&pa, host) == cudaSuccess && pa.type == cudaMemoryTypeHost && pa.devicePointer) {
      ensure32(e);
      k_pos_out<<<grid_for(e->nv), kBlock, 0, e->stream>>>(e->V, e->g.voxSize, (double*)pa.devicePointer);
      VXG_CK(cudaGetLastError());
      VXG_CK(cudaStreamSynchronize(e->stream));
      return VXG_OK;
    }
    cudaGetLastError();  // not a registered pointer: the staged path below
  }
  if (is_state_field(f)) ensure64(e, f);
  VXG_CK(cudaMemcpyAsync(host, e->field_ptr[f], (size_t)n * d.elem, cudaMemcpyDeviceToHost, e->stream));
  VXG_CK(cudaStreamSynchronize(e->stream));
  return VXG_OK;
}

int vxg_read_positions_async(vxg_engine* e, double* host) {
  if (!e || (!host && e->nv)) return VXG_E_ARG;
  if (!e->nv) return VXG_OK;
  VXG_CK(cudaSetDevice(e->device));
  const size_t bytes = sizeof(double) * 3 * (size_t)e->nv;
  if (!e->cstream) {
    VXG_CK(cudaStreamCreateWithFlags(&e->cstream, cudaStreamNonBlocking));
    for (int k = 0; k < 2; ++k) {
      VXG_CK(cudaEventCreateWithFlags(&e->ev_staged[k], cudaEventDisableTiming));
      VXG_CK(cudaEventCreateWithFlags(&e->ev_copied[k], cudaEventDisableTiming));
    }
  }
  if (e->stage_bytes != bytes) {  // first use, or the scene changed size: copies in flight end first
    VXG_CK(cudaStreamSynchronize(e->cstream));
    for (int k = 0; k < 2; ++k) {
      if (e->d_stage[k]) cudaFree(e->d_stage[k]);
      e->d_stage[k] = nullptr;
      e->stage_used[k] = false;
    }
    e->stage_bytes = 0;
    for (int k = 0; k < 2; ++k) VXG_CK(cudaMalloc(&e->d_stage[k], bytes));
    e->stage_bytes = bytes;
  }
  const int k = e->stage_next;
  e->stage_next ^= 1;
  if (e->stage_used[k]) VXG_CK(cudaStreamWaitEvent(e->stream, e->ev_copied[k], 0));
  if (e->precision == VXG_FP32C && (e->stale64 & (1u << VXG_F_POS))) {
    ensure32(e);
    k_pos_out<<<grid_for(e->nv), kBlock, 0, e->stream>>>(e->V, e->g.voxSize, e->d_stage[k]);
    VXG_CK(cudaGetLastError());
  } else {
    VXG_CK(cudaMemcpyAsync(e->d_stage[k], e->field_ptr[VXG_F_POS], bytes, cudaMemcpyDeviceToDevice, e->stream));
  }
  VXG_CK(cudaEventRecord(e->ev_staged[k], e->stream));
  VXG_CK(cudaStreamWaitEvent(e->cstream, e->ev_staged[k], 0));
  VXG_CK(cudaMemcpyAsync(host, e->d_stage[k], bytes, cudaMemcpyDeviceToHost, e->cstream));
  VXG_CK(cudaEventRecord(e->ev_copied[k], e->cstream));
  e->stage_used[k] = true;
  return VXG_OK;
}

int vxg_read_wait(vxg_engine* e) {
  if (!e) return VXG_E_ARG;
  if (!e->cstream) return VXG_OK;
  VXG_CK(cudaSetDevice(e->device));
  VXG_CK(cudaStreamSynchronize(e->cstream));
  return VXG_OK;
}

int vxg_set_tables(vxg_engine* e, const vxg_voxel_material* vm, int n_vm, const vxg_link_material* lm, int n_lm,
                   const vxg_external* ext, int n_ext) {
  if (!e || n_vm < 0 || n_lm < 0 || n_ext < 0) return VXG_E_ARG;
  VXG_CK(cudaSetDevice(e->device));
  int rc;
  if ((rc = upload_table(e, &e->d_vm, &e->cap_vm, &e->n_vm, vm, n_vm))) return rc;
  if ((rc = upload_table(e, &e->d_lm, &e->cap_lm, &e->n_lm, lm, n_lm))) return rc;
  if ((rc = upload_table(e, &e->d_ext, &e->cap_ext, &e->n_ext, ext, n_ext))) return rc;
  e->poisson_redo = true;
  e->tab_poisson = false;
  for (int k = 0; k < n_vm; ++k)
    if (vm[k].nu != 0.0f) e->tab_poisson = true;
  e->adj_scope = nullptr;
  for (int k = 0; k < n_lm && !e->adj_scope; ++k)
    if (!lm[k].linear) e->adj_scope = "a link material is not linear";
  // one Poisson's ratio for every voxel material: a link's ratio then depends on no Young's modulus
  // (CVX_MaterialLink combines the two eHat)
  for (int k = 1; k < n_vm && !e->adj_scope; ++k)
    if (vm[k].nu != vm[0].nu) e->adj_scope = "voxel materials with different Poisson's ratios";
  VXG_CK(cudaStreamSynchronize(e->stream));
  rebuild_view(e);
  return VXG_OK;
}

int vxg_set_externals(vxg_engine* e, const vxg_external* ext, int n_ext) {
  if (!e || n_ext < 0 || (n_ext && !ext)) return VXG_E_ARG;
  VXG_CK(cudaSetDevice(e->device));
  vxg_external* before = e->d_ext;
  int rc = upload_table(e, &e->d_ext, &e->cap_ext, &e->n_ext, ext, n_ext);
  if (rc) return rc;
  VXG_CK(cudaStreamSynchronize(e->stream));
  e->poisson_redo = true;        // tension terms of the Poisson strain read the externals
  if (e->d_ext != before) rebuild_view(e);  // captured graphs hold the table's address
  return VXG_OK;
}

int vxg_set_temperatures_sparse(vxg_engine* e, int n, const int* voxels, const float* temps) {
  if (!e || n < 0 || (n && (!voxels || !temps))) return VXG_E_ARG;
  if (n == 0) return VXG_OK;
  for (int i = 0; i < n; ++i)
    if (voxels[i] < 0 || voxels[i] >= e->nv) return fail(e, VXG_E_ARG, "vxg_set_temperatures_sparse: voxel index out of range");
  VXG_CK(cudaSetDevice(e->device));
  flush_rest(e);  // the sparse update recomputes only the edited voxels' links
  if (n > e->n_sp_cap) {
    if (e->d_sp_idx) cudaFree(e->d_sp_idx);
    if (e->d_sp_t) cudaFree(e->d_sp_t);
    e->d_sp_idx = nullptr;
    e->d_sp_t = nullptr;
    e->n_sp_cap = 0;
    VXG_CK(cudaMalloc(&e->d_sp_idx, sizeof(int) * (size_t)n));
    VXG_CK(cudaMalloc(&e->d_sp_t, sizeof(float) * (size_t)n));
    e->n_sp_cap = n;
  }
  VXG_CK(cudaMemcpyAsync(e->d_sp_idx, voxels, sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, e->stream));
  VXG_CK(cudaMemcpyAsync(e->d_sp_t, temps, sizeof(float) * (size_t)n, cudaMemcpyHostToDevice, e->stream));
  k_temp_sparse<<<grid_for(n), kBlock, 0, e->stream>>>(e->S, n, e->d_sp_idx, e->d_sp_t);
  if (e->nl) {
    if (e->precision == VXG_FP32C) k_rest_sparse<true><<<grid_for(6 * n), kBlock, 0, e->stream>>>(e->V, n, e->d_sp_idx);
    else k_rest_sparse<false><<<grid_for(6 * n), kBlock, 0, e->stream>>>(e->V, n, e->d_sp_idx);
  }
  VXG_CK(cudaGetLastError());
  VXG_CK(cudaStreamSynchronize(e->stream));
  if (e->precision == VXG_FP32C) e->stale64 |= 1u << VXG_F_REST_LENGTH;  // FP64 copy is now behind
  return VXG_OK;
}

int vxg_mesh_topology(vxg_engine* e, int n_vertices, const int* vertex_voxels, int n_quads, const int* quads) {
  if (!e || n_vertices < 0 || n_quads < 0 || (n_vertices && !vertex_voxels) || (n_quads && !quads)) return VXG_E_ARG;
  for (long long i = 0; i < 8ll * n_vertices; ++i)
    if (vertex_voxels[i] < -1 || vertex_voxels[i] >= e->nv) return fail(e, VXG_E_ARG, "vxg_mesh_topology: voxel index out of range");
  for (long long i = 0; i < 4ll * n_quads; ++i)
    if (quads[i] < 0 || quads[i] >= n_vertices) return fail(e, VXG_E_ARG, "vxg_mesh_topology: vertex index out of range");
  for (int i = 0; i < n_vertices; ++i) {
    bool any = false;
    for (int j = 0; j < 8; ++j) any |= vertex_voxels[8 * i + j] >= 0;
    if (!any) return fail(e, VXG_E_ARG, "vxg_mesh_topology: a vertex belongs to no voxel");
  }
  VXG_CK(cudaSetDevice(e->device));
  for (void* p : {(void*)e->d_mesh_vv, (void*)e->d_mesh_quads, (void*)e->d_mesh_vert, (void*)e->d_mesh_norm})
    if (p) cudaFree(p);
  e->d_mesh_vv = e->d_mesh_quads = nullptr;
  e->d_mesh_vert = e->d_mesh_norm = nullptr;
  e->n_mesh_vert = e->n_mesh_quad = 0;
  VXG_CK(cudaMalloc(&e->d_mesh_vv, sizeof(int) * 8 * (size_t)std::max(n_vertices, 1)));
  VXG_CK(cudaMalloc(&e->d_mesh_vert, sizeof(float) * 3 * (size_t)std::max(n_vertices, 1)));
  VXG_CK(cudaMalloc(&e->d_mesh_quads, sizeof(int) * 4 * (size_t)std::max(n_quads, 1)));
  VXG_CK(cudaMalloc(&e->d_mesh_norm, sizeof(float) * 3 * (size_t)std::max(n_quads, 1)));
  if (n_vertices)
    VXG_CK(cudaMemcpyAsync(e->d_mesh_vv, vertex_voxels, sizeof(int) * 8 * (size_t)n_vertices, cudaMemcpyHostToDevice, e->stream));
  if (n_quads)
    VXG_CK(cudaMemcpyAsync(e->d_mesh_quads, quads, sizeof(int) * 4 * (size_t)n_quads, cudaMemcpyHostToDevice, e->stream));
  VXG_CK(cudaStreamSynchronize(e->stream));
  e->n_mesh_vert = n_vertices;
  e->n_mesh_quad = n_quads;
  return VXG_OK;
}

static int check_topology(vxg_engine* e);
// an NVTX range for the length of a scope (named in profiler timelines; free without a profiler)
struct NvtxScope {
  explicit NvtxScope(const char* name) { nvtxRangePushA(name); }
  ~NvtxScope() { nvtxRangePop(); }
};
int vxg_mesh_update(vxg_engine* e, float* vertices, float* normals) {
  NvtxScope nvtx("vxg_mesh_update");
  if (!e) return VXG_E_ARG;
  VXG_CK(cudaSetDevice(e->device));
  flush_rest(e);
  if (int rc = check_topology(e)) return rc;
  ensure32(e);  // FP32C: host-written state first
  const int nvt = e->n_mesh_vert, nq = e->n_mesh_quad;
  if (nvt) {
    k_mesh_vertices<<<grid_for(nvt), kBlock, 0, e->stream>>>(e->S, e->V, e->precision == VXG_FP32C ? 1 : 0,
                                                            e->g.voxSize, nvt, e->d_mesh_vv, e->d_mesh_vert);
    if (nq) k_mesh_normals<<<grid_for(nq), kBlock, 0, e->stream>>>(nq, e->d_mesh_quads, e->d_mesh_vert, e->d_mesh_norm);
    VXG_CK(cudaGetLastError());
    if (vertices)
      VXG_CK(cudaMemcpyAsync(vertices, e->d_mesh_vert, sizeof(float) * 3 * (size_t)nvt, cudaMemcpyDeviceToHost, e->stream));
    if (normals && nq)
      VXG_CK(cudaMemcpyAsync(normals, e->d_mesh_norm, sizeof(float) * 3 * (size_t)nq, cudaMemcpyDeviceToHost, e->stream));
  }
  VXG_CK(cudaStreamSynchronize(e->stream));
  return VXG_OK;
}

int vxg_mesh_device_buffers(vxg_engine* e, const float** vertices, const float** normals) {
  if (!e) return VXG_E_ARG;
  if (vertices) *vertices = e->d_mesh_vert;
  if (normals) *normals = e->d_mesh_norm;
  return VXG_OK;
}

int vxg_set_powf_table(vxg_engine* e, int slot, float /*exponent*/, const float* table) {
  if (!e || slot < 0 || slot > 63 || !table) return VXG_E_ARG;
  VXG_CK(cudaSetDevice(e->device));
  const size_t per = (size_t)1 << 24;
  if (slot >= e->n_powslots) {
    float* np = nullptr;
    int ns = slot + 1;
    VXG_CK(cudaMalloc(&np, per * sizeof(float) * ns));
    if (e->d_powtab) {
      VXG_CK(cudaMemcpyAsync(np, e->d_powtab, per * sizeof(float) * e->n_powslots, cudaMemcpyDeviceToDevice, e->stream));
      VXG_CK(cudaStreamSynchronize(e->stream));
      cudaFree(e->d_powtab);
    }
    e->d_powtab = np;
    e->n_powslots = ns;
  }
  e->poisson_redo = true;
  VXG_CK(cudaMemcpyAsync(e->d_powtab + per * slot, table, per * sizeof(float), cudaMemcpyHostToDevice, e->stream));
  VXG_CK(cudaStreamSynchronize(e->stream));
  rebuild_view(e);
  return VXG_OK;
}

int vxg_set_globals(vxg_engine* e, const vxg_globals* g) {
  if (!e || !g) return VXG_E_ARG;
  e->g = *g;
  e->have_globals = true;
  e->V.s = (float)g->voxSize;
  e->graph_valid = false;
  return VXG_OK;
}

int vxg_set_nearby(vxg_engine* e, const int* offsets, const int* items, long long n_items) {
  if (!e || !offsets || (n_items > 0 && !items)) return VXG_E_ARG;
  if (offsets[0] != 0 || offsets[e->nv] != n_items) return fail(e, VXG_E_ARG, "vxg_set_nearby: offsets do not span the items");
  for (int v = 0; v < e->nv; ++v)
    if (offsets[v + 1] < offsets[v]) return fail(e, VXG_E_ARG, "vxg_set_nearby: offsets decrease");
  for (long long k = 0; k < n_items; ++k)
    if (items[k] < 0 || items[k] >= e->nv) return fail(e, VXG_E_ARG, "vxg_set_nearby: voxel index out of range");
  VXG_CK(cudaSetDevice(e->device));
  int rc = e->col.set_nearby(e->nv, offsets, items, n_items, e->stream);
  if (rc) return fail(e, rc, "nearby upload");
  rebuild_view(e);
  return VXG_OK;
}

// blocks of the pipelined link kernel resident on the whole GPU (occupancy queried once)
static int split_grid(vxg_engine* e, bool pois) {
  if (!e->lL_grid) {
    if (!e->n_sm) cudaDeviceGetAttribute(&e->n_sm, cudaDevAttrMultiProcessorCount, e->device);
    int nb = 0;
    if (pois) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_link32L<true>, 256, 0);
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_link32L<false>, 256, 0);
    e->lL_grid = std::max(1, e->n_sm) * std::max(1, nb);
  }
  return e->lL_grid;
}
static int lp_resident(vxg_engine* e, bool pois) {
  int& fit = e->lp_fit[pois ? 1 : 0];
  if (!fit) {
    if (!e->n_sm) cudaDeviceGetAttribute(&e->n_sm, cudaDevAttrMultiProcessorCount, e->device);
    int nb = 0;
    if (pois) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_link32p<true>, kLpT, kLpSmem);
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_link32p<false>, kLpT, kLpSmem);
    fit = std::max(1, nb);
  }
  int bps = e->lp_bps > 0 ? std::min(e->lp_bps, fit) : fit;
  return std::max(1, e->n_sm) * bps;
}

// a timing event between two passes; inside a stream capture it becomes an event-record node of
// the graph, so the GPU records it between the kernels with no host in between
static void pass_event(cudaEvent_t ev, cudaStream_t s) {
  cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
  cudaStreamIsCapturing(s, &st);
  if (st == cudaStreamCaptureStatusActive) cudaEventRecordWithFlags(ev, s, cudaEventRecordExternal);
  else cudaEventRecord(ev, s);
}

static bool fused_poisson(const vxg_engine* e) {
  return e->precision == VXG_FP32C && e->tab_poisson && e->poisson_fuse;
}
// FP32C at a fixed dt with the default one-kernel link pass and no Poisson pre-pass: the link pass
// can recompute the rest lengths from the temperatures itself (k_link32<..., ACT = true>)
static bool link_recomputes_rest(const vxg_engine* e, bool rec) {
  return e->precision == VXG_FP32C && e->nl && !rec && e->lp_bps == 0 && !e->link_split &&
         !(e->g.any_poisson && !fused_poisson(e));
}
// ---- body batches: groups, eligibility ---------------------------------------------------------
typedef void (*BodiesKernel)(vx32::View, float, int, const int4*, int, int*, float, float, const float*, int*,
                             const BodyCol*, int);
static BodiesKernel bodies_kernel(const vxg_engine* e) {
  const bool pois = e->tab_poisson, fuse = fused_poisson(e), act = e->act_mode != 0;
  if (act) {
    if (pois) return fuse ? k_bodies32<true, true, true> : k_bodies32<true, false, true>;
    return fuse ? k_bodies32<false, true, true> : k_bodies32<false, false, true>;
  }
  if (pois) return fuse ? k_bodies32<true, true, false> : k_bodies32<true, false, false>;
  return fuse ? k_bodies32<false, true, false> : k_bodies32<false, false, false>;
}
// The groups of the current topology: cut the voxel order wherever no link spans the cut (a
// difference array over each link's end indices), give each link the segment of its ends, and
// pack consecutive segments into groups of up to body_target voxels (a larger segment is a group
// of its own).  Needs the links ordered by segment, as a scene built body after body has them;
// otherwise no groups (n_groups 0) and batches run as passes.  Groups are listed largest first,
// the order the CTAs take them in.
static int build_groups(vxg_engine* e) {
  if (e->groups_valid && e->groups_target == e->body_target) return VXG_OK;
  e->n_groups = 0;
  e->groups_valid = true;
  e->groups_target = e->body_target;
  const int nv = e->nv, nl = e->nl;
  if (nv < 2 || nl < 1 || e->body_target <= 0) return VXG_OK;
  std::vector<int> lv((size_t)2 * nl);
  VXG_CK(cudaMemcpyAsync(lv.data(), e->S.lvox, sizeof(int) * 2 * (size_t)nl, cudaMemcpyDeviceToHost, e->stream));
  VXG_CK(cudaStreamSynchronize(e->stream));
  std::vector<int> cover((size_t)nv + 1, 0);
  for (int l = 0; l < nl; ++l) {
    const int a = std::min(lv[l], lv[(size_t)nl + l]), b = std::max(lv[l], lv[(size_t)nl + l]);
    if (a < 0 || b >= nv) return VXG_OK;  // validated before any step; never here
    cover[a] += 1;
    cover[b] -= 1;
  }
  std::vector<int> seg(nv), vstart(1, 0);
  int run = 0;
  for (int v = 0; v < nv; ++v) {
    seg[v] = (int)vstart.size() - 1;
    run += cover[v];
    if (run == 0 && v + 1 < nv) vstart.push_back(v + 1);
  }
  vstart.push_back(nv);
  const int nseg = (int)vstart.size() - 1;
  std::vector<int> lstart((size_t)nseg + 1, 0);
  for (int l = 0, prev = 0; l < nl; ++l) {
    const int sg = seg[lv[l]];
    if (sg < prev) return VXG_OK;  // links not in segment order
    prev = sg;
    lstart[sg + 1] += 1;
  }
  for (int k = 0; k < nseg; ++k) lstart[k + 1] += lstart[k];
  std::vector<int4> gr;
  int4 cur = make_int4(0, 0, 0, 0);
  for (int k = 0; k < nseg; ++k) {
    const int n = vstart[k + 1] - vstart[k];
    if (cur.y > cur.x && cur.y - cur.x + n > e->body_target) {
      gr.push_back(cur);
      cur = make_int4(vstart[k], vstart[k], lstart[k], lstart[k]);
    }
    cur.y = vstart[k + 1];
    cur.w = lstart[k + 1];
  }
  gr.push_back(cur);
  std::stable_sort(gr.begin(), gr.end(), [](const int4& p, const int4& q) {
    return (p.y - p.x) + (p.w - p.z) > (q.y - q.x) + (q.w - q.z);
  });
  if ((int)gr.size() > e->n_groups_cap) {
    if (e->d_groups) cudaFree(e->d_groups);
    e->d_groups = nullptr;
    e->n_groups_cap = 0;
    VXG_CK(cudaMalloc(&e->d_groups, sizeof(int4) * gr.size()));
    e->n_groups_cap = (int)gr.size();
  }
  if (!e->d_bctl) {
    VXG_CK(cudaMalloc(&e->d_bctl, 2 * sizeof(int)));
    const int init[2] = {0, INT_MAX};
    VXG_CK(cudaMemcpy(e->d_bctl, init, sizeof(init), cudaMemcpyHostToDevice));
  }
  VXG_CK(cudaMemcpy(e->d_groups, gr.data(), sizeof(int4) * gr.size(), cudaMemcpyHostToDevice));
  e->n_groups = (int)gr.size();
  return VXG_OK;
}
// The arrays an FP32C step writes (vx32::link_update, vx32::voxel_update, the actuation), as the
// columns k_bodies32 copies and a diverged batch puts back, and their copies (allocated once per
// scene size)
static int build_body_cols(vxg_engine* e) {
  if (e->d_body_cols) return VXG_OK;
  const size_t nv = (size_t)e->nv, nl = (size_t)e->nl;
  const View& B = e->S;
  uint32_t* v32 = (uint32_t*)e->arena32;
  uint32_t* l32 = (uint32_t*)(e->V.pos2);
  std::vector<BodyCol> c;
  auto add = [&](void* p, int words, int per_link) { c.push_back(BodyCol{(uint32_t*)p, nullptr, words, per_link}); };
  add(v32, 4, 0);           // P
  add(v32 + 4 * nv, 4, 0);  // Q
  for (int k = 0; k < 13; ++k) add(v32 + (8 + k) * nv, 1, 0);  // c, qc, lin, ang
  add(B.vflags, 1, 0);
  add(B.temp, 1, 0);
  for (int k = 0; k < 3; ++k) add(B.pStrain + k * nv, 1, 0);
  for (int k = 0; k < 22; ++k) add(l32 + k * nl, 1, 1);  // pos2, a1v, a2v, fN, fP, mN, mP, restDelta
  for (float* p : {B.tArea, B.tSS, B.strain, B.maxStrain, B.strainOffset, B.stress}) add(p, 1, 1);
  add(B.lflags, 1, 1);
  size_t words = 0;
  for (const BodyCol& x : c) words += (size_t)x.words * (x.per_link ? nl : nv);
  VXG_CK(cudaMalloc(&e->d_body_bak, sizeof(uint32_t) * std::max<size_t>(words, 1)));
  size_t at = 0;
  for (BodyCol& x : c) {
    x.dst = e->d_body_bak + at;
    at += (size_t)x.words * (x.per_link ? nl : nv);
  }
  e->body_cols = c;
  VXG_CK(cudaMalloc(&e->d_body_cols, sizeof(BodyCol) * c.size()));
  VXG_CK(cudaMemcpy(e->d_body_cols, c.data(), sizeof(BodyCol) * c.size(), cudaMemcpyHostToDevice));
  return VXG_OK;
}
// a diverged body batch: every array back to its copy from the start of the batch
static int restore_body_cols(vxg_engine* e) {
  for (const BodyCol& x : e->body_cols)
    VXG_CK(cudaMemcpyAsync(x.src, x.dst, sizeof(uint32_t) * x.words * (x.per_link ? e->nl : e->nv),
                           cudaMemcpyDeviceToDevice, e->stream));
  return VXG_OK;
}
// CTAs of the body-batch launch (all resident at once, no more than the groups)
static int bodies_grid(vxg_engine* e) {
  if (e->body_fit < 0) {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, bodies_kernel(e), kBodyCta, 0) != cudaSuccess) n = 0;
    cudaGetLastError();
    e->body_fit = n;
  }
  if (!e->n_sm) cudaDeviceGetAttribute(&e->n_sm, cudaDevAttrMultiProcessorCount, e->device);
  return std::min(e->n_groups, std::max(1, e->n_sm) * e->body_fit);
}
// whole batches in k_bodies32: FP32C, fixed dt, no collisions, no decision rows, the default link
// pass (in-step actuation's rest lengths computed in it), the Poisson cache filled by the voxel pass
// where it is used, and at least as many groups as SMs
static bool bodies_ok(vxg_engine* e, float dt) {
  if (!(e->body_target > 0 && e->precision == VXG_FP32C && dt > 0 && e->nl && e->nv && !e->g.collisions &&
        !e->dec_mode && e->timing != 1 && link_recomputes_rest(e, false)))
    return false;
  if (build_groups(e) != VXG_OK || build_body_cols(e) != VXG_OK) return false;
  if (!e->n_sm) cudaDeviceGetAttribute(&e->n_sm, cudaDevAttrMultiProcessorCount, e->device);
  return e->n_groups >= std::max(1, e->n_sm) && bodies_grid(e) > 0;
}
// before a batch: the Poisson caches the FP32C voxel pass filled ahead, after a host edit
static void poisson_refill(vxg_engine* e) {
  if (fused_poisson(e) && e->poisson_redo && e->g.any_poisson && e->nv) {
    k_poisson<true><<<grid_for(e->nv), kBlock, 0, e->stream>>>(e->S);
    e->n_launch += 1;
  }
  e->poisson_redo = false;
}

// enqueue one step (no synchronisation); in timing mode `ev` holds this step's 4 events.  `first`:
// the first step of a batch or of a captured chunk.
// k_validate once per change of the index fields or tables, before any kernel dereferences them
static const char* const kValField[] = {"", "voxel material", "voxel external", "voxel link", "link voxel",
                                        "link material", "material powf slot"};
static int check_topology(vxg_engine* e) {
  if (e->topo_ok) return VXG_OK;
  if (!e->d_bad) VXG_CK(cudaMalloc(&e->d_bad, sizeof(unsigned long long)));
  unsigned long long none = ~0ull, bad = 0;
  VXG_CK(cudaMemcpyAsync(e->d_bad, &none, sizeof(none), cudaMemcpyHostToDevice, e->stream));
  const int n = std::max(std::max(e->nv, e->nl), e->n_vm);
  if (n > 0) k_validate<<<grid_for(n), kBlock, 0, e->stream>>>(e->S, e->n_vm, e->n_lm, e->n_ext, e->n_powslots, e->d_bad);
  VXG_CK(cudaMemcpyAsync(&bad, e->d_bad, sizeof(bad), cudaMemcpyDeviceToHost, e->stream));
  VXG_CK(cudaStreamSynchronize(e->stream));
  if (bad != ~0ull) {
    char msg[160];
    const int field = (int)(bad >> 32);
    snprintf(msg, sizeof msg, "index out of range: %s, element %llu", field > 0 && field < 7 ? kValField[field] : "?",
             bad & 0xffffffffull);
    return fail(e, VXG_E_ARG, msg);
  }
  e->topo_ok = true;
  return VXG_OK;
}

// a launch that may overlap the previous kernel in the stream (the kernel waits for it itself)
extern "C++" {
template <typename... KArgs, typename... Args>
inline void launch_pdl(bool pdl, void (*kernel)(KArgs...), int grid, int block, cudaStream_t st, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = pdl ? 1 : 0;
  cudaLaunchKernelEx(&cfg, kernel, args...);
}
}

// rest_first: host-set temperatures not yet in the rest lengths; the step's link pass recomputes them
// (the caller only passes it where link_recomputes_rest holds)
static void enqueue_step(vxg_engine* e, float dt, int parity, bool first, cudaEvent_t* ev = nullptr,
                         bool rest_first = false) {
  const View& S = e->S;
  // the voxel pass's View: with collisions on it votes on the next step's stale test
  View Sv = S;
  vx32::View Vv = e->V;
  if (e->g.collisions && e->col.ready()) {
    e->col.voted(Sv, e->g, parity);
    Vv.B = Sv;
  }
  bool rec = dt < 0;
  const int bl = e->blk_link, bv = e->blk_voxel;
  const int gl = grid_of(e->nl, bl), gv = grid_of(e->nv, bv);
  if (ev) pass_event(ev[0], e->stream);
  // kernels this step launches (or, under capture, records)
  // overlap (launch_pdl) only where the kernel just before in the stream is known: a link pass
  // (which reads nothing before its wait) right after the previous step's voxel pass, and a voxel
  // pass right after its step's link pass (its early reads are the voxel's own state, which the
  // link pass never writes).  Any other kernel in between (actuation, the Poisson pre-pass, the
  // collision stage), a first step (conversions may precede it) or timing events make the launch
  // an ordinary one.
  const bool pdl_base = e->pdl && !ev && e->precision == VXG_FP32C;
  // FP32C at a fixed dt with the default link pass: the actuation's rest-length update happens in
  // the link pass itself (k_link32<..., ACT>), which directly follows the actuation kernel
  const bool act_fused = e->act_mode && e->nv && link_recomputes_rest(e, rec);
  const bool link_act = act_fused || (rest_first && link_recomputes_rest(e, rec));
  bool link_pdl = pdl_base && !first && (!e->act_mode || act_fused);
  long long nk = 1 + (e->nl ? 1 : 0) + (e->act_mode && e->nv ? 1 + (e->nl && !act_fused ? 1 : 0) : 0) +
                 (e->g.any_poisson && e->nv && !fused_poisson(e) ? 1 : 0);
  if (e->act_mode && e->nv) {
    const float* ph = e->act_mode == 2 ? e->d_phase : nullptr;
    const int fp32 = e->precision == VXG_FP32C ? 1 : 0;
    const float amp32 = (float)e->act_amp, w32 = (float)(2.0 * 3.141592653589793 * e->act_freq);
    // right after the previous step's voxel pass (not the first step of a batch): may overlap its tail
    launch_pdl(pdl_base && !first, k_actuate, grid_for(e->nv), kBlock, e->stream, S, e->act_amp, e->act_freq, ph, fp32,
               amp32, w32);
    if (e->nl && !act_fused) {
      if (e->precision == VXG_FP32C) k_rest32<<<grid_for(e->nl), kBlock, 0, e->stream>>>(e->V);
      else k_rest_length<<<grid_for(e->nl), kBlock, 0, e->stream>>>(S);
    }
  }
  // FP32C fills the cache in the voxel pass; caches the host invalidated are refilled before the
  // batch (poisson_refill), so no pre-pass runs inside it
  if (e->g.any_poisson && e->nv && !fused_poisson(e)) {
    k_poisson<false><<<grid_for(e->nv), kBlock, 0, e->stream>>>(S);
    link_pdl = false;
  }
  if (e->precision == VXG_FP32C) {
    if (e->nl) {
      const bool pois = e->tab_poisson;
      if (rec) {
        if (pois) k_link32<true, true, true><<<gl, bl, 0, e->stream>>>(e->V, parity);
        else k_link32<true, true, false><<<gl, bl, 0, e->stream>>>(e->V, parity);
      } else if (e->lp_bps != 0) {
        const int ntiles = (e->nl + kLpT - 1) / kLpT;
        const int grid = std::min(ntiles, lp_resident(e, pois));
        if (pois) k_link32p<true><<<grid, kLpT, kLpSmem, e->stream>>>(e->V, ntiles);
        else k_link32p<false><<<grid, kLpT, kLpSmem, e->stream>>>(e->V, ntiles);
      } else if (e->link_split) {
        // the general pass follows the small-angle pass directly, so it may always overlap its tail
        const int gL = std::min(grid_of(e->nl, 256), split_grid(e, pois));
        if (pois) {
          launch_pdl(link_pdl, k_link32s<true>, gl, bl, e->stream, e->V);
          launch_pdl(pdl_base, k_link32L<true>, gL, 256, e->stream, e->V);
        } else {
          launch_pdl(link_pdl, k_link32s<false>, gl, bl, e->stream, e->V);
          launch_pdl(pdl_base, k_link32L<false>, gL, 256, e->stream, e->V);
        }
        nk += 1;
      } else if (link_act) {
        if (pois) launch_pdl(link_pdl, k_link32<false, true, true, true>, gl, bl, e->stream, e->V, parity);
        else launch_pdl(link_pdl, k_link32<false, true, false, true>, gl, bl, e->stream, e->V, parity);
      } else {
        if (pois) launch_pdl(link_pdl, k_link32<false, true, true>, gl, bl, e->stream, e->V, parity);
        else launch_pdl(link_pdl, k_link32<false, true, false>, gl, bl, e->stream, e->V, parity);
      }
    }
    if (ev) pass_event(ev[1], e->stream);
    if (e->g.collisions) nk += e->col.enqueue(e->g, e->stream, first, parity);
    if (ev) pass_event(ev[2], e->stream);
    e->n_launch += nk;
    const bool voxel_pdl = pdl_base && e->nl && e->lp_bps == 0 && !e->g.collisions;
    if (fused_poisson(e)) {
      if (rec) k_voxel32<true, true><<<gv, bv, 0, e->stream>>>(Vv, dt, parity, e->g.fallback_freq2);
      else launch_pdl(voxel_pdl, k_voxel32<false, true>, gv, bv, e->stream, Vv, dt, parity, e->g.fallback_freq2);
    } else {
      if (rec) k_voxel32<true, false><<<gv, bv, 0, e->stream>>>(Vv, dt, parity, e->g.fallback_freq2);
      else launch_pdl(voxel_pdl, k_voxel32<false, false>, gv, bv, e->stream, Vv, dt, parity, e->g.fallback_freq2);
    }
    if (ev) pass_event(ev[3], e->stream);
    return;
  }
  if (e->nl) {
    if (rec) k_link<true, true><<<gl, bl, 0, e->stream>>>(S, parity);
    else k_link<false, true><<<gl, bl, 0, e->stream>>>(S, parity);
  }
  if (ev) pass_event(ev[1], e->stream);
  if (e->g.collisions) nk += e->col.enqueue(e->g, e->stream, first, parity);
  if (ev) pass_event(ev[2], e->stream);
  e->n_launch += nk;
  if (e->dec_mode) {  // one row of branch decisions per step (vxg_step checked the capacity)
    uint8_t* row = e->d_dec + (size_t)e->dec_step++ * (size_t)e->nv;
    if (e->dec_mode == 1) {
      if (rec) k_voxel<true, 1><<<gv, bv, 0, e->stream>>>(Sv, dt, parity, e->g.fallback_freq2, row);
      else k_voxel<false, 1><<<gv, bv, 0, e->stream>>>(Sv, dt, parity, e->g.fallback_freq2, row);
    } else {
      if (rec) k_voxel<true, 2><<<gv, bv, 0, e->stream>>>(Sv, dt, parity, e->g.fallback_freq2, row);
      else k_voxel<false, 2><<<gv, bv, 0, e->stream>>>(Sv, dt, parity, e->g.fallback_freq2, row);
    }
  } else if (rec) {
    k_voxel<true><<<gv, bv, 0, e->stream>>>(Sv, dt, parity, e->g.fallback_freq2);
  } else {
    k_voxel<false><<<gv, bv, 0, e->stream>>>(Sv, dt, parity, e->g.fallback_freq2);
  }
  if (ev) pass_event(ev[3], e->stream);
}

// every cached graph, after a change that any of them may have baked in
static void drop_graphs(vxg_engine* e) {
  for (cudaGraphExec_t* g : {&e->graph, &e->cgraph, &e->g1[0], &e->g1[1]})
    if (*g) {
      cudaGraphExecDestroy(*g);
      *g = nullptr;
    }
  e->graph_n = e->cgraph_n = -1;
}
// rest_first: the first step's link pass recomputes the rest lengths (enqueue_step)
static int capture(vxg_engine* e, int n, float dt, cudaGraphExec_t* out, long long* kernels, bool rest_first = false) {
  if (*out) { cudaGraphExecDestroy(*out); *out = nullptr; }
  cudaGraph_t g;
  VXG_CK(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
  const long long before = e->n_launch;
  for (int s = 0; s < n; ++s) enqueue_step(e, dt, s & 1, s == 0, nullptr, rest_first && s == 0);
  *kernels = e->n_launch - before;
  e->n_launch = before;  // counted per replay
  VXG_CK(cudaStreamEndCapture(e->stream, &g));
  cudaError_t c = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  if (c != cudaSuccess) return fail(e, VXG_E_CUDA, "graph instantiate", c);
  // upload now, so that the first replay (possibly timed) does not include it
  c = cudaGraphUpload(*out, e->stream);
  if (c != cudaSuccess) return fail(e, VXG_E_CUDA, "graph upload", c);
  return VXG_OK;
}

int vxg_step(vxg_engine* e, int nsteps, float dt, int* steps_done, int* diverged) {
  NvtxScope nvtx("vxg_step");
  if (!e || nsteps < 0) return VXG_E_ARG;
  if (!e->have_globals) return fail(e, VXG_E_STATE, "vxg_set_globals was not called");
  if (steps_done) *steps_done = 0;
  if (diverged) *diverged = 0;
  if (nsteps == 0 || dt == 0.0f) {
    if (steps_done) *steps_done = nsteps;
    return VXG_OK;
  }
  if (e->act_mode == 2 && e->n_phase < e->nv) return fail(e, VXG_E_STATE, "actuation phases cover fewer voxels than the scene");
  VXG_CK(cudaSetDevice(e->device));
  if (int rc = check_topology(e)) return rc;
  ensure32(e);
  if (e->precision == VXG_FP32C) e->stale64 = all_state_bits();
  // reset the per-batch control words: diverged, halt, steps, status, the dt maxima and the count of
  // deferred links (keep time and counters)
  static_assert(offsetof(Ctl, maxf) == 4 * sizeof(int) && offsetof(Ctl, n_large) == 4 * sizeof(int) + 2 * sizeof(unsigned) &&
                    offsetof(Ctl, time) == 6 * sizeof(int) + 2 * sizeof(unsigned),
                "control block layout");
  VXG_CK(cudaMemsetAsync(e->ctl, 0, offsetof(Ctl, time), e->stream));
  poisson_refill(e);
  if (e->dec_mode && e->dec_step + nsteps > e->dec_cap)
    return fail(e, VXG_E_SIZE, "vxg_step: more steps than the branch-decision rows set aside");
  // branch decisions take a row pointer per step: launched step by step, never captured
  bool use_graph = e->timing != 1 && nsteps > 1 && !e->dec_mode;
  // temperatures the host set since the last step: the first step's link pass recomputes the rest
  // lengths where it is launched on its own with the default link pass, else a pass does it now
  const int bodies = !e->body_rerun && bodies_ok(e, dt) ? bodies_grid(e) : 0;  // CTAs of a body batch, or 0
  if (bodies) use_graph = false;
  const bool rest_first = e->rest_pending && !bodies && !use_graph && e->timing != 1 && link_recomputes_rest(e, dt < 0);
  if (!rest_first) flush_rest(e);
  // a single step is replayed from a captured step as well (one launch instead of the step's
  // kernels), with the rest-length update in its link pass or without
  const bool use_g1 = nsteps == 1 && e->timing != 1 && !e->dec_mode && !bodies;
  const int g1k = rest_first ? 1 : 0;
  const int chunk = e->graph_chunk;
  if ((use_graph || use_g1) && !e->graph_valid) {
    drop_graphs(e);
    e->graph_valid = true;
  }
  // capture and instantiate the batch's graph before the batch timer starts (timing mode 2 times
  // the replay, not the capture)
  if (use_graph && nsteps >= chunk) {
    // long runs: one captured chunk (even length keeps the step parities aligned) replayed
    if (!e->cgraph || e->cgraph_dt != dt || e->cgraph_n != chunk) {
      int rc = capture(e, chunk, dt, &e->cgraph, &e->cgraph_kernels);
      if (rc) return rc;
      e->cgraph_dt = dt;
      e->cgraph_n = chunk;
    }
  } else if (use_graph) {
    if (!e->graph || e->graph_n != nsteps || e->graph_dt != dt) {
      int rc = capture(e, nsteps, dt, &e->graph, &e->graph_kernels);
      if (rc) return rc;
      e->graph_n = nsteps;
      e->graph_dt = dt;
    }
  } else if (use_g1) {
    if (!e->g1[g1k] || e->g1_dt[g1k] != dt) {
      int rc = capture(e, 1, dt, &e->g1[g1k], &e->g1_kernels[g1k], rest_first);
      if (rc) return rc;
      e->g1_dt[g1k] = dt;
    }
  }
  if (e->timing == 2) {
    for (int k = 0; k < 2; ++k)
      if (!e->bev[k]) VXG_CK(cudaEventCreate(&e->bev[k]));
    VXG_CK(cudaEventRecord(e->bev[0], e->stream));
  }
  if (e->g.collisions) e->n_launch += e->col.enqueue_surface(e->stream);  // the batch's surface list
  e->tev_used = 0;
  if (bodies) {
    const float* ph = e->act_mode == 2 ? e->d_phase : nullptr;
    const float amp32 = (float)e->act_amp, w32 = (float)(2.0 * 3.141592653589793 * e->act_freq);
    bodies_kernel(e)<<<bodies, kBodyCta, 0, e->stream>>>(e->V, dt, nsteps, e->d_groups, e->n_groups, e->d_bctl, amp32,
                                                          w32, ph, e->d_bctl + 1, e->d_body_cols,
                                                          (int)e->body_cols.size());
    k_bodies_done<<<1, 32, 0, e->stream>>>(e->ctl, dt, nsteps, e->d_bctl);
    e->n_launch += 2;
  } else if (use_g1) {
    VXG_CK(cudaGraphLaunch(e->g1[g1k], e->stream));
    e->n_launch += e->g1_kernels[g1k];
    e->rest_pending = false;
  } else if (use_graph) {
    if (nsteps >= chunk) {
      int full = nsteps / chunk;
      for (int k = 0; k < full; ++k) VXG_CK(cudaGraphLaunch(e->cgraph, e->stream));
      e->n_launch += full * e->cgraph_kernels;
      for (int s = full * chunk; s < nsteps; ++s) enqueue_step(e, dt, s & 1, s == full * chunk);
    } else {
      VXG_CK(cudaGraphLaunch(e->graph, e->stream));
      e->n_launch += e->graph_kernels;
    }
  } else if (e->timing == 1 && !e->dec_mode) {
    size_t need = (size_t)4 * nsteps;
    while (e->tev.size() < need) {
      cudaEvent_t x;
      VXG_CK(cudaEventCreate(&x));
      e->tev.push_back(x);
    }
    // the steps with their per-pass events, captured and replayed once so that the events time
    // the kernels, not the host's launch gaps
    cudaGraph_t g = nullptr;
    cudaGraphExec_t x = nullptr;
    VXG_CK(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
    for (int s = 0; s < nsteps; ++s) enqueue_step(e, dt, s & 1, s == 0, &e->tev[(size_t)4 * s]);
    cudaError_t c = cudaStreamEndCapture(e->stream, &g);
    if (c == cudaSuccess) c = cudaGraphInstantiate(&x, g, 0);
    if (g) cudaGraphDestroy(g);
    if (c == cudaSuccess) c = cudaGraphLaunch(x, e->stream);
    if (x) cudaGraphExecDestroy(x);
    if (c != cudaSuccess) return fail(e, VXG_E_CUDA, "timed batch", c);
    e->tev_used = nsteps;
  } else {
    for (int s = 0; s < nsteps; ++s) enqueue_step(e, dt, s & 1, s == 0, nullptr, rest_first && s == 0);
    e->rest_pending = false;
  }
  if (e->timing == 2) VXG_CK(cudaEventRecord(e->bev[1], e->stream));
  if (!e->h_ctl) {
    VXG_CK(cudaHostAlloc(&e->h_ctl, 4 * sizeof(int), cudaHostAllocMapped));
    VXG_CK(cudaHostGetDevicePointer(&e->h_ctl_dev, e->h_ctl, 0));
  }
  k_ctl_out<<<1, 32, 0, e->stream>>>(e->ctl, e->h_ctl_dev);
  e->n_launch += 1;
  VXG_CK(cudaStreamSynchronize(e->stream));
  const int* h = e->h_ctl;
  VXG_CK(cudaGetLastError());
  if (e->timing == 2) VXG_CK(cudaEventElapsedTime(&e->t_batch, e->bev[0], e->bev[1]));
  if (e->timing == 1 && e->tev_used > 0) {
    double a = 0, b = 0, c = 0;
    for (int s = 0; s < e->tev_used; ++s) {
      float x = 0, y = 0, z = 0;
      cudaEvent_t* ev = &e->tev[(size_t)4 * s];
      cudaEventElapsedTime(&x, ev[0], ev[1]);
      cudaEventElapsedTime(&y, ev[1], ev[2]);
      cudaEventElapsedTime(&z, ev[2], ev[3]);
      a += x; b += y; c += z;
    }
    e->t_link = (float)(a / e->tev_used);
    e->t_col = (float)(b / e->tev_used);
    e->t_vox = (float)(c / e->tev_used);
    cudaEventElapsedTime(&e->t_batch, e->tev[0], e->tev[(size_t)4 * (e->tev_used - 1) + 3]);
  }
  // h: diverged, halt, steps, status.  A body batch a group diverged in ends diverged without halt:
  // the batch again from its start, as passes
  if (bodies && h[0] && !h[1] && !h[3]) {
    if (int rc = restore_body_cols(e)) return rc;
    e->body_rerun = true;
    const int rc = vxg_step(e, nsteps, dt, steps_done, diverged);
    e->body_rerun = false;
    return rc;
  }
  if (steps_done) *steps_done = h[2];
  if (diverged) *diverged = h[1] ? 1 : 0;
  if (h[3]) return fail(e, VXG_E_DEVICE_STATUS, e->col.status_message(h[3]));
  return VXG_OK;
}

// ---- differentiated run ---------------------------------------------------------------------
int vxg_adjoint_com_x(vxg_engine* e, int nsteps, float dt, int checkpoint_every, const int* body_offsets,
                      int n_bodies, double* objective, double* dE, double* drho, double* dphase) {
  NvtxScope nvtx("vxg_adjoint_com_x");
  if (!e || nsteps <= 0 || !(dt > 0.0f) || checkpoint_every <= 0 || !body_offsets || n_bodies <= 0 || !objective)
    return VXG_E_ARG;
  if (!e->have_globals) return fail(e, VXG_E_STATE, "vxg_set_globals was not called");
  if (e->precision != VXG_FP64) return fail(e, VXG_E_STATE, "vxg_adjoint_com_x: the FP64 precision is differentiated");
  // its steps do not go through vxg_step, which bounds the decision rows
  if (e->dec_mode)
    return fail(e, VXG_E_STATE, "vxg_adjoint_com_x: branch decisions are being recorded or replayed (mode 0 first)");
  if (e->adj_scope) return fail(e, VXG_E_STATE, e->adj_scope);
  if (e->g.collisions) return fail(e, VXG_E_STATE, "vxg_adjoint_com_x: collisions are outside the differentiated scope");
  if (e->act_mode == 2 && e->n_phase < e->nv) return fail(e, VXG_E_STATE, "actuation phases cover fewer voxels than the scene");
  for (int b = 0; b < n_bodies; ++b)
    if (body_offsets[b] < 0 || body_offsets[b + 1] < body_offsets[b] || body_offsets[b + 1] > e->nv)
      return fail(e, VXG_E_ARG, "vxg_adjoint_com_x: body offsets out of range");
  VXG_CK(cudaSetDevice(e->device));
  if (int rc = check_topology(e)) return rc;
  const int nv = e->nv, nl = e->nl, K = std::min(checkpoint_every, nsteps);
  const int nck = (nsteps + K - 1) / K;
  const size_t ckb = e->arena_bytes + sizeof(Ctl);
  // one allocation for everything: checkpoints, final state, tape, adjoints
  size_t off_ck = 0, sz = (size_t)(nck + 1) * ckb;
  auto carve = [&](size_t bytes) { size_t o = (sz + 255) & ~(size_t)255; sz = o + bytes; return o; };
  size_t o_tv = carve(sizeof(double) * 13 * (size_t)nv * K), o_tvf = carve(sizeof(uint32_t) * (size_t)nv * K),
         o_tpd = carve(sizeof(float) * (size_t)nv * K), o_tl = carve(sizeof(double) * 9 * (size_t)nl * K),
         o_tlf = carve(sizeof(uint32_t) * (size_t)nl * K), o_tms = carve(sizeof(float) * (size_t)nl * K),
         o_tstr = carve(sizeof(float) * (size_t)nl * K), o_tps = carve(sizeof(float) * 3 * (size_t)nv * K),
         o_lps = carve(sizeof(double) * 6 * (size_t)nl), o_gs = carve(sizeof(double) * 6 * (size_t)nv),
         o_tt = carve(sizeof(float) * K),
         o_ttemp = carve(sizeof(float) * (size_t)nv * K),
         o_lam = carve(sizeof(double) * 13 * (size_t)nv), o_gfm = carve(sizeof(double) * 6 * (size_t)nv),
         o_mu = carve(sizeof(double) * 9 * (size_t)nl), o_lcon = carve(sizeof(double) * 14 * (size_t)nl),
         o_lpar = carve(sizeof(double) * 4 * (size_t)nl), o_lf = carve(sizeof(double) * 12 * (size_t)nl),
         o_gt = carve(sizeof(double) * nv), o_acc = carve(sizeof(double) * 3 * (size_t)nv),
         o_err = carve(sizeof(int)), o_off = carve(sizeof(int) * ((size_t)n_bodies + 1)),
         o_obj = carve(sizeof(double) * n_bodies);
  // the segment's link forces, taped when they fit in three quarters of the free memory (otherwise
  // each reverse step recomputes them)
  size_t o_tf = 0;
  {
    size_t free_b = 0, total_b = 0;
    const size_t need = sizeof(double) * 12 * (size_t)nl * K;
    if (nl && cudaMemGetInfo(&free_b, &total_b) == cudaSuccess && sz + need + 256 < free_b / 4 * 3)
      o_tf = carve(need);
    cudaGetLastError();
  }
  char* buf = nullptr;
  VXG_CK(cudaMalloc(&buf, sz));
  struct Free { char* p; ~Free() { if (p) cudaFree(p); } } guard{buf};
  AdjBuf T;
  T.K = K;
  T.tv = (double*)(buf + o_tv); T.tvf = (uint32_t*)(buf + o_tvf); T.tpd = (float*)(buf + o_tpd);
  T.tl = (double*)(buf + o_tl); T.tlf = (uint32_t*)(buf + o_tlf); T.ttime = (float*)(buf + o_tt);
  T.tms = (float*)(buf + o_tms);
  T.tstrain = (float*)(buf + o_tstr);
  T.tps = (float*)(buf + o_tps);
  T.lps = (double*)(buf + o_lps);
  T.gS = (double*)(buf + o_gs);
  T.ttemp = (float*)(buf + o_ttemp);
  T.tforce = o_tf ? (double*)(buf + o_tf) : nullptr;
  T.lam = (double*)(buf + o_lam); T.gFM = (double*)(buf + o_gfm); T.mu = (double*)(buf + o_mu);
  T.lcon = (double*)(buf + o_lcon); T.lpar = (double*)(buf + o_lpar); T.lforce = (double*)(buf + o_lf);
  T.gTempV = (double*)(buf + o_gt);
  T.accE = (double*)(buf + o_acc); T.accRho = T.accE + nv; T.accPhase = T.accE + 2 * (size_t)nv;
  T.err = (int*)(buf + o_err);
  int* d_off = (int*)(buf + o_off);
  double* d_obj = (double*)(buf + o_obj);
  ActParams A{e->act_mode, e->act_amp, e->act_freq, e->act_mode == 2 ? e->d_phase : nullptr};
  auto ck = [&](int c) { return buf + off_ck + (size_t)c * ckb; };
  auto save = [&](int c) -> int {
    VXG_CK(cudaMemcpyAsync(ck(c), e->arena, e->arena_bytes, cudaMemcpyDeviceToDevice, e->stream));
    VXG_CK(cudaMemcpyAsync(ck(c) + e->arena_bytes, e->ctl, sizeof(Ctl), cudaMemcpyDeviceToDevice, e->stream));
    return VXG_OK;
  };
  auto load = [&](int c) -> int {
    VXG_CK(cudaMemcpyAsync(e->arena, ck(c), e->arena_bytes, cudaMemcpyDeviceToDevice, e->stream));
    VXG_CK(cudaMemcpyAsync(e->ctl, ck(c) + e->arena_bytes, sizeof(Ctl), cudaMemcpyDeviceToDevice, e->stream));
    return VXG_OK;
  };
  int rc;
  // forward sweep, keeping the state at the start of every segment
  for (int c = 0; c < nck; ++c) {
    if ((rc = save(c))) return rc;
    int n = std::min(K, nsteps - c * K), done = 0, div = 0;
    if ((rc = vxg_step(e, n, dt, &done, &div))) return rc;
    if (done != n || div) return fail(e, VXG_E_STATE, "vxg_adjoint_com_x: the forward run diverged");
  }
  if ((rc = save(nck))) return rc;
  VXG_CK(cudaMemsetAsync(T.lam, 0, sizeof(double) * 13 * (size_t)nv, e->stream));
  VXG_CK(cudaMemsetAsync(T.mu, 0, sizeof(double) * 9 * (size_t)nl, e->stream));
  VXG_CK(cudaMemsetAsync(T.gS, 0, sizeof(double) * 6 * (size_t)nv, e->stream));
  VXG_CK(cudaMemsetAsync(T.accE, 0, sizeof(double) * 3 * (size_t)nv, e->stream));
  VXG_CK(cudaMemsetAsync(T.err, 0, sizeof(int), e->stream));
  VXG_CK(cudaMemcpyAsync(d_off, body_offsets, sizeof(int) * ((size_t)n_bodies + 1), cudaMemcpyHostToDevice, e->stream));
  k_adj_objective<<<n_bodies, 128, 0, e->stream>>>(e->S, T, d_off, d_obj);  // vxg_body_com's summation order
  VXG_CK(cudaGetLastError());
  const int gvx = grid_for(nv), glk = grid_for(std::max(nl, 1)), gboth = grid_for(std::max(nv, nl));
  // reverse sweep: per segment, re-run it from its checkpoint recording the tape, then walk back
  for (int c = nck - 1; c >= 0; --c) {
    if ((rc = load(c))) return rc;
    int n = std::min(K, nsteps - c * K);
    for (int s = 0; s < n; ++s) {
      k_tape_save<<<gboth, kBlock, 0, e->stream>>>(e->S, T, s);
      enqueue_step(e, dt, s & 1, s == 0);
      k_tape_step<<<gboth, kBlock, 0, e->stream>>>(e->S, T, s);
    }
    for (int s = n - 1; s >= 0; --s) {
      AdjBuf Ts = T;
      if (T.tforce) Ts.lforce = T.tforce + (size_t)s * 12 * nl;  // taped by the recomputation
      else if (nl) k_adj_link_forces<<<glk, kBlock, 0, e->stream>>>(e->S, T, A, s);
      k_adj_voxel<<<gvx, kBlock, 0, e->stream>>>(e->S, Ts, A, s, dt);
      if (nl) k_adj_link<<<glk, kBlock, 0, e->stream>>>(e->S, T, A, s);
      k_adj_gather<<<gvx, kBlock, 0, e->stream>>>(e->S, T, A, s);
      if (e->g.any_poisson) k_adj_ratio<<<gvx, kBlock, 0, e->stream>>>(e->S, T, s);
    }
    VXG_CK(cudaGetLastError());
  }
  if ((rc = load(nck))) return rc;
  int err = 0;
  VXG_CK(cudaMemcpyAsync(&err, T.err, sizeof(int), cudaMemcpyDeviceToHost, e->stream));
  VXG_CK(cudaMemcpyAsync(objective, d_obj, sizeof(double) * n_bodies, cudaMemcpyDeviceToHost, e->stream));
  if (dE) VXG_CK(cudaMemcpyAsync(dE, T.accE, sizeof(double) * nv, cudaMemcpyDeviceToHost, e->stream));
  if (drho) VXG_CK(cudaMemcpyAsync(drho, T.accRho, sizeof(double) * nv, cudaMemcpyDeviceToHost, e->stream));
  if (dphase) VXG_CK(cudaMemcpyAsync(dphase, T.accPhase, sizeof(double) * nv, cudaMemcpyDeviceToHost, e->stream));
  VXG_CK(cudaStreamSynchronize(e->stream));
  VXG_CK(cudaGetLastError());
  if (err & 1) return fail(e, VXG_E_STATE, "vxg_adjoint_com_x: a link's adjoint could not be taken");
  return VXG_OK;
}

int vxg_recommended_dt(vxg_engine* e, float* dt) {
  NvtxScope nvtx("vxg_recommended_dt");
  if (!e || !dt) return VXG_E_ARG;
  if (!e->have_globals) return fail(e, VXG_E_STATE, "vxg_set_globals was not called");
  VXG_CK(cudaSetDevice(e->device));
  flush_rest(e);
  if (int rc = check_topology(e)) return rc;
  int zeros[4] = {0, 0, 0, 0};
  VXG_CK(cudaMemcpyAsync(e->ctl, zeros, sizeof(zeros), cudaMemcpyHostToDevice, e->stream));
  unsigned z = 0u;
  VXG_CK(cudaMemcpyAsync(&e->ctl->maxf[0], &z, 4, cudaMemcpyHostToDevice, e->stream));
  ensure32(e);
  poisson_refill(e);
  if (e->g.any_poisson && e->nv) k_poisson<false><<<grid_for(e->nv), kBlock, 0, e->stream>>>(e->S);
  if (e->precision == VXG_FP32C) {
    if (e->nl) k_link32<true, false, false><<<grid_for(e->nl), kBlock, 0, e->stream>>>(e->V, 0);
    e->stale64 |= 1u << VXG_F_REST_LENGTH;
  } else if (e->nl) {
    k_link<true, false><<<grid_for(e->nl), kBlock, 0, e->stream>>>(e->S, 0);
  }
  unsigned u = 0;
  VXG_CK(cudaMemcpyAsync(&u, &e->ctl->maxf[0], 4, cudaMemcpyDeviceToHost, e->stream));
  VXG_CK(cudaStreamSynchronize(e->stream));
  VXG_CK(cudaGetLastError());
  float mx;
  std::memcpy(&mx, &u, 4);
  if (mx <= 0.0f) mx = e->g.fallback_freq2;
  *dt = (mx <= 0.0f) ? 0.0f : 1.0f / (6.283185f * sqrtf(mx));
  return VXG_OK;
}

int vxg_set_all_temperatures(vxg_engine* e, float t) {
  if (!e) return VXG_E_ARG;
  VXG_CK(cudaSetDevice(e->device));
  ensure32(e);
  if (e->nv) k_set_temp<<<grid_for(e->nv), kBlock, 0, e->stream>>>(e->S, t);
  if (e->precision == VXG_FP32C) {
    e->rest_pending = true;  // the next step's link pass (or a rest-length pass) recomputes them
    e->stale64 |= 1u << VXG_F_REST_LENGTH;
  } else if (e->nl) {
    k_rest_length<<<grid_for(e->nl), kBlock, 0, e->stream>>>(e->S);
  }
  VXG_CK(cudaGetLastError());
  return VXG_OK;
}

int vxg_set_temperatures(vxg_engine* e, const float* t) {
  if (!e || (!t && e->nv)) return VXG_E_ARG;
  VXG_CK(cudaSetDevice(e->device));
  ensure32(e);
  if (e->nv) {
    // pinned host memory: read by a kernel (no copy engine, which the overlapped position reads
    // use); anything else: a copy
    cudaPointerAttributes pa;
    if (cudaPointerGetAttributes(&pa, t) == cudaSuccess && pa.type == cudaMemoryTypeHost && pa.devicePointer) {
      const bool vec = ((reinterpret_cast<uintptr_t>(pa.devicePointer) | reinterpret_cast<uintptr_t>(e->S.temp)) & 15) == 0;
      k_temp_in<<<grid_for(vec ? (e->nv + 3) / 4 : e->nv), kBlock, 0, e->stream>>>(e->S, (const float*)pa.devicePointer);
    } else {
      cudaGetLastError();
      VXG_CK(cudaMemcpyAsync(e->S.temp, t, sizeof(float) * (size_t)e->nv, cudaMemcpyHostToDevice, e->stream));
    }
  }
  if (e->precision == VXG_FP32C) {
    e->rest_pending = true;  // the next step's link pass (or a rest-length pass) recomputes them
    e->stale64 |= 1u << VXG_F_REST_LENGTH;
  } else if (e->nl) {
    k_rest_length<<<grid_for(e->nl), kBlock, 0, e->stream>>>(e->S);
  }
  VXG_CK(cudaGetLastError());
  return VXG_OK;
}

int vxg_reduce(vxg_engine* e, int info, int type, float* out) {
  if (!e || !out || info < 0 || info > 9 || type < 0 || type > 3) return VXG_E_ARG;
  VXG_CK(cudaSetDevice(e->device));
  if (int rc = check_topology(e)) return rc;
  bool link = info == 5 || info == 6 || info == 7;
  int n = link ? e->nl : e->nv;
  if (n == 0) { *out = 0.0f; return VXG_OK; }
  if (info == 8) return fail(e, VXG_E_ARG, "PRESSURE is reduced on the host");
  ensure64_info(e, info);
  int blocks = std::min(4096, grid_for(n));
  k_reduce<<<blocks, kBlock, 0, e->stream>>>(e->S, info, n, e->d_partials);
  std::vector<double> h((size_t)3 * blocks);
  VXG_CK(cudaMemcpyAsync(h.data(), e->d_partials, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, e->stream));
  VXG_CK(cudaStreamSynchronize(e->stream));
  double mn = h[0], mx = h[1], sm = 0.0;
  for (int b = 0; b < blocks; ++b) {
    mn = std::min(mn, h[3 * b]);
    mx = std::max(mx, h[3 * b + 1]);
    sm += h[3 * b + 2];
  }
  switch (type) {
    case 0: *out = (float)mn; break;
    case 1: *out = (float)mx; break;
    case 2: *out = (float)sm; break;
    default: *out = (float)(sm / n); break;
  }
  return VXG_OK;
}

int vxg_set_actuation(vxg_engine* e, int mode, double amplitude, double frequency, const float* phase) {
  if (!e || mode < 0 || mode > 2 || (mode == 2 && !phase && e->nv)) return VXG_E_ARG;
  VXG_CK(cudaSetDevice(e->device));
  if (mode == 2 && e->nv) {
    if (e->n_phase < e->nv) {
      if (e->d_phase) cudaFree(e->d_phase);
      e->d_phase = nullptr;
      VXG_CK(cudaMalloc(&e->d_phase, sizeof(float) * (size_t)e->nv));
      e->n_phase = e->nv;
    }
    VXG_CK(cudaMemcpyAsync(e->d_phase, phase, sizeof(float) * (size_t)e->nv, cudaMemcpyHostToDevice, e->stream));
    VXG_CK(cudaStreamSynchronize(e->stream));
  }
  e->act_mode = mode;
  e->act_amp = amplitude;
  e->act_freq = frequency;
  e->graph_valid = false;
  return VXG_OK;
}

int vxg_body_com(vxg_engine* e, const int* offsets, int n_bodies, double* out) {
  if (!e || !offsets || !out || n_bodies <= 0) return VXG_E_ARG;
  for (int b = 0; b < n_bodies; ++b)  // each body a range inside the scene
    if (offsets[b] < 0 || offsets[b + 1] < offsets[b] || offsets[b + 1] > e->nv)
      return fail(e, VXG_E_SIZE, "vxg_body_com: offsets out of range");
  VXG_CK(cudaSetDevice(e->device));
  if (int rc = check_topology(e)) return rc;
  if (n_bodies > e->n_body_cap) {
    if (e->d_body_off) cudaFree(e->d_body_off);
    if (e->d_body_out) cudaFree(e->d_body_out);
    e->d_body_off = nullptr;
    e->d_body_out = nullptr;
    VXG_CK(cudaMalloc(&e->d_body_off, sizeof(int) * ((size_t)n_bodies + 1)));
    VXG_CK(cudaMalloc(&e->d_body_out, sizeof(double) * 3 * (size_t)n_bodies));
    e->n_body_cap = n_bodies;
  }
  ensure32(e);
  VXG_CK(cudaMemcpyAsync(e->d_body_off, offsets, sizeof(int) * ((size_t)n_bodies + 1), cudaMemcpyHostToDevice, e->stream));
  bool fp32 = e->precision == VXG_FP32C;
  k_body_com<<<n_bodies, 128, 0, e->stream>>>(e->S, fp32 ? e->V.P : nullptr, fp32 ? e->V.c : nullptr, e->g.voxSize,
                                             e->d_body_off, e->d_body_out);
  VXG_CK(cudaMemcpyAsync(out, e->d_body_out, sizeof(double) * 3 * (size_t)n_bodies, cudaMemcpyDeviceToHost, e->stream));
  VXG_CK(cudaStreamSynchronize(e->stream));
  VXG_CK(cudaGetLastError());
  return VXG_OK;
}

int vxg_set_launch(vxg_engine* e, int block_link, int block_voxel, int graph_chunk) {
  if (!e) return VXG_E_ARG;
  auto ok = [](int b) { return b == 64 || b == 128 || b == 256 || b == 512; };
  if ((block_link && !ok(block_link)) || (block_voxel && !ok(block_voxel)) || graph_chunk < 0) return VXG_E_ARG;
  if (block_link) e->blk_link = block_link;
  if (block_voxel) e->blk_voxel = block_voxel;
  if (graph_chunk) e->graph_chunk = (graph_chunk + 1) & ~1;  // even: the step parity repeats
  e->graph_valid = false;
  return VXG_OK;
}

int vxg_set_body_batches(vxg_engine* e, int voxels_per_group) {
  if (!e || voxels_per_group < 0) return VXG_E_ARG;
  e->body_target = voxels_per_group;
  return VXG_OK;
}
int vxg_get_body_batches(vxg_engine* e, int* voxels_per_group, int* groups) {
  if (!e || !voxels_per_group) return VXG_E_ARG;
  *voxels_per_group = e->body_target;
  if (groups) {
    *groups = 0;
    if (e->body_target > 0 && e->nv && e->nl) {
      VXG_CK(cudaSetDevice(e->device));
      if (int rc = check_topology(e)) return rc;
      if (int rc = build_groups(e)) return rc;
      *groups = e->n_groups;
    }
  }
  return VXG_OK;
}
int vxg_set_link_split(vxg_engine* e, int on) {
  if (!e || (on != 0 && on != 1)) return VXG_E_ARG;
  e->link_split = on;
  e->graph_valid = false;
  return VXG_OK;
}
int vxg_get_link_split(vxg_engine* e, int* on) {
  if (!e || !on) return VXG_E_ARG;
  *on = e->link_split;
  return VXG_OK;
}
int vxg_set_link_pipeline(vxg_engine* e, int blocks_per_sm) {
  if (!e || blocks_per_sm < -1 || blocks_per_sm > 64) return VXG_E_ARG;
  e->lp_bps = blocks_per_sm;
  e->graph_valid = false;
  return VXG_OK;
}
int vxg_set_poisson_fusion(vxg_engine* e, int on) {
  if (!e) return VXG_E_ARG;
  if (e->poisson_fuse != (on != 0)) {
    e->poisson_fuse = on != 0;
    e->poisson_redo = true;  // caches filled ahead of time are refilled at the lazy point
    e->graph_valid = false;
  }
  return VXG_OK;
}
int vxg_set_decisions(vxg_engine* e, int mode, long long steps) {
  if (!e || mode < 0 || mode > 2 || steps < 0) return VXG_E_ARG;
  if (mode && e->precision != VXG_FP64) return fail(e, VXG_E_STATE, "vxg_set_decisions: the FP64 path records decisions");
  VXG_CK(cudaSetDevice(e->device));
  if (mode && steps > e->dec_cap) {
    if (e->d_dec) cudaFree(e->d_dec);
    e->d_dec = nullptr;
    e->dec_cap = 0;
    VXG_CK(cudaMalloc(&e->d_dec, std::max<size_t>(1, (size_t)steps * (size_t)e->nv)));
    e->dec_cap = steps;
  }
  e->dec_mode = mode;
  e->dec_step = 0;
  e->graph_valid = false;
  return VXG_OK;
}
int vxg_get_decisions(vxg_engine* e, unsigned char* host, long long steps) {
  if (!e || !host || steps < 0 || steps > e->dec_cap) return VXG_E_ARG;
  VXG_CK(cudaSetDevice(e->device));
  if (steps && e->nv)
    VXG_CK(cudaMemcpyAsync(host, e->d_dec, (size_t)steps * (size_t)e->nv, cudaMemcpyDeviceToHost, e->stream));
  VXG_CK(cudaStreamSynchronize(e->stream));
  return VXG_OK;
}
int vxg_put_decisions(vxg_engine* e, const unsigned char* host, long long steps) {
  if (!e || !host || steps < 0 || steps > e->dec_cap) return VXG_E_ARG;
  VXG_CK(cudaSetDevice(e->device));
  if (steps && e->nv)
    VXG_CK(cudaMemcpyAsync(e->d_dec, host, (size_t)steps * (size_t)e->nv, cudaMemcpyHostToDevice, e->stream));
  VXG_CK(cudaStreamSynchronize(e->stream));
  return VXG_OK;
}
int vxg_get_link_pipeline(vxg_engine* e, int* blocks_per_sm) {
  if (!e || !blocks_per_sm) return VXG_E_ARG;
  *blocks_per_sm = e->lp_bps;
  return VXG_OK;
}
int vxg_get_launch(vxg_engine* e, int* block_link, int* block_voxel, int* graph_chunk) {
  if (!e) return VXG_E_ARG;
  if (block_link) *block_link = e->blk_link;
  if (block_voxel) *block_voxel = e->blk_voxel;
  if (graph_chunk) *graph_chunk = e->graph_chunk;
  return VXG_OK;
}

// Device copies of the whole simulation state (every field, the FP32C state, the control block
// and the collision buffers) kept in device memory: checkpoints for restarts and recomputation.
int vxg_snapshot(vxg_engine* e, int slot) {
  if (!e || slot < 0 || slot > 1023) return VXG_E_ARG;
  VXG_CK(cudaSetDevice(e->device));
  ensure32(e);
  flush_rest(e);
  if ((int)e->snaps.size() <= slot) e->snaps.resize(slot + 1);
  vxg_engine::Snap& sl = e->snaps[slot];
  const size_t sizes[4] = {e->arena_bytes, e->arena32_bytes, sizeof(Ctl), e->col.buf_bytes};
  char* const src[4] = {e->arena, e->arena32, (char*)e->ctl, e->col.buf};
  for (int k = 0; k < 4; ++k) {
    if (sl.p[k] && sl.n[k] != sizes[k]) { cudaFree(sl.p[k]); sl.p[k] = nullptr; sl.n[k] = 0; }
    if (!src[k] || !sizes[k]) continue;
    if (!sl.p[k]) VXG_CK(cudaMalloc(&sl.p[k], sizes[k]));
    sl.n[k] = sizes[k];
    VXG_CK(cudaMemcpyAsync(sl.p[k], src[k], sizes[k], cudaMemcpyDeviceToDevice, e->stream));
  }
  sl.nv = e->nv;
  sl.nl = e->nl;
  sl.precision = e->precision;
  VXG_CK(cudaStreamSynchronize(e->stream));
  return VXG_OK;
}

int vxg_restore(vxg_engine* e, int slot) {
  if (!e || slot < 0 || slot >= (int)e->snaps.size() || e->snaps[slot].nv < 0) return VXG_E_ARG;
  vxg_engine::Snap& sl = e->snaps[slot];
  const size_t sizes[4] = {e->arena_bytes, e->arena32_bytes, sizeof(Ctl), e->col.buf_bytes};
  char* const dst[4] = {e->arena, e->arena32, (char*)e->ctl, e->col.buf};
  if (sl.nv != e->nv || sl.nl != e->nl || sl.precision != e->precision)
    return fail(e, VXG_E_STATE, "vxg_restore: the scene changed since the snapshot");
  for (int k = 0; k < 4; ++k)
    if ((sl.p[k] != nullptr) != (dst[k] != nullptr && sizes[k] != 0) || (sl.p[k] && sl.n[k] != sizes[k]))
      return fail(e, VXG_E_STATE, "vxg_restore: buffer layout changed since the snapshot");
  VXG_CK(cudaSetDevice(e->device));
  for (int k = 0; k < 4; ++k)
    if (sl.p[k]) VXG_CK(cudaMemcpyAsync(dst[k], sl.p[k], sizes[k], cudaMemcpyDeviceToDevice, e->stream));
  VXG_CK(cudaStreamSynchronize(e->stream));
  if (e->precision == VXG_FP32C) {
    e->dirty64 = 0;
    e->stale64 = all_state_bits();
  }
  e->rest_pending = false;  // snapshots are taken with the rest lengths up to date
  e->poisson_redo = true;
  return VXG_OK;
}

// Picks the link and voxel block sizes and the graph chunk length by timing short runs on the
// current scene; the state is snapshotted before and restored after, so the simulation is unchanged.
int vxg_autotune(vxg_engine* e, int trial_steps, float dt, int* best_link, int* best_voxel, int* best_chunk) {
  NvtxScope nvtx("vxg_autotune");
  if (!e || trial_steps < 2) return VXG_E_ARG;
  const int slot = 1023;
  int rc = vxg_snapshot(e, slot);
  if (rc) return rc;
  const int cand[4] = {64, 128, 256, 512};
  float best = 1e30f;
  int bl = e->blk_link, bv = e->blk_voxel, bc = e->graph_chunk, bps = e->lp_bps;
  int timing = e->timing;
  e->timing = 1;
  float t_link_best = 1e30f;  // the best one-thread-per-link pass, against the pipelined one below
  e->lp_bps = 0;
  for (int a = 0; a < 4 && !rc; ++a)
    for (int b = 0; b < 4; ++b) {
      e->blk_link = cand[a];
      e->blk_voxel = cand[b];
      int done = 0, div = 0;
      if ((rc = vxg_step(e, trial_steps, dt, &done, &div))) break;
      if ((rc = vxg_restore(e, slot))) break;
      if (e->t_link + e->t_vox < best) {
        best = e->t_link + e->t_vox;
        t_link_best = e->t_link;
        bl = cand[a];
        bv = cand[b];
      }
    }
  e->blk_link = bl;
  e->blk_voxel = bv;
  bps = 0;
  // FP32C at a fixed dt: the split link pass against the single general pass
  if (!rc && e->precision == VXG_FP32C && dt > 0 && e->nl) {
    const int split0 = e->link_split;
    e->link_split = 1 - split0;
    int done = 0, div = 0;
    if (!(rc = vxg_step(e, trial_steps, dt, &done, &div)) && !(rc = vxg_restore(e, slot))) {
      if (e->t_link < t_link_best) t_link_best = e->t_link;
      else e->link_split = split0;
    }
  }
  // FP32C at a fixed dt: the pipelined link pass at several residencies
  if (!rc && e->precision == VXG_FP32C && dt > 0 && e->nl) {
    const int res[4] = {-1, 2, 3, 4};
    for (int a = 0; a < 4; ++a) {
      e->lp_bps = res[a];
      int done = 0, div = 0;
      if ((rc = vxg_step(e, trial_steps, dt, &done, &div))) break;
      if ((rc = vxg_restore(e, slot))) break;
      if (e->t_link < t_link_best) {
        t_link_best = e->t_link;
        bps = res[a];
      }
    }
  }
  e->lp_bps = bps;
  e->timing = timing;
  // graph chunk: replay throughput of a few candidate lengths
  if (!rc) {
    float bestc = 1e30f;
    const int chunks[4] = {8, 32, 128, 512};
    cudaEvent_t t0, t1;
    cudaEventCreate(&t0);
    cudaEventCreate(&t1);
    for (int k = 0; k < 4 && !rc; ++k) {
      e->graph_chunk = chunks[k];
      e->graph_valid = false;
      int n = std::max(chunks[k], trial_steps), done = 0, div = 0;
      if ((rc = vxg_step(e, chunks[k], dt, &done, &div))) break;  // capture outside the timing
      cudaEventRecord(t0, e->stream);
      if ((rc = vxg_step(e, n, dt, &done, &div))) break;
      cudaEventRecord(t1, e->stream);
      cudaEventSynchronize(t1);
      float ms = 0;
      cudaEventElapsedTime(&ms, t0, t1);
      if (ms / n < bestc) { bestc = ms / n; bc = chunks[k]; }
      if ((rc = vxg_restore(e, slot))) break;
    }
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
  }
  e->graph_chunk = bc;
  e->graph_valid = false;
  // The per-pass events above include each pass's launch gap and keep the passes from overlapping,
  // which on small scenes is most of a pass: the shapes they picked, the plain link kernel at the
  // same shapes, and the engine's defaults are compared once more as replayed batches
  if (!rc && e->nl) {
    struct Shape { int bl, bv, split, bps; };
    const Shape picked = {e->blk_link, e->blk_voxel, e->link_split, e->lp_bps};
    const Shape cands[3] = {picked, {picked.bl, picked.bv, 0, 0}, {e->precision == VXG_FP32C ? 128 : 256, 256, 0, 0}};
    const int timing0 = e->timing;
    float best_t = 1e30f;
    Shape best_s = picked;
    e->timing = 2;
    for (int k = 0; k < 3 && !rc; ++k) {
      const Shape& c = cands[k];
      if (k && c.bl == picked.bl && c.bv == picked.bv && c.split == picked.split && c.bps == picked.bps) continue;
      e->blk_link = c.bl;
      e->blk_voxel = c.bv;
      e->link_split = c.split;
      e->lp_bps = c.bps;
      e->graph_valid = false;
      int done = 0, div = 0;
      const int n = std::max(2 * bc, trial_steps);
      if ((rc = vxg_step(e, n, dt, &done, &div))) break;  // captures or warms up
      if ((rc = vxg_restore(e, slot))) break;
      if ((rc = vxg_step(e, n, dt, &done, &div))) break;
      if (e->t_batch < best_t) { best_t = e->t_batch; best_s = c; }
      if ((rc = vxg_restore(e, slot))) break;
    }
    e->timing = timing0;
    e->blk_link = best_s.bl;
    e->blk_voxel = best_s.bv;
    e->link_split = best_s.split;
    e->lp_bps = best_s.bps;
    e->graph_valid = false;
    bl = best_s.bl;
    bv = best_s.bv;
  }
  // FP32C at a fixed dt: body batches of several group sizes (1: every segment a group of its own)
  // against the replayed graphs, on batches of the trial length
  if (!rc && e->precision == VXG_FP32C && dt > 0) {
    const int target0 = e->body_target, timing0 = e->timing;
    const int cand[5] = {0, 1, 512, 2048, 8192};
    float best_t = 1e30f;
    int best_target = 0;
    e->timing = 2;
    for (int k = 0; k < 5 && !rc; ++k) {
      e->body_target = cand[k];
      if (k && !bodies_ok(e, dt)) continue;
      int done = 0, div = 0;
      const int n = std::max(2 * bc, trial_steps);
      if ((rc = vxg_step(e, n, dt, &done, &div))) break;  // captures or warms up
      if ((rc = vxg_restore(e, slot))) break;
      if ((rc = vxg_step(e, n, dt, &done, &div))) break;
      if (e->t_batch < best_t) { best_t = e->t_batch; best_target = cand[k]; }
      if ((rc = vxg_restore(e, slot))) break;
    }
    e->timing = timing0;
    e->body_target = rc ? target0 : best_target;
  }
  if (best_link) *best_link = bl;
  if (best_voxel) *best_voxel = bv;
  if (best_chunk) *best_chunk = bc;
  if (e->precision == VXG_FP32C) e->stale64 = all_state_bits();
  return rc;
}

int vxg_get_collisions(vxg_engine* e, int* pairs, int cap, int* n) {
  if (!e || !n) return VXG_E_ARG;
  VXG_CK(cudaSetDevice(e->device));
  int rc = e->col.get_pairs(pairs, cap, n, e->stream);
  return rc ? fail(e, rc, "collision readback") : VXG_OK;
}

int vxg_counters(vxg_engine* e, long long* out, int n) {
  if (!e || !out || n < 0) return VXG_E_ARG;
  VXG_CK(cudaSetDevice(e->device));
  unsigned long long h[VXG_C_COUNT];
  VXG_CK(cudaMemcpyAsync(h, e->ctl->counters, sizeof(h), cudaMemcpyDeviceToHost, e->stream));
  VXG_CK(cudaStreamSynchronize(e->stream));
  h[VXG_C_REBUILDS] = (unsigned long long)e->col.rebuilds();
  h[VXG_C_PAIRS] = (unsigned long long)e->col.pairs(e->stream);
  h[VXG_C_LAUNCHES] = (unsigned long long)e->n_launch;
  for (int i = 0; i < n && i < VXG_C_COUNT; ++i) out[i] = (long long)h[i];
  return VXG_OK;
}

int vxg_enable_timing(vxg_engine* e, int on) {
  if (!e) return VXG_E_ARG;
  if (on < 0 || on > 2) return VXG_E_ARG;
  e->timing = on;
  return VXG_OK;
}

int vxg_last_step_timing(vxg_engine* e, float* a, float* b, float* c) {
  if (!e) return VXG_E_ARG;
  if (a) *a = e->t_link;
  if (b) *b = e->t_col;
  if (c) *c = e->t_vox;
  return VXG_OK;
}

int vxg_last_batch_ms(vxg_engine* e, float* ms) {
  if (!e || !ms) return VXG_E_ARG;
  *ms = e->t_batch;
  return VXG_OK;
}

const char* vxg_last_error(const vxg_engine* e) { return e ? e->err.c_str() : "null engine"; }
void* vxg_stream(vxg_engine* e) { return e ? (void*)e->stream : nullptr; }
int vxg_synchronize(vxg_engine* e) {
  if (!e) return VXG_E_ARG;
  VXG_CK(cudaStreamSynchronize(e->stream));
  return VXG_OK;
}

}  // extern "C"
