// Collision stage of the time step: CVoxelyze::updateCollisions / regenerateCollisions and
// CVX_Collision::updateContactForce (src/Voxelyze.cpp:670-750, src/VX_Collision.cpp:15-56).
//
// Per step, on the engine stream:
//   c_surface  once per batch: the surface voxels as a list (warp ballot, one atomic per warp),
//              the only voxels the stale test and the rebuild visit
//   c_check    the first step of a batch (or of a captured chunk): each surface voxel tests its
//              drift from the position at the last rebuild (float copy, double distance, as the
//              reference) and raises the device "stale" flag; every later step takes the vote the
//              previous step's voxel pass cast from the positions it wrote (the same test on the
//              same numbers)
//   rebuild    only when stale (it exits at once otherwise); one cooperative launch (c_rebuild)
//              runs these phases with grid-wide barriers between them, or, where cooperative
//              launches are not available, six separate kernels:
//              c_insert  surface voxels into a uniform hash grid (cell = watch radius), open
//                        addressing on the packed cell key, one linked list per cell
//              c_count   each surface voxel counts partners within the watch radius that are not
//                        lattice neighbours (the 5-hop list, binary search) - all, and those after
//                        it; one warp per voxel, lane k walking the k-th of the 27 cells around it
//              c_scan    exclusive scans give each voxel its slot in the pair list and in the
//                        contact list
//              c_fill    each voxel's partners, packed by the lanes into the warp's shared buffer
//                        and placed by rank; pairs (i, j > i) land in the reference's list order
//                        (i ascending, then j ascending)
//              c_watch   each voxel's contact list: partners ascending, with the pair index found
//                        in the partner's sorted list (the order the reference's colWatch ends in),
//                        one lane per partner
//   c_contact  one thread per pair: the penalty + damping contact force (float math)
// The voxel pass subtracts each voxel's contact forces in its contact-list order.
#pragma once
#include <cooperative_groups.h>

struct ColCtl {
  int stale;        // rebuild needed this step
  int force_stale;  // set by the host when topology or the collision switch changed
  int npairs;
  int nwatch;
  int status;       // overflow bits
  int rebuilds;
  int vote[2];      // set by a voxel pass whose new positions make the pair list stale; slot =
                    // the step's parity (the stage of the next step reads it, and clears its own)
  int nsurf;        // surface voxels listed by c_surface
};

enum { VXG_COL_ST_PAIR_OVERFLOW = 1, VXG_COL_ST_WATCH_OVERFLOW = 2, VXG_COL_ST_LOCAL_OVERFLOW = 4,
       VXG_COL_ST_HASH_FULL = 8 };

constexpr int kMaxPartners = 128;
constexpr int kScanBlocks = 4096;  // most blocks a cooperative stage launch may have

struct ColView {
  int nv;
  unsigned long long hcap_mask;
  const double* pos;
  const double* linMom;
  // FP32C state (fp32 != 0): position = lattice index * voxel size + (d - c), momenta in FP32
  int fp32;
  const float4* P32;
  const float* c32;
  const float* lin32;
  const int* vidx;
  double s64;
  float s32;
  const int* vmat;
  const uint32_t* vflags;
  const float* temp;
  const vxg_voxel_material* vm;
  const int* nbOff;
  const int* nbItem;
  float* lastWatch;          // 3 nv
  unsigned long long* hkey;  // hcap
  int* hhead;                // hcap
  int* next;                 // nv
  int* cntGt;                // nv
  int* cntAll;               // nv
  int* surf;                 // nv: the surface voxels (c_surface), nsurf of them
  double* spos;              // 3 nv: a surface voxel's position at the rebuild (cpos), set by c_insert
  unsigned char* lcnt;       // 32 nv: partners lane k found in v's k-th neighbour cell (c_count)
  int* part;                 // 2 kScanBlocks: per-block totals of the grid-wide scan
  int* scell;                // 3 nv: its hash-grid cell coordinates, set by c_insert
  int* pairOff;              // nv + 1
  int* watchOff;             // nv + 1
  int* watchPartner;         // wcap
  int* watchItem;            // wcap
  int* pairI;                // pcap
  int* pairJ;
  float* pairStiff;
  float* pairDamp;
  float* pairForce;          // 3 pcap
  int pcap, wcap;
  double cell;               // hash cell edge
  double thr;                // watch radius squared (float value promoted)
  double recalc2;            // recalc distance squared (float value promoted)
  ColCtl* cc;
  vx64::Ctl* ctl;
};

__device__ __forceinline__ unsigned long long cell_key(long long cx, long long cy, long long cz) {
  const long long B = 1ll << 20;
  return ((unsigned long long)((cx + B) & 0x1FFFFF) << 42) | ((unsigned long long)((cy + B) & 0x1FFFFF) << 21) |
         (unsigned long long)((cz + B) & 0x1FFFFF);
}
__device__ __forceinline__ unsigned long long hash64(unsigned long long k) {
  k ^= k >> 33;
  k *= 0xff51afd7ed558ccdull;
  k ^= k >> 33;
  k *= 0xc4ceb9fe1a85ec53ull;
  k ^= k >> 33;
  return k;
}
__device__ __forceinline__ bool is_surface(const ColView& C, int v) { return !(C.vflags[v] & VXG_VF_INTERIOR); }

// component k of voxel v's position in double: the FP64 state, or the FP32C state converted
// exactly as a host read converts it (lattice origin + (d - c))
__device__ __forceinline__ double cpos(const ColView& C, int v, int k) {
  if (!C.fp32) return C.pos[k * C.nv + v];
  float d = reinterpret_cast<const float*>(&C.P32[v])[k];
  return C.vidx[k * C.nv + v] * C.s64 + ((double)d - (double)C.c32[k * C.nv + v]);
}

// one store of the stale word per block (a falling body moves most voxels past the threshold at
// once, and a store from each of their warps to one address would serialise)
// whether surface voxel v moved more than the rebuild distance since the last rebuild
__device__ __forceinline__ bool c_moved(const ColView& C, int v) {
  if (v >= C.nv || !is_surface(C, v)) return false;
  double dx = cpos(C, v, 0) - C.lastWatch[v], dy = cpos(C, v, 1) - C.lastWatch[C.nv + v],
         dz = cpos(C, v, 2) - C.lastWatch[2 * C.nv + v];
  return dx * dx + dy * dy + dz * dz > C.recalc2;
}
// The surface voxels as a dense list: a warp ballot of the interior flags, one atomic per warp for
// the list slots.  The list's order varies from run to run; every use of it writes per voxel (and
// the rebuild sorts what it collects), so results do not depend on it.  Interior voxels' partner
// counts are zeroed here, since the rebuild visits listed voxels only.
__global__ void c_surface(ColView C) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  const bool live = v < C.nv;
  const bool surf = live && is_surface(C, v);
  if (live && !surf) {
    C.cntAll[v] = 0;
    C.cntGt[v] = 0;
  }
  const unsigned m = __ballot_sync(0xffffffffu, surf);
  if (!m) return;
  const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(&C.cc->nsurf, __popc(m));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (surf) C.surf[base + __popc(m & ((1u << lane) - 1u))] = v;
}
// first step of a batch: the full stale test over the surface list; later steps: the vote the
// previous step's voxel pass cast (slot parity ^ 1).  Either way this step's slot is cleared for
// its own voxel pass.
__device__ __forceinline__ bool c_moved_listed(const ColView& C, int first, int stride) {
  bool moved = false;
  const int n = C.cc->nsurf;
  for (int i = first; i < n; i += stride) moved |= c_moved(C, C.surf[i]);
  return moved;
}
__global__ void c_check(ColView C, int full, int parity) {
  if (C.ctl->halt || C.ctl->diverged) return;  // the same for the whole launch
  const int first = blockIdx.x * blockDim.x + threadIdx.x;
  if (first == 0) {
    if (C.cc->force_stale || (!full && C.cc->vote[parity ^ 1])) C.cc->stale = 1;
    C.cc->vote[parity] = 0;
  }
  if (full && __syncthreads_or(c_moved_listed(C, first, gridDim.x * blockDim.x)) && threadIdx.x == 0) C.cc->stale = 1;
}

// rebuild only when c_check found the list stale and the step has not diverged (the same for
// every thread of a launch: nothing writes these words while a rebuild kernel runs)
__device__ __forceinline__ bool c_rebuilding(const ColView& C) {
  return C.cc->stale && !C.ctl->halt && !C.ctl->diverged;
}
__device__ __forceinline__ void c_clear_range(const ColView& C, unsigned long long first, unsigned long long stride) {
  for (unsigned long long i = first; i <= C.hcap_mask; i += stride) {
    C.hkey[i] = ~0ull;
    C.hhead[i] = -1;
  }
}
__global__ void c_clear(ColView C) {
  if (!c_rebuilding(C)) return;
  c_clear_range(C, blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x, (unsigned long long)gridDim.x * blockDim.x);
}


// each surface voxel's position and cell, computed once per rebuild: the pair tests then read
// them instead of rebuilding both positions (FP64 arithmetic, slow on GB300) for every candidate
__device__ void c_insert_one(const ColView& C, int v) {
  if (v >= C.nv || !is_surface(C, v)) return;
  const int nv = C.nv;
  const double p0 = cpos(C, v, 0), p1 = cpos(C, v, 1), p2 = cpos(C, v, 2);
  C.lastWatch[v] = (float)p0;
  C.lastWatch[nv + v] = (float)p1;
  C.lastWatch[2 * nv + v] = (float)p2;
  C.spos[v] = p0;
  C.spos[nv + v] = p1;
  C.spos[2 * nv + v] = p2;
  long long c[3];
  c[0] = (long long)floor(p0 / C.cell);
  c[1] = (long long)floor(p1 / C.cell);
  c[2] = (long long)floor(p2 / C.cell);
  C.scell[v] = (int)c[0];
  C.scell[nv + v] = (int)c[1];
  C.scell[2 * nv + v] = (int)c[2];
  unsigned long long k = cell_key(c[0], c[1], c[2]);
  unsigned long long h = hash64(k) & C.hcap_mask;
  for (unsigned long long probe = 0; probe <= C.hcap_mask; ++probe) {
    unsigned long long prev = atomicCAS(&C.hkey[h], ~0ull, k);
    if (prev == ~0ull || prev == k) {
      C.next[v] = atomicExch(&C.hhead[h], v);
      return;
    }
    h = (h + 1) & C.hcap_mask;
  }
  atomicOr(&C.cc->status, VXG_COL_ST_HASH_FULL);
}
__global__ void c_insert(ColView C) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (c_rebuilding(C) && i < C.cc->nsurf) c_insert_one(C, C.surf[i]);
}

__device__ __forceinline__ int find_cell(const ColView& C, unsigned long long k) {
  unsigned long long h = hash64(k) & C.hcap_mask;
  for (unsigned long long probe = 0; probe <= C.hcap_mask; ++probe) {
    unsigned long long cur = C.hkey[h];
    if (cur == k) return C.hhead[h];
    if (cur == ~0ull) return -1;
    h = (h + 1) & C.hcap_mask;
  }
  return -1;
}

__device__ __forceinline__ bool in_sorted(const int* a, int n, int x) {
  int lo = 0, hi = n;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (a[mid] < x) lo = mid + 1;
    else hi = mid;
  }
  return lo < n && a[lo] == x;
}

// is (v, u) a collision pair of regenerateCollisions (Voxelyze.cpp:735-745)?
__device__ __forceinline__ bool is_pair(const ColView& C, int v, int u) {
  int i = v < u ? v : u, j = v < u ? u : v;
  const int nv = C.nv;
  double dx = C.spos[i] - C.spos[j], dy = C.spos[nv + i] - C.spos[nv + j], dz = C.spos[2 * nv + i] - C.spos[2 * nv + j];
  if (dx * dx + dy * dy + dz * dz > C.thr) return false;
  int b = C.nbOff[i], e = C.nbOff[i + 1];
  return !in_sorted(C.nbItem + b, e - b, j);
}

__global__ void c_count(ColView C);

// exclusive scans of cntGt -> pairOff and cntAll -> watchOff by one block of up to 1024 threads
// (rebuilds are rare)
__device__ void c_scan_block(const ColView& C) {
  __shared__ int sg[1024], sa[1024];
  int t = threadIdx.x, T = blockDim.x;
  int chunk = (C.nv + T - 1) / T;
  int b = t * chunk, e = min(C.nv, b + chunk);
  int g = 0, a = 0;
  for (int i = b; i < e; ++i) { g += C.cntGt[i]; a += C.cntAll[i]; }
  sg[t] = g;
  sa[t] = a;
  __syncthreads();
  for (int o = 1; o < T; o <<= 1) {
    int vg = t >= o ? sg[t - o] : 0, va = t >= o ? sa[t - o] : 0;
    __syncthreads();
    sg[t] += vg;
    sa[t] += va;
    __syncthreads();
  }
  int pg = sg[t] - g, pa = sa[t] - a;
  for (int i = b; i < e; ++i) {
    C.pairOff[i] = pg;
    C.watchOff[i] = pa;
    pg += C.cntGt[i];
    pa += C.cntAll[i];
  }
  if (t == T - 1) {
    C.pairOff[C.nv] = sg[t];
    C.watchOff[C.nv] = sa[t];
    C.cc->npairs = sg[t];
    C.cc->nwatch = sa[t];
    if (sg[t] > C.pcap) atomicOr(&C.cc->status, VXG_COL_ST_PAIR_OVERFLOW);
    if (sa[t] > C.wcap) atomicOr(&C.cc->status, VXG_COL_ST_WATCH_OVERFLOW);
  }
}
__global__ void c_scan(ColView C) {
  if (c_rebuilding(C)) c_scan_block(C);
}

__global__ void c_fill(ColView C);

__global__ void c_watch(ColView C);

// ---- warp-cooperative rebuild phases ------------------------------------------------------------
// One warp per surface voxel v.  Lane k < 27 walks the list of the k-th cell around v's, so the 27
// list walks and their pair tests (distance, then a binary search of the nearby list) run side by
// side instead of one after another; lanes 27-31 only take part in the warp reductions.  Every
// warp-collective call below is reached by all 32 lanes.
template <class F>
__device__ __forceinline__ void warp_partners(const ColView& C, int v, int lane, F&& f) {
  if (lane >= 27) return;
  const long long c[3] = {C.scell[v], C.scell[C.nv + v], C.scell[2 * C.nv + v]};
  const int dz = lane / 9 - 1, dy = (lane / 3) % 3 - 1, dx = lane % 3 - 1;
  for (int u = find_cell(C, cell_key(c[0] + dx, c[1] + dy, c[2] + dz)); u >= 0; u = C.next[u])
    if (u != v && is_pair(C, v, u)) f(u);
}
__device__ __forceinline__ int warp_sum(int x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}
__device__ __forceinline__ int warp_excl_scan(int x, int lane) {
  int y = x;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, y, o);
    if (lane >= o) y += t;
  }
  return y - x;
}
__device__ void c_count_warp(const ColView& C, int v, int lane) {
  int all = 0, gt = 0;
  if (is_surface(C, v)) warp_partners(C, v, lane, [&](int u) { all++; gt += u > v; });
  // each lane's own count, for the fill phase's offsets (a count over 255 means more partners than
  // the fill phase accepts in total; it then reports the overflow)
  C.lcnt[(size_t)v * 32 + lane] = (unsigned char)min(all, 255);
  all = warp_sum(all);
  gt = warp_sum(gt);
  if (lane == 0) {
    C.cntAll[v] = all;
    C.cntGt[v] = gt;
  }
}
// v's partners, ascending, into the contact list and (for partners after v) the pair list.  The
// lanes' partners are packed into the warp's shared buffer (exclusive scan of the lane counts the
// count phase stored), then each element's place is its rank among them (the partners are
// distinct voxels).
__device__ void c_fill_warp(const ColView& C, int v, int lane, int* sbuf /* kMaxPartners, this warp's */) {
  if (!is_surface(C, v)) return;  // the same for the whole warp
  const int mine = C.lcnt[(size_t)v * 32 + lane];  // what this lane found in the count phase
  const int off = warp_excl_scan(mine, lane), n = warp_sum(mine);
  if (n > kMaxPartners) {
    if (lane == 0) atomicOr(&C.cc->status, VXG_COL_ST_LOCAL_OVERFLOW);
    return;
  }
  int k = off;
  warp_partners(C, v, lane, [&](int u) { sbuf[k++] = u; });
  __syncwarp();
  int less = 0;  // partners before v in index order
  for (int i = lane; i < n; i += 32) less += sbuf[i] < v;
  const int nLess = warp_sum(less);
  const int wo = C.watchOff[v], po = C.pairOff[v];
  const vxg_voxel_material& m1 = C.vm[C.vmat[v]];
  for (int i = lane; i < n; i += 32) {
    const int u = sbuf[i];
    int r = 0;
    for (int j = 0; j < n; ++j) r += sbuf[j] < u;
    C.watchPartner[wo + r] = u;
    if (u > v) {
      const vxg_voxel_material& m2 = C.vm[C.vmat[u]];
      const int c = po + (r - nLess);
      C.pairI[c] = v;
      C.pairJ[c] = u;
      // CVX_Collision::CVX_Collision  VX_Collision.cpp:17-23
      C.pairStiff[c] = 2.0f / (1.0f / m1.penetrationStiffness + 1.0f / m2.penetrationStiffness);
      C.pairDamp[c] = 0.5f * (m1.zetaCollision * m1.c2xSqMxExS + m2.zetaCollision * m2.c2xSqMxExS);
    }
  }
  __syncwarp();  // the buffer is reused by this warp's next voxel
}
// each partner's pair index in v's contact list, the partners of one voxel side by side
__device__ void c_watch_warp(const ColView& C, int v, int lane) {
  const int wo = C.watchOff[v], n = C.cntAll[v];
  const int nLess = n - C.cntGt[v];
  for (int k = lane; k < n; k += 32) {
    const int u = C.watchPartner[wo + k];
    int item;
    if (u > v) {
      item = (C.pairOff[v] + (k - nLess)) * 2;
    } else {
      const int uo = C.watchOff[u], ul = C.cntAll[u] - C.cntGt[u];
      const int* seg = C.watchPartner + uo + ul;
      int lo = 0, hi = C.cntGt[u];
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (seg[mid] < v) lo = mid + 1;
        else hi = mid;
      }
      item = (C.pairOff[u] + lo) * 2 + 1;
    }
    C.watchItem[wo + k] = item;
  }
}
// the surface list's voxels, one per warp, warps striding over the list
#define C_FOR_SURFACE_WARP(C, first_thread, threads, body)                                         \
  do {                                                                                           \
    const int lane_ = threadIdx.x & 31;                                                          \
    const int ns_ = (C).cc->nsurf;                                                               \
    for (int i_ = (first_thread) >> 5; i_ < ns_; i_ += (threads) >> 5) {                         \
      const int v_ = (C).surf[i_];                                                               \
      body(v_, lane_);                                                                           \
    }                                                                                            \
  } while (0)

__global__ void c_count(ColView C) {
  if (!c_rebuilding(C)) return;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  C_FOR_SURFACE_WARP(C, t, gridDim.x * blockDim.x, [&](int v, int lane) { c_count_warp(C, v, lane); });
}
__global__ void __launch_bounds__(256) c_fill(ColView C) {
  __shared__ int sbuf[8][kMaxPartners];
  if (!c_rebuilding(C) || C.cc->status) return;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  C_FOR_SURFACE_WARP(C, t, gridDim.x * blockDim.x, [&](int v, int lane) { c_fill_warp(C, v, lane, sbuf[threadIdx.x >> 5]); });
}
__global__ void c_watch(ColView C) {
  if (!c_rebuilding(C) || C.cc->status) return;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  C_FOR_SURFACE_WARP(C, t, gridDim.x * blockDim.x, [&](int v, int lane) { c_watch_warp(C, v, lane); });
}

// Exclusive scans of cntGt -> pairOff and cntAll -> watchOff over all voxels by the whole grid of a
// cooperative launch (256 threads per block): each block sums its contiguous share, a grid barrier,
// then each block adds the totals of the blocks before it and scans its share in coalesced tiles.
// Leaves the totals (pair and contact-list counts, overflow bits) in the control words; the caller
// puts a grid barrier after it.
__device__ __forceinline__ int block_sum256(int x, int* sh /* 8 */) {
  x = warp_sum(x);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = x;
  __syncthreads();
  int r = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) r += sh[k];
  return r;
}
// exclusive scan across the block; *total = the block's sum
__device__ __forceinline__ int block_excl_scan256(int x, int* sh /* 8 */, int* total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int e = warp_excl_scan(x, lane);
  __syncthreads();
  if (lane == 31) sh[w] = e + x;
  __syncthreads();
  int before = 0, all = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    before += k < w ? sh[k] : 0;
    all += sh[k];
  }
  *total = all;
  return before + e;
}
__device__ void c_scan_grid(const ColView& C, cooperative_groups::grid_group& grid) {
  __shared__ int sh[8];
  const int nv = C.nv, G = gridDim.x, b = blockIdx.x, t = threadIdx.x;
  const int chunk = (nv + G - 1) / G;
  const int lo = min(nv, b * chunk), hi = min(nv, lo + chunk);
  int g = 0, a = 0;
  for (int i = lo + t; i < hi; i += blockDim.x) {
    g += C.cntGt[i];
    a += C.cntAll[i];
  }
  g = block_sum256(g, sh);
  a = block_sum256(a, sh);
  if (t == 0) {
    C.part[2 * b] = g;
    C.part[2 * b + 1] = a;
  }
  grid.sync();
  int og = 0, oa = 0;
  for (int k = t; k < b; k += blockDim.x) {
    og += C.part[2 * k];
    oa += C.part[2 * k + 1];
  }
  og = block_sum256(og, sh);
  oa = block_sum256(oa, sh);
  for (int base = lo; base < hi; base += blockDim.x) {
    const int i = base + t;
    const int xg = i < hi ? C.cntGt[i] : 0, xa = i < hi ? C.cntAll[i] : 0;
    int tg, ta;
    const int eg = block_excl_scan256(xg, sh, &tg);
    const int ea = block_excl_scan256(xa, sh, &ta);
    if (i < hi) {
      C.pairOff[i] = og + eg;
      C.watchOff[i] = oa + ea;
    }
    og += tg;
    oa += ta;
  }
  if (b == G - 1 && t == 0) {  // the last block's running offsets are the totals
    C.pairOff[nv] = og;
    C.watchOff[nv] = oa;
    C.cc->npairs = og;
    C.cc->nwatch = oa;
    if (og > C.pcap) atomicOr(&C.cc->status, VXG_COL_ST_PAIR_OVERFLOW);
    if (oa > C.wcap) atomicOr(&C.cc->status, VXG_COL_ST_WATCH_OVERFLOW);
  }
}

// The whole rebuild in one cooperative launch: the phases above, separated by grid-wide barriers
// (a cooperative launch keeps every block resident, so the barriers end).  When the list is not
// stale every block returns at once, so a step pays one launch instead of six.
__global__ void __launch_bounds__(256) c_rebuild(ColView C) {
  __shared__ int sbuf[8][kMaxPartners];  // c_fill_warp's buffer, one per warp
  if (!c_rebuilding(C)) return;  // uniform: no block reaches a barrier unless all do
  cooperative_groups::grid_group grid = cooperative_groups::this_grid();
  const int first = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
  const int ns = C.cc->nsurf;
  c_clear_range(C, first, stride);
  grid.sync();
  for (int i = first; i < ns; i += stride) c_insert_one(C, C.surf[i]);
  grid.sync();
  C_FOR_SURFACE_WARP(C, first, stride, [&](int v, int lane) { c_count_warp(C, v, lane); });
  grid.sync();
  c_scan_grid(C, grid);
  grid.sync();
  if (C.cc->status) return;  // written before the last barrier: the same for every block
  C_FOR_SURFACE_WARP(C, first, stride, [&](int v, int lane) { c_fill_warp(C, v, lane, sbuf[threadIdx.x >> 5]); });
  grid.sync();
  if (C.cc->status) return;
  C_FOR_SURFACE_WARP(C, first, stride, [&](int v, int lane) { c_watch_warp(C, v, lane); });
}

// CVX_Voxel::baseSizeAverage for the envelope  VX_Voxel.h:90
__device__ __forceinline__ double col_bsa(const ColView& C, int v) {
  const vxg_voxel_material& m = C.vm[C.vmat[v]];
  float f = 1 + C.temp[v] * m.alphaCTE;
  return ((double)f * m.size[0] + (double)f * m.size[1] + (double)f * m.size[2]) / 3.0f;
}

// CVX_Collision::updateContactForce (VX_Collision.cpp:42-56) on the FP32C state, in FP32: the
// offset between the two voxels is the exact lattice offset plus the difference of their
// compensated displacements, so no two nearly equal absolute positions are subtracted
__device__ __forceinline__ float3 c_off32(const ColView& C, int a, int b) {
  const int nv = C.nv;
  float4 da = C.P32[a], db = C.P32[b];
  float r[3];
  const float dd[3] = {db.x - da.x, db.y - da.y, db.z - da.z};
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    float lat = (float)(C.vidx[k * nv + b] - C.vidx[k * nv + a]) * C.s32;
    float dc = C.c32[k * nv + b] - C.c32[k * nv + a];
    r[k] = lat + (dd[k] - dc);
  }
  return make_float3(r[0], r[1], r[2]);
}
__device__ __forceinline__ float col_bsa32(const ColView& C, int v) {
  const vxg_voxel_material& m = C.vm[C.vmat[v]];
  return m.sizeAvgF * (1 + C.temp[v] * m.alphaCTE);
}
__device__ void c_contact32(const ColView& C, int c, int a, int b) {
  const int nv = C.nv;
  float3 o = c_off32(C, a, b);
  float nom = (col_bsa32(C, a) + col_bsa32(C, b)) * 0.625f;
  float len = sqrtf(o.x * o.x + o.y * o.y + o.z * o.z);
  float rel = nom - len;
  float fx = 0, fy = 0, fz = 0;
  if (rel > 0) {
    float ux = o.x, uy = o.y, uz = o.z;
    if (len > 0) {
      float inv = 1.0f / len;
      ux = inv * o.x; uy = inv * o.y; uz = inv * o.z;
    }
    const vxg_voxel_material& m1 = C.vm[C.vmat[a]];
    const vxg_voxel_material& m2 = C.vm[C.vmat[b]];
    float v1x = m1.massInv * C.lin32[a], v1y = m1.massInv * C.lin32[nv + a], v1z = m1.massInv * C.lin32[2 * nv + a];
    float v2x = m2.massInv * C.lin32[b], v2y = m2.massInv * C.lin32[nv + b], v2z = m2.massInv * C.lin32[2 * nv + b];
    float relVel = (v1x * ux + v1y * uy + v1z * uz) - (v2x * ux + v2y * uy + v2z * uz);
    float k = C.pairStiff[c] * rel + C.pairDamp[c] * relVel;
    fx = ux * k; fy = uy * k; fz = uz * k;
  }
  C.pairForce[3 * c] = fx;
  C.pairForce[3 * c + 1] = fy;
  C.pairForce[3 * c + 2] = fz;
}

// CVX_Collision::updateContactForce  VX_Collision.cpp:42-56, one pair per thread of a resident grid
// (the pair count is known only on the device)
__device__ __forceinline__ void c_contact64(const ColView& C, int c, int a, int b);
// the contact forces of every listed pair, thread t of `threads`; thread 0 also closes the step's
// bookkeeping (rebuild count, stale words, status to the control block)
__device__ __forceinline__ void c_contact_all(const ColView& C, int t, int threads, bool rebuilt) {
  const int npairs = C.cc->npairs, status = C.cc->status;  // thread 0 clears neither
  if (t == 0) {
    if (rebuilt) C.cc->rebuilds += 1;
    C.cc->stale = 0;
    C.cc->force_stale = 0;
    if (status) atomicOr(&C.ctl->status, status << 8);
  }
  if (status) return;
  for (int c = t; c < npairs; c += threads) {
    int a = C.pairI[c], b = C.pairJ[c];
    if (C.fp32) c_contact32(C, c, a, b);
    else c_contact64(C, c, a, b);
  }
}
__global__ void c_contact(ColView C) {
  if (C.ctl->halt || C.ctl->diverged) return;
  c_contact_all(C, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x, C.cc->stale != 0);
}

// The whole stage in one cooperative launch: the stale test, the rebuild phases when it found the
// list stale, the contact forces, separated by grid-wide barriers (a cooperative launch keeps
// every block resident, so the barriers end; every branch around a barrier reads words that
// were written before the previous barrier, so all blocks take it alike).
// full: the first step of a batch (the stale test over the surface list, then a grid barrier);
// otherwise the vote of the previous step's voxel pass decides, read by every block from words no
// block of this launch writes before the decision is taken (force_stale is cleared only at the end,
// after the rebuild's barriers when it was set; vote[parity ^ 1] not at all), so all blocks take
// the same branch, and a step with nothing stale passes no barrier.
__global__ void __launch_bounds__(256) c_stage(ColView C, int full, int parity) {
  __shared__ int sbuf[8][kMaxPartners];  // c_fill_warp's buffer, one per warp
  if (C.ctl->halt || C.ctl->diverged) return;  // uniform: set before this launch
  cooperative_groups::grid_group grid = cooperative_groups::this_grid();
  const int first = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
  const int ns = C.cc->nsurf;
  bool stale;
  if (full) {
    if (first == 0) {
      if (C.cc->force_stale) C.cc->stale = 1;
      C.cc->vote[parity] = 0;
    }
    if (__syncthreads_or(c_moved_listed(C, first, stride)) && threadIdx.x == 0) C.cc->stale = 1;
    grid.sync();
    stale = C.cc->stale != 0;
  } else {
    stale = C.cc->force_stale || C.cc->vote[parity ^ 1];
    if (first == 0) C.cc->vote[parity] = 0;
  }
  if (stale) {
    c_clear_range(C, first, stride);
    grid.sync();
    for (int i = first; i < ns; i += stride) c_insert_one(C, C.surf[i]);
    grid.sync();
    C_FOR_SURFACE_WARP(C, first, stride, [&](int v, int lane) { c_count_warp(C, v, lane); });
    grid.sync();
    c_scan_grid(C, grid);
    grid.sync();
    if (!C.cc->status)
      C_FOR_SURFACE_WARP(C, first, stride, [&](int v, int lane) { c_fill_warp(C, v, lane, sbuf[threadIdx.x >> 5]); });
    grid.sync();
    if (!C.cc->status)
      C_FOR_SURFACE_WARP(C, first, stride, [&](int v, int lane) { c_watch_warp(C, v, lane); });
    grid.sync();
  }
  c_contact_all(C, first, stride, stale);
}
__device__ __forceinline__ void c_contact64(const ColView& C, int c, int a, int b) {
  const int nv = C.nv;
  float ox = (float)(C.pos[b] - C.pos[a]), oy = (float)(C.pos[nv + b] - C.pos[nv + a]),
        oz = (float)(C.pos[2 * nv + b] - C.pos[2 * nv + a]);
  float nom = (float)((col_bsa(C, a) + col_bsa(C, b)) * 0.625f);
  float rel = nom - sqrtf(ox * ox + oy * oy + oz * oz);
  float fx = 0, fy = 0, fz = 0;
  if (rel > 0) {
    float l = sqrtf(ox * ox + oy * oy + oz * oz);
    float ux = ox, uy = oy, uz = oz;
    if (l > 0) {
      float inv = (float)1.0 / l;
      ux = inv * ox; uy = inv * oy; uz = inv * oz;
    }
    const vxg_voxel_material& m1 = C.vm[C.vmat[a]];
    const vxg_voxel_material& m2 = C.vm[C.vmat[b]];
    double v1x = m1.massInv * C.linMom[a], v1y = m1.massInv * C.linMom[nv + a], v1z = m1.massInv * C.linMom[2 * nv + a];
    double v2x = m2.massInv * C.linMom[b], v2y = m2.massInv * C.linMom[nv + b], v2z = m2.massInv * C.linMom[2 * nv + b];
    float relVel = (float)((v1x * (double)ux + v1y * (double)uy + v1z * (double)uz) -
                           (v2x * (double)ux + v2y * (double)uy + v2z * (double)uz));
    float k = C.pairStiff[c] * rel + C.pairDamp[c] * relVel;
    fx = ux * k; fy = uy * k; fz = uz * k;
  }
  C.pairForce[3 * c] = fx;
  C.pairForce[3 * c + 1] = fy;
  C.pairForce[3 * c + 2] = fz;
}

struct Collide {
  ColView C{};
  ColCtl* cc = nullptr;
  char* buf = nullptr;
  size_t buf_bytes = 0;
  int* d_nb = nullptr;  // nearby CSR storage (offsets then items)
  int nv = 0;
  int pcap = 0, wcap = 0;
  int grid_pairs = 1;

  void release() {
    if (buf) cudaFree(buf);
    if (d_nb) cudaFree(d_nb);
    if (cc) cudaFree(cc);
    buf = nullptr;
    d_nb = nullptr;
    cc = nullptr;
  }
  // scene size changed: buffers are (re)allocated when collisions are first used (set_nearby)
  int resize(int n) {
    if (buf) cudaFree(buf);
    buf = nullptr;
    if (d_nb) cudaFree(d_nb);
    d_nb = nullptr;
    C.nbOff = C.nbItem = nullptr;
    C.watchOff = C.watchItem = nullptr;
    C.pairForce = nullptr;
    nv = n;
    coop_blocks = -1;
    stage_blocks = -1;
    if (!cc) {
      if (cudaMalloc(&cc, sizeof(ColCtl)) != cudaSuccess) return VXG_E_CUDA;
    }
    if (cudaMemset(cc, 0, sizeof(ColCtl)) != cudaSuccess) return VXG_E_CUDA;
    return VXG_OK;
  }
  int allocate() {
    int n = nv;
    unsigned long long hcap = 1024;
    while (hcap < 2ull * (unsigned long long)n) hcap <<= 1;
    pcap = std::max(1024, 32 * n);
    wcap = 2 * pcap;
    size_t bytes = 0;
    auto take = [&](size_t b) { size_t o = bytes; bytes += (b + 255) / 256 * 256; return o; };
    size_t o_last = take(sizeof(float) * 3 * (size_t)n);
    size_t o_hkey = take(8 * hcap), o_hhead = take(4 * hcap);
    size_t o_next = take(4 * (size_t)n), o_cg = take(4 * (size_t)n), o_ca = take(4 * (size_t)n);
    size_t o_surf = take(4 * (size_t)n), o_spos = take(24 * (size_t)n), o_scell = take(12 * (size_t)n);
    size_t o_lcnt = take(32 * (size_t)n), o_part = take(8 * (size_t)kScanBlocks);
    size_t o_po = take(4 * ((size_t)n + 1)), o_wo = take(4 * ((size_t)n + 1));
    size_t o_wp = take(4 * (size_t)wcap), o_wi = take(4 * (size_t)wcap);
    size_t o_pi = take(4 * (size_t)pcap), o_pj = take(4 * (size_t)pcap), o_ps = take(4 * (size_t)pcap),
           o_pd = take(4 * (size_t)pcap), o_pf = take(12 * (size_t)pcap);
    if (n == 0) return VXG_OK;
    if (cudaMalloc(&buf, bytes) != cudaSuccess) return VXG_E_CUDA;
    buf_bytes = bytes;
    if (cudaMemset(buf, 0, bytes) != cudaSuccess) return VXG_E_CUDA;
    C.nv = n;
    C.hcap_mask = hcap - 1;
    C.lastWatch = (float*)(buf + o_last);
    C.hkey = (unsigned long long*)(buf + o_hkey);
    C.hhead = (int*)(buf + o_hhead);
    C.next = (int*)(buf + o_next);
    C.cntGt = (int*)(buf + o_cg);
    C.cntAll = (int*)(buf + o_ca);
    C.surf = (int*)(buf + o_surf);
    C.spos = (double*)(buf + o_spos);
    C.scell = (int*)(buf + o_scell);
    C.lcnt = (unsigned char*)(buf + o_lcnt);
    C.part = (int*)(buf + o_part);
    C.pairOff = (int*)(buf + o_po);
    C.watchOff = (int*)(buf + o_wo);
    C.watchPartner = (int*)(buf + o_wp);
    C.watchItem = (int*)(buf + o_wi);
    C.pairI = (int*)(buf + o_pi);
    C.pairJ = (int*)(buf + o_pj);
    C.pairStiff = (float*)(buf + o_ps);
    C.pairDamp = (float*)(buf + o_pd);
    C.pairForce = (float*)(buf + o_pf);
    C.pcap = pcap;
    C.wcap = wcap;
    C.cc = cc;
    int dev = 0, n_sm = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
    grid_pairs = std::max(1, std::min((pcap + 255) / 256, 4 * n_sm));
    return VXG_OK;
  }
  int set_nearby(int n, const int* off, const int* items, long long n_items, cudaStream_t s) {
    if (n != nv) return VXG_E_SIZE;
    if (!buf) {
      int rc = allocate();
      if (rc) return rc;
    }
    if (d_nb) cudaFree(d_nb);
    d_nb = nullptr;
    size_t tot = (size_t)(n + 1) + (size_t)std::max<long long>(n_items, 1);
    if (cudaMalloc(&d_nb, 4 * tot) != cudaSuccess) return VXG_E_CUDA;
    if (cudaMemcpyAsync(d_nb, off, 4 * (size_t)(n + 1), cudaMemcpyHostToDevice, s) != cudaSuccess) return VXG_E_CUDA;
    if (n_items > 0 &&
        cudaMemcpyAsync(d_nb + n + 1, items, 4 * (size_t)n_items, cudaMemcpyHostToDevice, s) != cudaSuccess)
      return VXG_E_CUDA;
    int one = 1;
    if (cudaMemcpyAsync(&cc->force_stale, &one, 4, cudaMemcpyHostToDevice, s) != cudaSuccess) return VXG_E_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return VXG_E_CUDA;
    C.nbOff = d_nb;
    C.nbItem = d_nb + n + 1;
    return VXG_OK;
  }
  // FP32C engines: the collision stage reads the FP32C state (bind32 after bind)
  void bind32(const vx32::View& V) {
    C.fp32 = 1;
    C.P32 = V.P;
    C.c32 = V.c;
    C.lin32 = V.lin;
    C.vidx = V.B.vidx;
  }
  void bind(View& S) {
    C.fp32 = 0;
    C.pos = S.pos;
    C.linMom = S.linMom;
    C.vmat = S.vmat;
    C.vflags = S.vflags;
    C.temp = S.temp;
    C.vm = S.vm;
    C.ctl = S.ctl;
    S.colOff = C.watchOff;
    S.colItem = C.watchItem;
    S.colForce = C.pairForce;
    S.colVote = nullptr;  // set per launch when collisions are on (voted())
    S.colLast = C.lastWatch;
  }
  // the View a voxel pass gets when collisions are on: it votes for the next step's stage
  bool ready() const { return buf && C.nbOff; }
  void voted(View& S, const vxg_globals& g, int parity) {
    set_globals(g);
    S.colVote = ready() ? &cc->vote[parity & 1] : nullptr;
    S.colLast = C.lastWatch;
    S.colRecalc2 = C.recalc2;
    S.colS = C.s64;
  }
  // once per batch: the surface list the stage walks
  int enqueue_surface(cudaStream_t s) {
    if (!ready()) return 0;
    cudaMemsetAsync(&cc->nsurf, 0, sizeof(int), s);
    c_surface<<<std::max(1, (nv + 255) / 256), 256, 0, s>>>(C);
    return 1;
  }
  void set_globals(const vxg_globals& g) {
    float watchVx = 2 * g.boundingRadius + g.watchDistance;
    float watchMm = (float)(g.voxSize * watchVx);
    float recalc = (float)(g.voxSize * g.watchDistance / 2);
    C.thr = (double)(watchMm * watchMm);
    C.recalc2 = (double)(recalc * recalc);
    C.cell = (double)watchMm * 1.001;
    C.s64 = g.voxSize;
    C.s32 = (float)g.voxSize;
  }
  // the cooperative rebuild: blocks resident on the whole GPU (0: launch the six kernels instead)
  int coop_blocks = -1;
  int coop_grid() {
    if (coop_blocks < 0) {
      int dev = 0, n_sm = 1, coop = 0, per_sm = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
      cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
      if (coop && cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, c_rebuild, 256, 0) == cudaSuccess && per_sm > 0)
        coop_blocks = std::min(std::min(n_sm * per_sm, kScanBlocks), std::max(1, (nv + 255) / 256));
      else
        coop_blocks = 0;
      cudaGetLastError();
    }
    return coop_blocks;
  }
  // returns the number of kernels launched
  int enqueue_rebuild(cudaStream_t s) {
    const int gb = coop_grid();
    if (gb > 0) {
      void* args[] = {&C};
      if (cudaLaunchCooperativeKernel((const void*)c_rebuild, dim3(gb), dim3(256), args, 0, s) == cudaSuccess) return 1;
      cudaGetLastError();
      coop_blocks = 0;  // not available here: the separate kernels from now on
    }
    int gv = std::max(1, (nv + 255) / 256);
    c_clear<<<256, 256, 0, s>>>(C);
    c_insert<<<gv, 256, 0, s>>>(C);
    c_count<<<gv, 256, 0, s>>>(C);
    c_scan<<<1, 1024, 0, s>>>(C);
    c_fill<<<gv, 256, 0, s>>>(C);
    c_watch<<<gv, 256, 0, s>>>(C);
    return 6;
  }
  // Launches the stage on stream s; returns the number of kernels launched.  The rebuild exits at
  // once unless c_check found the pair list stale.  (A conditional graph node around separate
  // rebuild kernels measured slower than their early exits on GB300.)
  // the whole stage as one cooperative launch: blocks resident on the whole GPU (0: not available)
  int stage_blocks = -1;
  int stage_grid() {
    if (stage_blocks < 0) {
      int dev = 0, n_sm = 1, coop = 0, per_sm = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
      cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
      if (coop && cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, c_stage, 256, 0) == cudaSuccess && per_sm > 0)
        stage_blocks = std::min(std::min(n_sm * per_sm, kScanBlocks), std::max(1, (nv + 255) / 256));
      else
        stage_blocks = 0;
      cudaGetLastError();
    }
    return stage_blocks;
  }
  // full: the stale test itself (the first step of a batch or captured chunk); otherwise the vote
  // of the previous step's voxel pass
  int enqueue(const vxg_globals& g, cudaStream_t s, bool full, int parity) {
    if (!buf || !C.nbOff) return 0;
    set_globals(g);
    int fl = full ? 1 : 0, par = parity & 1;
    const int gs = stage_grid();
    if (gs > 0) {
      void* args[] = {&C, &fl, &par};
      if (cudaLaunchCooperativeKernel((const void*)c_stage, dim3(gs), dim3(256), args, 0, s) == cudaSuccess) return 1;
      cudaGetLastError();
      stage_blocks = 0;  // not available here: the separate kernels from now on
    }
    int gv = std::max(1, (nv + 255) / 256);
    c_check<<<gv, 256, 0, s>>>(C, fl, par);
    int n = enqueue_rebuild(s);
    c_contact<<<grid_pairs, 256, 0, s>>>(C);
    return 2 + n;
  }
  int get_pairs(int* out, int cap, int* n, cudaStream_t s) {
    *n = 0;
    if (!cc) return VXG_OK;
    ColCtl h;
    if (cudaMemcpyAsync(&h, cc, sizeof(h), cudaMemcpyDeviceToHost, s) != cudaSuccess) return VXG_E_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return VXG_E_CUDA;
    *n = h.npairs;
    int m = std::min(cap, h.npairs);
    if (m > 0 && out) {
      std::vector<int> a(m), b(m);
      if (cudaMemcpyAsync(a.data(), C.pairI, 4 * (size_t)m, cudaMemcpyDeviceToHost, s) != cudaSuccess) return VXG_E_CUDA;
      if (cudaMemcpyAsync(b.data(), C.pairJ, 4 * (size_t)m, cudaMemcpyDeviceToHost, s) != cudaSuccess) return VXG_E_CUDA;
      if (cudaStreamSynchronize(s) != cudaSuccess) return VXG_E_CUDA;
      for (int k = 0; k < m; ++k) { out[2 * k] = a[k]; out[2 * k + 1] = b[k]; }
    }
    return VXG_OK;
  }
  int rebuilds() {
    if (!cc) return 0;
    ColCtl h;
    cudaMemcpy(&h, cc, sizeof(h), cudaMemcpyDeviceToHost);
    return h.rebuilds;
  }
  int pairs(cudaStream_t) {
    if (!cc) return 0;
    ColCtl h;
    cudaMemcpy(&h, cc, sizeof(h), cudaMemcpyDeviceToHost);
    return h.npairs;
  }
  const char* status_message(int st) {
    int c = st >> 8;
    if (c & VXG_COL_ST_PAIR_OVERFLOW) return "collision pair list overflow";
    if (c & VXG_COL_ST_WATCH_OVERFLOW) return "collision contact list overflow";
    if (c & VXG_COL_ST_LOCAL_OVERFLOW) return "more than 128 collision partners for one voxel";
    if (c & VXG_COL_ST_HASH_FULL) return "collision hash table full";
    return "device status error";
  }
};
