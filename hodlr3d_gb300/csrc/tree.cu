// Device construction of the uniform octree: leaf keys, stable sort into tree
// order, leaf ranges, neighbour slots and interaction lists of every level.
//
// Reference: HODLR3D::HODLR3D (src/HODLR3D.cpp:3-15) -> createTree,
// assign_Tree_Interactions, assign_Center_Location, assignChargeLocations,
// assignNonLeafChargeLocations (src/HODLR3DTree.cpp:78-1619).
#include "common.cuh"
#include "tree.h"

namespace h3d {

struct Radii {
  double r[kMaxLevels + 1];
};

// Leaf of every point by the recursive octant comparison of
// assignChargeLocations (src/HODLR3DTree.cpp:1558-1608): at each level the
// point goes to the low side when equal to the box centre; the child centre
// is parent +- 0.5 * boxRadius[j] (assign_Center_Location :1518-1556).
__global__ void k_leaf_keys(int64_t n, const double* __restrict__ xyz, int levels, Radii rad,
                            uint32_t* __restrict__ keys, int32_t* __restrict__ vals) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
  double cx = 0.0, cy = 0.0, cz = 0.0;
  uint32_t k = 0;
  for (int j = 0; j < levels; ++j) {
    const double shift = __dmul_rn(0.5, rad.r[j]);
    const int bz = z <= cz ? 0 : 1;
    const int bx = x <= cx ? 0 : 1;
    const int by = y <= cy ? 0 : 1;
    k = 8u * k + (uint32_t)digit_of(bx, by, bz);
    cx = bx ? __dadd_rn(cx, shift) : __dsub_rn(cx, shift);
    cy = by ? __dadd_rn(cy, shift) : __dsub_rn(cy, shift);
    cz = bz ? __dadd_rn(cz, shift) : __dsub_rn(cz, shift);
  }
  keys[i] = k;
  vals[i] = (int32_t)i;
}

// ---- stable LSD radix sort, 8-bit digits, one warp per tile ---------------
constexpr int kSortTile = 1024;  // keys per warp tile (32 chunks of 32)

__global__ void k_radix_count(int64_t n, const uint32_t* __restrict__ keys, int shift,
                              int ntiles, int32_t* __restrict__ counts) {
  __shared__ int32_t hist[4][256];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int b = lane; b < 256; b += 32) hist[w][b] = 0;
  __syncwarp();
  const int tile = blockIdx.x * 4 + w;
  if (tile < ntiles) {
    const int64_t t0 = (int64_t)tile * kSortTile;
    for (int e = lane; e < kSortTile; e += 32) {
      const int64_t i = t0 + e;
      if (i < n) atomicAdd(&hist[w][(keys[i] >> shift) & 255u], 1);
    }
    __syncwarp();
    for (int b = lane; b < 256; b += 32) counts[(int64_t)b * ntiles + tile] = hist[w][b];
  }
}

// exclusive scan of m int32 values by one block of 1024 threads
__global__ void k_scan_exclusive(int64_t m, int32_t* __restrict__ data) {
  __shared__ int64_t part[1024];
  const int t = threadIdx.x;
  const int64_t per = (m + 1023) / 1024;
  const int64_t a = min(m, t * per), b = min(m, a + per);
  int64_t s = 0;
  for (int64_t i = a; i < b; ++i) s += data[i];
  part[t] = s;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    const int64_t v = t >= o ? part[t - o] : 0;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  int64_t run = part[t] - s;
  for (int64_t i = a; i < b; ++i) {
    const int64_t v = data[i];
    data[i] = (int32_t)run;
    run += v;
  }
}

__global__ void k_radix_scatter(int64_t n, const uint32_t* __restrict__ keys_in,
                                const int32_t* __restrict__ vals_in, int shift, int ntiles,
                                const int32_t* __restrict__ base, uint32_t* __restrict__ keys_out,
                                int32_t* __restrict__ vals_out) {
  __shared__ int32_t run[4][256];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tile = blockIdx.x * 4 + w;
  if (tile >= ntiles) return;
  for (int b = lane; b < 256; b += 32) run[w][b] = base[(int64_t)b * ntiles + tile];
  __syncwarp();
  const int64_t t0 = (int64_t)tile * kSortTile;
  const unsigned lt = (1u << lane) - 1u;
  for (int c = 0; c < kSortTile; c += 32) {
    const int64_t i = t0 + c + lane;
    const bool valid = i < n;
    const unsigned act = __ballot_sync(0xffffffffu, valid);
    if (!act) break;
    uint32_t key = 0;
    int32_t val = 0;
    int dig = 256 + lane;  // distinct dummy digits for invalid lanes
    if (valid) {
      key = keys_in[i];
      val = vals_in[i];
      dig = (int)((key >> shift) & 255u);
    }
    const unsigned peers = __match_any_sync(0xffffffffu, dig);
    const int rank = __popc(peers & lt);
    int pos = 0;
    if (valid) pos = run[w][dig] + rank;
    __syncwarp();
    if (valid) {
      keys_out[pos] = key;
      vals_out[pos] = val;
      if ((__ffs(peers) - 1) == lane) run[w][dig] += __popc(peers);
    }
    __syncwarp();
  }
}

// leaf_off[k] = first position with key >= k, k = 0..nleaf
__global__ void k_leaf_offsets(int64_t n, const uint32_t* __restrict__ keys, int64_t nleaf,
                               int32_t* __restrict__ leaf_off) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k > nleaf) return;
  int64_t lo = 0, hi = n;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if ((int64_t)keys[mid] < k) lo = mid + 1;
    else hi = mid;
  }
  leaf_off[k] = (int32_t)lo;
}

// centre of box k at level j by the same chain of additions as the reference
__device__ inline void box_centre(int j, int64_t k, const Radii& rad, double& cx, double& cy,
                                  double& cz) {
  cx = cy = cz = 0.0;
  for (int t = 0; t < j; ++t) {
    const int d = (int)((k >> (3 * (j - 1 - t))) & 7);
    const double shift = __dmul_rn(0.5, rad.r[t]);
    cx = digit_x(d) ? __dadd_rn(cx, shift) : __dsub_rn(cx, shift);
    cy = digit_y(d) ? __dadd_rn(cy, shift) : __dsub_rn(cy, shift);
    cz = digit_z(d) ? __dadd_rn(cz, shift) : __dsub_rn(cz, shift);
  }
}

// Sorted coordinates: FP64, and FP32 offsets from the leaf centre (the
// displacement between two points is then the exact FP64 centre difference
// plus a small FP32 offset difference).
__global__ void k_gather_points(int64_t n, const double* __restrict__ xyz,
                                const int32_t* __restrict__ perm,
                                const uint32_t* __restrict__ leaf_of, int levels, Radii rad,
                                double* __restrict__ xs, double* __restrict__ ys,
                                double* __restrict__ zs, float* __restrict__ xl,
                                float* __restrict__ yl, float* __restrict__ zl) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int64_t i = perm[t];
  const double x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
  xs[t] = x;
  ys[t] = y;
  zs[t] = z;
  double cx, cy, cz;
  box_centre(levels, leaf_of[t], rad, cx, cy, cz);
  xl[t] = (float)(x - cx);
  yl[t] = (float)(y - cy);
  zl[t] = (float)(z - cz);
}

__global__ void k_leaf_centres(int64_t nleaf, int levels, Radii rad, double* __restrict__ c) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= nleaf) return;
  box_centre(levels, k, rad, c[3 * k], c[3 * k + 1], c[3 * k + 2]);
}

__device__ inline void box_coords(int j, int64_t k, int& ix, int& iy, int& iz) {
  ix = iy = iz = 0;
  for (int t = j - 1; t >= 0; --t) {
    const int d = (int)((k >> (3 * t)) & 7);
    ix = 2 * ix + digit_x(d);
    iy = 2 * iy + digit_y(d);
    iz = 2 * iz + digit_z(d);
  }
}

__device__ inline int64_t box_id(int j, int ix, int iy, int iz) {
  int64_t k = 0;
  for (int t = j - 1; t >= 0; --t) k = 8 * k + digit_of((ix >> t) & 1, (iy >> t) & 1, (iz >> t) & 1);
  return k;
}

constexpr int kMaxIL = 152;  // 19 near parents x 8 children

// Neighbour slots and interaction list of every box of level j >= 1: the
// children of the parent's near boxes (itself and its face/edge neighbours;
// the reference never fills vertex slots, src/HODLR3DTree.cpp:123-125) are
// face/edge neighbours (slot 9(dz+1)+3(dy+1)+(dx+1), minus one above 13) or,
// otherwise, interaction-list entries (assign_Child0..7_Interaction,
// src/HODLR3DTree.cpp:111-1490).  Lists are written in ascending box order.
// mode 0: count only (il_count); mode 1: also write neighbours and pairs.
__global__ void k_box_lists(int j, int mode, int32_t* __restrict__ nbr_all,
                            int32_t* __restrict__ il_count, const int64_t* __restrict__ il_ptr,
                            int32_t* __restrict__ pair_tgt, int32_t* __restrict__ pair_src) {
  const int64_t nb = int64_t(1) << (3 * j);
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= nb) return;
  const int64_t gb = level_base(j) + k;
  int ix, iy, iz;
  box_coords(j, k, ix, iy, iz);
  const int px = ix >> 1, py = iy >> 1, pz = iz >> 1, pside = 1 << (j - 1);
  int32_t il[kMaxIL];
  int cnt = 0;
  int32_t nb26[26];
  for (int s = 0; s < 26; ++s) nb26[s] = -1;
  for (int ez = -1; ez <= 1; ++ez)
    for (int ey = -1; ey <= 1; ++ey)
      for (int ex = -1; ex <= 1; ++ex) {
        if (ex != 0 && ey != 0 && ez != 0) continue;
        const int qx = px + ex, qy = py + ey, qz = pz + ez;
        if (qx < 0 || qy < 0 || qz < 0 || qx >= pside || qy >= pside || qz >= pside) continue;
        for (int c = 0; c < 8; ++c) {
          const int bx = 2 * qx + digit_x(c), by = 2 * qy + digit_y(c), bz = 2 * qz + digit_z(c);
          const int dx = bx - ix, dy = by - iy, dz = bz - iz;
          if (dx == 0 && dy == 0 && dz == 0) continue;
          const int32_t b = (int32_t)box_id(j, bx, by, bz);
          const bool adj = abs(dx) <= 1 && abs(dy) <= 1 && abs(dz) <= 1 &&
                           !(dx != 0 && dy != 0 && dz != 0);
          if (adj) {
            int s = 9 * (dz + 1) + 3 * (dy + 1) + (dx + 1);
            if (s > 13) --s;
            nb26[s] = b;
          } else if (cnt < kMaxIL) {
            il[cnt++] = b;
          }
        }
      }
  if (mode == 0) {
    il_count[gb] = cnt;
    return;
  }
  for (int s = 0; s < 26; ++s) nbr_all[gb * 26 + s] = nb26[s];
  for (int a = 1; a < cnt; ++a) {  // insertion sort, at most 133 entries
    const int32_t v = il[a];
    int b = a - 1;
    while (b >= 0 && il[b] > v) {
      il[b + 1] = il[b];
      --b;
    }
    il[b + 1] = v;
  }
  const int64_t o = il_ptr[gb];
  for (int a = 0; a < cnt; ++a) {
    pair_tgt[o + a] = (int32_t)gb;
    pair_src[o + a] = (int32_t)(level_base(j) + il[a]);
  }
}

// The interaction relation is symmetric: for the pair q = (a, b) of box a the
// pair (b, a) sits in the list of box b; rev[q] is its index, so the list of
// box a read through rev enumerates the pairs whose source is a.
__global__ void k_reverse_pairs(int64_t npairs, const int32_t* __restrict__ pair_tgt,
                                const int32_t* __restrict__ pair_src,
                                const int64_t* __restrict__ il_ptr, int32_t* __restrict__ rev,
                                int32_t* __restrict__ err) {
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= npairs) return;
  const int32_t a = pair_tgt[q], b = pair_src[q];
  int64_t lo = il_ptr[b], hi = il_ptr[b + 1];
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (pair_src[mid] < a) lo = mid + 1;
    else hi = mid;
  }
  if (lo < il_ptr[b + 1] && pair_src[lo] == a) {
    rev[q] = (int32_t)lo;
  } else {
    rev[q] = -1;
    atomicExch(err, 1);
  }
}

// ---------------------------------------------------------------------------
// host-side launchers
// ---------------------------------------------------------------------------
static Radii make_radii(const double* r, int levels) {
  Radii R{};
  for (int j = 0; j <= levels && j <= kMaxLevels; ++j) R.r[j] = r[j];
  return R;
}

void launch_leaf_keys(cudaStream_t s, int64_t n, const double* xyz, int levels, const double* radii,
                      uint32_t* keys, int32_t* vals) {
  const int bs = 256;
  k_leaf_keys<<<(unsigned)((n + bs - 1) / bs), bs, 0, s>>>(n, xyz, levels, make_radii(radii, levels),
                                                          keys, vals);
}

void radix_sort_pairs(cudaStream_t s, int64_t n, int key_bits, uint32_t* keys, int32_t* vals,
                      uint32_t* keys_tmp, int32_t* vals_tmp, int32_t* counts, int* launches) {
  const int ntiles = (int)((n + kSortTile - 1) / kSortTile);
  const int nblk = (ntiles + 3) / 4;
  uint32_t* ki = keys;
  int32_t* vi = vals;
  uint32_t* ko = keys_tmp;
  int32_t* vo = vals_tmp;
  const int passes = (key_bits + 7) / 8;
  for (int p = 0; p < passes; ++p) {
    const int shift = 8 * p;
    k_radix_count<<<nblk, 128, 0, s>>>(n, ki, shift, ntiles, counts);
    k_scan_exclusive<<<1, 1024, 0, s>>>((int64_t)256 * ntiles, counts);
    k_radix_scatter<<<nblk, 128, 0, s>>>(n, ki, vi, shift, ntiles, counts, ko, vo);
    *launches += 3;
    uint32_t* tk = ki;
    ki = ko;
    ko = tk;
    int32_t* tv = vi;
    vi = vo;
    vo = tv;
  }
  if (ki != keys) {
    cudaMemcpyAsync(keys, ki, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync(vals, vi, n * sizeof(int32_t), cudaMemcpyDeviceToDevice, s);
  }
}

void launch_leaf_offsets(cudaStream_t s, int64_t n, const uint32_t* keys, int64_t nleaf,
                         int32_t* leaf_off) {
  const int bs = 256;
  k_leaf_offsets<<<(unsigned)((nleaf + 1 + bs - 1) / bs), bs, 0, s>>>(n, keys, nleaf, leaf_off);
}

void launch_gather_points(cudaStream_t s, int64_t n, const double* xyz, const int32_t* perm,
                          const uint32_t* leaf_of, int levels, const double* radii, double* xs,
                          double* ys, double* zs, float* xl, float* yl, float* zl) {
  const int bs = 256;
  k_gather_points<<<(unsigned)((n + bs - 1) / bs), bs, 0, s>>>(
      n, xyz, perm, leaf_of, levels, make_radii(radii, levels), xs, ys, zs, xl, yl, zl);
}

void launch_leaf_centres(cudaStream_t s, int64_t nleaf, int levels, const double* radii,
                         double* c) {
  const int bs = 256;
  k_leaf_centres<<<(unsigned)((nleaf + bs - 1) / bs), bs, 0, s>>>(nleaf, levels,
                                                                  make_radii(radii, levels), c);
}

void launch_box_lists(cudaStream_t s, int j, int mode, int32_t* nbr_all, int32_t* il_count,
                      const int64_t* il_ptr, int32_t* pair_tgt, int32_t* pair_src) {
  const int64_t nb = int64_t(1) << (3 * j);
  const int bs = 128;
  k_box_lists<<<(unsigned)((nb + bs - 1) / bs), bs, 0, s>>>(j, mode, nbr_all, il_count, il_ptr,
                                                           pair_tgt, pair_src);
}

void launch_reverse_pairs(cudaStream_t s, int64_t npairs, const int32_t* pair_tgt,
                          const int32_t* pair_src, const int64_t* il_ptr, int32_t* rev,
                          int32_t* err) {
  if (npairs == 0) return;
  const int bs = 256;
  k_reverse_pairs<<<(unsigned)((npairs + bs - 1) / bs), bs, 0, s>>>(npairs, pair_tgt, pair_src,
                                                                   il_ptr, rev, err);
}

}  // namespace h3d
