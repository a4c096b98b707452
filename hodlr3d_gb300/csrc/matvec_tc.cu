// Tensor-core (tcgen05, kind::tf32, 3xTF32) engine of the mixed-precision
// matvec for 17..32 right-hand sides (padded to 32).  Same operator and same
// owner writes as the CUDA-core engine in matvec.cu; the products run on the
// 5th-generation tensor cores with FP32 accumulators in TMEM.
//
//   ta_slice  per (level d-1 box "slice", share of its row tiles): T of the
//             pairs of levels 1..d-1 whose input box contains the slice, as a
//             tall GEMM [V_p1^T; V_p2^T; ...] X_slice (M = concatenated pair
//             columns in tiles of 128, K = slice points); level d-1 pairs get
//             T, the pairs above get slice partials
//   tred      FP64 sum of the slice partials
//   ta_leaf   per input leaf: the same for the leaf-level pairs
//   ut_tc     per (slice, 128 rows): long-K GEMM over the pairs of levels < d,
//             sum of U_p[rows] T_p
//   leaf_tc   per output leaf: long-K GEMM over its leaf-level pairs (U_p T_p)
//             and its near-field blocks (K_near X_near), plus the slice sum;
//             written once in the original order
//
// Each block streams a sequence of K = 32 chunks: (tile, item, k0), a tile
// being one M = 128 output tile and an item one operand pair (a factor A and
// its right-hand sides B) summed into it.  Operand rows are contiguous,
// 16-byte aligned runs of FP32 values (rows of the row-major FP32 U, columns
// of the FP32 V, rows of the FP32 near-field blocks, columns of X and T).
//
// A (the factors, streamed from HBM, in the split-exact TF32 form) is copied
// global -> shared with cp.async 16-byte copies, a warp moving 8 rows x 64
// contiguous bytes per instruction, into a row-major staging tile whose
// 16-byte columns are XOR-swizzled by the row; kAhead chunks are in flight.
// The thread owning a row (two per row, 16 K values each) reads it back,
// splits v = hi + lo (hi = v with the low 13 bits cleared, lo = v - hi, both
// exact TF32) and stores both parts to tensor memory.  B (the right-hand
// sides X or T, held in global memory as TF32 high and low parts) is copied
// to shared memory in the canonical K-major layout, [B_hi; B_lo] stacked as
// one N = 64 operand.  Two issuer warps then issue, per K = 8 step,
//   A_hi [B_hi | B_lo] -> accumulator D (N = 64: hi*hi, hi*lo)
//   A_lo B_hi          -> accumulator D2 (N = 32: lo*hi)
// (A read from tensor memory, so the tensor core reads only B from shared
// memory; the lo*lo term, below 2^-22 of the product, is left out).  Groups
// of kGroupChunks chunks alternate between two accumulator sets; a group is
// read back while the next one is multiplied, its hi*hi part summed with
// compensated (Kahan) FP32 additions (whose error matches an FP64 sum here at
// a fraction of the cost of GB300's FP64 units) and its cross parts with
// plain FP32 additions.
//
// Every mbarrier wait is bounded; a wait that gives up sets the error flag.
#include <algorithm>

#include "matvec.h"
#include "tc.cuh"

namespace h3d {

namespace {

constexpr int NR = 32;                     // right-hand sides (MMA N)
constexpr int KC = 32;                     // K per chunk
constexpr int WORKERS = 256;               // copy, split and read back: two threads per row
constexpr int THREADS = WORKERS + 64;      // plus two MMA issuer warps
constexpr int A_BYTES = 128 * KC * 4;      // A chunk (16 KB)
constexpr int B_BYTES = NR * KC * 4;       // one TF32 part of a B chunk (4 KB)
constexpr int SLOT_BYTES = A_BYTES + 2 * B_BYTES;  // copy slot: A, B hi, B lo
constexpr int kSlots = 8;                  // copy slots
constexpr int kAhead = kSlots - 2;         // chunks in flight ahead of the multiplied one
constexpr int TAB_OFF = kSlots * SLOT_BYTES;
constexpr int kMaxEntries = 768;           // table entries (pairs, near blocks) of one block
constexpr int ENTRY_BYTES = 32;
constexpr int SMEM_BYTES = TAB_OFF + kMaxEntries * ENTRY_BYTES + (kMaxEntries + 1) * 4;
constexpr uint32_t kWaitLimit = 1u << 22;
constexpr uint32_t IDESC64 = tc::idesc_tf32(128, 2 * NR);
constexpr uint32_t IDESC32 = tc::idesc_tf32(128, NR);
// tensor memory: accumulator set b at column 128 b (D: hi*hi 0..31, hi*lo
// 32..63; D2: lo*hi 64..95); A of chunk parity a at 256 + 64 a (hi 0..31,
// lo 32..63)
constexpr uint32_t kTmemCols = 512;
constexpr uint32_t TM_A = 256;
constexpr int kGroupChunks = 2;            // chunks per accumulation group (K = 64)

static_assert(SMEM_BYTES <= 227 * 1024, "shared memory");

__device__ __forceinline__ void kahan_add(float& s, float& c, float x) {
  const float y = x - c;
  const float t = s + y;
  c = (t - s) - y;
  s = t;
}

__device__ __forceinline__ void cp_async16(void* dst, const void* src, bool ok) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(tc::smem_addr(dst)),
               "l"(src), "r"(ok ? 16 : 0)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// One item of a block's stream as one thread sees it: its four A rows
// rb + 8 i (nullptr for a row outside the tile) with alen valid entries, and
// B column c at b + c * bs with blen valid entries; the item spans blen (a
// multiple of 4) values of K.
struct View {
  const float* arow[4];
  const float* b;  // high part; the low part at b + lo_off
  int64_t bs;
  int alen;
  int blen;
};

// A table entry of the long-K kernels: rows of A at a + i * as.
struct Item {
  const float* a;
  const float* b;
  int as;
  int bs;
  int alen;
  int blen;
};
static_assert(sizeof(Item) == ENTRY_BYTES, "entry");

// A table entry of the T kernels: pair column l has its A row at
// a + l * lda and its output (c, l) at dst[c * ld + l]; r values of l.  pad:
// the output is T (TF32 high and low parts, zero padded to ld), else a slice
// partial (FP32).
struct PairRow {
  const float* a;
  float* dst;
  int lda;
  int r;
  int ld;
  int pad;
};
static_assert(sizeof(PairRow) == ENTRY_BYTES, "entry");

struct Cursor {
  int tile, item, k0;
};

template <class Src>
__device__ __forceinline__ void cursor_skip(const Src& src, Cursor& cu) {
  while (cu.tile < src.ntiles()) {
    const int ni = src.nitems(cu.tile);
    while (cu.item < ni && src.klen(cu.tile, cu.item) <= 0) ++cu.item;
    if (cu.item < ni) return;
    ++cu.tile;
    cu.item = 0;
  }
}

template <class Src>
__device__ __forceinline__ void cursor_next(const Src& src, Cursor& cu) {
  cu.k0 += KC;
  if (cu.k0 < src.klen(cu.tile, cu.item)) return;
  cu.k0 = 0;
  ++cu.item;
  cursor_skip(src, cu);
}

// Streams the chunks of src through the tensor cores, called by all THREADS
// threads of the block.  Every worker thread calls src.finish(tile, sum, comp,
// cross) once a tile's products are summed (the tile's value is
// (sum - comp) + cross); returns the number of chunks (0 for every thread
// when src is empty).  Warps synchronise only through mbarriers:
//   bar[0..1]  ready: chunk of that parity split and copied (one arrival per
//              worker warp)
//   bar[2..3]  operands of chunk parity no longer read (one commit per issuer)
//   bar[4..5]  accumulator set complete (one commit per issuer)
template <class Src>
__device__ int run_stream(const Src& src, unsigned char* smem, uint64_t* bar, uint32_t tmem,
                          int64_t lo_off, int* err) {
  const int tid = threadIdx.x;
  Cursor lc{0, 0, 0};
  cursor_skip(src, lc);
  if (lc.tile >= src.ntiles()) return 0;

  if (tid >= WORKERS) {
    // issuer warps (lane 0): warp 8 A_hi [B_hi | B_lo] -> D, warp 9 A_lo B_hi
    // -> D2; each follows the chunk sequence with its own cursor
    if ((tid & 31) != 0) return 1;
    const bool second = tid >= WORKERS + 32;
    int c = 0, g = 0, gk = 0;
    for (;;) {
      Cursor nx = lc;
      cursor_next(src, nx);
      const bool stream_end = nx.tile >= src.ntiles();
      const bool close = nx.tile != lc.tile || gk == kGroupChunks - 1;
      const int buf = g & 1;
      if (!tc::mbar_wait(&bar[c & 1], (uint32_t)((c >> 1) & 1), kWaitLimit)) atomicExch(err, 1);
      tc::fence_after_sync();
      const uint32_t ab = tmem + TM_A + 64u * (uint32_t)(c & 1) + (second ? 32u : 0u);
      const uint32_t d = tmem + 128u * (uint32_t)buf + (second ? 64u : 0u);
      const uint64_t bd =
          tc::make_desc(tc::smem_addr(smem + (c % kSlots) * SLOT_BYTES + A_BYTES), 128, KC * 32);
#pragma unroll
      for (int ks = 0; ks < KC / 8; ++ks)
        tc::mma_tf32_ta(d, ab + 8u * ks, bd + (uint64_t)((ks * 256) >> 4), second ? IDESC32 : IDESC64,
                        (gk > 0 || ks > 0) ? 1u : 0u);
      tc::mma_commit(&bar[2 + (c & 1)]);
      if (close) {
        tc::mma_commit(&bar[4 + buf]);
        ++g;
        gk = 0;
      } else {
        ++gk;
      }
      if (stream_end) return c + 1;
      lc = nx;
      ++c;
    }
  }

  // worker threads.  Warp w owns rows 32 (w % 4) .. + 31 (its TMEM lanes)
  // and K quads 4 half .. 4 half + 3 of every chunk, half = w / 4: it copies
  // them (lane: k quad qa of rows rb + 8 i, i = 0..3) and splits them (lane:
  // row R), so a __syncwarp orders the two.  B: k quad qb of column cb.
  const int w = tid >> 5, lane = tid & 31, half = w >> 2;
  const int qa = 4 * half + (lane & 3);
  const int rb = 32 * (w & 3) + (lane >> 2);
  const uint32_t offA = (uint32_t)rb * 128u + ((uint32_t)(qa ^ (rb & 7)) << 4);  // row rb + 8 i: + 1024 i
  const int cb = 8 * (tid >> 6) + ((tid >> 2) & 7), qb = 4 * ((tid >> 5) & 1) + (tid & 3);
  const uint32_t offB = A_BYTES + tc::kmajor_off(cb, 4 * qb, KC);
  const int R = tid & 127;
  const uint32_t lane_base = ((uint32_t)((tid >> 5) & 3) * 32u) << 16;

  float sum[16], comp[16], cross[16];
#pragma unroll
  for (int j = 0; j < 16; ++j) sum[j] = comp[j] = cross[j] = 0.f;

  View lv{};
  int lv_tile = -1, lv_item = -1;
  int nload = 0, c = 0;
  int last = 0x7fffffff;  // index of the last chunk, once the loader has reached it
  uint32_t ends = 0;      // bit i: chunk c + i is the last of its tile
  auto load = [&]() {
    if (lc.tile != lv_tile || lc.item != lv_item) {
      src.view(lc.tile, lc.item, rb, lv);
      lv_tile = lc.tile;
      lv_item = lc.item;
    }
    unsigned char* sa = smem + (nload % kSlots) * SLOT_BYTES;
    const int k = lc.k0 + 4 * qa;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const bool ok = lv.arow[i] != nullptr && k < lv.alen;
      cp_async16(sa + offA + 1024 * i, ok ? lv.arow[i] + k : lv.b, ok);
    }
    const int kb = lc.k0 + 4 * qb;
    const bool ok = kb < lv.blen;
    const float* bsrc = ok ? lv.b + cb * lv.bs + kb : lv.b;
    cp_async16(sa + offB, bsrc, ok);
    cp_async16(sa + offB + B_BYTES, bsrc + lo_off, ok);
    const int t = lc.tile;
    cursor_next(src, lc);
    if (lc.tile != t) ends |= 1u << (nload - c);
    if (lc.tile >= src.ntiles()) last = nload;
    ++nload;
  };

  for (int i = 0; i < kAhead; ++i) {
    if (nload <= last) load();
    cp_async_commit();
  }

  auto read = [&](int g) {
    const uint32_t base = tmem + 128u * (uint32_t)(g & 1) + 16u * half + lane_base;
    if (!tc::mbar_wait(&bar[4 + (g & 1)], (uint32_t)((g >> 1) & 1), kWaitLimit)) atomicExch(err, 1);
    tc::fence_after_sync();
    float hh[16], x1[16], x2[16];
    tc::tmem_ld16(base, hh);
    tc::tmem_ld16(base + 32u, x1);
    tc::tmem_ld16(base + 64u, x2);
    tc::fence_before_sync();
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      kahan_add(sum[j], comp[j], hh[j]);
      cross[j] += x1[j] + x2[j];
    }
  };

  int g = 0, gk = 0, tile = 0, pend_tile = 0;
  bool pend = false;
  for (;;) {
    // the operands of chunk c - 2 (the copy slot refilled below and the
    // tensor-memory A of this chunk's parity) are no longer read
    if (c >= 2 && !tc::mbar_wait(&bar[2 + (c & 1)], (uint32_t)(((c - 2) >> 1) & 1), kWaitLimit))
      atomicExch(err, 1);
    if (nload <= last) load();
    cp_async_commit();
    cp_async_wait<kAhead>();
    __syncwarp();  // the warp's copies of this chunk (the other half of each row) have landed

    // split the row this thread owns and store it to tensor memory
    {
      const unsigned char* sa = smem + (c % kSlots) * SLOT_BYTES + (uint32_t)R * 128u;
      float hi[16], lo[16];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int qq = 4 * half + j;
        const float4 x = *reinterpret_cast<const float4*>(sa + ((uint32_t)(qq ^ (R & 7)) << 4));
        hi[4 * j] = tf32_rz(x.x);
        hi[4 * j + 1] = tf32_rz(x.y);
        hi[4 * j + 2] = tf32_rz(x.z);
        hi[4 * j + 3] = tf32_rz(x.w);
        lo[4 * j] = x.x - hi[4 * j];
        lo[4 * j + 1] = x.y - hi[4 * j + 1];
        lo[4 * j + 2] = x.z - hi[4 * j + 2];
        lo[4 * j + 3] = x.w - hi[4 * j + 3];
      }
      const uint32_t ta = tmem + TM_A + 64u * (uint32_t)(c & 1) + 16u * half + lane_base;
      tc::tmem_st16(ta, hi);
      tc::tmem_st16(ta + 32u, lo);
      tc::tmem_wait_st();
    }
    // B (copied by this warp's cp.async) to the tensor core's proxy; A stored
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncwarp();
    if (lane == 0) tc::mbar_arrive(&bar[c & 1]);
    const bool tile_end = ends & 1u;
    ends >>= 1;
    const bool close = tile_end || gk == kGroupChunks - 1;
    if (close) {
      if (pend) {
        read(g - 1);
        if (pend_tile != tile) {
          src.finish(pend_tile, sum, comp, cross);
#pragma unroll
          for (int j = 0; j < 16; ++j) sum[j] = comp[j] = cross[j] = 0.f;
        }
      }
      pend = true;
      pend_tile = tile;
      ++g;
      gk = 0;
    } else {
      ++gk;
    }
    if (tile_end) ++tile;
    if (c == last) break;
    ++c;
  }
  read(g - 1);
  src.finish(pend_tile, sum, comp, cross);
  cp_async_wait<0>();
  return c + 1;
}

__device__ __forceinline__ uint32_t block_setup(uint64_t* bar, uint32_t* tslot) {
  if (threadIdx.x < 32) tc::tmem_alloc(tslot, kTmemCols);
  if (threadIdx.x == 0) {
    tc::mbar_init(&bar[0], WORKERS / 32);
    tc::mbar_init(&bar[1], WORKERS / 32);
    for (int i = 2; i < 6; ++i) tc::mbar_init(&bar[i], 2);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  return *tslot;
}

__device__ __forceinline__ void block_teardown(uint32_t tmem) {
  tc::fence_before_sync();
  __syncthreads();
  if (threadIdx.x < 32) tc::tmem_dealloc(tmem, kTmemCols);
}

// Exclusive prefix sum of the ranks tab[0..n).r into s_cum[0..n] by warp 0.
__device__ __forceinline__ void warp0_scan(const PairRow* tab, int n, int* s_cum) {
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    int carry = 0;
    for (int base = 0; base < n; base += 32) {
      const int v = base + lane < n ? tab[base + lane].r : 0;
      int incl = v;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
      }
      if (base + lane < n) s_cum[base + lane] = carry + incl - v;
      carry += __shfl_sync(0xffffffffu, incl, 31);
    }
    if (lane == 0) s_cum[n] = carry;
  }
}

// ---------------------------------------------------------------------------
// Phase A: T = [V_p^T] X over one input box.  SLICE: the pairs of levels
// 1..d-1 over a level d-1 box; otherwise the leaf-level pairs over a leaf.
struct SrcTa {
  const PairRow* tab;
  const int* cum;
  int n;
  int rows;
  int tile0, tstep, ntile;
  int kin;
  const float* b;
  int64_t bs;
  int64_t lo_off;

  __device__ int ntiles() const { return ntile; }
  __device__ int nitems(int) const { return 1; }
  __device__ int klen(int, int) const { return kin; }
  __device__ bool locate(int t, int row, int& idx, int& l) const {
    const int rho = (tile0 + t * tstep) * 128 + row;
    if (rho >= rows) return false;
    int lo = 0, hi = n - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (cum[mid] <= rho) lo = mid;
      else hi = mid - 1;
    }
    idx = lo;
    l = rho - cum[lo];
    return true;
  }
  __device__ void view(int t, int, int rb, View& v) const {
    int idx = 0, l = 0;
    const bool in0 = locate(t, rb, idx, l);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      v.arow[i] = nullptr;
      if (in0) {
        const int rho = (tile0 + t * tstep) * 128 + rb + 8 * i;
        if (rho < rows) {
          while (cum[idx + 1] <= rho) ++idx;
          v.arow[i] = tab[idx].a + (int64_t)(rho - cum[idx]) * tab[idx].lda;
        }
      }
    }
    v.alen = kin;
    v.b = b;
    v.bs = bs;
    v.blen = kin;
  }
  __device__ void finish(int t, const float* sum, const float* comp, const float* cross) const {
    int idx, l;
    if (!locate(t, threadIdx.x & 127, idx, l)) return;
    const PairRow& e = tab[idx];
    const int c0 = (threadIdx.x >> 7) * 16;
    if (!e.pad) {  // slice partial
#pragma unroll
      for (int j = 0; j < 16; ++j) e.dst[(int64_t)(c0 + j) * e.ld + l] = (sum[j] - comp[j]) + cross[j];
      return;
    }
    // T as TF32 high and low parts, zero padded to ld
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      const float v = (sum[j] - comp[j]) + cross[j];
      const float hi = tf32_rn(v);
      float* o = e.dst + (int64_t)(c0 + j) * e.ld + l;
      o[0] = hi;
      o[lo_off] = tf32_rn(v - hi);
    }
    if (l == e.r - 1)
      for (int lp = e.r; lp < e.ld; ++lp)
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          float* o = e.dst + (int64_t)(c0 + j) * e.ld + lp;
          o[0] = 0.f;
          o[lo_off] = 0.f;
        }
  }
};

template <bool SLICE>
__global__ void __launch_bounds__(THREADS, 1) k_ta_tc(FarOp op, const float* __restrict__ Xt, int64_t N,
                                                      float* __restrict__ T, float* __restrict__ Pp,
                                                      int64_t lo_off, int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ uint64_t bar[6];
  __shared__ uint32_t tslot;
  PairRow* tab = reinterpret_cast<PairRow*>(smem + TAB_OFF);
  int* cum = reinterpret_cast<int*>(smem + TAB_OFF + kMaxEntries * ENTRY_BYTES);
  const int d = op.levels;
  const int64_t box = blockIdx.x;
  const int sh_in = SLICE ? 3 : 0;
  const int64_t i0 = op.leaf_off[box << sh_in], i1 = op.leaf_off[(box + 1) << sh_in];
  const int kin = (int)(i1 - i0);
  if (kin <= 0) return;
  const int jlo = SLICE ? 1 : d, jhi = SLICE ? d - 1 : d;
  int n = 0;
  for (int j = jlo; j <= jhi; ++j) {
    const int64_t gb = level_base(j) + (box >> (SLICE ? 3 * (d - 1 - j) : 0));
    n += (int)(op.il_ptr[gb + 1] - op.il_ptr[gb]);
  }
  if (n > kMaxEntries) {
    if (threadIdx.x == 0) atomicExch(err, 2);
    return;
  }
  if (n == 0) return;
  for (int idx = threadIdx.x; idx < n; idx += THREADS) {
    int j = jlo, base = 0;
    int64_t gb = 0;
    for (;; ++j) {
      gb = level_base(j) + (box >> (SLICE ? 3 * (d - 1 - j) : 0));
      const int cnt = (int)(op.il_ptr[gb + 1] - op.il_ptr[gb]);
      if (idx < base + cnt) break;
      base += cnt;
    }
    const int p = op.rev[op.il_ptr[gb] + (idx - base)];
    const int up = SLICE ? 3 * (d - 1 - j) : 0;
    const int64_t a = box >> up;
    const int64_t a0 = op.leaf_off[a << (3 * (d - j))];
    const int64_t lda = op.leaf_off[(a + 1) << (3 * (d - j))] - a0;
    const int r = op.rank[p];
    PairRow e;
    e.a = static_cast<const float*>(op.vfac[p]) + (i0 - a0);
    e.lda = (int)((lda + 3) & ~int64_t(3));
    e.r = r;
    e.pad = 0;
    if (!SLICE || j == d - 1) {
      e.pad = 1;
      e.ld = (r + 3) & ~3;
      e.dst = T + op.tr_off4[p] * NR;
    } else {
      e.ld = r;
      e.dst = Pp + (op.part_off[p] + (box - (a << up)) * (int64_t)r) * NR;
    }
    tab[idx] = e;
  }
  __syncthreads();
  warp0_scan(tab, n, cum);
  __syncthreads();
  const int rows = cum[n];
  const int ntiles_all = (rows + 127) / 128;
  if ((int)blockIdx.y >= ntiles_all) return;
  const uint32_t tmem = block_setup(bar, &tslot);
  SrcTa src;
  src.tab = tab;
  src.cum = cum;
  src.n = n;
  src.rows = rows;
  src.tile0 = blockIdx.y;
  src.tstep = gridDim.y;
  src.ntile = (ntiles_all - (int)blockIdx.y + (int)gridDim.y - 1) / (int)gridDim.y;
  src.kin = kin;
  src.b = Xt + i0;
  src.bs = N;
  src.lo_off = lo_off;
  run_stream(src, smem, bar, tmem, lo_off, err);
  block_teardown(tmem);
}

// FP64 sum of slice partials into the padded T: T_p[c][l] = sum_s P_p[s][c][l]
__global__ void k_tred_tc(FarOp op, const int32_t* __restrict__ pairs, const float* __restrict__ Pp,
                          float* __restrict__ T, int64_t lo_off) {
  const int p = pairs[blockIdx.x];
  const int r = op.rank[p], rp = (r + 3) & ~3;
  const int64_t ns = int64_t(1) << (3 * (op.levels - 1 - op.pair_level[p]));
  const float* src = Pp + op.part_off[p] * NR;
  float* dst = T + op.tr_off4[p] * NR;
  for (int o = threadIdx.x; o < rp * NR; o += blockDim.x) {
    const int c = o / rp, l = o - c * rp;
    double acc = 0.0;
    if (l < r)
      for (int64_t s = 0; s < ns; ++s) acc += (double)src[s * r * NR + c * r + l];
    const float hi = tf32_rn((float)acc);
    dst[o] = hi;
    dst[o + lo_off] = tf32_rn((float)(acc - (double)hi));
  }
}

// Items of one output tile (phase B).
struct SrcItems {
  const Item* items;
  int n;
  int nrows;
  __device__ int ntiles() const { return 1; }
  __device__ int nitems(int) const { return n; }
  __device__ int klen(int, int i) const { return items[i].blen; }
  __device__ void view(int, int i, int rb, View& v) const {
    const Item& it = items[i];
#pragma unroll
    for (int r = 0; r < 4; ++r)
      v.arow[r] = rb + 8 * r < nrows ? it.a + (int64_t)(rb + 8 * r) * it.as : nullptr;
    v.alen = it.alen;
    v.b = it.b;
    v.bs = it.bs;
    v.blen = it.blen;
  }
};

__device__ __forceinline__ Item pair_item(const FarOp& op, int p, int64_t row0, const float* T) {
  const int r = op.rank[p];
  const int rp = (r + 3) & ~3;
  Item it;
  it.a = static_cast<const float*>(op.ufac[p]) + row0 * rp;
  it.as = rp;
  it.alen = rp;
  it.b = T + op.tr_off4[p] * NR;
  it.bs = rp;
  it.blen = rp;
  return it;
}

struct SrcUt : SrcItems {
  double* ynl;
  int64_t N, r0;
  __device__ void finish(int, const float* sum, const float* comp, const float* cross) const {
    const int row = threadIdx.x & 127, c0 = (threadIdx.x >> 7) * 16;
    if (row >= nrows) return;
#pragma unroll
    for (int j = 0; j < 16; ++j)
      ynl[(int64_t)(c0 + j) * N + r0 + row] =
          ((double)sum[j] - (double)comp[j]) + (double)cross[j];
  }
};

// Phase B over the levels above the leaves: one block per (slice, 128 rows).
__global__ void __launch_bounds__(THREADS, 1) k_ut_tc(FarOp op, const float* __restrict__ T,
                                                      int64_t N, double* __restrict__ Ynl,
                                                      int64_t lo_off, int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ uint64_t bar[6];
  __shared__ uint32_t tslot;
  Item* items = reinterpret_cast<Item*>(smem + TAB_OFF);
  const int d = op.levels;
  const int64_t sb = blockIdx.x;
  const int64_t s0 = op.leaf_off[sb << 3], s1 = op.leaf_off[(sb + 1) << 3];
  const int64_t r0 = s0 + 128 * (int64_t)blockIdx.y;
  const int nrows = (int)min((int64_t)128, s1 - r0);
  if (nrows <= 0) return;
  int n = 0;
  for (int j = 1; j <= d - 1; ++j) {
    const int64_t gb = level_base(j) + (sb >> (3 * (d - 1 - j)));
    n += (int)(op.il_ptr[gb + 1] - op.il_ptr[gb]);
  }
  if (n > kMaxEntries) {
    if (threadIdx.x == 0) atomicExch(err, 2);
    return;
  }
  for (int idx = threadIdx.x; idx < n; idx += THREADS) {
    int j = 1, base = 0;
    int64_t gb = 0;
    for (;; ++j) {
      gb = level_base(j) + (sb >> (3 * (d - 1 - j)));
      const int cnt = (int)(op.il_ptr[gb + 1] - op.il_ptr[gb]);
      if (idx < base + cnt) break;
      base += cnt;
    }
    const int64_t a = sb >> (3 * (d - 1 - j));
    const int64_t a0 = op.leaf_off[a << (3 * (d - j))];
    items[idx] = pair_item(op, (int)(op.il_ptr[gb] + (idx - base)), r0 - a0, T);
  }
  __syncthreads();
  const uint32_t tmem = block_setup(bar, &tslot);
  SrcUt src;
  src.items = items;
  src.n = n;
  src.nrows = nrows;
  src.ynl = Ynl;
  src.N = N;
  src.r0 = r0;
  if (run_stream(src, smem, bar, tmem, lo_off, err) == 0 && threadIdx.x < WORKERS) {
    float z[16] = {};
    src.finish(0, z, z, z);
  }
  block_teardown(tmem);
}

struct SrcLeaf : SrcItems {
  const double* ynl;
  const int32_t* perm;
  double* y;
  int64_t N, ldy, t0;
  int nrhs, d;
  __device__ void finish(int, const float* sum, const float* comp, const float* cross) const {
    const int row = threadIdx.x & 127, c0 = (threadIdx.x >> 7) * 16;
    if (row >= nrows) return;
    const int64_t t = t0 + row;
    const int64_t orig = perm[t];
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      const int c = c0 + j;
      if (c < nrhs) {
        const double yn = d >= 2 ? ynl[(int64_t)c * N + t] : 0.0;
        y[(int64_t)c * ldy + orig] = (((double)sum[j] - (double)comp[j]) + (double)cross[j]) + yn;
      }
    }
  }
};

// Phase B at the leaf level plus the near field: one block per output leaf
// of at most 128 points.
__global__ void __launch_bounds__(THREADS, 1) k_leaf_tc(FarOp op, NearOp nr, const float* __restrict__ T,
                                                        const float* __restrict__ Xt, int64_t N,
                                                        const float* __restrict__ Knear,
                                                        const int64_t* __restrict__ near_off,
                                                        const double* __restrict__ Ynl,
                                                        const int32_t* __restrict__ perm, int nrhs,
                                                        double* __restrict__ Y, int64_t ldy,
                                                        int64_t lo_off, int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ uint64_t bar[6];
  __shared__ uint32_t tslot;
  Item* items = reinterpret_cast<Item*>(smem + TAB_OFF);
  const int d = op.levels;
  const int64_t k = blockIdx.x;
  const int64_t t0 = op.leaf_off[k];
  const int nk = (int)(op.leaf_off[k + 1] - t0);
  if (nk <= 0) return;
  const int64_t lk = level_base(d) + k;
  const int64_t q0 = op.il_ptr[lk];
  const int npair = (int)(op.il_ptr[lk + 1] - q0);
  const int n = npair + 27;
  if (n > kMaxEntries) {
    if (threadIdx.x == 0) atomicExch(err, 2);
    return;
  }
  for (int i = threadIdx.x; i < n; i += THREADS) {
    Item it;
    if (i < npair) {
      it = pair_item(op, (int)(q0 + i), 0, T);
    } else {
      const int sl = i - npair;  // neighbour slots 0..25, then the leaf itself
      const int64_t nn = sl < 26 ? (int64_t)nr.nbr_leaf[k * 26 + sl] : k;
      const int64_t off = near_off[k * 27 + sl];
      it.a = Knear;
      it.b = Xt;
      it.as = it.bs = it.alen = it.blen = 0;
      if (nn >= 0 && off >= 0) {
        const int64_t e0 = op.leaf_off[nn];
        const int ne = (int)(op.leaf_off[nn + 1] - e0);
        it.a = Knear + off;
        it.as = (ne + 3) & ~3;
        it.alen = it.as;
        it.b = Xt + e0;
        it.bs = (int)N;
        it.blen = ne;
      }
    }
    items[i] = it;
  }
  __syncthreads();
  const uint32_t tmem = block_setup(bar, &tslot);
  SrcLeaf src;
  src.items = items;
  src.n = n;
  src.nrows = nk;
  src.ynl = Ynl;
  src.perm = perm;
  src.y = Y;
  src.N = N;
  src.ldy = ldy;
  src.t0 = t0;
  src.nrhs = nrhs;
  src.d = d;
  if (run_stream(src, smem, bar, tmem, lo_off, err) == 0 && threadIdx.x < WORKERS) {
    float z[16] = {};
    src.finish(0, z, z, z);
  }
  block_teardown(tmem);
}

// X (original order, column-major) -> Xt[c * N + t] in tree order, FP32
__global__ void k_gather_xt(int64_t N, int nrhs, const double* __restrict__ X, int64_t ldx,
                            const int32_t* __restrict__ perm, float* __restrict__ Xt, int64_t lo_off) {
  const int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (o >= N * NR) return;
  const int c = (int)(o / N);
  const int64_t t = o - (int64_t)c * N;
  const double x = c < nrhs ? X[c * ldx + perm[t]] : 0.0;
  const float hi = tf32_rn((float)x);
  Xt[o] = hi;
  Xt[o + lo_off] = tf32_rn((float)(x - (double)hi));
}

// Near-field blocks of every leaf: for neighbour slot s (0..25, 26 = the leaf
// itself) a row-major nk x round4(ne) FP32 block at near_off[27 k + s], the
// kernel with the same displacement formula as the on-the-fly near field.
__global__ void k_near_blocks(const int32_t* __restrict__ leaf_off, NearOp nr,
                              const int64_t* __restrict__ near_off, float* __restrict__ Knear) {
  const int64_t k = blockIdx.x;
  const int sl = blockIdx.y;
  const int64_t off = near_off[k * 27 + sl];
  if (off < 0) return;
  const int64_t nn = sl < 26 ? (int64_t)nr.nbr_leaf[k * 26 + sl] : k;
  const int64_t t0 = leaf_off[k], e0 = leaf_off[nn];
  const int nk = (int)(leaf_off[k + 1] - t0), ne = (int)(leaf_off[nn + 1] - e0);
  const int nep = (ne + 3) & ~3;
  const float dcx = (float)(nr.centre[3 * k] - nr.centre[3 * nn]);
  const float dcy = (float)(nr.centre[3 * k + 1] - nr.centre[3 * nn + 1]);
  const float dcz = (float)(nr.centre[3 * k + 2] - nr.centre[3 * nn + 2]);
  for (int e = threadIdx.x; e < nk * nep; e += blockDim.x) {
    const int i = e / nep, j = e - i * nep;
    float v = 0.f;
    if (j < ne) {
      const int64_t ti = t0 + i, ej = e0 + j;
      v = (nn == k && i == j) ? (float)nr.kd.diag
                              : entry32_offdiag(nr.kd, (nr.xl[ti] - nr.xl[ej]) + dcx,
                                                (nr.yl[ti] - nr.yl[ej]) + dcy,
                                                (nr.zl[ti] - nr.zl[ej]) + dcz);
    }
    Knear[off + e] = tf32_split_value((double)v);
  }
}

}  // namespace

int tc_max_entries() { return kMaxEntries; }

int launch_near_blocks(cudaStream_t s, int64_t nleaf, const int32_t* leaf_off, const NearOp& near,
                       const int64_t* near_off, float* Knear) {
  k_near_blocks<<<dim3((unsigned)nleaf, 27), 256, 0, s>>>(leaf_off, near, near_off, Knear);
  return 1;
}

int launch_matvec_tc(cudaStream_t s, int64_t N, const int32_t* perm, const FarOp& far,
                     const NearOp& near, const TcBuffers& B, const double* X, int64_t ldx,
                     double* Y, int64_t ldy, int nrhs, MatvecProfiler* prof) {
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_ta_tc<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
    cudaFuncSetAttribute(k_ta_tc<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
    cudaFuncSetAttribute(k_ut_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
    cudaFuncSetAttribute(k_leaf_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
    attr = true;
  }
  int launches = 0;
  if (prof) prof->begin(s);
  k_gather_xt<<<(unsigned)((N * NR + 255) / 256), 256, 0, s>>>(N, nrhs, X, ldx, perm, B.xt,
                                                               B.lo_off);
  ++launches;
  if (prof) prof->mark(s, "gather");
  const int d = far.levels;
  if (d >= 2) {
    const int64_t nslice = int64_t(1) << (3 * (d - 1));
    // several blocks share a slice's row tiles when slices are few
    const int split = (int)std::max<int64_t>(1, std::min<int64_t>(32, (16 * 152) / nslice));
    k_ta_tc<true><<<dim3((unsigned)nslice, (unsigned)split), THREADS, SMEM_BYTES, s>>>(
        far, B.xt, N, B.t, B.p, B.lo_off, B.err);
    ++launches;
    if (prof) prof->mark(s, "ta_slice");
    if (B.n_upper > 0) {
      k_tred_tc<<<(unsigned)B.n_upper, 128, 0, s>>>(far, B.upper_pairs, B.p, B.t, B.lo_off);
      ++launches;
      if (prof) prof->mark(s, "tred");
    }
  }
  k_ta_tc<false><<<dim3((unsigned)far.nleaf, 1), THREADS, SMEM_BYTES, s>>>(far, B.xt, N, B.t, B.p,
                                                                           B.lo_off, B.err);
  ++launches;
  if (prof) prof->mark(s, "ta_leaf");
  if (d >= 2) {
    const int64_t nslice = int64_t(1) << (3 * (d - 1));
    const int tiles = (B.max_slice + 127) / 128;
    k_ut_tc<<<dim3((unsigned)nslice, (unsigned)std::max(1, tiles)), THREADS, SMEM_BYTES, s>>>(
        far, B.t, N, B.ynl, B.lo_off, B.err);
    ++launches;
    if (prof) prof->mark(s, "ut_tc");
  }
  k_leaf_tc<<<(unsigned)far.nleaf, THREADS, SMEM_BYTES, s>>>(far, near, B.t, B.xt, N, B.knear,
                                                             B.near_off, B.ynl, perm, nrhs, Y, ldy,
                                                             B.lo_off, B.err);
  ++launches;
  if (prof) prof->mark(s, "leaf_tc");
  return launches;
}

}  // namespace h3d
