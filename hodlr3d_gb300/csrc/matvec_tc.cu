// Tensor-core (tcgen05, kind::tf32, 3xTF32) engine of the mixed-precision
// matvec for up to 32 right-hand sides (zero padded to 32).  Same operator
// and same owner writes as the CUDA-core engine in matvec.cu, except that the
// leaf-level pairs enter as their dense FP32 blocks (smaller than their
// low-rank form at the ranks these leaves reach); the products run on the
// 5th-generation tensor cores with FP32 accumulators in TMEM.
//
//   ta_slice  per (level d-1 box "slice", share of its row tiles): T of the
//             pairs of levels 1..d-1 whose input box contains the slice, as a
//             tall GEMM [V_p1^T; V_p2^T; ...] X_slice per level (M = the pair
//             columns of the source box, stored one after the other, in tiles
//             of 128 rows, K = slice points); level d-1 pairs get T, the pairs
//             above get slice partials
//   tred      compensated sum of the slice partials
//   ut_tc     per (slice, 128 rows): long-K GEMM over the pairs of levels < d,
//             sum of U_p[rows] T_p
//   leaf_rows per output leaf: its dense blocks (near field and leaf-level
//             interaction list) times the sources' X, two blocks per tile,
//             plus the level sums; written once in the original order
//
// A block streams K = 64 chunks over its M = 128 output tiles.  A T tile (ta)
// runs over one K range, its input box; the tile of ut / leaf runs over its
// items (operand pairs: a factor A and its right-hand sides B, summed into
// the tile) one after the other.  In ta / ut three roles share the chunks,
// synchronised by mbarriers only:
//
//   producer (one warp)    copies A global -> shared with the tensor memory
//                          accelerator: 2D tiled loads from one tensor map per
//                          factor (boxes of 32 K x 128 rows, two K halves per
//                          chunk), 128-byte swizzle, zero fill outside the
//                          factor; up to kSlots chunks ahead
//   workers (8 warps)      copy B (X or T, 32 columns) with 16-byte cp.async
//                          into the 128-byte swizzled K-major layout, kAhead
//                          chunks ahead; split A and B into TF32 parts
//                          (below); read the accumulators back
//   issuer (one thread)    issues, per K = 8 step,
//                            A_hi [B_hi | B_lo] -> D cols 0..63 (hi*hi, hi*lo)
//                            A_lo B_hi          -> D cols 32..63 (+= lo*hi)
//                          with A read from tensor memory (the tensor core
//                          reads only B from shared memory); in order from
//                          one thread, so the second accumulates onto the first
//
// The factors, X and T are held in the split-exact FP32 form (common.cuh): v =
// hi + lo with hi = v with the 13 low mantissa bits cleared and lo = v - hi,
// both exact TF32.  The workers owning a row (two per row, 32 K values each)
// read it from the swizzled tile, store hi and lo to tensor memory.  X and T
// are written together with their low parts (lo_off floats further on): the
// T and U kernels copy B and its low parts; the leaf kernel copies B and
// writes the low parts next to it itself.  The tensor core reads B_hi from
// the full value.  The lo*lo term, below 2^-22 of the
// product, is left out.  Every chunk has its own accumulator (8 hi*hi MMAs,
// so that the truncating FP32 accumulation of the tensor core sees few
// additions: its bias stays well below 1e-6 of the product for all-positive
// data), one of kAcc in tensor memory, read back kLag chunks later while the
// next chunks are split and multiplied; its hi*hi part is summed with
// compensated (Kahan) FP32 additions (whose error matches an FP64 sum here at
// a fraction of the cost of GB300's FP64 units), its cross part with plain
// FP32 additions.  The waits of this pipeline poll without suspending the
// warp: a suspended warp resumes hundreds of cycles after the phase completes.
//
// Every mbarrier wait is bounded; a wait that gives up sets the error flag and
// the block's abort flag, after which no role issues new copies or products
// and the block drains those in flight (bounded) before it exits.
#include <cuda.h>

#include <algorithm>

#include "matvec.h"
#include "tc.cuh"

namespace h3d {

namespace {

constexpr int NR = 32;                     // right-hand sides (MMA N)
constexpr int KC = 64;                     // K per chunk (two 32-wide boxes of A)
constexpr int WORKERS = 256;               // copy B, split and read back: two threads per row
constexpr int NCOL = 16;                   // accumulator columns (right-hand sides) per worker
constexpr int ISSUER0 = WORKERS;           // warp 8: MMA issuer
constexpr int PRODUCER = WORKERS + 32;     // warp 9: A copies
constexpr int THREADS = PRODUCER + 32;
constexpr int A_HALF = 128 * 32 * 4;       // one 32-wide box of A (16 KB)
constexpr int A_BYTES = 2 * A_HALF;        // an A slot: one chunk (32 KB)
constexpr int B_HALF = 2 * NR * 128;       // B hi and lo rows of one K half (8 KB)
constexpr int B_LO = NR * 128;             // B_lo rows below B_hi in each K half
constexpr int B_SLOT = 2 * B_HALF;         // a B slot: one chunk, hi and lo (16 KB)
constexpr int kSlots = 4;                  // A ring: tiles in flight, freed once split
constexpr int kBSlots = 4;                 // B ring: freed once multiplied
constexpr int kABuf = 2;                   // tensor-memory A buffers
constexpr int kAcc = 3;                    // accumulators: one per chunk, read back kLag chunks later
constexpr int kLag = 2;
constexpr int kAhead = 2;                  // B chunks copied ahead of the one split into hi/lo
constexpr int B_RING = kSlots * A_BYTES;
constexpr int TAB_OFF = B_RING + kBSlots * B_SLOT;
constexpr int kMaxEntries = 768;           // table entries (pairs, near blocks) of one block
constexpr int ENTRY_BYTES = 32;
constexpr int SMEM_BYTES = TAB_OFF + kMaxEntries * ENTRY_BYTES + (kMaxEntries + 1) * 4;
constexpr uint32_t kWaitLimit = 1u << 17;   // polls of up to kWaitHintNs each: about 1 s
constexpr uint32_t kWaitHintNs = 8192;
constexpr uint32_t IDESC64 = tc::idesc_tf32(128, 2 * NR);
constexpr uint32_t IDESC32 = tc::idesc_tf32(128, NR);
// tensor memory: the accumulator of chunk c at column 64 (c % kAcc) (hi*hi
// 0..31; hi*lo + lo*hi 32..63); A of chunk c at 192 + 128 (c % kABuf) (hi
// 0..63, lo 64..127)
constexpr uint32_t kTmemCols = 512;
constexpr uint32_t TM_ACC = 64;
constexpr uint32_t TM_A = TM_ACC * kAcc;
constexpr uint32_t TM_ASTRIDE = 2 * KC;
// barriers
constexpr int BAR_FULL = 0;                // [kSlots] A of the slot landed (producer, tx)
constexpr int BAR_EMPTY = kSlots;          // [kSlots] A slot split (one arrival per worker warp)
constexpr int BAR_READY = 2 * kSlots;      // [kABuf] chunk c % kABuf split (one arrival per worker warp)
constexpr int BAR_DONE = BAR_READY + kABuf;  // [kAcc] chunk c % kAcc multiplied (issuer commits)
constexpr int BAR_DRAIN = BAR_DONE + kAcc;   // the issuer's products in flight completed
constexpr int NBAR = BAR_DRAIN + 1;
static_assert(kLag >= kABuf && kAcc > kLag && kAhead >= 1 && kAhead + kLag <= kBSlots, "chunk pipeline");

static_assert(SMEM_BYTES <= 227 * 1024, "shared memory");
static_assert(TM_A + TM_ASTRIDE * kABuf <= kTmemCols, "tensor memory");
static_assert(A_BYTES % 1024 == 0 && B_SLOT % 1024 == 0 && B_RING % 1024 == 0,
              "128-byte swizzled tiles start on 1024 bytes");

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

__device__ __forceinline__ void expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(tc::smem_addr(bar)),
               "r"(bytes)
               : "memory");
}
// 2D tiled tensor load of the box at (x, y) into shared memory, completing on bar
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
      "[%0], [%1, {%2, %3}], [%4];\n" ::"r"(tc::smem_addr(dst)),
      "l"(map), "r"(x), "r"(y), "r"(tc::smem_addr(bar))
      : "memory");
}

// Shared-memory descriptor of a K-major operand in the 128-byte swizzled
// layout (8-row atoms of 1024 bytes, each row 32 K values of 128 bytes whose
// 16-byte chunk j sits at chunk j ^ (row % 8)); a K = 8 step inside the row
// advances the start address by 32 bytes.  The tensor copies of A write this
// layout; the workers write B in it, which keeps their 16-byte shared-memory
// accesses free of bank conflicts.
__device__ __forceinline__ uint64_t desc_sw128(uint32_t saddr) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)1 << 16;             // leading byte offset 16 (unused by this layout)
  d |= (uint64_t)(1024 >> 4) << 32;   // stride byte offset: 8 rows of 128 bytes
  d |= (uint64_t)1 << 46;             // descriptor version
  d |= (uint64_t)2 << 61;             // 128-byte swizzle
  return d;
}

// byte offset of the 16-byte chunk (row n, K values 4 kc .. 4 kc + 3) in a
// 128-byte swizzled K-major tile whose K halves (32 values) are `half` apart
__device__ __forceinline__ uint32_t sw128_off(int n, int kc, int half) {
  return (uint32_t)((kc >> 3) * half + n * 128 + (((kc & 7) ^ (n & 7)) << 4));
}

// The B copies of one chunk: lane l of worker warp v copies k quad qb =
// l % 16 of the columns cb = 2 i + l / 16, i = 2 v, 2 v + 1, to
// bslot_off(i, l) of the slot, in the 128-byte swizzled layout (B_hi rows
// 0..31, B_lo rows 32..63 of each K half), and their low parts B_LO further.
// 16 consecutive lanes copy one column's 64 K values (256 contiguous bytes);
// a warp's 16-byte accesses fill four 128-byte rows, free of bank conflicts.
constexpr int BCOPIES = 16 / (WORKERS / 32);  // column pairs per worker warp
__device__ __forceinline__ int bslot_col(int i, int lane) { return 2 * i + (lane >> 4); }
__device__ __forceinline__ uint32_t bslot_off(int i, int lane) {
  return sw128_off(bslot_col(i, lane), lane & 15, B_HALF);
}

// A table entry of the long-K kernels: A is the box at (k, y) of map, B column
// c at b + c bs; blen values of K (a multiple of 4).
struct Item {
  const CUtensorMap* map;
  const float* b;
  int y;
  int bs;
  int blen;
  int pad;
};
static_assert(sizeof(Item) == ENTRY_BYTES, "entry");

// A table entry of the T kernels: its output (c, l), l < r, goes to
// dst[c * ld + l]; t: dst is T (split-exact, zero padded to round4(r)), else
// a slice partial (FP32).
struct PairRow {
  float* dst;
  int r;
  int ld;
  int t;
  int pad[3];
};
static_assert(sizeof(PairRow) == ENTRY_BYTES, "entry");

// Streams the chunks of src through the tensor cores, called by all THREADS
// threads of the block.  src: ntile tiles of cpt chunks; src.produce(c, a,
// bar, lane), called by the 32 lanes of the producer warp, issues the A
// copies of chunk c into a; src.load_b(c, slot, lane, i0) issues this
// worker's B copies of chunk c (both called for c = 0, 1, ... in order);
// every worker calls src.finish(tile, sum, comp, cross) once a tile's
// products are summed (the tile's value is (sum - comp) + cross).  Returns the
// number of chunks.
//
// A bounded wait that gives up sets the error flag and *abortp: every role
// then stops issuing copies and products, the issuer waits (bounded) for its
// products in flight and the producer for its copies in flight, and no tile
// is finished, before the block frees its tensor memory.
__device__ __forceinline__ void stream_give_up(int* err, volatile int* abortp) {
  atomicExch(err, 1);
  *abortp = 1;
}

// Test hook (hodlr3d_test_drop_copy): the producer of T-kernel block (0, 0)
// of the next launch stops before the copy of chunk g_drop_chunk, so the
// "landed" barrier of that chunk is never completed and the block's waits
// give up; read and cleared by that block (-1: off).
__device__ int g_drop_chunk = -1;

template <class Src>
__device__ int run_stream(Src& src, unsigned char* smem, uint64_t* bar, uint32_t tmem, int* err,
                          volatile int* abortp) {
  const int tid = threadIdx.x;
  const int cpt = src.cpt, nch = src.ntile * src.cpt;
  if (nch <= 0) return 0;

  if (tid >= PRODUCER) {
    // producer warp: lane 0 waits for the slot; the lanes issue the copies
    const int lane = tid & 31;
    int issued = 0;
    for (int c = 0; c < nch; ++c) {
      const int s = c % kSlots;
      if (c == src.drop) break;  // test hook: this chunk is never copied
      if (lane == 0 && c >= kSlots &&
          !tc::mbar_wait_spin(&bar[BAR_EMPTY + s], (uint32_t)(((c / kSlots) - 1) & 1)))
        stream_give_up(err, abortp);
      __syncwarp();
      if (*abortp) break;
      src.produce(c, smem + s * A_BYTES, &bar[BAR_FULL + s], lane);
      ++issued;
    }
    // copies in flight land before the block exits (bounded)
    if (lane == 0)
      for (int c = issued > kSlots ? issued - kSlots : 0; c < issued; ++c)
        if (!tc::mbar_wait_sleep(&bar[BAR_FULL + c % kSlots], (uint32_t)((c / kSlots) & 1), kWaitLimit,
                                 kWaitHintNs))
          stream_give_up(err, abortp);
    return nch;
  }

  if (tid >= ISSUER0) {
    // the issuer (warp 8, lane 0), per K step of 8: A_hi [B_hi | B_lo] -> D
    // columns 0..63, then A_lo B_hi -> D columns 32..63 (issued in order by
    // one thread, so the second always accumulates onto the first)
    if (tid != ISSUER0) return nch;
    for (int c = 0; c < nch; ++c) {
      if (!tc::mbar_wait_spin(&bar[BAR_READY + c % kABuf], (uint32_t)((c / kABuf) & 1)))
        stream_give_up(err, abortp);
      if (*abortp) break;
      tc::fence_after_sync();
      const uint32_t ab = tmem + TM_A + TM_ASTRIDE * (uint32_t)(c % kABuf);
      const uint32_t d = tmem + TM_ACC * (uint32_t)(c % kAcc);
      const uint32_t b0 = tc::smem_addr(smem + B_RING + (c % kBSlots) * B_SLOT);
#pragma unroll
      for (int ks = 0; ks < KC / 8; ++ks) {
        const uint64_t bd = desc_sw128(b0 + (uint32_t)((ks >> 2) * B_HALF + (ks & 3) * 32));
        tc::mma_tf32_ta(d, ab + 8u * ks, bd, IDESC64, ks > 0 ? 1u : 0u);
        tc::mma_tf32_ta(d + 32u, ab + (uint32_t)KC + 8u * ks, bd, IDESC32, 1u);
      }
      // chunk c multiplied: its accumulator is complete, its A buffer and B slot free
      tc::mma_commit(&bar[BAR_DONE + c % kAcc]);
    }
    // the products issued so far complete before the block frees tensor memory
    tc::mma_commit(&bar[BAR_DRAIN]);
    if (!tc::mbar_wait_sleep(&bar[BAR_DRAIN], 0u, kWaitLimit, kWaitHintNs))
      stream_give_up(err, abortp);
    return nch;
  }

  // workers.  Warp w owns rows 32 (w % 4) .. + 31 (its TMEM lanes), the K
  // half kq = w / 4 of every chunk (32 values, one 128-byte swizzled box of
  // A) and accumulator columns 16 kq .. 16 kq + 15; it copies the column
  // pairs i0, i0 + 1 of B.
  const int w = tid >> 5, lane = tid & 31, kq = w >> 2, i0 = BCOPIES * w;
  const int R = tid & 127;
  const uint32_t lane_base = ((uint32_t)((tid >> 5) & 3) * 32u) << 16;
  // a warp whose 32 rows all lie at or past the tile's live rows (a 64-point
  // leaf in a 128-row tile) skips splitting A: the tensor core still
  // multiplies its lanes of tensor memory (stale values) into accumulator
  // rows that no epilogue reads.  Warp-uniform, as tcgen05.st requires.
  const bool warp_live = 32 * ((tid >> 5) & 3) < src.live_rows();

  float sum[NCOL], comp[NCOL], cross[NCOL];
#pragma unroll
  for (int j = 0; j < NCOL; ++j) sum[j] = comp[j] = cross[j] = 0.f;

  // the accumulator of chunk r (multiplied: waited for by the caller) into
  // this thread's compensated sums
  auto read = [&](int r) {
    const uint32_t base = tmem + TM_ACC * (uint32_t)(r % kAcc) + (uint32_t)(NCOL * kq) + lane_base;
    tc::fence_after_sync();
    float hh[NCOL], xx[NCOL];
    tc::tmem_ld16x2(base, base + 32u, hh, xx);
    tc::fence_before_sync();
#pragma unroll
    for (int j = 0; j < NCOL; ++j) {
      kahan_add(sum[j], comp[j], hh[j]);
      cross[j] += xx[j];
    }
  };

  // B of the first kAhead chunks, one copy group per chunk (empty past the end)
  for (int c = 0; c < kAhead; ++c) {
    if (c < nch) src.load_b(c, smem + B_RING + (c % kBSlots) * B_SLOT, lane, i0);
    cp_async_commit();
  }

  // iteration c waits for the products of chunk c - kLag (which frees chunk
  // c's tensor-memory A buffer and the B slot of chunk c + kAhead), copies B
  // of chunk c + kAhead, splits chunk c and hands it to the issuer, then
  // reads chunk c - kLag back while chunk c is multiplied; kLag more
  // iterations read the last chunks.  The accumulator of chunk c - kLag is
  // next written by chunk c + 1, handed over in the next iteration.
  for (int c = 0; c < nch + kLag; ++c) {
    if (c >= kLag) {
      const int r = c - kLag;
      if (!tc::mbar_wait_spin(&bar[BAR_DONE + r % kAcc], (uint32_t)((r / kAcc) & 1)))
        stream_give_up(err, abortp);
      if (*abortp) break;
    }
    if (c < nch) {
      const int s = c % kSlots;
      if (c + kAhead < nch) src.load_b(c + kAhead, smem + B_RING + ((c + kAhead) % kBSlots) * B_SLOT, lane, i0);
      cp_async_commit();
      cp_async_wait<kAhead>();
      if (!tc::mbar_wait_spin(&bar[BAR_FULL + s], (uint32_t)((c / kSlots) & 1)))
        stream_give_up(err, abortp);
      if (*abortp) break;

      unsigned char* slot = smem + s * A_BYTES;
      {
        // the row this thread owns, from the 128-byte swizzled A box of its K half
        if (warp_live) {
          const unsigned char* sa = slot + kq * A_HALF + (uint32_t)R * 128u;
          float hi[32], lo[32];
  #pragma unroll
          for (int j = 0; j < 8; ++j) {
            const float4 x = *reinterpret_cast<const float4*>(sa + ((uint32_t)(j ^ (R & 7)) << 4));
            hi[4 * j] = tf32_rz(x.x);
            hi[4 * j + 1] = tf32_rz(x.y);
            hi[4 * j + 2] = tf32_rz(x.z);
            hi[4 * j + 3] = tf32_rz(x.w);
            lo[4 * j] = x.x - hi[4 * j];
            lo[4 * j + 1] = x.y - hi[4 * j + 1];
            lo[4 * j + 2] = x.z - hi[4 * j + 2];
            lo[4 * j + 3] = x.w - hi[4 * j + 3];
          }
          const uint32_t ta = tmem + TM_A + TM_ASTRIDE * (uint32_t)(c % kABuf) + 32u * kq + lane_base;
          tc::tmem_st32(ta, hi);
          tc::tmem_st32(ta + (uint32_t)KC, lo);
        }
        // the A slot is free once every worker warp has read its rows
        __syncwarp();
        if (lane == 0) tc::mbar_arrive(&bar[BAR_EMPTY + s]);
        tc::tmem_wait_st();
      }
      // B (this thread's copies, landed) to the tensor core's proxy; A stored
      // in tensor memory before the issuer multiplies it
      tc::fence_async_smem();
      tc::fence_before_sync();
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(&bar[BAR_READY + c % kABuf]);
    }
    if (c >= kLag) {
      const int r = c - kLag;
      read(r);
      if (r % cpt == cpt - 1) {
        src.finish(r / cpt, sum, comp, cross);
#pragma unroll
        for (int j = 0; j < NCOL; ++j) sum[j] = comp[j] = cross[j] = 0.f;
      }
    }
  }
  cp_async_wait<0>();
  return nch;
}

// 128-byte swizzled tensor copies need 1024-byte aligned destinations
__device__ __forceinline__ bool smem_misaligned(const unsigned char* smem, int* err) {
  if ((tc::smem_addr(smem) & 1023u) == 0) return false;
  if (threadIdx.x == 0) atomicExch(err, 3);
  return true;
}

__device__ __forceinline__ uint32_t block_setup(uint64_t* bar, uint32_t* tslot, int* abort_flag) {
  if (threadIdx.x < 32) tc::tmem_alloc(tslot, kTmemCols);
  if (threadIdx.x == 0) {
    *abort_flag = 0;
    tc::mbar_init(&bar[BAR_DRAIN], 1);
    for (int i = 0; i < kSlots; ++i) {
      tc::mbar_init(&bar[BAR_FULL + i], 1);
      tc::mbar_init(&bar[BAR_EMPTY + i], WORKERS / 32);
    }
    for (int i = 0; i < kABuf; ++i) tc::mbar_init(&bar[BAR_READY + i], WORKERS / 32);
    for (int i = 0; i < kAcc; ++i) tc::mbar_init(&bar[BAR_DONE + i], 1);
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

// Exclusive prefix sum of f(i), i < n, into out[0..n] by warp 0.
template <class F>
__device__ __forceinline__ void warp0_scan(int n, F f, int* out) {
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    int carry = 0;
    for (int base = 0; base < n; base += 32) {
      const int v = base + lane < n ? f(base + lane) : 0;
      int incl = v;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
      }
      if (base + lane < n) out[base + lane] = carry + incl - v;
      carry += __shfl_sync(0xffffffffu, incl, 31);
    }
    if (lane == 0) out[n] = carry;
  }
}

// index i with cum[i] <= v < cum[i + 1] (cum nondecreasing, cum[0] <= v < cum[n])
__device__ __forceinline__ int upper_index(const int* cum, int n, int v) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (cum[mid] <= v) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// ---------------------------------------------------------------------------
// Phase A: T = [V_p^T] X over one input box.  SLICE: the pairs of levels
// 1..d-1 over a level d-1 box; otherwise the leaf-level pairs over a leaf.
// The pairs of a level are the rows of their source box's V (one tensor map);
// a tile is 128 of those rows, tiles of the levels one after the other.
// lv[0][j]: first table entry of level j (lv[0][nlev] = n); lv[1][j]: first
// tile of level j (lv[1][nlev] = all tiles); lv[2][j]: column of the input
// box within the source box; lv[3][j]: the source box (all levels numbered
// together).
constexpr int kMaxLevels = 16;
struct SrcTa {
  const PairRow* tab;
  const int* cum;  // ranks before each entry
  const int (*lv)[kMaxLevels + 1];
  const CUtensorMap* vmaps;
  int n, nlev;
  int tile0, tstep, ntile, cpt;
  int kin;
  const float* b;
  int64_t bs, lo_off;
  // producer state (lane 0): the box of its current tile
  int pk = 0, pc = 0, px = 0, py = 0;
  const CUtensorMap* pmap = nullptr;
  int drop = -1;  // test hook: the chunk the producer stops before (-1: none)
  // worker state: K offset of the next B copy; the level, its first and
  // last-plus-one tiles and rows, and the table entry of this thread's row in
  // the last finished tile (rows only move forward)
  int wk = 0, fidx = 0, ftile0 = 0, ftile1 = 0, fbase = 0, fend = 0;

  // B is X over the input box: when kBSlots is a multiple of cpt, B slot s
  // always holds K range s % cpt, so B is copied and split in the first
  // kBSlots chunks only and read from the slot afterwards
  __device__ bool fresh_b(int c) const { return c < kBSlots || kBSlots % cpt != 0; }
  // tiles of V-stack rows: every row of a tile can be live
  __device__ int live_rows() const { return 128; }
  __device__ int level_of(int tg) const {
    int j = 0;
    while (j + 1 < nlev && lv[1][j + 1] <= tg) ++j;
    return j;
  }
  __device__ void produce(int, unsigned char* a, uint64_t* full, int lane) {
    if (lane != 0) return;
    if (pk == 0) {
      const int tg = tile0 + pc * tstep;
      const int j = level_of(tg);
      pmap = vmaps + lv[3][j];
      px = lv[2][j];
      py = (tg - lv[1][j]) * 128;
    }
    expect_tx(full, (uint32_t)A_BYTES);
    tma_load_2d(a, pmap, px + pk, py, full);
    tma_load_2d(a + A_HALF, pmap, px + pk + 32, py, full);
    pk += KC;
    if (pk >= cpt * KC) {
      pk = 0;
      ++pc;
    }
  }
  __device__ void load_b(int c, unsigned char* slot, int lane, int i0) {
    if (fresh_b(c)) {
      const int kb = wk + 4 * (lane & 15);
      const bool ok = kb < kin;
#pragma unroll
      for (int i = i0; i < i0 + BCOPIES; ++i) {
        const float* g = ok ? b + bslot_col(i, lane) * bs + kb : b;
        cp_async16(slot + bslot_off(i, lane), g, ok);
        cp_async16(slot + bslot_off(i, lane) + B_LO, g + lo_off, ok);
      }
    }
    wk += KC;
    if (wk >= cpt * KC) wk = 0;
  }
  __device__ void finish(int t, const float* sum, const float* comp, const float* cross) {
    const int tg = tile0 + t * tstep;
    const int v0 = (threadIdx.x & 127);
    if (tg >= ftile1) {  // first tile of a level: its bounds, then a search
      const int j = level_of(tg);
      ftile0 = lv[1][j];
      ftile1 = lv[1][j + 1];
      fbase = cum[lv[0][j]];
      fend = cum[lv[0][j + 1]];
      const int v = fbase + (tg - ftile0) * 128 + v0;
      if (v >= fend) return;
      fidx = upper_index(cum, n, v);
    }
    const int v = fbase + (tg - ftile0) * 128 + v0;
    if (v >= fend) return;
    // step forward to the entry holding row v, four entries per round trip
    for (;;) {
      const int c1 = cum[min(fidx + 1, n)], c2 = cum[min(fidx + 2, n)], c3 = cum[min(fidx + 3, n)],
                c4 = cum[min(fidx + 4, n)];
      if (v < c1) break;
      if (v < c2) { fidx += 1; break; }
      if (v < c3) { fidx += 2; break; }
      if (v < c4) { fidx += 3; break; }
      fidx += 4;
    }
    const int idx = fidx;
    // the entry's fields in registers: the stores below could alias the
    // table as far as the compiler knows, and would re-read it each time
    const PairRow e = tab[idx];
    const int l = v - cum[idx];
    const int c0 = (threadIdx.x >> 7) * NCOL;
    float* __restrict__ dst = e.dst + (int64_t)c0 * e.ld + l;
    const int64_t ld = e.ld;
    if (!e.t) {  // slice partial
#pragma unroll
      for (int j2 = 0; j2 < NCOL; ++j2) dst[j2 * ld] = (sum[j2] - comp[j2]) + cross[j2];
      return;
    }
    // T in the split-exact form and its low parts, zero padded to ld
#pragma unroll
    for (int j2 = 0; j2 < NCOL; ++j2) {
      const float v = (sum[j2] - comp[j2]) + cross[j2];
      const float hi = tf32_rz(v);
      const float tv = hi + tf32_rn(v - hi);
      dst[j2 * ld] = tv;
      dst[j2 * ld + lo_off] = tv - tf32_rz(tv);
    }
    if (l == e.r - 1)
      for (int lp = 1; lp < ((e.r + 3) & ~3) - e.r + 1; ++lp)
#pragma unroll
        for (int j2 = 0; j2 < NCOL; ++j2) dst[j2 * ld + lp] = dst[j2 * ld + lp + lo_off] = 0.f;
  }
};

template <bool SLICE>
__global__ void __launch_bounds__(THREADS, 1) k_ta_tc(FarOp op, const CUtensorMap* __restrict__ vmaps,
                                                      const float* __restrict__ Xt, int64_t N,
                                                      float* __restrict__ T, float* __restrict__ Pp,
                                                      int64_t lo_off, int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ uint64_t bar[NBAR];
  __shared__ uint32_t tslot;
  __shared__ int lv[4][kMaxLevels + 1];
  if (smem_misaligned(smem, err)) return;
  PairRow* tab = reinterpret_cast<PairRow*>(smem + TAB_OFF);
  int* cum = reinterpret_cast<int*>(smem + TAB_OFF + kMaxEntries * ENTRY_BYTES);
  const int d = op.levels;
  const int64_t box = blockIdx.x;
  const int sh_in = SLICE ? 3 : 0;
  const int64_t i0 = op.leaf_off[box << sh_in], i1 = op.leaf_off[(box + 1) << sh_in];
  const int kin = (int)(i1 - i0);
  if (kin <= 0) return;
  const int jlo = SLICE ? 1 : d, jhi = SLICE ? d - 1 : d;
  const int nlev = jhi - jlo + 1;
  if (nlev > kMaxLevels) {
    if (threadIdx.x == 0) atomicExch(err, 2);
    return;
  }
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
    const int r = op.rank[p];
    PairRow e;
    e.r = r;
    e.pad[0] = e.pad[1] = e.pad[2] = 0;
    if (!SLICE || j == d - 1) {
      e.t = 1;
      e.ld = op.tc_tld[p];
      e.dst = T + op.tc_toff[p];
    } else {
      e.t = 0;
      e.ld = r;
      e.dst = Pp + (op.part_off[p] + (box - (a << up)) * (int64_t)r) * NR;
    }
    tab[idx] = e;
  }
  __syncthreads();
  warp0_scan(n, [&](int i) { return tab[i].r; }, cum);
  __syncthreads();
  if (threadIdx.x == 0) {
    int first = 0, tiles = 0;
    for (int j = jlo; j <= jhi; ++j) {
      const int k = j - jlo;
      const int up = SLICE ? 3 * (d - 1 - j) : 0;
      const int64_t a = box >> up;
      const int64_t gb = level_base(j) + a;
      const int cnt = (int)(op.il_ptr[gb + 1] - op.il_ptr[gb]);
      lv[0][k] = first;
      lv[1][k] = tiles;
      lv[2][k] = (int)(i0 - op.leaf_off[a << (3 * (d - j))]);
      lv[3][k] = (int)gb;
      tiles += (cum[first + cnt] - cum[first] + 127) / 128;
      first += cnt;
    }
    lv[0][nlev] = first;
    lv[1][nlev] = tiles;
  }
  __syncthreads();
  const int ntiles_all = lv[1][nlev];
  if ((int)blockIdx.y >= ntiles_all) return;
  __shared__ int abort_flag;
  const uint32_t tmem = block_setup(bar, &tslot, &abort_flag);
  SrcTa src;
  src.tab = tab;
  src.cum = cum;
  src.lv = lv;
  src.vmaps = vmaps;
  src.n = n;
  src.nlev = nlev;
  src.tile0 = blockIdx.y;
  src.tstep = gridDim.y;
  src.ntile = (ntiles_all - (int)blockIdx.y + (int)gridDim.y - 1) / (int)gridDim.y;
  src.kin = kin;
  src.cpt = (kin + KC - 1) / KC;
  src.b = Xt + i0;
  src.bs = N;
  src.lo_off = lo_off;
  if (blockIdx.x == 0 && blockIdx.y == 0) {
    src.drop = *(volatile int*)&g_drop_chunk;
    __syncthreads();
    if (threadIdx.x == 0) g_drop_chunk = -1;
  }
  run_stream(src, smem, bar, tmem, err, &abort_flag);
  block_teardown(tmem);
}

// Sum of slice partials into the padded T (split-exact form), compensated
// FP32: T_p[c][l] = sum_s P_p[s][c][l]
__global__ void k_tred_tc(FarOp op, const int32_t* __restrict__ pairs, const float* __restrict__ Pp,
                          float* __restrict__ T, int64_t lo_off) {
  const int p = pairs[blockIdx.x];
  const int r = op.rank[p], rp = (r + 3) & ~3;
  const int64_t ns = int64_t(1) << (3 * (op.levels - 1 - op.pair_level[p]));
  const float* src = Pp + op.part_off[p] * NR;
  float* dst = T + op.tc_toff[p];
  const int64_t ld = op.tc_tld[p];
  for (int o = threadIdx.x; o < rp * NR; o += blockDim.x) {
    const int c = o / rp, l = o - c * rp;
    float sum = 0.f, comp = 0.f;
    if (l < r)
      for (int64_t s = 0; s < ns; ++s) kahan_add(sum, comp, src[s * r * NR + c * r + l]);
    const float tv = tf32_split_value((double)sum - (double)comp);
    dst[c * ld + l] = tv;
    dst[c * ld + l + lo_off] = tv - tf32_rz(tv);
  }
}

// Items of one output tile (phase B): item i takes chunks [cofs[i], cofs[i + 1]).
struct SrcItems {
  const Item* items;
  const int* cofs;
  int n;
  int nrows;
  int ntile, cpt;
  int drop = -1;  // test hook of the T kernel: never set here
  // producer cursor (lane 0): item, K offset, the item's map, row and K
  int pi = -1, pk = 0, py = 0, plen = 0;
  const CUtensorMap* pmap = nullptr;
  // worker cursor: item, K offset, the item's B (column 0), column stride and K
  int wi = -1, wk = 0, wbs = 0, wlen = 0;
  const float* wb = nullptr;
  int64_t lo_off = 0;  // the low parts of B, lo_off floats after B

  // rows of the block's tile that the epilogue writes (all items share them)
  __device__ int live_rows() const { return nrows; }
  // next item with K after item i
  __device__ int next_item(int i) const {
    ++i;
    while (cofs[i + 1] == cofs[i]) ++i;
    return i;
  }
  __device__ void produce(int, unsigned char* a, uint64_t* full, int lane) {
    if (lane != 0) return;
    if (pk >= plen) {
      pi = next_item(pi);
      const Item& it = items[pi];
      pmap = it.map;
      py = it.y;
      plen = it.blen;
      pk = 0;
    }
    expect_tx(full, (uint32_t)A_BYTES);
    tma_load_2d(a, pmap, pk, py, full);
    tma_load_2d(a + A_HALF, pmap, pk + 32, py, full);
    pk += KC;
  }
  __device__ void load_b(int, unsigned char* slot, int lane, int i0) {
    if (wk >= wlen) {
      wi = next_item(wi);
      const Item& it = items[wi];
      wb = it.b;
      wbs = it.bs;
      wlen = it.blen;
      wk = 0;
    }
    const int kb = wk + 4 * (lane & 15);
    const bool ok = kb < wlen;
#pragma unroll
    for (int i = i0; i < i0 + BCOPIES; ++i) {
      const float* g = ok ? wb + (int64_t)bslot_col(i, lane) * wbs + kb : wb;
      cp_async16(slot + bslot_off(i, lane), g, ok);
      cp_async16(slot + bslot_off(i, lane) + B_LO, g + lo_off, ok);
    }
    wk += KC;
  }
};

// The item of all pairs of target box gb (all levels numbered together):
// their U side by side (one tensor map), rows from y, times their T (32 x R).
__device__ __forceinline__ Item box_item(const FarOp& op, const CUtensorMap* umaps, int64_t gb, int y,
                                         const float* T) {
  Item it;
  it.map = umaps + gb;
  it.y = y;
  it.b = T + op.tc_tbox[gb];
  it.bs = op.tc_rbox[gb];
  it.blen = op.tc_rbox[gb];
  it.pad = 0;
  return it;
}

struct SrcUt : SrcItems {
  double* ynl;
  int64_t N, r0;
  __device__ void finish(int, const float* sum, const float* comp, const float* cross) const {
    const int row = threadIdx.x & 127, c0 = (threadIdx.x >> 7) * NCOL;
    if (row >= nrows) return;
#pragma unroll
    for (int j = 0; j < NCOL; ++j)
      ynl[(int64_t)(c0 + j) * N + r0 + row] =
          ((double)sum[j] - (double)comp[j]) + (double)cross[j];
  }
};

// Phase B over the levels above the leaves: one block per (slice, 128 rows).
__global__ void __launch_bounds__(THREADS, 1) k_ut_tc(FarOp op, const CUtensorMap* __restrict__ umaps,
                                                      const float* __restrict__ T, int64_t N,
                                                      double* __restrict__ Ynl, int64_t lo_off,
                                                      int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ uint64_t bar[NBAR];
  __shared__ uint32_t tslot;
  Item* items = reinterpret_cast<Item*>(smem + TAB_OFF);
  int* cofs = reinterpret_cast<int*>(smem + TAB_OFF + kMaxEntries * ENTRY_BYTES);
  if (smem_misaligned(smem, err)) return;
  const int d = op.levels;
  const int64_t sb = blockIdx.x;
  const int64_t s0 = op.leaf_off[sb << 3], s1 = op.leaf_off[(sb + 1) << 3];
  const int64_t r0 = s0 + 128 * (int64_t)blockIdx.y;
  const int nrows = (int)min((int64_t)128, s1 - r0);
  if (nrows <= 0) return;
  // one item per level: all pairs of the ancestor of the slice at that level
  const int n = d - 1;
  if (n > kMaxEntries) {
    if (threadIdx.x == 0) atomicExch(err, 2);
    return;
  }
  if (threadIdx.x < n) {
    const int j = 1 + threadIdx.x;
    const int64_t a = sb >> (3 * (d - 1 - j));
    const int64_t a0 = op.leaf_off[a << (3 * (d - j))];
    items[threadIdx.x] = box_item(op, umaps, level_base(j) + a, (int)(r0 - a0), T);
  }
  __syncthreads();
  warp0_scan(n, [&](int i) { return (items[i].blen + KC - 1) / KC; }, cofs);
  __shared__ int abort_flag;
  const uint32_t tmem = block_setup(bar, &tslot, &abort_flag);
  SrcUt src;
  src.items = items;
  src.cofs = cofs;
  src.n = n;
  src.nrows = nrows;
  src.ntile = 1;
  src.cpt = cofs[n];
  src.ynl = Ynl;
  src.N = N;
  src.r0 = r0;
  src.lo_off = lo_off;
  if (run_stream(src, smem, bar, tmem, err, &abort_flag) == 0 && threadIdx.x < WORKERS) {
    float z[NCOL] = {};
    src.finish(0, z, z, z);
  }
  block_teardown(tmem);
}

// X (original order, column-major) -> Xt[c * N + t] in tree order, split-exact
// FP32, and its low parts at Xt[lo_off + c * N + t]
__global__ void k_gather_xt(int64_t N, int nrhs, const double* __restrict__ X, int64_t ldx,
                            const int32_t* __restrict__ perm, float* __restrict__ Xt, int64_t lo_off) {
  const int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (o >= N * NR) return;
  const int c = (int)(o / N);
  const int64_t t = o - (int64_t)c * N;
  const float v = c < nrhs ? tf32_split_value(X[c * ldx + perm[t]]) : 0.f;
  Xt[o] = v;
  Xt[o + lo_off] = v - tf32_rz(v);
}

// Near-field blocks of every leaf: for neighbour slot s (0..25, 26 = the leaf
// itself) an nk x round4(ne) FP32 block at near_off[27 k + s], row stride
// near_ld[k] (the leaf's blocks side by side), the kernel with the same
// displacement formula as the on-the-fly near field.
__global__ void k_near_blocks(const int32_t* __restrict__ leaf_off, NearOp nr,
                              const int64_t* __restrict__ near_off,
                              const int32_t* __restrict__ near_ld, float* __restrict__ Knear) {
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
    Knear[off + (int64_t)i * near_ld[k] + j] = tf32_split_value((double)v);
  }
}

// lo parts of the near-field blocks for the FP64-accurate few-column form:
// the FP64 entry (the FP64 near field's formula, from the tree-ordered FP64
// points) minus the stored FP32 block entry, rounded to FP32
__global__ void k_near_lo(const int32_t* __restrict__ leaf_off, NearOp nr,
                          const int64_t* __restrict__ near_off, const int32_t* __restrict__ near_ld,
                          const float* __restrict__ Knear, float* __restrict__ Knearlo) {
  const int64_t k = blockIdx.x;
  const int sl = blockIdx.y;
  const int64_t off = near_off[k * 27 + sl];
  if (off < 0) return;
  const int64_t nn = sl < 26 ? (int64_t)nr.nbr_leaf[k * 26 + sl] : k;
  const int64_t t0 = leaf_off[k], e0 = leaf_off[nn];
  const int nk = (int)(leaf_off[k + 1] - t0), ne = (int)(leaf_off[nn + 1] - e0);
  const int nep = (ne + 3) & ~3;
  const int64_t ld = near_ld[k];
  for (int e = threadIdx.x; e < nk * nep; e += blockDim.x) {
    const int i = e / nep, j = e - i * nep;
    const int64_t o = off + (int64_t)i * ld + j;
    double v = 0.0;
    if (j < ne) {
      const int64_t ti = t0 + i, ej = e0 + j;
      v = (nn == k && i == j) ? nr.kd.diag
                              : entry64_offdiag(nr.kd, __dsub_rn(nr.xs[ti], nr.xs[ej]),
                                                __dsub_rn(nr.ys[ti], nr.ys[ej]),
                                                __dsub_rn(nr.zs[ti], nr.zs[ej]));
    }
    Knearlo[o] = (float)(v - (double)Knear[o]);
  }
}

// ---------------------------------------------------------------------------
// Leaf rows: the leaf level as dense blocks, two per tensor-core tile.
//
// Leaf k multiplies, at the leaf level, the dense blocks of its near field
// (itself and its face / edge neighbours) and of its leaf-level interaction
// list.  The low-rank form of a leaf-level pair is larger than the block
// itself at these ranks (64-point leaves at tol 1e-10: mean rank 47, so
// r (n + m) = 6016 entries against n m = 4096), so this engine keeps those
// blocks dense (FP32, split-exact TF32), side by side in one row-major
// nk x W_k matrix per leaf (LeafBlock: column x0, width round4(m)); the
// leaf-level T of the low-rank form is not needed.
//
// One block per leaf (nk <= 64).  Chunk c multiplies two blocks at once: rows
// 0..63 of the 128-row tile hold block 2c, rows 64..127 block 2c + 1, each
// over its own 64-wide K range, and B = [X_top | X_bottom] (64 columns): the
// wanted products are the diagonal quarters of D (rows 0..63 x columns 0..31,
// rows 64..127 x columns 32..63); both halves add to the leaf's rows and are
// combined at the end.  Per K = 8 step the issuer multiplies A_hi (tensor
// memory) by [B_hi | B_lo] (N = 128), then A_lo (tensor memory) by B_hi
// (N = 64) onto the hi*lo columns.  Accumulation groups are one chunk (8
// hi*hi MMAs per accumulator, two accumulators), read back and summed with
// compensated FP32 additions: the truncating FP32 accumulation of the tensor
// core stays below 1e-6 of same-sign sums.
//
// Every mbarrier wait is bounded.  A wait that gives up sets the error flag
// and the block-wide abort flag: no role issues new copies or products after
// that, the issuer waits (bounded) for its products in flight and the
// producer for its copies in flight before the block frees its tensor memory
// and exits.
namespace lr {
// roles of the leaf-row kernel: 16 worker warps (four per 32 TMEM lanes, one
// K quarter each), 1 issuer warp, 1 producer warp
constexpr int WORKERS = 512;
constexpr int ISSUER0 = WORKERS;
constexpr int PRODUCER = WORKERS + 32;
constexpr int THREADS = WORKERS + 64;
constexpr int NCOL = 8;                     // accumulator columns per worker
constexpr int KC = 64;
constexpr int NB = 2 * NR;                  // B columns: top and bottom right-hand sides
constexpr int A_HALF = 128 * 32 * 4;        // one K half of A (rows 0..127, 32 K): 16 KB
constexpr int A_BOX = 64 * 32 * 4;          // one 64-row box: 8 KB
constexpr int A_BYTES = 2 * A_HALF;         // an A slot: 32 KB
// B in the 128-byte swizzled K-major layout, per K half 128 rows (n 0..63
// B_hi, 64..127 B_lo) of 128 bytes: 16 KB; its low part 64 rows below
constexpr int B_HALF = 2 * NB * 32 * 4;
constexpr int B_LO = NB * 128;
constexpr int B_BYTES = 2 * B_HALF;         // a B slot: 32 KB
constexpr int kASlots = 3;                  // A tiles in flight (freed once split)
constexpr int kBSlots = 3;                  // B tiles (freed once multiplied), one copied ahead
constexpr int B_OFF = kASlots * A_BYTES;
constexpr int kMaxBlocks = 512;             // blocks of one leaf row (table in shared memory)
constexpr int TAB_OFF = B_OFF + kBSlots * B_BYTES;
constexpr int SMEM_BYTES = TAB_OFF + kMaxBlocks * (int)sizeof(LeafBlock);
constexpr uint32_t IDESC_HL = tc::idesc_tf32(128, 2 * NB);  // A_hi [B_hi | B_lo]
constexpr uint32_t IDESC_LH = tc::idesc_tf32(128, NB);      // A_lo B_hi
// tensor memory (512 columns): the accumulator of chunk c at 128 (c % 2)
// ([HH | X] with X = hi*lo + lo*hi, N = 128); A buffer c % 2 (hi 64, lo 64
// columns) at 256 + 128 (c % 2)
constexpr uint32_t TM_ACC = 128;
constexpr uint32_t TM_A = 256;
constexpr uint32_t TM_ASTRIDE = 128;
// FULL / EMPTY per A slot; READY / DONE per chunk parity (split / multiplied)
constexpr int BAR_FULL = 0, BAR_EMPTY = kASlots, BAR_READY = 2 * kASlots, BAR_DONE = BAR_READY + 2,
              BAR_DRAIN = BAR_DONE + 2, NBAR = BAR_DRAIN + 1;
static_assert(SMEM_BYTES <= 227 * 1024, "shared memory");
static_assert(64 * NR * 8 <= A_BYTES, "combine buffer fits an A slot");

__device__ __forceinline__ bool aborted(const volatile int* flag) { return *flag != 0; }

__device__ __forceinline__ void give_up(int* err, volatile int* flag) {
  atomicExch(err, 1);
  *flag = 1;
}

// rows of the workers' named barrier (barrier 1, the 512 worker threads)
__device__ __forceinline__ void workers_sync() { asm volatile("bar.sync 1, %0;\n" ::"n"(lr::WORKERS) : "memory"); }

__device__ __forceinline__ void tmem_ld8x2(uint32_t a0, uint32_t a1, float* v0, float* v1) {
  uint32_t r[16];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                 "=r"(r[7])
               : "r"(a0));
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
               : "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
                 "=r"(r[14]), "=r"(r[15])
               : "r"(a1));
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    v0[i] = __uint_as_float(r[i]);
    v1[i] = __uint_as_float(r[8 + i]);
  }
}
}  // namespace lr

// Dense FP32 blocks of the leaf rows: block i of leaf k (LeafBlock
// blocks[block_ptr[k] + i], source leaf src) is nk x round4(m) at column x0 of
// leaf k's matrix (row_base[k], row stride row_ld[k]), the kernel with the
// displacement formula of the FP32 near field, in the split-exact form; the
// columns past m are zero.
__global__ void k_row_blocks(const int32_t* __restrict__ leaf_off, NearOp nr,
                             const LeafBlock* __restrict__ blocks, const int32_t* __restrict__ block_ptr,
                             const int64_t* __restrict__ row_base, const int32_t* __restrict__ row_ld,
                             float* __restrict__ Krow) {
  const int64_t k = blockIdx.x;
  const int i = blockIdx.y;
  if (block_ptr[k] + i >= block_ptr[k + 1]) return;
  const LeafBlock b = blocks[block_ptr[k] + i];
  const int64_t nn = b.src;
  const int64_t t0 = leaf_off[k], e0 = leaf_off[nn];
  const int nk = (int)(leaf_off[k + 1] - t0), ne = b.len;
  const int nep = (ne + 3) & ~3;
  const int64_t ld = row_ld[k];
  float* dst = Krow + row_base[k] + b.x0;
  const float dcx = (float)(nr.centre[3 * k] - nr.centre[3 * nn]);
  const float dcy = (float)(nr.centre[3 * k + 1] - nr.centre[3 * nn + 1]);
  const float dcz = (float)(nr.centre[3 * k + 2] - nr.centre[3 * nn + 2]);
  for (int e = threadIdx.x; e < nk * nep; e += blockDim.x) {
    const int ii = e / nep, j = e - ii * nep;
    float v = 0.f;
    if (j < ne) {
      const int64_t ti = t0 + ii, ej = e0 + j;
      v = (nn == k && ii == j) ? (float)nr.kd.diag
                               : entry32_offdiag(nr.kd, (nr.xl[ti] - nr.xl[ej]) + dcx,
                                                 (nr.yl[ti] - nr.yl[ej]) + dcy,
                                                 (nr.zl[ti] - nr.zl[ej]) + dcz);
    }
    dst[(int64_t)ii * ld + j] = tf32_split_value((double)v);
  }
}

// The leaf level and the near field of leaf k = blockIdx.x, plus the level
// sums of the levels above (Ynl, d >= 2); owner write of the leaf's rows in
// the original order.
//
// Pipeline: the producer keeps up to kASlots A tiles in flight; per chunk c
// the workers wait for the products of chunk c - 2 and read its accumulator
// back, copy B of chunk c + 1 into the B slot chunk c - 2 used, split tile c
// into tensor memory (hi = the value itself, which the tensor core reads as
// TF32, and lo = its remainder; A buffer c % 2), which frees its
// shared-memory slot at once, write the low part of B, and signal "ready";
// the issuer multiplies chunk c into accumulator c % 2 while the workers
// move on to chunk c + 1.
__global__ void __launch_bounds__(lr::THREADS, 1) k_leaf_rows_tc(
    const int32_t* __restrict__ leaf_off, const LeafBlock* __restrict__ blocks,
    const int32_t* __restrict__ block_ptr, const CUtensorMap* __restrict__ rmaps,
    const float* __restrict__ Xt, int64_t N, const double* __restrict__ Ynl, int levels,
    const int32_t* __restrict__ perm, int nrhs, double* __restrict__ Y, int64_t ldy,
    int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ uint64_t bar[lr::NBAR];
  __shared__ uint32_t tslot;
  __shared__ int abort_flag;
  if (smem_misaligned(smem, err)) return;
  const int64_t k = blockIdx.x;
  const int64_t t0 = leaf_off[k];
  const int nk = (int)(leaf_off[k + 1] - t0);
  if (nk <= 0) return;
  if (nk > 64) {
    if (threadIdx.x == 0) atomicExch(err, 2);
    return;
  }
  const int nit = block_ptr[k + 1] - block_ptr[k];
  if (nit > lr::kMaxBlocks) {
    if (threadIdx.x == 0) atomicExch(err, 2);
    return;
  }
  const int nch = (nit + 1) / 2;
  // the leaf's block list, staged in shared memory
  LeafBlock* it = reinterpret_cast<LeafBlock*>(smem + lr::TAB_OFF);
  for (int i = threadIdx.x; i < nit; i += lr::THREADS) it[i] = blocks[block_ptr[k] + i];
  const CUtensorMap* map = rmaps + k;
  const int tid = threadIdx.x;
  volatile int* abortp = &abort_flag;
  if (tid < 32) tc::tmem_alloc(&tslot, kTmemCols);
  if (tid == 0) {
    abort_flag = 0;
    for (int i = 0; i < lr::kASlots; ++i) {
      tc::mbar_init(&bar[lr::BAR_FULL + i], 1);
      tc::mbar_init(&bar[lr::BAR_EMPTY + i], lr::WORKERS / 32);
    }
    for (int i = 0; i < 2; ++i) {
      tc::mbar_init(&bar[lr::BAR_READY + i], lr::WORKERS / 32);
      tc::mbar_init(&bar[lr::BAR_DONE + i], 1);
    }
    tc::mbar_init(&bar[lr::BAR_DRAIN], 1);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tslot;

  if (tid >= lr::PRODUCER) {
    // producer warp (lane 0): four 32 x 64 boxes per chunk (K halves of the
    // top and bottom blocks); a missing bottom block reads rows 64..127 of
    // the leaf's matrix, all outside it: zeros
    if ((tid & 31) == 0) {
      int issued = 0;
      for (int c = 0; c < nch; ++c) {
        const int s = c % lr::kASlots;
        if (c >= lr::kASlots &&
            !tc::mbar_wait_try(&bar[lr::BAR_EMPTY + s], (uint32_t)(((c / lr::kASlots) - 1) & 1)))
          lr::give_up(err, abortp);
        if (lr::aborted(abortp)) break;
        unsigned char* a = smem + s * lr::A_BYTES;
        const LeafBlock bt = it[2 * c];
        const bool hb = 2 * c + 1 < nit;
        const int xb = hb ? it[2 * c + 1].x0 : 0, yb = hb ? 0 : 64;
        expect_tx(&bar[lr::BAR_FULL + s], (uint32_t)lr::A_BYTES);
        tma_load_2d(a, map, bt.x0, 0, &bar[lr::BAR_FULL + s]);
        tma_load_2d(a + lr::A_HALF, map, bt.x0 + 32, 0, &bar[lr::BAR_FULL + s]);
        tma_load_2d(a + lr::A_BOX, map, xb, yb, &bar[lr::BAR_FULL + s]);
        tma_load_2d(a + lr::A_HALF + lr::A_BOX, map, xb + 32, yb, &bar[lr::BAR_FULL + s]);
        ++issued;
      }
      // copies in flight land before the block exits (bounded)
      for (int c = issued > lr::kASlots ? issued - lr::kASlots : 0; c < issued; ++c)
        if (!tc::mbar_wait_sleep(&bar[lr::BAR_FULL + c % lr::kASlots], (uint32_t)((c / lr::kASlots) & 1),
                                 kWaitLimit, kWaitHintNs))
          lr::give_up(err, abortp);
    }
  } else if (tid >= lr::ISSUER0) {
    // the issuer (lane 0 of warp 16), per K step of 8: A_hi [B_hi | B_lo] ->
    // [HH | X] (N = 128), then A_lo B_hi -> X (N = 64, accumulating), A from
    // tensor memory; in order from one thread
    if (tid == lr::ISSUER0) {
      for (int c = 0; c < nch; ++c) {
        if (!tc::mbar_wait_try(&bar[lr::BAR_READY + (c & 1)], (uint32_t)((c >> 1) & 1)))
          lr::give_up(err, abortp);
        if (lr::aborted(abortp)) break;
        tc::fence_after_sync();
        const uint32_t b0 = tc::smem_addr(smem + lr::B_OFF + (c % lr::kBSlots) * lr::B_BYTES);
        const uint32_t ab = tmem + lr::TM_A + lr::TM_ASTRIDE * (uint32_t)(c & 1);
        const uint32_t d = tmem + lr::TM_ACC * (uint32_t)(c & 1);
#pragma unroll
        for (int ks = 0; ks < lr::KC / 8; ++ks) {
          const uint64_t bd = desc_sw128(b0 + (uint32_t)((ks >> 2) * lr::B_HALF + (ks & 3) * 32));
          tc::mma_tf32_ta(d, ab + 8u * ks, bd, lr::IDESC_HL, ks > 0 ? 1u : 0u);
          tc::mma_tf32_ta(d + (uint32_t)lr::NB, ab + 64u + 8u * ks, bd, lr::IDESC_LH, 1u);
        }
        // chunk c multiplied: its accumulator complete, its A buffer and B slot free
        tc::mma_commit(&bar[lr::BAR_DONE + (c & 1)]);
      }
      // the products issued so far complete before the block frees tensor memory
      tc::mma_commit(&bar[lr::BAR_DRAIN]);
      if (!tc::mbar_wait_sleep(&bar[lr::BAR_DRAIN], 0u, kWaitLimit, kWaitHintNs))
        lr::give_up(err, abortp);
    }
  } else {
    // workers.  Thread (row R = tid % 128, K quarter kq = warp / 4): splits
    // 16 K values of row R of A into tensor memory, copies B's k quad
    // (tid % 16) of column tid / 16 for the top block and the bottom block,
    // and reads back accumulator columns 8 kq .. 8 kq + 7 of its half.
    const int w = tid >> 5, kq = w >> 2, R = tid & 127;
    const bool bottom = (w & 3) >= 2;  // rows 64..127: warp-uniform
    const uint32_t lane_base = ((uint32_t)(w & 3) * 32u) << 16;
    // B copies: 16 consecutive threads read 256 contiguous bytes of one
    // column; 8 of them write one 128-byte swizzled row (no bank conflicts)
    const int bcol = tid >> 4, bk = 4 * (tid & 15);
    const uint32_t boff_top = sw128_off(bcol, tid & 15, lr::B_HALF);
    const uint32_t boff_bot = sw128_off(bcol + NR, tid & 15, lr::B_HALF);
    float sum[lr::NCOL], comp[lr::NCOL], cross[lr::NCOL];
#pragma unroll
    for (int j = 0; j < lr::NCOL; ++j) sum[j] = comp[j] = cross[j] = 0.f;

    auto load_b = [&](int c) {
      unsigned char* bs = smem + lr::B_OFF + (c % lr::kBSlots) * lr::B_BYTES;
      const LeafBlock bt = it[2 * c];
      const bool okt = bk < bt.len;
      cp_async16(bs + boff_top, okt ? Xt + (int64_t)bcol * N + bt.src_off + bk : Xt, okt);
      bool okb = false;
      const float* srcb = Xt;
      if (2 * c + 1 < nit) {
        const LeafBlock bb = it[2 * c + 1];
        okb = bk < bb.len;
        if (okb) srcb = Xt + (int64_t)bcol * N + bb.src_off + bk;
      }
      cp_async16(bs + boff_bot, srcb, okb);
      cp_async_commit();
    };
    // waits for chunk c's products, then its accumulator into the sums
    auto read = [&](int c) {
      if (!tc::mbar_wait_try(&bar[lr::BAR_DONE + (c & 1)], (uint32_t)((c >> 1) & 1)))
        lr::give_up(err, abortp);
      const uint32_t acc = tmem + lr::TM_ACC * (uint32_t)(c & 1) + (bottom ? (uint32_t)NR : 0u) +
                           (uint32_t)(lr::NCOL * kq) + lane_base;
      tc::fence_after_sync();
      float hh[lr::NCOL], xx[lr::NCOL];
      lr::tmem_ld8x2(acc, acc + (uint32_t)lr::NB, hh, xx);
      tc::fence_before_sync();
#pragma unroll
      for (int j = 0; j < lr::NCOL; ++j) {
        kahan_add(sum[j], comp[j], hh[j]);
        cross[j] += xx[j];
      }
    };

    // iteration c: chunk c - 2 multiplied (its A buffer and its B slot, the
    // one chunk c + 1 fills, are free) and read back (its accumulator is the
    // one chunk c writes), then chunk c split and handed to the issuer while
    // chunk c - 1 is multiplied; the last two chunks are read after the loop
    if (nch > 0) load_b(0);
    int c = 0;
    for (; c < nch; ++c) {
      const int s = c % lr::kASlots;
      if (c >= 2) {
        read(c - 2);
        if (lr::aborted(abortp)) break;
      }
      if (c + 1 < nch) load_b(c + 1);
      if (!tc::mbar_wait_try(&bar[lr::BAR_FULL + s], (uint32_t)((c / lr::kASlots) & 1)))
        lr::give_up(err, abortp);
      if (lr::aborted(abortp)) break;
      {
        // row R, 16 K values, from the swizzled tile of its K half: hi (the
        // value itself) and lo into A buffer c % 2
        const unsigned char* sa = smem + s * lr::A_BYTES + (kq >> 1) * lr::A_HALF + (uint32_t)R * 128u;
        float hi[16], lo[16];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int qq = 4 * (kq & 1) + j;
          const float4 x = *reinterpret_cast<const float4*>(sa + ((uint32_t)(qq ^ (R & 7)) << 4));
          hi[4 * j] = x.x;
          hi[4 * j + 1] = x.y;
          hi[4 * j + 2] = x.z;
          hi[4 * j + 3] = x.w;
          lo[4 * j] = x.x - tf32_rz(x.x);
          lo[4 * j + 1] = x.y - tf32_rz(x.y);
          lo[4 * j + 2] = x.z - tf32_rz(x.z);
          lo[4 * j + 3] = x.w - tf32_rz(x.w);
        }
        const uint32_t ta = tmem + lr::TM_A + lr::TM_ASTRIDE * (uint32_t)(c & 1) + 16u * kq + lane_base;
        tc::tmem_st16(ta, hi);
        tc::tmem_st16(ta + 64u, lo);
      }
      // the A slot is free once every worker warp has read its rows
      __syncwarp();
      if ((tid & 31) == 0) tc::mbar_arrive(&bar[lr::BAR_EMPTY + s]);
      {
        // low parts of this thread's two B segments of chunk c, next to B_hi
        // (here cheaper than copying the precomputed ones: the copies of
        // this kernel are not hidden behind its split)
        if (c + 1 < nch) cp_async_wait<1>();
        else cp_async_wait<0>();
        unsigned char* bs = smem + lr::B_OFF + (c % lr::kBSlots) * lr::B_BYTES;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          unsigned char* sb = bs + (h ? boff_bot : boff_top);
          const float4 xb = *reinterpret_cast<const float4*>(sb);
          float4 lb;
          lb.x = xb.x - tf32_rz(xb.x);
          lb.y = xb.y - tf32_rz(xb.y);
          lb.z = xb.z - tf32_rz(xb.z);
          lb.w = xb.w - tf32_rz(xb.w);
          *reinterpret_cast<float4*>(sb + lr::B_LO) = lb;
        }
      }
      tc::tmem_wait_st();
      tc::fence_async_smem();
      tc::fence_before_sync();
      __syncwarp();
      if ((tid & 31) == 0) tc::mbar_arrive(&bar[lr::BAR_READY + (c & 1)]);
    }
    if (c == nch)
      for (int r = nch >= 2 ? nch - 2 : 0; r < nch && !lr::aborted(abortp); ++r) read(r);
    cp_async_wait<0>();
    // combine the halves: the bottom rows' sums go through shared memory
    // (A slot 0, free once every worker is past its last chunk)
    lr::workers_sync();
    double v[lr::NCOL];
#pragma unroll
    for (int j = 0; j < lr::NCOL; ++j) v[j] = ((double)sum[j] - (double)comp[j]) + (double)cross[j];
    double* comb = reinterpret_cast<double*>(smem);
    if (bottom) {
#pragma unroll
      for (int j = 0; j < lr::NCOL; ++j) comb[(R - 64) * NR + lr::NCOL * kq + j] = v[j];
    }
    lr::workers_sync();
    if (!bottom && R < nk && !lr::aborted(abortp)) {
      const int64_t t = t0 + R;
      const int64_t orig = perm[t];
#pragma unroll
      for (int j = 0; j < lr::NCOL; ++j) {
        const int cc = lr::NCOL * kq + j;
        if (cc < nrhs) {
          const double yn = levels >= 2 ? Ynl[(int64_t)cc * N + t] : 0.0;
          Y[(int64_t)cc * ldy + orig] = (v[j] + comb[R * NR + cc]) + yn;
        }
      }
    }
  }
  // teardown: every role is past its last use of tensor memory and shared memory
  tc::fence_before_sync();
  __syncthreads();
  if (tid < 32) tc::tmem_dealloc(tmem, kTmemCols);
}

}  // namespace

int launch_near_lo(cudaStream_t s, int64_t nleaf, const int32_t* leaf_off, const NearOp& near,
                   const int64_t* near_off, const int32_t* near_ld, const float* Knear,
                   float* Knearlo) {
  k_near_lo<<<dim3((unsigned)nleaf, 27), 256, 0, s>>>(leaf_off, near, near_off, near_ld, Knear, Knearlo);
  return 1;
}

int tc_max_entries() { return kMaxEntries; }
cudaError_t tc_set_drop_chunk(int chunk) {
  return cudaMemcpyToSymbol(g_drop_chunk, &chunk, sizeof(int));
}
int tc_max_row_blocks() { return lr::kMaxBlocks; }

int launch_row_blocks(cudaStream_t s, int64_t nleaf, int max_blocks, const int32_t* leaf_off,
                      const NearOp& near, const LeafBlock* blocks, const int32_t* block_ptr,
                      const int64_t* row_base, const int32_t* row_ld, float* Krow) {
  if (nleaf == 0 || max_blocks == 0) return 0;
  k_row_blocks<<<dim3((unsigned)nleaf, (unsigned)max_blocks), 256, 0, s>>>(
      leaf_off, near, blocks, block_ptr, row_base, row_ld, Krow);
  return 1;
}

int launch_near_blocks(cudaStream_t s, int64_t nleaf, const int32_t* leaf_off, const NearOp& near,
                       const int64_t* near_off, const int32_t* near_ld, float* Knear) {
  k_near_blocks<<<dim3((unsigned)nleaf, 27), 256, 0, s>>>(leaf_off, near, near_off, near_ld, Knear);
  return 1;
}

int launch_matvec_tc(cudaStream_t s, int64_t N, const int32_t* perm, const FarOp& far,
                     const NearOp& near, const TcBuffers& B, const double* X, int64_t ldx,
                     double* Y, int64_t ldy, int nrhs, MatvecProfiler* prof) {
  (void)near;
  static bool attr[kMaxDevices] = {};  // kernel attributes are per device
  const int dev = current_device();
  if (!attr[dev]) {
    cudaFuncSetAttribute(k_ta_tc<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
    cudaFuncSetAttribute(k_ut_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
    cudaFuncSetAttribute(k_leaf_rows_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, lr::SMEM_BYTES);
    attr[dev] = true;
  }
  const CUtensorMap* umaps = static_cast<const CUtensorMap*>(B.umaps);
  const CUtensorMap* vmaps = static_cast<const CUtensorMap*>(B.vmaps);
  const CUtensorMap* rmaps = static_cast<const CUtensorMap*>(B.rmaps);
  int launches = 0;
  if (prof) prof->begin(s);
  k_gather_xt<<<(unsigned)((N * NR + 255) / 256), 256, 0, s>>>(N, nrhs, X, ldx, perm, B.xt, B.lo_off);
  ++launches;
  if (prof) prof->mark(s, "gather");
  const int d = far.levels;
  if (d >= 2) {
    // T of the pairs above the leaves, then their U T: level sums in Ynl
    const int64_t nslice = int64_t(1) << (3 * (d - 1));
    // several blocks share a slice's row tiles when slices are few
    // (the default: about 16 blocks per SM in all; hodlr3d_autotune may pick another)
    const int split = B.ta_split > 0 ? std::min(B.ta_split, 64)
                                     : (int)std::max<int64_t>(1, std::min<int64_t>(32, (16 * 152) / nslice));
    k_ta_tc<true><<<dim3((unsigned)nslice, (unsigned)split), THREADS, SMEM_BYTES, s>>>(
        far, vmaps, B.xt, N, B.t, B.p, B.lo_off, B.err);
    ++launches;
    if (prof) prof->mark(s, "ta_slice");
    if (B.n_upper > 0) {
      k_tred_tc<<<(unsigned)B.n_upper, 256, 0, s>>>(far, B.upper_pairs, B.p, B.t, B.lo_off);
      ++launches;
      if (prof) prof->mark(s, "tred");
    }
    const int tiles = (B.max_slice + 127) / 128;
    k_ut_tc<<<dim3((unsigned)nslice, (unsigned)std::max(1, tiles)), THREADS, SMEM_BYTES, s>>>(
        far, umaps, B.t, N, B.ynl, B.lo_off, B.err);
    ++launches;
    if (prof) prof->mark(s, "ut_tc");
  }
  // the leaf level (dense blocks) and the near field, plus the level sums
  k_leaf_rows_tc<<<(unsigned)far.nleaf, lr::THREADS, lr::SMEM_BYTES, s>>>(
      far.leaf_off, B.blocks, B.block_ptr, rmaps, B.xt, N, B.ynl, d, perm, nrhs, Y, ldy, B.err);
  ++launches;
  if (prof) prof->mark(s, "leaf_rows");
  return launches;
}

}  // namespace h3d
